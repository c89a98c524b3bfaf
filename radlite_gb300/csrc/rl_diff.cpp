// rl_diff.cpp -- the differentiable line raytrace: spectra as a function of per-cell
// ln T, ln X (abundance) and line width, and their gradients by the adjoint walk.
//
// Forward:  LTE tables on the device (k_lte_cells / k_lte_lines), node widths from the
//           cell widths (k_node_lw), then the forward walk and reduction of the plain path.
// Backward: the adjoint walk (k_adjoint_jobs) accumulates dL/d ln T, dL/d ln X and
//           dL/d width per cell directly, through the tables' derivatives.
// The reference has no differentiable path; its inputs are the level populations the
// setup writes (pyradlite radlite.py:1106-1118 computes them in LTE, which is what the
// table kernel does). What stays fixed from the loaded model: grid, velocities, densities,
// dust opacities, star, camera, passband, the largest line width (velocity-window
// margin, telescope.F:401) and the FP32 intensity scale of each line. Dust is at the gas
// temperature.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "rl_geometry.cuh"
#include "rl_internal.h"

namespace rl {
template <typename T>
cudaError_t launch_lte(const LteParams<T>& P, cudaStream_t s);
template <typename T>
cudaError_t launch_node_lw(const NodeBuf<T>& nb, const double* b, int nth, cudaStream_t s);
template <typename T>
cudaError_t adjoint_grid(int nsm, int max_nfr, int every, int* blocks);
template <typename T>
long long adjoint_ckpt_per_warp(int kmax, int max_nfr, int every);
int adjoint_items(int nlines, int nrays, int every);
template <typename T>
cudaError_t launch_adjoint(const AdjJobs<T>& B, int blocks, cudaStream_t s);
template <typename T>
cudaError_t launch_adjoint_one(const AdjParams<T>& A, const AdjJobs<T>& B, int blocks, cudaStream_t s);
cudaError_t launch_adjoint_finish(const float4* g4, double* gT, double* gX, double* gb, long long n, cudaStream_t s);
}  // namespace rl

using namespace rl;

struct rl_diff {
  rl_ctx* ctx = nullptr;
  rl_model* md = nullptr;
  int iline0 = 0, nl = 0, precision = RL_FP32;
  int ncell = 0, nfr = 0, kmax = 0, cpl = 8, gsize = 1, adj_blocks = 0;
  Camera cam;
  std::vector<double> scale;
  bool has_isrf = false;   // star holds the outer-boundary-3 start table too
  // node records of this camera (own copy: the widths change with the parameters)
  DevBuf x0, z0, ri, nn, st, ds, dvf, vl, dvs, lw, wr, wt, c00, misc;
  // LTE constants and per-line channel data
  DevBuf Ek, lng, lines, dust, rho_m, lnQ, Emean, wch, velo, star, lc, dscale;
  // tables of the last forward
  DevBuf tab, nsum, dtab, width;
  DevBuf img, ring, flux, cnt, work, err, list;
  DevBuf tau, tauc;   // the gradient sweep: each walked channel's optical depth from the forward
  // adjoint
  DevBuf ckpt, ajob, aprefix, acnt, awork;
  DevBuf g4;   // FP32 adjoint: interleaved gradient accumulator [ncell]
  bool have_forward = false;
  int every = 0;   // adjoint: 0 the gradient sweep in walk order; 1 or 32 the reverse sweep
                   // with stored intensities every node or every 32 nodes
};

namespace {

constexpr double kHcK = 1.4387769;   // hc/k [cm K]

template <typename T>
NodeBuf<T> nodes(const rl_diff* d) {
  NodeBuf<T> nb;
  nb.nrays = d->cam.nrays; nb.kmax = d->kmax;
  nb.nnodes = d->nn.as<int>(); nb.status = d->st.as<int>();
  nb.ds = d->ds.as<T>(); nb.dvf = d->dvf.as<float>(); nb.vl = d->vl.as<T>(); nb.dvseg = d->dvs.as<T>();
  nb.lw = d->lw.as<T>(); nb.wr = d->wr.as<T>(); nb.wt = d->wt.as<T>(); nb.c00 = d->c00.as<int>();
  nb.misc = d->misc.as<unsigned>();
  return nb;
}

template <typename T>
WalkParams<T> walk_params(const rl_diff* d) {
  const Model& m = d->md->m;
  WalkParams<T> P;
  P.nb = nodes<T>(d);
  P.nth = m.nth; P.ncell = d->ncell; P.nlines = d->nl; P.nfr = d->nfr;
  P.gsize = d->gsize;
  P.nitems = ((d->nl + d->gsize - 1) / d->gsize) * d->cam.nrays;
  P.tab = d->tab.as<T>(); P.nsum = d->nsum.as<T>(); P.wch = d->wch.as<T>(); P.velo = d->velo.as<double>();
  P.star = d->star.as<T>(); P.lc = d->lc.as<LineConst<T>>();
  P.isrf = isrf_of(d->has_isrf, P.star, d->nl, d->nfr);
  P.aksmax_c = m.aksmax / 2.99792458e5;
  P.kq = (T)(3.33567e-6 * 2.99792458e5);
  P.fstar = (T)((m.rstar / d->cam.ri[1]) * (m.rstar / d->cam.ri[1]));
  P.img = d->img.as<T>();
  P.counters = d->cnt.as<unsigned long long>();
  P.work = d->work.as<int>();
  P.err = d->err.as<int>();
  P.list = d->list.as<unsigned short>();
  if (d->every == 0) { P.tau = d->tau.as<T>(); P.tauc = d->tauc.as<T>(); }
  return P;
}

// The gradient sweep takes each channel's optical depth along the ray from the forward
// walk: image-shaped buffers, allocated when that adjoint mode is in use.
template <typename T>
cudaError_t ensure_tau(rl_diff* d, bool need) {
  if (!need) return cudaSuccess;
  const size_t n = (size_t)d->nl * d->cam.nrays * d->nfr;
  cudaError_t e = d->tau.ensure(sizeof(T) * n);
  if (e == cudaSuccess) e = d->tauc.ensure(sizeof(T) * n);
  return e;
}

template <typename T>
int create(rl_diff* d) {
  rl_ctx* ctx = d->ctx;
  rl_model* md = d->md;
  const Model& m = md->m;
  cudaStream_t s = ctx->stream;
  int rc = upload_grid(md);
  if (rc) return rc;
  std::string err;
  if (setup_camera(m, md->incl_rad, md->nphi, md->dbdr, md->nrext, d->cam, err)) return set_err(ctx, RL_ERR_ARG, err);
  const Camera& cam = d->cam;
  d->ncell = m.ncell();
  d->nfr = m.nfr;
  if (d->nfr >= 2048) return set_err(ctx, RL_ERR_ARG, "at most 2047 channels per line are supported");
  if (cam.ri[1] < m.rstar) return set_err(ctx, RL_ERR_ARG, "central beam smaller than the star");
  d->kmax = rlg::max_nodes(m.nr, m.nth);
  const size_t nn = (size_t)cam.nrays * d->kmax;
  CUDA_TRY(d->x0.ensure(sizeof(double) * cam.nrays));
  CUDA_TRY(d->z0.ensure(sizeof(double) * cam.nrays));
  CUDA_TRY(d->ri.ensure(sizeof(double) * cam.ri.size()));
  CUDA_TRY(d->nn.ensure(sizeof(int) * cam.nrays));
  CUDA_TRY(d->st.ensure(sizeof(int) * cam.nrays));
  CUDA_TRY(d->ds.ensure(sizeof(T) * nn));
  CUDA_TRY(d->dvf.ensure(sizeof(float) * nn));
  CUDA_TRY(d->vl.ensure(sizeof(T) * nn));
  CUDA_TRY(d->dvs.ensure(sizeof(T) * nn));
  CUDA_TRY(d->lw.ensure(sizeof(T) * nn));
  CUDA_TRY(d->wr.ensure(sizeof(T) * nn));
  CUDA_TRY(d->wt.ensure(sizeof(T) * nn));
  CUDA_TRY(d->c00.ensure(sizeof(int) * nn));
  CUDA_TRY(d->misc.ensure(sizeof(unsigned) * nn));
  CUDA_TRY(h2d(d->x0.p, cam.x0.data(), sizeof(double) * cam.nrays, s));
  CUDA_TRY(h2d(d->z0.p, cam.z0.data(), sizeof(double) * cam.nrays, s));
  CUDA_TRY(h2d(d->ri.p, cam.ri.data(), sizeof(double) * cam.ri.size(), s));
  GeoParams gp = geo_params(md);
  gp.theta0 = cam.theta0;
  gp.x0 = d->x0.as<double>(); gp.z0 = d->z0.as<double>();
  CUDA_TRY(launch_geometry<T>(gp, nodes<T>(d), 0, cam.nrays, nullptr, s));
  std::vector<int> status(cam.nrays);
  CUDA_TRY(d2h(status.data(), d->st.p, sizeof(int) * cam.nrays, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  for (int r = 0; r < cam.nrays; r++)
    if (status[r] != 0)
      return set_err(ctx, RL_ERR_GEOMETRY, "geometry: ray " + std::to_string(r) + " failed with status " +
                                               std::to_string(status[r]));
  // per-line channel data and the fixed intensity scale (from the loaded populations)
  LineTables<T> lt;
  if (build_line_tables<T>(m, d->iline0, d->nl, lt, err)) return set_err(ctx, RL_ERR_ARG, err);
  d->scale = lt.scale;
  d->has_isrf = lt.has_isrf;
  // LTE constants
  const int nl = d->nl, ncell = d->ncell;
  std::vector<double> Ek(m.nlev), lng(m.nlev);
  for (int i = 0; i < m.nlev; i++) {
    Ek[i] = m.Ecm[i] * kHcK;
    lng[i] = std::log(m.gdeg[i]);
  }
  std::vector<LteLine> lines(nl);
  std::vector<double> dust((size_t)ncell * nl * 3, 0.0), rho_m(ncell);
  const double molpg = 1.0 / (m.umass * 1.6726e-24);
  for (int c = 0; c < ncell; c++) rho_m[c] = m.rho[c] * molpg;
  for (int l = 0; l < nl; l++) {
    const int il = d->iline0 - 1 + l;
    LteLine& L = lines[l];
    L.lu = m.lup[il] - 1; L.ld = m.ldn[il] - 1;
    const double lf = m.lfreq[il];
    L.nu = lf;
    L.Bud = 6.78171833781e46 * m.Aud[il] / (lf * lf * lf);
    L.Bdu = L.Bud * (m.gdeg[m.lup[il] - 1] / m.gdeg[m.ldn[il] - 1]);
    L.C1 = 5.27296241956e-28 * lf * m.Aud[il];
    L.C2 = 5.27296241956e-28 * lf;
    L.cphi = 0.56419583546 / (3.33567e-6 * std::fabs(lf));   // as prepare_line
    L.scale = lt.scale[l];
    // grey dust at the line centre (as prepare_line), without the Planck factor
    if (m.line_dust) {
      const int i = bracket(m.cnu, lf);
      if (i != 0 && i != m.ncont) {
        const double wgt = (lf - m.cnu[i - 1]) / (m.cnu[i] - m.cnu[i - 1]);
        for (int c = 0; c < ncell; c++) {
          double dabs = 0.0, scat = 0.0, ext = 0.0;
          for (int sp = 0; sp < m.nspec; sp++)
            for (int z = 0; z < m.nsize[sp]; z++) {
              const double* ka = &m.kabs[((size_t)sp * 4 + z) * m.ncont];
              const double* ks = &m.ksca[((size_t)sp * 4 + z) * m.ncont];
              const double dr = m.drho[(size_t)sp * ncell + c];
              dabs += dr * (wgt * ka[i] + (1.0 - wgt) * ka[i - 1]);
              ext += dr * (wgt * ka[i] + (1.0 - wgt) * ka[i - 1]) + dr * (wgt * ks[i] + (1.0 - wgt) * ks[i - 1]);
            }
          if (!m.scat.empty())
            scat = wgt * m.scat[(size_t)i * ncell + c] + (1.0 - wgt) * m.scat[(size_t)(i - 1) * ncell + c];
          double* q = &dust[((size_t)c * nl + l) * 3];
          q[0] = dabs; q[1] = scat; q[2] = ext;
        }
      }
    }
  }
  CUDA_TRY(d->Ek.ensure(sizeof(double) * m.nlev));
  CUDA_TRY(d->lng.ensure(sizeof(double) * m.nlev));
  CUDA_TRY(d->lines.ensure(sizeof(LteLine) * nl));
  CUDA_TRY(d->dust.ensure(sizeof(double) * dust.size()));
  CUDA_TRY(d->rho_m.ensure(sizeof(double) * ncell));
  CUDA_TRY(d->lnQ.ensure(sizeof(double) * ncell));
  CUDA_TRY(d->Emean.ensure(sizeof(double) * ncell));
  CUDA_TRY(d->wch.ensure(sizeof(T) * lt.wch.size()));
  CUDA_TRY(d->velo.ensure(sizeof(double) * lt.velo.size()));
  CUDA_TRY(d->star.ensure(sizeof(T) * lt.star.size()));
  CUDA_TRY(d->lc.ensure(sizeof(LineConst<T>) * nl));
  CUDA_TRY(d->dscale.ensure(sizeof(double) * nl));
  CUDA_TRY(d->tab.ensure(sizeof(T) * (size_t)ncell * nl * 4));
  CUDA_TRY(d->nsum.ensure(sizeof(T) * (size_t)ncell * nl));
  CUDA_TRY(d->dtab.ensure(sizeof(T) * (size_t)ncell * nl * 5));
  CUDA_TRY(d->width.ensure(sizeof(double) * ncell));
  CUDA_TRY(d->img.ensure(sizeof(T) * (size_t)nl * cam.nrays * d->nfr));
  CUDA_TRY(d->ring.ensure(sizeof(double) * (size_t)nl * (cam.nrr + 1) * d->nfr));
  CUDA_TRY(d->cnt.ensure(sizeof(unsigned long long) * kWalkCounters));
  CUDA_TRY(d->work.ensure(sizeof(int)));
  CUDA_TRY(d->err.ensure(sizeof(int)));
  CUDA_TRY(d->list.ensure(sizeof(unsigned short) * walk_list_elems(ctx->nsm, d->nfr)));
  CUDA_TRY(d->acnt.ensure(sizeof(unsigned long long) * 4));
  CUDA_TRY(d->awork.ensure(sizeof(int)));
  CUDA_TRY(d->ajob.ensure(sizeof(AdjParams<T>)));
  CUDA_TRY(d->aprefix.ensure(sizeof(int) * 2));
  CUDA_TRY(h2d(d->Ek.p, Ek.data(), sizeof(double) * m.nlev, s));
  CUDA_TRY(h2d(d->lng.p, lng.data(), sizeof(double) * m.nlev, s));
  CUDA_TRY(h2d(d->lines.p, lines.data(), sizeof(LteLine) * nl, s));
  CUDA_TRY(h2d(d->dust.p, dust.data(), sizeof(double) * dust.size(), s));
  CUDA_TRY(h2d(d->rho_m.p, rho_m.data(), sizeof(double) * ncell, s));
  CUDA_TRY(h2d(d->wch.p, lt.wch.data(), sizeof(T) * lt.wch.size(), s));
  CUDA_TRY(h2d(d->velo.p, lt.velo.data(), sizeof(double) * lt.velo.size(), s));
  CUDA_TRY(h2d(d->star.p, lt.star.data(), sizeof(T) * lt.star.size(), s));
  CUDA_TRY(h2d(d->lc.p, lt.lc.data(), sizeof(LineConst<T>) * nl, s));
  CUDA_TRY(h2d(d->dscale.p, lt.scale.data(), sizeof(double) * nl, s));
  // walk shape as the plain path: balanced groups of up to 8 lines
  walk_shape(nl, d->nfr, d->gsize, d->cpl);
  CUDA_TRY(adjoint_grid<T>(ctx->nsm, d->nfr, d->every, &d->adj_blocks));
  const long long per = adjoint_ckpt_per_warp<T>(d->kmax, d->nfr, d->every);
  CUDA_TRY(d->ckpt.ensure(sizeof(T) * (size_t)per * d->adj_blocks * 4));
  const int pre[2] = {0, adjoint_items(nl, cam.nrays, d->every)};
  CUDA_TRY(h2d(d->aprefix.p, pre, sizeof(pre), s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return 0;
}

template <typename T>
LteParams<T> lte_params(const rl_diff* d, const double* lnT, const double* lnX) {
  const Model& m = d->md->m;
  LteParams<T> L;
  L.ncell = d->ncell; L.nlev = m.nlev; L.nl = d->nl;
  L.lnT = lnT; L.lnX = lnX; L.rho_m = d->rho_m.as<double>(); L.Ek = d->Ek.as<double>(); L.lng = d->lng.as<double>();
  L.lines = d->lines.as<LteLine>(); L.dust = d->dust.as<double>();
  L.lnQ = d->lnQ.as<double>(); L.Emean = d->Emean.as<double>();
  L.tab = d->tab.as<T>(); L.nsum = d->nsum.as<T>(); L.dtab = d->dtab.as<T>();
  return L;
}

template <typename T>
ReduceParams reduce_params(const rl_diff* d) {
  ReduceParams rp;
  rp.nrays = d->cam.nrays; rp.nfr = d->nfr; rp.nphi = d->cam.nphi; rp.nrr = d->cam.nrr; rp.nlines = d->nl;
  rp.ri = d->ri.as<double>(); rp.dist2 = 3.08572e18 * 3.08572e18; rp.scale = d->dscale.as<double>();
  return rp;
}

template <typename T>
int forward(rl_diff* d, const double* lnT, const double* lnX, const double* width, double* flux, rl_stats* st) {
  rl_ctx* ctx = d->ctx;
  cudaStream_t s = ctx->stream;
  const Model& m = d->md->m;
  const LteParams<T> L = lte_params<T>(d, lnT, lnX);
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  CUDA_TRY(launch_lte<T>(L, s));
  CUDA_TRY(cudaMemcpyAsync(d->width.p, width, sizeof(double) * d->ncell, cudaMemcpyDeviceToDevice, s));
  CUDA_TRY(launch_node_lw<T>(nodes<T>(d), d->width.as<double>(), m.nth, s));
  CUDA_TRY(cudaMemsetAsync(d->cnt.p, 0, sizeof(unsigned long long) * kWalkCounters, s));
  CUDA_TRY(cudaMemsetAsync(d->work.p, 0, sizeof(int), s));
  CUDA_TRY(cudaMemsetAsync(d->err.p, 0, sizeof(int), s));
  CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  CUDA_TRY(ensure_tau<T>(d, d->every == 0));
  const WalkParams<T> P = walk_params<T>(d);
  CUDA_TRY(launch_walk<T>(P, d->cpl, ctx->nsm, s));
  CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  CUDA_TRY(launch_reduce<T>(reduce_params<T>(d), d->img.as<T>(), d->ring.as<double>(), flux, s));
  CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
  unsigned long long cnt[4] = {0, 0, 0, 0};
  int kerr = 0;
  CUDA_TRY(d2h(cnt, d->cnt.p, sizeof(cnt), s));
  CUDA_TRY(d2h(&kerr, d->err.p, sizeof(int), s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (kerr != 0) return set_err(ctx, RL_ERR_GEOMETRY, "walk: error code " + std::to_string(kerr));
  d->have_forward = true;
  if (st) {
    float a = 0, b = 0, c = 0;
    cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&c, ctx->ev[2], ctx->ev[3]);
    st->upload_ms += a; st->walk_ms += b; st->reduce_ms += c; st->total_ms += a + b + c;
    st->steps += cnt[0]; st->integrated += cnt[1]; st->node_visits += cnt[2];
    st->ray_channels += (unsigned long long)d->cam.nrays * d->nfr * d->nl;
    st->nrays = d->cam.nrays; st->nfr = d->nfr; st->kmax = d->kmax; st->nlines += d->nl;
  }
  return 0;
}

template <typename T>
int backward(rl_diff* d, const double* gflux, double* g_lnT, double* g_lnX, double* g_width, rl_stats* st) {
  rl_ctx* ctx = d->ctx;
  cudaStream_t s = ctx->stream;
  if (!d->have_forward) return set_err(ctx, RL_ERR_STATE, "rl_diff_backward: no forward pass to differentiate");
  AdjParams<T> A;
  A.W = walk_params<T>(d);
  A.gflux = gflux;
  A.ri = d->ri.as<double>();
  A.nphi = d->cam.nphi; A.nrr = d->cam.nrr;
  A.dtab = d->dtab.as<T>();
  A.g_lnT = g_lnT; A.g_lnX = g_lnX; A.g_b = g_width;
  if (sizeof(T) == 4) {
    CUDA_TRY(d->g4.ensure(sizeof(float4) * d->ncell));
    A.g4 = d->g4.as<float4>();
  }
  AdjJobs<T> B;
  B.jobs = d->ajob.as<AdjParams<T>>();
  B.item_prefix = d->aprefix.as<int>();
  B.njobs = 1; B.total = adjoint_items(d->nl, d->cam.nrays, d->every); B.max_nfr = d->nfr;
  B.ckpt = d->ckpt.as<T>();
  B.ckpt_warp = adjoint_ckpt_per_warp<T>(d->kmax, d->nfr, d->every);
  B.every = d->every;
  B.work = d->awork.as<int>();
  B.counters = d->acnt.as<unsigned long long>();
  CUDA_TRY(h2d(d->ajob.p, &A, sizeof A, s));
  CUDA_TRY(cudaMemsetAsync(g_lnT, 0, sizeof(double) * d->ncell, s));
  CUDA_TRY(cudaMemsetAsync(g_lnX, 0, sizeof(double) * d->ncell, s));
  CUDA_TRY(cudaMemsetAsync(g_width, 0, sizeof(double) * d->ncell, s));
  if (A.g4) CUDA_TRY(cudaMemsetAsync(A.g4, 0, sizeof(float4) * d->ncell, s));
  CUDA_TRY(cudaMemsetAsync(d->acnt.p, 0, sizeof(unsigned long long) * 4, s));
  CUDA_TRY(cudaMemsetAsync(d->err.p, 0, sizeof(int), s));
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  CUDA_TRY(launch_adjoint_one<T>(A, B, d->adj_blocks, s));
  if (A.g4) CUDA_TRY(launch_adjoint_finish(A.g4, g_lnT, g_lnX, g_width, d->ncell, s));
  CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  unsigned long long cnt[4] = {0, 0, 0, 0};
  int kerr = 0;
  CUDA_TRY(d2h(cnt, d->acnt.p, sizeof(cnt), s));
  CUDA_TRY(d2h(&kerr, d->err.p, sizeof(int), s));
  CUDA_TRY(cudaStreamSynchronize(s));
  if (kerr != 0) return set_err(ctx, RL_ERR_GEOMETRY, "adjoint: error code " + std::to_string(kerr));
  if (st) {
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]);
    st->walk_ms += a; st->reduce_ms += b; st->total_ms += a + b;
    st->steps += cnt[0];
    st->integrated += cnt[1];   // items whose continuum channel was zero (their copies get no gradient)
    if (d->every == 0) { st->refined_passes += cnt[2]; st->refined_channels += cnt[3]; }
    st->nrays = d->cam.nrays; st->nfr = d->nfr; st->kmax = d->kmax; st->nlines += d->nl;
  }
  return 0;
}

}  // namespace

// ---- many differentiable models in one launch sequence per direction ----
struct rl_diff_batch {
  rl_ctx* ctx = nullptr;
  int precision = -1;
  std::vector<rl_diff*> jobs;
  std::vector<size_t> cell_off, flux_off;
  size_t ncell = 0, nflux = 0;
  int max_nfr = 0, max_kmax = 0, adj_blocks = 0, every = 0;   // every: as rl_diff::every
  bool built = false, use_graph = true;
  DevBuf lnT, lnX, width, flux, gflux, g_lnT, g_lnX, g_width;
  DevBuf g4;   // FP32 adjoint: interleaved gradient accumulator [ncell]
  DevBuf walkjobs, redjobs, adjjobs, item_prefix, ring_prefix, line_prefix, adj_prefix, cnt, work, err, acnt, awork, ckpt,
      list;
  JobLaunch<float> Lf{};
  JobLaunch<double> Ld{};
  AdjJobs<float> Af{};
  AdjJobs<double> Ad{};
  unsigned long long* cnt_h = nullptr;
  int* err_h = nullptr;
  cudaGraph_t g[2] = {nullptr, nullptr};
  cudaGraphExec_t x[2] = {nullptr, nullptr};
  void drop_graphs() {
    for (int i = 0; i < 2; i++) {
      if (x[i]) cudaGraphExecDestroy(x[i]);
      if (g[i]) cudaGraphDestroy(g[i]);
      x[i] = nullptr; g[i] = nullptr;
    }
  }
  ~rl_diff_batch() {
    if (ctx) cudaSetDevice(ctx->device);
    drop_graphs();
    if (cnt_h) cudaFreeHost(cnt_h);
    if (err_h) cudaFreeHost(err_h);
  }
};

namespace {

template <typename T> JobLaunch<T>& launch_of(rl_diff_batch* b);
template <> JobLaunch<float>& launch_of<float>(rl_diff_batch* b) { return b->Lf; }
template <> JobLaunch<double>& launch_of<double>(rl_diff_batch* b) { return b->Ld; }
template <typename T> AdjJobs<T>& adj_of(rl_diff_batch* b);
template <> AdjJobs<float>& adj_of<float>(rl_diff_batch* b) { return b->Af; }
template <> AdjJobs<double>& adj_of<double>(rl_diff_batch* b) { return b->Ad; }

template <typename T>
int batch_build(rl_diff_batch* b) {
  rl_ctx* ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  const int nj = (int)b->jobs.size();
  if (nj == 0) return set_err(ctx, RL_ERR_STATE, "rl_diff_batch: no models");
  b->cell_off.assign(nj, 0);
  b->flux_off.assign(nj, 0);
  b->ncell = 0; b->nflux = 0; b->max_nfr = 0; b->max_kmax = 0;
  for (int j = 0; j < nj; j++) {
    const rl_diff* d = b->jobs[j];
    b->cell_off[j] = b->ncell;
    b->flux_off[j] = b->nflux;
    b->ncell += d->ncell;
    b->nflux += (size_t)d->nl * d->nfr;
    b->max_nfr = std::max(b->max_nfr, d->nfr);
    b->max_kmax = std::max(b->max_kmax, d->kmax);
  }
  CUDA_TRY(b->lnT.ensure(sizeof(double) * b->ncell));
  CUDA_TRY(b->lnX.ensure(sizeof(double) * b->ncell));
  CUDA_TRY(b->width.ensure(sizeof(double) * b->ncell));
  CUDA_TRY(b->g_lnT.ensure(sizeof(double) * b->ncell));
  CUDA_TRY(b->g4.ensure(sizeof(float4) * b->ncell));
  CUDA_TRY(b->g_lnX.ensure(sizeof(double) * b->ncell));
  CUDA_TRY(b->g_width.ensure(sizeof(double) * b->ncell));
  CUDA_TRY(b->flux.ensure(sizeof(double) * b->nflux));
  CUDA_TRY(b->gflux.ensure(sizeof(double) * b->nflux));
  CUDA_TRY(b->cnt.ensure(sizeof(unsigned long long) * kWalkCounters));
  CUDA_TRY(b->acnt.ensure(sizeof(unsigned long long) * 4));
  CUDA_TRY(b->work.ensure(sizeof(int)));
  CUDA_TRY(b->awork.ensure(sizeof(int)));
  CUDA_TRY(b->err.ensure(sizeof(int)));
  CUDA_TRY(b->list.ensure(sizeof(unsigned short) * walk_list_elems(ctx->nsm, b->max_nfr)));
  if (!b->cnt_h) CUDA_TRY(cudaMallocHost((void**)&b->cnt_h, sizeof(unsigned long long) * kWalkCounters));
  if (!b->err_h) CUDA_TRY(cudaMallocHost((void**)&b->err_h, sizeof(int) * 2));
  std::vector<WalkParams<T>> walk(nj);
  std::vector<RedJob<T>> red(nj);
  std::vector<AdjParams<T>> adj(nj);
  std::vector<int> itemp(nj + 1, 0), ringp(nj + 1, 0), linep(nj + 1, 0), adjp(nj + 1, 0);
  for (int j = 0; j < nj; j++) {
    rl_diff* d = b->jobs[j];
    CUDA_TRY(ensure_tau<T>(d, b->every == 0));   // the batch's adjoint mode, whatever the model's own
    WalkParams<T> w = walk_params<T>(d);
    w.tau = b->every == 0 ? d->tau.as<T>() : nullptr;
    w.tauc = b->every == 0 ? d->tauc.as<T>() : nullptr;
    w.counters = b->cnt.as<unsigned long long>();
    w.work = b->work.as<int>();
    w.err = b->err.as<int>();
    w.list = b->list.as<unsigned short>();
    walk[j] = w;
    red[j].p = reduce_params<T>(d);
    red[j].img = d->img.as<T>();
    red[j].ring = d->ring.as<double>();
    red[j].flux = b->flux.as<double>() + b->flux_off[j];
    AdjParams<T>& A = adj[j];
    A.W = w;
    A.gflux = b->gflux.as<double>() + b->flux_off[j];
    A.ri = d->ri.as<double>();
    A.nphi = d->cam.nphi; A.nrr = d->cam.nrr;
    A.dtab = d->dtab.as<T>();
    A.g_lnT = b->g_lnT.as<double>() + b->cell_off[j];
    A.g_lnX = b->g_lnX.as<double>() + b->cell_off[j];
    A.g_b = b->g_width.as<double>() + b->cell_off[j];
    A.g4 = sizeof(T) == 4 ? b->g4.as<float4>() + b->cell_off[j] : nullptr;
    itemp[j + 1] = itemp[j] + w.nitems;
    ringp[j + 1] = ringp[j] + d->nl * d->cam.nrr;
    linep[j + 1] = linep[j] + d->nl;
    adjp[j + 1] = adjp[j] + adjoint_items(d->nl, d->cam.nrays, b->every);
  }
  CUDA_TRY(b->walkjobs.ensure(sizeof(WalkParams<T>) * nj));
  CUDA_TRY(b->redjobs.ensure(sizeof(RedJob<T>) * nj));
  CUDA_TRY(b->adjjobs.ensure(sizeof(AdjParams<T>) * nj));
  CUDA_TRY(b->item_prefix.ensure(sizeof(int) * (nj + 1)));
  CUDA_TRY(b->ring_prefix.ensure(sizeof(int) * (nj + 1)));
  CUDA_TRY(b->line_prefix.ensure(sizeof(int) * (nj + 1)));
  CUDA_TRY(b->adj_prefix.ensure(sizeof(int) * (nj + 1)));
  CUDA_TRY(h2d(b->walkjobs.p, walk.data(), sizeof(WalkParams<T>) * nj, s));
  CUDA_TRY(h2d(b->redjobs.p, red.data(), sizeof(RedJob<T>) * nj, s));
  CUDA_TRY(h2d(b->adjjobs.p, adj.data(), sizeof(AdjParams<T>) * nj, s));
  CUDA_TRY(h2d(b->item_prefix.p, itemp.data(), sizeof(int) * (nj + 1), s));
  CUDA_TRY(h2d(b->ring_prefix.p, ringp.data(), sizeof(int) * (nj + 1), s));
  CUDA_TRY(h2d(b->line_prefix.p, linep.data(), sizeof(int) * (nj + 1), s));
  CUDA_TRY(h2d(b->adj_prefix.p, adjp.data(), sizeof(int) * (nj + 1), s));
  CUDA_TRY(adjoint_grid<T>(ctx->nsm, b->max_nfr, b->every, &b->adj_blocks));
  const long long per = adjoint_ckpt_per_warp<T>(b->max_kmax, b->max_nfr, b->every);
  CUDA_TRY(b->ckpt.ensure(sizeof(T) * (size_t)per * b->adj_blocks * 4));
  JobLaunch<T>& L = launch_of<T>(b);
  L = JobLaunch<T>{};
  L.njobs = nj; L.nsm = ctx->nsm; L.cpl = 4;
  L.geo = nullptr; L.ray_prefix = nullptr; L.nrays_total = 0;
  L.walk.jobs = b->walkjobs.as<WalkParams<T>>(); L.walk.item_prefix = b->item_prefix.as<int>();
  L.walk.njobs = nj; L.walk.total = itemp[nj]; L.walk.stride = 1; L.walk.max_nfr = b->max_nfr;
  L.walk.work = b->work.as<int>(); L.walk.counters = b->cnt.as<unsigned long long>();
  L.walk.list = b->list.as<unsigned short>();
  L.walk.tau = b->every == 0;
  L.reduce = true;
  L.red = b->redjobs.as<RedJob<T>>(); L.ring_prefix = b->ring_prefix.as<int>(); L.line_prefix = b->line_prefix.as<int>();
  L.nring_blocks = ringp[nj]; L.nline_blocks = linep[nj];
  AdjJobs<T>& A = adj_of<T>(b);
  A.jobs = b->adjjobs.as<AdjParams<T>>(); A.item_prefix = b->adj_prefix.as<int>();
  A.njobs = nj; A.total = adjp[nj]; A.max_nfr = b->max_nfr;
  A.ckpt = b->ckpt.as<T>(); A.ckpt_warp = per; A.every = b->every;
  A.work = b->awork.as<int>(); A.counters = b->acnt.as<unsigned long long>();
  CUDA_TRY(cudaStreamSynchronize(s));
  b->drop_graphs();
  b->built = true;
  return 0;
}

template <typename T>
cudaError_t batch_enqueue(rl_diff_batch* b, int dir, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  if (dir == 0) {
    for (size_t j = 0; j < b->jobs.size() && e == cudaSuccess; j++) {
      rl_diff* d = b->jobs[j];
      e = launch_lte<T>(lte_params<T>(d, b->lnT.as<double>() + b->cell_off[j], b->lnX.as<double>() + b->cell_off[j]), s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(d->width.p, b->width.as<double>() + b->cell_off[j], sizeof(double) * d->ncell,
                            cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess) e = launch_node_lw<T>(nodes<T>(d), d->width.as<double>(), d->md->m.nth, s);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(b->cnt.p, 0, sizeof(unsigned long long) * kWalkCounters, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->err.p, 0, sizeof(int), s);
    if (e == cudaSuccess) e = launch_jobs<T>(launch_of<T>(b), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->cnt_h, b->cnt.p, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->err_h, b->err.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  } else {
    e = cudaMemsetAsync(b->g_lnT.p, 0, sizeof(double) * b->ncell, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->g_lnX.p, 0, sizeof(double) * b->ncell, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->g_width.p, 0, sizeof(double) * b->ncell, s);
    if (e == cudaSuccess && sizeof(T) == 4) e = cudaMemsetAsync(b->g4.p, 0, sizeof(float4) * b->ncell, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->acnt.p, 0, sizeof(unsigned long long) * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->err.p, 0, sizeof(int), s);
    if (e == cudaSuccess) e = launch_adjoint<T>(adj_of<T>(b), b->adj_blocks, s);
    if (e == cudaSuccess && sizeof(T) == 4)
      e = launch_adjoint_finish(b->g4.as<float4>(), b->g_lnT.as<double>(), b->g_lnX.as<double>(),
                                b->g_width.as<double>(), (long long)b->ncell, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->cnt_h + 4, b->acnt.p, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->err_h + 1, b->err.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  }
  return e;
}

template <typename T>
int batch_run(rl_diff_batch* b, int dir, rl_stats* st) {
  rl_ctx* ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  if (!b->built) {
    int rc = batch_build<T>(b);
    if (rc) return rc;
  }
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  if (b->use_graph) {
    if (!b->x[dir]) {
      cudaGraph_t g = nullptr;
      CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
      const cudaError_t e = batch_enqueue<T>(b, dir, s);
      const cudaError_t e2 = cudaStreamEndCapture(s, &g);
      if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return set_err(ctx, RL_ERR_CUDA, std::string("rl_diff_batch: graph capture: ") +
                                              cudaGetErrorString(e != cudaSuccess ? e : e2));
      }
      b->g[dir] = g;
      CUDA_TRY(cudaGraphInstantiate(&b->x[dir], g, 0));
    }
    CUDA_TRY(cudaGraphLaunch(b->x[dir], s));
  } else {
    CUDA_TRY(batch_enqueue<T>(b, dir, s));
  }
  CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  CUDA_TRY(cudaStreamSynchronize(s));
  const int kerr = b->err_h[dir];
  if (kerr != 0) return set_err(ctx, RL_ERR_GEOMETRY, std::string(dir ? "adjoint" : "walk") + ": error code " +
                                                     std::to_string(kerr));
  if (dir == 0) for (rl_diff* d : b->jobs) d->have_forward = true;
  if (st) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    st->total_ms += ms;
    st->walk_ms += ms;
    const unsigned long long* c = b->cnt_h + 4 * dir;
    st->steps += c[0];
    st->integrated += c[1];
    if (dir == 0) {
      st->node_visits += c[2];
      for (rl_diff* d : b->jobs) {
        st->ray_channels += (unsigned long long)d->cam.nrays * d->nfr * d->nl;
        st->nlines += d->nl;
      }
    }
  }
  return 0;
}

}  // namespace

extern "C" {

int rl_diff_batch_create(rl_ctx* ctx, rl_diff_batch** out) {
  if (!ctx || !out) return set_err(ctx, RL_ERR_ARG, "rl_diff_batch_create: null argument");
  *out = nullptr;
  std::unique_ptr<rl_diff_batch> b(new rl_diff_batch);
  b->ctx = ctx;
  *out = b.release();
  return 0;
}

int rl_diff_batch_destroy(rl_diff_batch* b) {
  delete b;
  return 0;
}

int rl_diff_batch_add(rl_diff_batch* b, rl_diff* d) {
  if (!b || !d) return set_err(b ? b->ctx : nullptr, RL_ERR_ARG, "rl_diff_batch_add: null argument");
  rl_ctx* ctx = b->ctx;
  if (d->ctx != ctx) return set_err(ctx, RL_ERR_ARG, "rl_diff_batch_add: model of another context");
  if (b->precision >= 0 && d->precision != b->precision)
    return set_err(ctx, RL_ERR_ARG, "rl_diff_batch_add: all models of a batch have one precision");
  b->precision = d->precision;
  b->jobs.push_back(d);
  b->built = false;
  b->drop_graphs();
  return (int)b->jobs.size() - 1;
}

int rl_diff_batch_use_graph(rl_diff_batch* b, int enable) {
  if (!b) return set_err(nullptr, RL_ERR_ARG, "rl_diff_batch_use_graph: null batch");
  b->use_graph = enable != 0;
  return 0;
}

int rl_diff_batch_buffers(rl_diff_batch* b, double** lnT, double** lnX, double** width, double** flux, double** gflux,
                          double** g_lnT, double** g_lnX, double** g_width, long long* ncell, long long* nflux) {
  if (!b) return set_err(nullptr, RL_ERR_ARG, "rl_diff_batch_buffers: null batch");
  rl_ctx* ctx = b->ctx;
  CUDA_TRY(rl::enter_device(ctx->device));
  if (!b->built) {
    const int rc = b->precision == RL_FP64 ? batch_build<double>(b) : batch_build<float>(b);
    if (rc) return rc;
  }
  if (lnT) *lnT = b->lnT.as<double>();
  if (lnX) *lnX = b->lnX.as<double>();
  if (width) *width = b->width.as<double>();
  if (flux) *flux = b->flux.as<double>();
  if (gflux) *gflux = b->gflux.as<double>();
  if (g_lnT) *g_lnT = b->g_lnT.as<double>();
  if (g_lnX) *g_lnX = b->g_lnX.as<double>();
  if (g_width) *g_width = b->g_width.as<double>();
  if (ncell) *ncell = (long long)b->ncell;
  if (nflux) *nflux = (long long)b->nflux;
  return 0;
}

int rl_diff_batch_layout(rl_diff_batch* b, int job, long long* cell_offset, long long* flux_offset) {
  if (!b || job < 0 || job >= (int)b->jobs.size())
    return set_err(b ? b->ctx : nullptr, RL_ERR_ARG, "rl_diff_batch_layout: bad job");
  if (!b->built) {
    const int rc = rl_diff_batch_buffers(b, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                         nullptr, nullptr);
    if (rc) return rc;
  }
  if (cell_offset) *cell_offset = (long long)b->cell_off[job];
  if (flux_offset) *flux_offset = (long long)b->flux_off[job];
  return 0;
}

int rl_diff_batch_forward(rl_diff_batch* b, rl_stats* st) {
  if (!b) return set_err(nullptr, RL_ERR_ARG, "rl_diff_batch_forward: null batch");
  rl_ctx* ctx = b->ctx;
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return b->precision == RL_FP64 ? batch_run<double>(b, 0, st) : batch_run<float>(b, 0, st);
}

int rl_diff_batch_backward(rl_diff_batch* b, rl_stats* st) {
  if (!b) return set_err(nullptr, RL_ERR_ARG, "rl_diff_batch_backward: null batch");
  rl_ctx* ctx = b->ctx;
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return b->precision == RL_FP64 ? batch_run<double>(b, 1, st) : batch_run<float>(b, 1, st);
}


int rl_diff_create(rl_model* md, int iline0, int nlines, int precision, rl_diff** out) {
  if (!md || !out) return set_err(nullptr, RL_ERR_ARG, "rl_diff_create: null argument");
  rl_ctx* ctx = md->ctx;
  if (!ctx) return set_err(nullptr, RL_ERR_STATE, "model was loaded without a device context");
  *out = nullptr;
  if (precision != RL_FP32 && precision != RL_FP64) return set_err(ctx, RL_ERR_ARG, "rl_diff_create: precision");
  if (nlines < 1 || iline0 < 1 || iline0 + nlines - 1 > (int)md->m.lfreq.size())
    return set_err(ctx, RL_ERR_ARG, "rl_diff_create: line range outside the molecule's line list");
  CUDA_TRY(rl::enter_device(ctx->device));
  std::unique_ptr<rl_diff> d(new rl_diff);
  d->ctx = ctx; d->md = md; d->iline0 = iline0; d->nl = nlines; d->precision = precision;
  g_h2d = 0; g_d2h = 0;
  const int rc = precision == RL_FP64 ? create<double>(d.get()) : create<float>(d.get());
  if (rc) return rc;
  *out = d.release();
  return 0;
}

int rl_diff_destroy(rl_diff* d) {
  if (!d) return 0;
  if (d->ctx) cudaSetDevice(d->ctx->device);
  delete d;
  return 0;
}

int rl_diff_set_checkpoint(rl_diff* d, int every) {
  if (!d) return set_err(nullptr, RL_ERR_ARG, "rl_diff_set_checkpoint: null handle");
  rl_ctx* ctx = d->ctx;
  if (every != 0 && every != 1 && every != 32)
    return set_err(ctx, RL_ERR_ARG, "rl_diff_set_checkpoint: 0 (gradient sweep), 1 or 32");
  CUDA_TRY(rl::enter_device(ctx->device));
  d->every = every;
  d->have_forward = false;   // the forward of the other mode does not keep what this one needs
  const bool f64 = d->precision == RL_FP64;
  CUDA_TRY(f64 ? adjoint_grid<double>(ctx->nsm, d->nfr, every, &d->adj_blocks)
               : adjoint_grid<float>(ctx->nsm, d->nfr, every, &d->adj_blocks));
  const long long per = f64 ? adjoint_ckpt_per_warp<double>(d->kmax, d->nfr, every)
                            : adjoint_ckpt_per_warp<float>(d->kmax, d->nfr, every);
  const size_t el = f64 ? sizeof(double) : sizeof(float);
  CUDA_TRY(d->ckpt.ensure(el * (size_t)per * d->adj_blocks * 4));
  const int pre[2] = {0, adjoint_items(d->nl, d->cam.nrays, every)};
  CUDA_TRY(h2d(d->aprefix.p, pre, sizeof(pre), ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return 0;
}

int rl_diff_info(rl_diff* d, int* ncell, int* nlines, int* nfr, int* nrays) {
  if (!d) return set_err(nullptr, RL_ERR_ARG, "rl_diff_info: null handle");
  if (ncell) *ncell = d->ncell;
  if (nlines) *nlines = d->nl;
  if (nfr) *nfr = d->nfr;
  if (nrays) *nrays = d->cam.nrays;
  return 0;
}

int rl_diff_forward(rl_diff* d, const double* lnT, const double* lnX, const double* width, double* flux,
                    rl_stats* st) {
  if (!d || !lnT || !lnX || !width || !flux) return set_err(d ? d->ctx : nullptr, RL_ERR_ARG, "rl_diff_forward: null argument");
  rl_ctx* ctx = d->ctx;
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return d->precision == RL_FP64 ? forward<double>(d, lnT, lnX, width, flux, st)
                                 : forward<float>(d, lnT, lnX, width, flux, st);
}

int rl_diff_backward(rl_diff* d, const double* gflux, double* g_lnT, double* g_lnX, double* g_width, rl_stats* st) {
  if (!d || !gflux || !g_lnT || !g_lnX || !g_width)
    return set_err(d ? d->ctx : nullptr, RL_ERR_ARG, "rl_diff_backward: null argument");
  rl_ctx* ctx = d->ctx;
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return d->precision == RL_FP64 ? backward<double>(d, gflux, g_lnT, g_lnX, g_width, st)
                                 : backward<float>(d, gflux, g_lnT, g_lnX, g_width, st);
}

}  // extern "C"
