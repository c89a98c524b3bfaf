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
cudaError_t adjoint_grid(int nsm, int max_nfr, int* blocks);
template <typename T>
long long adjoint_ckpt_per_warp(int kmax, int every);
template <typename T>
cudaError_t launch_adjoint(const AdjJobs<T>& B, int blocks, cudaStream_t s);
}  // namespace rl

using namespace rl;

struct rl_diff {
  rl_ctx* ctx = nullptr;
  rl_model* md = nullptr;
  int iline0 = 0, nl = 0, precision = RL_FP32;
  int ncell = 0, nfr = 0, kmax = 0, cpl = 8, gsize = 1, adj_blocks = 0;
  Camera cam;
  std::vector<double> scale;
  // node records of this camera (own copy: the widths change with the parameters)
  DevBuf x0, z0, ri, nn, st, ds, dvf, vl, dvs, lw, wr, wt, c00, misc;
  // LTE constants and per-line channel data
  DevBuf Ek, lng, lines, dust, rho_m, lnQ, Emean, wch, velo, star, lc, dscale;
  // tables of the last forward
  DevBuf tab, nsum, dtab, width;
  DevBuf img, ring, flux, cnt, work, err;
  // adjoint
  DevBuf ckpt, ajob, aprefix, acnt, awork;
  bool have_forward = false;
  int every = 1;   // adjoint checkpoint interval (nodes)
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
  P.aksmax_c = m.aksmax / 2.99792458e5;
  P.kq = (T)(3.33567e-6 * 2.99792458e5);
  P.fstar = (T)((m.rstar / d->cam.ri[1]) * (m.rstar / d->cam.ri[1]));
  P.img = d->img.as<T>();
  P.counters = d->cnt.as<unsigned long long>();
  P.work = d->work.as<int>();
  P.err = d->err.as<int>();
  return P;
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
  CUDA_TRY(d->dtab.ensure(sizeof(double) * (size_t)ncell * nl * 5));
  CUDA_TRY(d->width.ensure(sizeof(double) * ncell));
  CUDA_TRY(d->img.ensure(sizeof(T) * (size_t)nl * cam.nrays * d->nfr));
  CUDA_TRY(d->ring.ensure(sizeof(double) * (size_t)nl * (cam.nrr + 1) * d->nfr));
  CUDA_TRY(d->cnt.ensure(sizeof(unsigned long long) * 4));
  CUDA_TRY(d->work.ensure(sizeof(int)));
  CUDA_TRY(d->err.ensure(sizeof(int)));
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
  const int ng = (nl + kWalkGroup - 1) / kWalkGroup;
  d->gsize = (nl + ng - 1) / ng;
  const int need = (d->gsize * d->nfr + 31) / 32;
  d->cpl = need <= 1 ? 1 : need <= 2 ? 2 : need <= 4 ? 4 : 8;
  CUDA_TRY(adjoint_grid<T>(ctx->nsm, d->nfr, &d->adj_blocks));
  const long long per = adjoint_ckpt_per_warp<T>(d->kmax, d->every);
  CUDA_TRY(d->ckpt.ensure(sizeof(T) * (size_t)per * d->adj_blocks * 4));
  const int pre[2] = {0, nl * cam.nrays};
  CUDA_TRY(h2d(d->aprefix.p, pre, sizeof(pre), s));
  CUDA_TRY(cudaStreamSynchronize(s));
  return 0;
}

template <typename T>
int forward(rl_diff* d, const double* lnT, const double* lnX, const double* width, double* flux, rl_stats* st) {
  rl_ctx* ctx = d->ctx;
  cudaStream_t s = ctx->stream;
  const Model& m = d->md->m;
  LteParams<T> L;
  L.ncell = d->ncell; L.nlev = m.nlev; L.nl = d->nl;
  L.lnT = lnT; L.lnX = lnX; L.rho_m = d->rho_m.as<double>(); L.Ek = d->Ek.as<double>(); L.lng = d->lng.as<double>();
  L.lines = d->lines.as<LteLine>(); L.dust = d->dust.as<double>();
  L.lnQ = d->lnQ.as<double>(); L.Emean = d->Emean.as<double>();
  L.tab = d->tab.as<T>(); L.nsum = d->nsum.as<T>(); L.dtab = d->dtab.as<double>();
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  CUDA_TRY(launch_lte<T>(L, s));
  CUDA_TRY(cudaMemcpyAsync(d->width.p, width, sizeof(double) * d->ncell, cudaMemcpyDeviceToDevice, s));
  CUDA_TRY(launch_node_lw<T>(nodes<T>(d), d->width.as<double>(), m.nth, s));
  CUDA_TRY(cudaMemsetAsync(d->cnt.p, 0, sizeof(unsigned long long) * 4, s));
  CUDA_TRY(cudaMemsetAsync(d->work.p, 0, sizeof(int), s));
  CUDA_TRY(cudaMemsetAsync(d->err.p, 0, sizeof(int), s));
  CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  const WalkParams<T> P = walk_params<T>(d);
  CUDA_TRY(launch_walk<T>(P, d->cpl, ctx->nsm, s));
  CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  ReduceParams rp;
  rp.nrays = d->cam.nrays; rp.nfr = d->nfr; rp.nphi = d->cam.nphi; rp.nrr = d->cam.nrr; rp.nlines = d->nl;
  rp.ri = d->ri.as<double>(); rp.dist2 = 3.08572e18 * 3.08572e18; rp.scale = d->dscale.as<double>();
  CUDA_TRY(launch_reduce<T>(rp, d->img.as<T>(), d->ring.as<double>(), flux, s));
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
  A.dtab = d->dtab.as<double>();
  A.g_lnT = g_lnT; A.g_lnX = g_lnX; A.g_b = g_width;
  AdjJobs<T> B;
  B.jobs = d->ajob.as<AdjParams<T>>();
  B.item_prefix = d->aprefix.as<int>();
  B.njobs = 1; B.total = d->nl * d->cam.nrays; B.max_nfr = d->nfr;
  B.ckpt = d->ckpt.as<T>();
  B.ckpt_warp = adjoint_ckpt_per_warp<T>(d->kmax, d->every);
  B.every = d->every;
  B.work = d->awork.as<int>();
  B.counters = d->acnt.as<unsigned long long>();
  CUDA_TRY(h2d(d->ajob.p, &A, sizeof A, s));
  CUDA_TRY(cudaMemsetAsync(g_lnT, 0, sizeof(double) * d->ncell, s));
  CUDA_TRY(cudaMemsetAsync(g_lnX, 0, sizeof(double) * d->ncell, s));
  CUDA_TRY(cudaMemsetAsync(g_width, 0, sizeof(double) * d->ncell, s));
  CUDA_TRY(cudaMemsetAsync(d->acnt.p, 0, sizeof(unsigned long long) * 4, s));
  CUDA_TRY(cudaMemsetAsync(d->err.p, 0, sizeof(int), s));
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  CUDA_TRY(launch_adjoint<T>(B, d->adj_blocks, s));
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
    st->nrays = d->cam.nrays; st->nfr = d->nfr; st->kmax = d->kmax; st->nlines += d->nl;
  }
  return 0;
}

}  // namespace

extern "C" {

int rl_diff_create(rl_model* md, int iline0, int nlines, int precision, rl_diff** out) {
  if (!md || !out) return set_err(nullptr, RL_ERR_ARG, "rl_diff_create: null argument");
  rl_ctx* ctx = md->ctx;
  if (!ctx) return set_err(nullptr, RL_ERR_STATE, "model was loaded without a device context");
  *out = nullptr;
  if (precision != RL_FP32 && precision != RL_FP64) return set_err(ctx, RL_ERR_ARG, "rl_diff_create: precision");
  if (nlines < 1 || iline0 < 1 || iline0 + nlines - 1 > (int)md->m.lfreq.size())
    return set_err(ctx, RL_ERR_ARG, "rl_diff_create: line range outside the molecule's line list");
  CUDA_TRY(cudaSetDevice(ctx->device));
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
  if (every != 1 && every != 32) return set_err(ctx, RL_ERR_ARG, "rl_diff_set_checkpoint: interval 1 or 32");
  CUDA_TRY(cudaSetDevice(ctx->device));
  d->every = every;
  const long long per = d->precision == RL_FP64 ? adjoint_ckpt_per_warp<double>(d->kmax, every)
                                                : adjoint_ckpt_per_warp<float>(d->kmax, every);
  const size_t el = d->precision == RL_FP64 ? sizeof(double) : sizeof(float);
  CUDA_TRY(d->ckpt.ensure(el * (size_t)per * d->adj_blocks * 4));
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
  CUDA_TRY(cudaSetDevice(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return d->precision == RL_FP64 ? forward<double>(d, lnT, lnX, width, flux, st)
                                 : forward<float>(d, lnT, lnX, width, flux, st);
}

int rl_diff_backward(rl_diff* d, const double* gflux, double* g_lnT, double* g_lnX, double* g_width, rl_stats* st) {
  if (!d || !gflux || !g_lnT || !g_lnX || !g_width)
    return set_err(d ? d->ctx : nullptr, RL_ERR_ARG, "rl_diff_backward: null argument");
  rl_ctx* ctx = d->ctx;
  CUDA_TRY(cudaSetDevice(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return d->precision == RL_FP64 ? backward<double>(d, gflux, g_lnT, g_lnX, g_width, st)
                                 : backward<float>(d, gflux, g_lnT, g_lnX, g_width, st);
}

}  // extern "C"
