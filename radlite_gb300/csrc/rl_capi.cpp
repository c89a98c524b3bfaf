// rl_capi.cpp -- the C ABI (include/rlgpu.h): device residency, camera geometry cache,
// per-line table upload, kernel orchestration on one stream, and the directory runner.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <ctime>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <type_traits>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/rlgpu.h"
#include "rl_device.h"
#include "rl_geometry.cuh"
#include "rl_host.h"
#include "rl_internal.h"

using namespace rl;

thread_local std::string g_last_error;
thread_local unsigned long long g_h2d = 0, g_d2h = 0;   // per call, reset by the entry points

namespace rl {
// Error text for entry points that take no context (read back with rl_last_error(NULL, ...)).
void set_last_error(const std::string& msg) { g_last_error = msg; }
int set_err(rl_ctx* c, int code, const std::string& msg) {
  g_last_error = msg;
  if (c) c->err = msg;
  return code;
}
cudaError_t h2d(void* dst, const void* src, size_t n, cudaStream_t s) {
  g_h2d += n;
  return cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, s);
}
cudaError_t d2h(void* dst, const void* src, size_t n, cudaStream_t s) {
  g_d2h += n;
  return cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, s);
}
}  // namespace rl

static void camera_defaults(rl_model* md) {
  md->incl_rad = md->m.incl_rad;
  md->nphi = md->m.nphi;
  md->dbdr = md->m.dbdr;
  md->nrext = md->m.nrext;
}

int rl::upload_grid(rl_model* md) {
  rl_ctx* ctx = md->ctx;
  if (md->grid_ready) return 0;
  const Model& m = md->m;
  std::vector<double> tan2(m.nth + 1, 0.0);
  for (int iy = 1; iy <= m.nth; iy++) { const double t = std::tan(m.TH[iy + 1]); tan2[iy] = t * t; }
  CUDA_TRY(md->dR.ensure(sizeof(double) * m.R.size()));
  CUDA_TRY(md->dTH.ensure(sizeof(double) * m.TH.size()));
  CUDA_TRY(md->dtan2.ensure(sizeof(double) * tan2.size()));
  CUDA_TRY(md->dvel.ensure(sizeof(double) * m.vel.size()));
  CUDA_TRY(md->dlw.ensure(sizeof(double) * m.lw.size()));
  cudaStream_t s = ctx->stream;
  CUDA_TRY(h2d(md->dR.p, m.R.data(), sizeof(double) * m.R.size(), s));
  CUDA_TRY(h2d(md->dTH.p, m.TH.data(), sizeof(double) * m.TH.size(), s));
  CUDA_TRY(h2d(md->dtan2.p, tan2.data(), sizeof(double) * tan2.size(), s));
  CUDA_TRY(h2d(md->dvel.p, m.vel.data(), sizeof(double) * m.vel.size(), s));
  CUDA_TRY(h2d(md->dlw.p, m.lw.data(), sizeof(double) * m.lw.size(), s));
  std::vector<float> velf(m.vel.begin(), m.vel.end()), lwf(m.lw.begin(), m.lw.end());
  std::vector<float> vell(m.vel.size());   // float-float low parts of the velocities
  for (size_t i = 0; i < vell.size(); i++) vell[i] = (float)(m.vel[i] - (double)velf[i]);
  CUDA_TRY(md->dvelf.ensure(sizeof(float) * velf.size()));
  CUDA_TRY(md->dvell.ensure(sizeof(float) * vell.size()));
  CUDA_TRY(md->dlwf.ensure(sizeof(float) * lwf.size()));
  CUDA_TRY(h2d(md->dvelf.p, velf.data(), sizeof(float) * velf.size(), s));
  CUDA_TRY(h2d(md->dvell.p, vell.data(), sizeof(float) * vell.size(), s));
  CUDA_TRY(h2d(md->dlwf.p, lwf.data(), sizeof(float) * lwf.size(), s));
  CUDA_TRY(cudaStreamSynchronize(s));
  md->grid_ready = true;
  return 0;
}

// Runs fn(w, nw) for w = 0 .. nw-1, each on a thread of its own (this one included); a
// worker that cannot get a thread runs on this one after the others have started.
template <typename F>
static void run_workers(int nw, const F& fn) {
  std::vector<std::thread> pool;
  int started = 1;
  try {
    for (; started < nw; started++) pool.emplace_back([&fn, started, nw] { fn(started, nw); });
  } catch (const std::system_error&) {
  }
  fn(0, nw);
  for (int w = started; w < nw; w++) fn(w, nw);
  for (auto& t : pool) t.join();
}

template <typename T>
int rl::build_line_tables(const Model& m, int iline0, int nl, LineTables<T>& out, std::string& err, bool with_isrf) {
  const int ncell = m.ncell(), nfr = m.nfr;
  const bool scaled = std::is_same<T, float>::value;
  out.nl = nl; out.ncell = ncell; out.nfr = nfr;
  out.tab.assign((size_t)nl * ncell * 4, (T)0); out.nsum.assign((size_t)nl * ncell, (T)0);
  const bool isrf = m.outer_bc == 3 && with_isrf;
  out.wch.assign((size_t)nl * nfr, (T)0); out.star.assign((size_t)(isrf ? 2 : 1) * nl * nfr, (T)0);
  out.velo.assign((size_t)nl * nfr, 0.0); out.scale.assign(nl, 1.0); out.lc.assign(nl, LineConst<T>{});
  out.mase.assign(nl, 0);
  out.has_isrf = isrf;
  // The lines are independent (prepare_line only reads the model). Host threads for models
  // of at least 2^18 cell-lines (the band model's 20 lines x 80000 cells take 0.15 s on one
  // core), at most 16. Lines go in batches of one per worker: the workers prepare the
  // batch's lines, then interleave them into the tables, each over a range of cells (the
  // cell-major layout puts neighbouring lines in one cache line). The tables are the same
  // whatever the worker count, and the error reported is that of the first failing line.
  const unsigned hc = std::thread::hardware_concurrency();
  const int nw = (double)nl * ncell >= 262144.0 ? std::min<int>({nl, 16, hc > 0 ? (int)hc : 1}) : 1;
  std::vector<LinePrep> lps((size_t)nw);
  std::vector<std::string> errs((size_t)nw);
  std::vector<char> bad((size_t)nw);
  for (int b = 0; b < nl; b += nw) {
    const int nb = std::min(nw, nl - b);
    run_workers(nb, [&](int w, int) {
      lps[w] = LinePrep();   // prepare_line sets the masing flag but never clears it
      bad[w] = prepare_line(m, iline0 + b + w, scaled, lps[w], errs[w], with_isrf) != 0;
    });
    for (int w = 0; w < nb; w++)
      if (bad[w]) { err = errs[w]; return RL_ERR_ARG; }
    // cell-major, line-minor: the corners of one node for consecutive lines are contiguous.
    // The line factors carry the profile normalisation (phi = cphi / lwav * e^{-u^2}).
    run_workers(nw, [&](int w, int n) {
      const int c0 = (int)((long long)ncell * w / n), c1 = (int)((long long)ncell * (w + 1) / n);
      for (int c = c0; c < c1; c++)
        for (int i = 0; i < nb; i++) {
          const LinePrep& lp = lps[i];
          const size_t o = (size_t)c * nl + b + i;
          out.tab[o * 4 + 0] = (T)(lp.tab[4 * (size_t)c + 0] * lp.cphi);
          out.tab[o * 4 + 1] = (T)(lp.tab[4 * (size_t)c + 1] * lp.cphi);
          out.tab[o * 4 + 2] = (T)lp.tab[4 * (size_t)c + 2];
          out.tab[o * 4 + 3] = (T)lp.tab[4 * (size_t)c + 3];
          out.nsum[o] = (T)lp.nsum[c];
        }
    });
    for (int i = 0; i < nb; i++) {
      const LinePrep& lp = lps[i];
      const int l = b + i;
      for (int k = 0; k < nfr; k++) {
        out.wch[(size_t)l * nfr + k] = (T)lp.wch[k];
        out.star[(size_t)l * nfr + k] = (T)lp.star[k];
        if (isrf) out.star[((size_t)nl + l) * nfr + k] = (T)lp.isrf[k];
        out.velo[(size_t)l * nfr + k] = lp.velo[k];
      }
      out.lc[l].cphi = (T)lp.cphi;
      out.lc[l].istart = (T)lp.istart;
      out.lc[l].scale = lp.scale;
      out.scale[l] = lp.scale;
      out.mase[l] = lp.mase;
    }
  }
  return 0;
}
template int rl::build_line_tables<float>(const Model&, int, int, LineTables<float>&, std::string&, bool);
template int rl::build_line_tables<double>(const Model&, int, int, LineTables<double>&, std::string&, bool);

template <typename T>
static int build_geometry(rl_model* md, rl_stats* st) {
  rl_ctx* ctx = md->ctx;
  cudaStream_t s = ctx->stream;
  if (md->geo_ready && md->geo_prec == md->precision) return 0;
  int rc = upload_grid(md);
  if (rc) return rc;
  std::string err;
  if (setup_camera(md->m, md->incl_rad, md->nphi, md->dbdr, md->nrext, md->cam, err))
    return set_err(ctx, RL_ERR_ARG, err);
  const Camera& cam = md->cam;
  md->kmax = rlg::max_nodes(md->m.nr, md->m.nth);
  const size_t nn = (size_t)cam.nrays * md->kmax;
  CUDA_TRY(md->dx0.ensure(sizeof(double) * cam.nrays));
  CUDA_TRY(md->dz0.ensure(sizeof(double) * cam.nrays));
  CUDA_TRY(md->dri.ensure(sizeof(double) * cam.ri.size()));
  CUDA_TRY(md->nb_nn.ensure(sizeof(int) * cam.nrays));
  CUDA_TRY(md->nb_st.ensure(sizeof(int) * cam.nrays));
  CUDA_TRY(md->nb_ds.ensure(sizeof(T) * nn));
  CUDA_TRY(md->nb_dvf.ensure(sizeof(float) * nn));
  CUDA_TRY(md->nb_vl.ensure(sizeof(T) * nn));
  CUDA_TRY(md->nb_dvs.ensure(sizeof(T) * nn));
  CUDA_TRY(md->nb_lw.ensure(sizeof(T) * nn));
  CUDA_TRY(md->nb_wr.ensure(sizeof(T) * nn));
  CUDA_TRY(md->nb_wt.ensure(sizeof(T) * nn));
  CUDA_TRY(md->nb_c00.ensure(sizeof(int) * nn));
  CUDA_TRY(md->nb_misc.ensure(sizeof(unsigned) * nn));
  CUDA_TRY(h2d(md->dx0.p, cam.x0.data(), sizeof(double) * cam.nrays, s));
  CUDA_TRY(h2d(md->dz0.p, cam.z0.data(), sizeof(double) * cam.nrays, s));
  CUDA_TRY(h2d(md->dri.p, cam.ri.data(), sizeof(double) * cam.ri.size(), s));
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  CUDA_TRY(launch_geometry<T>(geo_params(md), node_view<T>(md), 0, cam.nrays, nullptr, s));
  CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  std::vector<int> status(cam.nrays);
  CUDA_TRY(d2h(status.data(), md->nb_st.p, sizeof(int) * cam.nrays, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  if (st) st->geometry_ms += ms;
  for (int r = 0; r < cam.nrays; r++)
    if (status[r] != 0)
      return set_err(ctx, RL_ERR_GEOMETRY, "geometry: ray " + std::to_string(r) + " failed with status " + std::to_string(status[r]));
  md->geo_ready = true;
  md->geo_prec = md->precision;
  return 0;
}

// Image rows of chosen rays, gathered on the device after the walk (rl_image_rows).
struct RowRequest {
  const int* rays = nullptr;   // host ray indices
  int n = 0;
  double* out = nullptr;       // host [nl][n][nfr]
};

template <typename T>
static int run_lines(rl_model* md, int iline0, int nl, double* flux_out, double* image_out, unsigned char* mask_out,
                     rl_stats* st, const RowRequest* rows = nullptr) {
  rl_ctx* ctx = md->ctx;
  cudaStream_t s = ctx->stream;
  const Model& m = md->m;
  if (nl < 1 || iline0 < 1 || iline0 + nl - 1 > (int)m.lfreq.size())
    return set_err(ctx, RL_ERR_ARG, "line range outside the molecule's line list");
  int rc = build_geometry<T>(md, st);
  if (rc) return rc;
  const Camera& cam = md->cam;
  const int ncell = m.ncell(), nfr = m.nfr;
  // per-line tables (built on the host in FP64, kept on the device between calls)
  const bool cached = md->tab_line0 == iline0 && md->tab_nl == nl && md->tab_prec == md->precision;
  LineTables<T> lt;
  std::vector<double> scale = md->tab_scale;
  std::vector<char> mase = md->tab_mase;
  bool has_isrf = md->tab_isrf;
  if (!cached) {
    md->tab_line0 = -1;
    std::string err;
    if (build_line_tables<T>(m, iline0, nl, lt, err)) return set_err(ctx, RL_ERR_ARG, err);
    scale = lt.scale;
    mase = lt.mase;
    has_isrf = lt.has_isrf;
  }
  const std::vector<T>&tab = lt.tab, &nsum = lt.nsum, &wch = lt.wch, &star = lt.star;
  const std::vector<double>& velo = lt.velo;
  const std::vector<LineConst<T>>& lc = lt.lc;
  const size_t nimg = (size_t)nl * cam.nrays * nfr;
  if (!cached) {
    CUDA_TRY(md->dtab.ensure(sizeof(T) * tab.size()));
    CUDA_TRY(md->dnsum.ensure(sizeof(T) * nsum.size()));
    CUDA_TRY(md->dwch.ensure(sizeof(T) * wch.size()));
    CUDA_TRY(md->dstar.ensure(sizeof(T) * star.size()));
    CUDA_TRY(md->dvelo.ensure(sizeof(double) * velo.size()));
    CUDA_TRY(md->dlc.ensure(sizeof(LineConst<T>) * lc.size()));
    CUDA_TRY(md->dscale.ensure(sizeof(double) * nl));
  }
  CUDA_TRY(md->dimg.ensure(sizeof(T) * nimg));
  CUDA_TRY(md->dring.ensure(sizeof(double) * (size_t)nl * (cam.nrr + 1) * nfr));
  CUDA_TRY(md->dflux.ensure(sizeof(double) * (size_t)nl * nfr));
  CUDA_TRY(md->dcnt.ensure(sizeof(unsigned long long) * kWalkCounters));
  CUDA_TRY(md->dwork.ensure(sizeof(int)));
  CUDA_TRY(md->derr.ensure(sizeof(int)));
  CUDA_TRY(md->dlist.ensure(sizeof(unsigned short) * walk_list_elems(ctx->nsm, nfr)));
  if (mask_out) CUDA_TRY(md->dmask.ensure(nimg));
  if (rows) {
    for (int i = 0; i < rows->n; i++)
      if (rows->rays[i] < 0 || rows->rays[i] >= cam.nrays)
        return set_err(ctx, RL_ERR_ARG, "rl_image_rows: ray " + std::to_string(rows->rays[i]) + " outside 0.." +
                                            std::to_string(cam.nrays - 1));
    CUDA_TRY(md->drows.ensure(sizeof(int) * (size_t)rows->n));
    CUDA_TRY(md->drowout.ensure(sizeof(T) * (size_t)nl * rows->n * nfr));
  }
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  if (!cached) {
    CUDA_TRY(h2d(md->dtab.p, tab.data(), sizeof(T) * tab.size(), s));
    CUDA_TRY(h2d(md->dnsum.p, nsum.data(), sizeof(T) * nsum.size(), s));
    CUDA_TRY(h2d(md->dwch.p, wch.data(), sizeof(T) * wch.size(), s));
    CUDA_TRY(h2d(md->dstar.p, star.data(), sizeof(T) * star.size(), s));
    CUDA_TRY(h2d(md->dvelo.p, velo.data(), sizeof(double) * velo.size(), s));
    CUDA_TRY(h2d(md->dlc.p, lc.data(), sizeof(LineConst<T>) * lc.size(), s));
    CUDA_TRY(h2d(md->dscale.p, scale.data(), sizeof(double) * nl, s));
  }
  CUDA_TRY(cudaMemsetAsync(md->dcnt.p, 0, sizeof(unsigned long long) * kWalkCounters, s));
  CUDA_TRY(cudaMemsetAsync(md->dwork.p, 0, sizeof(int), s));
  CUDA_TRY(cudaMemsetAsync(md->derr.p, 0, sizeof(int), s));
  MaserFlags mf;
  CUDA_TRY(mf.arm(md->dmaser, mase, iline0, s));
  CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  WalkParams<T> P;
  P.nb = node_view<T>(md);
  P.maser = mf.dev;
  P.nth = m.nth; P.ncell = ncell; P.nlines = nl; P.nfr = nfr;
  int cpl = 4;
  {
    walk_shape(nl, nfr, P.gsize, cpl);                   // balanced line groups per ray
    P.nitems = ((nl + P.gsize - 1) / P.gsize) * cam.nrays;   // (line group, ray) work items
  }
  if (nfr >= 2048) return set_err(ctx, RL_ERR_ARG, "at most 2047 channels per line are supported");
  P.tab = md->dtab.as<T>(); P.nsum = md->dnsum.as<T>(); P.wch = md->dwch.as<T>(); P.velo = md->dvelo.as<double>();
  P.star = md->dstar.as<T>(); P.lc = md->dlc.as<LineConst<T>>();
  P.isrf = isrf_of(has_isrf, P.star, nl, nfr);
  P.aksmax_c = m.aksmax / 2.99792458e5;
  P.kq = (T)(3.33567e-6 * 2.99792458e5);
  P.fstar = (T)((m.rstar / cam.ri[1]) * (m.rstar / cam.ri[1]));
  P.img = md->dimg.as<T>();
  P.counters = md->dcnt.as<unsigned long long>();
  P.work = md->dwork.as<int>();
  P.err = md->derr.as<int>();
  P.list = md->dlist.as<unsigned short>();
  P.mask = mask_out ? md->dmask.as<unsigned char>() : nullptr;
  if (cam.ri[1] < m.rstar) return set_err(ctx, RL_ERR_ARG, "central beam smaller than the star");
  CUDA_TRY(launch_walk<T>(P, cpl, ctx->nsm, s, (md->checks & RL_CHECK_OVERSHOOT) != 0));
  CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  ReduceParams rp;
  rp.nrays = cam.nrays; rp.nfr = nfr; rp.nphi = cam.nphi; rp.nrr = cam.nrr; rp.nlines = nl;
  rp.ri = md->dri.as<double>(); rp.dist2 = 3.08572e18 * 3.08572e18; rp.scale = md->dscale.as<double>();
  CUDA_TRY(launch_reduce<T>(rp, md->dimg.as<T>(), md->dring.as<double>(), md->dflux.as<double>(), s));
  CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
  std::vector<T> rowbuf;
  if (rows && rows->n > 0) {
    rowbuf.resize((size_t)nl * rows->n * nfr);
    CUDA_TRY(h2d(md->drows.p, rows->rays, sizeof(int) * (size_t)rows->n, s));
    CUDA_TRY(launch_gather_rows<T>(md->dimg.as<T>(), cam.nrays, nfr, nl, md->drows.as<int>(), rows->n,
                                   md->drowout.as<T>(), s));
    CUDA_TRY(d2h(rowbuf.data(), md->drowout.p, sizeof(T) * rowbuf.size(), s));
  }
  if (flux_out)
    CUDA_TRY(d2h(flux_out, md->dflux.p, sizeof(double) * (size_t)nl * nfr, s));
  unsigned long long cnt[kWalkCounters] = {};
  int kerr = 0;
  CUDA_TRY(d2h(cnt, md->dcnt.p, sizeof(cnt), s));
  CUDA_TRY(d2h(&kerr, md->derr.p, sizeof(int), s));
  CUDA_TRY(mf.fetch(s));
  CUDA_TRY(cudaStreamSynchronize(s));
  mf.record(md->masing, m.lfreq.size());
  if (image_out) {
    std::vector<T> img(nimg);
    g_d2h += sizeof(T) * nimg;
    CUDA_TRY(cudaMemcpy(img.data(), md->dimg.p, sizeof(T) * nimg, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < nimg; i++) image_out[i] = (double)img[i] * scale[i / ((size_t)cam.nrays * nfr)];
  }
  for (size_t i = 0; i < rowbuf.size(); i++)
    rows->out[i] = (double)rowbuf[i] * scale[i / ((size_t)rows->n * nfr)];
  if (mask_out) {
    g_d2h += nimg;
    CUDA_TRY(cudaMemcpy(mask_out, md->dmask.p, nimg, cudaMemcpyDeviceToHost));
  }
  if (!cached) {
    md->tab_line0 = iline0; md->tab_nl = nl; md->tab_prec = md->precision; md->tab_scale = scale;
    md->tab_mase = mase;
    md->tab_isrf = has_isrf;
  }
  if (kerr != 0) return set_err(ctx, RL_ERR_GEOMETRY, "walk: error code " + std::to_string(kerr));
  if (st) {
    float a = 0, b = 0, c = 0;
    cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&c, ctx->ev[2], ctx->ev[3]);
    st->upload_ms += a; st->walk_ms += b; st->reduce_ms += c;
    st->steps += cnt[0]; st->integrated += cnt[1]; st->node_visits += cnt[2];
    st->node_passes += cnt[3]; st->packed_passes += cnt[4]; st->empty_steps += cnt[5];
    st->refined_passes += cnt[6]; st->sub_steps += cnt[7]; st->refined_channels += cnt[8];
    st->overshoots += cnt[9];
    st->ray_channels += (unsigned long long)cam.nrays * nfr * nl;
    st->nrays = cam.nrays; st->nfr = nfr; st->kmax = md->kmax; st->nlines += nl;
  }
  return 0;
}

static int dispatch_lines(rl_model* md, int iline0, int nl, double* flux, double* image, rl_stats* st,
                          unsigned char* mask = nullptr, const RowRequest* rows = nullptr) {
  g_h2d = 0; g_d2h = 0;
  const int rc = md->precision == RL_FP64 ? run_lines<double>(md, iline0, nl, flux, image, mask, st, rows)
                                          : run_lines<float>(md, iline0, nl, flux, image, mask, st, rows);
  if (st) { st->h2d_bytes += g_h2d; st->d2h_bytes += g_d2h; }
  return rc;
}

extern "C" {

int rl_create(rl_ctx** out, int device) {
  if (!out) return set_err(nullptr, RL_ERR_ARG, "rl_create: null output");
  *out = nullptr;
  std::unique_ptr<rl_ctx> c(new rl_ctx);
  c->device = device;
  rl_ctx* ctx = c.get();
  CUDA_TRY(cudaSetDevice(device));
  CUDA_TRY(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device));
  CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  for (auto& e : c->ev) CUDA_TRY(cudaEventCreate(&e));
  *out = c.release();
  return 0;
}

int rl_destroy(rl_ctx* ctx) {
  if (!ctx) return 0;
  cudaSetDevice(ctx->device);
  for (auto& e : ctx->ev) if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return 0;
}

int rl_last_error(rl_ctx* ctx, char* buf, size_t len) {
  const std::string& e = ctx ? ctx->err : g_last_error;
  if (buf && len) { std::snprintf(buf, len, "%s", e.c_str()); }
  return (int)e.size();
}

int rl_load_dir(rl_ctx* ctx, const char* dir, rl_model** out) {
  if (!dir || !out) return set_err(ctx, RL_ERR_ARG, "rl_load_dir: null argument");
  *out = nullptr;
  std::unique_ptr<rl_model> md(new rl_model);
  md->ctx = ctx;
  std::string err;
  if (load_dir(dir, md->m, err)) return set_err(ctx, RL_ERR_IO, err);
  camera_defaults(md.get());
  md->pvspec = md->m.pv;
  *out = md.release();
  return 0;
}

int rl_load_arrays(rl_ctx* ctx, const rl_model_arrays* a, rl_model** out) {
  if (!a || !out) return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: null argument");
  *out = nullptr;
  if (a->nr < 3 || a->nth < 2 || a->nlev < 2 || a->nlines_mol < 1 || !a->radius || !a->theta || !a->rho ||
      !a->abund || !a->width || !a->vel || !a->pop || !a->lev_up || !a->lev_low || !a->aud || !a->energy_cm ||
      !a->gdeg)
    return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: missing or inconsistent arrays");
  if (a->line_dust && (a->ncont < 2 || !a->freq || !a->dust_rho || !a->dust_temp || !a->kappa_abs || !a->kappa_scat))
    return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: dust arrays required with line_dust");
  std::unique_ptr<rl_model> md(new rl_model);
  md->ctx = ctx;
  Model& m = md->m;
  m.nr = a->nr; m.nth = a->nth; m.ny = 2 * a->nth;
  const int ncell = m.ncell();
  m.R.assign(m.nr + 4, 0.0);
  for (int i = 0; i < m.nr; i++) m.R[i + 2] = a->radius[i];
  auto R = [&](int ix) -> double& { return m.R[ix + 1]; };
  R(0) = R(1) * R(1) / R(2); R(-1) = R(0) * R(0) / R(1);
  R(m.nr + 1) = R(m.nr) * R(m.nr) / R(m.nr - 1); R(m.nr + 2) = R(m.nr + 1) * R(m.nr + 1) / R(m.nr);
  for (int ix = 1; ix < m.nr; ix++)
    if (!(R(ix + 1) > R(ix)) || R(ix + 1) / R(ix) - 1.0 < 1.0e-6)
      return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: radii must increase by more than the telescope safety number");
  m.TH.assign(m.ny + 4, 0.0);
  for (int i = 0; i < m.nth; i++) {
    if (a->theta[i] < 0.0 || a->theta[i] > 1.5707963268) return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: theta outside [0, pi/2]");
    m.TH[i + 2] = a->theta[i];
  }
  auto T = [&](int iy) -> double& { return m.TH[iy + 1]; };
  for (int iy = 1; iy <= m.nth; iy++) T(2 * m.nth + 1 - iy) = 3.14159265359 - T(iy);
  T(0) = -T(1); T(-1) = -T(2);
  const double twopi_f = (double)(2.0f * 3.1415926f);
  T(m.ny + 1) = twopi_f - T(m.ny); T(m.ny + 2) = twopi_f - T(m.ny - 1);
  m.rho.assign(a->rho, a->rho + ncell);
  m.abun.assign(a->abund, a->abund + ncell);
  m.lw.assign(a->width, a->width + ncell);
  m.vel.assign(a->vel, a->vel + 3 * (size_t)ncell);
  m.nlev = a->nlev;
  m.pop.assign(a->pop, a->pop + (size_t)ncell * a->nlev);
  m.Ecm.assign(a->energy_cm, a->energy_cm + a->nlev);
  m.gdeg.assign(a->gdeg, a->gdeg + a->nlev);
  m.lup.assign(a->lev_up, a->lev_up + a->nlines_mol);
  m.ldn.assign(a->lev_low, a->lev_low + a->nlines_mol);
  m.Aud.assign(a->aud, a->aud + a->nlines_mol);
  m.lfreq.resize(a->nlines_mol);
  for (int i = 0; i < a->nlines_mol; i++) {
    if (m.lup[i] < 1 || m.ldn[i] < 1 || m.lup[i] > m.nlev || m.ldn[i] > m.nlev || m.lup[i] <= m.ldn[i])
      return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: invalid line levels");
    m.lfreq[i] = 1.509160e26 * (1.986468498e-16 * m.Ecm[m.lup[i] - 1] - 1.986468498e-16 * m.Ecm[m.ldn[i] - 1]);
    if (!(m.lfreq[i] > 0.0)) return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: non-positive line frequency");
  }
  m.umass = a->umass;
  m.line_dust = a->line_dust;
  m.ncont = a->ncont;
  if (a->ncont > 0 && a->freq) m.cnu.assign(a->freq, a->freq + a->ncont);
  if (m.line_dust) {
    m.nspec = 1;
    m.nsize.assign(1, 1);
    m.drho.assign(a->dust_rho, a->dust_rho + ncell);
    m.dtemp.assign((size_t)4 * ncell, 0.0);
    std::copy(a->dust_temp, a->dust_temp + ncell, m.dtemp.begin());
    m.kabs.assign((size_t)4 * m.ncont, 0.0);
    m.ksca.assign((size_t)4 * m.ncont, 0.0);
    std::copy(a->kappa_abs, a->kappa_abs + m.ncont, m.kabs.begin());
    std::copy(a->kappa_scat, a->kappa_scat + m.ncont, m.ksca.begin());
  }
  m.rstar = a->rstar;
  m.starcont.assign(std::max(m.ncont, 0), 0.0);
  m.starpump = a->star_flux_1pc ? 1 : 0;
  if (a->star_flux_1pc)
    for (int i = 0; i < m.ncont; i++) m.starcont[i] = 3.0308410e36 * a->star_flux_1pc[i] / (m.rstar * m.rstar);
  m.outer_bc = a->outer_bc;
  if (m.outer_bc != 0 && m.outer_bc != 2) return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: outer boundary 0 or 2 (type 3 needs interstellfield.inp: use rl_load_dir)");
  m.incl_rad = a->incl_deg * 0.0174532925199;
  m.nphi = a->nphi; m.dbdr = a->dbdr; m.nrext = a->nrrayextra;
  m.vmax = a->vmax; m.dv = a->dv; m.radvelo = a->radvelo;
  m.ilstart = a->ilinestart; m.nlspec = a->nlines_spec; m.style = 1;
  m.molname = a->molname ? a->molname : "moldata";
  m.molfile = m.molname + ".dat";
  finish_model(m);
  if (m.nfr < 2) return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: passband needs at least 2 channels");
  if (m.ilstart < 1 || m.ilstart + m.nlspec - 1 > a->nlines_mol) return set_err(ctx, RL_ERR_ARG, "rl_load_arrays: line range");
  camera_defaults(md.get());
  *out = md.release();
  return 0;
}

int rl_model_free(rl_model* md) {
  if (!md) return 0;
  if (md->ctx) cudaSetDevice(md->ctx->device);
  delete md;
  return 0;
}

int rl_model_checksum(rl_model* md, unsigned long long* out) {
  if (!md || !out) return set_err(nullptr, RL_ERR_ARG, "rl_model_checksum: null argument");
  *out = model_checksum(md->m);
  return 0;
}

int rl_model_get_info(rl_model* md, rl_model_info* info) {
  if (!md || !info) return set_err(nullptr, RL_ERR_ARG, "rl_model_get_info: null argument");
  const Model& m = md->m;
  std::memset(info, 0, sizeof *info);
  info->nr = m.nr; info->nth = m.nth; info->nlev = m.nlev; info->nlines_mol = (int)m.lfreq.size();
  info->nlines_spec = m.nlspec; info->ilinestart = m.ilstart; info->nfr = m.nfr; info->nphi = md->nphi;
  info->dbdr = md->dbdr; info->nrrayextra = md->nrext;
  info->nrings = std::abs(md->nrext) + 10 + md->dbdr * (m.nr - 1);
  info->nrays = 1 + info->nrings * md->nphi;
  info->outer_bc = m.outer_bc; info->starpump = m.starpump; info->line_dust = m.line_dust;
  info->precision = md->precision;
  info->incl_deg = md->incl_rad * 57.2957795132; info->vmax = m.vmax; info->dv = m.dv; info->rstar = m.rstar;
  info->aksmax = m.aksmax;
  return 0;
}

int rl_set_camera(rl_model* md, double incl_deg, int nphi, int dbdr, int nrrayextra) {
  if (!md) return set_err(nullptr, RL_ERR_ARG, "rl_set_camera: null model");
  rl_ctx* ctx = md->ctx;
  if (md->incl_rad == incl_deg * 0.0174532925199 && md->nphi == nphi && md->dbdr == dbdr && md->nrext == nrrayextra)
    return 0;
  if (nphi < 1 || dbdr < 1 || nrrayextra == 0 || incl_deg == 0.0)
    return set_err(ctx, RL_ERR_ARG, "rl_set_camera: need nphi>0, dbdr>0, nrrayextra!=0, inclination!=0");
  md->incl_rad = incl_deg * 0.0174532925199;
  md->nphi = nphi; md->dbdr = dbdr; md->nrext = nrrayextra;
  md->geo_ready = false;
  return 0;
}

int rl_set_precision(rl_model* md, int precision) {
  if (!md) return set_err(nullptr, RL_ERR_ARG, "rl_set_precision: null model");
  if (precision != RL_FP32 && precision != RL_FP64) return set_err(md->ctx, RL_ERR_ARG, "rl_set_precision: RL_FP32 or RL_FP64");
  if (precision != md->precision) md->geo_ready = false;
  md->precision = precision;
  return 0;
}

int rl_set_checks(rl_model* md, int flags) {
  if (!md) return set_err(nullptr, RL_ERR_ARG, "rl_set_checks: null model");
  if (flags & ~RL_CHECK_OVERSHOOT) return set_err(md->ctx, RL_ERR_ARG, "rl_set_checks: unknown flags");
  md->checks = flags;
  return 0;
}

int rl_line_spectrum(rl_model* md, int iline, double* flux_out, double* velo_out, rl_stats* st) {
  if (!md || !flux_out) return set_err(nullptr, RL_ERR_ARG, "rl_line_spectrum: null argument");
  rl_ctx* ctx = md->ctx;
  if (!ctx) return set_err(nullptr, RL_ERR_STATE, "model was loaded without a device context");
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  int rc = dispatch_lines(md, iline, 1, flux_out, nullptr, st);
  if (rc) return rc;
  if (velo_out) {
    const Model& m = md->m;
    const double lf = m.lfreq[iline - 1], nu0 = std::fabs(lf);
    const double passb = 3.33567e-6 * nu0 * m.vmax, dnu = 2.0 * passb / (m.nfr - 1.0);
    for (int k = 0; k < m.nfr; k++) velo_out[k] = -2.99792458e5 * ((nu0 + (-passb + k * dnu)) - lf) / lf + m.radvelo;
  }
  return 0;
}

int rl_spectra(rl_model* md, int iline0, int nlines, double* flux_out, rl_stats* st) {
  if (!md || !flux_out) return set_err(nullptr, RL_ERR_ARG, "rl_spectra: null argument");
  rl_ctx* ctx = md->ctx;
  if (!ctx) return set_err(nullptr, RL_ERR_STATE, "model was loaded without a device context");
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return dispatch_lines(md, iline0, nlines, flux_out, nullptr, st);
}

int rl_line_image(rl_model* md, int iline, double* image_out, rl_stats* st) {
  if (!md || !image_out) return set_err(nullptr, RL_ERR_ARG, "rl_line_image: null argument");
  rl_ctx* ctx = md->ctx;
  if (!ctx) return set_err(nullptr, RL_ERR_STATE, "model was loaded without a device context");
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return dispatch_lines(md, iline, 1, nullptr, image_out, st);
}

int rl_image_rows(rl_model* md, int iline0, int nlines, int nsel, const int* rays, double* flux_out, double* rows_out,
                  rl_stats* st) {
  if (!md || (nsel > 0 && (!rays || !rows_out)) || nsel < 0)
    return set_err(nullptr, RL_ERR_ARG, "rl_image_rows: null argument or negative ray count");
  rl_ctx* ctx = md->ctx;
  if (!ctx) return set_err(nullptr, RL_ERR_STATE, "model was loaded without a device context");
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  RowRequest rq;
  rq.rays = rays; rq.n = nsel; rq.out = rows_out;
  return dispatch_lines(md, iline0, nlines, flux_out, nullptr, st, nullptr, &rq);
}

int rl_line_image_mask(rl_model* md, int iline, double* image_out, unsigned char* mask_out, rl_stats* st) {
  if (!md || !image_out || !mask_out) return set_err(nullptr, RL_ERR_ARG, "rl_line_image_mask: null argument");
  rl_ctx* ctx = md->ctx;
  if (!ctx) return set_err(nullptr, RL_ERR_STATE, "model was loaded without a device context");
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return dispatch_lines(md, iline, 1, nullptr, image_out, st, mask_out);
}

int rl_run_dir(const char* dir, int device, rl_stats* st) { return rl_run_dir_ex(dir, device, 0, st); }

// radlite.log: the record the reference appends around the telescope step
// (write_logmessage_start/_end, main.F:983-985, 1093-1095, 1121-1588), one line per
// list-directed write (a leading blank, integers in 12 columns). The start record lists
// the compile-time switches of the reference's spectrum build whose raytrace this library
// reproduces (configure_spectrum.h; the short-characteristics, ALI and interpolation
// switches of its level-population solver have no counterpart here), the precision of
// this run, and the raytrace's part of the problem setup. The end record lists the
// warnings the raytrace can raise: the overshoot warning (main.F:1547-1552).
static void log_stamp(char* d, size_t nd, char* h, size_t nh) {
  const auto now = std::chrono::system_clock::now();
  const std::time_t t = std::chrono::system_clock::to_time_t(now);
  const int ms = (int)(std::chrono::duration_cast<std::chrono::milliseconds>(now.time_since_epoch()).count() % 1000);
  std::tm tmv;
  localtime_r(&t, &tmv);
  std::snprintf(d, nd, "%02d-%02d-%04d", tmv.tm_mday, tmv.tm_mon + 1, tmv.tm_year + 1900);
  std::snprintf(h, nh, "%02d:%02d:%02d.%03d", tmv.tm_hour, tmv.tm_min, tmv.tm_sec, ms);
}

static void run_log_start(const std::string& dir, const rl_model* md, int flags) {
  FILE* fp = std::fopen((dir + "/radlite.log").c_str(), "a");
  if (!fp) return;
  char d[32], h[32];
  log_stamp(d, sizeof d, h, sizeof h);
  const Model& m = md->m;
  std::fprintf(fp, "\n\n\n =========== RUN OF RADICAL ===========\n Action       : spectrum/image\n"
                   " Starting Date: %s\n          Time: %s\n ......................................\n"
                   "       COMPILATION OF CODE:            \n",
               d, h);
  std::fprintf(fp,
               " Dimension = 2              (RADGRID_TWODIM)\n"
               " Include lines              (INCLUDE_LINES)\n"
               " Include dust continuum     (INCLUDE_DUST)\n"
               " Mirror in Theta : yes      (MIRROR_THETA)\n"
               " Quadrature                 (SRCQDR_PNT_2)\n"
               " Line profile refinement    (SUBGRID)\n"
               " Velocity window per ray    (NONREDUNDANT)\n"
               " Star in the central beam   (CENTRAL_SOURCE)\n");
  if (flags & RL_RUN_SAVE_IMCIR) std::fprintf(fp, " Circular images saved      (SAVE_IMCIR)\n");
  std::fprintf(fp, " radlite_gb300 line raytrace (GB300, sm_103a): %s\n",
               md->precision == RL_FP64 ? "FP64 transfer, FP64 crossings" : "FP32 transfer, FP64 crossings");
  std::fprintf(fp, " \n ......................................\n           SETUP OF PROBLEM:           \n");
  std::fprintf(fp, " frsize radius      = %12d\n frsize theta       = %12d\n bound cond outer   = %12d\n",
               m.nr, m.nth, m.outer_bc);
  std::fprintf(fp, " telescope nphi     = %12d\n telescope dbdr     = %12d\n telescope extra b  = %12d\n",
               md->nphi, md->dbdr, md->nrext);
  std::fprintf(fp, " \n");
  std::fclose(fp);
}

static void run_log_end(const std::string& dir, unsigned long long overshoots) {
  FILE* fp = std::fopen((dir + "/radlite.log").c_str(), "a");
  if (!fp) return;
  char d[32], h[32];
  log_stamp(d, sizeof d, h, sizeof h);
  std::fprintf(fp, " ......................................\n Warnings:\n");
  if (overshoots > 0)
    std::fprintf(fp, " * During Short Characteristic integration     \n"
                     "   there were overshoots in the quadrature.    \n"
                     "   These have been corrected automatically,    \n"
                     "   but they indicate poor grid resolution!     \n");
  else
    std::fprintf(fp, " <none>\n");
  std::fprintf(fp, " ......................................\n Finishing Date: %s\n          Time: %s\n"
                   " ========= END OF RUN RADLITE =========\n",
               d, h);
  std::fclose(fp);
}

// The warning make_freq_image_rectang prints after an image whose quadrature overshot
// (telescope.F:2204-2213).
static void warn_overshoot_image() {
  std::printf(" \n -----------------------------------------------\n"
              " |  WARNING:                                   |\n"
              " |  While making the image there were serious  |\n"
              " |  overshoots in the quadrature.              |\n"
              " |  These have been corrected automatically,   |\n"
              " |  but they indicate poor grid resolution!    |\n"
              " -----------------------------------------------\n");
  std::fflush(stdout);
}

// The reference's warning after each line whose render found masing: calc_line_spectrum
// writes it with (A35,I10) (telescope.F:1649-1652), calc_write_line_posvel list-directed
// (telescope.F:2020-2023).
static void warn_masing(const rl_model* md, int iline0, int nl, bool posvel) {
  for (int l = 0; l < nl; l++) {
    const size_t i = (size_t)iline0 - 1 + l;
    if (i < md->masing.size() && md->masing[i])
      std::printf("%s\n Will only warn once for this transition.\n",
                  posvel ? " WARNING: Masing detected!" : "          WARNING: Masing detected!");
  }
  std::fflush(stdout);   // in order with the caller's own output
}

int rl_run_dir_ex(const char* dir, int device, int flags, rl_stats* st_out) {
  if (flags & ~RL_RUN_SAVE_IMCIR) return set_err(nullptr, RL_ERR_ARG, "rl_run_dir_ex: unknown flags");
  rl_stats own;
  rl_stats* st = st_out ? st_out : &own;   // the run's totals feed the log's warnings
  std::memset(st, 0, sizeof *st);
  unsigned long long last_over = 0;        // overshoots of the last rendered image
  rl_ctx* ctx = nullptr;
  int rc = rl_create(&ctx, device);
  if (rc) return rc;
  rl_model* md = nullptr;
  rc = rl_load_dir(ctx, dir, &md);
  if (rc == 0) {
    md->checks = RL_CHECK_OVERSHOOT;   // the reference's default build takes the test
    run_log_start(dir, md, flags);
  }
  if (rc == 0 && md->m.command == 2 && md->m.pv.sizespec == 0) {   // telescope.F:207-210
    std::printf(" While reading linespectrum.inp:\n Size specifier in arcsec not yet implemented\n");
    std::fflush(stdout);
  }
  if (rc == 0 && md->m.command == 2) {
    // one lineposvel file per line (main.F:1061-1074); lines in chunks of at most 2 GB of
    // cube per array
    const Model& m = md->m;
    if (st) std::memset(st, 0, sizeof *st);
    PVCamera pc;
    std::string err;
    if (setup_pv_camera(m, md->pvspec, md->incl_rad, pc, err)) rc = set_err(ctx, RL_ERR_ARG, err);
    const size_t per_line = (size_t)m.nfr * pc.nx * pc.ny;
    const int chunk = rc ? 1 : (int)std::max<size_t>(1, std::min<size_t>(m.nlspec, (size_t)(2u << 30) / (8 * per_line + 1)));
    std::vector<double> I, tau;
    for (int l0 = 0; l0 < m.nlspec && rc == 0; l0 += chunk) {
      const int nl = std::min(chunk, m.nlspec - l0);
      I.resize(per_line * nl);
      tau.resize(per_line * nl);
      const unsigned long long over0 = st->overshoots;
      rc = dispatch_posvel(md, m.ilstart + l0, nl, I.data(), tau.data(), st);
      if (rc == 0) warn_masing(md, m.ilstart + l0, nl, true);
      // the reference clears its counter per rectangular image (telescope.F:2094); a
      // launch here renders the lines of one chunk
      last_over = st->overshoots - over0;
      if (rc == 0 && last_over > 0) warn_overshoot_image();
      for (int l = 0; l < nl && rc == 0; l++) {
        const int iline = m.ilstart + l0 + l;
        const std::string name = posvel_file_name(m, iline);
        if (name.empty()) { rc = set_err(ctx, RL_ERR_ARG, "position-velocity file names stop at line 99"); break; }
        if (write_posvel_file(std::string(dir) + "/" + name, m, pc, md->pvspec, iline, &I[per_line * l],
                              &tau[per_line * l], err))
          rc = set_err(ctx, RL_ERR_IO, err);
      }
    }
    if (rc == 0) {
      FILE* fp = std::fopen((std::string(dir) + "/radlite.success").c_str(), "w");
      if (fp) { std::fprintf(fp, " 1\n"); std::fclose(fp); }
    }
  } else if (rc == 0 && (flags & RL_RUN_SAVE_IMCIR)) {
    // a SAVE_IMCIR build: line by line, the circular image beside the spectrum
    // (telescope.F:1594-1615); the integration mask accumulates over the run's lines
    // because the reference never clears imcir_cmask
    const Model& m = md->m;
    std::vector<double> flux((size_t)m.nlspec * m.nfr);
    if (st) std::memset(st, 0, sizeof *st);
    std::vector<double> img;
    std::vector<unsigned char> mask, sticky;
    std::string err;
    for (int l = 0; l < m.nlspec && rc == 0; l++) {
      const int iline = m.ilstart + l;
      rl_stats one;
      std::memset(&one, 0, sizeof one);
      const int nrings = std::abs(md->nrext) + 10 + md->dbdr * (m.nr - 1);   // setup_camera's ring count
      const size_t n = (size_t)(1 + nrings * md->nphi) * m.nfr;
      img.resize(n); mask.resize(n);
      if (sticky.empty()) sticky.assign(n, 0);
      rc = dispatch_lines(md, iline, 1, &flux[(size_t)l * m.nfr], img.data(), &one, mask.data());
      if (rc) break;
      warn_masing(md, iline, 1, false);
      for (size_t i = 0; i < n; i++) sticky[i] |= mask[i];
      if (st) {
        st->steps += one.steps; st->integrated += one.integrated; st->node_visits += one.node_visits;
        st->ray_channels += one.ray_channels; st->walk_ms += one.walk_ms; st->geometry_ms += one.geometry_ms;
        st->reduce_ms += one.reduce_ms; st->upload_ms += one.upload_ms; st->nlines += 1;
        st->overshoots += one.overshoots;
        st->nrays = one.nrays; st->nfr = one.nfr; st->kmax = one.kmax;
      }
      const std::string name = imcir_file_name(m, iline);
      if (name.empty()) { rc = set_err(ctx, RL_ERR_ARG, "circular-image file names stop at line 99"); break; }
      if (write_imcir_file(std::string(dir) + "/" + name, m, md->cam, iline, img.data(), sticky.data(), err))
        rc = set_err(ctx, RL_ERR_IO, err);
    }
    if (rc == 0) {
      std::vector<int> lines;
      for (int i = 0; i < m.nlspec; i++) lines.push_back(m.ilstart + i);
      if (write_spectrum_file(std::string(dir) + "/linespectrum_" + m.molname + ".dat", m, md->cam, lines, flux, err))
        rc = set_err(ctx, RL_ERR_IO, err);
      else {
        FILE* fp = std::fopen((std::string(dir) + "/radlite.success").c_str(), "w");
        if (fp) { std::fprintf(fp, " 1\n"); std::fclose(fp); }
      }
    }
  } else if (rc == 0) {
    const Model& m = md->m;
    std::vector<double> flux((size_t)m.nlspec * m.nfr);
    if (st) std::memset(st, 0, sizeof *st);
    rc = dispatch_lines(md, m.ilstart, m.nlspec, flux.data(), nullptr, st);
    if (rc == 0) warn_masing(md, m.ilstart, m.nlspec, false);
    if (rc == 0) {
      std::vector<int> lines;
      for (int i = 0; i < m.nlspec; i++) lines.push_back(m.ilstart + i);
      std::string err;
      if (write_spectrum_file(std::string(dir) + "/linespectrum_" + m.molname + ".dat", m, md->cam, lines, flux, err))
        rc = set_err(ctx, RL_ERR_IO, err);
      else {
        FILE* fp = std::fopen((std::string(dir) + "/radlite.success").c_str(), "w");
        if (fp) { std::fprintf(fp, " 1\n"); std::fclose(fp); }
      }
    }
  }
  // circular images never clear the counter: a spectrum run warns for any overshoot
  if (rc == 0) run_log_end(dir, md->m.command == 2 ? last_over : st->overshoots);
  if (rc) g_last_error = ctx->err;
  rl_model_free(md);
  rl_destroy(ctx);
  return rc;
}

int rl_line_masing(rl_model* md, int iline, int* detected) {
  if (!md || !detected) return set_err(nullptr, RL_ERR_ARG, "rl_line_masing: null argument");
  if (iline < 1 || iline > (int)md->m.lfreq.size()) return set_err(md->ctx, RL_ERR_ARG, "rl_line_masing: line index out of range");
  *detected = (size_t)iline <= md->masing.size() ? md->masing[(size_t)iline - 1] : 0;
  return 0;
}

int rl_measure_peaks(rl_ctx* ctx, double* ffma_per_s, double* ex2_per_s) {
  if (!ctx || !ffma_per_s || !ex2_per_s) return set_err(ctx, RL_ERR_ARG, "rl_measure_peaks: null argument");
  CUDA_TRY(rl::enter_device(ctx->device));
  CUDA_TRY(measure_peaks(ctx->nsm, ctx->stream, ffma_per_s, ex2_per_s));
  return 0;
}

int rl_debug_trajectory(rl_model* md, int iray, int cap, double* s, double* r, double* th, double* mu, double* dvmu,
                        int* icr, int* ir, int* it) {
  if (!md) return set_err(nullptr, RL_ERR_ARG, "rl_debug_trajectory: null model");
  rl_ctx* ctx = md->ctx;
  if (!ctx) return set_err(nullptr, RL_ERR_STATE, "model was loaded without a device context");
  CUDA_TRY(rl::enter_device(ctx->device));
  int rc = upload_grid(md);
  if (rc) return rc;
  std::string err;
  Camera cam;
  if (setup_camera(md->m, md->incl_rad, md->nphi, md->dbdr, md->nrext, cam, err)) return set_err(ctx, RL_ERR_ARG, err);
  if (iray < 0 || iray >= cam.nrays) return set_err(ctx, RL_ERR_ARG, "rl_debug_trajectory: ray index out of range");
  if (cap < 0) return set_err(ctx, RL_ERR_ARG, "rl_debug_trajectory: negative capacity");
  const int kmax = rlg::max_nodes(md->m.nr, md->m.nth);
  cudaStream_t st = ctx->stream;
  DevBuf bx0, bz0, bnn, bst, bds, bdvf, bvl, bdvs, blw, bwr, bwt, bc00, bmisc, dbg, arr;
  CUDA_TRY(bx0.ensure(sizeof(double))); CUDA_TRY(bz0.ensure(sizeof(double)));
  CUDA_TRY(bnn.ensure(sizeof(int))); CUDA_TRY(bst.ensure(sizeof(int)));
  CUDA_TRY(bds.ensure(sizeof(double) * kmax)); CUDA_TRY(bdvf.ensure(sizeof(float) * kmax));
  CUDA_TRY(bvl.ensure(sizeof(double) * kmax)); CUDA_TRY(bdvs.ensure(sizeof(double) * kmax));
  CUDA_TRY(blw.ensure(sizeof(double) * kmax)); CUDA_TRY(bwr.ensure(sizeof(double) * kmax));
  CUDA_TRY(bwt.ensure(sizeof(double) * kmax)); CUDA_TRY(bc00.ensure(sizeof(int) * kmax));
  CUDA_TRY(bmisc.ensure(sizeof(unsigned) * kmax));
  const size_t per = (size_t)kmax;
  CUDA_TRY(arr.ensure((sizeof(double) * 5 + sizeof(int) * 3) * per));
  CUDA_TRY(dbg.ensure(sizeof(TrajDebug)));
  TrajDebug h;
  char* base = arr.as<char>();
  h.s = (double*)base; h.r = h.s + per; h.th = h.r + per; h.mu = h.th + per; h.dvmu = h.mu + per;
  h.icr = (int*)(h.dvmu + per); h.ir = h.icr + per; h.it = h.ir + per; h.cap = kmax;
  CUDA_TRY(h2d(dbg.p, &h, sizeof h, st));
  CUDA_TRY(h2d(bx0.p, &cam.x0[iray], sizeof(double), st));
  CUDA_TRY(h2d(bz0.p, &cam.z0[iray], sizeof(double), st));
  GeoParams p;
  const Model& m = md->m;
  p.nr = m.nr; p.nth = m.nth; p.ny = m.ny; p.rstar = m.rstar; p.theta0 = cam.theta0;
  p.R = md->dR.as<double>(); p.TH = md->dTH.as<double>(); p.tan2 = md->dtan2.as<double>();
  p.vel = md->dvel.as<double>(); p.lw = md->dlw.as<double>(); p.x0 = bx0.as<double>(); p.z0 = bz0.as<double>();
  p.velf = md->dvelf.as<float>(); p.vell = md->dvell.as<float>(); p.lwf = md->dlwf.as<float>();
  NodeBuf<double> nb;
  nb.nrays = 1; nb.kmax = kmax; nb.nnodes = bnn.as<int>(); nb.status = bst.as<int>();
  nb.ds = bds.as<double>(); nb.dvf = bdvf.as<float>(); nb.vl = bvl.as<double>(); nb.dvseg = bdvs.as<double>();
  nb.lw = blw.as<double>(); nb.wr = bwr.as<double>(); nb.wt = bwt.as<double>(); nb.c00 = bc00.as<int>();
  nb.misc = bmisc.as<unsigned>();
  CUDA_TRY(launch_geometry<double>(p, nb, 0, 1, dbg.as<TrajDebug>(), st));
  int n = 0, status = 0;
  CUDA_TRY(d2h(&n, bnn.p, sizeof(int), st));
  CUDA_TRY(d2h(&status, bst.p, sizeof(int), st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (status != 0) return set_err(ctx, RL_ERR_GEOMETRY, "geometry status " + std::to_string(status));
  const int c = std::min(n, cap);
  std::vector<double> hd(5 * per);
  std::vector<int> hi(3 * per);
  CUDA_TRY(cudaMemcpy(hd.data(), h.s, sizeof(double) * 5 * per, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(hi.data(), h.icr, sizeof(int) * 3 * per, cudaMemcpyDeviceToHost));
  for (int k = 0; k < c; k++) {
    if (s) s[k] = hd[k];
    if (r) r[k] = hd[per + k];
    if (th) th[k] = hd[2 * per + k];
    if (mu) mu[k] = hd[3 * per + k];
    if (dvmu) dvmu[k] = hd[4 * per + k];
    if (icr) icr[k] = hi[k];
    if (ir) ir[k] = hi[per + k];
    if (it) it[k] = hi[2 * per + k];
  }
  return n;
}

}  // extern "C"
