// rl_posvel.cu -- the position-velocity cube: linespectrum command 2 of the reference
// (calc_write_line_posvel, make_freq_image_rectang, setup_rays_rectang;
// telescope.F:1828-2475).
//
//   rays      the rectangular camera's pixel rays (host FP64, setup_pv_camera); pixels with
//             impact parameter b >= 0.999 R_nr are empty and never traced, the central ray
//             is traced only when the unresolved star is added.
//   k_geometry    the circular image's node kernel over the traced rays.
//   k_walk_pv     the circular image's walk with every channel of every ray integrated, no
//                 star mixing (charintline with rbeam 0) and the line-of-sight optical depth
//                 char_tau of each channel (Kahan-compensated in FP32); it counts the steps
//                 that fail the overshoot test (transfer.F:1548-1553) as well.
//   k_posvel_cube image epilogue instead of the spectrum reduction: scatter the traced rays
//                 into the [line][channel][iy][ix] cube in FP64, apply the intensity scale
//                 and smear the unresolved star over the four central pixels
//                 (telescope.F:2152-2206).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "rl_geometry.cuh"
#include "rl_internal.h"
#include "rl_walk.cuh"

namespace rl {

template <typename T, int C>
__global__ void __launch_bounds__(128, WalkMinBlocks<T>::value) k_walk_pv(WalkParams<T> P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  WarpSmem<T, C> W(smem_raw, nw, wib, kItemLines * P.nfr, P.list);
  unsigned long long steps = 0;   // this lane's formal-solution steps
  zero_counters(*W.SW, lane);
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(P.work, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= P.nitems) break;
    walk_item<T, C, true, false, true>(P, item, *W.S, *W.SS, *W.SW, W.list, lane, steps);
  }
  flush_counters(steps, *W.SW, P.counters, lane);
}

struct CubeParams {
  int nl, nfr, nx, ny, ntr;   // ntr: traced rays
  const int* pix;             // [nx*ny] traced ray of pixel (ix outer, iy inner), -1 = empty
  int star;                   // traced index of the central ray, -1 = no star added
  double srat;                // pi R*^2 / (4 spx spy)
  const double* scale;        // [nl] intensity scale of the walk
};

// One thread per output value; the cube is written in the file's order (per line and
// channel, iy outer, ix inner). The walk's image is [line][ray][channel].
template <typename T>
__global__ void k_posvel_cube(CubeParams c, const T* __restrict__ img, const T* __restrict__ tau,
                              double* __restrict__ I, double* __restrict__ tauo) {
  const size_t npix = (size_t)c.nx * c.ny;
  const size_t total = (size_t)c.nl * c.nfr * npix;
  const int cx = c.nx / 2, cy = c.ny / 2;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total; o += (size_t)gridDim.x * blockDim.x) {
    const size_t p = o % npix, lk = o / npix;
    const int k = (int)(lk % c.nfr), l = (int)(lk / c.nfr);
    const int ix = (int)(p % c.nx), iy = (int)(p / c.nx);
    const int t = __ldg(&c.pix[(size_t)ix * c.ny + iy]);
    double Iv = 0.0, tv = 0.0;
    if (t >= 0) {
      const size_t a = ((size_t)l * c.ntr + t) * c.nfr + k;
      Iv = (double)img[a] * c.scale[l];
      tv = (double)tau[a];
    }
    if (c.star >= 0 && (ix == cx - 1 || ix == cx) && (iy == cy - 1 || iy == cy)) {
      const double d = ((double)img[((size_t)l * c.ntr + c.star) * c.nfr + k] * c.scale[l]) * c.srat;
      Iv = d + (1.0 - c.srat) * Iv;
    }
    I[o] = Iv;
    tauo[o] = tv;
  }
}

template <typename T, int C>
static cudaError_t launch_walk_pv_c(const WalkParams<T>& P, int nsm, cudaStream_t s) {
  const int warps = kWalkWarps, threads = warps * 32;
  const size_t smem = (sizeof(WarpStage<T>) + sizeof(SlotState<T, C>) + sizeof(SubWork<T>)) * warps;
  cudaError_t e = cudaFuncSetAttribute(k_walk_pv<T, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_pv<T, C>, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (per_sm > kWalkBlocksPerSm) per_sm = kWalkBlocksPerSm;   // the list scratch holds this many
  long long blocks = (long long)nsm * per_sm;
  const long long need = ((long long)P.nitems + warps - 1) / warps;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  k_walk_pv<T, C><<<(unsigned)blocks, threads, smem, s>>>(P);
  return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_walk_pv(const WalkParams<T>& P, int cpl, int nsm, cudaStream_t s) {
  static_assert(!kListInSmem, "the position-velocity walk keeps its list in global scratch");
  switch (cpl) {
    case 1: return launch_walk_pv_c<T, 1>(P, nsm, s);
    case 2: return launch_walk_pv_c<T, 2>(P, nsm, s);
    case 4: return launch_walk_pv_c<T, 4>(P, nsm, s);
    default: return launch_walk_pv_c<T, 8>(P, nsm, s);
  }
}

// Lines iline0 .. iline0+nl-1 of the model's rectangular image; I_out and tau_out are
// [nl][nfr][ny][nx] (either may be null).
template <typename T>
static int run_posvel(rl_model* md, int iline0, int nl, double* I_out, double* tau_out, rl_stats* st) {
  rl_ctx* ctx = md->ctx;
  cudaStream_t s = ctx->stream;
  const Model& m = md->m;
  if (nl < 1 || iline0 < 1 || iline0 + nl - 1 > (int)m.lfreq.size())
    return set_err(ctx, RL_ERR_ARG, "line range outside the molecule's line list");
  if (m.nfr >= 2048) return set_err(ctx, RL_ERR_ARG, "at most 2047 channels per line are supported");
  std::string err;
  PVCamera pc;
  if (setup_pv_camera(m, md->pvspec, md->incl_rad, pc, err)) return set_err(ctx, RL_ERR_ARG, err);
  int rc = upload_grid(md);
  if (rc) return rc;
  // traced rays: the pixels inside 0.999 R_nr (telescope.F:2120) and the central ray
  const int npix = pc.nx * pc.ny;
  std::vector<int> pix(npix, -1);
  std::vector<double> tx, tz;
  tx.reserve(npix + 1); tz.reserve(npix + 1);
  for (int r = 0; r < npix; r++) {
    if (pc.b[r] < 0.999 * pc.rmax) {
      pix[r] = (int)tx.size();
      tx.push_back(pc.x0[r]); tz.push_back(pc.z0[r]);
    }
  }
  int star = -1;
  if (pc.starunres) {
    star = (int)tx.size();
    tx.push_back(0.0); tz.push_back(0.0);
  }
  const int ntr = (int)tx.size();
  const int nfr = m.nfr;
  const size_t ncube = (size_t)nl * nfr * npix;
  PVBuffers& B = md->pv;
  CUDA_TRY(B.I.ensure(sizeof(double) * (ncube ? ncube : 1)));
  CUDA_TRY(B.tauo.ensure(sizeof(double) * (ncube ? ncube : 1)));
  CUDA_TRY(B.pix.ensure(sizeof(int) * npix));
  CUDA_TRY(B.scale.ensure(sizeof(double) * nl));
  float geo_ms = 0.f, walk_ms = 0.f, red_ms = 0.f, up_ms = 0.f;
  unsigned long long cnt[kWalkCounters] = {};
  int kerr = 0;
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  CUDA_TRY(h2d(B.pix.p, pix.data(), sizeof(int) * npix, s));
  LineTables<T> lt;
  if (build_line_tables<T>(m, iline0, nl, lt, err, false)) return set_err(ctx, RL_ERR_ARG, err);
  MaserFlags mf;   // stays clear where no pixel ray crosses the grid
  mf.iline0 = iline0;
  mf.host.assign(nl, 0);
  CUDA_TRY(h2d(B.scale.p, lt.scale.data(), sizeof(double) * nl, s));
  if (ntr > 0) {
    const int kmax = rlg::max_nodes(m.nr, m.nth);
    CUDA_TRY(B.x0.ensure(sizeof(double) * ntr));
    CUDA_TRY(B.z0.ensure(sizeof(double) * ntr));
    CUDA_TRY(B.nodes.ensure<T>(ntr, kmax));
    CUDA_TRY(h2d(B.x0.p, tx.data(), sizeof(double) * ntr, s));
    CUDA_TRY(h2d(B.z0.p, tz.data(), sizeof(double) * ntr, s));
    const size_t nimg = (size_t)nl * ntr * nfr;
    CUDA_TRY(B.img.ensure(sizeof(T) * nimg));
    CUDA_TRY(B.tau.ensure(sizeof(T) * nimg));
    CUDA_TRY(B.tauc.ensure(sizeof(T) * nimg));
    CUDA_TRY(md->dtab.ensure(sizeof(T) * lt.tab.size()));
    CUDA_TRY(md->dnsum.ensure(sizeof(T) * lt.nsum.size()));
    CUDA_TRY(md->dwch.ensure(sizeof(T) * lt.wch.size()));
    CUDA_TRY(md->dstar.ensure(sizeof(T) * lt.star.size()));
    CUDA_TRY(md->dvelo.ensure(sizeof(double) * lt.velo.size()));
    CUDA_TRY(md->dlc.ensure(sizeof(LineConst<T>) * lt.lc.size()));
    CUDA_TRY(md->dcnt.ensure(sizeof(unsigned long long) * kWalkCounters));
    CUDA_TRY(md->dwork.ensure(sizeof(int)));
    CUDA_TRY(md->derr.ensure(sizeof(int)));
    CUDA_TRY(md->dlist.ensure(sizeof(unsigned short) * walk_list_elems(ctx->nsm, nfr)));
    md->tab_line0 = -1;   // the per-line device tables now hold this call's range
    CUDA_TRY(h2d(md->dtab.p, lt.tab.data(), sizeof(T) * lt.tab.size(), s));
    CUDA_TRY(h2d(md->dnsum.p, lt.nsum.data(), sizeof(T) * lt.nsum.size(), s));
    CUDA_TRY(h2d(md->dwch.p, lt.wch.data(), sizeof(T) * lt.wch.size(), s));
    CUDA_TRY(h2d(md->dstar.p, lt.star.data(), sizeof(T) * lt.star.size(), s));
    CUDA_TRY(h2d(md->dvelo.p, lt.velo.data(), sizeof(double) * lt.velo.size(), s));
    CUDA_TRY(h2d(md->dlc.p, lt.lc.data(), sizeof(LineConst<T>) * lt.lc.size(), s));
    CUDA_TRY(cudaMemsetAsync(md->dcnt.p, 0, sizeof(unsigned long long) * kWalkCounters, s));
    CUDA_TRY(cudaMemsetAsync(md->dwork.p, 0, sizeof(int), s));
    CUDA_TRY(cudaMemsetAsync(md->derr.p, 0, sizeof(int), s));
    CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    GeoParams gp = geo_params(md);
    gp.theta0 = pc.theta0;
    gp.x0 = B.x0.as<double>();
    gp.z0 = B.z0.as<double>();
    const NodeBuf<T> nb = B.nodes.view<T>(ntr, kmax);
    CUDA_TRY(launch_geometry<T>(gp, nb, 0, ntr, nullptr, s));
    CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
    WalkParams<T> P;
    P.nb = nb;
    P.nth = m.nth; P.ncell = m.ncell(); P.nlines = nl; P.nfr = nfr;
    int cpl = 4;
    {
      walk_shape(nl, nfr, P.gsize, cpl);
      P.nitems = ((nl + P.gsize - 1) / P.gsize) * ntr;
    }
    P.tab = md->dtab.as<T>(); P.nsum = md->dnsum.as<T>(); P.wch = md->dwch.as<T>(); P.velo = md->dvelo.as<double>();
    P.star = md->dstar.as<T>(); P.lc = md->dlc.as<LineConst<T>>();
    P.aksmax_c = m.aksmax / 2.99792458e5;
    P.kq = (T)(3.33567e-6 * 2.99792458e5);
    P.fstar = (T)0;
    P.img = B.img.as<T>(); P.tau = B.tau.as<T>(); P.tauc = B.tauc.as<T>();
    P.counters = md->dcnt.as<unsigned long long>();
    P.work = md->dwork.as<int>();
    P.err = md->derr.as<int>();
    P.list = md->dlist.as<unsigned short>();
    CUDA_TRY(mf.arm(md->dmaser, lt.mase, iline0, s));
    P.maser = mf.dev;
    CUDA_TRY(launch_walk_pv<T>(P, cpl, ctx->nsm, s));
    CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
  } else {
    CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
    CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
    CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
  }
  CubeParams cp;
  cp.nl = nl; cp.nfr = nfr; cp.nx = pc.nx; cp.ny = pc.ny; cp.ntr = ntr;
  cp.pix = B.pix.as<int>(); cp.star = star; cp.srat = pc.srat; cp.scale = B.scale.as<double>();
  {
    const long long blocks = std::min<long long>(((long long)ncube + 255) / 256, (long long)ctx->nsm * 16);
    k_posvel_cube<T><<<(unsigned)std::max<long long>(blocks, 1), 256, 0, s>>>(cp, B.img.as<T>(), B.tau.as<T>(),
                                                                              B.I.as<double>(), B.tauo.as<double>());
    CUDA_TRY(cudaGetLastError());
  }
  CUDA_TRY(cudaEventRecord(ctx->ev[4], s));
  if (ntr > 0) {
    CUDA_TRY(d2h(cnt, md->dcnt.p, sizeof(cnt), s));
    CUDA_TRY(d2h(&kerr, md->derr.p, sizeof(int), s));
    CUDA_TRY(mf.fetch(s));
  }
  CUDA_TRY(cudaStreamSynchronize(s));
  mf.record(md->masing, m.lfreq.size());
  if (kerr != 0) return set_err(ctx, RL_ERR_GEOMETRY, "position-velocity walk: error code " + std::to_string(kerr));
  if (I_out) {
    g_d2h += sizeof(double) * ncube;
    CUDA_TRY(cudaMemcpy(I_out, B.I.p, sizeof(double) * ncube, cudaMemcpyDeviceToHost));
  }
  if (tau_out) {
    g_d2h += sizeof(double) * ncube;
    CUDA_TRY(cudaMemcpy(tau_out, B.tauo.p, sizeof(double) * ncube, cudaMemcpyDeviceToHost));
  }
  cudaEventElapsedTime(&up_ms, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&geo_ms, ctx->ev[1], ctx->ev[2]);
  cudaEventElapsedTime(&walk_ms, ctx->ev[2], ctx->ev[3]);
  cudaEventElapsedTime(&red_ms, ctx->ev[3], ctx->ev[4]);
  if (st) {
    st->upload_ms += up_ms; st->geometry_ms += geo_ms; st->walk_ms += walk_ms; st->reduce_ms += red_ms;
    st->steps += cnt[0]; st->integrated += cnt[1]; st->node_visits += cnt[2];
    st->overshoots += cnt[9];
    st->ray_channels += (unsigned long long)ntr * nfr * nl;
    st->nrays = ntr; st->nfr = nfr; st->kmax = rlg::max_nodes(m.nr, m.nth); st->nlines += nl;
  }
  return 0;
}

int dispatch_posvel(rl_model* md, int iline0, int nl, double* I, double* tau, rl_stats* st) {
  g_h2d = 0; g_d2h = 0;
  const int rc = md->precision == RL_FP64 ? run_posvel<double>(md, iline0, nl, I, tau, st)
                                          : run_posvel<float>(md, iline0, nl, I, tau, st);
  if (st) { st->h2d_bytes += g_h2d; st->d2h_bytes += g_d2h; }
  return rc;
}

}  // namespace rl

using namespace rl;

extern "C" {

int rl_set_posvel(rl_model* md, const rl_posvel_spec* spec) {
  if (!md || !spec) return set_err(nullptr, RL_ERR_ARG, "rl_set_posvel: null argument");
  PVSpec p;
  p.nx = spec->nx; p.ny = spec->ny; p.szimx = spec->szimx; p.szimy = spec->szimy;
  p.phioff = spec->phioff; p.xoff = spec->xoff; p.yoff = spec->yoff; p.addstar = spec->addstar;
  PVCamera pc;
  std::string err;
  if (setup_pv_camera(md->m, p, md->incl_rad, pc, err)) return set_err(md->ctx, RL_ERR_ARG, "rl_set_posvel: " + err);
  md->pvspec = p;
  return 0;
}

int rl_get_posvel(rl_model* md, rl_posvel_spec* spec) {
  if (!md || !spec) return set_err(nullptr, RL_ERR_ARG, "rl_get_posvel: null argument");
  const PVSpec& p = md->pvspec;
  spec->nx = p.nx; spec->ny = p.ny; spec->szimx = p.szimx; spec->szimy = p.szimy;
  spec->phioff = p.phioff; spec->xoff = p.xoff; spec->yoff = p.yoff; spec->addstar = p.addstar;
  return 0;
}

int rl_posvel(rl_model* md, int iline0, int nlines, double* I_out, double* tau_out, rl_stats* st) {
  if (!md) return set_err(nullptr, RL_ERR_ARG, "rl_posvel: null model");
  rl_ctx* ctx = md->ctx;
  if (!ctx) return set_err(nullptr, RL_ERR_STATE, "model was loaded without a device context");
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  return dispatch_posvel(md, iline0, nlines, I_out, tau_out, st);
}

}  // extern "C"
