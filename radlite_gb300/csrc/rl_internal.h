// rl_internal.h -- library-internal state behind the opaque C handles, shared by the
// single-model entry points (rl_capi.cpp) and the multi-job batch (rl_batch.cpp).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/rlgpu.h"
#include "rl_device.h"
#include "rl_host.h"

namespace rl {
template <typename T>
cudaError_t launch_geometry(const GeoParams& p, const NodeBuf<T>& nb, int ray0, int nray, TrajDebug* dbg,
                            cudaStream_t s);
// check: count the steps that fail the reference's overshoot test in counters[9]
// (the plain walk with P.tau unset only)
template <typename T>
cudaError_t launch_walk(const WalkParams<T>& P, int cpl, int nsm, cudaStream_t s, bool check = false);
template <typename T>
cudaError_t launch_reduce(const ReduceParams& p, const T* img, double* ring, double* flux, cudaStream_t s);
template <typename T>
cudaError_t launch_jobs(const JobLaunch<T>& L, cudaStream_t s);
template <typename T>
cudaError_t launch_gather_rows(const T* img, int nrays, int nfr, int nl, const int* rays, int nsel, T* out,
                               cudaStream_t s);
cudaError_t measure_peaks(int nsm, cudaStream_t st, double* ffma_per_s, double* ex2_per_s);

constexpr int kWalkGroup = 12;   // lines of one walk tile at most (k_walk's kGroup)

// Work-item shape of a line range: balanced items of at most kItemLines lines (their
// channels are packed into tiles of 32*cpl pairs), and the channel slots per lane: 4 (one
// pass of four slots per tile) unless an item holds fewer pairs.
inline void walk_shape(int nl, int nfr, int& gsize, int& cpl) {
  const int ng = (nl + kItemLines - 1) / kItemLines;
  gsize = (nl + ng - 1) / ng;
  const long long pairs = (long long)gsize * nfr;
  cpl = pairs <= 32 ? 1 : pairs <= 64 ? 2 : 4;
}

// Owned device allocation that only grows.
struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      if (p) cudaFree(p);
      p = o.p; n = o.n; o.p = nullptr; o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { if (p) cudaFree(p); }
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n && p) return cudaSuccess;
    if (p) { cudaFree(p); p = nullptr; n = 0; }
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e == cudaSuccess) n = bytes;
    return e;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

// Per-line device tables of a line range, built on the host in FP64 (prepare_line).
template <typename T>
struct LineTables {
  int nl = 0, ncell = 0, nfr = 0;
  std::vector<T> tab;        // [ncell][nl][4]: j-factor*cphi, alpha-factor*cphi, dust j, dust alpha
  std::vector<T> nsum;       // [ncell][nl]
  std::vector<T> wch;        // [nl][nfr]
  std::vector<T> star;       // [nl][nfr] stellar intensity, then (outer boundary 3) [nl][nfr]
                             // the interstellar start intensity (isrf_of)
  std::vector<double> velo;  // [nl][nfr]
  std::vector<LineConst<T>> lc;
  std::vector<double> scale; // [nl]
  std::vector<char> mase;    // [nl] the line has a population inversion somewhere
  bool has_isrf = false;     // star holds the outer-boundary-3 start table after the stellar one
};
template <typename T>
int build_line_tables(const Model& m, int iline0, int nl, LineTables<T>& out, std::string& err,
                      bool with_isrf = true);

// The per-channel start intensities inside a device copy of LineTables::star (outer
// boundary 3), or null: the walk then starts every channel at LineConst::istart.
// Masing flags of a launch over lines iline0.. (mase: which of them have an inversion):
// cleared device flags when any has one, else null (the walk then skips the check).
// record() stores the flags read back after the launch in rl_model::masing.
struct MaserFlags {
  int* dev = nullptr;
  std::vector<int> host;
  int iline0 = 1;
  cudaError_t arm(rl::DevBuf& buf, const std::vector<char>& mase, int line0, cudaStream_t s) {
    iline0 = line0;
    host.assign(mase.size(), 0);
    bool any = false;
    for (char c : mase) any = any || c;
    if (!any) { dev = nullptr; return cudaSuccess; }
    cudaError_t e = buf.ensure(sizeof(int) * mase.size());
    if (e != cudaSuccess) return e;
    dev = static_cast<int*>(buf.p);
    return cudaMemsetAsync(dev, 0, sizeof(int) * mase.size(), s);
  }
  cudaError_t fetch(cudaStream_t s) {
    return dev ? cudaMemcpyAsync(host.data(), dev, sizeof(int) * host.size(), cudaMemcpyDeviceToHost, s) : cudaSuccess;
  }
  void record(std::vector<char>& masing, size_t nlines_mol) const {   // after the stream synchronised
    if (masing.size() != nlines_mol) masing.assign(nlines_mol, 0);
    for (size_t l = 0; l < host.size(); l++) masing[(size_t)iline0 - 1 + l] = host[l] != 0;
  }
};

template <typename T>
inline const T* isrf_of(bool has_isrf, const T* dstar, int nl, int nfr) {
  return has_isrf ? dstar + (size_t)nl * nfr : nullptr;
}

// Node records of a ray set (NodeBuf's arrays), grown on demand.
struct NodeStore {
  DevBuf nn, st, ds, dvf, vl, dvs, lw, wr, wt, c00, misc;
  template <typename T>
  cudaError_t ensure(size_t nrays, int kmax) {
    const size_t n = nrays * (size_t)kmax;
    cudaError_t e;
    if ((e = nn.ensure(sizeof(int) * nrays)) != cudaSuccess) return e;
    if ((e = st.ensure(sizeof(int) * nrays)) != cudaSuccess) return e;
    if ((e = ds.ensure(sizeof(T) * n)) != cudaSuccess) return e;
    if ((e = dvf.ensure(sizeof(float) * n)) != cudaSuccess) return e;
    if ((e = vl.ensure(sizeof(T) * n)) != cudaSuccess) return e;
    if ((e = dvs.ensure(sizeof(T) * n)) != cudaSuccess) return e;
    if ((e = lw.ensure(sizeof(T) * n)) != cudaSuccess) return e;
    if ((e = wr.ensure(sizeof(T) * n)) != cudaSuccess) return e;
    if ((e = wt.ensure(sizeof(T) * n)) != cudaSuccess) return e;
    if ((e = c00.ensure(sizeof(int) * n)) != cudaSuccess) return e;
    return misc.ensure(sizeof(unsigned) * n);
  }
  template <typename T>
  NodeBuf<T> view(int nrays, int kmax) const {
    NodeBuf<T> nb;
    nb.nrays = nrays; nb.kmax = kmax;
    nb.nnodes = nn.as<int>(); nb.status = st.as<int>();
    nb.ds = ds.as<T>(); nb.dvf = dvf.as<float>(); nb.vl = vl.as<T>(); nb.dvseg = dvs.as<T>();
    nb.lw = lw.as<T>(); nb.wr = wr.as<T>(); nb.wt = wt.as<T>(); nb.c00 = c00.as<int>(); nb.misc = misc.as<unsigned>();
    return nb;
  }
};

// Device buffers of the position-velocity cube (rl_posvel.cu).
struct PVBuffers {
  DevBuf x0, z0, pix, scale, img, tau, tauc, I, tauo;
  NodeStore nodes;
};
}  // namespace rl

struct rl_ctx {
  int device = 0, nsm = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[6] = {};
  std::string err;
};

struct rl_model {
  rl_ctx* ctx = nullptr;
  rl::Model m;
  int precision = RL_FP32;
  int checks = 0;   // RL_CHECK_* diagnostics of the line renders
  // camera request
  double incl_rad = 0.0;
  int nphi = 0, dbdr = 1, nrext = 0;
  // device copies of the grid and cell fields (uploaded once)
  bool grid_ready = false;
  rl::DevBuf dR, dTH, dtan2, dvel, dlw, dvelf, dvell, dlwf;
  // camera geometry cache
  bool geo_ready = false;
  int geo_prec = -1;
  rl::Camera cam;
  rl::DevBuf dx0, dz0, dri;
  rl::DevBuf nb_nn, nb_st, nb_ds, nb_dvf, nb_vl, nb_dvs, nb_lw, nb_wr, nb_wt, nb_c00, nb_misc;
  int kmax = 0;
  // per-line tables of the last line range (reused while the range and precision match)
  int tab_line0 = -1, tab_nl = 0, tab_prec = -1;
  std::vector<double> tab_scale;
  std::vector<char> tab_mase;
  bool tab_isrf = false;
  // masing found by the last render of each line of the molecule (spectrum or cube)
  std::vector<char> masing;
  // position-velocity cube: the image request and its buffers
  rl::PVSpec pvspec;
  rl::PVBuffers pv;
  // per-call buffers
  rl::DevBuf dmask;   // circular-image integration mask (on request)
  rl::DevBuf dmaser;  // per-line masing flags (launches with an inverted line)
  rl::DevBuf drows, drowout;   // rl_image_rows: chosen ray indices and their gathered rows
  rl::DevBuf dtab, dnsum, dwch, dvelo, dstar, dlc, dimg, dring, dflux, dscale, dcnt, dwork, derr, dlist;
};

extern thread_local std::string g_last_error;
extern thread_local unsigned long long g_h2d, g_d2h;   // bytes copied by the current call

namespace rl {
// Makes the context's device current at an entry point and drops an error that an
// earlier, unrelated runtime call left behind, so that the launch checks of this call
// (cudaGetLastError) report only this call's own launches.
inline cudaError_t enter_device(int device) {
  const cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) (void)cudaGetLastError();
  return e;
}
void set_last_error(const std::string& msg);
int set_err(rl_ctx* c, int code, const std::string& msg);
cudaError_t h2d(void* dst, const void* src, size_t n, cudaStream_t s);
cudaError_t d2h(void* dst, const void* src, size_t n, cudaStream_t s);
int upload_grid(rl_model* md);
// the position-velocity cube of lines iline0.. into [nl][nfr][ny][nx] (rl_posvel.cu)
int dispatch_posvel(rl_model* md, int iline0, int nl, double* I, double* tau, rl_stats* st);

inline GeoParams geo_params(const rl_model* md) {
  GeoParams p;
  const Model& m = md->m;
  p.nr = m.nr; p.nth = m.nth; p.ny = m.ny; p.rstar = m.rstar; p.theta0 = md->cam.theta0;
  p.R = md->dR.as<double>(); p.TH = md->dTH.as<double>(); p.tan2 = md->dtan2.as<double>();
  p.vel = md->dvel.as<double>(); p.lw = md->dlw.as<double>();
  p.velf = md->dvelf.as<float>(); p.vell = md->dvell.as<float>(); p.lwf = md->dlwf.as<float>();
  p.x0 = md->dx0.as<double>(); p.z0 = md->dz0.as<double>();
  return p;
}

template <typename T>
inline NodeBuf<T> node_view(const rl_model* md) {
  NodeBuf<T> nb;
  nb.nrays = md->cam.nrays;
  nb.kmax = md->kmax;
  nb.nnodes = md->nb_nn.as<int>();
  nb.status = md->nb_st.as<int>();
  nb.ds = md->nb_ds.as<T>();
  nb.dvf = md->nb_dvf.as<float>();
  nb.vl = md->nb_vl.as<T>();
  nb.dvseg = md->nb_dvs.as<T>();
  nb.lw = md->nb_lw.as<T>();
  nb.wr = md->nb_wr.as<T>();
  nb.wt = md->nb_wt.as<T>();
  nb.c00 = md->nb_c00.as<int>();
  nb.misc = md->nb_misc.as<unsigned>();
  return nb;
}
}  // namespace rl

#define CUDA_TRY(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return rl::set_err(ctx, RL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
