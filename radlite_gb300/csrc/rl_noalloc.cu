// rl_noalloc.cu -- rl_image_to_spectrum_noalloc: the circular image -> F_nu reduction
// for callers that must not allocate device memory.
//
// Who needs it: a host that owns every device buffer itself and cannot let a library
// call cudaMalloc. Examples are an application with its own pool or arena (a stream-
// ordered allocator that a foreign cudaMalloc would fragment or synchronise), and a
// driver that renders images with its own kernels and only wants them turned into
// spectra. The regular path (rl_spectra) keeps its ring sums in a buffer that the model
// grows on demand. This entry point keeps them in a fixed array that is part of the
// library's device image instead. That array is loaded with the module and held by
// every GPU that loads the library until the process exits.
//
// The reduction is the same two kernels as the regular path (k_ring_sum, then
// k_spectrum, both in rl_kernels.cu), so the result is the same sum in the same order.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "../../include/rlgpu.h"
#include "rl_device.h"

namespace rl {
template <typename T>
cudaError_t launch_reduce(const ReduceParams& p, const T* img, double* ring, double* flux, cudaStream_t s);
void set_last_error(const std::string& msg);
}  // namespace rl

namespace {

// Ring-sum scratch: (nrr + 1) * nfr doubles per line, 8 MiB in all. One line never
// needs more than this; several lines are reduced in chunks that each fit.
constexpr size_t kRingScratchDoubles = size_t(1) << 20;
static __device__ __align__(256) double g_ring_scratch[kRingScratchDoubles];

// Device address of the scratch on the current device, looked up on every call with that
// device current. A cached address would outlive a cudaDeviceReset or a change of the
// current context, after which it no longer names memory of this process; the look-up is
// cheap once the module is loaded. The first look-up in a context loads the module, so
// the first call in a context should not happen inside a stream capture.
int scratch_for_current_device(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_ring_scratch);
  if (e != cudaSuccess || !p) {
    rl::set_last_error(std::string("rl_image_to_spectrum_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return RL_ERR_CUDA;
  }
  *out = static_cast<double*>(p);
  return RL_OK;
}

template <typename T>
int reduce_chunks(const T* img, int nlines, int nrays, int nphi, int nrr, int nfr, const double* ri,
                  const double* scale, double dist2, double* flux, double* ring, cudaStream_t s) {
  const size_t per_line = (size_t)(nrr + 1) * nfr;
  int chunk = (int)(kRingScratchDoubles / per_line);
  if (chunk > 65535) chunk = 65535;   // grid y limit of the two kernels
  for (int l0 = 0; l0 < nlines; l0 += chunk) {
    const int nl = nlines - l0 < chunk ? nlines - l0 : chunk;
    rl::ReduceParams p;
    p.nrays = nrays; p.nfr = nfr; p.nphi = nphi; p.nrr = nrr; p.nlines = nl;
    p.ri = ri; p.dist2 = dist2; p.scale = scale + l0;
    // chunks run in stream order, so each one finds the scratch free
    cudaError_t e = rl::launch_reduce<T>(p, img + (size_t)l0 * nrays * nfr, ring, flux + (size_t)l0 * nfr, s);
    if (e != cudaSuccess) {
      rl::set_last_error(std::string("rl_image_to_spectrum_noalloc: launch: ") + cudaGetErrorString(e));
      return RL_ERR_CUDA;
    }
  }
  return RL_OK;
}

}  // namespace

extern "C" int rl_image_to_spectrum_noalloc(void* stream, int precision, const void* image, int nlines, int nrays,
                                            int nphi, int nrr, int nfr, const double* ri, const double* scale,
                                            double distance_pc, double* flux) {
  if (!image || !ri || !scale || !flux) {
    rl::set_last_error("rl_image_to_spectrum_noalloc: null device pointer");
    return RL_ERR_ARG;
  }
  if (precision != RL_FP32 && precision != RL_FP64) {
    rl::set_last_error("rl_image_to_spectrum_noalloc: precision must be RL_FP32 or RL_FP64");
    return RL_ERR_ARG;
  }
  if (nlines < 1 || nphi < 1 || nrr < 1 || nfr < 1 || !(distance_pc > 0.0)) {
    rl::set_last_error("rl_image_to_spectrum_noalloc: nlines, nphi, nrr, nfr and distance must be positive");
    return RL_ERR_ARG;
  }
  if ((long long)nrays != 1 + (long long)nrr * nphi) {
    rl::set_last_error("rl_image_to_spectrum_noalloc: nrays must be 1 + nrr * nphi (central beam + rings)");
    return RL_ERR_ARG;
  }
  const size_t per_line = (size_t)(nrr + 1) * nfr;
  if (per_line > kRingScratchDoubles) {
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "rl_image_to_spectrum_noalloc: (nrr + 1) * nfr = %zu ring sums exceed the fixed scratch of %zu "
                  "doubles; use rl_spectra for this camera",
                  per_line, kRingScratchDoubles);
    rl::set_last_error(msg);
    return RL_ERR_ARG;
  }
  double* ring = nullptr;
  const int rc = scratch_for_current_device(&ring);
  if (rc != RL_OK) return rc;
  const double d = distance_pc * 3.08572e18;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (precision == RL_FP32)
    return reduce_chunks<float>(static_cast<const float*>(image), nlines, nrays, nphi, nrr, nfr, ri, scale, d * d,
                                flux, ring, s);
  return reduce_chunks<double>(static_cast<const double*>(image), nlines, nrays, nphi, nrr, nfr, ri, scale, d * d,
                               flux, ring, s);
}
