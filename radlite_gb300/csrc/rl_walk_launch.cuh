// rl_walk_launch.cuh -- the walk kernels (one model; many jobs from one queue) and their
// launchers, templated on the channel slots per lane C and on TAU: whether the walk also
// keeps each integrated channel's optical depth along the ray (compensated) in
// WalkParams::tau / tauc, which the gradient sweep of the differentiable path reads, and on
// CHK: whether it counts the steps that fail the reference's overshoot test. The plain
// instances live in rl_kernels.cu, the TAU instances in rl_walk_tau.cu, the CHK ones in
// rl_walk_chk.cu.
#pragma once
#include <cuda_runtime.h>
#include "rl_device.h"
#include "rl_walk.cuh"

namespace rl {

template <typename T, int C, bool TAU, bool CHK = false>
__global__ void __launch_bounds__(128, WalkMinBlocks<T>::value) k_walk(WalkParams<T> P) {
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
    walk_item<T, C, false, TAU, CHK>(P, item, *W.S, *W.SS, *W.SW, W.list, lane, steps);
  }
  flush_counters(steps, *W.SW, P.counters, lane);
}

// Walk of many jobs (model, camera, line range) from one device queue: queue entry i
// is item i * stride of the concatenated item list (stride > 1 samples it for tuning);
// item_prefix[j] is the first item of job j. Each warp keeps the parameters of its
// current job in shared memory.
template <typename T, int C, bool TAU>
__global__ void __launch_bounds__(128, WalkMinBlocks<T>::value) k_walk_jobs(WalkJobs<T> B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ WalkParams<T> jp[4];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  WarpSmem<T, C> W(smem_raw, nw, wib, kItemLines * B.max_nfr, B.list);
  unsigned long long steps = 0;   // this lane's formal-solution steps
  zero_counters(*W.SW, lane);
  int cur = -1;
  const int nq = (B.total + B.stride - 1) / B.stride;
  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(B.work, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= nq) break;
    const int item = q * B.stride;
    const int j = find_job(B.item_prefix, B.njobs, item);
    if (j != cur) {
      __syncwarp();
      const int* src = reinterpret_cast<const int*>(B.jobs + j);
      int* dst = reinterpret_cast<int*>(&jp[wib]);
      for (int w = lane; w < (int)(sizeof(WalkParams<T>) / 4); w += 32) dst[w] = __ldg(src + w);
      __syncwarp();
      cur = j;
    }
    walk_item<T, C, false, TAU>(jp[wib], item - __ldg(&B.item_prefix[j]), *W.S, *W.SS, *W.SW, W.list, lane, steps);
  }
  flush_counters(steps, *W.SW, B.counters, lane);
}

template <typename T, int C, bool TAU, bool CHK = false>
cudaError_t launch_walk_c(const WalkParams<T>& P, int nsm, cudaStream_t s) {
  const int warps = 4, threads = warps * 32;
  const int capp = (kItemLines * P.nfr + 7) & ~7;
  const size_t smem = (sizeof(WarpStage<T>) + sizeof(SlotState<T, C>) + sizeof(SubWork<T>)) * warps +
                      (kListInSmem ? sizeof(unsigned short) * (size_t)capp * warps : 0);
  cudaError_t e = cudaFuncSetAttribute(k_walk<T, C, TAU, CHK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<T, C, TAU, CHK>, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (per_sm > kWalkBlocksPerSm) per_sm = kWalkBlocksPerSm;   // the list scratch holds this many
  long long blocks = (long long)nsm * per_sm;
  const long long need = ((long long)P.nitems + warps - 1) / warps;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  k_walk<T, C, TAU, CHK><<<(unsigned)blocks, threads, smem, s>>>(P);
  return cudaGetLastError();
}

template <typename T, int C, bool TAU>
cudaError_t launch_walk_jobs_c(const WalkJobs<T>& B, int nsm, cudaStream_t s) {
  const int warps = 4, threads = warps * 32;
  const int capp = (kItemLines * B.max_nfr + 7) & ~7;
  const size_t smem = (sizeof(WarpStage<T>) + sizeof(SlotState<T, C>) + sizeof(SubWork<T>)) * warps +
                      (kListInSmem ? sizeof(unsigned short) * (size_t)capp * warps : 0);
  cudaError_t e = cudaFuncSetAttribute(k_walk_jobs<T, C, TAU>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_jobs<T, C, TAU>, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (per_sm > kWalkBlocksPerSm) per_sm = kWalkBlocksPerSm;
  long long blocks = (long long)nsm * per_sm;
  const long long nq = ((long long)B.total + B.stride - 1) / B.stride;
  const long long need = (nq + warps - 1) / warps;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  k_walk_jobs<T, C, TAU><<<(unsigned)blocks, threads, smem, s>>>(B);
  return cudaGetLastError();
}

template <typename T, bool TAU, bool CHK = false>
cudaError_t launch_walk_t(const WalkParams<T>& P, int cpl, int nsm, cudaStream_t s) {
  switch (cpl) {
    case 1: return launch_walk_c<T, 1, TAU, CHK>(P, nsm, s);
    case 2: return launch_walk_c<T, 2, TAU, CHK>(P, nsm, s);
    case 4: return launch_walk_c<T, 4, TAU, CHK>(P, nsm, s);
    default: return launch_walk_c<T, 8, TAU, CHK>(P, nsm, s);
  }
}

template <typename T, bool TAU>
cudaError_t launch_walk_jobs_t(const WalkJobs<T>& B, int cpl, int nsm, cudaStream_t s) {
  switch (cpl) {
    case 1: return launch_walk_jobs_c<T, 1, TAU>(B, nsm, s);
    case 2: return launch_walk_jobs_c<T, 2, TAU>(B, nsm, s);
    case 4: return launch_walk_jobs_c<T, 4, TAU>(B, nsm, s);
    default: return launch_walk_jobs_c<T, 8, TAU>(B, nsm, s);
  }
}

}  // namespace rl
