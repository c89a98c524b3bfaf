// rl_kernels.cu -- sm_103a kernels of the line raytrace.
//
//   k_geometry   FP64, one thread per ray: crossing list + channel-independent node
//                fields (interpolation corners and weights, line width, projected
//                velocity) written once per camera and shared by every line.
//   k_walk<T,C>  one warp per (line, ray) work item pulled from a device queue; the
//                velocity channels of the ray are spread over the 32 lanes (C per lane).
//                Per 32-node chunk the lanes cooperatively interpolate the per-line cell
//                tables into shared memory; then every lane runs the formal solution of
//                its channels over the chunk. FP32: exponentials on the MUFU pipe
//                (ex2.approx), reciprocals with rcp.approx, series for small optical
//                depth. FP64: the reference arithmetic, used as a second oracle.
//   k_ring_sum / k_spectrum  deterministic FP64 image -> F_nu reduction.
#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include "rl_device.h"
#include "rl_geometry.cuh"
#include "rl_walk_common.cuh"
#include "rl_walk.cuh"
#include "rl_walk_launch.cuh"

namespace rl {

// the walk instances that also keep each channel's optical depth (rl_walk_tau.cu)
template <typename T>
cudaError_t launch_walk_tau(const WalkParams<T>& P, int cpl, int nsm, cudaStream_t s);
template <typename T>
cudaError_t launch_walk_jobs_tau(const WalkJobs<T>& B, int cpl, int nsm, cudaStream_t s);
// the walk instances that count the steps failing the overshoot test (rl_walk_chk.cu)
template <typename T>
cudaError_t launch_walk_chk(const WalkParams<T>& P, int cpl, int nsm, cudaStream_t s);

// ------------------------------------------------------------------------------------
// geometry
// ------------------------------------------------------------------------------------
__device__ __forceinline__ int ridx_dev(int it, int ny) {
  int v = it;
  if (v < 1) v = 1 - v;
  if (v > ny) v = 2 * ny + 1 - v;
  if (v > ny / 2) v = ny + 1 - v;
  return v;
}

template <typename T>
struct NodeEmitter {
  // The FP32 build stores every node value in FP32, so it forms the direction, the
  // projected velocity and the interpolation weights in float-float and the width in FP32
  // from the FP64 positions and cell differences; the FP64 build does all of it in FP64.
  static constexpr bool kFp32Direction = sizeof(T) == 4;
  const GeoParams* p;
  const rlg::Grid* g;
  NodeBuf<T>* nb;
  TrajDebug* dbg;
  size_t row;
  int k, status;
  int ir_prev, icr_prev;
  double s_prev, dvmu_prev;
  rlg::ff dvmu_prev_ff;

  __device__ bool operator()(const rlg::Node& n) {
    if (k >= nb->kmax) return false;
    if constexpr (sizeof(T) == 4) return emit_fp32(n);
    const int nr = p->nr, nth = p->nth, ny = p->ny;
    const double R0 = rlg::Rg(*g, n.ir), R1 = rlg::Rg(*g, n.ir + 1);
    const double T0 = rlg::Tg(*g, n.it), T1 = rlg::Tg(*g, n.it + 1);
    const double dr = (n.r - R0) / (R1 - R0);
    const double dt = (n.th - T0) / (T1 - T0);
    if (!(dr >= 0.0 && dr <= 1.0) || !(dt >= 0.0 && dt <= 1.0)) { status = rlg::kGeoRange; return false; }
    if (k == 0 && n.ir == 0) { status = rlg::kGeoStarStart; return false; }
    if (n.mu > 1.0) { status = rlg::kGeoMu; return false; }
    int r1;
    if (dr > 0.0) { r1 = n.ir + 1; if (r1 > nr) r1 = nr; } else { r1 = n.ir - 1; if (r1 < 1) r1 = 1; }
    const int t0 = ridx_dev(n.it, ny);
    const int t1 = ridx_dev(dt > 0.0 ? n.it + 1 : n.it - 1, ny);
    const int c00 = (n.ir - 1) * nth + (t0 - 1);
    const int dto = t1 - t0, dro = r1 - n.ir;
    const int c01 = c00 + dto, c10 = c00 + dro * nth, c11 = c10 + dto;
    double v[3];
    for (int i = 0; i < 3; i++)
      v[i] = (1.0 - dr) * ((1.0 - dt) * p->vel[3 * c00 + i] + dt * p->vel[3 * c01 + i]) +
             dr * ((1.0 - dt) * p->vel[3 * c10 + i] + dt * p->vel[3 * c11 + i]);
    const double lwv = (1.0 - dr) * ((1.0 - dt) * p->lw[c00] + dt * p->lw[c01]) +
                       dr * ((1.0 - dt) * p->lw[c10] + dt * p->lw[c11]);
    const double dvmu = 3.335668e-11 * (n.mu * v[0] + n.sinmu * (v[1] * n.sinphi + v[2] * n.cosphi));
    const double kv = 1.0 / 3.33567e-6;
    unsigned flags = 0;
    double ds = 0.0;
    if (k > 0) {
      ds = n.s - s_prev;
      const bool hole = (n.ir == 1 && ir_prev == 1 && n.icr == 1 && icr_prev == 1) ||
                        (n.ir == 1 && ir_prev == 0 && n.icr == 1 && icr_prev == 1);
      if (hole) { flags |= kFlagHole; ds = 0.0; }
    }
    if (n.ir <= 1) flags |= kFlagIr1;
    const size_t o = row + k;
    nb->ds[o] = (T)ds;
    nb->dvf[o] = (float)dvmu;
    nb->vl[o] = (T)(dvmu * kv);
    nb->dvseg[o] = (T)(k > 0 ? (dvmu - dvmu_prev) * kv : 0.0);
    nb->lw[o] = (T)lwv;
    nb->wr[o] = (T)dr;
    nb->wt[o] = (T)dt;
    nb->c00[o] = c00;
    nb->misc[o] = (unsigned)(dto + 32768) | ((unsigned)(dro + 1) << 16) | ((unsigned)n.icr << kIcrShift) | flags;
    if (dbg && k < dbg->cap) {
      dbg->s[k] = n.s; dbg->r[k] = n.r; dbg->th[k] = n.th; dbg->mu[k] = n.mu; dbg->dvmu[k] = dvmu;
      dbg->icr[k] = n.icr; dbg->ir[k] = n.ir; dbg->it[k] = n.it;
    }
    s_prev = n.s; dvmu_prev = dvmu; ir_prev = n.ir; icr_prev = n.icr;
    k++;
    return true;
  }

  __device__ bool emit_fp32(const rlg::Node& n) {
    const int nr = p->nr, nth = p->nth, ny = p->ny;
    const double R0 = rlg::Rg(*g, n.ir), R1 = rlg::Rg(*g, n.ir + 1);
    const double T0 = rlg::Tg(*g, n.it), T1 = rlg::Tg(*g, n.it + 1);
    // interpolation weights in float-float from the FP64 differences
    using rlg::ff;
    const ff drf = rlg::ff_div(rlg::ff_of(n.r - R0), rlg::ff_of(R1 - R0));
    const ff dtf = rlg::ff_div(rlg::ff_of(n.th - T0), rlg::ff_of(T1 - T0));
    const float dr = drf.hi, dt = dtf.hi;
    if (!(dr >= 0.0f && dr <= 1.0f) || !(dt >= 0.0f && dt <= 1.0f)) { status = rlg::kGeoRange; return false; }
    if (k == 0 && n.ir == 0) { status = rlg::kGeoStarStart; return false; }
    int r1;
    if (dr > 0.0f) { r1 = n.ir + 1; if (r1 > nr) r1 = nr; } else { r1 = n.ir - 1; if (r1 < 1) r1 = 1; }
    const int t0 = ridx_dev(n.it, ny);
    const int t1 = ridx_dev(dt > 0.0f ? n.it + 1 : n.it - 1, ny);
    const int c00 = (n.ir - 1) * nth + (t0 - 1);
    const int dto = t1 - t0, dro = r1 - n.ir;
    const int c01 = c00 + dto, c10 = c00 + dro * nth, c11 = c10 + dto;
    const float ar = RL_SUB(1.0f, dr), at = RL_SUB(1.0f, dt);
    // bilinear form with every rounding fixed (RL_FMA/RL_MUL), identical in every kernel
    auto bil = [&](float f00, float f01, float f10, float f11) {
      return RL_FMA(dr, RL_FMA(dt, f11, RL_MUL(at, f10)), RL_MUL(ar, RL_FMA(dt, f01, RL_MUL(at, f00))));
    };
    const float lwv = bil(p->lwf[c00], p->lwf[c01], p->lwf[c10], p->lwf[c11]);
    // the velocity and its projection omega.v/c in float-float, the FP64 formulas in the
    // same order: the window test, the segment velocity differences and the Doppler
    // offsets follow the FP64 values to FP32 rounding
    const ff arf = rlg::ff_sub(rlg::ff_c(1.0f), drf), atf = rlg::ff_sub(rlg::ff_c(1.0f), dtf);
    ff v[3];
    for (int i = 0; i < 3; i++) {
      const ff f00{p->velf[3 * c00 + i], p->vell[3 * c00 + i]}, f01{p->velf[3 * c01 + i], p->vell[3 * c01 + i]};
      const ff f10{p->velf[3 * c10 + i], p->vell[3 * c10 + i]}, f11{p->velf[3 * c11 + i], p->vell[3 * c11 + i]};
      v[i] = rlg::ff_add(rlg::ff_mul(arf, rlg::ff_add(rlg::ff_mul(atf, f00), rlg::ff_mul(dtf, f01))),
                         rlg::ff_mul(drf, rlg::ff_add(rlg::ff_mul(atf, f10), rlg::ff_mul(dtf, f11))));
    }
    const ff mu{n.mu_f, n.mu_l}, sinmu{n.sinmu_f, n.sinmu_l};
    const ff sinphi{n.sinphi_f, n.sinphi_l}, cosphi{n.cosphi_f, n.cosphi_l};
    const ff tang = rlg::ff_add(rlg::ff_mul(v[1], sinphi), rlg::ff_mul(v[2], cosphi));
    const ff dvmu = rlg::ff_mul(rlg::ff_of(3.335668e-11), rlg::ff_add(rlg::ff_mul(mu, v[0]), rlg::ff_mul(sinmu, tang)));
    const ff kv = rlg::ff_of(1.0 / 3.33567e-6);
    unsigned flags = 0;
    double ds = 0.0;
    if (k > 0) {
      ds = n.s - s_prev;
      const bool hole = (n.ir == 1 && ir_prev == 1 && n.icr == 1 && icr_prev == 1) ||
                        (n.ir == 1 && ir_prev == 0 && n.icr == 1 && icr_prev == 1);
      if (hole) { flags |= kFlagHole; ds = 0.0; }
    }
    if (n.ir <= 1) flags |= kFlagIr1;
    const size_t o = row + k;
    nb->ds[o] = (T)ds;
    nb->dvf[o] = dvmu.hi;
    nb->vl[o] = (T)rlg::ff_mul(dvmu, kv).hi;
    nb->dvseg[o] = (T)(k > 0 ? rlg::ff_mul(rlg::ff_sub(dvmu, dvmu_prev_ff), kv).hi : 0.0f);
    nb->lw[o] = (T)lwv;
    nb->wr[o] = (T)dr;
    nb->wt[o] = (T)dt;
    nb->c00[o] = c00;
    nb->misc[o] = (unsigned)(dto + 32768) | ((unsigned)(dro + 1) << 16) | ((unsigned)n.icr << kIcrShift) | flags;
    s_prev = n.s; dvmu_prev_ff = dvmu; ir_prev = n.ir; icr_prev = n.icr;
    k++;
    return true;
  }
};

template <typename T>
__device__ __forceinline__ void geometry_ray(const GeoParams& p, NodeBuf<T>& nb, int ray, TrajDebug* dbg) {
  rlg::Grid g;
  g.R = p.R; g.TH = p.TH; g.tan2 = p.tan2; g.nr = p.nr; g.nth = p.nth; g.ny = p.ny; g.rstar = p.rstar;
  NodeEmitter<T> em;
  em.p = &p; em.g = &g; em.nb = &nb; em.dbg = dbg; em.row = (size_t)ray * nb.kmax;
  em.k = 0; em.status = 0; em.ir_prev = -1; em.icr_prev = -1; em.s_prev = 0.0; em.dvmu_prev = 0.0;
  em.dvmu_prev_ff = rlg::ff_c(0.0f);
  int st = rlg::trace(g, p.x0[ray], p.z0[ray], p.theta0, em);
  if (em.status != 0) st = em.status;
  nb.nnodes[ray] = em.k;
  nb.status[ray] = st;
}

template <typename T>
__global__ void __launch_bounds__(128) k_geometry(GeoParams p, NodeBuf<T> nb, int ray0, int nray, TrajDebug* dbg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nray) return;
  geometry_ray<T>(p, nb, ray0 + i, dbg);
}

// Geometry of many cameras in one launch: thread i traces ray i of the concatenated
// ray list; ray_prefix[j] is the first ray of job j.
template <typename T>
__global__ void __launch_bounds__(128) k_geometry_jobs(const GeoJob<T>* __restrict__ jobs, const int* __restrict__ ray_prefix,
                                                       int njobs, int total) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int j = find_job(ray_prefix, njobs, i);
  GeoParams p = jobs[j].geo;
  NodeBuf<T> nb = jobs[j].nb;
  geometry_ray<T>(p, nb, i - ray_prefix[j], nullptr);
}


// ------------------------------------------------------------------------------------
// image -> spectrum (telescope.F:1346-1435), deterministic FP64
// ------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void ring_sum_one(const ReduceParams& p, const T* __restrict__ img, double* __restrict__ ring,
                                             int line, int ir) {
  for (int k = threadIdx.x; k < p.nfr; k += blockDim.x) {
    double d = 0.0;
    const T* base = img + ((size_t)line * p.nrays + 1 + (size_t)(ir - 1) * p.nphi) * p.nfr + k;
    for (int ip = 0; ip < p.nphi; ip++) d = d + (double)base[(size_t)ip * p.nfr];
    ring[((size_t)line * (p.nrr + 1) + ir) * p.nfr + k] = d;
  }
}

template <typename T>
__device__ __forceinline__ void spectrum_one(const ReduceParams& p, const T* __restrict__ img,
                                             const double* __restrict__ ring, double* __restrict__ flux, int line,
                                             int k) {
  const double pi = 3.14159265359;
  double slum = 0.0;
  double surf = pi * (p.ri[1] * p.ri[1]);
  slum = slum + surf * (double)img[((size_t)line * p.nrays) * p.nfr + k];
  for (int ir = 1; ir <= p.nrr; ir++) {
    surf = pi * (p.ri[ir + 1] * p.ri[ir + 1] - p.ri[ir] * p.ri[ir]);
    double d = ring[((size_t)line * (p.nrr + 1) + ir) * p.nfr + k];
    d = d / (1.0 * p.nphi);
    d = d * surf;
    slum = slum + d;
  }
  flux[(size_t)line * p.nfr + k] = p.scale[line] * slum / p.dist2;
}

template <typename T>
__global__ void k_ring_sum(ReduceParams p, const T* __restrict__ img, double* __restrict__ ring) {
  ring_sum_one<T>(p, img, ring, blockIdx.y, blockIdx.x + 1);   // ring 1..nrr of line blockIdx.y
}

template <typename T>
__global__ void k_spectrum(ReduceParams p, const T* __restrict__ img, const double* __restrict__ ring,
                           double* __restrict__ flux) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= p.nfr) return;
  spectrum_one<T>(p, img, ring, flux, blockIdx.y, k);
}

// Reduction of many jobs: block b of k_ring_sum_jobs is (line, ring) pair b of the
// concatenation (ring_prefix[j] = first pair of job j, nlines x nrr pairs per job);
// block b of k_spectrum_jobs is line b (line_prefix[j] = first line of job j).
template <typename T>
__global__ void k_ring_sum_jobs(const RedJob<T>* __restrict__ jobs, const int* __restrict__ ring_prefix, int njobs) {
  const int j = find_job(ring_prefix, njobs, blockIdx.x);
  const RedJob<T>& J = jobs[j];
  const int b = blockIdx.x - ring_prefix[j];
  ring_sum_one<T>(J.p, J.img, J.ring, b / J.p.nrr, b % J.p.nrr + 1);
}

template <typename T>
__global__ void k_spectrum_jobs(const RedJob<T>* __restrict__ jobs, const int* __restrict__ line_prefix, int njobs) {
  const int j = find_job(line_prefix, njobs, blockIdx.x);
  const RedJob<T>& J = jobs[j];
  const int line = blockIdx.x - line_prefix[j];
  for (int k = threadIdx.x; k < J.p.nfr; k += blockDim.x) spectrum_one<T>(J.p, J.img, J.ring, J.flux, line, k);
}

// rows of chosen rays: out[line][i][k] = img[line][rays[i]][k] (ray indices checked on the host)
template <typename T>
__global__ void k_gather_rows(const T* __restrict__ img, int nrays, int nfr, int nl, const int* __restrict__ rays,
                              int nsel, T* __restrict__ out) {
  const long long n = (long long)nl * nsel * nfr;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % nfr);
    const long long r = i / nfr;
    const int sel = (int)(r % nsel), line = (int)(r / nsel);
    out[i] = img[((size_t)line * nrays + rays[sel]) * nfr + k];
  }
}

// ------------------------------------------------------------------------------------
// pipe-throughput calibration (the denominators of the issue roofline)
// ------------------------------------------------------------------------------------
__global__ void k_peak_ffma(float* out, int iters, float x, float y) {
  float a[8];
#pragma unroll
  for (int i = 0; i < 8; i++) a[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
#pragma unroll
      for (int i = 0; i < 8; i++) a[i] = fmaf(a[i], x, y);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; i++) s += a[i];
  if (s == 1234.5f) out[blockIdx.x] = s;
}

__global__ void k_peak_ex2(float* out, int iters, float c) {
  float a[8];
#pragma unroll
  for (int i = 0; i < 8; i++) a[i] = threadIdx.x * 1e-6f + i * 1e-3f;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
#pragma unroll
      for (int i = 0; i < 8; i++) asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(a[i]) : "f"(a[i] * c));
    }
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; i++) s += a[i];
  if (s == 1234.5f) out[blockIdx.x] = s;
}

cudaError_t measure_peaks(int nsm, cudaStream_t st, double* ffma_per_s, double* ex2_per_s) {
  float* out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(float) * nsm * 64);
  if (e != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = nsm * 8, threads = 256;
  const int it_f = 8192, it_m = 1024;   // about 8 ms and 4 ms per launch at full clock
  *ffma_per_s = 0.0;
  *ex2_per_s = 0.0;
  for (int rep = 0; rep < 6; rep++) {   // the first launches ramp the clocks; keep the best rate
    float ms = 0.f;
    cudaEventRecord(a, st);
    k_peak_ffma<<<blocks, threads, 0, st>>>(out, it_f, 0.9999f, 1e-4f);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    if (ms > 0.f) *ffma_per_s = fmax(*ffma_per_s, (double)blocks * threads * it_f * 16 * 8 / (ms * 1e-3));
    cudaEventRecord(a, st);
    k_peak_ex2<<<blocks, threads, 0, st>>>(out, it_m, 0.5f);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    if (ms > 0.f) *ex2_per_s = fmax(*ex2_per_s, (double)blocks * threads * it_m * 16 * 8 / (ms * 1e-3));
  }
  e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  return e;
}

// ------------------------------------------------------------------------------------
// launchers (called from the host orchestration)
// ------------------------------------------------------------------------------------
template <typename T>
cudaError_t launch_geometry(const GeoParams& p, const NodeBuf<T>& nb, int ray0, int nray, TrajDebug* dbg,
                            cudaStream_t s) {
  if (nray <= 0) return cudaSuccess;
  const int bs = 128;
  k_geometry<T><<<(nray + bs - 1) / bs, bs, 0, s>>>(p, nb, ray0, nray, dbg);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_walk(const WalkParams<T>& P, int cpl, int nsm, cudaStream_t s, bool check) {
  if (P.tau) return launch_walk_tau<T>(P, cpl, nsm, s);   // rl_walk_tau.cu
  if (check) return launch_walk_chk<T>(P, cpl, nsm, s);   // rl_walk_chk.cu
  return launch_walk_t<T, false>(P, cpl, nsm, s);
}

template <typename T>
cudaError_t launch_reduce(const ReduceParams& p, const T* img, double* ring, double* flux, cudaStream_t s) {
  dim3 g1(p.nrr, p.nlines);
  k_ring_sum<T><<<g1, 256, 0, s>>>(p, img, ring);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  dim3 g2((p.nfr + 127) / 128, p.nlines);
  k_spectrum<T><<<g2, 128, 0, s>>>(p, img, ring, flux);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gather_rows(const T* img, int nrays, int nfr, int nl, const int* rays, int nsel, T* out,
                               cudaStream_t s) {
  const long long n = (long long)nl * nsel * nfr;
  if (n <= 0) return cudaSuccess;
  const long long blocks = std::min<long long>((n + 255) / 256, 65536);
  k_gather_rows<T><<<(unsigned)blocks, 256, 0, s>>>(img, nrays, nfr, nl, rays, nsel, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_jobs(const JobLaunch<T>& L, cudaStream_t s) {
  if (L.nrays_total > 0) {
    k_geometry_jobs<T><<<(L.nrays_total + 127) / 128, 128, 0, s>>>(L.geo, L.ray_prefix, L.njobs, L.nrays_total);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = cudaSuccess;
  if (L.walk_jobs) {
    e = cudaMemsetAsync(L.walk.work, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    e = L.walk.tau ? launch_walk_jobs_tau<T>(L.walk, L.cpl, L.nsm, s) : launch_walk_jobs_t<T, false>(L.walk, L.cpl, L.nsm, s);
  }
  if (e != cudaSuccess || !L.reduce) return e;
  k_ring_sum_jobs<T><<<L.nring_blocks, 256, 0, s>>>(L.red, L.ring_prefix, L.njobs);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_spectrum_jobs<T><<<L.nline_blocks, 128, 0, s>>>(L.red, L.line_prefix, L.njobs);
  return cudaGetLastError();
}

template cudaError_t launch_geometry<float>(const GeoParams&, const NodeBuf<float>&, int, int, TrajDebug*, cudaStream_t);
template cudaError_t launch_geometry<double>(const GeoParams&, const NodeBuf<double>&, int, int, TrajDebug*, cudaStream_t);
template cudaError_t launch_walk<float>(const WalkParams<float>&, int, int, cudaStream_t, bool);
template cudaError_t launch_walk<double>(const WalkParams<double>&, int, int, cudaStream_t, bool);
template cudaError_t launch_reduce<float>(const ReduceParams&, const float*, double*, double*, cudaStream_t);
template cudaError_t launch_reduce<double>(const ReduceParams&, const double*, double*, double*, cudaStream_t);
template cudaError_t launch_gather_rows<float>(const float*, int, int, int, const int*, int, float*, cudaStream_t);
template cudaError_t launch_gather_rows<double>(const double*, int, int, int, const int*, int, double*, cudaStream_t);
template cudaError_t launch_jobs<float>(const JobLaunch<float>&, cudaStream_t);
template cudaError_t launch_jobs<double>(const JobLaunch<double>&, cudaStream_t);

}  // namespace rl
