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
#include "rl_device.h"
#include "rl_geometry.cuh"

namespace rl {

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
  const GeoParams* p;
  const rlg::Grid* g;
  NodeBuf<T>* nb;
  TrajDebug* dbg;
  size_t row;
  int k, status;
  int ir_prev, icr_prev;
  double s_prev, dvmu_prev;

  __device__ bool operator()(const rlg::Node& n) {
    if (k >= nb->kmax) return false;
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
    const double dvmu = 3.335668e-11 * (n.mu * v[0] + sqrt(1.0 - n.mu * n.mu) * (v[1] * n.sinphi + v[2] * n.cosphi));
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
};

template <typename T>
__global__ void __launch_bounds__(128) k_geometry(GeoParams p, NodeBuf<T> nb, int ray0, int nray, TrajDebug* dbg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nray) return;
  const int ray = ray0 + i;
  rlg::Grid g;
  g.R = p.R; g.TH = p.TH; g.tan2 = p.tan2; g.nr = p.nr; g.nth = p.nth; g.ny = p.ny; g.rstar = p.rstar;
  NodeEmitter<T> em;
  em.p = &p; em.g = &g; em.nb = &nb; em.dbg = dbg; em.row = (size_t)ray * nb.kmax;
  em.k = 0; em.status = 0; em.ir_prev = -1; em.icr_prev = -1; em.s_prev = 0.0; em.dvmu_prev = 0.0;
  int st = rlg::trace(g, p.x0[ray], p.z0[ray], p.theta0, em);
  if (em.status != 0) st = em.status;
  nb.nnodes[ray] = em.k;
  nb.status[ray] = st;
}

// ------------------------------------------------------------------------------------
// walk: arithmetic helpers
// ------------------------------------------------------------------------------------
template <typename T> struct Math;

template <> struct Math<float> {
  // e^{-x} on the MUFU pipe
  static __device__ __forceinline__ float expneg(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(-1.4426950408889634f * x));
    return y;
  }
  static __device__ __forceinline__ float rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
  }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  // Formal-solution coefficients for optical depth d > 1e-6:
  //   x = e^{-d}, e0 = 1 - x, b = (d - e0)/d, a = e0 - b.
  // Below d = 0.7 the FP32 cancellation in d - e0 is avoided with Taylor series.
  static __device__ __forceinline__ void coeffs(float d, float& x, float& a, float& b) {
    if (d < 0.7f) {
      const float e0 = d * (1.f - d * (0.5f - d * (1.f / 6.f - d * (1.f / 24.f - d * (1.f / 120.f - d * (1.f / 720.f - d * (1.f / 5040.f - d * (1.f / 40320.f - d * (1.f / 362880.f)))))))));
      b = d * (0.5f - d * (1.f / 6.f - d * (1.f / 24.f - d * (1.f / 120.f - d * (1.f / 720.f - d * (1.f / 5040.f - d * (1.f / 40320.f - d * (1.f / 362880.f - d * (1.f / 3628800.f)))))))));
      x = 1.f - e0;
      a = e0 - b;
    } else {
      x = expneg(d);
      const float e0 = 1.f - x;
      b = (d - e0) * rcp(d);
      a = e0 - b;
    }
  }
};

template <> struct Math<double> {
  static __device__ __forceinline__ double expneg(double x) { return exp(-x); }
  static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ void coeffs(double d, double& x, double& a, double& b) {
    x = exp(-d);
    const double e0 = 1.0 - x;
    const double e1 = d - e0;
    b = e1 / d;
    a = e0 - b;
  }
};

template <typename T>
__device__ __forceinline__ T profile(T w, T vl, T rlw, T nrm) {
  const T u = (w - vl) * rlw;
  return nrm * Math<T>::expneg(u * u);
}

// One application of the linear-source formal solution (qdr_src_2, transfer.F:1498-1571)
// from point 0 (j0, a0, S0) to point 1 (j1, a1, S1) over half-length hds.
template <typename T>
__device__ __forceinline__ void formal(T& I, T j0, T a0, T S0, T j1, T a1, T S1, T hds) {
  const T dtau = (a0 + a1) * hds;
  const T theo = (j0 + j1) * hds;
  T x, a, b;
  if (dtau > (T)1.0e-6) {
    Math<T>::coeffs(dtau, x, a, b);
  } else {
    a = (T)0.5 * dtau; b = a; x = (T)1 - dtau;
  }
  const T src1 = a0 > (T)0 ? S0 : (a1 > (T)0 ? S1 : (T)0);
  const T src2 = a1 > (T)0 ? S1 : (a0 > (T)0 ? S0 : (T)0);
  T q = dtau > (T)1.0e-9f ? a * src1 + b * src2 : theo;
  q = q < theo ? q : theo;
  I = I * x + q;
}

template <typename T>
struct Pt { T jd, ad, jf, af, vl; };

// point state: emissivity, extinction and own source function at the walk position
template <typename T>
__device__ __forceinline__ void point_state(const Pt<T>& p, T phi, T& j, T& a, T& S) {
  j = p.jd + p.jf * phi;
  a = p.ad + p.af * phi;
  S = a > (T)0 ? j * Math<T>::rcp(a) : (T)0;
}

template <typename T>
struct WarpStage {
  T jf[32], af[32], jd[32], ad[32], vl[32];
  T hds[32], ds[32], rlw[32], nrm[32], dvs[32], q[32], ids[32];
  unsigned flags[32];
};

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T>
__device__ __forceinline__ void load_corners(const T* __restrict__ tab, int c00, unsigned misc, int nth, T wr, T wt,
                                             T& jf, T& af, T& jd, T& ad) {
  const int dto = (int)(misc & 0xFFFFu) - 32768;
  const int dro = (int)((misc >> 16) & 3u) - 1;
  const int c01 = c00 + dto, c10 = c00 + dro * nth, c11 = c10 + dto;
  T v00[4], v01[4] = {0, 0, 0, 0}, v10[4] = {0, 0, 0, 0}, v11[4] = {0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 4; i++) v00[i] = __ldg(&tab[4 * (size_t)c00 + i]);
  if (wt != (T)0) {
#pragma unroll
    for (int i = 0; i < 4; i++) v01[i] = __ldg(&tab[4 * (size_t)c01 + i]);
  }
  if (wr != (T)0) {
#pragma unroll
    for (int i = 0; i < 4; i++) v10[i] = __ldg(&tab[4 * (size_t)c10 + i]);
    if (wt != (T)0) {
#pragma unroll
      for (int i = 0; i < 4; i++) v11[i] = __ldg(&tab[4 * (size_t)c11 + i]);
    }
  }
  T out[4];
#pragma unroll
  for (int i = 0; i < 4; i++)
    out[i] = ((T)1 - wr) * (((T)1 - wt) * v00[i] + wt * v01[i]) + wr * (((T)1 - wt) * v10[i] + wt * v11[i]);
  jf = out[0]; af = out[1]; jd = out[2]; ad = out[3];
}

template <typename T>
__device__ __forceinline__ T load_nsum(const T* __restrict__ ns, int c00, unsigned misc, int nth, T wr, T wt) {
  const int dto = (int)(misc & 0xFFFFu) - 32768;
  const int dro = (int)((misc >> 16) & 3u) - 1;
  const int c01 = c00 + dto, c10 = c00 + dro * nth, c11 = c10 + dto;
  const T v00 = __ldg(&ns[c00]);
  const T v01 = wt != (T)0 ? __ldg(&ns[c01]) : (T)0;
  T v10 = 0, v11 = 0;
  if (wr != (T)0) { v10 = __ldg(&ns[c10]); if (wt != (T)0) v11 = __ldg(&ns[c11]); }
  return ((T)1 - wr) * (((T)1 - wt) * v00 + wt * v01) + wr * (((T)1 - wt) * v10 + wt * v11);
}

// Walk all channels held by this lane over the ray. Returns the formal-solution
// step count of the lane.
template <typename T, int C>
__device__ long long walk_ray(const WalkParams<T>& P, WarpStage<T>& S, int line, int ray, int K,
                              const short* list, int nint, T (&I)[C], int lane) {
  const NodeBuf<T>& nb = P.nb;
  const size_t row = (size_t)ray * nb.kmax;
  const T* tab = P.tab + (size_t)line * P.ncell * 4;
  const LineConst<T> lc = P.lc[line];
  const T* wch = P.wch + (size_t)line * P.nfr;
  const T* star = P.star + (size_t)line * P.nfr;
  const int nslot = (nint + 31) >> 5;
  T w[C], j0[C], a0[C], S0[C];
  int ch[C];
#pragma unroll
  for (int j = 0; j < C; j++) {
    const int idx = j * 32 + lane;
    ch[j] = idx < nint ? list[idx] : -1;
    w[j] = ch[j] >= 0 ? wch[ch[j]] : (T)0;
    I[j] = lc.istart;
    j0[j] = 0; a0[j] = 0; S0[j] = 0;
  }
  long long steps = 0;
  Pt<T> p0 = {0, 0, 0, 0, 0};
  T lw_last = 0;
  bool init = true, star_done = false;
  for (int kb = 0; kb < K; kb += 32) {
    const int k = kb + lane;
    T jf = 0, af = 0, jd = 0, ad = 0, vl = 0, ds = 0, dvs = 0, lwk = 0;
    unsigned misc = 0;
    if (k < K) {
      const size_t o = row + k;
      const T wr = nb.wr[o], wt = nb.wt[o];
      misc = nb.misc[o];
      load_corners(tab, nb.c00[o], misc, P.nth, wr, wt, jf, af, jd, ad);
      vl = nb.vl[o]; ds = nb.ds[o]; dvs = nb.dvseg[o]; lwk = nb.lw[o];
    }
    T lwp = __shfl_up_sync(0xffffffffu, lwk, 1);
    if (lane == 0) lwp = lw_last;
    lw_last = __shfl_sync(0xffffffffu, lwk, 31);
    const T lwav = (T)0.5 * (lwp + lwk);
    const T rlw = lwav > (T)0 ? Math<T>::div((T)1, lwav) : (T)0;
    const T qv = (dvs < (T)0 ? -dvs : dvs) * P.kq * rlw;
    S.jf[lane] = jf; S.af[lane] = af; S.jd[lane] = jd; S.ad[lane] = ad; S.vl[lane] = vl;
    S.hds[lane] = (T)0.5 * ds; S.ds[lane] = ds; S.rlw[lane] = rlw; S.nrm[lane] = lc.cphi * rlw;
    S.dvs[lane] = dvs; S.q[lane] = qv; S.ids[lane] = ds > (T)0 ? Math<T>::div((T)1, ds) : (T)0;
    S.flags[lane] = misc;
    __syncwarp();
    const int nn = min(32, K - kb);
    for (int n = 0; n < nn; n++) {
      const Pt<T> p1 = {S.jd[n], S.ad[n], S.jf[n], S.af[n], S.vl[n]};
      if (kb + n == 0) { p0 = p1; continue; }
      const unsigned fl = S.flags[n];
      if (fl & kFlagHole) init = true;
      if (ray == 0 && (fl & kFlagIr1) && !star_done) {
#pragma unroll
        for (int j = 0; j < C; j++)
          if (j < nslot && ch[j] >= 0) I[j] = ((T)1 - P.fstar) * I[j] + P.fstar * star[ch[j]];
        star_done = true;
        init = true;
      }
      const T rlw = S.rlw[n], nrm = S.nrm[n], hds = S.hds[n], q = S.q[n];
      const bool sub = (T)6 * q > (T)1;
#pragma unroll
      for (int j = 0; j < C; j++) {
        if (j >= nslot) break;
        if (ch[j] < 0) continue;
        if (init) {
          const T ph0 = profile(w[j], p0.vl, rlw, nrm);
          point_state(p0, ph0, j0[j], a0[j], S0[j]);
        }
        bool done = false;
        if (sub) {
          const T dsf = S.ds[n];
          const T s_c = dsf * (w[j] - p0.vl) / S.dvs[n];
          const T dls = dsf / q;
          const T sright = s_c + (T)3 * dls, sleft = s_c - (T)3 * dls;
          if (sright > (T)0 && sleft < dsf) {
            const T lg = (sright - sleft) / (T)30;
            const T ids = S.ids[n];
            T sp = 0;
            for (int i = 0; i <= 31; i++) {
              T s, e;
              Pt<T> pq;
              if (i < 31) {
                s = sleft + (T)i * lg;
                if (!(s > (T)0 && s < dsf)) continue;
                e = s * ids;
                const T ep = (T)1 - e;
                pq.jd = ep * p0.jd + e * p1.jd; pq.ad = ep * p0.ad + e * p1.ad;
                pq.jf = ep * p0.jf + e * p1.jf; pq.af = ep * p0.af + e * p1.af;
                pq.vl = ep * p0.vl + e * p1.vl;
              } else {
                s = dsf; pq = p1;
              }
              const T ph = profile(w[j], pq.vl, rlw, nrm);
              T j1, a1, S1;
              point_state(pq, ph, j1, a1, S1);
              formal(I[j], j0[j], a0[j], S0[j], j1, a1, S1, (T)0.5 * (s - sp));
              j0[j] = j1; a0[j] = a1; S0[j] = S1;
              sp = s;
              steps++;
            }
            done = true;
          }
        }
        if (!done) {
          const T ph = profile(w[j], p1.vl, rlw, nrm);
          T j1, a1, S1;
          point_state(p1, ph, j1, a1, S1);
          formal(I[j], j0[j], a0[j], S0[j], j1, a1, S1, hds);
          j0[j] = j1; a0[j] = a1; S0[j] = S1;
          steps++;
        }
      }
      init = false;
      p0 = p1;
    }
    __syncwarp();
  }
  return steps;
}

template <typename T, int C>
__global__ void __launch_bounds__(256) k_walk(WalkParams<T> P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int nfrp = (P.nfr + 7) & ~7;
  WarpStage<T>* stages = reinterpret_cast<WarpStage<T>*>(smem_raw);
  short* lists = reinterpret_cast<short*>(smem_raw + sizeof(WarpStage<T>) * nw);
  WarpStage<T>& S = stages[wib];
  short* list = lists + (size_t)wib * nfrp;
  __shared__ T cont_val[8];
  unsigned long long st_steps = 0, st_int = 0, st_nodes = 0;
  const NodeBuf<T>& nb = P.nb;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(P.work, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= P.nitems) break;
    const int line = item / nb.nrays, ray = item - line * nb.nrays;
    const int K = nb.nnodes[ray];
    if (nb.status[ray] != 0 || K < 1) {
      if (lane == 0) atomicCAS(P.err, 0, 100 + nb.status[ray]);
      continue;
    }
    const size_t row = (size_t)ray * nb.kmax;
    const double* velo = P.velo + (size_t)line * P.nfr;
    // 1. velocity window of the ray from node projected velocities (telescope.F:4265-4270)
    double lo = -1e300, hi = 1e300;
    if (ray != 0) {
      float mn = 1.0f, mx = -1.0f;
      const T* ns = P.nsum + (size_t)line * P.ncell;
      for (int k = lane; k < K - 1; k += 32) {
        const size_t o = row + k;
        const T n = load_nsum(ns, nb.c00[o], nb.misc[o], P.nth, nb.wr[o], nb.wt[o]);
        if (n > (T)1.0e-3) { const float d = nb.dvf[o]; mn = fminf(mn, d); mx = fmaxf(mx, d); }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, off));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
      }
      lo = (double)mn - 2.0 * P.aksmax_c;
      hi = (double)mx + 2.0 * P.aksmax_c;
    }
    // 2. channels to integrate: channel 1, the in-window channels, and the channel that
    //    supplies the continuum for the rest (telescope.F:541-613)
    int nint = 0, cont_ch = -1;
    bool in0 = true;
    if (ray != 0) in0 = velo[0] <= hi && velo[0] >= lo;
    if (ray != 0 && !in0) cont_ch = 0;
    for (int cb = 0; cb < P.nfr; cb += 32) {
      const int c = cb + lane;
      const bool valid = c < P.nfr;
      const bool in = valid && (ray == 0 || (velo[c] <= hi && velo[c] >= lo));
      if (cont_ch < 0 && ray != 0) {
        const unsigned outm = __ballot_sync(0xffffffffu, valid && !in && c >= 1);
        if (outm) cont_ch = cb + __ffs(outm) - 1;
      }
      const bool take = valid && (c == 0 || in || c == cont_ch);
      const unsigned m = __ballot_sync(0xffffffffu, take);
      if (take) list[nint + __popc(m & lanemask_lt())] = (short)c;
      nint += __popc(m);
    }
    __syncwarp();
    // 3. formal solution of the selected channels, in tiles of 32*C channels
    T* img = P.img + ((size_t)line * nb.nrays + ray) * P.nfr;
    T contv = 0;
    for (int tb = 0; tb < nint; tb += 32 * C) {
      const int nt = min(32 * C, nint - tb);
      T I[C];
      st_steps += walk_ray<T, C>(P, S, line, ray, K, list + tb, nt, I, lane);
#pragma unroll
      for (int j = 0; j < C; j++) {
        const int idx = j * 32 + lane;
        if (idx < nt) {
          const int c = list[tb + idx];
          img[c] = I[j];
          if (c == cont_ch) cont_val[wib] = I[j];
        }
      }
    }
    st_int += nint;
    st_nodes += (unsigned long long)nint * K;
    __syncwarp();
    if (cont_ch >= 0) contv = cont_val[wib];
    // 4. continuum copy for the rest of the channels
    if (cont_ch >= 0) {
      if (contv != (T)0) {
        for (int c = lane; c < P.nfr; c += 32) {
          const bool in = velo[c] <= hi && velo[c] >= lo;
          if (!(c == 0 || in || c == cont_ch)) img[c] = contv;
        }
      } else {
        // a zero continuum is recomputed channel by channel in the reference: integrate
        // every remaining out-of-window channel, then apply its sequential copy rule
        int n2 = 0;
        for (int cb = 0; cb < P.nfr; cb += 32) {
          const int c = cb + lane;
          const bool valid = c < P.nfr;
          const bool take = valid && !(c == 0 || (velo[c] <= hi && velo[c] >= lo) || c == cont_ch);
          const unsigned m = __ballot_sync(0xffffffffu, take);
          if (take) list[n2 + __popc(m & lanemask_lt())] = (short)c;
          n2 += __popc(m);
        }
        __syncwarp();
        for (int tb = 0; tb < n2; tb += 32 * C) {
          const int nt = min(32 * C, n2 - tb);
          T I[C];
          st_steps += walk_ray<T, C>(P, S, line, ray, K, list + tb, nt, I, lane);
#pragma unroll
          for (int j = 0; j < C; j++) {
            const int idx = j * 32 + lane;
            if (idx < nt) img[list[tb + idx]] = I[j];
          }
        }
        st_int += n2;
        st_nodes += (unsigned long long)n2 * K;
        __syncwarp();
        if (lane == 0) {
          T cur = 0;
          bool have = false;
          for (int c = 0; c < P.nfr; c++) {
            const bool in = velo[c] <= hi && velo[c] >= lo;
            if (c != cont_ch && (c == 0 || in)) continue;
            if (have) img[c] = cur;
            else if (img[c] != (T)0) { cur = img[c]; have = true; }
          }
        }
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    st_steps += __shfl_xor_sync(0xffffffffu, st_steps, off);
  }
  if (lane == 0) {
    atomicAdd(&P.counters[0], st_steps);
    atomicAdd(&P.counters[1], st_int);
    atomicAdd(&P.counters[2], st_nodes);
  }
}

// ------------------------------------------------------------------------------------
// image -> spectrum (telescope.F:1346-1435), deterministic FP64
// ------------------------------------------------------------------------------------
template <typename T>
__global__ void k_ring_sum(ReduceParams p, const T* __restrict__ img, double* __restrict__ ring) {
  const int ir = blockIdx.x + 1;        // ring 1..nrr
  const int line = blockIdx.y;
  for (int k = threadIdx.x; k < p.nfr; k += blockDim.x) {
    double d = 0.0;
    const T* base = img + ((size_t)line * p.nrays + 1 + (size_t)(ir - 1) * p.nphi) * p.nfr + k;
    for (int ip = 0; ip < p.nphi; ip++) d = d + (double)base[(size_t)ip * p.nfr];
    ring[((size_t)line * (p.nrr + 1) + ir) * p.nfr + k] = d;
  }
}

template <typename T>
__global__ void k_spectrum(ReduceParams p, const T* __restrict__ img, const double* __restrict__ ring,
                           double* __restrict__ flux) {
  const int line = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= p.nfr) return;
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
  const int it_f = 2048, it_m = 256;
  for (int rep = 0; rep < 2; rep++) {   // first pass warms up the clocks
    cudaEventRecord(a, st);
    k_peak_ffma<<<blocks, threads, 0, st>>>(out, it_f, 0.9999f, 1e-4f);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    *ffma_per_s = (double)blocks * threads * it_f * 16 * 8 / (ms * 1e-3);
    cudaEventRecord(a, st);
    k_peak_ex2<<<blocks, threads, 0, st>>>(out, it_m, 0.5f);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    *ex2_per_s = (double)blocks * threads * it_m * 16 * 8 / (ms * 1e-3);
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

template <typename T, int C>
static cudaError_t launch_walk_c(const WalkParams<T>& P, int nsm, cudaStream_t s) {
  const int warps = 8, threads = warps * 32;
  const int nfrp = (P.nfr + 7) & ~7;
  const size_t smem = sizeof(WarpStage<T>) * warps + sizeof(short) * (size_t)nfrp * warps;
  cudaError_t e = cudaFuncSetAttribute(k_walk<T, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<T, C>, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  long long blocks = (long long)nsm * per_sm;
  const long long need = ((long long)P.nitems + warps - 1) / warps;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  k_walk<T, C><<<(unsigned)blocks, threads, smem, s>>>(P);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_walk(const WalkParams<T>& P, int cpl, int nsm, cudaStream_t s) {
  switch (cpl) {
    case 1: return launch_walk_c<T, 1>(P, nsm, s);
    case 2: return launch_walk_c<T, 2>(P, nsm, s);
    case 4: return launch_walk_c<T, 4>(P, nsm, s);
    default: return launch_walk_c<T, 8>(P, nsm, s);
  }
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

template cudaError_t launch_geometry<float>(const GeoParams&, const NodeBuf<float>&, int, int, TrajDebug*, cudaStream_t);
template cudaError_t launch_geometry<double>(const GeoParams&, const NodeBuf<double>&, int, int, TrajDebug*, cudaStream_t);
template cudaError_t launch_walk<float>(const WalkParams<float>&, int, int, cudaStream_t);
template cudaError_t launch_walk<double>(const WalkParams<double>&, int, int, cudaStream_t);
template cudaError_t launch_reduce<float>(const ReduceParams&, const float*, double*, double*, cudaStream_t);
template cudaError_t launch_reduce<double>(const ReduceParams&, const double*, double*, double*, cudaStream_t);

}  // namespace rl
