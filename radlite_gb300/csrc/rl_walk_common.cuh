// rl_walk_common.cuh -- device arithmetic shared by the forward walk (rl_kernels.cu) and
// the adjoint walk (rl_adjoint.cu): formal-solution coefficients, the Gaussian profile,
// the linear-source step, the per-node line-table interpolation, and the out-of-line
// SUBGRID and state-reset segment routines. Both kernels include this one definition so
// that the adjoint's recomputed forward follows the forward's arithmetic.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "rl_device.h"

namespace rl {

// index j with prefix[j] <= x < prefix[j+1] (prefix ascending, prefix[0] = 0)
__device__ __forceinline__ int find_job(const int* __restrict__ prefix, int njobs, int x) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&prefix[mid]) <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ------------------------------------------------------------------------------------
// walk: arithmetic helpers
// ------------------------------------------------------------------------------------
// a * b + c with one rounding, written out so that every walk variant (scalar, packed
// pairs, the adjoint's recomputation) rounds each step alike
__device__ __forceinline__ float fmadd(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmadd(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename T> struct Math;

template <> struct Math<float> {
  // e^{-x} on the MUFU pipe
  static __device__ __forceinline__ float expneg(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(__fmul_rn(-1.4426950408889634f, x)));
    return y;
  }
  static __device__ __forceinline__ float rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
  }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  // Formal-solution coefficients for optical depth d (qdr_src_2, transfer.F:1517-1528):
  //   d > 1e-6:  x = e^{-d}, e0 = 1 - x, b = (d - e0)/d, a = e0 - b
  //   else:      a = b = d/2, x = 1 - d
  // Evaluated without branches (both forms, then selects) so that independent channels
  // interleave. Below d = 0.25 b comes from its Taylor series (the FP32 difference d - e0
  // cancels there) and e0 = d (1 - b); above, e^{-d} on the MUFU pipe.
  static __device__ __forceinline__ void coeffs(float d, float& x, float& a, float& b) {
    float xs, as, bs, xd, ad, bd;
    series(d, xs, as, bs);
    direct(d, xd, ad, bd);
    const bool ser = d < 0.25f;
    x = ser ? xs : xd; a = ser ? as : ad; b = ser ? bs : bd;
  }
  // d < 0.25: b from its Taylor series, e0 = d (1 - b), x = 1 - e0. Below d = 1e-6 the
  // reference uses a = b = d/2, x = 1 - d; the series agrees with that to O(d^2), below
  // FP32 resolution, so FP32 needs no separate branch. Horner form with one rounding per
  // operation, as the packed walk evaluates it.
  static __device__ __forceinline__ void series(float d, float& x, float& a, float& b) {
    float t = __fmaf_rn(d, -1.f / 5040.f, 1.f / 720.f);
    t = __fmaf_rn(-d, t, 1.f / 120.f);
    t = __fmaf_rn(-d, t, 1.f / 24.f);
    t = __fmaf_rn(-d, t, 1.f / 6.f);
    t = __fmaf_rn(-d, t, 0.5f);
    b = __fmul_rn(d, t);
    const float e0 = __fmaf_rn(-d, b, d);
    x = __fsub_rn(1.f, e0);
    a = __fsub_rn(e0, b);
  }
  static __device__ __forceinline__ void direct(float d, float& x, float& a, float& b) {
    x = expneg(d);
    const float e0 = __fsub_rn(1.f, x);
    b = __fmul_rn(__fsub_rn(d, e0), rcp(d));
    a = __fsub_rn(e0, b);
  }
};

template <> struct Math<double> {
  static __device__ __forceinline__ void series(double d, double& x, double& a, double& b) { coeffs(d, x, a, b); }
  static __device__ __forceinline__ void direct(double d, double& x, double& a, double& b) { coeffs(d, x, a, b); }
  static __device__ __forceinline__ double expneg(double x) { return exp(-x); }
  static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ void coeffs(double d, double& x, double& a, double& b) {
    if (d > 1.0e-6) {
      x = exp(-d);
      const double e0 = 1.0 - x;
      const double e1 = d - e0;
      b = e1 / d;
      a = e0 - b;
    } else {
      a = 0.5 * d; b = a; x = 1.0 - d;
    }
  }
};

// Packed FP32 pairs (sm_100 and later): one instruction works on two independent slots.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  unsigned long long ra, rb, rd;
  asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
  float2 d;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(rd));
  return d;
}
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float ex2(float x) {   // 2^x on the MUFU pipe
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Math<float>::series and ::direct on a pair of optical depths, with the same roundings
// per element.
__device__ __forceinline__ void series2(float2 d, float2& x, float2& a, float2& b) {
  const float2 nd = make_float2(-d.x, -d.y);
  float2 t = fma2(d, dup2(-1.f / 5040.f), dup2(1.f / 720.f));
  t = fma2(nd, t, dup2(1.f / 120.f));
  t = fma2(nd, t, dup2(1.f / 24.f));
  t = fma2(nd, t, dup2(1.f / 6.f));
  t = fma2(nd, t, dup2(0.5f));
  b = mul2(d, t);
  const float2 e0 = fma2(nd, b, d);
  x = sub2(dup2(1.f), e0);
  a = sub2(e0, b);
}
__device__ __forceinline__ void direct2(float2 d, float2& x, float2& a, float2& b) {
  const float2 m = mul2(d, dup2(-1.4426950408889634f));
  x = make_float2(ex2(m.x), ex2(m.y));
  const float2 e0 = sub2(dup2(1.f), x);
  b = mul2(sub2(d, e0), make_float2(Math<float>::rcp(d.x), Math<float>::rcp(d.y)));
  a = sub2(e0, b);
}

template <typename T>
__device__ __forceinline__ T profile(T w, T vl, T rlw, T nrm) {
  const T u = (w - vl) * rlw;
  return nrm * Math<T>::expneg(u * u);
}
template <>
__device__ __forceinline__ float profile<float>(float w, float vl, float rlw, float nrm) {
  const float u = __fmul_rn(__fsub_rn(w, vl), rlw);
  return __fmul_rn(nrm, Math<float>::expneg(__fmul_rn(u, u)));
}

// One application of the linear-source formal solution (qdr_src_2, transfer.F:1498-1571)
// from point 0 (j0, a0, S0) to point 1 (j1, a1, S1) over half-length hds. Returns the
// step's optical depth 0.5 (a0 + a1) ds, the increment of char_tau (line.F:4598).
// CHK: counts in `over` the overshoot test of the reference (transfer.F:1548-1553): the
// quadrature before the bracket above twice the theoretical maximum.
template <typename T, bool CHK>
__device__ __forceinline__ T formal_c(T& I, T j0, T a0, T S0, T j1, T a1, T S1, T hds, int& over) {
  const T dtau = (a0 + a1) * hds;
  const T theo = (j0 + j1) * hds;
  T x, a, b;
  Math<T>::coeffs(dtau, x, a, b);
  const T src1 = a0 > (T)0 ? S0 : (a1 > (T)0 ? S1 : (T)0);
  const T src2 = a1 > (T)0 ? S1 : (a0 > (T)0 ? S0 : (T)0);
  T q = dtau > (T)1.0e-9f ? fmadd(a, src1, b * src2) : theo;
  if constexpr (CHK) over += q > (T)2 * theo ? 1 : 0;
  q = q < theo ? q : theo;
  I = fmadd(I, x, q);
  return dtau;
}
template <typename T>
__device__ __forceinline__ T formal(T& I, T j0, T a0, T S0, T j1, T a1, T S1, T hds) {
  int unused = 0;
  return formal_c<T, false>(I, j0, a0, S0, j1, a1, S1, hds, unused);
}

template <typename T>
struct Pt { T jd, ad, jf, af, vl; };

// point state: emissivity, extinction and own source function at the walk position
template <typename T>
__device__ __forceinline__ void point_state(const Pt<T>& p, T phi, T& j, T& a, T& S) {
  j = fmadd(p.jf, phi, p.jd);
  a = fmadd(p.af, phi, p.ad);
  S = a > (T)0 ? j * Math<T>::rcp(a) : (T)0;
}

// Lines sharing one ray per work item. The integrated (line, channel) pairs of all of
// them are packed densely over the 32 lanes x C slots of the warp.
constexpr int kGroup = 12;
constexpr int kPass = 4;                  // slots walked together (independent chains per lane)
constexpr int kChBits = 11;               // channel index bits of a packed (line, channel)
constexpr int kMaxChannels = 1 << kChBits;

template <typename T>
struct alignas(16) LineVals { T jf, af, jd, ad; };

// Per-warp staging of one 32-node chunk; entry 0 carries the last node of the previous
// chunk, entries 1..32 the nodes of this chunk. The line tables are staged for the lines of
// one tile (at most kGroup); the per-line window and continuum data cover the whole item
// (at most kItemLines lines).
template <typename T>
struct WarpStage {
  LineVals<T> lv[kGroup][33];
  T vl[33], hds[33], ds[33], rlw[33], dvs[33];
  unsigned flags[33];
  float4 hot[33];      // FP32 walk: per-node values of the packed step as pairs {vl, vl, hds, hds}
  float2 hrl[33];      // and {1/width, 1/width}
  T contv[kItemLines];
  float mn[kItemLines], mx[kItemLines];
  int cont_ch[kItemLines];
  int lineoff[kItemLines + 1];   // first list entry of each line of the item
};

// Compacted SUBGRID work of one segment: the (slot, lane) channels whose refined window
// overlaps the segment, processed one per lane.
template <typename T>
struct SubWork {
  T I[128], j0[128], a0[128], S0[128], w[128];
  unsigned char l[128];
  // a warp's totals of a launch, kept here rather than in registers: integrated pairs, node
  // visits, node passes, packed passes, steps of empty segments, overshooting steps (the
  // checking walk); refined passes, their sub-steps, their refined channels
  unsigned long long ctr[6];
  unsigned rstat[3];
};

// Per-lane state of the walk slots between chunks and slot pairs.
template <typename T, int C>
struct SlotState {
  T I[C][32], j0[C][32], a0[C][32], S0[C][32], w[C][32];
  signed char ll[C][32];   // line of the slot within the group, -1 = empty
};

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T>
__device__ __forceinline__ LineVals<T> ld_lv(const T* p) {
  LineVals<T> v;
  if constexpr (sizeof(T) == 4) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(p));
    v.jf = q.x; v.af = q.y; v.jd = q.z; v.ad = q.w;
  } else {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    v.jf = a.x; v.af = a.y; v.jd = b.x; v.ad = b.y;
  }
  return v;
}

struct Corners { int c00, c01, c10, c11; };
__device__ __forceinline__ Corners corners(int c00, unsigned misc, int nth) {
  const int dto = (int)(misc & 0xFFFFu) - 32768;
  const int dro = (int)((misc >> 16) & 3u) - 1;
  Corners c;
  c.c00 = c00; c.c01 = c00 + dto; c.c10 = c00 + dro * nth; c.c11 = c.c10 + dto;
  return c;
}

// bilinear interpolation with the reference's weighting; zero-weight corners not read
template <typename T>
__device__ __forceinline__ LineVals<T> interp_lv(const T* __restrict__ tab, const Corners& c, int nl, int l, T wr,
                                                 T wt) {
  const LineVals<T> z = {0, 0, 0, 0};
  const LineVals<T> v00 = ld_lv(tab + 4 * ((size_t)c.c00 * nl + l));
  const LineVals<T> v01 = wt != (T)0 ? ld_lv(tab + 4 * ((size_t)c.c01 * nl + l)) : z;
  LineVals<T> v10 = z, v11 = z;
  if (wr != (T)0) {
    v10 = ld_lv(tab + 4 * ((size_t)c.c10 * nl + l));
    if (wt != (T)0) v11 = ld_lv(tab + 4 * ((size_t)c.c11 * nl + l));
  }
  const T ar = (T)1 - wr, at = (T)1 - wt;
  LineVals<T> o;
  o.jf = ar * (at * v00.jf + wt * v01.jf) + wr * (at * v10.jf + wt * v11.jf);
  o.af = ar * (at * v00.af + wt * v01.af) + wr * (at * v10.af + wt * v11.af);
  o.jd = ar * (at * v00.jd + wt * v01.jd) + wr * (at * v10.jd + wt * v11.jd);
  o.ad = ar * (at * v00.ad + wt * v01.ad) + wr * (at * v10.ad + wt * v11.ad);
  return o;
}

template <typename T>
__device__ __forceinline__ T interp_1(const T* __restrict__ v, const Corners& c, int nl, int l, T wr, T wt) {
  const T v00 = __ldg(&v[(size_t)c.c00 * nl + l]);
  const T v01 = wt != (T)0 ? __ldg(&v[(size_t)c.c01 * nl + l]) : (T)0;
  T v10 = 0, v11 = 0;
  if (wr != (T)0) {
    v10 = __ldg(&v[(size_t)c.c10 * nl + l]);
    if (wt != (T)0) v11 = __ldg(&v[(size_t)c.c11 * nl + l]);
  }
  return ((T)1 - wr) * (((T)1 - wt) * v00 + wt * v01) + wr * (((T)1 - wt) * v10 + wt * v11);
}

template <typename T>
struct SlotOutBase { T I, j0, a0, S0; int steps; };
// TAU: the walk also accumulates the optical depth of the segment's steps; CHK: it counts
// the steps that fail the overshoot test
template <typename T, bool TAU> struct SlotTau {};
template <typename T> struct SlotTau<T, true> { T dtau; };
template <bool CHK> struct SlotChk {};
template <> struct SlotChk<true> { int over; };
template <typename T, bool TAU = false, bool CHK = false>
struct SlotOutT : SlotOutBase<T>, SlotTau<T, TAU>, SlotChk<CHK> {};

// Segment with a state reset (first segment, central hole, star) or with SUBGRID
// refinement (line.F:4703-4833): interior points i = ia..ib of the 31-point grid over
// [s_c - 3 l, s_c + 3 l] strictly inside (0, ds), then the segment end. Kept out of line:
// it is rare, and inlining it per slot overflows the instruction cache.
template <typename T, bool TAU = false, bool CHK = false>
__device__ __noinline__ SlotOutT<T, TAU, CHK> slot_slow(bool init, bool sub, T w, LineVals<T> v0, LineVals<T> v1, T vl0,
                                               T vl1, T rl, T hds, T q, T dsf, T dvs, T ids, T I, T j0, T a0, T S0) {
  const Pt<T> p0 = {v0.jd, v0.ad, v0.jf, v0.af, vl0};
  const Pt<T> p1 = {v1.jd, v1.ad, v1.jf, v1.af, vl1};
  if (init) {
    const T ph0 = profile(w, vl0, rl, rl);
    point_state(p0, ph0, j0, a0, S0);
  }
  int ia = 1, ib = 0;
  T sleft = 0, lg = 0;
  if (sub) {
    const T s_c = dsf * (w - vl0) / dvs;
    const T dls = dsf / q;
    const T sright = s_c + (T)3 * dls;
    sleft = s_c - (T)3 * dls;
    if (sright > (T)0 && sleft < dsf) {
      lg = (sright - sleft) / (T)30;
      ia = 0;
      if (!(sleft > (T)0)) {
        ia = (int)((-sleft) / lg);
        ia = ia < 0 ? 0 : (ia > 31 ? 31 : ia);
        while (ia > 0 && sleft + (T)(ia - 1) * lg > (T)0) ia--;
        while (ia <= 30 && !(sleft + (T)ia * lg > (T)0)) ia++;
      }
      ib = 30;
      if (!(sleft + (T)30 * lg < dsf)) {
        ib = (int)((dsf - sleft) / lg);
        ib = ib < -1 ? -1 : (ib > 30 ? 30 : ib);
        while (ib < 30 && sleft + (T)(ib + 1) * lg < dsf) ib++;
        while (ib >= 0 && !(sleft + (T)ib * lg < dsf)) ib--;
      }
    }
  }
  int steps = 0, over = 0;
  T sp = 0, tau = 0;
  for (int i = ia; i <= ib + 1; i++) {
    T s;
    Pt<T> pq;
    if (i <= ib) {
      s = sleft + (T)i * lg;
      const T e = s * ids, ep = (T)1 - e;
      pq.jd = ep * p0.jd + e * p1.jd; pq.ad = ep * p0.ad + e * p1.ad;
      pq.jf = ep * p0.jf + e * p1.jf; pq.af = ep * p0.af + e * p1.af;
      pq.vl = ep * p0.vl + e * p1.vl;
    } else {
      s = dsf; pq = p1;
    }
    const T ph = profile(w, pq.vl, rl, rl);
    T j1, a1, S1;
    point_state(pq, ph, j1, a1, S1);
    const T h = (ia <= ib) ? (T)0.5 * (s - sp) : hds;
    const T dt = formal_c<T, CHK>(I, j0, a0, S0, j1, a1, S1, h, over);
    if constexpr (TAU) tau = tau + dt;
    j0 = j1; a0 = a1; S0 = S1;
    sp = s;
    steps++;
  }
  SlotOutT<T, TAU, CHK> o;
  o.I = I; o.j0 = j0; o.a0 = a0; o.S0 = S0; o.steps = steps;
  if constexpr (TAU) o.dtau = tau;
  if constexpr (CHK) o.over = over;
  return o;
}

// SUBGRID refinement of one (line, channel) over one segment whose refined window
// overlaps it: interior points ia..ib of the grid s_i = sleft + i*lg, i = 0..30, that lie
// strictly inside (0, ds), then the segment end (line.F:4769-4821). Called for those
// channels only.
template <typename T, bool TAU = false, bool CHK = false>
__device__ __noinline__ SlotOutT<T, TAU, CHK> slot_sub(T w, LineVals<T> v0, LineVals<T> v1, T vl0, T vl1, T rl, T dsf, T ids,
                                              T sleft, T lg, T ilg, T I, T j0, T a0, T S0) {
  int ia = 0;
  if (!(sleft > (T)0)) {
    ia = (int)(-sleft * ilg);
    ia = ia < 0 ? 0 : (ia > 31 ? 31 : ia);
    while (ia > 0 && sleft + (T)(ia - 1) * lg > (T)0) ia--;
    while (ia <= 30 && !(sleft + (T)ia * lg > (T)0)) ia++;
  }
  int ib = 30;
  if (!(sleft + (T)30 * lg < dsf)) {
    ib = (int)((dsf - sleft) * ilg);
    ib = ib < -1 ? -1 : (ib > 30 ? 30 : ib);
    while (ib < 30 && sleft + (T)(ib + 1) * lg < dsf) ib++;
    while (ib >= 0 && !(sleft + (T)ib * lg < dsf)) ib--;
  }
  int steps = 0, over = 0;
  T sp = 0, tau = 0;
  for (int i = ia; i <= ib + 1; i++) {
    T s;
    Pt<T> pq;
    if (i <= ib) {
      s = sleft + (T)i * lg;
      const T e = s * ids, ep = (T)1 - e;
      pq.jd = ep * v0.jd + e * v1.jd; pq.ad = ep * v0.ad + e * v1.ad;
      pq.jf = ep * v0.jf + e * v1.jf; pq.af = ep * v0.af + e * v1.af;
      pq.vl = ep * vl0 + e * vl1;
    } else {
      s = dsf;
      pq.jd = v1.jd; pq.ad = v1.ad; pq.jf = v1.jf; pq.af = v1.af; pq.vl = vl1;
    }
    const T ph = profile(w, pq.vl, rl, rl);
    T j1, a1, S1;
    point_state(pq, ph, j1, a1, S1);
    const T dt = formal_c<T, CHK>(I, j0, a0, S0, j1, a1, S1, (T)0.5 * (s - sp), over);
    if constexpr (TAU) tau = tau + dt;
    j0 = j1; a0 = a1; S0 = S1;
    sp = s;
    steps++;
  }
  SlotOutT<T, TAU, CHK> o;
  o.I = I; o.j0 = j0; o.a0 = a0; o.S0 = S0; o.steps = steps;
  if constexpr (TAU) o.dtau = tau;
  if constexpr (CHK) o.over = over;
  return o;
}

}  // namespace rl
