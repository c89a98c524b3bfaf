// rl_adjoint.cu -- the differentiable raytrace on sm_103a.
//
//   k_lte_cells / k_lte_lines  LTE level populations from per-cell temperature (the
//        partition sum over the molecule's levels, n_i = g_i e^{-E_i/kT} / Q as
//        pyradlite computes them, radlite.py:1106-1118), abundance and density, turned into
//        the walk's per-(cell, line) tables (line.F:1708-1823, line.F:3502-3677) plus
//        their temperature derivatives.
//   k_node_lw      node line widths from the cell widths with the stored interpolation
//        weights (get_line_dust_values, line.F:3965-4217), so the width is a parameter.
//   k_adjoint_jobs the reverse sweep of the formal solution along every ray. One warp per
//        (line, ray) item; the integrated channels of the item sit on the lanes, 32 x
//        kAdjSlots per tile. A forward pass keeps the intensity at the start of every
//        32-node chunk (checkpoint); the reverse pass then takes the chunks last to
//        first, recomputes the chunk forward from its checkpoint (intensities before
//        each segment in shared memory, SUBGRID sub-steps again in registers) and
//        propagates dL/dI backwards through the linear-source step (transfer.F:1498-1571,
//        line.F:4515-4848). Per node, the gradients with respect to the interpolated
//        line values and the line width are summed over the warp, folded with the
//        tables' temperature and abundance derivatives and scattered to the cell corners
//        as dL/d ln T, dL/d ln X, dL/d width with FP64 atomics.
//
// The recomputed forward uses the forward walk's own routines (rl_walk_common.cuh).
// Discrete decisions (velocity window, SUBGRID switch, sub-step index range, the
// N_up + N_low > 1e-3 test and the source-function fallbacks) are held fixed: the
// gradient is that of the branch the forward took.
#include <cuda_runtime.h>
#include <stdint.h>
#include "rl_device.h"
#include "rl_walk_common.cuh"
#include "rl_grad.cuh"

namespace rl {

// ------------------------------------------------------------------------------------
// LTE tables
// ------------------------------------------------------------------------------------
__global__ void k_lte_cells(LteParams<float> pf, LteParams<double> pd, bool fp64) {
  const int ncell = fp64 ? pd.ncell : pf.ncell;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int nlev = fp64 ? pd.nlev : pf.nlev;
  const double* Ek = fp64 ? pd.Ek : pf.Ek;
  const double* lng = fp64 ? pd.lng : pf.lng;
  const double T = exp((fp64 ? pd.lnT : pf.lnT)[c]);
  double m = -1e300;
  for (int i = 0; i < nlev; i++) m = fmax(m, lng[i] - Ek[i] / T);
  double q = 0.0, e = 0.0;
  for (int i = 0; i < nlev; i++) {
    const double x = exp(lng[i] - Ek[i] / T - m);
    q += x;
    e += x * (Ek[i] / T);
  }
  (fp64 ? pd.lnQ : pf.lnQ)[c] = m + log(q);
  (fp64 ? pd.Emean : pf.Emean)[c] = e / q;
}

template <typename R>
__global__ void k_lte_lines(LteParams<R> P) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)P.ncell * P.nl) return;
  const int c = (int)(i / P.nl), l = (int)(i - (long long)c * P.nl);
  const LteLine L = P.lines[l];
  const double Tk = exp(P.lnT[c]);
  const double lnQ = P.lnQ[c], Em = P.Emean[c];
  double pu = exp(P.lng[L.lu] - P.Ek[L.lu] / Tk - lnQ);
  double pd = exp(P.lng[L.ld] - P.Ek[L.ld] / Tk - lnQ);
  double du = P.Ek[L.lu] / Tk - Em, dd = P.Ek[L.ld] / Tk - Em;   // d ln n / d ln T
  if (pu < 1.0e-99) { pu = 0.0; du = 0.0; }                    // radlite.py:1117 trims these
  if (pd < 1.0e-99) { pd = 0.0; dd = 0.0; }
  const double xr = exp(P.lnX[c]) * P.rho_m[c];
  const double nup = pu * xr, ndn = pd * xr;
  const double jf = L.C1 * nup;
  const double af = L.C2 * (ndn * L.Bdu - nup * L.Bud);
  const double* du3 = P.dust + ((size_t)c * P.nl + l) * 3;
  double B = 0.0, TdB = 0.0;                                   // bplanck (setup.F:937-952) and T dB/dT
  if (Tk != 0.0) {
    const double x = 4.7989e-11 * L.nu / Tk;
    const double em1 = exp(x) - 1.0;
    const double core = 1.47455e-47 * L.nu * L.nu * L.nu / em1;
    B = core + 1.0e-290;
    TdB = core * x * (em1 + 1.0) / em1;
  }
  const double jd = du3[0] * B + du3[1];
  const double t0 = jf / L.scale * L.cphi, t1 = af * L.cphi, t2 = jd / L.scale;
  R* tb = P.tab + ((size_t)c * P.nl + l) * 4;
  tb[0] = (R)t0;
  tb[1] = (R)t1;
  tb[2] = (R)t2;
  tb[3] = (R)du3[2];
  P.nsum[(size_t)c * P.nl + l] = (R)(nup + ndn);
  R* dt = P.dtab + ((size_t)c * P.nl + l) * 5;
  dt[0] = (R)(t0 * du);
  dt[1] = (R)(L.C2 * L.cphi * (ndn * L.Bdu * dd - nup * L.Bud * du));
  dt[2] = (R)(du3[0] * TdB / L.scale);
  dt[3] = (R)t0;
  dt[4] = (R)t1;
}

// Node line widths from cell widths, with the weights the geometry stored (the same
// bilinear form as the geometry's own interpolation).
template <typename T>
__global__ void k_node_lw(NodeBuf<T> nb, const double* __restrict__ b, int nth) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)nb.nrays * nb.kmax) return;
  const int ray = (int)(i / nb.kmax), k = (int)(i - (long long)ray * nb.kmax);
  if (k >= nb.nnodes[ray]) return;
  const Corners c = corners(nb.c00[i], nb.misc[i], nth);
  const double dr = (double)nb.wr[i], dt = (double)nb.wt[i];
  const double v = (1.0 - dr) * ((1.0 - dt) * b[c.c00] + dt * b[c.c01]) + dr * ((1.0 - dt) * b[c.c10] + dt * b[c.c11]);
  nb.lw[i] = (T)v;
}

// ------------------------------------------------------------------------------------
// adjoint walk
// ------------------------------------------------------------------------------------
constexpr int kAdjSlots = 1;     // slots per lane per tile: 32 (line, channel) pairs

template <typename T>
struct AdjStage {
  LineVals<T> lv[33];
  T vl[33], hds[33], ds[33], rlw[33], q[33], ids[33], dvs[33], idvs[33], hw3[33], lg[33], ilg[33], wr[33], wt[33];
  unsigned flags[33], misc[33];
  int c00[33];
  T gacc[33][5];               // per node: d/d(jd, ad, jf, af) of the interpolated values, d/d lw
};

template <typename T>
struct AdjSlots {
  T Ibuf[33][kAdjSlots][32];   // intensity entering each segment of the current chunk
  T Isub[33][32];              // intensity entering each sub-step of a lane's refined segment
};

// d(x, a, b)/d(dtau) of the coefficients Math<T>::coeffs computes.
template <typename T>
__device__ __forceinline__ void coeffs_d(T d, T x, T a, T b, T& dx, T& da, T& db) {
  if constexpr (sizeof(T) == 4) {
    if (d < 0.25f) {   // derivative of the series form
      db = 0.5f - d * (1.f / 3.f - d * (1.f / 8.f - d * (1.f / 30.f - d * (1.f / 144.f - d * (1.f / 840.f)))));
      const float de0 = 1.f - b - d * db;
      dx = -de0;
      da = de0 - db;
    } else {
      dx = -x;
      db = a / d;
      da = x - db;
    }
  } else {
    if (d > 1.0e-6) {
      dx = -x;
      db = a / d;
      da = x - db;
    } else {
      dx = -1.0; da = 0.5; db = 0.5;
    }
  }
}

// One evaluated point: the line values v at velocity vl with profile width rl, as
// profile() and point_state() form them (phi = rl e^{-u^2}, u = (w - vl) rl;
// j = jd + jf phi, a = ad + af phi, S = j / a if a > 0), plus what the gradient reuses.
template <typename T>
struct PV { LineVals<T> v; T vl, u, E, phi, j, a, S, ra; };

template <typename T>
__device__ __forceinline__ PV<T> pv_eval(const LineVals<T>& v, T w, T vl, T rl) {
  PV<T> p;
  p.v = v; p.vl = vl;
  p.u = (w - vl) * rl;
  p.E = Math<T>::expneg(p.u * p.u);
  p.phi = rl * p.E;
  p.j = v.jd + v.jf * p.phi;
  p.a = v.ad + v.af * p.phi;
  p.ra = p.a > (T)0 ? Math<T>::rcp(p.a) : (T)0;
  p.S = p.a > (T)0 ? p.j * p.ra : (T)0;
  return p;
}

// Gradient through one evaluated point: dL/d(j, a, S) -> adds dL/d(jd, ad, jf, af) to acc
// and dL/d rl, dL/d vl through the profile.
template <typename T>
__device__ __forceinline__ void point_back(const PV<T>& p, T rl, T gj, T ga, T gS, T* acc, T& g_rl, T& g_vl) {
  // S = j/a enters only where a step used it: gS == 0 elsewhere, and there the FP32
  // reciprocal of a flushed opacity (inf) must not meet it (0 * inf)
  if (p.a > (T)0 && gS != (T)0) {
    gj += gS * p.ra;
    ga -= gS * p.S * p.ra;
  }
  acc[0] += gj;
  acc[1] += ga;
  acc[2] += gj * p.phi;
  acc[3] += ga * p.phi;
  const T gphi = gj * p.v.jf + ga * p.v.af;
  g_rl += gphi * p.E * ((T)1 - (T)2 * p.u * p.u);
  g_vl += gphi * (T)2 * p.u * rl * rl * p.E;
}

// One linear-source step backwards. In: the step's end values and the intensity before
// it; lam = dL/d(I after). Out: lam = dL/d(I before) and dL/d(j0, a0, S0, j1, a1, S1, h).
template <typename T>
struct StepGrad { T j0, a0, S0, j1, a1, S1, h; };

template <typename T>
__device__ __forceinline__ StepGrad<T> step_back(T Iprev, T& lam, T j0, T a0, T S0, T j1, T a1, T S1, T h) {
  const T dt = (a0 + a1) * h;
  const T th = (j0 + j1) * h;
  T x, ca, cb, dx, dca, dcb;
  Math<T>::coeffs(dt, x, ca, cb);
  coeffs_d<T>(dt, x, ca, cb, dx, dca, dcb);
  const T src1 = a0 > (T)0 ? S0 : S1;
  const T src2 = a1 > (T)0 ? S1 : S0;
  const T qraw = ca * src1 + cb * src2;
  const bool lin = dt > (T)1.0e-9f && qraw < th;
  const T L = lam;
  StepGrad<T> g;
  T g_dt = L * Iprev * dx;
  T g_th = (T)0, g1 = (T)0, g2 = (T)0;
  if (lin) {
    g_dt += L * (src1 * dca + src2 * dcb);
    g1 = L * ca;
    g2 = L * cb;
  } else {
    g_th = L;
  }
  g.a0 = g_dt * h; g.a1 = g_dt * h;
  g.j0 = g_th * h; g.j1 = g_th * h;
  g.S0 = (a0 > (T)0 ? g1 : (T)0) + (a1 > (T)0 ? (T)0 : g2);
  g.S1 = (a0 > (T)0 ? (T)0 : g1) + (a1 > (T)0 ? g2 : (T)0);
  g.h = g_dt * (a0 + a1) + g_th * (j0 + j1);
  lam = L * x;
  return g;
}

// Point values (j, a, S) of line values v at velocity vl with profile width rl.
template <typename T>
__device__ __forceinline__ void point_vals(const LineVals<T>& v, T w, T vl, T rl, T& j, T& a, T& S) {
  const PV<T> p = pv_eval(v, w, vl, rl);
  j = p.j; a = p.a; S = p.S;
}

template <typename T>
__device__ __forceinline__ LineVals<T> lerp_lv(const LineVals<T>& v0, const LineVals<T>& v1, T e) {
  const T ep = (T)1 - e;
  LineVals<T> o;
  o.jd = ep * v0.jd + e * v1.jd; o.ad = ep * v0.ad + e * v1.ad;
  o.jf = ep * v0.jf + e * v1.jf; o.af = ep * v0.af + e * v1.af;
  return o;
}

// Reverse of one refined or state-resetting segment. kind 0: one step over the whole
// segment; kind 1: SUBGRID points of a carried-state segment (slot_sub's grid); kind 2:
// SUBGRID points of a resetting segment (slot_slow's grid). It recomputes the points,
// their positions s_i = sleft + i lg (i = ia..ib, then the segment end) and the intensity
// before each sub-step, then walks them backwards. Accumulates into acc0 (node g-1) and
// acc1 (node g); returns dL/d rl of the segment; (cgj, cga) carry dL/d(j, a) of the end
// point in, and of the incoming point state out when it was carried (no reset).
template <typename T>
struct SlowOut {
  T lam, cgj, cga, g_rl;
  T acc0[4], acc1[4];
};

template <typename T>
__device__ __noinline__ SlowOut<T> seg_back_slow(bool init, int kind, T w, LineVals<T> v0, LineVals<T> v1, T vl0,
                                                  T vl1, T rl, T rl0, T hds, T q, T dsf, T dvs, T ids, T idvs, T hw3s,
                                                  T lgs, T ilgs, T Iin, T lam, T cgj, T cga, T* Isub) {
  // Isub: this lane's column of the warp's shared sub-step array (stride 32); the sub-step
  // positions are formed again in the reverse pass
  T acc0[4] = {0, 0, 0, 0}, acc1[4] = {0, 0, 0, 0};
  const PV<T> p0 = pv_eval(v0, w, vl0, init ? rl : rl0);   // incoming state
  const T j0 = p0.j, a0 = p0.a, S0 = p0.S;
  int ia = 1, ib = 0;
  T sleft = 0, lg = 0, ilg = 0;
  if (kind == 1) {
    const T s_c = sizeof(T) == 8 ? dsf * (w - vl0) / dvs : dsf * (w - vl0) * idvs;
    sleft = s_c - hw3s;
    lg = lgs;
    ilg = ilgs;
  } else if (kind == 2) {
    const T s_c = dsf * (w - vl0) / dvs;
    const T dls = dsf / q;
    const T sright = s_c + (T)3 * dls;
    sleft = s_c - (T)3 * dls;
    if (sright > (T)0 && sleft < dsf) {       // slot_slow refines only an overlapping window
      lg = (sright - sleft) / (T)30;
      ilg = (T)1 / lg;
    } else {
      kind = 0;
      sleft = 0;
    }
  }
  if (kind != 0) {
    ia = 0;
    if (!(sleft > (T)0)) {
      ia = (int)(-sleft * ilg);
      ia = ia < 0 ? 0 : (ia > 31 ? 31 : ia);
      while (ia > 0 && sleft + (T)(ia - 1) * lg > (T)0) ia--;
      while (ia <= 30 && !(sleft + (T)ia * lg > (T)0)) ia++;
    }
    ib = 30;
    if (!(sleft + (T)30 * lg < dsf)) {
      ib = (int)((dsf - sleft) * ilg);
      ib = ib < -1 ? -1 : (ib > 30 ? 30 : ib);
      while (ib < 30 && sleft + (T)(ib + 1) * lg < dsf) ib++;
      while (ib >= 0 && !(sleft + (T)ib * lg < dsf)) ib--;
    }
  }
  const bool halves = kind == 1 || (kind == 2 && ia <= ib);   // h = (s - s_prev)/2, else hds
  const T dls = q > (T)0 ? dsf / q : (T)0;
  int npt = 0;
  auto spos = [&](int m) -> T {   // end of sub-step m: grid point ia + m, or the segment end
    const int i = ia + m;
    return i <= ib ? sleft + (T)i * lg : dsf;
  };
  {
    T I = Iin, sj0 = j0, sa0 = a0, sS0 = S0;
    T sp = 0;
    for (int i = ia; i <= ib + 1; i++) {
      T s, pvl;
      LineVals<T> pv;
      if (i <= ib) {
        s = sleft + (T)i * lg;
        const T e = s * ids;
        pv = lerp_lv(v0, v1, e);
        pvl = ((T)1 - e) * vl0 + e * vl1;
      } else {
        s = dsf; pv = v1; pvl = vl1;
      }
      T j1, a1, S1;
      point_vals(pv, w, pvl, rl, j1, a1, S1);
      const T h = halves ? (T)0.5 * (s - sp) : hds;
      Isub[npt * 32] = I;
      npt++;
      formal(I, sj0, sa0, sS0, j1, a1, S1, h);
      sj0 = j1; sa0 = a1; sS0 = S1;
      sp = s;
    }
  }
  T g_rl = 0;
  T gj_next = cgj, ga_next = cga, gS_next = 0, gs_next = 0;
  // point m (the end of sub-step m), carried to the next iteration as its end point
  PV<T> pe;
  T e = (T)1;
  {
    const int i = ia + npt - 1;
    if (i <= ib) {
      e = spos(npt - 1) * ids;
      pe = pv_eval(lerp_lv(v0, v1, e), w, ((T)1 - e) * vl0 + e * vl1, rl);
    } else {
      pe = pv_eval(v1, w, vl1, rl);
    }
  }
  for (int m = npt - 1; m >= 0; m--) {
    const int i = ia + m;
    const bool interior = i <= ib;
    const T s = spos(m);
    const T sp = m > 0 ? spos(m - 1) : (T)0;
    PV<T> ps;
    T es = (T)0;
    if (m > 0) {
      es = sp * ids;
      ps = pv_eval(lerp_lv(v0, v1, es), w, ((T)1 - es) * vl0 + es * vl1, rl);
    } else {
      ps = p0;
    }
    const T h = halves ? (T)0.5 * (s - sp) : hds;
    const StepGrad<T> g = step_back<T>(Isub[m * 32], lam, ps.j, ps.a, ps.S, pe.j, pe.a, pe.S, h);
    T acc[4] = {0, 0, 0, 0};
    T gv = 0;
    point_back<T>(pe, rl, g.j1 + gj_next, g.a1 + ga_next, g.S1 + gS_next, acc, g_rl, gv);
    if (interior) {
      for (int k = 0; k < 4; k++) { acc0[k] += ((T)1 - e) * acc[k]; acc1[k] += e * acc[k]; }
      T ge = gs_next + (T)0.5 * g.h;
      ge += (acc[0] * (v1.jd - v0.jd) + acc[1] * (v1.ad - v0.ad) + acc[2] * (v1.jf - v0.jf) +
             acc[3] * (v1.af - v0.af) + gv * (vl1 - vl0)) * ids;
      // s_i = s_c - 3 dls + i dls/5 with dls = ds/q, q proportional to rl
      if (rl > (T)0) g_rl += ge * ((T)3 - (T)i / (T)5) * dls / rl;
    } else {
      for (int k = 0; k < 4; k++) acc1[k] += acc[k];
    }
    gs_next = -(T)0.5 * g.h;
    gj_next = g.j0; ga_next = g.a0; gS_next = g.S0;
    pe = ps;
    e = es;
  }
  if (init) {
    T gv = 0;
    point_back<T>(p0, rl, gj_next, ga_next, gS_next, acc0, g_rl, gv);
    cgj = 0; cga = 0;
  } else {
    T gj = gj_next, ga = ga_next;
    if (p0.a > (T)0 && gS_next != (T)0) {
      gj += gS_next * p0.ra;
      ga -= gS_next * p0.S * p0.ra;
    }
    cgj = gj; cga = ga;
  }
  SlowOut<T> o;
  o.lam = lam; o.cgj = cgj; o.cga = cga; o.g_rl = g_rl;
  for (int k = 0; k < 4; k++) { o.acc0[k] = acc0[k]; o.acc1[k] = acc1[k]; }
  return o;
}

// Stage nodes kb-1 .. kb+31 of a ray for line l (entries 0..32), as walk_ray stages them.
template <typename T>
__device__ __forceinline__ void adj_stage(const WalkParams<T>& P, AdjStage<T>& S, size_t row, int kb, int K, int l,
                                          int star_node, int lane) {
  const NodeBuf<T>& nb = P.nb;
  for (int pass = 0; pass < 2; pass++) {
    const int t = pass == 0 ? lane + 1 : 0;
    if (pass == 1 && lane != 0) continue;
    const int k = kb - 1 + t;
    if (k < 0 || k >= K) {
      const LineVals<T> z = {0, 0, 0, 0};
      S.lv[t] = z;
      S.vl[t] = 0; S.hds[t] = 0; S.ds[t] = 0; S.rlw[t] = 0; S.q[t] = 0; S.ids[t] = 0; S.dvs[t] = 0;
      S.idvs[t] = 0; S.hw3[t] = 0; S.lg[t] = 0; S.ilg[t] = 0; S.wr[t] = 0; S.wt[t] = 0;
      S.flags[t] = 0; S.misc[t] = 0; S.c00[t] = 0;
      continue;
    }
    const size_t o = row + k;
    const T wr = nb.wr[o], wt = nb.wt[o];
    const unsigned misc = nb.misc[o];
    const int c00 = nb.c00[o];
    const Corners c = corners(c00, misc, P.nth);
    S.lv[t] = interp_lv(P.tab, c, P.nlines, l, wr, wt);
    const T vl = nb.vl[o], ds = nb.ds[o], dvs = nb.dvseg[o], lwk = nb.lw[o];
    const T lwp = k >= 1 ? nb.lw[o - 1] : (T)0;
    const T lwav = (T)0.5 * (lwp + lwk);
    const T rlw = lwav > (T)0 ? Math<T>::div((T)1, lwav) : (T)0;
    const T qv = (dvs < (T)0 ? -dvs : dvs) * P.kq * rlw;
    const T dls = qv > (T)0 ? Math<T>::div(ds, qv) : (T)0;
    S.vl[t] = vl; S.hds[t] = (T)0.5 * ds; S.ds[t] = ds; S.rlw[t] = rlw; S.q[t] = qv;
    S.ids[t] = ds > (T)0 ? Math<T>::div((T)1, ds) : (T)0;
    S.dvs[t] = dvs;
    S.idvs[t] = dvs != (T)0 ? Math<T>::div((T)1, dvs) : (T)0;
    S.hw3[t] = (T)3 * dls;
    S.lg[t] = (T)6 * dls / (T)30;
    S.ilg[t] = dls > (T)0 ? Math<T>::div((T)30, (T)6 * dls) : (T)0;
    S.wr[t] = wr; S.wt[t] = wt; S.misc[t] = misc; S.c00[t] = c00;
    unsigned f = misc;
    if (k == 1 || (misc & kFlagHole) || k == star_node) f |= kFlagInit;
    if ((T)6 * qv > (T)1) f |= kFlagSub;
    S.flags[t] = f;
  }
  __syncwarp();
}

// Forward of one slot over segment kb+n (walk_ray's arithmetic for that slot).
template <typename T>
__device__ __forceinline__ void seg_fwd(const AdjStage<T>& S, int n, T w, T& I, T& j0, T& a0, T& S0,
                                        unsigned long long& steps) {
  const unsigned fl = S.flags[n + 1];
  const T vl1 = S.vl[n + 1], rl = S.rlw[n + 1], hds = S.hds[n + 1];
  if (!(fl & kFlagInit)) {
    bool ov = false;
    T s_c = 0;
    if (fl & kFlagSub) {
      const T vl0 = S.vl[n], dsf = S.ds[n + 1], hw3 = S.hw3[n + 1];
      s_c = sizeof(T) == 8 ? dsf * (w - vl0) / S.dvs[n + 1] : dsf * (w - vl0) * S.idvs[n + 1];
      ov = (s_c + hw3 > (T)0) && (s_c - hw3 < dsf);
    }
    if (ov) {
      const SlotOutT<T> o = slot_sub<T>(w, S.lv[n], S.lv[n + 1], S.vl[n], vl1, rl, S.ds[n + 1], S.ids[n + 1],
                                        s_c - S.hw3[n + 1], S.lg[n + 1], S.ilg[n + 1], I, j0, a0, S0);
      I = o.I; j0 = o.j0; a0 = o.a0; S0 = o.S0; steps += o.steps;
    } else {
      const LineVals<T> v = S.lv[n + 1];
      const T ph = profile(w, vl1, rl, rl);
      const T j1 = v.jd + v.jf * ph;
      const T a1 = v.ad + v.af * ph;
      const T S1 = a1 > (T)0 ? j1 * Math<T>::rcp(a1) : (T)0;
      const T dt = (a0 + a1) * hds;
      const T th = (j0 + j1) * hds;
      T x, ca, cb;
      Math<T>::coeffs(dt, x, ca, cb);
      const T src1 = a0 > (T)0 ? S0 : S1;
      const T src2 = a1 > (T)0 ? S1 : S0;
      T qv = dt > (T)1.0e-9f ? ca * src1 + cb * src2 : th;
      qv = qv < th ? qv : th;
      I = I * x + qv;
      j0 = j1; a0 = a1; S0 = S1;
      steps++;
    }
  } else {
    const SlotOutT<T> o = slot_slow<T>(true, (fl & kFlagSub) != 0, w, S.lv[n], S.lv[n + 1], S.vl[n], vl1, rl, hds,
                                       S.q[n + 1], S.ds[n + 1], S.dvs[n + 1], S.ids[n + 1], I, j0, a0, S0);
    I = o.I; j0 = o.j0; a0 = o.a0; S0 = o.S0; steps += o.steps;
  }
}

// Sum five per-lane values over the warp with a reduce-scatter (9 shuffles instead of
// 25): afterwards the lanes with (lane & 3) == 0 hold the total of value
// ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1).
template <typename T>
__device__ __forceinline__ T warp_sum5(const T* v, int lane) {
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  T a[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const T hi = i + 4 < 5 ? v[i + 4] : (T)0;
    const T send = b4 ? v[i] : hi;
    const T keep = b4 ? hi : v[i];
    a[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
  T c[2];
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const T send = b3 ? a[i] : a[i + 2];
    const T keep = b3 ? a[i + 2] : a[i];
    c[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  T d;
  {
    const T send = b2 ? c[0] : c[1];
    const T keep = b2 ? c[1] : c[0];
    d = keep + __shfl_xor_sync(0xffffffffu, send, 4);
  }
  d += __shfl_xor_sync(0xffffffffu, d, 2);
  d += __shfl_xor_sync(0xffffffffu, d, 1);
  return d;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// Scatter the per-node gradients of staged entries t0..t1 to the cell corners, folded
// into the cell parameters on the way: with the table derivatives dtab of each corner,
// dL/d ln T += w (g_jf dtab0 + g_af dtab1 + g_jd dtab2), dL/d ln X += w (g_jf tab0 +
// g_af tab1), dL/d width += w g_lw (the width enters through the node width only).
template <typename T>
__device__ __forceinline__ void adj_scatter(const AdjParams<T>& A, AdjStage<T>& S, int l, int t0, int t1, int lane) {
  for (int t = t0 + lane; t <= t1; t += 32) {
    const T* g = S.gacc[t];
    if (g[0] == (T)0 && g[2] == (T)0 && g[3] == (T)0 && g[4] == (T)0) continue;
    const Corners c = corners(S.c00[t], S.misc[t], A.W.nth);
    if constexpr (sizeof(T) == 4) {
      // FP32 walk: weights and products in FP32 (the FP64 pipe of this GPU is a small
      // fraction of the FP32 one), the three gradients of a corner in one vector atomic
      const float wr = S.wr[t], wt = S.wt[t];
      const float ar = 1.f - wr, at = 1.f - wt;
      const int cs[4] = {c.c00, c.c01, c.c10, c.c11};
      const float ws[4] = {ar * at, ar * wt, wr * at, wr * wt};
      const float gjd = g[0], gjf = g[2], gaf = g[3], glw = g[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (ws[q] == 0.f) continue;
        const float* d = A.dtab + ((size_t)cs[q] * A.W.nlines + l) * 5;
        const float gT = gjf * __ldg(d + 0) + gaf * __ldg(d + 1) + gjd * __ldg(d + 2);
        const float gX = gjf * __ldg(d + 3) + gaf * __ldg(d + 4);
        atomicAdd(A.g4 + cs[q], make_float4(ws[q] * gT, ws[q] * gX, ws[q] * glw, 0.f));
      }
      continue;
    }
    const double wr = (double)S.wr[t], wt = (double)S.wt[t];
    const double ar = 1.0 - wr, at = 1.0 - wt;
    const int cs[4] = {c.c00, c.c01, c.c10, c.c11};
    const double ws[4] = {ar * at, ar * wt, wr * at, wr * wt};
    const double gjd = (double)g[0], gjf = (double)g[2], gaf = (double)g[3], glw = (double)g[4];
    for (int q = 0; q < 4; q++) {
      if (ws[q] == 0.0) continue;
      const T* d = A.dtab + ((size_t)cs[q] * A.W.nlines + l) * 5;
      const double gT = gjf * (double)__ldg(d + 0) + gaf * (double)__ldg(d + 1) + gjd * (double)__ldg(d + 2);
      const double gX = gjf * (double)__ldg(d + 3) + gaf * (double)__ldg(d + 4);
      if (gT != 0.0) atomicAdd(A.g_lnT + cs[q], ws[q] * gT);
      if (gX != 0.0) atomicAdd(A.g_lnX + cs[q], ws[q] * gX);
      if (glw != 0.0) atomicAdd(A.g_b + cs[q], ws[q] * glw);   // node width: bilinear in all corners
    }
  }
  __syncwarp();
}

template <typename T>
__device__ void adjoint_item(const AdjParams<T>& A, int item, AdjStage<T>& S, AdjSlots<T>& SL, unsigned short* list,
                             T* ck, long long ckcap, int every, int lane, unsigned long long& steps,
                             unsigned long long& zero_cont) {
  const WalkParams<T>& P = A.W;
  const NodeBuf<T>& nb = P.nb;
  const int nrays = nb.nrays;
  const int l = item / nrays, ray = item - l * nrays;
  const int K = nb.nnodes[ray];
  if (nb.status[ray] != 0 || K < 1) {
    if (lane == 0) atomicCAS(P.err, 0, 100 + nb.status[ray]);
    return;
  }
  const size_t row = (size_t)ray * nb.kmax;
  // 1. velocity window of this line (as the forward)
  float mn = 1.0f, mx = -1.0f;
  if (ray != 0) {
    for (int k = lane; k < K - 1; k += 32) {
      const size_t o = row + k;
      const T wr = nb.wr[o], wt = nb.wt[o];
      const Corners c = corners(nb.c00[o], nb.misc[o], P.nth);
      if (interp_1(P.nsum, c, P.nlines, l, wr, wt) > (T)1.0e-3) {
        const float d = nb.dvf[o];
        mn = fminf(mn, d); mx = fmaxf(mx, d);
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, off));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
  }
  const double* velo = P.velo + (size_t)l * P.nfr;
  const double lo = (double)mn - 2.0 * P.aksmax_c, hi = (double)mx + 2.0 * P.aksmax_c;
  int cc = -1;
  if (ray != 0 && !(velo[0] <= hi && velo[0] >= lo)) cc = 0;
  int nint = 0;
  for (int cb = 0; cb < P.nfr; cb += 32) {
    const int c = cb + lane;
    const bool valid = c < P.nfr;
    const bool in = valid && (ray == 0 || (velo[c] <= hi && velo[c] >= lo));
    if (cc < 0 && ray != 0) {
      const unsigned outm = __ballot_sync(0xffffffffu, valid && !in && c >= 1);
      if (outm) cc = cb + __ffs(outm) - 1;
    }
    const bool take = valid && (c == 0 || in || c == cc);
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (take) list[nint + __popc(m & lanemask_lt())] = (unsigned short)c;
    nint += __popc(m);
  }
  __syncwarp();
  // dL/dI of this ray: F = scale * [pi ri1^2 I_0 + sum_rings pi (ri_{j+1}^2 - ri_j^2) mean_phi I] / d^2
  const double pi = 3.14159265359;
  double wray;
  if (ray == 0) wray = pi * A.ri[1] * A.ri[1];
  else {
    const int j = (ray - 1) / A.nphi + 1;
    wray = pi * (A.ri[j + 1] * A.ri[j + 1] - A.ri[j] * A.ri[j]) / (1.0 * A.nphi);
  }
  wray *= P.lc[l].scale / (3.08572e18 * 3.08572e18);
  const double* gf = A.gflux + (size_t)l * P.nfr;
  double gcopy = 0.0;   // channels that take the continuum channel's intensity
  if (cc >= 0) {
    for (int c = lane; c < P.nfr; c += 32) {
      const bool in = velo[c] <= hi && velo[c] >= lo;
      if (!(c == 0 || in || c == cc)) gcopy += gf[c];
    }
    gcopy = warp_sum(gcopy);
  }
  int star_node = -1;
  if (ray == 0) {
    for (int kb = 0; kb < K && star_node < 0; kb += 32) {
      const int k = kb + lane;
      const bool f = k >= 1 && k < K && (nb.misc[row + k] & kFlagIr1);
      const unsigned m = __ballot_sync(0xffffffffu, f);
      if (m) star_node = kb + __ffs(m) - 1;
    }
  }
  const int nchunk = (K + 31) / 32;
  const T fstar = P.fstar;
  for (int tb = 0; tb < nint; tb += 32 * kAdjSlots) {
    const int nt = min(32 * kAdjSlots, nint - tb);
    if ((long long)nchunk * 32 * (every == 1 ? 32 : kAdjSlots) > ckcap) {   // the scratch is sized for kmax
      if (lane == 0) atomicCAS(P.err, 0, 90);
      return;
    }
    // 2. forward with checkpoints
    T I[kAdjSlots], j0[kAdjSlots], a0[kAdjSlots], S0[kAdjSlots], w[kAdjSlots];
    int ch[kAdjSlots];
#pragma unroll
    for (int u = 0; u < kAdjSlots; u++) {
      const int idx = u * 32 + lane;
      ch[u] = idx < nt ? (int)list[tb + idx] : -1;
      w[u] = ch[u] >= 0 ? P.wch[(size_t)l * P.nfr + ch[u]] : (T)0;
      I[u] = ch[u] >= 0 ? (P.isrf ? P.isrf[(size_t)l * P.nfr + ch[u]] : P.lc[l].istart) : (T)0;
      j0[u] = 0; a0[u] = 0; S0[u] = 0;
    }
    for (int cix = 0; cix < nchunk; cix++) {
      const int kb = cix * 32;
      adj_stage(P, S, row, kb, K, l, star_node, lane);
      if (every != 1) {
#pragma unroll
        for (int u = 0; u < kAdjSlots; u++) ck[(size_t)cix * 32 * kAdjSlots + u * 32 + lane] = I[u];
      }
      const int nn = min(32, K - kb);
      const int n0 = kb == 0 ? 1 : 0;
      for (int n = n0; n < nn; n++) {
#pragma unroll
        for (int u = 0; u < kAdjSlots; u++) {
          if (ch[u] < 0) continue;
          if (kb + n == star_node) I[u] = ((T)1 - fstar) * I[u] + fstar * P.star[(size_t)l * P.nfr + ch[u]];
          if (every == 1) ck[((size_t)cix * 32 + n) * 32 + lane] = I[u];   // intensity entering the segment
          seg_fwd<T>(S, n, w[u], I[u], j0[u], a0[u], S0[u], steps);
        }
      }
      __syncwarp();
    }
    // seeds
    T lam[kAdjSlots], cgj[kAdjSlots], cga[kAdjSlots];
#pragma unroll
    for (int u = 0; u < kAdjSlots; u++) {
      lam[u] = 0; cgj[u] = 0; cga[u] = 0;
      if (ch[u] < 0) continue;
      double g = gf[ch[u]];
      if (ch[u] == cc) {
        g += gcopy;
        if (I[u] == (T)0) zero_cont++;
      }
      lam[u] = (T)(g * wray);
    }
    // 3. reverse, chunk by chunk
    for (int cix = nchunk - 1; cix >= 0; cix--) {
      const int kb = cix * 32;
      adj_stage(P, S, row, kb, K, l, star_node, lane);
      for (int t = lane; t < 33; t += 32)
#pragma unroll
        for (int k = 0; k < 5; k++) S.gacc[t][k] = 0;
      const int nn = min(32, K - kb);
      const int n0 = kb == 0 ? 1 : 0;
      // recompute the chunk from its checkpoint (interval 32), or read the stored
      // intensities back (interval 1)
#pragma unroll
      for (int u = 0; u < kAdjSlots && every != 1; u++) {
        T Iu = ck[(size_t)cix * 32 * kAdjSlots + u * 32 + lane];
        T sj = 0, sa = 0, sS = 0;
        if (ch[u] >= 0 && kb > 0) point_vals(S.lv[0], w[u], S.vl[0], S.rlw[0], sj, sa, sS);
        unsigned long long dummy = 0;
        for (int n = n0; n < nn; n++) {
          if (ch[u] >= 0) {
            if (kb + n == star_node) Iu = ((T)1 - fstar) * Iu + fstar * P.star[(size_t)l * P.nfr + ch[u]];
            SL.Ibuf[n][u][lane] = Iu;
            seg_fwd<T>(S, n, w[u], Iu, sj, sa, sS, dummy);
          }
        }
      }
      // interval 1: this chunk's stored intensities, fetched together into shared memory
      if (every == 1) {
        for (int n = n0; n < nn; n++) SL.Ibuf[n][0][lane] = ck[((size_t)cix * 32 + n) * 32 + lane];
      }
      __syncwarp();
      // walk the segments backwards
      T acc1[5] = {0, 0, 0, 0, 0};    // node kb+n
      T acc0[5] = {0, 0, 0, 0, 0};    // node kb+n-1
      for (int n = nn - 1; n >= n0; n--) {
        const unsigned fl = S.flags[n + 1];
        const T rl = S.rlw[n + 1], rl0 = S.rlw[n], hds = S.hds[n + 1];
        const LineVals<T> v0 = S.lv[n], v1 = S.lv[n + 1];
        const T vl0 = S.vl[n], vl1 = S.vl[n + 1];
        T grl_seg = 0;
#pragma unroll
        for (int u = 0; u < kAdjSlots; u++) {
          const bool valid = ch[u] >= 0;
          const T Ip = !valid ? (T)0 : SL.Ibuf[n][u][lane];
          const bool init = (fl & kFlagInit) != 0;
          const int kind = init ? ((fl & kFlagSub) ? 2 : 0) : 1;
          bool ov = false;
          T hw3 = S.hw3[n + 1], lgs = S.lg[n + 1], ilgs = S.ilg[n + 1];
          if (valid && !init && (fl & kFlagSub)) {
            const T dsf = S.ds[n + 1];
            const T s_c = sizeof(T) == 8 ? dsf * (w[u] - vl0) / S.dvs[n + 1] : dsf * (w[u] - vl0) * S.idvs[n + 1];
            ov = (s_c + hw3 > (T)0) && (s_c - hw3 < dsf);
          }
          const bool slow = valid && (init || ov);
          if (slow) {
            // refined or resetting segment
            const SlowOut<T> o = seg_back_slow<T>(init, kind, w[u], v0, v1, vl0, vl1, rl, rl0, hds, S.q[n + 1],
                                                  S.ds[n + 1], S.dvs[n + 1], S.ids[n + 1], S.idvs[n + 1], hw3, lgs,
                                                  ilgs, Ip, lam[u], cgj[u], cga[u], &SL.Isub[0][lane]);
            grl_seg += o.g_rl;
            lam[u] = o.lam; cgj[u] = o.cgj; cga[u] = o.cga;
#pragma unroll
            for (int k = 0; k < 4; k++) { acc0[k] += o.acc0[k]; acc1[k] += o.acc1[k]; }
          } else if (valid) {
            // regular step
            const PV<T> q0 = pv_eval(v0, w[u], vl0, rl0);
            const PV<T> q1 = pv_eval(v1, w[u], vl1, rl);
            const StepGrad<T> g = step_back<T>(Ip, lam[u], q0.j, q0.a, q0.S, q1.j, q1.a, q1.S, hds);
            T gv = 0;
            point_back<T>(q1, rl, g.j1 + cgj[u], g.a1 + cga[u], g.S1, acc1, grl_seg, gv);
            // carried start state: dL/dS folded into (j, a)
            T gj = g.j0, ga = g.a0;
            if (q0.a > (T)0 && g.S0 != (T)0) {
              gj += g.S0 * q0.ra;
              ga -= g.S0 * q0.S * q0.ra;
            }
            cgj[u] = gj; cga[u] = ga;
          }
          if (valid) {
            if (kb + n == star_node) lam[u] *= ((T)1 - fstar);
            steps++;
          }
        }
        // width: rl = 1 / (lw_{g-1}/2 + lw_g/2)
        const T glw = -(T)0.5 * rl * rl * grl_seg;
        acc0[4] += glw;
        acc1[4] += glw;
        // node kb+n is complete for this chunk: sum over the warp
        {
          const T s = warp_sum5(acc1, lane);
          const int idx = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
          if ((lane & 3) == 0 && idx < 5) S.gacc[n + 1][idx] += s;
        }
#pragma unroll
        for (int k = 0; k < 5; k++) {
          acc1[k] = acc0[k];
          acc0[k] = 0;
        }
      }
      // what is left belongs to node kb+n0-1 (entry n0)
      {
        const T s = warp_sum5(acc1, lane);
        const int idx = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
        if ((lane & 3) == 0 && idx < 5) S.gacc[n0][idx] += s;
      }
      __syncwarp();
      adj_scatter<T>(A, S, l, kb == 0 ? 1 : 0, nn, lane);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(128) k_adjoint_jobs(AdjJobs<T> B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ AdjParams<T> jp[4];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  AdjStage<T>* stages = reinterpret_cast<AdjStage<T>*>(smem_raw);
  AdjSlots<T>* slots = reinterpret_cast<AdjSlots<T>*>(smem_raw + sizeof(AdjStage<T>) * nw);
  unsigned short* lists =
      reinterpret_cast<unsigned short*>(smem_raw + (sizeof(AdjStage<T>) + sizeof(AdjSlots<T>)) * nw);
  const int capp = (B.max_nfr + 7) & ~7;
  unsigned short* list = lists + (size_t)wib * capp;
  T* ck = B.ckpt + ((size_t)blockIdx.x * nw + wib) * (size_t)B.ckpt_warp;
  unsigned long long steps = 0, zc = 0;
  int cur = -1;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(B.work, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= B.total) break;
    const int j = find_job(B.item_prefix, B.njobs, item);
    if (j != cur) {
      __syncwarp();
      const int* src = reinterpret_cast<const int*>(B.jobs + j);
      int* dst = reinterpret_cast<int*>(&jp[wib]);
      for (int w = lane; w < (int)(sizeof(AdjParams<T>) / 4); w += 32) dst[w] = __ldg(src + w);
      __syncwarp();
      cur = j;
    }
    adjoint_item<T>(jp[wib], item - __ldg(&B.item_prefix[j]), stages[wib], slots[wib], list, ck, B.ckpt_warp, B.every,
                    lane, steps, zc);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    steps += __shfl_xor_sync(0xffffffffu, steps, off);
    zc += __shfl_xor_sync(0xffffffffu, zc, off);
  }
  if (lane == 0) {
    atomicAdd(&B.counters[0], steps);
    if (zc) atomicAdd(&B.counters[1], zc);
  }
}

// The same for one job whose parameters are a kernel argument (the constant bank) rather
// than a shared-memory copy: the single-model adjoint.
template <typename T>
__global__ void __launch_bounds__(128) k_adjoint_one(AdjParams<T> A, AdjJobs<T> B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  AdjStage<T>* stages = reinterpret_cast<AdjStage<T>*>(smem_raw);
  AdjSlots<T>* slots = reinterpret_cast<AdjSlots<T>*>(smem_raw + sizeof(AdjStage<T>) * nw);
  unsigned short* lists =
      reinterpret_cast<unsigned short*>(smem_raw + (sizeof(AdjStage<T>) + sizeof(AdjSlots<T>)) * nw);
  const int capp = (B.max_nfr + 7) & ~7;
  unsigned short* list = lists + (size_t)wib * capp;
  T* ck = B.ckpt + ((size_t)blockIdx.x * nw + wib) * (size_t)B.ckpt_warp;
  unsigned long long steps = 0, zc = 0;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(B.work, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= B.total) break;
    adjoint_item<T>(A, item, stages[wib], slots[wib], list, ck, B.ckpt_warp, B.every, lane, steps, zc);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    steps += __shfl_xor_sync(0xffffffffu, steps, off);
    zc += __shfl_xor_sync(0xffffffffu, zc, off);
  }
  if (lane == 0) {
    atomicAdd(&B.counters[0], steps);
    if (zc) atomicAdd(&B.counters[1], zc);
  }
}

// The gradient sweep (rl_grad.cuh): one warp per (ray, line group) item from the queue;
// the list of each warp's item sits in its row of the job-wide scratch.
// Counters of the gradient sweep: [0] steps, [1] zero continuum channels (per lane), [2]
// node passes with refined or resetting segments, [3] those segments (warp-uniform).
template <typename T>
__device__ __forceinline__ void grad_flush(const AdjJobs<T>& B, int lane, unsigned long long steps,
                                           unsigned long long zc, unsigned long long rp, unsigned long long rc) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    steps += __shfl_xor_sync(0xffffffffu, steps, off);
    zc += __shfl_xor_sync(0xffffffffu, zc, off);
  }
  if (lane == 0) {
    atomicAdd(&B.counters[0], steps);
    if (zc) atomicAdd(&B.counters[1], zc);
    atomicAdd(&B.counters[2], rp);
    atomicAdd(&B.counters[3], rc);
  }
}

// FP32: three blocks per SM (at most 168 registers); FP64 keeps its registers
template <typename T> struct GradMinBlocks { static constexpr int value = sizeof(T) == 4 ? 3 : 1; };

template <typename T>
__global__ void __launch_bounds__(128, GradMinBlocks<T>::value) k_grad_jobs(AdjJobs<T> B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ AdjParams<T> jp[4];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  GradStage<T>* stages = reinterpret_cast<GradStage<T>*>(smem_raw);
  GradWork<T>* works = reinterpret_cast<GradWork<T>*>(smem_raw + sizeof(GradStage<T>) * nw);
  unsigned short* list =
      reinterpret_cast<unsigned short*>(B.ckpt + ((size_t)blockIdx.x * nw + wib) * (size_t)B.ckpt_warp);
  unsigned long long steps = 0, zc = 0, rp = 0, rc = 0;
  int cur = -1;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(B.work, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= B.total) break;
    const int j = find_job(B.item_prefix, B.njobs, item);
    if (j != cur) {
      __syncwarp();
      const int* src = reinterpret_cast<const int*>(B.jobs + j);
      int* dst = reinterpret_cast<int*>(&jp[wib]);
      for (int w = lane; w < (int)(sizeof(AdjParams<T>) / 4); w += 32) dst[w] = __ldg(src + w);
      __syncwarp();
      cur = j;
    }
    grad_item<T>(jp[wib], item - __ldg(&B.item_prefix[j]), stages[wib], works[wib], list, lane, steps, zc, rp, rc);
  }
  grad_flush(B, lane, steps, zc, rp, rc);
}

template <typename T>
__global__ void __launch_bounds__(128, GradMinBlocks<T>::value) k_grad_one(AdjParams<T> A, AdjJobs<T> B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  GradStage<T>* stages = reinterpret_cast<GradStage<T>*>(smem_raw);
  GradWork<T>* works = reinterpret_cast<GradWork<T>*>(smem_raw + sizeof(GradStage<T>) * nw);
  unsigned short* list =
      reinterpret_cast<unsigned short*>(B.ckpt + ((size_t)blockIdx.x * nw + wib) * (size_t)B.ckpt_warp);
  unsigned long long steps = 0, zc = 0, rp = 0, rc = 0;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(B.work, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= B.total) break;
    grad_item<T>(A, item, stages[wib], works[wib], list, lane, steps, zc, rp, rc);
  }
  grad_flush(B, lane, steps, zc, rp, rc);
}

// ------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------
template <typename T>
cudaError_t launch_lte(const LteParams<T>& P, cudaStream_t s) {
  LteParams<float> pf{};
  LteParams<double> pd{};
  bool fp64 = sizeof(T) == 8;
  if constexpr (sizeof(T) == 8) pd = P; else pf = P;
  k_lte_cells<<<(P.ncell + 127) / 128, 128, 0, s>>>(pf, pd, fp64);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const long long n = (long long)P.ncell * P.nl;
  k_lte_lines<T><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(P);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_node_lw(const NodeBuf<T>& nb, const double* b, int nth, cudaStream_t s) {
  const long long n = (long long)nb.nrays * nb.kmax;
  k_node_lw<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(nb, b, nth);
  return cudaGetLastError();
}

template <typename T>
size_t adjoint_smem(int max_nfr) {
  const int warps = 4;
  const int capp = (max_nfr + 7) & ~7;
  return (sizeof(AdjStage<T>) + sizeof(AdjSlots<T>)) * warps + sizeof(unsigned short) * (size_t)capp * warps;
}

template <typename T>
size_t grad_smem() { return (sizeof(GradStage<T>) + sizeof(GradWork<T>)) * 4; }

// Blocks of the persistent adjoint launch of checkpoint interval `every` (0: the gradient
// sweep); the scratch holds one region per warp.
template <typename T>
cudaError_t adjoint_grid(int nsm, int max_nfr, int every, int* blocks) {
  int per_sm = 0, per_sm1 = 0;
  cudaError_t e;
  if (every == 0) {
    const size_t smem = grad_smem<T>();
    e = cudaFuncSetAttribute(k_grad_jobs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_grad_one<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_grad_jobs<T>, 128, smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm1, k_grad_one<T>, 128, smem);
  } else {
    const size_t smem = adjoint_smem<T>(max_nfr);
    e = cudaFuncSetAttribute(k_adjoint_jobs<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_adjoint_one<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint_jobs<T>, 128, smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm1, k_adjoint_one<T>, 128, smem);
  }
  if (e != cudaSuccess) return e;
  per_sm = per_sm1 < per_sm ? per_sm1 : per_sm;   // the scratch is sized for the smaller grid
  *blocks = nsm * (per_sm < 1 ? 1 : per_sm);
  return cudaSuccess;
}

// Scratch per warp in elements of T: the reverse sweep's stored intensities (interval 1:
// every node, 32: every chunk start), or the gradient sweep's (line, channel) list.
template <typename T>
long long adjoint_ckpt_per_warp(int kmax, int max_nfr, int every) {
  if (every == 0) return ((long long)kGG * max_nfr * (long long)sizeof(unsigned short) + sizeof(T) - 1) / sizeof(T) + 8;
  return (long long)((kmax + 31) / 32) * 32 * (every == 1 ? 32 : kAdjSlots);
}

// Work items of one job: (line group, ray) for the gradient sweep, (line, ray) otherwise.
int adjoint_items(int nlines, int nrays, int every) {
  return (every == 0 ? (nlines + kGG - 1) / kGG : nlines) * nrays;
}

template <typename T>
cudaError_t launch_adjoint(const AdjJobs<T>& B, int blocks, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(B.work, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  if (B.every == 0) k_grad_jobs<T><<<blocks, 128, grad_smem<T>(), s>>>(B);
  else k_adjoint_jobs<T><<<blocks, 128, adjoint_smem<T>(B.max_nfr), s>>>(B);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_adjoint_one(const AdjParams<T>& A, const AdjJobs<T>& B, int blocks, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(B.work, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  if (B.every == 0) k_grad_one<T><<<blocks, 128, grad_smem<T>(), s>>>(A, B);
  else k_adjoint_one<T><<<blocks, 128, adjoint_smem<T>(B.max_nfr), s>>>(A, B);
  return cudaGetLastError();
}

// The FP32 adjoint's accumulated {ln T, ln X, width} gradients into the FP64 outputs.
__global__ void k_adj_finish(const float4* __restrict__ g4, double* gT, double* gX, double* gb, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float4 v = g4[i];
    gT[i] = (double)v.x;
    gX[i] = (double)v.y;
    gb[i] = (double)v.z;
  }
}

cudaError_t launch_adjoint_finish(const float4* g4, double* gT, double* gX, double* gb, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const long long blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_adj_finish<<<(unsigned)blocks, 256, 0, s>>>(g4, gT, gX, gb, n);
  return cudaGetLastError();
}

template cudaError_t launch_lte<float>(const LteParams<float>&, cudaStream_t);
template cudaError_t launch_lte<double>(const LteParams<double>&, cudaStream_t);
template cudaError_t launch_node_lw<float>(const NodeBuf<float>&, const double*, int, cudaStream_t);
template cudaError_t launch_node_lw<double>(const NodeBuf<double>&, const double*, int, cudaStream_t);
template cudaError_t adjoint_grid<float>(int, int, int, int*);
template cudaError_t adjoint_grid<double>(int, int, int, int*);
template long long adjoint_ckpt_per_warp<float>(int, int, int);
template long long adjoint_ckpt_per_warp<double>(int, int, int);
template cudaError_t launch_adjoint<float>(const AdjJobs<float>&, int, cudaStream_t);
template cudaError_t launch_adjoint<double>(const AdjJobs<double>&, int, cudaStream_t);
template cudaError_t launch_adjoint_one<float>(const AdjParams<float>&, const AdjJobs<float>&, int, cudaStream_t);
template cudaError_t launch_adjoint_one<double>(const AdjParams<double>&, const AdjJobs<double>&, int, cudaStream_t);

}  // namespace rl
