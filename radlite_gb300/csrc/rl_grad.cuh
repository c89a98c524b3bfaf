// rl_grad.cuh -- the gradient sweep of the differentiable raytrace, in walk order.
//
// The adjoint of one formal-solution step I_k = I_{k-1} x_k + Q_k propagates
// lam_{k-1} = lam_k x_k, and x_k = e^{-dtau_k}: the multiplier of every step is the
// seed times e^{-D_k}, with D_k the optical depth that the ray still crosses after step k
// (line.F:4598's char_tau counted from the observer's end). So the gradient needs no
// reverse walk: the forward walk sums each channel's optical depth along the ray
// (compensated, so that differences of two partial sums keep their digits; the walk's TAU
// instances), and this sweep walks the ray again, recomputes each step and takes its
// gradient at once with lam_k = seed e^{-(T_N - T_k)}, T_k summed alike as it goes. No
// intensities are stored. (T_k rounds a little differently from the walk's sum where the
// walk adds a refined segment's sub-steps before compensating: D_k is then off by a few
// units in the last place of that segment's optical depth.)
//
// Work layout: one warp per (ray, group of up to kGG lines). The integrated (line,
// channel) pairs of the group are dealt to the lanes so that every lane holds up to kGS
// channels of ONE line (kGS independent chains per lane). Per node the lanes sum their
// slots, a segmented suffix sum over the lanes of each line forms the (node, line)
// gradient, and the first lane of each line folds it into the cell parameters and
// scatters it to the four cell corners (one vector atomic per corner).
//
// Discrete decisions are held fixed, as in the reverse sweep: the velocity window, the
// SUBGRID switch and its sub-step range, the source-function fallbacks and the thin-step
// switch of qdr_src_2 (transfer.F:1498-1571).
#pragma once

namespace rl {

constexpr int kGS = 2;        // channel slots per lane (one line per lane)
constexpr int kGG = kGroup;   // lines per gradient work item

// explicitly rounded arithmetic, as the walk rounds each operation of a step
__device__ __forceinline__ float mulr(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mulr(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float addr(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double addr(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float subr(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double subr(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float divr(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double divr(double a, double b) { return __ddiv_rn(a, b); }

template <typename T>
__device__ __forceinline__ void kadd(T& s, T& c, T x) {   // compensated s += x (Kahan)
  const T y = subr(x, c);
  const T t = addr(s, y);
  c = subr(subr(t, s), y);
  s = t;
}

// Per-warp staging of one 32-node chunk for the lines of the item (entry t = node
// kb - 1 + t), the node data of the scatter, and the item's window and lane layout.
template <typename T>
struct GradStage {
  LineVals<T> lv[kGG][33];   // the lines of the current tile
  T vl[33], hds[33], ds[33], rlw[33], dvs[33], wr[33], wt[33];
  T gq[33], gids[33], gidvs[33], gdls[33], ghw3[33], glg[33], gilg[33];   // segment geometry (GSeg)
  int c00[33];
  unsigned misc[33], flags[33];
  double gcopy[kGG];      // gradient of the channels copied from the continuum channel
  float mn[kGG], mx[kGG];
  int cont_ch[kGG];
  int lineoff[kGG + 1];   // first list entry of each line
  int lanepre[kGG + 1];   // first lane (counted over the item's tiles) of each line
};

// SUBGRID geometry of a segment (line.F:4703-4742): measure q = |dv| / (width / c), the
// window half width 3 dls with dls = ds / q, grid spacing dls / 5.
template <typename T>
struct GSeg { T q, ids, idvs, dls, hw3, lg, ilg; };
template <typename T>
__device__ __forceinline__ GSeg<T> gseg(T ds, T dvs, T rlw, T kq) {
  GSeg<T> g;
  g.q = mulr(mulr(dvs < (T)0 ? -dvs : dvs, kq), rlw);
  g.ids = ds > (T)0 ? divr((T)1, ds) : (T)0;
  g.dls = g.q > (T)0 ? divr(ds, g.q) : (T)0;
  g.idvs = dvs != (T)0 ? divr((T)1, dvs) : (T)0;
  g.hw3 = mulr((T)3, g.dls);
  g.lg = divr(mulr((T)6, g.dls), (T)30);
  g.ilg = g.dls > (T)0 ? divr((T)30, mulr((T)6, g.dls)) : (T)0;
  return g;
}

// window centre of a channel in the segment
template <typename T>
__device__ __forceinline__ T gsc(T w, T vl0, T dsf, T dvs, const GSeg<T>& G) {
  return sizeof(T) == 8 ? divr(mulr(dsf, subr(w, vl0)), dvs) : mulr(mulr(dsf, subr(w, vl0)), G.idvs);
}

// Sub-step grid of a refined segment: kind 1, the window of a carried-state segment
// (slot_sub); kind 2, the window of a resetting segment (slot_slow), which refines only
// when it overlaps the segment. Points i = ia..ib at s_i = sleft + i lg lie strictly
// inside (0, ds); the last sub-step ends at the segment end. `halves`: the sub-steps'
// half lengths are (s_i - s_{i-1}) / 2, else the segment's own (one step).
template <typename T>
struct GGrid { T sleft, lg; int ia, ib; bool halves; };
template <typename T>
__device__ __forceinline__ T gpos(const GGrid<T>& g, int i) { return fmadd((T)i, g.lg, g.sleft); }

template <typename T>
__device__ GGrid<T> ggrid(int kind, T w, T vl0, T dsf, T dvs, const GSeg<T>& G) {
  GGrid<T> g;
  g.sleft = 0; g.lg = 0; g.ia = 1; g.ib = 0; g.halves = false;
  T ilg = 0;
  if (kind == 1) {
    g.sleft = subr(gsc(w, vl0, dsf, dvs, G), G.hw3);
    g.lg = G.lg;
    ilg = G.ilg;
    g.halves = true;
  } else if (kind == 2) {
    const T s_c = divr(mulr(dsf, subr(w, vl0)), dvs);
    const T sright = addr(s_c, G.hw3);
    const T sleft = subr(s_c, G.hw3);
    if (!(sright > (T)0 && sleft < dsf)) return g;
    g.sleft = sleft;
    g.lg = divr(subr(sright, sleft), (T)30);
    ilg = divr((T)1, g.lg);
  } else {
    return g;
  }
  int ia = 0;
  if (!(g.sleft > (T)0)) {
    ia = (int)mulr(-g.sleft, ilg);
    ia = ia < 0 ? 0 : (ia > 31 ? 31 : ia);
    while (ia > 0 && gpos(g, ia - 1) > (T)0) ia--;
    while (ia <= 30 && !(gpos(g, ia) > (T)0)) ia++;
  }
  int ib = 30;
  if (!(gpos(g, 30) < dsf)) {
    ib = (int)mulr(subr(dsf, g.sleft), ilg);
    ib = ib < -1 ? -1 : (ib > 30 ? 30 : ib);
    while (ib < 30 && gpos(g, ib + 1) < dsf) ib++;
    while (ib >= 0 && !(gpos(g, ib) < dsf)) ib--;
  }
  g.ia = ia; g.ib = ib;
  if (kind == 2) g.halves = ia <= ib;
  return g;
}

// One evaluated point: u = (w - vl) rl, E = e^{-u^2}, phi = rl E, j = jd + jf phi,
// a = ad + af phi, S = j / a where a > 0 (profile and point_state of the walk).
template <typename T>
struct GPt { T j, a, S, ra, E; };
template <typename T>
__device__ __forceinline__ T gpt_a(const LineVals<T>& v, T w, T vl, T rl, T& E) {
  const T u = mulr(subr(w, vl), rl);
  E = Math<T>::expneg(mulr(u, u));
  return fmadd(v.af, mulr(rl, E), v.ad);
}
template <typename T>
__device__ __forceinline__ GPt<T> gpt(const LineVals<T>& v, T w, T vl, T rl) {
  GPt<T> p;
  p.a = gpt_a(v, w, vl, rl, p.E);
  p.j = fmadd(v.jf, mulr(rl, p.E), v.jd);
  p.ra = p.a > (T)0 ? Math<T>::rcp(p.a) : (T)0;
  p.S = p.a > (T)0 ? mulr(p.j, p.ra) : (T)0;
  return p;
}

// interpolated line values and velocity at fraction e of the segment
template <typename T>
__device__ __forceinline__ void glerp(const LineVals<T>& v0, const LineVals<T>& v1, T vl0, T vl1, T e,
                                      LineVals<T>& v, T& vl) {
  const T ep = subr((T)1, e);
  v.jd = fmadd(e, v1.jd, mulr(ep, v0.jd)); v.ad = fmadd(e, v1.ad, mulr(ep, v0.ad));
  v.jf = fmadd(e, v1.jf, mulr(ep, v0.jf)); v.af = fmadd(e, v1.af, mulr(ep, v0.af));
  vl = fmadd(e, vl1, mulr(ep, vl0));
}

// derivatives of Math<T>::coeffs' (x, a, b) with respect to the optical depth, both forms
// evaluated and selected per slot
template <typename T>
__device__ __forceinline__ void gcoeffs_d(T d, T x, T a, T b, T& dx, T& da, T& db) {
  if constexpr (sizeof(T) == 4) {
    // below 0.25 the coefficients are the series forms (b from its Taylor series, e0 = d (1 - b))
    const float dbs = 0.5f - d * (1.f / 3.f - d * (1.f / 8.f - d * (1.f / 30.f - d * (1.f / 144.f - d * (1.f / 840.f)))));
    const float de0 = 1.f - b - d * dbs;
    const float dbd = a * Math<float>::rcp(d);
    const bool ser = d < 0.25f;
    db = ser ? dbs : dbd;
    dx = ser ? -de0 : -x;
    da = ser ? de0 - dbs : x - dbd;
  } else {
    if (d > 1.0e-6) {
      dx = -x; db = a / d; da = x - db;
    } else {
      dx = -1.0; da = 0.5; db = 0.5;
    }
  }
}

// The linear-source step of the walk (qdr_src_2) between points (j0, a0, S0) and
// (j1, a1, S1) over half length h, and its gradient for the multiplier lam of the
// intensity after it. Returns the new intensity; g: dL/d(j0 = j1 part, a part) per
// point (the step uses j and a of both points with the same weight h), dL/dS of each
// point, dL/dh.
template <typename T>
struct GStep { T x, gj, ga, gS0, gS1, gh, dt; };
template <typename T>
__device__ __forceinline__ void gstep_fwd(T& I, T j0, T a0, T S0, T j1, T a1, T S1, T h, T& x, T& ca, T& cb, T& dt,
                                          T& th, T& src1, T& src2, T& qraw) {
  dt = mulr(addr(a0, a1), h);
  th = mulr(addr(j0, j1), h);
  Math<T>::coeffs(dt, x, ca, cb);
  src1 = a0 > (T)0 ? S0 : S1;
  src2 = a1 > (T)0 ? S1 : S0;
  qraw = fmadd(ca, src1, mulr(cb, src2));
  T qv = dt > (T)1.0e-9f ? qraw : th;
  qv = qv < th ? qv : th;
  I = fmadd(I, x, qv);
}
template <typename T>
__device__ __forceinline__ GStep<T> gstep_back(T lam, T Ip, T j0, T a0, T j1, T a1, T h, T x, T ca, T cb, T dt, T th,
                                               T src1, T src2, T qraw) {
  T dx, dca, dcb;
  gcoeffs_d<T>(dt, x, ca, cb, dx, dca, dcb);
  const bool lin = dt > (T)1.0e-9f && qraw < th;
  const T g_dt = lam * Ip * dx + (lin ? lam * (src1 * dca + src2 * dcb) : (T)0);
  const T g_th = lin ? (T)0 : lam;
  const T g1 = lin ? lam * ca : (T)0, g2 = lin ? lam * cb : (T)0;
  GStep<T> g;
  g.ga = g_dt * h;
  g.gj = g_th * h;
  g.gS0 = (a0 > (T)0 ? g1 : (T)0) + (a1 > (T)0 ? (T)0 : g2);
  g.gS1 = (a0 > (T)0 ? (T)0 : g1) + (a1 > (T)0 ? g2 : (T)0);
  g.gh = g_dt * (a0 + a1) + g_th * (j0 + j1);
  return g;
}

// dL/d(j, a) of a point with its dL/dS folded in (S = j / a where a > 0)
template <typename T>
__device__ __forceinline__ void gfold(T a, T ra, T S, T gS, T& gj, T& ga) {
  if (a > (T)0 && gS != (T)0) {
    gj += gS * ra;
    ga -= gS * S * ra;
  }
}

// Gradient of a point through its evaluation (j = jd + jf phi, a = ad + af phi,
// phi = rl e^{-u^2}, u = (w - vl) rl): adds dL/d(jd, ad, jf, af) to acc and returns
// dL/d rl; g_vl receives dL/d vl.
template <typename T>
__device__ __forceinline__ T gpoint_back(const LineVals<T>& v, T w, T vl, T rl, T E, T gj, T ga, T* acc, T& g_vl) {
  const T u = (w - vl) * rl;
  const T phi = rl * E;
  acc[0] += gj; acc[1] += ga; acc[2] += gj * phi; acc[3] += ga * phi;
  const T gphi = gj * v.jf + ga * v.af;
  g_vl = gphi * (T)2 * u * rl * rl * E;
  return gphi * E * ((T)1 - (T)2 * u * u);
}

// One slot's state in the gradient sweep.
template <typename T>
struct GState {
  T I, j0, a0, S0, ra0, E0;   // intensity; the carried point (its values, 1/a, e^{-u^2})
  T pgj, pga;                 // the carried point's dL/d(j, a) from the step that ended at it
  T s, c;                     // compensated optical depth walked so far
};

// Contributions of one slot's segment: to node g-1 (dL/d(jd, jf, af)) and the width of
// the segment ending there (dL/d rl), and to node g and the width of this segment.
template <typename T>
struct GAcc { T p[3], rp, n[3], rn; };

// what a refined segment returns: the slot's new state, the updated contributions and
// the steps taken (passed by value so that the caller keeps both in registers)
template <typename T>
struct GRes { GState<T> st; GAcc<T> ac; int steps; };

// Per-warp queue of the refined and resetting segments of one node: the slots that need
// one are compacted over the lanes and processed one per lane (32 per round).
template <typename T>
struct GradWork {
  T st[10][32];   // slot state (GState fields), in and out
  T k[4][32];     // channel velocity, multiplier seed, optical depth of the whole ray (2)
  T ac[8][32];    // contributions (GAcc fields), out
  int line[32];
};

template <typename T>
__device__ __forceinline__ void gw_put(GradWork<T>& W, int q, const GState<T>& st) {
  W.st[0][q] = st.I; W.st[1][q] = st.j0; W.st[2][q] = st.a0; W.st[3][q] = st.S0; W.st[4][q] = st.ra0;
  W.st[5][q] = st.E0; W.st[6][q] = st.pgj; W.st[7][q] = st.pga; W.st[8][q] = st.s; W.st[9][q] = st.c;
}
template <typename T>
__device__ __forceinline__ GState<T> gw_get(const GradWork<T>& W, int q) {
  GState<T> st;
  st.I = W.st[0][q]; st.j0 = W.st[1][q]; st.a0 = W.st[2][q]; st.S0 = W.st[3][q]; st.ra0 = W.st[4][q];
  st.E0 = W.st[5][q]; st.pgj = W.st[6][q]; st.pga = W.st[7][q]; st.s = W.st[8][q]; st.c = W.st[9][q];
  return st;
}

// A refined or resetting segment of one slot, forward and gradient. kind 0: one step
// from a fresh start point; kind 1: the SUBGRID points of a carried segment; kind 2: the
// SUBGRID points of a resetting segment. rl0: width with which the carried start point
// was evaluated.
template <typename T>
__device__ __forceinline__ GRes<T> gseg_refined(int kind, bool init, T w, LineVals<T> v0, LineVals<T> v1, T vl0, T vl1,
                                             T rl, T rl0, T hds, T dsf, T dvs, GSeg<T> G, T seed, T sN, T cN,
                                             GState<T> st, GAcc<T> ac) {
  T tmp[4];
  T gv;
  // the start point: carried (evaluated with rl0), or fresh with this segment's width
  LineVals<T> pvv = v0;
  T pvl = vl0, prl = rl0, pe = 0;
  bool pint = false;
  if (init) {
    // the carried point ends here with what the step before it gave
    tmp[0] = tmp[1] = tmp[2] = tmp[3] = 0;
    ac.rp += gpoint_back(v0, w, vl0, rl0, st.E0, st.pgj, st.pga, tmp, gv);
    ac.p[0] += tmp[0]; ac.p[1] += tmp[2]; ac.p[2] += tmp[3];
    const GPt<T> p = gpt(v0, w, vl0, rl);
    st.j0 = p.j; st.a0 = p.a; st.S0 = p.S; st.ra0 = p.ra; st.E0 = p.E;
    st.pgj = 0; st.pga = 0;
    prl = rl;
  }
  const GGrid<T> gr = ggrid<T>(kind, w, vl0, dsf, dvs, G);
  int steps = 0;
  T sp = 0, ghh = 0;   // previous point's position; half its sub-step's dL/dh
  int ip = 0;          // previous point's grid index
  for (int i = gr.ia; i <= gr.ib + 1; i++) {
    const bool interior = i <= gr.ib;
    T s = dsf, e = (T)1, pvl1 = vl1;
    LineVals<T> v = v1;
    if (interior) {
      s = gpos(gr, i);
      e = mulr(s, G.ids);
      glerp(v0, v1, vl0, vl1, e, v, pvl1);
    }
    const GPt<T> p1 = gpt(v, w, pvl1, rl);
    const T h = gr.halves ? mulr((T)0.5, subr(s, sp)) : hds;
    const T Ip = st.I;
    T x, ca, cb, dt, th, src1, src2, qraw;
    gstep_fwd(st.I, st.j0, st.a0, st.S0, p1.j, p1.a, p1.S, h, x, ca, cb, dt, th, src1, src2, qraw);
    kadd(st.s, st.c, dt);
    const T D = subr(subr(sN, st.s), subr(cN, st.c));
    const T lam = seed * Math<T>::expneg(D);
    const GStep<T> g = gstep_back(lam, Ip, st.j0, st.a0, p1.j, p1.a, h, x, ca, cb, dt, th, src1, src2, qraw);
    // the previous point is complete
    T gj = st.pgj + g.gj, ga = st.pga + g.ga;
    gfold(st.a0, st.ra0, st.S0, g.gS0, gj, ga);
    tmp[0] = tmp[1] = tmp[2] = tmp[3] = 0;
    const T grl = gpoint_back(pvv, w, pvl, prl, st.E0, gj, ga, tmp, gv);
    if (!pint) {
      ac.p[0] += tmp[0]; ac.p[1] += tmp[2]; ac.p[2] += tmp[3];
      if (init) ac.rn += grl; else ac.rp += grl;
    } else {
      const T ep = (T)1 - pe;
      ac.p[0] += ep * tmp[0]; ac.p[1] += ep * tmp[2]; ac.p[2] += ep * tmp[3];
      ac.n[0] += pe * tmp[0]; ac.n[1] += pe * tmp[2]; ac.n[2] += pe * tmp[3];
      ac.rn += grl;
      // position of the point: s_i = s_c - 3 dls + i dls / 5, dls proportional to 1 / rl
      T ge = ghh - (T)0.5 * g.gh;
      ge += (tmp[0] * (v1.jd - v0.jd) + tmp[1] * (v1.ad - v0.ad) + tmp[2] * (v1.jf - v0.jf) +
             tmp[3] * (v1.af - v0.af) + gv * (vl1 - vl0)) * G.ids;
      if (rl > (T)0) ac.rn += ge * ((T)3 - (T)ip / (T)5) * G.dls / rl;
    }
    // this step's end point carries its part
    st.pgj = g.gj; st.pga = g.ga;
    gfold(p1.a, p1.ra, p1.S, g.gS1, st.pgj, st.pga);
    st.j0 = p1.j; st.a0 = p1.a; st.S0 = p1.S; st.ra0 = p1.ra; st.E0 = p1.E;
    ghh = (T)0.5 * g.gh;
    pvv = v; pvl = pvl1; prl = rl; pe = e; pint = interior; ip = i;
    sp = s;
    steps++;
  }
  GRes<T> r;
  r.st = st; r.ac = ac; r.steps = steps;
  return r;
}

// One regular step of one slot in the sweep: the step of the walk from the carried
// point to the node point, its gradient with the multiplier lamf e^{-D} (D the optical
// depth still ahead), the carried point completed (contributions to node g-1 and to the
// width of the segment ending there), and the node point carried on.
template <typename T>
__device__ __forceinline__ void gstep_regular(GState<T>& st, const LineVals<T>& v0, const LineVals<T>& v1, T w, T vl0,
                                              T vl1, T rl, T rl0, T hds, T lamf, T sN, T cN, GAcc<T>& ac) {
  const GPt<T> p1 = gpt(v1, w, vl1, rl);
  const T Ip = st.I;
  T x, ca, cb, dt, th, src1, src2, qraw;
  gstep_fwd(st.I, st.j0, st.a0, st.S0, p1.j, p1.a, p1.S, hds, x, ca, cb, dt, th, src1, src2, qraw);
  kadd(st.s, st.c, dt);
  const T lam = lamf == (T)0 ? (T)0 : lamf * Math<T>::expneg(subr(subr(sN, st.s), subr(cN, st.c)));
  const GStep<T> g = gstep_back(lam, Ip, st.j0, st.a0, p1.j, p1.a, hds, x, ca, cb, dt, th, src1, src2, qraw);
  T gj = st.pgj + g.gj, ga = st.pga + g.ga;
  gfold(st.a0, st.ra0, st.S0, g.gS0, gj, ga);
  T tmp[4] = {0, 0, 0, 0}, gv;
  ac.rp += gpoint_back(v0, w, vl0, rl0, st.E0, gj, ga, tmp, gv);
  ac.p[0] += tmp[0]; ac.p[1] += tmp[2]; ac.p[2] += tmp[3];
  st.pgj = g.gj; st.pga = g.ga;
  gfold(p1.a, p1.ra, p1.S, g.gS1, st.pgj, st.pga);
  st.j0 = p1.j; st.a0 = p1.a; st.S0 = p1.S; st.ra0 = p1.ra; st.E0 = p1.E;
}

// FP32: the regular steps of a lane's two slots as packed pairs (both slots belong to one
// line, so the node values are shared operands). Every element is rounded as in
// gstep_regular, so the optical depths equal the forward walk's. Slots that refine (skip) keep
// their state and contribute nothing here.
__device__ __forceinline__ float2 sel2(bool a, bool b, float2 t, float2 f) {
  return make_float2(a ? t.x : f.x, b ? t.y : f.y);
}
__device__ __forceinline__ void gstep_regular2(GState<float>* st, const LineVals<float>& v0, const LineVals<float>& v1,
                                               const float* w, float vl0, float vl1, float rl, float rl0, float hds,
                                               const float* lamf, const float* sN, const float* cN, const bool* skip,
                                               GAcc<float>& ac) {
  const float2 w2 = make_float2(w[0], w[1]);
  // the node point
  const float2 u1 = mul2(sub2(w2, dup2(vl1)), dup2(rl));
  const float2 m1 = mul2(dup2(-1.4426950408889634f), mul2(u1, u1));
  const float2 E1 = make_float2(ex2(m1.x), ex2(m1.y));
  const float2 ph1 = mul2(dup2(rl), E1);
  const float2 a1 = fma2(dup2(v1.af), ph1, dup2(v1.ad));
  const float2 j1 = fma2(dup2(v1.jf), ph1, dup2(v1.jd));
  const bool p1x = a1.x > 0.f, p1y = a1.y > 0.f;
  const float2 ra1 = make_float2(p1x ? Math<float>::rcp(a1.x) : 0.f, p1y ? Math<float>::rcp(a1.y) : 0.f);
  const float2 S1 = sel2(p1x, p1y, mul2(j1, ra1), dup2(0.f));
  // the step
  const float2 a0 = make_float2(st[0].a0, st[1].a0), j0 = make_float2(st[0].j0, st[1].j0);
  const float2 S0 = make_float2(st[0].S0, st[1].S0);
  const float2 dt = mul2(add2(a0, a1), dup2(hds));
  const float2 th = mul2(add2(j0, j1), dup2(hds));
  float2 xs, as, bs, xd, ad, bd;
  series2(dt, xs, as, bs);
  direct2(dt, xd, ad, bd);
  const bool sx = dt.x < 0.25f, sy = dt.y < 0.25f;
  const float2 x = sel2(sx, sy, xs, xd), ca = sel2(sx, sy, as, ad), cb = sel2(sx, sy, bs, bd);
  const bool p0x = a0.x > 0.f, p0y = a0.y > 0.f;
  const float2 src1 = sel2(p0x, p0y, S0, S1);
  const float2 src2 = sel2(p1x, p1y, S1, S0);
  const float2 qraw = fma2(ca, src1, mul2(cb, src2));
  const bool tx = dt.x > 1.0e-9f, ty = dt.y > 1.0e-9f;
  float2 qv = sel2(tx, ty, qraw, th);
  qv = sel2(qv.x < th.x, qv.y < th.y, qv, th);
  const float2 Ip = make_float2(st[0].I, st[1].I);
  const float2 In = fma2(Ip, x, qv);
  // optical depth walked and the multiplier
  float2 s2 = make_float2(st[0].s, st[1].s), c2 = make_float2(st[0].c, st[1].c);
  {
    const float2 y = sub2(dt, c2);
    const float2 t = add2(s2, y);
    c2 = sub2(sub2(t, s2), y);
    s2 = t;
  }
  const float2 D = sub2(sub2(make_float2(sN[0], sN[1]), s2), sub2(make_float2(cN[0], cN[1]), c2));
  const float2 mD = mul2(dup2(-1.4426950408889634f), D);
  const bool lx = lamf[0] != 0.f && !skip[0], ly = lamf[1] != 0.f && !skip[1];
  const float2 lam = sel2(lx, ly, mul2(make_float2(lamf[0], lamf[1]), make_float2(ex2(mD.x), ex2(mD.y))), dup2(0.f));
  // gradient of the step (gstep_back, two slots)
  const float2 r = make_float2(Math<float>::rcp(dt.x), Math<float>::rcp(dt.y));
  const float2 nd = make_float2(-dt.x, -dt.y);
  float2 dbs = fma2(nd, dup2(1.f / 840.f), dup2(1.f / 144.f));
  dbs = fma2(nd, dbs, dup2(1.f / 30.f));
  dbs = fma2(nd, dbs, dup2(1.f / 8.f));
  dbs = fma2(nd, dbs, dup2(1.f / 3.f));
  dbs = fma2(nd, dbs, dup2(0.5f));
  const float2 de0 = fma2(nd, dbs, sub2(dup2(1.f), cb));
  const float2 dbd = mul2(ca, r);
  const float2 db = sel2(sx, sy, dbs, dbd);
  const float2 dx = sel2(sx, sy, make_float2(-de0.x, -de0.y), make_float2(-x.x, -x.y));
  const float2 da = sel2(sx, sy, sub2(de0, dbs), sub2(x, dbd));
  const bool nx = tx && qraw.x < th.x, ny = ty && qraw.y < th.y;   // the linear-source branch
  const float2 g_dt = fma2(mul2(lam, Ip), dx, sel2(nx, ny, mul2(lam, fma2(src1, da, mul2(src2, db))), dup2(0.f)));
  const float2 g_th = sel2(nx, ny, dup2(0.f), lam);
  const float2 g1 = sel2(nx, ny, mul2(lam, ca), dup2(0.f)), g2 = sel2(nx, ny, mul2(lam, cb), dup2(0.f));
  const float2 gS0 = add2(sel2(p0x, p0y, g1, dup2(0.f)), sel2(p1x, p1y, dup2(0.f), g2));
  const float2 gS1 = add2(sel2(p0x, p0y, dup2(0.f), g1), sel2(p1x, p1y, g2, dup2(0.f)));
  const float2 ga = mul2(g_dt, dup2(hds)), gj = mul2(g_th, dup2(hds));
  // the carried point is complete: its pending part, this step's part, dL/dS folded in
  const float2 ra0 = make_float2(st[0].ra0, st[1].ra0);
  float2 gjs = add2(make_float2(st[0].pgj, st[1].pgj), gj), gas = add2(make_float2(st[0].pga, st[1].pga), ga);
  {
    const bool fx = p0x && gS0.x != 0.f, fy = p0y && gS0.y != 0.f;
    const float2 t = mul2(gS0, ra0);
    gjs = add2(gjs, sel2(fx, fy, t, dup2(0.f)));
    gas = sub2(gas, sel2(fx, fy, mul2(t, S0), dup2(0.f)));
  }
  gjs = sel2(skip[0], skip[1], dup2(0.f), gjs);
  gas = sel2(skip[0], skip[1], dup2(0.f), gas);
  {
    const float2 u0 = mul2(sub2(w2, dup2(vl0)), dup2(rl0));
    const float2 E0 = make_float2(st[0].E0, st[1].E0);
    const float2 phi0 = mul2(dup2(rl0), E0);
    const float2 gjp = mul2(gjs, phi0), gap = mul2(gas, phi0);
    ac.p[0] += gjs.x + gjs.y;
    ac.p[1] += gjp.x + gjp.y;
    ac.p[2] += gap.x + gap.y;
    const float2 gphi = fma2(gjs, dup2(v0.jf), mul2(gas, dup2(v0.af)));
    const float2 grl = mul2(mul2(gphi, E0), fma2(dup2(-2.f), mul2(u0, u0), dup2(1.f)));
    ac.rp += grl.x + grl.y;
  }
  // the node point carries this step's part
  float2 pgj = gj, pga = ga;
  {
    const bool fx = p1x && gS1.x != 0.f, fy = p1y && gS1.y != 0.f;
    const float2 t = mul2(gS1, ra1);
    pgj = add2(pgj, sel2(fx, fy, t, dup2(0.f)));
    pga = sub2(pga, sel2(fx, fy, mul2(t, S1), dup2(0.f)));
  }
#pragma unroll
  for (int u = 0; u < 2; u++) {
    if (skip[u]) continue;
    st[u].I = u == 0 ? In.x : In.y;
    st[u].s = u == 0 ? s2.x : s2.y; st[u].c = u == 0 ? c2.x : c2.y;
    st[u].pgj = u == 0 ? pgj.x : pgj.y; st[u].pga = u == 0 ? pga.x : pga.y;
    st[u].j0 = u == 0 ? j1.x : j1.y; st[u].a0 = u == 0 ? a1.x : a1.y; st[u].S0 = u == 0 ? S1.x : S1.y;
    st[u].ra0 = u == 0 ? ra1.x : ra1.y; st[u].E0 = u == 0 ? E1.x : E1.y;
  }
}

// the staged segment geometry of entry t
template <typename T>
__device__ __forceinline__ GSeg<T> stage_seg(const GradStage<T>& S, int t) {
  GSeg<T> g;
  g.q = S.gq[t]; g.ids = S.gids[t]; g.idvs = S.gidvs[t]; g.dls = S.gdls[t]; g.hw3 = S.ghw3[t]; g.lg = S.glg[t];
  g.ilg = S.gilg[t];
  return g;
}

// Stage nodes kb-1 .. kb+31 of a ray (entries 0..32) for lines l0 .. l0+gl-1.
template <typename T>
__device__ __forceinline__ void grad_stage(const WalkParams<T>& P, GradStage<T>& S, size_t row, int kb, int K, int l0,
                                           int gl, int star_node, int lane) {
  const NodeBuf<T>& nb = P.nb;
  for (int pass = 0; pass < 2; pass++) {
    const int t = pass == 0 ? lane + 1 : 0;
    if (pass == 1 && lane != 0) continue;
    const int k = kb - 1 + t;
    if (k < 0 || k >= K) {
      const LineVals<T> z = {0, 0, 0, 0};
      for (int l = 0; l < gl; l++) S.lv[l][t] = z;
      S.vl[t] = 0; S.hds[t] = 0; S.ds[t] = 0; S.rlw[t] = 0; S.dvs[t] = 0; S.wr[t] = 0; S.wt[t] = 0;
      S.gq[t] = 0; S.gids[t] = 0; S.gidvs[t] = 0; S.gdls[t] = 0; S.ghw3[t] = 0; S.glg[t] = 0; S.gilg[t] = 0;
      S.c00[t] = 0; S.misc[t] = 0; S.flags[t] = 0;
      continue;
    }
    const size_t o = row + k;
    const T wr = nb.wr[o], wt = nb.wt[o];
    const unsigned misc = nb.misc[o];
    const int c00 = nb.c00[o];
    const Corners c = corners(c00, misc, P.nth);
    for (int l = 0; l < gl; l++) S.lv[l][t] = interp_lv(P.tab, c, P.nlines, l0 + l, wr, wt);
    const T vl = nb.vl[o], ds = nb.ds[o], dvs = nb.dvseg[o], lwk = nb.lw[o];
    const T lwp = k >= 1 ? nb.lw[o - 1] : (T)0;
    const T lwav = (T)0.5 * (lwp + lwk);
    const T rlw = lwav > (T)0 ? Math<T>::div((T)1, lwav) : (T)0;
    S.vl[t] = vl; S.hds[t] = (T)0.5 * ds; S.ds[t] = ds; S.rlw[t] = rlw; S.dvs[t] = dvs;
    S.wr[t] = wr; S.wt[t] = wt; S.misc[t] = misc; S.c00[t] = c00;
    const GSeg<T> G = gseg<T>(ds, dvs, rlw, P.kq);
    S.gq[t] = G.q; S.gids[t] = G.ids; S.gidvs[t] = G.idvs; S.gdls[t] = G.dls; S.ghw3[t] = G.hw3; S.glg[t] = G.lg;
    S.gilg[t] = G.ilg;
    unsigned f = misc;
    if (k == 1 || (misc & kFlagHole) || k == star_node) f |= kFlagInit;
    if ((T)6 * G.q > (T)1) f |= kFlagSub;
    S.flags[t] = f;
  }
  __syncwarp();
}

// Fold a (node, line) gradient into the cell parameters and scatter it to the corners:
// dL/d ln T += w (g_jf dtab0 + g_af dtab1 + g_jd dtab2), dL/d ln X += w (g_jf dtab3 +
// g_af dtab4), dL/d width += w g_lw.
template <typename T>
__device__ __forceinline__ void gscatter(const AdjParams<T>& A, int l, int c00, unsigned misc, T wr, T wt, const T* g,
                                         T glw) {
  if (g[0] == (T)0 && g[1] == (T)0 && g[2] == (T)0 && glw == (T)0) return;
  const Corners c = corners(c00, misc, A.W.nth);
  const int cs[4] = {c.c00, c.c01, c.c10, c.c11};
  const T ar = (T)1 - wr, at = (T)1 - wt;
  const T ws[4] = {ar * at, ar * wt, wr * at, wr * wt};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    if (ws[q] == (T)0) continue;
    const T* d = A.dtab + ((size_t)cs[q] * A.W.nlines + l) * 5;
    const T gT = g[1] * __ldg(d + 0) + g[2] * __ldg(d + 1) + g[0] * __ldg(d + 2);
    const T gX = g[1] * __ldg(d + 3) + g[2] * __ldg(d + 4);
    if constexpr (sizeof(T) == 4) {
      atomicAdd(A.g4 + cs[q], make_float4(ws[q] * gT, ws[q] * gX, ws[q] * glw, 0.f));
    } else {
      if (gT != (T)0) atomicAdd(A.g_lnT + cs[q], ws[q] * gT);
      if (gX != (T)0) atomicAdd(A.g_lnX + cs[q], ws[q] * gX);
      if (glw != (T)0) atomicAdd(A.g_b + cs[q], ws[q] * glw);
    }
  }
}

// One gradient work item: line group gi of ray `ray`.
template <typename T>
__device__ void grad_item(const AdjParams<T>& A, int item, GradStage<T>& S, GradWork<T>& W, unsigned short* list,
                          int lane, unsigned long long& steps, unsigned long long& zero_cont, unsigned long long& rpass,
                          unsigned long long& rch) {
  const WalkParams<T>& P = A.W;
  const NodeBuf<T>& nb = P.nb;
  const int nrays = nb.nrays;
  const int gi = item / nrays, ray = item - gi * nrays;
  const int l0 = gi * kGG, gl = min(kGG, P.nlines - l0);
  const int K = nb.nnodes[ray];
  if (nb.status[ray] != 0 || K < 1) {
    if (lane == 0) atomicCAS(P.err, 0, 100 + nb.status[ray]);
    return;
  }
  const size_t row = (size_t)ray * nb.kmax;
  // 1. velocity window of every line (telescope.F:4265-4270), as the walk forms it
  {
    float mn[kGG], mx[kGG];
#pragma unroll
    for (int l = 0; l < kGG; l++) { mn[l] = 1.0f; mx[l] = -1.0f; }
    if (ray != 0) {
      for (int k = lane; k < K - 1; k += 32) {
        const size_t o = row + k;
        const T wr = nb.wr[o], wt = nb.wt[o];
        const Corners c = corners(nb.c00[o], nb.misc[o], P.nth);
        const float d = nb.dvf[o];
#pragma unroll
        for (int l = 0; l < kGG; l++) {
          if (l < gl && interp_1(P.nsum, c, P.nlines, l0 + l, wr, wt) > (T)1.0e-3) {
            mn[l] = fminf(mn[l], d); mx[l] = fmaxf(mx[l], d);
          }
        }
      }
#pragma unroll
      for (int l = 0; l < kGG; l++) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          mn[l] = fminf(mn[l], __shfl_xor_sync(0xffffffffu, mn[l], off));
          mx[l] = fmaxf(mx[l], __shfl_xor_sync(0xffffffffu, mx[l], off));
        }
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int l = 0; l < kGG; l++)
        if (l < gl) { S.mn[l] = mn[l]; S.mx[l] = mx[l]; }
    }
  }
  __syncwarp();
  // 2. the integrated (line, channel) pairs (telescope.F:541-613), the gradient that
  //    the copied channels hand to the continuum channel, and the lanes of every line
  int nint = 0, lanes = 0;
  for (int l = 0; l < gl; l++) {
    const int lineoff = nint;
    int cc = -1;
    const double* velo = P.velo + (size_t)(l0 + l) * P.nfr;
    const double lo = (double)S.mn[l] - 2.0 * P.aksmax_c, hi = (double)S.mx[l] + 2.0 * P.aksmax_c;
    if (ray != 0 && !(velo[0] <= hi && velo[0] >= lo)) cc = 0;
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
      if (take) list[nint + __popc(m & lanemask_lt())] = (unsigned short)((l << kChBits) | c);
      nint += __popc(m);
    }
    double gcopy = 0.0;
    if (cc >= 0) {
      const double* gf = A.gflux + (size_t)(l0 + l) * P.nfr;
      for (int c = lane; c < P.nfr; c += 32) {
        const bool in = velo[c] <= hi && velo[c] >= lo;
        if (!(c == 0 || in || c == cc)) gcopy += gf[c];
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) gcopy += __shfl_xor_sync(0xffffffffu, gcopy, off);
    }
    if (lane == 0) {
      S.lineoff[l] = lineoff; S.lanepre[l] = lanes; S.cont_ch[l] = cc; S.gcopy[l] = gcopy;
    }
    lanes += (nint - lineoff + kGS - 1) / kGS;
  }
  if (lane == 0) { S.lineoff[gl] = nint; S.lanepre[gl] = lanes; }
  __syncwarp();
  int star_node = -1;
  if (ray == 0) {
    for (int kb = 0; kb < K && star_node < 0; kb += 32) {
      const int k = kb + lane;
      const bool f = k >= 1 && k < K && (nb.misc[row + k] & kFlagIr1);
      const unsigned m = __ballot_sync(0xffffffffu, f);
      if (m) star_node = kb + __ffs(m) - 1;
    }
  }
  // the star's share at the node where the central beam first meets the innermost cell,
  // I -> (1 - f) I + f I*, scales the multiplier of every step before it by (1 - f)
  const T keep0 = star_node >= 0 ? (T)1 - P.fstar : (T)1;
  // dL/dI of this ray: F = scale [pi ri1^2 I_0 + sum_rings pi (ri_{j+1}^2 - ri_j^2) mean_phi I] / d^2
  const double pi = 3.14159265359;
  double wring;
  if (ray == 0) wring = pi * A.ri[1] * A.ri[1];
  else {
    const int j = (ray - 1) / A.nphi + 1;
    wring = pi * (A.ri[j + 1] * A.ri[j + 1] - A.ri[j] * A.ri[j]) / (1.0 * A.nphi);
  }
  wring /= 3.08572e18 * 3.08572e18;
  const int nchunk = (K + 31) / 32;
  // 3. tiles of 32 lanes
  for (int tile = 0; tile * 32 < lanes; tile++) {
    const int L = tile * 32 + lane;
    int li = -1, pb = 0, m = 0;
    if (L < lanes) {
      li = 0;
      while (S.lanepre[li + 1] <= L) li++;
      pb = S.lineoff[li] + (L - S.lanepre[li]) * kGS;
      m = min(kGS, S.lineoff[li + 1] - pb);
    }
    // the tile's lines: from the line of its first lane to that of its last; only those
    // are staged
    int tl0 = 0, tl1 = 0;
    {
      const int Lb = tile * 32, Le = min(tile * 32 + 31, lanes - 1);
      while (S.lanepre[tl0 + 1] <= Lb) tl0++;
      tl1 = tl0;
      while (S.lanepre[tl1 + 1] <= Le) tl1++;
    }
    const int tgl = tl1 - tl0 + 1;
    const int lit = li < 0 ? tl0 : li;   // the lane's line in the item (a staged one for idle lanes)
    const int lsafe = lit - tl0;         // and among the staged lines
    // segmented sums over the lanes of each line: lanes lane+d of the same line
    unsigned same = 0;
#pragma unroll
    for (int b = 0; b < 5; b++) {
      const int d = 1 << b;
      const int lo = __shfl_down_sync(0xffffffffu, li, d);
      if (lane + d < 32 && lo == li) same |= 1u << b;
    }
    const int lup = __shfl_up_sync(0xffffffffu, li, 1);
    const bool head = li >= 0 && (lane == 0 || lup != li);
    T w[kGS], seed[kGS], sN[kGS], cN[kGS];
    int ch[kGS];
    GState<T> st[kGS];
    const T istart = P.lc[l0 + lit].istart;
#pragma unroll
    for (int u = 0; u < kGS; u++) {
      ch[u] = -1; w[u] = 0; seed[u] = 0;
      T I0 = 0;
      if (u < m) {
        ch[u] = (int)(list[pb + u] & (kMaxChannels - 1));
        const size_t a = (size_t)(l0 + li) * P.nfr + ch[u];
        w[u] = P.wch[a];
        I0 = P.isrf ? P.isrf[a] : istart;
        double g = A.gflux[a];
        if (ch[u] == S.cont_ch[li]) g += S.gcopy[li];
        seed[u] = (T)(g * wring * P.lc[l0 + li].scale);
      }
      st[u].I = I0; st[u].j0 = 0; st[u].a0 = 0; st[u].S0 = 0; st[u].ra0 = 0; st[u].E0 = 0;
      st[u].pgj = 0; st[u].pga = 0; st[u].s = 0; st[u].c = 0;
    }
    // 3a. the optical depth of the whole ray per slot, as the forward walk summed it
#pragma unroll
    for (int u = 0; u < kGS; u++) {
      sN[u] = 0; cN[u] = 0;
      if (ch[u] >= 0) {
        const size_t a = ((size_t)(l0 + li) * nrays + ray) * P.nfr + ch[u];
        sN[u] = P.tau[a]; cN[u] = P.tauc[a];
      }
    }
    // 3b. the sweep: forward and gradient
    T keep = keep0;                // multiplier factor of the steps before the star node
    T carry[4] = {0, 0, 0, 0};     // this lane's contributions to the next node (jd, jf, af) and segment
    T hP[3] = {0, 0, 0}, hglw = 0; // head lane: the node awaiting its scatter
    T hwr = 0, hwt = 0;
    int hc00 = 0;
    unsigned hmisc = 0;
    bool hheld = false;
    for (int cix = 0; cix < nchunk; cix++) {
      const int kb = cix * 32;
      grad_stage(P, S, row, kb, K, l0 + tl0, tgl, star_node, lane);
      const int nn = min(32, K - kb);
      const int n0 = kb == 0 ? 1 : 0;
      for (int n = n0; n <= nn; n++) {
        GAcc<T> ac;
        ac.p[0] = carry[0]; ac.p[1] = carry[1]; ac.p[2] = carry[2]; ac.rp = carry[3];
        ac.n[0] = ac.n[1] = ac.n[2] = ac.rn = 0;
        const T rl0 = S.rlw[n];
        if (n < nn) {
          const unsigned fl = S.flags[n + 1];
          const T vl0 = S.vl[n], vl1 = S.vl[n + 1], rl = S.rlw[n + 1], hds = S.hds[n + 1];
          const T dsf = S.ds[n + 1], dvs = S.dvs[n + 1];
          const LineVals<T> v0 = S.lv[lsafe][n], v1 = S.lv[lsafe][n + 1];
          const bool init = (fl & kFlagInit) != 0, sub = (fl & kFlagSub) != 0;
          GSeg<T> G = {};
          if (init || sub) G = stage_seg(S, n + 1);
          bool need[kGS];
          if (kb + n == star_node) keep = (T)1;
#pragma unroll
          for (int u = 0; u < kGS; u++) {
            if (kb + n == star_node)
              st[u].I = ((T)1 - P.fstar) * st[u].I + P.fstar * P.star[(size_t)(l0 + lit) * P.nfr + (ch[u] < 0 ? 0 : ch[u])];
            bool ov = false;
            if (!init && sub) {
              const T sc = gsc(w[u], vl0, dsf, dvs, G);
              ov = ch[u] >= 0 && addr(sc, G.hw3) > (T)0 && subr(sc, G.hw3) < dsf;
            }
            need[u] = ch[u] >= 0 && (init || ov);
            if constexpr (!(sizeof(T) == 4 && kGS == 2)) {
              if (!init && !ov) {
                gstep_regular(st[u], v0, v1, w[u], vl0, vl1, rl, rl0, hds, ch[u] < 0 ? (T)0 : keep * seed[u], sN[u],
                              cN[u], ac);
                if (ch[u] >= 0) steps++;
              }
            }
          }
          if constexpr (sizeof(T) == 4 && kGS == 2) {
            if (!init) {
              const float lf[2] = {ch[0] < 0 ? 0.f : keep * seed[0], ch[1] < 0 ? 0.f : keep * seed[1]};
              gstep_regular2(st, v0, v1, w, vl0, vl1, rl, rl0, hds, lf, sN, cN, need, ac);
              steps += (ch[0] >= 0 && !need[0]) + (ch[1] >= 0 && !need[1]);
            }
          }
          // refined and resetting segments: the slots that need one, compacted over the
          // warp and walked one per lane
          int pos[kGS], cnt = 0;
#pragma unroll
          for (int u = 0; u < kGS; u++) {
            const unsigned mk = __ballot_sync(0xffffffffu, need[u]);
            pos[u] = cnt + __popc(mk & lanemask_lt());
            cnt += __popc(mk);
          }
          const int kind = init ? (sub ? 2 : 0) : 1;
          if (cnt > 0) { rpass++; rch += cnt; }   // warp-uniform counts
          for (int r0 = 0; r0 < cnt; r0 += 32) {
#pragma unroll
            for (int u = 0; u < kGS; u++) {
              const int q = pos[u] - r0;
              if (need[u] && q >= 0 && q < 32) {
                gw_put(W, q, st[u]);
                W.k[0][q] = w[u]; W.k[1][q] = keep * seed[u]; W.k[2][q] = sN[u]; W.k[3][q] = cN[u];
                W.line[q] = lsafe;
              }
            }
            __syncwarp();
            if (lane < cnt - r0) {
              const int lq = W.line[lane];
              GAcc<T> a0;
              a0.p[0] = a0.p[1] = a0.p[2] = a0.rp = a0.n[0] = a0.n[1] = a0.n[2] = a0.rn = 0;
              const GRes<T> r = gseg_refined<T>(kind, init, W.k[0][lane], S.lv[lq][n], S.lv[lq][n + 1], vl0, vl1, rl,
                                                rl0, hds, dsf, dvs, G, W.k[1][lane], W.k[2][lane], W.k[3][lane],
                                                gw_get(W, lane), a0);
              gw_put(W, lane, r.st);
              W.ac[0][lane] = r.ac.p[0]; W.ac[1][lane] = r.ac.p[1]; W.ac[2][lane] = r.ac.p[2]; W.ac[3][lane] = r.ac.rp;
              W.ac[4][lane] = r.ac.n[0]; W.ac[5][lane] = r.ac.n[1]; W.ac[6][lane] = r.ac.n[2]; W.ac[7][lane] = r.ac.rn;
              steps += r.steps;
            }
            __syncwarp();
#pragma unroll
            for (int u = 0; u < kGS; u++) {
              const int q = pos[u] - r0;
              if (need[u] && q >= 0 && q < 32) {
                st[u] = gw_get(W, q);
                ac.p[0] += W.ac[0][q]; ac.p[1] += W.ac[1][q]; ac.p[2] += W.ac[2][q]; ac.rp += W.ac[3][q];
                ac.n[0] += W.ac[4][q]; ac.n[1] += W.ac[5][q]; ac.n[2] += W.ac[6][q]; ac.rn += W.ac[7][q];
              }
            }
            __syncwarp();
          }
        } else if (cix == nchunk - 1) {
          // the ray's last point ends with what its last step gave
#pragma unroll
          for (int u = 0; u < kGS; u++) {
            T tmp[4] = {0, 0, 0, 0}, gv;
            ac.rp += gpoint_back(S.lv[lsafe][n], w[u], S.vl[n], rl0, st[u].E0, st[u].pgj, st[u].pga, tmp, gv);
            ac.p[0] += tmp[0]; ac.p[1] += tmp[2]; ac.p[2] += tmp[3];
          }
        } else {
          break;   // the chunk's last node is finished in the next chunk
        }
        carry[0] = ac.n[0]; carry[1] = ac.n[1]; carry[2] = ac.n[2]; carry[3] = ac.rn;
        // node kb+n-1 (entry n) of every line: sum over the line's lanes
        T v4[4] = {ac.p[0], ac.p[1], ac.p[2], ac.rp};
#pragma unroll
        for (int b = 0; b < 5; b++) {
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const T o = __shfl_down_sync(0xffffffffu, v4[q], 1 << b);
            if (same & (1u << b)) v4[q] += o;
          }
        }
        if (head) {
          // the segment ending at this node sets the width of both its nodes
          const T glw = -(T)0.5 * rl0 * rl0 * v4[3];
          hglw += glw;
          if (hheld) gscatter(A, l0 + li, hc00, hmisc, hwr, hwt, hP, hglw);
          hP[0] = v4[0]; hP[1] = v4[1]; hP[2] = v4[2]; hglw = glw;
          hc00 = S.c00[n]; hmisc = S.misc[n]; hwr = S.wr[n]; hwt = S.wt[n];
          hheld = true;
        }
      }
      __syncwarp();
    }
    if (head && hheld) gscatter(A, l0 + li, hc00, hmisc, hwr, hwt, hP, hglw);
    // an integrated continuum channel of exactly zero: the copies carry no gradient
#pragma unroll
    for (int u = 0; u < kGS; u++)
      if (ch[u] >= 0 && ch[u] == S.cont_ch[li] && st[u].I == (T)0) zero_cont++;
    __syncwarp();
  }
}

}  // namespace rl
