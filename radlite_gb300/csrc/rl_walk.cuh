// rl_walk.cuh -- the formal-solution walk of one (line group, ray) work item, shared by
// the circular-image kernels (rl_kernels.cu) and the position-velocity cube (rl_posvel.cu).
//
// PV = false: the circular image of calc_line_spectrum (telescope.F:339-631): the central
//   beam (ray 0) integrates every channel and mixes in the star; every other ray integrates
//   channel 1, its NONREDUNDANT velocity window and one continuum channel.
// PV = true: a pixel of the rectangular image (make_freq_image_rectang,
//   telescope.F:2061-2150): every channel of every ray, no star mixing (charintline with
//   rbeam 0), and the line-of-sight optical depth char_tau per channel.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "rl_device.h"
#include "rl_walk_common.cuh"

namespace rl {

// compensated summation s += x (Kahan), c carries the lost low-order part
template <typename T>
__device__ __forceinline__ void kahan_add(T& s, T& c, T x) {
  const T y = x - c;
  const T t = s + y;
  c = (t - s) - y;
  s = t;
}

// Thin-step switch of qdr_src_2 (transfer.F:1545-1549: Q = 0.5 (j1+j2) ds unless the
// optical depth exceeds the REAL literal 1e-9) without a compare: sat(2^100 (c - dt)) is 1
// for dt <= 1e-9f and 0 above (c is the next float above 1e-9f, scaled exactly by 2^100).
constexpr float kThinScale = 1.2676506002282294e30f;   // 2^100
constexpr float kThinBias = 1.00000008e-9f * 1.2676506002282294e30f;

// Segment-dependent SUBGRID quantities (line.F:4703-4742): the refinement measure q =
// |dvmu1 - dvmu0| / (width / c), 1/ds, 1/(vl1 - vl0), the refined window half width
// 3 l = 3 ds/q and the spacing lg of its 31-point grid.
template <typename T>
struct SegGeom { T q, ids, idvs, hw3, lg, ilg; };
template <typename T>
__device__ __forceinline__ SegGeom<T> seg_geom(T ds, T dvs, T rlw, T kq) {
  SegGeom<T> g;
  g.q = (dvs < (T)0 ? -dvs : dvs) * kq * rlw;
  g.ids = ds > (T)0 ? Math<T>::div((T)1, ds) : (T)0;
  const T dls = g.q > (T)0 ? Math<T>::div(ds, g.q) : (T)0;
  g.idvs = dvs != (T)0 ? Math<T>::div((T)1, dvs) : (T)0;
  g.hw3 = (T)3 * dls;
  g.lg = (T)6 * dls / (T)30;
  g.ilg = dls > (T)0 ? Math<T>::div((T)30, (T)6 * dls) : (T)0;
  return g;
}

// zero a warp's launch totals (SubWork::ctr, rstat) before its first item
template <typename T>
__device__ __forceinline__ void zero_counters(SubWork<T>& SW, int lane) {
  if (lane < 6) SW.ctr[lane] = 0;
  if (lane < 3) SW.rstat[lane] = 0;
  __syncwarp();
}

// Formal solution of the (line, channel) pairs list[0..nt) of lines l0.. of one ray.
// The per-line tables carry the profile normalisation 0.56419583546/(3.33567e-6 nu0), so
// the profile of every slot is rlw * exp(-u^2) with the node's shared 1/linewidth.
// Work order: per 32-node chunk, per pair of slots (two independent channels per lane),
// all nodes of the chunk; the slot state lives in shared memory between pairs.
// PV: also the optical depth of every slot, Kahan-compensated in P.tau / P.tauc (the slot's
// image position), and no star mixing.
// The list entries carry item line indices; lbase is the item line of l0 (the tile's first
// line), so that entry line - lbase indexes the tile's staged lines 0..gl-1.
// TAU (circular image): the slots' optical depth is kept as in the position-velocity walk
// (for the gradient sweep of the differentiable path); nothing else changes.
// CHK: every step also takes the reference's overshoot test (transfer.F:1548-1553), and the
// steps that fail it are counted in SW.ctr[5]; the results are the same.
template <typename T, int C, bool PV = false, bool TAU = false, bool CHK = false>
__device__ unsigned walk_ray(const WalkParams<T>& P, WarpStage<T>& S, SlotState<T, C>& SS, SubWork<T>& SW, int ray,
                              int K, int l0, int gl, const unsigned short* list, int nt, int lane, int lbase,
                              unsigned long long& steps_total) {
  // FP32 circular image: steps whose two nodes have positive opacity in every line of the
  // tile, with no state reset and no SUBGRID refinement, run packed (two slots per
  // instruction) without the source-function fallbacks of qdr_src_2, which are the
  // identity there. All other steps, and the FP64 and position-velocity walks, take the
  // general path.
  constexpr bool kFast = sizeof(T) == 4 && !PV;
  constexpr bool kTau = PV || TAU;
  // TAU with one pass per chunk (at most kPass slots per lane): the sums stay in registers
  // over the whole ray and are stored once at its end
  constexpr bool kTauReg = TAU && !PV && C <= kPass;
  T tauR[kPass], tcpR[kPass];
#pragma unroll
  for (int u = 0; u < kPass; u++) { tauR[u] = 0; tcpR[u] = 0; }
  const NodeBuf<T>& nb = P.nb;
  const size_t row = (size_t)ray * nb.kmax;
  const int nl = P.nlines;
  const int nslot = (nt + 31) >> 5;
  const int npass = (nslot + kPass - 1) / kPass;
  for (int j = 0; j < kPass * npass && j < C; j++) {
    const int idx = j * 32 + lane;
    int L = -1;
    T w = 0, I = 0;
    if (idx < nt) {
      const unsigned e = list[idx];
      L = (int)(e >> kChBits) - lbase;
      w = P.wch[(size_t)(l0 + L) * P.nfr + (e & (kMaxChannels - 1))];
      I = P.isrf ? P.isrf[(size_t)(l0 + L) * P.nfr + (e & (kMaxChannels - 1))] : P.lc[l0 + L].istart;
      if constexpr (kTau && !kTauReg) {
        const size_t a = ((size_t)(l0 + L) * nb.nrays + ray) * P.nfr + (e & (kMaxChannels - 1));
        P.tau[a] = 0; P.tauc[a] = 0;
      }
    }
    SS.ll[j][lane] = L; SS.w[j][lane] = w; SS.I[j][lane] = I;
    SS.j0[j][lane] = 0; SS.a0[j][lane] = 0; SS.S0[j][lane] = 0;
  }
  // central beam: the node where the ray first reaches the innermost cell mixes in the
  // star (telescope.F:4166-4191)
  int star_node = -1;
  if (!PV && ray == 0) {
    for (int kb = 0; kb < K && star_node < 0; kb += 32) {
      const int k = kb + lane;
      const bool f = k >= 1 && k < K && (nb.misc[row + k] & kFlagIr1);
      const unsigned m = __ballot_sync(0xffffffffu, f);
      if (m) star_node = kb + __ffs(m) - 1;
    }
  }
  // per-call counts (32-bit: a call walks one tile of one ray): formal-solution steps, node
  // passes, of them on the general path and empty, and the steps of empty segments
  unsigned steps = 0, passes = 0, general = 0, emptyp = 0, skipped = 0;
  int over = 0;   // CHK: this lane's steps that failed the overshoot test
  unsigned mbits = 0;   // tile lines whose line opacity x segment length fell below -0.01
  T lw_last = 0;
  bool pos_last = true, zero_last = false;
  for (int kb = 0; kb < K; kb += 32) {
    if (kb > 0) {   // carry the last node of the previous chunk into entry 0
      if (lane == 0) {
        S.vl[0] = S.vl[32]; S.hds[0] = S.hds[32]; S.ds[0] = S.ds[32]; S.rlw[0] = S.rlw[32];
        S.dvs[0] = S.dvs[32]; S.flags[0] = S.flags[32];
        if constexpr (kFast) { S.hot[0] = S.hot[32]; S.hrl[0] = S.hrl[32]; }
      }
      if (lane < gl) S.lv[lane][0] = S.lv[lane][32];
      __syncwarp();
    }
    const int k = kb + lane;
    T vl = 0, ds = 0, dvs = 0, lwk = 0;
    unsigned misc = 0;
    bool pos = true;    // every staged line has a positive dust opacity and no inversion here
    bool zero = true;   // every staged line's emissivity and opacity factors are 0 here
    if (k < K) {
      const size_t o = row + k;
      const T wr = nb.wr[o], wt = nb.wt[o];
      misc = nb.misc[o];
      const Corners c = corners(nb.c00[o], misc, P.nth);
      for (int l = 0; l < gl; l++) {
        const LineVals<T> v = interp_lv(P.tab, c, nl, l0 + l, wr, wt);
        S.lv[l][lane + 1] = v;
        if constexpr (kFast) {
          // a positive dust opacity (subnormal ones included: their reciprocal is +inf in both
          // forms of the step, and the source brackets pick the same values) and no inversion
          pos = pos && v.ad > 0.f && v.af >= 0.f;
          zero = zero && v.jd == 0.f && v.jf == 0.f && v.ad == 0.f && v.af == 0.f;
        }
      }
      vl = nb.vl[o]; ds = nb.ds[o]; dvs = nb.dvseg[o]; lwk = nb.lw[o];
    }
    T lwp = __shfl_up_sync(0xffffffffu, lwk, 1);
    if (lane == 0) lwp = lw_last;
    lw_last = __shfl_sync(0xffffffffu, lwk, 31);
    const T lwav = (T)0.5 * (lwp + lwk);
    const T rlw = lwav > (T)0 ? Math<T>::div((T)1, lwav) : (T)0;
    S.vl[lane + 1] = vl; S.hds[lane + 1] = (T)0.5 * ds; S.ds[lane + 1] = ds; S.rlw[lane + 1] = rlw;
    S.dvs[lane + 1] = dvs;
    {
      unsigned f = misc;
      if (k == 1 || (misc & kFlagHole) || k == star_node) f |= kFlagInit;
      if ((T)6 * ((dvs < (T)0 ? -dvs : dvs) * P.kq * rlw) > (T)1) f |= kFlagSub;
      if constexpr (kFast) {
        // the step ending at this node needs both of its nodes positive
        bool posp = __shfl_up_sync(0xffffffffu, pos, 1);
        if (lane == 0) posp = pos_last;
        pos_last = __shfl_sync(0xffffffffu, pos, 31);
        if (!(pos && posp)) f |= kFlagNeg;
        // a segment between two empty nodes leaves the intensity unchanged: j = a = 0 at both
        // ends gives dtau = 0, x = 1 and Q = 0.5 (j0 + j1) ds = 0, and the carried point
        // state stays (0, 0, 0)
        bool zerop = __shfl_up_sync(0xffffffffu, zero, 1);
        if (lane == 0) zerop = zero_last;
        zero_last = __shfl_sync(0xffffffffu, zero, 31);
        if (zero && zerop) f |= kFlagEmpty;
        // node values of the packed step, duplicated into pairs: {vl, vl, hds, hds},
        // {rl, rl} (the profile's 1/width)
        const float h = 0.5f * (float)ds;
        S.hot[lane + 1] = make_float4((float)vl, (float)vl, h, h);
        S.hrl[lane + 1] = make_float2((float)rlw, (float)rlw);
      }
      S.flags[lane + 1] = f;
    }
    __syncwarp();
    const int nn = min(32, K - kb);
    const int n0 = kb == 0 ? 1 : 0;   // node 0 of the ray starts the walk
    for (int pq = 0; pq < npass; pq++) {
      T I[kPass], j0[kPass], a0[kPass], S0[kPass], w[kPass];
      int Ls[kPass], lsl[kPass];
      int nv = 0;
#pragma unroll
      for (int u = 0; u < kPass; u++) {
        const int j = kPass * pq + u;
        if (j < C) {
          I[u] = SS.I[j][lane]; j0[u] = SS.j0[j][lane]; a0[u] = SS.a0[j][lane]; S0[u] = SS.S0[j][lane];
          w[u] = SS.w[j][lane]; Ls[u] = SS.ll[j][lane];
        } else {
          I[u] = 0; j0[u] = 0; a0[u] = 0; S0[u] = 0; w[u] = 0; Ls[u] = -1;
        }
        lsl[u] = Ls[u] < 0 ? 0 : Ls[u];
        nv += Ls[u] >= 0 ? 1 : 0;
      }
      // optical depth: the position-velocity walk adds every step compensated; the TAU walk
      // sums a pass's steps plainly (part) and adds that sum compensated at the pass end,
      // so that the loads below are needed only then
      T tau[kPass], tcp[kPass], part[kPass];
      size_t ta[kPass];
#pragma unroll
      for (int u = 0; u < kPass; u++) part[u] = 0;
      auto add_tau = [&](int u, T x) {
        if constexpr (PV) kahan_add(tau[u], tcp[u], x);
        else if constexpr (TAU) part[u] += x;
      };
      if constexpr (kTau && !kTauReg) {
#pragma unroll
        for (int u = 0; u < kPass; u++) {
          tau[u] = 0; tcp[u] = 0; ta[u] = 0;
          if (Ls[u] >= 0) {
            ta[u] = ((size_t)(l0 + Ls[u]) * nb.nrays + ray) * P.nfr +
                    (list[(kPass * pq + u) * 32 + lane] & (kMaxChannels - 1));
            tau[u] = P.tau[ta[u]]; tcp[u] = P.tauc[ta[u]];
          }
        }
      }
      // every node of the pass is one step per valid slot; refinement and resets add theirs
      passes += nn - n0;
      steps += (unsigned)nv * (unsigned)(nn - n0);
      for (int n = n0; n < nn; n++) {
        const int g = kb + n;
        const unsigned fl = S.flags[n + 1];
        if constexpr (kFast) {
          if ((fl & (kFlagEmpty | kFlagInit)) == kFlagEmpty) {
            skipped += nv;
            emptyp++;
            continue;
          }
          bool slow = (fl & (kFlagInit | kFlagNeg)) != 0;
          if (!slow && (fl & kFlagSub)) {
            // a SUBGRID window that overlaps the segment sends the node to the general path
            const T vl0 = S.vl[n], dsf = S.ds[n + 1];
            const SegGeom<T> G = seg_geom<T>(dsf, S.dvs[n + 1], S.rlw[n + 1], P.kq);
            bool any = false;
#pragma unroll
            for (int u = 0; u < kPass; u++) {
              const T s_c = dsf * (w[u] - vl0) * G.idvs;
              any = any || (Ls[u] >= 0 && (s_c + G.hw3 > (T)0) && (s_c - G.hw3 < dsf));
            }
            slow = __any_sync(0xffffffffu, any);
          }
          if (!slow) {
            const float4 h0 = S.hot[n + 1];
            const float2 vl2 = make_float2(h0.x, h0.y), hd2 = make_float2(h0.z, h0.w);
            const float2 rl2 = S.hrl[n + 1];
            float2 j1[kPass / 2], a1[kPass / 2], S1[kPass / 2], dt[kPass / 2], th[kPass / 2];
            bool ser = true, dir = true;
#pragma unroll
            for (int p = 0; p < kPass / 2; p++) {
              const LineVals<T> vA = S.lv[lsl[2 * p]][n + 1], vB = S.lv[lsl[2 * p + 1]][n + 1];
              const float2 u = mul2(sub2(make_float2(w[2 * p], w[2 * p + 1]), vl2), rl2);
              const float2 m = mul2(mul2(u, u), dup2(-1.4426950408889634f));
              const float2 ph = mul2(rl2, make_float2(ex2(m.x), ex2(m.y)));
              j1[p] = make_float2(fmaf(vA.jf, ph.x, vA.jd), fmaf(vB.jf, ph.y, vB.jd));
              a1[p] = make_float2(fmaf(vA.af, ph.x, vA.ad), fmaf(vB.af, ph.y, vB.ad));
              S1[p] = mul2(j1[p], make_float2(Math<float>::rcp(a1[p].x), Math<float>::rcp(a1[p].y)));
              dt[p] = mul2(add2(make_float2(a0[2 * p], a0[2 * p + 1]), a1[p]), hd2);
              th[p] = mul2(add2(make_float2(j0[2 * p], j0[2 * p + 1]), j1[p]), hd2);
              const bool sa = dt[p].x < 0.25f, sb = dt[p].y < 0.25f;
              ser = ser && sa && sb;
              dir = dir && !sa && !sb;
            }
            ser = __all_sync(0xffffffffu, ser);
            dir = __all_sync(0xffffffffu, dir);
            float2 x[kPass / 2], ca[kPass / 2], cb[kPass / 2];
            if (ser) {
#pragma unroll
              for (int p = 0; p < kPass / 2; p++) series2(dt[p], x[p], ca[p], cb[p]);
            } else if (dir) {
#pragma unroll
              for (int p = 0; p < kPass / 2; p++) direct2(dt[p], x[p], ca[p], cb[p]);
            } else {
#pragma unroll
              for (int p = 0; p < kPass / 2; p++) {
                float2 xs, as, bs, xd, ad, bd;
                series2(dt[p], xs, as, bs);
                direct2(dt[p], xd, ad, bd);
                const bool sa = dt[p].x < 0.25f, sb = dt[p].y < 0.25f;
                x[p] = make_float2(sa ? xs.x : xd.x, sb ? xs.y : xd.y);
                ca[p] = make_float2(sa ? as.x : ad.x, sb ? as.y : ad.y);
                cb[p] = make_float2(sa ? bs.x : bd.x, sb ? bs.y : bd.y);
              }
            }
#pragma unroll
            for (int p = 0; p < kPass / 2; p++) {
              const float2 Q = fma2(ca[p], make_float2(S0[2 * p], S0[2 * p + 1]), mul2(cb[p], S1[p]));
              const float2 thin = make_float2(__saturatef(fmaf(dt[p].x, -kThinScale, kThinBias)),
                                              __saturatef(fmaf(dt[p].y, -kThinScale, kThinBias)));
              if constexpr (CHK) {
                // before the bracket the quadrature is Q, or theo for an optically thin step
                // (empty slots take discarded steps and are not counted)
                over += (Ls[2 * p] >= 0 && (dt[p].x > 1.0e-9f ? Q.x > 2.f * th[p].x : th[p].x < 0.f)) ? 1 : 0;
                over += (Ls[2 * p + 1] >= 0 && (dt[p].y > 1.0e-9f ? Q.y > 2.f * th[p].y : th[p].y < 0.f)) ? 1 : 0;
              }
              const float2 Qb = fma2(thin, dup2(3.0e38f), Q);
              const float2 q = make_float2(fminf(Qb.x, th[p].x), fminf(Qb.y, th[p].y));
              const float2 In = fma2(make_float2(I[2 * p], I[2 * p + 1]), x[p], q);
              I[2 * p] = In.x; I[2 * p + 1] = In.y;
              if constexpr (TAU) { part[2 * p] += dt[p].x; part[2 * p + 1] += dt[p].y; }
              j0[2 * p] = j1[p].x; j0[2 * p + 1] = j1[p].y;
              a0[2 * p] = a1[p].x; a0[2 * p + 1] = a1[p].y;
              S0[2 * p] = S1[p].x; S0[2 * p + 1] = S1[p].y;
            }
            continue;
          }
        }
        general++;
        if (g == star_node) {
#pragma unroll
          for (int u = 0; u < kPass; u++)
            if (Ls[u] >= 0)
              I[u] = ((T)1 - P.fstar) * I[u] +
                     P.fstar * P.star[(size_t)(l0 + Ls[u]) * P.nfr + (list[(kPass * pq + u) * 32 + lane] & (kMaxChannels - 1))];
        }
        const T vl1 = S.vl[n + 1], rl = S.rlw[n + 1], hds = S.hds[n + 1];
        if (!(fl & kFlagInit)) {
          // SUBGRID window test of the reference (line.F:4733-4742): slots whose refined
          // window [s_c - 3l, s_c + 3l] overlaps (0, ds) keep their state here and are
          // refined below; all others take one formal-solution step
          bool ov[kPass];
          bool any = false;
#pragma unroll
          for (int u = 0; u < kPass; u++) ov[u] = false;
          SegGeom<T> G = {};
          if (fl & kFlagSub) {
            const T vl0 = S.vl[n], dsf = S.ds[n + 1];
            G = seg_geom<T>(dsf, S.dvs[n + 1], rl, P.kq);
#pragma unroll
            for (int u = 0; u < kPass; u++) {
              const T s_c = sizeof(T) == 8 ? dsf * (w[u] - vl0) / S.dvs[n + 1] : dsf * (w[u] - vl0) * G.idvs;
              ov[u] = Ls[u] >= 0 && (s_c + G.hw3 > (T)0) && (s_c - G.hw3 < dsf);
              any = any || ov[u];
            }
            any = __any_sync(0xffffffffu, any);
          }
          T j1[kPass], a1[kPass], S1[kPass], dt[kPass], th[kPass];
          bool ser_all = true, dir_all = true;
#pragma unroll
          for (int u = 0; u < kPass; u++) {
            const LineVals<T> v = S.lv[lsl[u]][n + 1];
            const T ph = profile(w[u], vl1, rl, rl);
            j1[u] = fmadd(v.jf, ph, v.jd);
            a1[u] = fmadd(v.af, ph, v.ad);
            S1[u] = a1[u] > (T)0 ? j1[u] * Math<T>::rcp(a1[u]) : (T)0;
            dt[u] = (a0[u] + a1[u]) * hds;
            th[u] = (j0[u] + j1[u]) * hds;
            const bool ser = dt[u] < (T)0.25;
            ser_all = ser_all && ser;
            dir_all = dir_all && !ser;
          }
          ser_all = __all_sync(0xffffffffu, ser_all);
          dir_all = __all_sync(0xffffffffu, dir_all);
          T x[kPass], ca[kPass], cb[kPass];
          if (ser_all) {
#pragma unroll
            for (int u = 0; u < kPass; u++) Math<T>::series(dt[u], x[u], ca[u], cb[u]);
          } else if (dir_all) {
#pragma unroll
            for (int u = 0; u < kPass; u++) Math<T>::direct(dt[u], x[u], ca[u], cb[u]);
          } else {
#pragma unroll
            for (int u = 0; u < kPass; u++) Math<T>::coeffs(dt[u], x[u], ca[u], cb[u]);
          }
#pragma unroll
          for (int u = 0; u < kPass; u++) {
            const T src1 = a0[u] > (T)0 ? S0[u] : S1[u];
            const T src2 = a1[u] > (T)0 ? S1[u] : S0[u];
            T qv = dt[u] > (T)1.0e-9f ? fmadd(ca[u], src1, cb[u] * src2) : th[u];
            if constexpr (CHK) over += (!ov[u] && Ls[u] >= 0 && qv > (T)2 * th[u]) ? 1 : 0;
            qv = qv < th[u] ? qv : th[u];
            if (!ov[u]) {
              I[u] = fmadd(I[u], x[u], qv);
              j0[u] = j1[u]; a0[u] = a1[u]; S0[u] = S1[u];
              if constexpr (kTau) add_tau(u, dt[u]);
            }
          }
          if (any) {
            // compact the refined channels over the warp, refine them one per lane
            int pos[kPass];
            int cnt = 0;
#pragma unroll
            for (int u = 0; u < kPass; u++) {
              const unsigned m = __ballot_sync(0xffffffffu, ov[u]);
              pos[u] = cnt + __popc(m & lanemask_lt());
              if (ov[u]) {
                SW.I[pos[u]] = I[u]; SW.j0[pos[u]] = j0[u]; SW.a0[pos[u]] = a0[u]; SW.S0[pos[u]] = S0[u];
                SW.w[pos[u]] = w[u]; SW.l[pos[u]] = (unsigned char)lsl[u];
              }
              cnt += __popc(m);
            }
            __syncwarp();
            const T vl0 = S.vl[n], dsf = S.ds[n + 1], dvsg = S.dvs[n + 1];
            unsigned mysub = 0;
            for (int p = lane; p < cnt; p += 32) {
              const T wp = SW.w[p];
              const int lp = SW.l[p];
              const T s_c = sizeof(T) == 8 ? dsf * (wp - vl0) / dvsg : dsf * (wp - vl0) * G.idvs;
              const SlotOutT<T, kTau, CHK> o = slot_sub<T, kTau, CHK>(wp, S.lv[lp][n], S.lv[lp][n + 1], vl0, vl1, rl, dsf, G.ids,
                                                        s_c - G.hw3, G.lg, G.ilg, SW.I[p], SW.j0[p], SW.a0[p], SW.S0[p]);
              SW.I[p] = o.I; SW.j0[p] = o.j0; SW.a0[p] = o.a0; SW.S0[p] = o.S0;
              if constexpr (kTau) SW.w[p] = o.dtau;   // the owner keeps w in a register
              steps += o.steps - 1;
              mysub += o.steps;
              if constexpr (CHK) over += o.over;
            }
            // refinement statistics in shared memory (this path is rare; registers are not)
            mysub = __reduce_add_sync(0xffffffffu, mysub);
            if (lane == 0) { SW.rstat[0] += 1; SW.rstat[1] += mysub; SW.rstat[2] += cnt; }
            __syncwarp();
#pragma unroll
            for (int u = 0; u < kPass; u++) {
              if (ov[u]) {
                I[u] = SW.I[pos[u]]; j0[u] = SW.j0[pos[u]]; a0[u] = SW.a0[pos[u]]; S0[u] = SW.S0[pos[u]];
                if constexpr (kTau) add_tau(u, SW.w[pos[u]]);
              }
            }
            __syncwarp();
          }
        } else {
          const bool init = true, sub = fl & kFlagSub;
          const T vl0 = S.vl[n], dsf = S.ds[n + 1], dvs = S.dvs[n + 1];
          const SegGeom<T> G = seg_geom<T>(dsf, dvs, rl, P.kq);
#pragma unroll
          for (int u = 0; u < kPass; u++) {
            if (Ls[u] < 0) continue;
            const SlotOutT<T, kTau, CHK> o = slot_slow<T, kTau, CHK>(init, sub, w[u], S.lv[Ls[u]][n], S.lv[Ls[u]][n + 1], vl0, vl1,
                                                       rl, hds, G.q, dsf, dvs, G.ids, I[u], j0[u], a0[u], S0[u]);
            I[u] = o.I; j0[u] = o.j0; a0[u] = o.a0; S0[u] = o.S0; steps += o.steps - 1;
            if constexpr (kTau) add_tau(u, o.dtau);
            if constexpr (CHK) over += o.over;
          }
        }
        if (P.maser) {
          // masing check of charintline (telescope.F:4291-4297): the line opacity at the
          // segment end (the next step's alpl0) times the segment length. Warp-uniform:
          // only launches holding a line with a population inversion take it. (Packed
          // steps have no inverted line, so they cannot meet it.)
          const T dsm = S.ds[n + 1];
#pragma unroll
          for (int u = 0; u < kPass; u++)
            if (Ls[u] >= 0 && S.lv[Ls[u]][n + 1].af * profile(w[u], vl1, rl, rl) * dsm < (T)-0.01) mbits |= 1u << Ls[u];
        }
      }
#pragma unroll
      for (int u = 0; u < kPass; u++) {
        const int j = kPass * pq + u;
        if (j < C) { SS.I[j][lane] = I[u]; SS.j0[j][lane] = j0[u]; SS.a0[j][lane] = a0[u]; SS.S0[j][lane] = S0[u]; }
        if constexpr (kTauReg) {
          kahan_add(tauR[u], tcpR[u], part[u]);
        } else if constexpr (kTau) {
          if constexpr (!PV) kahan_add(tau[u], tcp[u], part[u]);
          if (Ls[u] >= 0) { P.tau[ta[u]] = tau[u]; P.tauc[ta[u]] = tcp[u]; }
        }
      }
    }
    __syncwarp();
  }
  if constexpr (kTauReg) {
#pragma unroll
    for (int u = 0; u < kPass; u++) {
      const int idx = u * 32 + lane;
      if (u < C && idx < nt) {
        const unsigned e = list[idx];
        const size_t a = ((size_t)(l0 + (int)(e >> kChBits) - lbase) * nb.nrays + ray) * P.nfr + (e & (kMaxChannels - 1));
        P.tau[a] = tauR[u]; P.tauc[a] = tcpR[u];
      }
    }
  }
  if (P.maser) {
    mbits = __reduce_or_sync(0xffffffffu, mbits);
    if (lane == 0)
      for (; mbits; mbits &= mbits - 1) atomicExch(&P.maser[l0 + __ffs(mbits) - 1], 1);
  }
  if constexpr (CHK) over = __reduce_add_sync(0xffffffffu, over);
  if (lane == 0) {
    SW.ctr[2] += passes;
    SW.ctr[3] += kFast ? passes - general - emptyp : 0u;
    SW.ctr[4] += skipped;
    if constexpr (CHK) SW.ctr[5] += (unsigned)over;
  }
  steps_total += steps;
  return steps;
}

// One work item: line group g of ray `ray`, item = g * nrays + ray.
template <typename T, int C, bool PV = false, bool TAU = false, bool CHK = false>
__device__ __forceinline__ void walk_item(const WalkParams<T>& P, int item, WarpStage<T>& S, SlotState<T, C>& SS,
                                          SubWork<T>& SW, unsigned short* list, int lane,
                                          unsigned long long& steps) {
  const NodeBuf<T>& nb = P.nb;
  const int nl = P.nlines;
  const int g = item / nb.nrays, ray = item - g * nb.nrays;
  const int l0 = g * P.gsize, gl = min(P.gsize, nl - l0);
  const int K = nb.nnodes[ray];
  if (nb.status[ray] != 0 || K < 1) {
    if (lane == 0) atomicCAS(P.err, 0, 100 + nb.status[ray]);
    return;
  }
  const size_t row = (size_t)ray * nb.kmax;
  // 1. velocity window of the ray per line (telescope.F:4265-4270): node projected
  //    velocities where N_up + N_low exceeds 1e-3, nodes 0 .. K-2; lines in batches of
  //    kGroup
  for (int lb = 0; lb < gl; lb += kGroup) {
    float mn[kGroup], mx[kGroup];
#pragma unroll
    for (int l = 0; l < kGroup; l++) { mn[l] = 1.0f; mx[l] = -1.0f; }
    if (!PV && ray != 0) {
      for (int k = lane; k < K - 1; k += 32) {
        const size_t o = row + k;
        const T wr = nb.wr[o], wt = nb.wt[o];
        const Corners c = corners(nb.c00[o], nb.misc[o], P.nth);
        const float d = nb.dvf[o];
#pragma unroll
        for (int l = 0; l < kGroup; l++) {
          if (lb + l < gl && interp_1(P.nsum, c, nl, l0 + lb + l, wr, wt) > (T)1.0e-3) {
            mn[l] = fminf(mn[l], d); mx[l] = fmaxf(mx[l], d);
          }
        }
      }
#pragma unroll
      for (int l = 0; l < kGroup; l++) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          mn[l] = fminf(mn[l], __shfl_xor_sync(0xffffffffu, mn[l], off));
          mx[l] = fmaxf(mx[l], __shfl_xor_sync(0xffffffffu, mx[l], off));
        }
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int l = 0; l < kGroup; l++)
        if (lb + l < gl) { S.mn[lb + l] = mn[l]; S.mx[lb + l] = mx[l]; }
    }
  }
  __syncwarp();
  // 2. (line, channel) pairs to integrate: channel 1, the in-window channels and the
  //    channel that supplies the continuum of the others (telescope.F:541-613)
  int nint = 0;
  for (int l = 0; l < gl; l++) {
    if (lane == 0) S.lineoff[l] = nint;
    int cc = -1;
    const double* velo = P.velo + (size_t)(l0 + l) * P.nfr;
    const double lo = (double)S.mn[l] - 2.0 * P.aksmax_c, hi = (double)S.mx[l] + 2.0 * P.aksmax_c;
    if (!PV && ray != 0 && !(velo[0] <= hi && velo[0] >= lo)) cc = 0;
    for (int cb = 0; cb < P.nfr; cb += 32) {
      const int c = cb + lane;
      const bool valid = c < P.nfr;
      const bool in = valid && (PV || ray == 0 || (velo[c] <= hi && velo[c] >= lo));
      if (!PV && cc < 0 && ray != 0) {
        const unsigned outm = __ballot_sync(0xffffffffu, valid && !in && c >= 1);
        if (outm) cc = cb + __ffs(outm) - 1;
      }
      const bool take = valid && (c == 0 || in || c == cc);
      // integration mask of the circular-image file (imcir_cmask, telescope.F:548,575):
      // channel 1 and the window channels
      if (!PV && P.mask != nullptr && valid)
        P.mask[((size_t)(l0 + l) * nb.nrays + ray) * P.nfr + c] = (unsigned char)(c == 0 || in);
      const unsigned m = __ballot_sync(0xffffffffu, take);
      if (take) list[nint + __popc(m & lanemask_lt())] = (unsigned short)((l << kChBits) | c);
      nint += __popc(m);
    }
    if (lane == 0) S.cont_ch[l] = cc;
  }
  if (lane == 0) S.lineoff[gl] = nint;
  __syncwarp();
  // 3. formal solution of the selected pairs in tiles of at most 32*C pairs spanning at
  //    most kGroup lines: consecutive lines share a tile, so that the tiles' slots fill up
  for (int tb = 0; tb < nint;) {
    const int la = (int)(list[tb] >> kChBits);
    const int lcap = min(la + kGroup, gl);
    const int te = min(tb + 32 * C, S.lineoff[lcap]);
    const int nt = te - tb;
    const int lz = (int)(list[te - 1] >> kChBits);
    walk_ray<T, C, PV, TAU, CHK>(P, S, SS, SW, ray, K, l0 + la, lz - la + 1, list + tb, nt, lane, la, steps);
    for (int j = 0; j < C; j++) {
      const int idx = j * 32 + lane;
      if (idx < nt) {
        const unsigned e = list[tb + idx];
        const int l = (int)(e >> kChBits), c = (int)(e & (kMaxChannels - 1));
        const T Iv = SS.I[j][lane];
        P.img[((size_t)(l0 + l) * nb.nrays + ray) * P.nfr + c] = Iv;
        if (c == S.cont_ch[l]) S.contv[l] = Iv;
      }
    }
    __syncwarp();
    tb = te;
  }
  if (lane == 0) { SW.ctr[0] += nint; SW.ctr[1] += (unsigned long long)nint * K; }
  __syncwarp();
  // 4. continuum copy for the other channels of each line
  for (int l = 0; l < gl; l++) {
    const int cc = S.cont_ch[l];
    if (cc < 0) continue;
    const double* velo = P.velo + (size_t)(l0 + l) * P.nfr;
    const double lo = (double)S.mn[l] - 2.0 * P.aksmax_c, hi = (double)S.mx[l] + 2.0 * P.aksmax_c;
    T* img = P.img + ((size_t)(l0 + l) * nb.nrays + ray) * P.nfr;
    const T contv = S.contv[l];
    if (contv != (T)0) {
      for (int c = lane; c < P.nfr; c += 32) {
        const bool in = velo[c] <= hi && velo[c] >= lo;
        if (!(c == 0 || in || c == cc)) img[c] = contv;
      }
      continue;
    }
    // a zero continuum is recomputed channel by channel in the reference: integrate
    // every other out-of-window channel, then apply its sequential copy rule
    int n2 = 0;
    for (int cb = 0; cb < P.nfr; cb += 32) {
      const int c = cb + lane;
      const bool valid = c < P.nfr;
      const bool take = valid && !(c == 0 || (velo[c] <= hi && velo[c] >= lo) || c == cc);
      const unsigned m = __ballot_sync(0xffffffffu, take);
      if (take) list[n2 + __popc(m & lanemask_lt())] = (unsigned short)((l << kChBits) | c);
      n2 += __popc(m);
    }
    __syncwarp();
    for (int tb = 0; tb < n2; tb += 32 * C) {
      const int nt = min(32 * C, n2 - tb);
      walk_ray<T, C, false, false, CHK>(P, S, SS, SW, ray, K, l0 + l, 1, list + tb, nt, lane, l, steps);
      for (int j = 0; j < C; j++) {
        const int idx = j * 32 + lane;
        if (idx < nt) img[list[tb + idx] & (kMaxChannels - 1)] = SS.I[j][lane];
      }
    }
    if (lane == 0) { SW.ctr[0] += n2; SW.ctr[1] += (unsigned long long)n2 * K; }
    __syncwarp();
    if (lane == 0) {
      T cur = 0;
      bool have = false;
      for (int c = 0; c < P.nfr; c++) {
        const bool in = velo[c] <= hi && velo[c] >= lo;
        if (c != cc && (c == 0 || in)) continue;
        if (have) img[c] = cur;
        else if (img[c] != (T)0) { cur = img[c]; have = true; }
      }
    }
    __syncwarp();
  }
  __syncwarp();
}

// Per-warp regions of the walk: stage, slot state and SUBGRID work in shared memory;
// the (line, channel) list of the item in a per-warp global scratch row (L1-cached) when
// kListInSmem is false, which leaves room for four 4-warp blocks per SM. `listcap`
// (pairs) is kGroup x the largest channel count of the launch.
constexpr bool kListInSmem = false;
// FP32: four blocks per SM (at most 128 registers); FP64 (the parity path) keeps its registers.
template <typename T> struct WalkMinBlocks { static constexpr int value = sizeof(T) == 4 ? kWalkBlocksPerSm : 1; };

template <typename T, int C>
struct WarpSmem {
  WarpStage<T>* S; SlotState<T, C>* SS; SubWork<T>* SW; unsigned short* list;
  __device__ WarpSmem(unsigned char* raw, int nw, int wib, int listcap, unsigned short* gscratch) {
    const int capp = (listcap + 7) & ~7;
    S = reinterpret_cast<WarpStage<T>*>(raw) + wib;
    SS = reinterpret_cast<SlotState<T, C>*>(raw + sizeof(WarpStage<T>) * nw) + wib;
    SW = reinterpret_cast<SubWork<T>*>(raw + (sizeof(WarpStage<T>) + sizeof(SlotState<T, C>)) * nw) + wib;
    if (kListInSmem)
      list = reinterpret_cast<unsigned short*>(
                 raw + (sizeof(WarpStage<T>) + sizeof(SlotState<T, C>) + sizeof(SubWork<T>)) * nw) +
             (size_t)wib * capp;
    else
      list = gscratch + ((size_t)blockIdx.x * nw + wib) * capp;
  }
};

// counters[0] formal-solution steps, [1] integrated (line, channel) pairs, [2] node visits
// (pairs x nodes), [3] node passes of the walk (a pass = the tile's slots over one node),
// [4] of them taken on the packed FP32 path, [5] steps of empty segments (counted in [0],
// no arithmetic), [6] node passes with SUBGRID refinement, [7] the sub-steps of the refined
// channels, [8] the refined channels of those passes, [9] steps that failed the overshoot
// test (checking walks only). The buffers hold kWalkCounters values.
template <typename T>
__device__ __forceinline__ void flush_counters(unsigned long long steps, const SubWork<T>& SW,
                                               unsigned long long* counters, int lane) {
  __syncwarp();
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) steps += __shfl_xor_sync(0xffffffffu, steps, off);   // per lane
  if (lane == 0) {
    atomicAdd(&counters[0], steps);
#pragma unroll
    for (int i = 0; i < 5; i++) atomicAdd(&counters[1 + i], SW.ctr[i]);
    atomicAdd(&counters[6], (unsigned long long)SW.rstat[0]);
    atomicAdd(&counters[7], (unsigned long long)SW.rstat[1]);
    atomicAdd(&counters[8], (unsigned long long)SW.rstat[2]);
    atomicAdd(&counters[9], SW.ctr[5]);
  }
}

}  // namespace rl
