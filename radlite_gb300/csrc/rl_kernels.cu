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
#include "rl_walk_common.cuh"

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
  // The FP32 build stores every node value in FP32, so it forms the direction, the
  // projected velocity, the interpolation weights and the width in FP32 from the FP64
  // positions and cell differences; the FP64 build does all of it in FP64.
  static constexpr bool kFp32Direction = sizeof(T) == 4;
  const GeoParams* p;
  const rlg::Grid* g;
  NodeBuf<T>* nb;
  TrajDebug* dbg;
  size_t row;
  int k, status;
  int ir_prev, icr_prev;
  double s_prev, dvmu_prev;
  float dvmu_prev_f;

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
    const float dr = (float)(n.r - R0) / (float)(R1 - R0);
    const float dt = (float)(n.th - T0) / (float)(T1 - T0);
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
    float v[3];
    for (int i = 0; i < 3; i++)
      v[i] = bil(p->velf[3 * c00 + i], p->velf[3 * c01 + i], p->velf[3 * c10 + i], p->velf[3 * c11 + i]);
    const float lwv = bil(p->lwf[c00], p->lwf[c01], p->lwf[c10], p->lwf[c11]);
    const float tang = RL_FMA(v[1], n.sinphi_f, RL_MUL(v[2], n.cosphi_f));
    const float dvmu = RL_MUL(3.335668e-11f, RL_FMA(n.mu_f, v[0], RL_MUL(n.sinmu_f, tang)));
    const float kv = (float)(1.0 / 3.33567e-6);
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
    nb->dvf[o] = dvmu;
    nb->vl[o] = (T)RL_MUL(dvmu, kv);
    nb->dvseg[o] = (T)(k > 0 ? RL_MUL(RL_SUB(dvmu, dvmu_prev_f), kv) : 0.0f);
    nb->lw[o] = (T)lwv;
    nb->wr[o] = (T)dr;
    nb->wt[o] = (T)dt;
    nb->c00[o] = c00;
    nb->misc[o] = (unsigned)(dto + 32768) | ((unsigned)(dro + 1) << 16) | ((unsigned)n.icr << kIcrShift) | flags;
    s_prev = n.s; dvmu_prev_f = dvmu; ir_prev = n.ir; icr_prev = n.icr;
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
  em.dvmu_prev_f = 0.0f;
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

// Formal solution of the (line, channel) pairs list[0..nt) of lines l0.. of one ray.
// The per-line tables carry the profile normalisation 0.56419583546/(3.33567e-6 nu0), so
// the profile of every slot is rlw * exp(-u^2) with the node's shared 1/linewidth.
// Work order: per 32-node chunk, per pair of slots (two independent channels per lane),
// all nodes of the chunk; the slot state lives in shared memory between pairs.
template <typename T, int C>
__device__ long long walk_ray(const WalkParams<T>& P, WarpStage<T>& S, SlotState<T, C>& SS, SubWork<T>& SW, int ray,
                              int K, int l0, int gl, const unsigned short* list, int nt, int lane) {
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
      L = (int)(e >> kChBits);
      w = P.wch[(size_t)(l0 + L) * P.nfr + (e & (kMaxChannels - 1))];
      I = P.lc[l0 + L].istart;
    }
    SS.ll[j][lane] = L; SS.w[j][lane] = w; SS.I[j][lane] = I;
    SS.j0[j][lane] = 0; SS.a0[j][lane] = 0; SS.S0[j][lane] = 0;
  }
  // central beam: the node where the ray first reaches the innermost cell mixes in the
  // star (telescope.F:4166-4191)
  int star_node = -1;
  if (ray == 0) {
    for (int kb = 0; kb < K && star_node < 0; kb += 32) {
      const int k = kb + lane;
      const bool f = k >= 1 && k < K && (nb.misc[row + k] & kFlagIr1);
      const unsigned m = __ballot_sync(0xffffffffu, f);
      if (m) star_node = kb + __ffs(m) - 1;
    }
  }
  long long steps = 0;
  T lw_last = 0;
  for (int kb = 0; kb < K; kb += 32) {
    if (kb > 0) {   // carry the last node of the previous chunk into entry 0
      if (lane == 0) {
        S.vl[0] = S.vl[32]; S.hds[0] = S.hds[32]; S.ds[0] = S.ds[32]; S.rlw[0] = S.rlw[32];
        S.q[0] = S.q[32]; S.ids[0] = S.ids[32]; S.dvs[0] = S.dvs[32]; S.flags[0] = S.flags[32];
        S.idvs[0] = S.idvs[32]; S.hw3[0] = S.hw3[32]; S.lg[0] = S.lg[32]; S.ilg[0] = S.ilg[32];
      }
      if (lane < gl) S.lv[lane][0] = S.lv[lane][32];
      __syncwarp();
    }
    const int k = kb + lane;
    T vl = 0, ds = 0, dvs = 0, lwk = 0;
    unsigned misc = 0;
    if (k < K) {
      const size_t o = row + k;
      const T wr = nb.wr[o], wt = nb.wt[o];
      misc = nb.misc[o];
      const Corners c = corners(nb.c00[o], misc, P.nth);
      for (int l = 0; l < gl; l++) S.lv[l][lane + 1] = interp_lv(P.tab, c, nl, l0 + l, wr, wt);
      vl = nb.vl[o]; ds = nb.ds[o]; dvs = nb.dvseg[o]; lwk = nb.lw[o];
    }
    T lwp = __shfl_up_sync(0xffffffffu, lwk, 1);
    if (lane == 0) lwp = lw_last;
    lw_last = __shfl_sync(0xffffffffu, lwk, 31);
    const T lwav = (T)0.5 * (lwp + lwk);
    const T rlw = lwav > (T)0 ? Math<T>::div((T)1, lwav) : (T)0;
    S.vl[lane + 1] = vl; S.hds[lane + 1] = (T)0.5 * ds; S.ds[lane + 1] = ds; S.rlw[lane + 1] = rlw;
    S.q[lane + 1] = (dvs < (T)0 ? -dvs : dvs) * P.kq * rlw;
    S.ids[lane + 1] = ds > (T)0 ? Math<T>::div((T)1, ds) : (T)0;
    S.dvs[lane + 1] = dvs;
    {
      // refined window half width 3 l = 3 ds/q and the spacing of its 31-point grid
      const T qv = S.q[lane + 1];
      const T dls = qv > (T)0 ? Math<T>::div(ds, qv) : (T)0;
      S.idvs[lane + 1] = dvs != (T)0 ? Math<T>::div((T)1, dvs) : (T)0;
      S.hw3[lane + 1] = (T)3 * dls;
      S.lg[lane + 1] = (T)6 * dls / (T)30;
      S.ilg[lane + 1] = dls > (T)0 ? Math<T>::div((T)30, (T)6 * dls) : (T)0;
    }
    {
      unsigned f = misc;
      if (k == 1 || (misc & kFlagHole) || k == star_node) f |= kFlagInit;
      if ((T)6 * S.q[lane + 1] > (T)1) f |= kFlagSub;
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
      for (int n = n0; n < nn; n++) {
        const int g = kb + n;
        const unsigned fl = S.flags[n + 1];
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
          if (fl & kFlagSub) {
            const T vl0 = S.vl[n], dsf = S.ds[n + 1], hw3 = S.hw3[n + 1];
#pragma unroll
            for (int u = 0; u < kPass; u++) {
              const T s_c = sizeof(T) == 8 ? dsf * (w[u] - vl0) / S.dvs[n + 1] : dsf * (w[u] - vl0) * S.idvs[n + 1];
              ov[u] = Ls[u] >= 0 && (s_c + hw3 > (T)0) && (s_c - hw3 < dsf);
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
            j1[u] = v.jd + v.jf * ph;
            a1[u] = v.ad + v.af * ph;
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
            T qv = dt[u] > (T)1.0e-9f ? ca[u] * src1 + cb[u] * src2 : th[u];
            qv = qv < th[u] ? qv : th[u];
            if (!ov[u]) {
              I[u] = I[u] * x[u] + qv;
              j0[u] = j1[u]; a0[u] = a1[u]; S0[u] = S1[u];
            }
          }
          steps += nv;
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
            const T vl0 = S.vl[n], dsf = S.ds[n + 1], ids = S.ids[n + 1], hw3 = S.hw3[n + 1];
            const T lgv = S.lg[n + 1], ilg = S.ilg[n + 1], idvs = S.idvs[n + 1], dvsg = S.dvs[n + 1];
            for (int p = lane; p < cnt; p += 32) {
              const T wp = SW.w[p];
              const int lp = SW.l[p];
              const T s_c = sizeof(T) == 8 ? dsf * (wp - vl0) / dvsg : dsf * (wp - vl0) * idvs;
              const SlotOutT<T> o = slot_sub<T>(wp, S.lv[lp][n], S.lv[lp][n + 1], vl0, vl1, rl, dsf, ids, s_c - hw3,
                                                lgv, ilg, SW.I[p], SW.j0[p], SW.a0[p], SW.S0[p]);
              SW.I[p] = o.I; SW.j0[p] = o.j0; SW.a0[p] = o.a0; SW.S0[p] = o.S0;
              steps += o.steps - 1;
            }
            __syncwarp();
#pragma unroll
            for (int u = 0; u < kPass; u++) {
              if (ov[u]) { I[u] = SW.I[pos[u]]; j0[u] = SW.j0[pos[u]]; a0[u] = SW.a0[pos[u]]; S0[u] = SW.S0[pos[u]]; }
            }
            __syncwarp();
          }
        } else {
          const bool init = true, sub = fl & kFlagSub;
          const T vl0 = S.vl[n], q = S.q[n + 1], dsf = S.ds[n + 1], dvs = S.dvs[n + 1], ids = S.ids[n + 1];
#pragma unroll
          for (int u = 0; u < kPass; u++) {
            if (Ls[u] < 0) continue;
            const SlotOutT<T> o = slot_slow<T>(init, sub, w[u], S.lv[Ls[u]][n], S.lv[Ls[u]][n + 1], vl0, vl1, rl, hds,
                                               q, dsf, dvs, ids, I[u], j0[u], a0[u], S0[u]);
            I[u] = o.I; j0[u] = o.j0; a0[u] = o.a0; S0[u] = o.S0; steps += o.steps;
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kPass; u++) {
        const int j = kPass * pq + u;
        if (j < C) { SS.I[j][lane] = I[u]; SS.j0[j][lane] = j0[u]; SS.a0[j][lane] = a0[u]; SS.S0[j][lane] = S0[u]; }
      }
    }
    __syncwarp();
  }
  return steps;
}

struct WalkCounters { unsigned long long steps = 0, integ = 0, nodes = 0; };

// One work item: line group g of ray `ray`, item = g * nrays + ray.
template <typename T, int C>
__device__ __forceinline__ void walk_item(const WalkParams<T>& P, int item, WarpStage<T>& S, SlotState<T, C>& SS,
                                          SubWork<T>& SW, unsigned short* list, int lane, WalkCounters& wc) {
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
  //    velocities where N_up + N_low exceeds 1e-3, nodes 0 .. K-2
  float mn[kGroup], mx[kGroup];
#pragma unroll
  for (int l = 0; l < kGroup; l++) { mn[l] = 1.0f; mx[l] = -1.0f; }
  __syncwarp();
  if (ray != 0) {
    for (int k = lane; k < K - 1; k += 32) {
      const size_t o = row + k;
      const T wr = nb.wr[o], wt = nb.wt[o];
      const Corners c = corners(nb.c00[o], nb.misc[o], P.nth);
      const float d = nb.dvf[o];
#pragma unroll
      for (int l = 0; l < kGroup; l++) {
        if (l < gl && interp_1(P.nsum, c, nl, l0 + l, wr, wt) > (T)1.0e-3) {
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
    for (int l = 0; l < kGroup; l++) { S.mn[l] = mn[l]; S.mx[l] = mx[l]; }
  }
  __syncwarp();
  // 2. (line, channel) pairs to integrate: channel 1, the in-window channels and the
  //    channel that supplies the continuum of the others (telescope.F:541-613)
  int nint = 0;
  for (int l = 0; l < gl; l++) {
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
    if (lane == 0) S.cont_ch[l] = cc;
  }
  __syncwarp();
  // 3. formal solution of the selected pairs, in tiles of 32*C
  for (int tb = 0; tb < nint; tb += 32 * C) {
    const int nt = min(32 * C, nint - tb);
    wc.steps += walk_ray<T, C>(P, S, SS, SW, ray, K, l0, gl, list + tb, nt, lane);
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
  }
  wc.integ += nint;
  wc.nodes += (unsigned long long)nint * K;
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
      wc.steps += walk_ray<T, C>(P, S, SS, SW, ray, K, l0, gl, list + tb, nt, lane);
      for (int j = 0; j < C; j++) {
        const int idx = j * 32 + lane;
        if (idx < nt) img[list[tb + idx] & (kMaxChannels - 1)] = SS.I[j][lane];
      }
    }
    wc.integ += n2;
    wc.nodes += (unsigned long long)n2 * K;
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

__device__ __forceinline__ void flush_counters(WalkCounters wc, unsigned long long* counters, int lane) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) wc.steps += __shfl_xor_sync(0xffffffffu, wc.steps, off);
  if (lane == 0) {
    atomicAdd(&counters[0], wc.steps);
    atomicAdd(&counters[1], wc.integ);
    atomicAdd(&counters[2], wc.nodes);
  }
}

template <typename T, int C>
__global__ void __launch_bounds__(128, WalkMinBlocks<T>::value) k_walk(WalkParams<T> P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  WarpSmem<T, C> W(smem_raw, nw, wib, kGroup * P.nfr, P.list);
  WalkCounters wc;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(P.work, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= P.nitems) break;
    walk_item<T, C>(P, item, *W.S, *W.SS, *W.SW, W.list, lane, wc);
  }
  flush_counters(wc, P.counters, lane);
}

// Walk of many jobs (model, camera, line range) from one device queue: queue entry i
// is item i * stride of the concatenated item list (stride > 1 samples it for tuning);
// item_prefix[j] is the first item of job j. Each warp keeps the parameters of its
// current job in shared memory.
template <typename T, int C>
__global__ void __launch_bounds__(128, WalkMinBlocks<T>::value) k_walk_jobs(WalkJobs<T> B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ WalkParams<T> jp[4];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  WarpSmem<T, C> W(smem_raw, nw, wib, kGroup * B.max_nfr, B.list);
  WalkCounters wc;
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
    walk_item<T, C>(jp[wib], item - __ldg(&B.item_prefix[j]), *W.S, *W.SS, *W.SW, W.list, lane, wc);
  }
  flush_counters(wc, B.counters, lane);
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

template <typename T, int C>
static cudaError_t launch_walk_c(const WalkParams<T>& P, int nsm, cudaStream_t s) {
  const int warps = 4, threads = warps * 32;
  const int capp = (kGroup * P.nfr + 7) & ~7;
  const size_t smem = (sizeof(WarpStage<T>) + sizeof(SlotState<T, C>) + sizeof(SubWork<T>)) * warps +
                      (kListInSmem ? sizeof(unsigned short) * (size_t)capp * warps : 0);
  cudaError_t e = cudaFuncSetAttribute(k_walk<T, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk<T, C>, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (per_sm > kWalkBlocksPerSm) per_sm = kWalkBlocksPerSm;   // the list scratch holds this many
  long long blocks = (long long)nsm * per_sm;
  const long long need = ((long long)P.nitems + warps - 1) / warps;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  k_walk<T, C><<<(unsigned)blocks, threads, smem, s>>>(P);
  return cudaGetLastError();
}

template <typename T, int C>
static cudaError_t launch_walk_jobs_c(const WalkJobs<T>& B, int nsm, cudaStream_t s) {
  const int warps = 4, threads = warps * 32;
  const int capp = (kGroup * B.max_nfr + 7) & ~7;
  const size_t smem = (sizeof(WarpStage<T>) + sizeof(SlotState<T, C>) + sizeof(SubWork<T>)) * warps +
                      (kListInSmem ? sizeof(unsigned short) * (size_t)capp * warps : 0);
  cudaError_t e = cudaFuncSetAttribute(k_walk_jobs<T, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_jobs<T, C>, threads, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  if (per_sm > kWalkBlocksPerSm) per_sm = kWalkBlocksPerSm;
  long long blocks = (long long)nsm * per_sm;
  const long long nq = ((long long)B.total + B.stride - 1) / B.stride;
  const long long need = (nq + warps - 1) / warps;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  k_walk_jobs<T, C><<<(unsigned)blocks, threads, smem, s>>>(B);
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

template <typename T>
cudaError_t launch_jobs(const JobLaunch<T>& L, cudaStream_t s) {
  if (L.nrays_total > 0) {
    k_geometry_jobs<T><<<(L.nrays_total + 127) / 128, 128, 0, s>>>(L.geo, L.ray_prefix, L.njobs, L.nrays_total);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = cudaMemsetAsync(L.walk.work, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  switch (L.cpl) {
    case 1: e = launch_walk_jobs_c<T, 1>(L.walk, L.nsm, s); break;
    case 2: e = launch_walk_jobs_c<T, 2>(L.walk, L.nsm, s); break;
    case 4: e = launch_walk_jobs_c<T, 4>(L.walk, L.nsm, s); break;
    default: e = launch_walk_jobs_c<T, 8>(L.walk, L.nsm, s); break;
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
template cudaError_t launch_walk<float>(const WalkParams<float>&, int, int, cudaStream_t);
template cudaError_t launch_walk<double>(const WalkParams<double>&, int, int, cudaStream_t);
template cudaError_t launch_reduce<float>(const ReduceParams&, const float*, double*, double*, cudaStream_t);
template cudaError_t launch_reduce<double>(const ReduceParams&, const double*, double*, double*, cudaStream_t);
template cudaError_t launch_jobs<float>(const JobLaunch<float>&, cudaStream_t);
template cudaError_t launch_jobs<double>(const JobLaunch<double>&, cudaStream_t);

}  // namespace rl
