// rl_geometry.cuh -- FP64 ray/grid crossing geometry for one circular-image ray.
//
// Produces, in order along the ray, the crossings of the photon path with the R=const
// spheres and theta=const cones of the axisymmetric grid plus the extra points placed
// around the r- and theta-extrema, with the reference's selection filters and local
// direction (mu, phi). Semantics follow make_trajectory_c (RADLITE/telescope.F:2787-3720):
//   theta crossings  telescope.F:2959-3226   r crossings    telescope.F:3256-3345
//   extra points     telescope.F:3417-3603   merge/filters  telescope.F:3356-3363,3607-3677
//   mu, phi          telescope.F:3687-3718
// The crossing lists are not stored: each list element is regenerated from its index,
// because both lists have closed-form orderings (the theta-crossing set is a contiguous
// run of cone indices, since the discriminant grows monotonically with tan^2(theta)).
// Only the <= 34 extra points are kept per ray.
//
// All arithmetic is double precision: the crossing quadratics cancel near tangent points.
#pragma once
#include <math.h>

#ifndef RL_HD
#if defined(__CUDACC__)
#define RL_HD __host__ __device__ __forceinline__
#else
#define RL_HD inline
#endif
#endif

namespace rlg {

constexpr double kPi = 3.1415926535897932385;
constexpr double kTelEps = 1.0e-10;
constexpr int kExtraMax = 34;       // 1 + 4*4 around each extremum
constexpr int kAdPts = 4;           // points per sub-interval around an extremum

// Status codes written per ray (0 = fine).
enum GeoStatus : int {
  kGeoOk = 0,
  kGeoOutside = 1,          // trajectory misses the grid (no R > impact parameter)
  kGeoNegDiscr = 2,         // negative discriminant of an R crossing
  kGeoThetaNonContig = 3,   // theta-crossing set not contiguous (not expected)
  kGeoHuntFail = 4,         // theta extremum outside the radial grid index range
  kGeoOrder = 5,            // extra points around theta extremum out of order
  kGeoOverflow = 6,         // more nodes than the buffer row holds
  kGeoRange = 7,            // interpolation weight outside [0,1]
  kGeoStarStart = 8,        // ray would start on the stellar surface (not supported)
  kGeoMu = 9,               // |mu| > 1
};

struct Grid {
  const double* R;      // R(ix) = R[ix + 1], ix = -1 .. nr+2 (ghost nodes included)
  const double* TH;     // TH(iy) = TH[iy + 1], iy = -1 .. ny+2
  const double* tan2;   // tan(TH(iy))^2 for iy = 1 .. nth (index 0 unused)
  int nr, nth, ny;      // ny = 2*nth (mirrored about the equator)
  double rstar;
};

RL_HD double Rg(const Grid& g, int ix) { return g.R[ix + 1]; }
RL_HD double Tg(const Grid& g, int iy) { return g.TH[iy + 1]; }

// Bracketing search of x in the monotonic table xx(1..n) (1-based via acc()) from the guess
// g, with the index rules of RADLite's hunt (nrecip.F:157-197), stated here:
//   past(j):   x >= xx(j) in an ascending table (xx(n) > xx(1)), x < xx(j) otherwise
//   before(j): the opposite comparison, x < xx(j) ascending, x >= xx(j) otherwise
//   beyond(j): x > xx(j) ascending, x <= xx(j) otherwise
// 1. Bracket [L, H]. A guess outside 1..n gives L = 0, H = n + 1. Otherwise nodes are
//    probed at distances 1, 3, 7, 15, ... (2^i - 1) from g: if past(g), upwards while the
//    probe is <= n and past(probe) (L = the last node passed, g at least; H = the first
//    probe that is not, n + 1 past the end); else downwards while the probe is >= 1 and
//    before(probe) (H = the last such probe, g at least; L = the first probe that is not,
//    0 past the start).
// 2. Result: L plus the number of nodes strictly inside the bracket that x lies beyond; in
//    a monotonic table they come first, so a binary search counts them.
// So x equal to a node value xx(k) gives k when the bracket stopped on k (k = L), and k - 1
// when k lies strictly inside the bracket: r-crossings land exactly on nodes, and which
// cell they are assigned to follows these rules.
template <class Acc>
RL_HD int hunt(const Acc& acc, int n, double x, int g) {
  const bool asc = acc(n) > acc(1);
  int L = 0, H = n + 1;
  if (g >= 1 && g <= n) {
    if (asc ? x >= acc(g) : x < acc(g)) {
      L = g;
      for (int d = 1; ; d = 2 * d + 1) {
        const int p = g + d;
        if (p > n) break;
        if (!(asc ? x >= acc(p) : x < acc(p))) { H = p; break; }
        L = p;
      }
    } else {
      H = g;
      for (int d = 1; ; d = 2 * d + 1) {
        const int p = g - d;
        if (p < 1) break;
        if (!(asc ? x < acc(p) : x >= acc(p))) { L = p; break; }
        H = p;
      }
    }
  }
  int first = L + 1, count = H - L - 1;   // candidates L+1 .. H-1
  while (count > 0) {
    const int half = count >> 1;
    if (asc ? x > acc(first + half) : x <= acc(first + half)) {
      first += half + 1;
      count -= half + 1;
    } else {
      count = half;
    }
  }
  return first - 1;
}

struct RAcc { const Grid* g; RL_HD double operator()(int j) const { return Rg(*g, j); } };
struct TAcc { const Grid* g; RL_HD double operator()(int j) const { return Tg(*g, j); } };

struct Ray {
  double x0, z0, costh0, sinth0, costh02, sinth02, pitheta0, bimpact;
  double bnew, znew;                    // direction(): impact distance and offset in the ray plane
  float bnew_f, znew_f, costh0_f;       // FP32 copies for direction_ff (high parts)
  float bnew_l, znew_l, costh0_l;       //   and their low parts (x - (double)x_f)
  int iy0, isnr, isdblnr, caseA, iup;   // theta crossings
  int ir_min, ir_amount, ith_amount;    // r crossings
};

// One emitted node of the trajectory.
struct Node {
  double s, r, th, mu, sinmu, sinphi, cosphi;   // sinmu = sqrt(1 - mu^2)
  float mu_f, sinmu_f, sinphi_f, cosphi_f;      // the same from direction_ff (FP32 node values):
  float mu_l, sinmu_l, sinphi_l, cosphi_l;      //   high and low parts of a float-float value
  int icr, ir, it;
};

RL_HD double theta_at(const Ray& y, double s) {
  double t = atan(sqrt(y.x0 * y.x0 + y.sinth02 * s * s) / (y.z0 + y.costh0 * s));
  if (t < 0.0) t = t + kPi;
  return t;
}
RL_HD double radius_at(const Ray& y, double s) {
  return sqrt(y.x0 * y.x0 + y.z0 * y.z0 + s * s + 2.0 * y.z0 * y.costh0 * s);
}

RL_HD int init_ray(const Grid& g, double x0, double z0, double theta0, Ray& y) {
  y.x0 = x0; y.z0 = z0;
  y.pitheta0 = 0.5 * kPi - theta0;
  y.costh0 = cos(theta0); y.sinth0 = sin(theta0);
  y.costh02 = y.costh0 * y.costh0; y.sinth02 = y.sinth0 * y.sinth0;
  y.znew = z0 * y.sinth02;
  y.bnew = sqrt(x0 * x0 + z0 * z0 * y.sinth02);
  y.bnew_f = (float)y.bnew; y.znew_f = (float)y.znew; y.costh0_f = (float)y.costh0;
  y.bnew_l = (float)(y.bnew - (double)y.bnew_f);
  y.znew_l = (float)(y.znew - (double)y.znew_f);
  y.costh0_l = (float)(y.costh0 - (double)y.costh0_f);
  // theta=const cones with two crossings: contiguous suffix iy0..nth of the stored half
  int first = 0, count = 0;
  for (int iy = 1; iy <= g.nth; iy++) {
    const double tanth2 = g.tan2[iy];
    const double a = tanth2 * y.costh02 - y.sinth02;
    const double b = 2.0 * tanth2 * y.costh0 * z0;
    const double c = tanth2 * z0 * z0 - x0 * x0;
    const double sd = b * b - 4.0 * a * c;
    if (sd > 0.0) { if (count == 0) first = iy; count++; }
  }
  if (count > 0 && first + count - 1 != g.nth) return kGeoThetaNonContig;
  y.iy0 = first; y.isnr = count;
  int dbl = 0;
  for (int is = 1; is <= count; is++)
    if (fabs(0.5 * kPi - Tg(g, first + is - 1)) > fabs(y.pitheta0)) dbl++;
  y.isdblnr = dbl;
  y.iup = y.pitheta0 > 0.0 ? 1 : 0;
  y.caseA = (z0 * y.pitheta0 > 0.0) ? 1 : 0;
  y.ith_amount = 2 * count;
  // r crossings
  y.bimpact = sqrt(x0 * x0 + z0 * z0 * (1.0 - y.costh02));
  int ix = 1;
  for (; ix <= g.nr; ix++) if (Rg(g, ix) > y.bimpact) break;
  if (ix > g.nr) return kGeoOutside;
  y.ir_min = (y.bimpact <= g.rstar) ? 0 : ix;
  y.ir_amount = 2 * (g.nr + 1 - y.ir_min);
  return kGeoOk;
}

// Element iss (1-based) of the theta-crossing list: s and full-grid cone index.
RL_HD void th_elem(const Grid& g, const Ray& y, int iss, double& s, int& ith) {
  const int n = y.isnr, d = y.isdblnr;
  int is, root; bool flip;
  if (y.caseA) {
    if (iss <= n - d) { is = d + iss; root = 1; flip = y.iup; }
    else if (iss <= 2 * n - 2 * d) { is = 2 * n - d + 1 - iss; root = 2; flip = !y.iup; }
    else if (iss <= 2 * n - d) { is = d - (iss - (2 * n + 1 - 2 * d)); root = 1; flip = !y.iup; }
    else { is = 1 + (iss - (2 * n + 1 - d)); root = 2; flip = !y.iup; }
  } else {
    if (iss <= d) { is = d - (iss - 1); root = 1; flip = y.iup; }
    else if (iss <= 2 * d) { is = iss - d; root = 2; flip = y.iup; }
    else if (iss <= n + d) { is = iss - d; root = 1; flip = y.iup; }
    else { is = n - (iss - (n + d + 1)); root = 2; flip = !y.iup; }
  }
  const int iy = y.iy0 + is - 1;
  const double tanth2 = g.tan2[iy];
  const double a = tanth2 * y.costh02 - y.sinth02;
  const double b = 2.0 * tanth2 * y.costh0 * y.z0;
  const double c = tanth2 * y.z0 * y.z0 - y.x0 * y.x0;
  const double sd = sqrt(b * b - 4.0 * a * c);
  double s1 = (-b - sd) / (2.0 * a), s2 = (-b + sd) / (2.0 * a);
  if (s1 > s2) { const double t = s1; s1 = s2; s2 = t; }
  s = (root == 1) ? s1 : s2;
  ith = flip ? (g.ny + 1 - iy) : iy;
}
RL_HD double th_s_at(const Grid& g, const Ray& y, int iss) {
  if (iss < 1) return -1.0e30;
  if (iss > y.ith_amount) return 1.0e30;
  double s; int ith; th_elem(g, y, iss, s, ith); return s;
}

// Element isr (1-based) of the R-crossing list: s, radius and radial index.
RL_HD int r_elem(const Grid& g, const Ray& y, int isr, double& s, double& r, int& ix) {
  const int m = g.nr + 1 - y.ir_min;
  int root;
  if (isr <= m) { ix = g.nr - (isr - 1); root = 1; }
  else { ix = g.nr - (y.ir_amount - isr); root = 2; }
  r = (ix == 0) ? g.rstar : Rg(g, ix);
  const double a = 1.0, b = 2.0 * y.costh0 * y.z0;
  const double c = y.x0 * y.x0 + y.z0 * y.z0 - r * r;
  double sd = b * b - 4.0 * a * c + kTelEps * b * b;
  if (sd < 0.0) return kGeoNegDiscr;
  sd = sqrt(sd);
  s = (root == 1) ? (-b - sd) / (2.0 * a) : (-b + sd) / (2.0 * a);
  return kGeoOk;
}
// r_s(j) with the sentinels used by the extra-point intervals: -1e30 below the list,
// +1e30 above it (the reference reads an unset r_s(0) there; -1e30 drops those points).
RL_HD double r_s_at(const Grid& g, const Ray& y, int isr) {
  if (isr < 1) return -1.0e30;
  if (isr > y.ir_amount) return 1.0e30;
  double s, r; int ix;
  if (r_elem(g, y, isr, s, r, ix) != kGeoOk) return 1.0e30;
  return s;
}

struct Extra {
  int n;
  double s[kExtraMax], r[kExtraMax], th[kExtraMax];
  int ir[kExtraMax], it[kExtraMax];
};

// bisection of a generated ascending list (hunt0 with no usable guess)
template <class F>
RL_HD int bisect_list(const F& f, int n, double x) {
  int jlo = 0, jhi = n + 1;
  const bool ascnd = f(n) > f(1);
  while (jhi - jlo != 1) {
    const int jm = (jhi + jlo) / 2;
    if ((x > f(jm)) == ascnd) jlo = jm; else jhi = jm;
  }
  return jlo;
}
struct ThList { const Grid* g; const Ray* y; RL_HD double operator()(int j) const { return th_s_at(*g, *y, j); } };
struct RList { const Grid* g; const Ray* y; RL_HD double operator()(int j) const { return r_s_at(*g, *y, j); } };

// Extra points, generated directly in ascending s order per group, then merged.
RL_HD int make_extra(const Grid& g, const Ray& y, Extra& E, int& ixg, int& iyg) {
  const RAcc racc{&g};
  const TAcc tacc{&g};
  Extra A, B;   // radial-extremum group, theta-extremum group (each ascending in s)
  A.n = 0; B.n = 0;
  if (y.bimpact > Rg(g, 1)) {
    const double s3 = 0.0 - y.z0 * y.costh0;
    const RList rl{&g, &y};
    const int isrt = bisect_list(rl, y.ir_amount, s3);
    const double rs_m1 = r_s_at(g, y, isrt - 1), rs_0 = r_s_at(g, y, isrt);
    const double rs_p1 = r_s_at(g, y, isrt + 1), rs_p2 = r_s_at(g, y, isrt + 2);
    // ascending: (rs_m1, rs_0) pts, (rs_0, s3) pts, s3, (s3, rs_p1) pts, (rs_p1, rs_p2) pts
    const double lo[4] = {rs_m1, rs_0, s3, rs_p1};
    const double hi[4] = {rs_0, s3, rs_p1, rs_p2};
    // extremum itself is emitted between interval 1 and 2
    for (int q = 0; q < 4; q++) {
      if (q == 2) {
        A.s[A.n] = s3; A.r[A.n] = y.bimpact; A.th[A.n] = theta_at(y, s3);
        A.ir[A.n] = y.ir_min - 1;
        iyg = hunt(tacc, g.ny, A.th[A.n], iyg); A.it[A.n] = iyg;
        A.n++;
      }
      const double ds = (hi[q] - lo[q]) / (1.0 + 1.0 * kAdPts);
      for (int iad = 1; iad <= kAdPts; iad++) {
        const double s0 = iad * ds + lo[q];
        const double rr = radius_at(y, s0);
        A.s[A.n] = s0; A.r[A.n] = rr; A.th[A.n] = theta_at(y, s0);
        ixg = hunt(racc, g.nr, rr, ixg); A.ir[A.n] = ixg;
        iyg = hunt(tacc, g.ny, A.th[A.n], iyg); A.it[A.n] = iyg;
        A.n++;
      }
    }
  }
  {
    const double s3 = y.x0 * y.x0 * y.costh0 / (y.z0 * y.sinth02);
    const double rr = radius_at(y, s3);
    if (rr > Rg(g, 1) && rr < Rg(g, g.nr)) {
      ixg = hunt(racc, g.nr, rr, ixg);
      if (ixg == 0 || ixg == g.nr) return kGeoHuntFail;
      const int ixe = ixg;
      iyg = hunt(tacc, g.ny, theta_at(y, s3), iyg);
      const int iye = iyg;
      const ThList tl{&g, &y};
      const int isrt = bisect_list(tl, y.ith_amount, s3);
      const bool around = !(isrt - 4 + 1 < 1 || isrt + 4 > y.ith_amount);
      double lo[4] = {0, 0, 0, 0}, hi[4] = {0, 0, 0, 0};
      if (around) {
        const double t_m1 = th_s_at(g, y, isrt - 1), t_0 = th_s_at(g, y, isrt);
        const double t_p1 = th_s_at(g, y, isrt + 1), t_p2 = th_s_at(g, y, isrt + 2);
        lo[0] = t_m1; hi[0] = t_0; lo[1] = t_0; hi[1] = s3; lo[2] = s3; hi[2] = t_p1; lo[3] = t_p1; hi[3] = t_p2;
        for (int q = 0; q < 4; q++) if (!(hi[q] > lo[q])) return kGeoOrder;
      }
      for (int q = 0; q < 4; q++) {
        if (q == 2) {
          B.s[B.n] = s3; B.r[B.n] = rr; B.th[B.n] = theta_at(y, s3); B.ir[B.n] = ixe; B.it[B.n] = iye;
          B.n++;
        }
        if (!around) continue;
        const double ds = (hi[q] - lo[q]) / (1.0 + 1.0 * kAdPts);
        for (int iad = 1; iad <= kAdPts; iad++) {
          const double s0 = iad * ds + lo[q];
          const double r3 = radius_at(y, s0);
          ixg = hunt(racc, g.nr, r3, ixg);
          if (ixg == 0 || ixg == g.nr) continue;
          B.s[B.n] = s0; B.r[B.n] = r3; B.th[B.n] = theta_at(y, s0); B.ir[B.n] = ixg;
          iyg = hunt(tacc, g.ny, B.th[B.n], iyg); B.it[B.n] = iyg;
          B.n++;
        }
      }
    }
  }
  // merge the two ascending groups (a stable order by s, as the sorted list)
  int ia = 0, ib = 0;
  E.n = 0;
  while (ia < A.n || ib < B.n) {
    const bool takeA = (ib >= B.n) || (ia < A.n && !(B.s[ib] < A.s[ia]));
    const Extra& S = takeA ? A : B;
    const int k = takeA ? ia++ : ib++;
    E.s[E.n] = S.s[k]; E.r[E.n] = S.r[k]; E.th[E.n] = S.th[k]; E.ir[E.n] = S.ir[k]; E.it[E.n] = S.it[k];
    E.n++;
  }
  return kGeoOk;
}

// Local photon direction at a node (telescope.F:3687-3718), returned as mu, sqrt(1-mu^2),
// sin(phi), cos(phi); sin/cos follow from phi = asin(p) (x0<0) or pi - asin(p) directly.
// bnew (per ray) and the radius sqrt(bnew^2 + snew^2) give mu and sqrt(1 - mu^2) with one
// square root and one reciprocal.
RL_HD void direction(const Ray& y, double s, double& mu, double& sinmu, double& sinphi, double& cosphi) {
  const double bnew = y.bnew, znew = y.znew;
  const double snew = s + y.z0 * y.costh0;
  const double rr2 = bnew * bnew + snew * snew;
  const double irad = 1.0 / sqrt(rr2);
  mu = fmin(1.0, fmax(-1.0, snew * irad));   // the reciprocal may round |mu| past 1 on the axis
  sinmu = bnew * irad;
  const double q = znew + snew * y.costh0;
  const double dummy = bnew * sqrt(rr2 - q * q);
  const double sp = (dummy > 0.0) ? (bnew * bnew * y.costh0 - znew * snew) / dummy : 1.0e1 * kTelEps;
  sinphi = sp;
  const double c = sqrt(1.0 - sp * sp);
  cosphi = (y.x0 < 0.0) ? c : -c;
}

// The FP32 build's node values come from float-float ("double-single") arithmetic: a
// value is hi + lo with |lo| <= ulp(hi)/2, about 44 significant bits, built on the
// error-free transformations of Knuth (two-sum) and Dekker (two-product, here with a
// fused multiply-add). The projected velocity rounded to FP32 then equals the FP64
// value rounded to FP32 except within about 1e-13 of a rounding boundary, so the FP32
// build takes the reference's velocity-window decisions (REAL minvel/maxvel of the
// FP64 omega.v, telescope.F:4260-4265) as the FP64 build does.
// Every operation is spelled out (no contraction left to the compiler): the
// transformations need each rounding where it is written.
#ifdef __CUDA_ARCH__
#define RL_FMA(a, b, c) __fmaf_rn(a, b, c)
#define RL_MUL(a, b) __fmul_rn(a, b)
#define RL_ADD(a, b) __fadd_rn(a, b)
#define RL_SUB(a, b) __fsub_rn(a, b)
#define RL_DIV(a, b) __fdiv_rn(a, b)
#define RL_SQRT(a) __fsqrt_rn(a)
#else
#define RL_FMA(a, b, c) fmaf(a, b, c)
#define RL_MUL(a, b) ((a) * (b))
#define RL_ADD(a, b) ((a) + (b))
#define RL_SUB(a, b) ((a) - (b))
#define RL_DIV(a, b) ((a) / (b))
#define RL_SQRT(a) sqrtf(a)
#endif
struct ff { float hi, lo; };
RL_HD ff ff_of(double x) {
  ff r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}
RL_HD ff ff_c(float x) { return ff{x, 0.0f}; }
// a + b for |a| >= |b| (or a = 0): the rounded sum and its exact error
RL_HD ff ff_fast_two_sum(float a, float b) {
  const float s = RL_ADD(a, b);
  return ff{s, RL_SUB(b, RL_SUB(s, a))};
}
RL_HD ff ff_two_sum(float a, float b) {
  const float s = RL_ADD(a, b);
  const float bb = RL_SUB(s, a);
  return ff{s, RL_ADD(RL_SUB(a, RL_SUB(s, bb)), RL_SUB(b, bb))};
}
RL_HD ff ff_add(ff x, ff y) {
  const ff s = ff_two_sum(x.hi, y.hi);
  return ff_fast_two_sum(s.hi, RL_ADD(s.lo, RL_ADD(x.lo, y.lo)));
}
RL_HD ff ff_neg(ff x) { return ff{-x.hi, -x.lo}; }
RL_HD ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }
RL_HD ff ff_mul(ff x, ff y) {
  const float p = RL_MUL(x.hi, y.hi);
  float e = RL_FMA(x.hi, y.hi, -p);
  e = RL_FMA(x.hi, y.lo, e);
  e = RL_FMA(x.lo, y.hi, e);
  return ff_fast_two_sum(p, e);
}
RL_HD ff ff_div(ff x, ff y) {
  const float q1 = RL_DIV(x.hi, y.hi);
  const ff r = ff_sub(x, ff_mul(ff_c(q1), y));
  return ff_fast_two_sum(q1, RL_DIV(r.hi, y.hi));
}
// sqrt(x) for x >= 0 (0 for x <= 0): one correction of the FP32 root s by (x - s^2)/(2s)
RL_HD ff ff_sqrt(ff x) {
  if (!(x.hi > 0.0f)) return ff_c(0.0f);
  const float s = RL_SQRT(x.hi);
  const float p = RL_MUL(s, s);
  const float e = RL_FMA(s, s, -p);
  const float r = RL_ADD(RL_SUB(RL_SUB(x.hi, p), e), x.lo);
  return ff_fast_two_sum(s, RL_DIV(r, RL_ADD(s, s)));
}

// direction() in float-float from the FP64 position along the ray, the same formulas in
// the same order.
RL_HD void direction_ff(const Ray& y, double s, ff& mu, ff& sinmu, ff& sinphi, ff& cosphi) {
  const ff bnew{y.bnew_f, y.bnew_l}, znew{y.znew_f, y.znew_l}, c0{y.costh0_f, y.costh0_l};
  const ff snew = ff_of(s + y.z0 * y.costh0);
  const ff rr2 = ff_add(ff_mul(bnew, bnew), ff_mul(snew, snew));
  const ff irad = ff_div(ff_c(1.0f), ff_sqrt(rr2));
  mu = ff_mul(snew, irad);
  if (mu.hi > 1.0f || (mu.hi == 1.0f && mu.lo > 0.0f)) mu = ff_c(1.0f);
  if (mu.hi < -1.0f || (mu.hi == -1.0f && mu.lo < 0.0f)) mu = ff_c(-1.0f);
  sinmu = ff_mul(bnew, irad);
  const ff q = ff_add(znew, ff_mul(snew, c0));
  const ff dummy = ff_mul(bnew, ff_sqrt(ff_sub(rr2, ff_mul(q, q))));
  sinphi = dummy.hi > 0.0f ? ff_div(ff_sub(ff_mul(ff_mul(bnew, bnew), c0), ff_mul(znew, snew)), dummy)
                           : ff_of(1.0e1 * kTelEps);
  const ff c = ff_sqrt(ff_sub(ff_c(1.0f), ff_mul(sinphi, sinphi)));
  cosphi = (y.x0 < 0.0) ? c : ff_neg(c);
}

template <bool kFp32>
RL_HD void set_direction(const Ray& y, Node& nd) {
  if (kFp32) {
    ff mu, sinmu, sinphi, cosphi;
    direction_ff(y, nd.s, mu, sinmu, sinphi, cosphi);
    nd.mu_f = mu.hi; nd.mu_l = mu.lo; nd.sinmu_f = sinmu.hi; nd.sinmu_l = sinmu.lo;
    nd.sinphi_f = sinphi.hi; nd.sinphi_l = sinphi.lo; nd.cosphi_f = cosphi.hi; nd.cosphi_l = cosphi.lo;
  } else {
    direction(y, nd.s, nd.mu, nd.sinmu, nd.sinphi, nd.cosphi);
  }
}

// Walk the merged node sequence, calling emit(const Node&) for each accepted node.
// Returns a GeoStatus; emit returns false to stop (buffer full).
template <class Emit>
RL_HD int trace(const Grid& g, double x0, double z0, double theta0, Emit& emit) {
  Ray y;
  int st = init_ray(g, x0, z0, theta0, y);
  if (st != kGeoOk) return st;
  const RAcc racc{&g};
  const TAcc tacc{&g};
  int ixg = g.nr + 1, iyg = g.nth + 1;   // search guesses, carried between calls
  Extra E;
  st = make_extra(g, y, E, ixg, iyg);
  if (st != kGeoOk) return st;
  const double epsplus = 1.0e1 * kTelEps;
  const double rmaxt = Rg(g, g.nr) * (1.0 - epsplus), rmaxr = Rg(g, g.nr) * (1.0 + epsplus);
  const double rmint = Rg(g, 1) * (1.0 + epsplus), rminr = Rg(g, 1) * (1.0 - epsplus);
  const double sbeg = -1.0e30, send = 1.0e30;
  double sprev = -1.0e30;
  const int tr_amount = y.ir_amount + y.ith_amount;
  int ist = 1, isr = 1, ie = 0;
  double ths = 1.0e30, rs = 1.0e30, thr = 0.0, rr = 0.0;
  int thi = 0, rix = 0;
  auto load_th = [&](int i) {
    if (i > y.ith_amount) { ths = 1.0e30; return; }
    th_elem(g, y, i, ths, thi); thr = radius_at(y, ths);
  };
  auto load_r = [&](int i) -> int {
    if (i > y.ir_amount) { rs = 1.0e30; return kGeoOk; }
    return r_elem(g, y, i, rs, rr, rix);
  };
  load_th(1);
  st = load_r(1);
  if (st != kGeoOk) return st;
  Node nd;
  for (int iss = 1; iss <= tr_amount; iss++) {
    const double lim = ths < rs ? ths : rs;
    while (ie < E.n && E.s[ie] < lim) {
      if (E.r[ie] <= rmaxt && E.r[ie] >= rmint && (E.s[ie] - sprev) > kTelEps * E.r[ie] &&
          E.s[ie] >= sbeg && E.s[ie] <= send) {
        nd.icr = 3; nd.r = E.r[ie]; nd.th = E.th[ie]; nd.ir = E.ir[ie]; nd.it = E.it[ie]; nd.s = E.s[ie];
        set_direction<Emit::kFp32Direction>(y, nd);
        sprev = nd.s;
        if (!emit(nd)) return kGeoOverflow;
      }
      ie++;
    }
    if (ths < rs) {
      if (thr <= rmaxt && thr >= rmint && (ths - sprev) > kTelEps * thr && ths >= sbeg && ths <= send) {
        nd.icr = 2; nd.r = thr; nd.th = Tg(g, thi); nd.it = thi; nd.s = ths;
        if (thr < Rg(g, 1)) nd.ir = 0;
        else if (thr > Rg(g, g.nr)) nd.ir = g.nr;
        else { ixg = hunt(racc, g.nr, thr, ixg); nd.ir = ixg; }
        set_direction<Emit::kFp32Direction>(y, nd);
        sprev = nd.s;
        if (!emit(nd)) return kGeoOverflow;
      }
      ist++;
      load_th(ist);
    } else {
      if (rr <= rmaxr && rr >= rminr && (rs - sprev) > kTelEps * rr && rs >= sbeg && rs <= send) {
        nd.icr = 1; nd.r = rr; nd.th = theta_at(y, rs); nd.ir = rix; nd.s = rs;
        iyg = hunt(tacc, g.ny, nd.th, iyg); nd.it = iyg;
        set_direction<Emit::kFp32Direction>(y, nd);
        sprev = nd.s;
        if (!emit(nd)) return kGeoOverflow;
      }
      isr++;
      st = load_r(isr);
      if (st != kGeoOk) return st;
    }
  }
  return kGeoOk;
}

// Upper bound on the number of nodes of any ray for this grid.
RL_HD int max_nodes(int nr, int nth) { return 2 * (nr + 1) + 2 * nth + kExtraMax; }

}  // namespace rlg
