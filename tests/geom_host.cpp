// Test-only harness: the product's ray/grid geometry (rl_geometry.cuh) compiled for the
// host, so its node lists and interpolation corners can be checked against the oracle
// without a GPU. Not part of the library.
#include <cmath>
#include "../radlite_gb300/csrc/rl_geometry.cuh"

namespace {
struct Collect {
  static constexpr bool kFp32Direction = false;
  int cap, n;
  double *s, *r, *th, *mu;
  int *icr, *ir, *it;
  bool operator()(const rlg::Node& nd) {
    if (n >= cap) return false;
    s[n] = nd.s; r[n] = nd.r; th[n] = nd.th; mu[n] = nd.mu; icr[n] = nd.icr; ir[n] = nd.ir; it[n] = nd.it;
    n++;
    return true;
  }
};
}  // namespace

namespace {
struct Tab {
  const double* xx;   // xx[0..n-1] as xx(1..n)
  double operator()(int j) const { return xx[j - 1]; }
};
}  // namespace

extern "C" int geom_hunt(const double* xx, int n, double x, int guess) { return rlg::hunt(Tab{xx}, n, x, guess); }

extern "C" int geom_trace(int nr, int nth, const double* R, const double* TH, const double* tan2, double rstar,
                          double x0, double z0, double theta0, int cap, double* s, double* r, double* th, double* mu,
                          int* icr, int* ir, int* it, int* status) {
  rlg::Grid g;
  g.R = R; g.TH = TH; g.tan2 = tan2; g.nr = nr; g.nth = nth; g.ny = 2 * nth; g.rstar = rstar;
  Collect c{cap, 0, s, r, th, mu, icr, ir, it};
  *status = rlg::trace(g, x0, z0, theta0, c);
  return c.n;
}
