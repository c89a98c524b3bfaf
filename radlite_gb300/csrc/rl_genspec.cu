// rl_genspec.cu -- the spectrum post-processing of pyradlite's RadliteSpectrum.gen_spec
// (pyradlite/radlite.py:3001-3187, _process_spectrum): the line profiles of all cores are
// continuum-subtracted, resampled onto one fine wavelength grid of constant velocity
// step and summed, a continuum is interpolated between the line centres, the sum is
// smoothed with a Gaussian of the observing resolution and resampled at the requested
// sampling.
//
//   host      the grids, the kernel and its sum (FP64, numpy's operation order; pow and
//             exp from the host libm as numpy uses them)
//   k_gs_lines    per line: emission-only profile and the wavelength nodes of its box
//   k_gs_fine     per fine point: the lines' emission in line order, the continuum, Jy
//   k_gs_smooth   per fine point: Gaussian convolution with reflected edges
//   k_gs_out      per output point: linear resampling of the three spectra
//
// Every device operation is an explicit round-to-nearest add, multiply or divide, in
// the reference's order, so that no contraction into FMA changes a result.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "rl_internal.h"

namespace rl {

constexpr double kC0 = 2.99792458e10;      // cm/s
constexpr double kCinMu = kC0 * 1.0e4;     // micron/s
constexpr double kCinKm = kC0 / 1.0e5;     // km/s

// np.interp for x inside [xp[0], xp[n-1]]: j with xp[j] <= x < xp[j+1]; the nodes
// themselves return their value exactly.
__device__ __forceinline__ double interp_np(double x, const double* __restrict__ xp, const double* __restrict__ fp,
                                            int n) {
  if (x == xp[n - 1]) return fp[n - 1];
  int lo = 0, hi = n - 1;   // xp[lo] <= x < xp[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (xp[mid] <= x) lo = mid; else hi = mid;
  }
  if (xp[lo] == x) return fp[lo];
  const double slope = __ddiv_rn(__dsub_rn(fp[lo + 1], fp[lo]), __dsub_rn(xp[lo + 1], xp[lo]));
  return __dadd_rn(__dmul_rn(slope, __dsub_rn(x, xp[lo])), fp[lo]);
}

struct GsParams {
  int nlines, nfine, nout, nk, kc;
  const int* off;          // [nlines+1] first channel of each line in vel/flux
  const double* vel;       // concatenated ascending velocities [km/s]
  const double* flux;      // concatenated fluxes
  const double* freq;      // [nlines]
  double boxwidth, mumin, mumax, d2, ksum;
  double* em;              // [total channels] emission-only profile
  double* muold;           // [total channels + 2 nlines] box nodes of each line
  double* emold;           // same layout
  int* range;              // [nlines][2] first and last fine index inside the box
  double* cmu;             // [nlines+2] sorted line centres with the grid ends
  double* ccont;           // [nlines+2] continuum at the centres
  const double* fine;      // [nfine]
  double* full_em;         // [nfine]
  double* full_y;          // [nfine]
  double* full_cont;       // [nfine]
  double* res_em;          // [nfine]
  double* res_y;           // [nfine]
  const double* kern;      // [nk]
  const double* outmu;     // [nout]
  double *o_spec, *o_em, *o_cont, *o_freq;   // [nout]
};

// first index with fine[i] >= x (lower bound)
__device__ __forceinline__ int lower_bound(const double* a, int n, double x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Block l: line l. Continuum through the two edge channels (radlite.py:3079-3089), the
// emission-only profile, and the profile extended to the box edges in wavelength
// (radlite.py:3097-3106); its fine-grid index range.
__global__ void k_gs_lines(GsParams p) {
  const int l = blockIdx.x;
  const int a = p.off[l], n = p.off[l + 1] - a;
  const double* v = p.vel + a;
  const double* f = p.flux + a;
  const double xs[2] = {v[0], v[n - 1]}, ys[2] = {f[0], f[n - 1]};
  const double fr = p.freq[l];
  const double c0 = __ddiv_rn(kCinMu, fr);   // cinmu0/1.0/freq
  double* mo = p.muold + a + 2 * l;
  double* eo = p.emold + a + 2 * l;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double e = __dsub_rn(f[i], interp_np(v[i], xs, ys, 2));
    p.em[a + i] = e;
    eo[i + 1] = e;
    mo[i + 1] = __dadd_rn(__ddiv_rn(__dmul_rn(v[i], 1.0e9), fr), c0);
  }
  if (threadIdx.x == 0) {
    mo[0] = __dadd_rn(__ddiv_rn(__dmul_rn(-1.0 * p.boxwidth, 1.0e9), fr), c0);
    mo[n + 1] = __dadd_rn(__ddiv_rn(__dmul_rn(p.boxwidth, 1.0e9), fr), c0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    eo[0] = eo[1];
    eo[n + 1] = eo[n];
    const double x0 = 0.0;
    p.ccont[l] = interp_np(x0, xs, ys, 2);   // centre continuum, unsorted here
    // fine points with muold[0] <= fine <= muold[n+1]
    const int i0 = lower_bound(p.fine, p.nfine, mo[0]);
    int i1 = lower_bound(p.fine, p.nfine, mo[n + 1]);
    if (i1 < p.nfine && p.fine[i1] == mo[n + 1]) i1++;
    p.range[2 * l] = i0;
    p.range[2 * l + 1] = i1;   // exclusive
  }
}

// Fine point i: the emission of every line covering it, added in line order
// (radlite.py:3095-3114), the continuum between the sorted line centres
// (radlite.py:3118-3128), and the conversion to Jy at the distance (radlite.py:3131-3135).
__global__ void k_gs_fine(GsParams p) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.nfine; i += gridDim.x * blockDim.x) {
    const double x = p.fine[i];
    double acc = 0.0;
    for (int l = 0; l < p.nlines; l++) {
      if (i < p.range[2 * l] || i >= p.range[2 * l + 1]) continue;
      const int a = p.off[l] + 2 * l, n = p.off[l + 1] - p.off[l] + 2;
      acc = __dadd_rn(acc, interp_np(x, p.muold + a, p.emold + a, n));
    }
    const double cont = interp_np(x, p.cmu, p.ccont + p.nlines, p.nlines + 2);
    const double em = __ddiv_rn(__dmul_rn(acc, 1.0e23), p.d2);
    const double cj = __ddiv_rn(__dmul_rn(cont, 1.0e23), p.d2);
    p.full_em[i] = em;
    p.full_cont[i] = cj;
    p.full_y[i] = __dadd_rn(cj, em);
  }
}

// Gaussian smoothing (scipy.ndimage.convolve, mode 'reflect'), normalised by the kernel
// sum (radlite.py:3147-3152). The kernel is symmetric; its centre is nk/2, one sample to
// the left for an even length. The reflected extension (d c b a | a b c d | d c b a)
// repeats with period 2n, which matters for kernels longer than the grid.
__global__ void k_gs_smooth(GsParams p) {
  const int n = p.nfine;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double se = 0.0, sy = 0.0;
    for (int j = 0; j < p.nk; j++) {
      int t = (i + j - p.kc) % (2 * n);
      if (t < 0) t += 2 * n;
      if (t >= n) t = 2 * n - t - 1;
      const double w = p.kern[p.nk - 1 - j];
      se = __dadd_rn(se, __dmul_rn(p.full_em[t], w));
      sy = __dadd_rn(sy, __dmul_rn(p.full_y[t], w));
    }
    p.res_em[i] = __ddiv_rn(se, p.ksum);
    p.res_y[i] = __ddiv_rn(sy, p.ksum);
  }
}

// Output point k: linear resampling (radlite.py:3157-3170).
__global__ void k_gs_out(GsParams p) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < p.nout; k += gridDim.x * blockDim.x) {
    const double x = p.outmu[k];
    p.o_spec[k] = interp_np(x, p.fine, p.res_y, p.nfine);
    p.o_em[k] = interp_np(x, p.fine, p.res_em, p.nfine);
    p.o_cont[k] = interp_np(x, p.fine, p.full_cont, p.nfine);
    p.o_freq[k] = __ddiv_rn(kC0, __dmul_rn(x, 1.0e-4));
  }
}

// numpy's pairwise summation (np.sum of a 1-D float64 array)
static double pairwise_sum(const double* a, long n) {
  if (n < 8) {
    double s = 0.0;
    for (long i = 0; i < n; i++) s += a[i];
    return s;
  }
  if (n <= 128) {
    double r[8];
    for (int k = 0; k < 8; k++) r[k] = a[k];
    long i = 8;
    for (; i < n - (n % 8); i += 8)
      for (int k = 0; k < 8; k++) r[k] += a[i + k];
    double s = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
    for (; i < n; i++) s += a[i];
    return s;
  }
  long m = n / 2;
  m -= m % 8;
  return pairwise_sum(a, m) + pairwise_sum(a + m, n - m);
}

struct GsHost {
  double boxwidth = 0, vres = 0, mumin = 0, mumax = 0;
  std::vector<double> fine, out, kern;
  double ksum = 0;
};

// The grids and kernel of radlite.py:3030-3069, 3141-3144, in numpy's operation order.
static int gs_host(const rl_genspec_lines* in, const rl_genspec_params* p, GsHost& h, std::string& err) {
  const int nl = in->nlines;
  if (nl < 1 || !in->npts || !in->vel || !in->flux || !in->freq || !in->maxnumpoints) {
    err = "gen_spec: no lines or a null array";
    return -1;
  }
  if (!(p->obsres > 0.0) || !(p->vsampling > 0.0) || !(p->dist > 0.0)) {
    err = "gen_spec: obsres, vsampling and dist must be positive";
    return -1;
  }
  long off = 0;
  double maxvspan = 0.0;
  int imax = 0;
  for (int l = 0; l < nl; l++) {
    if (in->npts[l] < 2) { err = "gen_spec: a line needs at least 2 channels"; return -1; }
    // the reference leaves lines of frequency 0 out of the grid range but still divides
    // by their frequency (radlite.py:3045, 3097); such lines are rejected here
    if (!(in->freq[l] > 0.0)) { err = "gen_spec: a line's frequency is not positive"; return -1; }
    for (int i = 1; i < in->npts[l]; i++)
      if (!(in->vel[off + i] > in->vel[off + i - 1])) { err = "gen_spec: velocities must ascend"; return -1; }
    // the continuum is evaluated at velocity 0 (interp1d's bounds check in the reference)
    if (!(in->vel[off] <= 0.0 && in->vel[off + in->npts[l] - 1] >= 0.0)) {
      err = "gen_spec: a line's velocities do not span 0";
      return -1;
    }
    maxvspan = std::max(maxvspan, std::fabs(in->vel[off]));
    if (in->maxnumpoints[l] > in->maxnumpoints[imax]) imax = l;
    off += in->npts[l];
  }
  h.boxwidth = std::max(3 * maxvspan, 3 * p->obsres);
  long oi = 0;
  for (int l = 0; l < imax; l++) oi += in->npts[l];
  h.vres = in->vel[oi + 1] - in->vel[oi];
  double mulo = 0, muhi = 0;
  bool any = false;
  for (int l = 0; l < nl; l++) {
    const double mu = kCinMu / 1.0 / in->freq[l];
    if (!any || mu < mulo) mulo = mu;
    if (!any || mu > muhi) muhi = mu;
    any = true;
  }
  h.mumin = mulo - (h.boxwidth * 1.0e9 * mulo / kCinMu);
  h.mumax = muhi + (h.boxwidth * 1.0e9 * muhi / kCinMu);
  const double g = 1 + (h.vres / 1.0 / kCinKm);
  const long n = (long)(std::floor(std::log(h.mumax / 1.0 / h.mumin) / std::log(g)) + 1);
  const double gu = 1 + (p->vsampling / 1.0 / kCinKm);
  const long nu = (long)(std::floor(std::log(h.mumax / 1.0 / h.mumin) / std::log(gu)) + 1);
  if (n < 2 || nu < 1 || n > (1L << 28) || nu > (1L << 28)) { err = "gen_spec: grid size out of range"; return -1; }
  h.fine.resize(n);
  for (long i = 0; i < n; i++) h.fine[i] = h.mumin * std::pow(g, (double)i);
  h.out.resize(nu);
  for (long i = 0; i < nu; i++) h.out[i] = h.mumin * std::pow(gu, (double)i);
  // interp1d's bounds checks of the reference (ValueError there)
  if (h.fine[n - 1] > h.mumax) { err = "gen_spec: the fine grid ends above the continuum range"; return -1; }
  if (h.out[nu - 1] > h.fine[n - 1]) {
    char b[200];
    std::snprintf(b, sizeof b, "gen_spec: a value (%.17g) in x_new is above the interpolation range's maximum value (%.17g)",
                  h.out[nu - 1], h.fine[n - 1]);
    err = b;
    return -1;
  }
  const double nk = std::ceil(3.0 * p->obsres / h.vres);
  if (!(nk >= 1.0) || nk > 1.0e6) { err = "gen_spec: kernel length out of range"; return -1; }
  h.kern.resize((size_t)nk);
  const double bot = ((p->obsres / 1.0 / h.vres) * (p->obsres / 1.0 / h.vres)) * std::log(2.0);
  for (size_t j = 0; j < h.kern.size(); j++) {
    const double t = (double)j - ((nk - 1) / 2.0);
    h.kern[j] = std::exp((-1 * 2 * (t * t)) / bot);
  }
  h.ksum = pairwise_sum(h.kern.data(), (long)h.kern.size());
  return 0;
}

}  // namespace rl

using namespace rl;

extern "C" {

int rl_gen_spec_size(const rl_genspec_lines* in, const rl_genspec_params* p, long long* nout) {
  if (!in || !p || !nout) return set_err(nullptr, RL_ERR_ARG, "rl_gen_spec_size: null argument");
  GsHost h;
  std::string err;
  if (gs_host(in, p, h, err)) return set_err(nullptr, RL_ERR_ARG, err);
  *nout = (long long)h.out.size();
  return 0;
}

int rl_gen_spec(rl_ctx* ctx, const rl_genspec_lines* in, const rl_genspec_params* p, double* wavelength,
                double* frequency, double* spectrum, double* emission, double* continuum, rl_stats* st) {
  if (!ctx || !in || !p || !wavelength || !frequency || !spectrum || !emission || !continuum)
    return set_err(ctx, RL_ERR_ARG, "rl_gen_spec: null argument");
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  g_h2d = 0; g_d2h = 0;
  GsHost h;
  std::string err;
  if (gs_host(in, p, h, err)) return set_err(ctx, RL_ERR_ARG, err);
  const int nl = in->nlines;
  std::vector<int> off(nl + 1, 0);
  for (int l = 0; l < nl; l++) off[l + 1] = off[l] + in->npts[l];
  const long tot = off[nl];
  // line centres sorted by wavelength (a stable order), with the grid ends
  std::vector<int> order(nl);
  for (int l = 0; l < nl; l++) order[l] = l;
  std::vector<double> mu(nl);
  for (int l = 0; l < nl; l++) mu[l] = kCinMu / 1.0 / in->freq[l];
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return mu[a] < mu[b]; });
  std::vector<double> cmu(nl + 2);
  cmu[0] = h.mumin;
  for (int l = 0; l < nl; l++) cmu[l + 1] = mu[order[l]];
  cmu[nl + 1] = h.mumax;
  const long nf = (long)h.fine.size(), no = (long)h.out.size();
  DevBuf d_off, d_vel, d_flux, d_freq, d_em, d_muold, d_emold, d_range, d_cmu, d_ccont, d_fine, d_fem, d_fy, d_fc,
      d_rem, d_ry, d_kern, d_out, d_ospec, d_oem, d_ocont, d_ofreq;
  CUDA_TRY(d_off.ensure(sizeof(int) * (nl + 1)));
  CUDA_TRY(d_vel.ensure(sizeof(double) * tot));
  CUDA_TRY(d_flux.ensure(sizeof(double) * tot));
  CUDA_TRY(d_freq.ensure(sizeof(double) * nl));
  CUDA_TRY(d_em.ensure(sizeof(double) * tot));
  CUDA_TRY(d_muold.ensure(sizeof(double) * (tot + 2 * nl)));
  CUDA_TRY(d_emold.ensure(sizeof(double) * (tot + 2 * nl)));
  CUDA_TRY(d_range.ensure(sizeof(int) * 2 * nl));
  CUDA_TRY(d_cmu.ensure(sizeof(double) * (nl + 2)));
  CUDA_TRY(d_ccont.ensure(sizeof(double) * (2 * nl + 2)));
  CUDA_TRY(d_fine.ensure(sizeof(double) * nf));
  CUDA_TRY(d_fem.ensure(sizeof(double) * nf));
  CUDA_TRY(d_fy.ensure(sizeof(double) * nf));
  CUDA_TRY(d_fc.ensure(sizeof(double) * nf));
  CUDA_TRY(d_rem.ensure(sizeof(double) * nf));
  CUDA_TRY(d_ry.ensure(sizeof(double) * nf));
  CUDA_TRY(d_kern.ensure(sizeof(double) * h.kern.size()));
  CUDA_TRY(d_out.ensure(sizeof(double) * no));
  CUDA_TRY(d_ospec.ensure(sizeof(double) * no));
  CUDA_TRY(d_oem.ensure(sizeof(double) * no));
  CUDA_TRY(d_ocont.ensure(sizeof(double) * no));
  CUDA_TRY(d_ofreq.ensure(sizeof(double) * no));
  cudaStream_t s = ctx->stream;
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  CUDA_TRY(h2d(d_off.p, off.data(), sizeof(int) * (nl + 1), s));
  CUDA_TRY(h2d(d_vel.p, in->vel, sizeof(double) * tot, s));
  CUDA_TRY(h2d(d_flux.p, in->flux, sizeof(double) * tot, s));
  CUDA_TRY(h2d(d_freq.p, in->freq, sizeof(double) * nl, s));
  CUDA_TRY(h2d(d_cmu.p, cmu.data(), sizeof(double) * (nl + 2), s));
  CUDA_TRY(h2d(d_fine.p, h.fine.data(), sizeof(double) * nf, s));
  CUDA_TRY(h2d(d_kern.p, h.kern.data(), sizeof(double) * h.kern.size(), s));
  CUDA_TRY(h2d(d_out.p, h.out.data(), sizeof(double) * no, s));
  CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  GsParams P;
  P.nlines = nl; P.nfine = (int)nf; P.nout = (int)no; P.nk = (int)h.kern.size();
  P.kc = P.nk / 2 - (P.nk % 2 == 0 ? 1 : 0);
  // the kernel is applied flipped (convolution); the flipped centre for an even length
  // is one sample to the left of nk/2, so kc indexes the flipped kernel
  P.off = d_off.as<int>(); P.vel = d_vel.as<double>(); P.flux = d_flux.as<double>(); P.freq = d_freq.as<double>();
  P.boxwidth = h.boxwidth; P.mumin = h.mumin; P.mumax = h.mumax; P.d2 = p->dist * p->dist; P.ksum = h.ksum;
  P.em = d_em.as<double>(); P.muold = d_muold.as<double>(); P.emold = d_emold.as<double>(); P.range = d_range.as<int>();
  P.cmu = d_cmu.as<double>(); P.ccont = d_ccont.as<double>(); P.fine = d_fine.as<double>();
  P.full_em = d_fem.as<double>(); P.full_y = d_fy.as<double>(); P.full_cont = d_fc.as<double>();
  P.res_em = d_rem.as<double>(); P.res_y = d_ry.as<double>(); P.kern = d_kern.as<double>(); P.outmu = d_out.as<double>();
  P.o_spec = d_ospec.as<double>(); P.o_em = d_oem.as<double>(); P.o_cont = d_ocont.as<double>();
  P.o_freq = d_ofreq.as<double>();
  k_gs_lines<<<nl, 128, 0, s>>>(P);
  CUDA_TRY(cudaGetLastError());
  // centre continua in wavelength order: ccont[nl .. 2nl+1] = [c_first, sorted..., c_last]
  {
    std::vector<double> cc(nl);
    CUDA_TRY(d2h(cc.data(), d_ccont.p, sizeof(double) * nl, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<double> cs(nl + 2);
    for (int l = 0; l < nl; l++) cs[l + 1] = cc[order[l]];
    cs[0] = cs[1];
    cs[nl + 1] = cs[nl];
    CUDA_TRY(h2d(d_ccont.as<double>() + nl, cs.data(), sizeof(double) * (nl + 2), s));
  }
  const int blocks = std::max(1, std::min((int)((nf + 255) / 256), ctx->nsm * 8));
  k_gs_fine<<<blocks, 256, 0, s>>>(P);
  CUDA_TRY(cudaGetLastError());
  k_gs_smooth<<<blocks, 256, 0, s>>>(P);
  CUDA_TRY(cudaGetLastError());
  k_gs_out<<<std::max(1, std::min((int)((no + 255) / 256), ctx->nsm * 8)), 256, 0, s>>>(P);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
  CUDA_TRY(d2h(spectrum, d_ospec.p, sizeof(double) * no, s));
  CUDA_TRY(d2h(emission, d_oem.p, sizeof(double) * no, s));
  CUDA_TRY(d2h(continuum, d_ocont.p, sizeof(double) * no, s));
  CUDA_TRY(d2h(frequency, d_ofreq.p, sizeof(double) * no, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  std::memcpy(wavelength, h.out.data(), sizeof(double) * no);
  if (st) {
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]);
    st->upload_ms = a; st->walk_ms = b;
    st->nlines = nl; st->nfr = (int)no; st->nrays = (int)nf;
    st->h2d_bytes = g_h2d; st->d2h_bytes = g_d2h;
  }
  return 0;
}

}  // extern "C"
