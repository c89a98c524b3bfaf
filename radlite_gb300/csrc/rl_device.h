// rl_device.h -- plain structs shared by the host orchestration and the CUDA kernels.
#pragma once
#include <stddef.h>
#include <stdint.h>

namespace rl {

// Counters of a walk launch (flush_counters): steps, integrated pairs, node visits, node
// passes, packed node passes, steps of empty segments, refined passes, their sub-steps,
// their refined channels, steps that failed the overshoot test (checking walks).
constexpr int kWalkCounters = 10;
// Walk launch shape: 4-warp blocks, at most this many per SM (sizes the list scratch).
constexpr int kWalkBlocksPerSm = 4;
constexpr int kWalkWarps = 4;
// Lines of one walk work item at most (the list packs a line index into 5 bits).
constexpr int kItemLines = 32;
// Elements of one warp's list row for up to nfr channels per line.
inline size_t walk_list_row(int nfr) { return (size_t)((kItemLines * nfr + 7) & ~7); }
// Elements of the walk's list scratch for nsm SMs and up to nfr channels per line.
inline size_t walk_list_elems(int nsm, int nfr) {
  return (size_t)nsm * kWalkBlocksPerSm * kWalkWarps * walk_list_row(nfr);
}

// Per-node flag bits in NodeBuf::misc (bits 0-15: theta-corner offset + 32768,
// bits 16-17: radial-corner offset + 1).
constexpr unsigned kFlagHole = 1u << 20;   // segment ending here lies in the central hole
constexpr unsigned kFlagIr1 = 1u << 21;    // node on the innermost radial cell (ir == 1)
constexpr unsigned kFlagInit = 1u << 22;   // (walk) the segment ending here restarts the line state
constexpr unsigned kFlagSub = 1u << 23;    // (walk) the segment ending here may need sub-steps
constexpr unsigned kFlagEmpty = 1u << 25;  // (FP32 walk) every staged line has zero emissivity and
                                           // opacity at this node and the previous one
constexpr unsigned kFlagNeg = 1u << 24;    // (FP32 walk) some staged line lacks a positive opacity at
                                           // this node or the previous one
constexpr int kIcrShift = 18;              // bits 18-19: crossing type 1..3

// Node records of all rays of one camera, row-major by ray (row stride kmax).
template <typename T>
struct NodeBuf {
  int nrays = 0, kmax = 0;
  int* nnodes = nullptr;       // [nrays]
  int* status = nullptr;       // [nrays] geometry status (0 = fine)
  T* ds = nullptr;             // s_k - s_{k-1} (0 at k=0 and in the central hole)
  float* dvf = nullptr;        // (float) projected velocity / c  (window test)
  T* vl = nullptr;             // projected velocity in passband units (dvmu / 3.33567e-6)
  T* dvseg = nullptr;          // vl_k - vl_{k-1}, formed in FP64
  T* lw = nullptr;             // interpolated line width [km/s]
  T* wr = nullptr;             // radial interpolation weight
  T* wt = nullptr;             // theta interpolation weight
  int* c00 = nullptr;          // cell index of the base corner
  unsigned* misc = nullptr;    // corner offsets, crossing type, flags
};

// Debug copy of one ray's trajectory (filled only by the debug geometry launch).
struct TrajDebug {
  double* s; double* r; double* th; double* mu; double* dvmu; int* icr; int* ir; int* it;
  int cap;
};

struct GeoParams {
  int nr, nth, ny;
  double rstar, theta0;
  const double* R;      // [nr+4]
  const double* TH;     // [ny+4]
  const double* tan2;   // [nth+1]
  const double* vel;    // [ncell*3]
  const double* lw;     // [ncell]
  const float* velf;    // [ncell*3] FP32 copies for the FP32 build's node values
  const float* vell;    // [ncell*3] their low parts, vel - (double)velf (float-float velocity)
  const float* lwf;     // [ncell]
  const double* x0;     // [nrays]
  const double* z0;     // [nrays]
};

// Per-line constants of the walk.
template <typename T>
struct LineConst {
  T cphi;       // 0.56419583546 / (3.33567e-6 * nu0): profile normalisation times lwav
  T istart;     // outer-boundary start intensity (scaled)
  double scale; // intensity scale: spectrum = scale * sum
};

template <typename T>
struct WalkParams {
  NodeBuf<T> nb;
  int nth, ncell;
  int nlines, nfr, nitems;
  int gsize;                 // lines per work item (<= 8), groups balanced over the launch
  const T* tab;              // [nlines][ncell][4] = {j-factor, alpha-factor, dust j, dust alpha}
  const T* nsum;             // [nlines][ncell] N_up + N_low (window threshold)
  const T* wch;              // [nlines][nfr] channel velocity in passband units
  const double* velo;        // [nlines][nfr] dnu/nu0 (window test)
  const T* star;             // [nlines][nfr] scaled stellar intensity
  const T* isrf = nullptr;   // [nlines][nfr] scaled start intensity per channel (outer
                             //   boundary 3), or null: LineConst::istart for every channel
  const LineConst<T>* lc;    // [nlines]
  double aksmax_c;           // max line width / c
  T kq;                      // 3.33567e-6 * 2.99792458e5
  T fstar;                   // (R*/ri(1))^2 for the central beam
  T* img;                    // [nlines][nrays][nfr]
  T* tau = nullptr;          // [nlines][nrays][nfr] optical depth of each walked channel along the
  T* tauc = nullptr;         //   ray (char_tau) and its compensation term: the position-velocity
                             //   walk, and the walk of the differentiable forward (for the
                             //   gradient sweep); null otherwise
  unsigned char* mask = nullptr;  // optional [nlines][nrays][nfr]: 1 = channel 1 or inside the window
  int* maser = nullptr;      // optional [nlines]: set to 1 where a step's line opacity x segment
                             //   length falls below -0.01 (only launches with an inverted line)
  unsigned long long* counters;   // [0] steps, [1] integrated channels, [2] node visits
  int* work;                 // dynamic work counter
  int* err;                  // first error code
  unsigned short* list;      // per-warp (line, channel) list rows: blocks x 4 warps x ((8 nfr + 7) & ~7)
};

struct ReduceParams {
  int nrays, nfr, nphi, nrr, nlines;
  const double* ri;          // [nrr+2] ring edges
  double dist2;              // distance^2 [cm^2]
  const double* scale;       // [nlines]
};

// ---- many jobs (model, camera, line range) in one launch sequence ----
template <typename T>
struct GeoJob {
  GeoParams geo;
  NodeBuf<T> nb;
};

template <typename T>
struct WalkJobs {
  const WalkParams<T>* jobs;  // [njobs] (device)
  const int* item_prefix;     // [njobs+1] first item of each job
  int njobs, total;           // total = item_prefix[njobs]
  int stride;                 // 1, or > 1 to walk every stride-th item only (tuning samples)
  int max_nfr;                // largest channel count of the jobs (list row size)
  int* work;                  // queue counter
  unsigned long long* counters;
  unsigned short* list;       // per-warp list rows, as WalkParams::list with max_nfr
  bool tau = false;           // the jobs' walks also keep each channel's optical depth
};

template <typename T>
struct RedJob {
  ReduceParams p;
  const T* img;
  double* ring;
  double* flux;
};

template <typename T>
struct JobLaunch {
  int njobs, nsm, cpl;
  const GeoJob<T>* geo;      // [njobs] (device); nrays_total = 0 skips the geometry
  const int* ray_prefix;
  int nrays_total;
  WalkJobs<T> walk;
  bool walk_jobs = true;     // false: no walk launch (the jobs are walked by per-job launches)
  bool reduce;
  const RedJob<T>* red;      // [njobs] (device)
  const int* ring_prefix;    // [njobs+1] (line, ring) pairs
  const int* line_prefix;    // [njobs+1] lines
  int nring_blocks, nline_blocks;
};

// ---- differentiable path: LTE line tables from per-cell parameters, adjoint walk ----
struct LteLine {
  int lu, ld;                 // 0-based upper and lower level of the line
  double C1, C2, Bud, Bdu;    // j = C1 N_up phi, alpha = C2 (N_low Bdu - N_up Bud) phi
  double nu;                  // line frequency (dust Planck function at the line centre)
  double cphi, scale;         // profile normalisation; fixed intensity scale of the walk
};

template <typename T>
struct LteParams {
  int ncell, nlev, nl;
  const double* lnT;          // [ncell] ln gas (= dust) temperature
  const double* lnX;          // [ncell] ln molecular abundance
  const double* rho_m;        // [ncell] rho / (umass m_p): molecules per unit abundance
  const double* Ek;           // [nlev] level energies E hc/k [K]
  const double* lng;          // [nlev] ln statistical weight
  const LteLine* lines;       // [nl]
  const double* dust;         // [ncell][nl][3]: sum rho_d kappa_abs(nu0), scattering source, extinction
  double* lnQ;                // [ncell] ln partition sum (work)
  double* Emean;              // [ncell] mean level energy / kT (work)
  T* tab;                     // [ncell][nl][4] walk table
  T* nsum;                    // [ncell][nl] N_up + N_low
  T* dtab;                    // [ncell][nl][5]: d tab[0..2] / d lnT, tab[0], tab[1]
};

template <typename T>
struct AdjParams {
  WalkParams<T> W;            // the forward walk of this job (node records, tables, window data)
  const double* gflux;        // [nl][nfr] dL/dF_nu (F_nu at 1 pc)
  const double* ri;           // [nrr+2] ring edges
  int nphi, nrr;
  const T* dtab;              // [ncell][nl][5] table derivatives of the LTE tables (LteParams::dtab)
  double* g_lnT;              // [ncell] dL/d ln T, accumulated
  double* g_lnX;              // [ncell] dL/d ln X, accumulated
  double* g_b;                // [ncell] dL/d(cell line width), accumulated
  float4* g4 = nullptr;       // FP32 walk: [ncell] {dL/d ln T, dL/d ln X, dL/d width, 0} accumulated
                              //   with one vector atomic per corner instead of g_lnT/g_lnX/g_b
                              //   (launch_adjoint_finish converts them)
};

template <typename T>
struct AdjJobs {
  const AdjParams<T>* jobs;   // [njobs] (device)
  const int* item_prefix;     // [njobs+1]; a job has nlines x nrays items (line-major)
  int njobs, total, max_nfr;
  T* ckpt;                    // per-warp checkpoint scratch, ckpt_warp values each
  long long ckpt_warp;
  int every;                  // checkpoint interval in nodes: 1 (keep every intensity) or 32
  int* work;
  unsigned long long* counters;   // [0] adjoint steps, [1] items whose continuum was zero
};

}  // namespace rl
