// rl_batch.cpp -- many (model, camera, line range) jobs rendered by one launch sequence.
//
// The reference renders one line of one model per calc_line_spectrum call
// (main.F:1043-1049) and drivers run one process per model directory
// (radlite.py:592-595). Here a batch keeps the per-job inputs resident on the device
// (camera rays, per-line cell tables) and renders every job with three launches per
// memory wave: geometry of all cameras, one persistent walk over the concatenated
// (job, line group, ray) items fed from a device counter, and the image -> spectrum
// reduction of all jobs. The whole sequence is captured once in a CUDA graph and
// replayed. The line-group size and channel tile come from rl_batch_autotune, which
// times candidate shapes on a strided sample of the work.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#include "rl_geometry.cuh"
#include "rl_internal.h"

using namespace rl;

namespace {

constexpr size_t kAlign = 256;
// Streams the per-job walk launches of a run are spread over: a job's persistent launch
// holds the whole GPU until its work counter runs dry, and the launches queued on the
// other streams fill the SMs its tail leaves idle.
constexpr int kSideStreams = 4;
inline size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

struct BatchJob {
  rl_model* md = nullptr;
  int iline0 = 0, nl = 0;
  Camera cam;
  int kmax = 0, nfr = 0, ncell = 0;
  double aksmax = 0.0, fstar = 0.0;
  bool has_isrf = false;                               // star holds the outer-boundary-3 table too
  bool inverted = false;                               // some line has a population inversion
  int line_off = 0;                                    // first flag of the job in the batch's masing flags
  DevBuf x0, z0, ri;                                   // camera
  DevBuf tab, nsum, wch, velo, star, lc, scale;        // line tables of the batch precision
  size_t flux_off = 0;                                 // first value in the batch flux array
  size_t arena_off = 0;                                // node records, image, ring sums in the wave arena
  size_t node_bytes = 0, img_bytes = 0, ring_bytes = 0;
};

template <typename T>
struct Wave {
  std::vector<int> jobs;          // job indices, most expensive items first
  size_t bytes = 0;
  DevBuf dgeo, dwalk, dred, dray, ditem, dring, dline;
  JobLaunch<T> L{};
  std::vector<WalkParams<T>> hwalk;   // per-job walk launches, in queue order
  std::vector<int> side;              // stream of each of them
};

template <typename T>
struct Plan {
  std::vector<Wave<T>> waves;
};

}  // namespace

struct rl_batch {
  rl_ctx* ctx = nullptr;
  int precision = RL_FP32;
  std::vector<std::unique_ptr<BatchJob>> jobs;
  size_t nflux = 0;
  double mem_budget = 0.0;       // bytes per wave; 0 = 70% of the free device memory
  int gcap = kItemLines, cpl = 4;
  bool use_graph = true;
  bool built = false;
  bool geo_valid = false;        // node records of a single-wave batch are in the arena
  Plan<float> pf;
  Plan<double> pd;
  DevBuf arena, flux, counters, work, err, list;
  DevBuf jwork;                  // one work counter per job of a wave (per-job walk launches)
  cudaStream_t side[kSideStreams] = {};
  cudaEvent_t fork = nullptr, join[kSideStreams] = {};
  DevBuf maser;                  // [nlines_total] masing flags (jobs with an inverted line)
  bool any_inverted = false;
  double* flux_h = nullptr;
  int* maser_h = nullptr;
  unsigned long long* cnt_h = nullptr;
  int* err_h = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  unsigned long long ray_channels = 0;
  int nlines_total = 0;

  void drop_graph() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    gexec = nullptr; graph = nullptr;
  }
  ~rl_batch() {
    if (ctx) cudaSetDevice(ctx->device);
    drop_graph();
    for (int k = 0; k < kSideStreams; k++) {
      if (side[k]) cudaStreamDestroy(side[k]);
      if (join[k]) cudaEventDestroy(join[k]);
    }
    if (fork) cudaEventDestroy(fork);
    if (flux_h) cudaFreeHost(flux_h);
    if (maser_h) cudaFreeHost(maser_h);
    if (cnt_h) cudaFreeHost(cnt_h);
    if (err_h) cudaFreeHost(err_h);
  }
};

namespace {

// Work items of one job for a line-group cap: balanced groups of at most `gcap` lines.
inline void job_groups(int nl, int gcap, int& ng, int& gsize) {
  ng = (nl + gcap - 1) / gcap;
  gsize = (nl + ng - 1) / ng;
}

template <typename T>
int snapshot_job(rl_batch* b, BatchJob& J) {
  rl_ctx* ctx = b->ctx;
  rl_model* md = J.md;
  const Model& m = md->m;
  int rc = upload_grid(md);
  if (rc) return rc;
  std::string err;
  if (setup_camera(m, md->incl_rad, md->nphi, md->dbdr, md->nrext, J.cam, err)) return set_err(ctx, RL_ERR_ARG, err);
  J.kmax = rlg::max_nodes(m.nr, m.nth);
  J.nfr = m.nfr;
  J.ncell = m.ncell();
  J.aksmax = m.aksmax;
  if (J.nfr >= 2048) return set_err(ctx, RL_ERR_ARG, "at most 2047 channels per line are supported");
  if (J.cam.ri[1] < m.rstar) return set_err(ctx, RL_ERR_ARG, "central beam smaller than the star");
  J.fstar = (m.rstar / J.cam.ri[1]) * (m.rstar / J.cam.ri[1]);
  LineTables<T> lt;
  if (build_line_tables<T>(m, J.iline0, J.nl, lt, err)) return set_err(ctx, RL_ERR_ARG, err);
  J.has_isrf = lt.has_isrf;
  J.inverted = false;
  for (char c : lt.mase) J.inverted = J.inverted || c;
  cudaStream_t s = ctx->stream;
  const Camera& cam = J.cam;
  CUDA_TRY(J.x0.ensure(sizeof(double) * cam.nrays));
  CUDA_TRY(J.z0.ensure(sizeof(double) * cam.nrays));
  CUDA_TRY(J.ri.ensure(sizeof(double) * cam.ri.size()));
  CUDA_TRY(J.tab.ensure(sizeof(T) * lt.tab.size()));
  CUDA_TRY(J.nsum.ensure(sizeof(T) * lt.nsum.size()));
  CUDA_TRY(J.wch.ensure(sizeof(T) * lt.wch.size()));
  CUDA_TRY(J.star.ensure(sizeof(T) * lt.star.size()));
  CUDA_TRY(J.velo.ensure(sizeof(double) * lt.velo.size()));
  CUDA_TRY(J.lc.ensure(sizeof(LineConst<T>) * lt.lc.size()));
  CUDA_TRY(J.scale.ensure(sizeof(double) * lt.scale.size()));
  CUDA_TRY(h2d(J.x0.p, cam.x0.data(), sizeof(double) * cam.nrays, s));
  CUDA_TRY(h2d(J.z0.p, cam.z0.data(), sizeof(double) * cam.nrays, s));
  CUDA_TRY(h2d(J.ri.p, cam.ri.data(), sizeof(double) * cam.ri.size(), s));
  CUDA_TRY(h2d(J.tab.p, lt.tab.data(), sizeof(T) * lt.tab.size(), s));
  CUDA_TRY(h2d(J.nsum.p, lt.nsum.data(), sizeof(T) * lt.nsum.size(), s));
  CUDA_TRY(h2d(J.wch.p, lt.wch.data(), sizeof(T) * lt.wch.size(), s));
  CUDA_TRY(h2d(J.star.p, lt.star.data(), sizeof(T) * lt.star.size(), s));
  CUDA_TRY(h2d(J.velo.p, lt.velo.data(), sizeof(double) * lt.velo.size(), s));
  CUDA_TRY(h2d(J.lc.p, lt.lc.data(), sizeof(LineConst<T>) * lt.lc.size(), s));
  CUDA_TRY(h2d(J.scale.p, lt.scale.data(), sizeof(double) * lt.scale.size(), s));
  CUDA_TRY(cudaStreamSynchronize(s));
  const size_t nn = (size_t)cam.nrays * J.kmax;
  J.node_bytes = 2 * align_up(sizeof(int) * cam.nrays) + 6 * align_up(sizeof(T) * nn) +
                 3 * align_up(sizeof(float) * nn);   // dvf, c00, misc are 4-byte fields
  J.img_bytes = align_up(sizeof(T) * (size_t)J.nl * cam.nrays * J.nfr);
  J.ring_bytes = align_up(sizeof(double) * (size_t)J.nl * (cam.nrr + 1) * J.nfr);
  return 0;
}

// Per-item cost estimate used to order jobs inside a wave (longest first).
inline double item_cost(const BatchJob& J, int gcap) {
  int ng, gs;
  job_groups(J.nl, gcap, ng, gs);
  return (double)gs * J.nfr * J.kmax;
}

template <typename T>
Plan<T>& plan_of(rl_batch* b);
template <> Plan<float>& plan_of<float>(rl_batch* b) { return b->pf; }
template <> Plan<double>& plan_of<double>(rl_batch* b) { return b->pd; }

// Device descriptors of every wave for the current tile shape; all waves share the arena.
template <typename T>
int write_descriptors(rl_batch* b) {
  rl_ctx* ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  Plan<T>& P = plan_of<T>(b);
  char* base = b->arena.as<char>();
  int max_nfr = 0;
  for (auto& J : b->jobs) max_nfr = std::max(max_nfr, J->nfr);
  for (Wave<T>& W : P.waves) {
    std::sort(W.jobs.begin(), W.jobs.end(), [&](int x, int y) {
      return item_cost(*b->jobs[x], b->gcap) > item_cost(*b->jobs[y], b->gcap);
    });
    const int nj = (int)W.jobs.size();
    std::vector<GeoJob<T>> geo(nj);
    std::vector<WalkParams<T>> walk(nj);
    std::vector<RedJob<T>> red(nj);
    std::vector<int> rayp(nj + 1, 0), itemp(nj + 1, 0), ringp(nj + 1, 0), linep(nj + 1, 0);
    // per-job launches: each job to the stream with the least work queued so far (largest
    // jobs first), so that the streams end together
    W.side.assign(nj, 0);
    {
      double load[kSideStreams] = {};
      std::vector<int> order(nj);
      std::iota(order.begin(), order.end(), 0);
      auto job_cost = [&](int q) {
        const BatchJob& J = *b->jobs[W.jobs[q]];
        int ng, gs;
        job_groups(J.nl, b->gcap, ng, gs);
        return (double)ng * J.cam.nrays * item_cost(J, b->gcap);
      };
      std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return job_cost(x) > job_cost(y); });
      for (int q : order) {
        const int k = (int)(std::min_element(load, load + kSideStreams) - load);
        W.side[q] = k;
        load[k] += job_cost(q);
      }
    }
    const size_t list_stride = walk_list_elems(ctx->nsm, max_nfr);
    for (int q = 0; q < nj; q++) {
      BatchJob& J = *b->jobs[W.jobs[q]];
      size_t off = J.arena_off;   // fixed at build time: independent of the queue order
      rl_model* md = J.md;
      const Model& m = md->m;
      const Camera& cam = J.cam;
      const size_t nn = (size_t)cam.nrays * J.kmax;
      auto take = [&](size_t bytes) { char* p = base + off; off += align_up(bytes); return p; };
      NodeBuf<T> nb;
      nb.nrays = cam.nrays; nb.kmax = J.kmax;
      nb.nnodes = (int*)take(sizeof(int) * cam.nrays);
      nb.status = (int*)take(sizeof(int) * cam.nrays);
      nb.ds = (T*)take(sizeof(T) * nn);
      nb.vl = (T*)take(sizeof(T) * nn);
      nb.dvseg = (T*)take(sizeof(T) * nn);
      nb.lw = (T*)take(sizeof(T) * nn);
      nb.wr = (T*)take(sizeof(T) * nn);
      nb.wt = (T*)take(sizeof(T) * nn);
      nb.dvf = (float*)take(sizeof(float) * nn);
      nb.c00 = (int*)take(sizeof(int) * nn);
      nb.misc = (unsigned*)take(sizeof(unsigned) * nn);
      T* img = (T*)take(sizeof(T) * (size_t)J.nl * cam.nrays * J.nfr);
      double* ring = (double*)take(sizeof(double) * (size_t)J.nl * (cam.nrr + 1) * J.nfr);
      GeoParams gp = geo_params(md);
      gp.theta0 = cam.theta0;
      gp.x0 = J.x0.as<double>(); gp.z0 = J.z0.as<double>();
      geo[q].geo = gp;
      geo[q].nb = nb;
      int ng, gs;
      job_groups(J.nl, b->gcap, ng, gs);
      WalkParams<T>& w = walk[q];
      w.nb = nb;
      w.nth = m.nth; w.ncell = J.ncell; w.nlines = J.nl; w.nfr = J.nfr;
      w.gsize = gs; w.nitems = ng * cam.nrays;
      w.tab = J.tab.as<T>(); w.nsum = J.nsum.as<T>(); w.wch = J.wch.as<T>(); w.velo = J.velo.as<double>();
      w.star = J.star.as<T>(); w.lc = J.lc.as<LineConst<T>>();
      w.isrf = isrf_of(J.has_isrf, w.star, J.nl, J.nfr);
      w.aksmax_c = J.aksmax / 2.99792458e5;
      w.kq = (T)(3.33567e-6 * 2.99792458e5);
      w.fstar = (T)J.fstar;
      w.img = img;
      w.counters = b->counters.as<unsigned long long>();
      w.work = b->jwork.as<int>() + q;              // the per-job launch's own queue
      w.err = b->err.as<int>();
      w.list = b->list.as<unsigned short>() + list_stride * W.side[q];   // its stream's list rows
      w.maser = J.inverted ? b->maser.as<int>() + J.line_off : nullptr;
      RedJob<T>& r = red[q];
      r.p.nrays = cam.nrays; r.p.nfr = J.nfr; r.p.nphi = cam.nphi; r.p.nrr = cam.nrr; r.p.nlines = J.nl;
      r.p.ri = J.ri.as<double>(); r.p.dist2 = 3.08572e18 * 3.08572e18; r.p.scale = J.scale.as<double>();
      r.img = img; r.ring = ring; r.flux = b->flux.as<double>() + J.flux_off;
      rayp[q + 1] = rayp[q] + cam.nrays;
      itemp[q + 1] = itemp[q] + w.nitems;
      ringp[q + 1] = ringp[q] + J.nl * cam.nrr;
      linep[q + 1] = linep[q] + J.nl;
    }
    CUDA_TRY(W.dgeo.ensure(sizeof(GeoJob<T>) * nj));
    CUDA_TRY(W.dwalk.ensure(sizeof(WalkParams<T>) * nj));
    CUDA_TRY(W.dred.ensure(sizeof(RedJob<T>) * nj));
    CUDA_TRY(W.dray.ensure(sizeof(int) * (nj + 1)));
    CUDA_TRY(W.ditem.ensure(sizeof(int) * (nj + 1)));
    CUDA_TRY(W.dring.ensure(sizeof(int) * (nj + 1)));
    CUDA_TRY(W.dline.ensure(sizeof(int) * (nj + 1)));
    CUDA_TRY(h2d(W.dgeo.p, geo.data(), sizeof(GeoJob<T>) * nj, s));
    CUDA_TRY(h2d(W.dwalk.p, walk.data(), sizeof(WalkParams<T>) * nj, s));
    CUDA_TRY(h2d(W.dred.p, red.data(), sizeof(RedJob<T>) * nj, s));
    CUDA_TRY(h2d(W.dray.p, rayp.data(), sizeof(int) * (nj + 1), s));
    CUDA_TRY(h2d(W.ditem.p, itemp.data(), sizeof(int) * (nj + 1), s));
    CUDA_TRY(h2d(W.dring.p, ringp.data(), sizeof(int) * (nj + 1), s));
    CUDA_TRY(h2d(W.dline.p, linep.data(), sizeof(int) * (nj + 1), s));
    JobLaunch<T>& L = W.L;
    L.njobs = nj; L.nsm = ctx->nsm; L.cpl = b->cpl;
    L.geo = static_cast<GeoJob<T>*>(W.dgeo.p); L.ray_prefix = static_cast<int*>(W.dray.p); L.nrays_total = rayp[nj];
    L.walk.jobs = static_cast<WalkParams<T>*>(W.dwalk.p); L.walk.item_prefix = static_cast<int*>(W.ditem.p);
    L.walk.njobs = nj; L.walk.total = itemp[nj]; L.walk.stride = 1; L.walk.max_nfr = max_nfr;
    L.walk.work = b->work.as<int>(); L.walk.counters = b->counters.as<unsigned long long>();
    L.walk.list = b->list.as<unsigned short>();
    L.reduce = true;
    L.red = static_cast<RedJob<T>*>(W.dred.p); L.ring_prefix = static_cast<int*>(W.dring.p); L.line_prefix = static_cast<int*>(W.dline.p);
    L.nring_blocks = ringp[nj]; L.nline_blocks = linep[nj];
    W.hwalk = walk;
  }
  CUDA_TRY(cudaStreamSynchronize(s));
  b->drop_graph();
  return 0;
}

// Snapshot every job, split them into waves that fit the memory budget, allocate.
template <typename T>
int build(rl_batch* b) {
  rl_ctx* ctx = b->ctx;
  if (b->jobs.empty()) return set_err(ctx, RL_ERR_STATE, "rl_batch: no jobs");
  b->nflux = 0;
  b->ray_channels = 0;
  b->nlines_total = 0;
  for (auto& J : b->jobs) {
    int rc = snapshot_job<T>(b, *J);
    if (rc) return rc;
    J->flux_off = b->nflux;
    J->line_off = b->nlines_total;
    b->nflux += (size_t)J->nl * J->nfr;
    b->ray_channels += (unsigned long long)J->cam.nrays * J->nfr * J->nl;
    b->nlines_total += J->nl;
  }
  size_t budget = (size_t)b->mem_budget;
  if (budget == 0) {
    size_t fr = 0, tot = 0;
    CUDA_TRY(cudaMemGetInfo(&fr, &tot));
    budget = (size_t)(0.7 * (double)fr);
  }
  Plan<T>& P = plan_of<T>(b);
  P.waves.clear();
  P.waves.emplace_back();
  size_t arena = 0;
  for (int j = 0; j < (int)b->jobs.size(); j++) {
    const BatchJob& J = *b->jobs[j];
    const size_t need = J.node_bytes + J.img_bytes + J.ring_bytes;
    if (!P.waves.back().jobs.empty() && P.waves.back().bytes + need > budget) P.waves.emplace_back();
    P.waves.back().jobs.push_back(j);
    b->jobs[j]->arena_off = P.waves.back().bytes;
    P.waves.back().bytes += need;
    arena = std::max(arena, P.waves.back().bytes);
  }
  CUDA_TRY(b->arena.ensure(arena));
  CUDA_TRY(b->flux.ensure(sizeof(double) * b->nflux));
  CUDA_TRY(b->counters.ensure(sizeof(unsigned long long) * kWalkCounters));
  CUDA_TRY(b->work.ensure(sizeof(int)));
  CUDA_TRY(b->err.ensure(sizeof(int)));
  b->any_inverted = false;
  for (auto& J : b->jobs) b->any_inverted = b->any_inverted || J->inverted;
  CUDA_TRY(b->maser.ensure(sizeof(int) * std::max(1, b->nlines_total)));
  if (b->maser_h) { cudaFreeHost(b->maser_h); b->maser_h = nullptr; }
  CUDA_TRY(cudaMallocHost((void**)&b->maser_h, sizeof(int) * std::max(1, b->nlines_total)));
  std::memset(b->maser_h, 0, sizeof(int) * std::max(1, b->nlines_total));
  {
    int max_nfr = 0;
    for (auto& J : b->jobs) max_nfr = std::max(max_nfr, J->nfr);
    CUDA_TRY(b->list.ensure(sizeof(unsigned short) * walk_list_elems(ctx->nsm, max_nfr) * kSideStreams));
  }
  {
    size_t maxj = 1;
    for (const Wave<T>& W : P.waves) maxj = std::max(maxj, W.jobs.size());
    CUDA_TRY(b->jwork.ensure(sizeof(int) * maxj));
  }
  for (int k = 0; k < kSideStreams; k++) {
    if (!b->side[k]) CUDA_TRY(cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking));
    if (!b->join[k]) CUDA_TRY(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
  }
  if (!b->fork) CUDA_TRY(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  if (b->flux_h) { cudaFreeHost(b->flux_h); b->flux_h = nullptr; }
  CUDA_TRY(cudaMallocHost((void**)&b->flux_h, sizeof(double) * b->nflux));
  if (!b->cnt_h) CUDA_TRY(cudaMallocHost((void**)&b->cnt_h, sizeof(unsigned long long) * kWalkCounters));
  if (!b->err_h) CUDA_TRY(cudaMallocHost((void**)&b->err_h, sizeof(int)));
  int rc = write_descriptors<T>(b);
  if (rc) return rc;
  b->built = true;
  b->geo_valid = false;
  return 0;
}

// The launch sequence of one batch run (also the body of the captured graph). A batch
// whose jobs fit one wave keeps its node records in the arena after the first run, like
// a model keeps its camera geometry, and skips the geometry launch afterwards.
template <typename T>
cudaError_t enqueue(rl_batch* b, cudaStream_t s, bool skip_geometry) {
  cudaError_t e = cudaMemsetAsync(b->counters.p, 0, sizeof(unsigned long long) * kWalkCounters, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->err.p, 0, sizeof(int), s);
  if (e == cudaSuccess && b->any_inverted) e = cudaMemsetAsync(b->maser.p, 0, sizeof(int) * b->nlines_total, s);
  for (Wave<T>& W : plan_of<T>(b).waves) {
    if (e != cudaSuccess) return e;
    JobLaunch<T> L = W.L;
    if (!skip_geometry) {   // the geometry of every job of the wave in one launch
      L.walk_jobs = false;
      L.reduce = false;
      e = launch_jobs<T>(L, s);
      if (e != cudaSuccess) return e;
    }
    // one walk launch per job (the single-model kernel), spread over the side streams
    const int nj = (int)W.hwalk.size();
    e = cudaMemsetAsync(b->jwork.p, 0, sizeof(int) * nj, s);
    if (e == cudaSuccess) e = cudaEventRecord(b->fork, s);
    for (int k = 0; k < kSideStreams && e == cudaSuccess; k++) e = cudaStreamWaitEvent(b->side[k], b->fork, 0);
    for (int q = 0; q < nj && e == cudaSuccess; q++) e = launch_walk<T>(W.hwalk[q], b->cpl, L.nsm, b->side[W.side[q]]);
    for (int k = 0; k < kSideStreams && e == cudaSuccess; k++) {
      e = cudaEventRecord(b->join[k], b->side[k]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, b->join[k], 0);
    }
    if (e != cudaSuccess) return e;
    L.nrays_total = 0;
    L.walk_jobs = false;
    L.reduce = true;
    e = launch_jobs<T>(L, s);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->flux_h, b->flux.p, sizeof(double) * b->nflux, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->cnt_h, b->counters.p, sizeof(unsigned long long) * kWalkCounters, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->err_h, b->err.p, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && b->any_inverted)
    e = cudaMemcpyAsync(b->maser_h, b->maser.p, sizeof(int) * b->nlines_total, cudaMemcpyDeviceToHost, s);
  return e;
}

template <typename T>
int run(rl_batch* b, double* flux_out, rl_stats* st) {
  rl_ctx* ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  if (!b->built) {
    int rc = build<T>(b);
    if (rc) return rc;
  }
  const bool single = plan_of<T>(b).waves.size() == 1;
  const bool first = single && !b->geo_valid;     // computes the node records once
  CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
  if (first) {
    b->drop_graph();
    CUDA_TRY(enqueue<T>(b, s, false));
  } else if (b->use_graph) {
    if (!b->gexec) {
      cudaGraph_t g = nullptr;
      CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
      cudaError_t e = enqueue<T>(b, s, single);
      cudaError_t e2 = cudaStreamEndCapture(s, &g);
      if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return set_err(ctx, RL_ERR_CUDA, std::string("rl_batch: graph capture: ") +
                                              cudaGetErrorString(e != cudaSuccess ? e : e2));
      }
      b->graph = g;
      CUDA_TRY(cudaGraphInstantiate(&b->gexec, b->graph, 0));
    }
    CUDA_TRY(cudaGraphLaunch(b->gexec, s));
  } else {
    CUDA_TRY(enqueue<T>(b, s, single));
  }
  CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
  CUDA_TRY(cudaStreamSynchronize(s));
  g_d2h += sizeof(double) * b->nflux + sizeof(unsigned long long) * kWalkCounters + sizeof(int) +
           (b->any_inverted ? sizeof(int) * b->nlines_total : 0);
  if (*b->err_h != 0) {
    b->geo_valid = false;
    return set_err(ctx, RL_ERR_GEOMETRY, "rl_batch: walk error code " + std::to_string(*b->err_h));
  }
  if (first) b->geo_valid = true;
  if (flux_out) std::memcpy(flux_out, b->flux_h, sizeof(double) * b->nflux);
  if (st) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    st->walk_ms += ms;
    st->total_ms += ms;
    st->steps += b->cnt_h[0]; st->integrated += b->cnt_h[1]; st->node_visits += b->cnt_h[2];
    st->node_passes += b->cnt_h[3]; st->packed_passes += b->cnt_h[4]; st->empty_steps += b->cnt_h[5];
    st->refined_passes += b->cnt_h[6]; st->sub_steps += b->cnt_h[7];
    st->refined_channels += b->cnt_h[8];
    st->ray_channels += b->ray_channels;
    st->nlines += b->nlines_total;
  }
  return 0;
}

// Times the walk of wave 0 on every stride-th item for each candidate (line-group cap,
// channel slots) and keeps the fastest. Geometry of wave 0 is computed once first.
template <typename T>
int autotune(rl_batch* b, int stride, int* gbest, int* cbest, double* best_ms) {
  rl_ctx* ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  if (!b->built) {
    int rc = build<T>(b);
    if (rc) return rc;
  }
  Plan<T>& P = plan_of<T>(b);
  {
    JobLaunch<T> L = P.waves[0].L;
    L.reduce = false;
    L.walk.total = 0;                       // geometry only
    CUDA_TRY(cudaMemsetAsync(b->err.p, 0, sizeof(int), s));
    CUDA_TRY(launch_jobs<T>(L, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    b->geo_valid = false;   // the first run recomputes it with the final tile shape in place
  }
  int maxnl = 1;
  for (int j : P.waves[0].jobs) maxnl = std::max(maxnl, b->jobs[j]->nl);
  // the walk steps four slots per lane together, so fewer slots per tile leave
  // lanes of every pass empty, and eight need more shared memory than four 4-warp blocks
  // per SM leave beside the 12-line stage: the tuner varies the lines per item only
  const int gc[] = {2, 8, 16, kItemLines};
  const int cc[] = {4};
  // A sample of few items ends in a tail that the full walk does not have, so the default
  // shape (32 lines, 4 slots) keeps its place unless another shape beats it by 2%.
  double best = 1e300, best_score = 1e300;
  int bg = b->gcap, bc = b->cpl;
  for (int g : gc) {
    if (g > maxnl && g != gc[0]) continue;
    for (int c : cc) {
      b->gcap = g; b->cpl = c;
      int rc = write_descriptors<T>(b);
      if (rc) return rc;
      JobLaunch<T> L = P.waves[0].L;
      L.nrays_total = 0;                    // geometry already in place
      L.reduce = false;
      L.walk.stride = std::max(1, stride);
      float ms = 0.f;
      for (int rep = 0; rep < 2; rep++) {   // first repetition warms up
        CUDA_TRY(cudaMemsetAsync(b->counters.p, 0, sizeof(unsigned long long) * kWalkCounters, s));
        CUDA_TRY(cudaEventRecord(ctx->ev[0], s));
        CUDA_TRY(launch_jobs<T>(L, s));
        CUDA_TRY(cudaEventRecord(ctx->ev[1], s));
        CUDA_TRY(cudaStreamSynchronize(s));
        cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
      }
      const double score = (g == kItemLines && c == 4) ? 0.98 * ms : ms;
      if (score < best_score) { best_score = score; best = ms; bg = g; bc = c; }
    }
  }
  b->gcap = bg; b->cpl = bc;
  int rc = write_descriptors<T>(b);
  if (rc) return rc;
  if (gbest) *gbest = bg;
  if (cbest) *cbest = bc;
  if (best_ms) *best_ms = best;
  return 0;
}

}  // namespace

extern "C" {

int rl_batch_create(rl_ctx* ctx, int precision, rl_batch** out) {
  if (!ctx || !out) return set_err(ctx, RL_ERR_ARG, "rl_batch_create: null argument");
  if (precision != RL_FP32 && precision != RL_FP64) return set_err(ctx, RL_ERR_ARG, "rl_batch_create: precision");
  *out = nullptr;
  std::unique_ptr<rl_batch> b(new rl_batch);
  b->ctx = ctx;
  b->precision = precision;
  *out = b.release();
  return 0;
}

int rl_batch_destroy(rl_batch* b) {
  delete b;
  return 0;
}

int rl_batch_add(rl_batch* b, rl_model* md, int iline0, int nlines) {
  if (!b || !md) return set_err(b ? b->ctx : nullptr, RL_ERR_ARG, "rl_batch_add: null argument");
  rl_ctx* ctx = b->ctx;
  if (md->ctx != ctx) return set_err(ctx, RL_ERR_ARG, "rl_batch_add: model belongs to another context");
  if (nlines < 1 || iline0 < 1 || iline0 + nlines - 1 > (int)md->m.lfreq.size())
    return set_err(ctx, RL_ERR_ARG, "rl_batch_add: line range outside the molecule's line list");
  std::unique_ptr<BatchJob> J(new BatchJob);
  J->md = md; J->iline0 = iline0; J->nl = nlines;
  b->jobs.push_back(std::move(J));
  b->built = false;
  b->drop_graph();
  return (int)b->jobs.size() - 1;
}

int rl_batch_set_memory(rl_batch* b, double bytes) {
  if (!b || bytes < 0) return set_err(b ? b->ctx : nullptr, RL_ERR_ARG, "rl_batch_set_memory: bad argument");
  b->mem_budget = bytes;
  b->built = false;
  b->drop_graph();
  return 0;
}

int rl_batch_set_tiles(rl_batch* b, int lines_per_item, int channel_slots) {
  if (!b) return set_err(nullptr, RL_ERR_ARG, "rl_batch_set_tiles: null batch");
  if (lines_per_item < 1 || lines_per_item > kItemLines ||
      (channel_slots != 1 && channel_slots != 2 && channel_slots != 4 && channel_slots != 8))
    return set_err(b->ctx, RL_ERR_ARG, "rl_batch_set_tiles: lines_per_item 1..32, channel_slots 1, 2, 4 or 8");
  b->gcap = lines_per_item;
  b->cpl = channel_slots;
  if (!b->built) return 0;
  rl_ctx* ctx = b->ctx;
  CUDA_TRY(rl::enter_device(ctx->device));
  return b->precision == RL_FP64 ? write_descriptors<double>(b) : write_descriptors<float>(b);
}

int rl_batch_get_tiles(rl_batch* b, int* lines_per_item, int* channel_slots) {
  if (!b || !lines_per_item || !channel_slots) return set_err(nullptr, RL_ERR_ARG, "rl_batch_get_tiles: null argument");
  *lines_per_item = b->gcap;
  *channel_slots = b->cpl;
  return 0;
}

int rl_batch_use_graph(rl_batch* b, int enable) {
  if (!b) return set_err(nullptr, RL_ERR_ARG, "rl_batch_use_graph: null batch");
  b->use_graph = enable != 0;
  return 0;
}

int rl_batch_autotune(rl_batch* b, int sample_stride, int* lines_per_item, int* channel_slots, double* sample_ms) {
  if (!b) return set_err(nullptr, RL_ERR_ARG, "rl_batch_autotune: null batch");
  rl_ctx* ctx = b->ctx;
  CUDA_TRY(rl::enter_device(ctx->device));
  g_h2d = 0; g_d2h = 0;
  return b->precision == RL_FP64 ? autotune<double>(b, sample_stride, lines_per_item, channel_slots, sample_ms)
                                 : autotune<float>(b, sample_stride, lines_per_item, channel_slots, sample_ms);
}

int rl_batch_flux_size(rl_batch* b, long long* n) {
  if (!b || !n) return set_err(nullptr, RL_ERR_ARG, "rl_batch_flux_size: null argument");
  long long t = 0;
  for (auto& J : b->jobs) t += (long long)J->nl * J->md->m.nfr;
  *n = t;
  return 0;
}

int rl_batch_job_info(rl_batch* b, int job, long long* flux_offset, int* nlines, int* nfr) {
  if (!b || job < 0 || job >= (int)b->jobs.size()) return set_err(b ? b->ctx : nullptr, RL_ERR_ARG, "rl_batch_job_info: bad job");
  long long off = 0;
  for (int j = 0; j < job; j++) off += (long long)b->jobs[j]->nl * b->jobs[j]->md->m.nfr;
  if (flux_offset) *flux_offset = off;
  if (nlines) *nlines = b->jobs[job]->nl;
  if (nfr) *nfr = b->jobs[job]->md->m.nfr;
  return 0;
}

int rl_batch_run(rl_batch* b, double* flux_out, rl_stats* st) {
  if (!b) return set_err(nullptr, RL_ERR_ARG, "rl_batch_run: null batch");
  rl_ctx* ctx = b->ctx;
  CUDA_TRY(rl::enter_device(ctx->device));
  if (st) std::memset(st, 0, sizeof *st);
  g_h2d = 0; g_d2h = 0;
  const int rc = b->precision == RL_FP64 ? run<double>(b, flux_out, st) : run<float>(b, flux_out, st);
  if (st) { st->h2d_bytes += g_h2d; st->d2h_bytes += g_d2h; }
  return rc;
}

int rl_run_manifest(const char* manifest, int device, rl_stats* st) {
  if (!manifest) return set_err(nullptr, RL_ERR_ARG, "rl_run_manifest: null manifest");
  std::vector<std::string> dirs;
  {
    FILE* fp = std::fopen(manifest, "r");
    if (!fp) return set_err(nullptr, RL_ERR_IO, std::string("cannot open manifest ") + manifest);
    char buf[4096];
    while (std::fgets(buf, sizeof buf, fp)) {
      std::string d(buf);
      while (!d.empty() && (d.back() == '\n' || d.back() == '\r' || d.back() == ' ' || d.back() == '\t')) d.pop_back();
      size_t a = 0;
      while (a < d.size() && (d[a] == ' ' || d[a] == '\t')) a++;
      d = d.substr(a);
      if (!d.empty() && d[0] != '#') dirs.push_back(d);
    }
    std::fclose(fp);
  }
  if (dirs.empty()) return set_err(nullptr, RL_ERR_ARG, std::string("manifest lists no directories: ") + manifest);
  rl_ctx* ctx = nullptr;
  int rc = rl_create(&ctx, device);
  if (rc) return rc;
  std::vector<rl_model*> models(dirs.size(), nullptr);
  rl_batch* b = nullptr;
  rc = rl_batch_create(ctx, RL_FP32, &b);
  for (size_t i = 0; i < dirs.size() && rc == 0; i++) {
    rc = rl_load_dir(ctx, dirs[i].c_str(), &models[i]);
    if (rc) { set_err(ctx, rc, dirs[i] + ": " + ctx->err); break; }
    const Model& m = models[i]->m;
    if (m.command != 0) {
      rc = set_err(ctx, RL_ERR_ARG, dirs[i] + ": a batch renders line spectra (command 0); run position-velocity "
                                              "directories one by one");
      break;
    }
    const int job = rl_batch_add(b, models[i], m.ilstart, m.nlspec);
    if (job < 0) rc = job;
  }
  std::vector<double> flux;
  if (rc == 0) {
    long long n = 0;
    rl_batch_flux_size(b, &n);
    flux.assign((size_t)n, 0.0);
    rc = rl_batch_run(b, flux.data(), st);
  }
  for (size_t i = 0; i < dirs.size() && rc == 0; i++) {
    const BatchJob& J = *b->jobs[i];
    const Model& m = models[i]->m;
    std::vector<int> det(J.nl, 0);
    rl_batch_job_masing(b, (int)i, det.data());
    for (int l = 0; l < J.nl; l++)
      if (det[l]) std::printf("          WARNING: Masing detected!\n Will only warn once for this transition.\n");
    std::fflush(stdout);
    std::vector<int> lines;
    for (int l = 0; l < m.nlspec; l++) lines.push_back(m.ilstart + l);
    std::vector<double> f(flux.begin() + J.flux_off, flux.begin() + J.flux_off + (size_t)J.nl * J.nfr);
    std::string err;
    if (write_spectrum_file(dirs[i] + "/linespectrum_" + m.molname + ".dat", m, J.cam, lines, f, err)) {
      rc = set_err(ctx, RL_ERR_IO, err);
      break;
    }
    FILE* fp = std::fopen((dirs[i] + "/radlite.success").c_str(), "w");
    if (fp) { std::fprintf(fp, " 1\n"); std::fclose(fp); }
  }
  if (rc) g_last_error = ctx->err;
  rl_batch_destroy(b);
  for (rl_model* md : models) rl_model_free(md);
  rl_destroy(ctx);
  return rc;
}

int rl_batch_job_masing(rl_batch* b, int job, int* detected) {
  if (!b || !detected) return set_err(nullptr, RL_ERR_ARG, "rl_batch_job_masing: null argument");
  if (job < 0 || job >= (int)b->jobs.size()) return set_err(b->ctx, RL_ERR_ARG, "rl_batch_job_masing: job index");
  const BatchJob& J = *b->jobs[job];
  for (int l = 0; l < J.nl; l++) detected[l] = (b->built && J.inverted && b->maser_h) ? (b->maser_h[J.line_off + l] != 0) : 0;
  return 0;
}

int rl_batch_waves(rl_batch* b, int* nwaves) {
  if (!b || !nwaves) return set_err(nullptr, RL_ERR_ARG, "rl_batch_waves: null argument");
  *nwaves = (int)(b->precision == RL_FP64 ? b->pd.waves.size() : b->pf.waves.size());
  return 0;
}

}  // extern "C"
