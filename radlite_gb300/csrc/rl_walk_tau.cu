// rl_walk_tau.cu -- the walk instances that keep each integrated channel's optical depth
// (the forward of the differentiable path when its backward is the gradient sweep). A
// translation unit of its own, so that they compile beside the plain ones.
#include "rl_walk_launch.cuh"

namespace rl {

template <typename T>
cudaError_t launch_walk_tau(const WalkParams<T>& P, int cpl, int nsm, cudaStream_t s) {
  return launch_walk_t<T, true>(P, cpl, nsm, s);
}

template <typename T>
cudaError_t launch_walk_jobs_tau(const WalkJobs<T>& B, int cpl, int nsm, cudaStream_t s) {
  return launch_walk_jobs_t<T, true>(B, cpl, nsm, s);
}

template cudaError_t launch_walk_tau<float>(const WalkParams<float>&, int, int, cudaStream_t);
template cudaError_t launch_walk_tau<double>(const WalkParams<double>&, int, int, cudaStream_t);
template cudaError_t launch_walk_jobs_tau<float>(const WalkJobs<float>&, int, int, cudaStream_t);
template cudaError_t launch_walk_jobs_tau<double>(const WalkJobs<double>&, int, int, cudaStream_t);

}  // namespace rl
