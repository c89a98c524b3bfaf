// rl_walk_chk.cu -- the walk instances that also take the reference's overshoot test on
// every step (transfer.F:1548-1553) and count the steps that fail it; the RADlite_gpu run
// uses them, as the reference's default build has the test compiled in. Their results
// equal the plain walk's. A translation unit of its own, so that they compile beside the
// plain ones.
#include "rl_walk_launch.cuh"

namespace rl {

template <typename T>
cudaError_t launch_walk_chk(const WalkParams<T>& P, int cpl, int nsm, cudaStream_t s) {
  return launch_walk_t<T, false, true>(P, cpl, nsm, s);
}

template cudaError_t launch_walk_chk<float>(const WalkParams<float>&, int, int, cudaStream_t);
template cudaError_t launch_walk_chk<double>(const WalkParams<double>&, int, int, cudaStream_t);

}  // namespace rl
