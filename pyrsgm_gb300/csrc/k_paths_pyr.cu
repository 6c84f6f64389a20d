// k_paths_pyr.cu -- pyramid-level instantiations of the aggregation kernels.
#include "k_paths.cuh"

namespace pg {

template cudaError_t launch_paths_mode<true, 1>(const Jobs<1>&, const LevelExtent&, cudaStream_t);
template cudaError_t launch_paths_mode<true, kBatchJobs>(const Jobs<kBatchJobs>&, const LevelExtent&, cudaStream_t);

}  // namespace pg
