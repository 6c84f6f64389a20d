// k_paths_pyr.cu -- pyramid-level instantiations of the aggregation kernels.
#include "k_paths.cuh"

namespace pg {

template cudaError_t launch_paths_mode<true, 1>(const Jobs<1>&, const LevelExtent&, cudaStream_t);
template cudaError_t launch_paths_mode<true, kBatchJobs>(const Jobs<kBatchJobs>&, const LevelExtent&, cudaStream_t);

}  // namespace pg

extern "C" unsigned pyrsgm_gb300_fused_stalls(int reset)
{
    unsigned v = 0;
    if (cudaMemcpyFromSymbol(&v, pg::g_fused_stalls, sizeof v) != cudaSuccess) return 0xffffffffu;
    if (reset) {
        const unsigned z = 0;
        if (cudaMemcpyToSymbol(pg::g_fused_stalls, &z, sizeof z) != cudaSuccess) return 0xffffffffu;
    }
    return v;
}
