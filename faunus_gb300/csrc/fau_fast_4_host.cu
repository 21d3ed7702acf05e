// fau_fast_4_host.cu -- pipelined chain kernel instantiation: 1 producer + 4 compute warps, host proposals,
// whole cells only (launches with no system flagged for occupied-slot staging).
#include "fau_fast.cuh"

namespace fau {

cudaError_t fast_dispatch_4_host(const ChainArgs& a, int nb, int K, int nc, int nt, cudaStream_t st, bool prep)
{
    return launch_fast_inst<4, false, false>(a, nb, K, nc, nt, st, prep);
}

} // namespace fau
