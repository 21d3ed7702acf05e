// fau_fast_2_host.cu -- pipelined chain kernel instantiation: 1 producer + 2 compute warps, host proposals.
#include "fau_fast.cuh"

namespace fau {

cudaError_t fast_dispatch_2_host(const ChainArgs& a, int nb, int K, int nc, int nt, cudaStream_t st, bool prep)
{
    return launch_fast_inst<2, false>(a, nb, K, nc, nt, st, prep);
}

} // namespace fau
