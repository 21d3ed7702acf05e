// fau_fast_2_ph.cu -- pipelined chain kernel instantiation: 1 producer + 2 compute warps, device (Philox) proposals.
#include "fau_fast.cuh"

namespace fau {

cudaError_t fast_dispatch_2_ph(const ChainArgs& a, int nb, int K, int nc, int nt, cudaStream_t st, bool prep)
{
    return launch_fast_inst<2, true>(a, nb, K, nc, nt, st, prep);
}

} // namespace fau
