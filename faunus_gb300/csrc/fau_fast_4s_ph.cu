// fau_fast_4s_ph.cu -- pipelined chain kernel instantiation: 1 producer + 4 compute warps, device (Philox) proposals,
// cell lists staged by their occupied slots only.
#include "fau_fast.cuh"

namespace fau {

cudaError_t fast_dispatch_4_ph_sparse(const ChainArgs& a, int nb, int K, int nc, int nt, cudaStream_t st, bool prep)
{
    return launch_fast_inst<4, true, true>(a, nb, K, nc, nt, st, prep);
}

} // namespace fau
