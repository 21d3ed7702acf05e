// fau_chain_256_ph.cu -- chain kernel instantiation: 256 threads per chain, device (Philox) proposals.
#include "fau_chain.cuh"

namespace fau {

cudaError_t chain_dispatch_256_ph(const ChainArgs& a, int nb, int K, int nc, cudaStream_t st, bool prep)
{
    return launch_chain_inst<256, true>(a, nb, K, nc, st, prep);
}

} // namespace fau
