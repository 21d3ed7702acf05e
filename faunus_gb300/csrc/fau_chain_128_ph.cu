// fau_chain_128_ph.cu -- chain kernel instantiation: 128 threads per chain, device (Philox) proposals.
#include "fau_chain.cuh"

namespace fau {

cudaError_t chain_dispatch_128_ph(const ChainArgs& a, int nb, int K, int nc, cudaStream_t st, bool prep)
{
    return launch_chain_inst<128, true>(a, nb, K, nc, st, prep);
}

} // namespace fau
