// fau_chain_256_host.cu -- chain kernel instantiation: 256 threads per chain, host-fed proposals.
#include "fau_chain.cuh"

namespace fau {

cudaError_t chain_dispatch_256_host(const ChainArgs& a, int nb, int K, int nc, cudaStream_t st, bool prep)
{
    return launch_chain_inst<256, false>(a, nb, K, nc, st, prep);
}

} // namespace fau
