// fau_chain_256_ph.cu -- chain kernel instantiations: 256 threads per chain, device (Philox) proposals.
#include "fau_chain.cuh"

namespace fau {

cudaError_t chain_dispatch_256_ph(const ChainArgs& a, int nb, int K, int nc, int kpt, cudaStream_t st, bool prep)
{
    switch (kpt) {
    case 1: return launch_chain_inst<256, 1, true>(a, nb, K, nc, st, prep);
    case 2: return launch_chain_inst<256, 2, true>(a, nb, K, nc, st, prep);
    case 3: return launch_chain_inst<256, 3, true>(a, nb, K, nc, st, prep);
    case 5: return launch_chain_inst<256, 5, true>(a, nb, K, nc, st, prep);
    case 8: return launch_chain_inst<256, 8, true>(a, nb, K, nc, st, prep);
    case 12: return launch_chain_inst<256, 12, true>(a, nb, K, nc, st, prep);
    case 18: return launch_chain_inst<256, 18, true>(a, nb, K, nc, st, prep);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace fau
