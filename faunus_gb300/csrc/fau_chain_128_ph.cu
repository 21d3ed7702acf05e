// fau_chain_128_ph.cu -- chain kernel instantiations: 128 threads per chain, device (Philox) proposals.
#include "fau_chain.cuh"

namespace fau {

cudaError_t chain_dispatch_128_ph(const ChainArgs& a, int nb, int K, int nc, int kpt, cudaStream_t st, bool prep)
{
    switch (kpt) {
    case 1: return launch_chain_inst<128, 1, true>(a, nb, K, nc, st, prep);
    case 2: return launch_chain_inst<128, 2, true>(a, nb, K, nc, st, prep);
    case 4: return launch_chain_inst<128, 4, true>(a, nb, K, nc, st, prep);
    case 6: return launch_chain_inst<128, 6, true>(a, nb, K, nc, st, prep);
    case 9: return launch_chain_inst<128, 9, true>(a, nb, K, nc, st, prep);
    case 12: return launch_chain_inst<128, 12, true>(a, nb, K, nc, st, prep);
    case 18: return launch_chain_inst<128, 18, true>(a, nb, K, nc, st, prep);
    case 24: return launch_chain_inst<128, 24, true>(a, nb, K, nc, st, prep);
    case 36: return launch_chain_inst<128, 36, true>(a, nb, K, nc, st, prep);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace fau
