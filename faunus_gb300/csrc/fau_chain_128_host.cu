// fau_chain_128_host.cu -- chain kernel instantiations: 128 threads per chain, host-fed proposals.
#include "fau_chain.cuh"

namespace fau {

cudaError_t chain_dispatch_128_host(const ChainArgs& a, int nb, int K, int nc, int kpt, cudaStream_t st, bool prep)
{
    switch (kpt) {
    case 1: return launch_chain_inst<128, 1, false>(a, nb, K, nc, st, prep);
    case 2: return launch_chain_inst<128, 2, false>(a, nb, K, nc, st, prep);
    case 4: return launch_chain_inst<128, 4, false>(a, nb, K, nc, st, prep);
    case 6: return launch_chain_inst<128, 6, false>(a, nb, K, nc, st, prep);
    case 9: return launch_chain_inst<128, 9, false>(a, nb, K, nc, st, prep);
    case 12: return launch_chain_inst<128, 12, false>(a, nb, K, nc, st, prep);
    case 18: return launch_chain_inst<128, 18, false>(a, nb, K, nc, st, prep);
    case 24: return launch_chain_inst<128, 24, false>(a, nb, K, nc, st, prep);
    case 36: return launch_chain_inst<128, 36, false>(a, nb, K, nc, st, prep);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace fau
