// fau_mol_512.cu -- pipelined molecular-move kernel instantiation: 512 threads (1 preparing + 15
// compute warps, one CTA an SM), device proposals: a single chain's moves take less time, for
// launches of few molecular chains (the long jobs of a served stream).
#include "fau_mol.cuh"

namespace fau {

cudaError_t mol_dispatch_512(const ChainArgs& a, int nb, int K, int nc, cudaStream_t st, bool prep)
{
    return launch_mol_inst<512, 1, false>(a, nb, K, nc, st, prep);
}

} // namespace fau
