// fau_mol_256.cu -- pipelined molecular-move kernel instantiation: 256 threads (1 + 7 warps).
#include "fau_mol.cuh"

namespace fau {

cudaError_t mol_dispatch_256(const ChainArgs& a, int nb, int K, int nc, cudaStream_t st, bool prep)
{
    return launch_mol_inst<256>(a, nb, K, nc, st, prep);
}

size_t mol_smem_bytes_total(int K, int nc)
{
    return mol_smem_bytes(K, nc);
}

} // namespace fau
