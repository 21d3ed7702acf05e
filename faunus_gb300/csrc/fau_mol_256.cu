// fau_mol_256.cu -- pipelined molecular-move kernel instantiation: 256 threads (1 + 7 warps).
#include "fau_mol.cuh"

#include <cstdlib>

namespace fau {

// resident CTAs per SM the register allocation is sized for (FAU_MOL_MINB: 2, 3 or 4)
static int mol_minb()
{
    static int v = [] {
        const char* e = std::getenv("FAU_MOL_MINB");
        const int x = e ? std::atoi(e) : 2;
        return (x == 3 || x == 4) ? x : 2;
    }();
    return v;
}

cudaError_t mol_dispatch_256(const ChainArgs& a, int nb, int K, int nc, cudaStream_t st, bool prep)
{
    switch (mol_minb()) {
    case 3: return launch_mol_inst<256, 3>(a, nb, K, nc, st, prep);
    case 4: return launch_mol_inst<256, 4>(a, nb, K, nc, st, prep);
    default: return launch_mol_inst<256, 2>(a, nb, K, nc, st, prep);
    }
}

size_t mol_smem_bytes_total(int K, int nc)
{
    return mol_smem_bytes(K, nc);
}

} // namespace fau
