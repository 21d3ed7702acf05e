// fau_mol_256_host.cu -- pipelined molecular-move kernel instantiation: 256 threads (1 + 7
// warps), host proposals (reference-stream batches through fau_run_proposals_batch).
#include "fau_mol.cuh"

namespace fau {

cudaError_t mol_dispatch_256_host(const ChainArgs& a, int nb, int K, int nc, cudaStream_t st, bool prep)
{
    if (prep) {
        const cudaError_t e = launch_mol_inst<256, 2, true>(a, nb, K, nc, st, true);
        return e != cudaSuccess ? e : launch_mol_inst<256, 3, true>(a, nb, K, nc, st, true);
    }
    return mol_minb(nb) == 3 ? launch_mol_inst<256, 3, true>(a, nb, K, nc, st, false)
                             : launch_mol_inst<256, 2, true>(a, nb, K, nc, st, false);
}

} // namespace fau
