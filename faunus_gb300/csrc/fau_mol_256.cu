// fau_mol_256.cu -- pipelined molecular-move kernel instantiation: 256 threads (1 + 7 warps),
// device proposals (host proposals: fau_mol_256_host.cu).
#include "fau_mol.cuh"

#include <cstdlib>

namespace fau {

// Registers are sized for 2 or 3 resident CTAs per SM (128 or 80 per thread; 80 spills more,
// a full wave of 3 per SM measured ~4 % faster than one of 2).  A launch takes the size
// whose waves fill the SMs better: e.g. 608 chains on 152 SMs run as 2 waves of 2 per SM,
// 456 or 912 as waves of 3.  FAU_MOL_MINB=2 or 3 fixes it.
int mol_minb(int nblocks)
{
    static int forced = [] {
        const char* e = std::getenv("FAU_MOL_MINB");
        const int x = e ? std::atoi(e) : 0;
        return (x == 2 || x == 3) ? x : 0;
    }();
    if (forced) return forced;
    static int sms = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    auto fill = [&](int o, double speed) {
        const long long per_wave = (long long)o * sms;
        const long long waves = (nblocks + per_wave - 1) / per_wave;
        return speed * (double)nblocks / (double)(waves * per_wave);
    };
    return fill(3, 1.04) > fill(2, 1.0) ? 3 : 2;
}

cudaError_t mol_dispatch_256(const ChainArgs& a, int nb, int K, int nc, cudaStream_t st, bool prep)
{
    if (prep) { // every instance gets its shared-memory allowance before any capture
        cudaError_t e = launch_mol_inst<256, 2, false>(a, nb, K, nc, st, true);
        if (e == cudaSuccess) e = launch_mol_inst<256, 3, false>(a, nb, K, nc, st, true);
        return e != cudaSuccess ? e : mol_dispatch_256_host(a, nb, K, nc, st, true);
    }
    if (a.props) return mol_dispatch_256_host(a, nb, K, nc, st, false);
    return mol_minb(nb) == 3 ? launch_mol_inst<256, 3, false>(a, nb, K, nc, st, false)
                             : launch_mol_inst<256, 2, false>(a, nb, K, nc, st, false);
}

size_t mol_smem_bytes_total(int K, int nc)
{
    return mol_smem_bytes(K, nc);
}

} // namespace fau
