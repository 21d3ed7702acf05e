// fau_audit.cu -- the FP64 audit of the pipelined kernel's probe moves.
//
// After the last move of a launch each chain of fast_chain_kernel evaluates one more move (its
// next proposal) on its final state without deciding it, and leaves that move and its FP32
// energy change in the system's audit record.  This kernel re-evaluates the same move in FP64
// (fast_audit) and keeps the largest error of the FP32 change against it, so that every
// launch's result carries its error against FP64.  It is a kernel of its own because the FP64
// code, called from inside the chain kernel, cost that kernel's move loop its registers.
#include "fau_fast.cuh"

namespace fau {

// One CTA per system: the FP64 energy change of its probe and the FP32 one's error against it,
// relative to max(|dU|, S) and to |dU| (|dU| > 1e-3 kT), kept as the system's largest.
__global__ void __launch_bounds__(128) fast_audit_kernel(DevSys* const* sys)
{
    DevSys& G = *sys[blockIdx.x];
    if (!G.audit_pending) return;
    const FastMove& m = *reinterpret_cast<const FastMove*>(G.audit_rec);
    const bool cells = (G.flags & SYS_CELLS) != 0;
    const int cap_shift = cells ? __ffs(G.cap) - 1 : 0;
    const int K = (G.flags & SYS_EWALD) ? G.K : 0;
    double2 ad = fast_audit(G, m, K, threadIdx.x, 128, cells ? (m.nue << cap_shift) : G.n, cap_shift, cells);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ad.x += __shfl_xor_sync(0xffffffffu, ad.x, o);
        ad.y += __shfl_xor_sync(0xffffffffu, ad.y, o);
    }
    __shared__ double2 red[4];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ad;
    __syncthreads();
    if (threadIdx.x == 0) {
        double d64 = (G.flags & SYS_SURFACE) ? m.du_surf : 0.0, s64 = 0.0;
        for (int w = 0; w < 4; w++) {
            d64 += red[w].x;
            s64 += red[w].y;
        }
        const double err = fabs(G.audit_du - d64), den = fmax(fabs(d64), s64);
        G.audit_scaled_max = fmax(G.audit_scaled_max, den > 0.0 ? err / den : 0.0);
        if (fabs(d64) > 1e-3) G.audit_rel_max = fmax(G.audit_rel_max, err / fabs(d64));
        G.audit_samples += 1;
        G.audit_pending = 0;
    }
}

cudaError_t launch_fast_audit(DevSys* const* sys, int n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    fast_audit_kernel<<<n, 128, 0, st>>>(sys);
    return cudaGetLastError();
}

} // namespace fau
