// fau_audit.cu -- the FP64 audit of the pipelined kernels' probe moves.
//
// After the last move of a launch each chain of fast_chain_kernel (and of mol_chain_kernel and
// chain_kernel: probe_audit_kernel) evaluates one more move (its
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

// One CTA per system: the FP64 energy change of a probe of the molecular kernel or the chain
// kernel (a TranslateRotate or AtomicTranslateRotate move left undecided on the final state) and
// the FP32 one's error against it.  FP64 as the plain form evaluates it: for a molecular move
// GroupCutoff by FP64 mass-centre distances (src/energy.h:761-768) and the particles of the other
// groups, for a single atom every other particle; pair_u64 of FP64 minimum-image distances, the
// reciprocal change from FP64 phases against Q(k) as the chain holds it; S is pair_mag64 of every
// pair of both states plus (2 pi lB / V) A_k (|2 Re(Q* d)| + |d|^2) of every k-vector.
constexpr int kProbeAuditThreads = 256; // FP64 chains of dependent instructions: many warps hide them

__global__ void __launch_bounds__(kProbeAuditThreads) probe_audit_kernel(DevSys* const* sys)
{
    DevSys& G = *sys[blockIdx.x];
    if (!G.audit_pending) return;
    const ProbeRecord& p = *reinterpret_cast<const ProbeRecord*>(G.audit_rec);
    const bool molecular = p.kind == FAU_MOVE_MOLECULAR;
    const int g = molecular ? p.index : -1, m = p.m, b = p.first;
    const double cmo[3] = {molecular ? G.g_cm[3 * g] : 0.0, molecular ? G.g_cm[3 * g + 1] : 0.0,
                           molecular ? G.g_cm[3 * g + 2] : 0.0};
    double du = 0.0, sc = 0.0;
    for (int j = threadIdx.x; j < G.n; j += kProbeAuditThreads) {
        const int gj = G.group_of[j];
        if (molecular ? gj == g : j == b) continue;
        bool cut_o = false, cut_n = false;
        const double c2 = molecular && G.cut_g2g2 >= 0.0 ? group_cut2(G, g, gj) : -1.0;
        if (c2 >= 0.0 && !(G.g_flags[gj] & FAU_GROUP_ATOMIC)) {
            const double cmj[3] = {G.g_cm[3 * gj], G.g_cm[3 * gj + 1], G.g_cm[3 * gj + 2]};
            cut_o = sqdist_d(G, cmo, cmj) >= c2;
            cut_n = sqdist_d(G, p.cm_new, cmj) >= c2;
        }
        if (cut_o && cut_n) continue;
        const int tj = (int)(G.rec[j].w >> 24);
        const double xj[3] = {G.x[j], G.y[j], G.z[j]};
        for (int a = 0; a < m; a++) {
            const int i = b + a, ti = (int)(G.rec[i].w >> 24);
            if (!cut_n) {
                const double r2 = sqdist_d(G, p.xn[a], xj);
                du += pair_u64(G, ti, tj, r2);
                sc += pair_mag64(G, ti, tj, r2);
            }
            if (!cut_o) {
                const double xo[3] = {G.x[i], G.y[i], G.z[i]};
                const double r2 = sqdist_d(G, xo, xj);
                du -= pair_u64(G, ti, tj, r2);
                sc += pair_mag64(G, ti, tj, r2);
            }
        }
    }
    const int K = (G.flags & SYS_EWALD) ? G.K : 0;
    for (int k = threadIdx.x; k < K; k += kProbeAuditThreads) {
        int nx, ny, nz;
        kn_unpack(G.kn[k], nx, ny, nz);
        double dx = 0.0, dy = 0.0;
        for (int a = 0; a < m; a++) {
            const int i = b + a;
            const double q = G.itype_qd[G.rec[i].w >> 24];
            // phase / pi = 2 n.x / L
            const double po = 2.0 * ((nx * G.x[i]) * G.inv[0] + (ny * G.y[i]) * G.inv[1] + (nz * G.z[i]) * G.inv[2]);
            const double pn =
                2.0 * ((nx * p.xn[a][0]) * G.inv[0] + (ny * p.xn[a][1]) * G.inv[1] + (nz * p.xn[a][2]) * G.inv[2]);
            double so, co, sn, cn;
            sincospi(po, &so, &co);
            sincospi(pn, &sn, &cn);
            dx += q * (cn - co);
            dy += q * (sn - so);
        }
        const double2 qm = G.Q[k];
        const float2 pe = G.qpend[k]; // the probe folded the last accepted change (q_valid is 0)
        const double qx = qm.x + (double)pe.x, qy = qm.y + (double)pe.y;
        const double w = G.rec_pref * G.Akd[k];
        const double cross = 2.0 * (qx * dx + qy * dy), dd = dx * dx + dy * dy;
        du += w * (cross + dd);
        sc += w * (fabs(cross) + dd);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        du += __shfl_xor_sync(0xffffffffu, du, o);
        sc += __shfl_xor_sync(0xffffffffu, sc, o);
    }
    __shared__ double2 red[kProbeAuditThreads / 32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(du, sc);
    __syncthreads();
    if (threadIdx.x == 0) {
        double d64 = p.du_surf, s64 = 0.0;
        for (int w = 0; w < kProbeAuditThreads / 32; w++) {
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

cudaError_t launch_probe_audit(DevSys* const* sys, int n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    probe_audit_kernel<<<n, kProbeAuditThreads, 0, st>>>(sys);
    return cudaGetLastError();
}

} // namespace fau
