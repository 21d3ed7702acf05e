// fau_kernels.cu -- sm_103a kernels of the Metropolis MC energy hot path.
//
//   chain_kernel      persistent move loop, one CTA per Markov chain: proposal
//                     -> FP64 trial positions -> FP32 pair + Ewald dU with
//                     float-float sums -> FP64 Metropolis -> commit.  Replaces
//                     MetropolisMonteCarlo::performMove (src/montecarlo.cpp:139-187)
//                     for transrot / moltransrot moves.
//   total_pair_kernel FP64 Nonbonded pairing.all (src/energy.h:1290-1299).
//   q_rebuild_kernel  FP64 Q(k) = sum_j q_j e^{ik.r_j} (src/energy.cpp:191-206).
//   plain_*           the plain FP64 single-move form: one move per call,
//                     host-fed proposal and uniform (in-GPU comparison point).
#include "fau_chain.cuh"
#include "fau_fast.cuh"
#include "fau_dev.cuh"
#include "fau_kernels.h"

#include <cfloat>

namespace fau {

// ---------------------------------------------------------------- FP64 total energy
__device__ __forceinline__ double block_sum_d(double v, double* red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    __syncthreads();
    return s;
}

// Nonbonded pairing.all: each i pairs with j > i; same group only if not rigid,
// different groups unless the group cutoff applies.  out[0] += finite sum,
// flags[0] |= 1 for +inf terms, 2 for NaN terms.
__global__ void total_pair_kernel(const DevSys* Sp, double* out, int* flags)
{
    const DevSys& S = *Sp;
    __shared__ double red[32];
    double e = 0.0;
    int f = 0;
    const long long n = S.n;
    for (long long i = blockIdx.x; i < n; i += gridDim.x) {
        const double xi[3] = {S.x[i], S.y[i], S.z[i]};
        const int ti = S.rec[i].w >> 24;
        const int gi = S.group_of[i];
        const bool ai = S.g_flags[gi] & FAU_GROUP_ATOMIC;
        const bool rigid_i = S.g_flags[gi] & FAU_GROUP_RIGID;
        const double cmi[3] = {S.g_cm[3 * gi], S.g_cm[3 * gi + 1], S.g_cm[3 * gi + 2]};
        for (long long j = i + 1 + threadIdx.x; j < n; j += blockDim.x) {
            const int gj = S.group_of[j];
            if (gj == gi) {
                if (rigid_i) continue;
            }
            else if (S.cut_g2g2 >= 0.0 && !ai && !(S.g_flags[gj] & FAU_GROUP_ATOMIC)) {
                const double c2 = group_cut2(S, gi, gj);
                const double cmj[3] = {S.g_cm[3 * gj], S.g_cm[3 * gj + 1], S.g_cm[3 * gj + 2]};
                if (c2 >= 0.0 && sqdist_d(S, cmi, cmj) >= c2) continue;
            }
            const double xj[3] = {S.x[j], S.y[j], S.z[j]};
            const double u = pair_u64(S, ti, S.rec[j].w >> 24, sqdist_d(S, xi, xj));
            if (isnan(u)) f |= 2;
            else if (isinf(u)) f |= 1;
            else e += u;
        }
    }
    const double s = block_sum_d(e, red);
    if (f) atomicOr(flags, f);
    if (threadIdx.x == 0) out[blockIdx.x] = s; // per-block partial: summed in block order on the host
}

// The same sum for systems of atomic groups with a cell list (every pair term is zero beyond
// the pair cutoff, no wider than a cell): particle i pairs with the j > i of its neighbour
// cells, O(N x neighbours) instead of O(N^2).
__global__ void total_pair_cells_kernel(const DevSys* Sp, double* out, int* flags)
{
    const DevSys& S = *Sp;
    __shared__ double red[32];
    double e = 0.0;
    int f = 0;
    const int nbx = S.off_max[0] - S.off_min[0] + 1, nby = S.off_max[1] - S.off_min[1] + 1,
              nbz = S.off_max[2] - S.off_min[2] + 1;
    const int items = nbx * nby * nbz * S.cap;
    for (long long i = blockIdx.x; i < S.n; i += gridDim.x) {
        const double xi[3] = {S.x[i], S.y[i], S.z[i]};
        const int ti = S.rec[i].w >> 24;
        const int ci = S.cell_of[i];
        const int c0[3] = {ci % S.cdim[0], (ci / S.cdim[0]) % S.cdim[1], ci / (S.cdim[0] * S.cdim[1])};
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
            const int nb = it / S.cap, slot = it - nb * S.cap;
            const int o[3] = {nb % nbx + S.off_min[0], (nb / nbx) % nby + S.off_min[1], nb / (nbx * nby) + S.off_min[2]};
            int w[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                w[d] = c0[d] + o[d];
                if (w[d] < 0) w[d] += S.cdim[d];
                else if (w[d] >= S.cdim[d]) w[d] -= S.cdim[d];
            }
            const int c = w[0] + S.cdim[0] * (w[1] + S.cdim[1] * w[2]);
            if (slot >= S.cell_cnt[c]) continue;
            const long long j = S.cell_rec[(size_t)c * S.cap + slot].w & 0xFFFFFFu;
            if (j <= i) continue;
            const double xj[3] = {S.x[j], S.y[j], S.z[j]};
            const double u = pair_u64(S, ti, S.rec[j].w >> 24, sqdist_d(S, xi, xj));
            if (isnan(u)) f |= 2;
            else if (isinf(u)) f |= 1;
            else e += u;
        }
    }
    const double s = block_sum_d(e, red);
    if (f) atomicOr(flags, f);
    if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// out[2b] = sum_k A_k |Q_k|^2, out[2b+1] = sum_i self(i), per block b
__global__ void total_misc_kernel(const DevSys* Sp, double* out)
{
    const DevSys& S = *Sp;
    __shared__ double red[32];
    double e = 0.0, s = 0.0;
    if (S.flags & SYS_EWALD)
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < S.K; k += gridDim.x * blockDim.x) {
            const double2 q = S.Q[k];
            e += S.Akd[k] * (q.x * q.x + q.y * q.y);
        }
    if (S.flags & SYS_SELF)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x)
            s += S.itype_self[S.rec[i].w >> 24];
    const double te = block_sum_d(e, red);
    const double ts = block_sum_d(s, red);
    if (threadIdx.x == 0) {
        out[2 * blockIdx.x] = te;
        out[2 * blockIdx.x + 1] = ts;
    }
}

// ---------------------------------------------------------------- FP64 Q(k) rebuild
// Q_k = sum_j q_j e^{i k.r_j} from the FP64 master positions with k = 2 pi n / L
// and k.r = (kx x + ky y) + kz z, as PolicyIonIon::updateComplex
// (src/energy.cpp:191-206).  One CTA per k.
// the pending FP32 changes (and the last accepted move's, if not yet added) into the FP64
// master, as a chain's flush does; one block
__global__ void fold_q_kernel(DevSys* Sp)
{
    DevSys& S = *Sp;
    const bool valid = S.q_valid != 0;
    for (int k = threadIdx.x; k < S.K; k += blockDim.x) {
        float2 pe = S.qpend[k];
        if (valid) {
            const float2 d = S.qdlt[k];
            pe.x += d.x;
            pe.y += d.y;
        }
        if (pe.x != 0.f || pe.y != 0.f) {
            double2 q = S.Q[k];
            q.x += (double)pe.x;
            q.y += (double)pe.y;
            S.Q[k] = q;
        }
        S.qpend[k] = make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        S.q_valid = 0;
        S.q_since = 0;
    }
}

cudaError_t launch_fold_q(DevSys* dsys, int K, cudaStream_t st)
{
    if (K <= 0) return cudaSuccess;
    fold_q_kernel<<<1, 256, 0, st>>>(dsys);
    return cudaGetLastError();
}

__global__ void q_rebuild_kernel(const DevSys* Sp, double2* out)
{
    const DevSys& S = *Sp;
    __shared__ double rx[32], ry[32];
    const double twopi = 6.283185307179586476925286766559;
    for (int k = blockIdx.x; k < S.K; k += gridDim.x) {
        int nx, ny, nz;
        kn_unpack(S.kn[k], nx, ny, nz);
        const double kx = twopi * ((double)nx / S.L[0]), ky = twopi * ((double)ny / S.L[1]),
                     kz = twopi * ((double)nz / S.L[2]);
        double sx = 0.0, sy = 0.0;
        for (int j = threadIdx.x; j < S.n; j += blockDim.x) {
            const double ph = __dadd_rn(__dadd_rn(__dmul_rn(kx, S.x[j]), __dmul_rn(ky, S.y[j])), __dmul_rn(kz, S.z[j]));
            double s, c;
            sincos(ph, &s, &c);
            const double q = S.itype_qd[S.rec[j].w >> 24];
            sx += q * c;
            sy += q * s;
        }
        const double tx = block_sum_d(sx, rx);
        const double ty = block_sum_d(sy, ry);
        if (threadIdx.x == 0) out[k] = make_double2(tx, ty);
    }
}

// ---------------------------------------------------------------- plain FP64 single move
// du of moving m atoms (new FP64 positions in P.xn), FP64 pair math from the FP64
// master positions (sqdist) and FP64 Ewald phases k.r (src/energy.cpp:219-247).
__global__ void plain_pair_kernel(const DevSys* Sp, const PlainMove* P, double* out, int* flags)
{
    const DevSys& S = *Sp;
    __shared__ double red[32];
    double e = 0.0, sc = 0.0;
    int f = 0;
    const int m = P->m;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < S.n; j += gridDim.x * blockDim.x) {
        const int gj = S.group_of[j];
        if (P->kind == FAU_MOVE_ATOMIC) {
            const int i = P->first;
            if (j == i) continue;
            const int ti = S.rec[i].w >> 24, tj = S.rec[j].w >> 24;
            const double xj[3] = {S.x[j], S.y[j], S.z[j]};
            const double xo[3] = {S.x[i], S.y[i], S.z[i]};
            const double un = pair_u64(S, ti, tj, sqdist_d(S, P->xn[0], xj));
            const double uo = pair_u64(S, ti, tj, sqdist_d(S, xo, xj));
            if (isnan(un)) f |= 4; else if (isinf(un)) f |= 1; else { e += un; sc += fabs(un); }
            if (isnan(uo)) f |= 8; else if (isinf(uo)) f |= 2; else { e -= uo; sc += fabs(uo); }
        }
        else {
            const int g = P->group;
            if (gj == g) continue;
            bool cut_o = false, cut_n = false;
            const double c2 = S.cut_g2g2 >= 0.0 ? group_cut2(S, g, gj) : -1.0;
            if (c2 >= 0.0 && !(S.g_flags[gj] & FAU_GROUP_ATOMIC)) {
                const double cmj[3] = {S.g_cm[3 * gj], S.g_cm[3 * gj + 1], S.g_cm[3 * gj + 2]};
                const double cmo[3] = {S.g_cm[3 * g], S.g_cm[3 * g + 1], S.g_cm[3 * g + 2]};
                cut_o = sqdist_d(S, cmo, cmj) >= c2;
                cut_n = sqdist_d(S, P->cm_new, cmj) >= c2;
            }
            const double xj[3] = {S.x[j], S.y[j], S.z[j]};
            const int tj = S.rec[j].w >> 24;
            for (int a = 0; a < m; a++) {
                const int i = P->first + a;
                const int ti = S.rec[i].w >> 24;
                if (!cut_n) {
                    const double un = pair_u64(S, ti, tj, sqdist_d(S, P->xn[a], xj));
                    if (isnan(un)) f |= 4; else if (isinf(un)) f |= 1; else { e += un; sc += fabs(un); }
                }
                if (!cut_o) {
                    const double xo[3] = {S.x[i], S.y[i], S.z[i]};
                    const double uo = pair_u64(S, ti, tj, sqdist_d(S, xo, xj));
                    if (isnan(uo)) f |= 8; else if (isinf(uo)) f |= 2; else { e -= uo; sc += fabs(uo); }
                }
            }
        }
    }
    const double s = block_sum_d(e, red);
    const double s2 = block_sum_d(sc, red);
    if (f) atomicOr(flags, f);
    if (threadIdx.x == 0) {
        atomicAdd(out, s);
        atomicAdd(out + 2, s2);
    }
}

__global__ void plain_ewald_kernel(const DevSys* Sp, const PlainMove* P, double2* dq, double* out)
{
    const DevSys& S = *Sp;
    __shared__ double red[32];
    double e = 0.0;
    const double twopi = 6.283185307179586476925286766559;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < S.K; k += gridDim.x * blockDim.x) {
        int nx, ny, nz;
        kn_unpack(S.kn[k], nx, ny, nz);
        const double kx = twopi * ((double)nx / S.L[0]), ky = twopi * ((double)ny / S.L[1]),
                     kz = twopi * ((double)nz / S.L[2]);
        double dx = 0.0, dy = 0.0;
        for (int a = 0; a < P->m; a++) {
            const int i = P->first + a;
            const double q = S.itype_qd[S.rec[i].w >> 24];
            const double pn = (kx * P->xn[a][0] + ky * P->xn[a][1]) + kz * P->xn[a][2];
            const double po = (kx * S.x[i] + ky * S.y[i]) + kz * S.z[i];
            double sn, cn, so, co;
            sincos(pn, &sn, &cn);
            sincos(po, &so, &co);
            dx += q * cn - q * co;
            dy += q * sn - q * so;
        }
        dq[k] = make_double2(dx, dy);
        const double2 Q = S.Q[k];
        const double nx2 = (Q.x + dx) * (Q.x + dx) + (Q.y + dy) * (Q.y + dy);
        const double ox2 = Q.x * Q.x + Q.y * Q.y;
        e += S.Akd[k] * (nx2 - ox2);
    }
    const double s = block_sum_d(e, red);
    if (threadIdx.x == 0) atomicAdd(out + 1, s);
}

// commit of a plain move: positions, records, mass centre, cell list, Q += dq
__global__ void plain_commit_kernel(DevSys* Sp, const PlainMove* P, const double2* dq)
{
    DevSys& S = *Sp;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < S.K; k += gridDim.x * blockDim.x) {
        double2 q = S.Q[k];
        q.x += dq[k].x;
        q.y += dq[k].y;
        S.Q[k] = q;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int a = 0; a < P->m; a++) {
            const int i = P->first + a;
            S.x[i] = P->xn[a][0];
            S.y[i] = P->xn[a][1];
            S.z[i] = P->xn[a][2];
            uint4 r = S.rec[i];
            r.x = to_fixed(P->xn[a][0], S.fx_scale[0]);
            r.y = to_fixed(P->xn[a][1], S.fx_scale[1]);
            r.z = to_fixed(P->xn[a][2], S.fx_scale[2]);
            S.rec[i] = r;
            if ((S.flags & SYS_CELLS) && P->kind == FAU_MOVE_ATOMIC) {
                const int co = S.cell_of[i];
                int cc[3];
                cell_coords(S, P->xn[a], r, cc);
                const int cn = cell_index(S, cc);
                const int so = S.slot_of[i];
                if (co == cn) {
                    S.cell_rec[(size_t)co * S.cap + so] = r;
                }
                else {
                    const int last = S.cell_cnt[co] - 1;
                    if (so != last) {
                        const uint4 mvd = S.cell_rec[(size_t)co * S.cap + last];
                        S.cell_rec[(size_t)co * S.cap + so] = mvd;
                        S.slot_of[mvd.w & 0xFFFFFFu] = so;
                    }
                    S.cell_rec[(size_t)co * S.cap + last] = make_uint4(0u, 0u, 0u, kEmptySlot);
                    S.cell_cnt[co] = last;
                    const int sn = S.cell_cnt[cn];
                    if (sn >= S.cap) {
                        S.cell_rec[(size_t)co * S.cap + last] = r;
                        S.slot_of[i] = last;
                        S.cell_cnt[co] = last + 1;
                        S.err = FAU_ERR_CAPACITY;
                    }
                    else {
                        S.cell_rec[(size_t)cn * S.cap + sn] = r;
                        S.cell_cnt[cn] = sn + 1;
                        S.cell_of[i] = cn;
                        S.slot_of[i] = sn;
                    }
                }
            }
        }
        if (P->kind == FAU_MOVE_MOLECULAR) {
            const int g = P->group;
            for (int d = 0; d < 3; d++) S.g_cm[3 * g + d] = P->cm_new[d];
            S.g_cmrec[g] = make_uint4(to_fixed(P->cm_new[0], S.fx_scale[0]), to_fixed(P->cm_new[1], S.fx_scale[1]),
                                      to_fixed(P->cm_new[2], S.fx_scale[2]), 0u);
        }
        for (int d = 0; d < 3; d++) S.M[d] += P->dM[d];
        S.energy += P->du;
        S.moves += P->count_move;
        S.accepted += 1;
        S.sum_du += P->du;
    }
}

// ---------------------------------------------------------------- launchers
size_t chain_smem_bytes(int K, int nc) { return chain_smem_bytes_v2(K, nc); }

int chain_max_k(int threads) { return 6400; }

cudaError_t chain_launch_impl(const ChainArgs& a, int nblocks, int K, int nc, int threads, bool philox,
                              cudaStream_t st, bool prepare_only)
{
    if (threads == 128)
        return philox ? chain_dispatch_128_ph(a, nblocks, K, nc, st, prepare_only)
                      : chain_dispatch_128_host(a, nblocks, K, nc, st, prepare_only);
    return philox ? chain_dispatch_256_ph(a, nblocks, K, nc, st, prepare_only)
                  : chain_dispatch_256_host(a, nblocks, K, nc, st, prepare_only);
}

cudaError_t prepare_chain(int K, int nc, int threads, bool philox)
{
    ChainArgs a{};
    return chain_launch_impl(a, 0, K, nc, threads, philox, nullptr, true);
}

cudaError_t launch_chain(const ChainArgs& a, int nblocks, int K, int nc, int threads, bool philox, cudaStream_t st)
{
    return chain_launch_impl(a, nblocks, K, nc, threads, philox, st, false);
}

size_t fast_smem_bytes_total(int K, int nc, int nt)
{
    // dynamic part + the kernel's static shared memory (the widest instance's)
    return fast_smem_bytes(K, nc, nt, 8) + sizeof(FastShared<8>);
}

static cudaError_t fast_launch_impl(const ChainArgs& a, int nblocks, int K, int nc, int nt, int warps, bool philox,
                                    bool occ, cudaStream_t st, bool prepare_only)
{
    if (warps == 4 && occ)
        return philox ? fast_dispatch_4_ph_sparse(a, nblocks, K, nc, nt, st, prepare_only)
                      : fast_dispatch_4_host_sparse(a, nblocks, K, nc, nt, st, prepare_only);
    if (warps == 4)
        return philox ? fast_dispatch_4_ph(a, nblocks, K, nc, nt, st, prepare_only)
                      : fast_dispatch_4_host(a, nblocks, K, nc, nt, st, prepare_only);
    if (warps == 8 && philox)
        return occ ? fast_dispatch_8_ph_sparse(a, nblocks, K, nc, nt, st, prepare_only)
                   : fast_dispatch_8_ph(a, nblocks, K, nc, nt, st, prepare_only);
    if (warps == 2)
        return philox ? fast_dispatch_2_ph(a, nblocks, K, nc, nt, st, prepare_only)
                      : fast_dispatch_2_host(a, nblocks, K, nc, nt, st, prepare_only);
    return cudaErrorInvalidValue;
}

cudaError_t prepare_fast(int K, int nc, int nt, int warps, bool philox, bool occ)
{
    ChainArgs a{};
    return fast_launch_impl(a, 0, K, nc, nt, warps, philox, occ, nullptr, true);
}

cudaError_t launch_fast(const ChainArgs& a, int nblocks, int K, int nc, int nt, int warps, bool philox, bool occ,
                        cudaStream_t st)
{
    return fast_launch_impl(a, nblocks, K, nc, nt, warps, philox, occ, st, false);
}

// Partials layout in d_out: [0, kTotalPairBlocks) pair sums per block, then
// 2 * kTotalMiscBlocks (reciprocal, self) pairs; unused blocks write nothing, so
// the caller zeroes the buffer first.  Deterministic: no floating-point atomics.
cudaError_t launch_total(const DevSys* dsys, int n, int K, double* d_out, int* d_flags, cudaStream_t st, bool cells)
{
    int blocks = n < kTotalPairBlocks ? (n > 0 ? n : 1) : kTotalPairBlocks;
    if (cells) total_pair_cells_kernel<<<blocks, 256, 0, st>>>(dsys, d_out, d_flags);
    else total_pair_kernel<<<blocks, 256, 0, st>>>(dsys, d_out, d_flags);
    int kb = (K + n + 255) / 256;
    if (kb < 1) kb = 1;
    if (kb > kTotalMiscBlocks) kb = kTotalMiscBlocks;
    total_misc_kernel<<<kb, 256, 0, st>>>(dsys, d_out + kTotalPairBlocks);
    return cudaGetLastError();
}

cudaError_t launch_q_rebuild(const DevSys* dsys, int K, double2* out, cudaStream_t st)
{
    if (K <= 0) return cudaSuccess;
    q_rebuild_kernel<<<K < 2048 ? K : 2048, 256, 0, st>>>(dsys, out);
    return cudaGetLastError();
}

cudaError_t launch_plain_du(const DevSys* dsys, const PlainMove* pm, int n, int K, double2* dq, double* out, int* flags,
                            cudaStream_t st)
{
    int b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > 1024) b = 1024;
    plain_pair_kernel<<<b, 256, 0, st>>>(dsys, pm, out, flags);
    if (K > 0) {
        int kb = (K + 255) / 256;
        plain_ewald_kernel<<<kb, 256, 0, st>>>(dsys, pm, dq, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_plain_commit(DevSys* dsys, const PlainMove* pm, int K, const double2* dq, cudaStream_t st)
{
    int kb = (K + 255) / 256;
    if (kb < 1) kb = 1;
    plain_commit_kernel<<<kb, 256, 0, st>>>(dsys, pm, dq);
    return cudaGetLastError();
}

} // namespace fau
