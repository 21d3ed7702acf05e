// fau_sampler.cu -- device analysis: AtomRDF and SystemEnergy sampled into
// per-slot accumulators on the GPU, standalone or between the blocks of a
// batched launch (inside its CUDA graph), so sampling needs no host round trip.
//
// AtomRDF::sampleIdentical / sampleDifferent (src/analysis.cpp:1577-1600): all
// pairs of atoms of types a and b (i < j when a == b); r = |vdist(pi, pj)|;
// histogram bin floor(r * (1/dr)) (Equidistant2DTable::to_bin,
// src/aux/equidistant_table.h:32-39); the volume is summed per sample for
// PairFunction::_to_disk (src/analysis.cpp:724-737).  Bins are decided in FP32
// from the fixed-point records; a distance whose FP32 bin coordinate lies within
// its error bound of a bin edge is recomputed from the FP64 positions exactly as
// the FP64 oracle does, so the counts are identical to it.
// SystemEnergy::_sample (src/analysis.cpp:339-357): the running FP64 total energy
// (kept equal to the sum of the Hamiltonian's terms by the chain kernels).
#include "fau_dev.cuh"
#include "fau_kernels.h"

#include <cmath>
#include <cstring>
#include <vector>

using namespace fau;

struct fau_ctx;
extern "C" int fau_internal_ctx_stream(fau_ctx* c, cudaStream_t* st, int* device);
extern "C" int fau_internal_sys_view(fau_sys* s, fau_ctx** ctx, DevSys** d, int* K, int* n, int* n_groups,
                                     int* molecular_only, double* t_ref, int* knc);
extern "C" int fau_internal_fail(int code, const char* msg);

struct fau_sampler {
    fau_ctx* ctx = nullptr;
    cudaStream_t st = nullptr;
    int device = 0;
    fau_sampler_desc d{};
    double dxinv = 0.0;
    unsigned long long* hist = nullptr; // n_slots * (bins + 1)
    double* acc = nullptr;              // n_slots * 3: volume sum, energy sum, energy sum^2
    long long* cnt = nullptr;           // n_slots * 2: rdf samples, energy samples
    // staging for standalone sample() calls
    DevSys** sys_buf = nullptr;
    int* slot_buf = nullptr;
    int buf_cap = 0;
};

namespace {

constexpr int kRdfThreads = 256;

__global__ void __launch_bounds__(kRdfThreads) rdf_kernel(DevSys* const* sys, const int* slots, int n_slots,
                                                          int ta, int tb, float dxinv_f, double dxinv, int bins,
                                                          unsigned long long* hist)
{
    extern __shared__ unsigned int h_s[]; // bins + 1
    __shared__ uint4 tile[kRdfThreads];
    const DevSys& S = *sys[blockIdx.y];
    const int slot = slots ? slots[blockIdx.y] : (int)(blockIdx.y % n_slots);
    const int n = S.n;
    const int i0 = blockIdx.x * kRdfThreads;
    if (i0 >= n) return; // the whole CTA: no barrier is left waiting
    for (int b = threadIdx.x; b <= bins; b += kRdfThreads) h_s[b] = 0u;
    const int i = i0 + threadIdx.x;
    uint4 ri = make_uint4(0, 0, 0, 0);
    bool act = false;
    if (i < n) {
        ri = S.rec[i];
        act = S.itype_type[ri.w >> 24] == ta;
    }
    const bool same = ta == tb;
    const float lmax = (float)fmax(S.L[0], fmax(S.L[1], S.L[2]));
    const float g_abs = dxinv_f * lmax * 2e-9f + 1e-6f;
    double xi[3] = {0.0, 0.0, 0.0};
    if (act) {
        xi[0] = S.x[i];
        xi[1] = S.y[i];
        xi[2] = S.z[i];
    }
    __syncthreads();
    // i < j pairs for identical types: tiles from the CTA's own tile on
    for (int j0 = same ? i0 : 0; j0 < n; j0 += kRdfThreads) {
        const int jl = j0 + threadIdx.x;
        tile[threadIdx.x] = jl < n ? S.rec[jl] : make_uint4(0, 0, 0, kEmptySlot);
        __syncthreads();
        if (act) {
            const int m = min(kRdfThreads, n - j0);
            for (int q = 0; q < m; q++) {
                const int j = j0 + q;
                if (same && j <= i) continue;
                const uint4 rj = tile[q];
                if (S.itype_type[rj.w >> 24] != tb) continue;
                const float r = sqrtf(r2_fixed(S, ri, rj));
                const float t = r * dxinv_f;
                int b = (int)floorf(t);
                const float edge = fminf(t - floorf(t), ceilf(t) - t);
                if (edge <= t * 1e-6f + g_abs) { // near a bin edge: the FP64 distance decides
                    const double xj[3] = {S.x[j], S.y[j], S.z[j]};
                    const double rd = sqrt(sqdist_d(S, xi, xj));
                    b = (int)floor(rd * dxinv);
                }
                atomicAdd(&h_s[b < bins ? b : bins], 1u);
            }
        }
        __syncthreads();
    }
    unsigned long long* out = hist + (size_t)slot * (bins + 1);
    for (int b = threadIdx.x; b <= bins; b += kRdfThreads)
        if (h_s[b]) atomicAdd(out + b, (unsigned long long)h_s[b]);
}

// one thread per slot, systems in index order: deterministic FP64 sums
__global__ void slot_sum_kernel(DevSys* const* sys, int n, const int* slots, int n_slots, int rdf, int energy,
                                double* acc, long long* cnt)
{
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= n_slots) return;
    double v = acc[3 * slot], e1 = acc[3 * slot + 1], e2 = acc[3 * slot + 2];
    long long cr = cnt[2 * slot], ce = cnt[2 * slot + 1];
    for (int s = 0; s < n; s++) {
        const int sl = slots ? slots[s] : s % n_slots;
        if (sl != slot) continue;
        const DevSys& S = *sys[s];
        if (rdf) {
            v += S.L[0] * S.L[1] * S.L[2];
            cr++;
        }
        if (energy) {
            const double e = sys_energy(S);
            e1 += e;
            e2 += e * e;
            ce++;
        }
    }
    acc[3 * slot] = v;
    acc[3 * slot + 1] = e1;
    acc[3 * slot + 2] = e2;
    cnt[2 * slot] = cr;
    cnt[2 * slot + 1] = ce;
}

} // namespace

// enqueue one sample of n systems (device arrays) on `st`
cudaError_t fau_internal_sampler_launch(fau_sampler* s, DevSys* const* d_sys, int n, const int* d_slots, int max_n,
                                        cudaStream_t st)
{
    const fau_sampler_desc& d = s->d;
    if (d.rdf_bins > 0 && max_n > 0) {
        const dim3 grid((max_n + kRdfThreads - 1) / kRdfThreads, n);
        rdf_kernel<<<grid, kRdfThreads, sizeof(unsigned int) * (d.rdf_bins + 1), st>>>(
            d_sys, d_slots, d.n_slots, d.rdf_type_a, d.rdf_type_b, (float)s->dxinv, s->dxinv, d.rdf_bins, s->hist);
    }
    slot_sum_kernel<<<(d.n_slots + 127) / 128, 128, 0, st>>>(d_sys, n, d_slots, d.n_slots, d.rdf_bins > 0,
                                                              d.energy, s->acc, s->cnt);
    return cudaGetLastError();
}

int fau_internal_sampler_slots(const fau_sampler* s) { return s->d.n_slots; }
fau_ctx* fau_internal_sampler_ctx(const fau_sampler* s) { return s->ctx; }

extern "C" {

int fau_sampler_create(fau_ctx* ctx, const fau_sampler_desc* desc, fau_sampler** out)
{
    if (!ctx || !desc || !out) return fau_internal_fail(FAU_ERR_ARG, "null argument");
    if (desc->n_slots < 1) return fau_internal_fail(FAU_ERR_ARG, "n_slots must be >= 1");
    if (desc->rdf_bins < 0 || desc->rdf_bins > FAU_SAMPLER_MAX_BINS)
        return fau_internal_fail(FAU_ERR_ARG, "rdf_bins outside [0, FAU_SAMPLER_MAX_BINS]");
    if (desc->rdf_bins > 0 && !(desc->rdf_dr > 0.0 && std::isfinite(desc->rdf_dr)))
        return fau_internal_fail(FAU_ERR_ARG, "rdf_dr must be positive");
    if (desc->rdf_bins > 0 && (desc->rdf_type_a < 0 || desc->rdf_type_b < 0))
        return fau_internal_fail(FAU_ERR_ARG, "rdf atom types must be >= 0");
    fau_sampler* s = new fau_sampler;
    s->ctx = ctx;
    s->d = *desc;
    s->dxinv = desc->rdf_bins > 0 ? 1.0 / desc->rdf_dr : 0.0;
    fau_internal_ctx_stream(ctx, &s->st, &s->device);
    cudaSetDevice(s->device);
    const size_t nh = (size_t)desc->n_slots * (desc->rdf_bins + 1);
    bool ok = cudaMalloc(&s->hist, sizeof(unsigned long long) * nh) == cudaSuccess &&
              cudaMalloc(&s->acc, sizeof(double) * 3 * desc->n_slots) == cudaSuccess &&
              cudaMalloc(&s->cnt, sizeof(long long) * 2 * desc->n_slots) == cudaSuccess;
    if (ok && desc->rdf_bins > 0) {
        const int smem = (int)(sizeof(unsigned int) * (desc->rdf_bins + 1));
        ok = cudaFuncSetAttribute(rdf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess;
    }
    if (!ok) {
        fau_sampler_destroy(s);
        return fau_internal_fail(FAU_ERR_OOM, "sampler allocation failed");
    }
    *out = s;
    return fau_sampler_reset(s);
}

int fau_sampler_destroy(fau_sampler* s)
{
    if (!s) return FAU_OK;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->st);
    cudaFree(s->hist);
    cudaFree(s->acc);
    cudaFree(s->cnt);
    cudaFree(s->sys_buf);
    cudaFree(s->slot_buf);
    delete s;
    return FAU_OK;
}

int fau_sampler_reset(fau_sampler* s)
{
    if (!s) return fau_internal_fail(FAU_ERR_ARG, "null sampler");
    cudaSetDevice(s->device);
    const size_t nh = (size_t)s->d.n_slots * (s->d.rdf_bins + 1);
    if (cudaMemsetAsync(s->hist, 0, sizeof(unsigned long long) * nh, s->st) != cudaSuccess ||
        cudaMemsetAsync(s->acc, 0, sizeof(double) * 3 * s->d.n_slots, s->st) != cudaSuccess ||
        cudaMemsetAsync(s->cnt, 0, sizeof(long long) * 2 * s->d.n_slots, s->st) != cudaSuccess)
        return fau_internal_fail(FAU_ERR_CUDA, "sampler reset failed");
    return FAU_OK;
}

int fau_sampler_sample(fau_sampler* s, fau_sys* const* systems, int n, const int* slots)
{
    if (!s || !systems || n < 1) return fau_internal_fail(FAU_ERR_ARG, "invalid sample arguments");
    cudaSetDevice(s->device);
    std::vector<DevSys*> ds(n);
    int max_n = 0;
    for (int i = 0; i < n; i++) {
        fau_ctx* c;
        int K, np, ng, mo, knc;
        double tr;
        if (!systems[i]) return fau_internal_fail(FAU_ERR_ARG, "null system");
        fau_internal_sys_view(systems[i], &c, &ds[i], &K, &np, &ng, &mo, &tr, &knc);
        if (c != s->ctx) return fau_internal_fail(FAU_ERR_ARG, "system from another context");
        if (slots && (slots[i] < 0 || slots[i] >= s->d.n_slots))
            return fau_internal_fail(FAU_ERR_ARG, "slot outside [0, n_slots)");
        max_n = np > max_n ? np : max_n;
    }
    if (n > s->buf_cap) {
        cudaStreamSynchronize(s->st);
        cudaFree(s->sys_buf);
        cudaFree(s->slot_buf);
        s->sys_buf = nullptr;
        s->slot_buf = nullptr;
        s->buf_cap = 0;
        if (cudaMalloc(&s->sys_buf, sizeof(DevSys*) * n) != cudaSuccess ||
            cudaMalloc(&s->slot_buf, sizeof(int) * n) != cudaSuccess)
            return fau_internal_fail(FAU_ERR_OOM, "sampler staging allocation failed");
        s->buf_cap = n;
    }
    // pageable sources: the copies are staged before the calls return
    if (cudaMemcpyAsync(s->sys_buf, ds.data(), sizeof(DevSys*) * n, cudaMemcpyHostToDevice, s->st) != cudaSuccess ||
        (slots && cudaMemcpyAsync(s->slot_buf, slots, sizeof(int) * n, cudaMemcpyHostToDevice, s->st) != cudaSuccess))
        return fau_internal_fail(FAU_ERR_CUDA, "sampler staging copy failed");
    if (fau_internal_sampler_launch(s, s->sys_buf, n, slots ? s->slot_buf : nullptr, max_n, s->st) != cudaSuccess)
        return fau_internal_fail(FAU_ERR_CUDA, "sampler launch failed");
    return FAU_OK;
}

int fau_sampler_read(fau_sampler* s, uint64_t* rdf_hist, double* rdf_volume_sum, int64_t* rdf_samples,
                     double* energy_sum, double* energy_sum2, int64_t* energy_samples)
{
    if (!s) return fau_internal_fail(FAU_ERR_ARG, "null sampler");
    cudaSetDevice(s->device);
    const int ns = s->d.n_slots;
    std::vector<double> acc(3 * (size_t)ns);
    std::vector<long long> cnt(2 * (size_t)ns);
    if (rdf_hist && s->d.rdf_bins > 0 &&
        cudaMemcpyAsync(rdf_hist, s->hist, sizeof(unsigned long long) * (size_t)ns * (s->d.rdf_bins + 1),
                        cudaMemcpyDeviceToHost, s->st) != cudaSuccess)
        return fau_internal_fail(FAU_ERR_CUDA, "sampler read failed");
    if (cudaMemcpyAsync(acc.data(), s->acc, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, s->st) !=
            cudaSuccess ||
        cudaMemcpyAsync(cnt.data(), s->cnt, sizeof(long long) * cnt.size(), cudaMemcpyDeviceToHost, s->st) !=
            cudaSuccess ||
        cudaStreamSynchronize(s->st) != cudaSuccess)
        return fau_internal_fail(FAU_ERR_CUDA, "sampler read failed");
    for (int k = 0; k < ns; k++) {
        if (rdf_volume_sum) rdf_volume_sum[k] = acc[3 * k];
        if (energy_sum) energy_sum[k] = acc[3 * k + 1];
        if (energy_sum2) energy_sum2[k] = acc[3 * k + 2];
        if (rdf_samples) rdf_samples[k] = cnt[2 * k];
        if (energy_samples) energy_samples[k] = cnt[2 * k + 1];
    }
    return FAU_OK;
}

} // extern "C"
