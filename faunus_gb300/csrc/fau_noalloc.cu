// fau_noalloc.cu -- the FP64 nonbonded energy of a configuration, computed
// without any device allocation by the library.
//
// Who needs this: a caller that cannot call cudaMalloc -- typically a host
// simulation engine that owns every byte of device memory through its own
// pool and does not let a plugin allocate (cudaMalloc and cudaFree synchronise
// the device and fragment the pool), or a latency-critical loop that must not
// stall on an allocation.  Such a caller keeps its particles in its own device
// buffers and passes device pointers for every input and for the output.
//
// The only scratch is the file-scope array below: one FP64 partial sum per
// particle, FAU_NOALLOC_MAX_PARTICLES entries (512 KiB).  Every GPU context that
// loads this library's device code holds it until the process exits.  All calls
// share it and it keeps the last call's contents; each call overwrites the
// first n entries before reading them, so nothing has to start at zero.  Calls
// that overlap on the GPU (different streams or host threads) race on it.
//
// The array's device address is looked up once per CUDA context (the first call
// on a device, or the first after that device's context was destroyed and made
// again, e.g. by cudaDeviceReset): make such a call before any stream capture.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/fau_gpu.h"

extern "C" int fau_internal_fail(int code, const char* msg);

namespace {

static __device__ __align__(256) double g_noalloc_partial[FAU_NOALLOC_MAX_PARTICLES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// device address of the array per device, and the id of the context it was looked up in: a
// context made again (after cudaDeviceReset) loads the module again, possibly elsewhere
double* g_partial_ptr[kMaxDevices] = {nullptr};
unsigned long long g_partial_ctx[kMaxDevices] = {0};

// the unique id of the calling thread's current context (cuCtxGetId through the runtime's
// driver entry points, so that the library needs no link against the driver library); 0 if
// the driver does not provide it
unsigned long long current_context_id()
{
    using get_current_t = CUresult (*)(CUcontext*);
    using get_id_t = CUresult (*)(CUcontext, unsigned long long*);
    static get_current_t get_current = nullptr;
    static get_id_t get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        looked_up = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<get_current_t>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<get_id_t>(f);
        cudaGetLastError();
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&c) == CUDA_SUCCESS && c && get_id(c, &id) == CUDA_SUCCESS) return id;
    return 0;
}

// u(r) of one pair, FP64, terms in the order coulomb, LJ, WCA, HS (as the oracle and
// CombinedPairPotential::operator() src/potentials_base.h:234-240)
__device__ double pair_energy(const fau_nonbonded_args& a, int ta, int tb, double qa, double qb, double r2)
{
    if (a.pair_cutoff > 0.0 && r2 >= a.pair_cutoff * a.pair_cutoff) return 0.0;
    const int ab = ta * a.n_types + tb;
    double u = 0.0;
    if (a.pair_terms & FAU_PAIR_COULOMB) {
        if (a.coulomb_type == FAU_COUL_PLAIN) {
            u += a.bjerrum_length * qa * qb / sqrt(r2);
        }
        else {
            const double r = sqrt(r2) + 2.220446049250313e-16;
            if (r < a.coulomb_cutoff) {
                const double s = a.coulomb_type == FAU_COUL_EWALD ? erfc(a.coulomb_alpha * r) : 1.0;
                u += a.bjerrum_length * (qa * qb / r * s);
            }
        }
    }
    if (a.pair_terms & (FAU_PAIR_LJ | FAU_PAIR_WCA)) {
        const double s2 = a.sigma2[ab], e4 = a.eps4[ab];
        double x = s2 / r2;
        x = x * x * x;
        if (a.pair_terms & FAU_PAIR_LJ) u += e4 * (x * x - x);
        if (a.pair_terms & FAU_PAIR_WCA) u += (r2 > s2 * 1.2599210498948732) ? 0.0 : e4 * (x * x - x + 0.25);
    }
    if ((a.pair_terms & FAU_PAIR_HS) && r2 < a.hs_sigma2[ab]) u += __longlong_as_double(0x7ff0000000000000ULL);
    return u;
}

// partial[i] = sum_{j > i} u(r_ij), minimum image (Chameleon::sqdist src/geometry.h:460-485)
__global__ void noalloc_pair_kernel(fau_nonbonded_args a, double* partial)
{
    __shared__ double red[32];
    const double half[3] = {0.5 * a.box[0], 0.5 * a.box[1], 0.5 * a.box[2]};
    for (int i = blockIdx.x; i < a.n_particles; i += gridDim.x) {
        const double xi[3] = {a.pos[3 * i], a.pos[3 * i + 1], a.pos[3 * i + 2]};
        const int ti = a.type[i];
        const double qi = a.charge[i];
        double e = 0.0;
        for (int j = i + 1 + threadIdx.x; j < a.n_particles; j += blockDim.x) {
            double d[3];
            for (int k = 0; k < 3; k++) {
                double v = fabs(xi[k] - a.pos[3 * j + k]);
                // positions outside [-L/2, L/2] (an engine that has not wrapped them): whole box
                // lengths first (fmod is exact), then the reference's single subtraction
                if (v >= a.box[k]) v = fmod(v, a.box[k]);
                d[k] = v - (v > half[k] ? a.box[k] : 0.0);
            }
            const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
            e += pair_energy(a, ti, a.type[j], qi, a.charge[j], r2);
        }
        for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
            partial[i] = s;
        }
        __syncthreads();
    }
}

// energy = sum of the n partials in a fixed order (deterministic), one CTA
__global__ void noalloc_sum_kernel(const double* partial, int n, double* energy)
{
    __shared__ double red[1024];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *energy = red[0];
}

} // namespace

extern "C" int fau_nonbonded_energy_noalloc(const fau_nonbonded_args* a, double* energy_out, void* stream)
{
    if (!a || !energy_out) return fau_internal_fail(FAU_ERR_ARG, "null argument");
    if (a->coulomb_type < FAU_COUL_PLAIN || a->coulomb_type > FAU_COUL_EWALD)
        return fau_internal_fail(FAU_ERR_ARG, "coulomb_type: plain, cut or ewald only");
    if (a->pair_terms & ~(FAU_PAIR_COULOMB | FAU_PAIR_LJ | FAU_PAIR_WCA | FAU_PAIR_HS))
        return fau_internal_fail(FAU_ERR_ARG, "pair_terms: coulomb, LJ, WCA and HS only (no spline tables)");
    if (a->n_particles < 1 || a->n_particles > FAU_NOALLOC_MAX_PARTICLES)
        return fau_internal_fail(FAU_ERR_ARG,
                                 "n_particles outside [1, FAU_NOALLOC_MAX_PARTICLES = 65536]: the shared scratch "
                                 "array holds one partial sum per particle");
    if (!a->pos || !a->charge || !a->type || a->n_types < 1)
        return fau_internal_fail(FAU_ERR_ARG, "pos, charge, type and n_types are required");
    if ((a->pair_terms & (FAU_PAIR_LJ | FAU_PAIR_WCA)) && (!a->sigma2 || !a->eps4))
        return fau_internal_fail(FAU_ERR_ARG, "LJ/WCA need sigma2 and eps4");
    if ((a->pair_terms & FAU_PAIR_HS) && !a->hs_sigma2) return fau_internal_fail(FAU_ERR_ARG, "HS needs hs_sigma2");
    for (int k = 0; k < 3; k++)
        if (!(a->box[k] > 0.0) || !std::isfinite(a->box[k]))
            return fau_internal_fail(FAU_ERR_ARG, "box lengths must be positive and finite");
    // the settings the system entry point (fau_sys_create) also rejects
    if ((a->pair_terms & FAU_PAIR_COULOMB) && a->coulomb_type != FAU_COUL_PLAIN && !(a->coulomb_cutoff > 0.0))
        return fau_internal_fail(FAU_ERR_ARG, "coulomb_type cut or ewald needs a positive coulomb_cutoff");
    if ((a->pair_terms & FAU_PAIR_COULOMB) && a->coulomb_type == FAU_COUL_EWALD && !(a->coulomb_alpha >= 0.0))
        return fau_internal_fail(FAU_ERR_ARG, "coulomb_alpha must be >= 0");
    if (std::isnan(a->pair_cutoff))
        return fau_internal_fail(FAU_ERR_ARG, "pair_cutoff is NaN (<= 0 means no truncation)");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return fau_internal_fail(FAU_ERR_NODEVICE, "no current CUDA device");
    }
    double* partial = nullptr;
    {
        // set-up, once per device and context with that device current: the host-side name of
        // the array is not a device address, so look the address up and keep it
        std::lock_guard<std::mutex> lock(g_mu);
        const unsigned long long cid = current_context_id();
        if (!g_partial_ptr[dev] || cid != g_partial_ctx[dev]) {
            double* ptr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_partial);
            if (e != cudaSuccess) {
                g_partial_ptr[dev] = nullptr;
                return fau_internal_fail(FAU_ERR_CUDA, cudaGetErrorString(e));
            }
            g_partial_ptr[dev] = ptr;
            // the context is current now (the lookup made it so if it was not)
            g_partial_ctx[dev] = current_context_id();
        }
        partial = g_partial_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int blocks = a->n_particles < 4096 ? a->n_particles : 4096;
    noalloc_pair_kernel<<<blocks, 256, 0, st>>>(*a, partial);
    noalloc_sum_kernel<<<1, 1024, 0, st>>>(partial, a->n_particles, energy_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fau_internal_fail(FAU_ERR_CUDA, cudaGetErrorString(e));
    return FAU_OK;
}
