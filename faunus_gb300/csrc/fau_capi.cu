// fau_capi.cu -- host runtime behind the C ABI (include/fau_gpu.h).
//
// Owns device memory per system, builds the device tables (internal
// (type, charge) classes, pair matrices, Ewald k-vectors, cell list) and
// drives the kernels of fau_kernels.cu on the context's stream.
#include "fau_dev.cuh"
#include "fau_kernels.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

using namespace fau;

// ---------------------------------------------------------------- errors
static thread_local std::string g_last_error;

static int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CUDA_TRY(expr)                                                                                        \
    do {                                                                                                      \
        cudaError_t e_ = (expr);                                                                              \
        if (e_ != cudaSuccess) return fail(e_ == cudaErrorMemoryAllocation ? FAU_ERR_OOM : FAU_ERR_CUDA,      \
                                           "%s: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// ---------------------------------------------------------------- handles
struct fau_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t budget = 0, used = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // scratch for batched launches (grown on demand)
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    std::mutex mu;
    // caching device allocator: the blocks of destroyed systems, by size, reused by later
    // systems of this context (no cudaMalloc / cudaFree -- which synchronises the device --
    // per served job); returned to the driver when the context is destroyed
    std::multimap<size_t, void*> pool;
    size_t pool_bytes = 0;
};

// size class of a device block: multiples of 256 B up to 4 KiB, then 1/8 steps of the
// next power of two (at most 12.5 % slack)
static size_t block_class(size_t b)
{
    if (b <= 4096) return (b + 255) & ~size_t(255);
    size_t p = 4096;
    while (p < b) p <<= 1;
    const size_t step = p >> 3;
    return (b + step - 1) / step * step;
}

struct fau_sys {
    fau_ctx* ctx = nullptr;
    DevSys h{};                 // host mirror of the device struct (pointers are device pointers)
    DevSys* d = nullptr;        // device copy
    std::vector<void*> allocs;
    std::vector<size_t> alloc_bytes;
    size_t bytes = 0;
    int n = 0, n_groups = 0, K = 0;
    bool cells = false, molecular_only = false, all_atomic = true;
    std::vector<int> g_begin, g_flags, group_of;
    int max_group = 0;
    int precision = FAU_PREC_FP32C;
    // staging for run_proposals
    fau_proposal* d_props = nullptr;
    uint8_t* d_acc = nullptr;
    double* d_du = nullptr;
    fau_trial_result* d_detail = nullptr;
    size_t stage_cap = 0;
    PlainMove* d_plain = nullptr;
    double2* d_dq = nullptr;
    double* d_res = nullptr;
    double* d_partials = nullptr; // kTotalPartials per-block partial sums of the total energy
    int* d_flags = nullptr;
    DevSys** d_self = nullptr; // device array holding `d` (chain kernel argument)
    bool pending = false;      // a fau_energy_change trial waits for fau_commit_pending
    std::shared_ptr<const struct DescStore> desc; // the creating descriptor (volume moves rebuild from it)
};

// A host copy of a fau_sys_desc with its arrays (positions and mass centres excluded:
// they live on the device).  Shared by clones.
struct DescStore {
    fau_sys_desc d{};
    std::vector<double> charge, type_mass, sigma2, eps4, hs2, cut_pairs, spl_r2, spl_coef;
    std::vector<int> type, group_begin, group_molid, group_flags, spl_begin, spl_hs;
};

static std::shared_ptr<const DescStore> store_desc(const fau_sys_desc* d)
{
    auto st = std::make_shared<DescStore>();
    const size_t n = d->n_particles, g = d->n_groups, nt = d->n_types;
    auto cp = [](auto& v, const auto* p, size_t k) {
        if (p) v.assign(p, p + k);
        return p ? v.data() : nullptr;
    };
    st->d = *d;
    st->d.pos = nullptr;
    st->d.group_mass_center = nullptr;
    st->d.charge = cp(st->charge, d->charge, n);
    st->d.type = cp(st->type, d->type, n);
    st->d.group_begin = cp(st->group_begin, d->group_begin, g + 1);
    st->d.group_molid = cp(st->group_molid, d->group_molid, g);
    st->d.group_flags = cp(st->group_flags, d->group_flags, g);
    st->d.type_mass = cp(st->type_mass, d->type_mass, nt);
    st->d.sigma2 = cp(st->sigma2, d->sigma2, nt * nt);
    st->d.eps4 = cp(st->eps4, d->eps4, nt * nt);
    st->d.hs_sigma2 = cp(st->hs2, d->hs_sigma2, nt * nt);
    const size_t nm = d->cutoff_g2g_pairs && d->n_molids > 0 ? (size_t)d->n_molids * d->n_molids : 0;
    st->d.cutoff_g2g_pairs = nm ? cp(st->cut_pairs, d->cutoff_g2g_pairs, nm) : nullptr;
    if (d->pair_terms & FAU_PAIR_SPLINE) { // validated: nt^2 + 1 offsets, >= 2 knots a pair
        const size_t np = nt * nt, knots = (size_t)d->spline_begin[np];
        st->d.spline_begin = cp(st->spl_begin, d->spline_begin, np + 1);
        st->d.spline_r2 = cp(st->spl_r2, d->spline_r2, knots);
        st->d.spline_coef = cp(st->spl_coef, d->spline_coef, 6 * (knots - np));
        st->d.spline_hs = cp(st->spl_hs, d->spline_hs, np);
    }
    else {
        st->d.spline_begin = nullptr;
        st->d.spline_r2 = st->d.spline_coef = nullptr;
        st->d.spline_hs = nullptr;
    }
    return st;
}

template <class T>
static int dev_alloc(fau_sys* s, T** p, size_t count)
{
    const size_t b = block_class(std::max<size_t>(count, 1) * sizeof(T));
    if (s->ctx->budget && s->ctx->used + b > s->ctx->budget)
        return fail(FAU_ERR_OOM, "HBM budget exceeded (%zu + %zu > %zu bytes)", s->ctx->used, b, s->ctx->budget);
    void* v = nullptr;
    auto it = s->ctx->pool.find(b);
    if (it != s->ctx->pool.end()) { // a block of this class left by a destroyed system
        v = it->second;
        s->ctx->pool.erase(it);
        s->ctx->pool_bytes -= b;
    }
    else {
        CUDA_TRY(cudaMalloc(&v, b));
    }
    s->allocs.push_back(v);
    s->alloc_bytes.push_back(b);
    s->bytes += b;
    s->ctx->used += b;
    *p = static_cast<T*>(v);
    return FAU_OK;
}
template <class T>
static int upload(fau_sys* s, T** p, const T* src, size_t count)
{
    int rc = dev_alloc(s, p, count);
    if (rc) return rc;
    if (count) CUDA_TRY(cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, s->ctx->stream));
    return FAU_OK;
}

static void free_sys(fau_sys* s)
{
    // blocks go back to the context's pool (the caller has synchronised the stream)
    for (size_t a = 0; a < s->allocs.size(); a++) {
        s->ctx->pool.emplace(s->alloc_bytes[a], s->allocs[a]);
        s->ctx->pool_bytes += s->alloc_bytes[a];
    }
    if (s->ctx) s->ctx->used -= std::min(s->ctx->used, s->bytes);
    s->allocs.clear();
    s->alloc_bytes.clear();
    s->bytes = 0;
}

// ---------------------------------------------------------------- setup helpers
namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kTwo32 = 4294967296.0;

struct EwaldTable {
    std::vector<int> kn;
    std::vector<double> Ak;
};

// PolicyIonIon::updateBox (src/energy.cpp:133-186): nx in [0, nc], ny, nz in
// [-nc, nc], skip k^2 < 0.1 (2 pi / L_max)^2, spherical cut n^2 <= nc^2,
// A_k = f exp(-k^2 / 4 alpha^2) / k^2 with f = 2 for nx > 0 (kappa = 0).
EwaldTable build_kvectors(const double L[3], double alpha, double ncut, bool spherical)
{
    EwaldTable t;
    const int nc = (int)std::ceil(ncut);
    const double Lmax = std::max(L[0], std::max(L[1], L[2]));
    const double check_k2_zero = 0.1 * std::pow(2 * kPi / Lmax, 2);
    if ((2 * nc + 1) * (2 * nc + 1) * (2 * nc + 1) - 1 == 0) return t;
    const double nc2 = ncut * ncut;
    for (int nx = 0; nx <= nc; nx++) {
        const double dnx2 = double(nx * nx);
        const double factor = nx > 0 ? 2.0 : 1.0;
        for (int ny = -nc; ny <= nc; ny++) {
            const double dny2 = double(ny * ny);
            for (int nz = -nc; nz <= nc; nz++) {
                const double kx = 2 * kPi * (double(nx) / L[0]);
                const double ky = 2 * kPi * (double(ny) / L[1]);
                const double kz = 2 * kPi * (double(nz) / L[2]);
                const double k2 = (kx * kx + ky * ky) + kz * kz;
                if (k2 < check_k2_zero) continue;
                if (spherical && (dnx2 + dny2 + double(nz * nz)) / nc2 > 1) continue;
                t.kn.push_back((nx + 128) | ((ny + 128) << 8) | ((nz + 128) << 16));
                t.Ak.push_back(factor * std::exp(-k2 / (4 * alpha * alpha)) / k2);
            }
        }
    }
    return t;
}

int validate(const fau_sys_desc* d)
{
    if (!d) return fail(FAU_ERR_ARG, "null descriptor");
    if (d->n_particles < 1 || d->n_particles > (1 << 24) - 1)
        return fail(FAU_ERR_ARG, "n_particles %d outside [1, 2^24)", d->n_particles);
    if (!d->pos || !d->charge || !d->type) return fail(FAU_ERR_ARG, "pos, charge and type are required");
    if (d->n_groups < 1 || !d->group_begin) return fail(FAU_ERR_ARG, "at least one group is required");
    if (d->group_begin[0] != 0 || d->group_begin[d->n_groups] != d->n_particles)
        return fail(FAU_ERR_ARG, "group_begin must start at 0 and end at n_particles");
    for (int g = 0; g < d->n_groups; g++)
        if (d->group_begin[g + 1] < d->group_begin[g]) return fail(FAU_ERR_ARG, "group_begin not sorted");
    for (int k = 0; k < 3; k++)
        if (!(d->box[k] > 0.0)) return fail(FAU_ERR_ARG, "box lengths must be positive");
    if (d->n_types < 1) return fail(FAU_ERR_ARG, "n_types must be >= 1");
    if (d->cell_staging < 0 || d->cell_staging > 2) return fail(FAU_ERR_ARG, "cell_staging must be 0, 1 or 2");
    for (int i = 0; i < d->n_particles; i++) {
        if (d->type[i] < 0 || d->type[i] >= d->n_types) return fail(FAU_ERR_ARG, "particle %d: type out of range", i);
        for (int k = 0; k < 3; k++) {
            const double x = d->pos[3 * i + k];
            if (!std::isfinite(x)) return fail(FAU_ERR_ARG, "particle %d: non-finite position", i);
            if (std::fabs(x) > 0.5 * d->box[k]) return fail(FAU_ERR_ARG, "particle %d: position outside the box", i);
        }
        if (!std::isfinite(d->charge[i])) return fail(FAU_ERR_ARG, "particle %d: non-finite charge", i);
    }
    if ((d->pair_terms & (FAU_PAIR_LJ | FAU_PAIR_WCA)) && (!d->sigma2 || !d->eps4))
        return fail(FAU_ERR_ARG, "LJ/WCA need sigma2 and eps4 tables");
    if ((d->pair_terms & FAU_PAIR_HS) && !d->hs_sigma2) return fail(FAU_ERR_ARG, "HS needs hs_sigma2");
    if (d->ewald.enabled) {
        if (!(d->ewald.alpha > 0.0)) return fail(FAU_ERR_ARG, "ewald.alpha must be positive");
        if (d->ewald.ncutoff > 127) return fail(FAU_ERR_ARG, "ewald.ncutoff above 127");
    }
    if (d->coulomb_type < FAU_COUL_PLAIN || d->coulomb_type > FAU_COUL_TRUNC)
        return fail(FAU_ERR_ARG, "unknown coulomb_type %d", d->coulomb_type);
    if (d->coulomb_type != FAU_COUL_PLAIN && (d->pair_terms & FAU_PAIR_COULOMB) && !(d->coulomb_cutoff > 0.0))
        return fail(FAU_ERR_ARG, "coulomb_type %d needs a positive coulomb_cutoff", d->coulomb_type);
    if (d->coulomb_type == FAU_COUL_TRUNC) {
        if (d->coulomb_poly_n < 0 || d->coulomb_poly_n > FAU_COUL_MAX_POLY)
            return fail(FAU_ERR_ARG, "coulomb_poly_n %d outside [0, %d]", d->coulomb_poly_n, FAU_COUL_MAX_POLY);
        if (!std::isfinite(d->coulomb_erfc)) return fail(FAU_ERR_ARG, "non-finite coulomb_erfc");
        for (int k = 0; k < d->coulomb_poly_n; k++)
            if (!std::isfinite(d->coulomb_poly[k])) return fail(FAU_ERR_ARG, "non-finite coulomb_poly[%d]", k);
    }
    if (d->cutoff_g2g_pairs) {
        if (d->n_molids < 1 || d->n_molids > 4096) return fail(FAU_ERR_ARG, "n_molids %d outside [1, 4096]", d->n_molids);
        if (!d->group_molid) return fail(FAU_ERR_ARG, "cutoff_g2g_pairs needs group_molid");
        for (int g = 0; g < d->n_groups; g++)
            if (d->group_molid[g] < 0 || d->group_molid[g] >= d->n_molids)
                return fail(FAU_ERR_ARG, "group %d: molecule id %d outside [0, n_molids)", g, d->group_molid[g]);
        for (long k = 0; k < (long)d->n_molids * d->n_molids; k++)
            if (std::isnan(d->cutoff_g2g_pairs[k])) return fail(FAU_ERR_ARG, "cutoff_g2g_pairs holds NaN");
    }
    if (d->precision != FAU_PREC_FP32C && d->precision != FAU_PREC_FP64)
        return fail(FAU_ERR_ARG, "unknown precision %d", d->precision);
    if (d->isobaric && !std::isfinite(d->pressure)) return fail(FAU_ERR_ARG, "non-finite Isobaric pressure");
    if (d->maxenergy_set && std::isnan(d->maxenergy)) return fail(FAU_ERR_ARG, "maxenergy is NaN");
    if (d->pair_terms & ~(FAU_PAIR_COULOMB | FAU_PAIR_LJ | FAU_PAIR_WCA | FAU_PAIR_HS | FAU_PAIR_SPLINE))
        return fail(FAU_ERR_ARG, "unknown pair_terms bits 0x%x", d->pair_terms);
    if (d->pair_terms & FAU_PAIR_SPLINE) {
        if (!d->spline_begin || !d->spline_r2 || !d->spline_coef)
            return fail(FAU_ERR_ARG, "FAU_PAIR_SPLINE needs spline_begin, spline_r2 and spline_coef");
        const long np = (long)d->n_types * d->n_types;
        if (d->spline_begin[0] != 0) return fail(FAU_ERR_ARG, "spline_begin must start at 0");
        for (long ab = 0; ab < np; ab++) {
            const long b0 = d->spline_begin[ab], b1 = d->spline_begin[ab + 1];
            if (b1 - b0 < 2 || b1 - b0 > (1 << 20))
                return fail(FAU_ERR_ARG, "type pair %ld: %ld spline knots (2 .. 2^20)", ab, b1 - b0);
            for (long k = b0; k < b1; k++) {
                const double z = d->spline_r2[k];
                if (!std::isfinite(z) || z < 0.0 || (k > b0 && !(z > d->spline_r2[k - 1])))
                    return fail(FAU_ERR_ARG, "type pair %ld: spline knots must be finite, >= 0 and ascending", ab);
            }
            for (long k = 6 * (b0 - ab); k < 6 * (b1 - ab - 1); k++)
                if (!std::isfinite(d->spline_coef[k]))
                    return fail(FAU_ERR_ARG, "type pair %ld: non-finite spline coefficient", ab);
        }
    }
    return FAU_OK;
}

struct Layout {
    std::vector<int> itype;          // per particle
    std::vector<int> itype_type;     // per itype
    std::vector<double> itype_q;     // per itype
    bool cells = false;
    int cdim[3] = {1, 1, 1};
    double cell_len[3] = {0, 0, 0};
    int off_min[3] = {0, 0, 0}, off_max[3] = {0, 0, 0};
    int cap = 0;
    int K = 0;
    EwaldTable ew;
};

int plan_layout(const fau_sys_desc* d, Layout& lay)
{
    std::map<std::pair<int, double>, int> cls;
    lay.itype.resize(d->n_particles);
    for (int i = 0; i < d->n_particles; i++) {
        auto key = std::make_pair(d->type[i], d->charge[i]);
        auto it = cls.find(key);
        if (it == cls.end()) {
            if ((int)cls.size() == kMaxITypes)
                return fail(FAU_ERR_ARG, "more than %d distinct (type, charge) classes", kMaxITypes);
            it = cls.emplace(key, (int)cls.size()).first;
            lay.itype_type.push_back(d->type[i]);
            lay.itype_q.push_back(d->charge[i]);
        }
        lay.itype[i] = it->second;
    }
    bool all_atomic = true;
    for (int g = 0; g < d->n_groups; g++)
        if (!(d->group_flags ? (d->group_flags[g] & FAU_GROUP_ATOMIC) : 1)) all_atomic = false;
    // cell grid (GridBase::updateCellGrid src/celllistimpl.h:223-236) with the pair cutoff as
    // the minimal cell dimension; only for all-atomic systems with a finite cutoff.
    if (d->pair_cutoff > 0.0 && all_atomic) {
        int ncell = 1;
        for (int k = 0; k < 3; k++) {
            lay.cdim[k] = (int)std::floor(d->box[k] / std::min(d->box[k], d->pair_cutoff));
            lay.cell_len[k] = d->box[k] / double(lay.cdim[k]);
            // distance-1 neighbour offsets clamped by the periodic grid's wrap-around limits
            // (GridOffsets3D src/celllistimpl.cpp:15-31, src/celllistimpl.h:409-415)
            const double mid = (lay.cdim[k] - 1) * 0.5;
            lay.off_min[k] = std::max(-1, -(int)std::floor(mid));
            lay.off_max[k] = std::min(1, (int)std::ceil(mid));
            ncell *= lay.cdim[k];
        }
        if (d->box[0] < 2 * d->pair_cutoff || d->box[1] < 2 * d->pair_cutoff || d->box[2] < 2 * d->pair_cutoff)
            ncell = 0; // minimum image + cutoff already covers every pair: all-pairs is cheaper
        lay.cells = ncell >= 27;
    }
    if (d->ewald.enabled) {
        lay.ew = build_kvectors(d->box, d->ewald.alpha, d->ewald.ncutoff, d->ewald.spherical_sum != 0);
        lay.K = (int)lay.ew.kn.size();
    }
    return FAU_OK;
}

// slots per cell: at least the requested count (else twice the mean occupancy
// plus four), four more than the fullest cell, at least 8, rounded up to a
// power of two so a slot index splits into (cell, slot) by shifts
int cell_capacity(int requested, int maxc, double mean)
{
    int c = requested > 0 ? requested : (int)std::ceil(2.0 * mean) + 4;
    c = std::max(std::max(c, maxc + 4), 8);
    int p = 8;
    while (p < c) p *= 2;
    return p;
}

// bin one position, reference formula (bit-exact with the oracle)
int host_cell(const double* x, const double L[3], const int dims[3], const double cell[3])
{
    int c[3];
    for (int k = 0; k < 3; k++) {
        const double t = x[k] + 0.5 * L[k];
        int v = (int)std::floor(t / cell[k]);
        if (v < 0) v += dims[k] * (std::abs(v) / dims[k] + 1);
        else if (v >= dims[k]) v -= dims[k] * (v / dims[k]);
        c[k] = v;
    }
    return c[0] + dims[0] * (c[1] + dims[1] * c[2]);
}

size_t footprint_bytes(const fau_sys_desc* d, const Layout& lay, int cap)
{
    const size_t n = d->n_particles, g = d->n_groups, nt = lay.itype_q.size();
    size_t b = n * (3 * 8 + 16 + 4) + nt * (4 + 8 + 8) + (g + 1) * 4 + g * (4 + 24 + 16) + n * 4 +
               nt * nt * (16 + 32) + sizeof(DevSys);
    if (lay.cells) {
        const size_t nc = (size_t)lay.cdim[0] * lay.cdim[1] * lay.cdim[2];
        b += nc * 4 + nc * (size_t)cap * 16 + n * 8;
    }
    b += (size_t)lay.K * (4 + 4 + 8 + 16 + 16 + 8 + 8);
    b += sizeof(PlainMove) + 64 + sizeof(void*);
    if (d->cutoff_g2g_pairs && d->n_molids > 0) b += g * 4 + (size_t)d->n_molids * d->n_molids * (8 + 4);
    b += g * 64; // mass-centre cells of molecular groups (at most ~16 slots a group in practice)
    if (d->pair_terms & FAU_PAIR_SPLINE) { // every class pair a copy of its atom-type pair's table
        size_t most = 0;
        const size_t T = d->n_types;
        for (size_t ab = 0; ab < T * T; ab++)
            most = std::max(most, (size_t)(d->spline_begin[ab + 1] - d->spline_begin[ab]));
        b += nt * nt * (sizeof(SplineP) + most * (4 + 8 + 6 * (4 + 8)) + kSplineGrid * 4);
    }
    return b;
}

} // namespace

// ================================================================== C ABI
extern "C" {

int fau_abi_version(void) { return FAU_ABI_VERSION; }

const char* fau_strerror(int status)
{
    switch (status) {
    case FAU_OK: return "ok";
    case FAU_ERR_ARG: return "invalid argument";
    case FAU_ERR_OOM: return "out of device memory or HBM budget";
    case FAU_ERR_CUDA: return "CUDA error";
    case FAU_ERR_TIMEOUT: return "device wait timed out";
    case FAU_ERR_NAN: return "Metropolis error: energy cannot be NaN";
    case FAU_ERR_CAPACITY: return "cell list capacity exceeded";
    case FAU_ERR_STATE: return "invalid state";
    case FAU_ERR_NODEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

const char* fau_last_error(void) { return g_last_error.c_str(); }

int fau_ctx_create(int device, size_t hbm_budget_bytes, fau_ctx** out)
{
    if (!out) return fail(FAU_ERR_ARG, "null output");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(FAU_ERR_NODEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= count) return fail(FAU_ERR_ARG, "device %d out of range", device);
    CUDA_TRY(cudaSetDevice(device));
    fau_ctx* c = new fau_ctx;
    c->device = device;
    c->budget = hbm_budget_bytes;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
        delete c;
        return fail(FAU_ERR_CUDA, "stream/event creation failed");
    }
    *out = c;
    return FAU_OK;
}

int fau_ctx_destroy(fau_ctx* c)
{
    if (!c) return FAU_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->scratch) cudaFree(c->scratch);
    for (auto& kv : c->pool) cudaFree(kv.second);
    c->pool.clear();
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FAU_OK;
}

int fau_ctx_hbm_used(const fau_ctx* c, size_t* used)
{
    if (!c || !used) return fail(FAU_ERR_ARG, "null argument");
    *used = c->used;
    return FAU_OK;
}

int fau_sys_footprint(const fau_sys_desc* d, size_t* bytes)
{
    int rc = validate(d);
    if (rc) return rc;
    Layout lay;
    rc = plan_layout(d, lay);
    if (rc) return rc;
    int cap = 0;
    if (lay.cells) {
        const double ncell = (double)lay.cdim[0] * lay.cdim[1] * lay.cdim[2];
        cap = cell_capacity(d->cell_capacity, 0, d->n_particles / ncell);
    }
    *bytes = footprint_bytes(d, lay, cap);
    return FAU_OK;
}

static int refresh_energy(fau_sys* s);

int fau_sys_create(fau_ctx* ctx, const fau_sys_desc* d, fau_sys** out)
{
    const fau::NvtxRange nvtx_range("fau_sys_create");
    if (!ctx || !out) return fail(FAU_ERR_ARG, "null argument");
    int rc = validate(d);
    if (rc) return rc;
    CUDA_TRY(cudaSetDevice(ctx->device));
    Layout lay;
    rc = plan_layout(d, lay);
    if (rc) return rc;

    fau_sys* s = new fau_sys;
    s->ctx = ctx;
    s->n = d->n_particles;
    s->n_groups = d->n_groups;
    s->K = lay.K;
    s->cells = lay.cells;
    s->precision = d->precision;
    DevSys& h = s->h;
    std::memset(&h, 0, sizeof(h));
    auto bail = [&](int code) {
        cudaStreamSynchronize(ctx->stream);
        free_sys(s);
        delete s;
        return code;
    };

    // geometry
    for (int k = 0; k < 3; k++) {
        h.L[k] = d->box[k];
        h.half[k] = 0.5 * d->box[k];
        h.inv[k] = 1.0 / d->box[k];
        h.fx_scale[k] = kTwo32 / d->box[k];
        h.fx_len[k] = (float)(d->box[k] / kTwo32);
        h.fx_lend[k] = d->box[k] / kTwo32;
        h.inv_f[k] = (float)(1.0 / d->box[k]);
    }
    const int n = d->n_particles;
    h.n = n;
    h.n_groups = d->n_groups;

    // particles
    std::vector<double> x(n), y(n), z(n);
    std::vector<uint4> rec(n);
    for (int i = 0; i < n; i++) {
        x[i] = d->pos[3 * i];
        y[i] = d->pos[3 * i + 1];
        z[i] = d->pos[3 * i + 2];
        rec[i] = make_uint4(to_fixed(x[i], h.fx_scale[0]), to_fixed(y[i], h.fx_scale[1]), to_fixed(z[i], h.fx_scale[2]),
                            ((uint32_t)lay.itype[i] << 24) | (uint32_t)i);
    }
    // groups
    const int G = d->n_groups;
    s->g_begin.assign(d->group_begin, d->group_begin + G + 1);
    s->g_flags.resize(G);
    std::vector<int> group_of(n);
    std::vector<double> cm(3 * G, 0.0);
    std::vector<uint4> cmrec(G);
    std::vector<int> atomic_idx;
    bool molecular_only = true;
    for (int g = 0; g < G; g++) {
        s->g_flags[g] = d->group_flags ? d->group_flags[g] : FAU_GROUP_ATOMIC;
        const int b = d->group_begin[g], e = d->group_begin[g + 1];
        s->max_group = std::max(s->max_group, e - b);
        for (int i = b; i < e; i++) group_of[i] = g;
        if (s->g_flags[g] & FAU_GROUP_ATOMIC) {
            molecular_only = false;
            for (int i = b; i < e; i++) atomic_idx.push_back(i);
        }
        if (d->group_mass_center) {
            for (int k = 0; k < 3; k++) cm[3 * g + k] = d->group_mass_center[3 * g + k];
        }
        else if (!(s->g_flags[g] & FAU_GROUP_ATOMIC) && e > b) {
            // Group::updateMassCenter (src/group.cpp:136-157): shift by the middle particle,
            // weighted centre (src/geometry.h:505-526), boundary, shift back.
            const int mid = b + (e - b) / 2;
            const double sh[3] = {-d->pos[3 * mid], -d->pos[3 * mid + 1], -d->pos[3 * mid + 2]};
            double c[3] = {0, 0, 0}, ws = 0;
            for (int i = b; i < e; i++) {
                double p[3];
                for (int k = 0; k < 3; k++) {
                    p[k] = d->pos[3 * i + k] + sh[k];
                    if (std::fabs(p[k]) > h.half[k]) {
                        const double t = p[k] * h.inv[k];
                        p[k] -= h.L[k] * (int)(t > 0.0 ? t + 0.5 : t - 0.5);
                    }
                }
                const double w = d->type_mass ? d->type_mass[d->type[i]] : 1.0;
                for (int k = 0; k < 3; k++) c[k] += w * p[k];
                ws += w;
            }
            if (std::fabs(ws) > 2.220446049250313e-16) {
                for (int k = 0; k < 3; k++) {
                    double v = c[k] / ws - sh[k];
                    if (std::fabs(v) > h.half[k]) {
                        const double t = v * h.inv[k];
                        v -= h.L[k] * (int)(t > 0.0 ? t + 0.5 : t - 0.5);
                    }
                    cm[3 * g + k] = v;
                }
            }
        }
        cmrec[g] = make_uint4(to_fixed(cm[3 * g], h.fx_scale[0]), to_fixed(cm[3 * g + 1], h.fx_scale[1]),
                              to_fixed(cm[3 * g + 2], h.fx_scale[2]), 0u);
    }
    s->molecular_only = molecular_only;
    for (int g = 0; g < d->n_groups; g++)
        if (!(d->group_flags ? (d->group_flags[g] & FAU_GROUP_ATOMIC) : 1)) s->all_atomic = false;
    s->group_of = group_of;

    // pair tables over internal classes
    const int nt = (int)lay.itype_q.size();
    const int T = d->n_types;
    std::vector<PairF> pf(nt * nt);
    std::vector<double> pd(4 * nt * nt);
    for (int a = 0; a < nt; a++)
        for (int b = 0; b < nt; b++) {
            const int ta = lay.itype_type[a], tb = lay.itype_type[b];
            const double s2 = d->sigma2 ? d->sigma2[ta * T + tb] : 0.0;
            const double e4 = d->eps4 ? d->eps4[ta * T + tb] : 0.0;
            const double hs = d->hs_sigma2 ? d->hs_sigma2[ta * T + tb] : 0.0;
            const double qq = d->bjerrum_length * lay.itype_q[a] * lay.itype_q[b];
            pf[a * nt + b] = {(float)s2, (float)e4, (float)hs, (float)qq};
            pd[4 * (a * nt + b) + 0] = s2;
            pd[4 * (a * nt + b) + 1] = e4;
            pd[4 * (a * nt + b) + 2] = hs;
            pd[4 * (a * nt + b) + 3] = qq;
        }
    std::vector<float> iq(nt);
    std::vector<double> iqd(nt), iself(nt, 0.0);
    // self energy lB q^2 S'(0) / (2 Rc) = -1/2 lim_{r->0} (u - u~) (docs/_docs/energy.md:267-276):
    // Ewald S'(0) = -2 alpha Rc / sqrt(pi); FAU_COUL_TRUNC S'(0) = c_1 - e 2 alpha Rc / sqrt(pi)
    const bool has_self = (d->pair_terms & FAU_PAIR_COULOMB) &&
                          (d->coulomb_type == FAU_COUL_EWALD || d->coulomb_type == FAU_COUL_TRUNC);
    double self_pref = 0.0; // U_self / (lB q^2)
    if (d->coulomb_type == FAU_COUL_EWALD) self_pref = -d->coulomb_alpha / std::sqrt(kPi);
    if (d->coulomb_type == FAU_COUL_TRUNC) {
        const double c1 = d->coulomb_poly_n > 1 ? d->coulomb_poly[1] : 0.0;
        const double ds0 = c1 - d->coulomb_erfc * 2.0 * d->coulomb_alpha * d->coulomb_cutoff / std::sqrt(kPi);
        self_pref = ds0 / (2.0 * d->coulomb_cutoff);
    }
    for (int a = 0; a < nt; a++) {
        iq[a] = (float)lay.itype_q[a];
        iqd[a] = lay.itype_q[a];
        // NewCoulombGalore self energy for S = erfc(alpha r): -lB alpha / sqrt(pi) q^2
        if (has_self) iself[a] = d->bjerrum_length * (self_pref * iqd[a] * iqd[a]);
    }
    h.nt = nt;
    h.terms = d->pair_terms;
    h.coul_type = d->coulomb_type;
    h.lB = (float)d->bjerrum_length;
    h.lB_d = d->bjerrum_length;
    h.rc_coul = (float)d->coulomb_cutoff;
    h.rc_coul_d = d->coulomb_cutoff;
    h.rc2_coul = (float)(d->coulomb_cutoff * d->coulomb_cutoff);
    h.alpha = (float)d->coulomb_alpha;
    h.alpha_d = d->coulomb_alpha;
    if (d->coulomb_type == FAU_COUL_TRUNC) {
        h.npoly = d->coulomb_poly_n;
        for (int k = 0; k < d->coulomb_poly_n; k++) {
            h.cpoly_d[k] = d->coulomb_poly[k];
            h.cpoly[k] = (float)d->coulomb_poly[k];
        }
        h.cerfc_d = d->coulomb_erfc;
        h.cerfc = (float)d->coulomb_erfc;
        h.inv_rc_d = 1.0 / d->coulomb_cutoff;
        h.inv_rc = (float)h.inv_rc_d;
    }
    h.rc2_pair = d->pair_cutoff > 0 ? (float)(d->pair_cutoff * d->pair_cutoff) : 0.f;
    h.rc2_pair_d = d->pair_cutoff > 0 ? d->pair_cutoff * d->pair_cutoff : 0.0;
    h.cut_g2g2 = d->cutoff_g2g > 0 ? d->cutoff_g2g * d->cutoff_g2g : -1.0;
    std::vector<double> cut2_mol;
    std::vector<float> cut2_molf;
    std::vector<int> g_molid;
    if (d->cutoff_g2g_pairs && d->n_molids > 0) { // GroupCutoff::getCutoff per molecule-kind pair
        const size_t nm = (size_t)d->n_molids;
        cut2_mol.resize(nm * nm);
        cut2_molf.resize(nm * nm);
        h.cut_g2g2 = -1.0;
        for (size_t k = 0; k < nm * nm; k++) {
            const double c = d->cutoff_g2g_pairs[k];
            cut2_mol[k] = (c > 0 && std::isfinite(c)) ? c * c : -1.0;
            cut2_molf[k] = (float)cut2_mol[k];
            if (cut2_mol[k] >= 0.0) h.cut_g2g2 = 0.0; // some pair has a cutoff
        }
        g_molid.assign(d->group_molid, d->group_molid + d->n_groups);
        h.n_mol = d->n_molids;
    }
    h.cut_g2g2f = (float)h.cut_g2g2;
    // mass-centre cells of the molecular groups: as wide as the largest cutoff between molecule
    // kinds that have molecular groups (+1e-9), when every such pair has one and some axis holds
    // more than three; the molecular kernel lists them at its start and keeps them current
    std::vector<int> gc_cnt0;
    if (!s->all_atomic) {
        std::vector<char> used(std::max(1, h.n_mol), 0);
        for (int g = 0; g < d->n_groups; g++)
            if (!(d->group_flags ? (d->group_flags[g] & FAU_GROUP_ATOMIC) : 1)) used[h.n_mol > 0 ? g_molid[g] : 0] = 1;
        double rc2 = -1.0;
        bool finite = true;
        if (h.n_mol > 0) {
            for (int a = 0; a < h.n_mol; a++)
                for (int b = 0; b < h.n_mol; b++) {
                    if (!used[a] || !used[b]) continue;
                    const double c2 = cut2_mol[(size_t)a * h.n_mol + b];
                    if (c2 < 0.0) finite = false;
                    rc2 = std::max(rc2, c2);
                }
        }
        else {
            finite = h.cut_g2g2 >= 0.0;
            rc2 = h.cut_g2g2;
        }
        if (finite && rc2 > 0.0) {
            const double rc = std::sqrt(rc2) * (1.0 + 1e-9);
            int gd[3];
            long tot = 1;
            bool wide = true;
            for (int k = 0; k < 3; k++) {
                gd[k] = (int)std::floor(d->box[k] / rc);
                wide = wide && gd[k] >= 3;
                tot *= std::max(gd[k], 1);
            }
            if (wide && tot > 27 && tot <= (1L << 20)) {
                std::vector<int> cnt(tot, 0);
                int nmol = 0;
                for (int g = 0; g < d->n_groups; g++) {
                    if (d->group_flags ? (d->group_flags[g] & FAU_GROUP_ATOMIC) : 1) continue;
                    int c[3];
                    for (int k = 0; k < 3; k++) {
                        int v = (int)std::floor((cm[3 * g + k] + 0.5 * d->box[k]) * (gd[k] / d->box[k]));
                        c[k] = std::min(std::max(v, 0), gd[k] - 1);
                    }
                    cnt[c[0] + gd[0] * (c[1] + gd[1] * c[2])]++;
                    nmol++;
                }
                const int maxc = *std::max_element(cnt.begin(), cnt.end());
                const int want = std::max(64, std::max(2 * maxc, 4 * (int)std::ceil(nmol / (double)tot)));
                int cap = 32, sh = 5;
                while (cap < want) {
                    cap *= 2;
                    sh++;
                }
                for (int k = 0; k < 3; k++) {
                    h.gdim[k] = gd[k];
                    h.ginv[k] = gd[k] / d->box[k];
                }
                h.gncell = (int)tot;
                h.gcap = cap;
                h.gshift = sh;
                gc_cnt0.assign(tot, 0);
            }
        }
    }
    for (size_t a = 0; a < lay.itype_type.size() && a < (size_t)kMaxITypes; a++) h.itype_type[a] = lay.itype_type[a];
    const bool spread = fast_spread_cells(lay.cells, n, lay.cdim[0] * lay.cdim[1] * lay.cdim[2]);
    const bool occ = fast_occupied_slots(lay.cells) && (d->cell_staging == 0 || (d->cell_staging == 2 && spread));
    h.flags = (lay.cells ? SYS_CELLS : 0) | (d->ewald.enabled ? SYS_EWALD : 0) |
              ((d->ewald.enabled && d->ewald.epss >= 1.0) ? SYS_SURFACE : 0) | (has_self ? SYS_SELF : 0) |
              (occ ? SYS_OCC : 0) | (spread ? SYS_SPREAD : 0);
    h.beta_scale = 1.0;
    h.maxe = d->maxenergy_set ? 1 : 0;
    h.maxenergy = d->maxenergy_set ? d->maxenergy : std::numeric_limits<double>::infinity();

#define UP(dst, vec) \
    if ((rc = upload(s, &dst, vec.data(), vec.size()))) return bail(rc)
    UP(h.x, x);
    UP(h.y, y);
    UP(h.z, z);
    UP(h.rec, rec);
    UP(h.group_of, group_of);
    UP(h.itype_q, iq);
    UP(h.itype_qd, iqd);
    UP(h.itype_self, iself);
    UP(h.g_begin, s->g_begin);
    UP(h.g_flags, s->g_flags);
    UP(h.g_cm, cm);
    UP(h.g_cmrec, cmrec);
    UP(h.atomic_idx, atomic_idx);
    if (h.n_mol > 0) {
        UP(h.g_molid, g_molid);
        UP(h.cut2_mol, cut2_mol);
        UP(h.cut2_molf, cut2_molf);
    }
    h.n_atomic = molecular_only ? 0 : (int)atomic_idx.size();
    if (!molecular_only && (int)atomic_idx.size() == n) h.n_atomic = 0; // all atomic: index = particle
    UP(h.pair, pf);
    UP(h.pair_d, pd);
    if (h.gncell > 0) { // contents listed by the molecular kernel at its start
        std::vector<int> lst((size_t)h.gncell * h.gcap, 0);
        UP(h.gc_cnt, gc_cnt0);
        UP(h.gc_list, lst);
    }
    if (d->pair_terms & FAU_PAIR_SPLINE) { // nonbonded_splined: the atom-type pair tables per class pair
        std::vector<SplineP> spl(nt * nt);
        std::vector<float> zf, cf;
        std::vector<double> zd, cd;
        std::vector<int> grid;
        std::vector<int> at(T * T, -1); // atom-type pair -> its first class pair (tables shared)
        for (int a = 0; a < nt; a++)
            for (int b = 0; b < nt; b++) {
                const int ab = lay.itype_type[a] * T + lay.itype_type[b];
                if (at[ab] >= 0) {
                    spl[a * nt + b] = spl[at[ab]];
                    continue;
                }
                at[ab] = a * nt + b;
                const int b0 = d->spline_begin[ab], m = d->spline_begin[ab + 1] - b0;
                const double* z = d->spline_r2 + b0;
                const double* c = d->spline_coef + 6 * (size_t)(b0 - ab);
                SplineP q{};
                q.zmin_d = z[0];
                q.zmax_d = z[m - 1];
                q.zmin = (float)z[0];
                q.zmax = (float)z[m - 1];
                q.knot0 = (int)zf.size();
                q.coef0 = (int)cf.size();
                q.pieces = m - 1;
                q.grid0 = (int)grid.size();
                q.grid_n = kSplineGrid;
                q.inv_h = (float)(kSplineGrid / (z[m - 1] - z[0]));
                q.hs = d->spline_hs ? (d->spline_hs[ab] != 0) : 0;
                for (int k = 0; k < m; k++) {
                    zf.push_back((float)z[k]);
                    zd.push_back(z[k]);
                }
                for (int k = 0; k < 6 * (m - 1); k++) {
                    cf.push_back((float)c[k]);
                    cd.push_back(c[k]);
                }
                // each cell's start: the last piece whose lower knot is at or below it
                const double hz = (z[m - 1] - z[0]) / kSplineGrid;
                int i = 0;
                for (int g = 0; g < kSplineGrid; g++) {
                    const double zg = z[0] + g * hz;
                    while (i < m - 2 && z[i + 1] <= zg) i++;
                    grid.push_back(i);
                }
                spl[a * nt + b] = q;
            }
        UP(h.spl, spl);
        UP(h.spl_zf, zf);
        UP(h.spl_zd, zd);
        UP(h.spl_cf, cf);
        UP(h.spl_cd, cd);
        UP(h.spl_grid, grid);
    }

    // cell list
    if (lay.cells) {
        const int ncell = lay.cdim[0] * lay.cdim[1] * lay.cdim[2];
        std::vector<int> cnt(ncell, 0), cell_of(n), slot_of(n);
        for (int i = 0; i < n; i++) {
            const double p[3] = {x[i], y[i], z[i]};
            cell_of[i] = host_cell(p, d->box, lay.cdim, lay.cell_len);
            slot_of[i] = cnt[cell_of[i]]++;
        }
        const int maxc = *std::max_element(cnt.begin(), cnt.end());
        const int cap = cell_capacity(d->cell_capacity, maxc, n / (double)ncell);
        std::vector<uint4> crec((size_t)ncell * cap, make_uint4(0, 0, 0, 0xFFFFFFFFu));
        for (int i = 0; i < n; i++) crec[(size_t)cell_of[i] * cap + slot_of[i]] = rec[i];
        for (int k = 0; k < 3; k++) {
            h.cdim[k] = lay.cdim[k];
            h.cell_len[k] = lay.cell_len[k];
            h.off_min[k] = lay.off_min[k];
            h.off_max[k] = lay.off_max[k];
        }
        h.ncell = ncell;
        h.cap = cap;
        UP(h.cell_cnt, cnt);
        UP(h.cell_rec, crec);
        UP(h.cell_of, cell_of);
        UP(h.slot_of, slot_of);
    }

    // Ewald
    if (d->ewald.enabled) {
        std::vector<float> akf(lay.K);
        for (int k = 0; k < lay.K; k++) akf[k] = (float)lay.ew.Ak[k];
        h.K = lay.K;
        int knc = 0;
        for (int v : lay.ew.kn) {
            const int a = std::abs((v & 0xff) - 128), b = std::abs(((v >> 8) & 0xff) - 128),
                      c = std::abs(((v >> 16) & 0xff) - 128);
            knc = std::max(knc, std::max(a, std::max(b, c)));
        }
        h.knc = knc;
        if (lay.K > chain_max_k(128) || chain_smem_bytes(lay.K, knc) + 16384 > 227 * 1024)
            return bail(fail(FAU_ERR_ARG, "%d k-vectors exceed the chain kernel's shared-memory budget", lay.K));
        UP(h.kn, lay.ew.kn);
        UP(h.Ak, akf);
        UP(h.Akd, lay.ew.Ak);
        if ((rc = dev_alloc(s, &h.Q, lay.K))) return bail(rc);
        if ((rc = dev_alloc(s, &h.qpend, lay.K)) || (rc = dev_alloc(s, &h.qdlt, lay.K))) return bail(rc);
        if (cudaMemsetAsync(h.qpend, 0, sizeof(float2) * lay.K, ctx->stream) != cudaSuccess ||
            cudaMemsetAsync(h.qdlt, 0, sizeof(float2) * lay.K, ctx->stream) != cudaSuccess)
            return bail(fail(FAU_ERR_CUDA, "pending Q(k) initialisation failed"));
        const double V = d->box[0] * d->box[1] * d->box[2];
        h.rec_pref = 2 * kPi * d->bjerrum_length / V;
        const double const_inf = d->ewald.epss < 1 ? 0.0 : 1.0;
        h.surf_pref = const_inf * 2.0 * kPi / ((2.0 * d->ewald.epss + 1.0) * V) * d->bjerrum_length;
        double M[3] = {0, 0, 0};
        for (int i = 0; i < n; i++) {
            M[0] += d->charge[i] * x[i];
            M[1] += d->charge[i] * y[i];
            M[2] += d->charge[i] * z[i];
        }
        for (int k = 0; k < 3; k++) h.M[k] = M[k];
    }
#undef UP
    // staging
    if ((rc = dev_alloc(s, &s->d_plain, 1))) return bail(rc);
    if ((rc = dev_alloc(s, &s->d_res, 8))) return bail(rc);
    if ((rc = dev_alloc(s, &s->d_partials, kTotalPartials))) return bail(rc);
    if ((rc = dev_alloc(s, &s->d_flags, 4))) return bail(rc);
    if (lay.K > 0 && (rc = dev_alloc(s, &s->d_dq, lay.K))) return bail(rc);
    // the audit probe record of the pipelined kernels (single-atom and molecular)
    if ((rc = dev_alloc(s, &h.audit_rec, kAuditRecBytes))) return bail(rc);
    if ((rc = dev_alloc(s, &s->d, 1))) return bail(rc);
    if ((rc = dev_alloc(s, &s->d_self, 1))) return bail(rc);
    if (cudaMemcpyAsync(s->d, &h, sizeof(DevSys), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(s->d_self, &s->d, sizeof(DevSys*), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
        return bail(fail(FAU_ERR_CUDA, "upload of the system descriptor failed"));
    // Q(k) full update (src/energy.cpp:191-206) in FP64 on the device
    if (lay.K > 0) {
        if (launch_q_rebuild(s->d, lay.K, h.Q, ctx->stream) != cudaSuccess)
            return bail(fail(FAU_ERR_CUDA, "q rebuild launch failed"));
    }
    if ((rc = refresh_energy(s))) return bail(rc);
    s->desc = store_desc(d);
    *out = s;
    return FAU_OK;
}

// Deep copy of a resident system: every device array is copied device to device and
// every device pointer of the copy is re-pointed into the copy's own arrays.  As the
// reference builds its trial state as a second State from the same input
// (src/montecarlo.cpp:101-111), this builds replicas and served jobs that share an
// initial state without re-uploading or re-evaluating it.
int fau_sys_clone(const fau_sys* src, fau_sys** out)
{
    if (!src || !out) return fail(FAU_ERR_ARG, "null argument");
    if (src->pending) return fail(FAU_ERR_STATE, "clone of a system with a pending trial");
    fau_ctx* ctx = src->ctx;
    CUDA_TRY(cudaSetDevice(ctx->device));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    fau_sys* s = new fau_sys(*src);
    s->allocs.clear();
    s->alloc_bytes.clear();
    s->bytes = 0;
    auto bail = [&](int code) {
        cudaStreamSynchronize(ctx->stream);
        free_sys(s);
        delete s;
        return code;
    };
    std::vector<std::pair<char*, char*>> remap; // (src base, dst base) with sizes from src
    for (size_t a = 0; a < src->allocs.size(); a++) {
        char* dst = nullptr;
        int rc = dev_alloc(s, &dst, src->alloc_bytes[a]);
        if (rc) return bail(rc);
        if (cudaMemcpyAsync(dst, src->allocs[a], src->alloc_bytes[a], cudaMemcpyDeviceToDevice, ctx->stream) !=
            cudaSuccess)
            return bail(fail(FAU_ERR_CUDA, "clone copy failed"));
        remap.emplace_back(static_cast<char*>(src->allocs[a]), dst);
    }
    auto fix = [&](auto*& ptr) {
        if (!ptr) return;
        char* p = reinterpret_cast<char*>(ptr);
        for (size_t a = 0; a < remap.size(); a++) {
            char* b = remap[a].first;
            if (p >= b && p < b + src->alloc_bytes[a]) {
                ptr = reinterpret_cast<std::remove_reference_t<decltype(ptr)>>(remap[a].second + (p - b));
                return;
            }
        }
    };
    DevSys& h = s->h;
    fix(h.x); fix(h.y); fix(h.z); fix(h.rec); fix(h.group_of); fix(h.itype_q); fix(h.itype_qd); fix(h.itype_self);
    fix(h.g_begin); fix(h.g_flags); fix(h.g_cm); fix(h.g_cmrec); fix(h.atomic_idx); fix(h.pair); fix(h.pair_d);
    fix(h.g_molid); fix(h.cut2_mol); fix(h.cut2_molf); fix(h.qpend); fix(h.qdlt);
    fix(h.spl); fix(h.spl_zf); fix(h.spl_zd); fix(h.spl_cf); fix(h.spl_cd); fix(h.spl_grid);
    fix(h.gc_cnt); fix(h.gc_list); fix(h.audit_rec);
    fix(h.cell_cnt); fix(h.cell_rec); fix(h.cell_of); fix(h.slot_of); fix(h.kn); fix(h.Ak); fix(h.Akd); fix(h.Q);
    fix(s->d); fix(s->d_self); fix(s->d_props); fix(s->d_acc); fix(s->d_du); fix(s->d_detail); fix(s->d_plain);
    fix(s->d_dq); fix(s->d_res); fix(s->d_partials); fix(s->d_flags);
    // the copy's device struct: running fields from the source's device struct, pointers from h
    DevSys cur;
    if (cudaMemcpyAsync(&cur, src->d, sizeof(DevSys), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return bail(fail(FAU_ERR_CUDA, "clone state read failed"));
    DevSys nd = h;
    nd.energy = cur.energy;
    nd.e_acc_hi = cur.e_acc_hi;
    nd.e_acc_lo = cur.e_acc_lo;
    nd.beta_scale = cur.beta_scale;
    nd.q_valid = cur.q_valid;
    nd.q_since = cur.q_since;
    for (int k = 0; k < 3; k++) nd.M[k] = cur.M[k];
    nd.cap = cur.cap;
    nd.err = 0;
    nd.moves = nd.accepted = nd.pair_evals = nd.k_updates = 0;
    nd.sum_du = 0.0;
    nd.audit_scaled_max = nd.audit_rel_max = 0.0;
    nd.audit_samples = 0;
    nd.audit_pending = 0;
    h = nd;
    if (cudaMemcpyAsync(s->d, &nd, sizeof(DevSys), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(s->d_self, &s->d, sizeof(DevSys*), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return bail(fail(FAU_ERR_CUDA, "clone descriptor upload failed"));
    *out = s;
    return FAU_OK;
}

// ---------------------------------------------------------------- exact device state (checkpoints)
static int rebuild_cells(fau_sys* s, int cap);
static int pull_state(fau_sys* s);
namespace {
constexpr uint32_t kStateMagic = 0x53554146u; // "FAUS"
constexpr uint32_t kStateVersion = 1;

struct StateHeader {
    uint32_t magic, version;
    int32_t n, n_groups, K, ncell, cap, precision;
    double box[3];
    // running scalars of the device struct
    double energy, beta_scale, sum_du, M[3];
    float e_acc_hi, e_acc_lo;
    int32_t q_valid, q_since;
    uint64_t moves, accepted, pair_evals, k_updates, cycles;
};

// the device arrays a chain changes, in blob order: (device pointer, bytes)
std::vector<std::pair<void*, size_t>> state_arrays(const fau_sys* s)
{
    const DevSys& h = s->h;
    const size_t n = s->n, g = s->n_groups, K = s->K;
    std::vector<std::pair<void*, size_t>> a = {
        {h.x, 8 * n}, {h.y, 8 * n}, {h.z, 8 * n}, {h.rec, 16 * n}, {h.g_cm, h.g_cm ? 24 * g : 0},
        {h.g_cmrec, h.g_cmrec ? 16 * g : 0}, {h.Q, 16 * K}, {h.qpend, h.qpend ? 8 * K : 0},
        {h.qdlt, h.qdlt ? 8 * K : 0}};
    if (s->cells) {
        const size_t nc = (size_t)h.ncell, cap = (size_t)h.cap;
        a.push_back({h.cell_cnt, 4 * nc});
        a.push_back({h.cell_rec, 16 * nc * cap});
        a.push_back({h.cell_of, 4 * n});
        a.push_back({h.slot_of, 4 * n});
    }
    return a;
}
} // namespace

int fau_sys_state_size(const fau_sys* s, size_t* bytes)
{
    if (!s || !bytes) return fail(FAU_ERR_ARG, "null argument");
    size_t b = sizeof(StateHeader);
    for (auto& a : state_arrays(s)) b += a.second;
    *bytes = b;
    return FAU_OK;
}

int fau_sys_save_state(fau_sys* s, void* buf, size_t bytes)
{
    if (!s || !buf) return fail(FAU_ERR_ARG, "null argument");
    if (s->pending) return fail(FAU_ERR_STATE, "a trial is pending (fau_commit_pending first)");
    size_t need = 0;
    fau_sys_state_size(s, &need);
    if (bytes < need) return fail(FAU_ERR_ARG, "state buffer of %zu bytes, %zu needed", bytes, need);
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    cudaStream_t st = s->ctx->stream;
    DevSys cur;
    CUDA_TRY(cudaMemcpyAsync(&cur, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost, st));
    char* out = static_cast<char*>(buf);
    size_t off = sizeof(StateHeader);
    for (auto& a : state_arrays(s)) {
        if (a.second) CUDA_TRY(cudaMemcpyAsync(out + off, a.first, a.second, cudaMemcpyDeviceToHost, st));
        off += a.second;
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    StateHeader hd{};
    hd.magic = kStateMagic;
    hd.version = kStateVersion;
    hd.n = s->n;
    hd.n_groups = s->n_groups;
    hd.K = s->K;
    hd.ncell = s->cells ? cur.ncell : 0;
    hd.cap = s->cells ? cur.cap : 0;
    hd.precision = s->precision;
    for (int k = 0; k < 3; k++) {
        hd.box[k] = cur.L[k];
        hd.M[k] = cur.M[k];
    }
    hd.energy = cur.energy;
    hd.beta_scale = cur.beta_scale;
    hd.sum_du = cur.sum_du;
    hd.e_acc_hi = cur.e_acc_hi;
    hd.e_acc_lo = cur.e_acc_lo;
    hd.q_valid = cur.q_valid;
    hd.q_since = cur.q_since;
    hd.moves = cur.moves;
    hd.accepted = cur.accepted;
    hd.pair_evals = cur.pair_evals;
    hd.k_updates = cur.k_updates;
    hd.cycles = cur.cycles;
    std::memcpy(out, &hd, sizeof hd);
    return FAU_OK;
}

int fau_sys_load_state(fau_sys* s, const void* buf, size_t bytes)
{
    if (!s || !buf) return fail(FAU_ERR_ARG, "null argument");
    if (s->pending) return fail(FAU_ERR_STATE, "a trial is pending (fau_commit_pending first)");
    if (bytes < sizeof(StateHeader)) return fail(FAU_ERR_ARG, "state of %zu bytes is too short", bytes);
    StateHeader hd;
    std::memcpy(&hd, buf, sizeof hd);
    if (hd.magic != kStateMagic || hd.version != kStateVersion) return fail(FAU_ERR_ARG, "not a system state");
    const int ncell = s->cells ? s->h.ncell : 0;
    if (hd.n != s->n || hd.n_groups != s->n_groups || hd.K != s->K || hd.ncell != ncell ||
        hd.precision != s->precision)
        return fail(FAU_ERR_ARG, "state of another system shape (particles, groups, k-vectors or cells)");
    for (int k = 0; k < 3; k++)
        if (hd.box[k] != s->h.L[k])
            return fail(FAU_ERR_ARG, "state of another box: make the system with the saved box");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    cudaStream_t st = s->ctx->stream;
    CUDA_TRY(cudaStreamSynchronize(st));
    if (s->cells && hd.cap != s->h.cap) { // the saved list had grown: the same capacity first
        int rc = rebuild_cells(s, hd.cap);
        if (rc) return rc;
    }
    size_t need = 0;
    fau_sys_state_size(s, &need);
    if (bytes != need) return fail(FAU_ERR_ARG, "state of %zu bytes, %zu expected", bytes, need);
    const char* in = static_cast<const char*>(buf);
    size_t off = sizeof(StateHeader);
    for (auto& a : state_arrays(s)) {
        if (a.second) CUDA_TRY(cudaMemcpyAsync(a.first, in + off, a.second, cudaMemcpyHostToDevice, st));
        off += a.second;
    }
    DevSys cur;
    CUDA_TRY(cudaMemcpyAsync(&cur, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    cur.energy = hd.energy;
    cur.beta_scale = hd.beta_scale;
    cur.sum_du = hd.sum_du;
    cur.e_acc_hi = hd.e_acc_hi;
    cur.e_acc_lo = hd.e_acc_lo;
    cur.q_valid = hd.q_valid;
    cur.q_since = hd.q_since;
    for (int k = 0; k < 3; k++) cur.M[k] = hd.M[k];
    cur.moves = hd.moves;
    cur.accepted = hd.accepted;
    cur.pair_evals = hd.pair_evals;
    cur.k_updates = hd.k_updates;
    cur.cycles = hd.cycles;
    cur.err = 0;
    CUDA_TRY(cudaMemcpyAsync(s->d, &cur, sizeof(DevSys), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    s->h.energy = hd.energy;
    s->h.beta_scale = hd.beta_scale;
    return pull_state(s);
}

int fau_sys_destroy(fau_sys* s)
{
    if (!s) return FAU_OK;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    free_sys(s);
    delete s;
    return FAU_OK;
}

int fau_sys_num_kvectors(const fau_sys* s, int* k)
{
    if (!s || !k) return fail(FAU_ERR_ARG, "null argument");
    *k = s->K;
    return FAU_OK;
}

// copy the device struct's running fields back to the host mirror
static int pull_state(fau_sys* s)
{
    DevSys tmp;
    CUDA_TRY(cudaMemcpyAsync(&tmp, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost, s->ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    s->h.energy = sys_energy(tmp);
    for (int k = 0; k < 3; k++) s->h.M[k] = tmp.M[k];
    s->h.err = tmp.err;
    s->h.moves = tmp.moves;
    s->h.accepted = tmp.accepted;
    s->h.pair_evals = tmp.pair_evals;
    s->h.k_updates = tmp.k_updates;
    s->h.sum_du = tmp.sum_du;
    s->h.audit_scaled_max = tmp.audit_scaled_max;
    s->h.audit_rel_max = tmp.audit_rel_max;
    s->h.audit_samples = tmp.audit_samples;
    return FAU_OK;
}

static int compute_total(fau_sys* s, fau_energy_terms* t)
{
    cudaStream_t st = s->ctx->stream;
    CUDA_TRY(launch_fold_q(s->d, s->K, st)); // Q(k) = master + pending changes
    CUDA_TRY(cudaMemsetAsync(s->d_partials, 0, kTotalPartials * sizeof(double), st));
    CUDA_TRY(cudaMemsetAsync(s->d_flags, 0, 4 * sizeof(int), st));
    CUDA_TRY(launch_total(s->d, s->n, s->K, s->d_partials, s->d_flags, st, s->cells));
    std::vector<double> part(kTotalPartials);
    int f[4];
    DevSys tmp;
    CUDA_TRY(cudaMemcpyAsync(part.data(), s->d_partials, kTotalPartials * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(f, s->d_flags, sizeof(f), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&tmp, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    // sums in block order: deterministic for a given state
    double r[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < kTotalPairBlocks; b++) r[0] += part[b];
    for (int b = 0; b < kTotalMiscBlocks; b++) {
        r[1] += part[kTotalPairBlocks + 2 * b];
        r[2] += part[kTotalPairBlocks + 2 * b + 1];
    }
    const double inf = std::numeric_limits<double>::infinity();
    double nb = r[0];
    if (f[0] & 2) nb = std::numeric_limits<double>::quiet_NaN();
    else if (f[0] & 1) nb = inf;
    t->self = (tmp.flags & SYS_SELF) ? r[2] : 0.0;
    t->nonbonded = nb;
    t->ewald_rec = (tmp.flags & SYS_EWALD) ? tmp.rec_pref * r[1] : 0.0;
    double m2 = (tmp.M[0] * tmp.M[0] + tmp.M[1] * tmp.M[1]) + tmp.M[2] * tmp.M[2];
    t->ewald_surf = (tmp.flags & SYS_SURFACE) ? tmp.surf_pref * m2 : 0.0;
    // Hamiltonian::energy: [self], nonbonded, [ewald]; early break on a term >= maxenergy (+inf
    // unless set) or NaN
    double list[3];
    int nl = 0;
    if (tmp.flags & SYS_SELF) list[nl++] = t->self;
    list[nl++] = t->nonbonded;
    if (tmp.flags & SYS_EWALD) list[nl++] = t->ewald_surf + t->ewald_rec;
    double sum = 0.0;
    for (int i = 0; i < nl; i++) {
        sum += list[i];
        if (list[i] >= tmp.maxenergy || std::isnan(list[i])) break;
    }
    t->total = sum;
    return FAU_OK;
}

static int refresh_energy(fau_sys* s)
{
    fau_energy_terms t;
    int rc = compute_total(s, &t);
    if (rc) return rc;
    s->h.energy = t.total;
    const float zero2[2] = {0.f, 0.f};
    CUDA_TRY(cudaMemcpyAsync(&s->d->energy, &t.total, sizeof(double), cudaMemcpyHostToDevice, s->ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(&s->d->e_acc_hi, zero2, sizeof(zero2), cudaMemcpyHostToDevice, s->ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    return FAU_OK;
}

int fau_energy_total(fau_sys* s, fau_energy_terms* out)
{
    const fau::NvtxRange nvtx_range("fau_energy_total");
    if (!s || !out) return fail(FAU_ERR_ARG, "null argument");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    return compute_total(s, out);
}

static int ensure_stage(fau_sys* s, size_t n)
{
    if (n <= s->stage_cap) return FAU_OK;
    size_t cap = std::max<size_t>(n, 1024);
    int rc;
    if ((rc = dev_alloc(s, &s->d_props, cap))) return rc;
    if ((rc = dev_alloc(s, &s->d_acc, cap))) return rc;
    if ((rc = dev_alloc(s, &s->d_du, cap))) return rc;
    if ((rc = dev_alloc(s, &s->d_detail, cap))) return rc;
    s->stage_cap = cap;
    return FAU_OK;
}

static int chain_threads(const fau_sys* s)
{
    if (s->K >= 512 || s->n >= 4096) return 256;
    return s->K > 0 || s->n > 512 ? 256 : 128;
}

static int check_device_err(fau_sys* s)
{
    int rc = pull_state(s);
    if (rc) return rc;
    if (s->h.err != FAU_OK) {
        const int e = s->h.err;
        s->h.err = 0;
        CUDA_TRY(cudaMemsetAsync(&s->d->err, 0, sizeof(int), s->ctx->stream));
        CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
        return fail(e, "device reported: %s", fau_strerror(e));
    }
    return FAU_OK;
}

// Rebuild the cell list from the resident FP64 positions with a new capacity
// (after an overflow); reference binning formula, bit-exact with the oracle.
static int rebuild_cells(fau_sys* s, int cap)
{
    if (!s->cells) return FAU_OK;
    cudaStream_t st = s->ctx->stream;
    const int n = s->n;
    std::vector<double> x(n), y(n), z(n);
    std::vector<uint4> rec(n);
    CUDA_TRY(cudaMemcpyAsync(x.data(), s->h.x, 8 * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(y.data(), s->h.y, 8 * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(z.data(), s->h.z, 8 * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(rec.data(), s->h.rec, sizeof(uint4) * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    const int ncell = s->h.ncell;
    std::vector<int> cnt(ncell, 0), cell_of(n), slot_of(n);
    for (int i = 0; i < n; i++) {
        const double p[3] = {x[i], y[i], z[i]};
        cell_of[i] = host_cell(p, s->h.L, s->h.cdim, s->h.cell_len);
        slot_of[i] = cnt[cell_of[i]]++;
    }
    const int maxc = *std::max_element(cnt.begin(), cnt.end());
    cap = cell_capacity(cap, maxc, n / (double)ncell);
    std::vector<uint4> crec((size_t)ncell * cap, make_uint4(0, 0, 0, 0xFFFFFFFFu));
    for (int i = 0; i < n; i++) crec[(size_t)cell_of[i] * cap + slot_of[i]] = rec[i];
    uint4* nrec = nullptr;
    int rc = dev_alloc(s, &nrec, crec.size());
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(nrec, crec.data(), sizeof(uint4) * crec.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->h.cell_cnt, cnt.data(), 4 * ncell, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->h.cell_of, cell_of.data(), 4 * n, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->h.slot_of, slot_of.data(), 4 * n, cudaMemcpyHostToDevice, st));
    s->h.cell_rec = nrec;
    s->h.cap = cap;
    CUDA_TRY(cudaMemcpyAsync(&s->d->cell_rec, &nrec, sizeof(nrec), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(&s->d->cap, &cap, sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return FAU_OK;
}

static int run_chain(fau_sys* s, const fau_proposal* p, int n, uint8_t* acc, double* du, fau_trial_result* detail,
                     fau_run_stats* stats)
{
    if (n < 0) return fail(FAU_ERR_ARG, "negative move count");
    if (n == 0) {
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return FAU_OK;
    }
    for (int m = 0; m < n; m++) {
        if (p[m].kind == FAU_MOVE_ATOMIC) {
            if (p[m].index < 0 || p[m].index >= s->n) return fail(FAU_ERR_ARG, "proposal %d: particle out of range", m);
            if (!(s->g_flags[s->group_of[p[m].index]] & FAU_GROUP_ATOMIC))
                return fail(FAU_ERR_ARG, "proposal %d: single-atom move inside a molecular group is not supported", m);
        }
        else if (p[m].kind == FAU_MOVE_MOLECULAR) {
            if (p[m].index < 0 || p[m].index >= s->n_groups) return fail(FAU_ERR_ARG, "proposal %d: group out of range", m);
            if (s->g_flags[p[m].index] & FAU_GROUP_ATOMIC)
                return fail(FAU_ERR_ARG, "proposal %d: molecular move of an atomic group", m);
            if (s->g_begin[p[m].index + 1] - s->g_begin[p[m].index] > kMaxGroupAtoms)
                return fail(FAU_ERR_ARG, "proposal %d: group larger than %d atoms", m, kMaxGroupAtoms);
        }
        else if (p[m].kind != FAU_MOVE_NONE) {
            return fail(FAU_ERR_ARG, "proposal %d: unknown kind %d", m, p[m].kind);
        }
    }
    int rc = ensure_stage(s, (size_t)n);
    if (rc) return rc;
    cudaStream_t st = s->ctx->stream;
    CUDA_TRY(cudaMemcpyAsync(s->d_props, p, sizeof(fau_proposal) * n, cudaMemcpyHostToDevice, st));
    DevSys before;
    CUDA_TRY(cudaMemcpyAsync(&before, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost, st));
    float total_ms = 0.f;
    long long offset = 0;
    for (int attempt = 0; attempt < 16 && offset < n; attempt++) {
        ChainArgs a{};
        a.sys = s->d_self;
        a.moves = n - offset;
        a.props = s->d_props + offset;
        a.acc_out = acc ? s->d_acc + offset : nullptr;
        a.du_out = du ? s->d_du + offset : nullptr;
        a.detail = detail ? s->d_detail + offset : nullptr;
        // a proposal stream's launch ends with the audit probe (single trials with detail do not)
        a.audit = detail ? 0 : 1;
        CUDA_TRY(cudaEventRecord(s->ctx->ev0, st));
        CUDA_TRY(launch_chain(a, 1, s->K, s->h.knc, chain_threads(s), false, st));
        CUDA_TRY(cudaEventRecord(s->ctx->ev1, st));
        if (a.audit) CUDA_TRY(launch_probe_audit(s->d_self, 1, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, s->ctx->ev0, s->ctx->ev1);
        total_ms += ms;
        DevSys now;
        CUDA_TRY(cudaMemcpy(&now, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost));
        if (now.err == FAU_ERR_CAPACITY) {
            // a cell overflowed on an accepted move: the move is committed except for its
            // cell-list entry; rebuild the cell list with twice the capacity and resume
            offset += now.consumed;
            const int zero = 0;
            CUDA_TRY(cudaMemcpy(&s->d->err, &zero, sizeof(int), cudaMemcpyHostToDevice));
            if ((rc = rebuild_cells(s, 2 * s->h.cap))) return rc;
            continue;
        }
        offset = n;
    }
    if (acc) CUDA_TRY(cudaMemcpyAsync(acc, s->d_acc, n, cudaMemcpyDeviceToHost, st));
    if (du) CUDA_TRY(cudaMemcpyAsync(du, s->d_du, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (detail) CUDA_TRY(cudaMemcpyAsync(detail, s->d_detail, sizeof(fau_trial_result) * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    rc = check_device_err(s);
    if (stats) {
        stats->moves = (int64_t)(s->h.moves - before.moves);
        stats->accepted = (int64_t)(s->h.accepted - before.accepted);
        stats->pair_evals = (int64_t)(s->h.pair_evals - before.pair_evals);
        stats->k_updates = (int64_t)(s->h.k_updates - before.k_updates);
        stats->energy_change = s->h.sum_du - before.sum_du;
        stats->energy = s->h.energy;
        stats->max_rel_err = s->h.audit_scaled_max; // the audit probes' largest error since the system was made
        stats->device_ms = total_ms;
    }
    return rc;
}

static int plain_trial(fau_sys* s, int kind, int index, const double dr[3], const double* quat, double u01,
                       fau_trial_result* out);

static int run_segment(fau_sys* s, const fau_proposal* p, int n, uint8_t* acc, double* du, fau_run_stats* stats);

// Volume proposals split the stream: the chain runs the moves between them and
// fau_volume_move performs each volume move in order.
int fau_run_proposals(fau_sys* s, const fau_proposal* p, int n, uint8_t* acc, double* du, fau_run_stats* stats)
{
    const fau::NvtxRange nvtx_range("fau_run_proposals");
    if (!s || (!p && n > 0)) return fail(FAU_ERR_ARG, "null argument");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    int first_vol = -1;
    for (int m = 0; m < n && first_vol < 0; m++)
        if (p[m].kind == FAU_MOVE_VOLUME) first_vol = m;
    if (first_vol < 0) return run_segment(s, p, n, acc, du, stats);
    fau_run_stats tot{};
    auto add = [&](const fau_run_stats& x) {
        tot.moves += x.moves;
        tot.accepted += x.accepted;
        tot.pair_evals += x.pair_evals;
        tot.k_updates += x.k_updates;
        tot.energy_change += x.energy_change;
        tot.max_rel_err = std::max(tot.max_rel_err, x.max_rel_err);
        tot.device_ms += x.device_ms;
    };
    int a = 0, rc = FAU_OK;
    for (int m = first_vol; m <= n; m++) {
        if (m < n && p[m].kind != FAU_MOVE_VOLUME) continue;
        if (m > a) {
            fau_run_stats seg{};
            if ((rc = run_segment(s, p + a, m - a, acc ? acc + a : nullptr, du ? du + a : nullptr, &seg))) return rc;
            add(seg);
        }
        if (m == n) break;
        const double* L = s->h.L;
        const double v_new = std::exp(std::log(L[0] * L[1] * L[2]) + p[m].dr[0]);
        fau_trial_result r{};
        if ((rc = fau_volume_move(s, v_new, p[m].index, p[m].u, &r))) return rc;
        if (acc) acc[m] = (uint8_t)r.accepted;
        if (du) du[m] = r.du;
        fau_run_stats one{};
        one.moves = 1;
        one.accepted = r.accepted;
        one.energy_change = r.accepted ? r.du : 0.0;
        add(one);
        a = m + 1;
    }
    if (stats) {
        tot.energy = s->h.energy;
        *stats = tot;
    }
    return FAU_OK;
}

static int run_segment(fau_sys* s, const fau_proposal* p, int n, uint8_t* acc, double* du, fau_run_stats* stats)
{
    // a finite maxenergy: the chain kernel, the form that stops each state's term sum
    if (s->precision != FAU_PREC_FP64 || s->h.maxe) return run_chain(s, p, n, acc, du, nullptr, stats);
    // plain FP64 form: one move per call, host Metropolis
    int rc = pull_state(s);
    if (rc) return rc;
    const DevSys before = s->h;
    CUDA_TRY(cudaEventRecord(s->ctx->ev0, s->ctx->stream));
    for (int m = 0; m < n; m++) {
        fau_trial_result r{};
        if (p[m].kind == FAU_MOVE_ATOMIC) rc = fau_trial_atomic(s, p[m].index, p[m].dr, p[m].u, &r);
        else if (p[m].kind == FAU_MOVE_MOLECULAR) rc = fau_trial_group(s, p[m].index, p[m].dr, p[m].quat, p[m].u, &r);
        if (rc) return rc;
        if (acc) acc[m] = (uint8_t)r.accepted;
        if (du) du[m] = r.du;
    }
    CUDA_TRY(cudaEventRecord(s->ctx->ev1, s->ctx->stream));
    CUDA_TRY(cudaEventSynchronize(s->ctx->ev1));
    if ((rc = pull_state(s))) return rc;
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, s->ctx->ev0, s->ctx->ev1);
        stats->moves = (int64_t)(s->h.moves - before.moves);
        stats->accepted = (int64_t)(s->h.accepted - before.accepted);
        stats->pair_evals = 2 * (int64_t)(s->n - 1) * n;
        stats->k_updates = (int64_t)s->K * n;
        stats->energy_change = s->h.sum_du - before.sum_du;
        stats->energy = s->h.energy;
        stats->max_rel_err = 0.0;
        stats->device_ms = ms;
    }
    return FAU_OK;
}

// plain FP64 form: host computes the trial positions exactly like the device
static double hb(double a, double L, double half, double inv)
{
    if (std::fabs(a) > half) {
        const double t = a * inv;
        a -= L * (int)(t > 0.0 ? t + 0.5 : t - 0.5);
    }
    return a;
}

static int plain_trial(fau_sys* s, int kind, int index, const double dr[3], const double* quat, double u01,
                       fau_trial_result* out)
{
    CUDA_TRY(launch_fold_q(s->d, s->K, s->ctx->stream)); // the plain kernels read the FP64 master
    cudaStream_t st = s->ctx->stream;
    PlainMove pm{};
    pm.kind = kind;
    pm.count_move = 1;
    const DevSys& h = s->h;
    std::vector<double> xo;
    std::vector<double> qs;
    if (kind == FAU_MOVE_ATOMIC) {
        pm.first = index;
        pm.m = 1;
        pm.group = -1;
        double p[3];
        CUDA_TRY(cudaMemcpyAsync(&p[0], h.x + index, 8, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(&p[1], h.y + index, 8, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(&p[2], h.z + index, 8, cudaMemcpyDeviceToHost, st));
        uint4 r;
        CUDA_TRY(cudaMemcpyAsync(&r, h.rec + index, sizeof(uint4), cudaMemcpyDeviceToHost, st));
        double q;
        CUDA_TRY(cudaStreamSynchronize(st));
        CUDA_TRY(cudaMemcpy(&q, h.itype_qd + (r.w >> 24), 8, cudaMemcpyDeviceToHost));
        for (int k = 0; k < 3; k++) {
            pm.xn[0][k] = hb(p[k] + dr[k], h.L[k], h.half[k], h.inv[k]);
            pm.dM[k] = q * (pm.xn[0][k] - p[k]);
        }
    }
    else {
        const int b = s->g_begin[index], e = s->g_begin[index + 1];
        pm.first = b;
        pm.m = e - b;
        pm.group = index;
        std::vector<double> X(pm.m), Y(pm.m), Z(pm.m);
        std::vector<uint4> R(pm.m);
        double cm[3];
        CUDA_TRY(cudaMemcpyAsync(X.data(), h.x + b, 8 * pm.m, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(Y.data(), h.y + b, 8 * pm.m, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(Z.data(), h.z + b, 8 * pm.m, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(R.data(), h.rec + b, sizeof(uint4) * pm.m, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(cm, h.g_cm + 3 * index, 24, cudaMemcpyDeviceToHost, st));
        std::vector<double> iq(h.nt);
        CUDA_TRY(cudaMemcpyAsync(iq.data(), h.itype_qd, 8 * h.nt, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        for (int k = 0; k < 3; k++) pm.cm_new[k] = hb(cm[k] + dr[k], h.L[k], h.half[k], h.inv[k]);
        const bool rot = quat && !(quat[0] == 0.0 && quat[1] == 0.0 && quat[2] == 0.0 && quat[3] == 0.0);
        for (int a = 0; a < pm.m; a++) {
            const double o[3] = {X[a], Y[a], Z[a]};
            double v[3];
            for (int k = 0; k < 3; k++) v[k] = hb(o[k] + dr[k], h.L[k], h.half[k], h.inv[k]);
            if (rot) {
                for (int k = 0; k < 3; k++) v[k] = hb(v[k] - pm.cm_new[k], h.L[k], h.half[k], h.inv[k]);
                const double ux = quat[1], uy = quat[2], uz = quat[3], w = quat[0];
                double tx = uy * v[2] - uz * v[1], ty = uz * v[0] - ux * v[2], tz = ux * v[1] - uy * v[0];
                tx = tx + tx;
                ty = ty + ty;
                tz = tz + tz;
                const double cx = uy * tz - uz * ty, cy = uz * tx - ux * tz, cz = ux * ty - uy * tx;
                v[0] = v[0] + w * tx + cx;
                v[1] = v[1] + w * ty + cy;
                v[2] = v[2] + w * tz + cz;
                for (int k = 0; k < 3; k++) v[k] = hb(v[k] + pm.cm_new[k], h.L[k], h.half[k], h.inv[k]);
            }
            const double q = iq[R[a].w >> 24];
            for (int k = 0; k < 3; k++) {
                pm.xn[a][k] = v[k];
                pm.dM[k] += q * (v[k] - o[k]);
            }
        }
    }
    CUDA_TRY(cudaMemcpyAsync(s->d_plain, &pm, sizeof(pm), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(s->d_res, 0, 8 * sizeof(double), st));
    CUDA_TRY(cudaMemsetAsync(s->d_flags, 0, 4 * sizeof(int), st));
    CUDA_TRY(launch_plain_du(s->d, s->d_plain, s->n, s->K, s->d_dq, s->d_res, s->d_flags, st));
    double r[8];
    int f[4];
    CUDA_TRY(cudaMemcpyAsync(r, s->d_res, sizeof(r), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(f, s->d_flags, sizeof(f), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    const double du_nb = r[0];
    const double du_rec = s->K ? h.rec_pref * r[1] : 0.0;
    double du_surf = 0.0;
    if (h.flags & SYS_SURFACE) {
        double M[3];
        DevSys tmp;
        CUDA_TRY(cudaMemcpy(&tmp, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost));
        for (int k = 0; k < 3; k++) M[k] = tmp.M[k];
        double m2o = 0, m2n = 0;
        for (int k = 0; k < 3; k++) {
            m2o += M[k] * M[k];
            m2n += (M[k] + pm.dM[k]) * (M[k] + pm.dM[k]);
        }
        du_surf = h.surf_pref * (m2n - m2o);
    }
    const double inf = std::numeric_limits<double>::infinity();
    const bool ni = f[0] & 1, oi = f[0] & 2, nn = f[0] & 4, on = f[0] & 8;
    double du;
    if (on && !nn) du = -inf;
    else if (nn) du = inf;
    else if (ni) du = inf;
    else if (oi) du = -inf;
    else du = du_nb + (du_rec + du_surf);
    if (std::isnan(du)) return fail(FAU_ERR_NAN, "Metropolis error: energy cannot be NaN");
    const double x = du * h.beta_scale;
    bool acc;
    if (std::isinf(x) && x < 0) acc = true;
    else if (-x > 709.782712893384) acc = true;
    else acc = u01 <= std::exp(-x);
    if (out) {
        out->du = du;
        out->du_nonbonded = du_nb;
        out->du_ewald = du_rec + du_surf;
        out->err_scale = r[2];
        out->accepted = acc;
        out->new_inf = ni;
        out->old_inf = oi;
        out->pad = 0;
    }
    if (acc) {
        pm.du = du;
        CUDA_TRY(cudaMemcpyAsync(s->d_plain, &pm, sizeof(pm), cudaMemcpyHostToDevice, st));
        CUDA_TRY(launch_plain_commit(s->d, s->d_plain, s->K, s->d_dq, st));
    }
    else {
        unsigned long long one = 1;
        DevSys tmp;
        CUDA_TRY(cudaMemcpyAsync(&tmp, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        tmp.moves += one;
        CUDA_TRY(cudaMemcpyAsync(&s->d->moves, &tmp.moves, sizeof(one), cudaMemcpyHostToDevice, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return check_device_err(s);
}

int fau_trial_atomic(fau_sys* s, int particle, const double dr[3], double u01, fau_trial_result* out)
{
    if (!s || !dr) return fail(FAU_ERR_ARG, "null argument");
    if (particle < 0 || particle >= s->n) return fail(FAU_ERR_ARG, "particle out of range");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    if (!(s->g_flags[s->group_of[particle]] & FAU_GROUP_ATOMIC))
        return fail(FAU_ERR_ARG, "single-atom move inside a molecular group is not supported");
    // the system's precision decides the form: plain FP64 or the FP32C chain kernel
    if (s->precision == FAU_PREC_FP64 && !s->h.maxe) return plain_trial(s, FAU_MOVE_ATOMIC, particle, dr, nullptr, u01, out);
    fau_proposal p{};
    p.kind = FAU_MOVE_ATOMIC;
    p.index = particle;
    for (int k = 0; k < 3; k++) p.dr[k] = dr[k];
    p.u = u01;
    fau_trial_result r{};
    int rc = run_chain(s, &p, 1, nullptr, nullptr, &r, nullptr);
    if (out) *out = r;
    return rc;
}

int fau_trial_group(fau_sys* s, int group, const double dr[3], const double quat[4], double u01, fau_trial_result* out)
{
    if (!s || !dr) return fail(FAU_ERR_ARG, "null argument");
    if (group < 0 || group >= s->n_groups) return fail(FAU_ERR_ARG, "group out of range");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    if (s->g_flags[group] & FAU_GROUP_ATOMIC) return fail(FAU_ERR_ARG, "molecular move of an atomic group");
    if (s->g_begin[group + 1] - s->g_begin[group] > kMaxGroupAtoms)
        return fail(FAU_ERR_ARG, "group larger than %d atoms", kMaxGroupAtoms);
    if (s->precision == FAU_PREC_FP64 && !s->h.maxe) return plain_trial(s, FAU_MOVE_MOLECULAR, group, dr, quat, u01, out);
    fau_proposal p{};
    p.kind = FAU_MOVE_MOLECULAR;
    p.index = group;
    for (int k = 0; k < 3; k++) p.dr[k] = dr[k];
    if (quat)
        for (int k = 0; k < 4; k++) p.quat[k] = quat[k];
    p.u = u01;
    fau_trial_result r{};
    int rc = run_chain(s, &p, 1, nullptr, nullptr, &r, nullptr);
    if (out) *out = r;
    return rc;
}

// ---------------------------------------------------------------- volume move
namespace {
// Chameleon::boundary for a cuboid (src/geometry.h:407-427) with the given box
inline void wrap1(double& a, double L, double half, double inv)
{
    if (std::fabs(a) > half) {
        const double t = a * inv;
        a -= L * (int)(t > 0.0 ? t + 0.5 : t - 0.5);
    }
}
} // namespace

int fau_volume_move(fau_sys* s, double new_volume, int method, double u01, fau_trial_result* out)
{
    const fau::NvtxRange nvtx_range("fau_volume_move");
    if (!s) return fail(FAU_ERR_ARG, "null system");
    if (!(new_volume > 0.0) || !std::isfinite(new_volume)) return fail(FAU_ERR_ARG, "new volume must be positive");
    if (method < FAU_VOLUME_ISOTROPIC || method > FAU_VOLUME_ISOCHORIC)
        return fail(FAU_ERR_ARG, "unknown volume scaling method %d", method);
    if (s->pending) return fail(FAU_ERR_STATE, "volume move with a pending trial");
    if (!s->desc) return fail(FAU_ERR_STATE, "system has no descriptor to rebuild from");
    const bool isobaric = s->desc->d.isobaric != 0;
    const double pressure = s->desc->d.pressure;
    fau_ctx* ctx = s->ctx;
    CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    // the accepted state's energy
    fau_energy_terms eo;
    int rc = compute_total(s, &eo);
    if (rc) return rc;
    const int n = s->n, G = s->n_groups;
    std::vector<double> x(n), y(n), z(n), cm(3 * (size_t)G);
    DevSys cur;
    CUDA_TRY(cudaMemcpyAsync(x.data(), s->h.x, 8 * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(y.data(), s->h.y, 8 * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(z.data(), s->h.z, 8 * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(cm.data(), s->h.g_cm, 8 * 3 * (size_t)G, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&cur, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    // Cuboid::setVolume (src/geometry.cpp:57-90)
    const double* L = s->h.L;
    const double v_old = L[0] * L[1] * L[2];
    double sc[3];
    switch (method) {
    case FAU_VOLUME_ISOTROPIC: {
        const double a = std::cbrt(new_volume / v_old);
        sc[0] = sc[1] = sc[2] = a;
        break;
    }
    case FAU_VOLUME_XY: {
        const double a = std::sqrt(new_volume / v_old);
        sc[0] = sc[1] = a;
        sc[2] = 1.0;
        break;
    }
    case FAU_VOLUME_Z:
        sc[0] = sc[1] = 1.0;
        sc[2] = new_volume / v_old;
        break;
    default: { // isochoric: the shape changes, the volume stays
        const double a = std::cbrt(new_volume / v_old);
        sc[0] = sc[1] = a;
        sc[2] = 1 / (a * a);
        break;
    }
    }
    double Ln[3], hn[3], in[3];
    for (int k = 0; k < 3; k++) {
        Ln[k] = L[k] * sc[k];
        hn[k] = 0.5 * Ln[k];
        in[k] = 1.0 / Ln[k];
    }
    // Space::scaleVolume (src/space.cpp:249-301)
    std::vector<double> pos(3 * (size_t)n), cmn(cm);
    int n_count = 0; // Isobaric: particles of atomic groups + molecular groups
    for (int g = 0; g < G; g++) {
        const int b = s->g_begin[g], e = s->g_begin[g + 1];
        if (e == b) continue;
        if (s->g_flags[g] & FAU_GROUP_ATOMIC) {
            n_count += e - b;
            for (int i = b; i < e; i++) {
                double p[3] = {x[i] * sc[0], y[i] * sc[1], z[i] * sc[2]};
                for (int k = 0; k < 3; k++) {
                    wrap1(p[k], Ln[k], hn[k], in[k]);
                    pos[3 * (size_t)i + k] = p[k];
                }
            }
        }
        else {
            n_count += 1;
            double c[3], dc[3];
            for (int k = 0; k < 3; k++) {
                c[k] = cm[3 * (size_t)g + k] * sc[k];
                wrap1(c[k], Ln[k], hn[k], in[k]);
                dc[k] = c[k] - cm[3 * (size_t)g + k];
                cmn[3 * (size_t)g + k] = c[k];
            }
            for (int i = b; i < e; i++) {
                const double p0[3] = {x[i], y[i], z[i]};
                for (int k = 0; k < 3; k++) {
                    // Group::unwrap (src/group.h:349-356): cm + vdist(p, cm) in the old box
                    double d = p0[k] - cm[3 * (size_t)g + k];
                    if (d > s->h.half[k]) d -= L[k];
                    else if (d < -s->h.half[k]) d += L[k];
                    double p = cm[3 * (size_t)g + k] + d;
                    p += dc[k];
                    wrap1(p, Ln[k], hn[k], in[k]);
                    pos[3 * (size_t)i + k] = p;
                }
            }
        }
    }
    // the trial state: the same system rebuilt for the new box (k-vectors, A_k, cells,
    // fixed-point records, full Q(k) in FP64, FP64 total energy)
    fau_sys_desc nd = s->desc->d;
    for (int k = 0; k < 3; k++) nd.box[k] = Ln[k];
    nd.pos = pos.data();
    nd.group_mass_center = cmn.data();
    fau_sys* t = nullptr;
    if ((rc = fau_sys_create(ctx, &nd, &t))) return rc;
    auto drop = [&](fau_sys* q) {
        cudaStreamSynchronize(st);
        free_sys(q);
        delete q;
    };
    fau_energy_terms en;
    if ((rc = compute_total(t, &en))) {
        drop(t);
        return rc;
    }
    const double v_new = Ln[0] * Ln[1] * Ln[2];
    // Isobaric::energy first, then the Hamiltonian's terms (inf / NaN propagate)
    auto iso = [&](double v) { return isobaric ? pressure * v - (double)(n_count + 1) * std::log(v) : 0.0; };
    // the Isobaric term ends the sum when it reaches maxenergy (the other terms' stop is in total)
    const double maxe = s->h.maxenergy;
    auto with_iso = [&](double vi, double total) {
        const double ti = iso(vi);
        return (isobaric && !(ti < maxe)) ? ti : ti + total;
    };
    const double uo = with_iso(v_old, eo.total);
    const double un = with_iso(v_new, en.total);
    // getEnergyChange (src/montecarlo.cpp:193-209)
    const double inf = std::numeric_limits<double>::infinity();
    double du;
    if (std::isnan(uo) && !std::isnan(un)) du = -inf;
    else if (std::isnan(un)) du = inf;
    else if (un >= inf) du = inf;
    else if (uo >= inf) du = -inf;
    else du = un - uo;
    if (std::isnan(du)) {
        drop(t);
        return fail(FAU_ERR_NAN, "Metropolis error: energy cannot be NaN");
    }
    // metropolisCriterion (src/montecarlo.cpp:17-34)
    const double xb = du * cur.beta_scale;
    bool acc;
    if (std::isinf(xb) && xb < 0) acc = true;
    else if (-xb > 709.782712893384) acc = true;
    else acc = u01 <= std::exp(-xb);
    if (out) {
        out->du = du;
        out->du_nonbonded = en.nonbonded - eo.nonbonded;
        out->du_ewald = (en.ewald_rec + en.ewald_surf) - (eo.ewald_rec + eo.ewald_surf);
        out->err_scale = std::fabs(un) + std::fabs(uo);
        out->accepted = acc;
        out->new_inf = un >= inf;
        out->old_inf = uo >= inf;
        out->pad = 0;
    }
    // counters and PT temperature carried by whichever state is kept
    cur.moves += 1;
    if (acc) cur.accepted += 1;
    fau_sys* keep = acc ? t : s;
    DevSys* dk = keep->d;
    CUDA_TRY(cudaMemcpyAsync(&dk->moves, &cur.moves, sizeof(cur.moves), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(&dk->accepted, &cur.accepted, sizeof(cur.accepted), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(&dk->pair_evals, &cur.pair_evals, sizeof(cur.pair_evals), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(&dk->k_updates, &cur.k_updates, sizeof(cur.k_updates), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(&dk->cycles, &cur.cycles, sizeof(cur.cycles), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(&dk->beta_scale, &cur.beta_scale, sizeof(double), cudaMemcpyHostToDevice, st));
    // the audit history (the error against FP64 since the system was made) stays with the system
    CUDA_TRY(cudaMemcpyAsync(&dk->audit_scaled_max, &cur.audit_scaled_max, 2 * sizeof(double) + sizeof(unsigned long long),
                             cudaMemcpyHostToDevice, st));
    if (acc) {
        const double sdu = cur.sum_du + du;
        CUDA_TRY(cudaMemcpyAsync(&dk->sum_du, &sdu, sizeof(double), cudaMemcpyHostToDevice, st));
        // the caller's handle now holds the trial state; the old state's blocks go to the pool
        t->desc = s->desc;
        std::swap(*s, *t);
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    drop(t);
    return pull_state(s);
}

// internal accessors used by fau_batch.cu (not part of the public header)
int fau_internal_ctx_stream(fau_ctx* c, cudaStream_t* st, int* device)
{
    *st = c->stream;
    *device = c->device;
    return FAU_OK;
}
int fau_internal_sys_view(fau_sys* s, fau_ctx** ctx, DevSys** d, int* K, int* n, int* n_groups, int* molecular_only,
                          double* t_ref, int* knc)
{
    *knc = s->h.knc;
    *ctx = s->ctx;
    *d = s->d;
    *K = s->K;
    *n = s->n;
    *n_groups = s->n_groups;
    *molecular_only = s->molecular_only ? 1 : 0;
    *t_ref = 1.0;
    return FAU_OK;
}
int fau_internal_fail(int code, const char* msg) { return fail(code, "%s", msg); }
int fau_internal_sys_all_atomic(const fau_sys* s) { return s->all_atomic ? 1 : 0; }
int fau_internal_sys_classes(const fau_sys* s) { return s->h.nt; }
double fau_internal_sys_volume(const fau_sys* s) { return s->h.L[0] * s->h.L[1] * s->h.L[2]; }
int fau_internal_sys_maxe(const fau_sys* s) { return s->h.maxe; }
int fau_internal_sys_fp64(const fau_sys* s) { return s->precision == FAU_PREC_FP64 ? 1 : 0; }
int fau_internal_sys_occ(const fau_sys* s) { return (s->h.flags & SYS_OCC) && (s->h.flags & SYS_CELLS) ? 1 : 0; }
// after a batched chain stopped on a full cell: twice the capacity of the particle cells (their
// lists rebuilt from the positions) and of the mass-centre cells (listed again by the next launch)
int fau_internal_sys_regrow(fau_sys* s)
{
    int rc = FAU_OK;
    if (s->cells && (rc = rebuild_cells(s, 2 * s->h.cap))) return rc;
    if (s->h.gncell > 0) {
        const int cap = 2 * s->h.gcap, sh = s->h.gshift + 1;
        int* nl = nullptr;
        if ((rc = dev_alloc(s, &nl, (size_t)s->h.gncell * cap))) return rc;
        s->h.gc_list = nl;
        s->h.gcap = cap;
        s->h.gshift = sh;
        cudaStream_t st = s->ctx->stream;
        CUDA_TRY(cudaMemcpyAsync(&s->d->gc_list, &nl, sizeof(nl), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(&s->d->gcap, &cap, sizeof(int), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(&s->d->gshift, &sh, sizeof(int), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    return FAU_OK;
}

// a context-owned device scratch buffer of at least `bytes` (grown on demand; valid until the
// next call on this context -- batched calls synchronise their stream before returning)
int fau_internal_ctx_scratch(fau_ctx* c, size_t bytes, void** out)
{
    if (bytes > c->scratch_bytes) {
        if (c->scratch) {
            cudaStreamSynchronize(c->stream);
            cudaFree(c->scratch);
            c->scratch = nullptr;
            c->scratch_bytes = 0;
        }
        const size_t b = block_class(bytes);
        CUDA_TRY(cudaMalloc(&c->scratch, b));
        c->scratch_bytes = b;
    }
    *out = c->scratch;
    return FAU_OK;
}

int fau_energy_change(fau_sys* s, const fau_proposal* p, fau_trial_result* out)
{
    if (!s || !p) return fail(FAU_ERR_ARG, "null argument");
    if (s->pending) return fail(FAU_ERR_STATE, "a pending trial must be committed or rejected first");
    if (p->kind != FAU_MOVE_ATOMIC && p->kind != FAU_MOVE_MOLECULAR)
        return fail(FAU_ERR_ARG, "fau_energy_change needs an atomic or molecular proposal");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    if (p->kind == FAU_MOVE_ATOMIC) {
        if (p->index < 0 || p->index >= s->n) return fail(FAU_ERR_ARG, "particle out of range");
        if (!(s->g_flags[s->group_of[p->index]] & FAU_GROUP_ATOMIC))
            return fail(FAU_ERR_ARG, "single-atom move inside a molecular group is not supported");
    }
    else {
        if (p->index < 0 || p->index >= s->n_groups) return fail(FAU_ERR_ARG, "group out of range");
        if (s->g_flags[p->index] & FAU_GROUP_ATOMIC) return fail(FAU_ERR_ARG, "molecular move of an atomic group");
        if (s->g_begin[p->index + 1] - s->g_begin[p->index] > kMaxGroupAtoms)
            return fail(FAU_ERR_ARG, "group larger than %d atoms", kMaxGroupAtoms);
    }
    int rc = ensure_stage(s, 1);
    if (rc) return rc;
    cudaStream_t st = s->ctx->stream;
    CUDA_TRY(cudaMemcpyAsync(s->d_props, p, sizeof(fau_proposal), cudaMemcpyHostToDevice, st));
    ChainArgs a{};
    a.sys = s->d_self;
    a.moves = 1;
    a.props = s->d_props;
    a.detail = s->d_detail;
    a.pending = s->d_plain;
    a.pending_dq = s->K ? s->d_dq : nullptr;
    CUDA_TRY(launch_chain(a, 1, s->K, s->h.knc, chain_threads(s), false, st));
    fau_trial_result r{};
    CUDA_TRY(cudaMemcpyAsync(&r, s->d_detail, sizeof(r), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if ((rc = check_device_err(s))) return rc;
    r.accepted = 0;
    if (out) *out = r;
    s->pending = true;
    return FAU_OK;
}

int fau_commit_pending(fau_sys* s, int accept)
{
    if (!s) return fail(FAU_ERR_ARG, "null argument");
    if (!s->pending) return fail(FAU_ERR_STATE, "no pending trial");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    s->pending = false;
    cudaStream_t st = s->ctx->stream;
    if (accept) {
        CUDA_TRY(launch_plain_commit(s->d, s->d_plain, s->K, s->d_dq, st));
    }
    // a rejected trial needs no device work: the accepted state was never modified
    CUDA_TRY(cudaStreamSynchronize(st));
    const int rc = check_device_err(s);
    if (rc == FAU_ERR_CAPACITY) return rebuild_cells(s, 2 * s->h.cap);
    return rc;
}

int fau_get_positions(fau_sys* s, double* xyz)
{
    if (!s || !xyz) return fail(FAU_ERR_ARG, "null argument");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    std::vector<double> x(s->n), y(s->n), z(s->n);
    cudaStream_t st = s->ctx->stream;
    CUDA_TRY(cudaMemcpyAsync(x.data(), s->h.x, 8 * s->n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(y.data(), s->h.y, 8 * s->n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(z.data(), s->h.z, 8 * s->n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    for (int i = 0; i < s->n; i++) {
        xyz[3 * i] = x[i];
        xyz[3 * i + 1] = y[i];
        xyz[3 * i + 2] = z[i];
    }
    return FAU_OK;
}

int fau_get_mass_centers(fau_sys* s, double* xyz)
{
    if (!s || !xyz) return fail(FAU_ERR_ARG, "null argument");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    CUDA_TRY(cudaMemcpyAsync(xyz, s->h.g_cm, 24 * s->n_groups, cudaMemcpyDeviceToHost, s->ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    return FAU_OK;
}

int fau_get_cells(fau_sys* s, int* cell_out)
{
    if (!s || !cell_out) return fail(FAU_ERR_ARG, "null argument");
    if (!s->cells) {
        for (int i = 0; i < s->n; i++) cell_out[i] = -1;
        return FAU_OK;
    }
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    CUDA_TRY(cudaMemcpyAsync(cell_out, s->h.cell_of, 4 * s->n, cudaMemcpyDeviceToHost, s->ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    return FAU_OK;
}

int fau_get_cell_grid(const fau_sys* s, int dims[3])
{
    if (!s || !dims) return fail(FAU_ERR_ARG, "null argument");
    for (int k = 0; k < 3; k++) dims[k] = s->cells ? s->h.cdim[k] : 0;
    return FAU_OK;
}

int fau_refresh_energy(fau_sys* s, double* e)
{
    if (!s) return fail(FAU_ERR_ARG, "null system");
    if (s->pending) return fail(FAU_ERR_STATE, "refresh with a pending trial");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    const int rc = refresh_energy(s);
    if (rc) return rc;
    if (e) *e = s->h.energy;
    return FAU_OK;
}

int fau_get_box(const fau_sys* s, double* box)
{
    if (!s || !box) return fail(FAU_ERR_ARG, "null argument");
    for (int k = 0; k < 3; k++) box[k] = s->h.L[k];
    return FAU_OK;
}

int fau_get_running_energy(fau_sys* s, double* e)
{
    if (!s || !e) return fail(FAU_ERR_ARG, "null argument");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    int rc = pull_state(s);
    if (rc) return rc;
    *e = s->h.energy;
    return FAU_OK;
}

int fau_get_counters(fau_sys* s, int64_t* out)
{
    if (!s || !out) return fail(FAU_ERR_ARG, "null argument");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    int rc = pull_state(s);
    if (rc) return rc;
    out[0] = (int64_t)s->h.moves;
    out[1] = (int64_t)s->h.accepted;
    out[2] = (int64_t)s->h.pair_evals;
    out[3] = (int64_t)s->h.k_updates;
    return FAU_OK;
}

int fau_set_temperature_scale(fau_sys* s, double scale)
{
    if (!s || !(scale > 0.0) || !std::isfinite(scale)) return fail(FAU_ERR_ARG, "invalid scale");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    s->h.beta_scale = scale;
    CUDA_TRY(cudaMemcpyAsync(&s->d->beta_scale, &scale, sizeof(double), cudaMemcpyHostToDevice, s->ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    return FAU_OK;
}

int fau_get_q(fau_sys* s, double* q)
{
    if (!s || !q) return fail(FAU_ERR_ARG, "null argument");
    if (s->K == 0) return FAU_OK;
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    CUDA_TRY(launch_fold_q(s->d, s->K, s->ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(q, s->h.Q, sizeof(double2) * s->K, cudaMemcpyDeviceToHost, s->ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    return FAU_OK;
}

int fau_get_audit(fau_sys* s, double err_out[2], int64_t* samples)
{
    if (!s) return fail(FAU_ERR_ARG, "null argument");
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    DevSys cur;
    CUDA_TRY(cudaMemcpyAsync(&cur, s->d, sizeof(DevSys), cudaMemcpyDeviceToHost, s->ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    if (err_out) {
        err_out[0] = cur.audit_scaled_max;
        err_out[1] = cur.audit_rel_max;
    }
    if (samples) *samples = (int64_t)cur.audit_samples;
    return FAU_OK;
}

int fau_get_kvectors(fau_sys* s, int* n_out, double* k_out, double* ak_out)
{
    if (!s) return fail(FAU_ERR_ARG, "null argument");
    if (s->K == 0) return FAU_OK;
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    std::vector<int> kn(s->K);
    std::vector<double> ak(s->K);
    CUDA_TRY(cudaMemcpyAsync(kn.data(), s->h.kn, sizeof(int) * s->K, cudaMemcpyDeviceToHost, s->ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(ak.data(), s->h.Akd, sizeof(double) * s->K, cudaMemcpyDeviceToHost, s->ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    for (int k = 0; k < s->K; k++) {
        const int n[3] = {(kn[k] & 0xff) - 128, ((kn[k] >> 8) & 0xff) - 128, ((kn[k] >> 16) & 0xff) - 128};
        for (int d = 0; d < 3; d++) {
            if (n_out) n_out[3 * k + d] = n[d];
            // (2 pi) (n / L), as PolicyIonIon::updateBox forms it
            if (k_out) k_out[3 * k + d] = 2 * kPi * (double(n[d]) / s->h.L[d]);
        }
        if (ak_out) ak_out[k] = ak[k];
    }
    return FAU_OK;
}

int fau_q_rebuild(fau_sys* s, double* drift)
{
    const fau::NvtxRange nvtx_range("fau_q_rebuild");
    if (!s) return fail(FAU_ERR_ARG, "null argument");
    if (s->K == 0) {
        if (drift) *drift = 0.0;
        return FAU_OK;
    }
    CUDA_TRY(cudaSetDevice(s->ctx->device));
    cudaStream_t st = s->ctx->stream;
    std::vector<double2> before(s->K), after(s->K);
    CUDA_TRY(launch_fold_q(s->d, s->K, st));
    CUDA_TRY(cudaMemcpyAsync(before.data(), s->h.Q, sizeof(double2) * s->K, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(launch_q_rebuild(s->d, s->K, s->h.Q, st));
    CUDA_TRY(cudaMemcpyAsync(after.data(), s->h.Q, sizeof(double2) * s->K, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    double mx = 0.0;
    for (int k = 0; k < s->K; k++)
        mx = std::max(mx, std::max(std::fabs(before[k].x - after[k].x), std::fabs(before[k].y - after[k].y)));
    if (drift) *drift = mx;
    return FAU_OK;
}

} // extern "C"
