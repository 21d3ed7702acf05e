// fau_movegen.cpp -- host-side trial-move proposals drawn exactly as the
// reference's Move classes draw them, so a device chain fed with these
// proposals follows the reference's Markov chain.
//
// Streams: std::mt19937 `slump` (Move::slump, src/move.cpp:21) and `random`
// (global, src/random.cpp:62), uniform_real_distribution<double>(0,1)
// (Random::operator() src/random.cpp:57-60) and uniform_int_distribution<int>
// (Random::range / sample, src/random.h:47-66).
// Draw order of one performMove (src/montecarlo.cpp:139-187):
//   MoveCollection::sample (discrete_distribution on slump, src/move.cpp:513-526)
//   transrot   (src/move.cpp:267-293, randomAtom :328-346): group, particle,
//              randomUnitVector (src/core.cpp:249-261) then the scalar,
//              [unit vector + scalar when dprot > 0]
//   moltransrot (src/move.cpp:1670-1689): molecule from the global `random`,
//              unit vector then scalar, unit axis then angle
//   metropolisCriterion always draws one uniform (src/montecarlo.cpp:23-24),
//   and an empty change draws it too (:182-185).
// Where the reference's argument evaluation order is unspecified
// (`randomUnitVector(slump) * dp * slump()`) the unit vector is drawn first.
//
// Compiled without FMA contraction so the FP64 arithmetic is IEEE-exact.
#include "../../include/fau_gpu.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <sstream>
#include <string>
#include <vector>

extern "C" int fau_internal_fail(int code, const char* msg);

namespace {

struct Rng {
    std::mt19937 engine;
    std::uniform_real_distribution<double> dist01{0.0, 1.0};
    double operator()() { return dist01(engine); }
    int range(int lo, int hi) { return std::uniform_int_distribution<>(lo, hi)(engine); }
};

struct V3 {
    double x, y, z;
};

V3 unit_vector(Rng& r, const double dir[3])
{
    double p[3], n2;
    do {
        for (int k = 0; k < 3; k++) p[k] = (r() - 0.5) * dir[k];
        n2 = (p[0] * p[0] + p[1] * p[1]) + p[2] * p[2];
    } while (n2 > 0.25);
    const double n = std::sqrt(n2);
    return {p[0] / n, p[1] / n, p[2] / n};
}

struct MoveDef {
    int kind, volume_method = 0;
    double repeat, dp, dprot;
    double dir[3];
    std::vector<int> groups;
    std::vector<double> type_dp, type_dprot;
};

} // namespace

struct fau_movegen {
    Rng slump, random;
    std::vector<MoveDef> moves;
    std::discrete_distribution<unsigned int> pick;
    std::vector<int> g_begin, type;
};

extern "C" {

int fau_movegen_create(const fau_sys_desc* sp, const fau_move_desc* moves, int n_moves, uint32_t slump_seed,
                       uint32_t random_seed, int default_seeds, fau_movegen** out)
{
    if (!sp || !moves || n_moves < 1 || !out) return fau_internal_fail(FAU_ERR_ARG, "invalid movegen arguments");
    fau_movegen* g = new fau_movegen;
    if (!default_seeds) {
        g->slump.engine.seed(slump_seed);
        g->random.engine.seed(random_seed);
    }
    g->g_begin.assign(sp->group_begin, sp->group_begin + sp->n_groups + 1);
    g->type.assign(sp->type, sp->type + sp->n_particles);
    std::vector<double> w;
    for (int m = 0; m < n_moves; m++) {
        const fau_move_desc& d = moves[m];
        const bool vol = d.kind == FAU_MOVE_VOLUME;
        if ((d.kind != FAU_MOVE_ATOMIC && d.kind != FAU_MOVE_MOLECULAR && !vol) ||
            (!vol && (d.n_groups < 1 || !d.groups)) ||
            (vol && (d.volume_method < FAU_VOLUME_ISOTROPIC || d.volume_method > FAU_VOLUME_ISOCHORIC))) {
            delete g;
            return fau_internal_fail(FAU_ERR_ARG, "invalid move description");
        }
        MoveDef md;
        md.kind = d.kind;
        md.volume_method = d.volume_method;
        md.repeat = d.repeat;
        md.dp = d.dp;
        md.dprot = d.dprot;
        for (int k = 0; k < 3; k++) md.dir[k] = d.dir[k];
        if (!vol) md.groups.assign(d.groups, d.groups + d.n_groups);
        for (int gi : md.groups)
            if (gi < 0 || gi >= sp->n_groups) {
                delete g;
                return fau_internal_fail(FAU_ERR_ARG, "move group index out of range");
            }
        if (d.type_dp) md.type_dp.assign(d.type_dp, d.type_dp + sp->n_types);
        if (d.type_dprot) md.type_dprot.assign(d.type_dprot, d.type_dprot + sp->n_types);
        g->moves.push_back(md);
        w.push_back(d.repeat);
    }
    g->pick = std::discrete_distribution<unsigned int>(w.begin(), w.end());
    *out = g;
    return FAU_OK;
}

int fau_movegen_destroy(fau_movegen* g)
{
    delete g;
    return FAU_OK;
}

int fau_movegen_generate(fau_movegen* g, fau_proposal* out, int n)
{
    if (!g || (!out && n > 0) || n < 0) return fau_internal_fail(FAU_ERR_ARG, "invalid generate arguments");
    const double axis_dir[3] = {1.0, 1.0, 1.0};
    for (int it = 0; it < n; it++) {
        fau_proposal p;
        std::memset(&p, 0, sizeof(p));
        p.kind = FAU_MOVE_NONE;
        const MoveDef& m = g->moves[g->pick(g->slump.engine)];
        if (m.kind == FAU_MOVE_VOLUME) {
            // VolumeMove::setNewVolume (src/move.cpp:994-999): one slump() draw for ln V
            if (m.dp > 0.0) {
                p.kind = FAU_MOVE_VOLUME;
                p.index = m.volume_method;
                p.dr[0] = (g->slump() - 0.5) * m.dp;
            }
        }
        else if (m.kind == FAU_MOVE_ATOMIC) {
            const int gi = m.groups[g->slump.range(0, (int)m.groups.size() - 1)];
            const int b = g->g_begin[gi], size = g->g_begin[gi + 1] - b;
            if (size > 0) {
                const int particle = b + g->slump.range(0, size - 1);
                const int t = g->type[particle];
                double dp = m.dp, dprot = m.dprot;
                if (!m.type_dp.empty() && !std::isnan(m.type_dp[t])) dp = m.type_dp[t];
                if (!m.type_dprot.empty() && !std::isnan(m.type_dprot[t])) dprot = m.type_dprot[t];
                if (dp > 0.0) {
                    const V3 v = unit_vector(g->slump, m.dir);
                    const double s = g->slump();
                    p.dr[0] = v.x * dp * s;
                    p.dr[1] = v.y * dp * s;
                    p.dr[2] = v.z * dp * s;
                }
                if (dprot > 0.0) { // isotropic particles: rotation changes no energy, draws still happen
                    (void)unit_vector(g->slump, axis_dir);
                    (void)g->slump();
                }
                if (dp > 0.0 || dprot > 0.0) {
                    p.kind = FAU_MOVE_ATOMIC;
                    p.index = particle;
                }
            }
        }
        else {
            const int gi = m.groups[g->random.range(0, (int)m.groups.size() - 1)];
            double d2 = 0.0, a2 = 0.0;
            if (m.dp > 0.0) {
                const V3 v = unit_vector(g->slump, m.dir);
                const double s = g->slump();
                p.dr[0] = v.x * m.dp * s;
                p.dr[1] = v.y * m.dp * s;
                p.dr[2] = v.z * m.dp * s;
                d2 = (p.dr[0] * p.dr[0] + p.dr[1] * p.dr[1]) + p.dr[2] * p.dr[2];
            }
            if (m.dprot > 2.220446049250313e-16) {
                const V3 ax = unit_vector(g->slump, axis_dir);
                const double angle = m.dprot * (g->slump() - 0.5);
                const double ha = 0.5 * angle;
                const double sh = std::sin(ha);
                p.quat[0] = std::cos(ha);
                p.quat[1] = sh * ax.x;
                p.quat[2] = sh * ax.y;
                p.quat[3] = sh * ax.z;
                a2 = angle * angle;
            }
            if (d2 > 0.0 || a2 > 0.0) {
                p.kind = FAU_MOVE_MOLECULAR;
                p.index = gi;
            }
        }
        p.u = g->slump();
        out[it] = p;
    }
    return FAU_OK;
}

int fau_movegen_get_state(const fau_movegen* g, char* buf, size_t buflen)
{
    if (!g || !buf) return fau_internal_fail(FAU_ERR_ARG, "null argument");
    std::ostringstream os;
    os << g->slump.engine << "\n" << g->random.engine;
    const std::string s = os.str();
    if (s.size() + 1 > buflen) return fau_internal_fail(FAU_ERR_ARG, "state buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return FAU_OK;
}

int fau_movegen_set_state(fau_movegen* g, const char* state)
{
    if (!g || !state) return fau_internal_fail(FAU_ERR_ARG, "null argument");
    std::istringstream is(state);
    std::mt19937 a, b;
    is >> a >> b;
    if (!is) return fau_internal_fail(FAU_ERR_ARG, "malformed engine state");
    g->slump.engine = a;
    g->random.engine = b;
    return FAU_OK;
}

} // extern "C"
