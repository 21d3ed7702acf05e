/*
 * oracle.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU, FP64, IEEE (no fast-math, no FMA contraction) restatement of the
 * Faunus Metropolis Monte Carlo energy hot path.  The tests compare the GB300
 * library against it, and bench.py times it as the CPU baseline; nothing in the
 * product path may call it.  Every function cites the reference file:line it
 * follows (paths relative to the Faunus source tree).
 *
 * Parity status: pinned against the reference's own known-answer tests
 * (Ewald k-vector counts and two-ion energies, Ewald update/restore dU,
 * LJ mixing and force, hard-sphere thresholds, WCA, Coulomb Bjerrum length,
 * cell-grid arithmetic, RNG determinism) in tests/test_oracle_kat.py.
 * The Coulomb short-range functions of the external CoulombGalore library
 * (not vendored in the reference) are restated exactly from
 * docs/_docs/energy.md:169-205, whereas the reference splines them
 * (utol = 0.005/lB); real-space Ewald and cutoff-Coulomb energies are
 * therefore "parity unpinned" beyond that spline tolerance.
 *
 * Deliberate canonical choices where the reference's bits depend on its
 * build (Eigen SIMD width, argument evaluation order of overloaded operators):
 *   - |v|^2 is summed ((x*x + y*y) + z*z);
 *   - in `randomUnitVector(slump) * dp * slump()` the unit vector is drawn
 *     before the scalar (left to right, as clang evaluates it).
 */
#include "../include/fau_gpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace orc {

constexpr double pi = 3.141592653589793238462643383279502884;
constexpr double infty = std::numeric_limits<double>::infinity();
constexpr double neg_infty = -std::numeric_limits<double>::infinity();
constexpr double epsilon_dbl = std::numeric_limits<double>::epsilon();
constexpr double max_exp_argument = 709.782712893384; // src/units.h:16-17

struct Vec3 {
    double x = 0, y = 0, z = 0;
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline double sqnorm(const Vec3& a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }

// ---------------------------------------------------------------- geometry
// Cuboid periodic box: Chameleon::boundary / vdist / sqdist (src/geometry.h:407-485),
// anint (src/geometry.h:132-135).
struct Box {
    Vec3 len, half, inv;
    void set(const double L[3])
    {
        for (int d = 0; d < 3; d++) {
            len[d] = L[d];
            half[d] = 0.5 * L[d];
            inv[d] = 1.0 / L[d];
        }
    }
    static int anint(double x) { return int(x > 0.0 ? x + 0.5 : x - 0.5); }
    void boundary(Vec3& a) const
    {
        for (int d = 0; d < 3; d++)
            if (std::fabs(a[d]) > half[d]) a[d] -= len[d] * anint(a[d] * inv[d]);
    }
    Vec3 vdist(const Vec3& a, const Vec3& b) const
    {
        Vec3 r{a.x - b.x, a.y - b.y, a.z - b.z};
        for (int d = 0; d < 3; d++) {
            if (r[d] > half[d]) r[d] -= len[d];
            else if (r[d] < -half[d]) r[d] += len[d];
        }
        return r;
    }
    double sqdist(const Vec3& a, const Vec3& b) const
    {
        Vec3 d;
        for (int k = 0; k < 3; k++) {
            double v = std::fabs(a[k] - b[k]);
            d[k] = v - (v > half[k] ? len[k] : 0.0);
        }
        return sqnorm(d);
    }
    double volume() const { return len.x * len.y * len.z; }
};

// ---------------------------------------------------------------- pair potential
// Sum of the enabled terms in the order coulomb, LJ, WCA, HS
// (CombinedPairPotential::operator() src/potentials_base.h:234-240).
struct PairParams {
    int n_types = 0;
    std::vector<double> sigma2, eps4, hs2;
    int terms = 0, coul_type = FAU_COUL_PLAIN;
    double lB = 0, rc_coul = 0, alpha = 0, pair_cutoff2 = 0;
    // FAU_COUL_TRUNC: S(q) = cerfc erfc(alpha r) + sum_k cpoly[k] q^k (docs/_docs/energy.md:169-213
    // at infinite Debye length; the host turns each named scheme into these coefficients)
    double cerfc = 0;
    std::vector<double> cpoly;
    // FAU_PAIR_SPLINE: KnotData per atom-type pair (src/potentials.h:773-780): knots z in r^2
    // from spl_begin[ab], 6 coefficients a piece from 6 (spl_begin[ab] - ab)
    std::vector<int> spl_begin, spl_hs;
    std::vector<double> spl_z, spl_c;

    // Andrea::eval src/tabulate.h:188-207: the piece z_i < z <= z_{i+1} by lower_bound, then
    // Horner in z - z_i (absolute: the sum of |c_k| |dz|^k instead)
    double spline(size_t ab, double r2, bool absolute) const
    {
        const double* z = spl_z.data() + spl_begin[ab];
        const int m = spl_begin[ab + 1] - spl_begin[ab];
        long i = (long)(std::lower_bound(z, z + m, r2) - z) - 1;
        i = std::min(std::max(i, 0L), (long)m - 2);
        const double* c = spl_c.data() + 6 * (size_t(spl_begin[ab]) - ab) + 6 * i;
        const double dz = absolute ? std::fabs(r2 - z[i]) : r2 - z[i];
        double sum = 0;
        for (int k = 5; k > 0; k--) sum = dz * (sum + (absolute ? std::fabs(c[k]) : c[k]));
        return sum + (absolute ? std::fabs(c[0]) : c[0]);
    }
    // SplinedPotential::operator() src/potentials.h:807-823: 1 spline, 0 beyond the last knot,
    // -1 +inf (hard sphere), 2 the exact terms
    int spline_region(size_t ab, double r2) const
    {
        if (r2 >= spl_z[spl_begin[ab + 1] - 1]) return 0;
        if (r2 > spl_z[spl_begin[ab]]) return 1;
        return spl_hs[ab] ? -1 : 2;
    }

    double trunc_s(double r, bool absolute) const
    {
        const double q = r / rc_coul;
        double s = 0.0;
        for (size_t k = cpoly.size(); k-- > 0;) s = s * q + (absolute ? std::fabs(cpoly[k]) : cpoly[k]);
        if (cerfc != 0.0) s += (absolute ? std::fabs(cerfc) : cerfc) * std::erfc(alpha * r);
        return s;
    }

    double coulomb(double qa, double qb, double r2) const
    {
        if (coul_type == FAU_COUL_PLAIN) // Coulomb::operator() src/potentials.h:472-476
            return lB * qa * qb / std::sqrt(r2);
        // NewCoulombGalore::operator() src/potentials.h:591-598: r + epsilon, S(q), 0 beyond Rc
        const double r = std::sqrt(r2) + epsilon_dbl;
        if (r >= rc_coul) return 0.0;
        double s = 1.0;
        if (coul_type == FAU_COUL_EWALD) s = std::erfc(alpha * r);
        else if (coul_type == FAU_COUL_TRUNC) s = trunc_s(r, false);
        return lB * (qa * qb / r * s);
    }
    double operator()(int ta, int tb, double qa, double qb, double r2) const
    {
        if (pair_cutoff2 > 0.0 && r2 >= pair_cutoff2) return 0.0;
        const size_t ab = size_t(ta) * n_types + tb;
        if (terms & FAU_PAIR_SPLINE) {
            const int reg = spline_region(ab, r2);
            if (reg == 0) return 0.0;
            if (reg == 1) return spline(ab, r2, false);
            if (reg < 0) return infty;
        }
        double u = 0.0;
        if (terms & FAU_PAIR_COULOMB) u += coulomb(qa, qb, r2);
        if (terms & FAU_PAIR_LJ) { // LennardJones src/potentials.h:42-49
            double x = sigma2[ab] / r2;
            x = x * x * x;
            u += eps4[ab] * (x * x - x);
        }
        if (terms & FAU_PAIR_WCA) { // WeeksChandlerAndersen src/potentials.h:151-160
            double x = sigma2[ab];
            double w = 0.0;
            if (!(r2 > x * 1.2599210498948732)) {
                x = x / r2;
                x = x * x * x;
                w = eps4[ab] * (x * x - x + 0.25);
            }
            u += w;
        }
        if (terms & FAU_PAIR_HS) // HardSphere src/potentials.h:203-207
            u += (r2 < hs2[ab]) ? infty : 0.0;
        return u;
    }
    // sum of |summand| over the enabled terms: the floating-point error scale of a pair
    // energy.  The r^-12 and r^-6 parts of LJ / WCA count separately: they cancel near
    // r = sigma, where the rounding error of any evaluation scales with their sum.
    double magnitude(int ta, int tb, double qa, double qb, double r2) const
    {
        if (pair_cutoff2 > 0.0 && r2 >= pair_cutoff2) return 0.0;
        const size_t ab = size_t(ta) * n_types + tb;
        if (terms & FAU_PAIR_SPLINE) {
            const int reg = spline_region(ab, r2);
            if (reg == 1) return spline(ab, r2, true);
            if (reg != 2) return 0.0;
        }
        double m = 0.0;
        if (terms & FAU_PAIR_COULOMB) {
            if (coul_type == FAU_COUL_TRUNC) { // |qq/r| (|e| erfc + sum |c_k| q^k): S cancels to 0 at Rc
                const double r = std::sqrt(r2) + epsilon_dbl;
                if (r < rc_coul) m += std::fabs(lB * qa * qb / r) * trunc_s(r, true);
            }
            else
                m += std::fabs(coulomb(qa, qb, r2));
        }
        double x = sigma2[ab] / r2;
        x = x * x * x;
        const double e = std::fabs(eps4[ab]);
        if (terms & FAU_PAIR_LJ) m += e * (x * x + x);
        if ((terms & FAU_PAIR_WCA) && !(r2 > sigma2[ab] * 1.2599210498948732)) m += e * (x * x + x + 0.25);
        return std::isfinite(m) ? m : 0.0;
    }
    // self energy per particle (NewCoulombGalore::setSelfEnergy src/potentials.cpp:1599-1604)
    // = -1/2 lim_{r->0} (u - u~) = lB q^2 S'(0) / (2 Rc) (docs/_docs/energy.md:267-276)
    bool has_self() const { return (terms & FAU_PAIR_COULOMB) && coul_type != FAU_COUL_PLAIN; }
    double self(double q) const
    {
        if (!has_self()) return 0.0;
        if (coul_type == FAU_COUL_EWALD) return lB * (-alpha / std::sqrt(pi) * q * q);
        if (coul_type == FAU_COUL_TRUNC) {
            const double ds0 = (cpoly.size() > 1 ? cpoly[1] : 0.0) - cerfc * 2.0 * alpha * rc_coul / std::sqrt(pi);
            return lB * (ds0 / (2.0 * rc_coul) * q * q);
        }
        return 0.0; // S(q) == 1 near q = 0: no self energy
    }
};

// ---------------------------------------------------------------- Ewald
// EwaldData (src/energy.h:92-122, src/energy.cpp:28-59)
struct Ewald {
    bool enabled = false, ipbc = false, spherical = true;
    double alpha = 0, ncut = 0, epss = 0, lB = 0, const_inf = 0, check_k2_zero = 0;
    std::vector<Vec3> k;
    std::vector<double> Ak;
    std::vector<std::complex<double>> Q;

    // PolicyIonIon::updateBox src/energy.cpp:133-186 and the IPBC variant :356-404
    void updateBox(const Box& box)
    {
        const int nc = (int)std::ceil(ncut);
        const double Lmax = std::max(box.len.x, std::max(box.len.y, box.len.z));
        check_k2_zero = 0.1 * std::pow(2 * pi / Lmax, 2);
        k.clear();
        Ak.clear();
        const int ksize = (2 * nc + 1) * (2 * nc + 1) * (2 * nc + 1) - 1;
        if (ksize == 0) {
            k.push_back({1, 0, 0});
            Ak.push_back(0.0);
            Q.assign(1, {0, 0});
            return;
        }
        const double nc2 = ncut * ncut;
        const int start = ipbc ? 0 : 1;
        for (int nx = 0; nx <= nc; nx++) {
            const double dnx2 = double(nx * nx);
            const double xfactor = (nx > 0) ? 2.0 : 1.0;
            for (int ny = -nc * start; ny <= nc; ny++) {
                const double dny2 = double(ny * ny);
                const double yfactor = (ipbc && ny > 0) ? 2.0 : 1.0;
                for (int nz = -nc * start; nz <= nc; nz++) {
                    double factor = xfactor * yfactor;
                    if (ipbc && nz > 0) factor *= 2;
                    // 2 * pi * Point(n).cwiseQuotient(L): (2*pi) * (n / L) per component
                    Vec3 kv{2 * pi * (double(nx) / box.len.x), 2 * pi * (double(ny) / box.len.y),
                            2 * pi * (double(nz) / box.len.z)};
                    const double k2 = sqnorm(kv); // + kappa^2, kappa = 0
                    if (k2 < check_k2_zero) continue;
                    if (spherical) {
                        const double dnz2 = double(nz * nz);
                        if ((dnx2 + dny2 + dnz2) / nc2 > 1) continue;
                    }
                    k.push_back(kv);
                    Ak.push_back(factor * std::exp(-k2 / (4 * alpha * alpha)) / k2);
                }
            }
        }
        Q.assign(k.size(), {0, 0});
    }
    double dot(const Vec3& a, const Vec3& b) const { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
    std::complex<double> term(size_t kk, const Vec3& r, double q) const
    {
        if (ipbc) { // PolicyIonIonIPBC::updateComplex src/energy.cpp:406-419
            const Vec3& kv = k[kk];
            double c = std::cos(kv.x * r.x) * std::cos(kv.y * r.y) * std::cos(kv.z * r.z);
            return {c * q, 0.0};
        }
        const double qr = dot(k[kk], r);
        return q * std::complex<double>(std::cos(qr), std::sin(qr));
    }
    // full update src/energy.cpp:191-206
    void fullQ(const std::vector<Vec3>& pos, const std::vector<double>& charge)
    {
        for (size_t kk = 0; kk < k.size(); kk++) {
            std::complex<double> s(0, 0);
            for (size_t i = 0; i < pos.size(); i++) s += term(kk, pos[i], charge[i]);
            Q[kk] = s;
        }
    }
    // partial update src/energy.cpp:219-247: Q += q e(new) - q e(old) per moved atom
    void partialQ(const std::vector<Vec3>& new_pos, const std::vector<Vec3>& old_pos,
                  const std::vector<double>& q)
    {
        for (size_t kk = 0; kk < k.size(); kk++) {
            for (size_t a = 0; a < q.size(); a++) {
                Q[kk] += term(kk, new_pos[a], q[a]);
                Q[kk] -= term(kk, old_pos[a], q[a]);
            }
        }
    }
    // src/energy.cpp:524-531
    double reciprocal(const Box& box) const
    {
        double e = 0;
        for (size_t kk = 0; kk < Q.size(); kk++) e += Ak[kk] * std::norm(Q[kk]);
        return 2 * pi * e * lB / box.volume();
    }
    // src/energy.cpp:466-482 (ignores the change; all particles)
    double surface(const Box& box, const std::vector<Vec3>& pos, const std::vector<double>& q) const
    {
        if (const_inf < 0.5) return 0.0;
        Vec3 m{0, 0, 0};
        for (size_t i = 0; i < pos.size(); i++) {
            m.x += q[i] * pos[i].x;
            m.y += q[i] * pos[i].y;
            m.z += q[i] * pos[i].z;
        }
        return const_inf * 2.0 * pi / ((2.0 * epss + 1.0) * box.volume()) * sqnorm(m) * lB;
    }
    // PolicyIonIon::selfEnergy src/energy.cpp:484-518 (Change::everything branch, kappa = 0)
    double policySelf(const Box& box, const std::vector<double>& q) const
    {
        double q2 = 0, qt = 0;
        for (double c : q) {
            q2 += c * c;
            qt += c;
        }
        const double Vcc = -pi / 2.0 / alpha / alpha / (box.len.x * box.len.y * box.len.z) * qt * qt;
        return (-alpha * q2 / std::sqrt(pi) * (std::exp(0.0) + 0.0) + Vcc) * lB;
    }
};

// ---------------------------------------------------------------- RNG
// Random src/random.h:34-66, src/random.cpp:57-60
struct Random {
    std::mt19937 engine;
    std::uniform_real_distribution<double> dist01{0, 1};
    double operator()() { return dist01(engine); }
    int range(int a, int b) { return std::uniform_int_distribution<>(a, b)(engine); }
};
// randomUnitVector src/core.cpp:249-261
static Vec3 randomUnitVector(Random& rand, const Vec3& dir)
{
    double r2;
    Vec3 p;
    do {
        for (int i = 0; i < 3; i++) p[i] = (rand() - 0.5) * dir[i];
        r2 = sqnorm(p);
    } while (r2 > 0.25);
    const double n = std::sqrt(r2);
    return {p.x / n, p.y / n, p.z / n};
}

// quaternion from Eigen::AngleAxisd and Quaternion * vector (q v q*): restated
// from the standard formula v' = v + w t + u x t, t = 2 u x v.
struct Quat {
    double w = 1, x = 0, y = 0, z = 0;
};
static Quat angleAxis(double angle, const Vec3& axis)
{
    const double ha = 0.5 * angle;
    const double s = std::sin(ha);
    return {std::cos(ha), s * axis.x, s * axis.y, s * axis.z};
}
static Vec3 cross(const Vec3& a, const Vec3& b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static Vec3 rotateVec(const Quat& q, const Vec3& v)
{
    const Vec3 u{q.x, q.y, q.z};
    Vec3 t = cross(u, v);
    t = {t.x + t.x, t.y + t.y, t.z + t.z};
    const Vec3 c = cross(u, t);
    return {v.x + q.w * t.x + c.x, v.y + q.w * t.y + c.y, v.z + q.w * t.z + c.z};
}

// ---------------------------------------------------------------- system
struct Group {
    int begin = 0, end = 0, molid = 0, flags = 0;
    bool atomic() const { return flags & FAU_GROUP_ATOMIC; }
    bool rigid() const { return flags & FAU_GROUP_RIGID; }
    int size() const { return end - begin; }
};

struct System {
    Box box;
    std::vector<Vec3> pos;
    std::vector<double> q;
    std::vector<int> type;
    std::vector<Group> groups;
    std::vector<Vec3> cm;
    std::vector<double> mass; // per type
    std::vector<int> group_of;
    PairParams pair;
    Ewald ewald;
    double cutoff_g2g2 = std::numeric_limits<double>::max();
    int n_molids = 0;              // > 0: per molecule-kind pair cutoffs^2 below
    std::vector<double> cut2_pairs;
    bool isobaric = false;  // Isobaric term (src/energy.cpp:859-901) with `pressure` in kT / A^3
    double pressure = 0.0;
    double maxenergy = infty; // Hamiltonian maxenergy
    bool want_scale = true; // sum |u| over both states for tolerance checks (not in the reference)
    // MC bookkeeping (MetropolisMonteCarlo)
    double initial_energy = 0, sum_of_energy_changes = 0;

    // GroupCutoff::cut src/energy.h:761-768
    bool cut(int g1, int g2) const
    {
        if (groups[g1].atomic() || groups[g2].atomic()) return false;
        const double c2 = n_molids > 0 ? cut2_pairs[size_t(groups[g1].molid) * n_molids + groups[g2].molid] : cutoff_g2g2;
        return box.sqdist(cm[g1], cm[g2]) >= c2;
    }
    double u(int i, int j) const { return pair(type[i], type[j], q[i], q[j], box.sqdist(pos[i], pos[j])); }
    double mag(int i, int j) const { return pair.magnitude(type[i], type[j], q[i], q[j], box.sqdist(pos[i], pos[j])); }
    double u_at(const Vec3& ri, int ti, double qi, int j) const
    {
        return pair(ti, type[j], qi, q[j], box.sqdist(ri, pos[j]));
    }
    // massCenter with shift (src/geometry.h:505-526, 563-…)
    Vec3 massCenter(int g, const Vec3& shift) const
    {
        double ws = 0;
        Vec3 c{0, 0, 0};
        for (int i = groups[g].begin; i < groups[g].end; i++) {
            Vec3 p{pos[i].x + shift.x, pos[i].y + shift.y, pos[i].z + shift.z};
            box.boundary(p);
            const double w = mass.empty() ? 1.0 : mass[type[i]];
            c.x += w * p.x;
            c.y += w * p.y;
            c.z += w * p.z;
            ws += w;
        }
        if (std::fabs(ws) > epsilon_dbl) {
            c = {c.x / ws - shift.x, c.y / ws - shift.y, c.z / ws - shift.z};
            box.boundary(c);
            return c;
        }
        return {0, 0, 0};
    }
};

// pairing.all src/energy.h:1290-1299 (groupInternal :856-870 + group2group :980-989)
static double nonbondedAll(const System& s)
{
    double e = 0;
    for (size_t g = 0; g < s.groups.size(); g++) {
        const Group& G = s.groups[g];
        if (!G.rigid())
            for (int i = G.begin; i < G.end - 1; i++)
                for (int j = i + 1; j < G.end; j++) e += s.u(i, j);
        for (size_t h = g + 1; h < s.groups.size(); h++) {
            if (s.cut((int)g, (int)h)) continue;
            for (int i = G.begin; i < G.end; i++)
                for (int j = s.groups[h].begin; j < s.groups[h].end; j++) e += s.u(i, j);
        }
    }
    return e;
}
// single-atom change: group2all(group, index) :1183-1195 + groupInternal(group, index) :886-914
static double nonbondedAtom(const System& s, int i)
{
    const int g = s.group_of[i];
    const Group& G = s.groups[g];
    double e = 0;
    for (size_t h = 0; h < s.groups.size(); h++) {
        if ((int)h == g) continue;
        if (s.cut((int)h, g)) continue;
        for (int j = s.groups[h].begin; j < s.groups[h].end; j++) e += s.u(i, j);
    }
    if (!G.rigid()) { // internal = true for transrot
        for (int j = G.begin; j < i; j++) e += s.u(i, j);
        for (int j = i + 1; j < G.end; j++) e += s.u(i, j);
    }
    return e;
}
// whole-group change, internal = false: group2all(group) :1156-1163
static double nonbondedGroup(const System& s, int g)
{
    const Group& G = s.groups[g];
    double e = 0;
    for (size_t h = 0; h < s.groups.size(); h++) {
        if ((int)h == g) continue;
        if (s.cut(g, (int)h)) continue;
        for (int i = G.begin; i < G.end; i++)
            for (int j = s.groups[h].begin; j < s.groups[h].end; j++) e += s.u(i, j);
    }
    return e;
}

struct Terms {
    double self = 0, nb = 0, rec = 0, surf = 0, total = 0;
};

// Hamiltonian::energy src/energy.cpp:1227-1241: terms in order, early break on
// >= maxenergy (maximum_allowed_energy, +inf unless set, src/energy.cpp:1189-1193) or NaN,
// summed with std::accumulate.
static double accumulateTerms(const double* t, int n, double maxenergy)
{
    std::vector<double> latest;
    for (int i = 0; i < n; i++) {
        latest.push_back(t[i]);
        if (t[i] >= maxenergy || std::isnan(t[i])) break;
    }
    double s = 0.0;
    for (double v : latest) s += v;
    return s;
}

enum ChangeKind { CH_EVERYTHING, CH_ATOM, CH_GROUP };

static Terms energyOf(const System& s, ChangeKind kind, int index)
{
    Terms t;
    std::vector<double> list;
    if (s.pair.has_self()) { // ExternalPotential::energy src/externalpotential.cpp:94-126
        double e = 0;
        if (kind == CH_EVERYTHING) {
            for (size_t i = 0; i < s.pos.size(); i++) e += s.pair.self(s.q[i]);
        }
        else if (kind == CH_ATOM) {
            e = s.pair.self(s.q[index]);
        }
        else {
            for (int i = s.groups[index].begin; i < s.groups[index].end; i++) e += s.pair.self(s.q[i]);
        }
        t.self = e;
        list.push_back(e);
    }
    t.nb = (kind == CH_EVERYTHING) ? nonbondedAll(s) : (kind == CH_ATOM ? nonbondedAtom(s, index) : nonbondedGroup(s, index));
    list.push_back(t.nb);
    if (s.ewald.enabled) {
        t.surf = s.ewald.surface(s.box, s.pos, s.q);
        t.rec = s.ewald.reciprocal(s.box);
        list.push_back(t.surf + t.rec); // Ewald::energy src/energy.cpp:581-587
    }
    t.total = accumulateTerms(list.data(), (int)list.size(), s.maxenergy);
    return t;
}

// getEnergyChange src/montecarlo.cpp:193-209
static double getEnergyChange(double new_energy, double old_energy)
{
    if (std::isnan(old_energy) && !std::isnan(new_energy)) return neg_infty;
    if (std::isnan(new_energy)) return infty;
    if (new_energy > 0.0 && std::isinf(new_energy)) return infty;
    const double du = new_energy - old_energy;
    if (std::isnan(du)) return 0.0;
    return du;
}
// metropolisCriterion src/montecarlo.cpp:17-34, uniform already drawn by the caller.
// returns -1 for NaN (the reference throws)
static int metropolis(double du, double u)
{
    if (std::isnan(du)) return -1;
    if (std::isinf(du) && du < 0.0) return 1;
    if (-du > max_exp_argument) return 1;
    return u <= std::exp(-du) ? 1 : 0;
}

// ------------------------------------------------------------- trial moves
// performMove src/montecarlo.cpp:139-187 on host-fed proposals.
struct TrialOut {
    double du = 0, du_nb = 0, du_ew = 0, scale = 0;
    int accepted = 0, new_inf = 0, old_inf = 0, nan = 0;
};

// magnitude of the terms the reciprocal-energy change is summed from:
// (2 pi lB / V) sum_k A_k (|2 Re(conj(Q_old) d)| + |d|^2), d = Q_new - Q_old
static double ewaldScale(const System& s, const std::vector<std::complex<double>>& Qold)
{
    if (!s.ewald.enabled) return 0.0;
    double e = 0.0;
    for (size_t k = 0; k < Qold.size(); k++) {
        const std::complex<double> d = s.ewald.Q[k] - Qold[k];
        const double cross = 2.0 * (Qold[k].real() * d.real() + Qold[k].imag() * d.imag());
        e += s.ewald.Ak[k] * (std::fabs(cross) + std::norm(d));
    }
    return 2 * pi * e * s.ewald.lB / s.box.volume();
}

static TrialOut trialAtom(System& s, int i, const Vec3& dr, double u01)
{
    TrialOut out;
    // AtomicTranslateRotate::translateParticle src/move.cpp:225-240
    const Vec3 old = s.pos[i];
    Vec3 np{old.x + dr.x, old.y + dr.y, old.z + dr.z};
    s.box.boundary(np);
    const Terms eo = energyOf(s, CH_ATOM, i); // accepted state
    // scale: sum of |pair terms| over both states
    double scale = 0;
    auto addScale = [&]() {
        if (!s.want_scale) return;
        for (int j = 0; j < (int)s.pos.size(); j++)
            if (j != i) scale += s.mag(i, j);
    };
    addScale();
    std::vector<std::complex<double>> Qacc = s.ewald.Q;
    s.pos[i] = np;
    if (s.ewald.enabled) s.ewald.partialQ({np}, {old}, {s.q[i]}); // Ewald::updateState (trial)
    const Terms en = energyOf(s, CH_ATOM, i);
    addScale();
    if (s.want_scale) scale += ewaldScale(s, Qacc);
    // a sum that stopped before the Ewald term (maxenergy): the energy change then carries the
    // other state's whole Ewald energy, which joins the error scale
    if (s.want_scale && (!(en.nb < s.maxenergy) || !(eo.nb < s.maxenergy)))
        scale += std::fabs(en.rec + en.surf) + std::fabs(eo.rec + eo.surf);
    out.du = getEnergyChange(en.total, eo.total);
    out.du_nb = en.nb - eo.nb;
    out.du_ew = (en.rec + en.surf) - (eo.rec + eo.surf);
    out.scale = scale;
    out.new_inf = std::isinf(en.total) && en.total > 0;
    out.old_inf = std::isinf(eo.total) && eo.total > 0;
    const int acc = metropolis(out.du, u01);
    if (acc < 0) out.nan = 1;
    out.accepted = acc == 1;
    if (out.accepted) {
        s.sum_of_energy_changes += out.du;
    }
    else { // reject: trial.sync(accepted)
        s.pos[i] = old;
        s.ewald.Q = Qacc;
    }
    return out;
}

// TranslateRotate: Group::translate (src/group.cpp:115-123) then Group::rotate
// (src/group.cpp:110-113, Geometry::rotate src/geometry.h:613-627)
static void moveGroup(System& s, int g, const Vec3& dr, const Quat* q)
{
    Group& G = s.groups[g];
    Vec3& c = s.cm[g];
    c = {c.x + dr.x, c.y + dr.y, c.z + dr.z};
    s.box.boundary(c);
    for (int i = G.begin; i < G.end; i++) {
        Vec3& p = s.pos[i];
        p = {p.x + dr.x, p.y + dr.y, p.z + dr.z};
        s.box.boundary(p);
    }
    if (q) {
        const Vec3 shift{-s.cm[g].x, -s.cm[g].y, -s.cm[g].z};
        for (int i = G.begin; i < G.end; i++) {
            Vec3& p = s.pos[i];
            p = {p.x + shift.x, p.y + shift.y, p.z + shift.z};
            s.box.boundary(p);
            Vec3 r = rotateVec(*q, p);
            p = {r.x - shift.x, r.y - shift.y, r.z - shift.z};
            s.box.boundary(p);
        }
    }
}

static TrialOut trialGroup(System& s, int g, const Vec3& dr, const Quat* q, double u01)
{
    TrialOut out;
    const Group& G = s.groups[g];
    std::vector<Vec3> oldp(s.pos.begin() + G.begin, s.pos.begin() + G.end);
    const Vec3 oldcm = s.cm[g];
    const Terms eo = energyOf(s, CH_GROUP, g);
    double scale = 0;
    auto addScale = [&]() {
        if (!s.want_scale) return;
        for (size_t h = 0; h < s.groups.size(); h++) {
            if ((int)h == g || s.cut(g, (int)h)) continue;
            for (int i = G.begin; i < G.end; i++)
                for (int j = s.groups[h].begin; j < s.groups[h].end; j++) scale += s.mag(i, j);
        }
    };
    addScale();
    std::vector<std::complex<double>> Qacc = s.ewald.Q;
    moveGroup(s, g, dr, q);
    if (s.ewald.enabled) {
        std::vector<Vec3> np(s.pos.begin() + G.begin, s.pos.begin() + G.end);
        std::vector<double> qq(s.q.begin() + G.begin, s.q.begin() + G.end);
        s.ewald.partialQ(np, oldp, qq);
    }
    const Terms en = energyOf(s, CH_GROUP, g);
    addScale();
    if (s.want_scale) scale += ewaldScale(s, Qacc);
    // a sum that stopped before the Ewald term (maxenergy): the energy change then carries the
    // other state's whole Ewald energy, which joins the error scale
    if (s.want_scale && (!(en.nb < s.maxenergy) || !(eo.nb < s.maxenergy)))
        scale += std::fabs(en.rec + en.surf) + std::fabs(eo.rec + eo.surf);
    out.du = getEnergyChange(en.total, eo.total);
    out.du_nb = en.nb - eo.nb;
    out.du_ew = (en.rec + en.surf) - (eo.rec + eo.surf);
    out.scale = scale;
    out.new_inf = std::isinf(en.total) && en.total > 0;
    out.old_inf = std::isinf(eo.total) && eo.total > 0;
    const int acc = metropolis(out.du, u01);
    if (acc < 0) out.nan = 1;
    out.accepted = acc == 1;
    if (out.accepted) {
        s.sum_of_energy_changes += out.du;
    }
    else {
        std::copy(oldp.begin(), oldp.end(), s.pos.begin() + G.begin);
        s.cm[g] = oldcm;
        s.ewald.Q = Qacc;
    }
    return out;
}

// ------------------------------------------------------------- move generation
// MoveCollection (src/move.cpp:475-526), AtomicTranslateRotate (:190-365),
// TranslateRotate (:1559-1723).
struct MoveDef {
    int kind, volume_method = 0;
    double repeat, dp, dprot;
    Vec3 dir;
    std::vector<int> groups;
    std::vector<double> type_dp, type_dprot;
};
struct MoveGen {
    Random slump, random;
    std::vector<MoveDef> moves;
    std::discrete_distribution<unsigned int> dist;
    const System* sys = nullptr;

    fau_proposal next()
    {
        fau_proposal p;
        std::memset(&p, 0, sizeof(p));
        p.kind = FAU_MOVE_NONE;
        const MoveDef& m = moves[dist(slump.engine)]; // MoveCollection::sample
        if (m.kind == FAU_MOVE_VOLUME) {
            // VolumeMove::_move / setNewVolume (src/move.cpp:994-1006): dV = 0 is an empty change
            if (m.dp > 0.0) {
                p.kind = FAU_MOVE_VOLUME;
                p.index = m.volume_method;
                p.dr[0] = (slump() - 0.5) * m.dp;
            }
        }
        else if (m.kind == FAU_MOVE_ATOMIC) {
            // randomAtom: group then particle (src/move.cpp:328-346)
            const int gi = m.groups[slump.range(0, (int)m.groups.size() - 1)];
            const Group& G = sys->groups[gi];
            int particle = -1;
            if (G.size() > 0) particle = G.begin + slump.range(0, G.size() - 1);
            if (particle >= 0) {
                const int t = sys->type[particle];
                double dp = m.dp, dprot = m.dprot;
                if (!m.type_dp.empty() && !std::isnan(m.type_dp[t])) dp = m.type_dp[t];
                if (!m.type_dprot.empty() && !std::isnan(m.type_dprot[t])) dprot = m.type_dprot[t];
                if (dp > 0.0) {
                    const Vec3 v = randomUnitVector(slump, m.dir);
                    const double s = slump();
                    p.dr[0] = v.x * dp * s;
                    p.dr[1] = v.y * dp * s;
                    p.dr[2] = v.z * dp * s;
                }
                if (dprot > 0.0) { // rotation of the (isotropic) particle: draws only
                    (void)randomUnitVector(slump, {1, 1, 1});
                    (void)slump();
                }
                if (dp > 0.0 || dprot > 0.0) {
                    p.kind = FAU_MOVE_ATOMIC;
                    p.index = particle;
                }
            }
        }
        else {
            // findRandomMolecule uses the global `random` (src/move.cpp:1618-1628)
            const int gi = m.groups[random.range(0, (int)m.groups.size() - 1)];
            double d2 = 0, a2 = 0;
            if (m.dp > 0.0) {
                const Vec3 v = randomUnitVector(slump, m.dir);
                const double s = slump();
                p.dr[0] = v.x * m.dp * s;
                p.dr[1] = v.y * m.dp * s;
                p.dr[2] = v.z * m.dp * s;
                d2 = sqnorm({p.dr[0], p.dr[1], p.dr[2]});
            }
            if (m.dprot > epsilon_dbl) {
                const Vec3 axis = randomUnitVector(slump, {1, 1, 1});
                const double angle = m.dprot * (slump() - 0.5);
                const Quat q = angleAxis(angle, axis);
                p.quat[0] = q.w;
                p.quat[1] = q.x;
                p.quat[2] = q.y;
                p.quat[3] = q.z;
                a2 = angle * angle;
            }
            if (d2 > 0.0 || a2 > 0.0) {
                p.kind = FAU_MOVE_MOLECULAR;
                p.index = gi;
            }
        }
        p.u = slump(); // metropolisCriterion (or the empty-change draw)
        return p;
    }
};

// ------------------------------------------------------------- cell grid
// GridBase::updateCellGrid src/celllistimpl.h:223-236, coordinatesAt :139-143,
// index :125-129, periodic index wrap :313-327, positions shifted by +L/2
// (src/sasa.cpp:466-468).
static void cellGrid(const double L[3], double min_cell, int dims[3], double cell[3])
{
    for (int d = 0; d < 3; d++) {
        dims[d] = (int)std::floor(L[d] / std::min(L[d], min_cell));
        cell[d] = L[d] / double(dims[d]);
    }
}
static int cellIndexAt(const double L[3], const int dims[3], const double cell[3], const Vec3& p)
{
    int c[3];
    for (int d = 0; d < 3; d++) {
        const double x = p[d] + 0.5 * L[d];
        int v = (int)std::floor(x / cell[d]);
        if (v < 0) v += dims[d] * (std::abs(v) / dims[d] + 1);
        else if (v >= dims[d]) v -= dims[d] * (v / dims[d]);
        c[d] = v;
    }
    return c[0] + dims[0] * (c[1] + dims[1] * c[2]);
}

} // namespace orc

using namespace orc;

// ================================================================== C ABI
struct orc_sys {
    System s;
};
struct orc_movegen {
    MoveGen g;
};

static System buildSystem(const fau_sys_desc* d)
{
    System s;
    s.box.set(d->box);
    const int n = d->n_particles;
    s.pos.resize(n);
    s.q.assign(d->charge, d->charge + n);
    s.type.assign(d->type, d->type + n);
    for (int i = 0; i < n; i++) s.pos[i] = {d->pos[3 * i], d->pos[3 * i + 1], d->pos[3 * i + 2]};
    s.groups.resize(d->n_groups);
    s.group_of.assign(n, -1);
    for (int g = 0; g < d->n_groups; g++) {
        s.groups[g] = {d->group_begin[g], d->group_begin[g + 1], d->group_molid ? d->group_molid[g] : 0,
                       d->group_flags ? d->group_flags[g] : FAU_GROUP_ATOMIC};
        for (int i = s.groups[g].begin; i < s.groups[g].end; i++) s.group_of[i] = g;
    }
    const int nt = d->n_types;
    if (d->type_mass) s.mass.assign(d->type_mass, d->type_mass + nt);
    s.cm.resize(d->n_groups);
    for (int g = 0; g < d->n_groups; g++) {
        if (d->group_mass_center) {
            s.cm[g] = {d->group_mass_center[3 * g], d->group_mass_center[3 * g + 1], d->group_mass_center[3 * g + 2]};
        }
        else if (!s.groups[g].atomic() && s.groups[g].size() > 0) {
            // Group::updateMassCenter src/group.cpp:136-157
            const Vec3& a = s.pos[s.groups[g].begin + s.groups[g].size() / 2];
            s.cm[g] = s.massCenter(g, {-a.x, -a.y, -a.z});
        }
    }
    PairParams& P = s.pair;
    P.n_types = nt;
    P.sigma2.assign(size_t(nt) * nt, 0.0);
    P.eps4.assign(size_t(nt) * nt, 0.0);
    P.hs2.assign(size_t(nt) * nt, 0.0);
    if (d->sigma2) P.sigma2.assign(d->sigma2, d->sigma2 + size_t(nt) * nt);
    if (d->eps4) P.eps4.assign(d->eps4, d->eps4 + size_t(nt) * nt);
    if (d->hs_sigma2) P.hs2.assign(d->hs_sigma2, d->hs_sigma2 + size_t(nt) * nt);
    P.terms = d->pair_terms;
    P.coul_type = d->coulomb_type;
    P.lB = d->bjerrum_length;
    P.rc_coul = d->coulomb_cutoff;
    P.alpha = d->coulomb_alpha;
    P.pair_cutoff2 = d->pair_cutoff > 0 ? d->pair_cutoff * d->pair_cutoff : 0.0;
    if (d->coulomb_type == FAU_COUL_TRUNC) {
        P.cerfc = d->coulomb_erfc;
        P.cpoly.assign(d->coulomb_poly, d->coulomb_poly + std::max(0, std::min(d->coulomb_poly_n, FAU_COUL_MAX_POLY)));
    }
    if ((d->pair_terms & FAU_PAIR_SPLINE) && d->spline_begin && d->spline_r2 && d->spline_coef) {
        const size_t np = size_t(nt) * nt, knots = size_t(d->spline_begin[np]);
        P.spl_begin.assign(d->spline_begin, d->spline_begin + np + 1);
        P.spl_z.assign(d->spline_r2, d->spline_r2 + knots);
        P.spl_c.assign(d->spline_coef, d->spline_coef + 6 * (knots - np));
        P.spl_hs.assign(np, 0);
        if (d->spline_hs) P.spl_hs.assign(d->spline_hs, d->spline_hs + np);
    }
    else {
        P.terms &= ~FAU_PAIR_SPLINE;
    }
    if (d->cutoff_g2g > 0) s.cutoff_g2g2 = d->cutoff_g2g * d->cutoff_g2g;
    s.isobaric = d->isobaric != 0;
    s.maxenergy = d->maxenergy_set ? d->maxenergy : infty;
    s.pressure = d->pressure;
    if (d->cutoff_g2g_pairs && d->n_molids > 0) { // GroupCutoff::getCutoff per molecule-kind pair
        s.n_molids = d->n_molids;
        s.cut2_pairs.resize(size_t(d->n_molids) * d->n_molids);
        for (size_t k = 0; k < s.cut2_pairs.size(); k++) {
            const double c = d->cutoff_g2g_pairs[k];
            s.cut2_pairs[k] = (c > 0 && std::isfinite(c)) ? c * c : std::numeric_limits<double>::max();
        }
    }
    Ewald& E = s.ewald;
    E.enabled = d->ewald.enabled != 0;
    if (E.enabled) {
        E.alpha = d->ewald.alpha;
        E.ncut = d->ewald.ncutoff;
        E.spherical = d->ewald.spherical_sum != 0;
        E.epss = d->ewald.epss;
        E.const_inf = (E.epss < 1) ? 0 : 1;
        E.lB = d->bjerrum_length;
        E.updateBox(s.box);
        E.fullQ(s.pos, s.q);
    }
    return s;
}

extern "C" {

int orc_sys_create(const fau_sys_desc* d, orc_sys** out)
{
    if (!d || !out || d->n_particles < 0) return FAU_ERR_ARG;
    orc_sys* h = new orc_sys;
    h->s = buildSystem(d);
    *out = h;
    return FAU_OK;
}
int orc_sys_destroy(orc_sys* h)
{
    delete h;
    return FAU_OK;
}
int orc_energy_total(orc_sys* h, fau_energy_terms* t)
{
    Terms e = energyOf(h->s, CH_EVERYTHING, 0);
    t->self = e.self;
    t->nonbonded = e.nb;
    t->ewald_rec = e.rec;
    t->ewald_surf = e.surf;
    t->total = e.total;
    return FAU_OK;
}
static void fillTrial(const TrialOut& o, fau_trial_result* r)
{
    r->du = o.du;
    r->du_nonbonded = o.du_nb;
    r->du_ewald = o.du_ew;
    r->err_scale = o.scale;
    r->accepted = o.accepted;
    r->new_inf = o.new_inf;
    r->old_inf = o.old_inf;
    r->pad = 0;
}
int orc_trial_atomic(orc_sys* h, int i, const double dr[3], double u01, fau_trial_result* r)
{
    TrialOut o = trialAtom(h->s, i, {dr[0], dr[1], dr[2]}, u01);
    fillTrial(o, r);
    return o.nan ? FAU_ERR_NAN : FAU_OK;
}
int orc_trial_group(orc_sys* h, int g, const double dr[3], const double quat[4], double u01,
                    fau_trial_result* r)
{
    Quat q{quat[0], quat[1], quat[2], quat[3]};
    // an all-zero quaternion means "no rotation" (a rotation always has |q| = 1)
    const bool rot = !(quat[0] == 0.0 && quat[1] == 0.0 && quat[2] == 0.0 && quat[3] == 0.0);
    TrialOut o = trialGroup(h->s, g, {dr[0], dr[1], dr[2]}, rot ? &q : nullptr, u01);
    fillTrial(o, r);
    return o.nan ? FAU_ERR_NAN : FAU_OK;
}
// Apply a proposal stream (performMove per proposal).
int orc_volume_move(orc_sys* h, double new_volume, int method, double u01, fau_trial_result* r);
// one performMove of a host-fed proposal
static int orc_perform(orc_sys* h, const fau_proposal& p, fau_trial_result* r)
{
    if (p.kind == FAU_MOVE_ATOMIC) return orc_trial_atomic(h, p.index, p.dr, p.u, r);
    if (p.kind == FAU_MOVE_MOLECULAR) return orc_trial_group(h, p.index, p.dr, p.quat, p.u, r);
    if (p.kind == FAU_MOVE_VOLUME) // VolumeMove::setNewVolume (src/move.cpp:994-999)
        return orc_volume_move(h, std::exp(std::log(h->s.box.volume()) + p.dr[0]), p.index, p.u, r);
    return FAU_OK;
}
int orc_run_proposals(orc_sys* h, const fau_proposal* p, int n, uint8_t* acc_out, double* du_out,
                      fau_run_stats* st)
{
    fau_run_stats S;
    std::memset(&S, 0, sizeof(S));
    const auto t0 = std::chrono::steady_clock::now();
    for (int m = 0; m < n; m++) {
        fau_trial_result r;
        std::memset(&r, 0, sizeof(r));
        const int rc = orc_perform(h, p[m], &r);
        if (rc != FAU_OK) return rc;
        if (acc_out) acc_out[m] = (uint8_t)r.accepted;
        if (du_out) du_out[m] = r.du;
        S.moves++;
        S.accepted += r.accepted;
        if (r.accepted) S.energy_change += r.du;
    }
    S.device_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (st) *st = S;
    return FAU_OK;
}
// Same as orc_run_proposals, with every move's dU, per-term parts and
// magnitude scale (sum of |u| over both states) for tolerance checks.
int orc_run_proposals_detail(orc_sys* h, const fau_proposal* p, int n, fau_trial_result* out)
{
    for (int m = 0; m < n; m++) {
        fau_trial_result r;
        std::memset(&r, 0, sizeof(r));
        const int rc = orc_perform(h, p[m], &r);
        if (rc != FAU_OK) return rc;
        out[m] = r;
    }
    return FAU_OK;
}
int orc_get_positions(orc_sys* h, double* xyz)
{
    for (size_t i = 0; i < h->s.pos.size(); i++) {
        xyz[3 * i] = h->s.pos[i].x;
        xyz[3 * i + 1] = h->s.pos[i].y;
        xyz[3 * i + 2] = h->s.pos[i].z;
    }
    return FAU_OK;
}
int orc_get_box(orc_sys* h, double* box)
{
    box[0] = h->s.box.len.x;
    box[1] = h->s.box.len.y;
    box[2] = h->s.box.len.z;
    return FAU_OK;
}

int orc_get_mass_centers(orc_sys* h, double* xyz)
{
    for (size_t g = 0; g < h->s.cm.size(); g++) {
        xyz[3 * g] = h->s.cm[g].x;
        xyz[3 * g + 1] = h->s.cm[g].y;
        xyz[3 * g + 2] = h->s.cm[g].z;
    }
    return FAU_OK;
}
int orc_get_q(orc_sys* h, double* q)
{
    for (size_t k = 0; k < h->s.ewald.Q.size(); k++) {
        q[2 * k] = h->s.ewald.Q[k].real();
        q[2 * k + 1] = h->s.ewald.Q[k].imag();
    }
    return (int)h->s.ewald.Q.size();
}
int orc_num_kvectors(orc_sys* h) { return h->s.ewald.enabled ? (int)h->s.ewald.k.size() : 0; }
int orc_kvectors(orc_sys* h, double* kvec, double* Ak)
{
    for (size_t k = 0; k < h->s.ewald.k.size(); k++) {
        kvec[3 * k] = h->s.ewald.k[k].x;
        kvec[3 * k + 1] = h->s.ewald.k[k].y;
        kvec[3 * k + 2] = h->s.ewald.k[k].z;
        Ak[k] = h->s.ewald.Ak[k];
    }
    return (int)h->s.ewald.k.size();
}
// Energy change of a hypothetical single-atom move without committing (FP64 reference dU).
int orc_du_atomic(orc_sys* h, int i, const double dr[3], fau_trial_result* r)
{
    System copy = h->s; // cheap enough for test sizes
    TrialOut o = trialAtom(copy, i, {dr[0], dr[1], dr[2]}, 1.0);
    fillTrial(o, r);
    return FAU_OK;
}

// ---- Ewald policy energies for the known-answer tests (src/energy.cpp:249-317)
int orc_ewald_policy(int n, const double* pos, const double* q, const double box[3], double alpha,
                     double ncut, int spherical, double epss, double lB, int ipbc, double out[3], int* nk)
{
    Ewald E;
    E.enabled = true;
    E.ipbc = ipbc != 0;
    E.alpha = alpha;
    E.ncut = ncut;
    E.spherical = spherical != 0;
    E.epss = epss;
    E.const_inf = epss < 1 ? 0 : 1;
    E.lB = lB;
    Box B;
    B.set(box);
    E.updateBox(B);
    std::vector<Vec3> P(n);
    std::vector<double> Q(q, q + n);
    for (int i = 0; i < n; i++) P[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    E.fullQ(P, Q);
    out[0] = E.policySelf(B, Q);
    out[1] = E.surface(B, P, Q);
    out[2] = E.reciprocal(B);
    if (nk) *nk = (int)E.k.size();
    return FAU_OK;
}

// ---- pair energy of two particles (potential KATs)
int orc_pair_u(const fau_sys_desc* d, int ta, int tb, double qa, double qb, double r2, double* u)
{
    fau_sys_desc dd = *d;
    dd.n_particles = 0;
    dd.n_groups = 0;
    dd.ewald.enabled = 0;
    System s = buildSystem(&dd);
    *u = s.pair(ta, tb, qa, qb, r2);
    return FAU_OK;
}

// ---- Chameleon cuboid geometry (consistency KAT, src/geometry.cpp:1320-1371): per point
// pair, a wrapped by boundary(), vdist(a, b) and sqdist(a, b)
int orc_geometry(const double box[3], int n, const double* a, const double* b, double* a_wrapped, double* vd,
                 double* sq)
{
    Box B;
    B.set(box);
    for (int i = 0; i < n; i++) {
        Vec3 p{a[3 * i], a[3 * i + 1], a[3 * i + 2]}, q{b[3 * i], b[3 * i + 1], b[3 * i + 2]};
        const Vec3 d = B.vdist(p, q);
        sq[i] = B.sqdist(p, q);
        B.boundary(p);
        for (int k = 0; k < 3; k++) {
            a_wrapped[3 * i + k] = p[k];
            vd[3 * i + k] = d[k];
        }
    }
    return FAU_OK;
}

// ---- VolumeMove + Isobaric + Metropolis (src/move.cpp:994-1006, src/energy.cpp:884-901,
// src/montecarlo.cpp:139-187); the box scaled as Cuboid::setVolume (src/geometry.cpp:57-90) and
// the particles as Space::scaleVolume (src/space.cpp:249-301); the trial state's Ewald gets
// updateBox + a full Q update (Ewald::updateState with volume_change)
int orc_volume_move(orc_sys* h, double new_volume, int method, double u01, fau_trial_result* r)
{
    System& s = h->s;
    const double pressure = s.pressure;
    const Terms eo = energyOf(s, CH_EVERYTHING, 0);
    System t = s;
    const double v_old = s.box.volume();
    Vec3 sc{1, 1, 1};
    if (method == FAU_VOLUME_ISOTROPIC) {
        const double a = std::cbrt(new_volume / v_old);
        sc = {a, a, a};
    }
    else if (method == FAU_VOLUME_XY) {
        const double a = std::sqrt(new_volume / v_old);
        sc = {a, a, 1.0};
    }
    else if (method == FAU_VOLUME_Z) {
        sc = {1.0, 1.0, new_volume / v_old};
    }
    else {
        const double a = std::cbrt(new_volume / v_old);
        sc = {a, a, 1 / (a * a)};
    }
    const double Ln[3] = {s.box.len.x * sc.x, s.box.len.y * sc.y, s.box.len.z * sc.z};
    t.box.set(Ln);
    int n_count = 0;
    for (size_t g = 0; g < s.groups.size(); g++) {
        const Group& G = s.groups[g];
        if (G.size() == 0) continue;
        if (G.atomic()) {
            n_count += G.size();
            for (int i = G.begin; i < G.end; i++) {
                Vec3 p{s.pos[i].x * sc.x, s.pos[i].y * sc.y, s.pos[i].z * sc.z};
                t.box.boundary(p);
                t.pos[i] = p;
            }
        }
        else {
            n_count += 1;
            const Vec3 c0 = s.cm[g];
            Vec3 c{c0.x * sc.x, c0.y * sc.y, c0.z * sc.z};
            t.box.boundary(c);
            t.cm[g] = c;
            const Vec3 dc{c.x - c0.x, c.y - c0.y, c.z - c0.z};
            for (int i = G.begin; i < G.end; i++) {
                const Vec3 d = s.box.vdist(s.pos[i], c0); // Group::unwrap (src/group.h:349-356)
                Vec3 p{c0.x + d.x, c0.y + d.y, c0.z + d.z};
                p = {p.x + dc.x, p.y + dc.y, p.z + dc.z};
                t.box.boundary(p);
                t.pos[i] = p;
            }
        }
    }
    if (t.ewald.enabled) {
        t.ewald.updateBox(t.box);
        t.ewald.fullQ(t.pos, t.q);
    }
    const Terms en = energyOf(t, CH_EVERYTHING, 0);
    const double v_new = t.box.volume();
    auto total = [&](const Terms& e, double v) { // Isobaric first, then the Hamiltonian's terms
        std::vector<double> list;
        if (s.isobaric) list.push_back(pressure * v - double(n_count + 1) * std::log(v));
        if (s.pair.has_self()) list.push_back(e.self);
        list.push_back(e.nb);
        if (s.ewald.enabled) list.push_back(e.surf + e.rec);
        return accumulateTerms(list.data(), (int)list.size(), s.maxenergy);
    };
    const double uo = total(eo, v_old), un = total(en, v_new);
    const double du = getEnergyChange(un, uo);
    const int acc = metropolis(du, u01);
    if (acc < 0) return FAU_ERR_NAN;
    if (r) {
        r->du = du;
        r->du_nonbonded = en.nb - eo.nb;
        r->du_ewald = (en.rec + en.surf) - (eo.rec + eo.surf);
        r->err_scale = std::fabs(un) + std::fabs(uo);
        r->accepted = acc;
        r->new_inf = un >= infty;
        r->old_inf = uo >= infty;
        r->pad = 0;
    }
    if (acc) {
        t.sum_of_energy_changes += du;
        s = std::move(t);
    }
    return FAU_OK;
}

// ---- AtomRDF histogram (src/analysis.cpp:1556-1600): pairs of atoms of types a and b
// (i < j when a == b, AtomRDF::sampleIdentical), r = |vdist| (Chameleon, cuboid), bin
// floor(r * (1/dr)) as Equidistant2DTable::to_bin (src/aux/equidistant_table.h:32-39);
// bins >= n_bins are counted in hist[n_bins]
int orc_rdf(int n, const double* pos, const int* type, const double box[3], int ta, int tb, double dr, int n_bins,
            uint64_t* hist)
{
    Box B;
    B.set(box);
    const double dxinv = 1.0 / dr;
    auto sample = [&](int i, int j) {
        const Vec3 a{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}, b{pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]};
        const double r = std::sqrt(sqnorm(B.vdist(a, b)));
        const long long bin = (long long)std::floor(r * dxinv);
        hist[bin < n_bins ? bin : n_bins]++;
    };
    for (int i = 0; i < n; i++) {
        if (type[i] != ta) continue;
        if (ta == tb) {
            for (int j = i + 1; j < n; j++)
                if (type[j] == ta) sample(i, j);
        }
        else {
            for (int j = 0; j < n; j++)
                if (type[j] == tb) sample(i, j);
        }
    }
    return FAU_OK;
}

// ---- cell grid binning (bit-exact oracle for the device cell list)
int orc_cell_bin(const double box[3], double min_cell, int n, const double* pos, int* cells_out, int dims_out[3],
                 int offmin_out[3], int offmax_out[3])
{
    int dims[3];
    double cell[3];
    cellGrid(box, min_cell, dims, cell);
    for (int i = 0; i < n; i++)
        cells_out[i] = cellIndexAt(box, dims, cell, {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]});
    for (int d = 0; d < 3; d++) {
        dims_out[d] = dims[d];
        // distance-1 neighbour offsets (GridOffsets3D src/celllistimpl.cpp:15-31) clamped by the
        // wrap-around limits of PeriodicBoundaryGrid (src/celllistimpl.h:409-415)
        const double mid = (dims[d] - 1) * 0.5;
        offmin_out[d] = std::max(-1, -(int)std::floor(mid));
        offmax_out[d] = std::min(1, (int)std::ceil(mid));
    }
    return FAU_OK;
}

// ---- move generation and full Metropolis loop with the oracle's own RNG
int orc_movegen_create(orc_sys* h, const fau_move_desc* moves, int n_moves, uint32_t slump_seed, uint32_t random_seed,
                       int default_seeds, orc_movegen** out)
{
    orc_movegen* g = new orc_movegen;
    if (!default_seeds) {
        g->g.slump.engine.seed(slump_seed);
        g->g.random.engine.seed(random_seed);
    }
    std::vector<double> w;
    for (int m = 0; m < n_moves; m++) {
        MoveDef md;
        md.kind = moves[m].kind;
        md.repeat = moves[m].repeat;
        md.dp = moves[m].dp;
        md.dprot = moves[m].dprot;
        md.dir = {moves[m].dir[0], moves[m].dir[1], moves[m].dir[2]};
        md.volume_method = moves[m].volume_method;
        if (moves[m].groups) md.groups.assign(moves[m].groups, moves[m].groups + moves[m].n_groups);
        const int nt = h->s.pair.n_types;
        if (moves[m].type_dp) md.type_dp.assign(moves[m].type_dp, moves[m].type_dp + nt);
        if (moves[m].type_dprot) md.type_dprot.assign(moves[m].type_dprot, moves[m].type_dprot + nt);
        g->g.moves.push_back(md);
        w.push_back(md.repeat);
    }
    g->g.dist = std::discrete_distribution<unsigned int>(w.begin(), w.end());
    g->g.sys = &h->s;
    *out = g;
    return FAU_OK;
}
int orc_movegen_destroy(orc_movegen* g)
{
    delete g;
    return FAU_OK;
}
int orc_movegen_generate(orc_movegen* g, fau_proposal* out, int n)
{
    for (int i = 0; i < n; i++) out[i] = g->g.next();
    return FAU_OK;
}
// Full reference loop: draw a proposal and perform it, n times.
int orc_mc_run(orc_sys* h, orc_movegen* g, int n, uint8_t* acc_out, double* du_out, fau_run_stats* st)
{
    fau_run_stats S;
    std::memset(&S, 0, sizeof(S));
    const auto t0 = std::chrono::steady_clock::now();
    for (int m = 0; m < n; m++) {
        fau_proposal p = g->g.next();
        int rc = orc_run_proposals(h, &p, 1, acc_out ? acc_out + m : nullptr, du_out ? du_out + m : nullptr, nullptr);
        if (rc != FAU_OK) return rc;
        if (p.kind != FAU_MOVE_NONE) S.moves++;
    }
    S.device_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (st) *st = S;
    return FAU_OK;
}

// ---- CPU baseline: `n_chains` independent chains of the same system on
// `n_threads` host threads, each advancing `moves` proposals from its own
// generator (seeded chain index).  Returns total moves / wall second.
int orc_bench_chains(const fau_sys_desc* d, const fau_move_desc* moves, int n_moves, int n_chains, int n_threads,
                     int moves_per_chain, double* moves_per_sec, double* wall_s)
{
    std::vector<orc_sys*> sys(n_chains);
    std::vector<orc_movegen*> gen(n_chains);
    { // set-up (full Q(k) of every chain) in parallel, outside the timed region
        std::vector<std::thread> mk;
        for (int t = 0; t < n_threads; t++)
            mk.emplace_back([&, t]() {
                for (int c = t; c < n_chains; c += n_threads) {
                    orc_sys_create(d, &sys[c]);
                    sys[c]->s.want_scale = false;
                    orc_movegen_create(sys[c], moves, n_moves, 1000u + c, 2000u + c, 0, &gen[c]);
                }
            });
        for (auto& x : mk) x.join();
    }
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> th;
    std::vector<int> rcs(n_threads, FAU_OK);
    for (int t = 0; t < n_threads; t++) {
        th.emplace_back([&, t]() {
            for (int c = t; c < n_chains; c += n_threads) {
                int rc = orc_mc_run(sys[c], gen[c], moves_per_chain, nullptr, nullptr, nullptr);
                if (rc != FAU_OK) rcs[t] = rc;
            }
        });
    }
    for (auto& x : th) x.join();
    const double w = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (int c = 0; c < n_chains; c++) {
        orc_movegen_destroy(gen[c]);
        orc_sys_destroy(sys[c]);
    }
    *wall_s = w;
    *moves_per_sec = double(n_chains) * moves_per_chain / w;
    for (int rc : rcs)
        if (rc != FAU_OK) return rc;
    return FAU_OK;
}

// ---- RNG determinism KAT helpers (src/random.cpp:65-101)
double orc_random_default_first(void)
{
    Random r;
    return r();
}
int orc_random_state(uint32_t seed, int default_seed, char* buf, size_t len)
{
    Random r;
    if (!default_seed) r.engine.seed(seed);
    std::ostringstream os;
    os << r.engine;
    std::snprintf(buf, len, "%s", os.str().c_str());
    return (int)os.str().size();
}

} // extern "C"
