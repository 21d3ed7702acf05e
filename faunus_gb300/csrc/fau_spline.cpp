// fau_spline.cpp -- host-side tables of splined pair potentials (nonbonded_splined).
//
// Tabulate::Andrea::generate (src/tabulate.h:212-298) splines f(z), z = r^2, from zmax down to
// zmin in pieces: each piece is the quintic in (z - z_low) that matches f, f' and f'' at both
// of its ends (SetUBuffer, :106-136), the derivatives taken by central differences of step
// 1e-4 (TabulatorBase::f1/f2, :34-44). A piece is accepted when 11 points evenly spaced in r
// keep the spline within utol of f (and its slope within ftol of f'), else its length in r is
// cut by 0.9, at most 100 times (CheckUBuffer, :142-178). SplinedPotential
// (src/potentials.cpp:1453-1597) chooses [rmin, rmax] per atom-type pair from the functor and
// keeps hard-sphere repulsion only for pairs that are repulsive at the inner end.
//
// The tables are made once per system on the host; the device evaluates them (fau_dev.cuh
// spline_u32 / spline_u64). Compiled without FMA contraction, as the reference's arithmetic.
#include "../../include/fau_gpu.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

extern "C" int fau_internal_fail(int code, const char* msg);

namespace {

constexpr int kMaxPieces = 1200;   // Andrea::mngrid
constexpr int kMaxShrinks = 100;   // Andrea::ndr
constexpr double kShrink = 0.9;    // Andrea::drfrac
constexpr double kNumDr = 0.0001;  // TabulatorBase::numdr
constexpr double kSearchDr = 1e-2; // SplinedPotential::dr
constexpr int kSearchMax = 1000000;

struct Fn {
    fau_scalar_fn f;
    void* ctx;
    double operator()(double z) const { return f(z, ctx); }
    double d1(double z) const { return ((*this)(z + kNumDr * 0.5) - (*this)(z - kNumDr * 0.5)) / kNumDr; }
    double d2(double z) const { return (d1(z + kNumDr * 0.5) - d1(z - kNumDr * 0.5)) / kNumDr; }
};

// Coefficients c_0..c_5 of the quintic on [zl, zu] with the given value, slope and curvature
// at both ends; a piece where f and f' vanish at the lower end is all zero.
void quintic(double zl, double zu, double v0, double v1, double v2, double w0, double w1, double w2, double c[6])
{
    if (std::fabs(v0) < 1e-9 && std::fabs(v1) < 1e-9) {
        for (int k = 0; k < 6; k++) c[k] = 0.0;
        return;
    }
    const double h = zu - zl, h2 = h * h, h3 = h2 * h;
    c[0] = v0;
    c[1] = v1;
    c[2] = v2 * 0.5;
    // the remaining three from the upper end's value, slope and curvature
    const double a = 6 * (w0 - c[0] - c[1] * h - c[2] * h2) / h3;
    const double b = 2 * (w1 - c[1] - 2 * c[2] * h) / h2;
    const double g = (w2 - 2 * c[2]) / h;
    c[3] = (10 * a - 12 * b + 3 * g) / 6;
    c[4] = (-15 * a + 21 * b - 6 * g) / (6 * h);
    c[5] = (2 * a - 3 * b + g) / (2 * h2);
}

bool within_tolerance(const Fn& f, const double c[6], double rl, double ru, double utol, double ftol)
{
    const int n = 11;
    const double step = (ru - rl) / (n - 1);
    for (int i = 0; i < n; i++) {
        const double r = rl + step * ((double)i);
        const double z = r * r;
        const double dz = z - rl * rl;
        const double u = c[0] + dz * (c[1] + dz * (c[2] + dz * (c[3] + dz * (c[4] + dz * c[5]))));
        if (std::fabs(u - f(z)) > utol) return false;
        if (ftol > 0) {
            const double s = c[1] + dz * (2 * c[2] + dz * (3 * c[3] + dz * (4 * c[4] + dz * (5 * c[5]))));
            if (std::fabs(s - f.d1(z)) > ftol) return false;
        }
    }
    return true;
}

// pieces from zmax down to zmin; knots come out descending with their coefficient packets
int generate(const Fn& f, double zmin, double zmax, double utol, double ftol, std::vector<double>& knots,
             std::vector<double>& coef)
{
    const double rmin = std::sqrt(zmin), rmax = std::sqrt(zmax);
    knots.assign(1, rmax * rmax);
    coef.clear();
    double rupp = rmax;
    int piece = 0;
    for (; piece < kMaxPieces; piece++) {
        double dr = rupp - rmin;
        double rlow = rupp, zlow = 0.0, c[6];
        bool ok = false;
        for (int t = 0; t < kMaxShrinks; t++) {
            const double zupp = rupp * rupp;
            rlow = std::max(rupp - dr, rmin);
            zlow = rlow * rlow;
            quintic(zlow, zupp, f(zlow), f.d1(zlow), f.d2(zlow), f(zupp), f.d1(zupp), f.d2(zupp), c);
            if (within_tolerance(f, c, rlow, rupp, utol, ftol)) {
                rupp = rlow;
                ok = true;
                break;
            }
            dr *= kShrink;
        }
        if (!ok) return fau_internal_fail(FAU_ERR_ARG, "Andrea spline: no piece meets the tolerance (increase utol/ftol)");
        knots.push_back(zlow);
        coef.insert(coef.end(), c, c + 6);
        if (rlow <= rmin) break;
    }
    if (piece >= kMaxPieces) return fau_internal_fail(FAU_ERR_ARG, "Andrea spline: more than 1200 pieces (increase utol/ftol)");
    return FAU_OK;
}

// Andrea::eval on ascending knots: the piece z_i < z <= z_{i+1}
double eval(const std::vector<double>& knots, const std::vector<double>& coef, double z)
{
    long i = (long)(std::lower_bound(knots.begin(), knots.end(), z) - knots.begin()) - 1;
    i = std::min(std::max(i, 0L), (long)knots.size() - 2); // z outside (z_0, z_m]: the end piece
    const double* c = coef.data() + 6 * i;
    const double dz = z - knots[i];
    double s = 0;
    for (int k = 5; k > 0; k--) s = dz * (s + c[k]);
    return s + c[0];
}

int write_out(std::vector<double>& knots, std::vector<double>& coef, int cap, double* r2_out, double* coef_out,
              int* n_knots)
{
    const int m = (int)knots.size();
    if (m > cap) return fau_internal_fail(FAU_ERR_ARG, "spline table larger than the output capacity");
    // ascending: knots reversed, coefficient packets reversed as wholes
    for (int i = 0; i < m; i++) r2_out[i] = knots[m - 1 - i];
    const int p = m - 1;
    for (int i = 0; i < p; i++)
        for (int k = 0; k < 6; k++) coef_out[6 * i + k] = coef[6 * (p - 1 - i) + k];
    *n_knots = m;
    return FAU_OK;
}

// the functor of one atom-type pair: the desc's terms in FP64, as the exact evaluation
struct PairFn {
    const fau_sys_desc* d;
    int ab;
    double qq; // lB qa qb
    double value(double r2) const
    {
        const int t = d->pair_terms;
        double u = 0.0;
        if (t & FAU_PAIR_COULOMB) {
            if (d->coulomb_type == FAU_COUL_PLAIN) {
                u += qq / std::sqrt(r2);
            }
            else { // NewCoulombGalore: r + epsilon, S(q), zero at and beyond Rc
                const double r = std::sqrt(r2) + std::numeric_limits<double>::epsilon();
                if (r < d->coulomb_cutoff) {
                    double s = 1.0;
                    if (d->coulomb_type == FAU_COUL_EWALD) {
                        s = std::erfc(d->coulomb_alpha * r);
                    }
                    else if (d->coulomb_type == FAU_COUL_TRUNC) {
                        const double q = r / d->coulomb_cutoff;
                        s = 0.0;
                        for (int k = d->coulomb_poly_n - 1; k >= 0; k--) s = s * q + d->coulomb_poly[k];
                        if (d->coulomb_erfc != 0.0) s += d->coulomb_erfc * std::erfc(d->coulomb_alpha * r);
                    }
                    u += qq / r * s;
                }
            }
        }
        if (t & (FAU_PAIR_LJ | FAU_PAIR_WCA)) {
            const double s2 = d->sigma2[ab], e4 = d->eps4[ab];
            if (t & FAU_PAIR_LJ) {
                double x = s2 / r2;
                x = x * x * x;
                u += e4 * (x * x - x);
            }
            if ((t & FAU_PAIR_WCA) && !(r2 > s2 * 1.2599210498948732)) {
                double x = s2 / r2;
                x = x * x * x;
                u += e4 * (x * x - x + 0.25);
            }
        }
        if ((t & FAU_PAIR_HS) && r2 < d->hs_sigma2[ab]) u += std::numeric_limits<double>::infinity();
        return u;
    }
    static double call(double z, void* ctx) { return static_cast<const PairFn*>(ctx)->value(z); }
};

} // namespace

extern "C" {

int fau_andrea_generate(fau_scalar_fn f, void* ctx, double zmin, double zmax, double utol, double ftol, int cap,
                        double* r2_out, double* coef_out, int* n_knots)
{
    if (!f || !r2_out || !coef_out || !n_knots || cap < 2) return fau_internal_fail(FAU_ERR_ARG, "invalid spline arguments");
    if (!(zmin >= 0.0) || !(zmax > zmin) || !(utol > 0.0) || !std::isfinite(zmax))
        return fau_internal_fail(FAU_ERR_ARG, "spline needs 0 <= zmin < zmax and utol > 0");
    std::vector<double> knots, coef;
    const Fn fn{f, ctx};
    int rc = generate(fn, zmin, zmax, utol, ftol, knots, coef);
    if (rc) return rc;
    return write_out(knots, coef, cap, r2_out, coef_out, n_knots);
}

int fau_spline_tabulate(const fau_sys_desc* d, int type_a, int type_b, double charge_a, double charge_b,
                        double rmin_start, const fau_spline_opts* o, int cap, double* r2_out, double* coef_out,
                        int* n_knots, int* hs_out)
{
    if (!d || !o || !r2_out || !coef_out || !n_knots || !hs_out || cap < 2)
        return fau_internal_fail(FAU_ERR_ARG, "invalid spline arguments");
    if (type_a < 0 || type_b < 0 || type_a >= d->n_types || type_b >= d->n_types)
        return fau_internal_fail(FAU_ERR_ARG, "spline atom type out of range");
    if ((d->pair_terms & (FAU_PAIR_LJ | FAU_PAIR_WCA)) && (!d->sigma2 || !d->eps4))
        return fau_internal_fail(FAU_ERR_ARG, "LJ/WCA need sigma2 and eps4 tables");
    if ((d->pair_terms & FAU_PAIR_HS) && !d->hs_sigma2) return fau_internal_fail(FAU_ERR_ARG, "HS needs hs_sigma2");
    if (d->coulomb_type != FAU_COUL_PLAIN && (d->pair_terms & FAU_PAIR_COULOMB) && !(d->coulomb_cutoff > 0.0))
        return fau_internal_fail(FAU_ERR_ARG, "a cut Coulomb scheme needs a positive coulomb_cutoff");
    if (!(rmin_start > 0.0) || !(o->utol > 0.0) || !(o->u_at_rmin > 0.0) || !(o->u_at_rmax > 0.0))
        return fau_internal_fail(FAU_ERR_ARG, "spline needs rmin_start, utol, u_at_rmin and u_at_rmax > 0");
    const PairFn pf{d, type_a * d->n_types + type_b, d->bjerrum_length * charge_a * charge_b};
    const Fn f{&PairFn::call, const_cast<PairFn*>(&pf)};

    double rmin = rmin_start, rmax = o->rmax_start > 0.0 ? o->rmax_start : rmin_start * 10;
    // findLowerDistance: step rmin until |f| lies within 10 % of u_at_rmin
    for (int it = 0; rmin >= kSearchDr; it++) {
        if (it == kSearchMax) return fau_internal_fail(FAU_ERR_ARG, "pair potential spline: cannot determine rmin");
        const double u = std::fabs(f(rmin * rmin));
        if (u > o->u_at_rmin * 1.1) rmin += kSearchDr;
        else if (u < o->u_at_rmin / 1.1) rmin -= kSearchDr;
        else break;
    }
    // findUpperDistance: move rmax out until |f| <= u_at_rmax
    for (int it = 0; rmax >= kSearchDr; it++) {
        if (it == kSearchMax) return fau_internal_fail(FAU_ERR_ARG, "pair potential spline: cannot determine rmax");
        if (std::fabs(f(rmax * rmax)) > o->u_at_rmax) rmax += kSearchDr;
        else break;
    }
    if (!(rmin > 0.0) || !(rmin < rmax)) return fau_internal_fail(FAU_ERR_ARG, "pair potential spline: rmin >= rmax");
    std::vector<double> knots, coef;
    int rc = generate(f, rmin * rmin, rmax * rmax, o->utol, o->ftol, knots, coef);
    if (rc) return rc;
    rc = write_out(knots, coef, cap, r2_out, coef_out, n_knots);
    if (rc) return rc;
    // hard-sphere repulsion only where the spline is repulsive just above the first knot
    std::vector<double> zk(r2_out, r2_out + *n_knots), ck(coef_out, coef_out + 6 * (*n_knots - 1));
    *hs_out = (o->hardsphere && !(eval(zk, ck, zk[0] + kSearchDr) < 0)) ? 1 : 0;
    return FAU_OK;
}

} // extern "C"
