// pmgb_setup.cu -- host-side set-up of a system from its unit cell, natively: the replication
// factors for the cutoff, the replicated supercell, and the Ewald parameters, so that a screening
// loop or a drop-in call pays microseconds instead of interpreter time per framework.
//
//   replication_factors   src/forcefield.jl:120-158
//   replicate             Xtals.replicate, as called at src/henry.jl:86
//   setup_Ewald_sum       src/electrostatics.jl:256-272 -> determine_ewald_params (:123-141),
//                         required_kreps (:157-175), precompute_kvec_wts (:198-232)
//
// The two precision conditions of determine_ewald_params are solved by bisection on the
// reference's brackets ([0, 25] for alpha, [0, 100] for |k|^2_max) to machine precision, as a
// bracketing fzero converges.
#include "pmgb.h"
#include "pmgb_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

namespace {

// ε₀ in e²/(Å K) (src/electrostatics.jl:6)
double eps0() { return 8.854187817e-12 / (1.602176565e-19 * 1.602176565e-19) / 1.0e10 * 1.3806488e-23; }

// bisection of f on [lo, hi] (f(lo) and f(hi) of opposite signs) until the midpoint stops moving
template <class F>
double bisect(F f, double lo, double hi) {
    double flo = f(lo);
    for (int it = 0; it < 2000; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        const double fm = f(mid);
        if (fm == 0.0) return mid;
        if ((fm > 0.0) == (flo > 0.0)) {
            lo = mid;
            flo = fm;
        } else {
            hi = mid;
        }
    }
    return 0.5 * (lo + hi);
}

// 3x3 column-major helpers: m[i + 3j] = M(i, j)
double det3(const double m[9]) {
    return m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) +
           m[6] * (m[1] * m[5] - m[4] * m[2]);
}

// reciprocal lattice 2 pi inv(f_to_c); row i (rec[i][.]) is the i-th reciprocal vector
bool reciprocal(const double f[9], double rec[3][3]) {
    const double d = det3(f);
    if (!(std::fabs(d) > 0.0) || !std::isfinite(d)) return false;
    // inverse by cofactors: inv(i, j) = cof(j, i) / det
    const double c[3][3] = {{f[4] * f[8] - f[7] * f[5], -(f[1] * f[8] - f[7] * f[2]), f[1] * f[5] - f[4] * f[2]},
                            {-(f[3] * f[8] - f[6] * f[5]), f[0] * f[8] - f[6] * f[2], -(f[0] * f[5] - f[3] * f[2])},
                            {f[3] * f[7] - f[6] * f[4], -(f[0] * f[7] - f[6] * f[1]), f[0] * f[4] - f[3] * f[1]}};
    // c[j][i] is the cofactor of element (i, j) of f
    const double two_pi = 2.0 * M_PI;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) rec[i][j] = two_pi * c[j][i] / d;
    return true;
}

}  // namespace

extern "C" int pmgb_replication_factors(const double f_to_c[9], double r_cutoff, int32_t rep_out[3]) {
    if (!f_to_c || !rep_out || !(r_cutoff > 0.0) || !std::isfinite(r_cutoff)) return PMGB_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 9; ++i)
        if (!std::isfinite(f_to_c[i])) return PMGB_ERR_INVALID_ARGUMENT;
    if (!(std::fabs(det3(f_to_c)) > 0.0)) return PMGB_ERR_INVALID_ARGUMENT;
    const double* f = f_to_c;
    double a[3] = {f[0], f[1], f[2]}, b[3] = {f[3], f[4], f[5]}, c[3] = {f[6], f[7], f[8]};
    auto cross = [](const double* u, const double* v, double* w) {
        w[0] = u[1] * v[2] - u[2] * v[1];
        w[1] = u[2] * v[0] - u[0] * v[2];
        w[2] = u[0] * v[1] - u[1] * v[0];
    };
    // face normals of the unit cell (they do not change as the cell grows along its own vectors)
    double n_ab[3], n_ac[3], n_bc[3];
    cross(a, b, n_ab);
    cross(a, c, n_ac);
    cross(b, c, n_bc);
    auto norm = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); };
    // distance from the centre of the supercell to the face with normal n
    auto half_width = [&](const double* n) {
        const double ctr[3] = {0.5 * a[0] + 0.5 * b[0] + 0.5 * c[0], 0.5 * a[1] + 0.5 * b[1] + 0.5 * c[1],
                               0.5 * a[2] + 0.5 * b[2] + 0.5 * c[2]};
        return std::fabs(n[0] * ctr[0] + n[1] * ctr[1] + n[2] * ctr[2]) / norm(n);
    };
    int rep[3] = {1, 1, 1};
    const int cap = 1 << 20;  // a degenerate cell must not loop forever
    while (half_width(n_bc) < r_cutoff && rep[0] < cap) {
        ++rep[0];
        for (int d = 0; d < 3; ++d) a[d] += f[d];
    }
    while (half_width(n_ac) < r_cutoff && rep[1] < cap) {
        ++rep[1];
        for (int d = 0; d < 3; ++d) b[d] += f[3 + d];
    }
    while (half_width(n_ab) < r_cutoff && rep[2] < cap) {
        ++rep[2];
        for (int d = 0; d < 3; ++d) c[d] += f[6 + d];
    }
    if (rep[0] >= cap || rep[1] >= cap || rep[2] >= cap) return PMGB_ERR_INVALID_ARGUMENT;
    for (int d = 0; d < 3; ++d) rep_out[d] = rep[d];
    return PMGB_OK;
}

// setup_Ewald_sum for the box f_to_c: alpha, |k|^2_max, kreps and, when abc/wt are given, the
// k-vectors with their weights appended in the reference's order; n_k receives their count.
int pmgb_ewald_kvectors(const double f_to_c[9], double sr_cutoff, double precision, double* alpha_out,
                        double* max_k2_out, int32_t kreps_out[3], std::vector<int32_t>* abc, std::vector<double>* wt,
                        int64_t* n_k_out) {
    if (!f_to_c || !(sr_cutoff > 0.0) || !std::isfinite(sr_cutoff) || !(precision > 0.0) || !(precision < 1.0))
        return PMGB_ERR_INVALID_ARGUMENT;
    double rec[3][3];
    if (!reciprocal(f_to_c, rec)) return PMGB_ERR_INVALID_ARGUMENT;
    // determine_ewald_params
    const double alpha = bisect([&](double a) { return std::erfc(sr_cutoff * a) / sr_cutoff - precision; }, 0.0, 25.0);
    const double max_k2 = bisect(
        [&](double k2) {
            if (k2 == 0.0) return std::numeric_limits<double>::infinity();
            return 2.0 * std::exp(-k2 / (4.0 * alpha * alpha)) / k2 - precision;
        },
        0.0, 100.0);
    // required_kreps: the largest multiple of each reciprocal vector with |n b_i|^2 <= max_k2
    int kreps[3];
    for (int i = 0; i < 3; ++i) {
        int n = 0;
        for (;;) {
            ++n;
            const double kx = rec[i][0] * n, ky = rec[i][1] * n, kz = rec[i][2] * n;
            if (kx * kx + ky * ky + kz * kz > max_k2) break;
            if (n > (1 << 20)) return PMGB_ERR_INVALID_ARGUMENT;
        }
        kreps[i] = n - 1;
    }
    // precompute_kvec_wts: one of each +-k pair (ka >= 0, with the tie rules at ka = 0 and
    // ka = kb = 0), |k|^2 < max_k2, weight 2 exp(-k^2 / 4 alpha^2) / k^2 / eps0 / Omega
    const double omega = std::fabs(det3(f_to_c));
    const double e0 = eps0();
    int64_t n_k = 0;
    for (int ka = 0; ka <= kreps[0]; ++ka)
        for (int kb = -kreps[1]; kb <= kreps[1]; ++kb)
            for (int kc = -kreps[2]; kc <= kreps[2]; ++kc) {
                if (ka == 0 && kb == 0 && kc == 0) continue;
                if (ka == 0 && kb < 0) continue;
                if (ka == 0 && kb == 0 && kc < 0) continue;
                double k[3];
                for (int d = 0; d < 3; ++d) k[d] = ka * rec[0][d] + kb * rec[1][d] + kc * rec[2][d];
                const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
                if (!(k2 < max_k2)) continue;
                if (abc) abc->insert(abc->end(), {ka, kb, kc});
                if (wt) wt->push_back(2.0 * std::exp(-k2 / (4.0 * alpha * alpha)) / k2 / e0 / omega);
                ++n_k;
            }
    if (alpha_out) *alpha_out = alpha;
    if (max_k2_out) *max_k2_out = max_k2;
    if (kreps_out)
        for (int d = 0; d < 3; ++d) kreps_out[d] = kreps[d];
    if (n_k_out) *n_k_out = n_k;
    return PMGB_OK;
}

extern "C" int pmgb_ewald_setup(const double f_to_c[9], double sr_cutoff, double precision, int64_t capacity,
                                double* alpha_out, double* max_k2_out, int32_t kreps_out[3], int64_t* n_kvecs_out,
                                int32_t* kvec_abc, double* kvec_wt) {
    if (!n_kvecs_out || capacity < 0 || (capacity > 0 && (!kvec_abc || !kvec_wt))) return PMGB_ERR_INVALID_ARGUMENT;
    std::vector<int32_t> abc;
    std::vector<double> wt;
    int64_t n_k = 0;
    const int rc = pmgb_ewald_kvectors(f_to_c, sr_cutoff, precision, alpha_out, max_k2_out, kreps_out,
                                       capacity > 0 ? &abc : nullptr, capacity > 0 ? &wt : nullptr, &n_k);
    if (rc != PMGB_OK) return rc;
    *n_kvecs_out = n_k;
    if (capacity > 0 && n_k > capacity) return PMGB_ERR_INVALID_ARGUMENT;
    if (capacity > 0) {
        std::copy(abc.begin(), abc.end(), kvec_abc);
        std::copy(wt.begin(), wt.end(), kvec_wt);
    }
    return PMGB_OK;
}

// The supercell of henry_coefficient's set-up (src/henry.jl:78-86): replication factors for
// r_cutoff and the replicated arrays -- images (i, j, k) with k fastest, each holding every atom
// in order, fractional coordinates rescaled into the supercell, (x + shift) / rep
// (Xtals.replicate).  why names a failure.
int pmgb_make_supercell(const double f_to_c[9], double r_cutoff, int32_t n_atoms, const double* atom_xf,
                        const int32_t* atom_species, int32_t n_charges, const double* charge_xf,
                        const double* charge_q, PmgbSupercell& sc, const char** why) {
    *why = "bad arguments";
    if (!f_to_c || n_atoms < 0 || n_charges < 0 || (n_atoms > 0 && (!atom_xf || !atom_species)) ||
        (n_charges > 0 && (!charge_xf || !charge_q)))
        return PMGB_ERR_INVALID_ARGUMENT;
    int32_t* rep = sc.rep;
    if (pmgb_replication_factors(f_to_c, r_cutoff, rep) != PMGB_OK) {
        *why = "the box must be finite and non-singular and the cutoff positive";
        return PMGB_ERR_INVALID_ARGUMENT;
    }
    const int64_t n_img = int64_t(rep[0]) * rep[1] * rep[2];
    if (n_img * std::max(n_atoms, n_charges) > INT32_MAX) {
        *why = "supercell too large";
        return PMGB_ERR_INVALID_ARGUMENT;
    }
    auto replicate = [&](int32_t n, const double* xf, std::vector<double>& out_xf) {
        out_xf.resize(static_cast<size_t>(3 * n * n_img));
        size_t w = 0;
        for (int i = 0; i < rep[0]; ++i)
            for (int j = 0; j < rep[1]; ++j)
                for (int k = 0; k < rep[2]; ++k)
                    for (int32_t a = 0; a < n; ++a) {
                        out_xf[w++] = (xf[3 * a + 0] + i) / rep[0];
                        out_xf[w++] = (xf[3 * a + 1] + j) / rep[1];
                        out_xf[w++] = (xf[3 * a + 2] + k) / rep[2];
                    }
    };
    replicate(n_atoms, atom_xf, sc.atom_xf);
    replicate(n_charges, charge_xf, sc.charge_xf);
    sc.atom_species.clear();
    sc.charge_q.clear();
    sc.atom_species.reserve(static_cast<size_t>(n_atoms * n_img));
    sc.charge_q.reserve(static_cast<size_t>(n_charges * n_img));
    for (int64_t m = 0; m < n_img; ++m) {
        sc.atom_species.insert(sc.atom_species.end(), atom_species, atom_species + n_atoms);
        sc.charge_q.insert(sc.charge_q.end(), charge_q, charge_q + n_charges);
    }
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) sc.f_to_c[i + 3 * j] = f_to_c[i + 3 * j] * rep[j];
    return PMGB_OK;
}

extern "C" int pmgb_system_create_unitcell(pmgb_ctx* ctx, const double f_to_c[9], int32_t n_atoms,
                                           const double* atom_xf, const int32_t* atom_species, int32_t n_charges,
                                           const double* charge_xf, const double* charge_q, int32_t n_species,
                                           const double* epsilon, const double* sigma2, double r_cutoff,
                                           int32_t n_guest_atoms, const double* guest_atom_x,
                                           const int32_t* guest_atom_species, int32_t n_guest_charges,
                                           const double* guest_charge_x, const double* guest_charge_q,
                                           double ewald_precision, int32_t repfactors_out[3], pmgb_system** out) {
    if (!ctx) return PMGB_ERR_INVALID_ARGUMENT;
    int32_t rep[3] = {1, 1, 1};
    const int rc = pmgb_systems_create_unitcell(ctx, 1, &f_to_c, &n_atoms, &atom_xf, &atom_species, &n_charges,
                                                &charge_xf, &charge_q, &n_species, &epsilon, &sigma2, r_cutoff,
                                                &n_guest_atoms, &guest_atom_x, &guest_atom_species, &n_guest_charges,
                                                &guest_charge_x, &guest_charge_q, ewald_precision, 1, rep, out);
    if (rc == PMGB_OK && repfactors_out)
        for (int d = 0; d < 3; ++d) repfactors_out[d] = rep[d];
    return rc;
}
