/*
 * pm_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C, FP64 restatement of the PorousMaterials.jl (v0.4.2) Widom-insertion /
 * energy-grid path, used solely as the checker for the CUDA library (tests/, the
 * smoke() check and bench.py's cpu_baseline / --impl reference leg).  Nothing in the
 * product path links, loads or calls this file.
 *
 * Every function cites the reference file:line it follows.  The third-party pieces
 * the reference delegates to (Xtals.jl 0.4: Box, replicate, nearest_image!;
 * SpecialFunctions.jl 2: erfc; Roots.jl 2: fzero bracketing bisection) are restated
 * from their published behaviour and pinned by the reference's own golden tests
 * (tests/test_oracle_golden.py).
 *
 * Conventions: 3x3 matrices are column-major (Julia layout): m[i + 3*j] = M[i][j].
 * Coordinate arrays are 3 x n column-major: xf[3*k + d].
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants: src/PorousMaterials.jl:11-13, src/electrostatics.jl:6-7,
 *      src/vdw_energetics.jl:2 ---------------------------------------------- */
#define OR_PI 3.14159265358979323846
static const double OR_R2_OVERLAP = 0.1;

double or_eps0(void) {
    /* electrostatics.jl:6, evaluated left to right like Julia does */
    double q = 1.602176565e-19;
    return 8.854187817e-12 / (q * q) / 1.0e10 * 1.3806488e-23;
}
double or_four_pi_eps0(void) { return 4.0 * OR_PI * or_eps0(); } /* electrostatics.jl:7 */

/* ---- small linear algebra ------------------------------------------------- */
static void matvec(const double m[9], const double v[3], double out[3]) {
    for (int i = 0; i < 3; i++)
        out[i] = m[i] * v[0] + m[i + 3] * v[1] + m[i + 6] * v[2];
}
static void matmul(const double a[9], const double b[9], double out[9]) {
    double t[9];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            t[i + 3 * j] = a[i] * b[3 * j] + a[i + 3] * b[3 * j + 1] + a[i + 6] * b[3 * j + 2];
    memcpy(out, t, sizeof(t));
}
void or_inv3(const double m[9], double out[9]) {
#define M(i, j) m[(i) + 3 * (j)]
    double c00 = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
    double c01 = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
    double c02 = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
    double det = M(0, 0) * c00 + M(0, 1) * c01 + M(0, 2) * c02;
    double t[9];
    t[0 + 3 * 0] = c00 / det;
    t[0 + 3 * 1] = (M(0, 2) * M(2, 1) - M(0, 1) * M(2, 2)) / det;
    t[0 + 3 * 2] = (M(0, 1) * M(1, 2) - M(0, 2) * M(1, 1)) / det;
    t[1 + 3 * 0] = c01 / det;
    t[1 + 3 * 1] = (M(0, 0) * M(2, 2) - M(0, 2) * M(2, 0)) / det;
    t[1 + 3 * 2] = (M(0, 2) * M(1, 0) - M(0, 0) * M(1, 2)) / det;
    t[2 + 3 * 0] = c02 / det;
    t[2 + 3 * 1] = (M(0, 1) * M(2, 0) - M(0, 0) * M(2, 1)) / det;
    t[2 + 3 * 2] = (M(0, 0) * M(1, 1) - M(0, 1) * M(1, 0)) / det;
    memcpy(out, t, sizeof(t));
#undef M
}

/* ---- Xtals.jl Box(a, b, c, α, β, γ) (third-party; call site e.g.
 *      test/electrostatics.jl:28).  f_to_c columns are the lattice vectors,
 *      reciprocal lattice rows = 2π inv(f_to_c). ----------------------------- */
void or_box(double a, double b, double c, double alpha, double beta, double gamma,
            double f_to_c[9], double c_to_f[9], double recip[9], double *omega) {
    double ca = cos(alpha), cb = cos(beta), cg = cos(gamma), sg = sin(gamma);
    double om = a * b * c * sqrt(1.0 - ca * ca - cb * cb - cg * cg + 2.0 * ca * cb * cg);
    double f[9] = {a, 0.0, 0.0,
                   b * cg, b * sg, 0.0,
                   c * cb, c * (ca - cb * cg) / sg, om / (a * b * sg)};
    memcpy(f_to_c, f, sizeof(f));
    or_inv3(f, c_to_f);
    for (int k = 0; k < 9; k++) recip[k] = 2.0 * OR_PI * c_to_f[k];
    *omega = om;
}

/* ---- replication_factors: src/forcefield.jl:120-158 ---------------------- */
static void cross3(const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double norm3(const double a[3]) { return sqrt(dot3(a, a)); }

void or_replication_factors(const double f_to_c[9], double r_cutoff, int rep[3]) {
    double a[3], b[3], c[3], n_ab[3], n_ac[3], n_bc[3], c0[3];
    for (int i = 0; i < 3; i++) { a[i] = f_to_c[i]; b[i] = f_to_c[i + 3]; c[i] = f_to_c[i + 6]; }
    cross3(a, b, n_ab); cross3(a, c, n_ac); cross3(b, c, n_bc);
#define CENTER() for (int i = 0; i < 3; i++) c0[i] = 0.5 * a[i] + 0.5 * b[i] + 0.5 * c[i]
    CENTER();
    rep[0] = rep[1] = rep[2] = 1;
    while (fabs(dot3(n_bc, c0)) / norm3(n_bc) < r_cutoff) {
        rep[0]++; for (int i = 0; i < 3; i++) a[i] += f_to_c[i]; CENTER();
    }
    while (fabs(dot3(n_ac, c0)) / norm3(n_ac) < r_cutoff) {
        rep[1]++; for (int i = 0; i < 3; i++) b[i] += f_to_c[i + 3]; CENTER();
    }
    while (fabs(dot3(n_ab, c0)) / norm3(n_ab) < r_cutoff) {
        rep[2]++; for (int i = 0; i < 3; i++) c[i] += f_to_c[i + 6]; CENTER();
    }
#undef CENTER
}

/* ---- Xtals.jl nearest_image! (third-party; call sites vdw_energetics.jl:30,
 *      electrostatics.jl:377): one shift of each fractional component by
 *      -sign(d) when |d| > 0.5. -------------------------------------------- */
void or_nearest_image(double d[3]) {
    for (int k = 0; k < 3; k++)
        if (fabs(d[k]) > 0.5) d[k] -= (d[k] > 0.0) ? 1.0 : -1.0;
}

/* ---- lennard_jones: src/vdw_energetics.jl:19-22 --------------------------- */
double or_lennard_jones(double r2, double sig2, double eps) {
    double ratio = sig2 / r2;
    ratio = ratio * ratio * ratio;
    return 4.0 * eps * ratio * (ratio - 1.0);
}

/* ---- determine_ewald_params: src/electrostatics.jl:123-141.  Roots.fzero on a
 *      bracket is bisection to machine precision; restated as bisection. ---- */
static double bisect(double (*f)(double, const double *), const double *p, double lo, double hi) {
    double flo = f(lo, p);
    for (int it = 0; it < 2000; it++) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        double fm = f(mid, p);
        if (fm == 0.0) return mid;
        if ((fm > 0.0) == (flo > 0.0)) { lo = mid; flo = fm; } else { hi = mid; }
    }
    return 0.5 * (lo + hi);
}
static double sr_error(double alpha, const double *p) { return erfc(p[0] * alpha) / p[0] - p[1]; }
static double lr_error(double k2, const double *p) {
    if (k2 == 0.0) return INFINITY;
    return 2.0 * exp(-k2 / (4.0 * p[0] * p[0])) / k2 - p[1];
}
void or_determine_ewald_params(double sr_cutoff, double eps, double *alpha, double *max_k2) {
    double p[2] = {sr_cutoff, eps};
    *alpha = bisect(sr_error, p, 0.0, 25.0);
    double q[2] = {*alpha, eps};
    *max_k2 = bisect(lr_error, q, 0.0, 100.0);
}

/* ---- required_kreps: src/electrostatics.jl:157-175 ------------------------ */
void or_required_kreps(const double recip[9], double max_k2, int kreps[3]) {
    for (int abc = 0; abc < 3; abc++) {
        int n = 0;
        for (;;) {
            n++;
            double k[3];
            /* k = transpose(recip) * n e_abc = n * (row abc of recip) */
            for (int i = 0; i < 3; i++) k[i] = recip[abc + 3 * i] * n;
            if (dot3(k, k) > max_k2) { kreps[abc] = n - 1; break; }
        }
    }
}

/* ---- precompute_kvec_wts: src/electrostatics.jl:198-232.  Returns the number
 *      of k-vectors; writes at most max_out of them. ----------------------- */
int or_precompute_kvec_wts(const int kreps[3], const double recip[9], double alpha, double omega,
                           double max_k2, int max_out, int *kabc, double *wt) {
    int n = 0;
    double eps0 = or_eps0();
    for (int ka = 0; ka <= kreps[0]; ka++)
        for (int kb = -kreps[1]; kb <= kreps[1]; kb++)
            for (int kc = -kreps[2]; kc <= kreps[2]; kc++) {
                if (ka == 0 && kb == 0 && kc == 0) continue;
                if (ka == 0 && kb < 0) continue;
                if (ka == 0 && kb == 0 && kc < 0) continue;
                double k[3];
                for (int i = 0; i < 3; i++)
                    k[i] = recip[0 + 3 * i] * ka + recip[1 + 3 * i] * kb + recip[2 + 3 * i] * kc;
                double k2 = dot3(k, k);
                if (k2 < max_k2) {
                    if (n < max_out) {
                        kabc[3 * n] = ka; kabc[3 * n + 1] = kb; kabc[3 * n + 2] = kc;
                        wt[n] = 2.0 * exp(-k2 / (4.0 * alpha * alpha)) / k2 / eps0 / omega;
                    }
                    n++;
                }
            }
    return n;
}

/* ---- system: the replicated crystal + guest description ------------------- */
typedef struct {
    double f_to_c[9], c_to_f[9], recip[9];
    int n_fw; double *fw_xf; int *fw_sp;            /* crystal.atoms (Frac) */
    int n_q; double *q_xf; double *q;               /* crystal.charges (Frac) */
    int n_species; double *eps; double *sig2;       /* ljff.ϵ / ljff.σ² tables */
    double r2_cut;                                  /* ljff.r²_cutoff */
    int n_glj; int *g_sp;                           /* molecule.atoms species */
    int n_gq; double *g_q;                          /* molecule.charges q */
    /* Ewald (EwaldParams, electrostatics.jl:54-63) */
    int has_ewald; double alpha, sr_cut; int kreps[3];
    int n_k; int *kabc; double *wt;
    double *sk_re, *sk_im;                          /* structure factor, S(k) variant */
} or_system;

static void *dup(const void *p, size_t n) {
    if (n == 0) return NULL;
    void *q = malloc(n);
    memcpy(q, p, n);
    return q;
}

or_system *or_system_create(const double f_to_c[9], int n_fw, const double *fw_xf, const int *fw_sp,
                            int n_q, const double *q_xf, const double *q,
                            int n_species, const double *eps, const double *sig2, double r2_cut,
                            int n_glj, const int *g_sp, int n_gq, const double *g_q) {
    or_system *s = (or_system *)calloc(1, sizeof(or_system));
    memcpy(s->f_to_c, f_to_c, 9 * sizeof(double));
    or_inv3(s->f_to_c, s->c_to_f);
    for (int k = 0; k < 9; k++) s->recip[k] = 2.0 * OR_PI * s->c_to_f[k];
    s->n_fw = n_fw; s->fw_xf = dup(fw_xf, 3 * sizeof(double) * n_fw); s->fw_sp = dup(fw_sp, sizeof(int) * n_fw);
    s->n_q = n_q; s->q_xf = dup(q_xf, 3 * sizeof(double) * n_q); s->q = dup(q, sizeof(double) * n_q);
    s->n_species = n_species;
    s->eps = dup(eps, sizeof(double) * n_species * n_species);
    s->sig2 = dup(sig2, sizeof(double) * n_species * n_species);
    s->r2_cut = r2_cut;
    s->n_glj = n_glj; s->g_sp = dup(g_sp, sizeof(int) * n_glj);
    s->n_gq = n_gq; s->g_q = dup(g_q, sizeof(double) * n_gq);
    return s;
}

void or_system_set_ewald(or_system *s, double alpha, double sr_cut, const int kreps[3],
                         int n_k, const int *kabc, const double *wt) {
    s->has_ewald = 1; s->alpha = alpha; s->sr_cut = sr_cut;
    memcpy(s->kreps, kreps, 3 * sizeof(int));
    free(s->kabc); free(s->wt); free(s->sk_re); free(s->sk_im);
    s->n_k = n_k; s->kabc = dup(kabc, 3 * sizeof(int) * n_k); s->wt = dup(wt, sizeof(double) * n_k);
    s->sk_re = s->sk_im = NULL;
}

void or_system_destroy(or_system *s) {
    if (!s) return;
    free(s->fw_xf); free(s->fw_sp); free(s->q_xf); free(s->q); free(s->eps); free(s->sig2);
    free(s->g_sp); free(s->g_q); free(s->kabc); free(s->wt); free(s->sk_re); free(s->sk_im);
    free(s);
}

/* ---- vdw_energy(atoms_i, atoms_j, box, ljff): src/vdw_energetics.jl:25-47,
 *      reached via vdw_energy(crystal, molecule, ljff) at :62-64. --------- */
static double vdw_energy_scaled(const or_system *s, const double *g_xf, double *scale) {
    double energy = 0.0, mag = 0.0;
    for (int i = 0; i < s->n_glj; i++) {
        const double *xi = g_xf + 3 * i;
        int si = s->g_sp[i];
        for (int j = 0; j < s->n_fw; j++) {
            double dxf[3] = {s->fw_xf[3 * j] - xi[0], s->fw_xf[3 * j + 1] - xi[1], s->fw_xf[3 * j + 2] - xi[2]};
            or_nearest_image(dxf);
            double dx[3];
            matvec(s->f_to_c, dxf, dx);
            double r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
            if (r2 < s->r2_cut) {
                if (r2 < OR_R2_OVERLAP) { if (scale) *scale = INFINITY; return INFINITY; }
                int sj = s->fw_sp[j];
                double e = or_lennard_jones(r2, s->sig2[si * s->n_species + sj], s->eps[si * s->n_species + sj]);
                energy += e;
                /* magnitude of the repulsive and attractive parts separately */
                double ratio = s->sig2[si * s->n_species + sj] / r2;
                ratio = ratio * ratio * ratio;
                mag += 4.0 * fabs(s->eps[si * s->n_species + sj]) * ratio * (ratio + 1.0);
            }
        }
    }
    if (scale) *scale = mag;
    return energy;
}

double or_vdw_energy_sys(const or_system *s, const double *g_xf) { return vdw_energy_scaled(s, g_xf, NULL); }

/* ---- _ϕ direct e^{ik·r} form: src/electrostatics.jl:347-388 with fill_eikr!
 *      :288-306.  Scratch arrays are per calling thread (Eikr, :90-101). ---- */
typedef struct { double *ar, *ai, *br, *bi, *cr, *ci, *dxf; } or_eikr;

static or_eikr eikr_alloc(const or_system *s) {
    or_eikr e;
    int n = s->n_q > 0 ? s->n_q : 1;
    e.ar = malloc(sizeof(double) * n * (s->kreps[0] + 1));
    e.ai = malloc(sizeof(double) * n * (s->kreps[0] + 1));
    e.br = malloc(sizeof(double) * n * (2 * s->kreps[1] + 1));
    e.bi = malloc(sizeof(double) * n * (2 * s->kreps[1] + 1));
    e.cr = malloc(sizeof(double) * n * (2 * s->kreps[2] + 1));
    e.ci = malloc(sizeof(double) * n * (2 * s->kreps[2] + 1));
    e.dxf = malloc(sizeof(double) * n * 3);
    return e;
}
static void eikr_free(or_eikr *e) {
    free(e->ar); free(e->ai); free(e->br); free(e->bi); free(e->cr); free(e->ci); free(e->dxf);
}

/* fill_eikr!: column k of a (n_q x (2K+1)) array holds e^{i k k·dx}; offset K
 * maps k = -K..K (or 0..K when negatives are not requested). */
static void fill_eikr(double *er, double *ei, const double *kdx, int n, int krep, int incl_neg) {
    int off = incl_neg ? krep : 0;
    for (int c = 0; c < n; c++) { er[c + n * off] = 1.0; ei[c + n * off] = 0.0; }
    if (krep >= 1)
        for (int c = 0; c < n; c++) { er[c + n * (off + 1)] = cos(kdx[c]); ei[c + n * (off + 1)] = sin(kdx[c]); }
    for (int k = 2; k <= krep; k++)
        for (int c = 0; c < n; c++) {
            double pr = er[c + n * (off + k - 1)], pi = ei[c + n * (off + k - 1)];
            double br = er[c + n * (off + 1)], bi = ei[c + n * (off + 1)];
            er[c + n * (off + k)] = pr * br - pi * bi;
            ei[c + n * (off + k)] = pr * bi + pi * br;
        }
    if (incl_neg)
        for (int k = -krep; k <= -1; k++)
            for (int c = 0; c < n; c++) {
                er[c + n * (off + k)] = er[c + n * (off - k)];
                ei[c + n * (off + k)] = -ei[c + n * (off - k)];
            }
}

static void phi_direct(const or_system *s, const double xf[3], or_eikr *e, double *sr, double *lr) {
    int n = s->n_q;
    double *dxf = e->dxf;
    double *kd = malloc(sizeof(double) * 3 * (n > 0 ? n : 1));
    double M[9];
    matmul(s->recip, s->f_to_c, M); /* (box.reciprocal_lattice * box.f_to_c), :354 */
    for (int c = 0; c < n; c++) {
        for (int d = 0; d < 3; d++) dxf[3 * c + d] = s->q_xf[3 * c + d] - xf[d];
        double v[3];
        matvec(M, dxf + 3 * c, v);
        kd[c] = v[0]; kd[n + c] = v[1]; kd[2 * n + c] = v[2];
    }
    fill_eikr(e->ar, e->ai, kd, n, s->kreps[0], 0);
    fill_eikr(e->br, e->bi, kd + n, n, s->kreps[1], 1);
    fill_eikr(e->cr, e->ci, kd + 2 * n, n, s->kreps[2], 1);
    double plr = 0.0;
    for (int k = 0; k < s->n_k; k++) {
        int ka = s->kabc[3 * k], kb = s->kabc[3 * k + 1] + s->kreps[1], kc = s->kabc[3 * k + 2] + s->kreps[2];
        const double *ar = e->ar + n * ka, *ai = e->ai + n * ka;
        const double *br = e->br + n * kb, *bi = e->bi + n * kb;
        const double *cr = e->cr + n * kc, *ci = e->ci + n * kc;
        double kvec_pot = 0.0;
        for (int c = 0; c < n; c++) {
            double abr = ar[c] * br[c] - ai[c] * bi[c];
            double abi = ar[c] * bi[c] + ai[c] * br[c];
            kvec_pot += s->q[c] * (abr * cr[c] - abi * ci[c]);
        }
        plr += s->wt[k] * kvec_pot;
    }
    free(kd);
    /* short-range sum, :377-386 */
    double psr = 0.0, fpe = or_four_pi_eps0();
    for (int c = 0; c < n; c++) {
        double *d = dxf + 3 * c;
        or_nearest_image(d);
        double v[3];
        matvec(s->f_to_c, d, v);
        double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (r < s->sr_cut) psr += s->q[c] / r * erfc(r * s->alpha) / fpe;
    }
    *sr = psr; *lr = plr;
}

/* ---- structure-factor form of the same long-range sum (proved equal to the
 *      direct form in tests): φ_lr(x) = Σ_k wt_k Re[S(k) e^{-ik·x}],
 *      S(k) = Σ_c q_c e^{ik·r_c}, k·r = 2π (ka fa + kb fb + kc fc). -------- */
void or_structure_factor(or_system *s) {
    free(s->sk_re); free(s->sk_im);
    s->sk_re = malloc(sizeof(double) * (s->n_k > 0 ? s->n_k : 1));
    s->sk_im = malloc(sizeof(double) * (s->n_k > 0 ? s->n_k : 1));
    for (int k = 0; k < s->n_k; k++) {
        double re = 0.0, im = 0.0;
        int ka = s->kabc[3 * k], kb = s->kabc[3 * k + 1], kc = s->kabc[3 * k + 2];
        for (int c = 0; c < s->n_q; c++) {
            const double *f = s->q_xf + 3 * c;
            double ph = 2.0 * OR_PI * (ka * f[0] + kb * f[1] + kc * f[2]);
            re += s->q[c] * cos(ph);
            im += s->q[c] * sin(ph);
        }
        s->sk_re[k] = re; s->sk_im[k] = im;
    }
}
void or_get_structure_factor(const or_system *s, double *re, double *im) {
    memcpy(re, s->sk_re, sizeof(double) * s->n_k);
    memcpy(im, s->sk_im, sizeof(double) * s->n_k);
}

static void phi_sk(const or_system *s, const double xf[3], double *sr, double *lr, double *sr_mag) {
    double plr = 0.0;
    for (int k = 0; k < s->n_k; k++) {
        int ka = s->kabc[3 * k], kb = s->kabc[3 * k + 1], kc = s->kabc[3 * k + 2];
        double ph = 2.0 * OR_PI * (ka * xf[0] + kb * xf[1] + kc * xf[2]);
        /* Re[S e^{-i ph}] = Sr cos(ph) + Si sin(ph) */
        plr += s->wt[k] * (s->sk_re[k] * cos(ph) + s->sk_im[k] * sin(ph));
    }
    double psr = 0.0, fpe = or_four_pi_eps0();
    for (int c = 0; c < s->n_q; c++) {
        double d[3] = {s->q_xf[3 * c] - xf[0], s->q_xf[3 * c + 1] - xf[1], s->q_xf[3 * c + 2] - xf[2]};
        or_nearest_image(d);
        double v[3];
        matvec(s->f_to_c, d, v);
        double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (r < s->sr_cut) {
            double t = s->q[c] / r * erfc(r * s->alpha) / fpe;
            psr += t;
            if (sr_mag) *sr_mag += fabs(t);
        }
    }
    *sr = psr; *lr = plr;
}

/* ---- electrostatic_potential_energy(crystal, molecule, eparams, eikr):
 *      src/electrostatics.jl:331-342 ------------------------------------- */
static void es_energy(const or_system *s, const double *gq_xf, or_eikr *e, int use_sk, double *sr, double *lr,
                      double *sr_mag) {
    double tsr = 0.0, tlr = 0.0;
    if (sr_mag) *sr_mag = 0.0;
    for (int c = 0; c < s->n_gq; c++) {
        double psr, plr, m = 0.0;
        if (use_sk) { phi_sk(s, gq_xf + 3 * c, &psr, &plr, &m); if (sr_mag) *sr_mag += fabs(s->g_q[c]) * m; }
        else phi_direct(s, gq_xf + 3 * c, e, &psr, &plr);
        tsr += s->g_q[c] * psr;
        tlr += s->g_q[c] * plr;
    }
    *sr = tsr; *lr = tlr;
}

void or_energies_scaled(or_system *s, int64_t n_conf, const double *lj_xf, const double *q_xf,
                        int charged, int use_sk, int nthreads, double *out_vdw, double *out_sr,
                        double *out_lr, double *scale_vdw, double *scale_sr);

/* Batched single-configuration energies: for each configuration, the guest's
 * LJ sites (n_glj x 3 frac) and charges (n_gq x 3 frac).  es only when
 * `charged` (henry.jl:93,227-229).  out_vdw may be +Inf (overlap). */
void or_energies(or_system *s, int64_t n_conf, const double *lj_xf, const double *q_xf,
                 int charged, int use_sk, int nthreads,
                 double *out_vdw, double *out_sr, double *out_lr) {
    or_energies_scaled(s, n_conf, lj_xf, q_xf, charged, use_sk, nthreads, out_vdw, out_sr, out_lr, NULL, NULL);
}

/* Same, plus the magnitude scales Σ|LJ repulsive| + Σ|LJ attractive| and Σ|q_g| Σ|real-space
 * term| (S(k) form only) that bound the rounding error of an FP32 evaluation. */
void or_energies_scaled(or_system *s, int64_t n_conf, const double *lj_xf, const double *q_xf,
                        int charged, int use_sk, int nthreads, double *out_vdw, double *out_sr,
                        double *out_lr, double *scale_vdw, double *scale_sr) {
    if (charged && use_sk && !s->sk_re) or_structure_factor(s);
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        or_eikr e = {0};
        if (charged && !use_sk) e = eikr_alloc(s);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (int64_t i = 0; i < n_conf; i++) {
            double vm = 0.0, sm = 0.0;
            out_vdw[i] = vdw_energy_scaled(s, lj_xf + 3 * s->n_glj * i, &vm);
            double sr = 0.0, lr = 0.0;
            if (charged) es_energy(s, q_xf + 3 * s->n_gq * i, &e, use_sk, &sr, &lr, &sm);
            out_sr[i] = sr; out_lr[i] = lr;
            if (scale_vdw) scale_vdw[i] = vm;
            if (scale_sr) scale_sr[i] = sm;
        }
        if (charged && !use_sk) eikr_free(&e);
    }
    (void)nthreads;
}

/* ---- Widom block sums: src/henry.jl:212-244 (per block) ------------------
 * Insertion i belongs to block i / n_per_block.  block_out[3b..3b+2] =
 * (Σ e^{-βU}, Σ U_vdw e^{-βU}, Σ U_es e^{-βU}) accumulated in insertion order.
 */
void or_widom_blocks(const double *u_vdw, const double *u_es, int64_t n_ins, double temperature,
                     int n_blocks, int64_t n_per_block, double *block_out) {
    for (int b = 0; b < n_blocks; b++) block_out[3 * b] = block_out[3 * b + 1] = block_out[3 * b + 2] = 0.0;
    for (int64_t i = 0; i < n_ins; i++) {
        int b = (int)(i / n_per_block);
        if (b >= n_blocks) break;
        double ev = u_vdw[i], ee = u_es[i];
        double bf = exp(-(ev + ee) / temperature);
        block_out[3 * b] += bf;
        if (!isinf(ev) && !isinf(ee)) {
            block_out[3 * b + 1] += bf * ev;
            block_out[3 * b + 2] += bf * ee;
        }
    }
}

/* ---- pose -> site coordinates (translate_to! molecule.jl:176-179 and
 *      random_rotation!(::Molecule{Frac}, box) molecule.jl:269-281):
 *      x_site = xf_com + c_to_f (R b_site), b_site the Cartesian offset of the
 *      site from the centre of mass. ----------------------------------- */
void or_sites_from_poses(const or_system *s, int64_t n, const double *xf_com, const double *rot,
                         int n_sites, const double *body, double *out) {
    for (int64_t i = 0; i < n; i++) {
        const double *R = rot + 9 * i;
        for (int k = 0; k < n_sites; k++) {
            double rb[3], fr[3];
            matvec(R, body + 3 * k, rb);
            matvec(s->c_to_f, rb, fr);
            for (int d = 0; d < 3; d++) out[3 * (n_sites * i + k) + d] = xf_com[3 * i + d] + fr[d];
        }
    }
}

/* ---- energy_grid, single-site probe branch: src/grid.jl:291-338,354-359.
 *      Grid point (i,j,k) -> xf = (i/(n1-1), j/(n2-1), k/(n3-1)) ./ repfactors
 *      in the replicated box; data column-major with i fastest; K units. ---- */
void or_energy_grid(or_system *s, const int n_pts[3], const int rep[3], int nthreads, double *out) {
    int64_t n1 = n_pts[0], n2 = n_pts[1], n3 = n_pts[2];
    int64_t total = n1 * n2 * n3;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
#endif
    for (int64_t idx = 0; idx < total; idx++) {
        int64_t i = idx % n1, j = (idx / n1) % n2, k = idx / (n1 * n2);
        double xf[3] = {(n1 > 1 ? (double)i / (double)(n1 - 1) : 0.0) / rep[0],
                        (n2 > 1 ? (double)j / (double)(n2 - 1) : 0.0) / rep[1],
                        (n3 > 1 ? (double)k / (double)(n3 - 1) : 0.0) / rep[2]};
        out[idx] = or_vdw_energy_sys(s, xf);
    }
    (void)nthreads;
}

/* ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), host restatement used
 *      to check the device generator bit for bit. ------------------------- */
static uint32_t mulhilo32(uint32_t a, uint32_t b, uint32_t *hi) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    return (uint32_t)p;
}
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, hi1;
        uint32_t lo0 = mulhilo32(0xD2511F53u, c0, &hi0);
        uint32_t lo1 = mulhilo32(0xCD9E8D57u, c2, &hi1);
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
