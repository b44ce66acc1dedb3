/*
 * dftg_oracle.c -- CPU FP64 restatement of DFTCXX's grid Fock build.
 *
 * TEST INFRASTRUCTURE.  This library is the checker for the CUDA product in
 * dftcxx_gb300/: only tests/, __graft_entry__.smoke() and the CPU-baseline leg
 * of bench.py may load it.  The product never links or calls it.
 *
 * Every function restates the reference algorithm (ifilot/dftcxx, src/...) and
 * cites the file:line it follows.  Loops keep the reference's structure
 * (per-point Y_lm through atan2/acos and an associated-Legendre recursion,
 * one dense partial-pivot LU per (atom, l, m), linear spline-interval search,
 * serial XC double loop) so that, timed, it stands in for the reference's CPU
 * cost; OpenMP sits where the reference has `#pragma omp parallel for`.
 *
 * Parity pinning: the full reference program needs Eigen3 and Boost, which are
 * absent, so it cannot be built here.  Its dependency-free files are built into
 * oracle/_ref/ (quadrature.{h,cpp}, cspline.cpp, gamma.cpp) and pin the
 * Lebedev table, the cubic spline and the Boys function of this oracle.  The
 * composite steps (Becke weights, Poisson solve, XC and J assembly) are pinned
 * by analytic known-answer tests only (integrated charge, grid overlap vs the
 * analytic S, the Coulomb energy of Gaussian charge clouds, Lebedev exactness).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../dftcxx_gb300/csrc/lebedev_data.h"

#define ORC_PI 3.14159265358979323846      /* atomicgrid.h:50, functionals.h:54 */
#define ORC_PI_TRUNC 3.14159265359         /* cgf.cpp:103, integrals.cpp:342 */
#define ORC_LMAX_CAP 24

typedef struct {
    int natoms;
    int *Z;
    double *xyz;             /* [natoms][3] bohr */
    int nbf;
    double *bf_xyz;          /* [nbf][3] centre of each contracted function */
    int *bf_lmn;             /* [nbf][3] */
    int *bf_off;             /* [nbf+1] primitive offsets */
    double *pa, *pc, *pn;    /* primitive exponent, coefficient, norm */
    int nrad, leb, nang, lmax, nlm;
    size_t npts;
    double *r_n;             /* [nrad], r_n[0] largest */
    double *pos;             /* [npts][3] absolute */
    double *rel;             /* [npts][3] relative to the owning atom */
    double *w;               /* [npts] total weight (incl. Becke) */
    double *wb;              /* [npts] Becke weight */
    double *rho;             /* [npts] */
    double *phi;             /* [npts][nbf] */
    double *V;               /* [npts] total Hartree potential */
    double *Vown;            /* [npts] own-cell part */
    double *rho_lm;          /* [natoms][nrad][nlm] */
    double *U;               /* [natoms][nrad][nlm] */
    double *sx;              /* [nrad] increasing spline abscissae */
    double *sy;              /* [natoms][nlm][nrad] spline ordinates */
    double *sc;              /* [natoms][nlm][nrad-1][4] spline coefficients */
    int stride;              /* timing sample: point loops visit every stride-th point */
    double tm[4];            /* wall times: multipole+Poisson, cross-atom V, J, XC */
} orc_t;

static double orc_now(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

/* Bounded-sample timing mode (CPU baseline only): the cross-atom potential,
 * the J assembly and the XC matrix visit every stride-th point; the caller
 * scales their wall times (orc_get_timings) by stride.  Results are then not
 * the full build and must not be used as values. */

/* ---------------------------------------------------------------- basis */

static double dfact(int n) { double r = 1.0; for (int k = n; k > 1; k -= 2) r *= k; return r; }
static double fact(int n) { double r = 1.0; for (int k = 2; k <= n; ++k) r *= k; return r; }
static double ipow(double x, int n) { double r = 1.0; for (int k = 0; k < n; ++k) r *= x; return r; }

/* GTO normalisation, cgf.cpp:102-114 (truncated pi, cgf.cpp:103). */
double orc_gto_norm(double alpha, int l, int m, int n)
{
    double nom = pow(2.0, 2.0 * (l + m + n) + 3.0 / 2.0) * pow(alpha, (l + m + n) + 3.0 / 2.0);
    double denom = (l < 1 ? 1 : dfact(2 * l - 1)) * (m < 1 ? 1 : dfact(2 * m - 1)) *
                   (n < 1 ? 1 : dfact(2 * n - 1)) * pow(ORC_PI_TRUNC, 3.0 / 2.0);
    return sqrt(nom / denom);
}

/* CGF amplitude, cgf.cpp:49-57 and 146-154. */
static double cgf_amp(const orc_t *o, int i, const double *r)
{
    const double *c = o->bf_xyz + 3 * i;
    const int *q = o->bf_lmn + 3 * i;
    double dx = r[0] - c[0], dy = r[1] - c[1], dz = r[2] - c[2];
    double r2 = dx * dx + dy * dy + dz * dz;
    double sum = 0.0;
    for (int k = o->bf_off[i]; k < o->bf_off[i + 1]; ++k) {
        double amp = o->pn[k] * ipow(dx, q[0]) * ipow(dy, q[1]) * ipow(dz, q[2]) * exp(-o->pa[k] * r2);
        sum += o->pc[k] * amp;
    }
    return sum;
}

/* ------------------------------------------------------ spherical harmonics */

/* spherical_harmonics.cpp:28-33 */
double orc_sh_prefactor(int l, int m)
{
    const double pre = 1.0 / sqrt(4 * ORC_PI);
    int am = m < 0 ? -m : m;
    return pre * (m == 0 ? 1 : sqrt(2.0)) * sqrt((double)(2 * l + 1) * fact(l - am) / fact(l + am));
}

/* Associated Legendre P_n^m(x) with Condon-Shortley phase,
 * spherical_harmonics.cpp:81-117 (stack array instead of a heap vector). */
double orc_legendre_p(int n, int m, double x)
{
    double v[ORC_LMAX_CAP + 2];
    for (int j = 0; j <= n; ++j) v[j] = 0.0;
    if (m <= n) {
        v[m] = 1.0;
        double f = 1.0;
        for (int k = 0; k < m; ++k) { v[m] *= -f * sqrt(1.0 - x * x); f += 2.0; }
    }
    if (m + 1 <= n) v[m + 1] = x * (double)(2 * m + 1) * v[m];
    for (int j = m + 2; j <= n; ++j)
        v[j] = ((double)(2 * j - 1) * x * v[j - 1] + (double)(-j - m + 1) * v[j - 2]) / (double)(j - m);
    return v[n];
}

/* Y_lm = pre * P_l^|m|(cos pole) * {1, cos(m az), sin(-m az)},
 * spherical_harmonics.cpp:24-48, with the (r, azimuth, pole) conversion of
 * atomicgrid.cpp:282-285. */
static double ylm_dir(int l, int m, const double *p)
{
    double r = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    double az = atan2(p[1], p[0]);
    double pole = acos(p[2] / r);
    double a = (m == 0) ? 1.0 : (m > 0 ? cos((double)m * az) : sin(-(double)m * az));
    return orc_sh_prefactor(l, m) * orc_legendre_p(l, m < 0 ? -m : m, cos(pole)) * a;
}

double orc_ylm(int l, int m, double x, double y, double z)
{
    double p[3] = {x, y, z};
    return ylm_dir(l, m, p);
}

/* ------------------------------------------------------------ cubic spline */

/* Cspline::generate_spline, cspline.cpp:66-142.  x increasing, n >= 3.
 * coef: [n-1][4]. */
void orc_spline_build(int n, const double *x, const double *y, double *coef)
{
    double *A = calloc(n, sizeof(double)), *B = calloc(n, sizeof(double));
    double *C = calloc(n, sizeof(double)), *D = calloc(n, sizeof(double));
    double *Y = calloc(n, sizeof(double));
    double h0 = x[1] - x[0], h1 = x[2] - x[1];
    double r0 = (y[1] - y[0]) / h0, r1 = (y[2] - y[1]) / h1;
    B[0] = h1 * (h0 + h1);
    C[0] = (h0 + h1) * (h0 + h1);
    Y[0] = r0 * (3 * h0 * h1 + 2 * h1 * h1) + r1 * h0 * h0;
    for (int i = 1; i < n - 1; ++i) {
        h0 = x[i] - x[i - 1];
        h1 = x[i + 1] - x[i];
        r0 = (y[i] - y[i - 1]) / h0;
        r1 = (y[i + 1] - y[i]) / h1;
        A[i] = h1;
        B[i] = 2 * (h0 + h1);
        C[i] = h0;
        Y[i] = 3 * (r0 * h1 + r1 * h0);
    }
    A[n - 1] = (h0 + h1) * (h0 + h1);
    B[n - 1] = h0 * (h0 + h1);
    Y[n - 1] = r0 * h1 * h1 + r1 * (3 * h0 * h1 + 2 * h0 * h0);
    C[0] = C[0] / B[0];
    for (int i = 1; i < n - 1; ++i) C[i] = C[i] / (B[i] - A[i] * C[i - 1]);
    Y[0] = Y[0] / B[0];
    for (int i = 1; i < n; ++i) Y[i] = (Y[i] - A[i] * Y[i - 1]) / (B[i] - A[i] * C[i - 1]);
    D[n - 1] = Y[n - 1];
    for (int i = n - 1; i > 0; --i) D[i - 1] = Y[i - 1] - C[i - 1] * D[i];
    for (int i = 0; i < n - 1; ++i) {
        double dx = 1.0 / (x[i + 1] - x[i]);
        double dy = (y[i + 1] - y[i]) * dx;
        coef[4 * i + 0] = y[i];
        coef[4 * i + 1] = D[i];
        coef[4 * i + 2] = dx * (3 * dy - 2 * D[i] - D[i + 1]);
        coef[4 * i + 3] = dx * dx * (-2 * dy + D[i] + D[i + 1]);
    }
    free(A); free(B); free(C); free(D); free(Y);
}

/* Cspline::eval, cspline.cpp:151-172: clamp outside, linear interval search. */
static double spline_eval(int n, const double *x, const double *y, const double *coef, double xx)
{
    if (xx < x[0]) return y[0];
    if (xx >= x[n - 1]) return y[n - 1];
    for (int i = 1; i < n; ++i) {
        if (xx <= x[i]) {
            double t = xx - x[i - 1];
            const double *s = coef + 4 * (i - 1);
            return s[0] + s[1] * t + s[2] * t * t + s[3] * t * t * t;
        }
    }
    return 0.0;
}

void orc_spline_eval(int n, const double *x, const double *y, int nq, const double *xq, double *out)
{
    double *coef = malloc(sizeof(double) * 4 * (n - 1));
    orc_spline_build(n, x, y, coef);
    for (int i = 0; i < nq; ++i) out[i] = spline_eval(n, x, y, coef, xq[i]);
    free(coef);
}

/* ------------------------------------------------------------------ create */

static double becke_cutoff(double mu)
{
    /* MolecularGrid::cutoff / fk with k = 3, moleculargrid.cpp:310-329 */
    for (int i = 0; i < 3; ++i) mu = 3.0 / 2.0 * mu - 0.5 * pow(mu, 3.0);
    return 0.5 * (1.0 - mu);
}

static double dist3(const double *a, const double *b)
{
    double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

/* MolecularGrid::get_becke_weight_pn, moleculargrid.cpp:275-300 */
static double becke_pn(const orc_t *o, int i, const double *p0)
{
    double wprod = 1.0;
    const double *p1 = o->xyz + 3 * i;
    for (int j = 0; j < o->natoms; ++j) {
        if (i == j) continue;
        const double *p2 = o->xyz + 3 * j;
        double mu = (dist3(p0, p1) - dist3(p0, p2)) / dist3(p2, p1);
        wprod *= becke_cutoff(mu);
    }
    return wprod;
}

/*
 * Build molecule, basis and grid.  Basis functions are given per contracted
 * function: centre atom, (l,m,n) and a primitive range into alpha/coef.
 * Mirrors MolecularGrid::create_grid (moleculargrid.cpp:193-261) and
 * AtomicGrid::create_atomic_grid (atomicgrid.cpp:32-88).
 */
orc_t *orc_create(int natoms, const int *Z, const double *xyz,
                  int nbf, const int *bf_atom, const int *bf_lmn, const int *bf_nprim,
                  const double *alpha, const double *coef,
                  int nrad, int leb, int lmax)
{
    if (natoms < 1 || nbf < 1 || nrad < 3 || leb < 0 || leb >= DFTG_NUM_LEBEDEV_ORDERS ||
        lmax < 0 || lmax > ORC_LMAX_CAP)
        return NULL;
    orc_t *o = calloc(1, sizeof(orc_t));
    o->natoms = natoms;
    o->Z = malloc(sizeof(int) * natoms);
    o->xyz = malloc(sizeof(double) * 3 * natoms);
    memcpy(o->Z, Z, sizeof(int) * natoms);
    memcpy(o->xyz, xyz, sizeof(double) * 3 * natoms);
    o->nbf = nbf;
    o->bf_xyz = malloc(sizeof(double) * 3 * nbf);
    o->bf_lmn = malloc(sizeof(int) * 3 * nbf);
    o->bf_off = malloc(sizeof(int) * (nbf + 1));
    o->bf_off[0] = 0;
    for (int i = 0; i < nbf; ++i) {
        memcpy(o->bf_xyz + 3 * i, xyz + 3 * bf_atom[i], 3 * sizeof(double));
        memcpy(o->bf_lmn + 3 * i, bf_lmn + 3 * i, 3 * sizeof(int));
        o->bf_off[i + 1] = o->bf_off[i] + bf_nprim[i];
    }
    int np = o->bf_off[nbf];
    o->pa = malloc(sizeof(double) * np);
    o->pc = malloc(sizeof(double) * np);
    o->pn = malloc(sizeof(double) * np);
    for (int i = 0; i < nbf; ++i)
        for (int k = o->bf_off[i]; k < o->bf_off[i + 1]; ++k) {
            o->pa[k] = alpha[k];
            o->pc[k] = coef[k];
            o->pn[k] = orc_gto_norm(alpha[k], bf_lmn[3 * i], bf_lmn[3 * i + 1], bf_lmn[3 * i + 2]);
        }

    o->nrad = nrad;
    o->leb = leb;
    o->nang = dftg_lebedev_npts[leb];
    o->lmax = lmax;
    o->nlm = (lmax + 1) * (lmax + 1);
    o->npts = (size_t)natoms * nrad * o->nang;
    size_t n = o->npts;
    o->r_n = malloc(sizeof(double) * nrad);
    o->pos = malloc(sizeof(double) * 3 * n);
    o->rel = malloc(sizeof(double) * 3 * n);
    o->w = malloc(sizeof(double) * n);
    o->wb = malloc(sizeof(double) * n);
    o->rho = calloc(n, sizeof(double));
    o->V = calloc(n, sizeof(double));
    o->Vown = calloc(n, sizeof(double));
    o->phi = malloc(sizeof(double) * n * nbf);
    o->rho_lm = calloc((size_t)natoms * nrad * o->nlm, sizeof(double));
    o->U = calloc((size_t)natoms * nrad * o->nlm, sizeof(double));
    o->sx = malloc(sizeof(double) * nrad);
    o->sy = malloc(sizeof(double) * (size_t)natoms * o->nlm * nrad);
    o->sc = malloc(sizeof(double) * (size_t)natoms * o->nlm * (nrad - 1) * 4);
    o->stride = 1;

    const int off = dftg_lebedev_offset[leb];
    const double f = ORC_PI / (double)(nrad + 1);
    for (int a = 0; a < natoms; ++a) {
        const double *p1 = o->xyz + 3 * a;
        for (int p = 1; p <= nrad; ++p) {
            double w = f * pow(sin(f * (double)p), 2.0);
            double x = cos(f * (double)p);
            double r = (1.0 + x) / (1.0 - x);
            o->r_n[p - 1] = r;
            w = w / sqrt(1.0 - pow(x, 2.0)) * 2.0 / pow(1.0 - x, 2.0);
            for (int j = 0; j < o->nang; ++j) {
                size_t idx = ((size_t)a * nrad + (p - 1)) * o->nang + j;
                const double *L = dftg_lebedev_table[off + j];
                double p2[3] = {L[0] * r, L[1] * r, L[2] * r};
                for (int d = 0; d < 3; ++d) {
                    o->rel[3 * idx + d] = p2[d];
                    o->pos[3 * idx + d] = p1[d] + p2[d];
                }
                o->w[idx] = w * L[3];
            }
        }
    }
    /* Jacobian r^2 * 4 pi (atomicgrid.cpp:84-87) */
    for (size_t i = 0; i < n; ++i) {
        const double *p2 = o->rel + 3 * i;
        o->w[i] *= (p2[0] * p2[0] + p2[1] * p2[1] + p2[2] * p2[2]) * 4.0 * ORC_PI;
    }
    /* amplitudes (gridpoint.cpp:45-52) */
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; ++i)
        for (int k = 0; k < nbf; ++k) o->phi[(size_t)i * nbf + k] = cgf_amp(o, k, o->pos + 3 * i);
    /* Becke partition, moleculargrid.cpp:229-254 */
    for (int a = 0; a < natoms; ++a) {
        size_t base = (size_t)a * nrad * o->nang;
        #pragma omp parallel for schedule(static)
        for (long j = 0; j < (long)nrad * o->nang; ++j) {
            const double *p0 = o->pos + 3 * (base + j);
            double denom = 0.0, nom = 1.0;
            for (int k = 0; k < natoms; ++k) {
                double t = becke_pn(o, k, p0);
                denom += t;
                if (a == k) nom = t;
            }
            double bw = nom / denom;
            o->w[base + j] *= bw;
            o->wb[base + j] = bw;
        }
    }
    /* increasing spline abscissae (atomicgrid.cpp:535-545) */
    for (int i = 0; i < nrad; ++i) o->sx[i] = o->r_n[nrad - 1 - i];
    return o;
}

void orc_destroy(orc_t *o)
{
    if (!o) return;
    free(o->Z); free(o->xyz); free(o->bf_xyz); free(o->bf_lmn); free(o->bf_off);
    free(o->pa); free(o->pc); free(o->pn); free(o->r_n); free(o->pos); free(o->rel);
    free(o->w); free(o->wb); free(o->rho); free(o->phi); free(o->V); free(o->Vown);
    free(o->rho_lm); free(o->U); free(o->sx); free(o->sy); free(o->sc);
    free(o);
}

long orc_grid_size(const orc_t *o) { return (long)o->npts; }
void orc_set_sample_stride(orc_t *o, int s) { o->stride = s < 1 ? 1 : s; }
void orc_get_timings(const orc_t *o, double *out) { memcpy(out, o->tm, sizeof(o->tm)); }
int orc_nang(const orc_t *o) { return o->nang; }

void orc_get_weights(const orc_t *o, double *out) { memcpy(out, o->w, sizeof(double) * o->npts); }
void orc_get_becke_weights(const orc_t *o, double *out) { memcpy(out, o->wb, sizeof(double) * o->npts); }
void orc_get_densities(const orc_t *o, double *out) { memcpy(out, o->rho, sizeof(double) * o->npts); }
void orc_get_positions(const orc_t *o, double *out) { memcpy(out, o->pos, sizeof(double) * 3 * o->npts); }
void orc_get_potential(const orc_t *o, double *out) { memcpy(out, o->V, sizeof(double) * o->npts); }
void orc_get_radii(const orc_t *o, double *out) { memcpy(out, o->r_n, sizeof(double) * o->nrad); }
/* amplitudes as nbf x npts column-major == [npts][nbf] (moleculargrid.cpp:109-127) */
void orc_get_amplitudes(const orc_t *o, double *out) { memcpy(out, o->phi, sizeof(double) * o->npts * o->nbf); }
void orc_get_U(const orc_t *o, double *out) { memcpy(out, o->U, sizeof(double) * o->natoms * o->nrad * o->nlm); }
void orc_get_rho_lm(const orc_t *o, double *out) { memcpy(out, o->rho_lm, sizeof(double) * o->natoms * o->nrad * o->nlm); }

/* -------------------------------------------------------------- density */

/* GridPoint::set_density: rho = 2 phi^T (P phi), gridpoint.cpp:82-84.
 * P is nbf x nbf column-major. */
void orc_set_density(orc_t *o, const double *P)
{
    const int nbf = o->nbf;
    #pragma omp parallel
    {
        double *t = malloc(sizeof(double) * nbf);
        #pragma omp for schedule(static)
        for (long i = 0; i < (long)o->npts; ++i) {
            const double *f = o->phi + (size_t)i * nbf;
            for (int r = 0; r < nbf; ++r) {
                double s = 0.0;
                for (int c = 0; c < nbf; ++c) s += P[r + (size_t)c * nbf] * f[c];
                t[r] = s;
            }
            double d = 0.0;
            for (int r = 0; r < nbf; ++r) d += f[r] * t[r];
            o->rho[i] = 2.0 * d;
        }
        free(t);
    }
}

/* AtomicGrid::calculate_density, atomicgrid.cpp:520-530 */
static double atom_density(const orc_t *o, int a)
{
    size_t base = (size_t)a * o->nrad * o->nang, cnt = (size_t)o->nrad * o->nang;
    double d = 0.0;
    for (size_t i = 0; i < cnt; ++i) d += o->w[base + i] * o->rho[base + i];
    return d;
}

/* MolecularGrid::calculate_density, moleculargrid.cpp:157-166 */
double orc_calculate_density(const orc_t *o)
{
    double s = 0.0;
    for (int a = 0; a < o->natoms; ++a) s += atom_density(o, a);
    return s;
}

/* MolecularGrid::correct_densities, moleculargrid.cpp:132-146; returns c. */
double orc_correct_densities(orc_t *o)
{
    double sum = 0.0, charge = 0.0;
    for (int a = 0; a < o->natoms; ++a) {
        sum += atom_density(o, a);
        charge += o->Z[a];
    }
    double c = charge / sum;
    for (size_t i = 0; i < o->npts; ++i) o->rho[i] *= c;
    return c;
}

/* ---------------------------------------------------------------- LDA */

static double vwn_xx(double x, double b, double c) { return x * x + b * x + c; }

/* functionals.cpp:128-133 */
static double vwn_eps(double x, double a, double x0, double b, double c)
{
    double q = sqrt(4.0 * c - b * b);
    return a * (log(x * x / vwn_xx(x, b, c))
                - b * (x0 / vwn_xx(x0, b, c)) * log(pow(x - x0, 2.0) / vwn_xx(x, b, c))
                + (2.0 * b / q) * (1.0 - (x0 * (2.0 * x0 + b) / vwn_xx(x0, b, c))) * atan(q / (2.0 * x + b)));
}

/* functionals.cpp:144-150 */
static double vwn_deps(double x, double a, double x0, double b, double c)
{
    double q = sqrt(4.0 * c - b * b);
    return a * (2.0 / x - (2.0 * x + b) / vwn_xx(x, b, c)
                - 4.0 * b / (pow(2.0 * x + b, 2.0) + q * q) - (b * x0 / vwn_xx(x0, b, c))
                * (2.0 / (x - x0) - (2.0 * x + b) / vwn_xx(x, b, c) - 4.0 * (2.0 * x0 + b) / (pow(2.0 * x + b, 2.0) + q * q)));
}

/*
 * Slater exchange (functionals.cpp:24-63) and VWN correlation
 * (functionals.cpp:65-114) for one point, closed shell (rho_a = rho_b = rho/2,
 * dft.cpp:411-412).  Returns e_x + e_c (energy density per volume) and the
 * point potential 0.5*(vxa + vxb + vca + vcb) (dft.cpp:424).
 */
void orc_lda_point(double rho, double *exc_out, double *v_out)
{
    const double tol = 1e-10;
    const double xalpha = 2.0 / 3.0;
    const double fac = -2.25 * xalpha * pow(3.0 / 4.0 / ORC_PI, 1.0 / 3.0);
    double da = rho * 0.5, db = rho * 0.5;
    double ex = 0.0, vxa = 0.0, vxb = 0.0;
    if (!(da < tol)) { double r3 = pow(da, 1.0 / 3.0); ex += fac * da * r3; vxa += 4.0 / 3.0 * fac * r3; }
    if (!(db < tol)) { double r3 = pow(db, 1.0 / 3.0); ex += fac * db * r3; vxb += 4.0 / 3.0 * fac * r3; }
    double ec = 0.0, vca = 0.0, vcb = 0.0;
    double dens = da + db;
    if (!(dens < tol)) {
        double zeta = (da - db) / dens;
        double x = pow(3.0 / 4.0 / ORC_PI / dens, 1.0 / 6.0);
        double epsp = vwn_eps(x, 0.0310907, -0.10498, 3.72744, 12.9352);
        double depsp = vwn_deps(x, 0.0310907, -0.10498, 3.72744, 12.9352);
        double g = 1.125 * (pow(1.0 + zeta, 4.0 / 3.0) + pow(1.0 - zeta, 4.0 / 3.0) - 2.0);
        if (g < tol) {
            ec = epsp * dens;
            vca = epsp - (x / 6.0) * depsp;
            vcb = vca;
        } else {
            double epsf = vwn_eps(x, 0.01554535, -0.32500, 7.06042, 13.0045);
            double depsf = vwn_deps(x, 0.01554535, -0.32500, 7.06042, 13.0045);
            double eps = epsp + g * (epsf - epsp);
            double dg = 1.5 * (pow(1.0 + zeta, 1.0 / 3.0) - pow(1.0 - zeta, 1.0 / 3.0));
            double deps_dx = depsp + g * (depsf - depsp);
            double deps_dg = (epsf - epsp) * dg;
            ec = eps * dens;
            vca = eps - (x / 6.0) * deps_dx + deps_dg * (1.0 - zeta);
            vcb = eps - (x / 6.0) * deps_dx - deps_dg * (1.0 + zeta);
        }
    }
    *exc_out = ex + ec;
    *v_out = (vxa + vxb + vca + vcb) * 0.5;
}

/* DFT::calculate_exchange_correlation_matrix, dft.cpp:394-433.
 * XC is nbf x nbf (symmetric, full square written).  Returns E_xc. */
double orc_xc(orc_t *o, double *XC, double *vxc_out)
{
    const size_t n = o->npts;
    const int nbf = o->nbf;
    double *wva = malloc(sizeof(double) * n);
    double *e = malloc(sizeof(double) * n);
    #pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; ++i) {
        double ex, v;
        orc_lda_point(o->rho[i], &ex, &v);
        e[i] = ex;
        wva[i] = o->w[i] * v;
        if (vxc_out) vxc_out[i] = v;
    }
    double exc = 0.0;
    for (size_t i = 0; i < n; ++i) exc += o->w[i] * e[i];
    /* nbf^2 dot products over the grid, serial as in dft.cpp:426-432 */
    const size_t st = (size_t)o->stride;
    double t0 = orc_now();
    for (int i = 0; i < nbf; ++i)
        for (int j = 0; j < nbf; ++j) {
            double s = 0.0;
            for (size_t p = 0; p < n; p += st) s += wva[p] * o->phi[p * nbf + i] * o->phi[p * nbf + j];
            XC[i + (size_t)j * nbf] = s;
        }
    o->tm[3] = orc_now() - t0;
    free(wva);
    free(e);
    return exc;
}

/* ------------------------------------------------------------- Hartree */

/* AtomicGrid::calculate_rho_lm, atomicgrid.cpp:241-296 */
static void calc_rho_lm(orc_t *o, int a)
{
    const int nang = o->nang, nlm = o->nlm, off = dftg_lebedev_offset[o->leb];
    size_t base = (size_t)a * o->nrad * nang;
    double *R = o->rho_lm + (size_t)a * o->nrad * nlm;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < o->nrad; ++i) {
        int cnt = 0;
        for (int l = 0; l <= o->lmax; ++l)
            for (int m = -l; m <= l; ++m) {
                double s = 0.0;
                for (int j = 0; j < nang; ++j) {
                    size_t idx = base + (size_t)i * nang + j;
                    double y = ylm_dir(l, m, o->rel + 3 * idx);
                    s += o->rho[idx] * y * dftg_lebedev_table[off + j][3] * o->wb[idx];
                }
                R[(size_t)i * nlm + cnt] = s * 4.0 * ORC_PI;
                cnt++;
            }
    }
}

/* AtomicGrid::d2zdr2 / dzdrsq, atomicgrid.cpp:502-510 (m = 1) */
static double d2zdr2(double r, double m)
{
    double nom = m * m * (m + 3.0 * r);
    double denom = 2.0 * ORC_PI * pow((m * r) / ((m + r) * (m + r)), 1.5) * pow(m + r, 5.0);
    return nom / denom;
}
static double dzdrsq(double r, double m) { return m / (ORC_PI * ORC_PI * r * (m + r) * (m + r)); }

/* Finite-difference radial Poisson operator, atomicgrid.cpp:316-389.
 * A is (N+2)x(N+2) row-major. */
void orc_poisson_matrix(int N, const double *r_n, double *A)
{
    const double h = 1.0 / (double)(N + 1);
    const int S = N + 2;
    memset(A, 0, sizeof(double) * S * S);
#define M_(i, j) A[(size_t)(i) * S + (j)]
    for (int i = 0; i < S; ++i) {
        double c1 = 0.0, c2 = 0.0;
        if (i > 0 && i < N + 1) { c1 = dzdrsq(r_n[i - 1], 1.0); c2 = d2zdr2(r_n[i - 1], 1.0); }
        if (i == 0) { M_(0, 0) = 1.0; continue; }
        if (i == 1) {
            c1 /= 12.0 * h * h; c2 /= 12.0 * h;
            M_(i, 0) = 11.0 * c1 - 3.0 * c2; M_(i, 1) = -20.0 * c1 - 10.0 * c2;
            M_(i, 2) = 6.0 * c1 + 18.0 * c2; M_(i, 3) = 4.0 * c1 - 6.0 * c2;
            M_(i, 4) = -1.0 * c1 + 1.0 * c2;
            continue;
        }
        if (i == 2) {
            c1 /= 12.0 * h * h; c2 /= 60.0 * h;
            M_(i, 0) = -1.0 * c1 + 3.0 * c2; M_(i, 1) = 16.0 * c1 - 30.0 * c2;
            M_(i, 2) = -30.0 * c1 - 20.0 * c2; M_(i, 3) = 16.0 * c1 + 60.0 * c2;
            M_(i, 4) = -1.0 * c1 - 15.0 * c2; M_(i, 5) = 0.0 * c1 + 2.0 * c2;
            continue;
        }
        if (i == N - 1) {
            c1 /= 12.0 * h * h; c2 /= 60.0 * h;
            M_(i, N - 4) = 0.0 * c1 - 2.0 * c2; M_(i, N - 3) = -1.0 * c1 + 15.0 * c2;
            M_(i, N - 2) = 16.0 * c1 - 60.0 * c2; M_(i, N - 1) = -30.0 * c1 + 20.0 * c2;
            M_(i, N) = 16.0 * c1 + 30.0 * c2; M_(i, N + 1) = -1.0 * c1 - 3.0 * c2;
            continue;
        }
        if (i == N) {
            c1 /= 12.0 * h * h; c2 /= 12.0 * h;
            M_(i, N - 3) = -1.0 * c1 - 1.0 * c2; M_(i, N - 2) = 4.0 * c1 + 6.0 * c2;
            M_(i, N - 1) = 6.0 * c1 - 18.0 * c2; M_(i, N) = -20.0 * c1 + 10.0 * c2;
            M_(i, N + 1) = 11.0 * c1 + 3.0 * c2;
            continue;
        }
        if (i == N + 1) { M_(i, i) = 1.0; continue; }
        c1 /= 180.0 * h * h; c2 /= 60.0 * h;
        M_(i, i - 3) = 2.0 * c1 - 1.0 * c2; M_(i, i - 2) = -27.0 * c1 + 9.0 * c2;
        M_(i, i - 1) = 270.0 * c1 - 45.0 * c2; M_(i, i) = -490.0 * c1;
        M_(i, i + 1) = 270.0 * c1 + 45.0 * c2; M_(i, i + 2) = -27.0 * c1 - 9.0 * c2;
        M_(i, i + 3) = 2.0 * c1 + 1.0 * c2;
    }
#undef M_
}

/* Dense LU with partial pivoting, solving M b = g in place (g -> b).
 * Stands in for Eigen::PartialPivLU (atomicgrid.cpp:424-425). */
static void lu_solve(int S, double *M, double *g)
{
    for (int k = 0; k < S; ++k) {
        int p = k;
        double best = fabs(M[(size_t)k * S + k]);
        for (int i = k + 1; i < S; ++i) {
            double v = fabs(M[(size_t)i * S + k]);
            if (v > best) { best = v; p = i; }
        }
        if (p != k) {
            for (int j = 0; j < S; ++j) {
                double t = M[(size_t)k * S + j]; M[(size_t)k * S + j] = M[(size_t)p * S + j]; M[(size_t)p * S + j] = t;
            }
            double t = g[k]; g[k] = g[p]; g[p] = t;
        }
        double piv = M[(size_t)k * S + k];
        for (int i = k + 1; i < S; ++i) {
            double f = M[(size_t)i * S + k] / piv;
            if (f == 0.0) continue;
            M[(size_t)i * S + k] = f;
            for (int j = k + 1; j < S; ++j) M[(size_t)i * S + j] -= f * M[(size_t)k * S + j];
            g[i] -= f * g[k];
        }
    }
    for (int i = S - 1; i >= 0; --i) {
        double s = g[i];
        for (int j = i + 1; j < S; ++j) s -= M[(size_t)i * S + j] * g[j];
        g[i] = s / M[(size_t)i * S + i];
    }
}

/* AtomicGrid::calculate_U_lm, atomicgrid.cpp:301-466 (U_lm, own-cell V and
 * the splines of interpolate_sh_coeff, atomicgrid.cpp:535-556). */
static void calc_U_lm(orc_t *o, int a)
{
    const int N = o->nrad, S = N + 2, nlm = o->nlm, nang = o->nang;
    const double sqrt4pi = sqrt(4.0 * ORC_PI);
    const double q_n = atom_density(o, a);
    double *A = malloc(sizeof(double) * S * S);
    orc_poisson_matrix(N, o->r_n, A);
    double *U = o->U + (size_t)a * N * nlm;
    const double *R = o->rho_lm + (size_t)a * N * nlm;
    #pragma omp parallel for schedule(dynamic)
    for (int l = 0; l <= o->lmax; ++l) {
        double *M = malloc(sizeof(double) * S * S);
        double *g = malloc(sizeof(double) * S);
        for (int m = -l; m <= l; ++m) {
            int n = l * l + l + m;
            memcpy(M, A, sizeof(double) * S * S);
            for (int i = 0; i < S; ++i) {
                if (i == 0) { g[i] = (n == 0) ? sqrt4pi * q_n : 0.0; continue; }
                if (i == N + 1) { g[i] = 0.0; continue; }
                M[(size_t)i * S + i] -= (double)l * (double)(l + 1) / (o->r_n[i - 1] * o->r_n[i - 1]);
                g[i] = -4.0 * ORC_PI * o->r_n[i - 1] * R[(size_t)(i - 1) * nlm + n];
            }
            lu_solve(S, M, g);
            for (int i = 1; i < N + 1; ++i) U[(size_t)(i - 1) * nlm + n] = g[i];
        }
        free(M);
        free(g);
    }
    free(A);
    /* own-cell potential, atomicgrid.cpp:439-462 */
    size_t base = (size_t)a * N * nang;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < nang; ++j) o->Vown[base + (size_t)i * nang + j] = 0.0;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i)
        for (int l = 0; l <= o->lmax; ++l)
            for (int m = -l; m <= l; ++m) {
                int n = l * l + l + m;
                for (int j = 0; j < nang; ++j) {
                    size_t idx = base + (size_t)i * nang + j;
                    const double *p = o->rel + 3 * idx;
                    double r = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
                    o->Vown[idx] += 1.0 / r * ylm_dir(l, m, p) * U[(size_t)i * nlm + n];
                }
            }
    /* splines over increasing r (atomicgrid.cpp:535-556) */
    for (int k = 0; k < nlm; ++k) {
        double *y = o->sy + ((size_t)a * nlm + k) * N;
        for (int j = 0; j < N; ++j) y[j] = U[(size_t)(N - 1 - j) * nlm + k];
        orc_spline_build(N, o->sx, y, o->sc + ((size_t)a * nlm + k) * (N - 1) * 4);
    }
}

/* MolecularGrid::calculate_hartree_potential, moleculargrid.cpp:336-389,
 * with AtomicGrid::calculate_J_matrix (atomicgrid.cpp:471-488).
 * J is nbf x nbf; the 1/2 of atomicgrid.cpp:485 is included. */
void orc_hartree(orc_t *o, double *J)
{
    const int N = o->nrad, nlm = o->nlm, nang = o->nang, nbf = o->nbf;
    const long st = o->stride;
    double t0 = orc_now();
    for (int a = 0; a < o->natoms; ++a) {
        calc_rho_lm(o, a);
        calc_U_lm(o, a);
    }
    double t1 = orc_now();
    for (int i = 0; i < o->natoms; ++i) {
        size_t base = (size_t)i * N * nang;
        #pragma omp parallel for schedule(static)
        for (long j = 0; j < (long)N * nang; j += st) {
            double V = 0.0;
            const double *pp = o->pos + 3 * (base + j);
            for (int k = 0; k < o->natoms; ++k) {
                if (i == k) { V += o->Vown[base + j]; continue; }
                int lm = 0;
                for (int l = 0; l <= o->lmax; ++l)
                    for (int m = -l; m <= l; ++m) {
                        double d[3] = {pp[0] - o->xyz[3 * k], pp[1] - o->xyz[3 * k + 1], pp[2] - o->xyz[3 * k + 2]};
                        double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                        double y = ylm_dir(l, m, d);
                        const double *sy = o->sy + ((size_t)k * nlm + lm) * N;
                        const double *sc = o->sc + ((size_t)k * nlm + lm) * (N - 1) * 4;
                        V += 1.0 / r * y * spline_eval(N, o->sx, sy, sc, r);
                        lm++;
                    }
            }
            o->V[base + j] = V;
        }
    }
    double t2 = orc_now();
    memset(J, 0, sizeof(double) * nbf * nbf);
    double *Jj = malloc(sizeof(double) * nbf * nbf);
    for (int a = 0; a < o->natoms; ++a) {
        size_t base = (size_t)a * N * nang, cnt = (size_t)N * nang;
        #pragma omp parallel for schedule(dynamic)
        for (int i = 0; i < nbf; ++i)
            for (int j = i; j < nbf; ++j) {
                double s = 0.0;
                for (size_t p = 0; p < cnt; p += (size_t)st) {
                    size_t q = base + p;
                    s += o->w[q] * o->V[q] * o->phi[q * nbf + i] * o->phi[q * nbf + j];
                }
                Jj[i + (size_t)j * nbf] = Jj[j + (size_t)i * nbf] = s * 0.5;
            }
        for (int t = 0; t < nbf * nbf; ++t) J[t] += Jj[t];
    }
    free(Jj);
    o->tm[0] = t1 - t0;
    o->tm[1] = t2 - t1;
    o->tm[2] = orc_now() - t2;
}

/* ------------------------------------------------- one-electron integrals */

static double binomial(int a, int b)
{
    if ((a < 0) | (b < 0) | (a - b < 0)) return 1.0;
    return fact(a) / (fact(b) * fact(a - b));
}

/* integrals.cpp:279-290 */
static double binomial_prefactor(int s, int ia, int ib, double xpa, double xpb)
{
    double sum = 0.0;
    for (int t = 0; t < s + 1; ++t)
        if ((s - ia <= t) && (t <= ib))
            sum += binomial(ia, s - t) * binomial(ib, t) * ipow(xpa, ia - s + t) * ipow(xpb, ib - t);
    return sum;
}

/* integrals.cpp:265-273 */
static double overlap_1d(int l1, int l2, double x1, double x2, double gamma)
{
    double sum = 0.0;
    for (int i = 0; i < (1 + (int)floor(0.5 * (l1 + l2))); ++i)
        sum += binomial_prefactor(2 * i, l1, l2, x1, x2) * (i == 0 ? 1 : dfact(2 * i - 1)) / pow(2 * gamma, i);
    return sum;
}

/* primitive overlap, integrals.cpp:252-263 */
static double ovl_prim(double a1, int l1, int m1, int n1, const double *A,
                       double a2, int l2, int m2, int n2, const double *B)
{
    const double pi = 3.141592653589793238462643383279502884;
    double g = a1 + a2;
    double rab2 = 0.0, P[3];
    for (int d = 0; d < 3; ++d) { rab2 += (A[d] - B[d]) * (A[d] - B[d]); P[d] = (a1 * A[d] + a2 * B[d]) / g; }
    double pre = pow(pi / g, 1.5) * exp(-a1 * a2 * rab2 / g);
    return pre * overlap_1d(l1, l2, P[0] - A[0], P[0] - B[0], g) *
           overlap_1d(m1, m2, P[1] - A[1], P[1] - B[1], g) *
           overlap_1d(n1, n2, P[2] - A[2], P[2] - B[2], g);
}

/* primitive kinetic, integrals.cpp:101-121 (terms with l2<2 vanish) */
static double kin_prim(double a1, int l1, int m1, int n1, const double *A,
                       double a2, int l2, int m2, int n2, const double *B)
{
    double t0 = a2 * (2.0 * (l2 + m2 + n2) + 3.0) * ovl_prim(a1, l1, m1, n1, A, a2, l2, m2, n2, B);
    double t1 = -2.0 * pow(a2, 2.0) * (ovl_prim(a1, l1, m1, n1, A, a2, l2 + 2, m2, n2, B) +
                                       ovl_prim(a1, l1, m1, n1, A, a2, l2, m2 + 2, n2, B) +
                                       ovl_prim(a1, l1, m1, n1, A, a2, l2, m2, n2 + 2, B));
    double t2 = 0.0;
    if (l2 >= 2) t2 += l2 * (l2 - 1) * ovl_prim(a1, l1, m1, n1, A, a2, l2 - 2, m2, n2, B);
    if (m2 >= 2) t2 += m2 * (m2 - 1) * ovl_prim(a1, l1, m1, n1, A, a2, l2, m2 - 2, n2, B);
    if (n2 >= 2) t2 += n2 * (n2 - 1) * ovl_prim(a1, l1, m1, n1, A, a2, l2, m2, n2 - 2, B);
    return t0 + t1 - 0.5 * t2;
}

/*
 * Boys function F_m(x) with the reference's clamp x = max(|x|, 1e-8)
 * (gamma.cpp:41-46).  The reference evaluates it through Numerical-Recipes
 * incomplete gamma; here: the positive-term series
 *   F_m(x) = e^-x sum_k (2x)^k / ((2m+1)(2m+3)...(2m+2k+1))
 * for x < 40 and the erf closed form with upward recursion above.
 */
double orc_fgamma(int m, double x)
{
    x = fabs(x);
    if (x < 1e-8) x = 1e-8;
    if (x < 40.0) {
        double term = 1.0 / (2 * m + 1), sum = term;
        for (int k = 1; k < 400; ++k) {
            term *= 2.0 * x / (2 * m + 2 * k + 1);
            sum += term;
            if (term < sum * 1e-17) break;
        }
        return exp(-x) * sum;
    }
    double f = 0.5 * sqrt(ORC_PI / x) * erf(sqrt(x));
    double ex = exp(-x);
    for (int k = 0; k < m; ++k) f = ((2 * k + 1) * f - ex) / (2.0 * x);
    return f;
}

/* integrals.cpp:367-387 */
static void a_array(int l1, int l2, double pa, double pb, double cp, double g, double *arr)
{
    int imax = l1 + l2 + 1;
    for (int i = 0; i < imax; ++i) arr[i] = 0.0;
    for (int i = 0; i < imax; ++i)
        for (int r = 0; r <= i / 2; ++r)
            for (int u = 0; u <= (i - 2 * r) / 2; ++u) {
                int iI = i - 2 * r - u;
                arr[iI] += ((i & 1) ? -1.0 : 1.0) * binomial_prefactor(i, l1, l2, pa, pb) *
                           ((u & 1) ? -1.0 : 1.0) * fact(i) * ipow(cp, i - 2 * r - 2 * u) *
                           pow(0.25 / g, r + u) / fact(r) / fact(u) / fact(i - 2 * r - 2 * u);
            }
}

/* primitive nuclear attraction, integrals.cpp:336-365 */
static double nuc_prim(const double *A, int l1, int m1, int n1, double a1,
                       const double *B, int l2, int m2, int n2, double a2, const double *C)
{
    double g = a1 + a2, P[3], rab2 = 0.0, rcp2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        P[d] = (a1 * A[d] + a2 * B[d]) / g;
        rab2 += (A[d] - B[d]) * (A[d] - B[d]);
        rcp2 += (C[d] - P[d]) * (C[d] - P[d]);
    }
    double ax[16], ay[16], az[16];
    a_array(l1, l2, P[0] - A[0], P[0] - B[0], P[0] - C[0], g, ax);
    a_array(m1, m2, P[1] - A[1], P[1] - B[1], P[1] - C[1], g, ay);
    a_array(n1, n2, P[2] - A[2], P[2] - B[2], P[2] - C[2], g, az);
    double sum = 0.0;
    for (int i = 0; i <= l1 + l2; ++i)
        for (int j = 0; j <= m1 + m2; ++j)
            for (int k = 0; k <= n1 + n2; ++k)
                sum += ax[i] * ay[j] * az[k] * orc_fgamma(i + j + k, rcp2 * g);
    return -2.0 * ORC_PI_TRUNC / g * exp(-a1 * a2 * rab2 / g) * sum;
}

/* S, T and V (sum over nuclei), DFT::construct_matrices dft.cpp:184-199;
 * CGF contractions integrals.cpp:43-59, 77-93, 149-164. */
void orc_one_electron(const orc_t *o, double *S, double *T, double *Vn)
{
    const int nbf = o->nbf;
    #pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < nbf; ++i)
        for (int j = i; j < nbf; ++j) {
            const int *qi = o->bf_lmn + 3 * i, *qj = o->bf_lmn + 3 * j;
            const double *A = o->bf_xyz + 3 * i, *B = o->bf_xyz + 3 * j;
            double s = 0.0, t = 0.0, v = 0.0;
            for (int k = o->bf_off[i]; k < o->bf_off[i + 1]; ++k)
                for (int l = o->bf_off[j]; l < o->bf_off[j + 1]; ++l) {
                    double pre = o->pn[k] * o->pn[l] * o->pc[k] * o->pc[l];
                    s += pre * ovl_prim(o->pa[k], qi[0], qi[1], qi[2], A, o->pa[l], qj[0], qj[1], qj[2], B);
                    t += pre * kin_prim(o->pa[k], qi[0], qi[1], qi[2], A, o->pa[l], qj[0], qj[1], qj[2], B);
                }
            for (int c = 0; c < o->natoms; ++c) {
                double vs = 0.0;
                for (int k = o->bf_off[i]; k < o->bf_off[i + 1]; ++k)
                    for (int l = o->bf_off[j]; l < o->bf_off[j + 1]; ++l)
                        vs += o->pn[k] * o->pn[l] * o->pc[k] * o->pc[l] *
                              nuc_prim(A, qi[0], qi[1], qi[2], o->pa[k], B, qj[0], qj[1], qj[2], o->pa[l], o->xyz + 3 * c);
                v += vs * (double)o->Z[c];
            }
            S[i + (size_t)j * nbf] = S[j + (size_t)i * nbf] = s;
            T[i + (size_t)j * nbf] = T[j + (size_t)i * nbf] = t;
            Vn[i + (size_t)j * nbf] = Vn[j + (size_t)i * nbf] = v;
        }
}

/* ---- two-electron integrals: the reference's analytic Hartree path ----
 * Restatement of the Taketa-Huzinaga-O-ohata B-array formula that
 * Integrator::repulsion uses (integrals.cpp:388-466; THO, J. Phys. Soc. Japan
 * 21 (1966) 2313), with the truncated pi of integrals.cpp:394. */
static double fact_ratio2(int a, int b) { return fact(a) / fact(b) / fact(a - 2 * b); }   /* integrals.cpp:466 */

static double tho_fb(int i, int l1, int l2, double p, double a, double b, int r, double g)   /* :455-461 */
{
    return binomial_prefactor(i, l1, l2, p - a, p - b) * fact_ratio2(i, r) * pow(4.0 * g, r - i);
}

static void tho_b_array(int l1, int l2, int l3, int l4, double p, double a, double b, double q, double c,
                        double d, double g1, double g2, double delta, double *arr)   /* :420-452 */
{
    const int imax = l1 + l2 + l3 + l4 + 1;
    for (int i = 0; i < imax; ++i) arr[i] = 0.0;
    for (int i1 = 0; i1 < l1 + l2 + 1; ++i1)
        for (int i2 = 0; i2 < l3 + l4 + 1; ++i2)
            for (int r1 = 0; r1 < i1 / 2 + 1; ++r1)
                for (int r2 = 0; r2 < i2 / 2 + 1; ++r2)
                    for (int u = 0; u < (i1 + i2) / 2 - r1 - r2 + 1; ++u) {
                        const int e = i1 + i2 - 2 * (r1 + r2);
                        const int idx = e - u;
                        arr[idx] += tho_fb(i1, l1, l2, p, a, b, r1, g1) * ((i2 & 1) ? -1.0 : 1.0) *
                                    tho_fb(i2, l3, l4, q, c, d, r2, g2) * ((u & 1) ? -1.0 : 1.0) *
                                    fact_ratio2(e, u) * ipow(q - p, e - 2 * u) / ipow(delta, e - u);
                    }
}

/* primitive (ab|cd) with the norms folded in by the caller (integrals.cpp:388-418) */
static double eri_prim(const double *A, const int *la, double aa, const double *B, const int *lb, double ab,
                       const double *C, const int *lc, double ac, const double *D, const int *ld, double ad)
{
    const double g1 = aa + ab, g2 = ac + ad, delta = 0.25 * (1.0 / g1 + 1.0 / g2);
    double P[3], Q[3], rab2 = 0.0, rcd2 = 0.0, rpq2 = 0.0;
    for (int x = 0; x < 3; ++x) {
        P[x] = (aa * A[x] + ab * B[x]) / g1;
        Q[x] = (ac * C[x] + ad * D[x]) / g2;
        rab2 += (A[x] - B[x]) * (A[x] - B[x]);
        rcd2 += (C[x] - D[x]) * (C[x] - D[x]);
    }
    for (int x = 0; x < 3; ++x) rpq2 += (P[x] - Q[x]) * (P[x] - Q[x]);
    double bx[17], by[17], bz[17];
    tho_b_array(la[0], lb[0], lc[0], ld[0], P[0], A[0], B[0], Q[0], C[0], D[0], g1, g2, delta, bx);
    tho_b_array(la[1], lb[1], lc[1], ld[1], P[1], A[1], B[1], Q[1], C[1], D[1], g1, g2, delta, by);
    tho_b_array(la[2], lb[2], lc[2], ld[2], P[2], A[2], B[2], Q[2], C[2], D[2], g1, g2, delta, bz);
    double sum = 0.0;
    for (int i = 0; i <= la[0] + lb[0] + lc[0] + ld[0]; ++i)
        for (int j = 0; j <= la[1] + lb[1] + lc[1] + ld[1]; ++j)
            for (int k = 0; k <= la[2] + lb[2] + lc[2] + ld[2]; ++k)
                sum += bx[i] * by[j] * bz[k] * orc_fgamma(i + j + k, 0.25 * rpq2 / delta);
    return 2.0 * pow(ORC_PI_TRUNC, 2.5) / (g1 * g2 * sqrt(g1 + g2)) * exp(-aa * ab * rab2 / g1) *
           exp(-ac * ad * rcd2 / g2) * sum;
}

/* contracted (ij|kl), integrals.cpp:185-206 */
double orc_eri(const orc_t *o, int i, int j, int k, int l)
{
    const int f[4] = {i, j, k, l};
    double s = 0.0;
    for (int p = o->bf_off[i]; p < o->bf_off[i + 1]; ++p)
        for (int q = o->bf_off[j]; q < o->bf_off[j + 1]; ++q)
            for (int r = o->bf_off[k]; r < o->bf_off[k + 1]; ++r)
                for (int t = o->bf_off[l]; t < o->bf_off[l + 1]; ++t) {
                    const double pre = o->pc[p] * o->pn[p] * o->pc[q] * o->pn[q] * o->pc[r] * o->pn[r] * o->pc[t] * o->pn[t];
                    s += pre * eri_prim(o->bf_xyz + 3 * f[0], o->bf_lmn + 3 * f[0], o->pa[p],
                                        o->bf_xyz + 3 * f[1], o->bf_lmn + 3 * f[1], o->pa[q],
                                        o->bf_xyz + 3 * f[2], o->bf_lmn + 3 * f[2], o->pa[r],
                                        o->bf_xyz + 3 * f[3], o->bf_lmn + 3 * f[3], o->pa[t]);
                }
    return s;
}

/* every unique integral at the reference's teindex position (dft.cpp:254-288,
 * integrals.cpp:470-486): pairs ij = i(i+1)/2 + j (i >= j), index ij(ij+1)/2 + kl (ij >= kl) */
void orc_eri_list(const orc_t *o, double *out)
{
    const long npair = (long)o->nbf * (o->nbf + 1) / 2;
    #pragma omp parallel for schedule(dynamic)
    for (long ij = 0; ij < npair; ++ij) {
        int i = 0;
        while ((long)(i + 1) * (i + 2) / 2 <= ij) ++i;
        const int j = (int)(ij - (long)i * (i + 1) / 2);
        for (long kl = 0; kl <= ij; ++kl) {
            int k = 0;
            while ((long)(k + 1) * (k + 2) / 2 <= kl) ++k;
            const int l = (int)(kl - (long)k * (k + 1) / 2);
            out[ij * (ij + 1) / 2 + kl] = orc_eri(o, i, j, k, l);
        }
    }
}

/* DFT::calculate_hartree_potential_te_int (dft.cpp:452-477): J_ij = sum_kl P_kl (ij|kl) */
void orc_eri_coulomb(const orc_t *o, const double *P, double *J)
{
    const int n = o->nbf;
    #pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = 0.0;
            for (int k = 0; k < n; ++k)
                for (int l = 0; l <= k; ++l) {
                    const double pkl = (k == l ? 1.0 : 2.0) * P[k + (size_t)l * n];
                    if (pkl != 0.0) s += pkl * orc_eri(o, i, j, k, l);
                }
            J[i + (size_t)j * n] = J[j + (size_t)i * n] = s;
        }
}

/* DFT::calculate_nuclear_repulsion, dft.cpp:235-246 */
double orc_nuclear_repulsion(const orc_t *o)
{
    double e = 0.0;
    for (int i = 0; i < o->natoms; ++i)
        for (int j = i + 1; j < o->natoms; ++j)
            e += o->Z[i] * o->Z[j] / dist3(o->xyz + 3 * i, o->xyz + 3 * j);
    return e;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------ explicit-point XC step */

/*
 * The XC step on explicit points with explicit weights (no atoms, cells or
 * density correction), for the synthetic contraction workload:
 *   phi_i(p)  contracted Cartesian Gaussians about centre bf_centre[i]
 *             (cgf.cpp:49-57, 102-114, 146-154),
 *   rho_p     = 2 phi_p^T P phi_p (gridpoint.cpp:82-84),
 *   e_p, v_p  Slater + VWN (functionals.cpp:24-158, orc_lda_point),
 *   XC_ij     = sum_p w_p v_p phi_i(p) phi_j(p) (dft.cpp:424-432),
 * returning E_xc = sum_p w_p e_p.  rho_out [npts] and XC [nbf][nbf] (full
 * square) may be NULL.  Points run in parallel (OpenMP); the XC sums take
 * every stride-th point and scale by the stride (stride 1: exact).
 */
double orc_points_xc(long npts, const double *xyz, const double *w, int nbf, const double *centres,
                     const int *bf_centre, const int *lmn, const int *nprim, const double *alpha,
                     const double *coef, const double *P, int stride, double *rho_out, double *XC)
{
    int *off = malloc(sizeof(int) * (nbf + 1));
    off[0] = 0;
    for (int i = 0; i < nbf; ++i) off[i + 1] = off[i] + nprim[i];
    double *pcn = malloc(sizeof(double) * off[nbf]);
    for (int i = 0; i < nbf; ++i)
        for (int k = off[i]; k < off[i + 1]; ++k)
            pcn[k] = coef[k] * orc_gto_norm(alpha[k], lmn[3 * i], lmn[3 * i + 1], lmn[3 * i + 2]);
    if (stride < 1) stride = 1;
    const long ns = (npts + stride - 1) / stride;
    double *wv = malloc(sizeof(double) * ns);
    double *phis = malloc(sizeof(double) * (size_t)ns * nbf);
    double exc = 0.0;
    #pragma omp parallel for schedule(static) reduction(+ : exc)
    for (long s = 0; s < ns; ++s) {
        const long p = s * stride;
        double *phi = phis + (size_t)s * nbf;
        for (int i = 0; i < nbf; ++i) {
            const double *c = centres + 3 * bf_centre[i];
            const int *q = lmn + 3 * i;
            double dx = xyz[3 * p] - c[0], dy = xyz[3 * p + 1] - c[1], dz = xyz[3 * p + 2] - c[2];
            double r2 = dx * dx + dy * dy + dz * dz, v = 0.0;
            for (int k = off[i]; k < off[i + 1]; ++k)
                v += pcn[k] * ipow(dx, q[0]) * ipow(dy, q[1]) * ipow(dz, q[2]) * exp(-alpha[k] * r2);
            phi[i] = v;
        }
        double rho = 0.0;
        for (int i = 0; i < nbf; ++i) {
            double t = 0.0;
            for (int j = 0; j < nbf; ++j) t += P[(size_t)i * nbf + j] * phi[j];
            rho += phi[i] * t;
        }
        rho *= 2.0;
        if (rho_out) rho_out[p] = rho;
        double e, v;
        orc_lda_point(rho, &e, &v);
        exc += w[p] * e * stride;
        wv[s] = w[p] * v * stride;
    }
    if (XC) {
        #pragma omp parallel for schedule(dynamic)
        for (int i = 0; i < nbf; ++i)
            for (int j = i; j < nbf; ++j) {
                double sum = 0.0;
                for (long s = 0; s < ns; ++s) sum += wv[s] * phis[(size_t)s * nbf + i] * phis[(size_t)s * nbf + j];
                XC[(size_t)i * nbf + j] = sum;
                XC[(size_t)j * nbf + i] = sum;
            }
    }
    free(phis);
    free(wv);
    free(pcn);
    free(off);
    return exc;
}

/* ------------------------------------------------ atom-cell shards
 * The same build split by fuzzy cell (MolecularGrid keeps one AtomicGrid per
 * atom and sums their J blocks, moleculargrid.cpp:336-389), for checking the
 * exchange pattern of a sharded build on CPU ranks: each rank holds the cells
 * [c0, c0 + nc) and, between the calls below, the ranks exchange
 *   (1) the sum of w rho over all cells (all-reduce), for the correction factor
 *       of moleculargrid.cpp:132-146;
 *   (2) every cell's spline data (all-gather), for the cross-atom potential of
 *       moleculargrid.cpp:342-380;
 *   (3) J, XC and the energies (all-reduce). */

/* rho on the points of cells [c0, c0 + nc); returns their sum of w rho */
double orc_shard_density(orc_t *o, const double *P, int c0, int nc)
{
    const int nbf = o->nbf;
    const size_t per = (size_t)o->nrad * o->nang, p0 = (size_t)c0 * per, p1 = (size_t)(c0 + nc) * per;
    #pragma omp parallel
    {
        double *t = malloc(sizeof(double) * nbf);
        #pragma omp for schedule(static)
        for (long i = (long)p0; i < (long)p1; ++i) {
            const double *f = o->phi + (size_t)i * nbf;
            for (int r = 0; r < nbf; ++r) {
                double s = 0.0;
                for (int c = 0; c < nbf; ++c) s += P[r + (size_t)c * nbf] * f[c];
                t[r] = s;
            }
            double d = 0.0;
            for (int r = 0; r < nbf; ++r) d += f[r] * t[r];
            o->rho[i] = 2.0 * d;
        }
        free(t);
    }
    double s = 0.0;
    for (int a = c0; a < c0 + nc; ++a) s += atom_density(o, a);
    return s;
}

/* doubles of spline data per cell: ordinates [nlm][nrad], coefficients [nlm][nrad-1][4] */
long orc_shard_blob_doubles(const orc_t *o)
{
    return (long)o->nlm * o->nrad + (long)o->nlm * (o->nrad - 1) * 4;
}

/* correction factor cf = sum(Z over every atom) / total, applied to the
 * cells' rho; then rho_lm, the Poisson solve, the own-cell potential and the
 * splines of those cells; their spline data into blob [nc][blob doubles] */
void orc_shard_multipoles(orc_t *o, double total, int c0, int nc, double *blob)
{
    double charge = 0.0;
    for (int a = 0; a < o->natoms; ++a) charge += o->Z[a];
    const double cf = charge / total;
    const size_t per = (size_t)o->nrad * o->nang;
    for (size_t i = (size_t)c0 * per; i < (size_t)(c0 + nc) * per; ++i) o->rho[i] *= cf;
    const size_t ny = (size_t)o->nlm * o->nrad, nsc = (size_t)o->nlm * (o->nrad - 1) * 4;
    for (int a = c0; a < c0 + nc; ++a) {
        calc_rho_lm(o, a);
        calc_U_lm(o, a);
        double *b = blob + (size_t)(a - c0) * (ny + nsc);
        memcpy(b, o->sy + (size_t)a * ny, sizeof(double) * ny);
        memcpy(b + ny, o->sc + (size_t)a * nsc, sizeof(double) * nsc);
    }
}

/* with every cell's spline data (blob_all [natoms][blob doubles]): the total
 * potential on the cells' points, their J block (atomicgrid.cpp:471-488), their
 * part of XC and E_xc (dft.cpp:394-433); scal = {E_xc, sum w rho, 2 tr(P J_part)} */
void orc_shard_finish(orc_t *o, const double *blob_all, const double *P, int c0, int nc, double *J, double *XC,
                      double *scal)
{
    const int N = o->nrad, nlm = o->nlm, nang = o->nang, nbf = o->nbf;
    const size_t ny = (size_t)nlm * N, nsc = (size_t)nlm * (N - 1) * 4;
    for (int a = 0; a < o->natoms; ++a) {
        memcpy(o->sy + (size_t)a * ny, blob_all + (size_t)a * (ny + nsc), sizeof(double) * ny);
        memcpy(o->sc + (size_t)a * nsc, blob_all + (size_t)a * (ny + nsc) + ny, sizeof(double) * nsc);
    }
    for (int i = c0; i < c0 + nc; ++i) {
        size_t base = (size_t)i * N * nang;
        #pragma omp parallel for schedule(static)
        for (long j = 0; j < (long)N * nang; ++j) {
            double V = 0.0;
            const double *pp = o->pos + 3 * (base + j);
            for (int k = 0; k < o->natoms; ++k) {
                if (i == k) { V += o->Vown[base + j]; continue; }
                int lm = 0;
                for (int l = 0; l <= o->lmax; ++l)
                    for (int m = -l; m <= l; ++m) {
                        double d[3] = {pp[0] - o->xyz[3 * k], pp[1] - o->xyz[3 * k + 1], pp[2] - o->xyz[3 * k + 2]};
                        double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                        double y = ylm_dir(l, m, d);
                        const double *sy = o->sy + ((size_t)k * nlm + lm) * N;
                        const double *sc = o->sc + ((size_t)k * nlm + lm) * (N - 1) * 4;
                        V += 1.0 / r * y * spline_eval(N, o->sx, sy, sc, r);
                        lm++;
                    }
            }
            o->V[base + j] = V;
        }
    }
    memset(J, 0, sizeof(double) * nbf * nbf);
    memset(XC, 0, sizeof(double) * nbf * nbf);
    const size_t p0 = (size_t)c0 * N * nang, p1 = (size_t)(c0 + nc) * N * nang;
    double exc = 0.0, nel = 0.0;
    double *wv = malloc(sizeof(double) * (p1 - p0));
    for (size_t p = p0; p < p1; ++p) {
        double e, v;
        orc_lda_point(o->rho[p], &e, &v);
        exc += o->w[p] * e;
        nel += o->w[p] * o->rho[p];
        wv[p - p0] = o->w[p] * v;
    }
    #pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < nbf; ++i)
        for (int j = i; j < nbf; ++j) {
            double sj = 0.0, sx = 0.0;
            for (size_t p = p0; p < p1; ++p) {
                const double f = o->phi[p * nbf + i] * o->phi[p * nbf + j];
                sj += o->w[p] * o->V[p] * f;
                sx += wv[p - p0] * f;
            }
            J[i + (size_t)j * nbf] = J[j + (size_t)i * nbf] = 0.5 * sj;
            XC[i + (size_t)j * nbf] = XC[j + (size_t)i * nbf] = sx;
        }
    free(wv);
    double ej = 0.0;
    for (int i = 0; i < nbf; ++i)
        for (int j = 0; j < nbf; ++j) ej += P[i + (size_t)j * nbf] * J[j + (size_t)i * nbf];
    scal[0] = exc;
    scal[1] = nel;
    scal[2] = 2.0 * ej;
}
