/*
 * CPU oracle for the batched tridiagonal solve.  TEST INFRASTRUCTURE ONLY:
 * loaded by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py as the checker of the CUDA library, never by the library itself.
 * See oracle.h for the interface and the reference lines each solver follows.
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp).  The same
 * source builds on x86-64 and AArch64 and gives the same bits on both: only
 * IEEE-754 +,-,*,/ and fma() are used, with no contraction.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

static int g_threads = 0;

void orc_set_threads(int n) { g_threads = n; }

int orc_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

#define T float
#define SFX f32
#include "oracle_body.inc"
#include "oracle_block2.inc"
#undef T
#undef SFX

#define T double
#define SFX f64
#include "oracle_body.inc"
#include "oracle_block2.inc"
#undef T
#undef SFX

/* Pivoted LU of one system (the elimination of orc_gtsv without a right-hand
 * side): l = multipliers, u0/u1/u2 = diagonal and two super-diagonals of U,
 * piv[i] = 1 when rows i and i+1 were interchanged at step i. */
static int lu_factor(const double *a, const double *b, const double *c, int n,
                     double *l, double *u0, double *u1, double *u2, unsigned char *piv) {
    for (int i = 0; i < n; ++i) { u0[i] = b[i]; u1[i] = (i + 1 < n) ? c[i] : 0; u2[i] = 0; l[i] = 0; piv[i] = 0; }
    double sub_next = n > 1 ? a[1] : 0; /* sub-diagonal entry of row i+1 */
    for (int i = 0; i + 1 < n; ++i) {
        double sub = sub_next;
        sub_next = (i + 2 < n) ? a[i + 2] : 0;
        if (fabs(u0[i]) >= fabs(sub)) {
            if (u0[i] == 0) return i + 1;
            double m = sub / u0[i];
            u0[i + 1] = u0[i + 1] - m * u1[i];
            l[i] = m;
        } else {
            double m = u0[i] / sub;
            double t = u0[i + 1];
            u0[i] = sub;
            u0[i + 1] = u1[i] - m * t;
            if (i + 2 < n) { u2[i] = u1[i + 1]; u1[i + 1] = 0 - m * u1[i + 1]; }
            u1[i] = t;
            l[i] = m;
            piv[i] = 1;
        }
    }
    if (u0[n - 1] == 0) return n;
    return 0;
}

int orc_adjoint_f64(const double *A, const double *B, const double *C, const double *X,
                    const double *XB, double *GA, double *GB, double *GC, double *GD,
                    int n, int batch) {
    if (n <= 0 || batch <= 0) return 0;
    int info = 0;
#pragma omp parallel num_threads(orc_get_threads())
    {
        double *w = (double *)malloc(sizeof(double) * 5 * (size_t)n);
        unsigned char *piv = (unsigned char *)malloc((size_t)n);
#pragma omp for schedule(static)
        for (int j = 0; j < batch; ++j) {
            if (!w || !piv) continue;
            const size_t o = (size_t)j * n;
            double *l = w, *u0 = w + n, *u1 = w + 2 * (size_t)n, *u2 = w + 3 * (size_t)n, *z = w + 4 * (size_t)n;
            int bad = lu_factor(A + o, B + o, C + o, n, l, u0, u1, u2, piv);
            if (bad) {
#pragma omp critical
                { if (info == 0) info = bad; }
                continue;
            }
            /* U^T z = xbar (forward substitution) */
            for (int i = 0; i < n; ++i) {
                double s = XB[o + i];
                if (i >= 1) s = s - u1[i - 1] * z[i - 1];
                if (i >= 2) s = s - u2[i - 2] * z[i - 2];
                z[i] = s / u0[i];
            }
            /* lambda = E_0^T ... E_{n-2}^T z */
            for (int i = n - 2; i >= 0; --i) {
                z[i] = z[i] - l[i] * z[i + 1];
                if (piv[i]) { double t = z[i]; z[i] = z[i + 1]; z[i + 1] = t; }
            }
            const double *x = X + o;
            for (int i = 0; i < n; ++i) {
                GD[o + i] = z[i];
                GA[o + i] = (i > 0) ? -z[i] * x[i - 1] : 0.0;
                GB[o + i] = -z[i] * x[i];
                GC[o + i] = (i + 1 < n) ? -z[i] * x[i + 1] : 0.0;
            }
        }
        free(w);
        free(piv);
    }
    return info;
}

/* s + t with its rounding error (Knuth's TwoSum). */
static inline void two_sum(double s, double t, double *hi, double *lo) {
    double h = s + t;
    double bb = h - s;
    *hi = h;
    *lo = (s - (h - bb)) + (t - bb);
}

/* d - (a*xm + b*x0 + c*xp) with a compensated sum (Ogita-Rump-Oishi Dot2). */
static inline double resid1(double a, double b, double c, double d, double xm, double x0, double xp) {
    double s = d, err = 0, hi, lo;
    double coef[3] = {a, b, c}, xs[3] = {xm, x0, xp};
    for (int k = 0; k < 3; ++k) {
        double p = coef[k] * xs[k];
        double pe = fma(coef[k], xs[k], -p);
        two_sum(s, -p, &hi, &lo);
        s = hi;
        err += lo - pe;
    }
    return s + err;
}

void orc_residual_f64(const double *A, const double *B, const double *C, const double *D,
                      const double *X, double *R, int n, int batch) {
    if (n <= 0 || batch <= 0) return;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int j = 0; j < batch; ++j) {
        const size_t o = (size_t)j * n;
        for (int i = 0; i < n; ++i) {
            double xm = i > 0 ? X[o + i - 1] : 0.0, xp = i + 1 < n ? X[o + i + 1] : 0.0;
            double a = i > 0 ? A[o + i] : 0.0, c = i + 1 < n ? C[o + i] : 0.0;
            R[o + i] = resid1(a, B[o + i], c, D[o + i], xm, X[o + i], xp);
        }
    }
}

double orc_backward_error_f64(const double *A, const double *B, const double *C, const double *D,
                              const double *X, double *ETA, int n, int batch) {
    if (n <= 0 || batch <= 0) return 0.0;
    double worst = 0.0;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads()) reduction(max : worst)
    for (int j = 0; j < batch; ++j) {
        const size_t o = (size_t)j * n;
        double rn = 0, an = 0, xn = 0, dn = 0;
        int nan = 0;
        for (int i = 0; i < n; ++i) {
            double xm = i > 0 ? X[o + i - 1] : 0.0, xp = i + 1 < n ? X[o + i + 1] : 0.0;
            double a = i > 0 ? A[o + i] : 0.0, c = i + 1 < n ? C[o + i] : 0.0;
            double r = resid1(a, B[o + i], c, D[o + i], xm, X[o + i], xp);
            if (r != r || X[o + i] != X[o + i]) nan = 1;
            rn = fmax(rn, fabs(r));
            an = fmax(an, fabs(a) + fabs(B[o + i]) + fabs(c));
            xn = fmax(xn, fabs(X[o + i]));
            dn = fmax(dn, fabs(D[o + i]));
        }
        double den = an * xn + dn;
        double eta = nan ? INFINITY : (den > 0 ? rn / den : (rn > 0 ? INFINITY : 0.0));
        if (ETA) ETA[j] = eta;
        if (eta > worst) worst = eta;
    }
    return worst;
}

int orc_check_f64(const double *x, const double *xref, int size, double *stats) {
    double sum = 0, sq = 0, mx = 0;
    int arg = 0, have_nan = 0;
    for (int i = 0; i < size; ++i) {
        double e = fabs(x[i] - xref[i]);
        if (e != e) {
            if (!have_nan) { have_nan = 1; arg = i; }
            mx = e;
            sum += e;
            sq += e;
            continue;
        }
        sum += e;
        sq += e * e;
        if (!have_nan && e >= mx) { mx = e; arg = i; }
    }
    stats[0] = size > 0 ? sum / size : 0;
    stats[1] = size > 0 ? sqrt(sq / size) : 0;
    stats[2] = mx;
    return arg;
}
