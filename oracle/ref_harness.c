/*
 * ORACLE (test infrastructure only; x86-64 only; needs the reference tree).
 *
 * Host-side support that lets the reference's shipped, closed gfortran
 * libraries (FDFK2D lib_gnu/libHybrid.so, libPML.so, libFK3D.so) run as a
 * black box, the same way the reference executable would link them
 * (src/Makefile:106-125: -lHybrid -lPML -lFK3D -llapack -lblas -lfftw3).
 * The libraries import symbols that the reference executable or third-party
 * libraries normally provide; this file provides them:
 *
 *   - the FD operators diff1_, diffx1_, diff{x2,z2,xz,zx}_{reg,pml}_ (from
 *     fdfk_ops.c, a restatement of src/Submain.f90:167-1109);
 *   - the legacy FFTW3 Fortran interface dfftw_plan_dft_1d_,
 *     dfftw_execute_dft_, dfftw_execute_, dfftw_destroy_plan_ (FFTW 3.x,
 *     version unpinned in the reference): an unnormalised complex DFT of any
 *     length, X[k] = sum_n x[n] exp(sign * 2 pi i n k / N), computed with a
 *     mixed-radix / Bluestein FFT written here;
 *   - LAPACK zgetrf_ / zgetrs_ (LU with partial pivoting of a complex double
 *     matrix and the matching triangular solves; reference LAPACK semantics).
 *
 * It also records which operators the libraries call, with which arrays, so
 * tests can pin the restated time step against the shipped one.
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fdfk_ops.h"

/* ---------------------------------------------------------------------- */
/* Operator call trace                                                    */
/* ---------------------------------------------------------------------- */
#define TRACE_MAX 256
typedef struct {
    char name[16];
    int norder, nx, nz, npml, izt;
    const float *mat, *u;
    float *out;
    long dump_off; /* offset into the dump buffer: mat, u, out copies (each ncell floats) */
} trace_rec_t;

static int g_trace_on = 0;
static int g_trace_n = 0;
static trace_rec_t g_trace[TRACE_MAX];
static float *g_dump = NULL;
static long g_dump_cap = 0, g_dump_len = 0;
static long g_diff1_calls = 0, g_diffx1_calls = 0, g_point_n = 0;

void fdfk_ref_trace_enable(int on, long dump_cap_floats)
{
    g_trace_on = on;
    g_trace_n = 0;
    g_dump_len = 0;
    g_diff1_calls = 0;
    g_diffx1_calls = 0;
    g_point_n = 0;
    if (dump_cap_floats > g_dump_cap) {
        free(g_dump);
        g_dump = (float *)malloc(sizeof(float) * (size_t)dump_cap_floats);
        g_dump_cap = g_dump ? dump_cap_floats : 0;
    }
}

int fdfk_ref_trace_count(void) { return g_trace_n; }
const trace_rec_t *fdfk_ref_trace_get(int i) { return (i >= 0 && i < g_trace_n) ? &g_trace[i] : NULL; }
const float *fdfk_ref_trace_dump(void) { return g_dump; }
long fdfk_ref_trace_diff1_calls(void) { return g_diff1_calls; }
long fdfk_ref_trace_diffx1_calls(void) { return g_diffx1_calls; }
int fdfk_ref_trace_rec_size(void) { return (int)sizeof(trace_rec_t); }

void fdfk_trace_hook(const char *name, int norder, int nx, int nz, int npml, int izt,
                     const float *mat, const float *u, float *out)
{
    if (!g_trace_on || g_trace_n >= TRACE_MAX) return;
    trace_rec_t *r = &g_trace[g_trace_n];
    memset(r, 0, sizeof(*r));
    strncpy(r->name, name, sizeof(r->name) - 1);
    r->norder = norder; r->nx = nx; r->nz = nz; r->npml = npml; r->izt = izt;
    r->mat = mat; r->u = u; r->out = out;
    long ncell = (long)(nz + npml - izt + 1) * (long)(nx + 2 * npml);
    if (g_dump && g_dump_len + 3 * ncell <= g_dump_cap) {
        r->dump_off = g_dump_len;
        memcpy(g_dump + g_dump_len, mat, sizeof(float) * ncell);
        memcpy(g_dump + g_dump_len + ncell, u, sizeof(float) * ncell);
        g_dump_len += 3 * ncell;
    } else {
        r->dump_off = -1;
    }
}

void fdfk_trace_post(const char *name, int nx, int nz, int npml, int izt, float *out)
{
    (void)name;
    if (!g_trace_on || g_trace_n >= TRACE_MAX) return;
    trace_rec_t *r = &g_trace[g_trace_n];
    long ncell = (long)(nz + npml - izt + 1) * (long)(nx + 2 * npml);
    if (r->dump_off >= 0) memcpy(g_dump + r->dump_off + 2 * ncell, out, sizeof(float) * ncell);
    g_trace_n++;
}

static float *g_rows;
static long g_rows_max, g_row_len;
typedef struct {
    int which, ix, iz, dire;
    float d, val;
    const void *caller;
    const float *u;
} point_rec_t;
#define POINT_MAX 200000
static point_rec_t g_points[POINT_MAX];

void fdfk_trace_point(int which, const void *caller, int ix, int iz, int dire, float d, const float *u, float val)
{
    if (!g_trace_on) return;
    long i1 = __atomic_fetch_add(which == 1 ? &g_diff1_calls : &g_diffx1_calls, 1, __ATOMIC_RELAXED);
    (void)i1;
    long k = __atomic_fetch_add(&g_point_n, 1, __ATOMIC_RELAXED);
    if (k < POINT_MAX) {
        point_rec_t *p = &g_points[k];
        p->which = which; p->ix = ix; p->iz = iz; p->dire = dire; p->d = d; p->val = val;
        p->caller = caller; p->u = u;
        if (g_rows && k < g_rows_max) {
            /* copy the operand: a row (diffx1) or the full grid (diff1, first sight only) */
            memcpy(g_rows + (size_t)k * g_row_len, u, sizeof(float) * (size_t)(which == 2 ? g_row_len : 0));
        }
    }
}
void fdfk_ref_point_rows(long maxrec, long row_len)
{
    free(g_rows);
    g_rows = maxrec > 0 ? (float *)calloc((size_t)maxrec * (size_t)row_len, sizeof(float)) : NULL;
    g_rows_max = maxrec; g_row_len = row_len;
}
const float *fdfk_ref_point_row_data(void) { return g_rows; }
long fdfk_ref_point_count(void) { return g_point_n < POINT_MAX ? g_point_n : POINT_MAX; }
const point_rec_t *fdfk_ref_points(void) { return g_points; }
int fdfk_ref_point_rec_size(void) { return (int)sizeof(point_rec_t); }
/* Which loaded object contains an address (0: harness, else a dladdr name index). */
const char *fdfk_ref_object_of(const void *addr)
{
    Dl_info info;
    if (dladdr(addr, &info) && info.dli_fname) return info.dli_fname;
    return "?";
}

/* ---------------------------------------------------------------------- */
/* FFTW3 legacy Fortran interface (complex double, 1-D)                   */
/* ---------------------------------------------------------------------- */
typedef struct {
    int n, sign;
    double complex *in, *out;
    double complex *tw;   /* twiddles exp(sign 2 pi i k / n), k < n */
    double complex *work; /* scratch of n */
    /* Bluestein (used when n has a prime factor > 7) */
    int m;
    double complex *chirp, *bfft, *a;
    double complex *twm, *workm;
} fplan_t;

static void fft_rec(int n, int sign_unused, const double complex *x, int stride, double complex *y,
                    const double complex *tw, int twstride, double complex *work)
{
    (void)sign_unused;
    if (n == 1) { y[0] = x[0]; return; }
    int p = 0;
    for (int f = 2; f <= 7; ++f)
        if (n % f == 0) { p = f; break; }
    if (p == 0) p = n; /* direct DFT for the remaining factor */
    int m = n / p;
    /* sub-transforms of the decimated sequences */
    for (int r = 0; r < p; ++r) fft_rec(m, 0, x + r * stride, stride * p, work + r * m, tw, twstride * p, y);
    /* combine */
    for (int k = 0; k < m; ++k)
        for (int q = 0; q < p; ++q) {
            double complex s = 0;
            int kk = k + q * m;
            for (int r = 0; r < p; ++r) {
                long e = ((long)r * kk) % n;
                s += work[r * m + k] * tw[e * twstride];
            }
            y[kk] = s;
        }
}

static void fft_exec_small(const fplan_t *p, int n, const double complex *tw, double complex *work,
                           const double complex *x, double complex *y)
{
    /* y must not alias x; work has n entries; tw has n entries at stride 1 */
    double complex *tmp = (double complex *)malloc(sizeof(double complex) * (size_t)n);
    fft_rec(n, p->sign, x, 1, y, tw, 1, tmp);
    (void)work;
    free(tmp);
}

static int smooth(int n)
{
    for (int f = 2; f <= 7; ++f)
        while (n % f == 0) n /= f;
    return n == 1;
}

/* FFT / LU call log (observation only) */
#define FLOG_MAX 4096
typedef struct { int kind, n, sign; long off_in, off_out; } flog_t;
static flog_t g_flog[FLOG_MAX];
static int g_flog_n = 0, g_flog_on = 0;
static double complex *g_fdata = NULL;
static long g_fdata_len = 0, g_fdata_cap = 0;
static long g_plan_calls = 0, g_exec_calls = 0, g_lu_calls = 0, g_lus_calls = 0;
void fdfk_ref_flog(int on, long cap)
{
    g_flog_on = on; g_flog_n = 0; g_fdata_len = 0;
    g_plan_calls = g_exec_calls = g_lu_calls = g_lus_calls = 0;
    if (cap > g_fdata_cap) { free(g_fdata); g_fdata = (double complex *)malloc(sizeof(double complex) * cap); g_fdata_cap = cap; }
}
int fdfk_ref_flog_count(void) { return g_flog_n; }
const flog_t *fdfk_ref_flog_get(int i) { return &g_flog[i]; }
const double complex *fdfk_ref_flog_data(void) { return g_fdata; }
void fdfk_ref_flog_counts(long *out) { out[0] = g_plan_calls; out[1] = g_exec_calls; out[2] = g_lu_calls; out[3] = g_lus_calls; }
static void flog_add(int kind, int n, int sign, const double complex *in, const double complex *out, int nin, int nout)
{
    if (!g_flog_on) return;
    int k = __atomic_fetch_add(&g_flog_n, 1, __ATOMIC_RELAXED);
    if (k >= FLOG_MAX) return;
    long need = nin + nout;
    long off = __atomic_fetch_add(&g_fdata_len, need, __ATOMIC_RELAXED);
    flog_t *r = &g_flog[k];
    r->kind = kind; r->n = n; r->sign = sign; r->off_in = -1; r->off_out = -1;
    if (off + need <= g_fdata_cap) {
        if (nin) { memcpy(g_fdata + off, in, sizeof(double complex) * nin); r->off_in = off; }
        if (nout) { memcpy(g_fdata + off + nin, out, sizeof(double complex) * nout); r->off_out = off + nin; }
    }
}

void dfftw_plan_dft_1d_(int64_t *plan, const int *n, double complex *in, double complex *out, const int *sign,
                        const int *flags)
{
    if (g_flog_on) __atomic_fetch_add(&g_plan_calls, 1, __ATOMIC_RELAXED);
    (void)flags;
    fplan_t *p = (fplan_t *)calloc(1, sizeof(fplan_t));
    p->n = *n; p->sign = *sign; p->in = in; p->out = out;
    int N = p->n;
    p->tw = (double complex *)malloc(sizeof(double complex) * (size_t)N);
    for (int k = 0; k < N; ++k) p->tw[k] = cexp((double)p->sign * 2.0 * M_PI * I * (double)k / (double)N);
    if (!smooth(N)) {
        int m = 1;
        while (m < 2 * N - 1) m *= 2;
        p->m = m;
        p->chirp = (double complex *)malloc(sizeof(double complex) * (size_t)N);
        for (long k = 0; k < N; ++k) {
            long kk = (k * k) % (2L * N);
            p->chirp[k] = cexp((double)p->sign * M_PI * I * (double)kk / (double)N);
        }
        p->twm = (double complex *)malloc(sizeof(double complex) * (size_t)m);
        for (int k = 0; k < m; ++k) p->twm[k] = cexp(-2.0 * M_PI * I * (double)k / (double)m);
        p->bfft = (double complex *)calloc((size_t)m, sizeof(double complex));
        double complex *b = (double complex *)calloc((size_t)m, sizeof(double complex));
        b[0] = conj(p->chirp[0]);
        for (int k = 1; k < N; ++k) b[k] = b[m - k] = conj(p->chirp[k]);
        fplan_t q = {0};
        q.sign = -1;
        fft_exec_small(&q, m, p->twm, NULL, b, p->bfft);
        free(b);
        p->a = (double complex *)malloc(sizeof(double complex) * (size_t)m);
        p->workm = (double complex *)malloc(sizeof(double complex) * (size_t)m);
    }
    *plan = (int64_t)(intptr_t)p;
}

static void plan_exec(const fplan_t *p, const double complex *x, double complex *y)
{
    int N = p->n;
    if (!p->m) {
        double complex *t = (double complex *)malloc(sizeof(double complex) * (size_t)N);
        fft_exec_small(p, N, p->tw, NULL, x, t);
        memcpy(y, t, sizeof(double complex) * (size_t)N);
        free(t);
        return;
    }
    int m = p->m;
    double complex *a = (double complex *)calloc((size_t)m, sizeof(double complex));
    double complex *A = (double complex *)malloc(sizeof(double complex) * (size_t)m);
    for (int k = 0; k < N; ++k) a[k] = x[k] * p->chirp[k];
    fplan_t q = {0};
    q.sign = -1;
    fft_exec_small(&q, m, p->twm, NULL, a, A);
    for (int k = 0; k < m; ++k) A[k] *= p->bfft[k];
    /* inverse transform via conjugation */
    for (int k = 0; k < m; ++k) A[k] = conj(A[k]);
    fft_exec_small(&q, m, p->twm, NULL, A, a);
    for (int k = 0; k < N; ++k) y[k] = conj(a[k]) / (double)m * p->chirp[k];
    free(a);
    free(A);
}

void dfftw_execute_(const int64_t *plan)
{
    const fplan_t *p = (const fplan_t *)(intptr_t)*plan;
    double complex *tmp = g_flog_on ? (double complex *)malloc(sizeof(double complex) * p->n) : NULL;
    if (tmp) memcpy(tmp, p->in, sizeof(double complex) * p->n);
    plan_exec(p, p->in, p->out);
    if (g_flog_on) { __atomic_fetch_add(&g_exec_calls, 1, __ATOMIC_RELAXED); flog_add(1, p->n, p->sign, tmp, p->out, p->n, p->n); }
    free(tmp);
}

void dfftw_execute_dft_(const int64_t *plan, double complex *in, double complex *out)
{
    const fplan_t *p = (const fplan_t *)(intptr_t)*plan;
    double complex *tmp = g_flog_on ? (double complex *)malloc(sizeof(double complex) * p->n) : NULL;
    if (tmp) memcpy(tmp, in, sizeof(double complex) * p->n);
    plan_exec(p, in, out);
    if (g_flog_on) { __atomic_fetch_add(&g_exec_calls, 1, __ATOMIC_RELAXED); flog_add(2, p->n, p->sign, tmp, out, p->n, p->n); }
    free(tmp);
}

void dfftw_destroy_plan_(int64_t *plan)
{
    fplan_t *p = (fplan_t *)(intptr_t)*plan;
    if (!p) return;
    free(p->tw); free(p->chirp); free(p->bfft); free(p->a); free(p->twm); free(p->workm);
    free(p);
    *plan = 0;
}

/* ---------------------------------------------------------------------- */
/* LAPACK zgetrf_ / zgetrs_ (column-major, 1-based pivots)                */
/* ---------------------------------------------------------------------- */
static double cabs1(double complex z) { return fabs(creal(z)) + fabs(cimag(z)); }

void zgetrf_(const int *m_, const int *n_, double complex *a, const int *lda_, int *ipiv, int *info)
{
    int m = *m_, n = *n_, lda = *lda_;
    if (g_flog_on) { __atomic_fetch_add(&g_lu_calls, 1, __ATOMIC_RELAXED); flog_add(3, n, m, a, NULL, lda * n, 0); }
    *info = 0;
    int mn = m < n ? m : n;
    for (int j = 0; j < mn; ++j) {
        int p = j;
        double best = cabs1(a[j + (size_t)j * lda]);
        for (int i = j + 1; i < m; ++i) {
            double v = cabs1(a[i + (size_t)j * lda]);
            if (v > best) { best = v; p = i; }
        }
        ipiv[j] = p + 1;
        if (a[p + (size_t)j * lda] != 0.0) {
            if (p != j)
                for (int k = 0; k < n; ++k) {
                    double complex t = a[j + (size_t)k * lda];
                    a[j + (size_t)k * lda] = a[p + (size_t)k * lda];
                    a[p + (size_t)k * lda] = t;
                }
            double complex r = 1.0 / a[j + (size_t)j * lda];
            for (int i = j + 1; i < m; ++i) a[i + (size_t)j * lda] *= r;
        } else if (*info == 0) {
            *info = j + 1;
        }
        for (int k = j + 1; k < n; ++k) {
            double complex t = a[j + (size_t)k * lda];
            if (t != 0.0)
                for (int i = j + 1; i < m; ++i) a[i + (size_t)k * lda] -= a[i + (size_t)j * lda] * t;
        }
    }
}

void zgetrs_(const char *trans, const int *n_, const int *nrhs_, const double complex *a, const int *lda_,
             const int *ipiv, double complex *b, const int *ldb_, int *info, long trans_len)
{
    (void)trans_len;
    int n = *n_, nrhs = *nrhs_, lda = *lda_, ldb = *ldb_;
    *info = 0;
    char t = trans[0];
    if (g_flog_on) { __atomic_fetch_add(&g_lus_calls, 1, __ATOMIC_RELAXED); flog_add(4, n, nrhs * 100 + (int)t, b, NULL, ldb * nrhs, 0); }
    for (int r = 0; r < nrhs; ++r) {
        double complex *x = b + (size_t)r * ldb;
        if (t == 'N' || t == 'n') {
            for (int i = 0; i < n; ++i) {
                int p = ipiv[i] - 1;
                if (p != i) { double complex s = x[i]; x[i] = x[p]; x[p] = s; }
            }
            for (int j = 0; j < n; ++j)
                for (int i = j + 1; i < n; ++i) x[i] -= a[i + (size_t)j * lda] * x[j];
            for (int j = n - 1; j >= 0; --j) {
                x[j] /= a[j + (size_t)j * lda];
                for (int i = 0; i < j; ++i) x[i] -= a[i + (size_t)j * lda] * x[j];
            }
        } else {
            int cj = (t == 'C' || t == 'c');
            /* solve U^T y = b, then L^T x = y, then undo pivots */
            for (int j = 0; j < n; ++j) {
                double complex s = x[j];
                for (int i = 0; i < j; ++i) s -= (cj ? conj(a[i + (size_t)j * lda]) : a[i + (size_t)j * lda]) * x[i];
                x[j] = s / (cj ? conj(a[j + (size_t)j * lda]) : a[j + (size_t)j * lda]);
            }
            for (int j = n - 1; j >= 0; --j) {
                double complex s = x[j];
                for (int i = j + 1; i < n; ++i) s -= (cj ? conj(a[i + (size_t)j * lda]) : a[i + (size_t)j * lda]) * x[i];
                x[j] = s;
            }
            for (int i = n - 1; i >= 0; --i) {
                int p = ipiv[i] - 1;
                if (p != i) { double complex s = x[i]; x[i] = x[p]; x[p] = s; }
            }
        }
    }
}
