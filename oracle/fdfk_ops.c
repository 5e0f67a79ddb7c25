/*
 * ORACLE (test infrastructure only; never part of the product path).
 *
 * Plain-C restatement of the open-source finite-difference operators of
 * FDFK2D, src/Submain.f90.  Arrays use the reference's Fortran layout and
 * index ranges:
 *
 *   u, mat, out : real(izt:nz+npml, 1-npml:nx+npml), z fastest
 *   coef        : real(8)(1:norder, 1:norder), coef(j, n) for reduced order n
 *
 * The mixed-precision arithmetic follows Fortran's promotion rules exactly:
 * `mysum = mysum + coef(k,n)*(u(a) - u(b))` is a real_t difference, promoted to
 * double, multiplied by the double coefficient, added to the promoted real_t
 * accumulator and rounded back to real_t.
 *
 * Every routine is exported twice: with a trailing underscore and all
 * arguments by reference (the gfortran ABI the shipped libHybrid.so/libPML.so
 * import), and as fdfk_op_* taking values (used by the oracle time loop).
 */
#include "fdfk_ops.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define IMIN(a, b) ((a) < (b) ? (a) : (b))
#define IMAX(a, b) ((a) > (b) ? (a) : (b))

/* Fortran u(iz, ix) on the full grid. */
#define G(a, iz, ix) (a)[(size_t)((iz) - g->izt) + (size_t)((ix) - (1 - g->npml)) * (size_t)g->ldz]
#define COEF(c, j, n) (c)[((j) - 1) + ((n) - 1) * norder]

typedef struct {
    int nx, nz, npml, izt, ldz, ldx;
} grid_t;

static grid_t mkgrid(int nx, int nz, int npml, int izt)
{
    grid_t g;
    g.nx = nx; g.nz = nz; g.npml = npml; g.izt = izt;
    g.ldz = nz + npml - izt + 1;
    g.ldx = nx + 2 * npml;
    return g;
}

static inline real_t acc(real_t s, double c, real_t d)
{
    return (real_t)((double)s + c * (double)d);
}

/* ---------------------------------------------------------------------- */
/* fd_coef0 / fd_coef1 / fd_coef2: src/Submain.f90:1111-1245              */
/* ---------------------------------------------------------------------- */
void fdfk_op_fd_coef0(int norder, double *coef)
{
    memset(coef, 0, sizeof(double) * norder * norder);
    for (int i = 1; i <= norder; ++i)
        for (int j = 1; j <= i; ++j) {
            double t1 = 1.0, t2 = 1.0, t3 = 1.0;
            for (int k = 1; k <= j - 1; ++k) {
                t1 *= (double)((2 * k - 1) * (2 * k - 1));
                t2 *= ((double)((2 * j - 1) * (2 * j - 1)) - (double)((2 * k - 1) * (2 * k - 1)));
            }
            for (int k = j + 1; k <= i; ++k) {
                t1 *= (double)((2 * k - 1) * (2 * k - 1));
                t3 *= ((double)((2 * k - 1) * (2 * k - 1)) - (double)((2 * j - 1) * (2 * j - 1)));
            }
            t1 *= ((j + 1) % 2 == 0) ? 1.0 : -1.0;
            t2 *= (double)(2 * j - 1);
            COEF(coef, j, i) = t1 / t2 / t3;
        }
}

static void fd_coef_collocated(int norder, double *coef, int second)
{
    memset(coef, 0, sizeof(double) * norder * norder);
    for (int i = 1; i <= norder; ++i)
        for (int j = 1; j <= i; ++j) {
            double t1 = 1.0, t2 = 1.0, t3 = 1.0;
            for (int k = 1; k <= j - 1; ++k) {
                t1 *= (double)(k * k);
                t2 *= ((double)(j * j) - (double)(k * k));
            }
            for (int k = j + 1; k <= i; ++k) {
                t1 *= (double)(k * k);
                t3 *= ((double)(k * k) - (double)(j * j));
            }
            t1 *= ((j + 1) % 2 == 0) ? 1.0 : -1.0;
            t2 *= second ? (double)(j * j) : 2.0 * (double)j;
            COEF(coef, j, i) = t1 / t2 / t3;
        }
}

void fdfk_op_fd_coef1(int norder, double *coef) { fd_coef_collocated(norder, coef, 0); }
void fdfk_op_fd_coef2(int norder, double *coef) { fd_coef_collocated(norder, coef, 1); }

/* ---------------------------------------------------------------------- */
/* check_stability: src/Submain.f90:118-164.  Returns dt_stable (real_t).  */
/* ---------------------------------------------------------------------- */
real_t fdfk_op_dt_stable(int nx, int nz, int npml, int izt, int norder, real_t dx, real_t dz,
                        const double *coef2, const real_t *c)
{
    real_t h = dx > dz ? dx : dz;
    real_t cx = (h / dx) * (h / dx);
    real_t cz = (h / dz) * (h / dz);
    double sa = 0.0, s = 0.0;
    for (int j = 1; j <= norder; ++j) {
        sa += fabs(COEF(coef2, j, norder));
        s += COEF(coef2, j, norder);
    }
    real_t cfl = REAL_SQRT((real_t)(2.0 / ((double)(cx + cz) * (sa + s))));
    size_t ncell = (size_t)(nz + npml - izt + 1) * (size_t)(nx + 2 * npml);
    real_t vpmax = 0.0f;
    for (size_t i = 0; i < ncell; ++i) {
        real_t v = REAL_SQRT((c[3 * i + 1] + 2.0f * c[3 * i + 2]) / c[3 * i + 0]);
        if (v > vpmax) vpmax = v;
    }
    return cfl * h / vpmax;
}

/* ---------------------------------------------------------------------- */
/* diff1: src/Submain.f90:167-212 (pointwise collocated 1st derivative)   */
/* ---------------------------------------------------------------------- */
real_t fdfk_op_diff1(int norder, int dire, int nx, int nz, int npml, int izt, int ix, int iz,
                    real_t d, const double *coef, const real_t *u)
{
    grid_t gg = mkgrid(nx, nz, npml, izt), *g = &gg;
    int nox = IMIN(IMIN(ix + npml - 1, nx + npml - ix), norder);
    int noz = IMIN(IMIN(iz - izt, nz + npml - iz), norder);
    int kx = 2 - dire, kz = dire - 1;
    int node = kx * nox + kz * noz;
    real_t s = 0.0f;
    for (int k = 1; k <= node; ++k)
        s = acc(s, COEF(coef, k, node), G(u, iz + kz * k, ix + kx * k) - G(u, iz - kz * k, ix - kx * k));
    return s / d;
}

/* diffx1: src/Submain.f90:215-249 (1st derivative along a 1-D row). */
real_t fdfk_op_diffx1(int norder, int nx, int npml, int ix, real_t dx, const double *coef, const real_t *u)
{
    int no = IMIN(IMIN(ix + npml - 1, nx + npml - ix), norder);
    const real_t *r = u - (1 - npml); /* r[i] == u(i) */
    real_t s = 0.0f;
    for (int k = 1; k <= no; ++k) s = acc(s, COEF(coef, k, no), r[ix + k] - r[ix - k]);
    return s / dx;
}

/* ---------------------------------------------------------------------- */
/* Mixed-derivative operators                                             */
/* ---------------------------------------------------------------------- */

/* diffzx_reg: src/Submain.f90:251-409, active part 352-406. */
void fdfk_op_diffzx_reg(int norder, int nx, int nz, int npml, int izt, real_t dx, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out)
{
    grid_t gg = mkgrid(nx, nz, npml, izt), *g = &gg;
    size_t n = (size_t)g->ldz * g->ldx;
    real_t *v = (real_t *)calloc(n, sizeof(real_t));
#pragma omp parallel for schedule(static)
    for (int iz = 2; iz <= nz; ++iz) {
        int no = IMIN(IMIN(iz - izt, nz + npml - iz), norder);
        for (int ix = 1 - norder; ix <= nx + norder; ++ix) {
            real_t s = 0.0f;
            for (int k = 1; k <= no; ++k) s = acc(s, COEF(coef, k, no), G(u, iz + k, ix) - G(u, iz - k, ix));
            G(v, iz, ix) = G(mat, iz, ix) * s / dz;
        }
    }
    memset(out, 0, n * sizeof(real_t));
#pragma omp parallel for schedule(static)
    for (int ix = 1; ix <= nx; ++ix) {
        int no = IMIN(IMIN(ix + npml - 1, nx + npml - ix), norder);
        for (int iz = 2; iz <= nz; ++iz) {
            real_t s = 0.0f;
            for (int k = 1; k <= no; ++k) s = acc(s, COEF(coef, k, no), G(v, iz, ix + k) - G(v, iz, ix - k));
            G(out, iz, ix) = s / dx;
        }
    }
    free(v);
}

/* Mask of the PML region as used by the *_pml operators: the whole grid minus
 * the regular rectangle (iz in [z_lo, z_hi], ix in [x_lo, x_hi]), optionally
 * also minus the top row iz = izt. */
static inline int in_rect(int iz, int ix, int z_lo, int z_hi, int x_lo, int x_hi)
{
    return iz >= z_lo && iz <= z_hi && ix >= x_lo && ix <= x_hi;
}

/* diffzx_pml: src/Submain.f90:411-507. */
void fdfk_op_diffzx_pml(int norder, int nx, int nz, int npml, int izt, real_t dx, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out)
{
    grid_t gg = mkgrid(nx, nz, npml, izt), *g = &gg;
    size_t n = (size_t)g->ldz * g->ldx;
    real_t *v = (real_t *)calloc(n, sizeof(real_t));
    /* mask = 1; mask(1:nz, norder+1:nx-norder) = 0; mask(izt,:) = 0 */
#pragma omp parallel for schedule(static)
    for (int iz = izt + 1; iz <= nz + npml - 1; ++iz) {
        int no = IMIN(IMIN(iz - izt, nz + npml - iz), norder);
        for (int ix = 2 - npml; ix <= nx + npml - 1; ++ix) {
            if (in_rect(iz, ix, 1, nz, norder + 1, nx - norder)) continue;
            real_t s = 0.0f;
            for (int k = 1; k <= no; ++k) s = acc(s, COEF(coef, k, no), G(u, iz + k, ix) - G(u, iz - k, ix));
            G(v, iz, ix) = G(mat, iz, ix) * s / dz;
        }
    }
    memset(out, 0, n * sizeof(real_t));
    /* mask = 1; mask(1:nz, 1:nx) = 0; mask(izt,:) = 0 */
#pragma omp parallel for schedule(static)
    for (int ix = 2 - npml; ix <= nx + npml - 1; ++ix) {
        int no = IMIN(IMIN(ix + npml - 1, nx + npml - ix), norder);
        for (int iz = izt + 1; iz <= nz + npml - 1; ++iz) {
            if (in_rect(iz, ix, 1, nz, 1, nx)) continue;
            real_t s = 0.0f;
            for (int k = 1; k <= no; ++k) s = acc(s, COEF(coef, k, no), G(v, iz, ix + k) - G(v, iz, ix - k));
            G(out, iz, ix) = s / dx;
        }
    }
    free(v);
}

/* diffxz_reg: src/Submain.f90:509-664, active part 608-661. */
void fdfk_op_diffxz_reg(int norder, int nx, int nz, int npml, int izt, real_t dx, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out)
{
    grid_t gg = mkgrid(nx, nz, npml, izt), *g = &gg;
    size_t n = (size_t)g->ldz * g->ldx;
    real_t *v = (real_t *)calloc(n, sizeof(real_t));
#pragma omp parallel for schedule(static)
    for (int ix = 1; ix <= nx; ++ix) {
        int no = IMIN(IMIN(ix + npml - 1, nx + npml - ix), norder);
        for (int iz = 1; iz <= nz + norder; ++iz) {
            real_t s = 0.0f;
            for (int k = 1; k <= no; ++k) s = acc(s, COEF(coef, k, no), G(u, iz, ix + k) - G(u, iz, ix - k));
            G(v, iz, ix) = G(mat, iz, ix) * s / dx;
        }
    }
    memset(out, 0, n * sizeof(real_t));
#pragma omp parallel for schedule(static)
    for (int iz = 2; iz <= nz; ++iz) {
        int no = IMIN(IMIN(iz - izt, nz + npml - iz), norder);
        for (int ix = 1; ix <= nx; ++ix) {
            real_t s = 0.0f;
            for (int k = 1; k <= no; ++k) s = acc(s, COEF(coef, k, no), G(v, iz + k, ix) - G(v, iz - k, ix));
            G(out, iz, ix) = s / dz;
        }
    }
    free(v);
}

/* diffxz_pml: src/Submain.f90:666-762. */
void fdfk_op_diffxz_pml(int norder, int nx, int nz, int npml, int izt, real_t dx, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out)
{
    grid_t gg = mkgrid(nx, nz, npml, izt), *g = &gg;
    size_t n = (size_t)g->ldz * g->ldx;
    real_t *v = (real_t *)calloc(n, sizeof(real_t));
    /* mask = 1; mask(1:nz-norder, 1:nx) = 0 */
#pragma omp parallel for schedule(static)
    for (int ix = 2 - npml; ix <= nx + npml - 1; ++ix) {
        int no = IMIN(IMIN(ix + npml - 1, nx + npml - ix), norder);
        for (int iz = izt; iz <= nz + npml - 1; ++iz) {
            if (in_rect(iz, ix, 1, nz - norder, 1, nx)) continue;
            real_t s = 0.0f;
            for (int k = 1; k <= no; ++k) s = acc(s, COEF(coef, k, no), G(u, iz, ix + k) - G(u, iz, ix - k));
            G(v, iz, ix) = G(mat, iz, ix) * s / dx;
        }
    }
    memset(out, 0, n * sizeof(real_t));
    /* mask = 1; mask(1:nz, 1:nx) = 0; mask(izt,:) = 0 */
#pragma omp parallel for schedule(static)
    for (int iz = izt + 1; iz <= nz + npml - 1; ++iz) {
        int no = IMIN(IMIN(iz - izt, nz + npml - iz), norder);
        for (int ix = 2 - npml; ix <= nx + npml - 1; ++ix) {
            if (in_rect(iz, ix, 1, nz, 1, nx)) continue;
            real_t s = 0.0f;
            for (int k = 1; k <= no; ++k) s = acc(s, COEF(coef, k, no), G(v, iz + k, ix) - G(v, iz - k, ix));
            G(out, iz, ix) = s / dz;
        }
    }
    free(v);
}

/* ---------------------------------------------------------------------- */
/* Second-derivative operators with harmonic-averaged moduli              */
/* ---------------------------------------------------------------------- */

/* One point of d/dx(M d/dx u): src/Submain.f90:814-837. */
static inline real_t x2_point(const grid_t *g, int norder, const double *coef, const real_t *mat,
                             const real_t *u, int iz, int ix)
{
    int nx = g->nx, npml = g->npml;
    int no = IMIN(IMIN(ix + npml - 1, nx + npml - ix), norder);
    real_t s = 0.0f;
    for (int k = 1; k <= no; ++k) {
        int i = k - 1; /* int((2*k-1)/2) */
        int n1 = IMIN(IMIN(ix + i + npml - 1, nx + npml - ix - i), norder);
        real_t s1 = 0.0f;
        for (int j = 1; j <= n1; ++j) s1 = acc(s1, COEF(coef, j, n1), G(u, iz, ix + j + k - 1) - G(u, iz, ix - j + k));
        int n2 = IMIN(IMIN(ix - i + npml - 1, nx + npml - ix + i), norder);
        real_t s2 = 0.0f;
        for (int j = 1; j <= n2; ++j) s2 = acc(s2, COEF(coef, j, n2), G(u, iz, ix + j - k) - G(u, iz, ix - j - k + 1));
        real_t hp = 2.0f / (1.0f / G(mat, iz, ix + k) + 1.0f / G(mat, iz, ix + k - 1));
        real_t hm = 2.0f / (1.0f / G(mat, iz, ix - k + 1) + 1.0f / G(mat, iz, ix - k));
        s = acc(s, COEF(coef, k, no), hp * s1 - hm * s2);
    }
    return s;
}

/* One point of d/dz(M d/dz u): src/Submain.f90:988-1011. */
static inline real_t z2_point(const grid_t *g, int norder, const double *coef, const real_t *mat,
                             const real_t *u, int iz, int ix)
{
    int nz = g->nz, npml = g->npml, izt = g->izt;
    int no = IMIN(IMIN(iz - izt, nz + npml - iz), norder);
    real_t s = 0.0f;
    for (int k = 1; k <= no; ++k) {
        int i = k - 1;
        int n1 = IMIN(IMIN(iz + i - izt, nz + npml - iz - i), norder);
        real_t s1 = 0.0f;
        for (int j = 1; j <= n1; ++j) s1 = acc(s1, COEF(coef, j, n1), G(u, iz + j + k - 1, ix) - G(u, iz - j + k, ix));
        int n2 = IMIN(IMIN(iz - i - izt, nz + npml - iz + i), norder);
        real_t s2 = 0.0f;
        for (int j = 1; j <= n2; ++j) s2 = acc(s2, COEF(coef, j, n2), G(u, iz + j - k, ix) - G(u, iz - j - k + 1, ix));
        real_t hp = 2.0f / (1.0f / G(mat, iz + k, ix) + 1.0f / G(mat, iz + k - 1, ix));
        real_t hm = 2.0f / (1.0f / G(mat, iz - k + 1, ix) + 1.0f / G(mat, iz - k, ix));
        s = acc(s, COEF(coef, k, no), hp * s1 - hm * s2);
    }
    return s;
}

/* diffx2_reg: src/Submain.f90:764-849.  dx2 = 1.d0/(dx*dx) stored as real_t. */
void fdfk_op_diffx2_reg(int norder, int nx, int nz, int npml, int izt, real_t dx,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out)
{
    grid_t gg = mkgrid(nx, nz, npml, izt), *g = &gg;
    memset(out, 0, (size_t)g->ldz * g->ldx * sizeof(real_t));
    real_t dx2 = (real_t)(1.0 / (double)(dx * dx));
    /* mask(1:nz, 1:nx) = 1, loop iz = izt..nz */
#pragma omp parallel for schedule(static)
    for (int ix = 1; ix <= nx; ++ix)
        for (int iz = IMAX(izt, 1); iz <= nz; ++iz) G(out, iz, ix) = x2_point(g, norder, coef, mat, u, iz, ix) * dx2;
}

/* diffx2_pml: src/Submain.f90:851-937.  dx2 = 1.0/(dx*dx) in real_t. */
void fdfk_op_diffx2_pml(int norder, int nx, int nz, int npml, int izt, real_t dx,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out)
{
    grid_t gg = mkgrid(nx, nz, npml, izt), *g = &gg;
    memset(out, 0, (size_t)g->ldz * g->ldx * sizeof(real_t));
    real_t dx2 = 1.0f / (dx * dx);
#pragma omp parallel for schedule(static)
    for (int ix = 2 - npml; ix <= nx + npml - 1; ++ix)
        for (int iz = izt; iz <= nz + npml - 1; ++iz) {
            if (in_rect(iz, ix, 1, nz, 1, nx)) continue;
            G(out, iz, ix) = x2_point(g, norder, coef, mat, u, iz, ix) * dx2;
        }
}

/* diffz2_reg: src/Submain.f90:939-1023. */
void fdfk_op_diffz2_reg(int norder, int nx, int nz, int npml, int izt, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out)
{
    grid_t gg = mkgrid(nx, nz, npml, izt), *g = &gg;
    memset(out, 0, (size_t)g->ldz * g->ldx * sizeof(real_t));
    real_t dz2 = 1.0f / (dz * dz);
#pragma omp parallel for schedule(static)
    for (int iz = 2; iz <= nz; ++iz)
        for (int ix = 1; ix <= nx; ++ix) G(out, iz, ix) = z2_point(g, norder, coef, mat, u, iz, ix) * dz2;
}

/* diffz2_pml: src/Submain.f90:1025-1109. */
void fdfk_op_diffz2_pml(int norder, int nx, int nz, int npml, int izt, real_t dz,
                        const double *coef, const real_t *mat, const real_t *u, real_t *out)
{
    grid_t gg = mkgrid(nx, nz, npml, izt), *g = &gg;
    memset(out, 0, (size_t)g->ldz * g->ldx * sizeof(real_t));
    real_t dz2 = 1.0f / (dz * dz);
#pragma omp parallel for schedule(static)
    for (int iz = izt + 1; iz <= nz + npml - 1; ++iz)
        for (int ix = 1 - npml; ix <= nx + npml; ++ix) {
            if (in_rect(iz, ix, 1, nz, 1, nx)) continue;
            G(out, iz, ix) = z2_point(g, norder, coef, mat, u, iz, ix) * dz2;
        }
}

/* ---------------------------------------------------------------------- */
/* loadseis: src/Submain.f90:33-116 (discrete-delta receiver sampling).   */
/* ux, uz are the two-level arrays real(1:2, izt:nz+npml, 1-npml:nx+npml); */
/* level 1 is sampled.                                                     */
/* ---------------------------------------------------------------------- */
double fdfk_op_delta_weight(double x)
{
    double x2 = x * x, x3 = x2 * x;
    if (x <= 1.0)
        return 1.0 + x2 * (-5.0 / 4.0 + x2 * (21.0 / 4.0)) + x3 * (-35.0 / 12.0 + x2 * (-25.0 / 12.0));
    if (x <= 2.0)
        return -4.0 + (75.0 / 4.0) * x + x2 * (-245.0 / 8.0 + x2 * (-63.0 / 8.0)) + x3 * (545.0 / 24.0 + x2 * (25.0 / 24.0));
    if (x <= 3.0)
        return 18.0 + (-153.0 / 4.0) * x + x2 * (255.0 / 8.0 + x2 * (21.0 / 8.0)) + x3 * (-313.0 / 24.0 + x2 * (-5.0 / 24.0));
    return 0.0;
}

void fdfk_op_loadseis(int nx, int nz, int npml, int izt, real_t x0, real_t z0, real_t dx, real_t dz,
                      real_t rx, real_t rz, const real_t *ux, const real_t *uz, real_t *dispx, real_t *dispz)
{
    int ldz = nz + npml - izt + 1;
    int irx = (int)floor((rx - x0) / dx) + 1;
    int irz = (int)floor((rz - z0) / dz) + 1;
    real_t sx = 0.0f, sz = 0.0f;
    for (int ix = IMAX(1 - npml, irx - 3); ix <= IMIN(nx + npml, irx + 3); ++ix) {
        double x = fabs((double)((double)(x0 + (real_t)(ix - 1) * dx) - (double)rx)) / (double)dx;
        double bx = fdfk_op_delta_weight(x);
        for (int iz = IMAX(izt, irz - 3); iz <= IMIN(nz + npml, irz + 3); ++iz) {
            double z = fabs((double)((double)(z0 + (real_t)(iz - 1) * dz) - (double)rz)) / (double)dz;
            double ba = bx * fdfk_op_delta_weight(z);
            size_t o = 2 * ((size_t)(iz - izt) + (size_t)(ix - (1 - npml)) * (size_t)ldz);
            sx = (real_t)((double)sx + ba * (double)ux[o]);
            sz = (real_t)((double)sz + ba * (double)uz[o]);
        }
    }
    *dispx = sx;
    *dispz = sz;
}

/* ---------------------------------------------------------------------- */
/* gfortran-ABI exports (every argument by reference).                    */
/* ---------------------------------------------------------------------- */
void diff1_(const int *norder, const int *dire, const int *nx, const int *nz, const int *npml, const int *izt,
            const int *ix, const int *iz, const real_t *d, const double *coef, const real_t *u, real_t *tmp)
{
    *tmp = fdfk_op_diff1(*norder, *dire, *nx, *nz, *npml, *izt, *ix, *iz, *d, coef, u);
    fdfk_trace_point(1, __builtin_return_address(0), *ix, *iz, *dire, *d, u, *tmp);
}

void diffx1_(const int *norder, const int *nx, const int *npml, const int *ix, const real_t *dx,
             const double *coef, const real_t *u, real_t *tmp)
{
    *tmp = fdfk_op_diffx1(*norder, *nx, *npml, *ix, *dx, coef, u);
    fdfk_trace_point(2, __builtin_return_address(0), *ix, 0, 1, *dx, u, *tmp);
}

#define MIXED_EXPORT(name)                                                                              \
    void name##_(const int *norder, const int *nx, const int *nz, const int *npml, const int *izt,      \
                 const real_t *dx, const real_t *dz, const double *coef, const real_t *mat, const real_t *u, \
                 real_t *out)                                                                            \
    {                                                                                                   \
        fdfk_trace_hook(#name, *norder, *nx, *nz, *npml, *izt, mat, u, out);                            \
        fdfk_op_##name(*norder, *nx, *nz, *npml, *izt, *dx, *dz, coef, mat, u, out);                    \
        fdfk_trace_post(#name, *nx, *nz, *npml, *izt, out);                                             \
    }
#define SECOND_EXPORT(name)                                                                             \
    void name##_(const int *norder, const int *nx, const int *nz, const int *npml, const int *izt,      \
                 const real_t *d, const double *coef, const real_t *mat, const real_t *u, real_t *out)      \
    {                                                                                                   \
        fdfk_trace_hook(#name, *norder, *nx, *nz, *npml, *izt, mat, u, out);                            \
        fdfk_op_##name(*norder, *nx, *nz, *npml, *izt, *d, coef, mat, u, out);                          \
        fdfk_trace_post(#name, *nx, *nz, *npml, *izt, out);                                             \
    }

/* Optional observation hooks: the reference harness overrides these to record
 * which operators the shipped libraries call; the defaults do nothing. */
__attribute__((weak)) void fdfk_trace_hook(const char *name, int norder, int nx, int nz, int npml, int izt,
                                           const real_t *mat, const real_t *u, real_t *out)
{
    (void)name; (void)norder; (void)nx; (void)nz; (void)npml; (void)izt; (void)mat; (void)u; (void)out;
}
__attribute__((weak)) void fdfk_trace_point(int which, const void *caller, int ix, int iz, int dire, real_t d,
                                            const real_t *u, real_t val)
{
    (void)which; (void)caller; (void)ix; (void)iz; (void)dire; (void)d; (void)u; (void)val;
}
__attribute__((weak)) void fdfk_trace_post(const char *name, int nx, int nz, int npml, int izt, real_t *out)
{
    (void)name; (void)nx; (void)nz; (void)npml; (void)izt; (void)out;
}

MIXED_EXPORT(diffzx_reg)
MIXED_EXPORT(diffzx_pml)
MIXED_EXPORT(diffxz_reg)
MIXED_EXPORT(diffxz_pml)
SECOND_EXPORT(diffx2_reg)
SECOND_EXPORT(diffx2_pml)
SECOND_EXPORT(diffz2_reg)
SECOND_EXPORT(diffz2_pml)
