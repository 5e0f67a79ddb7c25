/*
 * ORACLE (test infrastructure only; never part of the product path).
 *
 * CPU restatement of one hybrid FD-FK time step of FDFK2D (`updatedispl_`,
 * call site src/FDFK2D.f90:516-522; shipped closed as lib_gnu/libHybrid.so
 * and lib_gnu/libPML.so) and of the time loop around it
 * (src/FDFK2D.f90:465-532).  The open operators come from fdfk_ops.c
 * (src/Submain.f90:167-1109).  The closed semantics below were recovered by
 * running the shipped libraries as a black box and are pinned against them:
 *
 * 1. Displacement leapfrog (two stored levels, level 1 = u^n, level 2 = u^{n-1}):
 *      u^{n+1} = 2 u^n - u^{n-1} + dt^2/rho * F,  level 2 <- old level 1.
 *    F_x = dxx(l2m ux) + dzx(lam uz) + dzz(mu ux) + dxz(mu uz)
 *    F_z = dzz(l2m uz) + dxz(lam ux) + dxx(mu uz) + dzx(mu ux)
 *    with the *_reg operators (l2m = lam + 2 mu computed in real_t).
 * 2. Hybrid injection (Alterman-Karal): the interior operators act on
 *    u + u_b(it) where u_b is added on the outer strips (Omega_II: the *_pml
 *    background strips); the PML operators act on u - u_b(it) where u_b is
 *    removed on the inner strips (Omega_I: the *_reg background strips).
 * 3. Free surface (top row iz = 1; applied in the PML-on-top mode too, item 5),
 *    stress image about the half row 1.5:
 *      F_x(1) = dxx(l2m ux) + Dx[lam(1) (uz(2)-uz(1))/dz] + 2/dz * sxz(1.5)
 *      F_z(1) = dxx(mu uz)  + Dx[mu(1) (ux(2)-ux(1))/dz]  + 2/dz * szz(1.5)
 *      sxz(1.5) = H(mu1,mu2)(ux2-ux1)/dz + (mu1 Dx uz1 + mu2 Dx uz2)/2
 *      szz(1.5) = H(l2m1,l2m2)(uz2-uz1)/dz + (lam1 Dx ux1 + lam2 Dx ux2)/2
 *    H = harmonic mean; Dx = collocated first derivative (diffx1) on the rows
 *    of the injected field.
 * 4. PML: three-way split field per component (u = u1 + u2 + u3), second-order
 *    PML of Komatitsch & Tromp (2003), damping d(s) = d0 (s/L)^npower,
 *    d0 = (npower+1) vpml ln(1/R0) / (2 L), L = npml*h, s = distance into the
 *    layer counted in whole cells (first PML cell s = h):
 *      rho (dt + dx)^2 u1       = Fxx + (P^{n+1} + P^n)/2
 *      rho (dt + dx)(dt + dz) u2 = Fmixed
 *      rho (dt + dz)^2 u3       = Fzz + (Q^{n+1} + Q^n)/2     (dz = 0 on the sides)
 *      (dt + dx) P = -dx' * S_x,  (dt + dz) Q = -dz' * S_z  (trapezoidal)
 *    S_x = l2m Dx ux / mu Dx uz, S_z = mu Dz ux / l2m Dz uz (diff1), signed
 *    dd/dx.  Centred differences in time.  On the right side the shipped
 *    update does not divide the u1 forcing by (1 + dx dt) except on the free
 *    surface row; this is reproduced.
 *
 * 5. PML on top (is_PML_top, izt = 1 - npml; pinned against the shipped step
 *    on random state for norder 1..4 and 8, square and oblong cells):
 *    - a fourth layer, rows izt+1..0 over every column but the outer frame
 *      (the corners belong to it), damped in x and z like the bottom layer,
 *      with the depth into it counted from row 1 (d' < 0), state in the top
 *      arrays (bp*t*, bu*t); row izt is outer frame like row nz+npml;
 *    - the interior update keeps the free-surface formula of item 3 on row 1
 *      (the shipped step applies it whatever is_PML_top says); the absorbing
 *      layers' row 1 uses the general split-field terms, and the right layer
 *      leaves the u1 forcing undivided on every row;
 *    - the absorbing layers' operator field is formed after the interior
 *      update: where no inner strip lies (rows 1..nz-nbd, columns
 *      nbd+1..nx-nbd) it holds the new u^{n+1}, elsewhere u^n minus the inner
 *      strips.  Only the top layer's stencils reach those cells.
 *    The FK background does not depend on izt (the shipped
 *    comput_background_wavefield_ gives the same strips for both modes).
 */
#include "fdfk_oracle.h"
#include "fdfk_ops.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define IMIN(a, b) ((a) < (b) ? (a) : (b))
#define IMAX(a, b) ((a) > (b) ? (a) : (b))

typedef struct {
    int nx, nz, npml, izt, ldz, ldx, norder, nbd;
} geo_t;

static inline size_t gi(const geo_t *g, int iz, int ix)
{
    return (size_t)(iz - g->izt) + (size_t)(ix - (1 - g->npml)) * (size_t)g->ldz;
}

/* index into a Fortran strip of shape (n1, n2, nt+1) at (r, c, t), 0-based r, c */
static inline size_t si(int n1, int n2, int r, int c, int t)
{
    return (size_t)r + (size_t)n1 * ((size_t)c + (size_t)n2 * (size_t)t);
}

static double dx1_row(const geo_t *g, const double *coef1, const real_t *row_base, size_t stride, int ix, real_t dx)
{
    /* collocated x-derivative of a grid row (row_base = element (iz, 1-npml), stride = ldz) */
    int norder = g->norder;
    int no = IMIN(IMIN(ix + g->npml - 1, g->nx + g->npml - ix), norder);
    size_t c = (size_t)(ix - (1 - g->npml));
    double s = 0.0;
    for (int k = 1; k <= no; ++k)
        s += coef1[(k - 1) + (no - 1) * norder] * ((double)row_base[(c + k) * stride] - (double)row_base[(c - k) * stride]);
    return s / dx;
}

static double dx1_rowd(const geo_t *g, const double *coef1, const double *row, int ix, real_t dx)
{
    int norder = g->norder;
    int no = IMIN(IMIN(ix + g->npml - 1, g->nx + g->npml - ix), norder);
    int c = ix - (1 - g->npml);
    double s = 0.0;
    for (int k = 1; k <= no; ++k) s += coef1[(k - 1) + (no - 1) * norder] * (row[c + k] - row[c - k]);
    return s / dx;
}

/* pointwise collocated derivative in x (dire 1) or z (dire 2) of a double field */
static double cd1(const geo_t *g, const double *coef1, const double *u, int iz, int ix, int dire, real_t d)
{
    int norder = g->norder;
    double s = 0.0;
    if (dire == 1) {
        int no = IMIN(IMIN(ix + g->npml - 1, g->nx + g->npml - ix), norder);
        for (int k = 1; k <= no; ++k) s += coef1[(k - 1) + (no - 1) * norder] * (u[gi(g, iz, ix + k)] - u[gi(g, iz, ix - k)]);
    } else {
        int no = IMIN(IMIN(iz - g->izt, g->nz + g->npml - iz), norder);
        for (int k = 1; k <= no; ++k) s += coef1[(k - 1) + (no - 1) * norder] * (u[gi(g, iz + k, ix)] - u[gi(g, iz - k, ix)]);
    }
    return s / d;
}

enum { OP_X2_L2M_X, OP_Z2_L2M_Z, OP_ZX_LAM_Z, OP_XZ_LAM_X, OP_Z2_MU_X, OP_X2_MU_Z, OP_XZ_MU_Z, OP_ZX_MU_X, NOPS };

static void run_ops(const fdfk_oracle_params *p, int pml, const real_t *l2m, const real_t *lam, const real_t *mu,
                    const double *coef0, const double *coef1, const real_t *tx, const real_t *tz, real_t *const out[NOPS])
{
    int a0 = p->norder, nx = p->nx, nz = p->nz, npml = p->npml, izt = p->izt;
    real_t dx = p->dx, dz = p->dz;
    if (!pml) {
        fdfk_op_diffx2_reg(a0, nx, nz, npml, izt, dx, coef0, l2m, tx, out[OP_X2_L2M_X]);
        fdfk_op_diffz2_reg(a0, nx, nz, npml, izt, dz, coef0, l2m, tz, out[OP_Z2_L2M_Z]);
        fdfk_op_diffzx_reg(a0, nx, nz, npml, izt, dx, dz, coef1, lam, tz, out[OP_ZX_LAM_Z]);
        fdfk_op_diffxz_reg(a0, nx, nz, npml, izt, dx, dz, coef1, lam, tx, out[OP_XZ_LAM_X]);
        fdfk_op_diffz2_reg(a0, nx, nz, npml, izt, dz, coef0, mu, tx, out[OP_Z2_MU_X]);
        fdfk_op_diffx2_reg(a0, nx, nz, npml, izt, dx, coef0, mu, tz, out[OP_X2_MU_Z]);
        fdfk_op_diffxz_reg(a0, nx, nz, npml, izt, dx, dz, coef1, mu, tz, out[OP_XZ_MU_Z]);
        fdfk_op_diffzx_reg(a0, nx, nz, npml, izt, dx, dz, coef1, mu, tx, out[OP_ZX_MU_X]);
    } else {
        fdfk_op_diffx2_pml(a0, nx, nz, npml, izt, dx, coef0, l2m, tx, out[OP_X2_L2M_X]);
        fdfk_op_diffz2_pml(a0, nx, nz, npml, izt, dz, coef0, l2m, tz, out[OP_Z2_L2M_Z]);
        fdfk_op_diffzx_pml(a0, nx, nz, npml, izt, dx, dz, coef1, lam, tz, out[OP_ZX_LAM_Z]);
        fdfk_op_diffxz_pml(a0, nx, nz, npml, izt, dx, dz, coef1, lam, tx, out[OP_XZ_LAM_X]);
        fdfk_op_diffz2_pml(a0, nx, nz, npml, izt, dz, coef0, mu, tx, out[OP_Z2_MU_X]);
        fdfk_op_diffx2_pml(a0, nx, nz, npml, izt, dx, coef0, mu, tz, out[OP_X2_MU_Z]);
        fdfk_op_diffxz_pml(a0, nx, nz, npml, izt, dx, dz, coef1, mu, tz, out[OP_XZ_MU_Z]);
        fdfk_op_diffzx_pml(a0, nx, nz, npml, izt, dx, dz, coef1, mu, tx, out[OP_ZX_MU_X]);
    }
}

/* Add (sign +1) the outer background strips or remove (sign -1) the inner ones. */
static void apply_strips(const fdfk_oracle_params *p, const geo_t *g, int it, const real_t *const strips[12], int comp,
                         int outer, real_t *t)
{
    int nx = p->nx, nz = p->nz, nbd = p->nbd;
    if (outer) {
        const real_t *L = strips[6 + comp], *Rr = strips[8 + comp], *B = strips[10 + comp];
        for (int c = 0; c < nbd; ++c)
            for (int r = 0; r < nz; ++r) {
                t[gi(g, 1 + r, 1 - nbd + c)] += L[si(nz, nbd, r, c, it)];
                t[gi(g, 1 + r, nx + 1 + c)] += Rr[si(nz, nbd, r, c, it)];
            }
        for (int c = 0; c < nx + 2 * nbd; ++c)
            for (int r = 0; r < nbd; ++r) t[gi(g, nz + 1 + r, 1 - nbd + c)] += B[si(nbd, nx + 2 * nbd, r, c, it)];
    } else {
        const real_t *L = strips[0 + comp], *Rr = strips[2 + comp], *B = strips[4 + comp];
        for (int c = 0; c < nbd; ++c)
            for (int r = 0; r < nz - nbd; ++r) {
                t[gi(g, 1 + r, 1 + c)] -= L[si(nz - nbd, nbd, r, c, it)];
                t[gi(g, 1 + r, nx - nbd + 1 + c)] -= Rr[si(nz - nbd, nbd, r, c, it)];
            }
        for (int c = 0; c < nx; ++c)
            for (int r = 0; r < nbd; ++r) t[gi(g, nz - nbd + 1 + r, 1 + c)] -= B[si(nbd, nx, r, c, it)];
    }
}

static inline double hmean(double a, double b) { return 2.0 / (1.0 / a + 1.0 / b); }

int fdfk_oracle_updatedispl(const fdfk_oracle_params *p, int it, const real_t *const strips[12], const real_t *c,
                            const double *coef0, const double *coef1, real_t *ux, real_t *uz, real_t *const bp[12],
                            real_t *const bu[24])
{
    const int top = p->izt != 1;   /* PML on top (item 5) */
    if (top && p->izt != 1 - p->npml) return -2;
    if (p->norder < 1 || p->nbd != 2 * p->norder - 1 || p->npml < p->nbd || p->nz <= p->nbd || p->nx < 1) return -1;
    geo_t G = {p->nx, p->nz, p->npml, p->izt, p->nz + p->npml - p->izt + 1, p->nx + 2 * p->npml, p->norder, p->nbd};
    const geo_t *g = &G;
    int nx = p->nx, nz = p->nz, npml = p->npml;
    real_t dx = p->dx, dz = p->dz;
    double dt = p->dt;
    size_t n = (size_t)g->ldz * g->ldx;

    real_t *w = (real_t *)malloc(sizeof(real_t) * n * (6 + 2 * NOPS));
    double *wd = (double *)malloc(sizeof(double) * n * 2);
    if (!w || !wd) { free(w); free(wd); return -3; }
    real_t *rho = w, *lam = w + n, *mu = w + 2 * n, *l2m = w + 3 * n, *tx = w + 4 * n, *tz = w + 5 * n;
    real_t *ops[NOPS];
    for (int k = 0; k < NOPS; ++k) ops[k] = w + (6 + k) * n;
    real_t *pops[NOPS];
    for (int k = 0; k < NOPS; ++k) pops[k] = w + (6 + NOPS + k) * n;
    for (size_t i = 0; i < n; ++i) {
        rho[i] = c[3 * i]; lam[i] = c[3 * i + 1]; mu[i] = c[3 * i + 2];
        l2m[i] = lam[i] + 2.0f * mu[i];
    }

    /* -------- interior: operators on u + u_b(outer strips) -------- */
    for (size_t i = 0; i < n; ++i) { tx[i] = ux[2 * i]; tz[i] = uz[2 * i]; }
    apply_strips(p, g, it, strips, 0, 1, tx);
    apply_strips(p, g, it, strips, 1, 1, tz);
    run_ops(p, 0, l2m, lam, mu, coef0, coef1, tx, tz, ops);

    /* -------- PML: operators on u^n - u_b(inner strips) (reads only level 1) -------- */
    real_t *px = (real_t *)malloc(sizeof(real_t) * n), *pz = (real_t *)malloc(sizeof(real_t) * n);
    if (!px || !pz) { free(w); free(wd); free(px); free(pz); return -3; }
    for (size_t i = 0; i < n; ++i) { px[i] = ux[2 * i]; pz[i] = uz[2 * i]; }
    apply_strips(p, g, it, strips, 0, 0, px);
    apply_strips(p, g, it, strips, 1, 0, pz);
    run_ops(p, 1, l2m, lam, mu, coef0, coef1, px, pz, pops);
    double *Sx = wd, *Sz = wd + n;
    for (size_t i = 0; i < n; ++i) { Sx[i] = px[i]; Sz[i] = pz[i]; }

    /* -------- interior update (rows 1..nz, cols 1..nx) -------- */
    real_t *nux1 = (real_t *)malloc(sizeof(real_t) * n), *nuz1 = (real_t *)malloc(sizeof(real_t) * n);
    if (!nux1 || !nuz1) { free(w); free(wd); free(px); free(pz); free(nux1); free(nuz1); return -3; }
#pragma omp parallel for schedule(static)
    for (int ix = 1; ix <= nx; ++ix) {
        for (int iz = 1; iz <= nz; ++iz) {
            size_t i = gi(g, iz, ix);
            double Fx, Fz;
            if (iz == 1) {
                size_t r1 = gi(g, 1, 1 - npml), r2 = gi(g, 2, 1 - npml);
                int cc = ix - (1 - npml);
                /* rows of the injected field, and the two derived rows lam(1) dz uz, mu(1) dz ux */
                double dA = 0.0, dB = 0.0;
                {
                    int no = IMIN(IMIN(ix + npml - 1, nx + npml - ix), g->norder);
                    for (int k = 1; k <= no; ++k) {
                        double ck = coef1[(k - 1) + (no - 1) * g->norder];
                        size_t ip = (size_t)(cc + k) * g->ldz, im = (size_t)(cc - k) * g->ldz;
                        double Ap = (double)lam[r1 + ip] * ((double)tz[r2 + ip] - (double)tz[r1 + ip]) / dz;
                        double Am = (double)lam[r1 + im] * ((double)tz[r2 + im] - (double)tz[r1 + im]) / dz;
                        double Bp = (double)mu[r1 + ip] * ((double)tx[r2 + ip] - (double)tx[r1 + ip]) / dz;
                        double Bm = (double)mu[r1 + im] * ((double)tx[r2 + im] - (double)tx[r1 + im]) / dz;
                        dA += ck * (Ap - Am);
                        dB += ck * (Bp - Bm);
                    }
                    dA /= dx;
                    dB /= dx;
                }
                double dz1 = dx1_row(g, coef1, tz + r1, g->ldz, ix, dx), dz2 = dx1_row(g, coef1, tz + r2, g->ldz, ix, dx);
                double dx1 = dx1_row(g, coef1, tx + r1, g->ldz, ix, dx), dx2 = dx1_row(g, coef1, tx + r2, g->ldz, ix, dx);
                size_t i1 = gi(g, 1, ix), i2 = gi(g, 2, ix);
                double sxz = hmean(mu[i1], mu[i2]) * ((double)ux[2 * i2] - (double)ux[2 * i1]) / dz +
                             ((double)mu[i1] * dz1 + (double)mu[i2] * dz2) / 2.0;
                double szz = hmean(l2m[i1], l2m[i2]) * ((double)uz[2 * i2] - (double)uz[2 * i1]) / dz +
                             ((double)lam[i1] * dx1 + (double)lam[i2] * dx2) / 2.0;
                Fx = (double)ops[OP_X2_L2M_X][i] + dA + 2.0 * sxz / dz;
                Fz = (double)ops[OP_X2_MU_Z][i] + dB + 2.0 * szz / dz;
            } else {
                Fx = (double)ops[OP_X2_L2M_X][i] + (double)ops[OP_ZX_LAM_Z][i] + (double)ops[OP_Z2_MU_X][i] +
                     (double)ops[OP_XZ_MU_Z][i];
                Fz = (double)ops[OP_Z2_L2M_Z][i] + (double)ops[OP_XZ_LAM_X][i] + (double)ops[OP_X2_MU_Z][i] +
                     (double)ops[OP_ZX_MU_X][i];
            }
            nux1[i] = (real_t)(2.0 * ux[2 * i] - (double)ux[2 * i + 1] + dt * dt * Fx / (double)rho[i]);
            nuz1[i] = (real_t)(2.0 * uz[2 * i] - (double)uz[2 * i + 1] + dt * dt * Fz / (double)rho[i]);
        }
    }

    if (top) {
        /* item 5: the operator field of the layers, formed after the interior update */
        for (size_t i = 0; i < n; ++i) { px[i] = ux[2 * i]; pz[i] = uz[2 * i]; }
        apply_strips(p, g, it, strips, 0, 0, px);
        apply_strips(p, g, it, strips, 1, 0, pz);
        for (int ix = p->nbd + 1; ix <= nx - p->nbd; ++ix)
            for (int iz = 1; iz <= nz - p->nbd; ++iz) {
                size_t i = gi(g, iz, ix);
                px[i] = nux1[i];
                pz[i] = nuz1[i];
            }
        run_ops(p, 1, l2m, lam, mu, coef0, coef1, px, pz, pops);
        for (size_t i = 0; i < n; ++i) { Sx[i] = px[i]; Sz[i] = pz[i]; }
    }

    /* -------- PML update -------- */
    double logr = log(1.0 / p->R0);
    double d0x = (p->npower + 1) * (double)p->vpml * logr / (2.0 * npml * dx);
    double d0z = (p->npower + 1) * (double)p->vpml * logr / (2.0 * npml * dz);
    double Lx = (double)npml * dx, Lz = (double)npml * dz;
    int npw = p->npower;
    /* free-surface rows of the PML-operator field */
    double *rowA = (double *)malloc(sizeof(double) * g->ldx), *rowB = (double *)malloc(sizeof(double) * g->ldx);
    double *rz1 = (double *)malloc(sizeof(double) * g->ldx), *rz2 = (double *)malloc(sizeof(double) * g->ldx);
    double *rx1 = (double *)malloc(sizeof(double) * g->ldx), *rx2 = (double *)malloc(sizeof(double) * g->ldx);
    for (int ix = 1 - npml; ix <= nx + npml; ++ix) {
        size_t i1 = gi(g, 1, ix), i2 = gi(g, 2, ix);
        int cc = ix - (1 - npml);
        rowA[cc] = (double)lam[i1] * (Sz[i2] - Sz[i1]) / dz;
        rowB[cc] = (double)mu[i1] * (Sx[i2] - Sx[i1]) / dz;
        rz1[cc] = Sz[i1]; rz2[cc] = Sz[i2]; rx1[cc] = Sx[i1]; rx2[cc] = Sx[i2];
    }

    /* sides: 0 = left, 1 = right, 2 = bottom, 3 = top (item 5) */
    for (int side = 0; side < (top ? 4 : 3); ++side) {
        int iz_lo, iz_hi, ix_lo, ix_hi;
        if (side == 0) { iz_lo = 1; iz_hi = nz; ix_lo = 2 - npml; ix_hi = 0; }
        else if (side == 1) { iz_lo = 1; iz_hi = nz; ix_lo = nx + 1; ix_hi = nx + npml - 1; }
        else if (side == 2) { iz_lo = nz + 1; iz_hi = nz + npml - 1; ix_lo = 2 - npml; ix_hi = nx + npml - 1; }
        else { iz_lo = p->izt + 1; iz_hi = 0; ix_lo = 2 - npml; ix_hi = nx + npml - 1; }
#pragma omp parallel for schedule(static)
        for (int ix = ix_lo; ix <= ix_hi; ++ix) {
            /* damping in x */
            double dxv = 0.0, dxp = 0.0;
            if (ix <= 0) {
                double s = (double)(1 - ix) * dx / Lx;
                dxv = d0x * pow(s, npw); dxp = -npw * d0x * pow(s, npw - 1) / Lx;
            } else if (ix > nx) {
                double s = (double)(ix - nx) * dx / Lx;
                dxv = d0x * pow(s, npw); dxp = npw * d0x * pow(s, npw - 1) / Lx;
            }
            for (int iz = iz_lo; iz <= iz_hi; ++iz) {
                double dzv = 0.0, dzp = 0.0;
                if (side == 2) {
                    double s = (double)(iz - nz) * dz / Lz;
                    dzv = d0z * pow(s, npw); dzp = npw * d0z * pow(s, npw - 1) / Lz;
                } else if (side == 3) {
                    double s = (double)(1 - iz) * dz / Lz;
                    dzv = d0z * pow(s, npw); dzp = -npw * d0z * pow(s, npw - 1) / Lz;
                }
                double yx = dxv * dt, yz = dzv * dt;
                size_t i = gi(g, iz, ix);
                double k = dt * dt / (double)rho[i];
                /* index into the side arrays */
                size_t ab, ap; /* bu index of level 1 (level 2 = +1), bp index */
                if (side == 0) { ap = (size_t)(iz - 1) + (size_t)nz * (size_t)(ix - (1 - npml)); ab = 2 * ap; }
                else if (side == 1) { ap = (size_t)(iz - 1) + (size_t)nz * (size_t)(ix - nx - 1); ab = 2 * ap; }
                else if (side == 2) { ap = (size_t)(iz - nz - 1) + (size_t)npml * (size_t)(ix - (1 - npml)); ab = 2 * ap; }
                else { ap = (size_t)(iz - (1 - npml)) + (size_t)npml * (size_t)(ix - (1 - npml)); ab = 2 * ap; }
                for (int comp = 0; comp < 2; ++comp) {
                    double F1, F2, F3, S1, S3 = 0.0;
                    if (iz == 1 && !top) {
                        int cc = ix - (1 - npml);
                        size_t i1 = gi(g, 1, ix), i2 = gi(g, 2, ix);
                        if (comp == 0) {
                            F1 = pops[OP_X2_L2M_X][i];
                            F2 = dx1_rowd(g, coef1, rowA, ix, dx) +
                                 ((double)mu[i1] * dx1_rowd(g, coef1, rz1, ix, dx) + (double)mu[i2] * dx1_rowd(g, coef1, rz2, ix, dx)) / dz;
                            F3 = 2.0 * hmean(mu[i1], mu[i2]) * (rx2[cc] - rx1[cc]) / dz / dz;
                            S1 = (double)l2m[i1] * dx1_rowd(g, coef1, rx1, ix, dx);
                        } else {
                            F1 = pops[OP_X2_MU_Z][i];
                            F2 = dx1_rowd(g, coef1, rowB, ix, dx) +
                                 ((double)lam[i1] * dx1_rowd(g, coef1, rx1, ix, dx) + (double)lam[i2] * dx1_rowd(g, coef1, rx2, ix, dx)) / dz;
                            F3 = 2.0 * hmean(l2m[i1], l2m[i2]) * (rz2[cc] - rz1[cc]) / dz / dz;
                            S1 = (double)mu[i1] * dx1_rowd(g, coef1, rz1, ix, dx);
                        }
                    } else if (comp == 0) {
                        F1 = pops[OP_X2_L2M_X][i];
                        F2 = (double)pops[OP_ZX_LAM_Z][i] + (double)pops[OP_XZ_MU_Z][i];
                        F3 = pops[OP_Z2_MU_X][i];
                        S1 = (double)l2m[i] * cd1(g, coef1, Sx, iz, ix, 1, dx);
                        if (side >= 2) S3 = (double)mu[i] * cd1(g, coef1, Sx, iz, ix, 2, dz);
                    } else {
                        F1 = pops[OP_X2_MU_Z][i];
                        F2 = (double)pops[OP_XZ_LAM_X][i] + (double)pops[OP_ZX_MU_X][i];
                        F3 = pops[OP_Z2_L2M_Z][i];
                        S1 = (double)mu[i] * cd1(g, coef1, Sz, iz, ix, 1, dx);
                        if (side >= 2) S3 = (double)l2m[i] * cd1(g, coef1, Sz, iz, ix, 2, dz);
                    }
                    real_t *bpx = bp[side == 0 ? 0 + comp : side == 1 ? 2 + comp : side == 2 ? 8 + 2 * comp : 4 + 2 * comp];
                    real_t *bpz = side == 2 ? bp[9 + 2 * comp] : side == 3 ? bp[5 + 2 * comp] : NULL;
                    int base = (side == 0 ? 0 : side == 1 ? 6 : side == 2 ? 12 : 18) + 3 * comp;
                    real_t *b1 = bu[base], *b2 = bu[base + 1], *b3 = bu[base + 2];
                    double Px = bpx[ap];
                    double Pxn = ((1.0 - yx / 2) * Px - dt * dxp * S1) / (1.0 + yx / 2);
                    double u1 = b1[ab], u1m = b1[ab + 1];
                    double n1;
                    if (side == 1 && (top || iz != 1))
                        n1 = ((2.0 - yx * yx) * u1 - (1.0 - yx) * u1m) / (1.0 + yx) + k * (F1 + (Pxn + Px) / 2.0);
                    else
                        n1 = ((2.0 - yx * yx) * u1 - (1.0 - yx) * u1m + k * (F1 + (Pxn + Px) / 2.0)) / (1.0 + yx);
                    double u2 = b2[ab], u2m = b2[ab + 1];
                    double n2 = ((2.0 - yx * yz) * u2 - (1.0 - (yx + yz) / 2.0) * u2m + k * F2) / (1.0 + (yx + yz) / 2.0);
                    double u3 = b3[ab], u3m = b3[ab + 1];
                    double n3;
                    if (bpz) {
                        double Pz = bpz[ap];
                        double Pzn = ((1.0 - yz / 2) * Pz - dt * dzp * S3) / (1.0 + yz / 2);
                        bpz[ap] = (real_t)Pzn;
                        n3 = ((2.0 - yz * yz) * u3 - (1.0 - yz) * u3m + k * (F3 + (Pzn + Pz) / 2.0)) / (1.0 + yz);
                    } else {
                        n3 = 2.0 * u3 - u3m + k * F3;
                    }
                    bpx[ap] = (real_t)Pxn;
                    b1[ab + 1] = b1[ab]; b1[ab] = (real_t)n1;
                    b2[ab + 1] = b2[ab]; b2[ab] = (real_t)n2;
                    b3[ab + 1] = b3[ab]; b3[ab] = (real_t)n3;
                    if (comp == 0) nux1[i] = (real_t)(n1 + n2 + n3);
                    else nuz1[i] = (real_t)(n1 + n2 + n3);
                }
            }
        }
    }

    /* -------- commit levels for every updated cell -------- */
    for (int ix = 2 - npml; ix <= nx + npml - 1; ++ix)
        for (int iz = top ? p->izt + 1 : 1; iz <= nz + npml - 1; ++iz) {
            size_t i = gi(g, iz, ix);
            ux[2 * i + 1] = ux[2 * i]; ux[2 * i] = nux1[i];
            uz[2 * i + 1] = uz[2 * i]; uz[2 * i] = nuz1[i];
        }

    free(rowA); free(rowB); free(rz1); free(rz2); free(rx1); free(rx2);
    free(nux1); free(nuz1); free(px); free(pz); free(w); free(wd);
    return 0;
}

int fdfk_oracle_simulate(const fdfk_oracle_params *p, const real_t *const strips[12], const real_t *c, int nrcv,
                         const real_t *rx, const real_t *rz, real_t x0, real_t z0, int nstp, int nsis,
                         real_t *seisx, real_t *seisz, int steps_limit)
{
    if (p->izt != 1 && p->izt != 1 - p->npml) return -2;
    int nx = p->nx, nz = p->nz, npml = p->npml, norder = p->norder;
    size_t n = (size_t)(nz + npml - p->izt + 1) * (size_t)(nx + 2 * npml);
    real_t *ux = (real_t *)calloc(2 * n, sizeof(real_t)), *uz = (real_t *)calloc(2 * n, sizeof(real_t));
    size_t side = (size_t)nz * npml, tb = (size_t)npml * (nx + 2 * npml);
    real_t *bpbuf = (real_t *)calloc(4 * side + 8 * tb, sizeof(real_t));
    real_t *bubuf = (real_t *)calloc(2 * (12 * side + 12 * tb), sizeof(real_t));
    double *coef0 = (double *)malloc(sizeof(double) * norder * norder), *coef1 = (double *)malloc(sizeof(double) * norder * norder);
    if (!ux || !uz || !bpbuf || !bubuf || !coef0 || !coef1) {
        free(ux); free(uz); free(bpbuf); free(bubuf); free(coef0); free(coef1);
        return -3;
    }
    fdfk_op_fd_coef0(norder, coef0);
    fdfk_op_fd_coef1(norder, coef1);
    real_t *bp[12], *bu[24];
    {
        real_t *q = bpbuf;
        for (int k = 0; k < 4; ++k) { bp[k] = q; q += side; }
        for (int k = 4; k < 12; ++k) { bp[k] = q; q += tb; }
        q = bubuf;
        for (int k = 0; k < 12; ++k) { bu[k] = q; q += 2 * side; }
        for (int k = 12; k < 24; ++k) { bu[k] = q; q += 2 * tb; }
    }
    int isis = 0, istp = 0, rc = 0;
    int last = p->nt;
    if (steps_limit >= 0 && steps_limit - 1 < last) last = steps_limit - 1;
    for (int it = 0; it <= last && rc == 0; ++it) {
        if (isis == it && istp <= nsis) {
            for (int r = 0; r < nrcv; ++r)
                fdfk_op_loadseis(nx, nz, npml, p->izt, x0, z0, p->dx, p->dz, rx[r], rz[r], ux, uz,
                                 &seisx[(size_t)istp + (size_t)(nsis + 1) * r], &seisz[(size_t)istp + (size_t)(nsis + 1) * r]);
            istp++;
            isis += nstp;
        }
        rc = fdfk_oracle_updatedispl(p, it, strips, c, coef0, coef1, ux, uz, bp, bu);
    }
    free(ux); free(uz); free(bpbuf); free(bubuf); free(coef0); free(coef1);
    return rc;
}
