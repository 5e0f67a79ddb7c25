/*
 * ORACLE (test infrastructure only; never part of the product path).
 *
 * The FP64 GPU oracle: the restated hybrid FD-FK time loop of oracle/fdfk_oracle.c
 * (the closed `updatedispl_` of lib_gnu/libHybrid.so + libPML.so, called from
 * src/FDFK2D.f90:516-522, inside the loop of src/FDFK2D.f90:465-532) run on the GPU
 * with every field, intermediate and background sample in double precision.  It
 * exists so that the FP32 solver's traces can be stated against an FP64 run at
 * the full sizes of the workloads (4001 x 2001 cells, 12001 steps), where the CPU
 * restatement would take hours.  Same mathematics as the C restatement, in plain
 * one-thread-per-cell kernels:
 *
 *   prep    u^n + outer background (Omega_II) for the interior operators, u^n - inner
 *           background (Omega_I) for the absorbing-layer operators
 *           (fdfk_oracle.c apply_strips);
 *   vmix    the inner products M * D u of the eight mixed-derivative operators
 *           (src/Submain.f90:352-406, 450-501, 608-661, 704-756: diffzx/diffxz
 *           *_reg and *_pml), with each operator's own region and zero elsewhere;
 *   rows    the free-surface rows of the absorbing-layer field (fdfk_oracle.c);
 *   update  per cell: the operators it needs (diffx2/diffz2 with harmonic-mean
 *           moduli, src/Submain.f90:814-837, 988-1011; the outer passes of the mixed
 *           operators), then the leapfrog update of a regular cell (free-surface
 *           row included) or the split-field update of an absorbing-layer cell;
 *   sample  loadseis (src/Submain.f90:33-116) of level 1 at the sampled steps.
 *
 * The harmonic means of neighbouring moduli are formed once per half point (the
 * same two reciprocals, sum and quotient as the operators form per use), and the
 * divisions by dx, dz become multiplications by their reciprocals; in double
 * precision both differ from the C restatement by rounding only (the pinning test
 * checks agreement with oracle/_build/libfdfk_oracle64.so).  The levels rotate
 * by pointer instead of being copied: the outermost ring of cells, which no step
 * writes, stays zero in all three planes.
 *
 * Free-surface mode only (izt = 1), like the C restatement.
 */
#include <cuda_runtime.h>

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

extern "C" {

typedef struct {
    int norder, nx, nz, npml, izt, npower, nbd, nt;
    double dx, dz, dt, vpml, R0;
} fdfk_oracle_gpu_params;

int fdfk_oracle_gpu_simulate(const fdfk_oracle_gpu_params *p, const double *const strips_dev[12], const float *c_host,
                             int nrcv, const double *rx, const double *rz, double x0, double z0, int nstp, int nsis,
                             double *seisx, double *seisz, int steps_limit, double *ux_out, double *uz_out);
}

namespace {

constexpr int kMaxOrder = 8;
constexpr int kThreads = 256;

__constant__ double c_coef0[kMaxOrder * kMaxOrder];   // coef(j, n) at [(j-1) + (n-1)*kMaxOrder]
__constant__ double c_coef1[kMaxOrder * kMaxOrder];

struct Geo {
    int norder, nx, nz, npml, nbd, ldz, ldx, nt;
    double dx, dz, rdx, rdz, dx2, dz2, dt;
};

__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }
__device__ __forceinline__ size_t gi(const Geo &g, int iz, int ix)
{
    return (size_t)(iz - 1) + (size_t)(ix - (1 - g.npml)) * (size_t)g.ldz;
}
__device__ __forceinline__ double C0(int j, int n) { return c_coef0[(j - 1) + (n - 1) * kMaxOrder]; }
__device__ __forceinline__ double C1(int j, int n) { return c_coef1[(j - 1) + (n - 1) * kMaxOrder]; }
__device__ __forceinline__ bool in_rect(int iz, int ix, int zl, int zh, int xl, int xh)
{
    return iz >= zl && iz <= zh && ix >= xl && ix <= xh;
}
__device__ __forceinline__ int nox(const Geo &g, int ix) { return imin(imin(ix + g.npml - 1, g.nx + g.npml - ix), g.norder); }
__device__ __forceinline__ int noz(const Geo &g, int iz) { return imin(imin(iz - 1, g.nz + g.npml - iz), g.norder); }

/* strip element (r, c, t) of a Fortran array (n1, n2, nt+1), 0-based r, c */
__device__ __forceinline__ double strip_at(const double *s, int n1, int n2, int r, int c, int t)
{
    return s[(size_t)r + (size_t)n1 * ((size_t)c + (size_t)n2 * (size_t)t)];
}

struct Strips {
    const double *s[12];
};

// ---------------------------------------------------------------------------
// prep: tx/tz = u^n (+ outer background), px/pz = u^n (- inner background)
// ---------------------------------------------------------------------------
__global__ void k_prep(Geo g, Strips st, int it, const double *u1x, const double *u1z, double *tx, double *tz,
                       double *px, double *pz)
{
    const size_t n = (size_t)g.ldz * g.ldx;
    const size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const int iz = 1 + (int)(i % g.ldz), ix = (1 - g.npml) + (int)(i / g.ldz);
    const int nx = g.nx, nz = g.nz, nbd = g.nbd;
    double ax = 0.0, az = 0.0, bx = 0.0, bz = 0.0;
    // outer strips (Omega_II)
    if (iz >= 1 && iz <= nz && ix >= 1 - nbd && ix <= 0) {
        ax = strip_at(st.s[6], nz, nbd, iz - 1, ix - (1 - nbd), it);
        az = strip_at(st.s[7], nz, nbd, iz - 1, ix - (1 - nbd), it);
    } else if (iz >= 1 && iz <= nz && ix >= nx + 1 && ix <= nx + nbd) {
        ax = strip_at(st.s[8], nz, nbd, iz - 1, ix - (nx + 1), it);
        az = strip_at(st.s[9], nz, nbd, iz - 1, ix - (nx + 1), it);
    } else if (iz >= nz + 1 && iz <= nz + nbd && ix >= 1 - nbd && ix <= nx + nbd) {
        ax = strip_at(st.s[10], nbd, nx + 2 * nbd, iz - nz - 1, ix - (1 - nbd), it);
        az = strip_at(st.s[11], nbd, nx + 2 * nbd, iz - nz - 1, ix - (1 - nbd), it);
    }
    // inner strips (Omega_I; the left and right strips overlap when nx < 2 nbd, and both apply)
    if (iz >= 1 && iz <= nz - nbd && ix >= 1 && ix <= nbd) {
        bx += strip_at(st.s[0], nz - nbd, nbd, iz - 1, ix - 1, it);
        bz += strip_at(st.s[1], nz - nbd, nbd, iz - 1, ix - 1, it);
    }
    if (iz >= 1 && iz <= nz - nbd && ix >= nx - nbd + 1 && ix <= nx) {
        bx += strip_at(st.s[2], nz - nbd, nbd, iz - 1, ix - (nx - nbd + 1), it);
        bz += strip_at(st.s[3], nz - nbd, nbd, iz - 1, ix - (nx - nbd + 1), it);
    }
    if (iz >= nz - nbd + 1 && iz <= nz && ix >= 1 && ix <= nx) {
        bx += strip_at(st.s[4], nbd, nx, iz - (nz - nbd + 1), ix - 1, it);
        bz += strip_at(st.s[5], nbd, nx, iz - (nz - nbd + 1), ix - 1, it);
    }
    const double vx = u1x[i], vz = u1z[i];
    tx[i] = vx + ax;
    tz[i] = vz + az;
    px[i] = vx - bx;
    pz[i] = vz - bz;
}

// collocated derivatives (without the 1/d factor) with the edge-reduced orders of the operators
__device__ __forceinline__ double dz_c(const Geo &g, const double *u, int iz, int ix)
{
    const int no = noz(g, iz);
    double s = 0.0;
    for (int k = 1; k <= no; ++k) s += C1(k, no) * (u[gi(g, iz + k, ix)] - u[gi(g, iz - k, ix)]);
    return s;
}
__device__ __forceinline__ double dx_c(const Geo &g, const double *u, int iz, int ix)
{
    const int no = nox(g, ix);
    double s = 0.0;
    for (int k = 1; k <= no; ++k) s += C1(k, no) * (u[gi(g, iz, ix + k)] - u[gi(g, iz, ix - k)]);
    return s;
}

struct Mat {
    const double *rho, *lam, *mu, *l2m;
    const double *hx_l2m, *hx_mu, *hz_l2m, *hz_mu;   // harmonic means at (iz, ix+1/2) and (iz+1/2, ix)
};

struct VArr {
    double *zx_lam_z, *xz_lam_x, *xz_mu_z, *zx_mu_x;          // regular operators
    double *pzx_lam_z, *pxz_lam_x, *pxz_mu_z, *pzx_mu_x;      // absorbing-layer operators
};

// ---------------------------------------------------------------------------
// vmix: inner products of the mixed operators, each over its own region
// ---------------------------------------------------------------------------
__global__ void k_vmix(Geo g, Mat m, const double *tx, const double *tz, const double *px, const double *pz, VArr v)
{
    const size_t n = (size_t)g.ldz * g.ldx;
    const size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const int iz = 1 + (int)(i % g.ldz), ix = (1 - g.npml) + (int)(i / g.ldz);
    const int nx = g.nx, nz = g.nz, npml = g.npml, no = g.norder;
    // diffzx_reg: iz 2..nz, ix 1-norder..nx+norder: v = mat Dz u / dz
    const bool zx_reg = iz >= 2 && iz <= nz && ix >= 1 - no && ix <= nx + no;
    // diffxz_reg: ix 1..nx, iz 1..nz+norder: v = mat Dx u / dx
    const bool xz_reg = ix >= 1 && ix <= nx && iz >= 1 && iz <= nz + no;
    // diffzx_pml: iz 2..nz+npml-1, ix 2-npml..nx+npml-1 minus (1..nz, norder+1..nx-norder)
    const bool zx_pml = iz >= 2 && iz <= nz + npml - 1 && ix >= 2 - npml && ix <= nx + npml - 1 &&
                        !in_rect(iz, ix, 1, nz, no + 1, nx - no);
    // diffxz_pml: ix 2-npml..nx+npml-1, iz 1..nz+npml-1 minus (1..nz-norder, 1..nx)
    const bool xz_pml = ix >= 2 - npml && ix <= nx + npml - 1 && iz >= 1 && iz <= nz + npml - 1 &&
                        !in_rect(iz, ix, 1, nz - no, 1, nx);
    const double lam = m.lam[i], mu = m.mu[i];
    v.zx_lam_z[i] = zx_reg ? lam * dz_c(g, tz, iz, ix) * g.rdz : 0.0;
    v.zx_mu_x[i] = zx_reg ? mu * dz_c(g, tx, iz, ix) * g.rdz : 0.0;
    v.xz_lam_x[i] = xz_reg ? lam * dx_c(g, tx, iz, ix) * g.rdx : 0.0;
    v.xz_mu_z[i] = xz_reg ? mu * dx_c(g, tz, iz, ix) * g.rdx : 0.0;
    v.pzx_lam_z[i] = zx_pml ? lam * dz_c(g, pz, iz, ix) * g.rdz : 0.0;
    v.pzx_mu_x[i] = zx_pml ? mu * dz_c(g, px, iz, ix) * g.rdz : 0.0;
    v.pxz_lam_x[i] = xz_pml ? lam * dx_c(g, px, iz, ix) * g.rdx : 0.0;
    v.pxz_mu_z[i] = xz_pml ? mu * dx_c(g, pz, iz, ix) * g.rdx : 0.0;
}

// d/dx(M d/dx u) at (iz, ix) (src/Submain.f90:814-837), without the 1/dx^2 factor
__device__ double x2_point(const Geo &g, const double *hx, const double *u, int iz, int ix)
{
    const int nx = g.nx, npml = g.npml, norder = g.norder;
    const int no = nox(g, ix);
    double s = 0.0;
    for (int k = 1; k <= no; ++k) {
        const int i = k - 1;
        const int n1 = imin(imin(ix + i + npml - 1, nx + npml - ix - i), norder);
        double s1 = 0.0;
        for (int j = 1; j <= n1; ++j) s1 += C0(j, n1) * (u[gi(g, iz, ix + j + k - 1)] - u[gi(g, iz, ix - j + k)]);
        const int n2 = imin(imin(ix - i + npml - 1, nx + npml - ix + i), norder);
        double s2 = 0.0;
        for (int j = 1; j <= n2; ++j) s2 += C0(j, n2) * (u[gi(g, iz, ix + j - k)] - u[gi(g, iz, ix - j - k + 1)]);
        const double hp = hx[gi(g, iz, ix + k - 1)], hm = hx[gi(g, iz, ix - k)];
        s += C0(k, no) * (hp * s1 - hm * s2);
    }
    return s;
}

// d/dz(M d/dz u) at (iz, ix) (src/Submain.f90:988-1011), without the 1/dz^2 factor
__device__ double z2_point(const Geo &g, const double *hz, const double *u, int iz, int ix)
{
    const int nz = g.nz, npml = g.npml, norder = g.norder;
    const int no = noz(g, iz);
    double s = 0.0;
    for (int k = 1; k <= no; ++k) {
        const int i = k - 1;
        const int n1 = imin(imin(iz + i - 1, nz + npml - iz - i), norder);
        double s1 = 0.0;
        for (int j = 1; j <= n1; ++j) s1 += C0(j, n1) * (u[gi(g, iz + j + k - 1, ix)] - u[gi(g, iz - j + k, ix)]);
        const int n2 = imin(imin(iz - i - 1, nz + npml - iz + i), norder);
        double s2 = 0.0;
        for (int j = 1; j <= n2; ++j) s2 += C0(j, n2) * (u[gi(g, iz + j - k, ix)] - u[gi(g, iz - j - k + 1, ix)]);
        const double hp = hz[gi(g, iz + k - 1, ix)], hm = hz[gi(g, iz - k, ix)];
        s += C0(k, no) * (hp * s1 - hm * s2);
    }
    return s;
}

// ---------------------------------------------------------------------------
// rows: free-surface rows of the absorbing-layer field, per column
// ---------------------------------------------------------------------------
struct Rows {
    double *A, *B, *z1, *z2, *x1, *x2;
};

__global__ void k_rows(Geo g, Mat m, const double *px, const double *pz, Rows r)
{
    const int cc = blockIdx.x * kThreads + threadIdx.x;
    if (cc >= g.ldx) return;
    const int ix = cc + (1 - g.npml);
    const size_t i1 = gi(g, 1, ix), i2 = gi(g, 2, ix);
    r.A[cc] = m.lam[i1] * (pz[i2] - pz[i1]) * g.rdz;
    r.B[cc] = m.mu[i1] * (px[i2] - px[i1]) * g.rdz;
    r.z1[cc] = pz[i1];
    r.z2[cc] = pz[i2];
    r.x1[cc] = px[i1];
    r.x2[cc] = px[i2];
}

// collocated x-derivative of a row array indexed by column (1/dx applied)
__device__ __forceinline__ double dx_row(const Geo &g, const double *row, int ix)
{
    const int no = nox(g, ix);
    const int c = ix - (1 - g.npml);
    double s = 0.0;
    for (int k = 1; k <= no; ++k) s += C1(k, no) * (row[c + k] - row[c - k]);
    return s * g.rdx;
}

struct Pml {
    // per side s (0 left, 1 right, 2 bottom) and component c: split fields 1..3 with two levels
    // interleaved (level 1 at 2*a, level 2 at 2*a+1), memory variables Px (and Pz on the bottom)
    double *b[3][2][3];
    double *px[3][2];
    double *pz[2];
    double d0x, d0z, Lx, Lz;
    int npower;
};

__device__ __forceinline__ double hmean(double a, double b) { return 2.0 / (1.0 / a + 1.0 / b); }

// ---------------------------------------------------------------------------
// update: one cell of the regular domain or of an absorbing layer
// ---------------------------------------------------------------------------
__global__ void k_update(Geo g, Mat m, const double *u1x, const double *u1z, const double *u2x, const double *u2z,
                         const double *tx, const double *tz, const double *px, const double *pz, VArr v, Rows r,
                         Pml P, double *nx_out, double *nz_out)
{
    const size_t n = (size_t)g.ldz * g.ldx;
    const size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const int iz = 1 + (int)(i % g.ldz), ix = (1 - g.npml) + (int)(i / g.ldz);
    const int nx = g.nx, nz = g.nz, npml = g.npml;
    const double dt = g.dt;
    if (ix >= 1 && ix <= nx && iz >= 1 && iz <= nz) {
        double Fx, Fz;
        if (iz == 1) {
            const int no = nox(g, ix);
            double dA = 0.0, dB = 0.0;
            for (int k = 1; k <= no; ++k) {
                const double ck = C1(k, no);
                const size_t p1 = gi(g, 1, ix + k), p2 = gi(g, 2, ix + k), q1 = gi(g, 1, ix - k), q2 = gi(g, 2, ix - k);
                const double Ap = m.lam[p1] * (tz[p2] - tz[p1]) * g.rdz, Am = m.lam[q1] * (tz[q2] - tz[q1]) * g.rdz;
                const double Bp = m.mu[p1] * (tx[p2] - tx[p1]) * g.rdz, Bm = m.mu[q1] * (tx[q2] - tx[q1]) * g.rdz;
                dA += ck * (Ap - Am);
                dB += ck * (Bp - Bm);
            }
            dA *= g.rdx;
            dB *= g.rdx;
            const double dz1 = dx_c(g, tz, 1, ix) * g.rdx, dz2 = dx_c(g, tz, 2, ix) * g.rdx;
            const double dx1 = dx_c(g, tx, 1, ix) * g.rdx, dx2 = dx_c(g, tx, 2, ix) * g.rdx;
            const size_t i1 = gi(g, 1, ix), i2 = gi(g, 2, ix);
            const double sxz = hmean(m.mu[i1], m.mu[i2]) * (u1x[i2] - u1x[i1]) * g.rdz + (m.mu[i1] * dz1 + m.mu[i2] * dz2) / 2.0;
            const double szz = hmean(m.l2m[i1], m.l2m[i2]) * (u1z[i2] - u1z[i1]) * g.rdz + (m.lam[i1] * dx1 + m.lam[i2] * dx2) / 2.0;
            Fx = x2_point(g, m.hx_l2m, tx, iz, ix) * g.dx2 + dA + 2.0 * sxz * g.rdz;
            Fz = x2_point(g, m.hx_mu, tz, iz, ix) * g.dx2 + dB + 2.0 * szz * g.rdz;
        } else {
            Fx = x2_point(g, m.hx_l2m, tx, iz, ix) * g.dx2 + dx_c(g, v.zx_lam_z, iz, ix) * g.rdx +
                 z2_point(g, m.hz_mu, tx, iz, ix) * g.dz2 + dz_c(g, v.xz_mu_z, iz, ix) * g.rdz;
            Fz = z2_point(g, m.hz_l2m, tz, iz, ix) * g.dz2 + dz_c(g, v.xz_lam_x, iz, ix) * g.rdz +
                 x2_point(g, m.hx_mu, tz, iz, ix) * g.dx2 + dx_c(g, v.zx_mu_x, iz, ix) * g.rdx;
        }
        const double k = dt * dt / m.rho[i];
        nx_out[i] = 2.0 * u1x[i] - u2x[i] + k * Fx;
        nz_out[i] = 2.0 * u1z[i] - u2z[i] + k * Fz;
        return;
    }
    int side;
    if (iz >= 1 && iz <= nz && ix >= 2 - npml && ix <= 0) side = 0;
    else if (iz >= 1 && iz <= nz && ix >= nx + 1 && ix <= nx + npml - 1) side = 1;
    else if (iz >= nz + 1 && iz <= nz + npml - 1 && ix >= 2 - npml && ix <= nx + npml - 1) side = 2;
    else return;
    const int npw = P.npower;
    double dxv = 0.0, dxp = 0.0;
    if (ix <= 0) {
        const double s = (double)(1 - ix) * g.dx / P.Lx;
        dxv = P.d0x * pow(s, npw);
        dxp = -npw * P.d0x * pow(s, npw - 1) / P.Lx;
    } else if (ix > nx) {
        const double s = (double)(ix - nx) * g.dx / P.Lx;
        dxv = P.d0x * pow(s, npw);
        dxp = npw * P.d0x * pow(s, npw - 1) / P.Lx;
    }
    double dzv = 0.0, dzp = 0.0;
    if (side == 2) {
        const double s = (double)(iz - nz) * g.dz / P.Lz;
        dzv = P.d0z * pow(s, npw);
        dzp = npw * P.d0z * pow(s, npw - 1) / P.Lz;
    }
    const double yx = dxv * dt, yz = dzv * dt;
    const double k = dt * dt / m.rho[i];
    size_t ap;
    if (side == 0) ap = (size_t)(iz - 1) + (size_t)nz * (size_t)(ix - (1 - npml));
    else if (side == 1) ap = (size_t)(iz - 1) + (size_t)nz * (size_t)(ix - nx - 1);
    else ap = (size_t)(iz - nz - 1) + (size_t)npml * (size_t)(ix - (1 - npml));
    const size_t ab = 2 * ap;
    for (int comp = 0; comp < 2; ++comp) {
        double F1, F2, F3, S1, S3 = 0.0;
        if (iz == 1) {
            const int cc = ix - (1 - npml);
            const size_t i1 = gi(g, 1, ix), i2 = gi(g, 2, ix);
            if (comp == 0) {
                F1 = x2_point(g, m.hx_l2m, px, iz, ix) * g.dx2;
                F2 = dx_row(g, r.A, ix) + (m.mu[i1] * dx_row(g, r.z1, ix) + m.mu[i2] * dx_row(g, r.z2, ix)) * g.rdz;
                F3 = 2.0 * hmean(m.mu[i1], m.mu[i2]) * (r.x2[cc] - r.x1[cc]) * g.rdz * g.rdz;
                S1 = m.l2m[i1] * dx_row(g, r.x1, ix);
            } else {
                F1 = x2_point(g, m.hx_mu, pz, iz, ix) * g.dx2;
                F2 = dx_row(g, r.B, ix) + (m.lam[i1] * dx_row(g, r.x1, ix) + m.lam[i2] * dx_row(g, r.x2, ix)) * g.rdz;
                F3 = 2.0 * hmean(m.l2m[i1], m.l2m[i2]) * (r.z2[cc] - r.z1[cc]) * g.rdz * g.rdz;
                S1 = m.mu[i1] * dx_row(g, r.z1, ix);
            }
        } else if (comp == 0) {
            F1 = x2_point(g, m.hx_l2m, px, iz, ix) * g.dx2;
            F2 = dx_c(g, v.pzx_lam_z, iz, ix) * g.rdx + dz_c(g, v.pxz_mu_z, iz, ix) * g.rdz;
            F3 = z2_point(g, m.hz_mu, px, iz, ix) * g.dz2;
            S1 = m.l2m[i] * dx_c(g, px, iz, ix) * g.rdx;
            if (side == 2) S3 = m.mu[i] * dz_c(g, px, iz, ix) * g.rdz;
        } else {
            F1 = x2_point(g, m.hx_mu, pz, iz, ix) * g.dx2;
            F2 = dz_c(g, v.pxz_lam_x, iz, ix) * g.rdz + dx_c(g, v.pzx_mu_x, iz, ix) * g.rdx;
            F3 = z2_point(g, m.hz_l2m, pz, iz, ix) * g.dz2;
            S1 = m.mu[i] * dx_c(g, pz, iz, ix) * g.rdx;
            if (side == 2) S3 = m.l2m[i] * dz_c(g, pz, iz, ix) * g.rdz;
        }
        double *b1 = P.b[side][comp][0], *b2 = P.b[side][comp][1], *b3 = P.b[side][comp][2];
        double *bpx = P.px[side][comp];
        const double Px = bpx[ap];
        const double Pxn = ((1.0 - yx / 2) * Px - dt * dxp * S1) / (1.0 + yx / 2);
        const double u1 = b1[ab], u1m = b1[ab + 1];
        double n1;
        if (side == 1 && iz != 1)
            n1 = ((2.0 - yx * yx) * u1 - (1.0 - yx) * u1m) / (1.0 + yx) + k * (F1 + (Pxn + Px) / 2.0);
        else
            n1 = ((2.0 - yx * yx) * u1 - (1.0 - yx) * u1m + k * (F1 + (Pxn + Px) / 2.0)) / (1.0 + yx);
        const double u2 = b2[ab], u2m = b2[ab + 1];
        const double n2 = ((2.0 - yx * yz) * u2 - (1.0 - (yx + yz) / 2.0) * u2m + k * F2) / (1.0 + (yx + yz) / 2.0);
        const double u3 = b3[ab], u3m = b3[ab + 1];
        double n3;
        if (side == 2) {
            double *bpz = P.pz[comp];
            const double Pz = bpz[ap];
            const double Pzn = ((1.0 - yz / 2) * Pz - dt * dzp * S3) / (1.0 + yz / 2);
            bpz[ap] = Pzn;
            n3 = ((2.0 - yz * yz) * u3 - (1.0 - yz) * u3m + k * (F3 + (Pzn + Pz) / 2.0)) / (1.0 + yz);
        } else {
            n3 = 2.0 * u3 - u3m + k * F3;
        }
        bpx[ap] = Pxn;
        b1[ab + 1] = u1; b1[ab] = n1;
        b2[ab + 1] = u2; b2[ab] = n2;
        b3[ab + 1] = u3; b3[ab] = n3;
        if (comp == 0) nx_out[i] = n1 + n2 + n3;
        else nz_out[i] = n1 + n2 + n3;
    }
}

// ---------------------------------------------------------------------------
// material and half-point harmonic means
// ---------------------------------------------------------------------------
__global__ void k_material(Geo g, const float *c, double *rho, double *lam, double *mu, double *l2m)
{
    const size_t n = (size_t)g.ldz * g.ldx;
    const size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    rho[i] = c[3 * i];
    lam[i] = c[3 * i + 1];
    mu[i] = c[3 * i + 2];
    l2m[i] = (double)c[3 * i + 1] + 2.0 * (double)c[3 * i + 2];
}

__global__ void k_hmeans(Geo g, const double *l2m, const double *mu, double *hx_l2m, double *hx_mu, double *hz_l2m,
                         double *hz_mu)
{
    const size_t n = (size_t)g.ldz * g.ldx;
    const size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    const int iz = 1 + (int)(i % g.ldz), ix = (1 - g.npml) + (int)(i / g.ldz);
    // same operand order as the operators: 2 / (1/M(right) + 1/M(left))
    if (ix < g.nx + g.npml) {
        const size_t j = gi(g, iz, ix + 1);
        hx_l2m[i] = 2.0 / (1.0 / l2m[j] + 1.0 / l2m[i]);
        hx_mu[i] = 2.0 / (1.0 / mu[j] + 1.0 / mu[i]);
    } else {
        hx_l2m[i] = hx_mu[i] = 0.0;
    }
    if (iz < g.ldz) {
        const size_t j = gi(g, iz + 1, ix);
        hz_l2m[i] = 2.0 / (1.0 / l2m[j] + 1.0 / l2m[i]);
        hz_mu[i] = 2.0 / (1.0 / mu[j] + 1.0 / mu[i]);
    } else {
        hz_l2m[i] = hz_mu[i] = 0.0;
    }
}

// ---------------------------------------------------------------------------
// loadseis: one thread per receiver, level 1 (src/Submain.f90:33-116)
// ---------------------------------------------------------------------------
__device__ double delta_weight(double x)
{
    const double x2 = x * x, x3 = x2 * x;
    if (x <= 1.0) return 1.0 + x2 * (-5.0 / 4.0 + x2 * (21.0 / 4.0)) + x3 * (-35.0 / 12.0 + x2 * (-25.0 / 12.0));
    if (x <= 2.0)
        return -4.0 + (75.0 / 4.0) * x + x2 * (-245.0 / 8.0 + x2 * (-63.0 / 8.0)) + x3 * (545.0 / 24.0 + x2 * (25.0 / 24.0));
    if (x <= 3.0)
        return 18.0 + (-153.0 / 4.0) * x + x2 * (255.0 / 8.0 + x2 * (21.0 / 8.0)) + x3 * (-313.0 / 24.0 + x2 * (-5.0 / 24.0));
    return 0.0;
}

__global__ void k_sample(Geo g, const double *ux, const double *uz, int nrcv, const double *rx, const double *rz,
                         double x0, double z0, double dx, double dz, int istp, int nsamp, double *sx, double *sz)
{
    const int r = blockIdx.x * kThreads + threadIdx.x;
    if (r >= nrcv) return;
    const int irx = (int)floor((rx[r] - x0) / dx) + 1;
    const int irz = (int)floor((rz[r] - z0) / dz) + 1;
    double ax = 0.0, az = 0.0;
    const int xlo = irx - 3 > 1 - g.npml ? irx - 3 : 1 - g.npml, xhi = imin(g.nx + g.npml, irx + 3);
    const int zlo = irz - 3 > 1 ? irz - 3 : 1, zhi = imin(g.nz + g.npml, irz + 3);
    for (int ix = xlo; ix <= xhi; ++ix) {
        const double bx = delta_weight(fabs(x0 + (double)(ix - 1) * dx - rx[r]) / dx);
        for (int iz = zlo; iz <= zhi; ++iz) {
            const double ba = bx * delta_weight(fabs(z0 + (double)(iz - 1) * dz - rz[r]) / dz);
            const size_t o = gi(g, iz, ix);
            ax += ba * ux[o];
            az += ba * uz[o];
        }
    }
    sx[(size_t)istp + (size_t)nsamp * r] = ax;
    sz[(size_t)istp + (size_t)nsamp * r] = az;
}

// restated fd_coef0 / fd_coef1 (src/Submain.f90:1111-1245), coef(j, n) for every reduced order n
void fd_coefs(int norder, double *c0, double *c1)
{
    memset(c0, 0, sizeof(double) * kMaxOrder * kMaxOrder);
    memset(c1, 0, sizeof(double) * kMaxOrder * kMaxOrder);
    for (int i = 1; i <= norder; ++i)
        for (int j = 1; j <= i; ++j) {
            double t1 = 1.0, t2 = 1.0, t3 = 1.0, u1 = 1.0, u2 = 1.0, u3 = 1.0;
            const double oj = (double)((2 * j - 1) * (2 * j - 1)), jj = (double)(j * j);
            for (int k = 1; k <= j - 1; ++k) {
                const double ok = (double)((2 * k - 1) * (2 * k - 1)), kk = (double)(k * k);
                t1 *= ok; t2 *= (oj - ok);
                u1 *= kk; u2 *= (jj - kk);
            }
            for (int k = j + 1; k <= i; ++k) {
                const double ok = (double)((2 * k - 1) * (2 * k - 1)), kk = (double)(k * k);
                t1 *= ok; t3 *= (ok - oj);
                u1 *= kk; u3 *= (kk - jj);
            }
            const double sg = ((j + 1) % 2 == 0) ? 1.0 : -1.0;
            c0[(j - 1) + (i - 1) * kMaxOrder] = sg * t1 / (t2 * (double)(2 * j - 1)) / t3;
            c1[(j - 1) + (i - 1) * kMaxOrder] = sg * u1 / (u2 * 2.0 * (double)j) / u3;
        }
}

struct Pool {
    void *ptrs[128];
    int n = 0;
    cudaError_t err = cudaSuccess;
    double *get(size_t count)
    {
        void *p = nullptr;
        if (err != cudaSuccess || n >= 128) return nullptr;
        err = cudaMalloc(&p, sizeof(double) * (count ? count : 1));
        if (err != cudaSuccess) return nullptr;
        cudaMemset(p, 0, sizeof(double) * (count ? count : 1));
        ptrs[n++] = p;
        return (double *)p;
    }
    ~Pool()
    {
        for (int i = 0; i < n; ++i) cudaFree(ptrs[i]);
    }
};

}  // namespace

/*
 * The FP64 time loop it = 0..nt (or the first steps_limit steps) with receiver sampling every nstp
 * steps into seisx/seisz ((nsis+1) x nrcv, sample fastest; host memory).  strips_dev: the twelve
 * background strips in double precision, device memory, reference layout (n1, n2, nt+1).  c_host:
 * material (rho, lambda, mu) as float (3, nz+npml, nx+2npml).  ux_out/uz_out (optional, host,
 * (nz+npml) x (nx+2npml) doubles): level 1 after the last step.  Returns 0 or a negative code.
 */
int fdfk_oracle_gpu_simulate(const fdfk_oracle_gpu_params *p, const double *const strips_dev[12], const float *c_host,
                             int nrcv, const double *rx, const double *rz, double x0, double z0, int nstp, int nsis,
                             double *seisx, double *seisz, int steps_limit, double *ux_out, double *uz_out)
{
    if (p->izt != 1) return -2;
    if (p->norder < 1 || p->norder > kMaxOrder || p->nbd != 2 * p->norder - 1 || p->npml < p->nbd || p->nz <= p->nbd ||
        p->nx < 1 || nstp < 1)
        return -1;
    Geo g;
    g.norder = p->norder; g.nx = p->nx; g.nz = p->nz; g.npml = p->npml; g.nbd = p->nbd; g.nt = p->nt;
    g.ldz = p->nz + p->npml;
    g.ldx = p->nx + 2 * p->npml;
    g.dx = p->dx; g.dz = p->dz;
    g.rdx = 1.0 / p->dx; g.rdz = 1.0 / p->dz;
    g.dx2 = 1.0 / (p->dx * p->dx); g.dz2 = 1.0 / (p->dz * p->dz);
    g.dt = p->dt;
    const size_t n = (size_t)g.ldz * g.ldx;
    double c0[kMaxOrder * kMaxOrder], c1[kMaxOrder * kMaxOrder];
    fd_coefs(p->norder, c0, c1);
    if (cudaMemcpyToSymbol(c_coef0, c0, sizeof(c0)) != cudaSuccess) return -4;
    if (cudaMemcpyToSymbol(c_coef1, c1, sizeof(c1)) != cudaSuccess) return -4;

    Pool pool;
    double *rho = pool.get(n), *lam = pool.get(n), *mu = pool.get(n), *l2m = pool.get(n);
    double *hxl = pool.get(n), *hxm = pool.get(n), *hzl = pool.get(n), *hzm = pool.get(n);
    double *U[3][2];
    for (int l = 0; l < 3; ++l)
        for (int c = 0; c < 2; ++c) U[l][c] = pool.get(n);
    double *tx = pool.get(n), *tz = pool.get(n), *px = pool.get(n), *pz = pool.get(n);
    VArr v{pool.get(n), pool.get(n), pool.get(n), pool.get(n), pool.get(n), pool.get(n), pool.get(n), pool.get(n)};
    Rows rows{pool.get(g.ldx), pool.get(g.ldx), pool.get(g.ldx), pool.get(g.ldx), pool.get(g.ldx), pool.get(g.ldx)};
    Pml P;
    const size_t side_n = (size_t)p->nz * p->npml, bot_n = (size_t)p->npml * g.ldx;
    for (int s = 0; s < 3; ++s)
        for (int c = 0; c < 2; ++c) {
            const size_t m = s < 2 ? side_n : bot_n;
            for (int k = 0; k < 3; ++k) P.b[s][c][k] = pool.get(2 * m);
            P.px[s][c] = pool.get(m);
        }
    P.pz[0] = pool.get(bot_n);
    P.pz[1] = pool.get(bot_n);
    const double logr = log(1.0 / p->R0);
    P.d0x = (p->npower + 1) * p->vpml * logr / (2.0 * p->npml * p->dx);
    P.d0z = (p->npower + 1) * p->vpml * logr / (2.0 * p->npml * p->dz);
    P.Lx = (double)p->npml * p->dx;
    P.Lz = (double)p->npml * p->dz;
    P.npower = p->npower;
    const int nsamp = nsis + 1;
    double *srx = pool.get(nrcv), *srz = pool.get(nrcv);
    double *sx = pool.get((size_t)nsamp * nrcv), *sz = pool.get((size_t)nsamp * nrcv);
    float *cd = nullptr;
    if (pool.err != cudaSuccess) return -3;
    if (cudaMalloc(&cd, sizeof(float) * 3 * n) != cudaSuccess) return -3;
    int rc = 0;
    do {
        if (cudaMemcpy(cd, c_host, sizeof(float) * 3 * n, cudaMemcpyHostToDevice) != cudaSuccess) { rc = -4; break; }
        if (nrcv > 0) {
            cudaMemcpy(srx, rx, sizeof(double) * nrcv, cudaMemcpyHostToDevice);
            cudaMemcpy(srz, rz, sizeof(double) * nrcv, cudaMemcpyHostToDevice);
        }
        const unsigned blocks = (unsigned)((n + kThreads - 1) / kThreads);
        k_material<<<blocks, kThreads>>>(g, cd, rho, lam, mu, l2m);
        k_hmeans<<<blocks, kThreads>>>(g, l2m, mu, hxl, hxm, hzl, hzm);
        Mat m{rho, lam, mu, l2m, hxl, hxm, hzl, hzm};
        Strips st;
        for (int k = 0; k < 12; ++k) st.s[k] = strips_dev[k];
        int last = p->nt;
        if (steps_limit >= 0 && steps_limit - 1 < last) last = steps_limit - 1;
        int isis = 0, istp = 0;
        int l1 = 0, l2 = 1, ln = 2;   // planes holding level 1, level 2 and the next level
        for (int it = 0; it <= last; ++it) {
            if (isis == it && istp <= nsis) {
                if (nrcv > 0)
                    k_sample<<<(nrcv + kThreads - 1) / kThreads, kThreads>>>(g, U[l1][0], U[l1][1], nrcv, srx, srz, x0, z0,
                                                                            p->dx, p->dz, istp, nsamp, sx, sz);
                istp++;
                isis += nstp;
            }
            k_prep<<<blocks, kThreads>>>(g, st, it, U[l1][0], U[l1][1], tx, tz, px, pz);
            k_vmix<<<blocks, kThreads>>>(g, m, tx, tz, px, pz, v);
            k_rows<<<(g.ldx + kThreads - 1) / kThreads, kThreads>>>(g, m, px, pz, rows);
            k_update<<<blocks, kThreads>>>(g, m, U[l1][0], U[l1][1], U[l2][0], U[l2][1], tx, tz, px, pz, v, rows, P,
                                           U[ln][0], U[ln][1]);
            const int t = l2;
            l2 = l1;
            l1 = ln;
            ln = t;
            if ((it & 255) == 255 && cudaGetLastError() != cudaSuccess) { rc = -5; break; }
        }
        if (rc) break;
        if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) { rc = -5; break; }
        if (nrcv > 0) {
            cudaMemcpy(seisx, sx, sizeof(double) * nsamp * nrcv, cudaMemcpyDeviceToHost);
            cudaMemcpy(seisz, sz, sizeof(double) * nsamp * nrcv, cudaMemcpyDeviceToHost);
        }
        if (ux_out) cudaMemcpy(ux_out, U[l1][0], sizeof(double) * n, cudaMemcpyDeviceToHost);
        if (uz_out) cudaMemcpy(uz_out, U[l1][1], sizeof(double) * n, cudaMemcpyDeviceToHost);
        if (cudaGetLastError() != cudaSuccess) rc = -5;
    } while (0);
    cudaFree(cd);
    return rc;
}
