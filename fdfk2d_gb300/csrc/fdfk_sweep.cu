// Fused hybrid FD-FK time step for sm_103a.  See fdfk_sweep.cuh.
//
// Operator semantics follow FDFK2D src/Submain.f90:
//   dxx(M u)  diffx2_* (:764-937)  staggered derivative of H(M) * staggered derivative
//   dzz(M u)  diffz2_* (:939-1109)
//   dzx(M u)  diffzx_* (:251-507)  collocated d/dx of M * collocated d/dz u
//   dxz(M u)  diffxz_* (:509-762)  collocated d/dz of M * collocated d/dx u
// with edge-reduced orders norder(ix) = min(ix+npml-1, nx+npml-ix, norder),
// norder(iz) = min(iz-izt, nz+npml-iz, norder).  H is the harmonic mean
// 2/(1/M_a + 1/M_b), formed with IEEE divisions as the reference forms it.
//
// The staggered products G = H * D_stag(u) are formed once per half point in
// shared memory and reused by the 2*norder output cells that read them; the
// reference recomputes them per output cell.  At a half point between cells a
// and a+1 the reference uses order(a) when the point lies right of the output
// cell and order(a+1) when it lies left of it; the two differ only within
// norder cells of the outer frame, where the second variant is recomputed.
#include "fdfk_sweep.cuh"

#include <cuda_runtime.h>

#include <algorithm>

namespace fdfk {

__constant__ float c_stag[kMaxOrder + 1][kMaxOrder + 1];  // [n][j]: fd_coef0(j, n), zero for j > n
__constant__ float c_coll[kMaxOrder + 1][kMaxOrder + 1];  // [n][j]: fd_coef1(j, n)

// Free-surface forcing terms of a row-1 cell, formed once per column of a tile that holds row 1:
// the interior update's (Dx[lam dz uz] and the half-row stress term of each component, added in
// that order), and the split-field update's F2 and F3 of each component.
enum { kFsA, kFsQx, kFsB, kFsQz, kFsF2x, kFsF3x, kFsF2z, kFsF3z, kFsTerms };

// Shared-memory layout of a TZ x TX tile (z fastest) for stencil half-order NO.
struct TileDims {
    int TZ, TX;
    int H;          // reach of dxx / dzz
    int UZ, UX;     // u tile
    int MZ, MX;     // material tile
    int XW, ZW;     // extents of the x- / z-consumed arrays
    int U, M, AX, AZ;
    int FS;         // free-surface terms of row 1 (kFsTerms per column)
    int total;      // floats
};

__host__ __device__ __forceinline__ TileDims tile_dims(int NO, int TZ, int TX)
{
    TileDims t;
    t.TZ = TZ; t.TX = TX;
    t.H = 2 * NO - 1;
    t.UZ = TZ + 2 * t.H; t.UX = TX + 2 * t.H;
    t.MZ = TZ + 2 * NO; t.MX = TX + 2 * NO;
    t.XW = TX + 2 * NO; t.ZW = TZ + 2 * NO;
    t.U = t.UZ * t.UX; t.M = t.MZ * t.MX;
    t.AX = TZ * t.XW; t.AZ = t.ZW * TX;
    t.FS = kFsTerms * TX;
    t.total = 2 * t.U + 4 * t.M + 4 * t.AX + 4 * t.AZ + t.FS;
    return t;
}

struct Rect {
    int side;       // 0 interior, 1 left PML, 2 right PML, 3 bottom PML
    int cls;        // tile class (StepArgs::tdz / tdx): 0 interior, 1 side PML, 2 bottom PML
    int z0, x0;     // first row / column of the tile
    int zlo, zhi, xlo, xhi;  // output rectangle (inclusive)
};

// Reciprocal to within 1 ulp (MUFU); the reference's IEEE divisions agree to rounding.
__device__ __forceinline__ float fast_rcp(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// (i % n, i / n) along i = i0, i0 + step, ... without a division per step.
struct Walk {
    int r, q, dr, dq, n;
    __device__ __forceinline__ Walk(int i0, int n_, int step)
        : r(i0 % n_), q(i0 / n_), dr(step % n_), dq(step / n_), n(n_) {}
    __device__ __forceinline__ void next()
    {
        r += dr;
        q += dq;
        if (r >= n) {
            r -= n;
            ++q;
        }
    }
};

__device__ __forceinline__ int ordx(const StepArgs& a, int ix, int NO)
{
    int n = min(min(ix + a.npml - 1, a.nx + a.npml - ix), NO);
    return n < 0 ? 0 : n;
}
__device__ __forceinline__ int ordz(const StepArgs& a, int iz, int NO)
{
    int n = min(min(iz - 1, a.nz + a.npml - iz), NO);
    return n < 0 ? 0 : n;
}
__device__ __forceinline__ size_t gidx(const StepArgs& a, int iz, int ix)
{
    return (size_t)(iz - 1) + (size_t)(ix + a.npml - 1) * (size_t)a.ldz;
}

// Address of the background at (iz, ix) on the outer strips (Omega_II): the x component,
// with the z component in pz; nullptr where there is none.
__device__ __forceinline__ const float* outer_bg_ptr(const StepArgs& a, int iz, int ix, const float*& pz)
{
    const int nx = a.nx, nz = a.nz, nbd = a.nbd, it = a.it;
    if (iz >= 1 && iz <= nz) {
        if (ix >= 1 - nbd && ix <= 0) {
            const size_t o = (size_t)(iz - 1) + (size_t)nz * ((size_t)(ix - (1 - nbd)) + (size_t)nbd * it);
            pz = a.strip[UZL_PML] + o;
            return a.strip[UXL_PML] + o;
        }
        if (ix >= nx + 1 && ix <= nx + nbd) {
            const size_t o = (size_t)(iz - 1) + (size_t)nz * ((size_t)(ix - nx - 1) + (size_t)nbd * it);
            pz = a.strip[UZR_PML] + o;
            return a.strip[UXR_PML] + o;
        }
    } else if (iz >= nz + 1 && iz <= nz + nbd && ix >= 1 - nbd && ix <= nx + nbd) {
        const size_t o = (size_t)(iz - nz - 1) + (size_t)nbd * ((size_t)(ix - (1 - nbd)) + (size_t)(nx + 2 * nbd) * it);
        pz = a.strip[UZB_PML] + o;
        return a.strip[UXB_PML] + o;
    }
    return nullptr;
}

// Address of the background at (iz, ix) on the inner strips (Omega_I), as outer_bg_ptr.
__device__ __forceinline__ const float* inner_bg_ptr(const StepArgs& a, int iz, int ix, const float*& pz)
{
    const int nx = a.nx, nz = a.nz, nbd = a.nbd, it = a.it;
    if (ix < 1 || ix > nx || iz < 1 || iz > nz) return nullptr;
    if (iz <= nz - nbd) {
        if (ix <= nbd) {
            const size_t o = (size_t)(iz - 1) + (size_t)(nz - nbd) * ((size_t)(ix - 1) + (size_t)nbd * it);
            pz = a.strip[UZL_REG] + o;
            return a.strip[UXL_REG] + o;
        }
        if (ix >= nx - nbd + 1) {
            const size_t o = (size_t)(iz - 1) + (size_t)(nz - nbd) * ((size_t)(ix - (nx - nbd + 1)) + (size_t)nbd * it);
            pz = a.strip[UZR_REG] + o;
            return a.strip[UXR_REG] + o;
        }
        return nullptr;
    }
    const size_t o = (size_t)(iz - (nz - nbd + 1)) + (size_t)nbd * ((size_t)(ix - 1) + (size_t)nx * it);
    pz = a.strip[UZB_REG] + o;
    return a.strip[UXB_REG] + o;
}

__device__ __forceinline__ Rect decode_tile(const StepArgs& a, int b)
{
    Rect r;
    int ni = a.tiles_int_z * a.tiles_int_x;
    int nl = a.tiles_l_z * a.tiles_l_x;
    if (b < ni) {
        r.side = 0;
        r.cls = 0;
        r.z0 = 1 + (b % a.tiles_int_z) * a.tdz[0]; r.x0 = 1 + (b / a.tiles_int_z) * a.tdx[0];
        r.zlo = 1; r.zhi = a.int_rows; r.xlo = 1; r.xhi = a.nx;
        return r;
    }
    b -= ni;
    if (b < 2 * nl) {
        int right = b >= nl;
        if (right) b -= nl;
        r.side = right ? 2 : 1;
        r.cls = 1;
        r.zlo = 1; r.zhi = a.nz;
        r.xlo = right ? a.nx + 1 : 1 - a.npml;
        r.xhi = right ? a.nx + a.npml : 0;
        r.z0 = 1 + (b % a.tiles_l_z) * a.tdz[1]; r.x0 = r.xlo + (b / a.tiles_l_z) * a.tdx[1];
        return r;
    }
    b -= 2 * nl;
    r.side = 3;
    r.cls = 2;
    r.zlo = a.nz + 1; r.zhi = a.nz + a.npml; r.xlo = 1 - a.npml; r.xhi = a.nx + a.npml;
    r.z0 = r.zlo + (b % a.tiles_b_z) * a.tdz[2]; r.x0 = r.xlo + (b / a.tiles_b_z) * a.tdx[2];
    return r;
}

// ---------------------------------------------------------------------------
// Receiver sampling (loadseis, src/Submain.f90:33-116), FP64 weights and sum.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double delta_weight(double x)
{
    double x2 = x * x, x3 = x2 * x;
    if (x <= 1.0) return 1.0 + x2 * (-5.0 / 4.0 + x2 * (21.0 / 4.0)) + x3 * (-35.0 / 12.0 + x2 * (-25.0 / 12.0));
    if (x <= 2.0)
        return -4.0 + (75.0 / 4.0) * x + x2 * (-245.0 / 8.0 + x2 * (-63.0 / 8.0)) + x3 * (545.0 / 24.0 + x2 * (25.0 / 24.0));
    if (x <= 3.0)
        return 18.0 + (-153.0 / 4.0) * x + x2 * (255.0 / 8.0 + x2 * (21.0 / 8.0)) + x3 * (-313.0 / 24.0 + x2 * (-5.0 / 24.0));
    return 0.0;
}

// The grid point (irx, irz) a receiver's 7 x 7 neighbourhood is centred on, which points of it lie
// in the model (bit q of the masks: point q = 7 * (column offset + 3) + row offset + 3) and each
// point's FP64 weight; formed once when the receivers are set.  Block r, 64 threads: thread q < 49
// forms point q.
__global__ void receiver_sites_kernel(int nrcv, int nx, int nz, int npml, float dx, float dz, float x0, float z0,
                                      const float* __restrict__ rxs, const float* __restrict__ rzs,
                                      int4* __restrict__ site, double* __restrict__ wout)
{
    const int r = blockIdx.x, q = threadIdx.x;
    if (r >= nrcv) return;
    const float rx = rxs[r], rz = rzs[r];
    const int irx = (int)floorf((rx - x0) / dx) + 1;
    const int irz = (int)floorf((rz - z0) / dz) + 1;
    const int xlo = max(1 - npml, irx - 3), xhi = min(nx + npml, irx + 3);
    const int zlo = max(1, irz - 3), zhi = min(nz + npml, irz + 3);
    const int ix = irx - 3 + q / 7, iz = irz - 3 + q % 7;
    const bool in = q < 49 && ix >= xlo && ix <= xhi && iz >= zlo && iz <= zhi;
    double w = 0.0;
    if (in) {
        const double x = fabs((double)__fadd_rn(x0, __fmul_rn((float)(ix - 1), dx)) - (double)rx) / (double)dx;
        const double z = fabs((double)__fadd_rn(z0, __fmul_rn((float)(iz - 1), dz)) - (double)rz) / (double)dz;
        w = delta_weight(x) * delta_weight(z);
    }
    if (q < 49) wout[(size_t)r * 49 + q] = w;
    const unsigned m = __ballot_sync(0xffffffffu, in);
    if ((q & 31) == 0) {
        int* s = reinterpret_cast<int*>(site + r);
        if (q == 0) { s[0] = irx; s[1] = irz; s[2] = (int)m; }
        else s[3] = (int)m;
    }
}

cudaError_t launch_receiver_sites(const StepArgs& a, int nrcv, float x0, float z0, const float* rx,
                                  const float* rz, int4* site, double* w, cudaStream_t s)
{
    if (nrcv <= 0) return cudaSuccess;
    receiver_sites_kernel<<<nrcv, 64, 0, s>>>(nrcv, a.nx, a.nz, a.npml, a.dx, a.dz, x0, z0, rx, rz, site, w);
    return cudaGetLastError();
}

// One warp per receiver: the lanes share the (at most) 7 x 7 grid points, each adds its points'
// weighted displacements in FP64 (weights formed by receiver_sites_kernel), and a shuffle reduction
// sums them (FP64).
__device__ void sample_receivers(const StepArgs& a, int blk)
{
    const int lane = threadIdx.x & 31;
    const int r = blk * (kThreads / 32) + (threadIdx.x >> 5);
    if (r >= a.nrcv) return;
    const float* ux = a.ux[a.cur];
    const float* uz = a.uz[a.cur];
    const int4 st = a.rsite[r];
    const double* w = a.rw + (size_t)r * 49;
    double sx = 0.0, sz = 0.0;
    for (int q = lane; q < 49; q += 32) {
        if ((((unsigned)(q < 32 ? st.z : st.w) >> (q & 31)) & 1u) == 0u) continue;
        const int ix = st.x - 3 + q / 7, iz = st.y - 3 + q % 7;
        const size_t g = gidx(a, iz, ix);
        const double wq = w[q];
        sx += wq * (double)ux[g];
        sz += wq * (double)uz[g];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_down_sync(0xffffffffu, sx, o);
        sz += __shfl_down_sync(0xffffffffu, sz, o);
    }
    if (lane == 0) {
        const size_t o = (size_t)a.sample_index + (size_t)a.nsamp * (size_t)r;
        a.seisx[o] = (float)sx;
        a.seisz[o] = (float)sz;
    }
}

// ---------------------------------------------------------------------------
// The step kernel.
// ---------------------------------------------------------------------------
// Block `blk` of one solve's tiled launch: a tile of the top band, an absorbing layer, or (past
// n_tiles) a block of receivers.
template <int NO>
__device__ __forceinline__ void step_block(const StepArgs& a, int blk)
{
    constexpr int H = 2 * NO - 1;
    extern __shared__ float sm[];
    if (blk >= a.n_tiles) {
        sample_receivers(a, blk - a.n_tiles);
        return;
    }
    const Rect R = decode_tile(a, blk);
    const TileDims T = tile_dims(NO, a.tdz[R.cls], a.tdx[R.cls]);
    const int TZ = T.TZ, TX = T.TX;
    const bool pml = R.side != 0;
    const int tid = threadIdx.x;
    const int nx = a.nx, nz = a.nz, npml = a.npml;
    const int NZ = a.NZ;

    float* sux = sm;
    float* suz = sux + T.U;
    float* sLam = suz + T.U;
    float* sMu = sLam + T.M;
    float* sRL2m = sMu + T.M;
    float* sRMu = sRL2m + T.M;
    float* gxA = sRMu + T.M;   // H(l2m) * Dstag_x(ux)   [label][z]
    float* gxB = gxA + T.AX;   // H(mu)  * Dstag_x(uz)
    float* v1 = gxB + T.AX;    // lam * Dz(uz)/dz        [x][z]  (dzx(lam uz))
    float* v4 = v1 + T.AX;     // mu  * Dz(ux)/dz                 (dzx(mu ux))
    float* gzA = v4 + T.AX;    // H(l2m) * Dstag_z(uz)   [x][label]
    float* gzB = gzA + T.AZ;   // H(mu)  * Dstag_z(ux)
    float* v2 = gzB + T.AZ;    // mu  * Dx(uz)/dx        [x][z]  (dxz(mu uz))
    float* v3 = v2 + T.AZ;     // lam * Dx(ux)/dx                 (dxz(lam ux))
    float* sFS = v3 + T.AZ;    // free-surface terms of row 1       [term][x]

    const float rdx = 1.0f / a.dx, rdz = 1.0f / a.dz;
    const float* uxc = a.ux[a.cur];
    const float* uzc = a.uz[a.cur];

    // ---- phase 0: field tile (with injection) and material tile -------------
    // kFill items per thread per round: every load of a round is issued before the first
    // shared-memory store, so a round costs one memory latency.
    constexpr int kFill = 4;
    Walk wu(tid, T.UZ, kThreads);     // (i % UZ, i / UZ) of this thread's items, in order
    for (int i0 = tid; i0 < T.U; i0 += kFill * kThreads) {
        float vx[kFill], vz[kFill], bx[kFill], bz[kFill];
#pragma unroll
        for (int q = 0; q < kFill; ++q) {
            const int i = i0 + q * kThreads;
            const int sz = wu.r, sx = wu.q;
            wu.next();
            vx[q] = 0.f; vz[q] = 0.f; bx[q] = 0.f; bz[q] = 0.f;
            if (i < T.U) {
                const int iz = R.z0 - H + sz, ix = R.x0 - H + sx;
                if (iz >= 1 && iz <= NZ && ix >= 1 - npml && ix <= nx + npml) {
                    const size_t g = gidx(a, iz, ix);
                    vx[q] = uxc[g];
                    vz[q] = uzc[g];
                    const float* pz = nullptr;
                    const float* px = pml ? inner_bg_ptr(a, iz, ix, pz) : outer_bg_ptr(a, iz, ix, pz);
                    if (px) {
                        bx[q] = __ldg(px);
                        bz[q] = __ldg(pz);
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < kFill; ++q) {
            const int i = i0 + q * kThreads;
            if (i < T.U) {
                sux[i] = pml ? vx[q] - bx[q] : vx[q] + bx[q];
                suz[i] = pml ? vz[q] - bz[q] : vz[q] + bz[q];
            }
        }
    }
    Walk wm(tid, T.MZ, kThreads);
    for (int i0 = tid; i0 < T.M; i0 += kFill * kThreads) {
        float l[kFill], m[kFill];
#pragma unroll
        for (int q = 0; q < kFill; ++q) {
            const int i = i0 + q * kThreads;
            const int mz = wm.r, mx = wm.q;
            wm.next();
            l[q] = 0.f; m[q] = 1.f;
            if (i < T.M) {
                const int iz = R.z0 - NO + mz, ix = R.x0 - NO + mx;
                if (iz >= 1 && iz <= NZ && ix >= 1 - npml && ix <= nx + npml) {
                    const size_t g = gidx(a, iz, ix);
                    l[q] = __ldg(a.lam + g);
                    m[q] = __ldg(a.mu + g);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < kFill; ++q) {
            const int i = i0 + q * kThreads;
            if (i < T.M) {
                const float l2 = l[q] + 2.0f * m[q];
                sLam[i] = l[q];
                sMu[i] = m[q];
                sRL2m[i] = fast_rcp(l2);
                sRMu[i] = fast_rcp(m[q]);
            }
        }
    }
    __syncthreads();

#define SU(arr, z, x) arr[((x) + H) * T.UZ + ((z) + H)]
#define SM(arr, z, x) arr[((x) + NO) * T.MZ + ((z) + NO)]

    // ---- free surface (row 1, stress image about row 1.5): its terms per column, once -------
    // Formed here by one thread per column rather than inside the output loop, where the row-1
    // cells of a warp would hold every other lane idle through the divisions.
    if (R.z0 == 1) {
        const float dx = a.dx, dz = a.dz;
        for (int x = tid; x < TX; x += kThreads) {
            const int nxo = ordx(a, R.x0 + x, NO);
            float dA = 0.f, dB = 0.f, dz1 = 0.f, dz2v = 0.f, dx1 = 0.f, dx2v = 0.f;
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                float c = c_coll[nxo][k];
                float Ap = SM(sLam, 0, x + k) * (SU(suz, 1, x + k) - SU(suz, 0, x + k)) / dz;
                float Am = SM(sLam, 0, x - k) * (SU(suz, 1, x - k) - SU(suz, 0, x - k)) / dz;
                float Bp = SM(sMu, 0, x + k) * (SU(sux, 1, x + k) - SU(sux, 0, x + k)) / dz;
                float Bm = SM(sMu, 0, x - k) * (SU(sux, 1, x - k) - SU(sux, 0, x - k)) / dz;
                dA = fmaf(c, Ap - Am, dA);
                dB = fmaf(c, Bp - Bm, dB);
                dz1 = fmaf(c, SU(suz, 0, x + k) - SU(suz, 0, x - k), dz1);
                dz2v = fmaf(c, SU(suz, 1, x + k) - SU(suz, 1, x - k), dz2v);
                dx1 = fmaf(c, SU(sux, 0, x + k) - SU(sux, 0, x - k), dx1);
                dx2v = fmaf(c, SU(sux, 1, x + k) - SU(sux, 1, x - k), dx2v);
            }
            dA /= dx; dB /= dx; dz1 /= dx; dz2v /= dx; dx1 /= dx; dx2v /= dx;
            const float mu1 = SM(sMu, 0, x), mu2 = SM(sMu, 1, x);
            const float la1 = SM(sLam, 0, x), la2 = SM(sLam, 1, x);
            const float hmu = 2.0f / (SM(sRMu, 0, x) + SM(sRMu, 1, x));
            const float hl2m = 2.0f / (SM(sRL2m, 0, x) + SM(sRL2m, 1, x));
            const float dux = SU(sux, 1, x) - SU(sux, 0, x);
            const float duz = SU(suz, 1, x) - SU(suz, 0, x);
            const float fsA = dA;                                   // Dx[lam(1) dz uz]
            const float fsB = dB;                                   // Dx[mu(1)  dz ux]
            const float fsx = hmu * dux / dz;                       // z part of sxz(1.5)
            const float fsz = hl2m * duz / dz;                      // z part of szz(1.5)
            // x parts of the half-row stresses
            const float dux1 = 0.5f * (mu1 * dz1 + mu2 * dz2v);     // (mu1 Dx uz1 + mu2 Dx uz2)/2
            const float duz1 = 0.5f * (la1 * dx1 + la2 * dx2v);     // (lam1 Dx ux1 + lam2 Dx ux2)/2
            sFS[kFsA * TX + x] = fsA;
            sFS[kFsQx * TX + x] = 2.0f * (fsx + dux1) / dz;
            sFS[kFsB * TX + x] = fsB;
            sFS[kFsQz * TX + x] = 2.0f * (fsz + duz1) / dz;
            sFS[kFsF2x * TX + x] = fsA + 2.0f * dux1 / dz;
            sFS[kFsF3x * TX + x] = 2.0f * fsx / dz;
            sFS[kFsF2z * TX + x] = fsB + 2.0f * duz1 / dz;
            sFS[kFsF3z * TX + x] = 2.0f * fsz / dz;
        }
    }

    // ---- phase 1a: x-direction staggered products and dzx operands -----------
    Walk w1(tid, TZ, kThreads);
    for (int i = tid; i < T.AX; i += kThreads, w1.next()) {
        const int z = w1.r, xl = w1.q;
        int iz = R.z0 + z;
        // staggered product at label L = xl - NO (half point between L and L+1)
        if (xl < T.XW - 1) {
            int L = xl - NO;
            int n = ordx(a, R.x0 + L, NO);
            float sx = 0.f, szv = 0.f;
#pragma unroll
            for (int j = 1; j <= NO; ++j) {
                float c = c_stag[n][j];
                sx = fmaf(c, SU(sux, z, L + j) - SU(sux, z, L + 1 - j), sx);
                szv = fmaf(c, SU(suz, z, L + j) - SU(suz, z, L + 1 - j), szv);
            }
            float hl = 2.0f * fast_rcp(SM(sRL2m, z, L) + SM(sRL2m, z, L + 1));
            float hm = 2.0f * fast_rcp(SM(sRMu, z, L) + SM(sRMu, z, L + 1));
            gxA[i] = hl * sx;
            gxB[i] = hm * szv;
        }
        // dzx operands at cell column x = xl - NO
        {
            int x = xl - NO;
            int ix = R.x0 + x;
            int n = ordz(a, iz, NO);
            float dzz = 0.f, dzx = 0.f;
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                float c = c_coll[n][k];
                dzz = fmaf(c, SU(suz, z + k, x) - SU(suz, z - k, x), dzz);
                dzx = fmaf(c, SU(sux, z + k, x) - SU(sux, z - k, x), dzx);
            }
            // diffzx_reg forms v on rows 2..nz; diffzx_pml on rows 2..NZ-1, columns 2-npml..nx+npml-1
            bool valid = pml ? (iz >= 2 && iz <= NZ - 1 && ix >= 2 - npml && ix <= nx + npml - 1)
                             : (iz >= 2 && iz <= nz && ix >= 1 - NO && ix <= nx + NO);
            v1[i] = valid ? SM(sLam, z, x) * dzz * rdz : 0.f;
            v4[i] = valid ? SM(sMu, z, x) * dzx * rdz : 0.f;
        }
    }
    // ---- phase 1b: z-direction staggered products and dxz operands -----------
    Walk w2(tid, T.ZW, kThreads);
    for (int i = tid; i < T.AZ; i += kThreads, w2.next()) {
        const int zl = w2.r, x = w2.q;
        int ix = R.x0 + x;
        if (zl < T.ZW - 1) {
            int L = zl - NO;
            int n = ordz(a, R.z0 + L, NO);
            float sz_ = 0.f, sx = 0.f;
#pragma unroll
            for (int j = 1; j <= NO; ++j) {
                float c = c_stag[n][j];
                sz_ = fmaf(c, SU(suz, L + j, x) - SU(suz, L + 1 - j, x), sz_);
                sx = fmaf(c, SU(sux, L + j, x) - SU(sux, L + 1 - j, x), sx);
            }
            float hl = 2.0f * fast_rcp(SM(sRL2m, L, x) + SM(sRL2m, L + 1, x));
            float hm = 2.0f * fast_rcp(SM(sRMu, L, x) + SM(sRMu, L + 1, x));
            gzA[i] = hl * sz_;
            gzB[i] = hm * sx;
        }
        {
            int z = zl - NO;
            int iz = R.z0 + z;
            int n = ordx(a, ix, NO);
            float dxz = 0.f, dxx = 0.f;
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                float c = c_coll[n][k];
                dxz = fmaf(c, SU(suz, z, x + k) - SU(suz, z, x - k), dxz);
                dxx = fmaf(c, SU(sux, z, x + k) - SU(sux, z, x - k), dxx);
            }
            // diffxz_reg forms v on rows 1..nz+norder, columns 1..nx; diffxz_pml on rows 1..NZ-1
            bool valid = pml ? (iz >= 1 && iz <= NZ - 1 && ix >= 2 - npml && ix <= nx + npml - 1)
                             : (iz >= 1 && iz <= nz + NO && ix >= 1 && ix <= nx);
            v2[i] = valid ? SM(sMu, z, x) * dxz * rdx : 0.f;
            v3[i] = valid ? SM(sLam, z, x) * dxx * rdx : 0.f;
        }
    }
    __syncthreads();

#define GXI(arr, z, L) arr[((L) + NO) * TZ + (z)]
#define VXI(arr, z, x) arr[((x) + NO) * TZ + (z)]
#define GZI(arr, L, x) arr[(x) * T.ZW + ((L) + NO)]
#define VZI(arr, z, x) arr[(x) * T.ZW + ((z) + NO)]

    // ---- phase 2: output cells ----------------------------------------------
    const float dx2 = pml ? a.dx2p : a.dx2r;
    Walk wc(tid, TZ, kThreads);
    for (int cell = tid; cell < TZ * TX; cell += kThreads, wc.next()) {
        const int z = wc.r, x = wc.q;
        const int iz = R.z0 + z;
        const int ix = R.x0 + x;
        if (iz < R.zlo || iz > R.zhi || ix < R.xlo || ix > R.xhi) continue;
        const size_t g = gidx(a, iz, ix);
        const int nxo = ordx(a, ix, NO);
        const int nzo = ordz(a, iz, NO);
        // every column ix-NO..ix (row iz-NO..iz) has the full order: no reduced-order half points
        const bool fullx = ix - NO >= NO - npml + 1 && ix <= nx + npml - NO;
        const bool fullz = iz - NO >= NO + 1 && iz <= NZ - NO;

        if (pml && (ix == 1 - npml || ix == nx + npml || iz == NZ)) {
            // outer frame: never advanced; keep level 1 across the plane swap
            a.ux[a.cur ^ 1][g] = uxc[g];
            a.uz[a.cur ^ 1][g] = uzc[g];
            continue;
        }

        const float kd = __ldg(a.kdt2 + g);

        // x-direction second derivatives dxx(l2m ux), dxx(mu uz)
        float x2a = 0.f, x2b = 0.f;
#pragma unroll
        for (int k = 1; k <= NO; ++k) {
            float c = c_stag[nxo][k];
            float pa = GXI(gxA, z, x + k - 1), pb = GXI(gxB, z, x + k - 1);
            float ma, mb;
            int Lm = x - k;
            int nr = fullx ? NO : ordx(a, ix - k + 1, NO);
            if (fullx || nr == ordx(a, ix - k, NO)) {
                ma = GXI(gxA, z, Lm); mb = GXI(gxB, z, Lm);
            } else {
                float s1 = 0.f, s2 = 0.f;
                for (int j = 1; j <= NO; ++j) {
                    float cj = c_stag[nr][j];
                    s1 = fmaf(cj, SU(sux, z, Lm + j) - SU(sux, z, Lm + 1 - j), s1);
                    s2 = fmaf(cj, SU(suz, z, Lm + j) - SU(suz, z, Lm + 1 - j), s2);
                }
                ma = 2.0f / (SM(sRL2m, z, Lm) + SM(sRL2m, z, Lm + 1)) * s1;
                mb = 2.0f / (SM(sRMu, z, Lm) + SM(sRMu, z, Lm + 1)) * s2;
            }
            x2a = fmaf(c, pa - ma, x2a);
            x2b = fmaf(c, pb - mb, x2b);
        }
        const float Fx2_l2m_ux = x2a * dx2;
        const float Fx2_mu_uz = x2b * dx2;

        // z-direction second derivatives dzz(l2m uz), dzz(mu ux)
        float z2a = 0.f, z2b = 0.f;
#pragma unroll
        for (int k = 1; k <= NO; ++k) {
            float c = c_stag[nzo][k];
            float pa = GZI(gzA, z + k - 1, x), pb = GZI(gzB, z + k - 1, x);
            float ma, mb;
            int Lm = z - k;
            int nr = fullz ? NO : ordz(a, iz - k + 1, NO);
            if (fullz || nr == ordz(a, iz - k, NO)) {
                ma = GZI(gzA, Lm, x); mb = GZI(gzB, Lm, x);
            } else {
                float s1 = 0.f, s2 = 0.f;
                for (int j = 1; j <= NO; ++j) {
                    float cj = c_stag[nr][j];
                    s1 = fmaf(cj, SU(suz, Lm + j, x) - SU(suz, Lm + 1 - j, x), s1);
                    s2 = fmaf(cj, SU(sux, Lm + j, x) - SU(sux, Lm + 1 - j, x), s2);
                }
                ma = 2.0f / (SM(sRL2m, Lm, x) + SM(sRL2m, Lm + 1, x)) * s1;
                mb = 2.0f / (SM(sRMu, Lm, x) + SM(sRMu, Lm + 1, x)) * s2;
            }
            z2a = fmaf(c, pa - ma, z2a);
            z2b = fmaf(c, pb - mb, z2b);
        }
        const float Fz2_l2m_uz = z2a * a.dz2;
        const float Fz2_mu_ux = z2b * a.dz2;

        // mixed derivatives
        float zxl = 0.f, zxm = 0.f, xzm = 0.f, xzl = 0.f;
#pragma unroll
        for (int k = 1; k <= NO; ++k) {
            float cx = c_coll[nxo][k], cz = c_coll[nzo][k];
            zxl = fmaf(cx, VXI(v1, z, x + k) - VXI(v1, z, x - k), zxl);
            zxm = fmaf(cx, VXI(v4, z, x + k) - VXI(v4, z, x - k), zxm);
            xzm = fmaf(cz, VZI(v2, z + k, x) - VZI(v2, z - k, x), xzm);
            xzl = fmaf(cz, VZI(v3, z + k, x) - VZI(v3, z - k, x), xzl);
        }
        const float Fzx_lam_uz = zxl * rdx, Fzx_mu_ux = zxm * rdx;
        const float Fxz_mu_uz = xzm * rdz, Fxz_lam_ux = xzl * rdz;

        float* uxn = a.ux[a.cur ^ 1];
        float* uzn = a.uz[a.cur ^ 1];
        const float ux0 = uxc[g], uz0 = uzc[g];

        if (!pml) {
            float Fx, Fz;
            if (iz == 1) {
                Fx = Fx2_l2m_ux + sFS[kFsA * TX + x] + sFS[kFsQx * TX + x];
                Fz = Fx2_mu_uz + sFS[kFsB * TX + x] + sFS[kFsQz * TX + x];
            } else {
                Fx = Fx2_l2m_ux + Fzx_lam_uz + Fz2_mu_ux + Fxz_mu_uz;
                Fz = Fz2_l2m_uz + Fxz_lam_ux + Fx2_mu_uz + Fzx_mu_ux;
            }
            uxn[g] = fmaf(kd, Fx, 2.0f * ux0 - uxn[g]);
            uzn[g] = fmaf(kd, Fz, 2.0f * uz0 - uzn[g]);
            continue;
        }

        // ---- PML cell: split-field update ----------------------------------
        // Absorbing-layer state of the cell, gathered in one round of loads (in flight while the
        // first derivatives below are formed) before any of it is written back.
        const int side = R.side;
        size_t ap = 0;
        float gPx[2], gPz[2], gU1[2], gU1m[2], gU2[2], gU2m[2], gU3[2], gU3m[2];
        DampCol dxc{0.f, 0.f, 1.f, 1.f}, dzc{0.f, 0.f, 1.f, 1.f};
        {
            if (side == 1) ap = (size_t)(iz - 1) + (size_t)nz * (size_t)(ix - (1 - npml));
            else if (side == 2) ap = (size_t)(iz - 1) + (size_t)nz * (size_t)(ix - nx - 1);
            else ap = (size_t)(iz - nz - 1) + (size_t)npml * (size_t)(ix - (1 - npml));
            const int base = side == 1 ? 0 : side == 2 ? 6 : 12;
            const int bpx0 = side == 1 ? 0 : side == 2 ? 2 : 8;
#pragma unroll
            for (int comp = 0; comp < 2; ++comp) {
                gPx[comp] = a.bp[side == 3 ? bpx0 + 2 * comp : bpx0 + comp][ap];
                gPz[comp] = side == 3 ? a.bp[9 + 2 * comp][ap] : 0.f;
                gU1[comp] = a.bu[base + 3 * comp + 0][a.cur][ap];
                gU1m[comp] = a.bu[base + 3 * comp + 0][a.cur ^ 1][ap];
                gU2[comp] = a.bu[base + 3 * comp + 1][a.cur][ap];
                gU2m[comp] = a.bu[base + 3 * comp + 1][a.cur ^ 1][ap];
                gU3[comp] = a.bu[base + 3 * comp + 2][a.cur][ap];
                gU3m[comp] = a.bu[base + 3 * comp + 2][a.cur ^ 1][ap];
            }
            dxc = a.dampx[ix + npml - 1];
            if (side == 3) dzc = a.dampz[iz - 1];
        }
        const float yx = dxc.y, yz = dzc.y;
        const float r2 = side == 3 ? fast_rcp(1.0f + 0.5f * (yx + yz)) : dxc.rh;   // 1 / (1 + (yx + yz)/2)

        // first derivatives for the memory variables (diff1 / diffx1 on the PML field)
        float dxux = 0.f, dxuz = 0.f, dzux = 0.f, dzuz = 0.f;
#pragma unroll
        for (int k = 1; k <= NO; ++k) {
            float cx = c_coll[nxo][k], cz = c_coll[nzo][k];
            dxux = fmaf(cx, SU(sux, z, x + k) - SU(sux, z, x - k), dxux);
            dxuz = fmaf(cx, SU(suz, z, x + k) - SU(suz, z, x - k), dxuz);
            dzux = fmaf(cz, SU(sux, z + k, x) - SU(sux, z - k, x), dzux);
            dzuz = fmaf(cz, SU(suz, z + k, x) - SU(suz, z - k, x), dzuz);
        }
        dxux *= rdx; dxuz *= rdx; dzux *= rdz; dzuz *= rdz;
        const float lam0 = SM(sLam, z, x), mu0 = SM(sMu, z, x), l2m0 = lam0 + 2.0f * mu0;

        const int base = side == 1 ? 0 : side == 2 ? 6 : 12;
        const int bpx0 = side == 1 ? 0 : side == 2 ? 2 : 8;
        const int nplane = a.cur ^ 1;
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
            float F1, F2, F3, S1, S3 = 0.f;
            if (iz == 1) {
                if (comp == 0) {
                    F1 = Fx2_l2m_ux;
                    F2 = sFS[kFsF2x * TX + x];
                    F3 = sFS[kFsF3x * TX + x];
                    S1 = l2m0 * dxux;
                } else {
                    F1 = Fx2_mu_uz;
                    F2 = sFS[kFsF2z * TX + x];
                    F3 = sFS[kFsF3z * TX + x];
                    S1 = mu0 * dxuz;
                }
            } else if (comp == 0) {
                F1 = Fx2_l2m_ux;
                F2 = Fzx_lam_uz + Fxz_mu_uz;
                F3 = Fz2_mu_ux;
                S1 = l2m0 * dxux;
                S3 = mu0 * dzux;
            } else {
                F1 = Fx2_mu_uz;
                F2 = Fxz_lam_ux + Fzx_mu_ux;
                F3 = Fz2_l2m_uz;
                S1 = mu0 * dxuz;
                S3 = l2m0 * dzuz;
            }
            (void)lam0;
            float* bpx = a.bp[side == 3 ? bpx0 + 2 * comp : bpx0 + comp];
            const float Px = gPx[comp];
            const float Pxn = ((1.0f - 0.5f * yx) * Px - dxc.dtdp * S1) * dxc.rh;
            bpx[ap] = Pxn;
            float* b1n = a.bu[base + 3 * comp + 0][nplane];
            float* b2n = a.bu[base + 3 * comp + 1][nplane];
            float* b3n = a.bu[base + 3 * comp + 2][nplane];
            const float u1 = gU1[comp], u1m = gU1m[comp];
            const float f1 = kd * (F1 + 0.5f * (Pxn + Px));
            float n1;
            if (side == 2 && iz != 1)
                n1 = ((2.0f - yx * yx) * u1 - (1.0f - yx) * u1m) * dxc.r1 + f1;
            else
                n1 = ((2.0f - yx * yx) * u1 - (1.0f - yx) * u1m + f1) * dxc.r1;
            const float u2 = gU2[comp], u2m = gU2m[comp];
            const float n2 = ((2.0f - yx * yz) * u2 - (1.0f - 0.5f * (yx + yz)) * u2m + kd * F2) * r2;
            const float u3 = gU3[comp], u3m = gU3m[comp];
            float n3;
            if (side == 3) {
                float* bpz = a.bp[9 + 2 * comp];
                const float Pz = gPz[comp];
                const float Pzn = ((1.0f - 0.5f * yz) * Pz - dzc.dtdp * S3) * dzc.rh;
                bpz[ap] = Pzn;
                n3 = ((2.0f - yz * yz) * u3 - (1.0f - yz) * u3m + kd * (F3 + 0.5f * (Pzn + Pz))) * dzc.r1;
            } else {
                n3 = fmaf(kd, F3, 2.0f * u3 - u3m);
            }
            b1n[ap] = n1;
            b2n[ap] = n2;
            b3n[ap] = n3;
            if (comp == 0) uxn[g] = n1 + n2 + n3;
            else uzn[g] = n1 + n2 + n3;
        }
    }
#undef SU
#undef SM
#undef GXI
#undef VXI
#undef GZI
#undef VZI
}

template <int NO>
__global__ void __launch_bounds__(kThreads, 3) fdfk_step_kernel(StepArgs a)
{
    step_block<NO>(a, blockIdx.x);
}

// A batch member's StepArgs copied by the whole block into shared memory (one barrier): the
// batched kernels then read their arguments from there instead of global memory throughout
// (the single-solve kernels have them as kernel parameters).
__device__ __forceinline__ void stage_args(StepArgs& dst, const StepArgs* src)
{
    static_assert(sizeof(StepArgs) % sizeof(int) == 0, "StepArgs is copied as words");
    const int* from = reinterpret_cast<const int*>(src);
    int* to = reinterpret_cast<int*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(StepArgs) / sizeof(int)); i += blockDim.x) to[i] = __ldg(from + i);
    __syncthreads();
}

// Largest s with off[s] <= blk (off[0] = 0, off[n] = total blocks).
__device__ __forceinline__ int batch_member(const int* __restrict__ off, int n, int blk)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= blk) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The tiled kernel over every member of a batch: member s owns blocks edge_off[s] .. edge_off[s+1]-1.
template <int NO>
__global__ void __launch_bounds__(kThreads, 3) fdfk_step_batch_kernel(BatchTab t)
{
    __shared__ StepArgs sa;
    const int s = batch_member(t.edge_off, t.n, blockIdx.x);
    if (!t.live[s]) return;                // the whole block returns: no barrier is split
    stage_args(sa, t.args + s);
    step_block<NO>(sa, blockIdx.x - t.edge_off[s]);
}

// Per-step bookkeeping of a batch on the device: time index, plane parity and receiver sampling of
// every member, written into its StepArgs before the step's kernels run.
__global__ void fdfk_batch_bump(BatchTab t)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= t.n) return;
    BatchDyn& d = t.dyn[s];
    StepArgs& a = t.args[s];
    if (!d.live || d.it > d.nt) {
        d.live = 0;
        t.live[s] = 0;
        return;
    }
    a.it = d.it;
    a.cur = d.cur;
    a.nrcv = 0;
    if (d.nrcv > 0 && d.isis == d.it && d.istp <= d.nsis) {
        a.nrcv = d.nrcv;
        a.sample_index = d.istp;
        d.istp += 1;
        d.isis += d.nstp;
    }
    t.live[s] = 1;
    d.it += 1;
    d.cur ^= 1;
}

// ---------------------------------------------------------------------------
// Host-side launch helpers
// ---------------------------------------------------------------------------
template <int NO>
static cudaError_t launch_no(const StepArgs& a, int n_sample_blocks, cudaStream_t s)
{
    static int configured = 0;   // dynamic shared memory opted in so far (bytes)
    size_t smem = 0;
    for (int c = 0; c < 3; ++c)
        smem = std::max(smem, sizeof(float) * (size_t)tile_dims(NO, a.tdz[c], a.tdx[c]).total);
    if ((int)smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(fdfk_step_kernel<NO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = (int)smem;
    }
    if (a.n_tiles + n_sample_blocks == 0) return cudaSuccess;
    fdfk_step_kernel<NO><<<a.n_tiles + n_sample_blocks, kThreads, smem, s>>>(a);
    return cudaGetLastError();
}

// Receiver-sampling blocks appended to a tiled launch (one warp per receiver).
int sample_blocks(int nrcv) { return nrcv > 0 ? (nrcv + kThreads / 32 - 1) / (kThreads / 32) : 0; }

cudaError_t launch_step(const StepArgs& a, cudaStream_t s)
{
    int nsb = sample_blocks(a.nrcv);
    switch (a.norder) {
    case 1: return launch_no<1>(a, nsb, s);
    case 2: return launch_no<2>(a, nsb, s);
    case 3: return launch_no<3>(a, nsb, s);
    case 4: return launch_no<4>(a, nsb, s);
    case 5: return launch_no<5>(a, nsb, s);
    case 6: return launch_no<6>(a, nsb, s);
    case 7: return launch_no<7>(a, nsb, s);
    case 8: return launch_no<8>(a, nsb, s);
    default: return cudaErrorInvalidValue;
    }
}

template <int NO>
static cudaError_t launch_batch_no(const BatchTab& t, int blocks, size_t smem, cudaStream_t s)
{
    static int configured = 0;
    if ((int)smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(fdfk_step_batch_kernel<NO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        configured = (int)smem;
    }
    if (blocks == 0) return cudaSuccess;
    fdfk_step_batch_kernel<NO><<<blocks, kThreads, smem, s>>>(t);
    return cudaGetLastError();
}

cudaError_t launch_step_batch(const BatchTab& t, int norder, int blocks, size_t smem, cudaStream_t s)
{
    switch (norder) {
    case 1: return launch_batch_no<1>(t, blocks, smem, s);
    case 2: return launch_batch_no<2>(t, blocks, smem, s);
    case 3: return launch_batch_no<3>(t, blocks, smem, s);
    case 4: return launch_batch_no<4>(t, blocks, smem, s);
    case 5: return launch_batch_no<5>(t, blocks, smem, s);
    case 6: return launch_batch_no<6>(t, blocks, smem, s);
    case 7: return launch_batch_no<7>(t, blocks, smem, s);
    case 8: return launch_batch_no<8>(t, blocks, smem, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_batch_bump(const BatchTab& t, cudaStream_t s)
{
    fdfk_batch_bump<<<(t.n + 127) / 128, 128, 0, s>>>(t);
    return cudaGetLastError();
}

size_t step_smem_for(const StepArgs& a)
{
    size_t smem = 0;
    for (int c = 0; c < 3; ++c)
        smem = std::max(smem, sizeof(float) * (size_t)tile_dims(a.norder, a.tdz[c], a.tdx[c]).total);
    return smem;
}

// Tile shapes and counts of the tiled kernel.  band_top: the fast path covers rows below
// int_rows, so the interior tiles are flat kBandTZ x kBandTX tiles of the top band.  The
// absorbing layers are cut into tiles whose thickness divides npml evenly (at most kPmlTile)
// and pml_run cells (kPmlRun when not tuned) along the layer.
void plan_tiles(StepArgs& a, bool band_top, int pml_run)
{
    if (pml_run < 8) pml_run = kPmlRun;
    auto cdiv = [](int x, int y) { return (x + y - 1) / y; };
    const int nt = cdiv(a.npml, kPmlTile);
    const int th = cdiv(a.npml, nt);
    a.tdz[0] = band_top ? kBandTZ : kTZ;
    a.tdx[0] = band_top ? kBandTX : kTX;
    a.tdz[1] = pml_run; a.tdx[1] = th;
    a.tdz[2] = th; a.tdx[2] = pml_run;
    a.tiles_int_z = cdiv(a.int_rows, a.tdz[0]);
    a.tiles_int_x = cdiv(a.nx, a.tdx[0]);
    a.tiles_l_z = cdiv(a.nz, a.tdz[1]);
    a.tiles_l_x = cdiv(a.npml, a.tdx[1]);
    a.tiles_b_z = cdiv(a.npml, a.tdz[2]);
    a.tiles_b_x = cdiv(a.NX, a.tdx[2]);
    a.n_tiles = a.tiles_int_z * a.tiles_int_x + 2 * a.tiles_l_z * a.tiles_l_x + a.tiles_b_z * a.tiles_b_x;
}

cudaError_t set_coefficients(const float* stag, const float* coll)
{
    cudaError_t e = cudaMemcpyToSymbol(c_stag, stag, sizeof(float) * (kMaxOrder + 1) * (kMaxOrder + 1));
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_coll, coll, sizeof(float) * (kMaxOrder + 1) * (kMaxOrder + 1));
}

}  // namespace fdfk

// The interior fast path shares the coefficient tables above.
#include "fdfk_march.cuh"
