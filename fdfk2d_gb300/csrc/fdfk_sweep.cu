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

// Shared-memory layout of a TZ x TX tile (z fastest) for stencil half-order NO.  The cells of a
// tile are handled in pairs of rows (z, z+1), z even, so every array has an even column stride
// and an even row origin: the two rows of a pair are one aligned 8-byte access.
struct TileDims {
    int TZ, TX;
    int TZe;        // TZ rounded up to even (rows TZ..TZe-1 are computed, never stored)
    int UZ, UX;     // u tile: rows -OU .. TZe+OU-1 (OU = 2 NO), columns -H .. TX+H-1 (H = 2 NO - 1)
    int MZ, MX;     // material tile: rows -OM .. TZe+OM-1 (OM = NO rounded up to even), columns -NO .. TX+NO-1
    int ZW;         // rows of the z-consumed arrays: -OM .. TZe+OM-1 (columns 0..TX-1)
    int XW;         // columns of the x-consumed arrays: -NO .. TX+NO-1 (rows 0..TZe-1)
    int U, M, AX, AZ;
    int FS;         // free-surface terms of row 1 (kFsTerms per column)
    int total;      // floats
};

__host__ __device__ __forceinline__ TileDims tile_dims(int NO, int TZ, int TX)
{
    TileDims t;
    const int H = 2 * NO - 1, OU = 2 * NO, OM = NO + (NO & 1);
    t.TZ = TZ; t.TX = TX;
    t.TZe = (TZ + 1) & ~1;
    t.UZ = t.TZe + 2 * OU; t.UX = TX + 2 * H;
    t.MZ = t.TZe + 2 * OM; t.MX = TX + 2 * NO;
    t.ZW = t.TZe + 2 * OM; t.XW = TX + 2 * NO;
    t.U = t.UZ * t.UX; t.M = t.MZ * t.MX;
    t.AX = t.TZe * t.XW; t.AZ = t.ZW * TX;
    t.FS = kFsTerms * TX;
    t.total = 2 * t.U + 4 * t.M + 6 * t.AX + 6 * t.AZ + ((t.FS + 1) & ~1);
    return t;
}

struct Rect {
    int side;       // 0 interior, 1 left PML, 2 right PML, 3 bottom PML, 4 top PML
    int cls;        // tile class (StepArgs::tdz / tdx): 0 interior, 1 side PML, 2 bottom and top PML
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

// (x / n, x % n) for 0 <= x < 2^20 and 1 <= n < 2^20: a single-precision reciprocal estimate is
// within one of the quotient, and one correction makes it exact (cheaper than the integer
// division sequence for a divisor known only at run time).
__device__ __forceinline__ void divmod_small(int x, int n, int& q, int& r)
{
    q = __float2int_rz(__fmul_rn(__int2float_rn(x), fast_rcp(__int2float_rn(n))));
    r = x - q * n;
    if (r < 0) {
        --q;
        r += n;
    } else if (r >= n) {
        ++q;
        r -= n;
    }
}

// (i % n, i / n) along i = i0, i0 + step, ... without a division per step: from (i0 / n, i0 % n)
// and (step / n, step % n).
struct Walk {
    int r, q, dr, dq, n;
    __device__ __forceinline__ Walk(int q0, int r0, int dq_, int dr_, int n_) : r(r0), q(q0), dr(dr_), dq(dq_), n(n_) {}
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
    int n = min(min(iz - a.izt, a.nz + a.npml - iz), NO);
    return n < 0 ? 0 : n;
}
__device__ __forceinline__ size_t gidx(const StepArgs& a, int iz, int ix)
{
    return (size_t)(iz - a.zorg) + (size_t)(ix + a.npml - 1) * (size_t)a.ldz;
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

__device__ __forceinline__ Rect decode_tile(const StepArgs& a, int b)
{
    Rect r;
    if (a.top_pass) {   // the top layer: rows izt+1..0 (row izt is outer frame), every column
        r.side = 4;
        r.cls = 2;
        r.zlo = a.izt + 1; r.zhi = 0; r.xlo = 1 - a.npml; r.xhi = a.nx + a.npml;
        int q, m;
        divmod_small(b, a.tiles_t_z, q, m);
        r.z0 = r.zlo + m * a.tdz[2]; r.x0 = r.xlo + q * a.tdx[2];
        return r;
    }
    int ni = a.tiles_int_z * a.tiles_int_x;
    int nl = a.tiles_l_z * a.tiles_l_x;
    if (b < ni) {
        r.side = 0;
        r.cls = 0;
        int q, m;
        divmod_small(b, a.tiles_int_z, q, m);
        r.z0 = 1 + m * a.tdz[0]; r.x0 = 1 + q * a.tdx[0];
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
        int q, m;
        divmod_small(b, a.tiles_l_z, q, m);
        r.z0 = 1 + m * a.tdz[1]; r.x0 = r.xlo + q * a.tdx[1];
        return r;
    }
    b -= 2 * nl;
    r.side = 3;
    r.cls = 2;
    r.zlo = a.nz + 1; r.zhi = a.nz + a.npml; r.xlo = 1 - a.npml; r.xhi = a.nx + a.npml;
    int q, m;
    divmod_small(b, a.tiles_b_z, q, m);
    r.z0 = r.zlo + m * a.tdz[2]; r.x0 = r.xlo + q * a.tdx[2];
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
__global__ void receiver_sites_kernel(int nrcv, int nx, int nz, int npml, int izt, float dx, float dz, float x0,
                                      float z0, const float* __restrict__ rxs, const float* __restrict__ rzs,
                                      int4* __restrict__ site, double* __restrict__ wout)
{
    const int r = blockIdx.x, q = threadIdx.x;
    if (r >= nrcv) return;
    const float rx = rxs[r], rz = rzs[r];
    const int irx = (int)floorf((rx - x0) / dx) + 1;
    const int irz = (int)floorf((rz - z0) / dz) + 1;
    const int xlo = max(1 - npml, irx - 3), xhi = min(nx + npml, irx + 3);
    const int zlo = max(izt, irz - 3), zhi = min(nz + npml, irz + 3);
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
    receiver_sites_kernel<<<nrcv, 64, 0, s>>>(nrcv, a.nx, a.nz, a.npml, a.izt, a.dx, a.dz, x0, z0, rx, rz, site, w);
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
        // explicit fused multiply-adds: the single-solve and batched copies of this code round alike
        const double wq = w[q];
        sx = fma(wq, (double)ux[g], sx);
        sz = fma(wq, (double)uz[g], sz);
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
// Every phase works on pairs of rows (z, z+1) of one column, z even within the tile.  The two
// rows go through the same operations, so each stencil tap and product is one packed FP32x2
// instruction, rounded per row exactly as the scalar fmaf / __fadd_rn / __fmul_rn, and each
// shared-memory operand of the pair one aligned 8-byte access.  All arithmetic is written with
// explicit rounding: a cell's result is the same whichever row of a pair it is, whatever the
// tile shape, and in the single-solve and batched kernels alike.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2s(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void sts2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }

// N consecutive rows of a z-fastest shared array from p (8-byte aligned): N/2 pair loads and, for
// odd N, one scalar load.
template <int N>
__device__ __forceinline__ void load_rows(const float* p, float (&w)[N])
{
#pragma unroll
    for (int i = 0; i + 1 < N; i += 2) {
        const float2 t = lds2(p + i);
        w[i] = t.x;
        w[i + 1] = t.y;
    }
    if constexpr ((N & 1) != 0) w[N - 1] = p[N - 1];
}

// Block `blk` of one solve's tiled launch: a tile of the top band, an absorbing layer, or (past
// n_tiles) a block of receivers.
template <int NO>
__device__ __forceinline__ void step_block(const StepArgs& a, int blk)
{
    constexpr int H = 2 * NO - 1;
    constexpr int OU = 2 * NO;              // row origin of the u tile (even)
    constexpr int OM = NO + (NO & 1);       // row origin of the material tile and the z-consumed arrays
    constexpr int NWIN = OM + NO + 2;       // rows z-OM .. z+1+NO: the z-stencil window of a pair
    extern __shared__ __align__(16) float sm[];
    if (blk >= a.n_tiles) {
        sample_receivers(a, blk - a.n_tiles);
        return;
    }
    const Rect R = decode_tile(a, blk);
    const TileDims T = tile_dims(NO, a.tdz[R.cls], a.tdx[R.cls]);
    const int TZ = T.TZ, TX = T.TX, TZe = T.TZe;
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
    // The staggered products at a half point L enter the second derivatives of the cells on both
    // sides of it: with the stencil order of column (row) L for the cells at or before L (gxA,
    // gxB, gzA, gzB) and with the order of column (row) L+1 for the cells after it (the "m"
    // arrays).  The two differ only next to the outer frame and the top rows, where the order drops.
    float* gxA = sRMu + T.M;   // H(l2m) * Dstag_x(ux)   [label][z]
    float* gxB = gxA + T.AX;   // H(mu)  * Dstag_x(uz)
    float* gxAm = gxB + T.AX;  // the same with the order of column L+1
    float* gxBm = gxAm + T.AX;
    float* v1 = gxBm + T.AX;   // lam * Dz(uz)/dz        [x][z]  (dzx(lam uz))
    float* v4 = v1 + T.AX;     // mu  * Dz(ux)/dz                 (dzx(mu ux))
    float* gzA = v4 + T.AX;    // H(l2m) * Dstag_z(uz)   [x][label]
    float* gzB = gzA + T.AZ;   // H(mu)  * Dstag_z(ux)
    float* gzAm = gzB + T.AZ;  // the same with the order of row L+1
    float* gzBm = gzAm + T.AZ;
    float* v2 = gzBm + T.AZ;   // mu  * Dx(uz)/dx        [x][z]  (dxz(mu uz))
    float* v3 = v2 + T.AZ;     // lam * Dx(ux)/dx                 (dxz(lam ux))
    float* sFS = v3 + T.AZ;    // free-surface terms of row 1       [term][x]

#define SU(arr, z, x) ((arr) + ((x) + H) * T.UZ + ((z) + OU))
#define SM(arr, z, x) ((arr) + ((x) + NO) * T.MZ + ((z) + OM))
#define GX(arr, z, L) ((arr) + ((L) + NO) * TZe + (z))
#define GZ(arr, L, x) ((arr) + (x) * T.ZW + ((L) + OM))

    const float rdx = 1.0f / a.dx, rdz = 1.0f / a.dz;
    // this thread's first item in the pair-row grids of P2 (field tile), M2 (material tile,
    // z-direction products) and PZ (x-direction products, output cells) pair rows; the block's
    // stride through them comes with the tile class
    const int P2 = T.UZ / 2, M2 = T.MZ / 2, PZ = TZe / 2;
    int qU, rU, qM, rM, qP, rP;
    divmod_small(tid, P2, qU, rU);
    divmod_small(tid, M2, qM, rM);
    divmod_small(tid, PZ, qP, rP);
    const int* const wq = a.wq[R.cls];
    const int* const wr = a.wr[R.cls];
    const float* uxc = a.ux[a.cur];
    const float* uzc = a.uz[a.cur];
    const int izt = a.izt;

    // ---- phase 0: field tile and material tile, by row pairs, and the background strips ------
    // One round of loads covers (for tiles up to kU * 256 field pairs and kM * 256 material
    // pairs) the whole tile: the field, the material and the strip values that meet the field
    // tile are all in flight before the first shared-memory store, so the phase costs one memory
    // latency.  The strips are added (regular field) or removed (absorbing layers' operator
    // field) after a barrier, in place: one rounding per value, as u + b / u - b.  The top layer's
    // launch reads the interior cells that no inner strip covers (rows 1..nz-nbd, columns
    // nbd+1..nx-nbd) at u^{n+1}, from the plane the step has just written: the reference forms the
    // absorbing layers' operator field after its interior update.
    {
        const float* const uxq = a.top_pass ? a.ux[a.cur ^ 1] : uxc;
        const float* const uzq = a.top_pass ? a.uz[a.cur ^ 1] : uzc;
        const int qz1 = nz - a.nbd, qx0 = a.nbd + 1, qx1 = nx - a.nbd;
        constexpr int kU = 3, kM = 2, kB = 2;
        const int NP = P2 * T.UX, NMP = M2 * T.MX;
        // the strip rectangles met by the field tile: element e of their concatenation is row
        // e % nzr_k, column e / nzr_k of rectangle k
        const int zt0 = R.z0 - OU, zt1 = R.z0 - OU + T.UZ - 1;
        const int xt0 = R.x0 - H, xt1 = R.x0 - H + T.UX - 1;
        int bz0[3], bx0[3], bnz[3], bcnt[3], brows[3], borg[3];
        const float* bxs[3];
        const float* bzs[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const StripBox& S = a.sbox[(pml ? 0 : 3) + k];
            const int z0 = max(S.zr0, zt0), z1 = min(S.zr1, zt1);
            const int x0 = max(S.xr0, xt0), x1 = min(S.xr1, xt1);
            const bool any = z0 <= z1 && x0 <= x1;
            bz0[k] = z0; bx0[k] = x0;
            bnz[k] = any ? z1 - z0 + 1 : 1;
            bcnt[k] = any ? (z1 - z0 + 1) * (x1 - x0 + 1) : 0;
            const long long plane = (long long)(S.rows * S.cols) * a.it;
            bxs[k] = a.strip[S.sx] + plane;
            bzs[k] = a.strip[S.sz] + plane;
            brows[k] = S.rows;
            borg[k] = S.org;
        }
        const int nb = bcnt[0] + bcnt[1] + bcnt[2];
        // strip element e: its shared-memory offset in the field tile and its two values
        auto bg_elem = [&](int e, int& off, float& vx, float& vz) {
            int k = 0;
            if (e >= bcnt[0]) { e -= bcnt[0]; k = 1; if (e >= bcnt[1]) { e -= bcnt[1]; k = 2; } }
            int xq, zr;
            divmod_small(e, k == 0 ? bnz[0] : k == 1 ? bnz[1] : bnz[2], xq, zr);
            const int iz = (k == 0 ? bz0[0] : k == 1 ? bz0[1] : bz0[2]) + zr;
            const int ix = (k == 0 ? bx0[0] : k == 1 ? bx0[1] : bx0[2]) + xq;
            const int o = iz + (k == 0 ? brows[0] : k == 1 ? brows[1] : brows[2]) * ix -
                          (k == 0 ? borg[0] : k == 1 ? borg[1] : borg[2]);
            vx = __ldg((k == 0 ? bxs[0] : k == 1 ? bxs[1] : bxs[2]) + o);
            vz = __ldg((k == 0 ? bzs[0] : k == 1 ? bzs[1] : bzs[2]) + o);
            off = (int)(SU(sux, iz - R.z0, ix - R.x0) - sux);
        };
        // the first kB strip elements of every thread, issued ahead of the field and material
        // loads (every thread sets its offsets, so none is left undefined for the pass below)
        float bvx[kB], bvz[kB];
        int boff[kB];
#pragma unroll
        for (int q = 0; q < kB; ++q) {
            boff[q] = -1;
            bvx[q] = 0.f;
            bvz[q] = 0.f;
            const int e = tid + q * kThreads;
            if (e < nb) bg_elem(e, boff[q], bvx[q], bvz[q]);
        }
        Walk wu(qU, rU, wq[0], wr[0], P2);   // (pair row, column) of this thread's field items, in order
        Walk wm(qM, rM, wq[1], wr[1], M2);   // the same for the material items
        for (int u0 = tid, m0 = tid; u0 < NP || m0 < NMP; u0 += kU * kThreads, m0 += kM * kThreads) {
            float2 vx[kU], vz[kU], l[kM], m[kM];
#pragma unroll
            for (int q = 0; q < kU; ++q) {
                const int i = u0 + q * kThreads;
                const int iz = R.z0 - OU + 2 * wu.r, ix = R.x0 - H + wu.q;
                wu.next();
                vx[q] = f2s(0.f);
                vz[q] = f2s(0.f);
                if (i < NP && ix >= 1 - npml && ix <= nx + npml) {
                    const long long g = (long long)(iz - a.zorg) + (long long)(ix + npml - 1) * a.ldz;
                    const bool qc = ix >= qx0 && ix <= qx1;
                    if (iz >= izt && iz <= NZ) {
                        const bool nw = qc && iz >= 1 && iz <= qz1;
                        vx[q].x = (nw ? uxq : uxc)[g];
                        vz[q].x = (nw ? uzq : uzc)[g];
                    }
                    if (iz + 1 >= izt && iz + 1 <= NZ) {
                        const bool nw = qc && iz + 1 >= 1 && iz + 1 <= qz1;
                        vx[q].y = (nw ? uxq : uxc)[g + 1];
                        vz[q].y = (nw ? uzq : uzc)[g + 1];
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kM; ++q) {
                const int i = m0 + q * kThreads;
                const int iz = R.z0 - OM + 2 * wm.r, ix = R.x0 - NO + wm.q;
                wm.next();
                l[q] = f2s(0.f); m[q] = f2s(1.f);
                if (i < NMP && ix >= 1 - npml && ix <= nx + npml) {
                    const long long g = (long long)(iz - a.zorg) + (long long)(ix + npml - 1) * a.ldz;
                    if (iz >= izt && iz <= NZ) { l[q].x = __ldg(a.lam + g); m[q].x = __ldg(a.mu + g); }
                    if (iz + 1 >= izt && iz + 1 <= NZ) { l[q].y = __ldg(a.lam + g + 1); m[q].y = __ldg(a.mu + g + 1); }
                }
            }
#pragma unroll
            for (int q = 0; q < kU; ++q) {
                const int i = u0 + q * kThreads;
                if (i < NP) {
                    sts2(sux + 2 * i, vx[q]);
                    sts2(suz + 2 * i, vz[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < kM; ++q) {
                const int i = m0 + q * kThreads;
                if (i < NMP) {
                    const float2 l2 = pfma(f2s(2.0f), m[q], l[q]);   // lambda + 2 mu (2 mu exact)
                    sts2(sLam + 2 * i, l[q]);
                    sts2(sMu + 2 * i, m[q]);
                    sts2(sRL2m + 2 * i, f2(fast_rcp(l2.x), fast_rcp(l2.y)));
                    sts2(sRMu + 2 * i, f2(fast_rcp(m[q].x), fast_rcp(m[q].y)));
                }
            }
        }
        __syncthreads();
        auto bg_apply = [&](int off, float vxb, float vzb) {
            sux[off] = pml ? __fsub_rn(sux[off], vxb) : __fadd_rn(sux[off], vxb);
            suz[off] = pml ? __fsub_rn(suz[off], vzb) : __fadd_rn(suz[off], vzb);
        };
#pragma unroll
        for (int q = 0; q < kB; ++q)
            if (boff[q] >= 0) bg_apply(boff[q], bvx[q], bvz[q]);
        for (int e = tid + kB * kThreads; e < nb; e += kThreads) {   // tiles with more strip cells
            int off;
            float vxb, vzb;
            bg_elem(e, off, vxb, vzb);
            bg_apply(off, vxb, vzb);
        }
    }
    __syncthreads();

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
                const float c = c_coll[nxo][k];
                const float Ap = __fdiv_rn(__fmul_rn(*SM(sLam, 0, x + k), __fsub_rn(*SU(suz, 1, x + k), *SU(suz, 0, x + k))), dz);
                const float Am = __fdiv_rn(__fmul_rn(*SM(sLam, 0, x - k), __fsub_rn(*SU(suz, 1, x - k), *SU(suz, 0, x - k))), dz);
                const float Bp = __fdiv_rn(__fmul_rn(*SM(sMu, 0, x + k), __fsub_rn(*SU(sux, 1, x + k), *SU(sux, 0, x + k))), dz);
                const float Bm = __fdiv_rn(__fmul_rn(*SM(sMu, 0, x - k), __fsub_rn(*SU(sux, 1, x - k), *SU(sux, 0, x - k))), dz);
                dA = fmaf(c, __fsub_rn(Ap, Am), dA);
                dB = fmaf(c, __fsub_rn(Bp, Bm), dB);
                dz1 = fmaf(c, __fsub_rn(*SU(suz, 0, x + k), *SU(suz, 0, x - k)), dz1);
                dz2v = fmaf(c, __fsub_rn(*SU(suz, 1, x + k), *SU(suz, 1, x - k)), dz2v);
                dx1 = fmaf(c, __fsub_rn(*SU(sux, 0, x + k), *SU(sux, 0, x - k)), dx1);
                dx2v = fmaf(c, __fsub_rn(*SU(sux, 1, x + k), *SU(sux, 1, x - k)), dx2v);
            }
            dA = __fdiv_rn(dA, dx); dB = __fdiv_rn(dB, dx);
            dz1 = __fdiv_rn(dz1, dx); dz2v = __fdiv_rn(dz2v, dx);
            dx1 = __fdiv_rn(dx1, dx); dx2v = __fdiv_rn(dx2v, dx);
            const float mu1 = *SM(sMu, 0, x), mu2 = *SM(sMu, 1, x);
            const float la1 = *SM(sLam, 0, x), la2 = *SM(sLam, 1, x);
            const float hmu = __fdiv_rn(2.0f, __fadd_rn(*SM(sRMu, 0, x), *SM(sRMu, 1, x)));
            const float hl2m = __fdiv_rn(2.0f, __fadd_rn(*SM(sRL2m, 0, x), *SM(sRL2m, 1, x)));
            const float dux = __fsub_rn(*SU(sux, 1, x), *SU(sux, 0, x));
            const float duz = __fsub_rn(*SU(suz, 1, x), *SU(suz, 0, x));
            // Dx[lam(1) dz uz], Dx[mu(1) dz ux]; z parts of sxz(1.5), szz(1.5)
            const float fsx = __fdiv_rn(__fmul_rn(hmu, dux), dz);
            const float fsz = __fdiv_rn(__fmul_rn(hl2m, duz), dz);
            // x parts of the half-row stresses: (mu1 Dx uz1 + mu2 Dx uz2)/2, (lam1 Dx ux1 + lam2 Dx ux2)/2
            const float dux1 = __fmul_rn(0.5f, fmaf(mu1, dz1, __fmul_rn(mu2, dz2v)));
            const float duz1 = __fmul_rn(0.5f, fmaf(la1, dx1, __fmul_rn(la2, dx2v)));
            sFS[kFsA * TX + x] = dA;
            sFS[kFsQx * TX + x] = __fdiv_rn(__fmul_rn(2.0f, __fadd_rn(fsx, dux1)), dz);
            sFS[kFsB * TX + x] = dB;
            sFS[kFsQz * TX + x] = __fdiv_rn(__fmul_rn(2.0f, __fadd_rn(fsz, duz1)), dz);
            sFS[kFsF2x * TX + x] = __fadd_rn(dA, __fdiv_rn(__fmul_rn(2.0f, dux1), dz));
            sFS[kFsF3x * TX + x] = __fdiv_rn(__fmul_rn(2.0f, fsx), dz);
            sFS[kFsF2z * TX + x] = __fadd_rn(dB, __fdiv_rn(__fmul_rn(2.0f, duz1), dz));
            sFS[kFsF3z * TX + x] = __fdiv_rn(__fmul_rn(2.0f, fsz), dz);
        }
    }

    // ---- phase 1: half-point products and mixed operands, by row pairs: the x-direction items
    // (1a) and then the z-direction items (1b) in one loop, so that the block's last, partly
    // filled round of items is shared by the two kinds instead of each having its own
    {
        const int n1a = PZ * T.XW, n1b = M2 * TX;
        Walk w1(qP, rP, wq[2], wr[2], PZ);
        // this thread's first 1b item: its first index at or past n1a in tid, tid + kThreads, ...
        const int kb = tid < n1a ? (n1a - tid + kThreads - 1) / kThreads : 0;
        int qb, rb;
        divmod_small(tid + kb * kThreads - n1a, M2, qb, rb);
        Walk w2(qb, rb, wq[1], wr[1], M2);   // ZW = MZ
        for (int i = tid; i < n1a + n1b; i += kThreads) {
          if (i < n1a) {
            // ---- 1a: x-direction staggered products and dzx operands
            const int z = 2 * w1.r, xl = w1.q;
            w1.next();
            const int iz = R.z0 + z;
            const int o = xl * TZe + z;
            // staggered products at label L = xl - NO (half point between columns L and L+1)
            if (xl < T.XW - 1) {
                const int L = xl - NO;
                const int n = ordx(a, R.x0 + L, NO), nm = ordx(a, R.x0 + L + 1, NO);
                float2 sx = f2s(0.f), szv = f2s(0.f);
#pragma unroll
                for (int j = 1; j <= NO; ++j) {
                    const float2 c = f2s(c_stag[n][j]);
                    sx = pfma(c, psub(lds2(SU(sux, z, L + j)), lds2(SU(sux, z, L + 1 - j))), sx);
                    szv = pfma(c, psub(lds2(SU(suz, z, L + j)), lds2(SU(suz, z, L + 1 - j))), szv);
                }
                const float2 rl = padd(lds2(SM(sRL2m, z, L)), lds2(SM(sRL2m, z, L + 1)));
                const float2 rm = padd(lds2(SM(sRMu, z, L)), lds2(SM(sRMu, z, L + 1)));
                const float2 hl = f2(2.0f * fast_rcp(rl.x), 2.0f * fast_rcp(rl.y));
                const float2 hm = f2(2.0f * fast_rcp(rm.x), 2.0f * fast_rcp(rm.y));
                sts2(gxA + o, pmul(hl, sx));
                sts2(gxB + o, pmul(hm, szv));
                float2 sxm = sx, szm = szv;
                if (nm != n) {
                    sxm = f2s(0.f);
                    szm = f2s(0.f);
#pragma unroll
                    for (int j = 1; j <= NO; ++j) {
                        const float2 c = f2s(c_stag[nm][j]);
                        sxm = pfma(c, psub(lds2(SU(sux, z, L + j)), lds2(SU(sux, z, L + 1 - j))), sxm);
                        szm = pfma(c, psub(lds2(SU(suz, z, L + j)), lds2(SU(suz, z, L + 1 - j))), szm);
                    }
                }
                sts2(gxAm + o, pmul(hl, sxm));
                sts2(gxBm + o, pmul(hm, szm));
            }
            // dzx operands at column x = xl - NO
            {
                const int x = xl - NO;
                const int ix = R.x0 + x;
                const int n0 = ordz(a, iz, NO), n1 = ordz(a, iz + 1, NO);
                float wz[NWIN], wx[NWIN];
                load_rows(SU(suz, z - OM, x), wz);
                load_rows(SU(sux, z - OM, x), wx);
                float2 dzz = f2s(0.f), dzx = f2s(0.f);
#pragma unroll
                for (int k = 1; k <= NO; ++k) {
                    const float2 c = f2(c_coll[n0][k], c_coll[n1][k]);
                    dzz = pfma(c, f2(__fsub_rn(wz[OM + k], wz[OM - k]), __fsub_rn(wz[OM + 1 + k], wz[OM + 1 - k])), dzz);
                    dzx = pfma(c, f2(__fsub_rn(wx[OM + k], wx[OM - k]), __fsub_rn(wx[OM + 1 + k], wx[OM + 1 - k])), dzx);
                }
                // diffzx_reg forms v on rows 2..nz; diffzx_pml on rows izt+1..NZ-1, columns
                // 2-npml..nx+npml-1 (the regular block it leaves out is read by no layer cell)
                const bool colv = pml ? (ix >= 2 - npml && ix <= nx + npml - 1) : (ix >= 1 - NO && ix <= nx + NO);
                const int zmin = pml ? izt + 1 : 2, zmax = pml ? NZ - 1 : nz;
                float2 a1 = pmul(pmul(lds2(SM(sLam, z, x)), dzz), f2s(rdz));
                float2 a4 = pmul(pmul(lds2(SM(sMu, z, x)), dzx), f2s(rdz));
                if (!(colv && iz >= zmin && iz <= zmax)) { a1.x = 0.f; a4.x = 0.f; }
                if (!(colv && iz + 1 >= zmin && iz + 1 <= zmax)) { a1.y = 0.f; a4.y = 0.f; }
                sts2(v1 + o, a1);
                sts2(v4 + o, a4);
            }
          } else {
            // ---- 1b: z-direction staggered products and dxz operands
            const int L = 2 * w2.r - OM, x = w2.q;   // rows / half-point labels L, L+1
            w2.next();
            const int ix = R.x0 + x;
            const int o = x * T.ZW + (L + OM);
            if (L <= TZ + NO - 2) {   // labels read by the output cells: -NO .. TZ+NO-2
                const int n0 = ordz(a, R.z0 + L, NO), n1 = ordz(a, R.z0 + L + 1, NO), n2 = ordz(a, R.z0 + L + 2, NO);
                // rows L+1-NO .. L+1+NO from the even row L - B
                constexpr int B = 2 * (NO / 2);
                float wz[NO + B + 2], wx[NO + B + 2];
                load_rows(SU(suz, L - B, x), wz);
                load_rows(SU(sux, L - B, x), wx);
                float2 szv = f2s(0.f), sx = f2s(0.f);
#pragma unroll
                for (int j = 1; j <= NO; ++j) {
                    const float2 c = f2(c_stag[n0][j], c_stag[n1][j]);
                    // half point L: u(L+j) - u(L+1-j); half point L+1: u(L+1+j) - u(L+2-j)
                    szv = pfma(c, f2(__fsub_rn(wz[B + j], wz[B + 1 - j]), __fsub_rn(wz[B + 1 + j], wz[B + 2 - j])), szv);
                    sx = pfma(c, f2(__fsub_rn(wx[B + j], wx[B + 1 - j]), __fsub_rn(wx[B + 1 + j], wx[B + 2 - j])), sx);
                }
                // the same half points with the orders of rows L+1 and L+2
                float2 szm = szv, sxm = sx;
                if (n0 != n1 || n1 != n2) {
                    szm = f2s(0.f);
                    sxm = f2s(0.f);
#pragma unroll
                    for (int j = 1; j <= NO; ++j) {
                        const float2 c = f2(c_stag[n1][j], c_stag[n2][j]);
                        szm = pfma(c, f2(__fsub_rn(wz[B + j], wz[B + 1 - j]), __fsub_rn(wz[B + 1 + j], wz[B + 2 - j])), szm);
                        sxm = pfma(c, f2(__fsub_rn(wx[B + j], wx[B + 1 - j]), __fsub_rn(wx[B + 1 + j], wx[B + 2 - j])), sxm);
                    }
                }
                // harmonic means over rows (L, L+1) and (L+1, L+2); row L+2 only where half point
                // L+1 is read (the material tile ends at row TZe+OM-1)
                const int L2 = L + 1 <= TZ + NO - 2 ? L + 2 : L + 1;
                const float2 rl = lds2(SM(sRL2m, L, x)), rm = lds2(SM(sRMu, L, x));
                const float rl2 = *SM(sRL2m, L2, x), rm2 = *SM(sRMu, L2, x);
                const float2 hl = f2(2.0f * fast_rcp(__fadd_rn(rl.x, rl.y)), 2.0f * fast_rcp(__fadd_rn(rl.y, rl2)));
                const float2 hm = f2(2.0f * fast_rcp(__fadd_rn(rm.x, rm.y)), 2.0f * fast_rcp(__fadd_rn(rm.y, rm2)));
                sts2(gzA + o, pmul(hl, szv));
                sts2(gzB + o, pmul(hm, sx));
                sts2(gzAm + o, pmul(hl, szm));
                sts2(gzBm + o, pmul(hm, sxm));
            }
            // dxz operands at rows L, L+1
            {
                const int iz = R.z0 + L;
                const int n = ordx(a, ix, NO);
                float2 dxz = f2s(0.f), dxx = f2s(0.f);
#pragma unroll
                for (int k = 1; k <= NO; ++k) {
                    const float2 c = f2s(c_coll[n][k]);
                    dxz = pfma(c, psub(lds2(SU(suz, L, x + k)), lds2(SU(suz, L, x - k))), dxz);
                    dxx = pfma(c, psub(lds2(SU(sux, L, x + k)), lds2(SU(sux, L, x - k))), dxx);
                }
                // diffxz_reg forms v on rows 1..nz+norder, columns 1..nx; diffxz_pml on rows izt..NZ-1
                // except the regular block rows 1..nz-norder x columns 1..nx (which the top layer reads)
                const bool colv = pml ? (ix >= 2 - npml && ix <= nx + npml - 1) : (ix >= 1 && ix <= nx);
                const int zmin = pml ? izt : 1, zmax = pml ? NZ - 1 : nz + NO;
                const bool blk = pml && ix >= 1 && ix <= nx;
                float2 a2 = pmul(pmul(lds2(SM(sMu, L, x)), dxz), f2s(rdx));
                float2 a3 = pmul(pmul(lds2(SM(sLam, L, x)), dxx), f2s(rdx));
                if (!(colv && iz >= zmin && iz <= zmax) || (blk && iz >= 1 && iz <= nz - NO)) { a2.x = 0.f; a3.x = 0.f; }
                if (!(colv && iz + 1 >= zmin && iz + 1 <= zmax) || (blk && iz + 1 >= 1 && iz + 1 <= nz - NO)) {
                    a2.y = 0.f;
                    a3.y = 0.f;
                }
                sts2(v2 + o, a2);
                sts2(v3 + o, a3);
            }
          }
        }
    }
    __syncthreads();

    // ---- phase 2: output cells, by row pairs -------------------------------------------
    const float2 dx2 = f2s(pml ? a.dx2p : a.dx2r), dz2 = f2s(a.dz2);
    const float2 rdx2 = f2s(rdx), rdz2 = f2s(rdz);
    float* const uxn = a.ux[a.cur ^ 1];
    float* const uzn = a.uz[a.cur ^ 1];
    Walk wc(qP, rP, wq[2], wr[2], PZ);
    for (int cell = tid; cell < PZ * TX; cell += kThreads, wc.next()) {
        const int z = 2 * wc.r, x = wc.q;
        const int iz = R.z0 + z;
        const int ix = R.x0 + x;
        // the first row of a pair lies in the tile whenever the second does (z + 1 < TZ implies
        // z < TZ, rows rise with z), so a pair is skipped or has its first row; its second row
        // may lie past the tile, the layer or the grid (then it is computed from clamped loads and
        // never stored)
        if (ix < R.xlo || ix > R.xhi || iz > R.zhi) continue;
        const bool in1 = z + 1 < TZ && iz + 1 <= R.zhi;
        const long long g = (long long)(iz - a.zorg) + (long long)(ix + npml - 1) * a.ldz;
        const long long g1 = in1 ? g + 1 : g;

        if (pml && (ix == 1 - npml || ix == nx + npml || iz == NZ)) {
            // outer frame: never advanced; keep level 1 across the plane swap (a pair that starts
            // on row NZ has no second row in the layer)
            uxn[g] = uxc[g];
            uzn[g] = uzc[g];
            if (in1) { uxn[g1] = uxc[g1]; uzn[g1] = uzc[g1]; }
            continue;
        }

        const int nxo = ordx(a, ix, NO);
        const int nz0 = ordz(a, iz, NO), nz1 = ordz(a, iz + 1, NO);
        const float2 kd = f2(__ldg(a.kdt2 + g), __ldg(a.kdt2 + g1));

        // x-direction second derivatives dxx(l2m ux), dxx(mu uz): half points x+k-1 after the cell,
        // x-k before it (the latter with the order of the column after the half point)
        float2 x2a = f2s(0.f), x2b = f2s(0.f);
#pragma unroll
        for (int k = 1; k <= NO; ++k) {
            const float2 c = f2s(c_stag[nxo][k]);
            const float2 pa = lds2(GX(gxA, z, x + k - 1)), pb = lds2(GX(gxB, z, x + k - 1));
            const float2 ma = lds2(GX(gxAm, z, x - k)), mb = lds2(GX(gxBm, z, x - k));
            x2a = pfma(c, psub(pa, ma), x2a);
            x2b = pfma(c, psub(pb, mb), x2b);
        }
        const float2 Fx2_l2m_ux = pmul(x2a, dx2);
        const float2 Fx2_mu_uz = pmul(x2b, dx2);

        // z-direction second derivatives dzz(l2m uz), dzz(mu ux): half points after the rows from
        // gzA / gzB, before them from gzAm / gzBm
        float2 z2a = f2s(0.f), z2b = f2s(0.f);
        {
            float pa[NO + 1], pb[NO + 1];   // labels z .. z+NO
            float ma[OM + 1], mb[OM + 1];   // labels z-OM .. z
            load_rows(GZ(gzA, z, x), pa);
            load_rows(GZ(gzB, z, x), pb);
            load_rows(GZ(gzAm, z - OM, x), ma);
            load_rows(GZ(gzBm, z - OM, x), mb);
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                const float2 c = f2(c_stag[nz0][k], c_stag[nz1][k]);
                z2a = pfma(c, f2(__fsub_rn(pa[k - 1], ma[OM - k]), __fsub_rn(pa[k], ma[OM + 1 - k])), z2a);
                z2b = pfma(c, f2(__fsub_rn(pb[k - 1], mb[OM - k]), __fsub_rn(pb[k], mb[OM + 1 - k])), z2b);
            }
        }
        const float2 Fz2_l2m_uz = pmul(z2a, dz2);
        const float2 Fz2_mu_ux = pmul(z2b, dz2);

        // mixed derivatives
        float2 zxl = f2s(0.f), zxm = f2s(0.f), xzm = f2s(0.f), xzl = f2s(0.f);
        {
            float w2[NWIN], w3[NWIN];   // rows z-OM .. z+1+NO of v2, v3
            load_rows(GZ(v2, z - OM, x), w2);
            load_rows(GZ(v3, z - OM, x), w3);
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                const float2 cx = f2s(c_coll[nxo][k]), cz = f2(c_coll[nz0][k], c_coll[nz1][k]);
                zxl = pfma(cx, psub(lds2(GX(v1, z, x + k)), lds2(GX(v1, z, x - k))), zxl);
                zxm = pfma(cx, psub(lds2(GX(v4, z, x + k)), lds2(GX(v4, z, x - k))), zxm);
                xzm = pfma(cz, f2(__fsub_rn(w2[OM + k], w2[OM - k]), __fsub_rn(w2[OM + 1 + k], w2[OM + 1 - k])), xzm);
                xzl = pfma(cz, f2(__fsub_rn(w3[OM + k], w3[OM - k]), __fsub_rn(w3[OM + 1 + k], w3[OM + 1 - k])), xzl);
            }
        }
        const float2 Fzx_lam_uz = pmul(zxl, rdx2), Fzx_mu_ux = pmul(zxm, rdx2);
        const float2 Fxz_mu_uz = pmul(xzm, rdz2), Fxz_lam_ux = pmul(xzl, rdz2);

        if (!pml) {
            float2 Fx = padd(padd(padd(Fx2_l2m_ux, Fzx_lam_uz), Fz2_mu_ux), Fxz_mu_uz);
            float2 Fz = padd(padd(padd(Fz2_l2m_uz, Fxz_lam_ux), Fx2_mu_uz), Fzx_mu_ux);
            if (iz == 1) {   // the first row of the pair is the free-surface row
                Fx.x = __fadd_rn(__fadd_rn(Fx2_l2m_ux.x, sFS[kFsA * TX + x]), sFS[kFsQx * TX + x]);
                Fz.x = __fadd_rn(__fadd_rn(Fx2_mu_uz.x, sFS[kFsB * TX + x]), sFS[kFsQz * TX + x]);
            }
            const float2 ux0 = f2(uxc[g], uxc[g1]), uz0 = f2(uzc[g], uzc[g1]);
            const float2 uxm = f2(uxn[g], uxn[g1]), uzm = f2(uzn[g], uzn[g1]);
            const float2 nxv = pfma(kd, Fx, psub(pmul(f2s(2.0f), ux0), uxm));
            const float2 nzv = pfma(kd, Fz, psub(pmul(f2s(2.0f), uz0), uzm));
            uxn[g] = nxv.x;
            uzn[g] = nzv.x;
            if (in1) { uxn[g1] = nxv.y; uzn[g1] = nzv.y; }
            continue;
        }

        // ---- absorbing-layer cells: split-field update ----------------------------------
        const int side = R.side;
        const bool up1 = in1 && iz + 1 != NZ;   // row NZ is outer frame
        // bottom (3) and top (4) layers: damped in x and z, both memory variables
        const bool zl = side >= 3;
        long long ap;   // state index of row iz (row iz+1: ap + 1)
        if (side == 1) ap = (long long)(iz - 1) + (long long)nz * (ix - (1 - npml));
        else if (side == 2) ap = (long long)(iz - 1) + (long long)nz * (ix - nx - 1);
        else if (side == 3) ap = (long long)(iz - nz - 1) + (long long)npml * (ix - (1 - npml));
        else ap = (long long)(iz - izt) + (long long)npml * (ix - (1 - npml));
        const int base = side == 1 ? 0 : side == 2 ? 6 : side == 3 ? 12 : 18;
        const int bpx0 = side == 1 ? 0 : side == 2 ? 2 : side == 3 ? 8 : 4;
        const int nplane = a.cur ^ 1;
        const long long ap1 = up1 ? ap + 1 : ap;
        auto ld = [&](const float* p) { return f2(p[ap], p[ap1]); };
        auto st = [&](float* p, float2 v) {
            p[ap] = v.x;
            if (up1) p[ap1] = v.y;
        };

        // first derivatives for the memory variables (diff1 / diffx1 on the PML field)
        float2 dxux = f2s(0.f), dxuz = f2s(0.f), dzux = f2s(0.f), dzuz = f2s(0.f);
        {
            float wx[NWIN], wz[NWIN];   // rows z-OM .. z+1+NO
            load_rows(SU(sux, z - OM, x), wx);
            load_rows(SU(suz, z - OM, x), wz);
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                const float2 cx = f2s(c_coll[nxo][k]), cz = f2(c_coll[nz0][k], c_coll[nz1][k]);
                dxux = pfma(cx, psub(lds2(SU(sux, z, x + k)), lds2(SU(sux, z, x - k))), dxux);
                dxuz = pfma(cx, psub(lds2(SU(suz, z, x + k)), lds2(SU(suz, z, x - k))), dxuz);
                dzux = pfma(cz, f2(__fsub_rn(wx[OM + k], wx[OM - k]), __fsub_rn(wx[OM + 1 + k], wx[OM + 1 - k])), dzux);
                dzuz = pfma(cz, f2(__fsub_rn(wz[OM + k], wz[OM - k]), __fsub_rn(wz[OM + 1 + k], wz[OM + 1 - k])), dzuz);
            }
        }
        dxux = pmul(dxux, rdx2); dxuz = pmul(dxuz, rdx2);
        dzux = pmul(dzux, rdz2); dzuz = pmul(dzuz, rdz2);
        const float2 lam0 = lds2(SM(sLam, z, x)), mu0 = lds2(SM(sMu, z, x));
        const float2 l2m0 = pfma(f2s(2.0f), mu0, lam0);

        const DampCol dxc = a.dampx[ix + npml - 1];
        DampCol dzc0{0.f, 0.f, 1.f, 1.f}, dzc1{0.f, 0.f, 1.f, 1.f};
        if (zl) {
            dzc0 = a.dampz[iz - izt];
            dzc1 = a.dampz[iz + 1 <= NZ ? iz + 1 - izt : iz - izt];
        }
        const float2 yx = f2s(dxc.y), yz = f2(dzc0.y, dzc1.y);
        // split 2: (2 - yx yz) u - (1 - (yx + yz)/2) u^{n-1}, over 1 + (yx + yz)/2
        const float2 hs = pmul(f2s(0.5f), padd(yx, yz));
        const float2 A2 = pfma(f2s(-dxc.y), yz, f2s(2.0f));
        const float2 B2 = psub(f2s(1.0f), hs);
        const float2 r2 = zl ? f2(fast_rcp(__fadd_rn(1.0f, hs.x)), fast_rcp(__fadd_rn(1.0f, hs.y))) : f2s(dxc.rh);
        // split 1 (x damping): (2 - yx^2) u - (1 - yx) u^{n-1}
        const float2 A1 = f2s(fmaf(-dxc.y, dxc.y, 2.0f)), B1 = f2s(__fsub_rn(1.0f, dxc.y));
        const float2 Cx = f2s(__fsub_rn(1.0f, __fmul_rn(0.5f, dxc.y)));   // 1 - yx/2
#pragma unroll
        for (int comp = 0; comp < 2; ++comp) {
            float2 F1, F2, F3, S1, S3;
            if (comp == 0) {
                F1 = Fx2_l2m_ux;
                F2 = padd(Fzx_lam_uz, Fxz_mu_uz);
                F3 = Fz2_mu_ux;
                S1 = pmul(l2m0, dxux);
                S3 = pmul(mu0, dzux);
            } else {
                F1 = Fx2_mu_uz;
                F2 = padd(Fxz_lam_ux, Fzx_mu_ux);
                F3 = Fz2_l2m_uz;
                S1 = pmul(mu0, dxuz);
                S3 = pmul(l2m0, dzuz);
            }
            // free-surface row of a side layer (first row of the pair; with the top layer, row 1
            // of the side layers takes the general terms)
            if (iz == 1 && izt == 1) {
                F2.x = sFS[(comp == 0 ? kFsF2x : kFsF2z) * TX + x];
                F3.x = sFS[(comp == 0 ? kFsF3x : kFsF3z) * TX + x];
            }
            float* bpx = a.bp[zl ? bpx0 + 2 * comp : bpx0 + comp];
            const float2 Px = ld(bpx);
            // memory variable: ((1 - yx/2) Px - dt d' S1) / (1 + yx/2)
            const float2 Pxn = pmul(pfma(f2s(-dxc.dtdp), S1, pmul(Cx, Px)), f2s(dxc.rh));
            const float2 u1 = ld(a.bu[base + 3 * comp + 0][a.cur]), u1m = ld(a.bu[base + 3 * comp + 0][nplane]);
            const float2 u2 = ld(a.bu[base + 3 * comp + 1][a.cur]), u2m = ld(a.bu[base + 3 * comp + 1][nplane]);
            const float2 u3 = ld(a.bu[base + 3 * comp + 2][a.cur]), u3m = ld(a.bu[base + 3 * comp + 2][nplane]);
            const float2 f1 = pmul(kd, pfma(f2s(0.5f), padd(Pxn, Px), F1));   // kd (F1 + (Pxn + Px)/2)
            const float2 t1 = pfma(A1, u1, pmul(f2s(-B1.x), u1m));
            const float2 n1o = pmul(padd(t1, f1), f2s(dxc.r1));
            float2 n1 = n1o;
            if (side == 2) {   // right layer below a free-surface row 1: the force is not divided by 1 + yx
                const float2 n1r = pfma(t1, f2s(dxc.r1), f1);
                n1 = f2(iz == 1 && izt == 1 ? n1o.x : n1r.x, n1r.y);
            }
            const float2 n2 = pmul(pfma(kd, F2, pfma(A2, u2, pmul(f2(-B2.x, -B2.y), u2m))), r2);
            float2 n3;
            if (zl) {
                float* bpz = a.bp[bpx0 + 1 + 2 * comp];
                const float2 Pz = ld(bpz);
                const float2 Cz = f2(__fsub_rn(1.0f, __fmul_rn(0.5f, dzc0.y)), __fsub_rn(1.0f, __fmul_rn(0.5f, dzc1.y)));
                const float2 Pzn = pmul(pfma(f2(-dzc0.dtdp, -dzc1.dtdp), S3, pmul(Cz, Pz)), f2(dzc0.rh, dzc1.rh));
                st(bpz, Pzn);
                const float2 A3 = pfma(f2(-dzc0.y, -dzc1.y), yz, f2s(2.0f));
                const float2 B3 = f2(-__fsub_rn(1.0f, dzc0.y), -__fsub_rn(1.0f, dzc1.y));
                const float2 t3 = pfma(A3, u3, pmul(B3, u3m));
                n3 = pmul(pfma(kd, pfma(f2s(0.5f), padd(Pzn, Pz), F3), t3), f2(dzc0.r1, dzc1.r1));
            } else {
                n3 = pfma(kd, F3, psub(pmul(f2s(2.0f), u3), u3m));
            }
            st(bpx, Pxn);
            st(a.bu[base + 3 * comp + 0][nplane], n1);
            st(a.bu[base + 3 * comp + 1][nplane], n2);
            st(a.bu[base + 3 * comp + 2][nplane], n3);
            const float2 un = padd(padd(n1, n2), n3);
            float* const out = comp == 0 ? uxn : uzn;
            out[g] = un.x;
            if (up1) out[g1] = un.y;
        }
        // second row on row NZ (outer frame): level 1 kept across the plane swap
        if (in1 && !up1) { uxn[g1] = uxc[g1]; uzn[g1] = uzc[g1]; }
    }
    // the top layer's outer row izt (never advanced): level 1 kept, by the tiles next to it
    if (R.side == 4 && R.z0 == izt + 1) {
        for (int x = tid; x < TX; x += kThreads) {
            const int ix = R.x0 + x;
            if (ix > R.xhi) break;
            const long long g = (long long)(izt - a.zorg) + (long long)(ix + npml - 1) * a.ldz;
            uxn[g] = uxc[g];
            uzn[g] = uzc[g];
        }
    }
#undef SU
#undef SM
#undef GX
#undef GZ
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

// The top layers of the members with the absorbing layer on top: member s owns blocks
// top_off[s] .. top_off[s+1]-1 of this launch, queued after the step's interior update.
template <int NO>
__global__ void __launch_bounds__(kThreads, 3) fdfk_step_top_batch_kernel(BatchTab t)
{
    __shared__ StepArgs sa;
    const int s = batch_member(t.top_off, t.n, blockIdx.x);
    if (!t.live[s]) return;                // the whole block returns: no barrier is split
    stage_args(sa, t.args + s);
    if (threadIdx.x == 0) {
        sa.top_pass = 1;
        sa.n_tiles = sa.tiles_t_z * sa.tiles_t_x;
        sa.nrcv = 0;
    }
    __syncthreads();
    step_block<NO>(sa, blockIdx.x - t.top_off[s]);
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
    // (a.top_pass: a.n_tiles counts the top layer's tiles, no receiver blocks)
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

cudaError_t launch_step_top(const StepArgs& a0, cudaStream_t s)
{
    if (a0.izt == 1) return cudaSuccess;
    StepArgs a = a0;
    a.top_pass = 1;
    a.n_tiles = a.tiles_t_z * a.tiles_t_x;
    a.nrcv = 0;
    switch (a.norder) {
    case 1: return launch_no<1>(a, 0, s);
    case 2: return launch_no<2>(a, 0, s);
    case 3: return launch_no<3>(a, 0, s);
    case 4: return launch_no<4>(a, 0, s);
    case 5: return launch_no<5>(a, 0, s);
    case 6: return launch_no<6>(a, 0, s);
    case 7: return launch_no<7>(a, 0, s);
    case 8: return launch_no<8>(a, 0, s);
    default: return cudaErrorInvalidValue;
    }
}

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

template <int NO>
static cudaError_t launch_top_batch_no(const BatchTab& t, int blocks, size_t smem, cudaStream_t s)
{
    static int configured = 0;
    if ((int)smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(fdfk_step_top_batch_kernel<NO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        configured = (int)smem;
    }
    if (blocks == 0) return cudaSuccess;
    fdfk_step_top_batch_kernel<NO><<<blocks, kThreads, smem, s>>>(t);
    return cudaGetLastError();
}

cudaError_t launch_step_top_batch(const BatchTab& t, int norder, int blocks, size_t smem, cudaStream_t s)
{
    switch (norder) {
    case 1: return launch_top_batch_no<1>(t, blocks, smem, s);
    case 2: return launch_top_batch_no<2>(t, blocks, smem, s);
    case 3: return launch_top_batch_no<3>(t, blocks, smem, s);
    case 4: return launch_top_batch_no<4>(t, blocks, smem, s);
    case 5: return launch_top_batch_no<5>(t, blocks, smem, s);
    case 6: return launch_top_batch_no<6>(t, blocks, smem, s);
    case 7: return launch_top_batch_no<7>(t, blocks, smem, s);
    case 8: return launch_top_batch_no<8>(t, blocks, smem, s);
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
// int_rows, so the interior tiles are flat tiles of the top band, all its rows (rounded up to
// even, at most 16) by kBandTX columns.  The
// absorbing layers are cut into tiles whose thickness divides npml evenly (at most kPmlTile)
// and pml_run cells (kPmlRun when not tuned) along the layer.
void plan_tiles(StepArgs& a, bool band_top, int pml_run)
{
    if (pml_run < 8) pml_run = kPmlRun;
    auto cdiv = [](int x, int y) { return (x + y - 1) / y; };
    const int nt = cdiv(a.npml, kPmlTile);
    const int th = cdiv(a.npml, nt);
    a.tdz[0] = band_top ? std::min((a.int_rows + 1) & ~1, 2 * kMaxOrder) : kTZ;
    a.tdx[0] = band_top ? kBandTX : kTX;
    a.tdz[1] = pml_run; a.tdx[1] = th;
    a.tdz[2] = th; a.tdx[2] = pml_run;
    a.tiles_int_z = cdiv(a.int_rows, a.tdz[0]);
    a.tiles_int_x = cdiv(a.nx, a.tdx[0]);
    a.tiles_l_z = cdiv(a.nz, a.tdz[1]);
    a.tiles_l_x = cdiv(a.npml, a.tdx[1]);
    a.tiles_b_z = cdiv(a.npml, a.tdz[2]);
    a.tiles_b_x = cdiv(a.NX, a.tdx[2]);
    // the top layer (rows izt+1..0) in the bottom tiles' shape, launched on its own (launch_step_top)
    a.tiles_t_z = a.izt < 1 ? cdiv(-a.izt, a.tdz[2]) : 0;
    a.tiles_t_x = a.izt < 1 ? a.tiles_b_x : 0;
    a.top_pass = 0;
    a.n_tiles = a.tiles_int_z * a.tiles_int_x + 2 * a.tiles_l_z * a.tiles_l_x + a.tiles_b_z * a.tiles_b_x;
    for (int c = 0; c < 3; ++c) {
        const TileDims T = tile_dims(a.norder, a.tdz[c], a.tdx[c]);
        const int n[3] = {T.UZ / 2, T.MZ / 2, T.TZe / 2};
        for (int d = 0; d < 3; ++d) {
            a.wq[c][d] = kThreads / n[d];
            a.wr[c][d] = kThreads % n[d];
        }
    }
    const int nx = a.nx, nz = a.nz, nbd = a.nbd;
    // a strip stored from (zr0, xr0), its rows from row 1 on and (xs: where it starts in x, past
    // the stored origin for the right inner strip, which starts after the left one where the two
    // would meet on narrow grids)
    auto box = [](int zr0, int zr1, int xr0, int xs, int xr1, int rows, int cols, int sx, int sz) {
        return StripBox{std::max(zr0, 1), zr1, xs, xr1, rows, cols, zr0 + rows * xr0, sx, sz};
    };
    a.sbox[0] = box(1, nz - nbd, 1, 1, nbd, nz - nbd, nbd, UXL_REG, UZL_REG);
    a.sbox[1] = box(1, nz - nbd, nx - nbd + 1, std::max(nx - nbd + 1, nbd + 1), nx, nz - nbd, nbd, UXR_REG, UZR_REG);
    a.sbox[2] = box(nz - nbd + 1, nz, 1, 1, nx, nbd, nx, UXB_REG, UZB_REG);
    a.sbox[3] = box(1, nz, 1 - nbd, 1 - nbd, 0, nz, nbd, UXL_PML, UZL_PML);
    a.sbox[4] = box(1, nz, nx + 1, nx + 1, nx + nbd, nz, nbd, UXR_PML, UZR_PML);
    a.sbox[5] = box(nz + 1, nz + nbd, 1 - nbd, 1 - nbd, nx + nbd, nbd, nx + 2 * nbd, UXB_PML, UZB_PML);
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
