// Interior fast path of the hybrid FD-FK step (sm_103a): the bulk of the
// regular domain, rows MarchArgs::z0..nz, columns 1..nx.
//
// Each warp owns a band of 64 rows (2 per lane; z is the contiguous axis, so
// every global access of a warp is one contiguous 256-byte run) and marches
// along x over a segment of columns.  x-direction stencils live in register
// windows that slide with the march; z-direction stencils read neighbouring
// rows with warp shuffles.  Nothing goes through shared memory and there is
// no block-level synchronisation.  The 2*norder halo rows on each side of a
// band are computed but not stored; bands overlap accordingly.  The first
// 2*norder march steps of a segment only fill the windows.
//
// Semantics are those of fdfk_step_kernel's interior tiles with full stencil
// orders (src/Submain.f90 diffx2/diffz2/diffxz/diffzx *_reg): the fast path
// starts below the rows where the top boundary reduces the order, and the
// outer background strips (Omega_II) are added to every loaded value that lies
// on them (Alterman-Karal injection).
//
// Included by fdfk_sweep.cu after the coefficient tables c_stag / c_coll are
// defined: constant memory is per translation unit without relocatable
// device code, so both kernels live in the same one.
#pragma once
#include "fdfk_sweep.cuh"

#include <cuda_runtime.h>

namespace fdfk {

namespace march {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float frcp(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Value of a two-rows-per-lane quantity at row offset D from this lane's first row.
template <int D>
__device__ __forceinline__ float zrow(float a0, float a1)
{
    constexpr int q = (D >= 0) ? D / 2 : -((1 - D) / 2);   // floor(D / 2)
    constexpr int e = D - 2 * q;                             // 0 or 1
    const float v = e ? a1 : a0;
    if constexpr (q == 0) return v;
    else if constexpr (q > 0) return __shfl_down_sync(kFull, v, q);
    else return __shfl_up_sync(kFull, v, -q);
}

// Collocated z-derivative sums (no 1/dz) of a column at this lane's two rows.
template <int NO>
__device__ __forceinline__ void dz_coll(float v0, float v1, float& d0, float& d1)
{
    float s0 = 0.f, s1 = 0.f;
#define FDFK_DZ(k)                                                                          \
    if constexpr (NO >= k) {                                                                \
        s0 = fmaf(c_coll[NO][k], zrow<k>(v0, v1) - zrow<-(k)>(v0, v1), s0);               \
        s1 = fmaf(c_coll[NO][k], zrow<(k) + 1>(v0, v1) - zrow<1 - (k)>(v0, v1), s1);      \
    }
    FDFK_DZ(1) FDFK_DZ(2) FDFK_DZ(3) FDFK_DZ(4)
#undef FDFK_DZ
    d0 = s0;
    d1 = s1;
}

// Staggered z-derivative sums at the half rows below this lane's rows
// (label L between rows L and L+1, for L = r0 and r0+1).
template <int NO>
__device__ __forceinline__ void dz_stag(float v0, float v1, float& d0, float& d1)
{
    float s0 = 0.f, s1 = 0.f;
#define FDFK_DS(j)                                                                          \
    if constexpr (NO >= j) {                                                                \
        s0 = fmaf(c_stag[NO][j], zrow<j>(v0, v1) - zrow<1 - (j)>(v0, v1), s0);            \
        s1 = fmaf(c_stag[NO][j], zrow<(j) + 1>(v0, v1) - zrow<2 - (j)>(v0, v1), s1);      \
    }
    FDFK_DS(1) FDFK_DS(2) FDFK_DS(3) FDFK_DS(4)
#undef FDFK_DS
    d0 = s0;
    d1 = s1;
}

// Staggered z-derivative of half-row quantities G (label = upper row) at this lane's rows:
// sum_k c_k (G(r+k-1) - G(r-k)).
template <int NO>
__device__ __forceinline__ void dz_of_half(float g0, float g1, float& d0, float& d1)
{
    float s0 = 0.f, s1 = 0.f;
#define FDFK_DH(k)                                                                          \
    if constexpr (NO >= k) {                                                                \
        s0 = fmaf(c_stag[NO][k], zrow<(k) - 1>(g0, g1) - zrow<-(k)>(g0, g1), s0);         \
        s1 = fmaf(c_stag[NO][k], zrow<(k)>(g0, g1) - zrow<1 - (k)>(g0, g1), s1);          \
    }
    FDFK_DH(1) FDFK_DH(2) FDFK_DH(3) FDFK_DH(4)
#undef FDFK_DH
    d0 = s0;
    d1 = s1;
}

}  // namespace march

template <int NO>
__global__ void __launch_bounds__(128) fdfk_march_kernel(StepArgs a, MarchArgs m)
{
    using namespace march;
    constexpr int W = 3 * NO;        // field window: columns x-NO .. x+2NO-1
    constexpr int WG = 2 * NO;       // staggered products: half points x-NO+1/2 .. x+NO-1/2
    constexpr int WV = 2 * NO + 1;   // dzx operands: columns x-NO .. x+NO

    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * (blockDim.x >> 5)) + (threadIdx.x >> 5);
    if (warp >= m.n_bands * m.n_segs) return;
    const int band = warp % m.n_bands, seg = warp / m.n_bands;
    const int b = m.z0 + band * m.band_out - 2 * NO;   // first row of the band
    const int r0 = b + 2 * lane;                        // this lane's rows r0, r0+1
    const int xs = 1 + seg * m.seg_len;
    const int xe = min(a.nx, xs + m.seg_len - 1);
    const int nx = a.nx, nz = a.nz, NZ = a.NZ, npml = a.npml, ldz = a.ldz;
    const bool store = lane >= NO && lane <= 31 - NO && r0 >= m.z0 && r0 <= nz;
    const bool store1 = store && r0 + 1 <= nz;
    const bool rows_in = r0 >= 1 && r0 + 1 <= NZ;
    const bool r0_in = r0 >= 1 && r0 <= NZ, r1_in = r0 + 1 >= 1 && r0 + 1 <= NZ;
    const bool r1_int = r0 + 1 <= nz;                   // second row above the bottom strip
    const bool bot = r0 + 1 > nz;                       // rows that may hold bottom background
    const int nbd = a.nbd, it = a.it;

    const float* __restrict__ uxc = a.ux[a.cur];
    const float* __restrict__ uzc = a.uz[a.cur];
    float* __restrict__ uxn = a.ux[a.cur ^ 1];
    float* __restrict__ uzn = a.uz[a.cur ^ 1];
    const float rdx = 1.0f / a.dx, rdz = 1.0f / a.dz;
    const float dx2 = a.dx2r, dz2 = a.dz2;

    auto colbase = [&](int ix) -> size_t { return (size_t)(ix + npml - 1) * (size_t)ldz + (size_t)(r0 - 1); };
    auto load_pair = [&](const float* __restrict__ p, size_t o, float& v0, float& v1) {
        if (rows_in) {
            const float2 v = __ldg(reinterpret_cast<const float2*>(p + o));
            v0 = v.x; v1 = v.y;
        } else {
            v0 = r0_in ? __ldg(p + o) : 0.f;
            v1 = r1_in ? __ldg(p + o + 1) : 0.f;
        }
    };
    // field column with the Omega_II background added; zero outside the grid
    auto load_u = [&](int ix, float& x0, float& x1, float& z0, float& z1) {
        if (ix < 1 - npml || ix > nx + npml) { x0 = x1 = z0 = z1 = 0.f; return; }
        const size_t o = colbase(ix);
        load_pair(uxc, o, x0, x1);
        load_pair(uzc, o, z0, z1);
        if ((ix <= 0 && ix >= 1 - nbd) || (ix > nx && ix <= nx + nbd)) {
            if (r0 >= 1 && r0 <= nz) {
                const bool left = ix <= 0;
                const size_t so = (size_t)(r0 - 1) + (size_t)nz * ((size_t)(left ? ix - (1 - nbd) : ix - nx - 1) + (size_t)nbd * it);
                const float* sx = a.strip[left ? UXL_PML : UXR_PML] + so;
                const float* sz = a.strip[left ? UZL_PML : UZR_PML] + so;
                x0 += __ldg(sx); z0 += __ldg(sz);
                if (r1_int) { x1 += __ldg(sx + 1); z1 += __ldg(sz + 1); }
            }
        }
        if (bot && ix >= 1 - nbd && ix <= nx + nbd) {
            const size_t cb = (size_t)(nx + 2 * nbd) * it + (size_t)(ix - (1 - nbd));
            if (r0 >= nz + 1 && r0 <= nz + nbd) {
                const size_t so = (size_t)(r0 - nz - 1) + (size_t)nbd * cb;
                x0 += __ldg(a.strip[UXB_PML] + so); z0 += __ldg(a.strip[UZB_PML] + so);
            }
            if (r0 + 1 >= nz + 1 && r0 + 1 <= nz + nbd) {
                const size_t so = (size_t)(r0 - nz) + (size_t)nbd * cb;
                x1 += __ldg(a.strip[UXB_PML] + so); z1 += __ldg(a.strip[UZB_PML] + so);
            }
        }
    };
    auto load_mat = [&](int ix, float& l0, float& l1, float& m0, float& m1) {
        if (ix < 1 - npml || ix > nx + npml) { l0 = l1 = 0.f; m0 = m1 = 1.f; return; }
        const size_t o = colbase(ix);
        if (rows_in) {
            const float2 l = __ldg(reinterpret_cast<const float2*>(a.lam + o));
            const float2 mm = __ldg(reinterpret_cast<const float2*>(a.mu + o));
            l0 = l.x; l1 = l.y; m0 = mm.x; m1 = mm.y;
        } else {
            l0 = r0_in ? __ldg(a.lam + o) : 0.f;
            l1 = r1_in ? __ldg(a.lam + o + 1) : 0.f;
            m0 = r0_in ? __ldg(a.mu + o) : 1.f;
            m1 = r1_in ? __ldg(a.mu + o + 1) : 1.f;
        }
    };

    float Ux[W][2], Uz[W][2];        // column x - NO + c
    float Ga[WG][2], Gb[WG][2];      // H(l2m) Dstag_x ux, H(mu) Dstag_x uz at half point x - NO + 1/2 + c
    float V1[WV][2], V4[WV][2];      // lam Dz uz / dz, mu Dz ux / dz at column x - NO + c
    float RL0[2], RL1[2], RM0[2], RM1[2];   // 1/l2m, 1/mu at columns x+NO-1 (0) and x+NO (1)

    // prologue: field columns x0-NO .. x0+2NO-2 and the reciprocals of column x0+NO-1
    const int x0 = xs - 2 * NO;
#pragma unroll
    for (int c = 0; c < W - 1; ++c) load_u(x0 - NO + c, Ux[c][0], Ux[c][1], Uz[c][0], Uz[c][1]);
    {
        float l0, l1, m0, m1;
        load_mat(x0 + NO - 1, l0, l1, m0, m1);
        RL1[0] = frcp(l0 + 2.0f * m0); RL1[1] = frcp(l1 + 2.0f * m1);
        RM1[0] = frcp(m0); RM1[1] = frcp(m1);
    }
#pragma unroll
    for (int c = 0; c < WG; ++c) { Ga[c][0] = Ga[c][1] = Gb[c][0] = Gb[c][1] = 0.f; }
#pragma unroll
    for (int c = 0; c < WV; ++c) { V1[c][0] = V1[c][1] = V4[c][0] = V4[c][1] = 0.f; }

    // the newest field and material columns are fetched one march step ahead of their use
    float pux0, pux1, puz0, puz1, pl0, pl1, pm0, pm1;
    load_u(x0 + 2 * NO - 1, pux0, pux1, puz0, puz1);
    load_mat(x0 + NO, pl0, pl1, pm0, pm1);

    for (int x = x0; x <= xe; ++x) {
        // newest field column x+2NO-1, newest material column x+NO
        Ux[W - 1][0] = pux0; Ux[W - 1][1] = pux1; Uz[W - 1][0] = puz0; Uz[W - 1][1] = puz1;
        const float ln0 = pl0, ln1 = pl1, mn0 = pm0, mn1 = pm1;
        load_u(x + 2 * NO, pux0, pux1, puz0, puz1);
        load_mat(x + 1 + NO, pl0, pl1, pm0, pm1);
        // operands of this column's update, issued before the arithmetic that hides their latency
        float lc0 = 0.f, lc1 = 0.f, mc0 = 1.f, mc1 = 1.f;
        float2 k2 = make_float2(0.f, 0.f), xp = k2, zp = k2;
        const size_t ox = colbase(x);
        if (x >= xs) {
            load_mat(x, lc0, lc1, mc0, mc1);
            if (store1) {
                k2 = __ldg(reinterpret_cast<const float2*>(a.kdt2 + ox));
                xp = *reinterpret_cast<const float2*>(uxn + ox);
                zp = *reinterpret_cast<const float2*>(uzn + ox);
            } else if (store) {
                k2.x = __ldg(a.kdt2 + ox);
                xp.x = uxn[ox];
                zp.x = uzn[ox];
            }
        }
        RL0[0] = RL1[0]; RL0[1] = RL1[1]; RM0[0] = RM1[0]; RM0[1] = RM1[1];
        RL1[0] = frcp(ln0 + 2.0f * mn0); RL1[1] = frcp(ln1 + 2.0f * mn1);
        RM1[0] = frcp(mn0); RM1[1] = frcp(mn1);

        // staggered products at the half point x+NO-1/2 (window columns 2NO-1 | 2NO)
        {
            float sx0 = 0.f, sx1 = 0.f, sz0 = 0.f, sz1 = 0.f;
#pragma unroll
            for (int j = 1; j <= NO; ++j) {
                const int cp = 2 * NO - 1 + j, cm = 2 * NO - j;
                sx0 = fmaf(c_stag[NO][j], Ux[cp][0] - Ux[cm][0], sx0);
                sx1 = fmaf(c_stag[NO][j], Ux[cp][1] - Ux[cm][1], sx1);
                sz0 = fmaf(c_stag[NO][j], Uz[cp][0] - Uz[cm][0], sz0);
                sz1 = fmaf(c_stag[NO][j], Uz[cp][1] - Uz[cm][1], sz1);
            }
            Ga[WG - 1][0] = 2.0f * frcp(RL0[0] + RL1[0]) * sx0;
            Ga[WG - 1][1] = 2.0f * frcp(RL0[1] + RL1[1]) * sx1;
            Gb[WG - 1][0] = 2.0f * frcp(RM0[0] + RM1[0]) * sz0;
            Gb[WG - 1][1] = 2.0f * frcp(RM0[1] + RM1[1]) * sz1;
        }
        // dzx operands at column x+NO (window column 2NO)
        {
            float dzz0, dzz1, dzx0, dzx1;
            dz_coll<NO>(Uz[2 * NO][0], Uz[2 * NO][1], dzz0, dzz1);
            dz_coll<NO>(Ux[2 * NO][0], Ux[2 * NO][1], dzx0, dzx1);
            V1[WV - 1][0] = ln0 * dzz0 * rdz; V1[WV - 1][1] = ln1 * dzz1 * rdz;
            V4[WV - 1][0] = mn0 * dzx0 * rdz; V4[WV - 1][1] = mn1 * dzx1 * rdz;
        }

        if (x >= xs) {
            // dxz operands at column x: mu Dx uz / dx, lam Dx ux / dx
            float s20 = 0.f, s21 = 0.f, s30 = 0.f, s31 = 0.f;
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                s20 = fmaf(c_coll[NO][k], Uz[NO + k][0] - Uz[NO - k][0], s20);
                s21 = fmaf(c_coll[NO][k], Uz[NO + k][1] - Uz[NO - k][1], s21);
                s30 = fmaf(c_coll[NO][k], Ux[NO + k][0] - Ux[NO - k][0], s30);
                s31 = fmaf(c_coll[NO][k], Ux[NO + k][1] - Ux[NO - k][1], s31);
            }
            const float v20 = mc0 * s20 * rdx, v21 = mc1 * s21 * rdx;
            const float v30 = lc0 * s30 * rdx, v31 = lc1 * s31 * rdx;
            // z staggered products at column x below this lane's rows
            float sa0, sa1, sb0, sb1;
            dz_stag<NO>(Uz[NO][0], Uz[NO][1], sa0, sa1);
            dz_stag<NO>(Ux[NO][0], Ux[NO][1], sb0, sb1);
            const float rl0 = frcp(lc0 + 2.0f * mc0), rl1 = frcp(lc1 + 2.0f * mc1);
            const float rm0 = frcp(mc0), rm1 = frcp(mc1);
            const float rl2 = zrow<2>(rl0, rl1), rm2 = zrow<2>(rm0, rm1);
            const float gzA0 = 2.0f * frcp(rl0 + rl1) * sa0, gzA1 = 2.0f * frcp(rl1 + rl2) * sa1;
            const float gzB0 = 2.0f * frcp(rm0 + rm1) * sb0, gzB1 = 2.0f * frcp(rm1 + rm2) * sb1;
            float z2a0, z2a1, z2b0, z2b1, xzm0, xzm1, xzl0, xzl1;
            dz_of_half<NO>(gzA0, gzA1, z2a0, z2a1);
            dz_of_half<NO>(gzB0, gzB1, z2b0, z2b1);
            dz_coll<NO>(v20, v21, xzm0, xzm1);
            dz_coll<NO>(v30, v31, xzl0, xzl1);

            float x2a0 = 0.f, x2a1 = 0.f, x2b0 = 0.f, x2b1 = 0.f;
            float zxl0 = 0.f, zxl1 = 0.f, zxm0 = 0.f, zxm1 = 0.f;
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                const float cs = c_stag[NO][k], cc = c_coll[NO][k];
                x2a0 = fmaf(cs, Ga[NO - 1 + k][0] - Ga[NO - k][0], x2a0);
                x2a1 = fmaf(cs, Ga[NO - 1 + k][1] - Ga[NO - k][1], x2a1);
                x2b0 = fmaf(cs, Gb[NO - 1 + k][0] - Gb[NO - k][0], x2b0);
                x2b1 = fmaf(cs, Gb[NO - 1 + k][1] - Gb[NO - k][1], x2b1);
                zxl0 = fmaf(cc, V1[NO + k][0] - V1[NO - k][0], zxl0);
                zxl1 = fmaf(cc, V1[NO + k][1] - V1[NO - k][1], zxl1);
                zxm0 = fmaf(cc, V4[NO + k][0] - V4[NO - k][0], zxm0);
                zxm1 = fmaf(cc, V4[NO + k][1] - V4[NO - k][1], zxm1);
            }
            if (store) {
                const float Fx0 = x2a0 * dx2 + zxl0 * rdx + z2b0 * dz2 + xzm0 * rdz;
                const float Fx1 = x2a1 * dx2 + zxl1 * rdx + z2b1 * dz2 + xzm1 * rdz;
                const float Fz0 = z2a0 * dz2 + xzl0 * rdz + x2b0 * dx2 + zxm0 * rdx;
                const float Fz1 = z2a1 * dz2 + xzl1 * rdz + x2b1 * dx2 + zxm1 * rdx;
                // own rows of an interior column carry no background: the window holds u^n
                if (store1) {
                    xp.x = fmaf(k2.x, Fx0, 2.0f * Ux[NO][0] - xp.x);
                    xp.y = fmaf(k2.y, Fx1, 2.0f * Ux[NO][1] - xp.y);
                    zp.x = fmaf(k2.x, Fz0, 2.0f * Uz[NO][0] - zp.x);
                    zp.y = fmaf(k2.y, Fz1, 2.0f * Uz[NO][1] - zp.y);
                    *reinterpret_cast<float2*>(uxn + ox) = xp;
                    *reinterpret_cast<float2*>(uzn + ox) = zp;
                } else {
                    uxn[ox] = fmaf(k2.x, Fx0, 2.0f * Ux[NO][0] - xp.x);
                    uzn[ox] = fmaf(k2.x, Fz0, 2.0f * Uz[NO][0] - zp.x);
                }
            }
        }

        // slide the windows by one column
#pragma unroll
        for (int c = 0; c < W - 1; ++c) {
            Ux[c][0] = Ux[c + 1][0]; Ux[c][1] = Ux[c + 1][1];
            Uz[c][0] = Uz[c + 1][0]; Uz[c][1] = Uz[c + 1][1];
        }
#pragma unroll
        for (int c = 0; c < WG - 1; ++c) {
            Ga[c][0] = Ga[c + 1][0]; Ga[c][1] = Ga[c + 1][1];
            Gb[c][0] = Gb[c + 1][0]; Gb[c][1] = Gb[c + 1][1];
        }
#pragma unroll
        for (int c = 0; c < WV - 1; ++c) {
            V1[c][0] = V1[c + 1][0]; V1[c][1] = V1[c + 1][1];
            V4[c][0] = V4[c + 1][0]; V4[c][1] = V4[c + 1][1];
        }
    }
}

template <int NO>
static cudaError_t launch_march_no(const StepArgs& a, const MarchArgs& m, cudaStream_t s)
{
    const int warps = m.n_bands * m.n_segs;
    const int blocks = (warps + 3) / 4;
    fdfk_march_kernel<NO><<<blocks, 128, 0, s>>>(a, m);
    return cudaGetLastError();
}

template <int NO>
static int warp_slots_no()
{
    int dev = 0, sms = 0, blocks = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fdfk_march_kernel<NO>, 128, 0) != cudaSuccess) return 0;
    return sms * blocks * 4;
}

// Resident warps of the fast-path kernel on the current device (0 if unknown).
int march_warp_slots(int norder)
{
    switch (norder) {
    case 1: return warp_slots_no<1>();
    case 2: return warp_slots_no<2>();
    case 3: return warp_slots_no<3>();
    case 4: return warp_slots_no<4>();
    default: return 0;
    }
}

cudaError_t launch_march(const StepArgs& a, const MarchArgs& m, cudaStream_t s)
{
    if (m.n_bands <= 0 || m.n_segs <= 0) return cudaSuccess;
    switch (a.norder) {
    case 1: return launch_march_no<1>(a, m, s);
    case 2: return launch_march_no<2>(a, m, s);
    case 3: return launch_march_no<3>(a, m, s);
    case 4: return launch_march_no<4>(a, m, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace fdfk
