// Interior fast path of the hybrid FD-FK step (sm_103a): the bulk of the
// regular domain, rows MarchArgs::z0..nz, columns 1..nx.
//
// Each warp owns a band of 64 rows (2 per lane; z is the contiguous axis, so
// every global access of a warp is one contiguous 256-byte run) and marches
// along x over a segment of columns, reading each field column once.  The
// x-direction stencils are evaluated in transposed (accumulator) form: every
// incoming column is folded with one FMA per stencil tap into a short chain of
// partial sums that advances with the march, so no operand windows are kept
// or shifted.  z-direction stencils read neighbouring rows with warp shuffles,
// one shuffle per distinct neighbour row.  Nothing goes through shared memory
// and there is no block-level synchronisation.  The 2*norder halo rows on
// each side of a band are computed but not stored; bands overlap accordingly.
//
// With newest column m, the pipeline delivers
//   S(h) = staggered x-derivative at half point h = m - NO + 1/2   (lag NO - 1/2)
//   Dx u  collocated x-derivative at column m - NO                  (lag NO)
//   V     = M Dz u / dz at column m                                  (lag 0)
// and accumulates the force of cells m - 2NO + 1 .. m + NO; cell
// m - 2NO + 1 is complete and is advanced in time.
//
// Semantics are those of fdfk_step_kernel's interior tiles with full stencil
// orders (src/Submain.f90 diffx2/diffz2/diffxz/diffzx *_reg): the fast path
// starts below the rows where the top boundary reduces the order, and the
// outer background strips (Omega_II) are added to every loaded value that
// lies on them (Alterman-Karal injection).
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

// Rows r0+LO .. r0+HI of a two-rows-per-lane quantity (one shuffle per row not held by this lane).
template <int LO, int HI>
struct ZCol {
    float v[HI - LO + 1];
    __device__ __forceinline__ ZCol(float a0, float a1) { fill<LO>(a0, a1); }
    template <int D>
    __device__ __forceinline__ void fill(float a0, float a1)
    {
        if constexpr (D <= HI) {
            v[D - LO] = zrow<D>(a0, a1);
            fill<D + 1>(a0, a1);
        }
    }
    __device__ __forceinline__ float operator()(int d) const { return v[d - LO]; }
};

// sum_k c1_k (q(r+k) - q(r-k)) at this lane's two rows
template <int NO>
__device__ __forceinline__ void dz_coll(float a0, float a1, float& d0, float& d1)
{
    const ZCol<-NO, NO + 1> z(a0, a1);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int k = 1; k <= NO; ++k) {
        s0 = fmaf(c_coll[NO][k], z(k) - z(-k), s0);
        s1 = fmaf(c_coll[NO][k], z(k + 1) - z(1 - k), s1);
    }
    d0 = s0;
    d1 = s1;
}

// sum_j c0_j (q(L+j) - q(L+1-j)) at the half rows L = r0, r0+1 (label = upper row)
template <int NO>
__device__ __forceinline__ void dz_stag(float a0, float a1, float& d0, float& d1)
{
    const ZCol<1 - NO, NO + 1> z(a0, a1);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int j = 1; j <= NO; ++j) {
        s0 = fmaf(c_stag[NO][j], z(j) - z(1 - j), s0);
        s1 = fmaf(c_stag[NO][j], z(j + 1) - z(2 - j), s1);
    }
    d0 = s0;
    d1 = s1;
}

// sum_k c0_k (G(r+k-1) - G(r-k)) of half-row quantities G at this lane's rows
template <int NO>
__device__ __forceinline__ void dz_half(float g0, float g1, float& d0, float& d1)
{
    const ZCol<-NO, NO> z(g0, g1);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int k = 1; k <= NO; ++k) {
        s0 = fmaf(c_stag[NO][k], z(k - 1) - z(-k), s0);
        s1 = fmaf(c_stag[NO][k], z(k) - z(1 - k), s1);
    }
    d0 = s0;
    d1 = s1;
}

}  // namespace march

template <int NO>
__global__ void __launch_bounds__(128) fdfk_march_kernel(StepArgs a, MarchArgs m)
{
    using namespace march;
    constexpr int NS = 2 * NO;       // staggered partial sums: half points m-NO+1/2 .. m+NO-1/2
    constexpr int ND = 2 * NO + 1;   // collocated partial sums: columns m-NO .. m+NO
    constexpr int NF = 3 * NO;       // force accumulators: cells m-2NO+1 .. m+NO
    constexpr int LAG = 2 * NO - 1;  // newest column minus completed cell

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

    // element offset of (r0, column ix); 32-bit: grids are below 2^31 cells
    const int rowoff = r0 - 1;
    auto colbase = [&](int ix) -> int { return (ix + npml - 1) * ldz + rowoff; };
    auto load_pair = [&](const float* __restrict__ p, int o, float& v0, float& v1) {
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
        const int o = colbase(ix);
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
        const int o = colbase(ix);
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

    // accumulator chains (index 0 = oldest), [row]
    float SA[NS][2], SB[NS][2];      // staggered d/dx of ux, uz
    float D2[ND][2], D3[ND][2];      // collocated d/dx of uz, ux
    float FX[NF][2], FZ[NF][2];      // forces
#pragma unroll
    for (int i = 0; i < NS; ++i) SA[i][0] = SA[i][1] = SB[i][0] = SB[i][1] = 0.f;
#pragma unroll
    for (int i = 0; i < ND; ++i) D2[i][0] = D2[i][1] = D3[i][0] = D3[i][1] = 0.f;
#pragma unroll
    for (int i = 0; i < NF; ++i) FX[i][0] = FX[i][1] = FZ[i][0] = FZ[i][1] = 0.f;

    // reciprocals of l2m and mu at the lagged column m-NO (left of the emitted half point)
    float rlp0 = 1.f, rlp1 = 1.f, rmp0 = 1.f, rmp1 = 1.f;
    // lam, mu at the lagged column m-NO (for the dxz operands)
    float lp0 = 0.f, lp1 = 0.f, mp0 = 1.f, mp1 = 1.f;

    const int m0 = xs - 2 * NO + 1;            // first march column
    const int m1 = xe + LAG;                    // last march column
    // one-step-ahead fetches
    float pux0, pux1, puz0, puz1, pl0, pl1, pm0, pm1, ql0, ql1, qm0, qm1;
    load_u(m0, pux0, pux1, puz0, puz1);
    load_mat(m0, pl0, pl1, pm0, pm1);
    load_mat(m0 - NO + 1, ql0, ql1, qm0, qm1);
    {
        float l0, l1, mm0, mm1;
        load_mat(m0 - NO, l0, l1, mm0, mm1);
        lp0 = l0; lp1 = l1; mp0 = mm0; mp1 = mm1;
        rlp0 = frcp(l0 + 2.0f * mm0); rlp1 = frcp(l1 + 2.0f * mm1);
        rmp0 = frcp(mm0); rmp1 = frcp(mm1);
    }

    for (int mc = m0; mc <= m1; ++mc) {
        // this column's data (fetched last step) and the next column's fetches
        const float ux0 = pux0, ux1 = pux1, uz0 = puz0, uz1 = puz1;
        const float ln0 = pl0, ln1 = pl1, mn0 = pm0, mn1 = pm1;      // material at mc
        const float lq0 = ql0, lq1 = ql1, mq0 = qm0, mq1 = qm1;      // material at mc-NO+1
        load_u(mc + 1, pux0, pux1, puz0, puz1);
        load_mat(mc + 1, pl0, pl1, pm0, pm1);
        load_mat(mc + 2 - NO, ql0, ql1, qm0, qm1);
        const int xc = mc - LAG;                 // cell completed this step
        const bool emit = xc >= xs;
        float2 k2 = make_float2(0.f, 0.f), xo = k2, zo = k2, xp = k2, zp = k2;
        const int oc = colbase(xc);
        if (emit) {
            if (store1) {
                k2 = __ldg(reinterpret_cast<const float2*>(a.kdt2 + oc));
                xo = __ldg(reinterpret_cast<const float2*>(uxc + oc));
                zo = __ldg(reinterpret_cast<const float2*>(uzc + oc));
                xp = *reinterpret_cast<const float2*>(uxn + oc);
                zp = *reinterpret_cast<const float2*>(uzn + oc);
            } else if (store) {
                k2.x = __ldg(a.kdt2 + oc);
                xo.x = __ldg(uxc + oc);
                zo.x = __ldg(uzc + oc);
                xp.x = uxn[oc];
                zp.x = uzn[oc];
            }
        }

        // --- x-staggered derivative: complete half point mc-NO+1/2, fold column mc into the chain
        float sa0 = fmaf(c_stag[NO][NO], ux0, SA[0][0]), sa1 = fmaf(c_stag[NO][NO], ux1, SA[0][1]);
        float sb0 = fmaf(c_stag[NO][NO], uz0, SB[0][0]), sb1 = fmaf(c_stag[NO][NO], uz1, SB[0][1]);
#pragma unroll
        for (int i = 0; i < NS - 1; ++i) {
            // slot i+1 is the half point mc-NO+1/2+(i+1); column mc enters it with +c_{NO-i-1}
            // (left of the point) or -c_{i+2-NO} (right of it)
            const int ip = i + 1;
            const float c = ip < NO ? c_stag[NO][NO - ip] : -c_stag[NO][ip - NO + 1];
            SA[i][0] = fmaf(c, ux0, SA[ip][0]); SA[i][1] = fmaf(c, ux1, SA[ip][1]);
            SB[i][0] = fmaf(c, uz0, SB[ip][0]); SB[i][1] = fmaf(c, uz1, SB[ip][1]);
        }
        SA[NS - 1][0] = 0.f; SA[NS - 1][1] = 0.f; SB[NS - 1][0] = 0.f; SB[NS - 1][1] = 0.f;

        // harmonic means at the completed half point (columns mc-NO | mc-NO+1)
        const float rlq0 = frcp(lq0 + 2.0f * mq0), rlq1 = frcp(lq1 + 2.0f * mq1);
        const float rmq0 = frcp(mq0), rmq1 = frcp(mq1);
        const float ga0 = 2.0f * frcp(rlp0 + rlq0) * sa0 * dx2, ga1 = 2.0f * frcp(rlp1 + rlq1) * sa1 * dx2;
        const float gb0 = 2.0f * frcp(rmp0 + rmq0) * sb0 * dx2, gb1 = 2.0f * frcp(rmp1 + rmq1) * sb1 * dx2;

        // --- x-collocated derivative: complete column mc-NO, fold column mc into the chain
        const float d20 = fmaf(c_coll[NO][NO], uz0, D2[0][0]), d21 = fmaf(c_coll[NO][NO], uz1, D2[0][1]);
        const float d30 = fmaf(c_coll[NO][NO], ux0, D3[0][0]), d31 = fmaf(c_coll[NO][NO], ux1, D3[0][1]);
#pragma unroll
        for (int j = 0; j < ND - 1; ++j) {
            // slot j+1 is column mc-NO+j+1: column mc enters with +c1_{NO-j-1} (left), -c1_{j+1-NO} (right)
            const int jp = j + 1;
            if (jp == NO) {
                D2[j][0] = D2[jp][0]; D2[j][1] = D2[jp][1];
                D3[j][0] = D3[jp][0]; D3[j][1] = D3[jp][1];
            } else {
                const float c = jp < NO ? c_coll[NO][NO - jp] : -c_coll[NO][jp - NO];
                D2[j][0] = fmaf(c, uz0, D2[jp][0]); D2[j][1] = fmaf(c, uz1, D2[jp][1]);
                D3[j][0] = fmaf(c, ux0, D3[jp][0]); D3[j][1] = fmaf(c, ux1, D3[jp][1]);
            }
        }
        D2[ND - 1][0] = 0.f; D2[ND - 1][1] = 0.f; D3[ND - 1][0] = 0.f; D3[ND - 1][1] = 0.f;

        // --- z-direction terms of column mc (cell chain slot LAG)
        float z2a0, z2a1, z2b0, z2b1;
        {
            float sza0, sza1, szb0, szb1;
            dz_stag<NO>(uz0, uz1, sza0, sza1);
            dz_stag<NO>(ux0, ux1, szb0, szb1);
            const float rl0 = frcp(ln0 + 2.0f * mn0), rl1 = frcp(ln1 + 2.0f * mn1);
            const float rm0 = frcp(mn0), rm1 = frcp(mn1);
            const float rl2 = zrow<2>(rl0, rl1), rm2 = zrow<2>(rm0, rm1);
            const float gzA0 = 2.0f * frcp(rl0 + rl1) * sza0, gzA1 = 2.0f * frcp(rl1 + rl2) * sza1;
            const float gzB0 = 2.0f * frcp(rm0 + rm1) * szb0, gzB1 = 2.0f * frcp(rm1 + rm2) * szb1;
            dz_half<NO>(gzA0, gzA1, z2a0, z2a1);
            dz_half<NO>(gzB0, gzB1, z2b0, z2b1);
        }
        // dzx operands of column mc: lam Dz uz / dz, mu Dz ux / dz
        float v10, v11, v40, v41;
        {
            float t0, t1, s0, s1;
            dz_coll<NO>(uz0, uz1, t0, t1);
            dz_coll<NO>(ux0, ux1, s0, s1);
            v10 = ln0 * t0 * rdz * rdx; v11 = ln1 * t1 * rdz * rdx;
            v40 = mn0 * s0 * rdz * rdx; v41 = mn1 * s1 * rdz * rdx;
        }
        // dxz of column mc-NO: Dz(mu Dx uz / dx) / dz, Dz(lam Dx ux / dx) / dz
        float xzm0, xzm1, xzl0, xzl1;
        dz_coll<NO>(mp0 * d20 * rdx, mp1 * d21 * rdx, xzm0, xzm1);
        dz_coll<NO>(lp0 * d30 * rdx, lp1 * d31 * rdx, xzl0, xzl1);

        // --- fold everything into the force chain (slot i = cell mc-LAG+i) and advance it by one
        // cell: slot 0 is complete and leaves the chain, slot i+1 moves to slot i (the move is the
        // destination of the first fused multiply-add of that slot).
        // staggered products at h = mc-NO+1/2 reach cells h -+ (k - 1/2): slots NO-k (+c_k), NO-1+k (-c_k)
        // dzx operands of column mc reach cells mc -+ k: slots LAG-k (+c1_k), LAG+k (-c1_k)
        float ex0 = 0.f, ex1 = 0.f, ez0 = 0.f, ez1 = 0.f;
#pragma unroll
        for (int i = 0; i < NF; ++i) {
            float fx0 = FX[i][0], fx1 = FX[i][1], fz0 = FZ[i][0], fz1 = FZ[i][1];
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                if (i == NO - k) {
                    fx0 = fmaf(c_stag[NO][k], ga0, fx0); fx1 = fmaf(c_stag[NO][k], ga1, fx1);
                    fz0 = fmaf(c_stag[NO][k], gb0, fz0); fz1 = fmaf(c_stag[NO][k], gb1, fz1);
                }
                if (i == NO - 1 + k) {
                    fx0 = fmaf(-c_stag[NO][k], ga0, fx0); fx1 = fmaf(-c_stag[NO][k], ga1, fx1);
                    fz0 = fmaf(-c_stag[NO][k], gb0, fz0); fz1 = fmaf(-c_stag[NO][k], gb1, fz1);
                }
                if (i == LAG - k) {
                    fx0 = fmaf(c_coll[NO][k], v10, fx0); fx1 = fmaf(c_coll[NO][k], v11, fx1);
                    fz0 = fmaf(c_coll[NO][k], v40, fz0); fz1 = fmaf(c_coll[NO][k], v41, fz1);
                }
                if (i == LAG + k) {
                    fx0 = fmaf(-c_coll[NO][k], v10, fx0); fx1 = fmaf(-c_coll[NO][k], v11, fx1);
                    fz0 = fmaf(-c_coll[NO][k], v40, fz0); fz1 = fmaf(-c_coll[NO][k], v41, fz1);
                }
            }
            if (i == LAG) {   // z terms of column mc
                fx0 = fmaf(z2b0, dz2, fx0); fx1 = fmaf(z2b1, dz2, fx1);
                fz0 = fmaf(z2a0, dz2, fz0); fz1 = fmaf(z2a1, dz2, fz1);
            }
            if (i == NO - 1) {  // dxz of column mc-NO
                fx0 = fmaf(xzm0, rdz, fx0); fx1 = fmaf(xzm1, rdz, fx1);
                fz0 = fmaf(xzl0, rdz, fz0); fz1 = fmaf(xzl1, rdz, fz1);
            }
            if (i == 0) {
                ex0 = fx0; ex1 = fx1; ez0 = fz0; ez1 = fz1;
            } else {
                FX[i - 1][0] = fx0; FX[i - 1][1] = fx1; FZ[i - 1][0] = fz0; FZ[i - 1][1] = fz1;
            }
        }
        FX[NF - 1][0] = FX[NF - 1][1] = FZ[NF - 1][0] = FZ[NF - 1][1] = 0.f;

        // cell xc is complete
        if (emit && store) {
            if (store1) {
                xp.x = fmaf(k2.x, ex0, 2.0f * xo.x - xp.x);
                xp.y = fmaf(k2.y, ex1, 2.0f * xo.y - xp.y);
                zp.x = fmaf(k2.x, ez0, 2.0f * zo.x - zp.x);
                zp.y = fmaf(k2.y, ez1, 2.0f * zo.y - zp.y);
                *reinterpret_cast<float2*>(uxn + oc) = xp;
                *reinterpret_cast<float2*>(uzn + oc) = zp;
            } else {
                uxn[oc] = fmaf(k2.x, ex0, 2.0f * xo.x - xp.x);
                uzn[oc] = fmaf(k2.x, ez0, 2.0f * zo.x - zp.x);
            }
        }

        // lagged material: column mc-NO+1 becomes the left neighbour of the next half point
        rlp0 = rlq0; rlp1 = rlq1; rmp0 = rmq0; rmp1 = rmq1;
        lp0 = lq0; lp1 = lq1; mp0 = mq0; mp1 = mq1;
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
