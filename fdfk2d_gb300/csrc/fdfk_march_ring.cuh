// The march of one warp, fed by asynchronous copies (included inside
// namespace fdfk::march by fdfk_march.cuh).
//
// Each lane copies its own two rows of every field with cp.async into a
// per-warp shared-memory ring, kAhead columns before they are used, so the
// DRAM latency is covered by the march itself instead of by registers.
//   ring A: ux, uz, lambda, mu of columns mc - (2NO-1) .. mc + kAhead (the
//           newest column, the lagged material column mc-NO+1 and the
//           emitted cell's u^n all come from here);
//   ring B: dt^2/rho and u^{n-1} of the cell emitted kAhead columns later.
// A lane only reads back what it copied itself, so cp.async.wait_group is the
// only synchronisation (no barrier, no spin loop).
//
// Every warp runs the same code.  Outside the regular domain (columns outside
// 1..nx, rows from nz down) u is read from the step's frame (StepArgs::fux,
// fuz: u^n with the Omega_II background already added, written by
// fdfk_frame_kernel); rows past NZ are padding rows of the planes (u = 0,
// lambda = 0, mu = 1); material columns left of the grid (npml < 3NO-1 only)
// are written into the ring as those constants.
template <int NO>
struct Ring {
    static constexpr int kAhead = 2;                            // columns fetched ahead of use
    static constexpr int kNeedA = kAhead + 2 * NO;              // ring-A columns live at once
    static constexpr int kSlotsA = kNeedA <= 4 ? 4 : kNeedA <= 8 ? 8 : 16;
    static constexpr int kSlotsB = 4;                           // >= kAhead + 1
    static constexpr int kFieldsA = 4;
    static constexpr int kFieldsB = 3;
    static constexpr int kWarpFloats = 64 * (kSlotsA * kFieldsA + kSlotsB * kFieldsB);
};

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ void st_shared2(float* smem, float v0, float v1)
{
    *reinterpret_cast<float2*>(smem) = make_float2(v0, v1);
}

// cp.async into a 32-bit shared-space address plus an immediate byte offset.
template <int OFF>
__device__ __forceinline__ void cp_async8_s(unsigned s, const float* g)
{
    asm volatile("cp.async.ca.shared.global [%0+%2], [%1], 8;\n" ::"r"(s), "l"(g), "n"(OFF) : "memory");
}
template <int OFF>
__device__ __forceinline__ void cp_async4_s(unsigned s, const float* g)
{
    asm volatile("cp.async.ca.shared.global [%0+%2], [%1], 4;\n" ::"r"(s), "l"(g), "n"(OFF) : "memory");
}
// z-derivatives of one shuffled column (rows r0-NO .. r0+NO+1), shared by the staggered and
// the collocated stencils of the same field.
template <int NO>
__device__ __forceinline__ void zc_stag(const ZCol<-NO, NO + 1>& z, float& d0, float& d1)
{
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int j = 1; j <= NO; ++j) {
        s0 = fmaf(c_stag[NO][j], z(j) - z(1 - j), s0);
        s1 = fmaf(c_stag[NO][j], z(j + 1) - z(2 - j), s1);
    }
    d0 = s0;
    d1 = s1;
}
template <int NO>
__device__ __forceinline__ void zc_coll(const ZCol<-NO, NO + 1>& z, float& d0, float& d1)
{
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int k = 1; k <= NO; ++k) {
        s0 = fmaf(c_coll[NO][k], z(k) - z(-k), s0);
        s1 = fmaf(c_coll[NO][k], z(k + 1) - z(1 - k), s1);
    }
    d0 = s0;
    d1 = s1;
}

template <int NO>
__device__ __forceinline__ void march_ring(const StepArgs& a, const MarchArgs& m, int lane, int b, int xs, int xe,
                                           float* ring)
{
    using RG = Ring<NO>;
    constexpr int NS = 2 * NO;       // staggered partial sums
    constexpr int ND = 2 * NO + 1;   // collocated partial sums
    constexpr int NF = 3 * NO;       // force accumulators
    constexpr int LAG = 2 * NO - 1;  // newest column minus completed cell

    const int r0 = b + 2 * lane;
    const int nx = a.nx, nz = a.nz, npml = a.npml, ldz = a.ldz;
    const bool store = lane >= NO && lane <= 31 - NO && r0 >= m.z0 && r0 <= nz;
    const bool store1 = store && r0 + 1 <= nz;
    const bool lane_frame = r0 + 1 > nz;       // both rows from the frame (row nz is copied there)

    const float* __restrict__ uxc = a.ux[a.cur];
    const float* __restrict__ uzc = a.uz[a.cur];
    float* __restrict__ uxn = a.ux[a.cur ^ 1];
    float* __restrict__ uzn = a.uz[a.cur ^ 1];
    const float* const uxl = lane_frame ? a.fux : uxc;    // u source of this lane inside columns 1..nx
    const float* const uzl = lane_frame ? a.fuz : uzc;
    const float rdx = 1.0f / a.dx, rdz = 1.0f / a.dz;
    const float dx2 = a.dx2r, dz2 = a.dz2;

    const int rowoff = r0 - 1;
    auto gofs = [&](int ix) -> int { return (ix + npml - 1) * ldz + rowoff; };
    float* const ringA = ring + 2 * lane;
    float* const ringB = ring + 64 * RG::kSlotsA * RG::kFieldsA + 2 * lane;
    auto slotA = [&](int col, int f) -> float* { return ringA + ((col & (RG::kSlotsA - 1)) * RG::kFieldsA + f) * 64; };
    auto slotB = [&](int col, int f) -> float* { return ringB + ((col & (RG::kSlotsB - 1)) * RG::kFieldsB + f) * 64; };
    // shared-space byte addresses of this lane's pair in field 0 of a column's slot
    const unsigned sA0 = (unsigned)__cvta_generic_to_shared(ringA), sB0 = (unsigned)__cvta_generic_to_shared(ringB);
    constexpr int kFA = 64 * 4, kFB = 64 * 4;                       // bytes between fields of a slot
    auto sA = [&](int col) -> unsigned { return sA0 + (unsigned)((col & (RG::kSlotsA - 1)) * RG::kFieldsA * kFA); };
    auto sB = [&](int col) -> unsigned { return sB0 + (unsigned)((col & (RG::kSlotsB - 1)) * RG::kFieldsB * kFB); };
    auto rdA = [&](int col, int f) -> float2 { return *reinterpret_cast<const float2*>(slotA(col, f)); };
    auto rdB = [&](int col, int f) -> float2 { return *reinterpret_cast<const float2*>(slotB(col, f)); };

    const int m0 = xs - 2 * NO + 1;            // first march column
    const int m1 = xe + LAG;                    // last march column
    const int c0 = m0 - NO;                     // first column whose material is needed
    // one commit group per column; ring B of column col holds the cell col - LAG
    auto issue = [&](int col) {
        if (col <= m1) {
            if (col < 1 - npml) {               // left of the grid (only the lagged material is used)
                st_shared2(slotA(col, 0), 0.f, 0.f);
                st_shared2(slotA(col, 1), 0.f, 0.f);
                st_shared2(slotA(col, 2), 0.f, 0.f);
                st_shared2(slotA(col, 3), 1.f, 1.f);
            } else {
                const int o = gofs(col);
                const bool fr = col < 1 || col > nx;
                const unsigned sa = sA(col);
                cp_async8_s<0 * kFA>(sa, (fr ? a.fux : uxl) + o);
                cp_async8_s<1 * kFA>(sa, (fr ? a.fuz : uzl) + o);
                cp_async8_s<2 * kFA>(sa, a.lam + o);
                cp_async8_s<3 * kFA>(sa, a.mu + o);
            }
            const int xcol = col - LAG;
            if (store && xcol >= xs) {
                const int oc = gofs(xcol);
                const unsigned sb = sB(col);
                if (store1) {
                    cp_async8_s<0 * kFB>(sb, a.kdt2 + oc);
                    cp_async8_s<1 * kFB>(sb, uxn + oc);
                    cp_async8_s<2 * kFB>(sb, uzn + oc);
                } else {   // only row r0 (= nz) is stored
                    cp_async4_s<0 * kFB>(sb, a.kdt2 + oc);
                    cp_async4_s<1 * kFB>(sb, uxn + oc);
                    cp_async4_s<2 * kFB>(sb, uzn + oc);
                    slotB(col, 0)[1] = 0.f; slotB(col, 1)[1] = 0.f; slotB(col, 2)[1] = 0.f;
                }
            }
        }
        cp_commit();
    };
    for (int c = c0; c < m0 + RG::kAhead; ++c) issue(c);
    cp_wait<RG::kAhead>();                      // columns c0 .. m0-1 have landed

    float SA[NS][2], SB[NS][2];
    float D2[ND][2], D3[ND][2];
    float FX[NF][2], FZ[NF][2];
#pragma unroll
    for (int i = 0; i < NS; ++i) SA[i][0] = SA[i][1] = SB[i][0] = SB[i][1] = 0.f;
#pragma unroll
    for (int i = 0; i < ND; ++i) D2[i][0] = D2[i][1] = D3[i][0] = D3[i][1] = 0.f;
#pragma unroll
    for (int i = 0; i < NF; ++i) FX[i][0] = FX[i][1] = FZ[i][0] = FZ[i][1] = 0.f;

    float lp0, lp1, mp0, mp1, rlp0, rlp1, rmp0, rmp1;
    {
        const float2 l = rdA(c0, 2), mm = rdA(c0, 3);
        lp0 = l.x; lp1 = l.y; mp0 = mm.x; mp1 = mm.y;
        rlp0 = frcp(lp0 + 2.0f * mp0); rlp1 = frcp(lp1 + 2.0f * mp1);
        rmp0 = frcp(mp0); rmp1 = frcp(mp1);
    }

    for (int mc = m0; mc <= m1; ++mc) {
        issue(mc + RG::kAhead);
        cp_wait<RG::kAhead>();                  // column mc has landed
        const float2 U = rdA(mc, 0), Z = rdA(mc, 1), LNv = rdA(mc, 2), MNv = rdA(mc, 3);
        const float2 LQv = rdA(mc - NO + 1, 2), MQv = rdA(mc - NO + 1, 3);
        const float ux0 = U.x, ux1 = U.y, uz0 = Z.x, uz1 = Z.y;
        const float ln0 = LNv.x, ln1 = LNv.y, mn0 = MNv.x, mn1 = MNv.y;
        const float lq0 = LQv.x, lq1 = LQv.y, mq0 = MQv.x, mq1 = MQv.y;
        const int xc = mc - LAG;
        const bool emit = xc >= xs;

        // --- x-staggered derivative
        float sa0 = fmaf(c_stag[NO][NO], ux0, SA[0][0]), sa1 = fmaf(c_stag[NO][NO], ux1, SA[0][1]);
        float sb0 = fmaf(c_stag[NO][NO], uz0, SB[0][0]), sb1 = fmaf(c_stag[NO][NO], uz1, SB[0][1]);
#pragma unroll
        for (int i = 0; i < NS - 1; ++i) {
            const int ip = i + 1;
            const float c = ip < NO ? c_stag[NO][NO - ip] : -c_stag[NO][ip - NO + 1];
            SA[i][0] = fmaf(c, ux0, SA[ip][0]); SA[i][1] = fmaf(c, ux1, SA[ip][1]);
            SB[i][0] = fmaf(c, uz0, SB[ip][0]); SB[i][1] = fmaf(c, uz1, SB[ip][1]);
        }
        SA[NS - 1][0] = 0.f; SA[NS - 1][1] = 0.f; SB[NS - 1][0] = 0.f; SB[NS - 1][1] = 0.f;

        const float rlq0 = frcp(lq0 + 2.0f * mq0), rlq1 = frcp(lq1 + 2.0f * mq1);
        const float rmq0 = frcp(mq0), rmq1 = frcp(mq1);
        const float ga0 = 2.0f * frcp(rlp0 + rlq0) * sa0 * dx2, ga1 = 2.0f * frcp(rlp1 + rlq1) * sa1 * dx2;
        const float gb0 = 2.0f * frcp(rmp0 + rmq0) * sb0 * dx2, gb1 = 2.0f * frcp(rmp1 + rmq1) * sb1 * dx2;

        // --- x-collocated derivative
        const float d20 = fmaf(c_coll[NO][NO], uz0, D2[0][0]), d21 = fmaf(c_coll[NO][NO], uz1, D2[0][1]);
        const float d30 = fmaf(c_coll[NO][NO], ux0, D3[0][0]), d31 = fmaf(c_coll[NO][NO], ux1, D3[0][1]);
#pragma unroll
        for (int j = 0; j < ND - 1; ++j) {
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

        // --- z-direction terms of column mc (one shuffled column per field for every z-stencil)
        const ZCol<-NO, NO + 1> zz(uz0, uz1), zx(ux0, ux1);
        float z2a0, z2a1, z2b0, z2b1;
        {
            float sza0, sza1, szb0, szb1;
            zc_stag<NO>(zz, sza0, sza1);
            zc_stag<NO>(zx, szb0, szb1);
            const float rl0 = frcp(ln0 + 2.0f * mn0), rl1 = frcp(ln1 + 2.0f * mn1);
            const float rm0 = frcp(mn0), rm1 = frcp(mn1);
            const float rl2 = zrow<2>(rl0, rl1), rm2 = zrow<2>(rm0, rm1);
            const float gzA0 = 2.0f * frcp(rl0 + rl1) * sza0, gzA1 = 2.0f * frcp(rl1 + rl2) * sza1;
            const float gzB0 = 2.0f * frcp(rm0 + rm1) * szb0, gzB1 = 2.0f * frcp(rm1 + rm2) * szb1;
            dz_half<NO>(gzA0, gzA1, z2a0, z2a1);
            dz_half<NO>(gzB0, gzB1, z2b0, z2b1);
        }
        float v10, v11, v40, v41;
        {
            float t0, t1, s0, s1;
            zc_coll<NO>(zz, t0, t1);
            zc_coll<NO>(zx, s0, s1);
            v10 = ln0 * t0 * rdz * rdx; v11 = ln1 * t1 * rdz * rdx;
            v40 = mn0 * s0 * rdz * rdx; v41 = mn1 * s1 * rdz * rdx;
        }
        float xzm0, xzm1, xzl0, xzl1;
        dz_coll<NO>(mp0 * d20 * rdx, mp1 * d21 * rdx, xzm0, xzm1);
        dz_coll<NO>(lp0 * d30 * rdx, lp1 * d31 * rdx, xzl0, xzl1);

        // --- force chain
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
            if (i == LAG) {
                fx0 = fmaf(z2b0, dz2, fx0); fx1 = fmaf(z2b1, dz2, fx1);
                fz0 = fmaf(z2a0, dz2, fz0); fz1 = fmaf(z2a1, dz2, fz1);
            }
            if (i == NO - 1) {
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
            const float2 k2 = rdB(mc, 0), xp = rdB(mc, 1), zp = rdB(mc, 2);
            const float2 xo = rdA(xc, 0), zo = rdA(xc, 1);
            float2 nxv, nzv;
            nxv.x = fmaf(k2.x, ex0, 2.0f * xo.x - xp.x);
            nxv.y = fmaf(k2.y, ex1, 2.0f * xo.y - xp.y);
            nzv.x = fmaf(k2.x, ez0, 2.0f * zo.x - zp.x);
            nzv.y = fmaf(k2.y, ez1, 2.0f * zo.y - zp.y);
            const int oc = gofs(xc);
            if (store1) {
                *reinterpret_cast<float2*>(uxn + oc) = nxv;
                *reinterpret_cast<float2*>(uzn + oc) = nzv;
            } else {
                uxn[oc] = nxv.x;
                uzn[oc] = nzv.x;
            }
        }

        rlp0 = rlq0; rlp1 = rlq1; rmp0 = rmq0; rmp1 = rmq1;
        lp0 = lq0; lp1 = lq1; mp0 = mq0; mp1 = mq1;
    }
    cp_wait<0>();
}
