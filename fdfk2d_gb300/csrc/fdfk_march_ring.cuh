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
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 1; j <= NO; ++j) s = ffma2(c_stag[NO][j], make_float2(z(j) - z(1 - j), z(j + 1) - z(2 - j)), s);
    d0 = s.x;
    d1 = s.y;
}
template <int NO>
__device__ __forceinline__ void zc_coll(const ZCol<-NO, NO + 1>& z, float& d0, float& d1)
{
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 1; k <= NO; ++k) s = ffma2(c_coll[NO][k], make_float2(z(k) - z(-k), z(k + 1) - z(1 - k)), s);
    d0 = s.x;
    d1 = s.y;
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

    const int rowoff = r0 - a.zorg;   // even: r0 is odd and 1 - zorg is even
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

    float2 SA[NS], SB[NS], D2[ND], D3[ND], FX[NF], FZ[NF];
    const float2 zero2 = make_float2(0.f, 0.f);
#pragma unroll
    for (int i = 0; i < NS; ++i) SA[i] = SB[i] = zero2;
#pragma unroll
    for (int i = 0; i < ND; ++i) D2[i] = D3[i] = zero2;
#pragma unroll
    for (int i = 0; i < NF; ++i) FX[i] = FZ[i] = zero2;

    // lambda + 2 mu is formed with one rounding (2 mu is exact), as by a fused multiply-add
    const float2 two = make_float2(2.0f, 2.0f);
    float2 LP = rdA(c0, 2), MP = rdA(c0, 3);
    float2 RLP = frcp2(ffma2(two, MP, LP)), RMP = frcp2(MP);

    // two columns per trip: the values carried to the next column alternate registers instead of moving
#pragma unroll 2
    for (int mc = m0; mc <= m1; ++mc) {
        issue(mc + RG::kAhead);
        cp_wait<RG::kAhead>();                  // column mc has landed
        const float2 U = rdA(mc, 0), Z = rdA(mc, 1), LNv = rdA(mc, 2), MNv = rdA(mc, 3);
        const float2 LQv = rdA(mc - NO + 1, 2), MQv = rdA(mc - NO + 1, 3);
        const float ux0 = U.x, ux1 = U.y, uz0 = Z.x, uz1 = Z.y;
        const int xc = mc - LAG;
        const bool emit = xc >= xs;

        // --- x-staggered derivative (both rows of the lane in one packed FMA)
        const float2 sa = ffma2(c_stag[NO][NO], U, SA[0]), sb = ffma2(c_stag[NO][NO], Z, SB[0]);
#pragma unroll
        for (int i = 0; i < NS - 1; ++i) {
            const int ip = i + 1;
            const float c = ip < NO ? c_stag[NO][NO - ip] : -c_stag[NO][ip - NO + 1];
            SA[i] = ffma2(c, U, SA[ip]);
            SB[i] = ffma2(c, Z, SB[ip]);
        }
        SA[NS - 1] = SB[NS - 1] = zero2;

        const float2 RLQ = frcp2(ffma2(two, MQv, LQv)), RMQ = frcp2(MQv);
        const float2 ga = fmul2(fmul2(fmul2(two, frcp2(fadd2(RLP, RLQ))), sa), dx2);
        const float2 gb = fmul2(fmul2(fmul2(two, frcp2(fadd2(RMP, RMQ))), sb), dx2);

        // --- x-collocated derivative
        const float2 d2 = ffma2(c_coll[NO][NO], Z, D2[0]), d3 = ffma2(c_coll[NO][NO], U, D3[0]);
#pragma unroll
        for (int j = 0; j < ND - 1; ++j) {
            const int jp = j + 1;
            if (jp == NO) {
                D2[j] = D2[jp];
                D3[j] = D3[jp];
            } else {
                const float c = jp < NO ? c_coll[NO][NO - jp] : -c_coll[NO][jp - NO];
                D2[j] = ffma2(c, Z, D2[jp]);
                D3[j] = ffma2(c, U, D3[jp]);
            }
        }
        D2[ND - 1] = D3[ND - 1] = zero2;

        // --- z-direction terms of column mc (one shuffled column per field for every z-stencil)
        const ZCol<-NO, NO + 1> zz(uz0, uz1), zx(ux0, ux1);
        float z2a0, z2a1, z2b0, z2b1;
        {
            float sza0, sza1, szb0, szb1;
            zc_stag<NO>(zz, sza0, sza1);
            zc_stag<NO>(zx, szb0, szb1);
            const float2 RL = frcp2(ffma2(two, MNv, LNv)), RM = frcp2(MNv);
            const float rl2 = zrow<2>(RL.x, RL.y), rm2 = zrow<2>(RM.x, RM.y);
            const float2 gzA = fmul2(fmul2(two, frcp2(fadd2(RL, make_float2(RL.y, rl2)))), make_float2(sza0, sza1));
            const float2 gzB = fmul2(fmul2(two, frcp2(fadd2(RM, make_float2(RM.y, rm2)))), make_float2(szb0, szb1));
            dz_half<NO>(gzA.x, gzA.y, z2a0, z2a1);
            dz_half<NO>(gzB.x, gzB.y, z2b0, z2b1);
        }
        float2 v1, v4;
        {
            float t0, t1, s0, s1;
            zc_coll<NO>(zz, t0, t1);
            zc_coll<NO>(zx, s0, s1);
            v1 = fmul2(fmul2(fmul2(LNv, make_float2(t0, t1)), rdz), rdx);
            v4 = fmul2(fmul2(fmul2(MNv, make_float2(s0, s1)), rdz), rdx);
        }
        float xzm0, xzm1, xzl0, xzl1;
        const float2 am = fmul2(fmul2(MP, d2), rdx), al = fmul2(fmul2(LP, d3), rdx);
        dz_coll<NO>(am.x, am.y, xzm0, xzm1);
        dz_coll<NO>(al.x, al.y, xzl0, xzl1);
        const float2 z2a = make_float2(z2a0, z2a1), z2b = make_float2(z2b0, z2b1);
        const float2 xzm = make_float2(xzm0, xzm1), xzl = make_float2(xzl0, xzl1);

        // --- force chain
        float2 ex = zero2, ez = zero2;
#pragma unroll
        for (int i = 0; i < NF; ++i) {
            float2 fx = FX[i], fz = FZ[i];
#pragma unroll
            for (int k = 1; k <= NO; ++k) {
                if (i == NO - k) {
                    fx = ffma2(c_stag[NO][k], ga, fx);
                    fz = ffma2(c_stag[NO][k], gb, fz);
                }
                if (i == NO - 1 + k) {
                    fx = ffma2(-c_stag[NO][k], ga, fx);
                    fz = ffma2(-c_stag[NO][k], gb, fz);
                }
                if (i == LAG - k) {
                    fx = ffma2(c_coll[NO][k], v1, fx);
                    fz = ffma2(c_coll[NO][k], v4, fz);
                }
                if (i == LAG + k) {
                    fx = ffma2(-c_coll[NO][k], v1, fx);
                    fz = ffma2(-c_coll[NO][k], v4, fz);
                }
            }
            if (i == LAG) {
                fx = ffma2(z2b, make_float2(dz2, dz2), fx);
                fz = ffma2(z2a, make_float2(dz2, dz2), fz);
            }
            if (i == NO - 1) {
                fx = ffma2(xzm, make_float2(rdz, rdz), fx);
                fz = ffma2(xzl, make_float2(rdz, rdz), fz);
            }
            if (i == 0) {
                ex = fx; ez = fz;
            } else {
                FX[i - 1] = fx; FZ[i - 1] = fz;
            }
        }
        FX[NF - 1] = FZ[NF - 1] = zero2;

        // cell xc is complete
        if (emit && store) {
            const float2 k2 = rdB(mc, 0), xp = rdB(mc, 1), zp = rdB(mc, 2);
            const float2 xo = rdA(xc, 0), zo = rdA(xc, 1);
            // 2 u^n - u^{n-1} is exact before its rounding, so one FMA gives it
            const float2 nxv = ffma2(k2, ex, ffma2(two, xo, make_float2(-xp.x, -xp.y)));
            const float2 nzv = ffma2(k2, ez, ffma2(two, zo, make_float2(-zp.x, -zp.y)));
            const int oc = gofs(xc);
            if (store1) {
                *reinterpret_cast<float2*>(uxn + oc) = nxv;
                *reinterpret_cast<float2*>(uzn + oc) = nzv;
            } else {
                uxn[oc] = nxv.x;
                uzn[oc] = nzv.x;
            }
        }

        RLP = RLQ; RMP = RMQ;
        LP = LQv; MP = MQv;
    }
    cp_wait<0>();
}
