// FK background wavefield on the GPU (replaces libFK3D's comput_background_wavefield_, call
// site src/FDFK2D.f90:429-431).  Spectra and responses in FP64; the frequency-to-time transform
// in double-float (df64, about 48 bits) on the FP32 pipes.
//
// Pipeline (one stream):
//   1. host: per-layer vertical slownesses, wave-vector matrices E (ux, uz,
//      sigma_xz, sigma_zz per unit amplitude of down P, down S, up P, up S) and
//      interface matrices C_j = E_j^-1 E_{j+1}; the damped Ricker samples;
//   2. fk_source_dft: W_k, k <= kmax, direct DFT against an exact twiddle table (FP64);
//   3. fk_layer_amps: one thread per (model, frequency) propagates the 4x4
//      layer matrices from the half-space to the surface, solves the 2x2
//      free-surface system for the downgoing half-space amplitudes and writes
//      every layer's amplitudes (phase referenced at the layer top) (FP64);
//   4. fk_depth_response: U_R, U_Z per (model, grid row, frequency), FP64, stored as df64;
//   5. fk_column_phase: W_k times the horizontal phase per (column, frequency), FP64, stored
//      as df64; fk_df_twiddles: the df64 twiddle tables;
//   6. per batch of strip series: fk_transform forms each series' half spectrum, folds it into
//      the input of a half-length complex inverse transform whose output is the real series
//      itself, runs that transform in shared memory (Stockham radix 4, df64), scales by
//      exp(alpha t)/N and writes the series as float; fk_epilogue transposes the batch into the
//      strips (time slowest).
//
// Why df64: GB300's FP64 rate is a small fraction of its FP32 rate, and the transform is the
// bulk of the arithmetic.  Plain FP32 is not enough: the output is multiplied by exp(alpha t),
// up to e^10, so the transform's rounding must stay below about 1e-12 of the series' maximum;
// df64's ~2^-48 unit roundoff over log2(M) stages keeps the strips within FP32 rounding of the
// FP64 restatement.
#include "fdfk_df64.cuh"
#include "fdfk_fk.cuh"
#include "fdfk_gb300.h"
#include "fdfk_sweep.cuh"

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace fdfk {

namespace {

constexpr double kPi = 3.14159265358979323846;

struct cd {
    double x, y;
};

__host__ __device__ __forceinline__ cd mk(double x, double y)
{
    cd r;
    r.x = x;
    r.y = y;
    return r;
}
__device__ __forceinline__ cd cmul(cd a, cd b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ cd cadd(cd a, cd b) { return mk(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ cd cexp_(cd z)
{
    double s, c;
    sincos(z.y, &s, &c);
    const double e = exp(z.x);
    return mk(e * c, e * s);
}
// i * (w - i alpha) * z * h
__device__ __forceinline__ cd i_wc_mul(double w, double alpha, cd z, double h)
{
    const double re = w * z.x + alpha * z.y;   // (w - i alpha) z
    const double im = w * z.y - alpha * z.x;
    return mk(-im * h, re * h);
}
// a / b (Smith's scaling)
__device__ __forceinline__ cd cdiv(cd a, cd b)
{
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, d = b.x + b.y * r;
        return mk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    const double r = b.x / b.y, d = b.y + b.x * r;
    return mk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}

struct FkLayer {
    double zt, h;    // top depth, thickness (0 for the half-space)
    cd sz[4];        // vertical slowness of down P, down S, up P, up S
    cd E[4][4];      // E[r][q]: component r (ux, uz, sxz, szz) of wave q per unit amplitude
    cd C[4][4];      // E_j^-1 E_{j+1}
};

struct FkGeom {
    int K;           // kmax + 1 frequencies carried
    int N;           // transform length
    int nh;          // N / 2
    double dw;       // 2 pi / (N dt)
    double alpha;
};

// Strip series table: series g (all strips, strip-major, point index q = i + n1 j).
struct SeriesTab {
    long long off[NSTRIP + 1];
    int n1[NSTRIP];
    int iz0[NSTRIP], ix0[NSTRIP];
    int model_side[NSTRIP];   // 0 left, 1 right, 2 bottom
    int nx, nbd, nrow;
    int bottom_pos;           // cos(baz_mean) >= 0
    float* dst[NSTRIP];
    long long per[NSTRIP];    // elements per time sample
};

struct SeriesPos {
    int s, iz, ix, model;
    long long q;
};

__device__ __forceinline__ SeriesPos decode(const SeriesTab& t, long long g)
{
    SeriesPos r;
    int s = 0;
#pragma unroll 1
    while (s < NSTRIP - 1 && g >= t.off[s + 1]) ++s;
    r.s = s;
    r.q = g - t.off[s];
    const int i = (int)(r.q % t.n1[s]);
    const int j = (int)(r.q / t.n1[s]);
    r.iz = t.iz0[s] + i;
    r.ix = t.ix0[s] + j;
    const int side = t.model_side[s];
    if (side < 2)
        r.model = side;
    else if (t.bottom_pos)
        r.model = r.ix <= t.nbd ? 0 : 1;
    else
        r.model = r.ix <= t.nx - t.nbd ? 0 : 1;
    return r;
}

__global__ void fk_twiddle(int N, cd* __restrict__ tw)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= N) return;
    double s, c;
    sincospi(2.0 * (double)m / (double)N, &s, &c);
    tw[m] = mk(c, -s);   // exp(-2 pi i m / N)
}

// W_k = sum_n w_n exp(-2 pi i k n / N), one block per k.
__global__ void fk_source_dft(int nt, int N, const double* __restrict__ w, const cd* __restrict__ tw,
                              cd* __restrict__ W)
{
    const int k = blockIdx.x;
    double re = 0.0, im = 0.0;
    for (int n = threadIdx.x; n <= nt; n += blockDim.x) {
        const cd t = tw[(int)(((long long)k * n) & (N - 1))];
        re += w[n] * t.x;
        im += w[n] * t.y;
    }
    __shared__ double sr[32], si[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sr[wid] = re;
        si[wid] = im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            a += sr[i];
            b += si[i];
        }
        W[k] = mk(a, b);
    }
}

// Layer amplitudes per (model, frequency): amps[m][(k * L + j) * 4 + q].
__global__ void fk_layer_amps(FkGeom g, const FkLayer* __restrict__ lay0, const FkLayer* __restrict__ lay1, int L0,
                              int L1, int inc, double inc_amp, double zref, cd* __restrict__ amp0,
                              cd* __restrict__ amp1)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * g.K) return;
    const int m = t / g.K, k = t - m * g.K;
    const FkLayer* Ly = m ? lay1 : lay0;
    const int L = m ? L1 : L0;
    cd* amp = m ? amp1 : amp0;
    const double w = g.dw * k, al = g.alpha;

    // G = T_0 T_1 ... T_{L-2}, T_j = diag(exp(i wc sz_q h_j)) C_j
    cd G[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) G[r][c] = mk(r == c ? 1.0 : 0.0, 0.0);
    for (int j = 0; j < L - 1; ++j) {
        cd e[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) e[q] = cexp_(i_wc_mul(w, al, Ly[j].sz[q], Ly[j].h));
        cd T[4][4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int c = 0; c < 4; ++c) T[q][c] = cmul(e[q], Ly[j].C[q][c]);
        cd Gn[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                cd acc = mk(0.0, 0.0);
#pragma unroll
                for (int q = 0; q < 4; ++q) acc = cadd(acc, cmul(G[r][q], T[q][c]));
                Gn[r][c] = acc;
            }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) G[r][c] = Gn[r][c];
    }
    // free surface at z = 0: rows 2, 3 of E_0 diag(exp(i wc sz_q zt_0)) G
    cd lam0[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) lam0[q] = cexp_(i_wc_mul(w, al, Ly[0].sz[q], Ly[0].zt));
    cd S[2][4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            cd acc = mk(0.0, 0.0);
#pragma unroll
            for (int q = 0; q < 4; ++q) acc = cadd(acc, cmul(cmul(Ly[0].E[r + 2][q], lam0[q]), G[q][c]));
            S[r][c] = acc;
        }
    // S[:, 0:2] d = -S[:, inc] * inc_amp
    const cd r0 = mk(-S[0][inc].x * inc_amp, -S[0][inc].y * inc_amp);
    const cd r1 = mk(-S[1][inc].x * inc_amp, -S[1][inc].y * inc_amp);
    const cd det = cadd(cmul(S[0][0], S[1][1]), mk(-(cmul(S[0][1], S[1][0])).x, -(cmul(S[0][1], S[1][0])).y));
    const cd n0 = cadd(cmul(r0, S[1][1]), mk(-(cmul(S[0][1], r1)).x, -(cmul(S[0][1], r1)).y));
    const cd n1 = cadd(cmul(S[0][0], r1), mk(-(cmul(S[1][0], r0)).x, -(cmul(S[1][0], r0)).y));
    cd a[4];
    a[0] = cdiv(n0, det);
    a[1] = cdiv(n1, det);
    a[2] = mk(inc == 2 ? inc_amp : 0.0, 0.0);
    a[3] = mk(inc == 3 ? inc_amp : 0.0, 0.0);
    // incident phase zero at zref: exp(-i wc sz_inc (zt_{L-1} - zref))
    const cd f = cexp_(i_wc_mul(w, al, Ly[L - 1].sz[inc], -(Ly[L - 1].zt - zref)));
    cd* out = amp + (size_t)k * L * 4;
#pragma unroll
    for (int q = 0; q < 4; ++q) out[(L - 1) * 4 + q] = cmul(a[q], f);
    for (int j = L - 2; j >= 0; --j) {
        cd e[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) e[q] = cexp_(i_wc_mul(w, al, Ly[j].sz[q], Ly[j].h));
        cd b[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            cd acc = mk(0.0, 0.0);
#pragma unroll
            for (int c = 0; c < 4; ++c) acc = cadd(acc, cmul(Ly[j].C[q][c], a[c]));
            b[q] = cmul(e[q], acc);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            a[q] = b[q];
            out[j * 4 + q] = cmul(b[q], f);
        }
    }
}

// U[(m * nrow + row) * K + k] = {U_R, U_Z} at z = z0 + row dz.
__global__ void fk_depth_response(FkGeom g, const FkLayer* __restrict__ lay0, const FkLayer* __restrict__ lay1,
                                  int L0, int L1, const cd* __restrict__ amp0, const cd* __restrict__ amp1, int nrow,
                                  double z0, double dz, float4* __restrict__ U)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = 2LL * nrow * g.K;
    if (t >= total) return;
    const int k = (int)(t % g.K);
    const long long mr = t / g.K;
    const int row = (int)(mr % nrow);
    const int m = (int)(mr / nrow);
    const FkLayer* Ly = m ? lay1 : lay0;
    const int L = m ? L1 : L0;
    const cd* amp = (m ? amp1 : amp0) + (size_t)k * L * 4;
    const double z = z0 + (double)row * dz;
    int j = 0;
    while (j + 1 < L && Ly[j + 1].zt <= z) ++j;
    const double d = z - Ly[j].zt;
    const double w = g.dw * k;
    cd ur = mk(0.0, 0.0), uz = mk(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const cd e = cmul(amp[j * 4 + q], cexp_(i_wc_mul(w, g.alpha, Ly[j].sz[q], -d)));
        ur = cadd(ur, cmul(e, Ly[j].E[0][q]));
        uz = cadd(uz, cmul(e, Ly[j].E[1][q]));
    }
    U[2 * t] = df64::from_double(ur.x, ur.y);
    U[2 * t + 1] = df64::from_double(uz.x, uz.y);
}

// Ph[c * K + k] = W_k exp(i wc_k D_c), D_c = p (cos(baz_c) (x_c' - x_centre) - r_ref).
__global__ void fk_column_phase(FkGeom g, int ncol, const double* __restrict__ D, const cd* __restrict__ W,
                                float4* __restrict__ Ph)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ncol * g.K) return;
    const int k = (int)(t % g.K);
    const int c = (int)(t / g.K);
    const double d = D[c];
    const cd e = cexp_(mk(g.alpha * d, g.dw * k * d));
    const cd v = cmul(W[k], e);
    Ph[t] = df64::from_double(v.x, v.y);
}

// df64 twiddle tables: twM[t] = exp(+2 pi i t / M), t < M (M = N / 2, the transform length) and
// twN[k] = exp(+2 pi i k / N), k < M (the fold's half-bin rotation).
__global__ void fk_df_twiddles(int M, float4* __restrict__ twM, float4* __restrict__ twN)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= M) return;
    double s, c;
    sincospi(2.0 * (double)t / (double)M, &s, &c);
    twM[t] = df64::from_double(c, s);
    sincospi((double)t / (double)M, &s, &c);
    twN[t] = df64::from_double(c, s);
}

// Bin j of the half spectrum of series p (df64): W_j * phase * U (times cos(baz) for the x
// component); zero from j = K on.
__device__ __forceinline__ df64::C series_bin(const FkGeom& g, const SeriesTab& tab, const SeriesPos& p, int j,
                                              const float4* __restrict__ U, const float4* __restrict__ Ph,
                                              const float2* __restrict__ cosd)
{
    if (j >= g.K) return df64::zero();
    const int c = p.ix - (1 - tab.nbd);
    const bool xcomp = (p.s & 1) == 0;
    const df64::C u = df64::unpack(__ldg(&U[(((size_t)p.model * tab.nrow + (p.iz - 1)) * g.K + j) * 2 + (xcomp ? 0 : 1)]));
    df64::C v = df64::cmul(df64::unpack(__ldg(&Ph[(size_t)c * g.K + j])), u);
    if (xcomp) {
        const float2 cp = __ldg(&cosd[c]);
        v = df64::cscale(v, cp.x, cp.y);
    }
    return v;
}

// Input of the half-length complex inverse transform that yields a real series: with M = N/2 and
// X the half spectrum (X_0 and X_M enter with their real parts, as for a real series),
//   Z_k = E_k + i O_k,  E_k = X_k + conj(X_{M-k}),  O_k = (X_k - conj(X_{M-k})) exp(+2 pi i k / N),
// sum_k Z_k exp(+2 pi i k m / M) = x[2m] + i x[2m+1], x the length-N real inverse transform of X.
__device__ __forceinline__ df64::C fold_bin(const df64::C& xk, const df64::C& xm, const float4& wN)
{
    const df64::C cm = df64::conj(xm);
    const df64::C e = df64::cadd(xk, cm);
    const df64::C o = df64::cmul(df64::csub(xk, cm), df64::unpack(wN));
    return df64::cadd(e, df64::times_i(o));
}

// Z_k of series p (k < M); zero unless k < K or M - k < K.
__device__ __forceinline__ df64::C fold_at(const FkGeom& g, const SeriesTab& tab, const SeriesPos& p, int k,
                                           const float4* __restrict__ U, const float4* __restrict__ Ph,
                                           const float2* __restrict__ cosd, const float4* __restrict__ twN)
{
    const int M = g.nh;
    df64::C xk = series_bin(g, tab, p, k, U, Ph, cosd);
    df64::C xm = k == 0 ? df64::zero() : series_bin(g, tab, p, M - k, U, Ph, cosd);
    if (k == 0) {
        xk.hi.y = 0.f;
        xk.lo.y = 0.f;
    }
    return fold_bin(xk, xm, __ldg(&twN[k]));
}

template <int Q>
struct TransformShape {
    static constexpr int kThreads = Q >= 512 ? Q / 16 : 32;
    static constexpr int kLog = Q <= 1 ? 0 : 1 + TransformShape<Q / 2>::kLog;
};
template <>
struct TransformShape<1> {
    static constexpr int kThreads = 32;
    static constexpr int kLog = 0;
};

// One Stockham stage of radix R (inverse sign) on the Q-point df64 sequence in shared memory, in
// place through registers: every thread reads all its butterflies' inputs, the block synchronises,
// then every thread writes its outputs.  Ns = product of the radices of the stages before.
// Twiddle w_{Ns R}^{kr} = w_M^{kr (Q / (Ns R)) P}.
template <int Q, int R>
__device__ __forceinline__ void stockham_stage(float4* sm, int Ns, int P, const float4* __restrict__ twM)
{
    constexpr int T = TransformShape<Q>::kThreads;
    constexpr int J = Q / R;                     // butterflies
    constexpr int BPT = (J + T - 1) / T;         // butterflies per thread
    df64::C v[BPT][R];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int j = threadIdx.x + t * T;
        if (j < J) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = df64::unpack(sm[j + r * J]);
        }
    }
    __syncthreads();
    const int step = Q / (Ns * R);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int j = threadIdx.x + t * T;
        if (j < J) {
            const int k = j & (Ns - 1);
            if (k != 0) {
#pragma unroll
                for (int r = 1; r < R; ++r)
                    v[t][r] = df64::cmul(v[t][r], df64::unpack(__ldg(&twM[(size_t)k * r * step * P])));
            }
            if constexpr (R == 2) {
                const df64::C a = v[t][0], b = v[t][1];
                v[t][0] = df64::cadd(a, b);
                v[t][1] = df64::csub(a, b);
            } else {
                // inverse 4-point DFT: X_q = sum_n v_n i^{nq}
                const df64::C a0 = df64::cadd(v[t][0], v[t][2]), a1 = df64::csub(v[t][0], v[t][2]);
                const df64::C a2 = df64::cadd(v[t][1], v[t][3]), a3 = df64::times_i(df64::csub(v[t][1], v[t][3]));
                v[t][0] = df64::cadd(a0, a2);
                v[t][2] = df64::csub(a0, a2);
                v[t][1] = df64::cadd(a1, a3);
                v[t][3] = df64::csub(a1, a3);
            }
            const int d = (j / Ns) * Ns * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) sm[d + r * Ns] = df64::pack(v[t][r]);
        }
    }
    __syncthreads();
}

// Series g0 + blockIdx.x, branch r = blockIdx.y of the M = P Q point inverse transform: with
// m = P m' + r (decimation in time of the output),
//   z_{P m' + r} = sum_{k' < Q} w_Q^{k' m'} [ w_M^{k' r} sum_{j < P} Z_{k' + Q j} w_P^{j r} ],
// a Q-point transform per branch.  Writes x[n] exp(alpha t_n) / N, n = 2m, 2m + 1 <= nt, as float
// into out[b * (nt + 1) + n].
template <int Q>
__global__ void __launch_bounds__(TransformShape<Q>::kThreads) fk_transform(
    FkGeom g, SeriesTab tab, long long g0, int P, int nt, const float4* __restrict__ U,
    const float4* __restrict__ Ph, const float2* __restrict__ cosd, const float4* __restrict__ twM,
    const float4* __restrict__ twN, const float2* __restrict__ escale, float* __restrict__ out)
{
    constexpr int T = TransformShape<Q>::kThreads;
    extern __shared__ float4 fk_sm[];
    __shared__ SeriesPos sp;
    const int b = blockIdx.x, r = blockIdx.y;
    if (threadIdx.x == 0) sp = decode(tab, g0 + b);
    __syncthreads();
    const SeriesPos p = sp;
    const int M = g.nh;
    if (P == 1) {
        // pairs (k, M - k): each spectral bin is formed once and feeds both folded bins
        for (int k = threadIdx.x; k <= M / 2; k += T) {
            if (k < g.K || M - k < g.K) {
                df64::C xk = series_bin(g, tab, p, k, U, Ph, cosd);
                df64::C xm = k == 0 ? df64::zero() : series_bin(g, tab, p, M - k, U, Ph, cosd);
                if (k == 0) {
                    xk.hi.y = 0.f;
                    xk.lo.y = 0.f;
                }
                fk_sm[k] = df64::pack(fold_bin(xk, xm, __ldg(&twN[k])));
                if (k > 0 && 2 * k < M) fk_sm[M - k] = df64::pack(fold_bin(xm, xk, __ldg(&twN[M - k])));
            } else {
                fk_sm[k] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (2 * k < M) fk_sm[M - k] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    } else {
        for (int kp = threadIdx.x; kp < Q; kp += T) {
            df64::C acc = df64::zero();
            for (int j = 0; j < P; ++j) {
                const int k = kp + Q * j;
                if (!(k < g.K || M - k < g.K)) continue;
                df64::C z = fold_at(g, tab, p, k, U, Ph, cosd, twN);
                const long long e = ((long long)j * r * Q) % M;          // w_P^{jr} = w_M^{jrQ}
                if (e) z = df64::cmul(z, df64::unpack(__ldg(&twM[e])));
                acc = df64::cadd(acc, z);
            }
            if (r && kp) acc = df64::cmul(acc, df64::unpack(__ldg(&twM[(size_t)kp * r])));
            fk_sm[kp] = df64::pack(acc);
        }
    }
    __syncthreads();
    int Ns = 1;
    if constexpr ((TransformShape<Q>::kLog & 1) != 0) {
        stockham_stage<Q, 2>(fk_sm, Ns, P, twM);
        Ns = 2;
    }
    if constexpr (Q >= 4) {
#pragma unroll 1
        for (; Ns < Q; Ns *= 4) stockham_stage<Q, 4>(fk_sm, Ns, P, twM);
    }
    float* const o = out + (size_t)b * (nt + 1);
    for (int mp = threadIdx.x; mp < Q; mp += T) {
        const long long n0 = 2LL * ((long long)P * mp + r);
        if (n0 > nt) continue;
        // x[n0] = Re z, x[n0+1] = Im z, each times its df64 scale exp(alpha t)/N (table padded to nt + 2);
        // the float nearest to the df64 product is the rounded sum of its two parts (no FP64 here: on
        // this GPU a few FP64 operations per output cost as much as the whole transform)
        const df64::C z = df64::unpack(fk_sm[mp]);
        const float2 e0 = __ldg(&escale[n0]), e1 = __ldg(&escale[n0 + 1]);
        const float2 eh = df64::f2(e0.x, e1.x), el = df64::f2(e0.y, e1.y);
        const float2 ph = df64::mul(z.hi, eh);
        float2 pe = df64::fma(z.hi, eh, df64::f2(-ph.x, -ph.y));
        pe = df64::fma(z.hi, el, pe);
        pe = df64::fma(z.lo, eh, pe);
        const float2 x = df64::add(ph, pe);
        o[n0] = x.x;
        if (n0 + 1 <= nt) o[n0 + 1] = x.y;
    }
}

// strips[s][q + per_s * n] = y[b][n], n = 0..nt; 32 x 32 tiles through shared memory.
__global__ void fk_epilogue(SeriesTab tab, long long g0, int nb, int nt, const float* __restrict__ y)
{
    __shared__ float tile[32][33];
    const int n0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int b = b0 + ty + 8 * r, n = n0 + tx;
        if (b < nb && n <= nt) tile[ty + 8 * r][tx] = y[(size_t)b * (nt + 1) + n];
    }
    __syncthreads();
    const int b = b0 + tx;
    if (b >= nb) return;
    const SeriesPos p = decode(tab, g0 + b);
    float* dst = tab.dst[p.s] + p.q;
    const long long per = tab.per[p.s];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int n = n0 + ty + 8 * r;
        if (n <= nt) dst[per * n] = tile[tx][ty + 8 * r];
    }
}

// Launches fk_transform for transform length Q (power of two, <= kMaxQ).
constexpr int kMaxQ = 4096;

template <int Q>
cudaError_t launch_transform_q(int q, dim3 grid, cudaStream_t st, const FkGeom& g, const SeriesTab& tab,
                               long long g0, int P, int nt, const float4* U, const float4* Ph, const float2* cosd,
                               const float4* twM, const float4* twN, const float2* esc, float* out)
{
    if constexpr (Q > 1) {
        if (q < Q) return launch_transform_q<Q / 2>(q, grid, st, g, tab, g0, P, nt, U, Ph, cosd, twM, twN, esc, out);
    }
    const size_t smem = sizeof(float4) * (size_t)Q;
    static bool configured = false;
    if (!configured) {
        const cudaError_t e =
            cudaFuncSetAttribute(fk_transform<Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    fk_transform<Q><<<grid, TransformShape<Q>::kThreads, smem, st>>>(g, tab, g0, P, nt, U, Ph, cosd, twM, twN, esc,
                                                                     out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- host side

using cplx = std::complex<double>;

bool invert4(const cplx A[4][4], cplx X[4][4])
{
    cplx M[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 8; ++c) M[r][c] = c < 4 ? A[r][c] : cplx(c - 4 == r ? 1.0 : 0.0, 0.0);
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::abs(M[r][c]) > std::abs(M[piv][c])) piv = r;
        if (std::abs(M[piv][c]) == 0.0) return false;
        if (piv != c)
            for (int k = 0; k < 8; ++k) std::swap(M[c][k], M[piv][k]);
        const cplx d = M[c][c];
        for (int k = 0; k < 8; ++k) M[c][k] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const cplx f = M[r][c];
            if (f == 0.0) continue;
            for (int k = 0; k < 8; ++k) M[r][k] -= f * M[c][k];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) X[r][c] = M[r][c + 4];
    return true;
}

// Wave vectors of one layer (same polarisation and stress normalisation as the
// restated response): fields vary as exp(i w (t + sx x - sz z)), sx = -p.
void layer_waves(double vp, double vs, double rho, double sx, cplx sz[4], cplx E[4][4])
{
    const cplx eta = std::sqrt(cplx(1.0 / (vp * vp) - sx * sx, 0.0));
    const cplx nu = std::sqrt(cplx(1.0 / (vs * vs) - sx * sx, 0.0));
    const double mu = rho * vs * vs, lam = rho * vp * vp - 2.0 * mu;
    const cplx pol[4][2] = {{sx * vp, eta * vp}, {nu * vs, -sx * vs}, {sx * vp, -eta * vp}, {nu * vs, sx * vs}};
    const cplx s[4] = {eta, nu, -eta, -nu};
    for (int q = 0; q < 4; ++q) {
        sz[q] = s[q];
        E[0][q] = pol[q][0];
        E[1][q] = pol[q][1];
        E[2][q] = mu * (s[q] * pol[q][0] + sx * pol[q][1]);
        E[3][q] = lam * sx * pol[q][0] + (lam + 2.0 * mu) * s[q] * pol[q][1];
    }
}

int build_layers(const float* model, int L, double rayp, std::vector<FkLayer>& out, std::string& err)
{
    out.assign(L, FkLayer{});
    std::vector<std::array<std::array<cplx, 4>, 4>> E(L);
    std::vector<std::array<cplx, 4>> S(L);
    for (int j = 0; j < L; ++j) {
        const double zt = model[4 * j], vp = model[4 * j + 1], vs = model[4 * j + 2], rho = model[4 * j + 3];
        if (!(vp > 0.0) || !(vs > 0.0) || !(rho > 0.0)) {
            err = "FK model layer " + std::to_string(j + 1) + ": vp, vs and rho must be positive";
            return FDFK_EINVAL;
        }
        if (j > 0 && !(zt > (double)model[4 * (j - 1)])) {
            err = "FK model layer tops must increase with depth";
            return FDFK_EINVAL;
        }
        cplx sz[4], e[4][4];
        layer_waves(vp, vs, rho, -rayp, sz, e);
        for (int q = 0; q < 4; ++q) {
            S[j][q] = sz[q];
            for (int r = 0; r < 4; ++r) E[j][r][q] = e[r][q];
        }
        out[j].zt = zt;
        out[j].h = j + 1 < L ? (double)model[4 * (j + 1)] - zt : 0.0;
        for (int q = 0; q < 4; ++q) out[j].sz[q] = mk(sz[q].real(), sz[q].imag());
        for (int r = 0; r < 4; ++r)
            for (int q = 0; q < 4; ++q) out[j].E[r][q] = mk(e[r][q].real(), e[r][q].imag());
    }
    for (int j = 0; j + 1 < L; ++j) {
        cplx A[4][4], Ai[4][4];
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) A[r][c] = E[j][r][c];
        if (!invert4(A, Ai)) {
            err = "FK model layer " + std::to_string(j + 1) + ": singular wave matrix";
            return FDFK_EINVAL;
        }
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                cplx acc = 0.0;
                for (int q = 0; q < 4; ++q) acc += Ai[r][q] * E[j + 1][q][c];
                out[j].C[r][c] = mk(acc.real(), acc.imag());
            }
    }
    return FDFK_OK;
}

// Work buffers of one call, stream-ordered: allocated and released on the call's stream, so the
// call neither waits for nor blocks other streams.
struct DevBufs {
    cudaStream_t stream = nullptr;
    std::vector<void*> ptrs;
    explicit DevBufs(cudaStream_t s) : stream(s) {}
    ~DevBufs()
    {
        for (void* p : ptrs) cudaFreeAsync(p, stream);
    }
    template <class T>
    cudaError_t alloc(T** p, size_t n)
    {
        *p = nullptr;
        cudaError_t e = cudaMallocAsync((void**)p, std::max<size_t>(n, 1) * sizeof(T), stream);
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
};

}  // namespace

size_t fk_strip_elems(int nx, int nz, int nbd, int k)
{
    const size_t X = nx, Z = nz, B = nbd;
    switch (k) {
    case UXL_REG: case UZL_REG: case UXR_REG: case UZR_REG: return (Z - B) * B;
    case UXB_REG: case UZB_REG: return B * X;
    case UXL_PML: case UZL_PML: case UXR_PML: case UZR_PML: return Z * B;
    default: return B * (X + 2 * B);
    }
}

#define FK_CK(call)                                                                              \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);                            \
            return e_ == cudaErrorMemoryAllocation ? FDFK_ENOMEM : FDFK_ECUDA;                   \
        }                                                                                        \
    } while (0)
int fk_background(const FkJob& J, float* const dst[12], cudaStream_t stream, std::string& err, long long* launches)
{
    if (J.nx < 1 || J.nbd < 1 || J.nz <= J.nbd || J.npml < J.nbd || J.nt < 1 || !(J.dt > 0.0) || !(J.dx > 0.0) ||
        !(J.dz > 0.0)) {
        err = "FK: need nx >= 1, nz > nbd >= 1, npml >= nbd, nt >= 1 and positive dt, dx, dz";
        return FDFK_EINVAL;
    }
    if (!J.bazs || !J.model[0] || !J.model[1]) {
        err = "FK: NULL back-azimuths or model";
        return FDFK_EINVAL;
    }
    for (int m = 0; m < 2; ++m)
        if (J.nlayer[m] < 1 || J.nlayer[m] > kFkMaxLayers) {
            err = "FK: layer count must be 1.." + std::to_string(kFkMaxLayers);
            return FDFK_EINVAL;
        }
    for (int k = 0; k < NSTRIP; ++k)
        if (!dst[k]) {
            err = "FK: NULL strip array";
            return FDFK_EINVAL;
        }

    // transform geometry
    FkGeom g{};
    long long N = 1;
    while (N < 2LL * (J.nt + 1)) N *= 2;
    if (N > (1LL << 23)) {   // the df64 twiddle tables hold N/2 entries
        err = "FK: nt too large (at most 4194302 time steps)";
        return FDFK_EINVAL;
    }
    g.N = (int)N;
    g.nh = g.N / 2;
    g.alpha = 10.0 / (J.nt * J.dt);
    g.dw = 2.0 * kPi / (N * J.dt);
    const long long kcut = (long long)std::floor(10.0 * J.f0 * (double)N * J.dt);
    g.K = (int)std::min<long long>(g.nh - 1, std::max<long long>(kcut, 0)) + 1;

    std::vector<FkLayer> lay[2];
    for (int m = 0; m < 2; ++m) {
        const int rc = build_layers(J.model[m], J.nlayer[m], J.rayp, lay[m], err);
        if (rc) return rc;
    }

    // damped, delayed Ricker samples and the output scale exp(alpha t_n) / N
    std::vector<double> w(J.nt + 1), escale(J.nt + 1);
    std::vector<float2> escf(J.nt + 2, float2{0.f, 0.f});   // df64 pairs, one spare entry
    for (int n = 0; n <= J.nt; ++n) {
        const double t = n * J.dt;
        const double a = (kPi * J.f0 * (t - 1.25 / J.f0)) * (kPi * J.f0 * (t - 1.25 / J.f0));
        w[n] = J.ds * (1.0 - 2.0 * a) * std::exp(-a) * std::exp(-g.alpha * t);
        escale[n] = std::exp(g.alpha * t) / (double)N;
        df64::split(escale[n], escf[n].x, escf[n].y);
    }

    // columns 1-nbd .. nx+nbd: cos(baz) (FP64, and split into a df64 pair) and the horizontal delay D
    const int NXb = J.nx + 2 * J.npml;
    double sum = 0.0;
    for (int i = 0; i < NXb; ++i) sum += J.bazs[i];
    const double cbar = std::cos(sum / (NXb + 1));
    const double half = 0.5 * (J.nx - 1) * J.dx;
    const double xcen = J.x0 + half;
    const double rref = half * std::fabs(cbar);
    const int ncol = J.nx + 2 * J.nbd;
    std::vector<double> D(ncol);
    std::vector<float2> cosd(ncol);
    for (int c = 0; c < ncol; ++c) {
        const int cx = c + 1 - J.nbd;
        const double cp = std::cos(J.bazs[cx - 1 + J.npml]);
        df64::split(cp, cosd[c].x, cosd[c].y);
        const double x = J.x0 + (cx - 1) * J.dx;
        D[c] = J.rayp * (cp * (x - xcen) - rref);
    }

    // series table
    SeriesTab tab{};
    const int side_of[NSTRIP] = {0, 0, 1, 1, 2, 2, 0, 0, 1, 1, 2, 2};
    tab.off[0] = 0;
    for (int s = 0; s < NSTRIP; ++s) {
        const bool reg = s < 6;
        const int side = side_of[s];
        int n1, iz0, ix0;
        if (side == 0) {
            n1 = reg ? J.nz - J.nbd : J.nz;
            iz0 = 1;
            ix0 = reg ? 1 : 1 - J.nbd;
        } else if (side == 1) {
            n1 = reg ? J.nz - J.nbd : J.nz;
            iz0 = 1;
            ix0 = reg ? J.nx - J.nbd + 1 : J.nx + 1;
        } else {
            n1 = J.nbd;
            iz0 = reg ? J.nz - J.nbd + 1 : J.nz + 1;
            ix0 = reg ? 1 : 1 - J.nbd;
        }
        tab.n1[s] = n1;
        tab.iz0[s] = iz0;
        tab.ix0[s] = ix0;
        tab.model_side[s] = side;
        tab.per[s] = (long long)fk_strip_elems(J.nx, J.nz, J.nbd, s);
        tab.off[s + 1] = tab.off[s] + tab.per[s];
        tab.dst[s] = dst[s];
    }
    tab.nx = J.nx;
    tab.nbd = J.nbd;
    tab.nrow = J.nz + J.nbd;
    tab.bottom_pos = cbar >= 0.0 ? 1 : 0;
    const long long nseries = tab.off[NSTRIP];

    DevBufs B(stream);
    FkLayer *d_lay0, *d_lay1;
    double *d_w, *d_D;
    float2* d_esc;
    float2* d_cos;
    cd *d_tw, *d_W, *d_amp0, *d_amp1;
    float4 *d_U, *d_Ph, *d_twM, *d_twN;
    FK_CK(B.alloc(&d_lay0, lay[0].size()));
    FK_CK(B.alloc(&d_lay1, lay[1].size()));
    FK_CK(B.alloc(&d_w, w.size()));
    FK_CK(B.alloc(&d_esc, escf.size()));
    FK_CK(B.alloc(&d_cos, cosd.size()));
    FK_CK(B.alloc(&d_D, D.size()));
    FK_CK(B.alloc(&d_tw, (size_t)g.N));
    FK_CK(B.alloc(&d_W, (size_t)g.K));
    FK_CK(B.alloc(&d_amp0, (size_t)g.K * J.nlayer[0] * 4));
    FK_CK(B.alloc(&d_amp1, (size_t)g.K * J.nlayer[1] * 4));
    FK_CK(B.alloc(&d_U, (size_t)2 * tab.nrow * g.K * 2));
    FK_CK(B.alloc(&d_Ph, (size_t)ncol * g.K));
    FK_CK(B.alloc(&d_twM, (size_t)g.nh));
    FK_CK(B.alloc(&d_twN, (size_t)g.nh));
    FK_CK(cudaMemcpyAsync(d_lay0, lay[0].data(), lay[0].size() * sizeof(FkLayer), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_lay1, lay[1].data(), lay[1].size() * sizeof(FkLayer), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_w, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_esc, escf.data(), escf.size() * sizeof(float2), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_cos, cosd.data(), cosd.size() * sizeof(float2), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_D, D.data(), D.size() * sizeof(double), cudaMemcpyHostToDevice, stream));

    long long nl = 0;
    fk_twiddle<<<(g.N + 255) / 256, 256, 0, stream>>>(g.N, d_tw);
    fk_df_twiddles<<<(g.nh + 255) / 256, 256, 0, stream>>>(g.nh, d_twM, d_twN);
    fk_source_dft<<<g.K, 256, 0, stream>>>(J.nt, g.N, d_w, d_tw, d_W);
    fk_layer_amps<<<(2 * g.K + 127) / 128, 128, 0, stream>>>(g, d_lay0, d_lay1, J.nlayer[0], J.nlayer[1],
                                                             J.p_wave ? 2 : 3, -1.0, J.z0 + (J.nz - 1) * J.dz,
                                                             d_amp0, d_amp1);
    {
        const long long n = 2LL * tab.nrow * g.K;
        fk_depth_response<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(g, d_lay0, d_lay1, J.nlayer[0],
                                                                          J.nlayer[1], d_amp0, d_amp1, tab.nrow,
                                                                          J.z0, J.dz, d_U);
    }
    {
        const long long n = (long long)ncol * g.K;
        fk_column_phase<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(g, ncol, d_D, d_W, d_Ph);
    }
    nl += 6;
    FK_CK(cudaGetLastError());

    // the transform: Q-point branches (Q <= kMaxQ, P = M / Q branches per series); batches of
    // series sized so that their float output (nt + 1 samples each) stays within a fixed budget
    const int M = g.nh;
    const int Q = std::min(M, kMaxQ), P = M / Q;
    const size_t per_series = (size_t)(J.nt + 1) * sizeof(float);
    const size_t budget = (size_t)1 << 30;
    long long bmax = std::max<long long>(1, std::min<long long>(nseries, (long long)(budget / per_series)));
    if (const char* e = std::getenv("FDFK_FK_BATCH")) {   // series per batch (tuning and tests)
        const long long v = std::atoll(e);
        if (v > 0) bmax = std::min(bmax, v);
    }
    bmax = std::min<long long>(bmax, 1 << 30);
    float* d_out;
    FK_CK(B.alloc(&d_out, (size_t)bmax * (J.nt + 1)));
    for (long long g0 = 0; g0 < nseries; g0 += bmax) {
        const int nb = (int)std::min<long long>(bmax, nseries - g0);
        FK_CK(launch_transform_q<kMaxQ>(Q, dim3(nb, P), stream, g, tab, g0, P, J.nt, d_U, d_Ph, d_cos, d_twM,
                                        d_twN, d_esc, d_out));
        const dim3 ge((J.nt + 1 + 31) / 32, (nb + 31) / 32);
        fk_epilogue<<<ge, dim3(32, 8), 0, stream>>>(tab, g0, nb, J.nt, d_out);
        nl += 2;
        FK_CK(cudaGetLastError());
    }
    if (launches) *launches += nl;
    return FDFK_OK;
}

}  // namespace fdfk
