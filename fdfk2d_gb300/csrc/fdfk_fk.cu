// FK background wavefield on the GPU in FP64 (replaces libFK3D's
// comput_background_wavefield_, call site src/FDFK2D.f90:429-431).
//
// Pipeline (one stream):
//   1. host: per-layer vertical slownesses, wave-vector matrices E (ux, uz,
//      sigma_xz, sigma_zz per unit amplitude of down P, down S, up P, up S) and
//      interface matrices C_j = E_j^-1 E_{j+1}; the damped Ricker samples;
//   2. fk_source_dft: W_k, k <= kmax, direct DFT against an exact twiddle table;
//   3. fk_layer_amps: one thread per (model, frequency) propagates the 4x4
//      layer matrices from the half-space to the surface, solves the 2x2
//      free-surface system for the downgoing half-space amplitudes and writes
//      every layer's amplitudes (phase referenced at the layer top);
//   4. fk_depth_response: U_R, U_Z per (model, grid row, frequency);
//   5. fk_column_phase: W_k times the horizontal phase per (column, frequency);
//   6. per batch of strip series: fk_assemble folds each half spectrum into
//      the input of a half-length complex inverse FFT (batched Z2Z, cuFFT,
//      in place) whose output is the real series, and
//      fk_epilogue scales by exp(alpha t)/N and transposes into the strips
//      (time slowest), float32.
#include "fdfk_fk.cuh"
#include "fdfk_gb300.h"
#include "fdfk_sweep.cuh"

#include <cufft.h>

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
                                  double z0, double dz, cd* __restrict__ U)
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
    U[2 * t] = ur;
    U[2 * t + 1] = uz;
}

// Ph[c * K + k] = W_k exp(i wc_k D_c), D_c = p (cos(baz_c) (x_c' - x_centre) - r_ref).
__global__ void fk_column_phase(FkGeom g, int ncol, const double* __restrict__ D, const cd* __restrict__ W,
                                cd* __restrict__ Ph)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ncol * g.K) return;
    const int k = (int)(t % g.K);
    const int c = (int)(t / g.K);
    const double d = D[c];
    const cd e = cexp_(mk(g.alpha * d, g.dw * k * d));
    Ph[t] = cmul(W[k], e);
}

// Half spectra of series [g0, g0 + nb): spec[b * (nh + 1) + k].
// Bin j (0..nh) of the half spectrum of series p: W_j * phase * U (times cos(baz) for the x
// component), zero from j = K on.
__device__ __forceinline__ cd series_bin(const FkGeom& g, const SeriesTab& tab, const SeriesPos& p, int j,
                                         const cd* __restrict__ U, const cd* __restrict__ Ph,
                                         const double* __restrict__ cosphi)
{
    if (j >= g.K) return mk(0.0, 0.0);
    const int c = p.ix - (1 - tab.nbd);
    const bool xcomp = (p.s & 1) == 0;
    const cd u = U[(((size_t)p.model * tab.nrow + (p.iz - 1)) * g.K + j) * 2 + (xcomp ? 0 : 1)];
    cd v = cmul(Ph[(size_t)c * g.K + j], u);
    if (xcomp) {
        const double cp = cosphi[c];
        v = mk(v.x * cp, v.y * cp);
    }
    return v;
}

// Input of the half-length complex inverse transform that yields a batch of real series: with
// M = N/2 and X the half spectrum (X_0 and X_M enter with their real parts, as for a real series),
//   Z_k = E_k + i O_k,  E_k = X_k + conj(X_{M-k}),  O_k = (X_k - conj(X_{M-k})) exp(+2 pi i k / N),
// sum_k Z_k exp(+2 pi i k m / M) = x[2m] + i x[2m+1], x the length-N real inverse transform of X.
// The complex output read as doubles is therefore x itself.
__device__ __forceinline__ cd fold_bin(cd xk, cd xm, cd t)   // t = exp(-2 pi i k / N)
{
    const cd e = mk(xk.x + xm.x, xk.y - xm.y);
    const cd d = mk(xk.x - xm.x, xk.y + xm.y);
    const cd o = mk(d.x * t.x + d.y * t.y, d.y * t.x - d.x * t.y);   // d * conj(t)
    return mk(e.x - o.y, e.y + o.x);
}

// One block row per series, one thread per bin pair (k, M - k), k = 0..M/2: each spectral bin is
// formed once and feeds both Z_k and Z_{M-k}.
__global__ void fk_assemble(FkGeom g, SeriesTab tab, long long g0, int nb, const cd* __restrict__ U,
                            const cd* __restrict__ Ph, const double* __restrict__ cosphi, const cd* __restrict__ tw,
                            cd* __restrict__ spec)
{
    __shared__ SeriesPos sp;
    const int b = blockIdx.y;
    if (b >= nb) return;
    if (threadIdx.x == 0) sp = decode(tab, g0 + b);
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int M = g.nh;
    if (k > M / 2) return;
    cd* const row = spec + (size_t)b * M;
    if (k < g.K || M - k < g.K) {
        const SeriesPos p = sp;
        cd xk = series_bin(g, tab, p, k, U, Ph, cosphi);
        cd xm = series_bin(g, tab, p, M - k, U, Ph, cosphi);
        if (k == 0) {
            xk.y = 0.0;
            xm.y = 0.0;
        }
        row[k] = fold_bin(xk, xm, tw[k]);
        if (k > 0 && 2 * k < M) row[M - k] = fold_bin(xm, xk, tw[M - k]);
    } else {
        row[k] = mk(0.0, 0.0);
        if (2 * k < M) row[M - k] = mk(0.0, 0.0);
    }
}

// strips[s][q + per_s * n] = float(y[b][n] * escale[n]), n = 0..nt; 32 x 32 tiles through shared memory.
__global__ void fk_epilogue(SeriesTab tab, long long g0, int nb, int N, int nt, const double* __restrict__ y,
                            const double* __restrict__ escale)
{
    __shared__ double tile[32][33];
    const int n0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int b = b0 + ty + 8 * r, n = n0 + tx;
        if (b < nb && n <= nt) tile[ty + 8 * r][tx] = y[(size_t)b * N + n];
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
        if (n <= nt) dst[per * n] = (float)(tile[tx][ty + 8 * r] * escale[n]);
    }
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

// Batched half-length Z2Z inverse plans, one per (device, length, batch), kept for the life of
// the process.  They own no work area: each call supplies its own (stream-ordered), so calls on
// different streams may use one plan at the same time.
struct Z2ZPlan {
    cufftHandle h = 0;
    size_t work = 0;
};

std::mutex g_plan_mu;
std::map<std::tuple<int, int, int>, Z2ZPlan> g_plans;

cufftResult z2z_plan(int m, int batch, Z2ZPlan& out)
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(g_plan_mu);
    const auto key = std::make_tuple(dev, m, batch);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) {
        out = it->second;
        return CUFFT_SUCCESS;
    }
    Z2ZPlan p;
    cufftResult r = cufftCreate(&p.h);
    if (r != CUFFT_SUCCESS) return r;
    int nn = m;
    if ((r = cufftSetAutoAllocation(p.h, 0)) != CUFFT_SUCCESS ||
        (r = cufftMakePlanMany(p.h, 1, &nn, nullptr, 1, m, nullptr, 1, m, CUFFT_Z2Z, batch, &p.work)) !=
            CUFFT_SUCCESS) {
        cufftDestroy(p.h);
        return r;
    }
    g_plans[key] = p;
    out = p;
    return CUFFT_SUCCESS;
}

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
#define FFT_CK(call)                                                                             \
    do {                                                                                         \
        cufftResult r_ = (call);                                                                 \
        if (r_ != CUFFT_SUCCESS) {                                                               \
            err = std::string(#call) + ": cuFFT status " + std::to_string((int)r_);              \
            return r_ == CUFFT_ALLOC_FAILED ? FDFK_ENOMEM : FDFK_ECUDA;                          \
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
    if (N > (1LL << 28)) {
        err = "FK: nt too large";
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
    for (int n = 0; n <= J.nt; ++n) {
        const double t = n * J.dt;
        const double a = (kPi * J.f0 * (t - 1.25 / J.f0)) * (kPi * J.f0 * (t - 1.25 / J.f0));
        w[n] = J.ds * (1.0 - 2.0 * a) * std::exp(-a) * std::exp(-g.alpha * t);
        escale[n] = std::exp(g.alpha * t) / (double)N;
    }

    // columns 1-nbd .. nx+nbd: cos(baz) and the horizontal delay D
    const int NXb = J.nx + 2 * J.npml;
    double sum = 0.0;
    for (int i = 0; i < NXb; ++i) sum += J.bazs[i];
    const double cbar = std::cos(sum / (NXb + 1));
    const double half = 0.5 * (J.nx - 1) * J.dx;
    const double xcen = J.x0 + half;
    const double rref = half * std::fabs(cbar);
    const int ncol = J.nx + 2 * J.nbd;
    std::vector<double> cosphi(ncol), D(ncol);
    for (int c = 0; c < ncol; ++c) {
        const int cx = c + 1 - J.nbd;
        cosphi[c] = std::cos(J.bazs[cx - 1 + J.npml]);
        const double x = J.x0 + (cx - 1) * J.dx;
        D[c] = J.rayp * (cosphi[c] * (x - xcen) - rref);
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
    double *d_w, *d_esc, *d_cos, *d_D;
    cd *d_tw, *d_W, *d_amp0, *d_amp1, *d_U, *d_Ph, *d_spec;
    FK_CK(B.alloc(&d_lay0, lay[0].size()));
    FK_CK(B.alloc(&d_lay1, lay[1].size()));
    FK_CK(B.alloc(&d_w, w.size()));
    FK_CK(B.alloc(&d_esc, escale.size()));
    FK_CK(B.alloc(&d_cos, cosphi.size()));
    FK_CK(B.alloc(&d_D, D.size()));
    FK_CK(B.alloc(&d_tw, (size_t)g.N));
    FK_CK(B.alloc(&d_W, (size_t)g.K));
    FK_CK(B.alloc(&d_amp0, (size_t)g.K * J.nlayer[0] * 4));
    FK_CK(B.alloc(&d_amp1, (size_t)g.K * J.nlayer[1] * 4));
    FK_CK(B.alloc(&d_U, (size_t)2 * tab.nrow * g.K * 2));
    FK_CK(B.alloc(&d_Ph, (size_t)ncol * g.K));
    FK_CK(cudaMemcpyAsync(d_lay0, lay[0].data(), lay[0].size() * sizeof(FkLayer), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_lay1, lay[1].data(), lay[1].size() * sizeof(FkLayer), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_w, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_esc, escale.data(), escale.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_cos, cosphi.data(), cosphi.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    FK_CK(cudaMemcpyAsync(d_D, D.data(), D.size() * sizeof(double), cudaMemcpyHostToDevice, stream));

    long long nl = 0;
    fk_twiddle<<<(g.N + 255) / 256, 256, 0, stream>>>(g.N, d_tw);
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
    nl += 5;
    FK_CK(cudaGetLastError());

    // batches of series: the half-length complex transform runs in place, N doubles per series
    const size_t per_series = (size_t)g.N * sizeof(double);
    const size_t budget = (size_t)2 << 30;
    long long bmax = std::max<long long>(1, std::min<long long>(nseries, (long long)(budget / per_series)));
    if (const char* e = std::getenv("FDFK_FK_BATCH")) {   // series per batch (tuning and tests)
        const long long v = std::atoll(e);
        if (v > 0) bmax = std::min(bmax, v);
    }
    const int nb_full = (int)std::min<long long>(bmax, 65535);
    FK_CK(B.alloc(&d_spec, (size_t)nb_full * g.nh));
    const int tail = (int)(nseries % nb_full);
    Z2ZPlan plan_full, plan_tail;
    FFT_CK(z2z_plan(g.nh, nb_full, plan_full));
    if (tail && nseries > nb_full) FFT_CK(z2z_plan(g.nh, tail, plan_tail));
    void* work = nullptr;
    FK_CK(B.alloc(reinterpret_cast<char**>(&work), std::max(plan_full.work, plan_tail.work)));
    for (long long g0 = 0; g0 < nseries; g0 += nb_full) {
        const int nb = (int)std::min<long long>(nb_full, nseries - g0);
        const dim3 ga((g.nh / 2 + 1 + 255) / 256, nb);
        fk_assemble<<<ga, 256, 0, stream>>>(g, tab, g0, nb, d_U, d_Ph, d_cos, d_tw, d_spec);
        const Z2ZPlan& pl = nb == nb_full ? plan_full : plan_tail;
        FFT_CK(cufftSetWorkArea(pl.h, work));
        FFT_CK(cufftSetStream(pl.h, stream));
        FFT_CK(cufftExecZ2Z(pl.h, (cufftDoubleComplex*)d_spec, (cufftDoubleComplex*)d_spec, CUFFT_INVERSE));
        const dim3 ge((J.nt + 1 + 31) / 32, (nb + 31) / 32);
        fk_epilogue<<<ge, dim3(32, 8), 0, stream>>>(tab, g0, nb, g.N, J.nt, reinterpret_cast<const double*>(d_spec),
                                                    d_esc);
        nl += 2;
        FK_CK(cudaGetLastError());
    }
    if (launches) *launches += nl;
    return FDFK_OK;
}

}  // namespace fdfk
