// Receiver functions by iterative time-domain deconvolution on the GPU (FP64): the
// downstream step of utils/makeRFitdecon.m (Ligorria and Ammon 1999, the
// time-domain variant of that file), one CUDA block per trace.
//
// Per trace: U = G*num and W = G*(den with the lag ends zeroed) ('same'
// convolutions with the Gaussian G); then, until the misfit stops improving by
// minderr or itmax spikes are placed: correlate the residual with W over the
// accepted lags, add the largest (first on ties) correlation as a spike, filter
// the spike train with G, convolve it with the unfiltered denominator and
// subtract it from U.  The Gaussian's samples that are exactly zero (far tails)
// are skipped, and the spike train is kept as its list of nonzero entries:
// neither changes any sum.
#include "fdfk_gb300.h"
#include "fdfk_session.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace fdfk {

namespace {

constexpr int kRfThreads = 256;
constexpr int kRfMaxSpikes = 4096;   // distinct spike positions kept per trace (<= itmax)

struct RfJob {
    int ntin, ntr, ld;
    int begnlag, endnlag, ml, L;     // accepted lags -begnlag..endnlag, spike train length L = 2 ml + 1
    int itmax;
    double minderr;
    int g0, g1, s;                   // nonzero support of G, 'same' offset floor(ntin / 2)
    const double* g;                 // [ntin]
    const float* num;                // [ntr][ld]
    const float* den;
    double* scratch;                 // per trace: WIN, U, W, R (ntin each), P0, RFP, RW (L each)
    double* rfp;                     // [ntr][L] final filtered spike train
    double* rms;                     // [ntr][itmax]
    int* iters;                      // [ntr]
};

__device__ double block_sum(double v, double* red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < kRfThreads / 32; ++i) t += red[i];
    __syncthreads();
    if (threadIdx.x == 0) red[0] = t;
    __syncthreads();
    const double r = red[0];
    __syncthreads();
    return r;
}

// conv(a, G, 'same')[i] over a's entries lo..hi-1 (the others are zero)
__device__ __forceinline__ double conv_g(const RfJob& J, const double* a, int lo, int hi, int i)
{
    const int jlo = max(lo, i + J.s - J.g1), jhi = min(hi - 1, i + J.s - J.g0);
    double acc = 0.0;
    for (int j = jlo; j <= jhi; ++j) acc = fma(a[j], J.g[i + J.s - j], acc);
    return acc;
}

__global__ void __launch_bounds__(kRfThreads) fdfk_rf_kernel(RfJob J)
{
    __shared__ double red[kRfThreads / 32];
    __shared__ int spikes[kRfMaxSpikes];
    __shared__ int n_spikes, rlo, rhi;
    __shared__ double s_derr, s_sumsq_i;
    __shared__ int wbest[kRfThreads / 32];
    const int tr = blockIdx.x, tid = threadIdx.x;
    const int N = J.ntin, L = J.L, ml = J.ml;
    double* WIN = J.scratch + (size_t)tr * (4 * (size_t)N + 3 * (size_t)L);
    double* U = WIN + N;
    double* W = U + N;
    double* R = W + N;
    double* P0 = R + N;
    double* RFP = P0 + L;
    double* RW = RFP + L;
    const float* num = J.num + (size_t)tr * J.ld;
    const float* den = J.den + (size_t)tr * J.ld;

    for (int i = tid; i < N; i += kRfThreads) {
        WIN[i] = (double)den[i];
        R[i] = (double)num[i];           // staging of the numerator
    }
    for (int i = tid; i < L; i += kRfThreads) P0[i] = 0.0;
    __syncthreads();
    // filtered numerator, filtered chopped denominator, and the power terms
    double pu = 0.0, pw = 0.0;
    for (int i = tid; i < N; i += kRfThreads) {
        const double u = conv_g(J, R, 0, N, i);
        U[i] = u;
        W[i] = conv_g(J, WIN, J.begnlag, N - J.endnlag, i);
        const double wf = conv_g(J, WIN, 0, N, i);
        pu = fma(u, u, pu);
        pw = fma(wf, wf, pw);
    }
    const double invpowU = 1.0 / block_sum(pu, red);
    const double invpowW = 1.0 / block_sum(pw, red);
    for (int i = tid; i < N; i += kRfThreads) R[i] = U[i];
    if (tid == 0) {
        n_spikes = 0;
        s_sumsq_i = 1.0;
        s_derr = 100.0 / invpowU + J.minderr;
        rlo = L;
        rhi = -1;
    }
    __syncthreads();

    const int lag1 = -J.begnlag, lag2 = J.endnlag;
    int it = 0;
    while (fabs(s_derr) > J.minderr && it < J.itmax) {
        ++it;
        // correlation of the residual with W at the accepted lags, and its largest magnitude (the
        // first lag on ties, as MATLAB's max)
        double bv = -1.0;
        int bk = lag1 + ml;              // a valid position whatever the values (NaN never wins)
        for (int m = lag1 + tid; m <= lag2; m += kRfThreads) {
            const int n0 = max(0, -m), n1 = min(N, N - m);
            double acc = 0.0;
            for (int n = n0; n < n1; ++n) acc = fma(R[n + m], W[n], acc);
            const double v = acc * invpowW;
            const int k = m + ml;
            RW[k] = v;
            if (fabs(v) > bv) {       // lags ascend within a thread: strict > keeps the first
                bv = fabs(v);
                bk = k;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_down_sync(0xffffffffu, bv, o);
            const int ok = __shfl_down_sync(0xffffffffu, bk, o);
            if (ov > bv || (ov == bv && ok < bk)) {
                bv = ov;
                bk = ok;
            }
        }
        if ((tid & 31) == 0) {
            red[tid >> 5] = bv;
            wbest[tid >> 5] = bk;
        }
        __syncthreads();
        if (tid == 0) {
            int kb = wbest[0];
            double vb = red[0];
            for (int w = 1; w < kRfThreads / 32; ++w)
                if (red[w] > vb || (red[w] == vb && wbest[w] < kb)) {
                    vb = red[w];
                    kb = wbest[w];
                }
            int p = n_spikes;                  // the sorted list of spike positions
            while (p > 0 && spikes[p - 1] > kb) --p;
            if (p == 0 || spikes[p - 1] != kb) {   // a new position (itmax <= kRfMaxSpikes)
                for (int q = n_spikes; q > p; --q) spikes[q] = spikes[q - 1];
                spikes[p] = kb;
                ++n_spikes;
            }
            P0[kb] += RW[kb];
            rlo = max(0, min(rlo, kb - J.s + J.g0));
            rhi = min(L - 1, max(rhi, kb - J.s + J.g1));
        }
        __syncthreads();
        // filtered spike train (conv(P0, G, 'same')) on its nonzero range
        for (int i = tid; i < L; i += kRfThreads) {
            double acc = 0.0;
            if (i >= rlo && i <= rhi)
                for (int q = 0; q < n_spikes; ++q) {
                    const int j = spikes[q], gi = i + J.s - j;
                    if (gi >= J.g0 && gi <= J.g1) acc = fma(P0[j], J.g[gi], acc);
                }
            RFP[i] = acc;
        }
        __syncthreads();
        // predicted numerator conv(den, RFP, 'same') and the new residual
        double ss = 0.0;
        for (int n = tid; n < N; n += kRfThreads) {
            const int jlo = max(0, n + ml - rhi), jhi = min(N - 1, n + ml - rlo);
            double up = 0.0;
            for (int j = jlo; j <= jhi; ++j) up = fma(WIN[j], RFP[n + ml - j], up);
            const double r = U[n] - up;
            R[n] = r;
            ss = fma(r, r, ss);
        }
        const double sumsq = block_sum(ss, red) * invpowU;
        if (tid == 0) {
            J.rms[(size_t)tr * J.itmax + (it - 1)] = sumsq;
            s_derr = 100.0 * (s_sumsq_i - sumsq);
            s_sumsq_i = sumsq;
        }
        __syncthreads();
    }
    for (int i = tid; i < L; i += kRfThreads) J.rfp[(size_t)tr * L + i] = it > 0 ? RFP[i] : 0.0;
    if (tid == 0) J.iters[tr] = it;
}

int mround(double x) { return (int)(x < 0 ? -std::floor(-x + 0.5) : std::floor(x + 0.5)); }

}  // namespace

}  // namespace fdfk

using namespace fdfk;

extern "C" int fdfk_rf_itdecon(const float* num, const float* den, int nt, int ntr, int ld, double dt, double minlag,
                               double maxlag, double tshift, double f0, int itmax, double minderr, double* rf,
                               int ldrf, int* nrf, double* rms, int* iters)
{
    if (!nrf || nt < 1 || ntr < 0 || ld < nt || !(dt > 0.0) || !(f0 > 0.0) || itmax < 0)
        return set_error(FDFK_EINVAL, "rf_itdecon: need nt >= 1, ld >= nt, dt > 0, f0 > 0, itmax >= 0");
    // lag counts and the reference's halving rule
    int endn = std::max(mround(maxlag / dt), 0), begn = std::max(mround(-minlag / dt), 0);
    while (begn + endn > nt) {
        if (begn > 0) { minlag *= 0.5; begn = std::max(mround(-minlag / dt), 0); }
        if (endn > 0) { maxlag *= 0.5; endn = std::max(mround(maxlag / dt), 0); }
    }
    const int ml = std::max(begn, endn), L = 2 * ml + 1;
    // output window of the filtered spike train (with the reference's time-shift rule)
    int i1 = ml - begn + 1, i2 = ml + endn + 1;   // 1-based
    const int shifti = mround(tshift / dt);
    if (shifti > 0) {
        i1 -= shifti;
        if (i1 <= 0) i1 = 1;
    } else if (shifti < 0) {
        i1 -= shifti;
        i2 = std::min(L, i2 - shifti);
    }
    *nrf = std::max(0, i2 - i1 + 1);
    if (!rf) return FDFK_OK;                       // length query
    if (!num || !den || ldrf < *nrf || (itmax > 0 && !rms) || !iters)
        return set_error(FDFK_EINVAL, "rf_itdecon: NULL array or ldrf < the receiver-function length");
    if (itmax > kRfMaxSpikes) return set_error(FDFK_EINVAL, "rf_itdecon: itmax must be <= 4096");
    if (ntr == 0) return FDFK_OK;
    // Gaussian filter and its nonzero support
    std::vector<double> g(nt);
    const double sigma = 1.0 / (std::sqrt(2.0) * f0), mu = dt * mround(0.5 * nt - 0.5);
    int g0 = nt, g1 = -1;
    for (int i = 0; i < nt; ++i) {
        const double x = (dt * i - mu) / sigma;
        g[i] = dt * (std::exp(-0.5 * x * x) / (sigma * std::sqrt(2.0 * 3.14159265358979323846)));
        if (g[i] != 0.0) { g0 = std::min(g0, i); g1 = std::max(g1, i); }
    }
    if (g1 < 0) return set_error(FDFK_EINVAL, "rf_itdecon: the Gaussian filter underflows everywhere");

    RfJob J{};
    J.ntin = nt; J.ntr = ntr; J.ld = nt;
    J.begnlag = begn; J.endnlag = endn; J.ml = ml; J.L = L;
    J.itmax = itmax; J.minderr = minderr;
    J.g0 = g0; J.g1 = g1; J.s = nt / 2;
    double *d_g = nullptr, *d_scratch = nullptr, *d_rfp = nullptr, *d_rms = nullptr;
    float *d_num = nullptr, *d_den = nullptr;
    int* d_it = nullptr;
    auto release = [&]() {
        cudaFree(d_g); cudaFree(d_scratch); cudaFree(d_rfp); cudaFree(d_rms); cudaFree(d_num); cudaFree(d_den);
        cudaFree(d_it);
    };
    const size_t per = 4 * (size_t)nt + 3 * (size_t)L;
    cudaError_t e = cudaMalloc((void**)&d_g, nt * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_scratch, per * ntr * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_rfp, (size_t)L * ntr * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_rms, (size_t)std::max(itmax, 1) * ntr * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_num, (size_t)nt * ntr * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_den, (size_t)nt * ntr * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_it, ntr * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(d_g, g.data(), nt * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy2D(d_num, nt * sizeof(float), num, (size_t)ld * sizeof(float), nt * sizeof(float), ntr,
                         cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy2D(d_den, nt * sizeof(float), den, (size_t)ld * sizeof(float), nt * sizeof(float), ntr,
                         cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        release();
        return set_error(e == cudaErrorMemoryAllocation ? FDFK_ENOMEM : FDFK_ECUDA,
                         std::string("rf_itdecon: ") + cudaGetErrorString(e));
    }
    J.g = d_g; J.num = d_num; J.den = d_den; J.scratch = d_scratch; J.rfp = d_rfp; J.rms = d_rms; J.iters = d_it;
    fdfk_rf_kernel<<<ntr, kRfThreads>>>(J);
    count_launches(1);
    e = cudaGetLastError();
    std::vector<double> rfp((size_t)L * ntr);
    if (e == cudaSuccess) e = cudaMemcpy(rfp.data(), d_rfp, rfp.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(iters, d_it, ntr * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && itmax > 0)
        e = cudaMemcpy(rms, d_rms, (size_t)itmax * ntr * sizeof(double), cudaMemcpyDeviceToHost);
    release();
    if (e != cudaSuccess) return set_error(FDFK_ECUDA, std::string("rf_itdecon: ") + cudaGetErrorString(e));
    for (int t = 0; t < ntr; ++t)
        for (int k = 0; k < *nrf; ++k) rf[(size_t)t * ldrf + k] = rfp[(size_t)t * L + (i1 - 1) + k];
    return FDFK_OK;
}
