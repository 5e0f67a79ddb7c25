// One updatedispl_-style time step whose device buffers are all carved from a
// fixed, file-scope static device array: no cudaMalloc / cudaFree and no
// allocating library call on any path of the call.
//
// Layout conversions that the session API does on the host (interleaved
// levels -> planes, material -> dt^2/rho, lambda, mu) run here as small
// kernels on raw copies of the caller's arrays held in the same scratch, so the
// call needs no host staging buffers either (the damping profile goes through
// a fixed static host table).
//
// Races: the scratch (and the static host table) is one per process and
// device; two calls that overlap in time - from two host threads, or on two
// streams of the same device - overwrite each other's data.  Calls must be
// serialised by the caller.  Each call returns only after its stream has
// drained, so consecutive calls from one thread are safe on any streams.
//
// First-call setup: the first call on a device resolves the scratch address
// with cudaGetSymbolAddress (which also loads this module) and caches it for
// that device; any failed CUDA call in this path drops the cached address, so
// the next call resolves it again (after a device reset the first call may
// fail once with FDFK_ECUDA).  No call may be made on a stream that is being
// captured, nor while any global-mode capture is in progress: every call does
// pageable copies and waits for its stream.
//
// The FD coefficient tables go to constant memory once per device, before
// this path runs (the caller, fdfk_step_noalloc, sees to it).
#include "fdfk_gb300.h"
#include "fdfk_noalloc.cuh"
#include "fdfk_sweep.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

namespace fdfk {

cudaError_t launch_step(const StepArgs& a, cudaStream_t s);

namespace {

__device__ __align__(256) float g_na_scratch[kNoAllocFloats];

constexpr int kMaxDevices = 64;
float* g_na_base[kMaxDevices] = {};

// Drops the cached scratch address of the current device (after a failed CUDA call).
void na_forget()
{
    int d = -1;
    if (cudaGetDevice(&d) == cudaSuccess && d >= 0 && d < kMaxDevices) g_na_base[d] = nullptr;
}
DampCol g_na_dampx[kNoAllocMaxDim];
DampCol g_na_dampz[kNoAllocMaxDim];

size_t up64(size_t n) { return (n + 63) / 64 * 64; }   // 256-byte granules

struct Deint {            // one interleaved (2, m) array <-> two planes
    float* raw;
    float* p0;
    float* p1;
    long long m;
    int n1, kind;         // rows per column; 0 left side, 1 right side, 2 bottom
};
struct DeintTab {
    Deint a[18];
};

__global__ void na_material(const float* __restrict__ c, int NZ, int NX, int ldz, double dt2, float* __restrict__ kd,
                            float* __restrict__ la, float* __restrict__ mu, int* __restrict__ flag, int zpad)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)ldz * NX) return;
    const int z = (int)(i % ldz) - zpad, x = (int)(i / ldz);
    if (z < 0 || z >= NZ) {
        kd[i] = 0.f;
        la[i] = 0.f;
        mu[i] = 1.f;
        return;
    }
    const size_t s = 3 * ((size_t)z + (size_t)NZ * x);
    const float rho = c[s], l = c[s + 1], m = c[s + 2];
    if (!(rho > 0.f)) atomicOr(flag, 1);
    kd[i] = (float)(dt2 / (double)rho);
    la[i] = l;
    mu[i] = m;
    if (!(m > 0.f) || !(__fadd_rn(l, __fmul_rn(2.0f, m)) > 0.f)) atomicOr(flag, 2);
}

// raw (2, NZ, NX) levels -> padded planes p0 (level 1), p1 (level 2) for ux and uz
__global__ void na_unpack_u(const float* __restrict__ rux, const float* __restrict__ ruz, int NZ, int NX, int ldz,
                            float* __restrict__ ux0, float* __restrict__ ux1, float* __restrict__ uz0,
                            float* __restrict__ uz1)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)ldz * NX) return;
    const int z = (int)(i % ldz), x = (int)(i / ldz);
    if (z >= NZ) {
        ux0[i] = ux1[i] = uz0[i] = uz1[i] = 0.f;
        return;
    }
    const size_t s = 2 * ((size_t)z + (size_t)NZ * x);
    ux0[i] = rux[s];
    ux1[i] = rux[s + 1];
    uz0[i] = ruz[s];
    uz1[i] = ruz[s + 1];
}

// planes -> raw levels: level 1 = new (u^{n+1}), level 2 = old (u^n); the outer frame keeps the caller's level 2
__global__ void na_pack_u(float* __restrict__ rux, float* __restrict__ ruz, int NZ, int NX, int ldz,
                          const float* __restrict__ uxn, const float* __restrict__ uxo,
                          const float* __restrict__ uzn, const float* __restrict__ uzo)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)ldz * NX) return;
    const int z = (int)(i % ldz), x = (int)(i / ldz);
    if (z >= NZ) return;
    const size_t d = 2 * ((size_t)z + (size_t)NZ * x);
    const bool frame = x == 0 || x == NX - 1 || z == NZ - 1;
    rux[d] = uxn[i];
    ruz[d] = uzn[i];
    if (!frame) {
        rux[d + 1] = uxo[i];
        ruz[d + 1] = uzo[i];
    }
}

__global__ void na_unpack_bu(DeintTab t)
{
    const Deint& a = t.a[blockIdx.y];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.m; i += (long long)gridDim.x * blockDim.x) {
        a.p0[i] = a.raw[2 * i];
        a.p1[i] = a.raw[2 * i + 1];
    }
}

// planes -> raw levels (level 1 = p1 = new, level 2 = p0 = old); outer-frame cells keep both caller levels
__global__ void na_pack_bu(DeintTab t, int npml, int NX)
{
    const Deint& a = t.a[blockIdx.y];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.m; i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i % a.n1), j = (int)(i / a.n1);
        const bool frame = a.kind == 0 ? j == 0 : a.kind == 1 ? j == npml - 1 : (r == npml - 1 || j == 0 || j == NX - 1);
        if (frame) continue;
        a.raw[2 * i] = a.p1[i];
        a.raw[2 * i + 1] = a.p0[i];
    }
}

}  // namespace

#define NA_CK(call)                                                                              \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);                            \
            na_forget();                                                                         \
            return FDFK_ECUDA;                                                                   \
        }                                                                                        \
    } while (0)

cudaError_t launch_material(const float* c, int NZ, int NX, int ldz, double dt2, float* kd, float* la, float* mu,
                            int* flag, cudaStream_t st, int zpad)
{
    const long long n = (long long)ldz * NX;
    na_material<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(c, NZ, NX, ldz, dt2, kd, la, mu, flag, zpad);
    return cudaGetLastError();
}

size_t noalloc_floats_needed(const fdfk_params& p)
{
    const size_t NZ = p.nz + p.npml, NX = p.nx + 2 * p.npml, ldz = (NZ + 31) / 32 * 32, n = ldz * NX;
    const size_t side = (size_t)p.nz * p.npml, tb = (size_t)p.npml * NX;
    const size_t nbd = p.nbd, nx = p.nx, nz = p.nz;
    size_t tot = up64(3 * n) + up64(4 * n);
    tot += 2 * (12 * up64(side) + 6 * up64(tb));                       // bu planes (l, r, b)
    tot += 4 * up64(side) + 4 * up64(tb);                              // bp (l, r, b)
    tot += up64(4 * NX) + up64(4 * NZ);                                // damping
    tot += 4 * up64((nz - nbd) * nbd) + 2 * up64(nbd * nx) + 4 * up64(nz * nbd) + 2 * up64(nbd * (nx + 2 * nbd));
    tot += up64(3 * NZ * NX) + 2 * up64(2 * NZ * NX);                  // raw c, ux, uz
    tot += 12 * up64(2 * side) + 6 * up64(2 * tb);                     // raw bu
    tot += 64;                                                         // status flag
    return tot;
}

int step_noalloc(const fdfk_params& p, int it, const float* const strips[12], const float* c, float* ux, float* uz,
                 float* const bp[12], float* const bu[24], cudaStream_t st, std::string& err, long long* launches)
{
    if (p.is_PML_top) {
        err = "the allocation-free step implements the free-surface top boundary only";
        return FDFK_EUNSUPPORTED;
    }
    const int NZ = p.nz + p.npml, NX = p.nx + 2 * p.npml, ldz = (NZ + 31) / 32 * 32;
    const size_t n = (size_t)ldz * NX;
    const size_t need = noalloc_floats_needed(p);
    if (need > kNoAllocFloats || NX > kNoAllocMaxDim || NZ > kNoAllocMaxDim) {
        err = "grid needs " + std::to_string(need) + " scratch floats; the static scratch holds " +
              std::to_string(kNoAllocFloats);
        return FDFK_EINVAL;
    }
    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        err = "device index out of range";
        return FDFK_EINVAL;
    }
    if (!g_na_base[dev]) {
        void* base = nullptr;
        NA_CK(cudaGetSymbolAddress(&base, g_na_scratch));
        g_na_base[dev] = static_cast<float*>(base);
    }
    float* cur = g_na_base[dev];
    auto take = [&](size_t floats) {
        float* r = cur;
        cur += up64(floats);
        return r;
    };
    const size_t side = (size_t)p.nz * p.npml, tb = (size_t)p.npml * NX;
    float* kd = take(3 * n);
    float* la = kd + n;
    float* mu = kd + 2 * n;
    float* pl = take(4 * n);
    float* ux0 = pl;
    float* ux1 = pl + n;
    float* uz0 = pl + 2 * n;
    float* uz1 = pl + 3 * n;
    float* bup[24][2] = {};
    for (int k = 0; k < 18; ++k)
        for (int l = 0; l < 2; ++l) bup[k][l] = take(k < 12 ? side : tb);
    float* bpp[12] = {};
    for (int k = 0; k < 12; ++k)
        if (k < 4 || k >= 8) bpp[k] = take(k < 4 ? side : tb);
    DampCol* dampx = reinterpret_cast<DampCol*>(take(4 * (size_t)NX));
    DampCol* dampz = reinterpret_cast<DampCol*>(take(4 * (size_t)NZ));
    float* sp[NSTRIP];
    size_t per[NSTRIP];
    for (int k = 0; k < NSTRIP; ++k) {
        const size_t nbd = p.nbd, nx = p.nx, nz = p.nz;
        per[k] = k == UXB_REG || k == UZB_REG ? nbd * nx
                 : k == UXB_PML || k == UZB_PML ? nbd * (nx + 2 * nbd)
                 : k < 6 ? (nz - nbd) * nbd : nz * nbd;
        sp[k] = take(per[k]);
    }
    float* rc = take(3 * (size_t)NZ * NX);
    float* rux = take(2 * (size_t)NZ * NX);
    float* ruz = take(2 * (size_t)NZ * NX);
    float* rbu[18];
    for (int k = 0; k < 18; ++k) rbu[k] = take(2 * (k < 12 ? side : tb));
    int* flag = reinterpret_cast<int*>(take(64));

    // damping profile (the closed form of the session path)
    {
        const double lg = std::log(1.0 / p.R0);
        const double Lx = (double)p.npml * p.dx, Lz = (double)p.npml * p.dz;
        const double d0x = (p.npower + 1) * (double)p.vpml * lg / (2.0 * Lx);
        const double d0z = (p.npower + 1) * (double)p.vpml * lg / (2.0 * Lz);
        for (int cx = 0; cx < NX; ++cx) {
            const int ix = cx + 1 - p.npml;
            double s = 0.0, sg = 0.0;
            g_na_dampx[cx] = make_damp(0.f, 0.f);
            if (ix <= 0) { s = (double)(1 - ix) * p.dx / Lx; sg = -1.0; }
            else if (ix > p.nx) { s = (double)(ix - p.nx) * p.dx / Lx; sg = 1.0; }
            else continue;
            const double d = d0x * std::pow(s, p.npower), dp = p.npower * d0x * std::pow(s, p.npower - 1) / Lx;
            g_na_dampx[cx] = make_damp((float)(d * p.dt), (float)(sg * dp * p.dt));
        }
        for (int r = 0; r < NZ; ++r) {
            const int iz = r + 1;
            g_na_dampz[r] = make_damp(0.f, 0.f);
            if (iz <= p.nz) continue;
            const double s = (double)(iz - p.nz) * p.dz / Lz;
            const double d = d0z * std::pow(s, p.npower), dp = p.npower * d0z * std::pow(s, p.npower - 1) / Lz;
            g_na_dampz[r] = make_damp((float)(d * p.dt), (float)(dp * p.dt));
        }
    }
    NA_CK(cudaMemcpyAsync(dampx, g_na_dampx, NX * sizeof(DampCol), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(dampz, g_na_dampz, NZ * sizeof(DampCol), cudaMemcpyHostToDevice, st));

    // raw inputs
    NA_CK(cudaMemcpyAsync(rc, c, 3 * (size_t)NZ * NX * sizeof(float), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(rux, ux, 2 * (size_t)NZ * NX * sizeof(float), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(ruz, uz, 2 * (size_t)NZ * NX * sizeof(float), cudaMemcpyHostToDevice, st));
    for (int k = 0; k < 12; ++k)
        if (bpp[k]) NA_CK(cudaMemcpyAsync(bpp[k], bp[k], (k < 4 ? side : tb) * sizeof(float), cudaMemcpyHostToDevice, st));
    DeintTab tab{};
    long long mmax = 0;
    for (int k = 0; k < 18; ++k) {
        const size_t m = k < 12 ? side : tb;
        NA_CK(cudaMemcpyAsync(rbu[k], bu[k], 2 * m * sizeof(float), cudaMemcpyHostToDevice, st));
        tab.a[k] = Deint{rbu[k], bup[k][0], bup[k][1], (long long)m, k < 12 ? p.nz : p.npml,
                         k < 6 ? 0 : k < 12 ? 1 : 2};
        mmax = std::max<long long>(mmax, (long long)m);
    }
    for (int k = 0; k < NSTRIP; ++k)
        NA_CK(cudaMemcpyAsync(sp[k], strips[k] + per[k] * (size_t)it, per[k] * sizeof(float), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemsetAsync(flag, 0, sizeof(int), st));   // the status flag must start at zero

    const unsigned nb = (unsigned)((n + 255) / 256);
    NA_CK(launch_material(rc, NZ, NX, ldz, p.dt * p.dt, kd, la, mu, flag, st));
    na_unpack_u<<<nb, 256, 0, st>>>(rux, ruz, NZ, NX, ldz, ux0, ux1, uz0, uz1);
    const dim3 gb((unsigned)std::min<long long>((mmax + 255) / 256, 1024), 18);
    na_unpack_bu<<<gb, 256, 0, st>>>(tab);
    NA_CK(cudaGetLastError());
    int hflag = 0;
    NA_CK(cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (launches) *launches += 3;
    if (hflag & 1) {
        err = "density must be positive everywhere";
        return FDFK_EINVAL;
    }
    if (hflag & 2) {
        err = "mu and lambda+2mu must be positive everywhere";
        return FDFK_EINVAL;
    }

    StepArgs a{};
    a.nx = p.nx; a.nz = p.nz; a.npml = p.npml; a.norder = p.norder; a.nbd = p.nbd;
    a.NZ = NZ; a.NX = NX; a.ldz = ldz;
    a.izt = 1; a.zorg = 1;
    a.dx = p.dx; a.dz = p.dz;
    a.dx2r = (float)(1.0 / (double)(p.dx * p.dx));
    a.dx2p = 1.0f / (p.dx * p.dx);
    a.dz2 = 1.0f / (p.dz * p.dz);
    a.dt = (float)p.dt;
    a.kdt2 = kd; a.lam = la; a.mu = mu;
    a.dampx = dampx; a.dampz = dampz;
    for (int k = 0; k < NSTRIP; ++k) a.strip[k] = sp[k];   // time index `it` copied as sample 0
    a.int_rows = p.nz;                                      // the general tiled kernel for every row
    plan_tiles(a, false);
    a.ux[0] = ux0; a.ux[1] = ux1; a.uz[0] = uz0; a.uz[1] = uz1;
    for (int k = 0; k < 24; ++k) { a.bu[k][0] = bup[k][0]; a.bu[k][1] = bup[k][1]; }
    for (int k = 0; k < 12; ++k) a.bp[k] = bpp[k];
    a.it = 0;
    a.cur = 0;
    a.nrcv = 0;
    NA_CK(launch_step(a, st));

    // u^{n+1} is in plane 1, u^n in plane 0
    na_pack_u<<<nb, 256, 0, st>>>(rux, ruz, NZ, NX, ldz, ux1, ux0, uz1, uz0);
    na_pack_bu<<<gb, 256, 0, st>>>(tab, p.npml, NX);
    NA_CK(cudaGetLastError());
    if (launches) *launches += 3;
    NA_CK(cudaMemcpyAsync(ux, rux, 2 * (size_t)NZ * NX * sizeof(float), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaMemcpyAsync(uz, ruz, 2 * (size_t)NZ * NX * sizeof(float), cudaMemcpyDeviceToHost, st));
    for (int k = 0; k < 12; ++k)
        if (bpp[k]) NA_CK(cudaMemcpyAsync(bp[k], bpp[k], (k < 4 ? side : tb) * sizeof(float), cudaMemcpyDeviceToHost, st));
    for (int k = 0; k < 18; ++k)
        NA_CK(cudaMemcpyAsync(bu[k], rbu[k], 2 * (k < 12 ? side : tb) * sizeof(float), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    return FDFK_OK;
}

}  // namespace fdfk
