// Interior fast path of the hybrid FD-FK step (sm_103a): the bulk of the
// regular domain, rows MarchArgs::z0..nz, columns 1..nx.
//
// Each warp owns a band of 64 rows (2 per lane; z is the contiguous axis, so
// every global access of a warp is one contiguous 256-byte run) and marches
// along x over a segment of columns, reading each field column once through a
// per-warp shared-memory ring filled by cp.async a few columns ahead
// (fdfk_march_ring.cuh).  The x-direction stencils are evaluated in
// transposed (accumulator) form: every incoming column is folded with one FMA
// per stencil tap into a short chain of partial sums that advances with the
// march, so no operand windows are kept or shifted.  The two rows of a lane go
// through the same operations, so each such FMA (and each per-row product) is
// one packed FP32x2 instruction for both rows, rounded per row as fmaf.  z-direction stencils
// read neighbouring rows with warp shuffles, one shuffle per distinct
// neighbour row.  There is no block-level synchronisation.  The 2*norder halo
// rows on each side of a band are computed but not stored; bands overlap
// accordingly.
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

// c * a + b on both rows of a lane at once (one packed FFMA2; per row the same rounding as fmaf).
__device__ __forceinline__ float2 ffma2(float c, float2 a, float2 b) { return __ffma2_rn(make_float2(c, c), a, b); }
__device__ __forceinline__ float2 ffma2(float2 c, float2 a, float2 b) { return __ffma2_rn(c, a, b); }
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fmul2(float c, float2 a) { return __fmul2_rn(make_float2(c, c), a); }
__device__ __forceinline__ float2 fmul2(float2 a, float c) { return __fmul2_rn(a, make_float2(c, c)); }
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 frcp2(float2 x) { return make_float2(frcp(x.x), frcp(x.y)); }

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
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 1; k <= NO; ++k) s = ffma2(c_coll[NO][k], make_float2(z(k) - z(-k), z(k + 1) - z(1 - k)), s);
    d0 = s.x;
    d1 = s.y;
}

// sum_k c0_k (G(r+k-1) - G(r-k)) of half-row quantities G at this lane's rows
template <int NO>
__device__ __forceinline__ void dz_half(float g0, float g1, float& d0, float& d1)
{
    const ZCol<-NO, NO> z(g0, g1);
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 1; k <= NO; ++k) s = ffma2(c_stag[NO][k], make_float2(z(k - 1) - z(-k), z(k) - z(1 - k)), s);
    d0 = s.x;
    d1 = s.y;
}

}  // namespace march

namespace march {

#include "fdfk_march_ring.cuh"

}  // namespace march

// Warp `warp` of one solve's fast-path launch.
template <int NO>
__device__ __forceinline__ void march_warp(const StepArgs& a, const MarchArgs& m, int warp)
{
    extern __shared__ float ring_smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    if (warp >= m.n_bands * m.n_segs) return;
    const int band = warp % m.n_bands, seg = warp / m.n_bands;
    const int b = m.z0 + band * m.band_out - 2 * NO;   // first row of the band
    const int xs = 1 + seg * m.seg_len;
    const int xe = min(a.nx, xs + m.seg_len - 1);
    float* ring = ring_smem + (size_t)wib * march::Ring<NO>::kWarpFloats;
    march::march_ring<NO>(a, m, lane, b, xs, xe, ring);
}

// ---------------------------------------------------------------------------
// The frame of a step: u^n plus the outer background (Omega_II, as the tiled
// kernel injects it) at every cell the fast path reads outside the regular
// domain -- columns 1-nbd..0 and nx+1..nx+nbd on rows 1..NZ, and rows
// nz..nz+nbd of columns 1..nx (row nz carries no background; it is copied so
// that a lane whose rows straddle nz reads both from the frame).  nbd =
// 2*norder-1 is the reach of the fast path's stencils.  Written before the
// march of the step, read only by it.
// ---------------------------------------------------------------------------
__host__ __device__ inline long long frame_cells(const StepArgs& a)
{
    return 2LL * a.nbd * a.NZ + (long long)(a.nbd + 1) * a.nx;
}

__device__ __forceinline__ void frame_cell(const StepArgs& a, long long i)
{
    const int nbd = a.nbd, NZ = a.NZ, nx = a.nx;
    const long long sidec = (long long)nbd * NZ;
    int iz, ix;
    if (i < 2 * sidec) {
        const bool right = i >= sidec;
        const long long j = right ? i - sidec : i;
        const int c = (int)(j / NZ);
        iz = (int)(j - (long long)c * NZ) + 1;
        ix = right ? nx + 1 + c : 1 - nbd + c;
    } else {
        const long long j = i - 2 * sidec;
        if (j >= (long long)(nbd + 1) * nx) return;
        const int c = (int)(j / (nbd + 1));
        iz = a.nz + (int)(j - (long long)c * (nbd + 1));
        ix = 1 + c;
    }
    const size_t g = gidx(a, iz, ix);
    float vx = a.ux[a.cur][g], vz = a.uz[a.cur][g];
    const float* pz = nullptr;
    const float* px = outer_bg_ptr(a, iz, ix, pz);
    if (px) {
        vx += __ldg(px);
        vz += __ldg(pz);
    }
    a.fux[g] = vx;
    a.fuz[g] = vz;
}

constexpr int kFrameThreads = 256;

__global__ void __launch_bounds__(kFrameThreads) fdfk_frame_kernel(StepArgs a)
{
    frame_cell(a, (long long)blockIdx.x * kFrameThreads + threadIdx.x);
}

// The frames of every live member of a batch: member s owns blocks frame_off[s] .. frame_off[s+1]-1.
__global__ void __launch_bounds__(kFrameThreads) fdfk_frame_batch_kernel(BatchTab t)
{
    __shared__ StepArgs sa;
    const int s = batch_member(t.frame_off, t.n, blockIdx.x);
    if (!t.live[s]) return;
    stage_args(sa, t.args + s);
    frame_cell(sa, (long long)(blockIdx.x - t.frame_off[s]) * kFrameThreads + threadIdx.x);
}

// Blocks of one member's frame launch.
int frame_blocks(const StepArgs& a)
{
    return (int)((frame_cells(a) + kFrameThreads - 1) / kFrameThreads);
}

template <int NO>
__global__ void __launch_bounds__(128) fdfk_march_kernel(StepArgs a, MarchArgs m)
{
    march_warp<NO>(a, m, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
}

// The fast path over every member of a batch: member s owns blocks march_off[s] .. march_off[s+1]-1.
template <int NO>
__global__ void __launch_bounds__(128) fdfk_march_batch_kernel(BatchTab t)
{
    __shared__ StepArgs sa;
    const int s = batch_member(t.march_off, t.n, blockIdx.x);
    if (!t.live[s]) return;
    stage_args(sa, t.args + s);
    march_warp<NO>(sa, t.march[s], (blockIdx.x - t.march_off[s]) * (blockDim.x >> 5) + (threadIdx.x >> 5));
}

template <int NO>
static size_t march_smem_bytes()
{
    return sizeof(float) * 4 * (size_t)march::Ring<NO>::kWarpFloats;
}

template <int NO>
static cudaError_t launch_march_no(const StepArgs& a, const MarchArgs& m, cudaStream_t s)
{
    const int warps = m.n_bands * m.n_segs;
    const int blocks = (warps + 3) / 4;
    const size_t smem = march_smem_bytes<NO>();
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(fdfk_march_kernel<NO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    fdfk_march_kernel<NO><<<blocks, 128, smem, s>>>(a, m);
    return cudaGetLastError();
}

template <int NO>
static int warp_slots_no()
{
    int dev = 0, sms = 0, blocks = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    const size_t smem = march_smem_bytes<NO>();
    if (cudaFuncSetAttribute(fdfk_march_kernel<NO>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fdfk_march_kernel<NO>, 128, smem) != cudaSuccess) return 0;
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

template <int NO>
static cudaError_t launch_march_batch_no(const BatchTab& t, int blocks, cudaStream_t s)
{
    const size_t smem = march_smem_bytes<NO>();
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(fdfk_march_batch_kernel<NO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    if (blocks == 0) return cudaSuccess;
    fdfk_march_batch_kernel<NO><<<blocks, 128, smem, s>>>(t);
    return cudaGetLastError();
}

cudaError_t launch_march_batch_fast(const BatchTab& t, int norder, int blocks, cudaStream_t s);

// The frames of a batch (frame_blocks blocks), then its fast path (blocks blocks); 0 blocks only
// opts the kernel into its shared memory.
cudaError_t launch_march_batch(const BatchTab& t, int norder, int frame_blocks_total, int blocks, cudaStream_t s)
{
    if (blocks > 0 && frame_blocks_total > 0) {
        fdfk_frame_batch_kernel<<<frame_blocks_total, kFrameThreads, 0, s>>>(t);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_march_batch_fast(t, norder, blocks, s);
}

cudaError_t launch_march_batch_fast(const BatchTab& t, int norder, int blocks, cudaStream_t s)
{
    switch (norder) {
    case 1: return launch_march_batch_no<1>(t, blocks, s);
    case 2: return launch_march_batch_no<2>(t, blocks, s);
    case 3: return launch_march_batch_no<3>(t, blocks, s);
    case 4: return launch_march_batch_no<4>(t, blocks, s);
    default: return cudaErrorInvalidValue;
    }
}

// The frame of the step, then the fast path (two launches); `after_frame` (if not null) is
// recorded on the stream between them.
cudaError_t launch_march_marked(const StepArgs& a, const MarchArgs& m, cudaStream_t s, cudaEvent_t after_frame)
{
    if (m.n_bands <= 0 || m.n_segs <= 0) return cudaSuccess;
    fdfk_frame_kernel<<<frame_blocks(a), kFrameThreads, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (after_frame && (e = cudaEventRecord(after_frame, s)) != cudaSuccess) return e;
    switch (a.norder) {
    case 1: return launch_march_no<1>(a, m, s);
    case 2: return launch_march_no<2>(a, m, s);
    case 3: return launch_march_no<3>(a, m, s);
    case 4: return launch_march_no<4>(a, m, s);
    default: return cudaErrorInvalidValue;
    }
}

// The frame of the step, then the fast path (two launches).
cudaError_t launch_march(const StepArgs& a, const MarchArgs& m, cudaStream_t s)
{
    return launch_march_marked(a, m, s, nullptr);
}

}  // namespace fdfk
