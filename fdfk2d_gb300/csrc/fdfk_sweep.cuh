// Device-side state and kernels of the hybrid FD-FK time step (sm_103a).
//
// One time step of FDFK2D's `updatedispl_` (call site src/FDFK2D.f90:516-522)
// is one launch of fdfk_step_kernel<NO>.  The grid of CTAs is split into
// interior tiles (rows 1..nz, columns 1..nx: leapfrog, Alterman-Karal
// injection from the outer background strips, stress-image free surface) and
// PML tiles (the absorbing frame: three-way split-field PML with memory
// variables, injection by removing the inner background strips).  Receiver
// sampling (loadseis, src/Submain.f90:33-116) runs in the same launch on
// extra CTAs, reading the level that the step itself never writes.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace fdfk {

constexpr int kMaxOrder = 8;   // FD order 16 (the reference caps norder at (npml+1)/2)
constexpr int kTZ = 32;        // default tile rows (z, the contiguous axis)
constexpr int kTX = 32;        // default tile columns (x)
constexpr int kBandTX = 64;    // columns of the flat top-band tiles (rows 1..2*norder) next to the fast path
constexpr int kPmlTile = 40;   // largest absorbing-layer thickness covered by one tile
constexpr int kPmlRun = 24;    // absorbing-layer tile length along the layer
constexpr int kThreads = 256;  // 8 warps per CTA

// Strip order = argument order of updatedispl_ (src/FDFK2D.f90:517-518).
enum Strip { UXL_REG, UZL_REG, UXR_REG, UZR_REG, UXB_REG, UZB_REG,
             UXL_PML, UZL_PML, UXR_PML, UZR_PML, UXB_PML, UZB_PML, NSTRIP };

struct DampCol {   // per column (x) or row (z): d*dt and dt*d' for the PML
    float y;       // d * dt
    float dtdp;    // dt * dd/ds (signed along +x or +z)
    float rh;      // 1 / (1 + y/2)
    float r1;      // 1 / (1 + y)
};

// One background strip as a rectangle of the grid: rows zr0..zr1, columns xr0..xr1, stored as
// strip[(iz - zr0) + rows * ((ix - xr0) + cols * it)] (time slowest) in strip arrays sx, sz.
struct StripBox {
    int zr0, zr1, xr0, xr1;
    int rows, cols;
    int org;        // zr0 + rows * xr0: the strip offset of (iz, ix) is iz + rows * ix - org
    int sx, sz;
};

// A DampCol from d*dt and dt*d' (the reciprocals formed in double, rounded once).
inline DampCol make_damp(float y, float dtdp)
{
    return DampCol{y, dtdp, (float)(1.0 / (1.0 + 0.5 * (double)y)), (float)(1.0 / (1.0 + (double)y))};
}

struct StepArgs {
    // geometry: rows izt..NZ (izt = 1: free surface on top; izt = 1 - npml: absorbing layer on
    // top), columns 1-npml..nx+npml; plane row 0 holds grid row zorg (zorg = izt, or izt - 1 so
    // that row 1 sits at an even plane row: the fast path's 8-byte row pairs stay aligned)
    int nx, nz, npml, norder, nbd;
    int NZ, NX, ldz;          // last row (nz + npml), columns, leading dimension (padded)
    int izt, zorg;
    float dx, dz;
    float dx2r, dx2p, dz2;    // 1/(dx*dx) as the regular (double-rounded) and PML (float) operators form it
    float dt;
    // material (column-major, ldz stride): k = dt^2/rho, lambda, mu
    const float* __restrict__ kdt2;
    const float* __restrict__ lam;
    const float* __restrict__ mu;
    // displacement planes [level parity]
    float* ux[2];
    float* uz[2];
    // frame of the fast path (u^n + outer background outside the regular domain), same layout
    float* fux;
    float* fuz;
    // PML split fields bu[array][plane] (24 arrays in updatedispl_ order; top unused)
    float* bu[24][2];
    float* bp[12];
    const DampCol* __restrict__ dampx;  // [NX]
    const DampCol* __restrict__ dampz;  // [NZ]
    // background strips (reference layout, time slowest), base of time 0
    const float* __restrict__ strip[NSTRIP];
    // tiles
    int int_rows;                       // interior rows [1, int_rows] handled by the tiled kernel
    int tiles_int_z, tiles_int_x;       // interior tiling
    int tiles_l_z, tiles_l_x;           // left / right PML tiling (same shape)
    int tiles_b_z, tiles_b_x;           // bottom PML tiling
    int tiles_t_z, tiles_t_x;           // top PML tiling (izt < 1; rows izt+1..0, the bottom tiles' shape)
    int top_pass;                       // 1: this launch is the top layer's (after the interior update)
    int n_tiles;                        // tiles of this launch (the top layer's alone when top_pass)
    int tdz[3], tdx[3];                 // tile rows / columns of the interior, side-PML and bottom-PML tiles
    // per tile class: the block's stride (kThreads items) through the item grids of its phases as
    // (pair rows, columns) steps, for the grids of P2 (field tile), M2 (material tile and the
    // z-direction products) and TZe/2 (x-direction products and output cells) pair rows
    int wq[3][3], wr[3][3];
    // the background strips: [0..2] inner (left, right, bottom; removed from the absorbing
    // layers' operator field), [3..5] outer (added to the regular field)
    StripBox sbox[6];
    // receivers sampled in the same launch (0 when this step takes no sample)
    int nrcv;
    int sample_index;          // istp
    int nsamp;                 // nsis + 1 (leading dimension of seis)
    float x0, z0;
    const float* __restrict__ rx;
    const float* __restrict__ rz;
    const int4* __restrict__ rsite;     // per receiver: grid point (ix, iz), masks of points 0..31, 32..48
    const double* __restrict__ rw;      // per receiver: FP64 weights of its 7 x 7 points
    float* seisx;
    float* seisz;
    int it;                    // time index of the background strips
    int cur;                   // plane holding u^n (the other holds u^{n-1}, overwritten by u^{n+1})
};

// Interior fast path (fdfk_march_kernel): rows [z0, nz], columns [1, nx].
struct MarchArgs {
    int z0;          // first output row (odd, >= 2*norder + 1)
    int band_out;    // output rows per warp band (64 - 4*norder)
    int n_bands;
    int seg_len;     // columns per warp segment
    int n_segs;
};

// Tile shapes and counts of fdfk_step_kernel for a (fdfk_sweep.cu); needs nx, nz, npml, NX, izt, int_rows.
void plan_tiles(StepArgs& a, bool band_top, int pml_run = kPmlRun);

// Dynamic shared memory of a's tiled launch.
size_t step_smem_for(const StepArgs& a);
// Receiver-sampling blocks a tiled launch appends for nrcv receivers.
int sample_blocks(int nrcv);
// Sites and weights of nrcv receivers at (rx, rz) (device arrays) for a's grid (nx, nz, npml, dx,
// dz) with origin (x0, z0): site[nrcv], w[49 * nrcv].
cudaError_t launch_receiver_sites(const StepArgs& a, int nrcv, float x0, float z0, const float* rx,
                                  const float* rz, int4* site, double* w, cudaStream_t s);

// Device-side per-member state of a batch (advanced by fdfk_batch_bump before every step).
struct BatchDyn {
    int live;                 // 0 once the member passed its last time index
    int it, nt, cur;
    int nrcv, nstp, nsis, isis, istp;
};

// Device tables of a batch (passed by value to the batched kernels).
struct BatchTab {
    int n;                    // members
    StepArgs* args;           // [n] per-member arguments (time fields written by the bump kernel)
    const MarchArgs* march;   // [n]
    BatchDyn* dyn;            // [n]
    int* live;                // [n] member takes part in the current step
    const int* edge_off;      // [n+1] first tiled-kernel block of each member
    const int* march_off;     // [n+1] first fast-path block of each member
    const int* frame_off;     // [n+1] first frame block of each member
    const int* top_off;       // [n+1] first block of each member's top-layer launch (izt < 1)
};

cudaError_t launch_step_batch(const BatchTab& t, int norder, int blocks, size_t smem, cudaStream_t s);
// The top absorbing layer's launch of one solve (izt < 1): after the interior update of the step,
// whose new values the layer's operator field reads (a with top_pass set by the call).
cudaError_t launch_step_top(const StepArgs& a, cudaStream_t s);
// The top layers of a batch's members with the absorbing layer on top, after the step's interior.
cudaError_t launch_step_top_batch(const BatchTab& t, int norder, int blocks, size_t smem, cudaStream_t s);
cudaError_t launch_batch_bump(const BatchTab& t, cudaStream_t s);
// Frame (frame_blocks blocks) and fast path (blocks blocks) of a batch step.
cudaError_t launch_march_batch(const BatchTab& t, int norder, int frame_blocks, int blocks, cudaStream_t s);
// Blocks of one solve's frame launch (the kernel that writes StepArgs::fux / fuz before the fast path).
int frame_blocks(const StepArgs& a);

// First plane row of a grid with top row izt: izt itself when 1 - izt is even, else one padding
// row above it (the fast path loads rows in 8-byte pairs starting at odd grid rows).
inline int plane_zorg(int izt) { return ((1 - izt) & 1) ? izt - 1 : izt; }

// Leading dimension of the planar arrays: rows zorg..nz+npml, or more when the fast path runs, whose
// last 64-row band may reach past nz + npml (to row nz + 63 - 2*norder); the extra rows are
// padding (u = 0, lambda = 0, mu = 1, dt^2/rho = 0), rounded to 32 rows.
inline int plane_ldz(int nz, int npml, int norder, bool fast_path, int izt = 1)
{
    const int zorg = plane_zorg(izt);
    int need = nz + npml - zorg + 1;
    if (fast_path && nz + 65 - 2 * norder - zorg > need) need = nz + 65 - 2 * norder - zorg;
    return (need + 31) / 32 * 32;
}

constexpr int kMarchSeg = 64;
constexpr int kMarchMaxOrder = 4;

}  // namespace fdfk
