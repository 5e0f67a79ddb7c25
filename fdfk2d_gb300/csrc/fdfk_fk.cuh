// FK background wavefield on the GPU (FP64): the replacement for libFK3D's
// comput_background_wavefield_ (call site src/FDFK2D.f90:429-431).
//
// For an incident P or SV plane wave from the half-space below a 1-D layered
// model with a free surface, the 12 background strips hold, at every strip
// point (x, z) and time t_n = n dt (n = 0..nt):
//
//   s(t_n) = exp(alpha t_n) / N * Re sum_k X_k exp(+2 pi i k n / N)
//   X_k    = W_k * U(z; w_k - i alpha) * exp(i (w_k - i alpha) p (cos(baz) (x - x_c) - x_c' |cos(baz_mean)|))
//
// with W the DFT of the damped, delayed Ricker source, N the smallest power of
// two >= 2 (nt + 1), alpha = 10 / (nt dt), k <= 10 f0 N dt, U the radial (times
// cos(baz)) or vertical displacement of the layered response, x_c the profile
// centre and x_c' = (nx - 1) dx / 2.  Left strips use the left model, right
// strips the right model; bottom strips use the model of the side the wave
// arrives from except the nbd columns below the other side strip.
#pragma once
#include <cuda_runtime.h>

#include <string>

namespace fdfk {

constexpr int kFkMaxLayers = 64;

struct FkJob {
    int nx, nz, npml, nbd, nt;
    bool p_wave;                 // src_type: .true. = P, .false. = SV
    double x0, z0, dx, dz;       // single-precision inputs widened
    double dt, ds, f0, rayp;     // ds and f0 are single-precision inputs widened
    const double* bazs;          // host, nx + 2 npml back-azimuths (rad), columns 1-npml..nx+npml
    int nlayer[2];               // left, right
    const float* model[2];       // host, (4, nlayer) column-major: z_top, vp, vs, rho
};

// Element count per time sample of strip k (reference shapes, src/FDFK2D.f90:328-355).
size_t fk_strip_elems(int nx, int nz, int nbd, int k);

// Computes the 12 strips into device arrays dst[k] (reference layout, time slowest,
// (nt + 1) samples), enqueued on `stream` (work buffers stream-ordered; the call
// returns without waiting for the GPU).  Returns 0 or a negative FDFK_E* status
// with `err` set.  `launches` is incremented by the number of kernels launched.
int fk_background(const FkJob& job, float* const dst[12], cudaStream_t stream, std::string& err,
                  long long* launches);

}  // namespace fdfk
