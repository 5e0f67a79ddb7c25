// Single time step with all device buffers carved from a fixed static device
// array (fdfk_noalloc.cu).
#pragma once
#include "fdfk_gb300.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <string>

namespace fdfk {

// Size of the static device scratch: 16 Mi floats (64 MiB).
constexpr size_t kNoAllocFloats = size_t(1) << 24;
// Largest NX or NZ the fixed host damping tables hold.
constexpr int kNoAllocMaxDim = 1 << 16;

// Scratch floats one step of this geometry needs (every region rounded up to 256 bytes).
size_t noalloc_floats_needed(const fdfk_params& p);

// One step of updatedispl_ semantics on the static scratch; `p` already validated and the FD
// coefficient tables already in constant memory on the current device.
int step_noalloc(const fdfk_params& p, int it, const float* const strips[12], const float* c, float* ux, float* uz,
                 float* const bp[12], float* const bu[24], cudaStream_t st, std::string& err, long long* launches);

// Material planes from the reference's material array c(3, NZ, NX) (rho, lambda, mu) on the
// device: dt^2/rho, lambda, mu with leading dimension ldz, row r of c at plane row r + zpad (plane
// rows before zpad and from zpad + NZ on are padding: 0, 0, 1).  Sets bit 0 of *flag where rho <= 0
// and bit 1 where mu <= 0 or lambda + 2 mu <= 0 (the checks of the session API).  Enqueued on st.
cudaError_t launch_material(const float* c, int NZ, int NX, int ldz, double dt2, float* kd, float* la, float* mu,
                            int* flag, cudaStream_t st, int zpad = 0);

}  // namespace fdfk
