// Private: the session object shared by the C-ABI translation units (sessions, batches).
#pragma once
#include "fdfk_gb300.h"
#include "fdfk_sweep.cuh"

#include <cuda_runtime.h>

#include <string>
#include <vector>

struct fdfk_batch;

struct fdfk_session {
    fdfk_params p{};
    int NZ = 0, NX = 0, ldz = 0;   // last row nz + npml, columns, plane leading dimension
    int izt = 1;                   // top row: 1 (free surface) or 1 - npml (absorbing layer on top)
    int zorg = 1;                  // grid row at plane row 0 (plane_zorg(izt))
    int rows = 0;                  // grid rows izt..NZ (the reference arrays' first extent)
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;     // second stream for the tiled kernel
    cudaEvent_t fork = nullptr, join = nullptr;
    float* kdt2 = nullptr;
    float* lam = nullptr;
    float* mu = nullptr;
    float* ux[2] = {nullptr, nullptr};
    float* uz[2] = {nullptr, nullptr};
    float* fux = nullptr;   // frame of the fast path (allocated when it runs)
    float* fuz = nullptr;
    float* bu[24][2] = {};
    float* bp[12] = {};
    fdfk::DampCol* dampx = nullptr;
    fdfk::DampCol* dampz = nullptr;
    float* strip[fdfk::NSTRIP] = {};
    std::vector<char> have_bg;   // per time index
    int cur = 0;
    int it = 0;
    // receivers
    int nrcv = 0, nstp = 1, nsis = -1, isis = 0, istp = 0;
    float x0 = 0.f, z0 = 0.f;
    float* rx = nullptr;
    float* rz = nullptr;
    int4* rsite = nullptr;
    double* rw = nullptr;
    float* seisx = nullptr;
    float* seisz = nullptr;
    fdfk::StepArgs base{};
    fdfk::MarchArgs march{};
    fdfk_batch* batch = nullptr;   // set while the session is a member of a batch
    int pml_run = fdfk::kPmlRun;   // absorbing-layer tile length (tunable)
};

namespace fdfk {
int set_error(int code, const std::string& msg);   // the calling thread's fdfk_last_error; returns code
void count_launches(long long n);                   // adds to fdfk_kernel_launches
}  // namespace fdfk
