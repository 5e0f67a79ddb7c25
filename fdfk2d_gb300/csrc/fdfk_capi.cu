// C ABI of fdfk_gb300: sessions, the one-shot time loop and the gfortran-ABI
// drop-in `updatedispl_`.  Declarations and contracts: include/fdfk_gb300.h.
#include "fdfk_fk.cuh"
#include "fdfk_gb300.h"
#include "fdfk_noalloc.cuh"
#include "fdfk_session.h"
#include "fdfk_sweep.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace fdfk {
cudaError_t launch_step(const StepArgs& a, cudaStream_t s);
cudaError_t launch_march(const StepArgs& a, const MarchArgs& m, cudaStream_t s);
cudaError_t launch_march_marked(const StepArgs& a, const MarchArgs& m, cudaStream_t s, cudaEvent_t after_frame);
int march_warp_slots(int norder);
cudaError_t set_coefficients(const float* stag, const float* coll);
}  // namespace fdfk

using namespace fdfk;

namespace {

thread_local std::string g_err;
std::atomic<long long> g_launches{0};

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

}  // namespace

namespace fdfk {
int set_error(int code, const std::string& msg) { return fail(code, msg); }
void count_launches(long long n) { g_launches += n; }
}  // namespace fdfk

namespace {

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return fail(FDFK_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Staggered (fd_coef0) and collocated (fd_coef1) first-derivative weights for
// every reduced order n = 1..8 (src/Submain.f90:1111-1200): the weights of the
// order-2n centred difference on a staggered / collocated stencil.
void fd_tables(float stag[kMaxOrder + 1][kMaxOrder + 1], float coll[kMaxOrder + 1][kMaxOrder + 1])
{
    for (int n = 0; n <= kMaxOrder; ++n)
        for (int j = 0; j <= kMaxOrder; ++j) stag[n][j] = coll[n][j] = 0.f;
    for (int n = 1; n <= kMaxOrder; ++n) {
        for (int j = 1; j <= n; ++j) {
            // staggered: nodes at odd half-integers (2k-1)/2
            double num = 1.0, den = 1.0;
            const double aj = (double)((2 * j - 1) * (2 * j - 1));
            for (int k = 1; k <= n; ++k) {
                if (k == j) continue;
                const double ak = (double)((2 * k - 1) * (2 * k - 1));
                num *= ak;
                den *= (k < j) ? (aj - ak) : (ak - aj);
            }
            double sgn = (j % 2 == 1) ? 1.0 : -1.0;
            stag[n][j] = (float)(sgn * num / (den * (double)(2 * j - 1)));
            // collocated: nodes at integers k
            double numc = 1.0, denc = 1.0;
            const double bj = (double)(j * j);
            for (int k = 1; k <= n; ++k) {
                if (k == j) continue;
                const double bk = (double)(k * k);
                numc *= bk;
                denc *= (k < j) ? (bj - bk) : (bk - bj);
            }
            coll[n][j] = (float)(sgn * numc / (denc * 2.0 * (double)j));
        }
    }
}

size_t strip_elems(const fdfk_params& p, int k)
{
    const size_t nx = p.nx, nz = p.nz, nbd = p.nbd;
    switch (k) {
    case UXL_REG: case UZL_REG: case UXR_REG: case UZR_REG: return (nz - nbd) * nbd;
    case UXB_REG: case UZB_REG: return nbd * nx;
    case UXL_PML: case UZL_PML: case UXR_PML: case UZR_PML: return nz * nbd;
    default: return nbd * (nx + 2 * nbd);
    }
}

// bu / bp array sizes (elements per plane) in the updatedispl_ argument order.
size_t bu_elems(const fdfk_params& p, int k)
{
    const size_t side = (size_t)p.nz * p.npml, tb = (size_t)p.npml * (p.nx + 2 * p.npml);
    return k < 12 ? side : tb;   // l, r then b, t
}
size_t bp_elems(const fdfk_params& p, int k)
{
    const size_t side = (size_t)p.nz * p.npml, tb = (size_t)p.npml * (p.nx + 2 * p.npml);
    return k < 4 ? side : tb;
}

}  // namespace

namespace {

int validate(const fdfk_params* p)
{
    if (!p) return fail(FDFK_EINVAL, "params is NULL");
    if (p->norder < 1 || p->norder > kMaxOrder) return fail(FDFK_EINVAL, "norder must be 1..8");
    if (p->nbd != 2 * p->norder - 1) return fail(FDFK_EINVAL, "nbd must equal 2*norder-1");
    if (p->npml < p->nbd) return fail(FDFK_EINVAL, "npml must be >= 2*norder-1");
    if (p->nx < 1 || p->nz <= p->nbd + 1) return fail(FDFK_EINVAL, "grid too small (need nx >= 1, nz > nbd+1)");
    if (p->nx < 2 * p->nbd) return fail(FDFK_EINVAL, "nx must be >= 2*nbd");
    if (p->nt < 0) return fail(FDFK_EINVAL, "nt must be >= 0");
    if (!(p->dx > 0.f) || !(p->dz > 0.f) || !(p->dt > 0.0)) return fail(FDFK_EINVAL, "dx, dz, dt must be positive");
    if (!(p->R0 > 0.0) || !(p->R0 < 1.0)) return fail(FDFK_EINVAL, "R0 must be in (0, 1)");
    if ((double)(p->nz + (p->is_PML_top ? 2 : 1) * p->npml) * (p->nx + 2 * p->npml) > 2.0e9)
        return fail(FDFK_EINVAL, "grid too large");
    return FDFK_OK;
}

void free_session(fdfk_session* s)
{
    if (!s) return;
    if (s->side) cudaStreamDestroy(s->side);
    if (s->fork) cudaEventDestroy(s->fork);
    if (s->join) cudaEventDestroy(s->join);
    cudaFree(s->kdt2); cudaFree(s->lam); cudaFree(s->mu);
    for (int l = 0; l < 2; ++l) { cudaFree(s->ux[l]); cudaFree(s->uz[l]); }
    cudaFree(s->fux); cudaFree(s->fuz);
    for (int k = 0; k < 24; ++k) for (int l = 0; l < 2; ++l) cudaFree(s->bu[k][l]);
    for (int k = 0; k < 12; ++k) cudaFree(s->bp[k]);
    cudaFree(s->dampx); cudaFree(s->dampz);
    for (int k = 0; k < NSTRIP; ++k) cudaFree(s->strip[k]);
    cudaFree(s->rx); cudaFree(s->rz); cudaFree(s->rsite); cudaFree(s->rw); cudaFree(s->seisx); cudaFree(s->seisz);
    delete s;
}

// The FD coefficient tables in constant memory, uploaded once per device (they depend on nothing
// but the order): a later session neither repeats the copy nor waits for the device.
cudaError_t ensure_coefficients()
{
    static std::mutex mu;
    static std::vector<char> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, 0);
    if (done[dev]) return cudaSuccess;
    float stag[kMaxOrder + 1][kMaxOrder + 1], coll[kMaxOrder + 1][kMaxOrder + 1];
    fd_tables(stag, coll);
    e = set_coefficients(&stag[0][0], &coll[0][0]);
    if (e == cudaSuccess) done[dev] = 1;
    return e;
}

// Material planes from c(3, NZ, NX): the raw array is copied to the device (stream-ordered
// scratch) and converted there (launch_material), then the validity flags are read back.  This
// runs on a stream of the highest priority, so that the wait for the flags does not queue behind
// long kernels of other sessions (an FK background, a batch) already on the device; the session's
// stream is ordered after it by an event.  `fresh`: the planes are new and nothing on the session's
// stream uses them yet; otherwise the upload first waits for the session's stream.
int upload_material(fdfk_session* s, const float* c, bool fresh)
{
    const size_t nc = 3 * (size_t)s->rows * s->NX;
    int lo = 0, hi = 0;
    cudaStream_t up = nullptr;
    cudaEvent_t done = nullptr;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&up, cudaStreamNonBlocking, hi);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
    if (!fresh && e == cudaSuccess) e = cudaEventRecord(done, s->stream);
    if (!fresh && e == cudaSuccess) e = cudaStreamWaitEvent(up, done, 0);
    float* d_c = nullptr;
    int* d_flag = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_c, nc * sizeof(float), up);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_flag, sizeof(int), up);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flag, 0, sizeof(int), up);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_c, c, nc * sizeof(float), cudaMemcpyHostToDevice, up);
    if (e == cudaSuccess)
        e = launch_material(d_c, s->rows, s->NX, s->ldz, s->p.dt * s->p.dt, s->kdt2, s->lam, s->mu, d_flag, up,
                            s->izt - s->zorg);
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, up);
    if (d_c) cudaFreeAsync(d_c, up);
    if (d_flag) cudaFreeAsync(d_flag, up);
    if (e == cudaSuccess) e = cudaEventRecord(done, up);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, done, 0);
    const cudaError_t e2 = up ? cudaStreamSynchronize(up) : cudaSuccess;
    if (e == cudaSuccess) e = e2;
    if (done) cudaEventDestroy(done);
    if (up) cudaStreamDestroy(up);
    if (e != cudaSuccess) return fail(FDFK_ECUDA, std::string("material upload: ") + cudaGetErrorString(e));
    g_launches += 1;
    if (flag & 1) return fail(FDFK_EINVAL, "density must be positive everywhere");
    if (flag & 2) return fail(FDFK_EINVAL, "mu and lambda+2mu must be positive everywhere");
    return FDFK_OK;
}

// Damping profile of the PML (see the module comment of the oracle step):
// d(s) = d0 (s/L)^npower, d0 = (npower+1) vpml ln(1/R0) / (2 L), s counted in
// whole cells from the interface (first PML cell s = h), L = npml*h.
void damping(const fdfk_params& p, std::vector<DampCol>& dx, std::vector<DampCol>& dz)
{
    // dz: rows izt..nz+npml (izt = 1 - npml with the absorbing layer on top: its depth counted
    // from row 1 upwards, d' < 0)
    const int izt = p.is_PML_top ? 1 - p.npml : 1;
    const int NX = p.nx + 2 * p.npml, NZ = p.nz + p.npml - izt + 1;
    const double lg = std::log(1.0 / p.R0);
    const double Lx = (double)p.npml * p.dx, Lz = (double)p.npml * p.dz;
    const double d0x = (p.npower + 1) * (double)p.vpml * lg / (2.0 * Lx);
    const double d0z = (p.npower + 1) * (double)p.vpml * lg / (2.0 * Lz);
    dx.assign(NX, make_damp(0.f, 0.f));
    dz.assign(NZ, make_damp(0.f, 0.f));
    for (int c = 0; c < NX; ++c) {
        int ix = c + 1 - p.npml;
        double s = 0.0, sg = 0.0;
        if (ix <= 0) { s = (double)(1 - ix) * p.dx / Lx; sg = -1.0; }
        else if (ix > p.nx) { s = (double)(ix - p.nx) * p.dx / Lx; sg = 1.0; }
        else continue;
        double d = d0x * std::pow(s, p.npower), dp = p.npower * d0x * std::pow(s, p.npower - 1) / Lx;
        dx[c] = make_damp((float)(d * p.dt), (float)(sg * dp * p.dt));
    }
    for (int r = 0; r < NZ; ++r) {
        int iz = r + izt;
        double s = 0.0, sg = 0.0;
        if (iz <= 0) { s = (double)(1 - iz) * p.dz / Lz; sg = -1.0; }
        else if (iz > p.nz) { s = (double)(iz - p.nz) * p.dz / Lz; sg = 1.0; }
        else continue;
        double d = d0z * std::pow(s, p.npower), dp = p.npower * d0z * std::pow(s, p.npower - 1) / Lz;
        dz[r] = make_damp((float)(d * p.dt), (float)(sg * dp * p.dt));
    }
}

int zero_state(fdfk_session* s)
{
    const size_t n = (size_t)s->ldz * s->NX;
    for (int l = 0; l < 2; ++l) {
        CK(cudaMemsetAsync(s->ux[l], 0, n * sizeof(float), s->stream));
        CK(cudaMemsetAsync(s->uz[l], 0, n * sizeof(float), s->stream));
    }
    if (s->fux) CK(cudaMemsetAsync(s->fux, 0, n * sizeof(float), s->stream));   // rows never written stay 0
    if (s->fuz) CK(cudaMemsetAsync(s->fuz, 0, n * sizeof(float), s->stream));
    for (int k = 0; k < 24; ++k)
        for (int l = 0; l < 2; ++l)
            if (s->bu[k][l]) CK(cudaMemsetAsync(s->bu[k][l], 0, bu_elems(s->p, k) * sizeof(float), s->stream));
    for (int k = 0; k < 12; ++k)
        if (s->bp[k]) CK(cudaMemsetAsync(s->bp[k], 0, bp_elems(s->p, k) * sizeof(float), s->stream));
    s->cur = 0;
    s->it = 0;
    s->isis = 0;
    s->istp = 0;
    return FDFK_OK;
}

// The tiled kernel's share of a step: top band (when the fast path runs), absorbing layers and
// receivers in one launch.
cudaError_t launch_edge(const fdfk_session* s, const StepArgs& a, cudaStream_t st, int* launches)
{
    (void)s;
    *launches = 1;
    return launch_step(a, st);
}

}  // namespace

extern "C" {

int fdfk_version(void) { return 100; }

const char* fdfk_last_error(void) { return g_err.c_str(); }

long long fdfk_kernel_launches(void) { return g_launches.load(); }

int fdfk_session_create(const fdfk_params* p, const float* c, fdfk_session** out)
{
    if (!out) return fail(FDFK_EINVAL, "out is NULL");
    *out = nullptr;
    int rc = validate(p);
    if (rc) return rc;
    if (!c) return fail(FDFK_EINVAL, "c is NULL");
    fdfk_session* s = new (std::nothrow) fdfk_session();
    if (!s) return fail(FDFK_ENOMEM, "host allocation failed");
    s->p = *p;
    s->NZ = p->nz + p->npml;
    s->NX = p->nx + 2 * p->npml;
    s->izt = p->is_PML_top ? 1 - p->npml : 1;
    s->zorg = plane_zorg(s->izt);
    s->rows = s->NZ - s->izt + 1;
    // FDFK_TILED_ONLY=1 keeps every cell on the tiled kernel (used to cross-check the two paths).
    const char* tiled_only = std::getenv("FDFK_TILED_ONLY");
    const bool march = p->norder <= kMarchMaxOrder && p->nz >= 2 * p->norder + 1 && !(tiled_only && tiled_only[0] == '1');
    s->ldz = plane_ldz(p->nz, p->npml, p->norder, march, s->izt);
    const size_t n = (size_t)s->ldz * s->NX;

    auto alloc = [&](void** ptr, size_t bytes) -> int {
        if (bytes == 0) { *ptr = nullptr; return FDFK_OK; }
        cudaError_t e = cudaMalloc(ptr, bytes);
        if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? FDFK_ENOMEM : FDFK_ECUDA,
                                          std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return FDFK_OK;
    };
#define AL(ptr, bytes) do { int r_ = alloc((void**)&(ptr), (bytes)); if (r_) { free_session(s); return r_; } } while (0)
    AL(s->kdt2, n * sizeof(float));
    AL(s->lam, n * sizeof(float));
    AL(s->mu, n * sizeof(float));
    for (int l = 0; l < 2; ++l) { AL(s->ux[l], n * sizeof(float)); AL(s->uz[l], n * sizeof(float)); }
    if (march) { AL(s->fux, n * sizeof(float)); AL(s->fuz, n * sizeof(float)); }
    const int nbu = p->is_PML_top ? 24 : 18;   // l, r, b, and t with the absorbing layer on top
    for (int k = 0; k < nbu; ++k)
        for (int l = 0; l < 2; ++l) AL(s->bu[k][l], bu_elems(*p, k) * sizeof(float));
    for (int k = 0; k < 12; ++k)
        if (k < 4 || k >= 8 || p->is_PML_top) AL(s->bp[k], bp_elems(*p, k) * sizeof(float));
    AL(s->dampx, s->NX * sizeof(DampCol));
    AL(s->dampz, s->rows * sizeof(DampCol));
    for (int k = 0; k < NSTRIP; ++k) AL(s->strip[k], strip_elems(*p, k) * (size_t)(p->nt + 1) * sizeof(float));
#undef AL
    s->have_bg.assign(p->nt + 1, 0);

    cudaError_t e = ensure_coefficients();
    if (e != cudaSuccess) { free_session(s); return fail(FDFK_ECUDA, std::string("coefficients: ") + cudaGetErrorString(e)); }

    // Nothing below waits for other work on the device: the copies from pageable host memory are
    // staged before each call returns, and the material conversion runs on its own stream.
    std::vector<DampCol> dx, dz;
    damping(*p, dx, dz);
    if ((rc = upload_material(s, c, true)) != FDFK_OK) { free_session(s); return rc; }
    if (cudaMemcpyAsync(s->dampx, dx.data(), dx.size() * sizeof(DampCol), cudaMemcpyHostToDevice, s->stream) != cudaSuccess ||
        cudaMemcpyAsync(s->dampz, dz.data(), dz.size() * sizeof(DampCol), cudaMemcpyHostToDevice, s->stream) != cudaSuccess) {
        free_session(s);
        return fail(FDFK_ECUDA, "damping upload failed");
    }
    if ((rc = zero_state(s)) != FDFK_OK) { free_session(s); return rc; }

    StepArgs& a = s->base;
    a.nx = p->nx; a.nz = p->nz; a.npml = p->npml; a.norder = p->norder; a.nbd = p->nbd;
    a.NZ = s->NZ; a.NX = s->NX; a.ldz = s->ldz;
    a.izt = s->izt; a.zorg = s->zorg;
    a.dx = p->dx; a.dz = p->dz;
    a.dx2r = (float)(1.0 / (double)(p->dx * p->dx));
    a.dx2p = 1.0f / (p->dx * p->dx);
    a.dz2 = 1.0f / (p->dz * p->dz);
    a.dt = (float)p->dt;
    a.kdt2 = s->kdt2; a.lam = s->lam; a.mu = s->mu;
    a.dampx = s->dampx; a.dampz = s->dampz;
    for (int k = 0; k < NSTRIP; ++k) a.strip[k] = s->strip[k];
    a.fux = s->fux; a.fuz = s->fuz;
    // Interior rows from 2*norder+1 down go to the marching fast path (orders <= kMarchMaxOrder): below
    // them every stencil has its full order.
    a.int_rows = march ? 2 * p->norder : p->nz;
    s->march.z0 = 2 * p->norder + 1;
    s->march.band_out = 64 - 4 * p->norder;
    s->march.n_bands = march ? (p->nz - 2 * p->norder + s->march.band_out - 1) / s->march.band_out : 0;
    // segments: about two waves of resident warps, so that the hardware block scheduler evens out
    // the per-SM progress, with 16..48 columns per segment (a segment re-primes its pipeline over
    // 3*norder-1 columns)
    s->march.seg_len = kMarchSeg;
    s->march.n_segs = march ? (p->nx + kMarchSeg - 1) / kMarchSeg : 0;
    if (march) {
        const int slots = march_warp_slots(p->norder);
        if (slots > 0) {
            const long long work = (long long)p->nx * s->march.n_bands;
            int len = (int)((work + 2LL * slots - 1) / (2LL * slots));
            len = len < 16 ? 16 : len > 48 ? 48 : len;
            // whole waves only: a few blocks left over would run alone at the end of the step
            while (len < 48 && (long long)((p->nx + len - 1) / len) * s->march.n_bands > 2LL * slots) ++len;
            s->march.seg_len = len;
            s->march.n_segs = (p->nx + len - 1) / len;
        }
        // FDFK_MARCH_SEGLEN=<columns> overrides the segment length (tuning)
        if (const char* sl = std::getenv("FDFK_MARCH_SEGLEN")) {
            const int v = std::atoi(sl);
            if (v >= 8) {
                s->march.seg_len = v;
                s->march.n_segs = (p->nx + v - 1) / v;
            }
        }
    }
    if (march) {
        cudaError_t e1 = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
        cudaError_t e2 = cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
        cudaError_t e3 = cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming);
        if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
            free_session(s);
            return fail(FDFK_ECUDA, "stream/event creation failed");
        }
    }
    plan_tiles(a, march);
    *out = s;
    return FDFK_OK;
}

int fdfk_session_set_stream(fdfk_session* s, void* stream)
{
    if (!s) return fail(FDFK_EINVAL, "session is NULL");
    const cudaStream_t ns = (cudaStream_t)stream;
    if (ns != s->stream) {
        // work already queued on the old stream (the state cleared at creation, uploads) comes first
        cudaEvent_t ev = nullptr;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        cudaError_t e = cudaEventRecord(ev, s->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ns, ev, 0);
        cudaEventDestroy(ev);
        if (e != cudaSuccess) return fail(FDFK_ECUDA, std::string("set_stream: ") + cudaGetErrorString(e));
    }
    s->stream = ns;
    return FDFK_OK;
}

int fdfk_session_upload_background(fdfk_session* s, const float* const strips[12], int t0, int count)
{
    if (s && s->batch) return fail(FDFK_ESTATE, "the session is a member of a batch");
    if (!s || !strips) return fail(FDFK_EINVAL, "NULL argument");
    if (t0 < 0 || count < 0 || t0 + count > s->p.nt + 1) return fail(FDFK_EINVAL, "time range outside 0..nt");
    for (int k = 0; k < NSTRIP; ++k) {
        if (!strips[k]) return fail(FDFK_EINVAL, "strip array is NULL");
        const size_t per = strip_elems(s->p, k);
        CK(cudaMemcpyAsync(s->strip[k] + per * t0, strips[k] + per * t0, per * (size_t)count * sizeof(float),
                           cudaMemcpyHostToDevice, s->stream));
    }
    for (int t = t0; t < t0 + count; ++t) s->have_bg[t] = 1;
    return FDFK_OK;
}

int fdfk_session_set_receivers(fdfk_session* s, int nrcv, const float* rx, const float* rz, float x0, float z0,
                               int nstp, int nsis)
{
    if (s && s->batch) return fail(FDFK_ESTATE, "the session is a member of a batch");
    if (!s) return fail(FDFK_EINVAL, "session is NULL");
    if (nrcv < 0 || (nrcv > 0 && (!rx || !rz)) || nstp < 1 || nsis < 0) return fail(FDFK_EINVAL, "bad receiver arguments");
    const float xmax = x0 + (s->p.nx - 1) * s->p.dx, zmax = z0 + (s->p.nz - 1) * s->p.dz;
    for (int r = 0; r < nrcv; ++r)
        if (rx[r] < x0 || rx[r] > xmax || rz[r] < z0 || rz[r] > zmax)
            return fail(FDFK_EINVAL, "receiver " + std::to_string(r + 1) + " lies outside the model");
    cudaFree(s->rx); cudaFree(s->rz); cudaFree(s->rsite); cudaFree(s->rw); cudaFree(s->seisx); cudaFree(s->seisz);
    s->rx = s->rz = s->seisx = s->seisz = nullptr;
    s->rsite = nullptr;
    s->rw = nullptr;
    s->nrcv = nrcv; s->nstp = nstp; s->nsis = nsis; s->x0 = x0; s->z0 = z0;
    if (nrcv > 0) {
        const size_t ns = (size_t)(nsis + 1) * nrcv;
        CK(cudaMalloc((void**)&s->rx, nrcv * sizeof(float)));
        CK(cudaMalloc((void**)&s->rz, nrcv * sizeof(float)));
        CK(cudaMalloc((void**)&s->seisx, ns * sizeof(float)));
        CK(cudaMalloc((void**)&s->seisz, ns * sizeof(float)));
        CK(cudaMemcpyAsync(s->rx, rx, nrcv * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->rz, rz, nrcv * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemsetAsync(s->seisx, 0, ns * sizeof(float), s->stream));
        CK(cudaMemsetAsync(s->seisz, 0, ns * sizeof(float), s->stream));
        CK(cudaMalloc((void**)&s->rsite, nrcv * sizeof(int4)));
        CK(cudaMalloc((void**)&s->rw, (size_t)nrcv * 49 * sizeof(double)));
        CK(fdfk::launch_receiver_sites(s->base, nrcv, x0, z0, s->rx, s->rz, s->rsite, s->rw, s->stream));
        fdfk::count_launches(1);
        // no wait: copies from pageable memory are staged before the call returns, and everything
        // that reads these arrays is ordered after them on the session's stream (a batch waits for
        // the stream when the session joins), so an FK background still running is not waited for
    }
    // the sampling clock restarts with the loop (src/FDFK2D.f90:315-316)
    s->isis = s->istp * nstp;
    return FDFK_OK;
}

int fdfk_session_advance(fdfk_session* s, int nsteps)
{
    if (!s) return fail(FDFK_EINVAL, "session is NULL");
    if (s->batch) return fail(FDFK_ESTATE, "the session is a member of a batch; advance the batch");
    if (nsteps < 0) return fail(FDFK_EINVAL, "nsteps must be >= 0");
    if (s->it + nsteps > s->p.nt + 1) return fail(FDFK_EINVAL, "advance past the last time index nt");
    for (int k = 0; k < nsteps; ++k) {
        const int it = s->it;
        if (!s->have_bg[it]) return fail(FDFK_ESTATE, "no background uploaded for time index " + std::to_string(it));
        StepArgs a = s->base;
        for (int l = 0; l < 2; ++l) { a.ux[l] = s->ux[l]; a.uz[l] = s->uz[l]; }
        for (int q = 0; q < 24; ++q) for (int l = 0; l < 2; ++l) a.bu[q][l] = s->bu[q][l];
        for (int q = 0; q < 12; ++q) a.bp[q] = s->bp[q];
        a.it = it;
        a.cur = s->cur;
        a.nrcv = 0;
        if (s->nrcv > 0 && s->isis == it && s->istp <= s->nsis) {
            a.nrcv = s->nrcv;
            a.sample_index = s->istp;
            a.nsamp = s->nsis + 1;
            a.x0 = s->x0; a.z0 = s->z0;
            a.rx = s->rx; a.rz = s->rz;
            a.rsite = s->rsite; a.rw = s->rw;
            a.seisx = s->seisx; a.seisz = s->seisz;
            s->istp += 1;
            s->isis += s->nstp;
        }
        if (s->march.n_bands > 0) {
            // The two kernels write disjoint cells and read only u^n: run the tiled one (top band,
            // PML, receivers) on a side stream next to the interior fast path.
            CK(cudaEventRecord(s->fork, s->stream));
            CK(cudaStreamWaitEvent(s->side, s->fork, 0));
            int nl = 0;
            cudaError_t e = launch_edge(s, a, s->side, &nl);
            if (e != cudaSuccess) return fail(FDFK_ECUDA, std::string("step launch: ") + cudaGetErrorString(e));
            e = launch_march(a, s->march, s->stream);
            if (e != cudaSuccess) return fail(FDFK_ECUDA, std::string("march launch: ") + cudaGetErrorString(e));
            CK(cudaEventRecord(s->join, s->side));
            CK(cudaStreamWaitEvent(s->stream, s->join, 0));
            g_launches.fetch_add(nl + 2);
        } else {
            cudaError_t e = launch_step(a, s->stream);
            if (e != cudaSuccess) return fail(FDFK_ECUDA, std::string("step launch: ") + cudaGetErrorString(e));
            g_launches.fetch_add(1);
        }
        if (s->izt != 1) {
            // the top absorbing layer after the interior update, whose new values it reads
            cudaError_t e = launch_step_top(a, s->stream);
            if (e != cudaSuccess) return fail(FDFK_ECUDA, std::string("top-layer launch: ") + cudaGetErrorString(e));
            g_launches.fetch_add(1);
        }
        s->cur ^= 1;
        s->it += 1;
    }
    return FDFK_OK;
}

int fdfk_session_advance_timed(fdfk_session* s, int nsteps, int sample_every, float* ms_interior, float* ms_edge,
                               float* ms_total)
{
    if (!s || !ms_interior || !ms_edge) return fail(FDFK_EINVAL, "NULL argument");
    if (sample_every < 1) return fail(FDFK_EINVAL, "sample_every must be at least 1");
    if (s->batch) return fail(FDFK_ESTATE, "the session is a member of a batch; advance the batch");
    *ms_interior = 0.f;
    *ms_edge = 0.f;
    if (ms_total) *ms_total = 0.f;
    if (nsteps <= 0) return fdfk_session_advance(s, nsteps);
    const bool two = s->march.n_bands > 0;
    // all events exist before the first step is queued, so their creation is not timed
    std::vector<cudaEvent_t> ev((size_t)nsteps * 4 + 2, nullptr);
    auto cleanup = [&]() { for (auto e : ev) if (e) cudaEventDestroy(e); };
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) { cleanup(); return fail(FDFK_ECUDA, "event creation failed"); }
    cudaEvent_t t_begin = ev[(size_t)nsteps * 4], t_end = ev[(size_t)nsteps * 4 + 1];
    cudaEventRecord(t_begin, s->stream);
    for (int k = 0; k < nsteps; ++k) {
        const int it = s->it;
        if (it > s->p.nt) { cleanup(); return fail(FDFK_EINVAL, "advance past the last time index nt"); }
        if (!s->have_bg[it]) { cleanup(); return fail(FDFK_ESTATE, "no background uploaded for time index " + std::to_string(it)); }
        StepArgs a = s->base;
        for (int l = 0; l < 2; ++l) { a.ux[l] = s->ux[l]; a.uz[l] = s->uz[l]; }
        for (int q = 0; q < 24; ++q) for (int l = 0; l < 2; ++l) a.bu[q][l] = s->bu[q][l];
        for (int q = 0; q < 12; ++q) a.bp[q] = s->bp[q];
        a.it = it;
        a.cur = s->cur;
        a.nrcv = 0;
        if (s->nrcv > 0 && s->isis == it && s->istp <= s->nsis) {
            a.nrcv = s->nrcv; a.sample_index = s->istp; a.nsamp = s->nsis + 1;
            a.x0 = s->x0; a.z0 = s->z0; a.rx = s->rx; a.rz = s->rz; a.seisx = s->seisx; a.seisz = s->seisz;
            a.rsite = s->rsite; a.rw = s->rw;
            s->istp += 1;
            s->isis += s->nstp;
        }
        // the kernels of every sample_every-th step are bracketed by event pairs
        const bool sampled = k % sample_every == 0;
        cudaEvent_t* e = &ev[(size_t)k * 4];
        cudaStream_t edge = two ? s->side : s->stream;
        if (two) {
            cudaEventRecord(s->fork, s->stream);
            cudaStreamWaitEvent(s->side, s->fork, 0);
        }
        if (sampled) cudaEventRecord(e[2], edge);
        int nl = 0;
        cudaError_t r = launch_edge(s, a, edge, &nl);
        if (sampled) cudaEventRecord(e[3], edge);
        if (r == cudaSuccess && two) {
            // e[0] .. e[1] brackets the fast-path kernel alone (the frame kernel runs before e[0])
            r = launch_march_marked(a, s->march, s->stream, sampled ? e[0] : nullptr);
            if (sampled) cudaEventRecord(e[1], s->stream);
            cudaEventRecord(s->join, s->side);
            cudaStreamWaitEvent(s->stream, s->join, 0);
        }
        if (r == cudaSuccess && s->izt != 1) {   // the top absorbing layer after the interior update
            r = launch_step_top(a, s->stream);
            nl += 1;
        }
        if (r != cudaSuccess) { cleanup(); return fail(FDFK_ECUDA, std::string("launch: ") + cudaGetErrorString(r)); }
        g_launches.fetch_add(nl + (two ? 2 : 0));
        s->cur ^= 1;
        s->it += 1;
    }
    cudaEventRecord(t_end, s->stream);
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) { cleanup(); return fail(FDFK_ECUDA, "synchronize failed"); }
    if (ms_total) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, t_begin, t_end) == cudaSuccess) *ms_total = t;
    }
    double ti = 0.0, te = 0.0;
    int ns = 0;
    for (int k = 0; k < nsteps; k += sample_every) {
        float t = 0.f;
        if (two && cudaEventElapsedTime(&t, ev[(size_t)k * 4], ev[(size_t)k * 4 + 1]) == cudaSuccess) ti += t;
        if (cudaEventElapsedTime(&t, ev[(size_t)k * 4 + 2], ev[(size_t)k * 4 + 3]) == cudaSuccess) te += t;
        ++ns;
    }
    cleanup();
    *ms_interior = (float)(ti / ns);
    *ms_edge = (float)(te / ns);
    return FDFK_OK;
}

int fdfk_session_interior_cells(const fdfk_session* s, long long* interior, long long* edge)
{
    if (!s || !interior || !edge) return fail(FDFK_EINVAL, "NULL argument");
    const long long total = (long long)s->rows * s->NX;
    *interior = s->march.n_bands > 0 ? (long long)(s->p.nz - 2 * s->p.norder) * s->p.nx : 0;
    *edge = total - *interior;
    return FDFK_OK;
}

int fdfk_session_step_index(const fdfk_session* s) { return s ? s->it : FDFK_EINVAL; }

int fdfk_session_synchronize(fdfk_session* s)
{
    if (s && s->batch) {
        const int rb = fdfk_batch_synchronize(s->batch);
        if (rb) return rb;
    }
    if (!s) return fail(FDFK_EINVAL, "session is NULL");
    CK(cudaStreamSynchronize(s->stream));
    return FDFK_OK;
}

int fdfk_session_download_seismograms(fdfk_session* s, float* seisx, float* seisz)
{
    if (s && s->batch) {
        const int rb = fdfk_batch_synchronize(s->batch);
        if (rb) return rb;
    }
    if (!s || !seisx || !seisz) return fail(FDFK_EINVAL, "NULL argument");
    if (s->nrcv == 0) return FDFK_OK;
    const size_t ns = (size_t)(s->nsis + 1) * s->nrcv;
    CK(cudaMemcpyAsync(seisx, s->seisx, ns * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(seisz, s->seisz, ns * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FDFK_OK;
}

int fdfk_session_download_seismogram_range(fdfk_session* s, int first, int count, float* seisx, float* seisz)
{
    if (s && s->batch) {
        const int rb = fdfk_batch_synchronize(s->batch);
        if (rb) return rb;
    }
    if (!s || !seisx || !seisz) return fail(FDFK_EINVAL, "NULL argument");
    if (first < 0 || count < 0 || first + count > s->nsis + 1) return fail(FDFK_EINVAL, "sample range outside 0..nsis");
    if (s->nrcv == 0 || count == 0) return FDFK_OK;
    const size_t pitch = (size_t)(s->nsis + 1) * sizeof(float);
    CK(cudaMemcpy2DAsync(seisx, count * sizeof(float), s->seisx + first, pitch, count * sizeof(float), s->nrcv,
                         cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpy2DAsync(seisz, count * sizeof(float), s->seisz + first, pitch, count * sizeof(float), s->nrcv,
                         cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FDFK_OK;
}

int fdfk_session_upload_state(fdfk_session* s, const float* ux, const float* uz, const float* const bp[12],
                              const float* const bu[24], int it)
{
    if (s && s->batch) return fail(FDFK_ESTATE, "the session is a member of a batch");
    if (!s || !ux || !uz || !bp || !bu) return fail(FDFK_EINVAL, "NULL argument");
    if (it < 0 || it > s->p.nt + 1) return fail(FDFK_EINVAL, "it outside 0..nt+1");
    const size_t n = (size_t)s->ldz * s->NX;
    std::vector<float> lv[4];
    for (auto& v : lv) v.assign(n, 0.f);
    const int zoff = s->izt - s->zorg;   // plane row of grid row izt
    for (int x = 0; x < s->NX; ++x)
        for (int z = 0; z < s->rows; ++z) {
            size_t src = 2 * ((size_t)z + (size_t)s->rows * x), dst = (size_t)(z + zoff) + (size_t)s->ldz * x;
            lv[0][dst] = ux[src]; lv[1][dst] = ux[src + 1];
            lv[2][dst] = uz[src]; lv[3][dst] = uz[src + 1];
        }
    s->cur = 0;
    CK(cudaMemcpyAsync(s->ux[0], lv[0].data(), n * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->ux[1], lv[1].data(), n * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->uz[0], lv[2].data(), n * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->uz[1], lv[3].data(), n * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    for (int k = 0; k < 12; ++k) {
        if (!s->bp[k]) continue;
        if (!bp[k]) return fail(FDFK_EINVAL, "bp array is NULL");
        CK(cudaMemcpyAsync(s->bp[k], bp[k], bp_elems(s->p, k) * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    }
    std::vector<float> pl[2];
    for (int k = 0; k < 24; ++k) {
        if (!s->bu[k][0]) continue;
        if (!bu[k]) return fail(FDFK_EINVAL, "bu array is NULL");
        const size_t m = bu_elems(s->p, k);
        pl[0].resize(m); pl[1].resize(m);
        for (size_t i = 0; i < m; ++i) { pl[0][i] = bu[k][2 * i]; pl[1][i] = bu[k][2 * i + 1]; }
        CK(cudaMemcpyAsync(s->bu[k][0], pl[0].data(), m * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        CK(cudaMemcpyAsync(s->bu[k][1], pl[1].data(), m * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    s->it = it;
    s->istp = 0;
    s->isis = 0;
    return FDFK_OK;
}

int fdfk_session_download_state(fdfk_session* s, float* ux, float* uz, float* const bp[12], float* const bu[24])
{
    if (s && s->batch) {
        const int rb = fdfk_batch_synchronize(s->batch);
        if (rb) return rb;
    }
    if (!s || !ux || !uz || !bp || !bu) return fail(FDFK_EINVAL, "NULL argument");
    const size_t n = (size_t)s->ldz * s->NX;
    std::vector<float> lv[4];
    for (auto& v : lv) v.resize(n);
    const int c = s->cur, o = c ^ 1;
    CK(cudaMemcpyAsync(lv[0].data(), s->ux[c], n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(lv[1].data(), s->ux[o], n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(lv[2].data(), s->uz[c], n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(lv[3].data(), s->uz[o], n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const int npml = s->p.npml, nx = s->p.nx;
    const int zoff = s->izt - s->zorg;   // plane row of grid row izt
    for (int x = 0; x < s->NX; ++x)
        for (int z = 0; z < s->rows; ++z) {
            size_t dst = 2 * ((size_t)z + (size_t)s->rows * x), src = (size_t)(z + zoff) + (size_t)s->ldz * x;
            const int ix = x + 1 - npml, iz = z + s->izt;
            // the outer frame is never advanced: its level 2 is left as the caller holds it
            const bool frame = ix == 1 - npml || ix == nx + npml || iz == s->NZ || (s->izt != 1 && iz == s->izt);
            ux[dst] = lv[0][src];
            uz[dst] = lv[2][src];
            if (!frame) { ux[dst + 1] = lv[1][src]; uz[dst + 1] = lv[3][src]; }
        }
    for (int k = 0; k < 12; ++k) {
        if (!s->bp[k]) continue;
        if (!bp[k]) return fail(FDFK_EINVAL, "bp array is NULL");
        CK(cudaMemcpyAsync(bp[k], s->bp[k], bp_elems(s->p, k) * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    }
    std::vector<float> pl[2];
    for (int k = 0; k < 24; ++k) {
        if (!s->bu[k][0]) continue;
        if (!bu[k]) return fail(FDFK_EINVAL, "bu array is NULL");
        const size_t m = bu_elems(s->p, k);
        pl[0].resize(m); pl[1].resize(m);
        CK(cudaMemcpyAsync(pl[0].data(), s->bu[k][c], m * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaMemcpyAsync(pl[1].data(), s->bu[k][o], m * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        // cells on the outer frame are never advanced: both levels stay as the caller holds them
        const bool sidearr = k < 12;
        const int n1 = sidearr ? s->p.nz : npml, n2 = sidearr ? npml : s->NX;
        for (int j = 0; j < n2; ++j)
            for (int r = 0; r < n1; ++r) {
                bool frame;
                if (sidearr) frame = (k < 6) ? j == 0 : j == npml - 1;
                else frame = (k < 18 ? r == npml - 1 : r == 0) || j == 0 || j == s->NX - 1;   // b / t
                if (frame) continue;
                const size_t i = (size_t)r + (size_t)n1 * j;
                bu[k][2 * i] = pl[0][i];
                bu[k][2 * i + 1] = pl[1][i];
            }
    }
    CK(cudaStreamSynchronize(s->stream));
    return FDFK_OK;
}

int fdfk_session_set_tuning(fdfk_session* s, int seg_len, int pml_run)
{
    if (!s) return fail(FDFK_EINVAL, "session is NULL");
    if (s->batch) return fail(FDFK_ESTATE, "the session is a member of a batch");
    if ((seg_len != 0 && (seg_len < 8 || seg_len > 1024)) || (pml_run != 0 && (pml_run < 8 || pml_run > 64)))
        return fail(FDFK_EINVAL, "segment length must be 8..1024 and tile length 8..64 (0 keeps the current)");
    if (pml_run) {
        // the tiles of that length must fit one block's shared memory (high orders, long runs)
        StepArgs trial = s->base;
        plan_tiles(trial, s->march.n_bands > 0, pml_run);
        int dev = 0, optin = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        if (step_smem_for(trial) > (size_t)optin)
            return fail(FDFK_EINVAL, "tile length " + std::to_string(pml_run) + " needs more shared memory than a block has");
        s->pml_run = pml_run;
        s->base = trial;
    }
    if (seg_len && s->march.n_bands > 0) {
        s->march.seg_len = seg_len;
        s->march.n_segs = (s->p.nx + seg_len - 1) / seg_len;
    }
    return FDFK_OK;
}

int fdfk_session_get_tuning(const fdfk_session* s, int* seg_len, int* pml_run)
{
    if (!s || !seg_len || !pml_run) return fail(FDFK_EINVAL, "NULL argument");
    *seg_len = s->march.n_bands > 0 ? s->march.seg_len : 0;
    *pml_run = s->pml_run;
    return FDFK_OK;
}

int fdfk_autotune(const fdfk_params* p, const float* c, int steps, int* seg_len, int* pml_run, float* ms_per_step)
{
    if (!p || !c || !seg_len || !pml_run || steps < 1) return fail(FDFK_EINVAL, "bad argument");
    const int runs[] = {12, 16, 24, 32, 48};
    std::vector<int> segs = {16, 24, 32, 48, 64, 96};
    // segment lengths (two passes: with the default and with the chosen absorbing-layer run), runs
    // in between; each candidate timed twice after two warm-up steps, the faster time kept; then
    // the three fastest shapes timed again in turn, three rounds, and the lowest total chosen (the
    // two kernels share the SMs, and a single short timing can misrank shapes a few percent apart)
    constexpr int kFinal = 3, kRounds = 3;
    // every timed window at least kWindowMs long (short windows of small models misrank shapes):
    // `steps` steps, or more (up to kMaxSteps) where a step is short; the scratch session's time
    // index restarts for every candidate, so its record covers one candidate's steps
    constexpr float kWindowMs = 4.0f;
    const int kMaxSteps = std::max(steps, 1000);
    fdfk_params q = *p;
    q.nt = 2 * kMaxSteps + 4;
    fdfk_session* s = nullptr;
    int rc = fdfk_session_create(&q, c, &s);
    if (rc) return rc;
    struct Guard {
        fdfk_session* s;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        ~Guard()
        {
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            fdfk_session_destroy(s);
        }
    } g{s};
    // a zero background: the timing of a step does not depend on the values
    for (int k = 0; k < NSTRIP; ++k)
        CK(cudaMemsetAsync(s->strip[k], 0, strip_elems(q, k) * (size_t)(q.nt + 1) * sizeof(float), s->stream));
    for (int t = 0; t <= q.nt; ++t) s->have_bg[t] = 1;
    CK(cudaEventCreate(&g.e0));
    CK(cudaEventCreate(&g.e1));
    int nsteps = steps;
    auto time_it = [&](int seg, int run, float& ms) -> int {
        int r = fdfk_session_set_tuning(s, seg, run);
        if (r) return r;
        s->it = 0;   // zero state and background: the values, and so the time index, do not matter
        if ((r = fdfk_session_advance(s, 2))) return r;   // warm-up (first launches of a shape)
        ms = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            float t = 0.f;
            CK(cudaEventRecord(g.e0, s->stream));
            if ((r = fdfk_session_advance(s, nsteps))) return r;
            CK(cudaEventRecord(g.e1, s->stream));
            CK(cudaEventSynchronize(g.e1));
            CK(cudaEventElapsedTime(&t, g.e0, g.e1));
            ms = std::min(ms, t / nsteps);
        }
        return FDFK_OK;
    };
    {   // the window length from one timing of the default shapes
        float ms0 = 0.f;
        if ((rc = time_it(0, 0, ms0))) return rc;
        if (ms0 * steps < kWindowMs)
            nsteps = std::min(kMaxSteps, (int)std::ceil(kWindowMs / std::max(ms0, 1e-4f)));
    }
    // plus the shortest segments that fill exactly one and two waves of resident fast-path warps
    // (a partly filled last wave leaves SMs idle at the end of the step)
    if (s->march.n_bands > 0) {
        const int slots = march_warp_slots(q.norder);
        for (int waves = 1; waves <= 2 && slots > 0; ++waves) {
            int len = 16;
            while (len < 1024 && (long long)((q.nx + len - 1) / len) * s->march.n_bands > (long long)waves * slots) ++len;
            if (std::find(segs.begin(), segs.end(), len) == segs.end()) segs.push_back(len);
        }
    }
    int best_seg = s->march.n_bands > 0 ? s->march.seg_len : 0, best_run = s->pml_run;
    float best = 1e30f, ms = 0.f;
    struct Shape {
        int seg, run;
        float ms;
    };
    std::vector<Shape> seen;
    auto note = [&](int seg, int run, float t) {
        for (Shape& v : seen)
            if (v.seg == seg && v.run == run) {
                v.ms = std::min(v.ms, t);
                return;
            }
        seen.push_back({seg, run, t});
    };
    if (s->march.n_bands > 0)
        for (int seg : segs) {
            if ((rc = time_it(seg, best_run, ms))) return rc;
            note(seg, best_run, ms);
            if (ms < best) { best = ms; best_seg = seg; }
        }
    for (int run : runs) {
        if ((rc = time_it(best_seg, run, ms))) {
            if (rc == FDFK_EINVAL) continue;          // tiles too large for this order: not a candidate
            return rc;
        }
        note(best_seg, run, ms);
        if (ms < best) { best = ms; best_run = run; }
    }
    if (s->march.n_bands > 0)
        for (int seg : segs) {
            if ((rc = time_it(seg, best_run, ms))) return rc;
            note(seg, best_run, ms);
            if (ms < best) { best = ms; best_seg = seg; }
        }
    std::sort(seen.begin(), seen.end(), [](const Shape& x, const Shape& y) { return x.ms < y.ms; });
    if (seen.size() > (size_t)kFinal) seen.resize(kFinal);
    std::vector<float> total(seen.size(), 0.f);
    for (int round = 0; round < kRounds && seen.size() > 1; ++round)
        for (size_t i = 0; i < seen.size(); ++i) {
            if ((rc = time_it(seen[i].seg, seen[i].run, ms))) return rc;
            total[i] += ms;
        }
    if (seen.size() > 1) {
        size_t w = 0;
        for (size_t i = 1; i < seen.size(); ++i)
            if (total[i] < total[w]) w = i;
        best_seg = seen[w].seg;
        best_run = seen[w].run;
        best = total[w] / kRounds;
    }
    *seg_len = best_seg;
    *pml_run = best_run;
    if (ms_per_step) *ms_per_step = best;
    return FDFK_OK;
}

int fdfk_session_snapshot(fdfk_session* s, float* ux, float* uz)
{
    if (!s || !ux || !uz) return fail(FDFK_EINVAL, "NULL argument");
    if (s->batch) {
        const int rb = fdfk_batch_synchronize(s->batch);
        if (rb) return rb;
    }
    // level 2 = the plane not holding u^n; rows 1..nz of columns 1..nx
    const int o = s->cur ^ 1;
    const size_t first = (size_t)s->ldz * s->p.npml + (size_t)(1 - s->zorg);
    const size_t pitch = (size_t)s->ldz * sizeof(float);
    CK(cudaMemcpy2DAsync(ux, s->p.nz * sizeof(float), s->ux[o] + first, pitch, s->p.nz * sizeof(float), s->p.nx,
                         cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpy2DAsync(uz, s->p.nz * sizeof(float), s->uz[o] + first, pitch, s->p.nz * sizeof(float), s->p.nx,
                         cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return FDFK_OK;
}

void fdfk_session_destroy(fdfk_session* s)
{
    if (s && s->batch) fdfk_batch_remove(s->batch, s);
    if (s && s->stream) cudaStreamSynchronize(s->stream);
    free_session(s);
}

int fdfk_simulate(const fdfk_params* p, const float* c, const float* const strips[12], int nrcv, const float* rx,
                  const float* rz, float x0, float z0, int nstp, int nsis, float* seisx, float* seisz)
{
    fdfk_session* s = nullptr;
    int rc = fdfk_session_create(p, c, &s);
    if (rc) return rc;
    if ((rc = fdfk_session_upload_background(s, strips, 0, p->nt + 1)) ||
        (rc = fdfk_session_set_receivers(s, nrcv, rx, rz, x0, z0, nstp, nsis)) ||
        (rc = fdfk_session_advance(s, p->nt + 1)) ||
        (rc = fdfk_session_download_seismograms(s, seisx, seisz))) {
        fdfk_session_destroy(s);
        return rc;
    }
    fdfk_session_destroy(s);
    return FDFK_OK;
}

// ---------------------------------------------------------------------------
// FK background
// ---------------------------------------------------------------------------
static int fk_job(const fdfk_fk_params* p, const double* bazs, int nll, const float* fkl, int nlr,
                  const float* fkr, FkJob& J)
{
    if (!p || !bazs || !fkl || !fkr) return fail(FDFK_EINVAL, "NULL argument");
    // the strips do not depend on izt (the grid's top row): the shipped library gives the same
    // background for the free-surface and the absorbing-layer-on-top modes
    if (p->izt > 1 || p->izt < 1 - p->npml) return fail(FDFK_EINVAL, "FK: izt must be 1 or 1 - npml");
    if (p->nx < 1 || p->nbd < 1 || p->nz <= p->nbd || p->npml < p->nbd || p->nt < 1 || !(p->dt > 0.0) ||
        !(p->dx > 0.f) || !(p->dz > 0.f))
        return fail(FDFK_EINVAL, "FK: need nx >= 1, nz > nbd >= 1, npml >= nbd, nt >= 1 and positive dt, dx, dz");
    if (nll < 1 || nlr < 1 || nll > kFkMaxLayers || nlr > kFkMaxLayers)
        return fail(FDFK_EINVAL, "FK: layer count must be 1.." + std::to_string(kFkMaxLayers));
    J.nx = p->nx; J.nz = p->nz; J.npml = p->npml; J.nbd = p->nbd; J.nt = p->nt;
    J.p_wave = p->src_type != 0;
    J.x0 = p->x0; J.z0 = p->z0; J.dx = p->dx; J.dz = p->dz;
    J.dt = p->dt; J.ds = p->ds; J.f0 = p->f0; J.rayp = p->rayp;
    J.bazs = bazs;
    J.nlayer[0] = nll; J.nlayer[1] = nlr;
    J.model[0] = fkl; J.model[1] = fkr;
    return FDFK_OK;
}

int fdfk_session_fk_background(fdfk_session* s, const fdfk_fk_params* p, const double* bazs, int nlayer_left,
                               const float* fk_left, int nlayer_right, const float* fk_right)
{
    if (s && s->batch) return fail(FDFK_ESTATE, "the session is a member of a batch");
    if (!s) return fail(FDFK_EINVAL, "session is NULL");
    FkJob J{};
    int rc = fk_job(p, bazs, nlayer_left, fk_left, nlayer_right, fk_right, J);
    if (rc) return rc;
    if (p->nx != s->p.nx || p->nz != s->p.nz || p->npml != s->p.npml || p->nbd != s->p.nbd || p->nt != s->p.nt)
        return fail(FDFK_EINVAL, "FK geometry (nx, nz, npml, nbd, nt) differs from the session's");
    std::string err;
    long long nl = 0;
    rc = fk_background(J, s->strip, s->stream, err, &nl);
    g_launches += nl;
    if (rc) return fail(rc, err);
    for (int t = 0; t <= s->p.nt; ++t) s->have_bg[t] = 1;
    return FDFK_OK;
}

int fdfk_fk_background(const fdfk_fk_params* p, const double* bazs, int nlayer_left, const float* fk_left,
                       int nlayer_right, const float* fk_right, float* const strips[12])
{
    FkJob J{};
    int rc = fk_job(p, bazs, nlayer_left, fk_left, nlayer_right, fk_right, J);
    if (rc) return rc;
    if (!strips) return fail(FDFK_EINVAL, "NULL strips");
    for (int k = 0; k < NSTRIP; ++k)
        if (!strips[k]) return fail(FDFK_EINVAL, "strip array is NULL");
    float* d[NSTRIP] = {};
    size_t bytes[NSTRIP];
    auto release = [&]() {
        for (int k = 0; k < NSTRIP; ++k) cudaFree(d[k]);
    };
    for (int k = 0; k < NSTRIP; ++k) {
        bytes[k] = fk_strip_elems(p->nx, p->nz, p->nbd, k) * (size_t)(p->nt + 1) * sizeof(float);
        if (cudaMalloc((void**)&d[k], bytes[k]) != cudaSuccess) {
            release();
            return fail(FDFK_ENOMEM, "FK: cudaMalloc of the strips failed");
        }
    }
    std::string err;
    long long nl = 0;
    rc = fk_background(J, d, nullptr, err, &nl);
    g_launches += nl;
    if (rc) {
        release();
        return fail(rc, err);
    }
    for (int k = 0; k < NSTRIP; ++k) {
        const cudaError_t e = cudaMemcpy(strips[k], d[k], bytes[k], cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            release();
            return fail(FDFK_ECUDA, std::string("FK: copy of the strips failed: ") + cudaGetErrorString(e));
        }
    }
    release();
    return FDFK_OK;
}

void comput_background_wavefield_(const int* nx, const int* nz, const int* npml, const int* izt, const int* nbd,
                                  const int* nt, const int* nlayer_left, const int* nlayer_right,
                                  const int* src_type, const float* x0, const float* z0, const float* dx,
                                  const float* dz, const double* dt, const float* ds, const float* f0,
                                  const double* rayp, const double* bazs, const float* fk_left,
                                  const float* fk_right, float* uxl_reg, float* uzl_reg, float* uxr_reg,
                                  float* uzr_reg, float* uxb_reg, float* uzb_reg, float* uxl_pml, float* uzl_pml,
                                  float* uxr_pml, float* uzr_pml, float* uxb_pml, float* uzb_pml)
{
    fdfk_fk_params p{};
    p.nx = *nx; p.nz = *nz; p.npml = *npml; p.izt = *izt; p.nbd = *nbd; p.nt = *nt;
    p.src_type = *src_type ? 1 : 0;
    p.x0 = *x0; p.z0 = *z0; p.dx = *dx; p.dz = *dz; p.dt = *dt; p.ds = *ds; p.f0 = *f0; p.rayp = *rayp;
    float* const strips[12] = {uxl_reg, uzl_reg, uxr_reg, uzr_reg, uxb_reg, uzb_reg,
                               uxl_pml, uzl_pml, uxr_pml, uzr_pml, uxb_pml, uzb_pml};
    if (fdfk_fk_background(&p, bazs, *nlayer_left, fk_left, *nlayer_right, fk_right, strips)) {
        std::fprintf(stderr, "fdfk_gb300 comput_background_wavefield_: %s\n", g_err.c_str());
        std::abort();
    }
}

// ---------------------------------------------------------------------------
// Single step on the static scratch (no allocation)
// ---------------------------------------------------------------------------
int fdfk_step_noalloc(const fdfk_params* p, int it, const float* const strips[12], const float* c, float* ux,
                      float* uz, float* const bp[12], float* const bu[24], void* stream)
{
    int rc = validate(p);
    if (rc) return rc;
    if (!strips || !c || !ux || !uz || !bp || !bu) return fail(FDFK_EINVAL, "NULL argument");
    for (int k = 0; k < NSTRIP; ++k)
        if (!strips[k]) return fail(FDFK_EINVAL, "strip array is NULL");
    for (int k = 0; k < 12; ++k)
        if ((k < 4 || k >= 8) && !bp[k]) return fail(FDFK_EINVAL, "bp array is NULL");
    for (int k = 0; k < 18; ++k)
        if (!bu[k]) return fail(FDFK_EINVAL, "bu array is NULL");
    if (it < 0 || it > p->nt) return fail(FDFK_EINVAL, "it outside 0..nt");
    // the coefficient tables, once per device (later calls neither copy nor wait)
    const cudaError_t ce = ensure_coefficients();
    if (ce != cudaSuccess) return fail(FDFK_ECUDA, std::string("coefficient tables: ") + cudaGetErrorString(ce));
    std::string err;
    long long nl = 0;
    rc = step_noalloc(*p, it, strips, c, ux, uz, bp, bu, (cudaStream_t)stream, err, &nl);
    g_launches += nl;
    if (rc) return fail(rc, err);
    return FDFK_OK;
}

long long fdfk_step_noalloc_capacity(void) { return (long long)kNoAllocFloats; }

long long fdfk_step_noalloc_need(const fdfk_params* p)
{
    if (validate(p)) return -1;
    return (long long)noalloc_floats_needed(*p);
}

// ---------------------------------------------------------------------------
// gfortran-ABI drop-in
// ---------------------------------------------------------------------------
static fdfk_session* g_legacy = nullptr;
static std::mutex g_legacy_mu;

// True when the caller's coef0/coef1 (real(8) coef(norder, norder), src/Submain.f90:1111-1200:
// fd_coef0 staggered, fd_coef1 collocated, every reduced order) are the tables this library
// computes itself; the step uses its own tables, so different ones must not pass silently.
static bool caller_coefficients_match(int norder, const double* coef0, const double* coef1)
{
    for (int n = 1; n <= norder; ++n)
        for (int j = 1; j <= norder; ++j) {
            double st = 0.0, co = 0.0;
            if (j <= n) {
                double num = 1.0, den = 1.0, numc = 1.0, denc = 1.0;
                const double aj = (double)((2 * j - 1) * (2 * j - 1)), bj = (double)(j * j);
                for (int k = 1; k <= n; ++k) {
                    if (k == j) continue;
                    const double ak = (double)((2 * k - 1) * (2 * k - 1)), bk = (double)(k * k);
                    num *= ak;
                    den *= (k < j) ? (aj - ak) : (ak - aj);
                    numc *= bk;
                    denc *= (k < j) ? (bj - bk) : (bk - bj);
                }
                const double sgn = (j % 2 == 1) ? 1.0 : -1.0;
                st = sgn * num / (den * (double)(2 * j - 1));
                co = sgn * numc / (denc * 2.0 * (double)j);
            }
            const size_t i = (size_t)(j - 1) + (size_t)(n - 1) * (size_t)norder;
            if (std::fabs(coef0[i] - st) > 1e-12 * std::fabs(st) + 1e-300) return false;
            if (std::fabs(coef1[i] - co) > 1e-12 * std::fabs(co) + 1e-300) return false;
        }
    return true;
}

void updatedispl_(const int* norder, const int* nx, const int* nz, const int* npml, const int* izt,
                  const int* is_PML_top, const int* npower, const int* nbd, const int* it, const int* nt,
                  const float* dx, const float* dz, const double* dt, const float* vpml, const double* R0,
                  const float* uxl_reg, const float* uzl_reg, const float* uxr_reg, const float* uzr_reg,
                  const float* uxb_reg, const float* uzb_reg, const float* uxl_pml, const float* uzl_pml,
                  const float* uxr_pml, const float* uzr_pml, const float* uxb_pml, const float* uzb_pml,
                  const float* c, const double* coef0, const double* coef1, float* ux, float* uz,
                  float* bpxlx, float* bpzlx, float* bpxrx, float* bpzrx, float* bpxtx, float* bpxtz, float* bpztx,
                  float* bpztz, float* bpxbx, float* bpxbz, float* bpzbx, float* bpzbz,
                  float* bux1l, float* bux2l, float* bux3l, float* buz1l, float* buz2l, float* buz3l,
                  float* bux1r, float* bux2r, float* bux3r, float* buz1r, float* buz2r, float* buz3r,
                  float* bux1b, float* bux2b, float* bux3b, float* buz1b, float* buz2b, float* buz3b,
                  float* bux1t, float* bux2t, float* bux3t, float* buz1t, float* buz2t, float* buz3t)
{
    // one legacy session per process: calls from several host threads take turns
    std::lock_guard<std::mutex> lock(g_legacy_mu);
    fdfk_params p{};
    p.norder = *norder; p.nx = *nx; p.nz = *nz; p.npml = *npml; p.is_PML_top = *is_PML_top ? 1 : 0;
    p.npower = *npower; p.nbd = *nbd; p.nt = 0; p.dx = *dx; p.dz = *dz; p.dt = *dt; p.vpml = *vpml; p.R0 = *R0;
    auto die = [](const char* what) {
        std::fprintf(stderr, "fdfk_gb300 updatedispl_: %s (%s)\n", what, g_err.c_str());
        std::abort();
    };
    if (*izt != (p.is_PML_top ? 1 - p.npml : 1)) { g_err = "izt"; die("izt must be 1, or 1 - npml with is_PML_top"); }
    if (p.norder < 1 || p.norder > kMaxOrder) { g_err = "norder"; die("stencil order outside 1..8"); }
    if (!caller_coefficients_match(p.norder, coef0, coef1)) {
        g_err = "coef0/coef1";
        die("coef0/coef1 are not the fd_coef0/fd_coef1 tables of this order");
    }
    const bool same = g_legacy && std::memcmp(&g_legacy->p, &p, sizeof(p)) == 0;
    if (!same) {
        fdfk_session_destroy(g_legacy);
        g_legacy = nullptr;
        if (fdfk_session_create(&p, c, &g_legacy)) die("session create failed");
    } else if (upload_material(g_legacy, c, false)) {
        die("material upload failed");
    }
    // the strips of this call, time index *it, uploaded as time 0 of a one-sample session
    const float* all[12] = {uxl_reg, uzl_reg, uxr_reg, uzr_reg, uxb_reg, uzb_reg,
                            uxl_pml, uzl_pml, uxr_pml, uzr_pml, uxb_pml, uzb_pml};
    const float* at[12];
    for (int k = 0; k < 12; ++k) at[k] = all[k] + strip_elems(p, k) * (size_t)(*it);
    (void)nt;
    float* bp[12] = {bpxlx, bpzlx, bpxrx, bpzrx, bpxtx, bpxtz, bpztx, bpztz, bpxbx, bpxbz, bpzbx, bpzbz};
    float* bu[24] = {bux1l, bux2l, bux3l, buz1l, buz2l, buz3l, bux1r, bux2r, bux3r, buz1r, buz2r, buz3r,
                     bux1b, bux2b, bux3b, buz1b, buz2b, buz3b, bux1t, bux2t, bux3t, buz1t, buz2t, buz3t};
    if (fdfk_session_upload_background(g_legacy, at, 0, 1) ||
        fdfk_session_upload_state(g_legacy, ux, uz, bp, bu, 0) ||
        fdfk_session_advance(g_legacy, 1) ||
        fdfk_session_download_state(g_legacy, ux, uz, bp, bu))
        die("step failed");
}

}  // extern "C"
