// Batches: many solves (sessions of one stencil order, any grid sizes) advanced
// together.  Every step of the batch is the same few launches whatever the number
// of members (plus one for the top layers when a member has the absorbing layer
// on top): a one-thread-per-member bump kernel that writes each member's time
// index, plane parity and receiver sampling into its device-resident
// StepArgs, then the fast path and the tiled kernel over all members' blocks
// (two streams, as for one session).  The per-step kernels read everything
// that changes from device memory, so a chunk of steps is captured once into
// a CUDA graph and replayed until the membership changes.
#include "fdfk_gb300.h"
#include "fdfk_session.h"
#include "fdfk_sweep.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

using namespace fdfk;

namespace fdfk {
int march_warp_slots(int norder);
}

struct fdfk_batch {
    int norder = 0;
    std::vector<fdfk_session*> members;
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    // device tables (capacity cap members)
    int cap = 0;
    StepArgs* d_args = nullptr;
    MarchArgs* d_march = nullptr;
    BatchDyn* d_dyn = nullptr;
    int* d_live = nullptr;
    int* d_edge_off = nullptr;
    int* d_march_off = nullptr;
    int* d_frame_off = nullptr;
    int* d_top_off = nullptr;
    int edge_blocks = 0, march_blocks = 0, frame_blocks = 0, top_blocks = 0;
    size_t smem = 0;
    bool dirty = true;         // tables do not match the members
    bool in_flight = false;    // device state newer than the members' host state
    int chunk = 32;            // steps per captured graph (0: no graph)
    int seg_len = 0;           // fast-path segment columns for every member (0: planned for the batch)
    int pml_run = 0;           // absorbing-layer tile length for every member (0: each member's own)
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
};

namespace {

#define BK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return set_error(FDFK_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

void drop_graph(fdfk_batch* b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_steps = 0;
}

void free_tables(fdfk_batch* b)
{
    cudaFree(b->d_args); cudaFree(b->d_march); cudaFree(b->d_dyn); cudaFree(b->d_live);
    cudaFree(b->d_edge_off); cudaFree(b->d_march_off); cudaFree(b->d_frame_off); cudaFree(b->d_top_off);
    b->d_args = nullptr; b->d_march = nullptr; b->d_dyn = nullptr; b->d_live = nullptr;
    b->d_edge_off = nullptr; b->d_march_off = nullptr; b->d_frame_off = nullptr; b->d_top_off = nullptr;
    b->cap = 0;
}

BatchTab table(const fdfk_batch* b)
{
    BatchTab t{};
    t.n = (int)b->members.size();
    t.args = b->d_args;
    t.march = b->d_march;
    t.dyn = b->d_dyn;
    t.live = b->d_live;
    t.edge_off = b->d_edge_off;
    t.march_off = b->d_march_off;
    t.frame_off = b->d_frame_off;
    t.top_off = b->d_top_off;
    return t;
}

// Pull the device state of every member back into its session.
int pull(fdfk_batch* b)
{
    if (!b->in_flight) return FDFK_OK;
    BK(cudaStreamSynchronize(b->stream));
    const int n = (int)b->members.size();
    std::vector<BatchDyn> dyn(n);
    if (n) BK(cudaMemcpy(dyn.data(), b->d_dyn, n * sizeof(BatchDyn), cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; ++i) {
        fdfk_session* s = b->members[i];
        s->it = dyn[i].it;
        s->cur = dyn[i].cur;
        s->isis = dyn[i].isis;
        s->istp = dyn[i].istp;
    }
    b->in_flight = false;
    return FDFK_OK;
}

// Rebuild and upload the device tables from the members' host state.
int rebuild(fdfk_batch* b)
{
    const int n = (int)b->members.size();
    drop_graph(b);
    if (n > b->cap) {
        free_tables(b);
        const int cap = std::max(n, 2 * b->cap);
        cudaError_t e = cudaSuccess;
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_args, cap * sizeof(StepArgs));
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_march, cap * sizeof(MarchArgs));
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_dyn, cap * sizeof(BatchDyn));
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_live, cap * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_edge_off, (cap + 1) * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_march_off, (cap + 1) * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_frame_off, (cap + 1) * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_top_off, (cap + 1) * sizeof(int));
        if (e != cudaSuccess) {
            free_tables(b);
            return set_error(FDFK_ENOMEM, std::string("batch tables: ") + cudaGetErrorString(e));
        }
        b->cap = cap;
    }
    std::vector<StepArgs> args(n);
    std::vector<MarchArgs> march(n);
    std::vector<BatchDyn> dyn(n);
    std::vector<int> live(n, 0), eoff(n + 1, 0), moff(n + 1, 0), foff(n + 1, 0), toff(n + 1, 0);
    size_t smem = 0;
    // fast-path segments re-planned for the whole batch: about two waves of resident warps over
    // all members' work, 16..96 columns per segment (a member alone plans for itself only; longer
    // segments spend fewer columns re-priming the pipeline, but past two waves the last one runs
    // partly empty)
    long long work = 0;
    for (const fdfk_session* s : b->members) work += (long long)s->p.nx * s->march.n_bands;
    const int slots = b->norder <= kMarchMaxOrder ? march_warp_slots(b->norder) : 0;
    int seg = kMarchSeg;
    if (slots > 0) {
        seg = (int)((work + 2LL * slots - 1) / (2LL * slots));
        seg = seg < 16 ? 16 : seg > 96 ? 96 : seg;
    }
    if (b->seg_len > 0) seg = b->seg_len;
    for (int i = 0; i < n; ++i) {
        const fdfk_session* s = b->members[i];
        StepArgs a = s->base;
        if (b->pml_run > 0) {   // the batch's absorbing-layer tiles, where they fit a block
            StepArgs t = a;
            plan_tiles(t, s->march.n_bands > 0, b->pml_run);
            if (step_smem_for(t) <= (size_t)227 * 1024) a = t;
        }
        for (int l = 0; l < 2; ++l) { a.ux[l] = s->ux[l]; a.uz[l] = s->uz[l]; }
        for (int q = 0; q < 24; ++q) for (int l = 0; l < 2; ++l) a.bu[q][l] = s->bu[q][l];
        for (int q = 0; q < 12; ++q) a.bp[q] = s->bp[q];
        a.it = s->it;
        a.cur = s->cur;
        a.nrcv = 0;
        a.nsamp = s->nsis + 1;
        a.x0 = s->x0; a.z0 = s->z0;
        a.rx = s->rx; a.rz = s->rz;
        a.rsite = s->rsite; a.rw = s->rw;
        a.seisx = s->seisx; a.seisz = s->seisz;
        args[i] = a;
        MarchArgs m = s->march;
        if (m.n_bands > 0) {
            m.seg_len = seg;
            m.n_segs = (s->p.nx + seg - 1) / seg;
        }
        march[i] = m;
        BatchDyn d{};
        d.it = s->it; d.nt = s->p.nt; d.cur = s->cur;
        d.nrcv = s->nrcv; d.nstp = s->nstp; d.nsis = s->nsis; d.isis = s->isis; d.istp = s->istp;
        d.live = s->it <= s->p.nt;
        dyn[i] = d;
        const int nsb = sample_blocks(s->nrcv);
        eoff[i + 1] = eoff[i] + a.n_tiles + nsb;
        moff[i + 1] = moff[i] + (m.n_bands * m.n_segs + 3) / 4;
        foff[i + 1] = foff[i] + (m.n_bands > 0 ? frame_blocks(a) : 0);
        toff[i + 1] = toff[i] + (a.izt != 1 ? a.tiles_t_z * a.tiles_t_x : 0);
        smem = std::max(smem, step_smem_for(a));
    }
    if (n) {
        BK(cudaMemcpy(b->d_args, args.data(), n * sizeof(StepArgs), cudaMemcpyHostToDevice));
        BK(cudaMemcpy(b->d_march, march.data(), n * sizeof(MarchArgs), cudaMemcpyHostToDevice));
        BK(cudaMemcpy(b->d_dyn, dyn.data(), n * sizeof(BatchDyn), cudaMemcpyHostToDevice));
        BK(cudaMemcpy(b->d_live, live.data(), n * sizeof(int), cudaMemcpyHostToDevice));
        BK(cudaMemcpy(b->d_edge_off, eoff.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
        BK(cudaMemcpy(b->d_march_off, moff.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
        BK(cudaMemcpy(b->d_frame_off, foff.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
        BK(cudaMemcpy(b->d_top_off, toff.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
    }
    b->edge_blocks = eoff[n];
    b->march_blocks = moff[n];
    b->frame_blocks = foff[n];
    b->top_blocks = toff[n];
    b->smem = smem;
    // opt the batched kernels into their shared memory outside any stream capture
    const BatchTab t = table(b);
    if (n) {
        BK(launch_step_batch(t, b->norder, 0, b->smem, b->stream));
        BK(launch_step_top_batch(t, b->norder, 0, b->smem, b->stream));
        if (b->norder <= kMarchMaxOrder) BK(launch_march_batch(t, b->norder, 0, 0, b->stream));
    }
    b->dirty = false;
    return FDFK_OK;
}

// One step of every live member: bump, then the tiled kernel on the side stream next to the
// frames and the fast path on the main stream.
cudaError_t step_once(fdfk_batch* b)
{
    const BatchTab t = table(b);
    cudaError_t e = launch_batch_bump(t, b->stream);
    if (e != cudaSuccess) return e;
    if ((e = cudaEventRecord(b->fork, b->stream)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(b->side, b->fork, 0)) != cudaSuccess) return e;
    if ((e = launch_step_batch(t, b->norder, b->edge_blocks, b->smem, b->side)) != cudaSuccess) return e;
    if (b->march_blocks > 0 &&
        (e = launch_march_batch(t, b->norder, b->frame_blocks, b->march_blocks, b->stream)) != cudaSuccess)
        return e;
    if ((e = cudaEventRecord(b->join, b->side)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(b->stream, b->join, 0)) != cudaSuccess) return e;
    // members with the absorbing layer on top: their top layers read the interior just updated
    if (b->top_blocks > 0) return launch_step_top_batch(t, b->norder, b->top_blocks, b->smem, b->stream);
    return cudaSuccess;
}

int launches_per_step(const fdfk_batch* b) { return 2 + (b->march_blocks > 0 ? 2 : 0) + (b->top_blocks > 0 ? 1 : 0); }

}  // namespace

extern "C" {

int fdfk_batch_create(int norder, fdfk_batch** out)
{
    if (!out) return set_error(FDFK_EINVAL, "out is NULL");
    *out = nullptr;
    if (norder < 1 || norder > kMaxOrder) return set_error(FDFK_EINVAL, "norder must be 1..8");
    fdfk_batch* b = new (std::nothrow) fdfk_batch();
    if (!b) return set_error(FDFK_ENOMEM, "host allocation failed");
    b->norder = norder;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess) {
        if (b->stream) cudaStreamDestroy(b->stream);
        if (b->side) cudaStreamDestroy(b->side);
        if (b->fork) cudaEventDestroy(b->fork);
        if (b->join) cudaEventDestroy(b->join);
        delete b;
        return set_error(FDFK_ECUDA, "batch stream/event creation failed");
    }
    *out = b;
    return FDFK_OK;
}

int fdfk_batch_add(fdfk_batch* b, fdfk_session* s)
{
    if (!b || !s) return set_error(FDFK_EINVAL, "NULL argument");
    if (s->batch) return set_error(FDFK_ESTATE, "the session already belongs to a batch");
    if (s->p.norder != b->norder) return set_error(FDFK_EINVAL, "the session's norder differs from the batch's");
    for (int t = s->it; t <= s->p.nt; ++t)
        if (!s->have_bg[t]) return set_error(FDFK_ESTATE, "the session has no background for time index " + std::to_string(t));
    int rc = pull(b);
    if (rc) return rc;
    // the batch's next step waits for the session's own uploads and FK background (no host wait)
    cudaEvent_t ready = nullptr;
    BK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ready, s->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, ready, 0);
    cudaEventDestroy(ready);
    if (e != cudaSuccess) return set_error(FDFK_ECUDA, std::string("batch add: ") + cudaGetErrorString(e));
    b->members.push_back(s);
    s->batch = b;
    b->dirty = true;
    return FDFK_OK;
}

int fdfk_batch_remove(fdfk_batch* b, fdfk_session* s)
{
    if (!b || !s) return set_error(FDFK_EINVAL, "NULL argument");
    if (s->batch != b) return set_error(FDFK_EINVAL, "the session is not a member of this batch");
    int rc = pull(b);
    if (rc) return rc;
    b->members.erase(std::find(b->members.begin(), b->members.end(), s));
    s->batch = nullptr;
    b->dirty = true;
    return FDFK_OK;
}

int fdfk_batch_set_tuning(fdfk_batch* b, int seg_len, int pml_run)
{
    if (!b || (seg_len != 0 && (seg_len < 8 || seg_len > 1024)) || (pml_run != 0 && (pml_run < 8 || pml_run > 64)))
        return set_error(FDFK_EINVAL, "segment length must be 8..1024 and tile length 8..64 (0: the default)");
    int rc = pull(b);
    if (rc) return rc;
    b->seg_len = seg_len;
    b->pml_run = pml_run;
    b->dirty = true;
    return FDFK_OK;
}

int fdfk_batch_set_graph_chunk(fdfk_batch* b, int steps)
{
    if (!b || steps < 0) return set_error(FDFK_EINVAL, "bad argument");
    if (steps != b->chunk) drop_graph(b);
    b->chunk = steps;
    return FDFK_OK;
}

int fdfk_batch_advance(fdfk_batch* b, int nsteps)
{
    if (!b) return set_error(FDFK_EINVAL, "batch is NULL");
    if (nsteps < 0) return set_error(FDFK_EINVAL, "nsteps must be >= 0");
    if (b->members.empty() || nsteps == 0) return FDFK_OK;
    if (b->dirty) {
        int rc = pull(b);
        if (rc) return rc;
        if ((rc = rebuild(b)) != FDFK_OK) return rc;
    }
    int done = 0;
    if (b->chunk > 0 && nsteps >= b->chunk) {
        if (!b->graph || b->graph_steps != b->chunk) {
            drop_graph(b);
            cudaGraph_t g = nullptr;
            BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = cudaSuccess;
            for (int k = 0; k < b->chunk && e == cudaSuccess; ++k) e = step_once(b);
            cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return set_error(FDFK_ECUDA, std::string("graph capture: ") +
                                                 cudaGetErrorString(e != cudaSuccess ? e : e2));
            }
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                b->graph = nullptr;
                return set_error(FDFK_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
            }
            b->graph_steps = b->chunk;
        }
        for (; done + b->chunk <= nsteps; done += b->chunk) {
            BK(cudaGraphLaunch(b->graph, b->stream));
            count_launches((long long)b->chunk * launches_per_step(b));
        }
    }
    for (; done < nsteps; ++done) {
        BK(step_once(b));
        count_launches(launches_per_step(b));
    }
    b->in_flight = true;
    return FDFK_OK;
}

int fdfk_batch_synchronize(fdfk_batch* b)
{
    if (!b) return set_error(FDFK_EINVAL, "batch is NULL");
    return pull(b);
}

int fdfk_batch_live(fdfk_batch* b)
{
    if (!b) return set_error(FDFK_EINVAL, "batch is NULL");
    int rc = pull(b);
    if (rc) return rc;
    int live = 0;
    for (const fdfk_session* s : b->members) live += s->it <= s->p.nt;
    return live;
}

int fdfk_batch_size(const fdfk_batch* b) { return b ? (int)b->members.size() : FDFK_EINVAL; }

void fdfk_batch_destroy(fdfk_batch* b)
{
    if (!b) return;
    pull(b);
    for (fdfk_session* s : b->members) s->batch = nullptr;
    drop_graph(b);
    free_tables(b);
    cudaStreamDestroy(b->stream);
    cudaStreamDestroy(b->side);
    cudaEventDestroy(b->fork);
    cudaEventDestroy(b->join);
    delete b;
}

}  // extern "C"
