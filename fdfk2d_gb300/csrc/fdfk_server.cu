// Serving loop over batches: solve requests are queued, admitted in arrival
// order while their device memory fits the budget (material, wavefield, PML
// state, the FK background of every time step and the seismograms stay
// resident for the whole solve), joined to one running batch, advanced a chunk
// of steps per pump (CUDA-graph replay, asynchronous) and retired into the
// caller's seismogram buffers as soon as they pass their last time index.
// Requests that arrive while others run join the batch at the next pump
// (continuous batching).  Single-threaded and caller-driven: the caller calls
// fdfk_server_pump in its own loop; the GPU runs the chunk launched by one
// pump while the caller works until the next pump.
#include "fdfk_gb300.h"
#include "fdfk_session.h"
#include "fdfk_sweep.cuh"

#include <cuda_runtime.h>

#include <chrono>
#include <deque>
#include <string>
#include <unordered_map>
#include <vector>

using namespace fdfk;

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Req {
    fdfk_solve_request r{};
    long long id = 0;
    int state = FDFK_REQ_QUEUED;
    fdfk_session* s = nullptr;
    long long bytes = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    std::string err;
};

}  // namespace

struct fdfk_server {
    int norder = 0;
    long long budget = 0;
    long long in_use = 0;
    int chunk = 32;
    fdfk_batch* batch = nullptr;
    std::deque<Req*> queue;
    std::vector<Req*> running;
    std::unordered_map<long long, Req*> all;
    long long next_id = 1;
    long long completed = 0, failed = 0;
};

namespace {

int finish(fdfk_server* sv, Req* q, int state, const std::string& err)
{
    if (q->s) {
        if (q->s->batch) fdfk_batch_remove(sv->batch, q->s);
        fdfk_session_destroy(q->s);
        q->s = nullptr;
        sv->in_use -= q->bytes;
    }
    q->state = state;
    q->err = err;
    q->t_done = now_s();
    if (state == FDFK_REQ_DONE) ++sv->completed;
    else ++sv->failed;
    return FDFK_OK;
}

// Create the session of a request, compute its FK background on the GPU, set its receivers.
int admit(fdfk_server* sv, Req* q)
{
    const fdfk_solve_request& r = q->r;
    fdfk_session* s = nullptr;
    int rc = fdfk_session_create(&r.p, r.c, &s);
    if (rc) return rc;
    q->s = s;
    sv->in_use += q->bytes;
    if ((rc = fdfk_session_fk_background(s, &r.fk, r.bazs, r.nlayer_left, r.fk_left, r.nlayer_right, r.fk_right)) ||
        (rc = fdfk_session_set_receivers(s, r.nrcv, r.rx, r.rz, r.x0, r.z0, r.nstp, r.nsis)) ||
        (rc = fdfk_batch_add(sv->batch, s)))
        return rc;
    q->state = FDFK_REQ_RUNNING;
    q->t_admit = now_s();
    return FDFK_OK;
}

}  // namespace

extern "C" {

long long fdfk_session_device_bytes(const fdfk_params* p, int nrcv, int nsis)
{
    if (!p || p->nx < 1 || p->nz < 1 || p->npml < 0 || p->nt < 0 || nrcv < 0) return -1;
    const bool fast = p->norder <= kMarchMaxOrder && p->nz >= 2 * p->norder + 1;
    const int izt = p->is_PML_top ? 1 - p->npml : 1;
    const long long NZ = p->nz + p->npml - izt + 1, NX = p->nx + 2LL * p->npml;
    const long long ldz = plane_ldz(p->nz, p->npml, p->norder, fast, izt);
    const long long n = ldz * NX;
    const long long side = (long long)p->nz * p->npml, tb = (long long)p->npml * NX;
    const long long nx = p->nx, nz = p->nz, nbd = p->nbd;
    const long long strips = 4 * (nz - nbd) * nbd + 2 * nbd * nx + 4 * nz * nbd + 2 * nbd * (nx + 2 * nbd);
    const long long ntb = p->is_PML_top ? 2 : 1;   // bottom, and top layer arrays
    long long f = (fast ? 9 : 7) * n + 2 * (12 * side + 6 * ntb * tb) + 4 * side + 4 * ntb * tb + strips * (p->nt + 1LL);
    f += 2LL * nrcv + (nrcv > 0 ? 2LL * (nsis + 1) * nrcv : 0);
    return 4 * f + (long long)sizeof(DampCol) * (NX + NZ);
}

int fdfk_server_create(int norder, long long hbm_budget_bytes, int chunk_steps, fdfk_server** out)
{
    if (!out) return set_error(FDFK_EINVAL, "out is NULL");
    *out = nullptr;
    if (hbm_budget_bytes <= 0 || chunk_steps < 1) return set_error(FDFK_EINVAL, "budget and chunk must be positive");
    fdfk_server* sv = new (std::nothrow) fdfk_server();
    if (!sv) return set_error(FDFK_ENOMEM, "host allocation failed");
    int rc = fdfk_batch_create(norder, &sv->batch);
    if (rc) {
        delete sv;
        return rc;
    }
    sv->norder = norder;
    sv->budget = hbm_budget_bytes;
    sv->chunk = chunk_steps;
    fdfk_batch_set_graph_chunk(sv->batch, chunk_steps);
    *out = sv;
    return FDFK_OK;
}

int fdfk_server_submit(fdfk_server* sv, const fdfk_solve_request* r, long long* id)
{
    if (!sv || !r || !id) return set_error(FDFK_EINVAL, "NULL argument");
    if (r->p.norder != sv->norder) return set_error(FDFK_EINVAL, "the request's norder differs from the server's");
    if (!r->c || !r->bazs || !r->fk_left || !r->fk_right || !r->seisx || !r->seisz || r->nrcv < 1 || r->nsis < 0)
        return set_error(FDFK_EINVAL, "request: missing inputs or outputs");
    Req* q = new (std::nothrow) Req();
    if (!q) return set_error(FDFK_ENOMEM, "host allocation failed");
    q->r = *r;
    q->id = sv->next_id++;
    q->bytes = fdfk_session_device_bytes(&r->p, r->nrcv, r->nsis);
    q->t_submit = now_s();
    if (q->bytes < 0 || q->bytes > sv->budget) {
        delete q;
        return set_error(FDFK_EINVAL, "request: the solve does not fit the server's memory budget");
    }
    sv->queue.push_back(q);
    sv->all[q->id] = q;
    *id = q->id;
    return FDFK_OK;
}

int fdfk_server_pump(fdfk_server* sv, int* in_flight)
{
    if (!sv) return set_error(FDFK_EINVAL, "server is NULL");
    // 1. retire members that passed their last time index (waits for the chunk in flight)
    int rc = fdfk_batch_synchronize(sv->batch);
    if (rc) return rc;
    std::vector<Req*> still;
    for (Req* q : sv->running) {
        if (q->s->it <= q->s->p.nt) {
            still.push_back(q);
            continue;
        }
        rc = fdfk_session_download_seismograms(q->s, q->r.seisx, q->r.seisz);
        finish(sv, q, rc ? FDFK_REQ_FAILED : FDFK_REQ_DONE, rc ? fdfk_last_error() : "");
    }
    sv->running.swap(still);
    // 2. admit queued requests in arrival order while the budget allows
    while (!sv->queue.empty() && sv->in_use + sv->queue.front()->bytes <= sv->budget) {
        Req* q = sv->queue.front();
        sv->queue.pop_front();
        rc = admit(sv, q);
        if (rc) finish(sv, q, FDFK_REQ_FAILED, fdfk_last_error());
        else sv->running.push_back(q);
    }
    // 3. launch the next chunk of steps for everything running (asynchronous)
    if (!sv->running.empty() && (rc = fdfk_batch_advance(sv->batch, sv->chunk)) != FDFK_OK) return rc;
    if (in_flight) *in_flight = (int)(sv->running.size() + sv->queue.size());
    return FDFK_OK;
}

int fdfk_server_request(fdfk_server* sv, long long id, int* state, double* t_submit, double* t_admit, double* t_done)
{
    if (!sv || !state) return set_error(FDFK_EINVAL, "NULL argument");
    auto it = sv->all.find(id);
    if (it == sv->all.end()) return set_error(FDFK_EINVAL, "unknown request id");
    const Req* q = it->second;
    *state = q->state;
    if (t_submit) *t_submit = q->t_submit;
    if (t_admit) *t_admit = q->t_admit;
    if (t_done) *t_done = q->t_done;
    if (q->state == FDFK_REQ_FAILED) set_error(FDFK_EINVAL, q->err);
    return FDFK_OK;
}

int fdfk_server_get_stats(const fdfk_server* sv, fdfk_server_stats* st)
{
    if (!sv || !st) return set_error(FDFK_EINVAL, "NULL argument");
    st->queued = (int)sv->queue.size();
    st->running = (int)sv->running.size();
    st->completed = sv->completed;
    st->failed = sv->failed;
    st->bytes_in_use = sv->in_use;
    st->budget = sv->budget;
    return FDFK_OK;
}

void fdfk_server_destroy(fdfk_server* sv)
{
    if (!sv) return;
    fdfk_batch_synchronize(sv->batch);
    for (Req* q : sv->running) finish(sv, q, FDFK_REQ_FAILED, "server destroyed");
    for (Req* q : sv->queue) q->state = FDFK_REQ_FAILED;
    fdfk_batch_destroy(sv->batch);
    for (auto& kv : sv->all) delete kv.second;
    delete sv;
}

}  // extern "C"
