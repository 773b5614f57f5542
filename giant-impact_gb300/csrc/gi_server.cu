// gi_server.cu -- continuous-batching serving loop for impact runs.
//
// Requests (bodies + step count) arrive at any time and wait in a FIFO
// queue.  Each round:
//   1. admit: the head of the queue joins the live set while a slot is free
//      and its device memory (two state buffers + scratch estimate) fits in
//      the HBM budget; its bodies are copied into a contiguous range of the
//      device pool (first-fit free list; the pool grows within the budget);
//   2. step: the live runs advance `steps_per_round` steps, all stepped runs
//      in one persistent force launch per step (gi_step_pingpong over the
//      run table); a run whose remaining steps run out mid-round simply drops
//      out of the next step's table.  GI_SERVE_SHARE steps every live run;
//      GI_SERVE_SHORTEST steps the runs with the least remaining work until
//      a step's pair interactions fill the GPU (one large run already does),
//      so short requests finish first and the GPU stays full;
//   3. retire: finished runs are copied to host memory and their range freed.
// A run's result depends only on its own bodies, N and the context's tuning
// table (the force kernel is batch-invariant), so it is the same alone and
// in any mix.  With device = GI_SERVER_DRY_RUN no GPU is used: admission,
// pool placement and stepping are simulated (state is left unchanged), which
// lets the scheduling logic be planned and tested on a CPU.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <vector>

#include "gi_internal.h"

namespace {

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
    long long id = 0;
    int state = GI_REQ_QUEUED;
    gi_run run{};
    int nsteps = 0;
    int steps_done = 0;
    std::vector<float> pos, vel;  // input until admitted, result once done
    double t_submit = 0, t_admit = 0, t_done = 0;
    long long bytes = 0;
    long long offset = -1;
    int where = 0;  // state buffer holding the run's current state
};

}  // namespace

struct gi_server {
    int device = 0;
    bool dry = false;
    gi_server_config cfg{};
    std::vector<gi_pair_params> params;
    gi_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;
    float *pos[2] = {nullptr, nullptr};
    float *vel[2] = {nullptr, nullptr};
    long long cap = 0;   // bodies in the pool
    long long high = 0;  // end of the highest range ever handed out
    std::map<long long, long long> free_;  // offset -> length, below `high`
    int cur = 0;
    std::deque<long long> queue;
    std::map<long long, Req> reqs;
    std::vector<long long> live;
    long long bytes_in_use = 0;
    long long next_id = 1;
    long long interactions = 0;
    long long rounds = 0;
    long long completed = 0;
    long long cancelled = 0;
};

namespace {

// Device bytes one run holds while live: both state buffers plus the
// context's scratch for it.  Zero-size runs hold nothing.
long long run_bytes(gi_server *s, int n)
{
    if (n <= 0) return 0;
    const long long state = 2LL * 2 * 16 * n;  // pos + vel, two buffers
    return state + (s->dry ? 0 : gi_internal_scratch_bytes(s->ctx, n));
}

// First-fit range of n bodies; grows the pool (copying live ranges) if none
// is free.  Returns -1 when the budget does not allow it.
long long pool_alloc(gi_server *s, long long n, int *st)
{
    *st = GI_OK;
    for (auto it = s->free_.begin(); it != s->free_.end(); ++it) {
        if (it->second >= n) {
            const long long off = it->first, len = it->second;
            s->free_.erase(it);
            if (len > n) s->free_[off + n] = len - n;
            return off;
        }
    }
    const long long off = s->high;
    if (off + n > s->cap) {
        long long want = std::max(2 * s->cap, off + n);
        want = std::max(want, 65536LL);
        // the pool's two state buffers must fit the budget together
        const long long limit = s->cfg.hbm_budget_bytes / (2LL * 2 * 16);
        if (want > limit) want = limit;
        if (want < off + n) return -1;
        if (!s->dry) {
            float *np[2] = {nullptr, nullptr}, *nv[2] = {nullptr, nullptr};
            cudaError_t e = cudaSuccess;
            for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
                e = cudaMalloc(&np[b], (size_t)want * 16);
                if (e == cudaSuccess) e = cudaMalloc(&nv[b], (size_t)want * 16);
            }
            for (int b = 0; b < 2 && e == cudaSuccess && s->high > 0; ++b) {
                e = cudaMemcpyAsync(np[b], s->pos[b], (size_t)s->high * 16, cudaMemcpyDeviceToDevice, s->stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(nv[b], s->vel[b], (size_t)s->high * 16, cudaMemcpyDeviceToDevice, s->stream);
            }
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e != cudaSuccess) {
                for (int b = 0; b < 2; ++b) { cudaFree(np[b]); cudaFree(nv[b]); }
                *st = gi_internal_fail(e == cudaErrorMemoryAllocation ? GI_ERR_OUT_OF_MEMORY : GI_ERR_CUDA,
                                       "serving pool growth failed");
                return -1;
            }
            for (int b = 0; b < 2; ++b) {
                cudaFree(s->pos[b]);
                cudaFree(s->vel[b]);
                s->pos[b] = np[b];
                s->vel[b] = nv[b];
            }
        }
        s->cap = want;
    }
    s->high = off + n;
    return off;
}

void pool_free(gi_server *s, long long off, long long n)
{
    if (n <= 0) return;
    auto it = s->free_.emplace(off, n).first;
    // merge with the next range
    auto nx = std::next(it);
    if (nx != s->free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        s->free_.erase(nx);
    }
    // merge with the previous range
    if (it != s->free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            s->free_.erase(it);
            it = pv;
        }
    }
    // give the top range back to the high-water mark
    if (it->first + it->second == s->high) {
        s->high = it->first;
        s->free_.erase(it);
    }
}

int admit(gi_server *s)
{
    while (!s->queue.empty() && (int)s->live.size() < s->cfg.max_live_runs) {
        Req &q = s->reqs[s->queue.front()];
        if (s->bytes_in_use + q.bytes > s->cfg.hbm_budget_bytes) break;  // FIFO: wait for room
        int st = GI_OK;
        const long long off = pool_alloc(s, q.run.n, &st);
        if (st) return st;
        if (off < 0) break;
        q.offset = off;
        q.where = s->cur;
        if (!s->dry && q.run.n > 0) {
            const size_t bytes = (size_t)q.run.n * 16;
            cudaError_t e = cudaMemcpyAsync(s->pos[s->cur] + 4 * off, q.pos.data(), bytes,
                                            cudaMemcpyHostToDevice, s->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(s->vel[s->cur] + 4 * off, q.vel.data(), bytes,
                                    cudaMemcpyHostToDevice, s->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e != cudaSuccess) return gi_internal_fail(GI_ERR_CUDA, "admission copy failed");
        }
        q.state = GI_REQ_LIVE;
        q.t_admit = now_s();
        s->bytes_in_use += q.bytes;
        s->live.push_back(q.id);
        s->queue.pop_front();
    }
    return GI_OK;
}

// Live runs to step next, by policy.
std::vector<long long> select_runs(gi_server *s)
{
    std::vector<long long> ids;
    for (long long id : s->live)
        if (s->reqs[id].nsteps > s->reqs[id].steps_done) ids.push_back(id);
    if (s->cfg.policy != GI_SERVE_SHORTEST || ids.empty()) return ids;
    auto work = [&](long long id) {
        const Req &q = s->reqs[id];
        return (double)(q.nsteps - q.steps_done) * (double)q.run.n * (double)q.run.n;
    };
    std::stable_sort(ids.begin(), ids.end(),
                     [&](long long a, long long b) { return work(a) < work(b); });
    const double fill = s->cfg.fill_interactions > 0 ? (double)s->cfg.fill_interactions : 2e9;
    double per_step = 0.0;
    size_t k = 0;
    while (k < ids.size() && (k == 0 || per_step < fill)) {
        const Req &q = s->reqs[ids[k]];
        per_step += (double)q.run.n * (double)(q.run.n - 1);
        ++k;
    }
    ids.resize(k);
    return ids;
}

int step_round(gi_server *s)
{
    const int S = s->cfg.steps_per_round;
    for (int k = 0; k < S;) {
        std::vector<gi_run> runs;
        std::vector<long long> ids = select_runs(s);
        int span = S - k;  // steps every selected run can take without dropping out
        for (long long id : ids) {
            Req &q = s->reqs[id];
            span = std::min(span, q.nsteps - q.steps_done);
            gi_run r = q.run;
            r.offset = (int)q.offset;
            runs.push_back(r);
            // a run left out of earlier steps may sit in the other state buffer
            if (q.where != s->cur && !s->dry && q.run.n > 0) {
                const size_t bytes = (size_t)q.run.n * 16;
                cudaError_t e = cudaMemcpyAsync(s->pos[s->cur] + 4 * q.offset,
                                                s->pos[q.where] + 4 * q.offset, bytes,
                                                cudaMemcpyDeviceToDevice, s->stream);
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(s->vel[s->cur] + 4 * q.offset,
                                        s->vel[q.where] + 4 * q.offset, bytes,
                                        cudaMemcpyDeviceToDevice, s->stream);
                if (e != cudaSuccess) return gi_internal_fail(GI_ERR_CUDA, "state copy failed");
            }
            q.where = s->cur;
        }
        if (runs.empty()) break;
        if (!s->dry) {
            const int b = s->cur;
            int st = gi_step_pingpong(s->ctx, s->pos[b], s->vel[b], s->pos[1 - b], s->vel[1 - b],
                                      runs.data(), (int)runs.size(), s->params.data(),
                                      (int)s->params.size(), span, s->stream);
            if (st) return st;
        }
        if (span & 1) s->cur ^= 1;
        for (size_t m = 0; m < ids.size(); ++m) {
            Req &q = s->reqs[ids[m]];
            q.steps_done += span;
            q.where = s->cur;
            s->interactions += (long long)span * q.run.n * (long long)(q.run.n - 1);
        }
        k += span;
    }
    return GI_OK;
}

int retire(gi_server *s, int *nret)
{
    *nret = 0;
    if (!s->dry) {
        cudaError_t e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return gi_internal_fail(GI_ERR_CUDA, "serving step failed");
    }
    std::vector<long long> keep;
    for (long long id : s->live) {
        Req &q = s->reqs[id];
        if (q.steps_done < q.nsteps) {
            keep.push_back(id);
            continue;
        }
        if (!s->dry && q.run.n > 0) {
            const size_t bytes = (size_t)q.run.n * 16;
            cudaError_t e = cudaMemcpyAsync(q.pos.data(), s->pos[q.where] + 4 * q.offset, bytes,
                                            cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(q.vel.data(), s->vel[q.where] + 4 * q.offset, bytes,
                                    cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
            if (e != cudaSuccess) return gi_internal_fail(GI_ERR_CUDA, "retirement copy failed");
        }
        pool_free(s, q.offset, q.run.n);
        s->bytes_in_use -= q.bytes;
        q.state = GI_REQ_DONE;
        q.t_done = now_s();
        ++s->completed;
        ++*nret;
    }
    s->live.swap(keep);
    return GI_OK;
}

}  // namespace

extern "C" int gi_server_create(int device, const gi_server_config *cfg,
                                const gi_pair_params *params, int nparams, gi_server **out)
{
    if (!cfg || !params || !out) return gi_internal_fail(GI_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (cfg->hbm_budget_bytes <= 0 || cfg->max_live_runs < 1 || cfg->steps_per_round < 1)
        return gi_internal_fail(GI_ERR_INVALID_ARG, "budget, slots and steps_per_round must be positive");
    if ((cfg->policy != GI_SERVE_SHARE && cfg->policy != GI_SERVE_SHORTEST) ||
        cfg->fill_interactions < 0)
        return gi_internal_fail(GI_ERR_INVALID_ARG, "unknown policy or negative fill");
    if (nparams < 1 || nparams > GI_MAX_PARAMS)
        return gi_internal_fail(GI_ERR_BAD_SIZE, "nparams out of range");
    gi_server *s = new gi_server();
    s->device = device;
    s->dry = device == GI_SERVER_DRY_RUN;
    s->cfg = *cfg;
    s->params.assign(params, params + nparams);
    if (!s->dry) {
        int st = gi_ctx_create(&s->ctx, device);
        if (st) { delete s; return st; }
        int prev = 0;
        cudaGetDevice(&prev);
        cudaSetDevice(device);
        cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        cudaSetDevice(prev);
        if (e != cudaSuccess) {
            gi_ctx_destroy(s->ctx);
            delete s;
            return gi_internal_fail(GI_ERR_CUDA, "stream creation failed");
        }
    }
    *out = s;
    return GI_OK;
}

extern "C" int gi_server_destroy(gi_server *s)
{
    if (!s) return GI_OK;
    if (!s->dry) {
        cudaStreamSynchronize(s->stream);
        for (int b = 0; b < 2; ++b) { cudaFree(s->pos[b]); cudaFree(s->vel[b]); }
        cudaStreamDestroy(s->stream);
        gi_ctx_destroy(s->ctx);
    }
    delete s;
    return GI_OK;
}

extern "C" int gi_server_submit(gi_server *s, const float *pos_host, const float *vel_host,
                                const gi_run *run, int nsteps, long long *id)
{
    if (!s || !run || !id) return gi_internal_fail(GI_ERR_INVALID_ARG, "NULL argument");
    if (run->n < 0 || run->nfe < 0 || run->nfe > run->n)
        return gi_internal_fail(GI_ERR_BAD_SIZE, "run n / nfe out of range");
    if (run->n > 0 && (!pos_host || !vel_host))
        return gi_internal_fail(GI_ERR_INVALID_ARG, "host body arrays are NULL");
    if (run->params < 0 || run->params >= (int)s->params.size())
        return gi_internal_fail(GI_ERR_INVALID_ARG, "params index out of range");
    if (nsteps < 0) return gi_internal_fail(GI_ERR_INVALID_ARG, "nsteps is negative");
    Req q;
    q.id = s->next_id++;
    q.run = *run;
    q.run.offset = 0;
    q.nsteps = nsteps;
    q.pos.assign(pos_host, pos_host + 4 * (size_t)run->n);
    q.vel.assign(vel_host, vel_host + 4 * (size_t)run->n);
    q.bytes = run_bytes(s, run->n);
    if (q.bytes > s->cfg.hbm_budget_bytes)
        return gi_internal_fail(GI_ERR_CAPACITY, "run needs more device memory than the whole budget");
    q.t_submit = now_s();
    *id = q.id;
    s->queue.push_back(q.id);
    s->reqs.emplace(q.id, std::move(q));
    return GI_OK;
}

extern "C" int gi_server_round(gi_server *s, int *nretired)
{
    if (!s) return gi_internal_fail(GI_ERR_INVALID_ARG, "server is NULL");
    int dummy = 0;
    if (!nretired) nretired = &dummy;
    *nretired = 0;
    int prev = 0;
    if (!s->dry) {
        cudaGetDevice(&prev);
        cudaSetDevice(s->device);
    }
    int st = admit(s);
    if (!st) st = step_round(s);
    if (!st) st = retire(s, nretired);
    ++s->rounds;
    if (!s->dry) cudaSetDevice(prev);
    return st;
}

extern "C" int gi_server_query(gi_server *s, long long id, gi_server_request_info *info)
{
    if (!s || !info) return gi_internal_fail(GI_ERR_INVALID_ARG, "NULL argument");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return gi_internal_fail(GI_ERR_INVALID_ARG, "unknown request id");
    const Req &q = it->second;
    info->state = q.state;
    info->n = q.run.n;
    info->steps_done = q.steps_done;
    info->nsteps = q.nsteps;
    info->t_submit = q.t_submit;
    info->t_admit = q.t_admit;
    info->t_done = q.t_done;
    info->bytes = q.bytes;
    return GI_OK;
}

extern "C" int gi_server_fetch(gi_server *s, long long id, float *pos_host, float *vel_host)
{
    if (!s) return gi_internal_fail(GI_ERR_INVALID_ARG, "server is NULL");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return gi_internal_fail(GI_ERR_INVALID_ARG, "unknown request id");
    Req &q = it->second;
    if (q.state != GI_REQ_DONE) return gi_internal_fail(GI_ERR_INVALID_ARG, "request not done");
    if (q.run.n > 0 && (!pos_host || !vel_host))
        return gi_internal_fail(GI_ERR_INVALID_ARG, "host body arrays are NULL");
    std::memcpy(pos_host, q.pos.data(), q.pos.size() * sizeof(float));
    std::memcpy(vel_host, q.vel.data(), q.vel.size() * sizeof(float));
    s->reqs.erase(it);
    return GI_OK;
}

extern "C" int gi_server_cancel(gi_server *s, long long id)
{
    if (!s) return gi_internal_fail(GI_ERR_INVALID_ARG, "server is NULL");
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return gi_internal_fail(GI_ERR_INVALID_ARG, "unknown request id");
    Req &q = it->second;
    if (q.state == GI_REQ_QUEUED) {
        s->queue.erase(std::find(s->queue.begin(), s->queue.end(), id));
    } else if (q.state == GI_REQ_LIVE) {
        // Between rounds nothing of this server is in flight (every round
        // ends with a stream synchronisation), so the range can be handed
        // back at once; the other live runs' ranges are not touched.
        s->live.erase(std::find(s->live.begin(), s->live.end(), id));
        pool_free(s, q.offset, q.run.n);
        s->bytes_in_use -= q.bytes;
    }
    s->reqs.erase(it);
    ++s->cancelled;
    return GI_OK;
}

extern "C" int gi_server_get_stats(gi_server *s, gi_server_stats *out)
{
    if (!s || !out) return gi_internal_fail(GI_ERR_INVALID_ARG, "NULL argument");
    out->live = (int)s->live.size();
    out->queued = (int)s->queue.size();
    out->completed = s->completed;
    out->rounds = s->rounds;
    out->bytes_in_use = s->bytes_in_use;
    out->pool_bodies = s->cap;
    out->interactions = s->interactions;
    out->cancelled = s->cancelled;
    return GI_OK;
}
