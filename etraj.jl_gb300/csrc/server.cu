// server.cu -- the continuously batching server of include/etraj.h.
#include "host.h"

// ---- server: continuous batching of many jobs on one GPU -----------------------------
// `slots` contexts, each with its own stream and buffers.  A submitted job waits
// in a FIFO queue until a slot is free and the device bytes it would add fit in
// the server's HBM budget; it is then enqueued on that slot and overlaps on the
// device with the jobs of the other slots.  A job's result depends on nothing
// but the job: no state is shared between slots.

struct etraj_server {
    int device = 0;
    size_t budget = 0;
    std::vector<etraj_ctx*> slot;
    std::vector<uint64_t> slot_ticket;  // 0: free
    struct Req {
        etraj_job job;
        etraj_result res;
        uint64_t ticket;
    };
    std::deque<Req> queue;
    std::map<uint64_t, JobRec> running;
    std::map<uint64_t, int> running_slot;
    struct Done {
        int status;
        std::string error;
        etraj_result res;
    };
    std::map<uint64_t, Done> done;
    uint64_t next_ticket = 1;
    std::string err;
    std::mutex mu;
};

namespace {

size_t server_used(const etraj_server* srv) {
    size_t u = 0;
    for (const etraj_ctx* c : srv->slot) u += c->used;
    return u;
}

void free_ctx_buffers(etraj_ctx* ctx) {
    for (auto& kv : ctx->bufs)
        if (kv.second.p) cudaFreeAsync(kv.second.p, ctx->stream);
    ctx->bufs.clear();
    ctx->used = 0;
}

// Retires finished jobs and admits queued ones (server lock held).
void server_progress(etraj_server* srv) {
    cudaSetDevice(srv->device);
    for (size_t i = 0; i < srv->slot.size(); ++i) {
        const uint64_t tk = srv->slot_ticket[i];
        if (!tk) continue;
        etraj_ctx* ctx = srv->slot[i];
        JobRec& r = srv->running[tk];
        cudaError_t e = cudaEventQuery(r.ev_done);
        if (e == cudaErrorNotReady) {
            cudaGetLastError();
            continue;
        }
        etraj_server::Done d;
        if (e == cudaSuccess) {
            d.status = finish_job(ctx, r);
        } else {
            d.status = cuda_err(ctx, e, "server job");
            release_job(ctx, r);
        }
        d.error = (d.status == ETRAJ_OK) ? std::string() : ctx->err;
        d.res = r.res;
        srv->done[tk] = d;
        srv->running.erase(tk);
        srv->running_slot.erase(tk);
        srv->slot_ticket[i] = 0;
    }
    while (!srv->queue.empty()) {
        int free_slot = -1;
        for (size_t i = 0; i < srv->slot.size(); ++i)
            if (!srv->slot_ticket[i]) {
                free_slot = (int)i;
                break;
            }
        if (free_slot < 0) return;
        etraj_server::Req& q = srv->queue.front();
        etraj_ctx* ctx = srv->slot[(size_t)free_slot];
        size_t growth = plan_growth(ctx, &q.job);
        if (server_used(srv) + growth > srv->budget) {
            // give back the buffers of idle slots, then re-plan
            for (size_t i = 0; i < srv->slot.size(); ++i)
                if (!srv->slot_ticket[i] && (int)i != free_slot) free_ctx_buffers(srv->slot[i]);
            growth = plan_growth(ctx, &q.job);
            if (server_used(srv) + growth > srv->budget) {
                free_ctx_buffers(ctx);
                growth = plan_growth(ctx, &q.job);
            }
            if (server_used(srv) + growth > srv->budget) {
                if (!srv->running.empty()) return;  // wait for memory
                etraj_server::Done d;
                d.status = ETRAJ_ERR_OUT_OF_MEMORY;
                d.error = "job needs " + std::to_string(growth) + " device bytes; server budget " +
                          std::to_string(srv->budget);
                d.res = q.res;
                srv->done[q.ticket] = d;
                srv->queue.pop_front();
                continue;
            }
        }
        JobRec r;
        r.res = q.res;
        r.staged = true;
        const int st = enqueue_job(ctx, &q.job, r);
        if (st != ETRAJ_OK) {
            release_job(ctx, r);
            etraj_server::Done d;
            d.status = st;
            d.error = ctx->err;
            d.res = q.res;
            srv->done[q.ticket] = d;
        } else {
            srv->running[q.ticket] = r;
            srv->running_slot[q.ticket] = free_slot;
            srv->slot_ticket[(size_t)free_slot] = q.ticket;
        }
        srv->queue.pop_front();
    }
}

// Takes a finished ticket's result (server lock held); NOT_READY while queued or running.
int server_take(etraj_server* srv, uint64_t tk, etraj_result* out) {
    auto it = srv->done.find(tk);
    if (it == srv->done.end()) {
        if (srv->running.count(tk)) return ETRAJ_ERR_NOT_READY;
        for (const auto& q : srv->queue)
            if (q.ticket == tk) return ETRAJ_ERR_NOT_READY;
        srv->err = "unknown ticket";
        return ETRAJ_ERR_NOT_FOUND;
    }
    double* ms = out->momentum_spec;
    double* amp = out->amplitude;
    *out = it->second.res;
    out->momentum_spec = ms;
    out->amplitude = amp;
    const int st = it->second.status;
    if (st != ETRAJ_OK) srv->err = it->second.error;
    srv->done.erase(it);
    return st;
}

}  // namespace

extern "C" {

int etraj_server_create(etraj_server** out, int device, int slots, size_t hbm_budget_bytes) {
    if (!out || slots < 1 || slots > 64) return ETRAJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    etraj_server* srv = new etraj_server();
    srv->device = device;
    for (int i = 0; i < slots; ++i) {
        etraj_ctx* c = nullptr;
        const int st = etraj_create(&c, device, hbm_budget_bytes);
        if (st != ETRAJ_OK) {
            for (etraj_ctx* d : srv->slot) etraj_destroy(d);
            delete srv;
            return st;
        }
        srv->slot.push_back(c);
        srv->slot_ticket.push_back(0);
    }
    // the server enforces one budget over all slots
    srv->budget = srv->slot[0]->budget;
    for (etraj_ctx* c : srv->slot) c->budget = (size_t)-1 / 2;
    *out = srv;
    return ETRAJ_OK;
}

void etraj_server_destroy(etraj_server* srv) {
    if (!srv) return;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        cudaSetDevice(srv->device);
        for (size_t i = 0; i < srv->slot.size(); ++i) {
            const uint64_t tk = srv->slot_ticket[i];
            if (!tk) continue;
            cudaEventSynchronize(srv->running[tk].ev_done);
            release_job(srv->slot[i], srv->running[tk]);
        }
    }
    for (etraj_ctx* c : srv->slot) etraj_destroy(c);
    delete srv;
}

int etraj_server_submit(etraj_server* srv, const etraj_job* job, etraj_result* out, uint64_t* ticket) {
    if (!srv || !job || !out || !ticket) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::string err;
    const int st = validate_job(job, err);
    if (st != ETRAJ_OK) {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->err = err;
        return st;
    }
    std::lock_guard<std::mutex> lk(srv->mu);
    const uint64_t tk = srv->next_ticket++;
    srv->queue.push_back(etraj_server::Req{*job, *out, tk});
    server_progress(srv);
    *ticket = tk;
    return ETRAJ_OK;
}

int etraj_server_poll(etraj_server* srv, uint64_t ticket, etraj_result* out) {
    if (!srv || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(srv->mu);
    server_progress(srv);
    return server_take(srv, ticket, out);
}

int etraj_server_wait(etraj_server* srv, uint64_t ticket, etraj_result* out, double timeout_s) {
    if (!srv || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            server_progress(srv);
            const int st = server_take(srv, ticket, out);
            if (st != ETRAJ_ERR_NOT_READY) return st;
        }
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_s >= 0.0 && el > timeout_s) {
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->err = "etraj_server_wait: timed out";
            return ETRAJ_ERR_TIMEOUT;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

int etraj_server_stats(etraj_server* srv, int64_t* running, int64_t* queued, size_t* hbm_in_use) {
    if (!srv) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(srv->mu);
    server_progress(srv);
    if (running) *running = (int64_t)srv->running.size();
    if (queued) *queued = (int64_t)srv->queue.size();
    if (hbm_in_use) *hbm_in_use = server_used(srv);
    return ETRAJ_OK;
}

const char* etraj_server_last_error(const etraj_server* srv) { return srv ? srv->err.c_str() : "no server"; }

}  // extern "C"
