// api.cu -- the C ABI of include/etraj.h: contexts, validation, host-side job
// set-up and the orchestration of the device pipeline.
//
// Pipeline of etraj_run (all launches on the context's stream, one host
// synchronization at the end):
//   k_batch_prepare  per time sample   (gen_electron_batch prologue)
//   k_sample         per candidate     (gen_electron_batch loop body)
//   compaction       order-preserving survivor list
//   k_integrate_*    per survivor      (Tsit5 solve + collection)
//   deposit          radix sort + segmented sums + canonical reductions
// This replaces the `@threads for i in 1:batch_num` loop of
// src/TrajectorySimulation.jl:154-157 and the reduction of write_output!
// (:521-543).

// The host side is split over job.cu, pipeline.cu, tune.cu, batch.cu and
// server.cu (host.h); this file holds the C entry points.
#include "host.h"

// ---- exported entry points --------------------------------------------------------
extern "C" {

const char* etraj_version(void) { return ETRAJ_VERSION_STRING; }

int etraj_create(etraj_ctx** out, int device, size_t hbm_budget_bytes) {
    if (!out) return ETRAJ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return ETRAJ_ERR_CUDA;
    }
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return ETRAJ_ERR_CUDA;
    etraj_ctx* ctx = new etraj_ctx();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    {
        // keep freed stream-ordered memory in this process's pool instead of
        // returning it at every synchronization (process-local setting)
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t reserve = (size_t)1 << 30;
    ctx->budget = hbm_budget_bytes ? hbm_budget_bytes : (free_b > reserve ? free_b - reserve : free_b / 2);
    if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
        delete ctx;
        return ETRAJ_ERR_CUDA;
    }
    for (int i = 0; i <= etraj_ctx::kStages; ++i) {
        if (cudaEventCreate(&ctx->stage_ev[i]) == cudaSuccess) continue;
        delete ctx;
        return ETRAJ_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
    return ETRAJ_OK;
}

void etraj_destroy(etraj_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->jobs) release_job(ctx, kv.second);
    for (auto& b : ctx->pinned_pool) cudaFreeHost(b.p);
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    for (auto& kv : ctx->bufs)
        if (kv.second.p) cudaFreeAsync(kv.second.p, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    if (ctx->bgexec) cudaGraphExecDestroy(ctx->bgexec);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (int i = 0; i <= etraj_ctx::kStages; ++i)
        if (ctx->stage_ev[i]) cudaEventDestroy(ctx->stage_ev[i]);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

const char* etraj_last_error(const etraj_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int etraj_set_stream(etraj_ctx* ctx, void* cuda_stream) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    // buffers are stream-ordered allocations: finish everything queued on the
    // old stream before the new one may touch them
    cudaStreamSynchronize(ctx->stream);
    ctx->stream = cuda_stream ? (cudaStream_t)cuda_stream : ctx->own_stream;
    return ETRAJ_OK;
}

int etraj_validate(const etraj_job* job, char* msg, size_t msg_len) {
    std::string err;
    int st = validate_job(job, err);
    if (msg && msg_len > 0) {
        std::strncpy(msg, err.c_str(), msg_len - 1);
        msg[msg_len - 1] = 0;
    }
    return st;
}

int etraj_batch_info(const etraj_job* job, int64_t* batch_num, int64_t* batch_max_size) {
    if (!job) return ETRAJ_ERR_INVALID_ARGUMENT;
    if (batch_num) *batch_num = job->sample_t_num;
    if (batch_max_size)
        *batch_max_size = job->sample_monte_carlo ? job->mc_kt_num
                                                  : job->ss_kd_num * ((job->dimension == 3) ? job->ss_kz_num : 1);
    return ETRAJ_OK;
}

int etraj_run(etraj_ctx* ctx, const etraj_job* job, etraj_result* out) {
    if (!ctx || !job || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return run_job(ctx, job, out);
}

int etraj_sample_batch(etraj_ctx* ctx, const etraj_job* job, int64_t batch_id, double* init, int64_t capacity,
                       int64_t* count) {
    if (!ctx || !job || !count) return ETRAJ_ERR_INVALID_ARGUMENT;
    if (batch_id < 1 || batch_id > job->sample_t_num)
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "batch_id out of range");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return sample_range(ctx, job, batch_id - 1, 1, init, capacity, count);
}

int etraj_sample_all(etraj_ctx* ctx, const etraj_job* job, double* init, int64_t capacity, int64_t* count) {
    if (!ctx || !job || !count) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return sample_range(ctx, job, 0, job->sample_t_num, init, capacity, count);
}

int etraj_integrate(etraj_ctx* ctx, const etraj_job* job, int64_t n, const double* init, double* final_state,
                    int32_t* status, int32_t* steps) {
    if (!ctx || !job || (n > 0 && !init) || n < 0) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    std::string err;
    int st = validate_job(job, err);
    if (st != ETRAJ_OK) return set_err(ctx, st, err);
    if (n == 0) return ETRAJ_OK;
    if (n >= ((int64_t)1 << 31)) return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "n too large");
    HostJob H;
    prepare_job(job, H);
    const DJob& J = H.J;
    // unpack the reference `init` columns into a structure of arrays
    std::vector<double> x((size_t)n), y((size_t)n), kx((size_t)n), ky((size_t)n), kz((size_t)n, 0.0),
        rate((size_t)n), ph((size_t)n, 0.0), t0((size_t)n);
    std::vector<int32_t> batch((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        const double* r = init + i * J.rows;
        size_t u = (size_t)i;
        x[u] = r[0];
        y[u] = r[1];
        if (J.dim == 2) {
            kx[u] = r[2]; ky[u] = r[3]; t0[u] = r[4]; rate[u] = r[5];
        } else {
            kx[u] = r[3]; ky[u] = r[4]; kz[u] = r[5]; t0[u] = r[6]; rate[u] = r[7];
        }
        if (J.phase != ETRAJ_PHASE_CTMC) ph[u] = r[J.rows - 1];
        batch[u] = (int32_t)i;
    }
    Pipeline P;
    ETRAJ_TRY(ensure_t(ctx, "soa.x", (size_t)n, &P.soa.x));
    ETRAJ_TRY(ensure_t(ctx, "soa.y", (size_t)n, &P.soa.y));
    ETRAJ_TRY(ensure_t(ctx, "soa.kx", (size_t)n, &P.soa.kx));
    ETRAJ_TRY(ensure_t(ctx, "soa.ky", (size_t)n, &P.soa.ky));
    ETRAJ_TRY(ensure_t(ctx, "soa.kz", (size_t)n, &P.soa.kz));
    ETRAJ_TRY(ensure_t(ctx, "soa.rate", (size_t)n, &P.soa.rate));
    ETRAJ_TRY(ensure_t(ctx, "soa.phase", (size_t)n, &P.soa.phase));
    ETRAJ_TRY(ensure_t(ctx, "soa.batch", (size_t)n, &P.soa.batch));
    ETRAJ_TRY(ensure_t(ctx, "t", (size_t)n, &P.t));
    ETRAJ_TRY(ensure_t(ctx, "count", 4, &P.count));
    ETRAJ_TRY(alloc_outputs(ctx, J, n, true, P));
    cudaStream_t s = ctx->stream;
    auto up = [&](void* d, const void* h, size_t b) { cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, s); };
    up(P.soa.x, x.data(), (size_t)n * 8);
    up(P.soa.y, y.data(), (size_t)n * 8);
    up(P.soa.kx, kx.data(), (size_t)n * 8);
    up(P.soa.ky, ky.data(), (size_t)n * 8);
    up(P.soa.kz, kz.data(), (size_t)n * 8);
    up(P.soa.rate, rate.data(), (size_t)n * 8);
    up(P.soa.phase, ph.data(), (size_t)n * 8);
    up(P.soa.batch, batch.data(), (size_t)n * 4);
    up(P.t, t0.data(), (size_t)n * 8);
    unsigned long long cn = (unsigned long long)n;
    up(P.count, &cn, sizeof cn);
    int nl = 0;
    ETRAJ_TRY(launch_integrate(ctx, J, P.soa, P.t, nullptr, P.count, P.out, n, P.work, job->precision,
                               *std::min_element(t0.begin(), t0.end()), &nl));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(ctx, e, "integrate launch");
    std::vector<int32_t> stv((size_t)n);
    if (final_state)
        cudaMemcpyAsync(final_state, P.out.final_state, (size_t)n * J.n_state * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(stv.data(), P.out.status, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
    if (steps) cudaMemcpyAsync(steps, P.out.steps, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(ctx, e, "etraj_integrate");
    if (status)
        for (int64_t i = 0; i < n; ++i) status[i] = stv[(size_t)i] & 0xff;
    return ETRAJ_OK;
}

// Asynchronous jobs on one context: enqueued on its stream in submission order
// (the host set-up of the next job overlaps the device work of the previous
// one); results are staged in pinned memory and copied out at poll/wait.
int etraj_submit(etraj_ctx* ctx, const etraj_job* job, etraj_result* out, uint64_t* ticket) {
    if (!ctx || !job || !ticket || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    const uint64_t tk = ctx->next_ticket++;
    JobRec& r = ctx->jobs[tk];
    r.ticket = tk;
    r.res = *out;
    r.staged = true;
    r.status = enqueue_job(ctx, job, r);
    if (r.status != ETRAJ_OK) {
        r.error = ctx->err;
        release_job(ctx, r);
    }
    *ticket = tk;
    return ETRAJ_OK;
}

namespace {
// Completes ticket tk of ctx if it is done (blocking when `block`).
int poll_locked(etraj_ctx* ctx, uint64_t tk, etraj_result* out, bool block) {
    auto it = ctx->jobs.find(tk);
    if (it == ctx->jobs.end()) return set_err(ctx, ETRAJ_ERR_NOT_FOUND, "unknown ticket");
    JobRec& r = it->second;
    int st = r.status;
    if (st == ETRAJ_OK) {
        cudaError_t e = block ? cudaEventSynchronize(r.ev_done) : cudaEventQuery(r.ev_done);
        if (e == cudaErrorNotReady) {
            cudaGetLastError();
            return ETRAJ_ERR_NOT_READY;
        }
        if (e != cudaSuccess) {
            st = cuda_err(ctx, e, "etraj_poll");
            release_job(ctx, r);
        } else {
            st = finish_job(ctx, r);
        }
    } else {
        ctx->err = r.error;
    }
    double* ms = out->momentum_spec;
    double* amp = out->amplitude;
    *out = r.res;
    out->momentum_spec = ms;
    out->amplitude = amp;
    ctx->jobs.erase(it);
    return st;
}
}  // namespace

int etraj_poll(etraj_ctx* ctx, uint64_t ticket, etraj_result* out) {
    if (!ctx || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return poll_locked(ctx, ticket, out, false);
}

int etraj_wait(etraj_ctx* ctx, uint64_t ticket, etraj_result* out) {
    if (!ctx || !out) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return poll_locked(ctx, ticket, out, true);
}

}  // extern "C"

extern "C" {

int etraj_run_batch(etraj_ctx* ctx, const etraj_job* jobs, int n_jobs, etraj_result* results,
                    const double* weights, double* weighted_spec) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    return run_batch(ctx, jobs, n_jobs, results, weights, weighted_spec);
}

int etraj_set_graphs(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->graphs = (enable != 0);
    if (!enable && (ctx->gexec || ctx->bgexec)) {
        cudaStreamSynchronize(ctx->stream);
        if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
        if (ctx->bgexec) cudaGraphExecDestroy(ctx->bgexec);
        ctx->gexec = ctx->bgexec = nullptr;
        ctx->gkey.clear();
        ctx->bgkey.clear();
    }
    return ETRAJ_OK;
}

int etraj_set_autotune(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->autotune = (enable != 0);
    if (!enable) ctx->tiles.clear();
    return ETRAJ_OK;
}

int etraj_bulk_tile(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int* threads,
                    int* blocks_per_sm, int* refill_min) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int key = (multi ? 1000 : 0) + dimension * 100 + phase * 10 + target;
    BulkTile t = kTileDefault;
    const bool found = find_tile(ctx, key, &t);
    if (threads) *threads = t.threads;
    if (blocks_per_sm) *blocks_per_sm = t.blocks_per_sm;
    if (refill_min) *refill_min = t.refill_min;
    return found ? ETRAJ_OK : ETRAJ_ERR_NOT_FOUND;
}

int etraj_set_bulk_tile(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int threads,
                        int blocks_per_sm, int refill_min) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    const int warps = (threads / 32) * blocks_per_sm;
    if ((threads != 64 && threads != 128 && threads != 256) || blocks_per_sm < 1 || warps > 24 ||
        refill_min < 1 || refill_min > 32)
        return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int key = (multi ? 1000 : 0) + dimension * 100 + phase * 10 + target;
    BulkTile old = kTileDefault;
    find_tile(ctx, key, &old);
    ctx->tiles[key] = BulkTile{threads, blocks_per_sm, refill_min, warps > 16 ? 3 : 2, old.chunk};
    return ETRAJ_OK;
}

int etraj_bulk_step_chunk(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int* steps) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int key = (multi ? 1000 : 0) + dimension * 100 + phase * 10 + target;
    BulkTile t = kTileDefault;
    const bool found = find_tile(ctx, key, &t);
    if (steps) *steps = t.chunk;
    return found ? ETRAJ_OK : ETRAJ_ERR_NOT_FOUND;
}

int etraj_set_bulk_step_chunk(etraj_ctx* ctx, int dimension, int phase, int target, int multi, int steps) {
    if (!ctx || steps < 16 || steps > (1 << 16)) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int key = (multi ? 1000 : 0) + dimension * 100 + phase * 10 + target;
    BulkTile t = kTileDefault;
    find_tile(ctx, key, &t);
    t.chunk = steps;
    ctx->tiles[key] = t;
    return ETRAJ_OK;
}

int etraj_set_straggler_repack(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->repack = (enable != 0);
    return ETRAJ_OK;
}

int etraj_set_static_assignment(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->static_assign = (enable != 0);
    return ETRAJ_OK;
}

int etraj_set_keep_final_states(etraj_ctx* ctx, int enable) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->keep_states = (enable != 0);
    return ETRAJ_OK;
}

namespace {
// Number of survivors of the kept job, after it has finished (ticket 0: the last job).
int dump_prepare(etraj_ctx* ctx, uint64_t ticket, int64_t* n) {
    if (!ctx->dump_valid || (ticket != 0 && ticket != ctx->dump_ticket))
        return set_err(ctx, ETRAJ_ERR_NOT_FOUND,
                       "final states are kept only for the context's last job, and only when "
                       "etraj_set_keep_final_states was on when it was enqueued");
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    unsigned long long c = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&c, ctx->dump_count, sizeof c, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(ctx, e, "final states");
    *n = (int64_t)c;
    return ETRAJ_OK;
}
}  // namespace

int etraj_dump_final_states(etraj_ctx* ctx, uint64_t ticket, double* p_inf, double* phase, int32_t* status) {
    if (!ctx) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    int64_t n = 0;
    ETRAJ_TRY(dump_prepare(ctx, ticket, &n));
    if (n == 0) return ETRAJ_OK;
    const TrajOut& o = ctx->dump_out;
    cudaError_t e = cudaSuccess;
    if (p_inf && e == cudaSuccess) e = cudaMemcpy(p_inf, o.p_inf, (size_t)n * 3 * 8, cudaMemcpyDeviceToHost);
    if (phase && e == cudaSuccess) e = cudaMemcpy(phase, o.fphase, (size_t)n * 8, cudaMemcpyDeviceToHost);
    if (status && e == cudaSuccess) e = cudaMemcpy(status, o.status, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(ctx, e, "final states");
    return ETRAJ_OK;
}

int etraj_dump_step_counts(etraj_ctx* ctx, uint64_t ticket, int32_t* steps) {
    if (!ctx || !steps) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    int64_t n = 0;
    ETRAJ_TRY(dump_prepare(ctx, ticket, &n));
    if (n == 0) return ETRAJ_OK;
    cudaError_t e = cudaMemcpy(steps, ctx->dump_out.steps, (size_t)n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(ctx, e, "step counts");
    return ETRAJ_OK;
}

int etraj_dump_min_radius(etraj_ctx* ctx, uint64_t ticket, double* rmin) {
    if (!ctx || !rmin) return ETRAJ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    int64_t n = 0;
    ETRAJ_TRY(dump_prepare(ctx, ticket, &n));
    if (!ctx->dump_out.rmin)
        return set_err(ctx, ETRAJ_ERR_UNSUPPORTED, "the least radius is tracked by the FP64 path only");
    if (n == 0) return ETRAJ_OK;
    cudaError_t e = cudaMemcpy(rmin, ctx->dump_out.rmin, (size_t)n * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(ctx, e, "least radius");
    return ETRAJ_OK;
}

int etraj_stage_times(etraj_ctx* ctx, double* ms, int n) {
    if (!ctx || !ms) return 0;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->stage_valid) return 0;
    if (cudaEventSynchronize(ctx->stage_ev[etraj_ctx::kStages]) != cudaSuccess) return 0;
    int k = 0;
    for (; k < etraj_ctx::kStages && k < n; ++k) {
        float f = 0.f;
        cudaEventElapsedTime(&f, ctx->stage_ev[k], ctx->stage_ev[k + 1]);
        ms[k] = f;
    }
    return k;
}

}  // extern "C"
