// pipeline.cu -- a job's device buffers and its pipeline on the context's stream:
// allocation against the HBM budget, the kernel sequence of etraj_run (sampling,
// compaction, integration, collection, deposit; captured once as a CUDA graph
// and replayed when the launch parameters repeat), pinned staging of results and
// completion.
#include "host.h"

int set_err(etraj_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_err(etraj_ctx* ctx, cudaError_t e, const char* where) {
    return set_err(ctx, ETRAJ_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Grow-only named device buffer, counted against the context's HBM budget.
int ensure(etraj_ctx* ctx, const char* name, size_t bytes, void** out) {
    if (bytes == 0) bytes = 256;
    if (ctx->dry) {
        auto it = ctx->bufs.find(name);
        const size_t have = (it == ctx->bufs.end()) ? 0 : it->second.bytes;
        if (have < bytes) ctx->dry_bytes += (bytes + bytes / 8) - have;
        *out = nullptr;
        return ETRAJ_OK;
    }
    DevBuf& b = ctx->bufs[name];
    if (b.bytes >= bytes) {
        *out = b.p;
        return ETRAJ_OK;
    }
    size_t grow = bytes + bytes / 8;
    if (ctx->used - b.bytes + grow > ctx->budget) {
        grow = bytes;
        if (ctx->used - b.bytes + grow > ctx->budget)
            return set_err(ctx, ETRAJ_ERR_OUT_OF_MEMORY,
                           std::string("HBM budget exceeded allocating ") + name + " (" +
                               std::to_string(bytes) + " bytes; budget " + std::to_string(ctx->budget) +
                               ", in use " + std::to_string(ctx->used) + ")");
    }
    // stream-ordered (de)allocation: a context's growth never waits for the
    // work of other contexts (cudaFree would synchronize the whole device)
    if (b.p) {
        cudaFreeAsync(b.p, ctx->stream);
        ctx->used -= b.bytes;
        b.p = nullptr;
        b.bytes = 0;
    }
    cudaError_t e = cudaMallocAsync(&b.p, grow, ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, ETRAJ_ERR_OUT_OF_MEMORY, std::string("cudaMalloc ") + name + ": " + cudaGetErrorString(e));
    }
    b.bytes = grow;
    ctx->used += grow;
    *out = b.p;
    return ETRAJ_OK;
}




int alloc_sampling(etraj_ctx* ctx, HostJob& H, Pipeline& P) {
    const DJob& J = H.J;
    const size_t n = (size_t)J.n_total;
    if (J.mol.on) {
        // the molecular tables; their addresses go into the device job
        double *clm = nullptr, *wint = nullptr, *tab = nullptr;
        float* tabf = nullptr;
        if (!H.mol_clm.empty()) ETRAJ_TRY(ensure_t(ctx, "mol.clm", H.mol_clm.size(), &clm));
        if (!H.mol_wint.empty()) ETRAJ_TRY(ensure_t(ctx, "mol.wint", H.mol_wint.size(), &wint));
        ETRAJ_TRY(ensure_t(ctx, "mol.tab", (size_t)J.n_t * (size_t)J.mol.stride, &tab));
        ETRAJ_TRY(ensure_t(ctx, "mol.tabf", (size_t)J.n_t * (size_t)J.mol.stride, &tabf));
        H.J.mol.clm = clm;
        H.J.mol.wint = wint;
        H.J.mol.tab = tab;
        H.J.mol.tabf = tabf;
    }
    ETRAJ_TRY(ensure_t(ctx, "t", H.t.size(), &P.t));
    ETRAJ_TRY(ensure_t(ctx, "kd", H.kd.size(), &P.kd));
    ETRAJ_TRY(ensure_t(ctx, "kz", H.kz.size(), &P.kz));
    ETRAJ_TRY(ensure_t(ctx, "batches", (size_t)J.n_t, &P.batches));
    ETRAJ_TRY(ensure_t(ctx, "soa.x", n, &P.soa.x));
    ETRAJ_TRY(ensure_t(ctx, "soa.y", n, &P.soa.y));
    ETRAJ_TRY(ensure_t(ctx, "soa.kx", n, &P.soa.kx));
    ETRAJ_TRY(ensure_t(ctx, "soa.ky", n, &P.soa.ky));
    ETRAJ_TRY(ensure_t(ctx, "soa.kz", n, &P.soa.kz));
    ETRAJ_TRY(ensure_t(ctx, "soa.rate", n, &P.soa.rate));
    if (J.phase != ETRAJ_PHASE_CTMC) ETRAJ_TRY(ensure_t(ctx, "soa.phase", n, &P.soa.phase));
    else P.soa.phase = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "soa.batch", n, &P.soa.batch));
    ETRAJ_TRY(ensure_t(ctx, "flag", n, &P.flag));
    ETRAJ_TRY(ensure_t(ctx, "idx", n, &P.idx));
    ETRAJ_TRY(ensure_t(ctx, "block_sums", (size_t)compact_blocks((int64_t)n) + 1, &P.block_sums));
    ETRAJ_TRY(ensure_t(ctx, "count", 4, &P.count));
    return ETRAJ_OK;
}

int alloc_outputs(etraj_ctx* ctx, const DJob& J, int64_t max_n, bool with_state, Pipeline& P) {
    const size_t n = (size_t)(max_n > 0 ? max_n : 1);
    if (!ctx->dry) ctx->dump_valid = false;  // the buffers now belong to a new job
    ETRAJ_TRY(ensure_t(ctx, "out.key", n, &P.out.key));
    ETRAJ_TRY(ensure_t(ctx, "out.c_re", n, &P.out.c_re));
    ETRAJ_TRY(ensure_t(ctx, "out.c_im", n, &P.out.c_im));
    ETRAJ_TRY(ensure_t(ctx, "out.w_ion", n, &P.out.w_ion));
    ETRAJ_TRY(ensure_t(ctx, "out.w_unc", n, &P.out.w_unc));
    ETRAJ_TRY(ensure_t(ctx, "out.status", n, &P.out.status));
    ETRAJ_TRY(ensure_t(ctx, "out.steps", n, &P.out.steps));
    if (with_state) ETRAJ_TRY(ensure_t(ctx, "out.final_state", n * (size_t)J.n_state, &P.out.final_state));
    else P.out.final_state = nullptr;
    if (ctx->keep_states) {
        ETRAJ_TRY(ensure_t(ctx, "out.p_inf", 3 * n, &P.out.p_inf));
        ETRAJ_TRY(ensure_t(ctx, "out.fphase", n, &P.out.fphase));
        ETRAJ_TRY(ensure_t(ctx, "out.rmin", n, &P.out.rmin));
    } else {
        P.out.p_inf = nullptr;
        P.out.fphase = nullptr;
        P.out.rmin = nullptr;
    }
    void* dep = nullptr;
    ETRAJ_TRY(ensure(ctx, "deposit", deposit_scratch_bytes(max_n), &dep));
    deposit_scratch_carve(dep, max_n, &P.dep);
    ETRAJ_TRY(ensure_t(ctx, "spec_re", (size_t)J.grid, &P.spec_re));
    ETRAJ_TRY(ensure_t(ctx, "spec_im", (size_t)J.grid, &P.spec_im));
    ETRAJ_TRY(ensure_t(ctx, "mspec", (size_t)J.grid, &P.mspec));
    ETRAJ_TRY(ensure_t(ctx, "sums", 2, &P.sums));
    ETRAJ_TRY(ensure_t(ctx, "counters", 1, &P.counters));
    ETRAJ_TRY(ensure_t(ctx, "work", kBulkCounters, &P.work));
    return ETRAJ_OK;
}

// The candidate kernel of a job: the bulk path samples in FP32 (ADK, SPANE and
// WFAT, atoms and molecules, while every kept rate stays in FP32's normal
// range; SPA for atoms), the FP64 path and molecular SPA in FP64.
int launch_sampler(int precision, const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                   DBatch* batches, InitSoA soa, uint8_t* flag, int sm_count, cudaStream_t s,
                   const SampleScratch* scr) {
    // (a Gaussian-proposal job samples in FP64 on every path)
    const bool fp32 = precision == ETRAJ_PRECISION_FP32_BULK && !J.gauss &&
                      (J.method == ETRAJ_SAMPLER_SPA ? !J.mol.on : J.cutoff >= kSample32MinCutoff);
    return fp32 ? launch_sample32_range(J, b0, nb, kd, kz, batches, soa, flag, sm_count, s)
                : launch_sample_range(J, b0, nb, kd, kz, batches, soa, flag, sm_count, s, scr);
}

// The FP64 SPA sampler's list and margin: double-float jobs drop candidates whose
// FP32 rate is below 0.8 x the cutoff (the same electrons survive: FP32's SPA rate
// is within 3e-3 of FP64's where both solve); FP64 jobs only those 100 times
// below, which keeps the oracle's sampler exactly.
SampleScratch sample_scratch(const Pipeline& P, int64_t n, int precision) {
    const float log_margin = (precision == ETRAJ_PRECISION_FP32_DF) ? -0.22314355f : -4.6051702f;
    return SampleScratch{P.idx, P.block_sums, compact_blocks(n) + 1, P.count, log_margin};
}

// Copies a job's host inputs (time and momentum samples, molecular tables) to the device.
void upload_inputs(const HostJob& H, const Pipeline& P, cudaStream_t s) {
    cudaMemcpyAsync(P.t, H.t.data(), H.t.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(P.kd, H.kd.data(), H.kd.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(P.kz, H.kz.data(), H.kz.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (!H.mol_clm.empty())
        cudaMemcpyAsync((void*)H.J.mol.clm, H.mol_clm.data(), H.mol_clm.size() * sizeof(double),
                        cudaMemcpyHostToDevice, s);
    if (!H.mol_wint.empty())
        cudaMemcpyAsync((void*)H.J.mol.wint, H.mol_wint.data(), H.mol_wint.size() * sizeof(double),
                        cudaMemcpyHostToDevice, s);
}

// Smallest radius beyond which every exp(-b r) term of the SAE potential and
// force is below 2^-26 Z: |a| (1 + b r) e^{-b r} (potential and force
// brackets), |a2| r e^{-b2 r} (potential) and |a2 b2| (r^2 + sc) e^{-b2 r}
// (force, relative to Z / r^2).  Each is decreasing beyond its maximum, so the
// first radius past all maxima where all hold is returned (1e30: never).
float sae_far_radius(const DTarget& T) {
    if (T.kind != ETRAJ_TARGET_SAE) return 1e30f;
    const double eps = std::ldexp(1.0, -26) * T.Z;
    const double a[3] = {T.a1, T.a2, T.a3}, b[3] = {T.b1, T.b2, T.b3};
    double rmin = 0.0;
    for (int i = 0; i < 3; ++i) {
        if (a[i] == 0.0) continue;
        if (!(b[i] > 0.0)) return 1e30f;
        rmin = std::max(rmin, 2.0 / b[i]);
    }
    auto ok = [&](double r) {
        for (int i = 0; i < 3; ++i) {
            if (a[i] == 0.0) continue;
            const double e = std::exp(-b[i] * r);
            if (std::fabs(a[i]) * (1.0 + b[i] * r) * e >= eps) return false;
            if (i == 1 && std::fabs(a[i]) * r * e >= eps) return false;
            if (i == 1 && std::fabs(a[i] * b[i]) * (r * r + T.sc) * e >= eps) return false;
        }
        return true;
    };
    double r = rmin;
    while (!ok(r)) {
        r *= 1.01;
        r += 0.01;
        if (r > 1e6) return 1e30f;
    }
    return (float)(r * 1.01);
}

// Bulk-integrator parameters: field table spanning [tmin, t_final] with
// spacing T_min/512 (T_min the shortest laser period).
void prepare_bulk(const DJob& J, double tmin, BulkParams& B) {
    std::memset(&B, 0, sizeof B);
    B.dim = J.dim;
    B.phase = J.phase;
    B.tgt = J.target.kind;
    double T = J.laser.m[0].period;
    if (J.laser.nmono == 2) T = std::min(T, J.laser.m[1].period);
    const double h = T / 512.0;
    B.T0 = tmin - h;
    B.n_int = (int)std::ceil((J.t_final - B.T0) / h) + 2;
    B.inv_h_d = 1.0 / h;
    B.max_iters = kBulkMaxIters;
    B.h = (float)h;
    B.inv_h = (float)(1.0 / h);
    B.t_final = J.t_final;
    const double q = (J.t_final - B.T0) / h;
    const double fl = std::floor(q);
    B.nf = (int)fl;
    B.ff = (float)(q - fl);
    B.rtol = (float)J.rtol;
    B.table_in_smem = ((size_t)B.n_int * 2 * sizeof(float4) <= (size_t)96 * 1024) ? 1 : 0;
    B.threads = 256;
    B.blocks_per_sm = 2;
    B.refill_min = 4;
    B.occ = 2;
    const DTarget& T_ = J.target;
    B.Z = (float)T_.Z;
    B.Ip = (float)T_.Ip;
    B.sc = (float)T_.sc;
    B.a1 = (float)T_.a1; B.b1 = (float)T_.b1;
    B.a2 = (float)T_.a2; B.b2 = (float)T_.b2;
    B.a3 = (float)T_.a3; B.b3 = (float)T_.b3;
    B.a2b2 = (float)(T_.a2 * T_.b2);
    B.r_far = sae_far_radius(T_);
}

// Double-float integrator parameters (integrate_setup.h) and its launch shapes:
// persistent grids, as many blocks as are resident, and no more than the job
// keeps busy (~4 electrons per lane).
void prepare_df(const DJob& J, double tmin, int64_t max_n, int sm_count, DFParams& D) {
    prepare_df_params(J, tmin, max_n, D);
    D.threads = df_threads(false);
    D.threads_main = df_threads(true);
    for (int main = 0; main < 2; ++main) {
        const int th = main ? D.threads_main : D.threads;
        const int64_t lanes_per_block = (int64_t)th * 4;
        const int64_t want = (max_n + lanes_per_block - 1) / lanes_per_block;
        const int64_t cap = (int64_t)sm_count * df_blocks_per_sm(D.dim, D.phase, D.tgt, main != 0, th);
        (main ? D.blocks_main : D.blocks) = (int)(want < 1 ? 1 : (want < cap ? want : cap));
    }
}

// The double-float integrator's buffers: the field table and the carried electrons
// (kDfCarryWords x max_n words).
int attach_df(etraj_ctx* ctx, DFParams& D) {
    float4* tab = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "field_table_df", (size_t)D.n_int * kDfTableF4, &tab));
    ETRAJ_TRY(ensure_t(ctx, "df_carry", (size_t)kDfCarryWords * (size_t)(D.max_n > 0 ? D.max_n : 1), &D.carry));
    D.table = tab;
    return ETRAJ_OK;
}


// ---- pinned staging and events, pooled per context ---------------------------------
int get_pinned(etraj_ctx* ctx, size_t bytes, PinnedBlock* out) {
    for (size_t i = 0; i < ctx->pinned_pool.size(); ++i) {
        if (ctx->pinned_pool[i].bytes >= bytes) {
            *out = ctx->pinned_pool[i];
            ctx->pinned_pool.erase(ctx->pinned_pool.begin() + (long)i);
            return ETRAJ_OK;
        }
    }
    void* p = nullptr;
    cudaError_t e = cudaMallocHost(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, ETRAJ_ERR_OUT_OF_MEMORY, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    out->p = p;
    out->bytes = bytes;
    return ETRAJ_OK;
}

void put_pinned(etraj_ctx* ctx, void* p, size_t bytes) {
    if (!p) return;
    if (ctx->pinned_pool.size() < 64) ctx->pinned_pool.push_back(PinnedBlock{p, bytes});
    else cudaFreeHost(p);
}

cudaEvent_t get_event(etraj_ctx* ctx) {
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

void release_job(etraj_ctx* ctx, JobRec& r) {
    if (r.staged) {
        put_pinned(ctx, r.pinned, r.pinned_bytes);
        if (r.ev_start) ctx->event_pool.push_back(r.ev_start);
        if (r.ev_done) ctx->event_pool.push_back(r.ev_done);
    }
    r.pinned = nullptr;
    r.ev_start = r.ev_done = nullptr;
}

// Device bytes a job would add to this context's buffers (0 for an invalid job,
// whose error comes at enqueue).
size_t plan_growth(etraj_ctx* ctx, const etraj_job* job) {
    std::string err;
    if (validate_job(job, err) != ETRAJ_OK) return 0;
    HostJob H;
    prepare_job(job, H);
    Pipeline P;
    ctx->dry = true;
    ctx->dry_bytes = 0;
    alloc_sampling(ctx, H, P);
    const bool bulk = (job->precision == ETRAJ_PRECISION_FP32_BULK);
    alloc_outputs(ctx, H.J, H.J.n_total, job->precision != ETRAJ_PRECISION_FP64, P);
    if (job->precision == ETRAJ_PRECISION_FP32_DF) {
        DFParams D;
        prepare_df_params(H.J, H.t.front(), H.J.n_total, D);
        attach_df(ctx, D);
    }
    if (bulk) {
        BulkParams B;
        prepare_bulk(H.J, H.t.front(), B);
        float4* tab = nullptr;
        ensure_t(ctx, "field_table", (size_t)B.n_int * 2, &tab);
        B.max_n = H.J.n_total;
        attach_park(ctx, B);
    }
    ctx->dry = false;
    return ctx->dry_bytes;
}

// The device work of one job, from the per-batch prologue to the deposit.
int enqueue_kernels(etraj_ctx* ctx, const etraj_job* job, const HostJob& H, const Pipeline& P, int* nl) {
    const DJob& J = H.J;
    cudaStream_t s = ctx->stream;
    int launches = 0;
    rec(ctx, ctx->stage_ev[0], s);
    launches += launch_batch_prepare(J, P.t, P.batches, s);
    const SampleScratch scr = sample_scratch(P, J.n_total, job->precision);
    launches += launch_sampler(job->precision, J, 0, J.n_t, P.kd, P.kz, P.batches, P.soa, P.flag, ctx->sm_count, s,
                               &scr);
    rec(ctx, ctx->stage_ev[1], s);
    launches += launch_compact(P.flag, J.n_total, P.idx, P.block_sums, compact_blocks(J.n_total) + 1, P.count, s);
    rec(ctx, ctx->stage_ev[2], s);
    ETRAJ_TRY(launch_integrate(ctx, J, P.soa, P.t, P.idx, P.count, P.out, J.n_total, P.work, job->precision,
                               H.t.front(), &launches, ctx->stage_ev + 3));
    rec(ctx, ctx->stage_ev[5], s);
    launches += launch_deposit(J, P.out, P.count, J.n_total, P.dep, P.spec_re, P.spec_im, P.mspec, P.sums,
                               P.counters, s);
    rec(ctx, ctx->stage_ev[6], s);
    ctx->stage_valid = true;
    *nl = launches;
    return ETRAJ_OK;
}

// With ctx->graphs the kernel sequence is captured once into a CUDA graph and
// replayed while the launch parameters (device job, buffer addresses, bulk
// launch shape, table size) stay the same; a job that needs an autotuning pass
// first runs without a graph.
int enqueue_kernels_maybe_graph(etraj_ctx* ctx, const etraj_job* job, const HostJob& H, const Pipeline& P,
                                int* launches) {
    const DJob& J = H.J;
    bool use_graph = ctx->graphs;
    int tile_k = -1;
    size_t n_int = 0;
    if (use_graph && job->precision == ETRAJ_PRECISION_FP32_BULK) {
        BulkParams B;
        prepare_bulk(J, H.t.front(), B);
        B.max_n = J.n_total;
        n_int = (size_t)B.n_int;
        tile_k = tile_key(B);
        if (ctx->autotune && !find_tile(ctx, tile_k, nullptr) && B.max_n >= ((int64_t)1 << 18)) use_graph = false;
        float4* tab = nullptr;  // allocate the field table and the park buffer outside the capture
        ETRAJ_TRY(ensure_t(ctx, "field_table", n_int * 2, &tab));
        ETRAJ_TRY(attach_park(ctx, B));
    }
    if (use_graph && job->precision == ETRAJ_PRECISION_FP32_DF) {
        DFParams D;  // allocate the field table and the carry buffer outside the capture
        prepare_df_params(J, H.t.front(), J.n_total, D);
        n_int = (size_t)D.n_int;
        ETRAJ_TRY(attach_df(ctx, D));
    }
    if (!use_graph) return enqueue_kernels(ctx, job, H, P, launches);
    const char* tab_name = (job->precision == ETRAJ_PRECISION_FP32_DF) ? "field_table_df" : "field_table";
    const char* aux_name = (job->precision == ETRAJ_PRECISION_FP32_DF) ? "df_carry" : "park";
    void* ptrs[2] = {ctx->bufs.count(tab_name) ? ctx->bufs[tab_name].p : nullptr,
                     ctx->bufs.count(aux_name) ? ctx->bufs[aux_name].p : nullptr};
    std::vector<unsigned char> key(sizeof J + sizeof P + sizeof(int) * 3 + sizeof(size_t) + sizeof ptrs);
    unsigned char* k = key.data();
    std::memcpy(k, &J, sizeof J);
    k += sizeof J;
    std::memcpy(k, &P, sizeof P);
    k += sizeof P;
    BulkTile t = kTileDefault;
    find_tile(ctx, tile_k, &t);
    const int extra[3] = {job->precision, t.threads * 1000 + t.blocks_per_sm * 10 + t.occ,
                          (t.refill_min * 4 + (ctx->repack ? 1 : 0) + (ctx->static_assign ? 2 : 0)) * 65536 +
                              t.chunk};
    std::memcpy(k, extra, sizeof extra);
    k += sizeof extra;
    std::memcpy(k, &n_int, sizeof n_int);
    k += sizeof n_int;
    std::memcpy(k, ptrs, sizeof ptrs);
    cudaStream_t s = ctx->stream;
    if (ctx->gexec && key == ctx->gkey) {
        cudaError_t e = cudaGraphLaunch(ctx->gexec, s);
        if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGraphLaunch");
        *launches = ctx->glaunches;
        ctx->stage_valid = true;
        return ETRAJ_OK;
    }
    if (key != ctx->gseen) {
        // first sighting: run directly; the same launch parameters again are captured
        ctx->gseen = key;
        return enqueue_kernels(ctx, job, H, P, launches);
    }
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return enqueue_kernels(ctx, job, H, P, launches);
    }
    ctx->capturing = true;
    const int st = enqueue_kernels(ctx, job, H, P, launches);
    ctx->capturing = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    cudaGraphExec_t ex = nullptr;
    if (st == ETRAJ_OK && e == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
        cudaGraphDestroy(g);
        if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = ex;
        ctx->gkey = key;
        ctx->glaunches = *launches;
        e = cudaGraphLaunch(ex, s);
        if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGraphLaunch");
        return ETRAJ_OK;
    }
    // capture failed: run the sequence directly
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (st != ETRAJ_OK) return st;
    return enqueue_kernels(ctx, job, H, P, launches);
}

// Enqueues one whole job on the context's stream: host set-up, copies of the
// time and momentum samples, every kernel, and the copies of the results.  With
// r.staged the results go to a pinned block and r.ev_done marks completion;
// otherwise they go straight to the caller's buffers.
int enqueue_job(etraj_ctx* ctx, const etraj_job* job, JobRec& r) {
    std::string err;
    int st = validate_job(job, err);
    if (st != ETRAJ_OK) return set_err(ctx, st, err);
    HostJob H;
    prepare_job(job, H);
    const DJob& J = H.J;
    Pipeline P;
    ETRAJ_TRY(alloc_sampling(ctx, H, P));
    ETRAJ_TRY(alloc_outputs(ctx, J, J.n_total, job->precision != ETRAJ_PRECISION_FP64, P));
    r.grid = J.grid;
    r.coherent = (J.phase != ETRAJ_PHASE_CTMC);
    const bool want_spec = r.res.momentum_spec != nullptr;
    const bool want_amp = r.res.amplitude != nullptr && r.coherent;
    double* dst_sums = r.direct_sums;
    Counters* dst_cnt = &r.direct_cnt;
    double* dst_spec = r.res.momentum_spec;
    double* dst_amp = r.res.amplitude;
    if (r.staged) {
        const size_t bytes = 2 * sizeof(double) + sizeof(Counters) + (want_spec ? (size_t)J.grid * 8 : 0) +
                             (want_amp ? (size_t)J.grid * 16 : 0);
        PinnedBlock blk;
        ETRAJ_TRY(get_pinned(ctx, bytes, &blk));
        r.pinned = blk.p;
        r.pinned_bytes = blk.bytes;
        char* base = (char*)blk.p;
        dst_sums = (double*)base;
        dst_cnt = (Counters*)(base + 2 * sizeof(double));
        char* rest = base + 2 * sizeof(double) + sizeof(Counters);
        dst_spec = want_spec ? (double*)rest : nullptr;
        dst_amp = want_amp ? (double*)(rest + (want_spec ? (size_t)J.grid * 8 : 0)) : nullptr;
        r.ev_start = get_event(ctx);
        r.ev_done = get_event(ctx);
        if (!r.ev_start || !r.ev_done) return set_err(ctx, ETRAJ_ERR_CUDA, "cudaEventCreate failed");
    } else {
        r.ev_start = ctx->ev0;
        r.ev_done = ctx->ev1;
    }
    cudaStream_t s = ctx->stream;
    upload_inputs(H, P, s);
    cudaEventRecord(r.ev_start, s);
    int launches = 0;
    ETRAJ_TRY(enqueue_kernels_maybe_graph(ctx, job, H, P, &launches));
    cudaMemcpyAsync(dst_sums, P.sums, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(dst_cnt, P.counters, sizeof(Counters), cudaMemcpyDeviceToHost, s);
    if (dst_spec) cudaMemcpyAsync(dst_spec, P.mspec, (size_t)J.grid * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (dst_amp) {
        cudaMemcpy2DAsync(dst_amp, 2 * sizeof(double), P.spec_re, sizeof(double), sizeof(double), (size_t)J.grid,
                          cudaMemcpyDeviceToHost, s);
        cudaMemcpy2DAsync(dst_amp + 1, 2 * sizeof(double), P.spec_im, sizeof(double), sizeof(double), (size_t)J.grid,
                          cudaMemcpyDeviceToHost, s);
    }
    cudaEventRecord(r.ev_done, s);
    r.launches = launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(ctx, e, "kernel launch");
    ctx->dump_valid = ctx->keep_states;
    ctx->dump_ticket = r.ticket;
    ctx->dump_out = P.out;
    if (job->precision != ETRAJ_PRECISION_FP64) ctx->dump_out.rmin = nullptr;  // filled by the FP64 path only
    ctx->dump_count = P.count;
    return ETRAJ_OK;
}

// Completes a job whose ev_done has been reached: fills the caller's result.
int finish_job(etraj_ctx* ctx, JobRec& r) {
    const double* sums = r.direct_sums;
    const Counters* cnt = &r.direct_cnt;
    if (r.staged) {
        const char* base = (const char*)r.pinned;
        sums = (const double*)base;
        cnt = (const Counters*)(base + 2 * sizeof(double));
        const char* rest = base + 2 * sizeof(double) + sizeof(Counters);
        if (r.res.momentum_spec) {
            std::memcpy(r.res.momentum_spec, rest, (size_t)r.grid * 8);
            rest += (size_t)r.grid * 8;
        }
        if (r.res.amplitude && r.coherent) std::memcpy(r.res.amplitude, rest, (size_t)r.grid * 16);
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.ev_start, r.ev_done);
    r.res.ion_prob = sums[0];
    r.res.ion_prob_uncollected = sums[1];
    r.res.num_effective_traj = (int64_t)cnt->n_eff;
    r.res.num_failed_traj = (int64_t)cnt->n_failed;
    r.res.num_ionized_traj = (int64_t)cnt->n_ionized;
    r.res.num_steps = (int64_t)cnt->n_steps;
    r.res.num_kernel_launches = r.launches;
    r.res.elapsed_ms = ms;
    const bool sort_failed = cnt->sort_err != 0;
    release_job(ctx, r);
    if (sort_failed) return set_err(ctx, ETRAJ_ERR_CUDA, "deposit: a look-back wait of the radix sort gave up");
    return ETRAJ_OK;
}

int run_job(etraj_ctx* ctx, const etraj_job* job, etraj_result* res) {
    JobRec r;
    r.res = *res;
    r.staged = false;
    ETRAJ_TRY(enqueue_job(ctx, job, r));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_err(ctx, e, "etraj_run");
    ETRAJ_TRY(finish_job(ctx, r));
    *res = r.res;
    return ETRAJ_OK;
}

