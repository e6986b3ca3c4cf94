// batch.cu -- multi-instance batches (many jobs in one integrator launch) and
// sampling without integration (etraj_sample_all).
#include "host.h"

// ---- multi-instance batch: many jobs in one integrator launch ------------------------
// The instances' time samples, candidates and field tables are concatenated;
// sampling runs per instance, then one compaction, one bulk-integrator launch
// whose work stealing spans every instance, one collection, one deposit into
// an instance-major grid, and per-instance reductions.  Every per-instance
// result equals that of the same job run alone.
int run_batch(etraj_ctx* ctx, const etraj_job* jobs, int n, etraj_result* res, const double* weights,
              double* wspec) {
    if (!jobs || !res || n < 1 || n > kMaxInstances)
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "etraj_run_batch: 1 to 64 jobs");
    if ((weights == nullptr) != (wspec == nullptr))
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "etraj_run_batch: weights and weighted_spec go together");
    const etraj_job& j0 = jobs[0];
    for (int i = 0; i < n; ++i) {
        std::string err;
        const int st = validate_job(&jobs[i], err);
        if (st != ETRAJ_OK) return set_err(ctx, st, "job " + std::to_string(i) + ": " + err);
        const etraj_job& ji = jobs[i];
        if (ji.target.kind == ETRAJ_TARGET_MOLECULE)
            return set_err(ctx, ETRAJ_ERR_UNSUPPORTED,
                           "etraj_run_batch: molecular targets are run one job at a time (etraj_run, etraj_submit)");
        bool same = ji.precision == ETRAJ_PRECISION_FP32_BULK && ji.dimension == j0.dimension &&
                    ji.traj_phase_method == j0.traj_phase_method && ji.traj_rtol == j0.traj_rtol &&
                    std::memcmp(&ji.target, &j0.target, sizeof ji.target) == 0;
        for (int d = 0; d < 3; ++d)
            same = same && ji.final_p_num[d] == j0.final_p_num[d] && ji.final_p_max[d] == j0.final_p_max[d];
        if (!same)
            return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT,
                           "etraj_run_batch: job " + std::to_string(i) +
                               " differs from job 0 in precision (must be FP32_BULK), dimension, phase method, "
                               "rtol, target or momentum grid");
    }
    std::vector<HostJob> H((size_t)n);
    for (int i = 0; i < n; ++i) prepare_job(&jobs[i], H[(size_t)i]);
    const int64_t grid1 = H[0].J.grid;
    if ((int64_t)n * grid1 >= (int64_t)0xFFFFFFFFll)
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "etraj_run_batch: instances x grid >= 2^32 bins");
    std::vector<int64_t> toff(n + 1, 0), koff(n + 1, 0), zoff(n + 1, 0), coff(n + 1, 0), tab_off(n + 1, 0);
    std::vector<BulkParams> B((size_t)n);
    for (int i = 0; i < n; ++i) {
        const HostJob& h = H[(size_t)i];
        toff[i + 1] = toff[i] + (int64_t)h.t.size();
        koff[i + 1] = koff[i] + (int64_t)h.kd.size();
        zoff[i + 1] = zoff[i] + (int64_t)h.kz.size();
        coff[i + 1] = coff[i] + h.J.n_total;
        prepare_bulk(h.J, h.t.front(), B[(size_t)i]);
        tab_off[i + 1] = tab_off[i] + 2 * (int64_t)B[(size_t)i].n_int;
    }
    const int64_t N = coff[n];
    if (toff[n] >= (int64_t)1 << 31)
        return set_err(ctx, ETRAJ_ERR_INVALID_ARGUMENT, "etraj_run_batch: more than 2^31 time samples");
    std::vector<double> t_all((size_t)toff[n]), kd_all((size_t)koff[n]), kz_all((size_t)zoff[n]);
    for (int i = 0; i < n; ++i) {
        const HostJob& h = H[(size_t)i];
        std::copy(h.t.begin(), h.t.end(), t_all.begin() + toff[i]);
        std::copy(h.kd.begin(), h.kd.end(), kd_all.begin() + koff[i]);
        std::copy(h.kz.begin(), h.kz.end(), kz_all.begin() + zoff[i]);
    }
    // buffers (the single-job names, sized for the whole batch)
    Pipeline P;
    DJob Jgrid = H[0].J;
    Jgrid.grid = (int64_t)n * grid1;
    HostJob Hsz;
    Hsz.J = Jgrid;
    Hsz.J.n_total = N;
    Hsz.J.n_t = toff[n];
    Hsz.t = t_all;
    Hsz.kd = kd_all;
    Hsz.kz = kz_all;
    ETRAJ_TRY(alloc_sampling(ctx, Hsz, P));
    ETRAJ_TRY(alloc_outputs(ctx, Jgrid, N, true, P));
    float4* tab = nullptr;
    BulkInst* d_inst = nullptr;
    int64_t* d_seg = nullptr;
    double *d_scr = nullptr, *d_isums = nullptr, *d_w = nullptr, *d_wout = nullptr;
    Counters* d_icnt = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "field_table", (size_t)tab_off[n], &tab));
    ETRAJ_TRY(ensure_t(ctx, "batch.inst", (size_t)n, &d_inst));
    ETRAJ_TRY(ensure_t(ctx, "batch.seg", (size_t)n + 1, &d_seg));
    ETRAJ_TRY(ensure_t(ctx, "batch.scratch", instance_scratch_doubles(N, n), &d_scr));
    ETRAJ_TRY(ensure_t(ctx, "batch.sums", (size_t)2 * n, &d_isums));
    ETRAJ_TRY(ensure_t(ctx, "batch.counters", (size_t)n, &d_icnt));
    if (weights) {
        ETRAJ_TRY(ensure_t(ctx, "batch.w", (size_t)n, &d_w));
        ETRAJ_TRY(ensure_t(ctx, "batch.wout", (size_t)grid1, &d_wout));
    }
    std::vector<BulkInst> inst((size_t)n);
    for (int i = 0; i < n; ++i) {
        const BulkParams& b = B[(size_t)i];
        BulkInst& q = inst[(size_t)i];
        q.table = tab + tab_off[i];
        q.cand_end = coff[i + 1];
        q.T0 = b.T0;
        q.inv_h_d = b.inv_h_d;
        q.t_final = b.t_final;
        q.t_off = (int)toff[i];
        q.n_int = b.n_int;
        q.nf = b.nf;
        q.ff = b.ff;
        q.h = b.h;
        q.inv_h = b.inv_h;
    }
    cudaStream_t s = ctx->stream;
    cudaMemcpyAsync(P.t, t_all.data(), t_all.size() * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(P.kd, kd_all.data(), kd_all.size() * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(P.kz, kz_all.data(), kz_all.size() * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_inst, inst.data(), inst.size() * sizeof(BulkInst), cudaMemcpyHostToDevice, s);
    if (weights) cudaMemcpyAsync(d_w, weights, (size_t)n * 8, cudaMemcpyHostToDevice, s);
    BulkParams M = B[0];
    M.table = nullptr;
    M.table_in_smem = 0;
    M.max_n = N;
    M.inst = d_inst;
    M.n_inst = n;
    // a batch runs as one launch (no rounds): it is throughput work, and its
    // resume rounds would run the parked electrons on a few SMs while no other
    // job waits for the rest (measured 140 ms against 121 ms for 64 instances)
    M.park_buf = nullptr;
    M.park_cap = 0;
    // the device work of the batch, from the first sampling launch to the weighted sum
    auto enqueue = [&](int* nl) -> int {
        int launches = 0;
        rec(ctx, ctx->ev0, s);
        rec(ctx, ctx->stage_ev[0], s);
        for (int i = 0; i < n; ++i) {
            const DJob& J = H[(size_t)i].J;
            DBatch* bat = P.batches + toff[i];
            launches += launch_batch_prepare(J, P.t + toff[i], bat, s);
            InitSoA so = P.soa;
            const int64_t c = coff[i];
            so.x += c; so.y += c; so.kx += c; so.ky += c; so.kz += c; so.rate += c; so.batch += c;
            if (so.phase) so.phase += c;
            launches += launch_sampler(ETRAJ_PRECISION_FP32_BULK, J, 0, J.n_t, P.kd + koff[i], P.kz + zoff[i], bat, so,
                                       P.flag + c, ctx->sm_count, s, nullptr);
        }
        rec(ctx, ctx->stage_ev[1], s);
        launches += launch_compact(P.flag, N, P.idx, P.block_sums, compact_blocks(N) + 1, P.count, s);
        rec(ctx, ctx->stage_ev[2], s);
        for (int i = 0; i < n; ++i) {
            const BulkParams& b = B[(size_t)i];
            launches += launch_field_table(H[(size_t)i].J, b.T0, 1.0 / b.inv_h_d, b.n_int, tab + tab_off[i], s);
        }
        ETRAJ_TRY(tuned_bulk_launch(ctx, M, P.soa, P.t, P.idx, P.count, P.work, P.out, &launches, ctx->stage_ev + 3));
        launches += launch_collect_bulk(H[0].J, P.soa, P.t, P.idx, P.count, P.out, N, ctx->sm_count, s, d_inst, n);
        rec(ctx, ctx->stage_ev[5], s);
        launches += launch_deposit(Jgrid, P.out, P.count, N, P.dep, P.spec_re, P.spec_im, P.mspec, P.sums, P.counters, s);
        launches += launch_instance_reductions(P.out, P.idx, P.count, d_inst, n, d_seg, d_scr, d_isums, d_icnt, s);
        if (weights) launches += launch_weighted_sum(P.mspec, n, grid1, d_w, d_wout, s);
        rec(ctx, ctx->stage_ev[6], s);
        rec(ctx, ctx->ev1, s);
        *nl = launches;
        return ETRAJ_OK;
    };
    int launches = 0;
    BulkTile tile;
    const bool tuned = !ctx->autotune || N < ((int64_t)1 << 18) || find_tile(ctx, tile_key(M), &tile);
    if (ctx->graphs && tuned) {
        // replayed when the same batch runs again on the same buffers and launch shape
        // (the inputs above are copied before and the results read after the graph)
        std::vector<unsigned char> key(1 + (size_t)n * sizeof(etraj_job) + sizeof P + 10 * sizeof(void*) +
                                       3 * sizeof(int));
        unsigned char* k = key.data();
        *k++ = 'B';
        std::memcpy(k, jobs, (size_t)n * sizeof(etraj_job));
        k += (size_t)n * sizeof(etraj_job);
        std::memcpy(k, &P, sizeof P);
        k += sizeof P;
        const void* ptrs[10] = {tab, d_inst, d_seg, d_scr, d_isums, d_icnt, d_w, d_wout, P.work, nullptr};
        std::memcpy(k, ptrs, sizeof ptrs);
        k += sizeof ptrs;
        BulkTile t = kTileDefault;
        find_tile(ctx, tile_key(M), &t);
        const int extra[3] = {t.threads * 1000 + t.blocks_per_sm * 10 + t.occ, t.refill_min * 65536 + t.chunk,
                              (ctx->static_assign ? 1 : 0) + (weights ? 2 : 0)};
        std::memcpy(k, extra, sizeof extra);
        if (ctx->bgexec && key == ctx->bgkey) {
            cudaError_t e = cudaGraphLaunch(ctx->bgexec, s);
            if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGraphLaunch (batch)");
            launches = ctx->bglaunches;
        } else if (key != ctx->bgseen) {
            ctx->bgseen = key;  // first sighting: direct; the same batch again is captured
            ETRAJ_TRY(enqueue(&launches));
        } else if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            ctx->capturing = true;
            const int st = enqueue(&launches);
            ctx->capturing = false;
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(s, &g);
            cudaGraphExec_t ex = nullptr;
            if (st == ETRAJ_OK && e == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
                cudaGraphDestroy(g);
                if (ctx->bgexec) cudaGraphExecDestroy(ctx->bgexec);
                ctx->bgexec = ex;
                ctx->bgkey = key;
                ctx->bglaunches = launches;
                e = cudaGraphLaunch(ex, s);
                if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGraphLaunch (batch)");
            } else {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                if (st != ETRAJ_OK) return st;
                ETRAJ_TRY(enqueue(&launches));
            }
        } else {
            cudaGetLastError();
            ETRAJ_TRY(enqueue(&launches));
        }
    } else {
        ETRAJ_TRY(enqueue(&launches));
    }
    ctx->stage_valid = true;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(ctx, e, "batch launch");
    std::vector<double> isums((size_t)2 * n);
    std::vector<Counters> icnt((size_t)n);
    unsigned long long sort_err = 0ull;
    cudaMemcpyAsync(&sort_err, &P.counters->sort_err, sizeof sort_err, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(isums.data(), d_isums, isums.size() * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(icnt.data(), d_icnt, icnt.size() * sizeof(Counters), cudaMemcpyDeviceToHost, s);
    const bool coherent = (H[0].J.phase != ETRAJ_PHASE_CTMC);
    for (int i = 0; i < n; ++i) {
        const int64_t o = (int64_t)i * grid1;
        if (res[i].momentum_spec)
            cudaMemcpyAsync(res[i].momentum_spec, P.mspec + o, (size_t)grid1 * 8, cudaMemcpyDeviceToHost, s);
        if (res[i].amplitude && coherent) {
            cudaMemcpy2DAsync(res[i].amplitude, 16, P.spec_re + o, 8, 8, (size_t)grid1, cudaMemcpyDeviceToHost, s);
            cudaMemcpy2DAsync(res[i].amplitude + 1, 16, P.spec_im + o, 8, 8, (size_t)grid1, cudaMemcpyDeviceToHost, s);
        }
    }
    if (weights) cudaMemcpyAsync(wspec, d_wout, (size_t)grid1 * 8, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(ctx, e, "etraj_run_batch");
    if (sort_err) return set_err(ctx, ETRAJ_ERR_CUDA, "deposit: a look-back wait of the radix sort gave up");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    for (int i = 0; i < n; ++i) {
        etraj_result& r = res[i];
        r.ion_prob = isums[(size_t)2 * i];
        r.ion_prob_uncollected = isums[(size_t)2 * i + 1];
        r.num_effective_traj = (int64_t)icnt[(size_t)i].n_eff;
        r.num_failed_traj = (int64_t)icnt[(size_t)i].n_failed;
        r.num_ionized_traj = (int64_t)icnt[(size_t)i].n_ionized;
        r.num_steps = (int64_t)icnt[(size_t)i].n_steps;
        r.num_kernel_launches = launches;
        r.elapsed_ms = ms;
    }
    return ETRAJ_OK;
}

// Copies sampled candidates back and assembles the reference's `init` columns.
int gather_rows(etraj_ctx* ctx, const HostJob& H, const Pipeline& P, int64_t g0, int64_t ng, double* init,
                int64_t capacity, int64_t* count) {
    const DJob& J = H.J;
    cudaStream_t s = ctx->stream;
    std::vector<uint8_t> flag((size_t)ng);
    std::vector<double> x((size_t)ng), y((size_t)ng), kx((size_t)ng), ky((size_t)ng), kz((size_t)ng),
        rate((size_t)ng), ph((size_t)ng);
    std::vector<int32_t> batch((size_t)ng);
    cudaMemcpyAsync(flag.data(), P.flag + g0, (size_t)ng, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(x.data(), P.soa.x + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(y.data(), P.soa.y + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(kx.data(), P.soa.kx + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ky.data(), P.soa.ky + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(kz.data(), P.soa.kz + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(rate.data(), P.soa.rate + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    if (P.soa.phase) cudaMemcpyAsync(ph.data(), P.soa.phase + g0, (size_t)ng * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(batch.data(), P.soa.batch + g0, (size_t)ng * 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(ctx, e, "sample copy-back");
    int64_t c = 0;
    for (int64_t i = 0; i < ng; ++i) {
        if (!flag[(size_t)i]) continue;
        if (c < capacity) {
            double* r = init + c * J.rows;
            int k = 0;
            r[k++] = x[(size_t)i];
            r[k++] = y[(size_t)i];
            if (J.dim == 3) r[k++] = 0.0;
            r[k++] = kx[(size_t)i];
            r[k++] = ky[(size_t)i];
            if (J.dim == 3) r[k++] = kz[(size_t)i];
            r[k++] = H.t[(size_t)batch[(size_t)i]];
            r[k++] = rate[(size_t)i];
            if (J.phase != ETRAJ_PHASE_CTMC) r[k++] = ph[(size_t)i];
        }
        ++c;
    }
    *count = c;
    return ETRAJ_OK;
}

int sample_range(etraj_ctx* ctx, const etraj_job* job, int64_t b0, int64_t nb, double* init, int64_t capacity,
                 int64_t* count) {
    std::string err;
    int st = validate_job(job, err);
    if (st != ETRAJ_OK) return set_err(ctx, st, err);
    HostJob H;
    prepare_job(job, H);
    Pipeline P;
    ETRAJ_TRY(alloc_sampling(ctx, H, P));
    cudaStream_t s = ctx->stream;
    upload_inputs(H, P, s);
    launch_batch_prepare(H.J, P.t, P.batches, s);
    const SampleScratch scr = sample_scratch(P, H.J.n_total, job->precision);
    launch_sampler(job->precision, H.J, b0, nb, P.kd, P.kz, P.batches, P.soa, P.flag, ctx->sm_count, s, &scr);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(ctx, e, "sample launch");
    return gather_rows(ctx, H, P, b0 * H.J.n_cand, nb * H.J.n_cand, init, capacity, count);
}

