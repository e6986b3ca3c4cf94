// tune.cu -- the bulk integrator's launch shapes and rounds: the autotuner, the
// park buffers of its step-budgeted rounds, and its launch.
#include "host.h"

// ---- autotuner of the bulk integrator's launch shape ----------------------------------
// Candidates: threads per block x blocks per SM x the register budget of the
// build (<= 128 registers: 16 warps per SM; <= 85: 24 warps) x the number of
// free lanes a warp waits for before it refills.  Each variant (dimension,
// phase, target, single/multi-instance) is tuned once per device and process,
// on the first 2^18 electrons of its first job with enough work, each electron
// capped at kTuneMaxIters steps (a job's slowest trajectory would otherwise set
// the time of every candidate), by timing every candidate twice with events.
// The choice is kept process-wide, so the contexts of a server tune a variant
// once between them.  Results do not depend on the launch shape (one electron
// per lane, deterministic deposit).
constexpr int kTuneMaxIters = 4096;

std::mutex g_tile_mu;                             // guards g_tiles; held across a tuning run
std::map<std::pair<int, int>, BulkTile> g_tiles;  // (device, variant) -> launch shape

// The context's launch shape for a variant: its own choice, else the process-wide one.
bool find_tile(etraj_ctx* ctx, int key, BulkTile* t) {
    auto it = ctx->tiles.find(key);
    if (it == ctx->tiles.end()) {
        if (!ctx->autotune) return false;
        std::lock_guard<std::mutex> lk(g_tile_mu);
        auto g = g_tiles.find({ctx->device, key});
        if (g == g_tiles.end()) return false;
        it = ctx->tiles.emplace(key, g->second).first;
    }
    if (t) *t = it->second;
    return true;
}

constexpr BulkTile kTileCandidates[] = {{256, 2, 4, 2, 1024}, {256, 2, 8, 2, 1024}, {256, 2, 2, 2, 1024},
                                        {256, 2, 16, 2, 1024}, {128, 4, 4, 2, 1024}, {128, 4, 8, 2, 1024},
                                        {128, 3, 4, 2, 1024}, {64, 8, 4, 2, 1024},   {256, 3, 4, 3, 1024},
                                        {256, 3, 8, 3, 1024}, {128, 6, 4, 3, 1024}, {128, 6, 8, 3, 1024}};
// step chunks the tuner tries once the shape is chosen (with rounds on)
constexpr int kChunkCandidates[] = {256, 4096};

// Stage events: inside a stream capture they become event-record nodes of the graph.
void rec(etraj_ctx* ctx, cudaEvent_t e, cudaStream_t s) {
    if (ctx->capturing) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else cudaEventRecord(e, s);
}

int tile_key(const BulkParams& B) { return ((B.n_inst > 0) ? 1000 : 0) + B.dim * 100 + B.phase * 10 + B.tgt; }

void apply_tile(BulkParams& B, const BulkTile& t) {
    B.threads = t.threads;
    B.blocks_per_sm = t.blocks_per_sm;
    B.refill_min = t.refill_min;
    B.occ = t.occ;
    B.chunk0 = t.chunk > 0 ? t.chunk : 1024;
    const size_t tb = (size_t)B.n_int * 2 * sizeof(float4);
    B.table_in_smem = (B.n_inst == 0 && tb <= (size_t)96 * 1024 && tb * (size_t)t.blocks_per_sm <= (size_t)200 * 1024)
                          ? 1 : 0;
}

int tuned_bulk_launch(etraj_ctx* ctx, BulkParams& B, const InitSoA& soa, const double* t, const int64_t* idx,
                      const unsigned long long* count, unsigned long long* work, const TrajOut& out,
                      int* launches, cudaEvent_t* ev) {
    cudaStream_t s = ctx->stream;
    const int key = tile_key(B);
    BulkTile chosen = kTileDefault;
    bool have = find_tile(ctx, key, &chosen);
    if (B.static_assign) {
        // the plain schedule: the tuned (or default) block shape, no tuning run
        apply_tile(B, chosen);
        if (ev) rec(ctx, ev[0], s);
        *launches += launch_integrate_bulk(B, soa, t, idx, count, work, out, ctx->sm_count, s);
        if (ev) rec(ctx, ev[1], s);
        return ETRAJ_OK;
    }
    std::unique_lock<std::mutex> tune_lk(g_tile_mu, std::defer_lock);
    if (!have && ctx->autotune && B.max_n >= ((int64_t)1 << 18)) {
        tune_lk.lock();  // one tuning run at a time; another context may have finished it meanwhile
        auto g = g_tiles.find({ctx->device, key});
        if (g != g_tiles.end()) {
            chosen = g->second;
            have = true;
            ctx->tiles[key] = chosen;
        }
    }
    if (!have && ctx->autotune && B.max_n >= ((int64_t)1 << 18)) {
        unsigned long long* sub = nullptr;
        ETRAJ_TRY(ensure_t(ctx, "tune.count", 1, &sub));
        *launches += launch_clamp_count(count, 1ull << 18, sub, s);
        const int nc = (int)(sizeof kTileCandidates / sizeof kTileCandidates[0]);
        std::vector<cudaEvent_t> evs((size_t)4 * nc);
        for (auto& e : evs) e = get_event(ctx);
        for (int rep = 0; rep < 2; ++rep) {
            for (int c = 0; c < nc; ++c) {
                BulkParams Bc = B;
                Bc.max_iters = kTuneMaxIters;
                apply_tile(Bc, kTileCandidates[c]);
                cudaEventRecord(evs[(size_t)(4 * c + 2 * rep)], s);
                *launches += launch_integrate_bulk(Bc, soa, t, idx, sub, work, out, ctx->sm_count, s);
                cudaEventRecord(evs[(size_t)(4 * c + 2 * rep + 1)], s);
            }
        }
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_err(ctx, e, "autotune");
        float best = 1e30f;
        BulkTile bt = kTileDefault;
        for (int c = 0; c < nc; ++c) {
            float m0 = 0.f, m1 = 0.f;
            cudaEventElapsedTime(&m0, evs[(size_t)(4 * c)], evs[(size_t)(4 * c + 1)]);
            cudaEventElapsedTime(&m1, evs[(size_t)(4 * c + 2)], evs[(size_t)(4 * c + 3)]);
            const float m = m0 < m1 ? m0 : m1;
            if (m < best) {
                best = m;
                bt = kTileCandidates[c];
            }
        }
        // second stage: the step chunk of the rounds, with the chosen shape
        if (B.park_buf) {
            const int nk = (int)(sizeof kChunkCandidates / sizeof kChunkCandidates[0]);
            for (int rep = 0; rep < 2; ++rep)
                for (int c = 0; c < nk; ++c) {
                    BulkParams Bc = B;
                    Bc.max_iters = kTuneMaxIters;
                    BulkTile tc = bt;
                    tc.chunk = kChunkCandidates[c];
                    apply_tile(Bc, tc);
                    cudaEventRecord(evs[(size_t)(4 * c + 2 * rep)], s);
                    *launches += launch_integrate_bulk(Bc, soa, t, idx, sub, work, out, ctx->sm_count, s);
                    cudaEventRecord(evs[(size_t)(4 * c + 2 * rep + 1)], s);
                }
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return cuda_err(ctx, e, "autotune");
            const BulkTile shape = bt;
            for (int c = 0; c < nk; ++c) {
                float m0 = 0.f, m1 = 0.f;
                cudaEventElapsedTime(&m0, evs[(size_t)(4 * c)], evs[(size_t)(4 * c + 1)]);
                cudaEventElapsedTime(&m1, evs[(size_t)(4 * c + 2)], evs[(size_t)(4 * c + 3)]);
                const float m = m0 < m1 ? m0 : m1;
                if (m < best) {
                    best = m;
                    bt = shape;
                    bt.chunk = kChunkCandidates[c];
                }
            }
        }
        for (auto& ev_ : evs) ctx->event_pool.push_back(ev_);
        ctx->tiles[key] = bt;
        g_tiles[{ctx->device, key}] = bt;
        chosen = bt;
    }
    if (tune_lk.owns_lock()) tune_lk.unlock();
    apply_tile(B, chosen);
    if (ev) rec(ctx, ev[0], s);
    *launches += launch_integrate_bulk(B, soa, t, idx, count, work, out, ctx->sm_count, s);
    if (ev) rec(ctx, ev[1], s);
    return ETRAJ_OK;
}

// The park buffer of the bulk integrator's rounds: two halves of max_n/16 +
// 4096 entries (at most 2^20) of kParkWords words.  An electron that finds
// the buffer full finishes in its current round, so the size only bounds how
// much the later rounds can repack.
int attach_park(etraj_ctx* ctx, BulkParams& B) {
    B.park_buf = nullptr;
    B.park_cap = 0;
    if (!ctx->repack) return ETRAJ_OK;
    const int cap = (int)std::min<int64_t>(B.max_n / 16 + 4096, (int64_t)1 << 20);
    uint32_t* buf = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "park", (size_t)2 * (size_t)cap * kParkWords, &buf));
    B.park_buf = buf;
    B.park_cap = cap;
    return ETRAJ_OK;
}

int launch_integrate(etraj_ctx* ctx, const DJob& J, const InitSoA& soa, const double* t, const int64_t* idx,
                     const unsigned long long* count, const TrajOut& out, int64_t max_n, unsigned long long* work,
                     int precision, double tmin, int* launches, cudaEvent_t* ev) {
    // ev (optional): events recorded after the field table [0] and the integrator [1]
    cudaStream_t s = ctx->stream;
    if (precision == ETRAJ_PRECISION_FP32_DF) {
        DFParams D;
        prepare_df(J, tmin, max_n, ctx->sm_count, D);
        ETRAJ_TRY(attach_df(ctx, D));
        DfTableNodes nodes;
        df_table_nodes(nodes);
        *launches += launch_field_table_df(J, D.T0, D.h_d, D.n_int, nodes, (float4*)D.table, s);
        if (ev) rec(ctx, ev[0], s);
        *launches += launch_integrate_df(D, soa, t, idx, count, work, out, s);
        if (ev) rec(ctx, ev[1], s);
        *launches += launch_collect_fp64(J, soa, t, idx, count, out, max_n, ctx->sm_count, s);
        return ETRAJ_OK;
    }
    if (precision != ETRAJ_PRECISION_FP32_BULK) {
        if (ev) rec(ctx, ev[0], s);
        *launches += launch_integrate_fp64(J, soa, t, idx, count, out, max_n, ctx->sm_count, s);
        if (ev) rec(ctx, ev[1], s);
        return ETRAJ_OK;
    }
    BulkParams B;
    prepare_bulk(J, tmin, B);
    B.max_n = max_n;
    float4* tab = nullptr;
    ETRAJ_TRY(ensure_t(ctx, "field_table", (size_t)B.n_int * 2, &tab));
    B.table = tab;
    B.static_assign = ctx->static_assign ? 1 : 0;
    if (!B.static_assign) ETRAJ_TRY(attach_park(ctx, B));
    *launches += launch_field_table(J, B.T0, (double)1.0 / B.inv_h_d, B.n_int, tab, s);
    ETRAJ_TRY(tuned_bulk_launch(ctx, B, soa, t, idx, count, work, out, launches, ev));
    *launches += launch_collect_bulk(J, soa, t, idx, count, out, max_n, ctx->sm_count, s);
    return ETRAJ_OK;
}

