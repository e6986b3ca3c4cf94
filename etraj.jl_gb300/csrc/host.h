// host.h -- the host side of the library, shared by its translation units:
//   job.cu       checks of a job and its host-side set-up (time and momentum
//                samples, the sampler's per-job constants);
//   pipeline.cu  a job's device buffers (grow-only, against the HBM budget), its
//                kernel sequence (direct or a replayed CUDA graph), result staging;
//   tune.cu      the bulk integrator's launch shapes (the autotuner) and rounds;
//   batch.cu     multi-instance batches, and sampling without integration;
//   server.cu    the continuously batching server;
//   api.cu       the C entry points of include/etraj.h.
// It holds the context, a job's host data and device buffers, and the functions
// one unit calls in another.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <chrono>
#include <deque>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "engine.h"
#include "integrate_setup.h"
#include "mol_check.h"

using namespace etraj;

#define ETRAJ_VERSION_STRING "etraj-gb300 1.0 (sm_103a)"

struct HostJob {
    DJob J;
    std::vector<double> t, kd, kz;
    std::vector<double> mol_clm, mol_wint;  // molecular target: copies of the caller's tables
};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// One enqueued job.  Its results land either straight in the caller's
// buffers (synchronous etraj_run) or in a pinned staging block that is copied
// out when the job completes (asynchronous submit and the server).
struct JobRec {
    uint64_t ticket = 0;         // 0: etraj_run's job
    int status = ETRAJ_OK;       // enqueue status; an error completes the job at once
    std::string error;
    etraj_result res{};          // the caller's output pointers; scalars filled at completion
    int64_t grid = 0;
    bool coherent = false;
    int launches = 0;
    bool staged = false;
    void* pinned = nullptr;      // staged: sums[2] | Counters | mspec[grid] | amplitude[2 grid]
    size_t pinned_bytes = 0;
    cudaEvent_t ev_start = nullptr, ev_done = nullptr;
    double direct_sums[2] = {0.0, 0.0};
    Counters direct_cnt{};
};

struct PinnedBlock {
    void* p = nullptr;
    size_t bytes = 0;
};

// Launch shape of the bulk integrator.
struct BulkTile {
    int threads, blocks_per_sm, refill_min, occ;
    int chunk;  // step chunk: round 0's step budget per electron (round r: chunk 16^r)
};


constexpr BulkTile kTileDefault = {256, 2, 4, 2, 1024};

struct etraj_ctx {
    int device = 0;
    int sm_count = 152;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    size_t budget = 0;
    size_t used = 0;
    std::string err;
    std::map<std::string, DevBuf> bufs;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // stage boundaries of the last etraj_run: sample | compact | field table |
    // integrate | collect | deposit
    static constexpr int kStages = 6;
    cudaEvent_t stage_ev[kStages + 1] = {};
    bool stage_valid = false;
    uint64_t next_ticket = 1;
    std::map<uint64_t, JobRec> jobs;       // asynchronous tickets of this context
    // per-survivor final states of the last job, kept with etraj_set_keep_final_states
    bool keep_states = false;
    bool dump_valid = false;
    uint64_t dump_ticket = 0;
    TrajOut dump_out{};
    const unsigned long long* dump_count = nullptr;
    std::vector<PinnedBlock> pinned_pool;  // staging blocks for reuse
    std::vector<cudaEvent_t> event_pool;
    // CUDA-graph replay of the per-job kernel sequence (opt-in): the graph of
    // the last captured job and the launch parameters it was captured with
    bool graphs = true;   // CUDA-graph replay of kernel sequences that repeat
    bool capturing = false;
    cudaGraphExec_t gexec = nullptr;
    std::vector<unsigned char> gkey;
    int glaunches = 0;
    cudaGraphExec_t bgexec = nullptr;  // the last multi-instance batch's graph
    std::vector<unsigned char> bgkey;
    int bglaunches = 0;
    std::vector<unsigned char> gseen, bgseen;  // the last keys run without a graph
    // bulk-integrator launch shapes chosen by the autotuner, per kernel variant
    bool autotune = true;
    bool repack = true;  // the bulk integrator's rounds with parking of long-running electrons
    bool static_assign = false;  // the bulk integrator with one electron per lane, no work stealing
    std::map<int, BulkTile> tiles;
    // sizing without allocating: ensure() only adds up the growth
    bool dry = false;
    size_t dry_bytes = 0;
    std::mutex mu;
};

int set_err(etraj_ctx* ctx, int code, const std::string& msg);
int cuda_err(etraj_ctx* ctx, cudaError_t e, const char* where);
// Grow-only named device buffer, counted against the context's HBM budget.
int ensure(etraj_ctx* ctx, const char* name, size_t bytes, void** out);

template <typename T>
int ensure_t(etraj_ctx* ctx, const char* name, size_t count, T** out) {
    void* p = nullptr;
    int st = ensure(ctx, name, count * sizeof(T), &p);
    *out = (T*)p;
    return st;
}

struct Pipeline {
    double* t = nullptr;
    double* kd = nullptr;
    double* kz = nullptr;
    DBatch* batches = nullptr;
    InitSoA soa{};
    uint8_t* flag = nullptr;
    int64_t* idx = nullptr;
    uint32_t* block_sums = nullptr;
    unsigned long long* count = nullptr;
    TrajOut out{};
    DepositScratch dep{};
    double* spec_re = nullptr;
    double* spec_im = nullptr;
    double* mspec = nullptr;
    double* sums = nullptr;
    Counters* counters = nullptr;
    unsigned long long* work = nullptr;
};

#define ETRAJ_TRY(x)                 \
    do {                             \
        int _st = (x);               \
        if (_st != ETRAJ_OK) return _st; \
    } while (0)

// job.cu
int validate_job(const etraj_job* job, std::string& err);
void prepare_job(const etraj_job* job, HostJob& H);

// pipeline.cu
int alloc_sampling(etraj_ctx* ctx, HostJob& H, Pipeline& P);
int alloc_outputs(etraj_ctx* ctx, const DJob& J, int64_t max_n, bool with_state, Pipeline& P);
int launch_sampler(int precision, const DJob& J, int64_t b0, int64_t nb, const double* kd, const double* kz,
                   DBatch* batches, InitSoA soa, uint8_t* flag, int sm_count, cudaStream_t s,
                   const SampleScratch* scr);
SampleScratch sample_scratch(const Pipeline& P, int64_t n, int precision);
void upload_inputs(const HostJob& H, const Pipeline& P, cudaStream_t s);
float sae_far_radius(const DTarget& T);
void prepare_bulk(const DJob& J, double tmin, BulkParams& B);
void prepare_df(const DJob& J, double tmin, int64_t max_n, int sm_count, DFParams& D);
int attach_df(etraj_ctx* ctx, DFParams& D);
int get_pinned(etraj_ctx* ctx, size_t bytes, PinnedBlock* out);
void put_pinned(etraj_ctx* ctx, void* p, size_t bytes);
cudaEvent_t get_event(etraj_ctx* ctx);
void release_job(etraj_ctx* ctx, JobRec& r);
size_t plan_growth(etraj_ctx* ctx, const etraj_job* job);
int enqueue_kernels(etraj_ctx* ctx, const etraj_job* job, const HostJob& H, const Pipeline& P, int* nl);
int enqueue_kernels_maybe_graph(etraj_ctx* ctx, const etraj_job* job, const HostJob& H, const Pipeline& P,
                                int* launches);
int enqueue_job(etraj_ctx* ctx, const etraj_job* job, JobRec& r);
int finish_job(etraj_ctx* ctx, JobRec& r);
int run_job(etraj_ctx* ctx, const etraj_job* job, etraj_result* res);

// tune.cu
bool find_tile(etraj_ctx* ctx, int key, BulkTile* t);
void rec(etraj_ctx* ctx, cudaEvent_t e, cudaStream_t s);
int tile_key(const BulkParams& B);
void apply_tile(BulkParams& B, const BulkTile& t);
int tuned_bulk_launch(etraj_ctx* ctx, BulkParams& B, const InitSoA& soa, const double* t, const int64_t* idx,
                      const unsigned long long* count, unsigned long long* work, const TrajOut& out, int* launches,
                      cudaEvent_t* ev);
int attach_park(etraj_ctx* ctx, BulkParams& B);
int launch_integrate(etraj_ctx* ctx, const DJob& J, const InitSoA& soa, const double* t, const int64_t* idx,
                     const unsigned long long* count, const TrajOut& out, int64_t max_n, unsigned long long* work,
                     int precision, double tmin, int* launches, cudaEvent_t* ev = nullptr);

// batch.cu
int run_batch(etraj_ctx* ctx, const etraj_job* jobs, int n, etraj_result* res, const double* weights,
              double* wspec);
int gather_rows(etraj_ctx* ctx, const HostJob& H, const Pipeline& P, int64_t g0, int64_t ng, double* init,
                int64_t capacity, int64_t* count);
int sample_range(etraj_ctx* ctx, const etraj_job* job, int64_t b0, int64_t nb, double* init, int64_t capacity,
                 int64_t* count);
