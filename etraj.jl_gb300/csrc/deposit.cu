// deposit.cu -- deterministic momentum-spectrum deposit and reductions.
//
// Reference: the deposit `spec_collect_current[pxIdx,pyIdx] += prob` (CTMC)
// or `+= sqrt(prob)*exp(1im*phase)` (QTMC/SCTS), TrajectorySimulation.jl:
// 384-392 (3D :484-492), the thread sum and abs2 of write_output! (:521-533)
// and the probability sums (:541-542).
//
// The reference's sum order depends on Julia's thread schedule.  Here the
// order is fixed and independent of the launch shape: each bin is summed
// left to right from 0.0 in trajectory order, which a stable LSD radix sort
// of (bin, trajectory) followed by one sequential pass per bin segment
// produces.  No floating-point atomics are used.  ion_prob and
// ion_prob_uncollected are 256-ary trees over trajectory order, each node
// summed left to right from 0.0.
//
// Roofline: HBM bound.  Per trajectory: read 4 B key once for the digit counts
// of every pass, then per pass read 8 B + write 8 B (one onesweep kernel); the
// per-bin pass reads 8 B of the sorted pair plus 16 B of contribution and 8 +
// 16 B per bin; passes = ceil(bits(grid+1)/9), each on at most 9 key bits.

#include "engine.h"

namespace etraj {
namespace {

constexpr int kThreads = 256;
constexpr int kRounds = 16;
constexpr int kTile = kThreads * kRounds;  // keys per block and pass
constexpr int kWarps = kThreads / 32;
constexpr int kMaxDigitBits = 9;           // a pass sorts on up to 9 key bits
constexpr int kMaxDigits = 1 << kMaxDigitBits;

constexpr int kMaxPasses = 4;              // keys of up to 36 bits
constexpr int kSub = kTile / kWarps;       // keys per warp and tile

// Width and first bit of pass p of a sort over `bits` key bits in `npass` passes.
__host__ __device__ inline void pass_digits(int bits, int npass, int p, int* w, int* shift) {
    int sh = 0;
    for (int q = 0; q < p; ++q) sh += bits / npass + ((q < bits % npass) ? 1 : 0);
    *w = bits / npass + ((p < bits % npass) ? 1 : 0);
    *shift = sh;
}

// ---- onesweep LSD radix sort (Adinets & Merrill 2022) -------------------------------
// One read of the keys counts the digits of every pass (k_onesweep_hist), one
// block turns each pass's counts into digit offsets (k_onesweep_scan), and each
// pass is one kernel that sorts tile after tile: a tile counts its digits, posts
// them, takes the sum of the earlier tiles' counts per digit by decoupled
// look-back, and scatters its keys stably.  Launches per sort: 2 + passes.

// Digit counts of every pass: ghist[p kMaxDigits + d].
__global__ void __launch_bounds__(kThreads)
k_onesweep_hist(const uint32_t* __restrict__ keys, const unsigned long long* __restrict__ count, int bits,
                int npass, uint32_t* __restrict__ ghist) {
    __shared__ uint32_t h[kMaxPasses][kMaxDigits];
    const int64_t n = (int64_t)*count;
    for (int i = threadIdx.x; i < kMaxPasses * kMaxDigits; i += kThreads) (&h[0][0])[i] = 0u;
    __syncthreads();
    int w[kMaxPasses], sh[kMaxPasses];
#pragma unroll
    for (int p = 0; p < kMaxPasses; ++p) {
        w[p] = 0;
        sh[p] = 0;
        if (p < npass) pass_digits(bits, npass, p, &w[p], &sh[p]);
    }
    for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        const uint32_t k = keys[i];
#pragma unroll
        for (int p = 0; p < kMaxPasses; ++p)
            if (p < npass) atomicAdd(&h[p][(k >> sh[p]) & ((1u << w[p]) - 1u)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npass * kMaxDigits; i += kThreads) {
        const uint32_t v = (&h[0][0])[i];
        if (v) atomicAdd(&ghist[i], v);
    }
}

// Exclusive prefix of each pass's digit counts (one block of kMaxDigits threads).
__global__ void __launch_bounds__(kMaxDigits)
k_onesweep_scan(const uint32_t* __restrict__ ghist, int npass, uint32_t* __restrict__ base) {
    __shared__ uint32_t ws[kMaxDigits / 32];
    const int d = threadIdx.x, lane = d & 31, warp = d >> 5;
    for (int p = 0; p < npass; ++p) {
        const uint32_t v = ghist[p * kMaxDigits + d];
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        uint32_t off = 0u;
        for (int q = 0; q < warp; ++q) off += ws[q];
        base[p * kMaxDigits + d] = off + x - v;
        __syncthreads();
    }
}

// Posts of the look-back: a 64-bit word per (tile, digit), the count in the low 32
// bits and above them 2p+1 ("this tile's count") or 2p+2 ("the count of this and
// every earlier tile") for pass p, so one region, cleared once per sort, serves
// every pass.  A block takes its tile from a counter, so every tile it waits for
// was taken earlier by a block that is running, and that block posts its own
// count before it waits on anything: the look-back needs no co-resident grid (a
// plain launch, which other streams' kernels can share the GPU with).  A wait
// gives up after kLookbackSpins polls (so it never should) and raises *err.
constexpr int kLookbackSpins = 1 << 22;
constexpr int kWindow = 16;  // posts a look-back step loads at once

__device__ __forceinline__ unsigned long long load_post(const unsigned long long* p) {
    return *(const volatile unsigned long long*)p;
}

// The lanes of the warp whose digit equals this lane's: one ballot per digit bit
// (bits + 1 of them: an absent key carries the digit 2^bits).
__device__ __forceinline__ unsigned digit_peers(uint32_t d, int bits) {
    unsigned peers = 0xffffffffu;
    for (int bit = 0; bit <= bits; ++bit) {
        const bool on = (d >> bit) & 1u;
        const unsigned b = __ballot_sync(0xffffffffu, on);
        peers &= on ? b : ~b;
    }
    return peers;
}

__global__ void __launch_bounds__(kThreads, 3)
k_onesweep_pass(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
                uint32_t* __restrict__ vout, const unsigned long long* __restrict__ count, int pass, int shift,
                int bits, const uint32_t* __restrict__ base, unsigned long long* __restrict__ post,
                unsigned int* __restrict__ tile_ctr, unsigned long long* __restrict__ err) {
    __shared__ uint32_t wc[kWarps][kMaxDigits];
    __shared__ uint32_t toff[kMaxDigits];
    __shared__ uint32_t s_tile;
    const int64_t n = (int64_t)*count;
    const int64_t ntiles = (n + kTile - 1) / kTile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const uint32_t nd = 1u << bits, mask = nd - 1u;
    const unsigned long long f_own = (unsigned long long)(2 * pass + 1) << 32;
    const unsigned long long f_inc = (unsigned long long)(2 * pass + 2) << 32;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(tile_ctr, 1u);
        for (uint32_t d = threadIdx.x; d < nd; d += kThreads)
            for (int w = 0; w < kWarps; ++w) wc[w][d] = 0u;
        __syncthreads();
        const int64_t tile = (int64_t)s_tile;
        if (tile >= ntiles) break;
        // the warp's part of the tile in registers, every load in flight at once
        // (key r of the lane is element sub + 32 r + lane)
        const int64_t sub = tile * kTile + (int64_t)warp * kSub;
        uint32_t kr[kSub / 32], vr[kSub / 32];
#pragma unroll
        for (int r = 0; r < kSub / 32; ++r) {
            const int64_t i = sub + r * 32 + lane;
            kr[r] = (i < n) ? kin[i] : 0u;
            vr[r] = (i < n) ? (vin ? vin[i] : (uint32_t)i) : 0u;
        }
        // digit counts of each warp's part of the tile
#pragma unroll
        for (int r = 0; r < kSub / 32; ++r) {
            const int64_t i = sub + r * 32 + lane;
            const uint32_t d = (i < n) ? (kr[r] >> shift) & mask : nd;
            const unsigned peers = digit_peers(d, bits);
            if (d < nd && lane == __ffs(peers) - 1) wc[warp][d] += __popc(peers);
        }
        __syncthreads();
        // post the tile's counts, sum the earlier tiles', post the running total
        for (uint32_t d = threadIdx.x; d < nd; d += kThreads) {
            uint32_t run = 0u;
            for (int w = 0; w < kWarps; ++w) {
                const uint32_t c = wc[w][d];
                wc[w][d] = run;
                run += c;
            }
            unsigned long long* mine = post + tile * kMaxDigits + d;
            atomicExch(mine, (tile == 0 ? f_inc : f_own) | run);
            uint32_t excl = 0u;
            if (tile > 0) {
                // walk back kWindow posts per round trip: all loads in flight at once,
                // then the window's counts in order up to the first running total
                int64_t t = tile - 1;
                int spins = 0;
                bool done = false;
                while (!done) {
                    unsigned long long v[kWindow];
#pragma unroll
                    for (int j = 0; j < kWindow; ++j)
                        v[j] = (t - j >= 0) ? load_post(post + (t - j) * kMaxDigits + d) : f_inc;
                    int used = 0;
#pragma unroll
                    for (int j = 0; j < kWindow; ++j) {
                        if (done || used < j) continue;  // stopped earlier in the window
                        const unsigned long long f = v[j] & 0xFFFFFFFF00000000ull;
                        if (f == f_inc) {
                            excl += (uint32_t)v[j];
                            done = true;
                        } else if (f == f_own) {
                            excl += (uint32_t)v[j];
                            used = j + 1;
                        }
                    }
                    if (!done) {
                        t -= used;
                        if (used < kWindow) {  // a post not there yet: wait a little
                            if (++spins > kLookbackSpins) {
                                atomicExch(err, 1ull);
                                break;
                            }
                            __nanosleep(32);
                        }
                    }
                }
                atomicExch(mine, f_inc | (unsigned long long)(excl + run));
            }
            toff[d] = base[d] + excl;
        }
        __syncthreads();
        // stable scatter: each warp writes its keys in index order
#pragma unroll
        for (int r = 0; r < kSub / 32; ++r) {
            const int64_t i = sub + r * 32 + lane;
            const bool valid = i < n;
            const uint32_t key = kr[r], val = vr[r];
            const uint32_t d = valid ? (key >> shift) & mask : nd;
            const unsigned peers = digit_peers(d, bits);
            const uint32_t pos = valid ? toff[d] + wc[warp][d] + __popc(peers & lt_mask) : 0u;
            __syncwarp();
            if (valid && lane == __ffs(peers) - 1) wc[warp][d] += __popc(peers);
            __syncwarp();
            if (valid && (int64_t)pos < n) {  // (pos >= n only after a look-back gave up)
                kout[pos] = key;
                vout[pos] = val;
            }
        }
        __syncthreads();
    }
}

// Per-bin sums over the sorted pairs, each bin left to right from 0.0, in two
// passes.  k_segment_bounds marks where each bin's segment of the sorted keys
// starts and ends; k_bin_sum then gives one thread to each bin.  Neighbouring
// bins of a spectrum hold similar numbers of trajectories, so the lanes of a
// warp add for about the same number of iterations.  (A thread per segment
// start instead leaves most lanes of a warp idle while one walks a long
// segment, and every FP64 add is issued for the whole warp on GB300's narrow
// FP64 pipe.)  The bounds (first, end) of bin k are two uint32 stored in the
// 8-byte slot spec_re[k], zeroed beforehand, so an empty bin reads (0, 0) and
// sums to +0.0, and k_bin_sum reads the slot before it writes the sum there,
// and the bin of the momentum spectrum (re, or re^2 + im^2 when coherent).
__global__ void __launch_bounds__(256)
k_segment_bounds(const uint32_t* __restrict__ keys, const unsigned long long* __restrict__ count,
                 uint32_t grid, uint32_t* __restrict__ bounds) {
    const int64_t n = (int64_t)*count;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t k = keys[p];
        if (k >= grid) continue;
        if (p == 0 || keys[p - 1] != k) bounds[2 * (int64_t)k] = (uint32_t)p;
        if (p == n - 1 || keys[p + 1] != k) bounds[2 * (int64_t)k + 1] = (uint32_t)(p + 1);
    }
}

__global__ void __launch_bounds__(256)
k_bin_sum(const uint32_t* __restrict__ vals, int64_t grid, const double* __restrict__ c_re,
          const double* __restrict__ c_im, int coherent, double* __restrict__ spec_re,
          double* __restrict__ spec_im, double* __restrict__ mspec) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < grid;
         g += (int64_t)gridDim.x * blockDim.x) {
        const uint2 b = reinterpret_cast<const uint2*>(spec_re)[g];
        double sr = 0.0, si = 0.0;
#pragma unroll 4
        for (uint32_t q = b.x; q < b.y; ++q) {
            const uint32_t v = vals[q];
            sr = sr + c_re[v];
            if (coherent) si = si + c_im[v];
        }
        spec_re[g] = sr;
        if (coherent) spec_im[g] = si;
        mspec[g] = coherent ? sr * sr + si * si : sr;
    }
}

int launch_bin_sums(const uint32_t* keys, const uint32_t* vals, const unsigned long long* count, int64_t max_n,
                    int64_t grid, const double* c_re, const double* c_im, int coherent, double* spec_re,
                    double* spec_im, double* mspec, cudaStream_t s) {
    int64_t pb = (max_n + 255) / 256;
    if (pb > 152 * 32) pb = 152 * 32;
    int64_t gb = (grid + 255) / 256;
    if (gb > 152 * 32) gb = 152 * 32;
    k_segment_bounds<<<(int)(pb > 0 ? pb : 1), 256, 0, s>>>(keys, count, (uint32_t)grid, (uint32_t*)spec_re);
    k_bin_sum<<<(int)(gb > 0 ? gb : 1), 256, 0, s>>>(vals, grid, c_re, c_im, coherent, spec_re, spec_im, mspec);
    return 2;
}

__global__ void k_finalize_spec(const double* __restrict__ re, const double* __restrict__ im,
                                int64_t grid, int coherent, double* __restrict__ out) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < grid;
         g += (int64_t)gridDim.x * blockDim.x)
        out[g] = coherent ? re[g] * re[g] + im[g] * im[g] : re[g];
}

// The 256-ary canonical tree over two arrays (ion_prob, ion_prob_uncollected).
// Level 0 reads n = *count elements, level k reads ceil(n / 256^k).  Each node
// holds 256 slots (absent ones +0.0) summed as a binary tree over consecutive
// pairs: lane j of the node's warp sums slots 8j..8j+7 in three pairwise
// levels, and five shuffle levels combine lanes (2i, 2i+1), (4i, 4i+2), ...
// No chain of dependent FP64 additions is longer than 8, which matters on
// GB300, whose FP64 unit has a long latency.

// The node over 256 slots whose lane j holds slots 8j..8j+7 in va/vb: its sums
// reach lane 0.
__device__ __forceinline__ void tree_node(double (&va)[8], double (&vb)[8], int lane, double* sa_out,
                                          double* sb_out) {
#pragma unroll
    for (int w = 4; w >= 1; w >>= 1) {
#pragma unroll
        for (int j = 0; j < w; ++j) {
            va[j] = va[2 * j] + va[2 * j + 1];
            vb[j] = vb[2 * j] + vb[2 * j + 1];
        }
    }
    double sa = va[0], sb = vb[0];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double ra = __shfl_down_sync(0xffffffffu, sa, o);
        const double rb = __shfl_down_sync(0xffffffffu, sb, o);
        if ((lane & (2 * o - 1)) == 0) {
            sa = sa + ra;
            sb = sb + rb;
        }
    }
    *sa_out = sa;
    *sb_out = sb;
}

// Nodes node0, node0 + stride, ... of a level over m inputs, one per warp.
__device__ __forceinline__ void tree_nodes(const double* a_in, const double* b_in, double* a_out, double* b_out,
                                           int64_t m, int64_t node0, int64_t stride, int lane) {
    const int64_t nb = (m + 255) / 256;
    for (int64_t node = node0; node < nb; node += stride) {
        const int64_t base = node * 256 + 8 * lane;
        double va[8], vb[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const bool in = base + j < m;
            va[j] = in ? __ldcg(a_in + base + j) : 0.0;
            vb[j] = in ? __ldcg(b_in + base + j) : 0.0;
        }
        double sa, sb;
        tree_node(va, vb, lane, &sa, &sb);
        if (lane == 0) {
            a_out[node] = sa;
            b_out[node] = sb;
        }
    }
}

constexpr int kTreeWarps = 8;

// One read of the per-trajectory outputs, in trajectory order, for all the
// deposit needs from them besides the sort: the digit counts of every sort pass
// (as k_onesweep_hist), level 0 of the canonical trees (tree_nodes) and the
// counters.  A warp takes a node of 256 trajectories, lane j its slots 8j..8j+7,
// loaded as 16-byte vectors when the node is whole and the arrays are aligned.
// The block that finishes last adds the tree's upper levels and writes the sums
// (sums[0] ion_prob, sums[1] ion_prob_uncollected; 0 for no trajectory).
__global__ void __launch_bounds__(32 * kTreeWarps)
k_deposit_prepass(const uint32_t* __restrict__ keys, const int32_t* __restrict__ status,
                  const int32_t* __restrict__ steps, const double* __restrict__ w_ion,
                  const double* __restrict__ w_unc, const unsigned long long* __restrict__ count, int bits,
                  int npass, uint32_t* __restrict__ ghist, double* __restrict__ a_out, double* __restrict__ b_out,
                  double* __restrict__ sums, unsigned int* __restrict__ done, Counters* __restrict__ c) {
    __shared__ uint32_t h[kMaxPasses][kMaxDigits];
    __shared__ unsigned long long part[3][kTreeWarps];
    const int64_t n = (int64_t)*count;
    int w[kMaxPasses], sh[kMaxPasses];
#pragma unroll
    for (int p = 0; p < kMaxPasses; ++p) {
        w[p] = 0;
        sh[p] = 0;
        if (p < npass) pass_digits(bits, npass, p, &w[p], &sh[p]);
    }
    for (int i = threadIdx.x; i < kMaxPasses * kMaxDigits; i += blockDim.x) (&h[0][0])[i] = 0u;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool vec = ((((uintptr_t)keys | (uintptr_t)status | (uintptr_t)steps | (uintptr_t)w_ion |
                        (uintptr_t)w_unc) & 15u) == 0u);
    unsigned long long f = 0, io = 0, st = 0;
    const int64_t nb = (n + 255) / 256;
    for (int64_t node = (int64_t)blockIdx.x * kTreeWarps + warp; node < nb;
         node += (int64_t)gridDim.x * kTreeWarps) {
        const int64_t base = node * 256 + 8 * lane;
        double va[8], vb[8];
        uint32_t k[8];
        int32_t sv[8], tv[8];
        int valid = 8;
        if (vec && node * 256 + 256 <= n) {
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const uint4 kk = reinterpret_cast<const uint4*>(keys + base)[q];
                const int4 ss = reinterpret_cast<const int4*>(status + base)[q];
                const int4 tt = reinterpret_cast<const int4*>(steps + base)[q];
                k[4 * q] = kk.x; k[4 * q + 1] = kk.y; k[4 * q + 2] = kk.z; k[4 * q + 3] = kk.w;
                sv[4 * q] = ss.x; sv[4 * q + 1] = ss.y; sv[4 * q + 2] = ss.z; sv[4 * q + 3] = ss.w;
                tv[4 * q] = tt.x; tv[4 * q + 1] = tt.y; tv[4 * q + 2] = tt.z; tv[4 * q + 3] = tt.w;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const double2 x = reinterpret_cast<const double2*>(w_ion + base)[q];
                const double2 y = reinterpret_cast<const double2*>(w_unc + base)[q];
                va[2 * q] = x.x; va[2 * q + 1] = x.y;
                vb[2 * q] = y.x; vb[2 * q + 1] = y.y;
            }
        } else {
            valid = (int)((n - base) < 0 ? 0 : ((n - base) > 8 ? 8 : (n - base)));
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const bool in = j < valid;
                k[j] = in ? keys[base + j] : 0u;
                sv[j] = in ? status[base + j] : 0;
                tv[j] = in ? steps[base + j] : 0;
                va[j] = in ? w_ion[base + j] : 0.0;
                vb[j] = in ? w_unc[base + j] : 0.0;
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (j < valid) {
#pragma unroll
                for (int p = 0; p < kMaxPasses; ++p)
                    if (p < npass) atomicAdd(&h[p][(k[j] >> sh[p]) & ((1u << w[p]) - 1u)], 1u);
                f += ((sv[j] & 0xff) != 0) ? 1ull : 0ull;
                io += (sv[j] & 0x100) ? 1ull : 0ull;
                st += (unsigned long long)tv[j];
            }
        }
        double sa, sb;
        tree_node(va, vb, lane, &sa, &sb);
        if (lane == 0) {
            a_out[node] = sa;
            b_out[node] = sb;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        f += __shfl_down_sync(0xffffffffu, f, o);
        io += __shfl_down_sync(0xffffffffu, io, o);
        st += __shfl_down_sync(0xffffffffu, st, o);
    }
    if (lane == 0) {
        part[0][warp] = f;
        part[1][warp] = io;
        part[2][warp] = st;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        unsigned long long v = 0;
        for (int q = 0; q < kTreeWarps; ++q) v += part[threadIdx.x][q];
        unsigned long long* dst = (threadIdx.x == 0) ? &c->n_failed : (threadIdx.x == 1) ? &c->n_ionized : &c->n_steps;
        if (v) atomicAdd(dst, v);
    }
#pragma unroll
    for (int p = 0; p < kMaxPasses; ++p)
        if (p < npass)
            for (int d = threadIdx.x; d < (1 << w[p]); d += blockDim.x) {
                const uint32_t v = h[p][d];
                if (v) atomicAdd(&ghist[p * kMaxDigits + d], v);
            }
    if (blockIdx.x == 0 && threadIdx.x == 0) c->n_eff = (unsigned long long)n;
    // the last block to finish sums the levels above 0 (the pattern of a fence and a
    // counter of finished blocks: no block waits for another)
    __shared__ bool s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(done, 1u) == gridDim.x - 1u);
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    int64_t m = nb;
    const double* ta = a_out;
    const double* tb = b_out;
    double* oa = a_out + nb;
    double* ob = b_out + nb;
    while (m > 1) {
        const int64_t nb1 = (m + 255) / 256;
        tree_nodes(ta, tb, oa, ob, m, warp, kTreeWarps, lane);
        __syncthreads();
        ta = oa;
        tb = ob;
        oa += nb1;
        ob += nb1;
        m = nb1;
    }
    if (threadIdx.x == 0) {
        sums[0] = (m == 1) ? __ldcg(ta) : 0.0;
        sums[1] = (m == 1) ? __ldcg(tb) : 0.0;
        *done = 0u;  // ready for the next launch
    }
}

__global__ void k_copy_count(const unsigned long long* __restrict__ count, Counters* __restrict__ c) {
    c->n_eff = *count;
}

int64_t tiles_for(int64_t n) { return (n + kTile - 1) / kTile; }
// digit counts and offsets of every pass, one tile counter per pass (+ padding)
constexpr int kOnesweepAuxWords = 2 * kMaxPasses * kMaxDigits + 64;
// the pre-pass's counter of finished blocks, in the padding after the tile counters
constexpr int kPrepassDoneWord = 2 * kMaxPasses * kMaxDigits + 32;

int64_t tree_size(int64_t n) {
    int64_t s = 0, m = n;
    do {
        m = (m + 255) / 256;
        s += m;
    } while (m > 1);
    return s + 2;
}

int key_bits(int64_t grid) {
    int b = 1;
    while (b < 40 && ((int64_t)1 << b) <= grid) ++b;
    return b;
}

// Blocks of a kernel that fit on the device at once, per device and kernel
// (Tag tells the kernels' caches apart).
template <int Tag>
int resident_blocks(const void* fn, int threads) {
    static int cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 152;
    }
    if (!cached[dev]) {
        int per_sm = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || per_sm < 1 ||
            sms < 1) {
            cudaGetLastError();
            return 152;
        }
        cached[dev] = per_sm * sms;
    }
    return cached[dev];
}

// The grid of k_onesweep_pass: as many blocks as fit on the device at once.
int onesweep_blocks() { return resident_blocks<0>((const void*)k_onesweep_pass, kThreads); }

// Stable LSD radix sort of (key, index) pairs on the low `bits` key bits, in as
// few passes of at most kMaxDigitBits as cover them (20 bits: 7 + 7 + 6; 25:
// 9 + 8 + 8).  The order is the same for any split: by key, then by index.
// The sorted pairs are left in the buffers *kout, *vout point to.  `post` holds
// kMaxDigits words per tile, `aux` the digit counts, offsets and tile counters
// (kOnesweepAuxWords), `err` is raised by a look-back that gives up.  With
// hist_ready the caller has cleared both (radix_clear) and counted the digits
// into aux itself (k_deposit_prepass).
int sort_passes(int bits) { return (bits + kMaxDigitBits - 1) / kMaxDigitBits; }

void radix_clear(int64_t max_n, unsigned long long* post, uint32_t* aux, cudaStream_t s) {
    cudaMemsetAsync(aux, 0, sizeof(uint32_t) * kOnesweepAuxWords, s);
    cudaMemsetAsync(post, 0, sizeof(unsigned long long) * (size_t)tiles_for(max_n) * kMaxDigits, s);
}

int radix_sort(const uint32_t* keys, const unsigned long long* count, int64_t max_n, int bits, bool hist_ready,
               uint32_t* const kbuf[2], uint32_t* const vbuf[2], unsigned long long* post, uint32_t* aux,
               unsigned long long* err, const uint32_t** kout, const uint32_t** vout, cudaStream_t s) {
    const int64_t nb = tiles_for(max_n);
    const int npass = sort_passes(bits);
    uint32_t* ghist = aux;
    uint32_t* base = aux + kMaxPasses * kMaxDigits;
    unsigned int* tile_ctr = aux + 2 * kMaxPasses * kMaxDigits;
    int launches = 1;
    if (!hist_ready) {
        radix_clear(max_n, post, aux, s);
        int hblocks = onesweep_blocks();
        if ((int64_t)hblocks > nb) hblocks = (int)nb;
        k_onesweep_hist<<<hblocks, kThreads, 0, s>>>(keys, count, bits, npass, ghist);
        ++launches;
    }
    k_onesweep_scan<<<1, kMaxDigits, 0, s>>>(ghist, npass, base);
    const uint32_t* kin = keys;
    const uint32_t* vin = nullptr;
    int which = 0;
    const int grid = (int)std::min<int64_t>(nb, onesweep_blocks());
    for (int p = 0; p < npass; ++p) {
        int w = 0, shift = 0;
        pass_digits(bits, npass, p, &w, &shift);
        uint32_t* ko = kbuf[which];
        uint32_t* vo = vbuf[which];
        const uint32_t* bp = base + p * kMaxDigits;
        unsigned int* tc = tile_ctr + p;
        k_onesweep_pass<<<grid, kThreads, 0, s>>>(kin, vin, ko, vo, count, p, shift, w, bp, post, tc, err);
        ++launches;
        kin = ko;
        vin = vo;
        which ^= 1;
    }
    *kout = kin;
    *vout = vin;
    return launches;
}

}  // namespace

size_t deposit_scratch_bytes(int64_t max_n) {
    int64_t nb = tiles_for(max_n > 0 ? max_n : 1);
    size_t bytes = 0;
    bytes += 4 * (size_t)max_n * sizeof(uint32_t) + 4 * 256;  // keys a/b, vals a/b
    bytes += (size_t)nb * kMaxDigits * sizeof(unsigned long long) + 256;
    bytes += (size_t)kOnesweepAuxWords * sizeof(uint32_t) + 256;
    bytes += 2 * (size_t)tree_size(max_n) * sizeof(double) + 512;
    return bytes;
}

void deposit_scratch_carve(void* base, int64_t max_n, DepositScratch* d) {
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    char* p = (char*)base;
    size_t off = 0;
    int64_t nb = tiles_for(max_n > 0 ? max_n : 1);
    d->keys_a = (uint32_t*)(p + off); off = align(off + (size_t)max_n * 4);
    d->keys_b = (uint32_t*)(p + off); off = align(off + (size_t)max_n * 4);
    d->vals_a = (uint32_t*)(p + off); off = align(off + (size_t)max_n * 4);
    d->vals_b = (uint32_t*)(p + off); off = align(off + (size_t)max_n * 4);
    d->post = (unsigned long long*)(p + off); off = align(off + (size_t)nb * kMaxDigits * 8);
    d->aux = (uint32_t*)(p + off); off = align(off + (size_t)kOnesweepAuxWords * 4);
    int64_t ts = tree_size(max_n);
    d->tree_a = (double*)(p + off); off = align(off + (size_t)ts * 8);
    d->tree_b = (double*)(p + off);
}

int launch_deposit(const DJob& J, const TrajOut& out, const unsigned long long* count, int64_t max_n,
                   DepositScratch d, double* spec_re, double* spec_im, double* momentum_spec,
                   double* sums, Counters* counters, cudaStream_t s) {
    int launches = 0;
    const int64_t grid = J.grid;
    const int coherent = (J.phase != ETRAJ_PHASE_CTMC) ? 1 : 0;
    cudaMemsetAsync(spec_re, 0, (size_t)grid * sizeof(double), s);
    if (coherent) cudaMemsetAsync(spec_im, 0, (size_t)grid * sizeof(double), s);
    cudaMemsetAsync(counters, 0, sizeof(Counters), s);
    if (max_n > 0) {
        // one read of the per-trajectory outputs: digit counts, the trees, counters
        const int bits = key_bits(grid);
        radix_clear(max_n, d.post, d.aux, s);
        const int64_t nodes = (max_n + 255) / 256;
        int pblocks = resident_blocks<1>((const void*)k_deposit_prepass, 32 * kTreeWarps);
        if ((int64_t)pblocks * kTreeWarps > nodes) pblocks = (int)((nodes + kTreeWarps - 1) / kTreeWarps);
        unsigned int* done = d.aux + kPrepassDoneWord;
        k_deposit_prepass<<<pblocks, 32 * kTreeWarps, 0, s>>>(out.key, out.status, out.steps, out.w_ion, out.w_unc,
                                                              count, bits, sort_passes(bits), d.aux, d.tree_a,
                                                              d.tree_b, sums, done, counters);
        ++launches;
        // stable LSD radix sort of (key, survivor index); keys are in [0, grid]
        uint32_t* kbuf[2] = {d.keys_a, d.keys_b};
        uint32_t* vbuf[2] = {d.vals_a, d.vals_b};
        const uint32_t *kin = nullptr, *vin = nullptr;
        launches += radix_sort(out.key, count, max_n, bits, true, kbuf, vbuf, d.post, d.aux,
                               &counters->sort_err, &kin, &vin, s);
        launches += launch_bin_sums(kin, vin, count, max_n, grid, out.c_re, out.c_im, coherent, spec_re,
                                    spec_im, momentum_spec, s);
    } else {
        cudaMemsetAsync(sums, 0, 2 * sizeof(double), s);
        k_copy_count<<<1, 1, 0, s>>>(count, counters);
        int fblocks = (int)((grid + 255) / 256);
        if (fblocks > 152 * 16) fblocks = 152 * 16;
        k_finalize_spec<<<fblocks, 256, 0, s>>>(spec_re, spec_im, grid, coherent, momentum_spec);
        launches += 2;
    }
    return launches;
}

// ---- per-instance results of a multi-instance launch ---------------------------------
// Survivors are ordered by candidate index and the instances' candidates are
// concatenated, so each instance's survivors form one segment [seg[i], seg[i+1]).

namespace {

__global__ void k_inst_segments(const int64_t* __restrict__ idx, const unsigned long long* __restrict__ count,
                                const BulkInst* __restrict__ inst, int n_inst, int64_t* __restrict__ seg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n_inst) return;
    const int64_t n = (int64_t)*count;
    if (i == 0) {
        seg[0] = 0;
        return;
    }
    // first survivor whose candidate index is >= cand_end of instance i-1
    const int64_t key = inst[i - 1].cand_end;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (idx[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    seg[i] = lo;
}

// The canonical ion_prob tree (tree_node's rule) over one instance's
// segment per block, levels ping-ponging between two scratch regions.
__global__ void __launch_bounds__(256)
k_inst_tree(const double* __restrict__ wa, const double* __restrict__ wb, const int64_t* __restrict__ seg,
            double* __restrict__ scratch, int64_t region, double* __restrict__ sums) {
    const int inst = blockIdx.x;
    const int64_t b0 = seg[inst], len = seg[inst + 1] - b0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // per instance: 4 arrays of ceil(len/256)+1 doubles (a, b in each of two
    // buffers) from 4 * (ceil(b0/256) + 2 inst); since ceil(x) + ceil(y) <=
    // ceil(x+y) + 1 the regions of consecutive instances do not overlap
    double* bufA = scratch + 4 * (((b0 + 255) >> 8) + 2 * (int64_t)inst);
    (void)region;
    const double* ina = wa + b0;
    const double* inb = wb + b0;
    double* outa = bufA;
    double* outb = bufA + ((len + 255) >> 8) + 1;
    double* alta = outb + ((len + 255) >> 8) + 1;
    double* altb = alta + ((len + 255) >> 8) + 1;
    int64_t m = len;
    if (m == 0) {
        if (threadIdx.x == 0) {
            sums[2 * inst] = 0.0;
            sums[2 * inst + 1] = 0.0;
        }
        return;
    }
    for (;;) {
        const int64_t nb = (m + 255) >> 8;
        for (int64_t node = warp; node < nb; node += (int64_t)(blockDim.x >> 5)) {
            const int64_t base = node * 256 + 8 * lane;
            double va[8], vb[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const bool in = base + j < m;
                va[j] = in ? ina[base + j] : 0.0;
                vb[j] = in ? inb[base + j] : 0.0;
            }
#pragma unroll
            for (int w = 4; w >= 1; w >>= 1) {
#pragma unroll
                for (int j = 0; j < w; ++j) {
                    va[j] = va[2 * j] + va[2 * j + 1];
                    vb[j] = vb[2 * j] + vb[2 * j + 1];
                }
            }
            double sa = va[0], sb = vb[0];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double ra = __shfl_down_sync(0xffffffffu, sa, o);
                const double rb = __shfl_down_sync(0xffffffffu, sb, o);
                if ((lane & (2 * o - 1)) == 0) {
                    sa = sa + ra;
                    sb = sb + rb;
                }
            }
            if (lane == 0) {
                outa[node] = sa;
                outb[node] = sb;
            }
        }
        __syncthreads();
        if (nb == 1) break;
        m = nb;
        ina = outa;
        inb = outb;
        double* ta = alta;
        double* tb = altb;
        alta = outa;
        altb = outb;
        outa = ta;
        outb = tb;
    }
    if (threadIdx.x == 0) {
        sums[2 * inst] = outa[0];
        sums[2 * inst + 1] = outb[0];
    }
}

__global__ void __launch_bounds__(256)
k_inst_counters(const int32_t* __restrict__ status, const int32_t* __restrict__ steps,
                const int64_t* __restrict__ seg, Counters* __restrict__ c) {
    const int inst = blockIdx.x;
    const int64_t b0 = seg[inst], b1 = seg[inst + 1];
    unsigned long long f = 0, io = 0, st = 0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        const int32_t v = status[i];
        f += ((v & 0xff) != 0) ? 1ull : 0ull;
        io += (v & 0x100) ? 1ull : 0ull;
        st += (unsigned long long)steps[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        f += __shfl_down_sync(0xffffffffu, f, o);
        io += __shfl_down_sync(0xffffffffu, io, o);
        st += __shfl_down_sync(0xffffffffu, st, o);
    }
    __shared__ unsigned long long part[3][8];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        part[0][w] = f;
        part[1][w] = io;
        part[2][w] = st;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a = 0, b = 0, d = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            a += part[0][k];
            b += part[1][k];
            d += part[2][k];
        }
        c[inst].n_eff = (unsigned long long)(b1 - b0);
        c[inst].n_failed = a;
        c[inst].n_ionized = b;
        c[inst].n_steps = d;
    }
}

// out[b] = sum_i w[i] * mspec[i * grid + b], instances in order from 0.0
__global__ void k_weighted_sum(const double* __restrict__ mspec, int n_inst, int64_t grid,
                               const double* __restrict__ w, double* __restrict__ out) {
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < grid;
         b += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int i = 0; i < n_inst; ++i) acc = acc + w[i] * mspec[(int64_t)i * grid + b];
        out[b] = acc;
    }
}

}  // namespace

size_t instance_scratch_doubles(int64_t max_n, int n_inst) {
    // regions up to 4 * (ceil(n/256) + 2 n_inst) (see k_inst_tree)
    return (size_t)4 * (size_t)(((max_n + 255) >> 8) + 2 * (int64_t)n_inst + 2);
}

int launch_instance_reductions(const TrajOut& out, const int64_t* idx, const unsigned long long* count,
                               const BulkInst* inst, int n_inst, int64_t* seg, double* scratch,
                               double* sums, Counters* counters, cudaStream_t s) {
    k_inst_segments<<<1, 128, 0, s>>>(idx, count, inst, n_inst, seg);
    k_inst_tree<<<n_inst, 256, 0, s>>>(out.w_ion, out.w_unc, seg, scratch, 0, sums);
    k_inst_counters<<<n_inst, 256, 0, s>>>(out.status, out.steps, seg, counters);
    return 3;
}

int launch_weighted_sum(const double* mspec, int n_inst, int64_t grid, const double* w, double* out,
                        cudaStream_t s) {
    int64_t blocks = (grid + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    k_weighted_sum<<<(int)(blocks > 0 ? blocks : 1), 256, 0, s>>>(mspec, n_inst, grid, w, out);
    return 1;
}

}  // namespace etraj

// ---- deposit without allocation ------------------------------------------------------
//
// Some callers cannot allocate device memory while they call into this library:
// a host that lets only its own memory pool own device memory (for example a
// Julia program whose CUDA.jl arrays are the only allocations it permits), a
// caller that reserves all of its memory before a latency-critical run, or code
// that must not synchronize the device, as cudaMalloc and cudaFree may.  For
// them etraj_deposit_noalloc runs the deterministic deposit (stable radix sort
// of (bin, electron), per-bin sums in electron order, |A|^2) on caller-owned
// inputs and outputs, with its sort scratch in one fixed device array declared
// below.  The array's size is fixed at build time (kNoallocMaxN contributions,
// about 10.5 MiB) and every GPU that loads this library holds it until the
// process exits.  Keys above the grid are taken as the grid ("not deposited")
// before the sort, so a bad key can neither alias a bin nor leave the sort's
// key range.

#include <mutex>

namespace etraj {
namespace {

constexpr int64_t kNoallocMaxN = (int64_t)1 << 19;
constexpr int64_t kNoallocTiles = (kNoallocMaxN + kTile - 1) / kTile;
// layout: clamped keys | keys_a | keys_b | vals_a | vals_b | look-back posts | aux | count, error flag
constexpr size_t kNoallocOffPost = (size_t)5 * kNoallocMaxN * sizeof(uint32_t);
constexpr size_t kNoallocOffAux = kNoallocOffPost + (size_t)kNoallocTiles * kMaxDigits * sizeof(unsigned long long);
constexpr size_t kNoallocOffCount = (kNoallocOffAux + (size_t)kOnesweepAuxWords * sizeof(uint32_t) + 255) & ~(size_t)255;
constexpr size_t kNoallocBytes = kNoallocOffCount + 256;

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};
int g_noalloc_sms[kMaxDevices] = {};

__global__ void k_set_count(unsigned long long* c, unsigned long long n) { *c = n; }

// The caller's keys with every key above the grid replaced by the grid, the
// "not deposited" key: the sort then sees only keys in [0, grid].
__global__ void k_clamp_keys(const uint32_t* __restrict__ in, int64_t n, uint32_t grid, uint32_t* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t k = in[i];
        out[i] = k > grid ? grid : k;
    }
}

}  // namespace
}  // namespace etraj

static __device__ __align__(256) unsigned char g_noalloc_scratch[etraj::kNoallocBytes];

namespace etraj {
namespace {

// Device address of g_noalloc_scratch on the current device.  The symbol's
// host-side name is only a stand-in, so the address is looked up once per
// device with that device current (cudaGetSymbolAddress) and cached, with the
// device's SM count (grid sizes).
int noalloc_scratch(void** out, int* sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ETRAJ_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return ETRAJ_ERR_CUDA;
        }
        int nsm = 0;
        if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1) {
            cudaGetLastError();
            return ETRAJ_ERR_CUDA;
        }
        g_noalloc_sms[dev] = nsm;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    *sms = g_noalloc_sms[dev];
    return ETRAJ_OK;
}

}  // namespace
}  // namespace etraj

extern "C" int etraj_deposit_noalloc(int64_t n, const uint32_t* key, const double* c_re,
                                     const double* c_im, int64_t grid, int coherent, double* spec_re,
                                     double* spec_im, double* momentum_spec, void* cuda_stream) {
    using namespace etraj;
    if (n < 0 || n > kNoallocMaxN) return ETRAJ_ERR_INVALID_ARGUMENT;
    if (grid < 1 || grid >= (int64_t)0xFFFFFFFFll) return ETRAJ_ERR_INVALID_ARGUMENT;
    if (!spec_re || !momentum_spec || (coherent && !spec_im)) return ETRAJ_ERR_INVALID_ARGUMENT;
    if (n > 0 && (!key || !c_re || (coherent && !c_im))) return ETRAJ_ERR_INVALID_ARGUMENT;
    void* base = nullptr;
    int sms = 0;
    int st = noalloc_scratch(&base, &sms);
    if (st != ETRAJ_OK) return st;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    unsigned char* p = (unsigned char*)base;
    uint32_t* kclamp = (uint32_t*)p;
    uint32_t* kbuf[2] = {(uint32_t*)p + kNoallocMaxN, (uint32_t*)p + 2 * kNoallocMaxN};
    uint32_t* vbuf[2] = {(uint32_t*)p + 3 * kNoallocMaxN, (uint32_t*)p + 4 * kNoallocMaxN};
    unsigned long long* post = (unsigned long long*)(p + kNoallocOffPost);
    uint32_t* aux = (uint32_t*)(p + kNoallocOffAux);
    unsigned long long* count = (unsigned long long*)(p + kNoallocOffCount);
    unsigned long long* err = count + 1;
    // the outputs start at zero; the scratch keeps the previous call's contents and
    // every part of it that is read is written first (count, histograms, sorted pairs)
    cudaMemsetAsync(spec_re, 0, (size_t)grid * sizeof(double), s);
    if (coherent) cudaMemsetAsync(spec_im, 0, (size_t)grid * sizeof(double), s);
    k_set_count<<<1, 1, 0, s>>>(count, (unsigned long long)n);
    if (n > 0) {
        const uint32_t *kin = nullptr, *vin = nullptr;
        int cblocks = (int)((n + 255) / 256);
        if (cblocks > sms * 8) cblocks = sms * 8;
        k_clamp_keys<<<cblocks, 256, 0, s>>>(key, n, (uint32_t)grid, kclamp);
        radix_sort(kclamp, count, n, key_bits(grid), false, kbuf, vbuf, post, aux, err, &kin, &vin, s);
        launch_bin_sums(kin, vin, count, n, grid, c_re, c_im, coherent, spec_re, spec_im, momentum_spec, s);
    } else {
        int fblocks = (int)((grid + 255) / 256);
        if (fblocks > sms * 16) fblocks = sms * 16;
        k_finalize_spec<<<fblocks, 256, 0, s>>>(spec_re, spec_im, grid, coherent, momentum_spec);
    }
    return (cudaGetLastError() == cudaSuccess) ? ETRAJ_OK : ETRAJ_ERR_CUDA;
}
