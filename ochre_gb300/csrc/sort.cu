// Stage 3: stable LSD radix sort of (key, value) pairs, onesweep style.
//
// Reference counterpart: the two sort_unstable_by_key calls of finish
// (rasterizer.rs:209, 211).  The reference's sorts are unstable, so the f32
// accumulation order inside a tile is unspecified there; this sort is stable,
// which makes the GPU result deterministic.
//
// Digits are 8 bits wide, or up to 11 (the tunable sort_digit_bits: fewer
// passes, larger per-tile histograms and look-back rows); a sort of k key bits
// takes ceil(k / width) passes of balanced widths.
// One upfront kernel histograms every digit of every pass; each pass
// then ranks a tile of keys in shared memory (per-warp counters with
// __match_any_sync for stable ranks), publishes its per-digit counts and
// resolves its global offsets by decoupled look-back over earlier tiles
// (bounded spins; a look-back word holds its flag and count together, so
// relaxed accesses suffice), and scatters through shared memory so that
// runs of equal digits leave as contiguous writes.
#include "common.cuh"
#include "internal.h"

#include <algorithm>
#include <utility>
#include <vector>

namespace ochre {

constexpr int SORT_BLOCK = 256;
constexpr int SORT_WARPS = SORT_BLOCK / 32;
constexpr int SORT_ITEMS = 15;
constexpr int SORT_TILE = SORT_BLOCK * SORT_ITEMS;
constexpr uint32_t LB_AGG = 1u << 30, LB_INC = 2u << 30, LB_MASK = (1u << 30) - 1u;
constexpr int LB_WINDOW = 8;      // predecessor tiles one digit's look-back reads per round
constexpr int SORT_MAX_PASSES = 8;

// The digits of a sort: pass p takes `width[p]` bits from bit `shift[p]`
// (widths balanced over the key bits, at most the digit width RB).
struct SortPlan {
    int passes;
    uint8_t shift[SORT_MAX_PASSES];
    uint8_t width[SORT_MAX_PASSES];
};

template <class K, int RB>
__global__ void __launch_bounds__(256) k_sort_hist(const K* __restrict__ keys, uint64_t n, const uint32_t* n_dev,
                                                   SortPlan plan, uint32_t* __restrict__ hist) {
    constexpr int RADIX = 1 << RB;
    constexpr int MAXP = (64 + RB - 1) / RB;
    __shared__ uint32_t sh[MAXP][RADIX];
    n = dev_count(n, n_dev);
    for (int i = threadIdx.x; i < MAXP * RADIX; i += blockDim.x) (&sh[0][0])[i] = 0u;
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const K k = keys[i];
#pragma unroll
        for (int p = 0; p < MAXP; p++)
            if (p < plan.passes) atomicAdd(&sh[p][(uint32_t)(k >> plan.shift[p]) & ((1u << plan.width[p]) - 1u)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < plan.passes * RADIX; i += blockDim.x) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(hist + i, v);
    }
}

// Exclusive scan of each pass's RADIX counts (one block per pass).
template <int RB>
__global__ void k_sort_offsets(const uint32_t* __restrict__ hist, uint32_t* __restrict__ off) {
    constexpr int RADIX = 1 << RB;
    constexpr int PER = RADIX / 256;   // consecutive digits per thread
    __shared__ uint32_t s[256];
    const int p = blockIdx.x, t = threadIdx.x;
    uint32_t v[PER], sum = 0;
#pragma unroll
    for (int q = 0; q < PER; q++) {
        v[q] = hist[p * RADIX + t * PER + q];
        sum += v[q];
    }
    s[t] = sum;
    __syncthreads();
    for (int k = 1; k < 256; k <<= 1) {
        const uint32_t a = t >= k ? s[t - k] : 0u;
        __syncthreads();
        s[t] += a;
        __syncthreads();
    }
    uint32_t run = s[t] - sum;
#pragma unroll
    for (int q = 0; q < PER; q++) {
        off[p * RADIX + t * PER + q] = run;
        run += v[q];
    }
}

// Shared memory of a onesweep block: the tile's keys and values, per-warp
// digit counters, the tile's digit starts and global digit bases, a word.
template <class K, int RB>
constexpr size_t onesweep_smem() {
    return (size_t)SORT_TILE * (sizeof(K) + 4) + ((size_t)SORT_WARPS * (1 << RB) + 2 * (1 << RB) + 4) * 4;
}

// Blocks per SM: three with 8-bit digits (register-bound otherwise: the
// 32-bit-key form would take more than 85 registers and drop to two); wider
// digits are held to two by their shared memory.
template <class K, int RB>
__global__ void __launch_bounds__(SORT_BLOCK, RB <= 8 ? 3 : 2) k_onesweep(
    const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in, K* __restrict__ keys_out,
    uint32_t* __restrict__ vals_out, uint64_t n, const uint32_t* n_dev, int shift, uint32_t mask,
    const uint32_t* __restrict__ digit_off, uint32_t* lookback, uint32_t* ticket, uint32_t* err) {
    constexpr int RADIX = 1 << RB;
    constexpr int PER = RADIX / SORT_BLOCK;   // digits per thread in the offset phase
    extern __shared__ __align__(16) unsigned char smem[];
    K* s_keys = reinterpret_cast<K*>(smem);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + SORT_TILE);
    uint32_t* s_whist = s_vals + SORT_TILE;               // [SORT_WARPS][RADIX]
    uint32_t* s_tile_excl = s_whist + SORT_WARPS * RADIX;  // [RADIX]
    uint32_t* s_gbase = s_tile_excl + RADIX;               // [RADIX]
    uint32_t* s_misc = s_gbase + RADIX;                    // [0]: tile id

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (run_aborted(err)) return;   // an earlier wait of the run gave up
    if (threadIdx.x == 0) s_misc[0] = atomicAdd(ticket, 1u);
    for (int i = lane; i < RADIX; i += 32) s_whist[warp * RADIX + i] = 0u;
    __syncthreads();
    const uint32_t tile = s_misc[0];
    const uint64_t tile_base = (uint64_t)tile * SORT_TILE;
    // device-held count (graph replays): tiles past it end before publishing;
    // every tile that sorts precedes them
    n = dev_count(n, n_dev);
    if (tile_base >= n) return;
    const uint64_t warp_base = tile_base + (uint64_t)warp * 32 * SORT_ITEMS;
    const uint32_t lt_mask = (1u << lane) - 1u;

    K key[SORT_ITEMS];
    uint32_t val[SORT_ITEMS];
    uint32_t rank[SORT_ITEMS];
    uint32_t dig[SORT_ITEMS];
    // every load of the tile first (all in flight together), then the ranking
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; k++) {
        const uint64_t i = warp_base + (uint64_t)k * 32 + lane;
        const bool valid = i < n;
        key[k] = valid ? keys_in[i] : (K)0;
        val[k] = valid ? vals_in[i] : 0u;
    }
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; k++) {
        const uint64_t i = warp_base + (uint64_t)k * 32 + lane;
        const bool valid = i < n;
        const uint32_t d = valid ? ((uint32_t)(key[k] >> shift) & mask) : (uint32_t)RADIX;
        dig[k] = d;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        uint32_t b = 0;
        if (lane == leader && d < (uint32_t)RADIX) {
            b = s_whist[warp * RADIX + d];
            s_whist[warp * RADIX + d] = b + __popc(peers);
        }
        b = __shfl_sync(0xffffffffu, b, leader);
        rank[k] = b + __popc(peers & lt_mask);
        __syncwarp();
    }
    __syncthreads();

    // PER digits per thread: exclusive over warps, tile count, look-back
#pragma unroll 1
    for (int q = 0; q < PER; q++) {
        const int d = threadIdx.x + q * SORT_BLOCK;
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < SORT_WARPS; w++) {
            const uint32_t c = s_whist[w * RADIX + d];
            s_whist[w * RADIX + d] = run;
            run += c;
        }
        uint32_t* my = lookback + (size_t)tile * RADIX + d;
        uint32_t excl = 0;
        if (tile == 0) {
            st_relaxed(my, LB_INC | run);
        } else {
            st_relaxed(my, LB_AGG | run);
            // windowed look-back: LB_WINDOW predecessors per round, read
            // together (one latency per round instead of one per tile), up
            // to the nearest inclusive value
            int64_t top = (int64_t)tile - 1;
            long long spins = 0;
            const long long poll_limit = spin_limit(err);
            // the nearest predecessor alone first: often it is inclusive already
            {
                const uint32_t v = ld_relaxed(lookback + (size_t)top * RADIX + d);
                if ((v & ~LB_MASK) == LB_INC) {
                    excl = v & LB_MASK;
                    top = -1;
                }
            }
            while (top >= 0) {
                uint32_t v[LB_WINDOW];
#pragma unroll
                for (int k = 0; k < LB_WINDOW; k++) {
                    const int64_t j = top - k;
                    v[k] = j >= 0 ? ld_relaxed(lookback + (size_t)j * RADIX + d) : LB_INC;   // before tile 0: an inclusive 0
                }
                int k_inc = LB_WINDOW;
#pragma unroll
                for (int k = LB_WINDOW - 1; k >= 0; k--)
                    if ((v[k] & ~LB_MASK) == LB_INC) k_inc = k;
                bool missing = false;
                uint32_t sum = 0;
#pragma unroll
                for (int k = 0; k < LB_WINDOW; k++) {
                    if (k <= k_inc) {
                        if ((v[k] & ~LB_MASK) == 0u) missing = true;
                        sum += v[k] & LB_MASK;
                    }
                }
                if (missing) {
                    if (wait_give_up(spins, poll_limit, err)) break;
                    if (spins > 64) __nanosleep(64);
                    continue;
                }
                excl += sum;
                if (k_inc < LB_WINDOW) break;
                top -= LB_WINDOW;
            }
            st_relaxed(my, LB_INC | (excl + run));
        }
        s_gbase[d] = digit_off[d] + excl;
        s_tile_excl[d] = run;
    }
    __syncthreads();
    if (warp == 0) {
        // block exclusive scan of the tile's digit counts: RADIX / 32 per lane
        constexpr int PL = RADIX / 32;
        uint32_t v[PL], sum = 0;
#pragma unroll
        for (int q = 0; q < PL; q++) { v[q] = s_tile_excl[lane * PL + q]; sum += v[q]; }
        uint32_t inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        uint32_t run = inc - sum;
#pragma unroll
        for (int q = 0; q < PL; q++) { s_tile_excl[lane * PL + q] = run; run += v[q]; }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; k++) {
        const uint32_t d = dig[k];
        if (d < (uint32_t)RADIX) {
            const uint32_t pos = s_tile_excl[d] + s_whist[warp * RADIX + d] + rank[k];
            s_keys[pos] = key[k];
            s_vals[pos] = val[k];
        }
    }
    __syncthreads();
    const uint64_t remain = n - tile_base;
    const int cnt = remain < (uint64_t)SORT_TILE ? (int)remain : SORT_TILE;
    for (int i = threadIdx.x; i < cnt; i += SORT_BLOCK) {
        const K k = s_keys[i];
        const uint32_t d = (uint32_t)(k >> shift) & mask;
        const uint32_t g = s_gbase[d] + ((uint32_t)i - s_tile_excl[d]);
        keys_out[g] = k;
        vals_out[g] = s_vals[i];
    }
}

template <class K, int RB>
static int sort_impl(ochre_gpu_ctx* ctx, uint64_t n, uint32_t key_bits, cudaStream_t s, uint32_t* passes_done) {
    constexpr int RADIX = 1 << RB;
    DevScalars* ds = dev_scalars(ctx);
    // graph replays: n is the capacity, the count is on the device, and every
    // pass runs (no read-back to skip passes whose digit is constant)
    const uint32_t* n_dev = ctx->plan ? &ds->n_entries : nullptr;
    SortPlan plan{};
    const uint32_t kb = std::max<uint32_t>(key_bits, 1u);
    plan.passes = (int)((kb + RB - 1) / RB);
    if (plan.passes > SORT_MAX_PASSES) return OCHRE_E_INVALID;
    for (int p = 0, at = 0; p < plan.passes; p++) {
        // balanced widths: the first kb % passes passes take one bit more
        const int w = (int)(kb / plan.passes) + (p < (int)(kb % plan.passes) ? 1 : 0);
        plan.shift[p] = (uint8_t)at;
        plan.width[p] = (uint8_t)w;
        at += w;
    }
    const int passes = plan.passes;
    const uint64_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    OCHRE_CUDA_TRY(ctx->sort_hist.ensure((size_t)passes * RADIX * 4 * 2));
    OCHRE_CUDA_TRY(ctx->sort_lookback.ensure((size_t)tiles * RADIX * 4));
    uint32_t* hist = ctx->sort_hist.as<uint32_t>();
    uint32_t* off = hist + passes * RADIX;
    OCHRE_CUDA_TRY(cudaMemsetAsync(hist, 0, (size_t)passes * RADIX * 4, s));
    K* kin = ctx->keys.as<K>();
    uint32_t* vin = ctx->vals.as<uint32_t>();
    K* kout = ctx->keys_alt.as<K>();
    uint32_t* vout = ctx->vals_alt.as<uint32_t>();
    {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        int blocks = (int)std::min<uint64_t>((n + 255) / 256, (uint64_t)std::max(sms, 1) * 8);
        OCHRE_LAUNCH(ctx, "sort_hist", s, k_sort_hist<K, RB><<<blocks, 256, 0, s>>>(kin, n, n_dev, plan, hist));
        OCHRE_CUDA_TRY(cudaGetLastError());
        OCHRE_LAUNCH(ctx, "sort_offsets", s, k_sort_offsets<RB><<<passes, 256, 0, s>>>(hist, off));
        OCHRE_CUDA_TRY(cudaGetLastError());
    }
    const size_t smem = onesweep_smem<K, RB>();
    OCHRE_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<K, RB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // Skip passes whose digit is constant over all keys (one bucket holds n).
    std::vector<uint32_t> h_hist;
    if (!n_dev) {
        h_hist.resize((size_t)passes * RADIX);
        OCHRE_CUDA_TRY(cudaMemcpyAsync(h_hist.data(), hist, (size_t)passes * RADIX * 4, cudaMemcpyDeviceToHost, s));
        OCHRE_CUDA_TRY(cudaStreamSynchronize(s));
    }
    uint32_t done = 0;
    for (int p = 0; p < passes; p++) {
        bool trivial = false;
        for (int d = 0; d < RADIX && !n_dev; d++)
            if (h_hist[(size_t)p * RADIX + d] == n) trivial = true;
        if (trivial) continue;
        OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->sort_lookback.p, 0, (size_t)tiles * RADIX * 4, s));
        OCHRE_CUDA_TRY(cudaMemsetAsync(&ds->sort_ticket, 0, 4, s));
        OCHRE_LAUNCH(ctx, "sort_onesweep", s, k_onesweep<K, RB><<<(unsigned)tiles, SORT_BLOCK, smem, s>>>(
            kin, vin, kout, vout, n, n_dev, plan.shift[p], (1u << plan.width[p]) - 1u, off + p * RADIX,
            ctx->sort_lookback.as<uint32_t>(), &ds->sort_ticket, &ds->err));
        OCHRE_CUDA_TRY(cudaGetLastError());
        K* tk = kin; kin = kout; kout = tk;
        uint32_t* tv = vin; vin = vout; vout = tv;
        done++;
    }
    if (kin != ctx->keys.as<K>()) {
        // leave the sorted result in ctx->keys / ctx->vals
        std::swap(ctx->keys, ctx->keys_alt);
        std::swap(ctx->vals, ctx->vals_alt);
    }
    *passes_done = done;
    return OCHRE_OK;
}

int stage_sort(ochre_gpu_ctx* ctx, uint64_t n, uint32_t key_bits, cudaStream_t s, uint32_t* passes) {
    *passes = 0;
    if (n <= 1) return OCHRE_OK;
    if (ctx->tune_sort_digit_bits == 11)
        return ctx->keys64 ? sort_impl<uint64_t, 11>(ctx, n, key_bits, s, passes)
                           : sort_impl<uint32_t, 11>(ctx, n, key_bits, s, passes);
    return ctx->keys64 ? sort_impl<uint64_t, 8>(ctx, n, key_bits, s, passes)
                       : sort_impl<uint32_t, 8>(ctx, n, key_bits, s, passes);
}

}  // namespace ochre
