// Stage 3: stable LSD radix sort of (key, value) pairs, onesweep style.
//
// Reference counterpart: the two sort_unstable_by_key calls of finish
// (rasterizer.rs:209, 211).  The reference's sorts are unstable, so the f32
// accumulation order inside a tile is unspecified there; this sort is stable,
// which makes the GPU result deterministic.
//
// One upfront kernel histograms every 8-bit digit of every pass; each pass
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

namespace ochre {

constexpr int SORT_BLOCK = 256;   // one thread per digit in the offset phase
constexpr int SORT_WARPS = SORT_BLOCK / 32;
constexpr int SORT_ITEMS = 15;
constexpr int SORT_TILE = SORT_BLOCK * SORT_ITEMS;
constexpr uint32_t LB_AGG = 1u << 30, LB_INC = 2u << 30, LB_MASK = (1u << 30) - 1u;
constexpr int LB_WINDOW = 8;      // predecessor tiles one digit's look-back reads per round

template <class K>
__global__ void __launch_bounds__(256) k_sort_hist(const K* __restrict__ keys, uint64_t n, const uint32_t* n_dev,
                                                   int passes, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[8][256];
    n = dev_count(n, n_dev);
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&sh[0][0])[i] = 0u;
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const K k = keys[i];
        for (int p = 0; p < passes; p++) atomicAdd(&sh[p][(uint32_t)(k >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(hist + i, v);
    }
}

// Exclusive scan of each pass's 256 counts (one block per pass).
__global__ void k_sort_offsets(const uint32_t* __restrict__ hist, uint32_t* __restrict__ off) {
    __shared__ uint32_t s[256];
    const int p = blockIdx.x, d = threadIdx.x;
    s[d] = hist[p * 256 + d];
    __syncthreads();
    for (int k = 1; k < 256; k <<= 1) {
        const uint32_t v = d >= k ? s[d - k] : 0u;
        __syncthreads();
        s[d] += v;
        __syncthreads();
    }
    off[p * 256 + d] = s[d] - hist[p * 256 + d];
}

// Three blocks per SM (register-bound otherwise: the 32-bit-key form would
// take more than 85 registers and drop to two).
template <class K>
__global__ void __launch_bounds__(SORT_BLOCK, 3) k_onesweep(const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                                                         K* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                         uint64_t n, const uint32_t* n_dev, int shift,
                                                         const uint32_t* __restrict__ digit_off,
                                                         uint32_t* lookback, uint32_t* ticket, uint32_t* err) {
    extern __shared__ __align__(16) unsigned char smem[];
    K* s_keys = reinterpret_cast<K*>(smem);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + SORT_TILE);
    uint32_t* s_whist = s_vals + SORT_TILE;            // [SORT_WARPS][256]
    uint32_t* s_tile_excl = s_whist + SORT_WARPS * 256; // [256]
    uint32_t* s_gbase = s_tile_excl + 256;              // [256]
    uint32_t* s_misc = s_gbase + 256;                   // [0]: tile id

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (run_aborted(err)) return;   // an earlier wait of the run gave up
    if (threadIdx.x == 0) s_misc[0] = atomicAdd(ticket, 1u);
    for (int i = lane; i < 256; i += 32) s_whist[warp * 256 + i] = 0u;
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
        const uint32_t d = valid ? ((uint32_t)(key[k] >> shift) & 255u) : 256u;
        dig[k] = d;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        uint32_t b = 0;
        if (lane == leader && d < 256u) {
            b = s_whist[warp * 256 + d];
            s_whist[warp * 256 + d] = b + __popc(peers);
        }
        b = __shfl_sync(0xffffffffu, b, leader);
        rank[k] = b + __popc(peers & lt_mask);
        __syncwarp();
    }
    __syncthreads();

    // one thread per digit: exclusive over warps, tile count, look-back
    {
        const int d = threadIdx.x;
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < SORT_WARPS; w++) {
            const uint32_t c = s_whist[w * 256 + d];
            s_whist[w * 256 + d] = run;
            run += c;
        }
        uint32_t* my = lookback + (size_t)tile * 256 + d;
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
                const uint32_t v = ld_relaxed(lookback + (size_t)top * 256 + d);
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
                    v[k] = j >= 0 ? ld_relaxed(lookback + (size_t)j * 256 + d) : LB_INC;   // before tile 0: an inclusive 0
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
        // block exclusive scan of run over digits -> tile-local digit starts
        s_tile_excl[d] = run;
    }
    __syncthreads();
    if (warp == 0) {
        // 256 values, 8 per lane
        uint32_t v[8], sum = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) { v[q] = s_tile_excl[lane * 8 + q]; sum += v[q]; }
        uint32_t inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        uint32_t run = inc - sum;
#pragma unroll
        for (int q = 0; q < 8; q++) { s_tile_excl[lane * 8 + q] = run; run += v[q]; }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SORT_ITEMS; k++) {
        const uint32_t d = dig[k];
        if (d < 256u) {
            const uint32_t pos = s_tile_excl[d] + s_whist[warp * 256 + d] + rank[k];
            s_keys[pos] = key[k];
            s_vals[pos] = val[k];
        }
    }
    __syncthreads();
    const uint64_t remain = n - tile_base;
    const int cnt = remain < (uint64_t)SORT_TILE ? (int)remain : SORT_TILE;
    for (int i = threadIdx.x; i < cnt; i += SORT_BLOCK) {
        const K k = s_keys[i];
        const uint32_t d = (uint32_t)(k >> shift) & 255u;
        const uint32_t g = s_gbase[d] + ((uint32_t)i - s_tile_excl[d]);
        keys_out[g] = k;
        vals_out[g] = s_vals[i];
    }
}

template <class K>
static int sort_impl(ochre_gpu_ctx* ctx, uint64_t n, uint32_t key_bits, cudaStream_t s, uint32_t* passes_done) {
    DevScalars* ds = dev_scalars(ctx);
    // graph replays: n is the capacity, the count is on the device, and every
    // pass runs (no read-back to skip passes whose digit is constant)
    const uint32_t* n_dev = ctx->plan ? &ds->n_entries : nullptr;
    const int passes = (int)((key_bits + 7) / 8);
    const uint64_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    OCHRE_CUDA_TRY(ctx->sort_hist.ensure((size_t)passes * 256 * 4 * 2));
    OCHRE_CUDA_TRY(ctx->sort_lookback.ensure((size_t)tiles * 256 * 4));
    uint32_t* hist = ctx->sort_hist.as<uint32_t>();
    uint32_t* off = hist + passes * 256;
    OCHRE_CUDA_TRY(cudaMemsetAsync(hist, 0, (size_t)passes * 256 * 4, s));
    K* kin = ctx->keys.as<K>();
    uint32_t* vin = ctx->vals.as<uint32_t>();
    K* kout = ctx->keys_alt.as<K>();
    uint32_t* vout = ctx->vals_alt.as<uint32_t>();
    {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        int blocks = (int)std::min<uint64_t>((n + 255) / 256, (uint64_t)std::max(sms, 1) * 8);
        OCHRE_LAUNCH(ctx, "sort_hist", s, k_sort_hist<K><<<blocks, 256, 0, s>>>(kin, n, n_dev, passes, hist));
        OCHRE_CUDA_TRY(cudaGetLastError());
        OCHRE_LAUNCH(ctx, "sort_offsets", s, k_sort_offsets<<<passes, 256, 0, s>>>(hist, off));
        OCHRE_CUDA_TRY(cudaGetLastError());
    }
    const size_t smem = (size_t)SORT_TILE * (sizeof(K) + 4) + (SORT_WARPS * 256 + 256 + 256 + 4) * 4;
    OCHRE_CUDA_TRY(cudaFuncSetAttribute(k_onesweep<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // Skip passes whose digit is constant over all keys (one bucket holds n).
    uint32_t h_hist[8 * 256];
    if (!n_dev) {
        OCHRE_CUDA_TRY(cudaMemcpyAsync(h_hist, hist, (size_t)passes * 256 * 4, cudaMemcpyDeviceToHost, s));
        OCHRE_CUDA_TRY(cudaStreamSynchronize(s));
    }
    uint32_t done = 0;
    for (int p = 0; p < passes; p++) {
        bool trivial = false;
        for (int d = 0; d < 256 && !n_dev; d++)
            if (h_hist[(size_t)p * 256 + d] == n) trivial = true;
        if (trivial) continue;
        OCHRE_CUDA_TRY(cudaMemsetAsync(ctx->sort_lookback.p, 0, (size_t)tiles * 256 * 4, s));
        OCHRE_CUDA_TRY(cudaMemsetAsync(&ds->sort_ticket, 0, 4, s));
        OCHRE_LAUNCH(ctx, "sort_onesweep", s, k_onesweep<K><<<(unsigned)tiles, SORT_BLOCK, smem, s>>>(kin, vin, kout, vout, n, n_dev, 8 * p, off + p * 256,
                                                                ctx->sort_lookback.as<uint32_t>(), &ds->sort_ticket,
                                                                &ds->err));
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
    return ctx->keys64 ? sort_impl<uint64_t>(ctx, n, key_bits, s, passes)
                       : sort_impl<uint32_t>(ctx, n, key_bits, s, passes);
}

}  // namespace ochre
