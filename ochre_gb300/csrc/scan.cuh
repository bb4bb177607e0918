// Single-pass device-wide exclusive scan with decoupled look-back.
//
// Generic over the value type T (a trivially copyable struct of 32-bit
// words), the associative operator, the input functor in(i) -> T and the
// output functor out(i, exclusive_prefix, own_value).  Tiles are numbered by
// an atomic ticket taken when a block starts, so a block only ever waits on
// blocks that are already resident; every wait is bounded (wait_give_up_warp)
// and a timeout sets ERR_TIMEOUT instead of hanging.
#pragma once

#include "common.cuh"

namespace ochre {

// A tile's aggregate and inclusive prefix, every 32-bit word of each in a
// 64-bit word whose high half is its flag (1: aggregate, 2: inclusive; 0:
// not yet).  One naturally aligned 64-bit access reads or writes a word with
// its flag, so a reader takes a value once all its words carry the flag, with
// relaxed accesses only, and one round of loads reads a predecessor's flags
// and values together.
template <class T>
struct ScanStatus {
    static constexpr int W = (int)(sizeof(T) / 4);
    uint64_t agg[W];
    uint64_t inc[W];
};
template <class T>
__device__ __forceinline__ void st_flagged(uint64_t* dst, const T& v, uint32_t flag) {
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&v);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); i++) st_relaxed64(dst + i, ((uint64_t)flag << 32) | s[i]);
}
// True when every word of the value carries `flag`; v receives the words.
template <class T>
__device__ __forceinline__ bool ld_flagged(const uint64_t* src, uint32_t flag, T& v) {
    uint32_t* d = reinterpret_cast<uint32_t*>(&v);
    bool ok = true;
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); i++) {
        const uint64_t w = ld_relaxed64(src + i);
        d[i] = (uint32_t)w;
        ok = ok && (uint32_t)(w >> 32) == flag;
    }
    return ok;
}

template <int BLOCK, int ITEMS, class T, class Op, class In, class Out>
__global__ void __launch_bounds__(BLOCK) k_scan(uint64_t n, const uint32_t* n_dev, In in, Out out, Op op,
                                                 T identity, ScanStatus<T>* status, uint32_t* ticket, T* total,
                                                 uint32_t* err) {
    constexpr int WARPS = BLOCK / 32;
    __shared__ uint32_t s_tile;
    __shared__ T s_warp[WARPS];
    __shared__ T s_prefix;
    // A count held on the device (graph replays): the grid covers the
    // capacity n, the scan covers min(*n_dev, n).  Tiles past the count end
    // before publishing anything; no tile that scans waits on them.
    n = dev_count(n, n_dev);
    // an earlier wait of the run gave up: its outputs (this scan's inputs) are
    // not valid; every block ends here, before publishing
    if (run_aborted(err)) return;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    if ((uint64_t)tile * (BLOCK * ITEMS) >= n) return;
    const uint64_t base = (uint64_t)tile * (BLOCK * ITEMS) + (uint64_t)threadIdx.x * ITEMS;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    T v[ITEMS];
    T acc = identity;
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
        const uint64_t i = base + k;
        v[k] = i < n ? in(i) : identity;
        acc = op(acc, v[k]);
    }
    // warp inclusive scan of per-thread aggregates
    T inc = acc;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const T o = shfl_up_T(inc, d);
        if (lane >= d) inc = op(o, inc);
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < WARPS ? s_warp[lane] : identity;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const T o = shfl_up_T(w, d);
            if (lane >= d) w = op(o, w);
        }
        // w = inclusive over warps; turn into exclusive per warp
        const T ex = shfl_up_T(w, 1);
        const T tile_agg = shfl_idx_T(w, WARPS - 1);
        if (lane < WARPS) s_warp[lane] = lane == 0 ? identity : ex;
        // Decoupled look-back by the whole warp, 32 predecessors per round:
        // lane k inspects tile top - k; the window up to the nearest inclusive
        // value is combined in tile order (earlier tiles on the left).
        T prefix = identity;
        ScanStatus<T>* me = status + tile;
        if (tile == 0) {
            if (lane == 0) st_flagged(me->inc, tile_agg, 2u);
        } else {
            if (lane == 0) st_flagged(me->agg, tile_agg, 1u);
            int64_t top = (int64_t)tile - 1;
            long long spins = 0;
            const long long poll_limit = spin_limit(err);
            while (top >= 0) {
                const int64_t j = top - lane;
                // the predecessor's inclusive prefix and aggregate, read together
                bool has_inc = true, has_agg = true;   // before tile 0: an inclusive identity
                T vi = identity, va = identity;
                if (j >= 0) {
                    has_inc = ld_flagged(status[j].inc, 2u, vi);
                    has_agg = ld_flagged(status[j].agg, 1u, va);
                }
                const uint32_t m2 = __ballot_sync(0xffffffffu, has_inc);
                const int limit = m2 ? __ffs(m2) - 1 : 31;   // lanes [0, limit] are needed
                const uint32_t need = limit == 31 ? 0xffffffffu : ((1u << (limit + 1)) - 1u);
                if (__ballot_sync(0xffffffffu, !has_inc && !has_agg) & need) {
                    if (wait_give_up_warp(spins, poll_limit, err)) break;
                    if (spins > 64) __nanosleep(64);
                    continue;
                }
                T v = identity;
                if (lane <= limit && j >= 0) v = has_inc ? vi : va;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const T o = shfl_down_T(v, d);
                    if (lane + d < 32) v = op(o, v);
                }
                prefix = op(shfl_idx_T(v, 0), prefix);
                if (m2) break;
                top -= 32;
            }
            if (lane == 0) st_flagged(me->inc, op(prefix, tile_agg), 2u);
        }
        if (lane == 0) {
            s_prefix = prefix;
            const uint64_t tile_end = (uint64_t)(tile + 1) * (BLOCK * ITEMS);
            if (tile_end >= n && total != nullptr) *total = op(prefix, tile_agg);
        }
    }
    __syncthreads();
    // exclusive prefix of this thread's first item
    T ex_lane = shfl_up_T(inc, 1);
    if (lane == 0) ex_lane = identity;
    T run = op(op(s_prefix, s_warp[warp]), ex_lane);
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
        const uint64_t i = base + k;
        if (i < n) out(i, run, v[k]);
        run = op(run, v[k]);
    }
}

struct OpSumU32 {
    __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a + b; }
};

// Launch helper.  `status` must hold at least scan_tiles(n) entries and,
// together with `ticket`, be zeroed on `stream` before the launch (done here).
constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 8;
inline uint64_t scan_tiles(uint64_t n) { return (n + SCAN_BLOCK * SCAN_ITEMS - 1) / (SCAN_BLOCK * SCAN_ITEMS); }

// `n_dev` (optional): the count lives on the device and `n` is its capacity.
// `first_ticket` (a test hook, else 0): tiles below it are never taken.
template <class T, class Op, class In, class Out>
cudaError_t launch_scan(uint64_t n, In in, Out out, Op op, T identity, void* status, uint32_t* ticket, T* total,
                        uint32_t* err, cudaStream_t stream, const uint32_t* n_dev = nullptr,
                        uint32_t first_ticket = 0u) {
    const uint64_t tiles = scan_tiles(n);
    if (tiles == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(status, 0, tiles * sizeof(ScanStatus<T>), stream);
    if (e != cudaSuccess) return e;
    if (first_ticket == 0u) {
        e = cudaMemsetAsync(ticket, 0, sizeof(uint32_t), stream);
    } else {
        static const uint32_t one = 1u;
        e = cudaMemcpyAsync(ticket, &one, sizeof(uint32_t), cudaMemcpyHostToDevice, stream);
    }
    if (e != cudaSuccess) return e;
    k_scan<SCAN_BLOCK, SCAN_ITEMS, T, Op, In, Out><<<(unsigned)tiles, SCAN_BLOCK, 0, stream>>>(
        n, n_dev, in, out, op, identity, reinterpret_cast<ScanStatus<T>*>(status), ticket, total, err);
    return cudaGetLastError();
}

}  // namespace ochre
