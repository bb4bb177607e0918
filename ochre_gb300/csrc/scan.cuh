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

template <class T>
struct ScanStatus {
    uint32_t flag;   // 0: nothing yet, 1: aggregate published, 2: inclusive prefix published
    uint32_t pad;
    T agg;
    T inc;
};

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
            if (lane == 0) {
                st_words(&me->inc, tile_agg);
                st_release(&me->flag, 2u);
            }
        } else {
            if (lane == 0) {
                st_words(&me->agg, tile_agg);
                st_release(&me->flag, 1u);
            }
            int64_t top = (int64_t)tile - 1;
            long long spins = 0;
            const long long poll_limit = spin_limit(err);
            while (top >= 0) {
                const int64_t j = top - lane;
                uint32_t f = 2u;   // before tile 0: an inclusive identity
                if (j >= 0) f = ld_acquire(&status[j].flag);
                const uint32_t m2 = __ballot_sync(0xffffffffu, f == 2u);
                const int limit = m2 ? __ffs(m2) - 1 : 31;   // lanes [0, limit] are needed
                const uint32_t need = limit == 31 ? 0xffffffffu : ((1u << (limit + 1)) - 1u);
                if (__ballot_sync(0xffffffffu, f == 0u) & need) {
                    if (wait_give_up_warp(spins, poll_limit, err)) break;
                    if (spins > 64) __nanosleep(64);
                    continue;
                }
                T v = identity;
                if (lane <= limit && j >= 0) v = ld_words(f == 2u ? &status[j].inc : &status[j].agg);
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const T o = shfl_down_T(v, d);
                    if (lane + d < 32) v = op(o, v);
                }
                prefix = op(shfl_idx_T(v, 0), prefix);
                if (m2) break;
                top -= 32;
            }
            if (lane == 0) {
                st_words(&me->inc, op(prefix, tile_agg));
                st_release(&me->flag, 2u);
            }
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
