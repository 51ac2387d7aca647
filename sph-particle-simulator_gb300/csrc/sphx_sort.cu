// Stable LSD radix sort of 32-bit cell keys (8-bit digits) and the device-wide exclusive
// scans used by the grid build.
//
// The number of passes is decided on the device (DevState::passes, from the number of
// significant key bits of this step's cell grid), so a whole step can be enqueued -- or
// captured -- without a host round trip: kMaxPasses pass launches are issued and the
// inactive ones return at once.  Pass p reads buffer (p & 1) and writes (p + 1) & 1; the
// result is in buffer (passes & 1).
//
// Stability: within a radix block, warp w owns the contiguous sub-range
// [w*512, (w+1)*512) and walks it in rounds of 32 consecutive keys; ranks inside a round
// come from __match_any_sync, ranks across rounds from a per-warp running count per
// digit, and ranks across warps from an exclusive scan of those counts.  Equal digits
// therefore keep their input order, which is what makes the cell-sorted order
// (cell, insertion index): the keys are produced in insertion order.
#include "sphx_internal.cuh"

namespace sphx {

// ---------------------------------------------------------------------------------------
// generic exclusive scan of uint32 values produced by a functor
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive scan of one value per thread across a kScanThreads block; returns the block
// total through *total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[kScanThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t incl = warp_incl_scan(v, lane);
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = (lane < kScanThreads / 32) ? warp_sums[lane] : 0u;
        s = warp_incl_scan(s, lane);
        if (lane < kScanThreads / 32) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t warp_off = warp ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[kScanThreads / 32 - 1];
    __syncthreads();
    return warp_off + incl - v;
}

template <class Src>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(Src src, uint32_t n, uint32_t* part) {
    if (!src.active()) return;
    const uint32_t base = blockIdx.x * kScanTileN + threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s += src(base + i);
    uint32_t total;
    block_excl_scan(s, &total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

// Single-block exclusive scan of the block partials; writes the grand total.
template <class Src>
__global__ void __launch_bounds__(1024) k_scan_partials(Src src, uint32_t* part, uint32_t nb,
                                                        uint32_t* total_out) {
    if (!src.active()) return;
    __shared__ uint32_t warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t per = (nb + 1023) / 1024;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t s = 0;
    for (uint32_t i = 0; i < per; ++i)
        if (b0 + i < nb) s += part[b0 + i];
    const uint32_t incl = warp_incl_scan(s, lane);
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) warp_sums[lane] = warp_incl_scan(warp_sums[lane], lane);
    __syncthreads();
    uint32_t run = (warp ? warp_sums[warp - 1] : 0u) + incl - s;
    for (uint32_t i = 0; i < per; ++i) {
        if (b0 + i < nb) {
            const uint32_t v = part[b0 + i];
            part[b0 + i] = run;
            run += v;
        }
    }
    if (threadIdx.x == 1023 && total_out) *total_out = run;
}

template <class Src, class Sink>
__global__ void __launch_bounds__(kScanThreads) k_scan_emit(Src src, Sink sink, uint32_t n,
                                                            const uint32_t* part) {
    if (!src.active()) return;
    const uint32_t base = blockIdx.x * kScanTileN + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = (base + i < n) ? src(base + i) : 0u;
        s += v[i];
    }
    uint32_t total;
    uint32_t run = block_excl_scan(s, &total) + part[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) sink(base + i, run, v[i]);
        run += v[i];
    }
}

template <class Src, class Sink>
static int scan(const LaunchCtx& L, Src src, Sink sink, uint32_t n, uint32_t* part,
                uint32_t* total_out) {
    const uint32_t nb = (n + kScanTileN - 1) / kScanTileN;
    if (nb == 0) return 0;
    k_scan_reduce<<<nb, kScanThreads, 0, L.stream>>>(src, n, part);
    k_scan_partials<<<1, 1024, 0, L.stream>>>(src, part, nb, total_out);
    k_scan_emit<<<nb, kScanThreads, 0, L.stream>>>(src, sink, n, part);
    return 3;
}

// ---------------------------------------------------------------------------------------
// radix sort
// ---------------------------------------------------------------------------------------

__global__ void __launch_bounds__(kRadixThreads) k_radix_hist(const uint32_t* __restrict__ keys,
                                                              int n, int pass, uint32_t* hist,
                                                              const DevState* ds) {
    if (ds->status || (uint32_t)pass >= ds->passes) return;
    __shared__ uint32_t h[kRadixBuckets];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int shift = pass * kRadixBits;
    const int base = blockIdx.x * kRadixTileN;
#pragma unroll 4
    for (int r = 0; r < kRadixItems; ++r) {
        const int i = base + r * kRadixThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & (kRadixBuckets - 1)], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

template <bool kImplicitVals>
__global__ void __launch_bounds__(kRadixThreads) k_radix_scatter(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int n, int pass,
    const uint32_t* __restrict__ offsets, const DevState* ds) {
    if (ds->status || (uint32_t)pass >= ds->passes) return;
    constexpr int kWarps = kRadixThreads / 32;
    constexpr int kRounds = kRadixItems;  // 16 rounds of 32 keys per warp
    __shared__ uint32_t cnt[kWarps][kRadixBuckets];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kWarps * kRadixBuckets; i += kRadixThreads)
        (&cnt[0][0])[i] = 0;
    __syncthreads();
    const int shift = pass * kRadixBits;
    const int wbase = blockIdx.x * kRadixTileN + warp * (kRounds * 32);
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint32_t key[kRounds], val[kRounds], rank[kRounds];
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const int i = wbase + r * 32 + lane;
        const bool ok = i < n;
        key[r] = ok ? keys_in[i] : 0u;
        val[r] = ok ? (kImplicitVals ? (uint32_t)i : vals_in[i]) : 0u;
        // lanes past the end get a digit value that no real key has
        const uint32_t d = ok ? ((key[r] >> shift) & (kRadixBuckets - 1)) : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t before = ok ? cnt[warp][d] : 0u;
        __syncwarp();
        if (ok && (peers & lt_mask) == 0) cnt[warp][d] = before + __popc(peers);
        __syncwarp();
        rank[r] = before + __popc(peers & lt_mask);
    }
    __syncthreads();
    // exclusive scan over warps per digit, plus the block's global offset for the digit
    {
        const int d = threadIdx.x;  // kRadixThreads == kRadixBuckets
        uint32_t run = offsets[d * gridDim.x + blockIdx.x];
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = cnt[w][d];
            cnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const int i = wbase + r * 32 + lane;
        if (i < n) {
            const uint32_t d = (key[r] >> shift) & (kRadixBuckets - 1);
            const uint32_t dst = cnt[warp][d] + rank[r];
            if (dst < (uint32_t)n) {  // always true for a consistent histogram
                keys_out[dst] = key[r];
                vals_out[dst] = val[r];
            }
        }
    }
}

struct HistSrc {
    const uint32_t* hist;
    const DevState* ds;
    int pass;
    __device__ bool active() const { return !ds->status && (uint32_t)pass < ds->passes; }
    __device__ uint32_t operator()(uint32_t i) const { return hist[i]; }
};
struct HistSink {
    uint32_t* hist;
    __device__ void operator()(uint32_t i, uint32_t excl, uint32_t) const { hist[i] = excl; }
};

int launch_radix_sort(const LaunchCtx& L, const Buffers& b, DevState* ds, int n) {
    const int nb = (n + kRadixTileN - 1) / kRadixTileN;
    int launches = 0;
    for (int pass = 0; pass < kMaxPasses; ++pass) {
        const int in = pass & 1, out = in ^ 1;
        k_radix_hist<<<nb, kRadixThreads, 0, L.stream>>>(b.key[in], n, pass, b.hist, ds);
        launches += 2 + scan(L, HistSrc{b.hist, ds, pass}, HistSink{b.hist},
                             (uint32_t)(nb * kRadixBuckets), b.scan_part, nullptr);
        if (pass == 0)
            k_radix_scatter<true><<<nb, kRadixThreads, 0, L.stream>>>(
                b.key[in], nullptr, b.key[out], b.val[out], n, pass, b.hist, ds);
        else
            k_radix_scatter<false><<<nb, kRadixThreads, 0, L.stream>>>(
                b.key[in], b.val[in], b.key[out], b.val[out], n, pass, b.hist, ds);
    }
    return launches;
}

// ---------------------------------------------------------------------------------------
// tile list: a tile starts at every tile_n-th particle of a cell, or (b.columns) of a cell
// column (x, y, *) -- of a column run (b.runs, k_column_runs) in a single-scene precision
// step -- contiguous in cell-sorted order; the non-finite group (key == ncells) is tiled
// the same way.  A column tile may span several cells: the passes walk the union of its
// particles' stencils.
// ---------------------------------------------------------------------------------------

// first cell of the column of cell `key` (the non-finite group is its own column)
__device__ __forceinline__ uint32_t column_base(uint32_t key, uint32_t k, const DevState* ds,
                                                const uint32_t* scene_s,
                                                const SceneInfo* scenes) {
    if (key >= ds->ncells) return key;
    uint32_t base = 0, d2 = (uint32_t)ds->dim[2];
    if (scenes) {
        const SceneInfo& sc = scenes[scene_s[k]];
        base = sc.base;
        d2 = (uint32_t)sc.dim[2];
    }
    return base + (key - base) / d2 * d2;
}

struct TileSrc {
    const uint32_t* key_s;
    const uint32_t* off;
    const DevState* ds;
    const uint32_t* scene_s;  // batched mode (else null)
    const SceneInfo* scenes;
    uint32_t tile_n;        // particles per tile
    int columns;            // 1: tiles along cell columns, else within cells
    const uint2* runs;      // columns: each cell's run (null: the whole column)
    __device__ bool active() const { return !ds->status; }
    __device__ uint32_t operator()(uint32_t k) const {
        const uint32_t key = key_s[k];
        uint32_t st;
        if (!columns || key >= ds->ncells) st = off[key];
        else if (runs) st = runs[key].x;
        else st = off[column_base(key, k, ds, scene_s, scenes)];
        return (k - st) % tile_n == 0 ? 1u : 0u;
    }
};
// Writes the tile starts and counts the occupied cells and the fullest one (the threads
// of a warp call it together: one atomic of each kind per warp and call).
struct TileSink {
    const uint32_t* key_s;
    const uint32_t* off;
    uint32_t* tile_start;
    DevState* ds;
    __device__ void operator()(uint32_t k, uint32_t excl, uint32_t v) const {
        if (v) tile_start[excl] = k;
        const uint32_t c = key_s[k];
        const bool start = c < ds->ncells && off[c] == k;
        const unsigned am = __activemask();
        const unsigned starts = __ballot_sync(am, start);
        if (!starts) return;
        const uint32_t occ = __reduce_max_sync(am, start ? off[c + 1] - k : 0u);
        if ((threadIdx.x & 31) == (uint32_t)(__ffs(am) - 1)) {
            atomicAdd(&ds->occupied, (uint32_t)__popc(starts));
            atomicMax(&ds->max_occ, occ);
        }
    }
};

int launch_tile_scan(const LaunchCtx& L, const Buffers& b, DevState* ds, int n) {
    const bool batched = b.nscenes > 0;
    const TileSrc src{b.key_s, b.off, ds, batched ? b.scene_s : nullptr,
                      batched ? b.scenes : nullptr, (uint32_t)b.tile_n, b.columns,
                      batched ? nullptr : b.runs};
    return scan(L, src, TileSink{b.key_s, b.off, b.tile_start, ds},
         (uint32_t)n, b.scan_part, &ds->n_tiles);
}

}  // namespace sphx
