// Grid build of one step (the GPU form of SpatialHash::build, spatial_hash.cpp:15-25),
// the CFL timestep (SPHEngine::compute_cfl_timestep, sph_engine.cpp:312-333), the FP64
// diagnostics and the host<->device packing kernels.
//
// Cells are the reference's own: floor(x * inv_cell) per axis with
// inv_cell = 1.0f / neighbor_search_radius (spatial_hash.h:30-36, 63-66).  Instead of a
// hash map of index vectors the occupied-cell box is laid out as a dense grid (folded
// per axis when the box is huge, see k_grid_setup) with a linear key
// ((cx * dy + cy) * dz + cz), the keys are radix-sorted stably from insertion order, and
// off[c] holds the first sorted position of cell c.  z is the fastest axis, so
// the three cells (cx+dx, cy+dy, cz-1..cz+1) of one stencil row are one contiguous range
// of the sorted arrays.  Particles with a NaN/inf coordinate get key == ncells: they sort
// last and are never anyone's neighbour (every distance test with them fails in the
// reference too).
#include "sphx_internal.cuh"

namespace sphx {

static inline int grid_blocks(const LaunchCtx& L, int n, int threads, int per_sm = 4) {
    const int need = (n + threads - 1) / threads;
    const int cap = L.num_sms * per_sm;
    return need < 1 ? 1 : (need < cap ? need : cap);
}

__global__ void k_begin_step(DevState* ds, int reset_bbox) {
    if (threadIdx.x != 0) return;
    ds->status = 0;
    if (reset_bbox) {
        for (int a = 0; a < 3; ++a) {
            ds->cmin[a] = 0x7fffffff;
            ds->cmax[a] = -0x7fffffff - 1;
        }
    }
    ds->nonfinite = 0;
    ds->vmax_bits = 0;
    ds->vmax64 = 0ull;
    ds->occupied = 0;
    ds->max_occ = 0;
    ds->n_tiles = 0;
    ds->work[0] = ds->work[1] = 0;
    ds->spread_work[0] = ds->spread_work[1] = 0;
    ds->n_spread = 0;
}

int launch_begin_step(const LaunchCtx& L, DevState* ds, int reset_bbox) {
    k_begin_step<<<1, 32, 0, L.stream>>>(ds, reset_bbox);
    return 1;
}

// ---- CFL ------------------------------------------------------------------------------

// max |v_i| over the particles, NaN lengths ignored: std::max(m, v) keeps m when v is NaN
// (sph_engine.cpp:316-322).  Non-negative floats order like their bit patterns.
__global__ void k_vmax(const float4* __restrict__ vel4, int n, DevState* ds) {
    uint32_t m = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 v = vel4[i];
        const float len = xsqrt(xdot3(v.x, v.y, v.z));
        if (!isnan(len)) m = max(m, __float_as_uint(len));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(&ds->vmax_bits, m);
}

// dt = min({dt_cfl, dt_force, timestep}) with std::min's first-smallest rule; then
// current_time_ += dt.
__global__ void k_set_dt(StepConst c, DevState* ds, float host_dt) {
    if (threadIdx.x != 0) return;
    float dt = host_dt;  // a NaN dt is used as given, like SPHEngine::step (cpp:99-101)
    if (host_dt <= 0.0f) {
        const float vmax = __uint_as_float(ds->vmax_bits);
        const float dt_cfl = xdiv(xmul(c.cfl, c.h), xadd(vmax, 1e-6f));
        const float alen = xsqrt(xdot3(ds->a0[0], ds->a0[1], ds->a0[2]));
        const float dt_force = xmul(c.cfl, xsqrt(xdiv(c.h, xadd(alen, 1e-6f))));
        dt = dt_cfl;
        if (dt_force < dt) dt = dt_force;
        if (c.timestep < dt) dt = c.timestep;
    }
    ds->dt = dt;
    ds->time = xadd(ds->time, dt);
}

// Precision mode: max |v| in FP64 (NaN ignored), then the same rule in FP64; time in FP64.
__global__ void k_vmax64(const float4* __restrict__ vel4, int n, DevState* ds) {
    unsigned long long m = 0ull;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 v = vel4[i];
        const double len = sqrt((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
        if (!isnan(len)) m = max(m, (unsigned long long)__double_as_longlong(len));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(&ds->vmax64, m);
}

__global__ void k_set_dt64(StepConst c, DevState* ds, float host_dt) {
    if (threadIdx.x != 0) return;
    double dt = host_dt;
    if (host_dt <= 0.0f) {
        const double vmax = __longlong_as_double((long long)ds->vmax64);
        const double cfl = c.cfl, h = c.h;
        const double dt_cfl = cfl * h / (vmax + 1e-6);
        const double a0 = sqrt((double)ds->a0[0] * ds->a0[0] + (double)ds->a0[1] * ds->a0[1] +
                               (double)ds->a0[2] * ds->a0[2]);
        const double dt_force = cfl * sqrt(h / (a0 + 1e-6));
        dt = dt_cfl;
        if (dt_force < dt) dt = dt_force;
        if ((double)c.timestep < dt) dt = c.timestep;
    }
    ds->dt64 = dt;
    ds->time64 += dt;
    ds->dt = (float)dt;
    ds->time = (float)ds->time64;
}

int launch_cfl(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds,
               float host_dt) {
    int launches = 1;
    if (host_dt <= 0.0f) {
        if (c.precise)
            k_vmax64<<<grid_blocks(L, c.n, 256), 256, 0, L.stream>>>(b.vel4, c.n, ds);
        else
            k_vmax<<<grid_blocks(L, c.n, 256), 256, 0, L.stream>>>(b.vel4, c.n, ds);
        ++launches;
    }
    if (c.precise) k_set_dt64<<<1, 32, 0, L.stream>>>(c, ds, host_dt);
    else k_set_dt<<<1, 32, 0, L.stream>>>(c, ds, host_dt);
    return launches;
}

// ---- grid -----------------------------------------------------------------------------

__global__ void k_bbox(const float4* __restrict__ pos4, int n, float inv_cell, DevState* ds) {
    int mn[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff};
    int mx[3] = {-0x7fffffff - 1, -0x7fffffff - 1, -0x7fffffff - 1};
    uint32_t bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = pos4[i];
        if (!finite3(p.x, p.y, p.z)) {
            ++bad;
            continue;
        }
        const int c[3] = {cell_coord(p.x, inv_cell), cell_coord(p.y, inv_cell),
                          cell_coord(p.z, inv_cell)};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn[a] = min(mn[a], c[a]);
            mx[a] = max(mx[a], c[a]);
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (mn[a] != 0x7fffffff) atomicMin(&ds->cmin[a], mn[a]);
            if (mx[a] != -0x7fffffff - 1) atomicMax(&ds->cmax[a], mx[a]);
        }
        if (bad) atomicAdd(&ds->nonfinite, bad);
    }
}

// Grid extent.  The occupied-cell box is laid out densely when it has at most max_cells
// cells.  Otherwise (particles spread over a huge box) every axis longer than F =
// floor(cbrt(max_cells)) >= 256 cells is folded: its cell index is taken modulo F.  Cells
// that fold onto each other are at least F - 2 cells apart, so a candidate from a folded
// neighbour fails the distance test; sets and visiting order are unchanged, only the
// number of candidates grows.
// Precision mode: the cells are stored; w != 0 marks a particle with no finite position.
__global__ void k_bbox_cells(const int4* __restrict__ cell4, int n, DevState* ds) {
    int mn[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff};
    int mx[3] = {-0x7fffffff - 1, -0x7fffffff - 1, -0x7fffffff - 1};
    uint32_t bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 c = cell4[i];
        if (c.w) {
            ++bad;
            continue;
        }
        mn[0] = min(mn[0], c.x); mn[1] = min(mn[1], c.y); mn[2] = min(mn[2], c.z);
        mx[0] = max(mx[0], c.x); mx[1] = max(mx[1], c.y); mx[2] = max(mx[2], c.z);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (mn[a] != 0x7fffffff) atomicMin(&ds->cmin[a], mn[a]);
            if (mx[a] != -0x7fffffff - 1) atomicMax(&ds->cmax[a], mx[a]);
        }
        if (bad) atomicAdd(&ds->nonfinite, bad);
    }
}

__global__ void k_keys_cells(const int4* __restrict__ cell4, int n, const DevState* ds,
                             uint32_t* __restrict__ keys) {
    if (ds->status) return;
    const int cx0 = ds->cmin[0], cy0 = ds->cmin[1], cz0 = ds->cmin[2];
    const uint32_t dx = ds->dim[0], dy = ds->dim[1], dz = ds->dim[2], nc = ds->ncells;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 c = cell4[i];
        uint32_t key = nc;
        if (!c.w) {
            const uint32_t x = (uint32_t)(c.x - cx0) % dx;
            const uint32_t y = (uint32_t)(c.y - cy0) % dy;
            const uint32_t z = (uint32_t)(c.z - cz0) % dz;
            key = (x * dy + y) * dz + z;
        }
        keys[i] = key;
    }
}

__global__ void k_grid_setup(int n, uint32_t max_cells, DevState* ds) {
    if (threadIdx.x != 0) return;
    if ((int)ds->nonfinite >= n) {  // no finite particle: a one-cell grid, all keys sentinel
        for (int a = 0; a < 3; ++a) {
            ds->cmin[a] = 0;
            ds->cmax[a] = 0;
        }
    }
    long long d[3];
    unsigned long long cells = 1;
    bool fits = true;
    for (int a = 0; a < 3; ++a) {
        d[a] = (long long)ds->cmax[a] - (long long)ds->cmin[a] + 1;
        if (d[a] > (long long)max_cells) fits = false;
        else if ((cells *= (unsigned long long)d[a]) > (unsigned long long)max_cells) fits = false;
    }
    long long fold = 1;
    if (!fits) {
        while ((fold + 1) * (fold + 1) * (fold + 1) <= (long long)max_cells) ++fold;
    }
    cells = 1;
    for (int a = 0; a < 3; ++a) {
        const bool w = !fits && d[a] > fold;
        ds->wrap[a] = w ? 1 : 0;
        ds->dim[a] = (int)(w ? fold : d[a]);
        cells *= (unsigned long long)ds->dim[a];
    }
    ds->ncells = (uint32_t)cells;
    const int bits = 32 - __clz(ds->ncells);  // key range is [0, ncells]
    ds->passes = (uint32_t)((bits + kRadixBits - 1) / kRadixBits);
}

__global__ void k_keys(const float4* __restrict__ pos4, int n, float inv_cell,
                       const DevState* ds, uint32_t* __restrict__ keys) {
    if (ds->status) return;
    const int cx0 = ds->cmin[0], cy0 = ds->cmin[1], cz0 = ds->cmin[2];
    const uint32_t dx = ds->dim[0], dy = ds->dim[1], dz = ds->dim[2], nc = ds->ncells;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = pos4[i];
        uint32_t key = nc;
        if (finite3(p.x, p.y, p.z)) {
            // relative cell index (< 2^31), folded on the axes that wrap
            const uint32_t x = (uint32_t)(cell_coord(p.x, inv_cell) - cx0) % dx;
            const uint32_t y = (uint32_t)(cell_coord(p.y, inv_cell) - cy0) % dy;
            const uint32_t z = (uint32_t)(cell_coord(p.z, inv_cell) - cz0) % dz;
            key = (x * dy + y) * dz + z;
        }
        keys[i] = key;
    }
}

// Gathers the state into cell-sorted order and keeps the sorted keys and permutation.
__global__ void k_reorder(const Buffers b, int n, DevState* ds) {
    if (ds->status) return;
    const int sel = ds->passes & 1;
    const uint32_t* __restrict__ ks = b.key[sel];
    const uint32_t* __restrict__ vs = b.val[sel];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        uint32_t id = vs[k];
        if (id >= (uint32_t)n) {  // never for a valid permutation: record, do not fault
            atomicExch(&ds->status, SPHX_ERR_CUDA);
            id = 0;
        }
        b.key_s[k] = ks[k];
        b.id_s[k] = id;
        b.pos4_s[k] = b.pos4[id];
        b.vel4_s[k] = b.vel4[id];
        if (b.cell4) b.cell4_s[k] = b.cell4[id];
        if (b.scene_s) b.scene_s[k] = b.scene_of[id];
    }
}

// off[c] = first sorted position whose key is >= c, for c in [0, ncells + 1];
// off[ncells] is the number of finite particles and off[ncells + 1] == n.
__global__ void k_offsets(const uint32_t* __restrict__ key_s, int n, const DevState* ds,
                          uint32_t* __restrict__ off) {
    if (ds->status) return;
    const uint32_t nc = ds->ncells;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= n; k += gridDim.x * blockDim.x) {
        const uint32_t lo = (k == 0) ? 0u : key_s[k - 1] + 1u;
        const uint32_t hi = (k == n) ? nc + 1u : key_s[k];
        for (uint32_t c = lo; c <= hi; ++c) off[c] = (uint32_t)k;
    }
}

// Precision-mode step (b.columns): each cell's particles put in z order (the in-cell
// offset quantised to 16 levels of cs/16, stable within a level), so that a run of
// consecutive particles of a cell column -- a tile -- is a compact slab across the cells.
// The order within a cell is free in this mode (its sums are judged against FP64, not
// against the reference's order).  One warp per cell; cells of more than kZOrderMax
// particles (collapsed states, whose tiles are dense anyway) keep their order.
constexpr int kZOrderMax = 128;
__global__ void __launch_bounds__(256) k_cell_zorder(const Buffers b, const DevState* ds,
                                                     float levels_per_unit) {
    if (ds->status) return;
    constexpr int kPer = kZOrderMax / 32;
    const uint32_t nc = ds->ncells;
    const int lane = threadIdx.x & 31;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < nc; c += nwarps) {
        const uint32_t a = b.off[c], cnt = b.off[c + 1] - a;
        if (cnt < 2 || cnt > (uint32_t)kZOrderMax) continue;
        float4 p[kPer], v[kPer];
        int4 ce[kPer];
        uint32_t id[kPer];
        int lev[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t q = (uint32_t)(j * 32 + lane);
            lev[j] = 16;  // no element
            if (q < cnt) {
                p[j] = b.pos4_s[a + q];
                v[j] = b.vel4_s[a + q];
                ce[j] = b.cell4_s[a + q];
                id[j] = b.id_s[a + q];
                lev[j] = min(15, max(0, (int)(p[j].z * levels_per_unit)));
            }
        }
        // stable counting sort over the 16 levels: an element's place is the number of
        // elements of lower levels plus those of its level before it
        int dest[kPer];
        uint32_t below = 0;
#pragma unroll 1
        for (int L = 0; L < 16; ++L) {
            uint32_t seen = below;
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const uint32_t m = __ballot_sync(0xffffffffu, lev[j] == L);
                if (lev[j] == L) dest[j] = (int)(seen + __popc(m & lt));
                seen += __popc(m);
            }
            below = seen;
        }
        __syncwarp();  // every lane holds its elements: the cell's range can be rewritten
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            if (lev[j] == 16) continue;
            const uint32_t k = a + (uint32_t)dest[j];
            b.pos4_s[k] = p[j];
            b.vel4_s[k] = v[j];
            b.cell4_s[k] = ce[j];
            b.id_s[k] = id[j];
        }
    }
}

int launch_build_grid(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                      DevState* ds) {
    const int n = c.n;
    const int gb = grid_blocks(L, n, 256);
    if (c.precise) k_bbox_cells<<<gb, 256, 0, L.stream>>>(b.cell4, n, ds);
    else k_bbox<<<gb, 256, 0, L.stream>>>(b.pos4, n, c.inv_cell, ds);
    k_grid_setup<<<1, 32, 0, L.stream>>>(n, c.max_cells, ds);
    if (c.precise) k_keys_cells<<<gb, 256, 0, L.stream>>>(b.cell4, n, ds, b.key[0]);
    else k_keys<<<gb, 256, 0, L.stream>>>(b.pos4, n, c.inv_cell, ds, b.key[0]);
    return 3 + launch_grid_sort(L, b, ds, n, c.cs);
}

static int launch_cell_zorder(const LaunchCtx& L, const Buffers& b, DevState* ds, int n,
                              float cs) {
    if (!b.columns || !b.cell4_s) return 0;
    // one warp per cell: blocks of 8 warps, enough of them for the occupied cells
    k_cell_zorder<<<grid_blocks(L, n, 256, 8), 256, 0, L.stream>>>(b, ds, 16.0f / cs);
    return 1;
}

// Precision-mode step, single scene: the runs of each cell column.  Cell z of a column
// starts a run when it is the column's first cell, or when z is a multiple of A =
// kRunAlign and the W = kRunWindow cells below z hold fewer than tile_n particles.  A tile
// whose first particle lies in cell z_a then ends by cell z_a + W + A - 1: the first
// multiple of A at or above z_a + W + 1, z_m, is at most z_a + W + A, and were the tile
// to reach cell z_m, cells z_m - W .. z_m - 1 would lie wholly in it, fewer than tile_n
// particles, so z_m starts a run.  Dense stretches stay one run; a sparse one is cut every
// A cells (a window of one cell and A = 1 would cut it at every cell).  runs[c] = the
// sorted positions where c's run starts and ends (the off of its first cell and of the
// next run's).  One warp per column: a max-scan over its cells 32 at a time upward for
// the starts, a min-scan downward for the ends.
__device__ __forceinline__ bool run_starts_at(const uint32_t* __restrict__ off, uint32_t cb,
                                              uint32_t z, uint32_t tile_n) {
    return z == 0 || (z > (uint32_t)kRunWindow && z % kRunAlign == 0 &&
                      off[cb + z] - off[cb + z - kRunWindow] < tile_n);
}
__global__ void __launch_bounds__(256) k_column_runs(const uint32_t* __restrict__ off,
                                                     const DevState* ds, uint32_t tile_n,
                                                     uint2* __restrict__ runs) {
    if (ds->status) return;
    const int d2 = ds->dim[2];
    if (d2 <= 0) return;
    const uint32_t ncol = ds->ncells / (uint32_t)d2;
    const int lane = threadIdx.x & 31;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t col = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); col < ncol;
         col += nwarps) {
        const uint32_t cb = col * (uint32_t)d2;
        int carry = 0;  // first cell of the run (column-relative)
        for (int z0 = 0; z0 < d2; z0 += 32) {
            const int z = z0 + lane;
            int v = (z < d2 && run_starts_at(off, cb, (uint32_t)z, tile_n)) ? z : carry;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v = max(v, u);
            }
            if (z < d2) runs[cb + z].x = off[cb + v];
            carry = __shfl_sync(0xffffffffu, v, 31);
        }
        carry = d2;  // first cell of the next run (d2: the column's end)
        for (int z0 = (d2 - 1) & ~31; z0 >= 0; z0 -= 32) {
            const int z = z0 + lane;
            int v = (z + 1 < d2 && run_starts_at(off, cb, (uint32_t)(z + 1), tile_n)) ? z + 1
                                                                                     : carry;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_down_sync(0xffffffffu, v, o);
                if (lane + o < 32) v = min(v, u);
            }
            if (z < d2) runs[cb + z].y = off[cb + v];
            carry = __shfl_sync(0xffffffffu, v, 0);
        }
    }
}

static int launch_column_runs(const LaunchCtx& L, const Buffers& b, DevState* ds, int n) {
    if (!b.columns || !b.runs || b.nscenes) return 0;
    k_column_runs<<<grid_blocks(L, n, 256, 2), 256, 0, L.stream>>>(b.off, ds,
                                                                   (uint32_t)b.tile_n, b.runs);
    return 1;
}

// Shared tail of the grid build: stable sort of the keys, gather into cell-sorted order,
// cell offsets, (b.columns) z order within the cells and column runs, tile list.
int launch_grid_sort(const LaunchCtx& L, const Buffers& b, DevState* ds, int n, float cs) {
    const int r = launch_radix_sort(L, b, ds, n);
    k_reorder<<<grid_blocks(L, n, 256, 8), 256, 0, L.stream>>>(b, n, ds);
    k_offsets<<<grid_blocks(L, n + 1, 256, 8), 256, 0, L.stream>>>(b.key_s, n, ds, b.off);
    const int z = launch_cell_zorder(L, b, ds, n, cs) + launch_column_runs(L, b, ds, n);
    return 2 + r + z + launch_tile_scan(L, b, ds, n);
}


// ---- FP64 diagnostics of the state after a step -----------------------------------------
// sums: mass, momentum x/y/z, kinetic energy, potential energy (-m g y), density.
// Fixed partition and fixed-order final sum: bit-reproducible run to run.
__global__ void __launch_bounds__(kDiagThreads) k_diag_partial(
    const float4* __restrict__ pos4, const float4* __restrict__ vel4,
    const float4* __restrict__ aux4_s, const int4* __restrict__ cell4, double cs, int n,
    float grav, double* __restrict__ part) {
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    const int per = (n + gridDim.x - 1) / gridDim.x;
    const int i0 = blockIdx.x * per, i1 = min(n, i0 + per);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const float4 p = pos4[i];
        const float4 v = vel4[i];
        const double m = p.w;
        s[0] += m;
        s[1] += m * v.x;
        s[2] += m * v.y;
        s[3] += m * v.z;
        s[4] += 0.5 * m * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
        const double y = cell4 ? (double)cell4[i].y * cs + (double)p.y : (double)p.y;
        s[5] += -m * (double)grav * y;
        if (aux4_s) s[6] += (double)aux4_s[i].x;  // null: no density pass on this set yet
    }
    __shared__ double red[kDiagThreads / 32][7];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        double v = s[k];
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 7) {
        double v = 0;
        for (int w = 0; w < kDiagThreads / 32; ++w) v += red[w][threadIdx.x];
        part[blockIdx.x * kDiagSums + threadIdx.x] = v;
    }
}

// One warp per sum: lane l adds partials l, l + 32, ... in order, then a fixed shuffle tree
// (the order never changes, so the sums are reproducible bit for bit).
__global__ void k_diag_final(const double* __restrict__ part, int nb, DevState* ds) {
    const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= 7) return;
    double v = 0;
    for (int b = lane; b < nb; b += 32) v += part[b * kDiagSums + k];
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) ds->sums[k] = v;
}

int launch_diag(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds) {
    k_diag_partial<<<b.diag_blocks, kDiagThreads, 0, L.stream>>>(
        b.pos4, b.vel4, b.aux4_s, c.precise ? b.cell4 : nullptr, c.cs_d, c.n, c.grav, b.diag_part);
    k_diag_final<<<1, 7 * 32, 0, L.stream>>>(b.diag_part, b.diag_blocks, ds);
    return 2;
}

// ---- packing ----------------------------------------------------------------------------

__global__ void k_pack(int n, const float* __restrict__ pos3, const float* __restrict__ vel3,
                       const float* __restrict__ mass, float4* __restrict__ pos4,
                       float4* __restrict__ vel4) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        pos4[i] = make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], mass[i]);
        vel4[i] = vel3 ? make_float4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.0f)
                       : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

void launch_pack(const LaunchCtx& L, int n, const float* pos3, const float* vel3,
                 const float* mass, float4* pos4, float4* vel4) {
    k_pack<<<grid_blocks(L, n, 256, 8), 256, 0, L.stream>>>(n, pos3, vel3, mass, pos4, vel4);
}

__global__ void k_unpack_state(int n, const float4* __restrict__ pos4,
                               const float4* __restrict__ vel4, float* __restrict__ pos3,
                               float* __restrict__ vel3) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (pos3) {
            const float4 p = pos4[i];
            pos3[3 * i] = p.x;
            pos3[3 * i + 1] = p.y;
            pos3[3 * i + 2] = p.z;
        }
        if (vel3) {
            const float4 v = vel4[i];
            vel3[3 * i] = v.x;
            vel3[3 * i + 1] = v.y;
            vel3[3 * i + 2] = v.z;
        }
    }
}

void launch_unpack_state(const LaunchCtx& L, int n, const float4* pos4, const float4* vel4,
                         float* pos3, float* vel3) {
    k_unpack_state<<<grid_blocks(L, n, 256, 8), 256, 0, L.stream>>>(n, pos4, vel4, pos3, vel3);
}

__global__ void k_unpack_sorted(int n, const uint32_t* __restrict__ id_s,
                                const float4* __restrict__ aux4_s,
                                const float4* __restrict__ acc4_s, float* __restrict__ rho,
                                float* __restrict__ pressure, float* __restrict__ acc3) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t id = id_s[k];
        const float4 a = aux4_s[k];
        if (rho) rho[id] = a.x;
        if (pressure) pressure[id] = a.y;
        if (acc3) {
            const float4 g = acc4_s[k];
            acc3[3 * id] = g.x;
            acc3[3 * id + 1] = g.y;
            acc3[3 * id + 2] = g.z;
        }
    }
}

void launch_unpack_sorted(const LaunchCtx& L, int n, const uint32_t* id_s, const float4* aux4_s,
                          const float4* acc4_s, float* rho, float* pressure, float* acc3) {
    k_unpack_sorted<<<grid_blocks(L, n, 256, 8), 256, 0, L.stream>>>(n, id_s, aux4_s, acc4_s,
                                                                     rho, pressure, acc3);
}

}  // namespace sphx

namespace sphx {

// Absolute position (double) -> integer cell + offset in [0, cs); non-finite -> w = 1.
__device__ __forceinline__ void to_cell(double X, double cs, int fp16, int& c, float& o) {
    double f = floor(X / cs);
    f = fmin(fmax(f, -(double)kCellClamp), (double)(kCellClamp - 1));
    c = (int)f;
    o = (float)(X - (double)c * cs);
    if (fp16) o = round_half(o);
    const float csf = (float)cs;
    if (o >= csf) {  // rounding reached the next cell
        o = 0.0f;
        c += 1;
    } else if (o < 0.0f) {
        o = 0.0f;
    }
}

__global__ void k_pack_cells(StepConst c, int n, const float* __restrict__ pos3f,
                             const double* __restrict__ pos3d, const float* __restrict__ vel3,
                             const float* __restrict__ mass, int4* __restrict__ cell4,
                             float4* __restrict__ pos4, float4* __restrict__ vel4) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double X[3];
        for (int a = 0; a < 3; ++a) X[a] = pos3d ? pos3d[3 * i + a] : (double)pos3f[3 * i + a];
        int4 cc = make_int4(0, 0, 0, 0);
        float o[3] = {0.0f, 0.0f, 0.0f};
        if (isfinite(X[0]) && isfinite(X[1]) && isfinite(X[2])) {
            to_cell(X[0], c.cs_d, c.fp16, cc.x, o[0]);
            to_cell(X[1], c.cs_d, c.fp16, cc.y, o[1]);
            to_cell(X[2], c.cs_d, c.fp16, cc.z, o[2]);
        } else {
            cc.w = 1;
            for (int a = 0; a < 3; ++a) o[a] = (float)X[a];
        }
        cell4[i] = cc;
        pos4[i] = make_float4(o[0], o[1], o[2], mass[i]);
        vel4[i] = vel3 ? make_float4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.0f)
                       : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

void launch_pack_cells(const LaunchCtx& L, const StepConst& c, int n, const float* pos3f,
                       const double* pos3d, const float* vel3, const float* mass, int4* cell4,
                       float4* pos4, float4* vel4) {
    k_pack_cells<<<grid_blocks(L, n, 256, 8), 256, 0, L.stream>>>(c, n, pos3f, pos3d, vel3, mass,
                                                                  cell4, pos4, vel4);
}

__global__ void k_unpack_cells(StepConst c, int n, const int4* __restrict__ cell4,
                               const float4* __restrict__ pos4, float* __restrict__ pos3f,
                               double* __restrict__ pos3d) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 cc = cell4[i];
        const float4 p = pos4[i];
        double X[3];
        if (cc.w) {
            X[0] = p.x; X[1] = p.y; X[2] = p.z;
        } else {
            X[0] = (double)cc.x * c.cs_d + (double)p.x;
            X[1] = (double)cc.y * c.cs_d + (double)p.y;
            X[2] = (double)cc.z * c.cs_d + (double)p.z;
        }
        for (int a = 0; a < 3; ++a) {
            if (pos3d) pos3d[3 * i + a] = X[a];
            if (pos3f) pos3f[3 * i + a] = (float)X[a];
        }
    }
}

void launch_unpack_cells(const LaunchCtx& L, const StepConst& c, int n, const int4* cell4,
                         const float4* pos4, float* pos3f, double* pos3d) {
    k_unpack_cells<<<grid_blocks(L, n, 256, 8), 256, 0, L.stream>>>(c, n, cell4, pos4, pos3f, pos3d);
}

}  // namespace sphx
