// Batched scenes: many independent SPH scenes advanced by one step's launches.
//
// Every scene keeps the reference's semantics on its own (its own parameters, walls,
// CFL timestep from its own particles and its own first particle's acceleration, its own
// current time).  The scenes share one cell grid in which each scene owns a dense block
// of cells starting at `base` (a scan over the scenes' cell counts); the key of a particle
// is base + its linear cell index inside the scene's block, so one stable radix sort
// orders all scenes by (scene, cell, insertion index), and the density / force passes take
// tiles of every scene from one work counter.  No particle of one scene ever meets a
// particle of another: the rows of a tile never leave its scene's block.  Each scene's
// results are therefore bit-identical to stepping that scene alone.
#include "sphx_internal.cuh"

namespace sphx {

static inline int blocks_for(const LaunchCtx& L, int n, int threads, int per_sm = 4) {
    const int need = (n + threads - 1) / threads;
    const int cap = L.num_sms * per_sm;
    return need < 1 ? 1 : (need < cap ? need : cap);
}

__global__ void k_batch_begin(SceneInfo* scenes, int nscenes, DevState* ds) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) {
        ds->status = 0;
        ds->nonfinite = 0;
        ds->occupied = 0;
        ds->max_occ = 0;
        ds->n_tiles = 0;
        ds->work[0] = 0;
        ds->work[1] = 0;
    }
    if (s >= nscenes) return;
    SceneInfo& sc = scenes[s];
    for (int a = 0; a < 3; ++a) {
        sc.cmin[a] = 0x7fffffff;
        sc.cmax[a] = -0x7fffffff - 1;
    }
    sc.nonfinite = 0;
    sc.vmax_bits = 0;
}

int launch_batch_begin(const LaunchCtx& L, const Buffers& b, DevState* ds) {
    k_batch_begin<<<(b.nscenes + 255) / 256, 256, 0, L.stream>>>(b.scenes, b.nscenes, ds);
    return 1;
}

// ---- CFL per scene --------------------------------------------------------------------

__global__ void k_batch_vmax(const float4* __restrict__ vel4, const uint32_t* __restrict__ scene_of,
                             int n, SceneInfo* scenes) {
    const int lane = threadIdx.x & 31;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n;
         base += gridDim.x * blockDim.x) {
        const int i = base + lane;
        uint32_t m = 0, s = 0xffffffffu;
        if (i < n) {
            const float4 v = vel4[i];
            const float len = xsqrt(xdot3(v.x, v.y, v.z));
            if (!isnan(len)) m = __float_as_uint(len);  // NaN ignored like std::max
            s = scene_of[i];
        }
        // lanes of one scene combine, then one atomic per scene per warp
        const uint32_t peers = __match_any_sync(0xffffffffu, s);
        uint32_t mm = m;
        for (uint32_t rest = peers; rest; rest &= rest - 1) {
            const int src = __ffs(rest) - 1;
            mm = max(mm, __shfl_sync(peers, m, src));
        }
        if (s != 0xffffffffu && lane == __ffs(peers) - 1 && mm) atomicMax(&scenes[s].vmax_bits, mm);
    }
}

// Per scene: dt = min({dt_cfl, dt_force, timestep}) (SPHEngine::compute_cfl_timestep,
// sph_engine.cpp:312-333) or the host dt; current_time_ += dt.
__global__ void k_batch_set_dt(SceneInfo* scenes, int nscenes, float host_dt) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nscenes) return;
    SceneInfo& sc = scenes[s];
    const StepConst& c = sc.c;
    float dt = host_dt;
    if (host_dt <= 0.0f) {
        const float vmax = __uint_as_float(sc.vmax_bits);
        const float dt_cfl = xdiv(xmul(c.cfl, c.h), xadd(vmax, 1e-6f));
        const float alen = xsqrt(xdot3(sc.a0[0], sc.a0[1], sc.a0[2]));
        const float dt_force = xmul(c.cfl, xsqrt(xdiv(c.h, xadd(alen, 1e-6f))));
        dt = dt_cfl;
        if (dt_force < dt) dt = dt_force;
        if (c.timestep < dt) dt = c.timestep;
    }
    if (sc.count == 0) return;  // SPHEngine::step is a no-op on an empty scene
    sc.dt = dt;
    sc.time = xadd(sc.time, dt);
}

int launch_batch_cfl(const LaunchCtx& L, const Buffers& b, DevState* ds, int n, float host_dt) {
    int k = 1;
    if (host_dt <= 0.0f) {
        k_batch_vmax<<<blocks_for(L, n, 256), 256, 0, L.stream>>>(b.vel4, b.scene_of, n, b.scenes);
        ++k;
    }
    k_batch_set_dt<<<(b.nscenes + 255) / 256, 256, 0, L.stream>>>(b.scenes, b.nscenes, host_dt);
    return k;
}

// ---- grid ------------------------------------------------------------------------------

__global__ void k_batch_bbox(const float4* __restrict__ pos4, const uint32_t* __restrict__ scene_of,
                             int n, SceneInfo* scenes) {
    const int lane = threadIdx.x & 31;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n;
         base += gridDim.x * blockDim.x) {
        const int i = base + lane;
        uint32_t s = 0xffffffffu;
        bool fin = false;
        int c[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff};
        int d[3] = {-0x7fffffff - 1, -0x7fffffff - 1, -0x7fffffff - 1};
        if (i < n) {
            s = scene_of[i];
            const float4 p = pos4[i];
            fin = finite3(p.x, p.y, p.z);
            if (fin) {
                const float ic = scenes[s].c.inv_cell;
                c[0] = d[0] = cell_coord(p.x, ic);
                c[1] = d[1] = cell_coord(p.y, ic);
                c[2] = d[2] = cell_coord(p.z, ic);
            }
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, s);
        const uint32_t bad = __popc(__ballot_sync(0xffffffffu, i < n && !fin) & peers);
        int mn[3] = {c[0], c[1], c[2]}, mx[3] = {d[0], d[1], d[2]};
        for (uint32_t rest = peers; rest; rest &= rest - 1) {
            const int src = __ffs(rest) - 1;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                mn[a] = min(mn[a], __shfl_sync(peers, c[a], src));
                mx[a] = max(mx[a], __shfl_sync(peers, d[a], src));
            }
        }
        if (s != 0xffffffffu && lane == __ffs(peers) - 1) {
            SceneInfo& sc = scenes[s];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (mn[a] != 0x7fffffff) atomicMin(&sc.cmin[a], mn[a]);
                if (mx[a] != -0x7fffffff - 1) atomicMax(&sc.cmax[a], mx[a]);
            }
            if (bad) atomicAdd(&sc.nonfinite, bad);
        }
    }
}

// One thread lays the scenes' blocks end to end (scenes are few: a serial scan is cheap).
__global__ void k_batch_grid_setup(SceneInfo* scenes, int nscenes, uint32_t max_cells,
                                   DevState* ds) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long total = 0;
    for (int s = 0; s < nscenes; ++s) {
        SceneInfo& sc = scenes[s];
        if (sc.nonfinite >= sc.count) {  // no finite particle: one cell, all keys sentinel
            for (int a = 0; a < 3; ++a) sc.cmin[a] = sc.cmax[a] = 0;
        }
        unsigned long long cells = 1;
        for (int a = 0; a < 3; ++a) {
            const long long d = (long long)sc.cmax[a] - (long long)sc.cmin[a] + 1;
            sc.dim[a] = (int)(d < 0x7fffffff ? d : 0x7fffffff);
            cells *= (unsigned long long)(d < (long long)max_cells ? d : (long long)max_cells + 1);
            if (cells > (unsigned long long)max_cells) cells = (unsigned long long)max_cells + 1;
        }
        sc.base = (uint32_t)(total < 0xffffffffull ? total : 0xffffffffull);
        sc.ncells = (uint32_t)(cells < 0xffffffffull ? cells : 0xffffffffull);
        total += cells;
        if (total > (unsigned long long)max_cells) break;
    }
    if (total > (unsigned long long)max_cells) {  // each scene's box must fit unfolded
        ds->status = SPHX_ERR_DOMAIN;
        ds->ncells = 0;
        ds->passes = 0;
        return;
    }
    ds->ncells = (uint32_t)total;
    for (int a = 0; a < 3; ++a) {
        ds->dim[a] = 1;
        ds->wrap[a] = 0;
    }
    const int bits = 32 - __clz(ds->ncells);
    ds->passes = (uint32_t)((bits + kRadixBits - 1) / kRadixBits);
}

__global__ void k_batch_keys(const float4* __restrict__ pos4, const uint32_t* __restrict__ scene_of,
                             int n, const SceneInfo* __restrict__ scenes, const DevState* ds,
                             uint32_t* __restrict__ keys) {
    if (ds->status) return;
    const uint32_t sentinel = ds->ncells;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const SceneInfo& sc = scenes[scene_of[i]];
        const float4 p = pos4[i];
        uint32_t key = sentinel;
        if (finite3(p.x, p.y, p.z)) {
            const float ic = sc.c.inv_cell;
            const uint32_t x = (uint32_t)(cell_coord(p.x, ic) - sc.cmin[0]);
            const uint32_t y = (uint32_t)(cell_coord(p.y, ic) - sc.cmin[1]);
            const uint32_t z = (uint32_t)(cell_coord(p.z, ic) - sc.cmin[2]);
            key = sc.base + (x * (uint32_t)sc.dim[1] + y) * (uint32_t)sc.dim[2] + z;
        }
        keys[i] = key;
    }
}

int launch_batch_grid(const LaunchCtx& L, const Buffers& b, DevState* ds, int n,
                      uint32_t max_cells) {
    const int gb = blocks_for(L, n, 256);
    k_batch_bbox<<<gb, 256, 0, L.stream>>>(b.pos4, b.scene_of, n, b.scenes);
    k_batch_grid_setup<<<1, 32, 0, L.stream>>>(b.scenes, b.nscenes, max_cells, ds);
    k_batch_keys<<<gb, 256, 0, L.stream>>>(b.pos4, b.scene_of, n, b.scenes, ds, b.key[0]);
    return 3 + launch_grid_sort(L, b, ds, n, 0.0f);
}

// ---- FP64 diagnostics per scene (one block per scene, fixed order) ----------------------
__global__ void __launch_bounds__(kDiagThreads) k_batch_diag(
    const float4* __restrict__ pos4, const float4* __restrict__ vel4,
    const float4* __restrict__ aux4_s, SceneInfo* scenes, const DevState* ds) {
    SceneInfo& sc = scenes[blockIdx.x];
    double s[6] = {0, 0, 0, 0, 0, 0};
    const double g = sc.c.grav;
    for (uint32_t i = sc.start + threadIdx.x; i < sc.start + sc.count; i += blockDim.x) {
        const float4 p = pos4[i];
        const float4 v = vel4[i];
        const double m = p.w;
        s[0] += m;
        s[1] += m * v.x;
        s[2] += m * v.y;
        s[3] += m * v.z;
        s[4] += 0.5 * m * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
        s[5] += -m * g * (double)p.y;
    }
    __shared__ double red[kDiagThreads / 32][6];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        double v = s[k];
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double v = 0;
        for (int w = 0; w < kDiagThreads / 32; ++w) v += red[w][threadIdx.x];
        sc.sums[threadIdx.x] = v;
    }
}

int launch_batch_diag(const LaunchCtx& L, const Buffers& b, DevState* ds) {
    k_batch_diag<<<b.nscenes, kDiagThreads, 0, L.stream>>>(b.pos4, b.vel4, b.aux4_s, b.scenes, ds);
    return 1;
}

}  // namespace sphx
