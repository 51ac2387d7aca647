// Standalone spatial hash on the GPU: the device side of SpatialHash::build / query /
// query_squared / get_cell_particles (src/spatial_hash.cpp:15-63).
//
// build() runs the step's grid pipeline (bbox, cell keys, stable radix sort, cell
// offsets) on the given positions with the hash's cell size.  A query visits the
// reference's stencil -- cells cq + (dx, dy, dz), each of dx, dy, dz in
// [-cell_radius, cell_radius] with cell_radius = ceil(sqrt(r2) * inv_cell) + 1, in
// lexicographic order -- and each cell's particles in insertion order, keeping those with
// dot(p - x_j, p - x_j) <= r2: the reference's list, element for element.
#include <cmath>
#include <vector>

#include "sphx_internal.cuh"

using namespace sphx;

struct sphx_grid {
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t capacity = 0;
    size_t n = 0;
    float cell_size = 0.0f;
    bool built = false;
    StepConst sc{};
    Buffers b{};
    DevState* ds = nullptr;
    float* stage = nullptr;  // 4 * capacity floats
    LaunchCtx L{};
    DevState host{};         // copy of the device state after the last build
};

namespace {

struct QueryArgs {
    const float* q;       // 3 floats per query
    int nq;
    float r2;
    int cr;               // stencil half-width in cells
    float inv_cell;
};

// One thread per query; kFill = false counts, kFill = true writes insertion indices.
template <bool kFill>
__global__ void k_grid_query(const QueryArgs a, const Buffers b, const DevState* ds,
                             uint32_t* counts, const uint64_t* offsets, int64_t* out) {
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= a.nq) return;
    const float px = a.q[3 * qi], py = a.q[3 * qi + 1], pz = a.q[3 * qi + 2];
    uint32_t found = 0;
    uint64_t pos = kFill ? offsets[qi] : 0;
    if (finite3(px, py, pz) && ds->status == 0) {
        const float4 p = make_float4(px, py, pz, 0.0f);
        const int d0 = ds->dim[0], d1 = ds->dim[1], d2 = ds->dim[2];
        // relative cell of the query (may lie outside the grid)
        const long long cx = (long long)cell_coord(px, a.inv_cell) - ds->cmin[0];
        const long long cy = (long long)cell_coord(py, a.inv_cell) - ds->cmin[1];
        const long long cz = (long long)cell_coord(pz, a.inv_cell) - ds->cmin[2];
        for (int dx = -a.cr; dx <= a.cr; ++dx) {
            long long X = cx + dx;
            if (ds->wrap[0]) X = ((X % d0) + d0) % d0;
            else if (X < 0 || X >= d0) continue;
            for (int dy = -a.cr; dy <= a.cr; ++dy) {
                long long Y = cy + dy;
                if (ds->wrap[1]) Y = ((Y % d1) + d1) % d1;
                else if (Y < 0 || Y >= d1) continue;
                const uint32_t rb = ((uint32_t)X * (uint32_t)d1 + (uint32_t)Y) * (uint32_t)d2;
                for (int dz = -a.cr; dz <= a.cr; ++dz) {
                    long long Z = cz + dz;
                    if (ds->wrap[2]) Z = ((Z % d2) + d2) % d2;
                    else if (Z < 0 || Z >= d2) continue;
                    const uint32_t k0 = b.off[rb + (uint32_t)Z], k1 = b.off[rb + (uint32_t)Z + 1];
                    for (uint32_t k = k0; k < k1; ++k) {
                        const float4 xj = b.pos4_s[k];
                        const float ddx = xsub(p.x, xj.x), ddy = xsub(p.y, xj.y),
                                    ddz = xsub(p.z, xj.z);
                        if (xdot3(ddx, ddy, ddz) <= a.r2) {
                            if (kFill) out[pos++] = (int64_t)b.id_s[k];
                            ++found;
                        }
                    }
                }
            }
        }
    }
    if (!kFill) counts[qi] = found;
}

int cuda_err(cudaError_t e) { return e == cudaErrorMemoryAllocation ? SPHX_ERR_OOM : SPHX_ERR_CUDA; }

#define GRID_CUDA(call)                             \
    do {                                            \
        cudaError_t e_ = (call);                    \
        if (e_ != cudaSuccess) return cuda_err(e_); \
    } while (0)

template <class T>
int galloc(T** p, size_t count) {
    *p = nullptr;
    if (cudaMalloc(reinterpret_cast<void**>(p), (count ? count : 1) * sizeof(T)) != cudaSuccess) {
        *p = nullptr;
        return SPHX_ERR_OOM;
    }
    return SPHX_OK;
}

void grid_free(sphx_grid* g) {
    Buffers& b = g->b;
    void* ptrs[] = {b.pos4, b.vel4, b.pos4_s, b.vel4_s, b.key[0], b.key[1], b.val[0], b.val[1],
                    b.key_s, b.id_s, b.off, b.tile_start, b.hist, b.scan_part, g->ds, g->stage};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (g->stream) cudaStreamDestroy(g->stream);
}

// the stencil half-width of SpatialHash::query_squared (spatial_hash.cpp:35)
int cell_radius(float r2, float inv_cell) {
    return static_cast<int>(std::ceil(std::sqrt(r2) * inv_cell)) + 1;
}

}  // namespace

extern "C" {

int sphx_grid_create(sphx_grid** out, size_t capacity) {
    if (!out) return SPHX_ERR_INVALID_ARG;
    *out = nullptr;
    if (capacity == 0 || capacity > (size_t)0x7fffffff - 64) return SPHX_ERR_INVALID_ARG;
    int devs = 0;
    if (cudaGetDeviceCount(&devs) != cudaSuccess || devs == 0) return SPHX_ERR_CUDA;
    sphx_grid* g = new sphx_grid();
    auto fail = [&](int rc) {
        grid_free(g);
        delete g;
        return rc;
    };
    if (cudaGetDevice(&g->device) != cudaSuccess) return fail(SPHX_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(SPHX_ERR_CUDA);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g->device);
    g->L.stream = g->stream;
    g->L.device = g->device;
    g->L.num_sms = sms > 0 ? sms : 1;
    g->L.warps_per_block = 4;
    g->capacity = capacity;
    int64_t max_cells = (int64_t)capacity * 4;
    if (max_cells < ((int64_t)1 << 24)) max_cells = (int64_t)1 << 24;
    if (max_cells > ((int64_t)1 << 31) - 4) max_cells = ((int64_t)1 << 31) - 4;
    g->sc.max_cells = (uint32_t)max_cells;
    Buffers& b = g->b;
    const size_t C = capacity;
    b.radix_blocks = (int)((C + kRadixTileN - 1) / kRadixTileN);
    const size_t hist_n = (size_t)b.radix_blocks * kRadixBuckets;
    const size_t pa = (hist_n + kScanTileN - 1) / kScanTileN, pb = (C + kScanTileN - 1) / kScanTileN;
    b.scan_part_cap = (int)((pa > pb ? pa : pb) + 1);
    int rc;
    if ((rc = galloc(&b.pos4, C)) || (rc = galloc(&b.vel4, C)) || (rc = galloc(&b.pos4_s, C)) ||
        (rc = galloc(&b.vel4_s, C)) || (rc = galloc(&b.key[0], C)) || (rc = galloc(&b.key[1], C)) ||
        (rc = galloc(&b.val[0], C)) || (rc = galloc(&b.val[1], C)) || (rc = galloc(&b.key_s, C)) ||
        (rc = galloc(&b.id_s, C)) || (rc = galloc(&b.off, (size_t)max_cells + 2)) ||
        (rc = galloc(&b.tile_start, C)) || (rc = galloc(&b.hist, hist_n)) ||
        (rc = galloc(&b.scan_part, (size_t)b.scan_part_cap)) || (rc = galloc(&g->ds, 1)) ||
        (rc = galloc(&g->stage, 4 * C)))
        return fail(rc);
    if (cudaMemset(g->ds, 0, sizeof(DevState)) != cudaSuccess) return fail(SPHX_ERR_CUDA);
    *out = g;
    return SPHX_OK;
}

void sphx_grid_destroy(sphx_grid* g) {
    if (!g) return;
    cudaSetDevice(g->device);
    cudaStreamSynchronize(g->stream);
    grid_free(g);
    delete g;
}

int sphx_grid_build(sphx_grid* g, size_t n, const float* pos_xyz, float cell_size) {
    if (!g) return SPHX_ERR_INVALID_ARG;
    if (n > g->capacity) return SPHX_ERR_CAPACITY;
    if (n > 0 && !pos_xyz) return SPHX_ERR_INVALID_ARG;
    if (!(cell_size > 0.0f) || !std::isfinite(cell_size) || !std::isfinite(1.0f / cell_size))
        return SPHX_ERR_INVALID_ARG;
    GRID_CUDA(cudaSetDevice(g->device));
    g->n = n;
    g->cell_size = cell_size;
    g->built = true;
    g->sc.n = (int)n;
    g->sc.inv_cell = 1.0f / cell_size;  // SpatialHash::set_cell_size (spatial_hash.h:63-66)
    if (n == 0) return SPHX_OK;
    float* s_pos = g->stage;
    float* s_mass = g->stage + 3 * g->capacity;
    GRID_CUDA(cudaMemcpyAsync(s_pos, pos_xyz, 3 * n * sizeof(float), cudaMemcpyHostToDevice, g->stream));
    GRID_CUDA(cudaMemsetAsync(s_mass, 0, n * sizeof(float), g->stream));
    launch_pack(g->L, (int)n, s_pos, nullptr, s_mass, g->b.pos4, g->b.vel4);
    launch_begin_step(g->L, g->ds, 1);
    launch_build_grid(g->L, g->sc, g->b, g->ds);
    GRID_CUDA(cudaGetLastError());
    GRID_CUDA(cudaStreamSynchronize(g->stream));
    GRID_CUDA(cudaMemcpy(&g->host, g->ds, sizeof(DevState), cudaMemcpyDeviceToHost));
    return g->host.status;
}

int sphx_grid_query(sphx_grid* g, size_t nq, const float* q_xyz, float radius_squared,
                    int64_t* counts, int64_t* idx, size_t* total_inout) {
    if (!g || !counts || !total_inout || (nq > 0 && !q_xyz)) return SPHX_ERR_INVALID_ARG;
    if (nq > (size_t)0x7fffffff) return SPHX_ERR_INVALID_ARG;
    GRID_CUDA(cudaSetDevice(g->device));
    const size_t cap = *total_inout;
    *total_inout = 0;
    if (nq == 0) return SPHX_OK;
    if (!g->built || g->n == 0 || !(radius_squared >= 0.0f) || !std::isfinite(radius_squared)) {
        for (size_t i = 0; i < nq; ++i) counts[i] = 0;  // nothing can be within r
        return SPHX_OK;
    }
    const int cr = cell_radius(radius_squared, g->sc.inv_cell);
    // a folded axis may not wrap the stencil onto itself
    for (int a = 0; a < 3; ++a)
        if (g->host.wrap[a] && 2 * (long long)cr + 1 > g->host.dim[a]) return SPHX_ERR_DOMAIN;
    float* d_q = nullptr;
    uint32_t* d_cnt = nullptr;
    uint64_t* d_off = nullptr;
    int64_t* d_out = nullptr;
    int rc = SPHX_OK;
    auto cleanup = [&]() {
        cudaFree(d_q);
        cudaFree(d_cnt);
        cudaFree(d_off);
        cudaFree(d_out);
    };
    if ((rc = galloc(&d_q, 3 * nq)) || (rc = galloc(&d_cnt, nq))) {
        cleanup();
        return rc;
    }
    QueryArgs qa{d_q, (int)nq, radius_squared, cr, g->sc.inv_cell};
    const int threads = 128, blocks = (int)((nq + threads - 1) / threads);
    std::vector<uint32_t> h_cnt(nq);
    cudaError_t e = cudaMemcpyAsync(d_q, q_xyz, 3 * nq * sizeof(float), cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) {
        k_grid_query<false><<<blocks, threads, 0, g->stream>>>(qa, g->b, g->ds, d_cnt, nullptr, nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h_cnt.data(), d_cnt, nq * sizeof(uint32_t), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) {
        cleanup();
        return cuda_err(e);
    }
    std::vector<uint64_t> off(nq);
    uint64_t total = 0;
    for (size_t i = 0; i < nq; ++i) {
        counts[i] = h_cnt[i];
        off[i] = total;
        total += h_cnt[i];
    }
    *total_inout = (size_t)total;
    if (!idx || total == 0) {
        cleanup();
        return SPHX_OK;
    }
    if (cap < total) {
        cleanup();
        return SPHX_ERR_OVERFLOW;
    }
    if ((rc = galloc(&d_off, nq)) || (rc = galloc(&d_out, total))) {
        cleanup();
        return rc;
    }
    e = cudaMemcpyAsync(d_off, off.data(), nq * sizeof(uint64_t), cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) {
        k_grid_query<true><<<blocks, threads, 0, g->stream>>>(qa, g->b, g->ds, nullptr, d_off, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(idx, d_out, total * sizeof(int64_t), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cleanup();
    return e == cudaSuccess ? SPHX_OK : cuda_err(e);
}

int sphx_grid_info(sphx_grid* g, size_t* occupied_cells, size_t* max_per_cell) {
    if (!g) return SPHX_ERR_INVALID_ARG;
    const bool any = g->built && g->n > 0;
    if (occupied_cells) *occupied_cells = any ? g->host.occupied : 0;
    if (max_per_cell) *max_per_cell = any ? g->host.max_occ : 0;
    return SPHX_OK;
}

int sphx_grid_cell(sphx_grid* g, int x, int y, int z, int64_t* idx, size_t* count_inout) {
    if (!g || !count_inout) return SPHX_ERR_INVALID_ARG;
    GRID_CUDA(cudaSetDevice(g->device));
    const size_t cap = *count_inout;
    *count_inout = 0;
    if (!g->built || g->n == 0) return SPHX_OK;
    const DevState& s = g->host;
    const int c[3] = {x, y, z};
    long long r[3];
    for (int a = 0; a < 3; ++a) {
        if (c[a] < s.cmin[a] || c[a] > s.cmax[a]) return SPHX_OK;  // no particle there
        r[a] = (long long)c[a] - s.cmin[a];
        if (s.wrap[a]) r[a] %= s.dim[a];
    }
    const uint32_t key = (uint32_t)((r[0] * s.dim[1] + r[1]) * s.dim[2] + r[2]);
    uint32_t range[2];
    GRID_CUDA(cudaMemcpy(range, g->b.off + key, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (range[1] <= range[0]) return SPHX_OK;
    const size_t cnt = range[1] - range[0];
    std::vector<uint32_t> ids(cnt);
    std::vector<float4> pos(cnt);
    GRID_CUDA(cudaMemcpy(ids.data(), g->b.id_s + range[0], cnt * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    GRID_CUDA(cudaMemcpy(pos.data(), g->b.pos4_s + range[0], cnt * sizeof(float4), cudaMemcpyDeviceToHost));
    // a folded grid cell can hold several true cells: keep the requested one
    size_t m = 0;
    std::vector<int64_t> keep;
    keep.reserve(cnt);
    const float inv = g->sc.inv_cell;
    for (size_t k = 0; k < cnt; ++k) {
        const float p[3] = {pos[k].x, pos[k].y, pos[k].z};
        bool same = true;
        for (int a = 0; a < 3 && same; ++a) {
            float f = std::floor(p[a] * inv);
            f = std::fmin(std::fmax(f, -(float)kCellClamp), (float)(kCellClamp - 1));
            same = (int)f == c[a];
        }
        if (same) keep.push_back(ids[k]);
    }
    m = keep.size();
    *count_inout = m;
    if (!idx) return SPHX_OK;
    if (cap < m) return SPHX_ERR_OVERFLOW;
    for (size_t k = 0; k < m; ++k) idx[k] = keep[k];
    return SPHX_OK;
}

}  // extern "C"
