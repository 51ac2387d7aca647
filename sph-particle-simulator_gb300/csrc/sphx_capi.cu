// C ABI of the sm_103a SPH step (include/sphx.h): context lifetime, device memory,
// host<->device transfers and the step's launch sequence.
#include <cmath>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <utility>
#include <vector>

#include "sphx_internal.cuh"

using namespace sphx;

struct sphx_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    size_t capacity = 0;
    size_t n = 0;
    sphx_tuning tuning{};
    sphx_params params{};
    bool have_params = false;
    bool have_fields = false;  // rho/P/acc of the current particle set exist
    bool diag_stale = false;   // a step ran since the FP64 sums were last computed
    StepConst sc{};
    Buffers b{};
    int kernel = SPHX_KERNEL_CUBIC_SPLINE;
    DevState* ds = nullptr;
    float* stage = nullptr;    // 11 * capacity floats (FP64 positions; all download fields)
    float4* snap_pos = nullptr;
    float4* snap_vel = nullptr;
    int4* snap_cell = nullptr;
    LaunchCtx L{};
    uint64_t steps = 0;
    uint64_t queries = 0;
    uint64_t launches = 0;  // kernels this context has launched for steps/evals
    double t_total = 0, t_nb = 0, t_den = 0, t_force = 0;
    // per-phase timing: events recorded into a ring, read back only when a slot is reused
    // or the stats are requested, so profiling adds no per-step host sync
    // batched scenes
    uint32_t nscenes = 0;
    bool scenes_nz = false;  // every scene's divisors admit the untested divisions (div_nz)
    uint32_t scene_cap = 0;
    std::vector<sphx_params> scene_params;
    std::vector<uint64_t> scene_start;
    // CUDA graph of the step (tuning.graph): captured after one warm-up step, replayed
    // while n, dt, parameters and scenes stay the same
    cudaGraphExec_t graph_exec = nullptr;
    bool graph_warm = false;
    uint64_t graph_version = ~0ull;
    float graph_dt = 0.0f;
    int graph_launches = 0;
    uint64_t version = 0;  // bumped by every change the graph depends on
    // headless rendering: colour staging, instance buffer, depth keys and image
    float* r_colors = nullptr;
    float* r_inst = nullptr;
    size_t r_cap = 0;  // particles the two above hold
    unsigned long long* r_keys = nullptr;
    uchar4* r_rgba = nullptr;
    size_t r_pix_cap = 0;
    int* h_status = nullptr;  // pinned host word: the device status, read with the results
    // second stream for device-to-host copies that can run beside the main stream's
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_unpacked = nullptr, ev_copied = nullptr;
    static constexpr int kProfRing = 64;
    struct ProfSlot {
        cudaEvent_t ev[5];
        bool pending;
    } prof[kProfRing] = {};
    int prof_head = 0;
};

namespace {

constexpr int kDefaultWarpsPerBlock = 4;

int cuda_fail(cudaError_t e) {
    if (e == cudaErrorMemoryAllocation) return SPHX_ERR_OOM;
    return SPHX_ERR_CUDA;
}

#define SPHX_CUDA(call)                            \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) return cuda_fail(e_); \
    } while (0)

template <class T>
int dmalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e);
    }
    return SPHX_OK;
}

// Host copy of CubicSplineKernel::W_3d (kernels.cpp:58-66) for the self term W(0); this
// file is compiled with -ffp-contract=off so float expressions round like the reference.
float host_cubic_w(float sigma, float q) {
    if (q >= 0.0f && q <= 1.0f) {
        return sigma * (2.0f / 3.0f - q * q + 0.5f * q * q * q);
    } else if (q > 1.0f && q <= 2.0f) {
        const float tmp = 2.0f - q;
        return sigma * (1.0f / 6.0f * tmp * tmp * tmp);
    }
    return 0.0f;
}


// Verifies the one-correction division sequence of xdiv_fixed for divisor b against IEEE
// float division, for every dividend significand of the binade [1, 2) (about 8 ms).
// Results are cached per divisor; only b in [2^-20, 2^20] qualifies.
bool verify_fixed_divisor(float b) {
    static std::mutex mu;
    static std::vector<std::pair<uint32_t, bool>> cache;
    if (!(b >= 0x1p-20f && b <= 0x1p20f)) return false;
    uint32_t bits;
    std::memcpy(&bits, &b, 4);
    {
        std::lock_guard<std::mutex> lock(mu);
        for (const auto& e : cache)
            if (e.first == bits) return e.second;
    }
    const float y = 1.0f / b;
    bool ok = true;
    for (uint32_t m = 0; m < (1u << 23) && ok; ++m) {
        const uint32_t abits = 0x3f800000u | m;
        float a;
        std::memcpy(&a, &abits, 4);
        const float q0 = a * y;
        const float r = std::fma(-q0, b, a);
        const float q1 = std::fma(r, y, q0);
        const float q = a / b;
        ok = (q1 == q);
    }
    std::lock_guard<std::mutex> lock(mu);
    cache.emplace_back(bits, ok);
    return ok;
}

}  // namespace

namespace sphx {

void step_const_from_params(const sphx_params& p, size_t n, int kernel, int mode,
                            uint32_t max_cells, StepConst& s) {
    s.max_cells = max_cells;
    s.n = (int)n;
    // SpatialHash::set_cell_size(neighbor_search_radius): inv = 1.0f / cell
    s.inv_cell = 1.0f / p.neighbor_search_radius;
    s.r2 = p.neighbor_search_radius * p.neighbor_search_radius;
    // CubicSplineKernel(h): h_sq = h*h, sigma_3d = 1 / (float(pi) * h * h * h)
    const float h = p.smoothing_length;
    s.h = h;
    s.h_sq = h * h;
    s.sigma = 1.0f / (static_cast<float>(M_PI) * h * h * h);
    // W(vec3(0)): q = length(0) / h
    const float q0 = std::sqrt(0.0f) / h;
    s.w0 = host_cubic_w(s.sigma, q0);
    s.kern = kernel;
    s.wnorm = s.wl = s.gs = s.gg = s.gl = s.g2s = 0.0f;
    if (kernel == SPHX_KERNEL_WENDLAND_C2) {
        // WendlandC2Kernel(h) (kernels.cpp:166-170); W(0) as WendlandC2Kernel::W computes it
        s.wnorm = 21.0f / (2.0f * static_cast<float>(M_PI) * h * h * h);
        s.wl = s.wnorm * (5.0f / s.h_sq);
        const float tmp = 1.0f - 0.5f * q0;
        s.w0 = s.wnorm * tmp * tmp * tmp * tmp * (2.0f * q0 + 1.0f);
    } else if (kernel == SPHX_KERNEL_GAUSSIAN) {
        // GaussianKernel(h) (kernels.cpp:203-208); W(0) = norm_ * exp(-0 * sigma_sq_inv_)
        s.gs = 1.0f / (h * h);
        s.wnorm = 1.0f / std::pow(static_cast<float>(M_PI) * h * h, 1.5f);
        s.gg = -2.0f * s.gs * s.wnorm;
        s.gl = 2.0f * s.gs * s.wnorm;
        s.g2s = 2.0f * s.gs;
        s.w0 = s.wnorm * std::exp(-0.0f * s.gs);
    }
    s.rest = p.rest_density;
    s.gas = p.gas_constant;
    s.visc = p.viscosity;
    s.grav = p.gravity;
    s.damping = p.damping;
    s.cfl = p.cfl_factor;
    s.timestep = p.timestep;
    s.lo[0] = p.xmin;
    s.hi[0] = p.xmax;
    s.lo[1] = p.ymin;
    s.hi[1] = p.ymax;
    s.lo[2] = p.zmin;
    s.hi[2] = p.zmax;
    s.rcp_h = 1.0f / h;
    s.rcp_hsq = 1.0f / s.h_sq;
    s.fast_div_h = verify_fixed_divisor(h) ? 1 : 0;
    s.fast_div_hsq = verify_fixed_divisor(s.h_sq) ? 1 : 0;
    // the cubic passes' untested divisions: |r| of a hit is at most r (1 + 2^-23) and the
    // Laplacian's numerator at most 2 sigma; both divisors verified (so h, h^2 in
    // [2^-20, 2^20] and sigma = 1/(pi h^3) within [2^-62, 2^59])
    s.div_nz = s.fast_div_h && s.fast_div_hsq && p.neighbor_search_radius > 0.0f &&
                       p.neighbor_search_radius <= 0x1p99f
                   ? 1 : 0;
    s.precise = mode != SPHX_MODE_EXACT;
    s.fp16 = mode == SPHX_MODE_PRECISE_FP16;
    s.cs = p.neighbor_search_radius;
    s.cs_d = (double)p.neighbor_search_radius;
    s.sw_cs = s.cs * s.rcp_h;  // 2 exactly for r_search = 2h
    s.sw_r2 = s.r2 * s.rcp_hsq;
    s.sw_r2m = s.sw_r2 * 1.0001f;
    s.sw_skip2 = 1e-12f * s.rcp_hsq;
}

}  // namespace sphx

namespace {

void fill_step_const_from(sphx_ctx* c, const sphx_params& p, size_t n, StepConst& s) {
    step_const_from_params(p, n, c->kernel, c->tuning.mode, c->sc.max_cells, s);
}

void fill_step_const(sphx_ctx* c) { fill_step_const_from(c, c->params, c->n, c->sc); }

__global__ void k_mass_of(int n, const float4* __restrict__ pos4, float* __restrict__ mass) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        mass[i] = pos4[i].w;
}

__global__ void k_f64_to_f32(int n3, const double* __restrict__ in, float* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

__global__ void k_f32_to_f64(int n3, const float* __restrict__ in, double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

void free_all(sphx_ctx* c) {
    Buffers& b = c->b;
    void* ptrs[] = {b.pos4, b.vel4,   b.pos4_s, b.vel4_s,     b.aux4_s,    b.acc4_s,
                    b.key[0], b.key[1], b.val[0], b.val[1],   b.key_s,     b.id_s,
                    b.off,  b.tile_start, b.hist, b.scan_part, b.diag_part, c->ds,
                    c->stage, c->snap_pos, c->snap_vel, c->snap_cell, b.cell4, b.cell4_s,
                    b.spread_tiles, b.runs,
                    b.scene_of, b.scene_s, b.scenes, b.hitmask, b.tile_slot,
                    c->r_colors, c->r_inst, c->r_keys, c->r_rgba};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (auto& slot : c->prof)
        for (auto& e : slot.ev)
            if (e) cudaEventDestroy(e);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->ev_unpacked) cudaEventDestroy(c->ev_unpacked);
    if (c->ev_copied) cudaEventDestroy(c->ev_copied);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
}

// Adds one recorded step's phase times to the accumulators (waits for it if needed).
int drain_slot(sphx_ctx* c, sphx_ctx::ProfSlot& slot) {
    if (!slot.pending) return SPHX_OK;
    slot.pending = false;
    SPHX_CUDA(cudaEventSynchronize(slot.ev[4]));
    float ms[4];
    for (int k = 0; k < 4; ++k) SPHX_CUDA(cudaEventElapsedTime(&ms[k], slot.ev[k], slot.ev[k + 1]));
    c->t_nb += ms[0] * 1e-3;
    c->t_den += ms[1] * 1e-3;
    c->t_force += ms[2] * 1e-3;
    c->t_total += (ms[0] + ms[1] + ms[2] + ms[3]) * 1e-3;
    return SPHX_OK;
}

int drain_all(sphx_ctx* c) {
    for (auto& slot : c->prof) {
        const int rc = drain_slot(c, slot);
        if (rc) return rc;
    }
    return SPHX_OK;
}

// Waits for the context's stream and returns the device status word (read on the stream,
// into pinned memory, so other streams are not waited for).
int sync_status(sphx_ctx* c) {
    SPHX_CUDA(cudaMemcpyAsync(c->h_status, c->ds, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    SPHX_CUDA(cudaGetLastError());
    return *c->h_status;
}

// The FP64 sums of the state (k_diag_*, k_batch_diag), computed when the stats are read
// rather than in every step: the reference's step computes no diagnostics (its
// get_total_mass / get_total_energy run on demand, src/sph_engine.cpp:187-200).  They
// cover the current particle state -- after a step, the state it produced -- and the
// densities of the last density pass (none yet: the density sum is 0).  Not counted in
// `launches` (the kernels of steps and evals).
int refresh_diag(sphx_ctx* c) {
    if (!c->diag_stale) return SPHX_OK;
    c->diag_stale = false;
    if (c->n == 0) return SPHX_OK;
    fill_step_const(c);
    if (c->b.nscenes > 0) {
        launch_batch_diag(c->L, c->b, c->ds);
    } else {
        Buffers bq = c->b;
        if (!c->have_fields) bq.aux4_s = nullptr;
        launch_diag(c->L, c->sc, bq, c->ds);
    }
    SPHX_CUDA(cudaGetLastError());
    return SPHX_OK;
}

int enter(sphx_ctx* c) {
    if (!c) return SPHX_ERR_INVALID_ARG;
    SPHX_CUDA(cudaSetDevice(c->device));
    return SPHX_OK;
}

int run_phases(sphx_ctx* c, float dt, bool integrate) {
    fill_step_const(c);
    sphx_ctx::ProfSlot* slot = nullptr;
    if (c->tuning.profile) {
        slot = &c->prof[c->prof_head];
        c->prof_head = (c->prof_head + 1) % sphx_ctx::kProfRing;
        const int rc = drain_slot(c, *slot);
        if (rc) return rc;
        SPHX_CUDA(cudaEventRecord(slot->ev[0], c->stream));
    }
    const bool batch = c->b.nscenes > 0;
    if (batch) c->sc.div_nz = c->scenes_nz ? 1 : 0;  // the passes' kernels serve all scenes
    int k = 0;
    if (batch) {
        k += launch_batch_begin(c->L, c->b, c->ds);
        if (integrate) k += launch_batch_cfl(c->L, c->b, c->ds, (int)c->n, dt);
        k += launch_batch_grid(c->L, c->b, c->ds, (int)c->n, c->sc.max_cells);
    } else {
        k += launch_begin_step(c->L, c->ds, 1);
        if (integrate) k += launch_cfl(c->L, c->sc, c->b, c->ds, dt);
        k += launch_build_grid(c->L, c->sc, c->b, c->ds);
    }
    if (slot) SPHX_CUDA(cudaEventRecord(slot->ev[1], c->stream));
    k += launch_density(c->L, c->sc, c->b, c->ds);
    if (slot) SPHX_CUDA(cudaEventRecord(slot->ev[2], c->stream));
    k += launch_force(c->L, c->sc, c->b, c->ds, integrate ? 1 : 0);
    if (slot) SPHX_CUDA(cudaEventRecord(slot->ev[3], c->stream));
    if (integrate) c->diag_stale = true;  // the FP64 sums: computed when read (refresh_diag)
    if (slot) {
        SPHX_CUDA(cudaEventRecord(slot->ev[4], c->stream));
        slot->pending = true;
    }
    SPHX_CUDA(cudaGetLastError());
    c->launches += (uint64_t)k;
    c->graph_launches = k;
    c->have_fields = true;
    return SPHX_OK;
}

// One step through a CUDA graph: the first step of a configuration runs eagerly (it warms
// up the per-kernel launch shapes), the next one is captured, later ones replay it.
int run_step_graph(sphx_ctx* c, float dt) {
    const bool same = c->graph_exec && c->graph_version == c->version && c->graph_dt == dt;
    if (!same) {
        if (c->graph_exec) {
            cudaGraphExecDestroy(c->graph_exec);
            c->graph_exec = nullptr;
        }
        if (!c->graph_warm || c->graph_version != c->version) {
            c->graph_warm = true;
            c->graph_version = c->version;
            c->graph_dt = dt;
            return run_phases(c, dt, true);
        }
        const int saved = c->tuning.profile;
        c->tuning.profile = 0;  // no host-side event reads inside a capture
        SPHX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = run_phases(c, dt, true);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        c->tuning.profile = saved;
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(e);
        const cudaError_t ei = cudaGraphInstantiate(&c->graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            c->graph_exec = nullptr;
            return cuda_fail(ei);
        }
        c->graph_version = c->version;
        c->graph_dt = dt;
        c->launches -= (uint64_t)c->graph_launches;  // captured, not launched
    }
    SPHX_CUDA(cudaGraphLaunch(c->graph_exec, c->stream));
    c->launches += (uint64_t)c->graph_launches;
    c->have_fields = true;
    return SPHX_OK;
}


// Device address of a host buffer the GPU can access in place (pinned: cudaHostAlloc or
// cudaHostRegister), or null (pageable memory: the caller's data go through staging).
// On Grace + Blackwell the kernels then read and write it over the coherent C2C link.
template <class T>
T* mapped(T* h) {
    if (!h) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? static_cast<T*>(a.devicePointer)
                                                             : nullptr;
}

// ---- headless rendering helpers ----------------------------------------------------------

// C = A * B for column-major 4x4 float matrices, each element summed k = 0..3 in order
void mat4_mul(const float* A, const float* B, float* C) {
    for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row) {
            float acc = A[row] * B[col * 4];
            for (int k = 1; k < 4; ++k) acc = acc + A[k * 4 + row] * B[col * 4 + k];
            C[col * 4 + row] = acc;
        }
}

int render_const(const sphx_render_params* p, RenderConst& r) {
    if (!p || p->width <= 0 || p->height <= 0 || p->width > 16384 || p->height > 16384 ||
        p->color_mode < SPHX_COLOR_VELOCITY || p->color_mode > SPHX_COLOR_TYPE ||
        !std::isfinite(p->particle_size))
        return SPHX_ERR_INVALID_ARG;
    float pv[16];
    mat4_mul(p->projection, p->view, pv);
    mat4_mul(pv, p->model, r.pvm);
    for (int a = 0; a < 3; ++a) {
        r.right[a] = p->view[a * 4];   // (view[0][0], view[1][0], view[2][0])
        r.up[a] = p->view[a * 4 + 1];  // (view[0][1], view[1][1], view[2][1])
        r.bg[a] = p->background[a];
    }
    r.size = p->particle_size;
    r.mode = p->color_mode;
    // lightDir = normalize((1, 1, 1)), normal = (0, 0, 1): diff = max(lightDir.z, 0)
    const float len = std::sqrt((1.0f * 1.0f + 1.0f * 1.0f) + 1.0f * 1.0f);
    const float lz = 1.0f / len;
    r.diffuse = lz > 0.0f ? lz : 0.0f;
    r.width = p->width;
    r.height = p->height;
    return SPHX_OK;
}

int render_buffers(sphx_ctx* c, size_t npix) {
    int rc;
    if (c->r_cap < c->capacity) {
        if (c->r_colors) cudaFree(c->r_colors);
        if (c->r_inst) cudaFree(c->r_inst);
        c->r_colors = c->r_inst = nullptr;
        c->r_cap = 0;
        if ((rc = dmalloc(&c->r_colors, 3 * c->capacity)) ||
            (rc = dmalloc(&c->r_inst, 20 * c->capacity)))
            return rc;
        c->r_cap = c->capacity;
    }
    if (npix > c->r_pix_cap) {
        if (c->r_keys) cudaFree(c->r_keys);
        if (c->r_rgba) cudaFree(c->r_rgba);
        c->r_keys = nullptr;
        c->r_rgba = nullptr;
        c->r_pix_cap = 0;
        if ((rc = dmalloc(&c->r_keys, npix)) || (rc = dmalloc(&c->r_rgba, npix))) return rc;
        c->r_pix_cap = npix;
    }
    return SPHX_OK;
}

RenderArgs render_args(sphx_ctx* c, const float* colors_dev) {
    RenderArgs a;
    a.n = (int)c->n;
    a.pos4 = c->b.pos4;
    a.vel4 = c->b.vel4;
    a.cell4 = c->b.cell4;
    a.cs = (double)c->params.neighbor_search_radius;
    a.colors = colors_dev;
    return a;
}


// ---- device generation helpers -----------------------------------------------------------

// The host-side constants of one shape, computed with the generator's float operations
// (glm vector ops are component-wise; int * float converts the int first).
int gen_shape(const sphx_shape& in, GenShape& g) {
    std::memset(&g, 0, sizeof(g));
    g.kind = in.kind;
    g.spacing = in.spacing;
    g.mass = in.mass;
    for (int a = 0; a < 3; ++a) g.vel[a] = in.velocity[a];
    const float sp = in.spacing;
    auto lattice_count = [](const int n[3]) -> uint64_t {
        if (n[0] <= 0 || n[1] <= 0 || n[2] <= 0) return 0;
        return (uint64_t)n[0] * (uint64_t)n[1] * (uint64_t)n[2];
    };
    switch (in.kind) {
        case SPHX_SHAPE_BLOCK: {
            if (!(sp > 0.0f) || !std::isfinite(sp)) return SPHX_ERR_INVALID_ARG;
            for (int a = 0; a < 3; ++a) {
                g.n[a] = static_cast<int>(in.size[a] / sp);
                g.start[a] = in.center[a] - in.size[a] * 0.5f;
            }
            const uint64_t c = lattice_count(g.n);
            if (c > 0xffffffffull) return SPHX_ERR_CAPACITY;
            g.count = (uint32_t)c;
            return SPHX_OK;
        }
        case SPHX_SHAPE_BOX: {
            if (!(sp > 0.0f) || !std::isfinite(sp)) return SPHX_ERR_INVALID_ARG;
            float half[3];
            for (int a = 0; a < 3; ++a) {
                half[a] = in.size[a] * 0.5f;
                g.start[a] = in.center[a] - half[a];
            }
            // faces in the reference's order: z = start.z, z = start.z + size.z,
            // x = start.x, x = start.x + size.x, y = start.y, y = start.y + size.y
            const int axes[6][3] = {{0, 1, 2}, {0, 1, 2}, {1, 2, 0}, {1, 2, 0}, {0, 2, 1}, {0, 2, 1}};
            uint64_t off = 0;
            for (int f = 0; f < 6; ++f) {
                for (int a = 0; a < 3; ++a) g.face_a[f][a] = axes[f][a];
                const int a3 = axes[f][2];
                g.face_val[f] = (f % 2 == 0) ? g.start[a3] : g.start[a3] + in.size[a3];
                const int n1 = static_cast<int>(in.size[axes[f][0]] / sp);
                const int n2 = static_cast<int>(in.size[axes[f][1]] / sp);
                g.face_n2[f] = n2 > 0 ? n2 : 1;
                g.face_off[f] = (uint32_t)off;
                if (n1 > 0 && n2 > 0) off += (uint64_t)n1 * (uint64_t)n2;
                if (off > 0xffffffffull) return SPHX_ERR_CAPACITY;
            }
            g.face_off[6] = (uint32_t)off;
            g.count = (uint32_t)off;
            return SPHX_OK;
        }
        case SPHX_SHAPE_SPHERE: {
            if (!(sp > 0.0f) || !std::isfinite(sp)) return SPHX_ERR_INVALID_ARG;
            const float r = in.size[0];
            const int nd = static_cast<int>(2.0f * r / sp);
            if (nd > 4096) return SPHX_ERR_CAPACITY;
            g.n[0] = g.n[1] = g.n[2] = nd > 0 ? nd : 0;
            for (int a = 0; a < 3; ++a) {
                g.center[a] = in.center[a];
                g.start[a] = in.center[a] - r;
            }
            g.r2 = r * r;
            return SPHX_OK;  // count: on the device
        }
        case SPHX_SHAPE_LATTICE: {
            for (int a = 0; a < 3; ++a) {
                g.n[a] = in.counts[a];
                g.origin[a] = in.center[a];
                if (in.center[a] != 0.0f) g.has_origin = 1;
            }
            g.jitter = in.jitter;
            g.seed = in.seed;
            const uint64_t c = lattice_count(g.n);
            if (c > 0xffffffffull) return SPHX_ERR_CAPACITY;
            g.count = (uint32_t)c;
            return SPHX_OK;
        }
        case SPHX_SHAPE_BALL: {
            const double R = in.ball_radius, bs = in.ball_spacing;
            if (!(bs > 0.0) || !(R >= 0.0) || !std::isfinite(R / bs)) return SPHX_ERR_INVALID_ARG;
            const double kq = R / bs;
            if (kq > 2000.0) return SPHX_ERR_CAPACITY;
            g.kmax = static_cast<int>(kq) + 1;
            g.n[0] = g.n[1] = g.n[2] = 2 * g.kmax + 1;
            for (int a = 0; a < 3; ++a) g.c64[a] = in.ball_center[a];
            g.sp64 = bs;
            g.R2 = R * R;
            return SPHX_OK;
        }
    }
    return SPHX_ERR_INVALID_ARG;
}

}  // namespace

extern "C" {

int sphx_version(void) { return SPHX_ABI_VERSION; }

const char* sphx_strerror(int code) {
    switch (code) {
        case SPHX_OK: return "ok";
        case SPHX_ERR_INVALID_ARG: return "invalid argument";
        case SPHX_ERR_OOM: return "out of memory";
        case SPHX_ERR_CUDA: return "CUDA runtime error";
        case SPHX_ERR_TIMEOUT: return "device-side wait timed out";
        case SPHX_ERR_CAPACITY: return "particle capacity exceeded";
        case SPHX_ERR_NOT_READY: return "parameters or particles not set";
        case SPHX_ERR_DOMAIN: return "cell grid cannot be laid out";
        case SPHX_ERR_OVERFLOW: return "output buffer too small";
        default: return "unknown sphx error";
    }
}

int sphx_create(sphx_ctx** out, size_t capacity, const sphx_tuning* tuning) {
    if (!out) return SPHX_ERR_INVALID_ARG;
    *out = nullptr;
    if (capacity == 0 || capacity > (size_t)0x7fffffff - 64) return SPHX_ERR_INVALID_ARG;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) return SPHX_ERR_CUDA;
    sphx_ctx* c = new (std::nothrow) sphx_ctx();
    if (!c) return SPHX_ERR_OOM;
    if (tuning) c->tuning = *tuning;
    if (c->tuning.mode < SPHX_MODE_EXACT || c->tuning.mode > SPHX_MODE_PRECISE_FP16) {
        delete c;
        return SPHX_ERR_INVALID_ARG;
    }
    if (c->tuning.warps_per_block <= 0 || c->tuning.warps_per_block > 4)
        c->tuning.warps_per_block = kDefaultWarpsPerBlock;
    if (c->tuning.tile_particles <= 0 || c->tuning.tile_particles > kTile)
        c->tuning.tile_particles = kTile;
    c->b.tile_n = c->tuning.tile_particles;
    c->b.columns = c->tuning.mode != SPHX_MODE_EXACT ? 1 : 0;  // the precision-mode sweeps' tiles
    c->tuning.bulk_copy = c->tuning.bulk_copy ? 1 : 0;
    int rc = SPHX_OK;
    auto fail = [&](int code) {
        free_all(c);
        delete c;
        return code;
    };
    if (cudaGetDevice(&c->device) != cudaSuccess) return fail(SPHX_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(SPHX_ERR_CUDA);
    c->stream = c->own_stream;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    c->L.device = c->device;
    c->L.num_sms = sms > 0 ? sms : 1;
    c->L.warps_per_block = c->tuning.warps_per_block;
    c->L.blocks_per_sm = c->tuning.blocks_per_sm;
    c->L.bulk_copy = c->tuning.bulk_copy;
    c->L.stream = c->stream;
    c->capacity = capacity;
    int64_t max_cells = c->tuning.max_grid_cells;
    if (max_cells <= 0) {
        max_cells = (int64_t)capacity * 4;
        if (max_cells < (int64_t)1 << 24) max_cells = (int64_t)1 << 24;
    }
    if (max_cells > ((int64_t)1 << 31) - 4) max_cells = ((int64_t)1 << 31) - 4;
    if (max_cells < 125) max_cells = 125;  // a folded axis needs >= 5 cells
    c->sc.max_cells = (uint32_t)max_cells;
    Buffers& b = c->b;
    const size_t C = capacity;
    b.radix_blocks = (int)((C + kRadixTileN - 1) / kRadixTileN);
    const size_t hist_n = (size_t)b.radix_blocks * kRadixBuckets;
    const size_t part_a = (hist_n + kScanTileN - 1) / kScanTileN;
    const size_t part_b = (C + kScanTileN - 1) / kScanTileN;
    b.scan_part_cap = (int)((part_a > part_b ? part_a : part_b) + 1);
    b.diag_blocks = c->L.num_sms * 2;
    if ((rc = dmalloc(&b.pos4, C)) || (rc = dmalloc(&b.vel4, C)) || (rc = dmalloc(&b.pos4_s, C)) ||
        (rc = dmalloc(&b.vel4_s, C)) || (rc = dmalloc(&b.aux4_s, C)) ||
        (rc = dmalloc(&b.acc4_s, C)) || (rc = dmalloc(&b.key[0], C)) ||
        (rc = dmalloc(&b.key[1], C)) || (rc = dmalloc(&b.val[0], C)) ||
        (rc = dmalloc(&b.val[1], C)) || (rc = dmalloc(&b.key_s, C)) ||
        (rc = dmalloc(&b.id_s, C)) || (rc = dmalloc(&b.off, (size_t)max_cells + 2)) ||
        (rc = dmalloc(&b.tile_start, C)) || (rc = dmalloc(&b.hist, hist_n)) ||
        (rc = dmalloc(&b.scan_part, (size_t)b.scan_part_cap)) ||
        (rc = dmalloc(&b.diag_part, (size_t)b.diag_blocks * kDiagSums)) ||
        (rc = dmalloc(&c->ds, 1)) || (rc = dmalloc(&c->stage, 11 * C)))
        return fail(rc);
    if (c->tuning.mode != SPHX_MODE_EXACT &&
        ((rc = dmalloc(&b.cell4, C)) || (rc = dmalloc(&b.cell4_s, C)) ||
         (rc = dmalloc(&b.spread_tiles, C)) ||
         (rc = dmalloc(&b.runs, (size_t)max_cells + 1))))
        return fail(rc);
    // Hit-mask pool (exact mode; the precision mode's sweeps keep no records): 4 records
    // (128 B each) per particle of capacity.  A dense state needs about 1.7-2.6 per particle
    // (32-particle tiles, 27-cell stencil); the rest is slack for the uneven split of tiles
    // over the warps.  Without the pool (or where a warp's region runs out) the force pass
    // repeats the distance tests.
    if (c->tuning.mode == SPHX_MODE_EXACT) {
        if (dmalloc(&b.tile_slot, C) == SPHX_OK) {
            unsigned long long cap = 4ull * C;
            if (cap > 0xffff0000ull) cap = 0xffff0000ull;  // record indices are 32-bit
            if (dmalloc(&b.hitmask, (size_t)cap * 32) == SPHX_OK) {
                b.hitmask_cap = cap;
            } else {
                cudaGetLastError();
                cudaFree(b.tile_slot);
                b.tile_slot = nullptr;
            }
        } else {
            cudaGetLastError();
        }
    }
    if (cudaMemset(c->ds, 0, sizeof(DevState)) != cudaSuccess) return fail(SPHX_ERR_CUDA);
    if (cudaHostAlloc(reinterpret_cast<void**>(&c->h_status), sizeof(int), cudaHostAllocDefault) !=
        cudaSuccess) {
        c->h_status = nullptr;
        return fail(SPHX_ERR_OOM);
    }
    *c->h_status = 0;
    if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_unpacked, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_copied, cudaEventDisableTiming) != cudaSuccess)
        return fail(SPHX_ERR_CUDA);
    if (cudaMemset(b.aux4_s, 0, C * sizeof(float4)) != cudaSuccess ||
        cudaMemset(b.acc4_s, 0, C * sizeof(float4)) != cudaSuccess)
        return fail(SPHX_ERR_CUDA);
    if (c->tuning.profile)
        for (auto& slot : c->prof)
            for (auto& e : slot.ev)
                if (cudaEventCreate(&e) != cudaSuccess) return fail(SPHX_ERR_CUDA);
    *out = c;
    return SPHX_OK;
}

void sphx_destroy(sphx_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
}

int sphx_set_stream(sphx_ctx* c, void* stream) {
    int rc = enter(c);
    if (rc) return rc;
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    c->L.stream = c->stream;
    return SPHX_OK;
}

int sphx_set_params(sphx_ctx* c, const sphx_params* p) {
    int rc = enter(c);
    if (rc) return rc;
    if (!p) return SPHX_ERR_INVALID_ARG;
    const float r = p->neighbor_search_radius;
    if (!(r > 0.0f) || !std::isfinite(r) || !std::isfinite(1.0f / r)) return SPHX_ERR_INVALID_ARG;
    const bool rebin = c->b.cell4 && c->have_params && c->n > 0 &&
                       p->neighbor_search_radius != c->params.neighbor_search_radius;
    if (rebin) {  // precision mode: cells are sized by the search radius -- re-split
        fill_step_const(c);
        double* s64 = reinterpret_cast<double*>(c->stage);
        float* s_mass = c->stage + 9 * c->capacity;
        float* s_vel = c->stage + 6 * c->capacity;
        launch_unpack_cells(c->L, c->sc, (int)c->n, c->b.cell4, c->b.pos4, nullptr, s64);
        launch_unpack_state(c->L, (int)c->n, c->b.pos4, c->b.vel4, nullptr, s_vel);
        k_mass_of<<<c->L.num_sms * 4, 256, 0, c->stream>>>((int)c->n, c->b.pos4, s_mass);
        c->params = *p;
        fill_step_const(c);
        launch_pack_cells(c->L, c->sc, (int)c->n, nullptr, s64, s_vel, s_mass, c->b.cell4,
                          c->b.pos4, c->b.vel4);
        SPHX_CUDA(cudaGetLastError());
        c->have_fields = false;
    }
    c->params = *p;
    c->have_params = true;
    c->version++;
    return SPHX_OK;
}

int sphx_set_kernel(sphx_ctx* c, int kernel) {
    int rc = enter(c);
    if (rc) return rc;
    if (kernel != SPHX_KERNEL_CUBIC_SPLINE && kernel != SPHX_KERNEL_WENDLAND_C2 &&
        kernel != SPHX_KERNEL_GAUSSIAN)
        return SPHX_ERR_INVALID_ARG;
    if (kernel != c->kernel) {
        c->kernel = kernel;
        if (c->nscenes) {  // refresh the scenes' constants, keep their state
            SPHX_CUDA(cudaStreamSynchronize(c->stream));
            std::vector<SceneInfo> info(c->nscenes);
            SPHX_CUDA(cudaMemcpy(info.data(), c->b.scenes, c->nscenes * sizeof(SceneInfo),
                                 cudaMemcpyDeviceToHost));
            for (uint32_t s = 0; s < c->nscenes; ++s)
                fill_step_const_from(c, c->scene_params[s], info[s].count, info[s].c);
            SPHX_CUDA(cudaMemcpy(c->b.scenes, info.data(), c->nscenes * sizeof(SceneInfo),
                                 cudaMemcpyHostToDevice));
        }
        c->have_fields = false;
        c->version++;
    }
    return SPHX_OK;
}

int sphx_get_kernel(sphx_ctx* c, int* kernel) {
    if (!c || !kernel) return SPHX_ERR_INVALID_ARG;
    *kernel = c->kernel;
    return SPHX_OK;
}

int sphx_upload(sphx_ctx* c, size_t n, const float* pos, const float* vel, const float* mass) {
    int rc = enter(c);
    if (rc) return rc;
    if (n > c->capacity) return SPHX_ERR_CAPACITY;
    if (n > 0 && (!pos || !mass)) return SPHX_ERR_INVALID_ARG;
    if (c->b.cell4 && !c->have_params) return SPHX_ERR_NOT_READY;  // cells need the cell size
    float* s_pos = c->stage;
    float* s_vel = c->stage + 3 * c->capacity;
    float* s_mass = c->stage + 6 * c->capacity;
    if (n > 0) {
        // pinned host buffers are read in place by the pack kernel; others are staged
        const float* m_pos = mapped(pos);
        const float* m_vel = mapped(vel);
        const float* m_mass = mapped(mass);
        if (m_pos) s_pos = const_cast<float*>(m_pos);
        else SPHX_CUDA(cudaMemcpyAsync(s_pos, pos, 3 * n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        if (vel) {
            if (m_vel) s_vel = const_cast<float*>(m_vel);
            else SPHX_CUDA(cudaMemcpyAsync(s_vel, vel, 3 * n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        }
        if (m_mass) s_mass = const_cast<float*>(m_mass);
        else SPHX_CUDA(cudaMemcpyAsync(s_mass, mass, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        if (c->b.cell4) {
            fill_step_const(c);
            launch_pack_cells(c->L, c->sc, (int)n, s_pos, nullptr, vel ? s_vel : nullptr, s_mass,
                              c->b.cell4, c->b.pos4, c->b.vel4);
        } else {
            launch_pack(c->L, (int)n, s_pos, vel ? s_vel : nullptr, s_mass, c->b.pos4, c->b.vel4);
        }
        SPHX_CUDA(cudaGetLastError());
    }
    // a captured step graph stays valid for a new particle set of the same size (same
    // buffers, same launch parameters); a size change or dropped scenes invalidate it
    if (n != c->n || c->nscenes) c->version++;
    c->n = n;
    c->have_fields = false;
    c->b.nscenes = 0;  // a new particle set: scenes must be set again
    c->nscenes = 0;
    return SPHX_OK;
}

int sphx_upload_f64(sphx_ctx* c, size_t n, const double* pos, const float* vel,
                    const float* mass) {
    int rc = enter(c);
    if (rc) return rc;
    if (n > c->capacity) return SPHX_ERR_CAPACITY;
    if (n > 0 && (!pos || !mass)) return SPHX_ERR_INVALID_ARG;
    if (c->b.cell4 && !c->have_params) return SPHX_ERR_NOT_READY;  // cells need the cell size
    double* s_pos = reinterpret_cast<double*>(c->stage);              // 6 floats per particle
    float* s_vel = c->stage + 6 * c->capacity;
    float* s_mass = c->stage + 9 * c->capacity;
    float* s_posf = c->stage + 6 * c->capacity;  // exact mode: converted positions (reuse)
    if (n > 0) {
        SPHX_CUDA(cudaMemcpyAsync(s_pos, pos, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        SPHX_CUDA(cudaMemcpyAsync(s_mass, mass, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
        if (c->b.cell4) {
            if (vel)
                SPHX_CUDA(cudaMemcpyAsync(s_vel, vel, 3 * n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
            fill_step_const(c);
            launch_pack_cells(c->L, c->sc, (int)n, nullptr, s_pos, vel ? s_vel : nullptr, s_mass,
                              c->b.cell4, c->b.pos4, c->b.vel4);
        } else {
            k_f64_to_f32<<<c->L.num_sms * 4, 256, 0, c->stream>>>((int)(3 * n), s_pos, s_posf);
            // velocities staged after the conversion, past the converted positions
            float* s_vel2 = reinterpret_cast<float*>(s_pos);  // positions consumed above
            SPHX_CUDA(cudaStreamSynchronize(c->stream));
            if (vel)
                SPHX_CUDA(cudaMemcpyAsync(s_vel2, vel, 3 * n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
            launch_pack(c->L, (int)n, s_posf, vel ? s_vel2 : nullptr, s_mass, c->b.pos4, c->b.vel4);
        }
        SPHX_CUDA(cudaGetLastError());
    }
    // a captured step graph stays valid for a new particle set of the same size (same
    // buffers, same launch parameters); a size change or dropped scenes invalidate it
    if (n != c->n || c->nscenes) c->version++;
    c->n = n;
    c->have_fields = false;
    c->b.nscenes = 0;  // a new particle set: scenes must be set again
    c->nscenes = 0;
    return SPHX_OK;
}

int sphx_size(sphx_ctx* c, size_t* n) {
    if (!c || !n) return SPHX_ERR_INVALID_ARG;
    *n = c->n;
    return SPHX_OK;
}

int sphx_step(sphx_ctx* c, float dt) {
    int rc = enter(c);
    if (rc) return rc;
    if (c->n == 0) return SPHX_OK;  // SPHEngine::step returns when empty (cpp:94)
    if (!c->have_params) return SPHX_ERR_NOT_READY;
    rc = c->tuning.graph ? run_step_graph(c, dt) : run_phases(c, dt, true);
    if (rc) return rc;
    c->steps++;
    c->queries += c->n;
    return SPHX_OK;
}

int sphx_set_scenes(sphx_ctx* c, uint32_t nscenes, const uint64_t* scene_start,
                    const sphx_params* params) {
    int rc = enter(c);
    if (rc) return rc;
    if (nscenes == 0) {
        c->b.nscenes = 0;
        c->nscenes = 0;
        c->version++;
        return SPHX_OK;
    }
    if (!scene_start || !params) return SPHX_ERR_INVALID_ARG;
    if (c->tuning.mode != SPHX_MODE_EXACT) return SPHX_ERR_INVALID_ARG;
    if (scene_start[0] != 0 || scene_start[nscenes] != c->n) return SPHX_ERR_INVALID_ARG;
    for (uint32_t s = 0; s < nscenes; ++s) {
        if (scene_start[s + 1] < scene_start[s]) return SPHX_ERR_INVALID_ARG;
        const float r = params[s].neighbor_search_radius;
        if (!(r > 0.0f) || !std::isfinite(r) || !std::isfinite(1.0f / r)) return SPHX_ERR_INVALID_ARG;
    }
    Buffers& b = c->b;
    if (!b.scene_of) {
        if ((rc = dmalloc(&b.scene_of, c->capacity)) || (rc = dmalloc(&b.scene_s, c->capacity)))
            return rc;
    }
    if (nscenes > c->scene_cap) {
        if (b.scenes) cudaFree(b.scenes);
        b.scenes = nullptr;
        if ((rc = dmalloc(&b.scenes, nscenes))) return rc;
        c->scene_cap = nscenes;
    }
    std::vector<SceneInfo> info(nscenes);
    std::vector<uint32_t> owner(c->n);
    for (uint32_t s = 0; s < nscenes; ++s) {
        SceneInfo& si = info[s];
        std::memset(&si, 0, sizeof(si));
        si.start = (uint32_t)scene_start[s];
        si.count = (uint32_t)(scene_start[s + 1] - scene_start[s]);
        fill_step_const_from(c, params[s], si.count, si.c);
        for (uint64_t i = scene_start[s]; i < scene_start[s + 1]; ++i) owner[i] = s;
    }
    bool all_nz = true;
    for (const SceneInfo& si : info) all_nz = all_nz && si.c.div_nz;
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    SPHX_CUDA(cudaMemcpy(b.scenes, info.data(), nscenes * sizeof(SceneInfo), cudaMemcpyHostToDevice));
    if (c->n) SPHX_CUDA(cudaMemcpy(b.scene_of, owner.data(), c->n * sizeof(uint32_t), cudaMemcpyHostToDevice));
    c->scene_params.assign(params, params + nscenes);
    c->scene_start.assign(scene_start, scene_start + nscenes + 1);
    c->nscenes = nscenes;
    c->scenes_nz = all_nz;
    b.nscenes = (int)nscenes;
    if (!c->have_params) {  // the context-wide parameters default to the first scene's
        c->params = params[0];
        c->have_params = true;
    }
    c->have_fields = false;
    c->version++;
    return SPHX_OK;
}

int sphx_autotune(sphx_ctx* c, float dt, int* warps_per_block, int* blocks_per_sm,
                  float* best_ms) {
    int rc = enter(c);
    if (rc) return rc;
    if (!c->have_params) return SPHX_ERR_NOT_READY;
    if (c->n == 0) return SPHX_OK;
    // save everything a step changes: device state words, scene records, particles
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    DevState ds_save;
    SPHX_CUDA(cudaMemcpy(&ds_save, c->ds, sizeof(DevState), cudaMemcpyDeviceToHost));
    std::vector<SceneInfo> sc_save(c->nscenes);
    if (c->nscenes)
        SPHX_CUDA(cudaMemcpy(sc_save.data(), c->b.scenes, c->nscenes * sizeof(SceneInfo), cudaMemcpyDeviceToHost));
    const bool had_snap = c->snap_pos != nullptr;
    std::vector<float4> keep_pos, keep_vel;
    std::vector<int4> keep_cell;
    if (had_snap) {  // the caller's snapshot must survive: keep it on the host meanwhile
        keep_pos.resize(c->n);
        keep_vel.resize(c->n);
        SPHX_CUDA(cudaMemcpy(keep_pos.data(), c->snap_pos, c->n * sizeof(float4), cudaMemcpyDeviceToHost));
        SPHX_CUDA(cudaMemcpy(keep_vel.data(), c->snap_vel, c->n * sizeof(float4), cudaMemcpyDeviceToHost));
        if (c->snap_cell) {
            keep_cell.resize(c->n);
            SPHX_CUDA(cudaMemcpy(keep_cell.data(), c->snap_cell, c->n * sizeof(int4), cudaMemcpyDeviceToHost));
        }
    }
    if ((rc = sphx_snapshot(c))) return rc;
    const int saved_profile = c->tuning.profile;
    const uint64_t saved_launches = c->launches;
    c->tuning.profile = 0;
    cudaEvent_t e0, e1;
    SPHX_CUDA(cudaEventCreate(&e0));
    SPHX_CUDA(cudaEventCreate(&e1));
    const int cand[][2] = {{4, 0}, {2, 0}, {4, 4}, {4, 2}, {2, 4}, {1, 0}};
    float best = 0.0f;
    int bw = c->L.warps_per_block, bb = c->L.blocks_per_sm;
    auto reset = [&]() -> int {
        SPHX_CUDA(cudaMemcpyAsync(c->ds, &ds_save, sizeof(DevState), cudaMemcpyHostToDevice, c->stream));
        if (c->nscenes)
            SPHX_CUDA(cudaMemcpyAsync(c->b.scenes, sc_save.data(), c->nscenes * sizeof(SceneInfo), cudaMemcpyHostToDevice, c->stream));
        SPHX_CUDA(cudaStreamSynchronize(c->stream));
        return sphx_restore(c);
    };
    for (const auto& cd : cand) {
        c->L.warps_per_block = cd[0];
        c->L.blocks_per_sm = cd[1];
        if ((rc = reset()) || (rc = run_phases(c, dt, true))) break;  // warm-up
        if ((rc = reset())) break;
        SPHX_CUDA(cudaEventRecord(e0, c->stream));
        if ((rc = run_phases(c, dt, true))) break;
        if ((rc = reset())) break;  // identical work for the second timed step
        if ((rc = run_phases(c, dt, true))) break;
        SPHX_CUDA(cudaEventRecord(e1, c->stream));
        SPHX_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        SPHX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (best == 0.0f || ms < best) {
            best = ms;
            bw = cd[0];
            bb = cd[1];
        }
    }
    // then the tile size at the chosen launch shape
    c->L.warps_per_block = bw;
    c->L.blocks_per_sm = bb;
    int bt = c->b.tile_n;
    const int tiles[] = {16, 24};
    for (const int tn : tiles) {
        if (rc) break;
        c->b.tile_n = tn;
        if ((rc = reset()) || (rc = run_phases(c, dt, true))) break;  // warm-up
        if ((rc = reset())) break;
        SPHX_CUDA(cudaEventRecord(e0, c->stream));
        if ((rc = run_phases(c, dt, true))) break;
        if ((rc = reset())) break;
        if ((rc = run_phases(c, dt, true))) break;
        SPHX_CUDA(cudaEventRecord(e1, c->stream));
        SPHX_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        SPHX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            bt = tn;
        }
    }
    c->b.tile_n = bt;
    c->tuning.tile_particles = bt;
    // then the force pass's staging: bulk copies against the lanes' own loads
    int bbulk = c->L.bulk_copy;
    if (!rc && c->tuning.mode == SPHX_MODE_EXACT) {
        c->L.bulk_copy = !bbulk;
        if (!(rc = reset()) && !(rc = run_phases(c, dt, true)) && !(rc = reset())) {
            SPHX_CUDA(cudaEventRecord(e0, c->stream));
            if (!(rc = run_phases(c, dt, true)) && !(rc = reset()) &&
                !(rc = run_phases(c, dt, true))) {
                SPHX_CUDA(cudaEventRecord(e1, c->stream));
                SPHX_CUDA(cudaEventSynchronize(e1));
                float ms = 0.0f;
                SPHX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best) {
                    best = ms;
                    bbulk = c->L.bulk_copy;
                }
            }
        }
    }
    c->L.bulk_copy = bbulk;
    c->tuning.bulk_copy = bbulk;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->L.warps_per_block = bw;
    c->L.blocks_per_sm = bb;
    c->tuning.warps_per_block = bw;
    c->tuning.blocks_per_sm = bb;
    c->tuning.profile = saved_profile;
    c->launches = saved_launches;
    int rc2 = reset();
    if (had_snap) {  // put the caller's snapshot back
        SPHX_CUDA(cudaMemcpy(c->snap_pos, keep_pos.data(), c->n * sizeof(float4), cudaMemcpyHostToDevice));
        SPHX_CUDA(cudaMemcpy(c->snap_vel, keep_vel.data(), c->n * sizeof(float4), cudaMemcpyHostToDevice));
        if (c->snap_cell)
            SPHX_CUDA(cudaMemcpy(c->snap_cell, keep_cell.data(), c->n * sizeof(int4), cudaMemcpyHostToDevice));
    }
    c->have_fields = false;
    c->version++;
    if (warps_per_block) *warps_per_block = bw;
    if (blocks_per_sm) *blocks_per_sm = bb;
    if (best_ms) *best_ms = best / 2.0f;
    return rc ? rc : rc2;
}

int sphx_get_tuning(sphx_ctx* c, sphx_tuning* out) {
    if (!c || !out) return SPHX_ERR_INVALID_ARG;
    *out = c->tuning;
    return SPHX_OK;
}

int sphx_alloc_host(void** out, size_t bytes) {
    if (!out) return SPHX_ERR_INVALID_ARG;
    *out = nullptr;
    if (bytes == 0) return SPHX_ERR_INVALID_ARG;
    if (cudaHostAlloc(out, bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return SPHX_ERR_OOM;
    }
    return SPHX_OK;
}

void sphx_free_host(void* ptr) {
    if (ptr) cudaFreeHost(ptr);
}

int sphx_get_scene_stats(sphx_ctx* c, uint32_t scene, sphx_scene_stats* out) {
    int rc = enter(c);
    if (rc) return rc;
    if (!out || scene >= c->nscenes) return SPHX_ERR_INVALID_ARG;
    rc = refresh_diag(c);
    if (rc) return rc;
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    SceneInfo si;
    SPHX_CUDA(cudaMemcpy(&si, c->b.scenes + scene, sizeof(SceneInfo), cudaMemcpyDeviceToHost));
    std::memset(out, 0, sizeof(*out));
    out->start = si.start;
    out->count = si.count;
    out->current_time = si.time;
    out->last_dt = si.dt;
    out->grid_cells = si.ncells;
    out->sum_mass = si.sums[0];
    out->momentum[0] = si.sums[1];
    out->momentum[1] = si.sums[2];
    out->momentum[2] = si.sums[3];
    out->kinetic_energy = si.sums[4];
    out->potential_energy = si.sums[5];
    return SPHX_OK;
}

int sphx_eval(sphx_ctx* c) {
    int rc = enter(c);
    if (rc) return rc;
    if (c->n == 0) return SPHX_OK;
    if (!c->have_params) return SPHX_ERR_NOT_READY;
    return run_phases(c, 0.0f, false);
}

// Every unpack and copy is enqueued behind the pending work, with the device status word;
// one synchronisation at the end.  Staging (11 floats per particle of capacity C): pos at
// [0, 3C), vel at [3C, 6C), rho at [6C, 7C), P at [7C, 8C), acc at [8C, 11C).
int sphx_download(sphx_ctx* c, float* pos, float* vel, float* rho, float* pressure, float* acc) {
    int rc = enter(c);
    if (rc) return rc;
    const size_t n = c->n;
    if (n == 0) return sync_status(c);
    // outputs go through device staging and the copy engines (on Grace + Blackwell the
    // copy engines write host memory faster than kernel stores over the C2C link do); the
    // copies are split over two streams so that two copy engines run at once
    float* s0 = c->stage;
    float* s1 = c->stage + 3 * c->capacity;
    float* s_rho = c->stage + 6 * c->capacity;
    float* s_p = c->stage + 7 * c->capacity;
    float* s_acc = c->stage + 8 * c->capacity;
    if (pos || vel) {
        launch_unpack_state(c->L, (int)n, c->b.pos4, c->b.vel4,
                            (pos && !c->b.cell4) ? s0 : nullptr, vel ? s1 : nullptr);
        if (pos && c->b.cell4) {
            fill_step_const(c);
            launch_unpack_cells(c->L, c->sc, (int)n, c->b.cell4, c->b.pos4, s0, nullptr);
        }
        SPHX_CUDA(cudaGetLastError());
    }
    if (rho || pressure || acc) {
        if (c->have_fields) {
            launch_unpack_sorted(c->L, (int)n, c->b.id_s, c->b.aux4_s, c->b.acc4_s,
                                 rho ? s_rho : nullptr, pressure ? s_p : nullptr,
                                 acc ? s_acc : nullptr);
            SPHX_CUDA(cudaGetLastError());
        } else {
            SPHX_CUDA(cudaMemsetAsync(s_rho, 0, 5 * c->capacity * sizeof(float), c->stream));
        }
    }
    SPHX_CUDA(cudaEventRecord(c->ev_unpacked, c->stream));
    SPHX_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_unpacked, 0));
    const size_t f = sizeof(float);
    if (pos) SPHX_CUDA(cudaMemcpyAsync(pos, s0, 3 * n * f, cudaMemcpyDeviceToHost, c->stream));
    if (vel) SPHX_CUDA(cudaMemcpyAsync(vel, s1, 3 * n * f, cudaMemcpyDeviceToHost, c->copy_stream));
    if (rho) SPHX_CUDA(cudaMemcpyAsync(rho, s_rho, n * f, cudaMemcpyDeviceToHost, c->stream));
    if (pressure) SPHX_CUDA(cudaMemcpyAsync(pressure, s_p, n * f, cudaMemcpyDeviceToHost, c->copy_stream));
    if (acc) SPHX_CUDA(cudaMemcpyAsync(acc, s_acc, 3 * n * f, cudaMemcpyDeviceToHost, c->copy_stream));
    SPHX_CUDA(cudaEventRecord(c->ev_copied, c->copy_stream));
    SPHX_CUDA(cudaStreamWaitEvent(c->stream, c->ev_copied, 0));
    SPHX_CUDA(cudaMemcpyAsync(c->h_status, c->ds, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    SPHX_CUDA(cudaGetLastError());
    return *c->h_status;  // a failed step's outputs are not to be used
}

int sphx_download_f64(sphx_ctx* c, double* pos_xyz) {
    int rc = enter(c);
    if (rc) return rc;
    if (!pos_xyz) return SPHX_ERR_INVALID_ARG;
    rc = sync_status(c);
    if (rc) return rc;
    const size_t n = c->n;
    if (n == 0) return SPHX_OK;
    double* s = reinterpret_cast<double*>(c->stage);
    if (c->b.cell4) {
        fill_step_const(c);
        launch_unpack_cells(c->L, c->sc, (int)n, c->b.cell4, c->b.pos4, nullptr, s);
    } else {
        float* sf = c->stage + 6 * c->capacity;
        launch_unpack_state(c->L, (int)n, c->b.pos4, c->b.vel4, sf, nullptr);
        k_f32_to_f64<<<c->L.num_sms * 4, 256, 0, c->stream>>>((int)(3 * n), sf, s);
    }
    SPHX_CUDA(cudaGetLastError());
    SPHX_CUDA(cudaMemcpyAsync(pos_xyz, s, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    return SPHX_OK;
}

int sphx_get_time_f64(sphx_ctx* c, double* current_time, double* last_dt) {
    int rc = enter(c);
    if (rc) return rc;
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    DevState s;
    SPHX_CUDA(cudaMemcpy(&s, c->ds, sizeof(DevState), cudaMemcpyDeviceToHost));
    const bool p = c->tuning.mode != SPHX_MODE_EXACT;
    if (current_time) *current_time = p ? s.time64 : (double)s.time;
    if (last_dt) *last_dt = p ? s.dt64 : (double)s.dt;
    return SPHX_OK;
}

int sphx_get_time(sphx_ctx* c, float* current_time, float* last_dt) {
    int rc = enter(c);
    if (rc) return rc;
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    DevState s;
    SPHX_CUDA(cudaMemcpy(&s, c->ds, sizeof(DevState), cudaMemcpyDeviceToHost));
    if (current_time) *current_time = s.time;
    if (last_dt) *last_dt = s.dt;
    return SPHX_OK;
}

int sphx_set_time(sphx_ctx* c, float t) {
    int rc = enter(c);
    if (rc) return rc;
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    SPHX_CUDA(cudaMemcpy(reinterpret_cast<char*>(c->ds) + offsetof(DevState, time), &t,
                         sizeof(float), cudaMemcpyHostToDevice));
    const double t64 = t;
    SPHX_CUDA(cudaMemcpy(reinterpret_cast<char*>(c->ds) + offsetof(DevState, time64), &t64,
                         sizeof(double), cudaMemcpyHostToDevice));
    return SPHX_OK;
}

int sphx_get_stats(sphx_ctx* c, sphx_stats* out) {
    int rc = enter(c);
    if (rc) return rc;
    if (!out) return SPHX_ERR_INVALID_ARG;
    rc = refresh_diag(c);
    if (rc) return rc;
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    rc = drain_all(c);
    if (rc) return rc;
    DevState s;
    SPHX_CUDA(cudaMemcpy(&s, c->ds, sizeof(DevState), cudaMemcpyDeviceToHost));
    std::memset(out, 0, sizeof(*out));
    out->total_time = c->t_total;
    out->neighbor_search_time = c->t_nb;
    out->density_computation_time = c->t_den;
    out->force_computation_time = c->t_force;
    out->integration_time = 0.0;
    out->max_neighbors = s.max_nn;
    out->total_neighbor_queries = c->queries;
    out->steps = c->steps;
    out->current_time = s.time;
    out->last_dt = s.dt;
    out->occupied_cells = s.occupied;
    out->max_cell_occupancy = s.max_occ;
    out->nonfinite_particles = s.nonfinite;
    out->grid_cells = s.ncells;
    out->sum_mass = s.sums[0];
    out->momentum[0] = s.sums[1];
    out->momentum[1] = s.sums[2];
    out->momentum[2] = s.sums[3];
    out->kinetic_energy = s.sums[4];
    out->potential_energy = s.sums[5];
    out->sum_density = s.sums[6];
    out->kernel_launches = c->launches;
    out->tiles = s.n_tiles;
    out->spread_tiles = s.n_spread;
    return s.status;
}

int sphx_reset_stats(sphx_ctx* c) {
    int rc = enter(c);
    if (rc) return rc;
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    rc = drain_all(c);
    if (rc) return rc;
    c->t_total = c->t_nb = c->t_den = c->t_force = 0.0;
    c->queries = 0;
    unsigned long long z = 0;
    SPHX_CUDA(cudaMemcpy(reinterpret_cast<char*>(c->ds) + offsetof(DevState, max_nn), &z,
                         sizeof(z), cudaMemcpyHostToDevice));
    return SPHX_OK;
}

int sphx_snapshot(sphx_ctx* c) {
    int rc = enter(c);
    if (rc) return rc;
    if (!c->snap_pos) {
        if ((rc = dmalloc(&c->snap_pos, c->capacity)) || (rc = dmalloc(&c->snap_vel, c->capacity)))
            return rc;
        if (c->b.cell4 && (rc = dmalloc(&c->snap_cell, c->capacity))) return rc;
    }
    if (c->n) {
        SPHX_CUDA(cudaMemcpyAsync(c->snap_pos, c->b.pos4, c->n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
        SPHX_CUDA(cudaMemcpyAsync(c->snap_vel, c->b.vel4, c->n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
        if (c->b.cell4)
            SPHX_CUDA(cudaMemcpyAsync(c->snap_cell, c->b.cell4, c->n * sizeof(int4), cudaMemcpyDeviceToDevice, c->stream));
    }
    return SPHX_OK;
}

int sphx_restore(sphx_ctx* c) {
    int rc = enter(c);
    if (rc) return rc;
    if (!c->snap_pos) return SPHX_ERR_NOT_READY;
    if (c->n) {
        SPHX_CUDA(cudaMemcpyAsync(c->b.pos4, c->snap_pos, c->n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
        SPHX_CUDA(cudaMemcpyAsync(c->b.vel4, c->snap_vel, c->n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
        if (c->b.cell4)
            SPHX_CUDA(cudaMemcpyAsync(c->b.cell4, c->snap_cell, c->n * sizeof(int4), cudaMemcpyDeviceToDevice, c->stream));
    }
    return SPHX_OK;
}

int sphx_debug_pairs(sphx_ctx* c, int64_t* counts, int64_t* idx, size_t* total_inout) {
    int rc = enter(c);
    if (rc) return rc;
    if (!counts || !total_inout) return SPHX_ERR_INVALID_ARG;
    if (!c->have_params) return SPHX_ERR_NOT_READY;
    const size_t n = c->n;
    if (n == 0) {
        *total_inout = 0;
        return SPHX_OK;
    }
    fill_step_const(c);
    c->have_fields = false;  // the grid rebuild below replaces the sorted permutation
    launch_begin_step(c->L, c->ds, 1);
    // the lists come in the reference's order: insertion order within each cell
    Buffers bq = c->b;
    bq.columns = 0;
    launch_build_grid(c->L, c->sc, bq, c->ds);
    uint32_t* d_cnt = nullptr;
    if ((rc = dmalloc(&d_cnt, n))) return rc;
    launch_pair_counts(c->L, c->sc, bq, c->ds, d_cnt);
    std::vector<uint32_t> h_cnt(n);
    cudaError_t e = cudaMemcpyAsync(h_cnt.data(), d_cnt, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_cnt);
    if (e != cudaSuccess) return cuda_fail(e);
    rc = sync_status(c);
    if (rc) return rc;
    std::vector<uint64_t> off(n);
    uint64_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        counts[i] = h_cnt[i];
        off[i] = total;
        total += h_cnt[i];
    }
    const size_t cap = *total_inout;
    *total_inout = (size_t)total;
    if (!idx) return SPHX_OK;
    if (cap < total) return SPHX_ERR_OVERFLOW;
    uint64_t* d_off = nullptr;
    int64_t* d_out = nullptr;
    if ((rc = dmalloc(&d_off, n))) return rc;
    if ((rc = dmalloc(&d_out, total))) {
        cudaFree(d_off);
        return rc;
    }
    e = cudaMemcpyAsync(d_off, off.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        launch_pair_fill(c->L, c->sc, bq, c->ds, d_off, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(idx, d_out, total * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_off);
    cudaFree(d_out);
    if (e != cudaSuccess) return cuda_fail(e);
    return SPHX_OK;
}

int sphx_debug_pairs_subset(sphx_ctx* c, size_t nsel, const int64_t* sel, int64_t* counts,
                            int64_t* idx, size_t* total_inout) {
    int rc = enter(c);
    if (rc) return rc;
    if ((nsel && (!sel || !counts)) || !total_inout) return SPHX_ERR_INVALID_ARG;
    if (!c->have_params) return SPHX_ERR_NOT_READY;
    const size_t n = c->n;
    for (size_t q = 0; q < nsel; ++q)
        if (sel[q] < 0 || (size_t)sel[q] >= n) return SPHX_ERR_INVALID_ARG;
    if (nsel == 0) {
        *total_inout = 0;
        return SPHX_OK;
    }
    fill_step_const(c);
    c->have_fields = false;  // the grid rebuild below replaces the sorted permutation
    launch_begin_step(c->L, c->ds, 1);
    // the lists come in the reference's order: insertion order within each cell
    Buffers bq = c->b;
    bq.columns = 0;
    launch_build_grid(c->L, c->sc, bq, c->ds);
    uint32_t* d_cnt = nullptr;
    if ((rc = dmalloc(&d_cnt, n))) return rc;
    launch_pair_counts(c->L, c->sc, bq, c->ds, d_cnt);
    std::vector<uint32_t> h_cnt(n);
    cudaError_t e = cudaMemcpyAsync(h_cnt.data(), d_cnt, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_cnt);
    if (e != cudaSuccess) return cuda_fail(e);
    rc = sync_status(c);
    if (rc) return rc;
    // each distinct selected particle's list once, at off[id]; kNoPairs for the others
    std::vector<uint64_t> off(n, kNoPairs);
    uint64_t uniq_total = 0, total = 0;
    for (size_t q = 0; q < nsel; ++q) {
        const size_t id = (size_t)sel[q];
        counts[q] = h_cnt[id];
        total += h_cnt[id];
        if (off[id] == kNoPairs) {
            off[id] = uniq_total;
            uniq_total += h_cnt[id];
        }
    }
    const size_t cap = *total_inout;
    *total_inout = (size_t)total;
    if (!idx) return SPHX_OK;
    if (cap < total) return SPHX_ERR_OVERFLOW;
    uint64_t* d_off = nullptr;
    int64_t* d_out = nullptr;
    if ((rc = dmalloc(&d_off, n))) return rc;
    if ((rc = dmalloc(&d_out, uniq_total))) {
        cudaFree(d_off);
        return rc;
    }
    std::vector<int64_t> lists(uniq_total ? uniq_total : 1);
    e = cudaMemcpyAsync(d_off, off.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        launch_pair_fill(c->L, c->sc, bq, c->ds, d_off, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && uniq_total)
        e = cudaMemcpyAsync(lists.data(), d_out, uniq_total * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d_off);
    cudaFree(d_out);
    if (e != cudaSuccess) return cuda_fail(e);
    uint64_t at = 0;
    for (size_t q = 0; q < nsel; ++q) {
        const size_t id = (size_t)sel[q];
        std::memcpy(idx + at, lists.data() + off[id], h_cnt[id] * sizeof(int64_t));
        at += h_cnt[id];
    }
    return SPHX_OK;
}

void sphx_camera_matrices(const float position[3], float yaw_deg, float pitch_deg,
                          float fov_deg, float aspect, float view[16], float projection[16]) {
    const float rad = 0.01745329251994329577f;
    auto normalize = [](float v[3]) {
        const float l = std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
        for (int a = 0; a < 3; ++a) v[a] = v[a] / l;
    };
    auto cross = [](const float a[3], const float b[3], float o[3]) {
        o[0] = a[1] * b[2] - b[1] * a[2];
        o[1] = a[2] * b[0] - b[2] * a[0];
        o[2] = a[0] * b[1] - b[0] * a[1];
    };
    const float yaw = yaw_deg * rad, pitch = pitch_deg * rad;
    float front[3] = {std::cos(yaw) * std::cos(pitch), std::sin(pitch),
                      std::sin(yaw) * std::cos(pitch)};
    normalize(front);
    const float world_up[3] = {0.0f, 1.0f, 0.0f};
    float right[3], up[3];
    cross(front, world_up, right);
    normalize(right);
    cross(right, front, up);
    normalize(up);
    // look-at from position towards position + front: s = normalize(f x up), u = s x f
    float f[3] = {front[0], front[1], front[2]};
    normalize(f);
    float sv[3], u[3];
    cross(f, up, sv);
    normalize(sv);
    cross(sv, f, u);
    const float* e = position;
    for (int k = 0; k < 16; ++k) view[k] = (k % 5 == 0) ? 1.0f : 0.0f;
    for (int a = 0; a < 3; ++a) {
        view[a * 4 + 0] = sv[a];
        view[a * 4 + 1] = u[a];
        view[a * 4 + 2] = -f[a];
    }
    view[12] = -((sv[0] * e[0] + sv[1] * e[1]) + sv[2] * e[2]);
    view[13] = -((u[0] * e[0] + u[1] * e[1]) + u[2] * e[2]);
    view[14] = (f[0] * e[0] + f[1] * e[1]) + f[2] * e[2];
    // perspective, depth mapped to [-1, 1] (near 0.1, far 100)
    const float zn = 0.1f, zf = 100.0f;
    const float t = std::tan(fov_deg * rad / 2.0f);
    for (int k = 0; k < 16; ++k) projection[k] = 0.0f;
    projection[0] = 1.0f / (aspect * t);
    projection[5] = 1.0f / t;
    projection[10] = -(zf + zn) / (zf - zn);
    projection[11] = -1.0f;
    projection[14] = -(2.0f * zf * zn) / (zf - zn);
}

int sphx_render_instances_device(sphx_ctx* c, const sphx_render_params* p,
                                 const float* colors_dev, float* instances_dev) {
    int rc = enter(c);
    if (rc) return rc;
    RenderConst r;
    if ((rc = render_const(p, r))) return rc;
    if (c->n > 0 && !instances_dev) return SPHX_ERR_INVALID_ARG;
    c->launches += launch_render_instances(c->L, r, render_args(c, colors_dev), instances_dev);
    SPHX_CUDA(cudaGetLastError());
    return SPHX_OK;
}

int sphx_render_instances(sphx_ctx* c, const sphx_render_params* p, const float* colors,
                          float* instances) {
    int rc = enter(c);
    if (rc) return rc;
    RenderConst r;
    if ((rc = render_const(p, r))) return rc;
    if (c->n == 0) return SPHX_OK;
    if (!instances) return SPHX_ERR_INVALID_ARG;
    if ((rc = render_buffers(c, 0))) return rc;
    if (colors)
        SPHX_CUDA(cudaMemcpyAsync(c->r_colors, colors, 3 * c->n * sizeof(float),
                                  cudaMemcpyHostToDevice, c->stream));
    c->launches += launch_render_instances(c->L, r, render_args(c, colors ? c->r_colors : nullptr),
                                           c->r_inst);
    SPHX_CUDA(cudaGetLastError());
    SPHX_CUDA(cudaMemcpyAsync(instances, c->r_inst, 20 * c->n * sizeof(float),
                              cudaMemcpyDeviceToHost, c->stream));
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    return SPHX_OK;
}

int sphx_render_image_device(sphx_ctx* c, const sphx_render_params* p, const float* colors_dev,
                             unsigned char* rgba_dev) {
    int rc = enter(c);
    if (rc) return rc;
    RenderConst r;
    if ((rc = render_const(p, r))) return rc;
    if (!rgba_dev) return SPHX_ERR_INVALID_ARG;
    const size_t npix = (size_t)p->width * p->height;
    if ((rc = render_buffers(c, npix))) return rc;
    c->launches += launch_render_image(c->L, r, render_args(c, colors_dev), c->r_keys,
                                       reinterpret_cast<uchar4*>(rgba_dev));
    SPHX_CUDA(cudaGetLastError());
    return SPHX_OK;
}

int sphx_render_image(sphx_ctx* c, const sphx_render_params* p, const float* colors,
                      unsigned char* rgba) {
    int rc = enter(c);
    if (rc) return rc;
    RenderConst r;
    if ((rc = render_const(p, r))) return rc;
    if (!rgba) return SPHX_ERR_INVALID_ARG;
    const size_t npix = (size_t)p->width * p->height;
    if ((rc = render_buffers(c, npix))) return rc;
    if (colors && c->n)
        SPHX_CUDA(cudaMemcpyAsync(c->r_colors, colors, 3 * c->n * sizeof(float),
                                  cudaMemcpyHostToDevice, c->stream));
    c->launches += launch_render_image(c->L, r, render_args(c, colors ? c->r_colors : nullptr),
                                       c->r_keys, c->r_rgba);
    SPHX_CUDA(cudaGetLastError());
    SPHX_CUDA(cudaMemcpyAsync(rgba, c->r_rgba, npix * 4, cudaMemcpyDeviceToHost, c->stream));
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    return SPHX_OK;
}

int sphx_generate(sphx_ctx* c, size_t nshapes, const sphx_shape* shapes, size_t* n_out) {
    int rc = enter(c);
    if (rc) return rc;
    if (nshapes > 0 && !shapes) return SPHX_ERR_INVALID_ARG;
    if (c->b.cell4 && !c->have_params) return SPHX_ERR_NOT_READY;  // cells need the cell size
    float* s_pos = c->stage;
    float* s_vel = c->stage + 3 * c->capacity;
    float* s_mass = c->stage + 6 * c->capacity;
    std::vector<GenShape> gs(nshapes);
    uint64_t max_rows = 0;
    for (size_t k = 0; k < nshapes; ++k) {
        if ((rc = gen_shape(shapes[k], gs[k]))) return rc;
        if (gs[k].kind == SPHX_SHAPE_SPHERE || gs[k].kind == SPHX_SHAPE_BALL)
            max_rows = std::max<uint64_t>(max_rows, (uint64_t)gs[k].n[0] * gs[k].n[1]);
    }
    uint32_t* rows = nullptr;
    if (max_rows && (rc = dmalloc(&rows, (size_t)max_rows + 1))) return rc;
    uint64_t total = 0;
    for (size_t k = 0; k < nshapes && !rc; ++k) {
        GenArgs g{gs[k], s_pos, s_vel, s_mass};
        const bool ball = g.s.kind == SPHX_SHAPE_SPHERE || g.s.kind == SPHX_SHAPE_BALL;
        if (ball) {
            const uint32_t nrows = (uint32_t)g.s.n[0] * (uint32_t)g.s.n[1];
            uint32_t cnt = 0;
            if (nrows) {
                launch_ball_count(c->L, g, rows);
                cudaError_t e = cudaMemcpyAsync(&cnt, rows + nrows, sizeof(uint32_t),
                                                cudaMemcpyDeviceToHost, c->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
                if (e != cudaSuccess) rc = cuda_fail(e);
            }
            g.s.count = cnt;
        }
        if (rc) break;
        if (total + g.s.count > c->capacity) {
            rc = SPHX_ERR_CAPACITY;
            break;
        }
        g.s.offset = (uint32_t)total;
        if (g.s.count) launch_generate(c->L, g, rows);
        total += g.s.count;
    }
    if (!rc) {
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e);
    }
    if (rows) {
        cudaStreamSynchronize(c->stream);
        cudaFree(rows);
    }
    if (rc) return rc;
    const size_t n = (size_t)total;
    if (n > 0) {
        if (c->b.cell4) {
            fill_step_const(c);
            launch_pack_cells(c->L, c->sc, (int)n, s_pos, nullptr, s_vel, s_mass, c->b.cell4,
                              c->b.pos4, c->b.vel4);
        } else {
            launch_pack(c->L, (int)n, s_pos, s_vel, s_mass, c->b.pos4, c->b.vel4);
        }
        SPHX_CUDA(cudaGetLastError());
    }
    c->n = n;
    c->have_fields = false;
    c->b.nscenes = 0;
    c->nscenes = 0;
    c->version++;
    if (n_out) *n_out = n;
    return SPHX_OK;
}

int sphx_generate_scene(sphx_ctx* c, int scene, float particle_mass, size_t* n_out) {
    sphx_shape sh[2];
    std::memset(sh, 0, sizeof(sh));
    auto set3 = [](float* d, float x, float y, float z) { d[0] = x, d[1] = y, d[2] = z; };
    size_t ns = 0;
    if (scene == SPHX_SCENE_DAM_BREAK) {
        // create_dam_break_setup(dam (0.4, 0.6, 0.8), fluid (0.2, 0.4, 0.8), 0.01)
        const float dam[3] = {0.4f, 0.6f, 0.8f}, fluid[3] = {0.2f, 0.4f, 0.8f}, sp = 0.01f;
        sh[0].kind = SPHX_SHAPE_BOX;
        set3(sh[0].center, 0.0f, dam[1] / 2.0f, 0.0f);
        set3(sh[0].size, dam[0], dam[1], dam[2]);
        sh[1].kind = SPHX_SHAPE_BLOCK;
        set3(sh[1].center, -dam[0] / 2.0f + fluid[0] / 2.0f, fluid[1] / 2.0f, 0.0f);
        set3(sh[1].size, fluid[0], fluid[1], fluid[2]);
        sh[0].spacing = sh[1].spacing = sp;
        ns = 2;
    } else if (scene == SPHX_SCENE_FLUID_DROP) {
        // create_fluid_drop_setup(centre (0, 0.5, 0), radius 0.1, spacing 0.008)
        sh[0].kind = SPHX_SHAPE_SPHERE;
        set3(sh[0].center, 0.0f, 0.5f, 0.0f);
        sh[0].size[0] = 0.1f;
        sh[0].spacing = 0.008f;
        ns = 1;
    } else if (scene == SPHX_SCENE_GRANULAR_FLOW) {
        // create_granular_flow_setup(pile (0.3, 0.4, 0.8), domain (1, 1, 1), 0.012)
        const float pile[3] = {0.3f, 0.4f, 0.8f}, dom[3] = {1.0f, 1.0f, 1.0f}, sp = 0.012f;
        sh[0].kind = SPHX_SHAPE_BOX;
        set3(sh[0].center, 0.0f, dom[1] / 2.0f, 0.0f);
        set3(sh[0].size, dom[0], dom[1], dom[2]);
        sh[1].kind = SPHX_SHAPE_BLOCK;
        set3(sh[1].center, 0.0f, pile[1] / 2.0f + sp, 0.0f);
        set3(sh[1].size, pile[0], pile[1], pile[2]);
        sh[0].spacing = sh[1].spacing = sp;
        ns = 2;
    } else {
        return SPHX_ERR_INVALID_ARG;
    }
    for (size_t k = 0; k < ns; ++k) sh[k].mass = particle_mass;
    return sphx_generate(c, ns, sh, n_out);
}

}  // extern "C"
