// Internal declarations of the sm_103a SPH step: device-resident state, per-step
// constants, exact-arithmetic helpers and the launch wrappers shared by the .cu files.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sphx.h"

namespace sphx {

constexpr int kWarp = 32;
constexpr int kTile = 32;              // particles of one cell handled by one warp
constexpr int kRadixBits = 8;
constexpr int kRadixBuckets = 1 << kRadixBits;
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 16;
constexpr int kRadixTileN = kRadixThreads * kRadixItems;  // keys per radix block
constexpr int kMaxPasses = 4;                             // 32-bit keys
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTileN = kScanThreads * kScanItems;
constexpr int kDiagThreads = 256;
constexpr int kDiagSums = 8;
constexpr int kCellClamp = 1 << 30;    // |cell coordinate| clamp for finite positions

// Constants of one step, computed on the host in float exactly as the reference does
// (SpatialHash::set_cell_size, spatial_hash.h:63-66; CubicSplineKernel ctor,
// kernels.cpp:12-14, 23-36) and passed to the kernels by value.
struct StepConst {
    int n;                 // particles loaded
    float inv_cell;        // 1.0f / neighbor_search_radius
    float r2;              // neighbor_search_radius * neighbor_search_radius
    float h, h_sq, sigma;  // kernel constants
    float w0;              // W(vec3(0)) -- the self term factor
    float rest, gas, visc, grav, damping, cfl, timestep;
    float lo[3], hi[3];    // box
    uint32_t max_cells;    // capacity of the dense cell grid
    // precision mode (positions = integer cell + FP32 in-cell offset)
    int precise;           // 1: cell + offset storage, compensated sums, FP64 CFL/time
    int fp16;              // 1: offsets rounded to binary16 at every write
    float cs;              // cell size of the storage and of the search grid (= r_search)
    double cs_d;           // the same, as double
    // division by the fixed divisors h and h*h (see xdiv_fixed)
    float rcp_h, rcp_hsq;  // RN(1/h), RN(1/h^2)
    // the precision sweeps' units (lengths in units of h), read from the kernel parameters
    // rather than held in registers: cs / h, r^2 / h^2, the same with the box cull's margin,
    // (1e-6 m / h)^2
    float sw_cs, sw_r2, sw_r2m, sw_skip2;
    int fast_div_h, fast_div_hsq;  // 1: the one-correction sequence is verified for it
    // smoothing kernel (SPHX_KERNEL_*) and the constants its constructor computes in float
    int kern;
    float wnorm;  // Wendland norm_factor_ 21/(2 pi h^3); Gaussian norm_ 1/(pi h^2)^1.5
    float wl;     // Wendland norm_factor_ * (5 / h_sq)
    float gs;     // Gaussian sigma_sq_inv_ = 1 / (h h)
    float gg;     // Gaussian -2 sigma_sq_inv_ norm_
    float gl;     // Gaussian 2 sigma_sq_inv_ norm_
    float g2s;    // Gaussian 2 sigma_sq_inv_
    int div_nz;   // 1: the cubic passes' dividends are in xdiv_fixed_nz's range by bounds
};

// Device-resident scalars written and read by the kernels of a step.
struct DevState {
    int status;                 // 0 or SPHX_ERR_* raised on the device
    int cmin[3], cmax[3];       // box of occupied cells (finite particles)
    int dim[3];                 // grid extent in cells per axis
    int wrap[3];                // 1: the axis is folded (cell index taken modulo dim)
    uint32_t ncells;            // dim product; also the key of non-finite particles
    uint32_t passes;            // radix passes needed this step
    uint32_t n_tiles;           // warp work items
    uint32_t nonfinite;         // particles with a NaN/inf coordinate
    uint32_t vmax_bits;         // max |v| (float bits) for the CFL rule
    uint32_t occupied;          // occupied cells
    uint32_t max_occ;           // particles in the fullest cell
    uint32_t work[2];           // tile counters of the density and force passes
    float dt;                   // dt of the current step
    float time;                 // current_time_
    float a0[4];                // accelerations_[0] (persists across steps)
    unsigned long long max_nn;  // max |N(i)| since the last stats reset
    double sums[kDiagSums];     // FP64 diagnostics of the state after the last step
    double dt64, time64;        // precision mode: dt and current time in FP64
    unsigned long long vmax64;  // precision mode: max |v| (FP64 bits)
    uint32_t n_spread;          // precision mode: spread tiles listed this step
    uint32_t spread_work[2];    // precision mode: tile counters of the spread-tile kernels
};

// Batched mode: one record per scene (device memory).  Scenes are contiguous ranges of
// the insertion order; each owns a dense block of grid cells starting at `base`.
struct SceneInfo {
    StepConst c;                // the scene's parameters and constants (c.n = count)
    uint32_t start, count;      // particle range in insertion order
    int cmin[3], cmax[3];       // box of occupied cells
    int dim[3];                 // grid extent of the scene
    uint32_t base, ncells;      // first grid cell, number of cells
    uint32_t nonfinite;
    uint32_t vmax_bits;
    float dt, time;             // the scene's dt of the current step and current_time_
    float a0[4];                // acceleration of the scene's first particle
    double sums[kDiagSums];     // FP64 diagnostics of the scene after the last step
};

// Grid geometry of one tile: the whole grid (single scene) or the tile's scene block.
struct Geom {
    int dim[3];
    int wrap[3];
    uint32_t base;      // first cell of the block
    uint32_t sentinel;  // key of the non-finite group (total number of cells)
};

struct Buffers {
    float4* pos4;     // insertion order: x, y, z, mass
    float4* vel4;     // insertion order: vx, vy, vz, 0
    float4* pos4_s;   // cell-sorted copies
    float4* vel4_s;
    float4* aux4_s;   // cell-sorted: rho, P, 2*rho, mass/rho
    float4* acc4_s;   // cell-sorted accelerations of the last step/eval
    int4* cell4;      // precision mode, insertion order: cell (x, y, z), w = 1 if not finite
    int4* cell4_s;    // precision mode, cell-sorted copy
    uint32_t* key[2]; // radix ping-pong
    uint32_t* val[2];
    uint32_t* key_s;  // sorted cell keys
    uint32_t* id_s;   // sorted position -> insertion index
    uint32_t* off;    // dense cell grid: first sorted position of each cell (max_cells + 2)
    uint32_t* tile_start;
    uint32_t* hist;   // radix histograms / offsets
    uint32_t* scan_part;
    double* diag_part;
    uint32_t* scene_of;  // batched mode: scene of each particle (insertion order)
    uint32_t* scene_s;   // batched mode: scene of each particle (cell-sorted)
    SceneInfo* scenes;   // batched mode: per-scene records
    int nscenes;         // 0: single scene
    // Hit masks of the density pass, reused by the force pass of the same step: record r
    // holds 32 words (word = lane: bit j set if candidate j of the chunk is within r of the
    // lane's particle).  Every warp of the density grid owns an equal region of the pool
    // and stores its tiles' records one after another, one record per chunk of the tile's
    // walk; tile_slot[t] = first record, or kNoSlot when the tile did not fit in what was
    // left of the region (the force pass then repeats the distance tests for that tile).
    uint32_t* hitmask = nullptr;
    uint32_t* tile_slot = nullptr;
    unsigned long long hitmask_cap = 0;  // records
    int radix_blocks;
    int scan_part_cap;
    int diag_blocks;
    int tile_n = kTile;  // particles per warp work item (1 .. kTile)
    // 1 (precision-mode step): each cell's particles are put in z order after the sort and
    // the tiles run along cell columns (x, y, *), spanning cells; 0: the reference's
    // insertion order within each cell and tiles within one cell
    int columns = 0;
    // precision mode: the tiles whose particles lie in cells far apart (listed by the density
    // sweep, swept by the spread-tile kernels), one entry per tile at most
    uint32_t* spread_tiles = nullptr;
    // precision mode, single scene (max_cells + 1): per cell, the sorted positions where its
    // column run -- the stretch of its column that one sequence of tiles fills
    // (k_column_runs) -- starts and ends; null: runs are whole columns
    uint2* runs = nullptr;
};
// A column run ends before cell z when z is a multiple of kRunAlign and the kRunWindow
// cells below z hold fewer particles than a tile: no tile of a run then reaches more than
// kRunCells = kRunWindow + kRunAlign - 1 cells past its first one (k_column_runs).
constexpr int kRunWindow = 2, kRunAlign = 3;
constexpr int kRunCells = kRunWindow + kRunAlign - 1;
constexpr uint32_t kNoSlot = 0xffffffffu;
constexpr uint64_t kNoPairs = ~0ull;  // pair fill: this particle's list is not wanted

// Device generation of initial conditions (sphx_gen.cu): one shape, its constants derived
// on the host with the generator's float operations.
struct GenShape {
    int kind;                 // SPHX_SHAPE_*
    uint32_t offset, count;   // first staged particle; particles (balls: after counting)
    float start[3], center[3], r2, spacing, mass, vel[3];
    int n[3];                 // lattice extents (balls: points per axis of the cube)
    uint32_t face_off[7];     // box: first particle of each face
    int face_n2[6];
    int face_a[6][3];         // box: (axis1, axis2, axis3) per face
    float face_val[6];
    float jitter;             // benchmark lattice
    uint64_t seed;
    float origin[3];
    int has_origin;
    double c64[3], sp64, R2;  // FP64 ball
    int kmax;
};
struct GenArgs {
    GenShape s;
    float* pos;   // staging: 3 floats per particle
    float* vel;
    float* mass;
};

// Headless rendering (sphx_render.cu): the shader pair's uniforms, derived on the host.
struct RenderConst {
    float pvm[16];          // projection * view * model, column-major
    float right[3], up[3];  // camera right / up: rows 0 and 1 of the view matrix
    float size;             // particleSize
    int mode;               // colorMode: 0 velocity, 1 density, 2 pressure, 3 type
    float diffuse;          // max(dot(normal, lightDir), 0) of the fragment shader
    int width, height;      // viewport = image
    float bg[3];            // clear colour
};
struct RenderArgs {
    int n;
    const float4* pos4;   // insertion order (precision mode: in-cell offsets)
    const float4* vel4;
    const int4* cell4;    // precision mode: cells (else null)
    double cs;            // precision mode: cell size
    const float* colors;  // per-particle colour (3 floats) or null (0, 0.5, 1)
};

// ---- exact float arithmetic: IEEE round-to-nearest, never contracted into FMA ---------
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }

// a / b for a fixed divisor b, correctly rounded: q0 = RN(a*y), r = a - q0*b (exact, by
// FMA), q = RN(q0 + r*y) with y = RN(1/b) -- Markstein's FMA correction (as in
// Brisebarre, Muller & Raina, "Accelerating correctly rounded floating-point division
// when the divisor is known in advance", IEEE TC 53(8), 2004).  The host verifies the
// sequence for the divisor against IEEE division over every dividend significand of one
// binade (`verified`); the sequence commutes with power-of-two scaling while every
// intermediate stays normal, which |a| in [2^-60, 2^60] and b in [2^-20, 2^20] ensure.
// Anything else (zero, subnormal, huge, NaN/inf dividend, unverified divisor) takes the
// IEEE division.
__device__ __forceinline__ float xdiv_fixed(float a, float b, float y, int verified) {
    const float aa = fabsf(a);
    if (verified && aa >= 0x1p-60f && aa <= 0x1p60f) {
        const float q0 = __fmul_rn(a, y);
        const float r = __fmaf_rn(-q0, b, a);
        return __fmaf_rn(r, y, q0);
    }
    return __fdiv_rn(a, b);
}

// xdiv_fixed without the range test, for dividends known to be +-0 or of magnitude in
// [2^-100, 2^100] with a verified divisor b in [2^-20, 2^20].  In that range q0 and the
// quotient are normal and the residual r is exact (a multiple of 2^(e_a - 46) >= 2^-146,
// at most about 2^-22 |a|), so the sequence scales exactly with powers of two of a and
// the verification on one binade covers every binade.  A zero dividend gives +0 whatever
// its sign; the callers whose dividend can be -0 restore the sign (xsign).
__device__ __forceinline__ float xdiv_fixed_nz(float a, float b, float y) {
    const float q0 = __fmul_rn(a, y);
    const float r = __fmaf_rn(-q0, b, a);
    return __fmaf_rn(r, y, q0);
}

// q with the sign bit of a (q = a / b for b > 0: only a zero quotient can lose it)
__device__ __forceinline__ float xsign(float q, float a) {
    return __int_as_float((__float_as_int(q) & 0x7fffffff) | (__float_as_int(a) & (int)0x80000000));
}

// Packed FP32 pairs (Blackwell f32x2 instructions): two IEEE round-to-nearest operations in
// one instruction, each element rounded exactly as the scalar __f*_rn would.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 upk2(f32x2 v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ f32x2 xsub2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 xmul2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 xadd2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ f32x2 xfma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// xdiv_fixed of a pair of dividends: the one-correction sequence with packed FP32 pairs
// when both dividends are in its range (-b is passed pre-negated: fma(q0, -b, a) is the
// exact a - q0 b), else element by element.
__device__ __forceinline__ f32x2 xdiv_fixed2(f32x2 a2, float b, float y, int verified) {
    const float2 a = upk2(a2);
    const float ax = fabsf(a.x), ay = fabsf(a.y);
    if (verified && ax >= 0x1p-60f && ax <= 0x1p60f && ay >= 0x1p-60f && ay <= 0x1p60f) {
        const f32x2 y2 = pk2(y, y);
        const f32x2 q0 = xmul2(a2, y2);
        const f32x2 r = xfma2(q0, pk2(-b, -b), a2);
        return xfma2(r, y2, q0);
    }
    return pk2(xdiv_fixed(a.x, b, y, verified), xdiv_fixed(a.y, b, y, verified));
}

// xdiv_fixed_nz of a pair of dividends, signs restored
__device__ __forceinline__ f32x2 xdiv_fixed2_nz(f32x2 a2, float b, float y) {
    const f32x2 y2 = pk2(y, y);
    const f32x2 q0 = xmul2(a2, y2);
    const f32x2 r = xfma2(q0, pk2(-b, -b), a2);
    const f32x2 q = xfma2(r, y2, q0);
    return (q & 0x7fffffff7fffffffull) | (a2 & 0x8000000080000000ull);
}

// glm::dot(v, v) = (x*x + y*y) + z*z (products rounded first)
__device__ __forceinline__ float xdot3(float x, float y, float z) {
    return xadd(xadd(xmul(x, x), xmul(y, y)), xmul(z, z));
}

// float(2)/float(3) and float(1)/float(6), the constants the reference folds at compile
// time in W_3d (kernels.cpp:58-66)
constexpr float kTwoThirds = 0x1.555556p-1f;
constexpr float kOneSixth = 0x1.555556p-3f;

// CubicSplineKernel::W_3d (kernels.cpp:58-66).  Both branches are evaluated and one is
// selected: the lanes of a warp hold q on both sides of 1, so a branch would run both
// paths anyway, plus the divergence handling.
__device__ __forceinline__ float cubic_w(const StepConst& c, float q) {
    const float w1 =
        xmul(c.sigma, xadd(xsub(kTwoThirds, xmul(q, q)), xmul(xmul(xmul(0.5f, q), q), q)));
    const float tmp = xsub(2.0f, q);
    const float w2 = xmul(c.sigma, xmul(xmul(xmul(kOneSixth, tmp), tmp), tmp));
    return (q >= 0.0f && q <= 1.0f) ? w1 : ((q > 1.0f && q <= 2.0f) ? w2 : 0.0f);
}

// scalar factor of CubicSplineKernel::gradW_3d (kernels.cpp:96-108):
// grad = factor * (r / |r|) / h ; r_len >= 1e-6 is the caller's business.  Branch-free
// like cubic_w.
__device__ __forceinline__ float cubic_grad_factor(const StepConst& c, float q) {
    const float f1 = xmul(c.sigma, xadd(xmul(-2.0f, q), xmul(xmul(1.5f, q), q)));
    const float tmp = xsub(2.0f, q);
    const float f2 = xmul(-c.sigma, xmul(xmul(0.5f, tmp), tmp));
    return (q >= 0.0f && q <= 1.0f) ? f1 : ((q > 1.0f && q <= 2.0f) ? f2 : 0.0f);
}

// CubicSplineKernel::laplacianW_3d (kernels.cpp:130-138).  The branch picks the
// numerator, one division follows: lanes of a warp hold q on both sides of 1, and a
// division per branch would run twice.  Outside both ranges (and for NaN q) the numerator
// is 0 and 0 / h_sq = +0, the reference's 0.0f.
template <bool kNZ = false>
__device__ __forceinline__ float cubic_lap(const StepConst& c, float q) {
    const float a = (q > 1.0f) ? xsub(2.0f, q) : xadd(-2.0f, xmul(3.0f, q));
    const bool in = (q >= 0.0f && q <= 1.0f) || (q > 1.0f && q <= 2.0f);
    const float num = in ? xmul(c.sigma, a) : 0.0f;
    // kNZ: a is 0 or at least 2^-23 in magnitude (2 - q and 3q - 2 are exact multiples of
    // ulp(q) or of ulp(3q)), so num is +0 or in [sigma 2^-24, 2 sigma], inside
    // xdiv_fixed_nz's range for the sigma the host admits
    return kNZ ? xdiv_fixed_nz(num, c.h_sq, c.rcp_hsq)
               : xdiv_fixed(num, c.h_sq, c.rcp_hsq, c.fast_div_hsq);
}

// WendlandC2Kernel::W after q = length(r)/h (kernels.cpp:172-178):
// norm * tmp^4 * (2q + 1), tmp = 1 - q/2, 0 for q >= 2
__device__ __forceinline__ float wendland_w(const StepConst& c, float q) {
    if (q >= 2.0f) return 0.0f;
    const float tmp = xsub(1.0f, xmul(0.5f, q));
    return xmul(xmul(xmul(xmul(xmul(c.wnorm, tmp), tmp), tmp), tmp), xadd(xmul(2.0f, q), 1.0f));
}

// WendlandC2Kernel::laplacianW after q (kernels.cpp:194-200):
// norm * (5 / h_sq) * tmp * tmp * (5q - 3), 0 for q >= 2
__device__ __forceinline__ float wendland_lap(const StepConst& c, float q) {
    if (q >= 2.0f) return 0.0f;
    const float tmp = xsub(1.0f, xmul(0.5f, q));
    return xmul(xmul(xmul(c.wl, tmp), tmp), xsub(xmul(5.0f, q), 3.0f));
}

__device__ __forceinline__ bool finite3(float x, float y, float z) {
    return isfinite(x) && isfinite(y) && isfinite(z);
}

// Cell coordinate of one axis: floor(x * inv_cell) as SpatialHash::get_grid_coords
// computes it (spatial_hash.h:30-36), clamped to +-2^30 so that every finite position
// has a well-defined cell (clamping keeps neighbouring cells neighbouring).
__device__ __forceinline__ int cell_coord(float x, float inv_cell) {
    float f = floorf(xmul(x, inv_cell));
    f = fminf(fmaxf(f, -(float)kCellClamp), (float)(kCellClamp - 1));
    return (int)f;
}

// ---- bulk copies (cp.async.bulk: the TMA unit's 1-D form) and mbarriers ----------------
// A warp stages a contiguous range of a cell-sorted array into its shared memory with one
// bulk copy per array, completed on an mbarrier (one arrival: the issuing lane's
// arrive.expect_tx with the byte count).  Source and destination 16-byte aligned, size a
// multiple of 16 bytes: whole float4 elements of cudaMalloc'd arrays.  The threads only
// read the staged buffers; a buffer is reused once every lane has passed a __syncwarp
// after its last read.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(arrivals)
                 : "memory");
}
// makes mbarrier initialisation visible to the bulk-copy (async) proxy
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier shared-memory accesses before later async-proxy accesses
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
            smem_u32(bar)),
        "r"(bytes)
        : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_test_parity(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase `parity` of bar to complete, giving up after kMbarWaitLimit polls
// (each poll may suspend the thread for a short, hardware-defined time): false = gave up.
constexpr uint32_t kMbarWaitLimit = 1u << 20;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t it = 0; it < kMbarWaitLimit; ++it)
        if (mbar_test_parity(bar, parity)) return true;
    return false;
}

// ---- precision mode helpers ----------------------------------------------------------

// Neumaier's compensated summation (Neumaier 1974): sum + running correction.
struct KSum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float t = s + x;
        if (fabsf(s) >= fabsf(x)) c += (s - t) + x;
        else c += (x - t) + s;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s + c; }
};

__device__ __forceinline__ float round_half(float x) { return __half2float(__float2half_rn(x)); }

// ---- host-side constants -------------------------------------------------------------
// The StepConst of one parameter block, for `n` particles, smoothing kernel `kernel`
// (SPHX_KERNEL_*) and mode `mode` (SPHX_MODE_*): every constant computed with the
// reference's float operations, the fixed-divisor checks run (cached per divisor).
void step_const_from_params(const sphx_params& p, size_t n, int kernel, int mode,
                            uint32_t max_cells, StepConst& s);

// ---- launch wrappers (host) --------------------------------------------------------
struct LaunchCtx {
    cudaStream_t stream;
    int device;  // CUDA device the launches go to (keys per-device launch-shape caches)
    int num_sms;
    int warps_per_block;
    int blocks_per_sm;
    int bulk_copy;  // 1: the force pass stages candidates with bulk copies (exact mode)
};

int launch_begin_step(const LaunchCtx& L, DevState* ds, int reset_bbox);
int launch_cfl(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds,
                float host_dt);
int launch_build_grid(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                       DevState* ds);
// cs: the precision mode's cell size (the in-cell z order of b.columns; else unused)
int launch_grid_sort(const LaunchCtx& L, const Buffers& b, DevState* ds, int n, float cs);
int launch_density(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds);
int launch_force(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds,
                  int integrate);
int launch_diag(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds);
// precision mode (single scene): the tile-sweep passes (sphx_sweep.cu)
int launch_density_sweep(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                         DevState* ds);
int launch_force_sweep(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds,
                       int integrate);
void launch_pair_counts(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                        DevState* ds, uint32_t* counts_by_id);
void launch_pair_fill(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                      DevState* ds, const uint64_t* offsets_by_id, int64_t* out_idx);

// batched mode (sphx_batch.cu)
int launch_batch_begin(const LaunchCtx& L, const Buffers& b, DevState* ds);
int launch_batch_cfl(const LaunchCtx& L, const Buffers& b, DevState* ds, int n, float host_dt);
int launch_batch_grid(const LaunchCtx& L, const Buffers& b, DevState* ds, int n,
                      uint32_t max_cells);
int launch_batch_diag(const LaunchCtx& L, const Buffers& b, DevState* ds);

// radix sort + scan (sphx_sort.cu)
int launch_radix_sort(const LaunchCtx& L, const Buffers& b, DevState* ds, int n);
int launch_tile_scan(const LaunchCtx& L, const Buffers& b, DevState* ds, int n);

// io (sphx_grid.cu)
void launch_pack(const LaunchCtx& L, int n, const float* pos3, const float* vel3,
                 const float* mass, float4* pos4, float4* vel4);
void launch_unpack_state(const LaunchCtx& L, int n, const float4* pos4, const float4* vel4,
                         float* pos3, float* vel3);
void launch_unpack_sorted(const LaunchCtx& L, int n, const uint32_t* id_s,
                          const float4* aux4_s, const float4* acc4_s, float* rho,
                          float* pressure, float* acc3);
// precision mode: absolute positions (float or double) <-> cell + offset
int launch_ball_count(const LaunchCtx& L, const GenArgs& g, uint32_t* rows);
int launch_generate(const LaunchCtx& L, const GenArgs& g, const uint32_t* rows);
int launch_render_instances(const LaunchCtx& L, const RenderConst& r, const RenderArgs& a,
                            float* out);
int launch_render_image(const LaunchCtx& L, const RenderConst& r, const RenderArgs& a,
                        unsigned long long* keys, uchar4* rgba);
void launch_pack_cells(const LaunchCtx& L, const StepConst& c, int n, const float* pos3f,
                       const double* pos3d, const float* vel3, const float* mass, int4* cell4,
                       float4* pos4, float4* vel4);
void launch_unpack_cells(const LaunchCtx& L, const StepConst& c, int n, const int4* cell4,
                         const float4* pos4, float* pos3f, double* pos3d);

}  // namespace sphx
