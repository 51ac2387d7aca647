// Precision-mode neighbour passes as tile sweeps: density + pressure, and force +
// acceleration + leapfrog + wall clamp, of the cell + offset step (compute_densities /
// compute_pressures / compute_forces, sph_engine.cpp:203-244, 370-443; integrate_leapfrog,
// cpp:290-310; apply_boundary_conditions, particle.cpp:122-153).
//
// The precision mode is judged against an FP64 evaluation, not against the reference's
// summation order, so its passes need neither the hit lists nor the in-order folds of the
// exact passes.  One warp owns one tile (up to 32 cell-sorted particles of one cell, one
// per lane) and sweeps the tile's stencil 32 candidates at a time: a chunk is staged in
// shared memory in the tile's frame, the candidates that no particle of the tile can reach
// are culled by the tile's box, and every lane evaluates every remaining candidate against
// its own particle, two candidates per packed FP32x2 instruction and without branches: the
// pair's term is formed whatever the distance and is zero (or zeroed) when the candidate is
// not a neighbour.  Every lane is busy on every instruction; the price is the terms of the
// culled box's non-neighbours, which costs less than listing the neighbours.
//
// The self pair is swept like any other: its W is W(0) (the reference's m_i W(0) term) and
// its force terms are zero (r = 0 skips the pressure term; v_i - v_i = 0).
//
// Smoothing kernels in the "max form" (a = max(2 - q, 0), b = max(1 - q, 0) for the cubic
// spline), which is zero beyond the support without a test:
//   cubic spline  dW/dq = sigma/2 (4 b^2 - a^2), d2W/dq2 = sigma (a - 4 b) (kernels.cpp:23-60,
//                 piecewise there); W itself keeps the piecewise form (sweep_w)
//   Wendland C2   t = max(1 - q/2, 0):  W = norm t^4 (1 + 2 q), dW/dq = -5 norm t^3 q,
//                 laplacian = norm (5/h^2) t^2 (5 q - 3)      (kernels.cpp:172-200)
//   Gaussian      no compact support: every term is masked by the neighbour test
//                                                             (kernels.cpp:210-225)
// A pair is a neighbour when |r|^2 <= r_search^2 (spatial_hash.cpp:46-50); when the search
// radius is at least the support 2h, the max form already zeroes every non-neighbour and
// the force sweep skips the test (kCut = false).
//
// Positions are swept in units of h (the tile's frame scaled by 1/h): |r|/h = q comes
// without a multiplication, and every force term that needs the direction uses r_vec / |r|,
// which is the same in any unit.  The pressure term of a pair closer than 1e-6 m, which the
// reference skips, is formed here (it is at most |grad W| 1e-6 m, far below the stated
// bound; a coincident pair, |r| = 0, gives exactly 0 as in the reference).
#include "sphx_passes.cuh"

namespace sphx {

namespace {

// ---- packed FP32 pairs ----------------------------------------------------------------
struct F2 {
    f32x2 v;
};
__device__ __forceinline__ F2 f2(float a) { return {pk2(a, a)}; }
__device__ __forceinline__ F2 f2(float a, float b) { return {pk2(a, b)}; }
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return {xadd2(a.v, b.v)}; }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return {xsub2(a.v, b.v)}; }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return {xmul2(a.v, b.v)}; }
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) { return {xfma2(a.v, b.v, c.v)}; }
__device__ __forceinline__ F2 max0(F2 a) {
    const float2 u = upk2(a.v);
    return f2(fmaxf(u.x, 0.0f), fmaxf(u.y, 0.0f));
}
__device__ __forceinline__ F2 keep(bool ka, bool kb, F2 a) {
    const float2 u = upk2(a.v);
    return f2(ka ? u.x : 0.0f, kb ? u.y : 0.0f);
}

// hardware square root and reciprocal square root (a few ulp; precision mode only)
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float exp_approx(float x) { return __expf(x); }

// position of the empty slots of a chunk: far enough to be no particle's neighbour, near
// enough that every term formed from it stays finite (|r|^2 of 3e30)
constexpr float kFar = 1.0e15f;

// The sweeps' lengths in units of h.
struct SweepUnits {
    float inv;   // 1/h: metres -> sweep units
    float cs;    // the cell size in sweep units
    float r2;    // r_search^2 / h^2: the neighbour test
    float r2m;   // the same with the box cull's margin
    float skip2; // (1e-6 m / h)^2: the Gaussian's pressure-term skip
};
__device__ __forceinline__ SweepUnits sweep_units(const StepConst& c) {
    return SweepUnits{c.rcp_h, c.sw_cs, c.sw_r2, c.sw_r2m, c.sw_skip2};
}
// A particle (cell, offset o, mass in o.w) in the tile's frame, in sweep units: the cell
// difference times the cell size plus the offset scaled, one rounding each (as frame_pos
// does in metres).
__device__ __forceinline__ float4 frame_pos_h(const int4& cell, const int4& frame,
                                              const float4& o, const SweepUnits& U) {
    return make_float4(fmaf((float)(cell.x - frame.x), U.cs, o.x * U.inv),
                       fmaf((float)(cell.y - frame.y), U.cs, o.y * U.inv),
                       fmaf((float)(cell.z - frame.z), U.cs, o.z * U.inv), o.w);
}

// W of two pairs (d2 = (|r|/h)^2 of each) up to the kernel's constant factor
// (sweep_w_scale); the Gaussian's exp(-|r|^2 / h^2) is exp(-d2).  The cubic spline is the
// reference's piecewise polynomial (2/3 - q^2 + q^3/2 on [0, 1], (2 - q)^3 / 6 beyond, with
// 2 - q clamped at 0), selected per pair: no cancellation at small q.
template <int K>
__device__ __forceinline__ F2 sweep_w(const StepConst& c, F2 d2) {
    const float2 e = upk2(d2.v);
    if (K == SPHX_KERNEL_GAUSSIAN) return f2(exp_approx(-e.x), exp_approx(-e.y));
    const F2 q = f2(sqrt_approx(e.x), sqrt_approx(e.y));
    if (K == SPHX_KERNEL_WENDLAND_C2) {
        const F2 t = max0(fma2(q, f2(-0.5f), f2(1.0f)));
        const F2 t2 = t * t;
        return (t2 * t2) * fma2(q, f2(2.0f), f2(1.0f));
    }
    const F2 w1 = fma2(q * q, fma2(q, f2(0.5f), f2(-1.0f)), f2(2.0f / 3.0f));
    const F2 t = max0(f2(2.0f) - q);
    const F2 w2 = (t * t) * (t * f2(1.0f / 6.0f));
    const float2 qv = upk2(q.v), a = upk2(w1.v), bb = upk2(w2.v);
    return f2(qv.x <= 1.0f ? a.x : bb.x, qv.y <= 1.0f ? a.y : bb.y);
}
__host__ __device__ __forceinline__ float sweep_w_scale(const StepConst& c) {
    return c.kern == SPHX_KERNEL_CUBIC_SPLINE ? c.sigma : c.wnorm;
}

// ---------------------------------------------------------------------------------------
// density + pressure
// ---------------------------------------------------------------------------------------
struct SweepDensitySmem {
    float4 box_lo, box_hi;  // the tile's box (kept here, not in registers, across the sweep)
    int2 seg[kMaxSegments];
    float4 xy[16];  // candidates 2p, 2p+1 of the chunk: x, x, y, y (tile frame)
    float4 zm[16];  // z, z, m, m
};
// The spread tiles' launch (sweep_density_spread) stages whole candidates; its own layout
// keeps the main launch's shared memory (and so its L1 share) as small as before.
struct SweepDensitySpreadSmem {
    int2 seg[kMaxSegments];
    int4 scell[32];   // candidate j of the chunk: its cell
    float4 soff[32];  // its offset in sweep units, mass
};

// A tile is spread when one of its particles lies more than kSpreadCells cells from the
// frame (a folded grid puts far cells together; on an unfolded grid the column runs keep
// every tile within kRunCells cells of its first particle's cell): frame
// coordinates that large would carry rounding of the size of their magnitude, so such a
// tile sweeps with each lane's own cell as its frame (the separation of a pair is
// (cell_j - cell_t) cs + (o_j - o_t), the cell difference exact), unculled, one candidate
// pair at a time.  Rare and slow; exact to the same few ulps as a compact tile.
constexpr int kSpreadCells = 4;
static_assert(kRunCells <= kSpreadCells, "a run's tiles would be spread");
// cell difference a - b as a float (wrapping: cells are clamped to +-2^30, so only a pair
// that far apart can wrap, and it stays far)
__device__ __forceinline__ float cdiff(int a, int b) {
    return (float)(int)((unsigned)a - (unsigned)b);
}
__device__ __forceinline__ bool far_cell(const int4& c, const int4& f) {
    return fabsf(cdiff(c.x, f.x)) > kSpreadCells || fabsf(cdiff(c.y, f.y)) > kSpreadCells ||
           fabsf(cdiff(c.z, f.z)) > kSpreadCells;
}
// A spread tile's offset o / h (sweep units) and mass.  The products are rounded on their
// own (__fmul_rn): the lane's particle and its own staged copy then give a separation of
// exactly 0, where a product contracted into the difference (fma(o, 1/h, -o')) would leave
// its rounding error, a separation of ~1e-8 h whose gradient term does not vanish.
__device__ __forceinline__ float4 spread_off(const float4& o, const SweepUnits& U) {
    return make_float4(__fmul_rn(o.x, U.inv), __fmul_rn(o.y, U.inv), __fmul_rn(o.z, U.inv),
                       o.w);
}
// separations (sweep units) of candidates a, b from the lane's particle (cell ct, offset ot)
__device__ __forceinline__ void spread_sep(const SweepUnits& U, const int4& ct, const float4& ot,
                                           const int4& ca, const float4& oa, const int4& cb,
                                           const float4& ob, F2& dx, F2& dy, F2& dz) {
    dx = f2(fmaf(cdiff(ct.x, ca.x), U.cs, ot.x - oa.x), fmaf(cdiff(ct.x, cb.x), U.cs, ot.x - ob.x));
    dy = f2(fmaf(cdiff(ct.y, ca.y), U.cs, ot.y - oa.y), fmaf(cdiff(ct.y, cb.y), U.cs, ot.y - ob.y));
    dz = f2(fmaf(cdiff(ct.z, ca.z), U.cs, ot.z - oa.z), fmaf(cdiff(ct.z, cb.z), U.cs, ot.z - ob.z));
}

// The density sweep of a spread tile: every candidate of every chunk against the lane's
// particle in the lane's own frame (ct, ot: its cell and offset in sweep units).
template <int kKern>
__device__ __forceinline__ void sweep_density_spread(const StepConst& c, const Buffers& b,
                                                  const SweepUnits& U,
                                                  SweepDensitySpreadSmem* S,
                                                  int nseg, int lane, bool valid, int4 ct,
                                                  float4 ot, KSum& rk, uint32_t& nn) {
    for (int sg = 0; sg < nseg; ++sg) {
        const int2 se = S->seg[sg];
        for (int s = se.x; s < se.y; s += 32) {
            const int m = min(32, se.y - s);
            __syncwarp();
            if (lane < m) {
                const float4 o = b.pos4_s[s + lane];
                S->scell[lane] = b.cell4_s[s + lane];
                S->soff[lane] = spread_off(o, U);
            } else {  // empty slot: far, no mass
                S->scell[lane] = ct;
                S->soff[lane] = make_float4(kFar, kFar, kFar, 0.0f);
            }
            __syncwarp();
            F2 acc = f2(0.0f);
            for (int j = 0; j < m; j += 2) {
                F2 dx, dy, dz;
                spread_sep(U, ct, ot, S->scell[j], S->soff[j], S->scell[j + 1], S->soff[j + 1],
                           dx, dy, dz);
                const F2 d2 = fma2(dx, dx, fma2(dy, dy, dz * dz));
                const float2 e = upk2(d2.v);
                const bool ha = valid && e.x <= U.r2, hb = valid && e.y <= U.r2;
                nn += (uint32_t)ha + (uint32_t)hb;
                acc = fma2(f2(S->soff[j].w, S->soff[j + 1].w), keep(ha, hb, sweep_w<kKern>(c, d2)),
                           acc);
            }
            const float2 a2 = upk2(acc.v);
            rk.add(a2.x + a2.y);
        }
    }
}

// The density epilogue of the lane's particle: rho, P and the force sweep's per-candidate
// factors (rho, P, m / (2 rho), (m / rho) mu).
__device__ __forceinline__ void density_out(const StepConst& c, const Buffers& b, int i,
                                            bool cells, float mi, const KSum& rk) {
    const float rho = cells ? rk.value() * sweep_w_scale(c) : xmul(mi, c.w0);
    const float P = xmul(c.gas, xsub(rho, c.rest));
    const float mr = xdiv(mi, rho);
    b.aux4_s[i] = make_float4(rho, P, 0.5f * mr, mr * c.visc);
}

// A tile with a particle more than kSpreadCells cells from its frame (listed for the
// spread launch by the density sweep, skipped by both sweeps).
__device__ __forceinline__ bool spread_tile(const Buffers& b, const Tile& T, int i, bool valid,
                                            const int4& frame) {
    return T.cells && __any_sync(kFull, valid && far_cell(b.cell4_s[i], frame));
}

// kCut: the search radius is below the support 2h (or the kernel is the Gaussian): W is
// selected by the neighbour test; otherwise W is already 0 beyond 2h and the test only
// counts the neighbours.
template <int kKern, bool kCut>
__global__ void __launch_bounds__(128, 6) k_density_sweep(const StepConst c, const Buffers b,
                                                          DevState* ds) {
    if (ds->status) return;
    extern __shared__ __align__(16) unsigned char smem_sweep_d[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    SweepDensitySmem* S = reinterpret_cast<SweepDensitySmem*>(smem_sweep_d) + warp;
    const uint32_t ntiles = ds->n_tiles;
    const Geom g = grid_geom(ds);
    const SweepUnits U = sweep_units(c);
    uint32_t my_max = 0;
    for (uint32_t t = next_tile(&ds->work[0], lane); t < ntiles; t = next_tile(&ds->work[0], lane)) {
        Tile T;
        float4 xi;
        bool valid;
        int4 frame;
        tile_setup_cells(c, b, g, b.tile_start[t], lane, T, xi, valid, frame);
        const int i = T.k0 + lane;
        if (spread_tile(b, T, i, valid, frame)) {
            if (lane == 0) b.spread_tiles[atomicAdd(&ds->n_spread, 1u)] = t;
            continue;  // swept by the spread launch
        }
        if (valid && T.cells) xi = frame_pos_h(b.cell4_s[i], frame, b.pos4_s[i], U);
        {
            const TileBox B = tile_box(xi, valid);
            if (lane == 0) {
                S->box_lo = make_float4(B.lo[0], B.lo[1], B.lo[2], 0.0f);
                S->box_hi = make_float4(B.hi[0], B.hi[1], B.hi[2], 0.0f);
            }
        }
        const F2 X = f2(xi.x), Y = f2(xi.y), Z = f2(xi.z);
        KSum rk;  // sum of m_j W_ij / scale over the stencil, the particle itself included
        uint32_t nn = 0;
        const int nseg = build_segments(b, g, T, lane, S->seg);
        __syncwarp();
        for (int sg = 0; sg < nseg; ++sg) {
            const int2 se = S->seg[sg];
            for (int s = se.x; s < se.y; s += 32) {
                const bool in = lane < se.y - s;
                float4 pl = make_float4(kFar, kFar, kFar, 0.0f);
                if (in) pl = frame_pos_h(b.cell4_s[s + lane], frame, b.pos4_s[s + lane], U);
                TileBox B;
                {
                    const float4 lo = S->box_lo, hi = S->box_hi;
                    B.lo[0] = lo.x, B.lo[1] = lo.y, B.lo[2] = lo.z;
                    B.hi[0] = hi.x, B.hi[1] = hi.y, B.hi[2] = hi.z;
                }
                const uint32_t surv = __ballot_sync(kFull, in && box_near(B, pl, U.r2m));
                if (!surv) continue;
                const int nsv = __popc(surv);
                __syncwarp();  // the previous chunk's reads are done
                {
                    // survivors packed to slots 0 .. nsv-1; an odd count is padded with an
                    // empty slot (written by lane 0 besides its own)
                    auto put = [&](int k, const float4& v) {
                        float* xy = reinterpret_cast<float*>(&S->xy[k >> 1]);
                        float* zm = reinterpret_cast<float*>(&S->zm[k >> 1]);
                        const int h = k & 1;
                        xy[h] = v.x;
                        xy[2 + h] = v.y;
                        zm[h] = v.z;
                        zm[2 + h] = v.w;
                    };
                    if ((surv >> lane) & 1u) put(__popc(surv & ((1u << lane) - 1u)), pl);
                    if (lane == 0 && (nsv & 1)) put(nsv, make_float4(kFar, kFar, kFar, 0.0f));
                }
                __syncwarp();
                F2 acc = f2(0.0f);
                const int np = (nsv + 1) >> 1;
                for (int p = 0; p < np; ++p) {
                    const ulonglong2 u0 = *reinterpret_cast<const ulonglong2*>(&S->xy[p]);
                    const ulonglong2 u1 = *reinterpret_cast<const ulonglong2*>(&S->zm[p]);
                    const F2 dx = X - F2{u0.x}, dy = Y - F2{u0.y}, dz = Z - F2{u1.x};
                    const F2 d2 = fma2(dx, dx, fma2(dy, dy, dz * dz));
                    const float2 e = upk2(d2.v);
                    const bool ha = e.x <= U.r2, hb = e.y <= U.r2;
                    nn += (uint32_t)ha + (uint32_t)hb;
                    const F2 w = sweep_w<kKern>(c, d2);
                    acc = fma2(F2{u1.y}, kCut ? keep(ha, hb, w) : w, acc);
                }
                const float2 a2 = upk2(acc.v);
                rk.add(a2.x + a2.y);  // compensated across chunks
            }
        }
        if (valid) {
            density_out(c, b, i, T.cells, xi.w, rk);
            my_max = max(my_max, nn);
        }
        __syncwarp();
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) my_max = max(my_max, __shfl_xor_sync(kFull, my_max, o));
    if (lane == 0 && my_max) atomicMax(&ds->max_nn, (unsigned long long)my_max);
}

// The spread tiles the density launch listed, each lane in its own frame (its own launch,
// so that this code and its shared memory stay out of the main one).
template <int kKern>
__global__ void __launch_bounds__(128, 4) k_density_sweep_spread(const StepConst c,
                                                                 const Buffers b,
                                                                 DevState* ds) {
    if (ds->status || ds->n_spread == 0) return;  // (an empty list: no atomics)
    extern __shared__ __align__(16) unsigned char smem_sweep_ds[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    SweepDensitySpreadSmem* S = reinterpret_cast<SweepDensitySpreadSmem*>(smem_sweep_ds) + warp;
    const uint32_t ntiles = ds->n_spread;
    const Geom g = grid_geom(ds);
    const SweepUnits U = sweep_units(c);
    uint32_t my_max = 0;
    for (uint32_t t = next_tile(&ds->spread_work[0], lane); t < ntiles;
         t = next_tile(&ds->spread_work[0], lane)) {
        Tile T;
        float4 xi;
        bool valid;
        int4 frame;
        tile_setup_cells(c, b, g, b.tile_start[b.spread_tiles[t]], lane, T, xi, valid, frame);
        const int i = T.k0 + lane;
        const int4 ct = valid ? b.cell4_s[i] : frame;
        const float4 o = valid ? b.pos4_s[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        KSum rk;
        uint32_t nn = 0;
        const int nseg = build_segments(b, g, T, lane, S->seg);
        __syncwarp();
        sweep_density_spread<kKern>(c, b, U, S, nseg, lane, valid, ct, spread_off(o, U), rk, nn);
        if (valid) {
            density_out(c, b, i, T.cells, xi.w, rk);
            my_max = max(my_max, nn);
        }
        __syncwarp();
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) my_max = max(my_max, __shfl_xor_sync(kFull, my_max, o));
    if (lane == 0 && my_max) atomicMax(&ds->max_nn, (unsigned long long)my_max);
}

// ---------------------------------------------------------------------------------------
// force + acceleration (+ leapfrog + wall clamp when kIntegrate)
// ---------------------------------------------------------------------------------------
struct SweepForceSmem {
    float4 box_lo, box_hi;  // the tile's box (kept here, not in registers, across the sweep)
    int2 seg[kMaxSegments];
    float4 xy[16];  // candidates 2p, 2p+1: x, x, y, y (tile frame)
    float4 zv[16];  // z, z, vx, vx
    float4 vv[16];  // vy, vy, vz, vz
    float4 pa[16];  // P, P, kg m/(2 rho), kg m/(2 rho)
    float2 va[16];  // kl (m/rho) mu, kl (m/rho) mu
};
// The spread tiles' launch (sweep_force_spread): candidate j's cell and offset (sweep
// units) in place of the frame coordinates; zv's z slots unused.
struct SweepForceSpreadSmem {
    int2 seg[kMaxSegments];
    int4 scell[32];
    float4 soff[32];
    float4 zv[16];
    float4 vv[16];
    float4 pa[16];
    float2 va[16];
};

// Pressure and viscosity factors of the kernel: the force on particle t from candidate j is
//   kg (m_j / (2 rho_j)) (P_t + P_j) G' r_vec  +  kl (m_j / rho_j) mu L' (v_j - v_t)
// with G' and L' the kernel's gradient and Laplacian shapes below: grad W_tj = -kg G' r_vec
// and laplacian W_tj = kl L' (r_vec = x_t - x_j, in units of h).
__host__ __device__ __forceinline__ float sweep_kg(const StepConst& c) {
    if (c.kern == SPHX_KERNEL_GAUSSIAN) return -c.gg * c.h;  // G' r_vec in h units
    if (c.kern == SPHX_KERNEL_WENDLAND_C2) return 5.0f * c.wnorm * c.rcp_h;
    return -0.5f * c.sigma * c.rcp_h;
}
__host__ __device__ __forceinline__ float sweep_kl(const StepConst& c) {
    if (c.kern == SPHX_KERNEL_GAUSSIAN) return c.gl;
    if (c.kern == SPHX_KERNEL_WENDLAND_C2) return c.wl;
    return c.sigma * c.rcp_hsq;
}

// One packed pair of candidates against the lane's particle; F accumulates.  kMask: zero
// the terms of non-neighbours by selection (needed when the search radius is below the
// support, for the Gaussian, and when a staged candidate carries a non-finite velocity or
// factor, which a zero factor would not cancel).
// The terms of a candidate pair from the separations x_t - x_j (dx, dy, dz, sweep units)
// and the candidates' velocities (vx, vy, vz) and factors (P, kg m/(2 rho); va).
template <int K, bool kMask>
__device__ __forceinline__ void sweep_force_terms(const SweepUnits& U, F2 dx, F2 dy, F2 dz,
                                                  F2 VX, F2 VY, F2 VZ, F2 PT, F2 vx, F2 vy,
                                                  F2 vz, F2 pj, F2 cpf, F2 va, F2& Fx, F2& Fy,
                                                  F2& Fz) {
    const F2 d2 = fma2(dx, dx, fma2(dy, dy, dz * dz));
    const float2 e = upk2(d2.v);
    F2 G, L;
    if (K == SPHX_KERNEL_GAUSSIAN) {
        const F2 ex = f2(exp_approx(-e.x), exp_approx(-e.y));
        G = keep(e.x >= U.skip2, e.y >= U.skip2, ex);
        L = ex * fma2(d2, f2(2.0f), f2(-3.0f));  // 2 |r|^2 / h^2 - 3
    } else {
        // 1/|r| (h units); a coincident pair gets a finite value and q = 0, where the
        // gradient shapes below are 0
        const F2 dd = d2 + f2(1e-30f);
        const float2 de = upk2(dd.v);
        const F2 R = f2(rsqrt_approx(de.x), rsqrt_approx(de.y));
        const F2 q = d2 * R;
        if (K == SPHX_KERNEL_WENDLAND_C2) {
            const F2 t = max0(fma2(q, f2(-0.5f), f2(1.0f)));
            const F2 t2 = t * t;
            G = ((t2 * t) * q) * R;
            L = t2 * fma2(q, f2(5.0f), f2(-3.0f));
        } else {
            const F2 a = max0(f2(2.0f) - q), b2 = max0(fma2(q, f2(-2.0f), f2(2.0f)));  // b2 = 2b
            G = ((b2 - a) * (b2 + a)) * R;  // 4 b^2 - a^2
            L = fma2(b2, f2(-2.0f), a);     // a - 4 b
        }
    }
    F2 cp = (PT + pj) * cpf * G;
    F2 cv = va * L;
    F2 dvx = vx - VX, dvy = vy - VY, dvz = vz - VZ;
    if (kMask) {
        const bool ha = e.x <= U.r2, hb = e.y <= U.r2;
        cp = keep(ha, hb, cp);
        cv = keep(ha, hb, cv);
        dvx = keep(ha, hb, dvx);
        dvy = keep(ha, hb, dvy);
        dvz = keep(ha, hb, dvz);
    }
    Fx = fma2(cv, dvx, fma2(cp, dx, Fx));
    Fy = fma2(cv, dvy, fma2(cp, dy, Fy));
    Fz = fma2(cv, dvz, fma2(cp, dz, Fz));
}

// Staged pair p (candidates 2p, 2p+1, tile frame) against the lane's particle.
template <int K, bool kMask>
__device__ __forceinline__ void sweep_force_pair(const SweepUnits& U, F2 X, F2 Y, F2 Z, F2 VX,
                                                 F2 VY, F2 VZ, F2 PT, const SweepForceSmem* S,
                                                 int p, F2& Fx, F2& Fy, F2& Fz) {
    const ulonglong2 u0 = *reinterpret_cast<const ulonglong2*>(&S->xy[p]);
    const ulonglong2 u1 = *reinterpret_cast<const ulonglong2*>(&S->zv[p]);
    const ulonglong2 u2 = *reinterpret_cast<const ulonglong2*>(&S->vv[p]);
    const ulonglong2 u3 = *reinterpret_cast<const ulonglong2*>(&S->pa[p]);
    const F2 va{*reinterpret_cast<const f32x2*>(&S->va[p])};
    sweep_force_terms<K, kMask>(U, X - F2{u0.x}, Y - F2{u0.y}, Z - F2{u1.x}, VX, VY, VZ, PT,
                                F2{u1.y}, F2{u2.x}, F2{u2.y}, F2{u3.x}, F2{u3.y}, va, Fx, Fy, Fz);
}

// The force sweep of a spread tile: every candidate of every chunk against the lane's
// particle in the lane's own frame (ct, ot), masked by the neighbour test.
template <int kKern>
__device__ __forceinline__ void sweep_force_spread(const Buffers& b, const SweepUnits& U, float kg,
                                                float kl, SweepForceSpreadSmem* S, int nseg,
                                                int lane, int4 ct, float4 ot, F2 VX, F2 VY,
                                                F2 VZ, F2 PT,
                                                KSum& Sx, KSum& Sy, KSum& Sz) {
    for (int sg = 0; sg < nseg; ++sg) {
        const int2 se = S->seg[sg];
        for (int s = se.x; s < se.y; s += 32) {
            const int m = min(32, se.y - s);
            int4 cl = ct;
            float4 ol = make_float4(kFar, kFar, kFar, 0.0f), vl = make_float4(0.f, 0.f, 0.f, 0.f),
                   al = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lane < m) {
                const float4 o = b.pos4_s[s + lane];
                cl = b.cell4_s[s + lane];
                ol = spread_off(o, U);
                vl = b.vel4_s[s + lane];
                al = b.aux4_s[s + lane];
            }
            __syncwarp();
            {
                const int p = lane >> 1, h = lane & 1;
                S->scell[lane] = cl;
                S->soff[lane] = ol;
                reinterpret_cast<float*>(&S->zv[p])[2 + h] = vl.x;
                reinterpret_cast<float*>(&S->vv[p])[h] = vl.y;
                reinterpret_cast<float*>(&S->vv[p])[2 + h] = vl.z;
                reinterpret_cast<float*>(&S->pa[p])[h] = al.y;
                reinterpret_cast<float*>(&S->pa[p])[2 + h] = kg * al.z;
                reinterpret_cast<float*>(&S->va[p])[h] = kl * al.w;
            }
            __syncwarp();
            F2 Fx = f2(0.0f), Fy = f2(0.0f), Fz = f2(0.0f);
            for (int j = 0; j < m; j += 2) {
                const int p = j >> 1;
                F2 dx, dy, dz;
                spread_sep(U, ct, ot, S->scell[j], S->soff[j], S->scell[j + 1], S->soff[j + 1],
                           dx, dy, dz);
                const ulonglong2 u1 = *reinterpret_cast<const ulonglong2*>(&S->zv[p]);
                const ulonglong2 u2 = *reinterpret_cast<const ulonglong2*>(&S->vv[p]);
                const ulonglong2 u3 = *reinterpret_cast<const ulonglong2*>(&S->pa[p]);
                const F2 va{*reinterpret_cast<const f32x2*>(&S->va[p])};
                sweep_force_terms<kKern, true>(U, dx, dy, dz, VX, VY, VZ, PT, F2{u1.y}, F2{u2.x},
                                               F2{u2.y}, F2{u3.x}, F2{u3.y}, va, Fx, Fy, Fz);
            }
            const float2 fx = upk2(Fx.v), fy = upk2(Fy.v), fz = upk2(Fz.v);
            Sx.add(fx.x + fx.y);
            Sy.add(fy.x + fy.y);
            Sz.add(fz.x + fz.y);
        }
    }
}

// The force epilogue of the lane's particle: the acceleration, and (kIntegrate) the
// leapfrog step with the wall clamp, scattered back to insertion order.
template <bool kIntegrate>
__device__ __forceinline__ void force_out(const StepConst& c, const Buffers& b, DevState* ds,
                                          int i, float mi, const KSum& Sx, const KSum& Sy,
                                          const KSum& Sz) {
    const float ax = Sx.value() / mi;
    const float ay = (Sy.value() + c.grav * mi) / mi;
    const float az = Sz.value() / mi;
    b.acc4_s[i] = make_float4(ax, ay, az, 0.0f);
    if (!kIntegrate) return;
    const uint32_t id = b.id_s[i];
    int4 cell = b.cell4_s[i];
    const float4 own = b.pos4_s[i];
    const float4 vi = b.vel4_s[i];  // loaded again: not held across the sweep
    float o[3] = {own.x, own.y, own.z}, v[3] = {vi.x, vi.y, vi.z};
    const float acc[3] = {ax, ay, az};
    if (!cell.w) integrate_cells(c, ds->dt, acc, o, v, cell);
    b.cell4[id] = cell;
    b.pos4[id] = make_float4(o[0], o[1], o[2], mi);
    b.vel4[id] = make_float4(v[0], v[1], v[2], 0.0f);
    if (id == 0) {
        ds->a0[0] = ax;
        ds->a0[1] = ay;
        ds->a0[2] = az;
    }
}

template <bool kIntegrate, int kKern, bool kCut>
__global__ void __launch_bounds__(128, 5) k_force_sweep(const StepConst c, const Buffers b,
                                                        DevState* ds) {
    if (ds->status) return;
    extern __shared__ __align__(16) unsigned char smem_sweep_f[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    SweepForceSmem* S = reinterpret_cast<SweepForceSmem*>(smem_sweep_f) + warp;
    const uint32_t ntiles = ds->n_tiles;
    const Geom g = grid_geom(ds);
    const SweepUnits U = sweep_units(c);
    const float kg = sweep_kg(c), kl = sweep_kl(c);
    for (uint32_t t = next_tile(&ds->work[1], lane); t < ntiles; t = next_tile(&ds->work[1], lane)) {
        Tile T;
        float4 xi;
        bool valid;
        int4 frame;
        tile_setup_cells(c, b, g, b.tile_start[t], lane, T, xi, valid, frame);
        const int i = T.k0 + lane;
        if (spread_tile(b, T, i, valid, frame))
            continue;  // listed by the density launch, swept by the spread launch
        if (valid && T.cells) xi = frame_pos_h(b.cell4_s[i], frame, b.pos4_s[i], U);
        {
            const TileBox B = tile_box(xi, valid);
            if (lane == 0) {
                S->box_lo = make_float4(B.lo[0], B.lo[1], B.lo[2], 0.0f);
                S->box_hi = make_float4(B.hi[0], B.hi[1], B.hi[2], 0.0f);
            }
        }
        F2 VX, VY, VZ, PT;
        {
            const float4 vi = valid ? b.vel4_s[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float Pi = valid ? b.aux4_s[i].y : 0.0f;
            VX = f2(vi.x), VY = f2(vi.y), VZ = f2(vi.z), PT = f2(Pi);
        }
        const F2 X = f2(xi.x), Y = f2(xi.y), Z = f2(xi.z);
        KSum Sx, Sy, Sz;  // force sums, compensated across chunks
        const int nseg = build_segments(b, g, T, lane, S->seg);
        __syncwarp();
        for (int sg = 0; sg < nseg; ++sg) {
            const int2 se = S->seg[sg];
            for (int s = se.x; s < se.y; s += 32) {
                const bool in = lane < se.y - s;
                float4 pl = make_float4(kFar, kFar, kFar, 0.0f);
                if (in) pl = frame_pos_h(b.cell4_s[s + lane], frame, b.pos4_s[s + lane], U);
                TileBox B;
                {
                    const float4 lo = S->box_lo, hi = S->box_hi;
                    B.lo[0] = lo.x, B.lo[1] = lo.y, B.lo[2] = lo.z;
                    B.hi[0] = hi.x, B.hi[1] = hi.y, B.hi[2] = hi.z;
                }
                const uint32_t surv = __ballot_sync(kFull, in && box_near(B, pl, U.r2m));
                if (!surv) continue;
                const int nsv = __popc(surv);
                const bool mine = (surv >> lane) & 1u;
                float4 vl = make_float4(0.f, 0.f, 0.f, 0.f), al = make_float4(0.f, 0.f, 0.f, 0.f);
                if (mine) {
                    vl = b.vel4_s[s + lane];
                    al = b.aux4_s[s + lane];
                }
                const float cpf = kg * al.z, cvf = kl * al.w;
                // a non-finite velocity or factor is not cancelled by a zero factor: such a
                // chunk takes the masked sweep
                const bool odd = !isfinite(vl.x + vl.y + vl.z + al.y + cpf + cvf);
                const bool masked = kCut || __any_sync(kFull, odd);
                __syncwarp();  // the previous chunk's reads are done
                // survivors packed to slots 0 .. nsv-1; an odd count is padded with an empty
                // slot (written by lane 0 besides its own)
                auto put = [&](int k, const float4& x, const float4& v, const float4& a3) {
                    const int p = k >> 1, h = k & 1;
                    float* xy = reinterpret_cast<float*>(&S->xy[p]);
                    float* zv = reinterpret_cast<float*>(&S->zv[p]);
                    float* vv = reinterpret_cast<float*>(&S->vv[p]);
                    float* pa = reinterpret_cast<float*>(&S->pa[p]);
                    float* va = reinterpret_cast<float*>(&S->va[p]);
                    xy[h] = x.x;
                    xy[2 + h] = x.y;
                    zv[h] = x.z;
                    zv[2 + h] = v.x;
                    vv[h] = v.y;
                    vv[2 + h] = v.z;
                    pa[h] = a3.x;
                    pa[2 + h] = a3.y;
                    va[h] = a3.z;
                };
                if (mine)
                    put(__popc(surv & ((1u << lane) - 1u)), pl, vl, make_float4(al.y, cpf, cvf, 0.f));
                if (lane == 0 && (nsv & 1)) {
                    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
                    put(nsv, make_float4(kFar, kFar, kFar, 0.0f), z, z);
                }
                __syncwarp();
                F2 Fx = f2(0.0f), Fy = f2(0.0f), Fz = f2(0.0f);
                const int np = (nsv + 1) >> 1;
                if (masked) {
                    for (int p = 0; p < np; ++p)
                        sweep_force_pair<kKern, true>(U, X, Y, Z, VX, VY, VZ, PT, S, p, Fx, Fy, Fz);
                } else {
                    for (int p = 0; p < np; ++p)
                        sweep_force_pair<kKern, false>(U, X, Y, Z, VX, VY, VZ, PT, S, p, Fx, Fy, Fz);
                }
                const float2 fx = upk2(Fx.v), fy = upk2(Fy.v), fz = upk2(Fz.v);
                Sx.add(fx.x + fx.y);
                Sy.add(fy.x + fy.y);
                Sz.add(fz.x + fz.y);
            }
        }
        __syncwarp();
        if (!valid) continue;
        force_out<kIntegrate>(c, b, ds, i, xi.w, Sx, Sy, Sz);
    }
}

// The spread tiles the density launch listed, each lane in its own frame (its own launch).
template <bool kIntegrate, int kKern>
__global__ void __launch_bounds__(128, 4) k_force_sweep_spread(const StepConst c,
                                                               const Buffers b, DevState* ds) {
    if (ds->status || ds->n_spread == 0) return;
    extern __shared__ __align__(16) unsigned char smem_sweep_fs[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    SweepForceSpreadSmem* S = reinterpret_cast<SweepForceSpreadSmem*>(smem_sweep_fs) + warp;
    const uint32_t ntiles = ds->n_spread;
    const Geom g = grid_geom(ds);
    const SweepUnits U = sweep_units(c);
    const float kg = sweep_kg(c), kl = sweep_kl(c);
    for (uint32_t t = next_tile(&ds->spread_work[1], lane); t < ntiles;
         t = next_tile(&ds->spread_work[1], lane)) {
        Tile T;
        float4 xi;
        bool valid;
        int4 frame;
        tile_setup_cells(c, b, g, b.tile_start[b.spread_tiles[t]], lane, T, xi, valid, frame);
        const int i = T.k0 + lane;
        const int4 ct = valid ? b.cell4_s[i] : frame;
        const float4 o = valid ? b.pos4_s[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        F2 VX, VY, VZ, PT;
        {
            const float4 vi = valid ? b.vel4_s[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float Pi = valid ? b.aux4_s[i].y : 0.0f;
            VX = f2(vi.x), VY = f2(vi.y), VZ = f2(vi.z), PT = f2(Pi);
        }
        KSum Sx, Sy, Sz;
        const int nseg = build_segments(b, g, T, lane, S->seg);
        __syncwarp();
        sweep_force_spread<kKern>(b, U, kg, kl, S, nseg, lane, ct, spread_off(o, U), VX, VY, VZ,
                                  PT, Sx, Sy, Sz);
        __syncwarp();
        if (!valid) continue;
        force_out<kIntegrate>(c, b, ds, i, xi.w, Sx, Sy, Sz);
    }
}

template <class K>
void launch_sweep(const LaunchCtx& L, LaunchShapeCache& cache, K kernel, size_t smem_per_warp,
                  const StepConst& c, const Buffers& b, DevState* ds) {
    const int threads = 32 * L.warps_per_block;
    const size_t sm = (size_t)L.warps_per_block * smem_per_warp;
    const int nb = cached_resident_blocks(cache, L, kernel, threads, sm);
    kernel<<<nb, threads, sm, L.stream>>>(c, b, ds);
}

template <int kKern, bool kCut>
void launch_density_sweep_v(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                            DevState* ds) {
    static LaunchShapeCache cache, cache_spread;
    launch_sweep(L, cache, k_density_sweep<kKern, kCut>, sizeof(SweepDensitySmem), c, b, ds);
    launch_sweep(L, cache_spread, k_density_sweep_spread<kKern>, sizeof(SweepDensitySpreadSmem),
                 c, b, ds);
}

template <int kKern>
void launch_density_sweep_k(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                            DevState* ds) {
    if (kKern == SPHX_KERNEL_GAUSSIAN || c.r2 < 4.0f * c.h_sq)
        launch_density_sweep_v<kKern, true>(L, c, b, ds);
    else
        launch_density_sweep_v<kKern, false>(L, c, b, ds);
}

template <bool kIntegrate, int kKern, bool kCut>
void launch_force_sweep_v(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                          DevState* ds) {
    static LaunchShapeCache cache, cache_spread;
    launch_sweep(L, cache, k_force_sweep<kIntegrate, kKern, kCut>, sizeof(SweepForceSmem), c, b,
                 ds);
    launch_sweep(L, cache_spread, k_force_sweep_spread<kIntegrate, kKern>,
                 sizeof(SweepForceSpreadSmem), c, b, ds);
}

template <int kKern>
void launch_force_sweep_k(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                          DevState* ds, int integrate) {
    // the max form zeroes every pair beyond the support 2h; a search radius below it needs
    // the neighbour test (the Gaussian has no compact support)
    const bool cut = kKern == SPHX_KERNEL_GAUSSIAN || c.r2 < 4.0f * c.h_sq;
    if (integrate) {
        if (cut) launch_force_sweep_v<true, kKern, true>(L, c, b, ds);
        else launch_force_sweep_v<true, kKern, false>(L, c, b, ds);
    } else {
        if (cut) launch_force_sweep_v<false, kKern, true>(L, c, b, ds);
        else launch_force_sweep_v<false, kKern, false>(L, c, b, ds);
    }
}

}  // namespace

int launch_density_sweep(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                         DevState* ds) {
    if (c.kern == SPHX_KERNEL_WENDLAND_C2) launch_density_sweep_k<SPHX_KERNEL_WENDLAND_C2>(L, c, b, ds);
    else if (c.kern == SPHX_KERNEL_GAUSSIAN) launch_density_sweep_k<SPHX_KERNEL_GAUSSIAN>(L, c, b, ds);
    else launch_density_sweep_k<SPHX_KERNEL_CUBIC_SPLINE>(L, c, b, ds);
    return 2;  // the main and the spread-tile launch
}

int launch_force_sweep(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds,
                       int integrate) {
    if (c.kern == SPHX_KERNEL_WENDLAND_C2)
        launch_force_sweep_k<SPHX_KERNEL_WENDLAND_C2>(L, c, b, ds, integrate);
    else if (c.kern == SPHX_KERNEL_GAUSSIAN)
        launch_force_sweep_k<SPHX_KERNEL_GAUSSIAN>(L, c, b, ds, integrate);
    else launch_force_sweep_k<SPHX_KERNEL_CUBIC_SPLINE>(L, c, b, ds, integrate);
    return 2;  // the main and the spread-tile launch
}

}  // namespace sphx
