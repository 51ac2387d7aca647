// Neighbour passes of the step: density + pressure, and force + leapfrog + wall clamp.
//
// Work decomposition: one warp owns one tile (up to 32 consecutive cell-sorted particles
// of one cell, one particle per lane).  All lanes of a tile share the tile's stencil:
// for each row (dx, dy) the cells cz+lo..cz+hi are one contiguous range of the sorted
// arrays; the warp stages that range through shared memory 32 candidates at a time and
// every lane tests every candidate against its own particle.
//
// Exactness.  The reference walks, for particle i, the cells (dx, dy, dz) of its stencil
// in lexicographic order and each cell's particles in insertion order
// (spatial_hash.cpp:31-57), and accumulates every sum sequentially in that order
// (sph_engine.cpp:370-432).  The sorted arrays hold each cell's particles in insertion
// order (stable sort from insertion order), the rows are walked in (dx, dy) order and
// each row in increasing z, so a lane meets its neighbours in exactly the reference's
// order.  The reference scans a 5x5x5 block (cell_radius = 2); a neighbour at distance
// <= r can only sit two cells away when the particle lies within rounding distance of a
// cell face, so the tile's stencil is 3x3x3, widened on an axis to the second layer when
// some lane is that close to a face (guard band eps below).  Every distance test and
// every term uses the reference's float operations in the reference's order with
// IEEE round-to-nearest and no contraction, so each lane's sums are bit-identical.
#include <atomic>

#include "sphx_internal.cuh"

namespace sphx {

struct Tile {
    int k0;       // first sorted position of the tile
    int cnt;      // particles in the tile (<= 32)
    bool cells;   // false for the group of non-finite particles (no neighbours)
    int cx, cy, cz;
    int lo[3], hi[3];
};

// Geometry of the whole grid (single scene).
__device__ __forceinline__ Geom grid_geom(const DevState* ds) {
    Geom g;
    for (int a = 0; a < 3; ++a) {
        g.dim[a] = ds->dim[a];
        g.wrap[a] = ds->wrap[a];
    }
    g.base = 0;
    g.sentinel = ds->ncells;
    return g;
}

// Geometry of one scene's block of cells (batched mode; scene grids are never folded).
__device__ __forceinline__ Geom scene_geom(const SceneInfo& sc, const DevState* ds) {
    Geom g;
    for (int a = 0; a < 3; ++a) {
        g.dim[a] = sc.dim[a];
        g.wrap[a] = 0;
    }
    g.base = sc.base;
    g.sentinel = ds->ncells;
    return g;
}

// Sets up the tile starting at sorted position k0; returns the lane's particle (valid
// lanes only).
__device__ __forceinline__ void tile_setup(const StepConst& c, const Buffers& b, const Geom& g,
                                           uint32_t k0, int lane, Tile& T, float4& xi,
                                           bool& valid) {
    const uint32_t key = b.key_s[k0];
    const uint32_t end = b.off[key + 1];
    T.k0 = (int)k0;
    T.cnt = (int)min(end - k0, (uint32_t)b.tile_n);
    valid = lane < T.cnt;
    xi = valid ? b.pos4_s[k0 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    T.cells = key < g.sentinel;
    if (!T.cells) return;
    const uint32_t local = key - g.base;
    const uint32_t dz = g.dim[2], dy = g.dim[1];
    T.cz = (int)(local % dz);
    T.cy = (int)((local / dz) % dy);
    T.cx = (int)(local / (dz * dy));
    const float x[3] = {xi.x, xi.y, xi.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // position inside the cell in cell units; the guard band covers the rounding of
        // x*inv_cell and of the distance test (a few ulps of |u|) with a wide margin
        const float u = xmul(x[a], c.inv_cell);
        const float frac = u - floorf(u);
        const float eps = 1.52587890625e-5f + fabsf(u) * 9.5367431640625e-7f;
        const bool near_lo = valid && frac < eps;
        const bool near_hi = valid && (1.0f - frac) < eps;
        T.lo[a] = __any_sync(0xffffffffu, near_lo) ? -2 : -1;
        T.hi[a] = __any_sync(0xffffffffu, near_hi) ? 2 : 1;
    }
}

// Precision mode: the tile's frame is the cell of its first particle; a position inside
// the frame is (cell - frame) * cs + offset, exact to a few ulps of the cell size however
// far the frame lies from the origin.
__device__ __forceinline__ float4 frame_pos(const int4& cell, const int4& frame, const float4& o,
                                            float cs) {
    return make_float4((float)(cell.x - frame.x) * cs + o.x, (float)(cell.y - frame.y) * cs + o.y,
                       (float)(cell.z - frame.z) * cs + o.z, o.w);
}

__device__ __forceinline__ void tile_setup_cells(const StepConst& c, const Buffers& b,
                                                 const Geom& g, uint32_t k0, int lane,
                                                 Tile& T, float4& xi, bool& valid,
                                                 int4& frame) {
    const uint32_t key = b.key_s[k0];
    const uint32_t nc = g.sentinel;
    const uint32_t end = b.off[key + 1];
    T.k0 = (int)k0;
    T.cnt = (int)min(end - k0, (uint32_t)b.tile_n);
    valid = lane < T.cnt;
    frame = b.cell4_s[k0];
    const float4 o = valid ? b.pos4_s[k0 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int4 ci = valid ? b.cell4_s[k0 + lane] : frame;
    xi = frame_pos(ci, frame, o, c.cs);
    T.cells = key < nc;
    if (!T.cells) {
        xi = o;
        return;
    }
    const uint32_t local = key - g.base;
    const uint32_t dz = g.dim[2], dy = g.dim[1];
    T.cz = (int)(local % dz);
    T.cy = (int)((local / dz) % dy);
    T.cx = (int)(local / (dz * dy));
    const float off[3] = {o.x, o.y, o.z};
    const float eps = c.cs * 2.44140625e-4f;  // 2^-12 cells
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const bool near_lo = valid && off[a] < eps;
        const bool near_hi = valid && (c.cs - off[a]) < eps;
        T.lo[a] = __any_sync(0xffffffffu, near_lo) ? -2 : -1;
        T.hi[a] = __any_sync(0xffffffffu, near_hi) ? 2 : 1;
    }
}

// Calls f(begin, end) for every stencil row of the tile, in the reference's order.  On a
// folded axis the neighbour index wraps; a row that wraps on z is two segments, visited
// in dz order.
template <class F>
__device__ __forceinline__ void for_each_row(const Buffers& b, const Geom& g, const Tile& T,
                                             F&& f) {
    if (!T.cells) return;
    const int d0 = g.dim[0], d1 = g.dim[1], d2 = g.dim[2];
    const bool w0 = g.wrap[0], w1 = g.wrap[1], w2 = g.wrap[2];
    // z range of every row: [z0, z1] plus, when z wraps past the end, [0, z2]
    int z0 = T.cz + T.lo[2], z1 = T.cz + T.hi[2], z2 = -1;
    int zp = -1, zq = -2;  // a wrapped piece at the front (dz < 0 past 0)
    if (w2) {
        if (z0 < 0) {
            zp = z0 + d2;
            zq = d2 - 1;
            z0 = 0;
        }
        if (z1 >= d2) {
            z2 = z1 - d2;
            z1 = d2 - 1;
        }
    } else {
        z0 = max(z0, 0);
        z1 = min(z1, d2 - 1);
    }
    for (int dx = T.lo[0]; dx <= T.hi[0]; ++dx) {
        int X = T.cx + dx;
        if (w0) X = (X + d0) % d0;
        else if (X < 0 || X >= d0) continue;
        for (int dy = T.lo[1]; dy <= T.hi[1]; ++dy) {
            int Y = T.cy + dy;
            if (w1) Y = (Y + d1) % d1;
            else if (Y < 0 || Y >= d1) continue;
            const uint32_t rb = g.base + ((uint32_t)X * (uint32_t)d1 + (uint32_t)Y) * (uint32_t)d2;
            if (zp <= zq) {
                const uint32_t a = b.off[rb + zp], e = b.off[rb + zq + 1];
                if (a < e) f((int)a, (int)e);
            }
            if (z0 <= z1) {
                const uint32_t a = b.off[rb + z0], e = b.off[rb + z1 + 1];
                if (a < e) f((int)a, (int)e);
            }
            if (z2 >= 0) {
                const uint32_t a = b.off[rb], e = b.off[rb + z2 + 1];
                if (a < e) f((int)a, (int)e);
            }
        }
    }
}

// The same walk as for_each_row, listed up front: writes the tile's non-empty row
// segments [a, e) to seg in visiting order and returns their number (<= 75: 5 x 5 rows of
// up to 3 pieces).  One lane per row (dx, dy) -- lane order is the rows' visiting order --
// and a warp scan places each row's pieces.
constexpr int kMaxSegments = 75;
__device__ __forceinline__ int build_segments(const Buffers& b, const Geom& g, const Tile& T,
                                              int lane, int2* seg) {
    if (!T.cells) return 0;
    const int d0 = g.dim[0], d1 = g.dim[1], d2 = g.dim[2];
    int z0 = T.cz + T.lo[2], z1 = T.cz + T.hi[2], z2 = -1;
    int zp = -1, zq = -2;
    if (g.wrap[2]) {
        if (z0 < 0) {
            zp = z0 + d2;
            zq = d2 - 1;
            z0 = 0;
        }
        if (z1 >= d2) {
            z2 = z1 - d2;
            z1 = d2 - 1;
        }
    } else {
        z0 = max(z0, 0);
        z1 = min(z1, d2 - 1);
    }
    const int ny = T.hi[1] - T.lo[1] + 1;
    const int nrows = (T.hi[0] - T.lo[0] + 1) * ny;
    int2 p0 = make_int2(0, 0), p1 = p0, p2 = p0;  // the row's pieces, in dz order
    bool v0 = false, v1 = false, v2 = false;
    if (lane < nrows) {
        int X = T.cx + T.lo[0] + lane / ny;
        int Y = T.cy + T.lo[1] + lane % ny;
        bool ok = true;
        if (g.wrap[0]) X = (X + d0) % d0;
        else ok = X >= 0 && X < d0;
        if (g.wrap[1]) Y = (Y + d1) % d1;
        else ok = ok && Y >= 0 && Y < d1;
        if (ok) {
            const uint32_t rb = g.base + ((uint32_t)X * (uint32_t)d1 + (uint32_t)Y) * (uint32_t)d2;
            if (zp <= zq) {
                p0 = make_int2((int)b.off[rb + zp], (int)b.off[rb + zq + 1]);
                v0 = p0.x < p0.y;
            }
            if (z0 <= z1) {
                p1 = make_int2((int)b.off[rb + z0], (int)b.off[rb + z1 + 1]);
                v1 = p1.x < p1.y;
            }
            if (z2 >= 0) {
                p2 = make_int2((int)b.off[rb], (int)b.off[rb + z2 + 1]);
                v2 = p2.x < p2.y;
            }
        }
    }
    const uint32_t np = (uint32_t)v0 + (uint32_t)v1 + (uint32_t)v2;
    uint32_t x = np;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    uint32_t at = x - np;
    if (v0) seg[at++] = p0;
    if (v1) seg[at++] = p1;
    if (v2) seg[at] = p2;
    return (int)__shfl_sync(0xffffffffu, x, 31);
}

// d = x_i - x_j; d2 = dot(d, d)  (spatial_hash.h:70-73, sph_engine.cpp:378, 400, 424)
struct Diff {
    float x, y, z, d2;
};
__device__ __forceinline__ Diff diff(const float4& xi, const float4& xj) {
    Diff d;
    d.x = xsub(xi.x, xj.x);
    d.y = xsub(xi.y, xj.y);
    d.z = xsub(xi.z, xj.z);
    d.d2 = xdot3(d.x, d.y, d.z);
    return d;
}
// diff(xi, xj).d2 with the x and y steps as packed FP32 pairs (same rounding)
__device__ __forceinline__ float diff_d2(const float4& xi, const float4& xj) {
    const f32x2 dxy = xsub2(pk2(xi.x, xi.y), pk2(xj.x, xj.y));
    const float dz = xsub(xi.z, xj.z);
    const float2 sq = upk2(xmul2(dxy, dxy));
    return xadd(xadd(sq.x, sq.y), xmul(dz, dz));
}

// a gradient component inside xdiv_fixed_nz's range: zero, or at least 2^-100 in
// magnitude (its upper bound, sigma, is the host's business)
__device__ __forceinline__ bool nz_range(float g) { return !(fabsf(g) < 0x1p-100f) || g == 0.0f; }

// ---------------------------------------------------------------------------------------
// Chunk machinery shared by the density and force passes.
//
// A row segment is consumed in chunks of 32 candidates staged in shared memory.  For a
// chunk, every lane first builds a 32-bit mask of its hits (the exact distance test; the
// candidates a warp-uniform bounding-box test rules out for the whole tile are skipped).
// The expensive per-pair terms are then computed FLATTENED: the warp's hits are listed
// (lane, candidate) in lane-then-candidate order and the 32 lanes work through that list
// together, writing each term to shared memory.  Finally every lane adds its own terms in
// candidate order -- the reference's order -- so each particle's sums are the same
// sequence of IEEE additions as in the reference, while the SIMT lanes stay busy on the
// costly terms regardless of how unevenly the hits fall on lanes.
// ---------------------------------------------------------------------------------------

constexpr uint32_t kFull = 0xffffffffu;
constexpr int kDensityBatch = 256;  // flattened terms computed per round (density)
constexpr int kForceBatch = 96;     // flattened terms computed per round (force)

__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t v, int lane, uint32_t& total) {
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(kFull, x, 31);
    return x - v;
}

// Writes this lane's hits (mask) to plist[o, o + popc(mask)) as (lane << 5) | candidate,
// in candidate order, two per iteration.
__device__ __forceinline__ void list_hits(uint16_t* plist, uint32_t mask, uint32_t o, int lane) {
    const uint32_t tag = (uint32_t)lane << 5;
    uint32_t mm = mask, k = o;
    while (mm) {
        const uint32_t a = __ffs(mm) - 1;
        mm &= mm - 1;
        plist[k] = (uint16_t)(tag | a);
        if (!mm) break;
        const uint32_t b = __ffs(mm) - 1;
        mm &= mm - 1;
        plist[k + 1] = (uint16_t)(tag | b);
        k += 2;
    }
}

// Axis-aligned box of the tile's particles (valid lanes).
struct TileBox {
    float lo[3], hi[3];
};
__device__ __forceinline__ TileBox tile_box(const float4& xi, bool valid) {
    TileBox B;
    const float inf = __int_as_float(0x7f800000);
    B.lo[0] = valid ? xi.x : inf;
    B.lo[1] = valid ? xi.y : inf;
    B.lo[2] = valid ? xi.z : inf;
    B.hi[0] = valid ? xi.x : -inf;
    B.hi[1] = valid ? xi.y : -inf;
    B.hi[2] = valid ? xi.z : -inf;
#pragma unroll
    for (int o = 16; o; o >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            B.lo[a] = fminf(B.lo[a], __shfl_xor_sync(kFull, B.lo[a], o));
            B.hi[a] = fmaxf(B.hi[a], __shfl_xor_sync(kFull, B.hi[a], o));
        }
    return B;
}

// Conservative: false only if no point of the box is within r of p (margin 1e-4 on r^2
// covers every rounding of this test and of the exact distance test).
__device__ __forceinline__ bool box_near(const TileBox& B, const float4& p, float r2_margin) {
    const float ex = fmaxf(fmaxf(B.lo[0] - p.x, p.x - B.hi[0]), 0.0f);
    const float ey = fmaxf(fmaxf(B.lo[1] - p.y, p.y - B.hi[1]), 0.0f);
    const float ez = fmaxf(fmaxf(B.lo[2] - p.z, p.z - B.hi[2]), 0.0f);
    return ex * ex + ey * ey + ez * ez <= r2_margin;
}

// Hit mask of this lane's particle against the staged chunk (candidates in `surv` only).
// Exact mode: the reference's rounded test; precision mode: contracted FP32 on
// frame-relative coordinates.
template <bool kPrecise>
__device__ __forceinline__ uint32_t chunk_hits(const float4* cand, uint32_t surv,
                                               const float4& xi, float r2) {
    uint32_t mask = 0;
#pragma unroll
    for (int jj = 0; jj < 32; ++jj) {
        if (surv & (1u << jj)) {
            float d2;
            if (kPrecise) {
                const float4 xj = cand[jj];
                const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                d2 = dx * dx + dy * dy + dz * dz;
            } else {
                d2 = diff(xi, cand[jj]).d2;
            }
            if (d2 <= r2) mask |= 1u << jj;
        }
    }
    return mask;
}

// chunk_hits<false> two candidates at a time with packed FP32 pairs: the same exact test
// (x_i - x_j per axis, (dx*dx + dy*dy) + dz*dz, <= r^2), element by element.  Candidates
// outside `surv` are farther than r from every lane (the box cull is conservative), so a
// pair is skipped only when both of its candidates are.
__device__ __forceinline__ uint32_t chunk_hits_x2(const float* cx, const float* cy,
                                                  const float* cz, uint32_t surv,
                                                  const float4& xi, float r2) {
    const f32x2 X = pk2(xi.x, xi.x), Y = pk2(xi.y, xi.y), Z = pk2(xi.z, xi.z);
    uint32_t mask = 0;
#pragma unroll
    for (int jj = 0; jj < 32; jj += 2) {
        if ((surv >> jj) & 3u) {
            const f32x2 dx = xsub2(X, *reinterpret_cast<const f32x2*>(cx + jj));
            const f32x2 dy = xsub2(Y, *reinterpret_cast<const f32x2*>(cy + jj));
            const f32x2 dz = xsub2(Z, *reinterpret_cast<const f32x2*>(cz + jj));
            const float2 d2 = upk2(xadd2(xadd2(xmul2(dx, dx), xmul2(dy, dy)), xmul2(dz, dz)));
            if (d2.x <= r2) mask |= 1u << jj;
            if (d2.y <= r2) mask |= 2u << jj;
        }
    }
    return mask;
}

// |r| and 1/|r| of a pair from d2 = |r|^2 with the hardware reciprocal square root (a few
// ulp): precision mode only.  A coincident pair (d2 = 0) gets |r| = 0 and 1/|r| = 0.
__device__ __forceinline__ void fast_len(float d2, float& r, float& rinv) {
    rinv = d2 > 0.0f ? rsqrtf(d2) : 0.0f;
    r = d2 * rinv;
}

// W(q) in precision mode: the same formula with contracted arithmetic, both branches
// evaluated and one selected (q of a hit is at most 2 up to rounding)
__device__ __forceinline__ float cubic_w_fast(const StepConst& c, float q) {
    const float t = 2.0f - q;
    const float w1 = c.sigma * fmaf(q * q, fmaf(0.5f, q, -1.0f), 2.0f / 3.0f);
    const float w2 = c.sigma * (1.0f / 6.0f) * (t * t * t);
    return q <= 1.0f ? w1 : (q <= 2.0f ? w2 : 0.0f);
}

// W of the pair (x_i - x_j = (dx, dy, dz), d2 = |.|^2) for smoothing kernel K.
// Exact mode: the reference's float operations (Kernel::W, kernels.cpp:140-143, 172-178,
// 210-213); precision mode: contracted arithmetic.
// kNZ: d2 <= r^2 (a hit), so |r| is +0 or in [2^-74.5, r (1 + 2^-23)], which the host
// keeps inside xdiv_fixed_nz's range
template <int K, bool kNZ = false>
__device__ __forceinline__ float pair_w_exact(const StepConst& c, float d2) {
    if (K == SPHX_KERNEL_GAUSSIAN) return xmul(c.wnorm, expf(xmul(-d2, c.gs)));
    const float q = kNZ ? xdiv_fixed_nz(xsqrt(d2), c.h, c.rcp_h)
                        : xdiv_fixed(xsqrt(d2), c.h, c.rcp_h, c.fast_div_h);
    return K == SPHX_KERNEL_WENDLAND_C2 ? wendland_w(c, q) : cubic_w(c, q);
}
// W of a pair in precision mode: contracted arithmetic, hardware reciprocal square root
// and exponential (errors of a few ulp per term, far inside the stated bounds)
template <int K>
__device__ __forceinline__ float pair_w_fast(const StepConst& c, float d2) {
    if (K == SPHX_KERNEL_GAUSSIAN) return c.wnorm * __expf(-d2 * c.gs);
    float r, rinv;
    fast_len(d2, r, rinv);
    const float q = r * c.rcp_h;
    if (K == SPHX_KERNEL_WENDLAND_C2) {
        const float t = fmaf(-0.5f, q, 1.0f);
        const float t2 = t * t;
        return q < 2.0f ? c.wnorm * (t2 * t2) * fmaf(2.0f, q, 1.0f) : 0.0f;
    }
    return cubic_w_fast(c, q);
}

// Work distribution: warps take tiles from a per-pass counter (dynamic, so crowded cells
// in degenerate states do not serialise the tail).
__device__ __forceinline__ uint32_t next_tile(uint32_t* ctr, int lane) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(ctr, 1u);
    return __shfl_sync(kFull, t, 0);
}

// ---------------------------------------------------------------------------------------
// density + pressure:  rho_i = m_i W(0) + sum_{j in N(i), j != i} m_j W(r_ij)
//                      P_i = k (rho_i - rho0)
// (compute_density / compute_pressure, sph_engine.cpp:370-388)
// ---------------------------------------------------------------------------------------
struct DensitySmem {
    float4 box_lo, box_hi;  // tile box (culling test)
    uint32_t mcur, mend;    // the warp's region of the hit-mask pool: [mcur, mend)
    int2 seg[kMaxSegments]; // the tile's row segments
    float4 cand[32];
    __align__(8) float cx[32];  // the candidates' coordinates again, as arrays: the exact
    __align__(8) float cy[32];  // test reads two candidates' x (y, z) in one 64-bit load
    __align__(8) float cz[32];
    float4 tpos[32];
    uint16_t plist[32 * 32];
    float tbuf[kDensityBatch];
};

template <bool kPrecise, bool kBatch, int kKern, bool kNZ>
__global__ void __launch_bounds__(128, kPrecise ? 9 : 10) k_density(const StepConst cp, const Buffers b,
                                                 DevState* ds) {
    if (ds->status) return;
    extern __shared__ __align__(16) unsigned char smem_raw_d[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    DensitySmem* S = reinterpret_cast<DensitySmem*>(smem_raw_d) + warp;
    const uint32_t ntiles = ds->n_tiles;
    // this warp's region of the hit-mask pool, filled tile after tile (record indices fit
    // 32 bits: the pool holds at most 0xffff0000 records)
    if (lane == 0) {
        const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
        const uint32_t region = b.hitmask ? (uint32_t)(b.hitmask_cap / nwarps) : 0u;
        S->mcur = (blockIdx.x * (blockDim.x >> 5) + warp) * region;
        S->mend = S->mcur + region;
    }
    __syncwarp();
    const float inf = __int_as_float(0x7f800000);
    uint32_t my_max = 0;
    for (uint32_t t = next_tile(&ds->work[0], lane); t < ntiles; t = next_tile(&ds->work[0], lane)) {
        const uint32_t k0 = b.tile_start[t];
        const int scene = kBatch ? (int)b.scene_s[k0] : 0;
        const StepConst& c = kBatch ? b.scenes[scene].c : cp;
        const Geom g = kBatch ? scene_geom(b.scenes[scene], ds) : grid_geom(ds);
        const float r2m = c.r2 * 1.0001f;
        Tile T;
        float4 xi;
        bool valid;
        int4 frame = make_int4(0, 0, 0, 0);
        if (kPrecise) tile_setup_cells(c, b, g, k0, lane, T, xi, valid, frame);
        else tile_setup(c, b, g, k0, lane, T, xi, valid);
        const int i = T.k0 + lane;
        {
            const TileBox B = tile_box(xi, valid);
            if (lane == 0) {
                S->box_lo = make_float4(B.lo[0], B.lo[1], B.lo[2], 0.0f);
                S->box_hi = make_float4(B.hi[0], B.hi[1], B.hi[2], 0.0f);
            }
        }
        S->tpos[lane] = xi;
        float rho = xmul(xi.w, c.w0);
        KSum rk;
        rk.s = rho;
        uint32_t nn = 0;
        // hit-mask records of this tile: from the warp's cursor on, one per chunk
        __syncwarp();
        const uint32_t slot = S->mcur, room = S->mend - slot;
        uint32_t nrec = 0;
        const int nseg = build_segments(b, g, T, lane, S->seg);
        __syncwarp();
        for (int sg = 0; sg < nseg; ++sg) {
            const int2 se = S->seg[sg];
            const int a = se.x, e = se.y;
            for (int s = a; s < e; s += kTile, ++nrec) {
                const int m = min(kTile, e - s);
                __syncwarp();
                float4 pl = lane < m ? b.pos4_s[s + lane] : make_float4(inf, inf, inf, 0.f);
                if (kPrecise && lane < m) pl = frame_pos(b.cell4_s[s + lane], frame, pl, c.cs);
                S->cand[lane] = pl;
                if (!kPrecise) {
                    S->cx[lane] = pl.x;
                    S->cy[lane] = pl.y;
                    S->cz[lane] = pl.z;
                }
                TileBox B;
                {
                    const float4 lo = S->box_lo, hi = S->box_hi;
                    B.lo[0] = lo.x, B.lo[1] = lo.y, B.lo[2] = lo.z;
                    B.hi[0] = hi.x, B.hi[1] = hi.y, B.hi[2] = hi.z;
                }
                const uint32_t surv = __ballot_sync(kFull, box_near(B, pl, r2m));
                __syncwarp();
                uint32_t* rec =
                    nrec < room ? b.hitmask + (size_t)(slot + nrec) * 32 + lane : nullptr;
                // streaming stores: the records must not evict the candidate arrays from L2
                if (!surv) {
                    if (rec) __stcs(rec, 0u);
                    continue;
                }
                uint32_t mask = 0u;
                if (valid) mask = kPrecise ? chunk_hits<true>(S->cand, surv, xi, c.r2)
                                           : chunk_hits_x2(S->cx, S->cy, S->cz, surv, xi, c.r2);
                if (rec) __stcs(rec, mask);
                nn += __popc(mask);
                const int self = i - s;
                const uint32_t selfbit = (unsigned)self < 32u ? 1u << self : 0u;
                mask &= ~selfbit;
                // dense chunk (collapsed cells): every particle of the tile hits every
                // candidate but itself; each lane adds its own terms in candidate order --
                // the flattened path's terms and additions, without the hit list and the
                // lane-by-lane fold
                const uint32_t all_m = m == 32 ? kFull : (1u << m) - 1u;
                if (__all_sync(kFull, !valid || mask == (all_m & ~selfbit))) {
                    float part = 0.0f;
                    for (int jj = 0; jj < m; ++jj) {
                        if (!valid || jj == self) continue;
                        const float4 xj = S->cand[jj];
                        if (kPrecise) {
                            const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                            part += xj.w * pair_w_fast<kKern>(c, fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                        } else {
                            rho = xadd(rho, xmul(xj.w, pair_w_exact<kKern, kNZ>(c, diff_d2(xi, xj))));
                        }
                    }
                    if (kPrecise) rk.add(part);
                    continue;
                }
                const uint32_t cnt = __popc(mask);
                uint32_t H;
                const uint32_t o = warp_excl_scan(cnt, lane, H);
                if (!H) continue;
                list_hits(S->plist, mask, o, lane);
                __syncwarp();
                float part = 0.0f;  // precision mode: this chunk's terms, one FP32 sum
                for (uint32_t base = 0; base < H; base += kDensityBatch) {
                    const uint32_t end = min(H, base + kDensityBatch);
                    for (uint32_t f = base + lane; f < end; f += 32) {
                        const uint32_t pr = S->plist[f];
                        const float4 xj = S->cand[pr & 31];
                        if (kPrecise) {
                            const float4 xt = S->tpos[pr >> 5];
                            const float dx = xt.x - xj.x, dy = xt.y - xj.y, dz = xt.z - xj.z;
                            S->tbuf[f - base] =
                                xj.w * pair_w_fast<kKern>(c, fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                        } else {
                            const float d2 = diff_d2(S->tpos[pr >> 5], xj);
                            S->tbuf[f - base] = xmul(xj.w, pair_w_exact<kKern, kNZ>(c, d2));
                        }
                    }
                    __syncwarp();
                    const uint32_t k1 = min(o + cnt, end);
                    if (kPrecise)
                        for (uint32_t k = max(o, base); k < k1; ++k) part += S->tbuf[k - base];
                    else
                        for (uint32_t k = max(o, base); k < k1; ++k) rho = xadd(rho, S->tbuf[k - base]);
                    __syncwarp();
                }
                if (kPrecise) rk.add(part);  // compensated across chunks
            }
        }
        if (b.hitmask && lane == 0) {
            const bool fits = nrec <= room;
            b.tile_slot[t] = fits ? slot : kNoSlot;
            if (fits) S->mcur = slot + nrec;
        }
        if (valid) {
            if (kPrecise) rho = rk.value();
            const float P = xmul(c.gas, xsub(rho, c.rest));
            // the per-candidate factors of the force pass's pair terms, each formed once here
            // with the rounding the reference applies per pair: exact mode (rho, P, 2 rho,
            // (m / rho) mu); precision mode (rho, P, m / (2 rho), (m / rho) mu)
            const float mr = xdiv(xi.w, rho);
            b.aux4_s[i] = kPrecise ? make_float4(rho, P, 0.5f * mr, mr * c.visc)
                                   : make_float4(rho, P, xmul(2.0f, rho), xmul(mr, c.visc));
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
// (compute_pressure_force / compute_viscosity_force / compute_acceleration,
//  sph_engine.cpp:390-443; integrate_leapfrog, cpp:290-310;
//  ParticleSystem::apply_boundary_conditions, particle.cpp:122-153)
// ---------------------------------------------------------------------------------------
struct ForceSmem {
    float4 box_lo, box_hi;  // tile box (the fallback walk's culling test)
    int2 seg[kMaxSegments]; // the tile's row segments
    float4 cpos[32], cvel[32], caux[32];
    float4 tpos[32], tvel[32];  // targets: x,y,z,m and vx,vy,vz,P
    uint16_t plist[32 * 32];
    float4 tbA[kForceBatch];  // -(pressure term) x, y and viscosity term x, y
    float2 tbB[kForceBatch];  // -(pressure term) z, viscosity term z
};

// The pair term of particle t against candidate j: the pressure-force contribution
// m_j * (P_t + P_j)/(2 rho_j) * gradW (the caller adds its negation, which equals
// subtracting it; +0 when |r| < 1e-6, where the reference skips it, and adding -0 leaves
// every float unchanged) and the viscosity contribution ((m_j/rho_j) mu (v_j - v_t))
// laplacianW (added), each with the reference's operations; aj.w holds (m_j/rho_j) mu.
template <int K>
__device__ __forceinline__ void force_term(const StepConst& c, const float4& xt,
                                           const float4& vt, float Pt, const float4& xj,
                                           const float4& vj, const float4& aj, float* p3,
                                           float* v3) {
    const Diff d = diff(xt, xj);
    const float r_len = xsqrt(d.d2);
    const bool skip = r_len < 1e-6f;
    p3[0] = p3[1] = p3[2] = 0.0f;
    float lap;
    if (K == SPHX_KERNEL_GAUSSIAN) {
        // GaussianKernel::gradW / laplacianW (kernels.cpp:215-225): both use
        // exp(-r_sq * sigma_sq_inv_) of the same r_sq -- one evaluation serves both
        const float e = expf(xmul(-d.d2, c.gs));
        if (!skip) {
            const float pt = xdiv(xadd(Pt, aj.y), aj.z);
            const float k = xmul(c.gg, e);
            const float sp = xmul(xj.w, pt);
            p3[0] = xmul(sp, xmul(k, d.x));
            p3[1] = xmul(sp, xmul(k, d.y));
            p3[2] = xmul(sp, xmul(k, d.z));
        }
        lap = xmul(xmul(c.gl, e), xsub(xmul(c.g2s, d.d2), 3.0f));
    } else {
        const float q = xdiv_fixed(r_len, c.h, c.rcp_h, c.fast_div_h);
        if (!skip) {
            const float pt = xdiv(xadd(Pt, aj.y), aj.z);
            const float sp = xmul(xj.w, pt);
            if (K == SPHX_KERNEL_WENDLAND_C2) {
                // WendlandC2Kernel::gradW (kernels.cpp:180-192):
                // norm * dW/dq * (r / (r_len h)), dW/dq = -5 tmp^3 q; 0 for q >= 2
                if (!(q >= 2.0f)) {
                    const float tmp = xsub(1.0f, xmul(0.5f, q));
                    const float dw = xmul(xmul(xmul(xmul(-5.0f, tmp), tmp), tmp), q);
                    const float gsc = xmul(c.wnorm, dw);
                    const float den = xmul(r_len, c.h);
                    p3[0] = xmul(sp, xmul(gsc, xdiv(d.x, den)));
                    p3[1] = xmul(sp, xmul(gsc, xdiv(d.y, den)));
                    p3[2] = xmul(sp, xmul(gsc, xdiv(d.z, den)));
                } else {
                    p3[0] = xmul(sp, 0.0f);
                    p3[1] = xmul(sp, 0.0f);
                    p3[2] = xmul(sp, 0.0f);
                }
            } else {
                float gx = 0.0f, gy = 0.0f, gz = 0.0f;
                if ((q >= 0.0f && q <= 1.0f) || (q > 1.0f && q <= 2.0f)) {
                    const float gf = cubic_grad_factor(c, q);
                    gx = xmul(gf, xdiv(d.x, r_len));
                    gy = xmul(gf, xdiv(d.y, r_len));
                    gz = xmul(gf, xdiv(d.z, r_len));
                }
                p3[0] = xmul(sp, xdiv_fixed(gx, c.h, c.rcp_h, c.fast_div_h));
                p3[1] = xmul(sp, xdiv_fixed(gy, c.h, c.rcp_h, c.fast_div_h));
                p3[2] = xmul(sp, xdiv_fixed(gz, c.h, c.rcp_h, c.fast_div_h));
            }
        }
        lap = K == SPHX_KERNEL_WENDLAND_C2 ? wendland_lap(c, q) : cubic_lap(c, q);
    }
    const float sv = aj.w;  // (m_j / rho_j) * mu, formed by the density pass
    v3[0] = xmul(xmul(sv, xsub(vj.x, vt.x)), lap);
    v3[1] = xmul(xmul(sv, xsub(vj.y, vt.y)), lap);
    v3[2] = xmul(xmul(sv, xsub(vj.z, vt.z)), lap);
}

// force_term<CUBIC_SPLINE> with the x and y components of every component-wise step done
// as packed FP32 pairs (same operations, same rounding, element by element); returns the
// record (-p.x, -p.y, v.x, v.y), (-p.z, v.z).  The pressure term is stored negated so that
// the caller's sums are all additions: x - p == x + (-p) in IEEE arithmetic, and the
// negated products are exact ((-s) * g == -(s * g)).  A skipped term is -0, the negation of
// the reference's +0 (x + (-0) == x - (+0) == x for every x).
// kNZ: the divisions by h and h^2 without range tests where bounds keep the dividends in
// xdiv_fixed_nz's range (|r| of a hit, the Laplacian's numerator); the gradient's
// components are tested once per pair and take the tested divisions only when one of
// them is nonzero and below 2^-100 in magnitude.
template <bool kNZ>
__device__ __forceinline__ void force_term_cubic_x2(const StepConst& c, const float4& xt,
                                                    const float4& vt, float Pt,
                                                    const float4& xj, const float4& vj,
                                                    const float4& aj, float4& A, float2& B) {
    const f32x2 dxy = xsub2(pk2(xt.x, xt.y), pk2(xj.x, xj.y));
    const float dz = xsub(xt.z, xj.z);
    const float2 sq = upk2(xmul2(dxy, dxy));
    const float r_len = xsqrt(xadd(xadd(sq.x, sq.y), xmul(dz, dz)));
    const float q = kNZ ? xdiv_fixed_nz(r_len, c.h, c.rcp_h)
                        : xdiv_fixed(r_len, c.h, c.rcp_h, c.fast_div_h);
    f32x2 pxy = pk2(-0.0f, -0.0f);
    float pz = -0.0f;
    if (kNZ) {
        // branch-free: every value is computed and the skipped cases are selected away (a
        // pair with |r| < 1e-6 may divide by zero here; its results are discarded)
        const bool live = !(r_len < 1e-6f);
        const bool in = (q >= 0.0f && q <= 1.0f) || (q > 1.0f && q <= 2.0f);
        const float sp = xmul(-xj.w, xdiv(xadd(Pt, aj.y), aj.z));  // -(m_j * pt)
        const float gf = cubic_grad_factor(c, q);
        const float2 d = upk2(dxy);
        const f32x2 gq = xmul2(pk2(gf, gf), pk2(xdiv(d.x, r_len), xdiv(d.y, r_len)));
        const float gzq = xmul(gf, xdiv(dz, r_len));
        const f32x2 gxy = in ? gq : pk2(0.0f, 0.0f);
        const float gz = in ? gzq : 0.0f;
        const float2 g = upk2(gxy);
        f32x2 pq;
        float pzq;
        if (nz_range(g.x) && nz_range(g.y) && nz_range(gz)) {
            pq = xmul2(pk2(sp, sp), xdiv_fixed2_nz(gxy, c.h, c.rcp_h));
            pzq = xmul(sp, xsign(xdiv_fixed_nz(gz, c.h, c.rcp_h), gz));
        } else {
            pq = xmul2(pk2(sp, sp), xdiv_fixed2(gxy, c.h, c.rcp_h, c.fast_div_h));
            pzq = xmul(sp, xdiv_fixed(gz, c.h, c.rcp_h, c.fast_div_h));
        }
        pxy = live ? pq : pxy;
        pz = live ? pzq : pz;
    } else if (!(r_len < 1e-6f)) {
        const float pt = xdiv(xadd(Pt, aj.y), aj.z);
        const float sp = xmul(-xj.w, pt);  // -(m_j * pt)
        f32x2 gxy = pk2(0.0f, 0.0f);
        float gz = 0.0f;
        if ((q >= 0.0f && q <= 1.0f) || (q > 1.0f && q <= 2.0f)) {
            const float gf = cubic_grad_factor(c, q);
            const float2 d = upk2(dxy);
            gxy = xmul2(pk2(gf, gf), pk2(xdiv(d.x, r_len), xdiv(d.y, r_len)));
            gz = xmul(gf, xdiv(dz, r_len));
        }
        pxy = xmul2(pk2(sp, sp), xdiv_fixed2(gxy, c.h, c.rcp_h, c.fast_div_h));
        pz = xmul(sp, xdiv_fixed(gz, c.h, c.rcp_h, c.fast_div_h));
    }
    const float lap = cubic_lap<kNZ>(c, q);
    const float sv = aj.w;  // (m_j / rho_j) * mu, formed by the density pass
    const f32x2 vxy = xmul2(xmul2(pk2(sv, sv), xsub2(pk2(vj.x, vj.y), pk2(vt.x, vt.y))),
                            pk2(lap, lap));
    const float vz = xmul(xmul(sv, xsub(vj.z, vt.z)), lap);
    const float2 p = upk2(pxy), v = upk2(vxy);
    A = make_float4(p.x, p.y, v.x, v.y);
    B = make_float2(pz, vz);
}

// Precision-mode pair term: the pressure and viscosity contributions of candidate j to the
// force on particle t, summed into one vector (the mode is judged against FP64, not against
// the reference's summation order), with contracted FP32 arithmetic, the hardware
// reciprocal square root and exponential, and the candidate's factors of the density
// pass in aj = (rho, P, m / (2 rho), (m / rho) mu).  Formulas: equations::compute_pressure_force /
// compute_viscosity_force (sph_engine.cpp:390-432) with grad W = g * r_vec and
// laplacian W = lap of the kernel; the pressure term is skipped for |r| < 1e-6.
template <int K>
__device__ __forceinline__ float3 force_term_fast(const StepConst& c, const float4& xt,
                                                  const float4& vt, float Pt, const float4& xj,
                                                  const float4& vj, const float4& aj) {
    const float dx = xt.x - xj.x, dy = xt.y - xj.y, dz = xt.z - xj.z;
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float r, rinv;
    fast_len(d2, r, rinv);
    float g, lap;
    if (K == SPHX_KERNEL_GAUSSIAN) {
        const float e = __expf(-d2 * c.gs);
        g = c.gg * e;
        lap = c.gl * e * fmaf(c.g2s, d2, -3.0f);
    } else {
        const float q = r * c.rcp_h;
        if (K == SPHX_KERNEL_WENDLAND_C2) {
            const float t = fmaf(-0.5f, q, 1.0f);
            const bool in = q < 2.0f;
            g = in ? c.wnorm * (-5.0f * (t * t * t) * q) * (rinv * c.rcp_h) : 0.0f;
            lap = in ? c.wl * (t * t) * fmaf(5.0f, q, -3.0f) : 0.0f;
        } else {
            const float t = 2.0f - q;
            const float gf = q <= 1.0f ? c.sigma * q * fmaf(1.5f, q, -2.0f)
                                       : (q <= 2.0f ? -0.5f * c.sigma * (t * t) : 0.0f);
            g = gf * (rinv * c.rcp_h);
            const float sh = c.sigma * c.rcp_hsq;
            lap = q <= 1.0f ? sh * fmaf(3.0f, q, -2.0f) : (q <= 2.0f ? sh * t : 0.0f);
        }
    }
    if (r < 1e-6f) g = 0.0f;
    const float cp = -(aj.z * (Pt + aj.y)) * g;  // -(m_j (P_t + P_j) / (2 rho_j)) g
    const float cv = aj.w * lap;                  // (m_j / rho_j) mu lap
    return make_float3(fmaf(cp, dx, cv * (vj.x - vt.x)), fmaf(cp, dy, cv * (vj.y - vt.y)),
                       fmaf(cp, dz, cv * (vj.z - vt.z)));
}

// Precision-mode leapfrog + wall clamp on cell + offset positions (FP64 clamp).
__device__ __forceinline__ void integrate_cells(const StepConst& c, float dt, const float* acc,
                                                float* o, float* v, int4& cell) {
    int* cc[3] = {&cell.x, &cell.y, &cell.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float half = 0.5f * acc[a] * dt;
        float vv = v[a] + half;
        float on = o[a] + vv * dt;
        vv = vv + half;
        v[a] = vv * c.damping;
        if (!isfinite(on)) {  // the position is lost: park the particle as non-finite
            cell.w = 1;
            o[a] = on;
            continue;
        }
        double X = (double)(*cc[a]) * c.cs_d + (double)on;
        if (X < (double)c.lo[a]) {
            X = c.lo[a];
            v[a] = v[a] * -0.8f;
        } else if (X > (double)c.hi[a]) {
            X = c.hi[a];
            v[a] = v[a] * -0.8f;
        }
        double f = floor(X / c.cs_d);
        f = fmin(fmax(f, -(double)kCellClamp), (double)(kCellClamp - 1));
        int ci = (int)f;
        float oo = (float)(X - (double)ci * c.cs_d);
        if (c.fp16) oo = round_half(oo);
        if (oo >= c.cs) {
            oo = 0.0f;
            ci += 1;
        } else if (oo < 0.0f) {
            oo = 0.0f;
        }
        *cc[a] = ci;
        o[a] = oo;
    }
}

template <bool kIntegrate, bool kPrecise, bool kBatch, int kKern, bool kNZ>
__global__ void __launch_bounds__(128, kPrecise ? 6 : 7) k_force(const StepConst cp, const Buffers b,
                                               DevState* ds) {
    if (ds->status) return;
    extern __shared__ __align__(16) unsigned char smem_raw_f[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ForceSmem* S = reinterpret_cast<ForceSmem*>(smem_raw_f) + warp;
    const uint32_t ntiles = ds->n_tiles;
    const float inf = __int_as_float(0x7f800000);
    for (uint32_t t = next_tile(&ds->work[1], lane); t < ntiles; t = next_tile(&ds->work[1], lane)) {
        const uint32_t k0 = b.tile_start[t];
        const int scene = kBatch ? (int)b.scene_s[k0] : 0;
        const StepConst& c = kBatch ? b.scenes[scene].c : cp;
        const Geom g = kBatch ? scene_geom(b.scenes[scene], ds) : grid_geom(ds);
        const float r2m = c.r2 * 1.0001f;
        Tile T;
        float4 xi;
        bool valid;
        int4 frame = make_int4(0, 0, 0, 0);
        if (kPrecise) tile_setup_cells(c, b, g, k0, lane, T, xi, valid, frame);
        else tile_setup(c, b, g, k0, lane, T, xi, valid);
        const int i = T.k0 + lane;
        const float4 vi0 = valid ? b.vel4_s[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float Pi = valid ? b.aux4_s[i].y : 0.0f;
        // hit masks of the density pass (same walk, same chunks, same tests)
        const uint32_t slot = b.tile_slot ? b.tile_slot[t] : kNoSlot;
        if (slot == kNoSlot) {
            const TileBox B = tile_box(xi, valid);
            if (lane == 0) {
                S->box_lo = make_float4(B.lo[0], B.lo[1], B.lo[2], 0.0f);
                S->box_hi = make_float4(B.hi[0], B.hi[1], B.hi[2], 0.0f);
            }
        }
        S->tpos[lane] = xi;
        S->tvel[lane] = make_float4(vi0.x, vi0.y, vi0.z, Pi);
        // force sums, packed: pressure (x, y), viscosity (x, y), (pressure z, viscosity z)
        f32x2 fpxy = pk2(0.0f, 0.0f), fvxy = pk2(0.0f, 0.0f), fz = pk2(0.0f, 0.0f);
        KSum Fx, Fy, Fz;  // precision mode: one compensated sum per component
        const uint32_t* rec = slot != kNoSlot ? b.hitmask + (size_t)slot * 32 + lane : nullptr;
        uint32_t mnext =
            rec && (size_t)(rec - b.hitmask) < (size_t)b.hitmask_cap * 32 ? __ldcs(rec) : 0u;
        const int nseg = build_segments(b, g, T, lane, S->seg);
        __syncwarp();
        for (int sg = 0; sg < nseg; ++sg) {
            const int2 se = S->seg[sg];
            const int a = se.x, e = se.y;
            for (int s = a; s < e; s += kTile, rec += rec ? 32 : 0) {
                const int m = min(kTile, e - s);
                uint32_t mask;
                __syncwarp();
                if (rec) {
                    mask = mnext;
                    // the next chunk's record, loaded a chunk ahead (past the tile's last
                    // chunk it reads another tile's record, or nothing at the pool's end)
                    mnext = (size_t)(rec + 32 - b.hitmask) < (size_t)b.hitmask_cap * 32
                                ? __ldcs(rec + 32) : 0u;
                    const uint32_t used = __reduce_or_sync(kFull, mask);  // candidates hit
                    if (!used) continue;
                    if (used & (1u << lane)) {
                        float4 pl = b.pos4_s[s + lane];
                        if (kPrecise) pl = frame_pos(b.cell4_s[s + lane], frame, pl, c.cs);
                        S->cpos[lane] = pl;
                        S->cvel[lane] = b.vel4_s[s + lane];
                        S->caux[lane] = b.aux4_s[s + lane];
                    }
                    __syncwarp();
                } else {
                    const bool in = lane < m;
                    float4 pl = in ? b.pos4_s[s + lane] : make_float4(inf, inf, inf, 0.f);
                    if (kPrecise && in) pl = frame_pos(b.cell4_s[s + lane], frame, pl, c.cs);
                    S->cpos[lane] = pl;
                    __syncwarp();
                    TileBox B;
                    const float4 lo = S->box_lo, hi = S->box_hi;
                    B.lo[0] = lo.x, B.lo[1] = lo.y, B.lo[2] = lo.z;
                    B.hi[0] = hi.x, B.hi[1] = hi.y, B.hi[2] = hi.z;
                    const uint32_t surv = __ballot_sync(kFull, box_near(B, pl, r2m));
                    if (!surv) continue;
                    if (surv & (1u << lane)) {
                        S->cvel[lane] = b.vel4_s[s + lane];
                        S->caux[lane] = b.aux4_s[s + lane];
                    }
                    __syncwarp();
                    mask = valid ? chunk_hits<kPrecise>(S->cpos, surv, xi, c.r2) : 0u;
                }
                const int self = i - s;
                if ((unsigned)self < 32u) mask &= ~(1u << self);
                const uint32_t cnt = __popc(mask);
                uint32_t H;
                const uint32_t o = warp_excl_scan(cnt, lane, H);
                if (!H) continue;
                list_hits(S->plist, mask, o, lane);
                __syncwarp();
                float px = 0.0f, py = 0.0f, pz = 0.0f;  // precision mode: this chunk's sums
                for (uint32_t base = 0; base < H; base += kForceBatch) {
                    const uint32_t end = min(H, base + kForceBatch);
                    for (uint32_t f = base + lane; f < end; f += 32) {
                        const uint32_t pr = S->plist[f];
                        const int tt = pr >> 5, jj = pr & 31;
                        float p3[3], v3[3];
                        const float4 vt = S->tvel[tt];
                        const uint32_t u = f - base;
                        if (!kPrecise && kKern == SPHX_KERNEL_CUBIC_SPLINE) {
                            float4 A;
                            float2 Bp;
                            force_term_cubic_x2<kNZ>(c, S->tpos[tt], vt, vt.w, S->cpos[jj],
                                                S->cvel[jj], S->caux[jj], A, Bp);
                            S->tbA[u] = A;
                            S->tbB[u] = Bp;
                            continue;
                        }
                        if (kPrecise) {
                            const float3 fv = force_term_fast<kKern>(c, S->tpos[tt], vt, vt.w,
                                                                     S->cpos[jj], S->cvel[jj],
                                                                     S->caux[jj]);
                            S->tbA[u] = make_float4(fv.x, fv.y, fv.z, 0.0f);
                            continue;
                        }
                        force_term<kKern>(c, S->tpos[tt], vt, vt.w, S->cpos[jj], S->cvel[jj],
                                          S->caux[jj], p3, v3);
                        S->tbA[u] = make_float4(-p3[0], -p3[1], v3[0], v3[1]);
                        S->tbB[u] = make_float2(-p3[2], v3[2]);
                    }
                    __syncwarp();
                    const uint32_t k1 = min(o + cnt, end);
                    for (uint32_t k = max(o, base); k < k1; ++k) {
                        const uint32_t u = k - base;
                        const float4 A = S->tbA[u];
                        if (kPrecise) {
                            px += A.x;
                            py += A.y;
                            pz += A.z;
                            continue;
                        }
                        const float2 Bv = S->tbB[u];
                        // the records hold -(pressure term): three packed additions
                        fpxy = xadd2(fpxy, pk2(A.x, A.y));
                        fvxy = xadd2(fvxy, pk2(A.z, A.w));
                        fz = xadd2(fz, pk2(Bv.x, Bv.y));
                    }
                    __syncwarp();
                }
                if (kPrecise) {  // compensated across chunks
                    Fx.add(px);
                    Fy.add(py);
                    Fz.add(pz);
                }
            }
        }
        __syncwarp();
        if (!valid) continue;
        const float mi = xi.w;
        float ax, ay, az;
        if (kPrecise) {
            ax = Fx.value() / mi;
            ay = (Fy.value() + c.grav * mi) / mi;
            az = Fz.value() / mi;
        } else {
            const float2 fp = upk2(fpxy), fv = upk2(fvxy), fzz = upk2(fz);
            const float fpz = fzz.x, fvz = fzz.y;
            ax = xdiv(xadd(xadd(fp.x, fv.x), xmul(0.0f, mi)), mi);
            ay = xdiv(xadd(xadd(fp.y, fv.y), xmul(c.grav, mi)), mi);
            az = xdiv(xadd(xadd(fpz, fvz), xmul(0.0f, mi)), mi);
        }
        b.acc4_s[i] = make_float4(ax, ay, az, 0.0f);
        if (!kIntegrate) continue;
        const float dt = kBatch ? b.scenes[scene].dt : ds->dt;
        const float4 vi = S->tvel[lane];
        const uint32_t id = b.id_s[i];
        if (kPrecise) {
            int4 cell = b.cell4_s[i];
            const float4 own = b.pos4_s[i];
            float o[3] = {own.x, own.y, own.z}, v[3] = {vi.x, vi.y, vi.z};
            const float acc[3] = {ax, ay, az};
            if (!cell.w) integrate_cells(c, dt, acc, o, v, cell);
            b.cell4[id] = cell;
            b.pos4[id] = make_float4(o[0], o[1], o[2], mi);
            b.vel4[id] = make_float4(v[0], v[1], v[2], 0.0f);
            if (id == 0) {
                ds->a0[0] = ax;
                ds->a0[1] = ay;
                ds->a0[2] = az;
            }
            continue;
        }
        float x[3] = {xi.x, xi.y, xi.z}, v[3] = {vi.x, vi.y, vi.z};
        const float acc[3] = {ax, ay, az};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float half = xmul(xmul(0.5f, acc[a]), dt);
            float vv = xadd(v[a], half);
            x[a] = xadd(x[a], xmul(vv, dt));
            vv = xadd(vv, half);
            v[a] = xmul(vv, c.damping);
            if (x[a] < c.lo[a]) {
                x[a] = c.lo[a];
                v[a] = xmul(v[a], -0.8f);
            } else if (x[a] > c.hi[a]) {
                x[a] = c.hi[a];
                v[a] = xmul(v[a], -0.8f);
            }
        }
        b.pos4[id] = make_float4(x[0], x[1], x[2], mi);
        b.vel4[id] = make_float4(v[0], v[1], v[2], 0.0f);
        if (kBatch) {
            if (id == b.scenes[scene].start) {  // accelerations_[0] of the scene
                b.scenes[scene].a0[0] = ax;
                b.scenes[scene].a0[1] = ay;
                b.scenes[scene].a0[2] = az;
            }
        } else if (id == 0) {
            ds->a0[0] = ax;
            ds->a0[1] = ay;
            ds->a0[2] = az;
        }
    }
}

// ---------------------------------------------------------------------------------------
// neighbour-list dump (test hook): same walk, lists written in iteration order
// ---------------------------------------------------------------------------------------
template <bool kFill, bool kPrecise>
__global__ void __launch_bounds__(128) k_pairs(const StepConst c, const Buffers b,
                                               const DevState* ds, uint32_t* counts_by_id,
                                               const uint64_t* off_by_id, int64_t* out) {
    if (ds->status) return;
    extern __shared__ float4 smem_p[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float4* cand = smem_p + warp * kTile;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t ntiles = ds->n_tiles;
    for (uint32_t t = blockIdx.x * (blockDim.x >> 5) + warp; t < ntiles; t += nwarps) {
        const uint32_t k0 = b.tile_start[t];
        const Geom g = grid_geom(ds);
        Tile T;
        float4 xi;
        bool valid;
        int4 frame = make_int4(0, 0, 0, 0);
        if (kPrecise) tile_setup_cells(c, b, g, k0, lane, T, xi, valid, frame);
        else tile_setup(c, b, g, k0, lane, T, xi, valid);
        const int i = T.k0 + lane;
        const uint32_t id = valid ? b.id_s[i] : 0u;
        uint64_t pos = (kFill && valid) ? off_by_id[id] : 0ull;
        const bool want = !kFill || pos != kNoPairs;  // fill: particles with an offset only
        uint32_t nn = 0;
        for_each_row(b, g, T, [&](int a, int e) {
            for (int s = a; s < e; s += kTile) {
                const int m = min(kTile, e - s);
                __syncwarp();
                if (lane < m) {
                    float4 p = b.pos4_s[s + lane];
                    if (kPrecise) p = frame_pos(b.cell4_s[s + lane], frame, p, c.cs);
                    cand[lane] = p;
                }
                __syncwarp();
                for (int jj = 0; jj < m; ++jj) {
                    float d2;
                    if (kPrecise) {
                        const float4 xj = cand[jj];
                        const float dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                        d2 = dx * dx + dy * dy + dz * dz;
                    } else {
                        d2 = diff(xi, cand[jj]).d2;
                    }
                    if (valid && d2 <= c.r2) {
                        if (kFill && want) out[pos++] = (int64_t)b.id_s[s + jj];
                        ++nn;
                    }
                }
            }
        });
        if (!kFill && valid) counts_by_id[id] = nn;
    }
}

// Persistent grid: as many CTAs as fit on the GPU (queried once per kernel).
template <class K>
static int resident_blocks(const LaunchCtx& L, K kernel, int threads, size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) !=
            cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    if (L.blocks_per_sm > 0 && L.blocks_per_sm < per_sm) per_sm = L.blocks_per_sm;
    return L.num_sms * per_sm;
}

// Grid sizes of the persistent passes, found once per (device, kernel instantiation, warps
// per block, requested CTAs per SM) and kept: one cache object per instantiation, indexed
// by device; any host thread may fill an entry (a racing fill stores the same value).
constexpr int kMaxCacheDevices = 64;
struct LaunchShapeCache {
    std::atomic<int> nb[kMaxCacheDevices][5][33];
    std::atomic<int>& at(const LaunchCtx& L) {
        const int d = L.device >= 0 && L.device < kMaxCacheDevices ? L.device : 0;
        const int w = L.warps_per_block >= 0 && L.warps_per_block <= 4 ? L.warps_per_block : 4;
        const int b = L.blocks_per_sm >= 0 && L.blocks_per_sm < 32 ? L.blocks_per_sm : 32;
        return nb[d][w][b];
    }
};

template <class K>
static int cached_resident_blocks(LaunchShapeCache& cache, const LaunchCtx& L, K kernel,
                                  int threads, size_t smem) {
    std::atomic<int>& slot = cache.at(L);
    int nb = slot.load(std::memory_order_relaxed);
    if (!nb) {
        nb = resident_blocks(L, kernel, threads, smem);
        slot.store(nb, std::memory_order_relaxed);
    }
    return nb;
}

static int pass_blocks(const LaunchCtx& L) {
    const int bps = L.blocks_per_sm > 0 ? L.blocks_per_sm : 8;
    return L.num_sms * bps;
}

template <bool kPrecise, bool kBatch, int kKern, bool kNZ = false>
static void launch_density_t(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                             DevState* ds) {
    const int threads = 32 * L.warps_per_block;
    const size_t sm = (size_t)L.warps_per_block * sizeof(DensitySmem);
    static LaunchShapeCache cache;
    const int nb = cached_resident_blocks(cache, L, k_density<kPrecise, kBatch, kKern, kNZ>,
                                          threads, sm);
    k_density<kPrecise, kBatch, kKern, kNZ><<<nb, threads, sm, L.stream>>>(c, b, ds);
}

template <int kKern>
static void launch_density_k(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                             DevState* ds) {
    const bool nz = kKern == SPHX_KERNEL_CUBIC_SPLINE && !c.precise && c.div_nz;
    if (b.nscenes > 0) {
        if (nz) launch_density_t<false, true, kKern, true>(L, c, b, ds);
        else launch_density_t<false, true, kKern>(L, c, b, ds);
    } else if (c.precise) launch_density_t<true, false, kKern>(L, c, b, ds);
    else if (nz) launch_density_t<false, false, kKern, true>(L, c, b, ds);
    else launch_density_t<false, false, kKern>(L, c, b, ds);
}

int launch_density(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds) {
    if (c.kern == SPHX_KERNEL_WENDLAND_C2) launch_density_k<SPHX_KERNEL_WENDLAND_C2>(L, c, b, ds);
    else if (c.kern == SPHX_KERNEL_GAUSSIAN) launch_density_k<SPHX_KERNEL_GAUSSIAN>(L, c, b, ds);
    else launch_density_k<SPHX_KERNEL_CUBIC_SPLINE>(L, c, b, ds);
    return 1;
}

template <bool kIntegrate, bool kPrecise, bool kBatch, int kKern, bool kNZ = false>
static void launch_force_t(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                           DevState* ds) {
    const int threads = 32 * L.warps_per_block;
    const size_t sm = (size_t)L.warps_per_block * sizeof(ForceSmem);
    static LaunchShapeCache cache;
    const int nb = cached_resident_blocks(
        cache, L, k_force<kIntegrate, kPrecise, kBatch, kKern, kNZ>, threads, sm);
    k_force<kIntegrate, kPrecise, kBatch, kKern, kNZ><<<nb, threads, sm, L.stream>>>(c, b, ds);
}

template <int kKern>
static void launch_force_k(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                           DevState* ds, int integrate) {
    const bool nz = kKern == SPHX_KERNEL_CUBIC_SPLINE && !c.precise && c.div_nz;
    if (b.nscenes > 0) {
        if (integrate) {
            if (nz) launch_force_t<true, false, true, kKern, true>(L, c, b, ds);
            else launch_force_t<true, false, true, kKern>(L, c, b, ds);
        } else launch_force_t<false, false, true, kKern>(L, c, b, ds);
    } else if (integrate) {
        if (c.precise) launch_force_t<true, true, false, kKern>(L, c, b, ds);
        else if (nz) launch_force_t<true, false, false, kKern, true>(L, c, b, ds);
        else launch_force_t<true, false, false, kKern>(L, c, b, ds);
    } else {
        if (c.precise) launch_force_t<false, true, false, kKern>(L, c, b, ds);
        else if (nz) launch_force_t<false, false, false, kKern, true>(L, c, b, ds);
        else launch_force_t<false, false, false, kKern>(L, c, b, ds);
    }
}

int launch_force(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds,
                 int integrate) {
    if (c.kern == SPHX_KERNEL_WENDLAND_C2)
        launch_force_k<SPHX_KERNEL_WENDLAND_C2>(L, c, b, ds, integrate);
    else if (c.kern == SPHX_KERNEL_GAUSSIAN)
        launch_force_k<SPHX_KERNEL_GAUSSIAN>(L, c, b, ds, integrate);
    else
        launch_force_k<SPHX_KERNEL_CUBIC_SPLINE>(L, c, b, ds, integrate);
    return 1;
}

void launch_pair_counts(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                        DevState* ds, uint32_t* counts_by_id) {
    const size_t sm = (size_t)L.warps_per_block * kTile * sizeof(float4);
    if (c.precise)
        k_pairs<false, true><<<pass_blocks(L), 32 * L.warps_per_block, sm, L.stream>>>(
            c, b, ds, counts_by_id, nullptr, nullptr);
    else
        k_pairs<false, false><<<pass_blocks(L), 32 * L.warps_per_block, sm, L.stream>>>(
            c, b, ds, counts_by_id, nullptr, nullptr);
}

void launch_pair_fill(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                      DevState* ds, const uint64_t* offsets_by_id, int64_t* out_idx) {
    const size_t sm = (size_t)L.warps_per_block * kTile * sizeof(float4);
    if (c.precise)
        k_pairs<true, true><<<pass_blocks(L), 32 * L.warps_per_block, sm, L.stream>>>(
            c, b, ds, nullptr, offsets_by_id, out_idx);
    else
        k_pairs<true, false><<<pass_blocks(L), 32 * L.warps_per_block, sm, L.stream>>>(
            c, b, ds, nullptr, offsets_by_id, out_idx);
}

}  // namespace sphx
