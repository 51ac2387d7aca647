// Shared device code of the neighbour passes (density + pressure in sphx_density.cu, force +
// leapfrog + wall clamp in sphx_force.cu, the neighbour-list dump in sphx_passes.cu): tiles,
// the stencil walk, the chunk machinery, the pair arithmetic helpers and the launch-shape
// cache.
//
// Work decomposition: one warp owns one tile (up to 32 consecutive cell-sorted particles of
// one cell column (x, y, *), one particle per lane; a tile may span several cells of its
// column).  All lanes of a tile share the tile's stencil: for each row (dx, dy) the cells
// cz+lo..cz+hi (covering every lane's cell +-1, +-2 near a face) are one contiguous range
// of the sorted arrays; the warp stages that range through shared memory 32 candidates at
// a time and every lane tests every candidate against its own particle.
//
// Exactness.  The reference walks, for particle i, the cells (dx, dy, dz) of its stencil
// in lexicographic order and each cell's particles in insertion order
// (spatial_hash.cpp:31-57), and accumulates every sum sequentially in that order
// (sph_engine.cpp:370-432).  The sorted arrays hold each cell's particles in insertion
// order (stable sort from insertion order), the rows are walked in (dx, dy) order and
// each row in increasing z, so a lane meets its neighbours in exactly the reference's
// order.  The reference scans a 5x5x5 block (cell_radius = 2); a neighbour at distance
// <= r can only sit two cells away when the particle lies within rounding distance of a
// cell face, so the tile's stencil is the 3x3x3 block of each of its cells, widened on an
// axis to the second layer when some lane is that close to a face (guard band eps below).
// Cells of the tile's rows outside a lane's own 5x5x5 block hold no neighbour of it (they
// are more than two cells away), so they add only misses to that lane's walk, and the
// cells of its block keep their relative order.  Every distance test and
// every term uses the reference's float operations in the reference's order with
// IEEE round-to-nearest and no contraction, so each lane's sums are bit-identical.
#pragma once
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

// End (sorted position) of the run a tile of cell `key` may fill: the cell, or (b.columns)
// its cell column -- its column run where b.runs holds them (single scene) -- (the
// non-finite group is its own column).
__device__ __forceinline__ uint32_t tile_run_end(const Buffers& b, const Geom& g, uint32_t key) {
    if (!b.columns || key >= g.sentinel) return b.off[key + 1];
    if (b.runs && !b.nscenes) return b.runs[key].y;
    const uint32_t d2 = (uint32_t)g.dim[2];
    return b.off[g.base + ((key - g.base) / d2 + 1u) * d2];
}

// The tile's z range relative to its first particle's cell: every lane's cell +-1, or +-2
// on the side where the lane lies within the guard band of a cell face.
__device__ __forceinline__ void tile_z_range(const Buffers& b, const Geom& g, uint32_t k0,
                                             int lane, bool valid, bool near_lo, bool near_hi,
                                             Tile& T) {
    const uint32_t kl = valid ? b.key_s[k0 + lane] : b.key_s[k0];
    const int rz = (int)((kl - g.base) % (uint32_t)g.dim[2]) - T.cz;  // >= 0 (sorted)
    T.lo[2] = __reduce_min_sync(0xffffffffu, rz + (near_lo ? -2 : -1));
    T.hi[2] = __reduce_max_sync(0xffffffffu, rz + (near_hi ? 2 : 1));
}

// Sets up the tile starting at sorted position k0; returns the lane's particle (valid
// lanes only).
__device__ __forceinline__ void tile_setup(const StepConst& c, const Buffers& b, const Geom& g,
                                           uint32_t k0, int lane, Tile& T, float4& xi,
                                           bool& valid) {
    const uint32_t key = b.key_s[k0];
    const uint32_t end = tile_run_end(b, g, key);
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
    bool lo_z = false, hi_z = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // position inside the cell in cell units; the guard band covers the rounding of
        // x*inv_cell and of the distance test (a few ulps of |u|) with a wide margin
        const float u = xmul(x[a], c.inv_cell);
        const float frac = u - floorf(u);
        const float eps = 1.52587890625e-5f + fabsf(u) * 9.5367431640625e-7f;
        const bool near_lo = valid && frac < eps;
        const bool near_hi = valid && (1.0f - frac) < eps;
        if (a == 2) {
            lo_z = near_lo;
            hi_z = near_hi;
        } else {
            T.lo[a] = __any_sync(0xffffffffu, near_lo) ? -2 : -1;
            T.hi[a] = __any_sync(0xffffffffu, near_hi) ? 2 : 1;
        }
    }
    tile_z_range(b, g, k0, lane, valid, lo_z, hi_z, T);
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
    const uint32_t end = tile_run_end(b, g, key);
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
    bool lo_z = false, hi_z = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const bool near_lo = valid && off[a] < eps;
        const bool near_hi = valid && (c.cs - off[a]) < eps;
        if (a == 2) {
            lo_z = near_lo;
            hi_z = near_hi;
        } else {
            T.lo[a] = __any_sync(0xffffffffu, near_lo) ? -2 : -1;
            T.hi[a] = __any_sync(0xffffffffu, near_hi) ? 2 : 1;
        }
    }
    tile_z_range(b, g, k0, lane, valid, lo_z, hi_z, T);
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
    if (w2 && z1 - z0 + 1 >= d2) {  // the range covers the folded axis: each cell once
        z0 = 0;
        z1 = d2 - 1;
    } else if (w2) {
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
    if (g.wrap[2] && z1 - z0 + 1 >= d2) {  // the range covers the folded axis: each cell once
        z0 = 0;
        z1 = d2 - 1;
    } else if (g.wrap[2]) {
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

// Hit mask of this lane's particle against the staged chunk (candidates in `surv` only):
// the reference's rounded test.
__device__ __forceinline__ uint32_t chunk_hits(const float4* cand, uint32_t surv,
                                               const float4& xi, float r2) {
    uint32_t mask = 0;
#pragma unroll
    for (int jj = 0; jj < 32; ++jj) {
        if (surv & (1u << jj)) {
            if (diff(xi, cand[jj]).d2 <= r2) mask |= 1u << jj;
        }
    }
    return mask;
}

// chunk_hits two candidates at a time with packed FP32 pairs: the same exact test
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

// W of the pair (x_i - x_j = (dx, dy, dz), d2 = |.|^2) for smoothing kernel K, with the
// reference's float operations (Kernel::W, kernels.cpp:140-143, 172-178, 210-213).
// kNZ: d2 <= r^2 (a hit), so |r| is +0 or in [2^-74.5, r (1 + 2^-23)], which the host
// keeps inside xdiv_fixed_nz's range
template <int K, bool kNZ = false>
__device__ __forceinline__ float pair_w_exact(const StepConst& c, float d2) {
    if (K == SPHX_KERNEL_GAUSSIAN) return xmul(c.wnorm, expf(xmul(-d2, c.gs)));
    const float q = kNZ ? xdiv_fixed_nz(xsqrt(d2), c.h, c.rcp_h)
                        : xdiv_fixed(xsqrt(d2), c.h, c.rcp_h, c.fast_div_h);
    return K == SPHX_KERNEL_WENDLAND_C2 ? wendland_w(c, q) : cubic_w(c, q);
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

// Work distribution: warps take tiles from a per-pass counter (dynamic, so crowded cells
// in degenerate states do not serialise the tail).
__device__ __forceinline__ uint32_t next_tile(uint32_t* ctr, int lane) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(ctr, 1u);
    return __shfl_sync(kFull, t, 0);
}

// Persistent grid: as many CTAs as fit on the GPU (queried once per kernel).
template <class K>
inline int resident_blocks(const LaunchCtx& L, K kernel, int threads, size_t smem) {
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
inline int cached_resident_blocks(LaunchShapeCache& cache, const LaunchCtx& L, K kernel,
                                  int threads, size_t smem) {
    std::atomic<int>& slot = cache.at(L);
    int nb = slot.load(std::memory_order_relaxed);
    if (!nb) {
        nb = resident_blocks(L, kernel, threads, smem);
        slot.store(nb, std::memory_order_relaxed);
    }
    return nb;
}

inline int pass_blocks(const LaunchCtx& L) {
    const int bps = L.blocks_per_sm > 0 ? L.blocks_per_sm : 8;
    return L.num_sms * bps;
}

}  // namespace sphx
