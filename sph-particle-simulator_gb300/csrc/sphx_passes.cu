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
#include "sphx_internal.cuh"

namespace sphx {

struct Tile {
    int k0;       // first sorted position of the tile
    int cnt;      // particles in the tile (<= 32)
    bool cells;   // false for the group of non-finite particles (no neighbours)
    int cx, cy, cz;
    int lo[3], hi[3];
};

// Sets up tile t for this warp; returns the lane's particle (valid lanes only).
__device__ __forceinline__ void tile_setup(const StepConst& c, const Buffers& b,
                                           const DevState* ds, uint32_t t, int lane, Tile& T,
                                           float4& xi, bool& valid) {
    const uint32_t k0 = b.tile_start[t];
    const uint32_t key = b.key_s[k0];
    const uint32_t nc = ds->ncells;
    const uint32_t end = b.off[key + 1];
    T.k0 = (int)k0;
    T.cnt = (int)min(end - k0, (uint32_t)kTile);
    valid = lane < T.cnt;
    xi = valid ? b.pos4_s[k0 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    T.cells = key < nc;
    if (!T.cells) return;
    const uint32_t dz = ds->dim[2], dy = ds->dim[1];
    T.cz = (int)(key % dz);
    T.cy = (int)((key / dz) % dy);
    T.cx = (int)(key / (dz * dy));
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

// Calls f(begin, end) for every stencil row of the tile, in the reference's order.  On a
// folded axis the neighbour index wraps; a row that wraps on z is two segments, visited
// in dz order.
template <class F>
__device__ __forceinline__ void for_each_row(const Buffers& b, const DevState* ds,
                                             const Tile& T, F&& f) {
    if (!T.cells) return;
    const int d0 = ds->dim[0], d1 = ds->dim[1], d2 = ds->dim[2];
    const bool w0 = ds->wrap[0], w1 = ds->wrap[1], w2 = ds->wrap[2];
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
            const uint32_t rb = ((uint32_t)X * (uint32_t)d1 + (uint32_t)Y) * (uint32_t)d2;
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

// ---------------------------------------------------------------------------------------
// density + pressure:  rho_i = m_i W(0) + sum_{j in N(i), j != i} m_j W(r_ij)
//                      P_i = k (rho_i - rho0)
// (compute_density / compute_pressure, sph_engine.cpp:370-388)
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_density(const StepConst c, const Buffers b,
                                                 DevState* ds) {
    if (ds->status) return;
    extern __shared__ float4 smem_d[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float4* cand = smem_d + warp * kTile;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t ntiles = ds->n_tiles;
    uint32_t my_max = 0;
    for (uint32_t t = blockIdx.x * (blockDim.x >> 5) + warp; t < ntiles; t += nwarps) {
        Tile T;
        float4 xi;
        bool valid;
        tile_setup(c, b, ds, t, lane, T, xi, valid);
        const int i = T.k0 + lane;
        float rho = xmul(xi.w, c.w0);
        uint32_t nn = 0;
        for_each_row(b, ds, T, [&](int a, int e) {
            for (int s = a; s < e; s += kTile) {
                const int m = min(kTile, e - s);
                __syncwarp();
                if (lane < m) cand[lane] = b.pos4_s[s + lane];
                __syncwarp();
                for (int jj = 0; jj < m; ++jj) {
                    const float4 xj = cand[jj];
                    const Diff d = diff(xi, xj);
                    if (valid && d.d2 <= c.r2) {
                        ++nn;
                        if (s + jj != i) {
                            const float q = xdiv(xsqrt(d.d2), c.h);
                            rho = xadd(rho, xmul(xj.w, cubic_w(c, q)));
                        }
                    }
                }
            }
        });
        if (valid) {
            const float P = xmul(c.gas, xsub(rho, c.rest));
            b.aux4_s[i] = make_float4(rho, P, xmul(2.0f, rho), xdiv(xi.w, rho));
            my_max = max(my_max, nn);
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) my_max = max(my_max, __shfl_xor_sync(0xffffffffu, my_max, o));
    if (lane == 0 && my_max) atomicMax(&ds->max_nn, (unsigned long long)my_max);
}

// ---------------------------------------------------------------------------------------
// force + acceleration (+ leapfrog + wall clamp when kIntegrate)
// (compute_pressure_force / compute_viscosity_force / compute_acceleration,
//  sph_engine.cpp:390-443; integrate_leapfrog, cpp:290-310;
//  ParticleSystem::apply_boundary_conditions, particle.cpp:122-153)
// ---------------------------------------------------------------------------------------
template <bool kIntegrate>
__global__ void __launch_bounds__(128) k_force(const StepConst c, const Buffers b,
                                               DevState* ds) {
    if (ds->status) return;
    extern __shared__ float4 smem_f[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float4* cp = smem_f + warp * (3 * kTile);
    float4* cv = cp + kTile;
    float4* ca = cv + kTile;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t ntiles = ds->n_tiles;
    const float dt = ds->dt;
    for (uint32_t t = blockIdx.x * (blockDim.x >> 5) + warp; t < ntiles; t += nwarps) {
        Tile T;
        float4 xi;
        bool valid;
        tile_setup(c, b, ds, t, lane, T, xi, valid);
        const int i = T.k0 + lane;
        const float4 vi = valid ? b.vel4_s[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float Pi = valid ? b.aux4_s[i].y : 0.0f;
        float fpx = 0.0f, fpy = 0.0f, fpz = 0.0f;
        float fvx = 0.0f, fvy = 0.0f, fvz = 0.0f;
        for_each_row(b, ds, T, [&](int a, int e) {
            for (int s = a; s < e; s += kTile) {
                const int m = min(kTile, e - s);
                __syncwarp();
                if (lane < m) {
                    cp[lane] = b.pos4_s[s + lane];
                    cv[lane] = b.vel4_s[s + lane];
                    ca[lane] = b.aux4_s[s + lane];
                }
                __syncwarp();
                for (int jj = 0; jj < m; ++jj) {
                    const float4 xj = cp[jj];
                    const Diff d = diff(xi, xj);
                    if (!(valid && d.d2 <= c.r2 && s + jj != i)) continue;
                    const float4 aj = ca[jj];
                    const float r_len = xsqrt(d.d2);
                    const float q = xdiv(r_len, c.h);
                    if (!(r_len < 1e-6f)) {
                        const float pt = xdiv(xadd(Pi, aj.y), aj.z);
                        float gx = 0.0f, gy = 0.0f, gz = 0.0f;
                        if ((q >= 0.0f && q <= 1.0f) || (q > 1.0f && q <= 2.0f)) {
                            const float gf = cubic_grad_factor(c, q);
                            gx = xmul(gf, xdiv(d.x, r_len));
                            gy = xmul(gf, xdiv(d.y, r_len));
                            gz = xmul(gf, xdiv(d.z, r_len));
                        }
                        gx = xdiv(gx, c.h);
                        gy = xdiv(gy, c.h);
                        gz = xdiv(gz, c.h);
                        const float sp = xmul(xj.w, pt);
                        fpx = xsub(fpx, xmul(sp, gx));
                        fpy = xsub(fpy, xmul(sp, gy));
                        fpz = xsub(fpz, xmul(sp, gz));
                    }
                    const float4 vj = cv[jj];
                    const float lap = cubic_lap(c, q);
                    const float sv = xmul(aj.w, c.visc);
                    fvx = xadd(fvx, xmul(xmul(sv, xsub(vj.x, vi.x)), lap));
                    fvy = xadd(fvy, xmul(xmul(sv, xsub(vj.y, vi.y)), lap));
                    fvz = xadd(fvz, xmul(xmul(sv, xsub(vj.z, vi.z)), lap));
                }
            }
        });
        if (!valid) continue;
        const float mi = xi.w;
        const float ax = xdiv(xadd(xadd(fpx, fvx), xmul(0.0f, mi)), mi);
        const float ay = xdiv(xadd(xadd(fpy, fvy), xmul(c.grav, mi)), mi);
        const float az = xdiv(xadd(xadd(fpz, fvz), xmul(0.0f, mi)), mi);
        b.acc4_s[i] = make_float4(ax, ay, az, 0.0f);
        if (!kIntegrate) continue;
        const uint32_t id = b.id_s[i];
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
        if (id == 0) {
            ds->a0[0] = ax;
            ds->a0[1] = ay;
            ds->a0[2] = az;
        }
    }
}

// ---------------------------------------------------------------------------------------
// neighbour-list dump (test hook): same walk, lists written in iteration order
// ---------------------------------------------------------------------------------------
template <bool kFill>
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
        Tile T;
        float4 xi;
        bool valid;
        tile_setup(c, b, ds, t, lane, T, xi, valid);
        const int i = T.k0 + lane;
        const uint32_t id = valid ? b.id_s[i] : 0u;
        uint64_t pos = (kFill && valid) ? off_by_id[id] : 0ull;
        uint32_t nn = 0;
        for_each_row(b, ds, T, [&](int a, int e) {
            for (int s = a; s < e; s += kTile) {
                const int m = min(kTile, e - s);
                __syncwarp();
                if (lane < m) cand[lane] = b.pos4_s[s + lane];
                __syncwarp();
                for (int jj = 0; jj < m; ++jj) {
                    const Diff d = diff(xi, cand[jj]);
                    if (valid && d.d2 <= c.r2) {
                        if (kFill) out[pos++] = (int64_t)b.id_s[s + jj];
                        ++nn;
                    }
                }
            }
        });
        if (!kFill && valid) counts_by_id[id] = nn;
    }
}

static int pass_blocks(const LaunchCtx& L) {
    const int bps = L.blocks_per_sm > 0 ? L.blocks_per_sm : 8;
    return L.num_sms * bps;
}

int launch_density(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds) {
    const int threads = 32 * L.warps_per_block;
    const size_t sm = (size_t)L.warps_per_block * kTile * sizeof(float4);
    k_density<<<pass_blocks(L), threads, sm, L.stream>>>(c, b, ds);
    return 1;
}

int launch_force(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds,
                 int integrate) {
    const int threads = 32 * L.warps_per_block;
    const size_t sm = (size_t)L.warps_per_block * 3 * kTile * sizeof(float4);
    if (integrate)
        k_force<true><<<pass_blocks(L), threads, sm, L.stream>>>(c, b, ds);
    else
        k_force<false><<<pass_blocks(L), threads, sm, L.stream>>>(c, b, ds);
    return 1;
}

void launch_pair_counts(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                        DevState* ds, uint32_t* counts_by_id) {
    const size_t sm = (size_t)L.warps_per_block * kTile * sizeof(float4);
    k_pairs<false><<<pass_blocks(L), 32 * L.warps_per_block, sm, L.stream>>>(
        c, b, ds, counts_by_id, nullptr, nullptr);
}

void launch_pair_fill(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                      DevState* ds, const uint64_t* offsets_by_id, int64_t* out_idx) {
    const size_t sm = (size_t)L.warps_per_block * kTile * sizeof(float4);
    k_pairs<true><<<pass_blocks(L), 32 * L.warps_per_block, sm, L.stream>>>(
        c, b, ds, nullptr, offsets_by_id, out_idx);
}

}  // namespace sphx
