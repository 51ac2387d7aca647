// Density + pressure pass of the step (compute_densities / compute_pressures,
// sph_engine.cpp:203-224, 370-388).
#include "sphx_passes.cuh"

namespace sphx {

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

// Cells holding more particles than this after the grid build mark a collapsed state, in
// which whole chunks are dense (every particle of a tile within r of every candidate).
constexpr uint32_t kDenseOccupancy = 128;

// kDense: the variant with the dense-chunk path.  Both variants are launched every step;
// each returns at once unless the grid's fullest cell says the state is its case, so the
// lattice-like states run the leaner code and the collapsed ones get the dense path.
template <bool kBatch, int kKern, bool kNZ, bool kDense>
__global__ void __launch_bounds__(128, kDense ? 9 : 10) k_density(
    const StepConst cp, const Buffers b, DevState* ds) {
    if (ds->status) return;
    if (kDense != (ds->max_occ > kDenseOccupancy)) return;
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
        tile_setup(c, b, g, k0, lane, T, xi, valid);
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
                const float4 pl = lane < m ? b.pos4_s[s + lane] : make_float4(inf, inf, inf, 0.f);
                S->cand[lane] = pl;
                S->cx[lane] = pl.x;
                S->cy[lane] = pl.y;
                S->cz[lane] = pl.z;
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
                if (valid) mask = chunk_hits_x2(S->cx, S->cy, S->cz, surv, xi, c.r2);
                if (rec) __stcs(rec, mask);
                nn += __popc(mask);
                const int self = i - s;
                if ((unsigned)self < 32u) mask &= ~(1u << self);
                const uint32_t cnt = __popc(mask);
                uint32_t H;
                const uint32_t o = warp_excl_scan(cnt, lane, H);
                if (!H) continue;
                // dense chunk (collapsed cells): the warp's hits are every (particle,
                // candidate) pair of the chunk except the self pairs -- the most there can be.
                // Each lane then adds its own terms in candidate order: the flattened path's
                // terms and additions, without the hit list and the lane-by-lane fold.
                const int lo = max(T.k0, s), hi = min(T.k0 + T.cnt, s + m);
                if (kDense && H == (uint32_t)(T.cnt * m - max(hi - lo, 0))) {
                    for (int jj = 0; jj < m; ++jj) {
                        if (!valid || jj == self) continue;
                        const float4 xj = S->cand[jj];
                        rho = xadd(rho, xmul(xj.w, pair_w_exact<kKern, kNZ>(c, diff_d2(xi, xj))));
                    }
                    continue;
                }
                list_hits(S->plist, mask, o, lane);
                __syncwarp();
                for (uint32_t base = 0; base < H; base += kDensityBatch) {
                    const uint32_t end = min(H, base + kDensityBatch);
                    for (uint32_t f = base + lane; f < end; f += 32) {
                        const uint32_t pr = S->plist[f];
                        const float4 xj = S->cand[pr & 31];
                        const float d2 = diff_d2(S->tpos[pr >> 5], xj);
                        S->tbuf[f - base] = xmul(xj.w, pair_w_exact<kKern, kNZ>(c, d2));
                    }
                    __syncwarp();
                    const uint32_t k1 = min(o + cnt, end);
                    for (uint32_t k = max(o, base); k < k1; ++k) rho = xadd(rho, S->tbuf[k - base]);
                    __syncwarp();
                }
            }
        }
        if (b.hitmask && lane == 0) {
            const bool fits = nrec <= room;
            b.tile_slot[t] = fits ? slot : kNoSlot;
            if (fits) S->mcur = slot + nrec;
        }
        if (valid) {
            const float P = xmul(c.gas, xsub(rho, c.rest));
            // the per-candidate factors of the force pass's pair terms, each formed once here
            // with the rounding the reference applies per pair: (rho, P, 2 rho, (m / rho) mu)
            const float mr = xdiv(xi.w, rho);
            b.aux4_s[i] = make_float4(rho, P, xmul(2.0f, rho), xmul(mr, c.visc));
            my_max = max(my_max, nn);
        }
        __syncwarp();
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) my_max = max(my_max, __shfl_xor_sync(kFull, my_max, o));
    if (lane == 0 && my_max) atomicMax(&ds->max_nn, (unsigned long long)my_max);
}

template <bool kBatch, int kKern, bool kNZ, bool kDense>
static void launch_density_v(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                             DevState* ds) {
    const int threads = 32 * L.warps_per_block;
    const size_t sm = (size_t)L.warps_per_block * sizeof(DensitySmem);
    static LaunchShapeCache cache;
    const int nb = cached_resident_blocks(
        cache, L, k_density<kBatch, kKern, kNZ, kDense>, threads, sm);
    k_density<kBatch, kKern, kNZ, kDense><<<nb, threads, sm, L.stream>>>(c, b, ds);
}

template <bool kBatch, int kKern, bool kNZ = false>
static void launch_density_t(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                             DevState* ds) {
    launch_density_v<kBatch, kKern, kNZ, false>(L, c, b, ds);
    launch_density_v<kBatch, kKern, kNZ, true>(L, c, b, ds);
}

template <int kKern>
static void launch_density_k(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                             DevState* ds) {
    const bool nz = kKern == SPHX_KERNEL_CUBIC_SPLINE && !c.precise && c.div_nz;
    if (b.nscenes > 0) {
        if (nz) launch_density_t<true, kKern, true>(L, c, b, ds);
        else launch_density_t<true, kKern>(L, c, b, ds);
    } else if (nz) launch_density_t<false, kKern, true>(L, c, b, ds);
    else launch_density_t<false, kKern>(L, c, b, ds);
}

// Precision mode (single scene) runs the tile sweep (sphx_sweep.cu); exact mode the lean and
// the dense-chunk variants of k_density.
int launch_density(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds) {
    if (c.precise && b.nscenes == 0) return launch_density_sweep(L, c, b, ds);
    if (c.kern == SPHX_KERNEL_WENDLAND_C2) launch_density_k<SPHX_KERNEL_WENDLAND_C2>(L, c, b, ds);
    else if (c.kern == SPHX_KERNEL_GAUSSIAN) launch_density_k<SPHX_KERNEL_GAUSSIAN>(L, c, b, ds);
    else launch_density_k<SPHX_KERNEL_CUBIC_SPLINE>(L, c, b, ds);
    return 2;  // the lean and the dense-chunk variant; one of them returns at once
}

}  // namespace sphx
