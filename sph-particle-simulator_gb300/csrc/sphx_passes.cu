// Neighbour-list dump of the step's walk (test hook behind sphx_debug_pairs).
#include "sphx_passes.cuh"

namespace sphx {

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
