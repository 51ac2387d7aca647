// Force + acceleration + leapfrog + wall-clamp pass of the step (compute_forces,
// sph_engine.cpp:226-244, 390-443; integrate_leapfrog, cpp:290-310; apply_boundary_conditions,
// particle.cpp:122-153).
#include "sphx_passes.cuh"

namespace sphx {

// ---------------------------------------------------------------------------------------
// force + acceleration (+ leapfrog + wall clamp when kIntegrate)
// (compute_pressure_force / compute_viscosity_force / compute_acceleration,
//  sph_engine.cpp:390-443; integrate_leapfrog, cpp:290-310;
//  ParticleSystem::apply_boundary_conditions, particle.cpp:122-153)
// ---------------------------------------------------------------------------------------
// Per-warp shared memory of the force pass.  kBulk: candidates staged by bulk copies into
// two buffers, the next chunk's copies in flight while the current chunk is worked on;
// otherwise one buffer filled by the lanes' own loads.
template <bool kBulk>
struct ForceSmem {
    uint64_t bar[2];        // mbarriers of the two bulk-copy buffers (kBulk)
    float4 box_lo, box_hi;  // tile box (the fallback walk's culling test)
    int2 seg[kMaxSegments]; // the tile's row segments
    float4 cpos[kBulk ? 2 : 1][32], cvel[kBulk ? 2 : 1][32], caux[kBulk ? 2 : 1][32];
    float4 tpos[32], tvel[32];  // targets: x,y,z,m and vx,vy,vz,P
    uint16_t plist[32 * 32];
    float4 tbA[kForceBatch];  // -(pressure term) x, y and viscosity term x, y
    float2 tbB[kForceBatch];  // -(pressure term) z, viscosity term z
};
static_assert(sizeof(ForceSmem<true>) % 16 == 0 && sizeof(ForceSmem<false>) % 16 == 0,
              "per-warp regions keep the staging buffers 16-byte aligned");
static_assert(4 * sizeof(ForceSmem<true>) <= 48 * 1024, "four warps within 48 KB");

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

// Cells holding more particles than this after the grid build mark a collapsed state, in
// which whole chunks are dense (every particle of a tile within r of every candidate).
constexpr uint32_t kDenseOccupancy = 128;

// kDense: the variant with the dense-chunk path (lane-load staging only).  With lane-load
// staging both variants are launched every step and each returns at once unless the grid's
// fullest cell says the state is its case.
template <bool kIntegrate, bool kBatch, int kKern, bool kNZ, bool kBulk, bool kDense>
__global__ void __launch_bounds__(128, kBulk || kDense ? 6 : 7) k_force(
    const StepConst cp, const Buffers b, DevState* ds) {
    if (ds->status) return;
    if (!kBulk && kDense != (ds->max_occ > kDenseOccupancy)) return;
    extern __shared__ __align__(16) unsigned char smem_raw_f[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    ForceSmem<kBulk>* S = reinterpret_cast<ForceSmem<kBulk>*>(smem_raw_f) + warp;
    if constexpr (kBulk) {
        if (lane == 0) {
            mbar_init(&S->bar[0], 1);
            mbar_init(&S->bar[1], 1);
            fence_mbar_init();
        }
        __syncwarp();
    }
    uint32_t parity = 0;  // bit q: the phase of buffer q's mbarrier to wait for next
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
        tile_setup(c, b, g, k0, lane, T, xi, valid);
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
        const int nseg = build_segments(b, g, T, lane, S->seg);
        __syncwarp();
        // One chunk's work once its candidates are staged (cpos/cvel/caux) and this lane's
        // hit mask is known: list the warp's hits, compute the pair terms flattened, and
        // add every lane's own terms in candidate order.
        auto process = [&](uint32_t mask, int s, int m, const float4* cpos, const float4* cvel,
                           const float4* caux) {
            const int self = i - s;
            if ((unsigned)self < 32u) mask &= ~(1u << self);
            const uint32_t cnt = __popc(mask);
            uint32_t H;
            const uint32_t o = warp_excl_scan(cnt, lane, H);
            if (!H) return;
            // dense chunk (collapsed cells): the warp's hits are every (particle, candidate)
            // pair of the chunk except the self pairs.  Each lane then forms its own terms,
            // candidate after candidate, and adds them to its sums: the flattened path's
            // terms (same inputs from shared memory) and additions, in the same order.  The
            // additions are scalar IEEE adds on the unpacked sums: the packed FP32x2 add fed
            // directly with the term values in registers gave last-bit differences in some
            // collapsed states (measured against the reference's fixtures), while scalar adds
            // (or a round trip of the terms through shared memory, as the flattened fold
            // does) are exact.
            const int lo = max(T.k0, s), hi = min(T.k0 + T.cnt, s + m);
            if (kDense && H == (uint32_t)(T.cnt * m - max(hi - lo, 0))) {
                const float4 xt = S->tpos[lane], vt = S->tvel[lane];
                float2 sp = upk2(fpxy), sv = upk2(fvxy), sz = upk2(fz);
                for (int jj = 0; jj < m; ++jj) {
                    if (!valid || jj == self) continue;
                    float4 A;
                    float2 Bv;
                    if (kKern == SPHX_KERNEL_CUBIC_SPLINE) {
                        force_term_cubic_x2<kNZ>(c, xt, vt, vt.w, cpos[jj], cvel[jj], caux[jj], A,
                                                 Bv);
                    } else {
                        float p3[3], v3[3];
                        force_term<kKern>(c, xt, vt, vt.w, cpos[jj], cvel[jj], caux[jj], p3, v3);
                        A = make_float4(-p3[0], -p3[1], v3[0], v3[1]);
                        Bv = make_float2(-p3[2], v3[2]);
                    }
                    sp.x = xadd(sp.x, A.x);
                    sp.y = xadd(sp.y, A.y);
                    sv.x = xadd(sv.x, A.z);
                    sv.y = xadd(sv.y, A.w);
                    sz.x = xadd(sz.x, Bv.x);
                    sz.y = xadd(sz.y, Bv.y);
                }
                fpxy = pk2(sp.x, sp.y);
                fvxy = pk2(sv.x, sv.y);
                fz = pk2(sz.x, sz.y);
                return;
            }
            list_hits(S->plist, mask, o, lane);
            __syncwarp();
            for (uint32_t base = 0; base < H; base += kForceBatch) {
                const uint32_t end = min(H, base + kForceBatch);
                for (uint32_t f = base + lane; f < end; f += 32) {
                    const uint32_t pr = S->plist[f];
                    const int tt = pr >> 5, jj = pr & 31;
                    float p3[3], v3[3];
                    const float4 vt = S->tvel[tt];
                    const uint32_t u = f - base;
                    if (kKern == SPHX_KERNEL_CUBIC_SPLINE) {
                        float4 A;
                        float2 Bp;
                        force_term_cubic_x2<kNZ>(c, S->tpos[tt], vt, vt.w, cpos[jj],
                                            cvel[jj], caux[jj], A, Bp);
                        S->tbA[u] = A;
                        S->tbB[u] = Bp;
                        continue;
                    }
                    force_term<kKern>(c, S->tpos[tt], vt, vt.w, cpos[jj], cvel[jj],
                                      caux[jj], p3, v3);
                    S->tbA[u] = make_float4(-p3[0], -p3[1], v3[0], v3[1]);
                    S->tbB[u] = make_float2(-p3[2], v3[2]);
                }
                __syncwarp();
                const uint32_t k1 = min(o + cnt, end);
                for (uint32_t k = max(o, base); k < k1; ++k) {
                    const uint32_t u = k - base;
                    const float4 A = S->tbA[u];
                    const float2 Bv = S->tbB[u];
                    // the records hold -(pressure term): three packed additions
                    fpxy = xadd2(fpxy, pk2(A.x, A.y));
                    fvxy = xadd2(fvxy, pk2(A.z, A.w));
                    fz = xadd2(fz, pk2(Bv.x, Bv.y));
                }
                __syncwarp();
            }
        };
        const uint32_t* rec = slot != kNoSlot ? b.hitmask + (size_t)slot * 32 + lane : nullptr;
        const size_t pool_words = (size_t)b.hitmask_cap * 32;
        auto record = [&](const uint32_t* r) -> uint32_t {  // a lane's word, if in the pool
            return r && (size_t)(r - b.hitmask) < pool_words ? __ldcs(r) : 0u;
        };
        if constexpr (!kBulk) {
            uint32_t mnext = record(rec);
            for (int sg = 0; sg < nseg; ++sg) {
                const int2 se = S->seg[sg];
                const int a = se.x, e = se.y;
                for (int s = a; s < e; s += kTile, rec += rec ? 32 : 0) {
                    const int m = min(kTile, e - s);
                    uint32_t mask;
                    __syncwarp();
                    if (rec) {
                        mask = mnext;
                        // the next chunk's record, loaded a chunk ahead (past the tile's
                        // last chunk it reads another tile's record, or nothing at the end)
                        mnext = record(rec + 32);
                        const uint32_t used = __reduce_or_sync(kFull, mask);  // candidates hit
                        if (!used) continue;
                        if (used & (1u << lane)) {
                            S->cpos[0][lane] = b.pos4_s[s + lane];
                            S->cvel[0][lane] = b.vel4_s[s + lane];
                            S->caux[0][lane] = b.aux4_s[s + lane];
                        }
                        __syncwarp();
                    } else {
                        const bool in = lane < m;
                        const float4 pl = in ? b.pos4_s[s + lane] : make_float4(inf, inf, inf, 0.f);
                        S->cpos[0][lane] = pl;
                        __syncwarp();
                        TileBox B;
                        const float4 lo = S->box_lo, hi = S->box_hi;
                        B.lo[0] = lo.x, B.lo[1] = lo.y, B.lo[2] = lo.z;
                        B.hi[0] = hi.x, B.hi[1] = hi.y, B.hi[2] = hi.z;
                        const uint32_t surv = __ballot_sync(kFull, box_near(B, pl, r2m));
                        if (!surv) continue;
                        if (surv & (1u << lane)) {
                            S->cvel[0][lane] = b.vel4_s[s + lane];
                            S->caux[0][lane] = b.aux4_s[s + lane];
                        }
                        __syncwarp();
                        mask = valid ? chunk_hits(S->cpos[0], surv, xi, c.r2) : 0u;
                    }
                    process(mask, s, m, S->cpos[0], S->cvel[0], S->caux[0]);
                }
            }
        } else {
            // Bulk copies (exact mode): chunks are bulk-copied (pos, vel, aux: contiguous ranges of the
            // sorted arrays) into the two buffers.  A chunk some particle of the tile needs
            // is copied while the chunk before it is worked on; the records (this lane's
            // mask words) are read two chunks ahead, so the decision never waits on a load.
            auto stage = [&](int qb, int s, int m) {
                if (lane == 0) {
                    const uint32_t bytes = (uint32_t)m * 16u;
                    fence_proxy_async_smem();
                    mbar_arrive_expect_tx(&S->bar[qb], 3u * bytes);
                    bulk_copy_g2s(S->cpos[qb], b.pos4_s + s, bytes, &S->bar[qb]);
                    bulk_copy_g2s(S->cvel[qb], b.vel4_s + s, bytes, &S->bar[qb]);
                    bulk_copy_g2s(S->caux[qb], b.aux4_s + s, bytes, &S->bar[qb]);
                }
            };
            int sg = 0, s = nseg ? S->seg[0].x : 0;
            uint32_t m_cur = record(rec), m_next = record(rec ? rec + 32 : nullptr);
            int q = 0;
            bool cur_staged = false;
            while (sg < nseg) {
                const int m = min(kTile, S->seg[sg].y - s);
                int sg_n = sg, s_n = s + kTile;  // the chunk after this one
                if (s_n >= S->seg[sg].y) {
                    ++sg_n;
                    if (sg_n < nseg) s_n = S->seg[sg_n].x;
                }
                const bool has_next = sg_n < nseg;
                const int m_n = has_next ? min(kTile, S->seg[sg_n].y - s_n) : 0;
                uint32_t mask = m_cur, used, used_next;
                if (rec) {
                    used = __reduce_or_sync(kFull, m_cur);  // candidates some lane hits
                    used_next = __reduce_or_sync(kFull, has_next ? m_next : 0u);
                    const uint32_t m_after = record(rec + 64);
                    m_cur = m_next;
                    m_next = m_after;
                    rec += 32;
                } else {  // no records: every chunk is staged and culled by the tile's box
                    used = ~0u;
                    used_next = has_next ? ~0u : 0u;
                }
                if (used) {
                    if (!cur_staged) stage(q, s, m);
                    const bool next_staged = used_next != 0u;
                    if (next_staged) stage(q ^ 1, s_n, m_n);
                    const bool arrived = mbar_wait(&S->bar[q], (parity >> q) & 1u);
                    if (!__all_sync(kFull, arrived)) {
                        // a bulk copy did not complete in time: record it, wait (bounded)
                        // for the copies in flight into the other buffer, leave the pass
                        if (lane == 0) atomicCAS(&ds->status, 0, SPHX_ERR_TIMEOUT);
                        if (next_staged) mbar_wait(&S->bar[q ^ 1], (parity >> (q ^ 1)) & 1u);
                        return;
                    }
                    parity ^= 1u << q;
                    const float4* cpos = S->cpos[q];
                    if (!rec) {
                        TileBox B;
                        const float4 lo = S->box_lo, hi = S->box_hi;
                        B.lo[0] = lo.x, B.lo[1] = lo.y, B.lo[2] = lo.z;
                        B.hi[0] = hi.x, B.hi[1] = hi.y, B.hi[2] = hi.z;
                        const uint32_t surv =
                            __ballot_sync(kFull, lane < m && box_near(B, cpos[lane], r2m));
                        mask = valid && surv ? chunk_hits(cpos, surv, xi, c.r2) : 0u;
                    }
                    process(mask, s, m, cpos, S->cvel[q], S->caux[q]);
                    __syncwarp();  // buffer q is free once every lane is past this point
                    if (next_staged) q ^= 1;
                    cur_staged = next_staged;
                } else {
                    // nothing to do here; start the next chunk's copies now if it is needed
                    cur_staged = used_next != 0u;
                    if (cur_staged) stage(q, s_n, m_n);
                }
                sg = sg_n;
                s = s_n;
            }
        }
        __syncwarp();
        if (!valid) continue;
        const float mi = xi.w;
        const float2 fp = upk2(fpxy), fv = upk2(fvxy), fzz = upk2(fz);
        const float fpz = fzz.x, fvz = fzz.y;
        const float ax = xdiv(xadd(xadd(fp.x, fv.x), xmul(0.0f, mi)), mi);
        const float ay = xdiv(xadd(xadd(fp.y, fv.y), xmul(c.grav, mi)), mi);
        const float az = xdiv(xadd(xadd(fpz, fvz), xmul(0.0f, mi)), mi);
        b.acc4_s[i] = make_float4(ax, ay, az, 0.0f);
        if (!kIntegrate) continue;
        const float dt = kBatch ? b.scenes[scene].dt : ds->dt;
        const float4 vi = S->tvel[lane];
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

template <bool kIntegrate, bool kBatch, int kKern, bool kNZ, bool kBulk, bool kDense>
static void launch_force_v(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                           DevState* ds) {
    const int threads = 32 * L.warps_per_block;
    const size_t sm = (size_t)L.warps_per_block * sizeof(ForceSmem<kBulk>);
    static LaunchShapeCache cache;
    const int nb = cached_resident_blocks(
        cache, L, k_force<kIntegrate, kBatch, kKern, kNZ, kBulk, kDense>, threads, sm);
    k_force<kIntegrate, kBatch, kKern, kNZ, kBulk, kDense>
        <<<nb, threads, sm, L.stream>>>(c, b, ds);
}

// Candidates are staged by the lanes' own loads or by bulk copies (L.bulk_copy, a tuning
// choice).  Returns the kernels launched.
template <bool kIntegrate, bool kBatch, int kKern, bool kNZ = false>
static int launch_force_t(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                          DevState* ds) {
    if (L.bulk_copy) {
        launch_force_v<kIntegrate, kBatch, kKern, kNZ, true, false>(L, c, b, ds);
        return 1;
    }
    launch_force_v<kIntegrate, kBatch, kKern, kNZ, false, false>(L, c, b, ds);
    launch_force_v<kIntegrate, kBatch, kKern, kNZ, false, true>(L, c, b, ds);
    return 2;
}

template <int kKern>
static int launch_force_k(const LaunchCtx& L, const StepConst& c, const Buffers& b,
                          DevState* ds, int integrate) {
    const bool nz = kKern == SPHX_KERNEL_CUBIC_SPLINE && c.div_nz;
    const bool batch = b.nscenes > 0;
    if (integrate) {
        if (batch) return nz ? launch_force_t<true, true, kKern, true>(L, c, b, ds)
                             : launch_force_t<true, true, kKern>(L, c, b, ds);
        return nz ? launch_force_t<true, false, kKern, true>(L, c, b, ds)
                  : launch_force_t<true, false, kKern>(L, c, b, ds);
    }
    if (batch) return launch_force_t<false, true, kKern>(L, c, b, ds);
    return nz ? launch_force_t<false, false, kKern, true>(L, c, b, ds)
              : launch_force_t<false, false, kKern>(L, c, b, ds);
}

// Precision mode (single scene) runs the tile sweep (sphx_sweep.cu); exact mode k_force.
int launch_force(const LaunchCtx& L, const StepConst& c, const Buffers& b, DevState* ds,
                 int integrate) {
    if (c.precise && b.nscenes == 0) return launch_force_sweep(L, c, b, ds, integrate);
    if (c.kern == SPHX_KERNEL_WENDLAND_C2)
        return launch_force_k<SPHX_KERNEL_WENDLAND_C2>(L, c, b, ds, integrate);
    if (c.kern == SPHX_KERNEL_GAUSSIAN)
        return launch_force_k<SPHX_KERNEL_GAUSSIAN>(L, c, b, ds, integrate);
    return launch_force_k<SPHX_KERNEL_CUBIC_SPLINE>(L, c, b, ds, integrate);
}

}  // namespace sphx
