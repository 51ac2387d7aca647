// Initial conditions generated on the device, particle for particle and bit for bit what
// the host generators produce (same loops, same float operations, same order), written
// into the upload staging buffers so that the rest is the upload path.
//
//   block    create_fluid_block (src/particle.cpp:166-187): an nx x ny x nz lattice from
//            start = center - size / 2, position = start + (i, j, k) * spacing
//   box      create_boundary_box (src/particle.cpp:189-226): six faces in the reference's
//            order, each an n1 x n2 lattice on one face plane
//   sphere   create_fluid_drop_setup's ball (src/sph_engine.cpp:492-515): the lattice
//            points of the cube around the centre with |p - center|^2 <= r^2
//   lattice  the benchmark lattice (project RNG): float32(i) * spacing + (2u - 1) * jitter
//            (+ origin), u a splitmix64 uniform of (seed, index, axis)
//   ball     the batched scenes' drop: lattice points c + k * spacing, |k| <= int(R / s) + 1,
//            kept where |k * spacing|^2 <= R^2, evaluated in FP64 then rounded to float
// Ball-shaped sets keep the (i, j, k) order: rows (i, j) count their points, an exclusive
// scan places the rows, and each row writes its points in k order.
#include "sphx_internal.cuh"

namespace sphx {

namespace {

// the project RNG: splitmix64 finaliser of (seed << 40) + 8 index + stream, top 24 bits
__device__ __forceinline__ float rng_uniform(uint64_t seed, uint64_t index, int stream) {
    const uint64_t golden = 0x9E3779B97F4A7C15ull;
    uint64_t z = ((seed << 40) + index * 8ull + (uint64_t)stream) * golden + golden;
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ull;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)((double)(z >> 40) * (1.0 / 16777216.0));
}

__device__ __forceinline__ void put(const GenArgs& g, uint32_t at, float x, float y, float z) {
    float* p = g.pos + 3 * (size_t)at;
    p[0] = x;
    p[1] = y;
    p[2] = z;
    float* v = g.vel + 3 * (size_t)at;
    v[0] = g.s.vel[0];
    v[1] = g.s.vel[1];
    v[2] = g.s.vel[2];
    g.mass[at] = g.s.mass;
}

__global__ void k_gen_block(const GenArgs g) {
    const GenShape& s = g.s;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < s.count;
         idx += gridDim.x * blockDim.x) {
        const uint32_t k = idx % (uint32_t)s.n[2];
        const uint32_t j = (idx / (uint32_t)s.n[2]) % (uint32_t)s.n[1];
        const uint32_t i = idx / ((uint32_t)s.n[2] * (uint32_t)s.n[1]);
        put(g, s.offset + idx, xadd(s.start[0], xmul((float)i, s.spacing)),
            xadd(s.start[1], xmul((float)j, s.spacing)), xadd(s.start[2], xmul((float)k, s.spacing)));
    }
}

__global__ void k_gen_box(const GenArgs g) {
    const GenShape& s = g.s;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < s.count;
         idx += gridDim.x * blockDim.x) {
        int f = 0;
        while (f < 5 && idx >= s.face_off[f + 1]) ++f;
        const uint32_t local = idx - s.face_off[f];
        const uint32_t i = local / (uint32_t)s.face_n2[f], j = local % (uint32_t)s.face_n2[f];
        float p[3] = {s.start[0], s.start[1], s.start[2]};
        const int a1 = s.face_a[f][0], a2 = s.face_a[f][1], a3 = s.face_a[f][2];
        p[a1] = xadd(s.start[a1], xmul((float)i, s.spacing));
        p[a2] = xadd(s.start[a2], xmul((float)j, s.spacing));
        p[a3] = s.face_val[f];
        put(g, s.offset + idx, p[0], p[1], p[2]);
    }
}

__global__ void k_gen_lattice(const GenArgs g) {
    const GenShape& s = g.s;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < s.count;
         idx += gridDim.x * blockDim.x) {
        const uint32_t k = idx % (uint32_t)s.n[2];
        const uint32_t j = (idx / (uint32_t)s.n[2]) % (uint32_t)s.n[1];
        const uint32_t i = idx / ((uint32_t)s.n[2] * (uint32_t)s.n[1]);
        const uint32_t ijk[3] = {i, j, k};
        float p[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            p[a] = xmul((float)ijk[a], s.spacing);
            if (s.jitter != 0.0f) {
                const float u = rng_uniform(s.seed, idx, a);
                p[a] = xadd(p[a], xmul(xsub(xmul(u, 2.0f), 1.0f), s.jitter));
            }
            if (s.has_origin) p[a] = xadd(p[a], s.origin[a]);
        }
        put(g, s.offset + idx, p[0], p[1], p[2]);
    }
}

// is lattice point (i, j, k) of a ball shape inside, and where is it
__device__ __forceinline__ bool ball_point(const GenShape& s, int i, int j, int k, float* p) {
    if (s.kind == SPHX_SHAPE_SPHERE) {
        const int ijk[3] = {i, j, k};
        float t[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            p[a] = xadd(s.start[a], xmul((float)ijk[a], s.spacing));
            t[a] = xsub(p[a], s.center[a]);
        }
        return xdot3(t[0], t[1], t[2]) <= s.r2;
    }
    // SPHX_SHAPE_BALL: k runs from -kmax; FP64 as the host generator evaluates it
    const double gx = (double)(i - s.kmax) * s.sp64, gy = (double)(j - s.kmax) * s.sp64,
                 gz = (double)(k - s.kmax) * s.sp64;
    p[0] = (float)__dadd_rn(s.c64[0], gx);
    p[1] = (float)__dadd_rn(s.c64[1], gy);
    p[2] = (float)__dadd_rn(s.c64[2], gz);
    return __dadd_rn(__dadd_rn(__dmul_rn(gx, gx), __dmul_rn(gy, gy)), __dmul_rn(gz, gz)) <= s.R2;
}

__global__ void k_ball_rows(const GenArgs g, uint32_t* rows) {
    const GenShape& s = g.s;
    const uint32_t nrows = (uint32_t)s.n[0] * (uint32_t)s.n[1];
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows;
         r += gridDim.x * blockDim.x) {
        const int i = (int)(r / (uint32_t)s.n[1]), j = (int)(r % (uint32_t)s.n[1]);
        uint32_t c = 0;
        float p[3];
        for (int k = 0; k < s.n[2]; ++k) c += ball_point(s, i, j, k, p) ? 1u : 0u;
        rows[r] = c;
    }
}

// exclusive scan of rows[0, n) in place by one block; rows[n] = total
__global__ void k_scan_rows(uint32_t* rows, uint32_t n) {
    __shared__ uint32_t part[1024];
    const uint32_t t = threadIdx.x, T = blockDim.x;
    const uint32_t per = (n + T - 1) / T;
    const uint32_t a = min(n, t * per), e = min(n, a + per);
    uint32_t sum = 0;
    for (uint32_t r = a; r < e; ++r) sum += rows[r];
    part[t] = sum;
    __syncthreads();
    for (uint32_t o = 1; o < T; o <<= 1) {  // inclusive Hillis-Steele scan of the parts
        const uint32_t v = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;
    for (uint32_t r = a; r < e; ++r) {
        const uint32_t c = rows[r];
        rows[r] = run;
        run += c;
    }
    if (t == T - 1) rows[n] = part[t];
}

__global__ void k_ball_write(const GenArgs g, const uint32_t* rows) {
    const GenShape& s = g.s;
    const uint32_t nrows = (uint32_t)s.n[0] * (uint32_t)s.n[1];
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows;
         r += gridDim.x * blockDim.x) {
        const int i = (int)(r / (uint32_t)s.n[1]), j = (int)(r % (uint32_t)s.n[1]);
        uint32_t at = s.offset + rows[r];
        float p[3];
        for (int k = 0; k < s.n[2]; ++k)
            if (ball_point(s, i, j, k, p)) put(g, at++, p[0], p[1], p[2]);
    }
}

int grid_for(const LaunchCtx& L, uint64_t n) {
    const uint64_t b = (n + 255) / 256;
    return (int)(b < (uint64_t)L.num_sms * 8 ? (b ? b : 1) : (uint64_t)L.num_sms * 8);
}

}  // namespace

int launch_ball_count(const LaunchCtx& L, const GenArgs& g, uint32_t* rows) {
    const uint32_t nrows = (uint32_t)g.s.n[0] * (uint32_t)g.s.n[1];
    k_ball_rows<<<grid_for(L, nrows), 256, 0, L.stream>>>(g, rows);
    k_scan_rows<<<1, 1024, 0, L.stream>>>(rows, nrows);
    return 2;
}

int launch_generate(const LaunchCtx& L, const GenArgs& g, const uint32_t* rows) {
    const GenShape& s = g.s;
    switch (s.kind) {
        case SPHX_SHAPE_BLOCK:
            if (s.count) k_gen_block<<<grid_for(L, s.count), 256, 0, L.stream>>>(g);
            return s.count ? 1 : 0;
        case SPHX_SHAPE_BOX:
            if (s.count) k_gen_box<<<grid_for(L, s.count), 256, 0, L.stream>>>(g);
            return s.count ? 1 : 0;
        case SPHX_SHAPE_LATTICE:
            if (s.count) k_gen_lattice<<<grid_for(L, s.count), 256, 0, L.stream>>>(g);
            return s.count ? 1 : 0;
        default: {
            const uint32_t nrows = (uint32_t)s.n[0] * (uint32_t)s.n[1];
            k_ball_write<<<grid_for(L, nrows), 256, 0, L.stream>>>(g, rows);
            return 1;
        }
    }
}

}  // namespace sphx
