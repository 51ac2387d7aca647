/* CPU restatement ("port") of the reference SPH step.  See sph_oracle.h.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  It restates, in plain C, the algorithm of:
 *   SpatialHash  build/query_squared          src/spatial_hash.h:20-36, spatial_hash.cpp:15-57
 *   CubicSplineKernel W/gradW/laplacianW      src/kernels.cpp:23-36, 58-66, 96-108, 130-143
 *   equations::*                              src/sph_engine.cpp:370-443
 *   SPHEngine::step and its phases            src/sph_engine.cpp:93-144, 203-353
 *   ParticleSystem::apply_boundary_conditions src/particle.cpp:122-153
 *   get_total_mass / get_total_energy /
 *   compute_conservation_errors               src/sph_engine.cpp:178-200
 * with the same data structures where they shape the cost (a serially built hash of cell
 * buckets, one growable neighbour list per particle, OpenMP loops over particles) and the
 * same float operation order everywhere, so that on the same inputs it produces the same
 * bits as the reference core compiled with IEEE float semantics (no FMA contraction, no
 * fast-math).  It must be compiled with -ffp-contract=off and without -ffast-math.
 */
#include "sph_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------ */
/* float helpers mirroring the GLM operations the reference uses                         */
/* ------------------------------------------------------------------------------------ */

/* glm::dot(v, v) = (x*x + y*y) + z*z, products rounded first. */
static inline float dot3(float x, float y, float z) {
    const float a = x * x, b = y * y, c = z * z;
    return (a + b) + c;
}

/* static_cast<int>(std::floor(v)) as the reference's x86-64 build evaluates it:
 * cvttss2si returns INT32_MIN for NaN and out-of-range values. */
static inline int32_t floor_to_int(float v) {
    const float f = floorf(v);
    if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int32_t)f;
}

/* SpatialHash::hash_position (src/spatial_hash.h:20-27): 21 bits per coordinate. */
static inline uint64_t pack_cell(int32_t x, int32_t y, int32_t z) {
    return ((uint64_t)((uint32_t)x & 0x1FFFFFu) << 42) |
           ((uint64_t)((uint32_t)y & 0x1FFFFFu) << 21) | (uint64_t)((uint32_t)z & 0x1FFFFFu);
}

/* Smoothing kernels: the three of create_kernel (src/kernels.cpp:226-236), constants
 * computed in float exactly as their constructors do (src/kernels.cpp:12-14, 23-36,
 * 166-170, 204-208).  kind: 0 CUBIC_SPLINE, 1 WENDLAND_C2, 2 GAUSSIAN (KernelType order,
 * src/kernels.h:94-98). */
typedef struct {
    int kind;
    float h, h_sq, sigma;   /* cubic: sigma_3d_ */
    float norm;             /* Wendland: norm_factor_; Gaussian: norm_ */
    float s;                /* Gaussian: sigma_sq_inv_ */
} kern;

static kern make_kernel(int kind, float h) {
    kern k;
    memset(&k, 0, sizeof(k));
    k.kind = kind;
    k.h = h;
    k.h_sq = h * h;
    k.sigma = 1.0f / ((((float)M_PI) * h) * h * h);
    if (kind == 1) k.norm = 21.0f / (((2.0f * (float)M_PI) * h) * h * h);
    if (kind == 2) {
        k.s = 1.0f / (h * h);
        k.norm = 1.0f / powf(((float)M_PI * h) * h, 1.5f);
    }
    return k;
}

/* CubicSplineKernel::W_3d (src/kernels.cpp:58-66) */
static inline float w3(const kern* k, float q) {
    if (q >= 0.0f && q <= 1.0f) {
        return k->sigma * (2.0f / 3.0f - q * q + 0.5f * q * q * q);
    } else if (q > 1.0f && q <= 2.0f) {
        const float tmp = 2.0f - q;
        return k->sigma * (1.0f / 6.0f * tmp * tmp * tmp);
    }
    return 0.0f;
}

/* Kernel::W(r): cubic W_3d(length(r)/h) (src/kernels.cpp:140-143, kernels.h:117-119);
 * WendlandC2Kernel::W (kernels.cpp:172-178); GaussianKernel::W (kernels.cpp:210-213) */
static inline float w_of(const kern* k, float rx, float ry, float rz) {
    if (k->kind == 2) {
        const float r_sq = dot3(rx, ry, rz);
        return k->norm * expf(-r_sq * k->s);
    }
    const float q = sqrtf(dot3(rx, ry, rz)) / k->h;
    if (k->kind == 1) {
        if (q >= 2.0f) return 0.0f;
        const float tmp = 1.0f - 0.5f * q;
        return k->norm * tmp * tmp * tmp * tmp * (2.0f * q + 1.0f);
    }
    return w3(k, q);
}

/* Kernel::gradW(r): cubic (src/kernels.cpp:96-108, 145-148); Wendland (kernels.cpp:180-192);
 * Gaussian (kernels.cpp:215-219) */
static inline void gradw_of(const kern* k, float rx, float ry, float rz, float* g) {
    if (k->kind == 2) {
        const float r_sq = dot3(rx, ry, rz);
        const float e = expf(-r_sq * k->s);
        const float c = -2.0f * k->s * k->norm * e;
        g[0] = c * rx;
        g[1] = c * ry;
        g[2] = c * rz;
        return;
    }
    if (k->kind == 1) {
        const float r_len = sqrtf(dot3(rx, ry, rz));
        g[0] = g[1] = g[2] = 0.0f;
        if (r_len < 1e-6f) return;
        const float q = r_len / k->h;
        if (q >= 2.0f) return;
        const float tmp = 1.0f - 0.5f * q;
        const float dw = -5.0f * tmp * tmp * tmp * q;
        const float c = k->norm * dw;
        const float den = r_len * k->h;
        g[0] = c * (rx / den);
        g[1] = c * (ry / den);
        g[2] = c * (rz / den);
        return;
    }
    const float q = sqrtf(dot3(rx, ry, rz)) / k->h;
    const float r_len = sqrtf(dot3(rx, ry, rz));
    if (r_len < 1e-6f) {
        g[0] = g[1] = g[2] = 0.0f;
        return;
    }
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;
    if (q >= 0.0f && q <= 1.0f) {
        const float c = k->sigma * (-2.0f * q + 1.5f * q * q);
        gx = c * (rx / r_len);
        gy = c * (ry / r_len);
        gz = c * (rz / r_len);
    } else if (q > 1.0f && q <= 2.0f) {
        const float tmp = 2.0f - q;
        const float c = -k->sigma * (0.5f * tmp * tmp);
        gx = c * (rx / r_len);
        gy = c * (ry / r_len);
        gz = c * (rz / r_len);
    }
    g[0] = gx / k->h;
    g[1] = gy / k->h;
    g[2] = gz / k->h;
}

/* Kernel::laplacianW(r): cubic (src/kernels.cpp:130-138, 150-153); Wendland
 * (kernels.cpp:194-200); Gaussian (kernels.cpp:221-225) */
static inline float lapw_of(const kern* k, float rx, float ry, float rz) {
    if (k->kind == 2) {
        const float r_sq = dot3(rx, ry, rz);
        const float e = expf(-r_sq * k->s);
        return 2.0f * k->s * k->norm * e * (2.0f * k->s * r_sq - 3.0f);
    }
    const float q = sqrtf(dot3(rx, ry, rz)) / k->h;
    if (k->kind == 1) {
        if (q >= 2.0f) return 0.0f;
        const float tmp = 1.0f - 0.5f * q;
        return k->norm * (5.0f / k->h_sq) * tmp * tmp * (5.0f * q - 3.0f);
    }
    if (q >= 0.0f && q <= 1.0f) {
        return k->sigma * (-2.0f + 3.0f * q) / k->h_sq;
    } else if (q > 1.0f && q <= 2.0f) {
        const float tmp = 2.0f - q;
        return k->sigma * tmp / k->h_sq;
    }
    return 0.0f;
}

/* ------------------------------------------------------------------------------------ */
/* spatial hash: cell key -> bucket of particle indices in insertion order               */
/* ------------------------------------------------------------------------------------ */

typedef struct {
    uint64_t* keys;     /* table of cell keys */
    int64_t* bucket;    /* table slot -> bucket id, -1 = empty */
    size_t mask;        /* table size - 1 */
    int64_t nbuckets;
    int64_t* start;     /* bucket -> first entry in items (nbuckets + 1) */
    int64_t* items;     /* particle indices grouped by bucket, insertion order */
    float inv_cell;
} cell_hash;

static inline uint64_t mix64(uint64_t z) {
    z ^= z >> 30;
    z *= 0xBF58476D1CE4E5B9ull;
    z ^= z >> 27;
    z *= 0x94D049BB133111EBull;
    z ^= z >> 31;
    return z;
}

static int64_t hash_find(const cell_hash* h, uint64_t key) {
    size_t s = (size_t)mix64(key) & h->mask;
    for (;;) {
        const int64_t b = h->bucket[s];
        if (b < 0) return -1;
        if (h->keys[s] == key) return b;
        s = (s + 1) & h->mask;
    }
}

/* SpatialHash::build (src/spatial_hash.cpp:15-25): serial, insertion order per bucket. */
static void hash_build(cell_hash* h, size_t n, const float* pos, float cell_size) {
    size_t tsize = 16;
    while (tsize < 2 * n + 16) tsize <<= 1;
    h->mask = tsize - 1;
    h->keys = (uint64_t*)malloc(tsize * sizeof(uint64_t));
    h->bucket = (int64_t*)malloc(tsize * sizeof(int64_t));
    for (size_t s = 0; s < tsize; ++s) h->bucket[s] = -1;
    h->inv_cell = 1.0f / cell_size;
    int64_t* pb = (int64_t*)malloc((n ? n : 1) * sizeof(int64_t));
    int64_t nb = 0;
    for (size_t i = 0; i < n; ++i) {
        const int32_t cx = floor_to_int(pos[3 * i] * h->inv_cell);
        const int32_t cy = floor_to_int(pos[3 * i + 1] * h->inv_cell);
        const int32_t cz = floor_to_int(pos[3 * i + 2] * h->inv_cell);
        const uint64_t key = pack_cell(cx, cy, cz);
        size_t s = (size_t)mix64(key) & h->mask;
        for (;;) {
            if (h->bucket[s] < 0) {
                h->bucket[s] = nb++;
                h->keys[s] = key;
                break;
            }
            if (h->keys[s] == key) break;
            s = (s + 1) & h->mask;
        }
        pb[i] = h->bucket[s];
    }
    h->nbuckets = nb;
    h->start = (int64_t*)calloc((size_t)nb + 1, sizeof(int64_t));
    for (size_t i = 0; i < n; ++i) h->start[pb[i] + 1]++;
    for (int64_t b = 0; b < nb; ++b) h->start[b + 1] += h->start[b];
    int64_t* cur = (int64_t*)malloc(((size_t)nb + 1) * sizeof(int64_t));
    memcpy(cur, h->start, ((size_t)nb + 1) * sizeof(int64_t));
    h->items = (int64_t*)malloc((n ? n : 1) * sizeof(int64_t));
    for (size_t i = 0; i < n; ++i) h->items[cur[pb[i]]++] = (int64_t)i;
    free(cur);
    free(pb);
}

static void hash_free(cell_hash* h) {
    free(h->keys);
    free(h->bucket);
    free(h->start);
    free(h->items);
    memset(h, 0, sizeof(*h));
}

/* one growable list per particle, like std::vector<size_t> with push_back */
typedef struct {
    int64_t* data;
    size_t size, cap;
} i64vec;

static inline void vec_push(i64vec* v, int64_t x) {
    if (v->size == v->cap) {
        const size_t nc = v->cap ? 2 * v->cap : 1;
        v->data = (int64_t*)realloc(v->data, nc * sizeof(int64_t));
        v->cap = nc;
    }
    v->data[v->size++] = x;
}

/* SpatialHash::query_squared (src/spatial_hash.cpp:31-57) */
static void hash_query(const cell_hash* h, const float* pos, float px, float py, float pz,
                       float radius_sq, i64vec* out) {
    out->data = NULL;
    out->size = out->cap = 0;
    const int32_t cx = floor_to_int(px * h->inv_cell);
    const int32_t cy = floor_to_int(py * h->inv_cell);
    const int32_t cz = floor_to_int(pz * h->inv_cell);
    const int cr = (int)ceilf(sqrtf(radius_sq) * h->inv_cell) + 1;
    for (int dx = -cr; dx <= cr; ++dx) {
        for (int dy = -cr; dy <= cr; ++dy) {
            for (int dz = -cr; dz <= cr; ++dz) {
                /* int addition wraps like the reference's x86 build */
                const int32_t x = (int32_t)((uint32_t)cx + (uint32_t)dx);
                const int32_t y = (int32_t)((uint32_t)cy + (uint32_t)dy);
                const int32_t z = (int32_t)((uint32_t)cz + (uint32_t)dz);
                const int64_t b = hash_find(h, pack_cell(x, y, z));
                if (b < 0) continue;
                for (int64_t e = h->start[b]; e < h->start[b + 1]; ++e) {
                    const int64_t j = h->items[e];
                    const float ddx = px - pos[3 * j];
                    const float ddy = py - pos[3 * j + 1];
                    const float ddz = pz - pos[3 * j + 2];
                    if (dot3(ddx, ddy, ddz) <= radius_sq) vec_push(out, j);
                }
            }
        }
    }
}

/* update_neighbor_lists (src/sph_engine.cpp:335-353) */
static void build_lists(size_t n, const float* pos, float cell_size, float radius, i64vec* nl,
                        uint64_t* max_nn) {
    cell_hash h;
    hash_build(&h, n, pos, cell_size);
    const float r2 = radius * radius;
    uint64_t mx = 0;
#pragma omp parallel for schedule(static) reduction(max : mx)
    for (long long i = 0; i < (long long)n; ++i) {
        free(nl[i].data);
        hash_query(&h, pos, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], r2, &nl[i]);
        if (nl[i].size > mx) mx = nl[i].size;
    }
    hash_free(&h);
    if (max_nn) *max_nn = mx;
}

int64_t orc_query(size_t n, const float* pos, float cell_size, float radius, int64_t* counts,
                  int64_t* idx) {
    i64vec* nl = (i64vec*)calloc(n ? n : 1, sizeof(i64vec));
    build_lists(n, pos, cell_size, radius, nl, NULL);
    int64_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        counts[i] = (int64_t)nl[i].size;
        if (idx) memcpy(idx + total, nl[i].data, nl[i].size * sizeof(int64_t));
        total += (int64_t)nl[i].size;
        free(nl[i].data);
    }
    free(nl);
    return total;
}

/* Lists of particles [i0, i1) into nl[0 .. i1 - i0) (released with free_block). */
static void query_block(const cell_hash* h, const float* pos, size_t i0, size_t i1, float r2,
                        i64vec* nl) {
#pragma omp parallel for schedule(static)
    for (long long i = (long long)i0; i < (long long)i1; ++i)
        hash_query(h, pos, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], r2, &nl[i - (long long)i0]);
}

static void free_block(i64vec* nl, size_t m) {
    for (size_t e = 0; e < m; ++e) {
        free(nl[e].data);
        nl[e].data = NULL;
        nl[e].size = nl[e].cap = 0;
    }
}

/* particles whose lists are held at a time by the field evaluations */
enum { kListBlock = 1 << 19 };

int64_t orc_query_subset(size_t n, const float* pos, float cell_size, float radius, size_t nq,
                         const int64_t* sel, int64_t* counts, int64_t* idx) {
    cell_hash h;
    hash_build(&h, n, pos, cell_size);
    i64vec* nl = (i64vec*)calloc(nq ? nq : 1, sizeof(i64vec));
    const float r2 = radius * radius;
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)nq; ++q) {
        const int64_t i = sel[q];
        hash_query(&h, pos, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], r2, &nl[q]);
    }
    int64_t total = 0;
    for (size_t q = 0; q < nq; ++q) {
        counts[q] = (int64_t)nl[q].size;
        if (idx) memcpy(idx + total, nl[q].data, nl[q].size * sizeof(int64_t));
        total += (int64_t)nl[q].size;
        free(nl[q].data);
    }
    free(nl);
    hash_free(&h);
    return total;
}

/* ------------------------------------------------------------------------------------ */
/* field phases                                                                          */
/* ------------------------------------------------------------------------------------ */

/* compute_densities -> equations::compute_density (src/sph_engine.cpp:203-212, 370-383) */
/* Particles [i0, i1); nl[i - i0] is particle i's list. */
static void densities(size_t i0, size_t i1, const float* pos, const float* mass,
                      const i64vec* nl, const kern* k, float* rho) {
    const float w0 = w_of(k, 0.0f, 0.0f, 0.0f);
#pragma omp parallel for schedule(static)
    for (long long i = (long long)i0; i < (long long)i1; ++i) {
        float d = mass[i] * w0;
        const i64vec* L = &nl[i - (long long)i0];
        for (size_t e = 0; e < L->size; ++e) {
            const int64_t j = L->data[e];
            if (j == i) continue;
            const float rx = pos[3 * i] - pos[3 * j];
            const float ry = pos[3 * i + 1] - pos[3 * j + 1];
            const float rz = pos[3 * i + 2] - pos[3 * j + 2];
            d += mass[j] * w_of(k, rx, ry, rz);
        }
        rho[i] = d;
    }
}

/* compute_pressures -> equations::compute_pressure (src/sph_engine.cpp:214-224, 385-388) */
static void pressures(size_t n, const float* rho, float rest, float gas, float* P) {
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) P[i] = gas * (rho[i] - rest);
}

/* compute_forces: pressure force, viscosity force, external force, acceleration
 * (src/sph_engine.cpp:226-244, 390-443) */
static void forces(size_t i0, size_t i1, const float* pos, const float* vel,
                   const float* mass, const i64vec* nl, const kern* k, const float* rho,
                   const float* P, float viscosity, float gravity, float* acc) {
#pragma omp parallel for schedule(static)
    for (long long i = (long long)i0; i < (long long)i1; ++i) {
        const i64vec* L = &nl[i - (long long)i0];
        float fpx = 0.0f, fpy = 0.0f, fpz = 0.0f;
        for (size_t e = 0; e < L->size; ++e) {
            const int64_t j = L->data[e];
            if (j == i) continue;
            const float rx = pos[3 * i] - pos[3 * j];
            const float ry = pos[3 * i + 1] - pos[3 * j + 1];
            const float rz = pos[3 * i + 2] - pos[3 * j + 2];
            const float r_len = sqrtf(dot3(rx, ry, rz));
            if (r_len < 1e-6f) continue;
            const float pt = (P[i] + P[j]) / (2.0f * rho[j]);
            float g[3];
            gradw_of(k, rx, ry, rz, g);
            const float s = mass[j] * pt;
            fpx -= s * g[0];
            fpy -= s * g[1];
            fpz -= s * g[2];
        }
        float fvx = 0.0f, fvy = 0.0f, fvz = 0.0f;
        for (size_t e = 0; e < L->size; ++e) {
            const int64_t j = L->data[e];
            if (j == i) continue;
            const float rx = pos[3 * i] - pos[3 * j];
            const float ry = pos[3 * i + 1] - pos[3 * j + 1];
            const float rz = pos[3 * i + 2] - pos[3 * j + 2];
            const float vx = vel[3 * j] - vel[3 * i];
            const float vy = vel[3 * j + 1] - vel[3 * i + 1];
            const float vz = vel[3 * j + 2] - vel[3 * i + 2];
            const float lap = lapw_of(k, rx, ry, rz);
            const float s = (mass[j] / rho[j]) * viscosity;
            fvx += (s * vx) * lap;
            fvy += (s * vy) * lap;
            fvz += (s * vz) * lap;
        }
        const float m = mass[i];
        const float ex = 0.0f * m, ey = gravity * m, ez = 0.0f * m;
        acc[3 * i] = ((fpx + fvx) + ex) / m;
        acc[3 * i + 1] = ((fpy + fvy) + ey) / m;
        acc[3 * i + 2] = ((fpz + fvz) + ez) / m;
    }
}

static void load_params(const float* p, float* out16) { memcpy(out16, p, 16 * sizeof(float)); }

void orc_fields(size_t n, const float* pos, const float* vel, const float* mass,
                const float* params16, float* rho, float* P, float* acc) {
    orc_fields_k(0, n, pos, vel, mass, params16, rho, P, acc);
}

void orc_fields_k(int kind, size_t n, const float* pos, const float* vel, const float* mass,
                  const float* params16, float* rho, float* P, float* acc) {
    float prm[16];
    load_params(params16, prm);
    const kern k = make_kernel(kind, prm[3]);
    /* The lists of a block of particles at a time (the same lists, so the same sums): the
     * lists of all particles of a 10M state would take about 22 GB. */
    cell_hash h;
    hash_build(&h, n, pos, prm[15]);
    const float r2 = prm[15] * prm[15];
    i64vec* nl = (i64vec*)calloc(kListBlock, sizeof(i64vec));
    for (size_t i0 = 0; i0 < n; i0 += kListBlock) {
        const size_t i1 = n - i0 < kListBlock ? n : i0 + kListBlock;
        query_block(&h, pos, i0, i1, r2, nl);
        densities(i0, i1, pos, mass, nl, &k, rho);
        free_block(nl, i1 - i0);
    }
    pressures(n, rho, prm[0], prm[1], P);
    for (size_t i0 = 0; i0 < n; i0 += kListBlock) {
        const size_t i1 = n - i0 < kListBlock ? n : i0 + kListBlock;
        query_block(&h, pos, i0, i1, r2, nl);
        forces(i0, i1, pos, vel, mass, nl, &k, rho, P, prm[2], prm[6], acc);
        free_block(nl, i1 - i0);
    }
    free(nl);
    hash_free(&h);
}

/* ---- FP64 re-evaluation over the same neighbour sets ---------------------------------- */
static inline double w3d(double sigma, double q) {
    if (q >= 0.0 && q <= 1.0) return sigma * (2.0 / 3.0 - q * q + 0.5 * q * q * q);
    if (q > 1.0 && q <= 2.0) {
        const double t = 2.0 - q;
        return sigma * (t * t * t / 6.0);
    }
    return 0.0;
}

/* W, grad W = G * r and laplacian W of the three kernels in double (same formulas as the
 * float versions above, evaluated in double) */
static inline double w_d(int kind, double h, double sigma, double rl) {
    const double q = rl / h;
    if (kind == 1) {
        if (q >= 2.0) return 0.0;
        const double t = 1.0 - 0.5 * q;
        return 21.0 / (2.0 * M_PI * h * h * h) * t * t * t * t * (2.0 * q + 1.0);
    }
    if (kind == 2) return exp(-rl * rl / (h * h)) / pow(M_PI * h * h, 1.5);
    return w3d(sigma, q);
}
static inline double g_d(int kind, double h, double rl) {
    const double q = rl / h;
    if (kind == 1) {
        if (q >= 2.0) return 0.0;
        const double t = 1.0 - 0.5 * q;
        return 21.0 / (2.0 * M_PI * h * h * h) * (-5.0 * t * t * t * q) / (rl * h);
    }
    /* kind 2 */
    return -2.0 / (h * h) * exp(-rl * rl / (h * h)) / pow(M_PI * h * h, 1.5);
}
static inline double lap_d(int kind, double h, double rl) {
    const double q = rl / h;
    if (kind == 1) {
        if (q >= 2.0) return 0.0;
        const double t = 1.0 - 0.5 * q;
        return 21.0 / (2.0 * M_PI * h * h * h) * (5.0 / (h * h)) * t * t * (5.0 * q - 3.0);
    }
    /* kind 2 */
    const double s = 1.0 / (h * h);
    return 2.0 * s * exp(-rl * rl * s) / pow(M_PI * h * h, 1.5) * (2.0 * s * rl * rl - 3.0);
}

void orc_fields_f64(size_t n, const float* pos, const float* vel, const float* mass,
                    const float* params16, double* rho, double* P, double* acc,
                    double* sum_abs) {
    orc_fields_f64_k(0, n, pos, vel, mass, params16, rho, P, acc, sum_abs);
}

void orc_fields_f64_k(int kind, size_t n, const float* pos, const float* vel,
                      const float* mass, const float* params16, double* rho, double* P,
                      double* acc, double* sum_abs) {
    float prm[16];
    load_params(params16, prm);
    const double h = prm[3], hsq = h * h, sigma = 1.0 / (M_PI * h * h * h);
    cell_hash hh;
    hash_build(&hh, n, pos, prm[15]);
    const float r2 = prm[15] * prm[15];
    i64vec* nl = (i64vec*)calloc(kListBlock, sizeof(i64vec));
    for (size_t i0 = 0; i0 < n; i0 += kListBlock) {
        const size_t i1 = n - i0 < kListBlock ? n : i0 + kListBlock;
        query_block(&hh, pos, i0, i1, r2, nl);
#pragma omp parallel for schedule(static)
        for (long long i = (long long)i0; i < (long long)i1; ++i) {
            const i64vec* L = &nl[i - (long long)i0];
            double d = (double)mass[i] * w_d(kind, h, sigma, 0.0);
            for (size_t e = 0; e < L->size; ++e) {
                const int64_t j = L->data[e];
                if (j == i) continue;
                const double rx = (double)pos[3 * i] - (double)pos[3 * j];
                const double ry = (double)pos[3 * i + 1] - (double)pos[3 * j + 1];
                const double rz = (double)pos[3 * i + 2] - (double)pos[3 * j + 2];
                d += (double)mass[j] * w_d(kind, h, sigma, sqrt(rx * rx + ry * ry + rz * rz));
            }
            rho[i] = d;
            P[i] = (double)prm[1] * (d - (double)prm[0]);
        }
        free_block(nl, i1 - i0);
    }
    for (size_t i0 = 0; i0 < n; i0 += kListBlock) {
        const size_t i1 = n - i0 < kListBlock ? n : i0 + kListBlock;
        query_block(&hh, pos, i0, i1, r2, nl);
#pragma omp parallel for schedule(static)
        for (long long i = (long long)i0; i < (long long)i1; ++i) {
            const i64vec* L = &nl[i - (long long)i0];
            double f[3] = {0, 0, 0}, sa[3] = {0, 0, 0};
            for (size_t e = 0; e < L->size; ++e) {
                const int64_t j = L->data[e];
                if (j == i) continue;
                const double r[3] = {(double)pos[3 * i] - (double)pos[3 * j],
                                     (double)pos[3 * i + 1] - (double)pos[3 * j + 1],
                                     (double)pos[3 * i + 2] - (double)pos[3 * j + 2]};
                const double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
                const double q = rl / h;
                if (rl >= 1e-6) {
                    const double s = (double)mass[j] * (P[i] + P[j]) / (2.0 * rho[j]);
                    if (kind == 0) {
                        double c = 0.0;
                        if (q <= 1.0) c = sigma * (-2.0 * q + 1.5 * q * q);
                        else if (q <= 2.0) c = -sigma * 0.5 * (2.0 - q) * (2.0 - q);
                        for (int a = 0; a < 3; ++a) {
                            const double t = s * c * (r[a] / rl) / h;
                            f[a] -= t;
                            sa[a] += fabs(t);
                        }
                    } else {
                        const double G = g_d(kind, h, rl);
                        for (int a = 0; a < 3; ++a) {
                            const double t = s * G * r[a];
                            f[a] -= t;
                            sa[a] += fabs(t);
                        }
                    }
                }
                double lap = 0.0;
                if (kind != 0) lap = lap_d(kind, h, rl);
                else if (q <= 1.0) lap = sigma * (-2.0 + 3.0 * q) / hsq;
                else if (q <= 2.0) lap = sigma * (2.0 - q) / hsq;
                const double s = (double)mass[j] / rho[j] * (double)prm[2];
                for (int a = 0; a < 3; ++a) {
                    const double t = s * ((double)vel[3 * j + a] - (double)vel[3 * i + a]) * lap;
                    f[a] += t;
                    sa[a] += fabs(t);
                }
            }
            const double m = mass[i];
            f[1] += (double)prm[6] * m;
            sa[1] += fabs((double)prm[6] * m);
            for (int a = 0; a < 3; ++a) {
                acc[3 * i + a] = f[a] / m;
                if (sum_abs) sum_abs[3 * i + a] = sa[a] / fabs(m);
            }
        }
        free_block(nl, i1 - i0);
    }
    free(nl);
    hash_free(&hh);
}

/* ---- FP64 evaluation on FP64 positions -------------------------------------------------- */
typedef struct {
    int64_t cx, cy, cz;
    int64_t idx;
} cell_item;

static int cmp_cell_item(const void* a, const void* b) {
    const cell_item* x = (const cell_item*)a;
    const cell_item* y = (const cell_item*)b;
    if (x->cx != y->cx) return x->cx < y->cx ? -1 : 1;
    if (x->cy != y->cy) return x->cy < y->cy ? -1 : 1;
    if (x->cz != y->cz) return x->cz < y->cz ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

/* first index in the sorted items with cell >= (x, y, z) */
static size_t cell_lower(const cell_item* it, size_t n, int64_t x, int64_t y, int64_t z) {
    size_t lo = 0, hi = n;
    while (lo < hi) {
        const size_t mid = (lo + hi) / 2;
        const cell_item* m = &it[mid];
        const int less = m->cx < x || (m->cx == x && (m->cy < y || (m->cy == y && m->cz < z)));
        if (less) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

int64_t orc_fields_f64d(size_t n, const double* pos, const float* vel, const float* mass,
                        const float* params16, double* rho, double* P, double* acc) {
    return orc_fields_f64d_s(n, pos, vel, mass, params16, rho, P, acc, NULL);
}

int64_t orc_fields_f64d_s(size_t n, const double* pos, const float* vel, const float* mass,
                          const float* params16, double* rho, double* P, double* acc,
                          double* sum_abs) {
    float prm[16];
    load_params(params16, prm);
    const double h = prm[3], hsq = h * h, sigma = 1.0 / (M_PI * h * h * h);
    const double r = prm[15], r2 = r * r, cs = r;
    cell_item* it = (cell_item*)malloc((n ? n : 1) * sizeof(cell_item));
    size_t m = 0;
    for (size_t i = 0; i < n; ++i) {
        const double* p = pos + 3 * i;
        if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]))) continue;
        it[m].cx = (int64_t)floor(p[0] / cs);
        it[m].cy = (int64_t)floor(p[1] / cs);
        it[m].cz = (int64_t)floor(p[2] / cs);
        it[m].idx = (int64_t)i;
        ++m;
    }
    qsort(it, m, sizeof(cell_item), cmp_cell_item);
    int64_t* cell_of = (int64_t*)malloc((n ? n : 1) * 3 * sizeof(int64_t));
    unsigned char* ok = (unsigned char*)calloc(n ? n : 1, 1);
    for (size_t k = 0; k < m; ++k) {
        const int64_t i = it[k].idx;
        cell_of[3 * i] = it[k].cx;
        cell_of[3 * i + 1] = it[k].cy;
        cell_of[3 * i + 2] = it[k].cz;
        ok[i] = 1;
    }
    int64_t pairs = 0;
    /* density and pressure over the 5x5x5 stencil (covers r = cell exactly) */
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : pairs)
    for (long long i = 0; i < (long long)n; ++i) {
        double d = (double)mass[i] * sigma * (2.0 / 3.0);
        if (ok[i]) {
            const double* pi = pos + 3 * i;
            for (int dx = -2; dx <= 2; ++dx)
                for (int dy = -2; dy <= 2; ++dy)
                    for (int dz = -2; dz <= 2; ++dz) {
                        const int64_t x = cell_of[3 * i] + dx, y = cell_of[3 * i + 1] + dy,
                                      z = cell_of[3 * i + 2] + dz;
                        for (size_t k = cell_lower(it, m, x, y, z);
                             k < m && it[k].cx == x && it[k].cy == y && it[k].cz == z; ++k) {
                            const int64_t j = it[k].idx;
                            const double* pj = pos + 3 * j;
                            const double rx = pi[0] - pj[0], ry = pi[1] - pj[1], rz = pi[2] - pj[2];
                            const double q2 = rx * rx + ry * ry + rz * rz;
                            if (q2 > r2) continue;
                            ++pairs;
                            if (j == i) continue;
                            d += (double)mass[j] * w3d(sigma, sqrt(q2) / h);
                        }
                    }
        }
        rho[i] = d;
        P[i] = (double)prm[1] * (d - (double)prm[0]);
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        double f[3] = {0, 0, 0}, sa[3] = {0, 0, 0};
        if (ok[i]) {
            const double* pi = pos + 3 * i;
            for (int dx = -2; dx <= 2; ++dx)
                for (int dy = -2; dy <= 2; ++dy)
                    for (int dz = -2; dz <= 2; ++dz) {
                        const int64_t x = cell_of[3 * i] + dx, y = cell_of[3 * i + 1] + dy,
                                      z = cell_of[3 * i + 2] + dz;
                        for (size_t k = cell_lower(it, m, x, y, z);
                             k < m && it[k].cx == x && it[k].cy == y && it[k].cz == z; ++k) {
                            const int64_t j = it[k].idx;
                            if (j == i) continue;
                            const double* pj = pos + 3 * j;
                            const double rv[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
                            const double q2 = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
                            if (q2 > r2) continue;
                            const double rl = sqrt(q2), q = rl / h;
                            if (rl >= 1e-6) {
                                double c = 0.0;
                                if (q <= 1.0) c = sigma * (-2.0 * q + 1.5 * q * q);
                                else if (q <= 2.0) c = -sigma * 0.5 * (2.0 - q) * (2.0 - q);
                                const double s = (double)mass[j] * (P[i] + P[j]) / (2.0 * rho[j]);
                                for (int a = 0; a < 3; ++a) {
                                    const double t = s * c * (rv[a] / rl) / h;
                                    f[a] -= t;
                                    sa[a] += fabs(t);
                                }
                            }
                            double lap = 0.0;
                            if (q <= 1.0) lap = sigma * (-2.0 + 3.0 * q) / hsq;
                            else if (q <= 2.0) lap = sigma * (2.0 - q) / hsq;
                            const double s = (double)mass[j] / rho[j] * (double)prm[2];
                            for (int a = 0; a < 3; ++a) {
                                const double t =
                                    s * ((double)vel[3 * j + a] - (double)vel[3 * i + a]) * lap;
                                f[a] += t;
                                sa[a] += fabs(t);
                            }
                        }
                    }
        }
        const double mm = mass[i];
        f[1] += (double)prm[6] * mm;
        sa[1] += fabs((double)prm[6] * mm);
        for (int a = 0; a < 3; ++a) {
            acc[3 * i + a] = f[a] / mm;
            if (sum_abs) sum_abs[3 * i + a] = sa[a] / fabs(mm);
        }
    }
    free(it);
    free(cell_of);
    free(ok);
    return pairs;
}

/* ------------------------------------------------------------------------------------ */
/* engine                                                                                */
/* ------------------------------------------------------------------------------------ */

struct orc_engine {
    size_t capacity, n;
    float *pos, *vel, *mass, *acc, *rho, *P;
    i64vec* nl;
    float prm[16];
    float cell_size;
    int initialized;
    int kind; /* smoothing kernel (0 cubic spline, the reference engine's fixed choice) */
    float time, last_dt;
    uint64_t steps, max_nn, total_q;
};

orc_engine* orc_engine_new(size_t capacity) {
    orc_engine* e = (orc_engine*)calloc(1, sizeof(orc_engine));
    const size_t c = capacity ? capacity : 1;
    e->capacity = capacity;
    e->pos = (float*)calloc(3 * c, sizeof(float));
    e->vel = (float*)calloc(3 * c, sizeof(float));
    e->mass = (float*)calloc(c, sizeof(float));
    e->acc = (float*)calloc(3 * c, sizeof(float));
    e->rho = (float*)calloc(c, sizeof(float));
    e->P = (float*)calloc(c, sizeof(float));
    e->nl = (i64vec*)calloc(c, sizeof(i64vec));
    /* SPHParameters defaults (src/sph_engine.h:14-34) */
    const float defaults[16] = {1000.0f, 2000.0f, 0.001f, 0.02f, 0.001f, 0.001f,
                                -9.81f,  0.99f,   0.4f,   -1.0f, 1.0f,   -1.0f,
                                1.0f,    -1.0f,   1.0f,   0.04f};
    memcpy(e->prm, defaults, sizeof(defaults));
    e->cell_size = defaults[3];
    return e;
}

void orc_engine_free(orc_engine* e) {
    if (!e) return;
    for (size_t i = 0; i < (e->capacity ? e->capacity : 1); ++i) free(e->nl[i].data);
    free(e->pos);
    free(e->vel);
    free(e->mass);
    free(e->acc);
    free(e->rho);
    free(e->P);
    free(e->nl);
    free(e);
}

/* SPHEngine::initialize (src/sph_engine.cpp:20-33) */
void orc_engine_set_kernel(orc_engine* e, int kind) { e->kind = kind; }

void orc_engine_initialize(orc_engine* e, const float* params16) {
    load_params(params16, e->prm);
    e->cell_size = e->prm[15];
    e->initialized = 1;
    e->max_nn = 0;
    e->total_q = 0;
}

void orc_engine_add(orc_engine* e, size_t n, const float* pos, const float* vel,
                    const float* mass) {
    for (size_t i = 0; i < n; ++i) {
        if (e->n >= e->capacity) continue; /* dropped, src/particle.cpp:27-32 */
        const size_t k = e->n++;
        for (int a = 0; a < 3; ++a) {
            e->pos[3 * k + a] = pos[3 * i + a];
            e->vel[3 * k + a] = vel ? vel[3 * i + a] : 0.0f;
        }
        e->mass[k] = mass[i];
    }
}

void orc_engine_clear(orc_engine* e) {
    e->n = 0;
    e->time = 0.0f;
    e->steps = 0;
}

/* SPHEngine::compute_cfl_timestep (src/sph_engine.cpp:312-333) */
static float cfl_timestep(const orc_engine* e) {
    float max_velocity = 0.0f;
    for (size_t i = 0; i < e->n; ++i) {
        const float v = sqrtf(dot3(e->vel[3 * i], e->vel[3 * i + 1], e->vel[3 * i + 2]));
        max_velocity = (max_velocity < v) ? v : max_velocity;
    }
    const float h = e->prm[3], cfl = e->prm[8];
    const float dt_cfl = cfl * h / (max_velocity + 1e-6f);
    const float a0 = sqrtf(dot3(e->acc[0], e->acc[1], e->acc[2]));
    const float dt_force = cfl * sqrtf(h / (a0 + 1e-6f));
    float r = dt_cfl;
    if (dt_force < r) r = dt_force;
    if (e->prm[5] < r) r = e->prm[5];
    return r;
}

/* SPHEngine::step (src/sph_engine.cpp:93-144) */
void orc_engine_step(orc_engine* e, float dt) {
    if (!e->initialized || e->n == 0) return;
    if (dt <= 0.0f) dt = cfl_timestep(e);
    e->last_dt = dt;
    const size_t n = e->n;
    uint64_t mx = 0;
    build_lists(n, e->pos, e->cell_size, e->prm[15], e->nl, &mx);
    e->total_q += n;
    if (mx > e->max_nn) e->max_nn = mx;
    const kern k = make_kernel(e->kind, e->prm[3]);
    densities(0, n, e->pos, e->mass, e->nl, &k, e->rho);
    pressures(n, e->rho, e->prm[0], e->prm[1], e->P);
    forces(0, n, e->pos, e->vel, e->mass, e->nl, &k, e->rho, e->P, e->prm[2], e->prm[6], e->acc);
    /* integrate_leapfrog (src/sph_engine.cpp:290-310) */
    const float damping = e->prm[7];
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        for (int a = 0; a < 3; ++a) {
            const float half = 0.5f * e->acc[3 * i + a] * dt;
            float v = e->vel[3 * i + a] + half;
            e->pos[3 * i + a] = e->pos[3 * i + a] + v * dt;
            v = v + half;
            e->vel[3 * i + a] = v * damping;
        }
    }
    /* ParticleSystem::apply_boundary_conditions (src/particle.cpp:122-153), serial */
    const float lo[3] = {e->prm[9], e->prm[11], e->prm[13]};
    const float hi[3] = {e->prm[10], e->prm[12], e->prm[14]};
    for (size_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) {
            if (e->pos[3 * i + a] < lo[a]) {
                e->pos[3 * i + a] = lo[a];
                e->vel[3 * i + a] *= -0.8f;
            } else if (e->pos[3 * i + a] > hi[a]) {
                e->pos[3 * i + a] = hi[a];
                e->vel[3 * i + a] *= -0.8f;
            }
        }
    }
    e->time += dt;
    e->steps++;
}

size_t orc_engine_size(const orc_engine* e) { return e->n; }
float orc_engine_time(const orc_engine* e) { return e->time; }
uint64_t orc_engine_step_count(const orc_engine* e) { return e->steps; }
float orc_engine_last_dt(const orc_engine* e) { return e->last_dt; }

void orc_engine_get(const orc_engine* e, float* pos, float* vel, float* acc, float* rho,
                    float* P) {
    if (pos) memcpy(pos, e->pos, 3 * e->n * sizeof(float));
    if (vel) memcpy(vel, e->vel, 3 * e->n * sizeof(float));
    if (acc) memcpy(acc, e->acc, 3 * e->n * sizeof(float));
    if (rho) memcpy(rho, e->rho, e->capacity * sizeof(float));
    if (P) memcpy(P, e->P, e->capacity * sizeof(float));
}

void orc_engine_set_state(orc_engine* e, const float* pos, const float* vel) {
    if (pos) memcpy(e->pos, pos, 3 * e->n * sizeof(float));
    if (vel) memcpy(e->vel, vel, 3 * e->n * sizeof(float));
}

void orc_engine_diag(const orc_engine* e, double* out6) {
    /* get_total_mass: sequential float sum of densities times h^3 */
    float s = 0.0f;
    for (size_t i = 0; i < e->n; ++i) s = s + e->rho[i];
    const float h = e->prm[3];
    const float total_mass = s * (h * h * h);
    /* get_total_energy: sequential float kinetic energy */
    float ke = 0.0f;
    for (size_t i = 0; i < e->n; ++i) {
        const float sp = dot3(e->vel[3 * i], e->vel[3 * i + 1], e->vel[3 * i + 2]);
        ke += 0.5f * e->mass[i] * sp;
    }
    const float initial_mass = (float)e->n * e->prm[4];
    out6[0] = total_mass;
    out6[1] = ke;
    out6[2] = fabsf(total_mass - initial_mass) / initial_mass;
    out6[3] = 0.0;
    out6[4] = (double)e->max_nn;
    out6[5] = (double)e->total_q;
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
