/* CPU restatement of the headless particle renderer (the reference's instanced billboard
 * shaders, shaders/particle.vert:20-40 and shaders/particle.frag:15-104, drawn as in
 * src/renderer.cpp:314-333 with the depth test of renderer.cpp:51).
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): the checker of the CUDA render kernels.  The
 * reference's own output is a GL framebuffer that cannot be produced here (no graphics
 * stack), so this restatement is pinned to the shader source as written, not to
 * reference output ("parity unpinned").  It fixes the float evaluation order of every
 * shader expression and the rasterisation rules:
 *   corners   pos = worldPos + (right * qx) * size + (up * qy) * size, clip = PVM * (pos, 1)
 *             with PVM = (projection * view) * model, sums in index order
 *   colour    the fragment shader's colour modes and 0.3 ambient + 0.7 diffuse
 *   raster    window = ((ndc + 1) * size / 2, ndc_z / 2 + 1/2); pixel centres; edge
 *             functions with a top-left tie rule; depth interpolated barycentrically;
 *             GL_LESS in draw (particle) order against the cleared depth 1.0
 * Compiled with -ffp-contract=off. */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    float view[16], projection[16], model[16];
    float particle_size;
    int color_mode;
    int width, height;
    float background[3];
} orc_render_params;

typedef struct {
    float pvm[16], right[3], up[3], size, diffuse, bg[3];
    int mode, width, height;
} rconst;

static void mat4_mul(const float* A, const float* B, float* C) {
    for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row) {
            float acc = A[row] * B[col * 4];
            for (int k = 1; k < 4; ++k) acc = acc + A[k * 4 + row] * B[col * 4 + k];
            C[col * 4 + row] = acc;
        }
}

static rconst derive(const orc_render_params* p) {
    rconst r;
    float pv[16];
    mat4_mul(p->projection, p->view, pv);
    mat4_mul(pv, p->model, r.pvm);
    for (int a = 0; a < 3; ++a) {
        r.right[a] = p->view[a * 4];
        r.up[a] = p->view[a * 4 + 1];
        r.bg[a] = p->background[a];
    }
    r.size = p->particle_size;
    r.mode = p->color_mode;
    const float len = sqrtf((1.0f * 1.0f + 1.0f * 1.0f) + 1.0f * 1.0f);
    const float lz = 1.0f / len;
    r.diffuse = lz > 0.0f ? lz : 0.0f;
    r.width = p->width;
    r.height = p->height;
    return r;
}

static inline float mix1(float x, float y, float t) { return x * (1.0f - t) + y * t; }
static inline float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }
static inline float len3(float x, float y, float z) {
    const float a = x * x, b = y * y, c = z * z;
    return sqrtf((a + b) + c);
}

static void shade(const rconst* r, float y, const float* v, const float* col, float* out) {
    float c[3];
    if (r->mode == 0) {
        const float t = clamp01(len3(v[0], v[1], v[2]) / 2.0f);
        c[0] = mix1(0.0f, 1.0f, t), c[1] = mix1(0.5f, 0.0f, t), c[2] = mix1(1.0f, 0.0f, t);
    } else if (r->mode == 1) {
        const float d = 1000.0f + y * 200.0f;
        const float t = clamp01((d - 1000.0f) / (2000.0f - 1000.0f));
        c[0] = mix1(0.7f, 0.0f, t), c[1] = mix1(0.9f, 0.2f, t), c[2] = mix1(1.0f, 0.5f, t);
    } else if (r->mode == 2) {
        const float pr = len3(v[0], v[1], v[2]) * 5000.0f;
        const float t = clamp01(pr / 10000.0f);
        c[0] = mix1(0.0f, 1.0f, t), c[1] = mix1(0.8f, 0.0f, t), c[2] = mix1(0.0f, 0.0f, t);
    } else {
        c[0] = col ? col[0] : 0.0f, c[1] = col ? col[1] : 0.5f, c[2] = col ? col[2] : 1.0f;
    }
    for (int a = 0; a < 3; ++a) out[a] = c[a] * 0.3f + (c[a] * r->diffuse) * 0.7f;
}

static const float quad[4][2] = {{-0.5f, -0.5f}, {0.5f, -0.5f}, {0.5f, 0.5f}, {-0.5f, 0.5f}};

static void corner(const rconst* r, const float* w, float qx, float qy, float* o) {
    float p[3];
    for (int a = 0; a < 3; ++a) p[a] = (w[a] + (r->right[a] * qx) * r->size) + (r->up[a] * qy) * r->size;
    for (int row = 0; row < 4; ++row)
        o[row] = ((r->pvm[row] * p[0] + r->pvm[4 + row] * p[1]) + r->pvm[8 + row] * p[2]) +
                 r->pvm[12 + row];
}

void orc_render_instances(const orc_render_params* p, size_t n, const float* pos,
                          const float* vel, const float* colors, float* out) {
    const rconst r = derive(p);
    for (size_t i = 0; i < n; ++i) {
        float* o = out + 20 * i;
        for (int k = 0; k < 4; ++k) corner(&r, pos + 3 * i, quad[k][0], quad[k][1], o + 4 * k);
        shade(&r, pos[3 * i + 1], vel + 3 * i, colors ? colors + 3 * i : NULL, o + 16);
        o[19] = 1.0f;
    }
}

typedef struct {
    float x, y, z;
} v3;

static inline float edge(v3 a, v3 b, float px, float py) {
    return (b.x - a.x) * (py - a.y) - (b.y - a.y) * (px - a.x);
}
static inline int top_left(v3 a, v3 b) {
    const float dx = b.x - a.x, dy = b.y - a.y;
    return dy < 0.0f || (dy == 0.0f && dx < 0.0f);
}

static void raster(const rconst* r, v3 a, v3 b, v3 c, int32_t idx, float* depth,
                   int32_t* owner) {
    float area = edge(a, b, c.x, c.y);
    if (area == 0.0f || !isfinite(area)) return;
    if (area < 0.0f) {
        const v3 t = b;
        b = c;
        c = t;
        area = -area;
    }
    const float xmin = fminf(a.x, fminf(b.x, c.x)), xmax = fmaxf(a.x, fmaxf(b.x, c.x));
    const float ymin = fminf(a.y, fminf(b.y, c.y)), ymax = fmaxf(a.y, fmaxf(b.y, c.y));
    const float fx0 = fmaxf(floorf(xmin - 0.5f), 0.0f);
    const float fx1 = fminf(ceilf(xmax - 0.5f), (float)(r->width - 1));
    const float fy0 = fmaxf(floorf(ymin - 0.5f), 0.0f);
    const float fy1 = fminf(ceilf(ymax - 0.5f), (float)(r->height - 1));
    if (!(fx0 <= fx1 && fy0 <= fy1)) return;
    const int tab = top_left(a, b), tbc = top_left(b, c), tca = top_left(c, a);
    for (int py = (int)fy0; py <= (int)fy1; ++py) {
        const float cy = (float)py + 0.5f;
        for (int px = (int)fx0; px <= (int)fx1; ++px) {
            const float cx = (float)px + 0.5f;
            const float w0 = edge(b, c, cx, cy), w1 = edge(c, a, cx, cy), w2 = edge(a, b, cx, cy);
            const int in = (w0 > 0.0f || (w0 == 0.0f && tbc)) && (w1 > 0.0f || (w1 == 0.0f && tca)) &&
                           (w2 > 0.0f || (w2 == 0.0f && tab));
            if (!in) continue;
            float z = ((w0 * a.z + w1 * b.z) + w2 * c.z) / area;
            z = z + 0.0f;
            if (!(z >= 0.0f && z < 1.0f)) continue;
            const size_t q = (size_t)py * r->width + px;
            if (z < depth[q]) {  /* GL_LESS, particles in draw order */
                depth[q] = z;
                owner[q] = idx;
            }
        }
    }
}

static inline unsigned char unorm8(float v) { return (unsigned char)lrintf(clamp01(v) * 255.0f); }

void orc_render_image(const orc_render_params* p, size_t n, const float* pos, const float* vel,
                      const float* colors, unsigned char* rgba) {
    const rconst r = derive(p);
    const size_t npix = (size_t)r.width * r.height;
    float* depth = (float*)malloc(npix * sizeof(float));
    int32_t* owner = (int32_t*)malloc(npix * sizeof(int32_t));
    for (size_t q = 0; q < npix; ++q) depth[q] = 1.0f, owner[q] = -1;
    for (size_t i = 0; i < n; ++i) {
        float c[4][4];
        int ok = 1;
        for (int k = 0; k < 4; ++k) {
            corner(&r, pos + 3 * i, quad[k][0], quad[k][1], c[k]);
            ok = ok && c[k][3] > 0.0f && c[k][2] >= -c[k][3] && c[k][2] <= c[k][3];
        }
        if (!ok) continue;
        v3 s[4];
        for (int k = 0; k < 4; ++k) {
            const float nx = c[k][0] / c[k][3], ny = c[k][1] / c[k][3], nz = c[k][2] / c[k][3];
            s[k].x = (nx + 1.0f) * (0.5f * (float)r.width);
            s[k].y = (ny + 1.0f) * (0.5f * (float)r.height);
            s[k].z = nz * 0.5f + 0.5f;
        }
        raster(&r, s[0], s[1], s[2], (int32_t)i, depth, owner);
        raster(&r, s[0], s[2], s[3], (int32_t)i, depth, owner);
    }
    for (size_t q = 0; q < npix; ++q) {
        unsigned char* o = rgba + 4 * q;
        if (owner[q] >= 0) {
            const size_t i = (size_t)owner[q];
            float col[3];
            shade(&r, pos[3 * i + 1], vel + 3 * i, colors ? colors + 3 * i : NULL, col);
            o[0] = unorm8(col[0]), o[1] = unorm8(col[1]), o[2] = unorm8(col[2]);
        } else {
            o[0] = unorm8(r.bg[0]), o[1] = unorm8(r.bg[1]), o[2] = unorm8(r.bg[2]);
        }
        o[3] = 255;
    }
    free(depth);
    free(owner);
}
