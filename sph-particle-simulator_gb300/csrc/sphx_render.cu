// Headless particle rendering: the reference's instanced-billboard shader pair
// (shaders/particle.vert:20-40, shaders/particle.frag:15-104, drawn by
// Renderer::render_particles_instanced, src/renderer.cpp:314-333) restated as CUDA
// kernels writing device buffers instead of a GL framebuffer.
//
//  k_render_instances  per particle: the 4 billboard corners in clip space
//                      (projection * view * model * vec4(pos, 1), corners of the quad
//                      (+-0.5, +-0.5) along the camera's right / up axes scaled by
//                      particleSize) and the fragment colour (colour mode + the shader's
//                      ambient/diffuse term, alpha 1)
//  k_render_raster     rasterises the instances' two triangles (GL_TRIANGLE_FAN 0-1-2,
//                      0-2-3) into a width x height depth buffer: pixel centres, top-left
//                      fill rule, depth = window z in [0, 1], GL_LESS against the cleared
//                      1.0; a 64-bit atomicMin of (depth bits, particle index) keeps the
//                      nearest fragment and, for equal depth, the first-drawn instance --
//                      what GL_LESS does in draw order
//  k_render_resolve    depth buffer -> RGBA8 (background where nothing was drawn; colour
//                      channels converted as GL does: round(clamp(c, 0, 1) * 255))
//
// All float arithmetic uses the exact (non-contracted, round-to-nearest) helpers in a fixed
// order, so the CPU restatement in oracle/render_oracle.c reproduces every output bit.
// Quads with a corner outside the clip volume's w > 0 / near / far range are not drawn
// (GL would clip them; particles are far smaller than the view distance).
#include "sphx_internal.cuh"

namespace sphx {

namespace {

// GLSL mix(x, y, a) = x * (1 - a) + y * a
__device__ __forceinline__ float mix1(float x, float y, float t) {
    return xadd(xmul(x, xsub(1.0f, t)), xmul(y, t));
}

// fragment colour of one particle (particle.frag:52-104)
__device__ __forceinline__ float3 shade(const RenderConst& r, float x, float y, float z,
                                        float vx, float vy, float vz, float cr, float cg,
                                        float cb) {
    float3 c;
    if (r.mode == 0) {
        // velocityToColor: mix(blue, red, clamp(|v| / 2, 0, 1))
        const float t = fminf(fmaxf(xdiv(xsqrt(xdot3(vx, vy, vz)), 2.0f), 0.0f), 1.0f);
        c = make_float3(mix1(0.0f, 1.0f, t), mix1(0.5f, 0.0f, t), mix1(1.0f, 0.0f, t));
    } else if (r.mode == 1) {
        // densityToColor(1000 + height * 200) (the shader's placeholder for density)
        const float d = xadd(1000.0f, xmul(y, 200.0f));
        const float t = fminf(fmaxf(xdiv(xsub(d, 1000.0f), xsub(2000.0f, 1000.0f)), 0.0f), 1.0f);
        c = make_float3(mix1(0.7f, 0.0f, t), mix1(0.9f, 0.2f, t), mix1(1.0f, 0.5f, t));
    } else if (r.mode == 2) {
        // pressureToColor(|v| * 5000) (the shader's placeholder for pressure)
        const float p = xmul(xsqrt(xdot3(vx, vy, vz)), 5000.0f);
        const float t = fminf(fmaxf(xdiv(p, 10000.0f), 0.0f), 1.0f);
        c = make_float3(mix1(0.0f, 1.0f, t), mix1(0.8f, 0.0f, t), mix1(0.0f, 0.0f, t));
    } else {
        c = make_float3(cr, cg, cb);  // type colour (the particle's own)
    }
    (void)x;
    (void)z;
    // ambient 0.3 + diffuse 0.7 * max(dot(normal, lightDir), 0)
    c.x = xadd(xmul(c.x, 0.3f), xmul(xmul(c.x, r.diffuse), 0.7f));
    c.y = xadd(xmul(c.y, 0.3f), xmul(xmul(c.y, r.diffuse), 0.7f));
    c.z = xadd(xmul(c.z, 0.3f), xmul(xmul(c.z, r.diffuse), 0.7f));
    return c;
}

// the particle's world position (insertion order; precision mode: cell + offset)
__device__ __forceinline__ float3 world_pos(const RenderArgs& a, int i) {
    const float4 p = a.pos4[i];
    if (!a.cell4) return make_float3(p.x, p.y, p.z);
    const int4 cl = a.cell4[i];
    if (cl.w) return make_float3(p.x, p.y, p.z);  // non-finite: kept as given
    return make_float3((float)((double)cl.x * a.cs + (double)p.x),
                       (float)((double)cl.y * a.cs + (double)p.y),
                       (float)((double)cl.z * a.cs + (double)p.z));
}

// clip-space position of corner (qx, qy) of particle i's billboard
__device__ __forceinline__ float4 corner(const RenderConst& r, float3 w, float qx, float qy) {
    // pos = worldPos + cameraRight * aPos.x * particleSize + cameraUp * aPos.y * particleSize
    const float px = xadd(xadd(w.x, xmul(xmul(r.right[0], qx), r.size)), xmul(xmul(r.up[0], qy), r.size));
    const float py = xadd(xadd(w.y, xmul(xmul(r.right[1], qx), r.size)), xmul(xmul(r.up[1], qy), r.size));
    const float pz = xadd(xadd(w.z, xmul(xmul(r.right[2], qx), r.size)), xmul(xmul(r.up[2], qy), r.size));
    float4 o;
    float* out = &o.x;
#pragma unroll
    for (int row = 0; row < 4; ++row)
        out[row] = xadd(xadd(xadd(xmul(r.pvm[row], px), xmul(r.pvm[4 + row], py)),
                             xmul(r.pvm[8 + row], pz)),
                        r.pvm[12 + row]);
    return o;
}

__constant__ float kQuad[4][2] = {{-0.5f, -0.5f}, {0.5f, -0.5f}, {0.5f, 0.5f}, {-0.5f, 0.5f}};

__global__ void k_render_instances(const RenderConst r, const RenderArgs a, float* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const float3 w = world_pos(a, i);
        const float4 v = a.vel4[i];
        float* o = out + (size_t)i * 20;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 c = corner(r, w, kQuad[k][0], kQuad[k][1]);
            o[4 * k] = c.x;
            o[4 * k + 1] = c.y;
            o[4 * k + 2] = c.z;
            o[4 * k + 3] = c.w;
        }
        const float cr = a.colors ? a.colors[3 * i] : 0.0f;
        const float cg = a.colors ? a.colors[3 * i + 1] : 0.5f;
        const float cb = a.colors ? a.colors[3 * i + 2] : 1.0f;
        const float3 c = shade(r, w.x, w.y, w.z, v.x, v.y, v.z, cr, cg, cb);
        o[16] = c.x;
        o[17] = c.y;
        o[18] = c.z;
        o[19] = 1.0f;
    }
}

// window coordinates of a clip-space vertex (viewport = the image, depth range [0, 1])
__device__ __forceinline__ float3 to_window(const RenderConst& r, float4 c) {
    const float nx = xdiv(c.x, c.w), ny = xdiv(c.y, c.w), nz = xdiv(c.z, c.w);
    return make_float3(xmul(xadd(nx, 1.0f), xmul(0.5f, (float)r.width)),
                       xmul(xadd(ny, 1.0f), xmul(0.5f, (float)r.height)),
                       xadd(xmul(nz, 0.5f), 0.5f));
}

__device__ __forceinline__ bool in_clip(float4 c) {
    return c.w > 0.0f && c.z >= -c.w && c.z <= c.w;
}

// edge function of (a, b) at p (twice the signed area of a, b, p)
__device__ __forceinline__ float edge(float3 a, float3 b, float px, float py) {
    return xsub(xmul(xsub(b.x, a.x), xsub(py, a.y)), xmul(xsub(b.y, a.y), xsub(px, a.x)));
}

// top-left rule for a counter-clockwise (positive area) triangle in y-up window space:
// a pixel centre exactly on an edge belongs to the triangle if the edge is a left edge
// (going down) or a top edge (horizontal, going left)
__device__ __forceinline__ bool top_left(float3 a, float3 b) {
    const float dx = xsub(b.x, a.x), dy = xsub(b.y, a.y);
    return dy < 0.0f || (dy == 0.0f && dx < 0.0f);
}

__device__ __forceinline__ void raster_triangle(const RenderConst& r, float3 a, float3 b,
                                                float3 c, uint32_t idx,
                                                unsigned long long* keys) {
    float area = edge(a, b, c.x, c.y);
    if (area == 0.0f || !isfinite(area)) return;  // degenerate, or a non-finite corner
    if (area < 0.0f) {  // both windings are drawn (no face culling): make it CCW
        const float3 t = b;
        b = c;
        c = t;
        area = -area;
    }
    const float xmin = fminf(a.x, fminf(b.x, c.x)), xmax = fmaxf(a.x, fmaxf(b.x, c.x));
    const float ymin = fminf(a.y, fminf(b.y, c.y)), ymax = fmaxf(a.y, fmaxf(b.y, c.y));
    // pixel (px, py) has its centre at (px + 0.5, py + 0.5); clamp in float before the
    // integer conversion (window coordinates of far off-screen corners can be huge)
    const float fx0 = fmaxf(floorf(xsub(xmin, 0.5f)), 0.0f);
    const float fx1 = fminf(ceilf(xsub(xmax, 0.5f)), (float)(r.width - 1));
    const float fy0 = fmaxf(floorf(xsub(ymin, 0.5f)), 0.0f);
    const float fy1 = fminf(ceilf(xsub(ymax, 0.5f)), (float)(r.height - 1));
    if (!(fx0 <= fx1 && fy0 <= fy1)) return;
    const int x0 = (int)fx0, x1 = (int)fx1, y0 = (int)fy0, y1 = (int)fy1;
    const bool tab = top_left(a, b), tbc = top_left(b, c), tca = top_left(c, a);
    for (int py = y0; py <= y1; ++py) {
        const float cy = (float)py + 0.5f;
        for (int px = x0; px <= x1; ++px) {
            const float cx = (float)px + 0.5f;
            const float w0 = edge(b, c, cx, cy), w1 = edge(c, a, cx, cy), w2 = edge(a, b, cx, cy);
            const bool in = (w0 > 0.0f || (w0 == 0.0f && tbc)) && (w1 > 0.0f || (w1 == 0.0f && tca)) &&
                            (w2 > 0.0f || (w2 == 0.0f && tab));
            if (!in) continue;
            // depth: barycentric interpolation of window z (affine in window space)
            // (+ 0 turns a -0 into +0, whose bits order correctly in the key)
            const float z =
                xadd(xdiv(xadd(xadd(xmul(w0, a.z), xmul(w1, b.z)), xmul(w2, c.z)), area), 0.0f);
            if (!(z >= 0.0f && z < 1.0f)) continue;  // GL_LESS against the cleared 1.0
            const unsigned long long key =
                ((unsigned long long)__float_as_uint(z) << 32) | (unsigned long long)idx;
            atomicMin(keys + (size_t)py * r.width + px, key);
        }
    }
}

__global__ void k_render_raster(const RenderConst r, const RenderArgs a,
                                unsigned long long* keys) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const float3 w = world_pos(a, i);
        float4 c[4];
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            c[k] = corner(r, w, kQuad[k][0], kQuad[k][1]);
            ok = ok && in_clip(c[k]);
        }
        if (!ok) continue;
        float3 s[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) s[k] = to_window(r, c[k]);
        raster_triangle(r, s[0], s[1], s[2], (uint32_t)i, keys);
        raster_triangle(r, s[0], s[2], s[3], (uint32_t)i, keys);
    }
}

__device__ __forceinline__ unsigned char to_unorm8(float v) {
    return (unsigned char)__float2int_rn(xmul(fminf(fmaxf(v, 0.0f), 1.0f), 255.0f));
}

// depth buffer -> RGBA8, rows bottom-up as GL stores them
__global__ void k_render_resolve(const RenderConst r, const RenderArgs a,
                                 const unsigned long long* keys, uchar4* rgba) {
    const size_t npix = (size_t)r.width * r.height;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix;
         p += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long key = keys[p];
        const uint32_t idx = (uint32_t)(key & 0xffffffffull);
        uchar4 o;
        if (idx < (uint32_t)a.n) {
            const float3 w = world_pos(a, (int)idx);
            const float4 v = a.vel4[idx];
            const float cr = a.colors ? a.colors[3 * idx] : 0.0f;
            const float cg = a.colors ? a.colors[3 * idx + 1] : 0.5f;
            const float cb = a.colors ? a.colors[3 * idx + 2] : 1.0f;
            const float3 c = shade(r, w.x, w.y, w.z, v.x, v.y, v.z, cr, cg, cb);
            o = make_uchar4(to_unorm8(c.x), to_unorm8(c.y), to_unorm8(c.z), 255);
        } else {
            o = make_uchar4(to_unorm8(r.bg[0]), to_unorm8(r.bg[1]), to_unorm8(r.bg[2]), 255);
        }
        rgba[p] = o;
    }
}

__global__ void k_fill_u64(unsigned long long* p, size_t n, unsigned long long v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

}  // namespace

// depth 1.0 (the bits of 1.0f) and no particle (index 0xffffffff)
constexpr unsigned long long kClearedKey = (0x3f800000ull << 32) | 0xffffffffull;

int launch_render_instances(const LaunchCtx& L, const RenderConst& r, const RenderArgs& a,
                            float* out) {
    if (a.n <= 0) return 0;
    const int blocks = min((a.n + 255) / 256, L.num_sms * 8);
    k_render_instances<<<blocks, 256, 0, L.stream>>>(r, a, out);
    return 1;
}

int launch_render_image(const LaunchCtx& L, const RenderConst& r, const RenderArgs& a,
                        unsigned long long* keys, uchar4* rgba) {
    const size_t npix = (size_t)r.width * r.height;
    const int pblocks = (int)min((npix + 255) / 256, (size_t)L.num_sms * 8);
    // cleared depth 1.0 with no particle: an index no particle has
    k_fill_u64<<<pblocks, 256, 0, L.stream>>>(keys, npix, kClearedKey);
    int k = 1;
    if (a.n > 0) {
        const int blocks = min((a.n + 127) / 128, L.num_sms * 16);
        k_render_raster<<<blocks, 128, 0, L.stream>>>(r, a, keys);
        ++k;
    }
    k_render_resolve<<<pblocks, 256, 0, L.stream>>>(r, a, keys, rgba);
    return k + 1;
}

}  // namespace sphx
