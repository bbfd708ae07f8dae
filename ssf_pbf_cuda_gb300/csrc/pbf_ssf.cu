// Headless screen-space fluid (SSF) rendering: the reference's per-frame GL
// passes (src/main.cpp:372-564; shaders in asset/shader/) written as CUDA
// kernels that fill device image buffers.  Nothing here touches a graphics
// API: the rasteriser's coverage and attribute interpolation, the depth
// test, bilinear texture filtering and blending are spelled out.
//
// Images are row-major, row 0 at the bottom (GL window coordinates); pixel
// (i, j) has its centre at (i + 0.5, j + 0.5).
//
// This file is compiled with -fmad=false: every product and sum is rounded
// on its own, in the order written, like the CPU restatement built with
// -ffp-contract=off.  The depth splat and the normal pass therefore agree
// with it bit for bit; blur and shading differ only where expf / powf do.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "pbf_engine.h"

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) {                              \
            pbf103::set_last_error(#call, e_);                \
            return PBF_ERROR_CUDA;                            \
        }                                                     \
    } while (0)

namespace pbf103 {
void set_last_error(const char *what, cudaError_t e);

namespace {

constexpr uint32_t kMaxSide = 8192;    // pixel-centre texel fetches stay exact up to here
constexpr uint32_t kEmptyDepth = 0x3f800000u;  // 1.0f, the depth clear (main.cpp:71-72)

// Per-frame constants, passed by value to every kernel.
struct Frame {
    uint32_t w, h, mode, pad;
    float proj[16], view[16], inv_proj[16];  // column-major m[c * 4 + r]
    float radius, point_scale, znear, zfar;
    float blur_radius, blur_scale, thickness, pad1;
    float clear[4];
    float incident[3];
    float inv_w, inv_h;  // 1 / width, 1 / height: tex_coord = (i + 0.5) * inv_w
};

// GLSL mat4 * vec4 (column-major), summed in column order.
__host__ __device__ inline float4 mat_vec(const float *m, float x, float y, float z, float w)
{
    return make_float4(m[0] * x + m[4] * y + m[8] * z + m[12] * w, m[1] * x + m[5] * y + m[9] * z + m[13] * w,
                       m[2] * x + m[6] * y + m[10] * z + m[14] * w, m[3] * x + m[7] * y + m[11] * z + m[15] * w);
}

__host__ __device__ inline float dot3(float ax, float ay, float az, float bx, float by, float bz)
{
    return ax * bx + ay * by + az * bz;
}

// ------------------------------------------------------------ depth splat --

// What the fragments of one particle share.
struct Splat {
    float x0, y0;       // quad: window corner a; sprite: window centre
    float rx, ry;       // quad: 1 / window width, height of the quad; sprite: 1 / size
    float ez;           // view-space depth of the centre (pos_from_eye.z)
    int i0, j0;         // first covered pixel column / row
    uint32_t bw, bh;    // covered pixel box
};

__device__ inline int clamp_pix(float v, uint32_t n)
{
    v = fminf(fmaxf(v, -1.f), (float)n);
    return (int)v;
}

// Pixels whose centre c satisfies lo <= c < hi: [first, last], clipped to
// the image; false when none.
__device__ inline bool centre_range(float lo, float hi, uint32_t n, int &first, int &last)
{
    int a = max(clamp_pix(floorf(lo - 0.5f), n), 0);
    for (int k = 0; k < 3 && a < (int)n && !((float)a + 0.5f >= lo); ++k) ++a;
    int b = min(clamp_pix(floorf(hi - 0.5f) + 1.f, n), (int)n - 1);
    for (int k = 0; k < 3 && b >= a && !((float)b + 0.5f < hi); ++k) --b;
    first = a;
    last = b;
    return a <= b && a < (int)n && (float)a + 0.5f >= lo && (float)b + 0.5f < hi;
}

// Per-particle set-up.  false: nothing of the particle reaches the image.
__device__ inline bool splat_setup(const Frame &f, float px, float py, float pz, Splat &s)
{
    const float4 e = mat_vec(f.view, px, py, pz, 1.f);  // vw * vec4(Position, 1), World = identity
    const float hw = (float)f.w * 0.5f, hh = (float)f.h * 0.5f;
    s.ez = e.z;
    float x0, x1, y0, y1;
    if (f.mode == PBF_SSF_SPLAT_QUAD) {
        // ssf_object.geom:21-50: corners P.xy +- 0.5 point_radius at P.zw
        const float hr = 0.5f * f.radius;
        const float ax = e.x - hr, ay = e.y - hr, dx = e.x + hr, by = e.y + hr;
        const float4 ca = mat_vec(f.proj, ax, ay, e.z, e.w);
        const float4 cd = mat_vec(f.proj, dx, ay, e.z, e.w);
        const float4 cb = mat_vec(f.proj, ax, by, e.z, e.w);
        // clip z and w depend on (z, w) alone, so the four corners clip alike
        if (!(-ca.w <= ca.z && ca.z <= ca.w)) return false;
        x0 = ca.x / ca.w * hw + hw;
        x1 = cd.x / cd.w * hw + hw;
        y0 = ca.y / ca.w * hh + hh;
        y1 = cb.y / cb.w * hh + hh;
        // counter-clockwise strip a, d, b, c is front-facing; a mirrored
        // quad is culled (GL_CULL_FACE, main.cpp:73)
        if (!(x1 > x0 && y1 > y0)) return false;
        s.x0 = x0;
        s.y0 = y0;
        s.rx = 1.f / (x1 - x0);
        s.ry = 1.f / (y1 - y0);
    } else {
        // ssf_point_sprite.vert:19-27: size = pointRadius * (pointScale / dist)
        const float dist = sqrtf(dot3(e.x, e.y, e.z, e.x, e.y, e.z));
        const float size = f.radius * (f.point_scale / dist);
        const float4 c = mat_vec(f.proj, e.x, e.y, e.z, 1.f);
        // a point is kept whole or dropped by its vertex's clip test
        if (!(-c.w <= c.x && c.x <= c.w && -c.w <= c.y && c.y <= c.w && -c.w <= c.z && c.z <= c.w)) return false;
        if (!(size > 0.f)) return false;
        const float xw = c.x / c.w * hw + hw, yw = c.y / c.w * hh + hh, half = size * 0.5f;
        x0 = xw - half;
        x1 = xw + half;
        y0 = yw - half;
        y1 = yw + half;
        s.x0 = xw;
        s.y0 = yw;
        s.rx = s.ry = 1.f / size;
    }
    int i1, j1;
    if (!centre_range(x0, x1, f.w, s.i0, i1) || !centre_range(y0, y1, f.h, s.j0, j1)) return false;
    s.bw = (uint32_t)(i1 - s.i0 + 1);
    s.bh = (uint32_t)(j1 - s.j0 + 1);
    return true;
}

// One fragment: ssf_object.frag:18-35 / ssf_point_sprite.frag:17-31.
// Returns the window depth, or a negative value when nothing is written.
// With the projection's z and w rows free of x and y, the depth needs only
// the z of pixelPos: clip.z / clip.w = (P22 z + P32) / (P23 z + P33).
__device__ inline float splat_fragment(const Frame &f, const Splat &s, int i, int j)
{
    const float cx = (float)i + 0.5f, cy = (float)j + 0.5f;
    float nx, ny;
    if (f.mode == PBF_SSF_SPLAT_QUAD) {
        // vertex_uv * 2 - 1; w is constant over the quad, so the perspective-
        // correct interpolation is the screen-space one
        nx = ((cx - s.x0) * s.rx) * 2.f - 1.f;
        ny = ((cy - s.y0) * s.ry) * 2.f - 1.f;
    } else {
        // gl_PointCoord (origin upper left) * (2, -2) + (-1, 1)
        nx = (0.5f + (cx - s.x0) * s.rx) * 2.f + -1.f;
        ny = (0.5f - (cy - s.y0) * s.ry) * -2.f + 1.f;
    }
    const float mag = nx * nx + ny * ny;
    if (mag > 1.f) return -1.f;  // discard: outside the circle
    const float pz = s.ez + sqrtf(1.f - mag) * f.radius;
    const float d = (f.proj[10] * pz + f.proj[14]) / (f.proj[11] * pz + f.proj[15]);
    if (d != d) return -1.f;
    return fminf(fmaxf(d, 0.f), 1.f) + 0.f;  // clamped to the depth range; + 0 turns -0 into +0
}

// Early depth rejection, exact: no fragment of the particle is nearer than
// its front point (nz = 1) by more than the rounding of the depth formula,
// so a pixel already holding a depth at or below the bound keeps it.
__device__ inline uint32_t front_bound(const Frame &f, float ez)
{
    const float pz = ez + f.radius;
    const float num = f.proj[10] * pz + f.proj[14], den = f.proj[11] * pz + f.proj[15];
    const float d = num / den;
    // |float - exact| <= 2^-22 (|P22 pz| + |P32|) / |den| + ulp / 2; four times that
    const float err = 4.f * (2.3841858e-7f * (fabsf(f.proj[10] * pz) + fabsf(f.proj[14])) / fabsf(den) + 6e-8f);
    const float b = d - err;
    if (!(b > 0.f)) return 0u;  // also NaN
    return __float_as_uint(fminf(b, 1.f));
}

// A particle's splat as the raster kernel reads it (32 B): (x0, y0, rx, ry)
// and (ez bits, depth bound bits, i0 | j0 << 16, bw | bh << 16); bw = 0 when
// nothing of the particle reaches the image.
struct SplatRec {
    float4 a;
    uint4 b;
};

// One thread per particle: the per-particle set-up, once.
template <int STRIDE>
__global__ void __launch_bounds__(256) k_ssf_setup(const float *__restrict__ x, const uint32_t *__restrict__ n_dev,
                                                   uint32_t n_arg, Frame f, SplatRec *__restrict__ rec)
{
    const uint32_t n = n_dev ? *n_dev : n_arg;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const float *xp = x + (size_t)p * STRIDE;
        Splat s;
        SplatRec r;
        if (splat_setup(f, __ldg(xp), __ldg(xp + 1), __ldg(xp + 2), s)) {
            r.a = make_float4(s.x0, s.y0, s.rx, s.ry);
            r.b = make_uint4(__float_as_uint(s.ez), front_bound(f, s.ez), (uint32_t)s.i0 | ((uint32_t)s.j0 << 16),
                             s.bw | (s.bh << 16));
        } else {
            r.a = make_float4(0.f, 0.f, 0.f, 0.f);
            r.b = make_uint4(0u, 0u, 0u, 0u);
        }
        rec[p] = r;
    }
}

// One warp per particle, lanes over its pixel box (stepped without
// division).  The depth test (GL_LESS against the cleared 1.0) is an atomic
// minimum on the float bits, which order like the values in [0, 1]; the
// result does not depend on the order of fragments.
__global__ void __launch_bounds__(256) k_ssf_raster(const SplatRec *__restrict__ rec,
                                                    const uint32_t *__restrict__ n_dev, uint32_t n_arg, Frame f,
                                                    uint32_t *__restrict__ depth)
{
    const uint32_t n = n_dev ? *n_dev : n_arg;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    // Draw near particles first, so the early rejection finds nearer depths
    // already in place: particle sets are often ordered along one axis
    // (lattices, cell-sorted phases), so walk them in reverse when the last
    // particle sits nearer the camera than the first.  Order changes no
    // result: the depth test keeps the minimum.
    bool reverse = false;
    if (n > 1) {
        const float z0 = __uint_as_float(rec[0].b.x), z1 = __uint_as_float(rec[n - 1].b.x);
        reverse = z1 > z0;  // view space looks down -z: larger z is nearer
    }
    for (uint32_t p0 = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); p0 < n; p0 += warps) {
        const uint32_t p = reverse ? n - 1 - p0 : p0;
        const uint4 rb = rec[p].b;
        const uint32_t bw = rb.w & 0xffffu;
        if (bw == 0u) continue;
        const float4 ra = rec[p].a;
        Splat q;
        q.x0 = ra.x;
        q.y0 = ra.y;
        q.rx = ra.z;
        q.ry = ra.w;
        q.ez = __uint_as_float(rb.x);
        q.i0 = (int)(rb.z & 0xffffu);
        q.j0 = (int)(rb.z >> 16);
        q.bw = bw;
        q.bh = rb.w >> 16;
        const uint32_t bound = rb.y;
        const uint32_t dj = 32u / q.bw, di = 32u % q.bw;
        // two cursors, 32 fragments apart, so two depth loads are in flight
        uint32_t ci = lane % q.bw, cj = lane / q.bw;
        uint32_t ci2 = ci + di, cj2 = cj + dj;
        if (ci2 >= q.bw) {
            ci2 -= q.bw;
            ++cj2;
        }
        while (cj < q.bh) {
            const bool two = cj2 < q.bh;
            const int i1 = q.i0 + (int)ci, j1 = q.j0 + (int)cj, i2 = q.i0 + (int)ci2, j2 = q.j0 + (int)cj2;
            uint32_t *d1 = depth + (size_t)j1 * f.w + (uint32_t)i1;
            uint32_t *d2 = two ? depth + (size_t)j2 * f.w + (uint32_t)i2 : d1;
            const uint32_t c1 = *d1, c2 = *d2;
            if (c1 > bound) {
                const float d = splat_fragment(f, q, i1, j1);
                if (d >= 0.f && __float_as_uint(d) < c1) atomicMin(d1, __float_as_uint(d));
            }
            if (two && c2 > bound) {
                const float d = splat_fragment(f, q, i2, j2);
                if (d >= 0.f && __float_as_uint(d) < c2) atomicMin(d2, __float_as_uint(d));
            }
            // both cursors advance 64 fragments
            ci = ci2 + di;
            cj = cj2 + dj;
            if (ci >= q.bw) {
                ci -= q.bw;
                ++cj;
            }
            ci2 = ci + di;
            cj2 = cj + dj;
            if (ci2 >= q.bw) {
                ci2 -= q.bw;
                ++cj2;
            }
        }
    }
}

__global__ void k_ssf_fill(uint32_t *__restrict__ dst, uint32_t value, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = value;
}

// --------------------------------------------------------- screen passes --

// texture(tex, (s, t)) of a one-channel float texture with GL_LINEAR and
// GL_CLAMP_TO_EDGE.  The filter weights keep 8 fractional bits, as in the
// texture unit, so a fetch at a texel centre returns the texel itself.
__device__ inline float sample(const float *__restrict__ T, uint32_t W, uint32_t H, float s, float t)
{
    const float u = s * (float)W - 0.5f, v = t * (float)H - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = rintf((u - fu) * 256.f) * (1.f / 256.f), b = rintf((v - fv) * 256.f) * (1.f / 256.f);
    const int iu = clamp_pix(fu, W), iv = clamp_pix(fv, H);
    const int i0 = min(max(iu, 0), (int)W - 1), i1 = min(max(iu + 1, 0), (int)W - 1);
    const int j0 = min(max(iv, 0), (int)H - 1), j1 = min(max(iv + 1, 0), (int)H - 1);
    // a texel with weight 0 adds +0 to a sum of non-negative terms: not loaded
    const float *r0 = T + (size_t)j0 * W, *r1 = T + (size_t)j1 * W;
    const float t00 = __ldg(r0 + i0), t10 = a != 0.f ? __ldg(r0 + i1) : 0.f;
    const float t01 = b != 0.f ? __ldg(r1 + i0) : 0.f, t11 = (a != 0.f && b != 0.f) ? __ldg(r1 + i1) : 0.f;
    const float a1 = 1.f - a, b1 = 1.f - b;
    return (a1 * b1) * t00 + (a * b1) * t10 + (a1 * b) * t01 + (a * b) * t11;
}

// ssf_blur.frag:27-34
__device__ inline float linearize(float d, const Frame &f) { return (2.f * f.znear) / (f.zfar + f.znear - d * (f.zfar - f.znear)); }
__device__ inline float exponentialize(float l, const Frame &f)
{
    return (f.zfar + f.znear - (2.f * f.znear) / l) / (f.zfar - f.znear);
}

// uvToEye: ssf_blur.frag:36-42 and ssf_shading.frag flip y (t * -2 + 1);
// ssf_normal.frag:17-23 does not (t * 2 - 1).
__device__ inline float3 uv_to_eye(const Frame &f, float s, float t, float d, bool flip)
{
    const float x = s * 2.f - 1.f;
    const float y = flip ? t * -2.f + 1.f : t * 2.f - 1.f;
    const float4 c = mat_vec(f.inv_proj, x, y, d, 1.f);
    return make_float3(c.x / c.w, c.y / c.w, c.z / c.w);
}

// gl_FragDepth written into a depth target cleared to 1.0 with GL_LESS
__device__ inline float depth_store(float v)
{
    if (v != v) return 1.f;
    return fminf(fmaxf(v, 0.f), 1.f);
}

// ssf_blur.frag:44-139: 8 taps along s and 8 along t (the centre twice),
// spatial weight exp(-x^2 r) and the range term as written.  exp(-x^2 r)
// depends on |x| only, so its five values are computed once; the range
// weight is exp(-0) = 1 where the shader's r2 is 0.
__global__ void __launch_bounds__(256) k_ssf_blur(const float *__restrict__ in, float *__restrict__ out, Frame f)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= f.w || j >= f.h) return;
    // the centre tap: at a texel centre the 8-bit filter weights round to 0
    // and 1 (sides up to 8192), so the filtered value is the texel itself
    const float ed = __ldg(in + (size_t)j * f.w + i);
    if (ed == 1.f) {
        out[(size_t)j * f.w + i] = 1.f;
        return;
    }
    const float s = ((float)i + 0.5f) * f.inv_w, t = ((float)j + 0.5f) * f.inv_h;
    const float lin = linearize(ed, f);
    const float3 p = uv_to_eye(f, s, t, ed, true);
    const float dist = sqrtf(dot3(p.x, p.y, p.z, p.x, p.y, p.z));
    const float br = f.blur_radius * f.blur_scale / dist;
    float wk[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) wk[k] = expf(-((float)(k * k) * br));
    float sum = 0.f, wsum = 0.f;
#pragma unroll
    for (int axis = 0; axis < 2; ++axis) {
#pragma unroll
        for (int k = -4; k < 4; ++k) {
            const float sd = axis == 0 ? sample(in, f.w, f.h, s + (float)k * br, t)
                                       : sample(in, f.w, f.h, s, t + (float)k * br);
            if (sd != 1.f) {
                const float sl = linearize(sd, f);
                const float w = wk[k < 0 ? -k : k];
                const float diff = sl - lin;
                const float r2 = fabsf(diff) < 0.01f ? diff * 100.f : 0.f;
                const float g = r2 != 0.f ? expf(-r2 * r2) : 1.f;
                sum = sum + sl * w * g;
                wsum = wsum + w * g;
            }
        }
    }
    if (wsum > 0.f) sum = sum / wsum;
    out[(size_t)j * f.w + i] = depth_store(exponentialize(sum, f));
}

__device__ inline float3 eye_at(const Frame &f, const float *__restrict__ D, int i, int j)
{
    const int ic = min(max(i, 0), (int)f.w - 1), jc = min(max(j, 0), (int)f.h - 1);
    const float s = ((float)i + 0.5f) * f.inv_w, t = ((float)j + 0.5f) * f.inv_h;
    return uv_to_eye(f, s, t, __ldg(D + (size_t)jc * f.w + ic), false);
}

// ssf_normal.frag:25-36: normalize(cross(dFdx(p), dFdy(p))) with fine
// derivatives of the 2x2 pixel quad; a quad partner on the empty side (or
// past an odd edge) still supplies its position, as a helper invocation does.
__global__ void __launch_bounds__(256) k_ssf_normal(const float *__restrict__ D, float4 *__restrict__ N, Frame f)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= f.w || j >= f.h) return;
    const size_t o = (size_t)j * f.w + i;
    if (__ldg(D + o) == 1.f) {  // discard: the target keeps its clear colour
        N[o] = make_float4(f.clear[0], f.clear[1], f.clear[2], f.clear[3]);
        return;
    }
    const int ie = (int)(i & ~1u), je = (int)(j & ~1u);
    const float3 px0 = eye_at(f, D, ie, (int)j), px1 = eye_at(f, D, ie + 1, (int)j);
    const float3 py0 = eye_at(f, D, (int)i, je), py1 = eye_at(f, D, (int)i, je + 1);
    const float dxx = px1.x - px0.x, dxy = px1.y - px0.y, dxz = px1.z - px0.z;
    const float dyx = py1.x - py0.x, dyy = py1.y - py0.y, dyz = py1.z - py0.z;
    const float cx = dxy * dyz - dyy * dxz, cy = dxz * dyx - dyz * dxx, cz = dxx * dyy - dyx * dxy;
    const float inv = 1.f / sqrtf(dot3(cx, cy, cz, cx, cy, cz));
    N[o] = make_float4(cx * inv, cy * inv, cz * inv, 1.f);
}

__device__ inline float clamp01(float v) { return fminf(fmaxf(v, 0.f), 1.f); }

// ssf_shading.frag:36-83, blended (SRC_ALPHA, ONE_MINUS_SRC_ALPHA) onto the
// cleared 8-bit framebuffer (main.cpp:541-564): source and factors clamp to
// [0, 1] first, as for a fixed-point colour buffer.
__global__ void __launch_bounds__(256) k_ssf_shade(const float *__restrict__ D, const float4 *__restrict__ N,
                                                   float4 *__restrict__ C, uchar4 *__restrict__ C8, Frame f)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= f.w || j >= f.h) return;
    const size_t o = (size_t)j * f.w + i;
    const float ed = __ldg(D + o);
    float4 out;
    if (ed == 1.f) {
        out = make_float4(f.clear[0], f.clear[1], f.clear[2], f.clear[3]);
    } else {
        const float4 n = N[o];
        const float th = clamp01(f.thickness);
        const float s = ((float)i + 0.5f) * f.inv_w, t = ((float)j + 0.5f) * f.inv_h;
        const float3 p = uv_to_eye(f, s, t, ed, true);
        const float il = f.incident[0], jl = f.incident[1], kl = f.incident[2];
        const float vr = 1.f / sqrtf(dot3(-p.x, -p.y, -p.z, -p.x, -p.y, -p.z));
        const float vx = -p.x * vr, vy = -p.y * vr, vz = -p.z * vr;
        const float hx = il + vx, hy = jl + vy, hz = kl + vz;
        const float hr = 1.f / sqrtf(dot3(hx, hy, hz, hx, hy, hz));
        const float specular = powf(fmaxf(0.f, dot3(hx * hr, hy * hr, hz * hr, n.x, n.y, n.z)), 50.f);
        const float diffuse = fmaxf(0.f, dot3(il, jl, kl, n.x, n.y, n.z));
        const float r0 = 0.3f;
        const float fres = r0 + (1.f - r0) * powf(1.f - dot3(n.x, n.y, n.z, vx, vy, vz), 5.f);
        const float ar = expf(-5.f * th), ag = expf(-1.f * th), ab = expf(-0.1f * th);
        const float a = th;
        const float ia = 1.f - a;
        out.x = clamp01(clamp01(ar * diffuse + specular * 1.f + 1.f * fres) * a + f.clear[0] * ia);
        out.y = clamp01(clamp01(ag * diffuse + specular * 1.f + 1.f * fres) * a + f.clear[1] * ia);
        out.z = clamp01(clamp01(ab * diffuse + specular * 1.f + 1.f * fres) * a + f.clear[2] * ia);
        out.w = clamp01(a * a + f.clear[3] * ia);
    }
    C[o] = out;
    C8[o] = make_uchar4((unsigned char)rintf(clamp01(out.x) * 255.f), (unsigned char)rintf(clamp01(out.y) * 255.f),
                        (unsigned char)rintf(clamp01(out.z) * 255.f), (unsigned char)rintf(clamp01(out.w) * 255.f));
}

// ------------------------------------------------------------------ host --

bool inverse4(const float *m, float *out)
{
    // Gauss-Jordan with partial pivoting in double, rounded once to float
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (a[piv][c] == 0.0 || !std::isfinite(a[piv][c])) return false;
        if (piv != c)
            for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
        const double d = a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            const double g = a[r][c];
            for (int k = 0; k < 8; ++k) a[r][k] -= g * a[c][k];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = (float)a[r][c + 4];
    return true;
}

}  // namespace
}  // namespace pbf103

using namespace pbf103;

struct pbf_ssf_renderer {
    int device = 0;
    int sms = 0;
    pbf_ssf_params p{};
    Frame f{};
    uint32_t *depth = nullptr;
    float *blur[2] = {nullptr, nullptr};
    float4 *normal = nullptr, *color = nullptr;
    uchar4 *rgba8 = nullptr;
    const float *blurred = nullptr, *blur_input = nullptr;
    SplatRec *rec = nullptr;   // per-particle splat records, grown to the largest particle bound seen
    uint32_t rec_cap = 0;
    uint32_t launches = 0;
};

namespace {

inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// glm::normalize: x * inversesqrt(dot(x, x)), inversesqrt = 1 / sqrt
void normalize3(float v[3])
{
    const float inv = 1.f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] = v[0] * inv;
    v[1] = v[1] * inv;
    v[2] = v[2] * inv;
}

void cross3(const float a[3], const float b[3], float out[3])
{
    out[0] = a[1] * b[2] - b[1] * a[2];
    out[1] = a[2] * b[0] - b[2] * a[0];
    out[2] = a[0] * b[1] - b[0] * a[1];
}

pbf_status launch_frame(pbf_ssf_renderer *r, const float *x, int stride, const uint32_t *n_dev, uint32_t n,
                        uint32_t n_upper, cudaStream_t st)
{
    CK(cudaSetDevice(r->device));
    const Frame &f = r->f;
    const uint32_t px = f.w * f.h;
    uint32_t launches = 0;
    k_ssf_fill<<<std::min<uint32_t>((px + 255) / 256, (uint32_t)r->sms * 8), 256, 0, st>>>(r->depth, kEmptyDepth, px);
    ++launches;
    if (n_upper) {
        if (n_upper > r->rec_cap) {
            // the only allocation on the frame path: the first frame of a
            // larger particle bound (cudaFree waits for frames in flight)
            CK(cudaFree(r->rec));
            r->rec = nullptr;
            r->rec_cap = 0;
            CK(cudaMalloc(&r->rec, sizeof(SplatRec) * (size_t)n_upper));
            r->rec_cap = n_upper;
        }
        const uint32_t sblocks = std::min<uint32_t>((n_upper + 255) / 256, (uint32_t)r->sms * 8);
        if (stride == 4)
            k_ssf_setup<4><<<sblocks, 256, 0, st>>>(x, n_dev, n, f, r->rec);
        else
            k_ssf_setup<3><<<sblocks, 256, 0, st>>>(x, n_dev, n, f, r->rec);
        const uint32_t rblocks = std::min<uint32_t>((n_upper + 7) / 8, (uint32_t)r->sms * 8);
        k_ssf_raster<<<rblocks, 256, 0, st>>>(r->rec, n_dev, n, f, r->depth);
        launches += 2;
    }
    const dim3 blk(32, 8), grd((f.w + 31) / 32, (f.h + 7) / 8);
    const float *src = reinterpret_cast<const float *>(r->depth), *prev = src;
    for (uint32_t k = 0; k < r->p.blur_passes; ++k) {
        float *dst = r->blur[k & 1];  // even, odd, even ... (main.cpp:430-509)
        k_ssf_blur<<<grd, blk, 0, st>>>(src, dst, f);
        ++launches;
        prev = src;
        src = dst;
    }
    k_ssf_normal<<<grd, blk, 0, st>>>(src, r->normal, f);
    k_ssf_shade<<<grd, blk, 0, st>>>(reinterpret_cast<const float *>(r->depth), r->normal, r->color, r->rgba8, f);
    launches += 2;
    CK(cudaGetLastError());
    r->blurred = src;
    r->blur_input = prev;
    r->launches = launches;
    return PBF_SUCCESS;
}

pbf_status image(pbf_ssf_renderer *r, int which, void **ptr, uint64_t *bytes)
{
    const uint64_t px = (uint64_t)r->f.w * r->f.h;
    switch (which) {
    case PBF_SSF_DEPTH: *ptr = r->depth; *bytes = 4 * px; break;
    case PBF_SSF_BLURRED: *ptr = const_cast<float *>(r->blurred); *bytes = 4 * px; break;
    case PBF_SSF_BLUR_INPUT: *ptr = const_cast<float *>(r->blur_input); *bytes = 4 * px; break;
    case PBF_SSF_NORMAL: *ptr = r->normal; *bytes = 16 * px; break;
    case PBF_SSF_COLOR: *ptr = r->color; *bytes = 16 * px; break;
    case PBF_SSF_RGBA8: *ptr = r->rgba8; *bytes = 4 * px; break;
    default: return PBF_ERROR_INVALID_ARGUMENT;
    }
    return PBF_SUCCESS;
}

void free_renderer(pbf_ssf_renderer *r)
{
    cudaSetDevice(r->device);
    cudaFree(r->depth);
    cudaFree(r->blur[0]);
    cudaFree(r->blur[1]);
    cudaFree(r->normal);
    cudaFree(r->color);
    cudaFree(r->rgba8);
    cudaFree(r->rec);
    delete r;
}

}  // namespace

extern "C" {

pbf_status pbf_ssf_params_init(pbf_ssf_params *p)
{
    if (!p) return PBF_ERROR_INVALID_ARGUMENT;
    std::memset(p, 0, sizeof(*p));
    p->width = 1280;
    p->height = 720;
    // src/common/controls.cpp:12-26 (initial state) and :66-110 (matrices)
    const float pi = 3.14159265358979323846f;
    const float h_ang = pi, v_ang = pi * -0.1f;
    const float znear = 0.1f, zfar = 50.f;
    const float dir[3] = {std::cos(v_ang) * std::sin(h_ang), std::sin(v_ang), std::cos(v_ang) * std::cos(h_ang)};
    const float right[3] = {std::sin(h_ang - 3.14f / 2.0f), 0.f, std::cos(h_ang - 3.14f / 2.0f)};
    float up[3];
    cross3(right, dir, up);
    // glm::perspective(45.0f, 4/3, near, far), fovy in radians
    const float fovy = 45.0f, aspect = 4.0f / 3.0f;
    const float tan_half = std::tan(fovy / 2.0f);
    float *P = p->projection;
    P[0] = 1.0f / (aspect * tan_half);
    P[5] = 1.0f / tan_half;
    P[10] = -(zfar + znear) / (zfar - znear);
    P[11] = -1.0f;
    P[14] = -(2.0f * zfar * znear) / (zfar - znear);
    // glm::lookAt(eye, eye + direction, up)
    const float eye[3] = {2.0f, 4.0f, 10.0f};
    const float center[3] = {eye[0] + dir[0], eye[1] + dir[1], eye[2] + dir[2]};
    float fw[3] = {center[0] - eye[0], center[1] - eye[1], center[2] - eye[2]};
    normalize3(fw);
    float sd[3];
    cross3(fw, up, sd);
    normalize3(sd);
    float u[3];
    cross3(sd, fw, u);
    float *V = p->view;
    V[0] = sd[0];
    V[4] = sd[1];
    V[8] = sd[2];
    V[1] = u[0];
    V[5] = u[1];
    V[9] = u[2];
    V[2] = -fw[0];
    V[6] = -fw[1];
    V[10] = -fw[2];
    V[12] = -(sd[0] * eye[0] + sd[1] * eye[1] + sd[2] * eye[2]);
    V[13] = -(u[0] * eye[0] + u[1] * eye[1] + u[2] * eye[2]);
    V[14] = fw[0] * eye[0] + fw[1] * eye[1] + fw[2] * eye[2];
    V[15] = 1.0f;
    p->point_radius = 0.18f;
    p->point_scale = P[5] * ((float)p->height * 0.5f);
    p->near_plane = znear;
    p->far_plane = zfar;
    p->blur_radius = 0.0000055f;
    p->blur_scale = (float)p->height / std::tan(45.f * 0.5f * 3.1415f / 180.f);
    p->blur_passes = 3;
    p->splat_mode = PBF_SSF_SPLAT_QUAD;
    p->thickness = 0.6f;
    p->clear_color[0] = p->clear_color[1] = p->clear_color[2] = 0.6f;
    p->clear_color[3] = 1.f;
    return PBF_SUCCESS;
}

pbf_status pbf_ssf_create(int device, const pbf_ssf_params *p, pbf_ssf_renderer **out)
{
    if (!p || !out) return PBF_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    if (p->width < 1 || p->height < 1 || p->width > kMaxSide || p->height > kMaxSide) return PBF_ERROR_BAD_PARAMETER;
    if (p->splat_mode > PBF_SSF_SPLAT_SPRITE || p->blur_passes > 64) return PBF_ERROR_BAD_PARAMETER;
    for (int k = 0; k < 16; ++k)
        if (!std::isfinite(p->projection[k]) || !std::isfinite(p->view[k])) return PBF_ERROR_BAD_PARAMETER;
    const float *P = p->projection;
    // x_clip on (x, z, w), y_clip on (y, z, w), z_clip and w_clip on (z, w)
    if (P[4] != 0.f || P[1] != 0.f || P[2] != 0.f || P[6] != 0.f || P[3] != 0.f || P[7] != 0.f)
        return PBF_ERROR_BAD_PARAMETER;
    if (!(p->point_radius > 0.f) || !(p->near_plane > 0.f) || !(p->far_plane > p->near_plane) ||
        !std::isfinite(p->far_plane) || !std::isfinite(p->blur_radius) || !std::isfinite(p->blur_scale) ||
        !std::isfinite(p->point_scale) || !std::isfinite(p->thickness))
        return PBF_ERROR_BAD_PARAMETER;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PBF_ERROR_NO_DEVICE;
    if (device < 0 || device >= ndev) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_ssf_renderer *r = new (std::nothrow) pbf_ssf_renderer;
    if (!r) return PBF_ERROR_OUT_OF_MEMORY;
    r->device = device;
    r->p = *p;
    Frame &f = r->f;
    f.w = p->width;
    f.h = p->height;
    f.mode = p->splat_mode;
    std::memcpy(f.proj, p->projection, sizeof f.proj);
    std::memcpy(f.view, p->view, sizeof f.view);
    if (!inverse4(f.proj, f.inv_proj)) {
        delete r;
        return PBF_ERROR_BAD_PARAMETER;
    }
    f.radius = p->point_radius;
    f.point_scale = p->point_scale;
    f.znear = p->near_plane;
    f.zfar = p->far_plane;
    f.blur_radius = p->blur_radius;
    f.blur_scale = p->blur_scale;
    f.thickness = p->thickness;
    std::memcpy(f.clear, p->clear_color, sizeof f.clear);
    f.inv_w = 1.f / (float)f.w;
    f.inv_h = 1.f / (float)f.h;
    // lightDir = View * World * vec4(1, 4, 1, 0) (ssf_shading.frag:39), normalised once
    const float4 l = mat_vec(f.view, 1.f, 4.f, 1.f, 0.f);
    float inc[3] = {l.x, l.y, l.z};
    normalize3(inc);
    std::memcpy(f.incident, inc, sizeof inc);
    const size_t px = (size_t)f.w * f.h;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&r->sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&r->depth, 4 * px);
    if (e == cudaSuccess) e = cudaMalloc(&r->blur[0], 4 * px);
    if (e == cudaSuccess) e = cudaMalloc(&r->blur[1], 4 * px);
    if (e == cudaSuccess) e = cudaMalloc(&r->normal, 16 * px);
    if (e == cudaSuccess) e = cudaMalloc(&r->color, 16 * px);
    if (e == cudaSuccess) e = cudaMalloc(&r->rgba8, 4 * px);
    if (e != cudaSuccess) {
        set_last_error("pbf_ssf_create", e);
        free_renderer(r);
        return e == cudaErrorMemoryAllocation ? PBF_ERROR_OUT_OF_MEMORY : PBF_ERROR_CUDA;
    }
    r->blurred = r->blur_input = reinterpret_cast<const float *>(r->depth);
    *out = r;
    return PBF_SUCCESS;
}

pbf_status pbf_ssf_destroy(pbf_ssf_renderer *r)
{
    if (!r) return PBF_ERROR_INVALID_ARGUMENT;
    free_renderer(r);
    return PBF_SUCCESS;
}

pbf_status pbf_ssf_render(pbf_ssf_renderer *r, const float *x_dev, uint32_t n, void *st)
{
    if (!r || (n && !x_dev)) return PBF_ERROR_INVALID_ARGUMENT;
    return launch_frame(r, x_dev, 3, nullptr, n, n, S(st));
}

pbf_status pbf_ssf_render_scene(pbf_ssf_renderer *r, pbf_batch *b, uint32_t scene_id, void *st)
{
    if (!r || !b) return PBF_ERROR_INVALID_ARGUMENT;
    Batch::SceneArrays A;
    pbf_status rc = b->b.scene_arrays(scene_id, &A);
    if (rc != PBF_SUCCESS) return rc;
    if (b->b.device() != r->device) return PBF_ERROR_INVALID_ARGUMENT;
    return launch_frame(r, reinterpret_cast<const float *>(A.x), 4, A.scene_num, 0, A.capacity, S(st));
}

pbf_status pbf_ssf_render_particles(pbf_ssf_renderer *r, pbf_handle *h, void *st)
{
    if (!r || !h) return PBF_ERROR_INVALID_ARGUMENT;
    Batch::SceneArrays A;
    pbf_status rc = h->b.scene_arrays(h->scene, &A);
    if (rc != PBF_SUCCESS) return rc;
    if (h->b.device() != r->device) return PBF_ERROR_INVALID_ARGUMENT;
    return launch_frame(r, reinterpret_cast<const float *>(A.x), 4, A.scene_num, 0, A.capacity, S(st));
}

pbf_status pbf_ssf_image_device(pbf_ssf_renderer *r, int which, void **ptr, uint64_t *bytes)
{
    if (!r || !ptr || !bytes) return PBF_ERROR_INVALID_ARGUMENT;
    return image(r, which, ptr, bytes);
}

pbf_status pbf_ssf_get_image(pbf_ssf_renderer *r, int which, void *dst, int dst_dev, void *st)
{
    if (!r || !dst) return PBF_ERROR_INVALID_ARGUMENT;
    void *src = nullptr;
    uint64_t bytes = 0;
    pbf_status rc = image(r, which, &src, &bytes);
    if (rc != PBF_SUCCESS) return rc;
    CK(cudaSetDevice(r->device));
    CK(cudaMemcpyAsync(dst, src, bytes, dst_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, S(st)));
    if (!dst_dev) CK(cudaStreamSynchronize(S(st)));
    return PBF_SUCCESS;
}

pbf_status pbf_ssf_frame_constants(const pbf_ssf_renderer *r, float inv_projection[16], float incident[3])
{
    if (!r) return PBF_ERROR_INVALID_ARGUMENT;
    if (inv_projection) std::memcpy(inv_projection, r->f.inv_proj, sizeof r->f.inv_proj);
    if (incident) std::memcpy(incident, r->f.incident, sizeof r->f.incident);
    return PBF_SUCCESS;
}

pbf_status pbf_ssf_last_launches(const pbf_ssf_renderer *r, uint32_t *n)
{
    if (!r || !n) return PBF_ERROR_INVALID_ARGUMENT;
    *n = r->launches;
    return PBF_SUCCESS;
}

}  // extern "C"
