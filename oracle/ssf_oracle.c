/* CPU restatement of the reference's screen-space fluid passes — TEST
 * INFRASTRUCTURE ONLY (the checker of the CUDA renderer; nothing in the
 * product links it).
 *
 * Follows, pass by pass, the GLSL the reference runs each frame
 * (yodaplusplus/ssf_pbf_cuda, cuda_pbf_with_ssf/src/main.cpp:372-564):
 *   depth splat   asset/shader/ssf_object.vert:13-17, ssf_object.geom:19-52,
 *                 ssf_object.frag:18-35 (quad) and ssf_point_sprite.vert:19-27,
 *                 ssf_point_sprite.frag:17-31 (sprite);
 *   blur          asset/shader/ssf_blur.frag:27-139;
 *   normals       asset/shader/ssf_normal.frag:17-36;
 *   shading       asset/shader/ssf_shading.frag:23-83, blended onto the
 *                 clear colour (main.cpp:76, 541-564).
 * Fixed-function steps are written as the GL specification states them:
 * viewport transform, pixel-centre coverage (tex_coord of pixel i taken as
 * (i + 0.5) * (1 / width)), point-sprite coordinates with
 * the upper-left origin, LINEAR + CLAMP_TO_EDGE filtering (weights with 8
 * fractional bits, as a texture unit keeps them), gl_FragDepth clamped to
 * [0, 1] and tested GL_LESS against the cleared 1.0, fine 2x2-quad
 * derivatives, and blending into a fixed-point colour buffer.
 *
 * Parity is unpinned against the reference itself: its passes run only
 * through OpenGL, which this project does not use.  Every product and sum
 * is rounded on its own (built with -ffp-contract=off) in the order the
 * CUDA kernels use, so splat and normals must agree bit for bit and blur
 * and shading within the error of expf / powf.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct OraSsf {
    uint32_t w, h, mode, pad;
    float proj[16], view[16], inv_proj[16];
    float radius, point_scale, znear, zfar;
    float blur_radius, blur_scale, thickness, pad1;
    float clear[4];
    float incident[3];
} OraSsf;

typedef struct { float x, y, z, w; } v4;

static v4 mv(const float *m, float x, float y, float z, float w)
{
    v4 r;
    r.x = m[0] * x + m[4] * y + m[8] * z + m[12] * w;
    r.y = m[1] * x + m[5] * y + m[9] * z + m[13] * w;
    r.z = m[2] * x + m[6] * y + m[10] * z + m[14] * w;
    r.w = m[3] * x + m[7] * y + m[11] * z + m[15] * w;
    return r;
}

static float dot3(float ax, float ay, float az, float bx, float by, float bz) { return ax * bx + ay * by + az * bz; }

static int clamp_pix(float v, uint32_t n)
{
    v = fminf(fmaxf(v, -1.f), (float)n);
    return (int)v;
}

static int mini(int a, int b) { return a < b ? a : b; }
static int maxi(int a, int b) { return a > b ? a : b; }

/* ---- depth splat ---- */

/* Window rectangle of covered pixel centres and the values the fragments
 * of one particle share; 0 = nothing of it reaches the image. */
typedef struct {
    float x0, x1, y0, y1, ax, ay, dx, by, ex, ey, ez;
    float rx, ry; /* 1 / window width, height of the quad; sprite: 1 / size */
    int i0, j0, i1, j1;
} Footprint;

static int footprint(const OraSsf *f, float px, float py, float pz, Footprint *s)
{
    /* ssf_object.vert:15-16: vw * vec4(Position, 1), World = identity */
    v4 e = mv(f->view, px, py, pz, 1.f);
    float hw = (float)f->w * 0.5f, hh = (float)f->h * 0.5f;
    s->ex = e.x;
    s->ey = e.y;
    s->ez = e.z;
    if (f->mode == 0) {
        /* ssf_object.geom:21-50: quad P.xy +- 0.5 point_radius at P.zw;
         * window rectangle from the viewport transform of corners a, d, b */
        float hr = 0.5f * f->radius;
        s->ax = e.x - hr;
        s->ay = e.y - hr;
        s->dx = e.x + hr;
        s->by = e.y + hr;
        v4 ca = mv(f->proj, s->ax, s->ay, e.z, e.w);
        v4 cd = mv(f->proj, s->dx, s->ay, e.z, e.w);
        v4 cb = mv(f->proj, s->ax, s->by, e.z, e.w);
        if (!(-ca.w <= ca.z && ca.z <= ca.w)) return 0; /* near / far clipping */
        s->x0 = ca.x / ca.w * hw + hw;
        s->x1 = cd.x / cd.w * hw + hw;
        s->y0 = ca.y / ca.w * hh + hh;
        s->y1 = cb.y / cb.w * hh + hh;
        if (!(s->x1 > s->x0 && s->y1 > s->y0)) return 0; /* back face culled */
        s->rx = 1.f / (s->x1 - s->x0);
        s->ry = 1.f / (s->y1 - s->y0);
    } else {
        /* ssf_point_sprite.vert:20-26 */
        float dist = sqrtf(dot3(e.x, e.y, e.z, e.x, e.y, e.z));
        float size = f->radius * (f->point_scale / dist);
        v4 c = mv(f->proj, e.x, e.y, e.z, 1.f);
        if (!(-c.w <= c.x && c.x <= c.w && -c.w <= c.y && c.y <= c.w && -c.w <= c.z && c.z <= c.w)) return 0;
        if (!(size > 0.f)) return 0;
        float xw = c.x / c.w * hw + hw, yw = c.y / c.w * hh + hh, half = size * 0.5f;
        s->x0 = xw - half;
        s->x1 = xw + half;
        s->y0 = yw - half;
        s->y1 = yw + half;
        s->ax = xw;
        s->ay = yw;
        s->dx = size;
        s->by = 0.f;
        s->rx = s->ry = 1.f / size;
    }
    s->i0 = maxi(clamp_pix(floorf(s->x0 - 0.5f), f->w), 0);
    s->j0 = maxi(clamp_pix(floorf(s->y0 - 0.5f), f->h), 0);
    s->i1 = mini(clamp_pix(floorf(s->x1 - 0.5f) + 1.f, f->w), (int)f->w - 1);
    s->j1 = mini(clamp_pix(floorf(s->y1 - 0.5f) + 1.f, f->h), (int)f->h - 1);
    return s->i1 >= s->i0 && s->j1 >= s->j0;
}

/* ssf_object.frag:20-33 / ssf_point_sprite.frag:19-29; < 0: no fragment */
static float fragment(const OraSsf *f, const Footprint *s, int i, int j)
{
    float cx = (float)i + 0.5f, cy = (float)j + 0.5f;
    if (!(cx >= s->x0 && cx < s->x1 && cy >= s->y0 && cy < s->y1)) return -1.f;
    float nx, ny, px, py, pz;
    if (f->mode == 0) {
        /* vertex_uv: screen-space interpolation over the quad (w is constant
         * on it), as (c - corner) * (1 / extent) */
        float u = (cx - s->x0) * s->rx, v = (cy - s->y0) * s->ry;
        nx = u * 2.f - 1.f; /* vertex_uv * 2 - 1 */
        ny = v * 2.f - 1.f;
        px = s->ax + u * (s->dx - s->ax); /* pos_from_eye, interpolated */
        py = s->ay + v * (s->by - s->ay);
    } else {
        float sc = 0.5f + (cx - s->ax) * s->rx, tc = 0.5f - (cy - s->ay) * s->ry; /* gl_PointCoord */
        nx = sc * 2.f + -1.f;
        ny = tc * -2.f + 1.f;
        px = s->ex;
        py = s->ey;
    }
    float mag = nx * nx + ny * ny;
    if (mag > 1.f) return -1.f;
    float nz = sqrtf(1.f - mag);
    px = px + nx * f->radius;
    py = py + ny * f->radius;
    pz = s->ez + nz * f->radius;
    float cz = f->proj[2] * px + f->proj[6] * py + f->proj[10] * pz + f->proj[14];
    float cw = f->proj[3] * px + f->proj[7] * py + f->proj[11] * pz + f->proj[15];
    float d = cz / cw;
    if (d != d) return -1.f;
    return fminf(fmaxf(d, 0.f), 1.f) + 0.f; /* clamped to the depth range, -0 as +0 */
}

/* depth[h][w]: cleared to 1, then the nearest fragment of every particle.
 * x: n positions, stride floats apart (3 = AoS float3, 4 = float4). */
void ora_ssf_splat(const OraSsf *f, const float *x, uint32_t n, int stride, float *depth)
{
    size_t px = (size_t)f->w * f->h;
    for (size_t k = 0; k < px; ++k) depth[k] = 1.f;
    for (uint32_t p = 0; p < n; ++p) {
        const float *xp = x + (size_t)p * stride;
        Footprint s;
        if (!footprint(f, xp[0], xp[1], xp[2], &s)) continue;
        for (int j = s.j0; j <= s.j1; ++j)
            for (int i = s.i0; i <= s.i1; ++i) {
                float d = fragment(f, &s, i, j);
                if (d >= 0.f && d < depth[(size_t)j * f->w + i]) depth[(size_t)j * f->w + i] = d;
            }
    }
}

/* ---- screen passes ---- */

static float sample(const float *T, uint32_t W, uint32_t H, float s, float t)
{
    float u = s * (float)W - 0.5f, v = t * (float)H - 0.5f;
    float fu = floorf(u), fv = floorf(v);
    float a = rintf((u - fu) * 256.f) * (1.f / 256.f), b = rintf((v - fv) * 256.f) * (1.f / 256.f);
    int iu = clamp_pix(fu, W), iv = clamp_pix(fv, H);
    int i0 = mini(maxi(iu, 0), (int)W - 1), i1 = mini(maxi(iu + 1, 0), (int)W - 1);
    int j0 = mini(maxi(iv, 0), (int)H - 1), j1 = mini(maxi(iv + 1, 0), (int)H - 1);
    float t00 = T[(size_t)j0 * W + i0], t10 = T[(size_t)j0 * W + i1];
    float t01 = T[(size_t)j1 * W + i0], t11 = T[(size_t)j1 * W + i1];
    float a1 = 1.f - a, b1 = 1.f - b;
    return (a1 * b1) * t00 + (a * b1) * t10 + (a1 * b) * t01 + (a * b) * t11;
}

static float linearize(float d, const OraSsf *f) { return (2.f * f->znear) / (f->zfar + f->znear - d * (f->zfar - f->znear)); }

static float exponentialize(float l, const OraSsf *f)
{
    return (f->zfar + f->znear - (2.f * f->znear) / l) / (f->zfar - f->znear);
}

static void uv_to_eye(const OraSsf *f, float s, float t, float d, int flip, float out[3])
{
    float x = s * 2.f - 1.f;
    float y = flip ? t * -2.f + 1.f : t * 2.f - 1.f;
    v4 c = mv(f->inv_proj, x, y, d, 1.f);
    out[0] = c.x / c.w;
    out[1] = c.y / c.w;
    out[2] = c.z / c.w;
}

static float depth_store(float v)
{
    if (v != v) return 1.f;
    return fminf(fmaxf(v, 0.f), 1.f);
}

/* One blur pass (ssf_blur.frag:44-139) of in[h][w] into out[h][w]. */
void ora_ssf_blur(const OraSsf *f, const float *in, float *out)
{
    for (uint32_t j = 0; j < f->h; ++j)
        for (uint32_t i = 0; i < f->w; ++i) {
            float s = ((float)i + 0.5f) * (1.f / (float)f->w), t = ((float)j + 0.5f) * (1.f / (float)f->h);
            float ed = sample(in, f->w, f->h, s, t);
            if (ed == 1.f) {
                out[(size_t)j * f->w + i] = 1.f;
                continue;
            }
            float lin = linearize(ed, f);
            float p[3];
            uv_to_eye(f, s, t, ed, 1, p);
            float dist = sqrtf(dot3(p[0], p[1], p[2], p[0], p[1], p[2]));
            float br = f->blur_radius * f->blur_scale / dist;
            float sum = 0.f, wsum = 0.f;
            for (int axis = 0; axis < 2; ++axis)
                for (int k = -4; k < 4; ++k) {
                    float sd = axis == 0 ? sample(in, f->w, f->h, s + (float)k * br, t)
                                         : sample(in, f->w, f->h, s, t + (float)k * br);
                    if (sd != 1.f) {
                        float sl = linearize(sd, f);
                        float r = (float)(k * k) * br;
                        float w = expf(-r);
                        float diff = sl - lin;
                        float r2 = fabsf(diff) < 0.01f ? diff * 100.f : 0.f;
                        float g = expf(-r2 * r2);
                        sum = sum + sl * w * g;
                        wsum = wsum + w * g;
                    }
                }
            if (wsum > 0.f) sum = sum / wsum;
            out[(size_t)j * f->w + i] = depth_store(exponentialize(sum, f));
        }
}

static void eye_at(const OraSsf *f, const float *D, int i, int j, float out[3])
{
    int ic = mini(maxi(i, 0), (int)f->w - 1), jc = mini(maxi(j, 0), (int)f->h - 1);
    float s = ((float)i + 0.5f) * (1.f / (float)f->w), t = ((float)j + 0.5f) * (1.f / (float)f->h);
    uv_to_eye(f, s, t, D[(size_t)jc * f->w + ic], 0, out);
}

/* normal4[h][w][4] from depth[h][w] (ssf_normal.frag:25-36). */
void ora_ssf_normal(const OraSsf *f, const float *D, float *N)
{
    for (uint32_t j = 0; j < f->h; ++j)
        for (uint32_t i = 0; i < f->w; ++i) {
            float *o = N + 4 * ((size_t)j * f->w + i);
            if (D[(size_t)j * f->w + i] == 1.f) {
                memcpy(o, f->clear, sizeof f->clear);
                continue;
            }
            int ie = (int)(i & ~1u), je = (int)(j & ~1u);
            float px0[3], px1[3], py0[3], py1[3];
            eye_at(f, D, ie, (int)j, px0);
            eye_at(f, D, ie + 1, (int)j, px1);
            eye_at(f, D, (int)i, je, py0);
            eye_at(f, D, (int)i, je + 1, py1);
            float dxx = px1[0] - px0[0], dxy = px1[1] - px0[1], dxz = px1[2] - px0[2];
            float dyx = py1[0] - py0[0], dyy = py1[1] - py0[1], dyz = py1[2] - py0[2];
            float cx = dxy * dyz - dyy * dxz, cy = dxz * dyx - dyz * dxx, cz = dxx * dyy - dyx * dxy;
            float inv = 1.f / sqrtf(dot3(cx, cy, cz, cx, cy, cz));
            o[0] = cx * inv;
            o[1] = cy * inv;
            o[2] = cz * inv;
            o[3] = 1.f;
        }
}

static float clamp01(float v) { return fminf(fmaxf(v, 0.f), 1.f); }

/* color4[h][w][4] and rgba8[h][w][4] from the unblurred depth and the
 * normals (ssf_shading.frag:36-83, blended onto the clear colour). */
void ora_ssf_shade(const OraSsf *f, const float *D, const float *N, float *C, uint8_t *C8)
{
    for (uint32_t j = 0; j < f->h; ++j)
        for (uint32_t i = 0; i < f->w; ++i) {
            size_t o = (size_t)j * f->w + i;
            float ed = D[o];
            float out[4];
            if (ed == 1.f) {
                memcpy(out, f->clear, sizeof out);
            } else {
                const float *n = N + 4 * o;
                float th = clamp01(f->thickness);
                float s = ((float)i + 0.5f) * (1.f / (float)f->w), t = ((float)j + 0.5f) * (1.f / (float)f->h);
                float p[3];
                uv_to_eye(f, s, t, ed, 1, p);
                float il = f->incident[0], jl = f->incident[1], kl = f->incident[2];
                float vr = 1.f / sqrtf(dot3(-p[0], -p[1], -p[2], -p[0], -p[1], -p[2]));
                float vx = -p[0] * vr, vy = -p[1] * vr, vz = -p[2] * vr;
                float hx = il + vx, hy = jl + vy, hz = kl + vz;
                float hr = 1.f / sqrtf(dot3(hx, hy, hz, hx, hy, hz));
                float specular = powf(fmaxf(0.f, dot3(hx * hr, hy * hr, hz * hr, n[0], n[1], n[2])), 50.f);
                float diffuse = fmaxf(0.f, dot3(il, jl, kl, n[0], n[1], n[2]));
                float r0 = 0.3f;
                float fres = r0 + (1.f - r0) * powf(1.f - dot3(n[0], n[1], n[2], vx, vy, vz), 5.f);
                float ar = expf(-5.f * th), ag = expf(-1.f * th), ab = expf(-0.1f * th);
                float a = th, ia = 1.f - a;
                out[0] = clamp01(clamp01(ar * diffuse + specular * 1.f + 1.f * fres) * a + f->clear[0] * ia);
                out[1] = clamp01(clamp01(ag * diffuse + specular * 1.f + 1.f * fres) * a + f->clear[1] * ia);
                out[2] = clamp01(clamp01(ab * diffuse + specular * 1.f + 1.f * fres) * a + f->clear[2] * ia);
                out[3] = clamp01(a * a + f->clear[3] * ia);
            }
            for (int c = 0; c < 4; ++c) {
                C[4 * o + c] = out[c];
                C8[4 * o + c] = (uint8_t)rintf(clamp01(out[c]) * 255.f);
            }
        }
}
