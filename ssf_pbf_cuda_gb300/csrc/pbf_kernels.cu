// Device kernels of the PBF solver step (sm_103a).
//
// One thread per particle; blocks walk a device-resident tile list in a
// grid-stride loop, each tile belonging to one scene, so the same kernels run
// a single scene (the plain step) or hundreds of scenes (the batched engine)
// with a fixed launch shape that a CUDA graph can capture once.
//
// Data layout (flat arrays over every scene's particle slots):
//   x, v, xs, xa, xb, xold, w, vt : float4 (xyz + unused w), 16-byte aligned
//   key, slot, tmp, perm          : uint32 per particle
//   nbr                           : uint32 [slot k][particle i] (coalesced per k)
//   count / offsets               : uint32 per cell (+1 deleted bucket per scene)
//
// Integer work (predict, cell hash, stable counting sort, neighbour
// acceptance) uses explicitly rounded intrinsics so that it is bit-exact
// against the CPU oracle.  Floating-point solver math follows the reference's
// operation order but uses rsqrtf (as the reference does).
#include <map>
#include <mutex>
#include <tuple>

#include "pbf_internal.h"
#include "pbf_sort.cuh"
#include "pbf103.h"

namespace pbf103 {
namespace {

// ---------------------------------------------------------------- helpers --

// static_cast<int>(floor(p / cell_width)), src/pbf/interaction/cuda/pbf_grid.h:20-33,
// with IEEE division (the reference build used -prec-div=false).
__device__ __forceinline__ int32_t cell_coord(float p, float cw)
{
    return __float2int_rd(__fdiv_rn(p, cw));
}

// calcGridHash with power-of-two wrap, pbf_grid.h:53-61.
__device__ __forceinline__ uint32_t hash3(uint32_t x, uint32_t y, uint32_t z, const SceneDesc &d)
{
    x &= d.gx - 1u;
    y &= d.gy - 1u;
    z &= d.gz - 1u;
    return z * d.gx * d.gy + y * d.gx + x;
}

// Alias class of a cell: which of the 2 x 2 x 2 periodic copies of the
// power-of-two table the (unwrapped) cell lies in.  With the table sized for
// cells of 2h (calcGridSize, pbf_type.cpp:141-162) but cells h wide, a
// bucket holds particles of cells G apart; only one class of a bucket can
// hold neighbours of a given cell.  Cells 2G apart share a class; they are
// far apart, so the distance test still rejects them.
__device__ __forceinline__ uint32_t alias_class(int32_t cx, int32_t cy, int32_t cz, const SceneDesc &d)
{
    const int sx = __ffs(d.gx) - 1, sy = __ffs(d.gy) - 1, sz = __ffs(d.gz) - 1;
    return (uint32_t)(((cz >> sz) & 1) << 2 | ((cy >> sy) & 1) << 1 | ((cx >> sx) & 1));
}

// Packed FP32 (two lanes of one 64-bit register pair per instruction):
// each lane is rounded exactly as the scalar operation (flush-to-zero like
// the rest of the build), so a pair of x and y terms costs one instruction
// and gives the scalar bits.
__device__ __forceinline__ void sub2(float &d0, float &d1, float a0, float a1, float b0, float b1)
{
    asm("{\n\t.reg .b64 pa, pb, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\t"
        "mov.b64 pb, {%4, %5};\n\t"
        "sub.rn.ftz.f32x2 pd, pa, pb;\n\t"
        "mov.b64 {%0, %1}, pd;\n\t}"
        : "=f"(d0), "=f"(d1)
        : "f"(a0), "f"(a1), "f"(b0), "f"(b1));
}

// c0 = fma(a0, b0, c0), c1 = fma(a1, b1, c1)
__device__ __forceinline__ void fma2(float &c0, float &c1, float a0, float a1, float b0, float b1)
{
    asm("{\n\t.reg .b64 pa, pb, pc;\n\t"
        "mov.b64 pa, {%2, %3};\n\t"
        "mov.b64 pb, {%4, %5};\n\t"
        "mov.b64 pc, {%0, %1};\n\t"
        "fma.rn.ftz.f32x2 pc, pa, pb, pc;\n\t"
        "mov.b64 {%0, %1}, pc;\n\t}"
        : "+f"(c0), "+f"(c1)
        : "f"(a0), "f"(a1), "f"(b0), "f"(b1));
}

// One 32-byte record (two float4) by one 256-bit load through the
// read-only path; p must be 32-byte aligned.
__device__ __forceinline__ void ld_rec(const float4 *p, float4 &a, float4 &b)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// r^2 exactly as findPair computes it (pbf_neighbor_search_util.cu:398):
// fmaf(dz, dz, fmaf(dy, dy, dx * dx)), no further contraction.
__device__ __forceinline__ float dist2_exact(float4 a, float4 b)
{
    float d0, d1;
    sub2(d0, d1, a.x, a.y, b.x, b.y);
    const float d2 = __fsub_rn(a.z, b.z);
    return __fmaf_rn(d2, d2, __fmaf_rn(d1, d1, __fmul_rn(d0, d0)));
}

// A listed pair at current positions (memorizeKernelPair,
// src/pbf/solver/cuda/pbf_kernel_memorization.cu:14-56, restated): the
// difference d = x_i - x_j, r^2, the poly6 value W = alpha w and the spiky
// gradient grad W = beta s d, with the scene factors alpha and beta left
// out of the per-pair terms (the sums apply them once per particle):
//   w = (1 - r^2 / h^2)^3                for r <= h, else 0
//   s = (1 - r / h)^2 / r                for 0 < r <= h, else 0
//   sr = s r = |grad W| / |beta|
// The clamps replace the reference's branches: 1 - r^2/h^2 and 1 - r/h are
// clamped at 0 (r > h), and r^2 enters the reciprocal square root no smaller
// than kMinR2, so a pair at distance 0 (d = 0, r = 0) gets a finite s (up
// to 1e15), a gradient s d of exactly 0 and sr = 0, as the reference's
// r^2 > 0 test gives.  |grad W|^2 is taken as sr^2, not s^2 r^2: the
// latter overflows at r = 0.
// Products and sums are rounded one by one or fused where written
// (__fmaf_rn), never contracted by the compiler, so every pass that calls
// these, in one lane or split over lanes, gets the same bits.
constexpr float kMinR2 = 1e-30f;

struct PairGeo {
    float d0, d1, d2, r2;
};

// PK: d0 and d1 by one packed subtraction (the same bits; faster in the
// delta-p pass of large steps, slower in the small steps' passes: measured)
template <bool PK = false>
__device__ __forceinline__ PairGeo pair_geo(float4 xi, float4 xj)
{
    PairGeo g;
    if (PK) {
        sub2(g.d0, g.d1, xi.x, xi.y, xj.x, xj.y);
    } else {
        g.d0 = __fsub_rn(xi.x, xj.x);
        g.d1 = __fsub_rn(xi.y, xj.y);
    }
    g.d2 = __fsub_rn(xi.z, xj.z);
    g.r2 = __fmaf_rn(g.d2, g.d2, __fmaf_rn(g.d1, g.d1, __fmul_rn(g.d0, g.d0)));
    return g;
}

struct PairWS {
    float W, s, sr;
};

// per-scene constants of the pair math, in registers for a particle's loop
struct PairConst {
    float ih2, inv_h;
};

__device__ __forceinline__ PairConst pair_const(const SceneDesc &d) { return PairConst{d.ih2, d.inv_h}; }

__device__ __forceinline__ PairWS pair_ws(float r2, const PairConst &c)
{
    const float inv_r = rsqrtf(fmaxf(r2, kMinR2));
    const float t = fmaxf(__fmaf_rn(-r2, c.ih2, 1.f), 0.f);
    const float W = __fmul_rn(__fmul_rn(t, t), t);
    const float r = __fmul_rn(r2, inv_r);
    const float u = fmaxf(__fmaf_rn(-r, c.inv_h, 1.f), 0.f);
    const float s = __fmul_rn(inv_r, __fmul_rn(u, u));
    return PairWS{W, s, __fmul_rn(s, r)};
}

// The sums of calcScalingFactorCUDA (pbf_constraint.cu:168-209) over a
// particle's list, added in list order, without the factors alpha and
// beta: sum w (W = alpha w), sum s d (grad W = beta s d) and sum (s r)^2.
// A particle's own pair (w = 1, no gradient) is not stored in its list; the
// passes start ks at 1 for it.
struct LamSum {
    float ks = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f, kg2 = 0.f;
    __device__ __forceinline__ void add(float W, float s, float d0, float d1, float d2, float sr)
    {
        ks = __fadd_rn(ks, W);
        g0 = __fmaf_rn(s, d0, g0);
        g1 = __fmaf_rn(s, d1, g1);
        g2 = __fmaf_rn(s, d2, g2);
        kg2 = __fmaf_rn(sr, sr, kg2);
    }
    __device__ __forceinline__ void add(const PairGeo &g, const PairWS &k) { add(k.W, k.s, g.d0, g.d1, g.d2, k.sr); }
    // lambda = C / (m^2 / rho0^2 |grad C|^2 + eps), with C = alpha m / rho0
    // sum w - 1 and m^2 / rho0^2 |grad C|^2 = m^2 beta^2 / rho0^2 K
    __device__ __forceinline__ float lambda(const SceneDesc &d) const
    {
        const float C = __fmaf_rn(ks, d.lam_c, -1.f);
        const float K = __fmaf_rn(g0, g0, __fmaf_rn(g2, g2, __fmaf_rn(g1, g1, kg2)));
        return __fdiv_rn(C, __fmaf_rn(d.lam_k, K, d.relax));
    }
};

// one listed pair's terms of the lambda sums
__device__ __forceinline__ void lam_add(LamSum &ls, float4 xi, float4 xj, const PairConst &c)
{
    const PairGeo g = pair_geo(xi, xj);
    ls.add(g, pair_ws(g.r2, c));
}

// WspikyDerivative, src/pbf/kernel/cuda/detail/pbf_kernel.inl:48-63.
__device__ __forceinline__ float wspiky_d(float r, float kinv_h)
{
    const float q = r * kinv_h;
    if (q <= 1.f) {
        const float ih2 = kinv_h * kinv_h;
        const float t = 1.f - q;
        return -14.3239448745f * (ih2 * ih2) * t * t;
    }
    return 0.f;
}

// responseInnerSphereBoundary, src/pbf/solver/cuda/boundary/pbf_sphere_boundary.cu:8-34
__device__ __forceinline__ void inner_sphere(bool &hit, float3 &dp, float3 p, float4 s)
{
    const float c0 = s.x - p.x, c1 = s.y - p.y, c2 = s.z - p.z;
    const float d2 = fmaf(c2, c2, fmaf(c1, c1, c0 * c0));
    if (d2 > s.w * s.w) {
        const float rinv = rsqrtf(d2);
        hit = true;
        dp.x = fmaf(c0, 1.0001f, dp.x);
        dp.y = fmaf(c1, 1.0001f, dp.y);
        dp.z = fmaf(c2, 1.0001f, dp.z);
        dp.x = fmaf(-s.w, c0 * rinv, dp.x);
        dp.y = fmaf(-s.w, c1 * rinv, dp.y);
        dp.z = fmaf(-s.w, c2 * rinv, dp.z);
    }
}

// responsePlaneBoundary, src/pbf/solver/cuda/boundary/pbf_plane_boundary.cu:6-45.
// Both of its hit cases need the projected point p behind the plane
// ((p - on) . n < 0); that is tested first, so a particle clear of the plane
// (the common case) skips the rest, with the same result.
__device__ __forceinline__ void plane(bool &hit, float3 &dp, float3 o, float3 p, float4 on, float4 n)
{
    const float pb0 = p.x - on.x, pb1 = p.y - on.y, pb2 = p.z - on.z;
    const float pb_n = fmaf(pb2, n.z, fmaf(pb1, n.y, pb0 * n.x));
    if (!(pb_n < 0.f)) return;
    const float pa0 = o.x - on.x, pa1 = o.y - on.y, pa2 = o.z - on.z;
    const float pa_n = fmaf(pa2, n.z, fmaf(pa1, n.y, pa0 * n.x));
    float3 is;
    if (pa_n == 0.f && pb_n == 0.f) {
        return;
    } else if (pa_n >= 0.f && pb_n < 0.f) {
        hit = true;
        const float f = fabsf(pa_n) / (fabsf(pa_n) + fabsf(pb_n));
        is.x = o.x + (p.x - o.x) * f;
        is.y = o.y + (p.y - o.y) * f;
        is.z = o.z + (p.z - o.z) * f;
    } else if (pa_n < 0.f && pb_n < 0.f) {
        hit = true;
        const float dd = -fmaf(on.z, n.z, fmaf(on.y, n.y, on.x * n.x));
        const float t = -(fmaf(p.z, n.z, fmaf(p.y, n.y, p.x * n.x)) + dd) / fmaf(n.z, n.z, fmaf(n.y, n.y, n.x * n.x));
        is.x = p.x + t * n.x;
        is.y = p.y + t * n.y;
        is.z = p.z + t * n.z;
    } else {
        return;
    }
    const float di0 = p.x - is.x, di1 = p.y - is.y, di2 = p.z - is.z;
    const float c = fmaf(di2, n.z, fmaf(di1, n.y, di0 * n.x));
    dp.x += -c * n.x;
    dp.y += -c * n.y;
    dp.z += -c * n.z;
}

// responseCollisionCUDA, src/pbf/solver/cuda/pbf_response_collision.cu:12-66 (and the
// fixed-sphere variant, pbf_constraint.cu:262-315).  old_x is the current
// position, as in the reference (pbf_response_collision.cu:31).  The
// reference repeats until no primitive reports a hit; here at most max_coll
// passes.  Returns false when the bound was reached.  A pass is a function
// of dp alone, so a pass that hits but leaves dp bit-for-bit unchanged (a
// projection too small to move the position, which the reference would
// repeat forever) would repeat identically up to the bound: the loop stops
// there with the same dp and the same result.
__device__ bool collide(const SceneDesc &d, const float4 *__restrict__ bnd, float3 x, float3 &dp)
{
    if (d.clear_box) {  // a box's walls: a position inside the clear box hits none, so pass 1 is the last
        const float px = x.x + dp.x, py = x.y + dp.y, pz = x.z + dp.z;
        if (d.box_lo[0] <= px && px <= d.box_hi[0] && d.box_lo[1] <= py && py <= d.box_hi[1] &&
            d.box_lo[2] <= pz && pz <= d.box_hi[2])
            return true;
    }
    for (uint32_t pass = 0; pass < d.max_coll; ++pass) {
        const float3 before = dp;
        float3 p = make_float3(x.x + dp.x, x.y + dp.y, x.z + dp.z);
        bool hit = false;
        if (d.builtin_sphere) {
            inner_sphere(hit, dp, p, make_float4(3.f, 3.f, 3.f, 3.f));
        } else {
            const float4 *b = bnd + d.b_off;
            const uint32_t ns = d.n_inner + d.n_outer;  // outer spheres use the inner routine
            for (uint32_t k = 0; k < ns; ++k) {
                inner_sphere(hit, dp, p, __ldg(b + k));
                p = make_float3(x.x + dp.x, x.y + dp.y, x.z + dp.z);
            }
            b += ns;
            for (uint32_t k = 0; k < d.n_planes; ++k) {
                plane(hit, dp, x, p, __ldg(b + 2 * k), __ldg(b + 2 * k + 1));
                p = make_float3(x.x + dp.x, x.y + dp.y, x.z + dp.z);
            }
        }
        if (!hit) return true;
        if (__float_as_uint(dp.x) == __float_as_uint(before.x) && __float_as_uint(dp.y) == __float_as_uint(before.y) &&
            __float_as_uint(dp.z) == __float_as_uint(before.z))
            return false;  // fixed point: every later pass repeats this one
    }
    return false;
}

// Visit the particles of the 27 cells around xp in the reference's order
// (z, y, x from -1 to 1; ascending sorted index inside a cell,
// pbf_neighbor_search_util.cu:428-452), as contiguous sorted-index ranges:
// r(st, en) gets [st, en) and returns false to stop the walk.  When the
// three x-cells of a row are consecutive hashes their particles form one
// range.  Every cell is visited (the reference-form XSPH and vorticity
// walks); with fewer than 3 cells on an axis a wrapped cell is visited more
// than once, as in the reference.
template <class R>
__device__ __forceinline__ void walk27_ranges(const SceneDesc &d, const uint32_t *__restrict__ offsets,
                                              uint32_t shift, float4 xp, R &&r)
{
    const uint32_t gx = (uint32_t)cell_coord(xp.x, d.cw), gy = (uint32_t)cell_coord(xp.y, d.cw),
                   gz = (uint32_t)cell_coord(xp.z, d.cw);
    const uint32_t *off = offsets + d.c_off;
    const uint32_t mx = d.gx - 1u;
    const uint32_t x0c = (gx - 1u) & mx, x2c = (gx + 1u) & mx;
    const bool contiguous = (x2c == x0c + 2u);
#pragma unroll 1
    for (int rr = 0; rr < 9; ++rr) {
        const int dz = rr / 3 - 1, dy = rr % 3 - 1;
        const uint32_t row = ((gz + (uint32_t)dz) & (d.gz - 1u)) * d.gx * d.gy +
                             ((gy + (uint32_t)dy) & (d.gy - 1u)) * d.gx;
        const uint32_t nseg = contiguous ? 1u : 3u;
#pragma unroll 1
        for (uint32_t sg = 0; sg < nseg; ++sg) {
            const uint32_t lo = contiguous ? x0c : (gx + sg - 1u) & mx;
            const uint32_t hi = contiguous ? x2c : lo;
            if (!r(__ldg(off + row + lo) + shift, __ldg(off + row + hi + 1u) + shift)) return;
        }
    }
}

// The neighbour-search walk: the same 27 cells in the same order as
// walk27_ranges, one range per cell, and inside a cell's bucket only the
// particles of the cell's alias class (chist holds the bucket's class
// counts): a bucket of one class is the sorted range itself (xa), a bucket
// without the class is skipped, and a mixed bucket gives the class's
// sub-range of the class-grouped walk copy (wx).  Candidates of the other
// classes lie at least G - 1 cells away and can never be accepted, and both
// arrays keep each class in sorted order with the sorted slot in .w, so the
// accepted sequence is the reference's.  Buckets marked kClassWhole (and
// every bucket of a scene with an axis of fewer than 4 cells, where the
// reference visits wrapped cells twice) are visited whole, in sorted order.
// r(src, st, en) gets the array and the range.
//
// PRUNE restricts the walk to cells that can hold a particle within h of xp
// (the binned position): a cell whose nearest point is farther than h holds
// no accepted candidate, so skipping it leaves the visited sequence of
// accepted candidates unchanged.  A 1e-3 relative margin covers the rounding
// of the cell assignment.  It applies only when every axis has at least 4
// cells (with fewer, the reference visits wrapped cells more than once).
template <bool PRUNE, class R>
__device__ __forceinline__ void walk27_cells(const SceneDesc &d, const uint32_t *__restrict__ offsets,
                                             const uint64_t *__restrict__ chist, const float4 *xa,
                                             const float4 *wx, uint32_t shift, float4 xp, R &&r, int rr0 = 0,
                                             int rr1 = 9)
{
    const int32_t icx = cell_coord(xp.x, d.cw), icy = cell_coord(xp.y, d.cw), icz = cell_coord(xp.z, d.cw);
    const bool prune = PRUNE && d.gx >= 4 && d.gy >= 4 && d.gz >= 4;
    float lx = 0.f, ly = 0.f, lz = 0.f, rx = 0.f, ry = 0.f, rz = 0.f;
    if (prune) {
        lx = xp.x - (float)icx * d.cw;
        ly = xp.y - (float)icy * d.cw;
        lz = xp.z - (float)icz * d.cw;
        rx = d.cw - lx;
        ry = d.cw - ly;
        rz = d.cw - lz;
    }
    const float lim = d.h2 * 1.001f;
    const int sx = __ffs(d.gx) - 1, sy = __ffs(d.gy) - 1, sz = __ffs(d.gz) - 1;
    const uint32_t *off = offsets + d.c_off;
    const uint64_t *ch = chist + d.c_off;
#pragma unroll 1
    for (int rr = rr0; rr < rr1; ++rr) {  // rows (dz, dy), z outermost: the reference's walk order
        const int dz = rr / 3 - 1, dy = rr % 3 - 1;
        bool left = true, right = true;
        if (prune) {
            const float ez = dz < 0 ? lz : (dz > 0 ? rz : 0.f);
            const float ey = dy < 0 ? ly : (dy > 0 ? ry : 0.f);
            const float eyz2 = ey * ey + ez * ez;
            if (eyz2 > lim) continue;
            left = eyz2 + lx * lx <= lim;
            right = eyz2 + rx * rx <= lim;
        }
        const int32_t ty = icy + dy, tz = icz + dz;
        const uint32_t row = ((uint32_t)tz & (d.gz - 1u)) * d.gx * d.gy + ((uint32_t)ty & (d.gy - 1u)) * d.gx;
        const uint32_t cyz = (uint32_t)(((tz >> sz) & 1) << 2 | ((ty >> sy) & 1) << 1);
#pragma unroll 1
        for (int dx = -1; dx <= 1; ++dx) {
            if ((dx < 0 && !left) || (dx > 0 && !right)) continue;
            const int32_t tx = icx + dx;
            const uint32_t b = row + ((uint32_t)tx & (d.gx - 1u));
            uint32_t st = __ldg(off + b);
            uint32_t en = __ldg(off + b + 1);
            const uint64_t h = __ldg(reinterpret_cast<const unsigned long long *>(ch + b));
            if (st == en) continue;
            const float4 *src = xa;
            if (h != kClassWhole) {
                const uint32_t sh = 8u * (cyz | (uint32_t)((tx >> sx) & 1));
                const uint32_t cnt = (uint32_t)((h >> sh) & 0xFFull);
                if (cnt == 0) continue;  // no particle of this cell in the bucket
                if (cnt != en - st) {    // several classes: this one's sub-range of the walk copy
                    const uint64_t lower = sh ? (h & ((1ull << sh) - 1ull)) : 0ull;
                    st += (uint32_t)((lower * 0x0101010101010101ull) >> 56);  // byte sum: bucket <= 255
                    en = st + cnt;
                    src = wx;
                }
            }
            if (!r(src, st + shift, en + shift)) return;
        }
    }
}

// walk27 with the per-neighbour work taken out of the walk: candidates that
// pass accept(j) are queued in a small per-thread buffer and handed to use(j)
// in batches, so the neighbour math is not executed masked for every
// candidate of the walk.  use() sees the accepted candidates in walk order.
template <class A, class U>
__device__ __forceinline__ void walk27_batched(const SceneDesc &d, const uint32_t *__restrict__ offsets,
                                               uint32_t shift, float4 xp, A &&accept, U &&use)
{
    constexpr int kBuf = 32;
    uint32_t buf[kBuf];
    int nb = 0;
    walk27_ranges(d, offsets, shift, xp, [&](uint32_t st, uint32_t en) -> bool {
        for (uint32_t j = st; j < en; ++j) {
            if (accept(j)) {
                buf[nb++] = j;
                if (nb == kBuf) {
                    for (int k = 0; k < kBuf; ++k) use(buf[k]);
                    nb = 0;
                }
            }
        }
        return true;
    });
    for (int k = 0; k < nb; ++k) use(buf[k]);
}

// The neighbour list is stored in quads of slots: slot k of particle slot i
// at nbr[(k / 4 * stride + i) * 4 + k % 4] (stride = particle slots), so a
// thread's four consecutive slots are one aligned 16-byte load and the
// quads of a warp's particles lie side by side (coalesced).  list_of is a
// particle's base, list_slot the offset of its slot k.
__device__ __forceinline__ uint32_t *list_of(uint32_t *nbr, uint32_t i) { return nbr + 4ull * i; }
__device__ __forceinline__ uint64_t list_slot(uint32_t k, uint64_t stride)
{
    return (uint64_t)(k >> 2) * stride * 4u + (k & 3u);
}

// One 16-byte row of a particle's list (a quad of u32 or an oct of u16
// slots), loaded and stored as streaming data (evict-first): the lists of a
// batch (hundreds of MB) pass through L2 once per pass, and the hint keeps
// them from evicting the positions the same passes gather (batched step
// +1%, the list-form vorticity pass -4%, interleaved A/B).
__device__ __forceinline__ uint4 list_ld(const uint4 *p) { return __ldcs(p); }
__device__ __forceinline__ void list_st(uint4 *p, uint4 v) { __stcs(p, v); }

__device__ __forceinline__ uint32_t quad_at(const uint4 &v, int j)
{
    return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// Visit list slots [0, nn) of one particle in list order.  Indices are
// requested CH at a time (CH / 4 quads), one chunk ahead of their use; the
// chunk (loads in flight against registers) is picked by the autotuner.
// Whole chunks call f without per-slot predicates; only the quad requests
// and the final partial chunk test against nn.
template <int CH, class F>
__device__ __forceinline__ void list_walk(const uint32_t *__restrict__ nl, uint64_t stride, uint32_t nn, F &&f)
{
    static_assert(CH % 4 == 0, "a chunk holds whole quads");
    constexpr int NQ = CH / 4;
    const uint4 *p = reinterpret_cast<const uint4 *>(nl);  // quad kq of the particle at p[kq * stride]
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    uint4 qn[NQ];
#pragma unroll
    for (int c = 0; c < NQ; ++c) qn[c] = ((uint32_t)(4 * c) < nn) ? list_ld(p + c * stride) : z;
    uint32_t k0 = 0;
    for (; k0 + CH <= nn; k0 += CH) {
        uint4 q[NQ];
#pragma unroll
        for (int c = 0; c < NQ; ++c) q[c] = qn[c];
        p += NQ * stride;
#pragma unroll
        for (int c = 0; c < NQ; ++c) qn[c] = (k0 + CH + 4 * c < nn) ? list_ld(p + c * stride) : z;
#pragma unroll
        for (int c = 0; c < CH; ++c) f(quad_at(q[c >> 2], c & 3));
    }
#pragma unroll
    for (int c = 0; c < CH - 1; ++c)
        if (k0 + c < nn) f(quad_at(qn[c >> 2], c & 3));
}

// Scenes of at most kList16Max particle slots (every batched scene) keep
// their lists as u16 scene-local indices in octs of 8 slots: slot k of
// particle slot i at nbr16[((k / 8) * stride + i) * 8 + k % 8], the same
// 16-byte rows as the quads of u32 lists, half as many of them, so a pass
// reads half the list bytes.  list16_slot is the u16 offset of slot k from
// the particle's base (list_of, as for quads).
__device__ __forceinline__ uint64_t list16_slot(uint32_t k, uint64_t stride)
{
    return (uint64_t)(k >> 3) * stride * 8u + (k & 7u);
}

__device__ __forceinline__ uint32_t oct_at(const uint4 &v, int j)
{
    const uint32_t w = j < 2 ? v.x : (j < 4 ? v.y : (j < 6 ? v.z : v.w));
    return (j & 1) ? (w >> 16) : (w & 0xFFFFu);
}

// list_walk over a u16 list: octs requested one chunk (8 slots) ahead;
// f gets base + the scene-local index: the particle's sorted slot for base
// = the scene's first slot, the scene-local index itself for base = 0 (for
// arrays offset by the scene's first slot, which saves the add per slot;
// measured faster in the XSPH and vorticity-apply passes only).
template <class F>
__device__ __forceinline__ void list_walk16(const uint32_t *__restrict__ nl, uint64_t stride, uint32_t nn,
                                            uint32_t base, F &&f)
{
    const uint4 *p = reinterpret_cast<const uint4 *>(nl);  // oct ko of the particle at p[ko * stride]
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    uint4 qn = (0u < nn) ? list_ld(p) : z;
    uint32_t k0 = 0;
    for (; k0 + 8 <= nn; k0 += 8) {
        const uint4 q = qn;
        p += stride;
        qn = (k0 + 8 < nn) ? list_ld(p) : z;
#pragma unroll
        for (int c = 0; c < 8; ++c) f(base + oct_at(q, c));
    }
#pragma unroll
    for (int c = 0; c < 7; ++c)
        if (k0 + c < nn) f(base + oct_at(qn, c));
}

// The list of one particle in either form: u32 quads (indices are sorted
// slots) or u16 octs (scene-local indices, base = the scene's first slot).
template <int CH, class F>
__device__ __forceinline__ void list_walk_any(bool l16, const uint32_t *__restrict__ nl, uint64_t stride,
                                              uint32_t nn, uint32_t base, F &&f)
{
    if (l16)
        list_walk16(nl, stride, nn, base, f);
    else
        list_walk<CH>(nl, stride, nn, f);
}

// list_walk in chunks of one quad with the quads requested two chunks
// ahead: eight indices in flight, one quad of them per use.
template <class F>
__device__ __forceinline__ void list_walk_ahead2(const uint32_t *__restrict__ nl, uint64_t stride, uint32_t nn,
                                                 F &&f)
{
    const uint4 *p = reinterpret_cast<const uint4 *>(nl);
    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
    uint4 q0 = (0u < nn) ? list_ld(p) : z;
    uint4 q1 = (4u < nn) ? list_ld(p + stride) : z;
    uint32_t k0 = 0;
    for (; k0 + 4 <= nn; k0 += 4) {
        const uint4 q = q0;
        q0 = q1;
        q1 = (k0 + 8 < nn) ? list_ld(p + (uint64_t)((k0 >> 2) + 2) * stride) : z;
        f(q.x);
        f(q.y);
        f(q.z);
        f(q.w);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
        if (k0 + c < nn) f(quad_at(q0, c));
}

// Per-tile prologue shared by the particle kernels.
#define TILE_LOOP_BEGIN                                                   \
    const uint32_t n_tiles_ = a.ctrl->n_tiles;                            \
    for (uint32_t t_ = blockIdx.x; t_ < n_tiles_; t_ += gridDim.x) {      \
        const uint32_t s = __ldg(a.tile_scene + t_);                      \
        const uint32_t local = __ldg(a.tile_start + t_) + threadIdx.x;
#define TILE_LOOP_END }

// --------------------------------------------------------------- kernels --

// predict (pbf_solve.cpp:16-25 -> multiplyAddCUDA x2, pbf_predict.cu:15-45),
// calcHash (pbf_neighbor_search_util.cu:20-37), checkDeleteParticle
// (pbf_delete.cu:9-28; deleted key = ncell, one past the last cell) and the
// histogram of countingSort (insertAndCountCUDA, pbf_counting_sort.cu:21-32).
// PACKED: the input phase is read from the packed AoS float3 buffers of a
// packed-input step (what k_unpack would have written), and the particles
// are numbered afresh.
template <bool PACKED>
__global__ void __launch_bounds__(512) k_predict_hash(StepArgs a)
{
    TILE_LOOP_BEGIN
    const uint32_t n = a.scene_num[s];
    if (local >= n) continue;
    const SceneDesc d = a.scenes[s];
    const uint32_t i = d.p_off + local;
    float4 xv, vv;
    uint32_t id;
    if (PACKED) {
        const PackedIn pin = *a.pin;
        const uint64_t q = 3ull * ((uint64_t)a.pack_off[s] + local);
        xv = make_float4(pin.x[q], pin.x[q + 1], pin.x[q + 2], 0.f);
        vv = pin.v ? make_float4(pin.v[q], pin.v[q + 1], pin.v[q + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
        id = local;
        if (local == 0) a.next_id[s] = n;
    } else {
        xv = a.x[i];
        vv = a.v[i];
        id = a.id[i];
    }
    const float dt = d.dt;
    float4 ps;
    ps.x = __fmaf_rn(__fmaf_rn(d.g[0], dt, vv.x), dt, xv.x);
    ps.y = __fmaf_rn(__fmaf_rn(d.g[1], dt, vv.y), dt, xv.y);
    ps.z = __fmaf_rn(__fmaf_rn(d.g[2], dt, vv.z), dt, xv.z);
    ps.w = __uint_as_float(id);  // the id travels with the prediction to k_gather
    const int32_t cx = cell_coord(ps.x, d.cw), cy = cell_coord(ps.y, d.cw), cz = cell_coord(ps.z, d.cw);
    uint32_t key = hash3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz, d);
    uint32_t cls = alias_class(cx, cy, cz, d);
    if (ps.x < d.amin[0] || d.amax[0] < ps.x || ps.y < d.amin[1] || d.amax[1] < ps.y || ps.z < d.amin[2] ||
        d.amax[2] < ps.z) {
        key = d.ncell;
        cls = 0;
    }
    a.cls[i] = (uint8_t)cls;
    if (!(isfinite(ps.x) && isfinite(ps.y) && isfinite(ps.z))) atomicOr(a.flags + s, PBF_FLAG_NONFINITE);
    a.xs[i] = ps;
    a.key[i] = key;
    a.slot[i] = atomicAdd(a.count + d.c_off + key, 1u);
    TILE_LOOP_END
}

// ---- exclusive scan of the cell counts (reduce, spine, down-sweep) ----
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v)
{
    const uint32_t lane = threadIdx.x & 31u;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

__global__ void __launch_bounds__(256) k_scan_reduce(StepArgs a)
{
    __shared__ uint32_t ws[kScanWarps];
    const uint32_t n = a.ctrl->n_cells;
    const uint32_t ntile = (n + kScanTile - 1) / kScanTile;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t t = blockIdx.x; t < ntile; t += gridDim.x) {
        const uint32_t base = t * kScanTile + warp * kScanItemsPerWarp;
        uint32_t sum = 0;
#pragma unroll
        for (uint32_t j = 0; j < 16; ++j) {
            const uint32_t idx = base + j * 32 + lane;
            if (idx < n) sum += a.count[idx];
        }
#pragma unroll
        for (uint32_t o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (lane == 0) ws[warp] = sum;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t tot = 0;
            for (uint32_t k = 0; k < kScanWarps; ++k) tot += ws[k];
            a.bsum[t] = tot;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(1024) k_scan_spine(StepArgs a)
{
    __shared__ uint32_t ws[32];
    __shared__ uint32_t carry;
    const uint32_t n = a.ctrl->n_cells;
    const uint32_t ntile = (n + kScanTile - 1) / kScanTile;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        carry = 0;
        *a.dense = 0;  // the bucket queues of this step's rank kernel
        *a.mid = 0;
    }
    __syncthreads();
    for (uint32_t base = 0; base < ntile; base += 1024) {
        const uint32_t idx = base + threadIdx.x;
        const uint32_t v = idx < ntile ? a.bsum[idx] : 0u;
        const uint32_t inc = warp_incl_scan(v);
        if (lane == 31) ws[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            const uint32_t wv = ws[lane];
            ws[lane] = warp_incl_scan(wv) - wv;
        }
        __syncthreads();
        const uint32_t c = carry;
        if (idx < ntile) a.bsum[idx] = c + ws[warp] + inc - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c + ws[warp] + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) a.offsets[n] = carry;
}

// The whole scan in one block for tables of at most 1024 * R cells, R
// rounds of 1024 held in registers: every round's counts are requested at
// once (coalesced), the rounds' warp scans run side by side, one warp turns
// the rounds' warp totals into offsets (carrying across rounds in order),
// and the offsets are written coalesced.  Two barriers in all.
template <uint32_t R>
__global__ void __launch_bounds__(1024) k_scan_single_reg(StepArgs a)
{
    __shared__ uint32_t ws[R][32];
    const uint32_t n = a.ctrl->n_cells;
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    if (t == 0) {
        *a.dense = 0;  // the bucket queues of this step's rank kernel
        *a.mid = 0;
    }
    uint32_t v[R], inc[R];
#pragma unroll
    for (uint32_t k = 0; k < R; ++k) {
        const uint32_t idx = k * 1024u + t;
        v[k] = idx < n ? a.count[idx] : 0u;
    }
#pragma unroll
    for (uint32_t k = 0; k < R; ++k) {
        inc[k] = warp_incl_scan(v[k]);
        if (lane == 31) ws[k][warp] = inc[k];
    }
    __syncthreads();
    if (warp == 0) {  // exclusive prefix of every (round, warp) total, rounds in order
        uint32_t carry = 0;
#pragma unroll
        for (uint32_t k = 0; k < R; ++k) {
            const uint32_t wv = ws[k][lane];
            const uint32_t wi = warp_incl_scan(wv);
            ws[k][lane] = carry + wi - wv;
            carry += __shfl_sync(0xffffffffu, wi, 31);
        }
        if (lane == 0) a.offsets[n] = carry;
    }
    __syncthreads();
#pragma unroll
    for (uint32_t k = 0; k < R; ++k) {
        const uint32_t idx = k * 1024u + t;
        if (idx < n) {
            a.offsets[idx] = ws[k][warp] + inc[k] - v[k];
            a.count[idx] = 0u;  // ready for the next step's histogram
        }
    }
}

// The whole scan in one block, for tables of at most kSingleScanMax cells
// (small scenes: one launch instead of three).
__global__ void __launch_bounds__(1024) k_scan_single(StepArgs a)
{
    __shared__ uint32_t ws[32];
    __shared__ uint32_t carry;
    const uint32_t n = a.ctrl->n_cells;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        carry = 0;
        *a.dense = 0;  // the bucket queues of this step's rank kernel
        *a.mid = 0;
    }
    __syncthreads();
    for (uint32_t base = 0; base < n; base += 1024) {
        const uint32_t idx = base + threadIdx.x;
        const uint32_t v = idx < n ? a.count[idx] : 0u;
        const uint32_t inc = warp_incl_scan(v);
        if (lane == 31) ws[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            const uint32_t wv = ws[lane];
            ws[lane] = warp_incl_scan(wv) - wv;
        }
        __syncthreads();
        const uint32_t c = carry;
        if (idx < n) {
            a.offsets[idx] = c + ws[warp] + inc - v;
            a.count[idx] = 0u;  // ready for the next step's histogram
        }
        __syncthreads();
        if (threadIdx.x == 1023) carry = c + ws[warp] + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) a.offsets[n] = carry;
}

__global__ void __launch_bounds__(256) k_scan_down(StepArgs a)
{
    __shared__ uint32_t ws[kScanWarps];
    const uint32_t n = a.ctrl->n_cells;
    const uint32_t ntile = (n + kScanTile - 1) / kScanTile;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (uint32_t t = blockIdx.x; t < ntile; t += gridDim.x) {
        const uint32_t base = t * kScanTile + warp * kScanItemsPerWarp;
        uint32_t vals[16];
        uint32_t sum = 0;
#pragma unroll
        for (uint32_t j = 0; j < 16; ++j) {
            const uint32_t idx = base + j * 32 + lane;
            vals[j] = idx < n ? a.count[idx] : 0u;
            sum += vals[j];
        }
        uint32_t wsum = sum;
#pragma unroll
        for (uint32_t o = 16; o > 0; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
        if (lane == 0) ws[warp] = wsum;
        __syncthreads();
        uint32_t run = a.bsum[t];
        for (uint32_t k = 0; k < warp; ++k) run += ws[k];
#pragma unroll
        for (uint32_t j = 0; j < 16; ++j) {
            const uint32_t idx = base + j * 32 + lane;
            const uint32_t inc = warp_incl_scan(vals[j]);
            if (idx < n) {
                a.offsets[idx] = run + inc - vals[j];
                a.count[idx] = 0u;  // ready for the next step's histogram
            }
            run += __shfl_sync(0xffffffffu, inc, 31);
        }
        __syncthreads();
    }
}

// tmp entries of scenes up to kClsLimit particles carry the member's alias
// class above its input index.  wpos of a particle outside a mixed-class
// bucket is kNoWalkCopy.
constexpr uint32_t kClsShift = 29;
constexpr uint32_t kClsLimit = 1u << kClsShift;
constexpr uint32_t kNoWalkCopy = 0xFFFFFFFFu;

// Scatter into the cell buckets in atomic-slot order (sortByCountingCUDA,
// pbf_counting_sort.cu:120-134).
__global__ void __launch_bounds__(512) k_scatter(StepArgs a)
{
    TILE_LOOP_BEGIN
    const uint32_t n = a.scene_num[s];
    if (local >= n) continue;
    const SceneDesc d = a.scenes[s];
    const uint32_t i = d.p_off + local;
    const uint32_t pos = a.offsets[d.c_off + a.key[i]] + a.slot[i];
    // the alias class rides in the top bits (scenes below 2^29 particles)
    a.tmp[pos] = d.capacity <= kClsLimit ? local | ((uint32_t)a.cls[i] << kClsShift) : local;
    TILE_LOOP_END
}

// Stable rank inside each bucket (count of smaller input indices): the
// permutation of a stable sort by cell (cub::DeviceRadixSort::SortPairs
// order), which reorderDataCUDA (pbf_neighbor_search_util.cu:143-154) then
// applies.  One thread per cell, cells in order, so the cell ranges, the
// bucket entries and the bucket's part of the permutation are read and
// written contiguously whatever the particles' input order.  Buckets of up
// to kMidMin members are ranked here; larger ones are queued for
// k_dense_sort (a warp per bucket up to kDenseMin members, a block beyond:
// a shared-memory sort up to kStableLimit members, a radix sort in global
// memory above, which degenerate inputs and mass deletion can reach).
constexpr uint32_t kStableLimit = 4096;
constexpr uint32_t kDenseMin = 64;
static_assert(kStableLimit * sizeof(uint32_t) == sizeof(RadixSmem), "the radix sort reuses the bitonic buffer");
__global__ void __launch_bounds__(kCellTileMax) k_rank_cells(StepArgs a)
{
    const uint32_t n0 = a.ctrl->n_tiles, nct = a.ctrl->n_cell_tiles;
    for (uint32_t t_ = blockIdx.x; t_ < nct; t_ += gridDim.x) {
        // the tile's scene: its fields once per tile, in registers
        const uint32_t s = __ldg(a.tile_scene + n0 + t_);
        const SceneDesc *sd = a.scenes + s;
        const uint32_t ncell = __ldg(&sd->ncell), c_off = __ldg(&sd->c_off), p_off = __ldg(&sd->p_off);
        const bool packed = __ldg(&sd->capacity) <= kClsLimit;
        const bool grouped = packed && __ldg(&sd->gx) >= 4 && __ldg(&sd->gy) >= 4 && __ldg(&sd->gz) >= 4;
        const uint32_t lc = __ldg(a.tile_start + n0 + t_) + threadIdx.x;
        if (lc > ncell) continue;  // local cells 0..ncell (ncell: the deleted bucket)
        const uint32_t gk = c_off + lc;
        const uint32_t st = __ldg(a.offsets + gk), en = __ldg(a.offsets + gk + 1);
        if (st == en) continue;
        const uint32_t b = en - st;
        if (b > kMidMin) {
            uint32_t *q = b > kDenseMin ? a.dense : a.mid;
            const uint32_t k = atomicAdd(q, 1u);
            q[1 + 2 * k] = gk;
            q[2 + 2 * k] = s;
            continue;
        }
        const uint32_t g0 = p_off + (st - __ldg(a.offsets + c_off));
        const uint32_t imask = packed ? kClsLimit - 1u : 0xFFFFFFFFu;
        // the alias class rides in the entries' top bits (scenes below 2^29
        // particles); the walk copy groups a bucket by class when the grid
        // is at least 4 cells on every axis
        uint32_t e[kMidMin];
        uint64_t hist = 0;
        for (uint32_t t = 0; t < b; ++t) {
            e[t] = __ldg(a.tmp + st + t);
            hist += 1ull << (8u * (packed ? e[t] >> kClsShift : 0u));
        }
        const uint32_t c0 = packed ? e[0] >> kClsShift : 0u;
        const bool mixed = grouped && hist != ((uint64_t)b << (8u * c0));
        for (uint32_t t = 0; t < b; ++t) {
            const uint32_t it = e[t] & imask, ct = packed ? e[t] >> kClsShift : 0u;
            uint32_t rank = 0, below = 0, frank = 0;
            for (uint32_t u = 0; u < b; ++u) {
                const uint32_t iu = e[u] & imask, cu = packed ? e[u] >> kClsShift : 0u;
                rank += iu < it ? 1u : 0u;
                below += cu < ct ? 1u : 0u;
                frank += (cu == ct && iu < it) ? 1u : 0u;
            }
            a.perm[g0 + rank] = it;
            a.wpos[g0 + rank] = mixed ? g0 + below + frank : kNoWalkCopy;
        }
        a.chist[gk] = grouped ? hist : kClassWhole;
    }
}

// The same ranks from the particle side, for small steps (latency bound:
// the per-cell kernel's b^2 loop in one thread lengthens the critical
// path): each particle counts the smaller input indices of its bucket.
// Buckets above kDenseMin members (of any size) are queued for
// k_dense_sort by their first member (atomic slot 0); nothing is queued for
// the warp tier.
__global__ void __launch_bounds__(512) k_rank_reorder(StepArgs a)
{
    TILE_LOOP_BEGIN
    const uint32_t n = a.scene_num[s];
    if (local >= n) continue;
    const SceneDesc d = a.scenes[s];
    const uint32_t i = d.p_off + local;
    const uint32_t gk = d.c_off + a.key[i];
    const uint32_t st = a.offsets[gk], en = a.offsets[gk + 1];
    // rank: members with a smaller input index (stable sorted order); for the
    // walk copy also members of a smaller class, members of the same class
    // with a smaller input index, and the bucket's class histogram
    const bool packed = d.capacity <= kClsLimit;
    const uint32_t imask = packed ? kClsLimit - 1u : 0xFFFFFFFFu;
    const uint32_t my_cls = a.cls[i];
    uint32_t rank = 0, below = 0, frank = 0;
    const bool grouped = packed && en - st <= 255u && d.gx >= 4 && d.gy >= 4 && d.gz >= 4;
    uint64_t hist = (uint64_t)(en - st) << (8u * my_cls);  // every member of my class
    bool mixed = false;
    if (en - st > kDenseMin) {
        // a dense bucket: one block of k_dense_sort orders it; its first
        // member by atomic slot queues it
        if (a.slot[i] == 0) {
            const uint32_t k = atomicAdd(a.dense, 1u);
            a.dense[1 + 2 * k] = gk;
            a.dense[2 + 2 * k] = s;
        }
        continue;
    }
    uint32_t diff = 0;
    for (uint32_t t = st; t < en; ++t) {
        const uint32_t e = __ldg(a.tmp + t);
        rank += ((e & imask) < local) ? 1u : 0u;
        diff |= (e >> kClsShift) ^ my_cls;
    }
    if (grouped && diff) {  // several classes: the class histogram and my place in the walk copy
        mixed = true;
        hist = 0;
        for (uint32_t t = st; t < en; ++t) {
            const uint32_t e = __ldg(a.tmp + t);
            const uint32_t mc = e >> kClsShift;
            below += (mc < my_cls) ? 1u : 0u;
            frank += (mc == my_cls && (e & imask) < local) ? 1u : 0u;
            hist += 1ull << (8u * mc);
        }
    }
    const uint32_t base = a.offsets[d.c_off];
    const uint32_t g = d.p_off + (st - base) + rank;
    // only 4-byte entries are scattered here; k_gather moves the 16-byte
    // particle data in sorted order (coalesced writes, as the reference's
    // reorderDataCUDA gathers).  Buckets holding more than one alias class
    // also place the particle in the class-grouped walk copy.
    a.wpos[g] = mixed ? d.p_off + (st - base) + below + frank : kNoWalkCopy;
    if (rank == 0) a.chist[gk] = grouped ? hist : kClassWhole;
    a.perm[g] = local;
    TILE_LOOP_END
}

// Buckets queued by the rank kernels (k_rank_cells queues medium and dense
// ones, k_rank_reorder dense ones).  Medium ones (kMidMin+1 .. kDenseMin
// members) first, a warp each: members in lanes, each ranked by counting
// over the others (broadcast by shuffle).  Dense ones (kDenseMin+1 ..
// kStableLimit) then, a block each: the bucket entries (input index, alias
// class in the top bits) are sorted in shared memory by input index (the
// stable sorted order) and, when the bucket mixes classes, by (class, index)
// (the walk copy's order).  Both give the permutation, class counts and
// walk-copy places of k_rank_cells' per-bucket count.  Buckets above
// kStableLimit get a block each too: a radix sort by input index in global
// memory (block_radix_stable), walked whole.
__device__ __forceinline__ uint32_t dense_key(uint32_t e, uint32_t imask)
{
    return e == 0xFFFFFFFFu ? 0xFFFFFFFFu : (e & imask);  // padding sorts last
}

template <bool FULL>
__device__ void bitonic_sort(uint32_t *v, uint32_t n, uint32_t imask)
{
    for (uint32_t size = 2; size <= n; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t t = threadIdx.x; t < (n >> 1); t += blockDim.x) {
                const uint32_t i = 2 * stride * (t / stride) + (t % stride), j = i + stride;
                const uint32_t vi = v[i], vj = v[j];
                const uint32_t ki = FULL ? vi : dense_key(vi, imask), kj = FULL ? vj : dense_key(vj, imask);
                const bool asc = (i & size) == 0;
                if ((ki > kj) == asc) {
                    v[i] = vj;
                    v[j] = vi;
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(kRadixThreads) k_dense_sort(StepArgs a)
{
    __shared__ __align__(16) uint32_t S[kStableLimit];
    __shared__ uint32_t W[kStableLimit];
    __shared__ uint32_t chist_cnt[8], rbase[16], rtot[16];
    {
        const uint32_t nm = *(volatile const uint32_t *)a.mid;
        const uint32_t lane = threadIdx.x & 31u, wpb = blockDim.x >> 5;
        for (uint32_t k = blockIdx.x * wpb + (threadIdx.x >> 5); k < nm; k += gridDim.x * wpb) {
            const uint32_t gk = a.mid[1 + 2 * k], s = a.mid[2 + 2 * k];
            const SceneDesc &d = a.scenes[s];
            const uint32_t st = a.offsets[gk], b = a.offsets[gk + 1] - st;
            const uint32_t g0 = d.p_off + (st - a.offsets[d.c_off]);
            const bool packed = d.capacity <= kClsLimit;
            const uint32_t imask = packed ? kClsLimit - 1u : 0xFFFFFFFFu;
            const bool grouped = packed && d.gx >= 4 && d.gy >= 4 && d.gz >= 4;
            const bool h0 = lane < b, h1 = 32u + lane < b;
            const uint32_t e0 = h0 ? a.tmp[st + lane] : 0u, e1 = h1 ? a.tmp[st + 32u + lane] : 0u;
            const uint32_t i0 = e0 & imask, i1 = e1 & imask;
            const uint32_t c0 = packed ? e0 >> kClsShift : 0u, c1 = packed ? e1 >> kClsShift : 0u;
            uint64_t hist = (h0 ? 1ull << (8u * c0) : 0ull) + (h1 ? 1ull << (8u * c1) : 0ull);
#pragma unroll
            for (uint32_t o = 16; o > 0; o >>= 1) hist += __shfl_xor_sync(0xffffffffu, hist, o);
            const uint32_t cf = __shfl_sync(0xffffffffu, c0, 0);
            const bool mixed = grouped && hist != ((uint64_t)b << (8u * cf));
            uint32_t r0 = 0, b0 = 0, f0 = 0, r1 = 0, b1 = 0, f1 = 0;
            for (uint32_t u = 0; u < b; ++u) {
                const uint32_t eu = __shfl_sync(0xffffffffu, u < 32u ? e0 : e1, u & 31u);
                const uint32_t iu = eu & imask, cu = packed ? eu >> kClsShift : 0u;
                r0 += iu < i0 ? 1u : 0u;
                b0 += cu < c0 ? 1u : 0u;
                f0 += (cu == c0 && iu < i0) ? 1u : 0u;
                r1 += iu < i1 ? 1u : 0u;
                b1 += cu < c1 ? 1u : 0u;
                f1 += (cu == c1 && iu < i1) ? 1u : 0u;
            }
            if (h0) {
                a.perm[g0 + r0] = i0;
                a.wpos[g0 + r0] = mixed ? g0 + b0 + f0 : kNoWalkCopy;
            }
            if (h1) {
                a.perm[g0 + r1] = i1;
                a.wpos[g0 + r1] = mixed ? g0 + b1 + f1 : kNoWalkCopy;
            }
            if (lane == 0) a.chist[gk] = grouped ? hist : kClassWhole;
        }
    }
    const uint32_t nd = *(volatile const uint32_t *)a.dense;
    for (uint32_t k = blockIdx.x; k < nd; k += gridDim.x) {
        const uint32_t gk = a.dense[1 + 2 * k], s = a.dense[2 + 2 * k];
        const SceneDesc &d = a.scenes[s];
        const uint32_t st = a.offsets[gk], en = a.offsets[gk + 1], b = en - st;
        const uint32_t base = a.offsets[d.c_off];
        const uint32_t g0 = d.p_off + (st - base);
        const bool packed = d.capacity <= kClsLimit;
        const uint32_t imask = packed ? kClsLimit - 1u : 0xFFFFFFFFu;
        if (b > kStableLimit) {  // the bucket's scatter entries are scratch once sorted into perm
            block_radix_stable(a.tmp + st, a.perm + g0, b, imask, radix_bits(d.capacity),
                               *reinterpret_cast<RadixSmem *>(S), rbase, rtot);
            for (uint32_t t = threadIdx.x; t < b; t += blockDim.x) a.wpos[g0 + t] = kNoWalkCopy;
            if (threadIdx.x == 0) a.chist[gk] = kClassWhole;
            __syncthreads();
            continue;
        }
        const bool grouped = packed && b <= 255u && d.gx >= 4 && d.gy >= 4 && d.gz >= 4;
        uint32_t P = 1;
        while (P < b) P <<= 1;
        if (threadIdx.x < 8) chist_cnt[threadIdx.x] = 0;
        __syncthreads();
        for (uint32_t t = threadIdx.x; t < P; t += blockDim.x) {
            const uint32_t e = t < b ? a.tmp[st + t] : 0xFFFFFFFFu;
            S[t] = e;
            W[t] = e;
            if (t < b && grouped) atomicAdd(&chist_cnt[e >> kClsShift], 1u);
        }
        __syncthreads();
        bitonic_sort<false>(S, P, imask);
        uint64_t hist = 0;
        uint32_t classes = 0;
        for (uint32_t c = 0; c < 8; ++c) {
            hist |= (uint64_t)chist_cnt[c] << (8u * c);
            classes += chist_cnt[c] ? 1u : 0u;
        }
        const bool mixed = grouped && classes > 1;
        if (mixed) bitonic_sort<true>(W, P, imask);  // (class, index) order
        for (uint32_t t = threadIdx.x; t < b; t += blockDim.x) {
            a.perm[g0 + t] = S[t] & imask;
            if (!mixed) a.wpos[g0 + t] = kNoWalkCopy;
        }
        if (mixed) {
            for (uint32_t w = threadIdx.x; w < b; w += blockDim.x) {
                const uint32_t key = W[w] & imask;  // its place in S (sorted by index)
                uint32_t lo = 0, hi = b;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if ((S[mid] & imask) < key) lo = mid + 1;
                    else hi = mid;
                }
                a.wpos[g0 + lo] = g0 + w;
            }
        }
        if (threadIdx.x == 0) a.chist[gk] = grouped ? hist : kClassWhole;
        __syncthreads();
    }
}

// Reorder in sorted order (reorderDataCUDA x2, pbf_neighbor_search_util.cu:143-154):
// sorted predicted positions (carrying their own slot in .w, which the
// neighbour walk records), sorted old positions and ids; the walk copy of
// mixed-class buckets.  PACKED: old positions from the packed input.
template <bool PACKED>
__global__ void __launch_bounds__(512) k_gather(StepArgs a)
{
    TILE_LOOP_BEGIN
    const uint32_t n = a.scene_num[s];
    if (local >= n) continue;
    const SceneDesc d = a.scenes[s];
    const uint32_t g = d.p_off + local;
    const uint32_t li = a.perm[g];
    const uint32_t i = d.p_off + li;
    const float4 ps = a.xs[i];
    const float4 xg = make_float4(ps.x, ps.y, ps.z, __uint_as_float(g));
    a.xa[g] = xg;
    if (PACKED) {
        const float *px = a.pin->x + 3ull * ((uint64_t)a.pack_off[s] + li);
        a.xold[g] = make_float4(px[0], px[1], px[2], 0.f);
    } else {
        a.xold[g] = a.x[i];
    }
    a.id_tmp[g] = __float_as_uint(ps.w);  // the id, stored beside the prediction
    const uint32_t w = a.wpos[g];
    if (w != kNoWalkCopy) a.wx[w] = xg;
    TILE_LOOP_END
}

// Neighbour list (detectNeighborsCUDA<uint32_t>, pbf_neighbor_search_util.cu:454-482,
// cap max_pair-1, self included) fused with the iteration-0 lambda
// (calcScalingFactorCUDA cached, pbf_constraint.cu:168-209): at iteration 0
// the working positions are the sorted predicted positions, so the pair
// terms can be summed while the list is built.
// SMEM: the accepted indices are collected in shared memory ([slot][thread]
// per block, conflict-free), then written to the list in whole quads (a
// warp's 16-byte stores contiguous) instead of one scattered 4-byte store per
// accepted candidate, and the lambda loop reads them back from shared memory.
template <bool SMEM>
__global__ void __launch_bounds__(512, 2) k_neighbors_lambda(StepArgs a)
{
    extern __shared__ uint32_t s_list[];  // SMEM: [slot][threadIdx.x]
    TILE_LOOP_BEGIN
    const SceneDesc d = a.scenes[s];
    const uint32_t base = a.offsets[d.c_off];
    const uint32_t live = a.offsets[d.c_off + d.ncell] - base;
    if (local >= live) continue;
    const uint32_t i = d.p_off + local;
    const uint32_t shift = d.p_off - base;
    const float4 xp = a.xa[i];
    const float h2 = d.h2;
    const PairConst pc = pair_const(d);
    const uint32_t cap = d.cap;
    const uint64_t stride = a.nbr_stride;
    uint32_t *nl = list_of(a.nbr, i);
    uint16_t *nl16 = reinterpret_cast<uint16_t *>(nl);  // u16 lists: scene-local indices
    const bool l16 = d.list16 != 0;
    const float4 *__restrict__ xa = a.xa;
    const float4 *__restrict__ wx = a.wx;
    // phase 1: the walk only tests and records (lanes of a warp accept
    // different candidates, so pair math inside the walk would run masked
    // for almost every candidate); a candidate's .w is its sorted slot
    // Candidates are fetched kNbFetch at a time (more loads in flight; a
    // group past the range's end reads up to kNbFetch - 1 records beyond it,
    // never accepted: xa and wx carry that many spare records at the end of
    // their allocations), all of the
    // group is tested first (independent chains), then the accepted ones are
    // appended in order up to the cap, so the first `cap` accepted ones are
    // the reference's.
    // The particle itself is accepted (r^2 = 0) and counts toward the cap at
    // its walk position, but the list does not store it: its pair terms are
    // w(0) = 1 in the density sum and exactly 0 everywhere else.  selfat
    // records the position (the debug getter's reference-layout list puts it
    // back), and the lambda sums start from 1.  SMEM: the walk collects
    // every accepted candidate, the particle's own slot is found in shared
    // memory afterwards and left out of the write-out, so the candidate loop
    // carries no extra state; otherwise the walk skips it as it stores.
    constexpr uint32_t kNbFetch = 4;
    uint32_t cnt = 0, selfat = kNotListed;
    walk27_cells<true>(d, a.offsets, a.chist, xa, wx, shift, xp,
                       [&](const float4 *src, uint32_t st, uint32_t en) -> bool {
        for (uint32_t q0 = st; q0 < en; q0 += kNbFetch) {
            float4 c[kNbFetch];
            const float4 *pq = src + q0;
#pragma unroll
            for (uint32_t k = 0; k < kNbFetch; ++k) c[k] = __ldg(pq + k);
            bool acc[kNbFetch];
#pragma unroll
            for (uint32_t k = 0; k < kNbFetch; ++k) acc[k] = (q0 + k < en) && dist2_exact(xp, c[k]) < h2;
#pragma unroll
            for (uint32_t k = 0; k < kNbFetch; ++k) {
                if (acc[k] && cnt < cap) {
                    const uint32_t q = __float_as_uint(c[k].w);
                    if (SMEM) {
                        s_list[cnt * blockDim.x + threadIdx.x] = q;
                    } else {
                        const uint32_t ks = cnt - (selfat < cnt ? 1u : 0u);  // stored entries before this one
                        if (q == i)
                            selfat = cnt;
                        else if (l16)
                            nl16[list16_slot(ks, stride)] = (uint16_t)(q - d.p_off);
                        else
                            nl[list_slot(ks, stride)] = q;
                    }
                    ++cnt;
                }
            }
            if (cnt == cap) return false;
        }
        return true;
    });
    const uint32_t *rd = s_list + threadIdx.x;
    if (SMEM) {
        for (uint32_t k = 0; k < cnt; ++k)
            if (rd[k * blockDim.x] == i) selfat = k;
    }
    cnt -= selfat < cnt ? 1u : 0u;  // entries stored
    a.nnb[i] = (uint8_t)cnt;
    a.selfat[i] = (uint8_t)selfat;
    // phase 2: lambda over the list just written (L2-resident; plain loads,
    // the read-only path may not see this kernel's own stores)
    LamSum ls;
    if (selfat != kNotListed) ls.ks = 1.f;
    if (SMEM) {  // the list from shared memory, written out slot by slot as it is summed
        // stored entry k is shared-memory entry k, or k + 1 from the
        // particle's own slot on
        auto src = [&](uint32_t k) { return rd[(k + (k >= selfat ? 1u : 0u)) * blockDim.x]; };
        // the list out in whole quads (u32) or octs (u16): one 16-byte store
        // per four or eight slots (slots past the count in the last one are
        // padding, never read)
        uint4 *wq = reinterpret_cast<uint4 *>(nl);
        if (l16) {
            for (uint32_t k0 = 0; k0 < cnt; k0 += 8) {
                uint32_t w[4];
#pragma unroll
                for (uint32_t j = 0; j < 4; ++j) {
                    const uint32_t lo = (k0 + 2 * j < cnt) ? src(k0 + 2 * j) - d.p_off : 0u;
                    const uint32_t hi = (k0 + 2 * j + 1 < cnt) ? src(k0 + 2 * j + 1) - d.p_off : 0u;
                    w[j] = (lo & 0xFFFFu) | (hi << 16);
                }
                list_st(wq + (uint64_t)(k0 >> 3) * stride, make_uint4(w[0], w[1], w[2], w[3]));
            }
        } else {
            for (uint32_t k0 = 0; k0 < cnt; k0 += 4) {
                uint32_t q4[4];
#pragma unroll
                for (uint32_t j = 0; j < 4; ++j) q4[j] = (k0 + j < cnt) ? src(k0 + j) : 0u;
                list_st(wq + (uint64_t)(k0 >> 2) * stride, make_uint4(q4[0], q4[1], q4[2], q4[3]));
            }
        }
#pragma unroll 4
        for (uint32_t k = 0; k < cnt; ++k) lam_add(ls, xp, __ldg(xa + src(k)), pc);
    } else {
#pragma unroll 4
        for (uint32_t k = 0; k < cnt; ++k) {
            const uint32_t q = l16 ? d.p_off + nl16[list16_slot(k, stride)] : nl[list_slot(k, stride)];
            lam_add(ls, xp, __ldg(xa + q), pc);
        }
    }
    a.lam[i] = ls.lambda(d);
    TILE_LOOP_END
}

// Small (latency-bound) steps: one particle's walk split over kSplit lanes
// of a warp, each walking a contiguous run of the nine (dz, dy) rows into a
// private buffer of at most cap entries.  A prefix over the group's counts
// then places every lane's entries after those of the rows before it, so the
// list holds the first cap accepted candidates in the reference's walk
// order, as k_neighbors_lambda's.  The group then sums the iteration-0
// lambda over the list in list order (lam_sum_split: the same sum, bit for
// bit).  Scenes with more than kSplitCap list slots walk in one lane.
constexpr uint32_t kSplitCap = 64;
static_assert(kSplit == 4 || kSplit == 8, "a particle's lanes share one aligned group of a warp");

// The (dz, dy) rows [rr0, rr1) of a particle's lane sub: rows shared evenly,
// the first lane taking the one left over.
__device__ __forceinline__ void split_rows(uint32_t sub, int &rr0, int &rr1)
{
    constexpr int per = 9 / (int)kSplit, extra = 9 - per * (int)kSplit;
    rr0 = sub == 0 ? 0 : extra + per * (int)sub;
    rr1 = extra + per * ((int)sub + 1);
}

// Small steps: a sum over one particle's list split over the particle's
// kSplit lanes.  Lane sub evaluates slots sub, sub + kSplit, ...; each
// round's terms reach every lane of the group by shuffles and are added in
// list order, so every lane ends with the one-lane sums, bit for bit.  List
// indices are requested two rounds ahead and positions one round ahead (a
// slot past the list reads index 0, a valid slot, and adds nothing).  RO:
// the list is read through the read-only path (it was not written by this
// kernel).
template <bool RO>
__device__ __forceinline__ uint32_t split_index(const uint32_t *nl, uint64_t stride, uint32_t nn, uint32_t k,
                                                bool l16, uint32_t base)
{
    if (k >= nn) return 0u;
    if (l16) {
        const uint16_t *p = reinterpret_cast<const uint16_t *>(nl) + list16_slot(k, stride);
        return base + (RO ? __ldg(p) : *p);
    }
    const uint32_t *p = nl + list_slot(k, stride);
    return RO ? __ldg(p) : *p;
}

template <bool RO>
__device__ __forceinline__ LamSum lam_sum_split(const uint32_t *nl, uint64_t stride, uint32_t nn,
                                                const float4 *__restrict__ xc, float4 xp, const SceneDesc &d,
                                                uint32_t sub, uint32_t gmask, bool self_listed)
{
    const PairConst pc = pair_const(d);
    const bool l16 = d.list16 != 0;
    const uint32_t base = d.p_off;
    LamSum ls;
    if (self_listed) ls.ks = 1.f;  // the particle's own w(0), first as in the one-lane passes
    float4 x0 = __ldg(xc + split_index<RO>(nl, stride, nn, sub, l16, base));
    uint32_t q1 = split_index<RO>(nl, stride, nn, sub + kSplit, l16, base);
    for (uint32_t k0 = 0; k0 < nn; k0 += kSplit) {
        const float4 x1 = __ldg(xc + q1);
        q1 = split_index<RO>(nl, stride, nn, k0 + 2 * kSplit + sub, l16, base);
        // this lane's pair (slot k0 + sub); a slot past the list reads
        // index 0 and is not added
        const PairGeo g = pair_geo(xp, x0);
        const PairWS k = pair_ws(g.r2, pc);
#pragma unroll
        for (uint32_t j = 0; j < kSplit; ++j) {
            const float W = __shfl_sync(gmask, k.W, j, kSplit);
            const float s = __shfl_sync(gmask, k.s, j, kSplit);
            const float d0 = __shfl_sync(gmask, g.d0, j, kSplit);
            const float d1 = __shfl_sync(gmask, g.d1, j, kSplit);
            const float d2 = __shfl_sync(gmask, g.d2, j, kSplit);
            const float sr = __shfl_sync(gmask, k.sr, j, kSplit);
            if (k0 + j < nn) ls.add(W, s, d0, d1, d2, sr);
        }
        x0 = x1;
    }
    return ls;
}
__global__ void __launch_bounds__(256) k_neighbors_split(StepArgs a, uint32_t tile)
{
    const uint32_t per_block = blockDim.x / kSplit;  // particles per block
    const uint32_t parts = tile / per_block;         // blocks per tile
    const uint32_t lane = threadIdx.x & 31u, sub = threadIdx.x % kSplit;
    const uint32_t gmask = ((1u << kSplit) - 1u) << (lane & ~(kSplit - 1u));  // the particle's lanes
    const uint32_t n_work = a.ctrl->n_tiles * parts;
    for (uint32_t u = blockIdx.x; u < n_work; u += gridDim.x) {
        const uint32_t t_ = u / parts;
        const uint32_t s = __ldg(a.tile_scene + t_);
        const uint32_t local = __ldg(a.tile_start + t_) + (u % parts) * per_block + threadIdx.x / kSplit;
        const SceneDesc d = a.scenes[s];
        const uint32_t base = a.offsets[d.c_off];
        const uint32_t live = a.offsets[d.c_off + d.ncell] - base;
        if (local >= live) continue;  // the same for the group's lanes
        const uint32_t i = d.p_off + local;
        const uint32_t shift = d.p_off - base;
        const float4 xp = a.xa[i];
        const float h2 = d.h2;
        const uint32_t cap = d.cap;
        const uint64_t stride = a.nbr_stride;
        uint32_t *nl = list_of(a.nbr, i);
        uint16_t *nl16 = reinterpret_cast<uint16_t *>(nl);
        const bool l16 = d.list16 != 0;
        auto put = [&](uint32_t k, uint32_t q) {  // slot k of the list := sorted slot q
            if (l16)
                nl16[list16_slot(k, stride)] = (uint16_t)(q - d.p_off);
            else
                nl[list_slot(k, stride)] = q;
        };
        const float4 *__restrict__ xa = a.xa;
        const float4 *__restrict__ wx = a.wx;
        // rows shared over the lanes (split_rows); one lane takes all nine
        // when the list does not fit the private buffer
        const bool one = cap > kSplitCap;
        int rr0 = sub == 0 ? 0 : 9, rr1 = 9;
        if (!one) split_rows(sub, rr0, rr1);
        uint32_t buf[kSplitCap];
        // cnt: candidates this lane accepted, the particle itself included
        // (it counts toward the cap at its walk position but is not stored;
        // tself is its place in this lane's run)
        uint32_t cnt = 0, tself = kNotListed;
        if (one && sub == 0) {  // write straight into the list
            walk27_cells<true>(d, a.offsets, a.chist, xa, wx, shift, xp,
                               [&](const float4 *src, uint32_t st, uint32_t en) -> bool {
                for (uint32_t q = st; q < en; ++q) {
                    const float4 c = __ldg(src + q);
                    if (dist2_exact(xp, c) < h2) {
                        const uint32_t qs = __float_as_uint(c.w);
                        if (qs == i) tself = cnt;
                        else put(cnt - (tself < cnt ? 1u : 0u), qs);
                        if (++cnt == cap) return false;
                    }
                }
                return true;
            });
        } else if (!one) {
            walk27_cells<true>(d, a.offsets, a.chist, xa, wx, shift, xp,
                               [&](const float4 *src, uint32_t st, uint32_t en) -> bool {
                for (uint32_t q0 = st; q0 < en; q0 += 4) {
                    float4 c[4];
                    const float4 *pq = src + q0;  // up to three spare records past the range
#pragma unroll
                    for (uint32_t k = 0; k < 4; ++k) c[k] = __ldg(pq + k);
                    bool acc[4];
#pragma unroll
                    for (uint32_t k = 0; k < 4; ++k) acc[k] = (q0 + k < en) && dist2_exact(xp, c[k]) < h2;
#pragma unroll
                    for (uint32_t k = 0; k < 4; ++k) {
                        if (acc[k] && cnt < cap) {
                            const uint32_t qs = __float_as_uint(c[k].w);
                            if (qs == i) tself = cnt;
                            buf[cnt] = qs;
                            ++cnt;
                        }
                    }
                    if (cnt == cap) return false;
                }
                return true;
            }, rr0, rr1);
        }
        // place the group's runs one after the other, up to cap
        uint32_t incl = cnt;
#pragma unroll
        for (uint32_t o = 1; o < kSplit; o <<= 1) {
            const uint32_t v = __shfl_up_sync(gmask, incl, o, kSplit);
            if (sub >= o) incl += v;
        }
        const uint32_t total = __shfl_sync(gmask, incl, kSplit - 1, kSplit);
        const uint32_t pre = incl - cnt;
        // the particle's own place in the group's list (one lane holds it)
        uint32_t gself = tself != kNotListed ? pre + tself : 0xFFFFFFFFu;
#pragma unroll
        for (uint32_t o = 1; o < kSplit; o <<= 1) gself = min(gself, __shfl_xor_sync(gmask, gself, o, kSplit));
        const bool listed = gself < cap;
        if (!one) {
            for (uint32_t t = 0; t < cnt && pre + t < cap; ++t) {
                const uint32_t g = pre + t;
                if (g != gself) put(g - (g > gself ? 1u : 0u), buf[t]);
            }
        }
        const uint32_t nn = (total < cap ? total : cap) - (listed ? 1u : 0u);
        __syncwarp(gmask);  // the list entries of the group are visible to all its lanes
        // lambda of iteration 0 over the list, split over the group's lanes
        const LamSum ls = lam_sum_split<false>(nl, stride, nn, xa, xp, d, sub, gmask, listed);
        if (sub == 0) {
            a.nnb[i] = (uint8_t)nn;
            a.selfat[i] = listed ? (uint8_t)gself : kNotListed;
            a.lam[i] = ls.lambda(d);
        }
    }
}

// lambda for iterations >= 1 (memorizeKernelCalc + calcScalingFactor,
// pbf_kernel_memorization.cu:93-134 and pbf_constraint.cu:168-209, without the
// per-pair cache: W and grad W are recomputed from positions).  One thread
// per particle; the neighbour sums run in list order.
template <int kChunk, bool LAMW>
__global__ void __launch_bounds__(512, 2) k_lambda(StepArgs a, float4 *__restrict__ xc)
{
    TILE_LOOP_BEGIN
    const SceneDesc d = a.scenes[s];
    const uint32_t base = a.offsets[d.c_off];
    const uint32_t live = a.offsets[d.c_off + d.ncell] - base;
    if (local >= live) continue;
    const uint32_t i = d.p_off + local;
    const PairConst pc = pair_const(d);
    const float4 xp = xc[i];
    LamSum ls;
    if (a.selfat[i] != kNotListed) ls.ks = 1.f;  // the particle's own w(0), not stored in the list
    list_walk_any<kChunk>(d.list16 != 0, list_of(a.nbr, i), a.nbr_stride, a.nnb[i], d.p_off,
                          [&](uint32_t q) { lam_add(ls, xp, __ldg(xc + q), pc); });
    // LAMW: lambda rides in .w of the positions this pass reads and the
    // delta-p pass gathers next (neighbours here use only .xyz); small,
    // latency-bound steps keep it in its own array, as the store into the
    // gathered array slows this pass's neighbour reads there
    const float lam = ls.lambda(d);
    if (LAMW)
        reinterpret_cast<float *>(xc + i)[3] = lam;
    else
        a.lam[i] = lam;
    TILE_LOOP_END
}

// s_corr forms, selected once per tile (a tile belongs to one scene).
enum ScorrForm { kScorrReference, kScorrTextbook, kScorrOff, kScorrTextbook4 };

struct ScorrConst {
    float sci;  // max(-lambda_i, 0), the reference form's own share
    float c;    // the factor of w^n: 10 alpha^4 / W(0.4h)^4 (reference), k alpha^n / W(dq h)^n (textbook)
    int sn;
};

// -(lambda_i + lambda_j + s_corr) for a pair (the coefficient of grad W in
// calcPositionUpdateCUDA, pbf_position_update.cu:131-188).  s_corr as a
// constant times a power of w = W / alpha: reference 10 W^4 / W(0.4h)^4
// (max(-lambda_i, 0) + max(-lambda_j, 0)) (pbf_position_update.cu:136-146),
// textbook k (W / W(dq h))^n (Macklin and Mueller 2013, eq. 13); its last
// product is fused into the sum.
template <int FORM>
__device__ __forceinline__ float dp_coef(float li, float lj, float W, const ScorrConst &c)
{
    const float ll = __fadd_rn(li, lj);
    if (FORM == kScorrReference) {
        const float w2 = __fmul_rn(W, W);
        const float tc = __fmul_rn(c.c, __fmul_rn(w2, w2));
        return -__fmaf_rn(__fadd_rn(c.sci, fmaxf(-lj, 0.f)), tc, ll);
    } else if (FORM == kScorrTextbook4) {
        const float w2 = __fmul_rn(W, W);
        return -__fmaf_rn(c.c, __fmul_rn(w2, w2), ll);
    } else if (FORM == kScorrTextbook) {
        float pw = 1.f;
        for (int e = 0; e < c.sn; ++e) pw = __fmul_rn(pw, W);
        return -__fmaf_rn(c.c, pw, ll);
    }
    return -ll;
}

__device__ __forceinline__ ScorrConst scorr_const(const SceneDesc &d, float li)
{
    ScorrConst c;
    c.sci = fmaxf(-li, 0.f);
    c.c = d.tensile_mode == PBF_TENSILE_REFERENCE ? d.tens_c : d.scorr_c;
    c.sn = d.scorr_n;
    return c;
}

// Sum over the list of -(lambda_i + lambda_j + s_corr) grad W (the body of
// calcPositionUpdateCUDA, pbf_position_update.cu:131-188), in list order:
// each pair adds (coefficient * s) d.
template <int kChunk, int FORM, bool LAMW>
__device__ __forceinline__ float3 dp_sum(const StepArgs &a, const SceneDesc &d, const float4 *__restrict__ xc,
                                         uint32_t i, float4 xp, float li)
{
    const PairConst pc = pair_const(d);
    const ScorrConst sc = scorr_const(d, li);
    const float *__restrict__ lam = a.lam;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    list_walk_any<kChunk>(d.list16 != 0, list_of(a.nbr, i), a.nbr_stride, a.nnb[i], d.p_off, [&](uint32_t q) {
        const float4 xq = __ldg(xc + q);
        const PairGeo g = pair_geo<LAMW>(xp, xq);
        const PairWS k = pair_ws(g.r2, pc);
        const float lj = LAMW ? xq.w : __ldg(lam + q);  // LAMW: lambda in .w of the positions
        const float f = __fmul_rn(dp_coef<FORM>(li, lj, k.W, sc), k.s);
        if (LAMW) {  // large steps: the x and y sums by one packed fma (measured faster there only)
            fma2(s0, s1, f, f, g.d0, g.d1);
        } else {
            s0 = __fmaf_rn(f, g.d0, s0);
            s1 = __fmaf_rn(f, g.d1, s1);
        }
        s2 = __fmaf_rn(f, g.d2, s2);
    });
    return make_float3(s0, s1, s2);
}

// A particle's delta-p from the list sum: scale, boundary response, x += dp
// into the second buffer, and on the last iteration the velocity and id.
__device__ __forceinline__ void dp_finish(const StepArgs &a, const SceneDesc &d, uint32_t s, uint32_t i, float4 xp,
                                          float3 sum, float4 *__restrict__ xo, float4 *__restrict__ vo, int last)
{
    float3 dp = make_float3(sum.x * d.dp_k, sum.y * d.dp_k, sum.z * d.dp_k);  // m beta / rho0
    const bool ok = collide(d, a.bnd, make_float3(xp.x, xp.y, xp.z), dp);
    if (!ok) atomicOr(a.flags + s, PBF_FLAG_COLLISION_LIMIT);
    const float4 xn = make_float4(xp.x + dp.x, xp.y + dp.y, xp.z + dp.z, 0.f);
    xo[i] = xn;
    if (last) {
        const float4 xo_ = a.xold[i];
        const float4 vn =
            make_float4(d.inv_dt * (xn.x - xo_.x), d.inv_dt * (xn.y - xo_.y), d.inv_dt * (xn.z - xo_.z), 0.f);
        vo[i] = vn;
        a.xv[2ull * i] = xn;  // the post passes gather x and v together
        a.xv[2ull * i + 1] = vn;
        a.id[i] = a.id_tmp[i];  // ids follow the particles into sorted order
    }
}

// delta-p with s_corr (calcPositionUpdateCUDA cached, pbf_position_update.cu:131-188),
// boundary response (pbf_response_collision.cu:12-66) and x += dp
// (updateInterimPositionCUDA, pbf_constraint.cu:335-345), written to a second
// buffer so neighbours still read the old positions.  On the last iteration
// the velocity update (updateVelocityCUDA, pbf_update.cu:25-39) is fused in:
// v = (x_new - x_old) / dt, written with x_new to the particle phase.
template <int kChunk, bool LAMW>
__global__ void __launch_bounds__(512, 2) k_dp(StepArgs a, const float4 *__restrict__ xc, float4 *__restrict__ xo,
                                               float4 *__restrict__ vo, int last)
{
    TILE_LOOP_BEGIN
    const SceneDesc d = a.scenes[s];
    const uint32_t base = a.offsets[d.c_off];
    const uint32_t live = a.offsets[d.c_off + d.ncell] - base;
    if (last && local == 0) a.scene_num[s] = live;
    if (local >= live) continue;
    const uint32_t i = d.p_off + local;
    const float4 xp = xc[i];
    const float li = LAMW ? xp.w : a.lam[i];
    float3 sum;
    if (d.tensile_mode == PBF_TENSILE_REFERENCE)
        sum = dp_sum<kChunk, kScorrReference, LAMW>(a, d, xc, i, xp, li);
    else if (d.tensile_mode == PBF_TENSILE_TEXTBOOK && d.scorr_n == 4)
        sum = dp_sum<kChunk, kScorrTextbook4, LAMW>(a, d, xc, i, xp, li);
    else if (d.tensile_mode == PBF_TENSILE_TEXTBOOK)
        sum = dp_sum<kChunk, kScorrTextbook, LAMW>(a, d, xc, i, xp, li);
    else
        sum = dp_sum<kChunk, kScorrOff, LAMW>(a, d, xc, i, xp, li);
    dp_finish(a, d, s, i, xp, sum, xo, vo, last);
    TILE_LOOP_END
}

// iters == 0: positions stay at the prediction; v from the velocity update.
__global__ void __launch_bounds__(512) k_finalize(StepArgs a, float4 *__restrict__ vo)
{
    TILE_LOOP_BEGIN
    const SceneDesc d = a.scenes[s];
    const uint32_t base = a.offsets[d.c_off];
    const uint32_t live = a.offsets[d.c_off + d.ncell] - base;
    if (local == 0) a.scene_num[s] = live;
    if (local >= live) continue;
    const uint32_t i = d.p_off + local;
    const float4 xn = a.xa[i];
    const float4 xo_ = a.xold[i];
    a.x[i] = xn;
    const float4 vn = make_float4(d.inv_dt * (xn.x - xo_.x), d.inv_dt * (xn.y - xo_.y), d.inv_dt * (xn.z - xo_.z), 0.f);
    vo[i] = vn;
    a.xv[2ull * i] = xn;
    a.xv[2ull * i + 1] = vn;
    a.id[i] = a.id_tmp[i];
    TILE_LOOP_END
}

// Vorticity, pass 1 (calcVorticityCUDA, pbf_vorticity_confinement.cu:87-115):
// omega_i = m/rho0 * sum_j (v_j - v_i) x r_hat * W'(r).  REF: the reference's
// uncapped 27-cell walk, with h passed where 1/h is expected
// (pbf_vorticity_confinement.cu:28); otherwise the textbook kernel over the
// step's neighbour list.  Each form is its own kernel (scenes of the other
// forms are skipped) so the list form keeps a lean register allocation.
template <bool REF, bool L16>
__global__ void __launch_bounds__(512) k_vort_omega(StepArgs a, const float4 *__restrict__ vs)
{
    TILE_LOOP_BEGIN
    const SceneDesc d = a.scenes[s];
    if (d.vort_mode != (REF ? PBF_VORTICITY_REFERENCE : PBF_VORTICITY_TEXTBOOK)) continue;
    if (!REF && (d.list16 != 0) != L16) continue;  // the other list format's instance
    const uint32_t base = a.offsets[d.c_off];
    const uint32_t live = a.offsets[d.c_off + d.ncell] - base;
    if (local >= live) continue;
    const uint32_t i = d.p_off + local;
    const float4 xi = a.x[i], vi = vs[i];
    const float kh = REF ? d.h : d.inv_h;
    const float4 *__restrict__ x = a.x;
    float w0 = 0.f, w1 = 0.f, w2 = 0.f;
    auto pair = [&](const float4 &xj, const float4 &vj) {
        const float p0 = xj.x - xi.x, p1 = xj.y - xi.y, p2 = xj.z - xi.z;
        const float r2 = p0 * p0 + p1 * p1 + p2 * p2;
        if (r2 > 0.f) {
            const float inv_r = rsqrtf(r2);
            const float v0 = vj.x - vi.x, v1 = vj.y - vi.y, v2 = vj.z - vi.z;
            const float wd = wspiky_d(r2 * inv_r, kh) * inv_r;
            w0 += (v1 * p2 - v2 * p1) * wd;
            w1 += (v2 * p0 - v0 * p2) * wd;
            w2 += (v0 * p1 - v1 * p0) * wd;
        }
    };
    // the walk form gathers x and then, for a pair at r > 0, v
    auto use = [&](uint32_t j) {
        const float4 xj = __ldg(x + j);
        const float p0 = xj.x - xi.x, p1 = xj.y - xi.y, p2 = xj.z - xi.z;
        if (p0 * p0 + p1 * p1 + p2 * p2 > 0.f) pair(xj, __ldg(vs + j));
    };
    // the list form gathers both with one 256-bit load of the (x, v) record
    auto use_rec = [&](uint32_t j) {
        float4 xj, vj;
        ld_rec(a.xv + 2ull * j, xj, vj);
        pair(xj, vj);
    };
    if (REF) {  // the kernel scaled by h reaches the whole 27-cell block
        walk27_batched(
            d, a.offsets, d.p_off - base, xi,
            [&](uint32_t j) -> bool {
                const float4 xj = __ldg(x + j);
                const float p0 = xj.x - xi.x, p1 = xj.y - xi.y, p2 = xj.z - xi.z;
                return p0 * p0 + p1 * p1 + p2 * p2 > 0.f;
            },
            use);
    } else {
        list_walk_any<4>(L16, list_of(a.nbr, i), a.nbr_stride, a.nnb[i], d.p_off, use_rec);
    }
    const float mr = d.m * d.inv_rho0;
    const float4 wi = make_float4(mr * w0, mr * w1, mr * w2, 0.f);
    a.w[i] = wi;
    // |omega| once per particle, beside the position (xs is free after the
    // reorder): pass 2 gathers both with one load per neighbour
    a.xs[i] = make_float4(xi.x, xi.y, xi.z, sqrtf(wi.x * wi.x + wi.y * wi.y + wi.z * wi.z));
    TILE_LOOP_END
}

// Vorticity, pass 2 (addVorticityConfinementCUDA, pbf_vorticity_confinement.cu:192-222).
template <bool REF, bool L16>
__global__ void __launch_bounds__(512) k_vort_apply(StepArgs a, float4 *__restrict__ vs)
{
    TILE_LOOP_BEGIN
    const SceneDesc d = a.scenes[s];
    if (d.vort_mode != (REF ? PBF_VORTICITY_REFERENCE : PBF_VORTICITY_TEXTBOOK)) continue;
    if (!REF && (d.list16 != 0) != L16) continue;  // the other list format's instance
    const uint32_t base = a.offsets[d.c_off];
    const uint32_t live = a.offsets[d.c_off + d.ncell] - base;
    if (local >= live) continue;
    const uint32_t i = d.p_off + local;
    const float4 xi = a.x[i];
    const float kh = REF ? d.h : d.inv_h;
    const float sgn = REF ? 1.f : -1.f;
    const float4 *__restrict__ x = a.x;
    const float4 *__restrict__ w = a.w;
    const uint32_t lb = (!REF && L16) ? d.p_off : 0u;  // use(j): j counts from lb
    const float4 *__restrict__ xw = a.xs + lb;          // (x_j, |omega_j|), stored by pass 1
    float n0 = 0.f, n1 = 0.f, n2 = 0.f;
    auto use = [&](uint32_t j) {
        const float4 xj = __ldg(xw + j);
        const float p0 = xj.x - xi.x, p1 = xj.y - xi.y, p2 = xj.z - xi.z;
        const float r2 = p0 * p0 + p1 * p1 + p2 * p2;
        if (r2 > 0.f) {
            const float inv_r = rsqrtf(r2);
            const float wl = xj.w;
            const float f = sgn * wl * wspiky_d(r2 * inv_r, kh) * inv_r;
            n0 += f * p0;
            n1 += f * p1;
            n2 += f * p2;
        }
    };
    if (REF) {
        walk27_batched(
            d, a.offsets, d.p_off - base, xi,
            [&](uint32_t j) -> bool {
                const float4 xj = __ldg(x + j);
                const float p0 = xj.x - xi.x, p1 = xj.y - xi.y, p2 = xj.z - xi.z;
                return p0 * p0 + p1 * p1 + p2 * p2 > 0.f;
            },
            use);
    } else {
        // quads of 4: fewer registers, more warps (measured)
        list_walk_any<4>(L16, list_of(a.nbr, i), a.nbr_stride, a.nnb[i], 0u, use);
    }
    const float4 wi = w[i];
    const float mr = d.m * d.inv_rho0;
    float4 v = vs[i];
    if (REF) {
        if (sqrtf(n0 * n0 + n1 * n1 + n2 * n2) > 0.f) {
            n0 = n0 * d.m * d.inv_rho0;
            n1 = n1 * d.m * d.inv_rho0;
            n2 = n2 * d.m * d.inv_rho0;
            const float ln = sqrtf(n0 * n0 + n1 * n1 + n2 * n2);
            n0 /= ln; n1 /= ln; n2 /= ln;
            const float c0 = n1 * wi.z - n2 * wi.y, c1 = n2 * wi.x - n0 * wi.z, c2 = n0 * wi.y - n1 * wi.x;
            v.x = v.x + d.vort_eps * c0 / d.inv_rho0 * d.dt;
            v.y = v.y + d.vort_eps * c1 / d.inv_rho0 * d.dt;
            v.z = v.z + d.vort_eps * c2 / d.inv_rho0 * d.dt;
        }
    } else {
        n0 *= mr; n1 *= mr; n2 *= mr;
        const float ln = sqrtf(n0 * n0 + n1 * n1 + n2 * n2);
        if (ln > 0.f) {
            n0 /= ln; n1 /= ln; n2 /= ln;
            const float c0 = n1 * wi.z - n2 * wi.y, c1 = n2 * wi.x - n0 * wi.z, c2 = n0 * wi.y - n1 * wi.x;
            v.x = v.x + d.dt * d.vort_eps * c0;
            v.y = v.y + d.dt * d.vort_eps * c1;
            v.z = v.z + d.dt * d.vort_eps * c2;
        }
    }
    vs[i] = v;
    TILE_LOOP_END
}

// XSPH (calcXSPHCUDA, pbf_xsph.cu:84-113): v_i += c m/rho0 sum_j (v_j - v_i) W(r_ij),
// NaN guard.  WALK: the reference's uncapped 27-cell walk (scenes with
// PBF_XSPH_WALK); otherwise over the step's neighbour list (scenes with
// PBF_XSPH_LIST), also copying vs to vo for scenes without XSPH.
template <bool WALK, bool L16>
__global__ void __launch_bounds__(512) k_xsph(StepArgs a, const float4 *__restrict__ vs, float4 *__restrict__ vo)
{
    TILE_LOOP_BEGIN
    const SceneDesc d = a.scenes[s];
    if ((d.xsph_mode == PBF_XSPH_WALK) != WALK) continue;
    if (!WALK && (d.list16 != 0) != L16) continue;  // the other list format's instance
    const uint32_t base = a.offsets[d.c_off];
    const uint32_t live = a.offsets[d.c_off + d.ncell] - base;
    if (local >= live) continue;
    const uint32_t i = d.p_off + local;
    const float4 xi = a.x[i], vi = vs[i];
    if (!WALK && d.xsph_mode == PBF_XSPH_OFF) {  // scene without XSPH in a batch that has some
        vo[i] = vi;
        continue;
    }
    const float inv_h = d.inv_h, alpha6 = d.alpha6;
    const float4 *__restrict__ x = a.x;
    const uint32_t lb = (!WALK && L16) ? d.p_off : 0u;  // use(j): j counts from lb
    const float4 *__restrict__ xb = x + lb;
    const float4 *__restrict__ vb = vs + lb;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    const float ih2 = inv_h * inv_h;
    auto use = [&](uint32_t j) {
        const float4 xj = __ldg(xb + j);
        const float p0 = xj.x - xi.x, p1 = xj.y - xi.y, p2 = xj.z - xi.z;
        // Wpoly6 from r^2 (q^2 = r^2 / h^2 instead of (|r| / h)^2: no square
        // root per pair; the two differ by rounding only)
        const float q2 = (p0 * p0 + p1 * p1 + p2 * p2) * ih2;
        const float t = 1.f - q2;
        const float W = (q2 <= 1.f) ? alpha6 * t * t * t : 0.f;
        const float4 vj = __ldg(vb + j);
        s0 += (vj.x - vi.x) * W;
        s1 += (vj.y - vi.y) * W;
        s2 += (vj.z - vi.z) * W;
    };
    if (WALK) {
        // W = 0 beyond h: those candidates add nothing (a non-finite velocity
        // of a non-neighbour is no longer folded into the sum; such particles
        // raise PBF_FLAG_NONFINITE in the next step's prediction)
        const float rcut2 = d.h2 * 1.0001f;
        walk27_batched(
            d, a.offsets, d.p_off - base, xi,
            [&](uint32_t j) -> bool {
                const float4 xj = __ldg(x + j);
                const float p0 = xj.x - xi.x, p1 = xj.y - xi.y, p2 = xj.z - xi.z;
                return p0 * p0 + p1 * p1 + p2 * p2 <= rcut2;
            },
            use);
    } else {
        if (L16)
            list_walk16(list_of(a.nbr, i), a.nbr_stride, a.nnb[i], 0u, use);
        else
            list_walk_ahead2(list_of(a.nbr, i), a.nbr_stride, a.nnb[i], use);
    }
    float4 out = vi;
    if (!(isnan(s0) || isnan(s1) || isnan(s2))) {
        const float c = d.xsph_c * d.m * d.inv_rho0;
        out.x = vi.x + c * s0;
        out.y = vi.y + c * s1;
        out.z = vi.z + c * s2;
    }
    vo[i] = out;
    TILE_LOOP_END
}

__global__ void __launch_bounds__(512) k_unpack(StepArgs a, const uint32_t *__restrict__ pack_off,
                                                const float *__restrict__ sx, const float *__restrict__ sv)
{
    TILE_LOOP_BEGIN
    const uint32_t n = a.scene_num[s];
    if (local >= n) continue;
    const uint64_t q = (uint64_t)pack_off[s] + local;
    const uint32_t i = a.scenes[s].p_off + local;
    a.x[i] = make_float4(sx[3 * q], sx[3 * q + 1], sx[3 * q + 2], 0.f);
    a.v[i] = sv ? make_float4(sv[3 * q], sv[3 * q + 1], sv[3 * q + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    a.id[i] = local;  // a whole-scene upload numbers the particles afresh
    if (local == 0) a.next_id[s] = n;
    TILE_LOOP_END
}

__global__ void __launch_bounds__(512) k_pack(StepArgs a, const uint32_t *__restrict__ pack_off,
                                              float *__restrict__ dx, float *__restrict__ dv)
{
    TILE_LOOP_BEGIN
    const uint32_t n = a.scene_num[s];
    if (local >= n) continue;
    const uint64_t q = (uint64_t)pack_off[s] + local;
    const uint32_t i = a.scenes[s].p_off + local;
    if (dx) {
        const float4 t = a.x[i];
        dx[3 * q] = t.x;
        dx[3 * q + 1] = t.y;
        dx[3 * q + 2] = t.z;
    }
    if (dv) {
        const float4 t = a.v[i];
        dv[3 * q] = t.x;
        dv[3 * q + 1] = t.y;
        dv[3 * q + 2] = t.z;
    }
    TILE_LOOP_END
}

__global__ void k_set_u32(uint32_t *dst, uint32_t value) { *dst = value; }

// Packed offsets of the active scenes from their live counts, on the device:
// pack_off[active[k]] = the counts of active[0..k) summed, counts[k] = the
// count of active[k] (k-th active scene in slot order).  One block.
__global__ void __launch_bounds__(1024) k_pack_offsets(const uint32_t *__restrict__ active, uint32_t n_active,
                                                       const uint32_t *__restrict__ scene_num,
                                                       uint32_t *__restrict__ pack_off, uint32_t *__restrict__ counts)
{
    __shared__ uint32_t ws[32];
    __shared__ uint32_t carry;
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    if (t == 0) carry = 0;
    __syncthreads();
    for (uint32_t k0 = 0; k0 < n_active; k0 += blockDim.x) {
        const uint32_t k = k0 + t;
        const uint32_t id = k < n_active ? active[k] : 0u;
        const uint32_t c = k < n_active ? scene_num[id] : 0u;
        const uint32_t incl = warp_incl_scan(c);
        if (lane == 31) ws[warp] = incl;
        __syncthreads();
        if (warp == 0) ws[lane] = warp_incl_scan(lane < (blockDim.x >> 5) ? ws[lane] : 0u);
        __syncthreads();
        const uint32_t before = carry + (warp ? ws[warp - 1] : 0u) + incl - c;
        if (k < n_active) {
            pack_off[id] = before;
            counts[k] = c;
        }
        __syncthreads();
        if (t == blockDim.x - 1) carry = before + c;
        __syncthreads();
    }
}

__global__ void k_aos3_to_f4(const float *__restrict__ src, float4 *__restrict__ dst, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], 0.f);
}

__global__ void k_f4_to_aos3(const float4 *__restrict__ src, float *__restrict__ dst, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float4 v = src[i];
        dst[3 * i] = v.x;
        dst[3 * i + 1] = v.y;
        dst[3 * i + 2] = v.z;
    }
}

}  // namespace

// The lambda / delta-p variants by neighbour chunk, selected at run time.
template <int CH>
struct PassFns {
    static const void *lambda() { return (const void *)k_lambda<CH, true>; }
    static const void *dp() { return (const void *)k_dp<CH, true>; }
    static void launch_lambda(const StepArgs &a, const LaunchShape &sh, float4 *cur, bool lamw, cudaStream_t st)
    {
        if (lamw)
            k_lambda<CH, true><<<sh.grid_lambda, sh.tile, 0, st>>>(a, cur);
        else
            k_lambda<CH, false><<<sh.grid_lambda, sh.tile, 0, st>>>(a, cur);
    }
    // lamw: lambda in .w of cur (iterations >= 1); iteration 0 reads it from lam
    static void launch_dp(const StepArgs &a, const LaunchShape &sh, const float4 *cur, float4 *out, float4 *vo,
                          int last, bool lamw, cudaStream_t st)
    {
        if (lamw)
            k_dp<CH, true><<<sh.grid_dp, sh.tile, 0, st>>>(a, cur, out, vo, last);
        else
            k_dp<CH, false><<<sh.grid_dp, sh.tile, 0, st>>>(a, cur, out, vo, last);
    }
};

#define PBF_PASS_DISPATCH(chunk, CALL) \
    if ((chunk) == 4) PassFns<4>::CALL; \
    else PassFns<8>::CALL;

// Resident blocks per SM of each kernel at a tile size (cached per device,
// tile and chunk: the step asks for its launch shape every time it runs).
Occupancy occupancy(uint32_t tile, uint32_t chunk)
{
    static std::mutex mu;
    static std::map<std::tuple<int, uint32_t, uint32_t>, Occupancy> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(dev, tile, chunk);
    {
        std::lock_guard<std::mutex> lk(mu);
        const auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    auto occ_b = [](const void *fn, uint32_t block) -> uint32_t {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, (int)block, 0);
        return b > 0 ? (uint32_t)b : 1u;
    };
    auto occ = [&](const void *fn) { return occ_b(fn, tile); };
    auto mn = [](uint32_t a, uint32_t b) { return a < b ? a : b; };
    Occupancy o;
    o.light = mn(mn(mn(occ((const void *)k_predict_hash<false>), occ((const void *)k_predict_hash<true>)),
                    occ((const void *)k_scatter)),
                 mn(mn(occ((const void *)k_rank_reorder), mn(occ((const void *)k_gather<false>),
                                                             occ((const void *)k_gather<true>))),
                    occ((const void *)k_finalize)));
    o.cells = occ_b((const void *)k_rank_cells, kCellTileMax);
    o.split = occ_b((const void *)k_neighbors_split, 256);
    o.nb = occ((const void *)k_neighbors_lambda<false>);
    cudaFuncSetAttribute((const void *)k_neighbors_lambda<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kNbSmemMax);
    const bool c4 = chunk == 4;
    o.lambda = occ(c4 ? PassFns<4>::lambda() : PassFns<8>::lambda());
    o.dp = occ(c4 ? PassFns<4>::dp() : PassFns<8>::dp());
    o.omega = mn(occ((const void *)k_vort_omega<false, false>), occ((const void *)k_vort_omega<false, true>));
    o.apply = mn(occ((const void *)k_vort_apply<false, false>), occ((const void *)k_vort_apply<false, true>));
    o.xsph = mn(occ((const void *)k_xsph<false, false>), occ((const void *)k_xsph<false, true>));
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = o;
    return o;
}

void launch_aos3_to_f4(const float *src, float4 *dst, uint32_t n, cudaStream_t st)
{
    if (n) k_aos3_to_f4<<<(n + 255) / 256, 256, 0, st>>>(src, dst, n);
}

void launch_f4_to_aos3(const float4 *src, float *dst, uint32_t n, cudaStream_t st)
{
    if (n) k_f4_to_aos3<<<(n + 255) / 256, 256, 0, st>>>(src, dst, n);
}

void launch_set_u32(uint32_t *dst, uint32_t value, cudaStream_t st) { k_set_u32<<<1, 1, 0, st>>>(dst, value); }

void launch_pack_offsets(const uint32_t *active, uint32_t n_active, const uint32_t *scene_num, uint32_t *pack_off,
                         uint32_t *counts, cudaStream_t st)
{
    if (n_active) k_pack_offsets<<<1, 1024, 0, st>>>(active, n_active, scene_num, pack_off, counts);
}

void launch_unpack(const StepArgs &a, const LaunchShape &sh, const uint32_t *pack_off, const float *src_x,
                   const float *src_v, cudaStream_t st)
{
    k_unpack<<<sh.grid, sh.tile, 0, st>>>(a, pack_off, src_x, src_v);
}

void launch_pack(const StepArgs &a, const LaunchShape &sh, const uint32_t *pack_off, float *dst_x, float *dst_v,
                 cudaStream_t st)
{
    k_pack<<<sh.grid, sh.tile, 0, st>>>(a, pack_off, dst_x, dst_v);
}

__global__ void k_set_packed_in(PackedIn *dst, const float *x, const float *v) { *dst = PackedIn{x, v}; }

void launch_set_packed_in(PackedIn *dst, const float *x, const float *v, cudaStream_t st)
{
    k_set_packed_in<<<1, 1, 0, st>>>(dst, x, v);
}

uint32_t enqueue_step(const StepArgs &a, const LaunchShape &sh, int iters, uint32_t post,
                      cudaStream_t st, StepHook *hook, bool packed)
{
    uint32_t nl = 0;
    const dim3 g(sh.grid), b(sh.tile);
#define PBF_LAUNCHED(name)                \
    do {                                  \
        ++nl;                             \
        if (hook) hook->launched(name);   \
    } while (0)
    if (packed)
        k_predict_hash<true><<<g, b, 0, st>>>(a);
    else
        k_predict_hash<false><<<g, b, 0, st>>>(a);
    PBF_LAUNCHED("k_predict_hash");
    if (sh.scan_grid == 0) {  // small table: one block
        switch (sh.scan_rounds) {  // rounds of 1024 cells held in registers
#define PBF_SCAN_ROUNDS(r) \
    case r: k_scan_single_reg<r><<<1, 1024, 0, st>>>(a); break;
        PBF_SCAN_ROUNDS(1) PBF_SCAN_ROUNDS(2) PBF_SCAN_ROUNDS(3) PBF_SCAN_ROUNDS(4)
        PBF_SCAN_ROUNDS(5) PBF_SCAN_ROUNDS(6) PBF_SCAN_ROUNDS(7) PBF_SCAN_ROUNDS(8)
        PBF_SCAN_ROUNDS(9) PBF_SCAN_ROUNDS(10) PBF_SCAN_ROUNDS(11) PBF_SCAN_ROUNDS(12)
        PBF_SCAN_ROUNDS(13) PBF_SCAN_ROUNDS(14) PBF_SCAN_ROUNDS(15) PBF_SCAN_ROUNDS(16)
#undef PBF_SCAN_ROUNDS
        default: k_scan_single<<<1, 1024, 0, st>>>(a); break;
        }
        PBF_LAUNCHED("k_scan_single");
    } else {
        k_scan_reduce<<<sh.scan_grid, 256, 0, st>>>(a);
        PBF_LAUNCHED("k_scan_reduce");
        k_scan_spine<<<1, 1024, 0, st>>>(a);
        PBF_LAUNCHED("k_scan_spine");
        k_scan_down<<<sh.scan_grid, 256, 0, st>>>(a);
        PBF_LAUNCHED("k_scan_down");
    }
    k_scatter<<<g, b, 0, st>>>(a);
    PBF_LAUNCHED("k_scatter");
    if (sh.small) {
        k_rank_reorder<<<g, b, 0, st>>>(a);
        PBF_LAUNCHED("k_rank_reorder");
    } else {
        k_rank_cells<<<sh.grid_cells, sh.cell_tile, 0, st>>>(a);
        PBF_LAUNCHED("k_rank_cells");
    }
    k_dense_sort<<<sh.grid, kRadixThreads, 0, st>>>(a);
    PBF_LAUNCHED("k_dense_sort");
    if (packed)
        k_gather<true><<<g, b, 0, st>>>(a);
    else
        k_gather<false><<<g, b, 0, st>>>(a);
    PBF_LAUNCHED("k_gather");
    if (sh.small) {
        k_neighbors_split<<<sh.grid_split, 256, 0, st>>>(a, sh.tile);
        PBF_LAUNCHED("k_neighbors_split");
    } else {
        if (sh.nb_smem)
            k_neighbors_lambda<true><<<sh.grid_nb, b, sh.nb_smem, st>>>(a);
        else
            k_neighbors_lambda<false><<<sh.grid_nb, b, 0, st>>>(a);
        PBF_LAUNCHED("k_neighbors_lambda");
    }
    const bool xsph = (post & (kPostXsphWalk | kPostXsphList)) != 0;
    float4 *vfinal = xsph ? a.vt : a.v;
    float4 *cur = a.xa, *nxt = a.xb;
    for (int it = 0; it < iters; ++it) {
        if (it > 0) {
            PBF_PASS_DISPATCH(sh.chunk, launch_lambda(a, sh, cur, !sh.small, st));
            PBF_LAUNCHED("k_lambda");
        }
        const bool last = (it == iters - 1);
        float4 *out = last ? a.x : nxt;
        PBF_PASS_DISPATCH(sh.chunk,
                          launch_dp(a, sh, cur, out, last ? vfinal : nullptr, last ? 1 : 0, it > 0 && !sh.small, st));
        PBF_LAUNCHED("k_dp");
        float4 *t = cur;
        cur = nxt;
        nxt = t;
    }
    if (iters <= 0) {
        k_finalize<<<g, b, 0, st>>>(a, vfinal);
        PBF_LAUNCHED("k_finalize");
    }
    // omega of every form before any apply: both forms read final positions
    // and velocities only
    // the list forms run one instance per list format present (each skips
    // the other format's scenes): one instance per format keeps its
    // registers, and so its occupancy, to that format's loop
    const bool l16 = (post & kPostList16) != 0, l32 = (post & kPostList32) != 0;
    if (post & kPostVortTextbook) {
        if (l32) {
            k_vort_omega<false, false><<<sh.grid_omega, b, 0, st>>>(a, vfinal);
            PBF_LAUNCHED("k_vort_omega");
        }
        if (l16) {
            k_vort_omega<false, true><<<sh.grid_omega, b, 0, st>>>(a, vfinal);
            PBF_LAUNCHED("k_vort_omega");
        }
    }
    if (post & kPostVortReference) {
        k_vort_omega<true, false><<<sh.grid_omega, b, 0, st>>>(a, vfinal);
        PBF_LAUNCHED("k_vort_omega_walk");
    }
    if (post & kPostVortTextbook) {
        if (l32) {
            k_vort_apply<false, false><<<sh.grid_apply, b, 0, st>>>(a, vfinal);
            PBF_LAUNCHED("k_vort_apply");
        }
        if (l16) {
            k_vort_apply<false, true><<<sh.grid_apply, b, 0, st>>>(a, vfinal);
            PBF_LAUNCHED("k_vort_apply");
        }
    }
    if (post & kPostVortReference) {
        k_vort_apply<true, false><<<sh.grid_apply, b, 0, st>>>(a, vfinal);
        PBF_LAUNCHED("k_vort_apply_walk");
    }
    if (post & kPostXsphList) {
        if (l32) {
            k_xsph<false, false><<<sh.grid_xsph, b, 0, st>>>(a, a.vt, a.v);
            PBF_LAUNCHED("k_xsph");
        }
        if (l16) {
            k_xsph<false, true><<<sh.grid_xsph, b, 0, st>>>(a, a.vt, a.v);
            PBF_LAUNCHED("k_xsph");
        }
    }
    if (post & kPostXsphWalk) {
        k_xsph<true, false><<<sh.grid_xsph, b, 0, st>>>(a, a.vt, a.v);
        PBF_LAUNCHED("k_xsph_walk");
    }
#undef PBF_LAUNCHED
    return nl;
}

}  // namespace pbf103
