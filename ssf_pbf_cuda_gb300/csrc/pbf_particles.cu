// Particle-set operations beside the solver step: stable particle ids and
// order restore, the reference's arrangement generators evaluated on the
// device, and a device-side emitter.  Appends read the live count on the
// device and are committed by a one-thread kernel, so none of them waits
// for the host.
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

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

// --------------------------------------------------------- arrangements --

// Everything a device thread needs to place point k of an arrangement.
// Counts and per-arrangement constants come from the host, computed with
// the reference's own float / double expressions.
struct ArrangePlan {
    int32_t kind;
    uint32_t count;
    float base[3];     // point 0 before offsets (volume / line: origin)
    float sp;          // spacing
    // volume: n[0..2] = x, y, z counts (z outermost)
    // rectangle: n[0] = fast count along axis fa, n[1] = slow count along sa
    // cylinder: n[0] = points per ring, n[1] = rings
    uint32_t n[3];
    int32_t fa, sa;    // rectangle: component of the fast / slow offset
    float dir[3];      // line: normalize(end - origin) * space
    float radius, theta_hat;
    int32_t hax, cax, sax;  // cylinder: components of h, r cos, r sin
};

namespace {

// static_cast<int>(range / space + epsilon * 10.0) + 1, pbf_arrangement.h:85-90
int axis_count(float range, float space)
{
    const float q = range / space;
    return static_cast<int>((double)q + std::numeric_limits<double>::epsilon() * 10.0) + 1;
}

pbf_status plan_arrangement(const pbf_arrangement *a, ArrangePlan *P)
{
    if (!a || !(a->space > 0.f) || !std::isfinite(a->space)) return PBF_ERROR_INVALID_ARGUMENT;
    std::memset(P, 0, sizeof(*P));
    P->kind = a->kind;
    P->sp = a->space;
    uint64_t count = 0;
    switch (a->kind) {
    case PBF_ARRANGE_VOLUME: {  // cartesian_volume, pbf_arrangement.h:82-99
        const int nx = axis_count(a->end[0] - a->origin[0], a->space);
        const int ny = axis_count(a->end[1] - a->origin[1], a->space);
        const int nz = axis_count(a->end[2] - a->origin[2], a->space);
        if (nx > 0 && ny > 0 && nz > 0) count = (uint64_t)nx * ny * nz;
        P->n[0] = nx > 0 ? nx : 0;
        P->n[1] = ny > 0 ? ny : 0;
        P->n[2] = nz > 0 ? nz : 0;
        for (int c = 0; c < 3; ++c) P->base[c] = a->origin[c];
        break;
    }
    case PBF_ARRANGE_RECTANGLE: {  // cartesian_rectangle, pbf_arrangement.h:123-163
        const float o0 = a->origin[0], o1 = a->origin[1];
        const int c0 = axis_count(a->end[0] - o0, a->space);  // first 2-D component's count
        const int c1 = axis_count(a->end[1] - o1, a->space);
        int nf, ns;
        if (a->axis == 0) {  // (axis_value, o.x, o.y) + (0, s*y, s*z); z outer, y inner
            P->base[0] = a->axis_value; P->base[1] = o0; P->base[2] = o1;
            P->fa = 1; P->sa = 2; nf = c0; ns = c1;
        } else if (a->axis == 1) {  // (o.y, axis_value, o.x) + (s*x, 0, s*z); z (from c0) outer, x (from c1) inner
            P->base[0] = o1; P->base[1] = a->axis_value; P->base[2] = o0;
            P->fa = 0; P->sa = 2; nf = c1; ns = c0;
        } else if (a->axis == 2) {  // (o.x, o.y, axis_value) + (s*x, s*y, 0); x (from c0) outer, y (from c1) inner
            P->base[0] = o0; P->base[1] = o1; P->base[2] = a->axis_value;
            P->fa = 1; P->sa = 0; nf = c1; ns = c0;
        } else {
            return PBF_ERROR_INVALID_ARGUMENT;
        }
        if (nf > 0 && ns > 0) count = (uint64_t)nf * ns;
        P->n[0] = nf > 0 ? nf : 0;
        P->n[1] = ns > 0 ? ns : 0;
        break;
    }
    case PBF_ARRANGE_LINE: {  // cartesian_line_inclusive, pbf_arrangement.h:8-18 (GLM length / normalize)
        const float d0 = a->end[0] - a->origin[0], d1 = a->end[1] - a->origin[1], d2 = a->end[2] - a->origin[2];
        const float dot = d0 * d0 + d1 * d1 + d2 * d2;
        const float len = std::sqrt(dot);
        if (!(dot > 0.f)) return PBF_ERROR_INVALID_ARGUMENT;  // normalize of a zero vector
        const float inv = 1.f / std::sqrt(dot);
        P->dir[0] = (d0 * inv) * a->space;
        P->dir[1] = (d1 * inv) * a->space;
        P->dir[2] = (d2 * inv) * a->space;
        const int n = static_cast<int>(std::floor(len / a->space)) + 1;
        count = n > 0 ? (uint64_t)n : 0;
        for (int c = 0; c < 3; ++c) P->base[c] = a->origin[c];
        break;
    }
    case PBF_ARRANGE_CYLINDER: {  // cartesian_cylinder, pbf_arrangement.h:212-244
        if (!(a->radius > 0.f) || !(a->space < 2.f * a->radius)) return PBF_ERROR_INVALID_ARGUMENT;
        const float pi = 3.14159265358979323846264338327950288f;
        const float theta = (float)(2.0 * std::asin(a->space / (2.0 * a->radius)));
        const float n = (float)std::floor(2.0 * pi / theta);
        const float theta_hat = (float)(2.0 * pi / n);
        uint32_t rings = 0;
        for (float h = 0.f; h < a->height; h += a->space) {
            if (++rings > (1u << 24)) return PBF_ERROR_INVALID_ARGUMENT;
        }
        const float o0 = a->origin[0], o1 = a->origin[1];
        if (a->axis == 0) {  // (axis_value, o.x, o.y) + (h, r cos, r sin)
            P->base[0] = a->axis_value; P->base[1] = o0; P->base[2] = o1;
            P->hax = 0; P->cax = 1; P->sax = 2;
        } else if (a->axis == 1) {  // (o.y, axis_value, o.x) + (r sin, h, r cos)
            P->base[0] = o1; P->base[1] = a->axis_value; P->base[2] = o0;
            P->hax = 1; P->cax = 2; P->sax = 0;
        } else if (a->axis == 2) {  // (o.x, o.y, axis_value) + (r cos, r sin, h)
            P->base[0] = o0; P->base[1] = o1; P->base[2] = a->axis_value;
            P->hax = 2; P->cax = 0; P->sax = 1;
        } else {
            return PBF_ERROR_INVALID_ARGUMENT;
        }
        P->n[0] = (uint32_t)n;
        P->n[1] = rings;
        P->radius = a->radius;
        P->theta_hat = theta_hat;
        count = (uint64_t)P->n[0] * rings;
        break;
    }
    default:
        return PBF_ERROR_INVALID_ARGUMENT;
    }
    if (count >= (1ull << 31)) return PBF_ERROR_CAPACITY;
    P->count = (uint32_t)count;
    return PBF_SUCCESS;
}

// Point k of the arrangement, in the reference's loop order, with the same
// float operations (no contraction: explicit round-to-nearest intrinsics).
__device__ float3 plan_point(const ArrangePlan &P, uint32_t k)
{
    float off[3] = {0.f, 0.f, 0.f};
    switch (P.kind) {
    case PBF_ARRANGE_VOLUME: {
        const uint32_t x = k % P.n[0], t = k / P.n[0];
        const uint32_t y = t % P.n[1], z = t / P.n[1];
        off[0] = __fmul_rn(P.sp, (float)x);
        off[1] = __fmul_rn(P.sp, (float)y);
        off[2] = __fmul_rn(P.sp, (float)z);
        break;
    }
    case PBF_ARRANGE_RECTANGLE:
        off[P.fa] = __fmul_rn(P.sp, (float)(k % P.n[0]));
        off[P.sa] = __fmul_rn(P.sp, (float)(k / P.n[0]));
        break;
    case PBF_ARRANGE_LINE:
        off[0] = __fmul_rn(P.dir[0], (float)k);
        off[1] = __fmul_rn(P.dir[1], (float)k);
        off[2] = __fmul_rn(P.dir[2], (float)k);
        break;
    default: {  // cylinder: h accumulated ring by ring as the reference's loop does
        const uint32_t ring = k / P.n[0], i = k % P.n[0];
        float h = 0.f;
        for (uint32_t r = 0; r < ring; ++r) h = __fadd_rn(h, P.sp);
        const float ang = __fmul_rn((float)i, P.theta_hat);
        off[P.hax] = h;
        off[P.cax] = __fmul_rn(P.radius, cosf(ang));
        off[P.sax] = __fmul_rn(P.radius, sinf(ang));
        break;
    }
    }
    return make_float3(__fadd_rn(P.base[0], off[0]), __fadd_rn(P.base[1], off[1]), __fadd_rn(P.base[2], off[2]));
}

// ------------------------------------------------------------- kernels --

// Whether a device-side append of n particles proceeds: the emitter rule
// num < max_fill * capacity (compared in double, as pbf_sphere_sim.cpp:386)
// and room for all n.
__device__ __forceinline__ bool fill_ok(uint32_t num, uint32_t capacity, double max_fill)
{
    return (double)num < (double)capacity * max_fill;
}
__device__ __forceinline__ bool fits(uint32_t num, uint32_t n, uint32_t capacity)
{
    return (uint64_t)num + n <= capacity;
}

struct PlanSource {
    ArrangePlan P;
    float4 v0;
    __device__ float4 x(uint32_t k) const
    {
        const float3 p = plan_point(P, k);
        return make_float4(p.x, p.y, p.z, 0.f);
    }
    __device__ float4 v(uint32_t) const { return v0; }
};

struct BufferSource {
    const float4 *px, *pv;
    __device__ float4 x(uint32_t k) const { return px[k]; }
    __device__ float4 v(uint32_t k) const { return pv[k]; }
};

// Copy n source particles after the live ones (x, v, ids); the scene's
// count is committed by k_append_commit in the next launch.
template <class Src>
__global__ void k_append(Src src, Batch::SceneArrays A, uint32_t n, double max_fill)
{
    const uint32_t num = *A.scene_num;
    if (!fill_ok(num, A.capacity, max_fill) || !fits(num, n, A.capacity)) return;
    const uint32_t id0 = *A.next_id;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        A.x[num + k] = src.x(k);
        A.v[num + k] = src.v(k);
        A.id[num + k] = id0 + k;
    }
}

__global__ void k_append_commit(Batch::SceneArrays A, uint32_t n, double max_fill)
{
    const uint32_t num = *A.scene_num;
    if (!fill_ok(num, A.capacity, max_fill)) return;
    if (!fits(num, n, A.capacity)) {
        atomicOr(A.flags, PBF_FLAG_CAPACITY);
        return;
    }
    *A.scene_num = num + n;
    *A.next_id += n;
}

// Pattern points into a plain buffer (an emitter's).
__global__ void k_plan_fill(ArrangePlan P, float4 v0, float4 *x, float4 *v)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < P.count; k += gridDim.x * blockDim.x) {
        const float3 p = plan_point(P, k);
        x[k] = make_float4(p.x, p.y, p.z, 0.f);
        v[k] = v0;
    }
}

// out[idx[g]] = (x, v)[g] for g < n and idx[g] < n_out (AoS float3 output).
__global__ void k_scatter_by_index(const float4 *__restrict__ x, const float4 *__restrict__ v,
                                   const uint32_t *__restrict__ idx, uint32_t n, float *ox, float *ov,
                                   uint32_t n_out)
{
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
        const uint32_t j = idx[g];
        if (j >= n_out) continue;
        if (ox) {
            const float4 t = x[g];
            ox[3ull * j] = t.x;
            ox[3ull * j + 1] = t.y;
            ox[3ull * j + 2] = t.z;
        }
        if (ov) {
            const float4 t = v[g];
            ov[3ull * j] = t.x;
            ov[3ull * j + 1] = t.y;
            ov[3ull * j + 2] = t.z;
        }
    }
}

__global__ void k_assign_ids(uint32_t *dst, const uint32_t *next_id, uint32_t n, int append)
{
    const uint32_t id0 = append ? *next_id : 0u;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) dst[k] = id0 + k;
}

__global__ void k_bump_next_id(uint32_t *next_id, uint32_t n, int append)
{
    *next_id = (append ? *next_id : 0u) + n;
}

uint32_t blocks_for(uint64_t n) { return (uint32_t)std::min<uint64_t>((n + 255) / 256, 4096); }

}  // namespace

void launch_assign_ids(uint32_t *dst, uint32_t *next_id, uint32_t n, bool append, cudaStream_t st)
{
    if (n) k_assign_ids<<<blocks_for(n), 256, 0, st>>>(dst, next_id, n, append ? 1 : 0);
    k_bump_next_id<<<1, 1, 0, st>>>(next_id, n, append ? 1 : 0);
}

// ------------------------------------------------------ batch methods --

static pbf_status append_plan(Batch &b, uint32_t scene, const ArrangePlan &P, float4 v0, double max_fill,
                              cudaStream_t st)
{
    Batch::SceneArrays A;
    pbf_status rc = b.scene_arrays(scene, &A);
    if (rc != PBF_SUCCESS) return rc;
    CK(cudaSetDevice(b.device()));
    if (P.count) k_append<PlanSource><<<blocks_for(P.count), 256, 0, st>>>(PlanSource{P, v0}, A, P.count, max_fill);
    k_append_commit<<<1, 1, 0, st>>>(A, P.count, max_fill);
    CK(cudaGetLastError());
    b.note_append(scene, P.count);
    return PBF_SUCCESS;
}

static pbf_status get_ids(Batch &b, uint32_t scene, uint32_t *ids, uint32_t *num, bool dst_dev, cudaStream_t st)
{
    uint32_t n = 0;
    pbf_status rc = b.get_num(scene, &n, st);
    if (rc != PBF_SUCCESS) return rc;
    if (num) *num = n;
    Batch::SceneArrays A;
    rc = b.scene_arrays(scene, &A);
    if (rc != PBF_SUCCESS) return rc;
    if (n && ids) {
        CK(cudaMemcpyAsync(ids, A.id, 4ull * n, dst_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return PBF_SUCCESS;
}

// out[index[g]] for the live particles; index = the last step's permutation
// (by_perm) or the particle ids.
static pbf_status scatter_out(Batch &b, uint32_t scene, bool by_perm, float *x, float *v, uint32_t n_out,
                              bool dst_dev, cudaStream_t st)
{
    if (by_perm && !b.perm_valid(scene)) return PBF_ERROR_NOT_READY;
    uint32_t n = 0;
    pbf_status rc = b.get_num(scene, &n, st);
    if (rc != PBF_SUCCESS) return rc;
    Batch::SceneArrays A;
    rc = b.scene_arrays(scene, &A);
    if (rc != PBF_SUCCESS) return rc;
    if (!n_out || (!x && !v)) return PBF_SUCCESS;
    const uint32_t *idx = by_perm ? A.perm : A.id;
    float *dx = x, *dv = v;
    void *tmp = nullptr;
    if (!dst_dev) {
        // stage on the device, starting from the caller's values so that
        // entries without a particle keep them
        CK(cudaMalloc(&tmp, 24ull * n_out));
        dx = x ? static_cast<float *>(tmp) : nullptr;
        dv = v ? static_cast<float *>(tmp) + 3ull * n_out : nullptr;
        if (x) CK(cudaMemcpyAsync(dx, x, 12ull * n_out, cudaMemcpyHostToDevice, st));
        if (v) CK(cudaMemcpyAsync(dv, v, 12ull * n_out, cudaMemcpyHostToDevice, st));
    }
    if (n) k_scatter_by_index<<<blocks_for(n), 256, 0, st>>>(A.x, A.v, idx, n, dx, dv, n_out);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && !dst_dev) {
        if (x) e = cudaMemcpyAsync(x, dx, 12ull * n_out, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess && v) e = cudaMemcpyAsync(v, dv, 12ull * n_out, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (tmp) cudaFree(tmp);
    if (e != cudaSuccess) {
        set_last_error("scatter_out", e);
        return PBF_ERROR_CUDA;
    }
    return PBF_SUCCESS;
}

}  // namespace pbf103

using namespace pbf103;

struct pbf_emitter {
    int device = 0;
    uint32_t n = 0;
    float4 *x = nullptr, *v = nullptr;
    ~pbf_emitter()
    {
        if (x) cudaFree(x);
        if (v) cudaFree(v);
    }
};

namespace {
inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

pbf_status emitter_alloc(int device, uint32_t n, pbf_emitter **out)
{
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PBF_ERROR_NO_DEVICE;
    if (device < 0 || device >= ndev) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_emitter *e = new (std::nothrow) pbf_emitter();
    if (!e) return PBF_ERROR_OUT_OF_MEMORY;
    e->device = device;
    e->n = n;
    cudaError_t ce = cudaSetDevice(device);
    if (ce == cudaSuccess) ce = cudaMalloc(&e->x, 16ull * (n ? n : 1));
    if (ce == cudaSuccess) ce = cudaMalloc(&e->v, 16ull * (n ? n : 1));
    if (ce != cudaSuccess) {
        set_last_error("pbf_emitter_create", ce);
        delete e;
        return PBF_ERROR_CUDA;
    }
    *out = e;
    return PBF_SUCCESS;
}

pbf_status emit(Batch &b, uint32_t scene, const pbf_emitter *e, double max_fill, cudaStream_t st)
{
    if (!e || !(max_fill >= 0.0)) return PBF_ERROR_INVALID_ARGUMENT;
    if (e->device != b.device()) return PBF_ERROR_INVALID_ARGUMENT;
    Batch::SceneArrays A;
    pbf_status rc = b.scene_arrays(scene, &A);
    if (rc != PBF_SUCCESS) return rc;
    CK(cudaSetDevice(b.device()));
    if (e->n)
        k_append<BufferSource><<<blocks_for(e->n), 256, 0, st>>>(BufferSource{e->x, e->v}, A, e->n, max_fill);
    k_append_commit<<<1, 1, 0, st>>>(A, e->n, max_fill);
    CK(cudaGetLastError());
    b.note_append(scene, e->n);
    return PBF_SUCCESS;
}

pbf_status generate(Batch &b, uint32_t scene, const pbf_arrangement *a, const float v0[3], cudaStream_t st,
                    uint32_t *n_points)
{
    ArrangePlan P;
    pbf_status rc = plan_arrangement(a, &P);
    if (rc != PBF_SUCCESS) return rc;
    if (n_points) *n_points = P.count;
    const float4 v = v0 ? make_float4(v0[0], v0[1], v0[2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    return append_plan(b, scene, P, v, std::numeric_limits<double>::infinity(), st);
}
}  // namespace

extern "C" {

pbf_status pbf_arrangement_count(const pbf_arrangement *a, uint32_t *n)
{
    if (!n) return PBF_ERROR_INVALID_ARGUMENT;
    ArrangePlan P;
    pbf_status rc = plan_arrangement(a, &P);
    if (rc == PBF_SUCCESS) *n = P.count;
    return rc;
}

pbf_status pbf_emitter_create(int device, const float *x, const float *v, uint32_t n, int src_dev, pbf_emitter **out)
{
    if (!out || (n && !x)) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_emitter *e = nullptr;
    pbf_status rc = emitter_alloc(device, n, &e);
    if (rc != PBF_SUCCESS) return rc;
    if (n) {
        // AoS float3 -> float4 on the device
        float *stage = nullptr;
        cudaError_t ce = cudaMalloc(&stage, 24ull * n);
        const float *sx = x, *sv = v;
        if (ce == cudaSuccess && !src_dev) {
            ce = cudaMemcpy(stage, x, 12ull * n, cudaMemcpyHostToDevice);
            if (ce == cudaSuccess && v) ce = cudaMemcpy(stage + 3ull * n, v, 12ull * n, cudaMemcpyHostToDevice);
            sx = stage;
            sv = v ? stage + 3ull * n : nullptr;
        }
        if (ce == cudaSuccess) {
            launch_aos3_to_f4(sx, e->x, n, 0);
            if (sv) launch_aos3_to_f4(sv, e->v, n, 0);
            else ce = cudaMemset(e->v, 0, 16ull * n);
        }
        if (ce == cudaSuccess) ce = cudaGetLastError();
        if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
        if (stage) cudaFree(stage);
        if (ce != cudaSuccess) {
            set_last_error("pbf_emitter_create", ce);
            delete e;
            return PBF_ERROR_CUDA;
        }
    }
    *out = e;
    return PBF_SUCCESS;
}

pbf_status pbf_emitter_create_arrangement(int device, const pbf_arrangement *a, const float v0[3],
                                          pbf_emitter **out)
{
    if (!out) return PBF_ERROR_INVALID_ARGUMENT;
    ArrangePlan P;
    pbf_status rc = plan_arrangement(a, &P);
    if (rc != PBF_SUCCESS) return rc;
    pbf_emitter *e = nullptr;
    rc = emitter_alloc(device, P.count, &e);
    if (rc != PBF_SUCCESS) return rc;
    const float4 v = v0 ? make_float4(v0[0], v0[1], v0[2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    if (P.count) k_plan_fill<<<blocks_for(P.count), 256>>>(P, v, e->x, e->v);
    cudaError_t ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    if (ce != cudaSuccess) {
        set_last_error("pbf_emitter_create_arrangement", ce);
        delete e;
        return PBF_ERROR_CUDA;
    }
    *out = e;
    return PBF_SUCCESS;
}

pbf_status pbf_emitter_size(const pbf_emitter *e, uint32_t *n)
{
    if (!e || !n) return PBF_ERROR_INVALID_ARGUMENT;
    *n = e->n;
    return PBF_SUCCESS;
}

pbf_status pbf_emitter_destroy(pbf_emitter *e)
{
    if (e) {
        cudaSetDevice(e->device);
        delete e;
    }
    return PBF_SUCCESS;
}

pbf_status pbf_get_particle_ids(pbf_handle *h, uint32_t *ids, int dst_dev, void *st)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->b.device()));
    return get_ids(h->b, h->scene, ids, nullptr, dst_dev != 0, S(st));
}

pbf_status pbf_restore_order(pbf_handle *h, float *x, float *v, uint32_t n_out, int dst_dev, void *st)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->b.device()));
    return scatter_out(h->b, h->scene, true, x, v, n_out, dst_dev != 0, S(st));
}

pbf_status pbf_get_particles_by_id(pbf_handle *h, float *x, float *v, uint32_t n_out, int dst_dev, void *st)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    CK(cudaSetDevice(h->b.device()));
    return scatter_out(h->b, h->scene, false, x, v, n_out, dst_dev != 0, S(st));
}

pbf_status pbf_generate(pbf_handle *h, const pbf_arrangement *a, const float v0[3], void *st, uint32_t *n_points)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    return generate(h->b, h->scene, a, v0, S(st), n_points);
}

pbf_status pbf_emit(pbf_handle *h, const pbf_emitter *e, double max_fill, void *st)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    return emit(h->b, h->scene, e, max_fill, S(st));
}

pbf_status pbf_batch_get_particle_ids(pbf_batch *b, uint32_t scene, uint32_t *ids, uint32_t *num, int dst_dev,
                                      void *st)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    CK(cudaSetDevice(b->b.device()));
    return get_ids(b->b, scene, ids, num, dst_dev != 0, S(st));
}

pbf_status pbf_batch_restore_order(pbf_batch *b, uint32_t scene, float *x, float *v, uint32_t n_out, int dst_dev,
                                   void *st)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    CK(cudaSetDevice(b->b.device()));
    return scatter_out(b->b, scene, true, x, v, n_out, dst_dev != 0, S(st));
}

pbf_status pbf_batch_get_particles_by_id(pbf_batch *b, uint32_t scene, float *x, float *v, uint32_t n_out,
                                         int dst_dev, void *st)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    CK(cudaSetDevice(b->b.device()));
    return scatter_out(b->b, scene, false, x, v, n_out, dst_dev != 0, S(st));
}

pbf_status pbf_batch_generate(pbf_batch *b, uint32_t scene, const pbf_arrangement *a, const float v0[3], void *st,
                              uint32_t *n_points)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    return generate(b->b, scene, a, v0, S(st), n_points);
}

pbf_status pbf_batch_emit(pbf_batch *b, uint32_t scene, const pbf_emitter *e, double max_fill, void *st)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    return emit(b->b, scene, e, max_fill, S(st));
}

}  // extern "C"
