// extern "C" entry points of include/pbf103.h (plain step, boundary, batch).
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "pbf_engine.h"

namespace pbf103 {
static thread_local std::string g_last_error;
void set_last_error(const char *what, cudaError_t e)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
}
}  // namespace pbf103

using namespace pbf103;

static std::atomic<uint64_t> g_boundary_uid{1};

namespace {
// boundary objects carry a unique id, so a handle notices a different
// boundary even when a freed one's address is reused
struct BoundaryWithId : pbf_boundary_t {
    uint64_t uid = 0;
};
uint64_t boundary_uid(const pbf_boundary_t *b) { return b ? static_cast<const BoundaryWithId *>(b)->uid : 0; }

inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

pbf_status set_dev(int dev)
{
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) {
        set_last_error("cudaSetDevice", e);
        return PBF_ERROR_CUDA;
    }
    return PBF_SUCCESS;
}
}  // namespace

extern "C" {

const char *pbf_status_string(pbf_status s)
{
    switch (s) {
    case PBF_SUCCESS: return "success";
    case PBF_ERROR_INVALID_ARGUMENT: return "invalid argument";
    case PBF_ERROR_CUDA: return "CUDA error";
    case PBF_ERROR_OUT_OF_MEMORY: return "out of device memory / arena full";
    case PBF_ERROR_CAPACITY: return "particle capacity exceeded";
    case PBF_ERROR_GRID_TOO_LARGE: return "grid_size is too large";
    case PBF_ERROR_BAD_PARAMETER: return "invalid physical parameter";
    case PBF_ERROR_NOT_FOUND: return "not found";
    case PBF_ERROR_BUDGET: return "HBM budget exceeded";
    case PBF_ERROR_NO_DEVICE: return "no CUDA device";
    case PBF_ERROR_NOT_READY: return "not ready";
    }
    return "unknown status";
}

const char *pbf_last_error(void) { return g_last_error.c_str(); }

int pbf_abi_version(void) { return PBF103_ABI_VERSION; }

pbf_status pbf_params_init(pbf_params *p)
{
    if (!p) return PBF_ERROR_INVALID_ARGUMENT;
    std::memset(p, 0, sizeof(*p));
    p->stable_density = 1000.f;
    p->stable_distance = 0.05f;
    p->particle_mass = 0.125f;
    p->smoothing_length = 0.1f;
    p->time_step = 1.f / 120.f;
    p->relaxation = 600.f;
    p->xsph_parameter = 0.01f;
    p->vc_parameter = 0.0005f;
    p->body_force[0] = 0.f;
    p->body_force[1] = -9.8f;
    p->body_force[2] = 0.f;
    p->max_pair_particle_num = 30;
    p->tensile_mode = PBF_TENSILE_REFERENCE;
    p->scorr_k = 0.1f;
    p->scorr_n = 4;
    p->scorr_dq = 0.2f;
    p->xsph_mode = 0;
    p->vorticity_mode = PBF_VORTICITY_OFF;
    p->max_collision_passes = 64;
    p->cell_width = 0.f;
    return PBF_SUCCESS;
}

// calcGridSize, src/pbf/pbf_type.cpp:141-162
pbf_status pbf_calc_grid_size(double cell_size, const float domain_end[3], uint32_t g[3])
{
    if (!domain_end || !g || !(cell_size > 0.0)) return PBF_ERROR_INVALID_ARGUMENT;
    uint32_t x = 1, y = 1, z = 1;
    for (;;) {
        const bool bx = x * cell_size > (double)domain_end[0];
        const bool by = y * cell_size > (double)domain_end[1];
        const bool bz = z * cell_size > (double)domain_end[2];
        if (bx && by && bz) break;
        x = bx ? x : x * 2;
        y = by ? y : y * 2;
        z = bz ? z : z * 2;
        if (x > 1028 || y > 1028 || z > 1028) return PBF_ERROR_GRID_TOO_LARGE;
    }
    g[0] = x;
    g[1] = y;
    g[2] = z;
    return PBF_SUCCESS;
}

pbf_status pbf_boundary_create(const float *inner, uint32_t n_inner, const float *outer, uint32_t n_outer,
                               const float *pts, const float *nrm, uint32_t n_planes, pbf_boundary_t **out)
{
    if (!out || (n_inner && !inner) || (n_outer && !outer) || (n_planes && (!pts || !nrm)))
        return PBF_ERROR_INVALID_ARGUMENT;
    BoundaryWithId *b = new (std::nothrow) BoundaryWithId();
    if (!b) return PBF_ERROR_OUT_OF_MEMORY;
    for (uint32_t k = 0; k < n_inner; ++k)
        b->prims.push_back(make_float4(inner[4 * k], inner[4 * k + 1], inner[4 * k + 2], inner[4 * k + 3]));
    for (uint32_t k = 0; k < n_outer; ++k)
        b->prims.push_back(make_float4(outer[4 * k], outer[4 * k + 1], outer[4 * k + 2], outer[4 * k + 3]));
    for (uint32_t k = 0; k < n_planes; ++k) {
        b->prims.push_back(make_float4(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2], 0.f));
        b->prims.push_back(make_float4(nrm[3 * k], nrm[3 * k + 1], nrm[3 * k + 2], 0.f));
    }
    b->n_inner = n_inner;
    b->n_outer = n_outer;
    b->n_planes = n_planes;
    b->uid = g_boundary_uid.fetch_add(1);
    *out = b;
    return PBF_SUCCESS;
}

pbf_status pbf_boundary_destroy(pbf_boundary_t *b)
{
    delete static_cast<BoundaryWithId *>(b);
    return PBF_SUCCESS;
}

// ---------------------------------------------------------------- plain --
struct pbf_handle_ex : pbf_handle {
    uint64_t bnd_uid = ~0ull;
};

pbf_status pbf_create(const pbf_params *params, uint32_t capacity, const float domain_end[3], int device,
                      pbf_handle **out)
{
    if (!params || !out || capacity == 0) return PBF_ERROR_INVALID_ARGUMENT;
    SceneDesc d;
    uint32_t grid[3];
    pbf_status rc = derive_desc(*params, domain_end, &d, grid);
    if (rc != PBF_SUCCESS) return rc;
    pbf_handle_ex *h = new (std::nothrow) pbf_handle_ex();
    if (!h) return PBF_ERROR_OUT_OF_MEMORY;
    rc = h->b.init(1, capacity, (uint64_t)d.ncell + 1, params->max_pair_particle_num, device);
    if (rc != PBF_SUCCESS) {
        delete h;
        return rc;
    }
    h->params = *params;
    if (domain_end) std::memcpy(h->domain_end, domain_end, sizeof(h->domain_end));
    const float big = 3.0e38f;
    const float amin[3] = {-big, -big, -big}, amax[3] = {big, big, big};
    uint32_t id = 0;
    rc = h->b.add_scene(*params, capacity, domain_end, nullptr, amin, amax, nullptr, nullptr, 0, false, 0, &id);
    if (rc != PBF_SUCCESS) {
        delete h;
        return rc;
    }
    h->scene = id;
    h->bnd_uid = 0;  // builtin sphere
    *out = h;
    return PBF_SUCCESS;
}

pbf_status pbf_destroy(pbf_handle *h)
{
    if (h) {
        cudaSetDevice(h->b.device());
        delete static_cast<pbf_handle_ex *>(h);
    }
    return PBF_SUCCESS;
}

pbf_status pbf_set_params(pbf_handle *h, const pbf_params *p)
{
    if (!h || !p) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = set_dev(h->b.device());
    if (rc) return rc;
    rc = h->b.set_scene_params(h->scene, *p);
    if (rc == PBF_SUCCESS) h->params = *p;
    return rc;
}

pbf_status pbf_get_params(pbf_handle *h, pbf_params *p)
{
    if (!h || !p) return PBF_ERROR_INVALID_ARGUMENT;
    *p = h->params;
    return PBF_SUCCESS;
}

pbf_status pbf_get_grid(pbf_handle *h, uint32_t g[3], float *cw)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    const SceneHost *s = h->b.scene(h->scene);
    if (!s) return PBF_ERROR_NOT_FOUND;
    if (g) {
        g[0] = s->desc.gx;
        g[1] = s->desc.gy;
        g[2] = s->desc.gz;
    }
    if (cw) *cw = s->desc.cw;
    return PBF_SUCCESS;
}

pbf_status pbf_set_particles(pbf_handle *h, const float *x, const float *v, uint32_t n, int src_dev, void *st)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = set_dev(h->b.device());
    if (rc) return rc;
    return h->b.set_particles(h->scene, x, v, n, src_dev != 0, false, S(st));
}

pbf_status pbf_add_particles(pbf_handle *h, const float *x, const float *v, uint32_t n, int src_dev, void *st)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = set_dev(h->b.device());
    if (rc) return rc;
    return h->b.set_particles(h->scene, x, v, n, src_dev != 0, true, S(st));
}

static pbf_status prepare_step(pbf_handle *h, const pbf_boundary_t *boundary, const float amin[3],
                               const float amax[3])
{
    if (!amin || !amax) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_handle_ex *hx = static_cast<pbf_handle_ex *>(h);
    pbf_status rc = set_dev(h->b.device());
    if (rc) return rc;
    const uint64_t uid = boundary_uid(boundary);
    if (uid != hx->bnd_uid) {
        rc = h->b.set_scene_boundary(h->scene, boundary);
        if (rc) return rc;
        hx->bnd_uid = uid;
    }
    return h->b.set_scene_area(h->scene, amin, amax);
}

pbf_status pbf_one_step(pbf_handle *h, const pbf_boundary_t *boundary, const float amin[3], const float amax[3],
                        int iters, void *st)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = prepare_step(h, boundary, amin, amax);
    if (rc) return rc;
    return h->b.step(iters, S(st));
}

pbf_status pbf_one_step_external(pbf_handle *h, float *x_dev, const pbf_boundary_t *boundary, const float amin[3],
                                 const float amax[3], int iters, void *st)
{
    if (!h || !x_dev) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = prepare_step(h, boundary, amin, amax);
    if (rc) return rc;
    uint32_t n = 0;
    rc = h->b.get_num(h->scene, &n, S(st));
    if (rc) return rc;
    rc = h->b.import_x_device(h->scene, x_dev, n, S(st));
    if (rc) return rc;
    rc = h->b.step(iters, S(st));
    if (rc) return rc;
    return h->b.export_x_device(h->scene, x_dev, S(st));
}

pbf_status pbf_get_num(pbf_handle *h, uint32_t *num)
{
    if (!h || !num) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = set_dev(h->b.device());
    if (rc) return rc;
    return h->b.get_num(h->scene, num, 0);
}

pbf_status pbf_get_particles(pbf_handle *h, float *x, float *v, int dst_dev, void *st)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = set_dev(h->b.device());
    if (rc) return rc;
    return h->b.get_particles(h->scene, x, v, nullptr, dst_dev != 0, S(st));
}

pbf_status pbf_get_flags(pbf_handle *h, uint32_t *flags, int clear)
{
    if (!h || !flags) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = set_dev(h->b.device());
    if (rc) return rc;
    return h->b.get_flags(h->scene, flags, clear != 0, 0);
}

pbf_status pbf_set_graph_mode(pbf_handle *h, int enable)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    h->b.set_graph_mode(enable != 0);
    return PBF_SUCCESS;
}

pbf_status pbf_get_neighbor_debug(pbf_handle *h, uint32_t *sorted_hash, uint32_t *perm, uint32_t *cell_start,
                                  uint32_t *cell_end, uint32_t *neighbor_list, uint32_t *n_in)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = set_dev(h->b.device());
    if (rc) return rc;
    return h->b.get_debug(h->scene, sorted_hash, perm, cell_start, cell_end, neighbor_list, n_in, 0);
}

pbf_status pbf_last_launches(pbf_handle *h, uint32_t *launches)
{
    if (!h || !launches) return PBF_ERROR_INVALID_ARGUMENT;
    *launches = h->b.last_launches();
    return PBF_SUCCESS;
}

pbf_status pbf_profile_step(pbf_handle *h, const pbf_boundary_t *boundary, const float amin[3],
                            const float amax[3], int iters, void *st, float *ms, char *names, uint32_t max,
                            uint32_t *n)
{
    if (!h) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = prepare_step(h, boundary, amin, amax);
    if (rc) return rc;
    return h->b.profile_step(iters, S(st), ms, names, max, n);
}

pbf_status pbf_batch_profile_step(pbf_batch *b, int iters, void *st, float *ms, char *names, uint32_t max,
                                  uint32_t *n)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.profile_step(iters, S(st), ms, names, max, n);
}

// ---------------------------------------------------------------- batch --
pbf_status pbf_batch_create(uint32_t max_scenes, uint64_t max_particles, uint64_t max_cells, uint32_t max_pair,
                            int device, pbf_batch **out)
{
    if (!out) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_batch *b = new (std::nothrow) pbf_batch();
    if (!b) return PBF_ERROR_OUT_OF_MEMORY;
    pbf_status rc = b->b.init(max_scenes, max_particles, max_cells, max_pair, device);
    if (rc != PBF_SUCCESS) {
        delete b;
        return rc;
    }
    *out = b;
    return PBF_SUCCESS;
}

pbf_status pbf_batch_destroy(pbf_batch *b)
{
    if (b) {
        cudaSetDevice(b->b.device());
        delete b;
    }
    return PBF_SUCCESS;
}

pbf_status pbf_scene_bytes(const pbf_params *p, uint32_t capacity, const float domain_end[3], uint64_t *bytes)
{
    if (!p || !bytes) return PBF_ERROR_INVALID_ARGUMENT;
    SceneDesc d;
    pbf_status rc = derive_desc(*p, domain_end, &d, nullptr);
    if (rc) return rc;
    *bytes = (uint64_t)capacity * bytes_per_particle(p->max_pair_particle_num) + ((uint64_t)d.ncell + 1) * 8 +
             sizeof(SceneDesc) + 16 * 64;
    return PBF_SUCCESS;
}

pbf_status pbf_batch_add_scene(pbf_batch *b, const pbf_params *p, uint32_t capacity, const float domain_end[3],
                               const pbf_boundary_t *boundary, const float amin[3], const float amax[3],
                               const float *x, const float *v, uint32_t n, int src_dev, void *st, uint32_t *id)
{
    if (!b || !p || !id) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.add_scene(*p, capacity, domain_end, boundary, amin, amax, x, v, n, src_dev != 0, S(st), id);
}

pbf_status pbf_batch_remove_scene(pbf_batch *b, uint32_t id)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    return b->b.remove_scene(id);
}

pbf_status pbf_batch_num_scenes(pbf_batch *b, uint32_t *n)
{
    if (!b || !n) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    *n = b->b.num_scenes();
    return PBF_SUCCESS;
}

pbf_status pbf_batch_step(pbf_batch *b, int iters, void *st)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.step(iters, S(st));
}

pbf_status pbf_batch_get_scene(pbf_batch *b, uint32_t id, float *x, float *v, uint32_t *num, int dst_dev, void *st)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.get_particles(id, x, v, num, dst_dev != 0, S(st));
}

pbf_status pbf_batch_get_flags(pbf_batch *b, uint32_t id, uint32_t *flags, int clear)
{
    if (!b || !flags) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.get_flags(id, flags, clear != 0, 0);
}

pbf_status pbf_batch_scene_ids(pbf_batch *b, uint32_t *ids, uint32_t max, uint32_t *n)
{
    if (!b || !n || (max && !ids)) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    std::vector<uint32_t> v;
    b->b.scene_ids(v);
    *n = (uint32_t)v.size();
    for (uint32_t k = 0; k < max && k < v.size(); ++k) ids[k] = v[k];
    return PBF_SUCCESS;
}

pbf_status pbf_batch_set_all(pbf_batch *b, const uint32_t *counts, const float *x, const float *v, int src_dev,
                             void *st)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.upload_all(counts, x, v, src_dev != 0, S(st));
}

pbf_status pbf_batch_get_all(pbf_batch *b, uint32_t *counts, float *x, float *v, int dst_dev, void *st)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.download_all(counts, x, v, dst_dev != 0, S(st));
}

pbf_status pbf_batch_step_packed(pbf_batch *b, int iters, const uint32_t *counts, const float *x_dev,
                                 const float *v_dev, void *st)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.step_packed(iters, counts, x_dev, v_dev, S(st));
}

pbf_status pbf_batch_get_all_async(pbf_batch *b, uint32_t *counts_dev, float *x_dev, float *v_dev, void *st)
{
    if (!b || !counts_dev) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.download_all_async(counts_dev, x_dev, v_dev, S(st));
}

pbf_status pbf_batch_autotune(pbf_batch *b, int iters, void *st, uint32_t *chosen)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    pbf_status rc = set_dev(b->b.device());
    if (rc) return rc;
    return b->b.autotune(iters, S(st), chosen);
}

pbf_status pbf_batch_set_tile(pbf_batch *b, uint32_t tile)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    return b->b.set_tile(tile);
}

pbf_status pbf_batch_set_chunk(pbf_batch *b, uint32_t chunk)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    return b->b.set_chunk(chunk);
}

pbf_status pbf_batch_get_launch_shape(pbf_batch *b, uint32_t *tile, uint32_t *chunk)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    if (tile) *tile = b->b.tile();
    if (chunk) *chunk = b->b.chunk();
    return PBF_SUCCESS;
}

pbf_status pbf_batch_set_cell_tile(pbf_batch *b, uint32_t cells)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    return b->b.set_cell_tile(cells);
}

pbf_status pbf_batch_get_cell_tile(pbf_batch *b, uint32_t *cells)
{
    if (!b || !cells) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    *cells = b->b.cell_tile();
    return PBF_SUCCESS;
}

pbf_status pbf_batch_set_graph_mode(pbf_batch *b, int enable)
{
    if (!b) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    b->b.set_graph_mode(enable != 0);
    return PBF_SUCCESS;
}

pbf_status pbf_batch_last_launches(pbf_batch *b, uint32_t *launches)
{
    if (!b || !launches) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(b->mu);
    *launches = b->b.last_launches();
    return PBF_SUCCESS;
}

}  // extern "C"
