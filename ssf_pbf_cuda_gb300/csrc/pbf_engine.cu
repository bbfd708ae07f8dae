// Host runtime of the PBF engine (see pbf_engine.h).
#include "pbf_engine.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

namespace pbf103 {

void set_last_error(const char *what, cudaError_t e);

#define CK(call)                                      \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) {                      \
            set_last_error(#call, e_);                \
            return e_ == cudaErrorMemoryAllocation ? PBF_ERROR_OUT_OF_MEMORY : PBF_ERROR_CUDA; \
        }                                             \
    } while (0)

// ------------------------------------------------------------ allocator --
void RangeAllocator::reset(uint64_t size)
{
    size_ = size;
    free_.clear();
    used_.clear();
    if (size) free_[0] = size;
}

bool RangeAllocator::alloc(uint64_t n, uint64_t *off)
{
    if (n == 0) {
        *off = 0;
        return true;
    }
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= n) {
            const uint64_t o = it->first, rem = it->second - n;
            free_.erase(it);
            if (rem) free_[o + n] = rem;
            used_[o] = n;
            *off = o;
            return true;
        }
    }
    return false;
}

void RangeAllocator::release(uint64_t off, uint64_t n)
{
    if (n == 0) return;
    used_.erase(off);
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        free_.erase(nx);
    }
    if (it != free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            free_.erase(it);
        }
    }
}

uint64_t RangeAllocator::high_water() const
{
    if (used_.empty()) return 0;
    auto it = std::prev(used_.end());
    return it->first + it->second;
}

uint64_t RangeAllocator::free_total() const
{
    uint64_t t = 0;
    for (auto &kv : free_) t += kv.second;
    return t;
}

// ----------------------------------------------------------- parameters --
static float wpoly6_host(float r, float inv_h)
{
    const float q = r * inv_h;
    const float alpha = 1.56668147065f * inv_h * inv_h * inv_h;
    if (q <= 1.f) {
        const float q2 = q * q;
        const float t = 1.f - q2;
        return alpha * t * t * t;
    }
    return 0.f;
}

static bool is_pow2(uint32_t v) { return v && !(v & (v - 1)); }

pbf_status derive_desc(const pbf_params &p, const float domain_end[3], SceneDesc *d, uint32_t grid[3])
{
    // pbf_particle::allocate rejects unset parameters (pbf_type.cpp:167-170);
    // strictly positive values are required here because they are divided by.
    if (!(p.stable_density > 0.f) || !(p.particle_mass > 0.f) || !(p.smoothing_length > 0.f) ||
        !(p.time_step > 0.f) || p.stable_distance < 0.f)
        return PBF_ERROR_BAD_PARAMETER;
    if (p.max_pair_particle_num < 2 || p.max_pair_particle_num > 256) return PBF_ERROR_INVALID_ARGUMENT;
    if (p.tensile_mode < 0 || p.tensile_mode > 2 || p.vorticity_mode < 0 || p.vorticity_mode > 2 ||
        p.xsph_mode < 0 || p.xsph_mode > 2 || p.scorr_n < 0 || p.scorr_n > 16 || p.max_collision_passes == 0)
        return PBF_ERROR_INVALID_ARGUMENT;
    const float cw = p.cell_width > 0.f ? p.cell_width : p.smoothing_length;
    uint32_t g[3];
    if (p.grid_size[0] && p.grid_size[1] && p.grid_size[2]) {
        for (int c = 0; c < 3; ++c) {
            if (!is_pow2(p.grid_size[c]) || p.grid_size[c] > 4096) return PBF_ERROR_GRID_TOO_LARGE;
            g[c] = p.grid_size[c];
        }
    } else {
        if (!domain_end) return PBF_ERROR_INVALID_ARGUMENT;
        if (pbf_calc_grid_size((double)cw * 2.0, domain_end, g) != PBF_SUCCESS) return PBF_ERROR_GRID_TOO_LARGE;
    }
    const uint64_t ncell = (uint64_t)g[0] * g[1] * g[2];
    if (ncell >= (1ull << 31)) return PBF_ERROR_GRID_TOO_LARGE;
    std::memset(d, 0, sizeof(*d));
    d->gx = g[0];
    d->gy = g[1];
    d->gz = g[2];
    d->ncell = (uint32_t)ncell;
    d->cap = p.max_pair_particle_num - 1;
    d->cw = cw;
    const float h = p.smoothing_length;
    const float inv_h = 1.f / h;
    const float inv_h2 = inv_h * inv_h;
    d->h = h;
    d->h2 = h * h;
    d->inv_h = inv_h;
    d->alpha = 1.56668147065f * inv_h * inv_h2;
    d->beta = -14.3239448745f * inv_h2 * inv_h2;
    d->alpha6 = 1.56668147065f * inv_h * inv_h * inv_h;
    d->m = p.particle_mass;
    d->inv_rho0 = 1.f / p.stable_density;
    d->m2rho2 = d->m * d->m * d->inv_rho0 * d->inv_rho0;
    d->relax = p.relaxation;
    d->dt = p.time_step;
    d->inv_dt = 1.f / p.time_step;
    // k = W(0.4h)^4, pow() evaluated in double then narrowed (pbf_solve.cpp:92,
    // pbf_position_update.cu:232)
    const float k = (float)std::pow((double)wpoly6_host(h * 0.4f, inv_h), 4);
    d->inv_k = 1.f / k;
    const float wdq = wpoly6_host(p.scorr_dq * h, inv_h);
    d->inv_wdq = wdq > 0.f ? 1.f / wdq : 0.f;
    d->scorr_k = p.scorr_k;
    d->scorr_n = p.scorr_n;
    // the pair passes sum t^3 = W / alpha and s' d = grad W / beta and
    // evaluate s_corr as a constant times a power of t^3:
    // 10 W^4 / W(0.4h)^4 = (10 alpha^4 / W(0.4h)^4) (t^3)^4 and
    // k (W / W(dq h))^n = (k alpha^n / W(dq h)^n) (t^3)^n
    d->ih2 = inv_h2;
    const double al = d->alpha, be = d->beta, mr = (double)d->m * (double)d->inv_rho0;
    d->tens_c = (float)(10.0 * std::pow(al / (double)wpoly6_host(h * 0.4f, inv_h), 4));
    d->scorr_c = wdq > 0.f ? (float)((double)p.scorr_k * std::pow(al / (double)wdq, p.scorr_n)) : 0.f;
    d->lam_c = (float)(al * mr);
    d->lam_k = (float)(mr * mr * be * be);
    d->dp_k = (float)(mr * be);
    d->tensile_mode = p.tensile_mode;
    d->xsph_mode = p.xsph_mode;
    d->vort_mode = p.vorticity_mode;
    d->xsph_c = p.xsph_parameter;
    d->vort_eps = p.vc_parameter;
    for (int c = 0; c < 3; ++c) d->g[c] = p.body_force[c];
    d->max_coll = p.max_collision_passes;
    d->builtin_sphere = 1;
    if (grid) std::memcpy(grid, g, sizeof(g));
    return PBF_SUCCESS;
}

uint64_t bytes_per_particle(uint32_t max_pair)
{
    // x v xs xa xb xold w vt wx (float4) + xv (2 float4) + key slot tmp perm id id_tmp wpos + lam + nnb +
    // selfat + cls + nbr
    return 11 * 16 + 7 * 4 + 4 + 1 + 1 + 1 + 16ull * ((max_pair - 1 + 3) / 4);  // list slots in whole quads
}

// ---------------------------------------------------------------- batch --
Batch::~Batch()
{
    for (cudaGraphExec_t e : exec_)
        if (e) cudaGraphExecDestroy(e);
    if (d_pin_) cudaFree(d_pin_);
    if (cap_stream_) cudaStreamDestroy(cap_stream_);
    if (small_done_) cudaEventDestroy(small_done_);
    if (h_small_) cudaFreeHost(h_small_);
    void *ptrs[] = {d_scenes_, d_tile_scene_, d_tile_start_, d_ctrl_, d_scene_num_, d_flags_, d_x_, d_v_,
                    d_xs_, d_xa_, d_xb_, d_xold_, d_w_, d_vt_, d_key_, d_slot_, d_tmp_, d_perm_, d_count_,
                    d_offsets_, d_bsum_, d_lam_, d_nbr_, d_nnb_, d_self_, d_bnd_, d_pack_off_, d_active_, d_xv_, d_id_, d_id_tmp_,
                    d_next_id_, d_cls_, d_wx_, d_chist_, d_wpos_, d_dense_, d_mid_};
    for (void *p : ptrs)
        if (p) cudaFree(p);
}

pbf_status Batch::init(uint32_t max_scenes, uint64_t max_particles, uint64_t max_cells, uint32_t max_pair,
                       int device)
{
    if (max_scenes == 0 || max_particles == 0 || max_cells == 0 || max_pair < 2 || max_pair > 256)
        return PBF_ERROR_INVALID_ARGUMENT;
    if (max_particles >= (1ull << 31) || max_cells >= (1ull << 32) - 8) return PBF_ERROR_INVALID_ARGUMENT;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return PBF_ERROR_NO_DEVICE;
    if (device < 0 || device >= ndev) return PBF_ERROR_INVALID_ARGUMENT;
    device_ = device;
    CK(cudaSetDevice(device_));
    CK(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device_));
    max_scenes_ = max_scenes;
    max_particles_ = max_particles;
    max_cells_ = max_cells;
    max_pair_ = max_pair;
    bnd_capacity_ = (uint64_t)max_scenes * 32 + 1024;
    // particle tiles (64 particles at the smallest tile) then cell tiles
    max_tiles_ = max_particles / 64 + max_scenes + 1 + max_cells / kCellTileMin + max_scenes + 1;
    const uint64_t P = max_particles, C = max_cells;
    auto A = [&](void **p, uint64_t bytes) -> cudaError_t {
        arena_bytes_ += bytes;
        return cudaMalloc(p, bytes ? bytes : 16);
    };
    CK(A((void **)&d_scenes_, sizeof(SceneDesc) * max_scenes));
    CK(A((void **)&d_tile_scene_, 4 * max_tiles_));
    CK(A((void **)&d_tile_start_, 4 * max_tiles_));
    CK(A((void **)&d_ctrl_, sizeof(Ctrl)));
    CK(A((void **)&d_scene_num_, 4ull * max_scenes));
    CK(A((void **)&d_flags_, 4ull * max_scenes));
    CK(A((void **)&d_next_id_, 4ull * max_scenes));
    float4 **f4[] = {&d_x_, &d_v_, &d_xs_, &d_xa_, &d_xb_, &d_xold_, &d_w_, &d_vt_, &d_wx_};
    // + kWalkSpare records: the neighbour walk reads candidates in groups of
    // four and may read up to three past the end of a range (never accepted)
    for (float4 **p : f4) CK(A((void **)p, 16 * (P + kWalkSpare)));
    CK(A((void **)&d_xv_, 32 * (P + kWalkSpare)));
    uint32_t **u4[] = {&d_key_, &d_slot_, &d_tmp_, &d_perm_, &d_id_, &d_id_tmp_, &d_wpos_};
    for (uint32_t **p : u4) CK(A((void **)p, 4 * P));
    CK(A((void **)&d_count_, 4 * (C + 4)));
    CK(A((void **)&d_offsets_, 4 * (C + 4)));
    CK(A((void **)&d_bsum_, 4 * ((C + kScanTile - 1) / kScanTile + 4)));
    CK(A((void **)&d_lam_, 4 * P));
    CK(A((void **)&d_nbr_, 16ull * ((max_pair - 1 + 3) / 4) * P));  // quads of 4 slots per particle
    CK(A((void **)&d_nnb_, P));
    CK(A((void **)&d_self_, P));
    CK(A((void **)&d_cls_, P));
    CK(A((void **)&d_dense_, 4 * (2 * (P / 64 + 1) + 1)));  // a dense bucket holds more than 64 particles
    CK(A((void **)&d_mid_, 4 * (2 * (P / 16 + 1) + 1)));    // a medium one more than 16
    CK(A((void **)&d_chist_, 8 * (C + 4)));
    CK(A((void **)&d_bnd_, 16 * bnd_capacity_));
    CK(A((void **)&d_pack_off_, 4ull * max_scenes));
    CK(A((void **)&d_active_, 4ull * max_scenes));
    CK(A((void **)&d_pin_, sizeof(PackedIn)));
    CK(cudaMallocHost((void **)&h_small_, 8ull * max_scenes + 64));
    CK(cudaEventCreateWithFlags(&small_done_, cudaEventDisableTiming));
    CK(cudaMemset(d_count_, 0, 4 * (C + 4)));
    CK(cudaMemset(d_offsets_, 0, 4 * (C + 4)));
    CK(cudaMemset(d_scene_num_, 0, 4ull * max_scenes));
    CK(cudaMemset(d_flags_, 0, 4ull * max_scenes));
    CK(cudaMemset(d_next_id_, 0, 4ull * max_scenes));
    CK(cudaMemset(d_ctrl_, 0, sizeof(Ctrl)));
    CK(cudaMemset(d_nnb_, 0, P));
    CK(cudaMemset(d_self_, kNotListed, P));
    CK(cudaMemset(d_v_, 0, 16 * P));
    CK(cudaMemset(d_x_, 0, 16 * P));
    CK(cudaStreamCreateWithFlags(&cap_stream_, cudaStreamNonBlocking));
    palloc_.reset(P);
    calloc_.reset(C);
    balloc_.reset(bnd_capacity_);
    bnd_host_.assign(bnd_capacity_, make_float4(0, 0, 0, 0));
    scenes_.clear();
    scenes_.reserve(max_scenes);
    return PBF_SUCCESS;
}

uint32_t Batch::num_scenes() const
{
    uint32_t n = 0;
    for (auto &s : scenes_) n += s.active ? 1 : 0;
    return n;
}

const SceneHost *Batch::scene(uint32_t id) const
{
    if (id >= scenes_.size() || !scenes_[id].active) return nullptr;
    return &scenes_[id];
}

bool Batch::can_fit(uint32_t capacity, uint64_t cells, uint64_t bnd_len) const
{
    // conservative: the largest free block of each arena must hold the request
    RangeAllocator p = palloc_, c = calloc_, b = balloc_;
    uint64_t o;
    return p.alloc(capacity, &o) && c.alloc(cells, &o) && b.alloc(bnd_len, &o) &&
           (num_scenes() < max_scenes_);
}

static void fill_boundary(const pbf_boundary_t *b, std::vector<float4> &out)
{
    out.clear();
    if (!b) return;
    out = b->prims;
}

// The clear box of a boundary made only of planes whose normals are unit
// axes (a box's walls).  For such a plane responsePlaneBoundary's
// (p - on) . n is +-(p_c - on_c) exactly, so p hits none of them when
// on_c <= p_c for each +e_c plane and p_c <= on_c for each -e_c plane:
// box_lo / box_hi are the largest / smallest of those on_c.  Any sphere,
// any other normal, or the built-in sphere leave the box off.
static void set_clear_box(SceneDesc &d, const pbf_boundary_t *b)
{
    d.clear_box = 0;
    for (int c = 0; c < 3; ++c) {
        d.box_lo[c] = -INFINITY;
        d.box_hi[c] = INFINITY;
    }
    if (!b || b->n_inner || b->n_outer) return;
    for (uint32_t k = 0; k < b->n_planes; ++k) {
        const float4 on = b->prims[2 * k], n = b->prims[2 * k + 1];
        const float nc[3] = {n.x, n.y, n.z}, oc[3] = {on.x, on.y, on.z};
        int axis = -1, zeros = 0;
        for (int c = 0; c < 3; ++c) {
            if (nc[c] == 0.f) ++zeros;
            else if (nc[c] == 1.f || nc[c] == -1.f) axis = c;
        }
        if (zeros != 2 || axis < 0) return;
        if (nc[axis] > 0.f) d.box_lo[axis] = std::max(d.box_lo[axis], oc[axis]);
        else d.box_hi[axis] = std::min(d.box_hi[axis], oc[axis]);
    }
    d.clear_box = 1;
}

pbf_status Batch::add_scene(const pbf_params &p, uint32_t capacity, const float domain_end[3],
                            const pbf_boundary_t *b, const float amin[3], const float amax[3], const float *x,
                            const float *v, uint32_t n, bool src_dev, cudaStream_t st, uint32_t *id)
{
    NvtxRange range("pbf add scene");
    if (capacity == 0 || n > capacity || !amin || !amax) return PBF_ERROR_INVALID_ARGUMENT;
    if (p.max_pair_particle_num > max_pair_) return PBF_ERROR_INVALID_ARGUMENT;
    SceneHost sh;
    sh.params = p;
    pbf_status rc = derive_desc(p, domain_end, &sh.desc, nullptr);
    if (rc != PBF_SUCCESS) return rc;
    uint32_t slot = UINT32_MAX;
    for (uint32_t k = 0; k < scenes_.size(); ++k)
        if (!scenes_[k].active) {
            slot = k;
            break;
        }
    if (slot == UINT32_MAX) {
        if (scenes_.size() >= max_scenes_) return PBF_ERROR_CAPACITY;
        slot = (uint32_t)scenes_.size();
        scenes_.emplace_back();
    }
    std::vector<float4> prims;
    fill_boundary(b, prims);
    sh.cells = (uint64_t)sh.desc.ncell + 1;
    sh.bnd_len = prims.size();
    uint64_t po, co, bo;
    if (!palloc_.alloc(capacity, &po)) return PBF_ERROR_OUT_OF_MEMORY;
    if (!calloc_.alloc(sh.cells, &co)) {
        palloc_.release(po, capacity);
        return PBF_ERROR_OUT_OF_MEMORY;
    }
    if (!balloc_.alloc(sh.bnd_len, &bo)) {
        palloc_.release(po, capacity);
        calloc_.release(co, sh.cells);
        return PBF_ERROR_OUT_OF_MEMORY;
    }
    sh.bnd_off = bo;
    sh.desc.p_off = (uint32_t)po;
    sh.desc.capacity = capacity;
    sh.desc.list16 = capacity <= kList16Max ? 1u : 0u;
    sh.desc.c_off = (uint32_t)co;
    sh.desc.b_off = (uint32_t)bo;
    sh.desc.builtin_sphere = b ? 0u : 1u;
    sh.desc.n_inner = b ? b->n_inner : 0;
    sh.desc.n_outer = b ? b->n_outer : 0;
    sh.desc.n_planes = b ? b->n_planes : 0;
    set_clear_box(sh.desc, b);
    for (int c = 0; c < 3; ++c) {
        sh.desc.amin[c] = amin[c];
        sh.desc.amax[c] = amax[c];
    }
    for (size_t k = 0; k < prims.size(); ++k) bnd_host_[bo + k] = prims[k];
    sh.active = true;
    sh.num_upper = 0;
    scenes_[slot] = sh;
    dirty_desc_ = dirty_tiles_ = true;
    dirty_bnd_ = dirty_bnd_ || !prims.empty();
    CK(cudaSetDevice(device_));
    CK(cudaMemsetAsync(d_scene_num_ + slot, 0, 4, st));
    CK(cudaMemsetAsync(d_flags_ + slot, 0, 4, st));
    *id = slot;
    if (n) {
        rc = set_particles(slot, x, v, n, src_dev, false, st);
        if (rc != PBF_SUCCESS) {
            remove_scene(slot);
            return rc;
        }
    }
    return PBF_SUCCESS;
}

pbf_status Batch::remove_scene(uint32_t id)
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    SceneHost &s = scenes_[id];
    palloc_.release(s.desc.p_off, s.desc.capacity);
    calloc_.release(s.desc.c_off, s.cells);
    balloc_.release(s.bnd_off, s.bnd_len);
    s.active = false;
    s.num_upper = 0;
    dirty_desc_ = dirty_tiles_ = true;
    return PBF_SUCCESS;
}

pbf_status Batch::set_particles(uint32_t id, const float *x, const float *v, uint32_t n, bool src_dev,
                                bool append, cudaStream_t st)
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    if (n && !x) return PBF_ERROR_INVALID_ARGUMENT;
    SceneHost &s = scenes_[id];
    CK(cudaSetDevice(device_));
    uint32_t start = 0;
    if (append) {
        pbf_status rc = get_num(id, &start, st);
        if (rc != PBF_SUCCESS) return rc;
    }
    if ((uint64_t)start + n > s.desc.capacity) return PBF_ERROR_CAPACITY;
    float4 *dx = d_x_ + s.desc.p_off + start;
    float4 *dv = d_v_ + s.desc.p_off + start;
    if (n) {
        const float *sx = x, *sv = v;
        if (!src_dev) {
            // raw AoS float3 goes to the scene's slice of the xs / vt scratch
            // (free between steps) and is widened on the device
            float *stx = reinterpret_cast<float *>(d_xs_ + s.desc.p_off + start);
            float *stv = reinterpret_cast<float *>(d_vt_ + s.desc.p_off + start);
            CK(cudaMemcpyAsync(stx, x, 12ull * n, cudaMemcpyHostToDevice, st));
            if (v) CK(cudaMemcpyAsync(stv, v, 12ull * n, cudaMemcpyHostToDevice, st));
            sx = stx;
            sv = v ? stv : nullptr;
        }
        launch_aos3_to_f4(sx, dx, n, st);
        if (sv) launch_aos3_to_f4(sv, dv, n, st);
        else CK(cudaMemsetAsync(dv, 0, 16ull * n, st));
        CK(cudaGetLastError());
    }
    // ids: a fresh set numbers the particles 0..n-1; an append continues
    // from the scene's device-side counter
    launch_assign_ids(d_id_ + s.desc.p_off + start, d_next_id_ + id, n, append, st);
    CK(cudaGetLastError());
    s.perm_valid = false;
    const uint32_t total = start + n;
    launch_set_u32(d_scene_num_ + id, total, st);
    CK(cudaGetLastError());
    if (s.num_upper != total) dirty_tiles_ = true;
    s.num_upper = total;
    return PBF_SUCCESS;
}

void Batch::scene_ids(std::vector<uint32_t> &ids) const
{
    ids.clear();
    for (uint32_t k = 0; k < scenes_.size(); ++k)
        if (scenes_[k].active) ids.push_back(k);
}

pbf_status Batch::upload_all(const uint32_t *counts, const float *x, const float *v, bool src_dev, cudaStream_t st)
{
    NvtxRange range("pbf set all");
    CK(cudaSetDevice(device_));
    std::vector<uint32_t> ids;
    scene_ids(ids);
    if (ids.empty()) return PBF_SUCCESS;
    if (!x) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = stage_counts(counts, ids, st);
    if (rc != PBF_SUCCESS) return rc;
    uint64_t tot = 0;
    for (uint32_t id : ids) tot += scenes_[id].num_upper;
    const float *sx = x, *sv = v;
    if (!src_dev && tot) {
        CK(cudaMemcpyAsync(d_xs_, x, 12 * tot, cudaMemcpyHostToDevice, st));
        sx = reinterpret_cast<const float *>(d_xs_);
        if (v) {
            CK(cudaMemcpyAsync(d_vt_, v, 12 * tot, cudaMemcpyHostToDevice, st));
            sv = reinterpret_cast<const float *>(d_vt_);
        }
    }
    if (ctrl_.n_tiles) launch_unpack(args(), shape_for(tile_), d_pack_off_, sx, sv, st);
    CK(cudaGetLastError());
    // k_unpack restarts the id counters of scenes with particles; the rest here
    for (size_t k = 0; k < ids.size(); ++k)
        if (scenes_[ids[k]].num_upper == 0) launch_set_u32(d_next_id_ + ids[k], 0, st);
    CK(cudaGetLastError());
    return PBF_SUCCESS;
}

pbf_status Batch::stage_counts(const uint32_t *counts, const std::vector<uint32_t> &ids, cudaStream_t st)
{
    for (size_t k = 0; k < ids.size(); ++k) {
        const uint32_t c = counts ? counts[k] : scenes_[ids[k]].num_upper;
        if (c > scenes_[ids[k]].desc.capacity) return PBF_ERROR_CAPACITY;
    }
    // the pinned scratch may still feed a previous copy
    CK(cudaEventSynchronize(small_done_));
    const size_t ns = scenes_.size();
    uint32_t *pack = h_small_, *nums = h_small_ + max_scenes_;
    std::memset(h_small_, 0, 8ull * max_scenes_);
    uint64_t tot = 0;
    for (size_t k = 0; k < ids.size(); ++k) {
        SceneHost &s = scenes_[ids[k]];
        const uint32_t c = counts ? counts[k] : s.num_upper;
        pack[ids[k]] = (uint32_t)tot;
        nums[ids[k]] = c;
        tot += c;
        if (s.num_upper != c) dirty_tiles_ = true;
        s.num_upper = c;
        s.perm_valid = false;
    }
    CK(cudaMemcpyAsync(d_pack_off_, pack, 4 * ns, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_scene_num_, nums, 4 * ns, cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(small_done_, st));
    return upload(st);
}

pbf_status Batch::step_packed(int iters, const uint32_t *counts, const float *x, const float *v, cudaStream_t st)
{
    NvtxRange range("pbf step packed");
    if (iters < 0 || iters > 1000) return PBF_ERROR_INVALID_ARGUMENT;
    CK(cudaSetDevice(device_));
    std::vector<uint32_t> ids;
    scene_ids(ids);
    if (ids.empty()) {
        last_launches_ = 0;
        return PBF_SUCCESS;
    }
    if (!x) return PBF_ERROR_INVALID_ARGUMENT;
    pbf_status rc = stage_counts(counts, ids, st);
    if (rc != PBF_SUCCESS) return rc;
    // the prediction restarts the id counters of scenes with particles; the rest here
    for (uint32_t id : ids)
        if (scenes_[id].num_upper == 0) launch_set_u32(d_next_id_ + id, 0, st);
    if (ctrl_.n_tiles == 0) {
        last_launches_ = 0;
        return PBF_SUCCESS;
    }
    launch_set_packed_in(d_pin_, x, v, st);
    CK(cudaGetLastError());
    rc = run(iters, st, true, true);
    if (rc == PBF_SUCCESS)
        for (auto &s : scenes_) s.perm_valid = s.active;
    return rc;
}

pbf_status Batch::download_all(uint32_t *counts, float *x, float *v, bool dst_dev, cudaStream_t st)
{
    NvtxRange range("pbf get all");
    std::vector<uint32_t> nums, fl, ids;
    pbf_status rc = read_all(nums, fl, false, st);
    if (rc != PBF_SUCCESS) return rc;
    scene_ids(ids);
    if (ids.empty()) return PBF_SUCCESS;
    CK(cudaEventSynchronize(small_done_));
    uint32_t *pack = h_small_;
    uint64_t tot = 0;
    for (size_t k = 0; k < ids.size(); ++k) {
        pack[ids[k]] = (uint32_t)tot;
        if (counts) counts[k] = nums[ids[k]];
        tot += nums[ids[k]];
    }
    CK(cudaMemcpyAsync(d_pack_off_, pack, 4 * scenes_.size(), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(small_done_, st));
    rc = upload(st);
    if (rc != PBF_SUCCESS) return rc;
    if (!tot) return PBF_SUCCESS;
    float *dx = x, *dv = v;
    if (!dst_dev) {
        dx = x ? reinterpret_cast<float *>(d_xs_) : nullptr;
        dv = v ? reinterpret_cast<float *>(d_vt_) : nullptr;
    }
    launch_pack(args(), shape_for(tile_), d_pack_off_, dx, dv, st);
    CK(cudaGetLastError());
    if (!dst_dev) {
        if (x) CK(cudaMemcpyAsync(x, dx, 12 * tot, cudaMemcpyDeviceToHost, st));
        if (v) CK(cudaMemcpyAsync(v, dv, 12 * tot, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    return PBF_SUCCESS;
}

pbf_status Batch::download_all_async(uint32_t *counts_dev, float *x_dev, float *v_dev, cudaStream_t st)
{
    NvtxRange range("pbf get all async");
    CK(cudaSetDevice(device_));
    pbf_status rc = upload(st);
    if (rc != PBF_SUCCESS) return rc;
    if (n_active_ == 0) return PBF_SUCCESS;
    launch_pack_offsets(d_active_, n_active_, d_scene_num_, d_pack_off_, counts_dev, st);
    if (ctrl_.n_tiles && (x_dev || v_dev)) launch_pack(args(), shape_for(tile_), d_pack_off_, x_dev, v_dev, st);
    CK(cudaGetLastError());
    return PBF_SUCCESS;
}

pbf_status Batch::set_scene_params(uint32_t id, const pbf_params &p)
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    SceneHost &s = scenes_[id];
    SceneDesc d;
    uint32_t g[3];
    pbf_params q = p;
    // the hash grid is part of the allocation; keep it
    q.grid_size[0] = s.desc.gx;
    q.grid_size[1] = s.desc.gy;
    q.grid_size[2] = s.desc.gz;
    pbf_status rc = derive_desc(q, nullptr, &d, g);
    if (rc != PBF_SUCCESS) return rc;
    if (d.ncell != s.desc.ncell || q.max_pair_particle_num > max_pair_) return PBF_ERROR_INVALID_ARGUMENT;
    d.p_off = s.desc.p_off;
    d.capacity = s.desc.capacity;
    d.list16 = s.desc.list16;
    d.c_off = s.desc.c_off;
    d.b_off = s.desc.b_off;
    d.builtin_sphere = s.desc.builtin_sphere;
    d.n_inner = s.desc.n_inner;
    d.n_outer = s.desc.n_outer;
    d.n_planes = s.desc.n_planes;
    d.clear_box = s.desc.clear_box;
    for (int c = 0; c < 3; ++c) {
        d.amin[c] = s.desc.amin[c];
        d.amax[c] = s.desc.amax[c];
        d.box_lo[c] = s.desc.box_lo[c];
        d.box_hi[c] = s.desc.box_hi[c];
    }
    s.desc = d;
    s.params = p;
    dirty_desc_ = true;
    return PBF_SUCCESS;
}

pbf_status Batch::set_scene_boundary(uint32_t id, const pbf_boundary_t *b)
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    SceneHost &s = scenes_[id];
    std::vector<float4> prims;
    fill_boundary(b, prims);
    if (prims.size() != s.bnd_len) {
        balloc_.release(s.bnd_off, s.bnd_len);
        uint64_t bo;
        if (!balloc_.alloc(prims.size(), &bo)) {
            s.bnd_len = 0;
            s.desc.builtin_sphere = 1;
            s.desc.n_inner = s.desc.n_outer = s.desc.n_planes = 0;
            set_clear_box(s.desc, nullptr);
            return PBF_ERROR_OUT_OF_MEMORY;
        }
        s.bnd_off = bo;
        s.bnd_len = prims.size();
    }
    for (size_t k = 0; k < prims.size(); ++k) bnd_host_[s.bnd_off + k] = prims[k];
    s.desc.b_off = (uint32_t)s.bnd_off;
    s.desc.builtin_sphere = b ? 0u : 1u;
    s.desc.n_inner = b ? b->n_inner : 0;
    s.desc.n_outer = b ? b->n_outer : 0;
    s.desc.n_planes = b ? b->n_planes : 0;
    set_clear_box(s.desc, b);
    dirty_desc_ = true;
    dirty_bnd_ = true;
    return PBF_SUCCESS;
}

pbf_status Batch::set_scene_area(uint32_t id, const float amin[3], const float amax[3])
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    SceneHost &s = scenes_[id];
    bool changed = false;
    for (int c = 0; c < 3; ++c) {
        changed |= s.desc.amin[c] != amin[c] || s.desc.amax[c] != amax[c];
        s.desc.amin[c] = amin[c];
        s.desc.amax[c] = amax[c];
    }
    if (changed) dirty_desc_ = true;
    return PBF_SUCCESS;
}

void Batch::rebuild_tiles()
{
    tile_scene_.clear();
    tile_start_.clear();
    for (uint32_t k = 0; k < scenes_.size(); ++k) {
        const SceneHost &s = scenes_[k];
        if (!s.active) continue;
        for (uint32_t st = 0; st < s.num_upper; st += tile_) {
            tile_scene_.push_back(k);
            tile_start_.push_back(st);
        }
    }
    ctrl_.n_tiles = (uint32_t)tile_scene_.size();
    // cell tiles: every cell of every active scene, the deleted bucket included
    for (uint32_t k = 0; k < scenes_.size(); ++k) {
        const SceneHost &s = scenes_[k];
        if (!s.active) continue;
        for (uint32_t c0 = 0; c0 <= s.desc.ncell; c0 += cell_tile_) {
            tile_scene_.push_back(k);
            tile_start_.push_back(c0);
        }
    }
    ctrl_.n_cell_tiles = (uint32_t)tile_scene_.size() - ctrl_.n_tiles;
    ctrl_.n_cells = (uint32_t)calloc_.high_water();
    ctrl_.n_scenes = (uint32_t)scenes_.size();
}

pbf_status Batch::upload(cudaStream_t st)
{
    CK(cudaSetDevice(device_));
    if (dirty_desc_) {
        std::vector<SceneDesc> h(scenes_.size());
        for (size_t k = 0; k < scenes_.size(); ++k) h[k] = scenes_[k].desc;
        if (!h.empty())
            CK(cudaMemcpyAsync(d_scenes_, h.data(), sizeof(SceneDesc) * h.size(), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        dirty_desc_ = false;
    }
    if (dirty_bnd_) {
        const uint64_t hw = balloc_.high_water();
        if (hw) CK(cudaMemcpyAsync(d_bnd_, bnd_host_.data(), 16 * hw, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        dirty_bnd_ = false;
    }
    if (dirty_tiles_) {
        NvtxRange range("pbf upload tile lists");
        rebuild_tiles();
        if (tile_scene_.size() > max_tiles_) return PBF_ERROR_CAPACITY;
        if (!tile_scene_.empty()) {
            CK(cudaMemcpyAsync(d_tile_scene_, tile_scene_.data(), 4 * tile_scene_.size(), cudaMemcpyHostToDevice,
                               st));
            CK(cudaMemcpyAsync(d_tile_start_, tile_start_.data(), 4 * tile_start_.size(), cudaMemcpyHostToDevice,
                               st));
        }
        CK(cudaMemcpyAsync(d_ctrl_, &ctrl_, sizeof(Ctrl), cudaMemcpyHostToDevice, st));
        std::vector<uint32_t> ids;
        scene_ids(ids);
        n_active_ = (uint32_t)ids.size();
        if (n_active_) CK(cudaMemcpyAsync(d_active_, ids.data(), 4ull * n_active_, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        dirty_tiles_ = false;
    }
    return PBF_SUCCESS;
}

LaunchShape Batch::shape_for(uint32_t tile) const
{
    LaunchShape sh;
    sh.tile = tile;
    sh.chunk = chunk_;
    const Occupancy o = occupancy(tile, chunk_);
    // Grids follow the tile counts rounded up to a power of two: every kernel
    // loops over the device-resident counts (surplus blocks exit at once), so
    // a captured graph survives scenes coming and going until a count
    // crosses a power of two (a served stream changes its scene set many
    // times a second).
    auto pow2 = [](uint32_t v) {
        uint32_t p = 1;
        while (p < v) p <<= 1;
        return p;
    };
    const uint32_t nt = std::max<uint32_t>(1, ctrl_.n_tiles);
    const uint32_t ntb = pow2(nt);
    auto g = [&](uint32_t bps) { return std::min<uint32_t>((uint32_t)sms_ * std::max<uint32_t>(1, bps), ntb); };
    sh.grid = g(o.light);
    sh.grid_nb = ntb;  // a block per tile: the walk's cost varies per tile, and fresh blocks balance it
    sh.grid_lambda = g(o.lambda);
    sh.grid_dp = g(o.dp);
    sh.grid_omega = g(o.omega);
    sh.grid_apply = g(o.apply);
    sh.grid_xsph = g(o.xsph);
    sh.grid_cells = pow2(std::max<uint32_t>(1, ctrl_.n_cell_tiles));  // a block per cell tile
    sh.cell_tile = cell_tile_;
    sh.small = (uint64_t)nt * tile <= kSmallStep ? 1u : 0u;
    sh.grid_split = std::min<uint32_t>((uint32_t)sms_ * std::max<uint32_t>(1, o.split), ntb * (tile / (256 / kSplit)));
    const uint32_t scan_tiles = std::max<uint32_t>(1, (ctrl_.n_cells + kScanTile - 1) / kScanTile);
    sh.scan_grid = std::min<uint32_t>(pow2(scan_tiles), (uint32_t)sms_ * 8);
    if (ctrl_.n_cells <= kSingleScanMax) sh.scan_grid = 0;  // one-block scan
    {  // the block's lists in shared memory when they fit
        const uint64_t b = (uint64_t)tile * (max_pair_ - 1u) * 4u;
        sh.nb_smem = b <= kNbSmemMax ? (uint32_t)b : 0u;
    }
    sh.scan_rounds = 0;
    if (sh.scan_grid == 0) {  // the table's rounds of 1024 cells, if they fit in registers
        const uint32_t r = std::max<uint32_t>(1, (ctrl_.n_cells + 1023u) / 1024u);
        if (r <= 16) sh.scan_rounds = r;
    }
    return sh;
}

StepArgs Batch::args() const
{
    StepArgs a;
    a.scenes = d_scenes_;
    a.tile_scene = d_tile_scene_;
    a.tile_start = d_tile_start_;
    a.ctrl = d_ctrl_;
    a.scene_num = d_scene_num_;
    a.flags = d_flags_;
    a.x = d_x_;
    a.v = d_v_;
    a.xs = d_xs_;
    a.key = d_key_;
    a.slot = d_slot_;
    a.tmp = d_tmp_;
    a.perm = d_perm_;
    a.count = d_count_;
    a.offsets = d_offsets_;
    a.bsum = d_bsum_;
    a.xa = d_xa_;
    a.xb = d_xb_;
    a.xold = d_xold_;
    a.id = d_id_;
    a.cls = d_cls_;
    a.wx = d_wx_;
    a.wpos = d_wpos_;
    a.dense = d_dense_;
    a.mid = d_mid_;
    a.chist = d_chist_;
    a.id_tmp = d_id_tmp_;
    a.next_id = d_next_id_;
    a.lam = d_lam_;
    a.nbr = d_nbr_;
    a.nnb = d_nnb_;
    a.selfat = d_self_;
    a.w = d_w_;
    a.vt = d_vt_;
    a.xv = d_xv_;
    a.bnd = d_bnd_;
    a.nbr_stride = max_particles_;
    a.pin = d_pin_;
    a.pack_off = d_pack_off_;
    return a;
}

uint32_t Batch::post_modes() const
{
    bool x_off = false, x_walk = false, x_list = false, v_ref = false, v_text = false, l16 = false, l32 = false;
    for (auto &s : scenes_)
        if (s.active) {
            l16 |= s.desc.list16 != 0;
            l32 |= s.desc.list16 == 0;
            x_off |= s.desc.xsph_mode == PBF_XSPH_OFF;
            x_walk |= s.desc.xsph_mode == PBF_XSPH_WALK;
            x_list |= s.desc.xsph_mode == PBF_XSPH_LIST;
            v_ref |= s.desc.vort_mode == PBF_VORTICITY_REFERENCE;
            v_text |= s.desc.vort_mode == PBF_VORTICITY_TEXTBOOK;
        }
    uint32_t m = 0;
    if (x_walk) m |= kPostXsphWalk;
    // the list-form XSPH kernel also copies the velocities of scenes without
    // XSPH when some scene of the batch has it
    if (x_list || (x_off && x_walk)) m |= kPostXsphList;
    if (v_ref) m |= kPostVortReference;
    if (v_text) m |= kPostVortTextbook;
    if (l16) m |= kPostList16;
    if (l32) m |= kPostList32;
    return m;
}

pbf_status Batch::run(int iters, cudaStream_t st, bool allow_graph, bool packed)
{
    const LaunchShape sh = shape_for(tile_);
    const uint32_t modes = post_modes();
    const int f = packed ? 1 : 0;
    if (allow_graph && graph_mode_) {
        GraphKey k;
        k.iters = iters;
        k.modes = modes;
        k.shape = sh;
        if (!exec_[f] || !(k == key_[f])) {
            if (exec_[f]) {
                cudaGraphExecDestroy(exec_[f]);
                exec_[f] = nullptr;
            }
            CK(cudaStreamBeginCapture(cap_stream_, cudaStreamCaptureModeThreadLocal));
            graph_launches_[f] = enqueue_step(args(), sh, iters, modes, cap_stream_, nullptr, packed);
            cudaGraph_t g = nullptr;
            CK(cudaStreamEndCapture(cap_stream_, &g));
            cudaError_t e = cudaGraphInstantiate(&exec_[f], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                exec_[f] = nullptr;
                set_last_error("cudaGraphInstantiate", e);
                return PBF_ERROR_CUDA;
            }
            key_[f] = k;
        }
        CK(cudaGraphLaunch(exec_[f], st));
        last_launches_ = graph_launches_[f];
    } else {
        last_launches_ = enqueue_step(args(), sh, iters, modes, st, nullptr, packed);
    }
    CK(cudaGetLastError());
    return PBF_SUCCESS;
}

namespace {
struct EventHook : StepHook {
    cudaStream_t st;
    std::vector<cudaEvent_t> ev;
    std::vector<std::string> names;
    void launched(const char *name) override
    {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, st);
        ev.push_back(e);
        names.emplace_back(name);
    }
};
}  // namespace

pbf_status Batch::profile_step(int iters, cudaStream_t st, float *ms, char *names, uint32_t max, uint32_t *n)
{
    if (iters < 0 || iters > 1000 || !n) return PBF_ERROR_INVALID_ARGUMENT;
    CK(cudaSetDevice(device_));
    pbf_status rc = upload(st);
    if (rc != PBF_SUCCESS) return rc;
    *n = 0;
    if (ctrl_.n_tiles == 0) return PBF_SUCCESS;
    EventHook hook;
    hook.st = st;
    cudaEvent_t e0;
    CK(cudaEventCreate(&e0));
    CK(cudaEventRecord(e0, st));
    last_launches_ = enqueue_step(args(), shape_for(tile_), iters, post_modes(), st, &hook);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    cudaEvent_t prev = e0;
    for (size_t k = 0; k < hook.ev.size(); ++k) {
        float t = 0.f;
        cudaEventElapsedTime(&t, prev, hook.ev[k]);
        if (k < max) {
            if (ms) ms[k] = t;
            if (names) {
                std::strncpy(names + 64 * k, hook.names[k].c_str(), 63);
                names[64 * k + 63] = 0;
            }
        }
        prev = hook.ev[k];
    }
    *n = (uint32_t)std::min<size_t>(hook.ev.size(), max);
    for (auto e : hook.ev) cudaEventDestroy(e);
    cudaEventDestroy(e0);
    return PBF_SUCCESS;
}

pbf_status Batch::step(int iters, cudaStream_t st)
{
    NvtxRange range("pbf step");
    if (iters < 0 || iters > 1000) return PBF_ERROR_INVALID_ARGUMENT;
    CK(cudaSetDevice(device_));
    pbf_status rc = upload(st);
    if (rc != PBF_SUCCESS) return rc;
    if (ctrl_.n_tiles == 0) {
        last_launches_ = 0;
        return PBF_SUCCESS;
    }
    rc = run(iters, st, true);
    if (rc == PBF_SUCCESS)
        for (auto &s : scenes_) s.perm_valid = s.active;
    return rc;
}

pbf_status Batch::scene_arrays(uint32_t id, SceneArrays *o)
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    const SceneDesc &d = scenes_[id].desc;
    o->x = d_x_ + d.p_off;
    o->v = d_v_ + d.p_off;
    o->id = d_id_ + d.p_off;
    o->perm = d_perm_ + d.p_off;
    o->stage = d_xs_ + d.p_off;
    o->scene_num = d_scene_num_ + id;
    o->next_id = d_next_id_ + id;
    o->flags = d_flags_ + id;
    o->offsets = d_offsets_ + d.c_off;
    o->p_off = d.p_off;
    o->capacity = d.capacity;
    o->c_off = d.c_off;
    o->ncell = d.ncell;
    return PBF_SUCCESS;
}

void Batch::note_append(uint32_t id, uint32_t n)
{
    SceneHost &s = scenes_[id];
    const uint32_t up = (uint32_t)std::min<uint64_t>((uint64_t)s.num_upper + n, s.desc.capacity);
    if (up != s.num_upper) dirty_tiles_ = true;
    s.num_upper = up;
    s.perm_valid = false;
}

pbf_status Batch::get_num(uint32_t id, uint32_t *num, cudaStream_t st)
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    CK(cudaSetDevice(device_));
    uint32_t n = 0;
    CK(cudaMemcpyAsync(&n, d_scene_num_ + id, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (n != scenes_[id].num_upper) {
        scenes_[id].num_upper = n;
        dirty_tiles_ = true;
    }
    *num = n;
    return PBF_SUCCESS;
}

pbf_status Batch::get_particles(uint32_t id, float *x, float *v, uint32_t *num, bool dst_dev, cudaStream_t st)
{
    uint32_t n = 0;
    pbf_status rc = get_num(id, &n, st);
    if (rc != PBF_SUCCESS) return rc;
    if (num) *num = n;
    if (!n) return PBF_SUCCESS;
    const SceneHost &s = scenes_[id];
    float *stage = reinterpret_cast<float *>(d_xs_ + s.desc.p_off);  // xs is free between steps
    float4 *srcs[2] = {d_x_ + s.desc.p_off, d_v_ + s.desc.p_off};
    float *dsts[2] = {x, v};
    for (int k = 0; k < 2; ++k) {
        if (!dsts[k]) continue;
        if (dst_dev) {
            launch_f4_to_aos3(srcs[k], dsts[k], n, st);
            CK(cudaGetLastError());
        } else {
            launch_f4_to_aos3(srcs[k], stage, n, st);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(dsts[k], stage, 12ull * n, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
    }
    return PBF_SUCCESS;
}

pbf_status Batch::get_flags(uint32_t id, uint32_t *flags, bool clear, cudaStream_t st)
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    CK(cudaSetDevice(device_));
    uint32_t f = 0;
    CK(cudaMemcpyAsync(&f, d_flags_ + id, 4, cudaMemcpyDeviceToHost, st));
    if (clear) CK(cudaMemsetAsync(d_flags_ + id, 0, 4, st));
    CK(cudaStreamSynchronize(st));
    *flags = f;
    return PBF_SUCCESS;
}

pbf_status Batch::read_all(std::vector<uint32_t> &nums, std::vector<uint32_t> &flags, bool clear_flags,
                           cudaStream_t st)
{
    CK(cudaSetDevice(device_));
    const size_t n = scenes_.size();
    nums.assign(n, 0);
    flags.assign(n, 0);
    if (!n) return PBF_SUCCESS;
    CK(cudaMemcpyAsync(nums.data(), d_scene_num_, 4 * n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(flags.data(), d_flags_, 4 * n, cudaMemcpyDeviceToHost, st));
    if (clear_flags) CK(cudaMemsetAsync(d_flags_, 0, 4 * n, st));
    CK(cudaStreamSynchronize(st));
    for (size_t k = 0; k < n; ++k)
        if (scenes_[k].active && scenes_[k].num_upper != nums[k]) {
            scenes_[k].num_upper = nums[k];
            dirty_tiles_ = true;
        }
    return PBF_SUCCESS;
}

pbf_status Batch::get_debug(uint32_t id, uint32_t *sorted_hash, uint32_t *perm, uint32_t *cell_start,
                            uint32_t *cell_end, uint32_t *neighbor_list, uint32_t *n_in_out, cudaStream_t st)
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    CK(cudaSetDevice(device_));
    CK(cudaStreamSynchronize(st));
    const SceneDesc &d = scenes_[id].desc;
    const uint64_t C = d.ncell;
    std::vector<uint32_t> off(C + 2);
    CK(cudaMemcpy(off.data(), d_offsets_ + d.c_off, 4 * (C + 2), cudaMemcpyDeviceToHost));
    const uint32_t base = off[0];
    const uint32_t n_in = off[C + 1] - base;
    const uint32_t live = off[C] - base;
    if (n_in_out) *n_in_out = n_in;
    std::vector<uint32_t> key(n_in), pm(n_in);
    if (n_in) {
        CK(cudaMemcpy(key.data(), d_key_ + d.p_off, 4ull * n_in, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(pm.data(), d_perm_ + d.p_off, 4ull * n_in, cudaMemcpyDeviceToHost));
    }
    if (perm) std::memcpy(perm, pm.data(), 4ull * n_in);
    if (sorted_hash)
        for (uint32_t p = 0; p < n_in; ++p) sorted_hash[p] = key[pm[p]];
    if (cell_start || cell_end)
        for (uint64_t c = 0; c < C; ++c) {
            const bool empty = off[c] == off[c + 1];
            if (cell_start) cell_start[c] = empty ? 0xFFFFFFFFu : off[c] - base;
            if (cell_end) cell_end[c] = empty ? 0xFFFFFFFFu : off[c + 1] - base;
        }
    if (neighbor_list) {
        const uint32_t mp = d.cap + 1;
        const uint64_t padded = ((uint64_t)live + 31) / 32 * 32;
        std::fill(neighbor_list, neighbor_list + padded * mp, 0xFFFFFFFFu);
        std::vector<uint8_t> nn(live), self(live);
        std::vector<uint32_t> quads(4ull * live);
        if (live) {
            CK(cudaMemcpy(nn.data(), d_nnb_ + d.p_off, live, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(self.data(), d_self_ + d.p_off, live, cudaMemcpyDeviceToHost));
        }
        auto at = [&](uint32_t k, uint32_t p) -> uint32_t & {
            return neighbor_list[((uint64_t)k << 5) + (p & 31) + (uint64_t)((p >> 5) << 5) * mp];
        };
        // rows of 16 bytes per particle: quads of 4 u32 sorted slots, or
        // octs of 8 u16 scene-local indices (scenes of at most kList16Max
        // slots).  Stored entry k is list slot k, or k + 1 from the particle's
        // own position on (the particle itself is listed but not stored).
        const uint32_t per_row = d.list16 ? 8u : 4u;
        for (uint32_t kq = 0; per_row * kq < d.cap && live; ++kq) {  // slots per_row*kq.. of every particle
            CK(cudaMemcpy(quads.data(), d_nbr_ + 4ull * ((uint64_t)kq * max_particles_ + d.p_off), 16ull * live,
                          cudaMemcpyDeviceToHost));
            const uint16_t *octs = reinterpret_cast<const uint16_t *>(quads.data());
            for (uint32_t k = per_row * kq; k < per_row * kq + per_row && k < d.cap; ++k)
                for (uint32_t p = 0; p < live; ++p)
                    if (k < nn[p])
                        at(k + (k >= self[p] ? 1u : 0u), p) =
                            d.list16 ? octs[8ull * p + (k & 7)] : quads[4ull * p + (k & 3)] - d.p_off;
        }
        for (uint32_t p = 0; p < live; ++p)
            if (self[p] != kNotListed) at(self[p], p) = p;
    }
    return PBF_SUCCESS;
}

pbf_status Batch::import_x_device(uint32_t id, const float *x_dev, uint32_t n, cudaStream_t st)
{
    if (id >= scenes_.size() || !scenes_[id].active) return PBF_ERROR_NOT_FOUND;
    if (n > scenes_[id].desc.capacity) return PBF_ERROR_CAPACITY;
    launch_aos3_to_f4(x_dev, d_x_ + scenes_[id].desc.p_off, n, st);
    CK(cudaGetLastError());
    return PBF_SUCCESS;
}

pbf_status Batch::export_x_device(uint32_t id, float *x_dev, cudaStream_t st)
{
    uint32_t n = 0;
    pbf_status rc = get_num(id, &n, st);
    if (rc != PBF_SUCCESS) return rc;
    launch_f4_to_aos3(d_x_ + scenes_[id].desc.p_off, x_dev, n, st);
    CK(cudaGetLastError());
    return PBF_SUCCESS;
}

pbf_status Batch::set_tile(uint32_t tile)
{
    if (tile != 64 && tile != 128 && tile != 256 && tile != 512) return PBF_ERROR_INVALID_ARGUMENT;
    if (tile != tile_) {
        tile_ = tile;
        dirty_tiles_ = true;
    }
    return PBF_SUCCESS;
}

pbf_status Batch::set_chunk(uint32_t chunk)
{
    if (chunk != 4 && chunk != 8) return PBF_ERROR_INVALID_ARGUMENT;
    chunk_ = chunk;
    return PBF_SUCCESS;
}

pbf_status Batch::set_cell_tile(uint32_t cells)
{
    if (cells < kCellTileMin || cells > kCellTileMax || (cells & (cells - 1))) return PBF_ERROR_INVALID_ARGUMENT;
    if (cells != cell_tile_) dirty_tiles_ = true;
    cell_tile_ = cells;
    return PBF_SUCCESS;
}

pbf_status Batch::autotune(int iters, cudaStream_t st, uint32_t *chosen)
{
    NvtxRange range("pbf autotune");
    CK(cudaSetDevice(device_));
    pbf_status rc = upload(st);
    if (rc != PBF_SUCCESS) return rc;
    if (ctrl_.n_tiles == 0) {
        if (chosen) *chosen = tile_;
        return PBF_SUCCESS;
    }
    const uint64_t hw = palloc_.high_water();
    float4 *sx = nullptr, *sv = nullptr;
    uint32_t *sn = nullptr, *sf = nullptr;
    CK(cudaMalloc(&sx, 16 * std::max<uint64_t>(hw, 1)));
    CK(cudaMalloc(&sv, 16 * std::max<uint64_t>(hw, 1)));
    CK(cudaMalloc(&sn, 4ull * max_scenes_));
    CK(cudaMalloc(&sf, 4ull * max_scenes_));
    auto save = [&]() -> cudaError_t {
        cudaMemcpyAsync(sx, d_x_, 16 * hw, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(sv, d_v_, 16 * hw, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(sn, d_scene_num_, 4ull * max_scenes_, cudaMemcpyDeviceToDevice, st);
        return cudaMemcpyAsync(sf, d_flags_, 4ull * max_scenes_, cudaMemcpyDeviceToDevice, st);
    };
    auto restore = [&]() -> cudaError_t {
        cudaMemcpyAsync(d_x_, sx, 16 * hw, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(d_v_, sv, 16 * hw, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(d_scene_num_, sn, 4ull * max_scenes_, cudaMemcpyDeviceToDevice, st);
        return cudaMemcpyAsync(d_flags_, sf, 4ull * max_scenes_, cudaMemcpyDeviceToDevice, st);
    };
    CK(save());
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const uint32_t cands[] = {128, 256, 512, 64};
    const uint32_t chunks[] = {8, 4};
    uint32_t best = tile_, best_chunk = chunk_;
    float best_ms = 1e30f;
    for (uint32_t t : cands)
    for (uint32_t ch : chunks) {
        set_tile(t);
        chunk_ = ch;
        rc = upload(st);
        if (rc != PBF_SUCCESS) break;
        for (int r = 0; r < 2; ++r) run(iters, st, false);  // warm-up
        CK(cudaEventRecord(e0, st));
        for (int r = 0; r < 8; ++r) run(iters, st, false);
        CK(cudaEventRecord(e1, st));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            best_ms = ms;
            best = t;
            best_chunk = ch;
        }
        CK(restore());
    }
    set_tile(best);
    chunk_ = best_chunk;
    // then the cells per CTA of the per-cell rank (large steps only rank per cell)
    uint32_t best_cells = cell_tile_;
    if (rc == PBF_SUCCESS && !shape_for(best).small) {
        best_ms = 1e30f;
        for (uint32_t c : {256u, 128u, 512u, 64u}) {
            set_cell_tile(c);
            rc = upload(st);
            if (rc != PBF_SUCCESS) break;
            for (int r = 0; r < 2; ++r) run(iters, st, false);
            CK(cudaEventRecord(e0, st));
            for (int r = 0; r < 8; ++r) run(iters, st, false);
            CK(cudaEventRecord(e1, st));
            CK(cudaEventSynchronize(e1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best_ms) {
                best_ms = ms;
                best_cells = c;
            }
            CK(restore());
        }
    }
    set_cell_tile(best_cells);
    rc = upload(st);
    CK(cudaStreamSynchronize(st));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sx);
    cudaFree(sv);
    cudaFree(sn);
    cudaFree(sf);
    if (chosen) *chosen = best;
    return rc;
}

}  // namespace pbf103
