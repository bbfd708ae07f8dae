// Host runtime of the PBF engine: device arena, scene table, tile list,
// CUDA-graph cache and autotuner.  The plain single-scene handle is a batch
// with one scene, so both paths run the same kernels.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "pbf103.h"
#include "pbf_internal.h"

struct pbf_boundary_t {
    std::vector<float4> prims;  // inner spheres, outer spheres, planes (point, normal)
    uint32_t n_inner = 0, n_outer = 0, n_planes = 0;
};

namespace pbf103 {

// First-fit allocator over [0, size) for particle and cell ranges.
class RangeAllocator {
public:
    explicit RangeAllocator(uint64_t size = 0) { reset(size); }
    void reset(uint64_t size);
    bool alloc(uint64_t n, uint64_t *off);
    void release(uint64_t off, uint64_t n);
    uint64_t high_water() const;
    uint64_t size() const { return size_; }
    uint64_t free_total() const;

private:
    uint64_t size_ = 0;
    std::map<uint64_t, uint64_t> free_;  // offset -> length
    std::map<uint64_t, uint64_t> used_;  // offset -> length
};

struct SceneHost {
    bool active = false;
    pbf_params params{};
    SceneDesc desc{};
    uint32_t num_upper = 0;   // host upper bound of the live count
    uint64_t cells = 0;       // ncell + 1 (deleted bucket)
    uint64_t bnd_len = 0;     // float4s in the boundary pool
    uint64_t bnd_off = 0;
    bool perm_valid = false;  // perm holds the last step's permutation of this scene's input
};

pbf_status derive_desc(const pbf_params &p, const float domain_end[3], SceneDesc *d, uint32_t grid[3]);
uint64_t bytes_per_particle(uint32_t max_pair);

class Batch {
public:
    Batch() = default;
    ~Batch();
    pbf_status init(uint32_t max_scenes, uint64_t max_particles, uint64_t max_cells, uint32_t max_pair,
                    int device);

    pbf_status add_scene(const pbf_params &p, uint32_t capacity, const float domain_end[3],
                         const pbf_boundary_t *b, const float amin[3], const float amax[3], const float *x,
                         const float *v, uint32_t n, bool src_dev, cudaStream_t st, uint32_t *id);
    pbf_status remove_scene(uint32_t id);
    pbf_status set_particles(uint32_t id, const float *x, const float *v, uint32_t n, bool src_dev, bool append,
                             cudaStream_t st);
    pbf_status set_scene_params(uint32_t id, const pbf_params &p);
    pbf_status set_scene_boundary(uint32_t id, const pbf_boundary_t *b);
    pbf_status set_scene_area(uint32_t id, const float amin[3], const float amax[3]);
    pbf_status step(int iters, cudaStream_t st);
    // upload_all from device buffers and step, without the unpack pass: the
    // step reads the packed input where it lies
    pbf_status step_packed(int iters, const uint32_t *counts, const float *x, const float *v, cudaStream_t st);
    pbf_status get_num(uint32_t id, uint32_t *num, cudaStream_t st);
    pbf_status get_particles(uint32_t id, float *x, float *v, uint32_t *num, bool dst_dev, cudaStream_t st);
    pbf_status get_flags(uint32_t id, uint32_t *flags, bool clear, cudaStream_t st);
    // live counts and flag words of every scene slot with one device read
    pbf_status read_all(std::vector<uint32_t> &nums, std::vector<uint32_t> &flags, bool clear_flags,
                        cudaStream_t st);
    pbf_status get_debug(uint32_t id, uint32_t *sorted_hash, uint32_t *perm, uint32_t *cell_start,
                         uint32_t *cell_end, uint32_t *neighbor_list, uint32_t *n_in, cudaStream_t st);
    // packed whole-batch moves (active scenes in slot order)
    void scene_ids(std::vector<uint32_t> &ids) const;
    pbf_status upload_all(const uint32_t *counts, const float *x, const float *v, bool src_dev, cudaStream_t st);
    pbf_status download_all(uint32_t *counts, float *x, float *v, bool dst_dev, cudaStream_t st);
    // the whole batch into device buffers with the packed offsets computed on
    // the device: no host synchronisation; counts_dev[k] for the k-th active scene
    pbf_status download_all_async(uint32_t *counts_dev, float *x_dev, float *v_dev, cudaStream_t st);
    pbf_status import_x_device(uint32_t id, const float *x_dev, uint32_t n, cudaStream_t st);
    // device arrays of one scene, for the particle-set operations (pbf_particles.cu)
    struct SceneArrays {
        float4 *x, *v;
        uint32_t *id, *perm, *scene_num, *next_id, *flags, *offsets;
        float4 *stage;         // the scene's xs slice: free between steps
        uint32_t p_off, capacity, c_off, ncell;
    };
    pbf_status scene_arrays(uint32_t id, SceneArrays *out);
    // host bookkeeping after a device-side append of up to n particles
    void note_append(uint32_t id, uint32_t n);
    bool perm_valid(uint32_t id) const { return id < scenes_.size() && scenes_[id].perm_valid; }
    pbf_status export_x_device(uint32_t id, float *x_dev, cudaStream_t st);
    pbf_status autotune(int iters, cudaStream_t st, uint32_t *chosen);
    // one step without a graph, with events between kernels
    pbf_status profile_step(int iters, cudaStream_t st, float *ms, char *names, uint32_t max, uint32_t *n);
    pbf_status set_tile(uint32_t tile);
    pbf_status set_chunk(uint32_t chunk);
    // cells per CTA of the per-cell rank (64, 128, 256 or 512)
    pbf_status set_cell_tile(uint32_t cells);
    uint32_t cell_tile() const { return cell_tile_; }
    uint32_t tile() const { return tile_; }
    uint32_t chunk() const { return chunk_; }
    void set_graph_mode(bool on) { graph_mode_ = on; }
    uint32_t last_launches() const { return last_launches_; }
    uint32_t num_scenes() const;
    const SceneHost *scene(uint32_t id) const;
    int device() const { return device_; }
    uint64_t arena_bytes() const { return arena_bytes_; }
    bool can_fit(uint32_t capacity, uint64_t cells, uint64_t bnd_len) const;
    // whether a scene of this size fits the empty arena at all
    bool ever_fits(uint32_t capacity, uint64_t cells) const
    {
        return capacity <= max_particles_ && cells <= max_cells_;
    }

private:
    pbf_status upload(cudaStream_t st);
    pbf_status run(int iters, cudaStream_t st, bool allow_graph, bool packed = false);
    // set the active scenes' counts (or keep them) and stage their pack offsets
    pbf_status stage_counts(const uint32_t *counts, const std::vector<uint32_t> &ids, cudaStream_t st);
    LaunchShape shape_for(uint32_t tile) const;
    uint32_t post_modes() const;  // kPost* bits of the active scenes
    void rebuild_tiles();
    StepArgs args() const;

    int device_ = 0;
    int sms_ = 152;
    uint32_t max_scenes_ = 0;
    uint64_t max_particles_ = 0, max_cells_ = 0;
    uint32_t max_pair_ = 30;
    uint64_t arena_bytes_ = 0;

    // device arena
    SceneDesc *d_scenes_ = nullptr;
    uint32_t *d_tile_scene_ = nullptr, *d_tile_start_ = nullptr;
    Ctrl *d_ctrl_ = nullptr;
    uint32_t *d_scene_num_ = nullptr, *d_flags_ = nullptr;
    float4 *d_x_ = nullptr, *d_v_ = nullptr, *d_xs_ = nullptr, *d_xa_ = nullptr, *d_xb_ = nullptr,
           *d_xold_ = nullptr, *d_w_ = nullptr, *d_vt_ = nullptr;
    uint32_t *d_key_ = nullptr, *d_slot_ = nullptr, *d_tmp_ = nullptr, *d_perm_ = nullptr;
    uint32_t *d_count_ = nullptr, *d_offsets_ = nullptr, *d_bsum_ = nullptr;
    float *d_lam_ = nullptr;
    uint32_t *d_nbr_ = nullptr;
    uint8_t *d_nnb_ = nullptr;
    uint8_t *d_self_ = nullptr;  // walk-order position of each particle in its own list
    float4 *d_bnd_ = nullptr;
    uint32_t *d_pack_off_ = nullptr;  // per-scene packed offsets for set_all/get_all
    uint32_t *d_active_ = nullptr;    // active scene slots in slot order (with the tile lists)
    uint32_t n_active_ = 0;
    uint32_t *d_id_ = nullptr, *d_id_tmp_ = nullptr;  // particle ids, phase order / sorted scratch
    uint32_t *d_next_id_ = nullptr;                   // per scene: next id to hand out
    uint8_t *d_cls_ = nullptr;                        // alias class per particle (input order)
    float4 *d_wx_ = nullptr;                          // class-grouped walk copy of the sorted positions
    float4 *d_xv_ = nullptr;                          // final (x, v) records, two float4 per particle slot
    uint64_t *d_chist_ = nullptr;                     // per cell: class counts of its bucket
    uint32_t *d_wpos_ = nullptr;                      // sorted slot -> walk-copy slot
    uint32_t *d_dense_ = nullptr;                     // dense-bucket queue
    uint32_t *d_mid_ = nullptr;                       // medium-bucket queue
    uint32_t *h_small_ = nullptr;     // pinned host scratch: pack offsets + counts
    cudaEvent_t small_done_ = nullptr;
    uint64_t bnd_capacity_ = 0;
    uint64_t max_tiles_ = 0;

    // host mirror
    std::vector<SceneHost> scenes_;
    std::vector<float4> bnd_host_;
    RangeAllocator palloc_, calloc_, balloc_;
    std::vector<uint32_t> tile_scene_, tile_start_;
    Ctrl ctrl_{};
    bool dirty_desc_ = true, dirty_tiles_ = true, dirty_bnd_ = true;

    // launch configuration and graph cache
    uint32_t tile_ = 256;
    uint32_t chunk_ = 8;
    uint32_t cell_tile_ = kCellTile;
    bool graph_mode_ = true;
    cudaStream_t cap_stream_ = nullptr;
    struct GraphKey {
        int iters = -1;
        uint32_t modes = 0;
        LaunchShape shape{};
        bool operator==(const GraphKey &o) const
        {
            return iters == o.iters && modes == o.modes && shape == o.shape;
        }
    };
    // one captured step per input form: [0] the phase, [1] packed input
    cudaGraphExec_t exec_[2] = {nullptr, nullptr};
    GraphKey key_[2];
    uint32_t graph_launches_[2] = {0, 0};
    uint32_t last_launches_ = 0;
    PackedIn *d_pin_ = nullptr;  // input buffers of the current packed-input step
};

}  // namespace pbf103

struct pbf_batch {
    pbf103::Batch b;
    std::mutex mu;
};

struct pbf_handle {
    pbf103::Batch b;
    uint32_t scene = 0;
    pbf_params params{};
    float domain_end[3] = {0, 0, 0};
    const pbf_boundary_t *last_boundary = nullptr;
    bool have_area = false;
    float amin[3] = {0, 0, 0}, amax[3] = {0, 0, 0};
};
