// Internal interfaces between the host runtime (pbf_engine.cu) and the
// device kernels (pbf_kernels.cu).  Not part of the C ABI.
#pragma once
#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

namespace pbf103 {

// A named NVTX range on the calling host thread for the life of the object
// (the host runtime's stages show up on a profiler's timeline; with no
// profiler attached a range costs a function-pointer test).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Per-scene constants, one 240-byte record per scene slot in device memory.
// Derived once on the host from pbf_params (the reference keeps these in
// __constant__ symbols and a function-static, pbf_position_update.cu:14-17,
// pbf_solve.cpp:92; here they are per scene so scenes never share state).
struct SceneDesc {
    uint32_t p_off;      // first particle slot of the scene in the flat arrays
    uint32_t capacity;   // particle slots owned by the scene
    uint32_t c_off;      // first cell of the scene in the flat cell arrays
    uint32_t ncell;      // Gx*Gy*Gz; cell ncell (local) is the deleted bucket
    uint32_t gx, gy, gz; // power-of-two hash grid
    uint32_t cap;        // neighbour slots usable (max_pair - 1)
    float cw;            // cell width
    float h2;            // h*h, neighbour acceptance
    float inv_h;         // 1/h
    float alpha;         // poly6 factor 1.56668147065 / h^3
    float beta;          // spiky-derivative factor -14.3239448745 / h^4
    float m;             // particle mass
    float inv_rho0;      // 1 / rest density
    float m2rho2;        // m^2 / rho0^2
    float relax;         // CFM epsilon
    float dt;
    float inv_dt;
    float inv_k;         // reference s_corr: 1 / W(0.4h)^4
    float inv_wdq;       // textbook s_corr: 1 / W(dq h)
    float scorr_k;
    int32_t scorr_n;
    int32_t tensile_mode;
    int32_t xsph_mode;
    int32_t vort_mode;
    float xsph_c;
    float vort_eps;
    float alpha6;        // 1.56668147065 * inv_h * inv_h * inv_h (Wpoly6 order)
    float h;
    float g[3];
    uint32_t max_coll;
    float amin[3];
    uint32_t b_off;      // first float4 of the scene's boundary primitives
    float amax[3];
    uint32_t n_inner;
    uint32_t n_outer;
    uint32_t n_planes;
    uint32_t builtin_sphere;
    float ih2;           // 1/h^2 (poly6 from r^2)
    // the pair passes sum W / alpha = t^3 and grad W / beta = s' d (t = 1 -
    // r^2/h^2, s' = (1 - r/h)^2 / r) and apply alpha and beta once per
    // particle, through these products (each computed in double):
    float tens_c;        // reference s_corr: 10 alpha^4 / W(0.4h)^4, the factor of (t^3)^4
    float scorr_c;       // textbook s_corr: k alpha^n / W(dq h)^n, the factor of (t^3)^n
    uint32_t list16;     // the neighbour list holds u16 scene-local indices (capacity <= 65,536)
    // clear_box: the boundary is planes with unit-axis normals only; a
    // projected position p with box_lo <= p <= box_hi hits none of them
    uint32_t clear_box;
    float box_lo[3], box_hi[3];
    float lam_c;         // alpha m / rho0: C = lam_c sum t^3 - 1
    float lam_k;         // m^2 beta^2 / rho0^2: the factor of |sum s' d|^2 + sum (s' r)^2
    float dp_k;          // m beta / rho0: delta-p = dp_k sum coef s' d
    uint32_t pad_[1];
};
static_assert(sizeof(SceneDesc) % 16 == 0, "SceneDesc must stay 16-byte sized");

// Device-resident launch control; lets a captured graph run on a scene set
// that changes between launches.
struct Ctrl {
    uint32_t n_tiles;       // particle tiles at the front of tile_scene/tile_start
    uint32_t n_cells;       // cell entries to scan (high-water mark of cell ranges)
    uint32_t n_scenes;
    uint32_t n_cell_tiles;  // cell tiles after them: LaunchShape::cell_tile cells of one scene each
};

// Device-resident pointers to a step's packed AoS float3 input
// (pbf_batch_step_packed): set by a one-thread kernel before each such step,
// so a captured graph reads whichever buffers the call names.
struct PackedIn {
    const float *x, *v;  // v may be null (zero velocities)
};

struct StepArgs {
    const SceneDesc *scenes;
    const uint32_t *tile_scene;   // tile -> scene
    const uint32_t *tile_start;   // tile -> first local particle index (cell tiles: first local cell)
    const Ctrl *ctrl;
    uint32_t *scene_num;          // particles per scene at step start
    uint32_t *flags;              // per-scene PBF_FLAG_* words
    float4 *x, *v;                // particle phase (sorted after each step)
    float4 *xs;                   // predicted positions, input order
    uint32_t *key, *slot, *tmp, *perm;
    uint32_t *count, *offsets, *bsum;
    float4 *xa, *xb, *xold;       // working positions (ping-pong) and sorted old x
    float *lam;
    uint32_t *nbr;                // nbr[k * nbr_stride + i]
    uint8_t *nnb;                 // list entries stored (the particle itself is not stored)
    uint8_t *selfat;              // position of the particle itself in its walk-order list, kNotListed if cut
    float4 *w, *vt;               // vorticity, XSPH velocity scratch
    float4 *xv;                   // final (x, v) side by side, 32 B per particle slot, for the list-form
                                  // vorticity pass's neighbour gathers (one 256-bit load per neighbour)
    const float4 *bnd;            // boundary primitives
    uint32_t *id, *id_tmp;        // particle ids (phase order) and their sorted copy
    uint8_t *cls;                 // alias class of each particle (input order)
    uint32_t *wpos;               // sorted slot -> walk-copy slot (mixed-class buckets only)
    uint32_t *dense;              // [0] count, then (cell, scene) pairs of buckets for k_dense_sort
    uint32_t *mid;                // the same for buckets of kMidMin+1 .. kDenseMin members
    float4 *wx;                   // walk copy of mixed-class buckets: grouped by class, .w = sorted slot
    uint64_t *chist;              // per cell: 8 x 8-bit class counts of its bucket, or kClassWhole
    uint32_t *next_id;            // per scene: id of the next particle added
    uint64_t nbr_stride;
    const PackedIn *pin;          // packed-input steps: the input buffers
    const uint32_t *pack_off;     // packed-input steps: first packed particle of each scene
};

struct LaunchShape {
    uint32_t tile;        // particles per tile = threads per block
    uint32_t grid;        // persistent grid (blocks) for the light tile kernels
    uint32_t scan_grid;   // grid for the scan kernels; 0 = the one-block scan
    uint32_t scan_rounds; // one-block scan: rounds of 1024 cells held in registers (1..16), 0 = looped
    uint32_t chunk;       // neighbours per chunk in the lambda / delta-p passes (4 or 8)
    // persistent grids of the heavy kernels, each from its own occupancy
    uint32_t grid_nb, grid_lambda, grid_dp, grid_omega, grid_apply, grid_xsph;
    uint32_t grid_cells;  // grid of k_rank_cells: a block of cell_tile threads per cell tile
    uint32_t cell_tile;   // cells per cell tile = threads per k_rank_cells block (autotuned)
    uint32_t small;       // latency-bound step (at most kSmallStep particle slots): split
                          // neighbour walk, per-particle rank, lambda kept in its own array
    uint32_t grid_split;  // grid of k_neighbors_split (blocks of 256 threads, 256 / kSplit particles each)
    uint32_t nb_smem;     // k_neighbors_lambda: bytes of shared memory for the block's lists (0 = stored directly)
    bool operator==(const LaunchShape &o) const
    {
        return tile == o.tile && grid == o.grid && scan_grid == o.scan_grid && scan_rounds == o.scan_rounds &&
               chunk == o.chunk &&
               grid_cells == o.grid_cells && cell_tile == o.cell_tile && small == o.small && grid_split == o.grid_split && nb_smem == o.nb_smem &&
               grid_nb == o.grid_nb && grid_lambda == o.grid_lambda && grid_dp == o.grid_dp &&
               grid_omega == o.grid_omega && grid_apply == o.grid_apply && grid_xsph == o.grid_xsph;
    }
};

// Resident blocks per SM of each kernel class at a tile size / chunk.
struct Occupancy {
    uint32_t light, nb, lambda, dp, omega, apply, xsph, cells, split;
};
Occupancy occupancy(uint32_t tile, uint32_t chunk);

// Called after every kernel launch of a step (per-kernel event timing).
struct StepHook {
    virtual void launched(const char *kernel_name) = 0;
    virtual ~StepHook() = default;
};

// Post-solve passes a step runs (bit set: some active scene needs that form).
enum : uint32_t {
    kPostXsphWalk = 1,       // XSPH, the reference's uncapped 27-cell walk
    kPostXsphList = 2,       // XSPH over the step's neighbour list (+ copy for scenes without XSPH)
    kPostVortReference = 4,  // vorticity, the reference's walk and kernel scaling
    kPostVortTextbook = 8,   // vorticity, textbook form over the neighbour list
    kPostList32 = 16,        // some scene keeps a u32 neighbour list (list forms launch per list format)
    kPostList16 = 32,        // some scene keeps a u16 neighbour list
};

// Enqueue one full solver step for every scene in the tile list.
// Returns the number of kernels launched.
// packed: the step reads its input positions and velocities from the packed
// AoS float3 buffers named in *a.pin (scene s from a.pack_off[s]) instead of
// the particle phase, and numbers the particles afresh, as an upload does.
uint32_t enqueue_step(const StepArgs &a, const LaunchShape &s, int iters, uint32_t post_modes,
                      cudaStream_t stream, StepHook *hook = nullptr, bool packed = false);
void launch_set_packed_in(PackedIn *dst, const float *x, const float *v, cudaStream_t st);

// Edge conversions between the ABI's AoS float3 and the internal float4.
void launch_aos3_to_f4(const float *src, float4 *dst, uint32_t n, cudaStream_t st);
void launch_f4_to_aos3(const float4 *src, float *dst, uint32_t n, cudaStream_t st);
void launch_set_u32(uint32_t *dst, uint32_t value, cudaStream_t st);
// pack_off[active[k]] = sum of the live counts of active[0..k), counts[k] =
// the live count of active[k], computed on the device (one block)
void launch_pack_offsets(const uint32_t *active, uint32_t n_active, const uint32_t *scene_num, uint32_t *pack_off,
                         uint32_t *counts, cudaStream_t st);
// ids of n particles added at dst: append ? *next_id + k : k; *next_id += / = n.
void launch_assign_ids(uint32_t *dst, uint32_t *next_id, uint32_t n, bool append, cudaStream_t st);
// Whole-batch moves between a packed AoS float3 buffer (active scenes in
// slot order, pack_off[s] = first packed particle of scene s) and the
// scene-sliced float4 phase arrays.  unpack uses the tile list (counts must
// already be in scene_num); pack writes the scene_num[s] first particles.
void launch_unpack(const StepArgs &a, const LaunchShape &sh, const uint32_t *pack_off, const float *src_x,
                   const float *src_v, cudaStream_t st);
void launch_pack(const StepArgs &a, const LaunchShape &sh, const uint32_t *pack_off, float *dst_x, float *dst_v,
                 cudaStream_t st);

// chist value of a bucket whose walk copy is in plain sorted order (more
// than 255 members, or a bucket left in atomic order)
constexpr uint64_t kClassWhole = ~0ull;

constexpr uint32_t kScanItemsPerWarp = 512;   // 32 lanes x 16
constexpr uint32_t kScanWarps = 8;
constexpr uint32_t kScanTile = kScanItemsPerWarp * kScanWarps;  // 4096 cells per scan tile
constexpr uint32_t kSingleScanMax = 65536;  // cells up to which one block scans the whole table
constexpr uint32_t kNbSmemMax = 96 * 1024;  // shared-memory budget for a k_neighbors_lambda block's lists
constexpr uint32_t kSplit = 4;  // small steps: lanes per particle in the split neighbour walk (blocks of 256)
constexpr uint32_t kCellTile = 256;         // default cells per cell tile = threads per k_rank_cells block
constexpr uint32_t kCellTileMin = 64, kCellTileMax = 512;  // the autotuner's range
constexpr uint32_t kMidMin = 16;            // buckets with more members are queued (warp or block per bucket)
constexpr uint32_t kSmallStep = 131072;     // particle slots up to which a step is latency bound
constexpr uint32_t kList16Max = 65536;      // scenes of at most this many slots keep u16 neighbour lists
constexpr uint8_t kNotListed = 0xFF;        // selfat of a particle the cap cut from its own list
constexpr uint32_t kWalkSpare = 4;          // spare float4 records after each per-particle array

}  // namespace pbf103
