/*
 * pbf103 — GB300-native Position-Based-Fluids solver step, C ABI.
 *
 * Drop-in surface for the reference simulator's solver API
 * (yodaplusplus/ssf_pbf_cuda, cuda_pbf_with_ssf/src/pbf/...):
 *
 *   reference                                              | this header
 *   -------------------------------------------------------+------------------------------
 *   pbf_parameter + pbf_external (pbf_type.h:49-72)        | pbf_params
 *   pbf_particle::allocate(num, domain_end)                | pbf_create
 *       (pbf_type.cpp:165-175), pbf_buffer::allocate       |
 *       (pbf_type.cpp:80-101)                              |
 *   pbf_particle::free / pbf_buffer::free                  | pbf_destroy
 *   pbf_boundary::allocate / free (pbf_boundary.cpp:4-33)  | pbf_boundary_create / _destroy
 *   pbf::one_step(particle, buf, [boundary,] area, iters)  | pbf_one_step
 *       (solver/pbf_solve.cpp:147-216)                     |
 *   cuda::addParticle (util/cuda/pbf_add.cu:12-28)         | pbf_add_particles
 *   phase.num / phase.x / phase.v (pbf_type.h:35-47)       | pbf_get_num / pbf_get_particles /
 *                                                          | pbf_set_particles
 *   one_step on a borrowed device x pointer                | pbf_one_step_external
 *       (simulator/dam/pbf_dam_sim.cpp:53-66)              |
 *   neighbor_search::getHash/getIndex/getCellStart/        | pbf_get_neighbor_debug
 *       getCellEnd/getNeighborList (pbf_neighbor_search.h:49-56)
 *   calcGridSize (pbf_type.cpp:141-162)                    | pbf_calc_grid_size
 *
 * Conventions that differ from the reference, on purpose:
 *   - every call returns a pbf_status; nothing calls exit();
 *   - all state is per handle (no __constant__ globals, no function statics),
 *     so handles are re-entrant across threads (one handle per thread);
 *   - positions/velocities cross the ABI as AoS float3 (the reference's
 *     dom_dim, 12 bytes), kept inside as float4 arrays;
 *   - the caller passes the CUDA stream (void* = cudaStream_t, NULL = legacy
 *     default stream);
 *   - the live particle count stays on the device during a step (no host sync);
 *     pbf_get_num synchronises the stream to read it.
 * Beside the plain step: a batched engine (pbf_batch_*) that advances many
 * scenes per launch, and a continuous-batching server (pbf_server_*).
 */
#ifndef PBF103_H
#define PBF103_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBF103_ABI_VERSION 1

typedef enum pbf_status {
    PBF_SUCCESS = 0,
    PBF_ERROR_INVALID_ARGUMENT = 1,
    PBF_ERROR_CUDA = 2,
    PBF_ERROR_OUT_OF_MEMORY = 3,
    PBF_ERROR_CAPACITY = 4,        /* more particles than the handle holds */
    PBF_ERROR_GRID_TOO_LARGE = 5,  /* reference: "grid_size is too large" + exit(-1) */
    PBF_ERROR_BAD_PARAMETER = 6,   /* reference: pbf_particle::allocate exit(-1) */
    PBF_ERROR_NOT_FOUND = 7,       /* unknown scene or request id */
    PBF_ERROR_BUDGET = 8,          /* HBM budget would be exceeded */
    PBF_ERROR_NO_DEVICE = 9,
    PBF_ERROR_NOT_READY = 10       /* result not available yet */
} pbf_status;

/* Device-side flags, accumulated per scene until read (pbf_get_flags). */
#define PBF_FLAG_NONFINITE 0x1u        /* a predicted position was NaN/Inf */
#define PBF_FLAG_COLLISION_LIMIT 0x2u  /* a particle hit max_collision_passes
                                          (the reference loops without bound,
                                          pbf_response_collision.cu:33) */
#define PBF_FLAG_CAPACITY 0x4u         /* a device-side append (pbf_generate,
                                          pbf_emit) did not fit the capacity
                                          and added nothing */

/* s_corr (tensile instability) forms */
#define PBF_TENSILE_REFERENCE 0  /* 10 W^4 / W(0.4h)^4 * (max(-l_i,0)+max(-l_j,0)),
                                    pbf_position_update.cu:132-151 */
#define PBF_TENSILE_TEXTBOOK 1   /* k (W / W(dq h))^n  (Macklin & Mueller 2013) */
#define PBF_TENSILE_OFF 2

/* vorticity confinement forms */
#define PBF_VORTICITY_OFF 0       /* as the reference's active step (pbf_solve.cpp:136-138) */
#define PBF_VORTICITY_REFERENCE 1 /* pbf_vorticity_confinement.cu formulas as written, uncapped
                                     27-cell walk around the final position */
#define PBF_VORTICITY_TEXTBOOK 2  /* omega = m/rho0 sum (v_j - v_i) x grad_j W,
                                     eta = m/rho0 sum |omega_j| grad_i W, v += dt eps (N x omega),
                                     over the step's neighbour list at the final positions */

/* XSPH forms */
#define PBF_XSPH_OFF 0            /* as the reference's active step */
#define PBF_XSPH_WALK 1           /* calcXSPHCUDA: uncapped 27-cell walk (pbf_xsph.cu:51-113) */
#define PBF_XSPH_LIST 2           /* same sum over the step's neighbour list */

typedef struct pbf_params {
    /* pbf_parameter, src/pbf/pbf_type.h:49-63 */
    float stable_density;   /* rho0, kg/m^3 */
    float stable_distance;  /* particle spacing, m */
    float particle_mass;    /* kg */
    float smoothing_length; /* h, m */
    float time_step;        /* s */
    float relaxation;       /* CFM epsilon, m^-2 */
    float xsph_parameter;   /* XSPH c (used when xsph_mode = 1) */
    float vc_parameter;     /* vorticity epsilon (used when vorticity_mode != 0) */
    /* pbf_external, src/pbf/pbf_type.h:69-72 */
    float body_force[3];    /* m/s^2 */
    /* neighbour list slots incl. the terminator; the reference fixes 30
       (pbf_neighbor_search.cpp:15), i.e. at most 29 listed neighbours */
    uint32_t max_pair_particle_num;
    int32_t tensile_mode;   /* PBF_TENSILE_* */
    float scorr_k;          /* textbook s_corr k */
    int32_t scorr_n;        /* textbook s_corr n */
    float scorr_dq;         /* textbook s_corr delta-q, in units of h */
    int32_t xsph_mode;      /* PBF_XSPH_* */
    int32_t vorticity_mode; /* PBF_VORTICITY_* */
    uint32_t max_collision_passes; /* bound on the collision projection loop */
    float cell_width;       /* 0 => smoothing_length (pbf_type.cpp:172) */
    uint32_t grid_size[3];  /* 0 => calcGridSize(2 * cell_width, domain_end) */
} pbf_params;

typedef struct pbf_handle pbf_handle;
typedef struct pbf_boundary_t pbf_boundary_t;
typedef struct pbf_batch pbf_batch;
typedef struct pbf_server pbf_server;

const char *pbf_status_string(pbf_status s);
/* Text of the last CUDA error seen by the calling thread ("" if none). */
const char *pbf_last_error(void);
int pbf_abi_version(void);

/* Defaults matching the reference's active step: reference s_corr, XSPH and
 * vorticity off, 30 neighbour slots, 64 collision passes, cell width h, grid
 * from calcGridSize.  Physical values are set to the dam-break config
 * (rho0 1000, spacing 0.05, h 0.1, m 0.125, dt 1/120, eps 600, g -9.8). */
pbf_status pbf_params_init(pbf_params *p);

/* calcGridSize, src/pbf/pbf_type.cpp:141-162 */
pbf_status pbf_calc_grid_size(double cell_size, const float domain_end[3], uint32_t grid_out[3]);

/* ---- boundary: pbf_boundary::allocate, src/pbf/pbf_boundary.cpp:4-25 ---- */
pbf_status pbf_boundary_create(const float *inner_spheres /* n x 4: cx,cy,cz,r */, uint32_t n_inner,
                               const float *outer_spheres /* n x 4 */, uint32_t n_outer,
                               const float *plane_points /* n x 3 */, const float *plane_normals /* n x 3 */,
                               uint32_t n_planes, pbf_boundary_t **out);
pbf_status pbf_boundary_destroy(pbf_boundary_t *b);

/* ---- single scene: pbf_particle + pbf_buffer + one_step ---- */
pbf_status pbf_create(const pbf_params *params, uint32_t capacity, const float domain_end[3], int device,
                      pbf_handle **out);
pbf_status pbf_destroy(pbf_handle *h);
pbf_status pbf_set_params(pbf_handle *h, const pbf_params *params); /* grid/cell width must not change */
pbf_status pbf_get_params(pbf_handle *h, pbf_params *params);
pbf_status pbf_get_grid(pbf_handle *h, uint32_t grid_out[3], float *cell_width);

/* x, v: n x 3 floats (AoS float3).  src_is_device: 1 if device pointers. */
pbf_status pbf_set_particles(pbf_handle *h, const float *x, const float *v, uint32_t n, int src_is_device,
                             void *stream);
pbf_status pbf_add_particles(pbf_handle *h, const float *x, const float *v, uint32_t n, int src_is_device,
                             void *stream);

/* pbf::one_step.  boundary == NULL selects the no-boundary overload (its
 * fixed inner sphere c=(3,3,3), r=3, pbf_constraint.cu:262-315).  Positions
 * and velocities are left in cell-sorted order; particles outside
 * [area_min, area_max] are deleted. */
pbf_status pbf_one_step(pbf_handle *h, const pbf_boundary_t *boundary, const float area_min[3],
                        const float area_max[3], int iters, void *stream);

/* one_step on a borrowed device pointer for x (AoS float3, valid only during
 * the call), as the simulators do with a GL-mapped buffer.  On return x_dev
 * holds the new sorted positions (num entries). */
pbf_status pbf_one_step_external(pbf_handle *h, float *x_dev, const pbf_boundary_t *boundary,
                                 const float area_min[3], const float area_max[3], int iters, void *stream);

pbf_status pbf_get_num(pbf_handle *h, uint32_t *num);
/* num x 3 floats each; either pointer may be NULL */
pbf_status pbf_get_particles(pbf_handle *h, float *x, float *v, int dst_is_device, void *stream);
pbf_status pbf_get_flags(pbf_handle *h, uint32_t *flags, int clear);
/* Use a CUDA graph for pbf_one_step (default on). */
pbf_status pbf_set_graph_mode(pbf_handle *h, int enable);

/* Integer intermediates of the last step, host buffers, reference layout:
 *   sorted_hash[n_in], perm[n_in]      (sorted -> input index; deleted particles last,
 *                                       with hash = number of cells)
 *   cell_start[C], cell_end[C]         (0xFFFFFFFF start for empty cells)
 *   neighbor_list[ceil32(num) * max_pair]  in the reference's warp-interleaved
 *                                       layout (pbf_neighbor_search_device_util.cu:15-21),
 *                                       0xFFFFFFFF in unused slots
 *   n_in = particles at the start of the last step.  Any pointer may be NULL. */
pbf_status pbf_get_neighbor_debug(pbf_handle *h, uint32_t *sorted_hash, uint32_t *perm, uint32_t *cell_start,
                                  uint32_t *cell_end, uint32_t *neighbor_list, uint32_t *n_in);

/* ---- neighbour-search sort without allocation ----
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they need the sort (code running under CUDA-graph stream
 * capture, plug-ins whose host owns all device allocations, real-time paths):
 * cell hash of x (n x 3 floats, device), stable counting sort by cell (a
 * cell's particles in ascending input index, at any bucket size), and cell
 * ranges, as pbf_one_step computes them for its predicted positions of a
 * scene whose simulation area holds every particle: there is no area check
 * here, so a particle outside the area is not deleted but hashed into the
 * wrapped table like any other.  perm_dev[n] receives sorted -> input index;
 * cell_start_dev / cell_end_dev [Gx*Gy*Gz] the ranges (0xFFFFFFFF for empty
 * cells).  Needs no handle and allocates nothing: its scratch is a fixed
 * device array (7.3 MB) that every GPU loading the library holds until exit.
 * Larger inputs return PBF_ERROR_CAPACITY.  The first call on a device looks
 * the array up and should come before any stream capture; the address is
 * kept for the life of the process, so after a cudaDeviceReset the process
 * must not call this entry point again.  Calls that overlap on the GPU share
 * the array and race, so the caller serialises them. */
#define PBF_NOALLOC_MAX_PARTICLES 262144u
#define PBF_NOALLOC_MAX_CELLS 524288u
pbf_status pbf_cell_sort_noalloc(const float *x_dev, uint32_t n, float cell_width, const uint32_t grid[3],
                                 uint32_t *perm_dev, uint32_t *cell_start_dev, uint32_t *cell_end_dev,
                                 void *stream);

/* ---- batched engine: many independent scenes, one launch per kernel per step ---- */
pbf_status pbf_batch_create(uint32_t max_scenes, uint64_t max_particles, uint64_t max_cells, uint32_t max_pair,
                            int device, pbf_batch **out);
pbf_status pbf_batch_destroy(pbf_batch *b);
/* Bytes of device memory one scene occupies (admission accounting). */
pbf_status pbf_scene_bytes(const pbf_params *params, uint32_t capacity, const float domain_end[3],
                           uint64_t *bytes);
pbf_status pbf_batch_add_scene(pbf_batch *b, const pbf_params *params, uint32_t capacity,
                               const float domain_end[3], const pbf_boundary_t *boundary,
                               const float area_min[3], const float area_max[3], const float *x,
                               const float *v, uint32_t n, int src_is_device, void *stream,
                               uint32_t *scene_id);
pbf_status pbf_batch_remove_scene(pbf_batch *b, uint32_t scene_id);
pbf_status pbf_batch_num_scenes(pbf_batch *b, uint32_t *n);
/* advance every scene by one step */
pbf_status pbf_batch_step(pbf_batch *b, int iters, void *stream);
pbf_status pbf_batch_get_scene(pbf_batch *b, uint32_t scene_id, float *x, float *v, uint32_t *num,
                               int dst_is_device, void *stream);
pbf_status pbf_batch_get_flags(pbf_batch *b, uint32_t scene_id, uint32_t *flags, int clear);
/* Active scene ids in ascending order (the order of the packed buffers below). */
pbf_status pbf_batch_scene_ids(pbf_batch *b, uint32_t *ids, uint32_t max, uint32_t *n);
/* Whole-batch upload / download of packed AoS float3 buffers: the active
 * scenes' particles back to back in scene-id order, counts[k] for the k-th
 * active scene (counts == NULL on upload keeps the current counts).  Host
 * buffers on upload must stay valid until the stream has consumed them
 * (as with cudaMemcpyAsync); get_all synchronises the stream. */
pbf_status pbf_batch_set_all(pbf_batch *b, const uint32_t *counts, const float *x, const float *v,
                             int src_is_device, void *stream);
pbf_status pbf_batch_get_all(pbf_batch *b, uint32_t *counts, float *x, float *v, int dst_is_device,
                             void *stream);
/* pbf_batch_set_all from device buffers followed by pbf_batch_step, in one
 * call without the unpack pass: the step's first passes read the packed
 * positions and velocities (scenes back to back in scene-id order, counts
 * as pbf_batch_set_all's) where they lie.  x_dev / v_dev (v_dev NULL: zero
 * velocities) must stay unchanged until the stream has run the step.  The
 * result is bit for bit that of pbf_batch_set_all + pbf_batch_step, and the
 * batch holds it as after pbf_batch_step.  No reference counterpart. */
pbf_status pbf_batch_step_packed(pbf_batch *b, int iters, const uint32_t *counts, const float *x_dev,
                                 const float *v_dev, void *stream);
/* pbf_batch_get_all into device buffers without a host round trip: the
 * packed offsets are computed on the device from the live counts, so the
 * call does not wait for the stream (after scenes were added or removed it
 * first uploads the scene tables, as pbf_batch_step does).  counts_dev[k] (device memory)
 * receives the k-th active scene's live count; read it once the stream has
 * reached this point.  x_dev / v_dev (either may be NULL) get the same packed
 * layout as pbf_batch_get_all and must hold the active scenes' capacities,
 * since the live counts are not known on the host when the call is made.
 * No reference counterpart. */
pbf_status pbf_batch_get_all_async(pbf_batch *b, uint32_t *counts_dev, float *x_dev, float *v_dev, void *stream);
/* Time candidate launch shapes on the current scenes and keep the fastest.
 * Leaves particle state unchanged. */
pbf_status pbf_batch_autotune(pbf_batch *b, int iters, void *stream, uint32_t *chosen_tile);
pbf_status pbf_batch_set_tile(pbf_batch *b, uint32_t tile);
/* Neighbour indices requested ahead per thread in the lambda / delta-p
 * passes (4 or 8; the autotuner also picks it).  Results do not depend on it.
 * No reference counterpart. */
pbf_status pbf_batch_set_chunk(pbf_batch *b, uint32_t chunk);
/* Current tile (particles per block) and chunk. */
pbf_status pbf_batch_get_launch_shape(pbf_batch *b, uint32_t *tile, uint32_t *chunk);
/* Cells per CTA of the per-cell stable rank of large steps (64, 128, 256 or
 * 512; the autotuner also picks it).  Results do not depend on it.  No
 * reference counterpart. */
pbf_status pbf_batch_set_cell_tile(pbf_batch *b, uint32_t cells);
pbf_status pbf_batch_get_cell_tile(pbf_batch *b, uint32_t *cells);
pbf_status pbf_batch_set_graph_mode(pbf_batch *b, int enable);
/* Kernels launched by the last pbf_batch_step / pbf_one_step call. */
pbf_status pbf_batch_last_launches(pbf_batch *b, uint32_t *launches);
pbf_status pbf_last_launches(pbf_handle *h, uint32_t *launches);
/* Advance one step without a CUDA graph, timing every kernel with CUDA
 * events on the stream: ms[k] and names[64 * k] (NUL-terminated) for the
 * k-th launch, at most max entries, *n written. */
pbf_status pbf_batch_profile_step(pbf_batch *b, int iters, void *stream, float *ms, char *names, uint32_t max,
                                  uint32_t *n);
pbf_status pbf_profile_step(pbf_handle *h, const pbf_boundary_t *boundary, const float area_min[3],
                            const float area_max[3], int iters, void *stream, float *ms, char *names, uint32_t max,
                            uint32_t *n);

/* ---- particle sets: ids, order restore, generators, emitters ----
 *
 * Every particle carries a 32-bit id that follows it through the per-step
 * sort.  pbf_set_particles numbers the particles 0..n-1; pbf_add_particles,
 * pbf_generate and pbf_emit continue from the scene's counter. */

/* Ids of the num particles in their current (sorted) order. */
pbf_status pbf_get_particle_ids(pbf_handle *h, uint32_t *ids, int dst_is_device, void *stream);
/* restoreOrder (src/pbf/interaction/cuda/pbf_neighbor_search_util.cu:156-170,
 * 344-359): x_out[perm[i]] = x[i] for the live particles, i.e. the order of
 * the last step's input.  n_out bounds the output (entries >= n_out and
 * those of deleted particles are left as they were).  Needs a step since
 * the last change of the particle set (else PBF_ERROR_NOT_READY). */
pbf_status pbf_restore_order(pbf_handle *h, float *x, float *v, uint32_t n_out, int dst_is_device, void *stream);
/* x_out[id] = x of the particle with that id, for ids < n_out (no reference
 * counterpart: the input order of the first step, across any number of steps). */
pbf_status pbf_get_particles_by_id(pbf_handle *h, float *x, float *v, uint32_t n_out, int dst_is_device,
                                   void *stream);

/* The reference's arrangement generators (src/pbf/util/pbf_arrangement.h),
 * evaluated on the device. */
#define PBF_ARRANGE_VOLUME 0     /* cartesian_volume(origin, end, space), :82-99 */
#define PBF_ARRANGE_RECTANGLE 1  /* cartesian_rectangle(axis, axis_value, origin2, end2, space), :123-163 */
#define PBF_ARRANGE_LINE 2       /* cartesian_line_inclusive(origin, end, space), :8-18 */
#define PBF_ARRANGE_CYLINDER 3   /* cartesian_cylinder(axis, axis_value, origin2, radius, height, space), :212-244 */
typedef struct pbf_arrangement {
    int32_t kind;        /* PBF_ARRANGE_* */
    int32_t axis;        /* rectangle / cylinder: 0 = "x", 1 = "y", 2 = "z" */
    float origin[3];     /* volume / line: 3-D; rectangle / cylinder: origin[0..1] is the 2-D origin */
    float end[3];        /* volume / line: 3-D; rectangle: end[0..1] is the 2-D end */
    float axis_value;    /* rectangle / cylinder */
    float radius;        /* cylinder */
    float height;        /* cylinder */
    float space;         /* particle spacing */
} pbf_arrangement;

/* Points an arrangement generates (host arithmetic, as the reference's loops). */
pbf_status pbf_arrangement_count(const pbf_arrangement *a, uint32_t *n);
/* Append the arrangement's points with velocity v0 on the device, after the
 * live particles, without a host round trip; if they do not fit the
 * capacity nothing is added and PBF_FLAG_CAPACITY is raised.  *n_points
 * (optional) receives the arrangement's point count. */
pbf_status pbf_generate(pbf_handle *h, const pbf_arrangement *a, const float v0[3], void *stream,
                        uint32_t *n_points);

/* Emitter: a fixed set of positions and velocities resident on a device
 * (the sphere scene's jet, src/simulator/sphere/pbf_sphere_sim.cpp:20-82). */
typedef struct pbf_emitter pbf_emitter;
pbf_status pbf_emitter_create(int device, const float *x, const float *v, uint32_t n, int src_is_device,
                              pbf_emitter **out);
pbf_status pbf_emitter_create_arrangement(int device, const pbf_arrangement *a, const float v0[3],
                                          pbf_emitter **out);
pbf_status pbf_emitter_size(const pbf_emitter *e, uint32_t *n);
pbf_status pbf_emitter_destroy(pbf_emitter *e);
/* Append the emitter's particles iff num < max_fill * capacity (the jet's
 * rule, pbf_sphere_sim.cpp:386-387) and they fit; decided on the device. */
pbf_status pbf_emit(pbf_handle *h, const pbf_emitter *e, double max_fill, void *stream);

/* The same for one scene of a batch. */
pbf_status pbf_batch_get_particle_ids(pbf_batch *b, uint32_t scene_id, uint32_t *ids, uint32_t *num,
                                      int dst_is_device, void *stream);
pbf_status pbf_batch_restore_order(pbf_batch *b, uint32_t scene_id, float *x, float *v, uint32_t n_out,
                                   int dst_is_device, void *stream);
pbf_status pbf_batch_get_particles_by_id(pbf_batch *b, uint32_t scene_id, float *x, float *v, uint32_t n_out,
                                         int dst_is_device, void *stream);
pbf_status pbf_batch_generate(pbf_batch *b, uint32_t scene_id, const pbf_arrangement *a, const float v0[3],
                              void *stream, uint32_t *n_points);
pbf_status pbf_batch_emit(pbf_batch *b, uint32_t scene_id, const pbf_emitter *e, double max_fill, void *stream);

/* ---- headless screen-space fluid rendering ----
 * The reference's per-frame GL passes (src/main.cpp:372-564) as CUDA kernels
 * writing device image buffers; no graphics API is involved.
 *   depth splat: ssf_object.vert/.geom/.frag (the quad main.cpp draws,
 *                main.cpp:372-393) or ssf_point_sprite.vert/.frag;
 *   blur:        ssf_blur.frag, blur_passes times, ping-pong (main.cpp:430-509);
 *   normals:     ssf_normal.frag on the last blurred depth (main.cpp:511-531);
 *   shading:     ssf_shading.frag over the unblurred depth, blended
 *                (SRC_ALPHA, ONE_MINUS_SRC_ALPHA) onto the clear colour
 *                (main.cpp:541-564).
 * Images are row-major with row 0 at the bottom (GL window coordinates). */
#define PBF_SSF_SPLAT_QUAD 0    /* ssf_object: view-space quad of side point_radius */
#define PBF_SSF_SPLAT_SPRITE 1  /* ssf_point_sprite: point of point_radius * point_scale / dist pixels */

#define PBF_SSF_DEPTH 0         /* float [h][w], window depth in [0, 1], 1 = empty */
#define PBF_SSF_BLURRED 1       /* float [h][w], the last blur pass's output */
#define PBF_SSF_BLUR_INPUT 2    /* float [h][w], the last blur pass's input */
#define PBF_SSF_NORMAL 3        /* float [h][w][4], eye-space normal, w = 1; empty pixels = clear colour */
#define PBF_SSF_COLOR 4         /* float [h][w][4], shaded colour blended onto the clear colour */
#define PBF_SSF_RGBA8 5         /* uint8 [h][w][4], PBF_SSF_COLOR quantised as an 8-bit framebuffer */

typedef struct pbf_ssf_params {
    uint32_t width, height;     /* 1280 x 720 (main.cpp:32) */
    float projection[16];       /* column-major, the Scene block's Projection */
    float view[16];             /* column-major, the Scene block's View (World = identity) */
    float point_radius;         /* 0.18 (main.cpp:388) */
    float point_scale;          /* sprite mode only: pixels per unit of point_radius / dist */
    float near_plane, far_plane;/* 0.1, 50 (src/common/controls.cpp:25-26) */
    float blur_radius;          /* 5.5e-6 (main.cpp:189) */
    float blur_scale;           /* height / tanf(45 * 0.5 * 3.1415 / 180) (main.cpp:445) */
    uint32_t blur_passes;       /* 3 (main.cpp:430-509) */
    uint32_t splat_mode;        /* PBF_SSF_SPLAT_* */
    float thickness;            /* thickness map value (see pbf_ssf_params_init) */
    float clear_color[4];       /* 0.6, 0.6, 0.6, 1 (main.cpp:76) */
} pbf_ssf_params;

typedef struct pbf_ssf_renderer pbf_ssf_renderer;

/* Defaults of the reference's first frame: controls.cpp's initial camera
 * (position (2, 4, 10), angles pi and -0.1 pi, glm::perspective(45.0f,
 * 4/3, 0.1, 50) with 45 taken as radians by GLM 0.9.7, glm::lookAt), all in
 * float on the host.  The reference's thickness pass loads a fragment
 * shader absent from its assets, so its thickness map is undefined; the
 * default here is 0.6, the value its clear leaves in the map.  point_scale
 * defaults to the projection's pixels per unit at unit distance. */
pbf_status pbf_ssf_params_init(pbf_ssf_params *p);
/* The projection must keep x on (x, z), y on (y, z), and clip z, w on (z, w)
 * (any glm::perspective / frustum / ortho), else PBF_ERROR_BAD_PARAMETER.
 * width and height: 1 .. 8192. */
pbf_status pbf_ssf_create(int device, const pbf_ssf_params *p, pbf_ssf_renderer **out);
pbf_status pbf_ssf_destroy(pbf_ssf_renderer *r);
/* One frame from n positions (device, AoS float3, as the reference's VBO). */
pbf_status pbf_ssf_render(pbf_ssf_renderer *r, const float *x_dev, uint32_t n, void *stream);
/* One frame from a handle's / a batch scene's resident particles; the live
 * count is read on the device (no host synchronisation). */
pbf_status pbf_ssf_render_particles(pbf_ssf_renderer *r, pbf_handle *h, void *stream);
pbf_status pbf_ssf_render_scene(pbf_ssf_renderer *r, pbf_batch *b, uint32_t scene_id, void *stream);
/* Copy one image (PBF_SSF_*) out; blocks on the stream when dst is host. */
pbf_status pbf_ssf_get_image(pbf_ssf_renderer *r, int which, void *dst, int dst_is_device, void *stream);
/* Device address and size in bytes of one image buffer (valid until destroy). */
pbf_status pbf_ssf_image_device(pbf_ssf_renderer *r, int which, void **ptr, uint64_t *bytes);
/* The inverse projection and the normalised light direction the passes use. */
pbf_status pbf_ssf_frame_constants(const pbf_ssf_renderer *r, float inv_projection[16], float incident[3]);
/* Kernels launched by the last frame. */
pbf_status pbf_ssf_last_launches(const pbf_ssf_renderer *r, uint32_t *n);

/* ---- continuous-batching server ---- */
typedef struct pbf_server_config {
    uint64_t hbm_budget_bytes;  /* admission budget for resident scenes */
    uint32_t max_scenes;        /* resident scene slots */
    uint64_t max_particles;     /* arena size, particles */
    uint64_t max_cells;         /* arena size, hash cells */
    uint32_t max_pair;          /* neighbour slots of the arena (30) */
    int32_t iters;              /* solver iterations per step (4) */
    int32_t device;
    uint32_t tile;              /* 0 = autotune on the first full batch */
} pbf_server_config;

typedef struct pbf_request_desc {
    pbf_params params;
    float domain_end[3];
    float area_min[3];
    float area_max[3];
    uint32_t n_planes;          /* up to 8 boundary planes (points/normals below) */
    float plane_points[8][3];
    float plane_normals[8][3];
    uint32_t capacity;          /* 0 => n */
    uint32_t horizon_steps;     /* steps to run before completion */
} pbf_request_desc;

typedef struct pbf_completion {
    uint64_t request_id;
    uint32_t num;               /* particles at completion */
    uint32_t steps;
    uint32_t flags;
    double arrival_s;           /* server clock, seconds */
    double admit_s;
    double complete_s;
} pbf_completion;

typedef struct pbf_server_stats {
    uint64_t submitted, admitted, completed, rejected;
    uint64_t substeps;
    uint64_t particle_steps;
    uint64_t resident_bytes, peak_resident_bytes;
    uint32_t resident_scenes, queued;
    double busy_s;              /* time spent inside batch steps */
    double elapsed_s;
} pbf_server_stats;

pbf_status pbf_server_create(const pbf_server_config *cfg, pbf_server **out);
pbf_status pbf_server_destroy(pbf_server *s);
/* x, v: host AoS float3, n particles; copied at submit time. */
pbf_status pbf_server_submit(pbf_server *s, const pbf_request_desc *req, const float *x, const float *v,
                             uint32_t n, uint64_t *request_id);
/* Start / stop the serving loop thread. */
pbf_status pbf_server_start(pbf_server *s);
pbf_status pbf_server_stop(pbf_server *s, int drain);
/* Run the loop on the calling thread until every submitted request is done. */
pbf_status pbf_server_run_until_idle(pbf_server *s);
pbf_status pbf_server_poll(pbf_server *s, pbf_completion *out, uint32_t max, uint32_t *n_out);
/* Result of a completed request (num x 3 floats each, host buffers). */
pbf_status pbf_server_result(pbf_server *s, uint64_t request_id, float *x, float *v, uint32_t *num);
pbf_status pbf_server_release(pbf_server *s, uint64_t request_id);
pbf_status pbf_server_get_stats(pbf_server *s, pbf_server_stats *st);
double pbf_server_clock(pbf_server *s);

#ifdef __cplusplus
}
#endif
#endif /* PBF103_H */
