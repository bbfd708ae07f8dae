/*
 * CPU oracle for the PBF solver step — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference simulator's step
 * (yodaplusplus/ssf_pbf_cuda, `pbf::one_step`, src/pbf/solver/pbf_solve.cpp:182-216)
 * used as the checker for the CUDA path.  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / reference arm may load it.  The product path
 * never links or calls it.
 *
 * Two arithmetic modes share one integer pipeline:
 *   - f32: follows the reference kernels' FP32 operation order and explicit
 *          fmaf chains (rsqrtf is replaced by the correctly rounded 1/sqrtf);
 *   - f64: the same algorithm with every solver quantity in double; the
 *          neighbour list is still decided in FP32 exactly as the reference
 *          decides it, so both modes see the same neighbour sets.
 */
#ifndef PBF_ORACLE_H
#define PBF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_params {
    float rest_density;      /* rho0 */
    float particle_mass;     /* m */
    float smoothing_length;  /* h */
    float time_step;         /* dt */
    float relaxation;        /* CFM epsilon, m^-2 */
    float xsph_c;            /* XSPH coefficient */
    float vorticity_eps;     /* vorticity confinement coefficient */
    float body_force[3];     /* gravity */
    float cell_width;        /* hash cell width (reference: h) */
    uint32_t grid[3];        /* power-of-two hash grid dims */
    uint32_t max_pair;       /* neighbour slots incl. terminator (reference: 30 -> 29 usable) */
    int32_t tensile_mode;    /* 0 reference, 1 textbook, 2 off */
    float scorr_k;           /* textbook s_corr k */
    int32_t scorr_n;         /* textbook s_corr n */
    float scorr_dq;          /* textbook s_corr delta-q in units of h */
    int32_t xsph_mode;       /* 0 off, 1 on */
    int32_t vorticity_mode;  /* 0 off, 1 reference formulas, 2 textbook */
    uint32_t max_collision_passes;
} ora_params;

typedef struct ora_boundary {
    uint32_t n_inner, n_outer, n_planes;
    const float *inner;      /* n_inner x (cx, cy, cz, r) */
    const float *outer;      /* n_outer x (cx, cy, cz, r) */
    const float *plane_pts;  /* n_planes x 3 */
    const float *plane_nrm;  /* n_planes x 3 */
    int32_t use_builtin_sphere; /* 1: the no-boundary overload's fixed sphere c=(3,3,3), r=3 */
} ora_boundary;

/* Cell-hash + stable counting sort of predicted positions (reference
 * calcHashCUDA + checkDeleteParticle + countingSort with a stable rank).
 * keys[n] (unsorted, deleted = C), perm[n] (sorted -> input index),
 * offsets[C + 2] (exclusive scan of the per-cell counts, offsets[C] = live). */
void ora_hash_sort(uint32_t n, const float *xs, float cell_width, const uint32_t grid[3],
                   const float area_min[3], const float area_max[3], int check_area,
                   uint32_t *keys, uint32_t *perm, uint32_t *offsets);

/* One full solver step.  x_in/v_in: n x 3 (AoS float3, any order).
 * Outputs are in sorted order (as the reference leaves them).
 * Optional outputs may be NULL.  Returns the largest number of collision
 * passes any particle needed (or -1 if one hit max_collision_passes). */
int ora_step(const ora_params *P, const ora_boundary *B,
             const float area_min[3], const float area_max[3], int iters, int use_f64,
             uint32_t n, const float *x_in, const float *v_in,
             float *x_out, float *v_out, uint32_t *num_out,
             uint32_t *keys_out, uint32_t *perm_out, uint32_t *offsets_out,
             uint32_t *nbr_out, uint8_t *nnb_out, float *lambda0_out);

/* Poly6 / spiky-derivative values as the reference's __host__ __device__
 * helpers compute them (src/pbf/kernel/cuda/detail/pbf_kernel.inl:34-63). */
float ora_wpoly6(float r, float inv_h);
float ora_wspiky_deriv(float r, float inv_h);

/* Reference grid sizing rule (src/pbf/pbf_type.cpp:141-162). Returns 0 on
 * success, -1 when an axis would exceed 1028. */
int ora_calc_grid_size(double cell_size, const float sim_end[3], uint32_t grid[3]);

int ora_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
