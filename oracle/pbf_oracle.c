/*
 * CPU oracle for the PBF solver step — TEST INFRASTRUCTURE ONLY (the checker,
 * never the product).  See pbf_oracle.h.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared (oracle/build_oracle.py).
 * -ffp-contract=off keeps every a*b+c unfused so the explicit fmaf() calls
 * are the only fused operations, as written in the reference kernels.
 */
#include "pbf_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int ora_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* floor + float->int32 conversion with the GPU's cvt.rmi.s32.f32 semantics
 * (saturating, NaN -> 0); the reference writes static_cast<int>(floor(p / w))
 * (src/pbf/interaction/cuda/pbf_grid.h:20-33). */
static inline int32_t floor_to_int(float v)
{
    if (v != v) return 0;
    const float f = floorf(v);
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f < -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}

/* calcGridHash with power-of-two wrap, src/pbf/interaction/cuda/pbf_grid.h:53-61.
 * Coordinates arrive as uint32 so that grid + offset wraps like the GPU's
 * two's-complement add. */
static inline uint32_t grid_hash(uint32_t gx, uint32_t gy, uint32_t gz, const uint32_t G[3])
{
    const uint32_t x = gx & (G[0] - 1u), y = gy & (G[1] - 1u), z = gz & (G[2] - 1u);
    return z * G[0] * G[1] + y * G[0] + x;
}

float ora_wpoly6(float r, float inv_h)
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

float ora_wspiky_deriv(float r, float inv_h)
{
    const float q = r * inv_h;
    const float inv_h2 = inv_h * inv_h;
    if (q <= 1.f) {
        const float t = 1.f - q;
        const float inv_h4 = inv_h2 * inv_h2;
        return -14.3239448745f * inv_h4 * t * t;
    }
    return 0.f;
}

/* src/pbf/pbf_type.cpp:141-162 (the reference calls it with 2h, pbf_type.cpp:173) */
int ora_calc_grid_size(double cell_size, const float sim_end[3], uint32_t g[3])
{
    uint32_t x = 1, y = 1, z = 1;
    for (;;) {
        const int bx = x * cell_size > (double)sim_end[0];
        const int by = y * cell_size > (double)sim_end[1];
        const int bz = z * cell_size > (double)sim_end[2];
        if (bx && by && bz) break;
        x = bx ? x : x * 2;
        y = by ? y : y * 2;
        z = bz ? z : z * 2;
        if (x > 1028 || y > 1028 || z > 1028) return -1;
    }
    g[0] = x; g[1] = y; g[2] = z;
    return 0;
}

/* calcHashCUDA (src/pbf/interaction/cuda/pbf_neighbor_search_util.cu:20-37),
 * checkDeleteParticleCUDA (src/pbf/util/cuda/pbf_delete.cu:9-28) and a
 * stable counting sort (the ordering cub::DeviceRadixSort::SortPairs gives,
 * pbf_neighbor_search_util.cu:186-198; the reference's default counting sort,
 * src/pbf/util/cuda/pbf_counting_sort.cu:21-178, produces the same
 * histogram and offsets with a non-deterministic order inside a cell).
 * Out-of-area particles get the key C (one past the last cell). */
void ora_hash_sort(uint32_t n, const float *xs, float cw, const uint32_t grid[3],
                   const float amin[3], const float amax[3], int check_area,
                   uint32_t *keys, uint32_t *perm, uint32_t *offsets)
{
    const uint32_t C = grid[0] * grid[1] * grid[2];
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const float *p = xs + 3 * i;
        const int32_t gx = floor_to_int(p[0] / cw);
        const int32_t gy = floor_to_int(p[1] / cw);
        const int32_t gz = floor_to_int(p[2] / cw);
        uint32_t key = grid_hash((uint32_t)gx, (uint32_t)gy, (uint32_t)gz, grid);
        if (check_area && (p[0] < amin[0] || amax[0] < p[0] || p[1] < amin[1] || amax[1] < p[1] ||
                           p[2] < amin[2] || amax[2] < p[2]))
            key = C;
        keys[i] = key;
    }
    memset(offsets, 0, sizeof(uint32_t) * ((size_t)C + 2));
    for (uint32_t i = 0; i < n; ++i) offsets[keys[i] + 1]++;
    for (uint32_t c = 0; c <= C; ++c) offsets[c + 1] += offsets[c];
    uint32_t *cursor = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)C + 1));
    memcpy(cursor, offsets, sizeof(uint32_t) * ((size_t)C + 1));
    for (uint32_t i = 0; i < n; ++i) perm[cursor[keys[i]]++] = i;
    free(cursor);
}

/* detectNeighborsCUDA<uint32_t> with findPair / searchCell / searchGrid,
 * src/pbf/interaction/cuda/pbf_neighbor_search_util.cu:386-482:
 * 27 cells in z, y, x order (-1..1), candidates in ascending sorted index,
 * accepted if r2 < h2 while fewer than cap (= max_pair - 1) are listed. */
static void build_neighbors(uint32_t n, const float *x0, const uint32_t *offsets, float cw,
                            const uint32_t grid[3], float h, uint32_t cap, uint32_t *nbr,
                            uint8_t *nnb)
{
    const float h2 = h * h;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)n; ++p) {
        const float *s = x0 + 3 * p;
        const int32_t gx = floor_to_int(s[0] / cw);
        const int32_t gy = floor_to_int(s[1] / cw);
        const int32_t gz = floor_to_int(s[2] / cw);
        uint32_t cnt = 0;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const uint32_t hc = grid_hash((uint32_t)gx + (uint32_t)dx, (uint32_t)gy + (uint32_t)dy,
                                                  (uint32_t)gz + (uint32_t)dz, grid);
                    for (uint32_t q = offsets[hc]; q < offsets[hc + 1]; ++q) {
                        if (cnt < cap) {
                            const float *o = x0 + 3 * (size_t)q;
                            const float d0 = s[0] - o[0], d1 = s[1] - o[1], d2 = s[2] - o[2];
                            const float r2 = fmaf(d2, d2, fmaf(d1, d1, d0 * d0));
                            if (r2 < h2) nbr[(size_t)p * cap + cnt++] = q;
                        }
                    }
                }
        for (uint32_t k = cnt; k < cap; ++k) nbr[(size_t)p * cap + k] = 0xFFFFFFFFu;
        nnb[p] = (uint8_t)cnt;
    }
}

/* ---- solver, instantiated in FP32 and FP64 ---- */
#define R float
#define FMA fmaf
#define SQRT sqrtf
#define FABS fabsf
#define LIT(x) ((float)(x))
#define CAT(name) name##_f32
#include "pbf_oracle_solve.inc"
#undef R
#undef FMA
#undef SQRT
#undef FABS
#undef LIT
#undef CAT

#define R double
#define FMA fma
#define SQRT sqrt
#define FABS fabs
#define LIT(x) ((double)(x))
#define CAT(name) name##_f64
#include "pbf_oracle_solve.inc"
#undef R
#undef FMA
#undef SQRT
#undef FABS
#undef LIT
#undef CAT

/* pbf::one_step (boundary overload), src/pbf/solver/pbf_solve.cpp:182-216:
 * predict (pbf_solve.cpp:16-25, kernels src/pbf/solver/cuda/pbf_predict.cu:15-45),
 * neighbour search (src/pbf/interaction/pbf_neighbor_search.cpp:92-170),
 * solveConstraint (pbf_solve.cpp:79-106) and update (pbf_solve.cpp:125-145). */
int ora_step(const ora_params *P, const ora_boundary *B, const float area_min[3],
             const float area_max[3], int iters, int use_f64, uint32_t n, const float *x_in,
             const float *v_in, float *x_out, float *v_out, uint32_t *num_out,
             uint32_t *keys_out, uint32_t *perm_out, uint32_t *offsets_out, uint32_t *nbr_out,
             uint8_t *nnb_out, float *lambda0_out)
{
    const uint32_t C = P->grid[0] * P->grid[1] * P->grid[2];
    const uint32_t cap = P->max_pair - 1;
    const size_t nn = n ? n : 1;
    float *xs = (float *)malloc(sizeof(float) * 3 * nn);
    uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * nn);
    uint32_t *perm = (uint32_t *)malloc(sizeof(uint32_t) * nn);
    uint32_t *offsets = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)C + 2));
    float *x0 = (float *)malloc(sizeof(float) * 3 * nn);
    float *xold = (float *)malloc(sizeof(float) * 3 * nn);
    uint32_t *nbr = (uint32_t *)malloc(sizeof(uint32_t) * nn * cap);
    uint8_t *nnb = (uint8_t *)malloc(nn);

    /* predict: v* = fma(g, dt, v); x* = fma(v*, dt, x) */
    const float dt = P->time_step;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i)
        for (int c = 0; c < 3; ++c) {
            const float vs = fmaf(P->body_force[c], dt, v_in[3 * i + c]);
            xs[3 * i + c] = fmaf(vs, dt, x_in[3 * i + c]);
        }

    ora_hash_sort(n, xs, P->cell_width, P->grid, area_min, area_max, 1, keys, perm, offsets);
    const uint32_t live = offsets[C];

    /* reorderDataCUDA x2, src/pbf/interaction/cuda/pbf_neighbor_search_util.cu:143-154 */
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)live; ++p)
        for (int c = 0; c < 3; ++c) {
            x0[3 * p + c] = xs[3 * (size_t)perm[p] + c];
            xold[3 * p + c] = x_in[3 * (size_t)perm[p] + c];
        }

    build_neighbors(live, x0, offsets, P->cell_width, P->grid, P->smoothing_length, cap, nbr, nnb);

    int rc;
    if (use_f64)
        rc = solve_f64(P, B, iters, live, x0, xold, offsets, nbr, nnb, cap, x_out, v_out, lambda0_out);
    else
        rc = solve_f32(P, B, iters, live, x0, xold, offsets, nbr, nnb, cap, x_out, v_out, lambda0_out);

    if (num_out) *num_out = live;
    if (keys_out) memcpy(keys_out, keys, sizeof(uint32_t) * n);
    if (perm_out) memcpy(perm_out, perm, sizeof(uint32_t) * n);
    if (offsets_out) memcpy(offsets_out, offsets, sizeof(uint32_t) * ((size_t)C + 2));
    if (nbr_out) memcpy(nbr_out, nbr, sizeof(uint32_t) * (size_t)live * cap);
    if (nnb_out) memcpy(nnb_out, nnb, live);

    free(xs); free(keys); free(perm); free(offsets); free(x0); free(xold); free(nbr); free(nnb);
    return rc;
}
