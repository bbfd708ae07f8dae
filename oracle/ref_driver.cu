// Driver for the reference's own PBF step — TEST INFRASTRUCTURE ONLY.
//
// Built by oracle/ref_build.py against the reference sources (never
// committed); runs pbf::one_step (src/pbf/solver/pbf_solve.cpp:147-216) once on
// an input file and dumps its outputs, so that the CPU oracle can be pinned
// to the reference's results.  Private members of neighbor_search are read
// for the sorted hash/index arrays (src/pbf/interaction/pbf_neighbor_search.h:69-89).
//
// post selects the velocity update after the solver iterations:
//   0  one_step as shipped: the vorticity overload of update, whose XSPH and
//      vorticity calls are commented out (pbf_solve.cpp:125-145);
//   1  the XSPH overload of update (pbf_solve.cpp:108-123): updateVelocity,
//      applyXSPH (src/pbf/solver/cuda/pbf_xsph.cu:120-152), updatePosition;
//   2  the vorticity overload with its commented calls active, in their
//      order (pbf_solve.cpp:134-141): updateVelocity, calcVorticity,
//      addVorticityConfinement (pbf_vorticity_confinement.cu:229-296),
//      applyXSPH, updatePosition;
//   3  the same without applyXSPH (velocity copied as pbf_solve.cpp:142).
// For post != 0 the driver runs one_step's body itself (predict,
// detectNeighbors, solveConstraint as pbf_solve.cpp:154-176 / 186-211).
//
// Input (little endian): "PBFI", u32 version, u32 n, u32 capacity, i32 iters,
//   i32 use_boundary, [version >= 2: i32 post], f32 params[8] (pbf_parameter
//   order), f32 body_force[3],
//   f32 domain_end[3], f32 area_min[3], f32 area_max[3], u32 n_inner, n_outer,
//   n_planes, f32 inner[4 n_inner], outer[4 n_outer], pts[3 n_planes],
//   nrm[3 n_planes], f32 x[3n], v[3n].
// Output: "PBFO", u32 num, u32 n_in, u32 grid[3], u32 max_pair, f32 x[3 num],
//   v[3 num], u32 sorted_hash[n_in], sorted_index[n_in], cell_start[C],
//   cell_end[C], neighbor_list[ceil32(num) * max_pair].
// With a third argument R > 0 the step is first timed: R steps, each from
// the input state (device-to-device reload inside the timed region), after
// one warm-up step; "ms_per_step <t>" is printed to stdout.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define private public
#include "pbf/pbf.h"
#include "pbf/interaction/pbf_neighbor_search.h"
#include "pbf/solver/cuda/pbf_update.h"
#undef private

namespace pbf {
// the boundary overload of the cached solveConstraint: defined in
// src/pbf/solver/pbf_solve.cpp:79-106, not declared in its header
void solveConstraint(dom_dim *interim_position, dom_dim *position_update, scalar_t *scaling_factor,
                     scalar_t *kernels, dom_dim *grad_kernels, const dom_dim *old_position,
                     const pbf_boundary &boundary, std::shared_ptr<neighbor_search> &ns,
                     scalar_t inv_stable_density, scalar_t particle_mass, scalar_t smoothing_length,
                     scalar_t relaxation, int num_iteration, int num_particle);
}  // namespace pbf

template <class T>
static void rd(FILE *f, T *p, size_t n)
{
    if (n && fread(p, sizeof(T), n, f) != n) {
        fprintf(stderr, "short read\n");
        exit(2);
    }
}
template <class T>
static void wr(FILE *f, const T *p, size_t n)
{
    if (n) fwrite(p, sizeof(T), n, f);
}

static void check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
        exit(3);
    }
}

int main(int argc, char **argv)
{
    if (argc != 3 && argc != 4) {
        fprintf(stderr, "usage: %s input.bin output.bin [timed_steps]\n", argv[0]);
        return 1;
    }
    const int reps = argc == 4 ? atoi(argv[3]) : 0;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 1;
    char magic[4];
    rd(f, magic, 4);
    if (memcmp(magic, "PBFI", 4)) return 1;
    uint32_t ver, n, cap;
    int32_t iters, use_b, post = 0;
    rd(f, &ver, 1);
    rd(f, &n, 1);
    rd(f, &cap, 1);
    rd(f, &iters, 1);
    rd(f, &use_b, 1);
    if (ver >= 2) rd(f, &post, 1);
    if (post < 0 || post > 3) {
        fprintf(stderr, "post mode %d\n", post);
        return 1;
    }
    float prm[8], g[3], dend[3], amin[3], amax[3];
    rd(f, prm, 8);
    rd(f, g, 3);
    rd(f, dend, 3);
    rd(f, amin, 3);
    rd(f, amax, 3);
    uint32_t ni, no, np;
    rd(f, &ni, 1);
    rd(f, &no, 1);
    rd(f, &np, 1);
    std::vector<float> inner(4 * ni), outer(4 * no), pts(3 * np), nrm(3 * np), x(3 * n), v(3 * n);
    rd(f, inner.data(), inner.size());
    rd(f, outer.data(), outer.size());
    rd(f, pts.data(), pts.size());
    rd(f, nrm.data(), nrm.size());
    rd(f, x.data(), x.size());
    rd(f, v.data(), v.size());
    fclose(f);

    pbf_particle part;
    part.parameter.stable_density = prm[0];
    part.parameter.stable_distance = prm[1];
    part.parameter.particle_mass = prm[2];
    part.parameter.smoothing_length = prm[3];
    part.parameter.time_step = prm[4];
    part.parameter.relaxation = prm[5];
    part.parameter.xsph_parameter = prm[6];
    part.parameter.vc_parameter = prm[7];
    part.external.body_force = dom_dim(g[0], g[1], g[2]);
    part.allocate(cap, dom_dim(dend[0], dend[1], dend[2]));
    part.phase.num = n;
    check(cudaMemcpy(part.phase.x, x.data(), 12ull * n, cudaMemcpyHostToDevice), "copy x");
    check(cudaMemcpy(part.phase.v, v.data(), 12ull * n, cudaMemcpyHostToDevice), "copy v");
    pbf_buffer buf;
    buf.allocate(cap, part.ns->getMaxPairParticleNum());
    const std::pair<dom_dim, dom_dim> area(dom_dim(amin[0], amin[1], amin[2]), dom_dim(amax[0], amax[1], amax[2]));
    std::vector<glm::vec4> in, out;
    std::vector<dom_dim> pp, pn;
    for (uint32_t k = 0; k < ni; ++k) in.emplace_back(inner[4 * k], inner[4 * k + 1], inner[4 * k + 2], inner[4 * k + 3]);
    for (uint32_t k = 0; k < no; ++k) out.emplace_back(outer[4 * k], outer[4 * k + 1], outer[4 * k + 2], outer[4 * k + 3]);
    for (uint32_t k = 0; k < np; ++k) {
        pp.emplace_back(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]);
        pn.emplace_back(nrm[3 * k], nrm[3 * k + 1], nrm[3 * k + 2]);
    }
    pbf_boundary bnd;
    if (use_b) bnd.allocate(in, out, pp, pn);
    // one_step's body with the post-solve update chosen by `post`
    auto step_post = [&]() {
        cudaDeviceSetCacheConfig(cudaFuncCachePreferL1);
        auto &phase = part.phase;
        auto &param = part.parameter;
        auto ns = part.ns;
        uint32_t &num = part.phase.num;
        const auto inv_rho0 = 1.f / param.stable_density;
        const auto m = param.particle_mass;
        const auto h = param.smoothing_length;
        const auto inv_t = 1.f / param.time_step;
        pbf::predict(buf.interim.x, buf.interim.v, phase.x, phase.v, part.external.body_force, param.time_step,
                     num);
        ns->detectNeighbors(buf.sorted_predicted_pos, buf.interim.x, buf.sorted_old_pos, phase.x, h, area, num);
        if (use_b)
            pbf::solveConstraint(buf.sorted_predicted_pos, buf.delta_position, buf.scaling_factor, buf.kernels,
                                 buf.grad_kernels, buf.sorted_old_pos, bnd, ns, inv_rho0, m, h, param.relaxation,
                                 iters, num);
        else
            pbf::solveConstraint(buf.sorted_predicted_pos, buf.delta_position, buf.scaling_factor, buf.kernels,
                                 buf.grad_kernels, buf.sorted_old_pos, ns, inv_rho0, m, h, param.relaxation, iters,
                                 num);
        if (post == 1) {
            pbf::update(phase.x, phase.v, buf.interim.v, buf.sorted_predicted_pos, buf.sorted_old_pos, ns, inv_t,
                        inv_rho0, m, h, param.xsph_parameter, num);
            return;
        }
        pbf::cuda::updateVelocity(buf.interim.v, buf.sorted_predicted_pos, buf.sorted_old_pos, inv_t, num);
        pbf::cuda::calcVorticity(buf.vorticity, buf.sorted_predicted_pos, buf.interim.v, *ns, h, m, inv_rho0, num);
        pbf::cuda::addVorticityConfinement(buf.interim.v, buf.vorticity, buf.sorted_predicted_pos, *ns, h, m,
                                           inv_rho0, param.vc_parameter, 1.f / inv_t, num);
        if (post == 2)
            pbf::cuda::applyXSPH(phase.v, buf.sorted_predicted_pos, buf.interim.v, ns, h, param.xsph_parameter,
                                 inv_rho0, m, num);
        else
            pbf::cuda::updateVelocity(phase.v, buf.interim.v, num);
        pbf::cuda::updatePosition(phase.x, buf.sorted_predicted_pos, num);
    };
    auto step = [&]() {
        if (post) step_post();
        else if (use_b) pbf::one_step(part, buf, bnd, area, iters);
        else pbf::one_step(part, buf, area, iters);
    };
    if (reps > 0) {
        float *x0 = nullptr, *v0 = nullptr;
        check(cudaMalloc(&x0, 12ull * n), "x0");
        check(cudaMalloc(&v0, 12ull * n), "v0");
        check(cudaMemcpy(x0, part.phase.x, 12ull * n, cudaMemcpyDeviceToDevice), "x0 copy");
        check(cudaMemcpy(v0, part.phase.v, 12ull * n, cudaMemcpyDeviceToDevice), "v0 copy");
        auto reload = [&]() {
            check(cudaMemcpy(part.phase.x, x0, 12ull * n, cudaMemcpyDeviceToDevice), "reload x");
            check(cudaMemcpy(part.phase.v, v0, 12ull * n, cudaMemcpyDeviceToDevice), "reload v");
            part.phase.num = n;
        };
        reload();
        step();
        check(cudaDeviceSynchronize(), "warm-up step");
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0);
        for (int r = 0; r < reps; ++r) {
            reload();
            step();
        }
        cudaEventRecord(e1);
        check(cudaEventSynchronize(e1), "timed steps");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        printf("ms_per_step %.6f\n", ms / reps);
        reload();
        cudaFree(x0);
        cudaFree(v0);
    }
    step();
    check(cudaDeviceSynchronize(), "one_step");

    pbf::neighbor_search &ns = *part.ns;
    const uint32_t num = part.phase.num;
    const dom_udim grid = ns.getGridSize();
    const uint32_t C = grid.x * grid.y * grid.z;
    const uint32_t mp = ns.getMaxPairParticleNum();
    std::vector<float> xo(3 * num), vo(3 * num);
    std::vector<uint32_t> sh(n), si(n), cs(C), ce(C), nl((size_t)((num + 31) / 32 * 32) * mp);
    check(cudaMemcpy(xo.data(), part.phase.x, 12ull * num, cudaMemcpyDeviceToHost), "x out");
    check(cudaMemcpy(vo.data(), part.phase.v, 12ull * num, cudaMemcpyDeviceToHost), "v out");
    check(cudaMemcpy(sh.data(), ns.sorted_hash_index.d_hash, 4ull * n, cudaMemcpyDeviceToHost), "hash");
    check(cudaMemcpy(si.data(), ns.sorted_hash_index.d_index, 4ull * n, cudaMemcpyDeviceToHost), "index");
    check(cudaMemcpy(cs.data(), ns.cell_start, 4ull * C, cudaMemcpyDeviceToHost), "cell_start");
    check(cudaMemcpy(ce.data(), ns.cell_end, 4ull * C, cudaMemcpyDeviceToHost), "cell_end");
    check(cudaMemcpy(nl.data(), ns.neighbor_list, 4ull * nl.size(), cudaMemcpyDeviceToHost), "list");

    FILE *o = fopen(argv[2], "wb");
    if (!o) return 1;
    fwrite("PBFO", 1, 4, o);
    const uint32_t hdr[6] = {num, n, grid.x, grid.y, grid.z, mp};
    wr(o, hdr, 6);
    wr(o, xo.data(), xo.size());
    wr(o, vo.data(), vo.size());
    wr(o, sh.data(), sh.size());
    wr(o, si.data(), si.size());
    wr(o, cs.data(), cs.size());
    wr(o, ce.data(), ce.size());
    wr(o, nl.data(), nl.size());
    fclose(o);
    return 0;
}
