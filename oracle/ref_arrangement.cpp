// Runs the reference's own arrangement generators (src/pbf/util/pbf_arrangement.h,
// from the copy that oracle/ref_build.py prepares under oracle/_ref/src) on
// the cases read from stdin and writes their points to stdout — TEST
// INFRASTRUCTURE ONLY: tests/golden/make_arrangement_golden.py builds and
// runs it to pin oracle/arrangement.py.
//
// stdin, one case per line:
//   volume ox oy oz ex ey ez space
//   rectangle axis axis_value ox oy ex ey space
//   line ox oy oz ex ey ez space
//   cylinder axis axis_value ox oy radius height space
// stdout per case: uint32 count, then count x 3 float32 (binary).
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "pbf/util/pbf_arrangement.h"

int main()
{
    std::string kind;
    while (std::cin >> kind) {
        dom_dim_vec pos;
        if (kind == "volume" || kind == "line") {
            float o[3], e[3], s;
            std::cin >> o[0] >> o[1] >> o[2] >> e[0] >> e[1] >> e[2] >> s;
            const glm::vec3 O(o[0], o[1], o[2]), E(e[0], e[1], e[2]);
            if (kind == "volume") pbf::cartesian_volume(pos, O, E, s);
            else pbf::cartesian_line_inclusive(pos, O, E, s);
        } else if (kind == "rectangle") {
            std::string axis;
            float av, o[2], e[2], s;
            std::cin >> axis >> av >> o[0] >> o[1] >> e[0] >> e[1] >> s;
            pbf::cartesian_rectangle(pos, axis, av, glm::vec2(o[0], o[1]), glm::vec2(e[0], e[1]), s);
        } else if (kind == "cylinder") {
            std::string axis;
            float av, o[2], r, h, s;
            std::cin >> axis >> av >> o[0] >> o[1] >> r >> h >> s;
            pbf::cartesian_cylinder(pos, axis, av, glm::vec2(o[0], o[1]), r, h, s);
        } else {
            return 2;
        }
        const uint32_t n = (uint32_t)pos.size();
        std::fwrite(&n, 4, 1, stdout);
        for (const auto &p : pos) {
            const float xyz[3] = {p.x, p.y, p.z};
            std::fwrite(xyz, 4, 3, stdout);
        }
    }
    return 0;
}
