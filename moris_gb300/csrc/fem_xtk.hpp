// fem_xtk.hpp -- the XFEM decomposition result shared by the host
// decomposition (fem_xtk.cpp) and the device one (fem_xtk_device.cu).
#pragma once

#include <cstdint>
#include <vector>

namespace fem {

struct IgVertex {
    int32_t kind;        // 0 background node, 1 face centre, 2 cell centre, 3 intersection
    int32_t parents[8];  // background nodes (kinds 0-2) or the two parent IG vertices (kind 3)
    double x[3];
    double value;        // level set (kinds 0-2) or edge coordinate t from parents[0] (kind 3)
};

}  // namespace fem

struct fem_xtk_model {
    int p = 1;
    int64_t ne[3] = {0, 0, 0}, nn[3] = {0, 0, 0}, nbk[3] = {0, 0, 0};
    // enriched interpolation mesh
    std::vector<double> coords;
    std::vector<int32_t> cells;
    std::vector<int64_t> t_off;
    std::vector<int32_t> t_bases;
    std::vector<double> t_w;
    std::vector<int32_t> cell_bg, cell_phase;
    int64_t num_enriched_bases = 0;
    // clusters
    std::vector<int32_t> uncut[2], cut[2];
    std::vector<int64_t> ig_off[2];
    std::vector<double> ig_x[2], ig_xi[2];
    std::vector<int32_t> ig_v[2];
    std::vector<int32_t> if_leader, if_follower;
    std::vector<int64_t> if_off;
    std::vector<double> if_x, if_xi;
    std::vector<int32_t> if_v;
    std::vector<int32_t> gh_leader[2], gh_follower[2];
    std::vector<double> gh_x[2], gh_xi_l[2], gh_xi_f[2];
    std::vector<fem::IgVertex> verts;
};

namespace fem {
// cube corner parametric coordinates and the facet node lists of HEX8
extern const int kHexSides[6][4];
extern const double kHexXi[8][3];
}  // namespace fem
