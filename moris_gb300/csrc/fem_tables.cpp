// fem_tables.cpp -- Gauss rules, Lagrange shape functions and facet maps of
// the reference element (host side; the kernels receive these as tables
// evaluated at the Gauss points).
//
// The point coordinates, their order and the weights are the reference's
// 15-significant-digit values (MTK/src/integration/
// cl_MTK_Integration_Coeffs_{Bar_1,Bar_3,Quad_2x2,Hex_2x2x2,Hex_3x3x3,Tri_3,
// Tri_7,Tet_4,Tet_11}.hpp) so that integration-point order and rounding match
// the reference element loop.  Shape functions follow MTK/src/interpolation/
// cl_MTK_Interpolation_Function_Lagrange_{Bar2,Quad4,Hex8,Tri3,Tet4}.hpp
// (tet barycentric order xi1, xi2, 1-xi1-xi2-xi3, xi3).
#include <cstring>

#include "fem_internal.hpp"
#include "fem_shape.hpp"

namespace fem {

namespace {
// 1D Gauss-Legendre abscissae as written in the reference tables
constexpr double kG2 = 0.577350269189626;
constexpr double kG3 = 0.774596669241483;

void push(Rule& r, double x, double y, double z, double w) {
    const double v[3] = {x, y, z};
    for (int d = 0; d < r.dim; ++d) r.pts.push_back(v[d]);
    r.w.push_back(w);
}
}  // namespace

Rule gauss_rule(int rule) {
    Rule r;
    switch (rule) {
        case FEM_GPU_RULE_BAR_1:
            r.dim = 1;
            push(r, 0.0, 0, 0, 2.0);
            break;
        case FEM_GPU_RULE_BAR_3:
            r.dim = 1;
            push(r, -0.7745966692414834, 0, 0, 5.555555555555556e-01);
            push(r, 0.0, 0, 0, 8.888888888888888e-01);
            push(r, 0.7745966692414834, 0, 0, 5.555555555555556e-01);
            break;
        case FEM_GPU_RULE_QUAD_2x2:
        case FEM_GPU_RULE_HEX_2x2x2: {
            // counter-clockwise in (x, y), then the upper z layer
            r.dim = rule == FEM_GPU_RULE_QUAD_2x2 ? 2 : 3;
            const double sx[4] = {-1, 1, 1, -1}, sy[4] = {-1, -1, 1, 1};
            const int layers = r.dim == 2 ? 1 : 2;
            for (int l = 0; l < layers; ++l)
                for (int k = 0; k < 4; ++k) push(r, sx[k] * kG2, sy[k] * kG2, (l ? 1.0 : -1.0) * kG2, 1.0);
            break;
        }
        case FEM_GPU_RULE_HEX_3x3x3: {
            // each z layer in hex27 node order: corners, edge mid-points, centre
            r.dim = 3;
            const double sx[9] = {-1, 1, 1, -1, 0, 1, 0, -1, 0};
            const double sy[9] = {-1, -1, 1, 1, -1, 0, 1, 0, 0};
            const double wc = 0.171467764060357, we = 0.274348422496571, wf = 0.438957475994513,
                         wm = 0.702331961591221;
            // weight of a point = product class: number of zero coordinates
            const double wt[4] = {wc, we, wf, wm};
            for (int l = 0; l < 3; ++l) {
                const double z = (l - 1) * kG3;
                for (int k = 0; k < 9; ++k) {
                    const int zeros = (sx[k] == 0) + (sy[k] == 0) + (l == 1);
                    push(r, sx[k] * kG3, sy[k] * kG3, z, wt[zeros]);
                }
            }
            break;
        }
        case FEM_GPU_RULE_TRI_3:
            r.dim = 2;
            push(r, 0.666666666666667, 0.166666666666667, 0, 0.333333333333333);
            push(r, 0.166666666666667, 0.666666666666667, 0, 0.333333333333333);
            push(r, 0.166666666666667, 0.166666666666667, 0, 0.333333333333333);
            break;
        case FEM_GPU_RULE_TRI_7: {
            r.dim = 2;
            const double a1 = 0.797426985353087, b1 = 0.101286507323456;
            const double a2 = 0.059715871789770, b2 = 0.470142064105115;
            const double w1 = 0.125939180544827, w2 = 0.132394152788506;
            push(r, 0.333333333333333, 0.333333333333333, 0, 0.225000000000000);
            push(r, a1, b1, 0, w1);
            push(r, b1, a1, 0, w1);
            push(r, b1, b1, 0, w1);
            push(r, a2, b2, 0, w2);
            push(r, b2, a2, 0, w2);
            push(r, b2, b2, 0, w2);
            break;
        }
        case FEM_GPU_RULE_TET_4: {
            r.dim = 3;
            const double a = 0.585410196624968, b = 0.138196601125010;
            push(r, a, b, b, 0.25);
            push(r, b, a, b, 0.25);
            push(r, b, b, b, 0.25);
            push(r, b, b, a, 0.25);
            break;
        }
        case FEM_GPU_RULE_TET_11: {
            // table weights are stored /6 in the reference and scaled by 6.0
            r.dim = 3;
            const double a = 0.7857142857142860, b = 0.0714285714285714;
            const double c = 0.3994035761667990, d = 0.1005964238332010;
            const double w1 = 6.0 * 0.0076222222222222, w2 = 6.0 * 0.0248888888888889;
            push(r, a, b, b, w1);
            push(r, b, a, b, w1);
            push(r, b, b, b, w1);
            push(r, b, b, a, w1);
            push(r, c, c, d, w2);
            push(r, c, d, d, w2);
            push(r, c, d, c, w2);
            push(r, d, c, d, w2);
            push(r, d, c, c, w2);
            push(r, d, d, c, w2);
            push(r, 0.25, 0.25, 0.25, 6.0 * -0.0131555555555556);
            break;
        }
        default:
            break;
    }
    r.n = r.dim ? (int)r.w.size() : 0;
    return r;
}

int cell_num_nodes(int cell) {
    switch (cell) {
        case FEM_GPU_CELL_QUAD4: return 4;
        case FEM_GPU_CELL_HEX8: return 8;
        case FEM_GPU_CELL_TRI3: return 3;
        case FEM_GPU_CELL_TET4: return 4;
        case FEM_GPU_CELL_LINE2: return 2;
        default: return 0;
    }
}

int cell_param_dim(int cell) {
    switch (cell) {
        case FEM_GPU_CELL_QUAD4: return 2;
        case FEM_GPU_CELL_HEX8: return 3;
        case FEM_GPU_CELL_TRI3: return 2;
        case FEM_GPU_CELL_TET4: return 3;
        case FEM_GPU_CELL_LINE2: return 1;
        default: return 0;
    }
}

void cell_param_coords(int cell, double* X) {
    switch (cell) {
        case FEM_GPU_CELL_LINE2: X[0] = -1; X[1] = 1; break;
        case FEM_GPU_CELL_QUAD4:
        case FEM_GPU_CELL_HEX8: {
            const int n = cell_num_nodes(cell), pd = cell_param_dim(cell);
            const double sx[4] = {-1, 1, 1, -1}, sy[4] = {-1, -1, 1, 1};
            for (int a = 0; a < n; ++a) {
                X[a * pd + 0] = sx[a % 4];
                X[a * pd + 1] = sy[a % 4];
                if (pd == 3) X[a * pd + 2] = a < 4 ? -1.0 : 1.0;
            }
            break;
        }
        case FEM_GPU_CELL_TRI3: {
            const double v[6] = {1, 0, 0, 1, 0, 0};
            std::memcpy(X, v, sizeof v);
            break;
        }
        case FEM_GPU_CELL_TET4: {
            const double v[12] = {1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 1};
            std::memcpy(X, v, sizeof v);
            break;
        }
        default: break;
    }
}

void lagrange(int cell, const double* xi, double* N, double* dN) {
    switch (cell) {
        case FEM_GPU_CELL_LINE2: Shape<4>::eval(xi, N, dN); break;
        case FEM_GPU_CELL_QUAD4: Shape<0>::eval(xi, N, dN); break;
        case FEM_GPU_CELL_HEX8: Shape<1>::eval(xi, N, dN); break;
        case FEM_GPU_CELL_TRI3: Shape<2>::eval(xi, N, dN); break;
        case FEM_GPU_CELL_TET4: Shape<3>::eval(xi, N, dN); break;
        default: break;
    }
}

// facet vertex lists: quad edges (MTK Cell_Info_Quad4 node_to_edge) and hex
// faces (MTK Cell_Info_Hex8 node_to_face, outward orientation)
const int* facet_vertices(int ip_cell, int ordinal, int* count) {
    static const int kQuad[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
    static const int kHex[6][4] = {{1, 5, 4, 0}, {1, 2, 6, 5}, {3, 7, 6, 2},
                                   {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};
    if (ip_cell == FEM_GPU_CELL_QUAD4 && ordinal >= 0 && ordinal < 4) {
        *count = 2;
        return kQuad[ordinal];
    }
    if (ip_cell == FEM_GPU_CELL_HEX8 && ordinal >= 0 && ordinal < 6) {
        *count = 4;
        return kHex[ordinal];
    }
    *count = 0;
    return nullptr;
}

}  // namespace fem
