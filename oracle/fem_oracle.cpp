/*
 * fem_oracle.cpp -- CPU oracle for the MORIS element hot path.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker and as the timed host-core
 * restatement.  The product library (moris_gb300/) never links or calls it.
 *
 * This file restates, routine by routine, the reference's algorithm on plain
 * column-major dense matrices (the reference's LINALG Matrix<> is
 * column-major too).  Paths are relative to the reference's projects/
 * directory.  The restatement keeps the reference's formulation: dense
 * B^T D B per Gauss point (CM_Struc_Linear), dense T^T K T per equation
 * object (MSI::Equation_Object), sorted per-type adof lists, |T| <= 1e-12
 * dropped per node (HMR T_Matrix_Base::evaluate).
 *
 * Parity pins: the Gauss tables and Lagrange shape functions are checked
 * against the reference's own fixture files (FEM/INT/test/data/ .bin files), the
 * element Jacobians against central finite differences of the residual as in
 * the reference's IWG unit tests, and the B-spline extraction against the
 * partition-of-unity checks of HMR/test/ut_HMR_T_Matrix.cpp.
 */
#include "fem_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <thread>
#include <vector>

namespace {

using real = double;

/* ------------------------------------------------------------------------ */
/* minimal column-major dense matrix (the reference's Matrix<DDRMat> layout) */
struct Mat {
    int r = 0, c = 0;
    std::vector<real> a;
    Mat() = default;
    Mat(int rr, int cc, real v = 0.0) : r(rr), c(cc), a((size_t)rr * cc, v) {}
    real& operator()(int i, int j) { return a[(size_t)i + (size_t)j * r]; }
    real operator()(int i, int j) const { return a[(size_t)i + (size_t)j * r]; }
    void fill(real v) { std::fill(a.begin(), a.end(), v); }
};

Mat mul(const Mat& A, const Mat& B) {
    Mat C(A.r, B.c, 0.0);
    for (int j = 0; j < B.c; ++j)
        for (int k = 0; k < A.c; ++k) {
            const real b = B(k, j);
            if (b == 0.0) continue;
            for (int i = 0; i < A.r; ++i) C(i, j) += A(i, k) * b;
        }
    return C;
}
Mat trans(const Mat& A) {
    Mat T(A.c, A.r);
    for (int i = 0; i < A.r; ++i)
        for (int j = 0; j < A.c; ++j) T(j, i) = A(i, j);
    return T;
}
void add_scaled(Mat& Y, real s, const Mat& X) {
    for (size_t i = 0; i < Y.a.size(); ++i) Y.a[i] += s * X.a[i];
}

/* ------------------------------------------------------------------------ */
/* Gauss tables.  Values and point order are those of the reference's
   MTK/src/integration/cl_MTK_Integration_Coeffs_*.hpp (15-digit literals,
   HEX_3x3x3 in its layer-wise corner/edge/centre order, TET_11 weights
   multiplied by 6 as in cl_MTK_Integration_Coeffs_Tet_11.hpp:117).         */
struct RuleTab {
    int dim, n;
    std::vector<real> pts;  // dim x n column-major
    std::vector<real> w;
};

RuleTab make_rule(int rule) {
    RuleTab t;
    const real g2 = 0.577350269189626;   // Quad_2x2 / Hex_2x2x2 literal
    const real g3 = 0.774596669241483;   // Hex_3x3x3 literal
    switch (rule) {
        case ORC_RULE_BAR_1:  // cl_MTK_Integration_Coeffs_Bar_1.hpp:50-63
            t.dim = 1; t.n = 1; t.pts = {0.0}; t.w = {2.0};
            break;
        case ORC_RULE_BAR_3:  // cl_MTK_Integration_Coeffs_Bar_3.hpp
            t.dim = 1; t.n = 3;
            t.pts = {-0.7745966692414834, 0.000000000000000, 0.7745966692414834};
            t.w = {5.555555555555556e-01, 8.888888888888888e-01, 5.555555555555556e-01};
            break;
        case ORC_RULE_QUAD_2x2: {  // cl_MTK_Integration_Coeffs_Quad_2x2.hpp
            t.dim = 2; t.n = 4;
            const real x[4] = {-g2, g2, g2, -g2}, y[4] = {-g2, -g2, g2, g2};
            for (int k = 0; k < 4; ++k) { t.pts.push_back(x[k]); t.pts.push_back(y[k]); }
            t.w = {1.0, 1.0, 1.0, 1.0};
            break;
        }
        case ORC_RULE_HEX_2x2x2: {  // cl_MTK_Integration_Coeffs_Hex_2x2x2.hpp:50-76
            t.dim = 3; t.n = 8;
            const real x[8] = {-g2, g2, g2, -g2, -g2, g2, g2, -g2};
            const real y[8] = {-g2, -g2, g2, g2, -g2, -g2, g2, g2};
            const real z[8] = {-g2, -g2, -g2, -g2, g2, g2, g2, g2};
            for (int k = 0; k < 8; ++k) { t.pts.push_back(x[k]); t.pts.push_back(y[k]); t.pts.push_back(z[k]); }
            t.w.assign(8, 1.0);
            break;
        }
        case ORC_RULE_HEX_3x3x3: {  // cl_MTK_Integration_Coeffs_Hex_3x3x3.hpp:50+
            t.dim = 3; t.n = 27;
            // per z-layer: 4 corners, 4 edge mid-points, centre (hex27 node order)
            const real lx[9] = {-g3, g3, g3, -g3, 0.0, g3, 0.0, -g3, 0.0};
            const real ly[9] = {-g3, -g3, g3, g3, -g3, 0.0, g3, 0.0, 0.0};
            const real lz[3] = {-g3, 0.0, g3};
            const real wo[9] = {0.171467764060357, 0.171467764060357, 0.171467764060357, 0.171467764060357,
                                0.274348422496571, 0.274348422496571, 0.274348422496571, 0.274348422496571,
                                0.438957475994513};
            const real wm[9] = {0.274348422496571, 0.274348422496571, 0.274348422496571, 0.274348422496571,
                                0.438957475994513, 0.438957475994513, 0.438957475994513, 0.438957475994513,
                                0.702331961591221};
            for (int l = 0; l < 3; ++l)
                for (int k = 0; k < 9; ++k) {
                    t.pts.push_back(lx[k]); t.pts.push_back(ly[k]); t.pts.push_back(lz[l]);
                    t.w.push_back(l == 1 ? wm[k] : wo[k]);
                }
            break;
        }
        case ORC_RULE_TRI_3:  // cl_MTK_Integration_Coeffs_Tri_3.hpp
            t.dim = 2; t.n = 3;
            t.pts = {0.666666666666667, 0.166666666666667, 0.166666666666667, 0.666666666666667,
                     0.166666666666667, 0.166666666666667};
            t.w = {0.333333333333333, 0.333333333333333, 0.333333333333333};
            break;
        case ORC_RULE_TRI_7: {  // cl_MTK_Integration_Coeffs_Tri_7.hpp
            t.dim = 2; t.n = 7;
            const real x[7] = {0.333333333333333, 0.797426985353087, 0.101286507323456, 0.101286507323456,
                               0.059715871789770, 0.470142064105115, 0.470142064105115};
            const real y[7] = {0.333333333333333, 0.101286507323456, 0.797426985353087, 0.101286507323456,
                               0.470142064105115, 0.059715871789770, 0.470142064105115};
            for (int k = 0; k < 7; ++k) { t.pts.push_back(x[k]); t.pts.push_back(y[k]); }
            t.w = {0.225000000000000, 0.125939180544827, 0.125939180544827, 0.125939180544827,
                   0.132394152788506, 0.132394152788506, 0.132394152788506};
            break;
        }
        case ORC_RULE_TET_4: {  // cl_MTK_Integration_Coeffs_Tet_4.hpp
            t.dim = 3; t.n = 4;
            const real a = 0.585410196624968, b = 0.138196601125010;
            const real x[4] = {a, b, b, b}, y[4] = {b, a, b, b}, z[4] = {b, b, b, a};
            for (int k = 0; k < 4; ++k) { t.pts.push_back(x[k]); t.pts.push_back(y[k]); t.pts.push_back(z[k]); }
            t.w.assign(4, 0.25);
            break;
        }
        case ORC_RULE_TET_11: {  // cl_MTK_Integration_Coeffs_Tet_11.hpp (weights x 6.0 at :117)
            t.dim = 3; t.n = 11;
            const real x[11] = {0.7857142857142860, 0.0714285714285714, 0.0714285714285714, 0.0714285714285714,
                                0.3994035761667990, 0.3994035761667990, 0.3994035761667990, 0.1005964238332010,
                                0.1005964238332010, 0.1005964238332010, 0.2500000000000000};
            const real y[11] = {0.0714285714285714, 0.7857142857142860, 0.0714285714285714, 0.0714285714285714,
                                0.3994035761667990, 0.1005964238332010, 0.1005964238332010, 0.3994035761667990,
                                0.3994035761667990, 0.1005964238332010, 0.2500000000000000};
            const real z[11] = {0.0714285714285714, 0.0714285714285714, 0.0714285714285714, 0.7857142857142860,
                                0.1005964238332010, 0.1005964238332010, 0.3994035761667990, 0.1005964238332010,
                                0.3994035761667990, 0.3994035761667990, 0.2500000000000000};
            const real w[11] = {0.0076222222222222, 0.0076222222222222, 0.0076222222222222, 0.0076222222222222,
                                0.0248888888888889, 0.0248888888888889, 0.0248888888888889, 0.0248888888888889,
                                0.0248888888888889, 0.0248888888888889, -0.0131555555555556};
            for (int k = 0; k < 11; ++k) {
                t.pts.push_back(x[k]); t.pts.push_back(y[k]); t.pts.push_back(z[k]);
                t.w.push_back(6.0 * w[k]);
            }
            break;
        }
        default:
            t.dim = 0; t.n = 0;
    }
    return t;
}

/* ------------------------------------------------------------------------ */
/* Lagrange shape functions, MTK/src/interpolation/
   cl_MTK_Interpolation_Function_Lagrange_{Bar2,Quad4,Hex8,Tri3,Tet4}.hpp     */
int cell_nodes(int cell) {
    switch (cell) {
        case ORC_CELL_QUAD4: return 4;
        case ORC_CELL_HEX8: return 8;
        case ORC_CELL_TRI3: return 3;
        case ORC_CELL_TET4: return 4;
        case ORC_CELL_LINE2: return 2;
    }
    return 0;
}
int cell_pdim(int cell) {
    switch (cell) {
        case ORC_CELL_QUAD4: return 2;
        case ORC_CELL_HEX8: return 3;
        case ORC_CELL_TRI3: return 2;
        case ORC_CELL_TET4: return 3;
        case ORC_CELL_LINE2: return 1;
    }
    return 0;
}

void shape(int cell, const real* xi, Mat& N, Mat& dN) {
    const int n = cell_nodes(cell), pd = cell_pdim(cell);
    N = Mat(1, n);
    dN = Mat(pd, n);
    switch (cell) {
        case ORC_CELL_LINE2: {  // ..._Lagrange_Bar2.hpp
            const real x = xi[0];
            N(0, 0) = 0.5 * (1.0 - x);
            N(0, 1) = 0.5 * (1.0 + x);
            dN(0, 0) = -0.5;
            dN(0, 1) = 0.5;
            break;
        }
        case ORC_CELL_QUAD4: {  // ..._Lagrange_Quad4.hpp:61-110
            const real x = xi[0], e = xi[1];
            N(0, 0) = ((1.0 - x) * (1.0 - e)) * 0.25;
            N(0, 1) = ((1.0 + x) * (1.0 - e)) * 0.25;
            N(0, 2) = ((1.0 + x) * (1.0 + e)) * 0.25;
            N(0, 3) = ((1.0 - x) * (1.0 + e)) * 0.25;
            dN(0, 0) = 0.25 * (e - 1.0);
            dN(1, 0) = 0.25 * (x - 1.0);
            dN(0, 1) = -0.25 * (e - 1.0);
            dN(1, 1) = -0.25 * (x + 1.0);
            dN(0, 2) = 0.25 * (e + 1.0);
            dN(1, 2) = 0.25 * (x + 1.0);
            dN(0, 3) = -0.25 * (e + 1.0);
            dN(1, 3) = -0.25 * (x - 1.0);
            break;
        }
        case ORC_CELL_HEX8: {  // ..._Lagrange_Hex8.hpp:83-160
            const real x = xi[0], e = xi[1], z = xi[2];
            N(0, 0) = -(e - 1.0) * (x - 1.0) * (z - 1.0) * 0.125;
            N(0, 1) = (e - 1.0) * (x + 1.0) * (z - 1.0) * 0.125;
            N(0, 2) = -(e + 1.0) * (x + 1.0) * (z - 1.0) * 0.125;
            N(0, 3) = (e + 1.0) * (x - 1.0) * (z - 1.0) * 0.125;
            N(0, 4) = (e - 1.0) * (x - 1.0) * (z + 1.0) * 0.125;
            N(0, 5) = -(e - 1.0) * (x + 1.0) * (z + 1.0) * 0.125;
            N(0, 6) = (e + 1.0) * (x + 1.0) * (z + 1.0) * 0.125;
            N(0, 7) = -(e + 1.0) * (x - 1.0) * (z + 1.0) * 0.125;
            // derivatives of the node-wise sign products (+-1 +- xi)...
            const real sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
            const real sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
            const real sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
            for (int a = 0; a < 8; ++a) {
                const real fx = 1.0 + sx[a] * x, fy = 1.0 + sy[a] * e, fz = 1.0 + sz[a] * z;
                dN(0, a) = 0.125 * sx[a] * fy * fz;
                dN(1, a) = 0.125 * sy[a] * fx * fz;
                dN(2, a) = 0.125 * sz[a] * fx * fy;
            }
            break;
        }
        case ORC_CELL_TRI3: {  // ..._Lagrange_Tri3.hpp:56-100
            N(0, 0) = xi[0];
            N(0, 1) = xi[1];
            N(0, 2) = 1.0 - xi[0] - xi[1];
            dN(0, 0) = 1.0; dN(1, 0) = 0.0;
            dN(0, 1) = 0.0; dN(1, 1) = 1.0;
            dN(0, 2) = -1.0; dN(1, 2) = -1.0;
            break;
        }
        case ORC_CELL_TET4: {  // ..._Lagrange_Tet4.hpp: order (xi1, xi2, 1-sum, xi3)
            N(0, 0) = xi[0];
            N(0, 1) = xi[1];
            N(0, 2) = 1.0 - xi[0] - xi[1] - xi[2];
            N(0, 3) = xi[2];
            dN(0, 0) = 1.0; dN(1, 0) = 0.0; dN(2, 0) = 0.0;
            dN(0, 1) = 0.0; dN(1, 1) = 1.0; dN(2, 1) = 0.0;
            dN(0, 2) = -1.0; dN(1, 2) = -1.0; dN(2, 2) = -1.0;
            dN(0, 3) = 0.0; dN(1, 3) = 0.0; dN(2, 3) = 1.0;
            break;
        }
    }
}

/* reference-element vertex parameter coordinates (get_param_coords) */
void param_coords(int cell, Mat& X) {
    const int n = cell_nodes(cell), pd = cell_pdim(cell);
    X = Mat(n, pd);
    if (cell == ORC_CELL_QUAD4) {
        const real v[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
        for (int a = 0; a < 4; ++a) for (int d = 0; d < 2; ++d) X(a, d) = v[a][d];
    } else if (cell == ORC_CELL_HEX8) {
        const real v[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                              {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
        for (int a = 0; a < 8; ++a) for (int d = 0; d < 3; ++d) X(a, d) = v[a][d];
    } else if (cell == ORC_CELL_TET4) {
        const real v[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 1}};
        for (int a = 0; a < 4; ++a) for (int d = 0; d < 3; ++d) X(a, d) = v[a][d];
    } else if (cell == ORC_CELL_TRI3) {
        const real v[3][2] = {{1, 0}, {0, 1}, {0, 0}};
        for (int a = 0; a < 3; ++a) for (int d = 0; d < 2; ++d) X(a, d) = v[a][d];
    } else if (cell == ORC_CELL_LINE2) {
        X(0, 0) = -1; X(1, 0) = 1;
    }
}

/* facet vertex maps: MTK/src/geometry/cell/cl_MTK_Cell_Info_Quad4.cpp:155
   (node_to_edge) and cl_MTK_Cell_Info_Hex8.cpp:177 (node_to_face).         */
const int QUAD4_SIDES[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
const int HEX8_SIDES[6][4] = {{1, 5, 4, 0}, {1, 2, 6, 5}, {3, 7, 6, 2}, {0, 4, 7, 3}, {0, 3, 2, 1}, {4, 5, 6, 7}};

/* ------------------------------------------------------------------------ */
/* Space_Interpolator: J = dN/dxi * Xhat (cl_MTK_Space_Interpolator.cpp:413),
   detJ (hex/quad general :1006, rect :1055/:954, tet /6 :1180, tri /2),
   inverse (3d :610, rect :676-706).                                          */
real det_bulk(const Mat& J, int cell, bool rect) {
    const int d = J.r;
    if (d == 2) {
        real det = rect ? J(0, 0) * J(1, 1) : J(0, 0) * J(1, 1) - J(0, 1) * J(1, 0);
        if (cell == ORC_CELL_TRI3) det /= 2.0;
        return det;
    }
    if (rect && cell == ORC_CELL_HEX8) return J(1, 1) * J(0, 0) * J(2, 2);
    real det = +J(0, 0) * (J(1, 1) * J(2, 2) - J(2, 1) * J(1, 2)) -
               J(0, 1) * (J(1, 0) * J(2, 2) - J(1, 2) * J(2, 0)) +
               J(0, 2) * (J(1, 0) * J(2, 1) - J(1, 1) * J(2, 0));
    if (cell == ORC_CELL_TET4) det /= 6.0;
    return det;
}

Mat inverse_ip(const Mat& J, bool rect) {
    const int d = J.r;
    Mat I(d, d, 0.0);
    if (rect) {
        for (int i = 0; i < d; ++i) I(i, i) = 1.0 / J(i, i);
        return I;
    }
    if (d == 2) {
        const real det = J(0, 0) * J(1, 1) - J(0, 1) * J(1, 0);
        const real inv = 1.0 / det;
        I(0, 0) = J(1, 1) * inv;
        I(0, 1) = -J(0, 1) * inv;
        I(1, 0) = -J(1, 0) * inv;
        I(1, 1) = J(0, 0) * inv;
        return I;
    }
    const real det = +J(0, 0) * (J(1, 1) * J(2, 2) - J(2, 1) * J(1, 2)) -
                     J(0, 1) * (J(1, 0) * J(2, 2) - J(1, 2) * J(2, 0)) +
                     J(0, 2) * (J(1, 0) * J(2, 1) - J(1, 1) * J(2, 0));
    const real inv = 1.0 / det;
    I(0, 0) = (J(1, 1) * J(2, 2) - J(2, 1) * J(1, 2)) * inv;
    I(0, 1) = (J(0, 2) * J(2, 1) - J(0, 1) * J(2, 2)) * inv;
    I(0, 2) = (J(0, 1) * J(1, 2) - J(0, 2) * J(1, 1)) * inv;
    I(1, 0) = (J(1, 2) * J(2, 0) - J(1, 0) * J(2, 2)) * inv;
    I(1, 1) = (J(0, 0) * J(2, 2) - J(0, 2) * J(2, 0)) * inv;
    I(1, 2) = (J(1, 0) * J(0, 2) - J(0, 0) * J(1, 2)) * inv;
    I(2, 0) = (J(1, 0) * J(2, 1) - J(2, 0) * J(1, 1)) * inv;
    I(2, 1) = (J(2, 0) * J(0, 1) - J(0, 0) * J(2, 1)) * inv;
    I(2, 2) = (J(0, 0) * J(1, 1) - J(1, 0) * J(0, 1)) * inv;
    return I;
}

/* ------------------------------------------------------------------------ */
/* CM_Struc_Linear_Isotropic constitutive matrices:
   full_plane_strain (FEM/INT/src/CM/cl_FEM_CM_Struc_Linear_Isotropic.cpp:282),
   full_plane_stress (:262), full_3d (:374).  Strain layout per
   CM_Struc_Linear::set_function_pointers (cl_FEM_CM_Struc_Linear.cpp:132-261).*/
Mat constitutive(int model, int dim, real E, real nu) {
    if (dim == 3) {
        Mat D(6, 6, 0.0);
        const real pre = E / (1.0 + nu) / (1.0 - 2.0 * nu);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) D(i, j) = pre * (i == j ? (1.0 - nu) : nu);
        for (int i = 3; i < 6; ++i) D(i, i) = pre * (1.0 - 2.0 * nu) / 2.0;
        return D;
    }
    if (model == ORC_MODEL_PLANE_STRESS) {
        Mat D(3, 3, 0.0);
        const real pre = E / (1.0 - nu * nu);
        D(0, 0) = pre;
        D(1, 1) = pre;
        D(0, 1) = pre * nu;
        D(1, 0) = pre * nu;
        D(2, 2) = pre * 0.5 * (1.0 - nu);
        return D;
    }
    Mat D(4, 4, 0.0);
    const real pre = E / (1.0 + nu) / (1.0 - 2.0 * nu);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D(i, j) = pre * (i == j ? (1.0 - nu) : nu);
    D(3, 3) = pre * (1.0 - 2.0 * nu) / 2.0;
    return D;
}

/* test strain B: CM_Struc_Linear::eval_teststrain_2d / _3d
   (cl_FEM_CM_Struc_Linear.cpp:503-592).  dNdx is dim x n.                   */
Mat test_strain(int model, const Mat& dNdx) {
    const int d = dNdx.r, n = dNdx.c;
    if (d == 3) {
        Mat B(6, 3 * n, 0.0);
        for (int a = 0; a < n; ++a) {
            B(0, a) = dNdx(0, a);
            B(4, a) = dNdx(2, a);
            B(5, a) = dNdx(1, a);
            B(1, n + a) = dNdx(1, a);
            B(3, n + a) = dNdx(2, a);
            B(5, n + a) = dNdx(0, a);
            B(2, 2 * n + a) = dNdx(2, a);
            B(3, 2 * n + a) = dNdx(1, a);
            B(4, 2 * n + a) = dNdx(0, a);
        }
        return B;
    }
    const int ns = (model == ORC_MODEL_PLANE_STRESS) ? 3 : 4;
    const int shear = ns - 1;
    Mat B(ns, 2 * n, 0.0);
    for (int a = 0; a < n; ++a) {
        B(0, a) = dNdx(0, a);
        B(1, n + a) = dNdx(1, a);
        B(shear, a) = dNdx(1, a);
        B(shear, n + a) = dNdx(0, a);
    }
    return B;
}

/* flatten_normal_2d / _3d (cl_FEM_CM_Struc_Linear.cpp:836-863) */
Mat flat_normal(const real* nrm, int dim, int nstress) {
    if (dim == 2) {
        Mat F(2, nstress, 0.0);
        F(0, 0) = nrm[0];
        F(0, nstress - 1) = nrm[1];
        F(1, 1) = nrm[1];
        F(1, nstress - 1) = nrm[0];
        return F;
    }
    Mat F(3, 6, 0.0);
    F(0, 0) = nrm[0];
    F(1, 1) = nrm[1];
    F(2, 2) = nrm[2];
    F(0, 4) = nrm[2];
    F(0, 5) = nrm[1];
    F(1, 3) = nrm[2];
    F(1, 5) = nrm[0];
    F(2, 3) = nrm[1];
    F(2, 4) = nrm[0];
    return F;
}

/* field N matrix for a vector field: Field_Interpolator::N()
   (FEM/INT/src/IP/cl_FEM_Field_Interpolator.cpp:310-400), type-major.       */
Mat field_N(const Mat& Nrow, int dim) {
    const int n = Nrow.c;
    Mat N(dim, dim * n, 0.0);
    for (int f = 0; f < dim; ++f)
        for (int a = 0; a < n; ++a) N(f, f * n + a) = Nrow(0, a);
    return N;
}

/* ------------------------------------------------------------------------ */
struct BulkSet {
    int ig_cell, rule, model;
    std::vector<int32_t> ip_cell;
    std::vector<int64_t> ig_off;  // empty => trivial
    std::vector<real> ig_coords, ig_param;
    std::vector<real> E;
    real nu;
    std::vector<real> node_rho;  // optional nodal density field
    real beta = 3.0;
    real thickness = 1.0;        // Thickness property (multiplies w*)
};
/* double-sided cluster set (interface / ghost): facets with vertex coords
   and their parametric coords in the leader and follower IP cells */
struct DoubleSet {
    int iwg, facet_cell, rule, model;
    std::vector<int32_t> leader, follower;
    std::vector<int64_t> fc_off;
    std::vector<real> fc_x, fc_xl, fc_xf;
    std::vector<real> EL, EF;
    real nu, alpha;
};
struct SideSet {
    int iwg, rule, model;
    std::vector<int32_t> ip_cell, ordinal;
    std::vector<real> E;
    real nu, alpha;
    real value[3];
    real thickness = 1.0;        // Thickness property (multiplies w*)
    bool has_select = false;     // Select property of the Dirichlet IWG (dim x dim)
    real select[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
};

}  // namespace

/* ======================================================================== */
struct orc_mesh {
    int dim;
    std::vector<real> coords;
    std::vector<int32_t> cells;
    int64_t num_bases;
    std::vector<int64_t> t_off;
    std::vector<int32_t> t_bases;
    std::vector<real> t_w;
};

struct orc_model {
    int dim, ip_cell, shape;
    int64_t num_nodes, num_cells, num_bases;
    std::vector<real> coords;
    std::vector<int32_t> cells;
    std::vector<int64_t> t_off;
    std::vector<int32_t> t_bases;
    std::vector<real> t_w;
    std::vector<BulkSet> bulk;
    std::vector<SideSet> side;
    std::vector<DoubleSet> dbl;
    // MSI products
    std::vector<int64_t> basis_rank;  // domain basis -> rank among used, -1 if unused
    int64_t num_used = 0;
    std::vector<std::vector<int32_t>> cell_ubases;  // sorted unique basis ranks per IP cell
    std::vector<int32_t> rowptr, colidx;
    bool finalized = false;
};

/* ------------------------------------------------------------------------ */
/* HMR: bspline_shape (HMR/src/fn_HMR_bspline_shape.cpp:20-58), Cox-de Boor on
   the element-local knot vector 2(i-p)-1, half-open support intervals.      */
static real bspline_shape(int p, int basis, real xi) {
    const int steps = 2 * (p + 1);
    std::vector<real> dxi(steps);
    for (int i = 0; i < steps; ++i) dxi[i] = ((real)i - (real)p) * 2.0 - 1.0;
    std::vector<real> N(p + 1, 0.0);
    for (int q = 0; q <= p; ++q)
        if (dxi[q + basis] <= xi && xi < dxi[q + basis + 1]) N[q] = 1.0;
    for (int q = 1; q <= p; ++q) {
        std::vector<real> Nold(N);
        for (int i = 0; i <= p - q; ++i) {
            const real A = xi - dxi[i + basis];
            const real B = dxi[i + basis + q + 1] - xi;
            N[i] = 0.5 * (A * Nold[i] + B * Nold[i + 1]) / (real)q;
        }
    }
    return N[0];
}

extern "C" {

/* Set::get_auto_integration_order (FEM/INT/src/CORE/cl_FEM_Set.cpp:2983-3185)
   for linear interpolation cells: the reference picks the rule from the set
   type and the integration cell's geometry.  kind 0 bulk, 1 side set,
   2 double side set; -1 if none.                                           */
int orc_auto_rule(int kind, int cell) {
    if (kind == 0) {
        if (cell == ORC_CELL_LINE2) return ORC_RULE_BAR_3;
        if (cell == ORC_CELL_QUAD4) return ORC_RULE_QUAD_2x2;
        if (cell == ORC_CELL_HEX8) return ORC_RULE_HEX_2x2x2;
        if (cell == ORC_CELL_TRI3) return ORC_RULE_TRI_7;
        if (cell == ORC_CELL_TET4) return ORC_RULE_TET_11;
        return -1;
    }
    if (kind == 1 || kind == 2) {
        if (cell == ORC_CELL_LINE2) return ORC_RULE_BAR_3;
        if (cell == ORC_CELL_QUAD4) return ORC_RULE_QUAD_2x2;
        if (cell == ORC_CELL_TRI3) return ORC_RULE_TRI_7;
    }
    return -1;
}

int orc_rule_size(int rule, int* dim, int* npts) {
    RuleTab t = make_rule(rule);
    if (t.n == 0) return 1;
    *dim = t.dim;
    *npts = t.n;
    return 0;
}
int orc_rule(int rule, double* pts, double* w) {
    RuleTab t = make_rule(rule);
    if (t.n == 0) return 1;
    std::memcpy(pts, t.pts.data(), sizeof(real) * t.pts.size());
    std::memcpy(w, t.w.data(), sizeof(real) * t.w.size());
    return 0;
}
int orc_cell_num_nodes(int cell) { return cell_nodes(cell); }
int orc_cell_param_dim(int cell) { return cell_pdim(cell); }
int orc_shape(int cell, const double* xi, double* N, double* dNdxi) {
    if (cell_nodes(cell) == 0) return 1;
    Mat n, dn;
    shape(cell, xi, n, dn);
    std::memcpy(N, n.a.data(), sizeof(real) * n.a.size());
    std::memcpy(dNdxi, dn.a.data(), sizeof(real) * dn.a.size());
    return 0;
}
double orc_bspline_shape(int order, int basis, double xi) { return bspline_shape(order, basis, xi); }

/* HMR level-0 uniform mesh.  Elements and bases are numbered i-fastest
   (BSpline_Mesh::create_basis_on_level_zero, HMR/src/cl_HMR_BSpline_Mesh.hpp:
   474-535); the node T rows are T = L (init_lagrange_matrix,
   cl_HMR_T_Matrix.hpp:433-463; level 0 needs no refinement matrix) evaluated
   by the first element that visits the node, dropping |T| <= 1e-12
   (T_Matrix_Base::evaluate, cl_HMR_T_Matrix_Base.cpp:394-420).              */
orc_mesh* orc_hmr_uniform(int dim, const int* ne, const double* len, int p) {
    if (dim < 2 || dim > 3 || p < 1 || p > 3) return nullptr;
    auto* m = new orc_mesh;
    m->dim = dim;
    int nn[3] = {1, 1, 1}, nb[3] = {1, 1, 1}, nel[3] = {1, 1, 1};
    for (int d = 0; d < dim; ++d) {
        nel[d] = ne[d];
        nn[d] = ne[d] + 1;
        nb[d] = ne[d] + p;
    }
    const int64_t num_nodes = (int64_t)nn[0] * nn[1] * nn[2];
    const int64_t num_cells = (int64_t)nel[0] * nel[1] * nel[2];
    m->num_bases = (int64_t)nb[0] * nb[1] * nb[2];
    m->coords.resize(num_nodes * dim);
    for (int64_t k = 0; k < nn[2]; ++k)
        for (int64_t j = 0; j < nn[1]; ++j)
            for (int64_t i = 0; i < nn[0]; ++i) {
                const int64_t id = i + nn[0] * (j + nn[1] * k);
                const int64_t ijk[3] = {i, j, k};
                for (int d = 0; d < dim; ++d) m->coords[id * dim + d] = len[d] * (real)ijk[d] / (real)nel[d];
            }
    const int npe = dim == 2 ? 4 : 8;
    Mat XI;
    param_coords(dim == 2 ? ORC_CELL_QUAD4 : ORC_CELL_HEX8, XI);
    m->cells.resize(num_cells * npe);
    std::vector<std::vector<std::pair<int32_t, real>>> rows(num_nodes);
    std::vector<char> done(num_nodes, 0);
    const int nlb = dim == 2 ? (p + 1) * (p + 1) : (p + 1) * (p + 1) * (p + 1);
    for (int64_t ek = 0; ek < nel[2]; ++ek)
        for (int64_t ej = 0; ej < nel[1]; ++ej)
            for (int64_t ei = 0; ei < nel[0]; ++ei) {
                const int64_t e = ei + nel[0] * (ej + nel[1] * ek);
                const int64_t eijk[3] = {ei, ej, ek};
                for (int a = 0; a < npe; ++a) {
                    int64_t nijk[3] = {0, 0, 0};
                    for (int d = 0; d < dim; ++d) nijk[d] = eijk[d] + (XI(a, d) > 0 ? 1 : 0);
                    const int64_t nid = nijk[0] + nn[0] * (nijk[1] + nn[1] * nijk[2]);
                    m->cells[e * npe + a] = (int32_t)nid;
                    if (done[nid]) continue;
                    done[nid] = 1;
                    for (int lb = 0; lb < nlb; ++lb) {
                        int l[3] = {lb % (p + 1), (lb / (p + 1)) % (p + 1), lb / ((p + 1) * (p + 1))};
                        real w = 1.0;
                        for (int d = 0; d < dim; ++d) w *= bspline_shape(p, l[d], XI(a, d));
                        if (std::abs(w) > 1e-12) {
                            int64_t bijk[3] = {0, 0, 0};
                            for (int d = 0; d < dim; ++d) bijk[d] = eijk[d] + l[d];
                            const int64_t bid = bijk[0] + nb[0] * (bijk[1] + (int64_t)nb[1] * bijk[2]);
                            rows[nid].push_back({(int32_t)bid, w});
                        }
                    }
                }
            }
    m->t_off.assign(num_nodes + 1, 0);
    for (int64_t n = 0; n < num_nodes; ++n) m->t_off[n + 1] = m->t_off[n] + (int64_t)rows[n].size();
    m->t_bases.resize(m->t_off[num_nodes]);
    m->t_w.resize(m->t_off[num_nodes]);
    for (int64_t n = 0; n < num_nodes; ++n)
        for (size_t k = 0; k < rows[n].size(); ++k) {
            m->t_bases[m->t_off[n] + k] = rows[n][k].first;
            m->t_w[m->t_off[n] + k] = rows[n][k].second;
        }
    return m;
}

void orc_mesh_sizes(const orc_mesh* m, int64_t* nn, int64_t* nc, int64_t* nb, int64_t* nnz) {
    const int npe = m->dim == 2 ? 4 : 8;
    *nn = (int64_t)m->coords.size() / m->dim;
    *nc = (int64_t)m->cells.size() / npe;
    *nb = m->num_bases;
    *nnz = (int64_t)m->t_bases.size();
}
void orc_mesh_arrays(const orc_mesh* m, double* coords, int32_t* cells, int64_t* t_off, int32_t* t_b,
                     double* t_w) {
    std::memcpy(coords, m->coords.data(), m->coords.size() * sizeof(real));
    std::memcpy(cells, m->cells.data(), m->cells.size() * sizeof(int32_t));
    std::memcpy(t_off, m->t_off.data(), m->t_off.size() * sizeof(int64_t));
    std::memcpy(t_b, m->t_bases.data(), m->t_bases.size() * sizeof(int32_t));
    std::memcpy(t_w, m->t_w.data(), m->t_w.size() * sizeof(real));
}
void orc_mesh_free(orc_mesh* m) { delete m; }

/* ------------------------------------------------------------------------ */
orc_model* orc_model_create(int dim, int ip_cell, int shape_kind, int64_t num_nodes, const double* coords,
                            int64_t num_cells, const int32_t* cells, int64_t num_bases, const int64_t* t_off,
                            const int32_t* t_b, const double* t_w) {
    auto* m = new orc_model;
    m->dim = dim;
    m->ip_cell = ip_cell;
    m->shape = shape_kind;
    m->num_nodes = num_nodes;
    m->num_cells = num_cells;
    m->num_bases = num_bases;
    const int npe = cell_nodes(ip_cell);
    m->coords.assign(coords, coords + num_nodes * dim);
    m->cells.assign(cells, cells + num_cells * npe);
    m->t_off.assign(t_off, t_off + num_nodes + 1);
    m->t_bases.assign(t_b, t_b + t_off[num_nodes]);
    m->t_w.assign(t_w, t_w + t_off[num_nodes]);
    return m;
}
void orc_model_free(orc_model* m) { delete m; }

int orc_model_add_bulk_set(orc_model* m, int ig_cell, int rule, int model, int64_t nc, const int32_t* ipc,
                           const int64_t* ig_off, const double* ig_coords, const double* ig_param,
                           const double* E, double nu) {
    if (rule < 0) rule = orc_auto_rule(0, ig_cell);
    if (m->finalized) return 1;
    BulkSet s;
    s.ig_cell = ig_cell;
    s.rule = rule;
    s.model = model;
    s.ip_cell.assign(ipc, ipc + nc);
    if (ig_off) {
        s.ig_off.assign(ig_off, ig_off + nc + 1);
        const int64_t nig = ig_off[nc];
        const int64_t per = (int64_t)cell_nodes(ig_cell) * m->dim;
        s.ig_coords.assign(ig_coords, ig_coords + nig * per);
        s.ig_param.assign(ig_param, ig_param + nig * per);
    }
    s.E.assign(E, E + nc);
    s.nu = nu;
    m->bulk.push_back(std::move(s));
    return 0;
}

int orc_model_set_density(orc_model* m, int set, const double* node_rho, double beta) {
    if (set < 0 || set >= (int)m->bulk.size()) return 1;
    m->bulk[set].node_rho.assign(node_rho, node_rho + m->num_nodes);
    m->bulk[set].beta = beta;
    return 0;
}

/* the Thickness property of a bulk set (IWG_Isotropic_Struc_Linear_Bulk,
   FEM/INT/src/IWG/cl_FEM_IWG_Isotropic_Struc_Linear_Bulk.cpp:84-85: w* is
   multiplied by it) */
int orc_model_set_bulk_thickness(orc_model* m, int set, double thickness) {
    if (set < 0 || set >= (int)m->bulk.size() || !(thickness > 0.0)) return 1;
    m->bulk[set].thickness = thickness;
    return 0;
}

/* Thickness and Select properties of the k-th side set: w* times the
   thickness (..._Neumann.cpp:66-67, ..._Dirichlet.cpp:103-104); the selection
   matrix M projects the Dirichlet terms (..._Dirichlet.cpp:66-81, 107-116),
   NULL = the identity */
int orc_model_set_side_options(orc_model* m, int side_set, double thickness, const double* select) {
    if (side_set < 0 || side_set >= (int)m->side.size() || !(thickness > 0.0)) return 1;
    SideSet& s = m->side[side_set];
    s.thickness = thickness;
    s.has_select = select != nullptr;
    for (int k = 0; k < 9; ++k) s.select[k] = 0.0;
    if (select)
        for (int i = 0; i < m->dim; ++i)
            for (int j = 0; j < m->dim; ++j) s.select[i * 3 + j] = select[i * m->dim + j];
    return 0;
}

int orc_model_add_side_set(orc_model* m, int iwg, int rule, int model, int64_t ns, const int32_t* ipc,
                           const int32_t* ord, const double* E, double nu, double alpha, const double* value) {
    if (rule < 0) rule = orc_auto_rule(1, m->dim == 2 ? ORC_CELL_LINE2 : ORC_CELL_QUAD4);
    if (m->finalized) return 1;
    SideSet s;
    s.iwg = iwg;
    s.rule = rule;
    s.model = model;
    s.ip_cell.assign(ipc, ipc + ns);
    s.ordinal.assign(ord, ord + ns);
    s.E.assign(E, E + ns);
    s.nu = nu;
    s.alpha = alpha;
    for (int d = 0; d < 3; ++d) s.value[d] = d < m->dim ? value[d] : 0.0;
    m->side.push_back(std::move(s));
    return 0;
}

int orc_model_add_double_side_set(orc_model* m, int iwg, int facet_cell, int rule, int model, int64_t nc,
                                  const int32_t* leader, const int32_t* follower, const int64_t* fc_off,
                                  const double* fc_x, const double* fc_xl, const double* fc_xf, const double* EL,
                                  const double* EF, double nu, double alpha) {
    if (rule < 0) rule = orc_auto_rule(2, facet_cell);
    if (m->finalized) return 1;
    DoubleSet s;
    s.iwg = iwg;
    s.facet_cell = facet_cell;
    s.rule = rule;
    s.model = model;
    s.leader.assign(leader, leader + nc);
    s.follower.assign(follower, follower + nc);
    s.fc_off.assign(fc_off, fc_off + nc + 1);
    const int64_t nv = fc_off[nc] * cell_nodes(facet_cell) * m->dim;
    s.fc_x.assign(fc_x, fc_x + nv);
    s.fc_xl.assign(fc_xl, fc_xl + nv);
    s.fc_xf.assign(fc_xf, fc_xf + nv);
    s.EL.assign(EL, EL + nc);
    s.EF.assign(EF, EF + nc);
    s.nu = nu;
    s.alpha = alpha;
    m->dbl.push_back(std::move(s));
    return 0;
}

/* geometry of one cut cluster / one double-sided cluster replaced (same
   number of integration cells / facets): the finite-difference perturbations
   of IG vertex coordinates of the reference's dR/dp (IWG::select_dRdp_FD_
   geometry_bulk, FEM/INT/src/IWG/cl_FEM_IWG.cpp:2997-3154) act on these.  */
int orc_model_update_ig(orc_model* m, int set, int64_t eq, const double* coords, const double* param) {
    if (set < 0 || set >= (int)m->bulk.size()) return 1;
    BulkSet& s = m->bulk[set];
    if (s.ig_off.empty() || eq < 0 || eq >= (int64_t)s.ip_cell.size()) return 1;
    const int64_t per = (int64_t)cell_nodes(s.ig_cell) * m->dim;
    const int64_t b = s.ig_off[eq] * per, n = (s.ig_off[eq + 1] - s.ig_off[eq]) * per;
    std::copy(coords, coords + n, s.ig_coords.begin() + b);
    std::copy(param, param + n, s.ig_param.begin() + b);
    return 0;
}
int orc_model_update_facets(orc_model* m, int set, int64_t eq, const double* coords, const double* lparam,
                            const double* fparam) {
    const int k = set - (int)m->bulk.size() - (int)m->side.size();
    if (k < 0 || k >= (int)m->dbl.size()) return 1;
    DoubleSet& s = m->dbl[k];
    if (eq < 0 || eq >= (int64_t)s.leader.size()) return 1;
    const int64_t per = (int64_t)cell_nodes(s.facet_cell) * m->dim;
    const int64_t b = s.fc_off[eq] * per, n = (s.fc_off[eq + 1] - s.fc_off[eq]) * per;
    std::copy(coords, coords + n, s.fc_x.begin() + b);
    std::copy(lparam, lparam + n, s.fc_xl.begin() + b);
    std::copy(fparam, fparam + n, s.fc_xf.begin() + b);
    return 0;
}

/* MSI: adof numbering by type then basis rank among used bases
   (Dof_Manager::create_adofs / set_owned_adofs_ids_by_type,
   FEM/MSI/src/cl_MSI_Dof_Manager.cpp:703-744, 820-985); element unique adof
   lists sorted per type (moris::unique, cl_MSI_Equation_Object.cpp:236,285);
   sparsity as the union of element adof lists per row
   (MSI_Solver_Interface::compute_sparsity_pattern,
   cl_MSI_Solver_Interface.cpp:309-588).                                      */
int orc_model_finalize(orc_model* m) {
    if (m->finalized) return 0;
    const int npe = cell_nodes(m->ip_cell);
    // used bases: referenced by any node of any IP cell that belongs to a set
    std::vector<char> cell_used(m->num_cells, 0);
    for (auto& s : m->bulk) for (auto c : s.ip_cell) cell_used[c] = 1;
    for (auto& s : m->side) for (auto c : s.ip_cell) cell_used[c] = 1;
    for (auto& s : m->dbl) {
        for (auto c : s.leader) cell_used[c] = 1;
        for (auto c : s.follower) cell_used[c] = 1;
    }
    std::vector<char> used(m->num_bases, 0);
    for (int64_t c = 0; c < m->num_cells; ++c) {
        if (!cell_used[c]) continue;
        for (int a = 0; a < npe; ++a) {
            const int32_t nd = m->cells[c * npe + a];
            for (int64_t k = m->t_off[nd]; k < m->t_off[nd + 1]; ++k) used[m->t_bases[k]] = 1;
        }
    }
    m->basis_rank.assign(m->num_bases, -1);
    m->num_used = 0;
    for (int64_t b = 0; b < m->num_bases; ++b)
        if (used[b]) m->basis_rank[b] = m->num_used++;
    m->cell_ubases.assign(m->num_cells, {});
    for (int64_t c = 0; c < m->num_cells; ++c) {
        if (!cell_used[c]) continue;
        std::vector<int32_t>& u = m->cell_ubases[c];
        for (int a = 0; a < npe; ++a) {
            const int32_t nd = m->cells[c * npe + a];
            for (int64_t k = m->t_off[nd]; k < m->t_off[nd + 1]; ++k)
                u.push_back((int32_t)m->basis_rank[m->t_bases[k]]);
        }
        std::sort(u.begin(), u.end());
        u.erase(std::unique(u.begin(), u.end()), u.end());
    }
    // sparsity: for every used basis the union of the basis lists of the
    // cells that contain it; row (type f, basis b) repeats it for every type
    const int64_t nu = m->num_used, nad = nu * m->dim;
    std::vector<std::vector<int64_t>> cells_of(nu);
    for (int64_t c = 0; c < m->num_cells; ++c)
        for (auto b : m->cell_ubases[c]) cells_of[b].push_back(c);
    std::vector<std::vector<int32_t>> uni(nu);
    for (int64_t b = 0; b < nu; ++b) {
        std::vector<int32_t>& u = uni[b];
        for (auto c : cells_of[b]) u.insert(u.end(), m->cell_ubases[c].begin(), m->cell_ubases[c].end());
    }
    // a double-sided equation object couples the leader's and the follower's bases
    for (auto& s : m->dbl)
        for (size_t i = 0; i < s.leader.size(); ++i) {
            const auto& L = m->cell_ubases[s.leader[i]];
            const auto& F = m->cell_ubases[s.follower[i]];
            for (auto b : L) uni[b].insert(uni[b].end(), F.begin(), F.end());
            for (auto b : F) uni[b].insert(uni[b].end(), L.begin(), L.end());
        }
    for (int64_t b = 0; b < nu; ++b) {
        std::vector<int32_t>& u = uni[b];
        std::sort(u.begin(), u.end());
        u.erase(std::unique(u.begin(), u.end()), u.end());
    }
    m->rowptr.assign(nad + 1, 0);
    for (int64_t r = 0; r < nad; ++r) m->rowptr[r + 1] = m->rowptr[r] + (int32_t)(m->dim * uni[r % nu].size());
    m->colidx.resize(m->rowptr[nad]);
    for (int64_t r = 0; r < nad; ++r) {
        int64_t k = m->rowptr[r];
        for (int g = 0; g < m->dim; ++g)
            for (auto cb : uni[r % nu]) m->colidx[k++] = (int32_t)(g * nu + cb);
    }
    m->finalized = true;
    return 0;
}

int64_t orc_model_num_adofs(const orc_model* m) { return m->num_used * m->dim; }
int64_t orc_model_nnz(const orc_model* m) { return m->rowptr.empty() ? 0 : m->rowptr.back(); }
int orc_model_num_sets(const orc_model* m) { return (int)(m->bulk.size() + m->side.size() + m->dbl.size()); }
int64_t orc_model_num_eq(const orc_model* m, int set) {
    if (set < (int)m->bulk.size()) return (int64_t)m->bulk[set].ip_cell.size();
    set -= (int)m->bulk.size();
    if (set < (int)m->side.size()) return (int64_t)m->side[set].ip_cell.size();
    set -= (int)m->side.size();
    if (set < (int)m->dbl.size()) return (int64_t)m->dbl[set].leader.size();
    return -1;
}
int orc_graph(const orc_model* m, int32_t* rowptr, int32_t* colidx) {
    if (!m->finalized) return 1;
    std::memcpy(rowptr, m->rowptr.data(), m->rowptr.size() * sizeof(int32_t));
    std::memcpy(colidx, m->colidx.data(), m->colidx.size() * sizeof(int32_t));
    return 0;
}

}  // extern "C"

/* ======================================================================== */
namespace {

int ip_cell_of(const orc_model* m, int set, int64_t eq) {
    if (set < (int)m->bulk.size()) return m->bulk[set].ip_cell[eq];
    set -= (int)m->bulk.size();
    if (set < (int)m->side.size()) return m->side[set].ip_cell[eq];
    return m->dbl[set - m->side.size()].leader[eq];
}
const DoubleSet* double_set(const orc_model* m, int set) {
    const int k = set - (int)m->bulk.size() - (int)m->side.size();
    return k >= 0 && k < (int)m->dbl.size() ? &m->dbl[k] : nullptr;
}

/* element adof ids: Equation_Object::get_equation_obj_dof_ids
   (cl_MSI_Equation_Object.cpp:506-554): types in requested order, each
   type's unique adofs ascending.                                            */
std::vector<int32_t> element_ids(const orc_model* m, int cell) {
    std::vector<int32_t> ids;
    for (int f = 0; f < m->dim; ++f)
        for (auto b : m->cell_ubases[cell]) ids.push_back((int32_t)(f * m->num_used + b));
    return ids;
}

/* element T per type: build_PADofMap (cl_MSI_Equation_Object.cpp:333-364):
   rows = element nodes, columns = sorted unique adofs; the full element T is
   block-diagonal over the dof types (build_PADofMap_1, :427-493).          */
Mat element_T(const orc_model* m, int cell) {
    const int npe = cell_nodes(m->ip_cell);
    const auto& u = m->cell_ubases[cell];
    std::map<int32_t, int> col;
    for (size_t k = 0; k < u.size(); ++k) col[u[k]] = (int)k;
    Mat T0(npe, (int)u.size(), 0.0);
    for (int a = 0; a < npe; ++a) {
        const int32_t nd = m->cells[(int64_t)cell * npe + a];
        for (int64_t k = m->t_off[nd]; k < m->t_off[nd + 1]; ++k)
            T0(a, col[(int32_t)m->basis_rank[m->t_bases[k]]]) = m->t_w[k];
    }
    const int d = m->dim;
    Mat T(d * npe, d * (int)u.size(), 0.0);
    for (int f = 0; f < d; ++f)
        for (int a = 0; a < npe; ++a)
            for (int j = 0; j < (int)u.size(); ++j) T(f * npe + a, f * (int)u.size() + j) = T0(a, j);
    return T;
}

Mat ip_coords(const orc_model* m, int cell) {
    const int npe = cell_nodes(m->ip_cell), d = m->dim;
    Mat X(npe, d);
    for (int a = 0; a < npe; ++a) {
        const int32_t nd = m->cells[(int64_t)cell * npe + a];
        for (int k = 0; k < d; ++k) X(a, k) = m->coords[(int64_t)nd * d + k];
    }
    return X;
}

/* Field interpolation at an IP-parametric point: N and dN/dx = J^-1 dN/dxi
   (Field_Interpolator::NBuild / dnNdxn(1), cl_FEM_Field_Interpolator.cpp:
   405, 464-495) with the IP-cell Jacobian (Space_Interpolator).             */
void ip_eval(const orc_model* m, const Mat& Xip, const real* xi_ip, Mat& Nrow, Mat& dNdx) {
    Mat dNdxi;
    shape(m->ip_cell, xi_ip, Nrow, dNdxi);
    Mat J = mul(dNdxi, Xip);
    Mat Ji = inverse_ip(J, m->shape == ORC_SHAPE_RECTANGULAR);
    dNdx = mul(Ji, dNdxi);
}

/* IWG_Isotropic_Struc_Linear_Bulk::compute_residual / compute_jacobian
   (FEM/INT/src/IWG/cl_FEM_IWG_Isotropic_Struc_Linear_Bulk.cpp:42-207):
   R += w B^T (D eps(u)),  K += w B^T (D B).                                 */
void iwg_bulk(const Mat& B, const Mat& D, const Mat& uvec, real w, Mat& K, Mat& R) {
    Mat eps = mul(B, uvec);
    Mat flux = mul(D, eps);
    Mat Bt = trans(B);
    add_scaled(R, w, mul(Bt, flux));
    add_scaled(K, w, mul(Bt, mul(D, B)));
}

/* Element_Bulk::compute_jacobian_and_residual (FEM/INT/src/ELEM/
   cl_FEM_Element_Bulk.cpp:258-355) over the IG cells of one cluster
   (Cluster::compute_jacobian_and_residual, cl_FEM_Cluster.cpp:444-459).
   IG->IP map: xi_IP = N_IG(xi_IG) * xihat_IG (Space_Interpolator::
   map_integration_point); weight w*detJ_IG; GPs with detJ < -1e-6 skipped
   (Geometry_Interpolator::sDetJInvJacLowerLimit, cl_FEM_Geometry_
   Interpolator.cpp:28).  The time slab [0,1] with BAR_1 (weight 2, time
   detJ 0.5) multiplies w*detJ by exactly 1.0.                                */
void bulk_pdof(const orc_model* m, const BulkSet& s, int64_t eq, const Mat& upd, Mat& K, Mat& R) {
    const int cell = s.ip_cell[eq];
    const int d = m->dim, npe = cell_nodes(m->ip_cell);
    const int nd = d * npe;
    K = Mat(nd, nd, 0.0);
    R = Mat(nd, 1, 0.0);
    Mat Xip = ip_coords(m, cell);
    RuleTab rt = make_rule(s.rule);
    Mat D = constitutive(s.model, d, s.E[eq], s.nu);
    Mat uvec(nd, 1);
    for (int f = 0; f < d; ++f)
        for (int a = 0; a < npe; ++a) uvec(f * npe + a, 0) = upd(a, f);
    const bool rect = m->shape == ORC_SHAPE_RECTANGULAR;
    int64_t g0 = 0, g1 = 1;
    if (!s.ig_off.empty()) { g0 = s.ig_off[eq]; g1 = s.ig_off[eq + 1]; }
    const int ign = cell_nodes(s.ig_cell);
    for (int64_t g = g0; g < g1; ++g) {
        Mat Xig, XIig;
        if (s.ig_off.empty()) {
            Xig = Xip;
            param_coords(m->ip_cell, XIig);
        } else {
            Xig = Mat(ign, d);
            XIig = Mat(ign, d);
            for (int a = 0; a < ign; ++a)
                for (int k = 0; k < d; ++k) {
                    Xig(a, k) = s.ig_coords[(g * ign + a) * d + k];
                    XIig(a, k) = s.ig_param[(g * ign + a) * d + k];
                }
        }
        const bool ig_rect = rect && s.ig_cell == m->ip_cell;
        for (int q = 0; q < rt.n; ++q) {
            const real* xig = &rt.pts[(size_t)q * rt.dim];
            Mat Nig, dNig;
            shape(s.ig_cell, xig, Nig, dNig);
            Mat Jig = mul(dNig, Xig);
            const real detJ = det_bulk(Jig, s.ig_cell, ig_rect);
            if (detJ < -1.0e-6) continue;
            const real wstar = rt.w[q] * detJ * s.thickness;
            Mat xip = mul(Nig, XIig);  // 1 x d
            Mat Nrow, dNdx;
            ip_eval(m, Xip, xip.a.data(), Nrow, dNdx);
            Mat B = test_strain(s.model, dNdx);
            if (!s.node_rho.empty()) {
                // density-dependent Young's modulus E0 rho(x)^beta, rho from the
                // density field interpolator (EXA/optimization/SIMP/SIMP.cpp:43-51)
                real rho = 0.0;
                for (int a = 0; a < npe; ++a) rho += Nrow(0, a) * s.node_rho[m->cells[(int64_t)cell * npe + a]];
                Mat Dq = constitutive(s.model, d, s.E[eq] * std::pow(rho, s.beta), s.nu);
                iwg_bulk(B, Dq, uvec, wstar, K, R);
            } else {
                iwg_bulk(B, D, uvec, wstar, K, R);
            }
        }
    }
}

/* Element_Sideset::compute_jacobian_and_residual (FEM/INT/src/ELEM/
   cl_FEM_Element_Sideset.cpp:261-330) on trivial side clusters: the side GI
   interpolates the facet vertices (physical coords and IP-param coords); the
   side detJ is |J| for lines and |t1 x t2| for quads (cl_MTK_Space_
   Interpolator.cpp:782, 841); the normal is (t_y, -t_x)/|t| for lines and
   t1 x t2 / |.| for quads (:1298-1344).
   Neumann: R -= w N^T t  (cl_FEM_IWG_Isotropic_Struc_Linear_Neumann.cpp:38).
   Dirichlet Nitsche (…_Dirichlet.cpp:52-240, beta = -1 symmetric / +1
   unsymmetric per IWG_Factory cl_FEM_IWG_Factory.cpp:196-200):
     R += w ( -N^T t(u) + beta (nD B)^T (u-g) + gamma N^T (u-g) )
     K += w ( beta (nD B)^T N + gamma N^T N - N^T (nD B) ),
   gamma = alpha E / h, h = facet length measure (SP_Dirichlet_Nitsche::
   eval_SP, cl_FEM_SP_Dirichlet_Nitsche.cpp:75-116; Cluster::compute_cluster_
   cell_length_measure, cl_FEM_Cluster.cpp:858-920).                          */
void side_pdof(const orc_model* m, const SideSet& s, int64_t eq, const Mat& upd, Mat& K, Mat& R) {
    const int cell = s.ip_cell[eq], ord = s.ordinal[eq];
    const int d = m->dim, npe = cell_nodes(m->ip_cell);
    const int nd = d * npe;
    K = Mat(nd, nd, 0.0);
    R = Mat(nd, 1, 0.0);
    Mat Xip = ip_coords(m, cell), XI;
    param_coords(m->ip_cell, XI);
    const int fcell = d == 2 ? ORC_CELL_LINE2 : ORC_CELL_QUAD4;
    const int nfv = d == 2 ? 2 : 4;
    Mat Xs(nfv, d), XIs(nfv, d);
    for (int a = 0; a < nfv; ++a) {
        const int v = d == 2 ? QUAD4_SIDES[ord][a] : HEX8_SIDES[ord][a];
        for (int k = 0; k < d; ++k) {
            Xs(a, k) = Xip(v, k);
            XIs(a, k) = XI(v, k);
        }
    }
    RuleTab rt = make_rule(s.rule);
    Mat D = constitutive(s.model, d, s.E[eq], s.nu);
    const int nstress = D.r;
    Mat uvec(nd, 1);
    for (int f = 0; f < d; ++f)
        for (int a = 0; a < npe; ++a) uvec(f * npe + a, 0) = upd(a, f);
    // facet measure (length in 2D, area in 3D) for the element size
    real hmeas = 0.0;
    for (int q = 0; q < rt.n; ++q) {
        Mat Ns, dNs;
        shape(fcell, &rt.pts[(size_t)q * rt.dim], Ns, dNs);
        Mat Jt = mul(dNs, Xs);
        real dj;
        if (d == 2) dj = std::sqrt(Jt(0, 0) * Jt(0, 0) + Jt(0, 1) * Jt(0, 1));
        else {
            const real c0 = Jt(0, 1) * Jt(1, 2) - Jt(0, 2) * Jt(1, 1);
            const real c1 = Jt(0, 2) * Jt(1, 0) - Jt(0, 0) * Jt(1, 2);
            const real c2 = Jt(0, 0) * Jt(1, 1) - Jt(0, 1) * Jt(1, 0);
            dj = std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
        }
        hmeas += rt.w[q] * dj;
    }
    // side length measure: dim-1 == 1 -> the measure itself; == 2 -> sqrt(4A/pi)
    const real h = (d == 2) ? hmeas : std::pow(4.0 * hmeas / M_PI, 1.0 / 2.0);
    const real gamma = s.alpha * s.E[eq] / h;
    const real beta = s.iwg == ORC_IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE ? -1.0 : 1.0;
    for (int q = 0; q < rt.n; ++q) {
        Mat Ns, dNs;
        shape(fcell, &rt.pts[(size_t)q * rt.dim], Ns, dNs);
        Mat Jt = mul(dNs, Xs);  // (d-1) x d, rows = tangents
        real detJ, nrm[3] = {0.0, 0.0, 0.0};
        if (d == 2) {
            detJ = std::sqrt(Jt(0, 0) * Jt(0, 0) + Jt(0, 1) * Jt(0, 1));
            nrm[0] = Jt(0, 1) / detJ;
            nrm[1] = -Jt(0, 0) / detJ;
        } else {
            const real c0 = Jt(0, 1) * Jt(1, 2) - Jt(0, 2) * Jt(1, 1);
            const real c1 = Jt(0, 2) * Jt(1, 0) - Jt(0, 0) * Jt(1, 2);
            const real c2 = Jt(0, 0) * Jt(1, 1) - Jt(0, 1) * Jt(1, 0);
            detJ = std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
            nrm[0] = c0 / detJ;
            nrm[1] = c1 / detJ;
            nrm[2] = c2 / detJ;
        }
        if (detJ < -1.0e-6) continue;
        const real wstar = rt.w[q] * detJ * s.thickness;
        Mat xip = mul(Ns, XIs);
        Mat Nrow, dNdx;
        ip_eval(m, Xip, xip.a.data(), Nrow, dNdx);
        Mat N = field_N(Nrow, d);
        Mat Nt = trans(N);
        if (s.iwg == ORC_IWG_STRUC_LINEAR_NEUMANN) {
            Mat t(d, 1);
            for (int k = 0; k < d; ++k) t(k, 0) = s.value[k];
            add_scaled(R, -wstar, mul(Nt, t));
            continue;
        }
        // selection matrix M (identity without a Select property)
        Mat M(d, d, 0.0);
        real mnorm = 0.0;
        for (int i = 0; i < d; ++i)
            for (int j = 0; j < d; ++j) {
                M(i, j) = s.has_select ? s.select[i * 3 + j] : (i == j ? 1.0 : 0.0);
                mnorm += M(i, j) * M(i, j);
            }
        if (std::sqrt(mnorm) < 1e-16) continue;  // a zero projection adds nothing
        Mat B = test_strain(s.model, dNdx);
        Mat Fn = flat_normal(nrm, d, nstress);
        Mat nDB = mul(Fn, mul(D, B));  // d x nd (testTraction == dTractiondDOF)
        Mat trac = mul(nDB, uvec);     // traction(n) = Fn * flux
        Mat jump = mul(N, uvec);
        for (int k = 0; k < d; ++k) jump(k, 0) -= s.value[k];
        Mat nDBt = trans(nDB);
        Mat Mjump = mul(M, jump);
        Mat r = mul(Nt, mul(M, trac));
        for (auto& v : r.a) v = -v;
        add_scaled(r, beta, mul(nDBt, Mjump));
        add_scaled(r, gamma, mul(Nt, Mjump));
        add_scaled(R, wstar, r);
        Mat MN = mul(M, N);
        Mat k = mul(nDBt, MN);
        for (auto& v : k.a) v *= beta;
        add_scaled(k, gamma, mul(Nt, MN));
        add_scaled(k, -1.0, mul(Nt, mul(M, nDB)));
        add_scaled(K, wstar, k);
    }
    (void)nstress;
}

/* measure of the cell cluster on an IP cell: the bulk clusters there, their
   integration cells' measures (xtk::Side_Cluster::compute_cluster_cell_measure
   -> associated cell cluster, XTK/src/cl_XTK_Side_Cluster.cpp:184-202; tet
   measure |det| / 6; an uncut cell's own measure sum_q w detJ).              */
real cell_cluster_volume(const orc_model* m, int cell) {
    real v = 0.0;
    for (const BulkSet& s : m->bulk)
        for (size_t i = 0; i < s.ip_cell.size(); ++i) {
            if (s.ip_cell[i] != cell) continue;
            if (s.ig_off.empty()) {
                Mat X = ip_coords(m, cell);
                RuleTab rt = make_rule(m->dim == 2 ? ORC_RULE_QUAD_2x2 : ORC_RULE_HEX_2x2x2);
                for (int q = 0; q < rt.n; ++q) {
                    Mat Nq, dNq;
                    shape(m->ip_cell, &rt.pts[(size_t)q * rt.dim], Nq, dNq);
                    Mat J = mul(dNq, X);
                    v += rt.w[q] * det_bulk(J, m->ip_cell, false);
                }
                continue;
            }
            const int ign = cell_nodes(s.ig_cell), d = m->dim;
            for (int64_t g = s.ig_off[i]; g < s.ig_off[i + 1]; ++g) {
                Mat Xg(ign, d);
                for (int a = 0; a < ign; ++a)
                    for (int k = 0; k < d; ++k) Xg(a, k) = s.ig_coords[(g * ign + a) * d + k];
                Mat XI;
                param_coords(s.ig_cell, XI);
                Mat Nq, dNq;
                shape(s.ig_cell, &XI.a[0], Nq, dNq);
                v += std::abs(det_bulk(mul(dNq, Xg), s.ig_cell, false));
            }
        }
    return v;
}

/* facet point of a double-sided cluster: side detJ (TRI3 |t1 x t2| / 2,
   QUAD4 |t1 x t2|, cl_MTK_Space_Interpolator.cpp:808-850) and the normal
   t1 x t2 / |.| (eval_normal_side_tri / _quad, :1349).                       */
void facet_point(const DoubleSet& s, int64_t f, const real* xq, real& detJ, real* n, Mat& Nf) {
    Mat dNf;
    shape(s.facet_cell, xq, Nf, dNf);
    const int nfv = cell_nodes(s.facet_cell);
    Mat X(nfv, 3);
    for (int a = 0; a < nfv; ++a)
        for (int k = 0; k < 3; ++k) X(a, k) = s.fc_x[(f * nfv + a) * 3 + k];
    Mat Jt = mul(dNf, X);
    const real c0 = Jt(0, 1) * Jt(1, 2) - Jt(0, 2) * Jt(1, 1);
    const real c1 = Jt(0, 2) * Jt(1, 0) - Jt(0, 0) * Jt(1, 2);
    const real c2 = Jt(0, 0) * Jt(1, 1) - Jt(0, 1) * Jt(1, 0);
    const real nn = std::sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    detJ = s.facet_cell == ORC_CELL_TRI3 ? nn / 2.0 : nn;
    // degenerate facet: zero measure, no normal (contributes nothing)
    const real inv = nn > 0.0 ? 1.0 / nn : 0.0;
    n[0] = c0 * inv;
    n[1] = c1 * inv;
    n[2] = c2 * inv;
}

/* flat normal of order 2 of the virtual-work ghost, 3D
   (IWG_Isotropic_Struc_Linear_Virtual_Work_Ghost::get_flat_normal_matrix,
   ..._Virtual_Work_Ghost.cpp:262-409) */
Mat ghost_flat_normal_3d(const real* n) {
    Mat F(3, 6, 0.0);
    F(0, 0) = n[0];
    F(1, 1) = n[1];
    F(2, 2) = n[2];
    F(1, 3) = n[2];
    F(2, 3) = n[1];
    F(0, 4) = n[2];
    F(2, 4) = n[0];
    F(0, 5) = n[1];
    F(1, 5) = n[0];
    return F;
}

/* Element_Double_Sideset::compute_jacobian_and_residual (FEM/INT/src/ELEM/
   cl_FEM_Element_Double_Sideset.cpp:283-347) over the facets of one
   double-sided cluster: leader / follower points from the facet's
   parametric vertices (get_follower_integration_point, :113), the leader
   normal, w* = w detJ, then
   - IWG_Isotropic_Struc_Linear_Interface::compute_residual / compute_jacobian
     (FEM/INT/src/IWG/cl_FEM_IWG_Isotropic_Struc_Linear_Interface.cpp:51-386)
     with SP_Nitsche_Interface::eval_SP (SP/cl_FEM_SP_Nitsche_Interface.cpp:
     51-97): gamma = 2 alpha |G| / (V_L/E_L + V_F/E_F), w_L, w_F the
     weights; beta = -1 symmetric / +1 unsymmetric (IWG_Factory, cl_FEM_IWG_
     Factory.cpp:202-206); linear CM, so dTestTraction = 0 and the SP has no
     dof dependency;
   - IWG_Isotropic_Struc_Linear_Virtual_Work_Ghost (..._Virtual_Work_Ghost.cpp:
     50-244) with SP_Ghost_Virtual_Work::eval_SP (SP/cl_FEM_SP_Ghost_Virtual_
     Work.cpp:30-38): gamma = alpha h^(2(p-1)+1), p = 1, h the side length
     measure sqrt(4 A / pi) (Cluster::compute_cluster_cell_length_measure,
     FEM/INT/src/ELEM/cl_FEM_Cluster.cpp:858-920);
   - IWG_Ghost_Normal_Field (FEM/INT/src/IWG/cl_FEM_IWG_Ghost_Normal_Field.cpp:
     36-233) with SP_Ghost_Displacement::eval_SP (SP/cl_FEM_SP_Ghost_
     Displacement.cpp:51-63): the penalty on the jump of the normal
     derivative of every displacement component, order 1 (linear IP cells):
       R_L += w gamma (dN_L/dn)_f [[du_f/dn]],  R_F -= w gamma (dN_F/dn)_f [[du_f/dn]],
       K_ST = +-w gamma (dN_S/dn) (dN_T/dn)^T per component (+ for S = T),
     gamma = alpha h^(2(1 - 1) + 1) E_L, E_L the leader's Material property,
     h the same side length measure.
   Output K (48 x 48) and R (48) in [leader pdofs | follower pdofs], each
   type-major.                                                                */
void double_pdof(const orc_model* m, const DoubleSet& s, int64_t eq, const Mat& updL, const Mat& updF, Mat& K,
                 Mat& R) {
    const int d = m->dim, npe = cell_nodes(m->ip_cell), nd = d * npe;
    K = Mat(2 * nd, 2 * nd, 0.0);
    R = Mat(2 * nd, 1, 0.0);
    const int cl = s.leader[eq], cf = s.follower[eq];
    Mat XL = ip_coords(m, cl), XF = ip_coords(m, cf);
    Mat DL = constitutive(s.model, d, s.EL[eq], s.nu), DF = constitutive(s.model, d, s.EF[eq], s.nu);
    Mat uL(nd, 1), uF(nd, 1);
    for (int f = 0; f < d; ++f)
        for (int a = 0; a < npe; ++a) {
            uL(f * npe + a, 0) = updL(a, f);
            uF(f * npe + a, 0) = updF(a, f);
        }
    RuleTab rt = make_rule(s.rule);
    const int nfv = cell_nodes(s.facet_cell);
    // cluster measures
    real area = 0.0;
    for (int64_t f = s.fc_off[eq]; f < s.fc_off[eq + 1]; ++f)
        for (int q = 0; q < rt.n; ++q) {
            real dj, n[3];
            Mat Nf;
            facet_point(s, f, &rt.pts[(size_t)q * rt.dim], dj, n, Nf);
            area += rt.w[q] * dj;
        }
    const bool normal_field = s.iwg == ORC_IWG_GHOST_NORMAL_FIELD;
    const bool ghost = s.iwg == ORC_IWG_STRUC_LINEAR_VW_GHOST || normal_field;
    real gamma, wl = 0.0, wf = 0.0;
    if (ghost) {
        const real h = std::pow(4.0 * area / M_PI, 1.0 / 2.0);
        gamma = s.alpha * std::pow(h, 2.0 * (1.0 - 1.0) + 1.0);
        if (normal_field) gamma *= s.EL[eq];
    } else {
        const real VL = cell_cluster_volume(m, cl), VF = cell_cluster_volume(m, cf);
        const real deno = VL / s.EL[eq] + VF / s.EF[eq];
        gamma = 2.0 * s.alpha * area / deno;
        wl = (VL / s.EL[eq]) / deno;
        wf = (VF / s.EF[eq]) / deno;
    }
    const real beta = s.iwg == ORC_IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE ? -1.0 : 1.0;
    Mat KLL(nd, nd, 0.0), KLF(nd, nd, 0.0), KFL(nd, nd, 0.0), KFF(nd, nd, 0.0), RL(nd, 1, 0.0), RF(nd, 1, 0.0);
    for (int64_t f = s.fc_off[eq]; f < s.fc_off[eq + 1]; ++f)
        for (int q = 0; q < rt.n; ++q) {
            real detJ, n[3];
            Mat Nf;
            facet_point(s, f, &rt.pts[(size_t)q * rt.dim], detJ, n, Nf);
            if (detJ < -1.0e-6) continue;
            const real w = rt.w[q] * detJ;
            Mat XIL(nfv, d), XIF(nfv, d);
            for (int a = 0; a < nfv; ++a)
                for (int k = 0; k < d; ++k) {
                    XIL(a, k) = s.fc_xl[(f * nfv + a) * d + k];
                    XIF(a, k) = s.fc_xf[(f * nfv + a) * d + k];
                }
            Mat xiL = mul(Nf, XIL), xiF = mul(Nf, XIF);
            Mat NrL, dL, NrF, dF;
            ip_eval(m, XL, xiL.a.data(), NrL, dL);
            ip_eval(m, XF, xiF.a.data(), NrF, dF);
            Mat BL = test_strain(s.model, dL), BF = test_strain(s.model, dF);
            Mat NL = field_N(NrL, d), NF = field_N(NrF, d);
            Mat Fn = flat_normal(n, d, 6);
            Mat tL = mul(Fn, mul(DL, BL)), tF = mul(Fn, mul(DF, BF));  // traction operators
            Mat tLt = trans(tL), tFt = trans(tF), NLt = trans(NL), NFt = trans(NF);
            if (normal_field) {
                // block-diagonal normal derivatives of the two sides
                Mat gL(nd, d, 0.0), gF(nd, d, 0.0);
                for (int fld = 0; fld < d; ++fld)
                    for (int a = 0; a < npe; ++a) {
                        real vl = 0.0, vf = 0.0;
                        for (int k = 0; k < d; ++k) {
                            vl += n[k] * dL(k, a);
                            vf += n[k] * dF(k, a);
                        }
                        gL(fld * npe + a, fld) = vl;
                        gF(fld * npe + a, fld) = vf;
                    }
                Mat jump = mul(trans(gL), uL);
                add_scaled(jump, -1.0, mul(trans(gF), uF));
                Mat gLt = trans(gL), gFt = trans(gF);
                add_scaled(RL, w * gamma, mul(gL, jump));
                add_scaled(RF, -w * gamma, mul(gF, jump));
                add_scaled(KLL, w * gamma, mul(gL, gLt));
                add_scaled(KFL, -w * gamma, mul(gF, gLt));
                add_scaled(KLF, -w * gamma, mul(gL, gFt));
                add_scaled(KFF, w * gamma, mul(gF, gFt));
                continue;
            }
            if (ghost) {
                Mat FnM = ghost_flat_normal_3d(n);
                Mat gL = trans(mul(FnM, BL)), gF = trans(mul(FnM, BF));  // B^T FnM^T
                Mat jump = mul(tL, uL);
                add_scaled(jump, -1.0, mul(tF, uF));
                add_scaled(RL, w * gamma, mul(gL, jump));
                add_scaled(RF, -w * gamma, mul(gF, jump));
                add_scaled(KLL, w * gamma, mul(gL, tL));
                add_scaled(KFL, -w * gamma, mul(gF, tL));
                add_scaled(KLF, -w * gamma, mul(gL, tF));
                add_scaled(KFF, w * gamma, mul(gF, tF));
                continue;
            }
            Mat trac = mul(tL, uL);
            for (auto& v : trac.a) v *= wl;
            add_scaled(trac, wf, mul(tF, uF));
            Mat jump = mul(NL, uL);
            add_scaled(jump, -1.0, mul(NF, uF));
            add_scaled(RL, -w, mul(NLt, trac));
            add_scaled(RL, w * beta * wl, mul(tLt, jump));
            add_scaled(RL, w * gamma, mul(NLt, jump));
            add_scaled(RF, w, mul(NFt, trac));
            add_scaled(RF, w * beta * wf, mul(tFt, jump));
            add_scaled(RF, -w * gamma, mul(NFt, jump));
            add_scaled(KLL, w * beta * wl, mul(tLt, NL));
            add_scaled(KLL, w * gamma, mul(NLt, NL));
            add_scaled(KLL, -w * wl, mul(NLt, tL));
            add_scaled(KFL, w * beta * wf, mul(tFt, NL));
            add_scaled(KFL, -w * gamma, mul(NFt, NL));
            add_scaled(KFL, w * wl, mul(NFt, tL));
            add_scaled(KLF, -w * beta * wl, mul(tLt, NF));
            add_scaled(KLF, -w * gamma, mul(NLt, NF));
            add_scaled(KLF, -w * wf, mul(NLt, tF));
            add_scaled(KFF, -w * beta * wf, mul(tFt, NF));
            add_scaled(KFF, w * gamma, mul(NFt, NF));
            add_scaled(KFF, w * wf, mul(NFt, tF));
        }
    for (int r = 0; r < nd; ++r) {
        R(r, 0) = RL(r, 0);
        R(nd + r, 0) = RF(r, 0);
        for (int c = 0; c < nd; ++c) {
            K(r, c) = KLL(r, c);
            K(r, nd + c) = KLF(r, c);
            K(nd + r, c) = KFL(r, c);
            K(nd + r, nd + c) = KFF(r, c);
        }
    }
}

/* element adof ids of any equation object (double-sided: leader's per-type
   lists then the follower's, get_equation_obj_dof_ids over two pdof systems) */
std::vector<int32_t> eq_ids(const orc_model* m, int set, int64_t eq) {
    const DoubleSet* ds = double_set(m, set);
    if (!ds) return element_ids(m, ip_cell_of(m, set, eq));
    std::vector<int32_t> a = element_ids(m, ds->leader[eq]), b = element_ids(m, ds->follower[eq]);
    a.insert(a.end(), b.begin(), b.end());
    return a;
}

/* Equation_Object::get_egn_obj_jacobian_and_residual (FEM/MSI/src/
   cl_MSI_Equation_Object.cpp:789-842): u_pdof = T u_adof (compute_my_pdof_
   values :1101-1131), K_a = T^T K T, R_a = T^T R.                            */
void element_adof(const orc_model* m, int set, int64_t eq, const double* u_adof, Mat& Ka, Mat& Ra) {
    if (const DoubleSet* ds = double_set(m, set)) {
        const int d = m->dim, npe = cell_nodes(m->ip_cell);
        Mat TL = element_T(m, ds->leader[eq]), TF = element_T(m, ds->follower[eq]);
        Mat T(TL.r + TF.r, TL.c + TF.c, 0.0);
        for (int r = 0; r < TL.r; ++r)
            for (int c = 0; c < TL.c; ++c) T(r, c) = TL(r, c);
        for (int r = 0; r < TF.r; ++r)
            for (int c = 0; c < TF.c; ++c) T(TL.r + r, TL.c + c) = TF(r, c);
        std::vector<int32_t> ids = eq_ids(m, set, eq);
        Mat ua((int)ids.size(), 1);
        for (size_t k = 0; k < ids.size(); ++k) ua(k, 0) = u_adof ? u_adof[ids[k]] : 0.0;
        Mat up = mul(T, ua);
        Mat updL(npe, d), updF(npe, d);
        for (int f = 0; f < d; ++f)
            for (int a = 0; a < npe; ++a) {
                updL(a, f) = up(f * npe + a, 0);
                updF(a, f) = up(d * npe + f * npe + a, 0);
            }
        Mat K, R;
        double_pdof(m, *ds, eq, updL, updF, K, R);
        Mat Tt = trans(T);
        Ka = mul(Tt, mul(K, T));
        Ra = mul(Tt, R);
        return;
    }
    const int cell = ip_cell_of(m, set, eq);
    const int d = m->dim, npe = cell_nodes(m->ip_cell);
    Mat T = element_T(m, cell);
    std::vector<int32_t> ids = element_ids(m, cell);
    Mat ua((int)ids.size(), 1);
    for (size_t k = 0; k < ids.size(); ++k) ua(k, 0) = u_adof ? u_adof[ids[k]] : 0.0;
    Mat up = mul(T, ua);  // (d*npe) x 1, type-major
    Mat upd(npe, d);
    for (int f = 0; f < d; ++f)
        for (int a = 0; a < npe; ++a) upd(a, f) = up(f * npe + a, 0);
    Mat K, R;
    if (set < (int)m->bulk.size()) bulk_pdof(m, m->bulk[set], eq, upd, K, R);
    else side_pdof(m, m->side[set - m->bulk.size()], eq, upd, K, R);
    Mat Tt = trans(T);
    Ka = mul(Tt, mul(K, T));
    Ra = mul(Tt, R);
}

}  // namespace

extern "C" {

int orc_element_topology(const orc_model* m, int set, int64_t eq, int32_t* ids, int32_t* n) {
    if (!m->finalized || set < 0 || set >= orc_model_num_sets(m)) return 1;
    if (eq < 0 || eq >= orc_model_num_eq(m, set)) return 1;
    std::vector<int32_t> v = eq_ids(m, set, eq);
    std::copy(v.begin(), v.end(), ids);
    *n = (int32_t)v.size();
    return 0;
}

int orc_element_matrices(const orc_model* m, int set, int64_t eq, const double* u_adof, double* K, double* R) {
    if (!m->finalized || set < 0 || set >= orc_model_num_sets(m)) return 1;
    if (eq < 0 || eq >= orc_model_num_eq(m, set)) return 1;
    Mat Ka, Ra;
    element_adof(m, set, eq, u_adof, Ka, Ra);
    std::memcpy(K, Ka.a.data(), Ka.a.size() * sizeof(real));
    std::memcpy(R, Ra.a.data(), Ra.a.size() * sizeof(real));
    return 0;
}

/* stress of a bulk equation object at an IP-parametric point:
   CM_Struc_Linear::flux = D eps(u) (FEM/INT/src/CM/cl_FEM_CM_Struc_Linear.cpp:
   280-302) with u_pdof = T u_adof; Voigt order of the model (3D: xx yy zz yz
   xz xy; plane strain: xx yy zz xy; plane stress: xx yy xy) */
int orc_element_flux(const orc_model* m, int set, int64_t eq, const double* xi, const double* u_adof,
                     double* flux, int32_t* ncomp) {
    if (!m->finalized || set < 0 || set >= (int)m->bulk.size()) return 1;
    const BulkSet& s = m->bulk[set];
    if (eq < 0 || eq >= (int64_t)s.ip_cell.size()) return 1;
    const int cell = s.ip_cell[eq];
    const int d = m->dim, npe = cell_nodes(m->ip_cell);
    Mat T = element_T(m, cell);
    std::vector<int32_t> ids = element_ids(m, cell);
    Mat ua((int)ids.size(), 1);
    for (size_t k = 0; k < ids.size(); ++k) ua(k, 0) = u_adof[ids[k]];
    Mat up = mul(T, ua);
    Mat Nrow, dNdx;
    ip_eval(m, ip_coords(m, cell), xi, Nrow, dNdx);
    real E = s.E[eq];
    if (!s.node_rho.empty()) {
        real rho = 0.0;
        for (int a = 0; a < npe; ++a) rho += Nrow(0, a) * s.node_rho[m->cells[(int64_t)cell * npe + a]];
        E *= std::pow(rho, s.beta);
    }
    Mat D = constitutive(s.model, d, E, s.nu);
    Mat sig = mul(D, mul(test_strain(s.model, dNdx), up));
    for (int i = 0; i < sig.r; ++i) flux[i] = sig(i, 0);
    *ncomp = sig.r;
    return 0;
}

int orc_element_pdof_matrices(const orc_model* m, int set, int64_t eq, const double* u_pdof, double* K,
                              double* R, int32_t* npdof) {
    if (set < 0 || set >= orc_model_num_sets(m) || double_set(m, set)) return 1;
    const int d = m->dim, npe = cell_nodes(m->ip_cell);
    Mat upd(npe, d);
    for (int f = 0; f < d; ++f)
        for (int a = 0; a < npe; ++a) upd(a, f) = u_pdof ? u_pdof[f * npe + a] : 0.0;
    Mat Kp, Rp;
    if (set < (int)m->bulk.size()) bulk_pdof(m, m->bulk[set], eq, upd, Kp, Rp);
    else side_pdof(m, m->side[set - m->bulk.size()], eq, upd, Kp, Rp);
    std::memcpy(K, Kp.a.data(), Kp.a.size() * sizeof(real));
    std::memcpy(R, Rp.a.data(), Rp.a.size() * sizeof(real));
    *npdof = d * npe;
    return 0;
}

/* Solver_Interface::fill_matrix_and_RHS (SOL/DLA/src/cl_DLA_Solver_
   Interface.cpp:317-379): set loop, equation-object loop, scatter of the
   column-major K_a through Sparse_Matrix_EpetraFECrs::fill_matrix
   (SOL/SOL_CORE/src/cl_Sparse_Matrix_EpetraFECrs.cpp:103-131, sum-into by
   global ids) and R_a through Vector_Epetra::sum_into_global_values.  The
   restatement partitions equation objects over std::threads and sums into
   the shared CSR with atomic adds.                                           */
int orc_assemble(const orc_model* m, const double* u_adof, double* vals, double* rhs, int nthreads,
                 int64_t eq_stride, int zero_first) {
    if (!m->finalized) return 1;
    if (nthreads < 1) nthreads = 1;
    if (eq_stride < 1) eq_stride = 1;
    const int64_t nnz = orc_model_nnz(m), nad = orc_model_num_adofs(m);
    if (zero_first) {
        std::memset(vals, 0, sizeof(real) * nnz);
        std::memset(rhs, 0, sizeof(real) * nad);
    }
    struct Item { int set; int64_t eq; };
    std::vector<Item> items;
    for (int s = 0; s < orc_model_num_sets(m); ++s)
        for (int64_t e = 0; e < orc_model_num_eq(m, s); e += eq_stride) items.push_back({s, e});
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            const int64_t i = next.fetch_add(1);
            if (i >= (int64_t)items.size()) break;
            Mat Ka, Ra;
            element_adof(m, items[i].set, items[i].eq, u_adof, Ka, Ra);
            std::vector<int32_t> ids = eq_ids(m, items[i].set, items[i].eq);
            const int n = (int)ids.size();
            for (int c = 0; c < n; ++c) {
                for (int r = 0; r < n; ++r) {
                    const int32_t row = ids[r], col = ids[c];
                    const int32_t* b = m->colidx.data() + m->rowptr[row];
                    const int32_t* e = m->colidx.data() + m->rowptr[row + 1];
                    const int64_t pos = std::lower_bound(b, e, col) - m->colidx.data();
                    std::atomic_ref<real>(vals[pos]).fetch_add(Ka(r, c), std::memory_order_relaxed);
                }
            }
            for (int r = 0; r < n; ++r)
                std::atomic_ref<real>(rhs[ids[r]]).fetch_add(Ra(r, 0), std::memory_order_relaxed);
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
    return 0;
}

/* plain (Jacobi-)preconditioned conjugate gradients; the reference delegates
   this to Trilinos AztecOO (AZ_cg + AZ_Jacobi, PRM/src/fn_PRM_SOL_
   Parameters.hpp:453-518), restated here as the textbook algorithm.        */
int orc_pcg(int64_t n, const int32_t* rp, const int32_t* ci, const double* v, const double* b, double* x,
            double rtol, int max_iter, int jacobi, int* iters, double* rel_res) {
    std::vector<real> r(n), z(n), p(n), q(n), dinv(n, 1.0);
    if (jacobi)
        for (int64_t i = 0; i < n; ++i)
            for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
                if (ci[k] == i) dinv[i] = 1.0 / v[k];
    auto spmv = [&](const real* in, real* out) {
        for (int64_t i = 0; i < n; ++i) {
            real s = 0.0;
            for (int32_t k = rp[i]; k < rp[i + 1]; ++k) s += v[k] * in[ci[k]];
            out[i] = s;
        }
    };
    spmv(x, q.data());
    real bn = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        r[i] = b[i] - q[i];
        bn += b[i] * b[i];
    }
    bn = std::sqrt(bn);
    if (bn == 0.0) bn = 1.0;
    real rz = 0.0, rn = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        z[i] = dinv[i] * r[i];
        p[i] = z[i];
        rz += r[i] * z[i];
        rn += r[i] * r[i];
    }
    int it = 0;
    while (std::sqrt(rn) / bn > rtol && it < max_iter) {
        spmv(p.data(), q.data());
        real pq = 0.0;
        for (int64_t i = 0; i < n; ++i) pq += p[i] * q[i];
        const real alpha = rz / pq;
        rn = 0.0;
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            rn += r[i] * r[i];
        }
        real rz1 = 0.0;
        for (int64_t i = 0; i < n; ++i) {
            z[i] = dinv[i] * r[i];
            rz1 += r[i] * z[i];
        }
        const real beta = rz1 / rz;
        rz = rz1;
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        ++it;
    }
    *iters = it;
    *rel_res = std::sqrt(rn) / bn;
    return std::sqrt(rn) / bn <= rtol ? 0 : 2;
}

// The same Jacobi-PCG with every loop split over nthreads host threads (row
// blocks; per-thread partial dot products summed in thread order), the CPU
// counterpart of the reference's AztecOO CG + Jacobi on a node's cores.
int orc_pcg_mt(int64_t n, const int32_t* rp, const int32_t* ci, const double* v, const double* b, double* x,
               double rtol, int max_iter, int nthreads, int* iters, double* rel_res) {
    const int T = std::max(1, nthreads);
    std::vector<real> r(n), z(n), p(n), q(n), dinv(n, 1.0);
    std::vector<real> part(3 * T);
    auto par = [&](auto&& body) {  // body(t, lo, hi) over row blocks
        std::vector<std::thread> th;
        for (int t = 0; t < T; ++t) {
            const int64_t lo = n * t / T, hi = n * (t + 1) / T;
            th.emplace_back([&, t, lo, hi] { body(t, lo, hi); });
        }
        for (auto& h : th) h.join();
    };
    auto sum = [&](int k) {
        real s = 0.0;
        for (int t = 0; t < T; ++t) s += part[3 * t + k];
        return s;
    };
    par([&](int t, int64_t lo, int64_t hi) {
        real bb = 0.0, rz = 0.0, rr = 0.0;
        for (int64_t i = lo; i < hi; ++i) {
            real s = 0.0, d = 1.0;
            for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
                s += v[k] * x[ci[k]];
                if (ci[k] == i) d = v[k];
            }
            dinv[i] = 1.0 / d;
            r[i] = b[i] - s;
            z[i] = dinv[i] * r[i];
            p[i] = z[i];
            bb += b[i] * b[i];
            rz += r[i] * z[i];
            rr += r[i] * r[i];
        }
        part[3 * t] = bb;
        part[3 * t + 1] = rz;
        part[3 * t + 2] = rr;
    });
    real bn = std::sqrt(sum(0));
    if (bn == 0.0) bn = 1.0;
    real rz = sum(1), rn = sum(2);
    int it = 0;
    while (std::sqrt(rn) / bn > rtol && it < max_iter) {
        par([&](int t, int64_t lo, int64_t hi) {
            real pq = 0.0;
            for (int64_t i = lo; i < hi; ++i) {
                real s = 0.0;
                for (int32_t k = rp[i]; k < rp[i + 1]; ++k) s += v[k] * p[ci[k]];
                q[i] = s;
                pq += p[i] * s;
            }
            part[3 * t] = pq;
        });
        const real alpha = rz / sum(0);
        par([&](int t, int64_t lo, int64_t hi) {
            real rr = 0.0, rz1 = 0.0;
            for (int64_t i = lo; i < hi; ++i) {
                x[i] += alpha * p[i];
                r[i] -= alpha * q[i];
                z[i] = dinv[i] * r[i];
                rr += r[i] * r[i];
                rz1 += r[i] * z[i];
            }
            part[3 * t] = rr;
            part[3 * t + 1] = rz1;
        });
        rn = sum(0);
        const real rz1 = sum(1);
        const real beta = rz1 / rz;
        rz = rz1;
        par([&](int, int64_t lo, int64_t hi) {
            for (int64_t i = lo; i < hi; ++i) p[i] = z[i] + beta * p[i];
        });
        ++it;
    }
    *iters = it;
    *rel_res = std::sqrt(rn) / bn;
    return std::sqrt(rn) / bn <= rtol ? 0 : 2;
}

}  // extern "C"
