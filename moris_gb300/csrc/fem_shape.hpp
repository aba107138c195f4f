// fem_shape.hpp -- reference-element shape functions usable on host and
// device (Lagrange QUAD4/HEX8/TRI3/TET4/LINE2 of the reference's
// MTK/src/interpolation/cl_MTK_Interpolation_Function_Lagrange_*.hpp).
#pragma once

#ifdef __CUDACC__
#define FEM_HD __host__ __device__ __forceinline__
#else
#define FEM_HD inline
#endif

namespace fem {

// dN layout: dN[i * n + a] = dN_a / dxi_i
template <int CELL>
struct Shape;

template <>
struct Shape<4> {  // LINE2
    static constexpr int n = 2, pd = 1;
    FEM_HD static void eval(const double* xi, double* N, double* dN) {
        N[0] = 0.5 * (1.0 - xi[0]);
        N[1] = 0.5 * (1.0 + xi[0]);
        dN[0] = -0.5;
        dN[1] = 0.5;
    }
};

template <>
struct Shape<0> {  // QUAD4
    static constexpr int n = 4, pd = 2;
    FEM_HD static void eval(const double* xi, double* N, double* dN) {
        const double sx[4] = {-1, 1, 1, -1}, sy[4] = {-1, -1, 1, 1};
        for (int a = 0; a < 4; ++a) {
            const double fx = 1.0 + sx[a] * xi[0], fy = 1.0 + sy[a] * xi[1];
            N[a] = fx * fy * 0.25;
            dN[a] = 0.25 * sx[a] * fy;
            dN[4 + a] = 0.25 * sy[a] * fx;
        }
    }
};

template <>
struct Shape<1> {  // HEX8
    static constexpr int n = 8, pd = 3;
    FEM_HD static void eval(const double* xi, double* N, double* dN) {
        for (int a = 0; a < 8; ++a) {
            const double sx = ((a & 3) == 1 || (a & 3) == 2) ? 1.0 : -1.0;
            const double sy = ((a & 3) >= 2) ? 1.0 : -1.0;
            const double sz = a >= 4 ? 1.0 : -1.0;
            const double fx = 1.0 + sx * xi[0], fy = 1.0 + sy * xi[1], fz = 1.0 + sz * xi[2];
            N[a] = fx * fy * fz * 0.125;
            dN[a] = 0.125 * sx * fy * fz;
            dN[8 + a] = 0.125 * sy * fx * fz;
            dN[16 + a] = 0.125 * sz * fx * fy;
        }
    }
};

template <>
struct Shape<2> {  // TRI3
    static constexpr int n = 3, pd = 2;
    FEM_HD static void eval(const double* xi, double* N, double* dN) {
        N[0] = xi[0];
        N[1] = xi[1];
        N[2] = 1.0 - xi[0] - xi[1];
        dN[0] = 1; dN[1] = 0; dN[2] = -1;
        dN[3] = 0; dN[4] = 1; dN[5] = -1;
    }
};

template <>
struct Shape<3> {  // TET4: (xi1, xi2, 1 - xi1 - xi2 - xi3, xi3)
    static constexpr int n = 4, pd = 3;
    FEM_HD static void eval(const double* xi, double* N, double* dN) {
        N[0] = xi[0];
        N[1] = xi[1];
        N[2] = 1.0 - xi[0] - xi[1] - xi[2];
        N[3] = xi[2];
        dN[0] = 1; dN[1] = 0; dN[2] = -1; dN[3] = 0;
        dN[4] = 0; dN[5] = 1; dN[6] = -1; dN[7] = 0;
        dN[8] = 0; dN[9] = 0; dN[10] = -1; dN[11] = 1;
    }
};

}  // namespace fem
