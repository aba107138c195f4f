// fem_gpu_moris_adapter.hpp -- the GPU element loop written into MORIS's
// distributed system through MORIS's own interfaces.
//
// Templated on the reference's types so that this header needs none of its
// headers: IdMatrix = moris::Matrix< DDSMat >, RealMatrix = moris::Matrix<
// DDRMat >, DistMatrix = moris::sol::Dist_Matrix, DistVector =
// moris::sol::Dist_Vector.  The calls it makes are those types' public API:
//   Matrix::set_size( rows, cols ), Matrix::operator()( i, j ),
//   Dist_Matrix::sum_into_values( rowIDs, columnIDs, values )
//       (SOL/SOL_CORE/src/cl_SOL_Dist_Matrix.hpp:101-104),
//   Dist_Matrix::matrix_global_assembly() (:110),
//   Dist_Vector::sum_into_global_values( ids, values, vectorIndex )
//       (SOL/SOL_CORE/src/cl_SOL_Dist_Vector.hpp:114-117),
//   Dist_Vector::vector_global_assembly() (:134).
//
// It replaces Solver_Interface::fill_matrix_and_RHS (SOL/DLA/src/
// cl_DLA_Solver_Interface.cpp:317-379): the same matrix and right-hand side
// (sum over the equation objects of K_a and R_a at the adof ids), assembled on
// the GPU as CSR and summed into the distributed objects one row at a time.
// Global ids are the adof ids of this library, which number the adofs as MSI
// does (per dof type, then by basis rank).
#pragma once

#include <cstdint>
#include <vector>

#include "fem_gpu_solver_interface.hpp"

namespace moris_gb300 {

template <class IdMatrix, class RealMatrix>
class Moris_Adapter {
  public:
    explicit Moris_Adapter(Gpu_Solver_Interface& gpu) : gpu_(gpu) {
        gpu_.build_graph(rowptr_, colidx_);
        vals_.resize(colidx_.size());
        rhs_.resize(rowptr_.size() - 1);
    }

    // Solver_Interface::fill_matrix_and_RHS( aMat, aVectorRHS ) with the adof
    // values u (host, one per adof id; NULL = zero state)
    template <class DistMatrix, class DistVector>
    void fill_matrix_and_RHS(const double* u_adof, DistMatrix* mat, DistVector* rhs_vector) {
        gpu_.fill_matrix_and_RHS(u_adof, vals_.data(), rhs_.data());
        const int64_t nrows = (int64_t)rowptr_.size() - 1;
        IdMatrix row, cols;
        RealMatrix v;
        for (int64_t r = 0; r < nrows; ++r) {
            const int32_t b = rowptr_[r], n = rowptr_[r + 1] - b;
            if (n == 0) continue;
            row.set_size(1, 1);
            row(0, 0) = (int32_t)r;
            cols.set_size(n, 1);
            v.set_size(1, n);
            for (int32_t k = 0; k < n; ++k) {
                cols(k, 0) = colidx_[b + k];
                v(0, k) = vals_[b + k];
            }
            mat->sum_into_values(row, cols, v);
        }
        IdMatrix ids;
        RealMatrix rv;
        ids.set_size(nrows, 1);
        rv.set_size(nrows, 1);
        for (int64_t r = 0; r < nrows; ++r) {
            ids(r, 0) = (int32_t)r;
            rv(r, 0) = rhs_[r];
        }
        rhs_vector->sum_into_global_values(ids, rv, 0);
        mat->matrix_global_assembly();
        rhs_vector->vector_global_assembly();
    }

    // Solver_Interface::get_element_topology( set, eq, aElementTopology )
    void get_element_topology(int set, long eq, IdMatrix& topology) const {
        std::vector<int32_t> ids;
        gpu_.get_element_topology(set, eq, ids);
        topology.set_size((long)ids.size(), 1);
        for (size_t k = 0; k < ids.size(); ++k) topology((long)k, 0) = ids[k];
    }

    // Solver_Interface::get_equation_object_operator_and_rhs( set, eq, K, R )
    // for bulk and side sets: K (n x n) and R (n x 1) in the order of the
    // element topology
    void get_equation_object_operator_and_rhs(int set, long eq, const double* u_adof, RealMatrix& K,
                                              RealMatrix& R) {
        std::vector<double> Kp, Rp;
        std::vector<int32_t> ids;
        gpu_.get_element_topology(set, eq, ids);
        gpu_.get_equation_object_operator_and_rhs(set, eq, u_adof, Kp, Rp);
        const long n = (long)ids.size(), nmax = (long)Rp.size();
        const int dim = gpu_.spatial_dim();
        const long width = nmax / dim, nb = n / dim;  // padded layout: row f * width + i
        K.set_size(n, n);
        R.set_size(n, 1);
        for (long c = 0; c < n; ++c) {
            const long pc = (c / nb) * width + c % nb;
            R(c, 0) = Rp[pc];
            for (long r = 0; r < n; ++r) K(r, c) = Kp[(size_t)pc * nmax + (r / nb) * width + r % nb];
        }
    }

    const std::vector<int32_t>& rowptr() const { return rowptr_; }
    const std::vector<int32_t>& colidx() const { return colidx_; }

  private:
    Gpu_Solver_Interface& gpu_;
    std::vector<int32_t> rowptr_, colidx_;
    std::vector<double> vals_, rhs_;
};

}  // namespace moris_gb300
