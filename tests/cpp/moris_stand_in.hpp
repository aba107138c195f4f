// moris_stand_in.hpp -- stand-ins for the few reference types the GPU adapter
// touches, with the reference's signatures (test infrastructure):
//   moris::Matrix< DDSMat / DDRMat >      LINALG/src/cl_Matrix.hpp (set_size,
//                                          operator()( i, j ), n_rows, n_cols)
//   moris::sol::Dist_Matrix               SOL/SOL_CORE/src/cl_SOL_Dist_Matrix.hpp:79-110
//   moris::sol::Dist_Vector               SOL/SOL_CORE/src/cl_SOL_Dist_Vector.hpp:114-134
//   moris::Solver_Interface               SOL/DLA/src/cl_DLA_Solver_Interface.hpp:566-568,
//                                          with fill_matrix_and_RHS made virtual (the
//                                          one-line patch the integration needs)
// The concrete matrix / vector below record what is summed into them.
#pragma once

#include <cstdint>
#include <map>
#include <utility>
#include <vector>

namespace moris {

struct DDSMat {};
struct DDRMat {};
template <class T> struct Elem;
template <> struct Elem<DDSMat> { using type = int32_t; };
template <> struct Elem<DDRMat> { using type = double; };

template <class T>
class Matrix {
  public:
    using value_type = typename Elem<T>::type;
    void set_size(long r, long c) {
        r_ = r;
        c_ = c;
        a_.assign((size_t)(r * c), value_type(0));
    }
    value_type& operator()(long i, long j) { return a_[(size_t)(i + j * r_)]; }
    const value_type& operator()(long i, long j) const { return a_[(size_t)(i + j * r_)]; }
    long n_rows() const { return r_; }
    long n_cols() const { return c_; }

  private:
    long r_ = 0, c_ = 0;
    std::vector<value_type> a_;  // column-major, as the reference's Matrix
};

namespace sol {

class Dist_Matrix {
  public:
    virtual ~Dist_Matrix() = default;
    virtual void sum_into_values(const Matrix<DDSMat>& aRowIDs, const Matrix<DDSMat>& aColumnIDs,
                                 const Matrix<DDRMat>& aMatrixValues) = 0;
    virtual void matrix_global_assembly() = 0;
};

class Dist_Vector {
  public:
    virtual ~Dist_Vector() = default;
    virtual void sum_into_global_values(const Matrix<DDSMat>& aGlobalIds, const Matrix<DDRMat>& aValues,
                                        const unsigned& aVectorIndex = 0) = 0;
    virtual void vector_global_assembly() = 0;
};

}  // namespace sol

class Solver_Interface {
  public:
    virtual ~Solver_Interface() = default;
    // cl_DLA_Solver_Interface.hpp:566-568, made virtual
    virtual void fill_matrix_and_RHS(sol::Dist_Matrix* aMat, sol::Dist_Vector* aVectorRHS) = 0;
};

// recording implementations (coordinate format)
class Recording_Matrix : public sol::Dist_Matrix {
  public:
    void sum_into_values(const Matrix<DDSMat>& rows, const Matrix<DDSMat>& cols,
                         const Matrix<DDRMat>& v) override {
        for (long i = 0; i < rows.n_rows() * rows.n_cols(); ++i)
            for (long j = 0; j < cols.n_rows() * cols.n_cols(); ++j)
                entries[{rows(i, 0), cols(j, 0)}] += v(i, j);
    }
    void matrix_global_assembly() override { assembled = true; }
    std::map<std::pair<int32_t, int32_t>, double> entries;
    bool assembled = false;
};

class Recording_Vector : public sol::Dist_Vector {
  public:
    explicit Recording_Vector(long n) : values((size_t)n, 0.0) {}
    void sum_into_global_values(const Matrix<DDSMat>& ids, const Matrix<DDRMat>& v, const unsigned&) override {
        for (long i = 0; i < ids.n_rows(); ++i) values[(size_t)ids(i, 0)] += v(i, 0);
    }
    void vector_global_assembly() override { assembled = true; }
    std::vector<double> values;
    bool assembled = false;
};

}  // namespace moris
