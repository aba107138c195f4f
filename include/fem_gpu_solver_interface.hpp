// fem_gpu_solver_interface.hpp -- header-only C++ layer over the C ABI in
// fem_gpu.h, shaped like the element-loop part of moris::Solver_Interface
// (SOL/DLA/src/cl_DLA_Solver_Interface.hpp:58-661) so that a reference-side
// adapter can forward its calls one to one:
//
//   get_num_sets()                              Solver_Interface::get_num_sets
//   get_num_equation_objects_on_set(set)        ::get_num_equation_objects_on_set
//   get_element_topology(set, eq, ids)          ::get_element_topology
//   get_equation_object_operator_and_rhs(...)   ::get_equation_object_operator_and_rhs
//   build_graph(rowptr, colidx)                 ::build_graph / compute_sparsity_pattern
//   fill_matrix_and_RHS(u, vals, rhs)           ::fill_matrix_and_RHS
//
// Errors are raised as std::runtime_error, the reference's MORIS_ERROR
// convention (MRS/ASR/src/fn_log_assert.hpp:33-92); the C ABI below never
// throws.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "fem_gpu.h"

namespace moris_gb300 {

inline void check(fem_gpu_status s, fem_gpu_ctx* c, const char* what) {
    if (s != FEM_GPU_OK)
        throw std::runtime_error(std::string(what) + ": " + fem_gpu_status_string(s) + " (" +
                                 (c ? fem_gpu_last_error(c) : "") + ")");
}

class Gpu_Solver_Interface {
  public:
    explicit Gpu_Solver_Interface(const fem_gpu_mesh_desc& mesh) : dim_(mesh.spatial_dim) {
        check(fem_gpu_create(&mesh, &ctx_), nullptr, "fem_gpu_create");
    }
    ~Gpu_Solver_Interface() { fem_gpu_destroy(ctx_); }
    Gpu_Solver_Interface(const Gpu_Solver_Interface&) = delete;
    Gpu_Solver_Interface& operator=(const Gpu_Solver_Interface&) = delete;

    int add_bulk_set(const fem_gpu_bulk_set_desc& d) {
        int32_t i = -1;
        check(fem_gpu_add_bulk_set(ctx_, &d, &i), ctx_, "add_bulk_set");
        return i;
    }
    int add_side_set(const fem_gpu_side_set_desc& d) {
        int32_t i = -1;
        check(fem_gpu_add_side_set(ctx_, &d, &i), ctx_, "add_side_set");
        return i;
    }
    int add_double_side_set(const fem_gpu_double_side_set_desc& d) {
        int32_t i = -1;
        check(fem_gpu_add_double_side_set(ctx_, &d, &i), ctx_, "add_double_side_set");
        return i;
    }
    void finalize() {
        check(fem_gpu_finalize(ctx_), ctx_, "finalize");
        check(fem_gpu_get_sizes(ctx_, &num_adofs_, &nnz_, &num_sets_), ctx_, "get_sizes");
    }

    int get_num_sets() const { return num_sets_; }
    long get_num_equation_objects_on_set(int set) const {
        int64_t n = 0;
        check(fem_gpu_get_num_equation_objects(ctx_, set, &n), ctx_, "num_equation_objects");
        return (long)n;
    }
    void get_element_topology(int set, long eq, std::vector<int32_t>& ids) const {
        int32_t nmax = 0, n = 0;
        check(fem_gpu_get_max_element_adofs(ctx_, set, &nmax), ctx_, "max_element_adofs");
        ids.resize(nmax);
        check(fem_gpu_get_element_topology(ctx_, set, eq, ids.data(), &n), ctx_, "element_topology");
        ids.resize(n);
    }
    // element operator (column-major, nmax x nmax, zero padded: row f * width +
    // i, width = nmax / dim, for bulk and side sets) and residual
    void get_equation_object_operator_and_rhs(int set, long eq, const double* u_adof_host, std::vector<double>& K,
                                              std::vector<double>& R) {
        int32_t nmax = 0;
        check(fem_gpu_get_max_element_adofs(ctx_, set, &nmax), ctx_, "max_element_adofs");
        K.assign((size_t)nmax * nmax, 0.0);
        R.assign(nmax, 0.0);
        check(fem_gpu_element_matrices(ctx_, set, eq, 1, u_adof_host, K.data(), R.data(), FEM_GPU_HOST_BUFFERS),
              ctx_, "element_matrices");
    }
    void build_graph(std::vector<int32_t>& rowptr, std::vector<int32_t>& colidx) {
        rowptr.resize(num_adofs_ + 1);
        colidx.resize(nnz_);
        check(fem_gpu_build_graph(ctx_, rowptr.data(), colidx.data(), FEM_GPU_HOST_BUFFERS), ctx_, "build_graph");
    }
    // host buffers: values in CSR order of build_graph, residual per adof
    void fill_matrix_and_RHS(const double* u_adof, double* csr_vals, double* rhs, bool device_buffers = false) {
        check(fem_gpu_assemble(ctx_, u_adof, csr_vals, rhs, device_buffers ? 0u : FEM_GPU_HOST_BUFFERS), ctx_,
              "assemble");
    }

    int spatial_dim() const { return dim_; }
    int64_t num_adofs() const { return num_adofs_; }
    int64_t nnz() const { return nnz_; }
    fem_gpu_ctx* handle() { return ctx_; }

  private:
    fem_gpu_ctx* ctx_ = nullptr;
    int dim_ = 0;
    int64_t num_adofs_ = 0, nnz_ = 0;
    int32_t num_sets_ = 0;
};

}  // namespace moris_gb300
