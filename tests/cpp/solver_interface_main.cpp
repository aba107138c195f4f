// solver_interface_main.cpp -- the integration path of INTEGRATION.md, run
// (test infrastructure).  A maintainer's Solver_Interface subclass forwards
// fill_matrix_and_RHS to the GPU adapter; the program calls it through the
// base pointer, as Linear_Problem::assemble_residual_and_jacobian does
// (SOL/DLA/src/cl_DLA_Linear_Problem.cpp:131-138), then the per-object calls
// get_element_topology / get_equation_object_operator_and_rhs, and writes
// everything for the Python side to compare with the oracle.
//
//   solver_interface_main <input> <output>
// input : int32 dim, nn, nc, nb, nz, nleft, nright; double coords[nn*dim];
//         int32 cells[nc*npe]; int64 t_off[nn+1]; int32 t_bases[nz];
//         double t_w[nz]; double E[nc]; int32 left[nleft]; int32 right[nright];
//         int64 nad; double u[nad]
// output: int64 nad, nentries; nentries x (int32 row, int32 col, double v);
//         double rhs[nad]; for each of the 3 sets: int64 neq, then per object
//         int32 n, int32 ids[n], double K[n*n] (column-major), double R[n]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fem_gpu_moris_adapter.hpp"
#include "moris_stand_in.hpp"

using moris::DDRMat;
using moris::DDSMat;
using moris::Matrix;

// what a maintainer adds: the GPU element loop behind the (patched, virtual)
// Solver_Interface::fill_matrix_and_RHS
class Gpu_MSI_Solver_Interface : public moris::Solver_Interface {
  public:
    Gpu_MSI_Solver_Interface(moris_gb300::Gpu_Solver_Interface& gpu, const double* u) : mAdapter(gpu), mU(u) {}
    void fill_matrix_and_RHS(moris::sol::Dist_Matrix* aMat, moris::sol::Dist_Vector* aVectorRHS) override {
        mAdapter.fill_matrix_and_RHS(mU, aMat, aVectorRHS);
    }
    moris_gb300::Moris_Adapter<Matrix<DDSMat>, Matrix<DDRMat>> mAdapter;
    const double* mU;
};

template <class T>
static void rd(FILE* f, T* p, size_t n) {
    if (n && std::fread(p, sizeof(T), n, f) != n) {
        std::fprintf(stderr, "short input\n");
        std::exit(2);
    }
}
template <class T>
static void wr(FILE* f, const T* p, size_t n) {
    if (n) std::fwrite(p, sizeof(T), n, f);
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int32_t h[7];
    rd(in, h, 7);
    const int dim = h[0], npe = dim == 2 ? 4 : 8;
    const int64_t nn = h[1], nc = h[2], nb = h[3], nz = h[4], nl = h[5], nr = h[6];
    std::vector<double> coords(nn * dim), tw(nz), E(nc);
    std::vector<int32_t> cells(nc * npe), tb(nz), left(nl), right(nr);
    std::vector<int64_t> toff(nn + 1);
    rd(in, coords.data(), coords.size());
    rd(in, cells.data(), cells.size());
    rd(in, toff.data(), toff.size());
    rd(in, tb.data(), tb.size());
    rd(in, tw.data(), tw.size());
    rd(in, E.data(), E.size());
    rd(in, left.data(), left.size());
    rd(in, right.data(), right.size());
    int64_t nad = 0;
    rd(in, &nad, 1);
    std::vector<double> u(nad);
    rd(in, u.data(), u.size());
    std::fclose(in);

    try {
        fem_gpu_mesh_desc mesh{};
        mesh.spatial_dim = dim;
        mesh.ip_cell_type = dim == 2 ? FEM_GPU_CELL_QUAD4 : FEM_GPU_CELL_HEX8;
        mesh.cell_shape = FEM_GPU_SHAPE_RECTANGULAR;
        mesh.num_nodes = nn;
        mesh.node_coords = coords.data();
        mesh.num_cells = nc;
        mesh.cell_nodes = cells.data();
        mesh.num_bases = nb;
        mesh.t_offsets = toff.data();
        mesh.t_bases = tb.data();
        mesh.t_weights = tw.data();
        moris_gb300::Gpu_Solver_Interface gpu(mesh);

        std::vector<int32_t> all(nc);
        for (int64_t i = 0; i < nc; ++i) all[i] = (int32_t)i;
        fem_gpu_bulk_set_desc bulk{};
        bulk.iwg_type = FEM_GPU_IWG_STRUC_LINEAR_BULK;
        bulk.ig_cell_type = mesh.ip_cell_type;
        bulk.integration_rule = FEM_GPU_RULE_AUTO;
        bulk.model_type = dim == 2 ? FEM_GPU_MODEL_PLANE_STRAIN : FEM_GPU_MODEL_3D;
        bulk.num_clusters = nc;
        bulk.cluster_ip_cell = all.data();
        bulk.youngs_modulus = E.data();
        bulk.poisson_ratio = 0.3;
        bulk.thickness = 0.5;
        gpu.add_bulk_set(bulk);

        std::vector<double> El(nl), Er(nr);
        std::vector<int32_t> ol(nl, 3), orr(nr, 1);
        for (int64_t i = 0; i < nl; ++i) El[i] = E[left[i]];
        for (int64_t i = 0; i < nr; ++i) Er[i] = E[right[i]];
        const double select[4] = {1.0, 0.0, 0.0, 0.0};  // a roller: x only
        fem_gpu_side_set_desc dir{};
        dir.iwg_type = FEM_GPU_IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE;
        dir.integration_rule = FEM_GPU_RULE_AUTO;
        dir.model_type = bulk.model_type;
        dir.num_sides = nl;
        dir.side_ip_cell = left.data();
        dir.side_ordinal = ol.data();
        dir.youngs_modulus = El.data();
        dir.poisson_ratio = 0.3;
        dir.nitsche_alpha = 100.0;
        dir.thickness = 0.5;
        dir.select_matrix = select;
        gpu.add_side_set(dir);
        fem_gpu_side_set_desc neu{};
        neu.iwg_type = FEM_GPU_IWG_STRUC_LINEAR_NEUMANN;
        neu.integration_rule = FEM_GPU_RULE_AUTO;
        neu.model_type = bulk.model_type;
        neu.num_sides = nr;
        neu.side_ip_cell = right.data();
        neu.side_ordinal = orr.data();
        neu.youngs_modulus = Er.data();
        neu.poisson_ratio = 0.3;
        neu.value[0] = 1e-3;
        neu.value[1] = -2e-3;
        neu.thickness = 0.5;
        gpu.add_side_set(neu);
        gpu.finalize();
        if (gpu.num_adofs() != nad) {
            std::fprintf(stderr, "adof count %lld != %lld\n", (long long)gpu.num_adofs(), (long long)nad);
            return 3;
        }

        // the reference's call sequence: a Solver_Interface pointer, fill_matrix_and_RHS
        Gpu_MSI_Solver_Interface impl(gpu, u.data());
        moris::Solver_Interface* si = &impl;
        moris::Recording_Matrix mat;
        moris::Recording_Vector rhs(nad);
        si->fill_matrix_and_RHS(&mat, &rhs);
        if (!mat.assembled || !rhs.assembled) return 4;

        FILE* out = std::fopen(argv[2], "wb");
        if (!out) return 2;
        const int64_t ne = (int64_t)mat.entries.size();
        wr(out, &nad, 1);
        wr(out, &ne, 1);
        for (const auto& kv : mat.entries) {
            const int32_t rc[2] = {kv.first.first, kv.first.second};
            wr(out, rc, 2);
            wr(out, &kv.second, 1);
        }
        wr(out, rhs.values.data(), rhs.values.size());
        for (int s = 0; s < gpu.get_num_sets(); ++s) {
            const int64_t neq = gpu.get_num_equation_objects_on_set(s);
            wr(out, &neq, 1);
            for (int64_t e = 0; e < neq; ++e) {
                Matrix<DDSMat> topo;
                Matrix<DDRMat> K, R;
                impl.mAdapter.get_element_topology(s, (long)e, topo);
                impl.mAdapter.get_equation_object_operator_and_rhs(s, (long)e, u.data(), K, R);
                const int32_t n = (int32_t)topo.n_rows();
                wr(out, &n, 1);
                for (int32_t i = 0; i < n; ++i) wr(out, &topo(i, 0), 1);
                for (int32_t c = 0; c < n; ++c)
                    for (int32_t r = 0; r < n; ++r) wr(out, &K(r, c), 1);
                for (int32_t r = 0; r < n; ++r) wr(out, &R(r, 0), 1);
            }
        }
        std::fclose(out);
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 5;
    }
    return 0;
}
