// fem_internal.hpp -- private declarations shared by the host (.cpp) and
// device (.cu) translation units of libfem_gpu.so.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fem_gpu.h"

namespace fem {

// ---- reference-element tables (fem_tables.cpp) --------------------------
struct Rule {
    int dim = 0, n = 0;
    std::vector<double> pts;  // n x dim, point-major
    std::vector<double> w;
};
Rule gauss_rule(int rule);
int cell_num_nodes(int cell);
int cell_param_dim(int cell);
// N (n), dNdxi (pdim x n, row-major: dNdxi[i*n + a])
void lagrange(int cell, const double* xi, double* N, double* dNdxi);
void cell_param_coords(int cell, double* xi_hat);  // n x pdim, node-major
const int* facet_vertices(int ip_cell, int ordinal, int* count);

// ---- host-side set data ----------------------------------------------------
struct DeviceBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// Everything a kernel reads for one set, laid out per equation object.
struct SetData {
    int kind = 0;  // 0 bulk, 1 side, 2 double-sided (interface / ghost)
    fem_gpu_bulk_set_desc bulk{};
    fem_gpu_side_set_desc side{};
    double bulk_thickness = 1.0;   // bulk sets: Thickness property (folded into E)
    double side_thickness = 1.0;   // side sets: w* factor (Thickness property)
    double side_select[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};  // side sets: Select matrix M (3 x 3 row-major)
    fem_gpu_double_side_set_desc dside{};
    int64_t neq = 0;
    std::vector<int32_t> ip_cell;
    std::vector<int64_t> ig_off;
    std::vector<double> ig_coords, ig_param;
    std::vector<double> E;
    std::vector<int32_t> ordinal;
    // double-sided sets: ip_cell holds the leaders
    std::vector<int32_t> fcell;                  // follower cells
    std::vector<int64_t> fc_off;                 // facet offsets [neq+1]
    std::vector<double> fc_x, fc_xl, fc_xf;      // facet vertex coords, param in leader / follower
    std::vector<double> EF;                      // follower modulus
    std::vector<double> vol;                     // [neq][2] leader / follower cluster volumes
    int nfv = 0;                                 // facet vertices
    std::vector<int32_t> vid;                    // IG vertex ids: cut bulk [ig][4], double [facet][nfv]
    DeviceBuf d_vid;
    std::vector<int32_t> link;                   // interface: [neq][4] leader (set, eq), follower (set, eq)
    DeviceBuf d_link;
    // finalize products (double-sided sets: two sides per equation object,
    // nb [neq][2], bases [neq][2][maxnb], T [neq][2][npe][maxnb],
    // xe [neq][2][npe][dim], sidx [neq][2 maxnb][2 maxnb])
    int maxnb = 0;                 // max unique bases per element (padding width)
    std::vector<int32_t> nb;       // [neq]
    std::vector<int32_t> bases;    // [neq][maxnb] basis ranks, -1 padded
    std::vector<double> T;         // [neq][npe][maxnb] dense element extraction
    std::vector<uint16_t> sidx;    // [neq][maxnb][maxnb] column slot of base j in row of base i
    std::vector<double> xe;        // [neq][npe][dim] interpolation-cell coordinates
    std::vector<double> node_rho;  // nodal density field (bulk, optional)
    std::vector<double> rhoe;      // [neq][npe] densities of the element's nodes
    DeviceBuf d_rho, d_nq;         // device copies: rhoe, N of the IP cell at the Gauss points
    // device copies
    DeviceBuf d_nb, d_bases, d_T, d_sidx, d_xe, d_E, d_ord;
    DeviceBuf d_dn, d_w;    // bulk: dN/dxi of the IP cell at the Gauss points, weights
    DeviceBuf d_pairs;      // bulk: upper-triangle index pairs of the pdof Gram matrix
    DeviceBuf d_ktab;       // bulk: K T item table of the CTA kernels
    DeviceBuf d_tri;        // bulk: T^T K T upper-triangle item table of the CTA kernels
    DeviceBuf d_g0;         // bulk: reference Gram table sum_q w_q dN/dxi dN/dxi
    DeviceBuf d_gp, d_gw;   // side: facet Gauss points and weights
    DeviceBuf d_sref;       // side: facet / cell shape values per ordinal and point
    DeviceBuf d_sgeo;       // side: per facet and point w*, normal, J^-1; 1/h (built once)
    DeviceBuf d_igoff, d_igx, d_igxi;            // cut clusters: integration cells
    DeviceBuf d_adjul;      // cut clusters: pdof values of u and lambda per cluster, cluster of each cell (sensitivities)
    DeviceBuf d_items;      // interface clusters: volume items (e * 2 + side, cell) of the sensitivities
    DeviceBuf d_tperm;      // cut clusters: integration cells grouped by their number of moving vertices
    int64_t tperm_off[5] = {0, 0, 0, 0, 0};  // group of cells with m moving vertices: [off[m-1], off[m]), m = 1..4
    int64_t nitems = 0;
    DeviceBuf d_fcoff, d_fcx, d_fcxl, d_fcxf;    // double-sided: facets
    DeviceBuf d_EF, d_vol;
    int ngp = 0;            // Gauss points of the set's rule
    int nbsel = 0;          // padded basis width of the kernel instance
    int variant = 0;        // bulk kernel variant (set by fem_gpu_autotune)
    double tuned_ms = 0.0;  // time of the chosen variant on the tuning run
};

}  // namespace fem

// Lagrange interpolation mesh with the extraction rows of its nodes
// (fem_hmr_uniform_mesh, fem_hmr_refined_mesh)
struct fem_hmr_mesh {
    int dim = 0;
    int64_t num_bases = 0;
    std::vector<double> coords;
    std::vector<int32_t> cells;
    std::vector<int64_t> t_off;
    std::vector<int32_t> t_bases;
    std::vector<double> t_w;
};

struct fem_gpu_ctx {
    int dim = 0, ip_cell = 0, shape = 0, npe = 0;
    int64_t num_nodes = 0, num_cells = 0, num_bases = 0;
    std::vector<double> coords;
    std::vector<int32_t> cells;
    std::vector<int64_t> t_off;
    std::vector<int32_t> t_bases;
    std::vector<double> t_w;
    std::vector<fem::SetData> sets;
    // MSI / graph products
    bool host_final = false, dev_final = false;
    int64_t num_used = 0;              // used bases
    std::vector<int64_t> basis_rank;   // domain basis -> rank or -1
    std::vector<int32_t> ulen;         // [num_used] |U(b)| (column union length per type)
    std::vector<int64_t> uoff;         // [num_used+1] offsets into ucols
    std::vector<int32_t> ucols;        // union lists (basis ranks, ascending)
    std::vector<int32_t> rowptr;       // [num_adofs+1]
    int64_t nnz = 0;
    // device state
    void* stream = nullptr;            // cudaStream_t
    bool own_stream = false;
    bool stream_set = false;           // caller chose a stream (NULL = legacy default stream)
    fem::DeviceBuf d_rowptr, d_ulen, d_tables, d_scratch, d_status;
    void* batch = nullptr;             // batched-launch state (fem_cluster.cu)
    void* host_pipe = nullptr;         // chunked assembly with overlapped copy-back (fem_device.cu)
    // IG vertex table (shape sensitivities)
    std::vector<int32_t> vkind, vpar;  // [nv], [nv][8]
    std::vector<double> vx, vval;      // [nv][3], [nv]
    fem::DeviceBuf d_vkind, d_vpar, d_vx;
    fem::DeviceBuf d_adjcuts;          // cut-set table of the sensitivity kernels
    bool adj_topo = false;             // vertex kinds / parents, vertex ids, links and items are on the device
    bool adj_coords = false;           // vertex coordinates are on the device
    fem::DeviceBuf d_vval;             // vertex values (phi at background parents)
    bool ls_phi = false;               // d_vval holds the current table's values
    fem::DeviceBuf d_lscols, d_lst;    // level-set field: coefficient ids and weights [nodes][width]
    int64_t ls_nbn = 0, ls_ncoef = 0;  // field sizes (0 nodes: none)
    int32_t ls_width = 0;
    int64_t ls_checked_nbn = -1;       // vertex parents checked against this many background nodes
    int64_t launches = 0;
    std::string err;
};

namespace fem {
// double-sided IWG families: the Nitsche interface (needs cluster volumes) or a ghost penalty
inline bool is_ghost_iwg(int iwg) {
    return iwg == FEM_GPU_IWG_STRUC_LINEAR_VW_GHOST || iwg == FEM_GPU_IWG_GHOST_NORMAL_FIELD;
}
fem_gpu_status fail(fem_gpu_ctx* c, fem_gpu_status s, const std::string& msg);
// multiprocessor count of the current device (cached per device; grid sizing)
int sm_count();
// device side (fem_device.cu)
fem_gpu_status device_finalize(fem_gpu_ctx* c);
void device_release(fem_gpu_ctx* c);
// cut / double-sided clusters (fem_cluster.cu)
fem_gpu_status cluster_finalize(fem_gpu_ctx* c, int set);
void cluster_release(fem_gpu_ctx* c);
bool cluster_set(const fem_gpu_ctx* c, int set);
fem_gpu_status cluster_launch_set(fem_gpu_ctx* c, int set, int mode, int64_t first, int64_t count, const double* u,
                                  double* vals, double* rhs, double* Kout, double* Rout, int nmax);
// measure of an IP cell (sum of w detJ over the 2^d Gauss rule)
double ip_cell_measure(const fem_gpu_ctx* c, int64_t cell);
// leader / follower cluster volumes of the interface sets (finalize and geometry updates)
fem_gpu_status interface_volumes(fem_gpu_ctx* c);
// one set's assembly through its kernel (fem_device.cu); vals / rhs may be NULL
fem_gpu_status assemble_set(fem_gpu_ctx* c, int set, const double* u, double* vals, double* rhs);
// device address of fem_gpu_pcg_noalloc's fixed array on the current device,
// resolved once per device (fem_solver.cu); loads that file's module
fem_gpu_status noalloc_prepare(fem_gpu_ctx* c);
// device memory of the sensitivity path (fem_sensitivity.cu)
void sensitivity_release(fem_gpu_ctx* c);

// Refined HMR meshes on the GPU (fem_hmr_device.cu): the hierarchy as the
// device sees it -- the refined elements of every level as sorted packed keys
// (HMR "mesh" coordinates counted from the first padding element, 20 bits per
// direction), the element-local basis offsets and the sizes.
constexpr int kHmrMaxLocal = 64;
struct HmrDevice {
    int dim = 0, p = 0, pad = 0, nloc = 0, levels = 0;  // levels: refined levels + 1
    int64_t ne[3] = {1, 1, 1};
    int local[kHmrMaxLocal][3] = {};
    std::vector<uint64_t> keys;  // level-major, sorted within a level
    std::vector<int64_t> koff;   // [levels + 1]
};
// element T matrices of `count` elements (level, mesh coordinates) computed
// on the GPU: pass 1 fills ndof; with T != nullptr pass 2 writes, per element
// i, T[toff[i] .. + nloc * ndof[i]) (column-major by dof, as the host's
// element_t) and dofs[dof_off[i] .. + ndof[i]] as (level, m0, m1, m2)
fem_gpu_status hmr_element_t_device(const HmrDevice& h, bool truncate, int64_t count, const int32_t* level,
                                    const int64_t* idx, int32_t* ndof, const int64_t* toff, double* T,
                                    int64_t* dofs);
// node rows on the GPU: for every first visit (element elem[k], node
// coordinates x[k*dim ..]), the element's local B-splines at the node times
// its T: rows[roff[k] .. + ndof[elem[k]]) (same operations and order as the
// host's evaluation)
fem_gpu_status hmr_node_rows_device(const HmrDevice& h, const double* len, int64_t nfirst, const int64_t* elem,
                                    const double* x, const int32_t* level, const int64_t* idx, const int32_t* ndof,
                                    const int64_t* toff, const double* T, const int64_t* roff, double* rows);
}  // namespace fem

// one multigrid V-cycle z = V r on the legacy default stream (fem_multigrid.cu)
bool mg_vcycle(fem_mg* g, const double* r, double* z);
// q = A p with the hierarchy's level-0 FP64 stencil (the operator the CSR
// holds, without column indices) and dot += p.q
bool mg_operator(fem_mg* g, const double* p, double* q, double* dot);
