/*
 * fem_oracle.h -- C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a plain C++ restatement of the
 * MORIS element hot path (FEM/INT Element_Bulk / Element_Sideset, the
 * isotropic linear-elasticity IWGs and CM, MTK shape functions and Gauss
 * tables, HMR level-0 B-spline extraction, MSI adof numbering and the
 * T^T K T projection, DLA/SOL CSR scatter).  It exists so that tests, the
 * smoke check and the CPU baseline leg of the benchmark can check the CUDA
 * product path against it.  The product library never links, loads or calls
 * it.  Every routine in fem_oracle.cpp cites the reference file:line it
 * restates.
 */
#ifndef MORIS_GB300_FEM_ORACLE_H
#define MORIS_GB300_FEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cell / rule / iwg enums are numerically identical to include/fem_gpu.h */
enum { ORC_CELL_QUAD4 = 0, ORC_CELL_HEX8 = 1, ORC_CELL_TRI3 = 2, ORC_CELL_TET4 = 3, ORC_CELL_LINE2 = 4 };
enum {
    ORC_RULE_BAR_1 = 0, ORC_RULE_BAR_3 = 1, ORC_RULE_QUAD_2x2 = 2, ORC_RULE_HEX_2x2x2 = 3,
    ORC_RULE_HEX_3x3x3 = 4, ORC_RULE_TRI_7 = 5, ORC_RULE_TET_4 = 6, ORC_RULE_TET_11 = 7,
    ORC_RULE_TRI_3 = 8
};
enum { ORC_MODEL_PLANE_STRAIN = 0, ORC_MODEL_PLANE_STRESS = 1, ORC_MODEL_3D = 2 };
enum { ORC_SHAPE_RECTANGULAR = 0, ORC_SHAPE_GENERAL = 1 };
enum {
    ORC_IWG_STRUC_LINEAR_BULK = 0,
    ORC_IWG_STRUC_LINEAR_NEUMANN = 1,
    ORC_IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE = 2,
    ORC_IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE = 3,
    ORC_IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE = 4,
    ORC_IWG_STRUC_LINEAR_INTERFACE_UNSYMMETRIC_NITSCHE = 5,
    ORC_IWG_STRUC_LINEAR_VW_GHOST = 6,
    ORC_IWG_GHOST_NORMAL_FIELD = 7
};

/* ---- reference-element tables ---------------------------------------- */
/* the reference's automatic integration rule of a set (kind 0 bulk, 1 side,
   2 double side) with integration cells `cell`, linear interpolation cells */
int orc_auto_rule(int kind, int cell);
int orc_rule_size(int rule, int* dim, int* npts);
/* points are stored one column per point (dim x npts, column-major) */
int orc_rule(int rule, double* pts, double* weights);
int orc_cell_num_nodes(int cell);
int orc_cell_param_dim(int cell);
/* N: 1 x n; dNdxi: pdim x n column-major */
int orc_shape(int cell, const double* xi, double* N, double* dNdxi);
double orc_bspline_shape(int order, int basis, double xi);

/* ---- HMR uniform level-0 mesh ----------------------------------------- */
typedef struct orc_mesh orc_mesh;
orc_mesh* orc_hmr_uniform(int dim, const int* nelem, const double* length, int bspline_order);
void orc_mesh_sizes(const orc_mesh* m, int64_t* num_nodes, int64_t* num_cells, int64_t* num_bases,
                    int64_t* t_nnz);
void orc_mesh_arrays(const orc_mesh* m, double* coords, int32_t* cell_nodes, int64_t* t_offsets,
                     int32_t* t_bases, double* t_weights);
void orc_mesh_free(orc_mesh* m);

/* ---- element model ------------------------------------------------------ */
typedef struct orc_model orc_model;
orc_model* orc_model_create(int dim, int ip_cell, int cell_shape, int64_t num_nodes,
                            const double* coords, int64_t num_cells, const int32_t* cell_nodes,
                            int64_t num_bases, const int64_t* t_offsets, const int32_t* t_bases,
                            const double* t_weights);
void orc_model_free(orc_model* m);
/* bulk set: one cluster per entry; ig_offsets == NULL means trivial clusters
   (the IG cell is the IP cell).  Otherwise cluster c owns IG cells
   [ig_offsets[c], ig_offsets[c+1]); ig_coords / ig_param hold nverts x dim
   doubles per IG cell (node-major). */
int orc_model_add_bulk_set(orc_model* m, int ig_cell, int rule, int model_type, int64_t num_clusters,
                           const int32_t* cluster_ip_cell, const int64_t* ig_offsets,
                           const double* ig_coords, const double* ig_param,
                           const double* youngs_modulus, double poisson);
/* optional nodal density field of bulk set `set`: E(x) = E0 rho(x)^beta */
int orc_model_set_density(orc_model* m, int set, const double* node_rho, double beta);
/* side set on IP-cell facets (trivial side clusters).  value = traction
   (Neumann) or prescribed displacement (Dirichlet), dim doubles per set. */
int orc_model_add_side_set(orc_model* m, int iwg, int rule, int model_type, int64_t num_sides,
                           const int32_t* side_ip_cell, const int32_t* side_ordinal,
                           const double* youngs_modulus, double poisson, double nitsche_alpha,
                           const double* value);
/* double-sided set (interface / ghost); sets are indexed bulk sets first,
   then side sets, then double-sided sets */
/* Thickness property of bulk set `set` (w* times thickness) */
int orc_model_set_bulk_thickness(orc_model* m, int set, double thickness);
/* Thickness and Select properties of the side_set-th side set; select is a
   dim x dim row-major matrix or NULL (identity) */
int orc_model_set_side_options(orc_model* m, int side_set, double thickness, const double* select);
int orc_model_add_double_side_set(orc_model* m, int iwg, int facet_cell, int rule, int model_type,
                                  int64_t num_clusters, const int32_t* leader, const int32_t* follower,
                                  const int64_t* facet_offsets, const double* facet_coords,
                                  const double* leader_param, const double* follower_param,
                                  const double* leader_E, const double* follower_E, double nu, double alpha);
/* replace the integration-cell / facet geometry of one cluster (same counts) */
int orc_model_update_ig(orc_model* m, int set, int64_t eq, const double* coords, const double* param);
int orc_model_update_facets(orc_model* m, int set, int64_t eq, const double* coords, const double* leader_param,
                            const double* follower_param);
int orc_model_finalize(orc_model* m);
int64_t orc_model_num_adofs(const orc_model* m);
int64_t orc_model_nnz(const orc_model* m);
int orc_model_num_sets(const orc_model* m);
int64_t orc_model_num_eq(const orc_model* m, int set);
int orc_graph(const orc_model* m, int32_t* rowptr, int32_t* colidx);
int orc_element_topology(const orc_model* m, int set, int64_t eq, int32_t* ids, int32_t* n);
/* element operator (column-major) and residual in adof space */
int orc_element_matrices(const orc_model* m, int set, int64_t eq, const double* u_adof,
                         double* K_colmajor, double* R);
/* pdof-space (before T^T K T) element matrices, for unit checks */
/* Voigt stress of bulk set `set`, equation object eq, at IP-parametric point
   xi; ncomp = number of components */
int orc_element_flux(const orc_model* m, int set, int64_t eq, const double* xi, const double* u_adof,
                     double* flux, int32_t* ncomp);
int orc_element_pdof_matrices(const orc_model* m, int set, int64_t eq, const double* u_pdof,
                              double* K_colmajor, double* R, int32_t* npdof);
/* full assembly; eq_stride > 1 assembles every eq_stride-th element only
   (bounded CPU samples).  vals: nnz doubles, rhs: num_adofs doubles, zeroed
   first unless zero_first == 0. */
int orc_assemble(const orc_model* m, const double* u_adof, double* vals, double* rhs, int nthreads,
                 int64_t eq_stride, int zero_first);
/* conjugate gradients with Jacobi preconditioner on a CSR matrix */
int orc_pcg(int64_t n, const int32_t* rowptr, const int32_t* colidx, const double* vals,
            const double* b, double* x, double rtol, int max_iter, int jacobi, int* iters,
            double* rel_res);
/* orc_pcg with its loops split over nthreads host threads */
int orc_pcg_mt(int64_t n, const int32_t* rowptr, const int32_t* colidx, const double* vals, const double* b,
               double* x, double rtol, int max_iter, int nthreads, int* iters, double* rel_res);

#ifdef __cplusplus
}
#endif
#endif
