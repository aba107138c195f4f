/*
 * fem_gpu.h -- C ABI of the GB300 element hot path (libfem_gpu.so).
 *
 * The library replaces the element loop behind MORIS's solver interface:
 *
 *   moris::Solver_Interface  (SOL/DLA/src/cl_DLA_Solver_Interface.hpp:58-661)
 *     fill_matrix_and_RHS            -> fem_gpu_assemble
 *     get_element_topology           -> fem_gpu_get_element_topology
 *     get_equation_object_operator_and_rhs
 *                                    -> fem_gpu_element_matrices
 *     build_graph / compute_sparsity_pattern
 *                                    -> fem_gpu_build_graph
 *     get_num_sets / get_num_equation_objects_on_set
 *                                    -> fem_gpu_get_sizes / fem_gpu_get_num_equation_objects
 *   fem::IWG_Factory::create_IWG(IWG_Type)  (FEM/INT/src/IWG/cl_FEM_IWG_Factory.hpp:43)
 *                                    -> the iwg_type of fem_gpu_add_*_set
 *   HMR T-matrix + MSI adof numbering (HMR/src/cl_HMR_T_Matrix_Base.cpp:306-457,
 *   FEM/MSI/src/cl_MSI_Dof_Manager.cpp:703-985)
 *                                    -> fem_gpu_mesh_desc node T rows + fem_gpu_finalize
 *   sol::Dist_Matrix::fill_matrix / Dist_Vector::sum_into_global_values
 *   (SOL/SOL_CORE/src/cl_Sparse_Matrix_EpetraFECrs.cpp:103-131)
 *                                    -> the CSR scatter inside fem_gpu_assemble
 *   Trilinos AztecOO CG + Jacobi (DLA/src/cl_DLA_Linear_Solver_Aztec.cpp:260-355)
 *                                    -> fem_gpu_pcg
 *   PETSc PCMG geometric multigrid (DLA/src/cl_DLA_Preconditioner_PETSc.cpp:77-345)
 *                                    -> fem_mg_create / fem_mg_apply / fem_gpu_fcg_mg
 *
 * Conventions (identical to the reference):
 *  - global ids are adof ids: type offset + rank of the B-spline basis among the
 *    used bases, types in order UX, UY(, UZ);
 *  - element adof lists are sorted ascending per type, types concatenated;
 *  - element matrices are column-major, square, of size nadof x nadof;
 *  - CSR rows are adofs, column indices ascending.
 *
 * Every function returns an fem_gpu_status and never throws.  A context is
 * single-threaded; calls are ordered on the context's CUDA stream.  Buffers
 * are device pointers unless FEM_GPU_HOST_BUFFERS is set in flags, in which
 * case the library stages the host<->device copies on its stream and
 * synchronises before returning.  fem_gpu_fem_hmr_* are host-only setup
 * helpers (an HMR-equivalent uniform-mesh generator) that need no GPU.
 */
#ifndef MORIS_GB300_FEM_GPU_H
#define MORIS_GB300_FEM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FEM_GPU_ABI_VERSION 3

typedef enum fem_gpu_status {
    FEM_GPU_OK = 0,
    FEM_GPU_BAD_ARG = 1,        /* null pointer, bad enum, size mismatch   */
    FEM_GPU_OOB_INDEX = 2,      /* node / cell / basis index out of range  */
    FEM_GPU_NONFINITE = 3,      /* NaN or Inf in inputs or results         */
    FEM_GPU_DETJ_NEGATIVE = 4,  /* (reserved; GPs below -1e-6 are skipped) */
    FEM_GPU_TIMEOUT = 5,        /* a bounded device wait ran out           */
    FEM_GPU_CUDA_ERROR = 6,     /* a CUDA runtime call failed              */
    FEM_GPU_NOT_FINALIZED = 7,  /* call needs fem_gpu_finalize first        */
    FEM_GPU_UNSUPPORTED = 8,    /* valid but not implemented combination   */
    FEM_GPU_OUT_OF_MEMORY = 9,
    FEM_GPU_NOT_CONVERGED = 10, /* iterative solve hit max iterations      */
    FEM_GPU_NO_DEVICE = 11      /* no usable CUDA device                    */
} fem_gpu_status;

/* cell topologies (mtk::Geometry_Type + interpolation order 1) */
enum { FEM_GPU_CELL_QUAD4 = 0, FEM_GPU_CELL_HEX8 = 1, FEM_GPU_CELL_TRI3 = 2, FEM_GPU_CELL_TET4 = 3,
       FEM_GPU_CELL_LINE2 = 4 };
/* Gauss rules (mtk::Integration_Order).  FEM_GPU_RULE_AUTO in a set
   descriptor picks the reference's automatic rule of that set
   (fem_gpu_auto_integration_rule with the interpolation cells' linear order). */
enum {
    FEM_GPU_RULE_AUTO = -1,
    FEM_GPU_RULE_BAR_1 = 0, FEM_GPU_RULE_BAR_3 = 1, FEM_GPU_RULE_QUAD_2x2 = 2, FEM_GPU_RULE_HEX_2x2x2 = 3,
    FEM_GPU_RULE_HEX_3x3x3 = 4, FEM_GPU_RULE_TRI_7 = 5, FEM_GPU_RULE_TET_4 = 6, FEM_GPU_RULE_TET_11 = 7,
    FEM_GPU_RULE_TRI_3 = 8
};
/* set kinds of fem_gpu_auto_integration_rule (fem::Element_Type) */
enum { FEM_GPU_SET_BULK = 0, FEM_GPU_SET_SIDESET = 1, FEM_GPU_SET_DOUBLE_SIDESET = 2 };
/* fem::Model_Type of CM_Struc_Linear_Isotropic */
enum { FEM_GPU_MODEL_PLANE_STRAIN = 0, FEM_GPU_MODEL_PLANE_STRESS = 1, FEM_GPU_MODEL_3D = 2 };
/* mtk::CellShape of the interpolation cells */
enum { FEM_GPU_SHAPE_RECTANGULAR = 0, FEM_GPU_SHAPE_GENERAL = 1 };
/* fem::IWG_Type subset (FEM/INT/src/IWG/cl_FEM_IWG_Factory.cpp:191-224, 463) */
enum {
    FEM_GPU_IWG_STRUC_LINEAR_BULK = 0,
    FEM_GPU_IWG_STRUC_LINEAR_NEUMANN = 1,
    FEM_GPU_IWG_STRUC_LINEAR_DIRICHLET_SYMMETRIC_NITSCHE = 2,
    FEM_GPU_IWG_STRUC_LINEAR_DIRICHLET_UNSYMMETRIC_NITSCHE = 3,
    FEM_GPU_IWG_STRUC_LINEAR_INTERFACE_SYMMETRIC_NITSCHE = 4,
    FEM_GPU_IWG_STRUC_LINEAR_INTERFACE_UNSYMMETRIC_NITSCHE = 5,
    FEM_GPU_IWG_STRUC_LINEAR_VW_GHOST = 6,   /* with SP_Ghost_Virtual_Work */
    FEM_GPU_IWG_GHOST_NORMAL_FIELD = 7       /* with SP_Ghost_Displacement */
};
/* flags */
enum {
    FEM_GPU_HOST_BUFFERS = 1u,      /* pointers are host memory                 */
    FEM_GPU_NO_JACOBIAN = 2u,       /* fem_gpu_assemble: residual only          */
    FEM_GPU_NO_RESIDUAL = 4u,       /* fem_gpu_assemble: Jacobian only          */
    FEM_GPU_ASYNC = 16u,            /* batched assembly: return without waiting
                                       for the device status (fem_gpu_check_status) */
    FEM_GPU_ACCUMULATE = 8u         /* do not zero csr_vals / rhs first         */
};

typedef struct fem_gpu_ctx fem_gpu_ctx;

/* Lagrange interpolation mesh with the HMR extraction rows of its nodes.
   Node n interpolates the B-spline bases t_bases[t_offsets[n] .. t_offsets[n+1])
   with weights t_weights[...] (mtk::Vertex interpolation of the HMR
   T-matrix).  Host pointers; copied by fem_gpu_create. */
typedef struct fem_gpu_mesh_desc {
    int32_t spatial_dim;          /* 2 or 3 */
    int32_t ip_cell_type;         /* FEM_GPU_CELL_QUAD4 (2D) or FEM_GPU_CELL_HEX8 (3D) */
    int32_t cell_shape;           /* FEM_GPU_SHAPE_* */
    int32_t reserved;
    int64_t num_nodes;
    const double* node_coords;    /* num_nodes x spatial_dim */
    int64_t num_cells;
    const int32_t* cell_nodes;    /* num_cells x nodes per cell */
    int64_t num_bases;            /* B-spline basis index range */
    const int64_t* t_offsets;     /* num_nodes + 1 */
    const int32_t* t_bases;
    const double* t_weights;
} fem_gpu_mesh_desc;

/* Bulk set: IWG_Isotropic_Struc_Linear_Bulk with CM_Struc_Linear_Isotropic
   over clusters (one interpolation cell each).  ig_offsets == NULL means
   trivial clusters (the integration cell is the interpolation cell);
   otherwise cluster c integrates IG cells [ig_offsets[c], ig_offsets[c+1])
   with ig_coords / ig_param_coords (vertices x dim, node-major) giving the
   physical and IP-parametric vertex coordinates.
   A set of any kind may be empty (num_clusters / num_sides == 0, its arrays
   may then be NULL): it keeps its set index and does no work. */
typedef struct fem_gpu_bulk_set_desc {
    int32_t iwg_type;             /* FEM_GPU_IWG_STRUC_LINEAR_BULK */
    int32_t ig_cell_type;         /* FEM_GPU_CELL_* */
    int32_t integration_rule;     /* FEM_GPU_RULE_* */
    int32_t model_type;           /* FEM_GPU_MODEL_* */
    int64_t num_clusters;
    const int32_t* cluster_ip_cell;
    const int64_t* ig_offsets;
    const double* ig_coords;
    const double* ig_param_coords;
    const double* youngs_modulus; /* per cluster (E0 when node_density is given) */
    double poisson_ratio;
    /* optional SIMP-style material: E(x) = youngs_modulus * rho(x)^density_exponent
       with rho interpolated at each Gauss point from this nodal field (one value
       per mesh node), as the reference's density-dependent Young's modulus
       property (EXA/optimization/SIMP/SIMP.cpp:43-51).  NULL = constant E. */
    const double* node_density;
    double density_exponent;
    /* optional, cut clusters: IG vertex id of every integration-cell vertex
       ([ig][nodes]; ids into the table of fem_gpu_set_ig_vertices) -- needed
       for the shape sensitivities only */
    const int32_t* ig_vertex_ids;
    /* the IWG's (and strain-energy IQI's) "Thickness" property: w* is
       multiplied by it (FEM/INT/src/IWG/cl_FEM_IWG_Isotropic_Struc_Linear_
       Bulk.cpp:84-85); 0 = no Thickness property (factor 1) */
    double thickness;
} fem_gpu_bulk_set_desc;

/* Side set on interpolation-cell facets (trivial side clusters):
   Neumann traction (value = traction vector) or Nitsche Dirichlet
   (value = prescribed displacement, gamma = alpha * E / h). */
typedef struct fem_gpu_side_set_desc {
    int32_t iwg_type;
    int32_t integration_rule;     /* BAR_3 for quad edges, QUAD_2x2 for hex faces */
    int32_t model_type;
    int32_t reserved;
    int64_t num_sides;
    const int32_t* side_ip_cell;
    const int32_t* side_ordinal;  /* mtk side ordinal of the facet */
    const double* youngs_modulus; /* per side */
    double poisson_ratio;
    double nitsche_alpha;
    double value[3];
    /* "Thickness" property of the Neumann and Dirichlet IWGs: w* is
       multiplied by it (..._Neumann.cpp:66-67, ..._Dirichlet.cpp:103-104);
       0 = no Thickness property (factor 1) */
    double thickness;
    /* Dirichlet IWGs: the "Select" property, a spatial_dim x spatial_dim
       row-major matrix M that projects the prescribed components (rollers:
       diag(1,0) clamps x only; ..._Dirichlet.cpp:66-81, 107-116); NULL = the
       identity.  Copied by fem_gpu_add_side_set.  Neumann sets ignore it. */
    const double* select_matrix;
} fem_gpu_side_set_desc;

/* Double-sided set: the Nitsche interface (IWG_Isotropic_Struc_Linear_
   Interface, FEM/INT/src/IWG/cl_FEM_IWG_Isotropic_Struc_Linear_Interface.cpp:
   51-386, with SP_Nitsche_Interface, SP/cl_FEM_SP_Nitsche_Interface.cpp:51-97)
   or the face-oriented virtual-work ghost penalty (IWG_Isotropic_Struc_Linear_
   Virtual_Work_Ghost, ..._Virtual_Work_Ghost.cpp:50-244, with
   SP_Ghost_Virtual_Work, SP/cl_FEM_SP_Ghost_Virtual_Work.cpp:30-38) or the
   normal-derivative ghost penalty (IWG_Ghost_Normal_Field, FEM/INT/src/IWG/
   cl_FEM_IWG_Ghost_Normal_Field.cpp:36-233, order 1, with
   SP_Ghost_Displacement, SP/cl_FEM_SP_Ghost_Displacement.cpp:51-63: gamma =
   alpha h E, E = leader_youngs_modulus as its Material property) over the
   facets of one leader / follower pair of IP cells (mtk::Double_Side_Cluster,
   Element_Double_Sideset, FEM/INT/src/ELEM/cl_FEM_Element_Double_Sideset.cpp:
   142-347).  Each equation object is one cluster: a list of facets given by
   their vertex coordinates and the vertices' parametric coordinates in the
   leader and in the follower IP cell (same vertex order).  The facet normal
   of that vertex order (TRI3: (x0-x2) x (x1-x2); QUAD4: t1 x t2) points out of
   the leader.  Interface volumes V_L / V_F of the Nitsche parameter are the
   measures of the bulk clusters on the leader / follower IP cells; the ghost
   element size is the side length measure of the cluster's facets. */
typedef struct fem_gpu_double_side_set_desc {
    int32_t iwg_type;             /* INTERFACE_SYMMETRIC / _UNSYMMETRIC_NITSCHE, VW_GHOST or GHOST_NORMAL_FIELD */
    int32_t facet_cell_type;      /* FEM_GPU_CELL_TRI3 or FEM_GPU_CELL_QUAD4 (3D only) */
    int32_t integration_rule;     /* TRI_3 / TRI_7 for triangles, QUAD_2x2 for quads */
    int32_t model_type;           /* FEM_GPU_MODEL_3D */
    int64_t num_clusters;
    const int32_t* leader_ip_cell;
    const int32_t* follower_ip_cell;
    const int64_t* facet_offsets;          /* [num_clusters+1] */
    const double* facet_coords;            /* [facets][vertices][3] */
    const double* leader_param_coords;     /* [facets][vertices][3] */
    const double* follower_param_coords;   /* [facets][vertices][3] */
    const double* leader_youngs_modulus;   /* [num_clusters] */
    const double* follower_youngs_modulus; /* [num_clusters] */
    double poisson_ratio;
    double alpha;                 /* Nitsche interface or ghost penalty parameter */
    const int32_t* facet_vertex_ids;       /* optional [facets][vertices], as ig_vertex_ids */
} fem_gpu_double_side_set_desc;

typedef struct fem_gpu_pcg_opts {
    double rel_tol;               /* on ||b - A x|| / ||b|| */
    int32_t max_iter;
    int32_t preconditioner;       /* 0 none, 1 Jacobi */
} fem_gpu_pcg_opts;

typedef struct fem_gpu_pcg_report {
    int32_t iterations;
    int32_t converged;
    double rel_residual;
    double seconds;
} fem_gpu_pcg_report;

/* ---- library ------------------------------------------------------------ */
int32_t fem_gpu_abi_version(void);
/* The reference's automatic integration rule, Set::get_auto_integration_order
   (FEM/INT/src/CORE/cl_FEM_Set.cpp:2983-3185): by set kind (FEM_GPU_SET_*),
   the geometry of the integration cells (bulk: QUAD4, HEX8, TRI3, TET4;
   sides: LINE2 or QUAD4 facets; double-sided: TRI3 or QUAD4 facets) and the
   interpolation order of the interpolation cells (1 linear, 2 quadratic,
   3 cubic).  FEM_GPU_UNSUPPORTED when the reference's choice is not one of
   this library's rules (e.g. TET_35 for quadratic tetrahedra). */
fem_gpu_status fem_gpu_auto_integration_rule(int32_t set_kind, int32_t cell_type, int32_t interpolation_order,
                                             int32_t* rule);
const char* fem_gpu_status_string(fem_gpu_status s);
/* number of CUDA devices (0 without a GPU; never fails) */
int32_t fem_gpu_device_count(void);

/* ---- HMR-equivalent uniform level-0 mesh (host only) ---------------------- */
typedef struct fem_hmr_mesh fem_hmr_mesh;
fem_gpu_status fem_hmr_uniform_mesh(int32_t spatial_dim, const int32_t* num_elements, const double* lengths,
                                    int32_t bspline_order, fem_hmr_mesh** out);
fem_gpu_status fem_hmr_mesh_sizes(const fem_hmr_mesh* m, int64_t* num_nodes, int64_t* num_cells,
                                  int64_t* num_bases, int64_t* t_nnz);
fem_gpu_status fem_hmr_mesh_arrays(const fem_hmr_mesh* m, double* node_coords, int32_t* cell_nodes,
                                   int64_t* t_offsets, int32_t* t_bases, double* t_weights);
fem_gpu_status fem_hmr_mesh_free(fem_hmr_mesh* m);

/* ---- refined (hierarchical) HMR meshes ----------------------------------------
   A graded tensor-product B-spline hierarchy with HMR's rules: ne domain
   elements per direction and max(staircase_buffer, order) padding elements
   around them (Parameters::get_padding_size, HMR/src/cl_HMR_Parameters.cpp:
   418-423); refinement as Background_Mesh_Base::perform_refinement
   (cl_HMR_Background_Mesh_Base.cpp:648-737: padding test of the queued domain
   elements within `padding_refinement` -- HMR's ceil(max polynomial / 2) --
   and the staircase buffer); basis states as BSpline_Mesh::
   determine_basis_state (cl_HMR_BSpline_Mesh.hpp:738-807); element T matrices
   as T_Matrix_Base::calculate_t_matrix, truncated or not (cl_HMR_T_Matrix_
   Base.cpp:41-248).  Element and basis indices are domain-relative (padding
   elements have negative indices); a level-l basis m has the support elements
   m - order .. m per direction. */
typedef struct fem_hmr_refined fem_hmr_refined;
fem_gpu_status fem_hmr_refined_create(int32_t spatial_dim, const int32_t* num_elements, const double* lengths,
                                      int32_t bspline_order, int32_t staircase_buffer, int32_t padding_refinement,
                                      fem_hmr_refined** out);
fem_gpu_status fem_hmr_refined_free(fem_hmr_refined* m);
/* one perform_refinement of the given active domain elements (levels[count],
   ijk[count][dim]) with the buffers above */
fem_gpu_status fem_hmr_refined_refine(fem_hmr_refined* m, int64_t count, const int32_t* levels, const int32_t* ijk);
/* the active domain elements in HMR's order (coarsest elements x fastest,
   each followed by its active descendants, children x fastest); NULL arrays =
   count only */
fem_gpu_status fem_hmr_refined_active_elements(const fem_hmr_refined* m, int64_t* count, int32_t* levels,
                                               int32_t* ijk);
/* the T matrix of one element: T[(order+1)^dim][ndof] row-major, rows in the
   element-local basis order of HMR's B-spline elements (HMR/src/cl_HMR_BSpline_
   Element_*.hpp), columns the active (truncated) bases that support the
   element, in calculate_t_matrix's order, with their level and ijk.  All
   output pointers NULL = size query (*ndof); capacity = columns of T. */
fem_gpu_status fem_hmr_refined_element_t_matrix(const fem_hmr_refined* m, int32_t level, const int32_t* ijk,
                                                int32_t truncate, int32_t capacity, int32_t* ndof, double* T,
                                                int32_t* dof_level, int32_t* dof_ijk);
/* The Lagrange mesh of the active domain elements (QUAD4 / HEX8 cells in the
   order of fem_hmr_refined_active_elements, nodes numbered by first visit)
   with the extraction row of every node over the active bases (ids ordered by
   level, then z, y, x): T_Matrix_Base::evaluate (cl_HMR_T_Matrix_Base.cpp:
   306-457).  Read it with fem_hmr_mesh_sizes / fem_hmr_mesh_arrays; it feeds
   fem_gpu_create like the uniform mesh (cells are axis-aligned bricks). */
fem_gpu_status fem_hmr_refined_mesh(const fem_hmr_refined* m, int32_t truncate, fem_hmr_mesh** out);
/* The same mesh with the element T matrices and the node rows evaluated on
   the GPU (one thread per element / per node; the refined elements of every
   level as sorted keys on the device).  The numbers equal the host's bit for
   bit: the T entries are exact dyadic fractions, and the node rows use the
   host's operations in its order. */
fem_gpu_status fem_hmr_refined_mesh_device(const fem_hmr_refined* m, int32_t truncate, fem_hmr_mesh** out);
/* T matrices of `count` elements (levels[count], domain-relative
   ijk[count][dim]) on the GPU: ndof[count]; T[count][(order+1)^dim][capacity]
   row-major, dof_level[count][capacity], dof_ijk[count][capacity][dim] as
   fem_hmr_refined_element_t_matrix gives them; all three NULL = size query
   (ndof only).  FEM_GPU_BAD_ARG when an element has more than `capacity`
   columns (ndof still set). */
fem_gpu_status fem_hmr_refined_element_t_matrices_device(const fem_hmr_refined* m, int32_t truncate, int64_t count,
                                                         const int32_t* levels, const int32_t* ijk, int32_t capacity,
                                                         int32_t* ndof, double* T, int32_t* dof_level,
                                                         int32_t* dof_ijk);

/* ---- XFEM decomposition of a uniform level-0 HEX8 mesh (host only) -------
   Input of the cut-cell path, standing in for the reference's XTK
   (XTK/src/cl_XTK_Model.cpp:690 decompose; 24-tet regular subdivision,
   cl_XTK_Regular_Subdivision_Interface.hpp:225; conformal cut along the
   linear level set; Heaviside enrichment, cl_XTK_Enrichment.cpp:1148-2362;
   ghost facets, cl_XTK_Ghost_Stabilization.cpp:45).  node_phi: level set at
   the (n0+1)(n1+1)(n2+1) background nodes (i fastest); phase 1 where
   phi < 0.  The enriched IP mesh (unzipped vertices, enriched extraction
   rows) feeds fem_gpu_mesh_desc; the clusters feed the bulk and
   double-sided sets.  IG vertex kinds: 0 background node (parents[0] = node),
   1 face centre (parents[0..3] = its corner nodes), 2 cell centre
   (parents[0..7]), 3 intersection on the IG edge parents[0] -> parents[1]
   (IG vertex ids, value = edge coordinate t); kinds 0-2 carry phi. */
typedef struct fem_xtk_model fem_xtk_model;
typedef struct fem_xtk_sizes {
    int64_t num_nodes, num_cells, num_bases, t_nnz;
    int64_t num_uncut[2], num_cut[2], num_ig_cells[2];
    int64_t num_interface, num_interface_facets;
    int64_t num_ghost[2];
    int64_t num_ig_vertices;
} fem_xtk_sizes;
fem_gpu_status fem_xtk_decompose(const int32_t* num_elements, const double* lengths, int32_t bspline_order,
                                 const double* node_phi, fem_xtk_model** out);
/* the same decomposition computed on the GPU (classification, subdivision and
   cut, first-touch numbering by sorts, enrichment, unzipping, clusters); the
   model is identical to fem_xtk_decompose's, array for array.  Inputs host
   arrays; FEM_GPU_UNSUPPORTED for meshes above 2^29 / 3 nodes. */
fem_gpu_status fem_xtk_decompose_device(const int32_t* num_elements, const double* lengths, int32_t bspline_order,
                                        const double* node_phi, fem_xtk_model** out);
fem_gpu_status fem_xtk_get_sizes(const fem_xtk_model* m, fem_xtk_sizes* sizes);
/* any output pointer may be NULL; sizes as reported by fem_xtk_get_sizes */
fem_gpu_status fem_xtk_get_ip_mesh(const fem_xtk_model* m, double* node_coords, int32_t* cell_nodes,
                                   int64_t* t_offsets, int32_t* t_bases, double* t_weights,
                                   int32_t* cell_background, int32_t* cell_phase);
/* per phase: uncut enriched cells, cut enriched cells and their TET4
   integration cells (coords / IP-parametric coords [ig][4][3], IG vertex ids) */
fem_gpu_status fem_xtk_get_bulk(const fem_xtk_model* m, int32_t phase, int32_t* uncut_cells, int32_t* cut_cells,
                                int64_t* ig_offsets, double* ig_coords, double* ig_param, int32_t* ig_vertices);
/* interface clusters: leader = phase-0 cell, follower = phase-1 cell of one
   background cell; TRI3 facets [f][3][3] (same parametric coords both sides) */
fem_gpu_status fem_xtk_get_interface(const fem_xtk_model* m, int32_t* leader, int32_t* follower,
                                     int64_t* offsets, double* coords, double* param, int32_t* vertices);
/* ghost clusters of one phase: one QUAD4 face [4][3] each */
fem_gpu_status fem_xtk_get_ghost(const fem_xtk_model* m, int32_t phase, int32_t* leader, int32_t* follower,
                                 double* coords, double* leader_param, double* follower_param);
fem_gpu_status fem_xtk_get_vertices(const fem_xtk_model* m, int32_t* kind, int32_t* parents, double* coords,
                                    double* value);
void fem_xtk_free(fem_xtk_model* m);

/* ---- model ------------------------------------------------------------- */
fem_gpu_status fem_gpu_create(const fem_gpu_mesh_desc* mesh, fem_gpu_ctx** out);
fem_gpu_status fem_gpu_destroy(fem_gpu_ctx* ctx);
/* cudaStream_t passed as void*.  Without this call the context creates its
   own non-blocking stream; after it, every call is ordered on the given
   stream (NULL selects the CUDA legacy default stream). */
fem_gpu_status fem_gpu_set_stream(fem_gpu_ctx* ctx, void* stream);
fem_gpu_status fem_gpu_add_bulk_set(fem_gpu_ctx* ctx, const fem_gpu_bulk_set_desc* desc, int32_t* set_index);
fem_gpu_status fem_gpu_add_side_set(fem_gpu_ctx* ctx, const fem_gpu_side_set_desc* desc, int32_t* set_index);
/* interface / ghost set; element adofs are the leader's per-type lists
   followed by the follower's (Equation_Object::get_equation_obj_dof_ids over
   its two pdof systems, FEM/MSI/src/cl_MSI_Equation_Object.cpp:506-554) */
fem_gpu_status fem_gpu_add_double_side_set(fem_gpu_ctx* ctx, const fem_gpu_double_side_set_desc* desc,
                                           int32_t* set_index);
/* host-side MSI work (adof numbering, element T, sparsity, scatter maps)
   plus the upload of everything the kernels read */
fem_gpu_status fem_gpu_finalize(fem_gpu_ctx* ctx);
/* like fem_gpu_finalize but host side only (no device allocation) */
fem_gpu_status fem_gpu_finalize_host(fem_gpu_ctx* ctx);

fem_gpu_status fem_gpu_get_sizes(const fem_gpu_ctx* ctx, int64_t* num_adofs, int64_t* nnz, int32_t* num_sets);
fem_gpu_status fem_gpu_get_num_equation_objects(const fem_gpu_ctx* ctx, int32_t set, int64_t* count);
fem_gpu_status fem_gpu_get_max_element_adofs(const fem_gpu_ctx* ctx, int32_t set, int32_t* n);
/* CSR graph of the assembled operator (rowptr: num_adofs+1, colidx: nnz) */
fem_gpu_status fem_gpu_build_graph(fem_gpu_ctx* ctx, int32_t* rowptr, int32_t* colidx, uint32_t flags);
/* element adof ids (host pointer, capacity >= max element adofs) */
fem_gpu_status fem_gpu_get_element_topology(const fem_gpu_ctx* ctx, int32_t set, int64_t eq, int32_t* ids,
                                            int32_t* n);
/* element operators of equation objects [first, first+count) of a set:
   K_colmajor: count x nmax x nmax, R: count x nmax (nmax = max element adofs
   of the set; smaller elements are zero padded).  u_adof: full solution
   vector (may be NULL for zero). */
fem_gpu_status fem_gpu_element_matrices(fem_gpu_ctx* ctx, int32_t set, int64_t first, int64_t count,
                                        const double* u_adof, double* K_colmajor, double* R, uint32_t flags);
/* fill_matrix_and_RHS: csr_vals (nnz) and rhs (num_adofs) = residual R(u) */
fem_gpu_status fem_gpu_assemble(fem_gpu_ctx* ctx, const double* u_adof, double* csr_vals, double* rhs,
                                uint32_t flags);
/* fill_matrix_and_RHS for every equation object of every bulk and
   double-sided set in ONE persistent launch (uneven clusters: uncut cells,
   cut clusters of 4 to hundreds of integration points, interface and ghost
   clusters), work items taken from a device queue in decreasing cost order,
   clusters above the split size cut into integration-point ranges.  The
   zero-fill, the queue reset, the persistent kernel and the boundary side
   sets are one CUDA graph, captured on the first call for a (u, vals, rhs)
   triple and replayed afterwards.  Device buffers only. */
fem_gpu_status fem_gpu_assemble_batched(fem_gpu_ctx* ctx, const double* u_adof, double* csr_vals, double* rhs,
                                        uint32_t flags);
/* waits for the context's stream and reports a non-finite element operator
   flagged by the kernels since the last check */
fem_gpu_status fem_gpu_check_status(fem_gpu_ctx* ctx);
/* autotuner of the batched launch: times CTA width x split size on the
   model's own clusters and keeps the fastest (setup-time, optional) */
fem_gpu_status fem_gpu_autotune_batched(fem_gpu_ctx* ctx, int32_t* warps, int32_t* split_points, double* ms);
fem_gpu_status fem_gpu_set_batched_config(fem_gpu_ctx* ctx, int32_t warps, int32_t split_points);
/* matrix-free Jacobian-vector product y = K x (no CSR) */
fem_gpu_status fem_gpu_apply(fem_gpu_ctx* ctx, const double* x, double* y, uint32_t flags);
/* preconditioned CG on a CSR operator built by fem_gpu_assemble */
fem_gpu_status fem_gpu_pcg(fem_gpu_ctx* ctx, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                           const double* b, double* x, const fem_gpu_pcg_opts* opts, fem_gpu_pcg_report* report,
                           uint32_t flags);
/* PCG for callers that cannot allocate device memory during the solve
   (host callbacks, real-time sections, frameworks with a fixed device
   memory budget).  No counterpart in the reference.  Same algorithm and
   arguments as fem_gpu_pcg, but the work vectors live in one fixed-size
   device array of the library (systems up to 131072 rows; larger ones are
   rejected with FEM_GPU_BAD_ARG, nothing allocated).  Calls no cudaMalloc /
   cudaFree.  fem_gpu_finalize resolves the array's device address on the
   current device, which loads the module that holds the array; after
   fem_gpu_finalize_host alone, the first call on a device does it (make that
   first call before any stream capture).  All calls share the array: calls
   that overlap on the GPU race. */
fem_gpu_status fem_gpu_pcg_noalloc(fem_gpu_ctx* ctx, const int32_t* rowptr, const int32_t* colidx,
                                   const double* vals, const double* b, double* x, const fem_gpu_pcg_opts* opts,
                                   fem_gpu_pcg_report* report, uint32_t flags);
/* Jacobi-PCG that copies the iterate x into snaps (device, max_snaps x
   num_adofs doubles) after every `every` iterations until convergence. */
fem_gpu_status fem_gpu_pcg_snapshots(fem_gpu_ctx* ctx, const int32_t* rowptr, const int32_t* colidx,
                                     const double* vals, const double* b, double* x, const fem_gpu_pcg_opts* opts,
                                     fem_gpu_pcg_report* report, int32_t every, double* snaps, int32_t max_snaps,
                                     int32_t* n_snaps);

/* ---- shape sensitivities (adjoint) ---------------------------------------
   The integration mesh of the cut clusters and interface facets as a table of
   IG vertices (the fem_xtk_get_vertices layout): kind 0 background node
   (parents[0] = node), 1 face centre (parents[0..3]), 2 cell centre
   (parents[0..7]), 3 intersection on the IG edge parents[0] -> parents[1]
   (IG vertex ids) at edge coordinate t: x = x_p0 + t (x_p1 - x_p0).  The
   design variables of the path are the level-set coefficients p; the
   intersection coordinates t carry all the dependence (GEN's
   Intersection_Node_Linear, GEN/src/PDV/cl_GEN_Intersection_Node_Linear.cpp:
   46-57, and Intersection_Node_Level_Set::append_dcoordinate_dadv,
   cl_GEN_Intersection_Node_Level_Set.cpp:43-100).  Host arrays. */
fem_gpu_status fem_gpu_set_ig_vertices(fem_gpu_ctx* ctx, int64_t num_vertices, const int32_t* kind,
                                       const int32_t* parents, const double* coords, const double* value);
/* new edge coordinates t of the intersection vertices (same topology):
   rewrites the coordinates and IP-parametric coordinates of every cut
   cluster's integration cells and every interface facet (rectangular IP
   cells), on the host and the device.  t: host [num_vertices] (entries of
   other kinds are ignored). */
fem_gpu_status fem_gpu_update_ig_vertices(fem_gpu_ctx* ctx, const double* t);
/* strain energy of the bulk sets, Q = sum 1/2 w* flux . strain
   (IQI_Strain_Energy::compute_QI, FEM/INT/src/IQI/cl_FEM_IQI_Strain_Energy.cpp:
   40-120), and dQ/du = K_bulk u (device buffers; q: host scalar) */
fem_gpu_status fem_gpu_strain_energy(fem_gpu_ctx* ctx, const double* u, double* dqdu, double* q);
/* adjoint shape sensitivity at the intersection vertices:
   G[v] = d/dt_v ( Q(u, t) - lambda^T R(u, t) ) for the cut clusters (bulk
   strain energy and residual) and the interface clusters (residual and the
   SP_Nitsche_Interface cluster measures), exact (forward-mode dual numbers
   over each integration cell's / facet's vertices).  With K^T lambda = dQ/du
   this is dQ/dt (Interpolation_Element::compute_dQIdp_explicit_implicit,
   FEM/INT/src/ELEM/cl_FEM_Interpolation_Element.cpp:820-948; the reference
   differentiates the residual by finite differences of the IG vertex
   coordinates, cl_FEM_IWG.cpp:2997-3154).  u, lambda: device adof vectors;
   G: device [num_vertices], overwritten. */
fem_gpu_status fem_gpu_drdp_adjoint(fem_gpu_ctx* ctx, const double* u, const double* lambda, double* G);
/* chain to the level-set coefficients: dqdp[j] = sum_v G[v] dt_v/dp_j with
   t = phi_0 / (phi_0 - phi_1) on the parents' level set, derived parents the
   mean of their background nodes, phi at a background node = sum_j
   tmat[node][k] p_(cols[node][k]) (width entries per node, e.g. the cubic
   B-spline field of fem_gen_bspline_tmatrix).  G, dqdp: device; cols, tmat:
   host [num_background_nodes][width] (validated and stored as by
   fem_gpu_set_level_set_field), or both NULL for the stored field, whose
   sizes must then match; dqdp overwritten. */
fem_gpu_status fem_gen_dqdp(fem_gpu_ctx* ctx, const double* G, int64_t num_background_nodes, int32_t width,
                            const int32_t* cols, const double* tmat, int64_t num_coefs, double* dqdp);
/* the design variables' level-set field, validated (every id in
   [0, num_coefs)) and kept on the device for the whole optimisation, so that
   each fem_gen_dqdp call moves no table (the reference's design-variable
   interface keeps the field's coefficient map the same way,
   FEM/MSI/src/cl_MSI_Design_Variable_Interface.hpp:35-240).  cols, tmat: host
   [num_background_nodes][width]. */
fem_gpu_status fem_gpu_set_level_set_field(fem_gpu_ctx* ctx, int64_t num_background_nodes, int32_t width,
                                           const int32_t* cols, const double* tmat, int64_t num_coefs);
/* tensor-product B-spline field of `order` on a uniform grid of
   num_coefs[d] = n_d + order coefficients over [0, lengths[d]] (HMR
   numbering, i fastest; BSpline_Field::get_dfield_dadvs,
   GEN/src/ADV/fields/cl_GEN_BSpline_Field.cpp:165): the (order+1)^3 basis
   values and coefficient ids at each point.  cols, vals: [num_points][(order+1)^3]. */
fem_gpu_status fem_gen_bspline_tmatrix(const int32_t* num_coefs, const double* lengths, int32_t order,
                                       int64_t num_points, const double* points, int32_t* cols, double* vals);

/* ---- learned coarse-grid correction (config 5) ---------------------------
   A 4-layer 3D convolution net (4 -> 32 -> 32 -> 32 -> 3 channels, 3x3x3,
   no biases, ReLU) on a coarse node grid of n^3 voxels; BF16 weights and
   activations, FP32 accumulation, tensor-core forward / data gradient, FP32
   weight gradient, Adam.  Weights (host FP32): layers concatenated, each
   [27][cout][cin], tap k = dx+1 + 3 (dy+1) + 9 (dz+1).  Inputs channels-last
   FP32 [samples][n^3][4], outputs / targets [samples][n^3][3]. */
typedef struct fem_cnn fem_cnn;
int64_t fem_cnn_num_weights(void);
fem_gpu_status fem_cnn_create(int32_t n, int32_t batch_max, uint64_t seed, fem_cnn** out);
fem_gpu_status fem_cnn_destroy(fem_cnn* cnn);
fem_gpu_status fem_cnn_set_weights(fem_cnn* cnn, const float* weights);
fem_gpu_status fem_cnn_get_weights(const fem_cnn* cnn, float* weights);
fem_gpu_status fem_cnn_forward(fem_cnn* cnn, const float* in4, int32_t samples, float* out3);
/* output scale sigma of the learned correction (fem_gpu_fcg applies
   s * sigma * f); training targets are divided by the same sigma */
fem_gpu_status fem_cnn_set_output_scale(fem_cnn* cnn, double scale);
double fem_cnn_get_output_scale(const fem_cnn* cnn);
/* mean-squared loss over the 3 output channels and its weight gradient */
fem_gpu_status fem_cnn_loss_grad(fem_cnn* cnn, const float* in4, const float* target3, int32_t samples, double* loss,
                                 float* grad);
fem_gpu_status fem_cnn_train_step(fem_cnn* cnn, const float* in4, const float* target3, int32_t samples, float lr,
                                  double* loss);

/* device time (ms per call, CUDA events on the net's stream, reps calls each)
   of the forward convolution of every layer, ms[0..3], and of the data
   gradients of layers 1..3, ms[4..6], on `samples` samples; the activation
   buffers hold whatever the last call left (their contents do not change the
   time).  No counterpart in the reference: it measures this library's own
   convolution kernels. */
fem_gpu_status fem_cnn_profile(fem_cnn* cnn, int32_t samples, int32_t reps, double* ms);
/* coarse input for a fine residual (node grid nf^3, coarsening factor F):
   channels 0..2 = R r / ||R r||, channel 3 = log10(restricted density) / 3;
   ||R r|| is reduced on the device into a library-wide accumulator, so calls
   must not overlap */
fem_gpu_status fem_lpc_restrict(int32_t nf, int32_t factor, const double* r, const double* node_density, float* coarse4,
                                double* scale);
/* training target: fine field injected at the coarse nodes, / scale */
fem_gpu_status fem_lpc_inject(int32_t nf, int32_t factor, const double* e, double scale, float* target3);
/* z += scale * P c: trilinear prolongation of a coarse 3-channel field
   (channels-last [nc^3][3], nc = (nf - 1) / factor + 1) into a fine
   type-major adof vector */
fem_gpu_status fem_lpc_prolong_add(int32_t nf, int32_t factor, const float* coarse3, double scale, double* z);
/* coarse3 = scale * P^T fine (the transpose of fem_lpc_prolong_add; the
   gradient of a fine objective with respect to the net's output) */
fem_gpu_status fem_lpc_prolong_transpose(int32_t nf, int32_t factor, const double* fine, double scale,
                                         float* coarse3);
/* y = A x on a CSR operator of n rows (device buffers) */
fem_gpu_status fem_gpu_spmv(int64_t n, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                            const double* x, double* y);
/* truncated flexible CG, FCG(8), with M(r) = D^-1 r + P sigma f(R r / s) s
   (cnn == NULL: M = D^-1); Jacobi-PCG is the fallback on breakdown or
   stagnation and the final residual is recomputed from b - A x.  Device
   buffers. */
fem_gpu_status fem_gpu_fcg(fem_gpu_ctx* ctx, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                           const double* b, double* x, fem_cnn* cnn, int32_t factor, const double* node_density,
                           const fem_gpu_pcg_opts* opts, fem_gpu_pcg_report* report, int32_t* used_fallback);

/* ---- geometric multigrid preconditioner ----------------------------------
   Replaces the reference's PETSc PCMG preconditioner
   (Preconditioner_PETSc::build_multigrid_preconditioner,
   SOL/DLA/src/cl_DLA_Preconditioner_PETSc.cpp:77-345, prolongations from
   Geometric_Multigrid, SOL/DLA/src/cl_DLA_Geometric_Multigrid.cpp:47-121):
   V-cycle with Galerkin coarse operators P^T A P, the linear B-spline
   two-scale relation (trilinear interpolation, factor 2 per level) as P,
   Chebyshev-accelerated point-Jacobi smoothing (the reference smooths with
   SOR) and a dense inverse on the coarsest grid (the reference uses LU).
   For 3D models on a cubic node grid of n^3 nodes (adof f n^3 + node, node =
   x + n (y + n z)) whose operator is the symmetric 27-point nodal stencil of
   linear B-splines (FEM_GPU_BAD_ARG otherwise); n - 1 must halve down to
   <= coarse_max.  Work is issued on the
   legacy default stream. */
typedef struct fem_mg fem_mg;
typedef struct fem_mg_opts {
    int32_t coarse_max;   /* coarsest node grid edge, 3..9 (default 5) */
    int32_t degree;       /* Chebyshev degree of pre- and post-smoothing, 1..8 (2) */
    double lo_frac;       /* smoothing interval [lo_frac, hi_frac] * lambda_max(D^-1 A) (0.1, 1.1) */
    double hi_frac;
    int32_t power_iters;  /* power iterations for lambda_max (12) */
    int32_t fp32_levels;  /* levels 0..fp32_levels-1 (never the coarsest) smooth in FP32, with an FP32
                             stencil copy and FP32 vectors (default 8: all but the coarsest) */
} fem_mg_opts;
fem_gpu_status fem_mg_default_opts(fem_mg_opts* opts);
/* builds the hierarchy from the assembled CSR (device); opts NULL = defaults */
fem_gpu_status fem_mg_create(fem_gpu_ctx* ctx, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                             const fem_mg_opts* opts, fem_mg** out);
fem_gpu_status fem_mg_destroy(fem_mg* mg);
int32_t fem_mg_num_levels(const fem_mg* mg);
double fem_mg_setup_seconds(const fem_mg* mg);
/* node grid edge and lambda_max(D^-1 A) of a level (lambda 0 on the coarsest) */
fem_gpu_status fem_mg_level_info(const fem_mg* mg, int32_t level, int32_t* n, double* lambda_max);
/* stencil of a level to host memory, [27][3][3][n^3] doubles (tap k =
   (dx+1) + 3 (dy+1) + 9 (dz+1), row component f, column component g) */
fem_gpu_status fem_mg_get_stencil(const fem_mg* mg, int32_t level, double* host_out);
/* one V-cycle z = V r (device vectors of num_adofs doubles) */
fem_gpu_status fem_mg_apply(fem_mg* mg, const double* r, double* z);
/* fem_gpu_fcg with the V-cycle in place of D^-1: M(r) = V r (+ the learned
   correction P sigma s f(R r / s) when cnn is given); same convergence test.  A learned
   correction that stalls the solve (4 iterations without a 10 % residual
   reduction) is switched off and the solve continues with the V-cycle alone
   (*used_fallback = 2); Jacobi-PCG stays the last fallback (*used_fallback = 1). */
fem_gpu_status fem_gpu_fcg_mg(fem_gpu_ctx* ctx, const int32_t* rowptr, const int32_t* colidx, const double* vals,
                              const double* b, double* x, fem_mg* mg, fem_cnn* cnn, int32_t factor,
                              const double* node_density, const fem_gpu_pcg_opts* opts, fem_gpu_pcg_report* report,
                              int32_t* used_fallback);
/* truncation depth m of FCG(m) (1..16, default 8) and the stagnation window
   (iterations without a 10 % residual reduction before the Jacobi-PCG
   fallback, default 200) of fem_gpu_fcg / fem_gpu_fcg_mg; process-wide */
fem_gpu_status fem_gpu_fcg_config(int32_t depth, int32_t window);

/* autotuner: times every kernel variant of each bulk set on (up to
   max_elements, <= 0 = all) of its elements, assembling into scratch
   buffers, and keeps the fastest per set.  Setup-time call; optional. */
fem_gpu_status fem_gpu_autotune(fem_gpu_ctx* ctx, int64_t max_elements);
fem_gpu_status fem_gpu_get_variant(const fem_gpu_ctx* ctx, int32_t set, int32_t* variant, double* tuned_ms,
                                   const char** name);
fem_gpu_status fem_gpu_set_variant(fem_gpu_ctx* ctx, int32_t set, int32_t variant);
/* in-run FP64 peak probe (FMA chains on every SM, CUDA-event timed), the
   roofline denominator of the FP64-bound element kernels */
fem_gpu_status fem_gpu_probe_fp64_tflops(int32_t iters, double* tflops);
/* FP64 tensor-core (DMMA m8n8k4) throughput, alone (mixed = 0) or with half
   of the warps issuing FP64 FMA chains at the same time (mixed = 1) */
fem_gpu_status fem_gpu_probe_dmma_tflops(int32_t iters, int32_t mixed, double* tflops);
/* number of kernel launches issued by the context since creation */
int64_t fem_gpu_launch_count(const fem_gpu_ctx* ctx);
/* ---- field output (VIS) -----------------------------------------------------
   Nodal values of an adof field at the interpolation-mesh nodes, out[f][node]
   = sum over the node's extraction row of w u[f nu + rank] (device buffers;
   out: dim x num_nodes), the values VIS::Output_Manager::write_field
   (FEM/VIS/src/cl_VIS_Output_Manager.cpp:679-785) writes at the vertices. */
fem_gpu_status fem_gpu_nodal_field(fem_gpu_ctx* ctx, const double* u_adof, double* out);
/* Stress sigma = D eps(u) of bulk-set equation objects at IP-parametric points:
   CM_Struc_Linear::flux (FEM/INT/src/CM/cl_FEM_CM_Struc_Linear.cpp:280-302),
   as the reference's stress IQIs and field output evaluate it.  Point k is
   equation object eq[k] at xi[k*dim ...] (host arrays); flux[k*ncomp ...] in
   the model's Voigt order (3D: xx yy zz yz xz xy; plane strain: xx yy zz xy;
   plane stress: xx yy xy), *ncomp set.  u_adof and flux are device buffers,
   or host buffers with FEM_GPU_HOST_BUFFERS.  The Thickness property does not
   scale the stress. */
fem_gpu_status fem_gpu_element_flux(fem_gpu_ctx* ctx, int32_t set, int64_t count, const int64_t* eq, const double* xi,
                                    const double* u_adof, double* flux, int32_t* ncomp, uint32_t flags);
/* Exodus II file of one element block and nodal fields at one time step (the
   reference writes through mtk::Writer_Exodus, MTK/src/io/cl_MTK_Writer_Exodus.
   cpp:112-420, and the SEACAS library; here the netCDF classic 64-bit-offset
   format is written directly).  Host arrays: coords [num_nodes][dim],
   cell_nodes [num_cells][nodes_per_cell] 0-based, field_values
   [num_fields][num_nodes]; elem_type e.g. "HEX8", "QUAD4". */
fem_gpu_status fem_vis_write_exodus(const char* path, int32_t dim, int64_t num_nodes, const double* coords,
                                    int64_t num_cells, int32_t nodes_per_cell, const int32_t* cell_nodes,
                                    const char* elem_type, int32_t num_fields, const char* const* field_names,
                                    const double* field_values, double time);

/* last error text of the context (never NULL) */
const char* fem_gpu_last_error(const fem_gpu_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif
