"""ctypes binding of libfem_gpu.so (the C ABI declared in include/fem_gpu.h).

The shared library is built in-tree by ``moris_gb300/build.py``.  Loading
fails loudly when it is missing: there is no Python or CPU fallback for any
compute entry point.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libfem_gpu.so")

# the structures below follow include/fem_gpu.h of this ABI version
ABI_VERSION = 3

P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
U32 = C.c_uint32
D = C.c_double


class MeshDesc(C.Structure):
    _fields_ = [("spatial_dim", I32), ("ip_cell_type", I32), ("cell_shape", I32), ("reserved", I32),
                ("num_nodes", I64), ("node_coords", P), ("num_cells", I64), ("cell_nodes", P),
                ("num_bases", I64), ("t_offsets", P), ("t_bases", P), ("t_weights", P)]


class BulkSetDesc(C.Structure):
    _fields_ = [("iwg_type", I32), ("ig_cell_type", I32), ("integration_rule", I32), ("model_type", I32),
                ("num_clusters", I64), ("cluster_ip_cell", P), ("ig_offsets", P), ("ig_coords", P),
                ("ig_param_coords", P), ("youngs_modulus", P), ("poisson_ratio", D), ("node_density", P),
                ("density_exponent", D), ("ig_vertex_ids", P), ("thickness", D)]


class SideSetDesc(C.Structure):
    _fields_ = [("iwg_type", I32), ("integration_rule", I32), ("model_type", I32), ("reserved", I32),
                ("num_sides", I64), ("side_ip_cell", P), ("side_ordinal", P), ("youngs_modulus", P),
                ("poisson_ratio", D), ("nitsche_alpha", D), ("value", D * 3), ("thickness", D),
                ("select_matrix", P)]


class DoubleSideSetDesc(C.Structure):
    _fields_ = [("iwg_type", I32), ("facet_cell_type", I32), ("integration_rule", I32), ("model_type", I32),
                ("num_clusters", I64), ("leader_ip_cell", P), ("follower_ip_cell", P), ("facet_offsets", P),
                ("facet_coords", P), ("leader_param_coords", P), ("follower_param_coords", P),
                ("leader_youngs_modulus", P), ("follower_youngs_modulus", P), ("poisson_ratio", D), ("alpha", D),
                ("facet_vertex_ids", P)]


class XtkSizes(C.Structure):
    _fields_ = [("num_nodes", I64), ("num_cells", I64), ("num_bases", I64), ("t_nnz", I64),
                ("num_uncut", I64 * 2), ("num_cut", I64 * 2), ("num_ig_cells", I64 * 2),
                ("num_interface", I64), ("num_interface_facets", I64), ("num_ghost", I64 * 2),
                ("num_ig_vertices", I64)]


class PcgOpts(C.Structure):
    _fields_ = [("rel_tol", D), ("max_iter", I32), ("preconditioner", I32)]


class PcgReport(C.Structure):
    _fields_ = [("iterations", I32), ("converged", I32), ("rel_residual", D), ("seconds", D)]


class MgOpts(C.Structure):
    _fields_ = [("coarse_max", I32), ("degree", I32), ("lo_frac", D), ("hi_frac", D), ("power_iters", I32),
                ("fp32_levels", I32)]


# name -> (restype, argtypes); this list is also the ABI surface the tests
# check against include/fem_gpu.h
SIGNATURES = {
    "fem_gpu_abi_version": (I32, []),
    "fem_hmr_refined_create": (I32, [I32, P, P, I32, I32, I32, P]),
    "fem_hmr_refined_free": (I32, [P]),
    "fem_hmr_refined_refine": (I32, [P, I64, P, P]),
    "fem_hmr_refined_active_elements": (I32, [P, P, P, P]),
    "fem_hmr_refined_element_t_matrix": (I32, [P, I32, P, I32, I32, P, P, P, P]),
    "fem_hmr_refined_mesh": (I32, [P, I32, P]),
    "fem_hmr_refined_mesh_device": (I32, [P, I32, P]),
    "fem_hmr_refined_element_t_matrices_device": (I32, [P, I32, I64, P, P, I32, P, P, P, P]),
    "fem_gpu_auto_integration_rule": (I32, [I32, I32, I32, P]),
    "fem_gpu_status_string": (C.c_char_p, [I32]),
    "fem_gpu_device_count": (I32, []),
    "fem_hmr_uniform_mesh": (I32, [I32, P, P, I32, P]),
    "fem_hmr_mesh_sizes": (I32, [P, P, P, P, P]),
    "fem_hmr_mesh_arrays": (I32, [P, P, P, P, P, P]),
    "fem_hmr_mesh_free": (I32, [P]),
    "fem_gpu_create": (I32, [P, P]),
    "fem_gpu_destroy": (I32, [P]),
    "fem_gpu_set_stream": (I32, [P, P]),
    "fem_gpu_add_bulk_set": (I32, [P, P, P]),
    "fem_gpu_add_side_set": (I32, [P, P, P]),
    "fem_gpu_add_double_side_set": (I32, [P, P, P]),
    "fem_gpu_assemble_batched": (I32, [P, P, P, P, U32]),
    "fem_gpu_check_status": (I32, [P]),
    "fem_gpu_autotune_batched": (I32, [P, P, P, P]),
    "fem_gpu_set_batched_config": (I32, [P, I32, I32]),
    "fem_xtk_decompose": (I32, [P, P, I32, P, P]),
    "fem_xtk_decompose_device": (I32, [P, P, I32, P, P]),
    "fem_xtk_get_sizes": (I32, [P, P]),
    "fem_xtk_get_ip_mesh": (I32, [P, P, P, P, P, P, P, P]),
    "fem_xtk_get_bulk": (I32, [P, I32, P, P, P, P, P, P]),
    "fem_xtk_get_interface": (I32, [P, P, P, P, P, P, P]),
    "fem_xtk_get_ghost": (I32, [P, I32, P, P, P, P, P]),
    "fem_xtk_get_vertices": (I32, [P, P, P, P, P]),
    "fem_xtk_free": (None, [P]),
    "fem_gpu_set_ig_vertices": (I32, [P, I64, P, P, P, P]),
    "fem_gpu_update_ig_vertices": (I32, [P, P]),
    "fem_gpu_strain_energy": (I32, [P, P, P, P]),
    "fem_gpu_drdp_adjoint": (I32, [P, P, P, P]),
    "fem_gen_dqdp": (I32, [P, P, I64, I32, P, P, I64, P]),
    "fem_gpu_set_level_set_field": (I32, [P, I64, I32, P, P, I64]),
    "fem_gen_bspline_tmatrix": (I32, [P, P, I32, I64, P, P, P]),
    "fem_gpu_finalize": (I32, [P]),
    "fem_gpu_finalize_host": (I32, [P]),
    "fem_gpu_get_sizes": (I32, [P, P, P, P]),
    "fem_gpu_get_num_equation_objects": (I32, [P, I32, P]),
    "fem_gpu_get_max_element_adofs": (I32, [P, I32, P]),
    "fem_gpu_build_graph": (I32, [P, P, P, U32]),
    "fem_gpu_get_element_topology": (I32, [P, I32, I64, P, P]),
    "fem_gpu_element_matrices": (I32, [P, I32, I64, I64, P, P, P, U32]),
    "fem_gpu_assemble": (I32, [P, P, P, P, U32]),
    "fem_gpu_apply": (I32, [P, P, P, U32]),
    "fem_gpu_pcg": (I32, [P, P, P, P, P, P, P, P, U32]),
    "fem_gpu_pcg_noalloc": (I32, [P, P, P, P, P, P, P, P, U32]),
    "fem_gpu_pcg_snapshots": (I32, [P, P, P, P, P, P, P, P, I32, P, I32, P]),
    "fem_cnn_num_weights": (I64, []),
    "fem_cnn_create": (I32, [I32, I32, C.c_uint64, P]),
    "fem_cnn_destroy": (I32, [P]),
    "fem_cnn_set_weights": (I32, [P, P]),
    "fem_cnn_get_weights": (I32, [P, P]),
    "fem_cnn_forward": (I32, [P, P, I32, P]),
    "fem_cnn_set_output_scale": (I32, [P, D]),
    "fem_cnn_get_output_scale": (D, [P]),
    "fem_cnn_loss_grad": (I32, [P, P, P, I32, P, P]),
    "fem_cnn_train_step": (I32, [P, P, P, I32, C.c_float, P]),
    "fem_cnn_profile": (I32, [P, I32, I32, P]),
    "fem_lpc_restrict": (I32, [I32, I32, P, P, P, P]),
    "fem_lpc_inject": (I32, [I32, I32, P, D, P]),
    "fem_lpc_prolong_add": (I32, [I32, I32, P, D, P]),
    "fem_lpc_prolong_transpose": (I32, [I32, I32, P, D, P]),
    "fem_gpu_spmv": (I32, [I64, P, P, P, P, P]),
    "fem_gpu_fcg": (I32, [P, P, P, P, P, P, P, I32, P, P, P, P]),
    "fem_gpu_fcg_mg": (I32, [P, P, P, P, P, P, P, P, I32, P, P, P, P]),
    "fem_gpu_fcg_config": (I32, [I32, I32]),
    "fem_mg_default_opts": (I32, [P]),
    "fem_mg_create": (I32, [P, P, P, P, P, P]),
    "fem_mg_destroy": (I32, [P]),
    "fem_mg_num_levels": (I32, [P]),
    "fem_mg_setup_seconds": (D, [P]),
    "fem_mg_level_info": (I32, [P, I32, P, P]),
    "fem_mg_get_stencil": (I32, [P, I32, P]),
    "fem_mg_apply": (I32, [P, P, P]),
    "fem_gpu_autotune": (I32, [P, I64]),
    "fem_gpu_get_variant": (I32, [P, I32, P, P, P]),
    "fem_gpu_set_variant": (I32, [P, I32, I32]),
    "fem_gpu_probe_fp64_tflops": (I32, [I32, P]),
    "fem_gpu_probe_dmma_tflops": (I32, [I32, I32, P]),
    "fem_gpu_launch_count": (I64, [P]),
    "fem_gpu_last_error": (C.c_char_p, [P]),
    "fem_gpu_nodal_field": (I32, [P, P, P]),
    "fem_gpu_element_flux": (I32, [P, I32, I64, P, P, P, P, P, U32]),
    "fem_vis_write_exodus": (I32, [C.c_char_p, I32, I64, P, I64, I32, P, C.c_char_p, I32, P, P, D]),
}

_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libfem_gpu.so is not built (%s); run moris_gb300/build.py" % LIB_PATH)
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        if lib.fem_gpu_abi_version() != ABI_VERSION:
            raise RuntimeError("libfem_gpu.so has ABI version %d, these bindings expect %d; rebuild it"
                               % (lib.fem_gpu_abi_version(), ABI_VERSION))
        _lib = lib
    return _lib
