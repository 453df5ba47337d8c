"""ctypes mirror of the C ABI (include/*.h) and loaders for the shared libraries.

The structs below have the same members, order and C types as the reference
project's headers (include/mesh.h, dual_mesh.h, complex_matrix.h,
inductance.h, potential.h, lu.h, complex_lu.h), so a struct filled here can be
handed to the GPU library exactly as a C caller of the reference API would.
"""
import ctypes as C
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)

GPU_LIB_PATH = os.path.join(PKG_DIR, "libpeec_gb300.so")
MESH_LIB_PATH = os.path.join(PKG_DIR, "libpeec_mesh.so")

c_double_p = C.POINTER(C.c_double)
c_int_p = C.POINTER(C.c_int)
c_size_t_p = C.POINTER(C.c_size_t)


class Mesh(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_size_t), ("n_quads", C.c_size_t), ("n_edges", C.c_size_t),
        ("xyz", c_double_p), ("quads", c_int_p), ("edges", c_int_p),
        ("cell_edges", c_int_p), ("cell_edge_signs", c_int_p),
        ("edge_vectors", c_double_p), ("edge_lengths", c_double_p),
        ("edge_directions", c_double_p), ("edge_centers", c_double_p),
        ("cell_centers", c_double_p), ("cell_areas", c_double_p),
        ("cell_normals", c_double_p),
    ]


class QuadPatch(C.Structure):
    _fields_ = [("points", C.c_double * 12), ("owner_id", C.c_int), ("cell_id", C.c_int)]


class PatchList(C.Structure):
    _fields_ = [("patches", C.POINTER(QuadPatch)), ("count", C.c_size_t),
                ("capacity", C.c_size_t)]


class DualMesh(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_size_t), ("n_edges", C.c_size_t),
        ("node_patches", C.POINTER(PatchList)), ("edge_patches", C.POINTER(PatchList)),
        ("node_region_areas", c_double_p), ("edge_region_areas", c_double_p),
        ("node_region_centers", c_double_p), ("edge_region_centers", c_double_p),
    ]


class Complex(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class InductanceOptions(C.Structure):
    _fields_ = [("far_order", C.c_int), ("near_order", C.c_int),
                ("touching_order", C.c_int), ("self_order", C.c_int),
                ("near_factor", C.c_double), ("parallel_threads", C.c_int),
                ("direction_tolerance", C.c_double)]


class InductanceMatrix(C.Structure):
    _fields_ = [("n", C.c_size_t), ("data", c_double_p)]


class PotentialOptions(C.Structure):
    _fields_ = [("far_order", C.c_int), ("near_order", C.c_int),
                ("touching_order", C.c_int), ("self_order", C.c_int),
                ("near_factor", C.c_double), ("parallel_threads", C.c_int)]


class PotentialMatrix(C.Structure):
    _fields_ = [("n", C.c_size_t), ("data", c_double_p)]


class Matrix(C.Structure):
    _fields_ = [("rows", C.c_size_t), ("cols", C.c_size_t), ("data", c_double_p)]


class IncidenceMatrix(C.Structure):
    _fields_ = [("rows", C.c_size_t), ("cols", C.c_size_t), ("data", c_double_p)]


class ResistanceMatrix(C.Structure):
    _fields_ = [("n", C.c_size_t), ("diagonal", c_double_p)]


class LUOptions(C.Structure):
    _fields_ = [("parallel_threads", C.c_int), ("pivot_tolerance", C.c_double),
                ("parallel_threshold", C.c_size_t)]


class LUFactorization(C.Structure):
    _fields_ = [("n", C.c_size_t), ("data", c_double_p), ("pivots", c_size_t_p),
                ("swap_count", C.c_size_t), ("matrix_scale", C.c_double),
                ("factorized", C.c_int)]


class ComplexLUOptions(C.Structure):
    _fields_ = [("parallel_threads", C.c_int), ("pivot_tolerance", C.c_double),
                ("parallel_threshold", C.c_size_t)]


class ComplexLUFactorization(C.Structure):
    _fields_ = [("n", C.c_size_t), ("data", C.POINTER(Complex)), ("pivots", c_size_t_p),
                ("swap_count", C.c_size_t), ("matrix_scale", C.c_double),
                ("row_scale", c_double_p), ("column_scale", c_double_p),
                ("factorized", C.c_int)]


P = C.POINTER

# Every symbol the drop-in headers declare, with its ctypes signature.
# (name, restype, argtypes)
DROP_IN_SYMBOLS = [
    # incidence.h
    ("incidence_init", None, [P(IncidenceMatrix)]),
    ("incidence_free", None, [P(IncidenceMatrix)]),
    ("incidence_build", C.c_int, [P(Mesh), P(IncidenceMatrix)]),
    ("incidence_check_row_sum", C.c_double, [P(IncidenceMatrix)]),
    ("incidence_print_info", None, [P(IncidenceMatrix)]),
    ("incidence_build_APAT", C.c_int, [P(Mesh), P(PotentialMatrix), P(Matrix), C.c_int]),
    ("incidence_build_PAT", C.c_int, [P(Mesh), P(PotentialMatrix), P(Matrix), C.c_int]),
    ("incidence_build_AS", C.c_int, [P(IncidenceMatrix), P(PotentialMatrix), P(Matrix), C.c_int]),
    # matrix_export.h
    ("matrix_export_dense_mtx", C.c_int, [C.c_char_p, c_double_p, C.c_size_t, C.c_size_t]),
    ("matrix_export_incidence_mtx", C.c_int, [C.c_char_p, P(Mesh)]),
    ("matrix_export_resistance_mtx", C.c_int, [C.c_char_p, P(ResistanceMatrix)]),
    ("matrix_export_peec_set", C.c_int,
     [C.c_char_p, P(Mesh), P(InductanceMatrix), P(PotentialMatrix), P(Matrix), P(ResistanceMatrix)]),
    # quadrature.h
    ("gauss_legendre_rule", C.c_int, [C.c_int, c_double_p, c_double_p]),
    ("triangle_area", C.c_double, [c_double_p, c_double_p, c_double_p]),
    ("quad_patch_area", C.c_double, [P(QuadPatch)]),
    ("quad_patch_size", C.c_double, [P(QuadPatch)]),
    ("quad_patch_min_vertex_distance", C.c_double, [P(QuadPatch), P(QuadPatch)]),
    ("quad_patch_classify_pair", C.c_int, [P(QuadPatch), P(QuadPatch), C.c_double]),
    ("quad_patch_kernel_1_over_r", C.c_double,
     [P(QuadPatch), P(QuadPatch), C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]),
    # inductance.h
    ("inductance_options_default", None, [P(InductanceOptions), C.c_int]),
    ("inductance_init", None, [P(InductanceMatrix)]),
    ("inductance_free", None, [P(InductanceMatrix)]),
    ("inductance_compute_pair", C.c_int,
     [P(Mesh), P(DualMesh), C.c_size_t, C.c_size_t, P(InductanceOptions), c_double_p]),
    ("inductance_compute_matrix", C.c_int,
     [P(Mesh), P(DualMesh), P(InductanceOptions), P(InductanceMatrix)]),
    ("inductance_print_info", None, [P(InductanceMatrix)]),
    # potential.h
    ("potential_options_default", None, [P(PotentialOptions), C.c_int]),
    ("potential_init", None, [P(PotentialMatrix)]),
    ("potential_free", None, [P(PotentialMatrix)]),
    ("potential_compute_pair", C.c_int,
     [P(Mesh), P(DualMesh), C.c_size_t, C.c_size_t, P(PotentialOptions), c_double_p]),
    ("potential_compute_matrix", C.c_int,
     [P(Mesh), P(DualMesh), P(PotentialOptions), P(PotentialMatrix)]),
    ("potential_print_info", None, [P(PotentialMatrix)]),
    ("potential_build_self_capacitance", C.c_int, [P(PotentialMatrix), c_double_p]),
    ("potential_self_voltage_to_charge", C.c_int,
     [P(PotentialMatrix), c_double_p, c_double_p]),
    ("potential_self_voltage_to_full_potential", C.c_int,
     [P(PotentialMatrix), c_double_p, c_double_p]),
    # lu.h
    ("lu_options_default", None, [P(LUOptions), C.c_int]),
    ("lu_init", None, [P(LUFactorization)]),
    ("lu_free", None, [P(LUFactorization)]),
    ("lu_factorize", C.c_int, [c_double_p, C.c_size_t, P(LUOptions), P(LUFactorization)]),
    ("lu_solve", C.c_int, [P(LUFactorization), c_double_p, c_double_p]),
    ("lu_solve_multiple", C.c_int,
     [P(LUFactorization), c_double_p, c_double_p, C.c_size_t, C.c_int]),
    ("lu_determinant", C.c_double, [P(LUFactorization)]),
    ("lu_print_info", None, [P(LUFactorization)]),
    # complex_lu.h
    ("complex_lu_options_default", None, [P(ComplexLUOptions), C.c_int]),
    ("complex_lu_init", None, [P(ComplexLUFactorization)]),
    ("complex_lu_free", None, [P(ComplexLUFactorization)]),
    ("complex_lu_factorize", C.c_int,
     [P(Complex), C.c_size_t, P(ComplexLUOptions), P(ComplexLUFactorization)]),
    ("complex_lu_solve", C.c_int, [P(ComplexLUFactorization), P(Complex), P(Complex)]),
    ("complex_lu_solve_multiple", C.c_int,
     [P(ComplexLUFactorization), P(Complex), P(Complex), C.c_size_t, C.c_int]),
    ("complex_lu_print_info", None, [P(ComplexLUFactorization)]),
]

class PeecAssemblyStats(C.Structure):
    _fields_ = [("near_pairs", C.c_ulonglong), ("potential_evaluations", C.c_ulonglong),
                ("far_point_pairs", C.c_ulonglong), ("near_pairs_evaluated", C.c_ulonglong),
                ("near_pairs_reevaluated", C.c_ulonglong),
                ("ms_prepare", C.c_double), ("ms_near", C.c_double), ("ms_far", C.c_double)]


class PeecHarmonicRequest(C.Structure):
    _fields_ = [("mesh", P(Mesh)), ("dual", P(DualMesh)), ("mesh_key", C.c_ulonglong),
                ("frequency", C.c_double), ("nrhs", C.c_size_t), ("k_hat", c_double_p),
                ("e_hat", c_double_p), ("mixed", C.c_int), ("tolerance", C.c_double),
                ("x", P(Complex))]


class PeecTransientRequest(C.Structure):
    _fields_ = [("mesh", P(Mesh)), ("dual", P(DualMesh)), ("mesh_key", C.c_ulonglong),
                ("scheme", C.c_int), ("dt", C.c_double), ("n_steps", C.c_size_t),
                ("K", C.c_double), ("alpha", C.c_double), ("beta", C.c_double), ("delay", C.c_double),
                ("strike_node", C.c_size_t), ("return_node", C.c_size_t),
                ("probe_nodes", P(C.c_int)), ("n_probe_nodes", C.c_size_t),
                ("probe_edges", P(C.c_int)), ("n_probe_edges", C.c_size_t),
                ("probes", c_double_p), ("I", c_double_p), ("V", c_double_p)]


class PeecRequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("fallback", C.c_int), ("backward_error", C.c_double),
                ("t_submit", C.c_double), ("t_start", C.c_double), ("t_end", C.c_double)]


class PeecSweepTuning(C.Structure):
    _fields_ = [("split_terms", C.c_int), ("sweeps", C.c_int), ("tile_bn", C.c_int)]


# include/peec_gb300.h
EXT_SYMBOLS = [
    ("peec_gb300_device_ready", C.c_int, []),
    ("peec_gb300_last_error", C.c_char_p, []),
    ("peec_gb300_launch_count", C.c_ulonglong, []),
    ("peec_gb300_stream", C.c_void_p, []),
    ("peec_gb300_device_alloc", C.c_void_p, [C.c_size_t]),
    ("peec_gb300_device_free", None, [C.c_void_p]),
    ("peec_gb300_host_alloc_pinned", C.c_void_p, [C.c_size_t]),
    ("peec_gb300_host_free_pinned", None, [C.c_void_p]),
    ("peec_gb300_copy_to_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    ("peec_gb300_copy_to_host", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    ("peec_gb300_copy_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    ("peec_gb300_synchronize", C.c_int, []),
    ("peec_gb300_event_record", C.c_void_p, []),
    ("peec_gb300_event_elapsed_ms", C.c_double, [C.c_void_p, C.c_void_p]),
    ("peec_gb300_event_destroy", None, [C.c_void_p]),
    ("peec_gb300_inductance_device", C.c_int,
     [P(Mesh), P(DualMesh), P(InductanceOptions), C.c_void_p, P(PeecAssemblyStats)]),
    ("peec_gb300_potential_device", C.c_int,
     [P(Mesh), P(DualMesh), P(PotentialOptions), C.c_void_p, P(PeecAssemblyStats)]),
    ("peec_gb300_set_far_precision", C.c_int, [C.c_int]),
    ("peec_gb300_set_near_reuse", C.c_int, [C.c_int]),
    ("peec_gb300_lu_factor_device", C.c_int,
     [C.c_void_p, C.c_size_t, C.c_double, C.c_void_p, C.c_void_p, c_double_p, c_int_p]),
    ("peec_gb300_lu_factor_device_noalloc", C.c_int,
     [C.c_void_p, C.c_size_t, C.c_double, C.c_void_p, C.c_void_p, c_double_p, c_int_p]),
    ("peec_gb300_complex_lu_factor_device", C.c_int,
     [C.c_void_p, C.c_size_t, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
      c_double_p, c_int_p]),
    ("peec_gb300_lu_solve_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t]),
    ("peec_gb300_complex_lu_solve_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
      C.c_size_t]),
    ("peec_gb300_set_factor_cache", C.c_int, [C.c_int]),
    ("peec_gb300_sweep_create", C.c_void_p,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t,
      c_double_p, c_double_p, P(PeecSweepTuning)]),
    ("peec_gb300_sweep_tune", C.c_int, [C.c_void_p, c_double_p, C.c_size_t, P(PeecSweepTuning), c_double_p]),
    ("peec_gb300_sweep_run", C.c_int,
     [C.c_void_p, c_double_p, C.c_size_t, C.c_double, C.c_void_p, c_double_p, c_int_p]),
    ("peec_gb300_sweep_tuning", C.c_int, [C.c_void_p, P(PeecSweepTuning)]),
    ("peec_gb300_sweep_split", C.c_int, [C.c_void_p, c_double_p, P(PeecSweepTuning)]),
    ("peec_gb300_sweep_destroy", None, [C.c_void_p]),
    ("peec_gb300_lu_timing_enable", None, [C.c_int]),
    ("peec_gb300_lu_timing", C.c_int, [c_double_p, c_double_p, c_double_p, c_double_p]),
    ("peec_gb300_lu_timing_trailing", C.c_int, [c_double_p, c_double_p]),
    ("peec_gb300_pipe_peaks", C.c_int, [c_double_p, c_double_p]),
    ("peec_gb300_tc_gemm", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
      C.c_longlong, C.c_int]),
    ("peec_gb300_tc_gemm_cplx", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
      C.c_longlong]),
    ("peec_gb300_round_to_f32_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]),
    ("peec_gb300_rcs_radiation_device", C.c_int,
     [C.POINTER(Mesh), C.POINTER(DualMesh), C.c_void_p, C.c_size_t, C.c_size_t, C.c_double, c_double_p,
      C.c_size_t, C.c_int, C.c_void_p]),
    ("peec_gb300_complex_solve_mixed_device", C.c_int,
     [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, C.c_double, C.c_int, c_double_p,
      c_int_p]),
    ("peec_gb300_complex_refine_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
      C.c_size_t, C.c_double, C.c_int, c_double_p, c_int_p]),
    ("peec_gb300_mixed_timing", C.c_int, [c_double_p, c_double_p, c_double_p]),
    ("peec_gb300_mixed_split_terms", C.c_int, []),
    ("peec_gb300_pat_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.POINTER(C.c_longlong)]),
    ("peec_gb300_apat_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p]),
    ("peec_gb300_as_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p]),
    ("peec_gb300_mixed_gmres_iterations", C.c_int, []),
    ("peec_gb300_harmonic_build_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_double,
      C.c_void_p]),
    ("peec_gb300_plane_wave_rhs_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, c_double_p, c_double_p, C.c_double,
      C.c_void_p]),
    ("peec_gb300_backward_error_device", C.c_int,
     [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, c_double_p]),
    ("peec_gb300_inductance_retarded_device", C.c_int,
     [P(Mesh), P(DualMesh), P(InductanceOptions), C.c_double, C.c_void_p, P(PeecAssemblyStats)]),
    ("peec_gb300_potential_retarded_device", C.c_int,
     [P(Mesh), P(DualMesh), P(PotentialOptions), C.c_double, C.c_void_p, P(PeecAssemblyStats)]),
    ("peec_gb300_harmonic_build_retarded_device", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_double, C.c_void_p]),
    ("peec_gb300_transient_create", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_int, C.c_double,
      P(C.c_void_p)]),
    ("peec_gb300_transient_lightning", C.c_int,
     [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_size_t, C.c_size_t,
      C.c_size_t, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
      C.c_size_t, C.c_void_p]),
    ("peec_gb300_transient_lightning_batch", C.c_int,
     [C.c_void_p, C.c_int, c_double_p, c_double_p, c_double_p, c_double_p, P(C.c_size_t), P(C.c_size_t),
      C.c_size_t, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p]),
    ("peec_gb300_transient_destroy", None, [C.c_void_p]),
    ("peec_gb300_server_create", C.c_void_p, [C.c_size_t, C.c_int]),
    ("peec_gb300_server_submit", C.c_longlong, [C.c_void_p, P(PeecHarmonicRequest)]),
    ("peec_gb300_server_submit_transient", C.c_longlong, [C.c_void_p, P(PeecTransientRequest)]),
    ("peec_gb300_server_wait", C.c_int, [C.c_void_p, C.c_longlong, P(PeecRequestResult)]),
    ("peec_gb300_server_clock", C.c_double, [C.c_void_p]),
    ("peec_gb300_server_destroy", None, [C.c_void_p]),
]

MESH_SYMBOLS = [
    ("peec_synth_plate", C.c_int, [C.c_double, C.c_double, C.c_int, C.c_int, P(Mesh)]),
    ("peec_synth_box", C.c_int,
     [C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, P(Mesh)]),
    ("peec_synth_from_arrays", C.c_int,
     [c_double_p, C.c_size_t, c_int_p, C.c_size_t, P(Mesh)]),
    ("peec_synth_topology", C.c_int, [P(Mesh)]),
    ("peec_synth_dual", C.c_int, [P(Mesh), P(DualMesh)]),
    ("peec_synth_mesh_free", None, [P(Mesh)]),
    ("peec_synth_dual_free", None, [P(DualMesh)]),
]


def _bind(lib, table):
    for name, res, args in table:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_cache = {}


def load_mesh_lib():
    """Host-only library with the synthetic mesher (no GPU needed)."""
    if "mesh" not in _cache:
        if not os.path.exists(MESH_LIB_PATH):
            raise RuntimeError("libpeec_mesh.so missing: run __graft_entry__.build()")
        _cache["mesh"] = _bind(C.CDLL(MESH_LIB_PATH), MESH_SYMBOLS)
    return _cache["mesh"]


def load_gpu_lib():
    """The sm_103a drop-in library.  Raises if it was not built: there is no
    CPU fallback for the product path."""
    if "gpu" not in _cache:
        if not os.path.exists(GPU_LIB_PATH):
            raise RuntimeError("libpeec_gb300.so missing: run __graft_entry__.build()")
        lib = C.CDLL(GPU_LIB_PATH)
        _bind(lib, DROP_IN_SYMBOLS)
        _bind(lib, EXT_SYMBOLS)
        _cache["gpu"] = lib
    return _cache["gpu"]
