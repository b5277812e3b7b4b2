"""ctypes binding of libsprgb300.so (the C ABI declared in include/spr_gb300.h).

The library is the only compute path: if it is missing this module raises,
there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsprgb300.so")

SPRG_OK = 0
SPRG_EINVAL = 1
SPRG_EPATCH = 2
SPRG_EFLAGS = 3
SPRG_ENOMEM = 4
SPRG_ECUDA = 5
SPRG_ESTATE = 6
SPRG_EEIGEN = 7
ERROR_NAMES = {1: "EINVAL", 2: "EPATCH", 3: "EFLAGS", 4: "ENOMEM", 5: "ECUDA", 6: "ESTATE", 7: "EEIGEN"}

SPRG_FP64 = 0
SPRG_FP32 = 1
SPRG_LEARNED = 2
MLP_PARAMS = 12611
MLP_INPUTS = 128
MLP_AUX = 5

SPLIT = 1 << 0
DONT_SPLIT = 1 << 1
COLLAPSE = 1 << 2
DONT_COLLAPSE = 1 << 3
NEED_NOT_SPLIT = 1 << 17
NEED_NOT_COLLAPSE = 1 << 18
BAD_QUALITY = 1 << 5
OK_QUALITY = 1 << 6
SIZE_IDENTITY = 0
SIZE_ISO = 1
SIZE_ANISO = 2
SIZE_LOG_ANISO = 3
MARK_SPLIT = 0
MARK_COLLAPSE = 1

# every symbol include/spr_gb300.h declares
EXPORTS = [
    "sprg_create", "sprg_destroy", "sprg_last_error", "sprg_set_precision", "sprg_set_stream",
    "sprg_get_grad_ip_field", "sprg_recover_field", "sprg_get_spr_size_field",
    "sprg_get_target_spr_size_field", "sprg_measure_edges", "sprg_measure_edges_aniso",
    "sprg_mark_edges", "sprg_measure_quality", "sprg_estimate_and_mark",
    "sprg_estimate_and_mark_resident", "sprg_apply_marks", "sprg_last_launch_count",
    "sprg_box_counts", "sprg_box_fill", "sprg_profile_enable", "sprg_profile_flush", "sprg_profile_report",
    "sprg_spr_size_from_recovered_noalloc", "sprg_debug_read",
    "sprg_set_mlp_params", "sprg_set_learned_options", "sprg_learned_features", "sprg_mlp_scratch_bytes",
    "sprg_mlp_forward", "sprg_mlp_grad", "sprg_mlp_adam", "sprg_hessian_metric",
    "sprg_aniso_estimate_and_mark_resident", "sprg_set_batch", "sprg_batch_info", "sprg_set_autotune",
    "sprg_tuning_report", "sprg_graph_capture", "sprg_graph_replay", "sprg_set_tiling",
    "sprg_measure_vertex_pairs", "sprg_get_maximum_edge_length", "sprg_get_average_edge_length",
    "sprg_max_iterations_for_length", "sprg_mark_bad_quality", "sprg_get_min_quality",
    "sprg_measure_edges_log_aniso", "sprg_measure_quality_log_aniso", "sprg_update_mesh",
    "sprg_smb_counts", "sprg_smb_read", "sprg_smb_write", "sprg_e2e_timing", "sprg_e2e_timing_report", "sprg_test_hooks",
    "sprg_rounding_dominated",
    "sprg_locality_order",
]
NOALLOC_MAX_ELEMS = 1 << 20


class SprgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


class MeshView(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("n_verts", ctypes.c_int64),
        ("n_elems", ctypes.c_int64),
        ("n_edges", ctypes.c_int64),
        ("coords", ctypes.c_void_p),
        ("elem_verts", ctypes.c_void_p),
        ("edge_verts", ctypes.c_void_p),
        ("vert_elem_offsets", ctypes.c_void_p),
        ("vert_elems", ctypes.c_void_p),
    ]


class MeshDelta(ctypes.Structure):
    """sprg_mesh_delta: new counts and the rows whose values are new."""
    _fields_ = [
        ("n_verts", ctypes.c_int64),
        ("n_elems", ctypes.c_int64),
        ("n_edges", ctypes.c_int64),
        ("n_vert_rows", ctypes.c_int64),
        ("vert_ids", ctypes.c_void_p),
        ("coords", ctypes.c_void_p),
        ("n_elem_rows", ctypes.c_int64),
        ("elem_ids", ctypes.c_void_p),
        ("elem_verts", ctypes.c_void_p),
        ("n_edge_rows", ctypes.c_int64),
        ("edge_ids", ctypes.c_void_p),
        ("edge_verts", ctypes.c_void_p),
        ("vert_elem_offsets", ctypes.c_void_p),
        ("vert_elems", ctypes.c_void_p),
    ]


class SizeInfo(ctypes.Structure):
    _fields_ = [
        ("eps_star_norm2", ctypes.c_double),
        ("error_sum", ctypes.c_double),
        ("size_factor", ctypes.c_double),
        ("n_expanded", ctypes.c_int64),
        ("n_fp64_refits", ctypes.c_int64),
        ("n_guard_edges", ctypes.c_int64),
        ("n_guard_unresolved", ctypes.c_int64),
        ("n_learned_fallback", ctypes.c_int64),
        ("n_rounding_dominated", ctypes.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load():
    """Returns the loaded library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -m core_gb300.build` "
            "(the estimate-and-mark pass has no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    I = ctypes.c_int
    D = ctypes.c_double
    lib.sprg_create.argtypes = [ctypes.POINTER(MeshView), I, ctypes.POINTER(P)]
    lib.sprg_destroy.argtypes = [P]
    lib.sprg_last_error.argtypes = [P]
    lib.sprg_last_error.restype = ctypes.c_char_p
    lib.sprg_set_precision.argtypes = [P, I]
    lib.sprg_set_stream.argtypes = [P, P]
    lib.sprg_get_grad_ip_field.argtypes = [P, P, I, I, P]
    lib.sprg_recover_field.argtypes = [P, P, I, P]
    lib.sprg_get_spr_size_field.argtypes = [P, P, I, D, P, ctypes.POINTER(SizeInfo)]
    lib.sprg_get_target_spr_size_field.argtypes = [P, P, I, ctypes.c_size_t, D, D, P, ctypes.POINTER(SizeInfo)]
    lib.sprg_measure_edges.argtypes = [P, P, P]
    lib.sprg_measure_edges_aniso.argtypes = [P, P, P, P]
    lib.sprg_mark_edges.argtypes = [P, I, P, ctypes.POINTER(ctypes.c_long)]
    lib.sprg_measure_quality.argtypes = [P, P, P, P, P]
    lib.sprg_estimate_and_mark.argtypes = [P, P, D, P, P, ctypes.POINTER(ctypes.c_long),
                                           ctypes.POINTER(ctypes.c_long), ctypes.POINTER(SizeInfo)]
    lib.sprg_estimate_and_mark_resident.argtypes = [P, P, D, P, P]
    lib.sprg_rounding_dominated.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    lib.sprg_apply_marks.argtypes = [ctypes.c_int64, P, P, P, ctypes.POINTER(ctypes.c_long),
                                     ctypes.POINTER(ctypes.c_long)]
    F = ctypes.c_float
    lib.sprg_hessian_metric.argtypes = [P, P, D, D, D, P, P]
    lib.sprg_set_batch.argtypes = [P, I, P, P, P]
    lib.sprg_set_autotune.argtypes = [P, I]
    lib.sprg_set_tiling.argtypes = [P, P, I, I]
    lib.sprg_tuning_report.argtypes = [P]
    lib.sprg_tuning_report.restype = ctypes.c_char_p
    lib.sprg_graph_capture.argtypes = [P, P, D, P, P]
    lib.sprg_graph_replay.argtypes = [P]
    lib.sprg_batch_info.argtypes = [P, P]
    lib.sprg_aniso_estimate_and_mark_resident.argtypes = [P, P, D, D, D, P, P, P]
    lib.sprg_set_mlp_params.argtypes = [P, P, I]
    lib.sprg_set_learned_options.argtypes = [P, I, D]
    lib.sprg_learned_features.argtypes = [P, P, P, P]
    lib.sprg_mlp_scratch_bytes.argtypes = [I]
    lib.sprg_mlp_scratch_bytes.restype = ctypes.c_size_t
    lib.sprg_mlp_forward.argtypes = [P, P, I, P, P, P]
    lib.sprg_mlp_grad.argtypes = [P, P, P, I, P, P, P, P]
    lib.sprg_mlp_adam.argtypes = [P, P, P, P, F, F, F, F, I, P]
    lib.sprg_profile_enable.argtypes = [P, I]
    lib.sprg_profile_flush.argtypes = [P]
    lib.sprg_profile_report.argtypes = [P, I]
    lib.sprg_profile_report.restype = ctypes.c_char_p
    lib.sprg_spr_size_from_recovered_noalloc.argtypes = [I, ctypes.c_int64, ctypes.c_int64, P, P, P, P, P, I, P, D,
                                                         P, ctypes.POINTER(D), P]
    lib.sprg_debug_read.argtypes = [P, ctypes.c_char_p, P, ctypes.c_size_t]
    lib.sprg_last_launch_count.argtypes = [P]
    lib.sprg_last_launch_count.restype = ctypes.c_int64
    lib.sprg_box_counts.argtypes = [I, I, I, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                    ctypes.POINTER(ctypes.c_int64)]
    lib.sprg_box_fill.argtypes = [I, I, I, D, D, D, P, P, P]
    lib.sprg_measure_vertex_pairs.argtypes = [P, I, P, P, P, ctypes.c_int64, P, P]
    lib.sprg_get_maximum_edge_length.argtypes = [P, I, P, P, P, ctypes.POINTER(D)]
    lib.sprg_get_average_edge_length.argtypes = [P, ctypes.POINTER(D)]
    lib.sprg_max_iterations_for_length.argtypes = [D]
    lib.sprg_mark_bad_quality.argtypes = [P, D, P, ctypes.POINTER(ctypes.c_long)]
    lib.sprg_get_min_quality.argtypes = [P, ctypes.POINTER(D)]
    lib.sprg_measure_edges_log_aniso.argtypes = [P, P, P, P]
    lib.sprg_update_mesh.argtypes = [P, ctypes.POINTER(MeshDelta)]
    lib.sprg_smb_counts.argtypes = [ctypes.c_char_p, ctypes.POINTER(I), ctypes.POINTER(ctypes.c_int64),
                                    ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    lib.sprg_smb_read.argtypes = [ctypes.c_char_p, P, P, P]
    lib.sprg_smb_write.argtypes = [ctypes.c_char_p, ctypes.POINTER(MeshView)]
    lib.sprg_measure_quality_log_aniso.argtypes = [P, P, P, P]
    lib.sprg_e2e_timing.argtypes = [P, I]
    lib.sprg_test_hooks.argtypes = [P, I, I]
    lib.sprg_locality_order.argtypes = [ctypes.POINTER(MeshView), P, P, P]
    lib.sprg_e2e_timing_report.argtypes = [P]
    lib.sprg_e2e_timing_report.restype = ctypes.c_char_p
    _lib = lib
    return lib


def check(rc, ctx=None):
    if rc != SPRG_OK:
        msg = load().sprg_last_error(ctx).decode() if ctx else ""
        raise SprgError(rc, msg)
