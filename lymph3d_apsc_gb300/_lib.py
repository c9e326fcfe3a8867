"""ctypes binding of liblymph3d_gb300.so (include/lymph3d_gpu.h, lymph3d_mesh.h).

The library is loaded from the package directory (built in-tree by
build.py).  Loading fails loudly: there is no Python or CPU stand-in for any
entry point.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_uint64, c_void_p
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "liblymph3d_gb300.so"

# ---- constants mirrored from include/lymph3d_gpu.h ----
LYMPH_OK = 0
LYMPH_EXIT_INSTAB = 2
LYMPH_EXIT_SETUP = 4
LYMPH_EXIT_SINGULARMTX = 5
LYMPH_EXIT_ELEM_ORIENT = 11
LYMPH_EXIT_NEIGHBOUR_EL_ERROR = 18
LYMPH_ERR_INVALID = 100
LYMPH_ERR_CUDA = 101
LYMPH_ERR_OOM = 102
LYMPH_ERR_ORDER = 103
LYMPH_ERR_TIMEOUT = 104
LYMPH_ERR_INDEX = 105

BC_DIRI = -1
BC_NEUM = -2
BC_ABSO = -3  # absorbing: no stiffness or load term, a damping block on its polyhedron
MESH_UNMATCHED = -9

FP64 = 0
MIXED = 1
MIXED_MF = 2  # FP32 self blocks, neighbour terms matrix-free from face quadrature

SLOT_U0, SLOT_UN, SLOT_V0, SLOT_UEX = 0, 1, 2, 3
LAYOUT_POLY_MAJOR, LAYOUT_FORTRAN = 0, 1
RHS_STAT, RHS_DYN = 0, 1
F_NULL, F_TIME, F_STAT = 0, 1, 2
GD_NULL, GD, GD_STAT = 0, 1, 2
GN_NULL, GN, GN_STAT = 0, 1, 2
FUN_IC_DISPLACEMENT, FUN_IC_VELOCITY, FUN_UEX, FUN_UEX_STAT = 0, 1, 2, 3
BLOCKS_K, BLOCKS_ADG = 0, 1
BCMODE_REFERENCE, BCMODE_ALL_DIRICHLET = 0, 1

P_I32 = POINTER(c_int32)
P_F64 = POINTER(c_double)


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("n_node", c_int32), ("n_tet", c_int32), ("n_poly", c_int32), ("n_mat", c_int32),
        ("coords", P_F64), ("tet_vert", P_I32), ("tet_poly", P_I32), ("tet_mat", P_I32),
        ("neigh", P_I32), ("fun_tag", P_I32), ("mat", P_F64),
    ]


class Params(ctypes.Structure):
    _fields_ = [("degree", c_int32), ("precision", c_int32), ("alpha", c_double), ("theta", c_double), ("dt", c_double)]


class LymphError(RuntimeError):
    """A non-zero status returned by the library (code = reference exit code or LYMPH_ERR_*)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


# name -> (restype, argtypes)
_SIGS = {
    "lymph_version": (c_int, []),
    "lymph_last_error": (c_char_p, []),
    "lymph_create": (c_int, [POINTER(MeshDesc), POINTER(Params), POINTER(c_void_p)]),
    "lymph_destroy": (c_int, [c_void_p]),
    "lymph_sizes": (c_int, [c_void_p, P_I32, P_I32, POINTER(c_int64), POINTER(c_int64)]),
    "lymph_make_matrices": (c_int, [c_void_p]),
    "lymph_make_rhs": (c_int, [c_void_p, c_int, c_int, c_int, c_int]),
    "lymph_modal_project": (c_int, [c_void_p, c_int, c_int, c_double]),
    "lymph_first_step": (c_int, [c_void_p, c_double]),
    "lymph_step": (c_int, [c_void_p, c_double]),
    "lymph_first_step_g": (c_int, [c_void_p, c_double]),
    "lymph_step_g": (c_int, [c_void_p, c_double]),
    "lymph_run_steps": (c_int, [c_void_p, c_double, c_int64, P_F64, POINTER(c_int64), POINTER(c_float),
                                POINTER(c_float)]),
    "lymph_get_state": (c_int, [c_void_p, c_int, P_F64, c_int]),
    "lymph_set_state": (c_int, [c_void_p, c_int, P_F64, c_int]),
    "lymph_copy_state": (c_int, [c_void_p, c_int, c_int]),
    "lymph_error_l2": (c_int, [c_void_p, c_int, c_int, P_F64]),
    "lymph_error_dg": (c_int, [c_void_p, c_int, c_int, P_F64]),
    "lymph_error_l2_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_int32, c_int32, P_F64]),
    "lymph_compute_error_l2_free": (c_int, [c_void_p, c_int, c_int, P_F64]),
    "lymph_compute_error_dg_free": (c_int, [c_void_p, c_int, c_int, P_F64]),
    "lymph_get_pattern": (c_int, [c_void_p, P_I32, P_I32]),
    "lymph_get_blocks": (c_int, [c_void_p, c_int, P_F64]),
    "lymph_get_self_blocks": (c_int, [c_void_p, P_F64]),
    "lymph_get_mass": (c_int, [c_void_p, c_int, P_F64]),
    "lymph_get_rhs": (c_int, [c_void_p, c_int, P_F64]),
    "lymph_get_poly_geometry": (c_int, [c_void_p, P_F64, P_F64]),
    "lymph_make_rhs_point": (c_int, [c_void_p, c_int, c_int32, P_F64, P_F64]),
    "lymph_make_rhs_double_couple": (c_int, [c_void_p, c_int, c_int32, P_F64, P_F64, c_double]),
    "lymph_set_dt": (c_int, [c_void_p, c_double]),
    "lymph_get_dt": (c_int, [c_void_p, P_F64]),
    "lymph_max_eigenvalue": (c_int, [c_void_p, c_int32, P_F64]),
    "lymph_batch_create": (c_int, [POINTER(c_void_p), c_int32, POINTER(c_void_p)]),
    "lymph_batch_destroy": (c_int, [c_void_p]),
    "lymph_batch_run": (c_int, [c_void_p, c_int64, P_F64, POINTER(c_float)]),
    "lymph_batch_autotune": (c_int, [c_void_p, c_int32, c_int32, P_I32, P_I32]),
    "lymph_batch_schedule": (c_int, [c_void_p, P_I32, P_I32, P_I32]),
    "lymph_mf_face_rule": (c_int, [c_int32, P_I32, P_F64]),
    "lymph_time_step_host": (c_int, [c_void_p, c_double, P_F64, P_F64, P_F64, c_int]),
    "lymph_checkpoint_save": (c_int, [c_void_p, c_char_p, c_double, c_int64]),
    "lymph_checkpoint_load": (c_int, [c_void_p, c_char_p, POINTER(c_double), POINTER(c_int64)]),
    "lymph_batch_launch_count": (c_int, [c_void_p, POINTER(c_int64)]),
    "lymph_energy": (c_int, [c_void_p, c_int, c_int, P_F64]),
    "lymph_apply_operator": (c_int, [c_void_p, P_F64, P_F64]),
    "lymph_mpnn_create": (c_int, [c_int32, c_int32, c_int32, c_int32, c_int32, POINTER(c_void_p)]),
    "lymph_mpnn_destroy": (c_int, [c_void_p]),
    "lymph_mpnn_num_params": (c_int64, [c_void_p]),
    "lymph_mpnn_set_params": (c_int, [c_void_p, POINTER(c_float)]),
    "lymph_mpnn_get_params": (c_int, [c_void_p, POINTER(c_float), POINTER(c_float)]),
    "lymph_mpnn_set_graph": (c_int, [c_void_p, c_int32, P_I32, P_I32, POINTER(c_float), POINTER(c_float)]),
    "lymph_mpnn_forward": (c_int, [c_void_p, POINTER(c_float), POINTER(c_float)]),
    "lymph_mpnn_loss_grad": (c_int, [c_void_p, POINTER(c_float), POINTER(c_float), P_F64]),
    "lymph_mpnn_adam": (c_int, [c_void_p, c_float, c_float, c_float, c_float]),
    "lymph_mpnn_launch_count": (c_int, [c_void_p, POINTER(c_int64)]),
    "lymph_surrogate_predict": (c_int, [c_void_p, c_void_p, c_int32, c_int32, c_double, P_F64]),
    "lymph_surrogate_residual": (c_int, [c_void_p, c_void_p, P_F64]),
    "lymph_surrogate_apply_fp32": (c_int, [c_void_p, c_int32]),
    "lymph_nodal_values": (c_int, [c_void_p, c_int, P_F64]),
    "lymph_mpnn_set_gate": (c_int, [c_void_p, c_int32, c_int32]),
    "lymph_mpnn_time_forward": (c_int, [c_void_p, c_int32, P_F64]),
    "lymph_mpnn_uses_tensor_cores": (c_int, [c_void_p]),
    "lymph_surrogate_features": (c_int, [c_void_p, c_void_p, c_double, POINTER(c_float), P_F64, P_F64, P_F64]),
    "lymph_surrogate_judge": (c_int, [c_void_p, c_void_p, c_int32, P_F64]),
    "lymph_launch_count": (c_int, [c_void_p, POINTER(c_int64)]),
    "lymph_device_bytes": (c_int, [c_void_p, POINTER(c_int64)]),
    "lymph_fp64_peak": (c_int, [c_int32, P_F64]),
    # mesh utilities (lymph3d_mesh.h)
    "lymph_mesh_cube_sizes": (c_int, [c_int32, c_int32, c_int32, P_I32, P_I32]),
    "lymph_mesh_cube": (c_int, [c_int32, c_int32, c_int32, P_F64, P_I32, P_I32]),
    "lymph_mesh_match_faces": (c_int, [c_int32, P_I32, P_I32, P_I32]),
    "lymph_mesh_tag_boundary": (c_int, [c_int32, P_I32, c_int32, P_I32, P_I32, P_I32, P_I32]),
    "lymph_mesh_apply_bc": (c_int, [c_int32, P_I32, c_int32, P_I32, P_I32]),
    "lymph_mesh_agglomerate": (c_int, [c_int32, P_I32, c_uint64, c_int32, c_int32, P_I32, P_I32]),
    "lymph_mesh_agglomerate_hex": (c_int, [c_int32, P_I32, P_I32]),
    "lymph_mesh_find_tet": (c_int, [c_int32, P_I32, P_F64, P_F64, P_I32]),
}

_lib = None


def declared_symbols():
    """Names of every entry point the headers declare (used by the export test)."""
    return list(_SIGS)


def load(build: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the in-tree library."""
    global _lib
    if _lib is not None:
        return _lib
    if build and os.environ.get("LYMPH_NO_BUILD") != "1":
        from .build import build as _build
        try:
            _build()
        except RuntimeError:
            if not LIB_PATH.exists():
                raise
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m lymph3d_apsc_gb300.build`")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str = "") -> None:
    if rc != LYMPH_OK:
        msg = load().lymph_last_error()
        raise LymphError(rc, f"{what}: {msg.decode() if msg else ''}")


def ptr(a, typ):
    """ctypes pointer into a contiguous numpy array."""
    return a.ctypes.data_as(POINTER(typ))
