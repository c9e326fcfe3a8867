"""Host-side mirror of the reference's `module matrix_free` (src/matrix_free.f90).

`MatrixFree` keeps the device context of one problem; its methods carry the
reference's subroutine names and argument meaning, with the Fortran
procedure arguments replaced by data-function ids and the driver's arrays
(u0_loc, un_loc, v0_loc, the exact-solution coefficients) by state slots that
live on the device.  Every method calls the C ABI (include/lymph3d_gpu.h);
errors come back as LymphError carrying the reference's exit code.

`run_reference_driver` replays the sequence of src/Lymph3D.f90:262-518.
"""
from __future__ import annotations

import math
from ctypes import byref, c_double, c_float, c_int32, c_int64, c_void_p

import numpy as np

from . import _lib
from ._lib import (FUN_IC_DISPLACEMENT, FUN_IC_VELOCITY, FUN_UEX, FUN_UEX_STAT, LAYOUT_POLY_MAJOR, RHS_DYN,
                   RHS_STAT, SLOT_U0, SLOT_UEX, SLOT_UN, SLOT_V0, check, ptr)
from .mesh import Mesh

SQRT2 = math.sqrt(2.0)
PI = 4.0 * math.atan(1.0)


def time_function(t: float) -> float:
    """sin(sqrt(2) pi t), problem_data_and_properties.f90:14-23."""
    return math.sin(SQRT2 * PI * t)


class MatrixFree:
    """One PolyDG elastodynamics problem on the GPU.

    Parameters mirror set_properties (alpha=10, theta=-1) and the Poly.input
    TIMESTEP; `precision` is _lib.FP64 (plain), _lib.MIXED (FP32 blocks) or
    _lib.MIXED_MF (FP32 self blocks, neighbour terms matrix-free in FP32).
    """

    def __init__(self, mesh: Mesh, degree: int, dt: float, alpha: float = 10.0, theta: float = -1.0,
                 precision: int = _lib.FP64):
        self.lib = _lib.load()
        self.mesh = mesh
        self._desc = mesh.desc()
        prm = _lib.Params(degree, precision, alpha, theta, dt)
        h = c_void_p()
        check(self.lib.lymph_create(byref(self._desc), byref(prm), byref(h)), "lymph_create")
        self.ctx = h
        self.degree, self.dt, self.alpha, self.theta, self.precision = degree, dt, alpha, theta, precision
        Np, npoly, nb, nfs = c_int32(), c_int32(), c_int64(), c_int64()
        check(self.lib.lymph_sizes(self.ctx, byref(Np), byref(npoly), byref(nb), byref(nfs)), "lymph_sizes")
        self.Np, self.n_poly, self.n_blocks, self.n_face_sides = Np.value, npoly.value, nb.value, nfs.value
        self.nd = 3 * self.Np

    # ---- lifetime ----
    def close(self):
        if getattr(self, "ctx", None):
            self.lib.lymph_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- reference entry points ----
    def MAKE_MATRICES_FREE(self):
        """matrix_free.f90:27-464 + the Cholesky factors of Lymph3D.f90:264-271."""
        check(self.lib.lymph_make_matrices(self.ctx), "MAKE_MATRICES_FREE")

    def MAKE_RHS_FREE(self, which: int, f_forcing: int, f_dirichlet: int, f_neumann: int):
        """matrix_free.f90:467-843 (which = RHS_STAT or RHS_DYN)."""
        check(self.lib.lymph_make_rhs(self.ctx, which, f_forcing, f_dirichlet, f_neumann), "MAKE_RHS_FREE")

    def COMPUTE_MODAL_COEFFICIENTS_FREE(self, f_analytic: int, slot: int, scale: float = 1.0):
        """matrix_free.f90:847-997: L2 projection into a state slot (times scale)."""
        check(self.lib.lymph_modal_project(self.ctx, f_analytic, slot, scale), "COMPUTE_MODAL_COEFFICIENTS_FREE")

    def FIRST_TIME_STEP_MATRIX_FREE(self, t: float):
        """matrix_free.f90:1100-1227: UN <- U0 + dt V0 + dt^2/2 M^-1 (F(t) - K U0)."""
        check(self.lib.lymph_first_step(self.ctx, t), "FIRST_TIME_STEP_MATRIX_FREE")

    def TIME_STEP_MATRIX_FREE(self, t: float):
        """matrix_free.f90:1230-1385 + the rotation u0_loc = un_loc; un_loc = usol."""
        check(self.lib.lymph_step(self.ctx, t), "TIME_STEP_MATRIX_FREE")

    def time_step_host(self, t: float, u0: np.ndarray, un: np.ndarray, usol: np.ndarray,
                       layout: int = LAYOUT_POLY_MAJOR) -> np.ndarray:
        """TIME_STEP_MATRIX_FREE with host arrays, the reference's argument list
        (matrix_free.f90:1230-1385): u0 = u^{n-1}, un = u^n in, usol = u^{n+1}
        out (filled in place), in the given layout; one C call
        (lymph_time_step_host)."""
        a = np.ascontiguousarray(u0, dtype=np.float64)
        b = np.ascontiguousarray(un, dtype=np.float64)
        if usol.dtype != np.float64 or not usol.flags.c_contiguous or usol.size != self.n_poly * self.nd:
            raise ValueError("usol must be a C-contiguous float64 array of the state's size")
        check(self.lib.lymph_time_step_host(self.ctx, t, ptr(a, c_double), ptr(b, c_double), ptr(usol, c_double), layout),
              "TIME_STEP_MATRIX_FREE")
        return usol

    def save_checkpoint(self, path, t: float, steps: int = 0):
        """Writes u^{n-1}, u^n, t and the step count (lymph_checkpoint_save)."""
        check(self.lib.lymph_checkpoint_save(self.ctx, str(path).encode(), t, steps), "save_checkpoint")

    def load_checkpoint(self, path):
        """Restores u^{n-1}, u^n from a checkpoint of the same run; returns
        (t, steps) (lymph_checkpoint_load)."""
        t, n = c_double(), c_int64()
        check(self.lib.lymph_checkpoint_load(self.ctx, str(path).encode(), byref(t), byref(n)), "load_checkpoint")
        return t.value, n.value

    def COMPUTE_ERROR_L2_MATRIX_FREE(self, slot_uh: int = SLOT_UN, slot_uex: int = SLOT_UEX) -> float:
        """matrix_free.f90:1388-1418: local sum of squares (no sqrt)."""
        out = c_double()
        check(self.lib.lymph_error_l2(self.ctx, slot_uh, slot_uex, byref(out)), "COMPUTE_ERROR_L2_MATRIX_FREE")
        return out.value

    def COMPUTE_ERROR_DG_MATRIX_FREE(self, slot_uh: int = SLOT_UN, slot_uex: int = SLOT_UEX) -> float:
        """matrix_free.f90:1421-1504: local sum of squares (no sqrt)."""
        out = c_double()
        check(self.lib.lymph_error_dg(self.ctx, slot_uh, slot_uex, byref(out)), "COMPUTE_ERROR_DG_MATRIX_FREE")
        return out.value

    # names used by the project specification for the two error routines
    COMPUTE_ERROR_L2_FREE = COMPUTE_ERROR_L2_MATRIX_FREE
    COMPUTE_ERROR_DG_FREE = COMPUTE_ERROR_DG_MATRIX_FREE

    # ---- loop and state access ----
    def run_steps(self, t: float, stop_time: float, max_steps: int = -1, kernel_timing: bool = False):
        """The time loop of Lymph3D.f90:389-418 (graph-launched).  Returns
        (t_after, n_steps, ms_total, ms_kernel)."""
        tt = c_double(t)
        n = c_int64()
        ms = c_float()
        mk = c_float()
        check(self.lib.lymph_run_steps(self.ctx, stop_time, max_steps, byref(tt), byref(n), byref(ms),
                                       byref(mk) if kernel_timing else None), "run_steps")
        return tt.value, n.value, ms.value, (mk.value if kernel_timing else None)

    def apply_operator(self, u: np.ndarray) -> np.ndarray:
        """K u in the context's precision (lymph_apply_operator): the operator
        apply of TIME_STEP_MATRIX_FREE before the mass-matrix solve."""
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(self.n_poly, self.nd)
        out = np.empty_like(u)
        check(self.lib.lymph_apply_operator(self.ctx, ptr(u, c_double), ptr(out, c_double)), "lymph_apply_operator")
        return out

    def get_state(self, slot: int, layout: int = LAYOUT_POLY_MAJOR) -> np.ndarray:
        out = np.empty(self.n_poly * self.nd, np.float64)
        check(self.lib.lymph_get_state(self.ctx, slot, ptr(out, c_double), layout), "get_state")
        return out.reshape((self.n_poly, self.nd) if layout == LAYOUT_POLY_MAJOR else (self.nd, self.n_poly))

    def set_state(self, slot: int, values: np.ndarray, layout: int = LAYOUT_POLY_MAJOR):
        v = np.ascontiguousarray(values, dtype=np.float64)
        check(self.lib.lymph_set_state(self.ctx, slot, ptr(v, c_double), layout), "set_state")

    def pattern(self):
        rp = np.empty(self.n_poly + 1, np.int32)
        col = np.empty(self.n_blocks, np.int32)
        check(self.lib.lymph_get_pattern(self.ctx, ptr(rp, c_int32), ptr(col, c_int32)), "get_pattern")
        return rp, col

    def blocks(self, which: int = _lib.BLOCKS_K) -> np.ndarray:
        out = np.empty((self.n_blocks, self.nd, self.nd), np.float64)
        check(self.lib.lymph_get_blocks(self.ctx, which, ptr(out, c_double)), "get_blocks")
        return out

    def self_blocks(self) -> np.ndarray:
        """The self blocks the step applies, [n_poly][3Np][3Np] row-major."""
        out = np.empty((self.n_poly, self.nd, self.nd), np.float64)
        check(self.lib.lymph_get_self_blocks(self.ctx, ptr(out, c_double)), "get_self_blocks")
        return out

    def mass(self, which: int) -> np.ndarray:
        out = np.empty((self.n_poly, self.Np, self.Np), np.float64)
        check(self.lib.lymph_get_mass(self.ctx, which, ptr(out, c_double)), "get_mass")
        return out

    def rhs(self, which: int) -> np.ndarray:
        out = np.empty((self.n_poly, self.nd), np.float64)
        check(self.lib.lymph_get_rhs(self.ctx, which, ptr(out, c_double)), "get_rhs")
        return out

    def poly_geometry(self):
        bb = np.empty((self.n_poly, 6), np.float64)
        hk = np.empty(self.n_poly, np.float64)
        check(self.lib.lymph_get_poly_geometry(self.ctx, ptr(bb, c_double), ptr(hk, c_double)), "poly_geometry")
        return bb, hk

    def launch_count(self) -> int:
        n = c_int64()
        check(self.lib.lymph_launch_count(self.ctx, byref(n)), "launch_count")
        return n.value

    def device_bytes(self) -> int:
        n = c_int64()
        check(self.lib.lymph_device_bytes(self.ctx, byref(n)), "device_bytes")
        return n.value


def run_reference_driver(solver: MatrixFree, stop_time: float, max_steps: int = -1, forcing=None):
    """Replays Lymph3D.f90:262-518 for test_num = 1 (manufactured solution):
    matrices, rhs_stat (null data), rhs_dyn (f_time, gd, gn), initial
    conditions, first step, the `t <= stop_time` loop, exact-solution
    projection scaled by time_function(t), and the L2 / DG errors.
    Returns dict(n_steps, t, err_L2, err_DG)."""
    s = solver
    s.MAKE_MATRICES_FREE()
    s.MAKE_RHS_FREE(RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
    f, gd, gn = forcing or (_lib.F_TIME, _lib.GD, _lib.GN)
    s.MAKE_RHS_FREE(RHS_DYN, f, gd, gn)
    t = 0.0
    s.COMPUTE_MODAL_COEFFICIENTS_FREE(FUN_IC_DISPLACEMENT, SLOT_U0)
    s.COMPUTE_MODAL_COEFFICIENTS_FREE(FUN_IC_VELOCITY, SLOT_V0)
    s.FIRST_TIME_STEP_MATRIX_FREE(t)
    t = t + s.dt
    t, n, ms, _ = s.run_steps(t, stop_time, max_steps - 1 if max_steps > 0 else -1)
    s.COMPUTE_MODAL_COEFFICIENTS_FREE(FUN_UEX, SLOT_UEX, time_function(t))
    e2 = s.COMPUTE_ERROR_L2_MATRIX_FREE(SLOT_UN, SLOT_UEX)
    ed = s.COMPUTE_ERROR_DG_MATRIX_FREE(SLOT_UN, SLOT_UEX)
    return {"n_steps": n + 1, "t": t, "err_L2": math.sqrt(e2), "err_DG": math.sqrt(ed), "loop_ms": ms}
