"""ctypes wrapper of the CPU oracle (oracle/lymph_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline arm of bench.py, as the checker.  The product never imports it.
"""
from __future__ import annotations

import ctypes
import math
import subprocess
from ctypes import POINTER, byref, c_char_p, c_double, c_int, c_int32, c_int64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liblymph_oracle.so"
# the same source built -O3 with FMA contraction: the timed CPU runs only
LIB_TIMING = HERE / "_build" / "liblymph_oracle_timing.so"

_libs = {}


def build() -> Path:
    src = HERE / "lymph_oracle.cpp"
    hdr = HERE.parent / "include" / "lymph3d_gpu.h"
    newest = max(src.stat().st_mtime, hdr.stat().st_mtime)
    if any(not p.exists() or p.stat().st_mtime < newest for p in (LIB, LIB_TIMING)):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load(timing: bool = False):
    """The checker library (FP contraction off), or with timing=True the
    -O3 build used only to time the CPU baseline."""
    key = "timing" if timing else "parity"
    if key not in _libs:
        build()
        lib = ctypes.CDLL(str(LIB_TIMING if timing else LIB))
        P_I32, P_F64 = POINTER(c_int32), POINTER(c_double)
        sigs = {
            "oracle_last_error": (c_char_p, []),
            "oracle_num_threads": (c_int, []),
            "oracle_set_data_perturbation": (None, [c_int]),
            "oracle_set_reverse_sums": (None, [c_int]),
            "oracle_set_explicit_inverse": (None, [c_int]),
            "oracle_set_device_order": (None, [c_int]),
            "oracle_set_planted_mistake": (None, [c_int]),
            "oracle_set_assemble_dg": (None, [c_int]),
            "oracle_set_threads": (None, [c_int]),
            "oracle_create": (c_int, [c_void_p, c_int, c_double, c_double, c_double, POINTER(c_void_p)]),
            "oracle_destroy": (c_int, [c_void_p]),
            "oracle_make_matrices": (c_int, [c_void_p]),
            "oracle_make_rhs": (c_int, [c_void_p, c_int, c_int, c_int, c_int]),
            "oracle_modal_project": (c_int, [c_void_p, c_int, c_int, c_double]),
            "oracle_first_step": (c_int, [c_void_p, c_double]),
            "oracle_step": (c_int, [c_void_p, c_double]),
            "oracle_run_steps": (c_int, [c_void_p, c_double, c_int64, P_F64, POINTER(c_int64)]),
            "oracle_get_state": (c_int, [c_void_p, c_int, P_F64]),
            "oracle_nodal_values": (c_int, [c_void_p, c_int, P_F64]),
            "oracle_make_rhs_double_couple": (c_int, [c_void_p, c_int, c_int, P_F64, P_F64, c_double]),
            "oracle_set_state": (c_int, [c_void_p, c_int, P_F64]),
            "oracle_error_l2": (c_int, [c_void_p, c_int, c_int, P_F64]),
            "oracle_error_dg": (c_int, [c_void_p, c_int, c_int, P_F64]),
            "oracle_get_pattern": (c_int, [c_void_p, P_I32, P_I32, POINTER(c_int64)]),
            "oracle_get_blocks": (c_int, [c_void_p, c_int, P_F64]),
            "oracle_get_mass": (c_int, [c_void_p, c_int, P_F64]),
            "oracle_get_rhs": (c_int, [c_void_p, c_int, P_F64]),
            "oracle_get_poly_geometry": (c_int, [c_void_p, P_F64, P_F64]),
            "oracle_get_kloc_reference_layout": (c_int, [c_void_p, c_int, P_F64]),
            "oracle_quadrature": (c_int, [c_int, POINTER(c_int), POINTER(c_int), P_F64, P_F64, P_F64, P_F64]),
            "oracle_gl1d": (c_int, [c_int, P_F64, P_F64]),
            "oracle_gauleg": (c_int, [c_int, P_F64, P_F64]),
            "oracle_basis_list": (c_int, [c_int, POINTER(c_int)]),
            "oracle_legendre": (c_int, [c_int, P_F64, c_int, c_double, c_double, P_F64, P_F64]),
            "oracle_cholesky": (c_int, [P_F64, c_int, P_F64]),
            "oracle_solve_lu": (c_int, [P_F64, P_F64, c_int, P_F64]),
            "oracle_time_function": (c_double, [c_double]),
            "oracle_match_faces": (c_int, [c_int, P_I32, P_I32, P_I32]),
            "oracle_neighbour_apply_pointwise": (c_int, [c_void_p, c_int, c_int, P_F64, P_F64]),
            "oracle_neighbour_apply_rule": (c_int, [c_void_p, c_int, c_int, P_F64, c_int, P_F64, P_F64]),
        }
        for k, (r, a) in sigs.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _libs[key] = lib
    return _libs[key]


def _p(a, t=c_double):
    return a.ctypes.data_as(POINTER(t))


class Oracle:
    """CPU FP64 restatement of the reference path for one problem."""

    def __init__(self, mesh, degree: int, dt: float, alpha: float = 10.0, theta: float = -1.0, timing: bool = False):
        self.lib = load(timing)
        self.mesh = mesh
        self._desc = mesh.desc()
        h = c_void_p()
        rc = self.lib.oracle_create(ctypes.addressof(self._desc), degree, alpha, theta, dt, byref(h))
        if rc:
            raise RuntimeError(f"oracle_create failed ({rc})")
        self.h = h
        self.degree, self.dt = degree, dt
        self.Np = (degree + 1) * (degree + 2) * (degree + 3) // 6
        self.nd = 3 * self.Np
        self.n_poly = mesh.n_poly
        self.n_tet = mesh.n_tet

    def close(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc:
            raise RuntimeError(f"{what}: [{rc}] {self.lib.oracle_last_error().decode()}")

    def make_matrices(self):
        self._chk(self.lib.oracle_make_matrices(self.h), "make_matrices")

    def make_rhs(self, which, f, d, n):
        self._chk(self.lib.oracle_make_rhs(self.h, which, f, d, n), "make_rhs")

    def modal_project(self, fun, slot, scale=1.0):
        self._chk(self.lib.oracle_modal_project(self.h, fun, slot, scale), "modal_project")

    def first_step(self, t):
        self._chk(self.lib.oracle_first_step(self.h, t), "first_step")

    def step(self, t):
        self._chk(self.lib.oracle_step(self.h, t), "step")

    def run_steps(self, t, stop_time, max_steps=-1):
        tt = c_double(t)
        n = c_int64()
        self._chk(self.lib.oracle_run_steps(self.h, stop_time, max_steps, byref(tt), byref(n)), "run_steps")
        return tt.value, n.value

    def make_rhs_double_couple(self, which, tet, strike, normal, M0):
        sv = np.ascontiguousarray(strike, np.float64)
        nv = np.ascontiguousarray(normal, np.float64)
        self._chk(self.lib.oracle_make_rhs_double_couple(self.h, which, tet, _p(sv), _p(nv), M0),
                  "make_rhs_double_couple")

    def nodal_values(self, slot):
        """EXPORT_SOLUTION's vertex evaluation: [n_tet, 4, 3]."""
        out = np.empty((self.n_tet, 4, 3))
        rc = self.lib.oracle_nodal_values(self.h, slot, _p(out))
        if rc:
            raise RuntimeError(f"oracle_nodal_values: {rc}")
        return out

    def get_state(self, slot):
        out = np.empty((self.n_poly, self.nd))
        self.lib.oracle_get_state(self.h, slot, _p(out))
        return out

    def set_state(self, slot, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.lib.oracle_set_state(self.h, slot, _p(v))

    def error_l2(self, a, b):
        o = c_double()
        self.lib.oracle_error_l2(self.h, a, b, byref(o))
        return o.value

    def error_dg(self, a, b):
        o = c_double()
        self.lib.oracle_error_dg(self.h, a, b, byref(o))
        return o.value

    def pattern(self):
        nb = c_int64()
        self.lib.oracle_get_pattern(self.h, None, None, byref(nb))
        rp = np.empty(self.n_poly + 1, np.int32)
        col = np.empty(nb.value, np.int32)
        self.lib.oracle_get_pattern(self.h, _p(rp, c_int32), _p(col, c_int32), None)
        return rp, col

    def blocks(self, which=0):
        rp, col = self.pattern()
        out = np.empty((col.size, self.nd, self.nd))
        self.lib.oracle_get_blocks(self.h, which, _p(out))
        return out

    def neighbour_apply_pointwise(self, P, Q, uq):
        """K_PQ u_Q from the face quadrature point by point (FP64)."""
        uq = np.ascontiguousarray(uq, dtype=np.float64)
        out = np.empty(self.nd)
        self._chk(self.lib.oracle_neighbour_apply_pointwise(self.h, int(P), int(Q), _p(uq), _p(out)),
                  "oracle_neighbour_apply_pointwise")
        return out

    def neighbour_apply_rule(self, P, Q, uq, xyw):
        """The same with a caller's triangle rule: xyw = (xi, eta, w) per node
        on the reference triangle (weights summing to 1/2)."""
        uq = np.ascontiguousarray(uq, dtype=np.float64)
        r = np.ascontiguousarray(xyw, dtype=np.float64)
        out = np.empty(self.nd)
        self._chk(self.lib.oracle_neighbour_apply_rule(self.h, int(P), int(Q), _p(uq), r.size // 3, _p(r), _p(out)),
                  "oracle_neighbour_apply_rule")
        return out

    def block_dict(self, which=0):
        rp, col = self.pattern()
        vals = self.blocks(which)
        d = {}
        for P in range(self.n_poly):
            for k in range(rp[P], rp[P + 1]):
                d[(P, int(col[k]))] = vals[k]
        return d

    def mass(self, which):
        out = np.empty((self.n_poly, self.Np, self.Np))
        self.lib.oracle_get_mass(self.h, which, _p(out))
        return out

    def rhs(self, which):
        out = np.empty((self.n_poly, self.nd))
        self.lib.oracle_get_rhs(self.h, which, _p(out))
        return out

    def poly_geometry(self):
        bb = np.empty((self.n_poly, 6))
        hk = np.empty(self.n_poly)
        self.lib.oracle_get_poly_geometry(self.h, _p(bb), _p(hk))
        return bb, hk


def run_reference_driver(o: Oracle, stop_time: float, max_steps: int = -1):
    """Lymph3D.f90:262-518 on the oracle (same sequence as the GPU driver)."""
    o.make_matrices()
    o.make_rhs(0, 0, 0, 0)
    o.make_rhs(1, 1, 1, 1)
    o.modal_project(0, 0)
    o.modal_project(1, 2)
    t = 0.0
    o.first_step(t)
    t = t + o.dt
    t, n = o.run_steps(t, stop_time, max_steps - 1 if max_steps > 0 else -1)
    g = load().oracle_time_function(t)
    o.modal_project(2, 3, g)
    e2 = o.error_l2(1, 3)
    ed = o.error_dg(1, 3)
    return {"n_steps": n + 1, "t": t, "err_L2": math.sqrt(e2), "err_DG": math.sqrt(ed)}
