"""Batched ensembles: many independent problems advanced by one persistent
launch per step (lymph_batch_* in include/lymph3d_gpu.h; with matrix-free
neighbour terms, one per degree present).

`make_ensemble` builds the seeded ensemble of uneven problems (cube meshes of
n^3 x 6 tetrahedra, BFS polyhedra, degree p per problem, a Ricker point
source, homogeneous Dirichlet boundaries, each with its own CFL-limited dt);
`Batch` runs them together.  The reference runs one problem per MPI job and
has neither a point-source wavelet nor a real CFL bound (its COMPUTE_CFL,
src/checks.f90:14-39, only compares dt with hmax); both are new here.
"""
from __future__ import annotations

import math
from ctypes import byref, c_double, c_float, c_int32, c_int64, c_void_p

import numpy as np

from . import _lib
from ._lib import check, ptr
from .matrix_free import MatrixFree
from . import mesh as M


def ricker(t: np.ndarray | float, f0: float, t0: float | None = None):
    """Ricker wavelet (1 - 2 pi^2 f0^2 (t-t0)^2) exp(-pi^2 f0^2 (t-t0)^2),
    delayed by t0 = 1.2 / f0 so that it starts near zero."""
    if t0 is None:
        t0 = 1.2 / f0
    a = (math.pi * f0 * (np.asarray(t, dtype=np.float64) - t0)) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


def time_sequence(t_start: float, dt: float, n: int) -> np.ndarray:
    """t_k by repeated addition, the way the reference's loop advances t."""
    out = np.empty(n)
    t = t_start
    for k in range(n):
        out[k] = t
        t = t + dt
    return out


def max_eigenvalue(s: MatrixFree, iters: int = 60) -> float:
    lam = c_double()
    check(s.lib.lymph_max_eigenvalue(s.ctx, iters, byref(lam)), "lymph_max_eigenvalue")
    return lam.value


def set_dt(s: MatrixFree, dt: float) -> None:
    check(s.lib.lymph_set_dt(s.ctx, dt), "lymph_set_dt")
    s.dt = dt


def point_source(s: MatrixFree, x0, direction, which: int = _lib.RHS_DYN) -> int:
    """rhs = direction phi(x0) on the polyhedron that contains x0."""
    m = s.mesh
    tv = np.ascontiguousarray(m.tet_vert, dtype=np.int32)
    X = np.ascontiguousarray(m.coords, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64)
    d = np.ascontiguousarray(direction, dtype=np.float64)
    tet = c_int32()
    check(s.lib.lymph_mesh_find_tet(m.n_tet, ptr(tv, c_int32), ptr(X, c_double), ptr(x, c_double), byref(tet)),
          "lymph_mesh_find_tet")
    check(s.lib.lymph_make_rhs_point(s.ctx, which, tet.value, ptr(x, c_double), ptr(d, c_double)),
          "lymph_make_rhs_point")
    return tet.value


def double_couple(s: MatrixFree, x0, strike, normal, M0: float, which: int = _lib.RHS_DYN) -> int:
    """Adds the double-couple load of moment (s n^T + n s^T) M0 / |T| on the
    tetrahedron T that contains x0 (lymph_make_rhs_double_couple)."""
    m = s.mesh
    tv = np.ascontiguousarray(m.tet_vert, dtype=np.int32)
    X = np.ascontiguousarray(m.coords, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64)
    sv = np.ascontiguousarray(strike, dtype=np.float64)
    nv = np.ascontiguousarray(normal, dtype=np.float64)
    tet = c_int32()
    check(s.lib.lymph_mesh_find_tet(m.n_tet, ptr(tv, c_int32), ptr(X, c_double), ptr(x, c_double), byref(tet)),
          "lymph_mesh_find_tet")
    check(s.lib.lymph_make_rhs_double_couple(s.ctx, which, tet.value, ptr(sv, c_double), ptr(nv, c_double), M0),
          "lymph_make_rhs_double_couple")
    return tet.value


# The batch kernel's tile shapes: column slices S for p = 1..4 (the C table
# kBatchShapes in csrc/batch.cu); lymph_batch_schedule reports the index.
BATCH_TILE_SHAPES = ((8, 8, 4, 3), (16, 10, 5, 3), (24, 10, 5, 2))


class Batch:
    """Problems advanced together; each keeps its own context."""

    def __init__(self, solvers: list[MatrixFree]):
        self.lib = _lib.load()
        self.solvers = list(solvers)
        arr = (c_void_p * len(solvers))(*[s.ctx for s in solvers])
        h = c_void_p()
        check(self.lib.lymph_batch_create(arr, len(solvers), byref(h)), "lymph_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.lymph_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def autotune(self, trial_steps: int = 3, use_cache: bool = True):
        g, o = c_int32(), c_int32()
        check(self.lib.lymph_batch_autotune(self.h, trial_steps, int(use_cache), byref(g), byref(o)),
              "lymph_batch_autotune")
        return g.value, o.value

    def schedule(self):
        """(grid, order, tile shape) the batch runs with."""
        g, o, sh = c_int32(), c_int32(), c_int32()
        check(self.lib.lymph_batch_schedule(self.h, byref(g), byref(o), byref(sh)), "lymph_batch_schedule")
        return g.value, o.value, sh.value

    def run(self, gvals: np.ndarray) -> float:
        """gvals: (n_problems, n_steps) time-function values; returns the
        device time of the loop in ms."""
        g = np.ascontiguousarray(gvals, dtype=np.float64)
        assert g.shape[0] == len(self.solvers)
        ms = c_float()
        check(self.lib.lymph_batch_run(self.h, g.shape[1], ptr(g, c_double), byref(ms)), "lymph_batch_run")
        return ms.value

    def launch_count(self) -> int:
        n = c_int64()
        check(self.lib.lymph_batch_launch_count(self.h, byref(n)), "lymph_batch_launch_count")
        return n.value


def make_ensemble(n_problems: int = 64, seed: int = 2, n_range=(8, 32), p_range=(1, 4), group=(4, 16),
                  precision: int = _lib.FP64, cfl: float = 0.8, material=(1.0, 1.0, 1.0), eig_iters: int = 60):
    """A seeded ensemble of independent problems.  Returns (solvers, meta) with the
    solvers assembled, sources set, dt chosen as cfl * 2/sqrt(lambda_max) and
    the first leapfrog step taken from rest."""
    rng = np.random.default_rng(seed)
    solvers, meta = [], []
    for k in range(n_problems):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        p = int(rng.integers(p_range[0], p_range[1] + 1))
        f0 = float(rng.uniform(5.0, 20.0))
        x0 = rng.uniform(0.2, 0.8, size=3)
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        m = M.cube(n, bc="dirichlet", agglomeration="bfs", seed=seed * 1000 + k, group=group, material=material)
        s = MatrixFree(m, p, 1.0, precision=precision)
        s.MAKE_MATRICES_FREE()
        s.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
        point_source(s, x0, d)
        lam = max_eigenvalue(s, eig_iters)
        dt = cfl * 2.0 / math.sqrt(lam)
        set_dt(s, dt)
        s.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_DISPLACEMENT, _lib.SLOT_U0)
        s.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_DISPLACEMENT, _lib.SLOT_V0)
        check(s.lib.lymph_first_step_g(s.ctx, float(ricker(0.0, f0))), "lymph_first_step_g")
        solvers.append(s)
        meta.append({"n": n, "p": p, "f0": f0, "x0": x0.tolist(), "dir": d.tolist(), "dt": dt, "lambda_max": lam,
                     "n_poly": s.n_poly, "dofs": 3 * s.Np * s.n_poly, "n_blocks": s.n_blocks})
    return solvers, meta


def ensemble_gvals(meta, n_steps: int, t_start_steps: int = 1) -> np.ndarray:
    """Ricker values of every problem at its own step times t_k = (k+1) dt
    (accumulated), for the steps after the first."""
    g = np.empty((len(meta), n_steps))
    for i, mt in enumerate(meta):
        ts = time_sequence(t_start_steps * mt["dt"], mt["dt"], n_steps)
        g[i] = ricker(ts, mt["f0"])
    return g
