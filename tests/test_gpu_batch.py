"""GPU tests of the multi-problem persistent launch, the point source and the
CFL bound.

* a batch of uneven problems (degrees 1-4, different meshes and dt) advanced
  by lymph_batch_run equals each problem stepped alone, bit for bit, in FP64,
  with FP32 blocks and with matrix-free neighbour terms;
* the autotuner leaves every problem's state as it found it;
* the point-source RHS is the delta functional: b . c = dir . u_h(x0);
* lymph_max_eigenvalue matches the largest |eigenvalue| of M^-1 K built
  densely from the oracle's blocks (1 %), dt from it is stable and 3x that
  dt is reported as EXIT_INSTAB (never a fault).
"""
import math

import numpy as np
import pytest
from numpy.polynomial import legendre as npleg

from lymph3d_apsc_gb300 import MatrixFree, _lib, mesh as M, time_function
from lymph3d_apsc_gb300 import ensemble as E
from lymph3d_apsc_gb300._lib import LymphError

pytestmark = pytest.mark.gpu

SPECS = [  # (mesh kwargs, degree, dt)
    (dict(n=2, agglomeration="tet"), 1, 1e-3),
    (dict(n=2, agglomeration="bfs", group=(4, 12), jitter=0.2), 2, 7e-4),
    (dict(n=3, agglomeration="bfs", group=(4, 16), seed=3, jitter=0.1), 3, 5e-4),
    (dict(n=2, agglomeration="hex", material=(1.0, 2.0, 1.0)), 4, 2e-4),
    (dict(n=3, bc="reference", agglomeration="bfs", group=(4, 12), seed=5), 4, 2e-4),
    (dict(n=1, bc="reference", agglomeration="hex"), 3, 5e-4),  # one polyhedron, no neighbours
]


def _prepared(spec, precision=_lib.FP64):
    kw, p, dt = spec
    s = MatrixFree(M.cube(**kw), p, dt, precision=precision)
    s.MAKE_MATRICES_FREE()
    s.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
    s.MAKE_RHS_FREE(_lib.RHS_DYN, _lib.F_TIME, _lib.GD, _lib.GN)
    s.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_DISPLACEMENT, _lib.SLOT_U0)
    s.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_VELOCITY, _lib.SLOT_V0)
    s.FIRST_TIME_STEP_MATRIX_FREE(0.0)
    return s


def _gvals(solvers, n):
    return np.array([[time_function(t) for t in E.time_sequence(s.dt, s.dt, n)] for s in solvers])


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED, _lib.MIXED_MF])
@pytest.mark.parametrize("n_steps", [37, 5])
def test_batch_equals_single_contexts_bitwise(require_gpu, precision, n_steps):
    batch_solvers = [_prepared(sp, precision) for sp in SPECS]
    alone = [_prepared(sp, precision) for sp in SPECS]
    b = E.Batch(batch_solvers)
    ms = b.run(_gvals(batch_solvers, n_steps))
    # the step kernel and the counter bump; matrix-free: the FP32 copy of u^n
    # and one step kernel per degree present
    per_step = 2 + len({sp[1] for sp in SPECS}) if precision == _lib.MIXED_MF else 2
    assert ms > 0 and b.launch_count() == per_step * n_steps
    for s, a in zip(batch_solvers, alone):
        a.run_steps(a.dt, 1e9, max_steps=n_steps)
        assert np.array_equal(s.get_state(_lib.SLOT_UN), a.get_state(_lib.SLOT_UN))
        assert np.array_equal(s.get_state(_lib.SLOT_U0), a.get_state(_lib.SLOT_U0))
    b.close()
    for x in batch_solvers + alone:
        x.close()


def test_autotune_restores_state_and_choice_is_valid(require_gpu, tmp_path, monkeypatch):
    monkeypatch.setenv("LYMPH_TUNE_CACHE", str(tmp_path / "tune.txt"))
    batch_solvers = [_prepared(sp) for sp in SPECS]
    alone = [_prepared(sp) for sp in SPECS]
    b = E.Batch(batch_solvers)
    before = [s.get_state(_lib.SLOT_UN).copy() for s in batch_solvers]
    grid, order = b.autotune(trial_steps=2, use_cache=False)
    assert grid % 152 == 0 or grid > 0
    assert order in (0, 1)
    for s, u in zip(batch_solvers, before):
        assert np.array_equal(s.get_state(_lib.SLOT_UN), u)
    assert (tmp_path / "tune.txt").exists()
    assert b.autotune(trial_steps=2, use_cache=True) == (grid, order)
    g2, o2, shape = b.schedule()
    assert (g2, o2) == (grid, order) and shape in (0, 1, 2)
    b.run(_gvals(batch_solvers, 20))
    for s, a in zip(batch_solvers, alone):
        a.run_steps(a.dt, 1e9, max_steps=20)
        ub, ua = s.get_state(_lib.SLOT_UN), a.get_state(_lib.SLOT_UN)
        if shape == 0:
            assert np.array_equal(ub, ua)
        else:  # another grouping of the same FP64 sums
            assert np.linalg.norm(ub - ua) <= 1e-11 * np.linalg.norm(ua)
    b.close()
    for x in batch_solvers + alone:
        x.close()


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED])
@pytest.mark.parametrize("shape", [1, 2])
def test_batch_tile_shapes_agree_with_single_contexts(require_gpu, tmp_path, monkeypatch, precision, shape):
    """Every tile shape the autotuner may pick is deterministic and gives the
    single-context result up to the rounding of another grouping of the row
    sums: FP64 blocks within 1e-11 relative after 20 steps; FP32 blocks no
    further from the FP64 result than 3x the single-context FP32 run is."""
    monkeypatch.setenv("LYMPH_TUNE_CACHE", str(tmp_path / "tune.txt"))
    batch_solvers = [_prepared(sp, precision) for sp in SPECS]
    again = [_prepared(sp, precision) for sp in SPECS]
    alone = [_prepared(sp, precision) for sp in SPECS]
    ref64 = [_prepared(sp, _lib.FP64) for sp in SPECS]
    # force the shape through the cache: tune once, then rewrite the entry
    b = E.Batch(batch_solvers)
    grid, order = b.autotune(trial_steps=1, use_cache=False)
    b.close()
    key = (tmp_path / "tune.txt").read_text().split()[0]
    (tmp_path / "tune.txt").write_text(f"{key} {grid} {order} {shape}\n")
    runs = []
    for solvers in (batch_solvers, again):
        bb = E.Batch(solvers)
        assert bb.schedule()[2] == shape
        bb.run(_gvals(solvers, 20))
        runs.append([s.get_state(_lib.SLOT_UN) for s in solvers])
        bb.close()
    for ub, ub2, a, r in zip(runs[0], runs[1], alone, ref64):
        assert np.array_equal(ub, ub2)
        a.run_steps(a.dt, 1e9, max_steps=20)
        ua = a.get_state(_lib.SLOT_UN)
        if precision == _lib.FP64:
            assert np.linalg.norm(ub - ua) <= 1e-11 * np.linalg.norm(ua)
        else:
            r.run_steps(r.dt, 1e9, max_steps=20)
            u64 = r.get_state(_lib.SLOT_UN)
            assert np.linalg.norm(ub - u64) <= 3.0 * np.linalg.norm(ua - u64) + 1e-12 * np.linalg.norm(u64)
    for x in batch_solvers + again + alone + ref64:
        x.close()


def _basis_at(x0, bbox, p):
    from oracle import oracle_py as O
    lib = O.load()
    Np = (p + 1) * (p + 2) * (p + 3) // 6
    bl = np.empty(3 * Np, np.int32)
    lib.oracle_basis_list(p, bl.ctypes.data_as(O.POINTER(O.ctypes.c_int)))
    bl = bl.reshape(Np, 3)
    vals = np.ones(Np)
    for d in range(3):
        a, b = bbox[2 * d], bbox[2 * d + 1]
        hb, mb = (b - a) / 2, (b + a) / 2
        xp = (x0[d] - mb) / hb
        for f in range(Np):
            c = np.zeros(bl[f, d] + 1)
            c[-1] = 1.0
            vals[f] *= npleg.legval(xp, c) / math.sqrt(hb)
    return vals


@pytest.mark.parametrize("p", [1, 3, 4])
def test_point_source_is_the_delta_functional(require_gpu, p):
    m = M.cube(3, agglomeration="bfs", group=(4, 12), jitter=0.2)
    s = MatrixFree(m, p, 1e-3)
    s.MAKE_MATRICES_FREE()
    x0, d = np.array([0.41, 0.37, 0.63]), np.array([0.6, -0.48, 0.64])
    tet = E.point_source(s, x0, d)
    b = s.rhs(_lib.RHS_DYN)
    P = int(m.tet_poly[tet])
    assert np.count_nonzero(np.abs(b).sum(axis=1)) == 1 and np.abs(b[P]).sum() > 0
    bb, _ = s.poly_geometry()
    phi = _basis_at(x0, bb[P], p)
    c = np.random.default_rng(1).standard_normal(b.shape)
    uh = np.array([phi @ c[P, i * s.Np:(i + 1) * s.Np] for i in range(3)])
    assert abs(np.sum(b * c) - d @ uh) <= 1e-12 * np.abs(b).sum() * np.abs(c).max()
    s.close()


def test_max_eigenvalue_matches_dense_spectrum(require_gpu):
    from oracle.oracle_py import Oracle
    m = M.cube(2, agglomeration="bfs", group=(4, 12), jitter=0.2, material=(1.0, 2.0, 1.0))
    p = 2
    s = MatrixFree(m, p, 1e-3)
    s.MAKE_MATRICES_FREE()
    lam = E.max_eigenvalue(s, 300)
    o = Oracle(m, p, 1e-3)
    o.make_matrices()
    nd, npoly = o.nd, o.n_poly
    K = np.zeros((npoly * nd, npoly * nd))
    for (P, Q), blk in o.block_dict(0).items():
        K[P * nd:(P + 1) * nd, Q * nd:(Q + 1) * nd] = blk
    Mi = np.zeros_like(K)
    for P, Mp in enumerate(o.mass(0)):
        inv = np.linalg.inv(Mp)
        for i in range(3):
            sl = slice(P * nd + i * o.Np, P * nd + (i + 1) * o.Np)
            Mi[sl, sl] = inv
    ev = np.abs(np.linalg.eigvals(Mi @ K)).max()
    assert abs(lam - ev) <= 0.01 * ev
    s.close()
    o.close()


def test_cfl_dt_is_stable_and_3x_is_reported_unstable(require_gpu):
    def run(factor):
        m = M.cube(3, agglomeration="bfs", group=(4, 12), seed=2)
        s = MatrixFree(m, 2, 1.0)
        s.MAKE_MATRICES_FREE()
        s.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
        E.point_source(s, [0.5, 0.45, 0.55], [0.0, 0.0, 1.0])
        lam = E.max_eigenvalue(s, 80)
        E.set_dt(s, factor * 2.0 / math.sqrt(lam))
        f0 = 12.0
        s.lib.lymph_first_step_g(s.ctx, float(E.ricker(0.0, f0)))
        g = E.ricker(E.time_sequence(s.dt, s.dt, 400), f0)
        b = E.Batch([s])
        try:
            b.run(g[None, :])
            u = s.get_state(_lib.SLOT_UN)
            return np.abs(u).max()
        finally:
            b.close()
            s.close()

    amp = run(0.8)
    assert np.isfinite(amp) and 0 < amp < 1e3
    with pytest.raises(LymphError) as e:
        run(3.0)
    assert e.value.code == _lib.LYMPH_EXIT_INSTAB


def test_small_ensemble_runs(require_gpu, tmp_path, monkeypatch):
    monkeypatch.setenv("LYMPH_TUNE_CACHE", str(tmp_path / "tune.txt"))
    solvers, meta = E.make_ensemble(n_problems=6, seed=2, n_range=(2, 4), p_range=(1, 4))
    assert {mt["p"] for mt in meta} <= {1, 2, 3, 4}
    b = E.Batch(solvers)
    b.autotune(trial_steps=2)
    ms = b.run(E.ensemble_gvals(meta, 64))
    assert ms > 0
    for s in solvers:
        u = s.get_state(_lib.SLOT_UN)
        assert np.all(np.isfinite(u)) and np.abs(u).max() > 0
    b.close()
    for s in solvers:
        s.close()
