"""The CUDA path on the inputs the reference itself holds, and at the sizes of
the benchmark configurations, against the CPU oracle.

* The reference's own decks src/tests/analytical/tet_{5,25,100,125}
  (committed as tests/golden/decks/*.npz by tests/golden/make_deck_fixtures.py)
  in the reference's own mode: one tetrahedron per polyhedron, boundary tags
  2-4 Dirichlet and 5-7 Neumann (MAKE_PARTITION_AND_MPI_FILES.f90:2105-2109),
  the driver's rho = lambda = mu = 1 override (Lymph3D.f90:196-203).  In this
  mode the oracle is the reference's algorithm itself
  (matrix_free.f90:27-1504 element by element).
  - u^n after every one of 25 steps at the deck's degree and at p = 2..4:
    ||u_gpu - u_ref|| / ||u_ref|| <= max(1e-12, 4 x floor) and <= 1e-12 in the
    mass-matrix norm (the bars of tests/test_gpu_parity.py);
  - the full driver sequence to the deck's own STOPTIME (1,000 steps; 3,183
    for tet_100 at p = 3): step count and final time equal, L2 and DG errors
    within 1e-10 relative of the oracle's committed values;
  - the two mixed operators (tensor-core FP32 blocks, matrix-free FP32
    neighbour terms) on tet_5 and tet_25 at p = 1..4: K u per polyhedron row
    within 2e-6 of the oracle's FP64 K u.
* The 125-polyhedron cube (5^3 hexahedra x 6 tetrahedra, one polyhedron per
  hexahedron, p = 2, rho = lambda = mu = 1, dt = 1e-4, T = 0.1: 1,000 steps by
  the `t <= T` rule of Lymph3D.f90:389-418): L2 / DG errors within 1e-10 of
  the oracle's.
* The 384,000-tetrahedron cube in 46,767 BFS polyhedra at p = 3 (rho = 1,
  lambda = 2, mu = 1, dt = 2e-5): the oracle assembles the whole operator on
  the host (15 GB of blocks) and both sides take three steps from the same
  coefficients; bar 1e-12 relative, Euclidean and mass norm, after each.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib, mesh as M
from lymph3d_apsc_gb300.matrix_free import run_reference_driver as gpu_driver
from oracle.oracle_py import Oracle, run_reference_driver as cpu_driver
from parity_util import TOL_STATE, every_step_parity, mass_norm_rel, rel, start_same

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
TOL_ERR = 1e-10


def deck(name):
    a = dict(np.load(GOLDEN / "decks" / f"{name}.npz"))
    a["name"] = name
    return M.deck_mesh(a)


def deck_golden(name):
    d = json.loads((GOLDEN / "decks" / "deck_driver.json").read_text())
    return next(x for x in d["decks"] if x["deck"] == name)


@pytest.mark.parametrize("name,p", [("tet_5", 1), ("tet_5", 2), ("tet_5", 3), ("tet_5", 4), ("tet_25", 1),
                                    ("tet_25", 2), ("tet_25", 4), ("tet_100", 3), ("tet_125", 1), ("tet_125", 2)])
def test_deck_every_step(require_gpu, name, p):
    m, prm = deck(name)
    assert m.info["unfound_tria"] == 0
    with MatrixFree(m, p, prm["dt"]) as g:
        o = Oracle(m, p, prm["dt"])
        g.MAKE_MATRICES_FREE()
        o.make_matrices()
        e, floor, worst = every_step_parity(m, p, g, o, n_steps=25)
        o.close()
    assert worst <= 1.0
    print(f"{name} p={p}: device vs oracle {e:.2e}, floor {floor:.2e}")


@pytest.mark.parametrize("name", ["tet_5", "tet_25", "tet_100", "tet_125"])
def test_deck_driver_to_stoptime(require_gpu, name):
    """The deck run as the reference's driver runs it: its degree, TIMESTEP
    and STOPTIME; errors against the oracle's committed values."""
    m, prm = deck(name)
    gold = deck_golden(name)
    with MatrixFree(m, prm["degree"], prm["dt"]) as g:
        r = gpu_driver(g, prm["stop_time"])
    assert r["n_steps"] == gold["n_steps"] and r["t"] == gold["t_final"]
    assert abs(r["err_L2"] - gold["err_L2"]) <= TOL_ERR * gold["err_L2"], (r["err_L2"], gold["err_L2"])
    assert abs(r["err_DG"] - gold["err_DG"]) <= TOL_ERR * gold["err_DG"], (r["err_DG"], gold["err_DG"])


def test_c0_full_run(require_gpu):
    """5^3 x 6 tetrahedra, 125 polyhedra, p = 2, dt = 1e-4 to T = 0.1."""
    gold = json.loads((GOLDEN / "c0_driver.json").read_text())
    m = M.cube(5, bc="dirichlet", agglomeration="hex")
    assert np.array_equal(m.tet_poly, np.load(GOLDEN / "elem_in_poly.npz")["c0"])
    with MatrixFree(m, 2, 1e-4) as g:
        r = gpu_driver(g, 0.1)
    o = Oracle(m, 2, 1e-4)
    ro = cpu_driver(o, 0.1)
    o.close()
    assert r["n_steps"] == ro["n_steps"] == gold["n_steps"] == 1000
    assert r["t"] == ro["t"] == gold["t_final"]
    for k in ("err_L2", "err_DG"):
        assert abs(ro[k] - gold[k]) <= 1e-12 * gold[k], k
        assert abs(r[k] - ro[k]) <= TOL_ERR * ro[k], (k, r[k], ro[k])


def test_c1_scale_three_steps(require_gpu):
    """The 46,767-polyhedron p = 3 operator of the benchmark, assembled by
    the oracle on the host, three steps against the device."""
    m = M.cube(40, bc="dirichlet", agglomeration="bfs", seed=0, group=(4, 12), material=(1.0, 2.0, 1.0))
    assert np.array_equal(m.tet_poly, np.load(GOLDEN / "elem_in_poly.npz")["c1"])
    p, dt = 3, 2e-5
    with MatrixFree(m, p, dt) as g:
        o = Oracle(m, p, dt)
        g.MAKE_MATRICES_FREE()
        o.make_matrices()
        start_same(g, o)
        Mm = o.mass(1)
        t = 0.0
        for k in range(3):
            if k == 0:
                g.FIRST_TIME_STEP_MATRIX_FREE(t)
                o.first_step(t)
            else:
                g.TIME_STEP_MATRIX_FREE(t)
                o.step(t)
            t += dt
            ref = o.get_state(_lib.SLOT_UN)
            got = g.get_state(_lib.SLOT_UN)
            e, em = rel(got, ref), mass_norm_rel(o, got, ref, Mm)
            print(f"c1 step {k}: relative {e:.2e}, mass norm {em:.2e}")
            assert e <= TOL_STATE and em <= TOL_STATE, (k, e, em)
        o.close()


@pytest.mark.parametrize("name", ["tet_5", "tet_25"])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_deck_mixed_operators(require_gpu, name, p):
    """The two mixed operators on the reference's decks (Dirichlet and Neumann
    faces, one tetrahedron per polyhedron): K u of every polyhedron row, FP32
    blocks from the tensor cores and the matrix-free FP32 neighbour terms,
    against the oracle's FP64 K u: <= TOL_APPLY_FP32 (2e-6) per row."""
    from parity_util import TOL_APPLY_FP32, oracle_apply, row_rel_max
    m, prm = deck(name)
    o = Oracle(m, p, prm["dt"])
    o.make_matrices()
    u = np.random.default_rng(20 + p).standard_normal((o.n_poly, o.nd))
    want = oracle_apply(o, u)
    o.close()
    for prec in (_lib.MIXED, _lib.MIXED_MF):
        with MatrixFree(m, p, prm["dt"], precision=prec) as g:
            g.MAKE_MATRICES_FREE()
            e = row_rel_max(g.apply_operator(u), want)
        print(f"{name} p={p} precision {prec}: {e:.2e}")
        assert e <= TOL_APPLY_FP32, (prec, e)
