"""Known-answer tests that pin the CPU oracle's mathematics.

The reference ships no golden vectors and cannot be compiled here (Fortran
+ MPI), so the oracle is pinned by properties its algorithm must have:
quadrature exactness, Legendre normalisation, SPD mass matrices, rigid-body
modes in the kernel of the operator, symmetry for SIPG, convergence rates of
the L2 projection, and the committed golden values of small runs
(tests/golden/, produced by tests/golden/make_golden.py).
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from lymph3d_apsc_gb300 import mesh as M
from oracle import oracle_py as O

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_quadrature_weights_sum_to_reference_volumes():
    lib = O.load()
    for p in range(1, 8):
        nq3, nq2 = O.c_int(), O.c_int()
        n3, n2 = (p + 1) ** 3, (p + 1) ** 2
        w3, w2 = np.empty(n3), np.empty(n2)
        x3, x2 = np.empty(4 * n3), np.empty(4 * n2)
        lib.oracle_quadrature(p, O.byref(nq3), O.byref(nq2), O._p(x3), O._p(w3), O._p(x2), O._p(w2))
        assert nq3.value == n3 and nq2.value == n2
        assert abs(w3.sum() - 1.0 / 6.0) < 1e-15
        assert abs(w2.sum() - 0.5) < 1e-15
        # nodes inside the reference simplex
        x3 = x3.reshape(n3, 4)
        assert np.all(x3[:, :3] >= 0) and np.all(x3[:, :3].sum(1) <= 1 + 1e-15)
        # xi^k (1-a)^2 in the collapsed variable: exact for k <= 2p-1; int_T xi^k = k!/(k+3)!
        k = 2 * p - 1
        exact = math.factorial(k) / math.factorial(k + 3)
        assert abs(np.sum(w3 * x3[:, 0] ** k) - exact) < 1e-14


def test_hardcoded_gauss_legendre_tables_match_gauleg():
    lib = O.load()
    for n in range(2, 8):
        xt, wt = np.empty(n), np.empty(n)
        xg, wg = np.empty(n), np.empty(n)
        lib.oracle_gl1d(n, O._p(xt), O._p(wt))
        lib.oracle_gauleg(n, O._p(xg), O._p(wg))
        it, ig = np.argsort(xt), np.argsort(xg)
        assert np.allclose(xt[it], xg[ig], atol=1e-15, rtol=0)
        assert np.allclose(wt[it], wg[ig], atol=1e-14, rtol=0)
        assert abs(wt.sum() - 2.0) < 1e-14


@pytest.mark.parametrize("deg", range(0, 8))
def test_scaled_legendre_orthogonality_on_bbox(deg):
    lib = O.load()
    n = 12
    x, w = np.empty(n), np.empty(n)
    lib.oracle_gauleg(n, O._p(x), O._p(w))
    a, b = 0.3, 1.7
    xs = 0.5 * (b - a) * x + 0.5 * (b + a)
    ws = 0.5 * (b - a) * w
    vals = {}
    for q in range(8):
        v, d = np.empty(n), np.empty(n)
        lib.oracle_legendre(n, O._p(xs), q, a, b, O._p(v), O._p(d))
        vals[q] = (v, d)
    for q in range(8):
        ip = float(np.sum(ws * vals[deg][0] * vals[q][0]))
        assert abs(ip - (2.0 / (2 * deg + 1) if q == deg else 0.0)) < 1e-13
    # derivative: d/dx L_p(xp)/sqrt(hb) = L'_p / (hb sqrt(hb)); check by finite differences
    hb = 0.5 * (b - a)
    v0, d0 = vals[deg]
    eps = 1e-6
    vp, vm = np.empty(n), np.empty(n)
    xp, xm = xs + eps, xs - eps  # keep the arrays alive across the calls
    lib.oracle_legendre(n, O._p(xp), deg, a, b, O._p(vp), None)
    lib.oracle_legendre(n, O._p(xm), deg, a, b, O._p(vm), None)
    fd = (vp - vm) / (2 * eps)
    if deg == 6:
        # the reference's hard-coded derivative of degree 6 carries a spurious
        # "- 5" constant (GradLegendreP, basis_function.f90:410); the oracle
        # keeps it, so L'_6 is off by -5/16 / (hb sqrt(hb)) everywhere
        fd = fd - 5.0 / 16.0 / (hb * math.sqrt(hb))
    assert np.allclose(fd, d0, atol=1e-6 * max(1, np.abs(d0).max()))


def test_basis_list_order_and_size():
    lib = O.load()
    for p in range(1, 7):
        Np = (p + 1) * (p + 2) * (p + 3) // 6
        bl = np.empty(3 * Np, np.int32)
        got = lib.oracle_basis_list(p, bl.ctypes.data_as(O.POINTER(O.ctypes.c_int)))
        bl = bl.reshape(Np, 3)
        assert got == Np
        assert tuple(bl[0]) == (p, 0, 0) and tuple(bl[-1]) == (0, 0, 0)
        assert np.all(bl.sum(1) <= p) and len({tuple(r) for r in bl}) == Np


def test_cholesky_and_solve_lu():
    lib = O.load()
    rng = np.random.default_rng(0)
    for n in (4, 10, 35):
        a = rng.standard_normal((n, n))
        A = a @ a.T + n * np.eye(n)
        R = np.empty((n, n))
        A = np.ascontiguousarray(A)
        assert lib.oracle_cholesky(O._p(A), n, O._p(R)) == 0
        assert np.allclose(np.triu(R), R) and np.allclose(R.T @ R, A, atol=1e-12 * np.abs(A).max())
        b = rng.standard_normal(n)
        x = np.empty(n)
        lib.oracle_solve_lu(O._p(R), O._p(b), n, O._p(x))
        assert np.allclose(A @ x, b, atol=1e-10)
    B, RB = -np.eye(3), np.empty((3, 3))
    assert lib.oracle_cholesky(O._p(B), 3, O._p(RB)) == 5  # EXIT_SINGULARMTX


@pytest.mark.parametrize("agg", ["tet", "hex", "bfs"])
def test_mass_is_spd_and_factor_reconstructs(agg):
    m = M.cube(2, agglomeration=agg, group=(4, 12), jitter=0.2)
    o = O.Oracle(m, 3, 1e-3)
    o.make_matrices()
    Mm, R = o.mass(1), o.mass(3)
    assert np.allclose(Mm, Mm.transpose(0, 2, 1), atol=1e-15)
    assert np.all(np.linalg.eigvalsh(Mm) > 0)
    assert np.allclose(np.einsum("pki,pkj->pij", R, R), Mm, atol=1e-13)


def _apply_K(o, u):
    rp, col = o.pattern()
    vals = o.blocks(0)
    y = np.zeros_like(u)
    for P in range(o.n_poly):
        for k in range(rp[P], rp[P + 1]):
            y[P] += vals[k] @ u[col[k]]
    return y


@pytest.mark.parametrize("lam,mu", [(1.0, 1.0), (2.0, 1.0)])
def test_operator_kills_translations_all_neumann(lam, mu):
    """With no Dirichlet face, K u = 0 for a constant displacement
    (no strain, no jump)."""
    m = M.cube(2, bc="dirichlet", agglomeration="bfs", group=(4, 12), material=(1.0, lam, mu), jitter=0.2)
    neigh = m.neigh.copy()
    neigh[neigh == -1] = -2  # every boundary face Neumann
    m.neigh = neigh
    o = O.Oracle(m, 2, 1e-3)
    o.make_matrices()
    u = np.zeros((o.n_poly, o.nd))
    # constant basis function is the last one (blist (0,0,0)); value 1/sqrt(hx hy hz)
    bb, _ = o.poly_geometry()
    hx, hy, hz = (bb[:, 1] - bb[:, 0]) / 2, (bb[:, 3] - bb[:, 2]) / 2, (bb[:, 5] - bb[:, 4]) / 2
    c = np.sqrt(hx * hy * hz)
    for i, amp in enumerate((0.3, -1.2, 0.7)):
        u[:, i * o.Np + o.Np - 1] = amp * c
    y = _apply_K(o, u)
    scale = max(abs(b).max() for b in o.blocks(0)) * np.abs(u).max()
    assert np.abs(y).max() <= 1e-12 * scale


def test_operator_symmetric_for_sipg_homogeneous_lambda_eq_mu():
    """theta = -1, lambda = mu: the global K is symmetric (K_PQ = K_QP^T)."""
    m = M.cube(2, bc="reference", agglomeration="bfs", group=(4, 12), jitter=0.2)
    o = O.Oracle(m, 2, 1e-3)
    o.make_matrices()
    d = o.block_dict(0)
    scale = max(np.abs(v).max() for v in d.values())
    for (P, Q), K in d.items():
        assert np.abs(K - d[(Q, P)].T).max() <= 1e-12 * scale


def test_reference_consistency_term_breaks_symmetry_when_lambda_ne_mu():
    """The reference's IT_E2 term (assemble_element.f90:610-616) pairs lambda
    and mu with transposed indices; with lambda != mu the assembled operator
    is not symmetric even for SIPG.  The oracle (and the GPU path) reproduce
    this on purpose."""
    m = M.cube(2, bc="dirichlet", agglomeration="tet", material=(1.0, 2.0, 1.0))
    o = O.Oracle(m, 1, 1e-3)
    o.make_matrices()
    d = o.block_dict(0)
    scale = max(np.abs(v).max() for v in d.values())
    asym = max(np.abs(K - d[(Q, P)].T).max() for (P, Q), K in d.items() if P != Q)
    assert asym > 1e-6 * scale


@pytest.mark.parametrize("p", [1, 2, 3])
def test_projection_converges_at_rate_p_plus_1(p):
    """||Pi_h u - u||_L2 ~ h^(p+1): checked through the L2 error of the
    projection of uex against a finer-mesh reference is awkward; instead the
    projected field's own L2 error is estimated from the difference of two
    projections (exact solution vs zero) via the DG mass norm identity
    ||Pi u||^2 = (Pi u, u) -> ||u||^2 from below at the expected rate."""
    exact_norm2 = 3 * 0.125  # int_[0,1]^3 (cos^2 sin^2 sin^2) = 1/8, three components
    errs = []
    for n in (2, 4):
        m = M.cube(n, agglomeration="tet")
        o = O.Oracle(m, p, 1e-3)
        o.make_matrices()
        o.modal_project(2, 3)
        # ||Pi u||^2 = u^T M u  (error_l2 of slot 3 against the zero slot 0)
        pn2 = o.error_l2(3, 0)
        errs.append(exact_norm2 - pn2)  # = ||u - Pi u||^2 by Pythagoras
    rate = 0.5 * math.log2(errs[0] / errs[1])
    assert errs[1] > 0 and rate > p + 1 - 0.45


def test_face_matching_agrees_with_independent_restatement():
    m = M.cube(3, agglomeration="tet", jitter=0.2)
    lib = O.load()
    tv = np.ascontiguousarray(m.tet_vert)
    nb = np.empty_like(tv)
    nf = np.empty_like(tv)
    lib.oracle_match_faces(tv.shape[0], O._p(tv, O.c_int32), O._p(nb, O.c_int32), O._p(nf, O.c_int32))
    neigh, nface = M.match_faces(tv)
    interior = nb >= 0
    assert np.array_equal(nb[interior], neigh[interior])
    assert np.array_equal(nf[interior], nface[interior])
    assert np.all(neigh[~interior] == -9)


def test_golden_driver_values():
    """Oracle driver runs pinned to the committed golden values."""
    gold = json.loads((GOLDEN / "oracle_driver.json").read_text())
    for case in gold["cases"]:
        m = M.cube(case["n"], bc=case["bc"], agglomeration=case["agglomeration"], seed=case["seed"],
                   group=tuple(case["group"]), jitter=case["jitter"], material=tuple(case["material"]))
        o = O.Oracle(m, case["p"], case["dt"])
        r = O.run_reference_driver(o, case["stop_time"])
        assert r["n_steps"] == case["n_steps"]
        assert abs(r["err_L2"] - case["err_L2"]) <= 1e-12 * case["err_L2"]
        assert abs(r["err_DG"] - case["err_DG"]) <= 1e-12 * case["err_DG"]
        u = o.get_state(1)
        assert abs(float(np.sum(u)) - case["sum_un"]) <= 1e-12 * max(1.0, abs(case["sum_un"]))
        assert abs(float(np.sum(u * u)) - case["sumsq_un"]) <= 1e-12 * case["sumsq_un"]


DECKS = GOLDEN / "decks"


def _deck(name):
    a = dict(np.load(DECKS / f"{name}.npz"))
    a["name"] = name
    return M.deck_mesh(a)


@pytest.mark.parametrize("deck", ["tet_5", "tet_25", "tet_100", "tet_125"])
def test_reference_deck_reads_and_runs(deck):
    """The reference's decks (committed fixtures of src/tests/analytical/*):
    every boundary triangle found on a tetrahedron face, every face matched,
    the decks' tags giving Dirichlet and Neumann faces, and the oracle's
    driver run reproducing its committed values."""
    mesh, prm = _deck(deck)
    assert mesh.info["unfound_tria"] == 0
    assert np.all(mesh.neigh != M._lib.MESH_UNMATCHED)
    # the decks mark z=0, z=1, x=1 Dirichlet and y=1, x=0, y=0 Neumann
    assert (mesh.neigh == -1).sum() > 0 and (mesh.neigh == -2).sum() > 0
    gold = next(x for x in json.loads((DECKS / "deck_driver.json").read_text())["decks"] if x["deck"] == deck)
    assert mesh.n_tet == gold["n_tet"] and prm["degree"] == gold["p"]
    o = O.Oracle(mesh, prm["degree"], prm["dt"])
    stop = prm["stop_time"] if deck != "tet_100" else 0.2
    r = O.run_reference_driver(o, stop)
    o.close()
    assert math.isfinite(r["err_L2"]) and math.isfinite(r["err_DG"])
    if deck != "tet_100":  # the full 3,183-step tet_100 run is left to the GPU test
        assert r["n_steps"] == gold["n_steps"] and r["t"] == gold["t_final"]
        assert abs(r["err_L2"] - gold["err_L2"]) <= 1e-12 * gold["err_L2"]
        assert abs(r["err_DG"] - gold["err_DG"]) <= 1e-12 * gold["err_DG"]


def test_agglomeration_fixtures():
    """elem_in_poly of the benchmark meshes equals the committed arrays: the
    125 hexahedra of the 5^3 cube and the seeded BFS grouping of the 40^3
    cube into 46,767 polyhedra of 4..15 tetrahedra."""
    fx = np.load(GOLDEN / "elem_in_poly.npz")
    c0 = M.cube(5, bc="dirichlet", agglomeration="hex")
    assert np.array_equal(c0.tet_poly, fx["c0"]) and c0.n_poly == 125
    c1 = M.cube(40, bc="dirichlet", agglomeration="bfs", seed=0, group=(4, 12))
    assert np.array_equal(c1.tet_poly, fx["c1"]) and c1.n_poly == 46767
    sizes = np.bincount(c1.tet_poly)
    assert sizes.min() >= 4 and sizes.max() <= 16


def test_c0_golden_driver():
    """The 125-polyhedron p = 2 run to T = 0.1 (1,000 steps) reproduces the
    committed oracle values."""
    gold = json.loads((GOLDEN / "c0_driver.json").read_text())
    o = O.Oracle(M.cube(5, bc="dirichlet", agglomeration="hex"), 2, 1e-4)
    r = O.run_reference_driver(o, 0.1)
    o.close()
    assert r["n_steps"] == gold["n_steps"] == 1000 and r["t"] == gold["t_final"]
    assert abs(r["err_L2"] - gold["err_L2"]) <= 1e-12 * gold["err_L2"]
    assert abs(r["err_DG"] - gold["err_DG"]) <= 1e-12 * gold["err_DG"]


@pytest.mark.parametrize("n,bc,agg,seed,group", [(3, "dirichlet", "bfs", 0, (4, 12)), (4, "reference", "bfs", 3, (4, 16)),
                                                 (5, "reference", "hex", 0, (6, 6)), (2, "dirichlet", "tet", 0, (1, 1))])
def test_oracle_mesh_builder_equals_the_library(n, bc, agg, seed, group):
    """oracle/mesh_py.py (the meshes of the CPU reference arm, built without
    the GPU library) gives the library's arrays bit for bit."""
    from oracle import mesh_py as MP
    a = M.cube(n, bc=bc, agglomeration=agg, seed=seed, group=group)
    b = MP.cube(n, bc=bc, agglomeration=agg, seed=seed, group=group)
    for k in ("coords", "tet_vert", "tet_poly", "tet_mat", "neigh", "fun_tag", "mat"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    m0 = M.cube(n, bc=bc, agglomeration=agg, seed=seed, group=group)
    c = M.cube(n, bc=bc, agglomeration=agg, seed=seed, group=group,
               poly_materials=M.lognormal_materials(m0.n_poly, seed=1))
    d = MP.cube(n, bc=bc, agglomeration=agg, seed=seed, group=group, lognormal_seed=1)
    assert np.array_equal(c.mat, d.mat) and np.array_equal(c.tet_mat, d.tet_mat)


def test_oracle_mesh_builder_reproduces_the_benchmark_grouping():
    from oracle import mesh_py as MP
    b = MP.cube(40, bc="dirichlet", agglomeration="bfs", seed=0, group=(4, 12))
    assert np.array_equal(b.tet_poly, np.load(GOLDEN / "elem_in_poly.npz")["c1"])
