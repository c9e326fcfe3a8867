"""The matrix-free neighbour contraction against the assembled block (CPU).

The mixed path with matrix-free neighbour terms (csrc/mf.cu) never forms the
neighbour block K_PQ: it evaluates u_Q and its gradient at P's face
quadrature points, forms the flux (G, s) and tests it against P's basis.  The
oracle evaluates that same point-wise contraction in FP64
(oracle_neighbour_apply_pointwise), and this test checks it against K_PQ u_Q
from the oracle's assembled blocks: the two are the same sums in another
order, so they agree to FP64 rounding (1e-12 normwise relative per block),
with heterogeneous materials (lambda != mu per polyhedron), jittered
tetrahedra and every interior-penalty variant theta = -1, 0, 1.

The GPU path integrates each shared triangle with its own symmetric rule,
exact to degree 2p with fewer nodes (lymph_mf_face_rule).  The second test
evaluates the point-wise contraction in FP64 with that rule and checks it
against the assembled block too: the face integrands have degree <= 2p, so
both rules give the same integrals up to FP64 rounding (1e-12).
"""
import numpy as np
import pytest

from lymph3d_apsc_gb300 import mesh as M
from oracle.oracle_py import Oracle


def _mesh():
    m0 = M.cube(3, bc="dirichlet", agglomeration="bfs", seed=1, group=(4, 12), jitter=0.15)
    return M.cube(3, bc="dirichlet", agglomeration="bfs", seed=1, group=(4, 12), jitter=0.15,
                  poly_materials=M.lognormal_materials(m0.n_poly, seed=3))


@pytest.mark.parametrize("theta", [-1.0, 0.0, 1.0])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_pointwise_neighbour_product_equals_the_block(p, theta):
    m = _mesh()
    o = Oracle(m, p, 1e-3, theta=theta)
    o.make_matrices()
    blocks = o.block_dict(0)
    rng = np.random.default_rng(p)
    worst, pairs = 0.0, 0
    for (P, Q), K in blocks.items():
        if P == Q:
            continue
        u = rng.standard_normal(o.nd)
        want = K @ u
        got = o.neighbour_apply_pointwise(P, Q, u)
        worst = max(worst, float(np.linalg.norm(got - want) / np.linalg.norm(want)))
        pairs += 1
    o.close()
    assert pairs >= 50
    print(f"p={p} theta={theta}: {pairs} neighbour blocks, worst relative difference {worst:.2e}")
    assert worst <= 1e-12, worst


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_exact_degree_face_rule_gives_the_same_block(p):
    from ctypes import POINTER, byref, c_double, c_int32
    from lymph3d_apsc_gb300 import _lib
    lib = _lib.load()
    n = c_int32()
    assert lib.lymph_mf_face_rule(p, byref(n), None) == 0
    xyw = np.zeros(3 * n.value)
    assert lib.lymph_mf_face_rule(p, byref(n), xyw.ctypes.data_as(POINTER(c_double))) == 0
    assert n.value < (p + 1) ** 2
    m = _mesh()
    o = Oracle(m, p, 1e-3, theta=-1.0)
    o.make_matrices()
    blocks = o.block_dict(0)
    rng = np.random.default_rng(10 + p)
    worst, pairs = 0.0, 0
    for (P, Q), K in blocks.items():
        if P == Q:
            continue
        u = rng.standard_normal(o.nd)
        want = K @ u
        got = o.neighbour_apply_rule(P, Q, u, xyw)
        worst = max(worst, float(np.linalg.norm(got - want) / np.linalg.norm(want)))
        pairs += 1
        if pairs >= 150:
            break
    o.close()
    print(f"p={p}: {n.value}-node rule, {pairs} neighbour blocks, worst relative difference {worst:.2e}")
    assert worst <= 1e-12, worst


@pytest.mark.parametrize("p", [2, 4])
def test_planted_face_mistakes_exceed_the_operator_bar(p):
    """The GPU bar on the operator apply (TOL_APPLY_FP32, per polyhedron row,
    tests/test_gpu_mf.py) is far below what any single face-term mistake
    does: with one mistake planted in the oracle's point-wise neighbour
    product (the penalty term dropped, the symmetry term's sign flipped, the
    consistency term dropped, one shared triangle left out), the rows of
    K u move by more than 100 x the bar (2e-2 and more against 2e-6)."""
    from ctypes import POINTER, byref, c_double, c_int32
    from lymph3d_apsc_gb300 import _lib
    from oracle.oracle_py import load as oracle_load
    from parity_util import TOL_APPLY_FP32, oracle_apply, row_rel_max
    lib = _lib.load()
    n = c_int32()
    lib.lymph_mf_face_rule(p, byref(n), None)
    xyw = np.zeros(3 * n.value)
    lib.lymph_mf_face_rule(p, byref(n), xyw.ctypes.data_as(POINTER(c_double)))
    m = _mesh()
    o = Oracle(m, p, 1e-3)
    o.make_matrices()
    rp, col = o.pattern()
    vals = o.blocks(0)
    u = np.random.default_rng(5).standard_normal((o.n_poly, o.nd))
    want = oracle_apply(o, u, vals)
    olib = oracle_load()

    def rows(plant):
        olib.oracle_set_planted_mistake(plant)
        try:
            out = np.zeros_like(u)
            for P in range(o.n_poly):
                for k in range(rp[P], rp[P + 1]):
                    Q = int(col[k])
                    out[P] += vals[k] @ u[Q] if Q == P else o.neighbour_apply_rule(P, Q, u[Q], xyw)
            return out
        finally:
            olib.oracle_set_planted_mistake(0)

    clean = row_rel_max(rows(0), want)
    assert clean <= 1e-12, clean
    for plant in (1, 2, 3, 4):
        e = row_rel_max(rows(plant), want)
        print(f"p={p} planted mistake {plant}: rows move by {e:.2e} (bar {TOL_APPLY_FP32:.0e})")
        assert e >= 100 * TOL_APPLY_FP32, (plant, e)
    o.close()
