"""The matrix-free neighbour path (LYMPH_MIXED_MF) against the FP64 oracle and
the FP32-block path (LYMPH_MIXED).

LYMPH_MIXED_MF keeps the FP32 self blocks and evaluates every neighbour block's
product at each step from the face quadrature in FP32 (Q's field and gradient
at P's quadrature points, tested against P's basis): the same sums as the
assembled block in another order, rounded in FP32 at more places (basis
values, geometry, the quadrature sums).  Bars (written in each assertion):
  * the operator apply alone, K u before M^-1 (lymph_apply_operator), with
    random coefficients, every polyhedron row against the oracle's FP64 K u
    from the assembled blocks: max_P ||(K u)_P - ref_P|| / ||ref_P|| <=
    TOL_APPLY_FP32 (2e-6) for both FP32 forms, <= 1e-13 for FP64 blocks; one
    dropped or mis-signed face term moves rows by > 100 x that bar
    (tests/test_mf_formula.py plants each mistake in the oracle);
  * the state after 20 leapfrog steps from the oracle's state, in the mass
    norm (the L2 norm of the field): relative <= TOL_STEPS_FP32 (2e-5) for
    both FP32 forms; the Euclidean differences of the coefficients (up to
    ~1e-1 after one step at p = 4 for both FP32 forms, through M^-1 whose
    condition number reaches ~1e7) are printed beside it;
  * L2 / DG errors against the manufactured solution after 0.1 s: <= 1.1 x
    the FP64 path's (the mixed-precision bar), on heterogeneous lognormal
    materials (an operator that is not symmetric);
  * graph-launched loop vs step-by-step calls, and two runs: bit-identical
    (fixed thread-to-point assignment, sums in a fixed order);
  * leapfrog energy: relative <= 1e-4 of the FP64 path's; the largest
    eigenvalue of M^-1 K after 40 power iterations, which have not converged,
    so FP32 rounding moves the estimate along its path: relative <= 2e-3;
  * lymph_get_blocks returns the FP64 operator this path evaluates.
"""
import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib
from lymph3d_apsc_gb300._lib import LymphError
from oracle.oracle_py import Oracle
from parity_util import TOL_APPLY_FP32, TOL_APPLY_FP64, TOL_STEPS_FP32, mass_norm_rel, oracle_apply, row_rel_max
from test_gpu_parity import KINDS, _mesh, rel

pytestmark = pytest.mark.gpu


def _prepared(m, p, precision, dt=1e-3):
    g = MatrixFree(m, p, dt, precision=precision)
    g.MAKE_MATRICES_FREE()
    g.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
    g.MAKE_RHS_FREE(_lib.RHS_DYN, _lib.F_TIME, _lib.GD, _lib.GN)
    g.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_DISPLACEMENT, _lib.SLOT_U0)
    g.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_VELOCITY, _lib.SLOT_V0)
    g.FIRST_TIME_STEP_MATRIX_FREE(0.0)
    return g


def _oracle(m, p, dt=1e-3):
    o = Oracle(m, p, dt)
    o.make_matrices()
    o.make_rhs(0, 0, 0, 0)
    o.make_rhs(1, 1, 1, 1)
    o.modal_project(0, 0)
    o.modal_project(1, 2)
    o.first_step(0.0)
    return o


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_operator_apply_against_fp64_oracle(require_gpu, kind, p):
    """K u of every precision, row by row, against the oracle's FP64 K u."""
    m = _mesh(kind)
    o = Oracle(m, p, 1e-3)
    o.make_matrices()
    u = np.random.default_rng(100 + p).standard_normal((o.n_poly, o.nd))
    want = oracle_apply(o, u)
    o.close()
    errs = {}
    for name, prec, bar in (("fp64", _lib.FP64, TOL_APPLY_FP64), ("fp32_blocks", _lib.MIXED, TOL_APPLY_FP32),
                            ("mixed_mf", _lib.MIXED_MF, TOL_APPLY_FP32)):
        with MatrixFree(m, p, 1e-3, precision=prec) as g:
            g.MAKE_MATRICES_FREE()
            errs[name] = row_rel_max(g.apply_operator(u), want)
        assert errs[name] <= bar, (name, errs[name])
    print(f"p={p} {kind}: K u row error fp64 {errs['fp64']:.2e} fp32-blocks {errs['fp32_blocks']:.2e} "
          f"mixed_mf {errs['mixed_mf']:.2e}")


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_mf_operator_and_steps_close_to_fp64(require_gpu, kind, p):
    m = _mesh(kind)
    o = _oracle(m, p)
    mf = _prepared(m, p, _lib.MIXED_MF)
    f32 = _prepared(m, p, _lib.MIXED)
    u0, un = o.get_state(_lib.SLOT_U0), o.get_state(_lib.SLOT_UN)
    for g in (mf, f32):
        g.set_state(_lib.SLOT_U0, u0)
        g.set_state(_lib.SLOT_UN, un)
    # one step: u^{n+1} - (2 u^n - u^{n-1}) = dt^2 M^-1 (F - K u^n)
    t = 1e-3
    base = 2.0 * un - u0
    o.step(t)
    for g in (mf, f32):
        g.TIME_STEP_MATRIX_FREE(t)
    d_o = o.get_state(_lib.SLOT_UN) - base
    e_mf = rel(mf.get_state(_lib.SLOT_UN) - base, d_o)
    e_32 = rel(f32.get_state(_lib.SLOT_UN) - base, d_o)
    # 20 more steps
    t += 1e-3
    o.run_steps(t, 1.0, max_steps=20)
    mf.run_steps(t, 1.0, max_steps=20)
    f32.run_steps(t, 1.0, max_steps=20)
    uo = o.get_state(_lib.SLOT_UN)
    s_mf = rel(mf.get_state(_lib.SLOT_UN), uo)
    s_32 = rel(f32.get_state(_lib.SLOT_UN), uo)
    m_mf = mass_norm_rel(o, mf.get_state(_lib.SLOT_UN), uo)
    m_32 = mass_norm_rel(o, f32.get_state(_lib.SLOT_UN), uo)
    print(f"p={p} {kind}: one apply mf {e_mf:.2e} fp32-blocks {e_32:.2e}; 20 steps mf {s_mf:.2e} fp32-blocks {s_32:.2e}"
          f"; mass norm mf {m_mf:.2e} fp32-blocks {m_32:.2e}")
    assert m_mf <= TOL_STEPS_FP32 and m_32 <= TOL_STEPS_FP32, (m_mf, m_32)
    for x in (mf, f32, o):
        x.close()


def _big_polyhedron_mesh():
    """5^3 hexahedra x 6 tets, one polyhedron per hexahedron, except the central
    3 x 3 x 3 block of hexahedra, which is one polyhedron of 162 tetrahedra with
    108 triangles shared with neighbours (more than the 64 whose neighbour index
    the kernel keeps in shared memory)."""
    from lymph3d_apsc_gb300 import mesh as M
    m = M.cube(5, bc="dirichlet", agglomeration="hex", material=(1.0, 2.0, 1.0), jitter=0.1)
    cell = np.clip(np.floor(m.coords[m.tet_vert].mean(axis=1) * 5).astype(int), 0, 4)
    inner = np.all((cell >= 1) & (cell <= 3), axis=1)
    tp = m.tet_poly.copy()
    tp[inner] = -1
    _, tp[~inner] = np.unique(tp[~inner], return_inverse=True)
    tp[inner] = tp[~inner].max() + 1
    return m.with_polyhedra(tp)


@pytest.mark.parametrize("p", [2, 4])
def test_mf_polyhedron_with_many_neighbour_triangles(require_gpu, p):
    m = _big_polyhedron_mesh()
    big = m.tet_poly.max()
    e2 = m.neigh.ravel()
    t = np.repeat(np.arange(m.n_tet), 4)
    ok = e2 >= 0
    shared = (m.tet_poly[t[ok]] == big) & (m.tet_poly[e2[ok]] != big)
    assert int(shared.sum()) == 108
    o = _oracle(m, p)
    mf = _prepared(m, p, _lib.MIXED_MF)
    f32 = _prepared(m, p, _lib.MIXED)
    for g in (mf, f32):
        g.set_state(_lib.SLOT_U0, o.get_state(_lib.SLOT_U0))
        g.set_state(_lib.SLOT_UN, o.get_state(_lib.SLOT_UN))
    t0 = 1e-3
    o.run_steps(t0, 1.0, max_steps=20)
    mf.run_steps(t0, 1.0, max_steps=20)
    f32.run_steps(t0, 1.0, max_steps=20)
    uo = o.get_state(_lib.SLOT_UN)
    s_mf = rel(mf.get_state(_lib.SLOT_UN), uo)
    s_32 = rel(f32.get_state(_lib.SLOT_UN), uo)
    m_mf = mass_norm_rel(o, mf.get_state(_lib.SLOT_UN), uo)
    m_32 = mass_norm_rel(o, f32.get_state(_lib.SLOT_UN), uo)
    print(f"p={p} big polyhedron: 20 steps mf {s_mf:.2e} fp32-blocks {s_32:.2e}; mass norm mf {m_mf:.2e} "
          f"fp32-blocks {m_32:.2e}")
    assert m_mf <= TOL_STEPS_FP32 and m_32 <= TOL_STEPS_FP32, (m_mf, m_32)
    for x in (mf, f32, o):
        x.close()


@pytest.mark.parametrize("theta", [0.0, 1.0])
@pytest.mark.parametrize("p", [2, 3])
def test_mf_other_interior_penalty_forms(require_gpu, theta, p):
    """theta = 0 (incomplete) and 1 (non-symmetric interior penalty): the
    matrix-free terms carry theta in the consistency term like the assembly."""
    m = _mesh("bfs_ref_jitter")
    o = Oracle(m, p, 1e-3, theta=theta)
    o.make_matrices()
    o.make_rhs(0, 0, 0, 0)
    o.make_rhs(1, 1, 1, 1)
    o.modal_project(0, 0)
    o.modal_project(1, 2)
    o.first_step(0.0)
    runs = []
    for prec in (_lib.MIXED_MF, _lib.MIXED):
        g = MatrixFree(m, p, 1e-3, theta=theta, precision=prec)
        g.MAKE_MATRICES_FREE()
        g.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
        g.MAKE_RHS_FREE(_lib.RHS_DYN, _lib.F_TIME, _lib.GD, _lib.GN)
        g.set_state(_lib.SLOT_U0, o.get_state(_lib.SLOT_U0))
        g.set_state(_lib.SLOT_UN, o.get_state(_lib.SLOT_UN))
        g.run_steps(1e-3, 1.0, max_steps=20)
        runs.append(g)
    o.run_steps(1e-3, 1.0, max_steps=20)
    uo = o.get_state(_lib.SLOT_UN)
    s_mf, s_32 = (rel(g.get_state(_lib.SLOT_UN), uo) for g in runs)
    m_mf, m_32 = (mass_norm_rel(o, g.get_state(_lib.SLOT_UN), uo) for g in runs)
    print(f"p={p} theta={theta}: 20 steps mf {s_mf:.2e} fp32-blocks {s_32:.2e}; mass norm mf {m_mf:.2e} "
          f"fp32-blocks {m_32:.2e}")
    assert m_mf <= TOL_STEPS_FP32 and m_32 <= TOL_STEPS_FP32, (m_mf, m_32)
    for x in runs + [o]:
        x.close()


@pytest.mark.parametrize("p", [2, 3, 4])
def test_mf_error_within_1p1_of_fp64(require_gpu, p):
    from lymph3d_apsc_gb300.matrix_free import run_reference_driver as gpu_driver
    m = _mesh("bfs_lognormal")
    with MatrixFree(m, p, 2e-3) as a:
        ra = gpu_driver(a, 0.1)
    with MatrixFree(m, p, 2e-3, precision=_lib.MIXED_MF) as b:
        rb = gpu_driver(b, 0.1)
    print(f"p={p}: L2 {rb['err_L2']:.4e} vs FP64 {ra['err_L2']:.4e}; DG {rb['err_DG']:.4e} vs {ra['err_DG']:.4e}")
    assert rb["n_steps"] == ra["n_steps"]
    assert rb["err_L2"] <= 1.1 * ra["err_L2"]
    assert rb["err_DG"] <= 1.1 * ra["err_DG"]


@pytest.mark.parametrize("p", [1, 3, 4])
def test_mf_graph_loop_bitwise_and_deterministic(require_gpu, p):
    m = _mesh("bfs_lognormal")
    a = _prepared(m, p, _lib.MIXED_MF)
    b = _prepared(m, p, _lib.MIXED_MF)
    c = _prepared(m, p, _lib.MIXED_MF)
    t = a.dt
    ta, n, _, _ = a.run_steps(t, 1.0, max_steps=37)
    assert n == 37
    for _ in range(37):
        b.TIME_STEP_MATRIX_FREE(t)
        t += b.dt
    assert ta == t
    for slot in (_lib.SLOT_UN, _lib.SLOT_U0):
        assert np.array_equal(a.get_state(slot), b.get_state(slot))
    tc, nc, _, mk = c.run_steps(c.dt, 1.0, max_steps=37, kernel_timing=True)
    assert nc == 37 and mk is not None and mk > 0
    assert np.array_equal(c.get_state(_lib.SLOT_UN), a.get_state(_lib.SLOT_UN))
    for x in (a, b, c):
        x.close()


@pytest.mark.parametrize("p", [2, 4])
def test_mf_energy_and_eigenvalue(require_gpu, p):
    from lymph3d_apsc_gb300.ensemble import max_eigenvalue
    from lymph3d_apsc_gb300.surrogate import energy
    m = _mesh("bfs_lognormal")
    a = _prepared(m, p, _lib.FP64)
    b = _prepared(m, p, _lib.MIXED_MF)
    a.run_steps(a.dt, 1.0, max_steps=10)
    b.set_state(_lib.SLOT_U0, a.get_state(_lib.SLOT_U0))
    b.set_state(_lib.SLOT_UN, a.get_state(_lib.SLOT_UN))
    ea, eb = energy(a), energy(b)
    la, lb = max_eigenvalue(a, 40), max_eigenvalue(b, 40)
    print(f"p={p}: energy {eb:.8e} vs {ea:.8e}; lambda_max {lb:.8e} vs {la:.8e}")
    assert abs(eb - ea) <= 1e-4 * abs(ea)
    assert abs(lb - la) <= 2e-3 * la
    a.close()
    b.close()


@pytest.mark.parametrize("p", [1, 3])
def test_mf_blocks_are_the_fp64_operator(require_gpu, p):
    m = _mesh("bfs_lognormal")
    with MatrixFree(m, p, 1e-3, precision=_lib.MIXED_MF) as a, MatrixFree(m, p, 1e-3) as b:
        a.MAKE_MATRICES_FREE()
        b.MAKE_MATRICES_FREE()
        assert np.array_equal(a.blocks(_lib.BLOCKS_K), b.blocks(_lib.BLOCKS_K))
        for which in range(5):
            assert np.array_equal(a.mass(which), b.mass(which))
