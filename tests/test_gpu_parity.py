"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Bars (written in each assertion):
  * set-up data (geometry, mass, Cholesky factors, operator blocks, RHS):
    normwise relative difference <= 1e-12;
  * modal coefficients after every step, both sides started from the same
    coefficients: ||u_gpu - u_ref|| / ||u_ref|| <= max(1e-12, 4 x floor),
    floor = the largest spread so far of three oracle runs that evaluate the
    same steps in other valid orders (reversed sums with fused multiply-adds
    and M^-1 as an explicit inverse; forward sums with the explicit inverse;
    the CUDA kernel's slice/accumulator order) from the reference-order run
    -- the ill-conditioned mass matrix (cond up to ~1e7 at p = 4) lifts that
    spread to 1e-12..1e-11 at p = 4; and
    <= 1e-12 in the mass-matrix norm (the L2 norm of the field);
  * L2 projections (COMPUTE_MODAL_COEFFICIENTS_FREE) solve with the mass
    matrix, whose condition number (bounding-box Legendre basis on a
    tetrahedron or an agglomerated polyhedron, up to ~1e7 at p = 4) amplifies
    the differences between the device's and the host's sin/cos (<= 2 ulp and
    < 1 ulp per call, three factors per value).  Their bar is
    max(1e-12, 2 x the oracle's own spread when its data values move by
    8 ulp) on the coefficients, and 1e-12 in the mass-matrix norm;
  * L2 / DG errors against the manufactured solution: relative <= 1e-10;
  * graph-launched loop vs step-by-step calls, and two runs: bit-identical.
Meshes are generated (structured cubes, optionally jittered, agglomerated
one-tet-per-polyhedron, per hexahedron, or by seeded BFS groups) at sizes the
oracle finishes in seconds; the smallest is one polyhedron with no neighbour
at all (every face on the boundary, Dirichlet and Neumann).
"""
import math

import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib, mesh as M
from lymph3d_apsc_gb300._lib import LymphError
from oracle.oracle_py import Oracle
from parity_util import every_step_parity, mass_norm_rel, rel

pytestmark = pytest.mark.gpu

TOL_SETUP = 1e-12
TOL_STATE = 1e-12
TOL_ERR = 1e-10


def _mesh(kind):
    if kind == "one_poly":  # the whole cube one polyhedron of 6 tets: no neighbour blocks
        return M.cube(1, bc="reference", agglomeration="hex", material=(1.0, 2.0, 1.0))
    if kind == "tet_dir":
        return M.cube(2, bc="dirichlet", agglomeration="tet")
    if kind == "tet_ref_jitter":
        return M.cube(2, bc="reference", agglomeration="tet", jitter=0.25)
    if kind == "hex_dir":
        return M.cube(3, bc="dirichlet", agglomeration="hex", material=(1.0, 2.0, 1.0))
    if kind == "bfs_ref_jitter":
        return M.cube(3, bc="reference", agglomeration="bfs", seed=0, group=(4, 12), jitter=0.2)
    if kind == "bfs_lognormal":
        m = M.cube(3, bc="dirichlet", agglomeration="bfs", seed=1, group=(4, 16), jitter=0.15)
        return M.cube(3, bc="dirichlet", agglomeration="bfs", seed=1, group=(4, 16), jitter=0.15,
                      poly_materials=M.lognormal_materials(m.n_poly, seed=1))
    raise KeyError(kind)


KINDS = ["one_poly", "tet_dir", "tet_ref_jitter", "hex_dir", "bfs_ref_jitter", "bfs_lognormal"]


@pytest.fixture(scope="module")
def pairs():
    cache = {}

    def get(kind, p, dt=1e-3, precision=_lib.FP64):
        key = (kind, p, dt, precision)
        if key not in cache:
            m = _mesh(kind)
            g = MatrixFree(m, p, dt, precision=precision)
            o = Oracle(m, p, dt)
            g.MAKE_MATRICES_FREE()
            o.make_matrices()
            cache[key] = (m, g, o)
        return cache[key]

    yield get
    for m, g, o in cache.values():
        g.close()
        o.close()


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_setup_parity(require_gpu, pairs, kind, p):
    m, g, o = pairs(kind, p)
    bb_g, hk_g = g.poly_geometry()
    bb_o, hk_o = o.poly_geometry()
    assert np.array_equal(bb_g, bb_o)
    assert rel(hk_g, hk_o) <= 1e-15
    for which in range(4):  # M_loc, M_modal_loc, R_M_loc, R_M_modal_loc
        assert rel(g.mass(which), o.mass(which)) <= TOL_SETUP, which
    rp, col = g.pattern()
    ref = o.block_dict(_lib.BLOCKS_K)
    assert len(ref) == len(col)
    for name, which in (("K", _lib.BLOCKS_K), ("A_dg", _lib.BLOCKS_ADG)):
        vals = g.blocks(which)
        ref = o.block_dict(which)
        num = den = 0.0
        for P in range(g.n_poly):
            assert col[rp[P]] == P  # self block first
            for k in range(rp[P], rp[P + 1]):
                r = ref[(P, int(col[k]))]
                num += float(np.sum((vals[k] - r) ** 2))
                den += float(np.sum(r ** 2))
        assert math.sqrt(num / den) <= TOL_SETUP, name


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("p", [1, 3, 4])
def test_rhs_and_projection_parity(require_gpu, pairs, kind, p):
    from oracle.oracle_py import load as oracle_load
    m, g, o = pairs(kind, p)
    for which, ids in ((_lib.RHS_DYN, (_lib.F_TIME, _lib.GD, _lib.GN)),
                       (_lib.RHS_STAT, (_lib.F_STAT, _lib.GD_STAT, _lib.GN_STAT))):
        g.MAKE_RHS_FREE(which, *ids)
        o.make_rhs(which, *ids)
        assert rel(g.rhs(which), o.rhs(which)) <= TOL_SETUP
    lib = oracle_load()
    for fun, slot in ((_lib.FUN_IC_VELOCITY, _lib.SLOT_V0), (_lib.FUN_UEX, _lib.SLOT_UEX)):
        g.COMPUTE_MODAL_COEFFICIENTS_FREE(fun, slot, 0.75)
        o.modal_project(fun, slot, 0.75)
        ref = o.get_state(slot)
        lib.oracle_set_data_perturbation(8)
        o.modal_project(fun, slot, 0.75)
        floor = rel(o.get_state(slot), ref)
        lib.oracle_set_data_perturbation(0)
        o.modal_project(fun, slot, 0.75)
        got = g.get_state(slot)
        assert rel(got, ref) <= max(TOL_SETUP, 2.0 * floor), (rel(got, ref), floor)
        assert mass_norm_rel(o, got, ref) <= TOL_SETUP


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("p", [1, 4])
def test_mass_inverse(require_gpu, pairs, kind, p):
    m, g, o = pairs(kind, p)
    Minv = g.mass(4)
    M_ = o.mass(0)
    eye = np.eye(g.Np)
    cond = max(np.linalg.cond(x) for x in M_)
    assert np.abs(np.einsum("pij,pjk->pik", M_, Minv) - eye).max() <= 64 * cond * 2.2e-16


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_step_parity_every_step(require_gpu, pairs, kind, p):
    """u^n after every one of 25 steps (first step included).  Three more
    oracle runs evaluate the same steps in other valid orders: (a) reversed
    sums with FMA and M^-1 as an explicit inverse, (b) forward sums with the
    explicit inverse, (c) the CUDA kernel's own order (column slices, two FMA
    accumulators each, explicit inverse).  The floor is their largest spread
    so far from the reference-order run (rounding noise accumulates over the
    steps, and one sample of it can fall low).  (c) runs on the oracle's own
    blocks and inverse, which differ from the device's set-up by rounding, so
    it is a floor variant, not a bitwise emulation of the device."""
    m, g, o = pairs(kind, p)
    e, floor, worst = every_step_parity(m, p, g, o, n_steps=25)
    assert worst <= 1.0
    print(f"p={p} {kind}: device vs reference order {e:.2e}, floor {floor:.2e}, bar ratio {worst:.2f}")


@pytest.mark.parametrize("kind", ["tet_ref_jitter", "bfs_ref_jitter", "bfs_lognormal"])
@pytest.mark.parametrize("p", [2, 3])
def test_driver_errors_match_oracle(require_gpu, kind, p):
    """The full Lymph3D.f90 sequence: L2 and DG errors equal the oracle's."""
    from lymph3d_apsc_gb300.matrix_free import run_reference_driver as gpu_driver
    from oracle.oracle_py import run_reference_driver as cpu_driver
    m = _mesh(kind)
    with MatrixFree(m, p, 2e-3) as g:
        rg = gpu_driver(g, 0.1)
    o = Oracle(m, p, 2e-3)
    ro = cpu_driver(o, 0.1)
    o.close()
    assert rg["n_steps"] == ro["n_steps"] and rg["t"] == ro["t"]
    assert abs(rg["err_L2"] - ro["err_L2"]) <= TOL_ERR * ro["err_L2"]
    assert abs(rg["err_DG"] - ro["err_DG"]) <= TOL_ERR * ro["err_DG"]


def _prepared(kind, p, precision=_lib.FP64, dt=1e-3):
    g = MatrixFree(_mesh(kind), p, dt, precision=precision)
    g.MAKE_MATRICES_FREE()
    g.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
    g.MAKE_RHS_FREE(_lib.RHS_DYN, _lib.F_TIME, _lib.GD, _lib.GN)
    g.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_DISPLACEMENT, _lib.SLOT_U0)
    g.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_VELOCITY, _lib.SLOT_V0)
    g.FIRST_TIME_STEP_MATRIX_FREE(0.0)
    return g


@pytest.mark.parametrize("p", [1, 3, 4])
def test_graph_loop_bitwise_equals_single_steps(require_gpu, p):
    a = _prepared("bfs_ref_jitter", p)
    b = _prepared("bfs_ref_jitter", p)
    t = a.dt
    ta, n, _, _ = a.run_steps(t, 1.0, max_steps=37)
    assert n == 37
    for _ in range(37):
        b.TIME_STEP_MATRIX_FREE(t)
        t += b.dt
    assert ta == t
    assert np.array_equal(a.get_state(_lib.SLOT_UN), b.get_state(_lib.SLOT_UN))
    assert np.array_equal(a.get_state(_lib.SLOT_U0), b.get_state(_lib.SLOT_U0))
    # per-launch-event path gives the same bits as the graph path
    c = _prepared("bfs_ref_jitter", p)
    tc, nc, _, mk = c.run_steps(c.dt, 1.0, max_steps=37, kernel_timing=True)
    assert nc == 37 and mk is not None and mk > 0
    assert np.array_equal(c.get_state(_lib.SLOT_UN), a.get_state(_lib.SLOT_UN))
    for x in (a, b, c):
        x.close()


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED_MF])
@pytest.mark.parametrize("layout", [_lib.LAYOUT_POLY_MAJOR, _lib.LAYOUT_FORTRAN])
def test_time_step_host_equals_the_separate_calls(require_gpu, precision, layout):
    """lymph_time_step_host (TIME_STEP_MATRIX_FREE with host u0, un in and
    usol out) gives the bits of set_state, set_state, lymph_step, get_state,
    and leaves the context in the same state."""
    a = _prepared("bfs_ref_jitter", 3, precision=precision)
    b = _prepared("bfs_ref_jitter", 3, precision=precision)
    rng = np.random.default_rng(11)
    shape = (a.n_poly, a.nd) if layout == _lib.LAYOUT_POLY_MAJOR else (a.nd, a.n_poly)
    u0 = rng.standard_normal(shape) * 1e-3
    un = rng.standard_normal(shape) * 1e-3
    t = 5 * a.dt
    for _ in range(3):
        usol = np.empty(a.n_poly * a.nd)
        a.time_step_host(t, u0, un, usol, layout)
        b.set_state(_lib.SLOT_U0, u0, layout)
        b.set_state(_lib.SLOT_UN, un, layout)
        b.TIME_STEP_MATRIX_FREE(t)
        ref = b.get_state(_lib.SLOT_UN, layout)
        assert np.array_equal(usol.reshape(shape), ref)
        assert np.array_equal(a.get_state(_lib.SLOT_U0), b.get_state(_lib.SLOT_U0))
        u0, un = un, usol.reshape(shape)
        t += a.dt
    a.close()
    b.close()


@pytest.mark.parametrize("precision", [_lib.FP64, _lib.MIXED_MF])
def test_checkpoint_resume_is_bitwise(require_gpu, tmp_path, precision):
    """A run stopped after 17 steps, checkpointed, and resumed in a new
    context gives the bits of the uninterrupted 40-step run; checkpoints of
    another degree or mesh are refused."""
    a = _prepared("bfs_ref_jitter", 3, precision=precision)
    t, n, _, _ = a.run_steps(a.dt, 1.0, max_steps=40)
    ref0, ref1 = a.get_state(_lib.SLOT_U0), a.get_state(_lib.SLOT_UN)
    b = _prepared("bfs_ref_jitter", 3, precision=precision)
    tb, nb, _, _ = b.run_steps(b.dt, 1.0, max_steps=17)
    path = tmp_path / "run.ckpt"
    b.save_checkpoint(path, tb, 1 + nb)
    c = _prepared("bfs_ref_jitter", 3, precision=precision)
    tc, steps = c.load_checkpoint(path)
    assert tc == tb and steps == 18
    assert np.array_equal(c.get_state(_lib.SLOT_UN), b.get_state(_lib.SLOT_UN))
    tc, nc, _, _ = c.run_steps(tc, 1.0, max_steps=40 - 17)
    assert tc == t
    assert np.array_equal(c.get_state(_lib.SLOT_U0), ref0)
    assert np.array_equal(c.get_state(_lib.SLOT_UN), ref1)
    other_p = _prepared("bfs_ref_jitter", 2, precision=precision)
    other_mesh = _prepared("hex_dir", 3, precision=precision)
    for g in (other_p, other_mesh):
        with pytest.raises(LymphError) as e:
            g.load_checkpoint(path)
        assert e.value.code == _lib.LYMPH_ERR_INVALID
    for g in (a, b, c, other_p, other_mesh):
        g.close()


def test_layout_roundtrip_and_fortran_order(require_gpu):
    g = _prepared("hex_dir", 2)
    u = g.get_state(_lib.SLOT_UN)
    uf = g.get_state(_lib.SLOT_UN, _lib.LAYOUT_FORTRAN)
    assert np.array_equal(uf, u.T)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(u.shape)
    g.set_state(_lib.SLOT_UEX, np.ascontiguousarray(x.T), _lib.LAYOUT_FORTRAN)
    assert np.array_equal(g.get_state(_lib.SLOT_UEX), x)
    g.close()


@pytest.mark.parametrize("p", [2, 4])
def test_mixed_precision_error_within_1p1_of_fp64(require_gpu, p):
    from lymph3d_apsc_gb300.matrix_free import run_reference_driver as gpu_driver
    m = _mesh("bfs_lognormal")
    with MatrixFree(m, p, 2e-3) as a:
        ra = gpu_driver(a, 0.1)
    with MatrixFree(m, p, 2e-3, precision=_lib.MIXED) as b:
        rb = gpu_driver(b, 0.1)
    assert rb["err_L2"] <= 1.1 * ra["err_L2"]
    assert rb["err_DG"] <= 1.1 * ra["err_DG"]


def test_instability_is_reported_not_faulted(require_gpu):
    """A NaN planted in the host copy of the state comes back as EXIT_INSTAB."""
    g = _prepared("tet_dir", 1)
    u = g.get_state(_lib.SLOT_UN)
    u[0, 0] = np.nan
    g.set_state(_lib.SLOT_UN, u)
    with pytest.raises(LymphError) as e:
        g.TIME_STEP_MATRIX_FREE(g.dt)
    assert e.value.code == _lib.LYMPH_EXIT_INSTAB
    g.close()


def test_non_spd_mass_is_reported(require_gpu):
    """A negative density makes M_loc negative definite: the reference's
    cholesky stops; here EXIT_SINGULARMTX comes back."""
    m = M.cube(1, agglomeration="tet", material=(-1.0, 1.0, 1.0))
    g = MatrixFree(m, 1, 1e-3)
    with pytest.raises(LymphError) as e:
        g.MAKE_MATRICES_FREE()
    assert e.value.code == _lib.LYMPH_EXIT_SINGULARMTX
    g.close()


def test_call_order_is_checked(require_gpu):
    g = MatrixFree(_mesh("tet_dir"), 1, 1e-3)
    with pytest.raises(LymphError) as e:
        g.TIME_STEP_MATRIX_FREE(0.0)
    assert e.value.code == _lib.LYMPH_ERR_ORDER
    g.close()
