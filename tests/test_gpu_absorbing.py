"""Absorbing boundaries on the GPU against the oracle (LYMPH_BC_ABSO: the
damping block of MAKE_DAMPING_FACE, src/assemble_element.f90:666-731, in the
leapfrog step of the polyhedra that have absorbing faces).

Bars (written in each assertion):
  * u^n after every one of 25 steps, both sides from the same coefficients:
    the bars of tests/test_gpu_parity.py (Euclidean <= max(1e-12, 4 x the
    oracle's own spread over valid evaluation orders, the damped solve
    included), mass norm <= 1e-12), p = 1..4, homogeneous and lognormal
    materials;
  * lymph_energy: constant (1e-9) on the traction-free mesh, decaying with
    absorbing faces, as on the oracle;
  * the FP32 operator forms (FP32 blocks, matrix-free FP32 face terms) on an
    absorbing mesh: the state after 20 steps within TOL_STEPS_FREE (1e-4) of
    the oracle in the mass norm.  This mesh has no Dirichlet face, so K has
    the rigid motions in its null space and the FP32 rounding of K u in those
    directions accumulates with no restoring force (measured up to 2.8e-5 at
    p = 4, against up to 6.5e-6 with Dirichlet faces, TOL_STEPS_FP32);
  * after lymph_set_dt, the steps equal an oracle made with the new dt (the
    damped polyhedra's M + dt/2 D is rebuilt).
"""
import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib
from lymph3d_apsc_gb300.ensemble import set_dt
from lymph3d_apsc_gb300.surrogate import energy
from oracle.oracle_py import Oracle
from parity_util import TOL_STATE, every_step_parity, mass_norm_rel, rel
from test_absorbing import _free_run, _mesh

pytestmark = pytest.mark.gpu

TOL_STEPS_FREE = 1e-4


@pytest.mark.parametrize("hetero", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_absorbing_every_step(require_gpu, p, hetero):
    m = _mesh(hetero=hetero)
    with MatrixFree(m, p, 1e-3) as g:
        o = Oracle(m, p, 1e-3)
        g.MAKE_MATRICES_FREE()
        o.make_matrices()
        e, floor, worst = every_step_parity(m, p, g, o, n_steps=25)
        o.close()
    assert worst <= 1.0
    print(f"absorbing p={p} hetero={hetero}: device vs oracle {e:.2e}, floor {floor:.2e}")


def _prepared(m, p, precision=_lib.FP64, dt=1e-3):
    g = MatrixFree(m, p, dt, precision=precision)
    g.MAKE_MATRICES_FREE()
    g.MAKE_RHS_FREE(_lib.RHS_STAT, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
    g.MAKE_RHS_FREE(_lib.RHS_DYN, _lib.F_NULL, _lib.GD_NULL, _lib.GN_NULL)
    g.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_DISPLACEMENT, _lib.SLOT_U0)
    g.COMPUTE_MODAL_COEFFICIENTS_FREE(_lib.FUN_IC_VELOCITY, _lib.SLOT_V0)
    g.FIRST_TIME_STEP_MATRIX_FREE(0.0)
    return g


@pytest.mark.parametrize("kind,decays", [("free", False), ("absorbing", True)])
def test_energy_on_the_device(require_gpu, kind, decays):
    g = _prepared(_mesh(kind), 2)
    E = [energy(g)]
    t = g.dt
    for _ in range(6):
        t, _, _, _ = g.run_steps(t, 1e9, 100)
        E.append(energy(g))
    g.close()
    E = np.array(E)
    print(kind, E)
    if decays:
        assert np.all(np.diff(E) < 0) and E[-1] < 0.2 * E[0], E
    else:
        assert np.abs(E / E[0] - 1).max() <= 1e-9, E


@pytest.mark.parametrize("precision", [_lib.MIXED, _lib.MIXED_MF])
@pytest.mark.parametrize("p", [2, 4])
def test_absorbing_fp32_forms(require_gpu, p, precision):
    m = _mesh(hetero=True)
    o = Oracle(m, p, 1e-3)
    _free_run(o)
    g = _prepared(m, p, precision)
    g.set_state(_lib.SLOT_U0, o.get_state(_lib.SLOT_U0))
    g.set_state(_lib.SLOT_UN, o.get_state(_lib.SLOT_UN))
    o.run_steps(1e-3, 1e9, 20)
    g.run_steps(1e-3, 1e9, 20)
    uo = o.get_state(_lib.SLOT_UN)
    em = mass_norm_rel(o, g.get_state(_lib.SLOT_UN), uo)
    print(f"p={p} precision={precision}: 20 absorbing steps, mass norm {em:.2e}")
    assert em <= TOL_STEPS_FREE
    g.close()
    o.close()


def test_new_dt_rebuilds_the_damped_solve(require_gpu):
    m = _mesh()
    p, dt1, dt2 = 2, 1e-3, 6e-4
    g = _prepared(m, p, dt=dt1)
    set_dt(g, dt2)
    o = Oracle(m, p, dt2)
    _free_run(o)
    g.set_state(_lib.SLOT_U0, o.get_state(_lib.SLOT_U0))
    g.set_state(_lib.SLOT_UN, o.get_state(_lib.SLOT_UN))
    t = dt2
    for _ in range(10):
        g.TIME_STEP_MATRIX_FREE(t)
        o.step(t)
        t += dt2
    e = rel(g.get_state(_lib.SLOT_UN), o.get_state(_lib.SLOT_UN))
    assert e <= 100 * TOL_STATE and mass_norm_rel(o, g.get_state(_lib.SLOT_UN), o.get_state(_lib.SLOT_UN)) <= TOL_STATE
    g.close()
    o.close()
