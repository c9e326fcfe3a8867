"""Absorbing boundaries (LYMPH_BC_ABSO): MAKE_DAMPING_FACE
(src/assemble_element.f90:666-731) as a damping term D in the leapfrog step,
  (M + dt/2 D) u^{n+1} = dt^2 (F - K u^n) + 2 M u^n - (M - dt/2 D) u^{n-1},
on the polyhedra that have absorbing faces (the reference's matrix-free
path leaves the call commented out, src/matrix_free.f90:279-287).

CPU (oracle): D is symmetric positive semi-definite with the impedance
matrix's value on constants; without forcing, the discrete leapfrog energy
stays constant on a traction-free mesh (to 1e-9 relative over 600 steps)
and decays with absorbing faces.
GPU: u^n after every step against the oracle with the bars of
tests/test_gpu_parity.py; the same energy behaviour through lymph_energy;
the FP32 operator forms on an absorbing mesh in the mass norm; a new dt
(lymph_set_dt) rebuilds M + dt/2 D.
"""
import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib, mesh as M
from oracle.oracle_py import Oracle


def _mesh(kind="absorbing", n=3, jitter=0.15, hetero=False):
    m = M.cube(n, bc="absorbing", agglomeration="bfs", seed=0, group=(4, 12), jitter=jitter)
    if hetero:
        m = M.cube(n, bc="absorbing", agglomeration="bfs", seed=0, group=(4, 12), jitter=jitter,
                   poly_materials=M.lognormal_materials(m.n_poly, seed=4))
    if kind == "free":  # the same mesh, every absorbing face traction-free instead
        nb = np.where(m.neigh == _lib.BC_ABSO, _lib.BC_NEUM, m.neigh).astype(np.int32)
        m = M.Mesh(m.coords, m.tet_vert, m.tet_poly, m.tet_mat, nb, m.fun_tag, m.mat, m.face_tag)
    return m


def _oracle_energy(o, dt):
    """E = 1/2 |(u^n - u^{n-1}) / dt|^2_M + 1/2 u^n . K u^{n-1}."""
    rp, col = o.pattern()
    K, Mr = o.blocks(0), o.mass(0)
    ua, ub = o.get_state(0), o.get_state(1)
    d = (ub - ua).reshape(o.n_poly, 3, o.Np) / dt
    Ku = np.zeros_like(ua)
    for P in range(o.n_poly):
        for k in range(rp[P], rp[P + 1]):
            Ku[P] += K[k] @ ua[col[k]]
    return 0.5 * np.einsum("pim,pmn,pin->", d, Mr, d) + 0.5 * float(np.sum(ub * Ku))


def _free_run(o):
    o.make_matrices()
    o.make_rhs(0, 0, 0, 0)
    o.make_rhs(1, 0, 0, 0)
    o.modal_project(0, 0)
    o.modal_project(1, 2)
    o.first_step(0.0)


def test_mesh_absorbing_faces():
    m = _mesh()
    bnd = m.neigh < 0
    assert (m.neigh == _lib.BC_ABSO).sum() == 5 * 2 * 9 and (m.neigh == _lib.BC_NEUM).sum() == 2 * 9
    assert np.all(m.face_tag[m.neigh == _lib.BC_NEUM] == 3) and bnd.sum() == 6 * 2 * 9


@pytest.mark.parametrize("kind,decays", [("free", False), ("absorbing", True)])
def test_oracle_energy_conserved_without_and_decaying_with_absorbing_faces(kind, decays):
    m = _mesh(kind)
    dt = 1e-3
    o = Oracle(m, 2, dt)
    _free_run(o)
    E = [_oracle_energy(o, dt)]
    t = dt
    for _ in range(6):
        t, _ = o.run_steps(t, 1e9, 100)
        E.append(_oracle_energy(o, dt))
    o.close()
    E = np.array(E)
    if decays:
        assert np.all(np.diff(E) < 0) and E[-1] < 0.2 * E[0], E
    else:
        assert np.abs(E / E[0] - 1).max() <= 1e-9, E


def test_oracle_damping_block_is_symmetric_psd():
    """D of every absorbing polyhedron, recovered from the first step of a
    unit velocity field: the first step subtracts D v^0 from the load, so
    the difference of two first steps (v^0 = e_k, and 0) is dt^2/2 M^-1 D e_k."""
    m = _mesh(n=2, jitter=0.0)
    p, dt = 1, 1e-3
    o = Oracle(m, p, dt)
    o.make_matrices()
    o.make_rhs(0, 0, 0, 0)
    o.make_rhs(1, 0, 0, 0)
    Mr = o.mass(0)
    nd, Np = o.nd, o.Np
    cols = []
    zero = np.zeros((o.n_poly, nd))
    o.set_state(0, zero)
    o.set_state(2, zero)
    o.first_step(0.0)
    base = o.get_state(1)
    P = int(np.nonzero([np.any(m.neigh[m.tet_poly == q] == _lib.BC_ABSO) for q in range(o.n_poly)])[0][0])
    for k in range(nd):
        v = zero.copy()
        v[P, k] = 1.0
        o.set_state(2, v)
        o.first_step(0.0)
        du = (o.get_state(1) - base)[P] - dt * v[P]   # = -dt^2/2 M^-1 D e_k
        x = -2.0 / dt ** 2 * du
        cols.append(np.concatenate([Mr[P] @ x[i * Np:(i + 1) * Np] for i in range(3)]))
    o.close()
    D = np.array(cols).T
    assert np.abs(D - D.T).max() <= 1e-10 * np.abs(D).max()
    w = np.linalg.eigvalsh(0.5 * (D + D.T))
    assert w.min() >= -1e-10 * w.max() and w.max() > 0
