"""Double-couple seismic source (MAKE_RHS_FREE's val_sism_el loop,
matrix_free.f90:602-664; MAKE_DOUBLE_COUPLE, assemble_element.f90:116-167).

CPU: the oracle's load is the known answer M' grad(phi) on the source
polyhedron's degree-1 basis functions (the tetrahedron quadrature integrates
a constant exactly, and the moment density carries 1/|T|), zero on the
constant one and on every other polyhedron.  GPU: the device load equals the
oracle's (<= 1e-12 relative) at p = 1..4, added to an existing RHS.
"""
import math

import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib, mesh as M
from lymph3d_apsc_gb300 import ensemble as E
from oracle import oracle_py as O
from oracle.oracle_py import Oracle

S_VEC = np.array([0.6, -0.48, 0.64])
N_VEC = np.array([0.0, 0.8, 0.6])
M0 = 2.5


def test_oracle_double_couple_known_answer():
    m = M.cube(2, bc="dirichlet", agglomeration="tet", jitter=0.2, seed=1)
    p = 1
    o = Oracle(m, p, 1e-3)
    o.make_matrices()
    o.make_rhs(1, 0, 0, 0)  # zero dynamic RHS
    t = 5
    o.make_rhs_double_couple(1, t, S_VEC, N_VEC, M0)
    b = o.rhs(1)
    P = int(m.tet_poly[t])
    assert np.count_nonzero(np.abs(b).sum(axis=1)) == 1 and np.abs(b[P]).sum() > 0
    bb, _ = o.poly_geometry()
    lib = O.load()
    bl = np.empty(3 * o.Np, np.int32)
    lib.oracle_basis_list(p, bl.ctypes.data_as(O.POINTER(O.ctypes.c_int)))
    bl = bl.reshape(o.Np, 3)
    Mp = (np.outer(S_VEC, N_VEC) + np.outer(N_VEC, S_VEC)) * M0
    hb = [(bb[P][2 * d + 1] - bb[P][2 * d]) / 2 for d in range(3)]
    for f in range(o.Np):
        grad = np.zeros(3)
        if bl[f].sum() == 1:  # degree-1 basis function: constant gradient along one axis
            d = int(np.argmax(bl[f]))
            grad[d] = 1.0 / (hb[d] * math.sqrt(hb[d]))
            for e in range(3):
                if e != d:
                    grad[d] /= math.sqrt(hb[e])
        want = Mp @ grad
        got = np.array([b[P, i * o.Np + f] for i in range(3)])
        assert np.abs(got - want).max() <= 1e-12 * max(np.abs(Mp).max() * np.abs(grad).max(), 1.0)
    o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_device_double_couple_matches_oracle(require_gpu, p):
    m = M.cube(3, bc="dirichlet", agglomeration="bfs", group=(4, 12), jitter=0.15, seed=2)
    x0 = [0.43, 0.51, 0.38]
    o = Oracle(m, p, 1e-3)
    o.make_matrices()
    o.make_rhs(1, 1, 1, 1)
    with MatrixFree(m, p, 1e-3) as g:
        g.MAKE_MATRICES_FREE()
        g.MAKE_RHS_FREE(_lib.RHS_DYN, _lib.F_TIME, _lib.GD, _lib.GN)
        tet = E.double_couple(g, x0, S_VEC, N_VEC, M0)
        got = g.rhs(_lib.RHS_DYN)
    o.make_rhs_double_couple(1, tet, S_VEC, N_VEC, M0)
    want = o.rhs(1)
    o.close()
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
