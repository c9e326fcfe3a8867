"""CPU-side checks of the C ABI and the host set-up code (no GPU needed).

* the library loads and exports every function declared in include/*.h;
* mesh utilities: cube generation (positive orientation, face tags), hashed
  face matching (symmetric, every interior face matched once), boundary
  conditions, BFS agglomeration (sizes, connectivity, determinism);
* argument validation and the failure of lymph_create without a device come
  back as status codes with a message, never as a crash;
* the matrix-free path's triangle rules integrate every monomial of degree
  <= 2p exactly (lymph_mf_face_rule needs no device).
"""
import ctypes
import re
from collections import deque
from ctypes import byref, c_void_p
from pathlib import Path

import numpy as np
import pytest

from lymph3d_apsc_gb300 import _lib, mesh as M

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:int|const char\*|double)\s+(lymph_\w+)\s*\(", txt, flags=re.M)
    return names


def test_every_declared_symbol_is_exported():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding knows every one of them
    assert set(names) <= set(_lib.declared_symbols()), set(names) - set(_lib.declared_symbols())


def test_version_and_last_error():
    lib = _lib.load()
    assert lib.lymph_version() >= 10000
    assert isinstance(lib.lymph_last_error(), bytes)


@pytest.mark.parametrize("n", [1, 2, 3])
def test_cube_orientation_tags_and_matching(n):
    m = M.cube(n, bc="reference", agglomeration="tet")
    X, tv = m.coords, m.tet_vert
    e1, e2, e3 = (X[tv[:, k]] - X[tv[:, 0]] for k in (1, 2, 3))
    det = np.einsum("ij,ij->i", e1, np.cross(e2, e3))
    assert np.all(det > 0) and np.allclose(det.sum() / 6.0, 1.0)
    nb, nf = M.match_faces(tv)
    interior = nb >= 0
    # symmetric matching
    t, f = np.nonzero(interior)
    assert np.all(nb[nb[t, f], nf[t, f]] == t)
    # boundary faces: 2 triangles per cube face cell, 6 faces
    assert (~interior).sum() == 12 * n * n
    assert np.all(m.face_tag[~interior] > 0) and np.all(m.face_tag[interior] == 0)
    # reference convention: tags 2,3,4 Dirichlet, 5,6,7 Neumann
    assert np.all(m.neigh[~interior][np.isin(m.face_tag[~interior], [2, 3, 4])] == _lib.BC_DIRI)
    assert np.all(m.neigh[~interior][np.isin(m.face_tag[~interior], [5, 6, 7])] == _lib.BC_NEUM)
    assert set(np.unique(m.fun_tag[~interior])) <= {1, 2, 3}


def test_all_dirichlet_mode():
    m = M.cube(2, bc="dirichlet", agglomeration="tet")
    assert (m.neigh == _lib.BC_NEUM).sum() == 0 and (m.neigh == _lib.BC_DIRI).sum() == 48


def _connected(tets, neigh):
    s = set(int(t) for t in tets)
    seen, q = {int(tets[0])}, deque([int(tets[0])])
    while q:
        t = q.popleft()
        for e in neigh[t]:
            if e in s and e not in seen:
                seen.add(e)
                q.append(e)
    return len(seen) == len(s)


@pytest.mark.parametrize("lo,hi,seed", [(4, 12, 0), (4, 16, 5), (1, 1, 0)])
def test_bfs_agglomeration(lo, hi, seed):
    m = M.cube(4, agglomeration="bfs", group=(lo, hi), seed=seed)
    nb, _ = M.match_faces(m.tet_vert)
    sizes = np.bincount(m.tet_poly)
    assert sizes.sum() == m.n_tet and sizes.max() <= hi + lo - 1
    assert np.all(sizes >= lo)
    for P in range(m.n_poly):
        assert _connected(np.nonzero(m.tet_poly == P)[0], nb)
    again = M.cube(4, agglomeration="bfs", group=(lo, hi), seed=seed)
    assert np.array_equal(again.tet_poly, m.tet_poly)


def test_headline_mesh_has_about_48k_polyhedra():
    """40^3 x 6 tets in groups of U{4..12} (mean 8): ~48,000 polyhedra."""
    m = M.cube(40, agglomeration="bfs", group=(4, 12), seed=0)
    assert m.n_tet == 384000
    assert 46000 <= m.n_poly <= 50000


def test_find_tet():
    m = M.cube(3, agglomeration="tet", jitter=0.2)
    lib = _lib.load()
    rng = np.random.default_rng(0)
    for _ in range(20):
        x = np.ascontiguousarray(rng.random(3) * 0.9 + 0.05)
        t = ctypes.c_int32()
        tv = np.ascontiguousarray(m.tet_vert)
        X = np.ascontiguousarray(m.coords)
        assert lib.lymph_mesh_find_tet(m.n_tet, _lib.ptr(tv, ctypes.c_int32), _lib.ptr(X, ctypes.c_double),
                                       _lib.ptr(x, ctypes.c_double), byref(t)) == 0
        v = X[tv[t.value]]
        lam = np.linalg.solve((v[1:] - v[0]).T, x - v[0])
        assert lam.min() >= -1e-12 and lam.sum() <= 1 + 1e-12


def test_create_rejects_bad_input_with_status_codes():
    lib = _lib.load()
    m = M.cube(1, agglomeration="tet")
    h = c_void_p()
    bad = M.Mesh(m.coords, m.tet_vert, m.tet_poly, m.tet_mat, m.neigh.copy(), m.fun_tag, m.mat)
    bad.neigh[0, 0] = 10**6  # neighbour out of range
    d = bad.desc()
    prm = _lib.Params(2, _lib.FP64, 10.0, -1.0, 1e-3)
    assert lib.lymph_create(byref(d), byref(prm), byref(h)) == _lib.LYMPH_EXIT_NEIGHBOUR_EL_ERROR
    assert b"neighbour" in lib.lymph_last_error()
    d = m.desc()
    prm = _lib.Params(7, _lib.FP64, 10.0, -1.0, 1e-3)
    assert lib.lymph_create(byref(d), byref(prm), byref(h)) == _lib.LYMPH_ERR_INVALID
    prm = _lib.Params(2, _lib.FP64, 10.0, -1.0, -1.0)
    assert lib.lymph_create(byref(d), byref(prm), byref(h)) == _lib.LYMPH_ERR_INVALID
    assert lib.lymph_create(None, byref(prm), byref(h)) == _lib.LYMPH_ERR_INVALID
    prm = _lib.Params(2, 7, 10.0, -1.0, 1e-3)  # unknown precision
    assert lib.lymph_create(byref(d), byref(prm), byref(h)) == _lib.LYMPH_ERR_INVALID
    # calls on no context are refused, not dereferenced
    x = np.zeros(4)
    px = x.ctypes.data_as(_lib.P_F64)
    assert lib.lymph_time_step_host(None, 0.0, px, px, px, _lib.LAYOUT_FORTRAN) == _lib.LYMPH_ERR_INVALID
    assert lib.lymph_checkpoint_save(None, b"x.ckpt", 0.0, 0) == _lib.LYMPH_ERR_INVALID
    assert lib.lymph_checkpoint_load(None, b"x.ckpt", None, None) == _lib.LYMPH_ERR_INVALID
    assert lib.lymph_step(None, 0.0) == _lib.LYMPH_ERR_INVALID
    assert lib.lymph_get_self_blocks(None, px) == _lib.LYMPH_ERR_INVALID


def test_create_without_device_fails_loudly():
    """On a machine with no GPU the library reports LYMPH_ERR_CUDA; it never
    falls back to a host computation."""
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is visible")
    lib = _lib.load()
    m = M.cube(1, agglomeration="tet")
    d = m.desc()
    prm = _lib.Params(1, _lib.FP64, 10.0, -1.0, 1e-3)
    h = c_void_p()
    assert lib.lymph_create(byref(d), byref(prm), byref(h)) == _lib.LYMPH_ERR_CUDA
    assert not h.value
    with pytest.raises(_lib.LymphError):
        from lymph3d_apsc_gb300 import MatrixFree
        MatrixFree(m, 1, 1e-3)


def test_matrix_free_face_rules_are_exact_to_degree_2p():
    """The triangle rules of the matrix-free neighbour terms (no device
    needed): interior nodes, positive weights summing to 1/2, and every
    monomial xi^i eta^j with i + j <= 2p integrated to i! j! / (i+j+2)!
    within 1e-15 -- the degree of the face integrands, to which the
    reference's collapsed Gauss rule with (p+1)^2 nodes is also exact."""
    from ctypes import POINTER, byref, c_double, c_int32
    from math import factorial
    lib = _lib.load()
    for p in (1, 2, 3, 4):
        n = c_int32()
        assert lib.lymph_mf_face_rule(p, byref(n), None) == 0
        assert n.value == {1: 3, 2: 6, 3: 12, 4: 16}[p] < (p + 1) ** 2
        xyw = np.zeros(3 * n.value)
        assert lib.lymph_mf_face_rule(p, byref(n), xyw.ctypes.data_as(POINTER(c_double))) == 0
        xi, eta, w = xyw[0::3], xyw[1::3], xyw[2::3]
        assert np.all(w > 0) and np.all(xi > 0) and np.all(eta > 0) and np.all(xi + eta < 1)
        for i in range(2 * p + 1):
            for j in range(2 * p + 1 - i):
                exact = factorial(i) * factorial(j) / factorial(i + j + 2)
                assert abs(np.sum(w * xi ** i * eta ** j) - exact) <= 1e-15, (p, i, j)
    assert lib.lymph_mf_face_rule(5, byref(n), None) != 0


def test_face_rules_are_what_their_derivation_script_gives():
    """csrc/derive_face_rules.py (least squares from seeded starts, then
    Gauss-Newton at 40 digits) reproduces the library's triangle rules: the
    same nodes and weights, in any order, to 1e-15."""
    import importlib.util
    from ctypes import POINTER, byref, c_double, c_int32
    spec = importlib.util.spec_from_file_location(
        "derive_face_rules", ROOT / "lymph3d_apsc_gb300" / "csrc" / "derive_face_rules.py")
    d = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(d)
    lib = _lib.load()
    for p in (1, 2, 3, 4):
        x, res = d.refine(d.STRUCT[p], 2 * p, d.first_guess(d.STRUCT[p], 2 * p), iters=6)
        assert float(res) < 1e-30
        pts, ws = d.nodes(d.STRUCT[p], x, d.mp.mpf(1))
        got = np.array(sorted((float(a), float(b), float(w)) for (a, b), w in zip(pts, ws)))
        n = c_int32()
        lib.lymph_mf_face_rule(p, byref(n), None)
        xyw = np.zeros(3 * n.value)
        lib.lymph_mf_face_rule(p, byref(n), xyw.ctypes.data_as(POINTER(c_double)))
        want = np.array(sorted(map(tuple, xyw.reshape(-1, 3))))
        assert got.shape == want.shape
        assert np.abs(got - want).max() <= 1e-15, p
