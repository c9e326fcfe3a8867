"""Benchmark meshes built without the GPU library (test infrastructure).

TEST INFRASTRUCTURE ONLY: the reference arm of bench.py and the tests use it
so that the CPU oracle can run the benchmark workloads in a process that never
loads liblymph3d_gb300.so.  It restates, in numpy and plain Python, the
library's host-side mesh set-up (lymph3d_apsc_gb300/csrc/mesh.cpp):

* the structured unit cube of n^3 hexahedra x 6 tetrahedra with the reference
  decks' boundary tags (z=0: 2, z=1: 3, x=1: 4, y=1: 5, x=0: 6, y=0: 7), the
  face vertex triples of MAKE_PARTITION_AND_MPI_FILES.f90:1087-1096;
* face matching (each interior triangle shared by exactly two tetrahedra);
* the boundary conditions (tags 2-4 Dirichlet, 5-7 Neumann as at
  MAKE_PARTITION_AND_MPI_FILES.f90:2105-2109, or every boundary face
  Dirichlet) and the space-function tags;
* the seeded BFS agglomeration into groups of min..max tetrahedra (splitmix64
  draws, stragglers merged into the smallest adjacent group, polyhedra
  numbered by first tetrahedron).

tests/test_oracle_kat.py checks that every array equals the library's.
"""
from __future__ import annotations

import ctypes
from collections import deque
from ctypes import POINTER, c_double, c_int32

import numpy as np

FACE_V = np.array([[0, 1, 2], [0, 1, 3], [1, 2, 3], [2, 0, 3]])
BC_DIRI, BC_NEUM, UNMATCHED = -1, -2, -9
MASK64 = (1 << 64) - 1


class MeshDesc(ctypes.Structure):
    """lymph_mesh_desc (include/lymph3d_gpu.h), the oracle's input."""
    _fields_ = [
        ("n_node", c_int32), ("n_tet", c_int32), ("n_poly", c_int32), ("n_mat", c_int32),
        ("coords", POINTER(c_double)), ("tet_vert", POINTER(c_int32)), ("tet_poly", POINTER(c_int32)),
        ("tet_mat", POINTER(c_int32)), ("neigh", POINTER(c_int32)), ("fun_tag", POINTER(c_int32)),
        ("mat", POINTER(c_double)),
    ]


class OracleMesh:
    """The arrays of lymph_mesh_desc, held for the oracle."""

    def __init__(self, coords, tet_vert, tet_poly, tet_mat, neigh, fun_tag, mat):
        self.coords = np.ascontiguousarray(coords, np.float64)
        self.tet_vert = np.ascontiguousarray(tet_vert, np.int32)
        self.tet_poly = np.ascontiguousarray(tet_poly, np.int32)
        self.tet_mat = np.ascontiguousarray(tet_mat, np.int32)
        self.neigh = np.ascontiguousarray(neigh, np.int32)
        self.fun_tag = np.ascontiguousarray(fun_tag, np.int32)
        self.mat = np.ascontiguousarray(mat, np.float64)

    @property
    def n_tet(self):
        return int(self.tet_vert.shape[0])

    @property
    def n_poly(self):
        return int(self.tet_poly.max()) + 1

    def desc(self) -> MeshDesc:
        d = MeshDesc()
        d.n_node, d.n_tet, d.n_poly, d.n_mat = self.coords.shape[0], self.n_tet, self.n_poly, self.mat.shape[0]
        d.coords = self.coords.ctypes.data_as(POINTER(c_double))
        d.tet_vert = self.tet_vert.ctypes.data_as(POINTER(c_int32))
        d.tet_poly = self.tet_poly.ctypes.data_as(POINTER(c_int32))
        d.tet_mat = self.tet_mat.ctypes.data_as(POINTER(c_int32))
        d.neigh = self.neigh.ctypes.data_as(POINTER(c_int32))
        d.fun_tag = self.fun_tag.ctypes.data_as(POINTER(c_int32))
        d.mat = self.mat.ctypes.data_as(POINTER(c_double))
        return d


def cube_arrays(n: int):
    """Nodes, tetrahedra (positively oriented) and face tags of the cube."""
    ax = np.arange(n + 1) / n
    k, j, i = np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij")
    coords = np.stack([ax[i.ravel()], ax[j.ravel()], ax[k.ravel()]], axis=1)

    def node(i, j, k):
        return i + (n + 1) * (j + (n + 1) * k)

    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    c, b, a = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = np.stack([a.ravel(), b.ravel(), c.ravel()], axis=1)          # hexahedra in (a fastest) order
    tv = np.empty((base.shape[0], 6, 4), np.int64)
    for p, perm in enumerate(perms):
        cur = base.copy()
        tv[:, p, 0] = node(cur[:, 0], cur[:, 1], cur[:, 2])
        for s in range(3):
            cur[:, perm[s]] += 1
            tv[:, p, s + 1] = node(cur[:, 0], cur[:, 1], cur[:, 2])
    tv = tv.reshape(-1, 4)
    e = coords[tv[:, 1:]] - coords[tv[:, :1]]
    det = np.einsum("ij,ij->i", e[:, 0], np.cross(e[:, 1], e[:, 2]))
    sw = det < 0
    tv[sw, 1], tv[sw, 2] = tv[sw, 2].copy(), tv[sw, 1].copy()
    fv = coords[tv[:, FACE_V]]                                          # [n_tet, 4, 3 vertices, 3]
    tag = np.zeros((tv.shape[0], 4), np.int32)
    for t_val, d, val in ((7, 1, 0.0), (6, 0, 0.0), (5, 1, 1.0), (4, 0, 1.0), (3, 2, 1.0), (2, 2, 0.0)):
        on = np.all(fv[..., d] == val, axis=2)
        tag[on] = t_val
    return coords, tv.astype(np.int32), tag


def match_faces(tv: np.ndarray) -> np.ndarray:
    """neigh[t, f] = the tetrahedron across face f, UNMATCHED on the boundary."""
    nt = tv.shape[0]
    keys = np.sort(tv[:, FACE_V].reshape(-1, 3), axis=1)
    order = np.lexsort((keys[:, 2], keys[:, 1], keys[:, 0]))
    ks = keys[order]
    same = np.all(ks[1:] == ks[:-1], axis=1)
    if np.any(same[1:] & same[:-1]):
        raise ValueError("a triangle is shared by more than two tetrahedra")
    neigh = np.full(nt * 4, UNMATCHED, np.int64)
    a, b = order[:-1][same], order[1:][same]
    neigh[a] = b // 4
    neigh[b] = a // 4
    return neigh.reshape(nt, 4).astype(np.int32)


def apply_bc(face_tag: np.ndarray, neigh: np.ndarray, all_dirichlet: bool):
    nb = neigh.copy()
    fun = np.zeros_like(nb)
    bnd = nb < 0
    if np.any(face_tag[bnd] == 0):
        raise ValueError("untagged boundary face")
    tag = face_tag[bnd]
    diri = np.isin(tag, (2, 3, 4)) | all_dirichlet
    nb[bnd] = np.where(diri, BC_DIRI, BC_NEUM)
    fun[bnd] = np.where((tag >= 2) & (tag <= 4), tag - 1, np.where((tag >= 5) & (tag <= 7), tag - 4, 1))
    return nb, fun


def _splitmix64(state: int):
    state = (state + 0x9E3779B97F4A7C15) & MASK64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return state, z ^ (z >> 31)


def agglomerate(neigh: np.ndarray, seed: int, min_size: int, max_size: int) -> np.ndarray:
    """Seeded BFS grouping on the matched neighbour table."""
    nt = neigh.shape[0]
    nbl = neigh.tolist()
    grp = [-1] * nt
    gsize = []
    s = seed & MASK64
    for t0 in range(nt):
        if grp[t0] >= 0:
            continue
        s, r = _splitmix64(s)
        target = min_size + r % (max_size - min_size + 1)
        g = len(gsize)
        gsize.append(0)
        q = deque([t0])
        grp[t0] = g
        while q and gsize[g] < target:
            t = q.popleft()
            if grp[t] != g:
                continue
            gsize[g] += 1
            row = nbl[t]
            for f in range(4):
                if gsize[g] + len(q) >= target:
                    break
                nn = row[f]
                if nn >= 0 and grp[nn] < 0:
                    grp[nn] = g
                    q.append(nn)
        for t in q:
            if grp[t] == g:
                grp[t] = -1
    ng = len(gsize)
    gsize = [0] * ng
    for t in range(nt):
        gsize[grp[t]] += 1
    merge_cap = max_size + min_size - 1
    parent = list(range(ng))

    def find(g):
        while parent[g] != g:
            parent[g] = parent[parent[g]]
            g = parent[g]
        return g

    members = [[] for _ in range(ng)]
    for t in range(nt):
        members[grp[t]].append(t)
    for g in range(ng):
        if find(g) != g or gsize[g] >= min_size:
            continue
        best = -1
        for t in members[g]:
            for f in range(4):
                nn = nbl[t][f]
                if nn < 0:
                    continue
                h = find(grp[nn])
                if h == g or gsize[h] + gsize[g] > merge_cap:
                    continue
                if best < 0 or gsize[h] < gsize[best]:
                    best = h
        if best >= 0:
            parent[g] = best
            gsize[best] += gsize[g]
            members[best].extend(members[g])
            members[g] = []
            gsize[g] = 0
    ids = [-1] * ng
    tp = np.empty(nt, np.int32)
    npoly = 0
    for t in range(nt):
        r = find(grp[t])
        if ids[r] < 0:
            ids[r] = npoly
            npoly += 1
        tp[t] = ids[r]
    return tp


def lognormal_materials(n_poly: int, seed: int, sigma: float = 0.5, rho: float = 1.0) -> np.ndarray:
    """Per-polyhedron lambda, mu ~ exp(sigma N(0,1)) (median 1), rho fixed."""
    rng = np.random.default_rng(seed)
    lam = np.exp(sigma * rng.standard_normal(n_poly))
    mu = np.exp(sigma * rng.standard_normal(n_poly))
    return np.stack([np.full(n_poly, rho), lam, mu], axis=1)


def cube(n: int, bc: str = "dirichlet", agglomeration: str = "tet", seed: int = 0, group=(4, 12),
         material=(1.0, 1.0, 1.0), lognormal_seed: int | None = None) -> OracleMesh:
    """The library's cube(n, bc, agglomeration, seed, group, material) without
    jitter; lognormal_seed gives per-polyhedron lognormal lambda, mu."""
    coords, tv, ftag = cube_arrays(n)
    matched = match_faces(tv)
    neigh, fun = apply_bc(ftag, matched, bc == "dirichlet")
    nt = tv.shape[0]
    if agglomeration == "tet":
        tp = np.arange(nt, dtype=np.int32)
    elif agglomeration == "hex":
        tp = (np.arange(nt) // 6).astype(np.int32)
    elif agglomeration == "bfs":
        tp = agglomerate(matched, seed, group[0], group[1])
    else:
        raise ValueError(agglomeration)
    if lognormal_seed is not None:
        mat = lognormal_materials(int(tp.max()) + 1, lognormal_seed)
        tmat = tp.copy()
    else:
        mat = np.array([material], np.float64)
        tmat = np.zeros(nt, np.int32)
    return OracleMesh(coords, tv, tp, tmat, neigh, fun, mat)
