"""Meshes for the hot path: the flattened Mesh_Structure of lymph3d_gpu.h.

* `cube(...)`: structured unit-cube meshes of n^3 hexahedra x 6 tetrahedra,
  boundary tagged with the reference decks' cube-face tags, agglomerated into
  polyhedra (one per tet, one per hexahedron, or seeded BFS groups).
* `read_deck(dir)`: a reference input deck (Poly.input, *.mate, *.mesh as
  parsed by src/Poly_readfile.f90:9-187, :327-707, :847-1050).

All integer work runs in the library's host code (lymph3d_mesh.h).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import P_F64, P_I32, check, ptr
from ctypes import c_double, c_int32, byref


@dataclass
class Mesh:
    coords: np.ndarray            # (n_node, 3) float64
    tet_vert: np.ndarray          # (n_tet, 4) int32
    tet_poly: np.ndarray          # (n_tet,) int32
    tet_mat: np.ndarray           # (n_tet,) int32
    neigh: np.ndarray             # (n_tet, 4) int32, BC_DIRI / BC_NEUM on the boundary
    fun_tag: np.ndarray           # (n_tet, 4) int32
    mat: np.ndarray               # (n_mat, 3) float64: rho, lambda, mu
    face_tag: np.ndarray | None = None
    info: dict = field(default_factory=dict)

    @property
    def n_tet(self) -> int:
        return int(self.tet_vert.shape[0])

    @property
    def n_poly(self) -> int:
        return int(self.tet_poly.max()) + 1 if self.tet_poly.size else 0

    @property
    def n_node(self) -> int:
        return int(self.coords.shape[0])

    def desc(self) -> _lib.MeshDesc:
        """ctypes descriptor; the arrays are pinned on the Mesh object."""
        for name in ("coords", "mat"):
            setattr(self, name, np.ascontiguousarray(getattr(self, name), dtype=np.float64))
        for name in ("tet_vert", "tet_poly", "tet_mat", "neigh", "fun_tag"):
            setattr(self, name, np.ascontiguousarray(getattr(self, name), dtype=np.int32))
        d = _lib.MeshDesc()
        d.n_node, d.n_tet, d.n_poly, d.n_mat = self.n_node, self.n_tet, self.n_poly, int(self.mat.shape[0])
        d.coords = ptr(self.coords, c_double)
        d.tet_vert = ptr(self.tet_vert, c_int32)
        d.tet_poly = ptr(self.tet_poly, c_int32)
        d.tet_mat = ptr(self.tet_mat, c_int32)
        d.neigh = ptr(self.neigh, c_int32)
        d.fun_tag = ptr(self.fun_tag, c_int32)
        d.mat = ptr(self.mat, c_double)
        return d

    def with_polyhedra(self, tet_poly: np.ndarray) -> "Mesh":
        return Mesh(self.coords, self.tet_vert, np.ascontiguousarray(tet_poly, dtype=np.int32), self.tet_mat,
                    self.neigh, self.fun_tag, self.mat, self.face_tag, dict(self.info))


def match_faces(tet_vert: np.ndarray):
    lib = _lib.load()
    tv = np.ascontiguousarray(tet_vert, dtype=np.int32)
    nt = tv.shape[0]
    neigh = np.empty((nt, 4), np.int32)
    nface = np.empty((nt, 4), np.int32)
    check(lib.lymph_mesh_match_faces(nt, ptr(tv, c_int32), ptr(neigh, c_int32), ptr(nface, c_int32)),
          "lymph_mesh_match_faces")
    return neigh, nface


def apply_bc(face_tag: np.ndarray, neigh: np.ndarray, mode: int):
    lib = _lib.load()
    ft = np.ascontiguousarray(face_tag, dtype=np.int32)
    nb = np.ascontiguousarray(neigh, dtype=np.int32).copy()
    fun = np.zeros_like(nb)
    check(lib.lymph_mesh_apply_bc(nb.shape[0], ptr(ft, c_int32), mode, ptr(nb, c_int32), ptr(fun, c_int32)),
          "lymph_mesh_apply_bc")
    return nb, fun


def agglomerate(neigh: np.ndarray, seed: int, min_size: int, max_size: int) -> np.ndarray:
    """Seeded BFS grouping (lymph_mesh_agglomerate); works on the matched
    neighbour table (boundary entries are ignored)."""
    lib = _lib.load()
    nb = np.ascontiguousarray(neigh, dtype=np.int32)
    tp = np.empty(nb.shape[0], np.int32)
    npoly = c_int32(0)
    check(lib.lymph_mesh_agglomerate(nb.shape[0], ptr(nb, c_int32), seed, min_size, max_size, ptr(tp, c_int32),
                                     byref(npoly)), "lymph_mesh_agglomerate")
    return tp


def cube(n: int, bc: str = "dirichlet", agglomeration: str = "tet", seed: int = 0, group=(4, 12),
         material=(1.0, 1.0, 1.0), poly_materials: np.ndarray | None = None, jitter: float = 0.0,
         jitter_seed: int = 7) -> Mesh:
    """Structured [0,1]^3 mesh of n^3 hexahedra x 6 tetrahedra.

    bc: "dirichlet" (every boundary face Dirichlet), "reference" (the decks'
    convention: z=0, z=1, x=1 Dirichlet; y=1, x=0, y=0 Neumann) or
    "absorbing" (z=1 a free surface, i.e. Neumann; every other boundary face
    absorbing, LYMPH_BC_ABSO).
    agglomeration: "tet" (one polyhedron per tetrahedron, the reference's only
    consistent mode), "hex" (6 tets per polyhedron) or "bfs" (seeded groups of
    group[0]..group[1] tets).
    poly_materials: optional (n_poly, 3) rho/lambda/mu per polyhedron.
    jitter: interior nodes are moved by jitter*h*U(-1/2,1/2)^3 (seeded) to
    make the tetrahedra irregular; jitter <= 0.3 keeps every det J > 0.
    """
    lib = _lib.load()
    nn, nt = c_int32(0), c_int32(0)
    check(lib.lymph_mesh_cube_sizes(n, n, n, byref(nn), byref(nt)), "lymph_mesh_cube_sizes")
    coords = np.empty((nn.value, 3), np.float64)
    tv = np.empty((nt.value, 4), np.int32)
    ftag = np.empty((nt.value, 4), np.int32)
    check(lib.lymph_mesh_cube(n, n, n, ptr(coords, c_double), ptr(tv, c_int32), ptr(ftag, c_int32)), "lymph_mesh_cube")
    if jitter > 0.0:
        rng = np.random.default_rng(jitter_seed)
        interior = np.all((coords > 0.0) & (coords < 1.0), axis=1)
        coords[interior] += jitter / n * (rng.random((int(interior.sum()), 3)) - 0.5)
    neigh, _ = match_faces(tv)
    matched = neigh.copy()
    mode = _lib.BCMODE_ALL_DIRICHLET if bc == "dirichlet" else _lib.BCMODE_REFERENCE
    neigh, fun = apply_bc(ftag, neigh, mode)
    if bc == "absorbing":
        neigh = set_absorbing(neigh, ftag, tags=(2, 4, 5, 6, 7))
        neigh[(neigh < 0) & (ftag == 3)] = _lib.BC_NEUM
    elif bc not in ("dirichlet", "reference"):
        raise ValueError(f"unknown boundary condition set {bc!r}")
    if agglomeration == "tet":
        tp = np.arange(nt.value, dtype=np.int32)
    elif agglomeration == "hex":
        tp = (np.arange(nt.value, dtype=np.int32) // 6).astype(np.int32)
    elif agglomeration == "bfs":
        tp = agglomerate(matched, seed, group[0], group[1])
    else:
        raise ValueError(f"unknown agglomeration {agglomeration!r}")
    if poly_materials is not None:
        mat = np.ascontiguousarray(poly_materials, dtype=np.float64)
        tmat = tp.copy()
    else:
        mat = np.array([material], np.float64)
        tmat = np.zeros(nt.value, np.int32)
    return Mesh(coords, tv, tp, tmat, neigh, fun, mat, ftag,
                {"n": n, "bc": bc, "agglomeration": agglomeration, "seed": seed, "group": tuple(group)})


def set_absorbing(neigh: np.ndarray, face_tag: np.ndarray, tags) -> np.ndarray:
    """The boundary faces whose tag is in `tags` become absorbing
    (LYMPH_BC_ABSO), the reference's ABSO records (Poly_readfile.f90:521)."""
    nb = np.array(neigh, dtype=np.int32, copy=True)
    sel = (nb < 0) & np.isin(face_tag, np.asarray(list(tags), dtype=np.int32))
    nb[sel] = _lib.BC_ABSO
    return nb


def lognormal_materials(n_poly: int, seed: int, sigma: float = 0.5, rho: float = 1.0) -> np.ndarray:
    """Per-polyhedron lambda, mu ~ exp(sigma N(0,1)) (median 1), rho fixed."""
    rng = np.random.default_rng(seed)
    lam = np.exp(sigma * rng.standard_normal(n_poly))
    mu = np.exp(sigma * rng.standard_normal(n_poly))
    return np.stack([np.full(n_poly, rho), lam, mu], axis=1)


# ---------------------------------------------------------------------------
# reference input decks
# ---------------------------------------------------------------------------
def _read_keywords(path: Path) -> dict:
    out = {}
    for line in path.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0].isupper():
            out[parts[0]] = parts[1]
    return out


def read_mate(path: Path, with_abso: bool = False):
    """MATE / DIRI / NEUM (and ABSO) records (Poly_readfile.f90:327-707).
    lambda = rho (vp^2 - 2 vs^2), mu = rho vs^2 (:393-412).  Returns
    (mats, diri, neum), and the ABSO tags as a fourth item with with_abso."""
    mats, diri, neum, abso = [], {}, {}, []
    for line in Path(path).read_text().splitlines():
        p = line.split()
        if not p:
            continue
        if p[0] == "MATE":
            tag, deg, rho, vs, vp = int(p[1]), int(p[2]), float(p[3]), float(p[4]), float(p[5])
            mats.append((tag, deg, rho, rho * (vp * vp - 2 * vs * vs), rho * vs * vs))
        elif p[0] == "DIRI":
            diri[int(p[1])] = int(p[2])
        elif p[0] == "NEUM":
            neum[int(p[1])] = int(p[2])
        elif p[0] == "ABSO":
            abso.append(int(p[1]))
    return (mats, diri, neum, abso) if with_abso else (mats, diri, neum)


def read_mesh_file(path: Path):
    """Nodes, tetrahedra (material tag + 4 nodes) and tagged boundary
    triangles of a .mesh file (READ_MESHFILE, Poly_readfile.f90:847-1050)."""
    lines = [l for l in Path(path).read_text().splitlines() if l.strip() and not l.startswith("#")]
    n_node, n_elem = (int(x) for x in lines[0].split()[:2])
    coords = np.array([[float(v) for v in l.split()[1:4]] for l in lines[1:1 + n_node]], np.float64)
    tets, tmat, tris, ttag = [], [], [], []
    for l in lines[1 + n_node:1 + n_node + n_elem]:
        m = re.match(r"\s*(\d+)\s+(-?\d+)\s+([A-Za-z]+)\s+(.*)", l)
        if not m:
            continue
        tag, kw, rest = int(m.group(2)), m.group(3).lower(), [int(v) for v in m.group(4).split()]
        if kw == "tetra":
            tets.append(rest[:4]); tmat.append(tag)
        elif kw == "tria":
            tris.append(rest[:3]); ttag.append(tag)
    return (coords, np.array(tets, np.int32) - 1, np.array(tmat, np.int32), np.array(tris, np.int32) - 1,
            np.array(ttag, np.int32))


def read_deck_arrays(deck_dir) -> dict:
    """The raw contents of a reference deck: nodes, tetrahedra with their
    material tags, tagged boundary triangles (0-based), the MATE table
    (tag, degree, rho, lambda, mu) and the Poly.input time parameters."""
    d = Path(deck_dir)
    kw = _read_keywords(d / "Poly.input")
    mats, diri, neum, abso = read_mate(d / (kw["MATFILE"] + ".mate"), with_abso=True)
    coords, tv, tmat, tris, ttag = read_mesh_file(d / (kw["GRIDFILE"] + ".mesh"))
    return {"coords": coords, "tet_vert": tv, "tet_mat_tag": tmat, "tria": tris, "tria_tag": ttag,
            "mate": np.array(mats, np.float64).reshape(-1, 5),
            "diri_tags": np.array(sorted(diri), np.int32), "neum_tags": np.array(sorted(neum), np.int32),
            "abso_tags": np.array(sorted(abso), np.int32),
            "dt": np.float64(kw.get("TIMESTEP", "1e-3")), "stop_time": np.float64(kw.get("STOPTIME", "1")),
            "name": d.name}


def deck_mesh(arrays: dict, override_materials: bool = True) -> tuple[Mesh, dict]:
    """Mesh of a deck's raw arrays (read_deck_arrays, or a fixture saved from
    it): boundary triangles tagged on the tetrahedra's faces, faces matched,
    the decks' tag convention applied (2-4 Dirichlet, 5-7 Neumann,
    MAKE_PARTITION_AND_MPI_FILES.f90:2105-2109), one polyhedron per
    tetrahedron; faces whose tag has an ABSO record are absorbing.  With
    override_materials the driver's rho = lambda = mu = 1 override
    (Lymph3D.f90:196-203) is applied."""
    lib = _lib.load()
    tv = np.ascontiguousarray(arrays["tet_vert"], dtype=np.int32)
    tris = np.ascontiguousarray(arrays["tria"], dtype=np.int32)
    ttag = np.ascontiguousarray(arrays["tria_tag"], dtype=np.int32)
    coords = np.ascontiguousarray(arrays["coords"], dtype=np.float64)
    mats = np.asarray(arrays["mate"], dtype=np.float64).reshape(-1, 5)
    ftag = np.zeros_like(tv)
    nunf = c_int32(0)
    check(lib.lymph_mesh_tag_boundary(tv.shape[0], ptr(tv, c_int32), tris.shape[0], ptr(tris, c_int32),
                                      ptr(ttag, c_int32), ptr(ftag, c_int32), byref(nunf)), "lymph_mesh_tag_boundary")
    neigh, _ = match_faces(tv)
    neigh, fun = apply_bc(ftag, neigh, _lib.BCMODE_REFERENCE)
    abso = arrays.get("abso_tags")
    if abso is not None and len(abso):
        neigh = set_absorbing(neigh, ftag, abso)
    tag_to_idx = {int(m[0]): i for i, m in enumerate(mats)}
    tet_mat = np.array([tag_to_idx[int(t)] for t in arrays["tet_mat_tag"]], np.int32)
    if override_materials:
        mat = np.ones((mats.shape[0], 3), np.float64)
    else:
        mat = np.ascontiguousarray(mats[:, 2:5])
    mesh = Mesh(coords, tv, np.arange(tv.shape[0], dtype=np.int32), tet_mat, neigh, fun, mat, ftag,
                {"deck": str(arrays.get("name", "")), "unfound_tria": nunf.value})
    params = {"dt": float(arrays["dt"]), "stop_time": float(arrays["stop_time"]), "degree": int(mats[0, 1])}
    return mesh, params


def read_deck(deck_dir, override_materials: bool = True) -> tuple[Mesh, dict]:
    """Reads a reference deck (Poly.input, *.mate, *.mesh).  Returns the mesh
    (one polyhedron per tetrahedron) and the Poly.input values."""
    return deck_mesh(read_deck_arrays(deck_dir), override_materials)
