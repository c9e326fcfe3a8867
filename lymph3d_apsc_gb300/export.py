"""Nodal values of the modal solution and the reference's output files.

`nodal_values` calls lymph_nodal_values (the evaluation loop of
EXPORT_SOLUTION, src/solution_processing.f90:62-194, on the device); the
writers restate the formats of src/export_file_formats.f90 in host code:
legacy ASCII VTK (VTK_WRITE_SOLUTION :16-212), VTU mesh + solution files
(VTU_WRITE_SOLUTION :257-480), the PVD collection (PVD_SETUP :215-251) and
the EnSight Gold ASCII set (ENSIGHT_WRITE_MESH :580-686,
ENSIGHT_WRITE_BOUNDARY :688-822, ENSIGHT_WRITE_SOLUTION :824-905,
ENSIGHT_WRITE_CASE :907-988).
Like the reference, every tetrahedron gets its own four points (the field
is discontinuous across elements), cells are VTK_TETRA (10), and the cell
data carry the polyhedron index of each tetrahedron (1-based, as the
reference's elem_in_poly).
"""
from __future__ import annotations

from ctypes import c_double
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import check, ptr
from .mesh import Mesh


def nodal_values(solver, slot: int = _lib.SLOT_UN) -> np.ndarray:
    """u at the four vertices of every tetrahedron: [n_tet, 4, 3]."""
    out = np.empty((solver.mesh.n_tet, 4, 3), np.float64)
    check(solver.lib.lymph_nodal_values(solver.ctx, slot, ptr(out, c_double)), "lymph_nodal_values")
    return out


def _points(mesh: Mesh) -> np.ndarray:
    return mesh.coords[mesh.tet_vert].reshape(-1, 3)


def write_vtk(path, mesh: Mesh, u_nod: np.ndarray | None = None, name: str = "u") -> Path:
    """Legacy ASCII VTK file in the layout of VTK_WRITE_SOLUTION."""
    path = Path(path)
    n = mesh.n_tet
    pts = _points(mesh)
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 3.0\nVTKFile\nASCII\n\nDATASET UNSTRUCTURED_GRID\n")
        f.write(f"POINTS {4 * n:12d} double\n")
        np.savetxt(f, pts, fmt="%16.8f")
        f.write(f"\nCELLS {n:12d}{5 * n:12d}\n")
        conn = np.hstack([np.full((n, 1), 4), np.arange(4 * n).reshape(n, 4)])
        np.savetxt(f, conn, fmt="%12d")
        f.write(f"\nCELL_TYPES {n:12d}\n")
        f.write("10\n" * n)
        f.write("\n")
        if u_nod is not None:
            f.write(f"POINT_DATA {4 * n:12d}\nVECTORS {name:>12s} double\n")
            np.savetxt(f, np.asarray(u_nod, np.float64).reshape(-1, 3), fmt="%20.10E")
            f.write("\n")
        f.write(f"CELL_DATA {n:12d}\nSCALARS POLYHEDRA int 1\nLOOKUP_TABLE default\n")
        np.savetxt(f, mesh.tet_poly + 1, fmt="%10d")
        f.write("\n")
    return path


def write_vtu(directory, mesh: Mesh, u_nod: np.ndarray | None = None, step: int = 0, name: str = "u"):
    """mesh.vtu (points and cells) and solution_<step>.vtu (point data) in
    the layout of VTU_WRITE_SOLUTION.  Returns the paths written."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    n = mesh.n_tet
    head = ('<?xml version="1.0"?>\n'
            '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">\n  <UnstructuredGrid>\n')
    tail = "    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n"
    mp = d / "mesh.vtu"
    with open(mp, "w") as f:
        f.write(head + f'    <Piece NumberOfPoints="{4 * n}" NumberOfCells="{n}">\n')
        f.write('    <Points>\n      <DataArray type="Float64" NumberOfComponents="3" format="ascii">\n')
        np.savetxt(f, _points(mesh), fmt="%16.8f")
        f.write("      </DataArray>\n    </Points>\n    <Cells>\n")
        f.write('      <DataArray type="Int32" Name="connectivity" format="ascii">\n')
        np.savetxt(f, np.arange(4 * n).reshape(n, 4), fmt="%12d")
        f.write('      </DataArray>\n      <DataArray type="Int32" Name="offsets" format="ascii">\n')
        np.savetxt(f, 4 * np.arange(1, n + 1), fmt="%12d")
        f.write('      </DataArray>\n      <DataArray type="UInt8" Name="types" format="ascii">\n')
        f.write(f"{10:12d}\n" * n)
        f.write("      </DataArray>\n    </Cells>\n" + tail)
    out = [mp]
    if u_nod is not None:
        sp = d / f"solution_{step}.vtu"
        with open(sp, "w") as f:
            f.write(head + f'    <Piece NumberOfPoints="{4 * n}">\n    <PointData>\n')
            f.write(f'      <DataArray type="Float64" Name="{name}" NumberOfComponents="3" format="ascii">\n')
            np.savetxt(f, np.asarray(u_nod, np.float64).reshape(-1, 3), fmt="%16.8f")
            f.write("      </DataArray>\n    </PointData>\n" + tail)
        out.append(sp)
    return out


def write_pvd(directory, steps) -> Path:
    """solution.pvd: mesh.vtu as part 0, solution_<step>.vtu as part 1 for
    every saved step (PVD_SETUP)."""
    d = Path(directory)
    p = d / "solution.pvd"
    steps = list(steps)
    with open(p, "w") as f:
        f.write('<?xml version="1.0"?>\n<VTKFile type="Collection" version="0.1" byte_order="LittleEndian">\n'
                "  <Collection>\n")
        f.write(f'    <DataSet timestep="{steps[0] if steps else 0}" part="0" file="mesh.vtu"/>\n')
        for s in steps:
            f.write(f'    <DataSet timestep="{s}" part="1" file="solution_{s}.vtu"/>\n')
        f.write("  </Collection>\n</VTKFile>\n")
    return p


# ---------------------------------------------------------------------------
# EnSight Gold, ASCII (fixed-width fields: floats E12.5, integers I10)
# ---------------------------------------------------------------------------
def _e12(values) -> str:
    """One E12.5 field per line, the EnSight ASCII float format."""
    return "".join(f"{v:12.5E}\n" for v in np.asarray(values, np.float64).ravel())


def _i10(values) -> str:
    return "".join(f"{int(v):10d}\n" for v in np.asarray(values).ravel())


def write_ensight_mesh(directory, mesh: Mesh):
    """mesh.geo (one part of tetra4 cells, every tetrahedron with its own four
    nodes, numbered 1..4 n_tet) and poly.sca (the polyhedron index of each
    tetrahedron, 1-based, as a per-element scalar): ENSIGHT_WRITE_MESH.  The
    node and element ids are written and declared "given" (the reference
    lists ids under "assign", where EnSight readers expect none).  Returns
    the paths written."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    n = mesh.n_tet
    pts = _points(mesh)
    geo = d / "mesh.geo"
    with open(geo, "w") as f:
        f.write("Ensight Gold\nUnstructured mesh part\nnode id given\nelement id given\n")
        f.write(f"part\n{1:10d}\nStatic mesh file\ncoordinates\n{4 * n:10d}\n")
        f.write(_i10(np.arange(1, 4 * n + 1)))
        for k in range(3):
            f.write(_e12(pts[:, k]))
        f.write(f"tetra4\n{n:10d}\n")
        f.write(_i10(np.arange(1, n + 1)))
        conn = np.arange(1, 4 * n + 1).reshape(n, 4)
        f.write("".join("".join(f"{v:10d}" for v in row) + "\n" for row in conn))
    sca = d / "poly.sca"
    with open(sca, "w") as f:
        f.write(f"scalar per element\npart\n{1:10d}\ntetra4\n")
        f.write(_e12(mesh.tet_poly + 1))
    return [geo, sca]


def write_ensight_boundary(directory, mesh: Mesh):
    """boundaries.geo (every boundary triangle, tria3, with its own three
    nodes), boundaries_tag.sca (the triangle's boundary tag from the mesh
    file, as a per-element scalar) and boundaries.case tying them together:
    ENSIGHT_WRITE_BOUNDARY.  Returns the paths written."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    t, f_ = np.nonzero(mesh.neigh < 0)
    face_v = np.array([[0, 1, 2], [0, 1, 3], [1, 2, 3], [2, 0, 3]])  # MAKE_PARTITION_AND_MPI_FILES.f90:1087-1096
    tri = mesh.tet_vert[t[:, None], face_v[f_]]
    pts = mesh.coords[tri].reshape(-1, 3)
    nb = int(t.size)
    if mesh.face_tag is not None:
        tags = mesh.face_tag[t, f_]
    else:
        tags = -mesh.neigh[t, f_]
    geo = d / "boundaries.geo"
    with open(geo, "w") as f:
        f.write("Ensight Gold\nUnstructured mesh part\nnode id given\nelement id given\n")
        f.write(f"part\n{1:10d}\nboundary faces\ncoordinates\n{3 * nb:10d}\n")
        f.write(_i10(np.arange(1, 3 * nb + 1)))
        for k in range(3):
            f.write(_e12(pts[:, k]))
        f.write(f"tria3\n{nb:10d}\n")
        f.write(_i10(np.arange(1, nb + 1)))
        conn = np.arange(1, 3 * nb + 1).reshape(nb, 3)
        f.write("".join("".join(f"{v:10d}" for v in row) + "\n" for row in conn))
    sca = d / "boundaries_tag.sca"
    with open(sca, "w") as f:
        f.write(f"scalar per element\npart\n{1:10d}\ntria3\n")
        f.write(_e12(tags))
    case = d / "boundaries.case"
    case.write_text("FORMAT\ntype: ensight gold\nGEOMETRY\nmodel: boundaries.geo\nVARIABLE\n"
                    "scalar per element: tag boundaries_tag.sca\n")
    return [geo, sca, case]


def write_ensight_solution(directory, u_nod: np.ndarray, step: int, name: str = "u") -> Path:
    """sol_tet_<step, 6 digits>.vec: the nodal vectors of every tetrahedron's
    four nodes, x components, then y, then z (ENSIGHT_WRITE_SOLUTION)."""
    if not 0 <= step < 1000000:
        raise ValueError("step must fit the six-digit file number")
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    u = np.asarray(u_nod, np.float64).reshape(-1, 3)
    p = d / f"sol_tet_{step:06d}.vec"
    with open(p, "w") as f:
        f.write(f"vector per node\npart\n{1:10d}\ncoordinates\n")
        for k in range(3):
            f.write(_e12(u[:, k]))
    return p


def write_ensight_case(directory, dt: float, stop_time: float, increment: int, name: str = "u") -> Path:
    """solution.case: the mesh, the nodal vector u in sol_tet_******.vec
    every `increment` steps from step 0, the per-element polyhedron index,
    and the time values (ENSIGHT_WRITE_CASE: floor(stop_time / dt) /
    increment + 1 steps at times i * increment * dt)."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    nsteps = int(np.floor(stop_time / dt)) // increment + 1
    times = [i * increment * dt for i in range(nsteps)]
    lines = ["FORMAT", "type: ensight gold", "GEOMETRY", "model: mesh.geo", "VARIABLE",
             f"vector per node: {1:10d} {name} sol_tet_******.vec", f"scalar per element: {1:10d} poly poly.sca",
             "TIME", f"time set: {1:10d}", f"number of steps: {nsteps:10d}", f"filename start number: {0:10d}",
             f"filename increment: {increment:10d}", "time values:"]
    for i in range(0, nsteps, 10):
        lines.append("".join(f"{t:12.5E}" for t in times[i:i + 10]))
    p = d / "solution.case"
    p.write_text("\n".join(lines) + "\n")
    return p


def read_ensight_geo(path):
    """(node coordinates [n, 3], connectivity [n_cells, k] 1-based, cell
    type) of a one-part file written by write_ensight_mesh /
    write_ensight_boundary (for tests and tools)."""
    lines = Path(path).read_text().splitlines()
    i = lines.index("coordinates")
    nn = int(lines[i + 1])
    ids_given = lines[2].strip() == "node id given"
    o = i + 2 + (nn if ids_given else 0)
    xyz = np.array([[float(lines[o + k * nn + j][:12]) for k in range(3)] for j in range(nn)])
    j = o + 3 * nn
    ctype, nc = lines[j].strip(), int(lines[j + 1])
    o = j + 2 + (nc if lines[3].strip() == "element id given" else 0)
    w = {"tetra4": 4, "tria3": 3}[ctype]
    conn = np.array([[int(lines[o + c][10 * q:10 * q + 10]) for q in range(w)] for c in range(nc)])
    return xyz, conn, ctype


def read_ensight_values(path, ncomp: int = 1):
    """The values of a per-node vector or per-element scalar file, shape
    [n, ncomp]."""
    lines = Path(path).read_text().splitlines()
    vals = np.array([float(ln[:12]) for ln in lines[4:]])
    return vals.reshape(ncomp, -1).T


def read_vtk_point_vectors(path) -> np.ndarray:
    """The POINT_DATA vectors of a file written by write_vtk (for tests)."""
    lines = Path(path).read_text().splitlines()
    i = next(k for k, ln in enumerate(lines) if ln.startswith("POINT_DATA"))
    n = int(lines[i].split()[1])
    return np.array([[float(v) for v in ln.split()] for ln in lines[i + 2:i + 2 + n]])
