"""Nodal values of the modal solution and the reference's output files.

`nodal_values` calls lymph_nodal_values (the evaluation loop of
EXPORT_SOLUTION, src/solution_processing.f90:62-194, on the device); the
writers restate the formats of src/export_file_formats.f90 in host code:
legacy ASCII VTK (VTK_WRITE_SOLUTION :16-212), VTU mesh + solution files
(VTU_WRITE_SOLUTION :257-480) and the PVD collection (PVD_SETUP :215-251).
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


def read_vtk_point_vectors(path) -> np.ndarray:
    """The POINT_DATA vectors of a file written by write_vtk (for tests)."""
    lines = Path(path).read_text().splitlines()
    i = next(k for k, ln in enumerate(lines) if ln.startswith("POINT_DATA"))
    n = int(lines[i].split()[1])
    return np.array([[float(v) for v in ln.split()] for ln in lines[i + 2:i + 2 + n]])
