"""Nodal values and output files (EXPORT_SOLUTION, export_file_formats.f90).

CPU: the oracle's vertex evaluation reproduces a projected polynomial
exactly at the vertices (the basis spans it), the VTK / VTU / PVD and
EnSight Gold writers produce the reference's layout and round-trip the
values (EnSight to its E12.5 precision).  GPU: the device
evaluation equals the oracle's (<= 1e-13 relative) on the same coefficients.
"""
import numpy as np
import pytest

from lymph3d_apsc_gb300 import MatrixFree, _lib, export, mesh as M
from oracle.oracle_py import Oracle


def _mesh():
    return M.cube(2, bc="dirichlet", agglomeration="bfs", group=(4, 12), jitter=0.2, seed=3)


def test_oracle_nodal_values_of_a_projection_converge():
    """The projected manufactured field, evaluated at the vertices,
    approaches uex there as p grows."""
    m = _mesh()
    errs = []
    for p in (1, 2, 3):
        o = Oracle(m, p, 1e-3)
        o.make_matrices()
        o.modal_project(_lib.FUN_UEX, 3)  # the spatial uex into the UEX slot
        nod = o.nodal_values(3)
        X = m.coords[m.tet_vert]  # [n_tet, 4, 3]
        s_, c_ = np.sin(np.pi * X), np.cos(np.pi * X)
        # uex of problem_data_and_properties.f90:245-254
        ex = np.stack([c_[..., 0] * s_[..., 1] * s_[..., 2], s_[..., 0] * c_[..., 1] * s_[..., 2],
                       s_[..., 0] * s_[..., 1] * c_[..., 2]], axis=-1)
        errs.append(np.abs(nod - ex).max())
        o.close()
    assert errs[2] < errs[1] < errs[0]


def test_vtk_writer_layout_and_round_trip(tmp_path):
    m = _mesh()
    rng = np.random.default_rng(0)
    u = rng.standard_normal((m.n_tet, 4, 3))
    p = export.write_vtk(tmp_path / "sol.vtk", m, u, name="u")
    lines = p.read_text().splitlines()
    assert lines[0] == "# vtk DataFile Version 3.0" and lines[4] == "DATASET UNSTRUCTURED_GRID"
    assert lines[5].split() == ["POINTS", str(4 * m.n_tet), "double"]
    assert any(ln.split()[:1] == ["CELL_TYPES"] for ln in lines)
    back = export.read_vtk_point_vectors(p)
    assert np.abs(back - u.reshape(-1, 3)).max() <= 1e-9 * np.abs(u).max()
    i = next(k for k, ln in enumerate(lines) if ln.startswith("CELL_DATA"))
    polys = np.array([int(v) for v in lines[i + 3:i + 3 + m.n_tet]])
    assert np.array_equal(polys, m.tet_poly + 1)


def test_vtu_and_pvd_files(tmp_path):
    m = _mesh()
    u = np.zeros((m.n_tet, 4, 3))
    files = export.write_vtu(tmp_path, m, u, step=7)
    assert [f.name for f in files] == ["mesh.vtu", "solution_7.vtu"]
    pvd = export.write_pvd(tmp_path, [0, 7]).read_text()
    assert 'file="mesh.vtu"' in pvd and 'file="solution_7.vtu"' in pvd
    assert f'NumberOfPoints="{4 * m.n_tet}" NumberOfCells="{m.n_tet}"' in files[0].read_text()


@pytest.mark.gpu
@pytest.mark.parametrize("p", [1, 3, 4])
def test_device_nodal_values_match_oracle(require_gpu, p, tmp_path):
    m = _mesh()
    o = Oracle(m, p, 1e-3)
    o.make_matrices()
    c = np.random.default_rng(p).standard_normal((m.n_poly, 3 * o.Np))
    o.set_state(1, c)
    want = o.nodal_values(1)
    with MatrixFree(m, p, 1e-3) as g:
        g.MAKE_MATRICES_FREE()
        g.set_state(_lib.SLOT_UN, c)
        got = export.nodal_values(g, _lib.SLOT_UN)
    o.close()
    assert np.linalg.norm(got - want) <= 1e-13 * np.linalg.norm(want)
    # the device values through the EnSight solution file and back
    back = export.read_ensight_values(export.write_ensight_solution(tmp_path, got, step=p), 3)
    assert np.abs(back - got.reshape(-1, 3)).max() <= 1e-5 * np.abs(got).max()


def test_ensight_mesh_solution_case_round_trip(tmp_path):
    """EnSight Gold ASCII set (ENSIGHT_WRITE_MESH / _SOLUTION / _CASE): the
    geometry, the per-element polyhedron index and the nodal vectors read
    back to the E12.5 precision of the format; the case file names them."""
    m = _mesh()
    rng = np.random.default_rng(1)
    u = rng.standard_normal((m.n_tet, 4, 3))
    geo, sca = export.write_ensight_mesh(tmp_path, m)
    xyz, conn, ctype = export.read_ensight_geo(geo)
    assert ctype == "tetra4" and conn.shape == (m.n_tet, 4)
    pts = m.coords[m.tet_vert].reshape(-1, 3)
    assert np.abs(xyz[conn - 1].reshape(-1, 3) - pts).max() <= 1e-5
    assert np.array_equal(export.read_ensight_values(sca)[:, 0].astype(int), m.tet_poly + 1)
    vec = export.write_ensight_solution(tmp_path, u, step=40)
    assert vec.name == "sol_tet_000040.vec"
    back = export.read_ensight_values(vec, 3)
    assert np.abs(back - u.reshape(-1, 3)).max() <= 1e-5 * np.abs(u).max()
    case = export.write_ensight_case(tmp_path, dt=1e-3, stop_time=0.1, increment=20).read_text().splitlines()
    assert case[:4] == ["FORMAT", "type: ensight gold", "GEOMETRY", "model: mesh.geo"]
    assert any(ln.startswith("vector per node:") and ln.endswith("u sol_tet_******.vec") for ln in case)
    assert any(ln.startswith("number of steps:") and int(ln.split()[-1]) == 6 for ln in case)
    i = case.index("time values:")
    times = [float(ln[k:k + 12]) for ln in case[i + 1:] for k in range(0, len(ln), 12)]
    assert np.allclose(times, [0.0, 0.02, 0.04, 0.06, 0.08, 0.1])


def test_ensight_boundary_faces(tmp_path):
    """ENSIGHT_WRITE_BOUNDARY: every boundary triangle once, with its three
    vertices on the cube's surface and the deck-style face tag."""
    m = M.cube(2, bc="reference", agglomeration="hex")
    geo, sca, case = export.write_ensight_boundary(tmp_path, m)
    xyz, conn, ctype = export.read_ensight_geo(geo)
    nb = int((m.neigh < 0).sum())
    assert ctype == "tria3" and conn.shape == (nb, 3) and nb == 6 * 2 * 2 * 2
    on_surface = np.any((np.abs(xyz) < 1e-12) | (np.abs(xyz - 1) < 1e-12), axis=1)
    assert on_surface.all()
    tags = export.read_ensight_values(sca)[:, 0].astype(int)
    assert sorted(set(tags.tolist())) == [2, 3, 4, 5, 6, 7]
    assert "model: boundaries.geo" in case.read_text()
