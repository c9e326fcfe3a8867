"""Generates the fixtures that tie the tests to inputs the reference holds.

1. tests/golden/decks/<deck>.npz: the contents of the reference's own input
   decks src/tests/analytical/tet_{5,25,100,125} (Poly.input, test1.mate,
   cube_size*.mesh), read by lymph3d_apsc_gb300.mesh.read_deck_arrays: nodes,
   tetrahedra with material tags, tagged boundary triangles (0-based), the
   MATE table (tag, degree, rho, lambda, mu), the DIRI / NEUM tags, TIMESTEP
   and STOPTIME.  The GPU machine has no copy of the reference, so the tests read
   these files instead of the decks.
2. tests/golden/decks/deck_driver.json: the oracle's driver run
   (Lymph3D.f90:262-518: assembly, RHS, projections, first step, the
   `t <= STOPTIME` loop, L2 / DG errors) on each deck in the reference's own
   mode (one tetrahedron per polyhedron, the deck's degree, TIMESTEP and
   STOPTIME, the driver's rho = lambda = mu = 1 override).
3. tests/golden/elem_in_poly.npz: the tetrahedron -> polyhedron map
   (elem_in_poly) of the benchmark meshes: the 5^3 x 6 cube with one
   polyhedron per hexahedron (750 tetrahedra, 125 polyhedra) and the
   40^3 x 6 cube grouped by the seeded BFS agglomeration (384,000
   tetrahedra, 46,767 polyhedra), so a change of the grouping or a machine
   that groups differently is caught.
4. tests/golden/c0_driver.json: the oracle's driver run of the 125-polyhedron
   case to T = 0.1 (dt = 1e-4, p = 2, rho = lambda = mu = 1).

Run from the repository root where the reference checkout is present:
    python tests/golden/make_deck_fixtures.py [reference_root]
The reference is only read here; no test reads it.
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from lymph3d_apsc_gb300 import mesh as M  # noqa: E402
from oracle import oracle_py as O  # noqa: E402

GOLDEN = Path(__file__).resolve().parent
DECKS = ["tet_5", "tet_25", "tet_100", "tet_125"]


def main():
    ref_root = Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference")
    deck_root = ref_root / "src" / "tests" / "analytical"
    out_dir = GOLDEN / "decks"
    out_dir.mkdir(exist_ok=True)
    driver = {"generator": "tests/golden/make_deck_fixtures.py", "decks": []}
    for name in DECKS:
        a = M.read_deck_arrays(deck_root / name)
        np.savez_compressed(out_dir / f"{name}.npz", **{k: v for k, v in a.items() if k != "name"})
        mesh, prm = M.deck_mesh(a)
        o = O.Oracle(mesh, prm["degree"], prm["dt"])
        r = O.run_reference_driver(o, prm["stop_time"])
        u = o.get_state(1)
        driver["decks"].append({"deck": name, "n_tet": mesh.n_tet, "p": prm["degree"], "dt": prm["dt"],
                                "stop_time": prm["stop_time"], "n_steps": r["n_steps"], "t_final": r["t"],
                                "err_L2": r["err_L2"], "err_DG": r["err_DG"], "sum_un": float(np.sum(u)),
                                "sumsq_un": float(np.sum(u * u))})
        o.close()
        print(driver["decks"][-1])
    (out_dir / "deck_driver.json").write_text(json.dumps(driver, indent=1) + "\n")

    c0 = M.cube(5, bc="dirichlet", agglomeration="hex")
    c1 = M.cube(40, bc="dirichlet", agglomeration="bfs", seed=0, group=(4, 12))
    np.savez_compressed(GOLDEN / "elem_in_poly.npz", c0=c0.tet_poly, c1=c1.tet_poly)
    print("elem_in_poly: c0", c0.n_poly, "polyhedra; c1", c1.n_poly, "polyhedra")

    o = O.Oracle(c0, 2, 1e-4)
    r = O.run_reference_driver(o, 0.1)
    u = o.get_state(1)
    o.close()
    c0d = {"generator": "tests/golden/make_deck_fixtures.py", "n": 5, "agglomeration": "hex", "p": 2, "dt": 1e-4,
           "stop_time": 0.1, "material": [1.0, 1.0, 1.0], "n_poly": c0.n_poly, "n_steps": r["n_steps"],
           "t_final": r["t"], "err_L2": r["err_L2"], "err_DG": r["err_DG"], "sum_un": float(np.sum(u)),
           "sumsq_un": float(np.sum(u * u))}
    (GOLDEN / "c0_driver.json").write_text(json.dumps(c0d, indent=1) + "\n")
    print(c0d)


if __name__ == "__main__":
    main()
