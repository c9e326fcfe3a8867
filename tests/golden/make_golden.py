"""Generates tests/golden/oracle_driver.json: the CPU oracle's results for
small driver runs (Lymph3D.f90 sequence).  The reference itself cannot be
built or run here (Fortran + MPI, no compiler), so these values pin the
oracle against regressions and let the GPU tests compare against numbers
that do not depend on the oracle being rebuilt.  Re-run after an
intentional change of the oracle:  python tests/golden/make_golden.py
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from lymph3d_apsc_gb300 import mesh as M  # noqa: E402
from oracle import oracle_py as O  # noqa: E402

CASES = [
    dict(n=2, bc="dirichlet", agglomeration="tet", seed=0, group=[1, 1], jitter=0.0, material=[1.0, 1.0, 1.0], p=1,
         dt=1e-3, stop_time=0.05),
    dict(n=2, bc="reference", agglomeration="tet", seed=0, group=[1, 1], jitter=0.25, material=[1.0, 1.0, 1.0], p=2,
         dt=1e-3, stop_time=0.05),
    dict(n=3, bc="dirichlet", agglomeration="hex", seed=0, group=[6, 6], jitter=0.0, material=[1.0, 2.0, 1.0], p=3,
         dt=1e-3, stop_time=0.03),
    dict(n=3, bc="reference", agglomeration="bfs", seed=0, group=[4, 12], jitter=0.2, material=[1.0, 2.0, 1.0], p=2,
         dt=1e-3, stop_time=0.05),
    dict(n=2, bc="dirichlet", agglomeration="bfs", seed=3, group=[4, 16], jitter=0.1, material=[1.0, 1.0, 1.0], p=4,
         dt=5e-4, stop_time=0.01),
]


def main():
    out = {"generator": "tests/golden/make_golden.py", "cases": []}
    for c in CASES:
        m = M.cube(c["n"], bc=c["bc"], agglomeration=c["agglomeration"], seed=c["seed"], group=tuple(c["group"]),
                   jitter=c["jitter"], material=tuple(c["material"]))
        o = O.Oracle(m, c["p"], c["dt"])
        r = O.run_reference_driver(o, c["stop_time"])
        u = o.get_state(1)
        out["cases"].append({**c, "n_poly": m.n_poly, "n_steps": r["n_steps"], "t_final": r["t"],
                             "err_L2": r["err_L2"], "err_DG": r["err_DG"], "sum_un": float(np.sum(u)),
                             "sumsq_un": float(np.sum(u * u))})
        print(out["cases"][-1])
    (Path(__file__).parent / "oracle_driver.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
