"""The N > 1 path of bench.py on CPU: two ranks over gloo (127.0.0.1).

One problem lives on one GPU, so N GPUs run N independent replicas (no
data-path collective): the only cross-rank operations are the barrier around
the timed region, the max of the per-rank times and the sum of the per-rank
DOF-steps.  These tests run them as two CPU processes, and run the
reference arm under torch.distributed.run, where rank 0 alone prints."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": "2",
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench
    info = bench.rank_setup(None)
    info["barrier"]()
    res = {"world": info["world"], "rank": info["rank"], "max": info["max"](1.5 + rank),
           "sum": info["sum"](10.0 * (rank + 1))}
    info["barrier"]()
    info["dist"].destroy_process_group()
    Path(out_dir, f"r{rank}.json").write_text(json.dumps(res))


def test_two_ranks_barrier_max_and_sum(tmp_path):
    mp.start_processes(_rank_main, args=(_free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r = [json.loads((tmp_path / f"r{i}.json").read_text()) for i in range(2)]
    for i, x in enumerate(r):
        assert x["world"] == 2 and x["rank"] == i
        assert x["max"] == 2.5      # the slowest rank's time
        assert x["sum"] == 30.0     # DOF-steps of both replicas


def test_reference_arm_prints_once_under_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--config", "c0", "--steps", "2", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
