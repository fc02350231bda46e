"""The multi-process paths of bench.py on CPU (gloo, world size 2): the
max-over-ranks combination of the replicas' step times, and the reference
arm, which only rank 0 runs (the other ranks exit 0 without work)."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5 * rank], ws)
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [2.0, 10.0, 0.5]


def test_max_over_ranks_single_rank():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks([3.0, 1.0], 1) == [3.0, 1.0]


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3"], env=env, cwd=str(ROOT), capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_times_one_complete_solve():
    """The reference arm's steps are consecutive chunks of one complete
    solve: the K timed steps fit inside the measured solve, and the solve is
    the reference's (its iteration count for the workload)."""
    import json
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--workload", "poisson2d-64", "--steps", "4", "--warmup", "3"],
                       cwd=str(ROOT), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "s"
    assert line["ms_per_step"] * line["steps"] <= line["value"] * 1e3 * (1 + 1e-9)
    solve = line["reference_solve"]
    assert solve["status"] == "converged_rtol"
    assert len(solve["chunk_s"]) == 7
    assert abs(sum(solve["chunk_s"]) - line["value"]) <= 0.05 * line["value"] + 1e-3
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle as O
    sys.path.insert(0, str(ROOT))
    from flecsolve_gb300 import problems as P
    A, b = P.workload("poisson2d-64")
    assert solve["iters"] == O.solve("cg", A, b, maxiter=20000, rtol=1e-8).iters
    assert line["cpu_baseline"]["kind"] == ("reference" if O.ref_available() else "port")
    assert line["cpu_baseline"]["projected"] is False
    assert line["config"]["rows"] == A.nrows and line["config"]["nnz"] == A.nnz
