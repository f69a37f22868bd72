"""The N>1 path of bench.py on the CPU: world_size-2 process groups over
gloo on 127.0.0.1.

bench.py --gpus N (under torchrun) runs N independent replicas of the
workload, one per GPU, each with its own seed and no collective on the data
path; the process group only brackets the timed region with barriers and
forms the whole-job figure (units of all ranks over the slowest rank's time).
``bench.Replicas`` is that logic with the backend as a parameter, so the same
code runs here over gloo.  The reference arm under torchrun runs on rank 0
alone; the other ranks exit 0 without work.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

RANK_CODE = r"""
import json, sys, time
sys.path.insert(0, sys.argv[1])
import bench

units = {0: 1000.0, 1: 3000.0}
ms = {0: 10.0, 1: 20.0}
rep = bench.Replicas("gloo")
rep.barrier()
t0 = time.perf_counter()
value, slowest = rep.total_rate(units[rep.rank], ms[rep.rank])
rep.barrier()
wl = bench.problem("two_zone", 1000, seed=1 + rep.rank)
print(json.dumps({"rank": rep.rank, "ws": rep.ws, "value": value, "slowest_ms": slowest,
                  "seed_in_xml": "<seed>%d</seed>" % (1 + rep.rank) in wl["xml"],
                  "xml": wl["xml"]}))
rep.close()
"""


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_env(rank: int, ws: int, port: int) -> dict:
    env = dict(os.environ)
    env.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws), "MASTER_ADDR": "127.0.0.1",
                "MASTER_PORT": str(port)})
    return env


def test_replicas_two_ranks_gloo():
    port = free_port()
    procs = [subprocess.Popen([sys.executable, "-c", RANK_CODE, str(ROOT)], env=rank_env(r, 2, port),
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    outs.sort(key=lambda o: o["rank"])
    for o in outs:
        assert o["ws"] == 2
        # (1000 + 3000) units over the slower rank's 20 ms
        assert o["slowest_ms"] == 20.0
        assert o["value"] == pytest.approx(4000 / 0.020, rel=1e-12)
        assert o["seed_in_xml"]
    # independent replicas: each rank's problem differs only by its seed
    a, b = outs[0]["xml"], outs[1]["xml"]
    assert a != b and a.replace("<seed>1</seed>", "<seed>2</seed>") == b


def test_replicas_single_rank(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    rep = bench.Replicas("gloo")
    assert rep.dist is None and rep.ws == 1 and rep.rank == 0
    rep.barrier()
    assert rep.total_rate(500.0, 250.0) == (2000.0, 250.0)
    rep.close()


def test_reference_arm_on_rank_zero_only(oracle_lib):
    """torchrun with two ranks on the reference arm: one JSON line (rank 0,
    n_gpus 2), both ranks exit 0."""
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--histories", "2000", "--steps", "1", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
