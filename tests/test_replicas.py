"""The multi-GPU path of bench.py on CPU: replicas over gloo, world size 2.

bench.py runs one independent replica per GPU; its only collective work is a
barrier around the timed region and the max over ranks of the step time
(opencslsolver_gb300/replicas.py).  Here two processes join a gloo group and
check exactly that host logic: both see the slowest rank's time, the job rate
is world x 1000 / max ms, and the reference arm's non-root ranks exit
without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


WORKER = r"""
import json, os, sys, time
sys.path.insert(0, os.environ["OCSL_ROOT"])
from opencslsolver_gb300.replicas import ReplicaGroup
g = ReplicaGroup("gloo")
ms = 10.0 * (g.rank + 1)           # rank 1 is the slow one
g.barrier()
worst = g.max_over_ranks(ms)
rate = g.job_rate(worst)
g.barrier()
print(json.dumps({"rank": g.rank, "world": g.world, "worst": worst, "rate": rate,
                  "root": g.is_root}))
g.close()
"""


def test_two_rank_gloo_group_reports_the_slowest_rank(tmp_path):
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), OCSL_ROOT=ROOT)
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert {o["rank"] for o in outs} == {0, 1}
    for o in outs:
        assert o["world"] == 2
        assert o["worst"] == 20.0
        assert o["rate"] == pytest.approx(2 * 1000.0 / 20.0)
    assert [o["root"] for o in sorted(outs, key=lambda o: o["rank"])] == [True, False]


def test_single_process_group_needs_no_backend():
    sys.path.insert(0, ROOT)
    from opencslsolver_gb300.replicas import ReplicaGroup

    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK") if k in os.environ}
    try:
        g = ReplicaGroup("nccl")  # world 1: no process group is created
        assert g.world == 1 and g.is_root
        assert g.max_over_ranks(3.5) == 3.5
        assert g.job_rate(50.0) == pytest.approx(20.0)
        g.barrier()
        g.close()
    finally:
        os.environ.update(env)


def test_reference_arm_non_root_rank_exits_without_work():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "0"], env=env, cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


def test_reference_arm_prints_its_line():
    """Rank 0 of the reference arm times the reference algorithm (the oracle's
    OpenMP port of ILU_BICGSTAB_solve) on the host and prints one JSON line
    with the contract's keys (small box here; the default is 128^3)."""
    import json

    env = dict(os.environ, RANK="0", LOCAL_RANK="0", WORLD_SIZE="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--size", "12", "--steps", "2", "--warmup", "1"], env=env, cwd=ROOT,
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    line = json.loads(p.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 2
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["config"]["n"] == 12 ** 3
    assert "12^3" in line["cpu_baseline"]["sample"]
