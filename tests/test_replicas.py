"""The replica path of bench.py (the residual path does not shard: each rank
runs its own copy of the workload) with two gloo ranks on the CPU: rank
discovery, the barrier, the slowest rank's time, the whole-job value, and
the reference arm's non-zero ranks leaving without work."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

RANK_SCRIPT = r"""
import json, time
import bench
ws, rank, local, pg = bench.dist()
bench.barrier(pg)
# rank r "takes" (r + 1) * 10 ms per step; the job reports the slowest
slowest = bench.max_over_ranks(pg, (rank + 1) * 10.0)
value = bench.replica_value(ws, 8123007, slowest)
t0 = time.perf_counter()
ref = bench.run_reference(None, rank, pg) if rank != 0 else "skipped"
ref_s = time.perf_counter() - t0
bench.barrier(pg)
print(json.dumps({"ws": ws, "rank": rank, "local": local, "slowest_ms": slowest, "value": value,
                  "ref": ref, "ref_s": ref_s}), flush=True)
pg.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_replicas():
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), PYTHONPATH=str(ROOT))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT], cwd=ROOT, env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    outs.sort(key=lambda d: d["rank"])
    assert [d["rank"] for d in outs] == [0, 1]
    assert all(d["ws"] == 2 for d in outs)
    assert [d["local"] for d in outs] == [0, 1]
    # every rank sees the slowest rank's time, and the job's value counts
    # both replicas' edges over it
    assert all(d["slowest_ms"] == 20.0 for d in outs)
    assert all(abs(d["value"] - 2 * 8123007 / 20e-3 / 1e6) < 1e-9 for d in outs)
    # the reference arm runs on rank 0 only: rank 1 returns at once
    assert outs[1]["ref"] is None and outs[1]["ref_s"] < 1.0
