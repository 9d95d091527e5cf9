"""The multi-GPU path of bench.py shards independent replicas: the replica
batch is one job of 512 replicas per rank, partitioned over the ranks by
LPT on particles x steps, with no collective on the data path; timing is a
barrier plus a max over ranks and the job's particle count a sum over ranks.
Run here as two gloo ranks on the CPU: the union of the ranks' replicas is
exactly the job, with no replica on two ranks, and the ranks' particle
counts are balanced."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
sys.path.insert(0, %r)
import numpy as np
import bench
d = bench.Dist()
d.barrier()
specs = bench.rank_specs("c4", d.rank, world=d.ws)
n = sum(s.N for s in specs)
out = {"rank": d.rank, "ws": d.ws, "max": d.max(10.0 + d.rank), "sum": d.sum(d.rank + 1),
       "n": n, "n_all": d.sum(n), "seeds": [int(s.seed) for s in specs],
       "sizes": [int(s.N) for s in specs], "r0": [float(s.r[0, 0]) for s in specs]}
d.barrier()
d.close()
print(json.dumps(out))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_run_independent_replica_sets():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD % ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=300)
        assert p.returncode == 0, e[-2000:]
        outs.append(json.loads(o.strip().splitlines()[-1]))
    a, b = sorted(outs, key=lambda x: x["rank"])
    assert a["ws"] == b["ws"] == 2
    assert a["max"] == b["max"] == 11.0
    assert a["sum"] == b["sum"] == 3.0
    assert a["n_all"] == b["n_all"] == a["n"] + b["n"]
    # one job of 1024 replicas: each replica on exactly one rank, identical
    # to the same replica of the whole job, particle counts balanced
    sys.path.insert(0, ROOT)
    from simulationcode_gb300 import workloads as W
    job = W.c4(nrep=1024)
    seeds = a["seeds"] + b["seeds"]
    assert sorted(seeds) == sorted(int(s.seed) for s in job) and len(set(seeds)) == 1024
    by_seed = {int(s.seed): s for s in job}
    for o in (a, b):
        for sd, n, r0 in zip(o["seeds"], o["sizes"], o["r0"]):
            assert by_seed[sd].N == n and float(by_seed[sd].r[0, 0]) == r0
    assert abs(a["n"] - b["n"]) <= max(s.N for s in job)
    assert abs(a["n"] - b["n"]) / (a["n"] + b["n"]) < 0.01


def test_lpt_partition_host_logic():
    sys.path.insert(0, ROOT)
    from simulationcode_gb300 import workloads as W
    work = [int(n) for n in W.c4_sizes(512 * 8)]
    for g in (1, 2, 3, 8):
        parts = W.lpt_partition(work, g)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(work)))
        loads = [sum(work[k] for k in p) for p in parts]
        # LPT bound: max load <= mean + the largest job
        assert max(loads) <= sum(loads) / g + max(work)
    assert W.lpt_partition(work[:512], 1)[0] == list(range(512))
    assert [s.seed for s in W.c4(nrep=1024, indices=[3, 700])] == [s.seed for s in W.c4(nrep=1024)[3:701:697]]
