"""The multi-GPU path of bench.py is replicas only: every rank runs its own
copy of the workload with its own seeds, with no collective on the data
path; timing is a barrier plus a max over ranks and the job's particle count
a sum over ranks.  Run here as two gloo ranks on the CPU."""
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
specs = bench.rank_specs("c4", d.rank)
n = sum(s.N for s in specs)
out = {"rank": d.rank, "ws": d.ws, "max": d.max(10.0 + d.rank), "sum": d.sum(d.rank + 1),
       "n": n, "n_all": d.sum(n), "sizes": [int(s.N) for s in specs[:8]],
       "r0": float(specs[0].r[0, 0])}
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
    # rank 0 keeps the canonical workload; rank 1 has its own replicas
    sys.path.insert(0, ROOT)
    from simulationcode_gb300 import workloads as W
    canon = W.c4()
    assert a["sizes"] == [int(s.N) for s in canon[:8]]
    assert a["r0"] == float(canon[0].r[0, 0])
    assert a["sizes"] != b["sizes"] or a["r0"] != b["r0"]
