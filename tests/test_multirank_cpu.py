"""The multi-rank path of bench.py (replicas, one per GPU, no data-path
collective) on CPU: two gloo ranks, the max-over-ranks timing reduction and
the per-rank seeded request streams."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import importlib.util, json, os, sys
sys.path.insert(0, os.environ["ROOT"])
spec = importlib.util.spec_from_file_location("bench", os.path.join(os.environ["ROOT"], "bench.py"))
bench = importlib.util.module_from_spec(spec)
spec.loader.exec_module(bench)
rank, ws, dist = bench.dist_init()
v = bench.max_over_ranks(float(rank + 1) * 1.5, dist)
s = bench.make_stream(5, offset=rank * 7919)
bench.barrier(dist)
print(json.dumps({"rank": rank, "ws": ws, "max": v, "first_h": float(s[0]["theta"][0])}))
dist.destroy_process_group()
'''


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks():
    port = _port()
    procs = []
    for r in range(2):
        env = dict(os.environ, ROOT=ROOT, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(__import__("json").loads(out.strip().splitlines()[-1]))
    assert [o["ws"] for o in outs] == [2, 2]
    assert all(o["max"] == 3.0 for o in outs)            # max over ranks of 1.5, 3.0
    assert outs[0]["first_h"] != outs[1]["first_h"]      # independent per-rank streams
