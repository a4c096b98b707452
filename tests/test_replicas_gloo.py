"""bench.py's multi-GPU path is replicas only (no data-path collective): the
ranks meet at barriers around the timed region and rank 0 reports the slowest
rank's time.  Checked here with world size 2 on the gloo backend (CPU, no
GPU): dist_init, barrier and max_over_ranks, and the reference arm's rank
gating (ranks other than 0 exit without work or output)."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
sys.path.insert(0, {root!r})
import bench
ws, rank, local = bench.dist_init()
bench.barrier(ws)
m = bench.max_over_ranks(ws, 1.5 + rank)
bench.barrier(ws)
out = {{"ws": ws, "rank": rank, "max": m}}
if rank != 0:
    import argparse
    a = argparse.Namespace(n=16, nrhs=1, tol_pow=10, qchoice=16, diag=float("nan"), steps=1,
                           warmup=3, gpus=ws)
    bench.run_reference(a)  # returns at once on rank != 0
    out["reference_gated"] = True
print(json.dumps(out), flush=True)
import torch.distributed as dist
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_on_gloo():
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), H3D_BACKEND="gloo",
                   CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=180)
        assert p.returncode == 0, e[-2000:]
        outs.append(o.strip().splitlines()[-1])
    import json
    res = [json.loads(o) for o in outs]
    assert sorted(r["rank"] for r in res) == [0, 1]
    assert all(r["ws"] == 2 and r["max"] == 2.5 for r in res)
    assert any(r.get("reference_gated") for r in res)
