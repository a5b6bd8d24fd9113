"""The bench's multi-process path on the CPU (gloo, world size 2).

With N GPUs the bench runs N independent replicas: a barrier on both sides
of the timed region and the maximum of the per-rank times. These tests run
that harness as two gloo ranks, and the reference arm under torchrun, where
rank 0 alone works and prints and the other rank exits 0.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

_RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import bench
rank, world = bench.dist_setup(2)
bench.barrier(world)
v = bench.max_over_ranks(10.0 + 5.0 * rank, world)
bench.barrier(world)
print(json.dumps({"rank": rank, "world": world, "max": v}))
import torch.distributed as dist
dist.destroy_process_group()
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_barrier_and_max_over_two_gloo_ranks():
    port = str(_free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=port, CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK_SCRIPT, str(ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err
    lines = [json.loads(o.strip().splitlines()[-1]) for o, _ in outs]
    assert sorted(d["rank"] for d in lines) == [0, 1]
    assert all(d["world"] == 2 and d["max"] == 15.0 for d in lines)


def test_reference_arm_under_torchrun_prints_one_line():
    port = str(_free_port())
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", port, str(ROOT / "bench.py"), "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--shape", "12", "10", "8"]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["steps"] == 1 and d["warmup"] == 1


_REF_MAPS = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import bench
args = bench.argparse.Namespace(shape=(10, 8, 6), steps=3, warmup=2)
out = bench.run_reference(args, 0, 1)
maps = open("/proc/self/maps").read()
print(json.dumps({"steps": out["steps"], "warmup": out["warmup"], "sample": out["cpu_baseline"]["sample"],
                  "product_lib": "libnw_gb300" in maps, "oracle_lib": "liboracle" in maps}))
"""


def test_reference_arm_runs_the_given_steps_without_the_product_library():
    r = subprocess.run([sys.executable, "-c", _REF_MAPS, str(ROOT)], capture_output=True, text=True,
                       timeout=600, env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["steps"] == 3 and d["warmup"] == 2 and "3 runs" in d["sample"]
    assert d["oracle_lib"] and not d["product_lib"]
