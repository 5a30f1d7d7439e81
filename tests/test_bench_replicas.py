"""Multi-rank path of bench.py on CPU: N independent replicas, barrier and
max-over-ranks timing through torch.distributed with the gloo backend,
world size 2 (replicas only -- the factorization itself has no collective)."""
import os
import socket
import subprocess
import sys

from conftest import ROOT

SCRIPT = r'''
import os, sys
sys.path.insert(0, os.environ["ROOT"])
import bench
rank, ws = bench.dist_init()
assert ws == 2
bench.barrier(ws)
v = bench.allmax(float(rank + 1) * 10.0, ws)
assert v == 20.0, v
print(f"rank{rank} ok {v}")
'''


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_replica_reduction(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(SCRIPT)
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, ROOT=ROOT, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate(timeout=180)[0] for p in procs]
    for p, o in zip(procs, outs):
        assert p.returncode == 0, o
    assert any("rank0 ok 20.0" in o for o in outs)


def test_reference_arm_sample_fits_its_budget():
    """The reference arm times the CPU port on a grid sized so that its steps
    and warm-ups take about five minutes on the machine's host (one full 80^3
    step is about 23 s, the work grows like k^6): the full grid for short
    runs, a smaller one of the same family for the driver's 20 + 5."""
    import types
    sys.path.insert(0, ROOT)
    import bench
    for steps, warm, want in ((1, 0, 80), (5, 3, 80), (10, 3, 80), (20, 5, 68)):
        k = bench.reference_sample_k(types.SimpleNamespace(steps=steps, warmup=warm, k=80))
        assert k == want, (steps, warm, k)
        assert k % 4 == 0
        assert (steps + warm) * 23.0 * (k / 80.0) ** 6 <= 300.0 or k == 80
    assert bench.reference_sample_k(types.SimpleNamespace(steps=20, warmup=5, k=40)) == 40
