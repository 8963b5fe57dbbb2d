"""The benchmark's replica harness on CPU: two gloo ranks (127.0.0.1) meet at
the barrier, agree on the slowest rank's time and count both ranks' steps;
`bench.py --impl reference` under two ranks prints one line from rank 0 and
nothing from rank 1."""
import os
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    from msplat_gb300 import replicas as R
    w, r, local = R.dist_env()
    R.init(w)
    R.barrier(w)
    slow = R.max_over_ranks(w, 1.0 + rank)          # rank 1 is the slower one: 2 s
    q.put((r, local, slow, R.job_rate(w, 10, slow)))
    R.finish(w)


def _free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_agree_on_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and [o[1] for o in out] == [0, 1]
    for _, _, slow, rate in out:
        assert slow == 2.0
        assert rate == 2 * 10 / 2.0     # both ranks' steps over the slowest rank's time


def test_reference_arm_rank1_exits_quietly():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
