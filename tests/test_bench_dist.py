"""The multi-rank path of bench.py on CPU ranks (gloo, world size 2): the
replicas run in lockstep (barrier), every rank takes the slowest rank's time
(max over ranks), the whole-job value counts all ranks' units, and the
reference arm runs on rank 0 only."""
import os
import socket
import types

import pytest

torch = pytest.importorskip("torch")
mp = torch.multiprocessing


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, q):
    import sys
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    r, w, _ = bench.init_dist(types.SimpleNamespace(impl="ours"))
    bench.barrier(w)
    t = bench.max_over_ranks(1.0 + r, w)          # rank 1 is the slow one
    value = 100.0 * w / t                          # units per rank x ranks / slowest time
    q.put((r, w, t, value))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[2] == 2.0 and o[3] == 100.0 for o in out)


def test_reference_arm_runs_on_rank_zero_only(capsys, monkeypatch):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    bench.main()
    assert capsys.readouterr().out == ""
