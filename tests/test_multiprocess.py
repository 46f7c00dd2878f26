"""The replica path of bench.py at world size 2 on CPU (gloo): the rendezvous, the
barrier, the max over ranks that times a step, and one configuration per rank."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, ws, port, out):
    sys.path.insert(0, ROOT)
    # the ranks run on the CPU (gloo), also on a machine with fewer GPUs than ranks
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    import bench
    r, w, local, dist = bench.dist_init(None)
    assert (r, w, local) == (rank, ws, rank)
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 10.0 * (rank + 1))  # per-rank step times
    seeds = bench.replica_inputs(rank)
    import torch
    gathered = [None] * ws
    dist.all_gather_object(gathered, seeds)
    # Gribov copies: this rank's share, a made-up functional per copy, the best of the
    # share, then the best over the ranks and the summed update count
    mine = bench.split_copies([64, 32], rank, ws)
    fake_f = lambda k, c: 2.5 + 1e-3 * ((37 * c + 11 * k) % 53)  # noqa: E731
    local = [max(((fake_f(k, c), c) for c in mine[k]), key=lambda fc: (fc[0], -fc[1]))
             for k in range(2)]
    best = bench.gather_best(dist, ws, local)
    total = bench.sum_over_ranks(dist, sum(len(m) for m in mine))
    out[rank] = (t, gathered, mine, best, total)
    dist.destroy_process_group()


def test_two_replicas_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        procs = [mp.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        res = dict(out)
    fake_f = lambda k, c: 2.5 + 1e-3 * ((37 * c + 11 * k) % 53)  # noqa: E731
    want = [max(((fake_f(k, c), c) for c in range(n)), key=lambda fc: (fc[0], -fc[1]))
            for k, n in enumerate([64, 32])]
    for rank in range(2):
        t, seeds, mine, best, total = res[rank]
        assert t == 20.0  # the slowest rank's time is every rank's
        assert seeds[0] != seeds[1]  # independent configurations
        assert [tuple(b) for b in best] == want  # every rank holds the global best copy
        assert total == 96
    for k, n in enumerate([64, 32]):
        a, b = set(res[0][2][k]), set(res[1][2][k])
        assert not a & b and a | b == set(range(n))  # disjoint shares covering all copies
