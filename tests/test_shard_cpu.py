"""Multi-rank path on CPU: world size 2 over gloo, cosmologies sharded with no
collective in the compute, C_l gathered on the host (the GPU compute is replaced by
the oracle so the host logic runs without a GPU)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from camb_gb300.shard import shard_range


def test_shard_ranges_cover_and_balance():
    for n in [0, 1, 5, 256, 1023]:
        for world in [1, 2, 3, 8]:
            parts = [shard_range(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
            sizes = [hi - lo for lo, hi in parts]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from camb_gb300 import _lib
    from camb_gb300.shard import get_results_sharded
    from oracle import oracle as orc
    from tests.cosmologies import draws

    def compute(ps, lmax):
        out = []
        for p in ps:
            T = _lib.Tables(p)
            icl = orc.cls(T, orc.los(T, orc.evolve_sources(T, 1), 1))
            cl = np.zeros((lmax + 1, 4))
            cl[T.ls, 0] = icl[:, 0]
            out.append(cl)
        return np.stack(out)

    ps = draws(3, seed=11, lmax=100)
    full = get_results_sharded(ps, 100, compute=compute)
    q.put((rank, full))
    dist.destroy_process_group()


def test_two_rank_gloo_gather_matches_single_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert np.array_equal(res[0], res[1])
    from camb_gb300 import _lib
    from oracle import oracle as orc
    from tests.cosmologies import draws
    for i, p in enumerate(draws(3, seed=11, lmax=100)):
        T = _lib.Tables(p)
        icl = orc.cls(T, orc.los(T, orc.evolve_sources(T, 1), 1))
        assert np.allclose(res[0][i][T.ls, 0], icl[:, 0], rtol=1e-12, atol=0)
