"""Replica (data-parallel) host logic on CPU: particle partitioning and the
all-reduce of the weighted sums over gloo ranks (world size 2, 127.0.0.1)."""
import os
import socket

import numpy as np
import pytest

from relion_gb300 import replicas


def test_divide_equally_partitions_exactly():
    for n in (0, 1, 7, 100, 20001):
        for size in (1, 2, 3, 8):
            ranges = [replicas.divide_equally(n, size, r) for r in range(size)]
            covered = []
            for first, last in ranges:
                covered.extend(range(first, last + 1))
            assert covered == list(range(n))
            counts = [last - first + 1 for first, last in ranges]
            assert max(counts) - min(counts) <= (1 if n else 0)


def test_half_sets():
    assert replicas.half_set_ranks(4, True) == [[0, 2], [1, 3]]
    assert replicas.half_set_ranks(3, False) == [[0, 1, 2]]


def _fake(rank):
    g = np.random.default_rng(100 + rank)
    wsum = dict(sigma2_noise=g.random(33), pdf_class=g.random(2), pdf_direction=g.random((2, 48)),
                sigma2_offset=float(g.random()), sumw_group=float(g.random()), LL=float(g.random()))
    vols = [((g.random((5, 5, 3)) + 1j * g.random((5, 5, 3))), g.random((5, 5, 3))) for _ in range(2)]
    return wsum, vols


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        wsum, vols = _fake(rank)
        s, v = replicas.combine_weighted_sums(wsum, vols)
        t = replicas.max_over_ranks([rank + 1.0, -rank])
        np.savez(os.path.join(out, f"r{rank}.npz"), s2=s["sigma2_noise"], pdir=s["pdf_direction"],
                 LL=s["LL"], d0=v[0][0], w1=v[1][1], t=np.array(t))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_combine_weighted_sums_gloo(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    parts = [_fake(r) for r in range(world)]
    want_s2 = sum(p[0]["sigma2_noise"] for p in parts)
    want_pdir = sum(p[0]["pdf_direction"] for p in parts)
    want_LL = sum(p[0]["LL"] for p in parts)
    want_d0 = sum(p[1][0][0] for p in parts)
    want_w1 = sum(p[1][1][1] for p in parts)
    for r in range(world):
        z = np.load(tmp_path / f"r{r}.npz")
        np.testing.assert_allclose(z["s2"], want_s2, rtol=1e-15)
        np.testing.assert_allclose(z["pdir"], want_pdir, rtol=1e-15)
        np.testing.assert_allclose(z["LL"], want_LL, rtol=1e-15)
        np.testing.assert_allclose(z["d0"], want_d0, rtol=1e-15)
        np.testing.assert_allclose(z["w1"], want_w1, rtol=1e-15)
        np.testing.assert_array_equal(z["t"], [2.0, 0.0])
