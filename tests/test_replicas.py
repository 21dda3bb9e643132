"""Replica (data-parallel) host logic on CPU: particle partitioning and the
all-reduce of the weighted sums over gloo ranks (world size 2, 127.0.0.1),
with fake sums and with the E-step sums of two half batches (the oracle's
E-step on CPU) against the one-rank E-step of the whole batch."""
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


def _estep_rank(rank, world, port, out, n):
    # the E-step of this rank's particle range (the oracle, on CPU), then the
    # all-reduce of its weighted sums and volumes over the gloo ranks
    import torch.distributed as dist
    from oracle import pyoracle
    from relion_gb300 import datagen
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ds = datagen.Dataset("cfg0_box64", seed=7, n_particles=n, healpix_order=1, psi_step=30.0)
        first, last = replicas.divide_equally(n, world, rank)
        res, _, ws, bd, bw = pyoracle.run(ds.model(), [ds.ref], _part(ds.particles(0, n), first, last))
        wsum = {k: ws[k] for k in ("sigma2_noise", "pdf_class", "pdf_direction", "sigma2_offset", "sumw_group", "LL",
                                   "ave_Pmax")}
        s, v = replicas.combine_weighted_sums(wsum, [(bd[0], bw[0])])
        np.savez(os.path.join(out, f"e{rank}.npz"), s2=s["sigma2_noise"], pdir=s["pdf_direction"], LL=s["LL"],
                 so=s["sigma2_offset"], d=v[0][0], w=v[0][1], pmax=res["pmax"], first=first)
    finally:
        dist.destroy_process_group()


def _part(batch, first, last):
    n = batch["n"]
    out = {k: (v[first:last + 1] if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == n else v)
           for k, v in batch.items()}
    out["n"] = last - first + 1
    return out


def test_estep_halves_combine_to_full_batch_gloo(tmp_path, oracle_lib):
    # two ranks, each the E-step of half a batch: the summed weighted sums and
    # volumes equal the one-rank E-step of the whole batch (FP64 sums in
    # another order: 1e-12), and each rank's particles get the same results
    mp = pytest.importorskip("torch.multiprocessing")
    from relion_gb300 import datagen
    world, n = 2, 5
    mp.spawn(_estep_rank, args=(world, _free_port(), str(tmp_path), n), nprocs=world, join=True)
    ds = datagen.Dataset("cfg0_box64", seed=7, n_particles=n, healpix_order=1, psi_step=30.0)
    res, _, ws, bd, bw = oracle_lib.run(ds.model(), [ds.ref], ds.particles(0, n))
    for r in range(world):
        z = np.load(tmp_path / f"e{r}.npz")
        np.testing.assert_allclose(z["s2"], ws["sigma2_noise"], rtol=1e-12)
        np.testing.assert_allclose(z["pdir"], ws["pdf_direction"], rtol=1e-12, atol=1e-300)
        np.testing.assert_allclose(z["LL"], ws["LL"], rtol=1e-12)
        np.testing.assert_allclose(z["so"], ws["sigma2_offset"], rtol=1e-12)
        assert np.linalg.norm(z["d"] - bd[0]) <= 1e-12 * np.linalg.norm(bd[0])
        assert np.linalg.norm(z["w"] - bw[0]) <= 1e-12 * np.linalg.norm(bw[0])
        first = int(z["first"])
        np.testing.assert_allclose(z["pmax"], res["pmax"][first:first + len(z["pmax"])], rtol=1e-12)
