"""GPU test of the replica path: two ranks (processes) on one GPU, each the
CUDA E-step of its half of a batch in its own bundle, then the one exchange
step, combine_weighted_sums (an all-reduce over gloo ranks on host buffers,
MlOptimiserMpi::combineAllWeightedSums), against the one-rank E-step of the
whole batch: PMAX to 1e-9 relative, the significant-sample counts within 1,
the summed weighted sums to 1e-6 and volumes to 1e-5 (FP32 staging sums in
atomic order).  The runs may differ by a pose
at the significance boundary (and so pick another of two nearly equal best
poses): the FP64 weight sums that set the threshold are formed by atomics in
another order.  The two ranks'
kernels never wait on each other; the only coordination is the host-side
collective after both E-steps are complete.
"""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("sigma2_noise", "pdf_class", "pdf_direction", "sigma2_offset", "sumw_group", "LL", "ave_Pmax")


def _estep(batch_range, n, precision):
    from relion_gb300 import datagen
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    ds = datagen.Dataset("cfg0_box64", seed=9, n_particles=n, healpix_order=1, psi_step=30.0)
    batch = ds.particles(0, n)
    first, last = batch_range
    part = {k: (v[first:last + 1] if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == n else v)
            for k, v in batch.items()}
    part["n"] = last - first + 1
    b = MlDeviceBundle(ds.model(precision=precision), device=0)
    r = ds.ref
    b.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    # the same fine-pass kernels for any batch (the automatic choice depends
    # on the batch's significant density)
    w = MlOptimiserCuda(b, fine_mode="sparse")
    res = w.do_expectation_some_particles(part)
    ws = b.get_wsum()
    vol = b.get_mdl_data(0)
    w.close()
    b.close()
    return res, {k: ws[k] for k in KEYS}, vol


def _rank(rank, world, port, out, n):
    import torch.distributed as dist
    from relion_gb300 import replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        first, last = replicas.divide_equally(n, world, rank)
        res, ws, vol = _estep((first, last), n, 0)
        s, v = replicas.combine_weighted_sums(ws, [vol])
        np.savez(os.path.join(out, f"g{rank}.npz"), first=first, pmax=res["pmax"], best=res["best_ihidden_over"],
                 nsig=res["nr_sign"],
                 d=v[0][0], w=v[0][1], **{"ws_" + k: np.asarray(s[k]) for k in KEYS})
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_on_halves_equal_one_rank(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import torch.multiprocessing as mp
    world, n = 2, 9
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path), n), nprocs=world, join=True)
    res, ws, (bd, bw) = _estep((0, n - 1), n, 0)
    for r in range(world):
        z = np.load(tmp_path / f"g{r}.npz")
        first, m = int(z["first"]), len(z["pmax"])
        np.testing.assert_allclose(z["pmax"], res["pmax"][first:first + m], rtol=1e-9)
        assert np.max(np.abs(z["nsig"] - res["nr_sign"][first:first + m])) <= 1
        print("rank", r, "best poses equal:", int(np.sum(z["best"] == res["best_ihidden_over"][first:first + m])), "/", m)
        for k in KEYS:
            a, b = np.ravel(z["ws_" + k]), np.ravel(np.asarray(ws[k]))
            assert np.linalg.norm(a - b) <= 1e-6 * max(np.linalg.norm(b), 1e-300), k
        assert np.linalg.norm(z["d"] - bd) <= 1e-5 * np.linalg.norm(bd)
        assert np.linalg.norm(z["w"] - bw) <= 1e-5 * np.linalg.norm(bw)
