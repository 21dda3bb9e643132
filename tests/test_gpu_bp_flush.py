"""GPU: the FP32 staging volumes of the backprojection are added into the
FP64 volumes once they hold GBR_OPT_BP_FLUSH particles, and before the
volumes are read, replaced or reconstructed.  Three batches with a flush
after every batch and with the flush deferred to the download give the same
volumes to the FP32 staging's run-to-run spread (1e-5, the oracle's volume
tolerance); clearing the weighted sums clears what is staged."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def _run(ds, batches, **opts):
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    b = MlDeviceBundle(ds.model(precision=1), device=0)
    b.setup_projector(0, ds.ref["data"], ds.ref["yinit"], ds.ref["zinit"], ds.ref["r_max"], ds.ref["pad"])
    w = MlOptimiserCuda(b, **opts)
    return b, w


def test_deferred_flush_equals_flush_per_batch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    ds = datagen.Dataset("cfg0_box64", seed=41, n_particles=24, healpix_order=1, psi_step=30.0)
    batches = [ds.particles(8 * i, 8) for i in range(3)]
    out = {}
    for name, flush in (("each", 0), ("deferred", 2048)):
        b, w = _run(ds, batches, bp_flush=flush)
        for bt in batches:
            w.do_expectation_some_particles(bt)
        out[name] = b.get_mdl_data(0)
        w.close()
        b.close()
    (d0, w0), (d1, w1) = out["each"], out["deferred"]
    assert np.linalg.norm(np.ravel(w0)) > 0
    # FP32 staging sums in atomic (run-dependent) order: ~1e-6 between runs
    assert _rel(d1, d0) <= 1e-5 and _rel(w1, w0) <= 1e-5


def test_reset_clears_staged_insertions():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    ds = datagen.Dataset("cfg0_box64", seed=42, n_particles=16, healpix_order=1, psi_step=30.0)
    first, second = ds.particles(0, 8), ds.particles(8, 8)
    b, w = _run(ds, None)
    w.do_expectation_some_particles(second)
    want = b.get_mdl_data(0)
    b.reset_wsum()
    w.do_expectation_some_particles(first)  # staged, not yet flushed
    b.reset_wsum()
    w.do_expectation_some_particles(second)
    got = b.get_mdl_data(0)
    assert _rel(got[0], want[0]) <= 1e-5 and _rel(got[1], want[1]) <= 1e-5
    w.close()
    b.close()


@pytest.mark.parametrize("cfg", ["cfg0_box64", "late"])
def test_direct_insertion_equals_slice_sums(cfg):
    """The sparse fine pass with each job's weighted slices inserted straight
    into the staging volumes (GBR_OPT_BP_DIRECT) against slices summed per
    orientation and then backprojected: same poses, weighted sums and
    volumes to FP32 rounding; on a first-iteration and a late-iteration
    (current size = box) shape."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    if cfg == "late":
        c = dict(datagen.CONFIGS["cfg0_box64"])
        c.update(current_size=64, coarse_size=24, ini_high=4.0)
        ds = datagen.Dataset(c, seed=45, n_particles=16, healpix_order=2, psi_step=15.0)
    else:
        ds = datagen.Dataset(cfg, seed=45, n_particles=16, healpix_order=1, psi_step=30.0)
    batches = [ds.particles(0, 8), ds.particles(8, 8)]
    out = {}
    for direct in (0, 1):
        b, w = _run(ds, batches, fine_mode="sparse", bp_direct=direct)
        res = [w.do_expectation_some_particles(bt) for bt in batches]
        out[direct] = (res, b.get_wsum(), b.get_mdl_data(0))
        w.close()
        b.close()
    (r0, ws0, (d0, w0)), (r1, ws1, (d1, w1)) = out[0], out[1]
    for a, b in zip(r1, r0):
        for k in ("rot", "tilt", "psi", "xoff", "yoff", "nr_sign"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    np.testing.assert_allclose(ws1["sigma2_noise"], ws0["sigma2_noise"], rtol=1e-6)
    assert np.linalg.norm(np.ravel(w0)) > 0
    assert _rel(d1, d0) <= 1e-5 and _rel(w1, w0) <= 1e-5
