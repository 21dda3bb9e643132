"""GPU: the autotuner (relion_gb300/autotune.py) on a small precision-form
batch: every candidate runs, the chosen settings are among them, the
bundle's weighted sums are clear afterwards, and the E-step with the chosen
settings gives the default worker's best poses and significant counts
(the coarse candidates are bit-identical; the fine-pass forms agree to FP32
rounding)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_small_batch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import autotune, datagen
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    ds = datagen.Dataset("cfg0_box64", seed=31, n_particles=8, healpix_order=2, psi_step=15.0)
    m = ds.model(precision=1)
    batch = ds.particles(0, 8)
    b = MlDeviceBundle(m, device=0)
    b.setup_projector(0, ds.ref["data"], ds.ref["yinit"], ds.ref["zinit"], ds.ref["r_max"], ds.ref["pad"])
    w_ref = MlOptimiserCuda(b)
    ref = w_ref.do_expectation_some_particles(batch)
    w_ref.close()
    b.reset_wsum()
    w = MlOptimiserCuda(b)
    autotune._cache.clear()
    out = autotune.tune(b, w, batch, repeats=1)
    print(out)
    assert len(out["coarse"]) == len(autotune.COARSE_CANDIDATES)
    assert all(np.isfinite(ms) for _, ms in out["coarse"] + out["fine"])
    chosen = out["options"]
    assert {k: chosen[k] for k in ("tile_group", "pair")} in autotune.COARSE_CANDIDATES
    ws = b.get_wsum()
    assert not np.any(ws["sigma2_noise"]) and ws["LL"] == 0.0
    d, wt = b.get_mdl_data(0)
    assert not np.any(d) and not np.any(wt)
    res = w.do_expectation_some_particles(batch)
    for k in ("rot", "tilt", "psi", "xoff", "yoff", "nr_sign"):
        np.testing.assert_array_equal(res[k], ref[k], err_msg=k)
    np.testing.assert_allclose(res["pmax"], ref["pmax"], rtol=1e-5)
    w.close()
    b.close()
