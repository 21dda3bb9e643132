"""GPU test of the tcgen05 (BF16, FP32-accumulate) coarse cross term.

The precision form evaluates the coarse diff2 with BF16 operands on the
tensor cores; it is compared with the plain FP32 path on the same inputs
through the C ABI.  Tolerance: the coarse relative diff2 (diff2 minus the
per-particle constant) agrees to 2 % of its range on the poses the tensor-core
pass stores (BF16 has an 8-bit
significand); every significant pose of the FP32 coarse pass is also
significant in BF16 for at least 95 % of the particles' weight, and the
FP32 fine pass gives the same best pose for at least 90 % of particles.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(model, refs, batch, precision):
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    m = dict(model)
    m["precision"] = precision
    b = MlDeviceBundle(m, device=0)
    for k, ref in enumerate(refs):
        b.setup_projector(k, ref["data"], ref["yinit"], ref["zinit"], ref["r_max"], ref["pad"])
    w = MlOptimiserCuda(b, debug=True)
    res = w.do_expectation_some_particles(batch)
    d = [w.debug_fetch(0, i) for i in range(len(res))]
    cw = [w.debug_fetch(1, i) for i in range(len(res))]
    w.close()
    b.close()
    return res, d, cw


@pytest.mark.parametrize("order,psi", [(1, 30.0), (2, 7.5)])
def test_tcgen05_coarse_matches_fp32(order, psi):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    ds = datagen.Dataset("cfg0_box64", seed=31, n_particles=8, healpix_order=order, psi_step=psi)
    model, batch = ds.model(), ds.particles(0, 8)
    r32, d32, w32 = _run(model, ds.refs, batch, 0)
    r16, d16, w16 = _run(model, ds.refs, batch, 1)
    for i in range(8):
        a, b = d32[i], d16[i]
        fin = np.isfinite(a)
        assert np.array_equal(fin, np.isfinite(b))
        ra = a[fin] - a[fin].min()
        rb = b[fin] - b[fin].min()
        err = np.max(np.abs(ra - rb))
        print("particle", i, "max |d diff2| =", err, "range", np.ptp(ra))
        assert err <= 0.02 * np.ptp(ra) + 1e-3
        # significant coarse weight mass of the FP32 pass that BF16 also keeps
        s32 = w32[i] >= r32["coarse_significant_weight"][i]
        s16 = w16[i] >= r16["coarse_significant_weight"][i]
        kept = w32[i][s32 & s16].sum() / w32[i][s32].sum()
        assert kept >= 0.95
    agree = np.mean(r32["best_ihidden_over"] == r16["best_ihidden_over"])
    print("best-pose agreement", agree)
    assert agree >= 0.9


def test_tcgen05_coarse_2d_classification():
    # 2D classification shape, +/-4 px in 1 px steps (49 translations: the
    # tensor-core pass with its row minima), 3 classes x 36 psi
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    c = dict(datagen.CONFIGS["cfg3_box128_2d"])
    c.update(box=64, pixel=3.0, classes=3, n_blobs=200, blob_radius=15.0, psi_step=10.0,
             offset_range_px=4.0, max_shift=2.0, snr=0.05)
    ds = datagen.Dataset(c, seed=41, n_particles=8)
    model, batch = ds.model(), ds.particles(0, 8)
    r32, d32, w32 = _run(model, ds.refs, batch, 0)
    r16, d16, w16 = _run(model, ds.refs, batch, 1)
    for i in range(8):
        a, b = d32[i], d16[i]
        fin = np.isfinite(a)
        # the tensor-core pass stores diff2 only near the particle's running
        # minimum (sparse stores; its minimum is always stored)
        st = np.isfinite(b)
        assert np.all(fin[st])
        ra, rb = a[st] - a[fin].min(), b[st] - b[st].min()
        assert np.max(np.abs(ra - rb)) <= 0.02 * np.ptp(a[fin] - a[fin].min()) + 1e-3
    assert np.mean(r32["best_ihidden_over"] == r16["best_ihidden_over"]) >= 0.9
    assert np.mean(r16["cls"] - 1 == batch["true_class"]) >= 0.75
