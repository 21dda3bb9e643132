"""GPU test of the coarse row skip of the tensor-core pass.

The tcgen05 epilogue records the minimum diff2 of every (particle,
orientation) row, and the coarse weight pass then reads only the rows whose
minimum lies within xs of the particle's minimum.  Every pose left out
weighs so little that all of them together stay below 1e-10 of the weight
sum (xs = ln(R T) + ln(pmax / pmin) + ln(1e10)), so the E-step results must
agree with the pass over all rows (worker option coarse_rows="full"): per-particle
results to 1e-9 relative with identical significant counts and best poses,
and the accumulated sums (sigma2 noise, backprojection), whose FP64 atomics
run in a different order on every run, to 1e-6 relative L2.  The debug copy
of the dense coarse weights must be identical too.  The coarse pass also
stores only the row segments near the running minimum (sparse diff2 writes,
with or without the debug read-back); the same bounds hold then, also when
the candidate lists overflow and the significance search reruns on the full
(partly unwritten) array (option cand_cap small), and when the block-local
candidate buffers overflow into direct appends (option cand_buf small).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(ds, model, batch, mode=None, debug=True, cand_cap=None, cand_buf=None):
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    b = MlDeviceBundle(model, device=0)
    r = ds.ref
    b.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    w = MlOptimiserCuda(b, debug=debug, coarse_rows=mode, cand_cap=cand_cap, cand_buf=cand_buf)
    res = w.do_expectation_some_particles(batch)
    cw = [w.debug_fetch(1, i) for i in range(len(res))] if debug else None
    wsum = b.get_wsum()
    data, weight = b.get_mdl_data(0)
    w.close()
    b.close()
    return res, cw, wsum, data, weight


def _rel(a, b):
    # relative L2 (complex volumes included)
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("seed", [17, 18])
def test_row_skip_matches_full_coarse_pass(seed):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    # +/-4 px in 1 px steps: 49 translations (the row skip needs T >= 32)
    ds = datagen.Dataset("cfg0_box64", seed=seed, n_particles=12, healpix_order=1, psi_step=30.0,
                         offset_range_px=4.0, offset_step_px=1.0)
    model = ds.model(precision=1)
    batch = ds.particles(0, 12)
    rf, cf, wf, df, gf = _run(ds, model, batch, mode="full")
    rn, cn, wn, dn, gn = _run(ds, model, batch)
    assert np.array_equal(rf["nr_sign"], rn["nr_sign"])
    assert np.array_equal(rf["best_ihidden_over"], rn["best_ihidden_over"])
    for k in ("coarse_sum_weight", "coarse_significant_weight", "pmax", "dLL", "fine_sum_weight"):
        np.testing.assert_allclose(rn[k], rf[k], rtol=1e-9, err_msg=k)
    for i in range(len(rf)):
        assert np.array_equal(cn[i], cf[i])
    for k in wf:
        assert _rel(wn[k], wf[k]) <= 1e-6, k
    # volumes: FP32 staging sums in atomic (run-dependent) order
    assert _rel(dn, df) <= 1e-5
    assert _rel(gn, gf) <= 1e-5


@pytest.mark.parametrize("cand_cap,cand_buf", [(None, None), (16, None), (None, 8)])
def test_sparse_writes_match_full_coarse_pass(cand_cap, cand_buf):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    ds = datagen.Dataset("cfg0_box64", seed=19, n_particles=12, healpix_order=1, psi_step=30.0,
                         offset_range_px=4.0, offset_step_px=1.0)
    model = ds.model(precision=1)
    batch = ds.particles(0, 12)
    rf, _, wf, df, gf = _run(ds, model, batch, mode="full", debug=False)
    rn, _, wn, dn, gn = _run(ds, model, batch, debug=False, cand_cap=cand_cap, cand_buf=cand_buf)
    assert np.array_equal(rf["nr_sign"], rn["nr_sign"])
    assert np.array_equal(rf["best_ihidden_over"], rn["best_ihidden_over"])
    for k in ("coarse_sum_weight", "coarse_significant_weight", "pmax", "dLL", "fine_sum_weight"):
        np.testing.assert_allclose(rn[k], rf[k], rtol=1e-9, err_msg=k)
    for k in wf:
        assert _rel(wn[k], wf[k]) <= 1e-6, k
    # volumes: FP32 staging sums in atomic (run-dependent) order
    assert _rel(dn, df) <= 1e-5
    assert _rel(gn, gf) <= 1e-5
