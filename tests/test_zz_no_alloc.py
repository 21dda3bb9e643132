"""GPU test of the significance-threshold entry point that allocates nothing.

gbr_significance_threshold_noalloc exists for callers that cannot allocate
device memory where they need the significance step (code in a region that
must not allocate, a host application that only hands over device pointers,
a fixed up-front memory budget).  It keeps its working memory in one fixed
device array inside the library.  The tests call it through the C ABI: twice
in a row on different inputs, checked against the threshold and
significant-sample count that the full E-step entry point (gbr_expect_batch)
reports for the same coarse weights; and on the full 64 rows the scratch
holds, on a side stream, with ties, rows longer than one histogram chunk and
a row without a positive weight, checked against the reference's
significance rule restated in numpy.  The file is named so that pytest
collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _coarse_case():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    ds = datagen.Dataset("cfg0_box64", seed=21, n_particles=6, healpix_order=1, psi_step=30.0)
    b = MlDeviceBundle(ds.model(), device=0)
    r = ds.ref
    b.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    w = MlOptimiserCuda(b, debug=True)
    res = w.do_expectation_some_particles(ds.particles(0, 6))
    weights = np.stack([w.debug_fetch(1, i) for i in range(6)]).astype(np.float32)
    w.close()
    b.close()
    return torch, res, weights


def _call(lib, torch, weights, fraction, stream=None):
    d_w = torch.from_numpy(np.ascontiguousarray(weights)).cuda()
    n, length = d_w.shape
    thr = torch.empty(n, dtype=torch.float32, device="cuda")
    # uint32_t outputs: 4-byte device buffer, read back as uint32
    nsig = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    handle = C.c_void_p(stream.cuda_stream) if stream is not None else None
    st = lib.gbr_significance_threshold_noalloc(d_w.data_ptr(), n, length, fraction, thr.data_ptr(),
                                                nsig.data_ptr(), handle)
    torch.cuda.synchronize()
    return st, thr.cpu().numpy(), nsig.cpu().numpy().view(np.uint32).astype(np.int64)


def _reference_rule(row, fraction):
    """The significance rule of src/ml_optimiser.cpp:8120-8165 (no --maxsig):
    positive weights sorted, taken from the largest down until their FP64
    running sum exceeds fraction x the total; the weight taken last and the
    number taken.  (0, +inf) for a row without a positive weight."""
    w = np.sort(row[row > 0].astype(np.float64))[::-1]
    if len(w) == 0:
        return 0, np.inf
    total = float(np.sum(row.astype(np.float64)))
    over = np.nonzero(np.cumsum(w) > fraction * total)[0]
    k = int(over[0]) + 1 if len(over) else len(w)
    return k, np.float32(w[k - 1])


def test_noalloc_threshold_matches_expect_batch_twice():
    from relion_gb300 import _lib
    torch, res, weights = _coarse_case()
    lib = _lib.load()
    # first call: all six particles
    st, thr, nsig = _call(lib, torch, weights, 0.999)
    assert st == 0, _lib.last_error()
    np.testing.assert_allclose(thr, res["coarse_significant_weight"].astype(np.float32), rtol=1e-6)
    np.testing.assert_array_equal(nsig, res["nr_sign"].astype(np.int64))
    # second call in a row on different inputs: the particles in reverse order
    # (the scratch still holds the first call's histograms and must be reset)
    st, thr2, nsig2 = _call(lib, torch, weights[::-1].copy(), 0.999)
    assert st == 0, _lib.last_error()
    np.testing.assert_allclose(thr2, res["coarse_significant_weight"][::-1].astype(np.float32), rtol=1e-6)
    np.testing.assert_array_equal(nsig2, res["nr_sign"][::-1].astype(np.int64))


def test_noalloc_rejects_too_many_rows():
    from relion_gb300 import _lib
    pytest.importorskip("torch")
    lib = _lib.load()
    dummy = C.c_float(0.0)
    p = C.addressof(dummy)  # rejected before any device work
    st = lib.gbr_significance_threshold_noalloc(p, 65, 10, 0.999, p, p, None)
    assert st == _lib.GBR_ERR_INVALID
    assert "exceed" in _lib.last_error()


def test_noalloc_full_scratch_on_side_stream():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(5)
    n, length = 64, 20000  # three 8192-entry histogram chunks per row
    # long-tailed positive weights with many exact ties (quantised) and zeros
    w = np.exp(-rng.exponential(4.0, size=(n, length))).astype(np.float32)
    w[:, ::3] = np.round(w[:, ::3] * 64.0) / 64.0
    w[rng.random((n, length)) < 0.2] = 0.0
    w[7] = 0.0                      # no positive weight
    w[9] = 0.25                     # one run of equal values
    w[11, :] = 0.0
    w[11, 123] = 2.0                # a single positive weight
    side = torch.cuda.Stream()
    for fraction in (0.999, 0.5):
        st, thr, nsig = _call(lib, torch, w, fraction, stream=side)
        assert st == 0, _lib.last_error()
        for i in range(n):
            k, t = _reference_rule(w[i], fraction)
            assert nsig[i] == k, (i, nsig[i], k)
            assert thr[i] == t, (i, thr[i], t)
    assert nsig[7] == 0 and np.isinf(thr[7])
    assert nsig[11] == 1 and thr[11] == 2.0
