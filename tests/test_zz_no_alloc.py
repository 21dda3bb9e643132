"""GPU test of the significance-threshold entry point that allocates nothing.

gbr_significance_threshold_noalloc exists for callers that cannot allocate
device memory where they need the significance step (code in a region that
must not allocate, a host application that only hands over device pointers,
a fixed up-front memory budget).  It keeps its working memory in one fixed
device array inside the library.  This test calls it through the C ABI, twice
in a row on different inputs, and checks both calls against the threshold
and significant-sample count that the full E-step entry point
(gbr_expect_batch) reports for the same coarse weights.  The file is named
so that pytest collects it last.
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


def _call(lib, torch, weights, fraction):
    d_w = torch.from_numpy(np.ascontiguousarray(weights)).cuda()
    n, length = d_w.shape
    thr = torch.empty(n, dtype=torch.float32, device="cuda")
    nsig = torch.empty(n, dtype=torch.int32, device="cuda")
    st = lib.gbr_significance_threshold_noalloc(d_w.data_ptr(), n, length, fraction, thr.data_ptr(),
                                                nsig.data_ptr(), None)
    torch.cuda.synchronize()
    return st, thr.cpu().numpy(), nsig.cpu().numpy().astype(np.int64)


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
