"""GPU: workers of one bundle driven from two threads at once (the reference
runs one MlOptimiserCuda per thread on a shared MlDeviceBundle).  The
bundle-wide lock serialises their calls: per-particle results equal the
one-thread run's (best poses bit for bit) and the weighted sums and volumes
agree to the FP32 staging's run-to-run spread."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def test_two_threads_one_bundle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    ds = datagen.Dataset("cfg0_box64", seed=43, n_particles=32, healpix_order=1, psi_step=30.0)
    parts = [ds.particles(8 * i, 8) for i in range(4)]

    def bundle():
        b = MlDeviceBundle(ds.model(precision=1), device=0)
        b.setup_projector(0, ds.ref["data"], ds.ref["yinit"], ds.ref["zinit"], ds.ref["r_max"], ds.ref["pad"])
        return b

    b1 = bundle()
    w1 = MlOptimiserCuda(b1)
    want = [w1.do_expectation_some_particles(p) for p in parts]
    ws1, vol1 = b1.get_wsum(), b1.get_mdl_data(0)
    w1.close()
    b1.close()

    b2 = bundle()
    workers = [MlOptimiserCuda(b2) for _ in range(2)]
    got = [None] * len(parts)
    errors = []

    def run(t):
        try:
            for i in range(t, len(parts), 2):
                got[i] = workers[t].do_expectation_some_particles(parts[i])
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(t,)) for t in range(2)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    ws2, vol2 = b2.get_wsum(), b2.get_mdl_data(0)
    for w in workers:
        w.close()
    b2.close()
    for a, b in zip(got, want):
        for k in ("rot", "tilt", "psi", "xoff", "yoff", "nr_sign"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
        np.testing.assert_allclose(a["pmax"], b["pmax"], rtol=1e-6)
    for k in ("sigma2_noise", "pdf_direction"):
        np.testing.assert_allclose(ws2[k], ws1[k], rtol=1e-6, atol=1e-300)
    assert _rel(vol2[0], vol1[0]) <= 1e-5 and _rel(vol2[1], vol1[1]) <= 1e-5
