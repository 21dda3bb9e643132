"""GPU parity in the late-iteration regime: the fine pass, the weighted sums
and the backprojection at the full box (current size = box), the coarse pass
at a small size, the reference sharp to Nyquist -- the shape of a refinement
near convergence (at box 256: 33,024 fine pixels per image against 1,104 in
the first iteration).  Box 64 (current size 64, coarse size 24, reference
low-passed at 4 A), HEALPix order 1, through the C ABI against the FP64
oracle, with the plain-path bounds of test_gpu_parity.py (relative diff2
<= 1e-5, normalised weights within 1e-4, volumes 1e-5 relative L2, best
pose equal), for both fine-pass forms; and the precision form's best poses
equal to the plain path's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _late_case(seed, n, precision=0):
    from relion_gb300 import datagen
    cfg = dict(datagen.CONFIGS["cfg0_box64"], current_size=64, coarse_size=24, ini_high=4.0)
    ds = datagen.Dataset(cfg, seed=seed, n_particles=n, healpix_order=1, psi_step=30.0)
    assert ds.current == 64 and ds.coarse == 24
    return ds.model(precision=precision), ds.refs, ds.particles(0, n)


@pytest.fixture(scope="module")
def cmp(oracle_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import compare
    return compare


@pytest.mark.parametrize("fine_mode", ["dense", "sparse"])
def test_late_regime_matches_oracle(cmp, fine_mode):
    m, refs, b = _late_case(21, 4)
    st = cmp.compare(m, refs, b, fine_mode=fine_mode)
    print(fine_mode, st)
    tol = cmp.TOL
    assert st["coarse_stored_all"]
    assert st["coarse_diff2_rel"] <= tol["coarse_diff2_rel"]
    assert st["fine_diff2_rel"] <= tol["fine_diff2_rel"]
    assert st["coarse_w_abs"] <= tol["weight_norm_abs"] and st["fine_w_abs"] <= tol["weight_norm_abs"]
    assert st["bp_data_rel_l2"] <= tol["bp_rel_l2"] and st["bp_weight_rel_l2"] <= tol["bp_rel_l2"]
    assert st["argmax_agree"] >= tol["argmax_agree"]
    assert st["sigma2_noise_rel"] <= 1e-5
    assert st["nr_sign_diff"] <= 1


def test_late_regime_precision_form_poses(cmp):
    m0, refs, b = _late_case(22, 6, precision=0)
    m1, _, _ = _late_case(22, 6, precision=1)
    r0 = cmp.run_gpu(m0, refs, b)[0]
    r1 = cmp.run_gpu(m1, refs, b)[0]
    for k in ("rot", "tilt", "psi", "xoff", "yoff"):
        np.testing.assert_array_equal(np.asarray(r1[k]), np.asarray(r0[k]), err_msg=k)
    np.testing.assert_allclose(r1["pmax"], r0["pmax"], rtol=1e-3)
