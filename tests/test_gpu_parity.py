"""GPU parity: the CUDA E-step (through the C ABI) against the FP64 CPU oracle.

Tolerances (plain FP32 path): relative diff2 <= 1e-5, max normalised-weight
difference <= 1e-4, backprojected-volume relative L2 <= 1e-5, best pose
(argmax) agreement, bit-exact pose bookkeeping (the fine-pass hidden
indices of both sides are compared as sets).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cmp(oracle_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import compare
    return compare


def _case(name, seed, n, **kw):
    from relion_gb300 import datagen
    ds = datagen.Dataset(name, seed=seed, n_particles=n, **kw)
    return ds.model(), ds.refs, ds.particles(0, n)


def _check(st, tol):
    print(st)
    assert st["coarse_stored_all"], "coarse computed sets differ"
    assert st["coarse_diff2_rel"] <= tol["coarse_diff2_rel"]
    assert st["coarse_w_abs"] <= tol["weight_norm_abs"]
    assert st["fine_diff2_rel"] <= tol["fine_diff2_rel"]
    assert st["fine_w_abs"] <= tol["weight_norm_abs"]
    assert st["bp_data_rel_l2"] <= tol["bp_rel_l2"]
    assert st["bp_weight_rel_l2"] <= tol["bp_rel_l2"]
    assert st["argmax_agree"] >= tol["argmax_agree"]
    assert st["sigma2_noise_rel"] <= 1e-5
    assert st["sumw_group_rel"] <= 1e-5
    assert st["pdf_direction_abs"] <= 1e-5
    assert st["dLL_abs"] <= 1e-2


@pytest.mark.parametrize("fine_mode", ["dense", "sparse"])
def test_parity_order1(cmp, fine_mode):
    m, refs, b = _case("cfg0_box64", 11, 6, healpix_order=1, psi_step=30.0)
    st = cmp.compare(m, refs, b, fine_mode=fine_mode)
    assert st["sig_mismatch"] == 0 and st["fine_set_mismatch"] == 0
    _check(st, cmp.TOL)


def test_parity_box64_config(cmp):
    # the box-64 configuration's own sampling: HEALPix order 2, psi 7.5, +/-4 px step 2
    m, refs, b = _case("cfg0_box64", 5, 2)
    st = cmp.compare(m, refs, b)
    _check(st, cmp.TOL)
    assert st["nr_sign_diff"] <= 2


def test_parity_three_classes(cmp):
    # classification shape: K=3 class volumes (15 % of the Gaussians displaced
    # per class), the class index packed in the hidden index, per-class
    # pdf_direction sums and one backprojected volume per class
    m, refs, b = _case("cfg0_box64", 23, 6, healpix_order=1, psi_step=30.0, classes=3)
    assert len(refs) == 3
    st = cmp.compare(m, refs, b)
    assert st["sig_mismatch"] == 0 and st["fine_set_mismatch"] == 0
    _check(st, cmp.TOL)


def _cfg2d(**kw):
    from relion_gb300 import datagen
    c = dict(datagen.CONFIGS["cfg3_box128_2d"])
    # the 2D classification shape at a size the oracle finishes in seconds
    c.update(box=64, pixel=3.0, classes=3, n_blobs=200, blob_radius=15.0, psi_step=10.0,
             offset_range_px=3.0, max_shift=2.0, snr=0.05)
    c.update(kw)
    return c


def test_parity_2d_classification(cmp):
    # ref_dim 2: psi-only sampling (2 oversampled psi), in-plane rotation and
    # back-rotation of padded 2D class references, per-class offset priors
    from relion_gb300 import datagen
    ds = datagen.Dataset(_cfg2d(), seed=29, n_particles=6)
    m = ds.model()
    m["prior_offset_class"] = np.array([[0.5, -0.25], [0.0, 0.0], [-1.0, 0.5]])
    st = cmp.compare(m, ds.refs, ds.particles(0, 6))
    assert st["sig_mismatch"] == 0 and st["fine_set_mismatch"] == 0
    _check(st, cmp.TOL)
    assert st["prior_offset_class_rel"] <= 1e-5
    assert st["sigma2_offset_rel"] <= 1e-5
