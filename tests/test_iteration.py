"""CPU checks of the host side of a refinement iteration
(relion_gb300.iteration): Npix_per_shell and maximizationOtherParameters
(src/ml_optimiser.cpp:5717-5730, 5090-5300) on hand-computed values."""
import numpy as np
import pytest


def test_npix_per_shell_and_model_update():
    from relion_gb300 import iteration
    n = iteration.npix_per_shell(8)
    want = np.zeros(5)
    for i in range(8):
        ip = i if i < 5 else i - 8
        for j in range(5):
            r = int(np.floor(np.sqrt(ip * ip + j * j) + 0.5))
            if r < 5 and not (j == 0 and ip < 0):
                want[r] += 1
    np.testing.assert_array_equal(n, want)
    assert n.sum() == 33
    model = dict(pdf_class=np.array([0.5, 0.5]), sigma2_noise=np.ones(5), sigma2_offset=10.,
                 avg_norm_correction=1., ref_dim=3)
    wsum = dict(pdf_class=np.array([3., 1.]), pdf_direction=np.array([1., 3., 0., 0.]),
                sigma2_offset=40., sigma2_noise=np.array([8., 4., 2., 0., 0.]), sumw_group=4.,
                avg_norm_correction=4.4, LL=-7., ave_Pmax=2.)
    iteration.maximization_other_parameters(model, wsum, np.array([1., 2., 4., 8., 8.]), True)
    np.testing.assert_allclose(model["pdf_class"], [0.75, 0.25])
    np.testing.assert_allclose(model["pdf_direction"], [0.25, 0.75, 0., 0.])
    assert model["sigma2_offset"] == 40. / (2 * 4.)
    assert model["avg_norm_correction"] == pytest.approx(1.1)
    # shells with no noise power take the previous shell's value
    np.testing.assert_allclose(model["sigma2_noise"], [1., 0.25, 1. / 16, 1. / 16, 1. / 16])
    assert model["ave_Pmax"] == 0.5
