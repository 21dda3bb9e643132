"""CPU tests: the oracle's E-step against the reference's own E-step.

The reference's MlOptimiser::getAllSquaredDifferences,
convertAllSquaredDifferencesToWeights and storeWeightedSums run in
oracle/_ref/ref_estep (built from the reference's sources by
oracle/build_ref.sh) on the same prepared particles as the oracle.  Golden
vectors of its results (tests/golden/ref_estep_golden.npz, made by
tests/golden/make_ref_estep_golden.py) pin the oracle everywhere; with the
reference tree present the reference also runs live on the box-64 shape.

Agreement: per-particle results (best pose and offsets, PMAX, dLL,
significant-sample count, the coarse and fine min diff2, weight sums and
significant weights), the weighted sums (sigma2 noise, pdf_direction,
sigma2_offset, sumw_group, LL, ave_Pmax) and the backprojected volumes to
1e-12 relative (bit-identical on x86-64; the volume samples of the golden
file are float32, hence 1e-6 there).  Live, also the coarse and fine diff2,
weights and significance sets of every pose.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_ref_estep_golden as G  # noqa: E402

GOLD = os.path.join(HERE, "golden", "ref_estep_golden.npz")


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(np.asarray(a) - np.asarray(b))) / max(np.linalg.norm(np.ravel(b)), 1e-300))


@pytest.mark.parametrize("case", G.CASES, ids=[c[0] for c in G.CASES])
def test_oracle_matches_reference_estep_golden(oracle_lib, case):
    g = np.load(GOLD)
    name, _, _, n, _ = case
    ds = G.dataset(case)
    m = ds.model()
    b = ds.particles(0, n)
    res, _, ws, bd, bw = oracle_lib.run(m, [ds.ref], b)
    for k in G.PER_PARTICLE:
        want = g["%s/%s" % (name, k)]
        got = np.asarray(res[k])
        if k in ("rot", "tilt", "psi", "xoff", "yoff", "nr_sign"):
            assert np.array_equal(got, want), k
        else:
            np.testing.assert_allclose(got, want, rtol=1e-12, atol=0, err_msg=k)
    for k in ("sigma2_noise", "pdf_direction"):
        assert _rel(np.ravel(ws[k]), g["%s/wsum_%s" % (name, k)]) <= 1e-12, k
    for k in ("sigma2_offset", "sumw_group", "LL", "ave_Pmax"):
        np.testing.assert_allclose(ws[k], g["%s/wsum_%s" % (name, k)], rtol=1e-12, err_msg=k)
    idx = g["%s/bp_idx" % name]
    assert _rel(bd[0].ravel()[idx], g["%s/bp_data_sub" % name]) <= 1e-6
    assert _rel(bw[0].ravel()[idx], g["%s/bp_weight_sub" % name]) <= 1e-6
    np.testing.assert_allclose(np.linalg.norm(bd[0]), g["%s/bp_data_norm" % name], rtol=1e-12)
    np.testing.assert_allclose(np.linalg.norm(bw[0]), g["%s/bp_weight_norm" % name], rtol=1e-12)


@pytest.mark.parametrize("order,psi,n", [(1, 30.0, 4), (2, 7.5, 2)])
def test_oracle_matches_reference_estep_live(oracle_lib, order, psi, n):
    from oracle import refpin
    if not refpin.estep_available():
        pytest.skip("oracle/_ref/ref_estep not built (reference tree absent)")
    from relion_gb300 import datagen
    ds = datagen.Dataset("cfg0_box64", seed=11, n_particles=n, healpix_order=order, psi_step=psi)
    m = ds.model()
    b = ds.particles(0, n)
    parts, rws, rbd, rbw = refpin.estep(m, ds.ref, b)
    res, dbg, ws, bd, bw = oracle_lib.run(m, [ds.ref], b, debug=True)
    for i in range(n):
        r, o = parts[i], dbg[i]
        for tag in ("coarse", "fine"):
            assert np.array_equal(r[tag + "_diff2"] != -999, o[tag + "_diff2"] != -999), tag
            assert _rel(o[tag + "_diff2"], r[tag + "_diff2"]) <= 1e-12
            assert _rel(o[tag + "_weight"], r[tag + "_weight"]) <= 1e-12
        assert np.array_equal(r["coarse_significant"], o["coarse_significant"].astype(bool))
        for k in ("rot", "tilt", "psi", "xoff", "yoff", "nr_sign"):
            assert res[k][i] == r[k], k
        for k in ("pmax", "dLL", "coarse_sum_weight", "fine_sum_weight", "fine_significant_weight"):
            assert res[k][i] == pytest.approx(r[k], rel=1e-12), k
    for k in ("sigma2_noise", "pdf_direction"):
        assert _rel(np.ravel(ws[k]), rws[k]) <= 1e-12, k
    for k in ("sigma2_offset", "sumw_group", "LL", "ave_Pmax"):
        assert ws[k] == pytest.approx(rws[k], rel=1e-12), k
    assert _rel(bd[0], rbd) <= 1e-12 and _rel(bw[0], rbw) <= 1e-12
