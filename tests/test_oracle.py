"""CPU tests: the oracle against the reference's golden vectors."""
import ctypes as C
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "healpix_ref.npz")


def test_ctf_known_answer(oracle_lib):
    g = np.load(GOLD)
    v = oracle_lib.ctf(*g["ctf_kat_args"])
    # reference tests/ctf.cpp:9 uses Catch2 Approx (relative 1.19e-5 * 100)
    assert v == pytest.approx(float(g["ctf_kat_value"][0]), rel=1.2e-3)
    assert abs(v - 0.59154) < 1e-4


@pytest.mark.parametrize("order", range(5))
def test_healpix_matches_reference_golden(oracle_lib, order):
    g = np.load(GOLD)
    o = oracle_lib.load()
    z, phi = C.c_double(), C.c_double()
    ix, iy, f = C.c_int64(), C.c_int64(), C.c_int64()
    for p in range(12 * 4 ** order):
        o.oracle_hpx_pix2ang_z_phi(C.c_int64(order), C.c_int64(p), C.byref(z), C.byref(phi))
        assert z.value == g["z_%d" % order][p] and phi.value == g["phi_%d" % order][p]  # bit-exact
        o.oracle_hpx_nest2xyf(C.c_int64(order), C.c_int64(p), C.byref(ix), C.byref(iy), C.byref(f))
        assert (ix.value, iy.value, f.value) == tuple(g["xyf_%d" % order][p])
        assert o.oracle_hpx_xyf2nest(order, ix.value, iy.value, f.value) == p


def test_healpix_matches_reference_live(oracle_lib):
    ref = oracle_lib.load_ref()
    if ref is None:
        pytest.skip("oracle/_ref not built (reference tree absent)")
    o = oracle_lib.load()
    z1, p1, z2, p2 = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    for order in (5, 6):
        for p in range(0, 12 * 4 ** order, 7):
            o.oracle_hpx_pix2ang_z_phi(C.c_int64(order), C.c_int64(p), C.byref(z1), C.byref(p1))
            ref.ref_hpx_pix2ang_z_phi(order, p, C.byref(z2), C.byref(p2))
            assert (z1.value, p1.value) == (z2.value, p2.value)


@pytest.mark.parametrize("order,psi,rng,step,expect", [
    (2, 7.5, 8.0, 4.0, (192, 48, 13)),      # box 64 configuration: +/-4 px step 2 at 2 A
    (3, -1.0, 6.0, 1.0, (768, 48, 113)),     # box 256 configuration: +/-6 px step 1 at 1 A
])
def test_sampling_sizes(oracle_lib, order, psi, rng, step, expect):
    assert tuple(oracle_lib.sampling_sizes(order, psi, rng, step)) == expect


def test_oversampled_children_are_finer_healpix(oracle_lib):
    o = oracle_lib.load()
    rot, tilt, psi = np.zeros(8), np.zeros(8), np.zeros(8)
    n = o.oracle_oversampled_orientations(C.c_int64(2), C.c_double(7.5), C.c_int64(5), C.c_int64(3),
                                          C.c_int64(1), rot.ctypes.data_as(C.c_void_p),
                                          tilt.ctypes.data_as(C.c_void_p), psi.ctypes.data_as(C.c_void_p))
    assert n == 8
    # two psi children per direction, +-psi_step/4 around the coarse psi (3 * 7.5)
    np.testing.assert_allclose(psi[:2], [22.5 - 1.875, 22.5 + 1.875])
    assert rot[0] == rot[1] and tilt[0] == tilt[1]


def test_oracle_estep_small(oracle_lib):
    from relion_gb300 import datagen
    ds = datagen.Dataset("cfg0_box64", seed=3, n_particles=2, healpix_order=1, psi_step=30.0)
    m = ds.model()
    b = ds.particles(0, 2)
    res, dbg, ws, bpd, bpw = oracle_lib.run(m, [ds.ref], b, debug=True)
    for i in range(2):
        w = dbg[i]["coarse_weight"]
        assert w.sum() == pytest.approx(res["coarse_sum_weight"][i], rel=1e-12)
        sig = dbg[i]["coarse_significant"].astype(bool)
        # significant set = weights >= threshold; its size >= NR_SIGN
        assert sig.sum() >= res["nr_sign"][i]
        fw = dbg[i]["fine_weight"]
        assert fw.sum() == pytest.approx(res["fine_sum_weight"][i], rel=1e-12)
        assert 0 < res["pmax"][i] <= 1
    # the normalised significant weights sum to (nearly) one per particle
    assert ws["sumw_group"] == pytest.approx(2.0, abs=2 * 2e-3)
    assert np.all(bpw >= 0) and bpw.sum() > 0
