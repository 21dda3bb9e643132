"""CPU tests: the oracle's building blocks against the reference's own code.

The reference's CPU sources for these functions are compiled (unmodified,
where they lie) into oracle/_ref/ref_pin by oracle/build_ref.sh, over shims
for FFTW (our own FFT), TIFF and PNG.  Golden vectors of it
(tests/golden/ref_pin_golden.npz, made by tests/golden/make_ref_pin_golden.py)
pin the oracle everywhere; where the reference tree is present the tests also
run the reference live, on larger cases.

Agreement:
  * Euler_angles2matrix, HEALPix sampling (oversampled orientations and
    translations, orders 1-3), CTF::getFftwImage and
    shiftImageInFourierTransform: bit-exact;
  * Projector::project and BackProjector::backproject2Dto3D: 1e-13 relative
    at every pixel, those exactly on the r_max circle included (the oracle
    decides them with the reference's inverted matrix and double-precision
    tests, as the reference does);
  * BackProjector::reconstruct (skip-gridding with and without the MAP term,
    and the gridding iterations) and Projector::computeFourierTransformMap:
    1e-13 relative L2.
"""
import ctypes as C
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_ref_pin_golden as G  # noqa: E402

GOLD = os.path.join(HERE, "golden", "ref_pin_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def inp():
    return G.inputs()


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


def _oracle_mats(po):
    return np.array([po.euler(*a) for a in G.ANGLES])


def _oracle_sampling(po, order, psi, orng, step, pix):
    o = po.load()
    P = C.c_void_p
    psi_eff = psi if psi > 0 else 360.0 / (6 * 2 ** order)
    ndir, npsi, ntr = po.sampling_sizes(order, psi_eff, orng, step)
    rot = np.zeros((ndir, npsi, 8, 3))
    r, t, p = np.zeros(8), np.zeros(8), np.zeros(8)
    for d in range(ndir):
        for q in range(npsi):
            o.oracle_oversampled_orientations(C.c_int64(order), C.c_double(psi_eff), C.c_int64(d), C.c_int64(q),
                                              C.c_int64(1), r.ctypes.data_as(P), t.ctypes.data_as(P),
                                              p.ctypes.data_as(P))
            rot[d, q] = np.stack([r, t, p], 1)
    tr = np.zeros((ntr, 4, 2))
    x, y = np.zeros(4), np.zeros(4)
    for it in range(ntr):
        o.oracle_oversampled_translations(C.c_double(orng), C.c_double(step), C.c_int64(it), C.c_int64(1),
                                          C.c_double(pix), x.ctypes.data_as(P), y.ctypes.data_as(P))
        tr[it] = np.stack([x, y], 1)
    return rot, tr


def _oracle_ctf(po, ori, angpix, p):
    out = np.zeros((ori, ori // 2 + 1))
    xs = ori * angpix
    for i in range(ori):
        ip = i if i < ori // 2 + 1 else i - ori
        for j in range(ori // 2 + 1):
            out[i, j] = po.ctf(*p, j / xs, ip / xs)
    return out


# ---- against the committed golden vectors ------------------------------------

def test_euler_bit_exact(oracle_lib, gold):
    assert np.array_equal(_oracle_mats(oracle_lib), gold["euler"])


def test_projection_matches_reference(oracle_lib, gold, inp):
    for k, A in enumerate(gold["euler"]):
        o = oracle_lib.project(inp["ref"], G.ORI, G.PAD, G.ORI, A)
        r = gold["project"][k]
        assert np.max(np.abs(o - r)) <= 1e-13 * np.abs(r).max()


def test_backprojection_matches_reference(oracle_lib, gold, inp):
    circ = G.circle_mask(G.ORI, G.ORI // 2)
    imgs = [np.where(circ, 0, f) for f in inp["imgs"]]
    wts = [np.where(circ, 0, w) for w in inp["wts"]]
    d, w = oracle_lib.backproject(G.ORI, G.PAD, G.ORI, G.ORI, gold["euler"], imgs, wts)
    assert _rel(d, gold["bp_data"]) <= 1e-13
    assert _rel(w, gold["bp_weight"]) <= 1e-13


@pytest.mark.parametrize("tag,skip,do_map", [("skip_map", True, True), ("skip_nomap", True, False),
                                             ("grid_map", False, True)])
def test_reconstruct_matches_reference(oracle_lib, gold, inp, tag, skip, do_map):
    vol = oracle_lib.reconstruct(gold["bp_data"], gold["bp_weight"], G.ORI, G.ORI, tau2=inp["tau2"], do_map=do_map,
                                 skip_gridding=skip, max_iter_preweight=10)
    assert _rel(vol, gold["recon_" + tag]) <= 1e-13


def test_fourier_map_matches_reference(oracle_lib, gold, inp):
    data, power = oracle_lib.projector_from_map(inp["vol"], G.ORI, do_gridding=True)
    assert _rel(data, gold["fmap_data"]) <= 1e-13
    assert _rel(power, gold["fmap_power"]) <= 1e-13


def test_ctf_image_bit_exact(oracle_lib, gold):
    for k, p in enumerate(G.CTF_PARAMS):
        assert np.array_equal(_oracle_ctf(oracle_lib, G.CTF_ORI, G.CTF_ANGPIX, p), gold["ctf"][k])


def test_shift_bit_exact(oracle_lib, gold, inp):
    assert np.array_equal(oracle_lib.shift(inp["shift_img"], 64.0, 1.5, -2.25), gold["shift"])


@pytest.mark.parametrize("k", range(len(G.SAMPLING)))
def test_sampling_bit_exact(oracle_lib, gold, k):
    rot, tr = _oracle_sampling(oracle_lib, *G.SAMPLING[k])
    assert tuple(gold["sampling_%d_shape" % k]) == rot.shape + tr.shape
    assert G.digest(rot) == str(gold["sampling_%d_rot_sha256" % k])
    assert G.digest(tr) == str(gold["sampling_%d_trans_sha256" % k])


# ---- against the reference run live (reference tree present) -------------------

@pytest.fixture(scope="module")
def live(oracle_lib):
    from oracle import refpin
    if not refpin.available():
        pytest.skip("oracle/_ref/ref_pin not built (reference tree absent)")
    return refpin


def test_live_projection_and_backprojection_box24(oracle_lib, live):
    rng = np.random.default_rng(7)
    ori, pad = 24, 2
    r_max = ori // 2
    ps = 2 * (int(pad * r_max + 0.5) + 1) + 1
    ref = dict(data=rng.standard_normal((ps, ps, ps // 2 + 1)) + 1j * rng.standard_normal((ps, ps, ps // 2 + 1)),
               r_max=r_max, yinit=-(ps // 2), zinit=-(ps // 2))
    ang = rng.uniform(-180, 180, (12, 3))
    mats = live.euler(ang)
    assert np.array_equal(mats, np.array([oracle_lib.euler(*a) for a in ang]))
    rp = live.project(ref, ori, pad, ori, mats)
    for k, A in enumerate(mats):
        o = oracle_lib.project(ref, ori, pad, ori, A)
        assert np.max(np.abs(o - rp[k])) <= 1e-13 * np.abs(rp[k]).max()
    X = ori // 2 + 1
    # every pixel, those on the r_max circle included
    imgs = [rng.standard_normal((ori, X)) + 1j * rng.standard_normal((ori, X)) for _ in mats]
    wts = [rng.random((ori, X)) for _ in mats]
    rd, rw, _ = live.backproject(ori, pad, ori, ori, mats, imgs, wts)
    od, ow = oracle_lib.backproject(ori, pad, ori, ori, mats, imgs, wts)
    assert _rel(od, rd) <= 1e-13 and _rel(ow, rw) <= 1e-13


def test_live_reconstruct_and_fourier_map_box16(oracle_lib, live):
    rng = np.random.default_rng(8)
    ori, pad = 16, 2
    vol = rng.standard_normal((ori, ori, ori))
    for cur, grid, mi in ((16, True, -1), (10, False, -1), (12, True, 3)):
        rd, _, rp = live.fourier_map(ori, pad, cur, vol, do_gridding=grid, min_ires=mi)
        od, op = oracle_lib.projector_from_map(vol, cur, do_gridding=grid, min_ires=mi)
        assert _rel(od, rd) <= 1e-13 and _rel(op, rp) <= 1e-13
    ang = rng.uniform(-180, 180, (30, 3))
    mats = live.euler(ang)
    circ = G.circle_mask(ori, ori // 2)
    X = ori // 2 + 1
    imgs = [np.where(circ, 0, rng.standard_normal((ori, X)) + 1j * rng.standard_normal((ori, X))) for _ in mats]
    wts = [np.where(circ, 0, rng.random((ori, X))) for _ in mats]
    d, w = oracle_lib.backproject(ori, pad, ori, ori, mats, imgs, wts)
    d, w = oracle_lib.bp_symmetrise(d, w, ori, ori)
    tau2 = np.linspace(3.0, 0.2, ori // 2 + 1)
    for skip, dm in ((True, True), (False, True)):
        r = live.reconstruct(ori, pad, ori, d, w, tau2, skip_gridding=skip, do_map=dm)
        o = oracle_lib.reconstruct(d, w, ori, ori, tau2=tau2, do_map=dm, skip_gridding=skip)
        assert _rel(o, r) <= 1e-13


def test_live_box256_sampling_and_ctf(oracle_lib, live):
    # the box-256 workload's grid (HEALPix order 3, 48 psi, +/-6 px step 1)
    rot, tr = live.sampling(3, -1.0, 6.0, 1.0, 1.0, 1)
    orot, otr = _oracle_sampling(oracle_lib, 3, -1.0, 6.0, 1.0, 1.0)
    assert np.array_equal(rot, orot) and np.array_equal(tr, otr)
    p = [12500.0, 11800.0, 41.0, 300.0, 2.7, 0.1, 0.0, 1.0, 0.0]
    assert np.array_equal(live.ctf_images(256, 1.0, [p])[0], _oracle_ctf(oracle_lib, 256, 1.0, p))
