"""GPU image preparation (getFourierTransformsAndCtfs on the device) against
the FP64 oracle, through the C ABI.

Tolerances: the device path uses FP32 images and FP32 cuFFT, the oracle
double precision throughout; Fourier images (masked and unmasked) agree to
relative L2 <= 1e-5 per particle, power spectra and high-resolution power to
1e-5 relative, CTF images to 1e-6 absolute (|CTF| <= 1), rounded offsets
exactly.  gbr_expect_images (preparation + E-step in one call) must give the
E-step results of gbr_expect_batch on the same prepared inputs (identical
best poses and significant counts, other results to 1e-6 relative).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(seed=3, n=6, norm=True):
    from relion_gb300 import datagen
    ds = datagen.Dataset("cfg0_box64", seed=seed, n_particles=n, healpix_order=1, psi_step=30.0)
    bi = ds.particle_images(0, n)
    g = np.random.default_rng(seed)
    bi["old_offset"] = g.uniform(-3.0, 3.0, size=(n, 2))
    bi["norm_correction"] = g.uniform(0.7, 1.3, size=n)
    m = ds.model()
    m["do_norm_correction"] = 1 if norm else 0
    m["avg_norm_correction"] = 0.9
    return ds, m, bi


def _bundle(ds, m):
    from relion_gb300.estep import MlDeviceBundle
    b = MlDeviceBundle(m, device=0)
    r = ds.ref
    b.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    b.set_optics(kV=300.0, Cs=2.7, Q0=0.1, particle_diameter=100.0, width_mask_edge=5.0)
    return b


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def test_prepare_images_matches_oracle(oracle_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import pyoracle
    from relion_gb300.estep import MlOptimiserCuda
    ds, m, bi = _setup()
    b = _bundle(ds, m)
    w = MlOptimiserCuda(b)
    gp = w.prepare_images(bi)
    w.close()
    b.close()
    p = dict(ori_size=m["ori_size"], current_size=m["current_size"], do_norm_correction=1,
             pixel_size=m["pixel_size"], mask_radius_px=100.0 / (2 * m["pixel_size"]), width_mask_edge=5.0,
             avg_norm_correction=0.9, kV=300.0, Cs=2.7, Q0=0.1)
    meta = dict(old_offset=bi["old_offset"], norm_correction=bi["norm_correction"],
                **{k: bi["ctf"][:, i] for i, k in enumerate(("defU", "defV", "defAngle", "Bfac", "scale",
                                                             "phase_shift"))})
    op = pyoracle.prepare_images(p, bi["images"].astype(np.float64), meta)
    assert np.array_equal(gp["old_offset"], op["old_offset"])
    for i in range(len(bi["images"])):
        assert _rel(gp["fimg"][i], op["fimg"][i]) <= 1e-5
        assert _rel(gp["fimg_nomask"][i], op["fimg_nomask"][i]) <= 1e-5
        assert _rel(gp["power_img"][i], op["power_img"][i]) <= 1e-5
    np.testing.assert_allclose(gp["highres_Xi2"], op["highres_Xi2"], rtol=1e-5)
    assert np.max(np.abs(gp["fctf"] - op["fctf"])) <= 1e-6


def test_expect_images_equals_expect_batch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300.estep import MlOptimiserCuda
    ds, m, bi = _setup(seed=5, n=8, norm=False)
    b = _bundle(ds, m)
    w = MlOptimiserCuda(b)
    gp = w.prepare_images(bi)
    batch = dict(n=8, fimg=gp["fimg"], fimg_nomask=gp["fimg_nomask"], fctf=gp["fctf"], power_img=gp["power_img"],
                 old_offset=gp["old_offset"], prior=bi["prior"], highres_Xi2=gp["highres_Xi2"],
                 norm_correction=bi["norm_correction"], scale=bi["scale"])
    r1 = w.do_expectation_some_particles(batch)
    r2 = w.do_expectation_images(bi)
    w.close()
    b.close()
    assert np.array_equal(r1["best_ihidden_over"], r2["best_ihidden_over"])
    assert np.array_equal(r1["nr_sign"], r2["nr_sign"])
    # the two calls prepare the images separately; the spectrum's FP32 partial
    # sums are added in a different order each time (highres_Xi2, hence the
    # per-particle diff2 constant and dLL, move by ~1e-8 relative)
    for k in ("pmax", "dLL", "coarse_sum_weight", "fine_sum_weight", "xoff", "yoff"):
        np.testing.assert_allclose(r2[k], r1[k], rtol=1e-6, err_msg=k)


def test_expect_images_from_star_and_mrc(tmp_path):
    # the data path of a run: MRC stack + STAR metadata on disk, native reader,
    # device image preparation and E-step; same results as the in-memory batch
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import io
    from relion_gb300.estep import MlOptimiserCuda
    ds, m, bi = _setup(seed=9, n=6, norm=False)
    n = len(bi["images"])
    pix = m["pixel_size"]
    io.write_mrc_stack(str(tmp_path / "parts.mrcs"), bi["images"], pix)
    io.write_star(str(tmp_path / "optics.star"), {"optics": {
        "rlnOpticsGroup": [1], "rlnVoltage": [300.0], "rlnSphericalAberration": [2.7],
        "rlnAmplitudeContrast": [0.1], "rlnImagePixelSize": [pix], "rlnImageSize": [m["ori_size"]]}})
    io.write_star(str(tmp_path / "parts.star"), {"particles": {
        "rlnImageName": ["%06d@parts.mrcs" % (i + 1) for i in range(n)],
        "rlnDefocusU": list(bi["ctf"][:, 0]), "rlnDefocusV": list(bi["ctf"][:, 1]),
        "rlnDefocusAngle": list(bi["ctf"][:, 2]),
        "rlnOriginXAngst": list(bi["old_offset"][:, 0] * pix), "rlnOriginYAngst": list(bi["old_offset"][:, 1] * pix),
        "rlnOpticsGroup": [1] * n}})
    star = tmp_path / "run.star"
    star.write_text((tmp_path / "optics.star").read_text() + (tmp_path / "parts.star").read_text())
    lb = io.load_particles(str(star))
    np.testing.assert_array_equal(lb["images"], bi["images"])
    b = _bundle(ds, m)
    w = MlOptimiserCuda(b)
    r_file = w.do_expectation_images(lb)
    r_mem = w.do_expectation_images(bi)
    w.close()
    b.close()
    assert np.array_equal(r_file["best_ihidden_over"], r_mem["best_ihidden_over"])
    assert np.array_equal(r_file["nr_sign"], r_mem["nr_sign"])
    np.testing.assert_allclose(r_file["pmax"], r_mem["pmax"], rtol=1e-5)


def test_staged_images_equal_direct():
    # gbr_stage_images: batches copied ahead on the copy stream (two slots,
    # reused) give the results of the direct calls
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300.estep import MlOptimiserCuda
    ds, m, _ = _setup(seed=11, n=12, norm=False)
    batches = []
    for k in range(3):
        bi = ds.particle_images(k * 4, 4)
        bi["images"] = torch.from_numpy(np.ascontiguousarray(bi["images"], np.float32)).pin_memory().numpy()
        batches.append(bi)
    b = _bundle(ds, m)
    w = MlOptimiserCuda(b)
    direct = [w.do_expectation_images(bi) for bi in batches]
    w.stage_images(batches[0])
    staged = []
    for k in range(3):
        if k + 1 < 3:
            w.stage_images(batches[k + 1])
        staged.append(w.do_expectation_images(batches[k]))
    w.close()
    b.close()
    for r1, r2 in zip(direct, staged):
        assert np.array_equal(r1["best_ihidden_over"], r2["best_ihidden_over"])
        assert np.array_equal(r1["nr_sign"], r2["nr_sign"])
        np.testing.assert_allclose(r2["pmax"], r1["pmax"], rtol=1e-6)
