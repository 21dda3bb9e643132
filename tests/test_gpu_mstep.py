"""GPU reconstruction side of an iteration against the FP64 oracle, through
the C ABI: Hermitian symmetrisation, updateSSNRarrays, reconstruct (with and
without gridding iterations, with the MAP term, upsizing and downsizing
windows, 2D), computeFourierTransformMap into the device projector, FSC, and
one E-step -> M-step chain.

Tolerances: both sides compute in double precision (cuFFT double transforms
on the device, the oracle's own radix-2 / Bluestein transforms on the host):
symmetrised volumes bit-exact; shell arrays 1e-12 relative; maps 1e-9
relative L2; the device projector is stored in FP32, so it agrees to 1e-6
relative L2 (power spectrum 1e-9).  The E-step -> reconstruction chain
inherits the FP32 E-step's backprojected-volume tolerance (1e-5).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def po(oracle_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import pyoracle
    return pyoracle


def _model(name="cfg0_box64", **kw):
    from relion_gb300 import datagen
    if name == "2d":
        # the 2D classification shape at a size the oracle finishes in seconds
        c = dict(datagen.CONFIGS["cfg3_box128_2d"])
        c.update(box=64, pixel=3.0, classes=2, n_blobs=200, blob_radius=15.0, psi_step=10.0,
                 offset_range_px=3.0, max_shift=2.0, snr=0.05)
        ds = datagen.Dataset(c, seed=3, n_particles=2)
    else:
        ds = datagen.Dataset(name, seed=3, n_particles=2, healpix_order=1, psi_step=30.0)
    m = ds.model()
    m.update(kw)
    return ds, m


def _bundle(m):
    from relion_gb300.estep import MlDeviceBundle
    return MlDeviceBundle(m, device=0)


def _random_volumes(b, seed):
    xd, yd, zd, yinit, zinit, r_max = b.backprojector_dims()
    rng = np.random.default_rng(seed)
    data = rng.normal(size=(zd, yd, xd)) + 1j * rng.normal(size=(zd, yd, xd))
    weight = rng.uniform(0.2, 3.0, size=(zd, yd, xd))
    k = np.arange(zd)[:, None, None] + zinit
    i = np.arange(yd)[None, :, None] + yinit
    j = np.arange(xd)[None, None, :]
    inside = (k * k + i * i + j * j) < (2 * r_max) ** 2
    return np.where(inside, data, 0), np.where(inside, weight, 0.)


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def test_symmetrise_and_ssnr(po):
    ds, m = _model()
    b = _bundle(m)
    ori, cur = m["ori_size"], m["current_size"]
    data, weight = _random_volumes(b, 1)
    b.set_mdl_data(0, data, weight)
    b.symmetrise(0)
    gd, gw = b.get_mdl_data(0)
    od, ow = po.bp_symmetrise(data, weight, ori, cur)
    assert np.array_equal(gd, od) and np.array_equal(gw, ow)
    rng = np.random.default_rng(2)
    tau2 = rng.uniform(0.01, 1.0, ori // 2 + 1)
    tau2[5] = 0.
    fsc = rng.uniform(-0.05, 1.0, ori // 2 + 1)
    for upd, whole in ((False, False), (True, False), (True, True)):
        g = b.update_ssnr_arrays(0, 1.2, tau2, fsc, upd, whole)
        o = po.update_ssnr(ow, ori, cur, tau2, 1.2, fsc, upd, whole)
        for k in o:
            np.testing.assert_allclose(g[k], o[k], rtol=1e-12, atol=1e-300, err_msg="%s %s" % (k, upd))
    b.close()


@pytest.mark.parametrize("cur,do_map,skip,name", [
    (None, False, True, "cfg0_box64"),       # current size 28: upsizing window
    (None, True, True, "cfg0_box64"),
    (64, True, True, "cfg0_box64"),          # r_max = ori/2: downsizing window
    (None, True, False, "cfg0_box64"),       # gridding iterations
    (None, True, True, "2d"),                # 2D class
])
def test_reconstruct(po, cur, do_map, skip, name):
    kw = {} if cur is None else dict(current_size=cur, coarse_size=min(cur, 28))
    ds, m = _model(name, **kw)
    b = _bundle(m)
    ori, dim = m["ori_size"], 2 if name == "2d" else 3
    data, weight = _random_volumes(b, 7)
    b.set_mdl_data(0, data, weight)
    b.symmetrise(0)
    data, weight = b.get_mdl_data(0)
    tau2 = np.random.default_rng(8).uniform(0.05, 2.0, ori // 2 + 1)
    kw = dict(do_map=do_map, tau2=tau2, tau2_fudge=1.3, normalise=2.5, minres_map=3, skip_gridding=skip,
              max_iter_preweight=3)
    g = b.reconstruct(0, **kw)
    o = po.reconstruct(data if dim == 3 else data[0], weight if dim == 3 else weight[0], ori, m["current_size"],
                       ref_dim=dim, **kw)
    b.close()
    assert g.shape == (ori,) * dim
    assert _rel(g, o) <= 1e-9, _rel(g, o)


@pytest.mark.parametrize("cur,grid,min_ires", [(28, True, -1), (64, False, 3)])
def test_projector_from_map(po, cur, grid, min_ires):
    ds, m = _model()
    b = _bundle(m)
    ori = m["ori_size"]
    vol = np.random.default_rng(4).normal(size=(ori,) * 3)
    ps = b.set_fourier_transform_map(0, vol, cur, grid, min_ires)
    P, geom = b.get_projector(0)
    b.close()
    oP, ops = po.projector_from_map(vol, cur, grid, min_ires)
    assert P.shape == oP.shape and geom["r_max"] == min(cur // 2, ori // 2)
    assert geom["yinit"] == -(oP.shape[1] // 2) and geom["zinit"] == -(oP.shape[0] // 2)
    assert _rel(P.astype(np.complex128), oP) <= 1e-6
    np.testing.assert_allclose(ps, ops, rtol=1e-9, atol=1e-300)


def test_fsc(po):
    ds, m = _model()
    b = _bundle(m)
    rng = np.random.default_rng(9)
    a = rng.normal(size=(64,) * 3)
    c = a + rng.normal(size=a.shape)
    g = b.fsc(a, c)
    b.close()
    np.testing.assert_allclose(g, po.fsc(a, c), rtol=1e-10)


def test_estep_then_reconstruct_then_project(po):
    """E-step on the device, its volumes symmetrised and reconstructed on the
    device, the map turned back into the next iteration's projector; the
    oracle runs the same chain in double precision."""
    from relion_gb300 import datagen
    ds = datagen.Dataset("cfg0_box64", seed=13, n_particles=6, healpix_order=1, psi_step=30.0)
    m, refs, batch = ds.model(), ds.refs, ds.particles(0, 6)
    ori, cur = m["ori_size"], m["current_size"]
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    b = MlDeviceBundle(m, device=0)
    r = refs[0]
    b.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    w = MlOptimiserCuda(b)
    w.do_expectation_some_particles(batch)
    ws = b.get_wsum()
    b.symmetrise(0)
    tau2 = np.full(ori // 2 + 1, 0.5)
    s = b.update_ssnr_arrays(0, 1.0, tau2)
    vol = b.reconstruct(0, do_map=True, tau2=s["tau2"], normalise=ws["pdf_class"][0])
    ps = b.set_fourier_transform_map(0, vol, cur)
    P, _ = b.get_projector(0)
    w.close()
    b.close()
    _, _, ows, obpd, obpw = po.run(m, refs, batch)
    od, ow = po.bp_symmetrise(obpd[0], obpw[0], ori, cur)
    os_ = po.update_ssnr(ow, ori, cur, tau2, 1.0)
    ovol = po.reconstruct(od, ow, ori, cur, tau2=os_["tau2"], do_map=True, normalise=ows["pdf_class"][0])
    oP, ops = po.projector_from_map(ovol, cur)
    assert _rel(vol, ovol) <= 1e-5, _rel(vol, ovol)
    assert _rel(P.astype(np.complex128), oP) <= 1e-5
    np.testing.assert_allclose(ps, ops, rtol=1e-4)


@pytest.mark.parametrize("cur,do_map,skip,name", [
    (None, True, True, "cfg0_box64"),
    (64, True, True, "cfg0_box64"),
    (None, True, False, "cfg0_box64"),
    (None, True, True, "2d"),
])
def test_reconstruct_fp32_transforms(po, cur, do_map, skip, name):
    # FP32 cuFFT transforms (weights, sums and maps FP64): within the
    # volume tolerance of the path, 1e-5 relative L2
    kw = {} if cur is None else dict(current_size=cur, coarse_size=min(cur, 28))
    ds, m = _model(name, **kw)
    b = _bundle(m)
    b.set_recon_precision(True)
    ori, dim = m["ori_size"], 2 if name == "2d" else 3
    data, weight = _random_volumes(b, 17)
    b.set_mdl_data(0, data, weight)
    b.symmetrise(0)
    data, weight = b.get_mdl_data(0)
    tau2 = np.random.default_rng(18).uniform(0.05, 2.0, ori // 2 + 1)
    kw = dict(do_map=do_map, tau2=tau2, tau2_fudge=1.3, normalise=2.5, minres_map=3, skip_gridding=skip,
              max_iter_preweight=3)
    g = b.reconstruct(0, **kw)
    o = po.reconstruct(data if dim == 3 else data[0], weight if dim == 3 else weight[0], ori, m["current_size"],
                       ref_dim=dim, **kw)
    # the map kept on the device feeds the projector exactly like the host copy
    b.reconstruct(0, to_host=False, **kw)
    ps_dev = b.set_fourier_transform_map(0, None, m["current_size"])
    P_dev, _ = b.get_projector(0)
    ps_host = b.set_fourier_transform_map(0, g, m["current_size"])
    P_host, _ = b.get_projector(0)
    fg = b.fsc(g, o)
    b.close()
    assert _rel(g, o) <= 1e-5, _rel(g, o)
    # (the two reconstructions differ only in the order of FP64 atomic sums)
    assert _rel(P_dev.astype(np.complex128), P_host.astype(np.complex128)) <= 1e-7
    np.testing.assert_allclose(ps_dev, ps_host, rtol=1e-12)
    assert np.max(np.abs(fg[1:] - 1.)) <= 1e-6


def test_projector_from_map_fp32_transforms(po):
    ds, m = _model()
    b = _bundle(m)
    b.set_recon_precision(True)
    ori = m["ori_size"]
    vol = np.random.default_rng(5).normal(size=(ori,) * 3)
    ps = b.set_fourier_transform_map(0, vol, 28)
    P, _ = b.get_projector(0)
    b.close()
    oP, ops = po.projector_from_map(vol, 28)
    assert _rel(P.astype(np.complex128), oP) <= 1e-5
    np.testing.assert_allclose(ps, ops, rtol=1e-5)
