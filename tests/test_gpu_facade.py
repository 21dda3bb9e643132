"""GPU: the E-step through the compiled C++ façade (relion_gb300/acc:
MlDeviceBundle::setupFixedSizedObjects, MlOptimiserCuda::
doThreadExpectationSomeParticles per thread, storeWeightedSumsIntoModel,
AccBackprojector::getMdlData) against the same calls made from Python over
ctypes on the same raw particle images.  The façade only marshals: best pose,
offsets, class and significant-sample count are bit-identical to the ctypes
path's; PMAX, dLL, norm, the weighted sums and the backprojected volumes agree
within the library's own run-to-run spread (atomic additions in the image
preparation and in the sums: last bits, 1e-6 relative allowed; FP32 staging of
the volumes: 1e-5)."""
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

META = 25  # METADATA_LINE_LENGTH
COLS = dict(rot=0, tilt=1, psi=2, xoff=3, yoff=4, cls=6, dLL=7, pmax=8, nr_sign=9, norm=10)


def _request(path, model, ref, imgs, nthreads, optics, device=0):
    K = int(model["nr_classes"])
    head = [model["ori_size"], K, model["current_size"], model["coarse_size"], model["padding_factor"],
            model["healpix_order"], model["psi_step"], model["offset_range"], model["offset_step"],
            model["pixel_size"], model["adaptive_fraction"], model["sigma2_fudge"], model["sigma2_offset"],
            model["avg_norm_correction"], model["do_norm_correction"], model["do_scale_correction"],
            model["do_map"], model["maximum_significants"], model["adaptive_oversampling"], model["precision"],
            device, nthreads, len(imgs["images"]), optics["kV"], optics["Cs"], optics["Q0"],
            optics["particle_diameter"], optics["width_mask_edge"], float(imgs["scale"][0]), model["ref_dim"]]
    parts = [np.asarray(head, np.float64)]
    d = np.asarray(ref["data"], np.complex128)
    z, y, x = d.shape
    # the façade converts the reference to float as gbr_projector_upload expects
    parts.append(np.asarray([x, y, z, ref["yinit"], ref["zinit"], ref["r_max"], ref["pad"]], np.float64))
    parts.append(d.view(np.float64).ravel())
    ndir = len(model["pdf_direction"]) // K
    parts += [np.asarray(model["sigma2_noise"], np.float64), np.asarray(model["pdf_class"], np.float64),
              np.asarray([ndir], np.float64), np.asarray(model["pdf_direction"], np.float64)]
    for i in range(len(imgs["images"])):
        md = np.zeros(META)
        md[3:5] = imgs["old_offset"][i]
        md[10] = imgs["norm_correction"][i]
        md[11:17] = imgs["ctf"][i]
        md[20:22] = imgs["prior"][i]
        parts += [np.asarray(imgs["images"][i], np.float64).ravel(), md]
    np.concatenate(parts).tofile(path)


def _response(path, n, model, bp_shape):
    out = np.fromfile(path, np.float64)
    K, half = int(model["nr_classes"]), model["ori_size"] // 2 + 1
    ndir = len(model["pdf_direction"]) // K
    k = 0
    md = out[k:k + n * META].reshape(n, META)
    k += n * META
    ws = dict(sigma2_noise=out[k:k + half])
    k += half
    ws["pdf_class"] = out[k:k + K]
    k += K
    ws["pdf_direction"] = out[k:k + K * ndir].reshape(K, ndir)
    k += K * ndir
    for s in ("sigma2_offset", "LL", "ave_Pmax", "avg_norm_correction", "sumw_group"):
        ws[s] = out[k]
        k += 1
    vols = []
    for _ in range(K):
        x, y, z = [int(v) for v in out[k:k + 3]]
        k += 3
        nv = x * y * z
        data = out[k:k + 2 * nv].view(np.complex128).reshape(z, y, x)
        k += 2 * nv
        weight = out[k:k + nv].reshape(z, y, x)
        k += nv
        vols.append((data, weight))
    assert k == len(out)
    return md, ws, vols


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32", "bf16"])
def test_facade_matches_ctypes_path(facade_driver, tmp_path, precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from relion_gb300 import datagen
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    from relion_gb300.replicas import divide_equally
    n, nthreads = 7, 2
    ds = datagen.Dataset("cfg0_box64", seed=11, n_particles=n, healpix_order=1, psi_step=30.0)
    model = ds.model(precision=precision)
    ref = ds.ref
    imgs = ds.particle_images(0, n)
    optics = dict(kV=300.0, Cs=2.7, Q0=0.1, particle_diameter=float(ds.cfg["diameter"]), width_mask_edge=5.0)

    def ctypes_path():
        # the same calls in the same order, from Python
        b = MlDeviceBundle(model, device=0)
        b.setup_projector(0, ref["data"], ref["yinit"], ref["zinit"], ref["r_max"], ref["pad"])
        b.set_optics(**optics)
        b.reserve(4 << 30)
        workers = [MlOptimiserCuda(b) for _ in range(nthreads)]
        res = []
        for t, w in enumerate(workers):
            first, last = divide_equally(n, nthreads, t)
            part = {k: np.ascontiguousarray(v[first:last + 1]) for k, v in imgs.items() if k in (
                "images", "old_offset", "prior", "norm_correction", "scale", "ctf")}
            res.append(w.do_expectation_images(part))
        ws = b.get_wsum()
        bd, bw = b.get_mdl_data(0)
        for w in workers:
            w.close()
        b.close()
        return np.concatenate(res), ws, bd, bw

    res, ws, bd, bw = ctypes_path()

    req, resp = tmp_path / "req.bin", tmp_path / "resp.bin"
    _request(req, model, ref, imgs, nthreads, optics)
    p = subprocess.run([facade_driver, str(req), str(resp)], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    md, fws, vols = _response(resp, n, model, bd.shape)

    # the discrete results -- pose, offsets, class, significant-sample count --
    # bit for bit
    for name in ("rot", "tilt", "psi", "xoff", "yoff", "cls", "nr_sign"):
        assert np.array_equal(md[:, COLS[name]], np.asarray(res[name], np.float64)), name

    # the rest within the run-to-run spread of the library itself: the image
    # preparation's background and spectrum sums and the E-step's FP64 sums
    # over blocks are atomic additions, whose order differs between runs in
    # the last bits (two runs of the ctypes path differ the same way)
    def close(got, want, what, tol):
        got, want = np.ravel(np.asarray(got, np.float64)), np.ravel(np.asarray(want, np.float64))
        err = float(np.max(np.abs(got - want)) / max(float(np.max(np.abs(want))), 1e-300))
        assert err <= tol, (what, err)
        return err

    errs = {k: close(md[:, COLS[k]], res[k], k, 1e-6) for k in ("pmax", "dLL", "norm")}
    for k in ("sigma2_noise", "pdf_class", "pdf_direction", "sigma2_offset", "LL", "ave_Pmax", "avg_norm_correction",
              "sumw_group"):
        errs[k] = close(fws[k], ws[k], k, 1e-6)
    # the volumes are summed in FP32 staging volumes (vector atomics, in an
    # order that differs between runs) before they reach the FP64 volumes:
    # ~1e-6 of the maximum between two runs; the oracle's tolerance applies
    errs["bp_data"] = close(vols[0][0].view(np.float64), bd.view(np.float64), "bp_data", 1e-5)
    errs["bp_weight"] = close(vols[0][1], bw, "bp_weight", 1e-5)
    print("relative difference to the ctypes path:", errs)
