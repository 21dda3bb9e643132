"""ctypes binding of the oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/liboracle.so (the CPU double-precision restatement of
the reference's E-step) and, if built, oracle/_ref/libref_healpix.so (the
reference's own HEALPix code).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs import this module.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
I64, F64, P = C.c_int64, C.c_double, C.c_void_p


class OracleModel(C.Structure):
    _fields_ = [(n, I64) for n in (
        "ori_size", "nr_classes", "current_size", "coarse_size", "padding_factor",
        "proj_r_max", "proj_xdim", "proj_ydim", "proj_zdim", "proj_yinit", "proj_zinit",
        "bp_r_max", "bp_xdim", "bp_ydim", "bp_zdim", "bp_yinit", "bp_zinit",
        "healpix_order", "adaptive_oversampling", "maximum_significants", "sigma2_len",
        "do_scale_correction", "do_norm_correction", "do_map", "ref_dim")] + \
        [(n, F64) for n in ("pixel_size", "psi_step", "offset_range", "offset_step",
                            "adaptive_fraction", "sigma2_fudge", "sigma2_offset",
                            "avg_norm_correction")] + \
        [(n, P) for n in ("ppref", "sigma2_noise", "pdf_class", "pdf_direction", "data_vs_prior",
                          "prior_offset_class")]


class OracleParticle(C.Structure):
    _fields_ = [(n, P) for n in ("fimg", "fimg_nomask", "fctf", "power_img")] + \
        [("old_offset", F64 * 2), ("prior", F64 * 2)] + \
        [(n, F64) for n in ("highres_Xi2", "norm_correction", "scale", "pad_")]


class OracleResult(C.Structure):
    _fields_ = [(n, F64) for n in (
        "rot", "tilt", "psi", "xoff", "yoff", "cls", "pmax", "dLL", "norm", "nr_sign",
        "coarse_min_diff2", "coarse_sum_weight", "coarse_significant_weight",
        "fine_min_diff2", "fine_sum_weight", "fine_significant_weight")] + \
        [("best_ihidden_over", I64), ("pad_", I64)]


class OracleDebug(C.Structure):
    _fields_ = [(n, P) for n in ("coarse_diff2", "coarse_weight", "coarse_significant",
                                 "fine_diff2", "fine_weight")]


class OracleWsum(C.Structure):
    _fields_ = [(n, P) for n in ("sigma2_noise", "pdf_class", "pdf_direction", "bp_data",
                                 "bp_weight")] + \
        [(n, F64) for n in ("sigma2_offset", "sumw_group", "LL", "ave_Pmax",
                            "avg_norm_correction", "wsum_signal_product",
                            "wsum_reference_power", "pad_")] + \
        [("prior_offset_class", P)]


_O = None
_R = None


def load():
    global _O
    if _O is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            raise RuntimeError("oracle not built: %s (run oracle/build.py)" % path)
        lib = C.CDLL(path)
        lib.oracle_expectation.restype = C.c_int
        lib.oracle_project.restype = None
        lib.oracle_backproject.restype = None
        lib.oracle_shift_ft.restype = None
        lib.oracle_euler.restype = None
        lib.oracle_set_threads.restype = C.c_int
        lib.oracle_set_threads.argtypes = [C.c_int]
        lib.oracle_prepare_images.restype = C.c_int
        lib.oracle_prepare_images.argtypes = [P, I64, P, P, P, P, P, P, P, P]
        lib.oracle_ctf.restype = F64
        lib.oracle_ctf.argtypes = [F64] * 11
        lib.oracle_hpx_xyf2nest.restype = I64
        lib.oracle_hpx_xyf2nest.argtypes = [I64] * 4
        lib.oracle_oversampled_orientations.restype = C.c_int
        lib.oracle_translations.restype = C.c_int
        lib.oracle_oversampled_translations.restype = C.c_int
        for f in ("oracle_bp_symmetrise", "oracle_update_ssnr", "oracle_reconstruct",
                  "oracle_projector_from_map", "oracle_fsc"):
            getattr(lib, f).restype = C.c_int
        lib.oracle_bp_symmetrise.argtypes = [P, P, P]
        lib.oracle_update_ssnr.argtypes = [P, P, F64, P, P, P, P, P, I64, I64]
        lib.oracle_reconstruct.argtypes = [P, P, P, P, P, P]
        lib.oracle_projector_from_map.argtypes = [I64, I64, I64, P, I64, I64, I64, P, P]
        lib.oracle_fsc.argtypes = [I64, I64, P, P, P]
        _O = lib
    return _O


def set_threads(n):
    """Host threads of the oracle's OpenMP loops (0: leave unchanged); returns
    the number in effect.  Works after another library (torch) has started
    the OpenMP runtime, where OMP_NUM_THREADS is no longer read."""
    return int(load().oracle_set_threads(int(n)))


def load_ref():
    """The reference's own Healpix_Base (None if oracle/_ref was not built)."""
    global _R
    if _R is None:
        path = os.path.join(HERE, "_ref", "libref_healpix.so")
        if not os.path.exists(path):
            return None
        lib = C.CDLL(path)
        lib.ref_hpx_xyf2nest.restype = C.c_int
        _R = lib
    return _R


def sampling_sizes(order, psi_step, offset_range, offset_step, ref_dim=3):
    """(ndir, npsi, ntrans); 2D (ref_dim 2): one direction, psi step 10 by default."""
    o = load()
    v = [I64() for _ in range(3)]
    if ref_dim == 2 and psi_step <= 0:
        psi_step = 10.0
    o.oracle_sampling_sizes(I64(order), F64(psi_step), F64(offset_range), F64(offset_step),
                            *[C.byref(x) for x in v])
    if ref_dim == 2:
        v[0].value = 1
    return [x.value for x in v]


def ctf(defU, defV, defAng, kV, Cs, Q0, Bfac, scale, phase_shift, X, Y):
    return load().oracle_ctf(defU, defV, defAng, kV, Cs, Q0, Bfac, scale, phase_shift, X, Y)


def directions(order):
    n = 12 * 4 ** order
    rot, tilt, ipix = np.zeros(n), np.zeros(n), np.zeros(n, np.int64)
    load().oracle_directions(I64(order), rot.ctypes.data_as(P), tilt.ctypes.data_as(P),
                             ipix.ctypes.data_as(P))
    return rot, tilt, ipix


def _geometry_model(ori, pad, ref=None, bp=None):
    """An OracleModel holding only the projector / backprojector geometry
    (for the building-block entry points)."""
    m = OracleModel()
    m.ori_size, m.nr_classes, m.padding_factor, m.ref_dim = ori, 1, pad, 3
    keep = []
    if ref is not None:
        d = np.ascontiguousarray(ref["data"], np.complex128)
        keep.append(d)
        m.proj_r_max = ref["r_max"]
        m.proj_zdim, m.proj_ydim, m.proj_xdim = d.shape
        m.proj_yinit, m.proj_zinit = ref["yinit"], ref["zinit"]
        m.ppref = d.ctypes.data
    if bp is not None:
        m.bp_r_max, m.bp_xdim, m.bp_ydim, m.bp_zdim = bp["r_max"], bp["xdim"], bp["ydim"], bp["zdim"]
        m.bp_yinit, m.bp_zinit = bp["yinit"], bp["zinit"]
    return m, keep


def project(ref, ori, pad, size, A):
    """The oracle's Projector::project of one 3x3 matrix -> [size][size/2+1]."""
    o = load()
    m, keep = _geometry_model(ori, pad, ref=ref)
    out = np.zeros((size, size // 2 + 1), np.complex128)
    a = np.ascontiguousarray(A, np.float64)
    o.oracle_project(C.byref(m), I64(0), a.ctypes.data_as(P), I64(size), out.ctypes.data_as(P))
    del keep
    return out


def backproject(ori, pad, current_size, size, mats, images, weights):
    """The oracle's backprojection of (matrix, image, weight) triplets into
    volumes of bp_geometry(current_size) -> (data complex, weight)."""
    o = load()
    g = bp_geometry(current_size, ori, pad)
    m, keep = _geometry_model(ori, pad, bp=g)
    data = np.zeros((g["zdim"], g["ydim"], g["xdim"]), np.complex128)
    wt = np.zeros((g["zdim"], g["ydim"], g["xdim"]))
    for A, f, w in zip(mats, images, weights):
        a = np.ascontiguousarray(A, np.float64)
        fi = np.ascontiguousarray(f, np.complex128)
        wi = np.ascontiguousarray(w, np.float64)
        o.oracle_backproject(C.byref(m), I64(0), a.ctypes.data_as(P), I64(size), fi.ctypes.data_as(P),
                             wi.ctypes.data_as(P), data.ctypes.data_as(P), wt.ctypes.data_as(P))
    del keep
    return data, wt


def shift(image, oridim, xshift, yshift):
    """The oracle's phase shift of a [size][size/2+1] image."""
    f = np.ascontiguousarray(image, np.complex128)
    out = np.zeros_like(f)
    load().oracle_shift_ft(f.ctypes.data_as(P), I64(f.shape[0]), F64(oridim), F64(xshift), F64(yshift),
                           out.ctypes.data_as(P))
    return out


def euler(rot, tilt, psi):
    A = np.zeros(9)
    load().oracle_euler(F64(rot), F64(tilt), F64(psi), A.ctypes.data_as(P))
    return A.reshape(3, 3)


def bp_geometry(current_size, ori_size, pad=2, ref_dim=3):
    """BackProjector::initialiseDataAndWeight sizes (3D volume, or one 2D plane)."""
    r_max = min(current_size // 2, ori_size // 2)
    pad_size = 2 * (int(pad * r_max + 0.5) + 1) + 1
    if ref_dim == 2:
        return dict(r_max=r_max, xdim=pad_size // 2 + 1, ydim=pad_size, zdim=1,
                    yinit=-(pad_size // 2), zinit=0)
    return dict(r_max=r_max, xdim=pad_size // 2 + 1, ydim=pad_size, zdim=pad_size,
                yinit=-(pad_size // 2), zinit=-(pad_size // 2))


def run(model, refs, batch, debug=False):
    """Oracle E-step for a batch.

    model: dict (same keys as relion_gb300's model dict); refs: list of
    reference dicts from relion_gb300.datagen.padded_reference (one per
    class); batch: host particle batch dict.  Returns (results, debug,
    wsum dict, bp_data [K][z][y][x] complex, bp_weight).
    """
    o = load()
    K = int(model["nr_classes"])
    keep = []

    def arr(a, dt=np.float64):
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data

    r0 = refs[0]
    ppref = np.stack([np.asarray(r["data"], np.complex128) for r in refs])
    ref_dim = int(model.get("ref_dim", 3) or 3)
    bg = bp_geometry(int(model["current_size"]), int(model["ori_size"]), int(model["padding_factor"]), ref_dim)
    m = OracleModel()
    for k in ("ori_size", "nr_classes", "current_size", "coarse_size", "padding_factor",
              "healpix_order", "adaptive_oversampling", "maximum_significants", "sigma2_len",
              "do_scale_correction", "do_norm_correction", "do_map"):
        setattr(m, k, int(model[k]))
    m.proj_r_max, m.proj_xdim, m.proj_ydim, m.proj_zdim = r0["r_max"], r0["xdim"], r0["ydim"], r0["zdim"]
    m.proj_yinit, m.proj_zinit = r0["yinit"], r0["zinit"]
    m.bp_r_max, m.bp_xdim, m.bp_ydim, m.bp_zdim = bg["r_max"], bg["xdim"], bg["ydim"], bg["zdim"]
    m.bp_yinit, m.bp_zinit = bg["yinit"], bg["zinit"]
    for k in ("pixel_size", "psi_step", "offset_range", "offset_step", "adaptive_fraction",
              "sigma2_fudge", "sigma2_offset", "avg_norm_correction"):
        setattr(m, k, float(model[k]))
    m.ppref = arr(ppref, np.complex128)
    m.sigma2_noise = arr(model["sigma2_noise"])
    m.pdf_class = arr(model["pdf_class"])
    m.pdf_direction = arr(model["pdf_direction"])
    m.data_vs_prior = arr(model["data_vs_prior"]) if model.get("data_vs_prior") is not None else None
    m.ref_dim = ref_dim
    poc = model.get("prior_offset_class")
    m.prior_offset_class = arr(np.zeros((K, 2)) if poc is None else poc)

    n = int(batch["n"])
    parts = (OracleParticle * n)()
    fimg = np.ascontiguousarray(batch["fimg"], np.complex64).astype(np.complex128)
    fnm = np.ascontiguousarray(batch["fimg_nomask"], np.complex64).astype(np.complex128)
    fctf = np.ascontiguousarray(batch["fctf"], np.float32).astype(np.float64)
    keep += [fimg, fnm, fctf]
    power = np.ascontiguousarray(batch["power_img"], np.float64)
    keep.append(power)
    for i in range(n):
        p = parts[i]
        p.fimg = fimg[i].ctypes.data
        p.fimg_nomask = fnm[i].ctypes.data
        p.fctf = fctf[i].ctypes.data
        p.power_img = power[i].ctypes.data
        p.old_offset[0], p.old_offset[1] = batch["old_offset"][i]
        p.prior[0], p.prior[1] = batch["prior"][i]
        p.highres_Xi2 = float(batch["highres_Xi2"][i])
        p.norm_correction = float(batch["norm_correction"][i])
        p.scale = float(batch["scale"][i])
    res = (OracleResult * n)()
    ndir, npsi, ntr = sampling_sizes(int(model["healpix_order"]), float(model["psi_step"]),
                                     float(model["offset_range"]), float(model["offset_step"]), ref_dim)
    RT = K * ndir * npsi * ntr
    ov = int(model["adaptive_oversampling"])
    nfine = RT * (2 ** ov if ref_dim == 2 else 8 ** ov) * 4 ** ov
    dbg = None
    dbg_arrays = []
    if debug:
        dbg = (OracleDebug * n)()
        for i in range(n):
            a = dict(coarse_diff2=np.zeros(RT), coarse_weight=np.zeros(RT),
                     coarse_significant=np.zeros(RT, np.uint8), fine_diff2=np.zeros(nfine),
                     fine_weight=np.zeros(nfine))
            for k, v in a.items():
                setattr(dbg[i], k, v.ctypes.data)
            dbg_arrays.append(a)
    half = int(model["ori_size"]) // 2 + 1
    vox = bg["xdim"] * bg["ydim"] * bg["zdim"]
    ws = dict(sigma2_noise=np.zeros(half), pdf_class=np.zeros(K), pdf_direction=np.zeros(K * ndir),
              bp_data=np.zeros((K, bg["zdim"], bg["ydim"], bg["xdim"]), np.complex128),
              bp_weight=np.zeros((K, bg["zdim"], bg["ydim"], bg["xdim"])),
              prior_offset_class=np.zeros((K, 2)))
    w = OracleWsum()
    for k in ("sigma2_noise", "pdf_class", "pdf_direction", "bp_data", "bp_weight", "prior_offset_class"):
        setattr(w, k, ws[k].ctypes.data)
    st = o.oracle_expectation(C.byref(m), I64(n), parts, res, dbg, C.byref(w))
    if st != 0:
        raise RuntimeError("oracle_expectation failed with status %d" % st)
    out = np.zeros(n, dtype=[(f, np.float64) for f, _ in OracleResult._fields_ if f != "pad_"])
    for i in range(n):
        for f in out.dtype.names:
            out[f][i] = getattr(res[i], f)
    wsum = {k: getattr(w, k) for k in ("sigma2_offset", "sumw_group", "LL", "ave_Pmax",
                                       "avg_norm_correction", "wsum_signal_product",
                                       "wsum_reference_power")}
    wsum.update(sigma2_noise=ws["sigma2_noise"], pdf_class=ws["pdf_class"],
                pdf_direction=ws["pdf_direction"].reshape(K, ndir),
                prior_offset_class=ws["prior_offset_class"])
    del keep, vox
    return out, dbg_arrays, wsum, ws["bp_data"], ws["bp_weight"]


class OraclePrepParams(C.Structure):
    _fields_ = [(n, I64) for n in ("ori_size", "current_size", "do_norm_correction", "pad_")] + \
        [(n, F64) for n in ("pixel_size", "mask_radius_px", "width_mask_edge", "avg_norm_correction",
                            "kV", "Cs", "Q0")]


class OracleImageMeta(C.Structure):
    _fields_ = [("old_offset", F64 * 2)] + \
        [(n, F64) for n in ("norm_correction", "defU", "defV", "defAngle", "Bfac", "scale", "phase_shift")]


META_FIELDS = ("norm_correction", "defU", "defV", "defAngle", "Bfac", "scale", "phase_shift")


def prepare_images(params, images, meta):
    """Oracle image preparation (getFourierTransformsAndCtfs).

    params: dict with the OraclePrepParams fields; images [n][ori][ori]
    real; meta: dict of per-particle arrays (old_offset [n][2] and
    META_FIELDS).  Returns dict(fimg, fimg_nomask, fctf, power_img,
    highres_Xi2, old_offset)."""
    o = load()
    pp = OraclePrepParams()
    for k, _ in OraclePrepParams._fields_:
        if k in params:
            setattr(pp, k, params[k])
    imgs = np.ascontiguousarray(images, np.float64)
    n, N = imgs.shape[0], imgs.shape[1]
    cur = int(params["current_size"])
    X = cur // 2 + 1
    ms = (OracleImageMeta * n)()
    for i in range(n):
        ms[i].old_offset[0], ms[i].old_offset[1] = meta["old_offset"][i]
        for k in META_FIELDS:
            setattr(ms[i], k, float(meta[k][i]))
    fimg = np.zeros((n, cur, X), np.complex128)
    fnm = np.zeros((n, cur, X), np.complex128)
    fctf = np.zeros((n, cur, X))
    power = np.zeros((n, N // 2 + 1))
    xi2 = np.zeros(n)
    off = np.zeros((n, 2))
    st = o.oracle_prepare_images(C.byref(pp), I64(n), imgs.ctypes.data, ms, fimg.ctypes.data, fnm.ctypes.data,
                                 fctf.ctypes.data, power.ctypes.data, xi2.ctypes.data, off.ctypes.data)
    if st != 0:
        raise RuntimeError("oracle_prepare_images failed with status %d" % st)
    return dict(fimg=fimg, fimg_nomask=fnm, fctf=fctf, power_img=power, highres_Xi2=xi2, old_offset=off)


# --- reconstruction side (oracle_mstep.cpp) -------------------------------
class OracleBpGeom(C.Structure):
    _fields_ = [(n, I64) for n in ("ori_size", "ref_dim", "pad", "r_max", "xdim", "ydim", "zdim",
                                   "yinit", "zinit")]


class OracleReconParams(C.Structure):
    _fields_ = [(n, I64) for n in ("max_iter_preweight", "do_map", "skip_gridding", "minres_map")] + \
        [(n, F64) for n in ("tau2_fudge", "normalise")]


def _bp_geom(ori_size, current_size, pad=2, ref_dim=3):
    g = bp_geometry(current_size, ori_size, pad, ref_dim)
    return OracleBpGeom(ori_size=ori_size, ref_dim=ref_dim, pad=pad, **g), g


def bp_symmetrise(data, weight, ori_size, current_size, pad=2, ref_dim=3):
    """BackProjector::enforceHermitianSymmetry on copies; returns (data, weight)."""
    gg, _ = _bp_geom(ori_size, current_size, pad, ref_dim)
    d = np.ascontiguousarray(data, np.complex128).copy()
    w = np.ascontiguousarray(weight, np.float64).copy()
    load().oracle_bp_symmetrise(C.byref(gg), d.ctypes.data, w.ctypes.data)
    return d, w


def update_ssnr(weight, ori_size, current_size, tau2, tau2_fudge=1.0, fsc=None, update_tau2_with_fsc=False,
                is_whole=False, pad=2, ref_dim=3):
    """BackProjector::updateSSNRarrays -> dict(tau2, sigma2, data_vs_prior, fourier_coverage)."""
    gg, _ = _bp_geom(ori_size, current_size, pad, ref_dim)
    ns = ori_size // 2 + 1
    t = np.array(tau2, np.float64).copy()
    out = [np.zeros(ns) for _ in range(3)]
    f = np.zeros(ns) if fsc is None else np.ascontiguousarray(fsc, np.float64)
    w = np.ascontiguousarray(weight, np.float64)
    st = load().oracle_update_ssnr(C.byref(gg), w.ctypes.data, F64(tau2_fudge), t.ctypes.data,
                                   *[o.ctypes.data for o in out], f.ctypes.data, I64(int(update_tau2_with_fsc)),
                                   I64(int(is_whole)))
    if st != 0:
        raise RuntimeError("oracle_update_ssnr failed with status %d" % st)
    return dict(tau2=t, sigma2=out[0], data_vs_prior=out[1], fourier_coverage=out[2])


def reconstruct(data, weight, ori_size, current_size, tau2=None, do_map=False, tau2_fudge=1.0, normalise=1.0,
                minres_map=5, skip_gridding=True, max_iter_preweight=10, pad=2, ref_dim=3):
    """BackProjector::reconstruct -> real-space map [ori]^ref_dim."""
    gg, _ = _bp_geom(ori_size, current_size, pad, ref_dim)
    p = OracleReconParams(max_iter_preweight=max_iter_preweight, do_map=int(do_map),
                          skip_gridding=int(skip_gridding), minres_map=minres_map, tau2_fudge=tau2_fudge,
                          normalise=normalise)
    t = np.zeros(ori_size // 2 + 1) if tau2 is None else np.ascontiguousarray(tau2, np.float64)
    vol = np.zeros((ori_size,) * ref_dim)
    d = np.ascontiguousarray(data, np.complex128)
    w = np.ascontiguousarray(weight, np.float64)
    st = load().oracle_reconstruct(C.byref(gg), d.ctypes.data, w.ctypes.data, C.byref(p), t.ctypes.data,
                                   vol.ctypes.data)
    if st != 0:
        raise RuntimeError("oracle_reconstruct failed with status %d" % st)
    return vol


def projector_from_map(vol, current_size, do_gridding=True, min_ires=-1, pad=2):
    """Projector::computeFourierTransformMap -> (padded Fourier reference, power spectrum)."""
    v = np.ascontiguousarray(vol, np.float64)
    ori, ref_dim = v.shape[-1], v.ndim
    r_max = min(current_size // 2, ori // 2) if current_size >= 0 else ori // 2
    ps = 2 * (int(pad * r_max + 0.5) + 1) + 1
    shape = (ps, ps, ps // 2 + 1) if ref_dim == 3 else (ps, ps // 2 + 1)
    proj = np.zeros(shape, np.complex128)
    power = np.zeros(ori // 2 + 1)
    st = load().oracle_projector_from_map(I64(ori), I64(ref_dim), I64(pad), v.ctypes.data, I64(current_size),
                                          I64(int(do_gridding)), I64(min_ires), proj.ctypes.data, power.ctypes.data)
    if st != 0:
        raise RuntimeError("oracle_projector_from_map failed with status %d" % st)
    return proj, power


def fsc(m1, m2):
    """getFSC of two real-space maps -> [ori/2+1]."""
    a = np.ascontiguousarray(m1, np.float64)
    b = np.ascontiguousarray(m2, np.float64)
    out = np.zeros(a.shape[-1] // 2 + 1)
    load().oracle_fsc(I64(a.shape[-1]), I64(a.ndim), a.ctypes.data, b.ctypes.data, out.ctypes.data)
    return out
