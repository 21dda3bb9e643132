"""Runs the reference's own CPU code through oracle/_ref/ref_pin (TEST
INFRASTRUCTURE ONLY).

ref_pin is built by oracle/build_ref.sh from the reference's sources (where
they lie) when the reference tree is present; every function here returns
None when it is not.  Request / response layouts are those of
oracle/ref/ref_pin_driver.cpp.  Only tests/ and tests/golden/ use this
module.
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(HERE, "_ref", "ref_pin")


def available():
    return os.path.exists(BIN) and os.access(BIN, os.X_OK)


def _call(mode, req):
    if not available():
        return None
    with tempfile.TemporaryDirectory() as d:
        rq, rs = os.path.join(d, "req.bin"), os.path.join(d, "out.bin")
        np.concatenate([np.ravel(np.asarray(x, np.float64)) for x in req]).tofile(rq)
        p = subprocess.run([BIN, mode, rq, rs], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
        if p.returncode != 0:
            raise RuntimeError("ref_pin %s failed: %s" % (mode, p.stderr.strip()))
        return np.fromfile(rs, np.float64)


def _cplx(a):
    a = np.ascontiguousarray(a, np.complex128)
    return a.view(np.float64).ravel()


def euler(angles):
    """Euler_angles2matrix of [n][3] (rot, tilt, psi) -> [n][3][3]."""
    a = np.asarray(angles, np.float64).reshape(-1, 3)
    out = _call("euler", [[len(a)], a])
    return None if out is None else out.reshape(len(a), 3, 3)


def project(ref, ori, pad, size, mats):
    """Projector::project of the padded reference dict (data [z][y][x]
    complex, yinit, zinit, r_max) for each 3x3 matrix -> [n][size][size/2+1]."""
    d = np.asarray(ref["data"])
    z, y, x = d.shape
    mats = np.asarray(mats, np.float64).reshape(-1, 3, 3)
    out = _call("project", [[ori, pad, ref["r_max"], x, y, z, ref["yinit"], ref["zinit"]], _cplx(d),
                            [size, len(mats)], mats])
    if out is None:
        return None
    return out.view(np.complex128).reshape(len(mats), size, size // 2 + 1)


def backproject(ori, pad, current_size, size, mats, images, weights):
    """BackProjector::backproject2Dto3D of each (matrix, image, weight) into
    volumes of BackProjector::initZeros(current_size); returns
    (data [z][y][x] complex, weight, (yinit, zinit))."""
    mats = np.asarray(mats, np.float64).reshape(-1, 3, 3)
    req = [[ori, pad, current_size, size, len(mats)]]
    for A, f, w in zip(mats, images, weights):
        req += [A, _cplx(f), np.asarray(w, np.float64)]
    out = _call("backproject", req)
    if out is None:
        return None
    xd, yd, zd, yi, zi = [int(v) for v in out[:5]]
    n = xd * yd * zd
    data = out[5:5 + 2 * n].view(np.complex128).reshape(zd, yd, xd)
    weight = out[5 + 2 * n:5 + 3 * n].reshape(zd, yd, xd)
    return data, weight, (yi, zi)


def ctf_images(ori, angpix, params):
    """CTF::getFftwImage (damping on, no padding) of [n][9] parameters
    (defU, defV, defAng, kV, Cs, Q0, Bfac, scale, phase_shift) ->
    [n][ori][ori/2+1]."""
    p = np.asarray(params, np.float64).reshape(-1, 9)
    out = _call("ctf", [[ori, angpix, len(p)], p])
    return None if out is None else out.reshape(len(p), ori, ori // 2 + 1)


def sampling(order, psi_step, offset_range, offset_step, pixel, oversampling):
    """HealpixSampling (C1): the oversampled (rot, tilt, psi) of every coarse
    (direction, psi) [ndir][npsi][nover_rot][3] and the oversampled
    translations in pixels [ntrans][nover_trans][2]."""
    out = _call("sampling", [[order, psi_step, offset_range, offset_step, pixel, oversampling]])
    if out is None:
        return None
    ndir, npsi, ntr = [int(v) for v in out[:3]]
    nor = 8 ** oversampling
    nrot = ndir * npsi * nor * 3
    rot = out[3:3 + nrot].reshape(ndir, npsi, nor, 3)
    tr = out[3 + nrot:].reshape(ntr, -1, 2)
    return rot, tr


def shift(image, oridim, xshift, yshift):
    """shiftImageInFourierTransform of a [size][size/2+1] image."""
    f = np.asarray(image)
    out = _call("shift", [[f.shape[0], oridim, xshift, yshift], _cplx(f)])
    return None if out is None else out.view(np.complex128).reshape(f.shape)


def reconstruct(ori, pad, current_size, data, weight, tau2, skip_gridding=True, max_iter_preweight=10, do_map=True,
                tau2_fudge=1.0, normalise=1.0, minres_map=5):
    """BackProjector::reconstruct of the given volumes -> map [ori]^3."""
    z, y, x = np.asarray(data).shape
    out = _call("reconstruct", [[ori, pad, current_size, int(skip_gridding), max_iter_preweight, int(do_map),
                                 tau2_fudge, normalise, minres_map, x, y, z], _cplx(data),
                                np.asarray(weight, np.float64), np.asarray(tau2, np.float64)])
    return None if out is None else out.reshape(ori, ori, ori)


def fourier_map(ori, pad, current_size, vol, do_gridding=True, min_ires=-1):
    """Projector::computeFourierTransformMap of a map [ori]^3 -> (data
    [z][y][x] complex, (yinit, zinit, r_max), power spectrum)."""
    out = _call("fouriermap", [[ori, pad, current_size, int(do_gridding), min_ires], np.asarray(vol, np.float64)])
    if out is None:
        return None
    xd, yd, zd, yi, zi, rmax = [int(v) for v in out[:6]]
    n = xd * yd * zd
    data = out[6:6 + 2 * n].view(np.complex128).reshape(zd, yd, xd)
    power = out[6 + 2 * n:]
    return data, (yi, zi, rmax), power


ESTEP_BIN = os.path.join(HERE, "_ref", "ref_estep")
METADATA = ("rot", "tilt", "psi", "xoff", "yoff", "cls", "dLL", "pmax", "nr_sign", "norm")
SCALARS = ("coarse_min_diff2", "coarse_sum_weight", "coarse_significant_weight", "fine_min_diff2",
           "fine_sum_weight", "fine_significant_weight", "max_weight")


def estep_available():
    return os.path.exists(ESTEP_BIN) and os.access(ESTEP_BIN, os.X_OK)


def estep(model, ref, batch):
    """The reference's CPU E-step (MlOptimiser::getAllSquaredDifferences,
    convertAllSquaredDifferencesToWeights for both passes, storeWeightedSums)
    on a prepared batch of one class, through oracle/_ref/ref_estep.
    Returns (per-particle list of dicts: coarse_diff2, coarse_weight,
    coarse_significant, fine_diff2, fine_weight and the scalars / metadata of
    SCALARS / METADATA; wsum dict; bp_data [z][y][x] complex; bp_weight)."""
    if not estep_available():
        return None
    d = np.asarray(ref["data"], np.complex128)
    z, y, x = d.shape
    n = int(batch["n"])
    m = model
    req = [[m["ori_size"], m["current_size"], m["coarse_size"], m["padding_factor"], m["healpix_order"],
            m["psi_step"], m["offset_range"], m["offset_step"], m["pixel_size"], m["adaptive_fraction"],
            m["sigma2_fudge"], m["sigma2_offset"], n, x, y, z, ref["yinit"], ref["zinit"], ref["r_max"]],
           _cplx(d), np.asarray(m["sigma2_noise"], np.float64), np.asarray(m["pdf_direction"], np.float64)]
    for i in range(n):
        req += [_cplx(batch["fimg"][i]), _cplx(batch["fimg_nomask"][i]), np.asarray(batch["fctf"][i], np.float64),
                np.asarray(batch["power_img"][i], np.float64), batch["old_offset"][i], batch["prior"][i],
                [batch["highres_Xi2"][i], batch["norm_correction"][i]]]
    with tempfile.TemporaryDirectory() as td:
        rq, rs = os.path.join(td, "req.bin"), os.path.join(td, "out.bin")
        np.concatenate([np.ravel(np.asarray(q, np.float64)) for q in req]).tofile(rq)
        p = subprocess.run([ESTEP_BIN, rq, rs], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
        if p.returncode != 0:
            raise RuntimeError("ref_estep failed: %s" % p.stderr.strip())
        out = np.fromfile(rs, np.float64)
    k = 0
    parts = []
    for i in range(n):
        rec = {}
        for ipass, tag in ((0, "coarse"), (1, "fine")):
            cnt = int(out[k])
            k += 1
            rec[tag + "_diff2"] = out[k:k + cnt]
            k += cnt
            rec[tag + "_weight"] = out[k:k + cnt]
            k += cnt
            if ipass == 0:
                rec["coarse_significant"] = out[k:k + cnt].astype(bool)
                k += cnt
        for s in SCALARS:
            rec[s] = out[k]
            k += 1
        for s in METADATA:
            rec[s] = out[k]
            k += 1
        parts.append(rec)
    half = int(m["ori_size"]) // 2 + 1
    ndir = len(m["pdf_direction"])
    ws = dict(sigma2_noise=out[k:k + half])
    k += half
    ws["pdf_class"] = out[k:k + 1]
    k += 1
    ws["pdf_direction"] = out[k:k + ndir]
    k += ndir
    for s in ("sigma2_offset", "sumw_group", "LL", "ave_Pmax", "avg_norm_correction"):
        ws[s] = out[k]
        k += 1
    xd, yd, zd = [int(v) for v in out[k:k + 3]]
    k += 3
    nv = xd * yd * zd
    bp_data = out[k:k + 2 * nv].view(np.complex128).reshape(zd, yd, xd)
    k += 2 * nv
    bp_weight = out[k:k + nv].reshape(zd, yd, xd)
    return parts, ws, bp_data, bp_weight
