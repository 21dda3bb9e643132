"""The oracle's reconstruction side (oracle/oracle_mstep.cpp) against an
independent numpy statement of the same reference functions, written with
numpy's FFT instead of the oracle's own radix-2 / Bluestein transforms:

  BackProjector::enforceHermitianSymmetry  src/backprojector.cpp:2148-2165
  BackProjector::updateSSNRarrays          src/backprojector.cpp:1041-1204
  BackProjector::reconstruct               src/backprojector.cpp:1379-1872
  Projector::computeFourierTransformMap    src/projector.cpp:116-593
  getFSC                                   src/fftw.cpp:481-525

Sizes are small (box 16 / 20, odd padded grids of 35 and 43 points) so that
the whole file runs in seconds; every comparison is to 1e-10 relative.
"""
import numpy as np
import pytest


def _round(x):
    x = np.asarray(x, np.float64)
    return np.where(x > 0, np.floor(x + 0.5), np.ceil(x - 0.5)).astype(np.int64)


def _freqs(N, dim):
    """FFTW half-layout frequencies (FOR_ALL_ELEMENTS_IN_FFTW_TRANSFORM)."""
    X = N // 2 + 1
    a = np.arange(N)
    f = np.where(a < X, a, a - N)
    j = np.arange(X)
    if dim == 3:
        return f[:, None, None], f[None, :, None], j[None, None, :]
    return np.zeros((1, 1), np.int64), f[:, None], j[None, :]


def _geom(ori, cur, dim, pad=2):
    from oracle import pyoracle
    return pyoracle.bp_geometry(cur, ori, pad, dim)


def _bp_index(g, kp, ip, jp, dim):
    if dim == 3:
        return (kp - g["zinit"], ip - g["yinit"], jp)
    return (ip - g["yinit"], jp)


def _random_bp(ori, cur, dim, seed, pad=2):
    """Random data / weight volumes inside r_max, Hermitian-consistent on x = 0."""
    from oracle import pyoracle
    g = _geom(ori, cur, dim, pad)
    rng = np.random.default_rng(seed)
    shape = (g["zdim"], g["ydim"], g["xdim"]) if dim == 3 else (g["ydim"], g["xdim"])
    data = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    weight = rng.uniform(0.5, 2.0, size=shape)
    if dim == 3:
        k = np.arange(g["zdim"])[:, None, None] + g["zinit"]
        i = np.arange(g["ydim"])[None, :, None] + g["yinit"]
    else:
        k = np.zeros((1, 1), np.int64)
        i = np.arange(g["ydim"])[:, None] + g["yinit"]
    j = np.arange(g["xdim"])[(None,) * (dim - 1) + (slice(None),)]
    r2 = k * k + i * i + j * j
    inside = r2 < (pad * g["r_max"]) ** 2
    data, weight = np.where(inside, data, 0), np.where(inside, weight, 0.)
    data, weight = pyoracle.bp_symmetrise(data, weight, ori, cur, pad, dim)
    return g, data, weight


def _np_symmetrise(g, data, weight, dim):
    d, w = data.copy(), weight.copy()
    zr = range(g["zinit"], g["zinit"] + g["zdim"]) if dim == 3 else [0]
    for iz in zr:
        for iy in range(0 if iz < 0 else 1, g["yinit"] + g["ydim"]):
            a = _bp_index(g, iz, iy, 0, dim)
            b = _bp_index(g, -iz, -iy, 0, dim)
            s = d[a] + np.conj(d[b])
            d[a], d[b] = s, np.conj(s)
            t = w[a] + w[b]
            w[a], w[b] = t, t
    return d, w


@pytest.mark.parametrize("dim", [3, 2])
def test_symmetrise(oracle_lib, dim):
    from oracle import pyoracle
    g = _geom(16, 16, dim)
    rng = np.random.default_rng(4)
    shape = (g["zdim"], g["ydim"], g["xdim"]) if dim == 3 else (g["ydim"], g["xdim"])
    data = rng.normal(size=shape) + 1j * rng.normal(size=shape)
    weight = rng.uniform(size=shape)
    d1, w1 = pyoracle.bp_symmetrise(data, weight, 16, 16, 2, dim)
    d2, w2 = _np_symmetrise(g, data, weight, dim)
    np.testing.assert_array_equal(d1, d2)
    np.testing.assert_array_equal(w1, w2)


def _np_ssnr(g, weight, ori, tau2, fudge, fsc, upd, whole, dim, pad=2):
    if dim == 3:
        k = np.arange(g["zdim"])[:, None, None] + g["zinit"]
        i = np.arange(g["ydim"])[None, :, None] + g["yinit"]
    else:
        k = np.zeros((1, 1), np.int64)
        i = np.arange(g["ydim"])[:, None] + g["yinit"]
    j = np.arange(g["xdim"])[(None,) * (dim - 1) + (slice(None),)]
    r2 = np.broadcast_to(k * k + i * i + j * j, weight.shape)
    ns = ori // 2 + 1
    max_r2 = int(_round(g["r_max"] * pad)) ** 2
    ovc = float(pad ** dim)
    m = r2 < max_r2
    ires = _round(np.sqrt(r2[m]) / pad)
    w = weight[m]
    s = np.bincount(ires, weights=ovc * w, minlength=ns)
    c = np.bincount(ires, minlength=ns).astype(np.float64)
    sigma2 = np.where(s > 1e-20, c / np.where(s > 0, s, 1), 0.)
    tau2 = np.array(tau2, np.float64)
    dvp = np.zeros(ns)
    if upd:
        f = np.maximum(0.001, fsc)
        if whole:
            f = np.sqrt(2. * f / (f + 1.))
        f = np.minimum(0.999, f)
        ssnr = f / (1. - f) * fudge
        tau2, dvp = ssnr * sigma2, ssnr
    t = tau2[ires]
    with np.errstate(divide="ignore"):
        invtau2 = np.where(t > 0, 1. / (ovc * fudge * np.where(t > 0, t, 1)), 1. / (0.001 * w))
    ratio = w / invtau2
    if not upd:
        dvp = np.bincount(ires, weights=ratio, minlength=ns)
    cov = np.bincount(ires, weights=(ratio >= 1.).astype(np.float64), minlength=ns)
    cnt = np.bincount(ires, minlength=ns).astype(np.float64)
    if not upd:
        dvp = np.where(np.arange(ns) > g["r_max"], 0., np.where(cnt < 0.001, 999., dvp / np.maximum(cnt, 1)))
    cov = np.where(cnt > 0, cov / np.maximum(cnt, 1), cov)
    return dict(tau2=tau2, sigma2=sigma2, data_vs_prior=dvp, fourier_coverage=cov)


@pytest.mark.parametrize("dim,upd,whole", [(3, False, False), (3, True, False), (3, True, True), (2, False, False)])
def test_update_ssnr(oracle_lib, dim, upd, whole):
    from oracle import pyoracle
    ori = 16
    g, data, weight = _random_bp(ori, 12, dim, 7)
    rng = np.random.default_rng(8)
    tau2 = rng.uniform(0.1, 2.0, ori // 2 + 1)
    tau2[3] = 0.
    fsc = rng.uniform(-0.1, 1.0, ori // 2 + 1)
    o = pyoracle.update_ssnr(weight, ori, 12, tau2, 1.5, fsc, upd, whole, 2, dim)
    n = _np_ssnr(g, weight, ori, tau2, 1.5, fsc, upd, whole, dim)
    for k in n:
        np.testing.assert_allclose(o[k], n[k], rtol=1e-12, atol=1e-300, err_msg=k)


def _real_coords(ori, dim):
    h = ori // 2
    a = np.arange(ori) - h
    if dim == 3:
        return a[:, None, None], a[None, :, None], a[None, None, :]
    return np.zeros((1, 1), np.int64), a[:, None], a[None, :]


def _np_gridding_correct(v, ori, dim, pad=2):
    k, i, j = _real_coords(ori, dim)
    r = np.sqrt((k * k + i * i + j * j).astype(np.float64))
    rv = np.where(r > 0, r / (ori * pad), 1.)
    sinc = np.sin(np.pi * rv) / (np.pi * rv)
    return np.where(r > 0, v / (sinc * sinc), v)


def _np_soft_mask(v, ori, dim):
    k, i, j = _real_coords(ori, dim)
    r = np.broadcast_to(np.sqrt((k * k + i * i + j * j).astype(np.float64)), v.shape)
    rad = ori / 2.
    rp = rad + 3.
    rc = 0.5 + 0.5 * np.cos(np.pi * (rp - r) / 3.)
    wgt = np.where(r < rad, 0., np.where(r > rp, 1., rc))
    bg = (wgt * v).sum() / wgt.sum()
    return np.where(r < rad, v, np.where(r > rp, bg, (1 - rc) * v + rc * bg))


def _blob_ratio(rval):
    from scipy.special import iv, jv
    a, alpha, n = 3.8, 15., 10000
    samp = 0.5 / n
    idx = (np.abs(rval) / samp).astype(np.int64)
    w = np.minimum(idx, n - 1) * samp
    s2 = 2 * np.pi * a * w
    sig = np.sqrt(np.abs(alpha * alpha - s2 * s2))
    f = np.where(s2 > alpha, jv(1.5, sig), iv(1.5, sig)) / sig ** 1.5
    f0 = iv(1.5, alpha) / alpha ** 1.5
    return np.where(idx >= n, 0., f / f0)


def _np_reconstruct(data, weight, ori, cur, dim, tau2=None, do_map=False, fudge=1., normalise=1., minres=5,
                    skip=True, niter=10, pad=2):
    g = _geom(ori, cur, dim, pad)
    N, r_max = g["ydim"], g["r_max"]
    kp, ip, jp = _freqs(N, dim)
    r2 = np.broadcast_to(kp * kp + ip * ip + jp * jp, ((N,) if dim == 3 else ()) + (N, N // 2 + 1))
    kb, ib, jb = np.broadcast_arrays(kp, ip, jp)
    idx = _bp_index(g, kb, ib, jb, dim)
    max_r2 = int(_round(r_max * pad)) ** 2
    Fw = np.where(r2 <= max_r2, weight[idx], 0.)
    if do_map:
        ires = _round(np.sqrt(r2) / pad)
        t = np.asarray(tau2)[np.minimum(ires, len(tau2) - 1)]
        inv = np.where(t > 0, 1. / (pad ** dim * fudge * np.where(t > 0, t, 1)),
                       np.where(Fw > 1e-20, 1. / (0.001 * np.where(Fw > 0, Fw, 1)), 0.))
        Fw = np.where((r2 < max_r2) & (ires >= minres), Fw + inv, Fw)
    if skip:
        Fc = np.where(r2 <= max_r2, data[idx], 0)
        rm2 = int(_round(r_max * pad * r_max * pad))
        m = r2 < rm2
        fl = np.floor(np.sqrt(r2) / pad).astype(np.int64)
        ra = np.bincount(fl[m], weights=Fw[m], minlength=r_max)[:r_max]
        cn = np.bincount(fl[m], minlength=r_max)[:r_max]
        ra = ra / (1000. * cn)
        w = np.maximum(Fw, ra[np.minimum(fl, r_max - 1)])
        Fc = np.where(w != 0, Fc / np.where(w != 0, w, 1), Fc)
    else:
        Fw = Fw / normalise
        Fn = np.where(r2 < max_r2, 1., 0.)
        sh = (N,) * dim
        a = np.arange(N)
        f = np.where(a < N // 2, a, a - N)
        if dim == 3:
            rr = np.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + f[None, None, :] ** 2)
        else:
            rr = np.sqrt(f[:, None] ** 2 + f[None, :] ** 2)
        blob = _blob_ratio(rr / (ori * pad))
        for _ in range(niter):
            M = np.fft.irfftn(Fn * Fw, s=sh, axes=tuple(range(dim))) * N ** dim
            Fc = np.fft.rfftn(M * blob) / N ** dim
            Fn = np.where(r2 < max_r2, Fn / np.maximum(1e-6, np.abs(Fc)), Fn)
        Fc = np.where(r2 <= max_r2, data[idx] / normalise, 0) * Fn
    No = 2 * ori if pad == 2 else int(_round(pad * ori)) + int(_round(pad * ori)) % 2
    X = N // 2 + 1
    Fo = np.zeros(((No,) if dim == 3 else ()) + (No, No // 2 + 1), np.complex128)
    if No // 2 + 1 > X:
        m = (kb * kb + ib * ib + jb * jb) <= (X - 1) ** 2
        if dim == 3:
            Fo[kb[m] % No, ib[m] % No, jb[m]] = Fc[m]
        else:
            Fo[ib[m] % No, jb[m]] = Fc[m]
    else:
        ko, io, jo = np.broadcast_arrays(*_freqs(No, dim))
        Fo = Fc[(ko % N, io % N, jo)] if dim == 3 else Fc[(io % N, jo)]
    par = np.indices(Fo.shape).sum(axis=0) & 1
    Fo = np.where(par == 1, -Fo, Fo)
    Mo = np.fft.irfftn(Fo, s=(No,) * dim, axes=tuple(range(dim))) * No ** dim
    off = No // 2 - ori // 2
    v = Mo[(slice(off, off + ori),) * dim] / (pad ** 3 * ori if dim == 3 else pad ** 2)
    return _np_gridding_correct(_np_soft_mask(v, ori, dim), ori, dim, pad)


@pytest.mark.parametrize("dim,cur,do_map,skip", [(3, 16, False, True), (3, 12, True, True), (2, 20, True, True),
                                                 (3, 16, True, False), (2, 12, False, False)])
def test_reconstruct(oracle_lib, dim, cur, do_map, skip):
    from oracle import pyoracle
    ori = 20 if dim == 2 else 16
    g, data, weight = _random_bp(ori, cur, dim, 11)
    rng = np.random.default_rng(12)
    tau2 = rng.uniform(0.05, 1.0, ori // 2 + 1)
    tau2[-2:] = 0.
    kw = dict(tau2=tau2, do_map=do_map, tau2_fudge=1.3, normalise=2.5, minres_map=2, skip_gridding=skip,
              max_iter_preweight=4)
    o = pyoracle.reconstruct(data, weight, ori, cur, pad=2, ref_dim=dim, **kw)
    n = _np_reconstruct(data, weight, ori, cur, dim, tau2, do_map, 1.3, 2.5, 2, skip, 4)
    assert o.shape == (ori,) * dim
    assert np.linalg.norm(o - n) <= 1e-10 * np.linalg.norm(n)


def _np_projector_from_map(vol, cur, do_gridding, min_ires, pad=2):
    ori, dim = vol.shape[-1], vol.ndim
    v = _np_gridding_correct(vol, ori, dim, pad) if do_gridding else vol
    No = pad * ori
    M = np.zeros((No,) * dim)
    off = No // 2 - ori // 2
    M[(slice(off, off + ori),) * dim] = v
    F = np.fft.rfftn(M) / No ** dim
    par = np.indices(F.shape).sum(axis=0) & 1
    F = np.where(par == 1, -F, F)
    r_max = min(cur // 2, ori // 2)
    ps = 2 * (int(_round(pad * r_max)) + 1) + 1
    kp, ip, jp = np.broadcast_arrays(*_freqs(No, dim))
    r2 = kp * kp + ip * ip + jp * jp
    max_r2 = int(_round(r_max * pad)) ** 2
    m = r2 <= max_r2
    normfft = pad ** 3 * ori if dim == 3 else pad ** 2
    val = F[m] * normfft
    P = np.zeros(((ps,) if dim == 3 else ()) + (ps, ps // 2 + 1), np.complex128)
    ires = _round(np.sqrt(r2[m]) / pad)
    ns = ori // 2 + 1
    pw = np.bincount(ires, weights=np.abs(val) ** 2 / 2., minlength=ns)
    cn = np.bincount(ires, minlength=ns).astype(np.float64)
    min_r2 = int(_round(min_ires * pad)) ** 2 if min_ires > 0 else -1
    val = np.where(r2[m] <= min_r2, 0, val)
    if dim == 3:
        P[kp[m] + ps // 2, ip[m] + ps // 2, jp[m]] = val
    else:
        P[ip[m] + ps // 2, jp[m]] = val
    return P, np.where(cn < 1, 0., pw / np.maximum(cn, 1))


@pytest.mark.parametrize("dim,cur,grid,min_ires", [(3, 12, True, -1), (3, 16, False, 2), (2, 20, True, -1)])
def test_projector_from_map(oracle_lib, dim, cur, grid, min_ires):
    from oracle import pyoracle
    ori = 20 if dim == 2 else 16
    vol = np.random.default_rng(21).normal(size=(ori,) * dim)
    P1, p1 = pyoracle.projector_from_map(vol, cur, grid, min_ires)
    P2, p2 = _np_projector_from_map(vol, cur, grid, min_ires)
    assert np.linalg.norm(P1 - P2) <= 1e-10 * np.linalg.norm(P2)
    np.testing.assert_allclose(p1, p2, rtol=1e-10)


@pytest.mark.parametrize("dim", [3, 2])
def test_fsc(oracle_lib, dim):
    from oracle import pyoracle
    rng = np.random.default_rng(30)
    a = rng.normal(size=(16,) * dim)
    b = a + 0.7 * rng.normal(size=a.shape)
    f = pyoracle.fsc(a, b)
    F1, F2 = np.fft.rfftn(a), np.fft.rfftn(b)
    kp, ip, jp = np.broadcast_arrays(*_freqs(16, dim))
    idx = _round(np.sqrt((kp * kp + ip * ip + jp * jp).astype(np.float64)))
    m = idx < 9
    num = np.bincount(idx[m], weights=(np.conj(F1) * F2).real[m], minlength=9)
    d1 = np.bincount(idx[m], weights=np.abs(F1[m]) ** 2, minlength=9)
    d2 = np.bincount(idx[m], weights=np.abs(F2[m]) ** 2, minlength=9)
    np.testing.assert_allclose(f, num / np.sqrt(d1 * d2), rtol=1e-10)
    np.testing.assert_allclose(pyoracle.fsc(a, a), np.ones(9), rtol=1e-12)
