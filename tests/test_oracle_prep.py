"""The oracle's image preparation (getFourierTransformsAndCtfs restated in
C++, test infrastructure) against an independent numpy statement of the same
steps: integer shift by the rounded old offset, norm correction, forward FFT
/ N^2, window to the current size with CenterFFTbySign, average-background
soft mask, power spectrum / highres_Xi2 of the masked image, CTF image."""
import numpy as np
import pytest


def _numpy_prep(p, imgs, meta):
    N, cur = p["ori_size"], p["current_size"]
    X, half, h = cur // 2 + 1, N // 2 + 1, N // 2
    out = dict(fimg=[], fimg_nomask=[], power_img=[], highres_Xi2=[], fctf=[])
    yy, xx = np.meshgrid(np.arange(N) - h, np.arange(N) - h, indexing="ij")
    r = np.sqrt(yy ** 2 + xx ** 2)
    R, Rp, w = p["mask_radius_px"], p["mask_radius_px"] + p["width_mask_edge"], p["width_mask_edge"]
    rc = 0.5 + 0.5 * np.cos(np.pi * (Rp - r) / w)

    def rnd(v):
        return int(v + 0.5) if v > 0 else int(v - 0.5)

    def window_center(F):
        rows = np.r_[0:X, N - (cur - X):N]
        W = F[rows, :X].copy()
        i, j = np.meshgrid(np.arange(cur), np.arange(X), indexing="ij")
        W[((i ^ j) & 1) == 1] *= -1
        return W

    for k in range(len(imgs)):
        f = p["avg_norm_correction"] / meta["norm_correction"][k] if p["do_norm_correction"] else 1.0
        dx, dy = rnd(meta["old_offset"][k][0]), rnd(meta["old_offset"][k][1])
        img = np.zeros((N, N))
        src = imgs[k] * f
        ys, xs = slice(max(dy, 0), N + min(dy, 0)), slice(max(dx, 0), N + min(dx, 0))
        img[ys, xs] = src[max(-dy, 0):N - max(dy, 0), max(-dx, 0):N - max(dx, 0)]
        out["fimg_nomask"].append(window_center(np.fft.rfft2(img) / N ** 2))
        outside = r >= R
        edge = outside & (r <= Rp)
        wts = np.where(r > Rp, 1.0, np.where(edge, rc, 0.0))
        bg = (wts * img).sum() / wts.sum()
        img = np.where(r > Rp, bg, np.where(edge, (1 - rc) * img + rc * bg, img))
        F = np.fft.rfft2(img) / N ** 2
        ip = np.where(np.arange(N) < half, np.arange(N), np.arange(N) - N)[:, None]
        jp = np.arange(half)[None, :]
        ires = np.floor(np.sqrt(ip ** 2 + jp ** 2) + 0.5).astype(int)
        ok = (ires > 0) & (ires < half) & ~((jp == 0) & (ip < 0))
        pw = np.zeros(half)
        np.add.at(pw, ires[ok], (np.abs(F) ** 2)[ok])
        out["power_img"].append(pw if cur < N else np.zeros(half))
        out["highres_Xi2"].append(pw[cur // 2 + 1:].sum() if cur < N else 0.0)
        out["fimg"].append(window_center(F))
    return {k: np.array(v) for k, v in out.items()}


def test_oracle_prepare_matches_numpy(oracle_lib):
    from oracle import pyoracle
    g = np.random.default_rng(7)
    N, n = 48, 3
    p = dict(ori_size=N, current_size=30, do_norm_correction=1, pixel_size=2.0, mask_radius_px=17.0,
             width_mask_edge=5.0, avg_norm_correction=0.8, kV=300.0, Cs=2.7, Q0=0.1)
    imgs = g.normal(size=(n, N, N))
    meta = dict(old_offset=np.array([[1.4, -2.6], [-0.5, 0.49], [3.0, 2.5]]), norm_correction=[1.0, 1.3, 0.7],
                defU=[15000.0, 20000.0, 12000.0], defV=[14000.0, 21000.0, 12500.0], defAngle=[10.0, 80.0, 170.0],
                Bfac=[0.0, 0.0, 0.0], scale=[1.0, 1.0, 1.0], phase_shift=[0.0, 0.0, 0.0])
    o = pyoracle.prepare_images(p, imgs, meta)
    e = _numpy_prep(p, imgs, meta)
    assert np.array_equal(o["old_offset"], [[1, -3], [-1, 0], [3, 3]])
    for k in ("fimg", "fimg_nomask", "power_img", "highres_Xi2"):
        np.testing.assert_allclose(o[k], e[k], rtol=1e-9, atol=1e-12, err_msg=k)
    # CTF image: the building block pinned by the reference's KAT, on the full-box frequencies
    X = 16
    ip = np.where(np.arange(30) < X, np.arange(30), np.arange(30) - 30)
    for k in range(n):
        want = np.array([[pyoracle.ctf(meta["defU"][k], meta["defV"][k], meta["defAngle"][k], 300.0, 2.7, 0.1,
                                       0.0, 1.0, 0.0, j / (N * 2.0), i / (N * 2.0)) for j in range(X)] for i in ip])
        np.testing.assert_allclose(o["fctf"][k], want, rtol=1e-12)
