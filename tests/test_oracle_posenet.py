"""The pose-proposal oracle's analytic gradient against central differences
(float64), and its feature binning on a hand-checked pixel set."""
import numpy as np

from oracle import posenet_oracle as po


def test_gradient_matches_central_differences():
    H, W, C1, C2, ND, B = 4, 6, 2, 3, 5, 3
    g = np.random.default_rng(5)
    o = po.layout(H, W, C1, C2, ND)
    p = g.normal(0, 0.5, o["n"])
    p[o["b1"]:o["w2"]] += 0.3  # most units active
    p[o["b2"]:o["w3"]] += 0.3
    feat = g.normal(0, 1, (B, H * W))
    t = g.random((B, ND))
    t /= t.sum(axis=1, keepdims=True)
    loss, grad = po.loss_grad(p, feat, t, H, W, C1, C2, ND)
    eps = 1e-6
    for i in g.choice(o["n"], 60, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        num = (po.loss_grad(pp, feat, t, H, W, C1, C2, ND)[0] -
               po.loss_grad(pm, feat, t, H, W, C1, C2, ND)[0]) / (2 * eps)
        assert abs(num - grad[i]) <= 1e-6 * max(1.0, abs(num)), (i, num, grad[i])
    assert np.isfinite(loss) and loss > 0


def test_pixel_bins():
    xy = np.array([[1, 0], [0, 1], [0, -1], [1, 1], [2, -2], [0, 0], [5, 0]], np.int32)
    b = po.pixel_bins(xy, H=3, W=4)
    # (1,0): ring 1, angle pi/2 -> bin 2; (0,1): angle pi -> wraps to 0;
    # (0,-1): angle 0 -> 0; (1,1): ring 1, 3pi/4 -> 3; (2,-2): ring 3, pi/4 -> 1
    assert list(b) == [2, 0, 0, 3, 2 * 4 + 1, -1, -1]


def _half_plane(fn, cur):
    """[cur][cur/2+1] complex image of a function of (x, y) on the FFTW half plane."""
    X = cur // 2 + 1
    y = np.arange(cur)
    y = np.where(y < X, y, y - cur)[:, None]
    x = np.arange(X)[None, :]
    return fn(x.astype(np.float64), y.astype(np.float64))


def test_features_translation_invariant_and_rotation_is_a_shift():
    # the design claims behind the features: a shift only changes phases
    # (power unchanged), a 90 degree in-plane rotation maps the pixel grid onto
    # itself and moves every angle bin by W/2 (angles are taken modulo pi)
    cur, H, W = 32, 12, 24
    xs, ys = np.meshgrid(np.arange(cur // 2 + 1), np.arange(cur))
    ys = np.where(ys < cur // 2 + 1, ys, ys - cur)
    r = np.sqrt(xs ** 2 + ys ** 2)
    keep = (r >= 1) & (r <= H)
    xy = np.stack([xs[keep], ys[keep]], 1).astype(np.int32)
    minv = np.full(len(xy), 0.5, np.float32)

    def f(x, y):  # Friedel-symmetric, anisotropic: power depends on direction
        return (np.exp(-((x - 0.3 * y) ** 2) / 30.0 - (y ** 2) / 8.0) * (1 + 0.5 * np.cos(0.7 * x * y))) + 0j

    a = _half_plane(f, cur)[None]
    sh = _half_plane(lambda x, y: f(x, y) * np.exp(-2j * np.pi * (3 * x - 5 * y) / cur), cur)[None]
    rot = _half_plane(lambda x, y: f(y, -x), cur)[None]  # f rotated by 90 degrees
    fa = po.features(a, xy, minv, H, W).reshape(H, W)
    fs = po.features(sh, xy, minv, H, W).reshape(H, W)
    fr = po.features(rot, xy, minv, H, W).reshape(H, W)
    np.testing.assert_allclose(fs, fa, rtol=1e-12, atol=1e-12)
    assert np.abs(fa).max() > 0.1
    # bins exactly on a boundary may fall either side: compare all but a few
    d = np.abs(np.roll(fa, W // 2, axis=1) - fr)
    assert np.mean(d < 1e-9) > 0.9, np.mean(d < 1e-9)
