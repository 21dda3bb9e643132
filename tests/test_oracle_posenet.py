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
