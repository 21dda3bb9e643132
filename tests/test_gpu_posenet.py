"""Learned pose proposal on the device (gbr_posenet_*) against the numpy
oracle, and what training buys.

Tolerances: features (FP32 bin sums in shared memory, FP32 log1p) to 1e-5
relative / absolute; loss to 1e-5 relative and each parameter block's
gradient to 1e-4 relative L2 (FP32 kernels against the float64 oracle).
Gain: after training on views generated from the bundle's reference, the
network's top-M directions (M = 1/8 of the directions) hold the exhaustive
E-step's best direction for at least 1.5x the fraction that M random
directions would (M / ndir), and clearly more often than the untrained
network.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bundle(ds, m):
    from relion_gb300.estep import MlDeviceBundle
    b = MlDeviceBundle(m, device=0)
    for k, r in enumerate(ds.refs):
        b.setup_projector(k, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    return b


def _need_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_features_match_oracle():
    _need_cuda()
    from oracle import posenet_oracle as po
    from relion_gb300 import datagen
    from relion_gb300.posenet import PoseProposer
    ds = datagen.Dataset("cfg0_box64", seed=3, n_particles=16)
    m = ds.model(precision=1)
    b = _bundle(ds, m)
    net = PoseProposer(b, nangle=24, max_batch=8, seed=2)  # two chunks of 8
    batch = ds.particles(0, 16)
    fg = net.features(batch["fimg"])
    xy, minv = net.pixels()
    fo = po.features(batch["fimg"], xy, minv, net.nring, net.nangle)
    net.close()
    b.close()
    assert np.count_nonzero(fo) > fo.size // 2
    np.testing.assert_allclose(fg, fo, rtol=1e-5, atol=1e-5)


def test_loss_grad_match_oracle():
    _need_cuda()
    from oracle import posenet_oracle as po
    from relion_gb300 import datagen
    from relion_gb300.posenet import PoseProposer
    ds = datagen.Dataset("cfg0_box64", seed=4, n_particles=4)
    m = ds.model(precision=1)
    b = _bundle(ds, m)
    net = PoseProposer(b, nangle=24, c1=8, c2=12, max_batch=8, seed=5)
    H, W, C1, C2, ND = net.nring, net.nangle, net.c1, net.c2, net.ndir
    g = np.random.default_rng(9)
    p = net.get_params().astype(np.float64)
    o = po.layout(H, W, C1, C2, ND)
    p[o["b1"]:o["w2"]] = 0.1
    p[o["b2"]:o["w3"]] = 0.1
    p[o["b3"]:] = g.normal(0, 0.1, ND)
    net.set_params(p.astype(np.float32))
    p32 = net.get_params().astype(np.float64)
    feat = g.normal(0, 1, (8, H * W)).astype(np.float32)
    t = (g.random((8, ND)) ** 4).astype(np.float32)
    t /= t.sum(axis=1, keepdims=True)
    lg, gg = net.loss_grad(feat, t)
    lo, go = po.loss_grad(p32, feat.astype(np.float64), t.astype(np.float64), H, W, C1, C2, ND)
    net.close()
    b.close()
    assert abs(lg - lo) <= 1e-5 * abs(lo)
    names = ["w1", "b1", "w2", "b2", "w3", "b3", "n"]
    for k, nxt in zip(names[:-1], names[1:]):
        a, r = gg[o[k]:o[nxt]], go[o[k]:o[nxt]]
        err = np.linalg.norm(a - r) / max(np.linalg.norm(r), 1e-30)
        assert err <= 1e-4, (k, err)


def _best_dirs(b, res):
    ih = np.asarray(res["best_ihidden_over"]) // (b.nover_rot * b.nover_trans)
    return (ih // b.ntrans // b.npsi) % b.ndir


def test_training_gain():
    _need_cuda()
    from relion_gb300 import datagen
    from relion_gb300.estep import MlOptimiserCuda
    from relion_gb300.posenet import PoseProposer
    ds = datagen.Dataset("cfg0_box64", seed=7, n_particles=512)
    m = ds.model(precision=1)
    b = _bundle(ds, m)
    pool = ds.particles(0, 256)["fctf"]
    test = ds.particles(256, 256)
    w = MlOptimiserCuda(b)
    best = _best_dirs(b, w.do_expectation_some_particles(test))
    w.close()
    net = PoseProposer(b, nangle=24, max_batch=256, seed=1)
    M = net.ndir // 8
    idx0, _ = net.propose(test["fimg"], M)
    loss = net.train(pool, steps=1500, batch=256, lr=2e-3)
    idx1, prob1 = net.propose(test["fimg"], M)
    ndir = net.ndir
    net.close()
    b.close()
    r0 = float(np.mean([best[i] in idx0[i] for i in range(len(best))]))
    r1 = float(np.mean([best[i] in idx1[i] for i in range(len(best))]))
    print("posenet: M %d of %d directions, recall untrained %.3f trained %.3f (uniform %.3f), loss %.3f" %
          (M, ndir, r0, r1, M / ndir, loss))
    assert np.all(np.diff(prob1, axis=1) <= 0)
    assert r1 >= 1.5 * M / ndir
    assert r1 >= r0 + 0.1


def test_block_probs_and_target_training():
    # tempered block probabilities against the oracle's softmax of the
    # network's logits, and a few steps on given target distributions lower
    # the loss on them (training on the E-step's own posteriors)
    _need_cuda()
    from oracle import posenet_oracle as po
    from relion_gb300 import datagen
    from relion_gb300.posenet import PoseProposer
    ds = datagen.Dataset("cfg0_box64", seed=5, n_particles=32)
    m = ds.model(precision=1)
    b = _bundle(ds, m)
    net = PoseProposer(b, nangle=12, c1=4, c2=6, max_batch=32, seed=2)
    batch = ds.particles(0, 32)
    feat = net.features(batch["fimg"])
    H, W, C1, C2, ND = net.nring, net.nangle, net.c1, net.c2, net.ndir
    params = net.get_params().astype(np.float64)
    for t, dpb in ((1.0, 1), (2.5, 4)):
        got = net.block_probs(batch["fimg"], dpb, t)
        logits = po.forward(params, feat.astype(np.float64), H, W, C1, C2, ND)["logits"] / t
        p = np.exp(logits - logits.max(axis=1, keepdims=True))
        p /= p.sum(axis=1, keepdims=True)
        want = p.reshape(len(p), ND // dpb, dpb).sum(axis=2)
        assert np.max(np.abs(got - want)) <= 1e-5
    target = np.zeros((32, ND), np.float32)
    target[np.arange(32), np.arange(32) % ND] = 1.0
    l0, _ = net.loss_grad(feat, target)
    net.train_targets(batch["fimg"], target, steps=50, batch=16, lr=1e-2)
    l1, _ = net.loss_grad(feat, target)
    print("target loss", l0, "->", l1)
    assert l1 < 0.5 * l0
    net.close()
    b.close()


def test_device_images_equal_host_images():
    """The proposer reads prepared images in device memory in place: the
    features, block probabilities and proposals equal those of the same
    images passed from the host, bit for bit."""
    _need_cuda()
    import torch
    from relion_gb300 import datagen
    from relion_gb300.posenet import PoseProposer
    ds = datagen.Dataset("cfg0_box64", seed=5, n_particles=12)
    b = _bundle(ds, ds.model(precision=1))
    net = PoseProposer(b, nangle=24, max_batch=8, seed=2)  # two chunks
    fimg = np.ascontiguousarray(ds.particles(0, 12)["fimg"], dtype=np.complex64)
    dev = torch.from_numpy(fimg).to("cuda")
    np.testing.assert_array_equal(net.features(dev), net.features(fimg))
    np.testing.assert_array_equal(net.block_probs(dev, 4, 1.5), net.block_probs(fimg, 4, 1.5))
    ih, ph = net.propose(fimg, 5)
    idv, pdv = net.propose(dev, 5)
    np.testing.assert_array_equal(idv, ih)
    np.testing.assert_array_equal(pdv, ph)
    net.close()
    b.close()


def test_top_blocks_on_device_match_host_selection():
    """gbr_posenet_propose_blocks: the device selection of the m most probable
    blocks equals a stable host sort of gbr_posenet_block_probs, and the
    mass their summed probability."""
    _need_cuda()
    from relion_gb300 import datagen
    from relion_gb300.posenet import PoseProposer
    ds = datagen.Dataset("cfg0_box64", seed=6, n_particles=20)
    b = _bundle(ds, ds.model(precision=1))
    net = PoseProposer(b, nangle=24, max_batch=8, seed=3)  # three chunks
    fimg = ds.particles(0, 20)["fimg"]
    for dpb, t, m in ((4, 1.7, 5), (1, 1.0, 12)):
        bp = net.block_probs(fimg, dpb, t)
        want = np.argsort(-bp, axis=1, kind="stable")[:, :m]
        idx, mass = net.propose_blocks(fimg, dpb, t, m)
        np.testing.assert_array_equal(idx, want)
        np.testing.assert_allclose(mass, np.take_along_axis(bp, want, 1).sum(1), rtol=1e-5)
    net.close()
    b.close()
