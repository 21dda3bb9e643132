"""Learned pose proposal: a small convolutional network that proposes the
top-M coarse viewing directions of each particle (gbr_posenet_* in
libgbrelion).  No counterpart in the reference, whose coarse search is
exhaustive (src/acc/acc_ml_optimiser_impl.h:1016-1414 scores every coarse
orientation); the exhaustive search stays the fallback and the measure of the
proposals.

The network is trained on the device by the library's own forward, backward
and Adam kernels, on views the library generates from the bundle's current
reference (its coarse projection table: one row per coarse orientation, so
the direction label is exact), with CTFs drawn from a pool of particle CTFs
and complex Gaussian noise of the model's sigma2.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check


class PoseProposer:
    def __init__(self, bundle, nring=None, nangle=24, c1=16, c2=32, max_batch=512, seed=1):
        self.lib = _lib.load()
        self.bundle = bundle
        if nring is None:
            nring = int(bundle.desc.coarse_size) // 2
        d = _lib.PosenetDesc(int(nring), int(nangle), int(c1), int(c2), int(max_batch), 0, int(seed))
        h = C.c_void_p()
        check(self.lib.gbr_posenet_create(bundle.h, C.byref(d), C.byref(h)))
        self.h = h
        v = [C.c_int64() for _ in range(4)]
        check(self.lib.gbr_posenet_sizes(h, *[C.byref(x) for x in v]))
        self.nparams, self.nfeat, self.ndir, self.npix = [x.value for x in v]
        self.nring, self.nangle, self.c1, self.c2, self.max_batch = nring, nangle, c1, c2, max_batch

    def close(self):
        if self.h:
            check(self.lib.gbr_posenet_destroy(self.h))
            self.h = None

    def pixels(self):
        """Active coarse pixels (x, y) [npix][2] and their noise weights 1/(2 sigma2)."""
        xy = np.zeros((self.npix, 2), np.int32)
        minv = np.zeros(self.npix, np.float32)
        check(self.lib.gbr_posenet_pixels(self.h, xy.ctypes.data, minv.ctypes.data))
        return xy, minv

    def get_params(self):
        p = np.zeros(self.nparams, np.float32)
        check(self.lib.gbr_posenet_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32).reshape(self.nparams)
        check(self.lib.gbr_posenet_set_params(self.h, p.ctypes.data))

    class _Images:
        """Prepared images as the library takes them: a host array (complex64,
        contiguous) or a CUDA tensor (complex64, contiguous; no host copy)."""

        def __init__(self, fimg):
            if hasattr(fimg, "data_ptr") and getattr(fimg, "is_cuda", False):
                import torch
                if fimg.dtype != torch.complex64 or not fimg.is_contiguous():
                    raise ValueError("device images must be contiguous complex64")
                self.keep, self.ptr, self.n = fimg, fimg.data_ptr(), int(fimg.shape[0])
            else:
                a = np.ascontiguousarray(fimg, dtype=np.complex64)
                self.keep, self.ptr, self.n = a, a.ctypes.data, len(a)

        def __len__(self):
            return self.n

    @staticmethod
    def _fimg(fimg):
        return PoseProposer._Images(fimg)

    def features(self, fimg):
        f = self._fimg(fimg)
        out = np.zeros((len(f), self.nfeat), np.float32)
        check(self.lib.gbr_posenet_features(self.h, f.ptr, len(f), out.ctypes.data))
        return out

    def loss_grad(self, feat, target):
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        target = np.ascontiguousarray(target, dtype=np.float32)
        loss = C.c_double()
        g = np.zeros(self.nparams, np.float32)
        check(self.lib.gbr_posenet_loss_grad(self.h, feat.ctypes.data, target.ctypes.data, len(feat),
                                             C.byref(loss), g.ctypes.data))
        return loss.value, g

    def train(self, ctf_pool, steps, batch=256, lr=1e-3):
        """Adam steps on generated views; returns the mean loss of the last steps."""
        pool = np.ascontiguousarray(ctf_pool, dtype=np.float32)
        loss = C.c_double()
        check(self.lib.gbr_posenet_train(self.h, pool.ctypes.data, len(pool), int(steps), int(batch), float(lr),
                                         C.byref(loss)))
        return loss.value

    def train_targets(self, fimg, target, steps, batch=256, lr=1e-3):
        """Adam steps on particle images with target distributions over the
        directions (e.g. the E-step's own posteriors); returns the mean loss
        of the last steps."""
        f = self._fimg(fimg)
        t = np.ascontiguousarray(target, dtype=np.float32)
        if t.shape != (len(f), self.ndir):
            raise ValueError("target must be [n][ndir]")
        loss = C.c_double()
        check(self.lib.gbr_posenet_train_targets(self.h, f.ptr, t.ctypes.data, len(f), int(steps),
                                                 int(min(batch, len(f), self.max_batch)), float(lr),
                                                 C.byref(loss)))
        return loss.value

    def block_probs(self, fimg, dirs_per_block, temperature=1.0):
        """Probability of each block of dirs_per_block consecutive directions
        [n][ndir / dirs_per_block] under softmax(logits / temperature)."""
        f = self._fimg(fimg)
        out = np.zeros((len(f), self.ndir // int(dirs_per_block)), np.float32)
        check(self.lib.gbr_posenet_block_probs(self.h, f.ptr, len(f), int(dirs_per_block),
                                               float(temperature), out.ctypes.data))
        return out

    def propose_blocks(self, fimg, dirs_per_block, temperature, m):
        """The m most probable blocks of dirs_per_block directions [n][m]
        (most probable first, lower index first among equals) and their
        summed probability [n], selected on the device."""
        f = self._fimg(fimg)
        idx = np.zeros((len(f), m), np.int32)
        mass = np.zeros(len(f), np.float32)
        check(self.lib.gbr_posenet_propose_blocks(self.h, f.ptr, len(f), int(dirs_per_block), float(temperature),
                                                  int(m), idx.ctypes.data, mass.ctypes.data))
        return idx, mass

    def propose(self, fimg, m):
        """Top-m directions [n][m] (most probable first) and their probabilities."""
        f = self._fimg(fimg)
        idx = np.zeros((len(f), m), np.int32)
        prob = np.zeros((len(f), m), np.float32)
        check(self.lib.gbr_posenet_propose(self.h, f.ptr, len(f), int(m), idx.ctypes.data,
                                           prob.ctypes.data))
        return idx, prob


def best_directions(bundle, results):
    """Coarse direction (within its class) of each particle's best fine pose
    (gbr_particle_result.best_ihidden_over, the hidden-index packing of
    HealpixSampling::getPositionOversampledSamplingPoint)."""
    h = np.asarray(results["best_ihidden_over"], np.int64)
    r = h // (bundle.nover_rot * bundle.nover_trans) // bundle.ntrans
    return (r // bundle.npsi) % bundle.ndir


def direction_targets(bundle, results, smoothing=0.0):
    """Target distributions over the directions from an E-step's results:
    the posterior's mode (best pose's direction), optionally with a uniform
    share `smoothing`."""
    d = best_directions(bundle, results)
    t = np.full((len(d), bundle.ndir), smoothing / bundle.ndir, np.float32)
    t[np.arange(len(d)), d] += 1.0 - smoothing
    return t


class BlockProposer:
    """Orientation blocks of the restricted coarse pass from the network.

    The network's probabilities over directions are summed per block (the
    four sibling directions of one parent HEALPix pixel); each particle
    scores its `blocks` most probable blocks (in every class), and falls
    back to the exhaustive search (ALL_BLOCKS) when those carry less than
    `mass_threshold` of its probability.  Called with a batch's prepared
    images, returns the int32 [n][m] block lists of
    MlOptimiserCuda.do_expectation_some_particles(batch, blocks=...)."""

    def __init__(self, net, bundle, blocks, mass_threshold=0.9, temperature=1.0):
        self.net = net
        self.nblk, self.dpb, _ = bundle.orientation_blocks()
        self.K = bundle.nr_classes
        self.ndir = bundle.ndir
        self.per_class = self.ndir // self.dpb
        self.blocks = int(min(blocks, self.per_class))
        self.mass_threshold = float(mass_threshold)
        self.temperature = float(temperature)
        self.last = None

    def block_probabilities(self, fimg):
        return self.net.block_probs(fimg, self.dpb, self.temperature)

    def calibrate(self, fimg, best_dirs, temperatures=None):
        """Temperature of the network's softmax judged by the exhaustive
        search: the value minimising the negative log-likelihood of the
        blocks holding the exhaustive E-step's best directions on a held-out
        set of particles (temperature scaling; the network's ranking is
        unchanged, its probabilities, and with them the fallback decision,
        become calibrated).  Returns the chosen temperature."""
        if temperatures is None:
            temperatures = np.geomspace(0.25, 32.0, 29)
        logp = np.log(np.maximum(self.net.block_probs(fimg, 1, 1.0).astype(np.float64), 1e-38))
        best_blk = np.asarray(best_dirs) // self.dpb
        nll = []
        for t in temperatures:
            z = logp / t
            z -= z.max(axis=1, keepdims=True)
            p = np.exp(z)
            p /= p.sum(axis=1, keepdims=True)
            bp = p.reshape(len(p), self.per_class, self.dpb).sum(axis=2)
            nll.append(-np.mean(np.log(np.maximum(bp[np.arange(len(bp)), best_blk], 1e-300))))
        self.temperature = float(temperatures[int(np.argmin(nll))])
        return self.temperature

    def __call__(self, fimg):
        from .estep import ALL_BLOCKS
        # the `blocks` most probable blocks (most probable first) and their
        # mass, selected on the device
        order, mass = self.net.propose_blocks(fimg, self.dpb, self.temperature, self.blocks)
        mass = mass.astype(np.float64)
        out = np.concatenate([order + c * self.per_class for c in range(self.K)], axis=1).astype(np.int32)
        fallback = mass < self.mass_threshold
        out[fallback, 0] = ALL_BLOCKS
        self.last = dict(mass=mass, fallback=fallback)
        return out


class LearnedBlocks:
    """Proposer for relion_gb300.iteration.HalfSet: on each iteration's
    bundle the network is trained on views of the current reference (the
    first time `train_steps` Adam steps, later `finetune_steps` from the
    previous iteration's parameters), then each batch gets the blocks of a
    BlockProposer.  release() (called by HalfSet after its E-step) keeps the
    parameters and frees the network before its bundle is closed."""

    def __init__(self, blocks, mass_threshold=0.9, train_steps=1500, finetune_steps=300, lr=2e-3, **net_kw):
        self.blocks, self.mass_threshold = blocks, mass_threshold
        self.train_steps, self.finetune_steps, self.lr = train_steps, finetune_steps, lr
        self.net_kw = dict(nangle=24, max_batch=256, seed=1)
        self.net_kw.update(net_kw)
        self.net = self.bundle = self.params = self.bp = None
        self.fallback = []

    def __call__(self, bundle, batch):
        if self.bundle is not bundle:
            self.release()
            self.net = PoseProposer(bundle, **self.net_kw)
            steps = self.train_steps
            if self.params is not None:
                self.net.set_params(self.params)
                steps = self.finetune_steps
            self.net.train(batch["fctf"], steps=steps, batch=min(256, self.net.max_batch), lr=self.lr)
            self.bundle = bundle
            self.bp = BlockProposer(self.net, bundle, self.blocks, self.mass_threshold)
        out = self.bp(batch["fimg"])
        self.fallback.append(float(np.mean(self.bp.last["fallback"])))
        return out

    def release(self):
        if self.net is not None:
            self.params = self.net.get_params()
            self.net.close()
        self.net = self.bundle = self.bp = None
