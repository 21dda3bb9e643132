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

    @staticmethod
    def _fimg(fimg):
        return np.ascontiguousarray(fimg, dtype=np.complex64)

    def features(self, fimg):
        f = self._fimg(fimg)
        out = np.zeros((len(f), self.nfeat), np.float32)
        check(self.lib.gbr_posenet_features(self.h, f.ctypes.data, len(f), out.ctypes.data))
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

    def propose(self, fimg, m):
        """Top-m directions [n][m] (most probable first) and their probabilities."""
        f = self._fimg(fimg)
        idx = np.zeros((len(f), m), np.int32)
        prob = np.zeros((len(f), m), np.float32)
        check(self.lib.gbr_posenet_propose(self.h, f.ctypes.data, len(f), int(m), idx.ctypes.data,
                                           prob.ctypes.data))
        return idx, prob
