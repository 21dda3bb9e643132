"""Python mirror of the reference's accelerated E-step surface.

The reference drives its GPU E-step through MlDeviceBundle (per device:
projectors, backprojectors, coarse projection plans) and MlOptimiserCuda
(per host thread: doThreadExpectationSomeParticles), see
src/acc/cuda/cuda_ml_optimiser.h:18-146 and src/ml_optimiser.cpp:3575-3868.
These classes keep those names and call libgbrelion's C ABI; the parity
tests and bench.py use them.  Every computation happens in the CUDA
library: there is no Python or CPU fallback.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, ptr


class MlDeviceBundle:
    """Device state of one iteration: model, pose grid, projector/backprojector.

    `model` is a dict with the gbr_model_desc fields plus the arrays
    sigma2_noise, pdf_class, pdf_direction (and data_vs_prior for --scale).
    """

    def __init__(self, model, device=0):
        self.lib = _lib.load()
        d = _lib.ModelDesc()
        for name, _ in _lib.ModelDesc._fields_:
            if name in model:
                setattr(d, name, model[name])
        self.desc = d
        h = C.c_void_p()
        check(self.lib.gbr_bundle_create(C.byref(d), int(device), C.byref(h)))
        self.h = h
        sz = [C.c_int64() for _ in range(5)]
        check(self.lib.gbr_sampling_sizes(h, *[C.byref(s) for s in sz]))
        self.ndir, self.npsi, self.ntrans, self.nover_rot, self.nover_trans = [s.value for s in sz]
        self.nr_classes = int(model["nr_classes"])
        self.device = int(device)
        self.ori_size = int(model["ori_size"])
        self._keep = []
        s2 = _lib.as_f64(model["sigma2_noise"])
        pc = _lib.as_f64(model["pdf_class"])
        pdir = _lib.as_f64(model["pdf_direction"])
        dvp = model.get("data_vs_prior")
        dvp = _lib.as_f64(dvp) if dvp is not None else None
        check(self.lib.gbr_model_set_arrays(h, ptr(s2), ptr(pc), ptr(pdir), ptr(dvp)))
        self.ref_dim = int(model.get("ref_dim", 3) or 3)
        if self.ref_dim == 2 and model.get("prior_offset_class") is not None:
            self.set_class_offsets(model["prior_offset_class"])

    # optics group and mask of the image preparation
    def set_optics(self, kV=300.0, Cs=2.7, Q0=0.1, particle_diameter=200.0, width_mask_edge=5.0):
        o = _lib.OpticsDesc(kV, Cs, Q0, particle_diameter, width_mask_edge, 0.0)
        check(self.lib.gbr_bundle_set_optics(self.h, C.byref(o)))

    # 2D classification: mymodel.prior_offset_class [K][2]
    def set_class_offsets(self, prior_offset_class):
        a = _lib.as_f64(np.asarray(prior_offset_class).reshape(self.nr_classes, 2))
        check(self.lib.gbr_model_set_class_offsets(self.h, ptr(a)))

    # wsum_model.prior_offset_class accumulated since the last reset
    def get_class_offsets(self):
        out = np.zeros((self.nr_classes, 2))
        check(self.lib.gbr_wsum_download_class_offsets(self.h, out.ctypes.data))
        return out

    # AccProjector::setMdlDim + initMdl
    def setup_projector(self, iclass, data, yinit, zinit, r_max, padding_factor):
        data = np.ascontiguousarray(data, dtype=np.complex64)
        zdim, ydim, xdim = data.shape
        check(self.lib.gbr_projector_upload(self.h, int(iclass), data.ctypes.data, xdim, ydim, zdim,
                                            int(yinit), int(zinit), int(r_max), int(padding_factor)))

    def orientation_blocks(self):
        """(number of blocks, directions per block, projection rows per block)
        of the restricted coarse pass (gbr_orientation_blocks)."""
        v = [C.c_int64() for _ in range(3)]
        check(self.lib.gbr_orientation_blocks(self.h, *[C.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def reserve(self, nbytes):
        check(self.lib.gbr_bundle_reserve(self.h, int(nbytes)))

    def backprojector_dims(self):
        v = [C.c_int64() for _ in range(6)]
        check(self.lib.gbr_backprojector_dims(self.h, *[C.byref(x) for x in v]))
        return [x.value for x in v]

    # AccBackprojector::getMdlData
    def get_mdl_data(self, iclass):
        xd, yd, zd, _, _, _ = self.backprojector_dims()
        data = np.zeros((zd, yd, xd), dtype=np.complex128)
        weight = np.zeros((zd, yd, xd), dtype=np.float64)
        check(self.lib.gbr_backprojector_download(self.h, int(iclass), data.ctypes.data, weight.ctypes.data))
        return data, weight

    def set_mdl_data(self, iclass, data, weight):
        """Replace one class's volumes (e.g. with the sums over all ranks)."""
        xd, yd, zd, _, _, _ = self.backprojector_dims()
        d = np.ascontiguousarray(data, dtype=np.complex128).reshape(zd, yd, xd)
        w = np.ascontiguousarray(weight, dtype=np.float64).reshape(zd, yd, xd)
        check(self.lib.gbr_backprojector_upload(self.h, int(iclass), d.ctypes.data, w.ctypes.data))

    # BackProjector::symmetrise (C1: enforceHermitianSymmetry)
    def symmetrise(self, iclass):
        check(self.lib.gbr_backprojector_symmetrise(self.h, int(iclass)))

    # BackProjector::updateSSNRarrays
    def update_ssnr_arrays(self, iclass, tau2_fudge, tau2, fsc=None, update_tau2_with_fsc=False,
                           is_whole_instead_of_half=False):
        """Returns dict(tau2, sigma2, data_vs_prior, fourier_coverage), [ori/2+1] each."""
        ns = self.ori_size // 2 + 1
        t = np.array(tau2, dtype=np.float64).reshape(ns).copy()
        out = [np.zeros(ns) for _ in range(3)]
        f = np.zeros(ns) if fsc is None else np.ascontiguousarray(fsc, dtype=np.float64)
        check(self.lib.gbr_update_ssnr(self.h, int(iclass), float(tau2_fudge), t.ctypes.data,
                                       *[o.ctypes.data for o in out], f.ctypes.data, int(update_tau2_with_fsc),
                                       int(is_whole_instead_of_half)))
        return dict(tau2=t, sigma2=out[0], data_vs_prior=out[1], fourier_coverage=out[2])

    def set_recon_precision(self, fp32):
        """Reconstruction-side transforms in FP32 (True) or FP64 (False, default)."""
        check(self.lib.gbr_recon_set_precision(self.h, 1 if fp32 else 0))

    # BackProjector::reconstruct
    def reconstruct(self, iclass, max_iter_preweight=10, do_map=False, tau2=None, tau2_fudge=1.0, normalise=1.0,
                    minres_map=5, skip_gridding=True, to_host=True):
        """Real-space map [ori]^ref_dim (mymodel.Iref[iclass]); with
        to_host=False the map stays on the device only (returns None)."""
        p = _lib.ReconParams(max_iter_preweight=int(max_iter_preweight), do_map=int(do_map),
                             skip_gridding=int(skip_gridding), minres_map=int(minres_map),
                             tau2_fudge=float(tau2_fudge), normalise=float(normalise))
        vol = np.zeros((self.ori_size,) * self.ref_dim) if to_host else None
        t = None if tau2 is None else np.ascontiguousarray(tau2, dtype=np.float64)
        check(self.lib.gbr_reconstruct(self.h, int(iclass), C.byref(p), None if t is None else t.ctypes.data,
                                       None if vol is None else vol.ctypes.data))
        return vol

    # Projector::computeFourierTransformMap (MlModel::setFourierTransformMaps)
    def set_fourier_transform_map(self, iclass, vol, current_size, do_gridding=True, min_ires=-1):
        """Fill class iclass's projector from a real-space map (None: the map
        the last reconstruct left on the device); returns its power spectrum."""
        v = None
        if vol is not None:
            v = np.ascontiguousarray(vol, dtype=np.float64)
            if v.shape != (self.ori_size,) * self.ref_dim:
                raise ValueError("map must be %s" % ((self.ori_size,) * self.ref_dim,))
        ps = np.zeros(self.ori_size // 2 + 1)
        check(self.lib.gbr_projector_from_map(self.h, int(iclass), None if v is None else v.ctypes.data,
                                              int(current_size), int(do_gridding), int(min_ires), ps.ctypes.data))
        return ps

    def get_projector(self, iclass):
        """(padded Fourier reference as complex64 [zdim][ydim][xdim], geometry dict)."""
        dims = np.zeros(7, np.int64)
        check(self.lib.gbr_projector_download(self.h, int(iclass), None, dims.ctypes.data))
        xd, yd, zd = (int(x) for x in dims[:3])
        data = np.zeros((zd, yd, xd), np.complex64)
        check(self.lib.gbr_projector_download(self.h, int(iclass), data.ctypes.data, dims.ctypes.data))
        geom = dict(zip(("xdim", "ydim", "zdim", "yinit", "zinit", "r_max", "pad"), (int(x) for x in dims)))
        return data, geom

    # getFSC
    def fsc(self, map1, map2):
        a = np.ascontiguousarray(map1, dtype=np.float64)
        b = np.ascontiguousarray(map2, dtype=np.float64)
        out = np.zeros(self.ori_size // 2 + 1)
        check(self.lib.gbr_fsc(self.h, a.ctypes.data, b.ctypes.data, out.ctypes.data))
        return out

    def get_wsum(self):
        s2 = np.zeros(self.ori_size // 2 + 1)
        pc = np.zeros(self.nr_classes)
        pdir = np.zeros(self.nr_classes * self.ndir)
        w = _lib.Wsum()
        w.sigma2_noise, w.pdf_class, w.pdf_direction = ptr(s2), ptr(pc), ptr(pdir)
        check(self.lib.gbr_wsum_download(self.h, C.byref(w)))
        out = {k: getattr(w, k) for k, _ in _lib.Wsum._fields_[3:] if k != "reserved_"}
        out.update(sigma2_noise=s2, pdf_class=pc, pdf_direction=pdir.reshape(self.nr_classes, self.ndir))
        return out

    def reset_wsum(self):
        check(self.lib.gbr_bundle_reset_wsum(self.h))

    def close(self):
        if self.h:
            self.lib.gbr_bundle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


RESULT_FIELDS = [n for n, _ in _lib.ParticleResult._fields_]
# numpy image of gbr_particle_result: the library writes the rows in place
RESULT_DTYPE = np.dtype([(n, np.int64 if t is _lib.I64 else np.float64)
                         for n, t in _lib.ParticleResult._fields_])
assert RESULT_DTYPE.itemsize == C.sizeof(_lib.ParticleResult)


# gbr_expect_batch_blocks: a block list starting with this scores every block
ALL_BLOCKS = -2

# gbr_worker_set_option selectors (include/gbrelion.h, gbr_worker_option)
WORKER_OPTIONS = dict(debug=1, fine_mode=2, coarse_rows=3, cand_cap=4, cand_buf=5, batch_cap=6, tile_group=7,
                      keep_a=8, pair=9, bp_flush=10, graph=11, bp_direct=12)
FINE_MODES = dict(auto=0, dense=1, sparse=2)
COARSE_ROWS = dict(skip=0, full=1)


class MlOptimiserCuda:
    """One E-step worker (stream + batch buffers) on a bundle.

    Keyword options (gbr_worker_set_option): fine_mode ("auto", "dense",
    "sparse"), coarse_rows ("skip", "full"), cand_cap, cand_buf, batch_cap
    (particles per pass of a call), tile_group (orientation tiles of 128 rows
    per group of the coarse tensor-core kernel's tile order), keep_a (1:
    projection tiles read with an L2 keep policy), pair (1: the coarse
    cross term on SM pairs, tcgen05 cta_group::2) and bp_flush (particles
    collected in the FP32 staging volumes before they are added into the
    FP64 volumes; 0: after every pass) and graph (1, default: the coarse
    segment of a pass captured as a CUDA graph and replayed; 0: launched
    directly) and bp_direct (1: the sparse fine pass inserts each job's
    weighted slices into the staging volumes from the weighted sums)."""

    def __init__(self, bundle, debug=False, **options):
        self.bundle = bundle
        self.lib = bundle.lib
        h = C.c_void_p()
        check(self.lib.gbr_worker_create(bundle.h, C.byref(h)))
        self.h = h
        if debug:
            check(self.lib.gbr_worker_set_debug(h, 1))
        for k, v in options.items():
            if v is not None:
                self.set_option(k, v)

    def set_option(self, name, value):
        if name not in WORKER_OPTIONS:
            raise ValueError("unknown worker option %r" % name)
        if name == "fine_mode" and isinstance(value, str):
            value = FINE_MODES[value]
        if name == "coarse_rows" and isinstance(value, str):
            value = COARSE_ROWS[value]
        check(self.lib.gbr_worker_set_option(self.h, WORKER_OPTIONS[name], int(value)))

    def do_expectation_some_particles(self, batch, blocks=None):
        """Run the E-step on a batch (dict of host arrays, or device pointers).

        Host batch keys: fimg, fimg_nomask (complex [n][cur][cur/2+1]), fctf
        (float [n][cur][cur/2+1]), power_img [n][ori/2+1], old_offset [n][2],
        prior [n][2], highres_Xi2 [n], norm_correction [n], scale [n].
        blocks: optional int32 [n][m] orientation blocks each particle scores
        in the coarse pass (gbr_expect_batch_blocks; a row starting with
        ALL_BLOCKS is searched exhaustively).
        Returns a structured numpy array of gbr_particle_result rows.
        """
        n = int(batch["n"]) if "n" in batch else len(batch["fimg"])
        b = _lib.ParticleBatch()
        b.n = n
        keep = []
        if batch.get("device_resident"):
            b.device_resident = 1
            for k in ("fimg", "fimg_nomask", "fctf", "power_img", "old_offset", "prior",
                      "highres_Xi2", "norm_correction", "scale"):
                setattr(b, k, int(batch[k]))
        else:
            def f32c(a):
                a = np.ascontiguousarray(a, dtype=np.complex64)
                keep.append(a)
                return a.ctypes.data

            def arr(a, dt):
                a = np.ascontiguousarray(a, dtype=dt)
                keep.append(a)
                return a.ctypes.data
            b.fimg = f32c(batch["fimg"])
            b.fimg_nomask = f32c(batch["fimg_nomask"])
            b.fctf = arr(batch["fctf"], np.float32)
            for k in ("power_img", "old_offset", "prior", "highres_Xi2", "norm_correction", "scale"):
                setattr(b, k, arr(batch[k], np.float64))
        out = np.zeros(n, dtype=RESULT_DTYPE)
        if blocks is None:
            check(self.lib.gbr_expect_batch(self.h, C.byref(b), out.ctypes.data))
        else:
            bl = np.ascontiguousarray(blocks, dtype=np.int32)
            if bl.ndim != 2 or bl.shape[0] != n:
                raise ValueError("blocks must be [n][m]")
            check(self.lib.gbr_expect_batch_blocks(self.h, C.byref(b), bl.ctypes.data, bl.shape[1],
                                                   out.ctypes.data))
        return out

    def _image_batch(self, batch, keep):
        b = _lib.ImageBatch()
        b.n = len(batch["images"])

        def arr(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a.ctypes.data
        b.images = arr(batch["images"], np.float32)
        for k in ("old_offset", "prior", "norm_correction", "scale", "ctf"):
            setattr(b, k, arr(batch[k], np.float64))
        return b

    def prepare_images(self, batch):
        """getFourierTransformsAndCtfs for a batch of host images (dict:
        images [n][ori][ori], old_offset, prior [n][2], norm_correction,
        scale [n], ctf [n][6]); returns the E-step inputs as numpy arrays
        (computed on the device, copied back)."""
        import torch
        keep = []
        b = self._image_batch(batch, keep)
        n, cur = b.n, int(self.bundle.desc.current_size)
        X, half = cur // 2 + 1, self.bundle.ori_size // 2 + 1
        dev = torch.device("cuda", self.bundle.device)
        out = dict(fimg=torch.empty((n, cur, X), dtype=torch.complex64, device=dev),
                   fimg_nomask=torch.empty((n, cur, X), dtype=torch.complex64, device=dev),
                   fctf=torch.empty((n, cur, X), dtype=torch.float32, device=dev),
                   power_img=torch.empty((n, half), dtype=torch.float64, device=dev),
                   highres_Xi2=torch.empty(n, dtype=torch.float64, device=dev),
                   old_offset=torch.empty((n, 2), dtype=torch.float64, device=dev))
        check(self.lib.gbr_prepare_images(self.h, C.byref(b), *[out[k].data_ptr() for k in (
            "fimg", "fimg_nomask", "fctf", "power_img", "highres_Xi2", "old_offset")]))
        return {k: v.cpu().numpy() for k, v in out.items()}

    def do_expectation_images(self, batch):
        """Image preparation and E-step of a batch of raw images in one call
        (gbr_expect_images); returns the result rows."""
        keep = []
        b = self._image_batch(batch, keep)
        out = np.zeros(b.n, dtype=RESULT_DTYPE)
        check(self.lib.gbr_expect_images(self.h, C.byref(b), out.ctypes.data))
        return out

    def stage_images(self, batch):
        """Start the upload of a host image batch into the worker's next
        staging slot (gbr_stage_images); a following do_expectation_images
        with the same batch uses it.  The images must already be a
        C-contiguous float32 array (ideally page-locked) that stays unchanged
        until then."""
        img = batch["images"]
        if not (isinstance(img, np.ndarray) and img.dtype == np.float32 and img.flags.c_contiguous):
            raise ValueError("stage_images needs C-contiguous float32 images (no temporary copy)")
        keep = []
        b = self._image_batch(batch, keep)
        check(self.lib.gbr_stage_images(self.h, C.byref(b)))

    def debug_fetch(self, what, i):
        cap = self.bundle.nr_classes * self.bundle.ndir * self.bundle.npsi * self.bundle.ntrans * \
            self.bundle.nover_rot * self.bundle.nover_trans
        buf = np.zeros(cap, dtype=np.int64 if what == 2 else np.float64)
        m = self.lib.gbr_worker_debug_fetch(self.h, int(what), int(i), buf.ctypes.data, cap)
        check(m)
        return buf[:m].copy()

    def stage_times(self):
        ms = np.zeros(16)
        n = C.c_int64()
        check(self.lib.gbr_worker_stage_times(self.h, ms.ctypes.data, 16, C.byref(n)))
        return ms[:n.value]

    def launch_count(self):
        n = C.c_int64()
        check(self.lib.gbr_worker_launch_count(self.h, C.byref(n)))
        return n.value

    def graph_stats(self):
        """(captures, replays) of the coarse segment's CUDA graph."""
        c, r = C.c_int64(), C.c_int64()
        check(self.lib.gbr_worker_graph_stats(self.h, C.byref(c), C.byref(r)))
        return c.value, r.value

    def close(self):
        if self.h:
            self.lib.gbr_worker_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


STAGES = ["prep", "norm_gemm", "cross_gemm", "weights_coarse", "sig_jobs", "diff2_fine",
          "weights_fine", "wsum", "backproject", "readback", "inputs", "host_final",
          "image_upload", "image_prep", "image_stage_copy", "image_stage_wait"]


def measure_fp32_peak(device=0):
    """Measured FP32 FMA throughput of the device in TFLOP/s."""
    lib = _lib.load()
    v = C.c_double()
    check(lib.gbr_measure_fp32_peak(int(device), C.byref(v)))
    return v.value
