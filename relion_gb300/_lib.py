"""ctypes binding of libgbrelion (include/gbrelion.h).

The library is the only compute path: if it is missing or cannot be
loaded, every call raises GbrError; there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

I64, F64, P = C.c_int64, C.c_double, C.c_void_p

GBR_OK, GBR_ERR_INVALID, GBR_ERR_CUDA, GBR_ERR_OOM = 0, -1, -2, -3
GBR_ERR_NUMERICAL, GBR_ERR_STATE, GBR_ERR_UNSUPPORTED = -4, -5, -6
PREC_FP32, PREC_BF16 = 0, 1


class GbrError(RuntimeError):
    """A libgbrelion call failed (status and the library's error text)."""

    def __init__(self, status, text):
        super().__init__("libgbrelion status %d: %s" % (status, text))
        self.status = status


class ModelDesc(C.Structure):
    _fields_ = [(n, I64) for n in (
        "ori_size", "nr_classes", "current_size", "coarse_size", "padding_factor",
        "healpix_order", "adaptive_oversampling", "maximum_significants", "sigma2_len",
        "do_scale_correction", "do_norm_correction", "do_map", "precision", "ref_dim")] + \
        [(n, F64) for n in (
            "pixel_size", "psi_step", "offset_range", "offset_step", "adaptive_fraction",
            "sigma2_fudge", "sigma2_offset", "avg_norm_correction")]


class ParticleBatch(C.Structure):
    _fields_ = [("n", I64), ("device_resident", I64), ("fimg", P), ("fimg_nomask", P),
                ("fctf", P), ("power_img", P), ("old_offset", P), ("prior", P),
                ("highres_Xi2", P), ("norm_correction", P), ("scale", P)]


class ParticleResult(C.Structure):
    _fields_ = [(n, F64) for n in (
        "rot", "tilt", "psi", "xoff", "yoff", "cls", "pmax", "dLL", "norm", "nr_sign",
        "coarse_min_diff2", "coarse_sum_weight", "coarse_significant_weight",
        "fine_min_diff2", "fine_sum_weight", "fine_significant_weight")] + \
        [("best_ihidden_over", I64), ("n_fine", I64)]


class Wsum(C.Structure):
    _fields_ = [("sigma2_noise", P), ("pdf_class", P), ("pdf_direction", P)] + \
        [(n, F64) for n in ("sigma2_offset", "sumw_group", "LL", "ave_Pmax",
                            "avg_norm_correction", "wsum_signal_product",
                            "wsum_reference_power", "reserved_")]


class OpticsDesc(C.Structure):
    _fields_ = [(n, F64) for n in ("kV", "Cs", "Q0", "particle_diameter", "width_mask_edge", "reserved_")]


class ImageBatch(C.Structure):
    _fields_ = [("n", I64), ("device_resident", I64)] + \
        [(n, P) for n in ("images", "old_offset", "prior", "norm_correction", "scale", "ctf")]


class MrcHeader(C.Structure):
    _fields_ = [(n, I64) for n in ("nx", "ny", "nz", "mode", "nsymbt", "swapped")] + \
        [("pixel_size", F64), ("data_offset", I64)]


class ReconParams(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("max_iter_preweight", "do_map", "skip_gridding", "minres_map")] + \
        [(n, F64) for n in ("tau2_fudge", "normalise")]


class PosenetDesc(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("nring", "nangle", "c1", "c2", "max_batch", "reserved")] + \
        [("seed", C.c_uint64)]


EXPORTS = {
    "gbr_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "gbr_version": (C.c_char_p, []),
    "gbr_bundle_create": (C.c_int, [C.POINTER(ModelDesc), C.c_int, C.POINTER(P)]),
    "gbr_projector_upload": (C.c_int, [P, I64, P, I64, I64, I64, I64, I64, I64, I64]),
    "gbr_model_set_arrays": (C.c_int, [P, P, P, P, P]),
    "gbr_model_set_class_offsets": (C.c_int, [P, P]),
    "gbr_bundle_reserve": (C.c_int, [P, C.c_size_t]),
    "gbr_worker_create": (C.c_int, [P, C.POINTER(P)]),
    "gbr_worker_set_debug": (C.c_int, [P, C.c_int]),
    "gbr_worker_set_option": (C.c_int, [P, C.c_int, I64]),
    "gbr_expect_batch": (C.c_int, [P, C.POINTER(ParticleBatch), P]),
    "gbr_orientation_blocks": (C.c_int, [P, C.POINTER(I64), C.POINTER(I64), C.POINTER(I64)]),
    "gbr_expect_batch_blocks": (C.c_int, [P, C.POINTER(ParticleBatch), P, I64, P]),
    "gbr_bundle_set_optics": (C.c_int, [P, C.POINTER(OpticsDesc)]),
    "gbr_prepare_images": (C.c_int, [P, C.POINTER(ImageBatch), P, P, P, P, P, P]),
    "gbr_expect_images": (C.c_int, [P, C.POINTER(ImageBatch), P]),
    "gbr_mrc_read_header": (C.c_int, [C.c_char_p, C.POINTER(MrcHeader)]),
    "gbr_mrc_read_images": (C.c_int, [C.c_char_p, I64, I64, P, C.c_int]),
    "gbr_mrc_write_stack": (C.c_int, [C.c_char_p, P, I64, I64, I64, F64]),
    "gbr_star_read": (C.c_int, [C.c_char_p, C.POINTER(P)]),
    "gbr_star_num_blocks": (I64, [P]),
    "gbr_star_block_info": (C.c_int, [P, I64, C.c_char_p, C.c_size_t, C.POINTER(I64), C.POINTER(I64),
                                      C.POINTER(C.c_int)]),
    "gbr_star_column_name": (C.c_int, [P, I64, I64, C.c_char_p, C.c_size_t]),
    "gbr_star_column_double": (C.c_int, [P, I64, C.c_char_p, P]),
    "gbr_star_value_string": (C.c_int, [P, I64, C.c_char_p, I64, C.c_char_p, C.c_size_t]),
    "gbr_star_free": (None, [P]),
    "gbr_sampling_sizes": (C.c_int, [P] + [C.POINTER(I64)] * 5),
    "gbr_worker_debug_fetch": (I64, [P, C.c_int, I64, P, I64]),
    "gbr_backprojector_dims": (C.c_int, [P] + [C.POINTER(I64)] * 6),
    "gbr_backprojector_download": (C.c_int, [P, I64, P, P]),
    "gbr_backprojector_upload": (C.c_int, [P, I64, P, P]),
    "gbr_backprojector_symmetrise": (C.c_int, [P, I64]),
    "gbr_update_ssnr": (C.c_int, [P, I64, F64, P, P, P, P, P, C.c_int, C.c_int]),
    "gbr_reconstruct": (C.c_int, [P, I64, P, P, P]),
    "gbr_projector_from_map": (C.c_int, [P, I64, P, I64, C.c_int, I64, P]),
    "gbr_fsc": (C.c_int, [P, P, P, P]),
    "gbr_stage_images": (C.c_int, [P, P]),
    "gbr_posenet_create": (C.c_int, [P, C.POINTER(PosenetDesc), C.POINTER(P)]),
    "gbr_posenet_destroy": (C.c_int, [P]),
    "gbr_posenet_sizes": (C.c_int, [P, P, P, P, P]),
    "gbr_posenet_pixels": (C.c_int, [P, P, P]),
    "gbr_posenet_get_params": (C.c_int, [P, P]),
    "gbr_posenet_set_params": (C.c_int, [P, P]),
    "gbr_posenet_features": (C.c_int, [P, P, I64, P]),
    "gbr_posenet_loss_grad": (C.c_int, [P, P, P, I64, P, P]),
    "gbr_posenet_train": (C.c_int, [P, P, I64, I64, I64, F64, P]),
    "gbr_posenet_propose": (C.c_int, [P, P, I64, I64, P, P]),
    "gbr_posenet_propose_blocks": (C.c_int, [P, P, I64, I64, F64, I64, P, P]),
    "gbr_posenet_train_targets": (C.c_int, [P, P, P, I64, I64, I64, F64, P]),
    "gbr_posenet_block_probs": (C.c_int, [P, P, I64, I64, F64, P]),
    "gbr_recon_set_precision": (C.c_int, [P, C.c_int]),
    "gbr_projector_download": (C.c_int, [P, I64, P, P]),
    "gbr_wsum_download": (C.c_int, [P, C.POINTER(Wsum)]),
    "gbr_wsum_download_class_offsets": (C.c_int, [P, P]),
    "gbr_bundle_reset_wsum": (C.c_int, [P]),
    "gbr_worker_stage_times": (C.c_int, [P, P, I64, C.POINTER(I64)]),
    "gbr_worker_launch_count": (C.c_int, [P, C.POINTER(I64)]),
    "gbr_worker_graph_stats": (C.c_int, [P, C.POINTER(I64), C.POINTER(I64)]),
    "gbr_measure_fp32_peak": (C.c_int, [C.c_int, C.POINTER(F64)]),
    "gbr_significance_threshold_noalloc": (C.c_int, [P, I64, I64, F64, P, P, P]),
    "gbr_worker_destroy": (C.c_int, [P]),
    "gbr_bundle_destroy": (C.c_int, [P]),
}

_LIB = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libgbrelion.so (building it first if it is absent)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise GbrError(GBR_ERR_STATE, "libgbrelion.so not built: %s" % path)
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def last_error():
    buf = C.create_string_buffer(4096)
    load().gbr_last_error(buf, 4096)
    return buf.value.decode(errors="replace")


def check(status):
    if status < 0:
        raise GbrError(int(status), last_error())
    return status


def ptr(a):
    """Address of a C-contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data


def as_f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)
