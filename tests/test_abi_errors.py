"""CPU checks of the C ABI's error convention (every gbr_* call returns 0 or
a negative gbr_status and leaves its text for gbr_last_error; the library
never aborts the caller), on inputs that fail before any device work:
malformed model descriptions, null handles and arguments, truncated or
foreign MRC files, missing STAR files and labels."""
import ctypes as C
import os

import numpy as np
import pytest

GBR_ERR_INVALID, GBR_ERR_CUDA = -1, -2


@pytest.fixture(scope="module")
def lib():
    from relion_gb300 import _lib
    return _lib


def test_bundle_create_rejects_bad_descriptions(lib):
    L = lib.load()
    d = lib.ModelDesc()
    h = C.c_void_p()
    assert L.gbr_bundle_create(None, 0, C.byref(h)) == GBR_ERR_INVALID
    assert L.gbr_bundle_create(C.byref(d), 0, C.byref(h)) == GBR_ERR_INVALID  # all sizes zero
    assert "invalid model description" in lib.last_error()
    # coarse size above the current size
    for k, v in dict(ori_size=64, nr_classes=1, current_size=20, coarse_size=24, padding_factor=2,
                     pixel_size=2.0, offset_step=2.0, offset_range=4.0, sigma2_len=33, healpix_order=1,
                     adaptive_oversampling=1, psi_step=30.0).items():
        setattr(d, k, v)
    assert L.gbr_bundle_create(C.byref(d), 0, C.byref(h)) == GBR_ERR_INVALID
    d.coarse_size = 20
    d.adaptive_oversampling = 2
    assert L.gbr_bundle_create(C.byref(d), 0, C.byref(h)) == -6  # GBR_ERR_UNSUPPORTED
    assert "oversampling" in lib.last_error()


def test_null_handles(lib):
    L = lib.load()
    assert L.gbr_backprojector_symmetrise(None, 0) == GBR_ERR_INVALID
    assert L.gbr_reconstruct(None, 0, None, None, None) == GBR_ERR_INVALID
    assert L.gbr_projector_from_map(None, 0, None, 28, 1, -1, None) == GBR_ERR_INVALID
    assert L.gbr_fsc(None, None, None, None) == GBR_ERR_INVALID
    assert L.gbr_backprojector_upload(None, 0, None, None) == GBR_ERR_INVALID
    assert L.gbr_bundle_destroy(None) == 0


def test_mrc_errors(lib, tmp_path):
    from relion_gb300 import io
    # truncated stack: header promises 4 images, the file holds 2.5
    data = np.zeros((4, 8, 8), np.float32)
    p = str(tmp_path / "t.mrcs")
    io.write_mrc_stack(p, data, 1.0)
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:1024 + int(2.5 * 8 * 8 * 4)])
    with pytest.raises(lib.GbrError) as e:
        io.read_mrc_images(p)
    assert e.value.status == GBR_ERR_INVALID
    # range beyond the stack
    io.write_mrc_stack(p, data, 1.0)
    with pytest.raises(lib.GbrError):
        io.read_mrc_images(p, 3, 2)
    # not an MRC file at all
    q = str(tmp_path / "x.mrc")
    open(q, "wb").write(b"not an mrc file")
    with pytest.raises(lib.GbrError):
        io.read_mrc_header(q)
    with pytest.raises(lib.GbrError):
        io.read_mrc_header(str(tmp_path / "missing.mrc"))


def test_star_errors(lib, tmp_path):
    from relion_gb300 import io
    with pytest.raises(lib.GbrError):
        io.StarFile(str(tmp_path / "missing.star"))
    p = tmp_path / "s.star"
    p.write_text("data_particles\n\nloop_\n_rlnImageName #1\n_rlnDefocusU #2\n1@a.mrcs 1.0\n")
    st = io.StarFile(str(p))
    # an absent label reads as the given default
    np.testing.assert_array_equal(st.column("particles", "rlnDefocusV", float, 7.0), [7.0])
    assert os.path.exists(str(p))


def test_posenet_null_arguments(lib):
    L = lib.load()
    h = C.c_void_p()
    d = lib.PosenetDesc(4, 12, 4, 4, 8, 0, 1)
    assert L.gbr_posenet_create(None, C.byref(d), C.byref(h)) == GBR_ERR_INVALID
    assert L.gbr_posenet_sizes(None, None, None, None, None) == GBR_ERR_INVALID
    assert L.gbr_posenet_train(None, None, 0, 1, 1, 1e-3, None) == GBR_ERR_INVALID
    assert L.gbr_posenet_propose(None, None, 0, 1, None, None) == GBR_ERR_INVALID
    assert L.gbr_posenet_loss_grad(None, None, None, 1, None, None) == GBR_ERR_INVALID
    assert L.gbr_posenet_destroy(None) == 0
