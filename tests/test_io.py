"""CPU tests of the data formats (MRC stacks, STAR tables) and the RELION
3.1+ particle reader, through the native reader / parser in libgbrelion.

MRC files of every supported mode are built here byte by byte from the
format's definition (1024-byte header: nx, ny, nz, mode at words 0-3, mx at
word 7, cell a at word 10, nsymbt at word 23; data after 1024 + nsymbt) and
read back; a big-endian file checks the byte-order detection.
"""
import os

import numpy as np
import pytest


def _header(nx, ny, nz, mode, nsymbt=0, pixel=1.5, endian="<"):
    h = np.zeros(256, dtype=endian + "i4")
    h[0], h[1], h[2], h[3] = nx, ny, nz, mode
    h[7], h[8], h[9] = nx, ny, nz
    h[23] = nsymbt
    b = bytearray(h.tobytes())
    b[40:44] = np.array([pixel * nx], dtype=endian + "f4").tobytes()
    return bytes(b)


def _write(path, header, ext, payload):
    with open(path, "wb") as f:
        f.write(header)
        f.write(ext)
        f.write(payload)


def test_mrc_roundtrip_float32(tmp_path):
    from relion_gb300 import io
    g = np.random.default_rng(1)
    data = g.normal(size=(7, 24, 32)).astype(np.float32)
    p = str(tmp_path / "stack.mrcs")
    io.write_mrc_stack(p, data, pixel_size=1.25)
    h = io.read_mrc_header(p)
    assert (h["nx"], h["ny"], h["nz"], h["mode"], h["nsymbt"], h["swapped"]) == (32, 24, 7, 2, 0, 0)
    assert abs(h["pixel_size"] - 1.25) < 1e-6 and h["data_offset"] == 1024
    raw = np.fromfile(p, dtype="<f4", offset=1024).reshape(7, 24, 32)
    np.testing.assert_array_equal(raw, data)
    sub = io.read_mrc_images(p, 2, 4, nthreads=3)
    np.testing.assert_array_equal(sub, data[2:6])


@pytest.mark.parametrize("mode", [0, 1, 6, 12, 101, 2])
def test_mrc_modes_and_extended_header(tmp_path, mode):
    from relion_gb300 import io
    g = np.random.default_rng(mode + 3)
    nx, ny, nz, ext = 10, 6, 3, 96
    if mode == 0:
        v = g.integers(-128, 128, size=(nz, ny, nx)).astype(np.int8)
        payload, want = v.tobytes(), v.astype(np.float32)
    elif mode == 1:
        v = g.integers(-30000, 30000, size=(nz, ny, nx)).astype("<i2")
        payload, want = v.tobytes(), v.astype(np.float32)
    elif mode == 6:
        v = g.integers(0, 65535, size=(nz, ny, nx)).astype("<u2")
        payload, want = v.tobytes(), v.astype(np.float32)
    elif mode == 12:
        v = g.normal(size=(nz, ny, nx)).astype("<f2")
        payload, want = v.tobytes(), v.astype(np.float32)
    elif mode == 101:
        v = g.integers(0, 16, size=(nz, ny, nx)).astype(np.uint8)
        flat = v.reshape(nz, -1)
        packed = (flat[:, 0::2] | (flat[:, 1::2] << 4)).astype(np.uint8)  # low nibble first
        payload, want = packed.tobytes(), v.astype(np.float32)
    else:
        v = g.normal(size=(nz, ny, nx)).astype(">f4")
        payload, want = v.tobytes(), v.astype(np.float32)
    endian = ">" if mode == 2 else "<"
    p = str(tmp_path / ("m%d.mrc" % mode))
    _write(p, _header(nx, ny, nz, mode, ext, endian=endian), b"\x07" * ext, payload)
    h = io.read_mrc_header(p)
    assert h["mode"] == mode and h["data_offset"] == 1024 + ext and h["swapped"] == (1 if mode == 2 else 0)
    np.testing.assert_array_equal(io.read_mrc_images(p), want)
    np.testing.assert_array_equal(io.read_mrc_images(p, 1, 2, nthreads=2), want[1:3])


STAR_TEXT = """
# a comment before any block
data_general

_rlnNrClasses  3
_rlnPixelSize  1.350000   # trailing comment

data_optics

loop_
_rlnOpticsGroupName #1
_rlnOpticsGroup #2
_rlnVoltage #3
_rlnSphericalAberration #4
_rlnAmplitudeContrast #5
_rlnImagePixelSize #6
_rlnImageSize #7
"optics group 1"  1  300.000000  2.700000  0.100000  1.350000  64

data_particles

loop_
_rlnImageName #1
_rlnDefocusU #2
_rlnDefocusV #3
_rlnDefocusAngle #4
_rlnOriginXAngst #5
_rlnOriginYAngst #6
_rlnOpticsGroup #7
000001@stack_a.mrcs  15000.5  14900.25  12.5  1.35  -2.70  1
000002@stack_a.mrcs  16000.0  15900.00  80.0  0.00   0.00  1
# comment between rows
000001@stack_b.mrcs  17000.0  16800.00 170.0 -4.05   1.35  1
"""


def test_star_blocks_loops_comments_quotes(tmp_path):
    from relion_gb300 import io
    p = tmp_path / "t.star"
    p.write_text(STAR_TEXT)
    st = io.StarFile(str(p))
    assert list(st.blocks) == ["general", "optics", "particles"]
    assert st.blocks["general"]["rlnNrClasses"] == ["3"]
    assert st.column("general", "rlnPixelSize")[0] == pytest.approx(1.35)
    assert st.blocks["optics"]["rlnOpticsGroupName"] == ["optics group 1"]
    assert st.column("optics", "_rlnImageSize", int)[0] == 64
    np.testing.assert_allclose(st.column("particles", "rlnDefocusU"), [15000.5, 16000.0, 17000.0])
    assert st.blocks["particles"]["rlnImageName"][2] == "000001@stack_b.mrcs"
    np.testing.assert_array_equal(st.column("particles", "rlnCtfBfactor", float, 0.0), [0.0, 0.0, 0.0])


def test_star_write_read_roundtrip(tmp_path):
    from relion_gb300 import io
    p = str(tmp_path / "w.star")
    io.write_star(p, {"particles": {"rlnImageName": ["1@a.mrcs", "2@a.mrcs"], "rlnDefocusU": [1.5, 2.5],
                                    "rlnClassNumber": [1, 2], "rlnMicrographName": ["mic 1", "mic 2"]}})
    st = io.StarFile(p)
    np.testing.assert_allclose(st.column("particles", "rlnDefocusU"), [1.5, 2.5])
    assert st.blocks["particles"]["rlnMicrographName"] == ["mic 1", "mic 2"]
    assert list(st.column("particles", "rlnClassNumber", int)) == [1, 2]


def test_load_particles(tmp_path):
    from relion_gb300 import io
    g = np.random.default_rng(5)
    a = g.normal(size=(2, 64, 64)).astype(np.float32)
    b = g.normal(size=(1, 64, 64)).astype(np.float32)
    io.write_mrc_stack(str(tmp_path / "stack_a.mrcs"), a, 1.35)
    io.write_mrc_stack(str(tmp_path / "stack_b.mrcs"), b, 1.35)
    p = tmp_path / "particles.star"
    p.write_text(STAR_TEXT)
    batch = io.load_particles(str(p))
    assert batch["n"] == 3 and batch["optics"]["box"] == 64
    assert batch["optics"]["kV"] == 300.0 and batch["optics"]["Q0"] == pytest.approx(0.1)
    np.testing.assert_array_equal(batch["images"][:2], a)
    np.testing.assert_array_equal(batch["images"][2], b[0])
    np.testing.assert_allclose(batch["old_offset"], [[1.0, -2.0], [0.0, 0.0], [-3.0, 1.0]])
    np.testing.assert_allclose(batch["ctf"][:, 0], [15000.5, 16000.0, 17000.0])
    np.testing.assert_allclose(batch["ctf"][:, 4], [1.0, 1.0, 1.0])
    part = io.load_particles(str(p), first=1, count=2)
    np.testing.assert_array_equal(part["images"][0], a[1])
