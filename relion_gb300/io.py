"""MRC image stacks and STAR metadata, and a RELION 3.1+ particle reader
feeding the device image preparation (gbr_expect_images).

MRC reading / writing and STAR parsing are native (libgbrelion io.cpp);
this module wraps them and writes STAR files.  Particle STAR files follow
the reference's 3.1 layout: a data_optics block (rlnOpticsGroup,
rlnVoltage, rlnSphericalAberration, rlnAmplitudeContrast,
rlnImagePixelSize, rlnImageSize) and a data_particles block
(rlnImageName "index@stack", rlnDefocusU/V/Angle, rlnOriginXAngst /
rlnOriginYAngst, optionally rlnCtfBfactor, rlnCtfScalefactor,
rlnPhaseShift, rlnNormCorrection, rlnOpticsGroup), as written by
MetaDataTable::write (src/metadata_table.cpp) and read by
Experiment::read (src/exp_model.cpp).
"""
import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check


def read_mrc_header(path):
    h = _lib.MrcHeader()
    check(_lib.load().gbr_mrc_read_header(os.fsencode(path), C.byref(h)))
    return {k: getattr(h, k) for k, _ in _lib.MrcHeader._fields_}


def read_mrc_images(path, first=0, count=None, out=None, nthreads=8):
    """Images [first, first + count) as float32 [count][ny][nx]; `out` may be
    a preallocated (e.g. page-locked) float32 array of that shape."""
    h = read_mrc_header(path)
    count = h["nz"] - first if count is None else count
    if out is None:
        out = np.empty((count, h["ny"], h["nx"]), np.float32)
    assert out.dtype == np.float32 and out.flags.c_contiguous and out.size >= count * h["ny"] * h["nx"]
    check(_lib.load().gbr_mrc_read_images(os.fsencode(path), int(first), int(count), out.ctypes.data,
                                          int(nthreads)))
    return out


def write_mrc_stack(path, data, pixel_size=1.0):
    a = np.ascontiguousarray(data, np.float32)
    if a.ndim == 2:
        a = a[None]
    nz, ny, nx = a.shape
    check(_lib.load().gbr_mrc_write_stack(os.fsencode(path), a.ctypes.data, nx, ny, nz, float(pixel_size)))


class StarFile:
    """Blocks of a STAR file: {block name: {label: [values as strings]}}."""

    def __init__(self, path):
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.gbr_star_read(os.fsencode(path), C.byref(h)))
        self.blocks = {}
        try:
            for ib in range(lib.gbr_star_num_blocks(h)):
                name = C.create_string_buffer(256)
                nc, nr, loop = C.c_int64(), C.c_int64(), C.c_int()
                check(lib.gbr_star_block_info(h, ib, name, 256, C.byref(nc), C.byref(nr), C.byref(loop)))
                cols = {}
                for ic in range(nc.value):
                    lab = C.create_string_buffer(256)
                    check(lib.gbr_star_column_name(h, ib, ic, lab, 256))
                    vals = []
                    buf = C.create_string_buffer(4096)
                    for r in range(nr.value):
                        check(lib.gbr_star_value_string(h, ib, lab.value, r, buf, 4096))
                        vals.append(buf.value.decode())
                    cols[lab.value.decode()] = vals
                self.blocks[name.value.decode()] = cols
        finally:
            lib.gbr_star_free(h)

    def column(self, block, label, dtype=float, default=None):
        cols = self.blocks[block]
        label = label.lstrip("_")
        if label not in cols:
            if default is None:
                raise KeyError("no column %s in block %s" % (label, block))
            n = len(next(iter(cols.values()))) if cols else 0
            return np.full(n, default, dtype=dtype)
        return np.array([dtype(v) for v in cols[label]])


def write_star(path, blocks):
    """blocks: {name: {label: sequence}}; one loop_ table per block."""
    with open(path, "w") as f:
        for name, cols in blocks.items():
            f.write("\n# version 30001\n\ndata_%s\n\nloop_\n" % name)
            labels = list(cols)
            for i, lab in enumerate(labels):
                f.write("_%s #%d\n" % (lab.lstrip("_"), i + 1))
            n = len(cols[labels[0]]) if labels else 0
            for r in range(n):
                vals = []
                for lab in labels:
                    v = cols[lab][r]
                    s = ("%.6f" % v) if isinstance(v, (float, np.floating)) else str(v)
                    vals.append('"%s"' % s if (" " in s or not s) else s)
                f.write(" ".join(vals) + "\n")
            f.write("\n")


def load_particles(star_path, first=0, count=None, nthreads=8, out=None):
    """RELION 3.1+ particles STAR -> image batch for gbr_expect_images.

    Returns dict(n, images [n][box][box] float32, old_offset [n][2] pixels,
    prior [n][2], norm_correction, scale, ctf [n][6]) plus the optics of the
    first group (kV, Cs, Q0, pixel_size, box).  Stacks are read natively into
    `out` (a float32 array, e.g. page-locked) when given."""
    st = StarFile(star_path)
    base = os.path.dirname(os.path.abspath(star_path))
    opt = "optics"
    px = st.column(opt, "rlnImagePixelSize")
    optics = dict(kV=float(st.column(opt, "rlnVoltage")[0]), Cs=float(st.column(opt, "rlnSphericalAberration")[0]),
                  Q0=float(st.column(opt, "rlnAmplitudeContrast")[0]), pixel_size=float(px[0]),
                  box=int(st.column(opt, "rlnImageSize", int)[0]))
    part = "particles"
    names = st.blocks[part]["rlnImageName"]
    total = len(names)
    count = total - first if count is None else count
    sel = slice(first, first + count)
    box = optics["box"]
    images = out if out is not None else np.empty((count, box, box), np.float32)
    # group consecutive entries of one stack into single native reads
    k = 0
    entries = [n.split("@") for n in names[sel]]
    while k < count:
        idx, stack = int(entries[k][0]), entries[k][1]
        j = k + 1
        while j < count and entries[j][1] == stack and int(entries[j][0]) == idx + (j - k):
            j += 1
        path = stack if os.path.isabs(stack) else os.path.join(base, stack)
        read_mrc_images(path, idx - 1, j - k, out=images[k:j], nthreads=nthreads)
        k = j
    pix = optics["pixel_size"]
    col = lambda lab, d: st.column(part, lab, float, d)[sel]
    old = np.stack([col("rlnOriginXAngst", 0.0), col("rlnOriginYAngst", 0.0)], 1) / pix
    ctf = np.stack([col("rlnDefocusU", 0.0), col("rlnDefocusV", 0.0), col("rlnDefocusAngle", 0.0),
                    col("rlnCtfBfactor", 0.0), col("rlnCtfScalefactor", 1.0), col("rlnPhaseShift", 0.0)], 1)
    return dict(n=count, images=images, old_offset=old, prior=np.zeros((count, 2)),
                norm_correction=col("rlnNormCorrection", 1.0), scale=np.ones(count), ctf=ctf, optics=optics)
