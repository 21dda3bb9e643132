"""Generate golden vectors of the reference's own CPU E-step (ref_estep_golden.npz).

Runs oracle/_ref/ref_estep (the reference's MlOptimiser::getAllSquaredDifferences,
convertAllSquaredDifferencesToWeights and storeWeightedSums, built by
oracle/build_ref.sh) on seeded prepared particles of two small shapes and
stores its per-particle results, weighted sums and backprojected volumes
(float64 scalars; of the volumes, as float32, every voxel of the outer shell
that the pixels on the r_max circle reach and a seeded sample of the others,
with the full norms).  The inputs are regenerated from the
seeds by the tests (relion_gb300.datagen), which compare the oracle (CPU
tests) and the CUDA E-step (GPU tests) with these outputs.

    RELION_REFERENCE=<reference tree> python tests/golden/make_ref_estep_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

# (name, dataset config, seed, particles, overrides)
CASES = [
    ("box32_hp1", "small32", 5, 4, dict(healpix_order=1, psi_step=30.0)),
    ("box32_hp2", "small32", 6, 2, dict(healpix_order=2, psi_step=15.0, offset_range_px=3.0, offset_step_px=1.0)),
    # a late iteration: the whole box as current size, a small coarse size and
    # a reference sharp to Nyquist (the coarse projection fills only the
    # coarse image's own circle, inside the reference's r_max)
    ("box32_late", "small32_late", 7, 3, dict(healpix_order=1, psi_step=30.0)),
]
PER_PARTICLE = ("rot", "tilt", "psi", "xoff", "yoff", "pmax", "dLL", "nr_sign", "coarse_min_diff2",
                "coarse_sum_weight", "coarse_significant_weight", "fine_min_diff2", "fine_sum_weight",
                "fine_significant_weight")


def config(name):
    """A box-32 shape of the box-64 generator (2 A pixels halved in count);
    "small32_late": the same in a late iteration (current size 32, coarse
    size 12, reference low-passed at Nyquist, 8 A)."""
    from relion_gb300 import datagen
    c = dict(datagen.CONFIGS["cfg0_box64"])
    c.update(box=32, pixel=4.0, n_blobs=150, blob_radius=10.0, max_shift=2.0, diameter=100.0, ini_high=24.0)
    if name == "small32_late":
        c.update(current_size=32, coarse_size=12, ini_high=8.0)
    return c


def volume_sample(shape, rmax_pad, n_inner=3000, seed=3):
    """Flat indices of the voxels within 1.8 of the padded r_max radius (those
    the pixels on the r_max circle reach) and of n_inner seeded others."""
    z, y, x = np.meshgrid(np.arange(shape[0]) - shape[0] // 2, np.arange(shape[1]) - shape[1] // 2,
                          np.arange(shape[2]), indexing="ij")
    r = np.sqrt(x * x + y * y + z * z).ravel()
    shell = np.nonzero(np.abs(r - rmax_pad) <= 1.8)[0]
    rest = np.setdiff1d(np.arange(r.size), shell)
    rng = np.random.default_rng(seed)
    inner = rng.choice(rest, min(n_inner, rest.size), replace=False)
    return np.sort(np.concatenate([shell, inner])).astype(np.int64)


def dataset(case):
    from relion_gb300 import datagen
    name, cfg, seed, n, kw = case
    return datagen.Dataset(config(cfg), seed=seed, n_particles=n, **kw)


def main():
    from oracle import build as obuild
    obuild.build()
    from oracle import refpin
    if not refpin.estep_available():
        raise SystemExit("oracle/_ref/ref_estep not built (set RELION_REFERENCE to the reference tree)")
    out = {}
    for case in CASES:
        name, _, _, n, _ = case
        ds = dataset(case)
        m = ds.model()
        b = ds.particles(0, n)
        parts, ws, bd, bw = refpin.estep(m, ds.ref, b)
        for k in PER_PARTICLE:
            out["%s/%s" % (name, k)] = np.array([p[k] for p in parts])
        for k in ("sigma2_noise", "pdf_direction"):
            out["%s/wsum_%s" % (name, k)] = np.asarray(ws[k])
        for k in ("sigma2_offset", "sumw_group", "LL", "ave_Pmax"):
            out["%s/wsum_%s" % (name, k)] = np.array(ws[k])
        idx = volume_sample(bd.shape, 2 * (m["current_size"] // 2))
        out["%s/bp_idx" % name] = idx
        out["%s/bp_data_sub" % name] = bd.ravel()[idx].astype(np.complex64)
        out["%s/bp_weight_sub" % name] = bw.ravel()[idx].astype(np.float32)
        out["%s/bp_data_norm" % name] = np.array(np.linalg.norm(bd))
        out["%s/bp_weight_norm" % name] = np.array(np.linalg.norm(bw))
        print(name, "particles", n, "volume", bd.shape, "current/coarse", m["current_size"], m["coarse_size"])
    path = os.path.join(HERE, "ref_estep_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
