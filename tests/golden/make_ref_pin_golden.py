"""Generate golden vectors of the reference's own CPU code (ref_pin_golden.npz).

Runs oracle/_ref/ref_pin (the reference's sources for projection,
backprojection, CTF images, HEALPix sampling, phase shifts, Euler matrices,
reconstruction and the Fourier map of a reference, built by
oracle/build_ref.sh) on small seeded inputs and stores the outputs; the
inputs are regenerated from the seeds in tests/test_oracle_refpin.py.
Results the oracle reproduces bit for bit are stored as SHA-256 digests of
their float64 bytes where the arrays would be large.

    RELION_REFERENCE=<reference tree> python tests/golden/make_ref_pin_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

# small cases (ori, padding 2): projection / backprojection / reconstruction
ORI, PAD = 12, 2
ANGLES = [(10.0, 20.0, 30.0), (-100.0, 45.0, 170.0), (0.0, 0.0, 0.0), (33.3, 91.2, -12.0), (145.0, 135.0, -77.5)]
CTF_PARAMS = [[10000.0, 12000.0, 90.0, 300.0, 2.7, 0.1, 0.0, 1.0, 0.0],
              [15000.0, 14000.0, 33.0, 200.0, 2.0, 0.07, 50.0, 0.9, 10.0],
              [8000.0, 25000.0, 170.0, 300.0, 2.7, 0.1, 0.0, 1.0, 0.0]]
CTF_ORI, CTF_ANGPIX = 48, 1.5
SAMPLING = [(1, 30.0, 8.0, 4.0, 2.0), (2, 7.5, 8.0, 2.0, 2.0), (3, -1.0, 6.0, 1.0, 1.0)]


def inputs(seed=11):
    """Seeded inputs of the small cases (regenerated by the tests)."""
    rng = np.random.default_rng(seed)
    r_max = ORI // 2
    ps = 2 * (int(PAD * r_max + 0.5) + 1) + 1
    ref = dict(data=rng.standard_normal((ps, ps, ps // 2 + 1)) + 1j * rng.standard_normal((ps, ps, ps // 2 + 1)),
               r_max=r_max, yinit=-(ps // 2), zinit=-(ps // 2))
    X = ORI // 2 + 1
    imgs = [rng.standard_normal((ORI, X)) + 1j * rng.standard_normal((ORI, X)) for _ in ANGLES]
    wts = [rng.random((ORI, X)) for _ in ANGLES]
    tau2 = np.linspace(2.0, 0.5, ORI // 2 + 1)
    vol = rng.standard_normal((ORI, ORI, ORI))
    shift_img = rng.standard_normal((ORI, X)) + 1j * rng.standard_normal((ORI, X))
    return dict(ref=ref, imgs=imgs, wts=wts, tau2=tau2, vol=vol, shift_img=shift_img)


def circle_mask(size, r_max):
    """Pixels of a [size][size/2+1] image exactly on the r_max circle."""
    y = np.array([i if i <= size // 2 else i - size for i in range(size)])[:, None]
    x = np.arange(size // 2 + 1)[None, :]
    return (x * x + y * y) == r_max * r_max


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).hexdigest()


def main():
    from oracle import build as obuild
    obuild.build()
    from oracle import refpin
    if not refpin.available():
        raise SystemExit("oracle/_ref/ref_pin not built (set RELION_REFERENCE to the reference tree)")
    inp = inputs()
    out = {}
    mats = refpin.euler(np.array(ANGLES))
    out["euler"] = mats
    out["project"] = refpin.project(inp["ref"], ORI, PAD, ORI, mats)
    circ = circle_mask(ORI, ORI // 2)
    imgs = [np.where(circ, 0, f) for f in inp["imgs"]]
    wts = [np.where(circ, 0, w) for w in inp["wts"]]
    d, w, _ = refpin.backproject(ORI, PAD, ORI, ORI, mats, imgs, wts)
    out["bp_data"], out["bp_weight"] = d, w
    for tag, skip, dm in (("skip_map", True, True), ("skip_nomap", True, False), ("grid_map", False, True)):
        out["recon_" + tag] = refpin.reconstruct(ORI, PAD, ORI, d, w, inp["tau2"], skip_gridding=skip, do_map=dm)
    fd, (yi, zi, rmax), fp = refpin.fourier_map(ORI, PAD, ORI, inp["vol"], do_gridding=True)
    out["fmap_data"], out["fmap_power"] = fd, fp
    out["ctf"] = refpin.ctf_images(CTF_ORI, CTF_ANGPIX, np.array(CTF_PARAMS))
    out["shift"] = refpin.shift(inp["shift_img"], 64.0, 1.5, -2.25)
    for k, (order, psi, rng_, step, pix) in enumerate(SAMPLING):
        rot, tr = refpin.sampling(order, psi, rng_, step, pix, 1)
        out["sampling_%d_shape" % k] = np.array(rot.shape + tr.shape)
        out["sampling_%d_rot_sha256" % k] = np.array(digest(rot))
        out["sampling_%d_trans_sha256" % k] = np.array(digest(tr))
    path = os.path.join(HERE, "ref_pin_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main()
