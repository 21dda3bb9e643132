"""Generate the HEALPix golden vectors from the reference's own code.

Runs the reference's Healpix_Base (src/Healpix_2.15a/healpix_base.cc,
compiled into oracle/_ref by oracle/build_ref.sh) for orders 0-4 and stores
pix2ang_z_phi and nest2xyf of every NEST pixel, plus the CTF known answer
of the reference's only unit test (tests/ctf.cpp:5-10), in healpix_ref.npz.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    from oracle import build as obuild
    obuild.build()
    from oracle import pyoracle
    ref = pyoracle.load_ref()
    if ref is None:
        raise SystemExit("oracle/_ref/libref_healpix.so not built (needs the reference tree)")
    out = {}
    for order in range(5):
        n = ref.ref_hpx_npix(order)
        z = np.zeros(n); phi = np.zeros(n); xyf = np.zeros((n, 3), np.int32)
        zz, pp = C.c_double(), C.c_double()
        a, b, f = C.c_int(), C.c_int(), C.c_int()
        for p in range(n):
            ref.ref_hpx_pix2ang_z_phi(order, p, C.byref(zz), C.byref(pp))
            z[p], phi[p] = zz.value, pp.value
            ref.ref_hpx_nest2xyf(order, p, C.byref(a), C.byref(b), C.byref(f))
            xyf[p] = (a.value, b.value, f.value)
        out["z_%d" % order] = z
        out["phi_%d" % order] = phi
        out["xyf_%d" % order] = xyf
    # tests/ctf.cpp:7-9: setValues(10000, 12000, 90, 300, 2.7, 0.1, 0, 1, 0); getCTF(10,10) ~ 0.59154
    out["ctf_kat_args"] = np.array([10000.0, 12000.0, 90.0, 300.0, 2.7, 0.1, 0.0, 1.0, 0.0, 10.0, 10.0])
    out["ctf_kat_value"] = np.array([0.59154])
    np.savez_compressed(os.path.join(HERE, "healpix_ref.npz"), **out)
    print("wrote", os.path.join(HERE, "healpix_ref.npz"))


if __name__ == "__main__":
    main()
