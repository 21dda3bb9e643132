"""Build the oracle (TEST INFRASTRUCTURE ONLY).

Compiles oracle/relion_oracle.cpp and oracle/oracle_mstep.cpp into
oracle/_build/liboracle.so and, when the environment variable
RELION_REFERENCE names the reference source tree, the reference's own code
into oracle/_ref (oracle/build_ref.sh): its HEALPix sources as
libref_healpix.so and the ref_pin driver over its CPU sources.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_healpix.so")
REF_PIN = os.path.join(HERE, "_ref", "ref_pin")
REF_ESTEP = os.path.join(HERE, "_ref", "ref_estep")


def build(force=False):
    os.makedirs(os.path.join(HERE, "_build"), exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("relion_oracle.cpp", "oracle_mstep.cpp")]
    hdr = os.path.join(HERE, "relion_oracle.h")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            [os.path.getmtime(s) for s in srcs] + [os.path.getmtime(hdr)]):
        subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17", "-fopenmp"]
                       + srcs + ["-o", LIB + ".tmp"], check=True)
        os.replace(LIB + ".tmp", LIB)
    ref = os.environ.get("RELION_REFERENCE", "")
    deps = [os.path.join(HERE, "build_ref.sh")] + [os.path.join(HERE, "ref", f) for f in os.listdir(os.path.join(HERE, "ref"))
                                                  if f.endswith(".cpp")]
    newest = max(os.path.getmtime(d) for d in deps)
    stale = any(not os.path.exists(f) or os.path.getmtime(f) < newest for f in (REF_PIN, REF_ESTEP))
    if ref and os.path.isdir(os.path.join(ref, "src", "Healpix_2.15a")) and (force or stale or
                                                                          not os.path.exists(REF_LIB)):
        subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True)
    return LIB


if __name__ == "__main__":
    build(force=True)
