"""CPU tests: the C-ABI library builds, loads and exports what the header declares."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "gbrelion.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gbr_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from relion_gb300 import build
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], stdout=subprocess.PIPE, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (gbr_[a-z_0-9]+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    assert len(declared_symbols()) >= 18


def test_library_loads_and_binds():
    from relion_gb300 import _lib
    lib = _lib.load()
    assert b"sm_103a" in lib.gbr_version()
    for name in declared_symbols():
        assert hasattr(lib, name)


def test_struct_layouts_match_header():
    import ctypes as C
    from relion_gb300 import _lib
    assert C.sizeof(_lib.ModelDesc) == 14 * 8 + 8 * 8
    assert C.sizeof(_lib.ParticleBatch) == 2 * 8 + 9 * 8
    assert C.sizeof(_lib.ParticleResult) == 16 * 8 + 2 * 8
    assert C.sizeof(_lib.Wsum) == 3 * 8 + 8 * 8


def test_errors_are_reported_without_gpu():
    import ctypes as C
    from relion_gb300 import _lib
    lib = _lib.load()
    d = _lib.ModelDesc()  # all zero: invalid
    h = C.c_void_p()
    st = lib.gbr_bundle_create(C.byref(d), 0, C.byref(h))
    assert st == _lib.GBR_ERR_INVALID
    assert "invalid" in _lib.last_error()
