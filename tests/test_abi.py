"""The C ABI library loads without a GPU and exports every entry point that
include/*.h declares; the Python binding knows each of them."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            txt = open(os.path.join(inc, fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(xdgcu_\w+)\s*\(", txt, re.M))
    return names


def test_library_exports_every_declared_symbol():
    from xdg_gb300 import _lib, build
    path = build.build()
    lib = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_lib.SIGNATURES) >= names


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        return
    from xdg_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    rc = L.xdgcu_create(ctypes.byref(h), 0)
    assert rc != 0 and not h.value
    assert b"device" in L.xdgcu_last_error(None)


def test_every_tuning_key_documented_and_handled():
    """Each tuning key the Python layer lists is documented in the header and
    handled by both xdgcu_set_tuning and xdgcu_get_tuning in the library
    source."""
    from xdg_gb300.engine import TUNING_KEYS
    with open(os.path.join(ROOT, "include", "xdgcu.h")) as f:
        header = f.read()
    with open(os.path.join(ROOT, "xdg_gb300", "csrc", "api.cu")) as f:
        src = f.read()
    for k in TUNING_KEYS:
        assert re.search(r'^\s*\*\s+"%s"' % re.escape(k), header, re.M), f"{k} not documented"
        assert src.count('k == "%s"' % k) >= 2, f"{k} not handled by set and get"
