"""The shared library loads and exports every entry point include/*.h declares (CPU only)."""
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(cfd2d_[a-z0-9_]+)\s*\(", src))
    return names


def test_every_declared_symbol_is_exported(capi):
    lib = capi.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in sorted(syms) if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_the_header(capi):
    assert declared_symbols() <= set(capi.SIGNATURES)


def test_no_device_is_reported_cleanly(capi, tmp_path):
    """Without a GPU, creating a solver fails with a status code, not a crash."""
    import torch
    if torch.cuda.is_available():
        return
    from conftest import load_golden, write_case
    g = load_golden("shock_tube_4bc")
    try:
        capi.Solver(write_case(tmp_path, g))
    except capi.CfdError as e:
        assert e.code in (501, 502)
    else:
        raise AssertionError("solver creation without a GPU must fail")
