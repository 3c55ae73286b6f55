"""The C ABI library builds, loads, and exports every entry point of include/ugrowth.h."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "ugrowth.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ug_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from unsupervised_growth_gb300 import build
    from unsupervised_growth_gb300.engine import EXPORTED
    path = build.build()
    lib = ctypes.CDLL(path)
    declared = header_functions()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(EXPORTED) == declared


def test_no_gpu_fails_loudly_or_runs():
    """Creating a context either works (GPU present) or returns an error status; never silently falls back."""
    from unsupervised_growth_gb300.engine import Engine, UGError
    try:
        e = Engine(precision=32)
    except UGError as err:
        assert err.status in (7, 1)
        return
    e.close()
