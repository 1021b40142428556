"""The C ABI library loads and exports every entry point include/staqdic.h
declares (no compute calls: no GPU needed)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    hdr = open(os.path.join(ROOT, "include", "staqdic.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(stdic_\w+)\s*\(", hdr)))


def test_header_declares_entry_points():
    names = _declared()
    for n in ("stdic_interp_bicubic", "stdic_img_gradient", "stdic_integer_search",
              "stdic_icgn_local", "stdic_icgn_subsets", "stdic_subpb1", "stdic_subpb2"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from staqdic import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_every_export():
    from staqdic import _lib
    assert sorted(_lib.EXPORTS) == _declared()
