"""The C-ABI library loads without a GPU and exports every entry point
declared in include/fs2d.h and include/fs3d.h (no compute calls are made
here)."""
import os
import re

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_symbols():
    syms = set()
    for h in ("fs2d.h", "fs3d.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        syms |= set(re.findall(r"\b(fs[23]d_[a-z_0-9]+)\s*\(", text))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "fs2d_create" in syms and "fs2d_run_frame" in syms and len(syms) >= 20


def test_library_exports_every_declared_symbol():
    import fs2d
    if not os.path.exists(fs2d.LIB_PATH):
        import build
        build.build()
    lib = fs2d.load()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes table covers the header exactly
    assert sorted(fs2d.SIGNATURES) == declared_symbols()


def test_default_options_are_the_reference_constants():
    import fs2d
    o = fs2d.default_options()
    assert (o.mic_tau, o.mic_sigma, o.pcg_tol, o.pcg_max_iters) == (0.999, 0.25, 1e-12, 200)
    assert o.precision == 0 and o.p2g_mode == 0 and o.extrapolate_band == 0


def test_last_error_callable_without_gpu():
    import fs2d
    assert isinstance(fs2d.load().fs2d_last_error(), bytes)
