"""The C-ABI library builds, loads and exports every entry point that
include/*.h declares (no device calls: runs without a GPU)."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+(lne_[A-Za-z0-9_]+)\s*\(", txt, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "lne_sparsify" in names and "lne_ctx_create" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(lib):
    from lightne_gb300 import _lib
    assert declared_symbols() <= set(_lib.SIGNATURES), declared_symbols() - set(_lib.SIGNATURES)


def test_version_and_error_without_device(lib):
    assert lib.lne_version().startswith(b"lightne_gb300")
    assert isinstance(lib.lne_last_error(), bytes)
    # NULL out pointer is rejected before any device work
    assert lib.lne_ctx_create(None, 0, None) != 0
    assert lib.lne_ctx_set_sparsify_slices(None, 8192, -1) != 0
    assert lib.lne_ctx_set_sparsify_batch(None, 0) != 0


def test_chebyshev_coefficients_match_scipy(lib):
    import numpy as np
    import scipy.special as ss
    from lightne_gb300.api import chebyshev_coefficients
    c = chebyshev_coefficients(10, 0.5)
    ref = [ss.iv(0, 0.5), -2 * ss.iv(1, 0.5)] + [(-2 if k & 1 else 2) * ss.iv(k, 0.5) for k in range(2, 10)]
    assert np.array_equal(c, np.array(ref, dtype=np.float32))


def test_status_and_precision_constants_match_header():
    from lightne_gb300 import _lib
    txt = open(os.path.join(ROOT, "include", "lightne_gb300.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"^#define (LNE_[A-Z0-9_]+) (\d+)", txt, re.M)}
    assert {"LNE_OK", "LNE_ERR_TABLE_FULL", "LNE_PREC_FP32", "LNE_PREC_BF16", "LNE_PREC_FP8",
            "LNE_PREC_FP16"} <= set(defs)
    for name, value in defs.items():
        if hasattr(_lib, name):
            assert getattr(_lib, name) == value, name
