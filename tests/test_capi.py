"""The C ABI library loads and exports every symbol include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(zeta_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    import zeta_gb300 as z
    lib = z.load_library()
    names = declared("zeta_cuda.h")
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers the whole header
    assert set(names) <= set(z.SIGNATURES), set(names) - set(z.SIGNATURES)


def test_calls_before_init_fail_loudly():
    import zeta_gb300 as z
    lib = z.load_library()
    import numpy as np
    b = np.zeros(7, dtype=np.uint64)
    out = ctypes.c_uint64()
    rc = lib.zeta_perft(b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), 0, 1, ctypes.byref(out))
    assert rc == -3  # ZETA_ERR_STATE: no CPU fallback
    with pytest.raises(z.ZetaError):
        z.perft(b, 0, 1)


def test_library_is_built_for_sm_103a_only():
    """The shared object carries sm_103a code only (checked from the build
    recipe, which passes a single -gencode)."""
    from zeta_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_setting_arguments_are_checked_on_the_host():
    """Settings are validated before any device work: a bad launch form or
    learned-ordering width is an argument error, a good one is accepted."""
    import zeta_gb300 as z
    for bad in (-1, 4):
        with pytest.raises(z.ZetaError):
            z.search_set_launch_form(bad)
    for form in (1, 2, 3, 0):
        z.search_set_launch_form(form)
    with pytest.raises(z.ZetaError):
        z.search_set_learned_order(0)
