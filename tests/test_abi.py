"""The C-ABI libraries load and export every symbol their headers declare
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header, prefix):
    text = open(os.path.join(ROOT, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(" + prefix + r"\w+)\s*\(", text)))


def test_product_exports_every_declared_symbol():
    from craystal_gb300 import build as b
    lib = ctypes.CDLL(b.build())
    names = declared("include/craystal_c.h", "cr_")
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_product_binding_covers_header():
    from craystal_gb300 import _lib
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared("include/craystal_c.h", "cr_")) <= bound


def test_oracle_exports_every_declared_symbol():
    import oracle
    lib = oracle.lib()
    names = declared("oracle/craystal_oracle.h", "orc_")
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_error_reporting_without_device():
    """Without a usable GPU the library reports an error code and message
    rather than crashing (on a GPU machine the call succeeds)."""
    import numpy as np
    import craystal_gb300 as cg
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    from craystal_gb300 import scenes
    data = scenes.random_triangle_scene(10)
    with pytest.raises(cg.CrayError) as e:
        cg.Scene(data)
    assert e.value.code in (2, 3) and str(e.value)


def test_invalid_arguments_are_rejected():
    import craystal_gb300 as cg
    lib = cg.load()
    out = ctypes.c_void_p()
    assert lib.cr_scene_create(None, None, None, 0, None, 0, None, 0, None, 0, None, 0, None) == 1
    assert b"NULL" in lib.cr_last_error()
    assert lib.cr_film_clear(None) == 1
    assert lib.cr_trace_closest(None, None, 0, None) == 1
    assert lib.cr_scene_set_traversal(None, 0) == 1
