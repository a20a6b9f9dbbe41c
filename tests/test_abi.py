"""The C-ABI library builds, loads and exports every symbol of include/sss.h
(no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "sss.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(sss_\w+)\(", text, re.M)))


def test_header_declares_the_entry_points():
    names = declared_symbols()
    from superspinsim_gb300._lib import SYMBOLS
    assert set(SYMBOLS) <= set(names)
    assert len(names) >= 10


def test_library_exports_every_declared_symbol():
    from superspinsim_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_errors_without_gpu_are_codes_not_crashes():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from superspinsim_gb300 import _lib
    import numpy as np
    with pytest.raises(_lib.SSSError) as e:
        _lib.Plan(np.zeros((5, 4, 4)), np.ones((1, 1)), np.array([0.5]))
    assert e.value.code in (-6, -3)
