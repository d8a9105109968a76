"""The C-ABI library builds, loads and exports every entry point that
include/*.h declares (no compute calls: this runs without a GPU)."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest
import torch

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"FGB_API\s+[\w\s\*]+?\b(fgb_\w+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib_path():
    from finchgb import build

    return build.build()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert {"fgb_spmv", "fgb_spmm", "fgb_sddmm", "fgb_ewise_reduce", "fgb_transpose"} <= names


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(str(lib_path))
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\b(fgb_\w+)\b", out))
    assert declared_symbols() <= exported
    # nothing but the declared API is exported under the fgb_ prefix
    assert exported <= declared_symbols()


def test_header_comments_every_entry_point():
    # every declaration (or group of declarations) sits under a comment that
    # says what it does and which reference interface it replaces, or that it
    # has no counterpart in the reference
    for h in (ROOT / "include").glob("*.h"):
        lines = h.read_text().splitlines()
        for i, ln in enumerate(lines):
            if re.match(r"\s*FGB_API\b", ln):
                above = lines[max(0, i - 14):i]
                assert any(a.rstrip().endswith("*/") for a in above), f"{h.name}:{i + 1} has no comment"


def test_python_binding_covers_header():
    from finchgb import _lib

    assert set(_lib.SIGNATURES) == declared_symbols()


def test_version_and_error_path_without_gpu(lib_path):
    from finchgb import _lib

    L = _lib.load()
    assert L.fgb_version() == 1
    if torch.cuda.is_available():
        pytest.skip("host has a GPU")
    h = ctypes.c_void_p()
    rc = L.fgb_ctx_create(0, ctypes.byref(h))
    assert rc == _lib.ECUDA
    assert "device" in _lib.last_error().lower()
    assert not h.value
    # argument validation happens before any CUDA call
    assert L.fgb_spmv(None, 0, None, None, 0, None, 0, 0, None) == _lib.EINVAL
    assert "null ctx" in _lib.last_error()


def test_no_cpu_fallback_in_device_layer():
    from finchgb import FinchGBError, device

    if torch.cuda.is_available():
        pytest.skip("host has a GPU")
    with pytest.raises(FinchGBError):
        device.context(0)
