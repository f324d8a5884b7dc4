"""The C-ABI library loads and exports every entry point include/smg.h
declares (no device needed)."""
import ctypes
import re
from pathlib import Path

from clustersm_gb300 import native

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "smg.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(smg_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) >= 30
    lib = ctypes.CDLL(str(native._LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings():
    for code in range(0, 14):
        assert native.lib.smg_strerror(code)
    assert native.lib.smg_strerror(999) == b"unknown status"


def test_open_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        return
    try:
        native.Context(0)
    except native.SmgError as e:
        assert e.status == 9  # SMG_ERR_NO_DEVICE
    else:
        raise AssertionError("smg_open succeeded without a device")
