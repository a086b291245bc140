"""The C-ABI library loads and exports every entry point the header declares."""
import ctypes as C
import pathlib
import re

from gfm_gb300 import abi

HEADER = pathlib.Path(__file__).resolve().parent.parent / "include" / "gfm_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gfm_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = abi.load_library()
    names = declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(n for n, _, _ in abi.SIGNATURES) == names


def test_struct_sizes_are_plausible():
    # ctypes mirrors must line up with the header's field order
    assert C.sizeof(abi.GfmIterStats) == 4 * 2 + 8 * (2 + 3 + 6 + 20 + 3 + 4 + 2) + 16
    assert abi.GfmParams.ntimesg.offset % 4 == 0


def test_device_query_without_gpu_is_an_error_not_a_crash():
    lib = abi.load_library()
    n = lib.gfm_gpu_device_count()
    assert isinstance(n, int)
    assert n >= 1 or n == abi.GFM_E_NODEVICE
