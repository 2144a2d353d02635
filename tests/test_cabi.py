"""CPU checks of the C-ABI boundary: the library loads without a GPU and
exports every entry point include/neci_gpu.h declares; the ctypes structs
match the header's layout."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

from neci_stable_gb300 import capi

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "neci_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(neci_gpu_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "neci_gpu_iterate" in names and "neci_gpu_annihilate" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib_path = capi._LIB_PATH
    if not lib_path.exists():
        pytest.skip("library not built (run __graft_entry__.build())")
    lib = C.CDLL(str(lib_path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes binding covers the same set
    assert set(capi.EXPORTS) <= set(declared_functions())


def _c_layout(struct_name):
    """Byte size of a header struct computed from its member declarations."""
    text = HEADER.read_text()
    body = re.search(r"typedef struct \{([^{}]*)\} " + struct_name + ";", text, re.S).group(1)
    size = 0
    align = {"int32_t": 4, "uint32_t": 4, "int64_t": 8, "uint64_t": 8, "double": 8}
    for typ, names in re.findall(r"^\s*(int32_t|uint32_t|int64_t|uint64_t|double)\s+([^;]+);", body, re.M):
        for nm in names.split(","):
            nm = nm.strip()
            count = 1
            m = re.match(r"(\w+)\[(\d+)\]", nm)
            if m:
                count = int(m.group(2))
            a = align[typ]
            size = (size + a - 1) // a * a + a * count
    return (size + 7) // 8 * 8


@pytest.mark.parametrize("cls,name", [(capi.System, "neci_gpu_system"), (capi.IterParams, "neci_gpu_iter_params"),
                                      (capi.IterStats, "neci_gpu_iter_stats"),
                                      (capi.TauStats, "neci_gpu_tau_stats"), (capi.Tuning, "neci_gpu_tuning")])
def test_struct_sizes_match_header(cls, name):
    assert C.sizeof(cls) == _c_layout(name)
