"""The C ABI library loads and exports every symbol include/flou_cuda.h declares (no GPU
needed: nothing is called)."""
import ctypes
import os
import re

import flou_cuda as F
from flou_cuda import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^\s*(?:const\s+char\s*\*|int32_t|void|double)\s+\**(flou_\w+)\s*\(", txt, re.M))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert {"flou_create", "flou_rhs", "flou_step", "flou_set_mesh", "flou_max_dt"} <= names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_prototypes_cover_header():
    assert declared_symbols() <= set(_lib.PROTOTYPES), declared_symbols() - set(_lib.PROTOTYPES)


def test_config_struct_layout():
    # flou_config: int32 dim, int32 equation, double gamma, double advection[3], 4 x int32,
    # double intensity, int32 nnodes  -> 72 bytes with natural alignment
    assert ctypes.sizeof(_lib.FlouConfig) == 72
    assert _lib.FlouConfig.gamma.offset == 8 and _lib.FlouConfig.numflux_intensity.offset == 56


def test_load_is_the_in_tree_library():
    lib = F.load()
    assert os.path.abspath(_lib.LIB_PATH).startswith(os.path.join(ROOT, "flou.jl_gb300"))
    assert lib is F.load()
