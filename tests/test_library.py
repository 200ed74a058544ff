"""The C ABI library loads and exports every entry point that include/*.h
declares (no compute: runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")

DECL = re.compile(r"^\s*(?:const\s+)?(?:void|int|double|char)\s*\**\s*(\w+)\s*\(", re.M)


def declared(header):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(DECL.findall(text)))


@pytest.fixture(scope="module")
def built():
    from flow_gb300 import build
    build.build()
    return build


def headers():
    return sorted(f for f in os.listdir(INCLUDE) if f.endswith(".h"))


def test_headers_declare_entry_points():
    names = declared("flow_gb300.h")
    for must in ("solve_hydro_2d", "set_timestep", "print_conservation",
                 "equation_of_state", "advect_momentum", "gb300_last_error"):
        assert must in names


@pytest.mark.parametrize("header", ["flow_gb300.h"])
def test_library_exports_every_declared_symbol(built, header):
    lib = ctypes.CDLL(built.LIB, mode=os.RTLD_LOCAL)
    missing = [n for n in declared(header) if not hasattr(lib, n)]
    assert not missing, missing


def test_status_calls_work_without_gpu(built):
    lib = ctypes.CDLL(built.LIB, mode=os.RTLD_LOCAL)
    lib.gb300_set_mode.argtypes = [ctypes.c_int]
    assert lib.gb300_set_mode(7) == 2          # unknown mode -> GB300_ERR_ARG
    assert lib.gb300_last_error() == 2
    lib.gb300_last_error_message.restype = ctypes.c_char_p
    assert b"unknown mode" in lib.gb300_last_error_message()
    lib.gb300_clear_error()
    assert lib.gb300_last_error() == 0
