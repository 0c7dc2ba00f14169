"""CPU checks of the C ABI library: it loads, exports every function that
include/mrpop.h declares, and validates arguments without touching a GPU."""
import ctypes as C
import re
from pathlib import Path

import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "mrpop.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mrpop_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_expected_entry_points(pkg):
    names = declared_functions()
    assert set(pkg.mrpop.EXPORTED) == set(names)


def test_library_exports_every_declared_symbol(lib_path):
    lib = C.CDLL(str(lib_path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_argument_validation_without_gpu(pkg, lib_path):
    lib = pkg.library(path=lib_path)
    h = C.c_void_p()
    assert lib.mrpop_robotset_create(0, None, C.byref(h)) == 1
    assert b"n_arms" in lib.mrpop_last_error()
    assert lib.mrpop_robotset_create(3, None, C.byref(h)) == 1  # no built-in 3-arm layout
    for n in (1, 4, 5):
        assert lib.mrpop_robotset_create(n, None, C.byref(h)) == 0
        # composite validate with null scene -> invalid argument, no device work
        assert lib.mrpop_validate_edges(None, h, None, None, 1, 32, 3, -1, None, None, None) == 1
        assert lib.mrpop_robotset_destroy(h) == 0
    assert lib.mrpop_version().startswith(b"mrpop-gb300")


def test_bad_flags_and_granularity_rejected(pkg, lib_path):
    import numpy as np
    lib = pkg.library(path=lib_path)
    rb = C.c_void_p()
    assert lib.mrpop_robotset_create(4, None, C.byref(rb)) == 0
    fake = C.c_void_p(1)  # never dereferenced: argument checks come first
    assert lib.mrpop_validate_edges(fake, rb, fake, fake, 4, 65, 3, -1, fake, fake, None) == 1
    assert b"granularity" in lib.mrpop_last_error()
    assert lib.mrpop_validate_edges(fake, rb, fake, fake, 4, 32, 0x100, -1, fake, fake, None) == 1
    assert lib.mrpop_validate_edges(fake, rb, fake, fake, 4, 32, 3, 4, fake, fake, None) == 1
    lib.mrpop_robotset_destroy(rb)


def test_server_arguments_rejected_without_gpu(pkg, lib_path):
    lib = pkg.library(path=lib_path)
    h = C.c_void_p()
    bad = pkg.mrpop.ServerConfig(1 << 20, 17, 0, 0)  # more than 16 launch slots
    assert lib.mrpop_server_create(C.byref(bad), C.byref(h)) == 1
    assert b"streams" in lib.mrpop_last_error()
    assert lib.mrpop_server_create(None, None) == 1
    assert lib.mrpop_session_open(None, 4, 64, 32, 0, C.byref(h)) == 1
    assert lib.mrpop_session_submit(None, None) == 1
    assert lib.mrpop_session_wait(None, 0) == 1
    assert lib.mrpop_session_close(None) == 0
    assert lib.mrpop_server_destroy(None) == 0


def test_session_and_plan_entry_points_reject_null_handles(pkg, lib_path):
    """The bindings of the serving and planning entry points marshal their
    arguments (checked on the CPU: null handles are refused before any device work)."""
    lib = pkg.library(path=lib_path)
    p = [C.c_void_p() for _ in range(4)]
    assert lib.mrpop_session_host_buffers(None, *[C.byref(x) for x in p]) == 1
    st = pkg.mrpop.PlanSettingsC(64, 60, 32, 5, 32, 1.0, 1.0, 7)
    res = pkg.mrpop.PlanResultC()
    start = (C.c_float * 28)()
    assert lib.mrpop_session_plan(None, None, None, 3, start, start, C.byref(st), None, 0, C.byref(res)) == 1
    assert lib.mrpop_plan(4, start, start, C.byref(st), pkg.mrpop.VALIDATE_FN(), None, None, 0, C.byref(res)) == 1
    assert lib.mrpop_plan(6, start, start, C.byref(st), pkg.mrpop.VALIDATE_FN(lambda *a: 0), None, None, 0,
                          C.byref(res)) == 1
    stats = pkg.mrpop.ServerStats()
    assert lib.mrpop_server_get_stats(None, C.byref(stats)) == 1
