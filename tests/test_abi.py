"""CPU tests of the C ABI: the library builds for sm_103a, loads, exports every
declared symbol, and validates arguments on the host before touching a GPU."""
import ctypes as C
import os
import re

import pytest

import isar_imaging_cuda_gb300 as g

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    return set(re.findall(r"^ISAR_API\s+[^;(]*?\b(\w+)\s*\(", src, re.M))


def test_library_exports_every_declared_symbol():
    lib = g.load()
    names = declared("isar_gb300.h")
    assert names == set(g.EXPORTS)
    for n in names:
        assert hasattr(lib, n), n


def test_create_rejects_bad_sizes_before_touching_the_device():
    lib = g.load()
    h = C.c_void_p()
    cases = [
        (g.radar(2048, 4096), "echo_num"),          # > 1024 (isar_imaging_export.cpp:144)
        (g.radar(256, 256), "range_num"),           # < range_num_cut (:148)
        (g.radar(1024, 512), "range_num"),          # < echo_num (:152)
        (g.radar(384, 1024), "power of two"),
        (g.radar(256, 3000), "power of two"),
        (g.radar(256, 1024, data_type=3), "data_type"),
    ]
    for rp, msg in cases:
        rc = lib.isar_create(C.byref(h), C.byref(rp), 0, None)
        assert rc == -1, (rp.echo_num, rp.range_num)
        assert msg in g.last_error()


def test_null_context_is_an_error():
    lib = g.load()
    assert lib.isar_image_host(None, None, None, 0, None) == -1
    assert lib.isar_destroy(None) == 0
    assert lib.isar_test_barrier_timeout(None, 100, 1) == -1
