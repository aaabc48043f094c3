"""CPU tests of the C ABI: the library builds for sm_103a, loads without a GPU, exports every entry
point include/skinny.h declares, and rejects bad arguments before touching the device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "skinny.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(skinny_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_the_reference_shaped_launchers():
    fns = declared_functions()
    for op in ("tsmttsm", "tsmm"):
        for s in ("s", "d", "c", "z", "dd"):
            assert f"skinny_{op}_{s}" in fns
    for f in ("skinny_create", "skinny_destroy", "skinny_tsmttsm", "skinny_tsmm", "skinny_svqb"):
        assert f in fns


def test_library_exports_every_declared_symbol(skinny_lib):
    for name in declared_functions():
        assert hasattr(skinny_lib, name), name


def test_python_binding_covers_every_declared_symbol():
    from skinny_matmul_gb300 import lib as L
    assert set(declared_functions()) <= set(L.SIGNATURES)


def test_status_strings(skinny_lib):
    from skinny_matmul_gb300 import lib as L
    for code, name in enumerate(L.STATUS_NAMES):
        assert skinny_lib.skinny_status_string(code).decode() == name


def test_bad_arguments_rejected_without_device(skinny_lib):
    from skinny_matmul_gb300 import lib as L
    one = ctypes.c_double(1.0)
    # null handle
    st = skinny_lib.skinny_tsmttsm(None, L.R64, L.ACC_NATIVE, 8, 8, 16, 16, 8, ctypes.byref(one), 16, 8,
                                   ctypes.byref(one), 32, 8, None)
    assert st == L.BAD_ARG
    # reference-shaped launcher with no device returns 0 and leaves a message
    r = skinny_lib.skinny_tsmttsm_d(1, 8, 8, 16, None, 8, 1.0, None, 8, 0.0, None, 8)
    assert r == 0


def test_group_and_grouping_arguments_rejected_without_device(skinny_lib):
    """skinny_group with no handle or a negative count, and set_grouping with a bad group size or
    no server, fail with SKINNY_BAD_ARG before any device work; a dry server accepts a valid
    grouping configuration."""
    from skinny_matmul_gb300 import lib as L
    from skinny_matmul_gb300.api import Server
    items = (L.GroupItem * 1)()
    assert skinny_lib.skinny_group(None, L.R64, items, 1, None) == L.BAD_ARG
    assert skinny_lib.skinny_group(None, L.R64, items, -1, None) == L.BAD_ARG
    assert skinny_lib.skinny_server_set_grouping(None, 1 << 20, 16) == L.BAD_ARG
    s = Server(None, 1 << 30)
    assert skinny_lib.skinny_server_set_grouping(s.s, 1 << 20, 0) == L.BAD_ARG
    assert skinny_lib.skinny_server_set_grouping(s.s, 1 << 20, 70000) == L.BAD_ARG
    assert skinny_lib.skinny_server_set_grouping(s.s, 0, 1) == L.OK  # grouping off
    s.close()


def test_launcher_list_shape():
    from skinny_matmul_gb300 import launchers
    for op in ("tsmttsm", "tsmm"):
        for dt in ("float32", "float64", "complex64", "complex128", "dd"):
            ls = launchers(op, dt)
            assert len(ls) == 1 and callable(ls[0][0]) and isinstance(ls[0][1], str)


def test_cpp_shim_header_compiles():
    """include/skinny.hpp (the reference's launcher spellings) compiles as C++17 against the CUDA
    headers, together with the C++ test program the GPU test runs."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    cuda_inc = "/usr/local/cuda/include"
    if gxx is None or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or the CUDA headers are missing")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-I", os.path.join(root, "include"), "-I", cuda_inc,
                        os.path.join(root, "tests", "cpp", "shim_driver.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
