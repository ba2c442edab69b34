"""The C-ABI library: loads without a GPU, exports every symbol declared in
include/cmgpu.h, and its struct layouts match the ctypes mirror."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "cmgpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(cm_\w+)\s*\(", src, re.M)))


def test_library_exports_header_symbols(cm):
    entry = __import__("__graft_entry__")
    path = entry.load_build().build()
    lib = C.CDLL(path)
    names = header_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(cm._native.EXPORTED)


def test_struct_sizes_match_header(cm):
    N = cm._native
    # field-by-field mirror of include/cmgpu.h on LP64
    assert C.sizeof(N.cm_system_desc) == 192
    assert C.sizeof(N.cm_frames) == 72
    assert C.sizeof(N.cm_counts) == 88
    assert C.sizeof(N.cm_raw_counts) == 64
    assert C.sizeof(N.cm_stats) == 104
    assert C.sizeof(N.cm_kernel_times) == 112
    assert C.sizeof(N.cm_server_desc) == 24
    assert C.sizeof(N.cm_request_info) == 48
    assert C.sizeof(N.cm_tuning) == 184
    assert C.sizeof(N.cm_dcd_layout) == 64
    assert C.sizeof(N.cm_contrib_query) == 24


STRUCTS = ("cm_system_desc", "cm_frames", "cm_counts", "cm_raw_counts", "cm_stats", "cm_kernel_times", "cm_tuning",
           "cm_dcd_layout", "cm_results", "cm_grid3d_desc", "cm_grid3d_out", "cm_server_desc", "cm_request_info",
           "cm_contrib_query")


def test_struct_layouts_match_c_compiler(cm, tmp_path):
    """Every field offset and struct size of the ctypes mirror equals what a
    C compiler makes of include/cmgpu.h."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    N = cm._native
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "cmgpu.h"', 'int main(void) {']
    for name in STRUCTS:
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for fname, _ in getattr(N, name)._fields_:
            lines.append(f'printf("{name}.{fname} %zu\\n", offsetof({name}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], check=True, capture_output=True, text=True)
               .stdout.splitlines())
    for name in STRUCTS:
        S = getattr(N, name)
        assert int(out[name]) == C.sizeof(S), name
        for fname, _ in S._fields_:
            assert int(out[f"{name}.{fname}"]) == getattr(S, fname).offset, f"{name}.{fname}"


def test_create_rejects_bad_descriptions_without_gpu(cm):
    """Argument checks run before any CUDA call, so they work without a GPU."""
    N = cm._native
    lib = N.load()
    d = N.cm_system_desc()
    d.api_version = N.CM_API_VERSION
    d.solute_nmols = d.solvent_nmols = 10
    d.solute_natomspermol = d.solvent_natomspermol = 3
    d.irefatom = 5  # > natomspermol
    d.cutoff = d.dbulk = 10.0
    d.binstep = 0.02
    d.nbins = 500
    d.n_random_samples = 10
    d.lcell = 1
    h = C.c_void_p()
    assert lib.cm_create(C.byref(d), C.byref(h)) == N.CM_EINVAL
    assert b"Reference atom index" in lib.cm_last_error(None)
    d.irefatom = 1
    d.usecutoff = 1
    assert lib.cm_create(C.byref(d), C.byref(h)) == N.CM_EINVAL
    assert b"bulk volume is zero" in lib.cm_last_error(None)
    d.usecutoff = 0
    d.nbins = 10
    assert lib.cm_create(C.byref(d), C.byref(h)) == N.CM_EINVAL
    d.nbins = 500
    d.launch = 7
    assert lib.cm_create(C.byref(d), C.byref(h)) == N.CM_EINVAL
    assert b"launch mode" in lib.cm_last_error(None)
    d.launch = N.CM_LAUNCH_GRAPH
    d.kernel_timing = 1   # per-launch timing events cannot be captured
    assert lib.cm_create(C.byref(d), C.byref(h)) == N.CM_EINVAL
    assert b"kernel_timing" in lib.cm_last_error(None)
    assert lib.cm_destroy(None) == N.CM_OK
    assert lib.cm_status_string(N.CM_EDEVICE) == b"device-side check failed"


def test_engine_fails_loudly_without_library(cm, tmp_path):
    N = cm._native
    with pytest.raises(N.NativeUnavailable):
        saved = N._lib
        N._lib = None
        try:
            N.load(str(tmp_path / "missing.so"))
        finally:
            N._lib = saved


def test_memory_cache_query_without_gpu(cm):
    """cm_memory_cache reads the process-wide block cache without touching a
    device (nothing is cached in a process that opened no handle) and rejects a
    bad device index."""
    N = cm._native
    lib = N.load()
    dev, host = C.c_int64(-1), C.c_int64(-1)
    assert lib.cm_memory_cache(0, 0, C.byref(dev), C.byref(host)) == N.CM_OK
    assert dev.value >= 0 and host.value >= 0
    assert lib.cm_memory_cache(-1, 0, None, None) == N.CM_EINVAL
    assert lib.cm_memory_cache(1 << 20, 0, None, None) == N.CM_EINVAL


def test_batch_create_rejects_bad_arguments_without_gpu(cm):
    N = cm._native
    lib = N.load()
    out = C.c_void_p()
    assert lib.cm_batch_create(None, 1, C.byref(out)) == N.CM_EINVAL
    arr = (C.c_void_p * 2)(None, None)
    assert lib.cm_batch_create(arr, 0, C.byref(out)) == N.CM_EINVAL
    assert lib.cm_batch_create(arr, 2, C.byref(out)) == N.CM_EINVAL
    assert b"NULL handle" in lib.cm_last_error(None)
    assert lib.cm_batch_submit(None, None) == N.CM_EINVAL
    assert lib.cm_batch_destroy(None) == N.CM_OK


def test_server_create_rejects_bad_arguments_without_gpu(cm):
    """Server argument checks come before any device use."""
    N = cm._native
    lib = N.load()
    d = N.cm_server_desc()
    d.device = 0
    d.frames_per_turn = -1
    s = C.c_void_p()
    assert lib.cm_server_create(C.byref(d), C.byref(s)) == N.CM_EINVAL
    assert b"negative" in lib.cm_server_last_error(None)
    assert lib.cm_server_destroy(None) == N.CM_OK
