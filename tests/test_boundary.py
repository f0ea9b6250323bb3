"""CPU tests of the drop-in boundary: the C-ABI library loads and exports every declared symbol,
and the host-side checks reject bad input before any device work."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from piclas_gb300 import EXPORTED_SYMBOLS, build, capi, library_path, load_library

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "piclas_gpu.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pic_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return load_library()


def test_header_matches_python_binding():
    assert header_functions() == sorted(EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", library_path()], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (pic_[a-z0-9_]+)\b", out))
    missing = [s for s in header_functions() if s not in exported]
    assert not missing, missing
    for s in header_functions():
        assert hasattr(lib, s)


def test_version_and_error_string(lib):
    assert b"sm_103a" in lib.pic_version()
    assert isinstance(lib.pic_last_error(), bytes)


def test_null_arguments_rejected_without_device_work(lib):
    h = C.c_void_p()
    assert lib.pic_create(None, None, C.byref(h)) == 1          # PIC_ERR_INVALID_ARGUMENT
    assert lib.pic_step(None, 1e-12, 1, None) == 1
    assert lib.pic_deposit(None, None) == 1
    assert lib.pic_get_status(None, None) == 1
    lib.pic_destroy(None)                                       # no-op


def test_bad_options_rejected(lib):
    from piclas_gb300.mesh import build_box_mesh
    mesh = build_box_mesh(2, 2, 2, 1)
    ms = capi.MeshStruct(mesh)
    h = C.c_void_p()
    cfg = capi.make_config(9, 1, 1, 0, [(-1.0, 1.0, 1.0)], 10)     # N = 9 unsupported
    assert lib.pic_create(C.byref(cfg), ms.ptr, C.byref(h)) == 1
    cfg = capi.make_config(1, 7, 1, 0, [(-1.0, 1.0, 1.0)], 10)     # unknown tracking
    assert lib.pic_create(C.byref(cfg), ms.ptr, C.byref(h)) == 1
    cfg = capi.make_config(1, 1, 2, 0, [(-1.0, 1.0, 1.0)], 10, sf_radius=0.0)   # SF without radius
    assert lib.pic_create(C.byref(cfg), ms.ptr, C.byref(h)) == 1
    assert b"radius" in lib.pic_last_error()


def test_time_step_factor_above_one_rejected(lib):
    """The reference stops with 'Species-specific time step only allows factors below 1!'
    (particle_emission_init.f90:218-219); pic_create rejects such a factor before any device work."""
    from piclas_gb300.mesh import build_box_mesh
    ms = capi.MeshStruct(build_box_mesh(2, 2, 2, 1))
    h = C.c_void_p()
    for f in (1.0000001, 3.0, float("inf"), float("nan"), -0.5):
        cfg = capi.make_config(1, 1, 1, 0, [(-1.0, 1.0, 1.0), (1.0, 1836.0, 1.0)], 10, time_step_factor=(1.0, f))
        assert lib.pic_create(C.byref(cfg), ms.ptr, C.byref(h)) == 1, f
        assert b"time_step_factor" in lib.pic_last_error()


def test_struct_sizes_match_c():
    # pic_config_t: 6 ints + 3*8 + 6 doubles + 2 doubles + 5 ints + 4 bytes tail padding (8-byte alignment)
    # ... + time_step_factor[8] + periodic_tracing + ref_mapping_guess (int32 each, in the former tail padding)
    assert C.sizeof(capi.PicConfig) == 6 * 4 + 3 * 8 * 8 + 6 * 8 + 2 * 8 + 5 * 4 + 4 + 8 * 8 + 4 + 4
    assert C.sizeof(capi.PicStatus) == 24


def test_mesh_and_config_layout_match_c(tmp_path):
    """The ctypes mirrors have the C structs' sizes and field offsets (compiled against include/piclas_gpu.h)."""
    src = tmp_path / "layout.c"
    fields = [f for f, _ in capi.PicMesh._fields_]
    lines = ["#include <stddef.h>", "#include <stdio.h>", f'#include "{HEADER}"', "int main(void) {",
             '  printf("%zu\\n", sizeof(pic_mesh_t));', '  printf("%zu\\n", sizeof(pic_config_t));']
    lines += [f'  printf("%zu\\n", offsetof(pic_mesh_t, {f}));' for f in fields]
    lines += ["  return 0;", "}"]
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == C.sizeof(capi.PicMesh)
    assert out[1] == C.sizeof(capi.PicConfig)
    assert out[2:] == [getattr(capi.PicMesh, f).offset for f in fields]


def test_p_adaption_mapping_checked_before_device_work(lib):
    """N_DG_Mapping is validated on the host: degrees outside 1..n_dg, offsets that are not the running sum of
    (Nloc+1)^3, or a missing N_Inter table are PIC_ERR_INVALID_ARGUMENT."""
    from piclas_gb300.mesh import build_box_mesh
    nl = np.array([1, 2, 3, 1, 2, 3, 1, 2], np.int32)
    mesh = build_box_mesh(2, 2, 2, 3, n_loc=nl)
    h = C.c_void_p()
    cfg = capi.make_config(3, 1, 1, 0, [(-1.0, 1.0, 1.0)], 10)
    for case in ("degree", "offset", "table"):
        ms = capi.MeshStruct(mesh)
        g = ms._keep["ndg"]
        if case == "degree":
            g[3, 1] = 4
        elif case == "offset":
            g[5, 0] += 1
        else:
            ms.struct.n_inter = C.POINTER(C.c_double)()
        assert lib.pic_create(C.byref(cfg), ms.ptr, C.byref(h)) == 1, case
        assert b"n_dg_mapping" in lib.pic_last_error() or b"n_inter" in lib.pic_last_error()
    cfg2 = capi.make_config(2, 1, 1, 0, [(-1.0, 1.0, 1.0)], 10)   # NMax below the largest degree
    assert lib.pic_create(C.byref(cfg2), capi.MeshStruct(mesh).ptr, C.byref(h)) == 1
