"""The C ABI of libtinytrace_cuda.so without a GPU: the library builds, loads and exports
every function include/tinytrace_cuda.h declares; struct sizes agree between the header, the
Python mirror and the reference layouts; host-side argument checks answer without a device.
No call here launches device work.
"""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tinytrace_gb300 import native

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "tinytrace_cuda.h"


def header_functions() -> set[str]:
    text = HEADER.read_text()
    return set(re.findall(r"^\s*(?:int32_t|const char\*)\s+(tt_\w+)\s*\(", text, re.M))


def header_defines() -> dict[str, int]:
    out = {}
    for name, value in re.findall(r"^#define\s+(TT_\w+)\s+(\d+)u?\b", HEADER.read_text(), re.M):
        out[name] = int(value)
    return out


@pytest.fixture(scope="module")
def lib():
    from tinytrace_gb300 import build

    build.build()
    return native.load()


def test_header_declares_the_python_signatures():
    assert header_functions() == set(native.SIGNATURES), "header and native.SIGNATURES disagree"


def test_library_exports_every_declared_function(lib):
    path = Path(lib._name)
    for name in sorted(header_functions()):
        assert hasattr(lib, name), f"{name} is not exported"
    nm = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True)
    if nm.returncode == 0:
        exported = {line.split()[-1] for line in nm.stdout.splitlines() if " T " in line}
        missing = header_functions() - exported
        assert not missing, missing


def test_constants_match_header():
    defines = header_defines()
    for name, value in defines.items():
        if hasattr(native, name):
            assert getattr(native, name) == value, name
    for name in ("TT_OK", "TT_ERR_NO_DEVICE", "TT_OPTION_ACCEL", "TT_ACCEL_FLAT", "TT_TRACE_NOALLOC_MAX_RAYS",
                 "TT_OPTION_LIGHT_VISIBILITY", "TT_OPTION_LIGHT_SELECTION", "TT_TEXTURE_BC5_UNORM"):
        assert name in defines


def test_struct_sizes():
    # src/lib.rs:234-250 Constants, src/asset/material.rs MaterialConstants / Material,
    # src/asset/mod.rs Vertex and EmissiveTriangle, src/scene.rs:236-246 Instance
    assert native.CONSTANTS_DTYPE.itemsize == 368
    assert native.MATERIAL_CONSTANTS_DTYPE.itemsize == 192
    assert native.MATERIAL_DTYPE.itemsize == 304
    assert native.VERTEX_DTYPE.itemsize == 8
    assert native.INSTANCE_DTYPE.itemsize == 208
    assert native.EMISSIVE_DTYPE.itemsize == 36
    assert native.MESH_DTYPE.itemsize == 32
    assert ctypes.sizeof(native.SceneStats) == 10 * 8
    assert ctypes.sizeof(native.TraversalCounters) == 8 * 8
    assert ctypes.sizeof(native.Timings) == 3 * 8
    assert ctypes.sizeof(native.MeshData) == 5 * 8 + 2 * 4
    assert ctypes.sizeof(native.EmissiveSource) == 9 * 8


def test_abi_version(lib):
    assert lib.tt_abi_version() == header_defines()["TT_ABI_VERSION"]


def test_host_side_errors_without_device(lib):
    assert lib.tt_context_create(0, None) == native.TT_ERR_INVALID_ARGUMENT
    assert b"null" in lib.tt_last_error()
    assert lib.tt_context_destroy(None) == native.TT_OK
    assert lib.tt_set_option(None, native.TT_OPTION_ACCEL, 0) == native.TT_ERR_INVALID_ARGUMENT
    assert lib.tt_synchronize(None) == native.TT_ERR_INVALID_ARGUMENT
    h = ctypes.c_void_p()
    rc = lib.tt_context_create(0, ctypes.byref(h))
    if rc == native.TT_ERR_NO_DEVICE:  # the usual case on a machine without a GPU
        assert b"no CUDA device" in lib.tt_last_error()
        assert not h.value
    else:
        assert rc == native.TT_OK
        assert lib.tt_context_destroy(h) == native.TT_OK


def test_load_fails_loudly_without_library(tmp_path, monkeypatch):
    monkeypatch.setenv("TINYTRACE_CUDA_LIB", str(tmp_path / "missing.so"))
    monkeypatch.setattr(native, "_lib", None)
    with pytest.raises(native.TinytraceError):
        native.load()


def test_handles_and_dtypes_roundtrip():
    c = np.zeros((), native.CONSTANTS_DTYPE)
    assert c.nbytes == 368
    assert native.NODE4_DTYPE.itemsize == 128 and native.TRI_RECORD_DTYPE.itemsize == 48


def _compile_c(tmp_path, header_dir: Path, name: str) -> subprocess.CompletedProcess:
    src = tmp_path / f"{name}.c"
    src.write_text('#include "tinytrace_cuda.h"\nint main(void) { return 0; }\n')
    return subprocess.run(["gcc", "-std=c11", "-Wall", "-pedantic", "-Werror", f"-I{header_dir}", "-c", str(src),
                           "-o", str(tmp_path / f"{name}.o")], capture_output=True, text=True)


def test_header_layout_checks_compile_as_c11(tmp_path):
    """The header's _Static_assert layout checks (sizes and field offsets of the reference's
    #[repr(C)] types) hold for a C11 compiler, and they catch a reordered field."""
    ok = _compile_c(tmp_path, HEADER.parent, "ok")
    assert ok.returncode == 0, ok.stderr
    bad_dir = tmp_path / "bad"
    bad_dir.mkdir()
    text = HEADER.read_text()
    swapped = text.replace("    uint32_t tonemap;\n    uint32_t light_sampling;\n",
                           "    uint32_t light_sampling;\n    uint32_t tonemap;\n")
    assert swapped != text
    (bad_dir / "tinytrace_cuda.h").write_text(swapped)
    bad = _compile_c(tmp_path, bad_dir, "bad")
    assert bad.returncode != 0 and "Constants.tonemap at 360" in bad.stderr


def test_rust_sys_crate_declares_every_function():
    """rust/tinytrace_cuda_sys mirrors the header: every declared function and every #define
    constant appear there (source-only crate: no Rust toolchain on this machine)."""
    text = (ROOT / "rust" / "tinytrace_cuda_sys" / "src" / "lib.rs").read_text()
    declared = set(re.findall(r"pub fn (tt_\w+)\(", text))
    assert declared == header_functions()
    consts = dict(re.findall(r"pub const (TT_\w+): \w+ = (\d+);", text))
    for name, value in header_defines().items():
        assert name in consts, name
        assert int(consts[name]) == value, name
