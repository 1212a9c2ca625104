"""CPU tests of the C ABI boundary: the library builds, loads, exports every
declared symbol, and validates arguments on the host (no GPU compute)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "holo.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(holo_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("holo_create", "holo_destroy", "holo_transform", "holo_transform_mc",
                 "holo_transform_batched", "holo_adjoint", "holo_last_error_string",
                 "holo_project", "holo_normalize_polar", "holo_plan_create"):
        assert must in names


def test_library_exports_every_declared_symbol(holo):
    lib = holo._native.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert set(declared_functions()) <= set(holo._native.SIGNATURES)


def test_header_is_plain_c_and_links(holo, tmp_path):
    """A C caller (the binding a cgo or FFI stub compiles against): the header is C99
    without warnings, and a program linked to libholo.so gets a status, never an exit,
    when there is no GPU to run on."""
    src = tmp_path / "caller.c"
    src.write_text('#include <stdio.h>\n#include "holo.h"\n'
                   "int main(void) {\n  holo_handle h;\n  int rc = holo_create(0, &h);\n"
                   "  if (rc == HOLO_OK) { holo_destroy(h); return 0; }\n"
                   '  printf("%d %s\\n", rc, holo_last_error_string());\n  return 0;\n}\n')
    lib_dir = os.path.dirname(holo._native.LIB_PATH)
    exe = tmp_path / "caller"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
                        "-I", os.path.join(REPO, "include"), str(src), "-L", lib_dir, "-lholo",
                        f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_abi_version(holo):
    assert holo._native.load().holo_abi_version() == 1


def test_variant_table_is_host_only(holo):
    for prec in ("split32", "fp64"):
        vs = holo.variants(prec)
        assert vs and all(v["target_tile"] == v["threads"] * v["targets_per_thread"] for v in vs)
        assert all(v["source_tile"] % 16 == 0 for v in vs)  # 16-byte bulk-copy granularity
    tts = {v["target_tile"] for v in holo.variants("split32")}
    assert {256, 512, 1024, 2048} <= tts  # Monte Carlo block sizes
    assert 0 <= holo.size_bucket(4096, 65536) < 8


def test_host_side_validation_without_gpu(holo):
    lib = holo._native.load()
    # null handles and outputs are rejected before any CUDA work
    assert lib.holo_transform(None, -1, 1e-6, None, None, None, 0, None, 0, None, 1, None) == -1
    assert lib.holo_plan_execute(None, -1, 1e-6, None, None, None, None) == -1
    out = ctypes.c_void_p()
    assert lib.holo_create(0, None) == -1
    rc = lib.holo_create(0, ctypes.byref(out))
    if rc != 0:  # no device here: a clean status, never an exit
        assert rc in (-7, -1, -2)
        assert lib.holo_last_error_string()
    else:
        lib.holo_destroy(out)
    assert lib.holo_variant_describe(1, 99, None, None, None, None, None, None) == -1
    assert lib.holo_set_variant(None, 1, 0, 0) == -1
    assert lib.holo_tile_order(None, None, 0, 0, None, None) == -1
    assert lib.holo_plan_tiling(None, None, None) == -1


def test_cli_help_and_argument_errors(holo):
    exe = os.path.join(os.path.dirname(holo.__file__), "holo")
    r = subprocess.run([exe, "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "-f {dir}" in r.stdout and "--precision" in r.stdout
    r = subprocess.run([exe, "-p", "7"], capture_output=True, text=True)
    assert r.returncode == 2 and "-p" in r.stderr
    r = subprocess.run([exe, "--precision", "fp16"], capture_output=True, text=True)
    assert r.returncode == 2
    r = subprocess.run([exe, "-w", "0"], capture_output=True, text=True)
    assert r.returncode == 2
    r = subprocess.run([exe, "--shape", "square"], capture_output=True, text=True)
    assert r.returncode == 2 and "shape" in r.stderr


def test_library_has_no_cpu_fallback(holo, tmp_path):
    """Loading fails loudly when libholo.so is absent."""
    with pytest.raises(ImportError):
        holo._native._lib, saved = None, holo._native._lib
        try:
            holo._native.load(str(tmp_path / "missing.so"))
        finally:
            holo._native._lib = saved
