"""The C-ABI library builds, loads, and exports every entry point that
include/*.h declares. No compute call is made here (no GPU needed)."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(nbody_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "nbody_create" in names and "nbody_update_host" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(nb):
    lib = ctypes.CDLL(nb.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol(nb):
    assert sorted(nb.SIGNATURES) == declared_functions()


def test_status_strings(nb):
    assert nb.lib().nbody_status_string(0) == b"ok"
    assert nb.lib().nbody_status_string(5) == b"device wait timed out"


def test_bad_arguments_rejected_without_device(nb):
    L = nb.lib()
    ctx = ctypes.c_void_p()
    assert L.nbody_create(ctypes.byref(ctx), 0, 0, 0, 0.01, 1.0, 0.25) == nb.ERR_ARG      # n = 0
    assert L.nbody_create(ctypes.byref(ctx), 0, 7, 16, 0.01, 1.0, 0.25) == nb.ERR_ARG     # bad mode
    assert L.nbody_create(ctypes.byref(ctx), 0, 0, 16, 0.01, -1.0, 0.25) == nb.ERR_ARG    # eps2 < 0
    assert L.nbody_create(None, 0, 0, 16, 0.01, 1.0, 0.25) == nb.ERR_ARG
    assert L.nbody_step(None, 1) == nb.ERR_ARG


def test_create_fails_loudly_without_gpu(nb):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(nb.NBodyError) as e:
        nb.ParticleSolverCUDA(0.01, 1.0, 128)
    assert e.value.status in (nb.ERR_CUDA, nb.ERR_NOMEM)


def test_header_is_plain_c_and_links(nb, tmp_path):
    """include/nbody_gb300.h compiles as C99 with warnings as errors, and a C
    program that takes the address of every declared function links against
    the library (what a cgo / FFI binding needs)."""
    import re
    import shutil
    import subprocess

    if shutil.which("gcc") is None:
        pytest.skip("gcc missing")
    hdr = os.path.join(ROOT, "include", "nbody_gb300.h")
    names = sorted(set(re.findall(r"^[a-z_ ]*?\*?\s*(nbody_\w+)\(", open(hdr).read(), re.M)))
    assert len(names) > 30
    src = tmp_path / "use.c"
    src.write_text('#include "nbody_gb300.h"\n#include <stdio.h>\ntypedef void (*fn)(void);\n'
                   "int main(void) {\n    fn f[] = {" + ", ".join(f"(fn){n}" for n in names) +
                   "};\n    printf(\"%d %s\\n\", (int)(sizeof f / sizeof f[0]), nbody_status_string(NBODY_ERR_ARG));\n"
                   "    return 0;\n}\n")
    exe = tmp_path / "use"
    libdir = os.path.dirname(nb.LIB_PATH)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", f"-I{ROOT}/include", str(src),
                        "-o", str(exe), f"-L{libdir}", "-lnbody_gb300", f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.split()[0] == str(len(names))
