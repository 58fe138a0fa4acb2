"""The C ABI boundary, without a GPU: libsgmd.so loads and exports every function the headers in
include/ declare, the parameter block has the reference's layout, and the reference's own host
program (SurfaceGrowth.cpp, unchanged) links against libsgmd.so in place of its SurfaceGrowth.cu.
"""
import ctypes as C
import re
import subprocess
import tempfile
from pathlib import Path

import pytest

from surfacegrowthconsole_gb300 import _lib as L

ROOT = Path(__file__).resolve().parent.parent
HEADERS = [ROOT / "include" / "sg_api.h", ROOT / "include" / "sg_refcompat.h"]
LINKED = ROOT / "oracle" / "_ref" / "sugr_on_sgmd"


def declared_c_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        text = re.sub(r"#[^\n]*", "", text)
        text = re.sub(r"typedef[^;]*;", "", text, flags=re.S)
        for stmt in text.split(";"):
            m = re.search(r"\b([A-Za-z_]\w*)\s*\([^()]*(?:\([^()]*\)[^()]*)*\)\s*$", stmt.strip())
            if m and m.group(1) not in ("if", "while", "sizeof", "AccumProps"):
                names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_reference_wrappers_and_the_sg_api():
    names = declared_c_functions()
    for n in ("CudaInitW", "SetParametersW", "InitCoordsW", "DoComputationsW", "sg_create", "sg_step",
              "sg_compute_forces_noalloc"):
        assert n in names
    assert len(names) > 40


def test_library_exports_every_declared_function():
    lib = L.lib()
    missing = [n for n in declared_c_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_accum_props_is_exported_with_the_reference_signature():
    # void AccumProps(int, SimParams *) with C++ linkage, as SurfaceGrowth.cpp calls it
    out = subprocess.run(["nm", "-D", "--defined-only", str(L.LIBPATH)], capture_output=True, text=True).stdout
    assert "_Z10AccumPropsiP9SimParams" in out


def test_simparams_layout_is_the_reference_layout():
    assert C.sizeof(L.SimParams) == 1112
    for field, off in (("kinEnergy", 152), ("szNameMe", 304), ("szRdfPath", 504), ("szDiffusePath", 848)):
        assert getattr(L.SimParams, field).offset == off, field


@pytest.mark.skipif(not LINKED.exists(), reason="the reference host program was not linked here "
                                                 "(oracle/ref/build_ref.sh needs the reference tree)")
def test_reference_host_program_links_and_runs_against_libsgmd():
    und = subprocess.run(["nm", "-D", "--undefined-only", str(LINKED)], capture_output=True, text=True).stdout
    for sym in ("CudaInitW", "SetParametersW", "InitCoordsW", "DoComputationsW", "_Z10AccumPropsiP9SimParams"):
        assert sym in und, f"{sym} is not taken from a shared library"
    deps = subprocess.run(["ldd", str(LINKED)], capture_output=True, text=True).stdout
    assert "libsgmd.so" in deps and "not found" not in deps
    # it starts and stops on its own checks (no device here, or no input file in an empty directory)
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([str(LINKED)], cwd=d, capture_output=True, text=True, timeout=60, stdin=subprocess.DEVNULL)
    assert r.returncode == 1
    assert any(m in r.stdout for m in ("no CUDA capable devices", "less than 1.2", "Error with input file"))
