"""In-tree build of the native parts: libsgmd.so (CUDA kernels + C ABI, sm_103a) and the test
infrastructure: the CPU oracle (oracle/liboracle.so) and the loader of the reference kernels'
cubin (oracle/librefkern.so).

Each translation unit compiles in its own process, all in parallel; a unit is rebuilt only
when a source or header it may include is newer than its object.  No CMake, one -gencode.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INC = ROOT / "include"
LIBDIR = PKG / "lib"
ORACLE = ROOT / "oracle"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOSTFLAGS = "-fPIC,-ffp-contract=off,-O2"

LIBSGMD = LIBDIR / "libsgmd.so"
LIBORACLE = ORACLE / "liboracle.so"
LIBREFKERN = ORACLE / "librefkern.so"  # loads the reference kernels' cubin (tests only)

# (source, extra flags): the PLAIN kernels are compiled without FMA contraction so their
# arithmetic follows the reference's operation order exactly.
CUDA_UNITS = [
    ("sg_kernels_plain.cu", ["-fmad=false"]),
    ("sg_kernels_mixed.cu", []),
    ("sg_engine.cu", []),
    ("sg_run.cu", []),
    ("sg_noalloc.cu", []),
    ("sg_adjoint.cu", []),
]
CXX_UNITS = ["sg_host.cpp", "sg_refcompat.cpp"]


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INC.glob("*.h")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _obj(src: str) -> Path:
    return LIBDIR / "obj" / (src.replace(".", "_") + ".o")


def build(verbose: bool = False, force: bool = False) -> None:
    """Compile everything that is out of date."""
    (LIBDIR / "obj").mkdir(parents=True, exist_ok=True)
    hdrs = _headers()
    jobs = []
    for src, extra in CUDA_UNITS:
        o = _obj(src)
        if force or _stale(o, [CSRC / src] + hdrs):
            jobs.append([NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", HOSTFLAGS,
                         "-I", str(INC), "-I", str(CSRC), *extra, "-c", str(CSRC / src), "-o", str(o)])
    for src in CXX_UNITS:
        o = _obj(src)
        if force or _stale(o, [CSRC / src] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I", str(INC), "-I", str(CSRC), "-I", str(CUDA_HOME / "include"),
                         "-c", str(CSRC / src), "-o", str(o)])
    oracle_src = ORACLE / "sg_oracle.cpp"
    if force or _stale(LIBORACLE, [oracle_src, ORACLE / "sg_oracle.h", INC / "sg_api.h", INC / "sg_simparams.h"]):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
                     "-Wall", "-Wno-unused-function", str(oracle_src), "-o", str(LIBORACLE)])
    refkern_src = ORACLE / "ref" / "refkern.cpp"
    if refkern_src.exists() and (force or _stale(LIBREFKERN, [refkern_src, INC / "sg_simparams.h"])):
        # linked against the driver stub; the real libcuda.so.1 resolves at load time
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-I", str(INC),
                     "-I", str(CUDA_HOME / "include"), str(refkern_src), "-o", str(LIBREFKERN),
                     "-L" + str(CUDA_HOME / "lib64" / "stubs"), "-lcuda"])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, fut in [(j, ex.submit(_run, j)) for j in jobs]:
            if verbose:
                print(" ".join(cmd[:2]), cmd[-3], file=sys.stderr)
            fut.result()
    objs = [_obj(s) for s, _ in CUDA_UNITS] + [_obj(s) for s in CXX_UNITS]
    cudalib = str(CUDA_HOME / "lib64")
    if force or _stale(LIBSGMD, objs):
        _run(["g++", "-shared", "-o", str(LIBSGMD), *map(str, objs), "-L" + cudalib, "-lcudart",
              "-Wl,-rpath," + cudalib, "-Wl,--no-undefined"])


def clean() -> None:
    shutil.rmtree(LIBDIR, ignore_errors=True)
    for f in (LIBORACLE, LIBREFKERN):
        if f.exists():
            f.unlink()


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print("built", LIBSGMD, LIBORACLE)
