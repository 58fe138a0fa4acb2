"""Record the DoComputationsW call of the reference's own host program, for the boundary test.

The reference's SurfaceGrowth.cpp (compiled unmodified into oracle/_ref/libsgref_host.so by
oracle/ref/build_ref.sh, where the reference tree is present) reads sugr_in.txt, derives the
parameter block (SetParams), sets up the job (SetupJob: velocities from its generator, zero
accelerations, zeroed properties, the result file with its header) and then calls
DoComputationsW(hr, hv, ha, &params, fResult, "sugr").  This script runs that sequence for one
short shear input and stores what the call receives: the parameter block bytes, hv, ha, the
result file's header bytes and name.  The positions hr come from InitCoordsW's lattice kernels,
which need a GPU: tests/test_boundary_gpu.py takes them from the reference's own kernels there.

Writes tests/golden/boundary_call.npz.  Run: python tests/golden/make_boundary_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
from make_golden import REFLIB, SEED, input_text  # noqa: E402

# the 22 rows of sugr_in.txt: shear regime, Ni slab of 150 atoms on a 7 x 9 sheet (2,016 C), 300 K,
# dt 1 fs, 100 steps, averages every 10, equilibration 20, shear increment 2 pN after a 30-step
# cooling interval (so the shear drive runs steps 51-100), pdb every 50 steps, RDF every step
# (the compiled-in limitRdf of 100 samples prints one RDF file at step 100), no backups.
ROWS = [2, 3, 7, 9, 0, 300, 150, 0.0087381, 2.4945, 100, 0.005, 10, 20, 2.0, 30, 0.03, 40, 1100, 50, 1, 0, 0]
OUT = HERE / "boundary_call.npz"


def record(out_path: str) -> None:
    lib = C.CDLL(str(REFLIB))
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        Path("sugr_in.txt").write_text(input_text(ROWS))
        a = C.create_string_buffer(1112)
        b = C.create_string_buffer(1112)
        nm = C.create_string_buffer(264)
        n = lib.sgref_setup(b"sugr_in.txt", SEED, a, b, nm)
        if n <= 0:
            raise SystemExit(f"sgref_setup failed: {n}")
        hv = np.zeros((n, 3), np.float32)
        ha = np.zeros((n, 3), np.float32)
        lib.sgref_get_vels(hv.ctypes.data_as(C.c_void_p))
        lib.sgref_get_accels(ha.ctypes.data_as(C.c_void_p))
        header = Path(nm.value.decode()).read_bytes()
        np.savez_compressed(out_path, rows=np.array([str(x) for x in ROWS]), seed=np.int64(SEED),
                            params=np.frombuffer(b.raw, np.uint8), hv=hv, ha=ha,
                            header=np.frombuffer(header, np.uint8), result_name=np.array(nm.value.decode()),
                            input_text=np.array(input_text(ROWS)))


def main() -> None:
    if len(sys.argv) > 2 and sys.argv[1] == "--record":
        record(sys.argv[2])
        return
    if not REFLIB.exists():
        sys.exit(f"{REFLIB} missing: run oracle/ref/build_ref.sh with the reference tree first")
    # a fresh process: the reference keeps its configuration in process globals
    subprocess.run([sys.executable, __file__, "--record", str(OUT)], check=True)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
