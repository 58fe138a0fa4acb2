"""Generate golden fixtures from the reference's own host code.

Runs where the reference tree is present and oracle/ref/build_ref.sh has built
oracle/_ref/libsgref_host.so from it.  Each case runs in a fresh
subprocess because the reference keeps its configuration in process globals.  Writes
tests/golden/ref_host.json plus the output files under tests/golden/ref_files/.

The fixtures pin: sugr_in.txt parsing + SetParams/SetupJob (the whole SimParams block, the
result-file name and header), InitVels velocities for a given seed, the RandR/VRand streams,
and the exact bytes of PrintSummary rows, CreatePdbFile, PrintRdf and the diffusion table.
"""
from __future__ import annotations

import base64
import ctypes as C
import hashlib
import json
import os
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REFLIB = ROOT / "oracle" / "_ref" / "libsgref_host.so"
FILES = HERE / "ref_files"

# (name, 22 row values) -- the rows of sugr_in.txt in the reference's order
CASES = {
    "bulk_ag_shipped": [0, 1, 8, 8, 8, 330, 25000, 0.0087381, 2.4945, 100000, 0.001, 250, 30000, 0.0001, 120000,
                        0.03, 40, 1100, 1000, 50, 0, 0],
    "bulk_cu_small": [0, 0, 4, 5, 6, 500, 100, 0.0087381, 2.4945, 2000, 0.002, 20, 10, 0.0001, 100, 0.03, 40, 1100,
                      100, 50, 0, 0],
    "shear_ni_300": [2, 3, 7, 9, 0, 300, 300, 0.0087381, 2.4945, 1000, 0.005, 100, 0, 0.0, 1000, 0.03, 40, 1100,
                     500, 100, 0, 0],
    "shear_ni_2000": [2, 3, 10, 12, 0, 700, 2000, 0.01, 2.6, 5000, 0.001, 250, 1000, 0.0001, 500, 0.03, 40, 1100,
                      1000, 50, 1, 0],
    "shear_au_25000": [2, 2, 30, 30, 0, 330, 25000, 0.0087381, 2.4945, 100000, 0.001, 250, 30000, 0.0001, 120000,
                       0.03, 40, 1100, 1000, 50, 0, 0],
    "growth_al_1500": [1, 4, 8, 8, 0, 600, 1500, 0.0087381, 2.4945, 10000, 0.001, 100, 500, 0.0001, 100, 0.05, 30,
                       200, 1000, 50, 0, 0],
    "growth_pb_50": [1, 5, 3, 2, 0, 0, 50, 0.0087381, 2.4945, 100, 0.001, 0, 10, 0.0001, 100, 0.03, 40, 10, 10, 5,
                     0, 0],
}
SEED = 12345


def input_text(vals) -> str:
    lines = ["# generated input", ""]
    for i, v in enumerate(vals):
        lines.append(f"{v}         # row {i + 1}")
        if i == 9:
            lines.append("   # an indented comment line")
    return "\n".join(lines) + "\n"


def one_case(name: str, vals, out: dict) -> None:
    lib = C.CDLL(str(REFLIB))
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        Path("sugr_in.txt").write_text(input_text(vals))
        a = C.create_string_buffer(1112)
        b = C.create_string_buffer(1112)
        nm = C.create_string_buffer(264)
        n = lib.sgref_setup(b"sugr_in.txt", SEED, a, b, nm)
        assert n > 0, n
        vel = (C.c_float * (3 * n))()
        lib.sgref_get_vels(vel)
        vbytes = bytes(vel)
        header = Path(nm.value.decode()).read_bytes()
        out.update(name=name, rows=vals, nMol=n, after_setparams=base64.b64encode(a.raw).decode(),
                   after_setup=base64.b64encode(b.raw).decode(), result_name=nm.value.decode(),
                   header=base64.b64encode(header).decode(), vel_sha256=hashlib.sha256(vbytes).hexdigest(),
                   vel_head=list(struct.unpack_from(f"{min(3 * n, 96)}f", vbytes)))


def writers(params_b64: str) -> dict:
    """Drive the reference writers on synthetic data; returns file names -> contents."""
    lib = C.CDLL(str(REFLIB))
    out = {}
    p = C.create_string_buffer(base64.b64decode(params_b64), 1112)
    nmol, nme = struct.unpack_from("ii", p.raw, 88)
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        # summary rows: 23 steps, stepAvg forced to 5 (offset 60)
        struct.pack_into("i", p, 60, 5)
        vals = (C.c_float * (16 * 23))()
        for s in range(23):
            for k in range(16):
                vals[16 * s + k] = ((s * 7 + k * 13) % 17 - 8) * 0.173 + (0.0371 * k if k != 3 else 0.51 + 0.01 * s)
        lib.sgref_summary_seq(p, 23, vals, b"summary.txt", C.c_float(12.625))
        # pdb: synthetic positions, stepCount 3 * stepPdb (offset 72 stepPdb, 68 stepCount)
        pos = (C.c_float * (4 * nmol))()
        for i in range(nmol):
            pos[4 * i + 0] = (i % 37) * 0.61 - 11.3
            pos[4 * i + 1] = (i % 23) * -0.47 + 5.2
            pos[4 * i + 2] = (i % 11) * 0.29 - 1.7
        stepPdb = struct.unpack_from("i", p.raw, 72)[0]
        for mult in (3, 150, 1200, 12000):
            struct.pack_into("i", p, 68, stepPdb * mult)
            lib.sgref_pdb(b"sugr", p, pos)
        # rdf: synthetic histogram, countRdf = 7, particle size set
        sz = struct.unpack_from("i", p.raw, 484)[0]
        hist = (C.c_uint * sz)(*[(k * 37) % 101 for k in range(sz)])
        struct.pack_into("i", p, 492, 7)
        struct.pack_into("fff", p, 444, 6.25, 7.5, 5.125)
        struct.pack_into("i", p, 68, 4321)
        lib.sgref_rdf(p, hist)
        # diffusion: 3 buffers of 8 values, limit 2, stepDiffuse 10
        struct.pack_into("iiiii", p, 828, 8, 3, 10, 2, 0)
        ncm = 70
        cm = (C.c_float * (3 * ncm))()
        for i in range(ncm):
            cm[3 * i] = 0.37 * i - 0.02 * i * i
            cm[3 * i + 1] = 0.11 * i
            cm[3 * i + 2] = -0.05 * i
        lib.sgref_diffusion_seq(p, ncm, cm, b"Diffuse.txt")
        for f in sorted(Path(".").iterdir()):
            data = f.read_bytes()
            if f.suffix == ".pdb" and nmol > 500:  # large snapshots: content hash only
                out[f.name] = {"sha256": hashlib.sha256(data).hexdigest(), "head": data[:1600].decode()}
            else:
                out[f.name] = base64.b64encode(data).decode()
        out["_summary_vals"] = [vals[i] for i in range(16 * 23)]
        out["_nmol"] = nmol
        out["_hist"] = list(hist)
        out["_cm"] = [cm[i] for i in range(3 * ncm)]
    return out


def rng_streams() -> dict:
    lib = C.CDLL(str(REFLIB))
    r = (C.c_float * 1000)()
    lib.sgref_rand(SEED, 1000, r)
    v3 = (C.c_float * 600)()
    lib.sgref_vrand(SEED, 200, v3, 0)
    v4 = (C.c_float * 600)()
    lib.sgref_vrand(SEED, 200, v4, 1)
    return dict(seed=SEED, randR=list(r), vrand=list(v3), vrand_f4=list(v4))


def main() -> None:
    if len(sys.argv) > 1 and sys.argv[1] == "--case":
        res = {}
        if sys.argv[2] == "__writers__":
            res = writers(sys.argv[3])
        elif sys.argv[2] == "__rng__":
            res = rng_streams()
        else:
            one_case(sys.argv[2], CASES[sys.argv[2]], res)
        print(json.dumps(res))
        return
    if not REFLIB.exists():
        sys.exit(f"{REFLIB} missing: run oracle/ref/build_ref.sh first")

    def sub(*args):
        r = subprocess.run([sys.executable, __file__, "--case", *args], capture_output=True, text=True, check=True)
        return json.loads(r.stdout)

    golden = {"cases": {}, "note": "generated by tests/golden/make_golden.py from the reference's host code"}
    for name in CASES:
        golden["cases"][name] = sub(name)
    golden["rng"] = sub("__rng__")
    # writers driven with the shear Ni and growth Al parameter blocks
    golden["writers"] = {}
    for name in ("shear_ni_300", "growth_pb_50", "bulk_cu_small"):
        golden["writers"][name] = sub("__writers__", golden["cases"][name]["after_setup"])
    (HERE / "ref_host.json").write_text(json.dumps(golden, indent=1))
    print("wrote", HERE / "ref_host.json")


if __name__ == "__main__":
    main()
