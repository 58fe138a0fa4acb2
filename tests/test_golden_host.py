"""The host layer against golden outputs recorded from the reference's own host code
(tests/golden/make_golden.py): sugr_in.txt parsing and SetParams/SetupJob (whole parameter
block, byte for byte), InitVels velocities, the RNG streams, the result-file name and header,
and the bytes written by the summary, pdb, rdf and diffusion writers."""
import base64
import ctypes as C
import hashlib
import json
import os
import struct
from pathlib import Path

import numpy as np
import pytest

import oracle
from surfacegrowthconsole_gb300 import _lib as L
from surfacegrowthconsole_gb300.engine import (default_input, init_coords, init_vels, read_input_file,
                                               set_params)

G = json.loads((Path(__file__).parent / "golden" / "ref_host.json").read_text())
CASES = sorted(G["cases"])


def write_input(path: Path, rows):
    lines = ["# generated input", ""]
    for i, v in enumerate(rows):
        lines.append(f"{v}         # row {i + 1}")
        if i == 9:
            lines.append("   # an indented comment line")
    path.write_text("\n".join(lines) + "\n")


def product_params(tmp_path, case):
    g = G["cases"][case]
    f = tmp_path / "sugr_in.txt"
    write_input(f, g["rows"])
    inp = read_input_file(str(f))
    inp.randSeed = 12345
    p = set_params(inp)
    return inp, p


@pytest.mark.parametrize("case", CASES)
def test_params_block_byte_identical(tmp_path, case):
    inp, p = product_params(tmp_path, case)
    v = init_vels(p)  # InitVels advances the seed, as SetupJob does
    ref = base64.b64decode(G["cases"][case]["after_setup"])
    mine = bytes(C.string_at(C.addressof(p), C.sizeof(p)))
    diff = [i for i in range(len(ref)) if ref[i] != mine[i]]
    assert not diff, f"{case}: {len(diff)} bytes differ, first at offset {diff[0]}"
    assert hashlib.sha256(v.tobytes()).hexdigest() == G["cases"][case]["vel_sha256"]


@pytest.mark.parametrize("case", CASES)
def test_result_file_name_and_header(tmp_path, case):
    inp, p = product_params(tmp_path, case)
    name = C.create_string_buffer(264)
    L.check(L.lib().sg_result_file_name(C.byref(p), name, 264))
    assert name.value.decode() == G["cases"][case]["result_name"]
    libc = L.libc()
    out = tmp_path / "hdr.txt"
    fp = libc.fopen(str(out).encode(), b"w")
    L.lib().sg_print_result_header(fp, C.byref(p), C.c_float(inp.deposEnergyEv))
    libc.fclose(fp)
    assert out.read_bytes() == base64.b64decode(G["cases"][case]["header"])


def test_rng_streams_via_growth_lattice():
    # regime-1 metal atoms are placed with VRandRfloat4 scaled to the box (SurfaceGrowth.cu:2562-2569)
    inp = default_input()
    inp.iRegime = 1; inp.nMolMe = 200; inp.ucx = 8; inp.ucy = 8; inp.randSeed = G["rng"]["seed"]
    p = set_params(inp)
    r = init_coords(p)
    ref = np.array(G["rng"]["vrand_f4"], np.float32).reshape(-1, 3)
    exp_x = np.float32(0.5) * np.float32(p.region.x) * ref[:, 0]
    exp_y = np.float32(0.5) * np.float32(p.region.y) * ref[:, 1]
    assert np.array_equal(r[:200, 0], exp_x) and np.array_equal(r[:200, 1], exp_y)


def _writers(case):
    return G["writers"][case]


@pytest.mark.parametrize("case", sorted(G["writers"]))
def test_summary_rows_byte_identical(tmp_path, case):
    w = _writers(case)
    p = L.SimParams.from_buffer_copy(base64.b64decode(G["cases"][case]["after_setup"]))
    p.stepAvg = 5
    vals = np.array(w["_summary_vals"], np.float32).reshape(23, 16)
    libc = L.libc()
    out = tmp_path / "summary.txt"
    fp = libc.fopen(str(out).encode(), b"a")
    lib = L.lib()
    lib.sg_accum_props(C.byref(p), 0)
    for s in range(23):
        v = vals[s]
        p.stepCount = s + 1
        p.totEnergy.val, p.potEnergy.val, p.kinEnergy.val, p.oneStep.val = v[0], v[1], v[2], v[3]
        p.centerOfMass.val, p.cmVel.val, p.frictForce.val = v[4], v[5], v[6]
        p.vSum.x, p.vSum.y, p.vSum.z = v[7], v[8], v[9]
        p.particleSize.x, p.particleSize.y, p.particleSize.z = v[10], v[11], v[12]
        p.totalShear = v[13]
        lib.sg_accum_props(C.byref(p), 1)
        if p.stepCount % p.stepAvg == 0:
            lib.sg_accum_props(C.byref(p), 2)
            lib.sg_print_summary(fp, C.byref(p))
            lib.sg_accum_props(C.byref(p), 0)
    libc.fflush(fp)
    libc.fclose(fp)
    with open(out, "a") as f:
        f.write("\nDuration of the simulation = %f s" % np.float32(12.625))
    assert out.read_bytes() == base64.b64decode(w["summary.txt"])


@pytest.mark.parametrize("case", sorted(G["writers"]))
def test_pdb_and_rdf_files_byte_identical(tmp_path, case, monkeypatch):
    w = _writers(case)
    p = L.SimParams.from_buffer_copy(base64.b64decode(G["cases"][case]["after_setup"]))
    n = w["_nmol"]
    i = np.arange(n)
    pos = np.zeros((n, 4), np.float32)
    pos[:, 0] = (i % 37).astype(np.float32) * np.float32(0.61) - np.float32(11.3)
    pos[:, 1] = (i % 23).astype(np.float32) * np.float32(-0.47) + np.float32(5.2)
    pos[:, 2] = (i % 11).astype(np.float32) * np.float32(0.29) - np.float32(1.7)
    # the reference computed these positions in double and stored floats
    pos[:, 0] = ((i % 37) * 0.61 - 11.3).astype(np.float32)
    pos[:, 1] = ((i % 23) * -0.47 + 5.2).astype(np.float32)
    pos[:, 2] = ((i % 11) * 0.29 - 1.7).astype(np.float32)
    monkeypatch.chdir(tmp_path)
    lib = L.lib()
    for mult in (3, 150, 1200, 12000):
        p.stepCount = p.stepPdb * mult
        L.check(lib.sg_create_pdb(b"sugr", C.byref(p), pos.ctypes.data_as(C.c_void_p)))
    for fname, ref in w.items():
        if not fname.endswith(".pdb"):
            continue
        data = (tmp_path / fname).read_bytes()
        if isinstance(ref, dict):
            assert hashlib.sha256(data).hexdigest() == ref["sha256"], fname
        else:
            assert data == base64.b64decode(ref), fname
    hist = np.array(w["_hist"], np.uint32)
    p.countRdf = 7
    p.particleSize.x, p.particleSize.y, p.particleSize.z = 6.25, 7.5, 5.125
    p.stepCount = 4321
    L.check(lib.sg_print_rdf(C.byref(p), hist.ctypes.data_as(C.c_void_p)))
    rdf_name = [k for k in w if k.startswith("rdf_")][0]
    assert (tmp_path / rdf_name).read_bytes() == base64.b64decode(w[rdf_name])


@pytest.mark.parametrize("case", sorted(G["writers"]))
def test_diffusion_table_oracle_and_writer(tmp_path, case):
    """The oracle's EvalDiffusion restatement fed the recorded centre-of-mass sequence, printed
    with the product's writer, reproduces the reference's Diffuse.txt."""
    w = _writers(case)
    p = L.SimParams.from_buffer_copy(base64.b64decode(G["cases"][case]["after_setup"]))
    p.nValDiffuse, p.nBuffDiffuse, p.stepDiffuse, p.limitDiffuseAv, p.countDiffuseAv = 8, 3, 10, 2, 0
    cm = np.array(w["_cm"], np.float32).reshape(-1, 3)
    tables = oracle.diffusion_replay(p, cm)
    libc = L.libc()
    out = tmp_path / "Diffuse.txt"
    fp = libc.fopen(str(out).encode(), b"w")
    for t in tables:
        L.lib().sg_print_diffusion(fp, C.byref(p), t.ctypes.data_as(C.c_void_p))
    libc.fclose(fp)
    assert out.read_bytes() == base64.b64decode(w["Diffuse.txt"])


def test_input_parser_quirks(tmp_path):
    """Leading blanks make a row's value 0 and a last line without newline is ignored, as in
    the reference's reader (SurfaceGrowth.cpp:647-686)."""
    f = tmp_path / "sugr_in.txt"
    f.write_text("2 # regime\n   3 # indented value reads as 0\n#c\n\n9\n11")
    inp = read_input_file(str(f))
    assert inp.iRegime == 2 and inp.iMaterial == 0 and inp.ucx == 9 and inp.ucy == 7  # 11 not read
