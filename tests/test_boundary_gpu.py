"""The drop-in boundary on the GPU: DoComputationsW called exactly as the reference's own host
program calls it.

tests/golden/boundary_call.npz holds what the reference's SurfaceGrowth.cpp (its own compiled
host code: sugr_in.txt parsing, SetParams, SetupJob) hands to DoComputationsW for a short shear
input — the parameter block bytes, the velocities, the accelerations and the result file's
header (SurfaceGrowth.cpp:131-148, 399-469).  The initial positions are InitCoordsW's lattice:
here they come from the reference's own lattice kernels (SurfaceGrowth.cu:2532-2609) where
their cubin is present, and must equal the library's InitCoordsW output bit for bit.

The call runs the whole simulation through libsgmd's DoComputationsW (the C ABI the reference
program links against) in a fresh directory: 100 steps with the shear drive on from step 51
(deltaF from a 2 pN increment), summary rows every 10 steps, an RDF file at step 100 and pdb
snapshots at steps 0, 50, 100.  An oracle run of the same call writes its files through the
same writers (tests/oracle_outputs.py).  Integer columns (step counts) and pdb atom records must
be identical; the values agree to the tolerances below (the GPU's CUDA transcendental functions
and the oracle's libm differ by a few ulp, which a 100-step trajectory carries forward).
"""
import ctypes as C
import os
from pathlib import Path

import numpy as np
import pytest

import oracle_outputs as OO
from surfacegrowthconsole_gb300 import _lib as L
from surfacegrowthconsole_gb300.engine import init_coords

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "boundary_call.npz"

# summary columns: 0 step, 1 impulse, 2 totEn, 3 totEn.rms, 4 potEn, 5 potEn.rms, 6 T, 7 T.rms,
# 8 oneStep (wall time: not compared), 9 Veloc_CM, 10 CM, 11 friction, 12-14 size, 15 shear force.
# column -> (relative tolerance, column whose largest magnitude scales it).  The rms columns are
# sqrt(sum2/n - mean^2) in FP32 (AccumProps, SurfaceGrowth.cu:2674-2683): the subtraction cancels
# all but the last digits of mean^2, so their error scales with the mean, not with the rms.
COL_TOL = {1: (1e-3, 1), 2: (1e-5, 2), 3: (1e-4, 2), 4: (1e-5, 4), 5: (1e-4, 4), 6: (1e-3, 6), 7: (1e-3, 6),
           9: (1e-3, 9), 10: (1e-5, 10), 11: (1e-2, 11), 12: (1e-4, 12), 13: (1e-4, 13), 14: (1e-4, 14),
           15: (1e-6, 15)}
PRINT_ULP = 2e-7  # %7.7f


def load_call():
    z = np.load(GOLD)
    p = L.SimParams.from_buffer_copy(bytes(z["params"]))
    return z, p


def initial_positions(p):
    """InitCoordsW's lattice through the library, pinned to the reference's kernels when their
    cubin is present; also applies InitCoordsW's initUcellMeX/Y to p."""
    q = p.copy()
    r = init_coords(q)
    try:
        import refkern
    except ImportError:
        refkern = None
    if refkern is not None and refkern.available("nofma") is None:
        rr, qr = refkern.init_coords(p, "nofma")
        assert np.array_equal(r.view(np.uint32), rr.view(np.uint32))
        assert (q.initUcellMeX, q.initUcellMeY) == (qr.initUcellMeX, qr.initUcellMeY)
    p.initUcellMeX, p.initUcellMeY = q.initUcellMeX, q.initUcellMeY
    return r


def call_docomputations(p, hr, hv, ha, header: bytes, result_name: str):
    """The reference's main(): result file open with its header, then DoComputationsW."""
    Path(result_name).write_bytes(header)
    libc = L.libc()
    f = libc.fopen(result_name.encode(), b"a")
    pdb = C.create_string_buffer(b"sugr", 264)
    try:
        err = L.lib().DoComputationsW(hr.ctypes.data, hv.ctypes.data, ha.ctypes.data, C.byref(p), f, pdb)
    finally:
        libc.fclose(f)
    assert err is None, err


def test_docomputations_replays_the_reference_programs_call(tmp_path, monkeypatch):
    z, p = load_call()
    assert p.iRegime == 2 and p.nMolMe == 150 and p.deltaF > 0
    assert p.stepEquil + p.stepCool < p.stepLimit  # the shear drive runs inside the call
    hr = initial_positions(p)
    hv = np.ascontiguousarray(z["hv"])
    ha = np.ascontiguousarray(z["ha"])
    header = bytes(z["header"])
    name = str(z["result_name"])

    gdir, odir = tmp_path / "gpu", tmp_path / "oracle"
    gdir.mkdir()
    odir.mkdir()
    p_gpu = p.copy()
    r_gpu, v_gpu, a_gpu = hr.copy(), hv.copy(), ha.copy()
    monkeypatch.chdir(gdir)
    call_docomputations(p_gpu, r_gpu, v_gpu, a_gpu, header, name)

    monkeypatch.chdir(odir)
    Path(name).write_bytes(header)
    orc = OO.run_oracle_with_writers(p.copy(), hr, hv, ha, name)
    po = orc.params()

    # the parameter block comes back with the step loop's final counters and shear
    assert p_gpu.stepCount == po.stepCount == p.stepLimit
    assert p_gpu.shear == po.shear and p_gpu.shear > 0
    assert p_gpu.totalShear == po.totalShear and p_gpu.totalShear > 0
    assert p_gpu.shear < (p.stepLimit - p.stepEquil - p.stepCool) * p.deltaF * 1.0001

    # the same set of files
    assert OO.listdir_outputs(str(gdir)) == OO.listdir_outputs(str(odir))
    assert sorted(os.listdir(gdir)) == sorted(os.listdir(odir))

    # summary rows
    g = OO.summary_rows(str(gdir / name))
    o = OO.summary_rows(str(odir / name))
    assert g.shape == o.shape == (p.stepLimit // p.stepAvg, 16)
    assert np.array_equal(g[:, 0], o[:, 0])
    assert open(gdir / name, "rb").read().startswith(header)
    # every comparison below is collected, then reported together
    bad = []
    for c, (rtol, sc) in COL_TOL.items():
        scale = float(np.abs(o[:, sc]).max())
        err = float(np.abs(g[:, c] - o[:, c]).max())
        if err > rtol * scale + 2 * PRINT_ULP:
            bad.append(f"summary column {c}: max diff {err:.3g} (scale {scale:.3g}, rtol {rtol:g})")
    if not ((o[-1, 15] > 0) and (o[:5, 15] == 0).all()):  # the shear force column: off, then on
        bad.append("shear force column")

    # pdb snapshots: identical atom records, coordinates to one unit of the last printed digit
    # (CreatePdbFile prints %-8.2lf angstrom, SurfaceGrowth.cu:2780-2790: a trajectory difference
    # of a few ulp may flip it)
    for f in sorted(x for x in os.listdir(gdir) if x.endswith(".pdb")):
        hg, xg = OO.pdb_coords(str(gdir / f))
        ho, xo = OO.pdb_coords(str(odir / f))
        if hg != ho:
            bad.append(f"{f}: atom records differ")
        elif np.abs(xg - xo).max() > 0.01 + 1e-9:
            bad.append(f"{f}: coordinates differ by {np.abs(xg - xo).max():.3g} A")

    # RDF file: the normalised histogram of 100 samples
    rdf = [x for x in os.listdir(gdir) if x.startswith("rdf")]
    if len(rdf) != 1:
        bad.append(f"RDF files: {rdf}")
    else:
        ng, no = OO.numbers(str(gdir / rdf[0])), OO.numbers(str(odir / rdf[0]))
        if ng.shape != no.shape or no.max() <= 0:
            bad.append("RDF file shape")
        else:
            l1 = np.abs(ng - no).sum() / np.abs(no).sum()
            print(f"RDF L1 distance {l1:.3g}, identical: {bool(np.array_equal(ng, no))}")
            if l1 >= 1e-3:
                bad.append(f"RDF L1 distance {l1:.3g}")

    # final state handed back through the host arrays
    ro, vo, ao = orc.get_state()
    if np.abs(r_gpu[:, :3] - ro[:, :3]).max() >= 1e-3:
        bad.append(f"final positions differ by {np.abs(r_gpu[:, :3] - ro[:, :3]).max():.3g}")
    if np.abs(v_gpu - vo).max() >= 1e-3 * max(1.0, float(np.abs(vo).max())):
        bad.append("final velocities")
    assert not bad, "; ".join(bad)
