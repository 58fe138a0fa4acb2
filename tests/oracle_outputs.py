"""TEST HELPER: a whole run of the CPU oracle written through the library's host writers.

The reference's DoComputationsW (SurfaceGrowthConsole/SurfaceGrowth.cu:2128-2494) writes a
summary row every stepAvg steps (AccumProps + PrintSummary, cu:2439-2445, 2689-2731), an
rdf_* file after every limitRdf samples (PrintRdf, cu:2812-2844), the Diffuse.txt tables
(EvalDiffusion / PrintDiffusion, cu:2865-2952) and a sugr_*.pdb snapshot at the start and every
stepPdb steps (CreatePdbFile, cu:2734-2810).  This module steps the FP32 oracle one step at a
time and, at the same steps, hands the oracle's values to the same writers (sg_accum_props,
sg_print_summary, sg_print_rdf, sg_print_diffusion, sg_create_pdb, which are byte-identical to
the reference's own, tests/test_golden_host.py), so that a run of the library and a run of the
oracle produce files that can be compared value by value.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

import oracle
from surfacegrowthconsole_gb300 import _lib as L

# the seven property accumulators in the order the oracle reports them
PROPS = ("totEnergy", "potEnergy", "kinEnergy", "oneStep", "centerOfMass", "cmVel", "frictForce")


def run_oracle_with_writers(p, r, v, a, result_path: str, pdb_prefix: str = "sugr"):
    """Runs p.stepLimit steps of the FP32 oracle from (r, v, a) in the current directory,
    appending summary rows to result_path; returns the oracle (final state)."""
    lib = L.lib()
    libc = L.libc()
    orc = oracle.OracleSim(p, 32)
    orc.set_state(r, v, a)
    if p.bPdb:
        q0 = orc.params()
        lib.sg_create_pdb(pdb_prefix.encode(), C.byref(q0), np.ascontiguousarray(r, np.float32).ctypes.data)
    fres = libc.fopen(result_path.encode(), b"a")
    fdiff = libc.fopen(p.szDiffusePath, b"w") if (p.iRegime == 2) else None
    n_rdf = n_diff = 0
    try:
        for sc in range(1, p.stepLimit + 1):
            orc.step(1)
            q = orc.params()
            while orc.num_diffusion_tables() > n_diff:
                t = orc.diffusion_table(n_diff)
                lib.sg_print_diffusion(fdiff, C.byref(q), t.ctypes.data)
                n_diff += 1
            if orc.num_rdf_prints() > n_rdf:
                qr = q.copy()
                qr.countRdf = p.limitRdf
                h = orc.rdf_print()
                lib.sg_print_rdf(C.byref(qr), h.ctypes.data)
                n_rdf += 1
            if sc % p.stepAvg == 0 and p.bResult:
                qa = q.copy()
                for name, prop in zip(PROPS, orc.last_avg()):
                    setattr(qa, name, prop)
                lib.sg_accum_props(C.byref(qa), 2)
                lib.sg_print_summary(fres, C.byref(qa))
            if p.bPdb and sc % p.stepPdb == 0:
                rr = orc.get_state()[0]
                lib.sg_create_pdb(pdb_prefix.encode(), C.byref(q), rr.ctypes.data)
    finally:
        libc.fclose(fres)
        if fdiff:
            libc.fclose(fdiff)
    return orc


def summary_rows(path: str) -> np.ndarray:
    """The numeric rows of a result file (16 columns each)."""
    rows = []
    for line in open(path).read().splitlines():
        f = line.split()
        if len(f) == 16 and f[0].isdigit():
            rows.append([float(x) for x in f])
    return np.array(rows)


def pdb_coords(path: str) -> tuple[list[str], np.ndarray]:
    """ATOM records of a pdb file: the fixed-column text before the coordinates, and x, y, z."""
    heads, xyz = [], []
    for line in open(path).read().splitlines():
        if line.startswith("ATOM"):
            heads.append(line[:30])
            xyz.append([float(line[30:38]), float(line[38:46]), float(line[46:54])])
    return heads, np.array(xyz)


def numbers(path: str) -> np.ndarray:
    """All numbers of a text file, in order (rdf and diffusion tables)."""
    out = []
    for line in open(path).read().splitlines():
        for tok in line.split():
            try:
                out.append(float(tok))
            except ValueError:
                pass
    return np.array(out)


def listdir_outputs(d: str) -> list[str]:
    return sorted(f for f in os.listdir(d) if f.startswith(("rdf", "sugr_", "Diffuse")))
