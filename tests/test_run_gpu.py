"""The whole-run path (sg_run, what DoComputationsW drives) on the GPU: the summary rows at every
stepAvg, the RDF files after every limitRdf samples, the Diffuse.txt tables and the pdb files,
at the reference's cadence and in its formats, with the values of a context stepped the same
way through sg_step."""
import glob
import os

import numpy as np
import pytest

from surfacegrowthconsole_gb300 import MODE_MIXED, MODE_PLAIN, workloads
from surfacegrowthconsole_gb300.engine import Simulation

pytestmark = pytest.mark.gpu

EV = 0.06275049


def _params(tmp):
    p, r, v = workloads.small(seed=71)
    p.stepLimit = 300
    p.stepAvg = 100
    p.stepRdf = 50
    p.limitRdf = 2
    p.bPdb = 1
    p.stepPdb = 100
    p.bBckup = 0
    p.stepDiffuse = 2
    p.nValDiffuse = 10
    p.nBuffDiffuse = 2
    p.limitDiffuseAv = 2
    p.szRdfPath = os.path.join(tmp, "rdf").encode()
    p.szDiffusePath = os.path.join(tmp, "Diffuse.txt").encode()
    return p, r, v


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_whole_run_writes_the_reference_outputs(tmp_path, mode):
    tmp = str(tmp_path)
    p, r, v = _params(tmp)
    assert p.iRegime == 2 and p.nMolMe > 0
    sim = Simulation(p, mode=mode)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    res = os.path.join(tmp, "sg.txt")
    sim.run(res, os.path.join(tmp, "sugr"))
    last = sim.thermo()
    sim.close()

    rows = [l.split() for l in open(res).read().splitlines() if l.strip() and l.split()[0].isdigit()]
    assert [int(x[0]) for x in rows] == [100, 200, 300]
    for x in rows:
        assert len(x) == 16 and all(np.isfinite(float(t)) for t in x)
    assert "Duration of the simulation" in open(res).read()

    rdf = sorted(glob.glob(os.path.join(tmp, "rdf_stepCount_*")))
    assert [int(f.split("_stepCount_")[1].split("_")[0]) for f in rdf] == [100, 200, 300]
    for f in rdf:
        assert len(open(f).read().splitlines()) == p.sizeHistRdf

    diff = open(os.path.join(tmp, "Diffuse.txt")).read().splitlines()
    heads = [i for i, l in enumerate(diff) if l == "diffusion"]
    assert heads, "no diffusion table"
    assert all(len(diff[h + 1:h + 1 + p.nValDiffuse]) == p.nValDiffuse for h in heads)

    assert len(glob.glob(os.path.join(tmp, "sugr_*.pdb"))) == 4  # the initial state + 3 outputs

    # the same steps through sg_step: the run's final state record
    ref = Simulation(p, mode=mode)
    ref.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    ref.step(300)
    t = ref.thermo()
    ref.close()
    assert t.stepCount == last.stepCount == 300
    assert np.isclose(float(t.totEnergy), float(last.totEnergy), rtol=1e-6, atol=1e-7)
    # the last summary row's mean total energy (eV) is the mean of the last 100 steps
    assert abs(float(rows[-1][2]) - float(t.totEnergy) * EV) < 0.05
