"""Backups on the GPU: the whole-run path writes bckup0/1.sugr at the reference's cadence
(SurfaceGrowth.cu:2456-2481, alternating files every stepBckup steps), and a context created
from a backup continues bit for bit like the run that was never interrupted in PLAIN.  MIXED
carries each position as a float pair (hi + lo); the reference's backup format stores the float
positions only, so a MIXED run resumes from the rounded positions and stays within a few ulp.
"""
import os

import numpy as np
import pytest

from surfacegrowthconsole_gb300 import MODE_MIXED, MODE_PLAIN, workloads
from surfacegrowthconsole_gb300.engine import Simulation
from test_backup import read_backup, write_backup

pytestmark = pytest.mark.gpu


def _rebuild_due_step(p, r, v, a, mode, lo, hi):
    sim = Simulation(p, mode=mode)
    sim.set_state(r, v, a)
    sim.step(lo)
    for k in range(lo, hi):
        sim.step(1)
        if sim.thermo().nebrNow:
            sim.close()
            return k + 1
    sim.close()
    raise AssertionError("no rebuild due in the window")


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED], ids=["plain", "mixed"])
def test_kill_and_resume_is_bit_exact(tmp_path, mode):
    p, r, v = workloads.small(seed=91)
    a = np.zeros((p.nMol, 3), np.float32)
    total = 60
    k = _rebuild_due_step(p, r, v, a, mode, 20, total - 5)  # past the thermostat step 25 or not
    run = Simulation(p, mode=mode)
    run.set_state(r, v, a)
    run.step(k)
    f = tmp_path / "bckup0.sugr"
    rk, vk, ak = run.get_state()
    write_backup(f, run.params(), rk, vk, ak)
    run.step(total - k)
    q, r2, v2, a2 = read_backup(f)
    assert q.stepCount == k and q.nebrNow == 1
    res = Simulation(q, mode=mode)
    res.set_state(r2, v2, a2)
    res.step(total - k)
    t0, t1 = run.thermo(), res.thermo()
    assert t0.stepCount == t1.stepCount == total
    if mode == MODE_PLAIN:
        for x, y in zip(run.get_state(), res.get_state()):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
        assert t0.totEnergy == t1.totEnergy
    else:
        (x0, v0, _), (x1, v1, _) = run.get_state(), res.get_state()
        assert np.abs(x0[:, :3] - x1[:, :3]).max() < 1e-4
        assert np.abs(v0 - v1).max() < 1e-4 * float(np.abs(v0).max())
        assert abs(t0.totEnergy - t1.totEnergy) < 1e-5 * abs(t0.totEnergy)
    run.close()
    res.close()


def test_whole_run_writes_alternating_backups(tmp_path, monkeypatch):
    """stepBckup 50 over 150 steps: bckup0 at 50, bckup1 at 100, bckup0 again at 150.  The
    last file holds the final state; a context resumed from the step-100 file with rebuilds in
    every step reaches it bit for bit."""
    monkeypatch.chdir(tmp_path)
    p, r, v = workloads.small(seed=92)
    p.stepLimit = 150
    p.stepAvg = 50
    p.bBckup = 1
    p.stepBckup = 50
    p.bPdb = 0
    a = np.zeros((p.nMol, 3), np.float32)
    sim = Simulation(p, force_rebuild=True)
    sim.set_state(r, v, a)
    sim.run(str(tmp_path / "sg.txt"))
    rf, vf, af = sim.get_state()
    sim.close()
    b0 = read_backup(tmp_path / p.szBckup0.decode())
    b1 = read_backup(tmp_path / p.szBckup1.decode())
    assert b0[0].stepCount == 150 and b1[0].stepCount == 100
    for x, y in zip((rf, vf, af), b0[1:]):
        assert np.array_equal(x, y)
    res = Simulation(b1[0], force_rebuild=True)
    res.set_state(*b1[1:])
    res.step(50)
    for x, y in zip((rf, vf, af), res.get_state()):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    res.close()
    assert os.path.getsize(tmp_path / p.szBckup0.decode()) == 1112 + p.nMol * 40
