"""MIXED ("chosen") form: the same model as PLAIN with hi/lo positions, FMA contraction,
tabulated EAM pair functions and FP64 reductions.  Checked against the FP64 oracle (forces on
thermalised states, NVE energy drift) and against PLAIN (same model: energies of one step)."""
import numpy as np
import pytest

import oracle
from surfacegrowthconsole_gb300 import MODE_MIXED, MODE_PLAIN, workloads
from surfacegrowthconsole_gb300.engine import Simulation

pytestmark = pytest.mark.gpu

EV = 0.06275049  # energy unit, eV


def thermalised(p, r, v, steps=40):
    """A state some steps into the run: forces no longer cancel to round-off as in the perfect
    lattices the generators build."""
    sim = Simulation(p)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    sim.step(steps)
    r2, v2, _ = sim.get_state()
    sim.close()
    return r2, v2


def forces(p, r, v, mode):
    sim = Simulation(p, mode=mode)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    sim.build_lists()
    sim.compute_forces()
    a = sim.get_state()[2].astype(np.float64)
    sim.close()
    return a


def bulk_ni(n=10, T=300, seed=5):
    return workloads.bulk_metal(n, T, seed)


@pytest.mark.parametrize("which", ["small", "production", "bulk"])
def test_forces_against_the_fp64_oracle(which):
    """RMS force error relative to the RMS force, MIXED and PLAIN against the FP64 oracle on the
    same FP32 positions: MIXED (FMA, tables) is no less accurate than PLAIN."""
    p, r, v = {"small": lambda: workloads.small(seed=81), "production": lambda: workloads.production(seed=2),
               "bulk": bulk_ni}[which]()
    r, v = thermalised(p, r, v)
    o = oracle.OracleSim(p, 64)
    o.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    o.build_lists()
    o.compute_forces()
    a64 = o.get_state64()[2]
    scale = np.sqrt((a64 ** 2).mean())
    err = {m: float(np.sqrt(((forces(p, r, v, m) - a64) ** 2).mean()) / scale) for m in (MODE_PLAIN, MODE_MIXED)}
    print(which, "rms force error vs FP64: plain", err[MODE_PLAIN], "mixed", err[MODE_MIXED])
    assert err[MODE_MIXED] <= 1e-4
    assert err[MODE_MIXED] <= 2.0 * err[MODE_PLAIN] + 1e-7


def test_replicas_together_equal_each_alone():
    reps = [workloads.small(seed=s) for s in (82, 83, 84)]
    plist = [w[0] for w in reps]
    sim = Simulation(plist, mode=MODE_MIXED)
    sim.set_state(np.concatenate([w[1] for w in reps]), np.concatenate([w[2] for w in reps]),
                  np.zeros((sum(q.nMol for q in plist), 3), np.float32))
    sim.step(30)
    for k, (q, r, v) in enumerate(reps):
        one = Simulation(q, mode=MODE_MIXED)
        one.set_state(r, v, np.zeros((q.nMol, 3), np.float32))
        one.step(30)
        rb, vb, _ = sim.get_state(k)
        ro, vo, _ = one.get_state()
        assert np.array_equal(rb, ro) and np.array_equal(vb, vo), f"replica {k}"
        assert sim.thermo(k).kinEnergy64 == one.thermo().kinEnergy64
        one.close()
    sim.close()


def test_one_step_energies_match_plain():
    p, r, v = workloads.production(seed=2)
    th = {}
    for m in (MODE_PLAIN, MODE_MIXED):
        sim = Simulation(p, mode=m)
        sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
        sim.step(1)
        th[m] = sim.thermo()
        sim.close()
    for k in ("kinEnergy", "potEnergy"):
        a, b = getattr(th[MODE_MIXED], k + "64"), getattr(th[MODE_PLAIN], k)
        assert abs(a - b) <= 2e-5 * abs(b), (k, a, b)


def test_nve_drift_no_worse_than_plain():
    """Bulk Ni (a conservative EAM system), 10,000 NVE steps (10 ps): the linear drift of the
    total energy.  The reference's graphene model does not conserve energy (it applies the
    second-neighbour angle force but leaves its energy out), so drift is measured on the metal."""
    p, r, v = bulk_ni()
    steps, every = 10000, 100
    drift = {}
    for m in (MODE_PLAIN, MODE_MIXED):
        sim = Simulation(p, mode=m)
        sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
        es = []
        for _ in range(steps // every):
            sim.step(every)
            t = sim.thermo()
            es.append(t.kinEnergy64 + t.potEnergy64 if m == MODE_MIXED else float(t.totEnergy))
        sim.close()
        x = np.arange(len(es)) * every
        drift[m] = abs(np.polyfit(x, np.array(es), 1)[0]) * 1e6 * EV  # eV / atom / ns (1 step = 1 fs)
    print("NVE drift eV/atom/ns: plain", drift[MODE_PLAIN], "mixed", drift[MODE_MIXED])
    assert drift[MODE_MIXED] <= drift[MODE_PLAIN] + 2e-5
    assert drift[MODE_MIXED] < 1e-3


def crowded_cell_state(n_blob=90, seed=7):
    """The 2,217-atom system with n_blob cluster atoms pressed into one cell of the vacuum above
    the sheet (well above the reference's 64-atom cap, far from every other atom)."""
    p, r, v = workloads.small(seed=seed)
    r = r.copy()
    L = np.array([p.region.x, p.region.y, p.region.z], np.float64)
    inv = np.array([p.invWidth.x, p.invWidth.y, p.invWidth.z], np.float64)
    cells = np.array([p.cells.x, p.cells.y, p.cells.z])
    c = np.array([cells[0] // 2, cells[1] // 2, cells[2] - 2])  # high above the sheet at z_0
    lo = c / inv - 0.5 * L
    rng = np.random.RandomState(seed)
    blob = lo + (0.2 + 0.6 * rng.uniform(size=(n_blob, 3))) / inv
    r[:n_blob, :3] = blob.astype(np.float32)
    return p, r, v


@pytest.mark.parametrize("n_blob", [90, 300], ids=["bucket", "compaction"])
def test_mixed_lists_a_cell_above_the_reference_cap(n_blob):
    """PLAIN keeps the reference's 64 atoms per cell and reports a fuller cell; MIXED builds the
    same cells and lists as the (uncapped) oracle: from its 256-slot buckets (90 atoms), or, for a
    cell above them (300 atoms), by ordered compaction over the replica's atoms.  The 300-atom
    cell's atoms have 299 neighbours each, so both sides take 512-entry list rows."""
    p, r, v = crowded_cell_state(n_blob=n_blob)
    if n_blob > 100:
        p.iNebrMax = 512
    a = np.zeros((p.nMol, 3), np.float32)
    orc = oracle.OracleSim(p, 32)
    orc.set_state(r, v, a)
    orc.build_lists()
    _, cs, _ = orc.cells()
    assert np.diff(cs).max() == n_blob > p.blockSize
    plain = Simulation(p, mode=MODE_PLAIN)
    plain.set_state(r, v, a)
    with pytest.raises(Exception) as e:
        plain.build_lists()
    assert "CELL_OVERFLOW" in str(e.value)
    plain.close()
    mixed = Simulation(p, mode=MODE_MIXED)
    mixed.set_state(r, v, a)
    mixed.build_lists()
    for g, o in zip(mixed.cells(), orc.cells()):
        assert np.array_equal(g, o)
    nn_g, nbl_g = mixed.nebr()
    nn_o, nbl_o = orc.nebr()
    assert np.array_equal(nn_g, nn_o) and np.array_equal(nbl_g, nbl_o)
    d = mixed.diag()
    assert d.max_cell_occupancy == n_blob and d.nebr_overflow == 0
    assert d.cell_overflow == (1 if n_blob > 4 * p.blockSize else 0)  # counted, not raised
    mixed.close()
