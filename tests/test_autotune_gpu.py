"""Launch-shape tuning and launch modes: the lanes per metal atom of the density and metal force passes (4, 8,
16, 32) change only the summation order of the metal sums; the list build's algorithm (a warp per cell
or a thread per atom), blocks per SM, item size and cell order change nothing; sg_autotune
restores the context's state, so a tuned run continues exactly as an untuned one switched to
the chosen shape at the same step."""
import numpy as np
import pytest

from surfacegrowthconsole_gb300 import MODE_MIXED, MODE_PLAIN, workloads
from surfacegrowthconsole_gb300.engine import Simulation

pytestmark = pytest.mark.gpu

SUM_ORDER_RTOL = 2e-6


def _forces(p, r, v, **shape):
    sim = Simulation(p, **shape)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    sim.build_lists()
    sim.compute_forces()
    rg, _, a = sim.get_state()
    out = (a.astype(np.float64), rg[:, 3].astype(np.float64), sim.rho().astype(np.float64), sim.nebr())
    sim.close()
    return out


@pytest.mark.parametrize("lanes", [4, 8, 32])
def test_metal_lanes_change_only_the_summation_order(lanes):
    p, r, v = workloads.production(seed=2, steps=10)
    a16, e16, rho16, _ = _forces(p, r, v)
    a, e, rho, _ = _forces(p, r, v, metal_lanes=lanes)
    m = p.nMolMe
    assert np.array_equal(a[m:], a16[m:]), "carbon forces do not depend on the metal lanes"
    for name, x, y in (("metal acc", a[:m], a16[:m]), ("energy", e, e16), ("rho", rho, rho16)):
        err = np.abs(x - y).max() / np.abs(y).max()
        assert err <= SUM_ORDER_RTOL, (name, err)


def _lists(p, r, v, **shape):
    sim = Simulation(p, **shape)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    sim.build_lists()
    out = (*sim.nebr(), *sim.short_lists())
    sim.close()
    return out


@pytest.mark.parametrize("which", ["small", "production", "bulk"])
def test_list_builds_and_shapes_change_nothing(which):
    """The three list builds (cell windows with warp- or lane-placed hits in any grid, order and
    item size; atom threads) give the same full, close and relevant lists."""
    p, r, v = {"small": lambda: workloads.small(seed=3), "production": lambda: workloads.production(seed=2, steps=10),
               "bulk": lambda: workloads.bulk_metal(8, 600.0, 7)}[which]()
    ref = _lists(p, r, v)
    for kw in ({"nebr_build": 1}, {"nebr_build": 2}, {"nebr_build": 2, "nebr_item_atoms": 4, "nebr_descending": 1},
               {"nebr_blocks_per_sm": 1, "nebr_item_atoms": 16},
               {"nebr_blocks_per_sm": 4, "nebr_descending": 1, "nebr_item_atoms": 4},
               {"nebr_blocks_per_sm": 32, "nebr_descending": 1, "nebr_item_atoms": 64}):
        got = _lists(p, r, v, **kw)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b), kw


def test_bad_shapes_are_refused():
    p, r, v = workloads.small(seed=3)
    for kw in ({"metal_lanes": 6}, {"nebr_blocks_per_sm": 33}, {"nebr_item_atoms": 3}, {"nebr_build": 3},
               {"carbon_blocks_per_sm": 10}):
        with pytest.raises(Exception):
            Simulation(p, **kw)
    sim = Simulation(p)
    with pytest.raises(Exception):
        sim.set_launch_shape({"metal_lanes": 64})
    with pytest.raises(Exception):
        sim.set_launch_shape({"carbon_blocks_per_sm": 9})
    assert sim.launch_shape() == {"metal_lanes": 16, "nebr_blocks_per_sm": 7, "nebr_descending": 0,
                                  "nebr_item_atoms": 8, "programmatic_launch": 1, "nebr_build": 0,
                                  "eam_table_smem": 0, "carbon_blocks_per_sm": 8}
    sim.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_autotune_restores_the_state(mode):
    p, r, v = workloads.production(seed=2, steps=10)
    a0 = np.zeros((p.nMol, 3), np.float32)
    tuned = Simulation(p, mode=mode)
    tuned.set_state(r, v, a0)
    tuned.step(30)
    rep = tuned.autotune(steps=10)
    shape = tuned.launch_shape()
    assert shape == {f: rep[f] for f in Simulation.SHAPE_FIELDS}
    assert shape["metal_lanes"] in (4, 8, 16, 32) and shape["nebr_blocks_per_sm"] in (2, 4, 7, 14)
    assert shape["nebr_item_atoms"] in (4, 6, 8, 16) and shape["nebr_build"] in (0, 1, 2)
    for k in ("4", "8", "16", "32"):
        assert rep["metal_lanes_ms_per_step"][k] > 0
    plain = Simulation(p, mode=mode)
    plain.set_state(r, v, a0)
    plain.step(30)
    for x, y in zip(tuned.get_state(), plain.get_state()):
        assert np.array_equal(x, y), "state after sg_autotune"
    plain.set_launch_shape(shape)
    tuned.step(40)
    plain.step(40)
    for x, y in zip(tuned.get_state(), plain.get_state()):
        assert np.array_equal(x, y), "40 steps after sg_autotune"
    t1, t2 = tuned.thermo(), plain.thermo()
    assert t1.kinEnergy64 == t2.kinEnergy64 and float(t1.potEnergy) == float(t2.potEnergy)
    tuned.close()
    plain.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_programmatic_launch_changes_nothing(mode):
    """With programmatic dependent launch every kernel of a step still waits for its predecessor
    before touching memory: the trajectory is bit-identical."""
    p, r, v = workloads.production(seed=2, steps=10)
    out = []
    for pdl in (False, True):
        sim = Simulation(p, mode=mode, programmatic_launch=pdl, force_rebuild=True)
        sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
        sim.step(25)
        out.append(sim.get_state())
        sim.close()
    for x, y in zip(*out):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("lanes", [4, 16, 32])
def test_staged_eam_table_changes_nothing(lanes):
    """MIXED: the metal passes with the EAM table staged in shared memory read the same table
    values and do the same arithmetic: bit-identical forces, densities and energies."""
    reps = [workloads.small(seed=s) for s in (91, 92)]
    plist = [w[0] for w in reps]
    r = np.concatenate([w[1] for w in reps])
    v = np.concatenate([w[2] for w in reps])
    out = []
    for staged in (0, 1):
        sim = Simulation(plist, mode=MODE_MIXED, metal_lanes=lanes, eam_table_smem=staged)
        assert sim.launch_shape()["eam_table_smem"] == staged
        sim.set_state(r, v, np.zeros((len(r), 3), np.float32))
        sim.step(5)
        out.append([sim.get_state(k) for k in range(2)] + [sim.rho(k) for k in range(2)])
        sim.close()
    for a, b in zip(out[0], out[1]):
        for x, y in zip(a, b) if isinstance(a, tuple) else [(a, b)]:
            assert np.array_equal(x, y)


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_carbon_blocks_per_sm_change_nothing(mode):
    """The carbon pass compiled for 8, 12 or 16 resident blocks per SM (another register budget,
    the same source): PLAIN (no contraction) is bit-identical, MIXED agrees to FP32 rounding."""
    p, r, v = workloads.production(seed=2, steps=10)
    out = {}
    for cb in (8, 12, 16):
        sim = Simulation(p, mode=mode, carbon_blocks_per_sm=cb)
        assert sim.launch_shape()["carbon_blocks_per_sm"] == cb
        sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
        sim.build_lists()
        sim.compute_forces()
        out[cb] = sim.get_state()
        sim.close()
    for cb in (12, 16):
        for x, y in zip(out[cb], out[8]):
            if mode == MODE_PLAIN:
                assert np.array_equal(x, y), cb
            else:
                err = np.abs(x.astype(np.float64) - y).max() / max(np.abs(y).max(), 1e-30)
                assert err <= SUM_ORDER_RTOL, (cb, err)
