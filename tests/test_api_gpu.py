"""The host-buffer calls of the sg_* C ABI: state uploads and downloads round-trip exactly, and
sg_step_thermo's record is the one sg_get_thermo reads after sg_step."""
import numpy as np
import pytest

from surfacegrowthconsole_gb300 import MODE_MIXED, MODE_PLAIN, workloads
from surfacegrowthconsole_gb300.engine import Simulation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_state_round_trip(mode):
    reps = [workloads.small(seed=s) for s in (61, 62)]
    plist = [w[0] for w in reps]
    sim = Simulation(plist, mode=mode)
    rng = np.random.RandomState(5)
    for k, (q, r, v) in enumerate(reps):  # one replica at a time
        a = rng.normal(size=(q.nMol, 3)).astype(np.float32)
        sim.set_state(r, v, a, rep=k)
        rg, vg, ag = sim.get_state(k)
        assert np.array_equal(rg, r) and np.array_equal(vg, v) and np.array_equal(ag, a)
    r_all = np.concatenate([w[1] for w in reps])
    v_all = np.concatenate([w[2] for w in reps])
    a_all = rng.normal(size=(len(r_all), 3)).astype(np.float32)
    sim.set_state(r_all, v_all, a_all)  # all replicas at once
    off = 0
    for k, (q, _, _) in enumerate(reps):
        r, v, a = sim.get_state(k)
        assert np.array_equal(r, r_all[off:off + q.nMol])
        assert np.array_equal(v, v_all[off:off + q.nMol])
        assert np.array_equal(a, a_all[off:off + q.nMol])
        off += q.nMol
    sim.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_step_thermo_is_step_then_thermo(mode):
    p, r, v = workloads.small(seed=63)
    a0 = np.zeros((p.nMol, 3), np.float32)
    one = Simulation(p, mode=mode)
    one.set_state(r, v, a0)
    t1 = one.step_thermo(7)
    two = Simulation(p, mode=mode)
    two.set_state(r, v, a0)
    two.step(7)
    t2 = two.thermo()
    for f, _ in t1._fields_:
        if f == "props":
            continue
        x, y = getattr(t1, f), getattr(t2, f)
        if hasattr(x, "x"):
            assert (x.x, x.y, x.z) == (y.x, y.y, y.z), f
        else:
            assert x == y, f
    assert one.step_readback_bytes() > 0
    one.close()
    two.close()
