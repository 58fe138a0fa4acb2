"""The persistent step (sg_options.persistent_step): one cooperative launch per MIXED step over
all replicas, its phases separated by grid-wide barriers with a bounded wait, against the same
step as a CUDA graph of one launch per phase.

The phases run the same device functions in both forms, so cells, lists and forces are
identical; the reduction runs 128-thread blocks over the same atoms per block (the graph's
kernel 512), so its FP32 partial sums group differently and the totals may differ in their
last bits -- the thermostat factor and the trajectories then agree to a few ulp, not bit for bit.
"""
import numpy as np
import pytest

from surfacegrowthconsole_gb300 import MODE_MIXED, workloads
from surfacegrowthconsole_gb300._lib import SgError
from surfacegrowthconsole_gb300.engine import Simulation

pytestmark = pytest.mark.gpu


def _pair(plist, states, **kw):
    out = []
    for persistent in (False, True):
        sim = Simulation(plist, mode=MODE_MIXED, persistent_step=persistent, **kw)
        for k, (r, v) in enumerate(states):
            sim.set_state(r, v, np.zeros((len(r), 3), np.float32), rep=k)
        out.append(sim)
    return out


def test_lists_and_forces_identical_to_the_graph_step():
    """One step with a rebuild on the 45,546-atom workload: the same cells, lists and forces."""
    p, r, v = workloads.production(seed=2, steps=10)
    g, q = _pair([p], [(r, v)], force_rebuild=True)
    g.step(1)
    q.step(1)
    for x, y in zip(g.cells(), q.cells()):
        assert np.array_equal(x, y)
    for x, y in zip(g.nebr(), q.nebr()):
        assert np.array_equal(x, y)
    rg, vg, ag = g.get_state()
    rq, vq, aq = q.get_state()
    assert np.array_equal(rg, rq)  # positions and per-atom energies of step 1
    assert np.array_equal(ag, aq)
    assert q.kernels_per_step() == 1
    g.close()
    q.close()


@pytest.mark.parametrize("which", ["small", "batched"])
def test_trajectory_matches_the_graph_step(which):
    """30 steps across the thermostat step 25: a single system, and twelve uneven replicas of
    the batched configuration stepped together."""
    if which == "small":
        systems = [workloads.small(seed=51)]
    else:
        systems = workloads.batched(n=12, seed=4, steps=5000)
    plist = [s[0] for s in systems]
    g, q = _pair(plist, [(s[1], s[2]) for s in systems])
    g.step(30)
    q.step(30)
    for k in range(len(plist)):
        rg, vg, _ = g.get_state(rep=k)
        rq, vq, _ = q.get_state(rep=k)
        assert np.abs(rg[:, :3] - rq[:, :3]).max() < 1e-4, k
        assert np.abs(vg - vq).max() <= 1e-4 * float(np.abs(vg).max()), k
        tg, tq = g.thermo(k), q.thermo(k)
        assert tg.stepCount == tq.stepCount == 30 and tg.rebuilds == tq.rebuilds
        assert abs(tg.totEnergy - tq.totEnergy) <= 1e-5 * abs(tg.totEnergy), k
    g.close()
    q.close()


def test_barrier_wait_that_runs_out_reports_timeout():
    """A barrier limit of 1 us: blocks that wait longer give up, flag SG_ERR_TIMEOUT in every
    replica and leave; the launch ends and sg_step reports the condition (no hang, no fault).
    The context is then discarded."""
    p, r, v = workloads.small(seed=52)
    sim = Simulation(p, mode=MODE_MIXED, persistent_step=True, persistent_wait_us=1)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    with pytest.raises(SgError) as e:
        sim.step(1)
    assert e.value.code == 8  # SG_ERR_TIMEOUT
    assert sim.diag().timeouts > 0
    sim.close()
    # a fresh context with the default limit steps normally
    ok = Simulation(p, mode=MODE_MIXED, persistent_step=True)
    ok.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    ok.step(3)
    assert ok.thermo().stepCount == 3
    ok.close()


def test_persistent_step_is_mixed_only():
    p, r, v = workloads.small(seed=53)
    with pytest.raises(SgError) as e:
        Simulation(p, persistent_step=True)  # PLAIN
    assert e.value.code == 10  # SG_ERR_UNSUPPORTED
