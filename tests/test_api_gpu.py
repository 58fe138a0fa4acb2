"""The host-buffer calls of the sg_* C ABI: state uploads and downloads round-trip exactly,
sg_step_thermo's record is the one sg_get_thermo reads after sg_step, and sg_step_from_host is
sg_set_state + sg_step + that record."""
import numpy as np
import pytest

from surfacegrowthconsole_gb300 import MODE_MIXED, MODE_PLAIN, workloads
from surfacegrowthconsole_gb300.engine import Simulation

pytestmark = pytest.mark.gpu


def _pinned(x):
    """A page-locked copy of x (the upload kernel reads such arrays in place)."""
    torch = pytest.importorskip("torch")
    y = torch.empty(x.shape, dtype=torch.float32, pin_memory=True).numpy()
    y[:] = x
    return y


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_state_round_trip(mode, pinned):
    reps = [workloads.small(seed=s) for s in (61, 62)]
    plist = [w[0] for w in reps]
    sim = Simulation(plist, mode=mode)
    rng = np.random.RandomState(5)
    host = _pinned if pinned else (lambda x: x)
    for k, (q, r, v) in enumerate(reps):  # one replica at a time
        a = rng.normal(size=(q.nMol, 3)).astype(np.float32)
        r, v, a = host(r), host(v), host(a)
        sim.set_state(r, v, a, rep=k)
        rg, vg, ag = sim.get_state(k)
        assert np.array_equal(rg, r) and np.array_equal(vg, v) and np.array_equal(ag, a)
    r_all = host(np.concatenate([w[1] for w in reps]))
    v_all = host(np.concatenate([w[2] for w in reps]))
    a_all = host(rng.normal(size=(len(r_all), 3)).astype(np.float32))
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


def _same_thermo(t1, t2):
    for f, _ in t1._fields_:
        if f == "props":
            continue
        x, y = getattr(t1, f), getattr(t2, f)
        if hasattr(x, "x"):
            assert (x.x, x.y, x.z) == (y.x, y.y, y.z), f
        else:
            assert x == y, f


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_step_from_host_is_set_state_then_step(mode, pinned):
    """One replica or all at once: the same states and thermo records as sg_set_state followed by
    sg_step / sg_step_thermo, over several calls in a row."""
    reps = [workloads.small(seed=s) for s in (64, 65)]
    plist = [w[0] for w in reps]
    r_all = np.concatenate([w[1] for w in reps])
    v_all = np.concatenate([w[2] for w in reps])
    rng = np.random.RandomState(9)
    a_all = rng.normal(scale=0.01, size=(len(r_all), 3)).astype(np.float32)
    one = Simulation(plist, mode=mode)
    two = Simulation(plist, mode=mode)
    for sim in (one, two):
        sim.set_state(r_all, v_all, a_all)
        sim.step(24)
    host = _pinned if pinned else (lambda x: x)
    r1, v1, a1 = one.get_state(1)
    r1 = r1.copy()
    r1[:, :3] += rng.normal(scale=1e-3, size=(len(r1), 3)).astype(np.float32)
    for k in range(3):
        r1, v1, a1 = host(r1), host(v1), host(a1)
        t1 = one.step_from_host(r1, v1, a1, nsteps=3, rep=1, thermo_rep=1)
        two.set_state(r1, v1, a1, rep=1)
        t2 = two.step_thermo(3, rep=1)
        _same_thermo(t1, t2)
        for x, y in zip(one.get_state(), two.get_state()):
            assert np.array_equal(x, y)
        r1, v1, a1 = one.get_state(1)
    ra, va, aa = (host(x) for x in one.get_state())
    assert one.step_from_host(ra, va, aa, nsteps=2, thermo_rep=None) is None
    two.set_state(ra, va, aa)
    two.step(2)
    for x, y in zip(one.get_state(), two.get_state()):
        assert np.array_equal(x, y)
    _same_thermo(one.thermo(0), two.thermo(0))
    one.close()
    two.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_published_record_is_the_current_step_over_many_calls(mode):
    """sg_step_thermo returns once the host sees the step's sequence number in the page-locked
    mirror; the record it then reads must be that step's, never the previous publish (the host
    reads the sequence number with acquire ordering: the Grace host is weakly ordered).  Over
    300 single-step calls every record equals sg_get_thermo's after a stream synchronisation."""
    p, r, v = workloads.small(seed=64)
    sim = Simulation(p, mode=mode)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    for i in range(300):
        t1 = sim.step_thermo(1)
        t2 = sim.thermo()
        assert t1.stepCount == t2.stepCount == i + 1
        _same_thermo(t1, t2)
    sim.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_published_records_of_every_replica(mode):
    """Five uneven replicas in one context: the record sg_step_thermo returns for each replica in
    turn, over 120 single-step calls (RDF steps among them; in MIXED most steps' reductions
    publish the records themselves, each replica's last block its own), equals sg_get_thermo's
    after a stream synchronisation, and single steps from host buffers publish every replica's
    record the same way."""
    systems = workloads.batched(n=5, seed=6, steps=5000)
    sim = Simulation([s[0] for s in systems], mode=mode)
    for k, (p, r, v) in enumerate(systems):
        sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32), rep=k)
    for i in range(120):
        k = i % 5
        t1 = sim.step_thermo(1, rep=k)
        t2 = sim.thermo(k)
        assert t1.stepCount == t2.stepCount == i + 1, (i, k)
        _same_thermo(t1, t2)
    hr, hv, ha = (np.ascontiguousarray(x) for x in sim.get_state())
    for i in range(10):
        t1 = sim.step_from_host(hr, hv, ha, nsteps=1, thermo_rep=i % 5)
        t2 = sim.thermo(i % 5)
        assert t1.stepCount == t2.stepCount == 121 + i, i
        _same_thermo(t1, t2)
    sim.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_record_after_launch_only_steps(mode):
    """Steps launched without a wait (sg_step_async) publish nothing; a call with no steps
    (sg_step_thermo with nsteps 0: the publish kernel alone) then returns the last of them,
    equal to sg_get_thermo's."""
    p, r, v = workloads.small(seed=65)
    sim = Simulation(p, mode=mode)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    for n in (7, 1, 93):  # the last batch crosses the RDF step 100
        sim.step_async(n)
        t1 = sim.step_thermo(0)
        t2 = sim.thermo()
        assert t1.stepCount == t2.stepCount
        _same_thermo(t1, t2)
    assert sim.thermo().stepCount == 101
    sim.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_steps_without_graphs_equal_steps_with_graphs(mode):
    """use_graphs = 0 enqueues each step's kernels one by one (the publish folded into the last
    step's reduction all the same): the same states and records as the graphs, over single-step
    calls, a batch of steps across an RDF step and steps from host buffers."""
    p, r, v = workloads.small(seed=66)
    a0 = np.zeros((p.nMol, 3), np.float32)
    sims = [Simulation(p, mode=mode, use_graphs=g) for g in (True, False)]
    for sim in sims:
        sim.set_state(r, v, a0)
    for i in range(5):
        t = [sim.step_thermo(1) for sim in sims]
        _same_thermo(t[0], t[1])
    t = [sim.step_thermo(97) for sim in sims]  # through the RDF step 100
    _same_thermo(t[0], t[1])
    hr, hv, ha = (np.ascontiguousarray(x) for x in sims[0].get_state())
    for i in range(3):
        t = [sim.step_from_host(hr, hv, ha, nsteps=1) for sim in sims]
        _same_thermo(t[0], t[1])
    for x, y in zip(sims[0].get_state(), sims[1].get_state()):
        assert np.array_equal(x, y)
    for sim in sims:
        sim.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_page_locked_block_equals_pageable_arrays(mode):
    """r, v, a as views of one page-locked block are read in place by the upload kernel,
    pageable arrays are copied first: the state and the trajectory are the same."""
    torch = pytest.importorskip("torch")
    p, r, v = workloads.small(seed=66)
    n = p.nMol
    a = np.random.RandomState(6).normal(size=(n, 3)).astype(np.float32)
    block = torch.empty(n * 10, dtype=torch.float32, pin_memory=True).numpy()
    br, bv, ba = block[:4 * n].reshape(n, 4), block[4 * n:7 * n].reshape(n, 3), block[7 * n:].reshape(n, 3)
    br[:], bv[:], ba[:] = r, v, a
    one = Simulation(p, mode=mode)
    two = Simulation(p, mode=mode)
    one.set_state(br, bv, ba)
    two.set_state(r.copy(), v.copy(), a.copy())
    for x, y in zip(one.get_state(), (r, v, a)):
        assert np.array_equal(x, y)
    for _ in range(3):
        t1 = one.step_from_host(br, bv, ba, nsteps=2)
        t2 = two.step_from_host(r.copy(), v.copy(), a.copy(), nsteps=2)
        _same_thermo(t1, t2)
    for x, y in zip(one.get_state(), two.get_state()):
        assert np.array_equal(x, y)
    one.close()
    two.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_upload_from_unaligned_pageable_arrays(mode):
    """r, v and a at 4-byte offsets inside one pageable buffer (r not on a 16-byte boundary)
    upload exactly, and a step from them equals one from aligned copies."""
    p, r, v = workloads.small(seed=67)
    n = p.nMol
    a = np.random.RandomState(7).normal(size=(n, 3)).astype(np.float32)
    buf = np.zeros(10 * n + 3, np.float32)
    hr = buf[1:1 + 4 * n].reshape(n, 4)
    hv = buf[2 + 4 * n:2 + 7 * n].reshape(n, 3)
    ha = buf[3 + 7 * n:3 + 10 * n].reshape(n, 3)
    hr[:], hv[:], ha[:] = r, v, a
    assert hr.ctypes.data % 16 != 0
    sim = Simulation(p, mode=mode)
    sim.set_state(hr, hv, ha)
    for x, y in zip(sim.get_state(), (r, v, a)):
        assert np.array_equal(x, y)
    t1 = sim.step_from_host(hr, hv, ha, nsteps=2)
    ref = Simulation(p, mode=mode)
    ref.set_state(r.copy(), v.copy(), a.copy())
    ref.step(2)
    _same_thermo(t1, ref.thermo())
    for x, y in zip(sim.get_state(), ref.get_state()):
        assert np.array_equal(x, y)
    sim.close()
    ref.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_step_from_host_loop_on_the_same_buffers(mode):
    """A caller's loop: the state refilled into the same buffers, one step from them, again --
    the library replays one graph of upload, step and publish for the buffers (read when the
    graph runs) -- equals set_state + step on another context, across an RDF step (a graph of
    another step variant) and a switch to other buffers."""
    p, r, v = workloads.small(seed=68)
    n = p.nMol
    a0 = np.zeros((n, 3), np.float32)
    warm = 95  # RDF steps come every 100 steps
    one = Simulation(p, mode=mode)
    two = Simulation(p, mode=mode)
    for s in (one, two):
        s.set_state(r, v, a0)
        s.step(warm)
    hr, hv, ha = np.zeros((n, 4), np.float32), np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
    for k in range(12):
        if k == 8:  # other buffers from here on
            hr, hv, ha = hr.copy(), hv.copy(), ha.copy()
        st = one.get_state()
        for x, y in zip((hr, hv, ha), st):
            x[:] = y
        t1 = one.step_from_host(hr, hv, ha, nsteps=1)
        two.set_state(*two.get_state())
        two.step(1)
        t2 = two.thermo()
        assert t1.stepCount == t2.stepCount == warm + k + 1
        _same_thermo(t1, t2)
        # the call's graph: the step's kernels and the upload kernel (in MIXED the integrator
        # reads the buffers itself); the publish kernel only in an RDF step (otherwise the
        # reduction publishes the record itself)
        rdf_step = t1.stepCount % p.stepRdf == 0
        extra = (1 if rdf_step else 0) + (0 if mode == MODE_MIXED else 1)
        assert one.kernels_per_step() == two.kernels_per_step() + extra, k
    for x, y in zip(one.get_state(), two.get_state()):
        assert np.array_equal(x, y)
    one.close()
    two.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_step_from_host_one_replica_of_several(mode):
    """Steps from one replica's buffers in a two-replica context (the graph then holds the upload
    kernel for that replica) equal set_state of that replica + step, replica by replica."""
    reps = [workloads.small(seed=s) for s in (69, 70)]
    plist = [w[0] for w in reps]
    one = Simulation(plist, mode=mode)
    two = Simulation(plist, mode=mode)
    for s in (one, two):
        for k, (q, r, v) in enumerate(reps):
            s.set_state(r, v, np.zeros((q.nMol, 3), np.float32), rep=k)
    n1 = plist[1].nMol
    hr, hv, ha = np.zeros((n1, 4), np.float32), np.zeros((n1, 3), np.float32), np.zeros((n1, 3), np.float32)
    for k in range(4):
        for x, y in zip((hr, hv, ha), one.get_state(1)):
            x[:] = y
        t1 = one.step_from_host(hr, hv, ha, nsteps=1, rep=1, thermo_rep=1)
        two.set_state(*two.get_state(1), rep=1)
        two.step(1)
        _same_thermo(t1, two.thermo(1))
    for k in range(2):
        for x, y in zip(one.get_state(k), two.get_state(k)):
            assert np.array_equal(x, y)
    one.close()
    two.close()
