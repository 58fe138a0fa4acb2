"""GPU parity: every phase of the PLAIN path against the FP32 CPU oracle on the same input.

Integer results (cell assignment and order, neighbour lists, RDF counts) and arithmetic that
uses no transcendental function (integrator, wrap, freeze mask, reduction trees) must be
bit-identical.  Forces and energies go through expf/powf/logf/acosf, whose CUDA and libm
implementations differ by a few ulp, so they are compared with a tolerance:
    |x_gpu - x_oracle| <= FORCE_RTOL * max|x_oracle| + FORCE_ATOL.
"""
import numpy as np
import pytest

import oracle
from surfacegrowthconsole_gb300 import MODE_MIXED, MODE_PLAIN, workloads
from surfacegrowthconsole_gb300.engine import Simulation, default_input, init_coords, init_vels, set_params

pytestmark = pytest.mark.gpu

FORCE_RTOL = 2e-5   # relative to the largest component
FORCE_ATOL = 1e-6
ENERGY_RTOL = 2e-5


def angle_atol(p):
    """Absolute force difference that acosf alone can cause on a carbon atom: CUDA's and libm's
    acosf differ by up to 2 ulp, and each of the atom's angle terms (3 own, up to 6 with second
    neighbours) turns one ulp of theta into mu_theta * ulp / sin(theta_0) of force.  In a flat
    sheet (theta = theta_0) these differences do not shrink with the force itself."""
    ulp = float(np.spacing(np.float32(p.theta_0)))
    return 2 * 9 * p.mu_theta * ulp / np.sin(p.theta_0)


def perturbed_small(seed=21, jitter=0.05):
    p, r, v = workloads.small(seed=seed)
    rng = np.random.RandomState(seed)
    r = r.copy()
    r[:, :3] += rng.normal(0, jitter, size=(p.nMol, 3)).astype(np.float32)
    a = np.zeros((p.nMol, 3), np.float32)
    return p, r, v, a


def make_pair(p, r, v, a, **kw):
    sim = Simulation(p, **kw)
    sim.set_state(r, v, a)
    orc = oracle.OracleSim(p, 32, force_rebuild=kw.get("force_rebuild", False))
    orc.set_state(r, v, a)
    return sim, orc


def close(x, y, rtol=FORCE_RTOL, atol=FORCE_ATOL):
    scale = max(float(np.abs(y).max()), 1e-30)
    err = np.abs(x.astype(np.float64) - y.astype(np.float64)).max()
    return err <= rtol * scale + atol, err / scale


def test_cells_and_neighbours_bit_exact():
    p, r, v, a = perturbed_small()
    sim, orc = make_pair(p, r, v, a)
    sim.build_lists()
    orc.build_lists()
    for g, o in zip(sim.cells(), orc.cells()):
        assert np.array_equal(g, o)
    nn_g, nbl_g = sim.nebr()
    nn_o, nbl_o = orc.nebr()
    assert np.array_equal(nn_g, nn_o)
    assert np.array_equal(nbl_g, nbl_o)  # same entries in the same order
    d = sim.diag()
    assert d.max_neighbours == nn_o.max() and d.nebr_overflow == 0
    sim.close()


def test_neighbours_bit_exact_production_workload():
    """The full graphene + Ni-cluster system: 149 cells of the clusters hold more than 16 atoms
    and are split into home-atom chunks by the list build; lists and forces as on the oracle."""
    p, r, v = workloads.production(seed=2, steps=10)
    a = np.zeros((p.nMol, 3), np.float32)
    sim, orc = make_pair(p, r, v, a)
    sim.build_lists()
    orc.build_lists()
    co_g, cs_g, ca_g = sim.cells()
    co_o, cs_o, ca_o = orc.cells()
    assert np.diff(cs_o).max() > 16
    assert np.array_equal(co_g, co_o) and np.array_equal(cs_g, cs_o) and np.array_equal(ca_g, ca_o)
    nn_g, nbl_g = sim.nebr()
    nn_o, nbl_o = orc.nebr()
    assert np.array_equal(nn_g, nn_o)
    assert np.array_equal(nbl_g, nbl_o)
    sim.compute_forces()
    orc.compute_forces()
    rg, _, ag = sim.get_state()
    ro, _, ao = orc.get_state()
    m = p.nMolMe
    ok, rel = close(ag[:m], ao[:m])
    assert ok, f"metal accelerations rel err {rel:.3g}"
    ok, rel = close(ag[m:], ao[m:], atol=angle_atol(p))
    assert ok, f"carbon accelerations rel err {rel:.3g}"
    ok, rel = close(rg[:, 3], ro[:, 3], rtol=ENERGY_RTOL)
    assert ok, f"per-atom energies rel err {rel:.3g}"
    sim.close()


def test_rdf_extension_against_fp64_all_pairs():
    """The 0-15 A / 300-bin metal RDF extension (culled all-pairs kernel) against the FP64
    all-pairs oracle.  FP32 distances put a pair within ~1e-5 of a bin edge into the neighbour
    bin now and then, so the histograms are compared by their L1 distance (the figure the
    precision report uses), and the pairs inside the range must agree to the pair."""
    from surfacegrowthconsole_gb300 import workloads as W
    rng15 = 15.0 / 1.42
    for p, r, v in (W.small(seed=71), W.production(seed=2, steps=10)):
        sim = Simulation(p, rdf_ext_bins=300, rdf_ext_range=rng15)
        sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
        sim.build_lists()
        sim.reset_rdf()
        sim.eval_rdf()
        h = sim.rdf_ext(0, 300).astype(np.int64)
        ho = oracle.rdf_allpairs(p, r, 300, rng15).astype(np.int64)
        sim.close()
        assert ho.sum() > 0
        assert abs(int(h.sum()) - int(ho.sum())) <= 4  # pairs at the 15 A edge only
        l1 = np.abs(h - ho).sum() / ho.sum()
        assert l1 < 1e-3, f"L1 distance {l1:.3g}"


def test_forces_energies_density():
    p, r, v, a = perturbed_small(seed=22)
    sim, orc = make_pair(p, r, v, a)
    sim.build_lists(); orc.build_lists()
    sim.compute_forces(); orc.compute_forces()
    rg, _, ag = sim.get_state()
    ro, _, ao = orc.get_state()
    ok, err = close(ag[:p.nMolMe], ao[:p.nMolMe]); assert ok, f"metal force rel err {err}"
    ok, err = close(ag[p.nMolMe:], ao[p.nMolMe:]); assert ok, f"carbon force rel err {err}"
    ok, err = close(rg[:, 3], ro[:, 3], rtol=ENERGY_RTOL); assert ok, f"energy rel err {err}"
    ok, err = close(sim.rho(), orc.rho()); assert ok, f"rho rel err {err}"
    ok, err = close(sim.friction(), orc.friction(), atol=1e-5); assert ok, f"friction rel err {err}"
    assert np.array_equal(rg[:, :3], ro[:, :3])
    sim.close()


def test_integrator_positions_bit_exact():
    # positions after one step depend only on Verlet part 1 + wrap + freeze (no transcendentals)
    p, r, v, a = perturbed_small(seed=23, jitter=0.0)  # unperturbed sheet: edge atoms sit on the freeze lines
    a = np.random.RandomState(1).normal(0, 3.0, size=(p.nMol, 3)).astype(np.float32)
    sim, orc = make_pair(p, r, v, a)
    sim.step(1); orc.step(1)
    rg, vg, _ = sim.get_state()
    ro, vo, _ = orc.get_state()
    assert np.array_equal(rg[:, :3], ro[:, :3])
    # frozen graphene edge atoms did not move
    frozen = np.all(rg[:, :3] == r[:, :3], axis=1)
    assert frozen[p.nMolMe:].sum() > 0
    ok, err = close(vg, vo); assert ok, err
    sim.close()


def test_step_reductions_follow_the_reference_tree():
    p, r, v, a = perturbed_small(seed=24)
    sim, orc = make_pair(p, r, v, a)
    sim.step(1)
    t = sim.thermo()
    rg, vg, ag = sim.get_state()
    fr = np.zeros(p.nMol, np.float32)
    fr[:p.nMolMe] = sim.friction()
    q = sim.params()
    red = lambda what, cm=0.0: oracle.reduce(q, what, rg, vg, fr[:p.nMolMe], cm)
    assert tuple(red(0)) == (t.vSum.x, t.vSum.y, t.vSum.z)
    assert red(1)[0] == t.vvMax
    assert red(3)[0] == t.uSum
    assert tuple(red(4)) == (t.centerOfMass.x, t.centerOfMass.y, t.centerOfMass.z)
    assert tuple(red(5)) == (t.cmVel.x, t.cmVel.y, t.cmVel.z)
    assert red(2, t.cmVel.x / p.nMolMe)[0] == t.vvSum
    assert red(8)[0] == t.frictForce
    smin, smax = red(6), red(7)
    assert np.float32(smax[0] - smin[0]) == np.float32(t.particleSize.x)
    sim.close()


def test_rdf_counts_bit_exact():
    p, r, v, a = perturbed_small(seed=25, jitter=0.02)
    sim, orc = make_pair(p, r, v, a)
    sim.build_lists(); orc.build_lists()
    sim.reset_rdf(); orc.reset_rdf()
    sim.eval_rdf(); orc.eval_rdf()
    hg, ho = sim.rdf(), orc.rdf()
    assert hg.sum() > 0
    assert np.array_equal(hg, ho)
    sim.close()


def test_trajectory_30_steps_with_thermostat():
    p, r, v, a = perturbed_small(seed=26, jitter=0.0)
    sim, orc = make_pair(p, r, v, a)
    sim.step(30); orc.step(30)   # crosses the thermostat step 25
    tg, to = sim.thermo(), orc.thermo()
    assert tg.stepCount == to.stepCount == 30
    assert tg.rebuilds == to.rebuilds
    for k in ("kinEnergy", "potEnergy", "totEnergy"):
        assert abs(getattr(tg, k) - getattr(to, k)) <= 1e-4 * abs(getattr(to, k)), k
    rg, vg, _ = sim.get_state()
    ro, vo, _ = orc.get_state()
    assert np.abs(rg[:, :3] - ro[:, :3]).max() < 1e-3
    ok, err = close(vg, vo, rtol=1e-3); assert ok, err
    sim.close()


def test_trajectory_production_workload():
    """The 45,546-atom workload (40,000 C + 8 Ni clusters, 700 K, lists rebuilt every step) for 30
    steps across the thermostat step 25, against the oracle from the same state."""
    p, r, v = workloads.production(seed=2, steps=100)
    a = np.zeros((p.nMol, 3), np.float32)
    sim, orc = make_pair(p, r, v, a, force_rebuild=True)
    sim.step(30); orc.step(30)
    tg, to = sim.thermo(), orc.thermo()
    assert tg.stepCount == to.stepCount == 30
    assert tg.rebuilds == to.rebuilds == 30
    for k in ("kinEnergy", "potEnergy", "totEnergy"):
        assert abs(getattr(tg, k) - getattr(to, k)) <= 1e-4 * abs(getattr(to, k)), k
    rg, vg, _ = sim.get_state()
    ro, vo, _ = orc.get_state()
    assert np.abs(rg[:, :3] - ro[:, :3]).max() < 1e-3
    ok, err = close(vg, vo, rtol=1e-3); assert ok, err
    sim.close()


def test_forced_rebuild_matches():
    p, r, v, a = perturbed_small(seed=27, jitter=0.0)
    sim, orc = make_pair(p, r, v, a, force_rebuild=True)
    sim.step(5); orc.step(5)
    assert sim.thermo().rebuilds == orc.thermo().rebuilds == 5
    nn_g, nbl_g = sim.nebr(); nn_o, nbl_o = orc.nebr()
    # lists of the last step are built from positions that agree to a few ulp; compare sets
    assert np.abs(nn_g - nn_o).max() <= 1
    sim.close()


def test_bulk_regime0():
    inp = default_input(); inp.iRegime = 0; inp.iMaterial = 3; inp.ucx = inp.ucy = inp.ucz = 5
    inp.temperatureK = 500; inp.deltaT = 0.005; inp.randSeed = 3; inp.stepEquil = 10 ** 6; inp.stepLimit = 10 ** 6
    p = set_params(inp); r = init_coords(p); v = init_vels(p); a = np.zeros((p.nMol, 3), np.float32)
    # a perfect lattice has forces that cancel to round-off: displace the atoms first
    r[:, :3] += np.random.RandomState(4).normal(0, 0.03, size=(p.nMol, 3)).astype(np.float32)
    sim, orc = make_pair(p, r, v, a)
    sim.build_lists(); orc.build_lists()
    sim.compute_forces(); orc.compute_forces()
    _, _, ag = sim.get_state(); _, _, ao = orc.get_state()
    ok, err = close(ag, ao); assert ok, err
    sim.step(20); orc.step(20)
    assert abs(sim.thermo().totEnergy - orc.thermo().totEnergy) < 1e-4 * abs(orc.thermo().totEnergy)
    sim.close()


def test_growth_regime1_deposition():
    inp = default_input(); inp.iRegime = 1; inp.iMaterial = 4; inp.ucx = 4; inp.ucy = 4; inp.nMolMe = 60
    inp.temperatureK = 400; inp.deltaT = 0.002; inp.randSeed = 9; inp.stepEquil = 5; inp.stepDeposit = 4
    inp.nMolToDeposit = 10; inp.stepLimit = 1000
    p = set_params(inp); r = init_coords(p); v = init_vels(p); a = np.zeros((p.nMol, 3), np.float32)
    sim, orc = make_pair(p, r, v, a)
    sim.step(24); orc.step(24)
    assert sim.params().nMolDeposited == orc.params().nMolDeposited == 40
    rg, _, _ = sim.get_state(); ro, _, _ = orc.get_state()
    assert np.abs(rg[:, :3] - ro[:, :3]).max() < 1e-3
    d = sim.diag()
    assert d.cell_range > 0  # parked atoms above the box stay out of the lists
    sim.close()


def test_batched_replicas_equal_single_runs():
    systems = [workloads.small(seed=s) for s in (31, 32)]
    inp = default_input(); inp.iRegime = 2; inp.ucx = 6; inp.ucy = 6; inp.nMolMe = 120; inp.randSeed = 5
    inp.deltaT = 0.005; inp.stepEquil = 0; inp.stepCool = 1000; inp.stepAvg = 100; inp.stepRdf = 100
    inp.limitRdf = 10; inp.deltaFpN = 0.0
    p3 = set_params(inp); r3 = init_coords(p3); v3 = init_vels(p3)
    systems.append((p3, r3, v3))
    ps = [s[0] for s in systems]
    batch = Simulation(ps)
    for k, (p, r, v) in enumerate(systems):
        batch.set_state(r, v, np.zeros((p.nMol, 3), np.float32), rep=k)
    batch.step(12)
    for k, (p, r, v) in enumerate(systems):
        single = Simulation(p)
        single.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
        single.step(12)
        rb, vb, ab = batch.get_state(rep=k)
        rs, vs, as_ = single.get_state()
        assert np.array_equal(rb, rs) and np.array_equal(vb, vs) and np.array_equal(ab, as_), k
        assert batch.thermo(k).totEnergy == single.thermo().totEnergy
        single.close()
    batch.close()


def test_neighbour_overflow_is_reported_not_faulted():
    p, r, v, a = perturbed_small(seed=28)
    p.iNebrMax = 12
    sim = Simulation(p)
    sim.set_state(r, v, a)
    with pytest.raises(Exception) as e:
        sim.build_lists()
    assert "NEBR_OVERFLOW" in str(e.value)
    d = sim.diag()
    assert d.nebr_overflow > 0 and d.max_neighbours > 12
    nn, _ = sim.nebr()
    assert nn.max() == 12
    sim.close()


def test_diffusion_matches_oracle():
    p, r, v = workloads.small(seed=41)
    p.stepDiffuse = 2; p.nValDiffuse = 6; p.nBuffDiffuse = 3; p.limitDiffuseAv = 2
    a = np.zeros((p.nMol, 3), np.float32)
    sim, orc = make_pair(p, r, v, a)
    sim.step(40); orc.step(40)
    rr_g, cnt_g, cav_g = sim.diffusion()
    rr_o, cnt_o, cav_o = orc.diffusion()
    assert np.array_equal(cnt_g, cnt_o) and cav_g == cav_o
    ok, err = close(rr_g, rr_o, rtol=1e-3, atol=1e-6); assert ok, err
    sim.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED], ids=["plain", "mixed"])
def test_batched_uneven_replicas_equal_single_runs(mode):
    """Twelve replicas of the batched configuration (graphene of 1,000-20,000 C, one Ni cluster
    of 50-2,000 atoms, 300-1,500 K, each from its own seed) stepped together in one context
    against each replica stepped alone.  PLAIN: bit for bit.  MIXED sums each replica's
    reductions in blocks whose size follows the launch's total atom count, so the batch and a
    single run may round a double-float sum differently (about 1e-14 relative): close, not
    identical."""
    systems = workloads.batched(n=12, seed=4, steps=5000)
    sizes = [s[0].nMol for s in systems]
    assert max(sizes) > 3 * min(sizes)  # uneven
    batch = Simulation([s[0] for s in systems], mode=mode)
    for k, (p, r, v) in enumerate(systems):
        batch.set_state(r, v, np.zeros((p.nMol, 3), np.float32), rep=k)
    steps = 30  # across the thermostat step 25
    batch.step(steps)
    for k, (p, r, v) in enumerate(systems):
        single = Simulation(p, mode=mode)
        single.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
        single.step(steps)
        rb, vb, ab = batch.get_state(rep=k)
        rs, vs, as_ = single.get_state()
        tb, ts = batch.thermo(k), single.thermo()
        assert tb.stepCount == ts.stepCount == steps and tb.rebuilds == ts.rebuilds, k
        if mode == MODE_PLAIN:
            assert np.array_equal(rb, rs) and np.array_equal(vb, vs) and np.array_equal(ab, as_), k
            assert tb.totEnergy == ts.totEnergy, k
        else:
            assert np.abs(rb[:, :3] - rs[:, :3]).max() < 1e-4, k
            ok, err = close(vb, vs, rtol=1e-4); assert ok, (k, err)
            assert abs(tb.totEnergy - ts.totEnergy) <= 1e-5 * abs(ts.totEnergy), k
        single.close()
    batch.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED], ids=["plain", "mixed"])
def test_batched_full_size_sampled_replicas_equal_single_runs(mode):
    """The batched configuration at its full size (256 replicas, 3.0 M atoms) stepped together;
    the smallest, the largest and two other replicas are each stepped alone from the same state
    and compared (PLAIN bit for bit; MIXED close, as above)."""
    systems = workloads.batched(n=256, seed=4, steps=5000)
    sizes = np.array([s[0].nMol for s in systems])
    assert sizes.sum() > 2_900_000
    batch = Simulation([s[0] for s in systems], mode=mode)
    for k, (p, r, v) in enumerate(systems):
        batch.set_state(r, v, np.zeros((p.nMol, 3), np.float32), rep=k)
    steps = 30
    batch.step(steps)
    for k in sorted({int(sizes.argmin()), int(sizes.argmax()), 17, 200}):
        p, r, v = systems[k]
        single = Simulation(p, mode=mode)
        single.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
        single.step(steps)
        rb, vb, ab = batch.get_state(rep=k)
        rs, vs, as_ = single.get_state()
        tb, ts = batch.thermo(k), single.thermo()
        assert tb.stepCount == ts.stepCount == steps and tb.rebuilds == ts.rebuilds, k
        if mode == MODE_PLAIN:
            assert np.array_equal(rb, rs) and np.array_equal(vb, vs) and np.array_equal(ab, as_), k
            assert tb.totEnergy == ts.totEnergy, k
        else:
            assert np.abs(rb[:, :3] - rs[:, :3]).max() < 1e-4, k
            ok, err = close(vb, vs, rtol=1e-4); assert ok, (k, err)
            assert abs(tb.totEnergy - ts.totEnergy) <= 1e-5 * abs(ts.totEnergy), k
        single.close()
    batch.close()


@pytest.mark.parametrize("mode", [MODE_PLAIN, MODE_MIXED])
def test_graphene_without_metal(mode):
    """A sheet with no metal atoms (960 C, the shear regime's schedule): no metal chain, no
    relevant-list metal entries, no centre of mass; lists bit-exact against the oracle, a
    30-step trajectory across the thermostat step against it."""
    from surfacegrowthconsole_gb300.workloads import DT_1FS, build_workload
    p, r, v = build_workload(5, 6, [], 300.0, 7, step_limit=100, step_avg=10, step_equil=0, step_rdf=50,
                             limit_rdf=5, delta_t=DT_1FS)
    assert p.nMolMe == 0
    a = np.zeros((p.nMol, 3), np.float32)
    sim, orc = make_pair(p, r, v, a, mode=mode)
    sim.build_lists(); orc.build_lists()
    for x, y in zip(sim.nebr(), orc.nebr()):
        assert np.array_equal(x, y)
    sim.step(30); orc.step(30)
    tg, to = sim.thermo(), orc.thermo()
    assert tg.stepCount == to.stepCount == 30
    for k in ("kinEnergy", "potEnergy", "totEnergy"):
        assert abs(getattr(tg, k) - getattr(to, k)) <= 1e-4 * abs(getattr(to, k)), k
    rg, vg, _ = sim.get_state()
    ro, vo, _ = orc.get_state()
    assert np.all(np.isfinite(rg)) and np.abs(rg[:, :3] - ro[:, :3]).max() < 1e-3
    sim.close()
