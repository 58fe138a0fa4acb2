"""Parity pinned to the reference's own kernels.

The reference's CUDA code (SurfaceGrowth.cu), compiled unmodified for sm_103a without FMA
contraction (oracle/ref/build_ref.sh), runs on the same injected states as the oracle and the
PLAIN CUDA path (oracle/refkern.py).  The reference fills a cell in atomicAdd order, which is not
fixed inside one 64-atom chunk; its cells are put in ascending index order (one of its possible
outcomes, the order the oracle and the CUDA path use) before its neighbour list is built.

Bit-exact: cell contents, neighbour lists, integrator positions, every reduction tree, RDF counts.
Forces, densities and energies: the reference kernels and the CUDA path both use CUDA's
expf/powf/logf/acosf, so they differ only by summation order; the oracle uses libm.
"""
import numpy as np
import pytest

import oracle
import refkern
from surfacegrowthconsole_gb300 import workloads
from surfacegrowthconsole_gb300.engine import Simulation

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(refkern.available("nofma") is not None,
                                 reason=f"reference kernels: {refkern.available('nofma')}")]

SUM_ORDER_RTOL = 2e-6   # CUDA path vs reference kernels: same math functions, other summation order
FORCE_RTOL = 2e-5       # oracle (libm) vs reference kernels (CUDA math)
FORCE_ATOL = 1e-6


def angle_atol(p):
    """acosf: CUDA and libm differ by up to 2 ulp; each of a carbon's (up to 9) angle terms turns
    one ulp of theta into mu_theta * ulp / sin(theta_0) of force."""
    ulp = float(np.spacing(np.float32(p.theta_0)))
    return 2 * 9 * p.mu_theta * ulp / np.sin(p.theta_0)


def close(x, y, rtol, atol=FORCE_ATOL):
    scale = max(float(np.abs(y).max()), 1e-30)
    err = float(np.abs(np.asarray(x, np.float64) - np.asarray(y, np.float64)).max())
    return err <= rtol * scale + atol, err / scale


def small_state(seed=31, jitter=0.05):
    p, r, v = workloads.small(seed=seed)
    rng = np.random.RandomState(seed)
    r = r.copy()
    r[:, :3] += rng.normal(0, jitter, size=(p.nMol, 3)).astype(np.float32)
    return p, r, v


def ref_cells_as_sorted_segments(ref, p):
    cell, mic = ref.cells()
    bs = p.blockSize
    return [np.sort(cell[c * bs:c * bs + mic[c]]) for c in range(len(mic))], mic


@pytest.mark.parametrize("which", ["small", "production"])
def test_cells_and_lists_equal_the_reference_kernels(which):
    if which == "small":
        p, r, v = small_state()
    else:
        p, r, v = workloads.production(seed=2, steps=10)
    ref = refkern.RefKernels(p, r, v)
    ref.bin()
    segs, mic = ref_cells_as_sorted_segments(ref, p)
    orc = oracle.OracleSim(p, 32)
    orc.set_state(r, v)
    orc.build_lists()
    _, cs, ca = orc.cells()
    assert np.array_equal(mic, np.diff(cs))
    for c, seg in enumerate(segs):
        assert np.array_equal(seg, ca[cs[c]:cs[c + 1]]), f"cell {c}"
    ref.canonicalize_cells()
    ref.build_nebr()
    nn_r, nbl_r = ref.nebr()
    nn_o, nbl_o = orc.nebr()
    assert np.array_equal(nn_r, nn_o)
    assert np.array_equal(nbl_r, nbl_o)
    sim = Simulation(p)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    sim.build_lists()
    nn_g, nbl_g = sim.nebr()
    assert np.array_equal(nn_g, nn_r)
    assert np.array_equal(nbl_g, nbl_r)
    sim.close()


@pytest.mark.parametrize("which", ["small", "production"])
def test_forces_match_the_reference_kernels(which):
    if which == "small":
        p, r, v = small_state(seed=32)
    else:
        p, r, v = workloads.production(seed=2, steps=10)
    a0 = np.zeros((p.nMol, 3), np.float32)
    ref = refkern.RefKernels(p, r, v, a0)
    ref.lists()
    ref.forces()
    rr, _, ar = ref.state()
    rho_r, fric_r = ref.rho(), ref.friction()
    m = p.nMolMe

    sim = Simulation(p)
    sim.set_state(r, v, a0)
    sim.build_lists()
    sim.compute_forces()
    rg, _, ag = sim.get_state()
    for name, x, y in (("metal acc", ag[:m], ar[:m]), ("carbon acc", ag[m:], ar[m:]),
                       ("energy", rg[:, 3], rr[:, 3]), ("rho", sim.rho(), rho_r),
                       ("friction", sim.friction(), fric_r)):
        ok, rel = close(x, y, SUM_ORDER_RTOL)
        assert ok, f"CUDA path vs reference kernels, {name}: rel err {rel:.3g}"
    sim.close()

    orc = oracle.OracleSim(p, 32)
    orc.set_state(r, v, a0)
    orc.build_lists()
    orc.compute_forces()
    ro, _, ao = orc.get_state()
    for name, x, y, atol in (("metal acc", ao[:m], ar[:m], FORCE_ATOL),
                             ("carbon acc", ao[m:], ar[m:], angle_atol(p)),
                             ("energy", ro[:, 3], rr[:, 3], FORCE_ATOL),
                             ("rho", orc.rho(), rho_r, FORCE_ATOL),
                             ("friction", orc.friction(), fric_r, 1e-5)):
        ok, rel = close(x, y, FORCE_RTOL, atol)
        assert ok, f"oracle vs reference kernels, {name}: rel err {rel:.3g}"


def test_integrator_reductions_and_rdf_equal_the_reference_kernels():
    p, r, v = small_state(seed=33, jitter=0.0)  # flat sheet: edge atoms on the freeze lines
    rng = np.random.RandomState(33)
    a = rng.normal(0, 3.0, size=(p.nMol, 3)).astype(np.float32)
    ref = refkern.RefKernels(p, r, v, a)
    ref.leapfrog(1)
    ref.boundary()
    r1, v1, _ = ref.state()
    orc = oracle.OracleSim(p, 32)
    orc.set_state(r, v, a)
    orc.step(1)
    ro, _, _ = orc.get_state()
    assert np.array_equal(r1[:, :3], ro[:, :3]), "Verlet part 1 + wrap + freeze"

    # every reduction kernel on one state, against the oracle's tree (x-only sums compare x)
    ref.lists()
    ref.forces()
    r2, v2, _ = ref.state()
    fric = ref.friction()
    cm_vel_x = float(ref.reduce(5)[0]) / p.nMolMe
    for what, comps in ((0, 3), (1, 1), (2, 1), (3, 1), (4, 3), (5, 3), (6, 3), (7, 3)):
        cmx = cm_vel_x if what == 2 else 0.0
        got = ref.reduce(what, cmx)[:comps]
        want = oracle.reduce(p, what, r2, v2, fric, cmx)[:comps]
        assert np.array_equal(got, want), f"reduction {what}: {got} vs {want}"
    assert np.float32(ref.net_force()) == oracle.reduce(p, 8, r2, v2, fric)[0]

    ref.rdf(0)
    orc2 = oracle.OracleSim(p, 32)
    orc2.set_state(r2[:, :4], v2)
    orc2.build_lists()
    orc2.reset_rdf()
    orc2.eval_rdf()
    assert ref.hist().sum() > 0
    assert np.array_equal(ref.hist(), orc2.rdf())


def test_trajectory_of_reference_kernels_matches_the_oracle():
    """Eight steps in the reference's step order (SurfaceGrowth.cu:2187-2366) with its own kernels,
    cells put in index order at every rebuild, against the oracle's steps."""
    p, r, v = small_state(seed=34, jitter=0.0)
    a0 = np.zeros((p.nMol, 3), np.float32)
    ref = refkern.RefKernels(p, r, v, a0)
    orc = oracle.OracleSim(p, 32, force_rebuild=True)
    orc.set_state(r, v, a0)
    for step in range(1, 9):
        ref.leapfrog(1)
        ref.boundary()
        ref.lists()
        ref.forces()
        ref.net_force()
        ref.leapfrog(2)
        cm_vel_x = float(ref.reduce(5)[0]) / p.nMolMe if p.nMolMe else 0.0
        ref.reduce(2, cm_vel_x)
        thermo_now = ((p.iRegime == 2 and step > p.stepEquil and step % p.stepThermostat == 0) or
                      (p.iRegime == 1 and step % p.stepThermostat == 0))
        if thermo_now:
            ref.thermostat(step)
    orc.step(8)
    rr, vr, _ = ref.state()
    ro, vo, _ = orc.get_state()
    assert np.abs(rr[:, :3] - ro[:, :3]).max() < 1e-4
    ok, rel = close(vr, vo, 1e-3)
    assert ok, f"velocities rel err {rel:.3g}"
