"""The CPU oracle against fixtures recorded from the reference's own CUDA kernels.

tests/golden/ref_kernels.npz was written by tests/golden/make_ref_kernel_golden.py, which runs the
reference's device code (SurfaceGrowth.cu, compiled unmodified for sm_103a without FMA
contraction) on a GB300.  These tests need no GPU: they pin the oracle, the checker of every
GPU parity test, to the reference's arithmetic on three regimes (graphene + Ni shear, bulk Ni,
Al growth after deposition).

Bit-exact: cell contents, neighbour lists, every reduction tree, RDF counts, integrator
positions.  Forces, densities, energies: the reference uses CUDA's expf/powf/logf/acosf and the
oracle libm's, which differ by a few ulp:
    |x_oracle - x_reference| <= FORCE_RTOL * max|x_reference| + atol.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from surfacegrowthconsole_gb300._lib import SimParams

FIX = Path(__file__).resolve().parent / "golden" / "ref_kernels.npz"
pytestmark = pytest.mark.skipif(not FIX.exists(), reason="reference-kernel fixture not recorded")

CASES = ["shear", "bulk", "growth"]
FORCE_RTOL = 2e-5
FORCE_ATOL = 1e-6

_data = None


def fix(case):
    global _data
    if _data is None:
        _data = dict(np.load(FIX))
    d = {k.split("__", 1)[1]: v for k, v in _data.items() if k.startswith(case + "__")}
    d["p"] = SimParams.from_buffer_copy(d["params"].tobytes())
    return d


def angle_atol(p):
    """acosf: CUDA and libm differ by up to 2 ulp; each of a carbon's (up to 9) angle terms turns
    one ulp of theta into mu_theta * ulp / sin(theta_0) of force."""
    ulp = float(np.spacing(np.float32(p.theta_0)))
    return 2 * 9 * p.mu_theta * ulp / np.sin(p.theta_0)


def close(x, y, rtol=FORCE_RTOL, atol=FORCE_ATOL):
    scale = max(float(np.abs(y).max()), 1e-30) if np.size(y) else 1.0
    err = float(np.abs(np.asarray(x, np.float64) - np.asarray(y, np.float64)).max()) if np.size(y) else 0.0
    return err <= rtol * scale + atol, err / scale


def oracle_on(d, force_rebuild=False):
    o = oracle.OracleSim(d["p"], 32, force_rebuild=force_rebuild)
    o.set_state(d["r"], d["v"], np.zeros((d["p"].nMol, 3), np.float32))
    return o


@pytest.mark.parametrize("case", CASES)
def test_cells_and_neighbour_lists(case):
    d = fix(case)
    o = oracle_on(d)
    o.build_lists()
    _, cs, ca = o.cells()
    assert np.array_equal(np.diff(cs), d["cell_counts"])
    assert np.array_equal(ca[:cs[-1]], d["cell_atoms"])
    nn, nbl = o.nebr()
    assert np.array_equal(nn, d["nn"])
    flat = np.concatenate([nbl[:nn[i], i] for i in range(d["p"].nMol)])
    assert np.array_equal(flat, d["nbl_flat"])


@pytest.mark.parametrize("case", CASES)
def test_forces_densities_energies(case):
    d = fix(case)
    p = d["p"]
    o = oracle_on(d)
    o.build_lists()
    o.compute_forces()
    r, _, a = o.get_state()
    m = p.nMolMe
    for name, x, y, atol in (("metal acc", a[:m], d["acc"][:m], FORCE_ATOL),
                             ("carbon acc", a[m:], d["acc"][m:], angle_atol(p)),
                             ("energy", r[:, 3], d["U"], FORCE_ATOL),
                             ("rho", o.rho(), d["rho"], FORCE_ATOL),
                             ("friction", o.friction(), d["friction"], 1e-5)):
        ok, rel = close(x, y, FORCE_RTOL, atol)
        assert ok, f"{case} {name}: rel err {rel:.3g}"


@pytest.mark.parametrize("case", CASES)
def test_reduction_trees(case):
    d = fix(case)
    p = d["p"]
    r = d["r"].copy()
    r[:, 3] = d["U"]  # the reductions ran on the state after the force pass
    fric = d["friction"]
    cmx = float(d["cm_vel_x"])
    for what, comps in ((0, 3), (1, 1), (2, 1), (3, 1), (4, 3), (5, 3), (6, 3), (7, 3)):
        if what >= 4 and p.nMolMe == 0:
            continue
        got = oracle.reduce(p, what, r, d["v"], fric, cmx if what == 2 else 0.0)[:comps]
        assert np.array_equal(got, d["reductions"][what][:comps]), f"{case} reduction {what}"
    if p.iRegime != 0 and p.nMolMe:
        assert oracle.reduce(p, 8, r, d["v"], fric)[0] == d["net_force"]


@pytest.mark.parametrize("case", [c for c in CASES])
def test_rdf_counts(case):
    d = fix(case)
    if "rdf" not in d:
        pytest.skip("RDF off in this case")
    o = oracle_on(d)
    o.build_lists()
    o.reset_rdf()
    o.eval_rdf()
    assert np.array_equal(o.rdf(), d["rdf"])


@pytest.mark.parametrize("case", ["shear", "bulk"])  # growth deposits atoms before Verlet part 1
def test_integrator_part1_and_wrap(case):
    d = fix(case)
    o = oracle.OracleSim(d["p"], 32)
    o.set_state(d["r"], d["v"], d["a_rand"])
    o.step(1)
    r, _, _ = o.get_state()
    assert np.array_equal(r[:, :3], d["r_after_part1"][:, :3])


def test_eight_steps_in_the_reference_order():
    d = fix("shear")
    o = oracle_on(d, force_rebuild=True)
    o.step(int(d["traj_steps"]))
    r, v, _ = o.get_state()
    assert np.abs(r[:, :3] - d["traj_r"][:, :3]).max() < 1e-4
    ok, rel = close(v, d["traj_v"], 1e-3)
    assert ok, f"velocities rel err {rel:.3g}"
