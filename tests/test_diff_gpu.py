"""The differentiation form on the GPU against its FP64 restatement (oracle.diff_eval, whose
gradients equal central finite differences: tests/test_diff_oracle.py): frame energies, forces,
force-matching loss and the adjoint gradients of energy and loss, on frames of the 2,217-atom
and of the ~20,000-atom graphene + Ni systems; and the torch.autograd harness."""
import numpy as np
import pytest

import oracle
from surfacegrowthconsole_gb300 import workloads
from surfacegrowthconsole_gb300.engine import DIFF_NPARAM, DiffModel, diff_init_theta

pytestmark = pytest.mark.gpu

GRAD_REL = 1e-4   # adjoint gradient against the FP64 gradient, relative to its largest component


def perturbed(theta, seed=7):
    rng = np.random.RandomState(seed)
    t = theta.copy()
    t[0] *= 1.2
    t[1] *= 0.97
    t[2:] *= 1 + 0.02 * rng.normal(size=DIFF_NPARAM - 2)
    return t


def rel_inf(x, y):
    return float(np.abs(np.asarray(x) - y).max() / np.abs(y).max())


@pytest.mark.parametrize("small_system", [True, False])
def test_gpu_gradients_match_the_fp64_model(small_system):
    frames, r = workloads.differentiation_frames(n_frames=2, small_system=small_system, warm=20, every=10)
    theta = diff_init_theta(frames[0])
    model = DiffModel(frames, r)
    ref = oracle.diff_eval(frames, r, perturbed(theta))[1].astype(np.float32)
    e64, f64, gE64, L64, gL64 = oracle.diff_eval(frames, r, theta, ref)

    e, gE = model.energy(theta)
    assert np.abs(e - e64).max() <= 1e-5 * np.abs(e64).max(), (e, e64)
    assert rel_inf(gE, gE64) < GRAD_REL, rel_inf(gE, gE64)

    f = model.forces(theta)
    rms = np.sqrt(((f - f64) ** 2).mean()) / np.sqrt((f64 ** 2).mean())
    assert rms < 1e-5, rms

    L, gL = model.force_matching(theta, ref)
    assert abs(L - L64) <= 1e-4 * L64, (L, L64)
    assert rel_inf(gL, gL64) < GRAD_REL, rel_inf(gL, gL64)
    print("energy grad rel", rel_inf(gE, gE64), "loss grad rel", rel_inf(gL, gL64))
    model.close()


def test_torch_autograd_harness_carries_the_adjoint_gradient_and_fits():
    torch = pytest.importorskip("torch")
    from surfacegrowthconsole_gb300.fitting import ForceMatchingLoss, fit
    frames, r = workloads.differentiation_frames(n_frames=2, small_system=True, warm=20, every=10)
    theta0 = diff_init_theta(frames[0])
    model = DiffModel(frames, r)
    ref = model.forces(perturbed(theta0))
    t = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    loss = ForceMatchingLoss.apply(t, model, ref)
    loss.backward()
    L, g = model.force_matching(theta0, ref)
    # two evaluations: the parameter sums use atomics, whose order varies (~1e-7 relative)
    assert abs(float(loss.detach()) - L) <= 1e-6 * L
    assert rel_inf(t.grad.numpy(), g) < 1e-5
    _, hist = fit(model, theta0, ref, steps=30, lr=5e-3)
    assert hist[-1] < 0.5 * hist[0], hist[::10]
    model.close()


@pytest.mark.parametrize("knots,rtol", [(29 * 35 + 1, 2e-5), (1024, 2e-4)], ids=["aligned", "interpolated"])
def test_fitted_theta_drives_the_mixed_step(knots, rtol):
    """A fitted theta loaded into a MIXED context (sg_load_diff_theta) gives the metal forces of
    the differentiation model on the same positions: EAM from the B-spline tables (each table
    piece a spline piece when the table knots include the spline knots; the spline's Hermite
    interpolant otherwise), LJ with theta's epsilon and sigma, the analytic embedding.  The list
    radius of the frame parameter block covers the LJ cutoff, so both sides sum the same pairs."""
    from surfacegrowthconsole_gb300 import MODE_MIXED
    from surfacegrowthconsole_gb300.engine import Simulation
    frames, r = workloads.differentiation_frames(n_frames=1, small_system=True, warm=20, every=10)
    q = frames[0]
    theta = perturbed(diff_init_theta(q), seed=11)
    model = DiffModel(frames, r)
    f_diff = model.forces(theta).reshape(-1, 3).astype(np.float64)
    model.close()
    sim = Simulation(q, mode=MODE_MIXED, eam_table_knots=knots)
    sim.load_diff_theta(theta)
    sim.set_state(r, np.zeros((q.nMol, 3), np.float32), np.zeros((q.nMol, 3), np.float32))
    sim.build_lists()
    sim.compute_forces()
    a = sim.get_state()[2].astype(np.float64)
    p = sim.params()
    sim.close()
    m = q.nMolMe
    f_mixed = a[:m] * np.float64(q.massMe)
    err = rel_inf(f_mixed, f_diff[:m])
    assert err < rtol, err
    assert np.isclose(p.epsLJ, np.float32(theta[0])) and np.isclose(p.sigmaLJ, np.float32(theta[1]))
