"""The differentiation form's formulas, without a GPU: the FP64 restatement of the model
(oracle.diff_eval) has energy and force-matching gradients equal to central finite differences
of its own energy and loss (h = 1e-4, FP64), and the initial spline coefficients reproduce the
reference's analytic EAM functions.  The GPU kernels are checked against this FP64 model in
tests/test_diff_gpu.py."""
import numpy as np
import pytest

import oracle
from surfacegrowthconsole_gb300 import workloads
from surfacegrowthconsole_gb300.engine import DIFF_NPARAM, diff_frame_params, diff_init_theta

H = 1e-4          # absolute central-difference step
REL_TOL = 1e-4    # the accuracy asked of the adjoint gradient


def frames_and_positions(n=2, seed=91):
    """Two jittered frames (+-0.05 A Gaussian) of the 2,217-atom graphene + Ni system."""
    p, r, _ = workloads.small(seed=1)
    q = diff_frame_params(p)
    rng = np.random.RandomState(seed)
    rs = []
    for _ in range(n):
        x = r.copy()
        x[:, :3] += rng.normal(0, 0.05 / 1.42, size=(p.nMol, 3)).astype(np.float32)
        rs.append(x)
    return [q] * n, np.concatenate(rs)


def perturbed(theta, seed=7):
    rng = np.random.RandomState(seed)
    t = theta.copy()
    t[0] *= 1.2
    t[1] *= 0.97
    t[2:] *= 1 + 0.02 * rng.normal(size=DIFF_NPARAM - 2)
    return t


def central(fn, theta, k):
    tp, tm = theta.copy(), theta.copy()
    tp[k] += H
    tm[k] -= H
    return (fn(tp) - fn(tm)) / (2 * H)


def check(grad, fd):
    scale = np.abs(fd).max()
    err = np.abs(grad - fd)
    bad = err > REL_TOL * np.abs(fd) + 1e-9 * scale
    assert not bad.any(), f"components {np.nonzero(bad)[0]}: adjoint {grad[bad]} vs FD {fd[bad]}"


def test_energy_gradient_equals_central_differences():
    frames, r = frames_and_positions()
    theta = diff_init_theta(frames[0])
    _, _, g, _, _ = oracle.diff_eval(frames, r, theta)
    fd = np.array([central(lambda t: oracle.diff_eval(frames, r, t)[0].sum(), theta, k) for k in range(DIFF_NPARAM)])
    check(g, fd)


def test_force_matching_gradient_equals_central_differences():
    frames, r = frames_and_positions()
    theta = diff_init_theta(frames[0])
    ref = oracle.diff_eval(frames, r, perturbed(theta))[1].astype(np.float32)
    _, _, _, loss, g = oracle.diff_eval(frames, r, theta, ref)
    assert loss > 0
    fd = np.array([central(lambda t: oracle.diff_eval(frames, r, t, ref)[3], theta, k) for k in range(DIFF_NPARAM)])
    check(g, fd)


def bspline_values(c, r0, h, r):
    x = (r - r0) / h
    k = np.clip(np.floor(x).astype(int), 0, 28)
    t = x - k
    u = 1 - t
    b = np.stack([u ** 3 / 6, (3 * t ** 3 - 6 * t ** 2 + 4) / 6, (-3 * t ** 3 + 3 * t ** 2 + 3 * t + 1) / 6, t ** 3 / 6])
    return sum(c[k + m] * b[m] for m in range(4))


@pytest.mark.parametrize("fn, off", [(0, 2), (1, 34)])
def test_initial_splines_fit_the_analytic_eam(fn, off):
    """phi (fn 0) and f (fn 1) of the fitted splines against the analytic forms on the spline's
    range; the error is small against the function's range of values."""
    frames, _ = frames_and_positions(1)
    p = frames[0]
    theta = diff_init_theta(p)
    r0 = 0.6 / p.rei
    rc = np.sqrt(p.rrCutEam)
    rs = np.linspace(r0, rc, 1001)[:-1]
    got = bspline_values(theta[off:off + 32], r0, (rc - r0) / 29, rs)
    want = np.array([oracle.eam_eval(p, fn, float(x), 64) for x in rs])
    # beyond the nearest-neighbour distance (where pairs live) the fit holds to 1e-3 of the range
    live = rs > 0.8 / p.rei
    err = np.abs(got - want)[live].max() / (want[live].max() - want[live].min())
    assert err < 1e-3, err
