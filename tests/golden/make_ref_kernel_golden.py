"""Generate golden fixtures from the reference's own CUDA kernels.

Runs on a machine with a GB300 and the reference kernels' cubin (oracle/_ref/
sgref_kernels_nofma.cubin, built from the reference tree by oracle/ref/build_ref.sh and carried
with the repository copy): `python tests/golden/make_ref_kernel_golden.py OUT.npz`.  Writes one
compressed .npz (tests/golden/ref_kernels.npz) that tests/test_golden_ref_kernels.py compares
with the CPU oracle, so that the oracle stays pinned to the reference's arithmetic in the CPU
test suite.

Cases: a graphene sheet with a Ni cluster (shear regime, jittered), bulk Ni (regime 0, jittered)
and the growth regime after 40 deposited Al atoms.  For each case the fixture holds the input
(the SimParams bytes, positions, velocities, a random acceleration for the integrator) and the
reference kernels' outputs: cell contents, neighbour lists, densities, accelerations, per-atom
energies, friction, every reduction, the RDF histogram, positions after Verlet part 1 + wrap,
and for the shear case the state after eight steps in the reference's step order.  Cells are put
in ascending index order before the list build (the reference's in-chunk atomicAdd order is not
fixed; this is one of its outcomes).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle  # noqa: E402
import refkern  # noqa: E402
from surfacegrowthconsole_gb300 import workloads  # noqa: E402
from surfacegrowthconsole_gb300.engine import default_input, init_coords, init_vels, set_params  # noqa: E402


def case_shear():
    p, r, v = workloads.small(seed=41)
    r = r.copy()
    r[:, :3] += np.random.RandomState(41).normal(0, 0.05, size=(p.nMol, 3)).astype(np.float32)
    return p, r, v


def case_bulk():
    inp = default_input(); inp.iRegime = 0; inp.iMaterial = 3; inp.ucx = inp.ucy = inp.ucz = 5
    inp.temperatureK = 500; inp.deltaT = 0.005; inp.randSeed = 3; inp.stepEquil = 10 ** 6
    inp.stepLimit = 10 ** 6
    p = set_params(inp)
    r = init_coords(p)
    v = init_vels(p)
    r[:, :3] += np.random.RandomState(42).normal(0, 0.03, size=(p.nMol, 3)).astype(np.float32)
    return p, r, v


def case_growth():
    inp = default_input(); inp.iRegime = 1; inp.iMaterial = 4; inp.ucx = 4; inp.ucy = 4; inp.nMolMe = 60
    inp.temperatureK = 400; inp.deltaT = 0.002; inp.randSeed = 9; inp.stepEquil = 5; inp.stepDeposit = 4
    inp.nMolToDeposit = 10; inp.stepLimit = 1000
    p = set_params(inp)
    r = init_coords(p)
    v = init_vels(p)
    o = oracle.OracleSim(p, 32)
    o.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    o.step(24)  # 40 atoms deposited, 20 still parked above the box
    r, v, _ = o.get_state()
    return o.params(), r, v


def record(name, p, r, v, out):
    n = p.nMol
    rng = np.random.RandomState({"shear": 1, "bulk": 2, "growth": 3}[name])
    a_rand = rng.normal(0, 3.0, size=(n, 3)).astype(np.float32)
    pre = f"{name}__"
    out[pre + "params"] = np.frombuffer(bytes(p), np.uint8).copy()
    out[pre + "r"] = np.ascontiguousarray(r, np.float32)
    out[pre + "v"] = np.ascontiguousarray(v, np.float32)
    out[pre + "a_rand"] = a_rand

    # integrator: Verlet part 1 + wrap with a random acceleration
    ref = refkern.RefKernels(p, r, v, a_rand)
    ref.leapfrog(1)
    ref.boundary()
    out[pre + "r_after_part1"] = ref.state()[0]

    # cells, lists, forces, reductions, RDF on the input state
    ref = refkern.RefKernels(p, r, v, np.zeros((n, 3), np.float32))
    ref.lists()
    cell, mic = ref.cells()
    bs = p.blockSize
    out[pre + "cell_counts"] = mic.astype(np.int32)
    out[pre + "cell_atoms"] = np.concatenate([cell[c * bs:c * bs + mic[c]] for c in range(len(mic))]).astype(np.int32)
    nn, nbl = ref.nebr()
    out[pre + "nn"] = nn
    out[pre + "nbl_flat"] = np.concatenate([nbl[:nn[i], i] for i in range(n)]).astype(np.int32)
    ref.forces()
    rr, vv, aa = ref.state()
    out[pre + "acc"] = aa
    out[pre + "U"] = rr[:, 3].copy()
    out[pre + "rho"] = ref.rho()
    fric = ref.friction()
    out[pre + "friction"] = fric
    cm_vel_x = float(ref.reduce(5)[0]) / p.nMolMe if p.nMolMe else 0.0
    red = np.zeros((8, 3), np.float32)
    for what in range(8):
        red[what] = ref.reduce(what, cm_vel_x if what == 2 else 0.0)
    out[pre + "reductions"] = red
    out[pre + "cm_vel_x"] = np.float32(cm_vel_x)
    out[pre + "net_force"] = np.float32(ref.net_force())
    if p.bRdf:
        ref.rdf(0)
        out[pre + "rdf"] = ref.hist()


def record_trajectory(name, p, r, v, out, steps=8):
    ref = refkern.RefKernels(p, r, v, np.zeros((p.nMol, 3), np.float32))
    for step in range(1, steps + 1):
        ref.leapfrog(1)
        ref.boundary()
        ref.lists()
        ref.forces()
        ref.net_force()
        ref.leapfrog(2)
        cm_vel_x = float(ref.reduce(5)[0]) / p.nMolMe if p.nMolMe else 0.0
        ref.reduce(2, cm_vel_x)
        if ((p.iRegime == 2 and step > p.stepEquil and step % p.stepThermostat == 0) or
                (p.iRegime == 1 and step % p.stepThermostat == 0)):
            ref.thermostat(step)
    rr, vv, _ = ref.state()
    out[f"{name}__traj_steps"] = np.int32(steps)
    out[f"{name}__traj_r"] = rr
    out[f"{name}__traj_v"] = vv


def main(path):
    out = {}
    for name, make in (("shear", case_shear), ("bulk", case_bulk), ("growth", case_growth)):
        p, r, v = make()
        record(name, p, r, v, out)
    p, r, v = case_shear()
    record_trajectory("shear", p, r, v, out)
    np.savez_compressed(path, **out)
    print("wrote", path, sum(x.nbytes for x in out.values()), "bytes before compression")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).resolve().parent / "ref_kernels.npz"))
