"""Seeded synthetic workloads of the benchmark configurations (nanoparticles on graphene).

All inputs are generated from a seed: no dataset is involved.  Units are the reference's
(length 1.42 A, time 0.2 ps; dt = 0.005 is 1 fs).  Metal is Ni (iMaterial 3), regime 2 (shear)
with the shear increment 0, so the shear drive stays off.
"""
from __future__ import annotations

import numpy as np

from .engine import build_workload

DT_1FS = 0.005


def small(seed: int = 1):
    """2,016 C (7 x 9 graphene units, 68.9 x 76.7 A) + one 201-atom Ni cluster (10 fcc shells),
    300 K, thermostat on (stepEquil 0, stepCool = stepLimit), RDF every 100 steps with limitRdf
    10, 1,000 steps."""
    return build_workload(7, 9, [201], 300.0, seed, step_limit=1000, step_avg=100, step_equil=0,
                          step_rdf=100, limit_rdf=10, delta_t=DT_1FS)


def production(seed: int = 2, steps: int = 10000):
    """40,000 C (25 x 50 units, 246 x 426 A) + 8 Ni clusters of U{300..1000} atoms at random
    x-y positions, 700 K, thermostat on; lists rebuilt every step (set by the caller through
    Simulation(force_rebuild=True)); RDF every 100 steps, diffusion sampled every 10 steps
    (nValDiffuse 100, nBuffDiffuse 10, limitDiffuseAv 5)."""
    rng = np.random.RandomState(seed)
    sizes = [int(x) for x in rng.randint(300, 1001, size=8)]
    return build_workload(25, 50, sizes, 700.0, seed, step_limit=steps, step_avg=100, step_equil=0,
                          step_rdf=100, limit_rdf=10, step_diffuse=10, n_val_diffuse=100, n_buff_diffuse=10,
                          limit_diffuse_av=5, delta_t=DT_1FS)


def precision(seed: int = 3, steps: int = 101000):
    """1,000,000 C (125 x 250 units) + 100,000 Ni in 64 clusters of 1,562-1,563 atoms, 1,000 K."""
    sizes = [1563] * 32 + [1562] * 32
    return build_workload(125, 250, sizes, 1000.0, seed, step_limit=steps, step_avg=100, step_equil=0,
                          step_cool=1000, step_rdf=500, limit_rdf=10, delta_t=DT_1FS)


def batched(n: int = 256, seed: int = 4, steps: int = 5000):
    """n independent replicas: graphene of U[1,000, 20,000] C rounded to 32*ux*uy with ux ~ uy,
    one Ni cluster of U{50..2,000} atoms, temperature U[300, 1,500] K."""
    rng = np.random.RandomState(seed)
    out = []
    for k in range(n):
        nc = rng.uniform(1000, 20000)
        cells = max(4, int(round(nc / 32)))
        ux = max(2, int(round(np.sqrt(cells * 6 / (8 * np.cos(np.pi / 6))))))  # square-ish sheet
        uy = max(2, int(round(cells / ux)))
        nme = int(rng.randint(50, 2001))
        T = float(rng.uniform(300, 1500))
        out.append(build_workload(ux, uy, [nme], T, seed * 100003 + k, step_limit=steps, step_avg=100,
                                  step_equil=0, step_rdf=100, limit_rdf=10, delta_t=DT_1FS))
    return out


def bulk_metal(n: int = 10, temperature_K: float = 300.0, seed: int = 5, material: int = 3):
    """Bulk fcc metal (regime 0; material in the reference's table order Cu 0, Ag 1, Au 2, Ni 3,
    Al 4, Pb 5; default Ni), n x n x n unit cells (4 n^3 atoms), no thermostat: an NVE system of
    the EAM alone, the conservative part of the model (the reference's graphene energy omits the
    second-neighbour angle term its forces apply)."""
    from .engine import default_input, init_coords, init_vels, set_params
    inp = default_input()
    inp.iRegime = 0
    inp.iMaterial = material
    inp.ucx = inp.ucy = inp.ucz = n
    inp.temperatureK = temperature_K
    inp.deltaT = DT_1FS
    inp.randSeed = seed
    inp.stepEquil = 10 ** 9
    inp.stepLimit = 10 ** 9
    p = set_params(inp)
    return p, init_coords(p), init_vels(p)


def differentiation_system(seed: int = 5):
    """~20,000 atoms: 18,432 C (24 x 24 units) + 2,000 Ni in one cluster, c2 settings (700 K)."""
    return build_workload(24, 24, [2000], 700.0, seed, step_limit=1000, step_avg=100, step_equil=0,
                          step_rdf=100, limit_rdf=10, delta_t=DT_1FS)


def differentiation_frames(n_frames: int = 64, seed: int = 5, every: int = 10, warm: int = 50,
                           jitter_A: float = 0.05, small_system: bool = False):
    """Frames of the differentiation form: snapshots every `every` steps of a trajectory of the
    ~20,000-atom system (or of the 2,217-atom system with small_system=True), each with Gaussian jitter
    of jitter_A angstrom per coordinate.  Runs the trajectory on the GPU.  Returns (frame
    parameter blocks, positions of all frames concatenated as (n_frames * nMol, 4) float32)."""
    from .engine import Simulation, diff_frame_params
    p, r, v = small(seed=seed) if small_system else differentiation_system(seed=seed)
    sim = Simulation(p)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    sim.step(warm)
    rng = np.random.RandomState(seed)
    out = []
    for _ in range(n_frames):
        sim.step(every)
        x = sim.get_state()[0].copy()
        x[:, :3] += rng.normal(0, jitter_A / 1.42, size=(p.nMol, 3)).astype(np.float32)
        x[:, 3] = 0.0
        out.append(x)
    sim.close()
    q = diff_frame_params(p)
    return [q] * n_frames, np.concatenate(out)
