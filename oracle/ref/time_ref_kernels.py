"""TEST INFRASTRUCTURE: times the reference GPU path as shipped on this GPU.

The reference's device code compiled unmodified with nvcc's default flags for sm_103a
(oracle/_ref/sgref_kernels.cubin, from oracle/ref/build_ref.sh) runs through oracle/librefkern.so:
the step loop's launches with the reference's launch shapes and its blocking device-to-host
copies after every reduction (SurfaceGrowth.cu:2141-2430), without file output.  Prints one JSON
line per workload: atom-steps/s, ms per step.

    python oracle/ref/time_ref_kernels.py [--steps K] [--warmup W] [--workload production|small|batched]

batched: the 256 replicas of the batched configuration one by one (the reference runs one
system per process), each for K steps after W warm-up steps; the value is all replicas' atoms x
K over the summed time.

The states are checked on the CPU oracle before the first launch (no cell above blockSize atoms,
no atom with iNebrMax neighbours or more): the reference kernels check no bounds.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import refkern  # noqa: E402
from surfacegrowthconsole_gb300 import workloads  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="production", choices=["production", "small", "batched"])
    ap.add_argument("--replicas", type=int, default=256)
    args = ap.parse_args()
    why = refkern.available("shipped")
    if why:
        print(json.dumps({"impl": "reference kernels as shipped", "unavailable": why}))
        return
    if args.workload == "batched":
        reps = workloads.batched(args.replicas, seed=4)
        total_ms, atoms = 0.0, 0
        for q, rq, vq in reps:
            ref = refkern.RefKernels(q, rq, vq, kind="shipped")
            ref.run_steps(args.warmup, force_rebuild=False)
            total_ms += ref.run_steps(args.steps, force_rebuild=False)
            atoms += q.nMol
        print(json.dumps({"impl": "reference kernels as shipped (nvcc default flags, sm_103a)",
                          "workload": f"{len(reps)} replicas of the batched configuration one by one, {atoms} atoms, "
                                      "lists rebuilt by the reference's rule",
                          "atoms": atoms, "steps": args.steps, "ms_all_replicas_per_step": total_ms / args.steps,
                          "value": atoms * args.steps / (total_ms * 1e-3), "unit": "atom-steps/s"}))
        return
    if args.workload == "production":
        p, r, v = workloads.production(seed=2)
        desc = f"graphene 40000 C + 8 Ni clusters ({p.nMolMe} Ni), {p.nMol} atoms, 700 K, lists rebuilt every step"
        force = True
    else:
        p, r, v = workloads.small(seed=1)
        desc = f"graphene 2016 C + 201-atom Ni cluster, {p.nMol} atoms, 300 K, lists rebuilt when due"
        force = False
    ref = refkern.RefKernels(p, r, v, kind="shipped")
    ref.run_steps(args.warmup, force_rebuild=force)
    ms = ref.run_steps(args.steps, force_rebuild=force)
    print(json.dumps({"impl": "reference kernels as shipped (nvcc default flags, sm_103a)", "workload": desc,
                      "atoms": p.nMol, "steps": args.steps, "ms_per_step": ms / args.steps,
                      "value": p.nMol * args.steps / (ms * 1e-3), "unit": "atom-steps/s",
                      "ncells": p.cells.x * p.cells.y * p.cells.z}))


if __name__ == "__main__":
    main()
