"""Steps a benchmark workload under a CUDA profiler range, for kernel profilers.

    python -m surfacegrowthconsole_gb300.profile_step [--workload production|batched|precision]
        [--mode plain|mixed] [--warmup 3] [--steps 1] [--replicas 16] [--shape JSON] [--rdf-step]
        [--from-host]

Builds the workload (--shape: a launch shape as sg_get_launch_shape reports it, a JSON object
of its fields, e.g. the one the benchmark's autotuning chose; default: the library's
defaults), steps it `warmup` times (graph capture, caches), then runs `steps` steps
between cudaProfilerStart and cudaProfilerStop, so that a profiler started with its
from-start profiling off (ncu --profile-from-start off) sees exactly those steps' kernels.
Lists are rebuilt every step for the production workload (as its benchmark does) and by the
reference's rule for the others.  --rdf-step: the production workload with the 0-15 A /
300-bin RDF extension on, warmed up to the step before an RDF sample, so that the profiled
step is an RDF step.  --from-host: every step is one sg_step_from_host call on the same host
arrays (r, v, a read from host memory by the step's first kernel, the thermo record published
back), as an end-to-end caller runs it.  Prints the kernel launches per step.
"""
from __future__ import annotations

import argparse
import ctypes
import json

import numpy as np

from . import MODE_MIXED, MODE_PLAIN, workloads
from .engine import Simulation


def _cudart():
    """The CUDA runtime libsgmd.so is linked against (already loaded with the library)."""
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    raise RuntimeError("the CUDA runtime library was not found")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="production", choices=["production", "batched", "precision"])
    ap.add_argument("--mode", default="plain", choices=["plain", "mixed"])
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--replicas", type=int, default=16)
    ap.add_argument("--shape", default="")
    ap.add_argument("--rdf-step", action="store_true")
    ap.add_argument("--from-host", action="store_true")
    a = ap.parse_args()
    if a.workload == "production":
        p, r, v = workloads.production(seed=2)
        plist = [p]
    elif a.workload == "precision":
        p, r, v = workloads.precision(seed=3)
        plist = [p]
    else:
        reps = workloads.batched(a.replicas, seed=4)
        plist = [w[0] for w in reps]
        r = np.concatenate([w[1] for w in reps])
        v = np.concatenate([w[2] for w in reps])
    n = int(sum(q.nMol for q in plist))
    ext = {"rdf_ext_bins": 300, "rdf_ext_range": 15.0 / 1.42} if a.rdf_step else {}
    sim = Simulation(plist, mode=MODE_MIXED if a.mode == "mixed" else MODE_PLAIN,
                     force_rebuild=a.workload == "production", **ext)
    sim.set_state(r, v, np.zeros((n, 3), np.float32))
    if a.shape:
        sim.set_launch_shape(json.loads(a.shape))
    warm = a.warmup
    if a.rdf_step:  # the first profiled step is an RDF step
        warm = max(warm, plist[0].stepRdf - 1)
        warm += (plist[0].stepRdf - 1 - warm) % plist[0].stepRdf
    if a.from_host:
        # the caller's arrays: the same buffers every call, so the step's graph is captured once
        rh = np.ascontiguousarray(r, dtype=np.float32)
        vh = np.ascontiguousarray(v, dtype=np.float32)
        ah = np.zeros((n, 3), np.float32)
        for _ in range(warm):
            sim.step_from_host(rh, vh, ah)
    else:
        sim.step(warm)
    rt = _cudart()
    rt.cudaProfilerStart()
    if a.from_host:
        for _ in range(a.steps):
            sim.step_from_host(rh, vh, ah)
    else:
        sim.step(a.steps)
    rt.cudaProfilerStop()
    print(f"{a.workload} {a.mode}: {n} atoms, {sim.kernels_per_step()} kernel launches per step, "
          f"{a.steps} profiled step(s), launch shape {sim.launch_shape()}")
    sim.close()


if __name__ == "__main__":
    main()
