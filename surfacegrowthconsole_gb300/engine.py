"""Python face of sgmd: configuration helpers and the `Simulation` class over the C ABI.

This mirrors the reference's host interface for the timestep path: the reference derives a
SimParams from sugr_in.txt (ReadInputFile/SetParams, SurfaceGrowth.cpp:189-396, 633-785),
fills initial coordinates and velocities (InitCoordsW/InitVels) and hands everything to
DoComputationsW (SurfaceGrowth.cu:2013-2529).  Here the same steps are `read_input_file`,
`set_params`, `init_coords`, `init_vels` and `Simulation(...).run(...)`, with the finer
per-phase calls (`build_lists`, `compute_forces`, `eval_rdf`, ...) used by the parity tests.
Arrays are numpy, in the reference's host layouts: positions (N, 4) float32 {x, y, z, U},
velocities and accelerations (N, 3) float32, metal atoms first.
"""
from __future__ import annotations

import ctypes as C
import json
from typing import Sequence

import numpy as np

from ._lib import (MODE_MIXED, MODE_PLAIN, Diag, Input, LaunchShape, Options, SimParams, Thermo, Workload,
                   check, lib, libc)

__all__ = ["Simulation", "read_input_file", "default_input", "set_params", "init_coords", "init_vels",
           "build_workload", "SimParams", "Input", "MODE_PLAIN", "MODE_MIXED"]


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def default_input() -> Input:
    inp = Input()
    lib().sg_default_input(C.byref(inp))
    return inp


def read_input_file(path: str, inp: Input | None = None) -> Input:
    """sugr_in.txt semantics: 22 positional rows on top of the compiled-in defaults."""
    inp = inp or default_input()
    check(lib().sg_read_input_file(str(path).encode(), C.byref(inp)))
    return inp


def set_params(inp: Input) -> SimParams:
    p = SimParams()
    check(lib().sg_set_params(C.byref(inp), C.byref(p)))
    return p


def init_coords(p: SimParams) -> np.ndarray:
    """Initial lattice of the regime (advances p's random seed in regime 1, sets initUcellMe*)."""
    r = np.zeros((p.nMol, 4), np.float32)
    check(lib().sg_init_coords(C.byref(p), _ptr(r)))
    return r


def init_vels(p: SimParams) -> np.ndarray:
    v = np.zeros((p.nMol, 3), np.float32)
    check(lib().sg_init_vels(C.byref(p), _ptr(v)))
    return v


def build_workload(ucx: int, ucy: int, cluster_sizes: Sequence[int], temperature_K: float, seed: int,
                   material: int = 3, clearance_A: float = 2.5, step_limit: int = 1000, step_avg: int = 100,
                   step_equil: int = 0, step_cool: int | None = None, step_rdf: int = 100, limit_rdf: int = 100,
                   step_diffuse: int = 0, n_val_diffuse: int = 0, n_buff_diffuse: int = 0,
                   limit_diffuse_av: int = 0, delta_t: float = 0.005):
    """Graphene sheet (32*ucx*ucy C) with fcc metal clusters; returns (params, r, v)."""
    sizes = (C.c_int * max(1, len(cluster_sizes)))(*cluster_sizes)
    w = Workload(ucx=ucx, ucy=ucy, iMaterial=material, n_clusters=len(cluster_sizes),
                 cluster_sizes=C.cast(sizes, C.POINTER(C.c_int)), temperatureK=temperature_K,
                 clearance_A=clearance_A, seed=seed, stepLimit=step_limit, stepAvg=step_avg,
                 stepEquil=step_equil, stepCool=step_limit if step_cool is None else step_cool,
                 stepRdf=step_rdf, limitRdf=limit_rdf, stepDiffuse=step_diffuse, nValDiffuse=n_val_diffuse,
                 nBuffDiffuse=n_buff_diffuse, limitDiffuseAv=limit_diffuse_av, deltaT=delta_t)
    p = SimParams()
    check(lib().sg_build_workload(C.byref(w), C.byref(p), None, None))
    r = np.zeros((p.nMol, 4), np.float32)
    v = np.zeros((p.nMol, 3), np.float32)
    check(lib().sg_build_workload(C.byref(w), C.byref(p), _ptr(r), _ptr(v)))
    return p, r, v


class Simulation:
    """One sgmd context: one or more replicas stepped together on one GPU."""

    def __init__(self, params: SimParams | Sequence[SimParams], mode: int = MODE_PLAIN, force_rebuild: bool = False,
                 use_graphs: bool = True, device: int = 0, rdf_ext_bins: int = 0, rdf_ext_range: float = 0.0,
                 eam_table_knots: int = 0, stream: int = 0, phase_timing: bool = False, metal_lanes: int = 0,
                 nebr_blocks_per_sm: int = 0, programmatic_launch: bool = True, nebr_descending: int = 0,
                 nebr_item_atoms: int = 0, nebr_build: int = 0, eam_table_smem: int = 0,
                 carbon_blocks_per_sm: int = 0, persistent_step: bool = False, persistent_wait_us: int = 0,
                 nebr_capacity: int = 0):
        plist = [params] if isinstance(params, SimParams) else list(params)
        arr = (SimParams * len(plist))(*plist)
        opt = Options()
        lib().sg_default_options(C.byref(opt))
        opt.mode = mode
        opt.force_rebuild = int(force_rebuild)
        opt.use_graphs = int(use_graphs)
        opt.device = device
        opt.rdf_ext_bins = rdf_ext_bins
        opt.rdf_ext_range = rdf_ext_range
        opt.eam_table_knots = eam_table_knots
        opt.stream = stream or None
        opt.phase_timing = int(phase_timing)
        opt.metal_lanes = metal_lanes
        opt.nebr_blocks_per_sm = nebr_blocks_per_sm
        opt.programmatic_launch = int(programmatic_launch)
        opt.nebr_descending = nebr_descending
        opt.nebr_item_atoms = nebr_item_atoms
        opt.nebr_build = nebr_build
        opt.eam_table_smem = eam_table_smem
        opt.carbon_blocks_per_sm = carbon_blocks_per_sm
        opt.persistent_step = int(persistent_step)
        opt.persistent_wait_us = persistent_wait_us
        opt.nebr_capacity = nebr_capacity
        h = C.c_void_p()
        check(lib().sg_create(arr, len(plist), C.byref(opt), C.byref(h)))
        self._h = h
        self.params0 = [q.copy() for q in plist]
        self.nrep = len(plist)

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def natoms(self, rep: int = -1) -> int:
        return lib().sg_num_atoms(self._h, rep)

    # -- state
    def _state_args(self, r, v, a, rep):
        n = self.natoms(rep)
        def prep(x, w):
            if x is None:
                return None
            x = np.ascontiguousarray(x, dtype=np.float32)
            if x.shape != (n, w):
                raise ValueError(f"expected shape {(n, w)}, got {x.shape}")
            return x
        return prep(r, 4), prep(v, 3), prep(a, 3)

    def set_state(self, r: np.ndarray | None, v: np.ndarray | None = None, a: np.ndarray | None = None,
                  rep: int = -1) -> None:
        r_, v_, a_ = self._state_args(r, v, a, rep)
        check(lib().sg_set_state(self._h, rep, _ptr(r_), _ptr(v_), _ptr(a_)))

    def step_from_host(self, r: np.ndarray | None, v: np.ndarray | None = None, a: np.ndarray | None = None,
                       nsteps: int = 1, rep: int = -1, thermo_rep: int | None = 0) -> Thermo | None:
        """set_state(r, v, a, rep), nsteps steps and replica thermo_rep's thermo record (None:
        no record) in one call with one wait (sg_step_from_host)."""
        r_, v_, a_ = self._state_args(r, v, a, rep)
        t = Thermo() if thermo_rep is not None else None
        check(lib().sg_step_from_host(self._h, rep, _ptr(r_), _ptr(v_), _ptr(a_), nsteps,
                                      0 if thermo_rep is None else thermo_rep,
                                      C.byref(t) if t is not None else None))
        return t

    def get_state(self, rep: int = -1):
        n = self.natoms(rep)
        r = np.zeros((n, 4), np.float32)
        v = np.zeros((n, 3), np.float32)
        a = np.zeros((n, 3), np.float32)
        check(lib().sg_get_state(self._h, rep, _ptr(r), _ptr(v), _ptr(a)))
        return r, v, a

    def params(self, rep: int = 0) -> SimParams:
        p = SimParams()
        check(lib().sg_get_params(self._h, rep, C.byref(p)))
        return p

    # -- stepping and phases
    def step(self, n: int = 1) -> None:
        check(lib().sg_step(self._h, n))

    def step_async(self, n: int = 1) -> None:
        """Launch n steps without waiting for them."""
        check(lib().sg_step_async(self._h, n))

    def kernels_per_step(self) -> int:
        return lib().sg_kernels_per_step(self._h)

    def phase_times(self) -> np.ndarray:
        """ms of the phases of the last step: integrate, rebuild (sort + list build), metal chain,
        carbon pass, forces (fork to join), reduce, extra (shear/RDF), list build alone."""
        out = np.zeros(8, np.float32)
        n = lib().sg_get_phase_times(self._h, _ptr(out), 8)
        if n < 0:
            check(-n)
        return out[:n]

    def step_thermo(self, nsteps: int = 1, rep: int = 0) -> Thermo:
        """nsteps steps and replica rep's thermo record, with one wait."""
        t = Thermo()
        check(lib().sg_step_thermo(self._h, nsteps, rep, C.byref(t)))
        return t

    def step_readback_bytes(self) -> int:
        return int(lib().sg_step_readback_bytes(self._h))

    def thermo(self, rep: int = 0) -> Thermo:
        t = Thermo()
        check(lib().sg_get_thermo(self._h, rep, C.byref(t)))
        return t

    def build_lists(self) -> None:
        check(lib().sg_build_lists(self._h))

    def compute_forces(self) -> None:
        check(lib().sg_compute_forces(self._h))

    def eval_rdf(self) -> None:
        check(lib().sg_eval_rdf(self._h))

    def reset_rdf(self) -> None:
        check(lib().sg_reset_rdf(self._h))

    # -- read-back
    def cells(self, rep: int = 0):
        p = self.params0[rep]
        nc = lib().sg_num_cells(self._h, rep)
        co = np.zeros(p.nMol, np.int32)
        cs = np.zeros(nc + 1, np.int32)
        ca = np.zeros(p.nMol, np.int32)
        check(lib().sg_get_cells(self._h, rep, _ptr(co), _ptr(cs), _ptr(ca)))
        return co, cs, ca

    def nebr(self, rep: int = 0):
        p = self.params0[rep]
        nn = np.zeros(p.nMol, np.int32)
        nbl = np.zeros((p.iNebrMax, p.nMol), np.int32)
        check(lib().sg_get_nebr(self._h, rep, _ptr(nn), _ptr(nbl)))
        return nn, nbl

    def short_lists(self, rep: int = 0):
        """The carbon pass's lists: (ns, sl[nMol, 8], nrl, rl[nMol, 48, 2]), local indices."""
        n = self.params0[rep].nMol
        ns, nrl = np.zeros(n, np.int32), np.zeros(n, np.int32)
        sl = np.zeros((n, 8), np.int32)
        rl = np.zeros((n, 48, 2), np.int32)
        check(lib().sg_get_carbon_lists(self._h, rep, _ptr(ns), _ptr(sl), _ptr(nrl), _ptr(rl)))
        return ns, sl, nrl, rl

    def rho(self, rep: int = 0) -> np.ndarray:
        out = np.zeros(self.params0[rep].nMolMe, np.float32)
        check(lib().sg_get_rho(self._h, rep, _ptr(out)))
        return out

    def friction(self, rep: int = 0) -> np.ndarray:
        out = np.zeros(self.params0[rep].nMolMe, np.float32)
        check(lib().sg_get_friction(self._h, rep, _ptr(out)))
        return out

    def rdf(self, rep: int = 0) -> np.ndarray:
        out = np.zeros(self.params0[rep].sizeHistRdf, np.uint32)
        check(lib().sg_get_rdf(self._h, rep, _ptr(out)))
        return out

    def rdf_ext(self, rep: int, nbins: int) -> np.ndarray:
        out = np.zeros(nbins, np.uint64)
        check(lib().sg_get_rdf_ext(self._h, rep, _ptr(out)))
        return out

    def diffusion(self, rep: int = 0):
        p = self.params0[rep]
        rr = np.zeros(p.nValDiffuse, np.float32)
        counts = np.zeros(p.nBuffDiffuse, np.int32)
        cav = C.c_int()
        check(lib().sg_get_diffusion(self._h, rep, _ptr(rr), _ptr(counts), C.byref(cav)))
        return rr, counts, cav.value

    def diag(self, rep: int = 0) -> Diag:
        d = Diag()
        check(lib().sg_get_diag(self._h, rep, C.byref(d)))
        return d

    def run(self, result_path: str | None, pdb_prefix: str = "sugr") -> None:
        """The whole simulation with the reference's output files (replica 0)."""
        L = libc()
        f = L.fopen(str(result_path).encode(), b"a") if result_path else None
        try:
            check(lib().sg_run(self._h, f, pdb_prefix.encode()))
        finally:
            if f:
                L.fclose(f)

    def load_diff_theta(self, theta: np.ndarray, rep: int = -1) -> None:
        """The differentiation form's fitted parameters (66 values) into this MIXED context's
        EAM tables and metal-carbon LJ parameters (sg_load_diff_theta)."""
        t = np.ascontiguousarray(theta, np.float64)
        check(lib().sg_load_diff_theta(self._h, rep, t.ctypes.data_as(C.c_void_p)))

    def autotune(self, steps: int = 20) -> dict:
        """Times the launch shapes (lanes per metal atom, list-build blocks per SM) on this
        context's state, keeps the fastest and restores the state; returns the timings."""
        buf = C.create_string_buffer(4096)
        check(lib().sg_autotune(self._h, steps, buf, len(buf)))
        return json.loads(buf.value.decode())

    SHAPE_FIELDS = ("metal_lanes", "nebr_blocks_per_sm", "nebr_descending", "nebr_item_atoms",
                    "programmatic_launch", "nebr_build", "eam_table_smem",
                    "carbon_blocks_per_sm")

    def launch_shape(self) -> dict:
        """The launch shape in use: the fields of sg_launch_shape."""
        s = LaunchShape()
        check(lib().sg_get_launch_shape(self._h, C.byref(s)))
        return {f: getattr(s, f) for f in self.SHAPE_FIELDS}

    def set_launch_shape(self, shape: dict) -> None:
        """Applies a launch shape (a dict as launch_shape() returns; missing fields keep their
        current values)."""
        cur = self.launch_shape()
        cur.update(shape)
        s = LaunchShape(*[cur[f] for f in self.SHAPE_FIELDS])
        check(lib().sg_set_launch_shape(self._h, C.byref(s)))


DIFF_NPARAM = 66  # SG_DIFF_NPARAM


def diff_frame_params(p: SimParams) -> SimParams:
    """The parameter block a differentiation frame is evaluated with (list radius covering the
    LJ cutoff); host only."""
    q = SimParams()
    check(lib().sg_diff_frame_params(C.byref(p), C.byref(q)))
    return q


def diff_init_theta(p: SimParams) -> np.ndarray:
    """theta at the reference model of a parameter block (splines fitted to the analytic EAM)."""
    t = np.zeros(DIFF_NPARAM)
    check(lib().sg_diff_init_theta(C.byref(p), _ptr(t)))
    return t


class DiffModel:
    """The differentiation form over a set of frames: energies, forces, force-matching loss and
    their gradients with respect to the 66 fit parameters (see include/sg_api.h)."""

    def __init__(self, frames: Sequence[SimParams], positions: np.ndarray, device: int = 0):
        arr = (SimParams * len(frames))(*frames)
        h = C.c_void_p()
        check(lib().sg_diff_create(arr, len(frames), device, C.byref(h)))
        self._h = h
        self.nframes = len(frames)
        self.n = lib().sg_diff_num_atoms(h)
        self.set_positions(positions)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sg_diff_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_positions(self, r: np.ndarray) -> None:
        r = np.ascontiguousarray(r, np.float32).reshape(self.n, 4)
        check(lib().sg_diff_set_positions(self._h, _ptr(r)))

    def energy(self, theta: np.ndarray, grad: bool = True):
        theta = np.ascontiguousarray(theta, np.float64)
        e = np.zeros(self.nframes)
        g = np.zeros(DIFF_NPARAM) if grad else None
        check(lib().sg_diff_energy(self._h, _ptr(theta), _ptr(e), _ptr(g)))
        return (e, g) if grad else e

    def forces(self, theta: np.ndarray) -> np.ndarray:
        theta = np.ascontiguousarray(theta, np.float64)
        f = np.zeros((self.n, 3), np.float32)
        check(lib().sg_diff_forces(self._h, _ptr(theta), _ptr(f)))
        return f

    def force_matching(self, theta: np.ndarray, ref_forces: np.ndarray, grad: bool = True):
        theta = np.ascontiguousarray(theta, np.float64)
        ref = np.ascontiguousarray(ref_forces, np.float32).reshape(self.n, 3)
        loss = np.zeros(1)
        g = np.zeros(DIFF_NPARAM) if grad else None
        check(lib().sg_diff_force_matching(self._h, _ptr(theta), _ptr(ref), _ptr(loss), _ptr(g)))
        return (float(loss[0]), g) if grad else float(loss[0])
