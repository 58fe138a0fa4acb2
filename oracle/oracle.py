"""TEST INFRASTRUCTURE: ctypes binding of the CPU oracle (oracle/liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as the
checker.  It is never the product path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
LIB = ROOT / "liboracle.so"

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} missing: run the build first")
        from surfacegrowthconsole_gb300._lib import Diag, SimParams, Thermo
        L = C.CDLL(str(LIB))
        V = C.c_void_p
        sigs = {
            "orc_create": (V, [C.POINTER(SimParams), C.c_int, C.c_int]),
            "orc_destroy": (None, [V]),
            "orc_set_threads": (None, [C.c_int]),
            "orc_get_threads": (C.c_int, []),
            "orc_set_state": (None, [V, V, V, V]),
            "orc_get_state": (None, [V, V, V, V]),
            "orc_get_state64": (None, [V, V, V, V]),
            "orc_metal_cm64": (None, [V, V]),
            "orc_set_state64": (None, [V, V, V, V]),
            "orc_step": (C.c_int, [V, C.c_int]),
            "orc_get_thermo": (None, [V, C.POINTER(Thermo)]),
            "orc_get_params": (None, [V, C.POINTER(SimParams)]),
            "orc_build_lists": (C.c_int, [V]),
            "orc_compute_forces": (C.c_int, [V]),
            "orc_eval_rdf": (C.c_int, [V]),
            "orc_reset_rdf": (None, [V]),
            "orc_num_cells": (C.c_int, [V]),
            "orc_get_cells": (None, [V, V, V, V]),
            "orc_get_nebr": (None, [V, V, V]),
            "orc_get_rho": (None, [V, V]),
            "orc_get_friction": (None, [V, V]),
            "orc_get_rdf": (None, [V, V]),
            "orc_get_diffusion": (None, [V, V, V, V]),
            "orc_get_diag": (None, [V, C.POINTER(Diag)]),
            "orc_reduce": (None, [C.POINTER(SimParams), C.c_int, V, V, V, C.c_float, V]),
            "orc_diffusion_replay": (C.c_int, [C.POINTER(SimParams), C.c_int, V, V, C.c_int]),
            "orc_eam_eval": (C.c_double, [C.POINTER(SimParams), C.c_int, C.c_double, C.c_int]),
            "orc_rdf_allpairs": (None, [C.POINTER(SimParams), V, C.c_int, C.c_double, V]),
            "orc_diff_eval": (C.c_int, [V, C.c_int, V, V, V, V, V, V, V, V]),
            "orc_get_last_avg": (None, [V, V]),
            "orc_num_prints": (C.c_int, [V, C.c_int]),
            "orc_get_rdf_print": (None, [V, V]),
            "orc_get_diffuse_print": (C.c_int, [V, C.c_int, V]),
        }
        for n, (r, a) in sigs.items():
            f = getattr(L, n)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleSim:
    """One system on the CPU oracle; precision 32 (reference arithmetic) or 64."""

    def __init__(self, params, precision: int = 32, force_rebuild: bool = False):
        self.p = params.copy()
        self.n = params.nMol
        self._h = lib().orc_create(C.byref(self.p), precision, int(force_rebuild))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def set_state(self, r, v=None, a=None):
        r = None if r is None else np.ascontiguousarray(r, np.float32)
        v = None if v is None else np.ascontiguousarray(v, np.float32)
        a = None if a is None else np.ascontiguousarray(a, np.float32)
        lib().orc_set_state(self._h, _p(r), _p(v), _p(a))

    def get_state(self):
        r = np.zeros((self.n, 4), np.float32)
        v = np.zeros((self.n, 3), np.float32)
        a = np.zeros((self.n, 3), np.float32)
        lib().orc_get_state(self._h, _p(r), _p(v), _p(a))
        return r, v, a

    def get_state64(self):
        r = np.zeros((self.n, 4))
        v = np.zeros((self.n, 3))
        a = np.zeros((self.n, 3))
        lib().orc_get_state64(self._h, _p(r), _p(v), _p(a))
        return r, v, a

    def metal_cm64(self):
        """Mean metal position in FP64."""
        out = np.zeros(3)
        lib().orc_metal_cm64(self._h, _p(out))
        return out

    def step(self, n: int = 1):
        lib().orc_step(self._h, n)

    def thermo(self):
        from surfacegrowthconsole_gb300._lib import Thermo
        t = Thermo()
        lib().orc_get_thermo(self._h, C.byref(t))
        return t

    def params(self):
        from surfacegrowthconsole_gb300._lib import SimParams
        q = SimParams()
        lib().orc_get_params(self._h, C.byref(q))
        return q

    def build_lists(self):
        lib().orc_build_lists(self._h)

    def compute_forces(self):
        lib().orc_compute_forces(self._h)

    def eval_rdf(self):
        lib().orc_eval_rdf(self._h)

    def reset_rdf(self):
        lib().orc_reset_rdf(self._h)

    def cells(self):
        nc = lib().orc_num_cells(self._h)
        co = np.zeros(self.n, np.int32)
        cs = np.zeros(nc + 1, np.int32)
        ca = np.zeros(self.n, np.int32)
        lib().orc_get_cells(self._h, _p(co), _p(cs), _p(ca))
        return co, cs, ca

    def nebr(self):
        nn = np.zeros(self.n, np.int32)
        nbl = np.zeros((self.p.iNebrMax, self.n), np.int32)
        lib().orc_get_nebr(self._h, _p(nn), _p(nbl))
        return nn, nbl

    def rho(self):
        out = np.zeros(self.p.nMolMe, np.float32)
        lib().orc_get_rho(self._h, _p(out))
        return out

    def friction(self):
        out = np.zeros(self.p.nMolMe, np.float32)
        lib().orc_get_friction(self._h, _p(out))
        return out

    def rdf(self):
        out = np.zeros(self.p.sizeHistRdf, np.uint32)
        lib().orc_get_rdf(self._h, _p(out))
        return out

    def diffusion(self):
        rr = np.zeros(self.p.nValDiffuse, np.float32)
        counts = np.zeros(self.p.nBuffDiffuse, np.int32)
        cav = C.c_int()
        lib().orc_get_diffusion(self._h, _p(rr), _p(counts), C.byref(cav))
        return rr, counts, cav.value

    def last_avg(self):
        """The seven property accumulators {val, sum, sum2} of the last averaging step, before
        they were zeroed: totEnergy, potEnergy, kinEnergy, oneStep, centerOfMass, cmVel,
        frictForce (PrintSummary's inputs)."""
        from surfacegrowthconsole_gb300._lib import Prop
        out = (Prop * 7)()
        lib().orc_get_last_avg(self._h, C.cast(out, C.c_void_p))
        return list(out)

    def num_rdf_prints(self) -> int:
        return lib().orc_num_prints(self._h, 0)

    def num_diffusion_tables(self) -> int:
        return lib().orc_num_prints(self._h, 1)

    def rdf_print(self):
        out = np.zeros(self.p.sizeHistRdf, np.uint32)
        lib().orc_get_rdf_print(self._h, _p(out))
        return out

    def diffusion_table(self, k: int):
        out = np.zeros(self.p.nValDiffuse, np.float32)
        if lib().orc_get_diffuse_print(self._h, k, _p(out)) != 0:
            raise IndexError(k)
        return out

    def diag(self):
        from surfacegrowthconsole_gb300._lib import Diag
        d = Diag()
        lib().orc_get_diag(self._h, C.byref(d))
        return d


def set_threads(n: int) -> None:
    lib().orc_set_threads(n)


def get_threads() -> int:
    return lib().orc_get_threads()


def reduce(params, what: int, r, v, fric=None, cm_vel_x: float = 0.0):
    out = np.zeros(3, np.float32)
    r = np.ascontiguousarray(r, np.float32)
    v = np.ascontiguousarray(v, np.float32)
    f = None if fric is None else np.ascontiguousarray(fric, np.float32)
    lib().orc_reduce(C.byref(params), what, _p(r), _p(v), _p(f), cm_vel_x, _p(out))
    return out


def eam_eval(params, which: int, x: float, precision: int = 64) -> float:
    return lib().orc_eam_eval(C.byref(params), which, x, precision)


def rdf_allpairs(params, r, nbins: int, rng: float):
    out = np.zeros(nbins, np.uint64)
    r = np.ascontiguousarray(r, np.float32)
    lib().orc_rdf_allpairs(C.byref(params), _p(r), nbins, rng, _p(out))
    return out


def diffusion_replay(params, cm):
    """Finished diffusion tables for a sequence of centre-of-mass samples (n, 3)."""
    cm = np.ascontiguousarray(cm, np.float32)
    maxt = 64
    out = np.zeros((maxt, params.nValDiffuse), np.float32)
    k = lib().orc_diffusion_replay(C.byref(params), len(cm), _p(cm), _p(out), maxt)
    return [out[i] for i in range(k)]


def diff_eval(frames, r, theta, ref=None):
    """The differentiation form in FP64: (energy per frame, forces (N, 3), dE/dtheta,
    loss, dL/dtheta); frames are parameter blocks from sg_diff_frame_params."""
    from surfacegrowthconsole_gb300._lib import SimParams
    arr = (SimParams * len(frames))(*frames)
    n = sum(q.nMol for q in frames)
    r = np.ascontiguousarray(r, np.float32).reshape(n, 4)
    theta = np.ascontiguousarray(theta, np.float64)
    rf = None if ref is None else np.ascontiguousarray(ref, np.float32).reshape(n, 3)
    e = np.zeros(len(frames))
    f = np.zeros((n, 3))
    gE = np.zeros(66)
    loss = np.zeros(1)
    gL = np.zeros(66)
    lib().orc_diff_eval(C.cast(arr, C.c_void_p), len(frames), _p(r), _p(theta), _p(rf), _p(e), _p(f), _p(gE),
                        _p(loss), _p(gL))
    return e, f, gE, float(loss[0]), gL
