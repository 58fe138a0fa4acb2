"""TEST INFRASTRUCTURE: runs the reference's own CUDA kernels on injected states.

The reference's device code (SurfaceGrowthConsole/SurfaceGrowth.cu) is compiled unmodified into
two sm_103a cubins by oracle/ref/build_ref.sh, from the read-only reference tree (so the cubins
exist only where that tree was present at build time): `nofma` (-fmad=false, the operation order
the oracle and the PLAIN kernels follow) and `shipped` (nvcc's default flags, the reference as
built).  oracle/librefkern.so (oracle/ref/refkern.cpp) loads one through the CUDA driver API and
launches the reference's kernels with the reference's launch shapes.

Used by the tests that pin the oracle and the CUDA path to the reference's arithmetic, by the
script that records the reference-kernel golden fixtures, and by bench.py for the timing of
"the reference GPU path as shipped".  Never the product path.

The reference kernels check no bounds.  Before any launch this wrapper checks, on the CPU
oracle, that no cell holds more than blockSize atoms and no atom has iNebrMax neighbours or
more, and refuses the state otherwise.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
LIB = ROOT / "librefkern.so"
CUBINS = {"nofma": ROOT / "_ref" / "sgref_kernels_nofma.cubin",
          "shipped": ROOT / "_ref" / "sgref_kernels.cubin"}

_lib = None
_open = None


class RefKernelError(RuntimeError):
    pass


def available(kind: str = "nofma") -> str | None:
    """None when the reference kernels can run here, else the reason."""
    if not LIB.exists():
        return f"{LIB.name} not built"
    if not CUBINS[kind].exists():
        return f"{CUBINS[kind].name} missing (built only where the reference tree is present)"
    return None


def _L():
    global _lib
    if _lib is None:
        L = C.CDLL(str(LIB))
        V = C.c_void_p
        I = C.c_int
        sigs = {
            "rk_last_error": (C.c_char_p, []),
            "rk_open": (I, [C.c_char_p]),
            "rk_close": (I, []),
            "rk_setup": (I, [V]),
            "rk_set_state": (I, [V, V, V]),
            "rk_get_state": (I, [V, V, V]),
            "rk_bin": (I, [C.POINTER(I)]),
            "rk_get_cells": (I, [V, V]),
            "rk_set_cells": (I, [V]),
            "rk_build_nebr": (I, [C.POINTER(I)]),
            "rk_get_nebr": (I, [V, V]),
            "rk_set_nebr": (I, [V, V]),
            "rk_forces": (I, []),
            "rk_get_rho": (I, [V]),
            "rk_get_friction": (I, [V]),
            "rk_net_force": (I, [V]),
            "rk_leapfrog": (I, [I]),
            "rk_boundary": (I, []),
            "rk_reduce": (I, [I, C.c_float, V]),
            "rk_thermostat": (I, [I]),
            "rk_rdf": (I, [I]),
            "rk_get_rdf": (I, [V]),
            "rk_run_steps": (I, [I, I, C.POINTER(C.c_float)]),
            "rk_shear": (I, [C.c_float, C.c_float, C.POINTER(C.c_uint)]),
            "rk_get_params": (I, [V]),
            "rk_init_coords": (I, [V, V]),
        }
        for n, (r, a) in sigs.items():
            f = getattr(L, n)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _ck(rc):
    if rc != 0:
        raise RefKernelError(f"reference kernel harness: {_L().rk_last_error().decode()} (rc {rc})")


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _prechecks(params, r):
    """The reference kernels write past CELL / NBL when a cell holds more than blockSize atoms
    or an atom has iNebrMax neighbours or more: refuse such states, judged on the CPU oracle."""
    from oracle import OracleSim
    o = OracleSim(params, 32)
    o.set_state(np.ascontiguousarray(r, np.float32))
    o.build_lists()
    _, cs, _ = o.cells()
    nn, _ = o.nebr()
    occ = int(np.diff(cs).max()) if len(cs) > 1 else 0
    if occ > params.blockSize:
        raise RefKernelError(f"a cell holds {occ} atoms > blockSize {params.blockSize}")
    if int(nn.max()) >= params.iNebrMax:
        raise RefKernelError(f"an atom has {int(nn.max())} neighbours >= iNebrMax {params.iNebrMax}")


class RefKernels:
    """The reference's arrays for one system on device 0 and its kernels.  One instance at a time
    (the harness holds one module and one set of arrays)."""

    def __init__(self, params, r, v=None, a=None, kind: str = "nofma", check: bool = True):
        global _open
        why = available(kind)
        if why:
            raise RefKernelError(why)
        if check:
            _prechecks(params, r)
        L = _L()
        if _open != kind:
            if _open is not None:
                L.rk_close()
            _ck(L.rk_open(str(CUBINS[kind]).encode()))
            _open = kind
        self.p = params
        self.n = params.nMol
        self.ncells = params.cells.x * params.cells.y * params.cells.z
        _ck(L.rk_setup(C.byref(params)))
        r4 = np.ascontiguousarray(r, np.float32).reshape(self.n, 4)
        v3 = None if v is None else np.ascontiguousarray(v, np.float32).reshape(self.n, 3)
        a3 = None if a is None else np.ascontiguousarray(a, np.float32).reshape(self.n, 3)
        _ck(L.rk_set_state(_p(r4), _p(v3), _p(a3)))

    # ---- cells and lists
    def bin(self):
        occ = C.c_int(0)
        _ck(_L().rk_bin(C.byref(occ)))
        return occ.value

    def cells(self):
        cell = np.zeros(self.p.maxMol + 1, np.int32)
        mic = np.zeros(self.ncells, np.uint32)
        _ck(_L().rk_get_cells(_p(cell), _p(mic)))
        return cell, mic

    def canonicalize_cells(self):
        """Sort every cell's atoms by index.  BinAtomsIntoCellsK fills a cell in the order in
        which its atomicAdds resolve (SurfaceGrowth.cu:572-575, 600-603), which inside one
        64-atom chunk is not fixed; ascending index is one of its possible outcomes and the
        order the oracle and the CUDA path use."""
        cell, mic = self.cells()
        bs = self.p.blockSize
        for c in np.nonzero(mic)[0]:
            seg = cell[c * bs:c * bs + mic[c]]
            seg.sort()
        _ck(_L().rk_set_cells(_p(cell)))
        return cell, mic

    def build_nebr(self):
        mx = C.c_int(0)
        _ck(_L().rk_build_nebr(C.byref(mx)))
        if mx.value >= self.p.iNebrMax:
            raise RefKernelError(f"neighbour count {mx.value} reached iNebrMax")
        return mx.value

    def nebr(self):
        nn = np.zeros(self.n, np.int32)
        nbl = np.zeros((self.p.iNebrMax, self.n), np.int32)  # NBL[j * nMol + i], column-major
        _ck(_L().rk_get_nebr(_p(nn), _p(nbl)))
        return nn, nbl

    def lists(self):
        """Bin, put every cell in ascending index order, build the neighbour list."""
        occ = self.bin()
        if occ > self.p.blockSize:
            raise RefKernelError(f"cell occupancy {occ} > blockSize")
        self.canonicalize_cells()
        return self.build_nebr()

    # ---- forces, integrator, reductions, RDF
    def forces(self):
        _ck(_L().rk_forces())

    def rho(self):
        out = np.zeros(max(self.p.nMolMe, 1), np.float32)
        _ck(_L().rk_get_rho(_p(out)))
        return out[:self.p.nMolMe]

    def friction(self):
        out = np.zeros(max(self.p.nMolMe, 1), np.float32)
        _ck(_L().rk_get_friction(_p(out)))
        return out[:self.p.nMolMe]

    def net_force(self):
        out = np.zeros(1, np.float32)
        _ck(_L().rk_net_force(_p(out)))
        return float(out[0])

    def leapfrog(self, part):
        _ck(_L().rk_leapfrog(part))

    def boundary(self):
        _ck(_L().rk_boundary())

    def reduce(self, which, cm_vel_x=0.0):
        out = np.zeros(3, np.float32)
        _ck(_L().rk_reduce(which, cm_vel_x, _p(out)))
        return out

    def thermostat(self, step_count):
        _ck(_L().rk_thermostat(step_count))

    def rdf(self, count_rdf=0):
        _ck(_L().rk_rdf(count_rdf))

    def hist(self):
        out = np.zeros(self.p.sizeHistRdf, np.uint32)
        _ck(_L().rk_get_rdf(_p(out)))
        return out

    def state(self):
        r = np.zeros((self.n, 4), np.float32)
        v = np.zeros((self.n, 3), np.float32)
        a = np.zeros((self.n, 3), np.float32)
        _ck(_L().rk_get_state(_p(r), _p(v), _p(a)))
        return r, v, a

    def shear(self, shear, center_of_mass_x):
        """ApplyShearK on the current state; returns the number of sheared metal atoms."""
        cnt = C.c_uint(0)
        _ck(_L().rk_shear(shear, center_of_mass_x, C.byref(cnt)))
        return cnt.value

    def params(self):
        """The step loop's host-side parameter block after run_steps."""
        out = self.p.copy()
        _ck(_L().rk_get_params(C.byref(out)))
        return out

    def run_steps(self, steps, force_rebuild=True):
        """The reference step loop's device work; returns elapsed ms."""
        ms = C.c_float(0)
        _ck(_L().rk_run_steps(steps, 1 if force_rebuild else 0, C.byref(ms)))
        return ms.value


def init_coords(params, kind: str = "nofma"):
    """The reference's lattice kernels as InitCoordsW launches them (SurfaceGrowth.cu:2532-2609):
    returns (positions (nMol, 4) float32, the parameter block with initUcellMeX/Y as the wrapper
    writes them).  Regime-1 metal rows are zeros (the reference fills them on the host)."""
    global _open
    why = available(kind)
    if why:
        raise RefKernelError(why)
    L = _L()
    if _open != kind:
        if _open is not None:
            L.rk_close()
        _ck(L.rk_open(str(CUBINS[kind]).encode()))
        _open = kind
    q = params.copy()
    out = np.zeros((q.nMol, 4), np.float32)
    _ck(L.rk_init_coords(C.byref(q), _p(out)))
    return out, q
