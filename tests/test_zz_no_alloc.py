"""sg_compute_forces_noalloc: the force evaluation for callers that cannot call cudaMalloc
(code under another framework's memory manager that owns the device heap, code that must not
stall the device with cudaMalloc/cudaFree synchronisation, plugins with a fixed footprint).
Its scratch is a static device array, so its results must equal those of the context path
(sg_build_lists + sg_compute_forces) on the same input, call after call, although every call
reuses the previous call's scratch contents."""
import ctypes as C

import numpy as np
import pytest

from surfacegrowthconsole_gb300 import _lib as L
from surfacegrowthconsole_gb300 import workloads
from surfacegrowthconsole_gb300.engine import Simulation

pytestmark = pytest.mark.gpu

FORCE_RTOL = 2e-5  # the tolerance of the parity tests (tests/test_parity_gpu.py)
FORCE_ATOL = 1e-6


def _context_forces(p, r, v):
    sim = Simulation(p)
    sim.set_state(r, v, np.zeros((p.nMol, 3), np.float32))
    sim.build_lists()
    sim.compute_forces()
    rg, _, ag = sim.get_state()
    sim.close()
    return rg[:, 3], ag


def _noalloc_forces(p, r):
    import torch
    dpos = torch.from_numpy(np.ascontiguousarray(r, np.float32)).cuda()
    dacc = torch.full((p.nMol, 4), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    L.check(L.lib().sg_compute_forces_noalloc(C.byref(p), C.c_void_p(dpos.data_ptr()), C.c_void_p(dacc.data_ptr()),
                                              C.c_void_p(stream)))
    return dpos.cpu().numpy()[:, 3], dacc.cpu().numpy()[:, :3]


def _close(x, y):
    scale = max(float(np.abs(y).max()), 1e-30)
    return float(np.abs(x.astype(np.float64) - y).max()) <= FORCE_RTOL * scale + FORCE_ATOL


def test_noalloc_forces_match_context_path_two_calls():
    p, r0, v = workloads.small(seed=61)
    rng = np.random.RandomState(61)
    # two calls in a row on different states: the second sees the first call's scratch
    for jitter in (0.05, 0.02):
        r = r0.copy()
        r[:, :3] += rng.normal(0, jitter, size=(p.nMol, 3)).astype(np.float32)
        u_ctx, a_ctx = _context_forces(p, r, v)
        u_na, a_na = _noalloc_forces(p, r)
        assert np.isfinite(a_na).all()
        assert _close(a_na, a_ctx), "accelerations differ from the context path"
        assert _close(u_na, u_ctx), "per-atom energies differ from the context path"


def test_noalloc_call_allocates_no_device_memory():
    """After a first call (which looks up the static array's address), a call leaves the
    device's free memory exactly as it was: no allocation, no growth of any pool."""
    import torch
    p, r, v = workloads.small(seed=63)
    dpos = torch.from_numpy(np.ascontiguousarray(r, np.float32)).cuda()
    dacc = torch.zeros((p.nMol, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    args = (C.byref(p), C.c_void_p(dpos.data_ptr()), C.c_void_p(dacc.data_ptr()), C.c_void_p(stream))
    L.check(L.lib().sg_compute_forces_noalloc(*args))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        L.check(L.lib().sg_compute_forces_noalloc(*args))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_cell_extents_whose_product_wraps():
    """A parameter block from outside with cell extents whose product overflows 32 bits is
    rejected, not wrapped into a small count that would pass the limit."""
    p, r, _ = workloads.small(seed=64)
    q = p.copy()
    q.cells.x, q.cells.y, q.cells.z = 65536, 65536, 2  # 2^33 cells: 0 in 32-bit arithmetic
    with pytest.raises(L.SgError) as e:
        _noalloc_forces(q, r)
    assert e.value.code == 1 and "exceeds the static scratch" in str(e.value)


def test_noalloc_rejects_systems_above_its_limit():
    p, r, _ = workloads.production(seed=62, steps=10)  # 45,546 atoms > SG_NOALLOC_MAX_ATOMS
    with pytest.raises(L.SgError) as e:
        _noalloc_forces(p, r)
    assert e.value.code == 1 and "exceeds the static scratch" in str(e.value)
