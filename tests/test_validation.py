"""sg_create's checks on the parameter blocks, without a GPU: an empty system, inconsistent atom
counts, a bad cell grid and replicas whose host-side schedules differ are rejected with
SG_ERR_INVALID before any device call; a valid block on a machine without a device fails with
SG_ERR_NO_DEVICE, never with a fault or a silent fallback.
"""
import ctypes as C

import pytest

from surfacegrowthconsole_gb300 import _lib as L
from surfacegrowthconsole_gb300 import workloads

SG_ERR_INVALID, SG_ERR_NO_DEVICE = 1, 4


def _create(blocks, n=None):
    arr = (L.SimParams * len(blocks))(*blocks)
    ctx = C.c_void_p()
    rc = L.lib().sg_create(C.cast(arr, C.POINTER(L.SimParams)), len(blocks) if n is None else n, None,
                           C.byref(ctx))
    msg = L.lib().sg_last_error().decode(errors="replace")
    if rc == 0:
        L.lib().sg_destroy(ctx)
    return rc, msg


def _small():
    p, _, _ = workloads.small()
    return p


def _copy(p):
    q = L.SimParams()
    C.memmove(C.byref(q), C.byref(p), C.sizeof(L.SimParams))
    return q


def test_empty_system_is_rejected():
    q = _copy(_small())
    q.nMol = 0
    q.nMolMe = 0
    rc, msg = _create([q])
    assert rc == SG_ERR_INVALID and "atom counts" in msg


def test_more_metal_than_atoms_is_rejected():
    q = _copy(_small())
    q.nMolMe = q.nMol + 1
    rc, msg = _create([q])
    assert rc == SG_ERR_INVALID and "atom counts" in msg


@pytest.mark.parametrize("axis", ["x", "y", "z"])
def test_empty_cell_grid_is_rejected(axis):
    q = _copy(_small())
    setattr(q.cells, axis, 0)
    rc, msg = _create([q])
    assert rc == SG_ERR_INVALID and "cell grid" in msg


def test_replicas_with_different_schedules_are_rejected():
    a, b = _copy(_small()), _copy(_small())
    b.stepRdf = a.stepRdf + 1
    rc, msg = _create([a, b])
    assert rc == SG_ERR_INVALID and "replica 1" in msg and "schedule" in msg


def test_no_replicas_is_rejected():
    rc, _ = _create([_copy(_small())], n=0)
    assert rc == SG_ERR_INVALID


def test_valid_system_without_a_device_reports_no_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    rc, msg = _create([_copy(_small())])
    assert rc == SG_ERR_NO_DEVICE, msg


def _noalloc(p, pos=1, acc=1):
    # every block here fails the checks that run before any device call, so the placeholder
    # pointers are never used; on a machine with a GPU these cases are left to the GPU tests,
    # which pass real buffers
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: covered with real buffers by the GPU tests")
    rc = L.lib().sg_compute_forces_noalloc(C.byref(p), C.c_void_p(pos), C.c_void_p(acc), None)
    return rc, L.lib().sg_last_error().decode(errors="replace")


def test_noalloc_rejects_null_buffers_and_bad_blocks():
    p = _copy(_small())
    assert _noalloc(p, pos=0)[0] == SG_ERR_INVALID
    assert _noalloc(p, acc=0)[0] == SG_ERR_INVALID
    q = _copy(p)
    q.nMol = 0
    assert _noalloc(q)[0] == SG_ERR_INVALID
    q = _copy(p)
    q.cells.z = 0
    assert _noalloc(q)[0] == SG_ERR_INVALID


def test_noalloc_rejects_systems_above_its_static_scratch():
    p = _copy(_small())
    q = _copy(p)
    q.nMol = 16384 + 1
    rc, msg = _noalloc(q)
    assert rc == SG_ERR_INVALID and "static scratch" in msg
    # extents whose product wraps a 32-bit int to a small value are still rejected
    q = _copy(p)
    q.cells.x, q.cells.y, q.cells.z = 65536, 65536, 1
    rc, msg = _noalloc(q)
    assert rc == SG_ERR_INVALID and "static scratch" in msg
    q = _copy(p)
    q.iNebrMax = 129
    rc, msg = _noalloc(q)
    assert rc == SG_ERR_INVALID and "static scratch" in msg
