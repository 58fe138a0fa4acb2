"""Backup files (bckup0/1.sugr) without a GPU: the byte layout of the reference's writer and a
write / read / resume cycle on the CPU oracle.

The reference writes, every stepBckup steps, the parameter block followed by the positions
(float4), velocities (float3) and accelerations (float3) of all atoms (SurfaceGrowth.cu:
2456-2481, four fwrite calls); it parses a restart flag (SurfaceGrowth.cpp:775) but has no
reader.  sg_read_backup is that reader.  A run resumed from a backup rebuilds its lists at its
first step (as the reference's own start does, SurfaceGrowth.cpp:418), so it continues bit for
bit like the uninterrupted run when the backup falls on a step after which a rebuild is due.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from surfacegrowthconsole_gb300 import _lib as L
from surfacegrowthconsole_gb300 import workloads


def write_backup(path, p, r, v, a):
    r = np.ascontiguousarray(r, np.float32)
    v = np.ascontiguousarray(v, np.float32)
    a = np.ascontiguousarray(a, np.float32)
    L.check(L.lib().sg_write_backup(str(path).encode(), C.byref(p), r.ctypes.data, v.ctypes.data, a.ctypes.data))


def read_backup(path):
    q = L.SimParams()
    L.check(L.lib().sg_read_backup(str(path).encode(), C.byref(q), None, None, None))  # nMol first
    r = np.zeros((q.nMol, 4), np.float32)
    v = np.zeros((q.nMol, 3), np.float32)
    a = np.zeros((q.nMol, 3), np.float32)
    L.check(L.lib().sg_read_backup(str(path).encode(), C.byref(q), r.ctypes.data, v.ctypes.data, a.ctypes.data))
    return q, r, v, a


def test_backup_byte_layout_is_the_references(tmp_path):
    p, r, v = workloads.small(seed=81)
    p.stepCount = 1234
    p.shear = 0.25
    a = np.random.RandomState(2).normal(size=(p.nMol, 3)).astype(np.float32)
    f = tmp_path / "bckup0.sugr"
    write_backup(f, p, r, v, a)
    data = f.read_bytes()
    n = p.nMol
    assert len(data) == 1112 + n * (16 + 12 + 12)
    assert data[:1112] == bytes(p)
    assert data[1112:1112 + 16 * n] == r.tobytes()
    assert data[1112 + 16 * n:1112 + 28 * n] == v.tobytes()
    assert data[1112 + 28 * n:] == a.tobytes()
    q, r2, v2, a2 = read_backup(f)
    assert bytes(q) == bytes(p)
    assert np.array_equal(r2, r) and np.array_equal(v2, v) and np.array_equal(a2, a)


def test_truncated_or_foreign_files_are_rejected(tmp_path):
    p, r, v = workloads.small(seed=82)
    a = np.zeros((p.nMol, 3), np.float32)
    f = tmp_path / "b.sugr"
    write_backup(f, p, r, v, a)
    data = f.read_bytes()
    (tmp_path / "short.sugr").write_bytes(data[:-12])
    (tmp_path / "long.sugr").write_bytes(data + b"\0" * 4)
    (tmp_path / "tiny.sugr").write_bytes(data[:500])
    bad = bytearray(data)
    bad[88:92] = (-5).to_bytes(4, "little", signed=True)  # nMol
    (tmp_path / "neg.sugr").write_bytes(bytes(bad))
    q = L.SimParams()
    for name in ("short", "long", "tiny", "neg"):
        rc = L.lib().sg_read_backup(str(tmp_path / f"{name}.sugr").encode(), C.byref(q), None, None, None)
        assert rc == 12, name  # SG_ERR_BAD_FILE
    rc = L.lib().sg_read_backup(str(tmp_path / "missing.sugr").encode(), C.byref(q), None, None, None)
    assert rc == 9  # SG_ERR_IO


def first_rebuild_due(orc, start, stop):
    """Steps the oracle from start to the first step k in [start, stop) after which a rebuild is
    due; returns k."""
    for k in range(start, stop):
        orc.step(1)
        if orc.thermo().nebrNow:
            return k + 1
    raise AssertionError("no rebuild due in the window")


@pytest.mark.parametrize("force_rebuild", [False, True], ids=["rule", "every_step"])
def test_kill_and_resume_on_the_oracle_is_bit_exact(tmp_path, force_rebuild):
    """Write a backup, read it back, continue in a fresh oracle: the same trajectory as the run
    that was never interrupted, across a thermostat step (25)."""
    p, r, v = workloads.small(seed=83)
    a = np.zeros((p.nMol, 3), np.float32)
    total = 40
    run = oracle.OracleSim(p, 32, force_rebuild=force_rebuild)
    run.set_state(r, v, a)
    k = 12 if force_rebuild else first_rebuild_due(run, 0, total - 5)
    if force_rebuild:
        run.step(k)
    f = tmp_path / "bckup0.sugr"
    rk, vk, ak = run.get_state()
    write_backup(f, run.params(), rk, vk, ak)
    run.step(total - k)

    q, r2, v2, a2 = read_backup(f)
    assert q.stepCount == k
    res = oracle.OracleSim(q, 32, force_rebuild=force_rebuild)
    res.set_state(r2, v2, a2)
    res.step(total - k)
    for x, y in zip(run.get_state(), res.get_state()):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    t0, t1 = run.thermo(), res.thermo()
    assert t0.stepCount == t1.stepCount == total
    assert t0.totEnergy == t1.totEnergy and t0.kinEnergy == t1.kinEnergy
