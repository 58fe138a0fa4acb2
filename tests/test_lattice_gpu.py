"""Initial lattices against the reference's own kernels on the GPU.

The reference builds its initial state on the device (InitCoordsW, SurfaceGrowth.cu:2532-2609):
InitFccCoordsK (cu:219-250) for the bulk crystal, InitGrapheneCoordsK (cu:301-394) for the sheet
and InitSlabCoordsK (cu:253-299) for the metal slab of the shear regime.  The library restates
them on the host (sg_init_coords).  The sheet's positions decide the freeze mask, which compares
positions with exact float equality (cu:416-424), so the restatement must be bit-identical.
These tests run the reference's kernels (oracle/refkern.py) with the wrapper's launch shapes on
the same parameter blocks and compare every coordinate bit for bit, plus initUcellMeX/Y, which
InitCoordsW writes back into the parameter block.
"""
import numpy as np
import pytest

import refkern
from surfacegrowthconsole_gb300.engine import default_input, init_coords, set_params

pytestmark = pytest.mark.gpu

# (regime, material, ucx, ucy, ucz, nMolMe)
CASES = [
    (0, 0, 4, 5, 6, 0),      # bulk Cu, unequal sides
    (0, 1, 8, 8, 8, 0),      # bulk Ag, the shipped input's crystal
    (0, 3, 10, 10, 10, 0),   # bulk Ni, 4,000 atoms
    (1, 4, 8, 8, 0, 1500),   # growth Al: sheet only (the metal comes from the host generator)
    (1, 5, 3, 2, 0, 50),
    (2, 3, 7, 9, 0, 300),    # shear Ni: sheet + one slab layer
    (2, 3, 7, 9, 0, 150),
    (2, 3, 10, 12, 0, 2001),  # several layers, a partial last cell
    (2, 2, 30, 30, 0, 25000),  # the shipped shear input's size (Au)
]


def params(case):
    reg, mat, ux, uy, uz, nme = case
    inp = default_input()
    inp.iRegime, inp.iMaterial, inp.ucx, inp.ucy, inp.ucz, inp.nMolMe = reg, mat, ux, uy, uz, nme
    inp.randSeed = 7
    return set_params(inp)


@pytest.fixture(scope="module", autouse=True)
def _reference_kernels():
    why = refkern.available("nofma")
    if why:
        pytest.skip(why)


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"regime{c[0]}_m{c[1]}_{c[2]}x{c[3]}x{c[4]}_me{c[5]}")
def test_lattice_bit_identical_to_the_reference_kernels(case):
    p = params(case)
    q = p.copy()
    r = init_coords(q)
    rr, qr = refkern.init_coords(p, "nofma")
    lo = p.nMolMe if p.iRegime == 1 else 0  # regime 1: metal from the host generator
    assert np.array_equal(r[lo:].view(np.uint32), rr[lo:].view(np.uint32))
    if p.iRegime == 2:
        assert (q.initUcellMeX, q.initUcellMeY) == (qr.initUcellMeX, qr.initUcellMeY)
        assert q.initUcellMeX > 0
    # the sheet sits at z_0 and some atoms lie on the freeze lines
    if p.iRegime != 0:
        assert np.all(r[p.nMolMe:, 2] == np.float32(p.z_0))


@pytest.mark.parametrize("case", [CASES[1], CASES[5], CASES[8]], ids=["bulk", "shear", "shear_large"])
def test_lattice_against_the_kernels_as_shipped(case):
    """The reference built with nvcc's default flags (FMA contraction on) fuses a lattice
    product with the following box shift (c * gap - 0.5 * region): one rounding of a box-sized
    intermediate fewer, so a coordinate may differ by up to one ulp of the box extent from the
    uncontracted arithmetic (the build the library and the parity tests follow; on a GB300 some
    thousands of coordinates per system differ, by as much as 40 ulp of a coordinate near the
    box centre).  Both builds freeze the same atoms: each compares the positions it generated."""
    if refkern.available("shipped"):
        pytest.skip(refkern.available("shipped"))
    p = params(case)
    r = init_coords(p.copy())
    rr, _ = refkern.init_coords(p, "shipped")
    lo = p.nMolMe if p.iRegime == 1 else 0
    diff = np.abs(r[lo:, :3].astype(np.float64) - rr[lo:, :3].astype(np.float64))
    box_ulp = float(np.spacing(np.float32(max(p.region.x, p.region.y, p.region.z))))
    print(f"shipped build: {int((diff > 0).sum())} of {diff.size} coordinates differ, "
          f"max {diff.max() / box_ulp:.2f} ulp of the box extent")
    assert diff.max() <= box_ulp
