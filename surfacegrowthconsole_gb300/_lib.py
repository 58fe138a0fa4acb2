"""ctypes binding of libsgmd.so (include/sg_api.h, include/sg_refcompat.h).

The structures below mirror the C headers field for field; `SimParams` has the byte layout of
the reference's SimParams (SurfaceGrowthConsole/SurfaceGrowth.h:69-186).  Loading fails loudly
when the library has not been built: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIBPATH = PKG / "lib" / "libsgmd.so"

c_float_p = C.POINTER(C.c_float)
c_int_p = C.POINTER(C.c_int)


class Float3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Float4(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("w", C.c_float)]


class Int3(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]


class UInt3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


class Prop(C.Structure):
    _fields_ = [("val", C.c_float), ("sum", C.c_float), ("sum2", C.c_float)]


MAX_PATH = 264


class SimParams(C.Structure):
    _fields_ = [
        ("region", Float3), ("vSum", Float3), ("initUcell", UInt3),
        ("deltaT", C.c_float), ("rCutC", C.c_float), ("rrCutC", C.c_float), ("temperature", C.c_float),
        ("velMag", C.c_float),
        ("moreCycles", C.c_int), ("stepAvg", C.c_int), ("stepEquil", C.c_int), ("stepCount", C.c_int),
        ("stepPdb", C.c_int), ("stepLimit", C.c_int), ("bPdb", C.c_int), ("bResult", C.c_int),
        ("nMol", C.c_int), ("nMolMe", C.c_int), ("gridSize", C.c_uint), ("blockSize", C.c_uint),
        ("cells", Int3), ("invWidth", Float3), ("rNebrShell", C.c_float), ("rrNebr", C.c_float),
        ("iNebrMax", C.c_int), ("maxMol", C.c_int), ("nebrNow", C.c_int), ("dispHi", C.c_float),
        ("kinEnergy", Prop), ("totEnergy", Prop), ("potEnergy", Prop), ("oneStep", Prop),
        ("a", C.c_float), ("re", C.c_float), ("fe", C.c_float), ("rhoe", C.c_float), ("alpha", C.c_float),
        ("beta", C.c_float), ("A", C.c_float), ("B", C.c_float), ("kappa", C.c_float), ("lambda_", C.c_float),
        ("Fn", C.c_float * 4), ("F", C.c_float * 4), ("eta", C.c_float), ("Fe", C.c_float),
        ("massMe", C.c_float), ("density", C.c_float), ("rCutEam", C.c_float), ("rrCutEam", C.c_float),
        ("rei", C.c_float), ("rhoei", C.c_float), ("szNameMe", C.c_char * 3),
        ("temperatureU", C.c_float), ("kB", C.c_float), ("enU", C.c_float), ("lengthU", C.c_float),
        ("forceU", C.c_float), ("massU", C.c_float),
        ("mu_r", C.c_float), ("theta_0", C.c_float), ("mu_theta", C.c_float), ("mu_p", C.c_float),
        ("z_0", C.c_float), ("stepThermostat", C.c_int), ("gammaBerendsen", C.c_float), ("stepCool", C.c_int),
        ("iRegime", C.c_int), ("sigmaLJ", C.c_float), ("epsLJ", C.c_float), ("rCutLJ", C.c_float),
        ("rrCutLJ", C.c_float), ("velMagDepos", C.c_float), ("randSeedP", C.c_int), ("stepDeposit", C.c_int),
        ("nMolDeposited", C.c_int), ("nMolToDeposit", C.c_int),
        ("centerOfMass", Prop), ("cmVel", Prop), ("frictForce", Prop), ("deltaF", C.c_float),
        ("particleSize", Float3), ("cellShiftZ", C.c_int), ("shear", C.c_float), ("totalShear", C.c_float),
        ("initUcellMeX", C.c_int), ("initUcellMeY", C.c_int),
        ("rangeRdf", C.c_float), ("limitRdf", C.c_int), ("sizeHistRdf", C.c_int), ("stepRdf", C.c_int),
        ("countRdf", C.c_int), ("intervalRdf", C.c_float), ("bRdf", C.c_int), ("szRdfPath", C.c_char * MAX_PATH),
        ("szBckup0", C.c_char * 20), ("szBckup1", C.c_char * 20), ("bBckup", C.c_int), ("bStartBckup", C.c_int),
        ("stepBckup", C.c_int), ("totalTime", C.c_float), ("iMaterial", C.c_int),
        ("nValDiffuse", C.c_int), ("nBuffDiffuse", C.c_int), ("stepDiffuse", C.c_int),
        ("limitDiffuseAv", C.c_int), ("countDiffuseAv", C.c_int), ("szDiffusePath", C.c_char * MAX_PATH),
    ]

    def copy(self) -> "SimParams":
        q = SimParams()
        C.memmove(C.byref(q), C.byref(self), C.sizeof(SimParams))
        return q


assert C.sizeof(SimParams) == 1112, C.sizeof(SimParams)


class Options(C.Structure):
    _fields_ = [
        ("mode", C.c_int), ("force_rebuild", C.c_int), ("use_graphs", C.c_int), ("device", C.c_int),
        ("stream", C.c_void_p), ("rdf_ext_bins", C.c_int), ("rdf_ext_range", C.c_float),
        ("eam_table_knots", C.c_int), ("metal_lanes", C.c_int), ("nebr_blocks_per_sm", C.c_int),
        ("phase_timing", C.c_int),
        ("programmatic_launch", C.c_int), ("nebr_descending", C.c_int), ("nebr_item_atoms", C.c_int),
        ("nebr_build", C.c_int), ("eam_table_smem", C.c_int), ("carbon_blocks_per_sm", C.c_int),
        ("persistent_step", C.c_int), ("persistent_wait_us", C.c_int), ("nebr_capacity", C.c_int),
    ]


class LaunchShape(C.Structure):
    _fields_ = [("metal_lanes", C.c_int), ("nebr_blocks_per_sm", C.c_int), ("nebr_descending", C.c_int),
                ("nebr_item_atoms", C.c_int), ("programmatic_launch", C.c_int), ("nebr_build", C.c_int),
                ("eam_table_smem", C.c_int), ("carbon_blocks_per_sm", C.c_int)]


class Thermo(C.Structure):
    _fields_ = [
        ("stepCount", C.c_int), ("nebrNow", C.c_int), ("rebuilds", C.c_int), ("countRdf", C.c_int),
        ("kinEnergy", C.c_float), ("potEnergy", C.c_float), ("totEnergy", C.c_float),
        ("vvSum", C.c_float), ("vvMax", C.c_float), ("uSum", C.c_float), ("dispHi", C.c_float),
        ("vSum", Float3), ("centerOfMass", Float3), ("cmVel", Float3), ("frictForce", C.c_float),
        ("particleSize", Float3), ("shear", C.c_float), ("totalShear", C.c_float),
        ("kinEnergy64", C.c_double), ("potEnergy64", C.c_double), ("virial64", C.c_double),
        ("props", Prop * 7),
    ]


class Diag(C.Structure):
    _fields_ = [
        ("max_neighbours", C.c_int), ("max_cell_occupancy", C.c_int), ("nebr_overflow", C.c_int),
        ("cell_range", C.c_int), ("cell_overflow", C.c_int), ("rdf_range", C.c_int), ("timeouts", C.c_int),
        ("reserved", C.c_int * 9),
    ]


class Input(C.Structure):
    _fields_ = [
        ("iRegime", C.c_int), ("iMaterial", C.c_int), ("ucx", C.c_int), ("ucy", C.c_int), ("ucz", C.c_int),
        ("temperatureK", C.c_float), ("nMolMe", C.c_int), ("epsilonEv", C.c_float), ("sigmaA", C.c_float),
        ("stepLimit", C.c_int), ("deltaT", C.c_float), ("stepAvg", C.c_int), ("stepEquil", C.c_int),
        ("deltaFpN", C.c_float), ("stepCool", C.c_int), ("deposEnergyEv", C.c_float),
        ("nMolToDeposit", C.c_int), ("stepDeposit", C.c_int), ("stepPdb", C.c_int), ("stepRdf", C.c_int),
        ("bBckup", C.c_int), ("bStartBckup", C.c_int),
        ("rNebrShell", C.c_float), ("iNebrMax", C.c_int), ("stepThermostat", C.c_int),
        ("gammaBerendsen", C.c_float), ("limitRdf", C.c_int), ("sizeHistRdf", C.c_int),
        ("nValDiffuse", C.c_int), ("nBuffDiffuse", C.c_int), ("stepDiffuse", C.c_int),
        ("limitDiffuseAv", C.c_int), ("stepBckup", C.c_int), ("randSeed", C.c_int),
        ("bPdb", C.c_int), ("bResult", C.c_int), ("bRdf", C.c_int),
    ]


class Workload(C.Structure):
    _fields_ = [
        ("ucx", C.c_int), ("ucy", C.c_int), ("iMaterial", C.c_int), ("n_clusters", C.c_int),
        ("cluster_sizes", c_int_p), ("temperatureK", C.c_float), ("clearance_A", C.c_float),
        ("seed", C.c_ulonglong), ("stepLimit", C.c_int), ("stepAvg", C.c_int), ("stepEquil", C.c_int),
        ("stepCool", C.c_int), ("stepRdf", C.c_int), ("limitRdf", C.c_int), ("stepDiffuse", C.c_int),
        ("nValDiffuse", C.c_int), ("nBuffDiffuse", C.c_int), ("limitDiffuseAv", C.c_int),
        ("deltaT", C.c_float),
    ]


SG_OK = 0
STATUS = {
    1: "SG_ERR_INVALID", 2: "SG_ERR_CUDA", 3: "SG_ERR_NOMEM", 4: "SG_ERR_NO_DEVICE",
    5: "SG_ERR_NEBR_OVERFLOW", 6: "SG_ERR_CELL_RANGE", 7: "SG_ERR_RDF_RANGE", 8: "SG_ERR_TIMEOUT",
    9: "SG_ERR_IO", 10: "SG_ERR_UNSUPPORTED", 11: "SG_ERR_CELL_OVERFLOW", 12: "SG_ERR_BAD_FILE",
}
MODE_PLAIN, MODE_MIXED = 0, 1


class SgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None

# name -> (restype, argtypes) of every exported function the Python layer uses
_SIGS = {
    "sg_version": (C.c_int, []),
    "sg_last_error": (C.c_char_p, []),
    "sg_default_options": (None, [C.POINTER(Options)]),
    "sg_create": (C.c_int, [C.POINTER(SimParams), C.c_int, C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "sg_destroy": (C.c_int, [C.c_void_p]),
    "sg_num_replicas": (C.c_int, [C.c_void_p]),
    "sg_num_atoms": (C.c_int, [C.c_void_p, C.c_int]),
    "sg_num_cells": (C.c_int, [C.c_void_p, C.c_int]),
    "sg_set_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_get_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_get_params": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(SimParams)]),
    "sg_step": (C.c_int, [C.c_void_p, C.c_int]),
    "sg_step_async": (C.c_int, [C.c_void_p, C.c_int]),
    "sg_kernels_per_step": (C.c_int, [C.c_void_p]),
    "sg_get_phase_times": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "sg_get_thermo": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Thermo)]),
    "sg_build_lists": (C.c_int, [C.c_void_p]),
    "sg_compute_forces": (C.c_int, [C.c_void_p]),
    "sg_eval_rdf": (C.c_int, [C.c_void_p]),
    "sg_reset_rdf": (C.c_int, [C.c_void_p]),
    "sg_get_cells": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_get_nebr": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "sg_get_carbon_lists": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_get_rho": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "sg_get_friction": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "sg_get_rdf": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "sg_get_rdf_ext": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "sg_get_diffusion": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_get_diag": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(Diag)]),
    "sg_run": (C.c_int, [C.c_void_p, C.c_void_p, C.c_char_p]),
    "sg_default_input": (None, [C.POINTER(Input)]),
    "sg_read_input_file": (C.c_int, [C.c_char_p, C.POINTER(Input)]),
    "sg_set_params": (C.c_int, [C.POINTER(Input), C.POINTER(SimParams)]),
    "sg_init_coords": (C.c_int, [C.POINTER(SimParams), C.c_void_p]),
    "sg_init_vels": (C.c_int, [C.POINTER(SimParams), C.c_void_p]),
    "sg_build_workload": (C.c_int, [C.POINTER(Workload), C.POINTER(SimParams), C.c_void_p, C.c_void_p]),
    "sg_accum_props": (None, [C.POINTER(SimParams), C.c_int]),
    "sg_print_summary": (C.c_int, [C.c_void_p, C.POINTER(SimParams)]),
    "sg_result_file_name": (C.c_int, [C.POINTER(SimParams), C.c_char_p, C.c_int]),
    "sg_print_result_header": (C.c_int, [C.c_void_p, C.POINTER(SimParams), C.c_float]),
    "sg_create_pdb": (C.c_int, [C.c_char_p, C.POINTER(SimParams), C.c_void_p]),
    "sg_print_rdf": (C.c_int, [C.POINTER(SimParams), C.c_void_p]),
    "sg_print_diffusion": (C.c_int, [C.c_void_p, C.POINTER(SimParams), C.c_void_p]),
    "sg_write_backup": (C.c_int, [C.c_char_p, C.POINTER(SimParams), C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_read_backup": (C.c_int, [C.c_char_p, C.POINTER(SimParams), C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_compute_forces_noalloc": (C.c_int, [C.POINTER(SimParams), C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_autotune": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_int]),
    "sg_step_thermo": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "sg_step_from_host": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                    C.c_void_p]),
    "sg_step_readback_bytes": (C.c_longlong, [C.c_void_p]),
    "sg_get_launch_shape": (C.c_int, [C.c_void_p, C.POINTER(LaunchShape)]),
    "sg_set_launch_shape": (C.c_int, [C.c_void_p, C.POINTER(LaunchShape)]),
    "sg_diff_frame_params": (C.c_int, [C.POINTER(SimParams), C.POINTER(SimParams)]),
    "sg_diff_create": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "sg_diff_destroy": (C.c_int, [C.c_void_p]),
    "sg_diff_num_atoms": (C.c_int, [C.c_void_p]),
    "sg_diff_set_positions": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sg_diff_init_theta": (C.c_int, [C.POINTER(SimParams), C.c_void_p]),
    "sg_diff_energy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_diff_forces": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_diff_force_matching": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sg_load_diff_theta": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "CudaInitW": (None, [C.c_int, C.c_void_p]),
    "SetParametersW": (None, [C.POINTER(SimParams)]),
    "InitCoordsW": (C.c_char_p, [C.c_void_p, C.c_void_p, C.POINTER(SimParams)]),
    "DoComputationsW": (C.c_char_p, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(SimParams), C.c_void_p,
                                     C.c_char_p]),
}


def lib() -> C.CDLL:
    """The loaded libsgmd.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIBPATH.exists():
            raise RuntimeError(f"{LIBPATH} is missing: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIBPATH), mode=os.RTLD_NOW | C.RTLD_GLOBAL)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != SG_OK:
        raise SgError(code, lib().sg_last_error().decode(errors="replace"))


def libc() -> C.CDLL:
    L = C.CDLL(None)
    L.fopen.restype = C.c_void_p
    L.fopen.argtypes = [C.c_char_p, C.c_char_p]
    L.fclose.argtypes = [C.c_void_p]
    L.fflush.argtypes = [C.c_void_p]
    return L
