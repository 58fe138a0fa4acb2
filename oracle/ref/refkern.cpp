// TEST INFRASTRUCTURE.  Runs the reference's own CUDA kernels (SurfaceGrowthConsole/
// SurfaceGrowth.cu, device code compiled unmodified into a cubin by oracle/ref/build_ref.sh)
// on states injected from Python, through the CUDA driver API.  Nothing of the reference is
// copied: the cubin is built from the read-only reference tree, and this file only loads it,
// allocates the reference's arrays (SurfaceGrowth.cu:2059-2102) and launches its kernels with
// the launch shapes of DoComputationsW (SurfaceGrowth.cu:2141-2430).
//
// Uses: pinning the oracle and the project's kernels against the reference's arithmetic on the
// GPU (tests/test_ref_kernels_gpu.py, tests/golden/make_ref_kernel_golden.py), and timing
// "the reference GPU path as shipped" (rk_run_steps restates the step loop's sequence of
// launches and blocking copies, SurfaceGrowth.cu:2141-2430, without its file output).
//
// The reference kernels check no bounds: a cell above blockSize atoms or an atom above
// iNebrMax neighbours writes past CELL / NBL.  The Python wrapper (oracle/refkern.py) checks
// both on the CPU oracle before any launch; rk_bin and rk_build_nebr repeat the check on what
// the kernels produced and report it.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sg_simparams.h"

namespace {

struct Fn {
  const char *name;  // length-prefixed name as it appears in the mangled symbol
  CUfunction f;
};

Fn g_fn[] = {
    {"13LeapfrogStepK", nullptr},          {"18ApplyBoundaryCondK", nullptr},
    {"18BinAtomsIntoCellsK", nullptr},     {"14BuildNebrListK", nullptr},
    {"14EamComputeRhoK", nullptr},         {"14ComputeForcesK", nullptr},
    {"12ComputeVSumK", nullptr},           {"13ComputeVvMaxK", nullptr},
    {"13ComputeVvSumK", nullptr},          {"17ComputePotEnergyK", nullptr},
    {"20ComputeCenterOfMassK", nullptr},   {"13ComputeCmVelK", nullptr},
    {"20ComputeParticleSizeK", nullptr},   {"16ComputeNetForceK", nullptr},
    {"24ApplyBerendsenThermostat", nullptr}, {"11ApplyShearK", nullptr},
    {"8EvalRdfK", nullptr},                {"12InsertAtomsK", nullptr},
    {"14InitFccCoordsK", nullptr},         {"15InitSlabCoordsK", nullptr},
    {"19InitGrapheneCoordsK", nullptr},
};
enum {
  F_LEAP, F_BOUND, F_BIN, F_NEBR, F_RHO, F_FORCES, F_VSUM, F_VVMAX, F_VVSUM, F_POT, F_CM, F_CMVEL,
  F_SIZE, F_NET, F_THERMO, F_SHEAR, F_RDF, F_INSERT, F_INIT_FCC, F_INIT_SLAB, F_INIT_GRAPHENE, F_COUNT
};

CUcontext g_ctx = nullptr;
CUmodule g_mod = nullptr;
CUdeviceptr g_dparams = 0;
sg_simparams g_p;
CUdeviceptr dr = 0, dv = 0, da = 0, hlp = 0, rho = 0, CELL = 0, NN = 0, NBL = 0, mic = 0, fric = 0, hist = 0;
unsigned g_grid = 0;  // reduction blocks: ceil(nMol / 1024)
std::string g_err;

int fail(CUresult r, const char *what) {
  const char *s = nullptr;
  cuGetErrorString(r, &s);
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, s ? s : "?");
  g_err = buf;
  return (int)r;
}
#define CU(call)                                   \
  do {                                             \
    CUresult r_ = (call);                          \
    if (r_ != CUDA_SUCCESS) return fail(r_, #call); \
  } while (0)

void freeAll() {
  CUdeviceptr *ps[] = {&dr, &dv, &da, &hlp, &rho, &CELL, &NN, &NBL, &mic, &fric, &hist};
  for (CUdeviceptr *p : ps)
    if (*p) {
      cuMemFree(*p);
      *p = 0;
    }
}

int launch(int which, unsigned grid, unsigned block, unsigned smem, void **args) {
  CU(cuLaunchKernel(g_fn[which].f, grid, 1, 1, block, 1, 1, smem, nullptr, args, nullptr));
  return 0;
}
// one block per cell x blockSize threads: the reference's dimGrid / dimBlock
int launchCells(int which, void **args) { return launch(which, g_p.gridSize, g_p.blockSize, 0, args); }
// reductions: ceil(nMol / 1024) blocks of 512 threads, 2 * 512 float3 of shared memory
int launchRed(int which, void **args) { return launch(which, g_grid, 512, 2 * 512 * 12, args); }

}  // namespace

extern "C" {

const char *rk_last_error(void) { return g_err.c_str(); }

// Load the cubin into the primary context of device 0 and resolve the kernels by name.
int rk_open(const char *cubin) {
  CU(cuInit(0));
  CUdevice dev;
  CU(cuDeviceGet(&dev, 0));
  CU(cuDevicePrimaryCtxRetain(&g_ctx, dev));
  CU(cuCtxSetCurrent(g_ctx));
  CU(cuModuleLoad(&g_mod, cubin));
  unsigned n = 0;
  CU(cuModuleGetFunctionCount(&n, g_mod));
  std::vector<CUfunction> fs(n);
  CU(cuModuleEnumerateFunctions(fs.data(), n, g_mod));
  for (CUfunction f : fs) {
    const char *name = nullptr;
    CU(cuFuncGetName(&name, f));
    for (Fn &k : g_fn)
      if (name && strncmp(name, "_Z", 2) == 0 && strncmp(name + 2, k.name, strlen(k.name)) == 0) k.f = f;
  }
  for (Fn &k : g_fn)
    if (!k.f) {
      g_err = std::string("kernel not found in the cubin: ") + k.name;
      return -1;
    }
  size_t bytes = 0;
  CU(cuModuleGetGlobal(&g_dparams, &bytes, g_mod, "dparams"));
  if (bytes != sizeof(sg_simparams)) {
    g_err = "dparams size differs from sg_simparams";
    return -1;
  }
  return 0;
}

int rk_close(void) {
  freeAll();
  if (g_mod) cuModuleUnload(g_mod);
  g_mod = nullptr;
  return 0;
}

// Copy the parameters into the reference's constant block and size its arrays
// (SurfaceGrowth.cu:2059-2102).
int rk_setup(const sg_simparams *p) {
  freeAll();
  g_p = *p;
  CU(cuMemcpyHtoD(g_dparams, p, sizeof(sg_simparams)));
  const size_t N = (size_t)p->nMol, ncells = (size_t)p->cells.x * p->cells.y * p->cells.z;
  g_grid = (unsigned)((p->nMol + 1023) / 1024);
  CU(cuMemAlloc(&dr, N * 16));
  CU(cuMemAlloc(&dv, N * 12));
  CU(cuMemAlloc(&da, N * 12));
  CU(cuMemAlloc(&hlp, std::max<size_t>(g_grid, 1) * 12));
  CU(cuMemAlloc(&rho, std::max<size_t>(p->nMolMe, 1) * 4));
  CU(cuMemAlloc(&CELL, ((size_t)p->maxMol + 1) * 4));
  CU(cuMemAlloc(&NN, N * 4));
  CU(cuMemAlloc(&NBL, N * p->iNebrMax * 4));
  CU(cuMemAlloc(&mic, ncells * 4));
  if (p->iRegime != 0 && p->nMolMe != 0) CU(cuMemAlloc(&fric, (size_t)p->nMolMe * 4));
  if (p->bRdf) {
    // one spare element: EvalRdfK adds a pair whose bin index rounds up to sizeHistRdf one
    // element past the histogram (SurfaceGrowth.cu:1988-1989)
    CU(cuMemAlloc(&hist, ((size_t)p->sizeHistRdf + 1) * 4));
    CU(cuMemsetD32(hist, 0, p->sizeHistRdf + 1));
  }
  return 0;
}

int rk_set_state(const float *r4, const float *v3, const float *a3) {
  const size_t N = g_p.nMol;
  CU(cuMemcpyHtoD(dr, r4, N * 16));
  if (v3) CU(cuMemcpyHtoD(dv, v3, N * 12));
  if (a3) CU(cuMemcpyHtoD(da, a3, N * 12));
  return 0;
}
int rk_get_state(float *r4, float *v3, float *a3) {
  const size_t N = g_p.nMol;
  CU(cuCtxSynchronize());
  if (r4) CU(cuMemcpyDtoH(r4, dr, N * 16));
  if (v3) CU(cuMemcpyDtoH(v3, dv, N * 12));
  if (a3) CU(cuMemcpyDtoH(a3, da, N * 12));
  return 0;
}

// Cell binning as the step loop does it when nebrNow is set (SurfaceGrowth.cu:2210-2222).
// Returns the largest cell occupancy seen.
int rk_bin(int *maxOcc) {
  const size_t N = g_p.nMol, ncells = (size_t)g_p.cells.x * g_p.cells.y * g_p.cells.z;
  CU(cuMemsetD32(CELL, 0xffffffffu, (size_t)g_p.maxMol + 1));
  CU(cuMemsetD32(NN, 0, N));
  CU(cuMemsetD32(NBL, 0xffffffffu, N * g_p.iNebrMax));
  CU(cuMemsetD32(mic, 0, ncells));
  void *args[] = {&dr, &CELL, &mic};
  if (int rc = launchCells(F_BIN, args)) return rc;
  std::vector<unsigned> m(ncells);
  CU(cuMemcpyDtoH(m.data(), mic, ncells * 4));
  *maxOcc = (int)*std::max_element(m.begin(), m.end());
  return 0;
}
int rk_get_cells(int *cell, unsigned *molsInCells) {
  const size_t ncells = (size_t)g_p.cells.x * g_p.cells.y * g_p.cells.z;
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(cell, CELL, ((size_t)g_p.maxMol + 1) * 4));
  CU(cuMemcpyDtoH(molsInCells, mic, ncells * 4));
  return 0;
}
int rk_set_cells(const int *cell) {
  CU(cuMemcpyHtoD(CELL, cell, ((size_t)g_p.maxMol + 1) * 4));
  return 0;
}
// BuildNebrListK over the current CELL (SurfaceGrowth.cu:2224); returns the largest NN.
int rk_build_nebr(int *maxNN) {
  const size_t N = g_p.nMol;
  CU(cuMemsetD32(NN, 0, N));
  CU(cuMemsetD32(NBL, 0xffffffffu, N * g_p.iNebrMax));
  void *args[] = {&dr, &CELL, &NN, &NBL};
  if (int rc = launchCells(F_NEBR, args)) return rc;
  std::vector<int> nn(N);
  CU(cuMemcpyDtoH(nn.data(), NN, N * 4));
  *maxNN = N ? *std::max_element(nn.begin(), nn.end()) : 0;
  return 0;
}
int rk_get_nebr(int *nn, int *nbl) {
  const size_t N = g_p.nMol;
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(nn, NN, N * 4));
  CU(cuMemcpyDtoH(nbl, NBL, N * g_p.iNebrMax * 4));
  return 0;
}
int rk_set_nebr(const int *nn, const int *nbl) {
  const size_t N = g_p.nMol;
  CU(cuMemcpyHtoD(NN, nn, N * 4));
  CU(cuMemcpyHtoD(NBL, nbl, N * g_p.iNebrMax * 4));
  return 0;
}

// Density and forces (SurfaceGrowth.cu:2234-2238).
int rk_forces(void) {
  if (g_p.nMolMe != 0) {
    void *a1[] = {&rho, &dr, &NN, &NBL};
    if (int rc = launchCells(F_RHO, a1)) return rc;
  }
  void *a2[] = {&da, &dr, &NN, &NBL, &rho, &fric};
  return launchCells(F_FORCES, a2);
}
int rk_get_rho(float *out) {
  CU(cuCtxSynchronize());
  if (g_p.nMolMe) CU(cuMemcpyDtoH(out, rho, (size_t)g_p.nMolMe * 4));
  return 0;
}
int rk_get_friction(float *out) {
  CU(cuCtxSynchronize());
  if (fric) CU(cuMemcpyDtoH(out, fric, (size_t)g_p.nMolMe * 4));
  return 0;
}
// ComputeNetForceK: sums the friction array in place; out = element 0 (SurfaceGrowth.cu:2248-2256).
int rk_net_force(float *out) {
  if (!fric) {
    *out = 0.f;
    return 0;
  }
  void *args[] = {&fric};
  if (int rc = launchRed(F_NET, args)) return rc;
  CU(cuMemcpyDtoH(out, fric, 4));
  return 0;
}

int rk_leapfrog(int part) {
  void *args[] = {&part, &dr, &dv, &da};
  return launchCells(F_LEAP, args);
}
int rk_boundary(void) {
  void *args[] = {&dr};
  return launchCells(F_BOUND, args);
}

// One reduction kernel; out = hlpArray[0] (float3).  which: 0 VSum, 1 VvMax, 2 VvSum (cmVelX),
// 3 PotEnergy, 4 CenterOfMass, 5 CmVel, 6 ParticleSize min, 7 ParticleSize max.
int rk_reduce(int which, float cmVelX, float *out3) {
  int rc = 0;
  int mm = (which == 7) ? 1 : 0;
  switch (which) {
    case 0: { void *a[] = {&dv, &hlp}; rc = launchRed(F_VSUM, a); break; }
    case 1: { void *a[] = {&dv, &hlp}; rc = launchRed(F_VVMAX, a); break; }
    case 2: { void *a[] = {&dv, &hlp, &cmVelX}; rc = launchRed(F_VVSUM, a); break; }
    case 3: { void *a[] = {&dr, &hlp}; rc = launchRed(F_POT, a); break; }
    case 4: { void *a[] = {&dr, &hlp}; rc = launchRed(F_CM, a); break; }
    case 5: { void *a[] = {&dv, &hlp}; rc = launchRed(F_CMVEL, a); break; }
    case 6:
    case 7: { void *a[] = {&dr, &hlp, &mm}; rc = launchRed(F_SIZE, a); break; }
    default: g_err = "bad reduction"; return -1;
  }
  if (rc) return rc;
  CU(cuMemcpyDtoH(out3, hlp, 12));
  return 0;
}

// ApplyBerendsenThermostat with vvSum read from hlpArray[0].x, as the step loop passes it
// after ComputeVvSumK (SurfaceGrowth.cu:2350-2360).
int rk_thermostat(int stepCount) {
  CUdeviceptr vv = hlp;
  void *args[] = {&dv, &vv, &stepCount};
  return launchCells(F_THERMO, args);
}

// ApplyShearK alone on the current state (SurfaceGrowth.cu:517-534), with the step loop's
// launch shape and counter (the first word of molsInCells, zeroed first, cu:2405-2411).
// Writes the number of metal atoms the shear was added to.
int rk_shear(float shear, float centerOfMassX, unsigned *count) {
  CU(cuMemsetD32(mic, 0, 1));
  CUdeviceptr cnt = mic;
  void *args[] = {&dr, &da, &shear, &centerOfMassX, &cnt};
  if (int rc = launchCells(F_SHEAR, args)) return rc;
  CU(cuMemcpyDtoH(count, mic, 4));
  return 0;
}

// The step loop's host-side scalars after rk_run_steps (stepCount, nebrNow, dispHi, shear,
// totalShear, countRdf as DoComputationsW keeps them in hparams).
int rk_get_params(sg_simparams *out) {
  *out = g_p;
  return 0;
}

// The device half of InitCoordsW (SurfaceGrowth.cu:2532-2609) with the reference's own lattice
// kernels and launch shapes: InitFccCoordsK for regime 0, InitGrapheneCoordsK for the sheet of
// regimes 1 and 2, and InitSlabCoordsK for the regime-2 metal slab (initUcellMeX/Y and the
// layer count computed as the wrapper does, and written back to *p like the wrapper does).
// The regime-1 metal atoms come from the host generator and are left as zeros here.  Loads
// *p into the constant block; needs no rk_setup.  The shapes are checked against the CUDA
// launch limits and the kernels' writes against the nMol-entry array before any launch.
int rk_init_coords(sg_simparams *p, float *hr) {
  const size_t N = (size_t)p->nMol;
  if (p->nMol <= 0 || p->nMolMe < 0 || p->nMolMe > p->nMol) {
    g_err = "rk_init_coords: bad atom counts";
    return -1;
  }
  unsigned fcc[3] = {0, 0, 0}, gr = 0, slab[3] = {0, 0, 0};
  if (p->iRegime == 0) {
    fcc[0] = p->initUcell.x; fcc[1] = p->initUcell.y; fcc[2] = p->initUcell.z;
    // InitFccCoordsK writes 4 atoms from n = 4 * (cell index) while n <= nMol - 4
    if ((size_t)4 * fcc[0] * fcc[1] * fcc[2] != N || fcc[2] == 0 || fcc[2] > 64 || fcc[1] > 65535) {
      g_err = "rk_init_coords: fcc shape outside the launch limits or nMol != 4 cells";
      return -1;
    }
  } else if (p->iRegime == 1 || p->iRegime == 2) {
    const int nC = p->nMol - p->nMolMe;
    if (nC % 32 != 0 || nC <= 0) {
      g_err = "rk_init_coords: carbon count not a positive multiple of 32";
      return -1;
    }
    gr = (unsigned)(nC / 32);
    if (p->iRegime == 2 && p->nMolMe != 0) {
      // integer conversions as the wrapper's (cu:2577-2579)
      const int ux = (int)((p->region.x - 2 * p->a) / p->a);
      const int uy = (int)((p->region.y - 2 * p->a) / p->a);
      if (ux <= 0 || uy <= 0) {
        g_err = "rk_init_coords: box too small for the metal slab";
        return -1;
      }
      const int layers = (int)ceil(p->nMolMe * 0.25 / (ux * uy));
      if (layers <= 0 || layers > 64 || uy > 65535) {
        g_err = "rk_init_coords: slab shape outside the launch limits";
        return -1;
      }
      p->initUcellMeX = ux;
      p->initUcellMeY = uy;
      slab[0] = (unsigned)ux; slab[1] = (unsigned)uy; slab[2] = (unsigned)layers;
    }
  } else {
    g_err = "rk_init_coords: unknown regime";
    return -1;
  }
  CU(cuMemcpyHtoD(g_dparams, p, sizeof(sg_simparams)));
  CUdeviceptr d = 0;
  CU(cuMemAlloc(&d, N * 16));
  int rc = 0;
  CUresult e = cuMemsetD32(d, 0, N * 4);
  void *args[] = {&d};
  if (e == CUDA_SUCCESS && p->iRegime == 0)
    e = cuLaunchKernel(g_fn[F_INIT_FCC].f, fcc[0], fcc[1], 1, 1, 1, fcc[2], 0, nullptr, args, nullptr);
  if (e == CUDA_SUCCESS && gr)
    e = cuLaunchKernel(g_fn[F_INIT_GRAPHENE].f, gr, 1, 1, 32, 1, 1, 0, nullptr, args, nullptr);
  if (e == CUDA_SUCCESS && slab[0])
    e = cuLaunchKernel(g_fn[F_INIT_SLAB].f, slab[0], slab[1], 1, 1, 1, slab[2], 0, nullptr, args, nullptr);
  if (e == CUDA_SUCCESS) e = cuCtxSynchronize();
  if (e == CUDA_SUCCESS) e = cuMemcpyDtoH(hr, d, N * 16);
  if (e != CUDA_SUCCESS) rc = fail(e, "rk_init_coords");
  cuMemFree(d);
  // the constant block goes back to the arrays' parameters, if a system is set up
  if (!rc && g_p.nMol > 0) CU(cuMemcpyHtoD(g_dparams, &g_p, sizeof(sg_simparams)));
  return rc;
}

int rk_rdf(int countRdf) {
  void *args[] = {&dr, &CELL, &hist, &countRdf};
  return launchCells(F_RDF, args);
}
int rk_get_rdf(unsigned *out) {
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(out, hist, (size_t)g_p.sizeHistRdf * 4));
  return 0;
}

// The step loop's device work for `steps` steps (SurfaceGrowth.cu:2141-2430): the same kernel
// launches with the same shapes, the same blocking device-to-host copies after every
// reduction, and the host-side rebuild and thermostat decisions.  File output, property
// averaging and diffusion bookkeeping (host work) are left out.  forceRebuild sets nebrNow
// every step.  Writes the elapsed wall time of the loop in ms (CUDA events).
int rk_run_steps(int steps, int forceRebuild, float *ms) {
  sg_simparams &hp = g_p;
  CUevent e0, e1;
  CU(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CU(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  CU(cuEventRecord(e0, nullptr));
  int rc = 0;
  float tmp3[3];
  for (int s = 0; s < steps && !rc; s++) {
    ++hp.stepCount;  // the constant block keeps the values of setup, as in the reference
    if ((rc = rk_leapfrog(1))) break;
    if ((rc = rk_boundary())) break;
    if (hp.nebrNow || forceRebuild) {
      hp.nebrNow = 0;
      hp.dispHi = 0.f;
      const size_t N = hp.nMol, ncells = (size_t)hp.cells.x * hp.cells.y * hp.cells.z;
      CU(cuMemsetD32(CELL, 0xffffffffu, (size_t)hp.maxMol + 1));
      CU(cuMemsetD32(NN, 0, N));
      CU(cuMemsetD32(NBL, 0xffffffffu, N * hp.iNebrMax));
      CU(cuMemsetD32(mic, 0, ncells));
      void *ab[] = {&dr, &CELL, &mic};
      if ((rc = launchCells(F_BIN, ab))) break;
      void *an[] = {&dr, &CELL, &NN, &NBL};
      if ((rc = launchCells(F_NEBR, an))) break;
    }
    if ((rc = rk_forces())) break;
    float frict = 0.f;
    if ((rc = rk_net_force(&frict))) break;
    if ((rc = rk_leapfrog(2))) break;
    float cmVelX = 0.f, cmX = 0.f;
    if (hp.nMolMe != 0) {
      if ((rc = rk_reduce(4, 0.f, tmp3))) break;
      cmX = tmp3[0] / hp.nMolMe;
      if ((rc = rk_reduce(5, 0.f, tmp3))) break;
      cmVelX = tmp3[0] / hp.nMolMe;
      if ((rc = rk_reduce(6, 0.f, tmp3))) break;
      if ((rc = rk_reduce(7, 0.f, tmp3))) break;
    }
    if ((rc = rk_reduce(0, 0.f, tmp3))) break;
    float vvMax[3];
    if ((rc = rk_reduce(1, 0.f, vvMax))) break;
    if ((rc = rk_reduce(2, cmVelX, tmp3))) break;
    if ((hp.iRegime == 2 && hp.stepCount > hp.stepEquil && hp.stepCount % hp.stepThermostat == 0) ||
        (hp.iRegime == 1 && hp.stepCount % hp.stepThermostat == 0))
      if ((rc = rk_thermostat(hp.stepCount))) break;
    if ((rc = rk_reduce(3, 0.f, tmp3))) break;
    hp.dispHi += sqrtf(vvMax[0]) * hp.deltaT;
    if (hp.dispHi > 0.5f * hp.rNebrShell) hp.nebrNow = 1;
    if (hp.iRegime == 2 && hp.nMolMe != 0 && hp.stepCount > hp.stepEquil + hp.stepCool) {
      if (cmVelX < 0.005f) hp.shear += hp.deltaF;
      CU(cuMemsetD32(mic, 0, 1));
      float shear = hp.shear;
      CUdeviceptr cnt = mic;
      void *as[] = {&dr, &da, &shear, &cmX, &cnt};
      if ((rc = launchCells(F_SHEAR, as))) break;
      unsigned nSheared = 0;
      CU(cuMemcpyDtoH(&nSheared, mic, 4));
      hp.totalShear = nSheared * hp.shear;
    }
    if (hp.bRdf != 0 && hp.stepCount % hp.stepRdf == 0) {
      if ((rc = rk_rdf(hp.countRdf))) break;
      if (++hp.countRdf == hp.limitRdf) hp.countRdf = 0;
    }
  }
  CU(cuEventRecord(e1, nullptr));
  CU(cuEventSynchronize(e1));
  CU(cuEventElapsedTime(ms, e0, e1));
  cuEventDestroy(e0);
  cuEventDestroy(e1);
  return rc;
}

}  // extern "C"
