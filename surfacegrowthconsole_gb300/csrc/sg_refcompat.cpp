// sg_refcompat.cpp - the reference's wrapper ABI (SurfaceGrowthConsole/SurfaceGrowth.h:217-235)
// implemented on top of the sg_* API, so that the reference's host program (SurfaceGrowth.cpp)
// links against libsgmd.so unchanged.  Failures never exit the process: a failure of
// CudaInitW/SetParametersW is remembered and returned by DoComputationsW through its error
// string, the way the reference reports its other errors.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sg_api.h"
#include "sg_refcompat.h"

static std::string g_pending;  // deferred failure of CudaInitW / SetParametersW

// SurfaceGrowth.cu:2614-2637
extern "C" void CudaInitW(int, char **) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    printf("cudaGetDeviceCount returned %d\n-> %s\n", (int)e, cudaGetErrorString(e));
    g_pending = std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e);
    return;
  }
  if (n == 0) printf("There are no available device(s) that support CUDA\n");
  else printf("Detected %d CUDA Capable device(s)\n", n);
  if (n > 0) cudaSetDevice(0);
}

// SurfaceGrowth.cu:2639-2650.  The parameters travel with every later call, so nothing is
// copied to the device here; the block is only checked.
extern "C" void SetParametersW(sg_simparams *p) {
  if (!p || p->nMol <= 0) g_pending = "SetParametersW: invalid parameter block";
}

// SurfaceGrowth.cu:2532-2609
extern "C" const char *InitCoordsW(sg_float4 *, sg_float4 *hr, sg_simparams *hparams) {
  if (!hr || !hparams) return "InitCoordsW: null argument";
  if (sg_init_coords(hparams, hr) != SG_OK) return "InitCoordsW: invalid lattice parameters";
  return nullptr;
}

static char *fail(char *buf, const char *prefix, const char *msg) {
  std::string s = std::string(prefix) + msg;
  strncpy(buf, s.c_str(), SG_MAX_PATH - 1);
  buf[SG_MAX_PATH - 1] = '\0';
  return buf;
}

// SurfaceGrowth.cu:2013-2529.  On return hr/hv/ha hold the final state and hparams the final
// counters and properties.
extern "C" char *DoComputationsW(sg_float4 *hr, sg_float3 *hv, sg_float3 *ha, sg_simparams *hparams,
                                 FILE *fResults, char *szPdbPath) {
  if (!g_pending.empty()) return fail(szPdbPath, "Problems with CUDA initialisation! Exception: ", g_pending.c_str());
  std::string prefix(szPdbPath ? szPdbPath : "sugr");
  sg_options opt;
  sg_default_options(&opt);
  sg_ctx *ctx = nullptr;
  int rc = sg_create(hparams, 1, &opt, &ctx);
  if (rc) return fail(szPdbPath, "Problems with memory allocation! Exception: ", sg_last_error());
  rc = sg_set_state(ctx, 0, hr, hv, ha);
  if (!rc) rc = sg_run(ctx, fResults, prefix.c_str());
  if (!rc) rc = sg_get_state(ctx, 0, hr, hv, ha);
  if (!rc) {
    sg_simparams q;
    rc = sg_get_params(ctx, 0, &q);
    if (!rc) *hparams = q;
  }
  if (rc) {
    std::string msg = sg_last_error();
    sg_destroy(ctx);
    return fail(szPdbPath, "Problems with computations! Exception: ", msg.c_str());
  }
  sg_destroy(ctx);
  return nullptr;
}

// SurfaceGrowth.cpp also calls one host function of SurfaceGrowth.cu besides the wrappers:
// AccumProps (C++ linkage, SurfaceGrowth.cu:2659-2731; called from SetupJob,
// SurfaceGrowth.cpp:417).  Exported here under the reference's name and signature so that the
// reference's host program links against this library unchanged.
struct SimParams;
void AccumProps(int icode, SimParams *hparams) {
  sg_accum_props(reinterpret_cast<sg_simparams *>(hparams), icode);
}
