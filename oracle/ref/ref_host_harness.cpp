// TEST INFRASTRUCTURE.  C entry surface over the reference's own host code, compiled
// together with SurfaceGrowth.cpp and SurfaceGrowth.cu by oracle/ref/build_ref.sh into
// oracle/_ref/libsgref_host.so.  Used only by tests/golden/make_golden.py to record golden
// outputs of the reference (parameter derivation, RNG, result-file header, summary rows,
// pdb/rdf/diffusion writers).  Each function calls the reference's function of the same
// role; only the bookkeeping around the calls (which the reference does inside
// DoComputationsW, SurfaceGrowth.cu:2439-2445 and 2314-2324) is written here.
#include "SurfaceGrowth.h"

#include <climits>
#include <cstring>
#include <vector>

// Globals and functions defined by SurfaceGrowth.cpp.
extern cudaDeviceProp g_hDeviceProp;
extern SimParams g_hSimParams;
extern float3 *g_hv, *g_ha;
extern TCHAR g_szResult[MAX_PATH];
int ReadInputFile(TCHAR *szInpFile);
int SetParams();
int SetupJob();
real RandR(SimParams *hparams);
void VRand(float3 *p, SimParams *hparams);
void FreeArrays();

// Host functions defined by SurfaceGrowth.cu.
void AccumProps(int icode, SimParams *hparams);
void PrintSummary(FILE *fp, SimParams *hparams);
int CreatePdbFile(char *szFilePath, SimParams *hparams, float4 *r);
void PrintRdf(SimParams *hparams, uint *hHistRdf);
void VRandRfloat4(float4 *p, SimParams *hparams);
void InitDiffusion(TBuf *tBuf, real *rrDiffuseAv, SimParams *hparams);
void EvalDiffusion(TBuf *tBuf, real *rrDiffuseAv, FILE *file, SimParams *hparams, float3 centerOfMass);

static int s_seed = 0;
static std::vector<float3> s_vels, s_accels;

extern "C" {

// Stand-ins for the CUDA wrappers that SurfaceGrowth.cpp calls (renamed at compile time).
void sgref_CudaInitW(int, char **) {}
void sgref_SetParametersW(SimParams *p) {
  if (s_seed != 0) p->randSeedP = s_seed;  // InitRand(0) just seeded from the clock
}
const char *sgref_InitCoordsW(float4 *, float4 *hr, SimParams *p) {
  memset(hr, 0, sizeof(float4) * p->nMol);
  return 0;
}
char *sgref_DoComputationsW(float4 *, float3 *, float3 *, SimParams *, FILE *, TCHAR *) { return 0; }

int sgref_sizeof_simparams(void) { return (int)sizeof(SimParams); }

// ReadInputFile + SetParams + SetupJob in the current directory.  Call once per process
// (the reference keeps its configuration in globals).
int sgref_setup(const char *inpath, int seed, SimParams *after_setparams, SimParams *after_setup,
                char *result_name) {
  s_seed = seed;
  g_hDeviceProp.maxGridSize[0] = INT_MAX;
  if (!ReadInputFile((TCHAR *)inpath)) return -1;
  if (!SetParams()) return -2;
  *after_setparams = g_hSimParams;
  if (!SetupJob()) return -3;
  *after_setup = g_hSimParams;
  s_vels.assign(g_hv, g_hv + g_hSimParams.nMol);
  s_accels.assign(g_ha, g_ha + g_hSimParams.nMol);
  strcpy(result_name, g_szResult);
  FreeArrays();  // also closes the result file holding the header
  return g_hSimParams.nMol;
}
void sgref_get_vels(float3 *out) { memcpy(out, s_vels.data(), s_vels.size() * sizeof(float3)); }
// The accelerations SetupJob hands to DoComputationsW (InitAccels, SurfaceGrowth.cpp:622-630).
void sgref_get_accels(float3 *out) { memcpy(out, s_accels.data(), s_accels.size() * sizeof(float3)); }

// RandR / VRand / VRandRfloat4 streams from a seed.
void sgref_rand(int seed, int n, float *out) {
  SimParams p;
  memset(&p, 0, sizeof(p));
  p.randSeedP = seed;
  for (int i = 0; i < n; i++) out[i] = RandR(&p);
}
void sgref_vrand(int seed, int n, float3 *out, int as_float4) {
  SimParams p;
  memset(&p, 0, sizeof(p));
  p.randSeedP = seed;
  for (int i = 0; i < n; i++) {
    if (as_float4) {
      float4 q;
      VRandRfloat4(&q, &p);
      out[i] = make_float3(q.x, q.y, q.z);
    } else {
      VRand(&out[i], &p);
    }
  }
}

// Drive AccumProps/PrintSummary as the step loop does, from per-step values:
// vals[16*s + ...] = totE, potE, kinE, oneStep, cm, cmVel, frict, vSum.x/y/z,
// size.x/y/z, totalShear, (unused), (unused).
int sgref_summary_seq(SimParams *p, int nsteps, const float *vals, const char *path, float totalTime) {
  FILE *f = fopen(path, "a");
  if (!f) return -1;
  AccumProps(0, p);
  for (int s = 0; s < nsteps; s++) {
    const float *v = vals + 16 * s;
    p->stepCount = s + 1;
    p->totEnergy.val = v[0];
    p->potEnergy.val = v[1];
    p->kinEnergy.val = v[2];
    p->oneStep.val = v[3];
    p->centerOfMass.val = v[4];
    p->cmVel.val = v[5];
    p->frictForce.val = v[6];
    p->vSum = make_float3(v[7], v[8], v[9]);
    p->particleSize = make_float3(v[10], v[11], v[12]);
    p->totalShear = v[13];
    AccumProps(1, p);
    if (p->stepCount % p->stepAvg == 0) {
      AccumProps(2, p);
      PrintSummary(f, p);
      AccumProps(0, p);
    }
  }
  fprintf(f, "\nDuration of the simulation = %f s", totalTime);
  fclose(f);
  return 0;
}

int sgref_pdb(const char *prefix, SimParams *p, float4 *r) {
  char buf[MAX_PATH];
  strcpy(buf, prefix);
  return CreatePdbFile(buf, p, r);
}

void sgref_rdf(SimParams *p, unsigned int *hist) { PrintRdf(p, hist); }

// EvalDiffusion over a sequence of centre-of-mass samples, output to path.
int sgref_diffusion_seq(SimParams *p, int n, const float *cm3, const char *path) {
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  std::vector<TBuf> tb(p->nBuffDiffuse);
  std::vector<std::vector<real>> store(p->nBuffDiffuse, std::vector<real>(p->nValDiffuse));
  std::vector<real> av(p->nValDiffuse);
  for (int b = 0; b < p->nBuffDiffuse; b++) tb[b].rrDiffuse = store[b].data();
  InitDiffusion(tb.data(), av.data(), p);
  for (int i = 0; i < n; i++)
    EvalDiffusion(tb.data(), av.data(), f, p, make_float3(cm3[3 * i], cm3[3 * i + 1], cm3[3 * i + 2]));
  fclose(f);
  return 0;
}

}  // extern "C"
