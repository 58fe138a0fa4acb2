// sg_host.cpp - host-side configuration of sgmd: the sugr_in.txt reader, parameter derivation,
// initial lattices and velocities, the synthetic nanoparticle workloads, and the reference's
// text/binary writers.  Compiled with -ffp-contract=off: every float/double expression below
// keeps the types of the reference's expression it restates (SurfaceGrowth.cpp for the
// parameter code, SurfaceGrowth.cu for the lattices and writers), so derived parameters and
// written files come out byte-identical to the reference's on x86 and Arm alike.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "sg_api.h"

namespace {

// Zhou-Wadley-Johnson EAM table of the reference (SurfaceGrowthProto.h:31-80), in its order:
// Cu(0), Ag(1), Au(2), Ni(3), Al(4), Pb(5).  Published material constants.
struct Material {
  const char *name;
  float re, fe, rhoe, alpha, beta, A, B, kappa, lambda, Fn[4], F[4], eta, Fe, massMe, density;
};
const Material kMaterials[6] = {
    {"Cu", 2.556162f, 1.554485f, 22.150141f, 7.669911f, 4.090619f, 0.327584f, 0.468735f, 0.431307f, 0.86214f,
     {-2.176490f, -0.140035f, 0.285621f, -1.750834f}, {-2.19f, 0.f, 0.702991f, 0.683705f}, 0.921150f,
     -2.191675f, 63.54f, 8930.f},
    {"Ag", 2.891814f, 1.106232f, 15.539255f, 7.944536f, 4.237086f, 0.266074f, 0.386272f, 0.425351f, 0.850703f,
     {-1.729619f, -0.221025f, 0.541558f, -0.967036f}, {-1.75f, 0.f, 0.983967f, 0.520904f}, 1.149461f,
     -1.751274f, 107.868f, 10490.f},
    {"Au", 2.885034f, 1.529021f, 21.319637f, 8.086176f, 4.312627f, 0.230728f, 0.336695f, 0.420755f, 0.841511f,
     {-2.930281f, -0.554034f, 1.489437f, -0.886809f}, {-2.98f, 0.f, 2.283863f, 0.494127f}, 1.286960f,
     -2.981365f, 196.9665f, 19302.f},
    {"Ni", 2.488746f, 2.007018f, 27.984706f, 8.029633f, 4.282471f, 0.439664f, 0.632771f, 0.413436f, 0.826873f,
     {-2.693996f, -0.066073f, 0.170482f, -2.457442f}, {-2.70f, 0.f, 0.282257f, 0.102879f}, 0.509860f,
     -2.700493f, 58.71f, 8902.f},
    {"Al", 2.886166f, 1.392302f, 20.226537f, 6.942419f, 3.702623f, 0.251519f, 0.313394f, 0.395132f, 0.790264f,
     {-2.806783f, -0.276173f, 0.893409f, -1.637201f}, {-2.83f, 0.f, 0.929508f, -0.682320f}, 0.779208f,
     -2.829437f, 26.98154f, 2698.9f},
    {"Pb", 3.499723f, 0.647872f, 8.906840f, 8.468412f, 4.516486f, 0.134878f, 0.203093f, 0.425877f, 0.851753f,
     {-1.419644f, -0.228622f, 0.630069f, -0.560952f}, {-1.44f, 0.f, 0.921049f, 0.108847f}, 1.172361f,
     -1.440494f, 207.19f, 11300.f},
};

const float kA0 = 1.42f;  // graphene bond length in A, the unit of length

// Rapaport's generator (SurfaceGrowth.h:38-41, SurfaceGrowth.cpp:573-577); the signed
// overflow of the reference is the wrap-around of this unsigned arithmetic.
float randR(sg_simparams *p) {
  uint32_t s = (uint32_t)p->randSeedP;
  s = (s * 314159269u + 453806245u) & 2147483647u;
  p->randSeedP = (int)s;
  return (float)((double)(int)s * 0.4656612873e-9);
}
// VRand (SurfaceGrowth.cpp:579-593): double literals.
void vRand(sg_float3 *q, sg_simparams *p) {
  float s = 2.f, x = 0.f, y = 0.f;
  while (s > 1.) {
    x = (float)(2. * randR(p) - 1.);
    y = (float)(2. * randR(p) - 1.);
    s = x * x + y * y;
  }
  q->z = (float)(1. - 2. * s);
  s = (float)(2. * sqrt(1. - s));
  q->x = s * x;
  q->y = s * y;
}
// VRandRfloat4 (SurfaceGrowth.cu:2847-2861): float literals.
void vRandF(sg_float4 *q, sg_simparams *p) {
  float s = 2.f, x = 0.f, y = 0.f;
  while (s > 1.f) {
    x = 2.f * randR(p) - 1.f;
    y = 2.f * randR(p) - 1.f;
    s = x * x + y * y;
  }
  q->z = 1.f - 2.f * s;
  s = 2.f * sqrtf(1.f - s);
  q->x = s * x;
  q->y = s * y;
}

}  // namespace

extern "C" void sg_default_input(sg_input *in) {
  // the reference's compiled-in defaults (SurfaceGrowth.cpp:35-90)
  memset(in, 0, sizeof(*in));
  in->iRegime = 2;
  in->iMaterial = 3;
  in->ucx = in->ucy = in->ucz = 7;
  in->temperatureK = 298.f;
  in->nMolMe = 300;
  in->epsilonEv = 0.0087381f;
  in->sigmaA = 2.4945f;
  in->stepLimit = 50000;
  in->deltaT = 0.001f;
  in->stepAvg = 250;
  in->stepEquil = 50000;
  in->deltaFpN = 0.0001f;
  in->stepCool = 5000;
  in->deposEnergyEv = 0.03f;
  in->nMolToDeposit = 40;
  in->stepDeposit = 11000;
  in->stepPdb = 500;
  in->stepRdf = 50;
  in->bBckup = 0;
  in->bStartBckup = 0;
  in->rNebrShell = 0.4f;
  in->iNebrMax = 128;
  in->stepThermostat = 25;
  in->gammaBerendsen = 0.005f;
  in->limitRdf = 100;
  in->sizeHistRdf = 200;
  in->nValDiffuse = 25000;
  in->nBuffDiffuse = 10;
  in->stepDiffuse = 100;
  in->limitDiffuseAv = 20;
  in->stepBckup = 10000;
  in->randSeed = 0;
  in->bPdb = 1;
  in->bResult = 1;
  in->bRdf = 1;
}

// ReadInputFile (SurfaceGrowth.cpp:633-785): newline-terminated lines, leading blanks and '#'
// lines skipped, row k sets value k, the value is the text up to the first space of the line
// as read (so a line with leading blanks yields an empty value, i.e. 0, as in the reference).
// A last line without newline is ignored, as in the reference.
extern "C" int sg_read_input_file(const char *path, sg_input *in) {
  FILE *f = fopen(path, "r");
  if (!f) return SG_ERR_IO;
  std::string line;
  int row = 0;
  int ch;
  while ((ch = fgetc(f)) != EOF) {
    if (ch != '\n') {
      line.push_back((char)ch);
      continue;
    }
    size_t i = 0;
    while (i < line.size() && line[i] == ' ') ++i;
    if (i == line.size() || line[i] == '#') {
      line.clear();
      continue;
    }
    ++row;
    // value: characters up to the first space (end of line also ends it)
    size_t e = line.find(' ');
    std::string tok = line.substr(0, e == std::string::npos ? line.size() : e);
    const char *t = tok.c_str();
    switch (row) {
      case 1: in->iRegime = atoi(t); break;
      case 2: in->iMaterial = atoi(t); break;
      case 3: in->ucx = atoi(t); break;
      case 4: in->ucy = atoi(t); break;
      case 5: in->ucz = atoi(t); break;
      case 6: in->temperatureK = (float)atof(t); break;
      case 7: in->nMolMe = atoi(t); break;
      case 8: in->epsilonEv = (float)atof(t); break;
      case 9: in->sigmaA = (float)atof(t); break;
      case 10: in->stepLimit = atoi(t); break;
      case 11: in->deltaT = (float)atof(t); break;
      case 12: in->stepAvg = atoi(t); break;
      case 13: in->stepEquil = atoi(t); break;
      case 14: in->deltaFpN = (float)atof(t); break;
      case 15: in->stepCool = atoi(t); break;
      case 16: in->deposEnergyEv = (float)atof(t); break;
      case 17: in->nMolToDeposit = atoi(t); break;
      case 18: in->stepDeposit = atoi(t); break;
      case 19: in->stepPdb = atoi(t); break;
      case 20: in->stepRdf = atoi(t); break;
      case 21: in->bBckup = atoi(t); break;
      case 22: in->bStartBckup = atoi(t); break;
      default: break;
    }
    line.clear();
  }
  fclose(f);
  return SG_OK;
}

// SetParams with EamInit and GrapheneInit (SurfaceGrowth.cpp:189-396, 480-545), plus the
// fields SetupJob sets before the run (stepCount 0, nebrNow 1, Props zeroed, Diffuse path).
extern "C" int sg_set_params(const sg_input *in, sg_simparams *out) {
  if (in->iMaterial < 0 || in->iMaterial > 5) return SG_ERR_INVALID;
  if (in->iRegime < 0 || in->iRegime > 2) return SG_ERR_INVALID;
  sg_simparams P;
  memset(&P, 0, sizeof(P));
  sg_simparams *p = &P;
  p->temperatureU = (float)(298 / 0.409246);
  p->enU = 0.06275049f;
  p->kB = 0.99999793f;
  p->lengthU = kA0;
  p->forceU = 14.1239836f;
  p->massU = 12.0107f;
  p->iRegime = in->iRegime;
  p->iMaterial = in->iMaterial;
  const Material &M = kMaterials[in->iMaterial];
  memcpy(p->szNameMe, M.name, 3);
  int ux = in->ucx < 2 ? 2 : in->ucx;
  int uy = in->ucy < 2 ? 2 : in->ucy;
  int uz = in->ucz;
  if (p->iRegime == 0) {
    p->nMolMe = 4 * ux * uy * uz;
    p->nMol = p->nMolMe;
  } else {
    p->nMolMe = in->nMolMe;
    p->nMol = p->nMolMe + 32 * ux * uy;
    uz = 0;
  }
  // EamInit
  p->re = M.re / kA0;
  p->a = (float)(p->re * sqrt(2.));
  p->fe = M.fe;
  p->rhoe = M.rhoe;
  p->alpha = M.alpha;
  p->beta = M.beta;
  p->A = M.A / p->enU;
  p->B = M.B / p->enU;
  p->kappa = M.kappa;
  p->lambda = M.lambda;
  for (int i = 0; i < 4; i++) {
    p->Fn[i] = M.Fn[i] / p->enU;
    p->F[i] = M.F[i] / p->enU;
  }
  p->eta = M.eta;
  p->Fe = M.Fe / p->enU;
  p->massMe = M.massMe / p->massU;
  p->density = (float)(M.density * 0.1435655 * 0.001);
  p->rCutEam = (float)(1.45 * p->a);
  p->rrCutEam = p->rCutEam * p->rCutEam;
  p->rei = 1 / p->re;
  p->rhoei = 1 / p->rhoe;
  // GrapheneInit
  p->mu_r = (float)(41.881 * kA0 * kA0 / p->enU);
  p->theta_0 = (float)(2. * M_PI / 3.);
  p->mu_theta = (float)(2.9959 * kA0 * kA0 / p->enU);
  p->mu_p = (float)(18.225 * kA0 * kA0 / p->enU);
  p->rCutC = 1.2f;
  p->rrCutC = p->rCutC * p->rCutC;
  p->epsLJ = in->epsilonEv / p->enU;
  p->sigmaLJ = in->sigmaA / kA0;
  p->rCutLJ = (float)(2.5 * p->sigmaLJ);
  p->rrCutLJ = p->rCutLJ * p->rCutLJ;
  // region and cells
  const float rNebrShell = in->rNebrShell;
  int cellShiftZ = 4;  // the reference's initial value (used by z_0 in bulk runs)
  sg_float3 region;
  if (p->iRegime == 0) {
    double s = 1. / pow((p->density * 0.25 / p->massMe), 1. / 3.);
    region.x = (float)(s * ux);
    region.y = (float)(s * uy);
    region.z = (float)(s * uz);
  } else {
    region.x = (float)(ux * 8 * cos(M_PI / 6.));
    region.y = (float)(uy * 6);
    const int n = p->nMolMe;
    if (p->iRegime == 1) {
      if (n == 0) cellShiftZ = 0;
      if (n > 0 && n < 100) cellShiftZ = 1;
      if (n >= 100 && n < 5000) cellShiftZ = 2;
      if (n >= 5000 && n < 10000) cellShiftZ = 3;
      if (n >= 10000 && n < 20000) cellShiftZ = 4;
      if (n >= 20000) cellShiftZ = 5;
      if (n != 0)
        region.z = (float)(1.8 * p->a * pow((0.25 * n), 0.33333333333) + p->a +
                           cellShiftZ * (p->rCutEam + rNebrShell));
      else
        region.z = 3 * (p->rCutEam + rNebrShell);
    } else {
      if (n == 0) cellShiftZ = 0;
      if (n > 0 && n < 100) cellShiftZ = 1;
      if (n >= 100 && n < 1000) cellShiftZ = 2;
      if (n >= 1000 && n < 5000) cellShiftZ = 3;
      if (n >= 5000 && n < 10000) cellShiftZ = 5;
      if (n >= 10000 && n < 20000) cellShiftZ = 7;
      if (n >= 20000) cellShiftZ = 9;
      if (n != 0)
        region.z = (float)(p->a * pow((0.25 * n), 0.33333333333) + 3.6 * p->a +
                           cellShiftZ * (p->rCutEam + rNebrShell));
      else
        region.z = 3 * (p->rCutEam + rNebrShell);
    }
  }
  {
    double s = 1.0 / (p->rCutEam + rNebrShell);
    p->cells.x = (int)(s * region.x);
    p->cells.y = (int)(s * region.y);
    p->cells.z = (int)(s * region.z);
  }
  p->initUcell = sg_uint3{(unsigned)ux, (unsigned)uy, (unsigned)uz};
  p->region = region;
  p->invWidth = sg_float3{p->cells.x / p->region.x, p->cells.y / p->region.y, p->cells.z / p->region.z};
  p->cellShiftZ = cellShiftZ;
  p->z_0 = (p->nMolMe != 0) ? -0.5f * p->region.z + p->cellShiftZ / p->invWidth.z : 0.f;
  float T = in->temperatureK <= 0 ? 298.f : in->temperatureK;
  p->temperature = T / p->temperatureU;
  p->stepLimit = in->stepLimit;
  p->stepAvg = in->stepAvg <= 0 ? 1 : in->stepAvg;
  p->stepEquil = in->stepEquil;
  p->stepPdb = in->stepPdb;
  p->moreCycles = 1;
  p->deltaT = in->deltaT;
  p->rNebrShell = rNebrShell;
  p->blockSize = 64;
  p->maxMol = p->cells.x * p->cells.y * p->cells.z * (int)p->blockSize;
  p->gridSize = (unsigned)(p->cells.x * p->cells.y * p->cells.z);
  p->rrNebr = (p->rCutEam + p->rNebrShell) * (p->rCutEam + p->rNebrShell);
  p->iNebrMax = in->iNebrMax;
  p->bPdb = in->bPdb;
  p->bResult = in->bResult;
  p->stepThermostat = in->stepThermostat;
  p->gammaBerendsen = in->gammaBerendsen;
  p->stepCool = (p->iRegime == 1) ? p->stepLimit : in->stepCool;
  p->deltaF = (float)(in->deltaFpN * p->forceU * 0.001);
  p->shear = 0.f;
  p->velMagDepos = sqrtf(2 * in->deposEnergyEv / (p->enU * p->massMe));
  p->stepDeposit = in->stepDeposit;
  p->nMolToDeposit = in->nMolToDeposit;
  p->nMolDeposited = (p->iRegime == 1) ? 0 : p->nMolMe;
  if (p->iRegime == 0)
    p->velMag = (float)sqrt(3 * (1. - 1. / p->nMol) * p->kB * p->temperature / p->massMe);
  else
    p->velMag = (float)sqrt(3 * (1. - 1. / (p->nMol)) * p->kB * p->temperature * p->nMol /
                            (p->nMol - p->nMolMe));
  p->rangeRdf = (float)(1.5 * p->rCutEam);
  p->limitRdf = in->limitRdf;
  p->sizeHistRdf = in->sizeHistRdf;
  p->stepRdf = in->stepRdf;
  p->countRdf = 0;
  p->intervalRdf = p->sizeHistRdf / p->rangeRdf;
  p->bRdf = in->bRdf;
  strcpy(p->szRdfPath, "rdf");
  strcpy(p->szBckup0, "bckup0.sugr");
  strcpy(p->szBckup1, "bckup1.sugr");
  p->bBckup = in->bBckup;
  p->bStartBckup = in->bStartBckup;
  p->stepBckup = in->stepBckup;
  p->totalTime = 0.f;
  p->nValDiffuse = in->nValDiffuse;
  p->nBuffDiffuse = in->nBuffDiffuse;
  p->stepDiffuse = in->stepDiffuse;
  p->limitDiffuseAv = in->limitDiffuseAv;
  p->countDiffuseAv = 0;
  // InitRand: explicit seed, else the clock as in the reference
  p->randSeedP = (in->randSeed != 0) ? in->randSeed : (int)(time(nullptr) % 60) + 1;
  // SetupJob's part
  p->stepCount = 0;
  p->nebrNow = 1;
  if (p->iRegime == 2) strcpy(p->szDiffusePath, "Diffuse.txt");
  *out = P;
  return SG_OK;
}

// ---- initial lattices (kernels of SurfaceGrowth.cu:223-394, run here on the host) ----------
static void fccLattice(const sg_simparams *p, sg_float4 *pos) {
  // InitFccCoordsK: grid(ux, uy) x block(1, 1, uz)
  const int gx = (int)p->initUcell.x, gy = (int)p->initUcell.y, gz = (int)p->initUcell.z;
  const float gapx = p->region.x / p->initUcell.x, gapy = p->region.y / p->initUcell.y,
              gapz = p->region.z / p->initUcell.z;
  for (int nz = 0; nz < gz; nz++)
    for (int ny = 0; ny < gy; ny++)
      for (int nx = 0; nx < gx; nx++) {
        int n = 4 * (nx + ny * gx + nz * gx * gy);
        if (n > p->nMol - 4) continue;
        float cx = nx + 0.25f, cy = ny + 0.25f, cz = nz + 0.25f;
        cx = cx * gapx; cy = cy * gapy; cz = cz * gapz;
        cx = cx + -0.5f * p->region.x; cy = cy + -0.5f * p->region.y; cz = cz + -0.5f * p->region.z;
        for (int j = 0; j < 4; j++) {
          sg_float4 &q = pos[n];
          q = sg_float4{cx, cy, cz, 0.f};
          if (j != 3) {
            if (j != 0) q.x += 0.5f * gapx;
            if (j != 1) q.y += 0.5f * gapy;
            if (j != 2) q.z += 0.5f * gapz;
          }
          n += 1;
        }
      }
}

// InitGrapheneCoordsK: 32 atoms (4 sub-cells of 8) per unit block, carbon atoms after metal.
static void grapheneSheet(const sg_simparams *p, sg_float4 *pos) {
  const float cos30 = 0.8660254038f;
  const int nC = p->nMol - p->nMolMe;
  for (int n = 0; n < nC; n++) {
    const int blk = n / 32, th = n % 32;
    int cy = blk / (int)p->initUcell.x;
    int cx = blk - cy * (int)p->initUcell.x;
    float dx = cx * 8.f * cos30;
    float dy = cy * 6.f;
    cy = (int)(th / 8.f);
    cx = (int)(th - cy * 8.f);
    float x = 0.f, y = 0.f;
    switch (cx) {
      case 0: x = cos30; y = 0.f; break;
      case 1: x = 0.f; y = 0.5f; break;
      case 2: x = 0.f; y = 1.5f; break;
      case 3: x = cos30; y = 2.f; break;
      case 4: x = 2.f * cos30; y = 1.5f; break;
      case 5: x = 2.f * cos30; y = 0.5f; break;
      case 6: x = 3.f * cos30; y = 2.f; break;
      case 7: x = 3.f * cos30; y = 0.f; break;
    }
    if (cy == 1) dx += 4.f * cos30;
    else if (cy == 2) dy += 3.f;
    else if (cy == 3) { dx += 4.f * cos30; dy += 3.f; }
    dx = dx + 0.5f * (cos30 - p->region.x);
    dy = dy + 0.5f * (1.f - p->region.y);
    pos[n + p->nMolMe] = sg_float4{x + dx, y + dy, p->z_0, 0.f};
  }
}

// InitSlabCoordsK with the launch shape chosen by InitCoordsW (cu:2581-2597).
static void slab(sg_simparams *p, sg_float4 *pos) {
  const int ucx = (int)((p->region.x - 2 * p->a) / p->a);
  const int ucy = (int)((p->region.y - 2 * p->a) / p->a);
  const int layers = (int)ceil(p->nMolMe * 0.25 / (ucx * ucy));
  p->initUcellMeX = ucx;
  p->initUcellMeY = ucy;
  const float rx = ucx * p->a, ry = ucy * p->a, rz = p->region.z;
  const float shiftY = (layers == 1) ? 0.5f * (ry - ceilf(0.25f * p->nMolMe / ucx) * p->a) : 0.f;
  const float gap = p->a;
  for (int nz = 0; nz < layers; nz++)
    for (int ny = 0; ny < ucy; ny++)
      for (int nx = 0; nx < ucx; nx++) {
        int n = 4 * (nx + ny * ucx + nz * ucx * ucy);
        float cx = nx + 0.25f, cy = ny + 0.25f, cz = nz + 0.25f;
        cx = cx * gap; cy = cy * gap; cz = cz * gap;
        cx = cx + -0.5f * rx; cy = cy + -0.5f * ry; cz = cz + -0.5f * rz;
        for (int j = 0; j < 4; j++) {
          if (n < p->nMolMe) {
            sg_float4 &q = pos[n];
            q.x = cx;
            q.y = cy + shiftY;
            q.z = cz + 0.5f * p->a + p->cellShiftZ / p->invWidth.z;
            q.w = 0.f;
            if (j != 3) {
              if (j != 0) q.x += 0.5f * gap;
              if (j != 1) q.y += 0.5f * gap;
              if (j != 2) q.z += 0.5f * gap;
            }
            n += 1;
          }
        }
      }
}

extern "C" int sg_init_coords(sg_simparams *p, sg_float4 *r) {
  if (!p || !r) return SG_ERR_INVALID;
  memset(r, 0, sizeof(sg_float4) * p->nMol);
  if (p->iRegime == 0) {
    if (p->initUcell.x == 0 || p->initUcell.y == 0 || p->initUcell.z == 0) return SG_ERR_INVALID;
    fccLattice(p, r);
  } else if (p->iRegime == 1) {
    grapheneSheet(p, r);
    for (int i = 0; i < p->nMolMe; i++) {
      vRandF(&r[i], p);
      r[i].x = 0.5f * p->region.x * r[i].x;
      r[i].y = 0.5f * p->region.y * r[i].y;
      r[i].z = 1.5f * p->region.z + 0.5f * (i + 1) * p->region.z;
      r[i].w = 0.f;
    }
  } else {
    grapheneSheet(p, r);
    if (p->nMolMe != 0) slab(p, r);
  }
  return SG_OK;
}

// InitVels (SurfaceGrowth.cpp:596-621).
extern "C" int sg_init_vels(sg_simparams *p, sg_float3 *v) {
  if (!p || !v) return SG_ERR_INVALID;
  sg_float3 vs{0.f, 0.f, 0.f};
  for (int n = 0; n < p->nMol; n++) {
    if (p->iRegime != 0 && n < p->nMolMe) {
      v[n] = sg_float3{0.f, 0.f, 0.f};
    } else {
      vRand(&v[n], p);
      v[n].x *= p->velMag;
      v[n].y *= p->velMag;
      v[n].z *= p->velMag;
      vs.x = vs.x + v[n].x;
      vs.y = vs.y + v[n].y;
      vs.z = vs.z + v[n].z;
    }
  }
  for (int n = 0; n < p->nMol; n++) {
    if (p->iRegime == 0 || n >= p->nMolMe) {
      v[n].x = (float)(v[n].x + (-1. / (p->nMol)) * vs.x);
      v[n].y = (float)(v[n].y + (-1. / (p->nMol)) * vs.y);
      v[n].z = (float)(v[n].z + (-1. / (p->nMol)) * vs.z);
    }
  }
  return SG_OK;
}

// ---- synthetic nanoparticle-on-graphene workloads -----------------------------------------
namespace {
uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// uniform in (0, 1) from a counter
double uni(uint64_t seed, uint64_t ctr) {
  return ((splitmix64(seed ^ splitmix64(ctr)) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
struct Site { int i, j, k; long long d2; };
}  // namespace

extern "C" int sg_build_workload(const sg_workload *w, sg_simparams *p, sg_float4 *r, sg_float3 *v) {
  if (!w || !p || w->n_clusters < 0 || w->ucx < 2 || w->ucy < 2) return SG_ERR_INVALID;
  int nMe = 0;
  for (int c = 0; c < w->n_clusters; c++) {
    if (w->cluster_sizes[c] < 1) return SG_ERR_INVALID;
    nMe += w->cluster_sizes[c];
  }
  sg_input in;
  sg_default_input(&in);
  in.iRegime = 2;
  in.iMaterial = w->iMaterial;
  in.ucx = w->ucx;
  in.ucy = w->ucy;
  in.nMolMe = nMe;
  in.temperatureK = w->temperatureK;
  in.stepLimit = w->stepLimit;
  in.stepAvg = w->stepAvg;
  in.stepEquil = w->stepEquil;
  in.stepCool = w->stepCool;
  in.stepRdf = w->stepRdf;
  if (w->limitRdf > 0) in.limitRdf = w->limitRdf;
  if (w->stepDiffuse > 0) in.stepDiffuse = w->stepDiffuse;
  if (w->nValDiffuse > 0) in.nValDiffuse = w->nValDiffuse;
  if (w->nBuffDiffuse > 0) in.nBuffDiffuse = w->nBuffDiffuse;
  if (w->limitDiffuseAv > 0) in.limitDiffuseAv = w->limitDiffuseAv;
  if (w->deltaT > 0) in.deltaT = w->deltaT;
  in.deltaFpN = 0.f;  // shear drive off
  in.randSeed = (int)(w->seed % 2147483646ull) + 1;
  int rc = sg_set_params(&in, p);
  if (rc) return rc;
  if (!r) return SG_OK;
  grapheneSheet(p, r);
  // fcc sites of an atom-centred sphere: integer points with an even coordinate sum, spacing
  // a/2, ordered by distance then lexicographically
  std::vector<Site> sites;
  int maxN = 0;
  for (int c = 0; c < w->n_clusters; c++) maxN = std::max(maxN, w->cluster_sizes[c]);
  int R = 2;
  while (true) {
    sites.clear();
    for (int i = -R; i <= R; i++)
      for (int j = -R; j <= R; j++)
        for (int k = -R; k <= R; k++)
          if (((i + j + k) & 1) == 0) sites.push_back(Site{i, j, k, (long long)i * i + j * j + k * k});
    // a full shell inside the cube is guaranteed for d2 <= R^2
    long long inside = 0;
    for (auto &s : sites) inside += (s.d2 <= (long long)R * R);
    if (inside >= maxN) break;
    R += 2;
  }
  std::sort(sites.begin(), sites.end(), [](const Site &x, const Site &y) {
    if (x.d2 != y.d2) return x.d2 < y.d2;
    if (x.i != y.i) return x.i < y.i;
    if (x.j != y.j) return x.j < y.j;
    return x.k < y.k;
  });
  const float h = 0.5f * p->a;
  const double clearance = w->clearance_A / kA0;
  std::vector<double> cxs, cys, crs;
  int n = 0;
  for (int c = 0; c < w->n_clusters; c++) {
    const int N = w->cluster_sizes[c];
    double rad = 0, zmin = 1e30;
    for (int s = 0; s < N; s++) {
      rad = std::max(rad, sqrt((double)sites[s].d2) * h);
      zmin = std::min(zmin, (double)sites[s].k * h);
    }
    // seeded non-overlapping placement (rejection sampling, bounded attempts)
    double px = 0, py = 0;
    bool ok = false;
    for (int attempt = 0; attempt < 10000 && !ok; attempt++) {
      px = (uni(w->seed, 4ull * (c * 10000ull + attempt)) - 0.5) * p->region.x;
      py = (uni(w->seed, 4ull * (c * 10000ull + attempt) + 1) - 0.5) * p->region.y;
      ok = true;
      for (size_t q = 0; q < cxs.size() && ok; q++) {
        double dx = px - cxs[q], dy = py - cys[q];
        dx -= p->region.x * std::nearbyint(dx / p->region.x);
        dy -= p->region.y * std::nearbyint(dy / p->region.y);
        if (sqrt(dx * dx + dy * dy) < rad + crs[q] + 2.0) ok = false;
      }
    }
    if (!ok) return SG_ERR_INVALID;  // the sheet is too small for these clusters
    cxs.push_back(px); cys.push_back(py); crs.push_back(rad);
    const double pz = p->z_0 + clearance - zmin;
    for (int s = 0; s < N; s++) {
      double x = px + sites[s].i * h, y = py + sites[s].j * h, z = pz + sites[s].k * h;
      x -= p->region.x * std::floor(x / p->region.x + 0.5);
      y -= p->region.y * std::floor(y / p->region.y + 0.5);
      r[n++] = sg_float4{(float)x, (float)y, (float)z, 0.f};
    }
  }
  if (v) {
    // Maxwell-Boltzmann velocities (Box-Muller on a counter-based stream), zero net momentum
    const double kT = (double)p->kB * p->temperature;
    double px = 0, py = 0, pz = 0, mtot = 0;
    std::vector<double> vv((size_t)3 * p->nMol);
    for (int i = 0; i < p->nMol; i++) {
      const double m = (i < p->nMolMe) ? (double)p->massMe : 1.0;
      const double sd = sqrt(kT / m);
      for (int d = 0; d < 3; d++) {
        const uint64_t ctr = 1000003ull + 6ull * i + 2 * d;
        const double u1 = uni(w->seed, ctr), u2 = uni(w->seed, ctr + 1);
        vv[3 * i + d] = sd * sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
      }
      px += m * vv[3 * i]; py += m * vv[3 * i + 1]; pz += m * vv[3 * i + 2];
      mtot += m;
    }
    for (int i = 0; i < p->nMol; i++) {
      v[i] = sg_float3{(float)(vv[3 * i] - px / mtot), (float)(vv[3 * i + 1] - py / mtot),
                       (float)(vv[3 * i + 2] - pz / mtot)};
    }
  }
  return SG_OK;
}

// ---- writers --------------------------------------------------------------------------------
static void propZero(sg_prop &v) { v.sum = v.sum2 = 0.f; }
static void propAccum(sg_prop &v) {
  v.sum += v.val;
  v.sum2 += v.val * v.val;
}
static void propAvg(sg_prop &v, int n) {
  v.sum /= n;
  const float d = v.sum2 / n - v.sum * v.sum;
  v.sum2 = (float)sqrt((d > 0.) ? (double)d : 0.);
}

extern "C" void sg_accum_props(sg_simparams *p, int icode) {
  sg_prop *all[7] = {&p->totEnergy, &p->potEnergy, &p->kinEnergy, &p->oneStep,
                     &p->centerOfMass, &p->cmVel, &p->frictForce};
  for (sg_prop *q : all) {
    if (icode == 0) propZero(*q);
    else if (icode == 1) propAccum(*q);
    else if (icode == 2) propAvg(*q, p->stepAvg);
  }
}

extern "C" int sg_print_summary(void *fpv, const sg_simparams *p) {
  FILE *fp = (FILE *)fpv;
  if (!fp) return SG_ERR_INVALID;
  float totEn = p->totEnergy.sum * p->enU;
  float totEnRms = p->totEnergy.sum2 * p->enU;
  float potEn = p->potEnergy.sum * p->enU;
  float potEnRms = p->potEnergy.sum2 * p->enU;
  float T = 2.f * p->kinEnergy.sum * p->temperatureU / (3 * p->kB);
  float TRms = 2.f * p->kinEnergy.sum2 * p->temperatureU / (3 * p->kB);
  fprintf(fp, "%5d\t %7.7f\t %7.7f\t %7.7f\t %7.7f\t %7.7f\t %7.7f\t %7.7f\t %7.7f\t", p->stepCount,
          (p->vSum.x + p->vSum.y + p->vSum.z) / p->nMol, totEn, totEnRms, potEn, potEnRms, T, TRms,
          p->oneStep.sum);
  float cm = p->centerOfMass.sum * p->lengthU;
  float fr = p->frictForce.sum / p->forceU;
  float sx = p->particleSize.x * p->lengthU, sy = p->particleSize.y * p->lengthU, sz = p->particleSize.z * p->lengthU;
  float ts = p->totalShear / p->forceU;
  fprintf(fp, "%7.7f\t %7.7f\t %7.6f\t %7.7f\t %7.7f\t %7.7f\t %7.7f\n", p->cmVel.sum, cm, fr, sx, sy, sz, ts);
  fflush(fp);
  return SG_OK;
}

extern "C" int sg_result_file_name(const sg_simparams *p, char *out, int out_len) {
  char buf[SG_MAX_PATH];
  const double T = p->temperature * p->temperatureU;
  if (p->iRegime == 0)
    snprintf(buf, sizeof buf, "_blk_x%i_y%i_z%i_Me%i_Av%i_Pdb%i_T%3.0f", p->initUcell.x, p->initUcell.y,
             p->initUcell.z, p->nMolMe, p->stepAvg, p->stepPdb, T);
  else if (p->iRegime == 1)
    snprintf(buf, sizeof buf, "_x%i_y%i_Me%i_Eq%i_Dep%i_TD%i_Pdb%i_T%3.0f", p->initUcell.x, p->initUcell.y,
             p->nMolMe, p->stepEquil, p->stepDeposit, p->nMolToDeposit, p->stepPdb, T);
  else
    snprintf(buf, sizeof buf, "_sh_x%i_y%i_Me%i_Eq%i_C%i_Av%i_Pdb%i_T%3.0f", p->initUcell.x, p->initUcell.y,
             p->nMolMe, p->stepEquil, p->stepCool, p->stepAvg, p->stepPdb, T);
  std::string s = std::string("sg") + buf + std::string(p->szNameMe, strnlen(p->szNameMe, 3)) + ".txt";
  if ((int)s.size() >= out_len) return SG_ERR_INVALID;
  strcpy(out, s.c_str());
  return SG_OK;
}

extern "C" int sg_print_result_header(void *fpv, const sg_simparams *p, float deposEnergyEv) {
  FILE *f = (FILE *)fpv;
  if (!f) return SG_ERR_INVALID;
  fprintf(f, "stepCnt\t impulse\t totEn(eV)\t totEn.rms(eV)\t potEn(eV)\t potEn.rms(eV)\t Tempr(K)\t T.rms(K)\t "
             "oneStep(ms)\t Veloc_CM\t CM(angstr)\t friction(nN)\t sizex(angstr)\t sizey(angstr)\t "
             "sizez(angstr)\t shearForce(nN)\t");
  if (p->bResult != 0) fprintf(f, "time step = %f\t", p->deltaT);
  if (p->bResult != 0 && p->iRegime == 1) fprintf(f, "deposit energy = %f eV\t", deposEnergyEv);
  if (p->bResult != 0 && p->iRegime == 2) fprintf(f, "increment of shear = %f pN\t", p->deltaF * 1000 / p->forceU);
  if (p->bResult != 0 && p->iRegime != 0) {
    fprintf(f, "epsilonLJ = %f eV\t", p->epsLJ * p->enU);
    fprintf(f, "sigmaLJ = %f angstrom", p->sigmaLJ * p->lengthU);
  }
  if (p->bResult != 0) fprintf(f, "\n");
  return SG_OK;
}

extern "C" int sg_create_pdb(const char *prefix, const sg_simparams *p, const sg_float4 *r) {
  char suffix[SG_MAX_PATH];
  memset(suffix, 0, sizeof suffix);
  const int i = p->stepCount / p->stepPdb;
  if (i < 100) snprintf(suffix, sizeof suffix, "_%i", i);
  else if (i < 1000) snprintf(suffix, sizeof suffix, "_%-3i", i);
  else if (i < 10000) snprintf(suffix, sizeof suffix, "_%-4i", i);
  std::string name = std::string(prefix) + suffix + ".pdb";
  FILE *f = fopen(name.c_str(), "w");
  if (!f) return SG_ERR_IO;
  const std::string me(p->szNameMe, strnlen(p->szNameMe, 3));
  const float m = 0.f;
  for (int k = 0; k < p->nMol; k++) {
    fprintf(f, "ATOM  ");
    fprintf(f, "%-7i", k);
    if (k >= p->nMolMe) fprintf(f, "C  ");
    else fprintf(f, "%2s ", me.c_str());
    fprintf(f, " ");
    if (k >= p->nMolMe) fprintf(f, " C   ");
    else fprintf(f, " %2s  ", me.c_str());
    fprintf(f, " ");
    fprintf(f, "    ");
    fprintf(f, "%-4i", 0);
    fprintf(f, "%-8.2lf", 1.42 * r[k].x);
    fprintf(f, "%-8.2lf", 1.42 * r[k].y);
    if (p->iRegime == 1 && k < p->nMolMe && k >= p->nMolDeposited)
      fprintf(f, "%-8.2lf", 1.42 * 2 * p->region.z);
    else
      fprintf(f, "%-8.2lf", 1.42 * r[k].z);
    fprintf(f, " %4.1lf", (double)m);
    fprintf(f, "  1.00");
    fprintf(f, "          ");
    if (k >= p->nMolMe) fprintf(f, " C");
    else fprintf(f, "%2s", me.c_str());
    fprintf(f, "  \n");
  }
  fclose(f);
  return SG_OK;
}

extern "C" int sg_print_rdf(const sg_simparams *p, const unsigned int *hist) {
  char buf[SG_MAX_PATH];
  snprintf(buf, sizeof buf, "_stepCount_%i_", p->stepCount);
  std::string name = std::string(p->szRdfPath) + buf + std::string(p->szNameMe, strnlen(p->szNameMe, 3)) + ".txt";
  float normFac = (float)((p->particleSize.x * p->particleSize.y * p->particleSize.z) *
                          (p->intervalRdf * p->intervalRdf * p->intervalRdf) / (2.f * M_PI * p->countRdf));
  normFac = normFac / p->nMolMe;
  normFac = normFac / p->nMolMe;
  FILE *f = fopen(name.c_str(), "w+");
  if (!f) return SG_ERR_IO;
  for (int n = 0; n < p->sizeHistRdf; n++) {
    const float rb = (n + 0.5f) * p->rangeRdf * p->lengthU / p->sizeHistRdf;
    const float h = (float)hist[n] * normFac / ((n - 0.5f) * (n - 0.5f));
    fprintf(f, "%8.4f\t %8.4f\n", rb, h);
  }
  fclose(f);
  return SG_OK;
}

extern "C" int sg_print_diffusion(void *fpv, const sg_simparams *p, const float *table) {
  FILE *f = (FILE *)fpv;
  if (!f) return SG_ERR_INVALID;
  fprintf(f, "diffusion\n");
  for (int j = 0; j < p->nValDiffuse; j++) {
    const float t = j * p->stepDiffuse * p->deltaT;
    fprintf(f, "%8.4f %8.4f\n", t, table[j]);
  }
  return SG_OK;
}

extern "C" int sg_write_backup(const char *path, const sg_simparams *p, const sg_float4 *r, const sg_float3 *v,
                               const sg_float3 *a) {
  FILE *f = fopen(path, "w+b");
  if (!f) return SG_ERR_IO;
  size_t ok = fwrite(p, sizeof(sg_simparams), 1, f);
  ok &= fwrite(r, sizeof(sg_float4), p->nMol, f) == (size_t)p->nMol;
  ok &= fwrite(v, sizeof(sg_float3), p->nMol, f) == (size_t)p->nMol;
  ok &= fwrite(a, sizeof(sg_float3), p->nMol, f) == (size_t)p->nMol;
  fclose(f);
  return ok ? SG_OK : SG_ERR_IO;
}

extern "C" int sg_read_backup(const char *path, sg_simparams *p, sg_float4 *r, sg_float3 *v, sg_float3 *a) {
  FILE *f = fopen(path, "rb");
  if (!f) return SG_ERR_IO;
  sg_simparams q;
  if (fread(&q, sizeof q, 1, f) != 1 || q.nMol <= 0 || q.nMolMe < 0 || q.nMolMe > q.nMol) {
    fclose(f);
    return SG_ERR_BAD_FILE;
  }
  // the file must hold exactly the three arrays after the parameter block
  fseek(f, 0, SEEK_END);
  const long want = (long)sizeof(sg_simparams) + (long)q.nMol * (long)(sizeof(sg_float4) + 2 * sizeof(sg_float3));
  if (ftell(f) != want) {
    fclose(f);
    return SG_ERR_BAD_FILE;
  }
  *p = q;
  if (r && v && a) {
    fseek(f, (long)sizeof(sg_simparams), SEEK_SET);
    bool ok = fread(r, sizeof(sg_float4), q.nMol, f) == (size_t)q.nMol;
    ok = ok && fread(v, sizeof(sg_float3), q.nMol, f) == (size_t)q.nMol;
    ok = ok && fread(a, sizeof(sg_float3), q.nMol, f) == (size_t)q.nMol;
    fclose(f);
    return ok ? SG_OK : SG_ERR_BAD_FILE;
  }
  fclose(f);
  return SG_OK;
}
