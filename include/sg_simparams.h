/*
 * sg_simparams.h - binary-compatible parameter block of the SurfaceGrowth step.
 *
 * The reference passes one struct (SimParams, SurfaceGrowthConsole/SurfaceGrowth.h:69-186)
 * by pointer across its C wrappers.  A drop-in must accept the same bytes, so this header
 * defines a struct with the same field order, types and therefore the same offsets
 * (1112 bytes, 4-byte alignment on LP64 gcc/clang; checked by static asserts below and by
 * tests/test_abi.py against a table generated from the reference header).
 *
 * Only plain C types are used: sg_float3/sg_int3/sg_uint3 have the layout of CUDA's
 * float3/int3/uint3 (three 4-byte members, 4-byte alignment), sg_prop the layout of the
 * reference's Prop {val,sum,sum2} (SurfaceGrowthConsole/ComputeDefs.h:53-55).
 *
 * Units (SurfaceGrowthConsole/SurfaceGrowth.cpp:192-197): length 1.42 A, energy
 * 0.06275049 eV, mass 12.0107 amu (carbon), time 0.2 ps, dt 0.001 = 0.2 fs.
 */
#ifndef SG_SIMPARAMS_H
#define SG_SIMPARAMS_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sg_float3 { float x, y, z; } sg_float3;
typedef struct sg_float4 { float x, y, z, w; } sg_float4;
typedef struct sg_int3 { int x, y, z; } sg_int3;
typedef struct sg_uint3 { unsigned int x, y, z; } sg_uint3;

/* Running property: current value, sum and sum of squares (ComputeDefs.h:53-61). */
typedef struct sg_prop { float val, sum, sum2; } sg_prop;

#define SG_MAX_PATH 264

/* Field-for-field image of SimParams (SurfaceGrowth.h:69-186).  Comments give the
 * meaning the reference assigns to each field. */
typedef struct sg_simparams {
    sg_float3 region;        /* simulation box (dimensionless) */
    sg_float3 vSum;          /* total impulse of the last step */
    sg_uint3 initUcell;      /* unit cells of the substrate / bulk crystal */
    float deltaT, rCutC, rrCutC, temperature, velMag;
    int moreCycles, stepAvg, stepEquil, stepCount, stepPdb, stepLimit;
    int bPdb, bResult;
    int nMol;                /* all atoms; indices [0,nMolMe) are metal, the rest carbon */
    int nMolMe;
    unsigned int gridSize;   /* number of cells (the reference launches one block per cell) */
    unsigned int blockSize;  /* 64: threads per block == maximum atoms per cell */
    sg_int3 cells;           /* cell grid for the neighbour search */
    sg_float3 invWidth;      /* cells / region */
    float rNebrShell, rrNebr;
    int iNebrMax, maxMol, nebrNow;
    float dispHi;
    sg_prop kinEnergy, totEnergy, potEnergy, oneStep;
    /* EAM (Zhou-Wadley-Johnson) parameters, dimensionless */
    float a, re, fe, rhoe, alpha, beta, A, B, kappa, lambda;
    float Fn[4], F[4];
    float eta, Fe, massMe, density, rCutEam, rrCutEam, rei, rhoei;
    char szNameMe[3];
    /* units */
    float temperatureU, kB, enU, lengthU, forceU, massU;
    /* graphene */
    float mu_r, theta_0, mu_theta, mu_p, z_0;
    /* Berendsen thermostat */
    int stepThermostat;
    float gammaBerendsen;
    int stepCool;
    int iRegime;             /* 0 bulk, 1 surface growth (deposition), 2 shear */
    float sigmaLJ, epsLJ, rCutLJ, rrCutLJ;
    /* deposition */
    float velMagDepos;
    int randSeedP, stepDeposit, nMolDeposited, nMolToDeposit;
    /* tribology */
    sg_prop centerOfMass, cmVel, frictForce;
    float deltaF;
    sg_float3 particleSize;
    int cellShiftZ;
    float shear, totalShear;
    int initUcellMeX, initUcellMeY;
    /* radial distribution function */
    float rangeRdf;
    int limitRdf, sizeHistRdf, stepRdf, countRdf;
    float intervalRdf;
    int bRdf;
    char szRdfPath[SG_MAX_PATH];
    /* backup */
    char szBckup0[20];
    char szBckup1[20];
    int bBckup, bStartBckup, stepBckup;
    float totalTime;
    int iMaterial;
    /* nanoparticle centre-of-mass diffusion */
    int nValDiffuse, nBuffDiffuse, stepDiffuse, limitDiffuseAv, countDiffuseAv;
    char szDiffusePath[SG_MAX_PATH];
} sg_simparams;

#ifdef __cplusplus
}
#include <cstddef>
static_assert(sizeof(sg_simparams) == 1112, "sg_simparams must match the reference SimParams size");
static_assert(offsetof(sg_simparams, kinEnergy) == 152, "layout");
static_assert(offsetof(sg_simparams, szNameMe) == 304, "layout");
static_assert(offsetof(sg_simparams, szRdfPath) == 504, "layout");
static_assert(offsetof(sg_simparams, szDiffusePath) == 848, "layout");
#endif

#endif /* SG_SIMPARAMS_H */
