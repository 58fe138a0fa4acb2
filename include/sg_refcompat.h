/*
 * sg_refcompat.h - the reference's own C wrapper ABI, implemented by libsgmd.so.
 *
 * These four symbols are what the reference's host program (SurfaceGrowth.cpp) binds to
 * (declared in SurfaceGrowthConsole/SurfaceGrowth.h:217-235, defined in
 * SurfaceGrowthConsole/SurfaceGrowth.cu:2005-2652).  Signatures are byte-compatible: the
 * reference's float4/float3 are sg_float4/sg_float3 here, SimParams is sg_simparams
 * (same 1112-byte layout), TCHAR is char.
 *
 * Behavioural differences, all on the failure paths only:
 *  - CudaInitW and SetParametersW never call exit(); a failure is remembered and reported
 *    by the next DoComputationsW as its error string (the reference exits the process,
 *    SurfaceGrowth.cu:2622 and 2648).
 *  - The graphics wrappers declared next to these (CudaGLInitW ... DoComputationsGLW,
 *    SurfaceGrowth.h:220-231) are declared but never defined by the reference; they are not
 *    provided here either.
 */
#ifndef SG_REFCOMPAT_H
#define SG_REFCOMPAT_H

#include <stdio.h>
#include "sg_simparams.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Selects device 0 (SurfaceGrowth.cu:2614-2637). */
void CudaInitW(int argc, char **argv);

/* Records the parameter block used by the following calls (SurfaceGrowth.cu:2639-2650). */
void SetParametersW(sg_simparams *hostParams);

/* Fills hr[nMol] with the regime's initial lattice (SurfaceGrowth.cu:2532-2609): fcc bulk
 * (regime 0), graphene + metal parked above the box (regime 1), graphene + fcc slab
 * (regime 2, also sets initUcellMeX/Y).  dr is ignored (the reference allocates and frees
 * its own scratch there).  Returns NULL or an error string. */
const char *InitCoordsW(sg_float4 *dr, sg_float4 *hr, sg_simparams *hparams);

/* Runs the whole simulation to hparams->stepLimit (SurfaceGrowth.cu:2013-2529), writing the
 * summary rows to fResults and rdf_*, sugr_*.pdb (prefix szPdbPath), Diffuse.txt and backup
 * files.  Returns 0 on success; on failure copies a message into szPdbPath (which must hold
 * SG_MAX_PATH bytes) and returns it, as the reference does. */
char *DoComputationsW(sg_float4 *hr, sg_float3 *hv, sg_float3 *ha, sg_simparams *hparams,
                      FILE *fResults, char *szPdbPath);

#ifdef __cplusplus
}
/* The reference's host program also calls AccumProps (C++ linkage; SurfaceGrowth.cu:2659-2731,
 * called from SurfaceGrowth.cpp:417): averages of the step properties, icode 0 zero / 1 add /
 * 2 average.  Exported with the reference's signature; SimParams is its name for sg_simparams. */
struct SimParams;
void AccumProps(int icode, SimParams *hparams);
#endif
#endif /* SG_REFCOMPAT_H */
