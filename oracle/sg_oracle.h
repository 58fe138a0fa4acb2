/*
 * sg_oracle.h - TEST INFRASTRUCTURE.  CPU restatement of the SurfaceGrowthConsole timestep,
 * used only as the checker by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg.  Nothing in the product (libsgmd.so, the Python package) links to or calls it.
 *
 * It restates SurfaceGrowthConsole/SurfaceGrowth.cu (kernels cu:397-1999, step loop
 * cu:2141-2489, host analysis cu:2659-2952) in plain C++, instantiated in float (same
 * operation order as the reference, compiled with -ffp-contract=off, host libm for the
 * transcendental functions) and in double (the same model evaluated in FP64, used as the
 * precision reference).  In-cell atom order is ascending atom index (the reference's order
 * is whatever its atomics produce; ascending index is one of its possible orders).
 *
 * Pinning: its host-side functions are checked against outputs of the reference's own host
 * code compiled here (oracle/ref/build_ref.sh -> oracle/_ref/, fixtures in tests/golden/);
 * the device-side parts are checked against the reference's CUDA kernels where those have
 * been run (tests/golden/ref_kernels_*), see tests/test_oracle_pins.py.
 */
#ifndef SG_ORACLE_H
#define SG_ORACLE_H

#include "../include/sg_api.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

/* precision: 32 or 64.  force_rebuild: rebuild lists every step. */
orc_sim *orc_create(const sg_simparams *p, int precision, int force_rebuild);
void orc_destroy(orc_sim *s);
void orc_set_threads(int n);
int orc_get_threads(void);

void orc_set_state(orc_sim *s, const sg_float4 *r, const sg_float3 *v, const sg_float3 *a);
void orc_get_state(orc_sim *s, sg_float4 *r, sg_float3 *v, sg_float3 *a);
/* FP64 view of the state: r4[4*nMol], v3[3*nMol], a3[3*nMol] */
void orc_get_state64(orc_sim *s, double *r4, double *v3, double *a3);
void orc_set_state64(orc_sim *s, const double *r4, const double *v3, const double *a3);

int orc_step(orc_sim *s, int nsteps);
void orc_get_thermo(orc_sim *s, sg_thermo *t);
void orc_get_params(orc_sim *s, sg_simparams *p);

int orc_build_lists(orc_sim *s);
int orc_compute_forces(orc_sim *s);
int orc_eval_rdf(orc_sim *s);
void orc_reset_rdf(orc_sim *s);

int orc_num_cells(orc_sim *s);
void orc_get_cells(orc_sim *s, int *cell_of_atom, int *cell_start, int *cell_atoms);
void orc_get_nebr(orc_sim *s, int *nn, int *nbl);
void orc_get_rho(orc_sim *s, float *rho);
void orc_get_friction(orc_sim *s, float *fric);
void orc_get_rdf(orc_sim *s, unsigned int *hist);
void orc_get_diffusion(orc_sim *s, float *rr_av, int *counts, int *count_av);
void orc_get_diag(orc_sim *s, sg_diag *d);

/* Reference-tree reductions on given arrays (SurfaceGrowth.cu:1101-1892), FP32.
 * what: 0 vSum, 1 vvMax, 2 vvSum, 3 potEnergy, 4 centerOfMass, 5 cmVel, 6 sizeMin,
 *       7 sizeMax, 8 frictForce.  out receives 3 floats. */
void orc_reduce(const sg_simparams *p, int what, const sg_float4 *r, const sg_float3 *v,
                const float *fric, float cmVelX, float *out);

/* EvalDiffusion/AccumDiffusion (SurfaceGrowth.cu:2898-2952) over a sequence of centre-of-mass
 * samples; writes each finished table (nValDiffuse floats) and returns how many. */
int orc_diffusion_replay(const sg_simparams *p, int n, const float *cm3, float *tables, int maxTables);

/* Analytic EAM pieces (SurfaceGrowth.cu:46-210) for known-answer tests. */
double orc_eam_eval(const sg_simparams *p, int which, double x, int precision);

/* All-pairs metal-metal histogram with minimum image, FP64 distances: bins of width
 * range/nbins, ordered pairs.  The check for the extended RDF. */
void orc_rdf_allpairs(const sg_simparams *p, const sg_float4 *r, int nbins, double range,
                      unsigned long long *hist);

#ifdef __cplusplus
}
#endif
#endif
