/*
 * sg_api.h - C ABI of sgmd, a GB300 (sm_103a) implementation of the SurfaceGrowthConsole
 * per-timestep force and integration path.
 *
 * Two layers are exported by libsgmd.so:
 *
 *  1. The reference's own wrapper ABI (sg_refcompat.h): CudaInitW, SetParametersW,
 *     InitCoordsW, DoComputationsW, with the reference's SimParams bytes
 *     (SurfaceGrowthConsole/SurfaceGrowth.h:217-235), so the reference's host program links
 *     against this library unchanged.
 *
 *  2. The finer sg_* API below.  Every call returns an int status (SG_OK == 0), never calls
 *     exit(), keeps no global simulation state (everything hangs off an sg_ctx) and takes
 *     plain pointers and sizes.  Host arrays use the reference's layouts: positions are
 *     float4 {x,y,z,U} (U = per-atom potential energy, written by the force pass), velocities
 *     and accelerations float3, all in the reference's atom order (metal atoms first).
 *
 * A context holds one or more independent replicas (systems).  Each replica is described by
 * one sg_simparams, i.e. exactly what the reference's SetParams() derives from sugr_in.txt;
 * all replicas of a context advance together and share one launch per kernel phase.
 *
 * Status codes other than SG_OK leave a message retrievable with sg_last_error().
 */
#ifndef SG_API_H
#define SG_API_H

#include "sg_simparams.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SG_API_VERSION 1

/* ---- status codes -------------------------------------------------------------------- */
enum {
    SG_OK = 0,
    SG_ERR_INVALID = 1,        /* bad argument or inconsistent parameters */
    SG_ERR_CUDA = 2,           /* CUDA runtime error */
    SG_ERR_NOMEM = 3,          /* device or host allocation failed */
    SG_ERR_NO_DEVICE = 4,      /* no CUDA device, or not an sm_103 device */
    SG_ERR_NEBR_OVERFLOW = 5,  /* an atom had more than iNebrMax neighbours (list truncated) */
    SG_ERR_CELL_RANGE = 6,     /* an atom mapped outside the cell grid (left out of the lists) */
    SG_ERR_RDF_RANGE = 7,      /* reserved: an RDF bin index that rounds to sizeHistRdf is dropped and
                                  counted in sg_diag.rdf_range, not reported */
    SG_ERR_TIMEOUT = 8,        /* a bounded device-side wait gave up */
    SG_ERR_IO = 9,             /* output file could not be written */
    SG_ERR_UNSUPPORTED = 10,   /* feature not available in this mode */
    SG_ERR_CELL_OVERFLOW = 11, /* PLAIN: more than blockSize (64) atoms in one cell (the reference's
                                  cap); MIXED: more than 4 x blockSize (256) */
    SG_ERR_BAD_FILE = 12       /* malformed input or checkpoint file */
};

/* ---- modes ------------------------------------------------------------------------------ */
enum {
    /* FP32 throughout, arithmetic in the reference's operation order without FMA
     * contraction, reductions in the reference's tree order.  Integer outputs (cell
     * assignment, neighbour lists, RDF counts) are bit-exact with the reference; forces
     * agree to within the accuracy of the CUDA/libm transcendental functions. */
    SG_MODE_PLAIN = 0,
    /* The same model: FP32 pair arithmetic with FMA, EAM pair functions from cubic tables (read
     * through L1), FP64 accumulation of energy/virial/momentum sums, FP64 thermostat factor and
     * MSD accumulators, and positions carried as a float hi/lo pair. */
    SG_MODE_MIXED = 1
};

typedef struct sg_options {
    int mode;              /* SG_MODE_PLAIN or SG_MODE_MIXED */
    int force_rebuild;     /* 1: rebuild cell and neighbour lists every step */
    int use_graphs;        /* 1: capture each step variant in a CUDA graph (default) */
    int device;            /* CUDA device ordinal */
    void *stream;          /* cudaStream_t to run on; NULL: the context creates its own */
    int rdf_ext_bins;      /* >0: also accumulate an all-pairs metal-metal RDF */
    float rdf_ext_range;   /* its range, dimensionless length */
    int eam_table_knots;   /* MIXED: intervals of the tabulated EAM pair functions (0: 1024; -1: analytic) */
    int metal_lanes;       /* lanes per metal atom in the density and metal force passes:
                            * 4, 8, 16 or 32 (0: 16) */
    int nebr_blocks_per_sm;/* resident 128-thread blocks per SM of the list build's work queue,
                            * 1..32 (0: 7, the blocks the list build keeps resident) */
    int phase_timing;      /* 1: record CUDA events between the phases of every step */
    int programmatic_launch; /* 1 (default): launch the kernels of a step with programmatic
                            * dependent launch (a kernel is launched once its predecessor's blocks
                            * have exited and waits for its completion); 0: off */
    int nebr_descending;   /* 1: the list build takes the non-crowded cells in descending cell
                            * order (0: ascending) */
    int nebr_item_atoms;   /* list build: most home atoms of one work item (a warp's share); a
                            * cell of more atoms is split into near-equal items, 4..64 (0: 8) */
    int nebr_build;        /* list build: 0 a warp per cell window, hits placed by the warp; 1 a
                            * thread per atom; 2 a warp per cell window, hits placed by one lane
                            * per home atom; the same lists */
    int eam_table_smem;    /* MIXED: 1 the metal passes stage the EAM table in shared memory
                            * (a grid of 4 blocks per SM), 0 read it through L1 */
    int carbon_blocks_per_sm; /* carbon pass compiled for 8, 12 or 16 resident 128-thread blocks
                            * per SM (64, 40 or 32 registers a thread; 0: 8) */
    int persistent_step;   /* MIXED: 1 runs each step as one cooperative launch over all replicas,
                            * its phases (integrate, cell scan and order, list build, density and
                            * carbon forces, metal forces, reduction) separated by grid-wide
                            * barriers instead of kernel boundaries; 0 (default): one launch per
                            * phase, captured in a CUDA graph.  Metal lanes 4 or 16, the cell-window
                            * list build. */
    int persistent_wait_us; /* persistent step: longest wait at a grid barrier, microseconds of
                            * the SM clock (0: 1,000,000); a launch whose wait runs out leaves with
                            * SG_ERR_TIMEOUT and the context must be destroyed */
    int nebr_capacity;     /* MIXED: entries per neighbour-list row, at least the parameter
                            * block's iNebrMax (0: iNebrMax); a hot system that crowds atoms keeps
                            * its full lists where PLAIN stops with SG_ERR_NEBR_OVERFLOW.
                            * sg_get_nebr still returns iNebrMax columns. */
} sg_options;

/* Initialise *opt with the defaults (PLAIN mode, graphs on, device 0). */
void sg_default_options(sg_options *opt);

typedef struct sg_ctx sg_ctx;

/* Last error message of the calling thread ("" if none). */
const char *sg_last_error(void);
int sg_version(void);

/* ---- context ------------------------------------------------------------------------------
 * Replaces the allocation and upload half of DoComputationsW
 * (SurfaceGrowthConsole/SurfaceGrowth.cu:2040-2126) and SetParametersW (cu:2639-2650).
 * params points to n_replicas consecutive sg_simparams.  A context is used by one host thread
 * at a time (its calls share the context's stream, graphs and host mirror); separate contexts
 * may be driven from separate threads. */
int sg_create(const sg_simparams *params, int n_replicas, const sg_options *opt, sg_ctx **out);
int sg_destroy(sg_ctx *ctx);
int sg_num_replicas(const sg_ctx *ctx);
/* Number of atoms of replica rep (rep < 0: all replicas). */
int sg_num_atoms(const sg_ctx *ctx, int rep);

/* Upload / download state of one replica (rep >= 0) or of all replicas concatenated
 * (rep == -1).  Any pointer may be NULL to skip that array.  Layouts as the reference's
 * host arrays hr/hv/ha (SurfaceGrowth.cpp:95-96).  A download first applies a pending
 * thermostat rescale, so it returns exactly the reference's end-of-step velocities.  An upload
 * reads the host arrays in place from the device where it can (any host memory on a device
 * that reads through the host's page tables, as a GB300 on NVLink-C2C; page-locked memory
 * elsewhere) and copies them first otherwise; it has finished with them when the call returns. */
int sg_set_state(sg_ctx *ctx, int rep, const sg_float4 *r, const sg_float3 *v, const sg_float3 *a);
int sg_get_state(sg_ctx *ctx, int rep, sg_float4 *r, sg_float3 *v, sg_float3 *a);

/* The replica's parameter block with the mutable fields (stepCount, Props, nebrNow,
 * dispHi, shear, countRdf, ...) as the reference would hold them after the last step. */
int sg_get_params(sg_ctx *ctx, int rep, sg_simparams *out);

/* ---- stepping ------------------------------------------------------------------------------
 * One timestep is the body of the reference loop DoComputationsW
 * (SurfaceGrowth.cu:2141-2489) without file output: Verlet part 1 + wrap, cell/neighbour
 * rebuild when nebrNow, EAM density, forces, friction sum, Verlet part 2, tribology
 * reductions, nanoparticle diffusion sample, momentum/max-v2/Sum mv2, Berendsen thermostat,
 * potential energy, rebuild criterion, shear, RDF sample, property accumulation.  Returns
 * when the steps are done: a one-block kernel copies the replica states to a page-locked host
 * mirror followed by a sequence number, which the call polls for up to 5 ms before it falls back
 * to synchronising the stream (which also reports a failed launch). */
int sg_step(sg_ctx *ctx, int nsteps);
/* Bytes sg_step copies back to the host after its steps (the replicas' state records). */
long long sg_step_readback_bytes(const sg_ctx *ctx);
/* The same steps, launched on the context's stream without waiting for them (no status from
 * the device is checked; call sg_step(ctx, 0) to synchronise and collect it). */
int sg_step_async(sg_ctx *ctx, int nsteps);
/* Kernel launches one step issues (for the step variant that ran last). */
int sg_kernels_per_step(sg_ctx *ctx);
/* With phase_timing on: durations in ms of the phases of the last step: integrate, rebuild
 * (counting sort + neighbour-list build), metal chain (density, metal forces, metal
 * centre-of-mass velocity; runs beside the carbon pass), carbon pass, forces (fork to join),
 * reduce, extra (shear/RDF), neighbour-list build alone.  Returns the number of phases (8), or
 * minus a status code. */
int sg_get_phase_times(sg_ctx *ctx, float *ms, int n);

typedef struct sg_thermo {
    int stepCount;
    int nebrNow;            /* lists will be rebuilt at the next step */
    int rebuilds;           /* rebuilds performed since creation */
    int countRdf;
    float kinEnergy, potEnergy, totEnergy; /* per-atom means, reference definition */
    float vvSum, vvMax, uSum, dispHi;
    sg_float3 vSum;                        /* total impulse (metal x mass-weighted) */
    sg_float3 centerOfMass;                /* metal centre of mass (wrapped coordinates) */
    sg_float3 cmVel;                       /* metal centre-of-mass velocity */
    float frictForce;                      /* x force of carbon on metal */
    sg_float3 particleSize;
    float shear, totalShear;
    double kinEnergy64, potEnergy64;       /* FP64 sums / nMol (MIXED; PLAIN: promoted) */
    double virial64;                       /* pair virial sum (MIXED; 0 in PLAIN) */
    sg_prop props[7];  /* totEnergy, potEnergy, kinEnergy, oneStep, centerOfMass, cmVel, frictForce */
} sg_thermo;
int sg_get_thermo(sg_ctx *ctx, int rep, sg_thermo *out);
/* sg_step, then replica rep's thermo record (as sg_get_thermo) from the same wait. */
int sg_step_thermo(sg_ctx *ctx, int nsteps, int rep, sg_thermo *thermo);
/* A step from host buffers in one call: sg_set_state(ctx, rep, r, v, a), then sg_step(ctx,
 * nsteps) and, if thermo is not NULL, replica thermo_rep's record, with one wait for the
 * whole (the copies are enqueued on the context's stream ahead of the steps; the host buffers
 * are free again when the call returns).  Results equal those of the three calls. */
int sg_step_from_host(sg_ctx *ctx, int rep, const sg_float4 *r, const sg_float3 *v, const sg_float3 *a,
                      int nsteps, int thermo_rep, sg_thermo *thermo);

/* ---- single phases on the current state (parity checks, harness) ---------------------- */
/* Cell binning + neighbour list from the current positions
 * (BinAtomsIntoCellsK cu:547-609 + BuildNebrListK cu:612-711). */
int sg_build_lists(sg_ctx *ctx);
/* EAM density and forces on the current state (EamComputeRhoK cu:716-773,
 * ComputeForcesK cu:776-1091): writes a, r.w and the metal friction array. */
int sg_compute_forces(sg_ctx *ctx);
/* One RDF sample (EvalRdfK cu:1895-1999) over the last-built cells, current positions. */
int sg_eval_rdf(sg_ctx *ctx);
int sg_reset_rdf(sg_ctx *ctx);

/* Counting-sort result, local atom indices: cell_of_atom[nMol] (linear cell index, -1 if the
 * atom fell outside the grid), cell_start[ncells+1], cell_atoms[nMol] (atoms grouped by cell,
 * ascending index inside a cell). */
int sg_get_cells(sg_ctx *ctx, int rep, int *cell_of_atom, int *cell_start, int *cell_atoms);
int sg_num_cells(const sg_ctx *ctx, int rep);
/* Neighbour list in the reference layout: nn[nMol], nbl[iNebrMax * nMol] column-major
 * (entry j of atom i at nbl[j*nMol + i]), local indices, unused entries -1. */
int sg_get_nebr(sg_ctx *ctx, int rep, int *nn, int *nbl);
/* The carbon pass's lists of each atom, local indices: ns[nMol] close-list lengths (-1: the
 * pass walks the full list), sl[nMol * 8] close entries (within rCutC + rNebrShell, list
 * order); nrl[nMol] relevant-list lengths (-1 as ns), rl[nMol * 48 * 2] relevant entries
 * {atom, position in the full list} (metal entries and close entries, list order).  Entries
 * past a length are -1.  Metal atoms have length 0. */
int sg_get_carbon_lists(sg_ctx *ctx, int rep, int *ns, int *sl, int *nrl, int *rl);
int sg_get_rho(sg_ctx *ctx, int rep, float *rho);          /* nMolMe values */
int sg_get_friction(sg_ctx *ctx, int rep, float *fric);    /* nMolMe values */
int sg_get_rdf(sg_ctx *ctx, int rep, unsigned int *hist);  /* sizeHistRdf counts */
int sg_get_rdf_ext(sg_ctx *ctx, int rep, unsigned long long *hist); /* rdf_ext_bins counts */
/* Diffusion accumulators (TBuf/rrDiffuseAv of SurfaceGrowth.cu:2021-2032): rr_av[nValDiffuse]
 * as currently accumulated, counts[nBuffDiffuse]. */
int sg_get_diffusion(sg_ctx *ctx, int rep, float *rr_av, int *counts, int *count_av);

typedef struct sg_diag {
    int max_neighbours;      /* largest neighbour count seen */
    int max_cell_occupancy;  /* largest atoms-per-cell seen */
    int nebr_overflow;       /* atoms whose list was truncated */
    int cell_range;          /* atoms left out of the grid */
    int cell_overflow;       /* cells above blockSize atoms */
    int rdf_range;           /* RDF samples dropped at the top bin (the reference writes them one
                                element past its histogram) */
    int timeouts;            /* bounded waits that gave up */
    int reserved[9];
} sg_diag;
int sg_get_diag(sg_ctx *ctx, int rep, sg_diag *out);

/* ---- whole run with the reference's outputs ------------------------------------------------
 * Runs replica 0 to stepLimit exactly as DoComputationsW does, writing the sg_* summary rows
 * to fResults (a FILE*), rdf_* files, sugr_*.pdb snapshots (name prefix pdb_prefix),
 * Diffuse.txt (regime 2) and bckup0/1.sugr backups, in the reference's formats. */
int sg_run(sg_ctx *ctx, void *fResults, const char *pdb_prefix);

/* ---- configuration (host) --------------------------------------------------------------- */
/* The 22 positional rows of sugr_in.txt (SurfaceGrowth.cpp:633-785). */
typedef struct sg_input {
    int iRegime, iMaterial;
    int ucx, ucy, ucz;
    float temperatureK;
    int nMolMe;
    float epsilonEv, sigmaA;
    int stepLimit;
    float deltaT;
    int stepAvg, stepEquil;
    float deltaFpN;
    int stepCool;
    float deposEnergyEv;
    int nMolToDeposit, stepDeposit, stepPdb, stepRdf, bBckup, bStartBckup;
    /* compiled-in globals of the reference that sugr_in.txt cannot set
     * (SurfaceGrowth.cpp:35-90); sg_default_input() gives the reference values */
    float rNebrShell;
    int iNebrMax, stepThermostat;
    float gammaBerendsen;
    int limitRdf, sizeHistRdf, nValDiffuse, nBuffDiffuse, stepDiffuse, limitDiffuseAv;
    int stepBckup, randSeed;   /* randSeed 0: time-based like the reference */
    int bPdb, bResult, bRdf;
} sg_input;
void sg_default_input(sg_input *in);
/* Parse sugr_in.txt semantics; returns SG_ERR_IO if the file cannot be opened. */
int sg_read_input_file(const char *path, sg_input *in);
/* SetParams (SurfaceGrowth.cpp:189-396) with EamInit/GrapheneInit (cpp:480-545). */
int sg_set_params(const sg_input *in, sg_simparams *p);
/* Initial coordinates (InitCoordsW cu:2532-2609 and its lattice kernels), nMol entries. */
int sg_init_coords(sg_simparams *p, sg_float4 *r);
/* Initial velocities with the reference's generator (InitVels cpp:596-621). */
int sg_init_vels(sg_simparams *p, sg_float3 *v);

/* Synthetic nanoparticle-on-graphene workload: a ucx x ucy graphene sheet (32*ucx*ucy C)
 * with n_clusters fcc metal clusters (atom-centred spheres of the given sizes) placed at
 * seeded random non-overlapping x-y positions, lowest atom clearance_A above the sheet,
 * Maxwell-Boltzmann velocities at temperatureK (FP64 counter-based generator, zero net
 * momentum).  Call with r == NULL to get the atom count in p->nMol. */
typedef struct sg_workload {
    int ucx, ucy, iMaterial;
    int n_clusters;
    const int *cluster_sizes;
    float temperatureK;
    float clearance_A;
    unsigned long long seed;
    int stepLimit, stepAvg, stepEquil, stepCool, stepRdf, limitRdf;
    int stepDiffuse, nValDiffuse, nBuffDiffuse, limitDiffuseAv;
    float deltaT;
} sg_workload;
int sg_build_workload(const sg_workload *w, sg_simparams *p, sg_float4 *r, sg_float3 *v);

/* ---- output writers (host), in the reference's formats --------------------------------------
 * These are what sg_run uses; exported so that a caller driving sg_step itself writes the
 * same files.  All take the parameter block with the Props as the step loop holds them. */
/* AccumProps (SurfaceGrowth.cu:2659-2686): icode 0 zero, 1 accumulate val, 2 average. */
void sg_accum_props(sg_simparams *p, int icode);
/* One summary row (PrintSummary, cu:2689-2731); Props must already be averaged. */
int sg_print_summary(void *fp, const sg_simparams *p);
/* Result-file name (sg + regime suffix + metal + .txt) and its header line
 * (SetupJob, SurfaceGrowth.cpp:420-469). */
int sg_result_file_name(const sg_simparams *p, char *out, int out_len);
int sg_print_result_header(void *fp, const sg_simparams *p, float deposEnergyEv);
/* sugr_<i>.pdb snapshot (CreatePdbFile, cu:2734-2810). */
int sg_create_pdb(const char *prefix, const sg_simparams *p, const sg_float4 *r);
/* rdf_stepCount_<n>_<metal>.txt (PrintRdf, cu:2812-2844); p->countRdf must equal the number
 * of samples in hist. */
int sg_print_rdf(const sg_simparams *p, const unsigned int *hist);
/* One "diffusion" table (PrintDiffusion, cu:2884-2895). */
int sg_print_diffusion(void *fp, const sg_simparams *p, const float *table);
/* Backup file bckup0/1.sugr (cu:2456-2481) and its reader (the reference parses the restart
 * flag but has no reader).  r/v/a may be NULL on read to query nMol from *p. */
int sg_write_backup(const char *path, const sg_simparams *p, const sg_float4 *r, const sg_float3 *v,
                    const sg_float3 *a);
int sg_read_backup(const char *path, sg_simparams *p, sg_float4 *r, sg_float3 *v, sg_float3 *a);

/* ---- force evaluation without device allocation ---------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc: code running
 * under another framework's memory manager that owns the device heap, code that must not
 * stall the device with the implicit synchronisation of cudaMalloc/cudaFree, plugins that may
 * not grow the device footprint per call.  Same work as sg_build_lists + sg_compute_forces on
 * one system: d_pos (nMol float4 {x,y,z,U}, device) is read and its .w receives the per-atom
 * potential energy, d_acc (nMol float4, device) receives the accelerations.  Everything else
 * lives in one static device array of SG_NOALLOC_SCRATCH_BYTES that every GPU loading the
 * library holds until the process exits; systems above the SG_NOALLOC_MAX_* limits are
 * rejected with SG_ERR_INVALID.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress), so make it before any stream capture.  That address is kept
 * for the device's primary context (the CUDA runtime's): do not call this after a
 * cudaDeviceReset, or with another driver-API context current.  All calls share the
 * array: calls that overlap on the GPU (other streams, other host threads) race and corrupt
 * each other's results.  The call synchronises `stream` (a cudaStream_t, NULL: the default
 * stream) to report device-side conditions.  It calls no cudaMalloc/cudaFree. */
#define SG_NOALLOC_MAX_ATOMS 16384
#define SG_NOALLOC_MAX_CELLS 65536   /* cell grid padded to whole scan tiles of 2048 cells */
#define SG_NOALLOC_MAX_NEBR 128      /* iNebrMax */
#define SG_NOALLOC_SCRATCH_BYTES (20u << 20)
int sg_compute_forces_noalloc(const sg_simparams *p, sg_float4 *d_pos, sg_float4 *d_acc, void *stream);

/* ---- differentiation ---------------------------------------------------------------------
 * The metal part of the model as a function of fit parameters, with its gradient from a
 * hand-written adjoint (no counterpart in the reference, which has fixed analytic potentials).
 * theta[SG_DIFF_NPARAM]:
 *   theta[0]      epsilon of the metal-carbon 12-6 Lennard-Jones term,
 *   theta[1]      its sigma (the cutoff stays the parameter block's rrCutLJ),
 *   theta[2..33]  the 32 uniform cubic B-spline coefficients of the EAM pair potential phi(r),
 *   theta[34..65] those of the EAM density function f(r),
 * both splines on SG_DIFF_SPLINE_INTERVALS equal intervals from 0.6 r_e to the EAM cutoff
 * (below 0.6 r_e the first cubic piece continues); the embedding function F(rho) is the
 * reference's analytic form.  Energy of a frame:
 *   E = sum over metal pairs (r < rCutEam) phi(r) + sum over metal atoms F(rho_i),
 *       rho_i = sum over metal neighbours (r < rCutEam) f(r),
 *     + sum over metal-carbon pairs (r < rCutLJ) 4 eps ((sigma/r)^12 - (sigma/r)^6);
 * the graphene bonded terms have no fit parameter and are left out; forces F = -grad_r E.
 * Frames are independent configurations of systems of the same kind (one parameter block per
 * frame; the frames' iNebrMax must agree).  Pair arithmetic in FP32, sums of energies, losses
 * and gradients in FP64 (through atomics: repeated calls agree to about 1e-7 relative).  The force-matching loss over all frames is
 *   L = (1 / (3 N)) sum_i |F_i(theta) - F_ref,i|^2      (N: atoms of all frames),
 * its gradient comes from the adjoint pass, which recomputes the densities instead of storing
 * them. */
#define SG_DIFF_NPARAM 66
#define SG_DIFF_SPLINE_COEFFS 32
#define SG_DIFF_SPLINE_INTERVALS 29
typedef struct sg_diff sg_diff;
/* The parameter block a frame is evaluated with: the list radius raised to cover the LJ
 * cutoff (the cell grid and iNebrMax follow), everything else as given.  Host only. */
int sg_diff_frame_params(const sg_simparams *in, sg_simparams *out);
int sg_diff_create(const sg_simparams *frame_params, int n_frames, int device, sg_diff **out);
int sg_diff_destroy(sg_diff *d);
int sg_diff_num_atoms(const sg_diff *d);
/* Positions of all frames, concatenated (float4, w ignored); builds the pair lists. */
int sg_diff_set_positions(sg_diff *d, const sg_float4 *r);
/* theta at the reference model of a parameter block: its epsilon and sigma, splines fitted by
 * least squares (FP64) to its analytic phi and f.  Host only. */
int sg_diff_init_theta(const sg_simparams *p, double *theta);
/* Energy of every frame (n_frames values) and, if grad is not NULL, dE/dtheta summed over the
 * frames. */
int sg_diff_energy(sg_diff *d, const double *theta, double *energy, double *grad);
/* Forces of all atoms of all frames (3 floats per atom). */
int sg_diff_forces(sg_diff *d, const double *theta, float *forces);
/* Force-matching loss against ref_forces (3 floats per atom, all frames) and, if grad is not
 * NULL, dL/dtheta. */
int sg_diff_force_matching(sg_diff *d, const double *theta, const float *ref_forces, double *loss,
                           double *grad);
/* A fitted theta into the simulated model: replica rep's (rep == -1: every replica's) MIXED EAM
 * tables become the B-splines phi(r) and f(r) of theta, its metal-carbon LJ epsilon and sigma
 * theta[0], theta[1]; the embedding function and the graphene terms stay.  The metal forces of
 * the context then equal sg_diff_forces(theta) on the same positions (with a list radius that
 * covers the LJ cutoff, as sg_diff_frame_params gives).  With eam_table_knots - 1 a multiple of
 * SG_DIFF_SPLINE_INTERVALS (1016, say) every table piece is a spline piece; with other knot
 * counts the table interpolates the spline.  MIXED only (SG_ERR_UNSUPPORTED in PLAIN, which
 * evaluates the reference's analytic functions). */
int sg_load_diff_theta(sg_ctx *ctx, int rep, const double *theta);

/* ---- tuning ------------------------------------------------------------------------------- */
/* Times the launch shapes of the tunable passes on the context's own state and keeps the
 * fastest: the metal lanes per atom (4, 8, 16, 32; `steps` steps each, the context's own
 * rebuild schedule), then the list build (its three forms, then for the cell-window forms the
 * home atoms per work item 4, 6, 8, 16, blocks per SM 2, 4, 8, 16 and cell order ascending or
 * descending), `steps` steps each with a rebuild in every step, then programmatic dependent
 * launch off and on, (MIXED) the EAM table read through L1 or staged in shared memory, and the
 * carbon pass's resident blocks per SM 8, 12, 16.  A
 * trial keeps the setting the context had unless another choice is more than 1% faster (each
 * timing is the faster of two runs).  Every device buffer and the host step counters are copied first
 * and put back after each trial, so the context continues from the state it had; the trials
 * change no results but the summation order of the metal passes.  `report` (if not NULL)
 * receives a JSON object with the milliseconds per step of every trial and the choice.
 * steps <= 0 selects 20. */
int sg_autotune(sg_ctx *ctx, int steps, char *report, int report_len);
/* The tunable launch shape: the options of the same names. */
typedef struct sg_launch_shape {
    int metal_lanes;        /* 4, 8, 16 or 32 */
    int nebr_blocks_per_sm; /* 1..32 */
    int nebr_descending;    /* 0 or 1 */
    int nebr_item_atoms;    /* 4..64 */
    int programmatic_launch; /* 0 or 1 */
    int nebr_build;         /* 0, 1 or 2 */
    int eam_table_smem;     /* 0 or 1 (MIXED) */
    int carbon_blocks_per_sm; /* 8, 12 or 16 */
} sg_launch_shape;
/* The launch shape in use (from the options, or as sg_autotune chose it). */
int sg_get_launch_shape(sg_ctx *ctx, sg_launch_shape *shape);
/* Sets the launch shape (a shape an earlier sg_autotune reported, for instance). */
int sg_set_launch_shape(sg_ctx *ctx, const sg_launch_shape *shape);

#ifdef __cplusplus
}
#endif
#endif /* SG_API_H */
