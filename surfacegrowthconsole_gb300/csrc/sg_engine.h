// sg_engine.h - internal: the context structure and the functions the translation units of
// libsgmd share.  Not part of the public C ABI (that is include/sg_api.h).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "sg_api.h"
#include "sg_device.cuh"

using sg::BlockTab;
using sg::RepConst;
using sg::RepState;

// ---- host-side tables ----------------------------------------------------------------------
struct DevTab {
  int *rep = nullptr, *start = nullptr;
  int n = 0;
  BlockTab view() const { return BlockTab{rep, start, n}; }
};

// The host buffers a step-from-host graph reads (replica, r, v, a).
struct HostBufs {
  int rep = -2;
  const void *r = nullptr, *v = nullptr, *a = nullptr;
  HostBufs() = default;
  HostBufs(int rep_, const void *r_, const void *v_, const void *a_) : rep(rep_), r(r_), v(v_), a(a_) {}
  bool operator==(const HostBufs &o) const { return rep == o.rep && r == o.r && v == o.v && a == o.a; }
};

struct sg_ctx {
  int nrep = 0, ntot = 0, ctot = 0, nebrMax = 128, rowStride = 128, ntiles = 0;
  sg_options opt;
  std::vector<sg_simparams> hp;  // parameters as given (mutable fields refreshed on demand)
  std::vector<RepConst> hrc;
  std::vector<int> tileFirst, redFirst, cmvFirst;
  std::vector<size_t> diffOffH;
  cudaStream_t stream = nullptr;
  bool ownStream = false;
  std::vector<void *> allocs;
  // device arrays
  RepConst *rc = nullptr;
  RepState *st = nullptr;
  float4 *pos = nullptr, *vel = nullptr, *acc = nullptr, *posLo = nullptr, *sortPos = nullptr;
  int *cellOf = nullptr, *slot = nullptr, *cellCount = nullptr, *cellStart = nullptr;
  int *tmpIdx = nullptr, *sortIdx = nullptr, *nn = nullptr, *nbl = nullptr, *ns = nullptr, *sl = nullptr;
  int *nrl = nullptr;
  unsigned *rl = nullptr;  // relevant lists (relPack entries)
  int nebrGrid = 0;
  int *activeCells = nullptr, *nebrWork = nullptr;
  int *bucket = nullptr, bucketCap = 64;  // atoms of each cell in arrival order, bucketCap slots per cell
  int *blockCount = nullptr;  // filed atoms per block of scanCells cells (zero between rebuilds)
  int2 *spill = nullptr;      // MIXED: {global cell, atom} of atoms past their cell's bucket
  int scanCells = sg::kScanCells;  // cells per block of the scan and ordering
  int nScanBlocks = 0;
  int2 *heavyItems = nullptr;
  float *rho = nullptr, *dF = nullptr, *Fv = nullptr, *fric = nullptr;
  float *partial = nullptr, *partialCmv = nullptr;
  int *dRedFirst = nullptr, *dCmvFirst = nullptr, *tileSum = nullptr, *dTileFirst = nullptr;
  unsigned *hist = nullptr;
  unsigned long long *histExt = nullptr;
  int4 *rdfPairs = nullptr;  // RDF extension: {replica, first A atom, first B atom} per tile pair
  int nRdfPairs = 0;
  int histStride = 0;
  float *diffBuf = nullptr;
  size_t *dDiffOff = nullptr;
  DevTab atomTab, metalTab, carbonTab, redTab, cmvTab, tileTab;
  DevTab metalTabT, carbonTabT;  // blocks of kMetalPerBlock / kCarbonPerBlock atoms
  DevTab rdfTab;                 // blocks of kRdfAtoms metal atoms (the RDF sample)
  // launch shape of the metal chain: lanes per atom and its block table (128 / lanes atoms per
  // block; lanes 4, 8, 16, 32 -> slot 0..3, made on first use, slot 2 is metalTabT)
  int metalLanes = sg::kMT;
  DevTab metalLaneTab[4];
  DevTab metalRun;
  int numSMs = 0, nebrBlocksPerSM = 8, nebrDescending = 0, nebrItemAtoms = sg::kItemAtoms;
  // list build: 0 cell windows, warp-placed hits (k_build_nebr); 1 atom threads
  // (k_build_nebr_atoms); 2 cell windows, lane-placed hits (k_build_nebr_lanes)
  int nebrAlgo = 0;
  bool eamStaged = false;  // MIXED: metal passes with the EAM table staged in shared memory
  bool pdl = false;  // programmatic dependent launch between the kernels of a step
  // the device reads any host memory through the host's page tables (address translation
  // services, as over NVLink-C2C): state uploads read the caller's arrays in place, pageable
  // or page-locked, with no pointer queries and no copies
  bool hostDirect = false;
  int carbonBlocks = 8;  // carbon pass: resident blocks per SM of its register budget (8, 12, 16)
  // persistent step (MIXED): one cooperative launch per step, grid barriers between phases
  bool persistent = false;
  int persistGrid = 0;
  unsigned *persistBar = nullptr;   // {arrived, generation} of the grid barrier
  long long persistWaitCycles = 0;  // longest barrier wait, SM clock cycles
  std::vector<std::pair<void *, size_t>> regions;  // every device buffer with its size
  int anyMetal = 0, anyCarbon = 0, maxHist = 0;
  // graphs keyed by variant bits (with G_FROM_HOST: upload from hostGraphBufs, step, publish)
  std::map<int, cudaGraphExec_t> graphs;
  HostBufs hostGraphBufs;
  // host mirror of the schedule
  int stepCount = 0;
  int countRdf = 0;
  std::vector<sg_prop> oneStep;  // per replica, host-accumulated step times
  void *mixed = nullptr;         // MIXED-mode buffers (sg_kernels_mixed.cu)
  float *stage = nullptr;        // 6 floats per atom: two host float3 arrays in transit
  RepState *hostSt = nullptr;    // pinned host mirror of the replica states (read with sg_step)
  volatile unsigned *hostSeq = nullptr;  // pinned, after the mirror: the last published sequence number
  unsigned *devSeq = nullptr;    // its device-side counter, then the publish's block count (not a snapshot region)
  unsigned pubSeq = 0;           // the number the host expects next
  cudaEvent_t phaseEv[9] = {};   // phase boundaries of a step (phase_timing)
  cudaStream_t side = nullptr;   // second stream: the metal force chain runs beside the carbon pass
  cudaEvent_t evFork = nullptr, evJoin = nullptr;
  int launchCount = 0;           // kernel launches counted while enqueueing a step
  std::map<int, int> kernelsPerVariant;
  int lastVariant = 0;
};


int sg_fail(int code, const char *fmt, ...);

int sg_read_state(sg_ctx *c, int rep, sg::RepState *out);
int sg_get_diffusion_print(sg_ctx *c, int rep, float *table, int *nprints);
int sg_next_variant(sg_ctx *c);
int sg_launch_step(sg_ctx *c, int variant, bool *rdfPrint);
int sg_check_flags(sg_ctx *c);

// MIXED mode (sg_kernels_mixed.cu)
int sg_mixed_init(sg_ctx *c);
void sg_mixed_free(sg_ctx *c);
// the MIXED integrator; with host arrays (all replicas, hostR 16-byte aligned, read in place)
// the step starts from them instead of the device state, as after an upload
int sg_mixed_enqueue_integrate(sg_ctx *c, int forceRebuild, const sg_float4 *hostR = nullptr,
                               const sg_float3 *hostV = nullptr, const sg_float3 *hostA = nullptr);
int sg_mixed_enqueue_forces(sg_ctx *c);
// registers a buffer the library allocated outside devAlloc (autotuner snapshots)
void sg_register_region(sg_ctx *c, void *p, size_t bytes);
// the MIXED reduction; publish: its last blocks also publish the replica states to the host
// mirror and raise the sequence number (the step's publish kernel folded in)
int sg_mixed_enqueue_reduce(sg_ctx *c, int forceRebuild, bool publish = false);
int sg_mixed_enqueue_persistent(sg_ctx *c, int forceRebuild);
int sg_mixed_persistent_blocks_per_sm(int metalLanes);
bool sg_mixed_staging_ok(sg_ctx *c);
