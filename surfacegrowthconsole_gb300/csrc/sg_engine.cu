// sg_engine.cu - context, device memory, step sequencing (CUDA graphs) and the sg_* C ABI.
//
// One step is a fixed sequence of launches, each covering every replica of the context:
//   integrate_first  (Verlet part 1 + wrap + pending thermostat + deposition + cell histogram)
//   [scan_tiles, scan_tile_prefix, scan_final, scatter, rank, build_nebr]  (rebuild; a
//        replica whose nebrNow flag is clear leaves these kernels at once)
//   rho, force_metal, force_carbon
//   cmvel, step_reduce (Verlet part 2 + all reductions + per-replica step control)
//   [shear] [rdf]    (only on steps where the host-known schedule asks for them)
// The sequence is captured once per variant into a CUDA graph and replayed, so a step costs
// one graph launch and no host synchronisation; the host reads results only at output
// points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <chrono>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "sg_api.h"
#include "sg_device.cuh"
#include "sg_engine.h"
#include "sg_kernels.h"

using namespace sg;

// ---- error plumbing ----------------------------------------------------------------------
static thread_local std::string g_err;
int sg_fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return sg_fail(e_ == cudaErrorMemoryAllocation ? SG_ERR_NOMEM : SG_ERR_CUDA, "%s: %s (%s:%d)", \
                     #call, cudaGetErrorString(e_), __FILE__, __LINE__);                      \
  } while (0)

extern "C" const char *sg_last_error(void) { return g_err.c_str(); }
extern "C" int sg_version(void) { return SG_API_VERSION; }

extern "C" void sg_default_options(sg_options *o) {
  memset(o, 0, sizeof(*o));
  o->mode = SG_MODE_PLAIN;
  o->use_graphs = 1;
  o->programmatic_launch = 1;
  o->rdf_ext_range = 0.f;
}

static int devAlloc(sg_ctx *c, void **p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return sg_fail(SG_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  c->allocs.push_back(*p);
  c->regions.emplace_back(*p, bytes);
  e = cudaMemsetAsync(*p, 0, bytes, c->stream);
  if (e != cudaSuccess) return sg_fail(SG_ERR_CUDA, "cudaMemset: %s", cudaGetErrorString(e));
  return SG_OK;
}
template <class T> static int devAllocT(sg_ctx *c, T **p, size_t n) {
  return devAlloc(c, (void **)p, n * sizeof(T));
}

static int uploadTab(sg_ctx *c, DevTab &t, const std::vector<int> &rep, const std::vector<int> &start) {
  t.n = (int)rep.size();
  int rc;
  if ((rc = devAllocT(c, &t.rep, std::max<size_t>(rep.size(), 1)))) return rc;
  if ((rc = devAllocT(c, &t.start, std::max<size_t>(start.size(), 1)))) return rc;
  if (t.n) {
    CK(cudaMemcpyAsync(t.rep, rep.data(), rep.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(t.start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  }
  return SG_OK;
}
// blocks of bs over [b, e) of each replica
static int makeRangeTab(sg_ctx *c, DevTab &t, int bs, int which) {
  std::vector<int> rep, start;
  for (int r = 0; r < c->nrep; r++) {
    const RepConst &P = c->hrc[r];
    int b = P.atomOff, e = P.atomOff + P.nMol;
    if (which == 1) e = P.atomOff + P.nMolMe;
    if (which == 2) b = P.atomOff + P.nMolMe;
    for (int s = b; s < e; s += bs) { rep.push_back(r); start.push_back(s); }
  }
  return uploadTab(c, t, rep, start);
}

// Parameters of one replica as the kernels read them.
static RepConst makeConst(const sg_simparams &p) {
  RepConst P;
  memset(&P, 0, sizeof(P));
  P.region[0] = p.region.x; P.region[1] = p.region.y; P.region[2] = p.region.z;
  P.invWidth[0] = p.invWidth.x; P.invWidth[1] = p.invWidth.y; P.invWidth[2] = p.invWidth.z;
  P.cells[0] = p.cells.x; P.cells[1] = p.cells.y; P.cells[2] = p.cells.z;
  P.ncells = p.cells.x * p.cells.y * p.cells.z;
  P.ncellsPad = ((P.ncells + 1 + kCellTile - 1) / kCellTile) * kCellTile;
  P.nMol = p.nMol;
  P.nMolMe = p.nMolMe;
  P.nRedBlocks = (p.nMol + kRedElems - 1) / kRedElems;
  P.scanCells = kScanCells;
  P.deltaT = p.deltaT;
  P.rrNebr = p.rrNebr;
  P.rNebrShell = p.rNebrShell;
  const float rs = p.rCutC + p.rNebrShell;
  P.rrShort = rs * rs;
  const float c30 = (float)cos(M_PI / 6.f);  // LeapfrogStepK, SurfaceGrowth.cu:416-421
  P.xLeft = 0.5f * (c30 - p.region.x);
  P.xRight = 0.5f * (p.region.x - c30);
  P.yBottom = 0.5f * (1.f - p.region.y);
  P.yTop = 0.5f * (p.region.y - 1.f);
  P.rei = p.rei; P.rhoei = p.rhoei; P.rhoe = p.rhoe; P.fe = p.fe; P.alpha = p.alpha;
  P.beta = p.beta; P.A = p.A; P.B = p.B; P.kappa = p.kappa; P.lambda = p.lambda;
  for (int i = 0; i < 4; i++) { P.Fn[i] = p.Fn[i]; P.F[i] = p.F[i]; }
  P.eta = p.eta; P.Fe = p.Fe; P.massMe = p.massMe; P.rrCutEam = p.rrCutEam;
  P.rrCutC = p.rrCutC; P.mu_r = p.mu_r; P.theta_0 = p.theta_0; P.mu_theta = p.mu_theta;
  P.mu_p = p.mu_p; P.z_0 = p.z_0; P.sigmaLJ = p.sigmaLJ; P.epsLJ = p.epsLJ; P.rrCutLJ = p.rrCutLJ;
  P.temperature = p.temperature; P.kB = p.kB; P.gammaBerendsen = p.gammaBerendsen;
  P.deltaF = p.deltaF; P.velMagDepos = p.velMagDepos;
  P.iRegime = p.iRegime; P.stepEquil = p.stepEquil; P.stepCool = p.stepCool;
  P.stepThermostat = p.stepThermostat > 0 ? p.stepThermostat : 1;
  P.stepDeposit = p.stepDeposit > 0 ? p.stepDeposit : 1;
  P.nMolToDeposit = p.nMolToDeposit;
  P.hasFric = (p.iRegime != 0 && p.nMolMe != 0) ? 1 : 0;
  P.rangeRdf = p.rangeRdf; P.intervalRdf = p.intervalRdf; P.sizeHistRdf = p.sizeHistRdf;
  P.bRdf = p.bRdf;
  P.nValDiffuse = p.nValDiffuse; P.nBuffDiffuse = p.nBuffDiffuse;
  P.stepDiffuse = p.stepDiffuse > 0 ? p.stepDiffuse : 1;
  P.limitDiffuseAv = p.limitDiffuseAv;
  P.stepAvg = p.stepAvg > 0 ? p.stepAvg : 1;
  P.invNMol = 1.0 / p.nMol;
  P.invNMolMe = p.nMolMe ? 1.0 / p.nMolMe : 0.0;
  P.invRegion[0] = 1.0 / p.region.x; P.invRegion[1] = 1.0 / p.region.y; P.invRegion[2] = 1.0 / p.region.z;
  return P;
}

static int validate(const sg_simparams *p, int n) {
  for (int r = 0; r < n; r++) {
    const sg_simparams &q = p[r];
    if (q.nMol <= 0 || q.nMolMe < 0 || q.nMolMe > q.nMol)
      return sg_fail(SG_ERR_INVALID, "replica %d: bad atom counts nMol=%d nMolMe=%d", r, q.nMol, q.nMolMe);
    if (q.cells.x < 1 || q.cells.y < 1 || q.cells.z < 1)
      return sg_fail(SG_ERR_INVALID, "replica %d: bad cell grid", r);
    if (q.iNebrMax < 1) return sg_fail(SG_ERR_INVALID, "replica %d: iNebrMax < 1", r);
    if (q.blockSize < 1 || q.blockSize > 1024)
      return sg_fail(SG_ERR_INVALID, "replica %d: blockSize %u (atoms per cell) outside 1..1024", r, q.blockSize);
    if (q.bRdf && (q.sizeHistRdf < 1 || q.stepRdf < 1 || q.limitRdf < 1))
      return sg_fail(SG_ERR_INVALID, "replica %d: bad RDF settings", r);
    if (q.iRegime == 2 && (q.nBuffDiffuse < 1 || q.nValDiffuse < 1 || q.limitDiffuseAv < 1 || q.nBuffDiffuse > 4096))
      return sg_fail(SG_ERR_INVALID, "replica %d: bad diffusion settings", r);
    if (r > 0) {  // one host-side schedule drives all replicas
      const sg_simparams &z = p[0];
      if (q.stepRdf != z.stepRdf || q.limitRdf != z.limitRdf || q.bRdf != z.bRdf ||
          q.stepCount != z.stepCount || q.stepAvg != z.stepAvg || q.iNebrMax != z.iNebrMax)
        return sg_fail(SG_ERR_INVALID, "replica %d: schedule differs from replica 0", r);
    }
  }
  return SG_OK;
}

static void destroyGraphs(sg_ctx *c) {
  for (auto &kv : c->graphs) cudaGraphExecDestroy(kv.second);
  c->graphs.clear();
}

// Launch shape of the metal chain: lanes per metal atom and the matching block table.
static int setMetalLanes(sg_ctx *c, int lanes) {
  const int slot = lanes == 4 ? 0 : lanes == 8 ? 1 : lanes == 16 ? 2 : lanes == 32 ? 3 : -1;
  if (slot < 0) return sg_fail(SG_ERR_INVALID, "metal_lanes %d: 4, 8, 16 or 32", lanes);
  if (c->persistent && lanes != 4 && lanes != kMT)
    return sg_fail(SG_ERR_UNSUPPORTED, "metal_lanes %d: the persistent step runs 4 or %d", lanes, kMT);
  DevTab &t = c->metalLaneTab[slot];
  if (!t.rep) {
    const int rc = makeRangeTab(c, t, 128 / lanes, 1);
    if (rc) return rc;
  }
  if (lanes != c->metalLanes) destroyGraphs(c);
  c->metalLanes = lanes;
  c->metalRun = t;
  return SG_OK;
}

// Grid of the list build's work queue: blocksPerSM resident blocks per SM, no more blocks
// than there are cells for their warps.
static void setNebrBlocks(sg_ctx *c, int blocksPerSM) {
  const int g = std::max(1, std::min((c->ctot + kNebrWarps - 1) / kNebrWarps, c->numSMs * blocksPerSM));
  if (g != c->nebrGrid) destroyGraphs(c);
  c->nebrGrid = g;
  c->nebrBlocksPerSM = blocksPerSM;
}

void sg_register_region(sg_ctx *c, void *p, size_t bytes) { c->regions.emplace_back(p, bytes); }

extern "C" int sg_create(const sg_simparams *params, int n_replicas, const sg_options *opt, sg_ctx **out) {
  if (!params || n_replicas < 1 || !out) return sg_fail(SG_ERR_INVALID, "sg_create: bad arguments");
  *out = nullptr;
  int rc = validate(params, n_replicas);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return sg_fail(SG_ERR_NO_DEVICE, "no CUDA device available");
  sg_ctx *c = new sg_ctx;
  if (opt) c->opt = *opt;
  else sg_default_options(&c->opt);
  if (c->opt.mode != SG_MODE_PLAIN && c->opt.mode != SG_MODE_MIXED) {
    delete c;
    return sg_fail(SG_ERR_INVALID, "unknown mode %d", c->opt.mode);
  }
  if (cudaSetDevice(c->opt.device) != cudaSuccess) {
    delete c;
    return sg_fail(SG_ERR_NO_DEVICE, "cannot select device %d", c->opt.device);
  }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, c->opt.device);
  const int numSMs = prop.multiProcessorCount;
  if (prop.major != 10 || prop.minor != 3) {
    delete c;
    return sg_fail(SG_ERR_NO_DEVICE, "device %d is sm_%d%d; this build targets sm_103 (GB300)",
                   c->opt.device, prop.major, prop.minor);
  }
  if (c->opt.stream) c->stream = (cudaStream_t)c->opt.stream;
  else {
    cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    c->ownStream = true;
  }
  cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  cudaEventCreateWithFlags(&c->evFork, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&c->evJoin, cudaEventDisableTiming);
  c->nrep = n_replicas;
  c->hp.assign(params, params + n_replicas);
  c->nebrMax = params[0].iNebrMax;
  if (c->opt.nebr_capacity) {
    if (c->opt.mode != SG_MODE_MIXED || c->opt.nebr_capacity < c->nebrMax) {
      sg_destroy(c);
      return sg_fail(SG_ERR_INVALID, "nebr_capacity %d: MIXED mode, at least iNebrMax %d", c->opt.nebr_capacity,
                     c->nebrMax);
    }
    c->nebrMax = c->opt.nebr_capacity;
  }
  c->rowStride = (c->nebrMax + 3) & ~3;
  c->stepCount = params[0].stepCount;
  c->countRdf = params[0].countRdf;
  c->oneStep.resize(n_replicas);
  for (int r = 0; r < n_replicas; r++) c->oneStep[r] = params[r].oneStep;
  for (int r = 0; r < n_replicas; r++)
    if (params[r].nMol >= kMaxReplicaAtoms) {
      sg_destroy(c);
      return sg_fail(SG_ERR_UNSUPPORTED, "replica %d: %d atoms, at most %d per replica", r, params[r].nMol,
                     kMaxReplicaAtoms - 1);
    }
  // layout of replicas
  int atomOff = 0, cellOff = 0, redOff = 0, cmvOff = 0;
  size_t diffOff = 0;
  for (int r = 0; r < n_replicas; r++) {
    RepConst P = makeConst(params[r]);
    P.atomOff = atomOff;
    P.cellOff = cellOff;
    c->redFirst.push_back(redOff);
    c->cmvFirst.push_back(cmvOff);
    c->diffOffH.push_back(diffOff);
    atomOff += P.nMol;
    cellOff += P.ncellsPad;
    redOff += P.nRedBlocks;
    cmvOff += (P.nMolMe + kRedElems - 1) / kRedElems;
    if (params[r].iRegime == 2) diffOff += DiffLayout::floatsPerRep(P.nBuffDiffuse, P.nValDiffuse);
    c->hrc.push_back(P);
    c->anyMetal |= (P.nMolMe > 0);
    c->anyCarbon |= (P.nMol > P.nMolMe);
    c->maxHist = std::max(c->maxHist, params[r].bRdf ? params[r].sizeHistRdf : 0);
  }
  c->ntot = atomOff;
  c->ctot = cellOff;
  // Cell capacity of the counting sort.  PLAIN keeps the reference's cap of blockSize (64) atoms
  // per cell (SurfaceGrowth.h:35, cu:582-583) and reports a cell above it as SG_ERR_CELL_OVERFLOW
  // where the reference would write past its cell array.  MIXED, which is not held to that
  // limit, files up to kMixedCellCapFactor times as many atoms per cell, so a crowded cell (a hot
  // system pressing atoms together) stays in the lists.
  c->bucketCap = 1;
  for (int r = 0; r < n_replicas; r++) c->bucketCap = std::max(c->bucketCap, (int)params[r].blockSize);
  if (c->opt.mode == SG_MODE_MIXED) {
    c->bucketCap *= kMixedCellCapFactor;
    for (auto &P : c->hrc) P.uncapped = 1;
  }
  // list build: one warp per home cell, a grid of a few resident blocks per SM walking the cells
  c->numSMs = numSMs;
  c->pdl = c->opt.programmatic_launch != 0;
  {
    int pageable = 0, hostTables = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, c->opt.device);
    cudaDeviceGetAttribute(&hostTables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, c->opt.device);
    // (pageable access without the host's page tables migrates pages on first touch: not used)
    c->hostDirect = pageable == 1 && hostTables == 1;
  }
  if (c->opt.persistent_step) {
    if (c->opt.mode != SG_MODE_MIXED) {
      sg_destroy(c);
      return sg_fail(SG_ERR_UNSUPPORTED, "persistent_step: MIXED mode only");
    }
    if (c->opt.persistent_wait_us < 0) {
      sg_destroy(c);
      return sg_fail(SG_ERR_INVALID, "persistent_wait_us %d: 0 (default) or more", c->opt.persistent_wait_us);
    }
    // one launch per step: no programmatic dependent launch, the cell-window list build
    c->persistent = true;
    c->pdl = false;
    int khz = 0;
    cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, c->opt.device);
    const long long us = c->opt.persistent_wait_us ? c->opt.persistent_wait_us : 1000000;
    c->persistWaitCycles = us * (long long)std::max(khz, 1000) / 1000;
  }
  if (c->opt.nebr_blocks_per_sm < 0 || c->opt.nebr_blocks_per_sm > 32) {
    sg_destroy(c);
    return sg_fail(SG_ERR_INVALID, "nebr_blocks_per_sm %d: 0 (default) or 1..32", c->opt.nebr_blocks_per_sm);
  }
  setNebrBlocks(c, c->opt.nebr_blocks_per_sm ? c->opt.nebr_blocks_per_sm : 7);
  c->nebrDescending = c->opt.nebr_descending ? 1 : 0;
  c->nebrItemAtoms = c->opt.nebr_item_atoms ? c->opt.nebr_item_atoms : kItemAtoms;
  if (c->opt.nebr_build < 0 || c->opt.nebr_build > 2) {
    sg_destroy(c);
    return sg_fail(SG_ERR_INVALID, "nebr_build %d: 0, 1 or 2", c->opt.nebr_build);
  }
  c->nebrAlgo = c->opt.nebr_build;
  c->eamStaged = c->opt.mode == SG_MODE_MIXED && c->opt.eam_table_smem != 0;  // sg_mixed_init may clear it
  {
    const int cb = c->opt.carbon_blocks_per_sm ? c->opt.carbon_blocks_per_sm : 8;
    if (cb != 8 && cb != 12 && cb != 16) {
      sg_destroy(c);
      return sg_fail(SG_ERR_INVALID, "carbon_blocks_per_sm %d: 0 (default), 8, 12 or 16", c->opt.carbon_blocks_per_sm);
    }
    c->carbonBlocks = cb;
  }
  if (c->nebrItemAtoms < kMinItemAtoms || c->nebrItemAtoms > 64) {
    sg_destroy(c);
    return sg_fail(SG_ERR_INVALID, "nebr_item_atoms %d: 0 (default) or %d..64", c->opt.nebr_item_atoms,
                   kMinItemAtoms);
  }
  const size_t N = c->ntot;
#define AL(ptr, n)                          \
  if ((rc = devAllocT(c, &ptr, (n)))) {     \
    sg_destroy(c);                          \
    return rc;                              \
  }
  AL(c->rc, n_replicas);
  AL(c->st, n_replicas);
  AL(c->pos, N); AL(c->vel, N); AL(c->acc, N); AL(c->sortPos, N);
  if (c->opt.mode == SG_MODE_MIXED) AL(c->posLo, N);
  AL(c->cellOf, N); AL(c->slot, N); AL(c->tmpIdx, N); AL(c->sortIdx, N);
  AL(c->cellCount, (size_t)c->ctot); AL(c->cellStart, (size_t)c->ctot);
  AL(c->nn, N); AL(c->ns, N);
  AL(c->sl, N * kShortMax);
  AL(c->nbl, N * c->rowStride);
  AL(c->nrl, N);
  AL(c->rl, N * kRelMax);
  AL(c->activeCells, (size_t)c->ctot);
  // a cell of n > t atoms (t = home atoms per item >= kMinItemAtoms) gives ceil(n / t) < n / t + 1
  // items: at most N / t + N / (t + 1) in all
  AL(c->heavyItems, (size_t)N / kMinItemAtoms + (size_t)N / (kMinItemAtoms + 1) + 16);
  AL(c->nebrWork, 4);  // next item, light items, heavy items, spill-list length
  if (c->opt.mode == SG_MODE_MIXED) AL(c->spill, std::max<size_t>(N, 1));
  AL(c->bucket, (size_t)c->ctot * c->bucketCap);
  AL(c->rho, N); AL(c->dF, N); AL(c->Fv, N); AL(c->fric, N);
  AL(c->partial, (size_t)std::max(redOff, 1) * kNumRed);
  AL(c->partialCmv, (size_t)std::max(cmvOff, 1) * 3);
  AL(c->dRedFirst, n_replicas); AL(c->dCmvFirst, n_replicas);
  c->histStride = std::max(c->maxHist, 1);
  AL(c->hist, (size_t)n_replicas * c->histStride);
  if (c->opt.rdf_ext_bins > 0) AL(c->histExt, (size_t)n_replicas * c->opt.rdf_ext_bins);
  AL(c->diffBuf, std::max<size_t>(diffOff, 1));
  AL(c->dDiffOff, n_replicas);
  AL(c->stage, 6 * N);  // v and a in transit at once
  if (cudaMallocHost(&c->hostSt, sizeof(RepState) * n_replicas + 64) != cudaSuccess) {
    c->hostSt = nullptr;
    sg_destroy(c);
    return sg_fail(SG_ERR_NOMEM, "cudaMallocHost(%zu)", sizeof(RepState) * n_replicas + 64);
  }
  c->hostSeq = reinterpret_cast<volatile unsigned *>(reinterpret_cast<char *>(c->hostSt) + sizeof(RepState) * n_replicas);
  *c->hostSeq = 0u;
  // the sequence counter and, after it, the publish's count of finished blocks
  if (cudaMalloc(&c->devSeq, 2 * sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(c->devSeq, 0, 2 * sizeof(unsigned)) != cudaSuccess) {
    sg_destroy(c);
    return sg_fail(SG_ERR_NOMEM, "cudaMalloc(sequence counter)");
  }
#undef AL
  if (c->opt.phase_timing)
    for (auto &e : c->phaseEv) cudaEventCreate(&e);
  // tables
  if ((rc = makeRangeTab(c, c->atomTab, 128, 0)) || (rc = makeRangeTab(c, c->metalTab, 128, 1)) ||
      (rc = makeRangeTab(c, c->carbonTab, 128, 2)) || (rc = makeRangeTab(c, c->metalTabT, kMetalPerBlock, 1)) ||
      (rc = makeRangeTab(c, c->carbonTabT, kCarbonPerBlock, 2)) || (rc = makeRangeTab(c, c->rdfTab, kRdfAtoms, 1))) {
    sg_destroy(c);
    return rc;
  }
  c->metalLaneTab[2] = c->metalTabT;
  if ((rc = setMetalLanes(c, c->opt.metal_lanes ? c->opt.metal_lanes : kMT))) {
    sg_destroy(c);
    return rc;
  }
  if (c->persistent) {
    if (c->nebrAlgo != 0) {
      sg_destroy(c);
      return sg_fail(SG_ERR_UNSUPPORTED, "persistent_step: the cell-window list build (nebr_build 0) only");
    }
    const int bps = sg_mixed_persistent_blocks_per_sm(c->metalLanes);
    if (bps < 1) {
      sg_destroy(c);
      return sg_fail(SG_ERR_UNSUPPORTED, "persistent_step: the step kernel cannot be resident");
    }
    c->persistGrid = bps * numSMs;
    if ((rc = devAllocT(c, &c->persistBar, 2))) {
      sg_destroy(c);
      return rc;
    }
    CK(cudaMemsetAsync(c->persistBar, 0, 2 * sizeof(unsigned), c->stream));
  }
  if (c->histExt) {
    // RDF extension: every pair (A, B >= A) of 64-atom metal tiles of each replica
    std::vector<int4> pairs;
    for (int r = 0; r < n_replicas; r++) {
      const RepConst &P = c->hrc[r];
      const int nt = (P.nMolMe + kRdfTile - 1) / kRdfTile;
      for (int a = 0; a < nt; a++)
        for (int b = a; b < nt; b++)
          pairs.push_back(make_int4(r, P.atomOff + a * kRdfTile, P.atomOff + b * kRdfTile, 0));
    }
    c->nRdfPairs = (int)pairs.size();
    if ((rc = devAllocT(c, &c->rdfPairs, std::max<size_t>(pairs.size(), 1)))) {
      sg_destroy(c);
      return rc;
    }
    if (!pairs.empty() && cudaMemcpy(c->rdfPairs, pairs.data(), pairs.size() * sizeof(int4),
                                     cudaMemcpyHostToDevice) != cudaSuccess) {
      sg_destroy(c);
      return sg_fail(SG_ERR_CUDA, "upload of the RDF tile pairs");
    }
  }
  {
    std::vector<int> rr, ss, cr, cs, tr, ts;
    for (int r = 0; r < n_replicas; r++) {
      const RepConst &P = c->hrc[r];
      for (int b = 0; b < P.nRedBlocks; b++) { rr.push_back(r); ss.push_back(b); }
      for (int b = 0; b < (P.nMolMe + kRedElems - 1) / kRedElems; b++) { cr.push_back(r); cs.push_back(b); }
      c->tileFirst.push_back((int)tr.size());
      for (int t = 0; t < P.ncellsPad; t += kCellTile) { tr.push_back(r); ts.push_back(t); }
    }
    c->ntiles = (int)tr.size();
    // cells per scan block: 2 kScanCells when that still gives two blocks per SM (large and
    // batched systems: fewer, fuller blocks), else kScanCells
    c->scanCells = (!c->persistent && (long long)c->ntiles * (kCellTile / (2 * kScanCells)) >= 2LL * std::max(numSMs, 1))
                       ? 2 * kScanCells : kScanCells;
    for (auto &P : c->hrc) P.scanCells = c->scanCells;
    c->nScanBlocks = c->ntiles * (kCellTile / c->scanCells);
    if ((rc = uploadTab(c, c->redTab, rr, ss)) || (rc = uploadTab(c, c->cmvTab, cr, cs)) ||
        (rc = uploadTab(c, c->tileTab, tr, ts))) {
      sg_destroy(c);
      return rc;
    }
    if ((rc = devAllocT(c, &c->tileSum, std::max<size_t>(tr.size(), 1))) ||
        (rc = devAllocT(c, &c->dTileFirst, n_replicas)) ||
        (rc = devAllocT(c, &c->blockCount, std::max<size_t>(tr.size() * (kCellTile / kScanCells), 1)))) {
      sg_destroy(c);
      return rc;
    }
  }
  // constants, initial state
  std::vector<RepState> hs(n_replicas);
  for (int r = 0; r < n_replicas; r++) {
    const sg_simparams &p = params[r];
    RepState &S = hs[r];
    memset(&S, 0, sizeof(S));
    S.stepCount = p.stepCount;
    S.nebrNow = 1;  // lists do not exist yet
    S.dispHi = p.dispHi;
    S.shear = p.shear;
    S.totalShear = p.totalShear;
    S.nMolDeposited = p.nMolDeposited;
    S.countRdf = p.countRdf;
    const sg_prop *pp[7] = {&p.totEnergy, &p.potEnergy, &p.kinEnergy, &p.oneStep,
                            &p.centerOfMass, &p.cmVel, &p.frictForce};
    for (int k = 0; k < 7; k++) {
      S.props[k][0] = pp[k]->val; S.props[k][1] = pp[k]->sum; S.props[k][2] = pp[k]->sum2;
    }
    S.countDiffuseAv = p.countDiffuseAv;
  }
  cudaError_t e = cudaMemcpyAsync(c->rc, c->hrc.data(), sizeof(RepConst) * n_replicas, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->st, hs.data(), sizeof(RepState) * n_replicas, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->dRedFirst, c->redFirst.data(), sizeof(int) * n_replicas, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->dCmvFirst, c->cmvFirst.data(), sizeof(int) * n_replicas, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->dTileFirst, c->tileFirst.data(), sizeof(int) * n_replicas, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->dDiffOff, c->diffOffH.data(), sizeof(size_t) * n_replicas, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) {
    sg_destroy(c);
    return sg_fail(SG_ERR_CUDA, "upload: %s", cudaGetErrorString(e));
  }
  // diffusion buffer counts start staggered (InitDiffusion, SurfaceGrowth.cu:2868-2871)
  for (int r = 0; r < n_replicas; r++) {
    const sg_simparams &p = params[r];
    if (p.iRegime != 2) continue;
    std::vector<float> tb((size_t)p.nBuffDiffuse * 7, 0.f);
    for (int nb = 0; nb < p.nBuffDiffuse; nb++) {
      int cnt = -nb * p.nValDiffuse / p.nBuffDiffuse;
      memcpy(&tb[7 * nb], &cnt, sizeof(int));
    }
    e = cudaMemcpyAsync(c->diffBuf + c->diffOffH[r], tb.data(), tb.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
      sg_destroy(c);
      return sg_fail(SG_ERR_CUDA, "upload: %s", cudaGetErrorString(e));
    }
  }
  if (c->opt.mode == SG_MODE_MIXED) {
    rc = sg_mixed_init(c);
    if (rc) {
      sg_destroy(c);
      return rc;
    }
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    sg_destroy(c);
    return sg_fail(SG_ERR_CUDA, "create: %s", cudaGetErrorString(e));
  }
  *out = c;
  return SG_OK;
}

extern "C" int sg_destroy(sg_ctx *c) {
  if (!c) return SG_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  destroyGraphs(c);
  sg_mixed_free(c);
  for (auto &e : c->phaseEv)
    if (e) cudaEventDestroy(e);
  for (void *p : c->allocs) cudaFree(p);
  if (c->hostSt) cudaFreeHost(c->hostSt);
  if (c->devSeq) cudaFree(c->devSeq);
  if (c->side) cudaStreamSynchronize(c->side);
  if (c->evFork) cudaEventDestroy(c->evFork);
  if (c->evJoin) cudaEventDestroy(c->evJoin);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->ownStream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return SG_OK;
}

extern "C" int sg_num_replicas(const sg_ctx *c) { return c ? c->nrep : 0; }
extern "C" int sg_num_atoms(const sg_ctx *c, int rep) {
  if (!c) return 0;
  if (rep < 0) return c->ntot;
  return (rep < c->nrep) ? c->hrc[rep].nMol : 0;
}
extern "C" int sg_num_cells(const sg_ctx *c, int rep) {
  return (c && rep >= 0 && rep < c->nrep) ? c->hrc[rep].ncells : 0;
}

static int repRange(sg_ctx *c, int rep, int &off, int &n) {
  if (rep < 0) { off = 0; n = c->ntot; return SG_OK; }
  if (rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "replica %d out of range", rep);
  off = c->hrc[rep].atomOff;
  n = c->hrc[rep].nMol;
  return SG_OK;
}

// Host float4 arrays have the device layout and are copied directly; float3 arrays go through
// a device staging buffer and a widening kernel.  With pinned host buffers every copy is a
// single DMA transfer.
// slot 0 or 1: which half of the staging buffer (3 floats per atom each)
static int download3(sg_ctx *c, const float4 *d, sg_float3 *h, int n) {
  k_pack3<<<(n + 255) / 256, 256, 0, c->stream>>>(d, c->stage, n);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(h, c->stage, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SG_OK;
}

// The device address of a host array the GPU can read in place (page-locked, mapped into the
// unified address space: cudaMallocHost, cudaHostAlloc, cudaHostRegister), else nullptr.
static const void *mappedHost(const void *h) {
  if (!h) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
    cudaGetLastError();  // not a pointer the runtime knows: an ordinary host array
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// A state upload, enqueued.  Where the device reads host memory through the host's page tables
// (a GB300 on NVLink-C2C), the host arrays are read in place by one kernel whatever their
// allocation: no pointer queries, no copy-engine transfer (a kernel reads the 1.82 MB of a
// 45,546-atom state in 13.7 us from pageable memory, 13.5 us from page-locked memory).
// Elsewhere page-locked arrays are read in place and others are copied first, r straight into
// pos, v and a into the staging buffer.  The same kernel unpacks v and a to float4, clears the
// low position words and cancels any thermostat rescale still pending from the previous step.
// The host arrays must stay valid until the stream has passed the kernel.
static int enqueueSetState(sg_ctx *c, int rep, const sg_float4 *r, const sg_float3 *v, const sg_float3 *a) {
  int off, n, rc;
  if ((rc = repRange(c, rep, off, n))) return rc;
  const float4 *sr;
  const float *sv, *sa;
  if (c->hostDirect) {
    // read in place through the host's page tables; r as float4 rows only when 16-byte aligned
    // (else copied first), v and a row by row at any 4-byte alignment
    sr = (reinterpret_cast<uintptr_t>(r) & 15) == 0 ? reinterpret_cast<const float4 *>(r) : nullptr;
    sv = reinterpret_cast<const float *>(v);
    sa = reinterpret_cast<const float *>(a);
  } else {
    sr = static_cast<const float4 *>(mappedHost(r));
    sv = static_cast<const float *>(mappedHost(v));
    sa = static_cast<const float *>(mappedHost(a));
  }
  if (r && !sr) CK(cudaMemcpyAsync(c->pos + off, r, (size_t)n * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
  if (v && !sv) {
    CK(cudaMemcpyAsync(c->stage, v, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    sv = c->stage;
  }
  if (a && !sa) {
    float *st = c->stage + 3 * (size_t)c->ntot;
    CK(cudaMemcpyAsync(st, a, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    sa = st;
  }
  const int m = std::max(n, c->nrep);
  k_unpack_state<<<(m + kUnpackAtoms - 1) / kUnpackAtoms, kUnpackAtoms, 0, c->stream>>>(
      sr, sv, sa, c->pos + off, c->vel + off, c->acc + off, (r && c->posLo) ? c->posLo + off : nullptr, n, c->st,
      c->nrep);
  CK(cudaGetLastError());
  return SG_OK;
}

extern "C" int sg_set_state(sg_ctx *c, int rep, const sg_float4 *r, const sg_float3 *v, const sg_float3 *a) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  const int rc = enqueueSetState(c, rep, r, v, a);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return SG_OK;
}

static int applyPending(sg_ctx *c) {
  if (c->atomTab.n) {
    k_apply_pending<<<c->atomTab.n, 128, 0, c->stream>>>(c->atomTab.view(), c->rc, c->st, c->vel);
    k_clear_pending<<<(c->nrep + 127) / 128, 128, 0, c->stream>>>(c->st, c->nrep);
    CK(cudaGetLastError());
  }
  return SG_OK;
}

extern "C" int sg_get_state(sg_ctx *c, int rep, sg_float4 *r, sg_float3 *v, sg_float3 *a) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  int off, n, rc;
  if ((rc = repRange(c, rep, off, n))) return rc;
  if (v && (rc = applyPending(c))) return rc;
  if (r) CK(cudaMemcpyAsync(r, c->pos + off, (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
  if (v && (rc = download3(c, c->vel + off, v, n))) return rc;
  if (a && (rc = download3(c, c->acc + off, a, n))) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return SG_OK;
}

// ---- launch sequences ---------------------------------------------------------------------
// graph keys: a step variant, | G_FROM_HOST (upload from hostGraphBufs, step, publish) or
// | G_PUBLISH (a step whose reduction publishes the replica states)
enum { V_SHEAR = 1, V_RDF = 2, V_RDF_ZERO = 4, G_FROM_HOST = 256, G_PUBLISH = 512 };

#define LAUNCH_OK() CK(cudaGetLastError())

static int enqueueRebuild(sg_ctx *c, int force) {
  const int fr = force;
  CK(launchScanRank(c->pdl, c->scanCells, c->nScanBlocks, c->stream, c->tileTab.rep, c->tileTab.start,
             c->dTileFirst, c->rc, c->st, c->cellCount, c->cellStart, c->bucketCap, fr, c->activeCells,
             c->heavyItems, c->nebrWork, c->nebrItemAtoms, c->blockCount, c->bucket, c->spill, c->cellOf, c->pos,
             c->sortIdx, c->sortPos, c->nn, c->ns, c->nrl));
  if (c->opt.phase_timing) cudaEventRecordWithFlags(c->phaseEv[8], c->stream, cudaEventRecordExternal);
  if (c->nebrAlgo == 1)
    CK(launchK(c->pdl, k_build_nebr_atoms, c->atomTab.n, 128, 0, c->stream, c->atomTab.view(), c->rc, c->st,
               c->cellOf, c->cellStart, c->sortPos, c->nn, c->nbl, c->ns, c->sl, c->nrl, c->rl, c->rowStride,
               c->nebrMax, c->nebrWork, fr, c->blockCount, c->nScanBlocks));
  else
    CK(launchK(c->pdl, c->nebrAlgo == 2 ? k_build_nebr_lanes : k_build_nebr, c->nebrGrid, kNebrWarps * 32, 0,
               c->stream, c->tileTab.rep, c->activeCells,
               c->heavyItems, c->nebrWork, c->rc, c->st, c->cellStart, c->sortPos, c->nn, c->nbl, c->ns, c->sl,
               c->nrl, c->rl, c->rowStride, c->nebrMax, c->nebrDescending, c->blockCount, c->nScanBlocks));
  return SG_OK;
}

// Forces: the carbon pass on the main stream, the metal chain (density, metal forces and, in
// a step, the metal centre-of-mass velocity) on the side stream; both join before the
// reduction.  Inside a capture the fork and join become graph edges.
static int enqueueForces(sg_ctx *c, bool withCmVel) {
  if (c->opt.mode == SG_MODE_MIXED) return sg_mixed_enqueue_forces(c);
  const bool fork = c->metalRun.n > 0;
  if (fork) {
    CK(cudaEventRecord(c->evFork, c->stream));
    CK(cudaStreamWaitEvent(c->side, c->evFork, 0));
    launchMetalChain(c->pdl, c->metalLanes, c->metalRun.n, 0, 0, c->side, c->metalRun.view(), c->rc, c->pos, c->acc, c->nn,
                     c->nbl, c->rho, c->dF, c->Fv, c->fric, c->rowStride);
    if (withCmVel && c->cmvTab.n)
      CK(launchK(c->pdl, k_cmvel, c->cmvTab.n, kRedThreads, 0, c->side, c->cmvTab.view(), c->rc, c->st, c->vel, c->acc,
                                                        c->partialCmv, c->dCmvFirst));
    if (c->opt.phase_timing) cudaEventRecordWithFlags(c->phaseEv[7], c->side, cudaEventRecordExternal);
    LAUNCH_OK();
  }
  if (c->carbonTabT.n)
    CK(launchCarbon(c->pdl, c->carbonBlocks, c->carbonTabT.n, c->stream, c->carbonTabT.view(), c->rc, c->pos, c->acc,
                    c->nn, c->nbl, c->ns, c->sl, c->nrl, c->rl, c->rowStride));
  if (c->opt.phase_timing) cudaEventRecordWithFlags(c->phaseEv[3], c->stream, cudaEventRecordExternal);
  LAUNCH_OK();
  if (fork) {
    CK(cudaEventRecord(c->evJoin, c->side));
    CK(cudaStreamWaitEvent(c->stream, c->evJoin, 0));
  } else if (c->opt.phase_timing) {
    cudaEventRecordWithFlags(c->phaseEv[7], c->stream, cudaEventRecordExternal);
  }
  return SG_OK;
}

static int enqueueRdf(sg_ctx *c, bool zero) {
  if (zero) {
    CK(cudaMemsetAsync(c->hist, 0, sizeof(unsigned) * c->nrep * c->histStride, c->stream));
    if (c->histExt)
      CK(cudaMemsetAsync(c->histExt, 0, sizeof(unsigned long long) * c->nrep * c->opt.rdf_ext_bins, c->stream));
  }
  if (c->rdfTab.n && c->maxHist > 0) {
    CK(launchK(c->pdl, k_rdf, c->rdfTab.n, 32 * kRdfAtoms, c->maxHist * sizeof(unsigned), c->stream,
               c->rdfTab.view(), c->rc, c->st, c->pos, c->cellOf, c->cellStart, c->sortIdx, c->hist, c->histStride));
    LAUNCH_OK();
  }
  if (c->histExt && c->nRdfPairs) {
    CK(launchK(c->pdl, k_rdf_ext, c->nRdfPairs, kRdfTile, c->opt.rdf_ext_bins * sizeof(unsigned), c->stream,
               c->rc, c->pos, c->rdfPairs, c->histExt, c->opt.rdf_ext_bins, c->opt.rdf_ext_range));
    LAUNCH_OK();
  }
  return SG_OK;
}

// External records: inside a stream capture they become event-record nodes of the graph
// (a plain record would only express a dependency between captured streams).
static void phaseMark(sg_ctx *c, int k) {
  if (c->opt.phase_timing) cudaEventRecordWithFlags(c->phaseEv[k], c->stream, cudaEventRecordExternal);
}

// One step, enqueued; with host arrays (MIXED, all replicas) the integrator starts from them.
// hostR/V/A (MIXED, all replicas): the integrator reads the step's state from these host arrays.
// publish: the reduction's last blocks publish the replica states (no publish kernel).
static int enqueueStep(sg_ctx *c, int variant, const sg_float4 *hostR = nullptr, const sg_float3 *hostV = nullptr,
                       const sg_float3 *hostA = nullptr, bool publish = false) {
  int rc;
  const int fr = c->opt.force_rebuild ? 1 : 0;
  if (c->persistent) {
    // the whole step in one cooperative launch, then the optional phases
    if ((rc = sg_mixed_enqueue_persistent(c, fr))) return rc;
    if ((variant & V_SHEAR) && c->metalTab.n) {
      CK(launchK(false, k_shear, c->metalTab.n, 128, 0, c->stream, c->metalTab.view(), c->rc, c->st, c->pos, c->acc));
      LAUNCH_OK();
    }
    if (variant & V_RDF) {
      if ((rc = enqueueRdf(c, (variant & V_RDF_ZERO) != 0))) return rc;
    }
    return SG_OK;
  }
  phaseMark(c, 0);
  if (c->opt.mode == SG_MODE_MIXED) {
    if ((rc = sg_mixed_enqueue_integrate(c, fr, hostR, hostV, hostA))) return rc;
  } else {
    CK(launchK(c->pdl, k_integrate_first, c->atomTab.n, 128, 0, c->stream, c->atomTab.view(), c->rc, c->st, c->pos,
               c->vel, c->acc, c->cellOf, c->slot, c->cellCount, fr, c->bucket, c->bucketCap,
               c->blockCount));
    LAUNCH_OK();
  }
  phaseMark(c, 1);
  if ((rc = enqueueRebuild(c, fr))) return rc;
  phaseMark(c, 2);
  if ((rc = enqueueForces(c, true))) return rc;
  phaseMark(c, 4);
  if (c->opt.mode == SG_MODE_MIXED) {
    if ((rc = sg_mixed_enqueue_reduce(c, fr, publish))) return rc;
  } else {
    CK(launchK(c->pdl, k_step_reduce, c->redTab.n, kRedThreads, 0, c->stream, c->redTab.view(), c->rc, c->st, c->pos, c->vel, c->acc,
                                                              c->fric, c->partial, c->dRedFirst, c->diffBuf,
                                                              c->dDiffOff, fr,
                                                              publish ? PublishArgs{c->hostSt, c->devSeq, c->hostSeq, c->nrep}
                                                                      : PublishArgs{}));
    LAUNCH_OK();
  }
  phaseMark(c, 5);
  if ((variant & V_SHEAR) && c->metalTab.n) {
    CK(launchK(c->pdl, k_shear, c->metalTab.n, 128, 0, c->stream, c->metalTab.view(), c->rc, c->st, c->pos, c->acc));
    LAUNCH_OK();
  }
  if (variant & V_RDF) {
    if ((rc = enqueueRdf(c, (variant & V_RDF_ZERO) != 0))) return rc;
  }
  phaseMark(c, 6);
  return SG_OK;
}

// Kernel launches of one step variant, counted from the graph that holds it.
static int countKernels(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return -1;
  std::vector<cudaGraphNode_t> nodes(n);
  cudaGraphGetNodes(g, nodes.data(), &n);
  int k = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
  }
  return k;
}

// Which optional phases the coming step needs (host-known schedule, SurfaceGrowth.cu:2398-2429).
static int stepVariant(sg_ctx *c) {
  const int sc = c->stepCount + 1;
  int v = 0;
  for (int r = 0; r < c->nrep; r++) {
    const sg_simparams &p = c->hp[r];
    if (p.iRegime == 2 && p.nMolMe != 0 && sc > p.stepEquil + p.stepCool) v |= V_SHEAR;
  }
  const sg_simparams &p0 = c->hp[0];
  if (p0.bRdf && (sc % p0.stepRdf == 0)) {
    v |= V_RDF;
    if (c->countRdf == 0) v |= V_RDF_ZERO;
  }
  return v;
}

static void advanceSchedule(sg_ctx *c, int variant, bool *rdfPrint) {
  c->stepCount++;
  if (rdfPrint) *rdfPrint = false;
  if (variant & V_RDF) {
    c->countRdf++;
    if (c->countRdf == c->hp[0].limitRdf) {
      if (rdfPrint) *rdfPrint = true;
      c->countRdf = 0;
    }
  }
}

// variant | G_PUBLISH: the step's reduction also publishes the replica states.
static int launchStep(sg_ctx *c, int variant) {
  const bool publish = (variant & G_PUBLISH) != 0;
  const int v = variant & ~G_PUBLISH;
  if (!c->opt.use_graphs || c->persistent) {  // the persistent step is one launch: no graph
    c->lastVariant = variant;
    if (c->persistent) c->kernelsPerVariant[variant] = 1 + ((variant & V_SHEAR) ? 1 : 0) +
                                                       ((variant & V_RDF) ? 1 + (c->histExt ? 1 : 0) : 0);
    return enqueueStep(c, v, nullptr, nullptr, nullptr, publish);
  }
  auto it = c->graphs.find(variant);
  if (it == c->graphs.end()) {
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueueStep(c, v, nullptr, nullptr, nullptr, publish);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc) {
      if (e == cudaSuccess) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return sg_fail(SG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    c->kernelsPerVariant[variant] = countKernels(g);
    cudaGraphExec_t ex;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return sg_fail(SG_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    it = c->graphs.emplace(variant, ex).first;
  }
  CK(cudaGraphLaunch(it->second, c->stream));
  c->lastVariant = variant;
  return SG_OK;
}

// Sticky device error bits -> status code (first set bit wins).
static int checkFlags(sg_ctx *c) {
  std::vector<RepState> hs(c->nrep);
  CK(cudaMemcpyAsync(hs.data(), c->st, sizeof(RepState) * c->nrep, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  int flags = 0;
  for (auto &s : hs) flags |= s.flags;
  if (!flags) return SG_OK;
  // a persistent step that gave up at a grid barrier left its counter mid-count
  if ((flags & (1 << SG_ERR_TIMEOUT)) && c->persistBar)
    CK(cudaMemsetAsync(c->persistBar, 0, 2 * sizeof(unsigned), c->stream));
  // report once, then clear
  for (int r = 0; r < c->nrep; r++) hs[r].flags = 0;
  int zero = 0;
  for (int r = 0; r < c->nrep; r++)
    CK(cudaMemcpyAsync(&c->st[r].flags, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int code = 1; code < 31; code++)
    if (flags & (1 << code))
      return sg_fail(code, "device reported condition %d (see sg_get_diag)", code);
  return SG_OK;
}

static void thermoFromState(sg_ctx *c, int rep, const RepState &S, sg_thermo *t);

// Flags of the replica states already copied to the host mirror: status, clearing them on the
// device (rare) as checkFlags does.
static int flagsFromMirror(sg_ctx *c) {
  int flags = 0;
  for (int r = 0; r < c->nrep; r++) flags |= c->hostSt[r].flags;
  return flags ? checkFlags(c) : SG_OK;
}

// The replica states to the page-locked mirror (flags, and sg_step_thermo's record), followed by
// a sequence number the host polls for (waitPublished).
static int enqueuePublish(sg_ctx *c) {
  const int nwords = (int)(sizeof(RepState) * c->nrep / 4);
  // a block per 1,024 words (a few replicas), at most 64: many replicas cross the host link in
  // parallel, one replica in one block
  const int blocks = std::max(1, std::min(64, (nwords + 1023) / 1024));
  k_publish_state<<<blocks, 256, 0, c->stream>>>(reinterpret_cast<const int *>(c->st),
                                                 reinterpret_cast<int *>(c->hostSt), nwords, c->devSeq, c->hostSeq,
                                                 c->devSeq + 1);
  CK(cudaGetLastError());
  return SG_OK;
}

// The host's wait for the publish just enqueued: a stream synchronisation's wake-up costs more
// than polling the sequence number.  After 5 ms of polling (long batches of steps, or a failed
// launch) the host synchronises the stream instead, which also reports any error.
static int waitPublished(sg_ctx *c) {
  const unsigned want = ++c->pubSeq;
  const auto t0 = std::chrono::steady_clock::now();
  bool seen = false;
  // The sequence number is read with acquire semantics: the mirror's words are plain loads, and
  // on a weakly ordered host (the Grace CPU of a GB300 node is Arm) nothing else would stop them
  // from being satisfied before the sequence load and returning the previous publish.  The
  // device side stores the words, fences system-wide, then stores the sequence number.
  const unsigned *seqp = const_cast<const unsigned *>(c->hostSeq);
  for (unsigned spin = 0;; spin++) {
    if (__atomic_load_n(seqp, __ATOMIC_ACQUIRE) == want) {
      seen = true;
      break;
    }
    if ((spin & 1023u) == 1023u && std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(5)) break;
  }
  if (!seen) {
    CK(cudaStreamSynchronize(c->stream));
    if (__atomic_load_n(seqp, __ATOMIC_ACQUIRE) != want) return sg_fail(SG_ERR_CUDA, "step results not published");
  }
  return flagsFromMirror(c);
}

// The steps, then the replica states published to the host mirror.  When the last step has no
// shear or RDF work (nothing after its reduction), that reduction publishes them; otherwise the
// publish kernel runs after the steps (and alone for nsteps = 0).
extern "C" int sg_step(sg_ctx *c, int nsteps) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  bool published = false;
  for (int s = 0; s < nsteps; s++) {
    const int v = stepVariant(c);
    const bool pub = s == nsteps - 1 && !c->persistent && c->redTab.n > 0 && !(v & (V_SHEAR | V_RDF));
    int rc = launchStep(c, pub ? (v | G_PUBLISH) : v);
    if (rc) return rc;
    advanceSchedule(c, v, nullptr);
    published = pub;
  }
  if (!published) {
    const int rc = enqueuePublish(c);
    if (rc) return rc;
  }
  return waitPublished(c);
}

extern "C" long long sg_step_readback_bytes(const sg_ctx *c) {
  return c ? (long long)sizeof(RepState) * c->nrep : 0;
}

extern "C" int sg_step_thermo(sg_ctx *c, int nsteps, int rep, sg_thermo *t) {
  if (!c || !t || rep < 0 || rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "sg_step_thermo: bad arguments");
  const int rc = sg_step(c, nsteps);
  if (rc) return rc;
  thermoFromState(c, rep, c->hostSt[rep], t);
  return SG_OK;
}

// One step from host buffers as one graph launch: the upload, the step's kernels and the
// publish.  In MIXED with all replicas uploaded the integrator reads the buffers itself (no
// upload kernel; otherwise the upload kernel runs first), and in a step without shear or RDF
// work (nothing after the reduction) the reduction's last blocks publish the states themselves
// (no publish kernel; otherwise the publish kernel runs last).  The graph holds the buffers'
// addresses only (read when it runs, through the host's page tables), so calls with the same
// buffers -- a caller's loop -- replay it; other buffers replace the context's graphs of this
// kind.
static int launchStepFromHost(sg_ctx *c, int rep, const sg_float4 *r, const sg_float3 *v, const sg_float3 *a,
                              int variant) {
  const HostBufs key{rep, r, v, a};
  if (!(key == c->hostGraphBufs)) {
    for (auto it = c->graphs.begin(); it != c->graphs.end();) {
      if (it->first & G_FROM_HOST) {
        cudaGraphExecDestroy(it->second);
        it = c->graphs.erase(it);
      } else {
        ++it;
      }
    }
    c->hostGraphBufs = key;
  }
  const int gk = variant | G_FROM_HOST;
  auto it = c->graphs.find(gk);
  if (it == c->graphs.end()) {
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const bool fused = c->opt.mode == SG_MODE_MIXED && rep == -1;
    const bool pubInReduce = c->redTab.n > 0 && !(variant & (V_SHEAR | V_RDF));
    int rc = fused ? SG_OK : enqueueSetState(c, rep, r, v, a);
    if (!rc)
      rc = fused ? enqueueStep(c, variant, r, v, a, pubInReduce)
                 : enqueueStep(c, variant, nullptr, nullptr, nullptr, pubInReduce);
    if (!rc && !pubInReduce) rc = enqueuePublish(c);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc) {
      if (e == cudaSuccess) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return sg_fail(SG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    c->kernelsPerVariant[gk] = countKernels(g);  // the upload (if any) and the publish included
    cudaGraphExec_t ex;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return sg_fail(SG_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    it = c->graphs.emplace(gk, ex).first;
  }
  CK(cudaGraphLaunch(it->second, c->stream));
  c->lastVariant = gk;
  return SG_OK;
}

extern "C" int sg_step_from_host(sg_ctx *c, int rep, const sg_float4 *r, const sg_float3 *v, const sg_float3 *a,
                                 int nsteps, int thermo_rep, sg_thermo *t) {
  if (!c || (t && (thermo_rep < 0 || thermo_rep >= c->nrep)) || nsteps < 0)
    return sg_fail(SG_ERR_INVALID, "sg_step_from_host: bad arguments");
  int rc;
  if (nsteps == 1 && c->hostDirect && c->opt.use_graphs && !c->persistent && r && v && a &&
      (reinterpret_cast<uintptr_t>(r) & 15) == 0) {
    int off, n;
    if ((rc = repRange(c, rep, off, n))) return rc;
    const int variant = stepVariant(c);
    if ((rc = launchStepFromHost(c, rep, r, v, a, variant))) return rc;
    advanceSchedule(c, variant, nullptr);
    if ((rc = waitPublished(c))) return rc;
    if (t) thermoFromState(c, thermo_rep, c->hostSt[thermo_rep], t);
    return SG_OK;
  }
  rc = enqueueSetState(c, rep, r, v, a);
  if (rc) return rc;
  // the upload, the steps and the state records back in one synchronisation
  if ((rc = sg_step(c, nsteps))) return rc;
  if (t) thermoFromState(c, thermo_rep, c->hostSt[thermo_rep], t);
  return SG_OK;
}

extern "C" int sg_kernels_per_step(sg_ctx *c) {
  if (!c) return -1;
  auto it = c->kernelsPerVariant.find(c->lastVariant);
  return it == c->kernelsPerVariant.end() ? -1 : it->second;
}

// Returns the number of phases, or minus a status code.
extern "C" int sg_get_phase_times(sg_ctx *c, float *ms, int n) {
  if (!c || !c->opt.phase_timing) return -sg_fail(SG_ERR_UNSUPPORTED, "phase_timing is off");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return -sg_fail(SG_ERR_CUDA, "%s", cudaGetErrorString(e));
  // integrate, rebuild (sort + list build), metal chain (side stream), carbon pass, forces
  // (fork to join), reduce, extra, list build alone
  const int from[8] = {0, 1, 2, 2, 2, 4, 5, 8}, to[8] = {1, 2, 7, 3, 4, 5, 6, 2};
  const int np = 8;
  for (int k = 0; k < np && k < n; k++) {
    float t = 0.f;
    e = cudaEventElapsedTime(&t, c->phaseEv[from[k]], c->phaseEv[to[k]]);
    if (e != cudaSuccess) return -sg_fail(SG_ERR_CUDA, "%s", cudaGetErrorString(e));
    ms[k] = t;
  }
  return np;
}

// Launch-only stepping for timing loops (no synchronisation, no flag check).
extern "C" int sg_step_async(sg_ctx *c, int nsteps) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  for (int s = 0; s < nsteps; s++) {
    const int v = stepVariant(c);
    int rc = launchStep(c, v);
    if (rc) return rc;
    advanceSchedule(c, v, nullptr);
  }
  return SG_OK;
}

extern "C" int sg_build_lists(sg_ctx *c) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  k_cell_bucket<<<c->atomTab.n, 128, 0, c->stream>>>(c->atomTab.view(), c->rc, c->pos, c->cellOf, c->slot,
                                                     c->cellCount, c->bucket, c->bucketCap, c->blockCount,
                                                     c->spill, c->nebrWork + 3);
  LAUNCH_OK();
  int rc = enqueueRebuild(c, 1);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return checkFlags(c);
}

extern "C" int sg_compute_forces(sg_ctx *c) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  int rc = enqueueForces(c, false);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return checkFlags(c);
}

extern "C" int sg_eval_rdf(sg_ctx *c) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  int rc = enqueueRdf(c, false);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return checkFlags(c);
}

extern "C" int sg_reset_rdf(sg_ctx *c) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  CK(cudaMemsetAsync(c->hist, 0, sizeof(unsigned) * c->nrep * c->histStride, c->stream));
  if (c->histExt)
    CK(cudaMemsetAsync(c->histExt, 0, sizeof(unsigned long long) * c->nrep * c->opt.rdf_ext_bins, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SG_OK;
}

// ---- read-back ---------------------------------------------------------------------------
int sg_read_state(sg_ctx *c, int rep, RepState *out) {
  CK(cudaMemcpyAsync(out, c->st + rep, sizeof(RepState), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SG_OK;
}

extern "C" int sg_get_thermo(sg_ctx *c, int rep, sg_thermo *t) {
  if (!c || !t || rep < 0 || rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "sg_get_thermo: bad arguments");
  RepState S;
  int rc = sg_read_state(c, rep, &S);
  if (rc) return rc;
  thermoFromState(c, rep, S, t);
  return SG_OK;
}

static void thermoFromState(sg_ctx *c, int rep, const RepState &S, sg_thermo *t) {
  memset(t, 0, sizeof(*t));
  t->stepCount = S.stepCount;
  t->nebrNow = S.nebrNow;
  t->rebuilds = S.rebuilds;
  t->countRdf = c->countRdf;
  t->kinEnergy = S.ke; t->potEnergy = S.pe; t->totEnergy = S.te;
  t->vvSum = S.red[RS_VVSUM]; t->vvMax = S.red[RS_VVMAX]; t->uSum = S.red[RS_USUM]; t->dispHi = S.dispHi;
  t->vSum = sg_float3{S.red[RS_VSUM_X], S.red[RS_VSUM_Y], S.red[RS_VSUM_Z]};
  t->centerOfMass = sg_float3{S.red[RS_CM_X], S.red[RS_CM_Y], S.red[RS_CM_Z]};
  t->cmVel = sg_float3{S.cmVel[0], S.cmVel[1], S.cmVel[2]};
  t->frictForce = S.frictVal;
  const sg_simparams &p = c->hp[rep];
  if (p.nMolMe != 0)
    t->particleSize = sg_float3{S.red[RS_MAX_X] - S.red[RS_MIN_X], S.red[RS_MAX_Y] - S.red[RS_MIN_Y],
                                S.red[RS_MAX_Z] - S.red[RS_MIN_Z]};
  t->shear = S.shear;
  t->totalShear = S.totalShear;
  t->kinEnergy64 = S.ke64;
  t->potEnergy64 = S.pe64;
  t->virial64 = S.virial64;
  for (int k = 0; k < 7; k++) t->props[k] = sg_prop{S.props[k][0], S.props[k][1], S.props[k][2]};
  t->props[3] = c->oneStep[rep];
}

extern "C" int sg_get_params(sg_ctx *c, int rep, sg_simparams *out) {
  if (!c || !out || rep < 0 || rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "sg_get_params: bad arguments");
  sg_thermo t;
  int rc = sg_get_thermo(c, rep, &t);
  if (rc) return rc;
  RepState S;
  if ((rc = sg_read_state(c, rep, &S))) return rc;
  sg_simparams p = c->hp[rep];
  p.stepCount = t.stepCount;
  p.nebrNow = t.nebrNow;
  p.dispHi = t.dispHi;
  p.vSum = t.vSum;
  p.totEnergy = t.props[0]; p.potEnergy = t.props[1]; p.kinEnergy = t.props[2];
  p.oneStep = t.props[3]; p.centerOfMass = t.props[4]; p.cmVel = t.props[5]; p.frictForce = t.props[6];
  p.particleSize = t.particleSize;
  p.shear = t.shear;
  p.totalShear = t.totalShear;
  p.countRdf = c->countRdf;
  p.countDiffuseAv = S.countDiffuseAv;
  p.nMolDeposited = S.nMolDeposited;
  p.moreCycles = (p.stepCount >= p.stepLimit) ? 0 : 1;
  *out = p;
  return SG_OK;
}

template <class T> static int readArr(sg_ctx *c, T *dst, const T *src, size_t n) {
  CK(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SG_OK;
}

extern "C" int sg_get_cells(sg_ctx *c, int rep, int *cellOfOut, int *cellStartOut, int *cellAtomsOut) {
  if (!c || rep < 0 || rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "sg_get_cells: bad arguments");
  const RepConst &P = c->hrc[rep];
  int rc;
  if (cellOfOut && (rc = readArr(c, cellOfOut, c->cellOf + P.atomOff, P.nMol))) return rc;
  std::vector<int> cs(P.ncells + 1);
  if ((rc = readArr(c, cs.data(), c->cellStart + P.cellOff, P.ncells + 1))) return rc;
  if (cellStartOut)
    for (int i = 0; i <= P.ncells; i++) cellStartOut[i] = cs[i] - P.atomOff;
  if (cellAtomsOut) {
    const int nb = cs[P.ncells] - P.atomOff;
    std::vector<int> idx(std::max(nb, 1));
    if (nb > 0 && (rc = readArr(c, idx.data(), c->sortIdx + P.atomOff, nb))) return rc;
    for (int i = 0; i < P.nMol; i++) cellAtomsOut[i] = (i < nb) ? idx[i] - P.atomOff : -1;
  }
  return SG_OK;
}

extern "C" int sg_get_carbon_lists(sg_ctx *c, int rep, int *nsOut, int *slOut, int *nrlOut, int *rlOut) {
  if (!c || rep < 0 || rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "sg_get_carbon_lists: bad arguments");
  const RepConst &P = c->hrc[rep];
  std::vector<int> ns(P.nMol), nrl(P.nMol);
  std::vector<int> sl((size_t)P.nMol * kShortMax), rl((size_t)P.nMol * kRelMax * 2);
  std::vector<unsigned> packed((size_t)P.nMol * kRelMax);
  int rc;
  if ((rc = readArr(c, ns.data(), c->ns + P.atomOff, P.nMol)) ||
      (rc = readArr(c, nrl.data(), c->nrl + P.atomOff, P.nMol)) ||
      (rc = readArr(c, sl.data(), c->sl + (size_t)P.atomOff * kShortMax, sl.size())) ||
      (rc = readArr(c, packed.data(), c->rl + (size_t)P.atomOff * kRelMax, packed.size())))
    return rc;
  for (size_t q = 0; q < packed.size(); q++) {  // {atom, position in the full list} pairs
    rl[2 * q] = (int)(packed[q] >> 8);
    rl[2 * q + 1] = (int)(packed[q] & 0xffu);
  }
  for (int i = 0; i < P.nMol; i++) {
    for (int e = 0; e < kShortMax; e++) {
      int &x = sl[(size_t)i * kShortMax + e];
      x = (e < ns[i]) ? x - P.atomOff : -1;
    }
    for (int e = 0; e < kRelMax; e++) {
      int *x = &rl[((size_t)i * kRelMax + e) * 2];
      if (e >= nrl[i]) x[0] = x[1] = -1;  // entries hold local indices already
    }
  }
  if (nsOut) memcpy(nsOut, ns.data(), sizeof(int) * P.nMol);
  if (nrlOut) memcpy(nrlOut, nrl.data(), sizeof(int) * P.nMol);
  if (slOut) memcpy(slOut, sl.data(), sizeof(int) * sl.size());
  if (rlOut) memcpy(rlOut, rl.data(), sizeof(int) * rl.size());
  return SG_OK;
}

extern "C" int sg_get_nebr(sg_ctx *c, int rep, int *nnOut, int *nblOut) {
  if (!c || rep < 0 || rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "sg_get_nebr: bad arguments");
  const RepConst &P = c->hrc[rep];
  std::vector<int> nn(P.nMol);
  int rc;
  if ((rc = readArr(c, nn.data(), c->nn + P.atomOff, P.nMol))) return rc;
  if (nnOut) memcpy(nnOut, nn.data(), sizeof(int) * P.nMol);
  if (nblOut) {
    std::vector<int> rows((size_t)P.nMol * c->rowStride);
    if ((rc = readArr(c, rows.data(), c->nbl + (size_t)P.atomOff * c->rowStride, rows.size()))) return rc;
    for (int j = 0; j < c->hp[rep].iNebrMax; j++)  // the reference layout: iNebrMax columns
      for (int i = 0; i < P.nMol; i++)
        nblOut[(size_t)j * P.nMol + i] = (j < nn[i]) ? rows[(size_t)i * c->rowStride + j] - P.atomOff : -1;
  }
  return SG_OK;
}

static int getMetalArr(sg_ctx *c, int rep, float *out, const float *src) {
  if (!c || rep < 0 || rep >= c->nrep || !out) return sg_fail(SG_ERR_INVALID, "bad arguments");
  const RepConst &P = c->hrc[rep];
  if (P.nMolMe == 0) return SG_OK;
  return readArr(c, out, src + P.atomOff, P.nMolMe);
}
extern "C" int sg_get_rho(sg_ctx *c, int rep, float *rho) { return getMetalArr(c, rep, rho, c ? c->rho : nullptr); }
extern "C" int sg_get_friction(sg_ctx *c, int rep, float *f) { return getMetalArr(c, rep, f, c ? c->fric : nullptr); }

extern "C" int sg_get_rdf(sg_ctx *c, int rep, unsigned int *hist) {
  if (!c || rep < 0 || rep >= c->nrep || !hist) return sg_fail(SG_ERR_INVALID, "bad arguments");
  return readArr(c, hist, c->hist + (size_t)rep * c->histStride, (size_t)c->hp[rep].sizeHistRdf);
}
extern "C" int sg_get_rdf_ext(sg_ctx *c, int rep, unsigned long long *hist) {
  if (!c || rep < 0 || rep >= c->nrep || !hist) return sg_fail(SG_ERR_INVALID, "bad arguments");
  if (!c->histExt) return sg_fail(SG_ERR_UNSUPPORTED, "extended RDF not enabled (rdf_ext_bins)");
  return readArr(c, hist, c->histExt + (size_t)rep * c->opt.rdf_ext_bins, (size_t)c->opt.rdf_ext_bins);
}

extern "C" int sg_get_diffusion(sg_ctx *c, int rep, float *rr_av, int *counts, int *count_av) {
  if (!c || rep < 0 || rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "bad arguments");
  const sg_simparams &p = c->hp[rep];
  if (p.iRegime != 2) return sg_fail(SG_ERR_UNSUPPORTED, "diffusion is measured in regime 2 only");
  const size_t nf = DiffLayout::floatsPerRep(p.nBuffDiffuse, p.nValDiffuse);
  std::vector<float> buf(nf);
  int rc;
  if ((rc = readArr(c, buf.data(), c->diffBuf + c->diffOffH[rep], nf))) return rc;
  const float *av = buf.data() + (size_t)p.nBuffDiffuse * 7 + (size_t)p.nBuffDiffuse * p.nValDiffuse;
  if (rr_av) memcpy(rr_av, av, sizeof(float) * p.nValDiffuse);
  if (counts)
    for (int nb = 0; nb < p.nBuffDiffuse; nb++) memcpy(&counts[nb], &buf[7 * nb], sizeof(int));
  if (count_av) {
    RepState S;
    if ((rc = sg_read_state(c, rep, &S))) return rc;
    *count_av = S.countDiffuseAv;
  }
  return SG_OK;
}

// The last finished diffusion table (what PrintDiffusion writes) and the number produced.
int sg_get_diffusion_print(sg_ctx *c, int rep, float *table, int *nprints) {
  const sg_simparams &p = c->hp[rep];
  const size_t nf = DiffLayout::floatsPerRep(p.nBuffDiffuse, p.nValDiffuse);
  int rc;
  if (table && (rc = readArr(c, table, c->diffBuf + c->diffOffH[rep] + nf - p.nValDiffuse, (size_t)p.nValDiffuse)))
    return rc;
  if (nprints) {
    RepState S;
    if ((rc = sg_read_state(c, rep, &S))) return rc;
    *nprints = S.diffPrints;
  }
  return SG_OK;
}

extern "C" int sg_get_diag(sg_ctx *c, int rep, sg_diag *d) {
  if (!c || !d || rep < 0 || rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "bad arguments");
  RepState S;
  int rc = sg_read_state(c, rep, &S);
  if (rc) return rc;
  memset(d, 0, sizeof(*d));
  d->max_neighbours = S.maxNeighbours;
  d->max_cell_occupancy = S.maxCellOcc;
  d->nebr_overflow = S.nebrOverflow;
  d->cell_range = S.cellRange;
  d->cell_overflow = S.cellOverflow;
  d->rdf_range = S.rdfRange;
  d->timeouts = S.timeouts;
  d->reserved[0] = S.shortStale;
  return SG_OK;
}

// Accessors for the other translation units of the library.
cudaStream_t sg_stream(sg_ctx *c) { return c->stream; }
const sg_simparams &sg_host_params(sg_ctx *c, int rep) { return c->hp[rep]; }
int sg_host_step_count(sg_ctx *c) { return c->stepCount; }
int sg_next_variant(sg_ctx *c) { return stepVariant(c); }
int sg_launch_step(sg_ctx *c, int variant, bool *rdfPrint) {
  int rc = launchStep(c, variant);
  if (rc) return rc;
  advanceSchedule(c, variant, rdfPrint);
  return SG_OK;
}
sg_prop &sg_one_step_prop(sg_ctx *c, int rep) { return c->oneStep[rep]; }
int sg_check_flags(sg_ctx *c) { return checkFlags(c); }

// ---- autotuner ----------------------------------------------------------------------------
// A copy of every device buffer of the context and of the host's step counters.  The trials
// run real steps on the context's own state; the copy is put back after each.
namespace {
struct Snapshot {
  void *dev = nullptr;           // one device block holding all buffers, or
  std::vector<char> host;        // a host copy when the device has no room
  std::vector<std::pair<void *, size_t>> regions;  // the buffers copied
  int stepCount = 0, countRdf = 0, lastVariant = 0;
};

int takeSnapshot(sg_ctx *c, Snapshot &s) {
  s.regions = c->regions;
  size_t total = 0;
  for (auto &r : s.regions) total += (r.second + 255) & ~size_t(255);
  CK(cudaStreamSynchronize(c->stream));
  if (cudaMalloc(&s.dev, std::max<size_t>(total, 256)) != cudaSuccess) {
    cudaGetLastError();
    s.dev = nullptr;
    s.host.resize(total);
  }
  size_t off = 0;
  for (auto &r : s.regions) {
    char *dst = s.dev ? static_cast<char *>(s.dev) + off : s.host.data() + off;
    CK(cudaMemcpyAsync(dst, r.first, r.second, s.dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                       c->stream));
    off += (r.second + 255) & ~size_t(255);
  }
  CK(cudaStreamSynchronize(c->stream));
  s.stepCount = c->stepCount;
  s.countRdf = c->countRdf;
  s.lastVariant = c->lastVariant;
  return SG_OK;
}

int restoreSnapshot(sg_ctx *c, const Snapshot &s) {
  CK(cudaStreamSynchronize(c->stream));
  size_t off = 0;
  for (auto &r : s.regions) {
    const char *src = s.dev ? static_cast<const char *>(s.dev) + off : s.host.data() + off;
    CK(cudaMemcpyAsync(r.first, src, r.second, s.dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                       c->stream));
    off += (r.second + 255) & ~size_t(255);
  }
  CK(cudaStreamSynchronize(c->stream));
  c->stepCount = s.stepCount;
  c->countRdf = s.countRdf;
  c->lastVariant = s.lastVariant;
  return SG_OK;
}

// Milliseconds per step: the faster of two runs of `steps` steps, after three warm-up steps
// (which capture the graphs).
int timeSteps(sg_ctx *c, int steps, float *msPerStep) {
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int rc = sg_step_async(c, 3);
  if (!rc) rc = checkFlags(c);
  float best = 0.f;
  for (int run = 0; run < 2 && !rc; run++) {
    CK(cudaEventRecord(e0, c->stream));
    rc = sg_step_async(c, steps);
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (run == 0 || ms < best) best = ms;
    if (!rc) rc = checkFlags(c);
  }
  *msPerStep = best / steps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

// The choice a trial keeps: the incumbent (the setting before tuning) unless the fastest choice
// beats it by more than kTuneMargin, about the spread of the timings themselves.
constexpr float kTuneMargin = 0.01f;
int pickChoice(const float *ms, const int *choice, int n, int incumbent) {
  int fast = 0, inc = -1;
  for (int k = 0; k < n; k++) {
    if (ms[k] < ms[fast]) fast = k;
    if (choice[k] == incumbent) inc = k;
  }
  if (inc < 0 || ms[fast] < ms[inc] * (1.f - kTuneMargin)) return choice[fast];
  return choice[inc];
}
}  // namespace

extern "C" int sg_autotune(sg_ctx *c, int steps, char *report, int report_len) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  if (steps <= 0) steps = 20;
  Snapshot snap;
  int rc = takeSnapshot(c, snap);
  if (rc) return rc;
  const int lanes0 = c->metalLanes, bps0 = c->nebrBlocksPerSM, desc0 = c->nebrDescending;
  const int item0 = c->nebrItemAtoms, fr0 = c->opt.force_rebuild;
  const bool pdl0 = c->pdl;
  const int algo0 = c->nebrAlgo;
  const bool staged0 = c->eamStaged;
  const int cb0 = c->carbonBlocks;
  const int laneChoice[4] = {4, 8, 16, 32}, bpsChoice[4] = {2, 4, 7, 14}, itemChoice[4] = {4, 6, 8, 16};
  const int algoChoice[3] = {0, 1, 2}, offOn[2] = {0, 1}, cbChoice[3] = {8, 12, 16};
  float laneMs[4] = {}, bpsMs[4] = {}, orderMs[2] = {}, itemMs[4] = {}, pdlMs[2] = {}, algoMs[3] = {};
  float stagedMs[2] = {}, cbMs[3] = {};
  bool bestStaged = staged0;
  int bestCb = cb0;
  int bestLanes = lanes0, bestBps = bps0, bestDesc = desc0, bestItem = item0, bestAlgo = algo0;
  bool bestPdl = pdl0;
  // 1. lanes per metal atom, on the context's own schedule
  // the persistent step runs 4 or 16 lanes, the cell-window list build on its own grid, no
  // programmatic launch, the table through L1 and one register budget: those trials are skipped
  // (their time reads 1e30)
  const bool P = c->persistent;
  const float kSkip = 1e30f;
  if (c->metalRun.n > 0) {
    for (int k = 0; k < 4 && !rc; k++) {
      if (P && laneChoice[k] != 4 && laneChoice[k] != kMT) {
        laneMs[k] = kSkip;
        continue;
      }
      if ((rc = restoreSnapshot(c, snap)) || (rc = setMetalLanes(c, laneChoice[k]))) break;
      rc = timeSteps(c, steps, &laneMs[k]);
    }
    if (!rc) bestLanes = pickChoice(laneMs, laneChoice, 4, lanes0);
  }
  // 2. the list build (atom threads or cell windows; for cell windows the home atoms per item,
  //    blocks per SM and cell order), with a rebuild in every step
  if (!rc && !(rc = setMetalLanes(c, bestLanes))) {
    c->opt.force_rebuild = 1;
    destroyGraphs(c);
    for (int a = 0; a < 3 && !rc; a++) {
      if (P && a != 0) {
        algoMs[a] = kSkip;
        continue;
      }
      if ((rc = restoreSnapshot(c, snap))) break;
      c->nebrAlgo = a;
      destroyGraphs(c);
      rc = timeSteps(c, steps, &algoMs[a]);
    }
    if (!rc) bestAlgo = pickChoice(algoMs, algoChoice, 3, algo0);
    c->nebrAlgo = bestAlgo;
    if (!rc && bestAlgo != 1) {
      for (int k = 0; k < 4 && !rc; k++) {
        if ((rc = restoreSnapshot(c, snap))) break;
        c->nebrItemAtoms = itemChoice[k];
        destroyGraphs(c);
        rc = timeSteps(c, steps, &itemMs[k]);
      }
      if (!rc) bestItem = pickChoice(itemMs, itemChoice, 4, item0);
      c->nebrItemAtoms = bestItem;
      destroyGraphs(c);
      for (int k = 0; k < 4 && !rc; k++) {
        if (P) {
          bpsMs[k] = kSkip;
          continue;
        }
        if ((rc = restoreSnapshot(c, snap))) break;
        setNebrBlocks(c, bpsChoice[k]);
        rc = timeSteps(c, steps, &bpsMs[k]);
      }
      if (!rc) bestBps = pickChoice(bpsMs, bpsChoice, 4, bps0);
      if (!rc) setNebrBlocks(c, bestBps);
      for (int d = 0; d < 2 && !rc; d++) {
        if ((rc = restoreSnapshot(c, snap))) break;
        c->nebrDescending = d;
        destroyGraphs(c);
        rc = timeSteps(c, steps, &orderMs[d]);
      }
      if (!rc) bestDesc = pickChoice(orderMs, offOn, 2, desc0);
    }
    c->opt.force_rebuild = fr0;
    destroyGraphs(c);
  }
  // 3. programmatic dependent launch, on the context's own schedule
  if (!rc) {
    c->nebrDescending = bestDesc;
    c->nebrItemAtoms = bestItem;
    c->nebrAlgo = bestAlgo;
    setNebrBlocks(c, bestBps);
    for (int k = 0; k < 2 && !rc; k++) {
      if (P) {
        pdlMs[k] = kSkip;
        continue;
      }
      if ((rc = restoreSnapshot(c, snap))) break;
      c->pdl = k == 1;
      destroyGraphs(c);
      rc = timeSteps(c, steps, &pdlMs[k]);
    }
    if (!rc) bestPdl = pickChoice(pdlMs, offOn, 2, pdl0 ? 1 : 0) == 1;
  }
  // 4. (MIXED) the EAM table through L1 or staged in shared memory
  if (!rc && !P && c->opt.mode == SG_MODE_MIXED && sg_mixed_staging_ok(c) && c->metalRun.n > 0) {
    c->pdl = bestPdl;
    for (int k = 0; k < 2 && !rc; k++) {
      if ((rc = restoreSnapshot(c, snap))) break;
      c->eamStaged = k == 1;
      destroyGraphs(c);
      rc = timeSteps(c, steps, &stagedMs[k]);
    }
    if (!rc) bestStaged = pickChoice(stagedMs, offOn, 2, staged0 ? 1 : 0) == 1;
  }
  // 5. the carbon pass's resident blocks per SM, on the context's own schedule
  if (!rc && !P && c->carbonTabT.n > 0) {
    c->pdl = bestPdl;
    c->eamStaged = bestStaged;
    for (int k = 0; k < 3 && !rc; k++) {
      if ((rc = restoreSnapshot(c, snap))) break;
      c->carbonBlocks = cbChoice[k];
      destroyGraphs(c);
      rc = timeSteps(c, steps, &cbMs[k]);
    }
    if (!rc) bestCb = pickChoice(cbMs, cbChoice, 3, cb0);
  }
  // the state as it was, with the chosen shape (the starting shape if a trial failed)
  const int rc2 = restoreSnapshot(c, snap);
  if (snap.dev) cudaFree(snap.dev);
  if (rc) {
    setMetalLanes(c, lanes0);
    setNebrBlocks(c, bps0);
    c->nebrDescending = desc0;
    c->nebrItemAtoms = item0;
    c->pdl = pdl0;
    c->nebrAlgo = algo0;
    c->eamStaged = staged0;
    c->carbonBlocks = cb0;
    destroyGraphs(c);
    return rc;
  }
  if (rc2) return rc2;
  if ((rc = setMetalLanes(c, bestLanes))) return rc;
  setNebrBlocks(c, bestBps);
  c->nebrDescending = bestDesc;
  c->nebrItemAtoms = bestItem;
  c->pdl = bestPdl;
  c->nebrAlgo = bestAlgo;
  c->eamStaged = bestStaged;
  c->carbonBlocks = bestCb;
  destroyGraphs(c);
  if (report && report_len > 0) {
    snprintf(report, report_len,
             "{\"steps\": %d, \"metal_lanes_ms_per_step\": {\"4\": %.6g, \"8\": %.6g, \"16\": %.6g, "
             "\"32\": %.6g}, \"nebr_blocks_per_sm_ms_per_step_rebuilding\": {\"2\": %.6g, \"4\": %.6g, "
             "\"7\": %.6g, \"14\": %.6g}, \"nebr_order_ms_per_step_rebuilding\": {\"ascending\": %.6g, "
             "\"descending\": %.6g}, \"nebr_item_atoms_ms_per_step_rebuilding\": {\"4\": %.6g, "
             "\"6\": %.6g, \"8\": %.6g, \"16\": %.6g}, \"programmatic_launch_ms_per_step\": {\"0\": %.6g, "
             "\"1\": %.6g}, \"nebr_build_ms_per_step_rebuilding\": {\"0\": %.6g, \"1\": %.6g, \"2\": %.6g}, "
             "\"eam_table_smem_ms_per_step\": {\"0\": %.6g, \"1\": %.6g}, "
             "\"carbon_blocks_per_sm_ms_per_step\": {\"8\": %.6g, \"12\": %.6g, \"16\": %.6g}, "
             "\"metal_lanes\": %d, \"nebr_blocks_per_sm\": %d, \"nebr_descending\": %d, "
             "\"nebr_item_atoms\": %d, \"programmatic_launch\": %d, \"nebr_build\": %d, "
             "\"eam_table_smem\": %d, \"carbon_blocks_per_sm\": %d, \"nebr_grid\": %d}",
             steps, laneMs[0], laneMs[1], laneMs[2], laneMs[3], bpsMs[0], bpsMs[1], bpsMs[2], bpsMs[3],
             orderMs[0], orderMs[1], itemMs[0], itemMs[1], itemMs[2], itemMs[3], pdlMs[0], pdlMs[1],
             algoMs[0], algoMs[1], algoMs[2], stagedMs[0], stagedMs[1], cbMs[0], cbMs[1], cbMs[2], c->metalLanes,
             c->nebrBlocksPerSM, c->nebrDescending, c->nebrItemAtoms, c->pdl ? 1 : 0, c->nebrAlgo,
             c->eamStaged ? 1 : 0, c->carbonBlocks, c->nebrGrid);
  }
  return SG_OK;
}

extern "C" int sg_set_launch_shape(sg_ctx *c, const sg_launch_shape *shape) {
  if (!c || !shape) return sg_fail(SG_ERR_INVALID, "null argument");
  if (shape->nebr_blocks_per_sm < 1 || shape->nebr_blocks_per_sm > 32)
    return sg_fail(SG_ERR_INVALID, "nebr_blocks_per_sm %d: 1..32", shape->nebr_blocks_per_sm);
  if (shape->nebr_descending != 0 && shape->nebr_descending != 1)
    return sg_fail(SG_ERR_INVALID, "nebr_descending %d: 0 or 1", shape->nebr_descending);
  if (shape->nebr_item_atoms < kMinItemAtoms || shape->nebr_item_atoms > 64)
    return sg_fail(SG_ERR_INVALID, "nebr_item_atoms %d: %d..64", shape->nebr_item_atoms, kMinItemAtoms);
  if (shape->programmatic_launch != 0 && shape->programmatic_launch != 1)
    return sg_fail(SG_ERR_INVALID, "programmatic_launch %d: 0 or 1", shape->programmatic_launch);
  if (shape->nebr_build < 0 || shape->nebr_build > 2)
    return sg_fail(SG_ERR_INVALID, "nebr_build %d: 0, 1 or 2", shape->nebr_build);
  if (shape->eam_table_smem != 0 && shape->eam_table_smem != 1)
    return sg_fail(SG_ERR_INVALID, "eam_table_smem %d: 0 or 1", shape->eam_table_smem);
  if (shape->eam_table_smem && !(c->opt.mode == SG_MODE_MIXED && sg_mixed_staging_ok(c)))
    return sg_fail(SG_ERR_UNSUPPORTED, "eam_table_smem: MIXED mode with tabulated EAM only");
  if (shape->carbon_blocks_per_sm != 8 && shape->carbon_blocks_per_sm != 12 && shape->carbon_blocks_per_sm != 16)
    return sg_fail(SG_ERR_INVALID, "carbon_blocks_per_sm %d: 8, 12 or 16", shape->carbon_blocks_per_sm);
  if (c->persistent && (shape->nebr_build != 0 || shape->programmatic_launch != 0 || shape->eam_table_smem != 0))
    return sg_fail(SG_ERR_UNSUPPORTED, "the persistent step: nebr_build 0, no programmatic launch, no staged table");
  CK(cudaStreamSynchronize(c->stream));
  const int rc = setMetalLanes(c, shape->metal_lanes);
  if (rc) return rc;
  setNebrBlocks(c, shape->nebr_blocks_per_sm);
  if (shape->nebr_descending != c->nebrDescending || shape->nebr_item_atoms != c->nebrItemAtoms ||
      (shape->programmatic_launch != 0) != c->pdl || shape->nebr_build != c->nebrAlgo)
    destroyGraphs(c);
  c->nebrAlgo = shape->nebr_build;
  if ((shape->eam_table_smem != 0) != c->eamStaged) destroyGraphs(c);
  c->eamStaged = shape->eam_table_smem != 0;
  c->nebrDescending = shape->nebr_descending;
  c->nebrItemAtoms = shape->nebr_item_atoms;
  c->pdl = shape->programmatic_launch != 0;
  if (shape->carbon_blocks_per_sm != c->carbonBlocks) destroyGraphs(c);
  c->carbonBlocks = shape->carbon_blocks_per_sm;
  return SG_OK;
}

extern "C" int sg_get_launch_shape(sg_ctx *c, sg_launch_shape *shape) {
  if (!c || !shape) return sg_fail(SG_ERR_INVALID, "null argument");
  memset(shape, 0, sizeof(*shape));
  shape->metal_lanes = c->metalLanes;
  shape->nebr_blocks_per_sm = c->nebrBlocksPerSM;
  shape->nebr_descending = c->nebrDescending;
  shape->nebr_item_atoms = c->nebrItemAtoms;
  shape->programmatic_launch = c->pdl ? 1 : 0;
  shape->nebr_build = c->nebrAlgo;
  shape->eam_table_smem = c->eamStaged ? 1 : 0;
  shape->carbon_blocks_per_sm = c->carbonBlocks;
  return SG_OK;
}
