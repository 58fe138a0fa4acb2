// sg_device.cuh - device-side data layout shared by the sgmd kernels.
//
// Layout in HBM (all replicas of a context concatenated, replica r owning the global atom
// range [atomOff, atomOff + nMol) with its metal atoms first, as in the reference):
//   pos   float4[Ntot]  x, y, z, U (U = per-atom potential energy, written by the force pass)
//   vel   float4[Ntot]  vx, vy, vz, -
//   acc   float4[Ntot]  ax, ay, az, -            (acceleration = force / mass)
//   posLo float4[Ntot]  low words of the hi/lo position pair (MIXED mode only)
//   cellOf int[Ntot]    local cell of the atom at the last rebuild (-1: outside the grid)
//   slot   int[Ntot]    arrival slot inside the cell (scratch of the counting sort)
//   cellCount int[Ctot], cellStart int[Ctot + R] (per-replica, tile-padded cell ranges)
//   sortIdx int[Ntot], sortPos float4[Ntot]  atoms grouped by cell, ascending index per cell
//   nn int[Ntot], nbl int[Ntot * rowStride] neighbour list, entry j of atom g at
//                                           nbl[g * rowStride + j] (rowStride = nebrMax rounded
//                                           up to a multiple of 4: 16-byte aligned rows)
//   nrl int[Ntot], rl u32[Ntot * kRelMax]   relevant list of a carbon atom: its metal entries
//                                           and entries within (rCutC+skin), each the index in
//                                           the replica and the position in the full list in
//                                           one word (relPack)
//   ns int[Ntot], sl int[Ntot * kShortMax]  close list of a carbon atom: its entries within
//                                           (rCutC+skin), in list order
//   rho/dF/Fv float[Ntot]   EAM density, F'(rho), F(rho) (metal atoms)
//   fric float[Ntot]       x force of carbon on each metal atom
// Per-replica constants live in RepConst, mutable per-replica scalars in RepState.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sg {

constexpr int kRedThreads = 512;  // reduction block: 512 threads x 2 elements (reference shape)
constexpr int kRedElems = 1024;
constexpr int kCellTile = 2048;   // cells per scan tile (cell ranges are padded to this)
constexpr int kNumRed = 16;       // values reduced per element in the step reduction
constexpr int kMT = 16;           // lanes per metal atom in the density and metal-force passes
constexpr int kCT = 4;            // lanes per carbon atom in the carbon-force pass
constexpr int kNebrWarps = 4;     // warps per block in the neighbour-list build (one home cell each)
constexpr int kWin = 512;         // candidates per shared-memory window of the lane-placed list build
constexpr int kFusedWin = 256;    // candidates per window pass of the fused list build
constexpr int kRelMax = 48;       // relevant-list capacity per carbon atom
constexpr int kShortMax = 8;      // close-list capacity per carbon atom (a multiple of 4)
constexpr int kRelPosLimit = 256; // relevant-list entries record list positions below this
constexpr int kMaxReplicaAtoms = 1 << 24;  // atoms of one replica (relevant entries index 24 bits)
constexpr int kHeavyCell = 16;    // list build: default home atoms per work item (larger cells split)
constexpr int kHeavyChunk = 8;    // sizes the item list of the fixed-size scratch (>= kHeavyCell / 2)
constexpr int kScanCells = 128;   // cells per block of the single-pass cell scan and ordering (or 2x)
constexpr int kScanRankThreads = 512;  // threads of that block (the ordering uses all of them)
constexpr int kMixThreads = 512;  // MIXED step reduction: threads per block
constexpr int kMixAtoms = 512;    // and the fewest atoms per block (1 per thread; up to 8 at large sizes)
constexpr int kUnpackAtoms = 256; // state upload: atoms (threads) per block
constexpr int kMinItemAtoms = 4;  // smallest home atoms per work item the engine allows
constexpr int kItemAtoms = 8;     // the engine's default home atoms per work item
constexpr int kMixedCellCapFactor = 4;  // MIXED: atoms per cell up to 4 x blockSize (256)
constexpr int kRdfAtoms = 4;      // RDF sample: metal atoms per 128-thread block (a warp each)
constexpr int kRdfTile = 64;      // RDF extension: metal atoms per tile (and threads per block)
constexpr int kMetalPerBlock = 128 / kMT;   // atoms per 128-thread block
constexpr int kCarbonPerBlock = 128 / kCT;

// Values of the step reduction (slot indices into a 16-float record).
enum RedSlot {
  RS_VSUM_X = 0, RS_VSUM_Y, RS_VSUM_Z,  // total impulse
  RS_VVMAX,                             // max v^2
  RS_VVSUM,                             // Sum m v^2 (metal v.x - V_cm in regime 2)
  RS_USUM,                              // Sum U
  RS_CM_X, RS_CM_Y, RS_CM_Z,            // Sum r (metal)
  RS_MIN_X, RS_MIN_Y, RS_MIN_Z,         // min r (metal, with the reference's zero padding)
  RS_MAX_X, RS_MAX_Y, RS_MAX_Z,
  RS_FRICT                              // Sum friction (metal)
};

struct RepConst {
  // geometry and bookkeeping
  float region[3], invWidth[3];
  int cells[3], ncells, ncellsPad;
  int atomOff, nMol, nMolMe, cellOff;
  int nRedBlocks;  // ceil(nMol / 1024)
  int scanCells;   // cells per block of the scan and ordering (kScanCells or 2 kScanCells)
  int uncapped;    // MIXED: a cell above the bucket capacity is ordered by compaction, not flagged
  int nRedBlocksM, redFirstM;  // MIXED reduction: blocks of kMixAtoms atoms, first partial slot
  // integrator
  float deltaT, rrNebr, rNebrShell, rrShort;
  float xLeft, xRight, yBottom, yTop;
  // EAM
  float rei, rhoei, rhoe, fe, alpha, beta, A, B, kappa, lambda, Fn[4], F[4], eta, Fe, massMe;
  float rrCutEam;
  // graphene and LJ
  float rrCutC, mu_r, theta_0, mu_theta, mu_p, z_0, sigmaLJ, epsLJ, rrCutLJ;
  // thermostat, shear, deposition
  float temperature, kB, gammaBerendsen, deltaF, velMagDepos;
  int iRegime, stepEquil, stepCool, stepThermostat, stepDeposit, nMolToDeposit;
  int hasFric;
  // RDF
  float rangeRdf, intervalRdf;
  int sizeHistRdf, bRdf;
  // diffusion
  int nValDiffuse, nBuffDiffuse, stepDiffuse, limitDiffuseAv;
  int stepAvg;
  // MIXED mode: tabulated EAM pair functions, knots r_k = rTabMin + k * rTabH, k < nTab,
  // at tabOff in the table buffer (nTab == 0: analytic)
  int tabOff;
  float rTabMin, rTabInv, rTabH;
  int nTab;
  // MIXED mode: FP64 reciprocals for the step control (no FP64 division on the device)
  double invNMol, invNMolMe, invRegion[3];
};

struct RepState {
  int stepCount;       // steps completed
  int nebrNow;         // rebuild at the next step
  int rebuilds;
  int thermoPending;   // 1: rescale velocities at the start of the next step
  float betaC, betaM;  // factors of the pending rescale
  int thermoMetal;     // pending rescale includes metal atoms
  float dispHi;
  float shear, totalShear;
  unsigned shearCount;
  int nMolDeposited;
  int countRdf;
  float cmVal, cmVelVal, frictVal;  // centerOfMass.val, cmVel.val, frictForce.val
  float ke, pe, te;
  float red[kNumRed];               // last step's reduced values
  float cmVel[3];                   // Sum v over metal (from the cmVel pass)
  double ke64, pe64, virial64;
  double red64[kNumRed];
  float props[7][3];                // totEnergy, potEnergy, kinEnergy, oneStep, cm, cmVel, frict
  float propsSnap[7][3];            // sums at the last stepAvg boundary (before averaging)
  int snapStep;
  int countDiffuseAv;
  int diffPrints;                   // number of Diffuse.txt tables produced
  unsigned redCounter;              // last-block counters
  unsigned cmvCounter;
  unsigned shearCounter;
  int flags;                        // sticky error bits (SG_ERR_* as 1 << code)
  int maxNeighbours, maxCellOcc, nebrOverflow, cellRange, cellOverflow, rdfRange, shortStale;
  int timeouts;                     // bounded device-side waits that gave up (persistent step)
  int pad[3];
};

// Relevant-list entry of a carbon atom: the neighbour's index relative to its replica's first
// atom (24 bits) and its position in the full list (8 bits), one 32-bit word, so that the
// carbon pass reads a typical row of about 7 entries in one 32-byte sector.  An atom whose full
// list holds more than kRelPosLimit entries has no relevant list (the pass walks the full list).
__host__ __device__ __forceinline__ unsigned relPack(int kLocal, int pos) {
  return ((unsigned)kLocal << 8) | ((unsigned)pos & 0xffu);
}

// Block-to-replica tables: block b of a launch covers [start[b], start[b] + bs) clipped to its
// replica's range; start is a global index (atoms) or local index (cells, reductions).
struct BlockTab {
  const int *rep;
  const int *start;
  int nblocks;
};

// Device diffusion buffers of one replica live in a flat float array:
//   tb[nBuff] {count, orgR.xyz, rTrue.xyz} as 7 floats, rr[nBuff][nVal], av[nVal],
//   print[nVal] (last finished table).
struct DiffLayout {
  static __host__ __device__ size_t floatsPerRep(int nBuff, int nVal) {
    return (size_t)nBuff * 7 + (size_t)nBuff * nVal + 2 * (size_t)nVal;
  }
};

// Offset of stencil cell o (0..26) in the reference's visiting order
// (SurfaceGrowthConsole/ComputeDefs.h:221-231): x outermost, then y, then z, each in the order
// 0, +1, -1.  Computed rather than read from a table: the lanes of a warp look up different
// cells at once, which a constant-memory table would serialise.
__device__ __forceinline__ int stencilStep(int i) { return i == 2 ? -1 : i; }

// Neighbour cell of local cell c at stencil offset o with the periodic shift
// (BuildNebrListK, SurfaceGrowth.cu:641-674).
__device__ __forceinline__ int stencilCell(const RepConst &P, int c, int o, float &sx, float &sy,
                                           float &sz) {
  int ccz = c / (P.cells[0] * P.cells[1]);
  int ccy = (c - ccz * P.cells[0] * P.cells[1]) / P.cells[0];
  int ccx = c - (ccz * P.cells[1] + ccy) * P.cells[0];
  int mx = ccx + stencilStep(o / 9), my = ccy + stencilStep((o / 3) % 3), mz = ccz + stencilStep(o % 3);
  sx = 0.f; sy = 0.f; sz = 0.f;
  if (mx >= P.cells[0]) { mx = 0; sx = P.region[0]; }
  else if (mx < 0) { mx = P.cells[0] - 1; sx = -P.region[0]; }
  if (my >= P.cells[1]) { my = 0; sy = P.region[1]; }
  else if (my < 0) { my = P.cells[1] - 1; sy = -P.region[1]; }
  if (mz >= P.cells[2]) { mz = 0; sz = P.region[2]; }
  else if (mz < 0) { mz = P.cells[2] - 1; sz = -P.region[2]; }
  return (mz * P.cells[1] + my) * P.cells[0] + mx;
}

// Cell of a position (BinAtomsIntoCellsK, SurfaceGrowth.cu:594-600); -1 when the linear index
// falls outside the grid (the reference then never bins the atom).
__device__ __forceinline__ int cellIndex(const RepConst &P, float x, float y, float z) {
  // a non-finite coordinate (a system that has blown up) is outside the grid, like an atom out of
  // the box: left out of the lists and counted, not filed into whatever cell the conversion gives
  if (!isfinite(x) || !isfinite(y) || !isfinite(z)) return -1;
  int cx = (int)((x + 0.5f * P.region[0]) * P.invWidth[0]);
  int cy = (int)((y + 0.5f * P.region[1]) * P.invWidth[1]);
  int cz = (int)((z + 0.5f * P.region[2]) * P.invWidth[2]);
  long long c = ((long long)cz * P.cells[1] + cy) * P.cells[0] + cx;
  return (c < 0 || c >= P.ncells) ? -1 : (int)c;
}

// Minimum image of one component as the force kernels do it (SurfaceGrowth.cu:750-759).
// Cell of atom g and its arrival slot in the cell; with a bucket (cap slots per cell, the
// reference's blockSize) the atom is also filed there, and counted in blockCount per block of
// P.scanCells cells (one atomic per block among the warp's atoms), for k_scan_rank.  An atom
// past the cap is not filed; uncapped (MIXED) it is counted all the same and, with a spill list,
// appended there as {global cell, atom} (spillCount: its length), where the scan finds it.
__device__ __forceinline__ void binAtom(const RepConst &P, int g, const float4 &r, int *cellOf, int *slot,
                                        int *cellCount, int *bucket, int cap, int *blockCount,
                                        int2 *spill = nullptr, int *spillCount = nullptr) {
  const int c = cellIndex(P, r.x, r.y, r.z);
  cellOf[g] = c;
  int key = -1;
  if (c >= 0) {
    const int s = atomicAdd(&cellCount[P.cellOff + c], 1);
    slot[g] = s;
    if (bucket && s < cap) {
      bucket[(size_t)(P.cellOff + c) * cap + s] = g;
      if (blockCount) key = (P.cellOff + c) / P.scanCells;
    } else if (bucket && P.uncapped) {
      if (spill) spill[atomicAdd(spillCount, 1)] = make_int2(P.cellOff + c, g);
      if (blockCount) key = (P.cellOff + c) / P.scanCells;
    }
  }
  if (blockCount) {
    const unsigned same = __match_any_sync(__activemask(), key);
    if (key >= 0 && __ffs(same) - 1 == (int)(threadIdx.x & 31)) atomicAdd(&blockCount[key], __popc(same));
  }
}

__device__ __forceinline__ float minImg(float d, float L) {
  if (d >= 0.5f * L) d -= L;
  else if (d < -0.5f * L) d += L;
  return d;
}

// The step control of a replica runs in the last block of its reduction on shared-memory copies
// of the replica's RepState and RepConst (its scalar code then sees shared-memory latency instead
// of L2 latency), which every reduction block loads while it reduces (nothing writes the state
// before the last block has arrived; the reduction is the only kernel of the step running), and
// writes the state back.
static_assert(sizeof(RepState) % 4 == 0, "RepState is copied as 32-bit words");
static_assert(sizeof(RepConst) % 4 == 0, "RepConst is copied as 32-bit words");
__device__ __forceinline__ void constToShared(const RepConst *g, RepConst *s) {
  const int *src = reinterpret_cast<const int *>(g);
  int *dst = reinterpret_cast<int *>(s);
  for (int i = threadIdx.x; i < (int)(sizeof(RepConst) / 4); i += blockDim.x) dst[i] = src[i];
}
__device__ __forceinline__ void stateFromShared(const RepState *s, RepState *g) {
  __syncthreads();
  const int *src = reinterpret_cast<const int *>(s);
  int *dst = reinterpret_cast<int *>(g);
  for (int i = threadIdx.x; i < (int)(sizeof(RepState) / 4); i += blockDim.x) dst[i] = src[i];
}

// Where a step's last blocks publish the replica states when the step's publish is folded into
// its reduction (hostSt null: no publish): the host mirror, the device-side sequence counter
// (seq[0]) with the publish's arrival count (seq[1]), the host's copy of the sequence number.
struct PublishArgs {
  RepState *hostSt = nullptr;
  unsigned *seq = nullptr;
  volatile unsigned *hostSeq = nullptr;
  int nrep = 0;
};

// Replica rep's final state s (shared memory, just written to its device record) into the host
// mirror; the last replica to arrive then raises the sequence number, after a system-wide fence
// that orders every replica's mirror words before it (the host reads the number with acquire
// ordering, then the mirror).  By the whole block.
__device__ __forceinline__ void publishReplica(const RepState *s, int rep, const PublishArgs &pub) {
  const int *src = reinterpret_cast<const int *>(s);
  int *dst = reinterpret_cast<int *>(pub.hostSt + rep);
  for (int i = threadIdx.x; i < (int)(sizeof(RepState) / 4); i += blockDim.x) dst[i] = src[i];
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(pub.seq + 1, 1u) == (unsigned)pub.nrep - 1u) {
    pub.seq[1] = 0;
    __threadfence();
    const unsigned n = pub.seq[0] + 1u;
    pub.seq[0] = n;
    __threadfence_system();
    *pub.hostSeq = n;
  }
}

__device__ __forceinline__ void setFlag(RepState *st, int code) {
  atomicOr(&st->flags, 1 << code);
}

// Programmatic dependent launch.  A kernel of the step chain, launched with the
// programmatic-serialization attribute, is scheduled once every block of its predecessor in the
// stream has exited (the implicit trigger: no kernel calls launch_dependents, so waiting blocks
// never hold SM slots the predecessor still needs), overlapping its launch with the
// predecessor's completion; it waits here, before its first global memory access, for the
// predecessor grid to complete with its memory visible.  Every kernel of the chain waits, so
// completion is transitive.  Launched without the attribute, the wait returns at once.
__device__ __forceinline__ void pdlEnter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

}  // namespace sg

#ifdef __CUDACC__
namespace sg {
// Launches kernel k on stream s, with the programmatic-serialization attribute when pdl is set
// (the kernel must begin with pdlEnter()).
template <typename... KArgs, typename... Args>
inline cudaError_t launchK(bool pdl, void (*k)(KArgs...), int grid, int block, size_t smem, cudaStream_t s,
                           Args... args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}
}  // namespace sg
#endif
