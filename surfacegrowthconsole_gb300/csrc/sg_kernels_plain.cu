// sg_kernels_plain.cu - PLAIN-mode (FP32 parity) kernels and the list-building kernels
// shared by both modes.  Compiled with -fmad=false: every expression below is evaluated in the
// reference's source order with separately rounded multiplies and adds, so integer results
// (cell assignment, neighbour lists, RDF counts) and all arithmetic not involving a
// transcendental function are bit-identical to the reference built without FMA contraction
// and to the CPU oracle built with -ffp-contract=off.
//
// All kernels are batched: blocks are assigned to replicas through BlockTab tables and never
// straddle two replicas, so per-replica constants are block-uniform.
#include "sg_device.cuh"
#include "sg_kernels.h"
#include "sg_lists.cuh"

namespace sg {

// ============================================================================================
// Integrator, part 1 (LeapfrogStepK part==1 + ApplyBoundaryCondK, SurfaceGrowth.cu:397-453),
// fused with: the Berendsen rescale decided at the end of the previous step
// (ApplyBerendsenThermostat, cu:455-485), regime-1 deposition (InsertAtomsK, cu:488-514,
// schedule cu:2148-2168) and, on rebuild steps, the histogram pass of the cell counting sort
// (cell index as BinAtomsIntoCellsK, cu:594-600).
// ============================================================================================
__device__ __forceinline__ bool isFrozen(const RepConst &P, int local, float x, float y) {
  if (local < P.nMolMe) return false;
  return !((x != P.xLeft) && (x < P.xRight) && (y != P.yTop) && (y != P.yBottom));
}

__device__ __forceinline__ void depositionPlan(const RepConst &P, const RepState &S, int sc,
                                               int &nDep, int &nTo, bool &act) {
  nDep = S.nMolDeposited;
  nTo = 0;
  act = false;
  if (P.iRegime != 1) return;
  if (sc <= P.stepEquil) {
    act = true;
  } else if (nDep < P.nMolMe) {
    act = true;
    if ((sc - P.stepEquil) % P.stepDeposit == 0) nTo = P.nMolToDeposit;
  }
}

__global__ void k_integrate_first(BlockTab tab, const RepConst *__restrict__ rc, RepState *st,
                                  float4 *__restrict__ pos, float4 *__restrict__ vel,
                                  const float4 *__restrict__ acc, int *__restrict__ cellOf,
                                  int *__restrict__ slot, int *__restrict__ cellCount,
                                  int forceRebuild, int *__restrict__ bucket, int cap,
                                  int *__restrict__ blockCount) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  RepState *S = st + rep;
  const int g = tab.start[blockIdx.x] + threadIdx.x;
  const int end = P.atomOff + P.nMol;
  if (g >= end) return;
  const int local = g - P.atomOff;
  const int sc = S->stepCount + 1;
  float4 r = pos[g];
  float4 v = vel[g];
  const float4 a = acc[g];
  // pending thermostat rescale of the previous step
  if (S->thermoPending) {
    if (local >= P.nMolMe) {
      const float b = S->betaC;
      v.x = b * v.x; v.y = b * v.y; v.z = b * v.z;
    } else if (S->thermoMetal) {
      const float b = S->betaM;
      v.x = b * v.x; v.y = b * v.y; v.z = b * v.z;
    }
  }
  // deposition (regime 1)
  if (local < P.nMolMe && P.iRegime == 1) {
    int nDep, nTo;
    bool act;
    depositionPlan(P, *S, sc, nDep, nTo, act);
    if (act) {
      if (local >= nDep && local < nDep + nTo) {
        r.z = 0.49f * P.region[2];
        v.z = -P.velMagDepos;
      }
      if (local >= nDep + nTo) {
        r.z = 1.5f * P.region[2] + 0.5f * (float)(local + 1) * P.region[2];
        v.x = 0.f; v.y = 0.f; v.z = 0.f;
      }
    }
  }
  // Verlet: half kick and drift, unless a frozen graphene edge atom
  if (!isFrozen(P, local, r.x, r.y)) {
    const float h = 0.5f * P.deltaT;
    v.x = v.x + h * a.x;
    v.y = v.y + h * a.y;
    v.z = v.z + h * a.z;
    r.x = r.x + P.deltaT * v.x;
    r.y = r.y + P.deltaT * v.y;
    r.z = r.z + P.deltaT * v.z;
  }
  // periodic wrap, one image per axis
  if (r.x >= 0.5f * P.region[0]) r.x -= P.region[0];
  else if (r.x < -0.5f * P.region[0]) r.x += P.region[0];
  if (r.y >= 0.5f * P.region[1]) r.y -= P.region[1];
  else if (r.y < -0.5f * P.region[1]) r.y += P.region[1];
  if (r.z >= 0.5f * P.region[2]) r.z -= P.region[2];
  else if (r.z < -0.5f * P.region[2]) r.z += P.region[2];
  pos[g] = r;
  vel[g] = v;
  if (forceRebuild || S->nebrNow) binAtom(P, g, r, cellOf, slot, cellCount, bucket, cap, blockCount);
}

// Histogram pass alone (used when lists are rebuilt outside a step).
__global__ void k_cell_count(BlockTab tab, const RepConst *__restrict__ rc,
                             const float4 *__restrict__ pos, int *__restrict__ cellOf,
                             int *__restrict__ slot, int *__restrict__ cellCount) {
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  const int g = tab.start[blockIdx.x] + threadIdx.x;
  if (g >= P.atomOff + P.nMol) return;
  const float4 r = pos[g];
  const int c = cellIndex(P, r.x, r.y, r.z);
  cellOf[g] = c;
  if (c >= 0) slot[g] = atomicAdd(&cellCount[P.cellOff + c], 1);
}

// Histogram and bucket pass alone (lists rebuilt outside a step).
__global__ void k_cell_bucket(BlockTab tab, const RepConst *__restrict__ rc, const float4 *__restrict__ pos,
                              int *__restrict__ cellOf, int *__restrict__ slot, int *__restrict__ cellCount,
                              int *__restrict__ bucket, int cap, int *__restrict__ blockCount,
                              int2 *__restrict__ spill, int *__restrict__ spillCount) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  const int g = tab.start[blockIdx.x] + threadIdx.x;
  if (g >= P.atomOff + P.nMol) return;
  binAtom(P, g, pos[g], cellOf, slot, cellCount, bucket, cap, blockCount, spill, spillCount);
}


// ============================================================================================
// Counting sort of atoms by cell: exclusive scan of the per-cell counts, in three passes
// (tile sums, per-replica tile prefix, in-tile scan), then scatter and in-cell ordering.
// ============================================================================================
__global__ void k_scan_tiles(BlockTab tab, const RepConst *__restrict__ rc, const RepState *st,
                             const int *__restrict__ cellCount, int *__restrict__ tileSum,
                             int forceRebuild) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  if (!rebuilding(st + rep, forceRebuild)) return;
  const RepConst &P = rc[rep];
  const int c0 = tab.start[blockIdx.x];  // local cell index of the tile start
  int s = 0;
  for (int c = c0 + threadIdx.x; c < c0 + kCellTile; c += blockDim.x) s += cellCount[P.cellOff + c];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  __shared__ int ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    int v = (threadIdx.x < (blockDim.x >> 5)) ? ws[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) tileSum[blockIdx.x] = v;
  }
}

// One block per replica: exclusive prefix over the replica's tiles (tiles of a replica are
// consecutive blocks of the tile table starting at tileFirst[rep]).  Block 0 also clears the
// list build's work counters (work, if not NULL) for k_scan_final and k_build_nebr.
__global__ void k_scan_tile_prefix(const RepConst *__restrict__ rc, const RepState *st,
                                   const int *__restrict__ tileFirst, int *__restrict__ tileSum,
                                   int forceRebuild, int *__restrict__ work) {
  pdlEnter();
  if (work && blockIdx.x == 0 && threadIdx.x < 3) work[threadIdx.x] = 0;
  const int rep = blockIdx.x;
  if (!rebuilding(st + rep, forceRebuild)) return;
  const RepConst &P = rc[rep];
  const int t0 = tileFirst[rep];
  const int nt = P.ncellsPad / kCellTile;
  __shared__ int carry;
  __shared__ int ws[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nt; base += blockDim.x) {
    const int t = base + threadIdx.x;
    int v = (t < nt) ? tileSum[t0 + t] : 0;
    // inclusive warp scan
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if ((threadIdx.x & 31) >= o) x += y;
    }
    if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      int w = (threadIdx.x < (blockDim.x >> 5)) ? ws[threadIdx.x] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, w, o);
        if (threadIdx.x >= o) w += y;
      }
      ws[threadIdx.x] = w;
    }
    __syncthreads();
    const int warpPrefix = (threadIdx.x >= 32) ? ws[(threadIdx.x >> 5) - 1] : 0;
    const int excl = carry + warpPrefix + x - v;
    if (t < nt) tileSum[t0 + t] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
}

// In-tile exclusive scan; writes global cellStart (index into the sorted arrays) and clears
// the counts for the next rebuild.  Also records the largest cell occupancy.
__global__ void k_scan_final(BlockTab tab, const RepConst *__restrict__ rc, RepState *st,
                             int *__restrict__ cellCount, const int *__restrict__ tileSum,
                             int *__restrict__ cellStart, int blockSizeCap, int forceRebuild,
                             int *__restrict__ active, int2 *__restrict__ heavy, int *__restrict__ work,
                             int itemAtoms) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  RepState *S = st + rep;
  if (!rebuilding(S, forceRebuild)) return;
  const RepConst &P = rc[rep];
  const int c0 = tab.start[blockIdx.x];
  constexpr int kPer = kCellTile / 256;  // launched with 256 threads
  int v[kPer];
  int sum = 0, occ = 0, over = 0;
  const int cb = P.cellOff + c0 + threadIdx.x * kPer;
#pragma unroll
  for (int i = 0; i < kPer; i++) {
    v[i] = cellCount[cb + i];
    occ = max(occ, v[i]);
    over += (v[i] > blockSizeCap) ? 1 : 0;
    sum += v[i];
  }
  __shared__ int ws[8];
  int x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) >= o) x += y;
  }
  if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x < 32) {
    int w = (threadIdx.x < 8) ? ws[threadIdx.x] : 0;
    for (int o = 1; o < 8; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (threadIdx.x >= o) w += y;
    }
    if (threadIdx.x < 8) ws[threadIdx.x] = w;
  }
  __syncthreads();
  int run = P.atomOff + tileSum[blockIdx.x] + ((threadIdx.x >= 32) ? ws[(threadIdx.x >> 5) - 1] : 0) + x - sum;
#pragma unroll
  for (int i = 0; i < kPer; i++) {
    cellStart[cb + i] = run;
    run += v[i];
    cellCount[cb + i] = 0;
  }
  // work items of the list build (any order): a cell of up to itemAtoms atoms is one item; a
  // cell of n > itemAtoms atoms is split into k = ceil(n / itemAtoms) items of n / k home atoms
  // (rounded), queued apart so that the list build takes them first.  A split item is
  // {cell, first home atom << 16 | home atoms}.
  int nLight = 0, nHeavy = 0;
#pragma unroll
  for (int i = 0; i < kPer; i++) {
    if (v[i] > 0 && c0 + threadIdx.x * kPer + i < P.ncells) {
      if (v[i] > itemAtoms) nHeavy += (v[i] + itemAtoms - 1) / itemAtoms;
      else nLight++;
    }
  }
  int preL = nLight, preH = nHeavy;
  for (int o = 1; o < 32; o <<= 1) {
    const int yl = __shfl_up_sync(0xffffffffu, preL, o);
    const int yh = __shfl_up_sync(0xffffffffu, preH, o);
    if ((threadIdx.x & 31) >= o) { preL += yl; preH += yh; }
  }
  const int sumL = __shfl_sync(0xffffffffu, preL, 31), sumH = __shfl_sync(0xffffffffu, preH, 31);
  int baseL = 0, baseH = 0;
  if ((threadIdx.x & 31) == 31) {
    if (sumL > 0) baseL = atomicAdd(&work[1], sumL);
    if (sumH > 0) baseH = atomicAdd(&work[2], sumH);
  }
  int outL = __shfl_sync(0xffffffffu, baseL, 31) + preL - nLight;
  int outH = __shfl_sync(0xffffffffu, baseH, 31) + preH - nHeavy;
#pragma unroll
  for (int i = 0; i < kPer; i++) {
    if (v[i] > 0 && c0 + threadIdx.x * kPer + i < P.ncells) {
      if (v[i] > itemAtoms) {
        const int k = (v[i] + itemAtoms - 1) / itemAtoms;
        for (int j = 0; j < k; j++) {
          const int h0 = j * v[i] / k, h1 = (j + 1) * v[i] / k;
          heavy[outH++] = make_int2(cb + i, (h0 << 16) | (h1 - h0));
        }
      } else {
        active[outL++] = cb + i;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    occ = max(occ, __shfl_xor_sync(0xffffffffu, occ, o));
    over += __shfl_xor_sync(0xffffffffu, over, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (occ > 0) atomicMax(&S->maxCellOcc, occ);
    if (over > 0) {
      atomicAdd(&S->cellOverflow, over);
      setFlag(S, 11 /*SG_ERR_CELL_OVERFLOW*/);
    }
  }
}

// Scatter atoms into their cell segments in arrival order.
__global__ void k_scatter(BlockTab tab, const RepConst *__restrict__ rc, RepState *st,
                          const int *__restrict__ cellOf, const int *__restrict__ slot,
                          const int *__restrict__ cellStart, int *__restrict__ tmpIdx,
                          int *__restrict__ nn, int *__restrict__ ns, int *__restrict__ nrl,
                          int forceRebuild) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  RepState *S = st + rep;
  if (!rebuilding(S, forceRebuild)) return;
  const RepConst &P = rc[rep];
  const int g = tab.start[blockIdx.x] + threadIdx.x;
  if (g >= P.atomOff + P.nMol) return;
  const int c = cellOf[g];
  if (c >= 0) {
    tmpIdx[cellStart[P.cellOff + c] + slot[g]] = g;
  } else {
    nn[g] = 0;  // an atom outside the grid has no neighbours (the reference clears NN)
    ns[g] = 0;
    nrl[g] = 0;
    atomicAdd(&S->cellRange, 1);
  }
}

// Order each cell by ascending atom index: the rank of an atom is the number of atoms of its
// cell with a smaller index.  Writes the sorted index and a sorted position copy whose w holds
// the atom index (as int bits) for the neighbour search.
__global__ void k_rank(BlockTab tab, const RepConst *__restrict__ rc, const RepState *st,
                       const int *__restrict__ cellOf, const int *__restrict__ cellStart,
                       const int *__restrict__ tmpIdx, const float4 *__restrict__ pos,
                       int *__restrict__ sortIdx, float4 *__restrict__ sortPos, int forceRebuild) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  if (!rebuilding(st + rep, forceRebuild)) return;
  const RepConst &P = rc[rep];
  const int g = tab.start[blockIdx.x] + threadIdx.x;
  if (g >= P.atomOff + P.nMol) return;
  const int c = cellOf[g];
  if (c < 0) return;
  const int b = cellStart[P.cellOff + c], e = cellStart[P.cellOff + c + 1];
  int rank = 0;
  for (int q = b; q < e; q++) rank += (tmpIdx[q] < g) ? 1 : 0;
  sortIdx[b + rank] = g;
  float4 r = pos[g];
  r.w = __int_as_float(g);
  sortPos[b + rank] = r;
}

// k_scan_rank: one block of kScanRankThreads threads per CELLS cells (sg_lists.cuh).
template <int CELLS>
__global__ void __launch_bounds__(kScanRankThreads) k_scan_rank(const int *__restrict__ tileRep,
                                                          const int *__restrict__ tileStart,
                                                          const int *__restrict__ tileFirst,
                                                          const RepConst *__restrict__ rc, RepState *st,
                                                          int *__restrict__ cellCount, int *__restrict__ cellStart,
                                                          int cap, int forceRebuild, int *__restrict__ active,
                                                          int2 *__restrict__ heavy, int *__restrict__ work,
                                                          int itemAtoms, const int *__restrict__ blockCount,
                                                          const int *__restrict__ bucket, const int *__restrict__ cellOf,
                                                          const float4 *__restrict__ pos, int *__restrict__ sortIdx,
                                                          float4 *__restrict__ sortPos, int *__restrict__ nn,
                                                          int *__restrict__ ns, int *__restrict__ nrl,
                                                          const int2 *__restrict__ spill) {
  pdlEnter();
  scanRankBody<CELLS, kScanRankThreads>(blockIdx.x, tileRep, tileStart, tileFirst, rc, st, cellCount, cellStart, cap,
                                        forceRebuild, active, heavy, work, itemAtoms, blockCount, bucket, cellOf,
                                        pos, sortIdx, sortPos, nn, ns, nrl, spill);
}

// k_scan_rank with `cells` (kScanCells or 2 kScanCells) cells per block.
cudaError_t launchScanRank(bool pdl, int cells, int grid, cudaStream_t s, const int *tileRep, const int *tileStart,
                           const int *tileFirst, const RepConst *rc, RepState *st, int *cellCount, int *cellStart,
                           int cap, int forceRebuild, int *active, int2 *heavy, int *work, int itemAtoms,
                           const int *blockCount, const int *bucket, const int2 *spill, const int *cellOf,
                           const float4 *pos, int *sortIdx, float4 *sortPos, int *nn, int *ns, int *nrl) {
  if (cells == 2 * kScanCells)
    return launchK(pdl, k_scan_rank<2 * kScanCells>, grid, kScanRankThreads, 0, s, tileRep, tileStart, tileFirst, rc,
                   st, cellCount, cellStart, cap, forceRebuild, active, heavy, work, itemAtoms, blockCount, bucket,
                   cellOf, pos, sortIdx, sortPos, nn, ns, nrl, spill);
  return launchK(pdl, k_scan_rank<kScanCells>, grid, kScanRankThreads, 0, s, tileRep, tileStart, tileFirst, rc, st,
                 cellCount, cellStart, cap, forceRebuild, active, heavy, work, itemAtoms, blockCount, bucket, cellOf,
                 pos, sortIdx, sortPos, nn, ns, nrl, spill);
}

#define SG_NEBR_PARAMS                                                                                 \
  const int *__restrict__ tileRep, const int *__restrict__ active, const int2 *__restrict__ heavy,      \
      int *work, const RepConst *__restrict__ rc, RepState *st, const int *__restrict__ cellStart,     \
      const float4 *__restrict__ sortPos, int *__restrict__ nn, int *__restrict__ nbl,                 \
      int *__restrict__ ns, int *__restrict__ sl, int *__restrict__ nrl, unsigned *__restrict__ rl,    \
      int rowStride, int nebrMax, int descending, int *__restrict__ blockCount, int nBlockCount
#define SG_NEBR_ARGS \
  tileRep, active, heavy, work, rc, st, cellStart, sortPos, nn, nbl, ns, sl, nrl, rl, rowStride, nebrMax, descending
// 72 registers a thread, seven blocks (28 warps) an SM: the kernel is bound by instruction
// issue, and at 64 registers (eight blocks) the compiler fits the loop's state with extra
// instructions (on the 45,546-atom workload: 30.5-30.8 us at 72 registers, 31.1-31.4 at 80,
// 33.0-33.3 at 64)
__global__ void __launch_bounds__(kNebrWarps * 32, 7) k_build_nebr(SG_NEBR_PARAMS) {
  pdlEnter();
  clearBlockCount(blockCount, nBlockCount);
  nebrFusedBody(SG_NEBR_ARGS);
}
__global__ void __launch_bounds__(kNebrWarps * 32) k_build_nebr_lanes(SG_NEBR_PARAMS) {
  pdlEnter();
  clearBlockCount(blockCount, nBlockCount);
  nebrLanesBody(SG_NEBR_ARGS);
}
#undef SG_NEBR_PARAMS
#undef SG_NEBR_ARGS

// The force passes (sg_forces.cuh) under their PLAIN names.
}  // namespace sg
#define SG_KN(name) name
#include "sg_forces.cuh"
namespace sg {

// ============================================================================================
// Neighbour list, atom-centric (the same lists as k_build_nebr).  One thread per atom, threads
// in the cell-sorted order, so that the lanes of a warp mostly share their home cell and read
// the same candidates.  Each thread walks the 27 stencil cells in the reference's order and
// each cell in ascending atom index, which is the reference's list order itself, and appends
// every hit to the atom's full list and, for a carbon atom, to its close list and relevant
// list, with the same arithmetic and limits as k_build_nebr.  The counters of the cell-window
// build are not used and are cleared here.
// ============================================================================================
__global__ void __launch_bounds__(128) k_build_nebr_atoms(BlockTab tab, const RepConst *__restrict__ rc,
                                                          RepState *st, const int *__restrict__ cellOf,
                                                          const int *__restrict__ cellStart,
                                                          const float4 *__restrict__ sortPos,
                                                          int *__restrict__ nn, int *__restrict__ nbl,
                                                          int *__restrict__ ns, int *__restrict__ sl,
                                                          int *__restrict__ nrl, unsigned *__restrict__ rl,
                                                          int rowStride, int nebrMax, int *__restrict__ work,
                                                          int forceRebuild, int *__restrict__ blockCount,
                                                          int nBlockCount) {
  pdlEnter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nBlockCount; i += gridDim.x * blockDim.x)
    blockCount[i] = 0;  // k_scan_rank has read them
  if (blockIdx.x == 0 && threadIdx.x < 4) work[threadIdx.x] = 0;
  const int rep = tab.rep[blockIdx.x];
  RepState *S = st + rep;
  if (!rebuilding(S, forceRebuild)) return;
  const RepConst &P = rc[rep];
  const int s = tab.start[blockIdx.x] + threadIdx.x;  // sorted position
  const int sortedEnd = cellStart[P.cellOff + P.ncells];  // atoms outside the grid are not sorted
  const bool valid = s < sortedEnd;
  int n = 0;
  if (valid) {
    const float4 A = sortPos[s];
    const int g = __float_as_int(A.w);
    const int c = cellOf[g];
    const int metalEnd = P.atomOff + P.nMolMe;
    const bool carbon = g >= metalEnd;
    const float rrNebr = P.rrNebr, rrShort = P.rrShort;
    int *row = nbl + (size_t)g * rowStride;
    int *srow = sl + (size_t)g * kShortMax;
    unsigned *rrow = rl + (size_t)g * kRelMax;
    int m = 0, r = 0;
    for (int o = 0; o < 27; o++) {
      float sx, sy, sz;
      const int C = P.cellOff + stencilCell(P, c, o, sx, sy, sz);
      const int qb = cellStart[C], qe = cellStart[C + 1];
      for (int q = qb; q < qe; q++) {
        const float4 B = sortPos[q];
        const int k = __float_as_int(B.w);
        // the reference subtracts the cell shift after the difference: both roundings kept
        float dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
        dx = dx - sx; dy = dy - sy; dz = dz - sz;
        const float rr = dx * dx + dy * dy + dz * dz;
        if (rr < rrNebr && k != g) {
          if (n < nebrMax) row[n] = k;
          if (carbon) {
            const bool close = rr < rrShort;
            if (close) {
              if (m < kShortMax) srow[m] = k;
              m++;
            }
            if (close || k < metalEnd) {
              if (r < kRelMax) rrow[r] = relPack(k - P.atomOff, n);
              r++;
            }
          }
          n++;
        }
      }
    }
    nn[g] = min(n, nebrMax);
    // -1: the carbon pass walks the full list instead
    ns[g] = carbon ? ((m > kShortMax || n > nebrMax) ? -1 : m) : 0;
    nrl[g] = carbon ? ((r > kRelMax || n > nebrMax || n > kRelPosLimit) ? -1 : r) : 0;
  }
  int want = n, over = (n > nebrMax) ? 1 : 0;
  for (int off = 16; off > 0; off >>= 1) {
    want = max(want, __shfl_xor_sync(0xffffffffu, want, off));
    over += __shfl_xor_sync(0xffffffffu, over, off);
  }
  if ((threadIdx.x & 31) == 0) {
    if (want > 0) atomicMax(&S->maxNeighbours, want);
    if (over > 0) {
      atomicAdd(&S->nebrOverflow, over);
      setFlag(S, 5 /*SG_ERR_NEBR_OVERFLOW*/);
    }
  }
}

// ============================================================================================
// Reductions in the reference's tree order (cu:1101-1892): a block of 512 threads reduces the
// 1024 elements [1024 b, 1024 b + 1024) with the stride-halving tree, the last block of the
// replica reduces the block partials in a zero-padded 1024-slot tree.
// ============================================================================================
__device__ __forceinline__ int slotOp(int s) {  // 0 add, 1 max, 2 min
  return (s == RS_VVMAX || (s >= RS_MAX_X && s <= RS_MAX_Z)) ? 1 : (s >= RS_MIN_X && s <= RS_MIN_Z) ? 2 : 0;
}
__device__ __forceinline__ float combine(int op, float a, float b) {
  if (op == 0) return a + b;
  if (op == 1) return (a < b) ? b : a;
  return (a > b) ? b : a;
}

// Tree over 512 per-thread values (after the first level, done in registers), for NV <= 16
// values per element, in the reference's pairing (x[t] += x[t + s] for s = 256 ... 1).  The
// values go through shared memory once; warp v then owns value v, its lane l holding the
// entries t = l + 32 k, k = 0..15, so the strides s >= 32 pair registers of the same lane and
// the strides 16..1 are shuffles.  Result valid in lane 0 of warp v (returned to thread 0 via
// shared memory in x[] of thread 0).
template <int NV>
__device__ __forceinline__ void blockTree512(float (&x)[NV], const int *ops, float (*sh)[kRedThreads]) {
  const int t = threadIdx.x;
  const int w = t >> 5, l = t & 31;
#pragma unroll
  for (int v = 0; v < NV; v++) sh[v][t] = x[v];
  __syncthreads();
  __shared__ float res[16];
  if (w < NV) {
    const int op = ops[w];
    float e[16];
#pragma unroll
    for (int k = 0; k < 16; k++) e[k] = sh[w][l + 32 * k];
#pragma unroll
    for (int k = 0; k < 8; k++) e[k] = combine(op, e[k], e[k + 8]);  // s = 256
#pragma unroll
    for (int k = 0; k < 4; k++) e[k] = combine(op, e[k], e[k + 4]);  // s = 128
#pragma unroll
    for (int k = 0; k < 2; k++) e[k] = combine(op, e[k], e[k + 2]);  // s = 64
    float y = combine(op, e[0], e[1]);                              // s = 32
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) y = combine(op, y, __shfl_down_sync(0xffffffffu, y, s));
    if (l == 0) res[w] = y;
  }
  __syncthreads();
  if (t == 0) {
#pragma unroll
    for (int v = 0; v < NV; v++) x[v] = res[v];
  }
  __syncthreads();
}

// Centre-of-mass velocity of the metal (ComputeCmVelK, cu:1560-1638) on the velocities after
// the second half kick, which k_step_reduce applies; launched over the metal reduction blocks.
__global__ void __launch_bounds__(kRedThreads) k_cmvel(BlockTab tab, const RepConst *__restrict__ rc,
                                                       RepState *st, const float4 *__restrict__ vel,
                                                       const float4 *__restrict__ acc,
                                                       float *__restrict__ partial,
                                                       const int *__restrict__ redFirst) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  RepState *S = st + rep;
  const int b = tab.start[blockIdx.x];  // local reduction block index
  const int t = threadIdx.x;
  const float h = 0.5f * P.deltaT;
  float e[2][3];
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int local = kRedElems * b + half * kRedThreads + t;
    if (local < P.nMolMe) {
      const float4 v = vel[P.atomOff + local];
      const float4 a = acc[P.atomOff + local];
      e[half][0] = v.x + h * a.x;
      e[half][1] = v.y + h * a.y;
      e[half][2] = v.z + h * a.z;
    } else {
      e[half][0] = e[half][1] = e[half][2] = 0.f;
    }
  }
  float x[3] = {e[0][0] + e[1][0], e[0][1] + e[1][1], e[0][2] + e[1][2]};
  __shared__ float sh[3][kRedThreads];
  const int ops[3] = {0, 0, 0};
  blockTree512<3>(x, ops, sh);
  __shared__ bool last;
  float *part = partial + (size_t)redFirst[rep] * 3;
  const int nMetalBlocks = (P.nMolMe + kRedElems - 1) / kRedElems;
  if (t == 0) {
    part[3 * b + 0] = x[0]; part[3 * b + 1] = x[1]; part[3 * b + 2] = x[2];
    __threadfence();
    const unsigned prev = atomicAdd(&S->cmvCounter, 1u);
    last = (prev == (unsigned)nMetalBlocks - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // final tree over the block partials (slots beyond the metal blocks are zero, as the
  // reference's non-metal blocks contribute zero sums)
  float y[3] = {0.f, 0.f, 0.f};
  float carry[3] = {0.f, 0.f, 0.f};
  for (int base = 0; base < nMetalBlocks; base += kRedElems) {
    float lo[3], hi[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      lo[c] = (base + t < nMetalBlocks) ? __ldcg(part + 3 * (base + t) + c) : 0.f;
      hi[c] = (base + kRedThreads + t < nMetalBlocks) ? __ldcg(part + 3 * (base + kRedThreads + t) + c) : 0.f;
      y[c] = lo[c] + hi[c];
    }
    __syncthreads();
    blockTree512<3>(y, ops, sh);
    if (t == 0) {
#pragma unroll
      for (int c = 0; c < 3; c++) carry[c] = (base == 0) ? y[c] : carry[c] + y[c];
    }
    __syncthreads();
  }
  if (t == 0) {
    S->cmVel[0] = carry[0]; S->cmVel[1] = carry[1]; S->cmVel[2] = carry[2];
    S->cmvCounter = 0;
  }
}

// Per-element values of the step reduction for local atom index `local`.
__device__ __forceinline__ void stepElem(const RepConst &P, int local, const float4 &r,
                                         const float4 &v, float frc, float cmVelX,
                                         float (&e)[kNumRed]) {
  if (local >= P.nMol) {
#pragma unroll
    for (int s = 0; s < kNumRed; s++) e[s] = 0.f;
    return;
  }
  const bool metal = local < P.nMolMe;
  e[RS_VSUM_X] = metal ? P.massMe * v.x : v.x;  // cu:1123-1126
  e[RS_VSUM_Y] = v.y;
  e[RS_VSUM_Z] = v.z;
  e[RS_VVMAX] = v.x * v.x + v.y * v.y + v.z * v.z;
  float vx = v.x;
  if (P.iRegime == 2 && metal) vx = vx - cmVelX;  // cu:1230-1234
  float vv = vx * vx + v.y * v.y + v.z * v.z;
  if (metal) vv = P.massMe * vv;
  e[RS_VVSUM] = vv;
  e[RS_USUM] = r.w;
  e[RS_CM_X] = metal ? r.x : 0.f;
  e[RS_CM_Y] = metal ? r.y : 0.f;
  e[RS_CM_Z] = metal ? r.z : 0.f;
  e[RS_MIN_X] = e[RS_CM_X]; e[RS_MIN_Y] = e[RS_CM_Y]; e[RS_MIN_Z] = e[RS_CM_Z];
  e[RS_MAX_X] = e[RS_CM_X]; e[RS_MAX_Y] = e[RS_CM_Y]; e[RS_MAX_Z] = e[RS_CM_Z];
  e[RS_FRICT] = metal ? frc : 0.f;
}

__device__ void stepControl(const RepConst &P, RepState *S, const float (&red)[kNumRed],
                            float *diff, int forceRebuild);

// Verlet part 2 (LeapfrogStepK part==2, cu:2253) fused with all property reductions of the
// step; the last block of each replica runs the step's scalar control (stepControl).
__global__ void __launch_bounds__(kRedThreads) k_step_reduce(
    BlockTab tab, const RepConst *__restrict__ rc, RepState *st, const float4 *__restrict__ pos,
    float4 *__restrict__ vel, const float4 *__restrict__ acc, const float *__restrict__ fric,
    float *__restrict__ partial, const int *__restrict__ redFirst, float *__restrict__ diffBuf,
    const size_t *__restrict__ diffOff, int forceRebuild, PublishArgs pub) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  RepState *S = st + rep;
  const int b = tab.start[blockIdx.x];
  const int t = threadIdx.x;
  const float h = 0.5f * P.deltaT;
  const float cmVelX = (P.nMolMe != 0) ? S->cmVel[0] / (float)P.nMolMe : 0.f;
  float e0[kNumRed], e1[kNumRed];
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int local = kRedElems * b + half * kRedThreads + t;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f), v = r;
    float frc = 0.f;
    if (local < P.nMol) {
      const int g = P.atomOff + local;
      r = pos[g];
      v = vel[g];
      if (!isFrozen(P, local, r.x, r.y)) {
        const float4 a = acc[g];
        v.x = v.x + h * a.x;
        v.y = v.y + h * a.y;
        v.z = v.z + h * a.z;
        vel[g] = v;
      }
      if (local < P.nMolMe && P.hasFric) frc = fric[g];
    }
    if (half == 0) stepElem(P, local, r, v, frc, cmVelX, e0);
    else stepElem(P, local, r, v, frc, cmVelX, e1);
  }
  int ops[kNumRed];
  float x[kNumRed];
#pragma unroll
  for (int s = 0; s < kNumRed; s++) {
    ops[s] = slotOp(s);
    x[s] = combine(ops[s], e0[s], e1[s]);
  }
  // the replica's constants and state into shared memory for the step control of whichever
  // block finishes last, loaded by every block before its tree (in this launch only the
  // counter of the blocks changes, and the last block resets its copy)
  __shared__ RepState sS;
  __shared__ RepConst sP;
  constToShared(&P, &sP);
  {
    const int *ss = reinterpret_cast<const int *>(S);
    int *sd = reinterpret_cast<int *>(&sS);
    for (int i = t; i < (int)(sizeof(RepState) / 4); i += kRedThreads) sd[i] = __ldcg(ss + i);
  }
  __shared__ float sh[kNumRed][kRedThreads];
  blockTree512<kNumRed>(x, ops, sh);
  __shared__ bool last;
  float *part = partial + (size_t)redFirst[rep] * kNumRed;
  if (t == 0) {
#pragma unroll
    for (int s = 0; s < kNumRed; s++) part[kNumRed * b + s] = x[s];
    __threadfence();
    const unsigned prev = atomicAdd(&S->redCounter, 1u);
    last = (prev == (unsigned)P.nRedBlocks - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  float y[kNumRed], carry[kNumRed];
  for (int base = 0; base < P.nRedBlocks; base += kRedElems) {
#pragma unroll
    for (int s = 0; s < kNumRed; s++) {
      const float lo = (base + t < P.nRedBlocks) ? __ldcg(part + kNumRed * (base + t) + s) : 0.f;
      const float hi = (base + kRedThreads + t < P.nRedBlocks) ? __ldcg(part + kNumRed * (base + kRedThreads + t) + s) : 0.f;
      y[s] = combine(ops[s], lo, hi);
    }
    __syncthreads();
    blockTree512<kNumRed>(y, ops, sh);
    if (t == 0) {
#pragma unroll
      for (int s = 0; s < kNumRed; s++) carry[s] = (base == 0) ? y[s] : combine(ops[s], carry[s], y[s]);
    }
    __syncthreads();
  }
  __shared__ float red[kNumRed];
  if (t == 0) {
#pragma unroll
    for (int s = 0; s < kNumRed; s++) red[s] = carry[s];
  }
  __syncthreads();
  float redv[kNumRed];
#pragma unroll
  for (int s = 0; s < kNumRed; s++) redv[s] = red[s];
  if (t == 0) sS.redCounter = 0;  // every block has counted in: ready for the next step
  stepControl(sP, &sS, redv, diffBuf ? diffBuf + diffOff[rep] : nullptr, forceRebuild);
  stateFromShared(&sS, S);
  if (pub.hostSt) publishReplica(&sS, rep, pub);
}

// Nint of ComputeDefs.h:70-71 (evaluated in double because of the 0.5 literal).
__device__ __forceinline__ int nintRef(float x) {
  return (x < 0.) ? (-(int)(0.5 - (double)x)) : ((int)(0.5 + (double)x));
}

// Scalar control of one step, run by the whole last block of the replica: the host-side
// statements of the reference step loop (cu:2305-2395, 2398-2414 bookkeeping, 2439-2445),
// the nanoparticle diffusion sample (EvalDiffusion/AccumDiffusion, cu:2898-2952), the
// thermostat decision (cu:2362-2373) and the rebuild criterion (cu:2389-2391).
__device__ void stepControl(const RepConst &P, RepState *S, const float (&red)[kNumRed],
                            float *diff, int forceRebuild) {
  const int t = threadIdx.x;
  const int sc = S->stepCount + 1;
  __shared__ int diffDue, accumNb[16], printNow;
  __shared__ float cmc[3];
  // the step's scalars in three independent parts, each on lane 0 of its own warp (no two of
  // them write the same field); the property sums after them
  if (t == 0) {
    // reduced values, metal centre of mass and its velocity, friction force, diffusion sample
#pragma unroll
    for (int s = 0; s < kNumRed; s++) S->red[s] = red[s];
    diffDue = 0;
    if (P.nMolMe != 0) {
      S->cmVal = red[RS_CM_X] / P.nMolMe;
      S->cmVelVal = S->cmVel[0] / P.nMolMe;
      S->frictVal = P.hasFric ? red[RS_FRICT] : 0.f;
      if (P.iRegime == 2 && sc > P.stepEquil && ((sc - P.stepEquil) % P.stepDiffuse == 0) && diff) {
        diffDue = 1;
        cmc[0] = red[RS_CM_X] / P.nMolMe;
        cmc[1] = red[RS_CM_Y] / P.nMolMe;
        cmc[2] = red[RS_CM_Z] / P.nMolMe;
      }
    } else {
      S->cmVal = 0.f; S->cmVelVal = 0.f; S->frictVal = 0.f;
    }
  } else if (t == 32) {
    // thermostat decision and energies
    const float vvSum = red[RS_VVSUM], uSum = red[RS_USUM];
    const bool thermo = ((P.iRegime == 2) && (sc > P.stepEquil) && (sc % P.stepThermostat == 0)) ||
                        ((P.iRegime == 1) && (sc % P.stepThermostat == 0));
    if (thermo) {
      const float kin = vvSum * 0.5f / P.nMol;
      S->betaC = sqrtf(1.f + P.gammaBerendsen * (P.temperature * 1.5f * P.kB / kin - 1.f));
      S->betaM = sqrtf(1.f + P.gammaBerendsen * (P.temperature * P.kB / kin - 1.f));
      S->thermoMetal = (P.iRegime == 2) && (sc > P.stepEquil) && (sc < P.stepEquil + P.stepCool);
      S->thermoPending = 1;
    } else {
      S->thermoPending = 0;
    }
    const float ke = 0.5f * vvSum / P.nMol, pe = uSum / P.nMol;
    S->ke = ke;
    S->pe = pe;
    S->te = ke + pe;
    S->ke64 = (double)ke;
    S->pe64 = (double)pe;
  } else if (t == 64) {
    // rebuild criterion, shear drive schedule, deposition
    if (forceRebuild || S->nebrNow) {
      S->nebrNow = 0;
      S->dispHi = 0.f;
      S->rebuilds++;
    }
    S->dispHi += sqrtf(red[RS_VVMAX]) * P.deltaT;
    if (S->dispHi > 0.5f * P.rNebrShell) S->nebrNow = 1;
    if (P.iRegime == 2 && P.nMolMe != 0 && sc > P.stepEquil + P.stepCool) {
      if (S->cmVel[0] / P.nMolMe < 0.005f) S->shear += P.deltaF;  // cmVelVal
      S->shearCount = 0;
    }
    if (P.iRegime == 1) {
      int nDep, nTo;
      bool act;
      depositionPlan(P, *S, sc, nDep, nTo, act);
      if (act) S->nMolDeposited = nDep + nTo;
    }
  }
  __syncthreads();
  // AccumProps(1) for every property but oneStep (host-side); the stepAvg snapshot
  if (t < 7 && t != 3) {
    const float val = (t == 0) ? S->te : (t == 1) ? S->pe : (t == 2) ? S->ke : (t == 4) ? S->cmVal
                    : (t == 5) ? S->cmVelVal : S->frictVal;
    S->props[t][0] = val;
    const float s1 = S->props[t][1] + val, s2 = S->props[t][2] + val * val;
    if (sc % P.stepAvg == 0) {
      S->propsSnap[t][0] = val;
      S->propsSnap[t][1] = s1;
      S->propsSnap[t][2] = s2;
      S->props[t][1] = 0.f;
      S->props[t][2] = 0.f;
    } else {
      S->props[t][1] = s1;
      S->props[t][2] = s2;
    }
  } else if (t == 3 && sc % P.stepAvg == 0) {
    S->propsSnap[3][0] = S->props[3][0];
    S->propsSnap[3][1] = S->props[3][1];
    S->propsSnap[3][2] = S->props[3][2];
    S->props[3][1] = 0.f;
    S->props[3][2] = 0.f;
  }
  if (t == 32) {
    if (sc % P.stepAvg == 0) S->snapStep = sc;
    S->stepCount = sc;
  }
  __syncthreads();
  if (!diffDue) return;
  // ---- diffusion sample (device copy of TBuf/rrDiffuseAv) ----
  const int nB = P.nBuffDiffuse, nV = P.nValDiffuse;
  float *tb = diff;                        // 7 floats per buffer
  float *rr = diff + (size_t)nB * 7;       // nB x nV
  float *av = rr + (size_t)nB * nV;        // nV
  float *pr = av + nV;                     // nV (last finished table)
  // one thread per buffer (the buffers are independent); the accumulation below runs only in
  // a step where a buffer fills
  int filled = 0;
  {
    for (int nb = t; nb < nB; nb += blockDim.x) {
      float *b = tb + 7 * nb;
      int count = __float_as_int(b[0]);
      if (count == 0) {
        b[1] = cmc[0]; b[2] = cmc[1]; b[3] = cmc[2];
        b[4] = cmc[0]; b[5] = cmc[1]; b[6] = cmc[2];
      }
      if (count >= 0) {
        const int ni = count;
        float *rrb = rr + (size_t)nb * nV;
        rrb[ni] = 0.f;
        float dx = b[4] - cmc[0], dy = b[5] - cmc[1], dz = b[6] - cmc[2];
        dx = dx / P.region[0]; dy = dy / P.region[1]; dz = dz / P.region[2];
        dx = (float)nintRef(dx); dy = (float)nintRef(dy); dz = (float)nintRef(dz);
        dx = dx * P.region[0]; dy = dy * P.region[1]; dz = dz * P.region[2];
        b[4] = cmc[0] + dx; b[5] = cmc[1] + dy; b[6] = cmc[2] + dz;
        dx = b[4] - b[1]; dy = b[5] - b[2]; dz = b[6] - b[3];
        rrb[ni] += dx * dx + dy * dy + dz * dz;
      }
      b[0] = __int_as_float(count + 1);
      filled |= (count + 1 == nV) ? 1 : 0;
    }
  }
  if (!__syncthreads_or(filled)) return;
  for (int nb = 0; nb < nB; nb++) {
    if (t == 0) {
      accumNb[0] = (__float_as_int(tb[7 * nb]) == nV);
      printNow = 0;
    }
    __syncthreads();
    if (accumNb[0]) {
      const float *rrb = rr + (size_t)nb * nV;
      for (int j = t; j < nV; j += blockDim.x) av[j] += rrb[j];
      __syncthreads();
      if (t == 0) {
        tb[7 * nb] = __int_as_float(0);
        S->countDiffuseAv++;
        printNow = (S->countDiffuseAv == P.limitDiffuseAv);
      }
      __syncthreads();
      if (printNow) {
        const int ia = 3 * 2 * P.stepDiffuse;
        const float fa = (float)ia * P.deltaT * (float)P.limitDiffuseAv;
        const float fac = (float)(1. / (double)fa);
        for (int j = t; j < nV; j += blockDim.x) {
          float vj = av[j];
          if (j >= 1) vj *= fac / j;
          pr[j] = vj;
          av[j] = 0.f;
        }
        __syncthreads();
        if (t == 0) {
          S->countDiffuseAv = 0;
          S->diffPrints++;
        }
      }
    }
    __syncthreads();
  }
}

// Shear drive (ApplyShearK, cu:517-534; schedule cu:2398-2413): after the step's control has
// updated the shear value, add it to a.x of metal atoms left of the centre of mass.
__global__ void k_shear(BlockTab tab, const RepConst *__restrict__ rc, RepState *st,
                        const float4 *__restrict__ pos, float4 *__restrict__ acc) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  RepState *S = st + rep;
  const int i = tab.start[blockIdx.x] + threadIdx.x;
  const int metalEnd = P.atomOff + P.nMolMe;
  const int sc = S->stepCount;  // already advanced by the control
  const bool active = (P.iRegime == 2) && (P.nMolMe != 0) && (sc > P.stepEquil + P.stepCool);
  if (!active) return;
  unsigned hit = 0;
  if (i < metalEnd) {
    const float dR = S->cmVal - pos[i].x;
    if (dR > 0.f) {
      acc[i].x += S->shear;
      hit = 1;
    }
  }
  unsigned cnt = __popc(__ballot_sync(0xffffffffu, hit));
  __shared__ unsigned bc;
  if (threadIdx.x == 0) bc = 0;
  __syncthreads();
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&bc, cnt);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (bc) atomicAdd(&S->shearCount, bc);
    __threadfence();
    const int nblk = (P.nMolMe + blockDim.x - 1) / blockDim.x;
    const unsigned prev = atomicAdd(&S->shearCounter, 1u);
    if (prev == (unsigned)nblk - 1) {
      __threadfence();
      S->totalShear = atomicAdd(&S->shearCount, 0u) * S->shear;
      S->shearCounter = 0;
    }
  }
}

// ============================================================================================
// RDF sample (EvalRdfK, cu:1895-1999): ordered metal pairs in the 27-cell stencil of the
// last-built cells, current positions.  One warp per metal atom (kRdfAtoms atoms per 128-thread
// block): lanes 0..26 look up the stencil cells (the reference's visiting order), a warp scan
// of their lengths lays the candidates out as one window, and the lanes stride over it, each
// finding its candidate's cell by binary search over the segment offsets.  Bins of the same
// value are merged across the warp (__match_any_sync) before one shared-memory atomic per
// distinct bin; the block adds its histogram to the replica's.  Counts do not depend on the
// order of the pairs, so they are the reference's bit for bit.
// ============================================================================================
__global__ void __launch_bounds__(128) k_rdf(BlockTab tab, const RepConst *__restrict__ rc, RepState *st,
                                             const float4 *__restrict__ pos, const int *__restrict__ cellOf,
                                             const int *__restrict__ cellStart, const int *__restrict__ sortIdx,
                                             unsigned *__restrict__ hist, int histStride) {
  pdlEnter();
  extern __shared__ unsigned shist[];
  __shared__ int sQb[kRdfAtoms][27], sOff[kRdfAtoms][28];
  __shared__ float4 sSh[kRdfAtoms][27];
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  RepState *S = st + rep;
  const int nb = P.sizeHistRdf;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) shist[b] = 0u;
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = tab.start[blockIdx.x] + w;
  const int metalEnd = P.atomOff + P.nMolMe;
  const float range2 = P.rangeRdf * P.rangeRdf;
  int dropped = 0;
  const bool active = (i < metalEnd) && (cellOf[i] >= 0);  // uniform across the warp
  if (active) {
    const float4 A = pos[i];
    const int c = cellOf[i];
    int len = 0;
    if (lane < 27) {
      float sx, sy, sz;
      const int C = stencilCell(P, c, lane, sx, sy, sz);
      const int qb = cellStart[P.cellOff + C];
      len = cellStart[P.cellOff + C + 1] - qb;
      sQb[w][lane] = qb;
      sSh[w][lane] = make_float4(sx, sy, sz, 0.f);
    }
    int incl = len;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += v;
    }
    if (lane < 27) sOff[w][lane] = incl - len;
    const int total = __shfl_sync(0xffffffffu, incl, 26);
    __syncwarp();
    for (int e0 = 0; e0 < total; e0 += 32) {  // the same trip count in every lane
      const int e = e0 + lane;
      int bin = -1;
      if (e < total) {
        int o = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (o + step < 27 && sOff[w][o + step] <= e) o += step;
        const int k = sortIdx[sQb[w][o] + e - sOff[w][o]];
        if (k < metalEnd && k != i) {
          const float4 B = pos[k];
          const float4 sh = sSh[w][o];
          float dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
          dx = dx - sh.x; dy = dy - sh.y; dz = dz - sh.z;
          const float rr = dx * dx + dy * dy + dz * dz;
          if (rr < range2) {
            bin = (int)(sqrtf(rr) * P.intervalRdf);
            if (bin < 0 || bin >= nb) {
              dropped++;
              bin = -1;
            }
          }
        }
      }
      const unsigned same = __match_any_sync(0xffffffffu, bin);
      if (bin >= 0 && lane == __ffs(same) - 1) atomicAdd(&shist[bin], (unsigned)__popc(same));
    }
  }
  __syncthreads();
  unsigned *h = hist + (size_t)rep * histStride;
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
    if (shist[b]) atomicAdd(&h[b], shist[b]);
  // a pair just inside rangeRdf whose bin index rounds up to sizeHistRdf: the reference adds it
  // one element past its histogram (SurfaceGrowth.cu:1988-1989), outside every printed bin; it
  // is dropped here and only counted (sg_diag.rdf_range), not reported as an error
  for (int o = 16; o > 0; o >>= 1) dropped += __shfl_xor_sync(0xffffffffu, dropped, o);
  if (dropped && lane == 0) atomicAdd(&S->rdfRange, dropped);
}


// RDF extension: all metal pairs of a replica within `range` into nbins (0-15 A / 300 bins in
// the benchmark), ordered pairs counted twice like the reference's histogram.  One 64-thread
// block per (A tile, B tile) pair of 64-atom metal tiles with B >= A (the pair table, built
// once per context): the block loads both tiles, takes their bounding boxes and leaves at once
// when the boxes are farther apart in the minimum image than the range (with a margin far above
// rounding) -- metal atoms are numbered cluster by cluster, so most tile pairs of a
// multi-cluster system drop out.  A surviving block walks its 64 x 64 pairs (j > i inside a
// self tile): per B atom every lane has its A atom's bin, lanes with the same bin are merged
// by __match_any_sync and their leader adds the merged count to a shared-memory histogram,
// which the block adds to the replica's global histogram at the end.  The pair tiles spread
// the work over every SM (the former one-block-per-A-tile form ran a serial walk over the
// remaining tiles in 44 blocks).
__global__ void __launch_bounds__(kRdfTile) k_rdf_ext(const RepConst *__restrict__ rc, const float4 *__restrict__ pos,
                                                      const int4 *__restrict__ pairs,
                                                      unsigned long long *__restrict__ hist, int nbins, float range) {
  pdlEnter();
  extern __shared__ unsigned eh[];
  __shared__ float4 tileB[kRdfTile];
  __shared__ float box[kRdfTile / 32][12];
  const int4 w = pairs[blockIdx.x];  // replica, first A atom, first B atom
  const RepConst &P = rc[w.x];
  const int me = P.atomOff + P.nMolMe;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const bool haveA = w.y + t < me, haveB = w.z + t < me;
  const float4 A = haveA ? pos[w.y + t] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 Bt = haveB ? pos[w.z + t] : make_float4(0.f, 0.f, 0.f, 0.f);
  tileB[t] = Bt;
  // bounding boxes of the two tiles: min x, y, z, max x, y, z of A, then of B
  float v[12] = {haveA ? A.x : 3.4e38f, haveA ? A.y : 3.4e38f, haveA ? A.z : 3.4e38f,
                 haveA ? A.x : -3.4e38f, haveA ? A.y : -3.4e38f, haveA ? A.z : -3.4e38f,
                 haveB ? Bt.x : 3.4e38f, haveB ? Bt.y : 3.4e38f, haveB ? Bt.z : 3.4e38f,
                 haveB ? Bt.x : -3.4e38f, haveB ? Bt.y : -3.4e38f, haveB ? Bt.z : -3.4e38f};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < 12; c++) {
      const float u = __shfl_xor_sync(0xffffffffu, v[c], o);
      v[c] = (c % 6 < 3) ? fminf(v[c], u) : fmaxf(v[c], u);
    }
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < 12; c++) box[wid][c] = v[c];
  __syncthreads();
#pragma unroll
  for (int c = 0; c < 12; c++) {
    float m = box[0][c];
#pragma unroll
    for (int k = 1; k < kRdfTile / 32; k++) m = (c % 6 < 3) ? fminf(m, box[k][c]) : fmaxf(m, box[k][c]);
    v[c] = m;
  }
  const float L[3] = {P.region[0], P.region[1], P.region[2]};
  const float invL[3] = {1.f / L[0], 1.f / L[1], 1.f / L[2]};
  const float r2max = range * range;
  // per axis, no pair can be closer in the minimum image than the folded centre distance minus
  // both half extents (every thread computes the same value from the same shared words, so the
  // exit below is uniform across the block)
  float gap2 = 0.f;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float hA = 0.5f * (v[3 + c] - v[c]), hB = 0.5f * (v[9 + c] - v[6 + c]);
    float d = 0.5f * (v[3 + c] + v[c]) - 0.5f * (v[9 + c] + v[6 + c]);
    d -= L[c] * rintf(d * invL[c]);
    const float g = fmaxf(fabsf(d) - hA - hB - 0.01f, 0.f);
    gap2 += g * g;
  }
  if (gap2 > r2max) return;
  for (int b = t; b < nbins; b += kRdfTile) eh[b] = 0u;
  __syncthreads();
  const float scale = nbins / range;
  const bool self = (w.y == w.z);
  const int nj = min(kRdfTile, me - w.z);
  for (int jj = 0; jj < nj; jj++) {
    const float4 B = tileB[jj];
    int bin = -1;
    if (haveA && (!self || jj > t)) {
      float dx = A.x - B.x, dy = A.y - B.y, dz = A.z - B.z;
      dx -= L[0] * rintf(dx * invL[0]);
      dy -= L[1] * rintf(dy * invL[1]);
      dz -= L[2] * rintf(dz * invL[2]);
      const float rr = dx * dx + dy * dy + dz * dz;
      if (rr < r2max) {
        const int b = (int)(sqrtf(rr) * scale);
        if (b < nbins) bin = b;
      }
    }
    const unsigned m = __match_any_sync(0xffffffffu, bin);
    if (bin >= 0 && lane == __ffs(m) - 1) atomicAdd(&eh[bin], 2u * (unsigned)__popc(m));
  }
  __syncthreads();
  for (int b = t; b < nbins; b += kRdfTile)
    if (eh[b]) atomicAdd(&hist[(size_t)w.x * nbins + b], (unsigned long long)eh[b]);
}

// Apply a pending thermostat rescale now (before the state is read back).
__global__ void k_apply_pending(BlockTab tab, const RepConst *__restrict__ rc, RepState *st,
                                float4 *__restrict__ vel) {
  pdlEnter();
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  const RepState *S = st + rep;
  const int g = tab.start[blockIdx.x] + threadIdx.x;
  if (g >= P.atomOff + P.nMol || !S->thermoPending) return;
  const int local = g - P.atomOff;
  float4 v = vel[g];
  if (local >= P.nMolMe) {
    const float b = S->betaC;
    v.x = b * v.x; v.y = b * v.y; v.z = b * v.z;
  } else if (S->thermoMetal) {
    const float b = S->betaM;
    v.x = b * v.x; v.y = b * v.y; v.z = b * v.z;
  } else {
    return;
  }
  vel[g] = v;
}

// float3 host layout <-> float4 device layout
__global__ void k_unpack3(const float *src, float4 *dst, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], 0.f);
}
__global__ void k_pack3(const float4 *src, float *dst, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float4 v = src[i];
    dst[3 * i] = v.x; dst[3 * i + 1] = v.y; dst[3 * i + 2] = v.z;
  }
}

// Floats [3 a0, 3 min(n, a0 + kUnpackAtoms)) of a float3 array into shared memory, read as
// float4 where the array is 16-byte aligned (3 a0 is a multiple of 4), each float once.
__device__ __forceinline__ void stageRows3(const float *src, int n, int a0, float *sm) {
  const int f0 = 3 * a0, f1 = 3 * min(n, a0 + kUnpackAtoms);
  const bool aligned = (reinterpret_cast<uintptr_t>(src) & 15) == 0;
  for (int q = threadIdx.x; 4 * q < f1 - f0; q += blockDim.x) {
    const int f = f0 + 4 * q;
    if (aligned && f + 4 <= f1) {
      const float4 x = reinterpret_cast<const float4 *>(src)[f >> 2];
      sm[4 * q] = x.x; sm[4 * q + 1] = x.y; sm[4 * q + 2] = x.z; sm[4 * q + 3] = x.w;
    } else {
      for (int k = 0; k < 4 && f + k < f1; k++) sm[4 * q + k] = src[f + k];
    }
  }
}

// A state upload's device half, kUnpackAtoms atoms per block: r (sr, when the host array is
// mapped) to pos, v and a (host float3 rows, mapped or staged) to float4 through shared
// memory (coalesced reads over the host link), the low position words cleared (MIXED), and any
// pending thermostat rescale of every replica cancelled.
__global__ void __launch_bounds__(kUnpackAtoms) k_unpack_state(const float4 *sr, const float *sv, const float *sa,
                                                               float4 *pos, float4 *vel, float4 *acc, float4 *posLo,
                                                               int n, RepState *st, int nrep) {
  __shared__ float sV[3 * kUnpackAtoms], sA[3 * kUnpackAtoms];
  const int a0 = blockIdx.x * kUnpackAtoms, t = threadIdx.x, i = a0 + t;
  // every read over the host link is issued before the barrier: one round trip
  float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
  if (sr && i < n) r = sr[i];
  if (a0 < n) {
    if (sv) stageRows3(sv, n, a0, sV);
    if (sa) stageRows3(sa, n, a0, sA);
  }
  __syncthreads();
  if (i < n) {
    if (sr) pos[i] = r;
    if (sv) vel[i] = make_float4(sV[3 * t], sV[3 * t + 1], sV[3 * t + 2], 0.f);
    if (sa) acc[i] = make_float4(sA[3 * t], sA[3 * t + 1], sA[3 * t + 2], 0.f);
    if (posLo) posLo[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (i < nrep) st[i].thermoPending = 0;
}

// The replica states to the host's page-locked mirror (dst, its device address), then a new
// sequence number next to it: the host waits for that number instead of a stream
// synchronisation.  The blocks of the grid copy a share of the words each and make them visible
// system-wide, then count themselves in (done); the last one, which sees every other block's
// words visible, stores the number (and resets the count for the next publish).
__global__ void k_publish_state(const int *src, int *dst, int nwords, unsigned *devSeq, volatile unsigned *hostSeq,
                                unsigned *done) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nwords; i += gridDim.x * blockDim.x)
    dst[i] = __ldcg(src + i);
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(done, 1u) == gridDim.x - 1) {
    *done = 0;
    __threadfence();
    const unsigned seq = *devSeq + 1u;
    *devSeq = seq;
    __threadfence_system();
    *hostSeq = seq;
  }
}

__global__ void k_clear_pending(RepState *st, int nrep) {
  pdlEnter();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nrep) st[r].thermoPending = 0;
}

}  // namespace sg
