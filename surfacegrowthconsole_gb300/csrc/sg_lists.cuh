// sg_lists.cuh - the cell scan with in-cell ordering and the neighbour-list build, as device
// functions of a block index: the engine's kernels (sg_kernels_plain.cu) run them one block per
// launch block, the persistent step (sg_kernels_mixed.cu) from its own loop over blocks.  Both
// units must build the same lists (the list order decides the graphene neighbours), and the
// MIXED unit compiles with FMA contraction: the squared distances of the list test are written
// with round-to-nearest intrinsics, which the compiler never contracts, so the lists are the
// reference's operation order in both units.
#pragma once
#include "sg_device.cuh"

namespace sg {

__device__ __forceinline__ bool rebuilding(const RepState *S, int forceRebuild) {
  return forceRebuild || S->nebrNow;
}

// dx*dx + dy*dy + dz*dz in that order, each product and sum rounded (no fused multiply-add).
__device__ __forceinline__ float sqDist(float dx, float dy, float dz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// ============================================================================================
// Counting sort in two passes (the engine's path).  The histogram pass (binAtom) files each
// atom in its cell's bucket and counts the filed atoms per block of P.scanCells cells
// (blockCount).  k_scan_rank: one block per P.scanCells cells takes its exclusive offset from
// the counts of the replica's earlier blocks (no wait on another block), scans its cells,
// writes cellStart and the list build's work items and orders each of its cells from its
// bucket; the list build clears blockCount for the next rebuild.
// ============================================================================================
// The cell scan and the in-cell ordering in one pass: one block of THREADS threads per
// CELLS cells takes its exclusive atom offset from the replica's earlier blocks' counts
// (blockCount), scans its cells (a thread per cell), writes cellStart and the list build's work
// items, then orders the atoms of its cells with all its threads: block entry e (cell j, bucket
// slot s) goes to position cellStart[j] + (number of atoms of j's bucket with a smaller index),
// a few entries per thread with their loads in flight together.  Atoms outside the grid get
// empty lists.  blockCount is cleared by the list build (all blocks have read it then).
// Scan block t of the tile table, by a block of THREADS threads (the engine's kernel runs
// kScanRankThreads; the persistent step runs its own block size).
template <int CELLS, int THREADS>
__device__ __forceinline__ void scanRankBody(int t, const int *__restrict__ tileRep, const int *__restrict__ tileStart,
                                             const int *__restrict__ tileFirst, const RepConst *__restrict__ rc,
                                             RepState *st, int *__restrict__ cellCount, int *__restrict__ cellStart,
                                             int cap, int forceRebuild, int *__restrict__ active,
                                             int2 *__restrict__ heavy, int *__restrict__ work, int itemAtoms,
                                             const int *__restrict__ blockCount, const int *__restrict__ bucket,
                                             const int *__restrict__ cellOf, const float4 *__restrict__ pos,
                                             int *__restrict__ sortIdx, float4 *__restrict__ sortPos,
                                             int *__restrict__ nn, int *__restrict__ ns, int *__restrict__ nrl,
                                             const int2 *__restrict__ spill) {
  constexpr int kSub = kCellTile / CELLS;  // scan blocks per tile of the tile table
  constexpr int kWarps = THREADS / 32;
  static_assert(CELLS % 32 == 0 && CELLS <= THREADS, "one cell per scan thread");
  __shared__ int ws[kWarps], wp[kWarps], wl[kWarps], wh[kWarps], wOcc[kWarps], wOver[kWarps];
  __shared__ int sEx[CELLS + 1];  // exclusive prefix of the block's cell counts
  __shared__ int sBaseL, sBaseH, sBase, sOver;
  const int rep = tileRep[t / kSub];
  RepState *S = st + rep;
  if (!rebuilding(S, forceRebuild)) return;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const RepConst &P = rc[rep];
  const int first = tileFirst[rep] * kSub;  // the replica's first scan block
  const int c0 = tileStart[t / kSub] + (t % kSub) * CELLS;
  const int cb = P.cellOff + c0;  // the block's first global cell
  const bool own = tid < CELLS;  // this thread scans cell tid of the block
  const int n = own ? cellCount[cb + tid] : 0;
  // atoms past the cap are not in the bucket: the reference's cap drops them and raises
  // SG_ERR_CELL_OVERFLOW; uncapped (MIXED), the cell keeps all of them and is ordered below by
  // compaction over the replica's atoms
  const int v = P.uncapped ? n : min(n, cap);
  int pre = 0;                // atoms filed in the replica's earlier blocks
  for (int q = first + tid; q < t; q += THREADS) pre += blockCount[q];
  // atoms outside the grid: empty lists (the reference clears their NN), counted in cellRange
  {
    const int lb = t - first, nb = P.ncellsPad / CELLS;
    int outside = 0;
    for (int g = P.atomOff + lb * THREADS + tid; g < P.atomOff + P.nMol; g += nb * THREADS)
      if (cellOf[g] < 0) {
        nn[g] = 0;
        ns[g] = 0;
        nrl[g] = 0;
        outside++;
      }
    if (outside) atomicAdd(&S->cellRange, outside);
  }
  int x = v;  // inclusive prefix inside the warp
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  for (int o = 16; o > 0; o >>= 1) pre += __shfl_xor_sync(0xffffffffu, pre, o);
  // work items of the list build: a cell of more than itemAtoms atoms splits into near-equal
  // items {cell, first << 16 | count}, the others are listed whole
  const bool live = own && v > 0 && c0 + tid < P.ncells;
  const int nHeavy = (live && v > itemAtoms) ? (v + itemAtoms - 1) / itemAtoms : 0;
  const int nLight = (live && v <= itemAtoms) ? 1 : 0;
  int preL = nLight, preH = nHeavy, occ = n, over = (n > cap) ? 1 : 0;
  for (int o = 1; o < 32; o <<= 1) {
    const int yl = __shfl_up_sync(0xffffffffu, preL, o);
    const int yh = __shfl_up_sync(0xffffffffu, preH, o);
    if (lane >= o) { preL += yl; preH += yh; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    occ = max(occ, __shfl_xor_sync(0xffffffffu, occ, o));
    over += __shfl_xor_sync(0xffffffffu, over, o);
  }
  if (lane == 31) {
    ws[wid] = x;
    wl[wid] = preL;
    wh[wid] = preH;
    wOcc[wid] = occ;
    wOver[wid] = over;
  }
  if (lane == 0) wp[wid] = pre;
  __syncthreads();
  if (tid == 0) {
    int tl = 0, th = 0, to = 0, tv = 0, ta = 0, tp = 0;
    for (int k = 0; k < kWarps; k++) {
      const int a = ws[k], l = wl[k], h = wh[k];
      ws[k] = ta; wl[k] = tl; wh[k] = th;  // exclusive warp offsets
      ta += a; tl += l; th += h;
      to = max(to, wOcc[k]);
      tv += wOver[k];
      tp += wp[k];
    }
    sEx[CELLS] = ta;
    sBase = P.atomOff + tp;
    sBaseL = tl > 0 ? atomicAdd(&work[1], tl) : 0;
    sBaseH = th > 0 ? atomicAdd(&work[2], th) : 0;
    if (to > 0) atomicMax(&S->maxCellOcc, to);
    if (tv > 0) {
      atomicAdd(&S->cellOverflow, tv);
      if (!P.uncapped) setFlag(S, 11 /*SG_ERR_CELL_OVERFLOW*/);
    }
    sOver = tv;
  }
  __syncthreads();
  const int ex = ws[wid] + x - v;  // exclusive prefix inside the block
  if (own) {
    sEx[tid] = ex;
    cellStart[cb + tid] = sBase + ex;
    cellCount[cb + tid] = 0;
  }
  if (live) {
    if (nHeavy) {
      int outH = sBaseH + wh[wid] + preH - nHeavy;
      for (int j = 0; j < nHeavy; j++) {
        const int h0 = j * v / nHeavy, h1 = (j + 1) * v / nHeavy;
        heavy[outH++] = make_int2(cb + tid, (h0 << 16) | (h1 - h0));
      }
    } else {
      active[sBaseL + wl[wid] + preL - nLight] = cb + tid;
    }
  }
  __syncthreads();
  // ordering: block entry e is slot s of cell j (the last cell whose prefix is <= e)
  const int nBlk = sEx[CELLS];
#pragma unroll 4
  for (int e = tid; e < nBlk; e += THREADS) {
    int j = 0;
#pragma unroll
    for (int step = CELLS / 2; step > 0; step >>= 1)
      if (sEx[j + step] <= e) j += step;
    const int b = sEx[j], m = sEx[j + 1] - b, s = e - b;
    if (m > cap) continue;  // uncapped cell above the bucket: ordered below
    const int *bk = bucket + (size_t)(cb + j) * cap;
    const int g = bk[s];
    int rank = 0;
    for (int q = 0; q < m; q++) rank += (bk[q] < g) ? 1 : 0;
    float4 r = pos[g];
    r.w = __int_as_float(g);
    sortIdx[sBase + b + rank] = g;
    sortPos[sBase + b + rank] = r;
  }
  // uncapped cells above the bucket (rare: a crowded cell of a hot system): the block gathers
  // the cell's atoms into its segment of sortIdx -- the bucket's cap atoms and the cell's entries
  // of the spill list -- then ranks each by the number of smaller indices in the segment, writes
  // sortPos in that order and finally sortIdx from it (O(m^2) per such cell, m its atoms)
  if (P.uncapped && sOver > 0) {
    __shared__ int sFill;
    const int nSpill = work[3];
    for (int j = 0; j < CELLS; j++) {
      const int b = sEx[j], m = sEx[j + 1] - b;
      if (m <= cap) continue;  // uniform across the block (shared values)
      int *seg = sortIdx + sBase + b;
      float4 *segPos = sortPos + sBase + b;
      const int *bk = bucket + (size_t)(cb + j) * cap;
      if (tid == 0) sFill = cap;
      for (int q = tid; q < cap; q += THREADS) seg[q] = bk[q];
      __syncthreads();
      for (int q = tid; q < nSpill; q += THREADS) {
        const int2 e = spill[q];
        if (e.x == cb + j) {
          const int at = atomicAdd(&sFill, 1);
          if (at < m) seg[at] = e.y;
        }
      }
      __threadfence_block();
      __syncthreads();
      for (int q = tid; q < m; q += THREADS) {
        const int g = seg[q];
        int rank = 0;
        for (int k = 0; k < m; k++) rank += (seg[k] < g) ? 1 : 0;
        float4 r = pos[g];
        r.w = __int_as_float(g);
        segPos[rank] = r;
      }
      __threadfence_block();
      __syncthreads();
      for (int q = tid; q < m; q += THREADS) seg[q] = __float_as_int(segPos[q].w);
      __syncthreads();
    }
  }
}


// ============================================================================================
// Neighbour list (BuildNebrListK, SurfaceGrowth.cu:612-711), cell-centric.  Warps take work
// items from the lists k_scan_rank wrote, through an atomic work counter: first the parts of
// the cells split into several items, then the other non-empty cells whole, in ascending cell
// order or (descending != 0) descending: the queue should end on cheap items, and in a surface
// system the dense metal cells sit at the high cell indices (z-major).  Lanes 0..26 look up
// the 27 stencil cells (reference visiting order); their segments, in that order and ascending
// atom index inside each, form the cell's window of candidates: exactly the order in which the
// reference's one-thread walk meets them.  A lane finds the segment of its window position by
// binary search over the segment offsets.  Two builds share this item set-up:
//  k_build_nebr (nebrFusedBody): per 32-candidate word of the window (one candidate per lane,
//    loaded while the previous word is tested) the warp tests four home atoms at a time, their
//    positions broadcast from shared memory.  Two ballots give a home atom's "within the list
//    radius" and "within rCutC + skin" masks, and the hits go straight to the rows: lane l
//    stores candidate l at the home atom's running length plus its rank among the mask's set
//    bits, so a word's entries of one row leave in one store.  For a carbon home the same
//    ranks place its close list (entries within rCutC + skin, read by the graphene
//    second-neighbour walk of the atoms bonded to it) and its relevant list (every metal entry
//    and every close entry, with its position in the full list: all the carbon-force pass
//    needs for the atom itself).  A word without hits for a home atom costs it the test only,
//    one without close or metal hits the full-list store only.  The running lengths live in
//    the home atom's lane.
//  k_build_nebr_lanes (nebrLanesBody): the masks of a window of kWin candidates kept in shared
//    memory, then lanes walking the hits of one home atom each: G = 32 / nh' lanes per home
//    atom (nh' = nh rounded up to a power of two), lane q of a group taking a contiguous share
//    of the window's words after the hits of the group's earlier lanes.
// Words without a periodic shift that cannot hold a home atom take a test without the shift
// and the self-pair test (subtracting a zero shift changes no bit).  Close and relevant lists
// rest on the skin, as the neighbour list itself does: no pair closes in by more than
// rNebrShell between rebuilds.
// ============================================================================================
struct NebrItem {
  int rep, hFirst, hLast, total, homeLen;  // home atoms [hFirst, hLast) of sortPos; window length
};

// The warp's next work item; false once the items are exhausted (every warp takes one ticket
// past the end, and the last one clears the counters for the next rebuild: all warps have read
// them by then).  Fills the warp's stencil tables: start of each of the 27 cells in sortPos
// (sQb), its offset in the window (sOff, 32 entries, the last five past any position) and its
// periodic shift (sSh, w = 1 when non-zero).
__device__ __forceinline__ bool nebrNextItem(int *work, int nLight, int nHeavy, const int2 *__restrict__ heavy,
                                             const int *__restrict__ active, const int *__restrict__ tileRep,
                                             const RepConst *__restrict__ rc, const int *__restrict__ cellStart,
                                             int descending, int lane, float4 *sSh, int *sQb, int *sOff,
                                             NebrItem &it) {
  const unsigned full = 0xffffffffu;
  int idx = 0;
  if (lane == 0) idx = atomicAdd(&work[0], 1);
  idx = __shfl_sync(full, idx, 0);
  if (idx >= nHeavy + nLight) {
    if (lane == 0 && idx == nHeavy + nLight + (int)gridDim.x * kNebrWarps - 1) {
      work[0] = 0;
      work[1] = 0;
      work[2] = 0;
      work[3] = 0;
    }
    return false;
  }
  int gc, hOff = 0, hCnt = 1 << 30;
  if (idx < nHeavy) {
    const int2 h = heavy[idx];
    gc = h.x;
    hOff = h.y >> 16;
    hCnt = h.y & 0xffff;
  } else {
    gc = active[descending ? nHeavy + nLight - 1 - idx : idx - nHeavy];
  }
  it.rep = tileRep[gc / kCellTile];
  const RepConst &P = rc[it.rep];
  const int c = gc - P.cellOff;
  const int hb = cellStart[gc], he = cellStart[gc + 1];
  it.hFirst = hb + hOff;
  it.hLast = min(he, it.hFirst + hCnt);
  it.homeLen = he - hb;  // stencil cell 0 is the home cell: window positions [0, homeLen)
  int len = 0;
  if (lane < 27) {
    float sx, sy, sz;
    const int C = P.cellOff + stencilCell(P, c, lane, sx, sy, sz);
    const int qb = cellStart[C];
    len = cellStart[C + 1] - qb;
    sQb[lane] = qb;
    sSh[lane] = make_float4(sx, sy, sz, (sx != 0.f || sy != 0.f || sz != 0.f) ? 1.f : 0.f);
  }
  int incl = len;  // inclusive prefix of the segment lengths
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(full, incl, d);
    if (lane >= d) incl += v;
  }
  sOff[lane] = (lane < 27) ? incl - len : 0x7fffffff;  // padded: the search needs no bound
  it.total = __shfl_sync(full, incl, 26);
  __syncwarp();
  return true;
}

// The candidate at window position e: its sortPos entry (w: the atom index) and its stencil
// cell o, the last one whose segment starts at or before e.
__device__ __forceinline__ float4 nebrCandidate(const float4 *__restrict__ sortPos, const int *sQb, const int *sOff,
                                                int e, int &o) {
  o = 0;
#pragma unroll
  for (int step = 16; step > 0; step >>= 1)
    if (sOff[o + step] <= e) o += step;
  return sortPos[sQb[o] + e - sOff[o]];
}

// The lengths of home atom `lane` (< nh) once its window is done: nn, and for a carbon atom ns
// and nrl (-1: the carbon pass walks the full list instead); the largest list and the rows
// that overflowed accumulate in want and over.
__device__ __forceinline__ void nebrFinishHome(int lane, int nh, int ga, int nMy, int mMy, int rMy, int metalEnd,
                                               int nebrMax, int *__restrict__ nn, int *__restrict__ ns,
                                               int *__restrict__ nrl, int &want, int &over) {
  if (lane < nh) {
    nn[ga] = min(nMy, nebrMax);
    ns[ga] = (ga < metalEnd) ? 0 : (mMy > kShortMax || nMy > nebrMax) ? -1 : mMy;
    nrl[ga] = (ga < metalEnd) ? 0 : (rMy > kRelMax || nMy > nebrMax || nMy > kRelPosLimit) ? -1 : rMy;
    want = max(want, nMy);
    over += (nMy > nebrMax) ? 1 : 0;
  }
}

// The item's largest list and overflowing rows into the replica's state, one atomic each.
__device__ __forceinline__ void nebrItemStats(int lane, RepState *S, int want, int over) {
  const unsigned full = 0xffffffffu;
  for (int off = 16; off > 0; off >>= 1) {
    want = max(want, __shfl_xor_sync(full, want, off));
    over += __shfl_xor_sync(full, over, off);
  }
  if (lane == 0) {
    atomicMax(&S->maxNeighbours, want);
    if (over > 0) {
      atomicAdd(&S->nebrOverflow, over);
      setFlag(S, 5 /*SG_ERR_NEBR_OVERFLOW*/);
    }
  }
  __syncwarp();
}

// A home-atom slot past the item's home atoms: far from every position and from the 1e30 of an
// empty candidate lane, so its squared distance overflows and it never hits.
__device__ __forceinline__ float4 nebrNoHome() { return make_float4(-1e30f, -1e30f, -1e30f, __int_as_float(-2)); }

// Store v at p when q, as a predicated store: the warp takes no branch for it.  (No memory
// clobber: the list build never reads what it stores.)
__device__ __forceinline__ void stPred(bool q, int *p, int v) {
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %0, 0;\n\t@q st.global.u32 [%1], %2;\n\t}" ::"r"((unsigned)q),
               "l"(p), "r"(v));
}

// U home atoms (a0 .. a0+U-1 of the warp's sHome) against this lane's candidate: the hit and
// close masks of each.  SHIFTED: the word holds a periodic image or the home cell, so the
// shift is subtracted and the self pair left out.
template <int U, bool SHIFTED>
__device__ __forceinline__ void nebrTest(const float4 *sHome, int a0, float bx, float by, float bz, float sx, float sy,
                                         float sz, int k, float rrNebr, float rrShort, unsigned (&mh)[U],
                                         unsigned (&mc)[U], int (&gh)[U]) {
  const unsigned full = 0xffffffffu;
#pragma unroll
  for (int u = 0; u < U; u++) {
    const float4 H = sHome[a0 + u];
    gh[u] = __float_as_int(H.w);
    float dx = H.x - bx, dy = H.y - by, dz = H.z - bz;
    if (SHIFTED) {
      // the reference subtracts the cell shift after the difference: both roundings kept
      dx = dx - sx;
      dy = dy - sy;
      dz = dz - sz;
    }
    const float rr = sqDist(dx, dy, dz);
    mh[u] = __ballot_sync(full, (rr < rrNebr) && (!SHIFTED || gh[u] != k));
    mc[u] = __ballot_sync(full, rr < rrShort);
  }
}

// Where a work item's lists go.
struct NebrOut {
  int *nbl, *sl;
  unsigned *rl;
  int rowStride, nebrMax, metalEnd, atomOff;
  float rrNebr, rrShort;
};

// Test U home atoms (a0 .. a0+U-1) against this lane's candidate k of word i, keep the hit and
// close masks for the close and relevant lists (sMask[i][a]), and store the hits in the rows
// at once; nMy is the running full-list length of home atom `lane`.
template <int U, bool SHIFTED>
__device__ __forceinline__ void nebrGroup(const float4 *sHome, uint2 (*sMask)[32], int i, int a0, int lane, float bx,
                                          float by, float bz, float sx, float sy, float sz, int k,
                                          const NebrOut &O, int &nMy) {
  const unsigned full = 0xffffffffu, lower = (1u << lane) - 1u;
  unsigned mh[U], mc[U];
  int gh[U];
  nebrTest<U, SHIFTED>(sHome, a0, bx, by, bz, sx, sy, sz, k, O.rrNebr, O.rrShort, mh, mc, gh);
#pragma unroll
  for (int u = 0; u < U; u++) {
    const unsigned h = mh[u];
    sMask[i][a0 + u] = make_uint2(h, mc[u]);  // the same value from every lane: no branch
    if (h == 0u) continue;  // warp-uniform: no entry for this home atom in this word
    const int a = a0 + u;
    const int j = __shfl_sync(full, nMy, a) + __popc(h & lower);
    stPred(((h >> lane) & 1u) && j < O.nebrMax, O.nbl + (size_t)gh[u] * O.rowStride + j, k);
    if (lane == a) nMy += __popc(h);
  }
}

template <int U>
__device__ __forceinline__ void nebrGroupAny(bool shifted, const float4 *sHome, uint2 (*sMask)[32], int i, int a0,
                                             int lane, float bx, float by, float bz, float sx, float sy, float sz,
                                             int k, const NebrOut &O, int &nMy) {
  if (shifted)
    nebrGroup<U, true>(sHome, sMask, i, a0, lane, bx, by, bz, sx, sy, sz, k, O, nMy);
  else
    nebrGroup<U, false>(sHome, sMask, i, a0, lane, bx, by, bz, sx, sy, sz, k, O, nMy);
}

// The close and relevant lists of the carbon home atoms for the window pass just tested (nw
// words, masks in sMask, atom indices in sK, metal candidates in sMetal): the lane of each
// carbon home atom walks the close and relevant bits of its words (few: a carbon atom has three
// close neighbours and metal ones only near a cluster); nPass is its full-list length before
// the pass (the entries' positions), mMy and rMy its running close- and relevant-list lengths.
__device__ __forceinline__ void nebrCarbonLists(const uint2 (*sMask)[32], const int *sK, const unsigned *sMetal, int nw,
                                                int nh, int lane, int ga, int nPass, const NebrOut &O, int &mMy,
                                                int &rMy) {
  if (lane >= nh || ga < O.metalEnd) return;
  int n = nPass, m = mMy, r = rMy;
  int *srow = O.sl + (size_t)ga * kShortMax;
  unsigned *rrow = O.rl + (size_t)ga * kRelMax;
  for (int i = 0; i < nw; i++) {
    const uint2 hc = sMask[i][lane];
    unsigned bits = hc.x & (hc.y | sMetal[i]);
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1;
      const int k = sK[32 * i + b];
      if ((hc.y >> b) & 1u) {
        if (m < kShortMax) srow[m] = k;
        m++;
      }
      // its position in the full list
      if (r < kRelMax) rrow[r] = relPack(k - O.atomOff, n + __popc(hc.x & ((1u << b) - 1u)));
      r++;
    }
    n += __popc(hc.x);
  }
  mMy = m;
  rMy = r;
}

__device__ __forceinline__ void nebrFusedBody(const int *__restrict__ tileRep, const int *__restrict__ active,
                                              const int2 *__restrict__ heavy, int *work,
                                              const RepConst *__restrict__ rc, RepState *st,
                                              const int *__restrict__ cellStart, const float4 *__restrict__ sortPos,
                                              int *__restrict__ nn, int *__restrict__ nbl, int *__restrict__ ns,
                                              int *__restrict__ sl, int *__restrict__ nrl, unsigned *__restrict__ rl,
                                              int rowStride, int nebrMax, int descending) {
  __shared__ int sK[kNebrWarps][kFusedWin];                  // atom index of each window position
  __shared__ uint2 sMask[kNebrWarps][kFusedWin / 32][32];    // [word][home atom]: {hit, close}
  __shared__ unsigned sMetal[kNebrWarps][kFusedWin / 32];    // [word]: candidate is a metal atom
  __shared__ float4 sHome[kNebrWarps][32];
  __shared__ float4 sSh[kNebrWarps][27];
  __shared__ int sQb[kNebrWarps][27], sOff[kNebrWarps][32];
  const unsigned full = 0xffffffffu;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nLight = work[1], nHeavy = work[2];
  NebrItem it;
  while (nebrNextItem(work, nLight, nHeavy, heavy, active, tileRep, rc, cellStart, descending, lane, sSh[w], sQb[w],
                      sOff[w], it)) {
    const RepConst &P = rc[it.rep];
    const int metalEnd = P.atomOff + P.nMolMe;
    const NebrOut O{nbl, sl, rl, rowStride, nebrMax, metalEnd, P.atomOff, P.rrNebr, P.rrShort};
    const int total = it.total;
    int want = 0, over = 0;
    for (int h0 = it.hFirst; h0 < it.hLast; h0 += 32) {
      const int nh = min(32, it.hLast - h0);
      const float4 Ah = (lane < nh) ? sortPos[h0 + lane] : nebrNoHome();
      sHome[w][lane] = Ah;
      const int ga = __float_as_int(Ah.w);
      const bool carbonHomes = __any_sync(full, lane < nh && ga >= metalEnd);
      int nMy = 0, mMy = 0, rMy = 0;  // list, close-list and relevant-list lengths of home atom `lane`
      __syncwarp();
      for (int base = 0; base < total; base += kFusedWin) {
        const int nw = (min(kFusedWin, total - base) + 31) >> 5;
        const int nPass = nMy;
        // this lane's candidate of the next word, loaded while the current word is tested
        int oN = 0;
        float4 BN = make_float4(0.f, 0.f, 0.f, 0.f);
        if (base + lane < total) BN = nebrCandidate(sortPos, sQb[w], sOff[w], base + lane, oN);
        for (int i = 0; i < nw; i++) {
          const int e = base + 32 * i + lane;
          const int o = oN;
          const float4 B = BN;
          if (i + 1 < nw && e + 32 < total) BN = nebrCandidate(sortPos, sQb[w], sOff[w], e + 32, oN);
          // this lane's candidate; past the window end it sits at 1e30 and never matches
          float bx = 1e30f, by = 1e30f, bz = 1e30f, sx = 0.f, sy = 0.f, sz = 0.f;
          int k = -1;
          bool shifted = false;
          if (e < total) {
            k = __float_as_int(B.w);
            bx = B.x;
            by = B.y;
            bz = B.z;
            const float4 sh = sSh[w][o];
            sx = sh.x;
            sy = sh.y;
            sz = sh.z;
            shifted = sh.w != 0.f;
          }
          if (carbonHomes) {
            sK[w][32 * i + lane] = k;
            const unsigned metalW = __ballot_sync(full, k >= 0 && k < metalEnd);
            if (lane == 0) sMetal[w][i] = metalW;
          }
          const bool shiftWord = __any_sync(full, shifted) || base + 32 * i < it.homeLen;
          int a0 = 0;
          for (; a0 + 4 <= nh; a0 += 4)
            nebrGroupAny<4>(shiftWord, sHome[w], sMask[w], i, a0, lane, bx, by, bz, sx, sy, sz, k, O, nMy);
          // the last one to three home atoms: a group of their size (one of four for three)
          const int rest = nh - a0;
          if (rest >= 3)
            nebrGroupAny<4>(shiftWord, sHome[w], sMask[w], i, a0, lane, bx, by, bz, sx, sy, sz, k, O, nMy);
          else if (rest == 2)
            nebrGroupAny<2>(shiftWord, sHome[w], sMask[w], i, a0, lane, bx, by, bz, sx, sy, sz, k, O, nMy);
          else if (rest == 1)
            nebrGroupAny<1>(shiftWord, sHome[w], sMask[w], i, a0, lane, bx, by, bz, sx, sy, sz, k, O, nMy);
        }
        __syncwarp();
        if (carbonHomes) nebrCarbonLists(sMask[w], sK[w], sMetal[w], nw, nh, lane, ga, nPass, O, mMy, rMy);
        __syncwarp();
      }
      nebrFinishHome(lane, nh, ga, nMy, mMy, rMy, metalEnd, nebrMax, nn, ns, nrl, want, over);
      __syncwarp();
    }
    nebrItemStats(lane, st + it.rep, want, over);
  }
}

__device__ __forceinline__ void nebrLanesBody(const int *__restrict__ tileRep, const int *__restrict__ active,
                                              const int2 *__restrict__ heavy, int *work,
                                              const RepConst *__restrict__ rc, RepState *st,
                                              const int *__restrict__ cellStart, const float4 *__restrict__ sortPos,
                                              int *__restrict__ nn, int *__restrict__ nbl, int *__restrict__ ns,
                                              int *__restrict__ sl, int *__restrict__ nrl, unsigned *__restrict__ rl,
                                              int rowStride, int nebrMax, int descending) {
  __shared__ int sK[kNebrWarps][kWin];                 // atom index of each window position
  __shared__ uint2 sMask[kNebrWarps][kWin / 32][32];   // [word][home atom]: {hit, close}
  __shared__ unsigned sMetal[kNebrWarps][kWin / 32];   // [word]: candidate is a metal atom
  __shared__ float4 sHome[kNebrWarps][32];
  __shared__ float4 sSh[kNebrWarps][27];
  __shared__ int sQb[kNebrWarps][27], sOff[kNebrWarps][32];
  const unsigned full = 0xffffffffu;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nLight = work[1], nHeavy = work[2];
  NebrItem it;
  while (nebrNextItem(work, nLight, nHeavy, heavy, active, tileRep, rc, cellStart, descending, lane, sSh[w], sQb[w],
                      sOff[w], it)) {
    const RepConst &P = rc[it.rep];
    const int metalEnd = P.atomOff + P.nMolMe;
    const float rrNebr = P.rrNebr, rrShort = P.rrShort;
    const int total = it.total;
    int want = 0, over = 0;
    for (int h0 = it.hFirst; h0 < it.hLast; h0 += 32) {
      const int nh = min(32, it.hLast - h0);
      const float4 Ah = (lane < nh) ? sortPos[h0 + lane] : nebrNoHome();
      sHome[w][lane] = Ah;
      const int ga = __float_as_int(Ah.w);
      int nMy = 0, mMy = 0, rMy = 0;  // list, close-list and relevant-list lengths of home atom `lane`
      __syncwarp();
      for (int base = 0; base < total; base += kWin) {
        const int nw = (min(kWin, total - base) + 31) >> 5;
        // ---- test pass: the hit and close masks of every home atom and word of the window
        int oN = 0;
        float4 BN = make_float4(0.f, 0.f, 0.f, 0.f);
        if (base + lane < total) BN = nebrCandidate(sortPos, sQb[w], sOff[w], base + lane, oN);
        for (int i = 0; i < nw; i++) {
          const int e = base + 32 * i + lane;
          const int o = oN;
          const float4 B = BN;
          if (i + 1 < nw && e + 32 < total) BN = nebrCandidate(sortPos, sQb[w], sOff[w], e + 32, oN);
          float bx = 1e30f, by = 1e30f, bz = 1e30f, sx = 0.f, sy = 0.f, sz = 0.f;
          int k = -1;
          bool shifted = false;
          if (e < total) {
            k = __float_as_int(B.w);
            bx = B.x;
            by = B.y;
            bz = B.z;
            const float4 sh = sSh[w][o];
            sx = sh.x;
            sy = sh.y;
            sz = sh.z;
            shifted = sh.w != 0.f;
            sK[w][32 * i + lane] = k;
          }
          sMetal[w][i] = __ballot_sync(full, k >= 0 && k < metalEnd);
          const bool plainWord = !__any_sync(full, shifted) && base + 32 * i >= it.homeLen;
          for (int a0 = 0; a0 < nh; a0 += 4) {
            unsigned mh[4], mc[4];
            int gh[4];
            if (plainWord)
              nebrTest<4, false>(sHome[w], a0, bx, by, bz, sx, sy, sz, k, rrNebr, rrShort, mh, mc, gh);
            else
              nebrTest<4, true>(sHome[w], a0, bx, by, bz, sx, sy, sz, k, rrNebr, rrShort, mh, mc, gh);
#pragma unroll
            for (int u = 0; u < 4; u++)
              if (a0 + u < nh) sMask[w][i][a0 + u] = make_uint2(mh[u], mc[u]);
          }
        }
        __syncwarp();
        // ---- emit pass: lane q of home atom a's group walks the set bits of a's masks in
        // words [i0, i1): its share of a's entries in list order, with the same limits and the
        // same close and relevant entries; the group's exclusive prefix of the hit counts
        // places them
        const int lg = 32 - __clz(nh - 1);  // log2 of nh rounded up to a power of two
        const int G = 32 >> lg;
        const int a = lane >> (5 - lg), q = lane & (G - 1);
        const int i0 = q * nw / G, i1 = (q + 1) * nw / G;
        int cn = 0, cm = 0, cr = 0;  // this lane's hits, close hits and relevant hits
        for (int i = i0; i < i1; i++) {
          const uint2 hc = sMask[w][i][a];
          cn += __popc(hc.x);
          cm += __popc(hc.x & hc.y);
          cr += __popc(hc.x & (hc.y | sMetal[w][i]));
        }
        int pn = cn, pm = cm, pr = cr;  // inclusive prefix inside the group
        for (int d = 1; d < G; d <<= 1) {
          const int yn = __shfl_up_sync(full, pn, d, G);
          const int ym = __shfl_up_sync(full, pm, d, G);
          const int yr = __shfl_up_sync(full, pr, d, G);
          if (q >= d) {
            pn += yn;
            pm += ym;
            pr += yr;
          }
        }
        const int g = __shfl_sync(full, ga, a);
        int n = __shfl_sync(full, nMy, a) + pn - cn;
        int m = __shfl_sync(full, mMy, a) + pm - cm;
        int r = __shfl_sync(full, rMy, a) + pr - cr;
        const int lastOfGroup = ((lane * G) & 31) + G - 1;  // for lane < nh: home `lane`'s group
        const int tn = __shfl_sync(full, pn, lastOfGroup);
        const int tm = __shfl_sync(full, pm, lastOfGroup);
        const int tr = __shfl_sync(full, pr, lastOfGroup);
        if (a < nh) {
          int *row = nbl + (size_t)g * rowStride;
          const bool carbonHome = g >= metalEnd;
          int *srow = sl + (size_t)g * kShortMax;
          unsigned *rrow = rl + (size_t)g * kRelMax;
          for (int i = i0; i < i1; i++) {
            const uint2 hc = sMask[w][i][a];
            const unsigned metalW = sMetal[w][i];
            unsigned bits = hc.x;
            while (bits) {
              const int b = __ffs(bits) - 1;
              bits &= bits - 1;
              const int k = sK[w][32 * i + b];
              if (n < nebrMax) row[n] = k;
              if (carbonHome) {
                const bool close = (hc.y >> b) & 1u;
                if (close) {
                  if (m < kShortMax) srow[m] = k;
                  m++;
                }
                if (close || ((metalW >> b) & 1u)) {
                  if (r < kRelMax) rrow[r] = relPack(k - P.atomOff, n);
                  r++;
                }
              }
              n++;
            }
          }
        }
        if (lane < nh) {
          nMy += tn;
          mMy += tm;
          rMy += tr;
        }
        __syncwarp();
      }
      nebrFinishHome(lane, nh, ga, nMy, mMy, rMy, metalEnd, nebrMax, nn, ns, nrl, want, over);
      __syncwarp();
    }
    nebrItemStats(lane, st + it.rep, want, over);
  }
}

// the binning's per-block counts, read by k_scan_rank, start the next rebuild at zero
__device__ __forceinline__ void clearBlockCount(int *blockCount, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) blockCount[i] = 0;
}

}  // namespace sg
