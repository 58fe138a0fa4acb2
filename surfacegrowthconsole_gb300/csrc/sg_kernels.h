// sg_kernels.h - kernel entry points of sgmd (device code in sg_kernels_plain.cu and
// sg_kernels_mixed.cu), launched by sg_engine.cu.
#pragma once
#include "sg_device.cuh"

namespace sg {

// ---- shared list building (PLAIN TU, also used by MIXED) ----
__global__ void k_integrate_first(BlockTab tab, const RepConst *rc, RepState *st, float4 *pos,
                                  float4 *vel, const float4 *acc, int *cellOf, int *slot,
                                  int *cellCount, int forceRebuild, int *bucket, int cap, int *blockCount);
__global__ void k_cell_count(BlockTab tab, const RepConst *rc, const float4 *pos, int *cellOf,
                             int *slot, int *cellCount);
__global__ void k_cell_bucket(BlockTab tab, const RepConst *rc, const float4 *pos, int *cellOf, int *slot,
                              int *cellCount, int *bucket, int cap, int *blockCount, int2 *spill, int *spillCount);
__global__ void k_build_nebr_atoms(BlockTab tab, const RepConst *rc, RepState *st, const int *cellOf,
                                   const int *cellStart, const float4 *sortPos, int *nn, int *nbl, int *ns,
                                   int *sl, int *nrl, unsigned *rl, int rowStride, int nebrMax, int *work,
                                   int forceRebuild, int *blockCount, int nBlockCount);
// the cell scan and in-cell ordering: one block of kScanRankThreads threads per `cells` cells
cudaError_t launchScanRank(bool pdl, int cells, int grid, cudaStream_t s, const int *tileRep, const int *tileStart,
                           const int *tileFirst, const RepConst *rc, RepState *st, int *cellCount, int *cellStart,
                           int cap, int forceRebuild, int *active, int2 *heavy, int *work, int itemAtoms,
                           const int *blockCount, const int *bucket, const int2 *spill, const int *cellOf,
                           const float4 *pos, int *sortIdx, float4 *sortPos, int *nn, int *ns, int *nrl);
__global__ void k_scan_tiles(BlockTab tab, const RepConst *rc, const RepState *st,
                             const int *cellCount, int *tileSum, int forceRebuild);
__global__ void k_scan_tile_prefix(const RepConst *rc, const RepState *st, const int *tileFirst,
                                   int *tileSum, int forceRebuild, int *work);
__global__ void k_scan_final(BlockTab tab, const RepConst *rc, RepState *st, int *cellCount,
                             const int *tileSum, int *cellStart, int blockSizeCap, int forceRebuild,
                             int *active, int2 *heavy, int *work, int itemAtoms);
__global__ void k_scatter(BlockTab tab, const RepConst *rc, RepState *st, const int *cellOf,
                          const int *slot, const int *cellStart, int *tmpIdx, int *nn, int *ns, int *nrl,
                          int forceRebuild);
__global__ void k_rank(BlockTab tab, const RepConst *rc, const RepState *st, const int *cellOf,
                       const int *cellStart, const int *tmpIdx, const float4 *pos, int *sortIdx,
                       float4 *sortPos, int forceRebuild);
// work[0]: next work item to take, work[1]: length of the cell list `active`, work[2]: length
// of the home-chunk list `heavy` (all reset before the scan of every rebuild).
__global__ void k_build_nebr(const int *tileRep, const int *active, const int2 *heavy, int *work, const RepConst *rc, RepState *st,
                             const int *cellStart, const float4 *sortPos, int *nn, int *nbl, int *ns, int *sl,
                             int *nrl, unsigned *rl, int rowStride, int nebrMax, int descending, int *blockCount,
                             int nBlockCount);
__global__ void k_build_nebr_lanes(const int *tileRep, const int *active, const int2 *heavy, int *work, const RepConst *rc, RepState *st,
                             const int *cellStart, const float4 *sortPos, int *nn, int *nbl, int *ns, int *sl,
                             int *nrl, unsigned *rl, int rowStride, int nebrMax, int descending, int *blockCount,
                             int nBlockCount);

// ---- PLAIN force and step kernels ----
__global__ void k_rho(BlockTab tab, const RepConst *rc, const float4 *pos, const int *nn,
                      const int *nbl, float *rho, float *dF, float *Fv, int rowStride);
__global__ void k_force_metal(BlockTab tab, const RepConst *rc, float4 *pos, float4 *acc,
                              const int *nn, const int *nbl, const float *dF, const float *Fv,
                              float *fric, int rowStride);
// the metal chain (k_rho, k_force_metal) with mt lanes per atom (4, 8, 16, 32) on the table of
// 128 / mt atoms per block
void launchMetalChain(bool pdl, int mt, int grid, int stagedGrid, size_t stagedSmem, cudaStream_t s, BlockTab tab, const RepConst *rc, float4 *pos,
                      float4 *acc, const int *nn, const int *nbl, float *rho, float *dF, float *Fv,
                      float *fric, int rowStride);
// the carbon pass with minBlocks (8, 12, 16) resident 128-thread blocks per SM
cudaError_t launchCarbon(bool pdl, int minBlocks, int grid, cudaStream_t s, BlockTab tab, const RepConst *rc,
                         float4 *pos, float4 *acc, const int *nn, const int *nbl, const int *ns, const int *sl,
                         const int *nrl, const unsigned *rl, int rowStride);
__global__ void k_cmvel(BlockTab tab, const RepConst *rc, RepState *st, const float4 *vel,
                        const float4 *acc, float *partial, const int *redFirst);
__global__ void k_step_reduce(BlockTab tab, const RepConst *rc, RepState *st, const float4 *pos,
                              float4 *vel, const float4 *acc, const float *fric, float *partial,
                              const int *redFirst, float *diffBuf, const size_t *diffOff,
                              int forceRebuild, PublishArgs pub);
__global__ void k_shear(BlockTab tab, const RepConst *rc, RepState *st, const float4 *pos,
                        float4 *acc);
__global__ void k_rdf(BlockTab tab, const RepConst *rc, RepState *st, const float4 *pos,
                      const int *cellOf, const int *cellStart, const int *sortIdx, unsigned *hist,
                      int histStride);
__global__ void k_rdf_ext(const RepConst *rc, const float4 *pos, const int4 *pairs, unsigned long long *hist,
                          int nbins, float range);
__global__ void k_apply_pending(BlockTab tab, const RepConst *rc, RepState *st, float4 *vel);
__global__ void k_clear_pending(RepState *st, int nrep);
__global__ void k_publish_state(const int *src, int *dst, int nwords, unsigned *devSeq, volatile unsigned *hostSeq,
                                unsigned *done);
__global__ void k_unpack_state(const float4 *sr, const float *sv, const float *sa, float4 *pos, float4 *vel,
                               float4 *acc, float4 *posLo, int n, RepState *st, int nrep);
__global__ void k_unpack3(const float *src, float4 *dst, int n);
__global__ void k_pack3(const float4 *src, float *dst, int n);

}  // namespace sg
