// sg_kernels_mixed.cu - the MIXED ("chosen") form of the step: the same model as PLAIN (same
// potentials, same neighbour-list semantics, the same force passes from sg_forces.cuh), with the
// numerics changed where they decide long-run accuracy and speed:
//  - positions are a hi/lo pair of floats: the drift r += dt v and the periodic wrap are done
//    with error-free transformations (TwoSum), so the position keeps ~48 significant bits
//    instead of rounding every step's tiny displacement to 24; forces and lists read the hi
//    word, which is the position rounded to float;
//  - FMA contraction is on (this unit is compiled without -fmad=false);
//  - the step's reductions (kinetic and potential energy, impulse, centre of mass, friction,
//    virial sum r.F) sum 64 atoms per warp in FP32 (the centre of mass as a double-float of
//    the hi/lo positions) and everything above in FP64, in a fixed order (warp totals, block
//    partials, one block over the partials): about 1e-9 relative on the totals; the thermostat
//    factor is computed in FP64, the diffusion MSD accumulators are FP64; the centre-of-mass velocity that the regime-2 kinetic energy subtracts comes out
//    of the same pass (sum m (vx - c)^2 = m (sum vx^2 - 2 c sum vx + n c^2)), so the separate
//    centre-of-mass-velocity launch of PLAIN is gone;
//  - the EAM pair functions phi(r), f(r) and their derivatives come from cubic Hermite tables
//    (cubic pieces on 1,024 intervals from 0.6 r_e to the cutoff, coefficients built in FP64
//    from the analytic forms) instead of
//    two expf and four powf per pair; the embedding function stays analytic (once per atom);
//  - particle size is the true extent of the metal (PLAIN keeps the reference's zero padding,
//    which puts 0 inside every min/max).
#include <cuda_runtime.h>

#include <vector>

#include "sg_device.cuh"
#include "sg_engine.h"
#include "sg_kernels.h"

#include <cmath>

#define SG_KN(name) name##_mixed
#define SG_EAM_TABLE
#define SG_FAST_RECIP
#include "sg_forces.cuh"
#include "sg_lists.cuh"

namespace sg {

// Values the MIXED step reduction accumulates in FP64 per block.
enum MixAcc {
  MA_VSUM_X = 0, MA_VSUM_Y, MA_VSUM_Z,  // impulse (metal x mass-scaled, as the reference)
  MA_VV_C,                              // carbon sum v^2
  MA_VVYZ_M,                            // metal sum vy^2 + vz^2
  MA_VX2_M, MA_VX_M,                    // metal sum vx^2, sum vx
  MA_VY_M, MA_VZ_M,                     // metal sum vy, vz (centre-of-mass velocity)
  MA_USUM,                              // sum U
  MA_CM_X, MA_CM_Y, MA_CM_Z,            // metal sum r (hi + lo)
  MA_FRICT,                             // friction sum
  MA_VIRIAL,                            // sum r . F
  kMixAcc
};
enum MixMax { MM_VVMAX = 0, MM_MIN_X, MM_MIN_Y, MM_MIN_Z, MM_MAX_X, MM_MAX_Y, MM_MAX_Z, kMixMax };

struct MixedBufs {
  float2 *partDF = nullptr;  // [reduction blocks][kMixAcc]: double-float block sums
  float *partF = nullptr;    // [reduction blocks][kMixMax]
  double *diff64 = nullptr;  // per replica: nB x 6 (orgR, rTrue), nB x nV (rr), nV (av)
  size_t *dDiffOff64 = nullptr;
  std::vector<size_t> diffOff64;
  unsigned *counter = nullptr;  // per replica: blocks done
  float4 *eamTab = nullptr;     // per replica nTab intervals x 2: cubic coefficients of phi, of f
  int mixAtoms = kMixAtoms;     // atoms per step-reduction block (512, 1024, 2048 or 4096)
  int *redRep = nullptr, *redStart = nullptr;  // reduction blocks: replica, block index in it
  int redN = 0;
  size_t stagedSmem = 0;        // shared memory of the staged metal kernels (the largest table)
  bool stagedOk = false;
};

template <int MT> static cudaError_t allowStagedSmem(size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(k_rho_staged_mixed<MT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_force_metal_staged_mixed<MT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return e;
}


__device__ __forceinline__ void twoSum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// hi += d exactly into (hi, lo), then renormalise so that hi is the pair rounded to float
__device__ __forceinline__ void addHiLo(float &hi, float &lo, float d) {
  float s, e;
  twoSum(hi, d, s, e);
  lo += e;
  const float t = s + lo;
  lo = lo - (t - s);
  hi = t;
}

// ============================================================================================
// Integrator part 1 with hi/lo positions (same schedule as k_integrate_first: pending
// thermostat, deposition, kick + drift, wrap, freeze mask, cell histogram on rebuild steps).
// ============================================================================================
// Floats [3 g0, 3 g1) of a float3 array into shared memory, as float4 where 16-byte aligned.
__device__ __forceinline__ void stageRows3Range(const float *src, int g0, int g1, float *sm) {
  const int f0 = 3 * g0, f1 = 3 * g1;
  const bool aligned = (reinterpret_cast<uintptr_t>(src + f0) & 15) == 0;
  for (int q = threadIdx.x; 4 * q < f1 - f0; q += blockDim.x) {
    const int f = f0 + 4 * q;
    if (aligned && f + 4 <= f1) {
      const float4 x = *reinterpret_cast<const float4 *>(src + f);
      sm[4 * q] = x.x; sm[4 * q + 1] = x.y; sm[4 * q + 2] = x.z; sm[4 * q + 3] = x.w;
    } else {
      for (int k = 0; k < 4 && f + k < f1; k++) sm[4 * q + k] = src[f + k];
    }
  }
}

// Block-table entry e (128 atoms), by a 128-thread block.  With host arrays (hostR, hostV,
// hostA: all replicas' r, v, a in global order, read in place through the host's page tables)
// the step starts from them as an upload would leave the state: the low position words zero,
// any pending thermostat rescale cancelled, the accelerations stored.
__device__ __forceinline__ void integrateMixedBody(int e, BlockTab tab, const RepConst *__restrict__ rc, RepState *st,
                                                   float4 *__restrict__ pos, float4 *__restrict__ posLo,
                                                   float4 *__restrict__ vel, float4 *__restrict__ acc,
                                                   int *__restrict__ cellOf, int *__restrict__ slot,
                                                   int *__restrict__ cellCount, int forceRebuild,
                                                   int *__restrict__ bucket, int cap, int *__restrict__ blockCount,
                                                   int2 *__restrict__ spill, int *__restrict__ spillCount,
                                                   const float4 *__restrict__ hostR = nullptr,
                                                   const float *__restrict__ hostV = nullptr,
                                                   const float *__restrict__ hostA = nullptr) {
  const int rep = tab.rep[e];
  const RepConst &P = rc[rep];
  RepState *S = st + rep;
  const int g = tab.start[e] + threadIdx.x;
  const int gEnd = P.atomOff + P.nMol;
  float4 r, lo, v, a;
  bool pending;
  if (hostR) {
    __shared__ float sV[3 * 128], sA[3 * 128];
    const int g0 = tab.start[e], g1 = min(gEnd, g0 + (int)blockDim.x);
    if (g < gEnd) r = hostR[g];  // every read over the host link before the barrier
    stageRows3Range(hostV, g0, g1, sV);
    stageRows3Range(hostA, g0, g1, sA);
    __syncthreads();
    if (g >= gEnd) return;
    const int t = threadIdx.x;
    v = make_float4(sV[3 * t], sV[3 * t + 1], sV[3 * t + 2], 0.f);
    a = make_float4(sA[3 * t], sA[3 * t + 1], sA[3 * t + 2], 0.f);
    lo = make_float4(0.f, 0.f, 0.f, 0.f);
    pending = false;
    acc[g] = a;
  } else {
    if (g >= gEnd) return;
    r = pos[g];
    lo = posLo[g];
    v = vel[g];
    a = acc[g];
    pending = S->thermoPending != 0;
  }
  const int local = g - P.atomOff;
  const int sc = S->stepCount + 1;
  if (pending) {
    if (local >= P.nMolMe) {
      const float b = S->betaC;
      v.x *= b; v.y *= b; v.z *= b;
    } else if (S->thermoMetal) {
      const float b = S->betaM;
      v.x *= b; v.y *= b; v.z *= b;
    }
  }
  if (local < P.nMolMe && P.iRegime == 1) {
    int nDep = S->nMolDeposited, nTo = 0;
    bool act = false;
    if (sc <= P.stepEquil) act = true;
    else if (nDep < P.nMolMe) {
      act = true;
      if ((sc - P.stepEquil) % P.stepDeposit == 0) nTo = P.nMolToDeposit;
    }
    if (act) {
      if (local >= nDep && local < nDep + nTo) {
        r.z = 0.49f * P.region[2]; lo.z = 0.f;
        v.z = -P.velMagDepos;
      }
      if (local >= nDep + nTo) {
        r.z = 1.5f * P.region[2] + 0.5f * (float)(local + 1) * P.region[2]; lo.z = 0.f;
        v.x = 0.f; v.y = 0.f; v.z = 0.f;
      }
    }
  }
  const bool frozen = (local >= P.nMolMe) &&
                      !((r.x != P.xLeft) && (r.x < P.xRight) && (r.y != P.yTop) && (r.y != P.yBottom));
  if (!frozen) {
    const float h = 0.5f * P.deltaT;
    v.x += h * a.x; v.y += h * a.y; v.z += h * a.z;
    addHiLo(r.x, lo.x, P.deltaT * v.x);
    addHiLo(r.y, lo.y, P.deltaT * v.y);
    addHiLo(r.z, lo.z, P.deltaT * v.z);
  }
  if (r.x >= 0.5f * P.region[0]) addHiLo(r.x, lo.x, -P.region[0]);
  else if (r.x < -0.5f * P.region[0]) addHiLo(r.x, lo.x, P.region[0]);
  if (r.y >= 0.5f * P.region[1]) addHiLo(r.y, lo.y, -P.region[1]);
  else if (r.y < -0.5f * P.region[1]) addHiLo(r.y, lo.y, P.region[1]);
  if (r.z >= 0.5f * P.region[2]) addHiLo(r.z, lo.z, -P.region[2]);
  else if (r.z < -0.5f * P.region[2]) addHiLo(r.z, lo.z, P.region[2]);
  pos[g] = r;
  posLo[g] = lo;
  vel[g] = v;
  if (forceRebuild || S->nebrNow) binAtom(P, g, r, cellOf, slot, cellCount, bucket, cap, blockCount, spill, spillCount);
}

__global__ void k_integrate_mixed(BlockTab tab, const RepConst *__restrict__ rc, RepState *st,
                                  float4 *__restrict__ pos, float4 *__restrict__ posLo,
                                  float4 *__restrict__ vel, float4 *__restrict__ acc,
                                  int *__restrict__ cellOf, int *__restrict__ slot,
                                  int *__restrict__ cellCount, int forceRebuild, int *__restrict__ bucket,
                                  int cap, int *__restrict__ blockCount, int2 *__restrict__ spill,
                                  int *__restrict__ spillCount, const float4 *__restrict__ hostR,
                                  const float *__restrict__ hostV, const float *__restrict__ hostA) {
  pdlEnter();
  integrateMixedBody(blockIdx.x, tab, rc, st, pos, posLo, vel, acc, cellOf, slot, cellCount, forceRebuild, bucket, cap,
                     blockCount, spill, spillCount, hostR, hostV, hostA);
}

// ============================================================================================
// Verlet part 2 fused with the FP64 step reductions; the last block of each replica sums the
// block partials in block order (deterministic) and runs the step control.
// ============================================================================================
// The centre of mass sums hi/lo positions as double-floats (an unevaluated float pair added
// with error-free transformations): FP64-class accuracy on the FP32 pipes, FP64 running at a
// small fraction of the FP32 rate on this GPU.
struct DF {
  float hi, lo;
};
#define ADDF(k, x) acc[k] = dfAdd(acc[k], DF{(x), 0.f})
__device__ __forceinline__ DF dfAdd(DF a, DF b) {
  float s, e;
  twoSum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  const float t = s + e;
  return DF{t, e - (t - s)};
}
__device__ __forceinline__ DF dfWarpSum(DF x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DF y{__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)};
    x = dfAdd(x, y);
  }
  return x;
}

__device__ void stepControlMixed(const RepConst &P, RepState *S, const double (&A)[kMixAcc],
                                 const float (&M)[kMixMax], double *diff, float *diffF,
                                 int forceRebuild);

// Reduction block e of the step (APT * THREADS atoms), by a block of THREADS threads: the
// engine's kernel runs THREADS = THREADS with APT atoms per thread (1, 2, 4 or 8, picked by
// size); the persistent step runs its own block size with the same atoms per block (APT 0: the
// atoms per thread `apt` at run time).
template <int APT, int THREADS>
__device__ __forceinline__ void reduceMixedBody(
    int e, int apt, BlockTab tab, const RepConst *__restrict__ rc, RepState *st, const float4 *__restrict__ pos,
    const float4 *__restrict__ posLo, float4 *__restrict__ vel, const float4 *__restrict__ acc4,
    const float *__restrict__ fric, float2 *__restrict__ partDF, float *__restrict__ partF,
    const int *__restrict__ redFirst, unsigned *counter, double *__restrict__ diff64,
    const size_t *__restrict__ diffOff64, float *__restrict__ diffF, const size_t *__restrict__ diffOffF,
    int forceRebuild, const PublishArgs pub = PublishArgs{}) {
  const int rep = tab.rep[e];
  const RepConst &P = rc[rep];
  RepState *S = st + rep;
  const int b = tab.start[e];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const float h = 0.5f * P.deltaT;
  // per thread and per warp (64 atoms) in FP32, except the centre of mass (double-float over
  // the hi/lo positions); warp totals and everything above in FP64
  float acc[kMixAcc];
#pragma unroll
  for (int k = 0; k < kMixAcc; k++) acc[k] = 0.f;
  DF cm[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  float mm[kMixMax] = {0.f, 3.4e38f, 3.4e38f, 3.4e38f, -3.4e38f, -3.4e38f, -3.4e38f};
  const int atomsPerThread = APT > 0 ? APT : apt;
#pragma unroll
  for (int half = 0; half < (APT > 0 ? APT : apt); half++) {
    const int local = atomsPerThread * THREADS * b + half * THREADS + t;
    if (local >= P.nMol) continue;
    const int g = P.atomOff + local;
    const float4 r = pos[g];
    float4 v = vel[g];
    const float4 a = acc4[g];
    const bool metal = local < P.nMolMe;
    const bool frozen = !metal && !((r.x != P.xLeft) && (r.x < P.xRight) && (r.y != P.yTop) && (r.y != P.yBottom));
    if (!frozen) {
      v.x += h * a.x; v.y += h * a.y; v.z += h * a.z;
      vel[g] = v;
    }
    acc[MA_VSUM_X] += metal ? P.massMe * v.x : v.x;
    acc[MA_VSUM_Y] += v.y;
    acc[MA_VSUM_Z] += v.z;
    const float vv = v.x * v.x + v.y * v.y + v.z * v.z;
    mm[MM_VVMAX] = fmaxf(mm[MM_VVMAX], vv);
    acc[MA_USUM] += r.w;
    acc[MA_VIRIAL] += (metal ? P.massMe : 1.f) * (r.x * a.x + r.y * a.y + r.z * a.z);
    if (metal) {
      const float4 l = posLo[g];
      acc[MA_VVYZ_M] += v.y * v.y + v.z * v.z;
      acc[MA_VX2_M] += v.x * v.x;
      acc[MA_VX_M] += v.x;
      acc[MA_VY_M] += v.y;
      acc[MA_VZ_M] += v.z;
      cm[0] = dfAdd(cm[0], DF{r.x, l.x});
      cm[1] = dfAdd(cm[1], DF{r.y, l.y});
      cm[2] = dfAdd(cm[2], DF{r.z, l.z});
      if (P.hasFric) acc[MA_FRICT] += fric[g];
      mm[MM_MIN_X] = fminf(mm[MM_MIN_X], r.x); mm[MM_MAX_X] = fmaxf(mm[MM_MAX_X], r.x);
      mm[MM_MIN_Y] = fminf(mm[MM_MIN_Y], r.y); mm[MM_MAX_Y] = fmaxf(mm[MM_MAX_Y], r.y);
      mm[MM_MIN_Z] = fminf(mm[MM_MIN_Z], r.z); mm[MM_MAX_Z] = fmaxf(mm[MM_MAX_Z], r.z);
    } else {
      acc[MA_VV_C] += vv;
    }
  }
  // the replica's constants and state into shared memory for the step control of whichever
  // block finishes last, loaded by every block while it reduces (nothing writes the state
  // before the last block has arrived)
  __shared__ RepState sS;
  __shared__ RepConst sP;
  {
    const int *cs = reinterpret_cast<const int *>(&P);
    int *cd = reinterpret_cast<int *>(&sP);
    for (int i = t; i < (int)(sizeof(RepConst) / 4); i += THREADS) cd[i] = cs[i];
    const int *ss = reinterpret_cast<const int *>(S);
    int *sd = reinterpret_cast<int *>(&sS);
    for (int i = t; i < (int)(sizeof(RepState) / 4); i += THREADS) sd[i] = __ldcg(ss + i);
  }
  __shared__ DF shDF[THREADS / 32][kMixAcc];
  __shared__ float shF[THREADS / 32][kMixMax];
#pragma unroll
  for (int k = 0; k < kMixAcc; k++) {
    if (k >= MA_CM_X && k <= MA_CM_Z) continue;
    float x = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) shDF[w][k] = DF{x, 0.f};
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const DF x = dfWarpSum(cm[c]);
    if (lane == 0) shDF[w][MA_CM_X + c] = x;
  }
#pragma unroll
  for (int k = 0; k < kMixMax; k++) {
    float x = mm[k];
    for (int o = 16; o > 0; o >>= 1) {
      const float y = __shfl_xor_sync(0xffffffffu, x, o);
      x = (k == MM_VVMAX || k >= MM_MAX_X) ? fmaxf(x, y) : fminf(x, y);
    }
    if (lane == 0) shF[w][k] = x;
  }
  __syncthreads();
  const int pb = P.redFirstM + b;
  if (t < kMixAcc) {
    DF x{0.f, 0.f};
    for (int k = 0; k < THREADS / 32; k++) x = dfAdd(x, shDF[k][t]);
    partDF[(size_t)pb * kMixAcc + t] = make_float2(x.hi, x.lo);
  } else if (t >= 32 && t < 32 + kMixMax) {
    const int k = t - 32;
    float x = shF[0][k];
    for (int j = 1; j < THREADS / 32; j++)
      x = (k == MM_VVMAX || k >= MM_MAX_X) ? fmaxf(x, shF[j][k]) : fminf(x, shF[j][k]);
    partF[(size_t)pb * kMixMax + k] = x;
  }
  if (t < kMixAcc || (t >= 32 && t < 32 + kMixMax)) __threadfence();  // partials visible first
  __syncthreads();
  __shared__ bool last;
  if (t == 0) last = (atomicAdd(&counter[rep], 1u) == (unsigned)P.nRedBlocksM - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // block partials in a fixed order (whichever block finished last), as double-floats on the
  // FP32 pipes (FP64 runs at a small fraction of their rate on this GPU; a double-float sum of
  // a few hundred partials keeps ~1e-14 relative, far below the FP32 warp sums' own rounding).
  // Sums: thread t adds value t % 16 of rows t / 16 + kG * i (kG = THREADS / 16 row groups,
  // four rows of predicated loads in flight, two chains), then the row groups of a warp meet in
  // a shuffle and the warps in one step.  Extremes: value t % 8 of rows t / 8 + kG2 * i.
  static_assert(THREADS % 32 == 0 && THREADS >= 64 && kMixAcc <= 16 && kMixMax <= 8, "final sums: 16 and 8 values per row");
  constexpr int kG = THREADS / 16, kG2 = THREADS / 8;
  __shared__ DF sW[THREADS / 32][16];
  __shared__ float sWF[THREADS / 32][8];
  __shared__ double tot[kMixAcc];
  __shared__ float totF[kMixMax];
  const int p0 = P.redFirstM, nb = P.nRedBlocksM;
  {
    const int k = t & 15;
    DF x0{0.f, 0.f}, x1{0.f, 0.f};
    if (k < kMixAcc) {
      for (int j0 = t >> 4; j0 < nb; j0 += 4 * kG) {
        float2 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int j = j0 + u * kG;
          v[u] = j < nb ? __ldcg(partDF + (size_t)(p0 + j) * kMixAcc + k) : make_float2(0.f, 0.f);
        }
        x0 = dfAdd(x0, DF{v[0].x, v[0].y});
        x1 = dfAdd(x1, DF{v[1].x, v[1].y});
        x0 = dfAdd(x0, DF{v[2].x, v[2].y});
        x1 = dfAdd(x1, DF{v[3].x, v[3].y});
      }
    }
    DF x = dfAdd(x0, x1);
    const DF y{__shfl_xor_sync(0xffffffffu, x.hi, 16), __shfl_xor_sync(0xffffffffu, x.lo, 16)};
    x = dfAdd(x, y);
    if (lane < 16) sW[w][lane] = x;
  }
  {
    const int k = t & 7;
    const bool isMax = (k == MM_VVMAX || k >= MM_MAX_X);
    const float neutral = isMax ? -3.4e38f : 3.4e38f;
    float y = neutral;
    if (k < kMixMax) {
      for (int j0 = t >> 3; j0 < nb; j0 += 4 * kG2) {
        float z[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int j = j0 + u * kG2;
          z[u] = j < nb ? __ldcg(partF + (size_t)(p0 + j) * kMixMax + k) : neutral;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) y = isMax ? fmaxf(y, z[u]) : fminf(y, z[u]);
      }
    }
#pragma unroll
    for (int o = 8; o < 32; o <<= 1) {
      const float z = __shfl_xor_sync(0xffffffffu, y, o);
      y = isMax ? fmaxf(y, z) : fminf(y, z);
    }
    if (lane < 8) sWF[w][lane] = y;
  }
  __syncthreads();
  if (t < kMixAcc) {
    DF x = sW[0][t];
#pragma unroll
    for (int q = 1; q < THREADS / 32; q++) x = dfAdd(x, sW[q][t]);
    tot[t] = (double)x.hi + (double)x.lo;
  } else if (t >= 32 && t < 32 + kMixMax) {
    const int k = t - 32;
    const bool isMax = (k == MM_VVMAX || k >= MM_MAX_X);
    float y = sWF[0][k];
#pragma unroll
    for (int q = 1; q < THREADS / 32; q++) y = isMax ? fmaxf(y, sWF[q][k]) : fminf(y, sWF[q][k]);
    totF[k] = y;
  }
  __syncthreads();
  if (t == 0) counter[rep] = 0;
  double A[kMixAcc];
  float M[kMixMax];
#pragma unroll
  for (int k = 0; k < kMixAcc; k++) A[k] = tot[k];
#pragma unroll
  for (int k = 0; k < kMixMax; k++) M[k] = totF[k];
  stepControlMixed(sP, &sS, A, M, diff64 ? diff64 + diffOff64[rep] : nullptr,
                   diffF ? diffF + diffOffF[rep] : nullptr, forceRebuild);
  stateFromShared(&sS, S);
  if (pub.hostSt) publishReplica(&sS, rep, pub);
}

template <int APT>
__global__ void __launch_bounds__(kMixThreads) k_step_reduce_mixed(
    BlockTab tab, const RepConst *__restrict__ rc, RepState *st, const float4 *__restrict__ pos,
    const float4 *__restrict__ posLo, float4 *__restrict__ vel, const float4 *__restrict__ acc4,
    const float *__restrict__ fric, float2 *__restrict__ partDF, float *__restrict__ partF,
    const int *__restrict__ redFirst, unsigned *counter, double *__restrict__ diff64,
    const size_t *__restrict__ diffOff64, float *__restrict__ diffF, const size_t *__restrict__ diffOffF,
    int forceRebuild, PublishArgs pub) {
  pdlEnter();
  reduceMixedBody<APT, kMixThreads>(blockIdx.x, APT, tab, rc, st, pos, posLo, vel, acc4, fric, partDF, partF, redFirst,
                                    counter, diff64, diffOff64, diffF, diffOffF, forceRebuild, pub);
}

// Step control in FP64 (same schedule as the PLAIN stepControl: properties, thermostat
// decision, rebuild criterion, shear, deposition bookkeeping, averages, diffusion).
__device__ void stepControlMixed(const RepConst &P, RepState *S, const double (&A)[kMixAcc],
                                 const float (&M)[kMixMax], double *diff, float *diffF,
                                 int forceRebuild) {
  const int t = threadIdx.x;
  const int sc = S->stepCount + 1;
  __shared__ int diffDue, accumNow, printNow;
  __shared__ double cmc[3];
  const bool metal = P.nMolMe != 0;
  const double invMe = P.invNMolMe;
  // the step's scalars in three independent parts, each on lane 0 of its own warp (no two of
  // them write the same field); the property sums after them
  if (t == 0) {
    // kinetic energy (regime 2 subtracts the metal centre-of-mass velocity from vx), thermostat
    const double nMe = P.nMolMe;
    double vvMetal = A[MA_VX2_M] + A[MA_VVYZ_M];
    if (metal && P.iRegime == 2) {
      const double cmvx = A[MA_VX_M] * invMe;
      vvMetal = A[MA_VX2_M] - 2.0 * cmvx * A[MA_VX_M] + nMe * cmvx * cmvx + A[MA_VVYZ_M];
    }
    const double vvSum = A[MA_VV_C] + (double)P.massMe * vvMetal;
    S->red[RS_VVSUM] = (float)vvSum;
    const double kin = 0.5 * vvSum * P.invNMol;
    const bool thermo = ((P.iRegime == 2) && (sc > P.stepEquil) && (sc % P.stepThermostat == 0)) ||
                        ((P.iRegime == 1) && (sc % P.stepThermostat == 0));
    if (thermo) {
      S->betaC = (float)sqrt(1.0 + (double)P.gammaBerendsen * ((double)P.temperature * 1.5 * P.kB / kin - 1.0));
      S->betaM = (float)sqrt(1.0 + (double)P.gammaBerendsen * ((double)P.temperature * P.kB / kin - 1.0));
      S->thermoMetal = (P.iRegime == 2) && (sc > P.stepEquil) && (sc < P.stepEquil + P.stepCool);
      S->thermoPending = 1;
    } else {
      S->thermoPending = 0;
    }
    const double pe64 = A[MA_USUM] * P.invNMol;
    S->ke64 = kin;
    S->pe64 = pe64;
    S->virial64 = A[MA_VIRIAL];
    S->ke = (float)kin;
    S->pe = (float)pe64;
    S->te = (float)(kin + pe64);
  } else if (t == 32) {
    // the reduced values, the metal centre of mass and its velocity, the friction force
    S->red[RS_VSUM_X] = (float)A[MA_VSUM_X]; S->red[RS_VSUM_Y] = (float)A[MA_VSUM_Y];
    S->red[RS_VSUM_Z] = (float)A[MA_VSUM_Z];
    S->red[RS_VVMAX] = M[MM_VVMAX];
    S->red[RS_USUM] = (float)A[MA_USUM];
    S->red[RS_CM_X] = (float)A[MA_CM_X]; S->red[RS_CM_Y] = (float)A[MA_CM_Y]; S->red[RS_CM_Z] = (float)A[MA_CM_Z];
    S->red[RS_MIN_X] = metal ? M[MM_MIN_X] : 0.f; S->red[RS_MIN_Y] = metal ? M[MM_MIN_Y] : 0.f;
    S->red[RS_MIN_Z] = metal ? M[MM_MIN_Z] : 0.f;
    S->red[RS_MAX_X] = metal ? M[MM_MAX_X] : 0.f; S->red[RS_MAX_Y] = metal ? M[MM_MAX_Y] : 0.f;
    S->red[RS_MAX_Z] = metal ? M[MM_MAX_Z] : 0.f;
    S->red[RS_FRICT] = (float)A[MA_FRICT];
    S->cmVel[0] = (float)A[MA_VX_M]; S->cmVel[1] = (float)A[MA_VY_M]; S->cmVel[2] = (float)A[MA_VZ_M];
    diffDue = 0;
    if (metal) {
      S->cmVal = (float)(A[MA_CM_X] * invMe);
      S->cmVelVal = (float)(A[MA_VX_M] * invMe);
      S->frictVal = P.hasFric ? (float)A[MA_FRICT] : 0.f;
      if (P.iRegime == 2 && sc > P.stepEquil && ((sc - P.stepEquil) % P.stepDiffuse == 0) && diff && diffF) {
        diffDue = 1;
        cmc[0] = A[MA_CM_X] * invMe; cmc[1] = A[MA_CM_Y] * invMe; cmc[2] = A[MA_CM_Z] * invMe;
      }
    } else {
      S->cmVal = 0.f; S->cmVelVal = 0.f; S->frictVal = 0.f;
    }
  } else if (t == 64) {
    // rebuild criterion, shear drive schedule, deposition count
    if (forceRebuild || S->nebrNow) {
      S->nebrNow = 0;
      S->dispHi = 0.f;
      S->rebuilds++;
    }
    S->dispHi += sqrtf(M[MM_VVMAX]) * P.deltaT;
    if (S->dispHi > 0.5f * P.rNebrShell) S->nebrNow = 1;
    if (P.iRegime == 2 && metal && sc > P.stepEquil + P.stepCool) {
      if ((float)(A[MA_VX_M] * invMe) < 0.005f) S->shear += P.deltaF;  // cmVelVal
      S->shearCount = 0;
    }
    if (P.iRegime == 1) {
      const int nDep = S->nMolDeposited;
      if (sc > P.stepEquil && nDep < P.nMolMe && (sc - P.stepEquil) % P.stepDeposit == 0)
        S->nMolDeposited = nDep + P.nMolToDeposit;
    }
  }
  __syncthreads();
  if (t < 7 && t != 3) {
    // property p = t: value, running sum and sum of squares; the stepAvg snapshot
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
    // oneStep (p = 3) is timed on the host: its sums are only snapshotted and cleared
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
  // ---- diffusion sample with FP64 accumulators (EvalDiffusion / AccumDiffusion,
  // SurfaceGrowth.cu:2898-2952); float mirrors of the counts, the running average and the
  // finished table keep the host readers' layout (DiffLayout)
  const int nB = P.nBuffDiffuse, nV = P.nValDiffuse;
  double *org = diff;                      // nB x 6: orgR, rTrue
  double *rr = diff + (size_t)nB * 6;      // nB x nV
  double *av = rr + (size_t)nB * nV;       // nV
  float *tbF = diffF;                      // nB x 7, element 0 = count (int bits)
  float *avF = diffF + (size_t)nB * 7 + (size_t)nB * nV;
  float *prF = avF + nV;
  // one thread per buffer (the buffers are independent); the accumulation below runs only in
  // a step where a buffer fills
  int filled = 0;
  {
    for (int nb = t; nb < nB; nb += blockDim.x) {
      double *o = org + 6 * nb;
      const int count = __float_as_int(tbF[7 * nb]);
      if (count == 0) {
        o[0] = cmc[0]; o[1] = cmc[1]; o[2] = cmc[2];
        o[3] = cmc[0]; o[4] = cmc[1]; o[5] = cmc[2];
      }
      if (count >= 0) {
        double *rrb = rr + (size_t)nb * nV;
        double d[3];
        for (int k = 0; k < 3; k++) {
          // unwrap the centre of mass by whole boxes (Nint of the jump, ComputeDefs.h:70-71)
          const double L = P.region[k];
          const double j = (o[3 + k] - cmc[k]) * P.invRegion[k];
          o[3 + k] = cmc[k] + L * (double)((j < 0.) ? -(long long)(0.5 - j) : (long long)(0.5 + j));
          d[k] = o[3 + k] - o[k];
        }
        rrb[count] = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      }
      tbF[7 * nb] = __int_as_float(count + 1);
      filled |= (count + 1 == nV) ? 1 : 0;
    }
  }
  if (!__syncthreads_or(filled)) return;
  for (int nb = 0; nb < nB; nb++) {
    if (t == 0) {
      accumNow = (__float_as_int(tbF[7 * nb]) == nV);
      printNow = 0;
    }
    __syncthreads();
    if (accumNow) {
      const double *rrb = rr + (size_t)nb * nV;
      for (int j = t; j < nV; j += blockDim.x) {
        av[j] += rrb[j];
        avF[j] = (float)av[j];
      }
      __syncthreads();
      if (t == 0) {
        tbF[7 * nb] = __int_as_float(0);
        S->countDiffuseAv++;
        printNow = (S->countDiffuseAv == P.limitDiffuseAv);
      }
      __syncthreads();
      if (printNow) {
        const double fac = 1.0 / (3.0 * 2.0 * P.stepDiffuse * (double)P.deltaT * P.limitDiffuseAv);
        for (int j = t; j < nV; j += blockDim.x) {
          double vj = av[j];
          if (j >= 1) vj *= fac / j;
          prF[j] = (float)vj;
          av[j] = 0.0;
          avF[j] = 0.f;
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

// ============================================================================================
// The persistent step: one cooperative launch runs a whole MIXED step over all replicas, its
// phases separated by a grid-wide barrier instead of kernel boundaries (the step loop of
// DoComputationsW, SurfaceGrowth.cu:2141-2489, as one launch).  Every block of the grid is
// resident (cooperative launch); each phase walks its block table with a grid stride, running
// the same device functions as the separate kernels:
//   integrate + cell histogram | scan + in-cell order | list build (its work queue spans the
//   grid) | EAM density and carbon forces | metal forces | reduction + step control.
// The barrier waits at most waitCycles clock cycles; a block that gives up sets SG_ERR_TIMEOUT
// in every replica's flags, counts it in the replica's timeouts and leaves the kernel, so the
// blocks still waiting give up at the same barrier in turn and the launch ends.  The context is
// then not usable (its state is partly stepped): destroy it.
// ============================================================================================
struct PersistArgs {
  BlockTab atomTab, metalTab, carbonTab, redTab;
  const int *tileRep, *tileStart, *tileFirst;
  int nScanBlocks;
  const RepConst *rc;
  RepState *st;
  float4 *pos, *posLo, *vel, *acc;
  int *cellOf, *slot, *cellCount, *cellStart, *bucket;
  int cap;
  int *blockCount, *active;
  int2 *heavy, *spill;
  int *work;
  int itemAtoms;
  int *sortIdx;
  float4 *sortPos;
  int *nn, *nbl, *ns, *sl, *nrl;
  unsigned *rl;
  int rowStride, nebrMax, descending;
  float *rho, *dF, *Fv, *fric;
  const float4 *eamTab;
  float2 *partDF;
  float *partF;
  const int *redFirst;
  unsigned *counter;
  double *diff64;
  const size_t *diffOff64;
  float *diffF;
  const size_t *diffOffF;
  int apt, forceRebuild, nrep;
  unsigned *bar;  // {arrived, generation}
  long long waitCycles;
};

// Grid-wide barrier with a bounded wait.  Thread 0 of each block reads the generation, makes
// the block's writes visible (fence) and arrives; the last block to arrive resets the count
// and advances the generation, the others wait until it changes or the limit runs out.
__device__ __noinline__ bool gridBarrier(const PersistArgs &a) {
  __syncthreads();
  __shared__ int sOk;
  if (threadIdx.x == 0) {
    volatile unsigned *gen = a.bar + 1;
    const unsigned g0 = *gen;
    __threadfence();
    bool ok = true;
    if (atomicAdd(a.bar, 1u) == gridDim.x - 1) {
      atomicExch(a.bar, 0u);
      __threadfence();
      atomicAdd(a.bar + 1, 1u);
    } else {
      const long long t0 = clock64();
      while (*gen == g0) {
        if (clock64() - t0 > a.waitCycles) {
          ok = false;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (!ok)
      for (int r = 0; r < a.nrep; r++) {
        setFlag(a.st + r, 8 /*SG_ERR_TIMEOUT*/);
        atomicAdd(&a.st[r].timeouts, 1);
      }
    sOk = ok;
  }
  __syncthreads();
  return sOk != 0;
}

template <int MT>
__global__ void __launch_bounds__(128) k_step_persistent(PersistArgs a) {
  const int G = gridDim.x;
  for (int e = blockIdx.x; e < a.atomTab.nblocks; e += G)
    integrateMixedBody(e, a.atomTab, a.rc, a.st, a.pos, a.posLo, a.vel, a.acc, a.cellOf, a.slot, a.cellCount,
                       a.forceRebuild, a.bucket, a.cap, a.blockCount, a.spill, a.work + 3);
  if (!gridBarrier(a)) return;
  for (int e = blockIdx.x; e < a.nScanBlocks; e += G) {
    scanRankBody<kScanCells, 128>(e, a.tileRep, a.tileStart, a.tileFirst, a.rc, a.st, a.cellCount, a.cellStart, a.cap,
                                  a.forceRebuild, a.active, a.heavy, a.work, a.itemAtoms, a.blockCount, a.bucket,
                                  a.cellOf, a.pos, a.sortIdx, a.sortPos, a.nn, a.ns, a.nrl, a.spill);
    __syncthreads();
  }
  if (!gridBarrier(a)) return;
  clearBlockCount(a.blockCount, a.nScanBlocks);
  nebrFusedBody(a.tileRep, a.active, a.heavy, a.work, a.rc, a.st, a.cellStart, a.sortPos, a.nn, a.nbl, a.ns, a.sl,
                  a.nrl, a.rl, a.rowStride, a.nebrMax, a.descending);
  if (!gridBarrier(a)) return;
  const int nm = a.metalTab.nblocks, nc = a.carbonTab.nblocks;
  for (int e = blockIdx.x; e < nm + nc; e += G) {
    if (e < nm) {
      const RepConst &P = a.rc[a.metalTab.rep[e]];
      rhoBody_mixed<MT>(e, P, a.metalTab, a.pos, a.nn, a.nbl, a.rho, a.dF, a.Fv, a.rowStride, a.eamTab + 2 * P.tabOff);
    } else {
      carbonBody_mixed(e - nm, a.carbonTab, a.rc, a.pos, a.acc, a.nn, a.nbl, a.ns, a.sl, a.nrl, a.rl, a.rowStride);
    }
    __syncthreads();
  }
  if (!gridBarrier(a)) return;
  for (int e = blockIdx.x; e < nm; e += G) {
    const RepConst &P = a.rc[a.metalTab.rep[e]];
    forceMetalBody_mixed<MT>(e, P, a.metalTab, a.pos, a.acc, a.nn, a.nbl, a.dF, a.Fv, a.fric, a.rowStride,
                             a.eamTab + 2 * P.tabOff);
  }
  if (!gridBarrier(a)) return;
  for (int e = blockIdx.x; e < a.redTab.nblocks; e += G) {
    reduceMixedBody<0, 128>(e, a.apt, a.redTab, a.rc, a.st, a.pos, a.posLo, a.vel, a.acc, a.fric, a.partDF, a.partF,
                            a.redFirst, a.counter, a.diff64, a.diffOff64, a.diffF, a.diffOffF, a.forceRebuild);
    __syncthreads();
  }
}

}  // namespace sg

using namespace sg;

#define MCK(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return sg_fail(SG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// phi(r), phi'(r), f(r), f'(r) of the Zhou-Wadley-Johnson forms (SurfaceGrowth.cu:46-69) in FP64
static void eamPairExact(const RepConst &P, double r, double out[4]) {
  const double rei = P.rei, x = r * rei;
  const double eA = std::exp(-(double)P.alpha * (x - 1.0)), eB = std::exp(-(double)P.beta * (x - 1.0));
  const double uk = x - P.kappa, ul = x - P.lambda;
  const double dA = 1.0 + std::pow(uk, 20.0), dB = 1.0 + std::pow(ul, 20.0);
  const double tA = P.alpha + 20.0 * std::pow(uk, 19.0) / dA, tB = P.beta + 20.0 * std::pow(ul, 19.0) / dB;
  out[0] = P.A * eA / dA - P.B * eB / dB;
  out[1] = (-(double)P.A * eA * tA / dA + (double)P.B * eB * tB / dB) * rei;
  out[2] = P.fe * eB / dB;
  out[3] = -(double)P.fe * rei * eB * tB / dB;
}

// Interval of width h with values g0, g1 and slopes d0, d1 at its ends: the coefficients of
// g(r_k + s) = c0 + c1 s + c2 s^2 + c3 s^3 (the cubic Hermite interpolant), expanded around the
// left end in FP64.
static float4 hermite(double g0, double d0, double g1, double d1, double h) {
  const double c2 = (3.0 * (g1 - g0) / h - 2.0 * d0 - d1) / h;
  const double c3 = (d0 + d1 - 2.0 * (g1 - g0) / h) / (h * h);
  return make_float4((float)g0, (float)d0, (float)c2, (float)c3);
}

bool sg_mixed_staging_ok(sg_ctx *c) {
  const MixedBufs *m = static_cast<const MixedBufs *>(c->mixed);
  return m && m->stagedOk;
}

int sg_mixed_init(sg_ctx *c) {
  MixedBufs *m = new MixedBufs;
  c->mixed = m;
  // EAM tables
  const int knots = (c->opt.eam_table_knots == 0) ? 1024 : c->opt.eam_table_knots;
  std::vector<float4> tab;
  for (int r = 0; r < c->nrep; r++) {
    RepConst &P = c->hrc[r];
    P.nTab = 0;
    if (knots < 2 || P.nMolMe == 0 || P.rei <= 0.f) continue;
    const double rmin = 0.6 / P.rei, rmax = std::sqrt((double)P.rrCutEam);
    const double h = (rmax - rmin) / (knots - 1);
    P.tabOff = (int)(tab.size() / 2);  // in intervals (two float4 each)
    P.nTab = knots;
    P.rTabMin = (float)rmin;
    P.rTabH = (float)h;
    P.rTabInv = (float)(1.0 / h);
    // interval k: g(r_k + s) = c0 + c1 s + c2 s^2 + c3 s^3, the cubic Hermite interpolant of
    // the values and slopes at r_k and r_k+1, expanded around r_k in FP64 (its derivative
    // c1 + 2 c2 s + 3 c3 s^2 then carries no cancellation of neighbouring table values)
    for (int k = 0; k < knots; k++) {
      double a[4], b[4];
      eamPairExact(P, rmin + k * h, a);
      eamPairExact(P, rmin + (k + 1) * h, b);
      for (int fn = 0; fn < 2; fn++) tab.push_back(hermite(a[2 * fn], a[2 * fn + 1], b[2 * fn], b[2 * fn + 1], h));
    }
  }
  // the staged metal kernels hold the largest replica table in shared memory
  int maxTab = 0;
  for (int r = 0; r < c->nrep; r++) maxTab = std::max(maxTab, c->hrc[r].nTab);
  m->stagedSmem = (size_t)2 * maxTab * sizeof(float4);
  m->stagedOk = maxTab > 0 && m->stagedSmem <= 160 * 1024;
  if (m->stagedOk && m->stagedSmem > 48 * 1024)
    m->stagedOk = allowStagedSmem<4>(m->stagedSmem) == cudaSuccess && allowStagedSmem<8>(m->stagedSmem) == cudaSuccess &&
                  allowStagedSmem<16>(m->stagedSmem) == cudaSuccess && allowStagedSmem<32>(m->stagedSmem) == cudaSuccess;
  cudaGetLastError();
  if (!m->stagedOk) c->eamStaged = false;
  MCK(cudaMalloc(&m->eamTab, sizeof(float4) * std::max<size_t>(tab.size(), 1)));
  sg_register_region(c, m->eamTab, sizeof(float4) * std::max<size_t>(tab.size(), 1));
  if (!tab.empty())
    MCK(cudaMemcpyAsync(m->eamTab, tab.data(), sizeof(float4) * tab.size(), cudaMemcpyHostToDevice, c->stream));
  MCK(cudaMemcpyAsync(c->rc, c->hrc.data(), sizeof(RepConst) * c->nrep, cudaMemcpyHostToDevice, c->stream));
  MCK(cudaStreamSynchronize(c->stream));
  // reduction blocks of m->mixAtoms atoms: the largest of 1024, 2048, 4096 that still gives two
  // blocks per SM, else 512 (more atoms per thread: fewer, longer blocks and fewer partials,
  // faster at the batched size; a single small system keeps 512 for its parallelism)
  {
    m->mixAtoms = kMixAtoms;
    for (int a = 8 * kMixAtoms; a > kMixAtoms; a /= 2) {
      long long blocks = 0;
      for (int r = 0; r < c->nrep; r++) blocks += (c->hrc[r].nMol + a - 1) / a;
      if (blocks >= 2LL * std::max(c->numSMs, 1)) {
        m->mixAtoms = a;
        break;
      }
    }
    std::vector<int> rr, ss;
    for (int r = 0; r < c->nrep; r++) {
      RepConst &P = c->hrc[r];
      P.nRedBlocksM = (P.nMol + m->mixAtoms - 1) / m->mixAtoms;
      P.redFirstM = (int)rr.size();
      for (int b = 0; b < P.nRedBlocksM; b++) { rr.push_back(r); ss.push_back(b); }
    }
    m->redN = (int)rr.size();
    MCK(cudaMalloc(&m->redRep, sizeof(int) * std::max<size_t>(rr.size(), 1)));
    sg_register_region(c, m->redRep, sizeof(int) * std::max<size_t>(rr.size(), 1));
    MCK(cudaMalloc(&m->redStart, sizeof(int) * std::max<size_t>(ss.size(), 1)));
    sg_register_region(c, m->redStart, sizeof(int) * std::max<size_t>(ss.size(), 1));
    MCK(cudaMemcpyAsync(m->redRep, rr.data(), sizeof(int) * rr.size(), cudaMemcpyHostToDevice, c->stream));
    MCK(cudaMemcpyAsync(m->redStart, ss.data(), sizeof(int) * ss.size(), cudaMemcpyHostToDevice, c->stream));
    MCK(cudaMemcpyAsync(c->rc, c->hrc.data(), sizeof(RepConst) * c->nrep, cudaMemcpyHostToDevice, c->stream));
    MCK(cudaStreamSynchronize(c->stream));
  }
  const int nRed = std::max(m->redN, 1);
  MCK(cudaMalloc(&m->partDF, sizeof(float2) * nRed * kMixAcc));
  sg_register_region(c, m->partDF, sizeof(float2) * nRed * kMixAcc);
  MCK(cudaMalloc(&m->partF, sizeof(float) * nRed * kMixMax));
  sg_register_region(c, m->partF, sizeof(float) * nRed * kMixMax);
  MCK(cudaMalloc(&m->counter, sizeof(unsigned) * c->nrep));
  sg_register_region(c, m->counter, sizeof(unsigned) * c->nrep);
  MCK(cudaMemsetAsync(m->counter, 0, sizeof(unsigned) * c->nrep, c->stream));
  size_t total = 0;
  m->diffOff64.resize(c->nrep);
  for (int r = 0; r < c->nrep; r++) {
    m->diffOff64[r] = total;
    const sg_simparams &p = c->hp[r];
    if (p.iRegime == 2) total += (size_t)p.nBuffDiffuse * 6 + (size_t)p.nBuffDiffuse * p.nValDiffuse + p.nValDiffuse;
  }
  MCK(cudaMalloc(&m->diff64, sizeof(double) * std::max<size_t>(total, 1)));
  sg_register_region(c, m->diff64, sizeof(double) * std::max<size_t>(total, 1));
  MCK(cudaMemsetAsync(m->diff64, 0, sizeof(double) * std::max<size_t>(total, 1), c->stream));
  MCK(cudaMalloc(&m->dDiffOff64, sizeof(size_t) * c->nrep));
  sg_register_region(c, m->dDiffOff64, sizeof(size_t) * c->nrep);
  MCK(cudaMemcpyAsync(m->dDiffOff64, m->diffOff64.data(), sizeof(size_t) * c->nrep, cudaMemcpyHostToDevice,
                      c->stream));
  MCK(cudaStreamSynchronize(c->stream));
  return SG_OK;
}

void sg_mixed_free(sg_ctx *c) {
  MixedBufs *m = static_cast<MixedBufs *>(c->mixed);
  if (!m) return;
  cudaFree(m->partDF);
  cudaFree(m->partF);
  cudaFree(m->counter);
  cudaFree(m->diff64);
  cudaFree(m->dDiffOff64);
  cudaFree(m->eamTab);
  cudaFree(m->redRep);
  cudaFree(m->redStart);
  delete m;
  c->mixed = nullptr;
}

int sg_mixed_enqueue_integrate(sg_ctx *c, int forceRebuild, const sg_float4 *hostR, const sg_float3 *hostV,
                               const sg_float3 *hostA) {
  if (!c->atomTab.n) return SG_OK;
  MCK(launchK(c->pdl, k_integrate_mixed, c->atomTab.n, 128, 0, c->stream, c->atomTab.view(), c->rc, c->st, c->pos, c->posLo, c->vel,
                                                         c->acc, c->cellOf, c->slot, c->cellCount, forceRebuild,
                c->bucket, c->bucketCap, c->blockCount, c->spill, c->nebrWork + 3,
                reinterpret_cast<const float4 *>(hostR), reinterpret_cast<const float *>(hostV),
                reinterpret_cast<const float *>(hostA)));
  MCK(cudaGetLastError());
  return SG_OK;
}

// The metal chain (density, metal forces) on the side stream beside the carbon pass, joined
// before the reduction, as in PLAIN; no centre-of-mass-velocity pass.
int sg_mixed_enqueue_forces(sg_ctx *c) {
  MixedBufs *m = static_cast<MixedBufs *>(c->mixed);
  const bool fork = c->metalRun.n > 0;
  if (fork) {
    MCK(cudaEventRecord(c->evFork, c->stream));
    MCK(cudaStreamWaitEvent(c->side, c->evFork, 0));
    launchMetalChain_mixed(c->pdl, c->metalLanes, c->metalRun.n, c->eamStaged ? c->numSMs * 4 : 0,
                           m->stagedSmem, c->side, c->metalRun.view(), c->rc, c->pos, c->acc,
                           c->nn, c->nbl, c->rho, c->dF, c->Fv, c->fric, c->rowStride, m->eamTab);
    if (c->opt.phase_timing) cudaEventRecordWithFlags(c->phaseEv[7], c->side, cudaEventRecordExternal);
    MCK(cudaGetLastError());
  }
  if (c->carbonTabT.n) {
    MCK(launchCarbon_mixed(c->pdl, c->carbonBlocks, c->carbonTabT.n, c->stream, c->carbonTabT.view(), c->rc, c->pos,
                           c->acc, c->nn, c->nbl, c->ns, c->sl, c->nrl, c->rl, c->rowStride));
  }
  if (c->opt.phase_timing) cudaEventRecordWithFlags(c->phaseEv[3], c->stream, cudaEventRecordExternal);
  MCK(cudaGetLastError());
  if (fork) {
    MCK(cudaEventRecord(c->evJoin, c->side));
    MCK(cudaStreamWaitEvent(c->stream, c->evJoin, 0));
  } else if (c->opt.phase_timing) {
    cudaEventRecordWithFlags(c->phaseEv[7], c->stream, cudaEventRecordExternal);
  }
  return SG_OK;
}

int sg_mixed_enqueue_reduce(sg_ctx *c, int forceRebuild, bool publish) {
  MixedBufs *m = static_cast<MixedBufs *>(c->mixed);
  if (!c->redTab.n) return SG_OK;
  auto kern = m->mixAtoms == 8 * kMixThreads   ? k_step_reduce_mixed<8>
              : m->mixAtoms == 4 * kMixThreads ? k_step_reduce_mixed<4>
              : m->mixAtoms == 2 * kMixThreads ? k_step_reduce_mixed<2>
                                               : k_step_reduce_mixed<1>;
  MCK(launchK(c->pdl, kern, m->redN, kMixThreads, 0, c->stream,
      BlockTab{m->redRep, m->redStart, m->redN}, c->rc, c->st, c->pos, c->posLo, c->vel, c->acc, c->fric, m->partDF, m->partF,
      c->dRedFirst, m->counter, m->diff64, m->dDiffOff64, c->diffBuf, c->dDiffOff, forceRebuild,
      publish ? PublishArgs{c->hostSt, c->devSeq, c->hostSeq, c->nrep} : PublishArgs{}));
  MCK(cudaGetLastError());
  return SG_OK;
}

// The differentiation form's fitted model in a MIXED context: phi and f become the uniform cubic
// B-splines of theta (SG_DIFF_SPLINE_COEFFS coefficients each on SG_DIFF_SPLINE_INTERVALS equal
// intervals from 0.6 r_e to the EAM cutoff, the piece of the end interval continuing past it),
// and the metal-carbon Lennard-Jones epsilon and sigma become theta[0], theta[1] (its cutoff
// stays the parameter block's).  Each table interval takes the values and slopes of the spline
// piece that holds its midpoint at both ends, so when the table's knots include the spline's
// (intervals - 1 a multiple of SG_DIFF_SPLINE_INTERVALS, e.g. eam_table_knots 1016) every table
// cubic is the spline's own piece; otherwise the table is the spline's Hermite interpolant.
extern "C" int sg_load_diff_theta(sg_ctx *c, int rep, const double *theta) {
  if (!c || !theta || rep < -1 || rep >= c->nrep) return sg_fail(SG_ERR_INVALID, "sg_load_diff_theta: bad arguments");
  if (c->opt.mode != SG_MODE_MIXED || !c->mixed)
    return sg_fail(SG_ERR_UNSUPPORTED, "sg_load_diff_theta: tables exist in MIXED mode only");
  MixedBufs *m = static_cast<MixedBufs *>(c->mixed);
  constexpr int kSC = SG_DIFF_SPLINE_COEFFS, kSI = SG_DIFF_SPLINE_INTERVALS;
  for (int r = (rep < 0 ? 0 : rep); r < (rep < 0 ? c->nrep : rep + 1); r++) {
    RepConst &P = c->hrc[r];
    if (P.nMolMe == 0) continue;
    if (P.nTab == 0) return sg_fail(SG_ERR_UNSUPPORTED, "sg_load_diff_theta: replica %d has no EAM table", r);
    const int knots = P.nTab;
    const double rmin = 0.6 / P.rei, rmax = std::sqrt((double)P.rrCutEam);
    const double h = (rmax - rmin) / (knots - 1);
    const double hs = (rmax - rmin) / kSI;
    // value and slope of spline `fn` (0: phi, 1: f) at r, on piece k
    auto spline = [&](int fn, int k, double r, double &g, double &d) {
      const double *cf = theta + 2 + fn * kSC + k;
      const double t = (r - rmin) / hs - k, t2 = t * t, t3 = t2 * t, u = 1.0 - t;
      g = (cf[0] * u * u * u + cf[1] * (3.0 * t3 - 6.0 * t2 + 4.0) + cf[2] * (-3.0 * t3 + 3.0 * t2 + 3.0 * t + 1.0) +
           cf[3] * t3) / 6.0;
      d = (cf[0] * (-0.5 * u * u) + cf[1] * (1.5 * t2 - 2.0 * t) + cf[2] * (-1.5 * t2 + t + 0.5) + cf[3] * (0.5 * t2)) / hs;
    };
    std::vector<float4> tab;
    tab.reserve((size_t)2 * knots);
    for (int k = 0; k < knots; k++) {
      const double ra = rmin + k * h, rb = rmin + (k + 1) * h;
      const int piece = std::max(0, std::min((int)std::floor((0.5 * (ra + rb) - rmin) / hs), kSI - 1));
      for (int fn = 0; fn < 2; fn++) {
        double g0, d0, g1, d1;
        spline(fn, piece, ra, g0, d0);
        spline(fn, piece, rb, g1, d1);
        tab.push_back(hermite(g0, d0, g1, d1, h));
      }
    }
    P.epsLJ = (float)theta[0];
    P.sigmaLJ = (float)theta[1];
    c->hp[r].epsLJ = P.epsLJ;
    c->hp[r].sigmaLJ = P.sigmaLJ;
    MCK(cudaMemcpyAsync(m->eamTab + (size_t)2 * P.tabOff, tab.data(), sizeof(float4) * tab.size(),
                        cudaMemcpyHostToDevice, c->stream));
  }
  MCK(cudaMemcpyAsync(c->rc, c->hrc.data(), sizeof(RepConst) * c->nrep, cudaMemcpyHostToDevice, c->stream));
  MCK(cudaStreamSynchronize(c->stream));
  return SG_OK;
}

// The persistent step (k_step_persistent) of one step on the context's stream: a cooperative
// launch of c->persistGrid blocks of 128 threads (all resident).
int sg_mixed_enqueue_persistent(sg_ctx *c, int forceRebuild) {
  MixedBufs *m = static_cast<MixedBufs *>(c->mixed);
  PersistArgs a;
  memset(&a, 0, sizeof(a));
  a.atomTab = c->atomTab.view();
  a.metalTab = c->metalRun.view();
  a.carbonTab = c->carbonTabT.view();
  a.redTab = BlockTab{m->redRep, m->redStart, m->redN};
  a.tileRep = c->tileTab.rep;
  a.tileStart = c->tileTab.start;
  a.tileFirst = c->dTileFirst;
  a.nScanBlocks = c->nScanBlocks;
  a.rc = c->rc;
  a.st = c->st;
  a.pos = c->pos; a.posLo = c->posLo; a.vel = c->vel; a.acc = c->acc;
  a.cellOf = c->cellOf; a.slot = c->slot; a.cellCount = c->cellCount; a.cellStart = c->cellStart;
  a.bucket = c->bucket; a.cap = c->bucketCap;
  a.blockCount = c->blockCount; a.active = c->activeCells; a.heavy = c->heavyItems; a.work = c->nebrWork;
  a.spill = c->spill;
  a.itemAtoms = c->nebrItemAtoms;
  a.sortIdx = c->sortIdx; a.sortPos = c->sortPos;
  a.nn = c->nn; a.nbl = c->nbl; a.ns = c->ns; a.sl = c->sl; a.nrl = c->nrl; a.rl = c->rl;
  a.rowStride = c->rowStride; a.nebrMax = c->nebrMax; a.descending = c->nebrDescending;
  a.rho = c->rho; a.dF = c->dF; a.Fv = c->Fv; a.fric = c->fric;
  a.eamTab = m->eamTab;
  a.partDF = m->partDF; a.partF = m->partF; a.redFirst = c->dRedFirst; a.counter = m->counter;
  a.diff64 = m->diff64; a.diffOff64 = m->dDiffOff64; a.diffF = c->diffBuf; a.diffOffF = c->dDiffOff;
  a.apt = m->mixAtoms / 128;
  a.forceRebuild = forceRebuild;
  a.nrep = c->nrep;
  a.bar = c->persistBar;
  a.waitCycles = c->persistWaitCycles;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(c->persistGrid);
  cfg.blockDim = dim3(128);
  cfg.stream = c->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (c->metalLanes == 4) MCK(cudaLaunchKernelEx(&cfg, k_step_persistent<4>, a));
  else MCK(cudaLaunchKernelEx(&cfg, k_step_persistent<kMT>, a));
  return SG_OK;
}

// Blocks per SM the persistent step can keep resident (its grid is that times the SM count).
int sg_mixed_persistent_blocks_per_sm(int metalLanes) {
  int n = 0;
  cudaError_t e = metalLanes == 4 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_persistent<4>, 128, 0)
                                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_step_persistent<kMT>, 128, 0);
  return e == cudaSuccess ? n : 0;
}
