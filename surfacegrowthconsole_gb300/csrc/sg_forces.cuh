// sg_forces.cuh - the force passes (EAM density, EAM + LJ metal forces, LJ + graphene carbon
// forces), written once and compiled twice: by sg_kernels_plain.cu with -fmad=false (PLAIN:
// the reference's operation order, kernels k_rho / k_force_metal / k_force_carbon) and by
// sg_kernels_mixed.cu with FMA contraction (MIXED: the same model, kernels *_mixed).  The
// including unit defines SG_KN(name) to name its kernels.
#pragma once
#include "sg_device.cuh"

#ifndef SG_KN
#error "define SG_KN(name) before including sg_forces.cuh"
#endif

// SG_FAST_RECIP (MIXED): quotients through reciprocals and reciprocal square roots (__fdividef,
// rsqrtf: a few ulp) shared between the terms that use them — the graphene angle and radial
// terms, the EAM pair distance and force, the LJ terms — instead of an IEEE division or square
// root per quotient of the reference's expressions (PLAIN keeps those for bit parity).  Fewer
// instructions for passes that are bound by instruction issue.
// SG_EAM_TABLE (MIXED): the EAM pair functions come from cubic Hermite tables instead of the
// analytic forms; the table buffer is one more kernel parameter, and the force bodies take the
// start of the replica's table (in global memory, or staged in shared memory).
#ifdef SG_EAM_TABLE
#define SG_EAM_PARAM , const float4 *__restrict__ eamTab
#define SG_EAM_ARG , eamTab
#define SG_EAM_BODY_PARAM , const float4 *tabBase
#define SG_EAM_BASE(P) , eamTab + 2 * (P).tabOff
#define SG_EAM_PAIR(P, r) eamPairTab(P, tabBase, r)
#define SG_EAM_DENS(P, r) eamDensTab(P, tabBase, r)
#else
#define SG_EAM_PARAM
#define SG_EAM_ARG
#define SG_EAM_BODY_PARAM
#define SG_EAM_BASE(P)
#define SG_EAM_PAIR(P, r) eamPair(P, r)
#define SG_EAM_DENS(P, r) eamDensity(P, r)
#endif

namespace sg {

// ============================================================================================
// EAM (Zhou-Wadley-Johnson analytic forms, SurfaceGrowth.cu:46-210).  The pair functions
// share their exponentials and powers; each value is the one the reference's separate
// function calls produce for the same argument.
// ============================================================================================
struct EamPair {
  float phi, dphi, df;
};
__device__ __forceinline__ EamPair eamPair(const RepConst &P, float r) {
  const float x = r * P.rei;
  const float xm1 = x - 1.f;
  const float eA = expf(-P.alpha * xm1);
  const float eB = expf(-P.beta * xm1);
  const float pk = x - P.kappa, pl = x - P.lambda;
  const float dA = 1.f + powf(pk, 20.f);
  const float dB = 1.f + powf(pl, 20.f);
  const float tA = P.alpha + 20.f * powf(pk, 19.f) / dA;
  const float tB = P.beta + 20.f * powf(pl, 19.f) / dB;
  EamPair e;
  e.phi = P.A * eA / dA - P.B * eB / dB;
  e.dphi = (-P.A * eA * tA / dA + P.B * eB * tB / dB) * P.rei;
  e.df = -P.fe * P.rei * eB * tB / dB;
  return e;
}
__device__ __forceinline__ float eamDensity(const RepConst &P, float r) {
  const float x = r * P.rei;
  return P.fe * expf(-P.beta * (x - 1.f)) / (1.f + powf(x - P.lambda, 20.f));
}
__device__ __forceinline__ float eamEmbed(const RepConst &P, float rho) {
  const float rhon = 0.85f * P.rhoe;
  if (rho < rhon) {
    const float rhoni = P.rhoei * 1.176471f;
    const float x = rho * rhoni - 1.f;
    return P.Fn[0] + P.Fn[1] * x + P.Fn[2] * x * x + P.Fn[3] * x * x * x;
  }
  const float rhoo = 1.15f * P.rhoe;
  if ((rho >= rhon) && (rho < rhoo)) {
    const float x = rho * P.rhoei - 1.f;
    return P.F[0] + P.F[1] * x + P.F[2] * x * x + P.F[3] * x * x * x;
  }
  if (rho >= rhoo) {
    const float x = rho * P.rhoei;
    return P.Fe * (1.f - logf(powf(x, P.eta))) * powf(x, P.eta);
  }
  return 0.f;
}
__device__ __forceinline__ float eamEmbedDeriv(const RepConst &P, float rho) {
  const float rhon = 0.85f * P.rhoe;
  if (rho < rhon) {
    const float rhoni = P.rhoei * 1.176471f;
    const float x = rho * rhoni - 1.f;
    return rhoni * (P.Fn[1] + 2.f * P.Fn[2] * x + 3.f * P.Fn[3] * x * x);
  }
  const float rhoo = 1.15f * P.rhoe;
  if ((rho >= rhon) && (rho < rhoo)) {
    const float y = rho * P.rhoei;
    return P.rhoei * (P.F[1] + 2.f * P.F[2] * (y - 1.f) + 3.f * P.F[3] * (y - 1.f) * (y - 1.f));
  }
  if (rho >= rhoo) {
    const float y = rho * P.rhoei;
    return -P.Fe * P.eta * P.rhoei * powf(y, (P.eta - 1.f)) * logf(powf(y, P.eta));
  }
  return 0.f;
}

#ifdef SG_EAM_TABLE
// Tabulated pair functions: on interval k (r_k = rTabMin + k h) each of phi and f is the cubic
// c0 + c1 s + c2 s^2 + c3 s^3 in s = r - r_k (the Hermite interpolant of the analytic values and
// slopes at both knots, expanded around r_k); the derivative is that of the cubic, so forces
// are the exact gradient of the tabulated energy.  Below the first knot (closer than any
// physical pair) the analytic forms.
__device__ __forceinline__ bool tabLocate(const RepConst &P, float r, int &k, float &sd) {
  if (P.nTab == 0 || r < P.rTabMin) return false;
  k = min((int)((r - P.rTabMin) * P.rTabInv), P.nTab - 1);
  sd = r - (P.rTabMin + (float)k * P.rTabH);
  return true;
}
// tab: the replica's table (interval k at tab[2k], tab[2k + 1]), in global or shared memory.
__device__ __forceinline__ EamPair eamPairTab(const RepConst &P, const float4 *tab, float r) {
  int k;
  float x;
  if (!tabLocate(P, r, k, x)) return eamPair(P, r);
  const float4 cp = tab[2 * k], cf = tab[2 * k + 1];
  EamPair e;
  e.phi = cp.x + x * (cp.y + x * (cp.z + x * cp.w));
  e.dphi = cp.y + x * (2.f * cp.z + 3.f * x * cp.w);
  e.df = cf.y + x * (2.f * cf.z + 3.f * x * cf.w);
  return e;
}
__device__ __forceinline__ float eamDensTab(const RepConst &P, const float4 *tab, float r) {
  int k;
  float x;
  if (!tabLocate(P, r, k, x)) return eamDensity(P, r);
  const float4 cf = tab[2 * k + 1];
  return cf.x + x * (cf.y + x * (cf.z + x * cf.w));
}
#endif

// Electron density of each metal atom (EamComputeRhoK, cu:716-773), plus F(rho) and F'(rho),
// which the reference re-evaluates per pair in the force kernel.  MT lanes share one metal
// atom (128 / MT atoms per block): lane l takes list entries l, l + MT, ...; the partial sums
// meet in a shuffle tree.  k_rho runs MT = kMT; k_rho_tpa<MT> the choices of the autotuner.
constexpr int kMetalBatch = 4;  // list entries per lane whose loads are issued together
template <int MT> __device__ __forceinline__ unsigned laneGroupMask() {
  return MT == 32 ? 0xffffffffu : ((1u << MT) - 1) << (threadIdx.x & 31 & ~(MT - 1));
}

// Block-table entry e (128 / MT atoms of replica rep) with replica constants P.
template <int MT>
__device__ __forceinline__ void SG_KN(rhoBody)(int e, const RepConst &P, BlockTab tab,
                                               const float4 *__restrict__ pos, const int *__restrict__ nn,
                                               const int *__restrict__ nbl, float *__restrict__ rho,
                                               float *__restrict__ dF, float *__restrict__ Fv,
                                               int rowStride SG_EAM_BODY_PARAM) {
  const int sub = threadIdx.x & (MT - 1);
  const unsigned gmask = laneGroupMask<MT>();
  const int i = tab.start[e] + threadIdx.x / MT;
  const int metalEnd = P.atomOff + P.nMolMe;
  const bool valid = i < metalEnd;
  float sum = 0.f;
  if (valid) {
    const float4 A = pos[i];
    const int n = nn[i];
    const int *row = nbl + (size_t)i * rowStride;
    // kMetalBatch entries per lane per round: their indices, then their positions, load
    // together (the sum still takes the entries in the same order)
    for (int j0 = sub; j0 < n; j0 += kMetalBatch * MT) {
      int k[kMetalBatch];
      float4 B[kMetalBatch];
#pragma unroll
      for (int q = 0; q < kMetalBatch; q++) k[q] = (j0 + q * MT < n) ? row[j0 + q * MT] : -1;
#pragma unroll
      for (int q = 0; q < kMetalBatch; q++) B[q] = (k[q] >= 0) ? pos[k[q]] : A;
#pragma unroll
      for (int q = 0; q < kMetalBatch; q++) {
        if (k[q] < 0) continue;
        const float dx = minImg(A.x - B[q].x, P.region[0]);
        const float dy = minImg(A.y - B[q].y, P.region[1]);
        const float dz = minImg(A.z - B[q].z, P.region[2]);
        const float rr = dx * dx + dy * dy + dz * dz;
#ifdef SG_FAST_RECIP
        if ((rr < P.rrCutEam) && (k[q] < metalEnd)) sum += SG_EAM_DENS(P, rr * rsqrtf(rr));
#else
        if ((rr < P.rrCutEam) && (k[q] < metalEnd)) sum += SG_EAM_DENS(P, sqrtf(rr));
#endif
      }
    }
  }
#pragma unroll
  for (int o = MT / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(gmask, sum, o);
  if (valid && sub == 0) {
    rho[i] = sum;
    dF[i] = eamEmbedDeriv(P, sum);
    Fv[i] = eamEmbed(P, sum);
  }
}

__global__ void __launch_bounds__(128) SG_KN(k_rho)(BlockTab tab, const RepConst *__restrict__ rc,
                                             const float4 *__restrict__ pos, const int *__restrict__ nn,
                                             const int *__restrict__ nbl, float *__restrict__ rho,
                                             float *__restrict__ dF, float *__restrict__ Fv,
                                             int rowStride SG_EAM_PARAM) {
  pdlEnter();
  const RepConst &P = rc[tab.rep[blockIdx.x]];
  SG_KN(rhoBody)<kMT>(blockIdx.x, P, tab, pos, nn, nbl, rho, dF, Fv, rowStride SG_EAM_BASE(P));
}
template <int MT>
__global__ void __launch_bounds__(128) SG_KN(k_rho_tpa)(BlockTab tab, const RepConst *__restrict__ rc,
                                                 const float4 *__restrict__ pos, const int *__restrict__ nn,
                                                 const int *__restrict__ nbl, float *__restrict__ rho,
                                                 float *__restrict__ dF, float *__restrict__ Fv,
                                                 int rowStride SG_EAM_PARAM) {
  pdlEnter();
  const RepConst &P = rc[tab.rep[blockIdx.x]];
  SG_KN(rhoBody)<MT>(blockIdx.x, P, tab, pos, nn, nbl, rho, dF, Fv, rowStride SG_EAM_BASE(P));
}

// Lennard-Jones metal-carbon term (cu:880-884).
__device__ __forceinline__ void ljTerms(const RepConst &P, float rr, float &fc, float &u) {
#ifdef SG_FAST_RECIP
  const float irr = __fdividef(1.f, rr);
  const float rri = P.sigmaLJ * P.sigmaLJ * irr;
  const float rri3 = rri * rri * rri;
  fc = 48.f * P.epsLJ * rri3 * (rri3 - 0.5f) * irr;
#else
  const float rri = P.sigmaLJ * P.sigmaLJ / rr;
  const float rri3 = rri * rri * rri;
  fc = 48.f * P.epsLJ * rri3 * (rri3 - 0.5f) * rri / (P.sigmaLJ * P.sigmaLJ);
#endif
  u = 4.f * P.epsLJ * rri3 * (rri3 - 1.f);
}

// Forces on metal atoms: EAM pair + embedding with metal neighbours, LJ with carbon neighbours
// (ComputeForcesK case 0, cu:856-897, epilogue cu:1069-1082); MT lanes per atom as in the
// density pass (k_force_metal: MT = kMT; k_force_metal_tpa<MT>: the autotuner's choices).
template <int MT>
__device__ __forceinline__ void SG_KN(forceMetalBody)(int e, const RepConst &P, BlockTab tab,
                                                      float4 *__restrict__ pos, float4 *__restrict__ acc,
                                                      const int *__restrict__ nn, const int *__restrict__ nbl,
                                                      const float *__restrict__ dF,
                                                      const float *__restrict__ Fv, float *__restrict__ fric,
                                                      int rowStride SG_EAM_BODY_PARAM) {
  const int sub = threadIdx.x & (MT - 1);
  const unsigned gmask = laneGroupMask<MT>();
  const int i = tab.start[e] + threadIdx.x / MT;
  const int metalEnd = P.atomOff + P.nMolMe;
  const bool valid = i < metalEnd;
  float fx = 0.f, fy = 0.f, fz = 0.f, rx = 0.f, u = 0.f;
  if (valid) {
    const float4 A = pos[i];
    const int n = nn[i];
    const float dFi = dF[i];
    const int *row = nbl + (size_t)i * rowStride;
    // batches of entries as in the density pass; same order of the sums
    for (int j0 = sub; j0 < n; j0 += kMetalBatch * MT) {
      int k[kMetalBatch];
      float4 B[kMetalBatch];
      float dFk[kMetalBatch];
#pragma unroll
      for (int q = 0; q < kMetalBatch; q++) k[q] = (j0 + q * MT < n) ? row[j0 + q * MT] : -1;
#pragma unroll
      for (int q = 0; q < kMetalBatch; q++) {
        B[q] = (k[q] >= 0) ? pos[k[q]] : A;
        dFk[q] = (k[q] >= 0 && k[q] < metalEnd) ? dF[k[q]] : 0.f;
      }
#pragma unroll
      for (int q = 0; q < kMetalBatch; q++) {
        if (k[q] < 0) continue;
        const float dx = minImg(A.x - B[q].x, P.region[0]);
        const float dy = minImg(A.y - B[q].y, P.region[1]);
        const float dz = minImg(A.z - B[q].z, P.region[2]);
        const float rr = dx * dx + dy * dy + dz * dz;
        if (k[q] < metalEnd) {
          if (rr >= P.rrCutEam) continue;  // the reference computes and then zeroes the term
#ifdef SG_FAST_RECIP
          const float ri = rsqrtf(rr);
          const float r = rr * ri;
#else
          const float r = sqrtf(rr);
#endif
          const EamPair e = SG_EAM_PAIR(P, r);
          float fc = -e.dphi;
          fc = fc - e.df * (dFi + dFk[q]);
#ifdef SG_FAST_RECIP
          fc = fc * ri;
#else
          fc = fc / r;
#endif
          fx = fx + fc * dx; fy = fy + fc * dy; fz = fz + fc * dz;
          u += e.phi;
        } else {
          if (rr >= P.rrCutLJ) continue;
          float fc, ul;
          ljTerms(P, rr, fc, ul);
          u += ul;
          fx = fx + fc * dx; fy = fy + fc * dy; fz = fz + fc * dz;
          rx = rx + fc * dx;
        }
      }
    }
  }
#pragma unroll
  for (int o = MT / 2; o > 0; o >>= 1) {
    fx += __shfl_xor_sync(gmask, fx, o);
    fy += __shfl_xor_sync(gmask, fy, o);
    fz += __shfl_xor_sync(gmask, fz, o);
    rx += __shfl_xor_sync(gmask, rx, o);
    u += __shfl_xor_sync(gmask, u, o);
  }
  if (valid && sub == 0) {
    acc[i] = make_float4(fx / P.massMe, fy / P.massMe, fz / P.massMe, 0.f);
    pos[i].w = 0.5f * u + Fv[i];
    if (P.hasFric) fric[i] = rx;
  }
}

__global__ void __launch_bounds__(128) SG_KN(k_force_metal)(BlockTab tab, const RepConst *__restrict__ rc,
                                                     float4 *__restrict__ pos, float4 *__restrict__ acc,
                                                     const int *__restrict__ nn, const int *__restrict__ nbl,
                                                     const float *__restrict__ dF, const float *__restrict__ Fv,
                                                     float *__restrict__ fric, int rowStride SG_EAM_PARAM) {
  pdlEnter();
  const RepConst &P = rc[tab.rep[blockIdx.x]];
  SG_KN(forceMetalBody)<kMT>(blockIdx.x, P, tab, pos, acc, nn, nbl, dF, Fv, fric, rowStride SG_EAM_BASE(P));
}
template <int MT>
__global__ void __launch_bounds__(128) SG_KN(k_force_metal_tpa)(BlockTab tab, const RepConst *__restrict__ rc,
                                                         float4 *__restrict__ pos, float4 *__restrict__ acc,
                                                         const int *__restrict__ nn, const int *__restrict__ nbl,
                                                         const float *__restrict__ dF,
                                                         const float *__restrict__ Fv, float *__restrict__ fric,
                                                         int rowStride SG_EAM_PARAM) {
  pdlEnter();
  const RepConst &P = rc[tab.rep[blockIdx.x]];
  SG_KN(forceMetalBody)<MT>(blockIdx.x, P, tab, pos, acc, nn, nbl, dF, Fv, fric, rowStride SG_EAM_BASE(P));
}

#ifdef SG_EAM_TABLE
// Staged variants (MIXED): a grid of at most stagedGrid blocks; each block copies its replica's
// table into shared memory (again when a later entry belongs to another replica) and walks the
// block-table entries blockIdx.x, blockIdx.x + gridDim.x, ...
template <int MT>
__global__ void __launch_bounds__(128) SG_KN(k_rho_staged)(BlockTab tab, const RepConst *__restrict__ rc,
                                                    const float4 *__restrict__ pos, const int *__restrict__ nn,
                                                    const int *__restrict__ nbl, float *__restrict__ rho,
                                                    float *__restrict__ dF, float *__restrict__ Fv,
                                                    int rowStride SG_EAM_PARAM) {
  extern __shared__ float4 sTab[];
  pdlEnter();
  int staged = -1;
  for (int e = blockIdx.x; e < tab.nblocks; e += gridDim.x) {
    const int rep = tab.rep[e];
    const RepConst &P = rc[rep];
    if (rep != staged) {
      __syncthreads();
      for (int q = threadIdx.x; q < 2 * P.nTab; q += blockDim.x) sTab[q] = eamTab[2 * P.tabOff + q];
      __syncthreads();
      staged = rep;
    }
    SG_KN(rhoBody)<MT>(e, P, tab, pos, nn, nbl, rho, dF, Fv, rowStride, sTab);
  }
}
template <int MT>
__global__ void __launch_bounds__(128) SG_KN(k_force_metal_staged)(BlockTab tab, const RepConst *__restrict__ rc,
                                                            float4 *__restrict__ pos, float4 *__restrict__ acc,
                                                            const int *__restrict__ nn, const int *__restrict__ nbl,
                                                            const float *__restrict__ dF,
                                                            const float *__restrict__ Fv,
                                                            float *__restrict__ fric, int rowStride SG_EAM_PARAM) {
  extern __shared__ float4 sTab[];
  pdlEnter();
  int staged = -1;
  for (int e = blockIdx.x; e < tab.nblocks; e += gridDim.x) {
    const int rep = tab.rep[e];
    const RepConst &P = rc[rep];
    if (rep != staged) {
      __syncthreads();
      for (int q = threadIdx.x; q < 2 * P.nTab; q += blockDim.x) sTab[q] = eamTab[2 * P.tabOff + q];
      __syncthreads();
      staged = rep;
    }
    SG_KN(forceMetalBody)<MT>(e, P, tab, pos, acc, nn, nbl, dF, Fv, fric, rowStride, sTab);
  }
}

template <int MT>
static void SG_KN(launchStaged)(bool pdl, int grid, size_t smem, cudaStream_t s, BlockTab tab, const RepConst *rc,
                                float4 *pos, float4 *acc, const int *nn, const int *nbl, float *rho, float *dF,
                                float *Fv, float *fric, int rowStride, const float4 *eamTab) {
  launchK(pdl, SG_KN(k_rho_staged)<MT>, grid, 128, smem, s, tab, rc, pos, nn, nbl, rho, dF, Fv, rowStride, eamTab);
  launchK(pdl, SG_KN(k_force_metal_staged)<MT>, grid, 128, smem, s, tab, rc, pos, acc, nn, nbl, dF, Fv, fric,
          rowStride, eamTab);
}
#endif

// The metal chain with MT lanes per metal atom (4, 8, 16 or 32; grid = the block table for
// 128 / MT atoms per block), from the host of the including unit; pdl: programmatic
// dependent launch; stagedGrid > 0 (MIXED): the staged variants on at most that many blocks
// with stagedSmem bytes of table (launch errors are left for cudaGetLastError).
void SG_KN(launchMetalChain)(bool pdl, int mt, int grid, int stagedGrid, size_t stagedSmem, cudaStream_t s,
                             BlockTab tab, const RepConst *rc, float4 *pos, float4 *acc, const int *nn,
                             const int *nbl, float *rho, float *dF, float *Fv, float *fric,
                             int rowStride SG_EAM_PARAM) {
#ifdef SG_EAM_TABLE
  if (stagedGrid > 0) {
    const int g = grid < stagedGrid ? grid : stagedGrid;
    switch (mt) {
      case 4: SG_KN(launchStaged)<4>(pdl, g, stagedSmem, s, tab, rc, pos, acc, nn, nbl, rho, dF, Fv, fric, rowStride, eamTab); break;
      case 8: SG_KN(launchStaged)<8>(pdl, g, stagedSmem, s, tab, rc, pos, acc, nn, nbl, rho, dF, Fv, fric, rowStride, eamTab); break;
      case 32: SG_KN(launchStaged)<32>(pdl, g, stagedSmem, s, tab, rc, pos, acc, nn, nbl, rho, dF, Fv, fric, rowStride, eamTab); break;
      default: SG_KN(launchStaged)<16>(pdl, g, stagedSmem, s, tab, rc, pos, acc, nn, nbl, rho, dF, Fv, fric, rowStride, eamTab);
    }
    return;
  }
#else
  (void)stagedGrid;
  (void)stagedSmem;
#endif
  switch (mt) {
    case 4:
      launchK(pdl, SG_KN(k_rho_tpa)<4>, grid, 128, 0, s, tab, rc, pos, nn, nbl, rho, dF, Fv, rowStride SG_EAM_ARG);
      launchK(pdl, SG_KN(k_force_metal_tpa)<4>, grid, 128, 0, s, tab, rc, pos, acc, nn, nbl, dF, Fv, fric,
              rowStride SG_EAM_ARG);
      break;
    case 8:
      launchK(pdl, SG_KN(k_rho_tpa)<8>, grid, 128, 0, s, tab, rc, pos, nn, nbl, rho, dF, Fv, rowStride SG_EAM_ARG);
      launchK(pdl, SG_KN(k_force_metal_tpa)<8>, grid, 128, 0, s, tab, rc, pos, acc, nn, nbl, dF, Fv, fric,
              rowStride SG_EAM_ARG);
      break;
    case 32:
      launchK(pdl, SG_KN(k_rho_tpa)<32>, grid, 128, 0, s, tab, rc, pos, nn, nbl, rho, dF, Fv, rowStride SG_EAM_ARG);
      launchK(pdl, SG_KN(k_force_metal_tpa)<32>, grid, 128, 0, s, tab, rc, pos, acc, nn, nbl, dF, Fv, fric,
              rowStride SG_EAM_ARG);
      break;
    default:
      launchK(pdl, SG_KN(k_rho), grid, 128, 0, s, tab, rc, pos, nn, nbl, rho, dF, Fv, rowStride SG_EAM_ARG);
      launchK(pdl, SG_KN(k_force_metal), grid, 128, 0, s, tab, rc, pos, acc, nn, nbl, dF, Fv, fric,
              rowStride SG_EAM_ARG);
  }
}

// Forces on carbon atoms (ComputeForcesK case 1, cu:899-1063, epilogue cu:1083-1088): LJ with
// metal neighbours and the harmonic graphene terms over the first three carbon neighbours
// within rCutC in list order, with the second-neighbour angle and out-of-plane terms of each.
// kCT = 4 lanes share one carbon atom.  The walk goes over the atom's relevant list (metal
// entries and close entries with their full-list positions; the full list when the relevant
// list overflowed), four entries at a time; a ballot finds, in list order, the first three
// close carbons (their data go to shared memory) and the full-list position p2 of the third.
// The reference reuses its list counter for the bonded loop (cu:989), so after the third close
// carbon its walk resumes at entry 4: metal entries at positions 4..p2 contribute their LJ term
// twice, and entry 3 is skipped when p2 == 2.  After the walk, lane q < 3 adds the
// second-neighbour terms of close carbon q (walking that neighbour's close list) and the
// own-angle term of close carbons q, q + 1, and lane 3 the radial and out-of-plane terms (the
// lanes 0..2 run one angle each, converged, instead of lane 3 running all three); the four
// partial sums meet in a shuffle tree.
__device__ __forceinline__ void relEntry(bool full, const int *row, const unsigned *rrow, int atomOff, int e,
                                         int &k, int &j) {
  if (full) { k = row[e]; j = e; }
  else { const unsigned v = rrow[e]; k = atomOff + (int)(v >> 8); j = (int)(v & 0xffu); }
}

// MINB: resident blocks per SM the register budget is cut for (8: 64 registers, 12: 40, 16:
// 32); more warps hide more of the gathers' latency at large sizes, fewer registers cost
// instructions (launchCarbon picks one, the autotuner times them).
// Block-table entry e of the carbon pass (128 / kCT carbon atoms), by a 128-thread block.
__device__ __forceinline__ void SG_KN(carbonBody)(int e, BlockTab tab, const RepConst *__restrict__ rc,
                                                  float4 *__restrict__ pos, float4 *__restrict__ acc,
                                                  const int *__restrict__ nn, const int *__restrict__ nbl,
                                                  const int *__restrict__ ns, const int *__restrict__ sl,
                                                  const int *__restrict__ nrl, const unsigned *__restrict__ rl,
                                                  int rowStride) {
  __shared__ float sD[128 / kCT][3][4];  // dx, dy, dz, |d| of close carbon q
  __shared__ float sZ[128 / kCT][3];     // its z - z_0
  __shared__ int sK[128 / kCT][3];       // its index
  const int rep = tab.rep[e];
  const RepConst &P = rc[rep];
  const int sub = threadIdx.x & (kCT - 1);
  const int a = threadIdx.x / kCT;  // atom slot in the block
  const int glane = threadIdx.x & 31 & ~(kCT - 1);
  const unsigned gmask = ((1u << kCT) - 1) << glane;
  const int i = tab.start[e] + a;
  const int metalEnd = P.atomOff + P.nMolMe;
  const bool valid = i < P.atomOff + P.nMol;
  float fx = 0.f, fy = 0.f, fz = 0.f, u = 0.f;
  int counti = 0, p2 = -1;
  const float4 A = valid ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const int nr = valid ? nrl[i] : 0;
  const bool full = nr < 0;
  const int nEnt = full ? nn[i] : nr;
  const int *row = nbl + (size_t)i * rowStride;
  const unsigned *rrow = rl + (size_t)i * kRelMax;
  for (int base = 0; base < nEnt; base += kCT) {
    const int e = base + sub;
    bool closeC = false;
    float lx = 0.f, ly = 0.f, lz = 0.f, lu = 0.f;
    float dx = 0.f, dy = 0.f, dz = 0.f, rr = 0.f, bz = 0.f;
    int k = -1, j = -1;
    if (e < nEnt) {
      relEntry(full, row, rrow, P.atomOff, e, k, j);
      const float4 B = pos[k];
      bz = B.z;
      dx = minImg(A.x - B.x, P.region[0]);
      dy = minImg(A.y - B.y, P.region[1]);
      dz = minImg(A.z - B.z, P.region[2]);
      rr = dx * dx + dy * dy + dz * dz;
      if (k < metalEnd) {
        if (rr < P.rrCutLJ) {
          float fc;
          ljTerms(P, rr, fc, lu);
          lx = fc * dx; ly = fc * dy; lz = fc * dz;
        }
      } else {
        closeC = rr < P.rrCutC;
      }
    }
    const unsigned bal = (__ballot_sync(gmask, closeC) >> glane) & ((1u << kCT) - 1);
    if (counti < 3) {
      if (closeC) {
        const int rank = counti + __popc(bal & ((1u << sub) - 1));
        if (rank < 3) {
          sD[a][rank][0] = dx; sD[a][rank][1] = dy; sD[a][rank][2] = dz; sD[a][rank][3] = sqrtf(rr);
          sZ[a][rank] = bz - P.z_0;
          sK[a][rank] = k;
        }
      }
      const int c2 = counti + __popc(bal);
      if (c2 >= 3) {  // the third close carbon is in this group of entries
        unsigned b = bal;
        for (int r = counti; r < 2; r++) b &= b - 1;  // drop the set bits of ranks counti..1
        p2 = __shfl_sync(gmask, j, glane + __ffs(b) - 1);
      }
      counti = min(c2, 3);
    }
    if (!(j == 3 && p2 == 2)) {  // entry 3 is never visited when the third NN sits at 2
      fx += lx; fy += ly; fz += lz; u += lu;
    }
  }
  // entries 4..p2 of the full list are walked a second time: their LJ terms repeat
  if (counti == 3 && p2 >= 4) {
    for (int e = sub; e < nEnt; e += kCT) {
      int k, j;
      relEntry(full, row, rrow, P.atomOff, e, k, j);
      if (j > p2) break;
      if (j < 4 || k >= metalEnd) continue;
      const float4 B = pos[k];
      const float dx = minImg(A.x - B.x, P.region[0]);
      const float dy = minImg(A.y - B.y, P.region[1]);
      const float dz = minImg(A.z - B.z, P.region[2]);
      const float rr = dx * dx + dy * dy + dz * dz;
      if (rr < P.rrCutLJ) {
        float fc, ul;
        ljTerms(P, rr, fc, ul);
        fx += fc * dx; fy += fc * dy; fz += fc * dz; u += ul;
      }
    }
  }
  __syncwarp(gmask);
  if (sub < 3 && sub < counti) {
    // second-neighbour terms of close carbon q = sub (cu:929-981)
    const int q = sub;
    const int k = sK[a][q];
    const float rnx = sD[a][q][0], rny = sD[a][q][1], rnz = sD[a][q][2], absR = sD[a][q][3];
    const float4 B = pos[k];
#ifdef SG_FAST_RECIP
    const float invR2 = __fdividef(1.f, absR * absR);
#endif
    // the neighbour's close list holds, in list order, every entry that can pass the rCutC test
    // below; four entries per load (a close-list row is 32 bytes, aligned)
    const int nk = ns[k];
    const bool fullk = nk < 0;
    const int lim = fullk ? nn[k] : nk;
    const int *src = fullk ? nbl + (size_t)k * rowStride : sl + (size_t)k * kShortMax;
    int countk = 0;
    for (int l0 = 0; l0 < lim && countk < 2; l0 += 4) {
      int mm[4];
      bool use[4];
      if (fullk) {
#pragma unroll
        for (int t = 0; t < 4; t++) {
          use[t] = l0 + t < lim;
          mm[t] = use[t] ? src[l0 + t] : 0;
        }
      } else {
        const int4 u = *reinterpret_cast<const int4 *>(src + l0);
        mm[0] = u.x; mm[1] = u.y; mm[2] = u.z; mm[3] = u.w;
#pragma unroll
        for (int t = 0; t < 4; t++) use[t] = l0 + t < lim;
      }
#pragma unroll
      for (int t = 0; t < 4; t++) {
        if (!use[t]) continue;
        const int m = mm[t];
        const float4 rm = pos[m];
        float ex = minImg(B.x - rm.x, P.region[0]);
        float ey = minImg(B.y - rm.y, P.region[1]);
        float ez = minImg(B.z - rm.z, P.region[2]);
        const float rr2 = ex * ex + ey * ey + ez * ez;
        if ((rr2 < P.rrCutC) && (m != i)) {
          ex = ex * (-1.f); ey = ey * (-1.f); ez = ez * (-1.f);
#ifdef SG_FAST_RECIP
          const float inv = __fdividef(1.f, absR * rr2);
          const float cs = (rnx * ex + rny * ey + rnz * ez) * inv;
          const float th = acosf(cs);
          const float dth = th - P.theta_0;
          const float tmp = P.mu_theta * dth * rsqrtf(1.f - cs * cs);
          float f = tmp * inv;
          fx = fx + f * ex; fy = fy + f * ey; fz = fz + f * ez;
          f = -tmp * cs * invR2;
          fx = fx + f * rnx; fy = fy + f * rny; fz = fz + f * rnz;
          f = -P.mu_p * (rm.z - P.z_0) * (1.f / 9.f);
#else
          const float cs = (rnx * ex + rny * ey + rnz * ez) / (absR * rr2);
          const float th = acosf(cs);
          const float dth = th - P.theta_0;
          const float tmp = P.mu_theta * dth / sqrtf(1.f - cs * cs);
          float f = tmp / (absR * rr2);
          fx = fx + f * ex; fy = fy + f * ey; fz = fz + f * ez;
          f = -tmp * cs / (absR * absR);
          fx = fx + f * rnx; fy = fy + f * rny; fz = fz + f * rnz;
          f = -P.mu_p * (rm.z - P.z_0) / 9.f;
#endif
          fz = fz + f;
          ++countk;
        }
        if (countk == 2) break;
      }
    }
  }
  if (counti == 3) {
    if (sub < 3) {
      // own-angle term of close carbons q, q + 1 (cu:1020-1061): one per lane 0..2
      const int p0 = sub, p1 = (sub == 2) ? 0 : sub + 1;
      const float rx0 = sD[a][p0][0], ry0 = sD[a][p0][1], rz0 = sD[a][p0][2], ar0 = sD[a][p0][3];
      const float rx1 = sD[a][p1][0], ry1 = sD[a][p1][1], rz1 = sD[a][p1][2], ar1 = sD[a][p1][3];
#ifdef SG_FAST_RECIP
      const float i0 = __fdividef(1.f, ar0), i1 = __fdividef(1.f, ar1);
      const float inv01 = i0 * i1;
      const float cs = (rx0 * rx1 + ry0 * ry1 + rz0 * rz1) * inv01;
      const float th = acosf(cs);
      const float dth = th - P.theta_0;
      const float tmp = P.mu_theta * dth * rsqrtf(1.f - cs * cs);
      float f = tmp * (1.f - ar0 * cs * i1) * inv01;
      fx = fx + f * rx1; fy = fy + f * ry1; fz = fz + f * rz1;
      f = tmp * (1.f - ar1 * cs * i0) * inv01;
#else
      const float cs = (rx0 * rx1 + ry0 * ry1 + rz0 * rz1) / (ar0 * ar1);
      const float th = acosf(cs);
      const float dth = th - P.theta_0;
      const float tmp = P.mu_theta * dth / sqrtf(1.f - cs * cs);
      float f = tmp * (1.f - ar0 * cs / ar1) / (ar0 * ar1);
      fx = fx + f * rx1; fy = fy + f * ry1; fz = fz + f * rz1;
      f = tmp * (1.f - ar1 * cs / ar0) / (ar0 * ar1);
#endif
      fx = fx + f * rx0; fy = fy + f * ry0; fz = fz + f * rz0;
      u += P.mu_theta * dth * dth;
    } else {
      // radial and out-of-plane terms (cu:985-1019): lane 3
      float dzs = 0.f;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        const float rx = sD[a][q][0], ry = sD[a][q][1], rz = sD[a][q][2], ar = sD[a][q][3];
#ifdef SG_FAST_RECIP
        const float f = -P.mu_r * (ar - 1.f) * __fdividef(1.f, ar);
#else
        const float f = -P.mu_r * (ar - 1.f) / ar;
#endif
        fx = fx + f * rx; fy = fy + f * ry; fz = fz + f * rz;
        u += P.mu_r * (ar - 1.f) * (ar - 1.f);
      }
      const float z0 = sZ[a][0], z1 = sZ[a][1], z2 = sZ[a][2];
      dzs = z0 + z1 + z2;
      float dZ = 2.f * (A.z - P.z_0) - dzs;
      fz = fz + -0.666666667f * P.mu_p * dZ;
      dZ = (A.z - P.z_0) - 0.33333333f * dzs;
      u += P.mu_p * dZ * dZ;
    }
  }
#pragma unroll
  for (int o = kCT / 2; o > 0; o >>= 1) {
    fx += __shfl_xor_sync(gmask, fx, o);
    fy += __shfl_xor_sync(gmask, fy, o);
    fz += __shfl_xor_sync(gmask, fz, o);
    u += __shfl_xor_sync(gmask, u, o);
  }
  if (valid && sub == 0) {
    acc[i] = make_float4(fx, fy, fz, 0.f);
    pos[i].w = 0.5f * u;
  }
}

template <int MINB>
__global__ void __launch_bounds__(128, MINB) SG_KN(k_force_carbon)(BlockTab tab, const RepConst *__restrict__ rc,
                                                      float4 *__restrict__ pos, float4 *__restrict__ acc,
                                                      const int *__restrict__ nn, const int *__restrict__ nbl,
                                                      const int *__restrict__ ns, const int *__restrict__ sl,
                                                      const int *__restrict__ nrl, const unsigned *__restrict__ rl,
                                                      int rowStride) {
  pdlEnter();
  SG_KN(carbonBody)(blockIdx.x, tab, rc, pos, acc, nn, nbl, ns, sl, nrl, rl, rowStride);
}

// The carbon pass with minBlocks (8, 12 or 16; others: 8) resident blocks per SM.
cudaError_t SG_KN(launchCarbon)(bool pdl, int minBlocks, int grid, cudaStream_t s, BlockTab tab,
                                const RepConst *rc, float4 *pos, float4 *acc, const int *nn, const int *nbl,
                                const int *ns, const int *sl, const int *nrl, const unsigned *rl, int rowStride) {
  switch (minBlocks) {
    case 12:
      return launchK(pdl, SG_KN(k_force_carbon)<12>, grid, 128, 0, s, tab, rc, pos, acc, nn, nbl, ns, sl, nrl, rl,
                     rowStride);
    case 16:
      return launchK(pdl, SG_KN(k_force_carbon)<16>, grid, 128, 0, s, tab, rc, pos, acc, nn, nbl, ns, sl, nrl, rl,
                     rowStride);
    default:
      return launchK(pdl, SG_KN(k_force_carbon)<8>, grid, 128, 0, s, tab, rc, pos, acc, nn, nbl, ns, sl, nrl, rl,
                     rowStride);
  }
}

}  // namespace sg
