// sg_adjoint.cu - the differentiation form: the metal part of the model (EAM with B-spline
// pair functions, metal-carbon Lennard-Jones) as a function of 66 fit parameters, its forces,
// and the gradients of the frame energies and of a force-matching loss from a hand-written
// adjoint pass.  No counterpart in the reference (its potentials are fixed analytic forms).
//
// Parameters theta: [0] epsilon, [1] sigma of the metal-carbon LJ; [2, 34) the cubic B-spline
// coefficients of phi(r); [34, 66) those of f(r), on 29 equal intervals from 0.6 r_e to the EAM
// cutoff.  On interval k (x = (r - r0) / h, t = x - k) a spline is sum_m c[k + m] b_m(t) with the
// uniform cubic B-spline weights b_0 = (1-t)^3/6, b_1 = (3t^3 - 6t^2 + 4)/6,
// b_2 = (-3t^3 + 3t^2 + 3t + 1)/6, b_3 = t^3/6: linear in the coefficients, C2 in r.
//
// Force matching.  With the residual e_i = 2 (F_i - F_ref,i) / (3N) held fixed,
//   dL/dtheta = -d/dtheta D,   D = sum_i e_i . dE/dr_i
//             = 1/2 sum_{i,j metal} phi'(r_ij) w_ij + sum_i F'(rho_i) g_i + sum_{MC} U'(r) w,
//   w_ij = rhat_ij . (e_i - e_j),  g_i = sum_j f'(r_ij) w_ij  (the change of rho_i along e),
// so  dD/dc_phi,k = 1/2 sum B_k'(r) w,   dD/dc_f,k = sum_i [F''(rho_i) g_i sum_j B_k(r_ij)
// + F'(rho_i) sum_j B_k'(r_ij) w_ij],  dD/d(eps, sigma) = sum_MC d U'(r)/d(eps, sigma) w.
// The adjoint kernel recomputes rho_i and g_i (first pass over the neighbours) and then adds
// these terms (second pass): nothing per pair is stored.
//
// Pair arithmetic in FP32 (FMA on), per-block parameter sums in shared-memory FP32 (a few
// thousand terms per block), energies, losses and gradients summed in FP64 across blocks.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sg_api.h"
#include "sg_device.cuh"
#include "sg_engine.h"
#include "sg_kernels.h"

namespace sg {

constexpr int kDP = SG_DIFF_NPARAM;
constexpr int kSC = SG_DIFF_SPLINE_COEFFS;
constexpr int kSI = SG_DIFF_SPLINE_INTERVALS;
constexpr int kPhi = 2, kDen = 2 + kSC;  // offsets of the two splines in theta
static_assert(kSC == kSI + 3 && kDP == 2 + 2 * kSC, "spline layout");

struct Spline {
  float r0, invH;  // first knot, 1 / interval width
};

// Interval and B-spline weights at r: values b[], derivatives with respect to r db[].
__device__ __forceinline__ int bspline(const Spline &s, float r, float (&b)[4], float (&db)[4]) {
  const float x = (r - s.r0) * s.invH;
  const int k = max(0, min((int)floorf(x), kSI - 1));
  const float t = x - (float)k, t2 = t * t, t3 = t2 * t, u = 1.f - t;
  b[0] = u * u * u * (1.f / 6.f);
  b[1] = (3.f * t3 - 6.f * t2 + 4.f) * (1.f / 6.f);
  b[2] = (-3.f * t3 + 3.f * t2 + 3.f * t + 1.f) * (1.f / 6.f);
  b[3] = t3 * (1.f / 6.f);
  db[0] = -0.5f * u * u * s.invH;
  db[1] = (1.5f * t2 - 2.f * t) * s.invH;
  db[2] = (-1.5f * t2 + t + 0.5f) * s.invH;
  db[3] = 0.5f * t2 * s.invH;
  return k;
}

// The reference's embedding function (SurfaceGrowth.cu:72-126 forms) with its first and second
// derivatives.
__device__ __forceinline__ void embedAll(const RepConst &P, float rho, float &F, float &Fp, float &Fpp) {
  const float rhon = 0.85f * P.rhoe, rhoo = 1.15f * P.rhoe;
  if (rho < rhon) {
    const float s = P.rhoei * 1.176471f, x = rho * s - 1.f;
    F = P.Fn[0] + x * (P.Fn[1] + x * (P.Fn[2] + x * P.Fn[3]));
    Fp = s * (P.Fn[1] + x * (2.f * P.Fn[2] + 3.f * x * P.Fn[3]));
    Fpp = s * s * (2.f * P.Fn[2] + 6.f * x * P.Fn[3]);
  } else if (rho < rhoo) {
    const float s = P.rhoei, x = rho * s - 1.f;
    F = P.F[0] + x * (P.F[1] + x * (P.F[2] + x * P.F[3]));
    Fp = s * (P.F[1] + x * (2.f * P.F[2] + 3.f * x * P.F[3]));
    Fpp = s * s * (2.f * P.F[2] + 6.f * x * P.F[3]);
  } else {
    const float y = rho * P.rhoei, ly = logf(y), yeta = powf(y, P.eta);
    F = P.Fe * (1.f - P.eta * ly) * yeta;
    Fp = -P.Fe * P.eta * P.eta * P.rhoei * yeta / y * ly;
    Fpp = -P.Fe * P.eta * P.eta * P.rhoei * P.rhoei * yeta / (y * y) * ((P.eta - 1.f) * ly + 1.f);
  }
}

__device__ __forceinline__ float spl(const float *c, int k, const float (&w)[4]) {
  return c[k] * w[0] + c[k + 1] * w[1] + c[k + 2] * w[2] + c[k + 3] * w[3];
}

// Block-wide parameter accumulator: shared FP32, flushed into the FP64 totals.
__device__ __forceinline__ void flushGrad(const float *sG, double *grad) {
  __syncthreads();
  for (int q = threadIdx.x; q < kDP; q += blockDim.x)
    if (sG[q] != 0.f) atomicAdd(&grad[q], (double)sG[q]);
}

__device__ __forceinline__ float warpSumF(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// ---- forward -----------------------------------------------------------------------------
// Density of every metal atom -> F'(rho) stored; F(rho) added to the frame energy.  kMT lanes
// per metal atom (kMetalPerBlock atoms per 128-thread block).
__global__ void __launch_bounds__(128) k_diff_rho(BlockTab tab, const RepConst *__restrict__ rc,
                                                  const float4 *__restrict__ pos, const int *__restrict__ nn,
                                                  const int *__restrict__ nbl, int rowStride,
                                                  const float *__restrict__ theta, Spline sp,
                                                  float *__restrict__ Fp, double *__restrict__ energy) {
  __shared__ float sT[kDP];
  for (int q = threadIdx.x; q < kDP; q += blockDim.x) sT[q] = theta[q];
  __syncthreads();
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  const int sub = threadIdx.x & (kMT - 1);
  const unsigned gmask = ((1u << kMT) - 1) << (threadIdx.x & 31 & ~(kMT - 1));
  const int i = tab.start[blockIdx.x] + threadIdx.x / kMT;
  const int metalEnd = P.atomOff + P.nMolMe;
  const bool valid = i < metalEnd;
  float rho = 0.f;
  if (valid) {
    const float4 A = pos[i];
    const int *row = nbl + (size_t)i * rowStride;
    for (int j = sub; j < nn[i]; j += kMT) {
      const int k = row[j];
      if (k >= metalEnd) continue;
      const float4 B = pos[k];
      const float dx = minImg(A.x - B.x, P.region[0]), dy = minImg(A.y - B.y, P.region[1]),
                  dz = minImg(A.z - B.z, P.region[2]);
      const float rr = dx * dx + dy * dy + dz * dz;
      if (rr >= P.rrCutEam) continue;
      float b[4], db[4];
      const int kk = bspline(sp, sqrtf(rr), b, db);
      rho += spl(sT + kDen, kk, b);
    }
  }
#pragma unroll
  for (int o = kMT / 2; o > 0; o >>= 1) rho += __shfl_xor_sync(gmask, rho, o);
  float Fv = 0.f;
  if (valid && sub == 0) {
    float F, Fd, Fdd;
    embedAll(P, rho, F, Fd, Fdd);
    Fp[i] = Fd;
    Fv = F;
  }
  Fv = warpSumF(Fv);
  if ((threadIdx.x & 31) == 0 && Fv != 0.f) atomicAdd(&energy[rep], (double)Fv);
}

// Forces on metal atoms (EAM + LJ with carbon neighbours), pair energies, and with grad != NULL
// dE/dtheta.
__global__ void __launch_bounds__(128) k_diff_force_metal(BlockTab tab, const RepConst *__restrict__ rc,
                                                          const float4 *__restrict__ pos,
                                                          const int *__restrict__ nn, const int *__restrict__ nbl,
                                                          int rowStride, const float *__restrict__ theta,
                                                          Spline sp, const float *__restrict__ Fp,
                                                          float4 *__restrict__ force, double *__restrict__ energy,
                                                          double *__restrict__ grad) {
  __shared__ float sT[kDP], sG[kDP];
  for (int q = threadIdx.x; q < kDP; q += blockDim.x) {
    sT[q] = theta[q];
    sG[q] = 0.f;
  }
  __syncthreads();
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  const int sub = threadIdx.x & (kMT - 1);
  const unsigned gmask = ((1u << kMT) - 1) << (threadIdx.x & 31 & ~(kMT - 1));
  const int i = tab.start[blockIdx.x] + threadIdx.x / kMT;
  const int metalEnd = P.atomOff + P.nMolMe;
  const bool valid = i < metalEnd;
  const float eps = sT[0], sig = sT[1];
  float fx = 0.f, fy = 0.f, fz = 0.f, u = 0.f;
  if (valid) {
    const float4 A = pos[i];
    const float Fpi = Fp[i];
    const int *row = nbl + (size_t)i * rowStride;
    for (int j = sub; j < nn[i]; j += kMT) {
      const int k = row[j];
      const float4 B = pos[k];
      const float dx = minImg(A.x - B.x, P.region[0]), dy = minImg(A.y - B.y, P.region[1]),
                  dz = minImg(A.z - B.z, P.region[2]);
      const float rr = dx * dx + dy * dy + dz * dz;
      if (k < metalEnd) {
        if (rr >= P.rrCutEam) continue;
        const float r = sqrtf(rr);
        float b[4], db[4];
        const int kk = bspline(sp, r, b, db);
        const float phi = spl(sT + kPhi, kk, b), dphi = spl(sT + kPhi, kk, db), df = spl(sT + kDen, kk, db);
        const float fc = -(dphi + df * (Fpi + Fp[k])) / r;
        fx += fc * dx; fy += fc * dy; fz += fc * dz;
        u += 0.5f * phi;
        if (grad) {
#pragma unroll
          for (int m = 0; m < 4; m++) {
            atomicAdd(&sG[kPhi + kk + m], 0.5f * b[m]);
            atomicAdd(&sG[kDen + kk + m], Fpi * b[m]);
          }
        }
      } else {
        if (rr >= P.rrCutLJ) continue;
        const float s2 = sig * sig / rr, s6 = s2 * s2 * s2, s12 = s6 * s6;
        const float fc = 24.f * eps * (2.f * s12 - s6) / rr;  // -U'(r) / r
        fx += fc * dx; fy += fc * dy; fz += fc * dz;
        u += 4.f * eps * (s12 - s6);                          // the whole pair, from the metal side
        if (grad) {
          atomicAdd(&sG[0], 4.f * (s12 - s6));                 // dU / d eps
          atomicAdd(&sG[1], 24.f * eps * (2.f * s12 - s6) / sig);  // dU / d sigma
        }
      }
    }
  }
#pragma unroll
  for (int o = kMT / 2; o > 0; o >>= 1) {
    fx += __shfl_xor_sync(gmask, fx, o);
    fy += __shfl_xor_sync(gmask, fy, o);
    fz += __shfl_xor_sync(gmask, fz, o);
    u += __shfl_xor_sync(gmask, u, o);
  }
  if (valid && sub == 0) force[i] = make_float4(fx, fy, fz, 0.f);
  float uw = (sub == 0 && valid) ? u : 0.f;
  uw = warpSumF(uw);
  if ((threadIdx.x & 31) == 0 && uw != 0.f) atomicAdd(&energy[rep], (double)uw);
  if (grad) flushGrad(sG, grad);
}

// Forces on carbon atoms: LJ with their metal neighbours (their energy is counted on the metal
// side).  One thread per carbon atom.
__global__ void __launch_bounds__(128, 8) k_diff_force_carbon(BlockTab tab, const RepConst *__restrict__ rc,
                                                           const float4 *__restrict__ pos,
                                                           const int *__restrict__ nn,
                                                           const int *__restrict__ nbl, int rowStride,
                                                           const float *__restrict__ theta,
                                                           float4 *__restrict__ force) {
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  const int i = tab.start[blockIdx.x] + threadIdx.x;
  if (i >= P.atomOff + P.nMol) return;
  const int metalEnd = P.atomOff + P.nMolMe;
  const float eps = theta[0], sig = theta[1];
  const float4 A = pos[i];
  const int *row = nbl + (size_t)i * rowStride;
  float fx = 0.f, fy = 0.f, fz = 0.f;
  for (int j = 0; j < nn[i]; j++) {
    const int k = row[j];
    if (k >= metalEnd) continue;
    const float4 B = pos[k];
    const float dx = minImg(A.x - B.x, P.region[0]), dy = minImg(A.y - B.y, P.region[1]),
                dz = minImg(A.z - B.z, P.region[2]);
    const float rr = dx * dx + dy * dy + dz * dz;
    if (rr >= P.rrCutLJ) continue;
    const float s2 = sig * sig / rr, s6 = s2 * s2 * s2, s12 = s6 * s6;
    const float fc = 24.f * eps * (2.f * s12 - s6) / rr;
    fx += fc * dx; fy += fc * dy; fz += fc * dz;
  }
  force[i] = make_float4(fx, fy, fz, 0.f);
}

// ---- force matching ------------------------------------------------------------------------
// Residual e_i = scale (F_i - F_ref,i) into resid (which holds F_ref on entry) and the loss sum
// |F_i - F_ref,i|^2 (times lossScale) into loss.
__global__ void k_diff_resid(int n, const float4 *__restrict__ force, float4 *__restrict__ resid, float scale,
                             double lossScale, double *__restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float s = 0.f;
  if (i < n) {
    const float4 f = force[i], ref = resid[i];
    const float ex = f.x - ref.x, ey = f.y - ref.y, ez = f.z - ref.z;
    s = ex * ex + ey * ey + ez * ez;
    resid[i] = make_float4(scale * ex, scale * ey, scale * ez, 0.f);
  }
  s = warpSumF(s);
  if ((threadIdx.x & 31) == 0 && s != 0.f) atomicAdd(loss, lossScale * (double)s);
}

// Adjoint of the force-matching loss over the metal atoms' pairs (every metal-metal pair from
// both sides, every metal-carbon pair from its metal side): dD/dtheta into grad (dL/dtheta is
// its negative).  First pass: rho_i and g_i recomputed; second pass: the gradient terms.
__global__ void __launch_bounds__(128) k_diff_adjoint(BlockTab tab, const RepConst *__restrict__ rc,
                                                      const float4 *__restrict__ pos,
                                                      const int *__restrict__ nn, const int *__restrict__ nbl,
                                                      int rowStride, const float *__restrict__ theta, Spline sp,
                                                      const float4 *__restrict__ resid, double *__restrict__ grad) {
  __shared__ float sT[kDP], sG[kDP];
  for (int q = threadIdx.x; q < kDP; q += blockDim.x) {
    sT[q] = theta[q];
    sG[q] = 0.f;
  }
  __syncthreads();
  const int rep = tab.rep[blockIdx.x];
  const RepConst &P = rc[rep];
  const int sub = threadIdx.x & (kMT - 1);
  const unsigned gmask = ((1u << kMT) - 1) << (threadIdx.x & 31 & ~(kMT - 1));
  const int i = tab.start[blockIdx.x] + threadIdx.x / kMT;
  const int metalEnd = P.atomOff + P.nMolMe;
  const bool valid = i < metalEnd;
  const float eps = sT[0], sig = sT[1];
  float4 A = make_float4(0.f, 0.f, 0.f, 0.f), Ei = A;
  const int *row = nbl + (size_t)i * rowStride;
  const int n = valid ? nn[i] : 0;
  float rho = 0.f, g = 0.f;
  if (valid) {
    A = pos[i];
    Ei = resid[i];
    for (int j = sub; j < n; j += kMT) {
      const int k = row[j];
      if (k >= metalEnd) continue;
      const float4 B = pos[k];
      const float dx = minImg(A.x - B.x, P.region[0]), dy = minImg(A.y - B.y, P.region[1]),
                  dz = minImg(A.z - B.z, P.region[2]);
      const float rr = dx * dx + dy * dy + dz * dz;
      if (rr >= P.rrCutEam) continue;
      const float r = sqrtf(rr);
      float b[4], db[4];
      const int kk = bspline(sp, r, b, db);
      const float4 Ek = resid[k];
      const float w = (dx * (Ei.x - Ek.x) + dy * (Ei.y - Ek.y) + dz * (Ei.z - Ek.z)) / r;
      rho += spl(sT + kDen, kk, b);
      g += spl(sT + kDen, kk, db) * w;
    }
  }
#pragma unroll
  for (int o = kMT / 2; o > 0; o >>= 1) {
    rho += __shfl_xor_sync(gmask, rho, o);
    g += __shfl_xor_sync(gmask, g, o);
  }
  if (valid) {
    float F, Fd, Fdd;
    embedAll(P, rho, F, Fd, Fdd);
    const float gF = Fdd * g;
    for (int j = sub; j < n; j += kMT) {
      const int k = row[j];
      const float4 B = pos[k];
      const float dx = minImg(A.x - B.x, P.region[0]), dy = minImg(A.y - B.y, P.region[1]),
                  dz = minImg(A.z - B.z, P.region[2]);
      const float rr = dx * dx + dy * dy + dz * dz;
      const float4 Ek = resid[k];
      const float de = dx * (Ei.x - Ek.x) + dy * (Ei.y - Ek.y) + dz * (Ei.z - Ek.z);
      if (k < metalEnd) {
        if (rr >= P.rrCutEam) continue;
        const float r = sqrtf(rr), w = de / r;
        float b[4], db[4];
        const int kk = bspline(sp, r, b, db);
#pragma unroll
        for (int m = 0; m < 4; m++) {
          atomicAdd(&sG[kPhi + kk + m], 0.5f * db[m] * w);
          atomicAdd(&sG[kDen + kk + m], gF * b[m] + Fd * db[m] * w);
        }
      } else {
        if (rr >= P.rrCutLJ) continue;
        const float r = sqrtf(rr), w = de / r;
        const float s2 = sig * sig / rr, s6 = s2 * s2 * s2, s12 = s6 * s6;
        atomicAdd(&sG[0], 24.f * (s6 - 2.f * s12) / r * w);                    // dU'/d eps
        atomicAdd(&sG[1], 144.f * eps * (s6 - 4.f * s12) / (r * sig) * w);     // dU'/d sigma
      }
    }
  }
  flushGrad(sG, grad);
}

}  // namespace sg

using namespace sg;

struct sg_diff {
  sg_ctx *ctx = nullptr;
  int nFrames = 0, n = 0;
  Spline sp{};
  float *theta = nullptr, *Fp = nullptr;
  float4 *force = nullptr, *resid = nullptr;
  double *energy = nullptr, *grad = nullptr, *loss = nullptr;
  sg_simparams p0{};
};

#define DCK(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return sg_fail(SG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// phi(r) and f(r) of the Zhou-Wadley-Johnson forms (SurfaceGrowth.cu:46-69) in FP64
static void eamAnalytic(const sg_simparams &p, double r, double &phi, double &f) {
  const double x = r * p.rei;
  const double eA = std::exp(-(double)p.alpha * (x - 1.0)), eB = std::exp(-(double)p.beta * (x - 1.0));
  const double dA = 1.0 + std::pow(x - p.kappa, 20.0), dB = 1.0 + std::pow(x - p.lambda, 20.0);
  phi = p.A * eA / dA - p.B * eB / dB;
  f = p.fe * eB / dB;
}

static Spline splineOf(const sg_simparams &p) {
  const double r0 = 0.6 / p.rei, rc = std::sqrt((double)p.rrCutEam);
  return Spline{(float)r0, (float)(kSI / (rc - r0))};
}

extern "C" int sg_diff_frame_params(const sg_simparams *in, sg_simparams *out) {
  if (!in || !out) return sg_fail(SG_ERR_INVALID, "sg_diff_frame_params: null argument");
  sg_simparams q = *in;
  const double rl = std::sqrt((double)std::max(q.rrCutEam, q.rrCutLJ));
  q.rrNebr = std::max(q.rrCutEam, q.rrCutLJ);
  q.cells.x = (int)(q.region.x / rl);
  q.cells.y = (int)(q.region.y / rl);
  q.cells.z = (int)(q.region.z / rl);
  if (q.cells.x < 3 || q.cells.y < 3 || q.cells.z < 3)
    return sg_fail(SG_ERR_INVALID, "box too small for the LJ cutoff (fewer than 3 cells in a direction)");
  q.invWidth = sg_float3{q.cells.x / q.region.x, q.cells.y / q.region.y, q.cells.z / q.region.z};
  q.gridSize = (unsigned)(q.cells.x * q.cells.y * q.cells.z);
  q.maxMol = (int)q.gridSize * (int)q.blockSize;
  q.iNebrMax = std::max(q.iNebrMax, 192);
  q.nebrNow = 1;
  *out = q;
  return SG_OK;
}

extern "C" int sg_diff_create(const sg_simparams *frames, int n, int device, sg_diff **out) {
  if (!frames || n < 1 || !out) return sg_fail(SG_ERR_INVALID, "sg_diff_create: bad arguments");
  *out = nullptr;
  std::vector<sg_simparams> q(n);
  for (int f = 0; f < n; f++) {
    if (frames[f].rei != frames[0].rei || frames[f].rrCutEam != frames[0].rrCutEam)
      return sg_fail(SG_ERR_INVALID, "sg_diff_create: frames must share the metal");
    if (int rc = sg_diff_frame_params(&frames[f], &q[f])) return rc;
  }
  sg_options o;
  sg_default_options(&o);
  o.use_graphs = 0;
  o.force_rebuild = 1;
  o.device = device;
  sg_ctx *c = nullptr;
  if (int rc = sg_create(q.data(), n, &o, &c)) return rc;
  sg_diff *d = new sg_diff;
  d->ctx = c;
  d->nFrames = n;
  d->n = sg_num_atoms(c, -1);
  d->sp = splineOf(q[0]);
  d->p0 = q[0];
  const size_t N = d->n;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&d->theta, sizeof(float) * kDP);
  if (e == cudaSuccess) e = cudaMalloc(&d->Fp, sizeof(float) * N);
  if (e == cudaSuccess) e = cudaMalloc(&d->force, sizeof(float4) * N);
  if (e == cudaSuccess) e = cudaMalloc(&d->resid, sizeof(float4) * N);
  if (e == cudaSuccess) e = cudaMalloc(&d->energy, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&d->grad, sizeof(double) * kDP);
  if (e == cudaSuccess) e = cudaMalloc(&d->loss, sizeof(double));
  if (e != cudaSuccess) {
    sg_diff_destroy(d);
    return sg_fail(SG_ERR_NOMEM, "sg_diff_create: %s", cudaGetErrorString(e));
  }
  *out = d;
  return SG_OK;
}

extern "C" int sg_diff_destroy(sg_diff *d) {
  if (!d) return SG_OK;
  cudaFree(d->theta); cudaFree(d->Fp); cudaFree(d->force); cudaFree(d->resid);
  cudaFree(d->energy); cudaFree(d->grad); cudaFree(d->loss);
  if (d->ctx) sg_destroy(d->ctx);
  delete d;
  return SG_OK;
}

extern "C" int sg_diff_num_atoms(const sg_diff *d) { return d ? d->n : 0; }

extern "C" int sg_diff_set_positions(sg_diff *d, const sg_float4 *r) {
  if (!d || !r) return sg_fail(SG_ERR_INVALID, "sg_diff_set_positions: null argument");
  if (int rc = sg_set_state(d->ctx, -1, r, nullptr, nullptr)) return rc;
  return sg_build_lists(d->ctx);
}

extern "C" int sg_diff_init_theta(const sg_simparams *pp, double *theta) {
  if (!pp || !theta) return sg_fail(SG_ERR_INVALID, "sg_diff_init_theta: null argument");
  const sg_simparams &p = *pp;
  theta[0] = p.epsLJ;
  theta[1] = p.sigmaLJ;
  // least squares on 40 points per interval, normal equations solved by Cholesky in FP64
  const Spline sp = splineOf(p);
  const double r0 = sp.r0, h = 1.0 / sp.invH;
  const int ns = 40 * kSI;
  std::vector<double> M(kSC * kSC, 0.0), rp(kSC, 0.0), rf(kSC, 0.0);
  for (int s = 0; s < ns; s++) {
    const double r = r0 + (s + 0.5) * (kSI * h) / ns;
    const double x = (r - r0) / h;
    const int k = std::max(0, std::min((int)std::floor(x), kSI - 1));
    const double t = x - k, u = 1.0 - t;
    const double b[4] = {u * u * u / 6, (3 * t * t * t - 6 * t * t + 4) / 6,
                         (-3 * t * t * t + 3 * t * t + 3 * t + 1) / 6, t * t * t / 6};
    double phi, f;
    eamAnalytic(p, r, phi, f);
    for (int a = 0; a < 4; a++) {
      rp[k + a] += b[a] * phi;
      rf[k + a] += b[a] * f;
      for (int c2 = 0; c2 < 4; c2++) M[(k + a) * kSC + k + c2] += b[a] * b[c2];
    }
  }
  for (int j = 0; j < kSC; j++) {  // Cholesky M = L L^T in place (lower triangle)
    for (int k = 0; k < j; k++) M[j * kSC + j] -= M[j * kSC + k] * M[j * kSC + k];
    M[j * kSC + j] = std::sqrt(M[j * kSC + j]);
    for (int i = j + 1; i < kSC; i++) {
      for (int k = 0; k < j; k++) M[i * kSC + j] -= M[i * kSC + k] * M[j * kSC + k];
      M[i * kSC + j] /= M[j * kSC + j];
    }
  }
  for (int which = 0; which < 2; which++) {
    std::vector<double> y = which == 0 ? rp : rf;
    for (int i = 0; i < kSC; i++) {
      for (int k = 0; k < i; k++) y[i] -= M[i * kSC + k] * y[k];
      y[i] /= M[i * kSC + i];
    }
    for (int i = kSC - 1; i >= 0; i--) {
      for (int k = i + 1; k < kSC; k++) y[i] -= M[k * kSC + i] * y[k];
      y[i] /= M[i * kSC + i];
    }
    for (int i = 0; i < kSC; i++) theta[(which == 0 ? kPhi : kDen) + i] = y[i];
  }
  return SG_OK;
}

static int uploadTheta(sg_diff *d, const double *theta) {
  float t[kDP];
  for (int q = 0; q < kDP; q++) t[q] = (float)theta[q];
  DCK(cudaMemcpyAsync(d->theta, t, sizeof t, cudaMemcpyHostToDevice, d->ctx->stream));
  return SG_OK;
}

// Forward pass: F'(rho), forces of all atoms, frame energies, optionally dE/dtheta.
static int forward(sg_diff *d, bool energyGrad) {
  sg_ctx *c = d->ctx;
  DCK(cudaMemsetAsync(d->energy, 0, sizeof(double) * d->nFrames, c->stream));
  DCK(cudaMemsetAsync(d->grad, 0, sizeof(double) * kDP, c->stream));
  DCK(cudaMemsetAsync(d->force, 0, sizeof(float4) * d->n, c->stream));
  if (c->metalTabT.n) {
    k_diff_rho<<<c->metalTabT.n, 128, 0, c->stream>>>(c->metalTabT.view(), c->rc, c->pos, c->nn, c->nbl,
                                                      c->rowStride, d->theta, d->sp, d->Fp, d->energy);
    k_diff_force_metal<<<c->metalTabT.n, 128, 0, c->stream>>>(c->metalTabT.view(), c->rc, c->pos, c->nn, c->nbl,
                                                              c->rowStride, d->theta, d->sp, d->Fp, d->force,
                                                              d->energy, energyGrad ? d->grad : nullptr);
  }
  if (c->carbonTab.n)
    k_diff_force_carbon<<<c->carbonTab.n, 128, 0, c->stream>>>(c->carbonTab.view(), c->rc, c->pos, c->nn,
                                                               c->nbl, c->rowStride, d->theta, d->force);
  DCK(cudaGetLastError());
  return SG_OK;
}

extern "C" int sg_diff_energy(sg_diff *d, const double *theta, double *energy, double *grad) {
  if (!d || !theta) return sg_fail(SG_ERR_INVALID, "sg_diff_energy: null argument");
  int rc;
  if ((rc = uploadTheta(d, theta)) || (rc = forward(d, grad != nullptr))) return rc;
  if (energy)
    DCK(cudaMemcpyAsync(energy, d->energy, sizeof(double) * d->nFrames, cudaMemcpyDeviceToHost, d->ctx->stream));
  if (grad) DCK(cudaMemcpyAsync(grad, d->grad, sizeof(double) * kDP, cudaMemcpyDeviceToHost, d->ctx->stream));
  DCK(cudaStreamSynchronize(d->ctx->stream));
  return SG_OK;
}

extern "C" int sg_diff_forces(sg_diff *d, const double *theta, float *forces) {
  if (!d || !theta || !forces) return sg_fail(SG_ERR_INVALID, "sg_diff_forces: null argument");
  int rc;
  if ((rc = uploadTheta(d, theta)) || (rc = forward(d, false))) return rc;
  sg_ctx *c = d->ctx;
  k_pack3<<<(d->n + 255) / 256, 256, 0, c->stream>>>(d->force, c->stage, d->n);
  DCK(cudaGetLastError());
  DCK(cudaMemcpyAsync(forces, c->stage, sizeof(float) * 3 * d->n, cudaMemcpyDeviceToHost, c->stream));
  DCK(cudaStreamSynchronize(c->stream));
  return SG_OK;
}

extern "C" int sg_diff_force_matching(sg_diff *d, const double *theta, const float *ref, double *loss,
                                      double *grad) {
  if (!d || !theta || !ref) return sg_fail(SG_ERR_INVALID, "sg_diff_force_matching: null argument");
  sg_ctx *c = d->ctx;
  int rc;
  if ((rc = uploadTheta(d, theta))) return rc;
  DCK(cudaMemcpyAsync(c->stage, ref, sizeof(float) * 3 * d->n, cudaMemcpyHostToDevice, c->stream));
  k_unpack3<<<(d->n + 255) / 256, 256, 0, c->stream>>>(c->stage, d->resid, d->n);
  DCK(cudaGetLastError());
  if ((rc = forward(d, false))) return rc;
  DCK(cudaMemsetAsync(d->loss, 0, sizeof(double), c->stream));
  const double inv3N = 1.0 / (3.0 * d->n);
  k_diff_resid<<<(d->n + 255) / 256, 256, 0, c->stream>>>(d->n, d->force, d->resid, (float)(2.0 * inv3N), inv3N,
                                                          d->loss);
  DCK(cudaGetLastError());
  if (grad) {
    DCK(cudaMemsetAsync(d->grad, 0, sizeof(double) * kDP, c->stream));
    if (c->metalTabT.n)
      k_diff_adjoint<<<c->metalTabT.n, 128, 0, c->stream>>>(c->metalTabT.view(), c->rc, c->pos, c->nn, c->nbl,
                                                            c->rowStride, d->theta, d->sp, d->resid, d->grad);
    DCK(cudaGetLastError());
    DCK(cudaMemcpyAsync(grad, d->grad, sizeof(double) * kDP, cudaMemcpyDeviceToHost, c->stream));
  }
  if (loss) DCK(cudaMemcpyAsync(loss, d->loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  DCK(cudaStreamSynchronize(c->stream));
  if (grad)
    for (int q = 0; q < kDP; q++) grad[q] = -grad[q];  // dL/dtheta = -dD/dtheta
  return SG_OK;
}
