// sg_oracle.cpp - TEST INFRASTRUCTURE: CPU restatement of the SurfaceGrowthConsole timestep.
// Used only as the checker (tests/, __graft_entry__.smoke(), bench.py cpu_baseline).  The
// product never links or calls this file.  See sg_oracle.h for what it restates and how it is
// pinned.  Built with -O2 -ffp-contract=off (no FMA contraction) and OpenMP over atoms.
//
// File:line citations refer to SurfaceGrowthConsole/SurfaceGrowth.cu (cu:),
// SurfaceGrowthConsole/SurfaceGrowth.cpp (cpp:) and SurfaceGrowthConsole/ComputeDefs.h (defs:).

#include "sg_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---- precision-dispatched math (host libm; CUDA's own implementations are not reproduced) --
inline float xexp(float x) { return expf(x); }
inline double xexp(double x) { return exp(x); }
inline float xpow(float x, float y) { return powf(x, y); }
inline double xpow(double x, double y) { return pow(x, y); }
inline float xlog(float x) { return logf(x); }
inline double xlog(double x) { return log(x); }
inline float xsqrt(float x) { return sqrtf(x); }
inline double xsqrt(double x) { return sqrt(x); }
inline float xacos(float x) { return acosf(x); }
inline double xacos(double x) { return acos(x); }

template <class R> struct V3 { R x, y, z; };
template <class R> struct V4 { R x, y, z, w; };

// The 27 cell offsets in the reference's visiting order (defs:221-231).
const int kOffsets[27][3] = {
    {0, 0, 0},  {0, 0, 1},  {0, 0, -1},  {0, 1, 0},  {0, 1, 1},  {0, 1, -1},  {0, -1, 0},
    {0, -1, 1}, {0, -1, -1}, {1, 0, 0},  {1, 0, 1},  {1, 0, -1}, {1, 1, 0},   {1, 1, 1},
    {1, 1, -1}, {1, -1, 0}, {1, -1, 1},  {1, -1, -1}, {-1, 0, 0}, {-1, 0, 1}, {-1, 0, -1},
    {-1, 1, 0}, {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 0}, {-1, -1, 1}, {-1, -1, -1}};

// Constants of the model in precision R.  Every constant is taken from the float parameter
// block (and float literals of the reference are kept as float values) so that the double
// instance evaluates the same model with less rounding.
template <class R> struct Model {
  R region[3], invWidth[3];
  int cells[3];
  R deltaT, rrNebr, rNebrShell;
  R rei, rhoei, rhoe, fe, alpha, beta, A, B, kappa, lambda, Fn[4], F[4], eta, Fe, massMe;
  R rrCutEam, rrCutC, mu_r, theta_0, mu_theta, mu_p, z_0;
  R sigmaLJ, epsLJ, rrCutLJ;
  R temperature, kB, gammaBerendsen;
  R rangeRdf, intervalRdf;
  R cos30;  // (float)cos(M_PI/6), as LeapfrogStepK computes it (cu:416)
  R xLeft, xRight, yBottom, yTop;
  void load(const sg_simparams &p) {
    region[0] = p.region.x; region[1] = p.region.y; region[2] = p.region.z;
    invWidth[0] = p.invWidth.x; invWidth[1] = p.invWidth.y; invWidth[2] = p.invWidth.z;
    cells[0] = p.cells.x; cells[1] = p.cells.y; cells[2] = p.cells.z;
    deltaT = p.deltaT; rrNebr = p.rrNebr; rNebrShell = p.rNebrShell;
    rei = p.rei; rhoei = p.rhoei; rhoe = p.rhoe; fe = p.fe; alpha = p.alpha; beta = p.beta;
    A = p.A; B = p.B; kappa = p.kappa; lambda = p.lambda;
    for (int i = 0; i < 4; i++) { Fn[i] = p.Fn[i]; F[i] = p.F[i]; }
    eta = p.eta; Fe = p.Fe; massMe = p.massMe; rrCutEam = p.rrCutEam; rrCutC = p.rrCutC;
    mu_r = p.mu_r; theta_0 = p.theta_0; mu_theta = p.mu_theta; mu_p = p.mu_p; z_0 = p.z_0;
    sigmaLJ = p.sigmaLJ; epsLJ = p.epsLJ; rrCutLJ = p.rrCutLJ;
    temperature = p.temperature; kB = p.kB; gammaBerendsen = p.gammaBerendsen;
    rangeRdf = p.rangeRdf; intervalRdf = p.intervalRdf;
    float c30 = (float)cos(M_PI / 6.f);
    cos30 = c30;
    // cu:418-421, evaluated in float as on the device
    xLeft = 0.5f * (c30 - p.region.x);
    xRight = 0.5f * (p.region.x - c30);
    yBottom = 0.5f * (1.f - p.region.y);
    yTop = 0.5f * (p.region.y - 1.f);
  }

  // ---- Zhou-Wadley-Johnson EAM (cu:46-210) --------------------------------------------
  R phi(R r) const {
    R x = r * rei;
    return A * xexp(-alpha * (x - R(1.f))) / (R(1.f) + xpow(x - kappa, R(20.f))) -
           B * xexp(-beta * (x - R(1.f))) / (R(1.f) + xpow(x - lambda, R(20.f)));
  }
  R f(R r) const {
    R x = r * rei;
    return fe * xexp(-beta * (x - R(1.f))) / (R(1.f) + xpow(x - lambda, R(20.f)));
  }
  R Fsmall(R rho) const {
    R rhoni = rhoei * R(1.176471f);
    R x = rho * rhoni - R(1.f);
    return Fn[0] + Fn[1] * x + Fn[2] * x * x + Fn[3] * x * x * x;
  }
  R Fmedium(R rho) const {
    R x = rho * rhoei - R(1.f);
    return F[0] + F[1] * x + F[2] * x * x + F[3] * x * x * x;
  }
  R Flarge(R rho) const {
    R x = rho * rhoei;
    return Fe * (R(1.f) - xlog(xpow(x, eta))) * xpow(x, eta);
  }
  R Femb(R rho) const {
    R rhon = R(0.85f) * rhoe;
    if (rho < rhon) return Fsmall(rho);
    R rhoo = R(1.15f) * rhoe;
    if ((rho >= rhon) && (rho < rhoo)) return Fmedium(rho);
    if (rho >= rhoo) return Flarge(rho);
    return R(0.f);
  }
  R dphi(R r) const {
    R x = r * rei;
    R dA = R(1.f) + xpow(x - kappa, R(20.f));
    R dB = R(1.f) + xpow(x - lambda, R(20.f));
    return (-A * xexp(-alpha * (x - R(1.f))) * (alpha + R(20.f) * xpow(x - kappa, R(19.f)) / dA) / dA +
            B * xexp(-beta * (x - R(1.f))) * (beta + R(20.f) * xpow(x - lambda, R(19.f)) / dB) / dB) *
           rei;
  }
  R df(R r) const {
    R x = r * rei;
    R dB = R(1.f) + xpow(x - lambda, R(20.f));
    return -fe * rei * xexp(-beta * (x - R(1.f))) *
           (beta + R(20.f) * xpow(x - lambda, R(19.f)) / dB) / dB;
  }
  R dFsmall(R rho) const {
    R rhoni = rhoei * R(1.176471f);
    R x = rho * rhoni - R(1.f);
    return rhoni * (Fn[1] + R(2.f) * Fn[2] * x + R(3.f) * Fn[3] * x * x);
  }
  R dFmedium(R rho) const {
    R y = rho * rhoei;
    return rhoei * (F[1] + R(2.f) * F[2] * (y - R(1.f)) + R(3.f) * F[3] * (y - R(1.f)) * (y - R(1.f)));
  }
  R dFlarge(R rho) const {
    R y = rho * rhoei;
    return -Fe * eta * rhoei * xpow(y, (eta - R(1.f))) * xlog(xpow(y, eta));
  }
  R dFemb(R rho) const {
    R rhon = R(0.85f) * rhoe;
    if (rho < rhon) return dFsmall(rho);
    R rhoo = R(1.15f) * rhoe;
    if ((rho >= rhon) && (rho < rhoo)) return dFmedium(rho);
    if (rho >= rhoo) return dFlarge(rho);
    return R(0.f);
  }

  // Minimum image as the force kernels do it (cu:750-759).
  void minImage(V3<R> &d) const {
    if (d.x >= R(0.5f) * region[0]) d.x -= region[0];
    else if (d.x < R(-0.5f) * region[0]) d.x += region[0];
    if (d.y >= R(0.5f) * region[1]) d.y -= region[1];
    else if (d.y < R(-0.5f) * region[1]) d.y += region[1];
    if (d.z >= R(0.5f) * region[2]) d.z -= region[2];
    else if (d.z < R(-0.5f) * region[2]) d.z += region[2];
  }
};

template <class R> inline R dot3(const V3<R> &a, const V3<R> &b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

// ---- reference reduction trees (cu:1101-1892) ---------------------------------------------
// Each block of 512 threads reduces 1024 consecutive elements with the stride-halving tree;
// the last block reduces the block partials in a 1024-slot array padded with zeros.
struct F3 { float x, y, z; };
enum class Op { Add, Max, Min };
inline void combine(F3 &a, const F3 &b, Op op) {
  switch (op) {
    case Op::Add: a.x = a.x + b.x; a.y = a.y + b.y; a.z = a.z + b.z; break;
    case Op::Max:
      if (a.x < b.x) a.x = b.x;
      if (a.y < b.y) a.y = b.y;
      if (a.z < b.z) a.z = b.z;
      break;
    case Op::Min:
      if (a.x > b.x) a.x = b.x;
      if (a.y > b.y) a.y = b.y;
      if (a.z > b.z) a.z = b.z;
      break;
  }
}
inline F3 tree1024(F3 *buf, Op op) {
  for (int s = 512; s >= 1; s >>= 1)
    for (int t = 0; t < s; t++) combine(buf[t], buf[t + s], op);
  return buf[0];
}
// elem(i) gives the (already masked) element value of index i < nElemGrid.
template <class G> F3 refReduce(int nMol, G elem, Op op) {
  int grid = (int)ceil((float)nMol / 1024);
  std::vector<F3> part(std::max(grid, 1));
  std::vector<F3> buf(1024);
  for (int b = 0; b < grid; b++) {
    for (int t = 0; t < 1024; t++) buf[t] = elem(1024 * b + t);
    part[b] = tree1024(buf.data(), op);
  }
  for (int t = 0; t < 1024; t++) buf[t] = (t < grid) ? part[t] : F3{0.f, 0.f, 0.f};
  return tree1024(buf.data(), op);
}

// ---- the simulation ------------------------------------------------------------------------
struct SimBase {
  virtual ~SimBase() {}
};

template <class R> struct Sim : SimBase {
  sg_simparams P;   // mutable fields are kept here exactly as the reference's hparams
  Model<R> M;
  int nMol, nMolMe, ncells, nebrMax;
  int forceRebuild;
  std::vector<V4<R>> r;
  std::vector<V3<R>> v, a;
  std::vector<int> cellOf, cellStart, cellAtoms, NN, NBL;
  std::vector<R> rho, dF, fric;
  std::vector<unsigned> hist;
  // diffusion (cu:2021-2032, h:189-196), FP32 as the reference
  struct TBuf { F3 orgR, rTrue; std::vector<float> rr; int count; };
  std::vector<TBuf> tbuf;
  std::vector<float> rrDiffuseAv;
  // last-step values
  F3 vSum{0, 0, 0}, cm{0, 0, 0}, cmv{0, 0, 0}, smin{0, 0, 0}, smax{0, 0, 0};
  float vvMax = 0, vvSum = 0, uSum = 0, frict = 0;
  double ke64 = 0, pe64 = 0;
  int rebuilds = 0;
  sg_diag diag;

  bool forceDiffusion = false;
  Sim(const sg_simparams &p, int frc, bool withDiffusion = false)
      : P(p), forceRebuild(frc), forceDiffusion(withDiffusion) {
    M.load(p);
    nMol = p.nMol;
    nMolMe = p.nMolMe;
    ncells = p.cells.x * p.cells.y * p.cells.z;
    nebrMax = p.iNebrMax;
    r.assign(nMol, V4<R>{0, 0, 0, 0});
    v.assign(nMol, V3<R>{0, 0, 0});
    a.assign(nMol, V3<R>{0, 0, 0});
    cellOf.assign(nMol, -1);
    cellStart.assign(ncells + 1, 0);
    cellAtoms.assign(nMol, -1);
    NN.assign(nMol, 0);
    NBL.assign((size_t)nMol * nebrMax, -1);
    rho.assign(std::max(nMolMe, 1), 0);
    dF.assign(std::max(nMolMe, 1), 0);
    fric.assign(std::max(nMolMe, 1), 0);
    hist.assign(std::max(p.sizeHistRdf, 1), 0);
    memset(&diag, 0, sizeof(diag));
    P.nebrNow = 1;  // no lists exist yet (a state resumed from a backup starts with a rebuild)
    if (P.iRegime == 2 || forceDiffusion) {
      tbuf.resize(P.nBuffDiffuse);
      for (int nb = 0; nb < P.nBuffDiffuse; nb++) {
        tbuf[nb].rr.assign(P.nValDiffuse, 0.f);
        tbuf[nb].count = -nb * P.nValDiffuse / P.nBuffDiffuse;  // cu:2870
      }
      rrDiffuseAv.assign(P.nValDiffuse, 0.f);
      P.countDiffuseAv = 0;
    }
  }

  bool isMetal(int k) const { return k < nMolMe; }

  // ---- Verlet (cu:397-434) and wrap (cu:436-453) ------------------------------------------
  bool frozen(int n) const {
    if (n < nMolMe) return false;
    return !((r[n].x != M.xLeft) && (r[n].x < M.xRight) && (r[n].y != M.yTop) && (r[n].y != M.yBottom));
  }
  void leapfrog(int part) {
    R h = R(0.5f) * M.deltaT;
#pragma omp parallel for schedule(static)
    for (int n = 0; n < nMol; n++) {
      if (frozen(n)) continue;
      v[n].x = v[n].x + h * a[n].x;
      v[n].y = v[n].y + h * a[n].y;
      v[n].z = v[n].z + h * a[n].z;
      if (part == 1) {
        r[n].x = r[n].x + M.deltaT * v[n].x;
        r[n].y = r[n].y + M.deltaT * v[n].y;
        r[n].z = r[n].z + M.deltaT * v[n].z;
      }
    }
  }
  void wrap() {
#pragma omp parallel for schedule(static)
    for (int n = 0; n < nMol; n++) {
      for (int c = 0; c < 3; c++) {
        R &x = (c == 0) ? r[n].x : (c == 1) ? r[n].y : r[n].z;
        if (x >= R(0.5f) * M.region[c]) x -= M.region[c];
        else if (x < R(-0.5f) * M.region[c]) x += M.region[c];
      }
    }
  }

  // ---- cell binning (cu:547-609): counting sort, ascending index within a cell -----------
  int cellIndex(const V4<R> &p) const {
    if (!std::isfinite((double)p.x) || !std::isfinite((double)p.y) || !std::isfinite((double)p.z)) return -1;
    int cx = (int)((p.x + R(0.5f) * M.region[0]) * M.invWidth[0]);
    int cy = (int)((p.y + R(0.5f) * M.region[1]) * M.invWidth[1]);
    int cz = (int)((p.z + R(0.5f) * M.region[2]) * M.invWidth[2]);
    long long c = ((long long)cz * M.cells[1] + cy) * M.cells[0] + cx;
    if (c < 0 || c >= ncells) return -1;  // never matches a block of the reference: not binned
    return (int)c;
  }
  void binAtoms() {
    std::vector<int> count(ncells, 0);
    int dropped = 0;
    for (int n = 0; n < nMol; n++) {
      int c = cellIndex(r[n]);
      cellOf[n] = c;
      if (c >= 0) count[c]++;
      else dropped++;
    }
    diag.cell_range += dropped;
    int s = 0, occ = 0;
    for (int c = 0; c < ncells; c++) {
      cellStart[c] = s;
      s += count[c];
      occ = std::max(occ, count[c]);
      if (count[c] > (int)P.blockSize) diag.cell_overflow++;
    }
    cellStart[ncells] = s;
    diag.max_cell_occupancy = std::max(diag.max_cell_occupancy, occ);
    std::vector<int> fill(cellStart.begin(), cellStart.end() - 1);
    for (int n = 0; n < nMol; n++)
      if (cellOf[n] >= 0) cellAtoms[fill[cellOf[n]]++] = n;
  }

  // Neighbour cell of cell c at stencil offset o with the periodic shift (cu:641-674).
  int stencilCell(int c, int o, V3<R> &shift) const {
    int ccz = c / (M.cells[0] * M.cells[1]);
    int ccy = (c - ccz * M.cells[0] * M.cells[1]) / M.cells[0];
    int ccx = c - (ccz * M.cells[1] + ccy) * M.cells[0];
    int mx = ccx + kOffsets[o][0], my = ccy + kOffsets[o][1], mz = ccz + kOffsets[o][2];
    shift = V3<R>{0, 0, 0};
    if (mx >= M.cells[0]) { mx = 0; shift.x = M.region[0]; }
    else if (mx < 0) { mx = M.cells[0] - 1; shift.x = -M.region[0]; }
    if (my >= M.cells[1]) { my = 0; shift.y = M.region[1]; }
    else if (my < 0) { my = M.cells[1] - 1; shift.y = -M.region[1]; }
    if (mz >= M.cells[2]) { mz = 0; shift.z = M.region[2]; }
    else if (mz < 0) { mz = M.cells[2] - 1; shift.z = -M.region[2]; }
    return (mz * M.cells[1] + my) * M.cells[0] + mx;
  }

  // ---- neighbour list (cu:612-711) ---------------------------------------------------------
  void buildNebr() {
    int maxnn = 0, over = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(max : maxnn) reduction(+ : over)
    for (int i = 0; i < nMol; i++) {
      for (int j = 0; j < nebrMax; j++) NBL[(size_t)j * nMol + i] = -1;
      int c = cellOf[i];
      int nn = 0, want = 0;
      if (c >= 0) {
        const V4<R> A = r[i];
        for (int o = 0; o < 27; o++) {
          V3<R> sh;
          int C = stencilCell(c, o, sh);
          for (int q = cellStart[C]; q < cellStart[C + 1]; q++) {
            int k = cellAtoms[q];
            const V4<R> &Bk = r[k];
            V3<R> d{A.x - Bk.x, A.y - Bk.y, A.z - Bk.z};
            d.x = d.x - sh.x; d.y = d.y - sh.y; d.z = d.z - sh.z;
            R rr = d.x * d.x + d.y * d.y + d.z * d.z;
            if ((rr < M.rrNebr) && (i != k)) {
              if (nn < nebrMax) NBL[(size_t)nn * nMol + i] = k;
              else over++;
              nn++;
              want++;
            }
          }
        }
      }
      maxnn = std::max(maxnn, want);
      NN[i] = std::min(nn, nebrMax);
    }
    diag.max_neighbours = std::max(diag.max_neighbours, maxnn);
    diag.nebr_overflow += over;
  }

  // ---- EAM density (cu:716-773), plus F(rho) and F'(rho) per metal atom --------------------
  void computeRho() {
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < nMolMe; i++) {
      const V4<R> A = r[i];
      R sum = 0;
      for (int j = 0; j < NN[i]; j++) {
        int k = NBL[(size_t)j * nMol + i];
        V3<R> d{A.x - r[k].x, A.y - r[k].y, A.z - r[k].z};
        M.minImage(d);
        R rr = d.x * d.x + d.y * d.y + d.z * d.z;
        if ((rr < M.rrCutEam) && isMetal(k)) sum += M.f(xsqrt(rr));
      }
      rho[i] = sum;
      dF[i] = M.dFemb(sum);
    }
  }

  // ---- forces (cu:776-1091) ------------------------------------------------------------
  void ljTerms(R rr, R &fc, R &u) const {
    R s2 = M.sigmaLJ * M.sigmaLJ;
    R rri = s2 / rr;
    R rri3 = rri * rri * rri;
    fc = R(48.f) * M.epsLJ * rri3 * (rri3 - R(0.5f)) * rri / (M.sigmaLJ * M.sigmaLJ);
    u = R(4.f) * M.epsLJ * rri3 * (rri3 - R(1.f));
  }
  static void addScaled(V3<R> &s, R c, const V3<R> &d) {
    s.x = s.x + c * d.x;
    s.y = s.y + c * d.y;
    s.z = s.z + c * d.z;
  }
  static void addZ(V3<R> &s, R fz) {
    s.x = s.x + R(0.f);
    s.y = s.y + R(0.f);
    s.z = s.z + fz;
  }
  void forceMetal(int i) {
    const V4<R> A = r[i];
    V3<R> fs{0, 0, 0}, fr{0, 0, 0};
    R uSumL = 0;
    R dFi = dF[i];
    for (int j = 0; j < NN[i]; j++) {
      int k = NBL[(size_t)j * nMol + i];
      V3<R> d{A.x - r[k].x, A.y - r[k].y, A.z - r[k].z};
      M.minImage(d);
      R rr = d.x * d.x + d.y * d.y + d.z * d.z;
      if (isMetal(k)) {
        if (rr >= M.rrCutEam) continue;  // the reference zeroes the term (cu:870, 876)
        R rd = xsqrt(rr);
        R fc = -M.dphi(rd);
        R u = M.phi(rd);
        fc = fc - M.df(rd) * (dFi + dF[k]);
        fc = fc / rd;
        addScaled(fs, fc, d);
        uSumL += u;
      } else {
        if (rr >= M.rrCutLJ) continue;  // cu:887-889
        R fc, u;
        ljTerms(rr, fc, u);
        uSumL += u;
        addScaled(fs, fc, d);
        addScaled(fr, fc, d);
      }
    }
    a[i] = V3<R>{fs.x / M.massMe, fs.y / M.massMe, fs.z / M.massMe};
    r[i].w = R(0.5f) * uSumL + M.Femb(rho[i]);
    fric[i] = fr.x;
  }
  void forceCarbon(int i) {
    const V4<R> A = r[i];
    V3<R> fs{0, 0, 0};
    R uSumL = 0;
    V3<R> rnn[3];
    R absR[3], dz[3];
    int counti = 0;
    const int nNeigh = NN[i];
    for (int j = 0; j < nNeigh; j++) {
      int k = NBL[(size_t)j * nMol + i];
      const V4<R> Bk = r[k];
      V3<R> d{A.x - Bk.x, A.y - Bk.y, A.z - Bk.z};
      M.minImage(d);
      R rr = d.x * d.x + d.y * d.y + d.z * d.z;
      if (isMetal(k)) {  // LJ from the carbon side (cu:900-917)
        if (rr >= M.rrCutLJ) continue;
        R fc, u;
        ljTerms(rr, fc, u);
        uSumL += u;
        addScaled(fs, fc, d);
        continue;
      }
      // carbon-carbon (cu:918-1062)
      if ((rr < M.rrCutC) && (counti < 3)) {
        absR[counti] = xsqrt(rr);
        dz[counti] = Bk.z - M.z_0;
        rnn[counti] = d;
        int countk = 0;
        for (int l = 0; l < NN[k]; l++) {
          int m = NBL[(size_t)l * nMol + k];
          const V4<R> rm = r[m];
          V3<R> e{Bk.x - rm.x, Bk.y - rm.y, Bk.z - rm.z};
          M.minImage(e);
          R rr2 = e.x * e.x + e.y * e.y + e.z * e.z;
          if ((rr2 < M.rrCutC) && (m != i)) {
            e.x = e.x * R(-1.f); e.y = e.y * R(-1.f); e.z = e.z * R(-1.f);
            R cs = dot3(rnn[counti], e) / (absR[counti] * rr2);
            R th = xacos(cs);
            R dth = th - M.theta_0;
            R tmp = M.mu_theta * dth / xsqrt(R(1.f) - cs * cs);
            R fc = tmp / (absR[counti] * rr2);
            addScaled(fs, fc, e);
            fc = -tmp * cs / (absR[counti] * absR[counti]);
            addScaled(fs, fc, rnn[counti]);
            fc = -M.mu_p * (rm.z - M.z_0) / R(9.f);
            addZ(fs, fc);
            ++countk;
          }
          if (countk == 2) break;
        }
        ++counti;
      }
      if (counti == 3) {
        for (int q = 0; q < 3; q++) {
          R fc = -M.mu_r * (absR[q] - R(1.f)) / absR[q];
          addScaled(fs, fc, rnn[q]);
          uSumL += M.mu_r * (absR[q] - R(1.f)) * (absR[q] - R(1.f));
        }
        R dZ = R(2.f) * (A.z - M.z_0) - (dz[0] + dz[1] + dz[2]);
        addZ(fs, R(-0.666666667f) * M.mu_p * dZ);
        dZ = (A.z - M.z_0) - R(0.33333333f) * (dz[0] + dz[1] + dz[2]);
        uSumL += M.mu_p * dZ * dZ;
        const int pa[3][2] = {{0, 1}, {1, 2}, {2, 0}};
        for (int q = 0; q < 3; q++) {
          int p0 = pa[q][0], p1 = pa[q][1];
          R cs = dot3(rnn[p0], rnn[p1]) / (absR[p0] * absR[p1]);
          R th = xacos(cs);
          R dth = th - M.theta_0;
          R tmp = M.mu_theta * dth / xsqrt(R(1.f) - cs * cs);
          R fc = tmp * (R(1.f) - absR[p0] * cs / absR[p1]) / (absR[p0] * absR[p1]);
          addScaled(fs, fc, rnn[p1]);
          fc = tmp * (R(1.f) - absR[p1] * cs / absR[p0]) / (absR[p0] * absR[p1]);
          addScaled(fs, fc, rnn[p0]);
          uSumL += M.mu_theta * dth * dth;
        }
        // The reference reuses its neighbour-loop counter for the radial loop above
        // (cu:989), so the walk resumes at list entry 4 after the bonded terms.
        j = 3;
        counti = 4;
      }
    }
    a[i] = fs;
    r[i].w = R(0.5f) * uSumL;
  }
  void computeForces() {
    if (nMolMe != 0) computeRho();
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < nMol; i++) {
      if (isMetal(i)) forceMetal(i);
      else forceCarbon(i);
    }
  }

  // ---- RDF sample (cu:1895-1999) -----------------------------------------------------------
  void evalRdf() {
    const R range2 = M.rangeRdf * M.rangeRdf;
    const int nb = P.sizeHistRdf;
    int dropped = 0;
    std::vector<unsigned> h(nb, 0);
#pragma omp parallel
    {
      std::vector<unsigned> hl(nb, 0);
      int dl = 0;
#pragma omp for schedule(dynamic, 64)
      for (int i = 0; i < nMolMe; i++) {
        int c = cellOf[i];
        if (c < 0) continue;
        const V4<R> A = r[i];
        for (int o = 0; o < 27; o++) {
          V3<R> sh;
          int C = stencilCell(c, o, sh);
          for (int q = cellStart[C]; q < cellStart[C + 1]; q++) {
            int k = cellAtoms[q];
            V3<R> d{A.x - r[k].x, A.y - r[k].y, A.z - r[k].z};
            d.x = d.x - sh.x; d.y = d.y - sh.y; d.z = d.z - sh.z;
            R rr = d.x * d.x + d.y * d.y + d.z * d.z;
            if ((rr < range2) && (i != k) && isMetal(k)) {
              int bin = (int)(xsqrt(rr) * M.intervalRdf);
              if (bin >= 0 && bin < nb) hl[bin]++;
              else dl++;
            }
          }
        }
      }
#pragma omp critical
      {
        for (int b = 0; b < nb; b++) h[b] += hl[b];
        dropped += dl;
      }
    }
    for (int b = 0; b < nb; b++) hist[b] += h[b];
    diag.rdf_range += dropped;
  }

  // ---- diffusion of the metal centre of mass (cu:2865-2952) ---------------------------------
  static int nint(float x) { return (x < 0.) ? (-(int)(0.5 - (x))) : ((int)(0.5 + (x))); }
  void evalDiffusion(F3 c) {
    for (int nb = 0; nb < P.nBuffDiffuse; nb++) {
      TBuf &b = tbuf[nb];
      if (b.count == 0) { b.orgR = c; b.rTrue = c; }
      if (b.count >= 0) {
        int ni = b.count;
        b.rr[ni] = 0.f;
        F3 d{b.rTrue.x - c.x, b.rTrue.y - c.y, b.rTrue.z - c.z};
        d.x = d.x / P.region.x; d.y = d.y / P.region.y; d.z = d.z / P.region.z;
        d.x = (float)nint(d.x); d.y = (float)nint(d.y); d.z = (float)nint(d.z);
        d.x = d.x * P.region.x; d.y = d.y * P.region.y; d.z = d.z * P.region.z;
        b.rTrue = F3{c.x + d.x, c.y + d.y, c.z + d.z};
        d = F3{b.rTrue.x - b.orgR.x, b.rTrue.y - b.orgR.y, b.rTrue.z - b.orgR.z};
        b.rr[ni] += d.x * d.x + d.y * d.y + d.z * d.z;
      }
      ++b.count;
    }
    // AccumDiffusion (cu:2898-2920); the printed table is handled by the writers.
    for (int nb = 0; nb < P.nBuffDiffuse; nb++) {
      TBuf &b = tbuf[nb];
      if (b.count == P.nValDiffuse) {
        for (int j = 0; j < P.nValDiffuse; j++) rrDiffuseAv[j] += b.rr[j];
        b.count = 0;
        ++P.countDiffuseAv;
        if (P.countDiffuseAv == P.limitDiffuseAv) {
          float fac = 1. / (3 * 2 * P.stepDiffuse * P.deltaT * P.limitDiffuseAv);
          for (int j = 1; j < P.nValDiffuse; j++) rrDiffuseAv[j] *= fac / j;
          lastDiffusePrint = rrDiffuseAv;
          diffuseTables.push_back(rrDiffuseAv);
          diffusePrints++;
          P.countDiffuseAv = 0;
          std::fill(rrDiffuseAv.begin(), rrDiffuseAv.end(), 0.f);
        }
      }
    }
  }
  std::vector<float> lastDiffusePrint;
  std::vector<std::vector<float>> diffuseTables;  // every printed table, in order
  int diffusePrints = 0;

  // ---- property accumulators (cu:2659-2686) -------------------------------------------------
  static void propZero(sg_prop &p) { p.sum = p.sum2 = 0.f; }
  static void propAccum(sg_prop &p) { p.sum += p.val; p.sum2 += p.val * p.val; }

  // ---- reductions of the step ----------------------------------------------------------------
  F3 elemF(int what, int i, float cmVelX) const {
    F3 z{0.f, 0.f, 0.f};
    switch (what) {
      case 0: {
        if (i >= nMol) return z;
        F3 e{(float)v[i].x, (float)v[i].y, (float)v[i].z};
        if (i < nMolMe) e.x = (float)M.massMe * e.x;
        return e;
      }
      case 1: {
        if (i >= nMol) return z;
        F3 e{(float)v[i].x, (float)v[i].y, (float)v[i].z};
        e.x = e.x * e.x + e.y * e.y + e.z * e.z;
        return e;
      }
      case 2: {
        if (i >= nMol) return z;
        F3 e{(float)v[i].x, (float)v[i].y, (float)v[i].z};
        if (P.iRegime == 2 && i < nMolMe) e.x = e.x - cmVelX;
        e.x = e.x * e.x + e.y * e.y + e.z * e.z;
        if (i < nMolMe) e.x = (float)M.massMe * e.x;
        return e;
      }
      case 3:
        if (i >= nMol) return z;
        return F3{(float)r[i].w, 0.f, 0.f};
      case 4: case 6: case 7:
        if (i >= nMolMe) return z;
        return F3{(float)r[i].x, (float)r[i].y, (float)r[i].z};
      case 5:
        if (i >= nMolMe) return z;
        return F3{(float)v[i].x, (float)v[i].y, (float)v[i].z};
      case 8:
        if (i >= nMolMe) return z;
        return F3{(float)fric[i], 0.f, 0.f};
    }
    return z;
  }
  F3 reduceF(int what, float cmVelX) const {
    Op op = (what == 1 || what == 7) ? Op::Max : (what == 6) ? Op::Min : Op::Add;
    return refReduce(nMol, [&](int i) { return elemF(what, i, cmVelX); }, op);
  }
  // FP64 instance: plain FP64 sums (the tree order matters only for FP32 parity).
  F3 reduceD(int what, double cmVelX, double *s64) const {
    double s[3] = {0, 0, 0};
    bool isMax = (what == 1 || what == 7), isMin = (what == 6);
    int lim = (what >= 4) ? nMolMe : nMol;
    if (isMax || isMin) {
      // the reference's min/max see the zero padding of its grid (cu:1669-1682)
      for (int c = 0; c < 3; c++) s[c] = 0.0;
    }
    for (int i = 0; i < lim; i++) {
      double e[3];
      switch (what) {
        case 0: e[0] = (double)v[i].x * (i < nMolMe ? (double)M.massMe : 1.0); e[1] = v[i].y; e[2] = v[i].z; break;
        case 1: e[0] = (double)v[i].x * v[i].x + (double)v[i].y * v[i].y + (double)v[i].z * v[i].z; e[1] = e[2] = 0; break;
        case 2: {
          double vx = v[i].x;
          if (P.iRegime == 2 && i < nMolMe) vx -= cmVelX;
          e[0] = vx * vx + (double)v[i].y * v[i].y + (double)v[i].z * v[i].z;
          if (i < nMolMe) e[0] *= (double)M.massMe;
          e[1] = e[2] = 0;
          break;
        }
        case 3: e[0] = r[i].w; e[1] = e[2] = 0; break;
        case 4: case 6: case 7: e[0] = r[i].x; e[1] = r[i].y; e[2] = r[i].z; break;
        case 5: e[0] = v[i].x; e[1] = v[i].y; e[2] = v[i].z; break;
        default: e[0] = fric[i]; e[1] = e[2] = 0; break;
      }
      for (int c = 0; c < 3; c++) {
        if (isMax) s[c] = std::max(s[c], e[c]);
        else if (isMin) s[c] = std::min(s[c], e[c]);
        else s[c] += e[c];
      }
    }
    if (s64) { s64[0] = s[0]; s64[1] = s[1]; s64[2] = s[2]; }
    return F3{(float)s[0], (float)s[1], (float)s[2]};
  }
  F3 reduce(int what, float cmVelX, double *s64 = nullptr) const {
    if (sizeof(R) == sizeof(float)) {
      F3 o = reduceF(what, cmVelX);
      if (s64) { s64[0] = o.x; s64[1] = o.y; s64[2] = o.z; }
      return o;
    }
    return reduceD(what, cmVelX, s64);
  }

  // ---- thermostat (cu:455-485) ---------------------------------------------------------------
  void thermostat(float vvSumF, double vvSum64) {
    int step = P.stepCount;
    R kin = (sizeof(R) == sizeof(float)) ? R(vvSumF) * R(0.5f) / R(nMol) : R(vvSum64) * R(0.5f) / R(nMol);
    R betaC = xsqrt(R(1.f) + M.gammaBerendsen * (M.temperature * R(1.5f) * M.kB / kin - R(1.f)));
    R betaM = xsqrt(R(1.f) + M.gammaBerendsen * (M.temperature * M.kB / kin - R(1.f)));
    bool metalOn = (P.iRegime == 2) && (step > P.stepEquil) && (step < P.stepEquil + P.stepCool);
    for (int n = 0; n < nMol; n++) {
      if (n >= nMolMe) { v[n].x = betaC * v[n].x; v[n].y = betaC * v[n].y; v[n].z = betaC * v[n].z; }
      else if (metalOn) { v[n].x = betaM * v[n].x; v[n].y = betaM * v[n].y; v[n].z = betaM * v[n].z; }
    }
  }

  // ---- deposition (cu:488-514, schedule cu:2148-2168) -----------------------------------
  void insertAtoms(int nDep, int nToDep) {
    R z = R(0.49f) * M.region[2];
    for (int n = 0; n < nMolMe; n++) {
      if (n >= nDep && n < nDep + nToDep) { r[n].z = z; v[n].z = -R(P.velMagDepos); }
      if (n >= nDep + nToDep) {
        r[n].z = R(1.5f) * M.region[2] + R(0.5f) * R(n + 1) * M.region[2];
        v[n] = V3<R>{0, 0, 0};
      }
    }
  }

  // ---- one step (cu:2141-2489 without file output) -------------------------------------
  int step() {
    ++P.stepCount;
    const int sc = P.stepCount;
    if (P.iRegime == 1) {
      if (sc <= P.stepEquil) insertAtoms(P.nMolDeposited, 0);
      else if (P.nMolDeposited < nMolMe) {
        int nTo = ((sc - P.stepEquil) % P.stepDeposit == 0) ? P.nMolToDeposit : 0;
        insertAtoms(P.nMolDeposited, nTo);
        P.nMolDeposited += nTo;
      }
    }
    leapfrog(1);
    wrap();
    if (forceRebuild) P.nebrNow = 1;
    if (P.nebrNow) {
      P.nebrNow = 0;
      P.dispHi = 0.f;
      binAtoms();
      buildNebr();
      rebuilds++;
    }
    computeForces();
    bool hasFric = (P.iRegime != 0) && (nMolMe != 0);
    frict = hasFric ? reduce(8, 0.f).x : 0.f;
    leapfrog(2);
    if (nMolMe != 0) {
      cm = reduce(4, 0.f);
      cmv = reduce(5, 0.f);
      smin = reduce(6, 0.f);
      smax = reduce(7, 0.f);
      F3 ps{smax.x - smin.x, smax.y - smin.y, smax.z - smin.z};
      P.centerOfMass.val = cm.x / nMolMe;
      P.cmVel.val = cmv.x / nMolMe;
      P.frictForce.val = frict;
      P.particleSize = sg_float3{ps.x, ps.y, ps.z};
      if (P.iRegime == 2 && sc > P.stepEquil && ((sc - P.stepEquil) % P.stepDiffuse == 0)) {
        F3 c{cm.x / nMolMe, cm.y / nMolMe, cm.z / nMolMe};
        evalDiffusion(c);
      }
    } else {
      P.centerOfMass.val = 0.f; P.cmVel.val = 0.f; P.frictForce.val = 0.f;
      P.particleSize = sg_float3{0.f, 0.f, 0.f};
    }
    vSum = reduce(0, 0.f);
    vvMax = reduce(1, 0.f).x;
    double vv64[3];
    vvSum = reduce(2, P.cmVel.val, vv64).x;
    bool thermo = ((P.iRegime == 2) && (sc > P.stepEquil) && (sc % P.stepThermostat == 0)) ||
                  ((P.iRegime == 1) && (sc % P.stepThermostat == 0));
    if (thermo) thermostat(vvSum, vv64[0]);
    double pe[3];
    uSum = reduce(3, 0.f, pe).x;
    P.dispHi += sqrtf(vvMax) * P.deltaT;
    if (P.dispHi > 0.5f * P.rNebrShell) P.nebrNow = 1;
    P.kinEnergy.val = 0.5f * vvSum / nMol;
    P.potEnergy.val = uSum / nMol;
    P.totEnergy.val = P.kinEnergy.val + P.potEnergy.val;
    ke64 = 0.5 * vv64[0] / nMol;
    pe64 = pe[0] / nMol;
    P.vSum = sg_float3{vSum.x, vSum.y, vSum.z};
    if (P.iRegime == 2 && nMolMe != 0 && sc > P.stepEquil + P.stepCool) {
      if (P.cmVel.val < 0.005f) P.shear += P.deltaF;
      unsigned cnt = 0;
      for (int n = 0; n < nMolMe; n++) {
        float dR = P.centerOfMass.val - (float)r[n].x;
        if (dR > 0.f) { a[n].x += R(P.shear); cnt++; }
      }
      P.totalShear = cnt * P.shear;
    }
    if (P.bRdf && (sc % P.stepRdf == 0)) {
      if (P.countRdf == 0) std::fill(hist.begin(), hist.end(), 0u);
      evalRdf();
      ++P.countRdf;
      if (P.countRdf == P.limitRdf) {
        lastRdfPrint = hist;
        rdfPrints++;
        P.countRdf = 0;
      }
    }
    P.oneStep.val = 0.f;
    propAccum(P.totEnergy); propAccum(P.potEnergy); propAccum(P.kinEnergy); propAccum(P.oneStep);
    propAccum(P.centerOfMass); propAccum(P.cmVel); propAccum(P.frictForce);
    if (sc % P.stepAvg == 0) {
      lastAvg[0] = P.totEnergy; lastAvg[1] = P.potEnergy; lastAvg[2] = P.kinEnergy;
      // the seven accumulators as PrintSummary receives them (before AccumProps(0))
      lastAvg7[0] = P.totEnergy; lastAvg7[1] = P.potEnergy; lastAvg7[2] = P.kinEnergy; lastAvg7[3] = P.oneStep;
      lastAvg7[4] = P.centerOfMass; lastAvg7[5] = P.cmVel; lastAvg7[6] = P.frictForce;
      propZero(P.totEnergy); propZero(P.potEnergy); propZero(P.kinEnergy); propZero(P.oneStep);
      propZero(P.centerOfMass); propZero(P.cmVel); propZero(P.frictForce);
    }
    if (sc >= P.stepLimit) P.moreCycles = 0;
    return 0;
  }
  std::vector<unsigned> lastRdfPrint;
  int rdfPrints = 0;
  sg_prop lastAvg[3];
  sg_prop lastAvg7[7];
};

struct Handle {
  int prec;
  Sim<float> *f = nullptr;
  Sim<double> *d = nullptr;
};

template <class R> void setState(Sim<R> &s, const sg_float4 *r, const sg_float3 *v, const sg_float3 *a) {
  for (int i = 0; i < s.nMol; i++) {
    if (r) s.r[i] = V4<R>{r[i].x, r[i].y, r[i].z, r[i].w};
    if (v) s.v[i] = V3<R>{v[i].x, v[i].y, v[i].z};
    if (a) s.a[i] = V3<R>{a[i].x, a[i].y, a[i].z};
  }
}
template <class R> void getState(Sim<R> &s, sg_float4 *r, sg_float3 *v, sg_float3 *a) {
  for (int i = 0; i < s.nMol; i++) {
    if (r) r[i] = sg_float4{(float)s.r[i].x, (float)s.r[i].y, (float)s.r[i].z, (float)s.r[i].w};
    if (v) v[i] = sg_float3{(float)s.v[i].x, (float)s.v[i].y, (float)s.v[i].z};
    if (a) a[i] = sg_float3{(float)s.a[i].x, (float)s.a[i].y, (float)s.a[i].z};
  }
}
template <class R> void getThermo(Sim<R> &s, sg_thermo *t) {
  memset(t, 0, sizeof(*t));
  t->stepCount = s.P.stepCount;
  t->nebrNow = s.P.nebrNow;
  t->rebuilds = s.rebuilds;
  t->countRdf = s.P.countRdf;
  t->kinEnergy = s.P.kinEnergy.val;
  t->potEnergy = s.P.potEnergy.val;
  t->totEnergy = s.P.totEnergy.val;
  t->vvSum = s.vvSum; t->vvMax = s.vvMax; t->uSum = s.uSum; t->dispHi = s.P.dispHi;
  t->vSum = sg_float3{s.vSum.x, s.vSum.y, s.vSum.z};
  t->centerOfMass = sg_float3{s.cm.x, s.cm.y, s.cm.z};
  t->cmVel = sg_float3{s.cmv.x, s.cmv.y, s.cmv.z};
  t->frictForce = s.frict;
  t->particleSize = s.P.particleSize;
  t->shear = s.P.shear; t->totalShear = s.P.totalShear;
  t->kinEnergy64 = s.ke64; t->potEnergy64 = s.pe64;
  t->props[0] = s.P.totEnergy; t->props[1] = s.P.potEnergy; t->props[2] = s.P.kinEnergy;
  t->props[3] = s.P.oneStep; t->props[4] = s.P.centerOfMass; t->props[5] = s.P.cmVel;
  t->props[6] = s.P.frictForce;
}

template <class R> void getState64(Sim<R> &s, double *r4, double *v3, double *a3) {
  for (int i = 0; i < s.nMol; i++) {
    if (r4) { r4[4 * i] = s.r[i].x; r4[4 * i + 1] = s.r[i].y; r4[4 * i + 2] = s.r[i].z; r4[4 * i + 3] = s.r[i].w; }
    if (v3) { v3[3 * i] = s.v[i].x; v3[3 * i + 1] = s.v[i].y; v3[3 * i + 2] = s.v[i].z; }
    if (a3) { a3[3 * i] = s.a[i].x; a3[3 * i + 1] = s.a[i].y; a3[3 * i + 2] = s.a[i].z; }
  }
}
// Mean position of the metal atoms in FP64 (wrapped positions, as the reference's
// centerOfMass; SurfaceGrowth.cu:1706-1760 sums them in its reduction tree).
template <class R> void metalCm64(const Sim<R> &s, double *cm) {
  double x = 0, y = 0, z = 0;
  for (int i = 0; i < s.P.nMolMe; i++) { x += s.r[i].x; y += s.r[i].y; z += s.r[i].z; }
  const double inv = s.P.nMolMe ? 1.0 / s.P.nMolMe : 0.0;
  cm[0] = x * inv; cm[1] = y * inv; cm[2] = z * inv;
}
template <class R> void setState64(Sim<R> &s, const double *r4, const double *v3, const double *a3) {
  for (int i = 0; i < s.nMol; i++) {
    if (r4) s.r[i] = V4<R>{(R)r4[4 * i], (R)r4[4 * i + 1], (R)r4[4 * i + 2], (R)r4[4 * i + 3]};
    if (v3) s.v[i] = V3<R>{(R)v3[3 * i], (R)v3[3 * i + 1], (R)v3[3 * i + 2]};
    if (a3) s.a[i] = V3<R>{(R)a3[3 * i], (R)a3[3 * i + 1], (R)a3[3 * i + 2]};
  }
}
template <class R> void getCells(Sim<R> &S, int *co, int *cs, int *ca) {
  if (co) std::copy(S.cellOf.begin(), S.cellOf.end(), co);
  if (cs) std::copy(S.cellStart.begin(), S.cellStart.end(), cs);
  if (ca) std::copy(S.cellAtoms.begin(), S.cellAtoms.end(), ca);
}
template <class R> void getNebr(Sim<R> &S, int *nn, int *nbl) {
  if (nn) std::copy(S.NN.begin(), S.NN.end(), nn);
  if (nbl) std::copy(S.NBL.begin(), S.NBL.end(), nbl);
}
template <class R> void getVec(const std::vector<R> &v, int n, float *out) {
  for (int i = 0; i < n; i++) out[i] = (float)v[i];
}
template <class R> void getDiff(Sim<R> &S, float *rr, int *counts, int *cav) {
  if (rr) std::copy(S.rrDiffuseAv.begin(), S.rrDiffuseAv.end(), rr);
  if (counts)
    for (size_t i = 0; i < S.tbuf.size(); i++) counts[i] = S.tbuf[i].count;
  if (cav) *cav = S.P.countDiffuseAv;
}

}  // namespace

struct orc_sim { Handle h; };

#define DISPATCH(s, call) ((s)->h.prec == 32 ? (s)->h.f->call : (s)->h.d->call)

// ---- differentiation form in FP64 ----------------------------------------------------------
// TEST INFRASTRUCTURE: the model of surfacegrowthconsole_gb300/csrc/sg_adjoint.cu restated in
// FP64 (energies, forces, force-matching loss, and the gradients of both by the same adjoint
// formulas), for the GPU checks and for checking the formulas against central finite
// differences.  Pair lists come from the FP32 list code on the same frame parameters, so they
// are the lists the GPU builds; every pair term is then evaluated in FP64.
namespace diff {
constexpr int NP = 66, SC = 32, SI = 29, PHI = 2, DEN = 34;

struct Frame {
  sg_simparams p;
  Model<double> M;
  int n, nMe;
  std::vector<int> NN, NBL;
  std::vector<V4<double>> r;
  double r0, h;
};

static int bsp(const Frame &f, double r, double b[4], double db[4]) {
  const double x = (r - f.r0) / f.h;
  const int k = std::max(0, std::min((int)std::floor(x), SI - 1));
  const double t = x - k, u = 1.0 - t;
  b[0] = u * u * u / 6; b[1] = (3 * t * t * t - 6 * t * t + 4) / 6;
  b[2] = (-3 * t * t * t + 3 * t * t + 3 * t + 1) / 6; b[3] = t * t * t / 6;
  db[0] = -0.5 * u * u / f.h; db[1] = (1.5 * t * t - 2 * t) / f.h;
  db[2] = (-1.5 * t * t + t + 0.5) / f.h; db[3] = 0.5 * t * t / f.h;
  return k;
}

static void embed(const sg_simparams &P, double rho, double &F, double &Fp, double &Fpp) {
  const double rhoe = P.rhoe, rhoei = P.rhoei;
  if (rho < 0.85f * P.rhoe) {
    const double s = rhoei * (double)1.176471f, x = rho * s - 1.0;
    F = P.Fn[0] + x * (P.Fn[1] + x * (P.Fn[2] + x * P.Fn[3]));
    Fp = s * (P.Fn[1] + x * (2.0 * P.Fn[2] + 3.0 * x * P.Fn[3]));
    Fpp = s * s * (2.0 * P.Fn[2] + 6.0 * x * P.Fn[3]);
  } else if (rho < 1.15f * P.rhoe) {
    const double s = rhoei, x = rho * s - 1.0;
    F = P.F[0] + x * (P.F[1] + x * (P.F[2] + x * P.F[3]));
    Fp = s * (P.F[1] + x * (2.0 * P.F[2] + 3.0 * x * P.F[3]));
    Fpp = s * s * (2.0 * P.F[2] + 6.0 * x * P.F[3]);
  } else {
    const double eta = P.eta, y = rho * rhoei, ly = std::log(y), ye = std::pow(y, eta);
    F = P.Fe * (1.0 - eta * ly) * ye;
    Fp = -P.Fe * eta * eta * rhoei * ye / y * ly;
    Fpp = -P.Fe * eta * eta * rhoei * rhoei * ye / (y * y) * ((eta - 1.0) * ly + 1.0);
  }
  (void)rhoe;
}

static double mi(double d, double L) { return d - L * std::nearbyint(d / L); }

// pair geometry of (i, k): d = r_i - r_k (minimum image), rr
static void geom(const Frame &f, int i, int k, double d[3], double &rr) {
  const double L[3] = {f.p.region.x, f.p.region.y, f.p.region.z};
  d[0] = mi(f.r[i].x - f.r[k].x, L[0]); d[1] = mi(f.r[i].y - f.r[k].y, L[1]); d[2] = mi(f.r[i].z - f.r[k].z, L[2]);
  rr = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
}
}  // namespace diff

extern "C" {

orc_sim *orc_create(const sg_simparams *p, int precision, int force_rebuild) {
  orc_sim *s = new orc_sim;
  s->h.prec = precision == 64 ? 64 : 32;
  if (s->h.prec == 32) s->h.f = new Sim<float>(*p, force_rebuild);
  else s->h.d = new Sim<double>(*p, force_rebuild);
  return s;
}
void orc_destroy(orc_sim *s) {
  if (!s) return;
  delete s->h.f;
  delete s->h.d;
  delete s;
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_state(orc_sim *s, const sg_float4 *r, const sg_float3 *v, const sg_float3 *a) {
  if (s->h.prec == 32) setState(*s->h.f, r, v, a);
  else setState(*s->h.d, r, v, a);
}
void orc_get_state(orc_sim *s, sg_float4 *r, sg_float3 *v, sg_float3 *a) {
  if (s->h.prec == 32) getState(*s->h.f, r, v, a);
  else getState(*s->h.d, r, v, a);
}
void orc_get_state64(orc_sim *s, double *r4, double *v3, double *a3) {
  if (s->h.prec == 32) getState64(*s->h.f, r4, v3, a3);
  else getState64(*s->h.d, r4, v3, a3);
}
void orc_metal_cm64(orc_sim *s, double *cm) {
  if (s->h.prec == 32) metalCm64(*s->h.f, cm);
  else metalCm64(*s->h.d, cm);
}
void orc_set_state64(orc_sim *s, const double *r4, const double *v3, const double *a3) {
  if (s->h.prec == 32) setState64(*s->h.f, r4, v3, a3);
  else setState64(*s->h.d, r4, v3, a3);
}
int orc_step(orc_sim *s, int nsteps) {
  for (int i = 0; i < nsteps; i++) DISPATCH(s, step());
  return 0;
}
void orc_get_thermo(orc_sim *s, sg_thermo *t) {
  if (s->h.prec == 32) getThermo(*s->h.f, t);
  else getThermo(*s->h.d, t);
}
void orc_get_params(orc_sim *s, sg_simparams *p) { *p = (s->h.prec == 32) ? s->h.f->P : s->h.d->P; }
int orc_build_lists(orc_sim *s) {
  if (s->h.prec == 32) { s->h.f->binAtoms(); s->h.f->buildNebr(); }
  else { s->h.d->binAtoms(); s->h.d->buildNebr(); }
  return 0;
}
int orc_compute_forces(orc_sim *s) {
  DISPATCH(s, computeForces());
  return 0;
}
int orc_eval_rdf(orc_sim *s) {
  DISPATCH(s, evalRdf());
  return 0;
}
void orc_reset_rdf(orc_sim *s) {
  if (s->h.prec == 32) std::fill(s->h.f->hist.begin(), s->h.f->hist.end(), 0u);
  else std::fill(s->h.d->hist.begin(), s->h.d->hist.end(), 0u);
}
int orc_num_cells(orc_sim *s) { return (s->h.prec == 32) ? s->h.f->ncells : s->h.d->ncells; }
void orc_get_cells(orc_sim *s, int *co, int *cs, int *ca) {
  if (s->h.prec == 32) getCells(*s->h.f, co, cs, ca);
  else getCells(*s->h.d, co, cs, ca);
}
void orc_get_nebr(orc_sim *s, int *nn, int *nbl) {
  if (s->h.prec == 32) getNebr(*s->h.f, nn, nbl);
  else getNebr(*s->h.d, nn, nbl);
}
void orc_get_rho(orc_sim *s, float *rho) {
  if (s->h.prec == 32) getVec(s->h.f->rho, s->h.f->nMolMe, rho);
  else getVec(s->h.d->rho, s->h.d->nMolMe, rho);
}
void orc_get_friction(orc_sim *s, float *fric) {
  if (s->h.prec == 32) getVec(s->h.f->fric, s->h.f->nMolMe, fric);
  else getVec(s->h.d->fric, s->h.d->nMolMe, fric);
}
void orc_get_rdf(orc_sim *s, unsigned int *hist) {
  const std::vector<unsigned> &h = (s->h.prec == 32) ? s->h.f->hist : s->h.d->hist;
  std::copy(h.begin(), h.end(), hist);
}
void orc_get_diffusion(orc_sim *s, float *rr, int *counts, int *cav) {
  if (s->h.prec == 32) getDiff(*s->h.f, rr, counts, cav);
  else getDiff(*s->h.d, rr, counts, cav);
}
// Output bookkeeping of the step loop, for driving the reference's writers from an oracle run:
// the seven property accumulators of the last averaging step (totEnergy, potEnergy, kinEnergy,
// oneStep, centerOfMass, cmVel, frictForce, before they were zeroed), the number of RDF prints
// and diffusion tables so far (kind 0 / 1), the last printed RDF histogram and table k.
void orc_get_last_avg(orc_sim *s, sg_prop *out7) {
  for (int k = 0; k < 7; k++) out7[k] = (s->h.prec == 32) ? s->h.f->lastAvg7[k] : s->h.d->lastAvg7[k];
}
int orc_num_prints(orc_sim *s, int kind) {
  if (s->h.prec == 32) return kind == 0 ? s->h.f->rdfPrints : (int)s->h.f->diffuseTables.size();
  return kind == 0 ? s->h.d->rdfPrints : (int)s->h.d->diffuseTables.size();
}
void orc_get_rdf_print(orc_sim *s, unsigned *hist) {
  const std::vector<unsigned> &h = (s->h.prec == 32) ? s->h.f->lastRdfPrint : s->h.d->lastRdfPrint;
  std::copy(h.begin(), h.end(), hist);
}
int orc_get_diffuse_print(orc_sim *s, int k, float *table) {
  const auto &t = (s->h.prec == 32) ? s->h.f->diffuseTables : s->h.d->diffuseTables;
  if (k < 0 || k >= (int)t.size()) return -1;
  std::copy(t[k].begin(), t[k].end(), table);
  return 0;
}
void orc_get_diag(orc_sim *s, sg_diag *d) { *d = (s->h.prec == 32) ? s->h.f->diag : s->h.d->diag; }

void orc_reduce(const sg_simparams *p, int what, const sg_float4 *r, const sg_float3 *v,
                const float *fric, float cmVelX, float *out) {
  Sim<float> S(*p, 0);
  setState(S, r, v, nullptr);
  if (fric)
    for (int i = 0; i < p->nMolMe; i++) S.fric[i] = fric[i];
  F3 o = S.reduce(what, cmVelX);
  out[0] = o.x; out[1] = o.y; out[2] = o.z;
}

int orc_diffusion_replay(const sg_simparams *p, int n, const float *cm3, float *tables, int maxTables) {
  Sim<float> S(*p, 0, true);
  int produced = 0;
  for (int i = 0; i < n; i++) {
    int before = S.diffusePrints;
    S.evalDiffusion(F3{cm3[3 * i], cm3[3 * i + 1], cm3[3 * i + 2]});
    if (S.diffusePrints != before && produced < maxTables) {
      std::copy(S.lastDiffusePrint.begin(), S.lastDiffusePrint.end(), tables + (size_t)produced * p->nValDiffuse);
      produced++;
    }
  }
  return produced;
}

double orc_eam_eval(const sg_simparams *p, int which, double x, int precision) {
  if (precision == 64) {
    Model<double> m; m.load(*p);
    switch (which) {
      case 0: return m.phi(x); case 1: return m.f(x); case 2: return m.Femb(x);
      case 3: return m.dphi(x); case 4: return m.df(x); default: return m.dFemb(x);
    }
  }
  Model<float> m; m.load(*p);
  float xf = (float)x;
  switch (which) {
    case 0: return m.phi(xf); case 1: return m.f(xf); case 2: return m.Femb(xf);
    case 3: return m.dphi(xf); case 4: return m.df(xf); default: return m.dFemb(xf);
  }
}

void orc_rdf_allpairs(const sg_simparams *p, const sg_float4 *r, int nbins, double range,
                      unsigned long long *hist) {
  int n = p->nMolMe;
  double L[3] = {p->region.x, p->region.y, p->region.z};
  std::fill(hist, hist + nbins, 0ull);
  double scale = nbins / range;
  for (int i = 0; i < n; i++)
    for (int k = 0; k < n; k++) {
      if (i == k) continue;
      double d[3] = {(double)r[i].x - r[k].x, (double)r[i].y - r[k].y, (double)r[i].z - r[k].z};
      for (int c = 0; c < 3; c++) d[c] -= L[c] * std::nearbyint(d[c] / L[c]);
      double rr = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      double rd = sqrt(rr);
      if (rd < range) {
        int b = (int)(rd * scale);
        if (b >= 0 && b < nbins) hist[b]++;
      }
    }
}

// Frames (their parameter blocks from sg_diff_frame_params), positions of all frames
// concatenated; ref may be NULL (no loss).  Outputs may be NULL.
int orc_diff_eval(const sg_simparams *frames, int nFrames, const sg_float4 *r, const double *theta,
                  const float *ref, double *energy, double *forces, double *gradE, double *loss, double *gradL) {
  using namespace diff;
  std::vector<Frame> F(nFrames);
  int off = 0, ntot = 0;
  for (int q = 0; q < nFrames; q++) ntot += frames[q].nMol;
  std::vector<double> force((size_t)3 * ntot, 0.0), gE(NP, 0.0), gD(NP, 0.0), en(nFrames, 0.0);
  std::vector<double> Fp((size_t)ntot, 0.0), Fpp((size_t)ntot, 0.0), rhoA((size_t)ntot, 0.0);
  const double eps = theta[0], sig = theta[1];
  for (int q = 0; q < nFrames; q++) {
    Frame &f = F[q];
    f.p = frames[q];
    f.M.load(f.p);
    f.n = f.p.nMol;
    f.nMe = f.p.nMolMe;
    f.r0 = 0.6 / (double)f.p.rei;
    f.h = (std::sqrt((double)f.p.rrCutEam) - f.r0) / SI;
    Sim<float> S(f.p, 1);
    for (int i = 0; i < f.n; i++) S.r[i] = V4<float>{r[off + i].x, r[off + i].y, r[off + i].z, 0.f};
    S.binAtoms();
    S.buildNebr();
    f.NN = S.NN;
    f.NBL = S.NBL;
    f.r.resize(f.n);
    for (int i = 0; i < f.n; i++) f.r[i] = V4<double>{r[off + i].x, r[off + i].y, r[off + i].z, 0.0};
    // densities and embedding
    for (int i = 0; i < f.nMe; i++) {
      double rho = 0;
      for (int j = 0; j < f.NN[i]; j++) {
        const int k = f.NBL[(size_t)j * f.n + i];
        if (k >= f.nMe) continue;
        double d[3], rr;
        geom(f, i, k, d, rr);
        if (rr >= (double)f.p.rrCutEam) continue;
        double b[4], db[4];
        const int kk = bsp(f, std::sqrt(rr), b, db);
        for (int m = 0; m < 4; m++) rho += theta[DEN + kk + m] * b[m];
      }
      double Fv, Fd, Fdd;
      embed(f.p, rho, Fv, Fd, Fdd);
      rhoA[off + i] = rho; Fp[off + i] = Fd; Fpp[off + i] = Fdd;
      en[q] += Fv;
    }
    // forces, pair energies, energy gradient
    for (int i = 0; i < f.nMe; i++) {
      for (int j = 0; j < f.NN[i]; j++) {
        const int k = f.NBL[(size_t)j * f.n + i];
        double d[3], rr;
        geom(f, i, k, d, rr);
        if (k < f.nMe) {
          if (rr >= (double)f.p.rrCutEam) continue;
          const double rl = std::sqrt(rr);
          double b[4], db[4];
          const int kk = bsp(f, rl, b, db);
          double phi = 0, dphi = 0, df = 0;
          for (int m = 0; m < 4; m++) {
            phi += theta[PHI + kk + m] * b[m]; dphi += theta[PHI + kk + m] * db[m]; df += theta[DEN + kk + m] * db[m];
            gE[PHI + kk + m] += 0.5 * b[m];
            gE[DEN + kk + m] += Fp[off + i] * b[m];
          }
          const double fc = -(dphi + df * (Fp[off + i] + Fp[off + k])) / rl;
          for (int c = 0; c < 3; c++) force[3 * (off + i) + c] += fc * d[c];
          en[q] += 0.5 * phi;
        } else {
          if (rr >= (double)f.p.rrCutLJ) continue;
          const double s2 = sig * sig / rr, s6 = s2 * s2 * s2, s12 = s6 * s6;
          const double fc = 24.0 * eps * (2.0 * s12 - s6) / rr;
          for (int c = 0; c < 3; c++) {
            force[3 * (off + i) + c] += fc * d[c];
            force[3 * (off + k) + c] -= fc * d[c];
          }
          en[q] += 4.0 * eps * (s12 - s6);
          gE[0] += 4.0 * (s12 - s6);
          gE[1] += 24.0 * eps * (2.0 * s12 - s6) / sig;
        }
      }
    }
    off += f.n;
  }
  double L = 0;
  if (ref) {
    const double inv3N = 1.0 / (3.0 * ntot);
    std::vector<double> e((size_t)3 * ntot);
    for (size_t t = 0; t < e.size(); t++) {
      const double x = force[t] - (double)ref[t];
      L += x * x * inv3N;
      e[t] = 2.0 * inv3N * x;
    }
    off = 0;
    for (int q = 0; q < nFrames; q++) {
      Frame &f = F[q];
      for (int i = 0; i < f.nMe; i++) {
        const double *ei = &e[3 * (off + i)];
        // g_i
        double g = 0;
        for (int j = 0; j < f.NN[i]; j++) {
          const int k = f.NBL[(size_t)j * f.n + i];
          if (k >= f.nMe) continue;
          double d[3], rr;
          geom(f, i, k, d, rr);
          if (rr >= (double)f.p.rrCutEam) continue;
          const double rl = std::sqrt(rr);
          const double *ek = &e[3 * (off + k)];
          const double w = (d[0] * (ei[0] - ek[0]) + d[1] * (ei[1] - ek[1]) + d[2] * (ei[2] - ek[2])) / rl;
          double b[4], db[4];
          const int kk = bsp(f, rl, b, db);
          for (int m = 0; m < 4; m++) g += theta[DEN + kk + m] * db[m] * w;
        }
        for (int j = 0; j < f.NN[i]; j++) {
          const int k = f.NBL[(size_t)j * f.n + i];
          double d[3], rr;
          geom(f, i, k, d, rr);
          const double rl = std::sqrt(rr);
          const double *ek = &e[3 * (off + k)];
          const double w = (d[0] * (ei[0] - ek[0]) + d[1] * (ei[1] - ek[1]) + d[2] * (ei[2] - ek[2])) / rl;
          if (k < f.nMe) {
            if (rr >= (double)f.p.rrCutEam) continue;
            double b[4], db[4];
            const int kk = bsp(f, rl, b, db);
            for (int m = 0; m < 4; m++) {
              gD[PHI + kk + m] += 0.5 * db[m] * w;
              gD[DEN + kk + m] += Fpp[off + i] * g * b[m] + Fp[off + i] * db[m] * w;
            }
          } else {
            if (rr >= (double)f.p.rrCutLJ) continue;
            const double s2 = sig * sig / rr, s6 = s2 * s2 * s2, s12 = s6 * s6;
            gD[0] += 24.0 * (s6 - 2.0 * s12) / rl * w;
            gD[1] += 144.0 * eps * (s6 - 4.0 * s12) / (rl * sig) * w;
          }
        }
      }
      off += f.n;
    }
  }
  if (energy) std::copy(en.begin(), en.end(), energy);
  if (forces) std::copy(force.begin(), force.end(), forces);
  if (gradE) std::copy(gE.begin(), gE.end(), gradE);
  if (loss) *loss = L;
  if (gradL) for (int t = 0; t < NP; t++) gradL[t] = -gD[t];
  return 0;
}

}  // extern "C"
