// sg_noalloc.cu - force evaluation that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code running under another framework's memory manager,
// which owns the device heap and forbids raw allocations; code that must not stall other work
// on the device with the implicit synchronisation of cudaMalloc/cudaFree; plugins that may not
// grow the process's device footprint per call.  sg_compute_forces_noalloc serves them: the
// caller passes device buffers for the inputs and outputs, and every intermediate of the
// evaluation (cell counts and starts, sorted atoms, neighbour lists, EAM densities, the
// parameter block, the block tables) lives in one file-scope static device array of
// SG_NOALLOC_SCRATCH_BYTES, which every GPU that loads the library holds until the process
// exits.
//
// The work is the same kernel chain as sg_build_lists + sg_compute_forces of a context: cell
// counting sort, neighbour list, EAM density, metal and carbon forces.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "sg_api.h"
#include "sg_device.cuh"
#include "sg_engine.h"
#include "sg_kernels.h"

using namespace sg;

namespace {

constexpr size_t kScratchBytes = SG_NOALLOC_SCRATCH_BYTES;
constexpr int kBs = 128;
constexpr int kMaxBlocks = (SG_NOALLOC_MAX_ATOMS + kBs - 1) / kBs;
// table capacity: the metal pass has the smallest blocks (kMetalPerBlock atoms)
constexpr int kMaxTabBlocks = (SG_NOALLOC_MAX_ATOMS + kMetalPerBlock - 1) / kMetalPerBlock;
constexpr int kMaxTiles = SG_NOALLOC_MAX_CELLS / kCellTile;

// The scratch of every call on this device.  Host code must not take its address directly:
// the host-side name is only a stand-in; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Carving of the scratch array (offsets in bytes, each 256-byte aligned).
struct Carve {
  size_t rc, st, tabRep, tabStart, tileRep, tileStart, tileFirst, tileSum, cellCount, cellStart;
  size_t cellOf, slot, tmpIdx, sortIdx, nn, ns, sl, sortPos, rho, dF, Fv, fric, nbl, nrl, rl, active, heavy, work, total;
};
constexpr size_t up(size_t x) { return (x + 255) & ~size_t(255); }
constexpr Carve carve() {
  Carve c{};
  size_t o = 0;
  const size_t N = SG_NOALLOC_MAX_ATOMS;
  c.rc = o; o += up(sizeof(RepConst));
  c.st = o; o += up(sizeof(RepState));
  c.tabRep = o; o += up(3 * kMaxTabBlocks * sizeof(int));    // atom, metal, carbon tables
  c.tabStart = o; o += up(3 * kMaxTabBlocks * sizeof(int));
  c.tileRep = o; o += up(kMaxTiles * sizeof(int));
  c.tileStart = o; o += up(kMaxTiles * sizeof(int));
  c.tileFirst = o; o += up(sizeof(int));
  c.tileSum = o; o += up(kMaxTiles * sizeof(int));
  c.cellCount = o; o += up(SG_NOALLOC_MAX_CELLS * sizeof(int));
  c.cellStart = o; o += up(SG_NOALLOC_MAX_CELLS * sizeof(int));
  c.cellOf = o; o += up(N * sizeof(int));
  c.slot = o; o += up(N * sizeof(int));
  c.tmpIdx = o; o += up(N * sizeof(int));
  c.sortIdx = o; o += up(N * sizeof(int));
  c.nn = o; o += up(N * sizeof(int));
  c.ns = o; o += up(N * sizeof(int));
  c.sl = o; o += up(N * kShortMax * sizeof(int));
  c.sortPos = o; o += up(N * sizeof(float4));
  c.rho = o; o += up(N * sizeof(float));
  c.dF = o; o += up(N * sizeof(float));
  c.Fv = o; o += up(N * sizeof(float));
  c.fric = o; o += up(N * sizeof(float));
  c.nbl = o; o += up(N * SG_NOALLOC_MAX_NEBR * sizeof(int));
  c.nrl = o; o += up(N * sizeof(int));
  c.rl = o; o += up(N * kRelMax * sizeof(unsigned));
  c.active = o; o += up(SG_NOALLOC_MAX_CELLS * sizeof(int));
  c.heavy = o; o += up(((size_t)N / kHeavyChunk + (size_t)N / (kHeavyCell + 1) + 16) * sizeof(int2));
  c.work = o; o += up(3 * sizeof(int));
  c.total = o;
  return c;
}
constexpr Carve kCarve = carve();
static_assert(kCarve.total <= kScratchBytes, "scratch layout exceeds the static array");

// Device address of g_scratch per device ordinal, set up once per device.  The address belongs
// to the context that was current at set-up: the device's primary context, the one the CUDA
// runtime uses.  A caller that resets the device (cudaDeviceReset) or drives the device through
// another driver-API context is outside what this cache supports.
constexpr int kMaxDevices = 64;
unsigned char *g_base[kMaxDevices] = {};
std::mutex g_mu;

// Writes the parameter block, clears the state block and the cell counts, and fills the
// block tables of a single system: everything that must start fresh on every call.
__global__ void k_noalloc_setup(RepConst P, RepState *st, RepConst *rc, int *tabRep, int *tabStart,
                                int *tileRep, int *tileStart, int *tileFirst, int *cellCount, int *work) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  if (t == 0) {
    *rc = P;
    memset(st, 0, sizeof(RepState));
    st->nebrNow = 1;
    *tileFirst = 0;
  }
  for (int b = t; b < kMaxTabBlocks; b += stride) {
    tabRep[b] = 0; tabStart[b] = b * kBs;                                   // atoms, 128 per block
    tabRep[kMaxTabBlocks + b] = 0; tabStart[kMaxTabBlocks + b] = b * kMetalPerBlock;
    tabRep[2 * kMaxTabBlocks + b] = 0; tabStart[2 * kMaxTabBlocks + b] = P.nMolMe + b * kCarbonPerBlock;
  }
  for (int k = t; k < P.ncellsPad / kCellTile; k += stride) {
    tileRep[k] = 0;
    tileStart[k] = k * kCellTile;
  }
  for (int c = t; c < P.ncellsPad; c += stride) cellCount[c] = 0;
  if (t < 3) work[t] = 0;
}

RepConst constFor(const sg_simparams &p) {
  RepConst P;
  memset(&P, 0, sizeof(P));
  P.region[0] = p.region.x; P.region[1] = p.region.y; P.region[2] = p.region.z;
  P.invWidth[0] = p.invWidth.x; P.invWidth[1] = p.invWidth.y; P.invWidth[2] = p.invWidth.z;
  P.cells[0] = p.cells.x; P.cells[1] = p.cells.y; P.cells[2] = p.cells.z;
  P.ncells = p.cells.x * p.cells.y * p.cells.z;
  P.ncellsPad = ((P.ncells + 1 + kCellTile - 1) / kCellTile) * kCellTile;
  P.nMol = p.nMol; P.nMolMe = p.nMolMe;
  P.nRedBlocks = (p.nMol + kRedElems - 1) / kRedElems;
  P.deltaT = p.deltaT; P.rrNebr = p.rrNebr; P.rNebrShell = p.rNebrShell;
  const float rs = p.rCutC + p.rNebrShell;
  P.rrShort = rs * rs;
  P.rei = p.rei; P.rhoei = p.rhoei; P.rhoe = p.rhoe; P.fe = p.fe; P.alpha = p.alpha; P.beta = p.beta;
  P.A = p.A; P.B = p.B; P.kappa = p.kappa; P.lambda = p.lambda;
  for (int i = 0; i < 4; i++) { P.Fn[i] = p.Fn[i]; P.F[i] = p.F[i]; }
  P.eta = p.eta; P.Fe = p.Fe; P.massMe = p.massMe; P.rrCutEam = p.rrCutEam;
  P.rrCutC = p.rrCutC; P.mu_r = p.mu_r; P.theta_0 = p.theta_0; P.mu_theta = p.mu_theta; P.mu_p = p.mu_p;
  P.z_0 = p.z_0; P.sigmaLJ = p.sigmaLJ; P.epsLJ = p.epsLJ; P.rrCutLJ = p.rrCutLJ;
  P.hasFric = (p.iRegime != 0 && p.nMolMe != 0) ? 1 : 0;
  P.iRegime = p.iRegime;
  return P;
}

}  // namespace

extern "C" int sg_compute_forces_noalloc(const sg_simparams *p, sg_float4 *d_pos, sg_float4 *d_acc, void *stream) {
  if (!p || !d_pos || !d_acc) return sg_fail(SG_ERR_INVALID, "sg_compute_forces_noalloc: null argument");
  if (p->nMol <= 0 || p->nMolMe < 0 || p->nMolMe > p->nMol || p->cells.x < 1 || p->cells.y < 1 || p->cells.z < 1)
    return sg_fail(SG_ERR_INVALID, "sg_compute_forces_noalloc: inconsistent parameter block");
  // the cell count in 64 bits: a parameter block from outside may hold any extents, and an int
  // product could wrap to a small value that passes the limit
  const long long ncells64 = (long long)p->cells.x * p->cells.y * p->cells.z;
  const long long ncellsPad64 = ((ncells64 + 1 + kCellTile - 1) / kCellTile) * kCellTile;
  if (p->nMol > SG_NOALLOC_MAX_ATOMS || ncellsPad64 > SG_NOALLOC_MAX_CELLS || p->iNebrMax > SG_NOALLOC_MAX_NEBR ||
      p->iNebrMax < 1)
    return sg_fail(SG_ERR_INVALID,
                   "sg_compute_forces_noalloc: system exceeds the static scratch (nMol %d of max %d, "
                   "padded cells %lld of max %d, iNebrMax %d of max %d)",
                   p->nMol, SG_NOALLOC_MAX_ATOMS, ncellsPad64, SG_NOALLOC_MAX_CELLS, p->iNebrMax, SG_NOALLOC_MAX_NEBR);
  const int ncellsPad = (int)ncellsPad64;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return sg_fail(SG_ERR_NO_DEVICE, "sg_compute_forces_noalloc: no current device");
  unsigned char *base;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {  // set-up, once per device, with that device current
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_scratch);
      if (e != cudaSuccess)
        return sg_fail(SG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
      g_base[dev] = (unsigned char *)ptr;
    }
    base = g_base[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  const Carve &K = kCarve;
  RepConst *rc = (RepConst *)(base + K.rc);
  RepState *st = (RepState *)(base + K.st);
  int *tabRep = (int *)(base + K.tabRep), *tabStart = (int *)(base + K.tabStart);
  int *tileRep = (int *)(base + K.tileRep), *tileStart = (int *)(base + K.tileStart);
  int *tileFirst = (int *)(base + K.tileFirst), *tileSum = (int *)(base + K.tileSum);
  int *cellCount = (int *)(base + K.cellCount), *cellStart = (int *)(base + K.cellStart);
  int *cellOf = (int *)(base + K.cellOf), *slot = (int *)(base + K.slot), *tmpIdx = (int *)(base + K.tmpIdx);
  int *sortIdx = (int *)(base + K.sortIdx), *nn = (int *)(base + K.nn), *ns = (int *)(base + K.ns);
  int *sl = (int *)(base + K.sl);
  float4 *sortPos = (float4 *)(base + K.sortPos);
  float *rho = (float *)(base + K.rho), *dF = (float *)(base + K.dF), *Fv = (float *)(base + K.Fv);
  float *fric = (float *)(base + K.fric);
  int *nbl = (int *)(base + K.nbl), *nrl = (int *)(base + K.nrl);
  unsigned *rl = (unsigned *)(base + K.rl);
  int *active = (int *)(base + K.active), *work = (int *)(base + K.work);
  int2 *heavy = (int2 *)(base + K.heavy);
  float4 *pos = (float4 *)d_pos, *acc = (float4 *)d_acc;

  const RepConst P = constFor(*p);
  const int N = p->nMol;
  const int nAtomBlk = (N + kBs - 1) / kBs;
  const int nMetalBlk = (p->nMolMe + kMetalPerBlock - 1) / kMetalPerBlock;
  const int nCarbBlk = (N - p->nMolMe + kCarbonPerBlock - 1) / kCarbonPerBlock;
  const int nTiles = ncellsPad / kCellTile;
  BlockTab atomTab{tabRep, tabStart, nAtomBlk};
  BlockTab metalTab{tabRep + kMaxTabBlocks, tabStart + kMaxTabBlocks, nMetalBlk};
  BlockTab carbTab{tabRep + 2 * kMaxTabBlocks, tabStart + 2 * kMaxTabBlocks, nCarbBlk};
  BlockTab tileTab{tileRep, tileStart, nTiles};


  k_noalloc_setup<<<64, 256, 0, s>>>(P, st, rc, tabRep, tabStart, tileRep, tileStart, tileFirst, cellCount, work);
  k_cell_count<<<nAtomBlk, kBs, 0, s>>>(atomTab, rc, pos, cellOf, slot, cellCount);
  k_scan_tiles<<<nTiles, 256, 0, s>>>(tileTab, rc, st, cellCount, tileSum, 1);
  k_scan_tile_prefix<<<1, 1024, 0, s>>>(rc, st, tileFirst, tileSum, 1, nullptr);
  k_scan_final<<<nTiles, 256, 0, s>>>(tileTab, rc, st, cellCount, tileSum, cellStart, (int)p->blockSize, 1, active,
                                      heavy, work, kHeavyCell);
  k_scatter<<<nAtomBlk, kBs, 0, s>>>(atomTab, rc, st, cellOf, slot, cellStart, tmpIdx, nn, ns, nrl, 1);
  k_rank<<<nAtomBlk, kBs, 0, s>>>(atomTab, rc, st, cellOf, cellStart, tmpIdx, pos, sortIdx, sortPos, 1);
  const int rowStride = (p->iNebrMax + 3) & ~3;
  k_build_nebr<<<256, kNebrWarps * 32, 0, s>>>(tileRep, active, heavy, work, rc, st, cellStart, sortPos, nn, nbl, ns,
                                               sl, nrl, rl, rowStride, p->iNebrMax, 0,
                                               nullptr, 0);
  if (nMetalBlk) {
    k_rho<<<nMetalBlk, kBs, 0, s>>>(metalTab, rc, pos, nn, nbl, rho, dF, Fv, rowStride);
    k_force_metal<<<nMetalBlk, kBs, 0, s>>>(metalTab, rc, pos, acc, nn, nbl, dF, Fv, fric, rowStride);
  }
  if (nCarbBlk) launchCarbon(false, 8, nCarbBlk, s, carbTab, rc, pos, acc, nn, nbl, ns, sl, nrl, rl, rowStride);
  e = cudaGetLastError();
  if (e != cudaSuccess) return sg_fail(SG_ERR_CUDA, "sg_compute_forces_noalloc launch: %s", cudaGetErrorString(e));
  int flags = 0;
  e = cudaMemcpyAsync(&flags, &st->flags, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return sg_fail(SG_ERR_CUDA, "sg_compute_forces_noalloc: %s", cudaGetErrorString(e));
  for (int code = 1; code < 31; code++)
    if (flags & (1 << code)) return sg_fail(code, "sg_compute_forces_noalloc: device reported condition %d", code);
  return SG_OK;
}
