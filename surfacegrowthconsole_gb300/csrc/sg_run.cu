// sg_run.cu - whole-simulation driver with the reference's outputs (DoComputationsW loop,
// SurfaceGrowth.cu:2128-2494): steps run as CUDA-graph launches back to back; the host
// synchronises only where an output is due (summary row every stepAvg steps, rdf file after
// limitRdf samples, pdb every stepPdb steps, Diffuse.txt tables, backups, the last step).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "sg_api.h"
#include "sg_engine.h"

using namespace sg;

namespace {
struct Events {
  std::vector<cudaEvent_t> ev;
  cudaEvent_t get(size_t i) {
    while (ev.size() <= i) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev.push_back(e);
    }
    return ev[i];
  }
  ~Events() {
    for (auto e : ev) cudaEventDestroy(e);
  }
};
// host mirror of the diffusion buffer counters (InitDiffusion/EvalDiffusion/AccumDiffusion),
// so the host knows without reading the device when a table is finished
struct DiffMirror {
  std::vector<int> count;
  int countAv = 0;
  void init(const sg_simparams &p) {
    count.resize(p.nBuffDiffuse);
    for (int nb = 0; nb < p.nBuffDiffuse; nb++) count[nb] = -nb * p.nValDiffuse / p.nBuffDiffuse;
    countAv = p.countDiffuseAv;
  }
  int sample(const sg_simparams &p) {  // returns the number of tables finished
    for (int nb = 0; nb < p.nBuffDiffuse; nb++) ++count[nb];
    int prints = 0;
    for (int nb = 0; nb < p.nBuffDiffuse; nb++)
      if (count[nb] == p.nValDiffuse) {
        count[nb] = 0;
        if (++countAv == p.limitDiffuseAv) {
          countAv = 0;
          prints++;
        }
      }
    return prints;
  }
};
}  // namespace

extern "C" int sg_run(sg_ctx *c, void *fResultsV, const char *pdbPrefix) {
  if (!c) return sg_fail(SG_ERR_INVALID, "null context");
  if (c->nrep != 1) return sg_fail(SG_ERR_UNSUPPORTED, "sg_run drives a single replica");
  FILE *fResults = (FILE *)fResultsV;
  sg_simparams p0 = c->hp[0];
  const sg_simparams &P = c->hp[0];
  int rc;
  FILE *fDiff = nullptr;
  DiffMirror dm;
  if (P.iRegime == 2) {
    fDiff = fopen(P.szDiffusePath, "w");
    if (!fDiff) return sg_fail(SG_ERR_IO, "Cannot open diffuse file!");
    dm.init(P);
  }
  std::vector<sg_float4> hr(P.nMol);
  std::vector<sg_float3> hv(P.nMol), ha(P.nMol);
  if (P.bPdb) {
    if ((rc = sg_get_state(c, 0, hr.data(), nullptr, nullptr))) return rc;
    sg_simparams q;
    if ((rc = sg_get_params(c, 0, &q))) return rc;
    sg_create_pdb(pdbPrefix ? pdbPrefix : "sugr", &q, hr.data());
  }
  Events ev;
  size_t nev = 0;  // events recorded since the last synchronisation: 2 per step
  int iBckup = 1;
  float totalTime = p0.totalTime;
  std::vector<float> table(P.nValDiffuse > 0 ? P.nValDiffuse : 1);
  std::vector<unsigned> hist(P.sizeHistRdf > 0 ? P.sizeHistRdf : 1);
  cudaStream_t s = c->stream;
  while (true) {
    const int sc = c->stepCount + 1;
    const int variant = sg_next_variant(c);
    cudaEventRecord(ev.get(nev++), s);
    bool rdfPrint = false;
    if ((rc = sg_launch_step(c, variant, &rdfPrint))) return rc;
    cudaEventRecord(ev.get(nev++), s);
    int diffPrints = 0;
    if (P.iRegime == 2 && P.nMolMe != 0 && sc > P.stepEquil && ((sc - P.stepEquil) % P.stepDiffuse == 0))
      diffPrints = dm.sample(P);
    const bool avg = (sc % P.stepAvg == 0);
    const bool pdb = P.bPdb && (sc % P.stepPdb == 0);
    const bool bck = P.bBckup && (sc % P.stepBckup == 0);
    const bool last = sc >= P.stepLimit;
    if (!(avg || pdb || bck || last || rdfPrint || diffPrints)) continue;
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return sg_fail(SG_ERR_CUDA, "step %d: %s", sc, cudaGetErrorString(e));
    // step times of the steps since the last synchronisation (oneStep property)
    sg_prop &os = c->oneStep[0];
    for (size_t k = 0; k + 1 < nev; k += 2) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev.get(k), ev.get(k + 1));
      os.val = ms;
      os.sum += os.val;
      os.sum2 += os.val * os.val;
      totalTime += ms * 0.001f;
    }
    nev = 0;
    if ((rc = sg_check_flags(c))) return rc;
    sg_simparams q;
    if ((rc = sg_get_params(c, 0, &q))) return rc;
    for (int k = 0; k < diffPrints; k++) {
      if ((rc = sg_get_diffusion_print(c, 0, table.data(), nullptr))) return rc;
      sg_print_diffusion(fDiff, &q, table.data());
    }
    if (rdfPrint) {
      if ((rc = sg_get_rdf(c, 0, hist.data()))) return rc;
      sg_simparams qr = q;
      qr.countRdf = P.limitRdf;
      sg_print_rdf(&qr, hist.data());
    }
    if (avg) {
      // sums at the boundary (device snapshot) + the host's oneStep sums, then PropAvg
      RepState S;
      if ((rc = sg_read_state(c, 0, &S))) return rc;
      sg_simparams qa = q;
      sg_prop *pp[7] = {&qa.totEnergy, &qa.potEnergy, &qa.kinEnergy, &qa.oneStep,
                        &qa.centerOfMass, &qa.cmVel, &qa.frictForce};
      for (int k = 0; k < 7; k++)
        if (k != 3) *pp[k] = sg_prop{S.propsSnap[k][0], S.propsSnap[k][1], S.propsSnap[k][2]};
      qa.oneStep = os;
      sg_accum_props(&qa, 2);
      if (P.bResult && fResults) sg_print_summary(fResults, &qa);
      os.sum = os.sum2 = 0.f;
    }
    if (pdb || bck) {
      if ((rc = sg_get_state(c, 0, hr.data(), bck ? hv.data() : nullptr, bck ? ha.data() : nullptr))) return rc;
      if (pdb) sg_create_pdb(pdbPrefix ? pdbPrefix : "sugr", &q, hr.data());
      if (bck) {
        q.totalTime = totalTime;
        sg_write_backup(iBckup ? P.szBckup0 : P.szBckup1, &q, hr.data(), hv.data(), ha.data());
        iBckup = !iBckup;
      }
    }
    if (last) break;
  }
  if (P.bResult && fResults) fprintf(fResults, "\nDuration of the simulation = %f s", totalTime);
  c->hp[0].totalTime = totalTime;
  if (fDiff) fclose(fDiff);
  return SG_OK;
}
