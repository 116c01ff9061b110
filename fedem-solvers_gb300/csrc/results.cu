// results.cu -- results database of the primary response: one record per
// model and completed time step, written on the GPU into a small ring buffer,
// copied to the host at the engine's synchronisation points and appended to
// one file per model.
//
// The record follows the reference's primary response output
// (src/vpmSolver/saveModule.f90:615-663 writeSolverDB1, with the time-step
// header of src/vpmCommon/rdbModule.f90:669-736 writeTimeStepDB): the step
// number (32-bit integer), the time (64-bit), then for every triad its
// position matrix ur (3 x 4, column by column) when it has six DOFs or its
// translation ur(:,4) when it has three (saveModule.f90:3411-3434
// writeTriadDB1), then for every superelement its frame supTR (3 x 4) and, for
// a reduced part, its generalized DOF values (saveModule.f90:3605-3627
// writeSupelDB1).  Values are double precision or single precision (the
// reference's -double1 option).  A record of the current state is written
// when the database is opened, as the reference saves the initial
// configuration before time stepping (solverModule.f90:512-513).  The file
// header is this library's own text block (the reference's header layout
// lives in the results-database library of its absent fedem-foundation
// submodule): it names the record layout, precision and record size.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"

namespace fgpu {
namespace {

// one block per model: the record of its current state when its step has just
// completed (or unconditionally when all != 0), into ring slot count % ring
__global__ void kRecordStep(DevData d, RecordPlan r, int all) {
  pdlEntry();
  const int m = blockIdx.x;
  if (m >= d.m.n) return;
  if (!all && !(d.m.flags[m] & FL_STEPDONE)) return;
  const long long cnt = r.count[m];
  double* rec = r.buf + r.off[m] + (cnt % r.ring) * (long long)r.vals[m];
  if (threadIdx.x == 0) {
    rec[0] = (double)d.m.nStep[m];
    rec[1] = d.m.time[m];
  }
  // triads: 12 values (six DOFs) or 3 (three DOFs) at their record offsets
  const int t0 = d.m.triOff[m], nt = d.m.ntri[m];
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    const int g = t0 + t, nd = d.triNdof[g];
    const double* U = d.ur + 12 * (size_t)g;
    double* o = rec + r.triRec[g];
    if (nd == 6)
      for (int k = 0; k < 12; ++k) o[k] = U[k];
    else if (nd == 3)
      for (int k = 0; k < 3; ++k) o[k] = U[9 + k];
  }
  // beam superelements: frame supTR (entry-major element arrays)
  const int e0 = d.m.elOff[m], ne = d.m.nel[m];
  double* eb = rec + r.elRec[m];
  for (int e = threadIdx.x; e < ne; e += blockDim.x)
    for (int k = 0; k < 12; ++k) eb[12 * e + k] = d.supTr[(size_t)k * d.nelTot + e0 + e];
  // reduced parts: frame and generalized DOF values
  for (int p = r.partFirst[m] + threadIdx.x; p < r.partFirst[m + 1]; p += blockDim.x) {
    double* o = rec + r.partRec[p];
    for (int k = 0; k < 12; ++k) o[k] = d.pSupTr[12 * (size_t)p + k];
    const int ng = d.pNgen[p];
    for (int k = 0; k < ng; ++k) o[12 + k] = d.pGen[d.pGenOff[p] + k];
  }
  __syncthreads();
  if (threadIdx.x == 0) r.count[m] = cnt + 1;
}

}  // namespace

void launchRecordStep(const DevData& d, const RecordPlan& r, bool all, cudaStream_t s) {
  if (d.m.n > 0) pdlLaunch(kRecordStep, d.m.n, 128, 0, s, d, r, all ? 1 : 0);
}

int Engine::resultsOpen(const std::string& dir, bool asDouble, std::string& err,
                        const std::vector<std::string>* paths, double saveStart) {
  if (rec_.on) {
    err = "the results database is already open";
    return -1;
  }
  const int nm = d_.m.n;
  RecordPlan& r = rec_.plan;
  r.ring = kRecordRing;
  std::vector<long long> off(nm);
  std::vector<int> vals(nm), triRec(d_.ntriTot), elRec(nm), partFirst(nm + 1, 0), partRec(d_.npartTot > 0 ? d_.npartTot : 1);
  long long tot = 0;
  int pBase = 0;
  rec_.files.assign(nm, nullptr);
  rec_.asDouble = asDouble;
  for (int m = 0; m < nm; ++m) {
    const HostModel& h = *hm_[m];
    int v = 2;
    std::string layout;
    char line[256];
    for (int t = 0; t < h.ntri; ++t) {
      triRec[modelTriOff_[m] + t] = v;
      const int nd = h.triNdof[t];
      if (nd == 6 || nd == 3) {
        snprintf(line, sizeof line, "#triad %d %s\n", h.triId[t], nd == 6 ? "position 3x4" : "translation 3");
        layout += line;
      }
      v += nd == 6 ? 12 : (nd == 3 ? 3 : 0);
    }
    elRec[m] = v;
    for (int e = 0; e < h.nel; ++e) {
      snprintf(line, sizeof line, "#supel %d frame 3x4\n", h.elId[e]);
      layout += line;
    }
    v += 12 * h.nel;
    partFirst[m] = pBase;
    for (int p = 0; p < h.npart; ++p) {
      partRec[pBase + p] = v;
      snprintf(line, sizeof line, "#part %d frame 3x4 generalized %d\n", p + 1, h.pNgen[p]);
      layout += line;
      v += 12 + h.pNgen[p];
    }
    pBase += h.npart;
    vals[m] = v;
    off[m] = tot;
    tot += (long long)v * r.ring;
    const std::string path =
        paths && m < (int)paths->size() ? (*paths)[m] : dir + "/model" + std::to_string(m) + ".res";
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) {
      err = "cannot open " + path;
      for (FILE*& g : rec_.files)
        if (g) fclose(g), g = nullptr;
      return -2;
    }
    const size_t recBytes = 4 + 8 + (size_t)(v - 2) * (asDouble ? 8 : 4);
    fprintf(f, "#FEDEM results database: primary response\n#model %d\n", m);
    fprintf(f, "#precision %s\n#record bytes %zu: step int32, time float64, then in this order:\n",
            asDouble ? "double" : "single", recBytes);
    fputs(layout.c_str(), f);
    fputs("#data\n", f);
    rec_.files[m] = f;
  }
  partFirst[nm] = pBase;
  // device arrays, released with the engine's other allocations
  bool failed = false;
  auto dalloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes > 0 ? bytes : 8) != cudaSuccess) {
      failed = true;
      return nullptr;
    }
    cudaMemsetAsync(p, 0, bytes > 0 ? bytes : 8, stream_);
    allocs_.push_back(p);
    deviceBytes_ += bytes;
    return p;
  };
  r.buf = (double*)dalloc(sizeof(double) * (size_t)tot);
  r.off = (long long*)dalloc(sizeof(long long) * nm);
  r.vals = (int*)dalloc(sizeof(int) * nm);
  r.triRec = (int*)dalloc(sizeof(int) * (size_t)d_.ntriTot);
  r.elRec = (int*)dalloc(sizeof(int) * nm);
  r.partFirst = (int*)dalloc(sizeof(int) * (nm + 1));
  r.partRec = (int*)dalloc(sizeof(int) * partRec.size());
  r.count = (long long*)dalloc(sizeof(long long) * nm);
  if (failed) {
    err = "out of device memory for the results ring";
    for (FILE*& g : rec_.files)
      if (g) fclose(g), g = nullptr;
    return -3;
  }
  cudaMemcpyAsync(r.off, off.data(), sizeof(long long) * nm, cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(r.vals, vals.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  if (d_.ntriTot > 0)
    cudaMemcpyAsync(r.triRec, triRec.data(), sizeof(int) * d_.ntriTot, cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(r.elRec, elRec.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(r.partFirst, partFirst.data(), sizeof(int) * (nm + 1), cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(r.partRec, partRec.data(), sizeof(int) * partRec.size(), cudaMemcpyHostToDevice, stream_);
  rec_.vals = vals;
  rec_.off = off;
  // no save before saveStart (solverRoutinesModule.f90:590-592: time + 0.1 minInc < saveStart)
  rec_.saveStart = saveStart;
  rec_.epsT = nm > 0 ? 0.1 * hm_[0]->ctl.minInc : 0.0;
  rec_.written.assign(nm, 0);
  rec_.on = true;
  // the batched iteration is captured again with the record kernel in it
  if (graphExec_) cudaGraphExecDestroy(graphExec_), graphExec_ = nullptr;
  if (graph_) cudaGraphDestroy(graph_), graph_ = nullptr;
  // the current state: the initial configuration, or where the models are now
  launchRecordStep(d_, r, true, stream_);
  return resultsDrain(err);
}

// Copies the records written since the last drain to the host and appends
// them to the files.  Called after every synchronised chunk of iterations
// (at most kRecordRing - 1 iterations apart, one record per model and
// iteration at most).
int Engine::resultsDrain(std::string& err) {
  if (!rec_.on) return 0;
  const int nm = d_.m.n;
  std::vector<long long> cnt(nm);
  cudaMemcpyAsync(cnt.data(), rec_.plan.count, sizeof(long long) * nm, cudaMemcpyDeviceToHost, stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) {
    err = "results: device error";
    return -4;
  }
  const int ring = rec_.plan.ring;
  for (int m = 0; m < nm; ++m) {
    const long long n = cnt[m] - rec_.written[m];
    if (n <= 0) continue;
    if (n > ring) {
      err = "results: records overwritten before they were read";
      return -5;
    }
    const int v = rec_.vals[m];
    rec_.host.resize((size_t)v * n);
    for (long long k = 0; k < n; ++k) {
      const long long slot = (rec_.written[m] + k) % ring;
      cudaMemcpyAsync(rec_.host.data() + (size_t)k * v, rec_.plan.buf + rec_.off[m] + slot * v, sizeof(double) * v,
                      cudaMemcpyDeviceToHost, stream_);
    }
    if (cudaStreamSynchronize(stream_) != cudaSuccess) {
      err = "results: device error";
      return -4;
    }
    FILE* f = rec_.files[m];
    std::vector<float> fl(rec_.asDouble ? 0 : v - 2);
    bool ok = true;
    for (long long k = 0; k < n; ++k) {
      const double* rec = rec_.host.data() + (size_t)k * v;
      if (rec[1] + rec_.epsT < rec_.saveStart) continue;
      const int step = (int)rec[0];
      ok = ok && fwrite(&step, sizeof(int), 1, f) == 1;
      ok = ok && fwrite(rec + 1, sizeof(double), 1, f) == 1;
      if (rec_.asDouble) {
        ok = ok && fwrite(rec + 2, sizeof(double), v - 2, f) == (size_t)(v - 2);
      } else {
        for (int q = 0; q < v - 2; ++q) fl[q] = (float)rec[2 + q];
        ok = ok && fwrite(fl.data(), sizeof(float), v - 2, f) == (size_t)(v - 2);
      }
    }
    if (!ok) {
      err = "results: writing model " + std::to_string(m) + "'s file failed";
      return -6;
    }
    rec_.written[m] = cnt[m];
  }
  return 0;
}

int Engine::resultsClose(std::string& err) {
  if (!rec_.on) return 0;
  int rc = resultsDrain(err);
  for (FILE*& f : rec_.files)
    if (f) {
      if (fclose(f) != 0 && rc == 0) {
        err = "results: closing a file failed";
        rc = -7;
      }
      f = nullptr;
    }
  rec_.on = false;
  if (graphExec_) cudaGraphExecDestroy(graphExec_), graphExec_ = nullptr;
  if (graph_) cudaGraphDestroy(graph_), graph_ = nullptr;
  return rc;
}

}  // namespace fgpu
