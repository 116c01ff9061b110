// engine.cu -- host orchestration of the batched GB300 Newton engine.
//
// One batched iteration performs, for every active model, exactly one Newton
// iteration of the reference's NewmarkInt loop
// (src/vpmSolver/newmarkRoutinesModule.f90:711-1024):
//   begin-step control -> predictor vectors -> predictor element pass ->
//   force gather + residual -> [tangent: element Newton matrices -> CSR ->
//   multifrontal factor] -> solve (+ FP64 refinement) -> increment (vectors,
//   triads) -> element pass with the new positions -> norms + convergence.
// The sequence is a fixed list of launches, captured once in a CUDA graph
// and replayed; models that are idle or in another phase early-exit on their
// per-model flags, so models of uneven size and iteration count share launches.

#include <array>
#include <atomic>
#include <chrono>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "engine.h"

namespace fgpu {

#define FG_CHECK(call)                                            \
  do {                                                            \
    cudaError_t e_ = (call);                                      \
    if (e_ != cudaSuccess) {                                      \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);  \
      return -900;                                                \
    }                                                             \
  } while (0)

Engine::~Engine() {
  cudaSetDevice(device_);
  if (rec_.on) {
    std::string err;
    resultsClose(err);
  }
  if (graphExec_) cudaGraphExecDestroy(graphExec_);
  if (graph_) cudaGraphDestroy(graph_);
  if (stream_) cudaStreamSynchronize(stream_);
  for (cudaEvent_t ev : ev_)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : evRun_)
    if (ev) cudaEventDestroy(ev);
  if (evChunk_) cudaEventDestroy(evChunk_);
  for (void* p : allocs_) cudaFree(p);
  if (hActive_) cudaFreeHost(hActive_);
  if (hStates_) cudaFreeHost(hStates_);
  if (side_) cudaStreamSynchronize(side_);
  if (evFork_) cudaEventDestroy(evFork_);
  if (evJoin_) cudaEventDestroy(evJoin_);
  if (evFork2_) cudaEventDestroy(evFork2_);
  if (evJoin2_) cudaEventDestroy(evJoin2_);
  if (side_) cudaStreamDestroy(side_);
  if (stream_) cudaStreamDestroy(stream_);
}

template <typename T>
T* Engine::alloc(size_t n) {
  if (n == 0) n = 1;
  void* p = nullptr;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
    allocFailed_ = true;
    return nullptr;
  }
  cudaMemsetAsync(p, 0, n * sizeof(T), stream_);
  allocs_.push_back(p);
  deviceBytes_ += n * sizeof(T);
  return static_cast<T*>(p);
}

namespace {
thread_local long long t_putBytes = 0;  // host -> device bytes of the current upload

template <typename T>
cudaError_t put(T* dst, const std::vector<T>& src, cudaStream_t s) {
  if (src.empty()) return cudaSuccess;
  t_putBytes += (long long)(src.size() * sizeof(T));
  return cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}
// fn(k) for every model k on the host's threads; each model writes its own
// ranges of the batch arrays (offsets fixed beforehand), so the result does not
// depend on the schedule
template <typename F>
void forEachModel(int nm, F fn) {
  const int hw = (int)std::thread::hardware_concurrency();
  const int nt = std::max(1, std::min(nm, hw > 0 ? hw : 1));
  if (nt <= 1) {
    for (int k = 0; k < nm; ++k) fn(k);
    return;
  }
  std::atomic<int> next{0};
  std::vector<std::thread> pool;
  pool.reserve(nt);
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&] {
      for (int k = next.fetch_add(1); k < nm; k = next.fetch_add(1)) fn(k);
    });
  for (auto& th : pool) th.join();
}

// setup trace: with FGPU_SETUP_TRACE set, each phase of the upload waits for the
// stream and prints its host + device time to stderr
struct SetupTrace {
  bool on = std::getenv("FGPU_SETUP_TRACE") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const char* phase, cudaStream_t s) {
    if (!on) return;
    cudaStreamSynchronize(s);
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "fgpu setup %-24s %8.1f ms\n", phase, std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};
}  // namespace

int Engine::upload(const std::vector<const HostModel*>& models, const EngineOptions& opt, std::string& err) {
  hm_ = models;
  opt_ = opt;
  t_putBytes = 0;
  FG_CHECK(cudaGetDevice(&device_));
  if (!opt_.fp32Factor) opt_.refineSweeps = 1;
  if (opt_.refineSweeps < 1) opt_.refineSweeps = 1;
  FG_CHECK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  SetupTrace trace;
  // the forked assembly is decided once the batch's object counts are known (below)
  forkAssembly_ = false;
  fuseBackward_ = false;
  const int nm = (int)models.size();
  // ---- global offsets --------------------------------------------------------
  modelTriOff_.assign(nm, 0);
  modelDofOff_.assign(nm, 0);
  modelEqOff_.assign(nm, 0);
  modelElOff_.assign(nm, 0);
  modelSlotOff_.assign(nm, 0);
  std::vector<int> frontOff(nm, 0);
  std::vector<int64_t> contribOff(nm, 0), eqContribOff(nm, 0), rowsOff(nm, 0), lOff(nm, 0), uOff(nm, 0),
      wOff(nm, 0), childOff(nm, 0), relOff(nm, 0), asmOff(nm, 0);
  int ntri = 0, ndof = 0, neq = 0, nel = 0, nfr = 0, nax = 0;
  std::vector<int> modelAxOff(nm, 0);
  std::vector<int64_t> mrXBase(nm, 0);  // start of each model's expanded matrices (parts, dependent triads)
  int64_t nslot = 0, ncontrib = 0, neqc = 0, nrows = 0, nl = 0, nu = 0, nw = 0, nch = 0, nrel = 0, nasm = 0,
          nxm = 0;
  bool anyC = false;
  for (int k = 0; k < nm; ++k) {
    const HostModel& h = *models[k];
    modelTriOff_[k] = ntri; modelDofOff_[k] = ndof; modelEqOff_[k] = neq; modelElOff_[k] = nel;
    modelAxOff[k] = nax;
    nax += h.nax;
    mrXBase[k] = nxm;
    nxm += h.cxMatSize;
    modelSlotOff_[k] = nslot; frontOff[k] = nfr; contribOff[k] = ncontrib; eqContribOff[k] = neqc;
    rowsOff[k] = nrows; lOff[k] = nl; uOff[k] = nu; wOff[k] = nw; childOff[k] = nch; relOff[k] = nrel;
    asmOff[k] = nasm;
    ntri += h.ntri; ndof += h.ndof; neq += h.neq; nel += h.nel; nfr += (int)h.fronts.size();
    nslot += (int64_t)h.colInd.size(); ncontrib += (int64_t)h.slotSrc.size(); neqc += (int64_t)h.eqSrc.size();
    nrows += (int64_t)h.frontRows.size(); nl += h.lSize; nu += h.uSize; nw += h.wSize;
    nch += (int64_t)h.childList.size(); nrel += (int64_t)h.relIndex.size(); nasm += (int64_t)h.asmSlot.size();
    for (uint8_t c : h.hasC) anyC |= c != 0;
  }
  if (12LL * nel + 6LL * nax > INT_MAX || neqc > INT_MAX) { err = "batch too large for 32-bit gather indices"; return -901; }
  d_.naxTot = nax;
  d_.ntriTot = ntri; d_.ndofTot = ndof; d_.neqTot = neq; d_.nelTot = nel; d_.nslotTot = nslot;
  d_.nfrontTot = nfr;
  trace.mark("offsets", stream_);
  // ---- per-model control -------------------------------------------------------
  DevModels& M = d_.m;
  M.n = nm;
  auto iv = [&](std::vector<int>& v) { v.assign(nm, 0); };
  std::vector<int> triOff(nm), ntriV(nm), dofOff(nm), ndofV(nm), eqOff(nm), neqV(nm), elOff(nm), nelV(nm);
  std::vector<double> tStart(nm), tEnd(nm), dt(nm), minInc(nm), alpha(nm), beta(nm), gamma(nm), wD(3 * nm),
      wF(3 * nm), grav(3 * nm), tolV(18 * nm), scaleN(3 * nm, -1.0), equTol(nm), equLim(nm), tQs(nm),
      sumWd2(nm, 0.0), sumWf2(nm, 0.0);
  std::vector<int> tolC(18 * nm), maxIt(nm), minIt(nm), fixedIt(nm), nUpdat(nm), maxSeq(nm), staticMode(nm),
      staticDone(nm);
  std::vector<long long> stepLimit(nm, LLONG_MAX);
  iv(maxIt);
  for (int k = 0; k < nm; ++k) {
    const HostModel& h = *models[k];
    const Control& c = h.ctl;
    triOff[k] = modelTriOff_[k]; ntriV[k] = h.ntri; dofOff[k] = modelDofOff_[k]; ndofV[k] = h.ndof;
    eqOff[k] = modelEqOff_[k]; neqV[k] = h.neq; elOff[k] = modelElOff_[k]; nelV[k] = h.nel;
    tStart[k] = c.tStart; tEnd[k] = c.tEnd; dt[k] = c.tInc; minInc[k] = c.minInc;
    alpha[k] = c.alpha; beta[k] = c.beta; gamma[k] = c.gamma;
    for (int q = 0; q < 3; ++q) { wD[3 * k + q] = c.wDisp[q]; wF[3 * k + q] = c.wForce[q]; grav[3 * k + q] = c.gravity[q]; }
    for (int q = 0; q < 18; ++q) { tolC[18 * k + q] = c.tolCode[q]; tolV[18 * k + q] = c.tolVal[q]; }
    maxIt[k] = c.maxIt; minIt[k] = c.minIt; fixedIt[k] = c.fixedIt; nUpdat[k] = c.nUpdat; maxSeq[k] = c.maxSeqNoUpdate;
    double eqTol = c.initEquilibrium ? c.tolInitEquil : 0.0, eqLim = c.initEquilibrium ? c.limInitEquilStep : 0.0;
    equTol[k] = eqTol; equLim[k] = eqLim;
    staticMode[k] = (eqLim > 0.0 && h.neq > 0) ? (eqTol > 0.0 ? 2 : 1) : 0;
    staticDone[k] = staticMode[k] == 0 ? 1 : 0;
    tQs[k] = c.tQStatic;
    // the norms' weight sums over the free DOFs (constant), in DOF order
    for (int i = 0; i < h.ndof; ++i)
      if (h.meqn[i] >= 0) {
        const int t = h.dofType[i] - 1;
        sumWd2[k] += c.wDisp[t] * c.wDisp[t];
        sumWf2[k] += c.wForce[t] * c.wForce[t];
      }
  }
#define UP_I(field, vec) if (!(M.field = alloc<int>(nm)) || put(M.field, vec, stream_) != cudaSuccess) { err = "alloc " #field; return -902; }
#define UP_D(field, vec, n) if (!(M.field = alloc<double>(n)) || put(M.field, vec, stream_) != cudaSuccess) { err = "alloc " #field; return -902; }
  UP_I(triOff, triOff); UP_I(ntri, ntriV); UP_I(dofOff, dofOff); UP_I(ndof, ndofV);
  UP_I(eqOff, eqOff); UP_I(neq, neqV); UP_I(elOff, elOff); UP_I(nel, nelV);
  UP_D(time, tStart, nm); UP_D(dt, dt, nm); UP_D(tStart, tStart, nm); UP_D(tEnd, tEnd, nm);
  UP_D(minInc, minInc, nm); UP_D(alpha, alpha, nm); UP_D(beta, beta, nm); UP_D(gamma, gamma, nm);
  UP_D(scaleN, scaleN, 3 * nm); UP_D(wDisp, wD, 3 * nm); UP_D(wForce, wF, 3 * nm); UP_D(gravity, grav, 3 * nm);
  UP_D(tolVal, tolV, 18 * nm); UP_D(equTol, equTol, nm); UP_D(equLim, equLim, nm); UP_D(tQs, tQs, nm);
  UP_D(sumWd2, sumWd2, nm); UP_D(sumWf2, sumWf2, nm);
  if (!(M.tolCode = alloc<int>(18 * nm)) || put(M.tolCode, tolC, stream_) != cudaSuccess) { err = "alloc tolCode"; return -902; }
  UP_I(maxIt, maxIt); UP_I(minIt, minIt); UP_I(fixedIt, fixedIt); UP_I(nUpdat, nUpdat); UP_I(maxSeq, maxSeq);
  UP_I(staticMode, staticMode); UP_I(staticDone, staticDone);
#undef UP_I
#undef UP_D
  M.sacc = alloc<double>(nm); M.svel = alloc<double>(nm); M.pc = alloc<double>(4 * nm);
  M.normVal = alloc<double>(18 * nm); M.deln = alloc<double>(nm); M.staticScale = alloc<double>(nm);
  M.state = alloc<int>(nm); M.flags = alloc<int>(nm); M.status = alloc<int>(nm); M.iter = alloc<int>(nm);
  M.nSeqNoUpd = alloc<int>(nm); M.negPiv = alloc<int>(nm); M.staticIter = alloc<int>(nm); M.staticNinc = alloc<int>(nm);
  M.nStep = alloc<long long>(nm); M.nIter = alloc<long long>(nm); M.stepLimit = alloc<long long>(nm);
  M.qsCount = alloc<int>(nm);
  if (put(M.stepLimit, stepLimit, stream_) != cudaSuccess) { err = "upload stepLimit"; return -902; }

  trace.mark("control", stream_);
  // ---- triads, DOFs, equations ---------------------------------------------------
  std::vector<double> ur(12 * (size_t)ntri), qext(neq);
  std::vector<int> triFirst(ntri), triNd(ntri), triModel(ntri), meqn(ndof), dofType(ndof), dofModel(ndof),
      eqModel(neq);
  for (int k = 0; k < nm; ++k)
    if (models[k]->ur.size() != 12 * (size_t)models[k]->ntri || models[k]->qext.size() != (size_t)models[k]->neq) {
      err = "inconsistent host model arrays";
      return -902;
    }
  forEachModel(nm, [&](int k) {
    const HostModel& h = *models[k];
    std::copy(h.ur.begin(), h.ur.end(), ur.begin() + 12 * (size_t)modelTriOff_[k]);
    for (int t = 0; t < h.ntri; ++t) {
      const int g = modelTriOff_[k] + t;
      triFirst[g] = h.triFirstDof[t] + modelDofOff_[k];
      triNd[g] = h.triNdof[t];
      triModel[g] = k;
    }
    for (int i = 0; i < h.ndof; ++i) {
      const int g = modelDofOff_[k] + i;
      meqn[g] = h.meqn[i] >= 0 ? h.meqn[i] + modelEqOff_[k] : h.meqn[i];
      dofType[g] = h.dofType[i];
      dofModel[g] = k;
    }
    for (int i = 0; i < h.neq; ++i) eqModel[modelEqOff_[k] + i] = k;
    std::copy(h.qext.begin(), h.qext.end(), qext.begin() + modelEqOff_[k]);
  });
  // external function channels of every model (values set by the caller, zero at start)
  modelExtOff_.assign(nm, 0);
  int nextTot = 0;
  for (int k = 0; k < nm; ++k) {
    modelExtOff_[k] = nextTot;
    nextTot += models[k]->nExt;
  }
  modelExtCnt_.resize(nm);
  std::vector<double> extInit(std::max(nextTot, 1), 0.0);
  for (int k = 0; k < nm; ++k) {
    modelExtCnt_[k] = models[k]->nExt;
    for (int c = 0; c < (int)models[k]->extInit.size() && c < models[k]->nExt; ++c)
      extInit[modelExtOff_[k] + c] = models[k]->extInit[c];
  }
  auto extAt = [&](int k, int ch) { return ch < (int)models[k]->extInit.size() ? models[k]->extInit[ch] : 0.0; };
  // engine-driven loads: constant part kept, start-time value in qext
  std::vector<double> qextBase = qext, ldF0, ldF1, ldEA, ldEB, ldSin;
  std::vector<int> ldEq, ldPtr(1, 0), ldCh;
  for (int k = 0; k < nm; ++k) {
    const HostModel& h = *models[k];
    for (size_t q = 0; q < h.ldEq.size(); ++q) {
      const int eq = h.ldEq[q] + modelEqOff_[k];
      ldEq.push_back(eq);
      double v = qextBase[eq];
      for (int j = h.ldPtr[q]; j < h.ldPtr[q + 1]; ++j) {
        ldF0.push_back(h.ldF0[j]); ldF1.push_back(h.ldF1[j]); ldEA.push_back(h.ldEA[j]); ldEB.push_back(h.ldEB[j]);
        const int ch = h.ldCh[j];
        ldCh.push_back(ch >= 0 ? ch + modelExtOff_[k] : -1);
        const double* sp = &h.ldSin[4 * (size_t)j];
        for (int q = 0; q < 4; ++q) ldSin.push_back(sp[q]);
        double ev = ch >= 0 ? extAt(k, ch) : h.ldEA[j] * h.ctl.tStart + h.ldEB[j];
        if (sp[2] != 0.0 || sp[3] != 0.0) ev += sp[3] + sp[2] * std::sin(2.0 * M_PI * (sp[0] * h.ctl.tStart - sp[1]));
        v += h.ldF0[j] + h.ldF1[j] * ev;
      }
      qext[eq] = v;
      ldPtr.push_back((int)ldF0.size());
    }
  }
#define UPV(ptr, T, vec) if (!(ptr = alloc<T>(vec.size())) || put(ptr, vec, stream_) != cudaSuccess) { err = "upload " #ptr; return -903; }
  UPV(d_.ur, double, ur);
  UPV(d_.triFirstDof, int, triFirst); UPV(d_.triNdof, int, triNd); UPV(d_.triModel, int, triModel);
  UPV(d_.meqn, int, meqn); UPV(d_.dofType, int, dofType); UPV(d_.dofModel, int, dofModel);
  UPV(d_.eqModel, int, eqModel); UPV(d_.qext, double, qext);
  d_.nldTot = (int)ldEq.size();
  UPV(d_.qextBase, double, qextBase); UPV(d_.ldEq, int, ldEq); UPV(d_.ldPtr, int, ldPtr);
  UPV(d_.ldF0, double, ldF0); UPV(d_.ldF1, double, ldF1); UPV(d_.ldEA, double, ldEA); UPV(d_.ldEB, double, ldEB);
  UPV(d_.ldCh, int, ldCh);
  UPV(d_.ldSin, double, ldSin);
  d_.nextTot = nextTot;
  UPV(d_.extVal, double, extInit);
  {
    // prescribed deflections and their predictor right-hand-side terms
    std::vector<int> motModel, motOff(nm), mrEq, mrMot, motCh;
    std::vector<double> d0, d1, eA, eB, D0;
    std::vector<int64_t> mrPtr(1, 0), mrSrc;
    bool anyLinearQs = false;
    for (int k = 0; k < nm; ++k) {
      const HostModel& h = *models[k];
      motOff[k] = (int)motModel.size();
      for (size_t j = 0; j < h.motD0.size(); ++j) {
        motModel.push_back(k);
        d0.push_back(h.motD0[j]); d1.push_back(h.motD1[j]); eA.push_back(h.motEA[j]); eB.push_back(h.motEB[j]);
        const int ch = h.motCh[j];
        motCh.push_back(ch >= 0 ? ch + modelExtOff_[k] : -1);
        // start-time value (updatePrescribedMotionsB, motionRoutinesModule.f90:213-245)
        D0.push_back(h.motD0[j] + h.motD1[j] * (ch >= 0 ? extAt(k, ch) : h.motEA[j] * h.ctl.tStart + h.motEB[j]));
      }
      for (size_t q = 0; q < h.mrEq.size(); ++q) {
        mrEq.push_back(h.mrEq[q] + modelEqOff_[k]);
        for (int t = h.mrPtr[q]; t < h.mrPtr[q + 1]; ++t) {
          const int src = h.mrSrc[t];
          if (src < 144 * h.nel) {
            const int e = src / 144, entry = src % 144;
            mrSrc.push_back((int64_t)entry * nel + e + modelElOff_[k]);
          } else if (src < 144 * h.nel + 36 * h.nax) {
            const int a = (src - 144 * h.nel) / 36, entry = (src - 144 * h.nel) % 36;
            mrSrc.push_back((int64_t)144 * nel + (int64_t)entry * nax + modelAxOff[k] + a);
          } else {  // the expanded matrix of a part (or of an element with a dependent triad)
            mrSrc.push_back((int64_t)144 * nel + 36LL * nax + mrXBase[k] + (src - 144 * h.nel - 36 * h.nax));
          }
          mrMot.push_back(h.mrMot[t] + motOff[k]);
        }
        mrPtr.push_back((int64_t)mrSrc.size());
      }
      anyLinearQs |= h.ctl.tQStatic > h.ctl.tStart && h.ctl.fixedIt == -1;
    }
    d_.nmotTot = (int)motModel.size();
    d_.nmrTot = (int)mrEq.size();
    UPV(d_.motModel, int, motModel); UPV(d_.modelMotOff, int, motOff);
    UPV(d_.motD0, double, d0); UPV(d_.motD1, double, d1); UPV(d_.motEA, double, eA); UPV(d_.motEB, double, eB);
    UPV(d_.motD, double, D0);
    UPV(d_.motCh, int, motCh);
    d_.motCc = alloc<double>(motModel.size());
    UPV(d_.mrEq, int, mrEq); UPV(d_.mrMot, int, mrMot); UPV(d_.mrPtr, int64_t, mrPtr); UPV(d_.mrSrc, int64_t, mrSrc);
    d_.linearIters = opt_.fp32Factor ? 3 : 1;
    d_.sinEpsOverEps = std::sin(0.0005) / 0.0005;
    if (anyLinearQs) {
      d_.urQs = alloc<double>(12 * (size_t)ntri); d_.supTrQs = alloc<double>(12 * (size_t)nel);
      d_.urdQs = alloc<double>(ndof); d_.urddQs = alloc<double>(ndof);
    }
  }
  d_.urd = alloc<double>(ndof); d_.urdd = alloc<double>(ndof); d_.dk = alloc<double>(ndof); d_.ak = alloc<double>(ndof);
  d_.rinc = alloc<double>(ndof); d_.sinc0 = alloc<double>(ndof); d_.sinc1 = alloc<double>(ndof); d_.sinc2 = alloc<double>(ndof);
  d_.FSk = alloc<double>(neq); d_.FDk = alloc<double>(neq); d_.FIk = alloc<double>(neq); d_.Qk = alloc<double>(neq);
  d_.FIact = alloc<double>(neq); d_.res = alloc<double>(neq); d_.del = alloc<double>(neq);
  d_.extRhs = alloc<double>(neq);
  d_.x64 = alloc<double>(neq); d_.xref = alloc<double>(neq); d_.rref = alloc<double>(neq); d_.x32 = alloc<float>(neq);
  {
    // DOF chunks of at most 2048 DOFs (eight per thread of a 256-thread block;
    // 1024 and 4096 were measured slower), each inside one model
    const int CH = 2048;
    std::vector<int> cm, cs, ce, mco(nm), mnc(nm);
    for (int k = 0; k < nm; ++k) {
      mco[k] = (int)cm.size();
      const int d0 = modelDofOff_[k], nd = models[k]->ndof;
      for (int s = 0; s < nd; s += CH) {
        cm.push_back(k);
        cs.push_back(d0 + s);
        ce.push_back(d0 + std::min(nd, s + CH));
      }
      mnc[k] = (int)cm.size() - mco[k];
    }
    d_.nchunkTot = (int)cm.size();
    UPV(d_.chunkModel, int, cm); UPV(d_.chunkStart, int, cs); UPV(d_.chunkEnd, int, ce);
    UPV(d_.modelChunkOff, int, mco); UPV(d_.modelNchunk, int, mnc);
    normChunkOff_ = mco;
    normChunkCnt_ = mnc;
    d_.partial = alloc<double>(21 * (size_t)std::max(1, d_.nchunkTot));
  }
  d_.rhs32 = nullptr;

  trace.mark("triads, DOFs, norms", stream_);
  // ---- elements (SoA) -------------------------------------------------------------
  auto soa = [&](int width, auto getter) {
    std::vector<double> v((size_t)width * nel);
    forEachModel(nm, [&](int k) {
      const HostModel& h = *models[k];
      for (int c = 0; c < width; ++c)
        for (int e = 0; e < h.nel; ++e) v[(size_t)c * nel + modelElOff_[k] + e] = getter(h, e, c);
    });
    return v;
  };
  {
    auto fg = soa(36, [](const HostModel& h, int e, int c) { return h.fg[36 * (size_t)e + c]; });
    UPV(d_.fg, double, fg);
    auto S = soa(12, [](const HostModel& h, int e, int c) { return h.supTr[12 * (size_t)e + c]; });
    UPV(d_.supTr, double, S);
    auto R = soa(12, [](const HostModel& h, int e, int c) { return h.triRelSup[12 * (size_t)e + c]; });
    UPV(d_.triRelSup, double, R);
    auto T = soa(24, [](const HostModel& h, int e, int c) { return h.trUnd[24 * (size_t)e + c]; });
    UPV(d_.trUnd, double, T);
    auto O = soa(9, [](const HostModel& h, int e, int c) { return h.elOffset[9 * (size_t)e + c]; });
    UPV(d_.offset, double, O);
  }
  {
    // principal-axes beam pattern: 26 upper-triangle pairs (row, col), 0-based
    static const int pat[26][2] = {{0, 0}, {0, 6},  {1, 1},  {1, 5},  {1, 7},   {1, 11},  {2, 2},
                                   {2, 4}, {2, 8},  {2, 10}, {3, 3},  {3, 9},   {4, 4},   {4, 8},
                                   {4, 10}, {5, 5}, {5, 7},  {5, 11}, {6, 6},   {7, 7},   {7, 11},
                                   {8, 8}, {8, 10}, {9, 9},  {10, 10}, {11, 11}};
    bool inPat[144] = {false};
    for (auto& p : pat) inPat[p[0] + 12 * p[1]] = inPat[p[1] + 12 * p[0]] = true;
    std::vector<uint8_t> modelSparse(nm, 1);
    if (opt_.compressBeams)
      forEachModel(nm, [&](int k) {
        const HostModel& h = *models[k];
        for (int e = 0; e < h.nel && modelSparse[k]; ++e)
          for (int q = 0; q < 144; ++q) {
            if (inPat[q]) continue;
            if (h.K[144 * (size_t)e + q] != 0.0 || h.M[144 * (size_t)e + q] != 0.0 ||
                (h.hasC[e] && h.C[144 * (size_t)e + q] != 0.0)) {
              modelSparse[k] = 0;
              break;
            }
          }
      });
    bool sparse = opt_.compressBeams;
    for (int k = 0; k < nm; ++k) sparse = sparse && modelSparse[k];
    d_.beamSparse = sparse ? 1 : 0;
    if (sparse) {
      auto pack = [&](const std::vector<double> HostModel::*mat) {
        std::vector<double> v((size_t)26 * nel);
        forEachModel(nm, [&](int k) {
          const HostModel& h = *models[k];
          const std::vector<double>& src = h.*mat;
          for (int q = 0; q < 26; ++q)
            for (int e = 0; e < h.nel; ++e)
              v[(size_t)q * nel + modelElOff_[k] + e] = src[144 * (size_t)e + pat[q][0] + 12 * pat[q][1]];
        });
        return v;
      };
      auto K26 = pack(&HostModel::K);
      UPV(d_.K26, double, K26);
      auto M26 = pack(&HostModel::M);
      UPV(d_.M26, double, M26);
      if (anyC) {
        auto C26 = pack(&HostModel::C);
        UPV(d_.C26, double, C26);
      } else {
        d_.C26 = alloc<double>(1);
      }
    }
  }
  // full 12x12 matrices: read on the device only by batches that are not compressed
  if (!d_.beamSparse) {
    {
      auto K = soa(144, [](const HostModel& h, int e, int c) { return h.K[144 * (size_t)e + c]; });
      UPV(d_.K, double, K);
    }
    {
      auto Mm = soa(144, [](const HostModel& h, int e, int c) { return h.M[144 * (size_t)e + c]; });
      UPV(d_.M, double, Mm);
    }
    if (anyC) {
      auto C = soa(144, [](const HostModel& h, int e, int c) { return h.C[144 * (size_t)e + c]; });
      UPV(d_.C, double, C);
    } else {
      d_.C = alloc<double>(1);
    }
    d_.N = alloc<double>(144 * (size_t)nel);
  } else {
    d_.K = alloc<double>(1);
    d_.M = alloc<double>(1);
    d_.C = alloc<double>(1);
    d_.N = alloc<double>(1);
  }
  d_.elMat = alloc<double>(144 * (size_t)nel);
  d_.finit = alloc<double>(12 * (size_t)nel);
  d_.finitPrev = alloc<double>(12 * (size_t)nel);
  d_.Fel = alloc<double>(48 * (size_t)nel);
  {
    std::vector<int> elTri(2 * (size_t)nel), elRef(3 * (size_t)nel), elModel(nel);
    std::vector<double> ss(nel), kd(nel);
    std::vector<uint8_t> hc(nel), hv(nel);
    forEachModel(nm, [&](int k) {
      const HostModel& h = *models[k];
      for (int e = 0; e < h.nel; ++e) {
        int g = modelElOff_[k] + e;
        for (int n = 0; n < 2; ++n) elTri[(size_t)n * nel + g] = h.elTri[2 * e + n] + modelTriOff_[k];
        for (int j = 0; j < 3; ++j) elRef[(size_t)j * nel + g] = h.elRef[3 * e + j];
        elModel[g] = k;
        ss[g] = h.stifScl[e];
        kd[g] = h.kDmp[e];
        hc[g] = h.hasC[e];
        hv[g] = h.hasVld[e];
      }
    });
    UPV(d_.elTri, int, elTri); UPV(d_.elRef, int, elRef); UPV(d_.elModel, int, elModel);
    UPV(d_.stifScl, double, ss); UPV(d_.kDmp, double, kd); UPV(d_.hasC, uint8_t, hc); UPV(d_.hasVld, uint8_t, hv);
  }
  trace.mark("elements", stream_);
  // ---- axial springs and dampers ------------------------------------------------------
  {
    std::vector<uint8_t> kind(nax);
    std::vector<int> tri(2 * (size_t)nax), axModel(nax);
    std::vector<double> s0(nax), l0(nax), al(nax), d0(nax);
    for (int k = 0; k < nm; ++k) {
      const HostModel& h = *models[k];
      for (int a = 0; a < h.nax; ++a) {
        const int g = modelAxOff[k] + a;
        kind[g] = h.axKind[a];
        for (int n = 0; n < 2; ++n) tri[(size_t)n * nax + g] = h.axTri[2 * a + n] + modelTriOff_[k];
        axModel[g] = k;
        s0[g] = h.axS0[a]; l0[g] = h.axL0[a]; al[g] = h.axAlpha2[a]; d0[g] = h.axD0[a];
      }
    }
    UPV(d_.axKind, uint8_t, kind); UPV(d_.axTri, int, tri); UPV(d_.axModel, int, axModel);
    UPV(d_.axS0, double, s0); UPV(d_.axL0, double, l0); UPV(d_.axAlpha2, double, al); UPV(d_.axD0, double, d0);
    d_.axN = alloc<double>(3 * (size_t)nax);
    d_.axLen = alloc<double>(nax);
    d_.FelA = alloc<double>(12 * (size_t)nax);
    d_.elMatA = alloc<double>(36 * (size_t)nax);
  }
  trace.mark("axial elements", stream_);
  // ---- master-slave joints and the elements holding a dependent triad ---------------------
  std::vector<int> modelJointOff(nm, 0), modelCxOff(nm, 0);
  std::vector<int64_t> cxMatBase(nm, 0), cxVecBase(nm, 0);
  {
    int nj = 0, ncx = 0;
    int64_t xm = 0, xv = 0;
    for (int k = 0; k < nm; ++k) {
      const HostModel& h = *models[k];
      modelJointOff[k] = nj;
      modelCxOff[k] = ncx;
      cxMatBase[k] = xm;
      cxVecBase[k] = xv;
      nj += h.njoint;
      ncx += (int)h.cxEl.size();
      xm += h.cxMatSize;
      xv += h.cxVecSize;
    }
    d_.njointTot = nj;
    d_.ncxTot = ncx;
    if (nj > 0) {
      std::vector<int> jS, jM, jNM, jNc, jF, jNd, jNmat, jOff, jMod, jL, jI, jCE, dep(ndof, -1), cEl, cNx, cMO, cVO,
          cNode;
      std::vector<double> jV, jPT, jS0;
      for (int k = 0; k < nm; ++k) {
        const HostModel& h = *models[k];
        for (int j = 0; j < h.njoint; ++j) {
          jS.push_back(h.jSlave[j] + modelTriOff_[k]);
          jM.push_back(h.jMaster[j] + modelTriOff_[k]);
          jNM.push_back(h.jNM[j]);
          jNc.push_back(h.jNM[j] + h.jNdof[j]);
          jF.push_back(h.jFirstDof[j] + modelDofOff_[k]);
          jNd.push_back(h.jNdof[j]);
          jNmat.push_back(h.jNmats[j]);
          jOff.push_back((int)jL.size());
          jMod.push_back(k);
          for (int q = h.jDofOff[j]; q < h.jDofOff[j + 1]; ++q) {
            jL.push_back(h.jLdof[q]);
            jI.push_back(h.jImat[q]);
            jV.push_back(h.jVar0[q]);
          }
          for (int q = 0; q < 12; ++q) {
            jPT.push_back(h.jPosInT[12 * j + q]);
            jS0.push_back(h.jSTPos0[12 * j + q]);
            const int e = h.jColEq[12 * j + q];
            jCE.push_back(e >= 0 ? e + modelEqOff_[k] : -1);
          }
        }
        for (int i = 0; i < h.ndof; ++i)
          if (h.dofDep[i] >= 0) dep[modelDofOff_[k] + i] = h.dofDep[i] + 6 * modelJointOff[k];
        for (size_t c = 0; c < h.cxEl.size(); ++c) {
          const int e = h.cxEl[c];
          cEl.push_back(e + modelElOff_[k]);
          cNx.push_back(h.cxNx[c]);
          cMO.push_back((int)(cxMatBase[k] + h.cxMatOff[c]));
          cVO.push_back((int)(cxVecBase[k] + h.cxVecOff[c]));
          for (int n = 0; n < 2; ++n) {
            const int dd = h.dofDep[h.triFirstDof[h.elTri[2 * e + n]]];
            cNode.push_back(dd >= 0 ? dd / 6 + modelJointOff[k] : -1);
          }
        }
      }
      UPV(d_.jSlave, int, jS); UPV(d_.jMaster, int, jM); UPV(d_.jNM, int, jNM); UPV(d_.jNcol, int, jNc);
      UPV(d_.jFirstDof, int, jF); UPV(d_.jNdof, int, jNd); UPV(d_.jNmats, int, jNmat); UPV(d_.jDofOff, int, jOff);
      UPV(d_.jModel, int, jMod); UPV(d_.jLdof, int, jL); UPV(d_.jImat, int, jI); UPV(d_.jVar, double, jV);
      UPV(d_.jPosInT, double, jPT); UPV(d_.jSTPos0, double, jS0); UPV(d_.jColEq, int, jCE);
      UPV(d_.dofDep, int, dep);
      d_.jT = alloc<double>(72 * (size_t)nj);
      UPV(d_.cxEl, int, cEl); UPV(d_.cxNx, int, cNx); UPV(d_.cxMatOff, int, cMO); UPV(d_.cxVecOff, int, cVO);
      UPV(d_.cxNode, int, cNode);
    }
    if (xm >= INT_MAX / 2 || xv >= INT_MAX / 2) { err = "too many expanded element entries"; return -901; }
    if (xm > 0 || xv > 0) {
      d_.elMatX = alloc<double>((size_t)std::max<int64_t>(xm, 1));
      d_.FelX = alloc<double>((size_t)std::max<int64_t>(xv, 1));
    }
  }
  trace.mark("joints", stream_);
  // ---- reduced parts -------------------------------------------------------------------
  {
    int np = 0;
    for (int k = 0; k < nm; ++k) np += models[k]->npart;
    d_.npartTot = np;
    if (np > 0) {
      std::vector<int> pModel, pN, pNtri, pNgen, pTriOff, pTri, pTriJoint, pRef, pGenFirst, pGenOff, pVecOff, pNx,
          pXMat, pXVec;
      std::vector<int64_t> pMatOff;
      std::vector<double> pOffset, pSupTr, pRel, pTrUnd, pK, pM, pC, pFg, pSs, pKd, pGen;
      std::vector<uint8_t> pHasC, pHasVld;
      int64_t vecBase = 0, matBase = 0;
      int genBase = 0;
      for (int k = 0; k < nm; ++k) {
        const HostModel& h = *models[k];
        for (int p = 0; p < h.npart; ++p) {
          const int n = 6 * h.pNtri[p] + h.pNgen[p];
          pModel.push_back(k);
          pN.push_back(n);
          pNtri.push_back(h.pNtri[p]);
          pNgen.push_back(h.pNgen[p]);
          pTriOff.push_back((int)pTri.size());
          for (int t = 0; t < h.pNtri[p]; ++t) {
            const int tri = h.pTri[h.pTriOff[p] + t];
            pTri.push_back(tri + modelTriOff_[k]);
            const int dd = h.dofDep[h.triFirstDof[tri]];
            pTriJoint.push_back(dd >= 0 ? dd / 6 + modelJointOff[k] : -1);
            for (int q = 0; q < 12; ++q) pTrUnd.push_back(h.pTrUnd[12 * (size_t)(h.pTriOff[p] + t) + q]);
          }
          for (int j = 0; j < 3; ++j) pRef.push_back(h.pRef[3 * p + j]);
          for (int q = 0; q < 9; ++q) pOffset.push_back(h.pOffset[9 * (size_t)p + q]);
          for (int q = 0; q < 12; ++q) {
            pSupTr.push_back(h.pSupTr[12 * (size_t)p + q]);
            pRel.push_back(h.pTriRelSup[12 * (size_t)p + q]);
          }
          pGenFirst.push_back(h.pGenFirstDof[p] + modelDofOff_[k]);
          pGenOff.push_back(genBase + h.pGenOff[p]);
          pVecOff.push_back((int)(vecBase + h.pVecOff[p]));
          pMatOff.push_back(matBase + h.pMatOff[p]);
          pNx.push_back(h.pNx[p]);
          pXMat.push_back((int)(cxMatBase[k] + h.pXMatOff[p]));
          pXVec.push_back((int)(cxVecBase[k] + h.pXVecOff[p]));
          pSs.push_back(h.pStifScl[p]);
          pKd.push_back(h.pKDmp[p]);
          pHasC.push_back(h.pHasC[p]);
          pHasVld.push_back(h.pHasVld[p]);
          d_.partMaxN = std::max(d_.partMaxN, n);
          d_.partMaxNx = std::max(d_.partMaxNx, h.pNx[p]);
        }
        pK.insert(pK.end(), h.pK.begin(), h.pK.end());
        pM.insert(pM.end(), h.pM.begin(), h.pM.end());
        pC.insert(pC.end(), h.pC.begin(), h.pC.end());
        pFg.insert(pFg.end(), h.pFg.begin(), h.pFg.end());
        int ngen = 0, nvec = 0;
        for (int p = 0; p < h.npart; ++p) {
          ngen += h.pNgen[p];
          nvec += 6 * h.pNtri[p] + h.pNgen[p];
        }
        genBase += ngen;
        vecBase += nvec;
        matBase += (int64_t)h.pK.size();
      }
      pGen.assign(genBase, 0.0);
      partVecTot_ = (size_t)vecBase;
      if (sizeof(double) * ((size_t)d_.partMaxN * std::max(d_.partMaxN, d_.partMaxNx) +
                            (size_t)d_.partMaxN * d_.partMaxN) > 200 * 1024) {
        err = "a part's expanded Newton matrix does not fit in shared memory";
        return -905;
      }
      UPV(d_.pModel, int, pModel); UPV(d_.pN, int, pN); UPV(d_.pNtri, int, pNtri); UPV(d_.pNgen, int, pNgen);
      UPV(d_.pTriOff, int, pTriOff); UPV(d_.pTri, int, pTri); UPV(d_.pTriJoint, int, pTriJoint);
      UPV(d_.pRef, int, pRef); UPV(d_.pGenFirstDof, int, pGenFirst); UPV(d_.pGenOff, int, pGenOff);
      UPV(d_.pVecOff, int, pVecOff); UPV(d_.pNx, int, pNx); UPV(d_.pXMatOff, int, pXMat);
      UPV(d_.pXVecOff, int, pXVec); UPV(d_.pMatOff, int64_t, pMatOff);
      UPV(d_.pOffset, double, pOffset); UPV(d_.pSupTr, double, pSupTr); UPV(d_.pTriRelSup, double, pRel);
      UPV(d_.pTrUnd, double, pTrUnd); UPV(d_.pK, double, pK); UPV(d_.pM, double, pM); UPV(d_.pC, double, pC);
      UPV(d_.pFg, double, pFg); UPV(d_.pStifScl, double, pSs); UPV(d_.pKDmp, double, pKd);
      UPV(d_.pHasC, uint8_t, pHasC); UPV(d_.pHasVld, uint8_t, pHasVld); UPV(d_.pGen, double, pGen);
      d_.pFinit = alloc<double>((size_t)std::max<int64_t>(vecBase, 1));
      d_.pFinitPrev = alloc<double>((size_t)std::max<int64_t>(vecBase, 1));
      cudaMemsetAsync(d_.pFinit, 0, sizeof(double) * (size_t)std::max<int64_t>(vecBase, 1), stream_);
      cudaMemsetAsync(d_.pFinitPrev, 0, sizeof(double) * (size_t)std::max<int64_t>(vecBase, 1), stream_);
      if (preparePartKernels(d_) != 0) { err = "part kernels: shared memory"; return -905; }
    }
  }
  trace.mark("parts", stream_);
  // ---- CSR and gather maps -----------------------------------------------------------
  {
    if (ncontrib >= INT_MAX || 144LL * nel + 36LL * nax >= INT_MAX) {
      err = "batch too large for 32-bit CSR gather lists";
      return -901;
    }
    std::vector<int64_t> rowPtr(neq + 1, 0);
    std::vector<int> slotPtr(nslot + 1, 0), slotSrc(ncontrib);
    std::vector<int> colInd(nslot), slotModel(nslot), eqPtr(neq + 1, 0), eqSrc(neqc);
    forEachModel(nm, [&](int k) {
      const HostModel& h = *models[k];
      for (int i = 0; i < h.neq; ++i) {
        rowPtr[modelEqOff_[k] + i + 1] = modelSlotOff_[k] + h.rowPtr[i + 1];
        eqPtr[modelEqOff_[k] + i + 1] = (int)(eqContribOff[k] + h.eqPtr[i + 1]);
      }
      const int64_t s0 = modelSlotOff_[k];
      for (size_t s = 0; s < h.colInd.size(); ++s) {
        colInd[s0 + s] = h.colInd[s] + modelEqOff_[k];
        slotModel[s0 + s] = k;
        slotPtr[s0 + s + 1] = (int)(contribOff[k] + h.slotPtr[s + 1]);
      }
      int64_t o = contribOff[k];
      const int hx = 144 * h.nel + 36 * h.nax, hv = 12 * h.nel + 6 * h.nax;
      for (int src : h.slotSrc) {
        if (src < 144 * h.nel) {
          int e = src / 144, entry = src % 144;
          slotSrc[o++] = entry * nel + modelElOff_[k] + e;
        } else if (src < hx) {  // axial element entry
          int a = (src - 144 * h.nel) / 36, entry = (src - 144 * h.nel) % 36;
          slotSrc[o++] = 144 * nel + entry * nax + modelAxOff[k] + a;
        } else {  // expanded matrix of an element with a dependent triad
          slotSrc[o++] = (int)(144LL * nel + 36LL * nax + cxMatBase[k] + (src - hx));
        }
      }
      o = eqContribOff[k];
      for (int src : h.eqSrc) {
        if (src < 12 * h.nel) {
          int e = src / 12, loc = src % 12;
          eqSrc[o++] = loc * nel + modelElOff_[k] + e;
        } else if (src < hv) {
          int a = (src - 12 * h.nel) / 6, loc = (src - 12 * h.nel) % 6;
          eqSrc[o++] = 12 * nel + loc * nax + modelAxOff[k] + a;
        } else {  // expanded forces of an element with a dependent triad
          eqSrc[o++] = (int)(12LL * nel + 6LL * nax + cxVecBase[k] + (src - hv));
        }
      }
    });
    UPV(d_.rowPtr, int64_t, rowPtr); UPV(d_.colInd, int, colInd); UPV(d_.slotPtr, int, slotPtr);
    UPV(d_.slotSrc, int, slotSrc); UPV(d_.slotModel, int, slotModel); UPV(d_.eqPtr, int, eqPtr);
    {
      std::vector<int> blockModel((nslot + kSlotBlock - 1) / kSlotBlock, -1);
      for (size_t b = 0; b < blockModel.size(); ++b) {
        const int64_t s0 = (int64_t)b * kSlotBlock, s1 = std::min<int64_t>(nslot, s0 + kSlotBlock) - 1;
        blockModel[b] = slotModel[s0] == slotModel[s1] ? slotModel[s0] : -1;
      }
      UPV(d_.slotBlockModel, int, blockModel);
    }
    UPV(d_.eqSrc, int, eqSrc);
    d_.csrVal = alloc<double>(nslot);
  }
  trace.mark("CSR and gather maps", stream_);
  // ---- fronts ------------------------------------------------------------------------------
  {
    std::vector<int> npiv(nfr), nrow(nfr), parent(nfr), fmodel(nfr), nchild(nfr), nasmv(nfr), frontRows(nrows),
        childList(nch), relIndex(nrel), asmPos(nasm);
    std::vector<int64_t> rowOffV(nfr), lOffV(nfr), uOffV(nfr), wOffV(nfr), childOffV(nfr), relOffV(nfr),
        asmOffV(nfr), asmSlot(nasm);
    forEachModel(nm, [&](int k) {
      const HostModel& h = *models[k];
      for (size_t f = 0; f < h.fronts.size(); ++f) {
        const Front& fr = h.fronts[f];
        const size_t g = frontOff[k] + f;
        npiv[g] = fr.npiv;
        nrow[g] = fr.nrow;
        parent[g] = fr.parent >= 0 ? fr.parent + frontOff[k] : -1;
        fmodel[g] = k;
        nchild[g] = fr.nchild;
        nasmv[g] = fr.nasm;
        rowOffV[g] = fr.rowOff + rowsOff[k];
        lOffV[g] = fr.lOff + lOff[k];
        uOffV[g] = fr.uOff + uOff[k];
        wOffV[g] = fr.wOff + wOff[k];
        childOffV[g] = fr.childOff + childOff[k];
        relOffV[g] = fr.relOff + relOff[k];
        asmOffV[g] = fr.asmOff + asmOff[k];
      }
      for (size_t i = 0; i < h.frontRows.size(); ++i) frontRows[rowsOff[k] + i] = h.frontRows[i] + modelEqOff_[k];
      for (size_t i = 0; i < h.childList.size(); ++i) childList[childOff[k] + i] = h.childList[i] + frontOff[k];
      std::copy(h.relIndex.begin(), h.relIndex.end(), relIndex.begin() + relOff[k]);
      for (size_t i = 0; i < h.asmSlot.size(); ++i) asmSlot[asmOff[k] + i] = (int64_t)h.asmSlot[i] + modelSlotOff_[k];
      std::copy(h.asmPos.begin(), h.asmPos.end(), asmPos.begin() + asmOff[k]);
    });
    // children's update matrices: lower triangles packed column by column into one
    // segment per parent, children in order, with their positions in the parent front
    std::vector<int64_t> segOff(nfr, 0), uOffPacked(nfr, 0);
    std::vector<int> segLen(nfr, 0);
    int64_t nuPacked = 0;
    for (int f = 0; f < nfr; ++f) {
      segOff[f] = nuPacked;
      if (nrow[f] > 1024 || nchild[f] >= 2048) { err = "front too large for the packed update layout"; return -909; }
      for (int c = 0; c < nchild[f]; ++c) {
        const int ch = childList[childOffV[f] + c];
        const int64_t cu = nrow[ch] - npiv[ch];
        uOffPacked[ch] = nuPacked;
        nuPacked += cu * (cu + 1) / 2;
      }
      segLen[f] = (int)(nuPacked - segOff[f]);
    }
    // positions of the packed entries in their parent front, filled per model
    std::vector<int> segPos(nuPacked);
    forEachModel(nm, [&](int k) {
      const int fEnd = k + 1 < nm ? frontOff[k + 1] : nfr;
      for (int f = frontOff[k]; f < fEnd; ++f) {
        int64_t o = segOff[f];
        for (int c = 0; c < nchild[f]; ++c) {
          const int ch = childList[childOffV[f] + c];
          const int cu = nrow[ch] - npiv[ch];
          const int* rel = &relIndex[relOffV[ch]];
          for (int b = 0; b < cu; ++b)
            for (int a = b; a < cu; ++a) segPos[o++] = (c << 20) | (rel[a] + nrow[f] * rel[b]);
        }
      }
    });
    nu = nuPacked;
    uOffV = uOffPacked;
    pplan_.maxSeg = 1;
    pplan_.maxAsm = 1;
    for (int f = 0; f < nfr; ++f) {
      pplan_.maxSeg = std::max(pplan_.maxSeg, segLen[f]);
      pplan_.maxAsm = std::max(pplan_.maxAsm, nasmv[f]);
    }
    // algorithmic bytes of the factorisation fused with the first forward
    // elimination, per front (E: factor precision): original entries and their
    // positions, children's update matrices and positions in, L and the packed
    // update matrix out; pivot rows' indices and right-hand side (FP64) in,
    // children's update vectors with their gather entries in, pivot solution
    // and update vector out
    {
      const double E = opt_.fp32Factor ? 4.0 : 8.0;
      factorBytes_ = 0.0;
      for (int f = 0; f < nfr; ++f) {
        const double nr = nrow[f], np = npiv[f], nuf = nr - np;
        double ncg = 0.0;
        for (int c = 0; c < nchild[f]; ++c) {
          const int ch = childList[childOffV[f] + c];
          ncg += nrow[ch] - npiv[ch];
        }
        factorBytes_ += nasmv[f] * (4.0 + E) + segLen[f] * (4.0 + E) + E * nr * np + E * nuf * (nuf + 1.0) / 2.0 +
                        np * (4.0 + 8.0 + E) + ncg * (8.0 + E) + E * nuf;
      }
    }
    UPV(d_.fSegOff, int64_t, segOff); UPV(d_.fSegLen, int, segLen); UPV(d_.segPos, int, segPos);
    {
      std::vector<int> slotAsm(nslot, -1);
      for (size_t k = 0; k < asmSlot.size(); ++k) slotAsm[asmSlot[k]] = (int)k;
      if ((int64_t)asmSlot.size() >= INT_MAX) { err = "batch too large for 32-bit assembly indices"; return -908; }
      UPV(d_.slotAsm, int, slotAsm);
      if (opt_.fp32Factor) d_.asmVal32 = alloc<float>(asmSlot.size());
      else d_.asmVal64 = alloc<double>(asmSlot.size());
    }
    UPV(d_.fNpiv, int, npiv); UPV(d_.fNrow, int, nrow); UPV(d_.fParent, int, parent); UPV(d_.fModel, int, fmodel);
    UPV(d_.fNchild, int, nchild); UPV(d_.fNasm, int, nasmv);
    UPV(d_.fRowOff, int64_t, rowOffV); UPV(d_.fLOff, int64_t, lOffV); UPV(d_.fUOff, int64_t, uOffV);
    UPV(d_.fWOff, int64_t, wOffV); UPV(d_.fChildOff, int64_t, childOffV); UPV(d_.fRelOff, int64_t, relOffV);
    UPV(d_.fAsmOff, int64_t, asmOffV);
    UPV(d_.frontRows, int, frontRows); UPV(d_.childList, int, childList); UPV(d_.relIndex, int, relIndex);
    UPV(d_.asmSlot, int64_t, asmSlot); UPV(d_.asmPos, int, asmPos);
    trace.mark("front structure", stream_);
    {
      // per-front list of the children's update rows: W source index and (child
      // ordinal << 16 | row in this front), children in order
      std::vector<int> cgOff(nfr + 1, 0), cgSrc, cgDst;
      for (int f = 0; f < nfr; ++f) {
        for (int c = 0; c < nchild[f]; ++c) {
          const int ch = childList[childOffV[f] + c];
          const int cu = nrow[ch] - npiv[ch];
          for (int a = 0; a < cu; ++a) {
            cgSrc.push_back((int)(wOffV[ch] + a));
            cgDst.push_back((c << 16) | relIndex[relOffV[ch] + a]);
          }
        }
        cgOff[f + 1] = (int)cgSrc.size();
      }
      if (nw >= INT_MAX) { err = "batch too large for 32-bit update-vector indices"; return -908; }
      UPV(d_.cgOff, int, cgOff); UPV(d_.cgSrc, int, cgSrc); UPV(d_.cgDst, int, cgDst);
    }
    if (opt_.fp32Factor) {
      d_.L32 = alloc<float>(nl); d_.U32 = alloc<float>(nu); d_.w32 = alloc<float>(nw);
      if (!d_.L32 || !d_.U32 || !d_.w32) { err = "out of device memory (factor)"; return -904; }
    } else {
      d_.L64 = alloc<double>(nl); d_.U64 = alloc<double>(nu); d_.w64 = alloc<double>(nw);
      if (!d_.L64 || !d_.U64 || !d_.w64) { err = "out of device memory (factor)"; return -904; }
    }
    // large fronts (more than kLargeFrontRows rows) and all their ancestors go to
    // the block-per-front kernels; the warp kernels size their shared memory by
    // the small fronts only
    std::vector<unsigned char> large(nfr, 0);
    std::vector<int> nLargeChild(nfr, 0);
    for (int f = 0; f < nfr; ++f) {
      if (nrow[f] > kLargeFrontRows) large[f] = 1;
      if (large[f] && parent[f] >= 0) large[parent[f]] = 1;  // parents follow their children
    }
    int maxRowAll = 1, maxRowLarge = 0, nLargeFronts = 0;
    for (int f = 0; f < nfr; ++f) {
      if (large[f]) {
        maxRowLarge = std::max(maxRowLarge, nrow[f]);
        ++nLargeFronts;
        if (parent[f] >= 0) ++nLargeChild[parent[f]];
      } else {
        maxRowAll = std::max(maxRowAll, nrow[f]);
      }
    }
    if (((size_t)maxRowAll * maxRowAll + 3 * maxRowAll) * (opt_.fp32Factor ? 4 : 8) > 200 * 1024) {
      err = "front too large for the shared-memory front kernels";
      return -905;
    }
    if (maxRowLarge >= 1024) { err = "front of 1024 rows or more"; return -905; }
    UPV(d_.fLarge, uint8_t, large);
    UPV(d_.fNlarge, int, nLargeChild);
    pplan_.fLarge = d_.fLarge;
    pplan_.fNlarge = d_.fNlarge;
    pplan_.maxRowLarge = maxRowLarge;
    // leaf-to-root path lengths: parents follow their children in each model's order
    std::vector<int> pathLen(nfr, 1);
    for (int f = nfr - 1; f >= 0; --f) {
      if (parent[f] > f) pathLen[f] = pathLen[parent[f]] + 1;
      else if (parent[f] >= 0) { err = "assembly tree not in post-order"; return -907; }
    }
    // tasks with the longest paths first: the cascades' critical paths (the
    // deep trees of the large models) start in the first wave of warps
    std::vector<int> leaves, largeTasks;
    for (int f = 0; f < nfr; ++f) {
      if (nchild[f] == 0 && !large[f]) leaves.push_back(f);
      if (large[f] && nLargeChild[f] == 0) largeTasks.push_back(f);
    }
    std::stable_sort(leaves.begin(), leaves.end(), [&](int a, int b) { return pathLen[a] > pathLen[b]; });
    std::stable_sort(largeTasks.begin(), largeTasks.end(), [&](int a, int b) { return pathLen[a] > pathLen[b]; });
    if (!largeTasks.empty()) {
      int* dLT = nullptr;
      UPV(dLT, int, largeTasks);
      pplan_.largeTasks = dLT;
    }
    pplan_.nLargeTasks = (int)largeTasks.size();
    int* dLeaves = nullptr;
    UPV(dLeaves, int, leaves);
    pplan_.leaves = dLeaves;
    pplan_.nLeaves = (int)leaves.size();
    // forward-elimination tasks: fronts whose children are all leaves become
    // groups (one warp eliminates the children and the front, passing the
    // update vectors in shared memory) when every front of the group takes the fast
    // forward elimination (at most 64 rows and 64 gathered child rows, its L
    // block within the staging capacity); other leaves are tasks of their own
    pplan_.maxRow = maxRowAll;
    pplan_.maxNpiv = 1;
    for (int f = 0; f < nfr; ++f)
      if (!large[f]) pplan_.maxNpiv = std::max(pplan_.maxNpiv, npiv[f]);
    const long long capL = stagingCapacity(pplan_, opt_.fp32Factor ? sizeof(float) : sizeof(double));
    auto fastFront = [&](int f) { return nrow[f] <= 64 && (long long)nrow[f] * npiv[f] <= capL; };
    std::vector<char> inGroup(nfr, 0), isHead(nfr, 0);
    for (int f = 0; f < nfr; ++f) {
      if (nchild[f] == 0 || nchild[f] > 8 || !fastFront(f)) continue;
      bool ok = true;
      int ncg = 0;
      for (int c = 0; c < nchild[f] && ok; ++c) {
        const int ch = childList[childOffV[f] + c];
        ok = nchild[ch] == 0 && fastFront(ch);
        ncg += nrow[ch] - npiv[ch];
      }
      if (!ok || ncg > 64) continue;
      isHead[f] = 1;
      for (int c = 0; c < nchild[f]; ++c) inGroup[childList[childOffV[f] + c]] = 1;
    }
    std::vector<int> tasks, taskLen;
    for (int f = 0; f < nfr; ++f) {
      if (isHead[f]) { tasks.push_back(f | (1 << 30)); taskLen.push_back(pathLen[f] + 1); }
      else if (nchild[f] == 0 && !inGroup[f]) { tasks.push_back(f); taskLen.push_back(pathLen[f]); }
    }
    if (nfr >= (1 << 30)) { err = "too many fronts for the task encoding"; return -910; }
    std::vector<int> order(tasks.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = (int)k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return taskLen[a] > taskLen[b]; });
    std::vector<int> sortedTasks(tasks.size());
    for (size_t k = 0; k < order.size(); ++k) sortedTasks[k] = tasks[order[k]];
    int* dTasks = nullptr;
    UPV(dTasks, int, sortedTasks);
    trace.mark("child gathers, leaves, tasks", stream_);
    pplan_.tasks = dTasks;
    pplan_.nTasks = (int)sortedTasks.size();
    // backward queue: fronts whose children are all leaves solve them inline;
    // roots and chain counts per model (the queue's initial slots and total):
    // a chain ends at a leaf not solved inline or at an inline front
    std::vector<unsigned char> bwInline(nfr, 0);
    for (int f = 0; f < nfr; ++f) {
      bool all = nchild[f] > 0 && !large[f];
      for (int c = 0; c < nchild[f] && all; ++c) all = nchild[childList[childOffV[f] + c]] == 0;
      bwInline[f] = all ? 1 : 0;
    }
    // the warp queue starts at the tops of the small subtrees (roots, or fronts
    // under a large parent); the large-front queue at the large roots, its
    // chains ending at large fronts without large children
    auto smallTop = [&](int f) { return !large[f] && (parent[f] < 0 || large[parent[f]]); };
    std::vector<int> rootOff(nm + 1, 0), roots, leafCnt(nm, 0);
    std::vector<int> rootOffL(nm + 1, 0), rootsL, chainL(nm, 0);
    for (int f = 0; f < nfr; ++f) {
      if (smallTop(f)) ++rootOff[fmodel[f] + 1];
      if (!large[f] && (bwInline[f] || (nchild[f] == 0 && !(parent[f] >= 0 && bwInline[parent[f]]))))
        ++leafCnt[fmodel[f]];
      if (large[f] && parent[f] < 0) ++rootOffL[fmodel[f] + 1];
      if (large[f] && nLargeChild[f] == 0) ++chainL[fmodel[f]];
    }
    for (int m = 0; m < nm; ++m) rootOffL[m + 1] += rootOffL[m];
    rootsL.resize(rootOffL[nm]);
    {
      std::vector<int> fill(rootOffL.begin(), rootOffL.end() - 1);
      for (int f = 0; f < nfr; ++f)
        if (large[f] && parent[f] < 0) rootsL[fill[fmodel[f]]++] = f;
    }
    {
      unsigned char* dInline = nullptr;
      UPV(dInline, unsigned char, bwInline);
      pplan_.bwInline = dInline;
    }
    for (int m = 0; m < nm; ++m) rootOff[m + 1] += rootOff[m];
    roots.resize(rootOff[nm]);
    {
      std::vector<int> fill(rootOff.begin(), rootOff.end() - 1);
      for (int f = 0; f < nfr; ++f)
        if (smallTop(f)) roots[fill[fmodel[f]]++] = f;
    }
    int *dRootOff = nullptr, *dRoots = nullptr, *dLeafCnt = nullptr;
    UPV(dRootOff, int, rootOff);
    UPV(dRoots, int, roots);
    UPV(dLeafCnt, int, leafCnt);
    // iteration counters in one block, zeroed by one memset per iteration:
    // active models (int) and elements (long long), the backward queues'
    // counters (4 per solve), the factorisation's per-front counters and one set
    // per refinement forward elimination (each + its leaf counter)
    const int nq = std::max(1, opt_.fp32Factor ? opt_.refineSweeps : 1);
    // with large fronts: their queue counters (4 per solve) and per-front counters
    // (factor + one set per refinement forward elimination) follow
    const size_t largeInts = nLargeFronts > 0 ? 4 * (size_t)nq + (size_t)nq * (nfr + 1) : 0;
    ctrInts_ = 4 + 4 * (size_t)nq + (size_t)nq * (nfr + 1) + largeInts;
    ctrBlock_ = alloc<int>(ctrInts_);
    if (!ctrBlock_) { err = "out of device memory (counters)"; return -906; }
    dActive_ = ctrBlock_;
    dActiveEl_ = reinterpret_cast<long long*>(ctrBlock_ + 2);
    pplan_.bwCtr = ctrBlock_ + 4;
    pplan_.cntFactor = ctrBlock_ + 4 + 4 * nq;
    pplan_.cntForward = pplan_.cntFactor + (nfr + 1);
    pplan_.bwQueue = alloc<int>((size_t)nq * std::max<size_t>(leaves.size(), 1));
    queueInts_ = (size_t)nq * std::max<size_t>(leaves.size(), 1);
    if (nLargeFronts > 0) {
      pplan_.bwLCtr = pplan_.cntFactor + (size_t)nq * (nfr + 1);
      pplan_.cntLargeFactor = pplan_.bwLCtr + 4 * nq;
      pplan_.cntLargeForward = pplan_.cntLargeFactor + (nfr + 1);
      pplan_.largeStride = std::max<int>((int)largeTasks.size(), 1);
      pplan_.bwLQueue = alloc<int>((size_t)nq * pplan_.largeStride);
      largeQueueInts_ = (size_t)nq * pplan_.largeStride;
      int *dRootOffL = nullptr, *dRootsL = nullptr, *dChainL = nullptr;
      UPV(dRootOffL, int, rootOffL);
      UPV(dRootsL, int, rootsL);
      UPV(dChainL, int, chainL);
      seed_.strideL = pplan_.largeStride;
      seed_.rootOffL = dRootOffL;
      seed_.rootsL = dRootsL;
      seed_.slotCntL = dChainL;
      seed_.queueL = pplan_.bwLQueue;
      seed_.ctrL = pplan_.bwLCtr;
    }
    seed_.nq = nq;
    seed_.stride = (int)std::max<size_t>(leaves.size(), 1);
    seed_.rootOff = dRootOff;
    seed_.roots = dRoots;
    seed_.slotCnt = dLeafCnt;
    seed_.queue = pplan_.bwQueue;
    seed_.ctr = pplan_.bwCtr;
    pplan_.errFlag = alloc<int>(1);
    d_.errFlag = pplan_.errFlag;
  }
#undef UPV
  trace.mark("queues and counters", stream_);
  if (allocFailed_) { err = "out of device memory"; return -906; }
  FG_CHECK(cudaMallocHost(&hActive_, sizeof(int)));
  FG_CHECK(cudaMallocHost(&hStates_, sizeof(int) * (size_t)std::max(nm, 1)));
  FG_CHECK(cudaMallocHost(&hActiveEl_, sizeof(long long)));
  for (cudaEvent_t& ev : ev_) FG_CHECK(cudaEventCreate(&ev));
  // mutable state for snapshot/restore (everything a run changes that is read
  // before it is rewritten), with the layout of each array's per-model slices
  {
    // per model and kind: first object and object count
    int64_t off[14] = {0};
    for (auto& r : mRange_) r.assign(nm, {0, 0});
    for (int k = 0; k < nm; ++k) {
      const HostModel& h = *models[k];
      int64_t cnt[14] = {0};
      cnt[SK_TRIAD] = h.ntri;
      cnt[SK_DOF] = h.ndof;
      cnt[SK_EQ] = h.neq;
      cnt[SK_MODEL] = 1;
      cnt[SK_ELEM] = h.nel;
      cnt[SK_AXIAL] = h.nax;
      cnt[SK_MOTION] = (int64_t)h.motD0.size();
      cnt[SK_EXT] = h.nExt;
      cnt[SK_PART] = h.npart;
      for (int p = 0; p < h.npart; ++p) {
        cnt[SK_PARTVEC] += 6 * h.pNtri[p] + h.pNgen[p];
        cnt[SK_PARTGEN] += h.pNgen[p];
      }
      cnt[SK_JVAR] = (int64_t)h.jLdof.size();
      cnt[SK_JOINT] = h.njoint;
      cnt[SK_XVEC] = h.cxVecSize;
      for (int q = 0; q < 14; ++q) {
        mRange_[q][k] = {off[q], cnt[q]};
        off[q] += cnt[q];
      }
    }
    stride_[SK_ELEM] = nel;
    stride_[SK_AXIAL] = d_.naxTot;
  }
  const size_t D = sizeof(double);
  auto reg = [&](void* p, size_t elem, int kind, int width, size_t count, const char* tag) {
    mutable_.push_back({p, elem * (size_t)width * count});
    stateArrays_.push_back({static_cast<char*>(p), elem, kind, width, tag});
  };
  reg(d_.ur, D, SK_TRIAD, 12, ntri, "ur");
  {
    double* dofArr[8] = {d_.urd, d_.urdd, d_.dk, d_.ak, d_.rinc, d_.sinc0, d_.sinc1, d_.sinc2};
    const char* dofTag[8] = {"urd", "urdd", "dk", "ak", "rinc", "sinc0", "sinc1", "sinc2"};
    for (int q = 0; q < 8; ++q) reg(dofArr[q], D, SK_DOF, 1, ndof, dofTag[q]);
    double* eqArr[8] = {d_.FSk, d_.FDk, d_.FIk, d_.Qk, d_.FIact, d_.res, d_.del, d_.extRhs};
    const char* eqTag[8] = {"FSk", "FDk", "FIk", "Qk", "FIact", "res", "del", "extRhs"};
    for (int q = 0; q < 8; ++q) reg(eqArr[q], D, SK_EQ, 1, neq, eqTag[q]);
  }
  reg(M.dt, D, SK_MODEL, 1, nm, "dt");
  reg(d_.supTr, D, SK_ELEM, 12, nel, "supTr");
  reg(d_.finit, D, SK_ELEM, 12, nel, "finit");
  reg(d_.finitPrev, D, SK_ELEM, 12, nel, "finitPrev");
  reg(d_.Fel, D, SK_ELEM, 48, nel, "Fel");
  reg(M.time, D, SK_MODEL, 1, nm, "time");
  reg(M.sacc, D, SK_MODEL, 1, nm, "sacc");
  reg(M.svel, D, SK_MODEL, 1, nm, "svel");
  reg(M.deln, D, SK_MODEL, 1, nm, "deln");
  reg(M.staticScale, D, SK_MODEL, 1, nm, "staticScale");
  reg(M.scaleN, D, SK_MODEL, 3, nm, "scaleN");
  reg(M.gravity, D, SK_MODEL, 3, nm, "gravity");
  reg(M.pc, D, SK_MODEL, 4, nm, "pc");
  reg(M.normVal, D, SK_MODEL, 18, nm, "normVal");
  {
    int* ia[9] = {M.state, M.flags, M.status, M.iter, M.nSeqNoUpd, M.negPiv, M.staticIter, M.staticNinc,
                  M.staticDone};
    const char* it[9] = {"state", "flags", "status", "iter", "nSeqNoUpd", "negPiv", "staticIter", "staticNinc",
                         "staticDone"};
    for (int q = 0; q < 9; ++q) reg(ia[q], sizeof(int), SK_MODEL, 1, nm, it[q]);
  }
  reg(M.nStep, sizeof(long long), SK_MODEL, 1, nm, "nStep");
  reg(M.nIter, sizeof(long long), SK_MODEL, 1, nm, "nIter");
  reg(M.stepLimit, sizeof(long long), SK_MODEL, 1, nm, "stepLimit");
  reg(M.qsCount, sizeof(int), SK_MODEL, 1, nm, "qsCount");
  if (d_.nldTot > 0) reg(d_.qext, D, SK_EQ, 1, neq, "qext");
  if (d_.nextTot > 0) reg(d_.extVal, D, SK_EXT, 1, d_.nextTot, "extVal");
  if (d_.nmotTot > 0) {
    reg(d_.motD, D, SK_MOTION, 1, d_.nmotTot, "motD");
    reg(d_.motCc, D, SK_MOTION, 1, d_.nmotTot, "motCc");
  }
  if (d_.urQs) {  // the state pure linear quasi-static steps restart from
    reg(d_.urQs, D, SK_TRIAD, 12, ntri, "urQs");
    reg(d_.supTrQs, D, SK_ELEM, 12, nel, "supTrQs");
    reg(d_.urdQs, D, SK_DOF, 1, ndof, "urdQs");
    reg(d_.urddQs, D, SK_DOF, 1, ndof, "urddQs");
  }
  if (d_.naxTot > 0) {
    reg(d_.axN, D, SK_AXIAL, 3, d_.naxTot, "axN");
    reg(d_.axLen, D, SK_AXIAL, 1, d_.naxTot, "axLen");
    reg(d_.FelA, D, SK_AXIAL, 12, d_.naxTot, "FelA");
  }
  if (d_.npartTot > 0) {
    reg(d_.pSupTr, D, SK_PART, 12, d_.npartTot, "pSupTr");
    reg(d_.pFinit, D, SK_PARTVEC, 1, partVecTot_, "pFinit");
    reg(d_.pFinitPrev, D, SK_PARTVEC, 1, partVecTot_, "pFinitPrev");
    int64_t ng = 0;
    for (int k = 0; k < nm; ++k) ng += mRange_[SK_PARTGEN][k][1];
    if (ng) reg(d_.pGen, D, SK_PARTGEN, 1, (size_t)ng, "pGen");
  }
  if (d_.njointTot > 0) {
    int64_t nv = 0;
    for (int k = 0; k < nm; ++k) nv += mRange_[SK_JVAR][k][1];
    if (nv) reg(d_.jVar, D, SK_JVAR, 1, (size_t)nv, "jVar");
    reg(d_.jT, D, SK_JOINT, 72, d_.njointTot, "jT");
  }
  {
    int64_t xv = 0;
    for (int k = 0; k < nm; ++k) xv += mRange_[SK_XVEC][k][1];
    if (xv && d_.njointTot > 0) reg(d_.FelX, D, SK_XVEC, 1, (size_t)xv, "FelX");
  }
  uploadedBytes_ = t_putBytes;
  // beam elements only (no axial elements, joints or reduced parts, whose
  // Newton matrices read state the element pass updates): forked assembly
  forkAssembly_ = d_.nelTot > 0 && d_.naxTot == 0 && d_.njointTot == 0 && d_.npartTot == 0 && d_.ncxTot == 0;
  // the first solve's back substitution inside the factorisation's launch;
  // FGPU_NO_FUSED_BACKWARD set at batch creation keeps it a launch of its own
  // (the same results: tests compare the two)
  fuseBackward_ = fusableBackward(pplan_, opt_.fp32Factor) && std::getenv("FGPU_NO_FUSED_BACKWARD") == nullptr;
  FG_CHECK(cudaStreamSynchronize(stream_));
  FG_CHECK(cudaGetLastError());
  trace.mark("state registry", stream_);
  return 0;
}

int Engine::snapshot() {
  size_t total = 0;
  for (auto& m : mutable_) total += (m.second + 255) & ~size_t(255);
  if (!backup_) {
    backup_ = alloc<char>(total);
    if (!backup_) return -930;
  }
  size_t off = 0;
  for (auto& m : mutable_) {
    cudaMemcpyAsync(backup_ + off, m.first, m.second, cudaMemcpyDeviceToDevice, stream_);
    off += (m.second + 255) & ~size_t(255);
  }
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -931;
}

int Engine::restore() {
  if (!backup_) return -932;
  size_t off = 0;
  for (auto& m : mutable_) {
    cudaMemcpyAsync(m.first, backup_ + off, m.second, cudaMemcpyDeviceToDevice, stream_);
    off += (m.second + 255) & ~size_t(255);
  }
  invalidateNewtonScales();
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -933;
}

// the element Newton matrices are not part of the saved state: scale factors
// no step can have make the next tangent iteration rebuild them
void Engine::invalidateNewtonScales() {
  scaleSentinel_.assign(3 * (size_t)d_.m.n, -1.0e300);
  cudaMemcpyAsync(d_.m.scaleN, scaleSentinel_.data(), sizeof(double) * scaleSentinel_.size(),
                  cudaMemcpyHostToDevice, stream_);
}

int Engine::timeFactor(int reps, double* msPerLaunch, double* bytes) {
  const int nm = d_.m.n;
  std::vector<int> flags(nm), status(nm), neg(nm), all(nm, FL_ACTIVE | FL_TANGENT);
  cudaMemcpyAsync(flags.data(), d_.m.flags, sizeof(int) * nm, cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(status.data(), d_.m.status, sizeof(int) * nm, cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(neg.data(), d_.m.negPiv, sizeof(int) * nm, cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  cudaMemcpyAsync(d_.m.flags, all.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const size_t cntBytes = sizeof(int) * ((size_t)d_.nfrontTot + 1);
  auto clear = [&]() {
    cudaMemsetAsync(pplan_.cntFactor, 0, cntBytes, stream_);
    if (pplan_.cntLargeFactor) cudaMemsetAsync(pplan_.cntLargeFactor, 0, cntBytes, stream_);
  };
  clear();
  enqueueFactor(stream_);  // warm-up
  cudaEventRecord(e0, stream_);
  for (int k = 0; k < reps; ++k) {
    clear();
    enqueueFactor(stream_);
  }
  cudaEventRecord(e1, stream_);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaMemcpyAsync(d_.m.flags, flags.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(d_.m.status, status.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(d_.m.negPiv, neg.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -946;
  if (msPerLaunch) *msPerLaunch = reps > 0 ? ms / reps : 0.0;
  if (bytes) *bytes = factorBytes_;
  return 0;
}

// ---- autotuner ------------------------------------------------------------
// Launch shapes are timed on the batch's own fronts before its first batched
// iteration and the fastest kept.  Only shapes that give the same results to
// the last bit are candidates (panel variant, warps per block, cluster size),
// so the choice -- which depends on timing -- never changes a result.  Front
// bucketing (which fronts go to warps, which to clusters) changes the
// arithmetic and is therefore fixed (kLargeFrontRows), not tuned.
// The probe runs while no model has started a step: the factors and solve
// vectors it overwrites are scratch until the first iteration's
// factorisation, which every model does (its first iteration updates the
// tangent).  Its flags, status and pivot counters are restored.
namespace {
std::mutex g_shapeMutex;
std::map<std::string, std::array<int, 4>> g_shapeCache;  // batch structure -> tuned shape
}  // namespace

int Engine::setLaunchShape(const int* sh) {
  if (iterated_) return -1;
  if (sh[0] < 0 || sh[0] > 2) return -2;
  for (int k = 1; k <= 2; ++k)
    if (sh[k] != 4 && sh[k] != 8 && sh[k] != 16) return -2;
  if (sh[3] != 2 && sh[3] != 4 && sh[3] != 8 && sh[3] != 16) return -2;
  pplan_.factorPanel = sh[0];
  pplan_.forwardWarps = sh[1];
  pplan_.backwardWarps = sh[2];
  pplan_.largeCluster = sh[3];
  shapeFixed_ = tuned_ = true;
  probeMs_ = 0.0;
  return 0;
}

int Engine::launchShape(int* sh, double* probeMs) const {
  sh[0] = pplan_.factorPanel;
  sh[1] = pplan_.forwardWarps;
  sh[2] = pplan_.backwardWarps;
  sh[3] = pplan_.largeCluster;
  if (probeMs) *probeMs = probeMs_;
  return tuned_ ? 1 : 0;
}

void Engine::ensureTuned() {
  if (tuned_) return;
  tuned_ = true;
  if (iterated_ || d_.nfrontTot <= 0) return;
  if (autotune() != 0) {  // keep the defaults
    pplan_.factorPanel = 0;
    pplan_.forwardWarps = pplan_.backwardWarps = pplan_.largeCluster = 8;
  }
}

int Engine::autotune() {
  const auto t0 = std::chrono::steady_clock::now();
  char key[256];
  snprintf(key, sizeof key, "dev%d f%d s%d r%d p%d L%d n%d l%d t%d", device_, opt_.fp32Factor ? 1 : 0,
           opt_.refineSweeps, pplan_.maxRow, pplan_.maxNpiv, pplan_.maxRowLarge,
           (int)std::lround(std::log2((double)d_.nfrontTot + 1.0)), (int)std::lround(std::log2(pplan_.nLeaves + 1.0)),
           pplan_.nLargeTasks > 0 ? (int)std::lround(std::log2(pplan_.nLargeTasks + 1.0)) : -1);
  {
    std::lock_guard<std::mutex> lk(g_shapeMutex);
    auto it = g_shapeCache.find(key);
    if (it != g_shapeCache.end()) {
      pplan_.factorPanel = it->second[0];
      pplan_.forwardWarps = it->second[1];
      pplan_.backwardWarps = it->second[2];
      pplan_.largeCluster = it->second[3];
      return 0;
    }
  }
  const int nm = d_.m.n;
  const bool f32 = opt_.fp32Factor;
  std::vector<int> flags(nm), status(nm), neg(nm), all(nm, FL_ACTIVE | FL_TANGENT);
  cudaMemcpyAsync(flags.data(), d_.m.flags, sizeof(int) * nm, cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(status.data(), d_.m.status, sizeof(int) * nm, cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(neg.data(), d_.m.negPiv, sizeof(int) * nm, cudaMemcpyDeviceToHost, stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -1;
  cudaMemcpyAsync(d_.m.flags, all.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  launchProbeEntries(d_, f32, stream_);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // mean milliseconds of `work` over 3 launches after one warm-up; `prep`
  // (counters, queue seeds, inputs) is enqueued before each and not timed
  auto timeIt = [&](const std::function<void()>& prep, const std::function<void()>& work) -> float {
    float tot = 0.f;
    for (int r = 0; r < 4; ++r) {
      prep();
      cudaEventRecord(e0, stream_);
      work();
      cudaEventRecord(e1, stream_);
      if (cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (r > 0) tot += ms;
    }
    return tot / 3.f;
  };
  const double* rhs = d_.del;
  bool ok = true;
  // 1. small-front factorisation: panel variant
  {
    float best = -1.f;
    int pick = 0;
    for (int pv = 0; pv <= 2; ++pv) {
      pplan_.factorPanel = pv;
      const float t = timeIt([&] { resetIterationCounters(stream_); },
                             [&] { launchFactorForwardCascade(d_, pplan_, f32, rhs, stream_); });
      if (t < 0.f) ok = false;
      if (t >= 0.f && (best < 0.f || t < best)) best = t, pick = pv;
    }
    pplan_.factorPanel = pick;
  }
  // 2. large fronts: cluster size (the small cascade runs first, untimed)
  if (ok && pplan_.nLargeTasks > 0) {
    float best = -1.f;
    int pick = 8;
    for (int c : {8, 4, 2, 16}) {
      if (c > 8 && largeClusterCapacity(pplan_, f32, c) < 1) continue;  // not on this device
      pplan_.largeCluster = c;
      const float t = timeIt(
          [&] {
            resetIterationCounters(stream_);
            launchFactorForwardCascade(d_, pplan_, f32, rhs, stream_);
          },
          [&] { launchLargeFactorForward(d_, pplan_, f32, rhs, stream_); });
      if (t < 0.f) ok = false;
      if (t >= 0.f && (best < 0.f || t < best)) best = t, pick = c;
    }
    pplan_.largeCluster = pick;
  }
  // 3. forward elimination of a refinement sweep: warps per block
  if (ok && f32 && opt_.refineSweeps > 1) {
    float best = -1.f;
    int pick = 8;
    for (int w : {8, 4, 16}) {
      pplan_.forwardWarps = w;
      const float t = timeIt([&] { resetIterationCounters(stream_); },
                             [&] {
                               launchForwardCascade(d_, pplan_, f32, rhs, 1, stream_);
                               launchLargeForward(d_, pplan_, f32, rhs, 1, stream_);
                             });
      if (t < 0.f) ok = false;
      if (t >= 0.f && (best < 0.f || t < best)) best = t, pick = w;
    }
    pplan_.forwardWarps = pick;
  }
  // 4. back substitution: warps per block (queues seeded for every model)
  if (ok) {
    float best = -1.f;
    int pick = 8;
    for (int w : {8, 4, 16}) {
      pplan_.backwardWarps = w;
      const float t = timeIt(
          [&] {
            resetIterationCounters(stream_);
            launchSeedBackward(d_, seed_, stream_);
          },
          [&] {
            launchLargeBackward(d_, pplan_, f32, 0, opt_.refineSweeps == 1, stream_);
            launchBackward(d_, pplan_, f32, 0, opt_.refineSweeps == 1, stream_);
          });
      if (t < 0.f) ok = false;
      if (t >= 0.f && (best < 0.f || t < best)) best = t, pick = w;
    }
    pplan_.backwardWarps = pick;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // a bounded wait that ran out in the probe would leave the error flag set
  int errFlag = 0;
  cudaMemcpyAsync(&errFlag, pplan_.errFlag, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(d_.m.flags, flags.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(d_.m.status, status.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(d_.m.negPiv, neg.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  resetIterationCounters(stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess || !ok || errFlag) {
    cudaMemsetAsync(pplan_.errFlag, 0, sizeof(int), stream_);
    cudaStreamSynchronize(stream_);
    return -1;
  }
  probeMs_ = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  std::lock_guard<std::mutex> lk(g_shapeMutex);
  g_shapeCache[key] = {pplan_.factorPanel, pplan_.forwardWarps, pplan_.backwardWarps, pplan_.largeCluster};
  return 0;
}

long long Engine::phaseTimings(double* ms, long long* elems, int n) {
  for (int k = 0; k < n && k < 5; ++k) ms[k] = phaseMs_[k];
  if (elems) *elems = phaseElems_;
  return phaseSamples_;
}

void Engine::resetPhaseTimings() {
  phaseMs_[0] = phaseMs_[1] = phaseMs_[2] = phaseMs_[3] = phaseMs_[4] = 0.0;
  phaseSamples_ = phaseElems_ = 0;
}

void Engine::enqueueFactor(cudaStream_t s, bool withBackward) {
  // factorisation and the first forward elimination in one cascade (small
  // fronts by warps, then the large fronts above them by thread blocks)
  launchFactorForwardCascade(d_, pplan_, opt_.fp32Factor, d_.del, s, withBackward, opt_.refineSweeps <= 1);
  launchLargeFactorForward(d_, pplan_, opt_.fp32Factor, d_.del, s);
}

// phase-timing events: external event nodes inside a captured graph, plain
// records when the iteration is launched directly (the external flag is only
// valid during stream capture)
void Engine::recordPhase(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cs);
  if (cs == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal);
  else
    cudaEventRecord(ev, s);
}

void Engine::enqueueSolve(cudaStream_t s, bool timedForward, bool backwardDone) {
  const bool f32 = opt_.fp32Factor;
  const int sw = opt_.refineSweeps;
  // the timed back substitution: the first solve's, or the second's when the
  // first ran inside the factorisation's launch
  const int timedBackward = backwardDone && sw > 1 ? 1 : 0;
  for (int sweep = 0; sweep < sw; ++sweep) {
    // the right-hand side is read and the solution stored inside the launches;
    // the first forward elimination ran with the factorisation
    if (sweep > 0) launchRefineResidual(d_, s);
    if (sweep == 1 && timedForward) recordPhase(ev_[5], s);
    if (sweep > 0) {
      launchForwardCascade(d_, pplan_, f32, f32 ? d_.rref : d_.del, sweep, s);
      launchLargeForward(d_, pplan_, f32, f32 ? d_.rref : d_.del, sweep, s);
    }
    if (sweep == 1 && timedForward) recordPhase(ev_[6], s);
    if (sweep == timedBackward && timedForward) recordPhase(ev_[7], s);
    if (!(sweep == 0 && backwardDone)) {
      launchLargeBackward(d_, pplan_, f32, sweep, sweep == sw - 1, s);
      launchBackward(d_, pplan_, f32, sweep, sweep == sw - 1, s);
    }
    if (sweep == timedBackward && timedForward) recordPhase(ev_[8], s);
  }
}

// the iteration's counters to zero and its backward queue slots to empty (-1):
// two memsets, before the step-start kernel seeds the queues
void Engine::resetIterationCounters(cudaStream_t s) {
  cudaMemsetAsync(ctrBlock_, 0, sizeof(int) * ctrInts_, s);
  if (queueInts_) cudaMemsetAsync(pplan_.bwQueue, 0xff, sizeof(int) * queueInts_, s);
  if (largeQueueInts_) cudaMemsetAsync(pplan_.bwLQueue, 0xff, sizeof(int) * largeQueueInts_, s);
}

// first half of a Newton iteration: step start (predictor) or the corrector's
// right-hand side, and the Newton matrix when the tangent is updated
// the side stream and its fork/join events, created at first use
bool Engine::sideReady() {
  if (side_) return true;
  if (cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&evFork_, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&evJoin_, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&evFork2_, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&evJoin2_, cudaEventDisableTiming) != cudaSuccess) {
    if (side_) cudaStreamDestroy(side_);
    side_ = nullptr;
    return false;
  }
  return true;
}

void Engine::enqueueAssembly(cudaStream_t s) {
  iterated_ = true;
  resetIterationCounters(s);
  launchBeginStep(d_, dActive_, dActiveEl_, seed_, s);
  launchQsRestore(d_, s);
  // Beam-only batches: the element Newton matrices and their CSR gather read
  // the flags and scales of the step start, the element frames and the
  // constant element matrices, none of which the predictor, the predictor's
  // element pass (no frame update) or the residual write, and they write
  // nothing those read -- so they run on the side stream beside them, joined
  // before the prescribed-motion right-hand side that needs both.
  const bool fork = forkAssembly_ && sideReady();
  if (fork) {
    cudaEventRecord(evFork_, s);
    cudaStreamWaitEvent(side_, evFork_, 0);
    launchBuildElementNewton(d_, side_);
    launchRotateElementNewton(d_, side_);
    launchCsrGather(d_, side_);
    cudaEventRecord(evJoin_, side_);
  }
  launchMotions(d_, s);
  launchLoads(d_, s);
  launchPredictDofs(d_, s);
  launchElements(d_, EM_PRED, s);
  launchResidual(d_, s);
  if (fork) {
    cudaStreamWaitEvent(s, evJoin_, 0);
  } else {
    launchBuildElementNewton(d_, s);
    launchRotateElementNewton(d_, s);
    launchCsrGather(d_, s);
  }
  launchMotionRhs(d_, s);
}

// second half: factorisation and solves, the increment, the element pass and
// the convergence test
void Engine::enqueueSolveUpdate(cudaStream_t s) {
  // Batches without large fronts run the first solve's back substitution in
  // the factorisation's launch: a model's back substitution starts as soon as
  // its own elimination is done, beside the other models' factorisations.
  const bool fuse = fuseBackward_;
  recordPhase(ev_[0], s);
  enqueueFactor(s, fuse);
  recordPhase(ev_[1], s);
  enqueueSolve(s, true, fuse);
  recordPhase(ev_[2], s);
  launchIncrement(d_, s);
  recordPhase(ev_[3], s);
  // the partial norms read the increments and the residual, which the element
  // pass does not touch; the convergence test after the join also sees every
  // status bit the element pass set (a failed corotation)
  const bool fork = sideReady();
  if (fork) {
    cudaEventRecord(evFork2_, s);
    cudaStreamWaitEvent(side_, evFork2_, 0);
    launchNormsPartial(d_, side_);
    cudaEventRecord(evJoin2_, side_);
  }
  launchElements(d_, EM_INC, s);
  recordPhase(ev_[4], s);
  if (fork) {
    cudaStreamWaitEvent(s, evJoin2_, 0);
    launchControlStepEnd(d_, s);
  } else {
    launchNormsControl(d_, s);
  }
  if (rec_.on) launchRecordStep(d_, rec_.plan, false, s);
}

int Engine::assembleIteration() {
  ensureTuned();
  enqueueAssembly(stream_);
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -940;
}

int Engine::solveUpdateIteration() {
  enqueueSolveUpdate(stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -941;
  std::string err;
  return resultsDrain(err) ? -942 : 0;
}

void Engine::setStepLimitOf(int m, long long lim) {
  cudaMemcpyAsync(d_.m.stepLimit + m, &lim, sizeof(long long), cudaMemcpyHostToDevice, stream_);
  cudaStreamSynchronize(stream_);
}

// ---- linear-solver seam of one model -------------------------------------
namespace {
// the flags of a seam call: model m alone, with `fl`
void seamFlags(const DevData& d, int m, int fl, cudaStream_t s) {
  std::vector<int> v((size_t)d.m.n, 0);
  v[m] = fl;
  cudaMemcpyAsync(d.m.flags, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice, s);
  cudaStreamSynchronize(s);  // v goes out of scope
}
}  // namespace

int Engine::seamAssemble(int m, double sM, double sC, double sK) {
  if (m < 0 || m >= d_.m.n) return -1;
  if (modelState(m) == ST_ITER) return -2;  // inside a step: its factor is in use
  ensureTuned();
  seamFlags(d_, m, FL_ACTIVE | FL_TANGENT | FL_REBUILD, stream_);
  // scale factors as the element kernels read them: M, K, C
  const double sc[3] = {sM, sK, sC};
  cudaMemcpyAsync(d_.m.scaleN + 3 * (size_t)m, sc, sizeof sc, cudaMemcpyHostToDevice, stream_);
  launchBuildElementNewton(d_, stream_);
  launchRotateElementNewton(d_, stream_);
  launchCsrGather(d_, stream_);
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -3;
}

int Engine::seamFactor(int m) {
  if (m < 0 || m >= d_.m.n) return -1;
  if (modelState(m) == ST_ITER) return -2;
  int st0 = 0, neg0 = 0, st = 0, neg = 0;
  cudaMemcpyAsync(&st0, d_.m.status + m, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(&neg0, d_.m.negPiv + m, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  const int zero = 0;
  cudaMemcpyAsync(d_.m.status + m, &zero, sizeof(int), cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(d_.m.negPiv + m, &zero, sizeof(int), cudaMemcpyHostToDevice, stream_);
  seamFlags(d_, m, FL_ACTIVE | FL_TANGENT, stream_);
  resetIterationCounters(stream_);
  enqueueFactor(stream_);
  cudaMemcpyAsync(&st, d_.m.status + m, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(&neg, d_.m.negPiv + m, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -4;
  // the model's own status and pivot count are its stepping's, not the seam's
  cudaMemcpyAsync(d_.m.status + m, &st0, sizeof(int), cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(d_.m.negPiv + m, &neg0, sizeof(int), cudaMemcpyHostToDevice, stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -4;
  return (st & SS_SINGULAR) ? -3 : neg;
}

int Engine::seamSolve(int m, double* rhs, int nrhs) {
  if (m < 0 || m >= d_.m.n || nrhs < 0) return -1;
  if (modelState(m) == ST_ITER) return -2;
  const int n = hm_[m]->neq;
  seamFlags(d_, m, FL_ACTIVE, stream_);
  for (int r = 0; r < nrhs; ++r) {
    double* b = rhs + (size_t)r * n;
    cudaMemcpyAsync(d_.del + modelEqOff_[m], b, sizeof(double) * n, cudaMemcpyHostToDevice, stream_);
    resetIterationCounters(stream_);
    launchSeedBackward(d_, seed_, stream_);
    enqueueFactor(stream_);  // forward elimination only (no tangent flag)
    enqueueSolve(stream_);
    cudaMemcpyAsync(b, d_.del + modelEqOff_[m], sizeof(double) * n, cudaMemcpyDeviceToHost, stream_);
    if (cudaStreamSynchronize(stream_) != cudaSuccess) return -4;
  }
  int err = 0;
  cudaMemcpyAsync(&err, pplan_.errFlag, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  return err ? -5 : 0;
}

int Engine::prepareStiffnessSolves() {
  const int nm = d_.m.n;
  savedFlags_.assign(nm, 0);
  cudaMemcpyAsync(savedFlags_.data(), d_.m.flags, sizeof(int) * nm, cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  std::vector<int> fl(nm, FL_ACTIVE | FL_TANGENT | FL_REBUILD);
  std::vector<double> sc(3 * (size_t)nm);
  for (int k = 0; k < nm; ++k) { sc[3 * k] = 0.0; sc[3 * k + 1] = 1.0; sc[3 * k + 2] = 0.0; }
  cudaMemcpyAsync(d_.m.flags, fl.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(d_.m.scaleN, sc.data(), sizeof(double) * sc.size(), cudaMemcpyHostToDevice, stream_);
  launchBuildElementNewton(d_, stream_);
  launchRotateElementNewton(d_, stream_);
  launchCsrGather(d_, stream_);
  resetIterationCounters(stream_);
  enqueueFactor(stream_);
  // solves from here on: active, no tangent update
  std::fill(fl.begin(), fl.end(), FL_ACTIVE);
  cudaMemcpyAsync(d_.m.flags, fl.data(), sizeof(int) * nm, cudaMemcpyHostToDevice, stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -948;
  std::vector<int> st(nm);
  cudaMemcpy(st.data(), d_.m.status, sizeof(int) * nm, cudaMemcpyDeviceToHost);
  for (int k = 0; k < nm; ++k)
    if (st[k] & SS_SINGULAR) return -3;
  return 0;
}

int Engine::solveStiffness(int m, const double* b, double* x) {
  const int n = hm_[m]->neq;
  cudaMemcpyAsync(d_.del + modelEqOff_[m], b, sizeof(double) * n, cudaMemcpyHostToDevice, stream_);
  resetIterationCounters(stream_);
  launchSeedBackward(d_, seed_, stream_);
  enqueueFactor(stream_);  // forward elimination only (no tangent flag)
  enqueueSolve(stream_);
  cudaMemcpyAsync(x, d_.del + modelEqOff_[m], sizeof(double) * n, cudaMemcpyDeviceToHost, stream_);
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -949;
}

int Engine::endStiffnessSolves() {
  if (!savedFlags_.empty())
    cudaMemcpyAsync(d_.m.flags, savedFlags_.data(), sizeof(int) * savedFlags_.size(), cudaMemcpyHostToDevice,
                    stream_);
  invalidateNewtonScales();
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -950;
}

int Engine::setExtValue(int m, int ch, double v) {
  if (m < 0 || m >= (int)modelExtOff_.size() || ch < 0 || ch >= modelExtCnt_[m]) return -1;
  cudaMemcpyAsync(d_.extVal + modelExtOff_[m] + ch, &v, sizeof(double), cudaMemcpyHostToDevice, stream_);
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -947;
}

double Engine::extValue(int m, int ch) {
  if (m < 0 || m >= (int)modelExtOff_.size() || ch < 0 || ch >= modelExtCnt_[m]) return 0.0;
  double v = 0.0;
  cudaMemcpyAsync(&v, d_.extVal + modelExtOff_[m] + ch, sizeof(double), cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  return v;
}

int Engine::setTimeStep(int m, double dt) {
  cudaMemcpyAsync(d_.m.dt + m, &dt, sizeof(double), cudaMemcpyHostToDevice, stream_);
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -942;
}

// solverModule.f90:1868-1901 (setRhsVector with keepDuringIterations): in the
// predictor of a step the vector is also kept as external forces of the
// step's later iterations; the right-hand side is replaced or added to
int Engine::setRhs(int m, const double* v, bool add) {
  const int n = hm_[m]->neq;
  double* dst = d_.del + modelEqOff_[m];
  int it = -1;
  cudaMemcpyAsync(&it, d_.m.iter + m, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  if (it == 0)
    cudaMemcpyAsync(d_.extRhs + modelEqOff_[m], v, sizeof(double) * n, cudaMemcpyHostToDevice, stream_);
  if (!add) {
    cudaMemcpyAsync(dst, v, sizeof(double) * n, cudaMemcpyHostToDevice, stream_);
  } else {
    std::vector<double> cur(n);
    cudaMemcpyAsync(cur.data(), dst, sizeof(double) * n, cudaMemcpyDeviceToHost, stream_);
    cudaStreamSynchronize(stream_);
    for (int i = 0; i < n; ++i) cur[i] += v[i];
    cudaMemcpyAsync(dst, cur.data(), sizeof(double) * n, cudaMemcpyHostToDevice, stream_);
  }
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -943;
}

size_t Engine::stateBytes() const {
  size_t total = 0;
  for (auto& m : mutable_) total += m.second;
  return total;
}

int Engine::saveStateTo(void* host) {
  size_t off = 0;
  for (auto& m : mutable_) {
    cudaMemcpyAsync(static_cast<char*>(host) + off, m.first, m.second, cudaMemcpyDeviceToHost, stream_);
    off += m.second;
  }
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -944;
}

int Engine::restoreStateFrom(const void* host) {
  size_t off = 0;
  for (auto& m : mutable_) {
    cudaMemcpyAsync(m.first, static_cast<const char*>(host) + off, m.second, cudaMemcpyHostToDevice, stream_);
    off += m.second;
  }
  invalidateNewtonScales();
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -945;
}

// byte ranges of model m's share of a state array: one contiguous range for
// the object-major kinds, one per row for the SoA kinds (elements, axial
// elements: row c holds every object's value c)
void Engine::modelSlices(const StateArray& a, int m, std::vector<std::pair<size_t, size_t>>& out) const {
  out.clear();
  const int64_t first = mRange_[a.kind][m][0], cnt = mRange_[a.kind][m][1];
  if (cnt == 0) return;
  if (a.kind == SK_ELEM || a.kind == SK_AXIAL) {
    const int64_t stride = stride_[a.kind];
    for (int c = 0; c < a.width; ++c)
      out.push_back({(size_t)(c * stride + first) * a.elem, (size_t)cnt * a.elem});
  } else {
    out.push_back({(size_t)first * a.width * a.elem, (size_t)cnt * a.width * a.elem});
  }
}

// A model's state blob: per state array holding a share of the model, its tag
// (length byte + characters), the byte count (8 bytes) and the bytes of its
// slices.  The arrays an engine registers depend on its batch (a batch without
// prescribed motions has no motion state), so the blob names them; a receiving
// engine takes the arrays it has and leaves the others as set up (the model
// does not use them: an engine registers every array any of its models uses).
int Engine::extractModelState(int m, std::vector<char>& out) {
  if (m < 0 || m >= numModels()) return -1;
  std::vector<std::pair<size_t, size_t>> sl;
  out.clear();
  struct Pending { size_t dst, src, n; char* base; };
  std::vector<Pending> copies;
  for (const StateArray& a : stateArrays_) {
    modelSlices(a, m, sl);
    uint64_t bytes = 0;
    for (auto& r : sl) bytes += r.second;
    if (bytes == 0) continue;
    out.push_back((char)a.tag.size());
    out.insert(out.end(), a.tag.begin(), a.tag.end());
    const char* bp = reinterpret_cast<const char*>(&bytes);
    out.insert(out.end(), bp, bp + sizeof(bytes));
    for (auto& r : sl) {
      copies.push_back({out.size(), r.first, r.second, a.p});
      out.resize(out.size() + r.second);
    }
  }
  for (auto& c : copies) cudaMemcpyAsync(out.data() + c.dst, c.base + c.src, c.n, cudaMemcpyDeviceToHost, stream_);
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -946;
}

int Engine::injectModelState(int m, const std::vector<char>& in) {
  if (m < 0 || m >= numModels()) return -1;
  std::vector<std::pair<size_t, size_t>> sl;
  size_t off = 0;
  while (off < in.size()) {
    const size_t tl = (unsigned char)in[off];
    if (off + 1 + tl + sizeof(uint64_t) > in.size()) return -2;
    const std::string tag(in.data() + off + 1, tl);
    uint64_t bytes = 0;
    std::memcpy(&bytes, in.data() + off + 1 + tl, sizeof(bytes));
    off += 1 + tl + sizeof(bytes);
    if (off + bytes > in.size()) return -2;
    for (const StateArray& a : stateArrays_) {
      if (a.tag != tag) continue;
      modelSlices(a, m, sl);
      uint64_t have = 0;
      for (auto& r : sl) have += r.second;
      if (have != bytes) return -2;  // a different model
      size_t o = off;
      for (auto& r : sl) {
        cudaMemcpyAsync(a.p + r.first, in.data() + o, r.second, cudaMemcpyHostToDevice, stream_);
        o += r.second;
      }
    }
    off += bytes;
  }
  // this engine's element Newton matrices were not built with the scales the
  // state records: rebuilt at the model's next tangent; no step limit
  const double bad[3] = {-1.0, -1.0, -1.0};
  const long long lim = LLONG_MAX;
  cudaMemcpyAsync(d_.m.scaleN + 3 * m, bad, sizeof(bad), cudaMemcpyHostToDevice, stream_);
  cudaMemcpyAsync(d_.m.stepLimit + m, &lim, sizeof(lim), cudaMemcpyHostToDevice, stream_);
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -947;
}

int Engine::parkModels(const std::vector<int>& ms) {
  const int nm = numModels();
  std::vector<int> st(nm);
  std::vector<long long> steps(nm), lim(nm);
  cudaMemcpyAsync(st.data(), d_.m.state, sizeof(int) * nm, cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(steps.data(), d_.m.nStep, sizeof(long long) * nm, cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(lim.data(), d_.m.stepLimit, sizeof(long long) * nm, cudaMemcpyDeviceToHost, stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -948;
  for (int m : ms) {
    if (m < 0 || m >= nm) return -1;
    lim[m] = steps[m] + (st[m] == ST_ITER ? 1 : 0);
  }
  cudaMemcpyAsync(d_.m.stepLimit, lim.data(), sizeof(long long) * nm, cudaMemcpyHostToDevice, stream_);
  return cudaStreamSynchronize(stream_) == cudaSuccess ? 0 : -949;
}

void Engine::enqueueIteration(cudaStream_t s) {
  enqueueAssembly(s);
  enqueueSolveUpdate(s);
  const int nl = 1, sw = opt_.refineSweeps;
  // kernels per batched iteration: 12 fixed (begin step, predict, elements x2, residual,
  // element Newton build + rotate (one fused kernel for compressed beams), CSR gather,
  // increment, norms partial + control, step end) + the factorisation with the first
  // forward elimination + per further solve a refinement residual and a forward
  // elimination + a back substitution per solve (the first solve's inside the
  // factorisation's launch when fused)
  const int solveLaunches = (2 * sw - 1 + (sw - 1)) * (pplan_.nLargeTasks > 0 ? 2 : 1) -
                            (fuseBackward_ ? 1 : 0);
  launchesPerIter_ = (d_.beamSparse ? 11 : 12) + nl * (pplan_.nLargeTasks > 0 ? 2 : 1) + solveLaunches +
                     (d_.urQs ? 1 : 0) +
                     (d_.nmotTot > 0 ? 1 : 0) + (d_.nmrTot > 0 ? 1 : 0) + (d_.naxTot > 0 ? 3 : 0) +
                     (d_.nldTot > 0 ? 1 : 0) + (d_.njointTot > 0 ? 2 : 0) + (d_.ncxTot > 0 ? 3 : 0) +
                     (rec_.on ? 1 : 0);
}

int Engine::readActive() {
  cudaMemcpyAsync(hActive_, dActive_, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  return *hActive_;
}

int Engine::initialState(std::string& err) {
  SetupTrace trace;
  // staticEquilibriumModule.f90:50-437: iterate the models that asked for it
  launchStaticBegin(d_, dActive_, BackwardSeed{}, stream_);
  launchElements(d_, EM_STATIC_INIT, stream_);
  launchBuildElementNewton(d_, stream_);
  for (int guard = 0; guard < 100000; ++guard) {
    resetIterationCounters(stream_);
    launchStaticBegin(d_, dActive_, seed_, stream_);
    if (readActive() == 0) break;
    launchStaticResidual(d_, stream_);
    launchBuildElementNewton(d_, stream_);
    launchRotateElementNewton(d_, stream_);
    launchCsrGather(d_, stream_);
    enqueueFactor(stream_);
    enqueueSolve(stream_);
    launchStaticNorm(d_, stream_);
    launchStaticIncrement(d_, stream_);
    launchElements(d_, EM_STATIC, stream_);
    launchStaticFinish(d_, stream_);
  }
  // finalStaticUpdate: zero velocities, corotated update and forces of every model
  cudaMemsetAsync(d_.m.flags, 0, sizeof(int) * d_.m.n, stream_);
  launchElements(d_, EM_FINAL, stream_);
  FG_CHECK(cudaMemcpyAsync(d_.finitPrev, d_.finit, sizeof(double) * 12 * (size_t)d_.nelTot,
                           cudaMemcpyDeviceToDevice, stream_));
  if (d_.npartTot > 0)
    FG_CHECK(cudaMemcpyAsync(d_.pFinitPrev, d_.pFinit, sizeof(double) * partVecTot_, cudaMemcpyDeviceToDevice,
                             stream_));
  FG_CHECK(cudaMemsetAsync(d_.rinc, 0, sizeof(double) * (size_t)d_.ndofTot, stream_));
  if (d_.urQs) {
    // the state pure linear quasi-static steps restart from
    const size_t D = sizeof(double);
    FG_CHECK(cudaMemcpyAsync(d_.urQs, d_.ur, D * 12 * (size_t)d_.ntriTot, cudaMemcpyDeviceToDevice, stream_));
    FG_CHECK(cudaMemcpyAsync(d_.supTrQs, d_.supTr, D * 12 * (size_t)d_.nelTot, cudaMemcpyDeviceToDevice, stream_));
    FG_CHECK(cudaMemcpyAsync(d_.urdQs, d_.urd, D * (size_t)d_.ndofTot, cudaMemcpyDeviceToDevice, stream_));
    FG_CHECK(cudaMemcpyAsync(d_.urddQs, d_.urdd, D * (size_t)d_.ndofTot, cudaMemcpyDeviceToDevice, stream_));
  }
  FG_CHECK(cudaStreamSynchronize(stream_));
  FG_CHECK(cudaGetLastError());
  // a model whose initial equilibrium failed (singular, NaN, no convergence)
  // stays in its error state with its status bits; the others go on
  trace.mark("initial state", stream_);
  return 0;
}

// A bounded wait that nothing ends: one warp of the back-substitution queue
// kernel waits for a queue slot that is never filled, with `spins` polls.
// Returns the error flag the wait set (1 when it ran out).  Test hook for the
// failure path: afterwards every active model of the engine fails with
// SS_TIMEOUT at its next convergence test.
int Engine::probeWaitTimeout(long long spins, int* flag) {
  int* q = nullptr;
  if (cudaMalloc(&q, sizeof(int) * 8) != cudaSuccess) return -955;
  const int init[8] = {-1, 0, 0, 0, 0, 0, 1, 0};  // queue slot 0 empty; ctr = {take 0, fill 0, total 1}
  cudaMemcpyAsync(q, init, sizeof(init), cudaMemcpyHostToDevice, stream_);
  launchBackwardWaitProbe(d_, pplan_, q, q + 4, spins, stream_);
  int f = 0;
  cudaMemcpyAsync(&f, pplan_.errFlag, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  const cudaError_t e = cudaStreamSynchronize(stream_);
  cudaFree(q);
  if (e != cudaSuccess) return -956;
  if (flag) *flag = f;
  return 0;
}

int Engine::probeRootWaitTimeout(long long spins, int* flag) {
  const int nf = d_.nfrontTot;
  if (nf <= 0 || d_.m.n <= 0) return -957;
  // a root of model 0, marked active for the probe (its flags are put back)
  std::vector<int> parent(nf), fmodel(nf);
  cudaMemcpyAsync(parent.data(), d_.fParent, sizeof(int) * nf, cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(fmodel.data(), d_.fModel, sizeof(int) * nf, cudaMemcpyDeviceToHost, stream_);
  int fl0 = 0;
  cudaMemcpyAsync(&fl0, d_.m.flags, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -956;
  int root = -1;
  for (int f = 0; f < nf && root < 0; ++f)
    if (parent[f] < 0 && fmodel[f] == 0) root = f;
  if (root < 0) return -957;
  // queue slot 0 = the root; ctr = {take 0, fill 1, total 1}; counters zero
  const size_t ints = 8 + (size_t)nf + 1;
  int* q = nullptr;
  if (cudaMalloc(&q, sizeof(int) * ints) != cudaSuccess) return -955;
  const int init[8] = {root, 0, 0, 0, 0, 1, 1, 0};
  cudaMemsetAsync(q, 0, sizeof(int) * ints, stream_);
  cudaMemcpyAsync(q, init, sizeof(init), cudaMemcpyHostToDevice, stream_);
  const int act = fl0 | FL_ACTIVE;
  cudaMemcpyAsync(d_.m.flags, &act, sizeof(int), cudaMemcpyHostToDevice, stream_);
  launchRootWaitProbe(d_, pplan_, q, q + 4, q + 8, spins, stream_);
  cudaMemcpyAsync(d_.m.flags, &fl0, sizeof(int), cudaMemcpyHostToDevice, stream_);
  int f = 0;
  cudaMemcpyAsync(&f, pplan_.errFlag, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  const cudaError_t e = cudaStreamSynchronize(stream_);
  cudaFree(q);
  if (e != cudaSuccess) return -956;
  if (flag) *flag = f;
  return 0;
}

int Engine::run(long long maxBatched, RunStats* stats) {
  ensureTuned();
  if (opt_.useGraph && !graphExec_) {
    cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal);
    enqueueIteration(stream_);
    if (cudaStreamEndCapture(stream_, &graph_) != cudaSuccess) return -920;
    if (cudaGraphInstantiate(&graphExec_, graph_, 0) != cudaSuccess) return -921;
  }
  if (!evRun_[0]) {
    cudaEventCreate(&evRun_[0]);
    cudaEventCreate(&evRun_[1]);
  }
  auto t0 = std::chrono::steady_clock::now();
  cudaEventRecord(evRun_[0], stream_);
  long long done = 0;
  // an odd chunk length: the phase durations are sampled from the last
  // iteration of each chunk, and with two iterations per time step an even
  // length would always sample the same kind (predictor or corrector)
  const int chunk = 7;
  while (done < maxBatched) {
    int n = (int)std::min<long long>(chunk, maxBatched - done);
    for (int k = 0; k < n; ++k) {
      if (opt_.useGraph) cudaGraphLaunch(graphExec_, stream_);
      else enqueueIteration(stream_);
    }
    done += n;
    cudaMemcpyAsync(hActiveEl_, dActiveEl_, sizeof(long long), cudaMemcpyDeviceToHost, stream_);
    int active = readActive();
    // sample the phase durations of the last iteration of this chunk
    float t0 = 0.f, t1 = 0.f, t2 = 0.f;
    if (cudaEventElapsedTime(&t0, ev_[3], ev_[4]) == cudaSuccess &&
        cudaEventElapsedTime(&t1, ev_[0], ev_[1]) == cudaSuccess &&
        cudaEventElapsedTime(&t2, ev_[1], ev_[2]) == cudaSuccess && (*hActiveEl_ > 0 || (active > 0 && d_.npartTot > 0))) {
      phaseMs_[0] += t0;
      phaseMs_[1] += t1;
      phaseMs_[2] += t2;
      float t3 = 0.0f;
      if (opt_.refineSweeps > 1 && cudaEventElapsedTime(&t3, ev_[5], ev_[6]) == cudaSuccess)
        phaseMs_[3] += t3;
      float t4 = 0.0f;
      if (cudaEventElapsedTime(&t4, ev_[7], ev_[8]) == cudaSuccess) phaseMs_[4] += t4;
      phaseElems_ += *hActiveEl_;
      ++phaseSamples_;
    }
    if (rec_.on) {
      std::string err;
      if (resultsDrain(err)) return -924;
    }
    if (active == 0) break;
  }
  cudaEventRecord(evRun_[1], stream_);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) return -922;
  if (cudaGetLastError() != cudaSuccess) return -923;
  lastRunSec_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  float devMs = 0.f;
  cudaEventElapsedTime(&devMs, evRun_[0], evRun_[1]);
  lastRunDevSec_ = 1.0e-3 * devMs;
  if (stats) {
    std::vector<long long> it(d_.m.n), st(d_.m.n);
    std::vector<int> state(d_.m.n);
    cudaMemcpy(it.data(), d_.m.nIter, sizeof(long long) * d_.m.n, cudaMemcpyDeviceToHost);
    cudaMemcpy(st.data(), d_.m.nStep, sizeof(long long) * d_.m.n, cudaMemcpyDeviceToHost);
    cudaMemcpy(state.data(), d_.m.state, sizeof(int) * d_.m.n, cudaMemcpyDeviceToHost);
    stats->newtonIterations = 0;
    stats->timeSteps = 0;
    stats->modelsDone = stats->modelsFailed = 0;
    for (int k = 0; k < d_.m.n; ++k) {
      stats->newtonIterations += it[k];
      stats->timeSteps += st[k];
      stats->modelsDone += state[k] == ST_DONE;
      stats->modelsFailed += state[k] == ST_ERROR;
    }
    stats->batchedIterations += done;
  }
  return 0;
}

int Engine::launchChunk(int n) {
  ensureTuned();
  if (opt_.useGraph && !graphExec_) {
    cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal);
    enqueueIteration(stream_);
    if (cudaStreamEndCapture(stream_, &graph_) != cudaSuccess) return -920;
    if (cudaGraphInstantiate(&graphExec_, graph_, 0) != cudaSuccess) return -921;
  }
  if (!evChunk_ && cudaEventCreateWithFlags(&evChunk_, cudaEventDisableTiming) != cudaSuccess) return -924;
  for (int k = 0; k < n; ++k) {
    if (opt_.useGraph) cudaGraphLaunch(graphExec_, stream_);
    else enqueueIteration(stream_);
  }
  cudaMemcpyAsync(hActive_, dActive_, sizeof(int), cudaMemcpyDeviceToHost, stream_);
  cudaMemcpyAsync(hStates_, d_.m.state, sizeof(int) * (size_t)d_.m.n, cudaMemcpyDeviceToHost, stream_);
  cudaEventRecord(evChunk_, stream_);
  chunkPending_ = true;
  return 0;
}

int Engine::pollChunk(bool* ready, int* active) {
  *ready = false;
  if (!chunkPending_) {
    *ready = true;
    *active = 1;
    return 0;
  }
  cudaError_t q = cudaEventQuery(evChunk_);
  if (q == cudaErrorNotReady) return 0;
  if (q != cudaSuccess) return -925;
  chunkPending_ = false;
  *ready = true;
  *active = *hActive_;
  if (rec_.on) {
    std::string err;
    if (resultsDrain(err)) return -926;
  }
  return 0;
}

long long Engine::totalIterations() {
  std::vector<long long> it(d_.m.n);
  cudaMemcpyAsync(it.data(), d_.m.nIter, sizeof(long long) * it.size(), cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  long long s = 0;
  for (long long v : it) s += v;
  return s;
}

void Engine::setStepLimit(long long lim) {
  std::vector<long long> v(d_.m.n, lim);
  cudaMemcpyAsync(d_.m.stepLimit, v.data(), sizeof(long long) * v.size(), cudaMemcpyHostToDevice, stream_);
  cudaStreamSynchronize(stream_);
}

int Engine::advanceOneStep(int m, int* state) {
  long long s0 = modelSteps(m);
  std::vector<long long> lim(d_.m.n, 0);
  lim[m] = s0 + 1;
  cudaMemcpyAsync(d_.m.stepLimit, lim.data(), sizeof(long long) * lim.size(), cudaMemcpyHostToDevice, stream_);
  int rc = run(1000000, nullptr);
  if (state) *state = modelState(m);
  return rc;
}

namespace {
template <typename T>
T readOne(const T* p, cudaStream_t s) {
  T v{};
  cudaMemcpyAsync(&v, p, sizeof(T), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  return v;
}
}  // namespace

int Engine::modelState(int m) { return readOne(d_.m.state + m, stream_); }
int Engine::modelStatus(int m) { return readOne(d_.m.status + m, stream_); }
double Engine::modelTime(int m) { return readOne(d_.m.time + m, stream_); }
double Engine::modelDt(int m) { return readOne(d_.m.dt + m, stream_); }
long long Engine::modelSteps(int m) { return readOne(d_.m.nStep + m, stream_); }
long long Engine::modelIterations(int m) { return readOne(d_.m.nIter + m, stream_); }

int Engine::getTriadUr(int m, double* ur) {
  int n = hm_[m]->ntri;
  cudaMemcpyAsync(ur, d_.ur + 12 * (size_t)modelTriOff_[m], sizeof(double) * 12 * n, cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  return n;
}

int Engine::getElementFrames(int m, double* supTr12) {
  const int n = hm_[m]->nel;
  std::vector<double> soa(12 * (size_t)n);
  for (int k = 0; k < 12; ++k)
    cudaMemcpyAsync(soa.data() + (size_t)k * n, d_.supTr + (size_t)k * d_.nelTot + modelElOff_[m],
                    sizeof(double) * n, cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  for (int e = 0; e < n; ++e)
    for (int k = 0; k < 12; ++k) supTr12[12 * (size_t)e + k] = soa[(size_t)k * n + e];
  return n;
}

int Engine::getNorms(int m, double* n18) {
  cudaMemcpyAsync(n18, d_.m.normVal + 18 * m, sizeof(double) * 18, cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  return 18;
}

int Engine::getCsrValues(int m, double* vals) {
  size_t n = hm_[m]->colInd.size();
  cudaMemcpyAsync(vals, d_.csrVal + modelSlotOff_[m], sizeof(double) * n, cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  return (int)n;
}

int Engine::getEqVector(int m, int which, double* v) {
  const double* src = which == 0 ? d_.FSk : which == 1 ? d_.FDk : which == 2 ? d_.FIk : which == 3 ? d_.Qk
                      : which == 4 ? d_.res : d_.del;
  int n = hm_[m]->neq;
  cudaMemcpyAsync(v, src + modelEqOff_[m], sizeof(double) * n, cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  return n;
}

}  // namespace fgpu
