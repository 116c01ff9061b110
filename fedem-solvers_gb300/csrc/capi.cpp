// capi.cpp -- the exported C ABI: the reference's solver-core entry points
// (src/vpmSolver/solverInterface.h, one model per process) and the batched
// fgpu_* API.  Both drive the same GPU engine; there is no CPU solver path.

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "eigen.h"
#include "../../include/fedem_solver_core.h"
#include "../../include/fgpu.h"
#include "engine.h"
#include "host_model.h"
#include "server.h"

using namespace fgpu;

namespace {

thread_local std::string g_lastError;

int fail(int code, const std::string& msg) {
  g_lastError = msg;
  return code;
}

// The device fgpu_set_device chose for the engines created from now on (-1:
// the calling thread's current device).  The library links its own CUDA
// runtime, so a device selected through another runtime (a framework's) is not
// seen here: callers on several GPUs must name theirs with fgpu_set_device.
std::atomic<int> g_device{-1};

int selectDevice(std::string& err) {
  const int dev = g_device.load();
  if (dev < 0) return 0;
  cudaError_t e = cudaSetDevice(dev);
  if (e != cudaSuccess) {
    err = std::string("cudaSetDevice failed: ") + cudaGetErrorString(e);
    return -960;
  }
  return 0;
}

// Makes an engine's device current for the rest of an entry point (each
// thread has its own current device in the CUDA runtime).
struct OnDevice {
  explicit OnDevice(int dev) {
    if (dev >= 0) cudaSetDevice(dev);
  }
};

// ---------------------------------------------------------------------------
// legacy singleton (solverInterface.C:49 keeps the same kind of global state)
// ---------------------------------------------------------------------------
struct Singleton {
  std::unique_ptr<HostModel> model;
  std::unique_ptr<Engine> engine;
  bool finished = false;
  bool inStep = false;  // startStep assembled an iteration that solveIteration has not solved
  int ierr = 0;
};
std::unique_ptr<Singleton> g_core;

bool readFileText(const std::string& path, std::string& text) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  std::stringstream ss;
  ss << in.rdbuf();
  text = ss.str();
  return true;
}

std::string optionValue(int argc, char** argv, const char* key) {
  std::string k = std::string("-") + key + "=";
  for (int a = 0; a < argc; ++a) {
    if (!argv || !argv[a]) continue;
    std::string s(argv[a]);
    if (s.compare(0, k.size(), k) == 0) {
      std::string v = s.substr(k.size());
      if (v.size() >= 2 && (v[0] == '"' || v[0] == '\'') && v.back() == v[0]) v = v.substr(1, v.size() - 2);
      return v;
    }
  }
  return std::string();
}

// a boolean option: -key, -key+ or -key=true/1 sets it, -key- or -key=false/0 clears it
bool optionBool(int argc, char** argv, const char* key, bool def) {
  const std::string k = std::string("-") + key;
  bool v = def;
  for (int a = 0; a < argc; ++a) {
    if (!argv || !argv[a]) continue;
    const std::string s(argv[a]);
    if (s == k || s == k + "+") v = true;
    else if (s == k + "-") v = false;
    else if (s.compare(0, k.size() + 1, k + "=") == 0) {
      const std::string w = s.substr(k.size() + 1);
      v = !(w == "0" || w == "false" || w == "f" || w == "no" || w == "off");
    }
  }
  return v;
}

bool hasFlag(int argc, char** argv, const char* key) {
  std::string k = std::string("-") + key;
  for (int a = 0; a < argc; ++a)
    if (argv && argv[a] && (k == argv[a] || k + "+" == argv[a])) return true;
  return false;
}

int triadIndex(const HostModel& m, int id) {
  for (int t = 0; t < m.ntri; ++t)
    if (m.triId[t] == id) return t;
  return -1;
}

bool hasReachedEnd(const Singleton& s) {
  const Control& c = s.model->ctl;
  double t = s.engine->modelTime(0);
  return c.tStart <= c.tEnd && t + 0.1 * c.minInc > c.tEnd;
}

}  // namespace

struct fgpu_model {
  HostModel m;
};

struct fgpu_batch {
  Engine engine;
  std::vector<const HostModel*> models;
  RunStats stats;
};

struct fgpu_server {
  Server srv;
};

extern "C" {

// ===========================================================================
// solverInterface.h entry points
// ===========================================================================

int solverInit(int argc, char** argv, const char* cfsi, const double* stateData, int ndat,
               const double* /*gagesData*/, int /*ngda*/, const double* extInput, int* nxinp) {
  g_core.reset();
  std::string text;
  if (cfsi) {
    text = cfsi;
  } else {
    std::string path = optionValue(argc, argv, "fsifile");
    if (path.empty()) return fail(-1, "no model: give cfsi or -fsifile");
    if (!readFileText(path, text)) return fail(-2, "cannot read " + path);
  }
  auto s = std::make_unique<Singleton>();
  s->model = std::make_unique<HostModel>();
  std::string err;
  const char* const* cargv = const_cast<const char* const*>(argv);
  int rc = buildModel(text.c_str(), argc, cargv, *s->model, err);
  if (rc) return fail(rc < 0 ? rc : -100 - rc, err);
  // initial external function values (solverInterface.C:575-576): extInput[0..*nxinp)
  if (extInput && nxinp && *nxinp > 0) {
    s->model->extInit.assign(extInput, extInput + std::min(*nxinp, s->model->nExt));
    s->model->extInit.resize(s->model->nExt, 0.0);
  }
  EngineOptions opt;
  opt.fp32Factor = hasFlag(argc, argv, "gpuMixed");
  opt.refineSweeps = opt.fp32Factor ? 4 : 1;
  if ((rc = selectDevice(err))) return fail(rc, err);
  s->engine = std::make_unique<Engine>();
  std::vector<const HostModel*> ms{s->model.get()};
  rc = s->engine->upload(ms, opt, err);
  if (!rc) rc = s->engine->initialState(err);
  if (rc) return fail(rc, err);
  if (s->engine->modelState(0) == ST_ERROR) {  // the initial static equilibrium failed
    const int st = s->engine->modelStatus(0);
    return fail((st & SS_SINGULAR) ? -3 : -1,
                (st & SS_SINGULAR) ? "singular system matrix in the initial static equilibrium"
                                   : "the initial static equilibrium failed");
  }
  if (stateData && ndat > 0) {  // restart from an in-core state array (saveState of the same model)
    if ((size_t)ndat * sizeof(double) < s->engine->stateBytes()) return fail(-2, "state array too short");
    if (s->engine->restoreStateFrom(stateData)) return fail(-3, "restoring the state failed");
  }
  // primary response database (solverModule.f90:352, saveStep at :512-513 and
  // after every step; -double1, -savestart as solverInterface.C:390-391)
  const std::string frs1 = optionValue(argc, argv, "frs1file");
  if (!frs1.empty()) {
    const std::string ss = optionValue(argc, argv, "savestart");
    const std::vector<std::string> paths{frs1};
    if ((rc = s->engine->resultsOpen("", optionBool(argc, argv, "double1", true), err, &paths,
                                     ss.empty() ? 0.0 : std::atof(ss.c_str()))))
      return fail(rc, err);
  }
  g_core = std::move(s);
  return 0;
}

// solverInterface.h:87 -- the engine's mutable state from a saveState array
// (results database options are not part of this path and are ignored)
int restartFromState(const double* stateData, const int ndat, const int) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || !stateData) return fail(-1, "no model or no state data");
  const size_t bytes = g_core->engine->stateBytes();
  if ((size_t)ndat * sizeof(double) < bytes) return fail(-2, "state array too short");
  if (int rc = g_core->engine->restoreStateFrom(stateData)) return fail(rc, "restoring the state failed");
  g_core->inStep = false;
  g_core->ierr = 0;
  g_core->finished = false;
  return 0;
}

// solverInterface.h:110 (solverInterface.C:858-910) -- nStep steps; before
// each, the step's time (times, nInc >= nStep) and the external function values
// 1..nIn (inputs, nIn per step) are applied; after each, the nOut functions
// fOut are evaluated into outputs (nOut per step); the state is saved into
// stateData at the end when nDat > 0.  False at the end of the simulation or
// on error (*ierr != 0).
bool solveWindow(int nStep, int nInc, int nIn, int nOut, const int* fOut, const double* times,
                 const double* inputs, double* outputs, int nDat, double* stateData, int* ierr) {
  int lerr = 0;
  int& e = ierr ? *ierr : lerr;
  e = 0;
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || g_core->ierr) {
    e = g_core ? g_core->ierr : -1;
    return false;
  }
  if (!times) nInc = 0;
  if (!inputs) nIn = 0;
  if (!outputs || !fOut) nOut = 0;
  if (!stateData) nDat = 0;
  if (nInc > 0 && nInc < nStep) {
    e = nInc - nStep;  // too short times array
    return false;
  }
  bool more = true;
  for (int i = 0; i < nStep && more && e == 0; ++i) {
    if (nInc > 0 && !setTime(times[i])) e = -1;
    for (int j = 0; j < nIn; ++j)
      if (!setExtFunc(1 + j, inputs[(size_t)i * nIn + j])) --e;
    if (e == 0) more = solveNext(&e);
    for (int j = 0; j < nOut && e == 0; ++j) outputs[(size_t)i * nOut + j] = evalFunc(fOut[j], nullptr, -1.0, &e);
  }
  if (e == 0 && nDat > 0 && !saveState(stateData, nDat)) e = -2;
  return e == 0 && more;
}

// solverInterface.h:118 -- doubles needed by saveState
int getStateSize(void) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) return 0;
  return (int)((g_core->engine->stateBytes() + sizeof(double) - 1) / sizeof(double));
}
int getTransformationStateSize(void) { return 0; }
int getPartDeformationStateSize(int) { return 0; }
int getPartStressStateSize(int) { return 0; }
int getGagesSize(void) { return 0; }
// solverInterface.h:156 -- the mutable state (positions, velocities, frames,
// forces, step and iteration counters) into an in-core array
bool saveState(double* stateData, const int ndat) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || !stateData || g_core->inStep) return false;
  if ((size_t)ndat * sizeof(double) < g_core->engine->stateBytes()) return false;
  return g_core->engine->saveStateTo(stateData) == 0;
}
bool saveTransformationState(double*, const int) { return false; }
bool saveGages(double*, const int) { return false; }
bool savePartDeformationState(int, double*, const int) { return false; }
bool savePartStressState(int, double*, const int) { return false; }
bool getStrainsFromDisp(const double*, const int*, double*, const int, const int) { return false; }
bool getBeamForcesFromDisp(const double*, const int*, double*, const int, const int) { return false; }
bool getRelDisp(const double*, const int*, double*, const int, const int) { return false; }
bool getRespVars(const double*, const int*, double*, const int, const int) { return false; }

bool solveNext(int* ierr) {
  if (ierr) *ierr = 0;
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) {
    if (ierr) *ierr = -1;
    return false;
  }
  Singleton& s = *g_core;
  if (s.ierr) {
    if (ierr) *ierr = s.ierr;
    return false;
  }
  if (s.inStep) return solveIteration(ierr, true);  // finish the step startStep began
  if (hasReachedEnd(s)) return false;
  int state = 0;
  int rc = s.engine->advanceOneStep(0, &state);
  if (rc || state == ST_ERROR) {
    int st = s.engine->modelStatus(0);
    s.ierr = rc ? rc : (st & SS_SINGULAR) ? -3 : (st & SS_MAXIT) ? 1 : -1;
    if (ierr) *ierr = s.ierr;
    return false;
  }
  s.finished = hasReachedEnd(s);
  return !s.finished;
}

// solverInterface.h:262 -- predictor and the first linearised system of the next step
bool startStep(int* ierr) {
  int lerr = 0;
  int& e = ierr ? *ierr : lerr;
  e = 0;
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || g_core->ierr) {
    e = g_core ? g_core->ierr : -1;
    return false;
  }
  Singleton& s = *g_core;
  if (s.inStep) {
    e = -999;  // a step is already started (the reference's state check)
    return false;
  }
  if (hasReachedEnd(s)) return false;
  s.engine->setStepLimitOf(0, s.engine->modelSteps(0) + 1);
  if (int rc = s.engine->assembleIteration()) {
    s.ierr = e = rc;
    return false;
  }
  s.inStep = true;
  return true;
}

// solverInterface.h:278 -- solves the assembled system, updates the model and
// assembles the next iteration unless converged; with `all`, until convergence
bool solveIteration(int* ierr, bool all) {
  int lerr = 0;
  int& e = ierr ? *ierr : lerr;
  e = 0;
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || g_core->ierr) {
    e = g_core ? g_core->ierr : -1;
    return false;
  }
  Singleton& s = *g_core;
  if (!s.inStep) {
    e = -999;  // step not started
    return false;
  }
  for (;;) {
    if (int rc = s.engine->solveUpdateIteration()) {
      s.ierr = e = rc;
      return false;
    }
    const int state = s.engine->modelState(0);
    if (state == ST_ERROR) {
      const int st = s.engine->modelStatus(0);
      s.ierr = e = (st & SS_SINGULAR) ? -3 : (st & SS_MAXIT) ? 1 : -1;
      s.inStep = false;
      return false;
    }
    if (state == ST_NEED_STEP) {  // converged: the step is complete
      s.inStep = false;
      s.finished = hasReachedEnd(s);
      return all ? !s.finished : false;
    }
    if (int rc = s.engine->assembleIteration()) {
      s.ierr = e = rc;
      return false;
    }
    if (!all) return true;
  }
}
// solverInterface.h:293 (solverModule.f90:1004-1092) -- the nmod lowest
// eigenmodes of K phi = lambda M phi at the current state: eval = sqrt|lambda|
// / 2 pi (Hz), evec = M-orthonormal eigenvectors, nmod columns in equation
// order (neq each) or DOF order (ndof each, zero at fixed and prescribed DOFs).
// *ierr = number of negative eigenvalues, or a positive count when the Lanczos
// iteration did not converge every mode; < 0 on error.  useLaPack is ignored
// (one Lanczos solver).  Between steps only.
bool solveEigenModes(const int nmod, double* eval, double* evec, bool dofOrder, int, int* ierr) {
  int lerr = 0;
  int& e = ierr ? *ierr : lerr;
  e = 0;
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || g_core->ierr || !eval) {
    e = g_core ? (g_core->ierr ? g_core->ierr : -1) : -1;
    return false;
  }
  Singleton& s = *g_core;
  if (s.inStep) {
    e = -999;
    return false;
  }
  const HostModel& m = *s.model;
  if (m.njoint > 0 || m.npart > 0) {
    // the mass matrix of the eigenproblem is assembled from the beam elements
    // on the host; joints' constraint equations and parts are not in it
    e = -998;
    return false;
  }
  std::vector<double> lambda, vecs;
  int nNeg = 0;
  const int rc = lowestModes(*s.engine, m, nmod, lambda, vecs, nNeg);
  if (rc < 0) {
    e = rc;
    return false;
  }
  const double twoPi = 8.0 * std::atan(1.0);
  for (int k = 0; k < nmod; ++k) eval[k] = std::sqrt(std::fabs(lambda[k])) / twoPi;
  if (evec) {
    for (int k = 0; k < nmod; ++k) {
      const double* v = &vecs[(size_t)m.neq * k];
      if (dofOrder) {
        double* o = evec + (size_t)m.ndof * k;
        for (int i = 0; i < m.ndof; ++i) o[i] = m.meqn[i] >= 0 ? v[m.meqn[i]] : 0.0;
      } else {
        std::memcpy(evec + (size_t)m.neq * k, v, sizeof(double) * m.neq);
      }
    }
  }
  e = nNeg + rc;
  return true;
}
bool solveInverse(const double*, const int*, const int*, int, int, int* ierr) {
  if (ierr) *ierr = -1;
  return false;
}

int solverDone(bool) {
  g_core.reset();
  return 0;
}
void solverClose(void) { g_core.reset(); }

// solverInterface.h:342 -- value of external function channel funcId (1-based)
// for the next step; false when the model has no such channel
bool setExtFunc(int funcId, double value) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) return false;
  return g_core->engine->setExtValue(0, funcId - 1, value) == 0;
}

double getTime(bool nextStep, int* ierr) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) {
    if (ierr) *ierr = -1;
    return 0.0;
  }
  if (ierr) *ierr = 0;
  double t = g_core->engine->modelTime(0);
  return nextStep ? t + g_core->engine->modelDt(0) : t;
}

// solverInterface.h:355 -- time increment of the next step: nextTime - time
// (solverModule.f90:1558-1600: a negative increment or one above maxInc is an
// error, one below minInc is raised to it)
bool setTime(double nextTime) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || g_core->inStep) return false;
  const Control& c = g_core->model->ctl;
  const double dt = nextTime - g_core->engine->modelTime(0);
  if (dt < 0.0) return false;
  if (dt >= c.minInc && dt > c.maxInc) return false;
  return g_core->engine->setTimeStep(0, dt < c.minInc ? c.minInc : dt) == 0;
}

// solverInterface.h:383 -- value of the engine with user id uid, or (with a
// tag) of the first engine with that tag (solverModule.f90:1602-1640:
// a user id match wins; no match gives zero); x >= 0 without a tag
// evaluates the engine's function at x instead of its current argument
double evalFunc(int uid, const char* tag, double x, int* ierr) {
  int lerr = 0;
  int& e = ierr ? *ierr : lerr;
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) {
    e = -999;  // outside model scope
    return 0.0;
  }
  Singleton& s = *g_core;
  const HostModel& m = *s.model;
  const bool hasX = !tag && x >= 0.0;
  auto value = [&](size_t k) {
    if (m.engFType[k] == 3) return s.engine->extValue(0, m.engCh[k]);
    if (m.engFType[k] == 2) return m.engFc[k];
    const double arg = hasX ? x : (m.engTimeArg[k] ? s.engine->modelTime(0) : 0.0);
    if (m.engFType[k] == 4) {  // SINUSOIDAL: frequency, delay, amplitude, mean
      const double* sp = &m.engSin[4 * k];
      return sp[3] + sp[2] * std::sin(2.0 * M_PI * (sp[0] * arg - sp[1]));
    }
    return m.engFType[k] == 1 ? m.engFc[k] * arg : arg;
  };
  bool found = false;
  double tagValue = 0.0;
  for (size_t k = 0; k < m.engId.size(); ++k) {
    if (m.engUserId[k] == uid) return value(k);
    if (tag && !found && m.engTag[k] == tag) {
      found = true;
      tagValue = value(k);
      if (uid <= 0) return tagValue;
    }
  }
  return 0.0;  // no such engine: zero
}
// solverInterface.h:398 -- user id of the first engine with the tag, -1 if none
int getFuncId(const char* tag) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) return -999;
  if (!tag) return -1;
  const HostModel& m = *g_core->model;
  for (size_t k = 0; k < m.engId.size(); ++k)
    if (m.engTag[k] == tag) return m.engUserId[k];
  return -1;
}

int getEquations(int bid, int* meqn) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) return 0;
  const HostModel& m = *g_core->model;
  int t = triadIndex(m, bid);
  if (t < 0) return 0;
  for (int k = 0; k < m.triNdof[t]; ++k) meqn[k] = m.meqn[m.triFirstDof[t] + k] + 1;
  return m.triNdof[t];
}

int getStateVar(int bid, double* var) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) return 0;
  const HostModel& m = *g_core->model;
  int t = triadIndex(m, bid);
  if (t < 0 || m.triNdof[t] < 3) return 0;
  std::vector<double> ur(12 * (size_t)m.ntri);
  g_core->engine->getTriadUr(0, ur.data());
  for (int r = 0; r < 3; ++r) var[r] = ur[12 * (size_t)t + 9 + r];
  return 3;
}

int getSystemSize(bool dofs) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) return 0;
  return dofs ? g_core->model->ndof : g_core->model->neq;
}

// Dense system stiffness (1), mass (2) or damping (3) matrix at the current
// configuration: the element matrices rotated to system axes with the current
// frames (as AddInSupMat / MATTRA), the axial springs' and dampers' n n^T blocks
// (calcSpringStiffness without geometric stiffness, addInDamperMat), assembled
// over the free equations.
static void assembleSystemMatrix(int iMat, double* Smat) {
  const HostModel& m = *g_core->model;
  const int neq = m.neq;
  std::memset(Smat, 0, sizeof(double) * (size_t)neq * neq);
  std::vector<double> frames(12 * (size_t)m.nel), ur(12 * (size_t)m.ntri);
  g_core->engine->getElementFrames(0, frames.data());
  g_core->engine->getTriadUr(0, ur.data());
  auto add = [&](int i, int j, double v) { Smat[(size_t)i + (size_t)neq * j] += v; };
  for (int e = 0; e < m.nel; ++e) {
    const double* X = iMat == 1 ? &m.K[144 * (size_t)e] : iMat == 2 ? &m.M[144 * (size_t)e] : &m.C[144 * (size_t)e];
    if (iMat == 3 && !m.hasC[e]) continue;
    const double scl = iMat == 2 ? 1.0 : m.stifScl[e];
    const double* R = &frames[12 * (size_t)e];  // column-major 3x3 rotation first
    const int* q = &m.elEq[12 * (size_t)e];
    for (int bj = 0; bj < 4; ++bj)
      for (int bi = 0; bi < 4; ++bi) {
        double W[9];
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) {
            double v = 0.0;
            for (int k = 0; k < 3; ++k) v += R[r + 3 * k] * (scl * X[(3 * bi + k) + 12 * (3 * bj + c)]);
            W[r + 3 * c] = v;
          }
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) {
            const int i = q[3 * bi + r], j = q[3 * bj + c];
            if (i < 0 || j < 0) continue;
            double v = 0.0;
            for (int k = 0; k < 3; ++k) v += W[r + 3 * k] * R[c + 3 * k];
            add(i, j, v);
          }
      }
  }
  for (int a = 0; a < m.nax; ++a) {
    const double* x1 = &ur[12 * (size_t)m.axTri[2 * a] + 9];
    const double* x2 = &ur[12 * (size_t)m.axTri[2 * a + 1] + 9];
    double n[3] = {x2[0] - x1[0], x2[1] - x1[1], x2[2] - x1[2]};
    const double L = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(L > 0.0)) continue;
    for (double& c : n) c /= L;
    double coeff = 0.0;
    if (m.axKind[a] == 0) coeff = iMat == 1 ? m.axS0[a] : iMat == 3 ? m.axS0[a] * m.axAlpha2[a] : 0.0;
    else coeff = iMat == 3 ? m.axD0[a] : 0.0;
    if (coeff == 0.0) continue;
    const int* q = &m.axEq[6 * (size_t)a];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        if (q[i] < 0 || q[j] < 0) continue;
        const double v = n[i % 3] * n[j % 3] * coeff;
        add(q[i], q[j], (i / 3 == j / 3) ? v : -v);
      }
  }
}

bool getSystemMatrix(double* Smat, int iMat) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || !Smat || iMat < 0 || iMat > 3) return false;
  const HostModel& m = *g_core->model;
  if (iMat > 0) {
    // assembled on the host from the beam elements and axial springs/dampers;
    // joints' constraint equations and parts are not in it
    if (m.njoint > 0 || m.npart > 0) return false;
    assembleSystemMatrix(iMat, Smat);
    return true;
  }
  std::vector<double> v(m.colInd.size());
  g_core->engine->getCsrValues(0, v.data());
  std::memset(Smat, 0, sizeof(double) * (size_t)m.neq * m.neq);
  for (int i = 0; i < m.neq; ++i)
    for (int k = m.rowPtr[i]; k < m.rowPtr[i + 1]; ++k) Smat[(size_t)i + (size_t)m.neq * m.colInd[k]] = v[k];
  return true;
}
bool getNewtonMatrix(double* Nmat) { return getSystemMatrix(Nmat, 0); }
bool getStiffnessMatrix(double* Kmat) { return getSystemMatrix(Kmat, 1); }
bool getMassMatrix(double* Mmat) { return getSystemMatrix(Mmat, 2); }
bool getDampingMatrix(double* Cmat) { return getSystemMatrix(Cmat, 3); }

bool getElementStiffnessMatrix(double* Kmat, int bid) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core) return false;
  const HostModel& m = *g_core->model;
  for (int e = 0; e < m.nel; ++e)
    if (m.elId[e] == bid) {
      std::memcpy(Kmat, &m.K[144 * (size_t)e], sizeof(double) * 144);
      return true;
    }
  return false;
}

// solverInterface.h:472 -- iVec < 5: the current right-hand side of the
// linearised system (solverModule.f90:1834-1849), 5: the external load vector
bool getRhsVector(double* Rvec, int iVec) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || !Rvec) return false;
  g_core->engine->getEqVector(0, iVec == 5 ? 3 : 5, Rvec);
  return true;
}
// solverInterface.h:478-484 -- replace / add to the right-hand side of the
// iteration assembled by startStep or solveIteration
bool setRhsVector(const double* Rvec) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || !Rvec || !g_core->inStep) return false;
  return g_core->engine->setRhs(0, Rvec, false) == 0;
}
bool addRhsVector(const double* Rvec) {
  OnDevice onDev(g_core ? g_core->engine->device() : -1);
  if (!g_core || !Rvec || !g_core->inStep) return false;
  return g_core->engine->setRhs(0, Rvec, true) == 0;
}
bool getJointSprCoeff(double*, int) { return false; }

// ===========================================================================
// fgpu.h batched API
// ===========================================================================

int fgpu_model_create(const char* fsi, int argc, const char* const* argv, fgpu_model** out) {
  if (!out) return fail(-1, "null output handle");
  *out = nullptr;
  auto h = std::make_unique<fgpu_model>();
  std::string err;
  int rc = buildModel(fsi, argc, argv, h->m, err);
  if (rc) return fail(rc, err);
  *out = h.release();
  return 0;
}

void fgpu_model_destroy(fgpu_model* m) { delete m; }

int fgpu_model_sizes(const fgpu_model* h, long long* s) {
  if (!h || !s) return fail(-1, "null argument");
  const HostModel& m = h->m;
  s[0] = m.ntri; s[1] = m.ndof; s[2] = m.neq; s[3] = m.nel; s[4] = (long long)m.colInd.size();
  s[5] = (long long)m.fronts.size(); s[6] = m.maxFront; s[7] = m.maxHeight + 1;
  return 0;
}

int fgpu_model_meqn(const fgpu_model* h, int* meqn) {
  if (!h || !meqn) return fail(-1, "null argument");
  for (int i = 0; i < h->m.ndof; ++i) meqn[i] = h->m.meqn[i] + 1;
  return 0;
}

int fgpu_model_csr_pattern(const fgpu_model* h, int* rowptr, int* cols) {
  if (!h) return fail(-1, "null argument");
  if (rowptr) std::memcpy(rowptr, h->m.rowPtr.data(), sizeof(int) * h->m.rowPtr.size());
  if (cols) std::memcpy(cols, h->m.colInd.data(), sizeof(int) * h->m.colInd.size());
  return 0;
}

int fgpu_model_symbolic(const fgpu_model* h, int* perm, int* info4) {
  if (!h) return fail(-1, "null argument");
  if (perm) std::memcpy(perm, h->m.perm.data(), sizeof(int) * h->m.perm.size());
  if (info4)
    for (size_t f = 0; f < h->m.fronts.size(); ++f) {
      const Front& fr = h->m.fronts[f];
      info4[4 * f] = fr.npiv; info4[4 * f + 1] = fr.nrow; info4[4 * f + 2] = fr.parent; info4[4 * f + 3] = fr.height;
    }
  return 0;
}

int fgpu_model_element_matrix(const fgpu_model* h, int iel, int which, double* mat) {
  if (!h || !mat || iel < 0 || iel >= h->m.nel || which < 0 || which > 2) return fail(-1, "bad argument");
  const std::vector<double>& src = which == 0 ? h->m.K : which == 1 ? h->m.M : h->m.C;
  std::memcpy(mat, &src[144 * (size_t)iel], sizeof(double) * 144);
  return 0;
}

int fgpu_batch_create(int n, fgpu_model* const* models, int mixed, int sweeps, fgpu_batch** out) {
  if (!out || !models || n <= 0) return fail(-1, "bad argument");
  *out = nullptr;
  auto b = std::make_unique<fgpu_batch>();
  for (int k = 0; k < n; ++k) {
    if (!models[k]) return fail(-1, "null model handle");
    b->models.push_back(&models[k]->m);
  }
  EngineOptions opt;
  opt.fp32Factor = mixed != 0;
  opt.refineSweeps = sweeps > 0 ? sweeps : (mixed ? 2 : 1);
  std::string err;
  int rc = selectDevice(err);
  if (!rc) rc = b->engine.upload(b->models, opt, err);
  if (!rc) rc = b->engine.initialState(err);
  if (rc) return fail(rc, err);
  *out = b.release();
  return 0;
}

void fgpu_batch_destroy(fgpu_batch* b) { delete b; }

int fgpu_batch_run(fgpu_batch* b, long long maxBatched, long long* s8) {
  if (!b) return fail(-1, "null batch");
  OnDevice onDev(b->engine.device());
  RunStats st;
  b->engine.setStepLimit(1LL << 62);
  int rc = b->engine.run(maxBatched > 0 ? maxBatched : (1LL << 40), &st);
  if (rc) return fail(rc, "batched run failed (CUDA error)");
  if (s8) {
    s8[0] = st.newtonIterations; s8[1] = st.timeSteps; s8[2] = st.batchedIterations;
    s8[3] = st.modelsDone; s8[4] = st.modelsFailed; s8[5] = b->engine.launchesPerIteration();
    s8[6] = (long long)(b->engine.lastRunSeconds() * 1.0e6);
    s8[7] = (long long)(b->engine.lastRunDeviceSeconds() * 1.0e6);
    s8[8] = b->engine.uploadedBytes();
    s8[9] = 0;
  }
  return 0;
}

int fgpu_batch_model_info(fgpu_batch* b, int k, int* state, int* status, double* time, long long* steps,
                          long long* iters) {
  if (!b || k < 0 || k >= b->engine.numModels()) return fail(-1, "bad model index");
  OnDevice onDev(b->engine.device());
  if (state) *state = b->engine.modelState(k);
  if (status) *status = b->engine.modelStatus(k);
  if (time) *time = b->engine.modelTime(k);
  if (steps) *steps = b->engine.modelSteps(k);
  if (iters) *iters = b->engine.modelIterations(k);
  return 0;
}

int fgpu_batch_get_triads(fgpu_batch* b, int k, double* ur) {
  if (!b || !ur || k < 0 || k >= b->engine.numModels()) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  b->engine.getTriadUr(k, ur);
  return 0;
}

long long fgpu_batch_get_all_triads(fgpu_batch* b, double* ur) {
  if (!b || !ur) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  long long off = 0;
  for (int k = 0; k < b->engine.numModels(); ++k) off += 12LL * b->engine.getTriadUr(k, ur + off);
  return off;
}

int fgpu_batch_get_newton_values(fgpu_batch* b, int k, double* vals) {
  if (!b || !vals || k < 0 || k >= b->engine.numModels()) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  b->engine.getCsrValues(k, vals);
  return 0;
}

int fgpu_batch_get_vector(fgpu_batch* b, int k, int which, double* v) {
  if (!b || !v || k < 0 || k >= b->engine.numModels() || which < 0 || which > 5) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  b->engine.getEqVector(k, which, v);
  return 0;
}

int fgpu_batch_get_norms(fgpu_batch* b, int k, double* n18) {
  if (!b || !n18 || k < 0 || k >= b->engine.numModels()) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  b->engine.getNorms(k, n18);
  return 0;
}

int fgpu_batch_norms_noalloc(fgpu_batch* b, int k, double* n18) {
  if (!b || !n18 || k < 0 || k >= b->engine.numModels()) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  std::string err;
  int rc = normsNoAlloc(b->engine.devData(), k, b->engine.normChunkOffset(k), b->engine.normChunkCount(k),
                        b->engine.device(), b->engine.stream(), n18, err);
  return rc ? fail(rc, err) : 0;
}

int fgpu_batch_step(fgpu_batch* b, int k, int* state) {
  if (!b || k < 0 || k >= b->engine.numModels()) return fail(-1, "bad model index");
  OnDevice onDev(b->engine.device());
  int rc = b->engine.advanceOneStep(k, state);
  return rc ? fail(rc, "step failed") : 0;
}

int fgpu_batch_snapshot(fgpu_batch* b) {
  if (!b) return fail(-1, "null batch");
  OnDevice onDev(b->engine.device());
  int rc = b->engine.snapshot();
  return rc ? fail(rc, "snapshot failed") : 0;
}

int fgpu_batch_restore(fgpu_batch* b) {
  if (!b) return fail(-1, "null batch");
  OnDevice onDev(b->engine.device());
  int rc = b->engine.restore();
  return rc ? fail(rc, "restore failed (no snapshot?)") : 0;
}

long long fgpu_batch_phase_timings(fgpu_batch* b, double* ms4, long long* elems, int reset) {
  if (!b || !ms4) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  long long n = b->engine.phaseTimings(ms4, elems);
  if (reset) b->engine.resetPhaseTimings();
  return n;
}

long long fgpu_batch_phase_timings_n(fgpu_batch* b, double* ms, int n, long long* elems, int reset) {
  if (!b || !ms || n < 1 || n > 5) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  long long k = b->engine.phaseTimings(ms, elems, n);
  if (reset) b->engine.resetPhaseTimings();
  return k;
}

int fgpu_batch_time_factor(fgpu_batch* b, int reps, double* out2) {
  if (!b || !out2 || reps < 1) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  return b->engine.timeFactor(reps, out2, out2 + 1);
}

int fgpu_batch_set_launch_shape(fgpu_batch* b, const int* shape4) {
  if (!b || !shape4) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  const int rc = b->engine.setLaunchShape(shape4);
  if (rc == -1) return fail(-2, "launch shapes can only be set before the batch's first iteration");
  if (rc < 0) return fail(-3, "launch shape out of range (panel 0/1/2, warps 4/8/16, cluster 2/4/8/16)");
  return 0;
}

int fgpu_batch_results_open(fgpu_batch* b, const char* dir, int doublePrecision) {
  if (!b || !dir) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  std::string err;
  if (int rc = b->engine.resultsOpen(dir, doublePrecision != 0, err)) return fail(rc, err);
  return 0;
}

int fgpu_batch_results_close(fgpu_batch* b) {
  if (!b) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  std::string err;
  if (int rc = b->engine.resultsClose(err)) return fail(rc, err);
  return 0;
}

int fgpu_batch_assemble_newton(fgpu_batch* b, int model, double sM, double sC, double sK) {
  if (!b || model < 0 || model >= b->engine.numModels()) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  const int rc = b->engine.seamAssemble(model, sM, sC, sK);
  if (rc == -2) return fail(rc, "the model is inside a time step");
  return rc ? fail(rc, "assembly failed") : 0;
}

int fgpu_batch_factor(fgpu_batch* b, int model) {
  if (!b || model < 0 || model >= b->engine.numModels()) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  const int rc = b->engine.seamFactor(model);
  if (rc == -3) return fail(rc, "singular Newton matrix");
  if (rc == -2) return fail(rc, "the model is inside a time step");
  return rc < 0 ? fail(rc, "factorisation failed") : rc;
}

int fgpu_batch_solve(fgpu_batch* b, int model, double* rhs, int nrhs) {
  if (!b || !rhs || model < 0 || model >= b->engine.numModels() || nrhs < 0) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  const int rc = b->engine.seamSolve(model, rhs, nrhs);
  if (rc == -2) return fail(rc, "the model is inside a time step");
  if (rc == -5) return fail(rc, "a bounded wait of the back substitution ran out");
  return rc ? fail(rc, "solve failed") : 0;
}

int fgpu_batch_launch_shape(fgpu_batch* b, int* shape4, double* probeMs) {
  if (!b || !shape4) return fail(-1, "bad argument");
  return b->engine.launchShape(shape4, probeMs);
}

int fgpu_server_create(double budget, int mixed, int sweeps, int maxModels, int minBatch, double maxWait,
                       fgpu_server** out) {
  if (!out) return fail(-1, "null output handle");
  EngineOptions opt;
  opt.fp32Factor = mixed != 0;
  opt.refineSweeps = sweeps > 0 ? sweeps : (mixed ? 2 : 1);
  std::string err;
  if (int rc = selectDevice(err)) return fail(rc, err);
  int dev = 0;
  cudaGetDevice(&dev);
  auto* s = new fgpu_server{Server((size_t)(budget > 0 ? budget : 64.0e9), opt, maxModels, 4, dev)};
  s->srv.setBatchingWindow(minBatch, maxWait);
  *out = s;
  return 0;
}

void fgpu_server_destroy(fgpu_server* s) { delete s; }

int fgpu_server_submit(fgpu_server* s, fgpu_model* m, int* id) {
  if (!s || !m) return fail(-1, "bad argument");
  int r = s->srv.submit(&m->m);
  if (id) *id = r;
  return 0;
}

int fgpu_server_pump(fgpu_server* s) {
  if (!s) return fail(-1, "null server");
  int rc = s->srv.pump();
  return rc < 0 ? fail(rc, ("server pump failed (" + std::to_string(rc) + ")").c_str()) : rc;
}

int fgpu_server_status(fgpu_server* s, long long* st) {
  if (!s || !st) return fail(-1, "bad argument");
  st[0] = s->srv.numRequests();
  st[1] = s->srv.pending();
  st[2] = s->srv.liveEngines();
  st[3] = (long long)s->srv.bytesInUse();
  return 0;
}

int fgpu_server_set_max_engines(fgpu_server* s, int n) {
  if (!s) return fail(-1, "bad argument");
  s->srv.setMaxEngines(n);
  return 0;
}

int fgpu_server_slot_reuse(fgpu_server* s, double share, long long* rebatches) {
  if (!s) return fail(-1, "bad argument");
  if (share >= 0.0) s->srv.setSlotReuse(share);
  if (rebatches) *rebatches = s->srv.rebatches();
  return 0;
}

double fgpu_server_now(fgpu_server* s) { return s ? s->srv.now() : 0.0; }

int fgpu_server_request(fgpu_server* s, int id, int* state, double* t3, long long* iters, long long* steps) {
  if (!s || id < 0 || id >= s->srv.numRequests()) return fail(-1, "bad request id");
  const Request& r = s->srv.request(id);
  if (state) *state = r.state;
  if (t3) { t3[0] = r.arrival; t3[1] = r.admitted; t3[2] = r.finished; }
  if (iters) *iters = r.iterations;
  if (steps) *steps = r.steps;
  return 0;
}

int fgpu_server_result(fgpu_server* s, int id, double* ur) {
  if (!s || !ur || id < 0 || id >= s->srv.numRequests()) return fail(-1, "bad argument");
  const Request& r = s->srv.request(id);
  if (r.state != 2) return fail(-2, "request not finished");
  std::memcpy(ur, r.ur.data(), sizeof(double) * r.ur.size());
  return 0;
}

int fgpu_batch_probe_wait_timeout(fgpu_batch* b, long long spins, int* flag) {
  if (!b || spins < 1) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  int rc = b->engine.probeWaitTimeout(spins, flag);
  return rc ? fail(rc, "wait probe failed") : 0;
}

int fgpu_batch_probe_root_wait_timeout(fgpu_batch* b, long long spins, int* flag) {
  if (!b || spins < 1) return fail(-1, "bad argument");
  OnDevice onDev(b->engine.device());
  int rc = b->engine.probeRootWaitTimeout(spins, flag);
  return rc ? fail(rc, "root wait probe failed") : 0;
}

int fgpu_set_device(int ordinal) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return fail(-960, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (ordinal < 0 || ordinal >= n)
    return fail(-961, "device ordinal " + std::to_string(ordinal) + " outside 0.." + std::to_string(n - 1));
  e = cudaSetDevice(ordinal);
  if (e != cudaSuccess) return fail(-962, std::string("cudaSetDevice failed: ") + cudaGetErrorString(e));
  g_device.store(ordinal);
  return 0;
}

int fgpu_get_device(int* ordinal, char* pciBusId, int len) {
  int dev = g_device.load();
  if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return fail(-960, "no CUDA device");
  if (ordinal) *ordinal = dev;
  if (pciBusId && len > 0) {
    cudaError_t e = cudaDeviceGetPCIBusId(pciBusId, len, dev);
    if (e != cudaSuccess) return fail(-963, std::string("cudaDeviceGetPCIBusId failed: ") + cudaGetErrorString(e));
  }
  return 0;
}

int fgpu_batch_device(const fgpu_batch* b) { return b ? b->engine.device() : fail(-1, "null batch"); }

const char* fgpu_last_error(void) { return g_lastError.c_str(); }

}  // extern "C"
