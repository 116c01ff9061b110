// server.cpp -- continuous batching of simulation requests (see server.h).
//
// The reference solver has no serving mode; per request the semantics are
// solverInit + solveNext until the end time (src/vpmSolver/solverInterface.h:65, :247).

#include "server.h"

#include <array>
#include <string>

namespace fgpu {

Server::Server(size_t budgetBytes, const EngineOptions& opt, int maxModelsPerBatch, int chunk, int device)
    : budget_(budgetBytes), device_(device), opt_(opt), maxModels_(maxModelsPerBatch > 0 ? maxModelsPerBatch : 1 << 30),
      chunk_(chunk > 0 ? chunk : 4), t0_(std::chrono::steady_clock::now()) {}

Server::~Server() {
  for (auto& st : starting_)
    if (st.rc.valid()) st.rc.wait();  // engines being built finish before the server goes
  for (auto& r : retiring_)
    if (r.valid()) r.wait();
}

// A finished engine is destroyed on a host thread of its own: freeing device
// memory waits for the device, and the pump must keep the other engines fed.
void Server::retire(std::unique_ptr<Engine> e) {
  for (size_t k = 0; k < retiring_.size();) {
    if (retiring_[k].wait_for(std::chrono::seconds(0)) == std::future_status::ready) {
      retiring_.erase(retiring_.begin() + (long)k);
    } else {
      ++k;
    }
  }
  const int dev = device_;
  retiring_.push_back(std::async(std::launch::async, [dev, e = std::move(e)]() mutable {
    cudaSetDevice(dev);
    e.reset();
  }));
}

double Server::now() const {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
}

// device footprint of one model in an engine (element SoA, vectors, CSR, fronts)
size_t Server::estimateBytes(const HostModel& m, const EngineOptions& opt) {
  size_t el = (size_t)m.nel * (144 * 8 * 4 + 36 * 8 + 12 * 8 * 7 + 48 * 8 + 24 * 8 + 9 * 8 + 64);
  size_t dof = (size_t)m.ndof * (8 * 8 + 12);
  size_t eq = (size_t)m.neq * (8 * 12 + 24);
  size_t csr = m.colInd.size() * (8 + 4 + 4 + 8) + m.slotSrc.size() * 8;
  size_t fr = (size_t)(m.lSize + m.uSize + m.wSize) * (opt.fp32Factor ? 4 : 8) + m.fronts.size() * 96 +
              m.asmSlot.size() * 12 + m.frontRows.size() * 4;
  return el + dof + eq + csr + fr + (1 << 16);
}

int Server::submit(const HostModel* m) {
  Request r;
  r.model = m;
  r.arrival = now();
  reqs_.push_back(r);
  pending_.push_back((int)reqs_.size() - 1);
  return (int)reqs_.size() - 1;
}

// Uploads the models `ms` (requests `ids`) into a new engine for job j,
// computes their initial state, and puts the carried state of the first
// carried->size() of them back (models moved from another engine, between
// steps).  Touches only j and its arguments (it may run on its own thread).
int Server::startEngine(Job& j, const std::vector<int>& ids, const std::vector<const HostModel*>& ms,
                        const std::vector<std::vector<char>>* carried) {
  j.engine = std::make_unique<Engine>();
  std::string err;
  int rc = j.engine->upload(ms, opt_, err);
  if (!rc) rc = j.engine->initialState(err);
  if (!rc && carried)
    for (size_t k = 0; k < carried->size() && !rc; ++k) rc = j.engine->injectModelState((int)k, (*carried)[k]);
  if (rc) return rc;
  j.ids = ids;
  j.bytes = j.engine->deviceBytes();
  j.parking = false;
  return 0;
}

int Server::admit() {
  if (pending_.empty()) return 0;
  if (maxEngines_ > 0 && liveEngines() >= maxEngines_) return 0;
  // one engine build at a time: requests arriving meanwhile join the next one
  if (!starting_.empty()) return 0;
  // batching window: wait for a few requests unless the device is idle
  bool idle = liveEngines() == 0;
  double waited = now() - reqs_[pending_.front()].arrival;
  if (!idle && (int)pending_.size() < minBatch_ && waited < maxWait_) return 0;
  std::vector<int> take;
  size_t bytes = 0;
  while (!pending_.empty() && (int)take.size() < maxModels_) {
    int id = pending_.front();
    size_t b = estimateBytes(*reqs_[id].model, opt_);
    if (inUse_ + bytes + b > budget_ && !(take.empty() && liveEngines() == 0)) break;
    take.push_back(id);
    bytes += b;
    pending_.pop_front();
  }
  if (take.empty()) return 0;
  // the engine is built on a host thread of its own; its requests count as
  // running and its estimated memory as in use until finishStarts takes it
  Starting st;
  st.job = std::make_unique<Job>();
  st.ids = take;
  st.reserved = bytes;
  const double t = now();
  std::vector<const HostModel*> ms;
  for (int id : take) {
    reqs_[id].state = 1;
    reqs_[id].admitted = t;
    ms.push_back(reqs_[id].model);
  }
  inUse_ += bytes;
  Job* jp = st.job.get();
  const int dev = device_, chunk = chunk_;
  const std::array<int, 4> shape = shape_;
  const bool haveShape = haveShape_;
  st.rc = std::async(std::launch::async, [this, jp, take, ms, dev, chunk, shape, haveShape]() {
    if (cudaSetDevice(dev) != cudaSuccess) return -953;
    int rc = startEngine(*jp, take, ms, nullptr);
    if (!rc && haveShape) jp->engine->setLaunchShape(shape.data());
    if (!rc && jp->engine->launchChunk(chunk)) rc = -950;
    return rc;
  });
  starting_.push_back(std::move(st));
  return 1;
}

// Takes the engines whose build finished into the running jobs (or fails
// their requests).  Returns the number of requests failed, < 0 never.
int Server::finishStarts() {
  int failed = 0;
  for (size_t k = 0; k < starting_.size();) {
    Starting& st = starting_[k];
    if (st.rc.wait_for(std::chrono::seconds(0)) != std::future_status::ready) {
      ++k;
      continue;
    }
    const int rc = st.rc.get();
    inUse_ -= st.reserved;
    if (rc) {
      const double t = now();
      for (int id : st.ids) { reqs_[id].state = 3; reqs_[id].finished = t; }
      failed += (int)st.ids.size();
    } else {
      inUse_ += st.job->bytes;
      if (!haveShape_) {
        // the first engine's tuned launch shapes serve every later engine
        // (no probe per engine; results do not depend on the shapes)
        double ms = 0.0;
        haveShape_ = st.job->engine->launchShape(shape_.data(), &ms) == 1;
      }
      jobs_.push_back(std::move(*st.job));
    }
    starting_.erase(starting_.begin() + (long)k);
  }
  return failed;
}

// Moves the running models of job k (all stopped between steps) into a new
// engine together with the waiting requests that fit the memory the old engine
// frees: the job is removed and the new engine built on its own host thread.
// Returns the number of requests admitted.
int Server::rebatch(size_t k) {
  Job& old = jobs_[k];
  std::vector<int> keep;
  std::vector<std::vector<char>> carried;
  for (size_t q = 0; q < old.ids.size(); ++q) {
    const int id = old.ids[q];
    if (reqs_[id].state != 1) continue;
    carried.emplace_back();
    if (old.engine->extractModelState((int)q, carried.back())) return -954;
    keep.push_back(id);
  }
  size_t bytes = 0;
  for (int id : keep) bytes += estimateBytes(*reqs_[id].model, opt_);
  std::vector<int> take = keep;
  int added = 0;
  while (!pending_.empty() && (int)take.size() < maxModels_) {
    const int id = pending_.front();
    const size_t b = estimateBytes(*reqs_[id].model, opt_);
    if (inUse_ - old.bytes + bytes + b > budget_) break;
    take.push_back(id);
    bytes += b;
    pending_.pop_front();
    ++added;
  }
  inUse_ -= old.bytes;
  std::unique_ptr<Engine> oldEngine = std::move(old.engine);
  jobs_.erase(jobs_.begin() + (long)k);
  // the new engine is built on a host thread of its own, as for an admission
  const double t = now();
  for (size_t q = keep.size(); q < take.size(); ++q) {
    reqs_[take[q]].state = 1;
    reqs_[take[q]].admitted = t;
  }
  Starting st;
  st.job = std::make_unique<Job>();
  st.ids = take;
  st.reserved = bytes;
  inUse_ += bytes;
  std::vector<const HostModel*> ms;
  for (int id : take) ms.push_back(reqs_[id].model);
  Job* jp = st.job.get();
  const int dev = device_, chunk = chunk_;
  const std::array<int, 4> shape = shape_;
  const bool haveShape = haveShape_;
  st.rc = std::async(std::launch::async, [this, jp, take, ms, dev, chunk, shape, haveShape,
                                           carried = std::move(carried), oldEngine = std::move(oldEngine)]() mutable {
    if (cudaSetDevice(dev) != cudaSuccess) return -953;
    oldEngine.reset();  // the device memory of the old engine goes first
    int rc = startEngine(*jp, take, ms, &carried);
    if (!rc && haveShape) jp->engine->setLaunchShape(shape.data());
    if (!rc && jp->engine->launchChunk(chunk)) rc = -950;
    return rc;
  });
  starting_.push_back(std::move(st));
  ++rebatches_;
  return added;
}

// Completes the requests of a job whose models reached their end time (or
// failed) by the last chunk: results and finish time per request, while the
// job's other models keep running.  all = true collects every request left.
int Server::collect(Job& j, bool all) {
  const int* states = j.engine->chunkStates();
  double t = now();
  int n = 0;
  for (size_t k = 0; k < j.ids.size(); ++k) {
    Request& r = reqs_[j.ids[k]];
    if (r.state != 1) continue;
    const int st = states ? states[k] : ST_ITER;
    if (!all && st != ST_DONE && st != ST_ERROR) continue;
    r.ur.resize(12 * (size_t)r.model->ntri);
    j.engine->getTriadUr((int)k, r.ur.data());
    r.iterations = j.engine->modelIterations((int)k);
    r.steps = j.engine->modelSteps((int)k);
    r.state = j.engine->modelState((int)k) == ST_DONE ? 2 : 3;
    r.finished = t;
    ++n;
  }
  return n;
}

int Server::pump() {
  if (cudaSetDevice(device_) != cudaSuccess) return -953;
  int finished = finishStarts();
  // collect finished requests and engines, keep the others fed
  for (size_t k = 0; k < jobs_.size();) {
    Job& j = jobs_[k];
    bool ready = false;
    int active = 1;
    if (j.engine->pollChunk(&ready, &active)) return -951;
    if (ready && active == 0 && j.parking) {
      // every running model stopped between steps: move them (and waiting requests)
      finished += collect(j, false);
      bool running = false;
      for (int id : j.ids) running |= reqs_[id].state == 1;
      if (running) {
        const int a = rebatch(k);  // removes job k
        if (a < 0) return a;
        continue;
      }
    }
    if (ready && active == 0) {
      finished += collect(j, true);
      inUse_ -= j.bytes;
      retire(std::move(j.engine));
      jobs_.erase(jobs_.begin() + (long)k);
      continue;
    }
    if (ready) {
      finished += collect(j, false);
      // slot reuse: enough of this engine's models finished and requests wait
      if (!j.parking && reuseShare_ > 0.0 && !pending_.empty()) {
        std::vector<int> running;
        for (size_t q = 0; q < j.ids.size(); ++q)
          if (reqs_[j.ids[q]].state == 1) running.push_back((int)q);
        const size_t done = j.ids.size() - running.size();
        if (!running.empty() && (double)done >= reuseShare_ * (double)j.ids.size()) {
          if (j.engine->parkModels(running)) return -955;
          j.parking = true;
        }
      }
      if (j.engine->launchChunk(chunk_)) return -952;
    }
    ++k;
  }
  // admit what fits (several admission rounds if memory allows)
  for (int r = 0; r < 4 && !pending_.empty(); ++r) {
    int a = admit();
    if (a < 0) return a;
    if (a == 0) break;
  }
  return finished;
}

}  // namespace fgpu
