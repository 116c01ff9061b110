// server.h -- continuous batching of simulation requests on one GPU.
//
// Requests (one model each) are admitted as soon as device memory allows:
// every admission round takes the pending requests that fit the remaining
// HBM budget into a new engine with its own stream, so work of requests that
// arrive while others run overlaps on the device.  Each request keeps its
// state resident until it reaches its end time, when it is completed (results
// and finish time) at the next chunk boundary although the other models of
// its engine go on.  Slots of finished requests are reused: when an engine
// has finished a set share of its models and requests are waiting, its
// running models stop at the end of their current step, their state moves
// into a new engine together with the waiting requests that fit, and they
// continue there exactly as they would have (the old engine's memory, finished
// slots included, is released).  Finished engines release their memory.
// A new engine is built (upload, initial state, first chunk), and a finished
// one destroyed, on a host thread of its own, so the engines already running
// stay fed meanwhile.
#pragma once

#include <array>
#include <chrono>
#include <deque>
#include <future>
#include <memory>
#include <vector>

#include "engine.h"

namespace fgpu {

struct Request {
  const HostModel* model = nullptr;
  double arrival = 0.0, admitted = -1.0, finished = -1.0;
  long long iterations = 0, steps = 0;
  int state = 0;  // 0 pending, 1 running, 2 done, 3 failed
  std::vector<double> ur;  // final triad positions
};

class Server {
 public:
  // device: the CUDA device every engine of this server runs on
  Server(size_t budgetBytes, const EngineOptions& opt, int maxModelsPerBatch, int chunk, int device);
  int submit(const HostModel* m);  // returns the request id (arrival stamped now)
  // One pass: admit pending requests that fit, keep every live engine fed with
  // a chunk of batched iterations, collect finished engines.  Returns the
  // number of requests finished in this pass (< 0 on error).
  int pump();
  double now() const;
  const Request& request(int id) const { return reqs_[id]; }
  int numRequests() const { return (int)reqs_.size(); }
  int pending() const { return (int)pending_.size(); }
  int liveEngines() const { return (int)(jobs_.size() + starting_.size()); }
  size_t bytesInUse() const { return inUse_; }

 private:
  struct Job {
    std::unique_ptr<Engine> engine;
    std::vector<int> ids;
    size_t bytes = 0;
    bool parking = false;  // running models stop at their next step end for a move
  };
  // an engine being built on its own host thread for admitted requests
  struct Starting {
    std::unique_ptr<Job> job;
    std::vector<int> ids;
    size_t reserved = 0;  // estimated bytes held in inUse_ until it is built
    std::future<int> rc;
  };
  static size_t estimateBytes(const HostModel& m, const EngineOptions& opt);
  int admit();
  int collect(Job& j, bool all);
  int startEngine(Job& j, const std::vector<int>& ids, const std::vector<const HostModel*>& ms,
                  const std::vector<std::vector<char>>* carried);
  int finishStarts();
  void retire(std::unique_ptr<Engine> e);
  std::array<int, 4> shape_{};  // launch shapes tuned by the first engine, for the later ones
  bool haveShape_ = false;
  std::vector<std::future<void>> retiring_;
  int rebatch(size_t k);

  size_t budget_, inUse_ = 0;
  int device_ = 0;
  EngineOptions opt_;
  int maxModels_, chunk_;
  int minBatch_ = 8;        // admission waits for this many requests ...
  double maxWait_ = 0.02;   // ... or this long (s), unless the device is idle

 public:
  void setBatchingWindow(int minBatch, double maxWaitSec) {
    minBatch_ = minBatch > 0 ? minBatch : 1;
    maxWait_ = maxWaitSec;
  }
  // Share of an engine's models that must have finished before its slots are
  // reused for waiting requests (0: never; engines then end as a whole).
  void setSlotReuse(double share) { reuseShare_ = share; }
  // At most this many engines at a time (0: as many as memory allows).
  void setMaxEngines(int n) { maxEngines_ = n > 0 ? n : 0; }
  int maxEngines_ = 0;
  long long rebatches() const { return rebatches_; }
  double reuseShare_ = 0.25;
  long long rebatches_ = 0;
  std::vector<Request> reqs_;
  std::deque<int> pending_;
  std::vector<Job> jobs_;
  std::vector<Starting> starting_;
  std::chrono::steady_clock::time_point t0_;

 public:
  ~Server();
};

}  // namespace fgpu
