// server.h -- continuous batching of simulation requests on one GPU.
//
// Requests (one model each) are admitted as soon as device memory allows:
// every admission round takes the pending requests that fit the remaining
// HBM budget into a new engine with its own stream, so work of requests that
// arrive while others run overlaps on the device.  Each request keeps its
// state resident until it reaches its end time, when it is completed (results
// and finish time) at the next chunk boundary although the other models of
// its engine go on; finished engines release their memory for the next
// admissions.
#pragma once

#include <chrono>
#include <deque>
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
  int liveEngines() const { return (int)jobs_.size(); }
  size_t bytesInUse() const { return inUse_; }

 private:
  struct Job {
    std::unique_ptr<Engine> engine;
    std::vector<int> ids;
    size_t bytes = 0;
  };
  static size_t estimateBytes(const HostModel& m, const EngineOptions& opt);
  int admit();
  int collect(Job& j, bool all);

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
  std::vector<Request> reqs_;
  std::deque<int> pending_;
  std::vector<Job> jobs_;
  std::chrono::steady_clock::time_point t0_;
};

}  // namespace fgpu
