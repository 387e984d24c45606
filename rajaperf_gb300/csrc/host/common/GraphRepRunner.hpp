// CUDA-graph rep runner.
//
// The suite's GPU variants launch every rep from the host
// (e.g. stream/TRIAD-Cuda.cpp:49-61), so at small sizes the time is launch
// overhead.  GraphRepRunner captures a rep body (any sequence of libb200
// calls on the given stream) `reps` times into one CUDA graph, instantiates
// it once, and replays it.  Capture happens outside the timed region; replay
// happens inside it.  Long rep loops are captured in chunks of at most
// `max_reps_per_graph` reps and the chunk graph is replayed.
#pragma once

#include "b200.h"

#include <cstdint>
#include <functional>
#include <vector>

namespace rajaperf {

class GraphRepRunner {
 public:
  using RepBody = std::function<void(b200_stream_t)>;

  explicit GraphRepRunner(int64_t max_reps_per_graph = 1024);
  ~GraphRepRunner();
  GraphRepRunner(const GraphRepRunner&) = delete;
  GraphRepRunner& operator=(const GraphRepRunner&) = delete;

  // Captures reps x body.  Throws std::runtime_error on a CUDA error or when
  // the body fails during capture.
  void capture(int64_t reps, const RepBody& body);
  // Replays the captured rep loop once (asynchronously on the runner's
  // stream); call synchronize() or a device sync to wait.
  void launch();
  void synchronize();

  int64_t capturedReps() const { return reps_; }
  b200_stream_t stream() const { return stream_; }

 private:
  void reset();

  int64_t max_chunk_;
  int64_t reps_ = 0;
  int64_t chunk_ = 0;
  int64_t chunk_launches_ = 0;
  b200_stream_t stream_ = nullptr;
  void* chunk_graph_ = nullptr;     // cudaGraphExec_t of `chunk_` reps
  void* tail_graph_ = nullptr;      // cudaGraphExec_t of the remainder
};

// One CUDA graph over several independent rep bodies: capture forks from a
// capture stream into one stream per body, records that body's `reps` reps
// there (so they stay in order) and joins every branch back.  The bodies must
// share no device data; the branches then run concurrently on the GPU.
class ParallelGraph {
 public:
  ParallelGraph(const std::vector<GraphRepRunner::RepBody>& bodies, int64_t reps);
  ~ParallelGraph();
  ParallelGraph(const ParallelGraph&) = delete;
  ParallelGraph& operator=(const ParallelGraph&) = delete;

  void launch();
  void synchronize();

 private:
  void* stream_ = nullptr;  // cudaStream_t the graph is launched on
  void* exec_ = nullptr;    // cudaGraphExec_t
};

}  // namespace rajaperf
