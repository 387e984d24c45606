#include "GraphRepRunner.hpp"

#include "DataUtils.hpp"

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

namespace rajaperf {

namespace {

cudaGraphExec_t captureReps(cudaStream_t s, int64_t reps,
                            const GraphRepRunner::RepBody& body) {
  checkCuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
            "cudaStreamBeginCapture");
  try {
    for (int64_t r = 0; r < reps; ++r) body(reinterpret_cast<b200_stream_t>(s));
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(s, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  cudaGraph_t graph = nullptr;
  checkCuda(cudaStreamEndCapture(s, &graph), "cudaStreamEndCapture");
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  checkCuda(e, "cudaGraphInstantiate");
  return exec;
}

}  // namespace

GraphRepRunner::GraphRepRunner(int64_t max_reps_per_graph)
    : max_chunk_(max_reps_per_graph > 0 ? max_reps_per_graph : 1) {
  cudaStream_t s = nullptr;
  checkCuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking),
            "cudaStreamCreate");
  stream_ = reinterpret_cast<b200_stream_t>(s);
}

GraphRepRunner::~GraphRepRunner() {
  reset();
  if (stream_) cudaStreamDestroy(reinterpret_cast<cudaStream_t>(stream_));
}

void GraphRepRunner::reset() {
  if (chunk_graph_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(chunk_graph_));
  if (tail_graph_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(tail_graph_));
  chunk_graph_ = tail_graph_ = nullptr;
  reps_ = chunk_ = chunk_launches_ = 0;
}

void GraphRepRunner::capture(int64_t reps, const RepBody& body) {
  reset();
  if (reps <= 0) return;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream_);
  chunk_ = reps < max_chunk_ ? reps : max_chunk_;
  chunk_launches_ = reps / chunk_;
  int64_t tail = reps - chunk_launches_ * chunk_;
  chunk_graph_ = captureReps(s, chunk_, body);
  if (tail > 0) tail_graph_ = captureReps(s, tail, body);
  reps_ = reps;
}

void GraphRepRunner::launch() {
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream_);
  for (int64_t i = 0; i < chunk_launches_; ++i) {
    checkCuda(cudaGraphLaunch(static_cast<cudaGraphExec_t>(chunk_graph_), s),
              "cudaGraphLaunch");
  }
  if (tail_graph_) {
    checkCuda(cudaGraphLaunch(static_cast<cudaGraphExec_t>(tail_graph_), s),
              "cudaGraphLaunch");
  }
}

void GraphRepRunner::synchronize() {
  checkCuda(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream_)),
            "cudaStreamSynchronize");
}

}  // namespace rajaperf
