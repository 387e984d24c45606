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

ParallelGraph::ParallelGraph(const std::vector<GraphRepRunner::RepBody>& bodies,
                             int64_t reps) {
  cudaStream_t main = nullptr;
  checkCuda(cudaStreamCreateWithFlags(&main, cudaStreamNonBlocking), "cudaStreamCreate");
  stream_ = main;
  std::vector<cudaStream_t> branch(bodies.size(), nullptr);
  std::vector<cudaEvent_t> done(bodies.size(), nullptr);
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  auto cleanup = [&]() {
    for (cudaStream_t b : branch)
      if (b) cudaStreamDestroy(b);
    for (cudaEvent_t e : done)
      if (e) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (graph) cudaGraphDestroy(graph);
  };
  try {
    checkCuda(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate");
    for (size_t i = 0; i < bodies.size(); ++i) {
      checkCuda(cudaStreamCreateWithFlags(&branch[i], cudaStreamNonBlocking),
                "cudaStreamCreate");
      checkCuda(cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    checkCuda(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal),
              "cudaStreamBeginCapture");
    try {
      checkCuda(cudaEventRecord(fork, main), "cudaEventRecord");
      for (size_t i = 0; i < bodies.size(); ++i) {
        checkCuda(cudaStreamWaitEvent(branch[i], fork, 0), "cudaStreamWaitEvent");
        for (int64_t r = 0; r < reps; ++r) bodies[i](reinterpret_cast<b200_stream_t>(branch[i]));
        checkCuda(cudaEventRecord(done[i], branch[i]), "cudaEventRecord");
        checkCuda(cudaStreamWaitEvent(main, done[i], 0), "cudaStreamWaitEvent");
      }
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(main, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    checkCuda(cudaStreamEndCapture(main, &graph), "cudaStreamEndCapture");
    cudaGraphExec_t exec = nullptr;
    checkCuda(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
    exec_ = exec;
  } catch (...) {
    cleanup();
    cudaStreamDestroy(main);
    stream_ = nullptr;
    throw;
  }
  cleanup();
}

ParallelGraph::~ParallelGraph() {
  if (exec_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(exec_));
  if (stream_) cudaStreamDestroy(static_cast<cudaStream_t>(stream_));
}

void ParallelGraph::launch() {
  checkCuda(cudaGraphLaunch(static_cast<cudaGraphExec_t>(exec_),
                            static_cast<cudaStream_t>(stream_)),
            "cudaGraphLaunch");
}

void ParallelGraph::synchronize() {
  checkCuda(cudaStreamSynchronize(static_cast<cudaStream_t>(stream_)), "cudaStreamSynchronize");
}

}  // namespace rajaperf
