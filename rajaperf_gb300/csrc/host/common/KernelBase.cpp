#include "KernelBase.hpp"

#include "GraphRepRunner.hpp"
#include "TuningTable.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace rajaperf {

KernelBase::KernelBase(KernelID kid, const RunParams& params)
    : run_params(params), checksum_scale_factor(1.0), kernel_id(kid),
      name(getFullKernelName(kid)) {}

KernelBase::~KernelBase() = default;

// Same rule as the suite's KernelBase.cpp:115-125, plus the per-kernel size
// map (a --size-map entry overrides --size/--sizefact for that kernel).
Index_type KernelBase::getTargetProblemSize() const {
  double per_kernel = run_params.getKernelSize(kernel_id);
  if (per_kernel >= 0.0) return static_cast<Index_type>(per_kernel);
  if (run_params.getSizeMeaning() == RunParams::Direct)
    return static_cast<Index_type>(run_params.getSize());
  return static_cast<Index_type>(default_prob_size * run_params.getSizeFactor());
}

// KernelBase.cpp:127-136.
Index_type KernelBase::getRunReps() const {
  if (run_params.getInputState() == RunParams::CheckRun)
    return static_cast<Index_type>(run_params.getCheckRunReps());
  return static_cast<Index_type>(default_reps * run_params.getRepFactor());
}

void KernelBase::setVariantDefined(VariantID vid) {
  if (!isVariantAvailable(vid)) return;
  setGB300TuningDefinitions(vid);
  size_t nt = getNumVariantTunings(vid);
  checksum[vid].assign(nt, 0.0L);
  num_exec[vid].assign(nt, 0);
  min_time[vid].assign(nt, std::numeric_limits<double>::max());
  max_time[vid].assign(nt, -std::numeric_limits<double>::max());
  tot_time[vid].assign(nt, 0.0);
}

void KernelBase::setGB300TuningDefinitions(VariantID vid) {
  addVariantTuningName(vid, getDefaultTuningName());
  addVariantTuningName(vid, "graph");
  for (const NamedTune& nt : named_tunes) addVariantTuningName(vid, nt.name);
}

void KernelBase::addTuning(const std::string& tname, const b200_tune& t,
                           bool graph) {
  named_tunes.push_back(NamedTune{tname, t, graph});
}

size_t KernelBase::getVariantTuningIndex(VariantID vid,
                                         const std::string& tname) const {
  const auto& names = getVariantTuningNames(vid);
  for (size_t t = 0; t < names.size(); ++t)
    if (names[t] == tname) return t;
  return getUnknownTuningIdx();
}

b200_tune KernelBase::getTune(size_t tune_idx) const {
  b200_tune t{};
  const std::string& tname = getVariantTuningName(Base_GB300, tune_idx);
  bool named = false;
  for (const NamedTune& nt : named_tunes) {
    if (nt.name == tname) {
      t = nt.tune;
      named = true;
      break;
    }
  }
  if (!named) TuningTable::instance().lookup(name, actual_prob_size, &t);
  if (run_params.getWaitLimitUs() > 0) t.wait_limit_us = run_params.getWaitLimitUs();
  return t;
}

void KernelBase::checkWorkspace(void* ws, size_t bytes, const char* what) const {
  if (!ws) return;
  const int st = b200_workspace_status(ws, bytes, getStream());
  if (st != B200_OK)
    throw std::runtime_error(std::string(what) + ": " +
                             (st == B200_ERR_TIMEOUT ? "device-side wait timed out: " : "") +
                             b200_last_error_string());
}

void KernelBase::injectLookbackStall(void* ws, size_t bytes, const b200_tune& tn,
                                     bool pointers_aligned) const {
  const long k = run_params.getInjectLookbackStall();
  if (k <= 0 || !ws) return;
  // Only the persistent ring kernel bounds its tile ids by the tile count,
  // so only it may start with tickets already taken.
  if (tn.algo != 0 || tn.vec == 1 || !pointers_aligned || bytes < 256)
    throw std::runtime_error("--inject-lookback-stall needs the pipelined (algo 0) kernel");
  // ticket word: low 32 bits = tickets taken, high 32 bits = launch epoch
  unsigned long long word = 0;
  checkCuda(cudaMemcpy(&word, ws, sizeof(word), cudaMemcpyDeviceToHost), "stall: read");
  word += static_cast<unsigned long long>(k);
  checkCuda(cudaMemcpy(ws, &word, sizeof(word), cudaMemcpyHostToDevice), "stall: write");
}

bool KernelBase::isGraphTuning(size_t tune_idx) const {
  const std::string& tname = getVariantTuningName(Base_GB300, tune_idx);
  if (tname == "graph") return true;
  for (const NamedTune& nt : named_tunes)
    if (nt.name == tname) return nt.graph;
  return false;
}

void KernelBase::synchronize() {
  checkCuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
}

void KernelBase::startTimer() {
  synchronize();
  timer_start = std::chrono::steady_clock::now();
}

void KernelBase::stopTimer() {
  synchronize();
  auto t1 = std::chrono::steady_clock::now();
  timer_elapsed += std::chrono::duration<double>(t1 - timer_start).count();
  recordExecTime();
}

void KernelBase::recordExecTime() {
  num_exec[running_variant].at(running_tuning)++;
  double t = timer_elapsed;
  min_time[running_variant].at(running_tuning) =
      std::min(min_time[running_variant].at(running_tuning), t);
  max_time[running_variant].at(running_tuning) =
      std::max(max_time[running_variant].at(running_tuning), t);
  tot_time[running_variant].at(running_tuning) += t;
}

void KernelBase::execute(VariantID vid, size_t tune_idx) {
  running_variant = vid;
  running_tuning = tune_idx;
  resetTimer();
  resetHostIO();
  detail::resetDataInitCount();
  try {
    setUp(vid, tune_idx);
    runKernel(vid, tune_idx);
    updateChecksum(vid, tune_idx);
  } catch (...) {
    try { tearDown(vid, tune_idx); } catch (...) {}
    running_variant = NumVariants;
    running_tuning = getUnknownTuningIdx();
    throw;
  }
  tearDown(vid, tune_idx);
  running_variant = NumVariants;
  running_tuning = getUnknownTuningIdx();
}

void KernelBase::runKernel(VariantID vid, size_t tune_idx) {
  if (!hasVariantDefined(vid)) return;
  runGB300Variant(vid, tune_idx);
}

void KernelBase::runGB300Variant(VariantID, size_t tune_idx) {
  prepareRun(tune_idx);
  if (hostData() && !host_io_declared_)
    throw std::runtime_error(name + " has no --host-data form");
  if (hostData() && !staged_.empty()) {
    swapStaged(true);
    try {
      runReps(tune_idx, getRunReps(), stagedBody(makeRepBody(tune_idx)));
    } catch (...) {
      swapStaged(false);
      throw;
    }
    swapStaged(false);
  } else {
    runReps(tune_idx, getRunReps(), makeRepBody(tune_idx));
  }
  finishRun(tune_idx);
}

bool KernelBase::hostData() const { return run_params.getHostData(); }

void KernelBase::resetHostIO() {
  for (Staged& st : staged_) {
    if (*st.member == st.dev) *st.member = st.host;
    deallocDeviceBytes(st.dev);
  }
  staged_.clear();
  host_io_declared_ = false;
  h2d_bytes_per_rep = 0;
  d2h_bytes_per_rep = 0;
}

void KernelBase::stageBytes(void** member, Size_type bytes, unsigned io) {
  if (!hostData()) return;
  Staged st{member, *member, allocDeviceBytes(bytes), bytes, io};
  staged_.push_back(st);
  hostArrayBytes(bytes, io);
}

void KernelBase::hostArrayBytes(Size_type bytes, unsigned io) {
  if (!hostData()) return;
  host_io_declared_ = true;
  if (io & kIn) h2d_bytes_per_rep += bytes;
  if (io & kOut) d2h_bytes_per_rep += bytes;
}

void KernelBase::unstage(void** member) {
  for (size_t k = 0; k < staged_.size(); ++k) {
    if (staged_[k].member != member) continue;
    if (*member == staged_[k].dev) *member = staged_[k].host;
    deallocDeviceBytes(staged_[k].dev);
    staged_.erase(staged_.begin() + static_cast<std::ptrdiff_t>(k));
    return;
  }
}

// During the timed loop the staged members point to their device buffers,
// which start as copies of the host arrays (untimed): the parts of an array
// that no rep writes (boundaries of a stencil's output, a zone list's
// ghosts) then hold the host values, and scratch arrays start initialised.
void KernelBase::swapStaged(bool to_device) {
  for (Staged& st : staged_) {
    if (to_device) copyToDevice(st.dev, st.host, st.bytes);
    *st.member = to_device ? st.dev : st.host;
  }
}

// One rep with host-resident data: the kIn arrays are copied in from pinned
// host memory, the kernel runs on the device buffers, the kOut arrays are
// copied back, all on the rep's stream (so a graph tuning captures the
// copies with the kernels).
KernelBase::RepBody KernelBase::stagedBody(RepBody inner) {
  const std::vector<Staged> st = staged_;
  return [st, inner](b200_stream_t s) {
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(s);
    for (const Staged& a : st)
      if (a.io & kIn)
        checkCuda(cudaMemcpyAsync(a.dev, a.host, a.bytes, cudaMemcpyHostToDevice, cs),
                  "host-data copy in");
    inner(s);
    for (const Staged& a : st)
      if (a.io & kOut)
        checkCuda(cudaMemcpyAsync(a.host, a.dev, a.bytes, cudaMemcpyDeviceToHost, cs),
                  "host-data copy out");
  };
}

void KernelBase::runReps(size_t tune_idx, Index_type reps,
                         const std::function<void(b200_stream_t)>& rep_body) {
  if (!isGraphTuning(tune_idx)) {
    startTimer();
    for (RepIndex_type irep = 0; irep < reps; ++irep) rep_body(getStream());
    stopTimer();
    return;
  }
  GraphRepRunner runner;
  runner.capture(reps, rep_body);
  startTimer();
  runner.launch();
  stopTimer();
}

void KernelBase::allocAndInitData(Real_ptr& ptr, Size_type len, VariantID vid) {
  allocData(ptr, len, vid);
  initDeviceData(run_params, ptr, len);
}

void KernelBase::allocAndInitDataConst(Real_ptr& ptr, Size_type len,
                                       Real_type val, VariantID vid) {
  allocData(ptr, len, vid);
  initDeviceDataConst(ptr, len, val);
}

void KernelBase::allocAndInitDataConst(Index_type*& ptr, Size_type len,
                                       Index_type val, VariantID vid) {
  allocData(ptr, len, vid);
  initDeviceDataConst(ptr, len, val);
}

void KernelBase::allocAndInitDataRandSign(Real_ptr& ptr, Size_type len,
                                          VariantID vid) {
  allocData(ptr, len, vid);
  initDeviceDataRandSign(run_params, ptr, len);
}

void KernelBase::allocAndInitDataRandValue(Real_ptr& ptr, Size_type len,
                                           VariantID vid) {
  allocData(ptr, len, vid);
  initDeviceDataRandValue(run_params, ptr, len);
}

}  // namespace rajaperf
