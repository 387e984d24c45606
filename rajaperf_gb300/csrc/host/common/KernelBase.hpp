// Base class of every Base_GB300 kernel.
//
// Same plugin contract as the suite's common/KernelBase.hpp:70-604: a kernel
// subclass sets its sizes, reps, bytes and FLOPs in its constructor, then the
// executor calls execute(vid, tune) = setUp -> runKernel -> updateChecksum ->
// tearDown (KernelBase.cpp:359-377).  Timing brackets the rep loop with a
// device synchronisation on both sides (KernelBase.hpp:484-501).
//
// GB300 specifics:
//  - data helpers allocate and fill DEVICE memory (DataUtils.hpp);
//  - runGB300Variant() replaces run<Backend>Variant();
//  - every kernel has the tunings "default" (one library call per rep) and
//    "graph" (the rep loop captured once into a CUDA graph, then replayed
//    between startTimer/stopTimer), plus kernel-specific launch shapes;
//  - launch shapes for "default"/"graph" come from the tuning table when one
//    is loaded, else from the library defaults.
#pragma once

#include "DataUtils.hpp"
#include "RAJAPerfSuite.hpp"
#include "RPTypes.hpp"
#include "RunParams.hpp"

#include "b200.h"

#include <chrono>
#include <functional>
#include <limits>
#include <string>
#include <vector>

namespace rajaperf {

class KernelBase {
 public:
  static constexpr size_t getUnknownTuningIdx() {
    return std::numeric_limits<size_t>::max();
  }
  static std::string getDefaultTuningName() { return "default"; }

  KernelBase(KernelID kid, const RunParams& params);
  virtual ~KernelBase();

  KernelID getKernelID() const { return kernel_id; }
  const std::string& getName() const { return name; }

  // ---- properties set by subclass constructors ----
  void setDefaultProblemSize(Index_type size) { default_prob_size = size; }
  void setActualProblemSize(Index_type size) { actual_prob_size = size; }
  void setDefaultReps(Index_type reps) { default_reps = reps; }
  void setItsPerRep(Index_type its) { its_per_rep = its; }
  void setKernelsPerRep(Index_type nk) { kernels_per_rep = nk; }
  void setBytesReadPerRep(Index_type b) { bytes_read_per_rep = b; }
  void setBytesWrittenPerRep(Index_type b) { bytes_written_per_rep = b; }
  void setBytesAtomicModifyWrittenPerRep(Index_type b) { bytes_atomic_per_rep = b; }
  void setFLOPsPerRep(Index_type f) { flops_per_rep = f; }
  void setComplexity(Complexity ac) { complexity = ac; }
  void setUsesFeature(FeatureID fid) { uses_feature[fid] = true; }

  void setVariantDefined(VariantID vid);
  void addVariantTuningName(VariantID vid, std::string tname) {
    variant_tuning_names[vid].emplace_back(std::move(tname));
  }
  // Tunings of the Base_GB300 variant; subclasses add launch shapes.
  virtual void setGB300TuningDefinitions(VariantID vid);

  // ---- getters used by reports ----
  Index_type getDefaultProblemSize() const { return default_prob_size; }
  Index_type getActualProblemSize() const { return actual_prob_size; }
  Index_type getDefaultReps() const { return default_reps; }
  Index_type getItsPerRep() const { return its_per_rep; }
  Index_type getKernelsPerRep() const { return kernels_per_rep; }
  Index_type getBytesPerRep() const {
    return bytes_read_per_rep + bytes_written_per_rep + 2 * bytes_atomic_per_rep;
  }
  Index_type getBytesReadPerRep() const { return bytes_read_per_rep; }
  Index_type getBytesWrittenPerRep() const { return bytes_written_per_rep; }
  Index_type getBytesAtomicModifyWrittenPerRep() const { return bytes_atomic_per_rep; }
  Index_type getFLOPsPerRep() const { return flops_per_rep; }
  Complexity getComplexity() const { return complexity; }
  bool usesFeature(FeatureID fid) const { return uses_feature[fid]; }

  Index_type getTargetProblemSize() const;
  Index_type getRunReps() const;

  bool hasVariantDefined(VariantID vid) const {
    return !variant_tuning_names[vid].empty();
  }
  size_t getNumVariantTunings(VariantID vid) const {
    return variant_tuning_names[vid].size();
  }
  const std::string& getVariantTuningName(VariantID vid, size_t t) const {
    return variant_tuning_names[vid].at(t);
  }
  const std::vector<std::string>& getVariantTuningNames(VariantID vid) const {
    return variant_tuning_names[vid];
  }
  size_t getVariantTuningIndex(VariantID vid, const std::string& tname) const;

  bool wasVariantTuningRun(VariantID vid, size_t t) const {
    return t != getUnknownTuningIdx() && num_exec[vid].at(t) > 0;
  }
  double getLastTime() const { return timer_elapsed; }
  double getMinTime(VariantID vid, size_t t) const { return min_time[vid].at(t); }
  double getMaxTime(VariantID vid, size_t t) const { return max_time[vid].at(t); }
  double getTotTime(VariantID vid, size_t t) const { return tot_time[vid].at(t); }
  int getNumExec(VariantID vid, size_t t) const { return num_exec[vid].at(t); }
  Checksum_type getChecksum(VariantID vid, size_t t) const {
    return checksum[vid].at(t);
  }

  // setUp -> runKernel -> updateChecksum -> tearDown.
  void execute(VariantID vid, size_t tune_idx);

  void startTimer();
  void stopTimer();
  void resetTimer() { timer_elapsed = 0.0; }
  void synchronize();

  // ---- data helpers: device memory, or pinned host memory with --host-data ----
  template <typename T>
  void allocData(T*& ptr, Size_type len, VariantID) {
    ptr = static_cast<T*>(hostData() ? allocPinnedBytes(len * sizeof(T))
                                     : allocDeviceBytes(len * sizeof(T)));
  }
  template <typename T>
  void deallocData(T*& ptr, VariantID) {
    unstage(reinterpret_cast<void**>(&ptr));
    deallocDataBytes(ptr);
    ptr = nullptr;
  }

  // ---- host-resident data (--host-data) ----
  // The arrays allocated above live in pinned host memory, and each rep moves
  // its data across the host link inside the timed loop.  A kernel that
  // streams through its arrays once reads and writes them in host memory
  // directly and declares them with hostArray() (for the byte counts only).
  // One that iterates over them, or gathers, declares them with stageArray():
  // during the timed loop the member then points to a device buffer, and each
  // rep first copies the kIn arrays in from host memory and, after the
  // kernel, copies the kOut arrays back (arrays with neither are device-only
  // scratch the rep rewrites).  The device buffers start as copies of the
  // host arrays, taken before the timed loop.  A kernel that declares no array has no
  // host-data form, and its run fails with --host-data.
  enum : unsigned { kIn = 1u, kOut = 2u };
  bool hostData() const;
  template <typename T>
  void stageArray(T*& member, Size_type len, unsigned io) {
    stageBytes(reinterpret_cast<void**>(&member), len * sizeof(T), io);
  }
  template <typename T>
  void hostArray(const T* ptr, Size_type len, unsigned io) {
    (void)ptr;
    hostArrayBytes(len * sizeof(T), io);
  }
  // Bytes crossing the host link per rep in each direction (--host-data).
  Index_type getH2DBytesPerRep() const { return h2d_bytes_per_rep; }
  Index_type getD2HBytesPerRep() const { return d2h_bytes_per_rep; }
  void allocAndInitData(Real_ptr& ptr, Size_type len, VariantID vid);
  void allocAndInitDataConst(Real_ptr& ptr, Size_type len, Real_type val,
                             VariantID vid);
  void allocAndInitDataConst(Index_type*& ptr, Size_type len, Index_type val,
                             VariantID vid);
  void allocAndInitDataRandSign(Real_ptr& ptr, Size_type len, VariantID vid);
  void allocAndInitDataRandValue(Real_ptr& ptr, Size_type len, VariantID vid);
  void initData(Real_type& d, VariantID) { detail::initData(d); }

  long double calcChecksum(const Real_type* ptr, Size_type len, VariantID) {
    return calcChecksumDevice(ptr, len, 1.0);
  }
  long double calcChecksum(const Real_type* ptr, Size_type len,
                           Real_type scale_factor, VariantID) {
    return calcChecksumDevice(ptr, len, scale_factor);
  }

  // ---- GB300 execution helpers ----
  b200_stream_t getStream() const { return nullptr; }
  // Launch shape for a tuning (table entry for this kernel and size, the
  // tuning's own shape, or zeros = library default).
  b200_tune getTune(size_t tune_idx) const;
  // Throws when a bounded device-side wait of a call on this workspace gave
  // up since its last check (b200_workspace_status; clears the workspace).
  void checkWorkspace(void* ws, size_t bytes, const char* what) const;
  // --inject-lookback-stall: marks tickets of a lookback workspace as taken
  // before a run (untimed), so that a lookback wait runs out.
  void injectLookbackStall(void* ws, size_t bytes, const b200_tune& tn,
                           bool pointers_aligned) const;
  bool isGraphTuning(size_t tune_idx) const;
  // Runs `reps` repetitions of `rep_body` between startTimer and stopTimer,
  // either as direct calls or, for a graph tuning, as one captured graph.
  void runReps(size_t tune_idx, Index_type reps,
               const std::function<void(b200_stream_t)>& rep_body);

  // ---- per-kernel hooks ----
  using RepBody = std::function<void(b200_stream_t)>;

  virtual void runKernel(VariantID vid, size_t tune_idx);
  virtual void setUp(VariantID vid, size_t tune_idx) = 0;
  virtual void updateChecksum(VariantID vid, size_t tune_idx) = 0;
  virtual void tearDown(VariantID vid, size_t tune_idx) = 0;

  // Base_GB300 rep loop: prepareRun (untimed; e.g. the Polybench copies of
  // the initial state, POLYBENCH_JACOBI_2D.hpp:30-36), then the timed rep
  // loop of makeRepBody(), then finishRun (untimed; e.g. reading a device
  // reduction result back).
  virtual void runGB300Variant(VariantID vid, size_t tune_idx);
  virtual void prepareRun(size_t /*tune_idx*/) {}
  virtual RepBody makeRepBody(size_t tune_idx) = 0;
  virtual void finishRun(size_t /*tune_idx*/) {}

  // Extra tuning names of this kernel mapped to launch shapes.
  struct NamedTune {
    std::string name;
    b200_tune tune;
    bool graph;
  };
  void addTuning(const std::string& tname, const b200_tune& t, bool graph = false);

 protected:
  const RunParams& run_params;
  std::vector<Checksum_type> checksum[NumVariants];
  Checksum_type checksum_scale_factor;

 private:
  void recordExecTime();

  void stageBytes(void** member, Size_type bytes, unsigned io);
  void hostArrayBytes(Size_type bytes, unsigned io);
  void unstage(void** member);
  void resetHostIO();
  RepBody stagedBody(RepBody inner);
  void swapStaged(bool to_device);

  struct Staged {
    void** member;   // the kernel's pointer member
    void* host;      // its pinned host array
    void* dev;       // the device buffer it points to during the timed loop
    Size_type bytes;
    unsigned io;
  };
  std::vector<Staged> staged_;
  bool host_io_declared_ = false;
  Index_type h2d_bytes_per_rep = 0, d2h_bytes_per_rep = 0;

  KernelID kernel_id;
  std::string name;

  Index_type default_prob_size = -1;
  Index_type default_reps = -1;
  Index_type actual_prob_size = -1;
  Index_type its_per_rep = -1;
  Index_type kernels_per_rep = -1;
  Index_type bytes_read_per_rep = -1;
  Index_type bytes_written_per_rep = -1;
  Index_type bytes_atomic_per_rep = -1;
  Index_type flops_per_rep = -1;
  Complexity complexity = Complexity::NumComplexities;
  bool uses_feature[NumFeatures] = {};

  std::vector<std::string> variant_tuning_names[NumVariants];
  std::vector<NamedTune> named_tunes;

  VariantID running_variant = NumVariants;
  size_t running_tuning = getUnknownTuningIdx();

  std::chrono::steady_clock::time_point timer_start;
  double timer_elapsed = 0.0;

  std::vector<int> num_exec[NumVariants];
  std::vector<double> min_time[NumVariants];
  std::vector<double> max_time[NumVariants];
  std::vector<double> tot_time[NumVariants];
};

}  // namespace rajaperf
