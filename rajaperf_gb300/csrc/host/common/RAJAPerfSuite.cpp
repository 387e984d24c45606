// Name tables and lookups for the identifiers in RAJAPerfSuite.hpp.
#include "RAJAPerfSuite.hpp"

#include <array>
#include <iostream>

namespace rajaperf {

namespace {

const std::array<std::string, NumGroups>& groupNames() {
  static const std::array<std::string, NumGroups> names = {
      "Basic", "Lcals", "Polybench", "Stream", "Apps", "Algorithm", "Comm"};
  return names;
}

const std::array<std::string, NumKernels>& kernelNames() {
  static const std::array<std::string, NumKernels> names = {
      "Basic_DAXPY",        "Basic_INDEXLIST",     "Basic_INDEXLIST_3LOOP",
      "Basic_INIT3",        "Basic_MULADDSUB",     "Basic_MULTI_REDUCE",
      "Lcals_DIFF_PREDICT", "Lcals_EOS",           "Lcals_FIRST_DIFF",
      "Lcals_FIRST_MIN",    "Lcals_HYDRO_1D",      "Lcals_HYDRO_2D",
      "Lcals_INT_PREDICT",  "Lcals_PLANCKIAN",     "Polybench_3MM",
      "Polybench_FDTD_2D",  "Polybench_GEMM",      "Polybench_HEAT_3D",
      "Polybench_JACOBI_2D", "Stream_ADD",         "Stream_COPY",
      "Stream_DOT",         "Stream_MUL",          "Stream_TRIAD",
      "Apps_DEL_DOT_VEC_2D", "Apps_ENERGY",        "Apps_PRESSURE",
      "Apps_VOL3D",         "Algorithm_SCAN",      "Algorithm_REDUCE_SUM",
      "Algorithm_MEMSET",   "Algorithm_MEMCPY",    "Algorithm_HISTOGRAM",
      "Comm_HALO_PACKING",  "Comm_HALO_PACKING_FUSED"};
  return names;
}

const std::string& unknown() {
  static const std::string s = "Unknown";
  return s;
}

}  // namespace

const std::string& getGroupName(GroupID gid) {
  if (gid < 0 || gid >= NumGroups) return unknown();
  return groupNames()[gid];
}

const std::string& getFullKernelName(KernelID kid) {
  if (kid < 0 || kid >= NumKernels) return unknown();
  return kernelNames()[kid];
}

std::string getKernelName(KernelID kid) {
  const std::string& full = getFullKernelName(kid);
  std::size_t pos = full.find('_');
  return pos == std::string::npos ? full : full.substr(pos + 1);
}

const std::string& getVariantName(VariantID vid) {
  static const std::string names[NumVariants] = {"Base_GB300"};
  if (vid < 0 || vid >= NumVariants) return unknown();
  return names[vid];
}

bool isVariantAvailable(VariantID vid) { return vid == Base_GB300; }
bool isVariantGPU(VariantID vid) { return vid == Base_GB300; }

const std::string& getFeatureName(FeatureID fid) {
  static const std::string names[NumFeatures] = {
      "Forall", "Kernel", "Launch", "Sort", "Scan",
      "Workgroup", "Reduction", "Atomic", "View"};
  if (fid < 0 || fid >= NumFeatures) return unknown();
  return names[fid];
}

const std::string& getComplexityName(Complexity ac) {
  static const std::string names[] = {"N", "N_logN", "N^(3/2)", "N^(2/3)"};
  int i = static_cast<int>(ac);
  if (i < 0 || i >= static_cast<int>(Complexity::NumComplexities)) return unknown();
  return names[i];
}

KernelID getKernelIDFromName(const std::string& name) {
  for (int k = 0; k < NumKernels; ++k) {
    KernelID kid = static_cast<KernelID>(k);
    if (name == getFullKernelName(kid) || name == getKernelName(kid)) return kid;
  }
  return NumKernels;
}

GroupID getGroupIDFromName(const std::string& name) {
  for (int g = 0; g < NumGroups; ++g) {
    if (name == groupNames()[g]) return static_cast<GroupID>(g);
  }
  return NumGroups;
}

GroupID getGroupOfKernel(KernelID kid) {
  const std::string& full = getFullKernelName(kid);
  return getGroupIDFromName(full.substr(0, full.find('_')));
}

std::ostream& getCout() { return std::cout; }

std::ostream& getNullStream() {
  static std::ostream null_stream(nullptr);
  return null_stream;
}

}  // namespace rajaperf
