// Registry for the oracle build of the RAJA Performance Suite's own Base_Seq
// kernels.  It implements the free functions that the suite's
// common/RAJAPerfSuite.hpp declares (common/RAJAPerfSuite.cpp:441-1175 in the
// suite), restricted to the kernels this project accelerates.  Name strings
// follow the suite's enum spelling because the suite's RunParams parses them.
#include "common/RAJAPerfSuite.hpp"
#include "common/KernelBase.hpp"
#include "common/RunParams.hpp"

#include "stream/COPY.hpp"
#include "stream/MUL.hpp"
#include "stream/ADD.hpp"
#include "stream/TRIAD.hpp"
#include "stream/DOT.hpp"
#include "lcals/HYDRO_1D.hpp"
#include "lcals/HYDRO_2D.hpp"
#include "lcals/EOS.hpp"
#include "lcals/FIRST_DIFF.hpp"
#include "lcals/INT_PREDICT.hpp"
#include "lcals/FIRST_MIN.hpp"
#include "lcals/DIFF_PREDICT.hpp"
#include "lcals/PLANCKIAN.hpp"
#include "apps/DEL_DOT_VEC_2D.hpp"
#include "apps/VOL3D.hpp"
#include "apps/ENERGY.hpp"
#include "apps/PRESSURE.hpp"
#include "polybench/POLYBENCH_JACOBI_2D.hpp"
#include "polybench/POLYBENCH_HEAT_3D.hpp"
#include "polybench/POLYBENCH_FDTD_2D.hpp"
#include "polybench/POLYBENCH_GEMM.hpp"
#include "polybench/POLYBENCH_3MM.hpp"
#include "algorithm/SCAN.hpp"
#include "algorithm/REDUCE_SUM.hpp"
#include "basic/DAXPY.hpp"
#include "basic/INIT3.hpp"
#include "basic/MULADDSUB.hpp"
#include "basic/INDEXLIST.hpp"
#include "basic/INDEXLIST_3LOOP.hpp"
#include "basic/MULTI_REDUCE.hpp"
#include "algorithm/MEMSET.hpp"
#include "algorithm/MEMCPY.hpp"
#include "algorithm/HISTOGRAM.hpp"
#include "comm/HALO_PACKING.hpp"
#include "comm/HALO_PACKING_FUSED.hpp"

#include <iostream>
#include <string>
#include <vector>

namespace rajaperf {

namespace {

const std::vector<std::string>& groupNames() {
  static const std::vector<std::string> names = {
    "Basic", "Lcals", "Polybench", "Stream", "Apps", "Algorithm", "Comm"};
  return names;
}

struct KName { KernelID id; const char* full; };

const std::vector<KName>& kernelNames() {
  static const std::vector<KName> names = {
    {Stream_COPY, "Stream_COPY"}, {Stream_MUL, "Stream_MUL"},
    {Stream_ADD, "Stream_ADD"}, {Stream_TRIAD, "Stream_TRIAD"},
    {Stream_DOT, "Stream_DOT"},
    {Lcals_HYDRO_1D, "Lcals_HYDRO_1D"}, {Lcals_HYDRO_2D, "Lcals_HYDRO_2D"},
    {Lcals_EOS, "Lcals_EOS"}, {Lcals_FIRST_DIFF, "Lcals_FIRST_DIFF"},
    {Lcals_INT_PREDICT, "Lcals_INT_PREDICT"},
    {Lcals_FIRST_MIN, "Lcals_FIRST_MIN"},
    {Lcals_DIFF_PREDICT, "Lcals_DIFF_PREDICT"},
    {Lcals_PLANCKIAN, "Lcals_PLANCKIAN"},
    {Apps_DEL_DOT_VEC_2D, "Apps_DEL_DOT_VEC_2D"}, {Apps_VOL3D, "Apps_VOL3D"},
    {Apps_ENERGY, "Apps_ENERGY"}, {Apps_PRESSURE, "Apps_PRESSURE"},
    {Polybench_JACOBI_2D, "Polybench_JACOBI_2D"},
    {Polybench_HEAT_3D, "Polybench_HEAT_3D"},
    {Polybench_FDTD_2D, "Polybench_FDTD_2D"},
    {Polybench_GEMM, "Polybench_GEMM"}, {Polybench_3MM, "Polybench_3MM"},
    {Algorithm_SCAN, "Algorithm_SCAN"},
    {Algorithm_REDUCE_SUM, "Algorithm_REDUCE_SUM"},
    {Basic_DAXPY, "Basic_DAXPY"}, {Basic_INIT3, "Basic_INIT3"},
    {Basic_MULADDSUB, "Basic_MULADDSUB"},
    {Basic_INDEXLIST, "Basic_INDEXLIST"},
    {Basic_INDEXLIST_3LOOP, "Basic_INDEXLIST_3LOOP"},
    {Basic_MULTI_REDUCE, "Basic_MULTI_REDUCE"},
    {Algorithm_MEMSET, "Algorithm_MEMSET"}, {Algorithm_MEMCPY, "Algorithm_MEMCPY"},
    {Algorithm_HISTOGRAM, "Algorithm_HISTOGRAM"},
    {Comm_HALO_PACKING, "Comm_HALO_PACKING"},
    {Comm_HALO_PACKING_FUSED, "Comm_HALO_PACKING_FUSED"},
  };
  return names;
}

std::string& unknownName() { static std::string s = "Unknown"; return s; }

}  // namespace

const std::string& getGroupName(GroupID gid) {
  if (gid < 0 || gid >= NumGroups) return unknownName();
  return groupNames()[gid];
}

const std::string& getFullKernelName(KernelID kid) {
  static std::vector<std::string> table;
  if (table.empty()) {
    table.assign(NumKernels, std::string());
    for (KernelID k = static_cast<KernelID>(0); k < NumKernels;
         k = static_cast<KernelID>(k + 1)) {
      table[k] = "Unsupported_" + std::to_string(static_cast<int>(k));
    }
    for (const KName& kn : kernelNames()) table[kn.id] = kn.full;
  }
  if (kid < 0 || kid >= NumKernels) return unknownName();
  return table[kid];
}

std::string getKernelName(KernelID kid) {
  const std::string& full = getFullKernelName(kid);
  std::size_t pos = full.find('_');
  return full.substr(pos + 1);
}

const std::string& getVariantName(VariantID vid) {
  static const std::vector<std::string> names = {
    "Base_Seq", "Lambda_Seq", "RAJA_Seq",
    "Base_OpenMP", "Lambda_OpenMP", "RAJA_OpenMP",
    "Base_OMPTarget", "RAJA_OMPTarget",
    "Base_CUDA", "Lambda_CUDA", "RAJA_CUDA",
    "Base_HIP", "Lambda_HIP", "RAJA_HIP",
    "Kokkos_Lambda", "Base_SYCL", "RAJA_SYCL",
#if defined(RAJA_PERFSUITE_ENABLE_GB300)
    "Base_GB300",
#endif
  };
  if (vid < 0 || vid >= NumVariants) return unknownName();
  return names[vid];
}

#if defined(RAJA_PERFSUITE_ENABLE_GB300)
// the suite built with the Base_GB300 variant registered (integration.py)
bool isVariantAvailable(VariantID vid) { return vid == Base_Seq || vid == Base_GB300; }
bool isVariantGPU(VariantID vid) { return vid == Base_GB300; }
#else
bool isVariantAvailable(VariantID vid) { return vid == Base_Seq; }
bool isVariantGPU(VariantID) { return false; }
#endif

const std::string& getFeatureName(FeatureID fid) {
  static const std::vector<std::string> names = {
    "Forall", "Kernel", "Launch", "Sort", "Scan", "Workgroup",
    "Reduction", "Atomic", "View"};
  if (fid < 0 || fid >= NumFeatures) return unknownName();
  return names[fid];
}

const std::string& getComplexityName(Complexity ac) {
  static const std::vector<std::string> names = {
    "N", "N_logN", "N^(3/2)", "N^(2/3)"};
  int i = static_cast<int>(ac);
  if (i < 0 || i >= static_cast<int>(names.size())) return unknownName();
  return names[i];
}

const std::string& getDataSpaceName(DataSpace cd) {
  static const std::vector<std::string> names = {
    "Host", "Omp", "OmpTarget",
    "CudaPinned", "CudaManaged", "CudaManagedHostPreferred",
    "CudaManagedDevicePreferred", "CudaManagedHostPreferredDeviceAccessed",
    "CudaManagedDevicePreferredHostAccessed", "CudaDevice",
    "HipHostAdviseFine", "HipHostAdviseCoarse", "HipPinned", "HipPinnedFine",
    "HipPinnedCoarse", "HipManaged", "HipManagedAdviseFine",
    "HipManagedAdviseCoarse", "HipDevice", "HipDeviceFine",
    "SyclPinned", "SyclManaged", "SyclDevice",
    "NumSpaces", "Copy", "EndPseudoSpaces"};
  int i = static_cast<int>(cd);
  if (i < 0 || i >= static_cast<int>(names.size())) return unknownName();
  return names[i];
}

bool isDataSpaceAvailable(DataSpace ds) { return ds == DataSpace::Host; }
bool isPseudoDataSpace(DataSpace ds) { return ds == DataSpace::Copy; }

KernelBase* getKernelObject(KernelID kid, const RunParams& rp) {
  switch (kid) {
    case Stream_COPY: return new stream::COPY(rp);
    case Stream_MUL: return new stream::MUL(rp);
    case Stream_ADD: return new stream::ADD(rp);
    case Stream_TRIAD: return new stream::TRIAD(rp);
    case Stream_DOT: return new stream::DOT(rp);
    case Lcals_HYDRO_1D: return new lcals::HYDRO_1D(rp);
    case Lcals_HYDRO_2D: return new lcals::HYDRO_2D(rp);
    case Lcals_EOS: return new lcals::EOS(rp);
    case Lcals_FIRST_DIFF: return new lcals::FIRST_DIFF(rp);
    case Lcals_INT_PREDICT: return new lcals::INT_PREDICT(rp);
    case Lcals_FIRST_MIN: return new lcals::FIRST_MIN(rp);
    case Lcals_DIFF_PREDICT: return new lcals::DIFF_PREDICT(rp);
    case Lcals_PLANCKIAN: return new lcals::PLANCKIAN(rp);
    case Apps_DEL_DOT_VEC_2D: return new apps::DEL_DOT_VEC_2D(rp);
    case Apps_VOL3D: return new apps::VOL3D(rp);
    case Apps_ENERGY: return new apps::ENERGY(rp);
    case Apps_PRESSURE: return new apps::PRESSURE(rp);
    case Polybench_JACOBI_2D: return new polybench::POLYBENCH_JACOBI_2D(rp);
    case Polybench_HEAT_3D: return new polybench::POLYBENCH_HEAT_3D(rp);
    case Polybench_FDTD_2D: return new polybench::POLYBENCH_FDTD_2D(rp);
    case Polybench_GEMM: return new polybench::POLYBENCH_GEMM(rp);
    case Polybench_3MM: return new polybench::POLYBENCH_3MM(rp);
    case Algorithm_SCAN: return new algorithm::SCAN(rp);
    case Algorithm_REDUCE_SUM: return new algorithm::REDUCE_SUM(rp);
    case Basic_DAXPY: return new basic::DAXPY(rp);
    case Basic_INIT3: return new basic::INIT3(rp);
    case Basic_MULADDSUB: return new basic::MULADDSUB(rp);
    case Basic_INDEXLIST: return new basic::INDEXLIST(rp);
    case Basic_INDEXLIST_3LOOP: return new basic::INDEXLIST_3LOOP(rp);
    case Basic_MULTI_REDUCE: return new basic::MULTI_REDUCE(rp);
    case Algorithm_MEMSET: return new algorithm::MEMSET(rp);
    case Algorithm_MEMCPY: return new algorithm::MEMCPY(rp);
    case Algorithm_HISTOGRAM: return new algorithm::HISTOGRAM(rp);
    case Comm_HALO_PACKING: return new comm::HALO_PACKING(rp);
    case Comm_HALO_PACKING_FUSED: return new comm::HALO_PACKING_FUSED(rp);
    default: return nullptr;
  }
}

std::ostream* makeNullStream() { return new std::ostream(nullptr); }
std::ostream& getNullStream() { static std::ostream* s = makeNullStream(); return *s; }
std::ostream& getCout() { return std::cout; }

}  // namespace rajaperf
