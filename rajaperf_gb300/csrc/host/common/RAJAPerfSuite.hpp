// Kernel / variant / group identifiers and the kernel factory.
//
// Follows the suite's common/RAJAPerfSuite.hpp:47-344: group, kernel and
// variant enums plus name lookups.  The kernel list is the loop-kernel hot
// path this library accelerates; names are spelled as in the suite
// ("Stream_TRIAD") so command lines and reports stay interchangeable.  The
// only variant is Base_GB300.
#pragma once

#include "RPTypes.hpp"

#include <ostream>
#include <string>

namespace rajaperf {

class KernelBase;
class RunParams;

enum GroupID {
  Basic = 0,
  Lcals,
  Polybench,
  Stream,
  Apps,
  Algorithm,
  Comm,
  NumGroups
};

enum KernelID {
  Basic_DAXPY = 0,
  Basic_INDEXLIST,
  Basic_INDEXLIST_3LOOP,
  Basic_INIT3,
  Basic_MULADDSUB,
  Basic_MULTI_REDUCE,

  Lcals_DIFF_PREDICT,
  Lcals_EOS,
  Lcals_FIRST_DIFF,
  Lcals_FIRST_MIN,
  Lcals_HYDRO_1D,
  Lcals_HYDRO_2D,
  Lcals_INT_PREDICT,
  Lcals_PLANCKIAN,

  Polybench_3MM,
  Polybench_FDTD_2D,
  Polybench_GEMM,
  Polybench_HEAT_3D,
  Polybench_JACOBI_2D,

  Stream_ADD,
  Stream_COPY,
  Stream_DOT,
  Stream_MUL,
  Stream_TRIAD,

  Apps_DEL_DOT_VEC_2D,
  Apps_ENERGY,
  Apps_PRESSURE,
  Apps_VOL3D,

  Algorithm_SCAN,
  Algorithm_REDUCE_SUM,
  Algorithm_MEMSET,
  Algorithm_MEMCPY,
  Algorithm_HISTOGRAM,

  Comm_HALO_PACKING,
  Comm_HALO_PACKING_FUSED,

  NumKernels
};

enum VariantID {
  Base_GB300 = 0,
  NumVariants
};

enum FeatureID {
  Forall = 0,
  Kernel,
  Launch,
  Sort,
  Scan,
  Workgroup,
  Reduction,
  Atomic,
  View,
  NumFeatures
};

enum struct Complexity {
  N = 0,
  N_logN,
  N_to_the_three_halves,
  N_to_the_two_thirds,
  NumComplexities
};

const std::string& getGroupName(GroupID gid);
std::string getKernelName(KernelID kid);
const std::string& getFullKernelName(KernelID kid);
const std::string& getVariantName(VariantID vid);
bool isVariantAvailable(VariantID vid);
bool isVariantGPU(VariantID vid);
const std::string& getFeatureName(FeatureID fid);
const std::string& getComplexityName(Complexity ac);

// Kernel id for a full ("Stream_TRIAD") or short ("TRIAD") name; NumKernels
// when unknown.
KernelID getKernelIDFromName(const std::string& name);
GroupID getGroupIDFromName(const std::string& name);
GroupID getGroupOfKernel(KernelID kid);

// Creates the kernel object (caller owns it).  Defined next to the kernels.
KernelBase* getKernelObject(KernelID kid, const RunParams& run_params);

std::ostream& getCout();
std::ostream& getNullStream();

}  // namespace rajaperf
