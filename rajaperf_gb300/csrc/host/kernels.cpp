// Kernel factory: the suite's getKernelObject (common/RAJAPerfSuite.cpp:
// 788-1136) restricted to the kernels this library implements.
#include "common/RAJAPerfSuite.hpp"
#include "algorithm/Algorithm.hpp"
#include "apps/Apps.hpp"
#include "basic/Basic.hpp"
#include "comm/Comm.hpp"
#include "lcals/Lcals.hpp"
#include "polybench/Polybench.hpp"
#include "stream/Stream.hpp"

namespace rajaperf {

KernelBase* getKernelObject(KernelID kid, const RunParams& rp) {
  switch (kid) {
    case Stream_COPY: return new stream::COPY(rp);
    case Stream_MUL: return new stream::MUL(rp);
    case Stream_ADD: return new stream::ADD(rp);
    case Stream_TRIAD: return new stream::TRIAD(rp);
    case Stream_DOT: return new stream::DOT(rp);
    case Basic_DAXPY: return new basic::DAXPY(rp);
    case Basic_INIT3: return new basic::INIT3(rp);
    case Basic_MULADDSUB: return new basic::MULADDSUB(rp);
    case Basic_INDEXLIST: return new basic::INDEXLIST(rp);
    case Basic_INDEXLIST_3LOOP: return new basic::INDEXLIST_3LOOP(rp);
    case Basic_MULTI_REDUCE: return new basic::MULTI_REDUCE(rp);
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
    case Algorithm_MEMSET: return new algorithm::MEMSET(rp);
    case Algorithm_MEMCPY: return new algorithm::MEMCPY(rp);
    case Algorithm_HISTOGRAM: return new algorithm::HISTOGRAM(rp);
    case Comm_HALO_PACKING: return new comm::HALO_PACKING(rp);
    case Comm_HALO_PACKING_FUSED: return new comm::HALO_PACKING_FUSED(rp);
    default: return nullptr;
  }
}

}  // namespace rajaperf
