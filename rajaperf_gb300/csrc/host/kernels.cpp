// Kernel factory: the suite's getKernelObject (common/RAJAPerfSuite.cpp:
// 788-1136) restricted to the kernels this library implements.
#include "common/RAJAPerfSuite.hpp"
#include "stream/Stream.hpp"

namespace rajaperf {

KernelBase* getKernelObject(KernelID kid, const RunParams& rp) {
  switch (kid) {
    case Stream_COPY: return new stream::COPY(rp);
    case Stream_MUL: return new stream::MUL(rp);
    case Stream_ADD: return new stream::ADD(rp);
    case Stream_TRIAD: return new stream::TRIAD(rp);
    case Stream_DOT: return new stream::DOT(rp);
    default: return nullptr;
  }
}

}  // namespace rajaperf
