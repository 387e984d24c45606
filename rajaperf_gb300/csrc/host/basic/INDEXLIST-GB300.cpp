// Basic_INDEXLIST and Basic_INDEXLIST_3LOOP: the indices i with x[i] < 0, in
// order, and their count.  Follow the suite's basic/INDEXLIST.cpp:22-80 and
// basic/INDEXLIST_3LOOP.cpp:22-92: x with random signs, the list array from
// the Int_type formula, checksum over the whole list plus the length.  Both
// run the single-pass b200_basic_indexlist; INDEXLIST_3LOOP keeps the suite's
// three-loop byte and kernel counts.
#include "Basic.hpp"

namespace rajaperf {
namespace basic {

namespace {

template <typename K>
void setUpIndexList(K* k, Real_ptr& x, Int_ptr& list, int64_t*& dlen, void*& ws,
                    size_t& ws_bytes, Index_type& len, VariantID vid) {
  const Index_type n = k->getActualProblemSize();
  k->allocAndInitDataRandSign(x, n, vid);
  k->allocData(list, n, vid);
  initDeviceDataInt(list, n);
  len = -1;
  dlen = static_cast<int64_t*>(allocDeviceBytes(sizeof(int64_t)));
  ws_bytes = b200_indexlist_workspace_bytes(n);
  ws = allocDeviceBytes(ws_bytes);
  zeroDeviceBytes(ws, ws_bytes);
}

}  // namespace

INDEXLIST::INDEXLIST(const RunParams& params) : KernelBase(rajaperf::Basic_INDEXLIST, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(100);
  setActualProblemSize(getTargetProblemSize());
  setItsPerRep(getActualProblemSize());
  setKernelsPerRep(1);
  setBytesReadPerRep(1 * sizeof(Index_type) + 1 * sizeof(Real_type) * getActualProblemSize());
  setBytesWrittenPerRep(1 * sizeof(Index_type) +
                        1 * sizeof(Int_type) * getActualProblemSize() / 2);
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(0);
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setUsesFeature(Scan);
  setVariantDefined(Base_GB300);
}

void INDEXLIST::setUp(VariantID vid, size_t) {
  setUpIndexList(this, m_x, m_list, m_dlen, m_ws, m_ws_bytes, m_len, vid);
}

KernelBase::RepBody INDEXLIST::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_basic_indexlist(m_x, m_list, n, m_dlen, m_ws, m_ws_bytes, &tn, s),
              "b200_basic_indexlist");
  };
}

void INDEXLIST::prepareRun(size_t tune_idx) {
  injectLookbackStall(m_ws, m_ws_bytes, getTune(tune_idx),
                      reinterpret_cast<uintptr_t>(m_x) % 16 == 0);
}

void INDEXLIST::finishRun(size_t) {
  checkWorkspace(m_ws, m_ws_bytes, "Basic_INDEXLIST");
  int64_t len = -1;
  copyToHost(&len, m_dlen, sizeof(len));
  m_len = static_cast<Index_type>(len);
}

void INDEXLIST::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksumDevice(m_list, getActualProblemSize(), 1.0);
  checksum[vid][tune_idx] += Checksum_type(m_len);
}

void INDEXLIST::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_list, vid);
  deallocDeviceBytes(m_dlen);
  deallocDeviceBytes(m_ws);
  m_dlen = nullptr;
  m_ws = nullptr;
}

INDEXLIST_3LOOP::INDEXLIST_3LOOP(const RunParams& params)
    : KernelBase(rajaperf::Basic_INDEXLIST_3LOOP, params) {
  setDefaultProblemSize(1000000);
  setDefaultReps(100);
  setActualProblemSize(getTargetProblemSize());
  const Index_type n = getActualProblemSize();
  setItsPerRep(3 * n + 1);
  setKernelsPerRep(3);
  setBytesReadPerRep(1 * sizeof(Real_type) * n + 1 * sizeof(Index_type) +
                     1 * sizeof(Index_type) * (n + 1) + 1 * sizeof(Index_type) * (n + 1));
  setBytesWrittenPerRep(1 * sizeof(Index_type) * n + 1 * sizeof(Index_type) +
                        1 * sizeof(Index_type) * (n + 1) + 1 * sizeof(Int_type) * (n + 1) / 2);
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(0);
  setComplexity(Complexity::N);
  setUsesFeature(Forall);
  setUsesFeature(Scan);
  setVariantDefined(Base_GB300);
}

void INDEXLIST_3LOOP::setUp(VariantID vid, size_t) {
  setUpIndexList(this, m_x, m_list, m_dlen, m_ws, m_ws_bytes, m_len, vid);
}

KernelBase::RepBody INDEXLIST_3LOOP::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const Index_type n = getActualProblemSize();
  return [=](b200_stream_t s) {
    checkB200(b200_basic_indexlist(m_x, m_list, n, m_dlen, m_ws, m_ws_bytes, &tn, s),
              "b200_basic_indexlist");
  };
}

void INDEXLIST_3LOOP::prepareRun(size_t tune_idx) {
  injectLookbackStall(m_ws, m_ws_bytes, getTune(tune_idx),
                      reinterpret_cast<uintptr_t>(m_x) % 16 == 0);
}

void INDEXLIST_3LOOP::finishRun(size_t) {
  checkWorkspace(m_ws, m_ws_bytes, "Basic_INDEXLIST_3LOOP");
  int64_t len = -1;
  copyToHost(&len, m_dlen, sizeof(len));
  m_len = static_cast<Index_type>(len);
}

void INDEXLIST_3LOOP::updateChecksum(VariantID vid, size_t tune_idx) {
  checksum[vid][tune_idx] += calcChecksumDevice(m_list, getActualProblemSize(), 1.0);
  checksum[vid][tune_idx] += Checksum_type(m_len);
}

void INDEXLIST_3LOOP::tearDown(VariantID vid, size_t) {
  deallocData(m_x, vid);
  deallocData(m_list, vid);
  deallocDeviceBytes(m_dlen);
  deallocDeviceBytes(m_ws);
  m_dlen = nullptr;
  m_ws = nullptr;
}

}  // namespace basic
}  // namespace rajaperf
