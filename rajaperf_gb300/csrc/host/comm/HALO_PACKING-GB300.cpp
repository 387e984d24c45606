// Comm_HALO_PACKING and Comm_HALO_PACKING_FUSED in one process.  Follow the
// suite's comm/HALO_base.cpp:22-285 (grid, 26 neighbour offsets, send/receive
// extents and index lists), comm/HALO_PACKING.cpp:18-170 and
// HALO_PACKING_FUSED.cpp (sizes, set-up order, checksum over the variables
// and the send buffers).  One rep packs every (neighbour, variable) segment,
// then unpacks every segment, in two launches of b200_comm_halo_packing.
#include "Comm.hpp"

#include <cmath>
#include <stdexcept>

namespace rajaperf {
namespace comm {

namespace {

constexpr int kNumNeighbors = 26;

// comm/HALO_base.cpp:80-116: faces, edges, corners.
const int kOffsets[kNumNeighbors][3] = {
    {-1, 0, 0},   {1, 0, 0},   {0, -1, 0},  {0, 1, 0},   {0, 0, -1},  {0, 0, 1},
    {-1, -1, 0},  {-1, 1, 0},  {1, -1, 0},  {1, 1, 0},   {-1, 0, -1}, {-1, 0, 1},
    {1, 0, -1},   {1, 0, 1},   {0, -1, -1}, {0, -1, 1},  {0, 1, -1},  {0, 1, 1},
    {-1, -1, -1}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},
    {1, 1, -1},   {1, 1, 1}};

// Cells [first, second) along one axis (comm/HALO_base.cpp:118-162).
void bounds(int offset, bool send, Index_type w, Index_type dim, Index_type* lo,
            Index_type* hi) {
  if (offset == -1) {
    *lo = send ? w : 0;
    *hi = send ? w + w : w;
  } else if (offset == 0) {
    *lo = w;
    *hi = w + dim;
  } else {
    *lo = send ? w + dim - w : w + dim;
    *hi = send ? w + dim : w + dim + w;
  }
}

}  // namespace

HaloGeometry::HaloGeometry(double target_size, Index_type width) : halo_width(width) {
  const double cbrt_run_size = std::cbrt(target_size) + std::cbrt(3) - 1;
  for (int d = 0; d < 3; ++d) grid_dims[d] = static_cast<Index_type>(cbrt_run_size);
  var_size = (grid_dims[0] + 2 * width) * (grid_dims[1] + 2 * width) *
             (grid_dims[2] + 2 * width);
}

void HaloGeometry::makeLists() {
  const Index_type js = grid_dims[0] + 2 * halo_width;
  const Index_type ks = js * (grid_dims[1] + 2 * halo_width);
  pack_lists.assign(kNumNeighbors, {});
  unpack_lists.assign(kNumNeighbors, {});
  for (int l = 0; l < kNumNeighbors; ++l) {
    for (int pass = 0; pass < 2; ++pass) {
      const bool send = (pass == 0);
      Index_type lo[3], hi[3];
      for (int d = 0; d < 3; ++d) bounds(kOffsets[l][d], send, halo_width, grid_dims[d], &lo[d], &hi[d]);
      std::vector<Int_type>& list = send ? pack_lists[l] : unpack_lists[l];
      for (Index_type k = lo[2]; k < hi[2]; ++k)
        for (Index_type j = lo[1]; j < hi[1]; ++j)
          for (Index_type i = lo[0]; i < hi[0]; ++i)
            list.push_back(static_cast<Int_type>(i + j * js + k * ks));
    }
  }
}

HaloPackingBase::HaloPackingBase(KernelID kid, const RunParams& params, bool fused)
    : KernelBase(kid, params),
      m_geo(1.0, params.getHaloWidth()) {
  setDefaultProblemSize(100 * 100 * 100);
  setDefaultReps(200);
  m_geo = HaloGeometry(getTargetProblemSize(), params.getHaloWidth());
  // the suite sets grid_dims[0] * grid_dims[1] * grid_dims[1] (HALO_base.cpp:45)
  setActualProblemSize(m_geo.grid_dims[0] * m_geo.grid_dims[1] * m_geo.grid_dims[1]);
  m_num_vars = params.getHaloNumVars();
  setItsPerRep(m_num_vars * (m_geo.var_size - getActualProblemSize()));
  setKernelsPerRep(fused ? 2 : 2 * kNumNeighbors * m_num_vars);
  setBytesReadPerRep(1 * sizeof(Int_type) * getItsPerRep() + 1 * sizeof(Real_type) * getItsPerRep() +
                     1 * sizeof(Int_type) * getItsPerRep() + 1 * sizeof(Real_type) * getItsPerRep());
  setBytesWrittenPerRep(1 * sizeof(Real_type) * getItsPerRep() +
                        1 * sizeof(Real_type) * getItsPerRep());
  setBytesAtomicModifyWrittenPerRep(0);
  setFLOPsPerRep(0);
  setComplexity(Complexity::N_to_the_two_thirds);
  setUsesFeature(Forall);
  setVariantDefined(Base_GB300);
}

void HaloPackingBase::setUp(VariantID vid, size_t) {
  m_geo.makeLists();
  // HALO_base.cpp:218-276: every list is allocated and initialised (then
  // overwritten), send then receive per neighbour: one init count each
  m_pack_lists.assign(kNumNeighbors, nullptr);
  m_unpack_lists.assign(kNumNeighbors, nullptr);
  for (int l = 0; l < kNumNeighbors; ++l) {
    for (int pass = 0; pass < 2; ++pass) {
      const std::vector<Int_type>& h = pass == 0 ? m_geo.pack_lists[l] : m_geo.unpack_lists[l];
      Int_ptr& d = pass == 0 ? m_pack_lists[l] : m_unpack_lists[l];
      allocData(d, h.size(), vid);
      copyToDevice(d, h.data(), h.size() * sizeof(Int_type));
      detail::incDataInitCount();
    }
  }
  // HALO_PACKING.cpp:71-81: var[i] = i + v (after an initialisation that counts)
  m_vars.assign(m_num_vars, nullptr);
  std::vector<Real_type> h(m_geo.var_size);
  for (Index_type v = 0; v < m_num_vars; ++v) {
    allocData(m_vars[v], m_geo.var_size, vid);
    for (Index_type i = 0; i < m_geo.var_size; ++i) h[i] = static_cast<Real_type>(i + v);
    copyToDevice(m_vars[v], h.data(), m_geo.var_size * sizeof(Real_type));
    detail::incDataInitCount();
  }
  // HALO_PACKING.cpp:85-109: pack, then unpack buffers of num_vars x list length
  m_pack_buffers.assign(kNumNeighbors, nullptr);
  m_unpack_buffers.assign(kNumNeighbors, nullptr);
  for (int l = 0; l < kNumNeighbors; ++l)
    allocAndInitData(m_pack_buffers[l], m_num_vars * m_geo.pack_lists[l].size(), vid);
  for (int l = 0; l < kNumNeighbors; ++l)
    allocAndInitData(m_unpack_buffers[l], m_num_vars * m_geo.unpack_lists[l].size(), vid);
  m_pack_segs.clear();
  m_unpack_segs.clear();
  for (int l = 0; l < kNumNeighbors; ++l) {
    const int64_t lp = static_cast<int64_t>(m_geo.pack_lists[l].size());
    const int64_t lu = static_cast<int64_t>(m_geo.unpack_lists[l].size());
    for (Index_type v = 0; v < m_num_vars; ++v) {
      m_pack_segs.push_back({m_vars[v], m_pack_lists[l], m_pack_buffers[l] + v * lp, lp});
      m_unpack_segs.push_back({m_vars[v], m_unpack_lists[l], m_unpack_buffers[l] + v * lu, lu});
    }
  }
}

KernelBase::RepBody HaloPackingBase::makeRepBody(size_t tune_idx) {
  const b200_tune tn = getTune(tune_idx);
  const std::vector<b200_halo_seg> pack = m_pack_segs, unpack = m_unpack_segs;
  return [=](b200_stream_t s) {
    checkB200(b200_comm_halo_packing(pack.data(), static_cast<int32_t>(pack.size()),
                                     unpack.data(), static_cast<int32_t>(unpack.size()), &tn,
                                     s),
              "b200_comm_halo_packing");
  };
}

void HaloPackingBase::updateChecksum(VariantID vid, size_t tune_idx) {
  for (Real_ptr var : m_vars) checksum[vid][tune_idx] += calcChecksum(var, m_geo.var_size, vid);
  for (int l = 0; l < kNumNeighbors; ++l)
    checksum[vid][tune_idx] +=
        calcChecksum(m_pack_buffers[l], m_num_vars * m_geo.pack_lists[l].size(), vid);
}

void HaloPackingBase::tearDown(VariantID vid, size_t) {
  for (Real_ptr& p : m_unpack_buffers) deallocData(p, vid);
  for (Real_ptr& p : m_pack_buffers) deallocData(p, vid);
  for (Real_ptr& p : m_vars) deallocData(p, vid);
  for (Int_ptr& p : m_pack_lists) deallocData(p, vid);
  for (Int_ptr& p : m_unpack_lists) deallocData(p, vid);
  m_unpack_buffers.clear();
  m_pack_buffers.clear();
  m_vars.clear();
  m_pack_lists.clear();
  m_unpack_lists.clear();
  m_pack_segs.clear();
  m_unpack_segs.clear();
}

HALO_PACKING::HALO_PACKING(const RunParams& params)
    : HaloPackingBase(rajaperf::Comm_HALO_PACKING, params, false) {}

HALO_PACKING_FUSED::HALO_PACKING_FUSED(const RunParams& params)
    : HaloPackingBase(rajaperf::Comm_HALO_PACKING_FUSED, params, true) {}

}  // namespace comm
}  // namespace rajaperf
