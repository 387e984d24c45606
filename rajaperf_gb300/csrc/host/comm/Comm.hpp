// Comm group kernels (suite src/comm) that run in one process: HALO_PACKING
// and HALO_PACKING_FUSED.  The MPI exchange kernels stay out of scope.
#pragma once

#include "common/KernelDecl.hpp"

#include <vector>

namespace rajaperf {
namespace comm {

// The halo geometry of the suite's comm/HALO_base.{hpp,cpp}: a cube of
// grid_dims cells plus halo_width cells on every side, and for each of the 26
// neighbours the index list of the cells it is sent (the boundary layer
// inside the grid) and of the halo cells it fills.
struct HaloGeometry {
  Index_type grid_dims[3] = {0, 0, 0};
  Index_type halo_width = 0;
  Index_type var_size = 0;  // (grid + 2 halo)^3
  std::vector<std::vector<Int_type>> pack_lists, unpack_lists;  // 26 each
  HaloGeometry(double target_size, Index_type width);
  void makeLists();
};

// HALO_PACKING and HALO_PACKING_FUSED share everything but their name and
// the suite's kernels-per-rep count.
class HaloPackingBase : public KernelBase {
 public:
  HaloPackingBase(KernelID kid, const RunParams& params, bool fused);
  void setUp(VariantID vid, size_t tune_idx) override;
  void updateChecksum(VariantID vid, size_t tune_idx) override;
  void tearDown(VariantID vid, size_t tune_idx) override;
  RepBody makeRepBody(size_t tune_idx) override;

 private:
  HaloGeometry m_geo;
  Index_type m_num_vars = 0;
  std::vector<Real_ptr> m_vars;
  std::vector<Int_ptr> m_pack_lists, m_unpack_lists;
  std::vector<Real_ptr> m_pack_buffers, m_unpack_buffers;
  std::vector<b200_halo_seg> m_pack_segs, m_unpack_segs;
};

class HALO_PACKING : public HaloPackingBase {
 public:
  explicit HALO_PACKING(const RunParams& params);
};

class HALO_PACKING_FUSED : public HaloPackingBase {
 public:
  explicit HALO_PACKING_FUSED(const RunParams& params);
};

}  // namespace comm
}  // namespace rajaperf
