// HALO_PACKING / HALO_PACKING_FUSED (comm group, one process): gather each
// neighbour's boundary cells of every variable into its pack buffer
// (buffer[i] = var[list[i]]), then scatter each unpack buffer into the halo
// cells (var[list[i]] = buffer[i]).
//
// The suite's GPU variants launch one kernel per (neighbour, variable) and
// direction -- 2 x 26 x num_vars launches per rep.  Here one launch packs every
// segment and a second one unpacks every segment: blockIdx.y picks the
// segment (its fields are uniform kernel-parameter loads), blockIdx.x a chunk
// of block x items entries of it; chunks past a short segment's end exit at
// once.  The unpack launch runs after the pack launch, so packs always see
// the variables as they were before this call's unpacks; unpack segments run
// concurrently, so two of them writing the same element land in unspecified
// order (the suite's halo lists never overlap: every halo cell belongs to one
// neighbour).
#include "b200_internal.cuh"

using namespace b200;

namespace {

constexpr int kBlock = 256;
constexpr int kItems = 4;
constexpr int kMaxSegments = 256;

struct SegTable {
  b200_halo_seg seg[kMaxSegments];
};

template <bool PACK>
__global__ void __launch_bounds__(kBlock) halo_kernel(const __grid_constant__ SegTable t) {
  const b200_halo_seg& s = t.seg[blockIdx.y];
  const int64_t base = static_cast<int64_t>(blockIdx.x) * (kBlock * kItems);
  if (base >= s.len) return;
  int32_t idx[kItems];
#pragma unroll
  for (int u = 0; u < kItems; ++u) {
    const int64_t i = base + u * kBlock + threadIdx.x;
    idx[u] = (i < s.len) ? __ldg(s.list + i) : 0;
  }
  if (PACK) {
    double v[kItems];
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      const int64_t i = base + u * kBlock + threadIdx.x;
      v[u] = (i < s.len) ? s.var[idx[u]] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      const int64_t i = base + u * kBlock + threadIdx.x;
      if (i < s.len) s.buffer[i] = v[u];
    }
  } else {
    double v[kItems];
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      const int64_t i = base + u * kBlock + threadIdx.x;
      v[u] = (i < s.len) ? __ldcs(s.buffer + i) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kItems; ++u) {
      const int64_t i = base + u * kBlock + threadIdx.x;
      if (i < s.len) s.var[idx[u]] = v[u];
    }
  }
}

// Copies the segments into a parameter table; returns the chunks needed by
// the longest one (0 if every segment is empty).
int fill(SegTable& t, const b200_halo_seg* segs, int n, const char* name, int* chunks) {
  int64_t longest = 0;
  for (int k = 0; k < n; ++k) {
    const b200_halo_seg& s = segs[k];
    if (s.len < 0 || (s.len > 0 && (!s.var || !s.list || !s.buffer)))
      return invalid("%s: bad segment %d", name, k);
    t.seg[k] = s;
    if (s.len > longest) longest = s.len;
  }
  const int64_t c = ceil_div(longest, kBlock * kItems);
  if (c > 0x7fffffffLL) return invalid("%s: segment too long", name);
  *chunks = static_cast<int>(c);
  return B200_OK;
}

}  // namespace

extern "C" {

int b200_comm_halo_packing(const b200_halo_seg* pack, int32_t n_pack,
                           const b200_halo_seg* unpack, int32_t n_unpack,
                           const b200_tune* tune, b200_stream_t stream) {
  (void)tune;
  const char* name = "b200_comm_halo_packing";
  if (n_pack < 0 || n_unpack < 0 || n_pack > kMaxSegments || n_unpack > kMaxSegments ||
      (n_pack > 0 && !pack) || (n_unpack > 0 && !unpack))
    return invalid("%s: bad segment tables (at most %d per direction)", name, kMaxSegments);
  cudaStream_t st = as_stream(stream);
  SegTable tp, tu;
  int cp = 0, cu = 0, launches = 0;
  int rc = fill(tp, pack, n_pack, name, &cp);
  if (rc != B200_OK) return rc;
  rc = fill(tu, unpack, n_unpack, name, &cu);
  if (rc != B200_OK) return rc;
  if (n_pack > 0 && cp > 0) {
    halo_kernel<true><<<dim3(static_cast<unsigned>(cp), static_cast<unsigned>(n_pack)), kBlock,
                        0, st>>>(tp);
    ++launches;
  }
  if (n_unpack > 0 && cu > 0) {
    halo_kernel<false><<<dim3(static_cast<unsigned>(cu), static_cast<unsigned>(n_unpack)),
                         kBlock, 0, st>>>(tu);
    ++launches;
  }
  if (launches == 0) return B200_OK;
  return after_launch(name, launches);
}

}  // extern "C"
