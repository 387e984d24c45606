// INDEXLIST (and INDEXLIST_3LOOP): list[count++] = i for every i with
// x[i] < 0, in index order, and the final count.
//
// One pass, stream compaction on the decoupled lookback of b200_lookback.cuh.
// A CTA owns a tile of 8 warps x 32 lanes x 32 items; each warp owns a
// contiguous segment of 1024 items and reads it row by row (coalesced,
// 16-byte item pairs when x is aligned).  Ballots per row give every selected
// item its rank inside the row; the warp's running count orders the rows; a
// scan of the warp counts orders the warps; the lookback gives the tile's
// base count.  The indices are then written to consecutive list entries.
// The suite's INDEXLIST_3LOOP
// (counts, exclusive scan of counts, list from count changes) produces the
// same list and count; it runs through the same single pass.
#include "b200_internal.cuh"
#include "b200_lookback.cuh"

using namespace b200;

namespace {

constexpr int kBlock = 256;
constexpr int kItems = 32;
constexpr int kTile = kBlock * kItems;  // 8192 items
constexpr int kSeg = 32 * kItems;       // a warp's segment: 1024 items

// VEC: 16-byte loads, lane L of row u holds items seg + 64u + 2L and +1 (x
// 16-byte aligned, n even or the tile full); otherwise 8-byte loads, lane L
// of row u holds item seg + 32u + L.  Ranks follow index order either way.
template <bool VEC>
__global__ void __launch_bounds__(kBlock, 3)
indexlist_kernel(const double* __restrict__ x, int32_t* __restrict__ list, int64_t n,
                 int64_t* __restrict__ len, ScanHeader* __restrict__ hdr,
                 TileDesc* __restrict__ descs) {
  constexpr int kRows = VEC ? kItems / 2 : kItems;
  __shared__ long long s_woff[kBlock / 32];
  __shared__ long long s_agg;
  __shared__ long long s_excl;
  __shared__ unsigned int s_tile_id;
  __shared__ unsigned long long s_epoch;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  take_tile(hdr, &s_tile_id, &s_epoch);
  const unsigned int tile = s_tile_id;
  const unsigned long long epoch = s_epoch;
  const unsigned long long AGG = epoch * 4 + 1, INC = epoch * 4 + 2;
  const int64_t seg = static_cast<int64_t>(tile) * kTile + warp * kSeg;

  unsigned int b0[kRows], b1[kRows];  // ballots of the even / odd items of a row
  int wcount = 0;
#pragma unroll
  for (int u = 0; u < kRows; ++u) {
    if (VEC) {
      const int64_t i = seg + 64 * u + 2 * lane;
      double2 v = make_double2(0.0, 0.0);
      if (i + 1 < n) {
        v = __ldcs(reinterpret_cast<const double2*>(x + i));
      } else if (i < n) {
        v.x = __ldcs(x + i);
      }
      b0[u] = __ballot_sync(0xffffffffu, i < n && v.x < 0.0);
      b1[u] = __ballot_sync(0xffffffffu, i + 1 < n && v.y < 0.0);
      wcount += __popc(b0[u]) + __popc(b1[u]);
    } else {
      const int64_t i = seg + 32 * u + lane;
      b0[u] = __ballot_sync(0xffffffffu, (i < n) && (__ldcs(x + i) < 0.0));
      b1[u] = 0u;
      wcount += __popc(b0[u]);
    }
  }
  if (lane == 0) s_woff[warp] = wcount;
  __syncthreads();
  if (warp == 0) {
    const long long w = (lane < kBlock / 32) ? s_woff[lane] : 0;
    long long wi = w;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const long long o = __shfl_up_sync(0xffffffffu, wi, off);
      if (lane >= off) wi += o;
    }
    if (lane < kBlock / 32) s_woff[lane] = wi - w;
    const long long agg = __shfl_sync(0xffffffffu, wi, kBlock / 32 - 1);
    if (tile > 0) {
      if (lane == 0) desc_store(descs + tile, AGG, to_bits<long long>(agg));
      const long long excl = lookback_exclusive<long long>(descs, tile, AGG, INC, hdr);
      if (lane == 0) {
        desc_store(descs + tile, INC, to_bits<long long>(excl + agg));
        s_excl = excl;
        s_agg = agg;
      }
    } else if (lane == 0) {
      desc_store(descs, INC, to_bits<long long>(agg));
      s_excl = 0;
      s_agg = agg;
    }
  }
  __syncthreads();
  long long off = s_excl + s_woff[warp];
  const unsigned int below = (1u << lane) - 1u;
#pragma unroll
  for (int u = 0; u < kRows; ++u) {
    if (VEC) {
      const int64_t i = seg + 64 * u + 2 * lane;
      const int r = __popc(b0[u] & below) + __popc(b1[u] & below);
      const bool s0 = (b0[u] >> lane) & 1u, s1 = (b1[u] >> lane) & 1u;
      if (s0) list[off + r] = static_cast<int32_t>(i);
      if (s1) list[off + r + (s0 ? 1 : 0)] = static_cast<int32_t>(i + 1);
      off += __popc(b0[u]) + __popc(b1[u]);
    } else {
      if ((b0[u] >> lane) & 1u)
        list[off + __popc(b0[u] & below)] = static_cast<int32_t>(seg + 32 * u + lane);
      off += __popc(b0[u]);
    }
  }
  // the tile holding item n-1 knows the total
  if (tid == 0 && static_cast<int64_t>(tile + 1) * kTile >= n) *len = s_excl + s_agg;
}

int64_t tiles_of(int64_t n) { return ceil_div(n > 0 ? n : 1, kTile); }

}  // namespace

extern "C" {

size_t b200_indexlist_workspace_bytes(int64_t n) {
  return 256 + static_cast<size_t>(tiles_of(n)) * sizeof(TileDesc);
}

int b200_basic_indexlist(const double* x, int32_t* list, int64_t n, int64_t* len,
                         void* workspace, size_t workspace_bytes, const b200_tune* tune,
                         b200_stream_t stream) {
  if (n < 0 || !len || (n > 0 && (!x || !list)))
    return invalid("b200_basic_indexlist: bad args");
  if (n > 0x7fffffffLL) return invalid("b200_basic_indexlist: n exceeds the int32 list range");
  const size_t need = b200_indexlist_workspace_bytes(n);
  if (workspace && !aligned16(workspace))
    return invalid("b200_basic_indexlist: workspace not 16-byte aligned");
  if (!workspace || workspace_bytes < need) {
    set_error("b200_basic_indexlist: workspace %zu bytes, need %zu", workspace_bytes, need);
    return B200_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  if (n == 0) {
    const cudaError_t e = cudaMemsetAsync(len, 0, sizeof(int64_t), st);
    if (e != cudaSuccess) {
      set_error("b200_basic_indexlist: %s", cudaGetErrorString(e));
      return B200_ERR_LAUNCH;
    }
    return B200_OK;
  }
  char* w = static_cast<char*>(workspace);
  ScanHeader* hdr = reinterpret_cast<ScanHeader*>(w);
  TileDesc* descs = reinterpret_cast<TileDesc*>(w + 256);
  const unsigned tiles = static_cast<unsigned>(tiles_of(n));
  if (aligned16(x) && !(tune && tune->vec == 1))
    indexlist_kernel<true><<<tiles, kBlock, 0, st>>>(x, list, n, len, hdr, descs);
  else
    indexlist_kernel<false><<<tiles, kBlock, 0, st>>>(x, list, n, len, hdr, descs);
  return after_launch("b200_basic_indexlist");
}

}  // extern "C"
