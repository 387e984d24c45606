#include "DataUtils.hpp"

#include <algorithm>

#include "b200.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

namespace rajaperf {
namespace detail {

namespace {
int data_init_count = 0;
}

void resetDataInitCount() { data_init_count = 0; }
void incDataInitCount() { ++data_init_count; }
int getDataInitCount() { return data_init_count; }

void initData(Real_type& d) {
  Real_type factor = (data_init_count % 2 ? 0.1 : 0.2);
  d = factor * 1.1 / 1.12345;
  incDataInitCount();
}

}  // namespace detail

void checkB200(int status, const char* what) {
  if (status != B200_OK) {
    throw std::runtime_error(std::string(what) + ": " + b200_last_error_string());
  }
}

void checkCuda(int err, const char* what) {
  if (err != cudaSuccess) {
    throw std::runtime_error(std::string(what) + ": " +
                             cudaGetErrorString(static_cast<cudaError_t>(err)));
  }
}

void* allocDeviceBytes(Size_type nbytes) {
  void* p = nullptr;
  checkCuda(cudaMalloc(&p, nbytes ? nbytes : 256), "cudaMalloc");
  return p;
}

void deallocDeviceBytes(void* p) {
  if (p) cudaFree(p);
}

void* allocPinnedBytes(Size_type nbytes) {
  void* p = nullptr;
  checkCuda(cudaHostAlloc(&p, nbytes ? nbytes : 256, cudaHostAllocMapped | cudaHostAllocPortable),
            "cudaHostAlloc");
  return p;
}

bool isHostMemory(const void* p) {
  cudaPointerAttributes a{};
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

void deallocDataBytes(void* p) {
  if (!p) return;
  if (isHostMemory(p)) cudaFreeHost(p);
  else cudaFree(p);
}

// The copies name no direction: with unified addressing the runtime takes it
// from the pointers, so the same helpers serve device arrays and the pinned
// host arrays of --host-data.
void copyToDevice(void* d, const void* h, Size_type nbytes) {
  if (nbytes) checkCuda(cudaMemcpy(d, h, nbytes, cudaMemcpyDefault), "H2D copy");
}

void copyToHost(void* h, const void* d, Size_type nbytes) {
  if (nbytes) checkCuda(cudaMemcpy(h, d, nbytes, cudaMemcpyDefault), "D2H copy");
}

void copyDeviceToDevice(void* dst, const void* src, Size_type nbytes) {
  if (nbytes) checkCuda(cudaMemcpy(dst, src, nbytes, cudaMemcpyDefault), "D2D copy");
}

void zeroDeviceBytes(void* d, Size_type nbytes) {
  if (nbytes) checkCuda(cudaMemset(d, 0, nbytes), "cudaMemset");
}

double uniformValue(unsigned long long seed, unsigned long long stream,
                    unsigned long long i, double lo, double hi) {
  auto mix = [](unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
  };
  unsigned long long key = mix(seed + 0x9e3779b97f4a7c15ULL * (stream + 1));
  unsigned long long bits = mix(key + 0x9e3779b97f4a7c15ULL * (i + 1));
  double u = static_cast<double>(bits >> 11) * 0x1.0p-53;
  return lo + (hi - lo) * u;
}

void initDeviceData(const RunParams& rp, Real_ptr d, Size_type len) {
  int count = detail::getDataInitCount();
  if (rp.getInitMode() == RunParams::InitUniform) {
    checkB200(b200_init_uniform(d, static_cast<int64_t>(len), rp.getSeed(),
                                static_cast<uint64_t>(count), rp.getInitLo(),
                                rp.getInitHi(), nullptr),
              "b200_init_uniform");
  } else {
    Real_type factor = (count % 2 ? 0.1 : 0.2);
    checkB200(b200_init_reference(d, static_cast<int64_t>(len), factor, nullptr),
              "b200_init_reference");
  }
  detail::incDataInitCount();
}

void initDeviceDataConst(Real_ptr d, Size_type len, Real_type val) {
  checkB200(b200_init_const(d, static_cast<int64_t>(len), val, nullptr),
            "b200_init_const");
  detail::incDataInitCount();
}

void initDeviceDataConst(Index_type* d, Size_type len, Index_type val) {
  checkB200(b200_init_const_i64(reinterpret_cast<int64_t*>(d),
                                static_cast<int64_t>(len), val, nullptr),
            "b200_init_const_i64");
  detail::incDataInitCount();
}

void initDeviceDataRandSign(const RunParams& rp, Real_ptr d, Size_type len) {
  if (rp.getInitMode() == RunParams::InitUniform) {
    initDeviceData(rp, d, len);
    return;
  }
  // Signs from the C library generator seeded as in DataUtils.cpp:546.
  int count = detail::getDataInitCount();
  Real_type factor = (count % 2 ? 0.1 : 0.2);
  std::vector<int8_t> sign(len);
  std::srand(4793);
  for (Size_type i = 0; i < len; ++i) {
    Real_type s = Real_type(std::rand()) / RAND_MAX;
    sign[i] = (s < 0.5 ? -1 : 1);
  }
  int8_t* dsign = static_cast<int8_t*>(allocDeviceBytes(len));
  copyToDevice(dsign, sign.data(), len);
  int st = b200_init_reference_signed(d, dsign, static_cast<int64_t>(len), factor,
                                      nullptr);
  cudaDeviceSynchronize();
  deallocDeviceBytes(dsign);
  checkB200(st, "b200_init_reference_signed");
  detail::incDataInitCount();
}

void initDeviceDataRandValue(const RunParams& rp, Real_ptr d, Size_type len) {
  if (rp.getInitMode() == RunParams::InitUniform) {
    initDeviceData(rp, d, len);
    return;
  }
  // Values rand()/RAND_MAX seeded as in DataUtils.cpp:560-569.
  std::vector<Real_type> h(len);
  std::srand(4793);
  for (Size_type i = 0; i < len; ++i) h[i] = Real_type(std::rand()) / RAND_MAX;
  copyToDevice(d, h.data(), len * sizeof(Real_type));
  detail::incDataInitCount();
}

void initDeviceDataInt(Int_ptr d, Size_type len) {
  std::vector<Int_type> h(len);
  std::srand(4793);
  for (Size_type i = 0; i < len; ++i) {
    const Real_type signfact = Real_type(std::rand()) / RAND_MAX;
    h[i] = (signfact < 0.5 ? -1 : 1);
  }
  // (rand() == RAND_MAX would put the index at len: skipped here, written
  // out of bounds by the suite)
  Real_type signfact = Real_type(std::rand()) / RAND_MAX;
  const Size_type ilo = static_cast<Size_type>(len * signfact);
  if (ilo < len) h[ilo] = -58;
  signfact = Real_type(std::rand()) / RAND_MAX;
  const Size_type ihi = static_cast<Size_type>(len * signfact);
  if (ihi < len) h[ihi] = 19;
  copyToDevice(d, h.data(), len * sizeof(Int_type));
  detail::incDataInitCount();
}

std::vector<Real_type> hostRandValues(Size_type len) {
  std::vector<Real_type> h(len);
  std::srand(4793);
  for (Size_type i = 0; i < len; ++i) h[i] = Real_type(std::rand()) / RAND_MAX;
  detail::incDataInitCount();
  return h;
}

std::vector<Index_type> hostBinAssignment(Size_type len, Index_type num_bins,
                                          RunParams::BinAssignmentAlgorithm algo) {
  using A = RunParams::BinAssignmentAlgorithm;
  std::vector<Index_type> bins(len);
  if (algo == A::Random) {
    const std::vector<Real_type> data = hostRandValues(len);
    for (Size_type i = 0; i < len; ++i) {
      Index_type b = static_cast<Index_type>(data[i] * num_bins);
      if (b >= num_bins) b = num_bins - 1;
      if (b < 0) b = 0;
      bins[i] = b;
    }
    return bins;
  }
  std::vector<Real_type> bounds;
  if (algo == A::RunsRandomSizes) {
    bounds = hostRandValues(static_cast<Size_type>(num_bins));
    std::sort(bounds.begin(), bounds.end());
  } else {
    bounds.resize(static_cast<Size_type>(num_bins));
    for (Index_type b = 0; b < num_bins; ++b)
      bounds[b] = (algo == A::RunsEvenSizes) ? static_cast<Real_type>(b + 1) / num_bins : 0.0;
  }
  Index_type bin = 0;
  for (Size_type i = 0; i < len; ++i) {
    const Real_type pos = static_cast<Real_type>(i) / len;
    while (bin + 1 < num_bins && pos >= bounds[bin]) bin += 1;
    bins[i] = bin;
  }
  return bins;
}

namespace {

template <typename Getter>
long double kahanChecksum(Getter data, Size_type len, Real_type scale_factor) {
  long double tchk = 0.0;
  long double ckahan = 0.0;
  for (Size_type j = 0; j < len; ++j) {
    long double x = (std::abs(std::sin(j + 1.0)) + 0.5) * data(j);
    long double y = x - ckahan;
    volatile long double t = tchk + y;
    volatile long double z = t - tchk;
    ckahan = z - y;
    tchk = t;
  }
  tchk *= scale_factor;
  return tchk;
}

}  // namespace

long double calcChecksumHost(const Real_type* h, Size_type len,
                             Real_type scale_factor) {
  return kahanChecksum([h](Size_type j) { return static_cast<long double>(h[j]); },
                       len, scale_factor);
}

long double calcChecksumHost(const long long* h, Size_type len,
                             Real_type scale_factor) {
  return kahanChecksum([h](Size_type j) { return static_cast<long double>(h[j]); },
                       len, scale_factor);
}

long double calcChecksumDevice(const Real_type* d, Size_type len,
                               Real_type scale_factor) {
  std::vector<Real_type> h(len);
  copyToHost(h.data(), d, len * sizeof(Real_type));
  return calcChecksumHost(h.data(), len, scale_factor);
}

long double calcChecksumDevice(const Int_type* d, Size_type len, Real_type scale_factor) {
  std::vector<Int_type> h(len);
  copyToHost(h.data(), d, len * sizeof(Int_type));
  return kahanChecksum([&h](Size_type j) { return static_cast<long double>(h[j]); }, len,
                       scale_factor);
}

long double calcChecksumHost(const unsigned long long* h, Size_type len,
                             Real_type scale_factor) {
  return kahanChecksum([h](Size_type j) { return static_cast<long double>(h[j]); }, len,
                       scale_factor);
}

long double calcChecksumDevice(const Index_type* d, Size_type len,
                               Real_type scale_factor) {
  std::vector<long long> h(len);
  copyToHost(h.data(), d, len * sizeof(long long));
  return calcChecksumHost(h.data(), len, scale_factor);
}

}  // namespace rajaperf
