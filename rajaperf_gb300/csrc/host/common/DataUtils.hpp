// Device data allocation, initialisation and checksums for Base_GB300.
//
// Follows the suite's common/DataUtils.{hpp,cpp}: arrays are initialised in
// the order the kernel's setUp requests them and every initialisation bumps
// the data-init counter (DataUtils.cpp:131-147), whose parity picks the 0.1 /
// 0.2 factor of the deterministic formula (DataUtils.cpp:504-513).  Arrays
// live in device memory and are filled on the device with bit-identical
// arithmetic; values that come from the C library's rand()
// (DataUtils.cpp:542-569) are generated on the host and copied.
//
// The checksum is the suite's weighted Kahan sum in long double
// (DataUtils.cpp:600-621), computed on the host after a device-to-host copy.
#pragma once

#include "RPTypes.hpp"
#include "RunParams.hpp"

#include <cstdint>
#include <vector>

namespace rajaperf {
namespace detail {

void resetDataInitCount();
void incDataInitCount();
int getDataInitCount();

// Scalar value of the deterministic formula at the current count
// (DataUtils.cpp:589-595); bumps the count.
void initData(Real_type& d);

}  // namespace detail

// Device allocation (cudaMalloc); throws std::runtime_error on failure.
void* allocDeviceBytes(Size_type nbytes);
void deallocDeviceBytes(void* p);
// Pinned host memory mapped into the device's address space (the suite's
// CudaPinned data space): kernels read and write it across the host link.
void* allocPinnedBytes(Size_type nbytes);
bool isHostMemory(const void* p);
// Frees device or pinned host memory, whichever p is.
void deallocDataBytes(void* p);

// Fills a device array.  Each call bumps the data-init counter once.
void initDeviceData(const RunParams& rp, Real_ptr d, Size_type len);
void initDeviceDataConst(Real_ptr d, Size_type len, Real_type val);
void initDeviceDataConst(Index_type* d, Size_type len, Index_type val);
void initDeviceDataRandSign(const RunParams& rp, Real_ptr d, Size_type len);
void initDeviceDataRandValue(const RunParams& rp, Real_ptr d, Size_type len);
// Int_type arrays: +-1 by the C library generator, then -58 and 19 at two
// generated positions (DataUtils.cpp:477-497), in either init mode.
void initDeviceDataInt(Int_ptr d, Size_type len);
// rand()/RAND_MAX values seeded as the suite seeds them (DataUtils.cpp:560-569),
// on the host; bumps the data-init counter.
std::vector<Real_type> hostRandValues(Size_type len);
// The bin of every item for HISTOGRAM / MULTI_REDUCE, as their setUp assigns
// them (algorithm/HISTOGRAM.cpp:73-131): runs whose boundaries are sorted
// random values, even runs, one bin, or a random bin per item.
std::vector<Index_type> hostBinAssignment(Size_type len, Index_type num_bins,
                                          RunParams::BinAssignmentAlgorithm algo);

// Host <-> device copies (synchronous).
void copyToDevice(void* d, const void* h, Size_type nbytes);
void copyToHost(void* h, const void* d, Size_type nbytes);
void copyDeviceToDevice(void* dst, const void* src, Size_type nbytes);
void zeroDeviceBytes(void* d, Size_type nbytes);

// The suite's checksum of a device array.
long double calcChecksumDevice(const Real_type* d, Size_type len,
                               Real_type scale_factor);
long double calcChecksumDevice(const Index_type* d, Size_type len,
                               Real_type scale_factor);
long double calcChecksumDevice(const Int_type* d, Size_type len, Real_type scale_factor);
// ... and of host data.
long double calcChecksumHost(const Real_type* h, Size_type len,
                             Real_type scale_factor);
long double calcChecksumHost(const long long* h, Size_type len,
                             Real_type scale_factor);
long double calcChecksumHost(const unsigned long long* h, Size_type len,
                             Real_type scale_factor);

// Counter-based uniform value of the uniform input mode (identical to the
// device generator b200_init_uniform).
double uniformValue(unsigned long long seed, unsigned long long stream,
                    unsigned long long i, double lo, double hi);

// Throws std::runtime_error carrying b200_last_error_string() when a
// library call failed.
void checkB200(int status, const char* what);
// Throws on a CUDA runtime error.
void checkCuda(int cuda_error, const char* what);

}  // namespace rajaperf
