// common.cuh — shared host/device plumbing for libgbfem.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include "gbfem.h"

namespace gbfem
{

// Thrown inside the library; every extern "C" entry point converts it into a
// status code plus the thread-local message returned by gbfem_last_error().
struct Error : std::runtime_error
{
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void setLastError(const std::string& msg);

inline void require(bool cond, const char* msg, int code = GBFEM_EINVAL)
{
  if (!cond)
  {
    throw Error(code, msg);
  }
}

inline void cudaCheck(cudaError_t err, const char* what)
{
  if (err != cudaSuccess)
  {
    throw Error(GBFEM_ECUDA, std::string(what) + ": " + cudaGetErrorString(err));
  }
}

template <class F>
int guarded(F&& fn)
{
  try
  {
    fn();
    return GBFEM_OK;
  }
  catch (const Error& e)
  {
    setLastError(e.what());
    return e.code;
  }
  catch (const std::bad_alloc&)
  {
    setLastError("host allocation failed");
    return GBFEM_ENOMEM;
  }
  catch (const std::exception& e)
  {
    setLastError(e.what());
    return GBFEM_EINVAL;
  }
}

inline cudaStream_t asStream(void* s)
{
  return static_cast<cudaStream_t>(s);
}

inline unsigned blocksFor(long long n, int threads)
{
  const long long b = (n + threads - 1) / threads;
  return static_cast<unsigned>(b > 0 ? b : 1);
}

// Device allocation owned by a handle; setup-time only (never on hot calls).
template <class T>
T* deviceAlloc(long long n)
{
  void* p = nullptr;
  if (n <= 0)
  {
    return nullptr;
  }
  const cudaError_t err = cudaMalloc(&p, sizeof(T) * static_cast<size_t>(n));
  if (err != cudaSuccess)
  {
    throw Error(GBFEM_ENOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(err));
  }
  return static_cast<T*>(p);
}

inline void deviceFree(void* p)
{
  if (p != nullptr)
  {
    cudaFree(p);
  }
}

// Device-side validation: the first failing thread records (code, index);
// the host reads the record after the setup kernels (setup syncs anyway).
struct DeviceStatus
{
  int code;
  int index;
};

enum DeviceErr : int
{
  kDevOk                = 0,
  kDevResDofRange       = 1,
  kDevStateDofRange     = 2,
  kDevNegativeLocal     = 3,
  kDevBcRange           = 4,
  kDevBcDuplicate       = 5,
  kDevBcNoDiag          = 6,
  kDevBcDupDiag         = 7,
  kDevSingularJacobian  = 8,
  kDevRowOverflow       = 9,
  kDevPatternInvalid    = 10,
  kDevNodeRange         = 11,
};

__device__ inline void devFail(DeviceStatus* st, int code, int index)
{
  if (atomicCAS(&st->code, 0, code) == 0)
  {
    st->index = index;
  }
}

const char* deviceErrorMessage(int code);

// Checks the device status word after a synchronize; throws on failure.
void checkDeviceStatus(DeviceStatus* d_status, cudaStream_t stream);

// Exclusive scan of n int32 counts into out[0..n] (out[n] = total); returns
// the total as int64 (read back; setup only). Fails if the total overflows
// the femx Index range (int32), like AssemblyMap's checkedAdd.
long long exclusiveScan(const int* in, int* out, long long n, cudaStream_t s);

// Same for int64 counts (element Jacobian sizes) written as int32 offsets.
long long exclusiveScan64to32(const long long* in, int* out, long long n,
                              cudaStream_t s);

// FP64 reduction-add at L2 without a return value.
__device__ __forceinline__ void redAdd(double* addr, double v)
{
  asm volatile("red.global.add.f64 [%0], %1;" ::"l"(addr), "d"(v) : "memory");
}

} // namespace gbfem
