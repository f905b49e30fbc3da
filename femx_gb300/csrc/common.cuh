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
  kDevStageTimeout      = 12,
};

__device__ inline void devFail(DeviceStatus* st, int code, int index)
{
  if (atomicCAS(&st->code, 0, code) == 0)
  {
    st->index = index;
  }
}

const char* deviceErrorMessage(int code);

// One-dimensional bulk copy global -> shared memory by the tensor memory
// accelerator (cp.async.bulk), its completion counted in bytes on an
// mbarrier. Call from every thread of the block: thread 0 initialises the
// barrier and issues the copy; all threads wait for the barrier's phase 0.
// dst and src 16-byte aligned, bytes a multiple of 16. The wait is bounded
// (try_wait suspends for a hardware time slice per attempt); it returns
// false if the copy has not landed after kStageSpin attempts, and the
// caller reports that through its status word.
constexpr int kStageSpin = 1 << 20;

__device__ __forceinline__ bool bulkStage(void* dst, const void* src, unsigned bytes,
                                          unsigned long long* bar)
{
  const unsigned b = static_cast<unsigned>(__cvta_generic_to_shared(bar));
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  if (threadIdx.x == 0)
  {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], "
                 "%2, [%3];" ::"r"(d),
                 "l"(src), "r"(bytes), "r"(b)
                 : "memory");
  }
  __syncthreads();
  unsigned done = 0;
  for (int it = 0; it < kStageSpin && done == 0; ++it)
  {
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(b)
                 : "memory");
  }
  return done != 0;
}

// Programmatic dependent launch (sm_90+). zeroForNext() clears the output
// arrays of the assembly that follows it on the stream, in a kernel that
// lets that assembly launch at once (griddepcontrol.launch_dependents); the
// assembly, launched by launchDependent(), loads and computes its first
// elements while the zeros are written and calls awaitPrerequisites()
// (griddepcontrol.wait: returns once the zero kernel has completed and its
// stores are visible) before its first global reduction. In a kernel that
// was not launched as a dependent, the wait returns at once. The zero kernel
// itself waits for all earlier work on the stream, as any launch does.
__device__ __forceinline__ void awaitPrerequisites()
{
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// a[0..na) = 0 and b[0..nb) = 0 (either may be empty), as a dependent-launch
// primary.
void zeroForNext(double* a, long long na, double* b, long long nb, cudaStream_t s);

// A second stream owned by the calling host thread, with its own events,
// for work that runs beside the caller's stream inside one library call
// (fork: event on the caller's stream, side stream waits; join: the
// reverse). Created on the thread's first use (setup); later calls
// allocate nothing. Fork/join through events is CUDA-graph capturable.
struct SideStream
{
  static constexpr int kEvents = 8;
  int                  dev     = -1;
  cudaStream_t         s       = nullptr;
  cudaEvent_t          ev[kEvents]{};
  void                 release();
  void                 ensure();
  ~SideStream() { release(); }
};
SideStream& sideStream(); // this thread's, ensured for the current device

// A launch as a dependent (dependent = true) or an ordinary one, with
// `smem` bytes of dynamic shared memory.
template <class... P, class... A>
void launchMaybeDependentSmem(bool dependent, void (*kernel)(P...), unsigned grid,
                              unsigned block, unsigned smem, cudaStream_t s, A&&... args)
{
  cudaLaunchConfig_t  cfg{};
  cudaLaunchAttribute attr[1];
  attr[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.gridDim                                        = dim3(grid);
  cfg.blockDim                                       = dim3(block);
  cfg.dynamicSmemBytes                               = smem;
  cfg.stream                                         = s;
  cfg.attrs                                          = attr;
  cfg.numAttrs                                       = dependent ? 1 : 0;
  cudaCheck(cudaLaunchKernelEx(&cfg, kernel, static_cast<A&&>(args)...), "kernel launch");
}

template <class... P, class... A>
void launchMaybeDependent(bool dependent, void (*kernel)(P...), unsigned grid, unsigned block,
                          cudaStream_t s, A&&... args)
{
  launchMaybeDependentSmem(dependent, kernel, grid, block, 0u, s, static_cast<A&&>(args)...);
}

template <class... P, class... A>
void launchDependent(void (*kernel)(P...), unsigned grid, unsigned block, cudaStream_t s,
                     A&&... args)
{
  launchMaybeDependent(true, kernel, grid, block, s, static_cast<A&&>(args)...);
}

// Checks the device status word after a synchronize; throws on failure.
void checkDeviceStatus(DeviceStatus* d_status, cudaStream_t stream);

// Exclusive scan of n int32 counts into out[0..n] (out[n] = total); returns
// the total as int64 (read back; setup only). Fails if the total overflows
// the femx Index range (int32), like AssemblyMap's checkedAdd.
long long exclusiveScan(const int* in, int* out, long long n, cudaStream_t s);

// Same for int64 counts (element Jacobian sizes) written as int32 offsets.
long long exclusiveScan64to32(const long long* in, int* out, long long n,
                              cudaStream_t s);

// Rare-path hardware conversions, kept out of line so the compiler branches
// around them instead of predicating them into every conversion (they issue
// on the FP64 pipe).
static __device__ __noinline__ double f32ToF64Slow(float f)
{
  return static_cast<double>(f);
}
static __device__ __noinline__ float f64ToF32Slow(double d)
{
  return __double2float_rn(d);
}

// Exact float -> double conversion from the IEEE-754 fields, on the integer
// pipe. On GB300 the hardware conversion issues on the FP64 pipe (the scarce
// one), so kernels whose element math runs in FP32 convert with this.
// Normal numbers and zeros take the integer path; subnormal, infinite and NaN
// inputs (absent from FE data) fall back to the hardware conversion.
__device__ __forceinline__ double f32ToF64(float f)
{
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if ((u & 0x7fffffffu) == 0u)
  {
    return __longlong_as_double(static_cast<long long>(u & 0x80000000u) << 32);
  }
  if (e - 1u >= 0xfeu)
  {
    return f32ToF64Slow(f);
  }
  const unsigned long long bits =
      (static_cast<unsigned long long>(u & 0x80000000u) << 32)
      | (static_cast<unsigned long long>(e + 896u) << 52)
      | (static_cast<unsigned long long>(u & 0x7fffffu) << 29);
  return __longlong_as_double(static_cast<long long>(bits));
}

// Branch-free float -> double for the Jacobian scatter loops: exact for
// zeros, normal numbers, infinities and NaNs; a subnormal float (magnitude
// below 2^-126, only reachable by underflow in the FP32 element math) becomes
// a zero of the same sign. Seven integer operations and no call, against the
// two branches and the out-of-line fallback of f32ToF64.
__device__ __forceinline__ double f32ToF64Ftz(float f)
{
  const unsigned u    = __float_as_uint(f);
  const unsigned m    = u & 0x7fffffffu;
  const unsigned bias = m >= 0x7f800000u ? 0x70000000u : 0x38000000u; // exponent 896 or 2047
  const bool     norm = m >= 0x00800000u;
  const unsigned hi   = (norm ? (m >> 3) + bias : 0u) | (u & 0x80000000u);
  const unsigned lo   = norm ? (u << 29) : 0u;
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
}

// double -> float with round-to-nearest-even, from the IEEE-754 fields on
// the integer pipe (same reason as above). Values whose float result is
// normal take the integer path; zeros are exact; anything that would be
// subnormal, infinite or NaN uses the hardware conversion.
__device__ __forceinline__ float f64ToF32(double d)
{
  const unsigned long long b  = static_cast<unsigned long long>(__double_as_longlong(d));
  const unsigned           hi = static_cast<unsigned>(b >> 32);
  const unsigned           lo = static_cast<unsigned>(b);
  const unsigned           s  = hi & 0x80000000u;
  const int                fe = static_cast<int>((hi >> 20) & 0x7ffu) - 1023 + 127;
  if ((b << 1) == 0ull)
  {
    return __uint_as_float(s);
  }
  if (fe <= 0 || fe >= 255)
  {
    return f64ToF32Slow(d);
  }
  const unsigned m    = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rem  = lo & 0x1fffffffu;
  const unsigned half = 0x10000000u;
  unsigned       r    = s | (static_cast<unsigned>(fe) << 23) | m;
  r += (rem > half || (rem == half && (m & 1u))) ? 1u : 0u; // carry may round up to inf
  return __uint_as_float(r);
}

// 1/x in FP64 by Newton-Raphson refinement of a single-precision seed: each
// step r <- r + r (1 - x r) squares the relative error, so the seed's 2^-22
// becomes 2^-44 and then falls below double rounding; the result is within
// two ulps of the correctly rounded reciprocal. Four FP64 FMAs replace the
// division sequence (GB300's FP64 pipe is the scarce one). |x| outside
// [2^-120, 2^120] (the seed would leave the float range) takes the division.
__device__ __forceinline__ double rcpF64(double x)
{
  const unsigned e = (static_cast<unsigned>(__double2hiint(x)) >> 20) & 0x7ffu;
  if (e - (1023u - 120u) > 240u)
  {
    return 1.0 / x;
  }
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(f64ToF32(x)));
  double r = f32ToF64(r0);
  double d = fma(-x, r, 1.0);
  r        = fma(r, d, r);
  d        = fma(-x, r, 1.0);
  return fma(r, d, r);
}

// 1/sqrt(x) in FP64 by the same scheme: a single-precision seed and two
// Newton-Raphson steps y <- y + (y/2)(1 - x y^2) (quadratic convergence),
// within two ulps of the correctly rounded value. x outside [2^-120, 2^120]
// (including 0) takes 1 / sqrt(x).
__device__ __forceinline__ double rsqrtF64(double x)
{
  const unsigned e = (static_cast<unsigned>(__double2hiint(x)) >> 20) & 0x7ffu;
  if (e - (1023u - 120u) > 240u || __double2hiint(x) < 0)
  {
    return 1.0 / sqrt(x);
  }
  float y0;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(f64ToF32(x)));
  double y = f32ToF64(y0);
#pragma unroll
  for (int i = 0; i < 2; ++i)
  {
    const double d = fma(-x * y, y, 1.0);
    y              = fma(0.5 * y, d, y);
  }
  return y;
}

template <class T>
__device__ __forceinline__ T fromF64(double d);
template <>
__device__ __forceinline__ double fromF64<double>(double d)
{
  return d;
}
template <>
__device__ __forceinline__ float fromF64<float>(double d)
{
  return f64ToF32(d);
}
__device__ __forceinline__ double toF64(double d)
{
  return d;
}
__device__ __forceinline__ double toF64(float f)
{
  return f32ToF64(f);
}
__device__ __forceinline__ double toF64Ftz(double d)
{
  return d;
}
__device__ __forceinline__ double toF64Ftz(float f)
{
  return f32ToF64Ftz(f);
}

// FP64 reduction-add at L2 without a return value.
__device__ __forceinline__ void redAdd(double* addr, double v)
{
  asm volatile("red.global.add.f64 [%0], %1;" ::"l"(addr), "d"(v) : "memory");
}

// Adds v into *addr: an FP64 reduction at L2, or, in coloured assembly
// (kPlain: no other thread of the launch touches addr), a plain
// read-add-write.
template <bool kPlain>
__device__ __forceinline__ void addTo(double* addr, double v)
{
  if constexpr (kPlain)
  {
    *addr += v;
  }
  else
  {
    redAdd(addr, v);
  }
}

} // namespace gbfem
