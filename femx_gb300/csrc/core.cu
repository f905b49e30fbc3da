// core.cu — error plumbing, device status checks and the setup-time scan.
#include <algorithm>
#include <climits>
#include <cstdint>
#include <string>
#include <vector>

#include "common.cuh"

namespace gbfem
{

namespace
{
thread_local std::string g_last_error;

constexpr int kScanThreads = 1024;
constexpr int kScanItems   = 4;
constexpr int kScanTile    = kScanThreads * kScanItems;

// Exclusive scan of one tile per block; block totals go to `sums`.
__global__ void scanTiles(long long* d, long long n, long long* sums)
{
  __shared__ long long warp_tot[kScanThreads / 32];
  const long long base = static_cast<long long>(blockIdx.x) * kScanTile
                         + static_cast<long long>(threadIdx.x) * kScanItems;
  long long v[kScanItems];
  long long local = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
  {
    const long long idx = base + i;
    v[i]                = idx < n ? d[idx] : 0;
    local += v[i];
  }
  // inclusive warp scan of per-thread totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long incl = local;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1)
  {
    const long long t = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off)
    {
      incl += t;
    }
  }
  if (lane == 31)
  {
    warp_tot[warp] = incl;
  }
  __syncthreads();
  if (warp == 0)
  {
    long long w  = warp_tot[lane];
    long long wi = w;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1)
    {
      const long long t = __shfl_up_sync(0xffffffffu, wi, off);
      if (lane >= off)
      {
        wi += t;
      }
    }
    warp_tot[lane] = wi - w; // exclusive warp offsets
    if (lane == 31)
    {
      sums[blockIdx.x] = wi;
    }
  }
  __syncthreads();
  long long run = warp_tot[warp] + incl - local;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
  {
    const long long idx = base + i;
    if (idx < n)
    {
      d[idx] = run;
    }
    run += v[i];
  }
}

__global__ void addTileOffsets(long long* d, long long n, const long long* offs)
{
  const long long base = static_cast<long long>(blockIdx.x) * kScanTile;
  const long long add  = offs[blockIdx.x];
  for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
  {
    const long long idx = base + i;
    if (idx < n)
    {
      d[idx] += add;
    }
  }
}

// Exclusive in-place scan; the grand total is written to *total.
void scanInPlace(long long* d, long long n, long long* total, cudaStream_t s)
{
  const long long tiles = (n + kScanTile - 1) / kScanTile;
  long long*      sums  = deviceAlloc<long long>(tiles + 1);
  try
  {
    scanTiles<<<static_cast<unsigned>(tiles), kScanThreads, 0, s>>>(d, n, sums);
    cudaCheck(cudaGetLastError(), "scan launch");
    if (tiles > 1)
    {
      scanInPlace(sums, tiles, total, s);
      addTileOffsets<<<static_cast<unsigned>(tiles), 256, 0, s>>>(d, n, sums);
      cudaCheck(cudaGetLastError(), "scan offsets launch");
    }
    else
    {
      cudaCheck(cudaMemcpyAsync(total, sums, sizeof(long long),
                                cudaMemcpyDeviceToDevice, s),
                "scan total copy");
    }
    cudaCheck(cudaStreamSynchronize(s), "scan");
  }
  catch (...)
  {
    deviceFree(sums);
    throw;
  }
  deviceFree(sums);
}

template <class T>
__global__ void widen(const T* in, long long* out, long long n)
{
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < n)
  {
    out[i] = static_cast<long long>(in[i]);
  }
}

__global__ void narrow(const long long* in, int* out, long long n,
                       const long long* total)
{
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < n)
  {
    out[i] = static_cast<int>(in[i]);
  }
  else if (i == n)
  {
    out[n] = static_cast<int>(*total);
  }
}

template <class T>
long long scanTo32(const T* in, int* out, long long n, cudaStream_t s)
{
  long long* tmp = deviceAlloc<long long>(n + 1);
  long long  total_h = 0;
  try
  {
    if (n > 0)
    {
      widen<<<blocksFor(n, 256), 256, 0, s>>>(in, tmp, n);
      cudaCheck(cudaGetLastError(), "scan widen launch");
      scanInPlace(tmp, n, tmp + n, s);
      cudaCheck(cudaMemcpy(&total_h, tmp + n, sizeof(long long),
                           cudaMemcpyDeviceToHost),
                "scan total readback");
    }
    if (total_h > INT_MAX)
    {
      throw Error(GBFEM_EINVAL,
                  "AssemblyMap flattened data exceeds the Index range");
    }
    if (n > 0)
    {
      narrow<<<blocksFor(n + 1, 256), 256, 0, s>>>(tmp, out, n, tmp + n);
      cudaCheck(cudaGetLastError(), "scan narrow launch");
    }
    else
    {
      cudaCheck(cudaMemsetAsync(out, 0, sizeof(int), s), "scan memset");
    }
    cudaCheck(cudaStreamSynchronize(s), "scan narrow");
  }
  catch (...)
  {
    deviceFree(tmp);
    throw;
  }
  deviceFree(tmp);
  return total_h;
}

__device__ void zeroRange(double* p, long long n, long long tid, long long nt)
{
  if (n <= 0)
  {
    return;
  }
  // one leading double when p is not 16-byte aligned, then pairs, then a tail
  const long long head = (reinterpret_cast<std::uintptr_t>(p) & 15u) != 0 ? 1 : 0;
  const long long m    = n - head;
  if (tid == 0)
  {
    if (head != 0)
    {
      p[0] = 0.0;
    }
    if ((m & 1) != 0)
    {
      p[n - 1] = 0.0;
    }
  }
  // Descending: the grid's last writes are the lowest addresses, where the
  // dependent element kernel, walking its elements in order, adds first;
  // those lines are then still in L2 when its reductions reach them.
  double2*        q  = reinterpret_cast<double2*>(p + head);
  const long long np = m / 2;
  for (long long i = np - 1 - tid; i >= 0; i -= nt)
  {
    q[i] = make_double2(0.0, 0.0);
  }
}

__global__ void __launch_bounds__(256) zeroForNextKernel(double* a, long long na, double* b,
                                                          long long nb)
{
  asm volatile("griddepcontrol.launch_dependents;");
  const long long tid = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  const long long nt  = static_cast<long long>(gridDim.x) * blockDim.x;
  zeroRange(b, nb, tid, nt); // the (small) residual first, the matrix values last
  zeroRange(a, na, tid, nt);
}

int smCount()
{
  thread_local int dev = -1, count = 0;
  int              d   = 0;
  cudaCheck(cudaGetDevice(&d), "cudaGetDevice");
  if (d != dev)
  {
    cudaCheck(cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, d),
              "SM count");
    dev = d;
  }
  return count;
}

} // namespace

void SideStream::release()
{
  for (cudaEvent_t& e : ev)
  {
    if (e != nullptr)
    {
      cudaEventDestroy(e);
      e = nullptr;
    }
  }
  if (s != nullptr)
  {
    cudaStreamDestroy(s);
    s = nullptr;
  }
  dev = -1;
}

void SideStream::ensure()
{
  int d = 0;
  cudaCheck(cudaGetDevice(&d), "cudaGetDevice");
  if (d == dev)
  {
    return;
  }
  release();
  cudaCheck(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "side stream");
  for (cudaEvent_t& e : ev)
  {
    cudaCheck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "side event");
  }
  dev = d;
}

SideStream& sideStream()
{
  thread_local SideStream side;
  side.ensure();
  return side;
}

void zeroForNext(double* a, long long na, double* b, long long nb, cudaStream_t s)
{
  if (na <= 0 && nb <= 0)
  {
    return;
  }
  // two 256-thread blocks per SM: all resident at once, so that every block
  // has signalled the dependent launch early, and room is left on each SM
  // for the dependent assembly's blocks
  const long long pairs = (std::max(na, 0LL) + std::max(nb, 0LL)) / 2 + 1;
  const unsigned  grid  = std::min<unsigned>(2u * smCount(), blocksFor(pairs, 256));
  zeroForNextKernel<<<grid, 256, 0, s>>>(a, na > 0 ? na : 0, b, nb > 0 ? nb : 0);
  cudaCheck(cudaGetLastError(), "zero-fill launch");
}

void setLastError(const std::string& msg)
{
  g_last_error = msg;
}

const char* deviceErrorMessage(int code)
{
  switch (code)
  {
  case kDevResDofRange:
    return "AssemblyMap residual DOF is out of range";
  case kDevStateDofRange:
    return "AssemblyMap state DOF is out of range";
  case kDevNegativeLocal:
    return "AssemblyMap local dimensions must be non-negative";
  case kDevBcRange:
    return "BoundaryMap constrained DOF is out of range";
  case kDevBcDuplicate:
    return "BoundaryMap constrained DOFs must be unique";
  case kDevBcNoDiag:
    return "BoundaryMap constrained row has no diagonal entry";
  case kDevBcDupDiag:
    return "BoundaryMap constrained row has duplicate diagonal entries";
  case kDevSingularJacobian:
    return "Singular 2D Jacobian.";
  case kDevRowOverflow:
    return "AssemblyMap row exceeds the supported candidate count";
  case kDevPatternInvalid:
    return "CSR pattern row pointers or column indices are invalid";
  case kDevNodeRange:
    return "Geometry element connectivity is out of range";
  case kDevStageTimeout:
    return "Staging the reference tables in shared memory timed out";
  default:
    return "unknown device error";
  }
}

void checkDeviceStatus(DeviceStatus* d_status, cudaStream_t stream)
{
  DeviceStatus h{0, 0};
  cudaCheck(cudaMemcpyAsync(&h, d_status, sizeof(h), cudaMemcpyDeviceToHost,
                            stream),
            "status readback");
  cudaCheck(cudaStreamSynchronize(stream), "status sync");
  if (h.code != kDevOk)
  {
    throw Error(GBFEM_EDATA, std::string(deviceErrorMessage(h.code))
                                 + " (index " + std::to_string(h.index) + ")");
  }
}

long long exclusiveScan(const int* in, int* out, long long n, cudaStream_t s)
{
  return scanTo32(in, out, n, s);
}

long long exclusiveScan64to32(const long long* in, int* out, long long n,
                              cudaStream_t s)
{
  return scanTo32(in, out, n, s);
}

} // namespace gbfem

extern "C" {

const char* gbfem_last_error(void)
{
  return gbfem::g_last_error.c_str();
}

int gbfem_version(void)
{
  return 1;
}

} // extern "C"
