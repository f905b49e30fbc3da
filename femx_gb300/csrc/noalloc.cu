// noalloc.cu — Dirichlet forward-solve preparation for callers that cannot
// allocate device memory.
//
// gbfem_prepare_forward_solve needs a BoundaryMap handle, and building one
// calls cudaMalloc. Some callers cannot do that: code that runs while another
// allocator owns the device memory (for example a PyTorch process whose
// caching allocator has reserved it), or a real-time solver loop that must not
// pay for allocation or risk fragmentation. This entry point does the same
// work — femx's makeBoundaryMap + prepareForwardSolve
// (femx/assembly/BoundaryMap.cpp:59-139, 218-247) — straight from the DOF
// list and the CSR pattern, with its scratch in one fixed-size array that the
// library owns from the moment it is loaded:
//
//   g_noalloc_scratch — a file-scope static __device__ array of
//   kNoAllocScratchWords 32-bit words (8 MiB + 256 B). It holds a status word
//   and one column -> constraint slot per matrix row, so the call accepts at
//   most GBFEM_NOALLOC_MAX_ROWS (2,097,152) rows. Every GPU that loads the
//   library keeps this array until the process exits.
//
// The array is shared by every call. A call leaves it cleared (all zero)
// when it returns, so the next call starts from a clean state; two calls
// whose kernels overlap on the GPU (different streams, no ordering between
// them) would race on it, so callers must order them.
#include <mutex>

#include "common.cuh"

namespace
{
using gbfem::DeviceStatus;

constexpr long long kStatusWords       = 64; // status word, padded to 256 B
constexpr long long kNoAllocScratchWords = kStatusWords + GBFEM_NOALLOC_MAX_ROWS;

// Word 0..1: DeviceStatus; words kStatusWords.. : constraint slot + 1 of
// each column (0 = unconstrained). Zero-initialised at module load.
static __device__ __align__(256) int g_noalloc_scratch[kNoAllocScratchWords];

// Host code cannot use the array's name as a device address; the address is
// looked up once per device, with that device current. A device reset
// (cudaDeviceReset) unloads the module and makes the cached address stale,
// so the entry point must not be used after one in the same process.
//
// g_dirty[dev] is set while a call has constraint slots marked in the array
// and cleared once the call has enqueued their clearing. If a call throws in
// between (a failed launch, copy or synchronisation), the next call on that
// device clears the whole array before it uses it.
constexpr int kMaxDevices = 64;
std::mutex    g_addr_mutex;
int*          g_addr[kMaxDevices]  = {};
bool          g_dirty[kMaxDevices] = {};

int* scratchAddress(int* dev_out)
{
  int dev = 0;
  gbfem::cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
  gbfem::require(dev >= 0 && dev < kMaxDevices, "device index out of range");
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  if (g_addr[dev] == nullptr)
  {
    void* p = nullptr;
    gbfem::cudaCheck(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                     "cudaGetSymbolAddress(no-allocation scratch)");
    g_addr[dev] = static_cast<int*>(p);
  }
  *dev_out = dev;
  return g_addr[dev];
}

bool takeDirty(int dev)
{
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  const bool d = g_dirty[dev];
  g_dirty[dev] = false;
  return d;
}

void setDirty(int dev, bool d)
{
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  g_dirty[dev] = d;
}

__global__ void naValidatePattern(int rows, int cols, const int* __restrict__ row_ptr,
                                  const int* __restrict__ col_ind, DeviceStatus* st)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows)
  {
    return;
  }
  const int k0 = row_ptr[r], k1 = row_ptr[r + 1];
  if (k1 < k0 || (r == 0 && k0 != 0))
  {
    gbfem::devFail(st, gbfem::kDevPatternInvalid, r);
    return;
  }
  for (int k = k0; k < k1; ++k)
  {
    if (col_ind[k] < 0 || col_ind[k] >= cols)
    {
      gbfem::devFail(st, gbfem::kDevPatternInvalid, r);
      return;
    }
  }
}

// Marks constrained columns with slot + 1; rejects out-of-range and repeated
// DOFs (BoundaryMap.cpp:73-81).
__global__ void naMark(int nb, int rows, const int* __restrict__ dofs,
                       int* __restrict__ slot, DeviceStatus* st)
{
  const int ib = blockIdx.x * blockDim.x + threadIdx.x;
  if (ib >= nb)
  {
    return;
  }
  const int dof = dofs[ib];
  if (dof < 0 || dof >= rows)
  {
    gbfem::devFail(st, gbfem::kDevBcRange, ib);
    return;
  }
  if (atomicCAS(&slot[dof], 0, ib + 1) != 0)
  {
    gbfem::devFail(st, gbfem::kDevBcDuplicate, ib);
  }
}

// Every constrained row needs exactly one diagonal entry (BoundaryMap.cpp:
// 91-110).
__global__ void naCheckDiag(int nb, int rows, const int* __restrict__ dofs,
                            const int* __restrict__ row_ptr,
                            const int* __restrict__ col_ind, DeviceStatus* st)
{
  const int ib = blockIdx.x * blockDim.x + threadIdx.x;
  if (ib >= nb)
  {
    return;
  }
  const int r = dofs[ib];
  if (r < 0 || r >= rows)
  {
    return; // already flagged by naMark
  }
  int       n = 0;
  for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
  {
    n += col_ind[k] == r ? 1 : 0;
  }
  if (n == 0)
  {
    gbfem::devFail(st, gbfem::kDevBcNoDiag, ib);
  }
  else if (n > 1)
  {
    gbfem::devFail(st, gbfem::kDevBcDupDiag, ib);
  }
}

// One thread per row. Unconstrained rows subtract A[r][c] g_c for their
// constrained columns in constraint order with separate multiply and
// subtract roundings (the CPU loop's order, BoundaryMap.cpp:224-238) and
// zero those entries; constrained rows become identity rows with rhs = g.
// The entries are taken in (constraint slot, CSR position) order, so a row
// that holds the same constrained column twice (femx's CsrPattern does not
// forbid repeated columns) subtracts and zeroes both, as femx's column list
// does (BoundaryMap.cpp:113-124 lists every matching entry in row order).
__global__ void naApply(int rows, const int* __restrict__ row_ptr,
                        const int* __restrict__ col_ind, const int* __restrict__ slot,
                        double* __restrict__ vals, double* __restrict__ rhs,
                        const double* __restrict__ g)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows)
  {
    return;
  }
  const int k0 = row_ptr[r], k1 = row_ptr[r + 1];
  const int own = slot[r];
  if (own != 0)
  {
    for (int k = k0; k < k1; ++k)
    {
      vals[k] = col_ind[k] == r ? 1.0 : 0.0;
    }
    rhs[r] = g[own - 1];
    return;
  }
  double acc   = 0.0;
  bool   any   = false;
  int    last  = 0;  // slots are 1-based; 0 = before the first constraint
  int    lastk = -1; // CSR position of the entry applied last
  for (;;)
  {
    // Next entry after (last, lastk) in (slot, k) order. k ascends in the
    // scan, so the first entry met with the smallest qualifying slot is the
    // one with the smallest k.
    int best = 0x7fffffff, bk = -1;
    for (int k = k0; k < k1; ++k)
    {
      const int sl = slot[col_ind[k]];
      if (sl != 0 && (sl > last || (sl == last && k > lastk)) && sl < best)
      {
        best = sl;
        bk   = k;
      }
    }
    if (bk < 0)
    {
      break;
    }
    if (!any)
    {
      acc = rhs[r];
      any = true;
    }
    acc      = __dsub_rn(acc, __dmul_rn(vals[bk], g[best - 1]));
    vals[bk] = 0.0;
    last     = best;
    lastk    = bk;
  }
  if (any)
  {
    rhs[r] = acc;
  }
}

__global__ void naClear(int nb, const int* __restrict__ dofs, int rows,
                        int* __restrict__ slot)
{
  const int ib = blockIdx.x * blockDim.x + threadIdx.x;
  if (ib < nb)
  {
    const int dof = dofs[ib];
    if (dof >= 0 && dof < rows)
    {
      slot[dof] = 0;
    }
  }
}

} // namespace

extern "C" int gbfem_prepare_forward_solve_noalloc(int num_bcs, const int* dofs, int rows,
                                                    const int* row_ptr, const int* col_ind,
                                                    double* vals, double* rhs,
                                                    const double* bc_vals, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(num_bcs >= 0 && rows >= 0, "BoundaryMap sizes must be non-negative");
    require(rows <= GBFEM_NOALLOC_MAX_ROWS,
            "rows exceed the no-allocation scratch capacity (2097152 rows)");
    require(num_bcs == 0 || (dofs != nullptr && bc_vals != nullptr),
            "BoundaryMap DOF list is null");
    require(rows == 0 || (row_ptr && col_ind && vals && rhs), "BoundaryMap pattern is null");
    require(rhs != bc_vals, "BoundaryMap RHS and prescribed values must not alias");
    require(static_cast<const void*>(rhs) != vals
                && static_cast<const void*>(bc_vals) != vals,
            "BoundaryMap vectors must not alias matrix values");
    if (num_bcs == 0 || rows == 0)
    {
      return;
    }
    cudaStream_t   s = asStream(stream);
    int            dev    = 0;
    int*           base   = scratchAddress(&dev);
    auto*          status = reinterpret_cast<DeviceStatus*>(base);
    int*           slot   = base + kStatusWords;
    const unsigned rb     = blocksFor(rows, 256);
    const unsigned bb     = blocksFor(num_bcs, 256);

    if (takeDirty(dev))
    {
      // An earlier call failed with slots marked: start from a zero array.
      setDirty(dev, true);
      cudaCheck(cudaMemsetAsync(base, 0, sizeof(int) * kNoAllocScratchWords, s),
                "scratch reset");
      setDirty(dev, false);
    }
    cudaCheck(cudaMemsetAsync(status, 0, sizeof(DeviceStatus), s), "status reset");
    naValidatePattern<<<rb, 256, 0, s>>>(rows, rows, row_ptr, col_ind, status);
    cudaCheck(cudaGetLastError(), "pattern check launch");
    DeviceStatus h{0, 0};
    cudaCheck(cudaMemcpyAsync(&h, status, sizeof(h), cudaMemcpyDeviceToHost, s),
              "status readback");
    cudaCheck(cudaStreamSynchronize(s), "pattern check");
    if (h.code != kDevOk)
    {
      cudaCheck(cudaMemsetAsync(status, 0, sizeof(DeviceStatus), s), "status reset");
      cudaCheck(cudaStreamSynchronize(s), "status reset");
      throw Error(GBFEM_EDATA, deviceErrorMessage(h.code));
    }

    setDirty(dev, true);
    naMark<<<bb, 256, 0, s>>>(num_bcs, rows, dofs, slot, status);
    cudaCheck(cudaGetLastError(), "constraint mark launch");
    naCheckDiag<<<bb, 256, 0, s>>>(num_bcs, rows, dofs, row_ptr, col_ind, status);
    cudaCheck(cudaGetLastError(), "diagonal check launch");
    cudaCheck(cudaMemcpyAsync(&h, status, sizeof(h), cudaMemcpyDeviceToHost, s),
              "status readback");
    cudaCheck(cudaStreamSynchronize(s), "constraint check");
    if (h.code == kDevOk)
    {
      naApply<<<rb, 256, 0, s>>>(rows, row_ptr, col_ind, slot, vals, rhs, bc_vals);
      cudaCheck(cudaGetLastError(), "forward-solve launch");
    }
    // Leave the shared scratch cleared for the next call, on success or not.
    naClear<<<bb, 256, 0, s>>>(num_bcs, dofs, rows, slot);
    cudaCheck(cudaGetLastError(), "scratch clear launch");
    cudaCheck(cudaMemsetAsync(status, 0, sizeof(DeviceStatus), s), "status reset");
    setDirty(dev, false);
    if (h.code != kDevOk)
    {
      cudaCheck(cudaStreamSynchronize(s), "scratch clear");
      throw Error(GBFEM_EDATA, deviceErrorMessage(h.code));
    }
  });
}
