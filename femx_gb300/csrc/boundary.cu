// boundary.cu — GPU build of femx's BoundaryMap and the Dirichlet operations
// (femx/assembly/BoundaryMap.cpp:38-247, BoundaryMap.cu:16-211).
//
// Build: constrained DOFs are flagged per column; one thread per CSR row
// finds entries in constrained columns (counts, diagonals, and the
// per-row lifting counts); per-constraint buckets are filled by atomics and
// then ordered by CSR slot, which is the reference's row-ascending order.
//
// Lifting (prepareForwardSolve) uses a row-grouped list built here: one
// thread per unconstrained row touching constrained columns subtracts
// A[r][c] g_c in constraint order with separate multiply and subtract
// roundings, i.e. exactly the sequence of the CPU loop (BoundaryMap.cpp:
// 224-238), so rhs is bit-identical; no atomics are needed.
#include "maps.cuh"

namespace
{
using gbfem::DeviceStatus;

// femx's CsrPattern validates monotone row pointers and column ranges on
// construction (femx/linalg/CsrPattern.hpp:42-217); a caller-supplied
// pattern is checked here before any column index is used.
__global__ void validatePattern(int rows, int cols, const int* __restrict__ row_ptr,
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
    const int c = col_ind[k];
    if (c < 0 || c >= cols)
    {
      gbfem::devFail(st, gbfem::kDevPatternInvalid, r);
      return;
    }
  }
}

__global__ void flagConstraints(int nb, int rows, const int* __restrict__ dofs,
                                int* __restrict__ bc_by_col,
                                int* __restrict__ bc_rows,
                                int* __restrict__ bc_mask, DeviceStatus* st)
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
  if (atomicCAS(&bc_by_col[dof], -1, ib) != -1)
  {
    gbfem::devFail(st, gbfem::kDevBcDuplicate, ib);
    return;
  }
  bc_rows[ib]  = dof;
  bc_mask[dof] = 1;
}

__global__ void scanRows(int rows, const int* __restrict__ row_ptr,
                         const int* __restrict__ col_ind,
                         const int* __restrict__ bc_by_col,
                         const int* __restrict__ bc_mask,
                         int* __restrict__ col_count, int* __restrict__ diag,
                         int* __restrict__ lift_count, DeviceStatus* st)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows)
  {
    return;
  }
  int lifts = 0;
  for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
  {
    const int c  = col_ind[k];
    const int ib = bc_by_col[c];
    if (ib >= 0)
    {
      atomicAdd(&col_count[ib], 1);
      if (c == r && atomicCAS(&diag[ib], -1, k) != -1)
      {
        gbfem::devFail(st, gbfem::kDevBcDupDiag, ib);
      }
      ++lifts;
    }
  }
  lift_count[r] = bc_mask[r] == 0 ? lifts : 0;
}

__global__ void checkDiag(int nb, const int* __restrict__ bc_rows,
                          const int* __restrict__ row_ptr,
                          const int* __restrict__ diag,
                          int* __restrict__ row_begin,
                          int* __restrict__ row_end, DeviceStatus* st)
{
  const int ib = blockIdx.x * blockDim.x + threadIdx.x;
  if (ib >= nb)
  {
    return;
  }
  if (diag[ib] < 0)
  {
    gbfem::devFail(st, gbfem::kDevBcNoDiag, ib);
  }
  const int r   = bc_rows[ib];
  row_begin[ib] = row_ptr[r];
  row_end[ib]   = row_ptr[r + 1];
}

__global__ void bucketColumns(int rows, const int* __restrict__ row_ptr,
                              const int* __restrict__ col_ind,
                              const int* __restrict__ bc_by_col,
                              const int* __restrict__ col_offsets,
                              int* __restrict__ cursor, int* __restrict__ tmp_k,
                              int* __restrict__ tmp_r)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows)
  {
    return;
  }
  for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
  {
    const int ib = bc_by_col[col_ind[k]];
    if (ib >= 0)
    {
      const int slot = col_offsets[ib] + atomicAdd(&cursor[ib], 1);
      tmp_k[slot]    = k;
      tmp_r[slot]    = r;
    }
  }
}

// One warp per constraint: order its entries by CSR slot (all distinct).
__global__ void orderColumns(int nb, const int* __restrict__ col_offsets,
                             const int* __restrict__ tmp_k,
                             const int* __restrict__ tmp_r,
                             int* __restrict__ col_entries,
                             int* __restrict__ col_rows)
{
  const int lane = threadIdx.x & 31;
  const int ib   = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (ib >= nb)
  {
    return;
  }
  const int beg = col_offsets[ib], n = col_offsets[ib + 1] - beg;
  for (int i = lane; i < n; i += 32)
  {
    const int k    = tmp_k[beg + i];
    int       rank = 0;
    for (int j = 0; j < n; ++j)
    {
      rank += tmp_k[beg + j] < k ? 1 : 0;
    }
    col_entries[beg + rank] = k;
    col_rows[beg + rank]    = tmp_r[beg + i];
  }
}

__global__ void compactLiftRows(int rows, const int* __restrict__ lift_count,
                                const int* __restrict__ lift_off_all,
                                const int* __restrict__ row_rank,
                                int* __restrict__ lift_rows,
                                int* __restrict__ lift_offsets)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows)
  {
    return;
  }
  if (lift_count[r] > 0)
  {
    const int i     = row_rank[r];
    lift_rows[i]    = r;
    lift_offsets[i] = lift_off_all[r];
  }
}

// One thread per lifting row: collect (slot, constraint) pairs in slot
// order, then insertion-sort them by constraint index.
__global__ void fillLift(int nl, const int* __restrict__ lift_rows,
                         const int* __restrict__ lift_offsets,
                         const int* __restrict__ row_ptr,
                         const int* __restrict__ col_ind,
                         const int* __restrict__ bc_by_col,
                         int* __restrict__ lift_k, int* __restrict__ lift_ib)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nl)
  {
    return;
  }
  const int r   = lift_rows[t];
  const int beg = lift_offsets[t];
  int       n   = 0;
  for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
  {
    const int ib = bc_by_col[col_ind[k]];
    if (ib >= 0)
    {
      int pos = beg + n;
      while (pos > beg && lift_ib[pos - 1] > ib)
      {
        lift_ib[pos] = lift_ib[pos - 1];
        lift_k[pos]  = lift_k[pos - 1];
        --pos;
      }
      lift_ib[pos] = ib;
      lift_k[pos]  = k;
      ++n;
    }
  }
}

__global__ void flagPositive(int n, const int* __restrict__ in,
                             int* __restrict__ out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    out[i] = in[i] > 0 ? 1 : 0;
  }
}

// ---- hot-path kernels ------------------------------------------------------

// Sixteen lanes per constrained row: the row's entries are zeroed (and its
// diagonal set) by coalesced stores, instead of one thread walking the row.
constexpr int kRowLanes = 16;

__global__ void replaceRowsKernel(int nb, const int* __restrict__ row_begin,
                                  const int* __restrict__ row_end,
                                  const int* __restrict__ diag,
                                  double* __restrict__ vals, double d)
{
  const int t  = blockIdx.x * blockDim.x + threadIdx.x;
  const int ib = t / kRowLanes, j = t % kRowLanes;
  if (ib >= nb)
  {
    return;
  }
  // launched as a dependent of the assembly: the row extents are the map's
  // own (immutable) data; the values are the assembly's output
  const int kb = row_begin[ib], ke = row_end[ib], kd = diag[ib];
  gbfem::awaitPrerequisites();
  for (int k = kb + j; k < ke; k += kRowLanes)
  {
    vals[k] = k == kd ? d : 0.0;
  }
}

__global__ void replaceResKernel(int nb, const int* __restrict__ bc_rows,
                                 const double* __restrict__ state,
                                 const double* __restrict__ g,
                                 double* __restrict__ res)
{
  const int ib = blockIdx.x * blockDim.x + threadIdx.x;
  if (ib < nb)
  {
    const int r = bc_rows[ib];
    gbfem::awaitPrerequisites(); // state, values and residual come from earlier work
    res[r] = state[r] - g[ib];
  }
}

__global__ void zeroBoundaryKernel(int nb, const int* __restrict__ bc_rows,
                                   double* __restrict__ v)
{
  const int ib = blockIdx.x * blockDim.x + threadIdx.x;
  if (ib < nb)
  {
    v[bc_rows[ib]] = 0.0;
  }
}

// Fused forward-solve preparation: threads [0, nl) lift unconstrained rows,
// threads [nl, nl + nb) turn constrained rows into identity rows. The two
// sets of rows are disjoint, so one launch suffices.
__global__ void forwardSolveKernel(int nl, const int* __restrict__ lift_rows,
                                   const int* __restrict__ lift_offsets,
                                   const int* __restrict__ lift_k,
                                   const int* __restrict__ lift_ib, int nb,
                                   const int* __restrict__ bc_rows,
                                   const int* __restrict__ row_begin,
                                   const int* __restrict__ row_end,
                                   const int* __restrict__ diag,
                                   double* __restrict__ vals,
                                   double* __restrict__ rhs,
                                   const double* __restrict__ g)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nl)
  {
    const int r   = lift_rows[t];
    double    acc = rhs[r];
    for (int i = lift_offsets[t]; i < lift_offsets[t + 1]; ++i)
    {
      const int k = lift_k[i];
      acc         = __dsub_rn(acc, __dmul_rn(vals[k], g[lift_ib[i]]));
      vals[k]     = 0.0;
    }
    rhs[r] = acc;
  }
  else if (t < nl + nb)
  {
    const int ib = t - nl;
    for (int k = row_begin[ib]; k < row_end[ib]; ++k)
    {
      vals[k] = 0.0;
    }
    vals[diag[ib]]   = 1.0;
    rhs[bc_rows[ib]] = g[ib];
  }
}

struct Scratch
{
  void* p[10] = {};
  ~Scratch()
  {
    for (void* q : p)
    {
      gbfem::deviceFree(q);
    }
  }
};

} // namespace

gbfem_boundary_map::~gbfem_boundary_map()
{
  for (int* p : {bc_rows, diag, col_offsets, col_entries, col_rows, bc_mask,
                 row_begin, row_end, lift_rows, lift_offsets, lift_k, lift_ib})
  {
    gbfem::deviceFree(p);
  }
}

extern "C" int gbfem_boundary_map_create(int num_bcs, const int* dofs, int rows,
                                         int cols, const int* row_ptr,
                                         const int* col_ind,
                                         unsigned long long layout_id,
                                         void* stream, gbfem_boundary_map** out)
{
  using namespace gbfem;
  return guarded([&] {
    require(out != nullptr, "BoundaryMap output handle is null");
    *out = nullptr;
    require(rows == cols, "BoundaryMap requires a square CSR pattern");
    require(num_bcs >= 0 && rows >= 0, "BoundaryMap sizes must be non-negative");
    require(num_bcs == 0 || dofs != nullptr, "BoundaryMap DOF list is null");
    require(rows == 0 || (row_ptr != nullptr && (col_ind != nullptr)),
            "BoundaryMap pattern is null");
    cudaStream_t s = asStream(stream);
    auto*        b = new gbfem_boundary_map;
    try
    {
      b->num_rows  = rows;
      b->num_cols  = cols;
      b->num_bcs   = num_bcs;
      b->layout_id = layout_id;
      int nnz      = 0;
      if (rows > 0)
      {
        cudaCheck(cudaMemcpyAsync(&nnz, row_ptr + rows, sizeof(int),
                                  cudaMemcpyDeviceToHost, s),
                  "BoundaryMap nnz readback");
        cudaCheck(cudaStreamSynchronize(s), "BoundaryMap nnz readback");
      }
      b->nnz = nnz;

      b->bc_rows     = deviceAlloc<int>(num_bcs);
      b->diag        = deviceAlloc<int>(num_bcs);
      b->col_offsets = deviceAlloc<int>(num_bcs + 1LL);
      b->bc_mask     = deviceAlloc<int>(rows);
      b->row_begin   = deviceAlloc<int>(num_bcs);
      b->row_end     = deviceAlloc<int>(num_bcs);
      Scratch sc;
      auto* status    = deviceAlloc<DeviceStatus>(1);
      sc.p[0]         = status;
      auto* bc_by_col = deviceAlloc<int>(cols);
      sc.p[1]         = bc_by_col;
      auto* count     = deviceAlloc<int>(num_bcs + 1LL);
      sc.p[2]         = count;
      auto* lift_cnt  = deviceAlloc<int>(rows + 1LL);
      sc.p[3]         = lift_cnt;
      auto* lift_off  = deviceAlloc<int>(rows + 1LL);
      sc.p[4]         = lift_off;
      auto* row_flag  = deviceAlloc<int>(rows + 1LL);
      sc.p[5]         = row_flag;
      auto* row_rank  = deviceAlloc<int>(rows + 1LL);
      sc.p[6]         = row_rank;

      cudaCheck(cudaMemsetAsync(status, 0, sizeof(DeviceStatus), s), "memset");
      if (rows > 0)
      {
        validatePattern<<<blocksFor(rows, 256), 256, 0, s>>>(rows, cols, row_ptr,
                                                             col_ind, status);
        cudaCheck(cudaGetLastError(), "BoundaryMap pattern check launch");
      }
      checkDeviceStatus(status, s);
      if (cols > 0)
      {
        cudaCheck(cudaMemsetAsync(bc_by_col, 0xff, sizeof(int) * cols, s), "memset");
      }
      if (rows > 0)
      {
        cudaCheck(cudaMemsetAsync(b->bc_mask, 0, sizeof(int) * rows, s), "memset");
      }
      if (num_bcs > 0)
      {
        cudaCheck(cudaMemsetAsync(b->diag, 0xff, sizeof(int) * num_bcs, s), "memset");
        cudaCheck(cudaMemsetAsync(count, 0, sizeof(int) * (num_bcs + 1LL), s), "memset");
        flagConstraints<<<blocksFor(num_bcs, 256), 256, 0, s>>>(
            num_bcs, rows, dofs, bc_by_col, b->bc_rows, b->bc_mask, status);
        cudaCheck(cudaGetLastError(), "BoundaryMap flag launch");
      }
      checkDeviceStatus(status, s);
      if (rows > 0)
      {
        scanRows<<<blocksFor(rows, 256), 256, 0, s>>>(
            rows, row_ptr, col_ind, bc_by_col, b->bc_mask, count, b->diag,
            lift_cnt, status);
        cudaCheck(cudaGetLastError(), "BoundaryMap scan launch");
      }
      if (num_bcs > 0)
      {
        checkDiag<<<blocksFor(num_bcs, 256), 256, 0, s>>>(
            num_bcs, b->bc_rows, row_ptr, b->diag, b->row_begin, b->row_end,
            status);
        cudaCheck(cudaGetLastError(), "BoundaryMap diag launch");
      }
      checkDeviceStatus(status, s);

      const long long ncol = exclusiveScan(count, b->col_offsets, num_bcs, s);
      b->num_col_entries   = static_cast<int>(ncol);
      b->col_entries       = deviceAlloc<int>(ncol);
      b->col_rows          = deviceAlloc<int>(ncol);
      auto* tmp_k          = deviceAlloc<int>(ncol);
      sc.p[7]              = tmp_k;
      auto* tmp_r          = deviceAlloc<int>(ncol);
      sc.p[8]              = tmp_r;
      if (num_bcs > 0 && rows > 0)
      {
        cudaCheck(cudaMemsetAsync(count, 0, sizeof(int) * (num_bcs + 1LL), s), "memset");
        bucketColumns<<<blocksFor(rows, 256), 256, 0, s>>>(
            rows, row_ptr, col_ind, bc_by_col, b->col_offsets, count, tmp_k, tmp_r);
        cudaCheck(cudaGetLastError(), "BoundaryMap bucket launch");
        orderColumns<<<blocksFor(num_bcs * 32LL, 256), 256, 0, s>>>(
            num_bcs, b->col_offsets, tmp_k, tmp_r, b->col_entries, b->col_rows);
        cudaCheck(cudaGetLastError(), "BoundaryMap order launch");
      }

      // Row-grouped lifting list.
      const long long nlift_entries = exclusiveScan(lift_cnt, lift_off, rows, s);
      if (rows > 0)
      {
        flagPositive<<<blocksFor(rows, 256), 256, 0, s>>>(rows, lift_cnt, row_flag);
        cudaCheck(cudaGetLastError(), "BoundaryMap lift flag launch");
      }
      const long long nl = exclusiveScan(row_flag, row_rank, rows, s);
      b->num_lift_rows   = static_cast<int>(nl);
      b->lift_rows       = deviceAlloc<int>(nl);
      b->lift_offsets    = deviceAlloc<int>(nl + 1);
      b->lift_k          = deviceAlloc<int>(nlift_entries);
      b->lift_ib         = deviceAlloc<int>(nlift_entries);
      if (nl > 0)
      {
        compactLiftRows<<<blocksFor(rows, 256), 256, 0, s>>>(
            rows, lift_cnt, lift_off, row_rank, b->lift_rows, b->lift_offsets);
        cudaCheck(cudaGetLastError(), "BoundaryMap lift compact launch");
        const int total = static_cast<int>(nlift_entries);
        cudaCheck(cudaMemcpyAsync(b->lift_offsets + nl, &total, sizeof(int),
                                  cudaMemcpyHostToDevice, s),
                  "BoundaryMap lift total");
        fillLift<<<blocksFor(nl, 128), 128, 0, s>>>(
            static_cast<int>(nl), b->lift_rows, b->lift_offsets, row_ptr,
            col_ind, bc_by_col, b->lift_k, b->lift_ib);
        cudaCheck(cudaGetLastError(), "BoundaryMap lift fill launch");
      }
      else
      {
        cudaCheck(cudaMemsetAsync(b->lift_offsets, 0, sizeof(int), s), "memset");
      }
      cudaCheck(cudaStreamSynchronize(s), "BoundaryMap build");
    }
    catch (...)
    {
      delete b;
      throw;
    }
    *out = b;
  });
}

extern "C" int gbfem_boundary_map_get_view(const gbfem_boundary_map* b,
                                           gbfem_boundary_map_view* info)
{
  using namespace gbfem;
  return guarded([&] {
    require(b != nullptr && info != nullptr, "BoundaryMap handle is null");
    info->num_rows        = b->num_rows;
    info->num_cols        = b->num_cols;
    info->nnz             = b->nnz;
    info->num_bcs         = b->num_bcs;
    info->num_col_entries = b->num_col_entries;
    info->layout_id       = b->layout_id;
    info->bc_rows         = b->bc_rows;
    info->diag            = b->diag;
    info->col_offsets     = b->col_offsets;
    info->col_entries     = b->col_entries;
    info->col_rows        = b->col_rows;
    info->bc_mask         = b->bc_mask;
  });
}

extern "C" void gbfem_boundary_map_destroy(gbfem_boundary_map* b)
{
  delete b;
}

extern "C" int gbfem_replace_rows(const gbfem_boundary_map* b, double* vals,
                                  double d, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(b != nullptr, "BoundaryMap handle is null");
    if (b->num_bcs == 0)
    {
      return;
    }
    require(vals != nullptr, "BoundaryMap matrix values are null");
    // dependent launches: start while the kernel before them drains
    launchDependent(replaceRowsKernel, blocksFor(static_cast<long long>(b->num_bcs) * kRowLanes, 256),
                    256, asStream(stream),
                    b->num_bcs, static_cast<const int*>(b->row_begin),
                    static_cast<const int*>(b->row_end), static_cast<const int*>(b->diag), vals, d);
    cudaCheck(cudaGetLastError(), "replaceRows launch");
  });
}

extern "C" int gbfem_replace_res(const gbfem_boundary_map* b,
                                 const double* state, const double* g,
                                 double* res, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(b != nullptr, "BoundaryMap handle is null");
    require(state != res && g != res,
            "BoundaryMap residual output must not alias its inputs");
    if (b->num_bcs == 0)
    {
      return;
    }
    launchDependent(replaceResKernel, blocksFor(b->num_bcs, 256), 256, asStream(stream),
                    b->num_bcs, static_cast<const int*>(b->bc_rows), state, g, res);
    cudaCheck(cudaGetLastError(), "replaceRes launch");
  });
}

extern "C" int gbfem_zero_boundary(const gbfem_boundary_map* b, double* v,
                                   void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(b != nullptr, "BoundaryMap handle is null");
    if (b->num_bcs == 0)
    {
      return;
    }
    zeroBoundaryKernel<<<blocksFor(b->num_bcs, 256), 256, 0, asStream(stream)>>>(
        b->num_bcs, b->bc_rows, v);
    cudaCheck(cudaGetLastError(), "zeroBoundary launch");
  });
}

extern "C" int gbfem_prepare_forward_solve(const gbfem_boundary_map* b,
                                           double* vals, double* rhs,
                                           const double* g, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(b != nullptr, "BoundaryMap handle is null");
    require(rhs != g, "BoundaryMap RHS and prescribed values must not alias");
    require(rhs != vals && g != vals,
            "BoundaryMap vectors must not alias matrix values");
    if (b->num_bcs == 0)
    {
      return;
    }
    const int total = b->num_lift_rows + b->num_bcs;
    forwardSolveKernel<<<blocksFor(total, 128), 128, 0, asStream(stream)>>>(
        b->num_lift_rows, b->lift_rows, b->lift_offsets, b->lift_k, b->lift_ib,
        b->num_bcs, b->bc_rows, b->row_begin, b->row_end, b->diag, vals, rhs, g);
    cudaCheck(cudaGetLastError(), "prepareForwardSolve launch");
  });
}
