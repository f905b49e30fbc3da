// transpose.cu — explicit CSR transpose with a cached value permutation,
// femx MatrixHandler::transpose (femx/linalg/handler/MatrixHandler.cpp:
// 140-155, MatrixHandler.cu:401-512): the transposed pattern and the
// permutation are built once per source layout; each transpose then only
// moves the values.
//
// Build (GPU): entries are counted per source column (= transposed row),
// the counts scanned into the transposed row_ptr, entries placed and each
// transposed row sorted by source row, so the transposed column indices are
// ascending like the reference's. The apply kernel gathers: transposed slot
// p reads source slot src[p] (coalesced writes).
#include "common.cuh"

struct gbfem_csr_transpose
{
  int  rows = 0, cols = 0, nnz = 0; // of the source
  int* t_row_ptr = nullptr;         // [cols + 1]
  int* t_col_ind = nullptr;         // [nnz]
  int* src       = nullptr;         // [nnz] source slot of transposed slot

  ~gbfem_csr_transpose()
  {
    gbfem::deviceFree(t_row_ptr);
    gbfem::deviceFree(t_col_ind);
    gbfem::deviceFree(src);
  }
};

namespace
{

__global__ void countColumns(int nnz, const int* __restrict__ col_ind, int cols,
                             int* __restrict__ cnt, gbfem::DeviceStatus* bad)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz)
  {
    return;
  }
  const int c = col_ind[k];
  if (static_cast<unsigned>(c) >= static_cast<unsigned>(cols))
  {
    gbfem::devFail(bad, gbfem::kDevPatternInvalid, k);
    return;
  }
  atomicAdd(cnt + c, 1);
}

__global__ void placeEntries(int rows, const int* __restrict__ row_ptr,
                             const int* __restrict__ col_ind, const int* __restrict__ t_row_ptr,
                             int* __restrict__ fill, int* __restrict__ t_col_ind,
                             int* __restrict__ src)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows)
  {
    return;
  }
  for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
  {
    const int c = col_ind[k];
    const int p = t_row_ptr[c] + atomicAdd(fill + c, 1);
    t_col_ind[p] = r;
    src[p]       = k;
  }
}

__global__ void sortTransposedRows(int cols, const int* __restrict__ t_row_ptr,
                                   int* __restrict__ t_col_ind, int* __restrict__ src)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols)
  {
    return;
  }
  const int b = t_row_ptr[c], e = t_row_ptr[c + 1];
  for (int a = b + 1; a < e; ++a)
  {
    const int r = t_col_ind[a], k = src[a];
    int       q = a - 1;
    while (q >= b && t_col_ind[q] > r)
    {
      t_col_ind[q + 1] = t_col_ind[q];
      src[q + 1]       = src[q];
      --q;
    }
    t_col_ind[q + 1] = r;
    src[q + 1]       = k;
  }
}

__global__ void gatherValues(int nnz, const int* __restrict__ src, const double* __restrict__ vals,
                             double* __restrict__ t_vals)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nnz)
  {
    t_vals[p] = vals[src[p]];
  }
}

} // namespace

extern "C" int gbfem_csr_transpose_create(int rows, int cols, const int* row_ptr,
                                          const int* col_ind, void* stream,
                                          gbfem_csr_transpose** out)
{
  using namespace gbfem;
  return guarded([&] {
    require(out != nullptr, "CSR transpose output handle is null");
    *out = nullptr;
    require(rows >= 0 && cols >= 0, "CSR dimensions must be non-negative");
    require(row_ptr != nullptr && (rows == 0 || col_ind != nullptr),
            "CSR pattern arrays must not be null");
    cudaStream_t s = asStream(stream);
    int          nnz = 0;
    cudaCheck(cudaMemcpyAsync(&nnz, row_ptr + rows, sizeof(int), cudaMemcpyDeviceToHost, s),
              "CSR nnz readback");
    cudaCheck(cudaStreamSynchronize(s), "CSR nnz readback");
    require(nnz >= 0, "CSR pattern is invalid");
    auto* t = new gbfem_csr_transpose;
    try
    {
      t->rows      = rows;
      t->cols      = cols;
      t->nnz       = nnz;
      t->t_row_ptr = deviceAlloc<int>(cols + 1LL);
      t->t_col_ind = deviceAlloc<int>(nnz);
      t->src       = deviceAlloc<int>(nnz);
      int*          cnt = deviceAlloc<int>(cols + 1LL);
      DeviceStatus* bad = deviceAlloc<DeviceStatus>(1);
      try
      {
        cudaCheck(cudaMemsetAsync(cnt, 0, sizeof(int) * (cols + 1LL), s), "memset");
        cudaCheck(cudaMemsetAsync(bad, 0, sizeof(DeviceStatus), s), "memset");
        if (nnz > 0)
        {
          countColumns<<<blocksFor(nnz, 256), 256, 0, s>>>(nnz, col_ind, cols, cnt, bad);
          cudaCheck(cudaGetLastError(), "CSR transpose count launch");
        }
        DeviceStatus bad_h{};
        cudaCheck(cudaMemcpyAsync(&bad_h, bad, sizeof(DeviceStatus), cudaMemcpyDeviceToHost, s),
                  "CSR transpose status readback");
        cudaCheck(cudaStreamSynchronize(s), "CSR transpose count");
        require(bad_h.code == 0, "CSR column index is out of range");
        exclusiveScan(cnt, t->t_row_ptr, cols, s);
        cudaCheck(cudaMemsetAsync(cnt, 0, sizeof(int) * (cols + 1LL), s), "memset");
        if (rows > 0 && nnz > 0)
        {
          placeEntries<<<blocksFor(rows, 256), 256, 0, s>>>(rows, row_ptr, col_ind,
                                                            t->t_row_ptr, cnt, t->t_col_ind,
                                                            t->src);
          sortTransposedRows<<<blocksFor(cols, 256), 256, 0, s>>>(cols, t->t_row_ptr,
                                                                 t->t_col_ind, t->src);
          cudaCheck(cudaGetLastError(), "CSR transpose build launch");
        }
        cudaCheck(cudaStreamSynchronize(s), "CSR transpose build");
      }
      catch (...)
      {
        deviceFree(cnt);
        deviceFree(bad);
        throw;
      }
      deviceFree(cnt);
      deviceFree(bad);
    }
    catch (...)
    {
      delete t;
      throw;
    }
    *out = t;
  });
}

extern "C" int gbfem_csr_transpose_get_view(const gbfem_csr_transpose* t,
                                            gbfem_csr_transpose_view* v)
{
  using namespace gbfem;
  return guarded([&] {
    require(t != nullptr && v != nullptr, "CSR transpose handle is null");
    v->rows      = t->cols;
    v->cols      = t->rows;
    v->nnz       = t->nnz;
    v->row_ptr   = t->t_row_ptr;
    v->col_ind   = t->t_col_ind;
    v->src_slot  = t->src;
  });
}

extern "C" int gbfem_csr_transpose_apply(const gbfem_csr_transpose* t, const double* vals,
                                         double* t_vals, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(t != nullptr, "CSR transpose handle is null");
    require(t->nnz == 0 || (vals != nullptr && t_vals != nullptr),
            "CSR transpose values must not be null");
    require(vals != t_vals, "CSR transpose does not support in-place output");
    if (t->nnz > 0)
    {
      gatherValues<<<blocksFor(t->nnz, 256), 256, 0, asStream(stream)>>>(t->nnz, t->src, vals,
                                                                         t_vals);
      cudaCheck(cudaGetLastError(), "CSR transpose launch");
    }
  });
}

extern "C" void gbfem_csr_transpose_destroy(gbfem_csr_transpose* t)
{
  delete t;
}
