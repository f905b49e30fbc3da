// spmv.cu — FP64 CSR SpMV, transpose SpMV and axpby, replacing
// MatrixHandler<CudaCsrBackend>::matvec / matvecT (cuSPARSE CSR_ALG1,
// femx/linalg/handler/MatrixHandler.cu:335-398,514-542) and
// VectorHandler<Cuda>::axpby (VectorHandler.cu:124-136).
//
// matvec: one thread per row. FE rows are short (7 entries for P1, ~30 for
// Taylor-Hood), a warp's rows are contiguous in memory, so the 32 threads
// together stream a contiguous stretch of vals/col_ind and L1 serves the
// per-thread walk; each nonzero costs exactly one FP64 FMA, the minimum on a
// part whose FP64 rate is the scarce resource (on GB300 the FMAs alone take
// about as long as streaming the matrix from HBM). x is gathered through L2.
// Each lane loads one row pointer; its row end comes from the next lane.
//
// Semantics follow cuSPARSE (the reference's device path): y is not read when
// beta == 0.
#include "common.cuh"

namespace
{

template <bool kBeta>
__global__ void __launch_bounds__(256)
    spmvRows(int rows, const int* __restrict__ row_ptr,
             const int* __restrict__ col_ind, const double* __restrict__ vals,
             const double* __restrict__ x, double* __restrict__ y,
             double alpha, double beta)
{
  const int r    = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  // every lane of the warp takes part in the shuffle; row_ptr has rows + 1
  // entries, so lanes past the last row read the end pointer
  const int k0 = __ldg(row_ptr + (r < rows ? r : rows));
  int       k1 = __shfl_down_sync(0xffffffffu, k0, 1);
  if (lane == 31)
  {
    k1 = __ldg(row_ptr + (r + 1 < rows ? r + 1 : rows));
  }
  if (r >= rows)
  {
    return;
  }
  double acc = 0.0;
  for (int k = k0; k < k1; ++k)
  {
    acc = fma(__ldg(vals + k), __ldg(x + __ldg(col_ind + k)), acc);
  }
  y[r] = kBeta ? alpha * acc + beta * y[r] : alpha * acc;
}

__global__ void scaleVec(int n, double beta, double* __restrict__ y)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    y[i] = beta == 0.0 ? 0.0 : beta * y[i];
  }
}

__global__ void __launch_bounds__(256)
    spmvTRows(int rows, const int* __restrict__ row_ptr,
              const int* __restrict__ col_ind, const double* __restrict__ vals,
              const double* __restrict__ x, double* __restrict__ y,
              double alpha)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows)
  {
    return;
  }
  const double v = alpha * x[r];
  for (int k = row_ptr[r]; k < row_ptr[r + 1]; ++k)
  {
    gbfem::redAdd(y + col_ind[k], vals[k] * v);
  }
}

__global__ void axpbyKernel(int n, double a, const double* __restrict__ x,
                            double b, double* __restrict__ y)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    y[i] = b == 0.0 ? a * x[i] : a * x[i] + b * y[i];
  }
}

__global__ void expKernel(int n, const double* __restrict__ x, double* __restrict__ y)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    y[i] = exp(x[i]);
  }
}

void checkArgs(int rows, int cols, const int* row_ptr, const double* x,
               double* y)
{
  gbfem::require(rows >= 0 && cols >= 0,
                 "CSR matvec dimensions must be non-negative");
  gbfem::require(rows == 0 || (row_ptr && x && y), "CSR matvec inputs are null");
  gbfem::require(x != y, "CSR matvec input and output must not alias");
}

} // namespace

extern "C" int gbfem_spmv(int rows, int cols, const int* row_ptr,
                          const int* col_ind, const double* vals,
                          const double* x, double* y, double alpha, double beta,
                          void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    checkArgs(rows, cols, row_ptr, x, y);
    if (rows == 0)
    {
      return;
    }
    const unsigned b = blocksFor(rows, 256);
    if (beta == 0.0)
    {
      spmvRows<false><<<b, 256, 0, asStream(stream)>>>(rows, row_ptr, col_ind,
                                                       vals, x, y, alpha, beta);
    }
    else
    {
      spmvRows<true><<<b, 256, 0, asStream(stream)>>>(rows, row_ptr, col_ind,
                                                      vals, x, y, alpha, beta);
    }
    cudaCheck(cudaGetLastError(), "matvec launch");
  });
}

extern "C" int gbfem_spmv_t(int rows, int cols, const int* row_ptr,
                            const int* col_ind, const double* vals,
                            const double* x, double* y, double alpha,
                            double beta, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    checkArgs(rows, cols, row_ptr, x, y);
    cudaStream_t s = asStream(stream);
    if (cols > 0 && beta != 1.0)
    {
      scaleVec<<<blocksFor(cols, 256), 256, 0, s>>>(cols, beta, y);
      cudaCheck(cudaGetLastError(), "matvecT scale launch");
    }
    if (rows == 0)
    {
      return;
    }
    spmvTRows<<<blocksFor(rows, 256), 256, 0, s>>>(rows, row_ptr, col_ind, vals,
                                                   x, y, alpha);
    cudaCheck(cudaGetLastError(), "matvecT launch");
  });
}

extern "C" int gbfem_axpby(int n, double a, const double* x, double b,
                           double* y, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(n >= 0, "axpby size must be non-negative");
    if (n == 0)
    {
      return;
    }
    require(x != nullptr && y != nullptr, "axpby inputs are null");
    axpbyKernel<<<blocksFor(n, 256), 256, 0, asStream(stream)>>>(n, a, x, b, y);
    cudaCheck(cudaGetLastError(), "axpby launch");
  });
}

extern "C" int gbfem_exp(int n, const double* x, double* y, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(n >= 0, "exp size must be non-negative");
    if (n == 0)
    {
      return;
    }
    require(x != nullptr && y != nullptr, "exp inputs are null");
    expKernel<<<blocksFor(n, 256), 256, 0, asStream(stream)>>>(n, x, y);
    cudaCheck(cudaGetLastError(), "exp launch");
  });
}
