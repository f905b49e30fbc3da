// measure.cu — FP64 FMA throughput probe (see include/gbfem_measure.h).
#include "common.cuh"
#include "dfloat.cuh"
#include "gbfem_measure.h"

namespace
{
__global__ void fp64FmaProbe(int iters, double* out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double    a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
  {
    a[i] = 1.0 + 1.0e-9 * (t + i);
  }
  const double m = 0.999999999, c = 1.0e-12;
  for (int it = 0; it < iters; ++it)
  {
#pragma unroll
    for (int i = 0; i < 8; ++i)
    {
      a[i] = fma(a[i], m, c);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i)
  {
    s += a[i];
  }
  out[t] = s;
}
__global__ void convertProbe(int n, const double* in, float* out_f, double* out_d)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    const float f = gbfem::f64ToF32(in[i]);
    out_f[i]      = f;
    out_d[i]      = gbfem::f32ToF64(f);
  }
}
__global__ void convertFtzProbe(int n, const float* in, double* out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    out[i] = gbfem::f32ToF64Ftz(in[i]);
  }
}
__global__ void rcpProbe(int n, const double* in, double* out, int rsqrt)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    out[i] = rsqrt ? gbfem::rsqrtF64(in[i]) : gbfem::rcpF64(in[i]);
  }
}
__global__ void ddProbe(int n, const double* in, float* hi, float* lo, const float* jhi,
                        const float* jlo, double* joined)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
  {
    const gbfem::Dd d = gbfem::ddSplitInt(in[i]);
    hi[i]             = d.hi;
    lo[i]             = d.lo;
    joined[i]         = gbfem::ddJoinInt(gbfem::Dd(jhi[i], jlo[i]));
  }
}
} // namespace

extern "C" int gbfem_probe_rcp(int n, const double* in, double* out, int rsqrt, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(n >= 0 && (n == 0 || (in && out)), "probe arguments are invalid");
    if (n > 0)
    {
      rcpProbe<<<blocksFor(n, 256), 256, 0, asStream(stream)>>>(n, in, out, rsqrt);
      cudaCheck(cudaGetLastError(), "reciprocal probe launch");
    }
  });
}

extern "C" int gbfem_probe_convert_ftz(int n, const float* in, double* out, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(n >= 0 && (n == 0 || (in && out)), "probe arguments are invalid");
    if (n > 0)
    {
      convertFtzProbe<<<blocksFor(n, 256), 256, 0, asStream(stream)>>>(n, in, out);
      cudaCheck(cudaGetLastError(), "convert probe launch");
    }
  });
}

extern "C" int gbfem_probe_convert(int n, const double* in, float* out_f,
                                   double* out_d, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(n >= 0 && (n == 0 || (in && out_f && out_d)), "probe arguments are invalid");
    if (n > 0)
    {
      convertProbe<<<blocksFor(n, 256), 256, 0, asStream(stream)>>>(n, in, out_f, out_d);
      cudaCheck(cudaGetLastError(), "convert probe launch");
    }
  });
}

extern "C" int gbfem_probe_fp64_fma(int blocks, int threads, int iters,
                                    double* out, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(blocks > 0 && threads > 0 && threads <= 1024 && iters > 0 && out,
            "probe arguments are invalid");
    fp64FmaProbe<<<blocks, threads, 0, asStream(stream)>>>(iters, out);
    cudaCheck(cudaGetLastError(), "probe launch");
  });
}

extern "C" int gbfem_probe_dd(int n, const double* in, float* hi, float* lo, const float* jhi,
                              const float* jlo, double* joined, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(n >= 0 && (n == 0 || (in && hi && lo && jhi && jlo && joined)),
            "probe arguments are invalid");
    if (n > 0)
    {
      ddProbe<<<blocksFor(n, 256), 256, 0, asStream(stream)>>>(n, in, hi, lo, jhi, jlo, joined);
      cudaCheck(cudaGetLastError(), "double-float probe launch");
    }
  });
}
