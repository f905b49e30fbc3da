// gather.cuh — the row pass of deterministic assembly.
//
// An element pass has written one record per element row (e, i): the row's
// entries (16 values, padded) and its residual term, numbered so that the
// records of CSR row r are gather_off[r] .. gather_off[r + 1] in ascending
// (e, i) order (maps.cuh). This pass sums, for every row, its records into
// the row's CSR segment in record order — the order femx's CPU loop adds
// element blocks (Assembly.hpp:186-223) — and writes the segment and the
// residual once. No atomics and no zero-fill: every slot of a row is
// written, and the result is bitwise reproducible.
//
// FP32 records are accumulated as unevaluated float pairs (hi + lo, Knuth's
// TwoSum: hi + lo equals the running sum of the float addends up to the
// rounding of lo), then converted exactly and added once in FP64, so the
// accumulation error is at the level of an FP64 sum while the additions run
// on the FP32 pipe. FP64 records are summed in FP64.
#pragma once

#include "common.cuh"

namespace gbfem
{

constexpr int kGatherThreads = 128;          // 8 half-warps
constexpr int kGatherRows    = 32;           // rows per block
constexpr int kGatherMaxRow  = 256;          // positions are bytes
constexpr int kGatherPrefetch = 8;           // records loaded ahead per row

template <class T>
struct GatherAcc;
template <>
struct GatherAcc<float>
{
  using type = float2; // (hi, lo)
  __device__ static type zero() { return make_float2(0.f, 0.f); }
  __device__ static void add(type& a, float v)
  {
    const float s  = a.x + v;
    const float bb = s - a.x;
    const float er = (a.x - (s - bb)) + (v - bb);
    a.x            = s;
    a.y += er;
  }
  __device__ static double value(const type& a) { return f32ToF64(a.x) + f32ToF64(a.y); }
};
template <>
struct GatherAcc<double>
{
  using type = double;
  __device__ static type   zero() { return 0.0; }
  __device__ static void   add(type& a, double v) { a += v; }
  __device__ static double value(const type& a) { return a; }
};

// Rows [blockIdx.x * 32, +32): half-warp h sums rows h, h + 8, ...; then
// warp 0 sums the 32 residuals, one row per lane.
template <class T>
__global__ void __launch_bounds__(kGatherThreads)
    gatherRowsKernel(int num_rows, int nc, const int* __restrict__ off,
                     const T* __restrict__ rec, const unsigned char* __restrict__ pos,
                     const int* __restrict__ row_ptr, const double* __restrict__ rres,
                     double* __restrict__ vals, double* __restrict__ res)
{
  using Acc = GatherAcc<T>;
  __shared__ typename Acc::type buf[kGatherThreads / 16][kGatherMaxRow];
  const int      h     = threadIdx.x >> 4;
  const int      j     = threadIdx.x & 15;
  const unsigned hmask = 0xffffu << (16 * (h & 1));
  const int      r0    = blockIdx.x * kGatherRows;
  if (vals != nullptr)
  {
    for (int rr = h; rr < kGatherRows; rr += kGatherThreads / 16)
    {
      const int r = r0 + rr;
      if (r >= num_rows)
      {
        break; // uniform within the half-warp
      }
      const int rs = row_ptr[r];
      const int L  = row_ptr[r + 1] - rs;
      for (int q = j; q < L; q += 16)
      {
        buf[h][q] = Acc::zero();
      }
      const int kb = off[r], ke = off[r + 1];
      for (int k0 = kb; k0 < ke; k0 += kGatherPrefetch)
      {
        const int n = min(kGatherPrefetch, ke - k0); // uniform in the half-warp
        T         v[kGatherPrefetch];
        int       p[kGatherPrefetch];
#pragma unroll
        for (int t = 0; t < kGatherPrefetch; ++t)
        {
          if (t < n)
          {
            const long long k = k0 + t;
            v[t]              = rec[k * 16 + j];
            p[t]              = pos[k * 16 + j];
          }
        }
        __syncwarp(hmask);
#pragma unroll
        for (int t = 0; t < kGatherPrefetch; ++t)
        {
          if (t < n)
          {
            if (j < nc)
            {
              Acc::add(buf[h][p[t]], v[t]);
            }
            __syncwarp(hmask);
          }
        }
      }
      for (int q = j; q < L; q += 16)
      {
        vals[rs + q] = Acc::value(buf[h][q]);
      }
      __syncwarp(hmask);
    }
  }
  if (threadIdx.x < 32)
  {
    const int r = r0 + threadIdx.x;
    if (r < num_rows)
    {
      double acc = 0.0;
      for (int k = off[r]; k < off[r + 1]; ++k)
      {
        acc += rres[k];
      }
      res[r] = acc;
    }
  }
}

} // namespace gbfem
