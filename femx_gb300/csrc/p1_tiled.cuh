// p1_tiled.cuh — owner-computes (tiled) assembly of the kappa-weighted P1
// Poisson residual and Jacobian: the atomic-free replacement of the element
// pass with FP64 reductions (tiles.cu builds the tiles and explains them).
//
// One block per tile, three phases separated by block barriers:
//   0. the tile's vertices are staged in shared memory: coordinates (FP64),
//      state and nodal source (converted to the arithmetic type T);
//   1. each tile element is evaluated once: its three off-diagonal stiffness
//      entries (one per edge, the matrix is symmetric) and its three
//      residual terms, into shared memory;
//   2. each owned row walks its CSR slots: slot (r, c) sums the one or two
//      element edges joining r and c and is written once; the diagonal is
//      minus the sum of the off-diagonals (P1 element rows sum to zero, as
//      femx's quadrature sum of dN_i . dN_j JxW does); the residual is the
//      sum of the element terms the row's slots carry.
// Every CSR value and residual entry is written exactly once with a plain
// store: no zero fill, no atomics, the same bits on every run.
//
// T = double: plain FP64. T = gbfem::Dd: FP64-accurate double-float on the
// FP32 pipe; the only FP64 instructions are the four coordinate
// differences per element (they carry the mesh scale exactly), every
// conversion runs on the integer pipe (ddSplitInt / ddJoinInt). T = float:
// FP32 element arithmetic, FP64 outputs.
//
// Element formulas (edge vectors a = x1 - x0, b = x2 - x0, c = b - a):
//   det = a x b,  s = kappa / (2 |det|)
//   K01 = -s b.c,  K02 = s a.c,  K12 = -s a.b   (the cotangent weights)
//   residual: r0 = K01 (u1-u0) + K02 (u2-u0), r1 = K12 (u2-u1) - K01 (u1-u0),
//             r2 = -(K02 (u2-u0) + K12 (u2-u1)), minus the load
//             F_i = |det|/24 (f_i + f0 + f1 + f2) (the order-2 rule is exact
//             for the P1-interpolated source).
#pragma once

#include "dfloat.cuh"
#include "maps.cuh"

namespace
{
using gbfem::Dd;

struct P1TileArgs
{
  const int*           row_off;
  const int*           rows;
  const int*           elem_off;
  const int*           elems;
  const unsigned*      tconn;
  const int*           vert_off;
  const int*           vert_dof;
  const int*           vert_node;
  const unsigned*      slot_ref;
  const int*           row_ptr;
  const double2*       coords;
  const double*        kappa;
  const double*        f;
  const double*        u;
  double*              res;
  double*              vals;
  gbfem::DeviceStatus* status;
};

template <class T>
__device__ __forceinline__ T tSplit(double d);
template <>
__device__ __forceinline__ double tSplit<double>(double d)
{
  return d;
}
template <>
__device__ __forceinline__ float tSplit<float>(double d)
{
  return gbfem::f64ToF32(d);
}
template <>
__device__ __forceinline__ Dd tSplit<Dd>(double d)
{
  return gbfem::ddSplitInt(d);
}

__device__ __forceinline__ double tJoin(double v)
{
  return v;
}
__device__ __forceinline__ double tJoin(float v)
{
  return gbfem::f32ToF64Ftz(v);
}
__device__ __forceinline__ double tJoin(Dd v)
{
  return gbfem::ddJoinInt(v);
}

__device__ __forceinline__ double tRcp(double x)
{
  return gbfem::rcpF64(x);
}
__device__ __forceinline__ float tRcp(float x)
{
  return __frcp_rn(x);
}
__device__ __forceinline__ Dd tRcp(Dd x)
{
  return gbfem::ddRcp(x);
}

__device__ __forceinline__ double tLead(double x)
{
  return x;
}
__device__ __forceinline__ double tLead(float x)
{
  return x;
}
__device__ __forceinline__ double tLead(Dd x)
{
  return x.hi;
}

template <class T>
__device__ __forceinline__ T tAbs(T x)
{
  return tLead(x) < 0.0 ? -x : x;
}

// Row sums: double-float terms are added with TwoSum of the leading parts
// and the trailing parts summed unnormalised (Dot2-style accumulation),
// normalised once before the conversion; float and double add plainly.
template <class T>
__device__ __forceinline__ T tAcc(T acc, T x)
{
  return acc + x;
}
template <>
__device__ __forceinline__ Dd tAcc<Dd>(Dd acc, Dd x)
{
  const float s  = __fadd_rn(acc.hi, x.hi);
  const float bb = __fsub_rn(s, acc.hi);
  const float e  = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(x.hi, bb));
  return Dd(s, __fadd_rn(__fadd_rn(acc.lo, x.lo), e));
}
template <class T>
__device__ __forceinline__ T tNorm(T x)
{
  return x;
}
template <>
__device__ __forceinline__ Dd tNorm<Dd>(Dd x)
{
  return gbfem::ddQuick(x.hi, x.lo);
}

// a x + b y with one rounding chain (Dot2 for double-float: both products
// split exactly, their leading parts added with TwoSum, every error and
// cross term gathered in the trailing part)
template <class T>
__device__ __forceinline__ T tDot2(T a, T x, T b, T y)
{
  return a * x + b * y;
}
template <>
__device__ __forceinline__ Dd tDot2<Dd>(Dd a, Dd x, Dd b, Dd y)
{
  const float p  = __fmul_rn(a.hi, x.hi);
  const float pe = __fmaf_rn(a.hi, x.hi, -p);
  const float q  = __fmul_rn(b.hi, y.hi);
  const float qe = __fmaf_rn(b.hi, y.hi, -q);
  const float s  = __fadd_rn(p, q);
  const float bb = __fsub_rn(s, p);
  float       e  = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(q, bb));
  e              = __fadd_rn(e, __fadd_rn(pe, qe));
  e              = __fmaf_rn(a.hi, x.lo, e);
  e              = __fmaf_rn(a.lo, x.hi, e);
  e              = __fmaf_rn(b.hi, y.lo, e);
  e              = __fmaf_rn(b.lo, y.hi, e);
  return gbfem::ddQuick(s, e);
}

// exact scaling by a power of two
__device__ __forceinline__ double tScale(double x, float p2)
{
  return x * p2;
}
__device__ __forceinline__ float tScale(float x, float p2)
{
  return x * p2;
}
__device__ __forceinline__ Dd tScale(Dd x, float p2)
{
  return Dd(__fmul_rn(x.hi, p2), __fmul_rn(x.lo, p2));
}

// tile-local edge record in shared memory: edge k of element l (opposite
// its vertex k) at 3 l + k holds the edge's stiffness entry and the
// residual term of vertex k + 1 (mod 3)
template <class T>
struct EdgeRec
{
  T K;
  T R;
};

template <class T>
constexpr int tileSmemBytes(int verts, int elems, bool load)
{
  return verts * static_cast<int>(sizeof(double2) + (load ? 2 : 1) * sizeof(T))
         + 3 * elems * static_cast<int>(sizeof(EdgeRec<T>));
}

constexpr int kTileThreads = 256; // rows per tile at most; elements at most twice that
constexpr int kRowPrefetch = 8;   // slot records of a row held in registers

template <class T, bool kLoad, bool kJac>
__global__ void __launch_bounds__(kTileThreads) p1TiledKernel(P1TileArgs a)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int t   = blockIdx.x;
  const int v0  = a.vert_off[t];
  const int nv  = a.vert_off[t + 1] - v0;
  const int e0  = a.elem_off[t];
  const int nel = a.elem_off[t + 1] - e0;
  const int r0  = a.row_off[t];
  const int nr  = a.row_off[t + 1] - r0;

  double2*    sx = reinterpret_cast<double2*>(smem);
  T*          su = reinterpret_cast<T*>(sx + nv);
  T*          sf = su + nv;
  EdgeRec<T>* se = reinterpret_cast<EdgeRec<T>*>(sf + (kLoad ? nv : 0));

  // the row phase's global inputs, loaded before the barriers so that their
  // latency hides behind the vertex and element phases
  const int i  = threadIdx.x;
  int       r  = -1, rs = 0, re = 0;
  unsigned  w[kRowPrefetch];
  if (i < nr)
  {
    r  = a.rows[r0 + i];
    rs = a.row_ptr[r];
    re = a.row_ptr[r + 1];
  }
#pragma unroll
  for (int k = 0; k < kRowPrefetch; ++k)
  {
    w[k] = rs + k < re ? a.slot_ref[rs + k] : 0u;
  }
  // the element phase's global inputs (at most two elements per thread)
  unsigned ec[2];
  double   ek[2];
#pragma unroll
  for (int h = 0; h < 2; ++h)
  {
    const int l = i + h * kTileThreads;
    ec[h]       = l < nel ? a.tconn[e0 + l] : 0u;
    ek[h]       = l < nel ? a.kappa[a.elems[e0 + l]] : 0.0;
  }

  // 0. vertices
  for (int j = i; j < nv; j += kTileThreads)
  {
    const int d = a.vert_dof[v0 + j];
    const int n = a.vert_node[v0 + j];
    sx[j]       = a.coords[n];
    su[j]       = tSplit<T>(a.u[d]);
    if (kLoad)
    {
      sf[j] = tSplit<T>(a.f[n]);
    }
  }
  __syncthreads();

  // 1. elements
#pragma unroll
  for (int h = 0; h < 2; ++h)
  {
    const int l = i + h * kTileThreads;
    if (l >= nel)
    {
      break;
    }
    const unsigned c    = ec[h];
    const double   kap  = ek[h];
    const int      i0   = c & 1023u, i1 = (c >> 10) & 1023u, i2 = c >> 20;
    const double2  x0   = sx[i0], x1 = sx[i1], x2 = sx[i2];
    const T        ax   = tSplit<T>(x1.x - x0.x), ay = tSplit<T>(x1.y - x0.y);
    const T        bx   = tSplit<T>(x2.x - x0.x), by = tSplit<T>(x2.y - x0.y);
    const T        det  = tDot2(ax, by, -bx, ay);
    T              adet = tAbs(det);
    if (!(tLead(adet) >= 1.0e-30))
    {
      gbfem::devFail(a.status, gbfem::kDevSingularJacobian, a.elems[e0 + l]);
      adet = T(1);
    }
    const T s   = tScale(tSplit<T>(kap) * tRcp(adet), 0.5f);
    const T cx  = bx - ax, cy = by - ay;
    const T k12 = -(s * tDot2(ax, bx, ay, by));
    const T k01 = -(s * tDot2(bx, cx, by, cy));
    const T k02 = s * tDot2(ax, cx, ay, cy);
    const T u0 = su[i0], u1 = su[i1], u2 = su[i2];
    const T P = k01 * (u1 - u0), Q = k02 * (u2 - u0), R = k12 * (u2 - u1);
    T       rr0 = P + Q, rr1 = R - P, rr2 = -(Q + R);
    if (kLoad)
    {
      const T f0 = sf[i0], f1 = sf[i1], f2 = sf[i2];
      const T fs = f0 + f1 + f2;
      const T cf = adet * T(1.0 / 24.0);
      rr0 -= cf * (f0 + fs);
      rr1 -= cf * (f1 + fs);
      rr2 -= cf * (f2 + fs);
    }
    se[3 * l + 0] = EdgeRec<T>{k12, rr1};
    se[3 * l + 1] = EdgeRec<T>{k02, rr2};
    se[3 * l + 2] = EdgeRec<T>{k01, rr0};
  }
  __syncthreads();

  // 2. rows
  if (i < nr)
  {
    T    off = T(0), res = T(0);
    int  ds  = -1;
    auto slot = [&](int sl, unsigned wk) {
      if (wk == 0xffffffffu)
      {
        ds = sl;
        return;
      }
      const EdgeRec<T> e1 = se[wk & 0xfffu];
      T                K  = e1.K;
      if (wk & 0x1000u)
      {
        res = tAcc(res, e1.R);
      }
      const unsigned o2 = (wk >> 13) & 0xfffu;
      if (o2 != 0xfffu)
      {
        const EdgeRec<T> e2 = se[o2];
        K                   = K + e2.K;
        if (wk & 0x2000000u)
        {
          res = tAcc(res, e2.R);
        }
      }
      off = tAcc(off, K);
      if (kJac)
      {
        a.vals[sl] = tJoin(K);
      }
    };
#pragma unroll
    for (int k = 0; k < kRowPrefetch; ++k)
    {
      if (rs + k < re)
      {
        slot(rs + k, w[k]);
      }
    }
    for (int sl = rs + kRowPrefetch; sl < re; ++sl)
    {
      slot(sl, a.slot_ref[sl]);
    }
    if (kJac && ds >= 0)
    {
      a.vals[ds] = tJoin(-tNorm(off));
    }
    a.res[r] = tJoin(tNorm(res));
  }
}

// Launch over all tiles of the map (gbfem_assembly_map_enable_tiles).
template <class T, bool kLoad, bool kJac>
void launchP1Tiled(const P1TileArgs& a, const gbfem_assembly_map* m, cudaStream_t s)
{
  const int bytes = tileSmemBytes<T>(m->tile_max_verts, m->tile_max_elems, kLoad);
  if (bytes > 48 * 1024)
  {
    gbfem::cudaCheck(cudaFuncSetAttribute(p1TiledKernel<T, kLoad, kJac>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
                     "tiled assembly shared memory");
  }
  if (m->num_tiles > 0)
  {
    p1TiledKernel<T, kLoad, kJac><<<m->num_tiles, kTileThreads, bytes, s>>>(a);
  }
}

} // namespace
