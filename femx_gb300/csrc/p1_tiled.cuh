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

// tile-local element record in shared memory: the three edge weights
// (edge k opposite vertex k) and the three residual terms
template <class T>
struct TileElem
{
  T k[3];
  T r[3];
};

template <class T>
constexpr int tileSmemBytes(int verts, int elems, bool load)
{
  return verts * static_cast<int>(sizeof(double2) + (load ? 2 : 1) * sizeof(T))
         + elems * static_cast<int>(sizeof(TileElem<T>));
}

template <class T, bool kLoad, bool kJac>
__global__ void __launch_bounds__(256) p1TiledKernel(P1TileArgs a)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int t   = blockIdx.x;
  const int v0  = a.vert_off[t];
  const int nv  = a.vert_off[t + 1] - v0;
  const int e0  = a.elem_off[t];
  const int nel = a.elem_off[t + 1] - e0;
  const int r0  = a.row_off[t];
  const int nr  = a.row_off[t + 1] - r0;

  double2*     sx = reinterpret_cast<double2*>(smem);
  T*           su = reinterpret_cast<T*>(sx + nv);
  T*           sf = su + nv;
  TileElem<T>* se = reinterpret_cast<TileElem<T>*>(sf + (kLoad ? nv : 0));

  // 0. vertices
  for (int i = threadIdx.x; i < nv; i += blockDim.x)
  {
    const int d = a.vert_dof[v0 + i];
    const int n = a.vert_node[v0 + i];
    sx[i]       = a.coords[n];
    su[i]       = tSplit<T>(a.u[d]);
    if (kLoad)
    {
      sf[i] = tSplit<T>(a.f[n]);
    }
  }
  __syncthreads();

  // 1. elements
  for (int l = threadIdx.x; l < nel; l += blockDim.x)
  {
    const unsigned c    = a.tconn[e0 + l];
    const int      i0   = c & 1023u, i1 = (c >> 10) & 1023u, i2 = c >> 20;
    const double2  x0   = sx[i0], x1 = sx[i1], x2 = sx[i2];
    const T        ax   = tSplit<T>(x1.x - x0.x), ay = tSplit<T>(x1.y - x0.y);
    const T        bx   = tSplit<T>(x2.x - x0.x), by = tSplit<T>(x2.y - x0.y);
    const T        det  = ax * by - bx * ay;
    T              adet = tAbs(det);
    const int      e    = a.elems[e0 + l];
    if (!(tLead(adet) >= 1.0e-30))
    {
      gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
      adet = T(1);
    }
    const T s   = tSplit<T>(a.kappa[e]) * tRcp(adet) * T(0.5);
    const T cx  = bx - ax, cy = by - ay;
    const T k12 = -(s * (ax * bx + ay * by));
    const T k01 = -(s * (bx * cx + by * cy));
    const T k02 = s * (ax * cx + ay * cy);
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
    TileElem<T>& E = se[l];
    E.k[0]         = k12;
    E.k[1]         = k02;
    E.k[2]         = k01;
    E.r[0]         = rr0;
    E.r[1]         = rr1;
    E.r[2]         = rr2;
  }
  __syncthreads();

  // 2. rows
  for (int i = threadIdx.x; i < nr; i += blockDim.x)
  {
    const int r  = a.rows[r0 + i];
    const int rs = a.row_ptr[r], re = a.row_ptr[r + 1];
    T         off = T(0), res = T(0);
    int       ds  = -1;
    for (int sl = rs; sl < re; ++sl)
    {
      const unsigned w = a.slot_ref[sl];
      if (w == 0xffffffffu)
      {
        ds = sl;
        continue;
      }
      T K = T(0);
#pragma unroll
      for (int h = 0; h < 2; ++h)
      {
        const unsigned p = h == 0 ? (w & 0xffffu) : (w >> 16);
        if (p != 0xffffu)
        {
          const TileElem<T>& E = se[p >> 4];
          const unsigned     k = (p >> 2) & 3u;
          K                    = h == 0 ? E.k[k] : K + E.k[k];
          if (p & 2u)
          {
            // the row's vertex is the edge end after (which-end 0) or
            // before (1) the opposite vertex
            const unsigned v = (p & 1u) ? (k + 2u) % 3u : (k + 1u) % 3u;
            res += E.r[v];
          }
        }
      }
      off += K;
      if (kJac)
      {
        a.vals[sl] = tJoin(K);
      }
    }
    if (kJac && ds >= 0)
    {
      a.vals[ds] = tJoin(-off);
    }
    a.res[r] = tJoin(res);
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
    p1TiledKernel<T, kLoad, kJac><<<m->num_tiles, 256, bytes, s>>>(a);
  }
}

} // namespace
