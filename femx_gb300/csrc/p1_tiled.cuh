// p1_tiled.cuh — owner-computes (tiled) assembly of the kappa-weighted P1
// Poisson residual and Jacobian: the atomic-free replacement of the element
// pass with FP64 reductions (tiles.cu builds the tiles and explains them).
//
// One block per tile, four phases separated by block barriers:
//   0. the tile's vertices are staged in shared memory: coordinates, state
//      and nodal source (converted to the arithmetic type T);
//   1. each tile element is evaluated once: its three off-diagonal stiffness
//      entries (one per edge, the matrix is symmetric) and its three
//      residual terms, into shared memory;
//   2. each owned row walks its CSR slots: slot (r, c) sums the one or two
//      element edges joining r and c; the diagonal is minus the sum of the
//      off-diagonals (P1 element rows sum to zero, as femx's quadrature sum
//      of dN_i . dN_j JxW does); the residual is the sum of the element terms
//      the row's slots carry. Values are staged in shared memory as FP64;
//   3. the staged rows are written out run by run (consecutive rows have
//      consecutive CSR slots), coalesced (the double-float kernel stores
//      its rows directly from phase 2 instead, see tileStaged).
// Every CSR value and residual entry is written exactly once with a plain
// store: no zero fill, no atomics, the same bits on every run. The global
// inputs of phases 1 and 2 (element connectivity and coefficient, row
// extents and slot records) are loaded at the start, so that their latency
// hides behind phase 0.
//
// T = double: plain FP64. T = gbfem::Dd: FP64-accurate double-float on the
// FP32 pipe; the only FP64 instructions are the four coordinate differences
// per element (they carry the mesh scale exactly), every conversion runs on
// the integer pipe (ddSplitInt / ddJoinInt). T = float: FP32 element
// arithmetic, edge vectors from an exact split of the coordinates (no FP64
// instruction), FP64 outputs.
//
// Element formulas (edge vectors a = x1 - x0, b = x2 - x0, c = b - a):
//   det = a x b,  s = kappa / (2 |det|)
//   K01 = -s b.c,  K02 = s a.c,  K12 = -s a.b   (the cotangent weights)
//   residual: r0 = K01 (u1-u0) + K02 (u2-u0), r1 = K12 (u2-u1) - K01 (u1-u0),
//             r2 = -(K02 (u2-u0) + K12 (u2-u1)), minus the load
//             F_i = |det|/24 (f_i + f0 + f1 + f2) (the order-2 rule is exact
//             for the P1-interpolated source).
#pragma once

#include <type_traits>

#include "dfloat.cuh"
#include "maps.cuh"

namespace
{
using gbfem::Dd;

struct P1TileArgs
{
  const int*           row_off;
  const int4*          row_info;
  const int*           run_off;
  const int4*          runs;
  const int*           elem_off;
  const int*           elems;
  const unsigned*      tconn;
  const int*           vert_off;
  const int*           vert_dof;
  const int*           vert_node;
  const unsigned*      slot_ref;
  const double2*       coords;
  const double*        kappa;
  const double*        f;
  const double*        u;
  double*              res;
  double*              vals;
  const double*        u_state; // residual VJP: the state (u is then the adjoint)
  double*              g_m;     // residual VJP: per-element control gradient
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

// the leading part, compared in its own type (a widening to double would be
// a conversion on GB300's slow FP64 pipe)
__device__ __forceinline__ double tLead(double x)
{
  return x;
}
__device__ __forceinline__ float tLead(float x)
{
  return x;
}
__device__ __forceinline__ float tLead(Dd x)
{
  return x.hi;
}

template <class T>
__device__ __forceinline__ T tAbs(T x)
{
  return tLead(x) < 0.0f ? -x : x;
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

// x split exactly into three floats on the integer pipe: the leading 24
// significant bits, the next 23 and the last 6 (the x, y, z members), each
// lower part placed under an implicit one that is subtracted again in FP32
// (exact). Finite |x| in [2^-80, 2^127) splits exactly; smaller parts become
// 0 below that (an absolute error under 2^-132). The FP32 kernel forms its
// edge vectors from the leading two parts, (a.x - b.x) + (a.y - b.y): the
// mesh scale survives the subtraction of nearby coordinates.
__device__ __forceinline__ float3 split3Int(double x)
{
  const unsigned hi32 = static_cast<unsigned>(__double2hiint(x));
  const unsigned lo32 = static_cast<unsigned>(__double2loint(x));
  const unsigned sgn  = hi32 & 0x80000000u;
  const unsigned ax   = hi32 & 0x7fffffffu;
  const unsigned e    = ax >> 20;
  if (e >= 1150u)
  {
    return make_float3(gbfem::f64ToF32(x), 0.0f, 0.0f);
  }
  const unsigned hb = sgn | __funnelshift_l(lo32, ax - 0x38000000u, 3);
  const unsigned e2 = (e - 919u) << 23, e3 = (e - 942u) << 23;
  const float    a2 = __fsub_rn(__uint_as_float(sgn | e2 | ((lo32 >> 6) & 0x7fffffu)),
                                __uint_as_float(sgn | e2));
  const float    a3 = __fsub_rn(__uint_as_float(sgn | e3 | ((lo32 & 0x3fu) << 17)),
                                __uint_as_float(sgn | e3));
  return make_float3(e > 896u ? __uint_as_float(hb) : 0.0f, e >= 920u ? a2 : 0.0f,
                     e >= 943u ? a3 : 0.0f);
}

// Coordinates as staged in shared memory: FP64 for the FP64 and the
// double-float kernels (their edge vectors are four FP64 subtractions, which
// the otherwise idle FP64 pipe absorbs more cheaply than an exact float
// difference costs in issue slots), the leading two parts of the exact split
// for the FP32 kernel.
template <class T>
struct VertXY
{
  double2 p;
};
template <>
struct VertXY<float>
{
  float2 x, y;
};

template <class T>
__device__ __forceinline__ VertXY<T> stageXY(double2 p)
{
  return VertXY<T>{p};
}
template <>
__device__ __forceinline__ VertXY<float> stageXY<float>(double2 p)
{
  const float3 x = split3Int(p.x), y = split3Int(p.y);
  return VertXY<float>{make_float2(x.x, x.y), make_float2(y.x, y.y)};
}

// the edge vector x_j - x_i in T
template <class T>
__device__ __forceinline__ void edge(const VertXY<T>& i, const VertXY<T>& j, T& dx, T& dy);
template <>
__device__ __forceinline__ void edge<double>(const VertXY<double>& i, const VertXY<double>& j,
                                             double& dx, double& dy)
{
  dx = j.p.x - i.p.x;
  dy = j.p.y - i.p.y;
}
template <>
__device__ __forceinline__ void edge<Dd>(const VertXY<Dd>& i, const VertXY<Dd>& j, Dd& dx,
                                         Dd& dy)
{
  dx = gbfem::ddSplitInt(j.p.x - i.p.x);
  dy = gbfem::ddSplitInt(j.p.y - i.p.y);
}
template <>
__device__ __forceinline__ void edge<float>(const VertXY<float>& i, const VertXY<float>& j,
                                            float& dx, float& dy)
{
  dx = __fsub_rn(j.x.x, i.x.x) + __fsub_rn(j.x.y, i.x.y);
  dy = __fsub_rn(j.y.x, i.y.x) + __fsub_rn(j.y.y, i.y.y);
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

constexpr int kTileThreads = 256; // rows per tile at most; elements at most twice that
constexpr int kRowPrefetch = 8;   // slot records of a row held in registers

__host__ __device__ constexpr int align16(int b)
{
  return (b + 15) & ~15;
}

// Row output: staged in shared memory and written out in coalesced runs
// (FP32 and FP64 kernels, which wait on memory), or stored directly from the
// row phase (double-float kernel, which is bound by instruction issue and
// pays more for the extra phase than for scattered stores).
template <class T>
constexpr bool tileStaged()
{
  return !std::is_same<T, Dd>::value;
}

// Shared-memory layout of a block (sizes from the map's largest tile): the
// edge records and the runs live through the whole kernel; the staged
// vertices (phases 0-1) and the staged row values (phases 2-3) share one
// region, separated by the barrier after phase 1.
template <class T>
struct TileSmem
{
  int e, runs, xy, u, f, v, r, total;
  __host__ __device__ TileSmem(int verts, int elems, int slots, int rows, int runs_, bool load)
  {
    if (!tileStaged<T>())
    {
      slots = rows = runs_ = 0;
    }
    e              = 0;
    runs           = align16(e + 3 * elems * static_cast<int>(sizeof(EdgeRec<T>)));
    xy             = align16(runs + runs_ * static_cast<int>(sizeof(int4)));
    u              = align16(xy + verts * static_cast<int>(sizeof(VertXY<T>)));
    f              = align16(u + verts * static_cast<int>(sizeof(T)));
    const int vend = align16(f + (load ? verts * static_cast<int>(sizeof(T)) : 0));
    v              = xy;
    r              = align16(v + slots * static_cast<int>(sizeof(double)));
    const int rend = align16(r + rows * static_cast<int>(sizeof(double)));
    total          = vend > rend ? vend : rend;
  }
};

// Resident blocks per SM the register allocation is held to (measured on
// the 1024x1024 benchmark mesh): five for the issue-bound double-float
// kernel (48 registers; 101 -> 91 us against the unbounded 57), six for the
// latency-bound FP32 kernel (40 registers; 81 -> 70 us), three for the
// FP64-pipe-bound FP64 kernel.
template <class T>
constexpr int tileMinBlocks()
{
  return std::is_same<T, Dd>::value ? 5 : (std::is_same<T, float>::value ? 6 : 3);
}

// kVjp: the residual VJPs instead (no load, no Jacobian): u holds the
// adjoint lambda, u_state the state; the row phase sums (K lambda)_r into
// res (= g_u) and each element's owner tile writes g_m[e] = lambda_e^T K_e
// u_e = -sum over its edges of K_ab (lambda_a - lambda_b)(u_a - u_b).
template <class T, bool kLoad, bool kJac, bool kVjp = false>
__global__ void __launch_bounds__(kTileThreads, tileMinBlocks<T>())
    p1TiledKernel(P1TileArgs a, int max_verts, int max_elems, int max_slots, int max_runs)
{
  static_assert(!kVjp || (!kLoad && !kJac), "the VJP form has no load and no Jacobian");
  constexpr bool kStage  = tileStaged<T>();
  constexpr bool kSecond = kLoad || kVjp; // a second staged vertex field
  extern __shared__ __align__(16) unsigned char smem[];
  const TileSmem<T> L(max_verts, max_elems, max_slots, kTileThreads, max_runs, kSecond);
  VertXY<T>*        sx = reinterpret_cast<VertXY<T>*>(smem + L.xy);
  T*                su = reinterpret_cast<T*>(smem + L.u);
  T*                sf = reinterpret_cast<T*>(smem + L.f);
  EdgeRec<T>*       se = reinterpret_cast<EdgeRec<T>*>(smem + L.e);
  double*           sv = reinterpret_cast<double*>(smem + L.v);
  double*           sr = reinterpret_cast<double*>(smem + L.r);
  int4*             sq = reinterpret_cast<int4*>(smem + L.runs);

  const int t   = blockIdx.x;
  const int i   = threadIdx.x;
  const int v0  = a.vert_off[t];
  const int nv  = a.vert_off[t + 1] - v0;
  const int e0  = a.elem_off[t];
  const int nel = a.elem_off[t + 1] - e0;
  const int r0  = a.row_off[t];
  const int nr  = a.row_off[t + 1] - r0;
  const int q0  = a.run_off[t];
  const int nq  = a.run_off[t + 1] - q0;

  // phase 1 and 2 inputs, loaded first (latency hidden behind phase 0)
  int4 row = make_int4(0, 0, 0, 0);
  if (i < nr)
  {
    row = a.row_info[r0 + i];
  }
  unsigned w[kRowPrefetch];
#pragma unroll
  for (int k = 0; k < kRowPrefetch; ++k)
  {
    w[k] = row.y + k < row.z ? a.slot_ref[row.y + k] : 0u;
  }
  unsigned ec[2];
  int      eg[2];
  double   ek[2];
#pragma unroll
  for (int h = 0; h < 2; ++h)
  {
    const int l = i + h * kTileThreads;
    ec[h]       = l < nel ? a.tconn[e0 + l] : 0u;
    eg[h]       = l < nel ? a.elems[e0 + l] : 0;
    ek[h]       = l < nel ? a.kappa[eg[h]] : 0.0;
  }
  const int4 run = kStage && i < nq ? a.runs[q0 + i] : make_int4(0, 0, 0, 0);

  // 0. vertices
  for (int j = i; j < nv; j += kTileThreads)
  {
    const int d = a.vert_dof[v0 + j];
    const int n = a.vert_node[v0 + j];
    sx[j]       = stageXY<T>(a.coords[n]);
    su[j]       = tSplit<T>(a.u[d]);
    if (kLoad)
    {
      sf[j] = tSplit<T>(a.f[n]);
    }
    if (kVjp)
    {
      sf[j] = tSplit<T>(a.u_state[d]);
    }
  }
  if (kStage && i < nq)
  {
    sq[i] = run;
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
    const unsigned c  = ec[h];
    const int      i0 = c & 1023u, i1 = (c >> 10) & 1023u, i2 = (c >> 20) & 1023u;
    T              ax, ay, bx, by;
    edge<T>(sx[i0], sx[i1], ax, ay);
    edge<T>(sx[i0], sx[i2], bx, by);
    const T det  = tDot2(ax, by, -bx, ay);
    T       adet = tAbs(det);
    if (!(tLead(adet) >= 1.0e-30f))
    {
      gbfem::devFail(a.status, gbfem::kDevSingularJacobian, eg[h]);
      adet = T(1);
    }
    const T s   = tScale(tSplit<T>(ek[h]) * tRcp(adet), 0.5f);
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
    if (kVjp && (c & 0x40000000u) && a.g_m != nullptr)
    {
      // this tile owns the element (its first vertex's row)
      const T w0 = sf[i0], w1 = sf[i1], w2 = sf[i2];
      a.g_m[eg[h]] = tJoin(-(P * (w1 - w0) + Q * (w2 - w0) + R * (w2 - w1)));
    }
    se[3 * l + 0] = EdgeRec<T>{k12, rr1};
    se[3 * l + 1] = EdgeRec<T>{k02, rr2};
    se[3 * l + 2] = EdgeRec<T>{k01, rr0};
  }
  __syncthreads();

  // 2. rows, staged in shared memory
  if (i < nr && (!kVjp || a.res != nullptr))
  {
    T    off = T(0), res = T(0);
    int  dk  = -1;
    auto slot = [&](int k, unsigned wk) {
      if (wk == 0xffffffffu)
      {
        dk = k;
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
        if (kStage)
        {
          sv[row.w + k] = tJoin(K);
        }
        else
        {
          a.vals[row.y + k] = tJoin(K);
        }
      }
    };
    const int len = row.z - row.y;
#pragma unroll
    for (int k = 0; k < kRowPrefetch; ++k)
    {
      if (k < len)
      {
        slot(k, w[k]);
      }
    }
    for (int k = kRowPrefetch; k < len; ++k)
    {
      slot(k, a.slot_ref[row.y + k]);
    }
    if (kJac && dk >= 0)
    {
      if (kStage)
      {
        sv[row.w + dk] = tJoin(-tNorm(off));
      }
      else
      {
        a.vals[row.y + dk] = tJoin(-tNorm(off));
      }
    }
    if (kStage)
    {
      sr[i] = tJoin(tNorm(res));
    }
    else
    {
      a.res[row.x] = tJoin(tNorm(res));
    }
  }
  if (!kStage)
  {
    return;
  }
  __syncthreads();

  // 3. coalesced write-out, one warp per run of consecutive rows
  const int warp = i >> 5, lane = i & 31;
  for (int q = warp; q < nq - 1; q += kTileThreads / 32)
  {
    const int4 b = sq[q], n = sq[q + 1];
    if (kJac)
    {
      for (int j = lane; j < n.w - b.w; j += 32)
      {
        a.vals[b.z + j] = sv[b.w + j];
      }
    }
    for (int j = lane; j < n.y - b.y; j += 32)
    {
      a.res[b.x + j] = sr[b.y + j];
    }
  }
}

// Launch over all tiles of the map (gbfem_assembly_map_enable_tiles).
template <class T, bool kLoad, bool kJac, bool kVjp = false>
void launchP1Tiled(const P1TileArgs& a, const gbfem_assembly_map* m, cudaStream_t s)
{
  const TileSmem<T> L(m->tile_max_verts, m->tile_max_elems, m->tile_max_slots, kTileThreads,
                      m->tile_max_runs, kLoad || kVjp);
  if (L.total > 48 * 1024)
  {
    gbfem::cudaCheck(cudaFuncSetAttribute(p1TiledKernel<T, kLoad, kJac, kVjp>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, L.total),
                     "tiled assembly shared memory");
  }
  if (m->num_tiles > 0)
  {
    p1TiledKernel<T, kLoad, kJac, kVjp><<<m->num_tiles, kTileThreads, L.total, s>>>(
        a, m->tile_max_verts, m->tile_max_elems, m->tile_max_slots, m->tile_max_runs);
  }
}

} // namespace
