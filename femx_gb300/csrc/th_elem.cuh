// th_elem.cuh — device code of the Taylor-Hood P2/P1 element, shared by the
// standalone assembly kernel (th.cu) and the batched persistent kernel
// (batch.cu). See th.cu for the formulation.
#pragma once

#include <type_traits>

#include "dfloat.cuh"
#include "maps.cuh"

namespace
{
using gbfem::DeviceStatus;

constexpr int kLanes         = 16;
constexpr int kElemsPerBlock = 8;
constexpr int kThreads       = kLanes * kElemsPerBlock;
constexpr int kNq            = 6;

// 16-byte aligned with a size that is a multiple of 16 bytes (456 values),
// so that one bulk copy stages a table in shared memory.
template <class R>
struct alignas(16) ThRef
{
  R N[kNq][6];       // P2 values at the quadrature points
  R wN[kNq][6];      // w_q N^_a(q)
  R dNr[kNq][6][2];  // P2 reference gradients at the quadrature points
  R S00[6][6], S11[6][6], S01[6][6]; // S^00, S^11, S^01 + S^10
  R T[3][6][6];      // sum_q w N^_a N^_b lambda_v
  R C[2][6][3];      // sum_q w psi^_b dN^_a,k
  R dNv[3][6][2];    // P2 reference gradients at the vertices
  R P[kNq][3];       // P1 (pressure) values at the quadrature points
  R w[kNq];
};

constexpr void p2Eval(double r, double s, double* N, double* dN)
{
  const double l0 = 1.0 - r - s, l1 = r, l2 = s;
  const double g0[2] = {-1.0, -1.0}, g1[2] = {1.0, 0.0}, g2[2] = {0.0, 1.0};
  N[0] = l0 * (2.0 * l0 - 1.0);
  N[1] = l1 * (2.0 * l1 - 1.0);
  N[2] = l2 * (2.0 * l2 - 1.0);
  N[3] = 4.0 * l0 * l1;
  N[4] = 4.0 * l1 * l2;
  N[5] = 4.0 * l2 * l0;
  for (int d = 0; d < 2; ++d)
  {
    dN[0 * 2 + d] = (4.0 * l0 - 1.0) * g0[d];
    dN[1 * 2 + d] = (4.0 * l1 - 1.0) * g1[d];
    dN[2 * 2 + d] = (4.0 * l2 - 1.0) * g2[d];
    dN[3 * 2 + d] = 4.0 * (l1 * g0[d] + l0 * g1[d]);
    dN[4 * 2 + d] = 4.0 * (l2 * g1[d] + l1 * g2[d]);
    dN[5 * 2 + d] = 4.0 * (l0 * g2[d] + l2 * g0[d]);
  }
}

constexpr ThRef<double> makeRef()
{
  ThRef<double> t{};
  const double  a1 = 0.445948490915964886, w1 = 0.223381589678011466 * 0.5;
  const double  a2 = 0.091576213509770743, w2 = 0.109951743655321868 * 0.5;
  const double  q[kNq][3] = {{a1, a1, w1}, {1.0 - 2.0 * a1, a1, w1},
                            {a1, 1.0 - 2.0 * a1, w1}, {a2, a2, w2},
                            {1.0 - 2.0 * a2, a2, w2}, {a2, 1.0 - 2.0 * a2, w2}};
  const double  dP[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
  double        lam[kNq][3]{};
  for (int i = 0; i < kNq; ++i)
  {
    double N[6]{}, dN[12]{};
    p2Eval(q[i][0], q[i][1], N, dN);
    lam[i][0] = 1.0 - q[i][0] - q[i][1];
    lam[i][1] = q[i][0];
    lam[i][2] = q[i][1];
    t.P[i][0] = lam[i][0];
    t.P[i][1] = lam[i][1];
    t.P[i][2] = lam[i][2];
    t.w[i]    = q[i][2];
    for (int a = 0; a < 6; ++a)
    {
      t.N[i][a]      = N[a];
      t.wN[i][a]     = q[i][2] * N[a];
      t.dNr[i][a][0] = dN[2 * a];
      t.dNr[i][a][1] = dN[2 * a + 1];
    }
  }
  for (int a = 0; a < 6; ++a)
  {
    for (int b = 0; b < 6; ++b)
    {
      double s00 = 0.0, s11 = 0.0, s01 = 0.0;
      double tv[3] = {0.0, 0.0, 0.0};
      for (int i = 0; i < kNq; ++i)
      {
        const double w = t.w[i];
        s00 += w * t.dNr[i][a][0] * t.dNr[i][b][0];
        s11 += w * t.dNr[i][a][1] * t.dNr[i][b][1];
        s01 += w * (t.dNr[i][a][0] * t.dNr[i][b][1] + t.dNr[i][a][1] * t.dNr[i][b][0]);
        for (int v = 0; v < 3; ++v)
        {
          tv[v] += w * t.N[i][a] * t.N[i][b] * lam[i][v];
        }
      }
      t.S00[a][b] = s00;
      t.S11[a][b] = s11;
      t.S01[a][b] = s01;
      for (int v = 0; v < 3; ++v)
      {
        t.T[v][a][b] = tv[v];
      }
    }
    for (int b = 0; b < 3; ++b)
    {
      for (int k = 0; k < 2; ++k)
      {
        double c = 0.0;
        for (int i = 0; i < kNq; ++i)
        {
          c += t.w[i] * lam[i][b] * t.dNr[i][a][k];
        }
        t.C[k][a][b] = c;
      }
    }
  }
  const double vx[3][2] = {{0.0, 0.0}, {1.0, 0.0}, {0.0, 1.0}};
  for (int v = 0; v < 3; ++v)
  {
    double N[6]{}, dN[12]{};
    p2Eval(vx[v][0], vx[v][1], N, dN);
    for (int s = 0; s < 6; ++s)
    {
      t.dNv[v][s][0] = dN[2 * s];
      t.dNv[v][s][1] = dN[2 * s + 1];
    }
  }
  (void)dP;
  return t;
}

template <class R>
constexpr R refCast(double d)
{
  return static_cast<R>(d);
}
template <>
constexpr gbfem::DF refCast<gbfem::DF>(double d)
{
  return gbfem::dfConst(d);
}
template <>
constexpr gbfem::Dd refCast<gbfem::Dd>(double d)
{
  return gbfem::Dd(d);
}

template <class R>
constexpr ThRef<R> castRef()
{
  const ThRef<double> d = makeRef();
  ThRef<R>            r{};
  for (int q = 0; q < kNq; ++q)
  {
    r.w[q] = refCast<R>(d.w[q]);
    for (int b = 0; b < 3; ++b)
    {
      r.P[q][b] = refCast<R>(d.P[q][b]);
    }
    for (int a = 0; a < 6; ++a)
    {
      r.N[q][a]      = refCast<R>(d.N[q][a]);
      r.wN[q][a]     = refCast<R>(d.wN[q][a]);
      r.dNr[q][a][0] = refCast<R>(d.dNr[q][a][0]);
      r.dNr[q][a][1] = refCast<R>(d.dNr[q][a][1]);
    }
  }
  for (int a = 0; a < 6; ++a)
  {
    for (int b = 0; b < 6; ++b)
    {
      r.S00[a][b] = refCast<R>(d.S00[a][b]);
      r.S11[a][b] = refCast<R>(d.S11[a][b]);
      r.S01[a][b] = refCast<R>(d.S01[a][b]);
      for (int v = 0; v < 3; ++v)
      {
        r.T[v][a][b] = refCast<R>(d.T[v][a][b]);
      }
    }
    for (int b = 0; b < 3; ++b)
    {
      r.C[0][a][b] = refCast<R>(d.C[0][a][b]);
      r.C[1][a][b] = refCast<R>(d.C[1][a][b]);
    }
  }
  for (int v = 0; v < 3; ++v)
  {
    for (int s2 = 0; s2 < 6; ++s2)
    {
      r.dNv[v][s2][0] = refCast<R>(d.dNv[v][s2][0]);
      r.dNv[v][s2][1] = refCast<R>(d.dNv[v][s2][1]);
    }
  }
  return r;
}

__device__ const ThRef<double> kRefD = makeRef();
__device__ const ThRef<float>  kRefF = castRef<float>();

__device__ __forceinline__ const ThRef<double>* refTables(double)
{
  return &kRefD;
}
__device__ __forceinline__ const ThRef<float>* refTables(float)
{
  return &kRefF;
}

// Lane shuffle within an element's 16 lanes.
template <class T>
__device__ __forceinline__ T laneShfl(T v, int src)
{
  return __shfl_sync(0xffffffffu, v, src, kLanes);
}

// acc + x y: a fused multiply-add in float and double; in double-float the
// Dot2 accumulation of Ogita, Rump and Oishi (the product's leading part
// added by TwoSum, its rounding error and the cross terms collected in the
// trailing part, left unnormalised until accNorm).
__device__ __forceinline__ float mac(float acc, float x, float y)
{
  return acc + x * y;
}
__device__ __forceinline__ double mac(double acc, double x, double y)
{
  return acc + x * y;
}
__device__ __forceinline__ gbfem::Dd mac(gbfem::Dd acc, gbfem::Dd x, gbfem::Dd y)
{
  const float p  = __fmul_rn(x.hi, y.hi);
  const float pe = __fmaf_rn(x.hi, y.hi, -p);
  const float s  = __fadd_rn(acc.hi, p);
  const float bb = __fsub_rn(s, acc.hi);
  const float se = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  float       lo = __fadd_rn(acc.lo, __fadd_rn(se, pe));
  lo             = __fmaf_rn(x.hi, y.lo, lo);
  lo             = __fmaf_rn(x.lo, y.hi, lo);
  return {s, lo};
}
__device__ __forceinline__ float accNorm(float x)
{
  return x;
}
__device__ __forceinline__ double accNorm(double x)
{
  return x;
}
__device__ __forceinline__ gbfem::Dd accNorm(gbfem::Dd x)
{
  const gbfem::DF t = gbfem::dfTwoSum(x.hi, x.lo);
  return {t.hi, t.lo};
}

struct ThArgs
{
  int                  ne;
  int                  num_nodes;
  const int*           dofs;  // [ne][15]
  const int*           conn6; // [ne][6]
  const double2*       coords;
  double               nu;
  const double*        state;
  const int*           row_ptr;
  const unsigned char* jac_pos; // [ne][15][16] or null
  const int*           jac_map; // fallback
  double*              res;
  double*              vals;
  const double*        lam;     // adjoint for the fused state VJP, or null
  double*              g_state; // J^T lam accumulated here when lam != null
  DeviceStatus*        status;
  // row-gather output (kGather): record index of element row (e, l), the
  // records' 16 values (float or double) and residual terms
  const int*           gslot;
  void*                geb;
  double*              gres;
  // coloured pass: the colour's element list (ne = its length), or null
  const int*           elems;
};

template <class T>
struct ElemShared
{
  T   st[16];
  T   aInvJ[4];  // |det| * J^-1
  T   invJ[4];
  T   G3[3];     // nu |det| (J^-1 J^-T): 00, 11, 01
  T   ut[kNq][2];
  T   vq[kNq][6]; // |det| dN^_b(q) . ut_q
  T   Gv[3][4];   // |det| grad u at the vertices, [v][c*2+e]
  int ok;
  // pads the record to 16 words mod 32, so that the two elements of a warp
  // (lanes 0-15 and 16-31) write lane-consecutive fields into disjoint banks
  int pad[sizeof(T) == 4 ? 24 : 1];
};
static_assert(sizeof(ElemShared<float>) % 128 == 64 && sizeof(ElemShared<double>) % 128 == 64,
              "element record stride must be 16 words mod 32");

// FP64 residual by direct quadrature (MIXED mode): state, geometry and the
// per-quadrature-point reference-coordinate fluxes Ft[q][c][k], sources
// src[q][c] and weighted divergence dq[q] of one element.
struct Res64
{
  double st[16];
  double invJ[4];
  double ad;
  double Ft[kNq][2][2];
  double src[kNq][2];
  double dq[kNq];
};

// Shared memory of one 128-thread block working on up to 8 elements.
template <class T>
struct alignas(16) ThSmem
{
  ThRef<T>      ref;
  unsigned long long bar; // completion of the reference tables' bulk copy
  ElemShared<T> sh[kElemsPerBlock];
  // Each element's 15x15 block staged row by row (row stride 17, element
  // stride 272 = 16 mod 32 words) so that both the row-wise writes and the
  // column-wise reads of the two elements of a warp are free of bank
  // conflicts, and the start of every row's CSR segment.
  T   outv[kElemsPerBlock][16][17];
  int rs[kElemsPerBlock][16];
  T   lam[kElemsPerBlock][16];
};

// MIXED mode adds the FP64 residual staging.
template <class T>
struct ThSmemMixed : ThSmem<T>
{
  Res64 r64[kElemsPerBlock];
};

// Stages the reference tables in shared memory: one bulk copy by the tensor
// memory accelerator when a status word is given (a timed-out wait is
// reported there), a block-wide copy loop otherwise. Follow with
// __syncthreads before thBlock.
template <class T>
__device__ __forceinline__ void thStageRef(ThSmem<T>& sm, DeviceStatus* status = nullptr)
{
  static_assert(sizeof(ThRef<T>) % 16 == 0, "bulk copies move multiples of 16 bytes");
  if (status != nullptr)
  {
    if (!gbfem::bulkStage(&sm.ref, refTables(T()), sizeof(ThRef<T>), &sm.bar)
        && threadIdx.x == 0)
    {
      gbfem::devFail(status, gbfem::kDevStageTimeout, blockIdx.x);
    }
    return;
  }
  const T* src = reinterpret_cast<const T*>(refTables(T()));
  T*       dst = reinterpret_cast<T*>(&sm.ref);
  for (int i = threadIdx.x; i < int(sizeof(ThRef<T>) / sizeof(T)); i += kThreads)
  {
    dst[i] = src[i];
  }
}

// FP64 residual of local row l from the staged quadrature-point fluxes.
__device__ __forceinline__ double rowRes64(const Res64& R, int l)
{
  const ThRef<double>& rd = kRefD;
  double               r6 = 0;
  if (l < 12)
  {
    const int sa = l >> 1, cc = l & 1;
#pragma unroll
    for (int q = 0; q < kNq; ++q)
    {
      r6 += R.Ft[q][cc][0] * rd.dNr[q][sa][0] + R.Ft[q][cc][1] * rd.dNr[q][sa][1]
            + R.src[q][cc] * rd.N[q][sa];
    }
  }
  else
  {
#pragma unroll
    for (int q = 0; q < kNq; ++q)
    {
      r6 -= rd.P[q][l - 12] * R.dq[q];
    }
  }
  return r6;
}

// One 16-value record, 16-byte aligned: vector stores.
__device__ __forceinline__ void storeRecord(float* dst, const float (&v)[16])
{
  float4* d = reinterpret_cast<float4*>(dst);
#pragma unroll
  for (int i = 0; i < 4; ++i)
  {
    d[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
  }
}
__device__ __forceinline__ void storeRecord(double* dst, const double (&v)[16])
{
  double2* d = reinterpret_cast<double2*>(dst);
#pragma unroll
  for (int i = 0; i < 8; ++i)
  {
    d[i] = make_double2(v[2 * i], v[2 * i + 1]);
  }
}

// The whole block works on elements [e_base, e_base + 8). Call from every
// thread of a kThreads-wide block after thStageRef + __syncthreads.
// kRes64 (with kRes = false): the residual is evaluated in FP64 by direct
// quadrature alongside the T-precision Jacobian (the MIXED Newton scheme):
//   R_(a,c) = sum_q [ Ft_c(q) . dN^_a(q) + src_c(q) N^_a(q) ],
//   Ft_c = J^-1 W (nu grad u_c - p e_c),  src_c = W u . grad u_c,
//   R_p(b)  = -sum_q psi^_b(q) W div u(q).
template <class T, bool kJac, bool kRes, bool kVjp, bool kRes64 = false, bool kGather = false,
          bool kPlain = false>
__device__ __forceinline__ void thBlock(const ThArgs& a, int e_base, ThSmem<T>& sm)
{
  static_assert(!(kRes && kRes64), "one residual precision at a time");
  static_assert(!(kGather && kVjp), "the fused VJP scatters its column sums");
  static_assert(!(kGather && kPlain), "one output scheme at a time");
  const ThRef<T>& ref = sm.ref;
  const int       l   = threadIdx.x & (kLanes - 1);
  const int       le  = threadIdx.x / kLanes;
  // element slot e_base + le of this launch: an element index, or, in a
  // coloured pass, an index into the colour's element list
  const int       idx = e_base + le;
  const bool      has = idx < a.ne;
  const int       e   = (kPlain && has) ? a.elems[idx] : idx;
  ElemShared<T>&  S   = sm.sh[le];

  Res64* R64 = nullptr;
  if constexpr (kRes64)
  {
    R64 = &static_cast<ThSmemMixed<T>&>(sm).r64[le];
  }
  // Every global load whose address is known up front is issued here, so
  // that the row-pointer and position loads (which depend on the dof load)
  // overlap the geometry and quadrature work instead of following it.
  int   h_rs  = 0;
  uint4 h_pos = make_uint4(0, 0, 0, 0);
  if (has && l < 15)
  {
    const int hd = a.dofs[15 * e + l];
    if (kJac && !kGather)
    {
      h_rs = a.row_ptr[hd];
      if (a.jac_pos != nullptr)
      {
        h_pos = *reinterpret_cast<const uint4*>(a.jac_pos + (15LL * e + l) * 16);
      }
    }
    const double sv = a.state[hd];
    S.st[l]         = gbfem::fromF64<T>(sv);
    if (kRes64)
    {
      R64->st[l] = sv;
    }
    if (kVjp)
    {
      sm.lam[le][l] = gbfem::fromF64<T>(a.lam[a.dofs[15 * e + l]]);
    }
  }
  // Geometry, spread over the element's lanes: lanes 0-5 check one
  // connectivity entry each, lanes 0-2 load their vertex, lanes 1 and 2 form
  // the FP64 edge vectors x_v - x_0 (they carry the mesh scale) and convert
  // them; lane 15 forms the inverse Jacobian from the shuffled edges and
  // stores it. Every lane runs the shuffles (the warp is converged here).
  constexpr unsigned kAll = 0xffffffffu;
  int                node = 0;
  bool               bad  = false;
  if (has && l < 6)
  {
    node = a.conn6[6 * e + l];
    bad  = static_cast<unsigned>(node) >= static_cast<unsigned>(a.num_nodes);
  }
  const bool nodes_ok = ((__ballot_sync(kAll, bad) >> (threadIdx.x & 16)) & 0x3fu) == 0u;
  double2    xv       = make_double2(0.0, 0.0);
  if (has && nodes_ok && l < 3)
  {
    xv = a.coords[node];
  }
  const double dex = xv.x - __shfl_sync(kAll, xv.x, 0, kLanes);
  const double dey = xv.y - __shfl_sync(kAll, xv.y, 0, kLanes);
  const T      ex = gbfem::fromF64<T>(dex), ey = gbfem::fromF64<T>(dey);
  // J[a][b] = d x_a / d r_b of the affine map (vertex nodes)
  const T j00 = laneShfl(ex, 1), j10 = laneShfl(ey, 1);
  const T j01 = laneShfl(ex, 2), j11 = laneShfl(ey, 2);
  double  dj[4] = {0.0, 0.0, 0.0, 0.0}; // FP64 edges, for the FP64 residual only
  if constexpr (kRes64)
  {
    dj[0] = __shfl_sync(kAll, dex, 1, kLanes);
    dj[1] = __shfl_sync(kAll, dex, 2, kLanes);
    dj[2] = __shfl_sync(kAll, dey, 1, kLanes);
    dj[3] = __shfl_sync(kAll, dey, 2, kLanes);
  }
  if (has && l == 15)
  {
    S.ok = 0;
    if (!nodes_ok)
    {
      gbfem::devFail(a.status, gbfem::kDevNodeRange, e);
    }
    else
    {
      if constexpr (kRes64)
      {
        const double ddet = dj[0] * dj[3] - dj[1] * dj[2];
        const double dinv = gbfem::rcpF64(ddet);
        R64->invJ[0]       = dj[3] * dinv;
        R64->invJ[1]       = -dj[1] * dinv;
        R64->invJ[2]       = -dj[2] * dinv;
        R64->invJ[3]       = dj[0] * dinv;
        R64->ad            = fabs(ddet);
      }
      const T det = j00 * j11 - j01 * j10;
      const T ad  = det < T(0) ? -det : det;
      if (ad >= T(1.0e-30))
      {
        S.ok        = 1;
        T inv;
        if constexpr (std::is_same<T, double>::value)
        {
          inv = gbfem::rcpF64(det);
        }
        else
        {
          inv = T(1) / det;
        }
        const T i00 = j11 * inv, i01 = -j01 * inv;
        const T i10 = -j10 * inv, i11 = j00 * inv;
        S.invJ[0]   = i00;
        S.invJ[1]   = i01;
        S.invJ[2]   = i10;
        S.invJ[3]   = i11;
        S.aInvJ[0]  = ad * i00;
        S.aInvJ[1]  = ad * i01;
        S.aInvJ[2]  = ad * i10;
        S.aInvJ[3]  = ad * i11;
        const T nad = gbfem::fromF64<T>(a.nu) * ad;
        S.G3[0]     = nad * (i00 * i00 + i01 * i01);
        S.G3[1]     = nad * (i10 * i10 + i11 * i11);
        S.G3[2]     = nad * (i00 * i10 + i01 * i11);
      }
      else
      {
        gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
      }
    }
  }
  __syncthreads();
  const bool live = has && S.ok;
  if (live && l < 12)
  {
    // |det| grad u at vertex v: [c][e] = sum_k aInvJ[k][e] sum_s u_(s,c) dNv
    const int v = l >> 2, c = (l >> 1) & 1, ee = l & 1;
    T         g0 = 0, g1 = 0;
#pragma unroll
    for (int s2 = 0; s2 < 6; ++s2)
    {
      const T us = S.st[2 * s2 + c];
      g0 += us * ref.dNv[v][s2][0];
      g1 += us * ref.dNv[v][s2][1];
    }
    S.Gv[v][c * 2 + ee] = g0 * S.aInvJ[0 * 2 + ee] + g1 * S.aInvJ[1 * 2 + ee];
  }
  if (live && l < kNq)
  {
    const int q  = l;
    T         u0 = 0, u1 = 0;
#pragma unroll
    for (int s2 = 0; s2 < 6; ++s2)
    {
      u0 += ref.N[q][s2] * S.st[2 * s2];
      u1 += ref.N[q][s2] * S.st[2 * s2 + 1];
    }
    // ut_k = sum_d Jinv[k][d] u_d, so that u . dN_b = dN^_b . ut
    S.ut[q][0] = S.aInvJ[0] * u0 + S.aInvJ[1] * u1;
    S.ut[q][1] = S.aInvJ[2] * u0 + S.aInvJ[3] * u1;
  }
  if (kRes64 && live && l >= 6 && l < 6 + kNq)
  {
    // FP64 quadrature-point state and fluxes, reference tables from global
    const ThRef<double>& rd = kRefD;
    const int            q  = l - 6;
    double               u0 = 0, u1 = 0, r00 = 0, r01 = 0, r10 = 0, r11 = 0;
#pragma unroll
    for (int s2 = 0; s2 < 6; ++s2)
    {
      const double v0 = R64->st[2 * s2], v1 = R64->st[2 * s2 + 1];
      const double n = rd.N[q][s2], g0 = rd.dNr[q][s2][0], g1 = rd.dNr[q][s2][1];
      u0 += n * v0;
      u1 += n * v1;
      r00 += v0 * g0; // sum_s u_(s,c) dN^_s,k  as [c][k]
      r01 += v0 * g1;
      r10 += v1 * g0;
      r11 += v1 * g1;
    }
    const double* iJ = R64->invJ;
    // grad u_c [e] = sum_k r_ck invJ[k][e]
    const double G00 = r00 * iJ[0] + r01 * iJ[2], G01 = r00 * iJ[1] + r01 * iJ[3];
    const double G10 = r10 * iJ[0] + r11 * iJ[2], G11 = r10 * iJ[1] + r11 * iJ[3];
    double       pq  = 0;
#pragma unroll
    for (int b = 0; b < 3; ++b)
    {
      pq += rd.P[q][b] * R64->st[12 + b];
    }
    const double W   = rd.w[q] * R64->ad;
    const double nu  = a.nu;
    // physical fluxes W (nu grad u_c - p e_c), mapped by J^-1: Ft_c[k] =
    // sum_e invJ[k][e] F_c[e], so that F_c . dN_a = Ft_c . dN^_a
    const double F00 = W * (nu * G00 - pq), F01 = W * nu * G01;
    const double F10 = W * nu * G10, F11 = W * (nu * G11 - pq);
    R64->Ft[q][0][0] = iJ[0] * F00 + iJ[1] * F01;
    R64->Ft[q][0][1] = iJ[2] * F00 + iJ[3] * F01;
    R64->Ft[q][1][0] = iJ[0] * F10 + iJ[1] * F11;
    R64->Ft[q][1][1] = iJ[2] * F10 + iJ[3] * F11;
    R64->src[q][0]   = W * (u0 * G00 + u1 * G01);
    R64->src[q][1]   = W * (u0 * G10 + u1 * G11);
    R64->dq[q]       = W * (G00 + G11);
  }
  __syncthreads();
  if (live)
  {
    for (int i = l; i < kNq * 6; i += kLanes)
    {
      const int q = i / 6, b = i % 6;
      S.vq[q][b]  = ref.dNr[q][b][0] * S.ut[q][0] + ref.dNr[q][b][1] * S.ut[q][1];
    }
  }
  __syncthreads();
  const bool row_lane = live && l < 15;

  // Row l: velocity (sa, c) for l < 12, pressure b = l - 12 otherwise.
  // FP32 (kCompOrder): je[b] -> column (b, 0), jo[b] -> column (b, 1) on
  // every row, so that all lanes store column 2b, then 2b + 1: with the row
  // stride of 17 words those stores hit distinct banks for the two elements
  // of a warp. FP64 keeps the own/other-component order on velocity rows
  // (je -> (b, c), jo -> (b, 1 - c)), which needs fewer registers there.
  // jp[b] -> pressure column b.
  constexpr bool kCompOrder = sizeof(T) == 4;
  T              je[6], jo[6], jp[3] = {0, 0, 0};
  T   r = 0;
  int c = 0;
  // FP32: the scalar block da[sa][b] (diffusion + convection) is the same for
  // the two component rows 2sa and 2sa + 1, so each lane of the pair forms it
  // for the columns b = c, c + 2, c + 4 and takes the other three from its
  // partner. Every lane runs this (the shuffles need the whole warp); lanes of
  // pressure rows or rejected elements form values that are never used.
  T dsh[3] = {0, 0, 0}, dpt[3] = {0, 0, 0};
  if constexpr (kCompOrder)
  {
    const int sa = (l < 12 ? l : 0) >> 1, cb = l & 1;
#pragma unroll
    for (int j = 0; j < 3; ++j)
    {
      const int b  = 2 * j + cb;
      T         da = S.G3[0] * ref.S00[sa][b] + S.G3[1] * ref.S11[sa][b]
             + S.G3[2] * ref.S01[sa][b];
#pragma unroll
      for (int q = 0; q < kNq; ++q)
      {
        da += ref.wN[q][sa] * S.vq[q][b];
      }
      dsh[j] = da;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j)
    {
      dpt[j] = __shfl_xor_sync(kAll, dsh[j], 1);
    }
  }
  if (row_lane && l < 12)
  {
    const int sa = l >> 1;
    c            = l & 1;
    // kCompOrder: G0/G1 = grad u_c at the vertices, components 0 and 1, and
    // the scalar block da sits on the diagonal component (w0 = 1 for c = 0,
    // w1 = 1 for c = 1). Otherwise G0/G1 = own/other component.
    const int k0 = kCompOrder ? 0 : c, k1 = kCompOrder ? 1 : c ^ 1;
    const T   G0[3] = {S.Gv[0][c * 2 + k0], S.Gv[1][c * 2 + k0], S.Gv[2][c * 2 + k0]};
    const T   G1[3] = {S.Gv[0][c * 2 + k1], S.Gv[1][c * 2 + k1], S.Gv[2][c * 2 + k1]};
    const T   w0    = c == 0 ? T(1) : T(0), w1 = T(1) - w0;
    if constexpr (kCompOrder)
    {
#pragma unroll
      for (int b = 0; b < 6; ++b)
      {
        const T da = (b & 1) == c ? dsh[b >> 1] : dpt[b >> 1];
        const T m0 = ref.T[0][sa][b] * G0[0] + ref.T[1][sa][b] * G0[1]
                     + ref.T[2][sa][b] * G0[2];
        const T m1 = ref.T[0][sa][b] * G1[0] + ref.T[1][sa][b] * G1[1]
                     + ref.T[2][sa][b] * G1[2];
        je[b]      = da * w0 + m0;
        jo[b]      = da * w1 + m1;
        r += da * S.st[2 * b + c];
      }
    }
    else
    {
      // the scalar block da[b] = diffusion + convection of the six columns,
      // accumulated column-interleaved (six independent chains)
      T da[6];
#pragma unroll
      for (int b = 0; b < 6; ++b)
      {
        da[b] = S.G3[0] * ref.S00[sa][b];
      }
#pragma unroll
      for (int b = 0; b < 6; ++b)
      {
        da[b] = mac(mac(da[b], S.G3[1], ref.S11[sa][b]), S.G3[2], ref.S01[sa][b]);
      }
#pragma unroll
      for (int q = 0; q < kNq; ++q)
      {
#pragma unroll
        for (int b = 0; b < 6; ++b)
        {
          da[b] = mac(da[b], ref.wN[q][sa], S.vq[q][b]);
        }
      }
#pragma unroll
      for (int b = 0; b < 6; ++b)
      {
        da[b]    = accNorm(da[b]);
        T m0     = ref.T[0][sa][b] * G0[0], m1 = ref.T[0][sa][b] * G1[0];
        m0       = accNorm(mac(mac(m0, ref.T[1][sa][b], G0[1]), ref.T[2][sa][b], G0[2]));
        m1       = accNorm(mac(mac(m1, ref.T[1][sa][b], G1[1]), ref.T[2][sa][b], G1[2]));
        je[b]    = da[b] + m0;
        jo[b]    = m1;
        r        = mac(r, da[b], S.st[2 * b + c]);
      }
    }
    const T ic0 = S.aInvJ[0 * 2 + c], ic1 = S.aInvJ[1 * 2 + c];
#pragma unroll
    for (int b = 0; b < 3; ++b)
    {
      if constexpr (kCompOrder)
      {
        jp[b] = -(ic0 * ref.C[0][sa][b] + ic1 * ref.C[1][sa][b]);
        r += jp[b] * S.st[12 + b];
      }
      else
      {
        jp[b] = -accNorm(mac(ic0 * ref.C[0][sa][b], ic1, ref.C[1][sa][b]));
        r     = mac(r, jp[b], S.st[12 + b]);
      }
    }
    r = accNorm(r);
  }
  else if (row_lane)
  {
    const int b = l - 12;
#pragma unroll
    for (int sa = 0; sa < 6; ++sa)
    {
      const T c0 = ref.C[0][sa][b], c1 = ref.C[1][sa][b];
      if constexpr (kCompOrder)
      {
        je[sa] = -(S.aInvJ[0] * c0 + S.aInvJ[2] * c1);
        jo[sa] = -(S.aInvJ[1] * c0 + S.aInvJ[3] * c1);
        r += je[sa] * S.st[2 * sa] + jo[sa] * S.st[2 * sa + 1];
      }
      else
      {
        je[sa] = -accNorm(mac(S.aInvJ[0] * c0, S.aInvJ[2], c1));
        jo[sa] = -accNorm(mac(S.aInvJ[1] * c0, S.aInvJ[3], c1));
        r      = mac(mac(r, je[sa], S.st[2 * sa]), jo[sa], S.st[2 * sa + 1]);
      }
    }
    r = accNorm(r);
  }
  if constexpr (kGather)
  {
    if (row_lane)
    {
      // one record per element row: its 15 entries (+ one pad) and its
      // residual term; the row kernel sums the records of each CSR row
      const int k = a.gslot[15 * e + l];
      if (kRes)
      {
        a.gres[k] = gbfem::toF64(r);
      }
      if constexpr (kRes64)
      {
        a.gres[k] = rowRes64(*R64, l);
      }
      if (kJac)
      {
        T          v[16];
        const bool swap = !kCompOrder && l < 12 && c == 1;
  #pragma unroll
        for (int b = 0; b < 6; ++b)
        {
          v[2 * b]     = swap ? jo[b] : je[b];
          v[2 * b + 1] = swap ? je[b] : jo[b];
        }
  #pragma unroll
        for (int b = 0; b < 3; ++b)
        {
          v[12 + b] = jp[b]; // zero on pressure rows
        }
        v[15] = T(0);
        storeRecord(static_cast<T*>(a.geb) + 16LL * k, v);
      }
    }
    if (has && !live && l < 15)
    {
      // a rejected element (reported through the status word) adds nothing
      const int k = a.gslot[15 * e + l];
      a.gres[k]   = 0.0;
      if (kJac)
      {
        T z[16];
  #pragma unroll
        for (int i = 0; i < 16; ++i)
        {
          z[i] = T(0);
        }
        storeRecord(static_cast<T*>(a.geb) + 16LL * k, z);
      }
    }
  }
  // Every global reduction below adds into arrays that the previous kernel
  // on the stream zero-fills; a kernel launched as its dependent may have
  // started before that fill completed (no-op otherwise).
  gbfem::awaitPrerequisites();
  if (!kGather && row_lane)
  {
    // reloaded (an L1 hit) rather than kept live through the element math
    const int row_dof = a.dofs[15 * e + l];
    if (kRes)
    {
      gbfem::addTo<kPlain>(a.res + row_dof, gbfem::toF64(r));
    }
    if constexpr (kRes64)
    {
      gbfem::addTo<kPlain>(a.res + row_dof, rowRes64(*R64, l));
    }
    if (kJac)
    {
      // one store sequence for velocity and pressure rows (no divergence):
      // local columns 2b (component 0), 2b + 1 (component 1), then the
      // pressure columns, zero on pressure rows (the pressure-pressure block
      // is structurally present and zero: the scatter adds nothing to it)
      T* ov = sm.outv[le][l];
      if (kCompOrder || l >= 12)
      {
#pragma unroll
        for (int b = 0; b < 6; ++b)
        {
          ov[2 * b]     = je[b];
          ov[2 * b + 1] = jo[b];
        }
      }
      else
      {
#pragma unroll
        for (int b = 0; b < 6; ++b)
        {
          ov[2 * b + c]       = je[b];
          ov[2 * b + (c ^ 1)] = jo[b];
        }
      }
#pragma unroll
      for (int b = 0; b < 3; ++b)
      {
        ov[12 + b] = jp[b];
      }
      sm.rs[le][l] = h_rs;
    }
  }
  if (kJac && !kGather)
  {
    __syncwarp();
    if (live && l < 15)
    {
      // Lane l owns local column l of every row of its element: a half-warp
      // instruction adds one row's 15 entries, which lie in one CSR row
      // segment, so the L2 reductions coalesce.
      if (a.vals != nullptr) // null: J^T lam only (the element block is staged, not kept)
      {
        unsigned char pos[16];
        if (a.jac_pos != nullptr)
        {
          const unsigned wd[4] = {h_pos.x, h_pos.y, h_pos.z, h_pos.w};
#pragma unroll
          for (int i = 0; i < 16; ++i)
          {
            pos[i] = static_cast<unsigned char>(wd[i >> 2] >> (8 * (i & 3)));
          }
        }
#pragma unroll
        for (int row = 0; row < 15; ++row)
        {
          if (row < 12 || l < 12)
          {
            const int slot = a.jac_pos != nullptr ? sm.rs[le][row] + pos[row]
                                                  : a.jac_map[225LL * e + 15 * row + l];
            gbfem::addTo<kPlain>(a.vals + slot, gbfem::toF64Ftz(sm.outv[le][row][l]));
          }
        }
      }
      if (kVjp)
      {
        // fused state VJP: (J_e^T lam_e)_l, a reduction over the rows
        T acc = 0;
#pragma unroll
        for (int row = 0; row < 15; ++row)
        {
          if (row < 12 || l < 12)
          {
            acc += sm.outv[le][row][l] * sm.lam[le][row];
          }
        }
        gbfem::addTo<kPlain>(a.g_state + a.dofs[15 * e + l], gbfem::toF64(acc));
      }
    }
  }
  __syncthreads(); // the block's shared staging is reused by the next call
}

template <class T, bool kJac, bool kRes>
// 12 resident blocks per SM (at most 40 registers): the kernel waits mostly
// on its dependent gathers (dofs -> state and row pointers, connectivity ->
// coordinates), and more resident elements hide more of that latency.
__global__ void __launch_bounds__(kThreads, 12) thKernel(ThArgs a)
{
  __shared__ ThSmem<T> sm;
  thStageRef(sm, a.status);
  __syncthreads();
  thBlock<T, kJac, kRes, false>(a, blockIdx.x * kElemsPerBlock, sm);
}

// Coloured passes (one launch per colour, a.elems = the colour's
// elements): plain read-add-writes instead of FP64 reductions.
template <class T, bool kJac, bool kRes>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 12 : 4) thKernelColour(ThArgs a)
{
  __shared__ ThSmem<T> sm;
  thStageRef(sm, a.status);
  __syncthreads();
  thBlock<T, kJac, kRes, false, false, false, true>(a, blockIdx.x * kElemsPerBlock, sm);
}

template <class T, bool kRes>
__global__ void __launch_bounds__(kThreads) thVjpKernelColour(ThArgs a)
{
  __shared__ ThSmem<T> sm;
  thStageRef(sm, a.status);
  __syncthreads();
  thBlock<T, true, kRes, true, false, false, true>(a, blockIdx.x * kElemsPerBlock, sm);
}

// MIXED: FP32-quadrature Jacobian and FP64 residual in one pass.
__global__ void __launch_bounds__(kThreads) thKernelMixed(ThArgs a)
{
  __shared__ ThSmemMixed<float> sm;
  thStageRef(sm, a.status);
  __syncthreads();
  thBlock<float, true, false, false, true>(a, blockIdx.x * kElemsPerBlock, sm);
}

// State VJP g += J(u)^T lam without storing J (vals null), plus the
// residual when kRes.
template <class T, bool kRes>
__global__ void __launch_bounds__(kThreads) thVjpKernel(ThArgs a)
{
  __shared__ ThSmem<T> sm;
  thStageRef(sm, a.status);
  __syncthreads();
  thBlock<T, true, kRes, true>(a, blockIdx.x * kElemsPerBlock, sm);
}

// Reference tables in constant memory: the thread-per-element kernel below
// reads every entry with the same address across the warp (broadcast).
__constant__ ThRef<double> kRefC = makeRef();

// FP64 residual, one thread per element, by direct quadrature:
//   R_(a,c) = sum_q [Ft_c(q) . dN^_a(q) + src_c(q) N^_a(q)],
//   Ft_c = J^-1 W (nu grad u_c - p e_c),  src_c = W u . grad u_c,
//   R_p(b)  = -sum_q psi^_b(q) W div u(q),   W = w_q |det|.
// All 32 lanes work (FP64 issue, not lanes, is the bound on GB300); used for
// the residual-only FP64 path and, next to the FP32-quadrature Jacobian
// kernel, for the MIXED Newton scheme.
// Scalar adapters: the residual below is written once over S = double (the
// FP64 path) and S = DF (double-float on the FP32 pipe, the MIXED path).
template <class S>
__device__ __forceinline__ S sFromF64(double d);
template <>
__device__ __forceinline__ double sFromF64<double>(double d)
{
  return d;
}
template <>
__device__ __forceinline__ gbfem::DF sFromF64<gbfem::DF>(double d)
{
  return gbfem::dfFromF64(d);
}
// acc + x*y, and the end of an accumulation
__device__ __forceinline__ double sFma(double x, double y, double acc)
{
  return acc + x * y;
}
__device__ __forceinline__ gbfem::DF sFma(gbfem::DF x, gbfem::DF y, gbfem::DF acc)
{
  return gbfem::dfFma(x, y, acc);
}
__device__ __forceinline__ double sNorm(double x)
{
  return x;
}
__device__ __forceinline__ gbfem::DF sNorm(gbfem::DF x)
{
  return gbfem::dfNorm(x);
}
__device__ __forceinline__ double sToF64(double x)
{
  return x;
}
__device__ __forceinline__ double sToF64(gbfem::DF x)
{
  return gbfem::dfToF64(x);
}

template <class S, bool kPlain = false>
__device__ __forceinline__ void thResidualElem(const ThArgs& a, int idx, const ThRef<S>& rd)
{
  if (idx >= a.ne)
  {
    return;
  }
  const int e = a.elems != nullptr ? a.elems[idx] : idx; // coloured: the colour's list
  int nodes[3];
  for (int k = 0; k < 6; ++k)
  {
    const int nk = a.conn6[6 * e + k];
    if (static_cast<unsigned>(nk) >= static_cast<unsigned>(a.num_nodes))
    {
      gbfem::devFail(a.status, gbfem::kDevNodeRange, e);
      return;
    }
    if (k < 3)
    {
      nodes[k] = nk;
    }
  }
  // geometry in FP64 (a few operations per element)
  const double2 x0 = a.coords[nodes[0]], x1 = a.coords[nodes[1]], x2 = a.coords[nodes[2]];
  const double  j00 = x1.x - x0.x, j01 = x2.x - x0.x;
  const double  j10 = x1.y - x0.y, j11 = x2.y - x0.y;
  const double  det = j00 * j11 - j01 * j10;
  if (!(fabs(det) >= 1.0e-30))
  {
    gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
    return;
  }
  const double inv   = gbfem::rcpF64(det);
  const S      iJ[4] = {sFromF64<S>(j11 * inv), sFromF64<S>(-j01 * inv),
                        sFromF64<S>(-j10 * inv), sFromF64<S>(j00 * inv)};
  const S      ad    = sFromF64<S>(fabs(det));
  const S      zero  = sFromF64<S>(0.0);
  S            st[15], r[15];
  int          dofs[15];
#pragma unroll
  for (int l = 0; l < 15; ++l)
  {
    dofs[l] = a.dofs[15 * e + l];
    st[l]   = sFromF64<S>(a.state[dofs[l]]);
    r[l]    = zero;
  }
  const S nu = sFromF64<S>(a.nu);
  // double-float code is ~10x longer per operation: fully unrolled over the
  // points it overflows the instruction cache, so it keeps the point loop
  constexpr int kUnrollQ = std::is_same<S, double>::value ? kNq : 1;
#pragma unroll kUnrollQ
  for (int q = 0; q < kNq; ++q)
  {
    S u0 = zero, u1 = zero, r00 = zero, r01 = zero, r10 = zero, r11 = zero;
#pragma unroll
    for (int s2 = 0; s2 < 6; ++s2)
    {
      const S v0 = st[2 * s2], v1 = st[2 * s2 + 1];
      const S n = rd.N[q][s2], g0 = rd.dNr[q][s2][0], g1 = rd.dNr[q][s2][1];
      u0  = sFma(n, v0, u0);
      u1  = sFma(n, v1, u1);
      r00 = sFma(g0, v0, r00);
      r01 = sFma(g1, v0, r01);
      r10 = sFma(g0, v1, r10);
      r11 = sFma(g1, v1, r11);
    }
    u0  = sNorm(u0);
    u1  = sNorm(u1);
    r00 = sNorm(r00);
    r01 = sNorm(r01);
    r10 = sNorm(r10);
    r11 = sNorm(r11);
    const S G00 = sNorm(sFma(r01, iJ[2], r00 * iJ[0]));
    const S G01 = sNorm(sFma(r01, iJ[3], r00 * iJ[1]));
    const S G10 = sNorm(sFma(r11, iJ[2], r10 * iJ[0]));
    const S G11 = sNorm(sFma(r11, iJ[3], r10 * iJ[1]));
    S       pq  = zero;
#pragma unroll
    for (int b = 0; b < 3; ++b)
    {
      pq = sFma(rd.P[q][b], st[12 + b], pq);
    }
    pq          = sNorm(pq);
    const S W   = rd.w[q] * ad;
    const S F00 = W * (nu * G00 - pq), F01 = W * (nu * G01);
    const S F10 = W * (nu * G10), F11 = W * (nu * G11 - pq);
    const S Ft[2][2] = {{sNorm(sFma(iJ[1], F01, iJ[0] * F00)), sNorm(sFma(iJ[3], F01, iJ[2] * F00))},
                        {sNorm(sFma(iJ[1], F11, iJ[0] * F10)), sNorm(sFma(iJ[3], F11, iJ[2] * F10))}};
    const S src[2]   = {W * sNorm(sFma(u1, G01, u0 * G00)), W * sNorm(sFma(u1, G11, u0 * G10))};
    const S dq       = W * (G00 + G11);
#pragma unroll
    for (int sa = 0; sa < 6; ++sa)
    {
#pragma unroll
      for (int c = 0; c < 2; ++c)
      {
        S t = sFma(Ft[c][0], rd.dNr[q][sa][0], r[2 * sa + c]);
        t   = sFma(Ft[c][1], rd.dNr[q][sa][1], t);
        r[2 * sa + c] = sNorm(sFma(src[c], rd.N[q][sa], t));
      }
    }
#pragma unroll
    for (int b = 0; b < 3; ++b)
    {
      r[12 + b] = sNorm(sFma(-rd.P[q][b], dq, r[12 + b]));
    }
  }
  gbfem::awaitPrerequisites(); // the residual's zero fill may still be running
#pragma unroll
  for (int l = 0; l < 15; ++l)
  {
    gbfem::addTo<kPlain>(a.res + dofs[l], sToF64(r[l]));
  }
}

// Reference tables in constant memory (warp-uniform operands).
__constant__ ThRef<gbfem::DF> kRefDF = castRef<gbfem::DF>();

template <bool kPlain = false>
__device__ __forceinline__ void thResidual64Elem(const ThArgs& a, int e)
{
  thResidualElem<double, kPlain>(a, e, kRefC);
}

// MIXED residual: double-float arithmetic (~44 significant bits) on the
// FP32 pipe; error against the FP64 residual ~1e-14 relative.
template <bool kPlain = false>
__device__ __forceinline__ void thResidualDFElem(const ThArgs& a, int e)
{
  thResidualElem<gbfem::DF, kPlain>(a, e, kRefDF);
}

// Row-gather variants: the element pass writes records, no atomics.
template <class T, bool kJac, bool kRes>
__global__ void __launch_bounds__(kThreads) thKernelGather(ThArgs a)
{
  __shared__ ThSmem<T> sm;
  thStageRef(sm, a.status);
  __syncthreads();
  thBlock<T, kJac, kRes, false, false, true>(a, blockIdx.x * kElemsPerBlock, sm);
}

__global__ void __launch_bounds__(kThreads) thKernelMixedGather(ThArgs a)
{
  __shared__ ThSmemMixed<float> sm;
  thStageRef(sm, a.status);
  __syncthreads();
  thBlock<float, true, false, false, true, true>(a, blockIdx.x * kElemsPerBlock, sm);
}

} // namespace

