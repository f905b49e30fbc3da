// th.cu — Taylor-Hood P2/P1 steady Navier-Stokes Newton residual and
// Jacobian through femx's assemble contract (femx/assembly/CudaAssembly.hpp:
// 319-364). The element has 15 local DOFs (12 velocity, 3 pressure) in
// MixedFESpace order (MixedFESpace.cpp:57-84), and uses the published
// 6-point degree-4 triangle rule (Dunavant).
//
// On GB300 the FP64 pipe (~1 TFLOP/s measured) bounds the plain path, so the
// element is factorised to spend as few FP64 operations as possible while
// giving exactly the quadrature sums of the row operator (up to rounding):
//   diffusion  D_ab = sum_kl Gh_kl S^kl_ab,  Gh = nu|det| J^-1 J^-T and
//              S^kl_ab = sum_q w_q dN^_a,k dN^_b,l (reference constants);
//   reaction   M^ce_ab = |det| sum_v G_v[c][e] T^v_ab: grad u of a P2 field
//              is linear, so its quadrature values are the vertex values G_v
//              interpolated, T^v_ab = sum_q w_q N^_a N^_b lambda_v(q);
//   pressure   B_(a,c),b = -|det| sum_k Jinv[k][c] C^k_ab,
//              C^k_ab = sum_q w_q psi^_b dN^_a,k;
//   convection A_ab = |det| sum_q w_q N^_a (dN^_b . ut_q), ut_q = J^-T-free
//              transform Jinv u_q, the only term kept at quadrature points.
// The residual follows from the same blocks: R_(a,c) = sum_b (D+A)_ab
// u_(b,c) + sum_b B_(a,c),b p_b, R_p(b) = sum_(a,e) B_(a,e),b u_(a,e).
//
// Layouts: FP32 quadrature (thKernel, th_elem.cuh) gives a 16-lane group
// one element — shared stages compute the geometry, the quadrature-point
// transforms and the vertex gradients once, then lane l produces local row l
// (15 entries + residual). Plain FP64 (thElemKernel64) and FP64-accurate
// double-float (thElemKernelDd) give one thread one element (below): FP64
// issue, resp. the double-float instruction count, is their bound, and a
// thread per element keeps every lane of every instruction busy.
// Output: lanes scatter-add with FP64 reductions at L2 through the compact
// in-row position map (fastest). With GBFEM_DETERMINISTIC, lane l writes its
// row as one record instead and a row pass (gather.cuh) sums each CSR row's
// records in element order — no atomics, no zero-fill, bitwise
// reproducible, about 1.5x the time of the atomic path.
#include <atomic>
#include <utility>

#include "gather.cuh"
#include "th_elem.cuh"

namespace
{

template <bool kPlain = false>
__global__ void __launch_bounds__(128) thResidual64Kernel(ThArgs a)
{
  thResidual64Elem<kPlain>(a, blockIdx.x * blockDim.x + threadIdx.x);
}

template <bool kPlain = false>
__global__ void __launch_bounds__(128) thResidualDFKernel(ThArgs a)
{
  thResidualDFElem<kPlain>(a, blockIdx.x * blockDim.x + threadIdx.x);
}

// Reference tables as compile-time constants: terms whose table entry is
// zero (the P2 vertex gradients, the diffusion tensors and the pressure
// tensors are about half zeros; entries below 1e-14 are quadrature-sum
// residues of exact zeros) are left out of the FP64 element at compile time.
constexpr ThRef<double> kRefX = makeRef();

constexpr bool tabNz(double v)
{
  return v > 1.0e-14 || v < -1.0e-14;
}

template <class F, int... I>
__device__ __forceinline__ void staticForImpl(F& f, std::integer_sequence<int, I...>)
{
  (f(std::integral_constant<int, I>{}), ...);
}

// f(std::integral_constant<int, i>) for i = 0 .. N-1, unrolled: table
// indices that are constant expressions.
template <int N, class F>
__device__ __forceinline__ void staticFor(F&& f)
{
  staticForImpl(f, std::make_integer_sequence<int, N>{});
}

// x C^0_(sa,b) + y C^1_(sa,b) with the zero entries of C left out.
template <int sa, int b>
__device__ __forceinline__ double presCol(double x, double y)
{
  constexpr double c0 = kRefX.C[0][sa][b], c1 = kRefX.C[1][sa][b];
  if constexpr (tabNz(c0) && tabNz(c1))
  {
    return x * c0 + y * c1;
  }
  else if constexpr (tabNz(c0))
  {
    return x * c0;
  }
  else if constexpr (tabNz(c1))
  {
    return y * c1;
  }
  else
  {
    return 0.0;
  }
}

// Shared-memory slot groups of the symmetric reaction entries: pair (a, b),
// a < b, is formed in row a and read back in row b; groups are reused once
// their pair's row has been reached (at most nine pairs are live at once).
struct PairSlots
{
  int g[6][6];
  int groups;
};
constexpr PairSlots makePairSlots()
{
  PairSlots p{};
  int       freeAt[15] = {};
  int       ng         = 0;
  for (int a = 0; a < 6; ++a)
  {
    for (int b = a + 1; b < 6; ++b)
    {
      int g = -1;
      for (int k = 0; k < ng; ++k)
      {
        if (freeAt[k] <= a)
        {
          g = k;
          break;
        }
      }
      if (g < 0)
      {
        g = ng++;
      }
      freeAt[g] = b;
      p.g[a][b] = g;
      p.g[b][a] = g;
    }
  }
  p.groups = ng;
  return p;
}
constexpr PairSlots kPairSlots = makePairSlots();
static_assert(kPairSlots.groups * 4 <= 36, "reaction slots exceed the staging area");

// Two pairs that share a group are never live together: one is read back
// (in row b) no later than the other is formed (in its row a). Row a reads
// its pairs (b < a) before it forms its own (b > a).
constexpr bool pairSlotsDisjoint()
{
  for (int a0 = 0; a0 < 6; ++a0)
  {
    for (int b0 = a0 + 1; b0 < 6; ++b0)
    {
      for (int a1 = 0; a1 < 6; ++a1)
      {
        for (int b1 = a1 + 1; b1 < 6; ++b1)
        {
          const bool same = a0 == a1 && b0 == b1;
          if (!same && kPairSlots.g[a0][b0] == kPairSlots.g[a1][b1] && !(b0 <= a1 || b1 <= a0))
          {
            return false;
          }
        }
      }
    }
  }
  return true;
}
static_assert(pairSlotsDisjoint(), "two live reaction pairs share a slot group");

// dynamic shared memory of thElemKernel64: each thread's reaction entries
constexpr int kTh64PresBytes = 36 * 128 * static_cast<int>(sizeof(double));

// Plain FP64 Jacobian + residual, one thread per element. The same
// factorised element as thBlock (diffusion from the reference tensors S,
// convection from the quadrature transforms, reaction from the vertex
// gradients, pressure blocks from C) with the reference tables in constant
// memory (warp-uniform operands). FP64 issue is the bound on GB300, and an
// FP64 warp instruction costs the same with 1 or 32 active lanes, so every
// lane owns a whole element: about half the FP64 warp instructions of the
// 16-lane layout, whose geometry and quadrature stages run on few lanes.
// Rows are produced one at a time (warp-uniform), staged in shared memory
// and added row-coalesced: a half-warp adds one element row per FP64
// reduction instruction, positions from the row-major in-row map (loaded
// before the row's values are computed and staged next to them).
// Four resident blocks per SM (128 registers, a few spilled to L1) measured
// faster than two or three with fewer spills: more warps keep the FP64 pipe
// fed.
// The terms whose reference-table entry is zero are left out at compile time
// (kRefX, staticFor: 416 -> 355 us on the 256x256 cavity), the pressure
// rows copy the pressure columns that the velocity rows staged in dynamic
// shared memory, with the pressure residual accumulated there (355 -> 349
// us), and the reaction terms accumulate onto D + A by FMA (349 -> 331 us).
// The reaction block M^ce_ab = sum_v T^v_ab G_v[c][e] is symmetric in (a, b):
// row (a, c) forms the entries b > a and keeps them in its dynamic shared
// memory (kPairSlots groups) for row (b, c), which reads them back instead
// of forming them (120 FMAs per element fewer); the pressure rows recompute
// their pressure columns, which no longer have the shared memory
// (331 -> 309 us).
// kPlain: a coloured pass (a.elems = the colour's elements, which share no
// DOF): plain read-add-writes instead of FP64 reductions; needs pos_rows.
// kVjp: the state VJP g += J^T lam without forming J: each row's values are
// multiplied by the row's adjoint value and summed into the thread's staging
// row (its 15 entries of J_e^T lam_e), added to g_state at the end; no
// residual, no CSR write.
template <bool kPlain = false, bool kVjp = false>
__global__ void __launch_bounds__(128, 4) thElemKernel64(ThArgs a, const unsigned char* pos_rows)
{
  extern __shared__ double sB64[]; // [36][128]: reaction entries M^cc, M^c,other of pair groups
  __shared__ double buf[4][32][17];
  __shared__ int    rsb[4][32];
  __shared__ uint4  posb[4][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e0   = blockIdx.x * 128 + warp * 32;
  const int idx  = e0 + lane;
  bool      live = idx < a.ne;
  const int e    = (kPlain && live) ? a.elems[idx] : idx;
  const ThRef<double>& R = kRefC;

  double aInvJ[4] = {0, 0, 0, 0}, G3[3] = {0, 0, 0};
  if (live)
  {
    for (int k = 0; k < 6; ++k)
    {
      if (static_cast<unsigned>(a.conn6[6 * e + k]) >= static_cast<unsigned>(a.num_nodes))
      {
        gbfem::devFail(a.status, gbfem::kDevNodeRange, e);
        live = false;
      }
    }
  }
  if (live)
  {
    const double2 x0 = a.coords[a.conn6[6 * e + 0]];
    const double2 x1 = a.coords[a.conn6[6 * e + 1]];
    const double2 x2 = a.coords[a.conn6[6 * e + 2]];
    const double  j00 = x1.x - x0.x, j01 = x2.x - x0.x;
    const double  j10 = x1.y - x0.y, j11 = x2.y - x0.y;
    const double  det = j00 * j11 - j01 * j10;
    const double  ad  = det < 0.0 ? -det : det;
    if (ad >= 1.0e-30)
    {
      const double inv = gbfem::rcpF64(det);
      const double i00 = j11 * inv, i01 = -j01 * inv, i10 = -j10 * inv, i11 = j00 * inv;
      aInvJ[0]         = ad * i00;
      aInvJ[1]         = ad * i01;
      aInvJ[2]         = ad * i10;
      aInvJ[3]         = ad * i11;
      const double nad = a.nu * ad;
      G3[0]            = nad * (i00 * i00 + i01 * i01);
      G3[1]            = nad * (i10 * i10 + i11 * i11);
      G3[2]            = nad * (i00 * i10 + i01 * i11);
    }
    else
    {
      gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
      live = false;
    }
  }
  double st[15];
#pragma unroll
  for (int l = 0; l < 15; ++l)
  {
    st[l] = live ? a.state[a.dofs[15 * e + l]] : 0.0;
  }
  double Gv[3][2][2] = {}, ut[kNq][2] = {};
  if (live)
  {
    staticFor<3>([&](auto V) {
      constexpr int v = decltype(V)::value;
#pragma unroll
      for (int c = 0; c < 2; ++c)
      {
        double g0 = 0, g1 = 0;
        staticFor<6>([&](auto S2) {
          constexpr int    s2 = decltype(S2)::value;
          constexpr double d0 = kRefX.dNv[v][s2][0], d1 = kRefX.dNv[v][s2][1];
          if constexpr (tabNz(d0))
          {
            g0 += st[2 * s2 + c] * d0;
          }
          if constexpr (tabNz(d1))
          {
            g1 += st[2 * s2 + c] * d1;
          }
        });
        Gv[v][c][0] = g0 * aInvJ[0] + g1 * aInvJ[2];
        Gv[v][c][1] = g0 * aInvJ[1] + g1 * aInvJ[3];
      }
    });
#pragma unroll
    for (int q = 0; q < kNq; ++q)
    {
      double u0 = 0, u1 = 0;
#pragma unroll
      for (int s2 = 0; s2 < 6; ++s2)
      {
        u0 += R.N[q][s2] * st[2 * s2];
        u1 += R.N[q][s2] * st[2 * s2 + 1];
      }
      ut[q][0] = aInvJ[0] * u0 + aInvJ[1] * u1;
      ut[q][1] = aInvJ[2] * u0 + aInvJ[3] * u1;
    }
  }

  const bool jac = !kVjp && a.vals != nullptr;
  // row l: CSR start and positions (loaded ahead of the values); VJP: the
  // row's adjoint value
  double lrow = 0.0;
  auto   rowRef = [&](int l, int& rs, uint4& pw) {
    rs = -1;
    pw = make_uint4(0, 0, 0, 0);
    if constexpr (kVjp)
    {
      lrow = live ? a.lam[a.dofs[15 * e + l]] : 0.0;
    }
    if (live && jac)
    {
      rs = a.row_ptr[a.dofs[15 * e + l]];
      if (pos_rows != nullptr)
      {
        pw = *reinterpret_cast<const uint4*>(pos_rows + (15LL * e + l) * 16);
      }
    }
  };
  // row values go straight to this lane's staging row bv (not held in
  // registers: the row loop is register-bound); VJP: bv accumulates J_e^T
  // lam_e
  double* const bv = buf[warp][lane];
  if constexpr (kVjp)
  {
#pragma unroll
    for (int j = 0; j < 15; ++j)
    {
      bv[j] = 0.0;
    }
  }
  auto put = [&](int j, double x) {
    if constexpr (kVjp)
    {
      bv[j] += x * lrow;
    }
    else
    {
      bv[j] = x;
    }
  };
  auto stage = [&](int l, int rs, const uint4& pw, double r) {
    if constexpr (kVjp)
    {
      return;
    }
    gbfem::awaitPrerequisites(); // the outputs' zero fill may still be running
    if (live)
    {
      gbfem::addTo<kPlain>(a.res + a.dofs[15 * e + l], r);
    }
    if (jac)
    {
      rsb[warp][lane]  = rs;
      posb[warp][lane] = pw;
    }
  };
  auto scatterRow = [&](int l) {
    if (!jac)
    {
      return;
    }
    __syncwarp();
    const int j = lane & 15;
#pragma unroll 4
    for (int t2 = 0; t2 < 16; ++t2)
    {
      const int t  = 2 * t2 + (lane >> 4);
      const int rs = rsb[warp][t];
      if (j < 15 && rs >= 0 && (l < 12 || j < 12))
      {
        const int slot = pos_rows != nullptr
                             ? rs + reinterpret_cast<const unsigned char*>(&posb[warp][t])[j]
                             : a.jac_map[225LL * (e0 + t) + 15 * l + j];
        gbfem::addTo<kPlain>(a.vals + slot, buf[warp][t][j]);
      }
    }
    __syncwarp();
  };

  // vq[q][b] = dN^_b(q) . ut_q does not depend on the row: formed once per
  // element (72 FMAs) instead of once per velocity node row pair (432)
  double vq[kNq][6];
  staticFor<kNq>([&](auto Q) {
    constexpr int q = decltype(Q)::value;
    staticFor<6>([&](auto B) {
      constexpr int    b  = decltype(B)::value;
      constexpr double d0 = kRefX.dNr[q][b][0], d1 = kRefX.dNr[q][b][1];
      if constexpr (tabNz(d0) && tabNz(d1))
      {
        vq[q][b] = d0 * ut[q][0] + d1 * ut[q][1];
      }
      else if constexpr (tabNz(d0))
      {
        vq[q][b] = d0 * ut[q][0];
      }
      else if constexpr (tabNz(d1))
      {
        vq[q][b] = d1 * ut[q][1];
      }
      else
      {
        vq[q][b] = 0.0;
      }
    });
  });

  double rp[3] = {0.0, 0.0, 0.0};
  staticFor<6>([&](auto SA) {
    constexpr int sa = decltype(SA)::value;
    double        da[6];
    staticFor<6>([&](auto B) {
      constexpr int    b   = decltype(B)::value;
      constexpr double s00 = kRefX.S00[sa][b], s11 = kRefX.S11[sa][b], s01 = kRefX.S01[sa][b];
      double           d   = 0.0;
      if constexpr (tabNz(s00))
      {
        d += G3[0] * s00;
      }
      if constexpr (tabNz(s11))
      {
        d += G3[1] * s11;
      }
      if constexpr (tabNz(s01))
      {
        d += G3[2] * s01;
      }
#pragma unroll
      for (int q = 0; q < kNq; ++q)
      {
        d += R.wN[q][sa] * vq[q][b];
      }
      da[b] = d;
    });
#pragma unroll
    for (int c = 0; c < 2; ++c)
    {
      int   rs;
      uint4 pw;
      rowRef(2 * sa + c, rs, pw);
      const int oc = c ^ 1;
      double    r  = 0;
      staticFor<6>([&](auto B) {
        constexpr int b = decltype(B)::value;
        double        mcc, mco;
        if constexpr (b < sa)
        {
          // the mirror entries, formed in row (b, c)
          constexpr int g = kPairSlots.g[b][sa];
          mcc             = da[b] + sB64[(4 * g + 2 * c) * 128 + threadIdx.x];
          mco             = sB64[(4 * g + 2 * c + 1) * 128 + threadIdx.x];
        }
        else if constexpr (b == sa)
        {
          mcc = da[b];
          mcc += R.T[0][sa][b] * Gv[0][c][c];
          mcc += R.T[1][sa][b] * Gv[1][c][c];
          mcc += R.T[2][sa][b] * Gv[2][c][c];
          mco = R.T[0][sa][b] * Gv[0][c][oc] + R.T[1][sa][b] * Gv[1][c][oc]
                + R.T[2][sa][b] * Gv[2][c][oc];
        }
        else
        {
          constexpr int g  = kPairSlots.g[sa][b];
          const double  mr = R.T[0][sa][b] * Gv[0][c][c] + R.T[1][sa][b] * Gv[1][c][c]
                            + R.T[2][sa][b] * Gv[2][c][c];
          mco = R.T[0][sa][b] * Gv[0][c][oc] + R.T[1][sa][b] * Gv[1][c][oc]
                + R.T[2][sa][b] * Gv[2][c][oc];
          sB64[(4 * g + 2 * c) * 128 + threadIdx.x]     = mr;
          sB64[(4 * g + 2 * c + 1) * 128 + threadIdx.x] = mco;
          mcc                                           = da[b] + mr;
        }
        put(2 * b + c, mcc);
        put(2 * b + oc, mco);
        r += da[b] * st[2 * b + c];
      });
      staticFor<3>([&](auto B) {
        constexpr int b  = decltype(B)::value;
        const double  vp = -presCol<sa, b>(aInvJ[c], aInvJ[2 + c]);
        put(12 + b, vp);
        r += vp * st[12 + b];
        rp[b] += vp * st[2 * sa + c];
      });
      stage(2 * sa + c, rs, pw, r);
      scatterRow(2 * sa + c);
    }
  });
  staticFor<3>([&](auto B) {
    constexpr int b = decltype(B)::value;
    int           rs;
    uint4         pw;
    rowRef(12 + b, rs, pw);
    staticFor<6>([&](auto SA) {
      constexpr int sa = decltype(SA)::value;
      put(2 * sa, -presCol<sa, b>(aInvJ[0], aInvJ[2]));
      put(2 * sa + 1, -presCol<sa, b>(aInvJ[1], aInvJ[3]));
    });
    if constexpr (!kVjp)
    {
      bv[12] = bv[13] = bv[14] = 0.0; // structurally present, nothing added
    }
    stage(12 + b, rs, pw, rp[b]);
    scatterRow(12 + b);
  });
  if constexpr (kVjp)
  {
    gbfem::awaitPrerequisites(); // the gradient's zero fill may still be running
    if (live)
    {
#pragma unroll
      for (int j = 0; j < 15; ++j)
      {
        gbfem::addTo<kPlain>(a.g_state + a.dofs[15 * e + j], bv[j]);
      }
    }
  }
}

// Double-float reference tables in constant memory (warp-uniform operands).
__constant__ ThRef<gbfem::Dd> kRefCDd = castRef<gbfem::Dd>();

// x y in double-float, left unnormalised: TwoProduct of the leading parts
// with the cross terms in the trailing part, the first term of a Dot2 sum
// (mac adds the others).
__device__ __forceinline__ gbfem::Dd ddProd(gbfem::Dd x, gbfem::Dd y)
{
  const float p  = __fmul_rn(x.hi, y.hi);
  float       lo = __fmaf_rn(x.hi, y.hi, -p);
  lo             = __fmaf_rn(x.hi, y.lo, lo);
  lo             = __fmaf_rn(x.lo, y.hi, lo);
  return {p, lo};
}

// A double-float as the double it stands for (normalised, then joined
// without FP64 instructions).
__device__ __forceinline__ double ddOut(gbfem::Dd x)
{
  return gbfem::ddJoinInt(accNorm(x));
}

// acc + x k for a compile-time k that a float holds exactly (the P2
// vertex gradients are small integers): the product's error is k x.lo alone
template <int kNum>
__device__ __forceinline__ gbfem::Dd macExact(gbfem::Dd acc, gbfem::Dd x)
{
  constexpr float k = static_cast<float>(kNum);
  if constexpr (kNum == 1 || kNum == -1)
  {
    const float p  = kNum == 1 ? x.hi : -x.hi;
    const float s  = __fadd_rn(acc.hi, p);
    const float bb = __fsub_rn(s, acc.hi);
    const float se = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    return {s, __fadd_rn(acc.lo, __fadd_rn(se, kNum == 1 ? x.lo : -x.lo))};
  }
  else
  {
    const float p  = __fmul_rn(x.hi, k);
    const float pe = __fmaf_rn(x.hi, k, -p);
    const float s  = __fadd_rn(acc.hi, p);
    const float bb = __fsub_rn(s, acc.hi);
    const float se = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    return {s, __fmaf_rn(x.lo, k, __fadd_rn(acc.lo, __fadd_rn(se, pe)))};
  }
}

constexpr int kThDdThreads = 128;
// dynamic shared memory of thElemKernelDd: each thread's convection matrix
constexpr int kThDdConvBytes = 36 * kThDdThreads * static_cast<int>(sizeof(float2));

// FP64-accurate Jacobian + residual, one thread per element, in double-float
// arithmetic on the FP32 pipe: the element of thElemKernel64 with every
// product-sum a Dot2 accumulation (ddProd, then mac; normalised once at its
// end), so that FP64 issue (1/64 of the FP32 rate on GB300) no longer bounds
// it. FP64 is left for the four edge subtractions; the state, the edges and
// every output cross between double and double-float on the integer pipe
// (ddSplitInt, ddJoinInt). The convection
// matrix A_ab = sum_q w_q N^_a (dN^_b . ut_q) is formed once per element
// into shared memory (a column of 36 double-floats per thread, read back
// conflict-free) so that the row loop holds only the state, the vertex
// gradients and the geometry factors in registers; the diffusion D_ab is
// added onto it there once (zero entries of S left out at compile time), and
// the vertex gradients use the P2 gradient values as exact integers
// (178.8 -> 175.8 us). Rows are staged and added row-coalesced as in
// thElemKernel64. kPlain: a coloured pass, as there.
// kVjp: the state VJP g += J^T lam, as in thElemKernel64 (each row's values
// times the row's adjoint value summed into the thread's staging row, here
// as double-float pairs; joined and added to g_state at the end).
template <bool kPlain = false, bool kVjp = false>
__global__ void __launch_bounds__(kThDdThreads, 4)
    thElemKernelDd(ThArgs a, const unsigned char* pos_rows)
{
  using gbfem::Dd;
  extern __shared__ float2 sConv[]; // [36][kThDdThreads]
  __shared__ double buf[4][32][17];
  __shared__ int    rsb[4][32];
  __shared__ uint4  posb[4][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e0   = blockIdx.x * kThDdThreads + warp * 32;
  const int idx  = e0 + lane;
  bool      live = idx < a.ne;
  const int e    = (kPlain && live) ? a.elems[idx] : idx;
  const ThRef<Dd>& R = kRefCDd;

  // geometry: the edges by FP64 subtraction (the coordinates can be far
  // larger than the edges), everything else in double-float; |det| J^-1 =
  // sign(det) adj(J) needs no division, nu |det| J^-1 J^-T one reciprocal
  Dd e00 = Dd(0.0f, 0.0f), e01 = e00, e10 = e00, e11 = e00;
  if (live)
  {
    for (int k = 0; k < 6; ++k)
    {
      if (static_cast<unsigned>(a.conn6[6 * e + k]) >= static_cast<unsigned>(a.num_nodes))
      {
        gbfem::devFail(a.status, gbfem::kDevNodeRange, e);
        live = false;
      }
    }
  }
  if (live)
  {
    const double2 x0 = a.coords[a.conn6[6 * e + 0]];
    const double2 x1 = a.coords[a.conn6[6 * e + 1]];
    const double2 x2 = a.coords[a.conn6[6 * e + 2]];
    e00              = gbfem::ddSplitInt(x1.x - x0.x);
    e01              = gbfem::ddSplitInt(x2.x - x0.x);
    e10              = gbfem::ddSplitInt(x1.y - x0.y);
    e11              = gbfem::ddSplitInt(x2.y - x0.y);
  }
  const Dd   det = accNorm(mac(ddProd(e00, e11), -e01, e10));
  const bool neg = det.hi < 0.0f;
  const Dd   ad  = neg ? -det : det;
  if (live && !(ad.hi >= 1.0e-30f))
  {
    gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
    live = false;
  }
  Dd iJ[4], G3[3], st[15]; // |det| J^-1 (row-major), nu |det| J^-1 J^-T (00, 11, 01)
  iJ[0] = neg ? -e11 : e11;
  iJ[1] = neg ? e01 : -e01;
  iJ[2] = neg ? e10 : -e10;
  iJ[3] = neg ? -e00 : e00;
  {
    const Dd nur = live ? gbfem::ddSplitInt(a.nu) * gbfem::ddRcp(ad) : Dd(0.0f, 0.0f);
    G3[0]        = accNorm(mac(ddProd(e11, e11), e01, e01)) * nur;
    G3[1]        = accNorm(mac(ddProd(e10, e10), e00, e00)) * nur;
    G3[2]        = -(accNorm(mac(ddProd(e11, e10), e01, e00)) * nur);
  }
#pragma unroll
  for (int l = 0; l < 15; ++l)
  {
    st[l] = gbfem::ddSplitInt(live ? a.state[a.dofs[15 * e + l]] : 0.0);
  }

  // vertex gradients of the velocity, G_v[c][k]
  Dd Gv[3][2][2];
  staticFor<3>([&](auto V) {
    constexpr int v = decltype(V)::value;
#pragma unroll
    for (int c = 0; c < 2; ++c)
    {
      Dd g0 = Dd(0.0f, 0.0f), g1 = Dd(0.0f, 0.0f);
      staticFor<6>([&](auto S2) {
        constexpr int s2 = decltype(S2)::value;
        constexpr int k0 = static_cast<int>(kRefX.dNv[v][s2][0]);
        constexpr int k1 = static_cast<int>(kRefX.dNv[v][s2][1]);
        static_assert(k0 == kRefX.dNv[v][s2][0] && k1 == kRefX.dNv[v][s2][1],
                      "the vertex gradients are integers");
        if constexpr (k0 != 0)
        {
          g0 = macExact<k0>(g0, st[2 * s2 + c]);
        }
        if constexpr (k1 != 0)
        {
          g1 = macExact<k1>(g1, st[2 * s2 + c]);
        }
      });
      g0          = accNorm(g0);
      g1          = accNorm(g1);
      Gv[v][c][0] = accNorm(mac(ddProd(g0, iJ[0]), g1, iJ[2]));
      Gv[v][c][1] = accNorm(mac(ddProd(g0, iJ[1]), g1, iJ[3]));
    }
  });
  // quadrature-point transforms ut_q = |det| J^-1 u_q
  Dd ut[kNq][2];
#pragma unroll
  for (int q = 0; q < kNq; ++q)
  {
    Dd u0 = ddProd(R.N[q][0], st[0]), u1 = ddProd(R.N[q][0], st[1]);
#pragma unroll
    for (int s2 = 1; s2 < 6; ++s2)
    {
      u0 = mac(u0, R.N[q][s2], st[2 * s2]);
      u1 = mac(u1, R.N[q][s2], st[2 * s2 + 1]);
    }
    u0       = accNorm(u0);
    u1       = accNorm(u1);
    ut[q][0] = accNorm(mac(ddProd(iJ[0], u0), iJ[1], u1));
    ut[q][1] = accNorm(mac(ddProd(iJ[2], u0), iJ[3], u1));
  }
  // convection matrix A[sa][b] = sum_q wN[q][sa] (dN^_b(q) . ut_q), one
  // column b at a time, into this thread's column of sConv
  float2* const colA = sConv + threadIdx.x;
#pragma unroll 1
  for (int b = 0; b < 6; ++b)
  {
    Dd vq[kNq];
#pragma unroll
    for (int q = 0; q < kNq; ++q)
    {
      vq[q] = accNorm(mac(ddProd(R.dNr[q][b][0], ut[q][0]), R.dNr[q][b][1], ut[q][1]));
    }
#pragma unroll
    for (int sa = 0; sa < 6; ++sa)
    {
      Dd t = ddProd(R.wN[0][sa], vq[0]);
#pragma unroll
      for (int q = 1; q < kNq; ++q)
      {
        t = mac(t, R.wN[q][sa], vq[q]);
      }
      t                                   = accNorm(t);
      colA[(6 * sa + b) * kThDdThreads] = make_float2(t.hi, t.lo);
    }
  }

  // the diffusion D_ab = G3 . S_ab onto A_ab (zero entries of S left out
  // at compile time), normalised: the row loop reads D + A as it is
  staticFor<6>([&](auto SA) {
    constexpr int sa = decltype(SA)::value;
    staticFor<6>([&](auto B) {
      constexpr int    b   = decltype(B)::value;
      constexpr double s00 = kRefX.S00[sa][b], s11 = kRefX.S11[sa][b], s01 = kRefX.S01[sa][b];
      const float2     cv  = colA[(6 * sa + b) * kThDdThreads];
      Dd               d   = Dd(cv.x, cv.y);
      if constexpr (tabNz(s00))
      {
        d = mac(d, G3[0], Dd(s00));
      }
      if constexpr (tabNz(s11))
      {
        d = mac(d, G3[1], Dd(s11));
      }
      if constexpr (tabNz(s01))
      {
        d = mac(d, G3[2], Dd(s01));
      }
      d                                 = accNorm(d);
      colA[(6 * sa + b) * kThDdThreads] = make_float2(d.hi, d.lo);
    });
  });

  const bool jac = !kVjp && a.vals != nullptr;
  // row l: CSR start and positions (loaded ahead of the values); VJP: the
  // row's adjoint value
  Dd   lrow   = Dd(0.0f, 0.0f);
  auto rowRef = [&](int l, int& rs, uint4& pw) {
    rs = -1;
    pw = make_uint4(0, 0, 0, 0);
    if constexpr (kVjp)
    {
      lrow = gbfem::ddSplitInt(live ? a.lam[a.dofs[15 * e + l]] : 0.0);
    }
    if (live && jac)
    {
      rs = a.row_ptr[a.dofs[15 * e + l]];
      if (pos_rows != nullptr)
      {
        pw = *reinterpret_cast<const uint4*>(pos_rows + (15LL * e + l) * 16);
      }
    }
  };
  double* const bv  = buf[warp][lane];
  float2* const bvd = reinterpret_cast<float2*>(bv); // VJP: J_e^T lam_e as pairs
  if constexpr (kVjp)
  {
#pragma unroll
    for (int j = 0; j < 15; ++j)
    {
      bvd[j] = make_float2(0.0f, 0.0f);
    }
  }
  // entry j of the current row: staged as a double, or (VJP) times the row's
  // adjoint value into the thread's J_e^T lam_e
  auto put = [&](int j, Dd x) {
    if constexpr (kVjp)
    {
      const float2 g = bvd[j];
      const Dd     t = mac(Dd(g.x, g.y), x, lrow);
      bvd[j]         = make_float2(t.hi, t.lo);
    }
    else
    {
      bv[j] = ddOut(x);
    }
  };
  auto stage = [&](int l, int rs, const uint4& pw, double r) {
    if constexpr (kVjp)
    {
      return;
    }
    gbfem::awaitPrerequisites(); // the outputs' zero fill may still be running
    if (live)
    {
      gbfem::addTo<kPlain>(a.res + a.dofs[15 * e + l], r);
    }
    if (jac)
    {
      rsb[warp][lane]  = rs;
      posb[warp][lane] = pw;
    }
  };
  auto scatterRow = [&](int l) {
    if (!jac)
    {
      return;
    }
    __syncwarp();
    const int j = lane & 15;
#pragma unroll 4
    for (int t2 = 0; t2 < 16; ++t2)
    {
      const int t  = 2 * t2 + (lane >> 4);
      const int rs = rsb[warp][t];
      if (j < 15 && rs >= 0 && (l < 12 || j < 12))
      {
        const int slot = pos_rows != nullptr
                             ? rs + reinterpret_cast<const unsigned char*>(&posb[warp][t])[j]
                             : a.jac_map[225LL * (e0 + t) + 15 * l + j];
        gbfem::addTo<kPlain>(a.vals + slot, buf[warp][t][j]);
      }
    }
    __syncwarp();
  };

  // velocity rows (sa, c)
  Dd rp[3] = {Dd(0.0f, 0.0f), Dd(0.0f, 0.0f), Dd(0.0f, 0.0f)}; // pressure residual
#pragma unroll 1
  for (int sa = 0; sa < 6; ++sa)
  {
    Dd da[6]; // diffusion + convection, D_ab + A_ab
#pragma unroll
    for (int b = 0; b < 6; ++b)
    {
      const float2 cv = colA[(6 * sa + b) * kThDdThreads];
      da[b]           = Dd(cv.x, cv.y);
    }
    // the two component rows share everything but the component: one
    // rolled loop over c (half the code of an unrolled pair, which the
    // instruction cache does not hold), the component's operands selected
#pragma unroll 1
    for (int c = 0; c < 2; ++c)
    {
      int   rs;
      uint4 pw;
      rowRef(2 * sa + c, rs, pw);
      const bool c1 = c != 0;
      Dd         gcc[3], gco[3]; // G_v[c][c], G_v[c][other]
#pragma unroll
      for (int v = 0; v < 3; ++v)
      {
        gcc[v] = c1 ? Gv[v][1][1] : Gv[v][0][0];
        gco[v] = c1 ? Gv[v][1][0] : Gv[v][0][1];
      }
      const Dd jc = c1 ? iJ[1] : iJ[0], jc2 = c1 ? iJ[3] : iJ[2];
      Dd       r, ssa = Dd(0.0f, 0.0f); // ssa: this row's own state value
#pragma unroll
      for (int b = 0; b < 6; ++b)
      {
        const Dd sb = c1 ? st[2 * b + 1] : st[2 * b];
        ssa         = b == sa ? sb : ssa;
        r           = b == 0 ? ddProd(da[0], sb) : mac(r, da[b], sb);
        const Dd t0 = R.T[0][sa][b], t1 = R.T[1][sa][b], t2 = R.T[2][sa][b];
        Dd       mcc = mac(da[b], t0, gcc[0]);
        mcc          = mac(mac(mcc, t1, gcc[1]), t2, gcc[2]);
        Dd mco       = ddProd(t0, gco[0]);
        mco          = mac(mac(mco, t1, gco[1]), t2, gco[2]);
        put(2 * b + c, mcc);
        put(2 * b + 1 - c, mco);
      }
      // the pressure columns B_(sa,c),b; the pressure rows are their
      // transpose: the values go to the column slots of A[sa][.] (read into
      // da above, free now), slot 6 sa + 3 c + b, and the pressure residual
      // R_p(b) = sum B_(sa,c),b u_(sa,c) accumulates here
      double* const bslot = reinterpret_cast<double*>(colA) + (6 * sa + 3 * c) * kThDdThreads;
#pragma unroll
      for (int b = 0; b < 3; ++b)
      {
        const Dd vp = -accNorm(mac(ddProd(jc, R.C[0][sa][b]), jc2, R.C[1][sa][b]));
        if constexpr (kVjp)
        {
          put(12 + b, vp);
          reinterpret_cast<float2*>(bslot)[b * kThDdThreads] = make_float2(vp.hi, vp.lo);
        }
        else
        {
          const double vj         = gbfem::ddJoinInt(vp);
          bv[12 + b]              = vj;
          bslot[b * kThDdThreads] = vj;
        }
        r     = mac(r, vp, st[12 + b]);
        rp[b] = mac(rp[b], vp, ssa);
      }
      stage(2 * sa + c, rs, pw, ddOut(r));
      scatterRow(2 * sa + c);
    }
  }
  // pressure rows b: the negative divergence block, the pressure columns
  // staged above (slot 6 sa + 3 c + b = 3 k + b for column k = 2 sa + c)
  const double* const colB = reinterpret_cast<const double*>(colA);
#pragma unroll 1
  for (int b = 0; b < 3; ++b)
  {
    int   rs;
    uint4 pw;
    rowRef(12 + b, rs, pw);
#pragma unroll
    for (int k = 0; k < 12; ++k)
    {
      if constexpr (kVjp)
      {
        const float2 v = reinterpret_cast<const float2*>(colB)[(3 * k + b) * kThDdThreads];
        put(k, Dd(v.x, v.y));
      }
      else
      {
        bv[k] = colB[(3 * k + b) * kThDdThreads];
      }
    }
    if constexpr (!kVjp)
    {
      bv[12] = bv[13] = bv[14] = 0.0; // structurally present, nothing added
    }
    const Dd r = b == 0 ? rp[0] : (b == 1 ? rp[1] : rp[2]);
    stage(12 + b, rs, pw, ddOut(r));
    scatterRow(12 + b);
  }
  if constexpr (kVjp)
  {
    gbfem::awaitPrerequisites(); // the gradient's zero fill may still be running
    if (live)
    {
#pragma unroll
      for (int j = 0; j < 15; ++j)
      {
        const float2 g = bvd[j];
        gbfem::addTo<kPlain>(a.g_state + a.dofs[15 * e + j], ddOut(Dd(g.x, g.y)));
      }
    }
  }
}

// thElemKernelDd and thElemKernel64 take more than the default 48 KB of
// shared memory per block (the convection columns, the pressure columns are
// dynamic shared memory): allow that, and ask for the largest shared-memory
// carveout so that four blocks fit on an SM. Once per device.
void thPrepareSharedMemory()
{
  static std::atomic<unsigned long long> done{0}; // one bit per device below 64
  int dev = 0;
  gbfem::cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
  const unsigned long long bit = dev < 64 ? 1ull << dev : 0ull; // others: set every time
  if (bit != 0 && (done.load(std::memory_order_acquire) & bit) != 0)
  {
    return;
  }
  auto set = [](auto k, int bytes) {
    gbfem::cudaCheck(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
                     "Taylor-Hood element kernel shared memory");
    gbfem::cudaCheck(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                          cudaSharedmemCarveoutMaxShared),
                     "Taylor-Hood element kernel carveout");
  };
  set(thElemKernelDd<false>, kThDdConvBytes);
  set(thElemKernelDd<true>, kThDdConvBytes);
  set(thElemKernelDd<false, true>, kThDdConvBytes);
  set(thElemKernelDd<true, true>, kThDdConvBytes);
  set(thElemKernel64<false>, kTh64PresBytes);
  set(thElemKernel64<true>, kTh64PresBytes);
  set(thElemKernel64<false, true>, kTh64PresBytes);
  set(thElemKernel64<true, true>, kTh64PresBytes);
  done.fetch_or(bit, std::memory_order_acq_rel);
}

} // namespace

namespace gbfem
{

// The Taylor-Hood assembly behind gbfem_assemble_th_ns. zero = true: the
// outputs are zero-filled here and the element kernels launch as dependents
// of that fill; zero = false: the caller has zero-filled res and vals on the
// stream (or on a stream it has joined) and the kernels launch ordinarily.
void assembleTaylorHood(const gbfem_assembly_map* map, int num_p2_nodes, const double* coords,
                        const int* conn6, double nu, const double* state, double* res,
                        double* vals, int precision, cudaStream_t s, bool zero)
{
  {
    require(map != nullptr, "AssemblyMap handle is null");
    require(map->num_elems == 0
                || (map->uniform_res == 15 && map->uniform_state == 15),
            "Taylor-Hood element expects 15 DOFs per element");
    require(map->num_res == map->num_states && map->same_dofs,
            "Taylor-Hood assembly expects identical residual and state DOF "
            "tables");
    require(num_p2_nodes >= 0, "Geometry node count must be non-negative");
    require(map->num_elems == 0 || (coords && conn6 && state),
            "Assembly inputs must not be null");
    require(res != nullptr, "Assembly residual output is null");
    require(res != state && vals != state && (vals == nullptr || res != vals),
            "Assembly state, residual, and matrix values must not alias");
    const bool det = (precision & GBFEM_DETERMINISTIC) != 0;
    const bool col = (precision & GBFEM_COLOURED) != 0;
    precision &= ~(GBFEM_DETERMINISTIC | GBFEM_COLOURED);
    require(!(det && col), "deterministic and coloured assembly are exclusive");
    require(!col || map->num_elems == 0 || map->colour_elems != nullptr,
            "coloured assembly needs gbfem_assembly_map_enable_colouring on the map");
    require(precision >= GBFEM_PREC_FP64 && precision <= GBFEM_PREC_DOUBLE_FLOAT,
            "unknown precision mode");
    require(!det || map->num_elems == 0 || map->gather_off != nullptr,
            "deterministic assembly needs gbfem_assembly_map_enable_gather on the map");
    require((reinterpret_cast<uintptr_t>(coords) & 15) == 0,
            "Geometry coordinates must be 16-byte aligned");
    const bool gather = det && map->num_elems > 0;
    const bool dep    = zero;
    if (!gather && zero)
    {
      // the FP32-quadrature element kernel is launched as a dependent of
      // this zero fill and overlaps it up to its first reduction
      zeroForNext(vals, vals != nullptr ? map->nnz : 0, res, map->num_res, s);
    }
    if (map->num_elems == 0)
    {
      return;
    }
    ThArgs a{};
    a.ne        = map->num_elems;
    a.num_nodes = num_p2_nodes;
    a.dofs    = map->state_dofs;
    a.conn6   = conn6;
    a.coords  = reinterpret_cast<const double2*>(coords);
    a.nu      = nu;
    a.state   = state;
    a.jac_map = map->jac_map;
    a.row_ptr = map->row_ptr;
    a.jac_pos = map->pos_stride == 16 ? map->jac_pos : nullptr;
    a.res     = res;
    a.vals    = vals;
    a.status  = map->status;
    const unsigned blocks = blocksFor(a.ne, kElemsPerBlock);
    const bool     jac    = vals != nullptr;
    if (gather)
    {
      // deterministic two-pass assembly: element records, then row sums
      a.gslot               = map->gather_slot;
      a.geb                 = map->gather_eb;
      a.gres                = map->gather_res;
      const bool     f64    = precision == GBFEM_PREC_FP64
                       || precision == GBFEM_PREC_DOUBLE_FLOAT
                       || (precision == GBFEM_PREC_MIXED && !jac);
      const unsigned rblk   = blocksFor(map->num_res, kGatherRows);
      if (f64)
      {
        jac ? thKernelGather<double, true, true><<<blocks, kThreads, 0, s>>>(a)
            : thKernelGather<double, false, true><<<blocks, kThreads, 0, s>>>(a);
        cudaCheck(cudaGetLastError(), "Taylor-Hood element pass launch");
        gatherRowsKernel<double><<<rblk, kGatherThreads, 0, s>>>(
            map->num_res, 15, map->gather_off, map->gather_eb, map->gather_pos, map->row_ptr,
            map->gather_res, vals, res);
      }
      else
      {
        if (precision == GBFEM_PREC_FP32_QUAD)
        {
          jac ? thKernelGather<float, true, true><<<blocks, kThreads, 0, s>>>(a)
              : thKernelGather<float, false, true><<<blocks, kThreads, 0, s>>>(a);
        }
        else
        {
          thKernelMixedGather<<<blocks, kThreads, 0, s>>>(a);
        }
        cudaCheck(cudaGetLastError(), "Taylor-Hood element pass launch");
        gatherRowsKernel<float><<<rblk, kGatherThreads, 0, s>>>(
            map->num_res, 15, map->gather_off, reinterpret_cast<const float*>(map->gather_eb),
            map->gather_pos, map->row_ptr, map->gather_res, vals, res);
      }
      cudaCheck(cudaGetLastError(), "Taylor-Hood row pass launch");
      return;
    }
    // One element pass: every element in one launch (FP64 reductions), or,
    // coloured, one launch per colour in colour order (plain adds; the
    // colour's element list in a.elems). Only a pass's first launch may be a
    // dependent of the zero fill.
    auto pass = [&](auto&& launch, bool first_dep) {
      if (!col)
      {
        launch(a, first_dep, false);
        return;
      }
      for (int c = 0; c < map->num_colours; ++c)
      {
        ThArgs ac = a;
        ac.elems  = map->colour_elems + map->colour_off_host[c];
        ac.ne     = map->colour_off_host[c + 1] - map->colour_off_host[c];
        if (ac.ne > 0)
        {
          launch(ac, first_dep && c == 0, true);
        }
      }
    };
    auto eb = [](const ThArgs& x) { return blocksFor(x.ne, 128); };
    auto gb = [](const ThArgs& x) { return blocksFor(x.ne, kElemsPerBlock); };
    auto res64 = [&](const ThArgs& x, bool d, bool plain) {
      plain ? launchMaybeDependent(d, thResidual64Kernel<true>, eb(x), 128, s, x)
            : launchMaybeDependent(d, thResidual64Kernel<false>, eb(x), 128, s, x);
    };
    auto resDF = [&](const ThArgs& x, bool d, bool plain) {
      plain ? launchMaybeDependent(d, thResidualDFKernel<true>, eb(x), 128, s, x)
            : launchMaybeDependent(d, thResidualDFKernel<false>, eb(x), 128, s, x);
    };
    if (precision == GBFEM_PREC_FP64 && jac)
    {
      require(!col || map->jac_pos_rows != nullptr,
              "coloured Taylor-Hood assembly needs the compact position map");
      thPrepareSharedMemory();
      pass(
          [&](const ThArgs& x, bool d, bool plain) {
            plain ? launchMaybeDependentSmem(d, thElemKernel64<true>, eb(x), 128,
                                             kTh64PresBytes, s, x, map->jac_pos_rows)
                  : launchMaybeDependentSmem(d, thElemKernel64<false>, eb(x), 128,
                                             kTh64PresBytes, s, x, map->jac_pos_rows);
          },
          dep);
    }
    else if (precision == GBFEM_PREC_DOUBLE_FLOAT)
    {
      if (jac)
      {
        require(!col || map->jac_pos_rows != nullptr,
                "coloured Taylor-Hood assembly needs the compact position map");
        thPrepareSharedMemory();
        pass(
            [&](const ThArgs& x, bool d, bool plain) {
              plain ? launchMaybeDependentSmem(d, thElemKernelDd<true>, eb(x), kThDdThreads,
                                               kThDdConvBytes, s, x, map->jac_pos_rows)
                    : launchMaybeDependentSmem(d, thElemKernelDd<false>, eb(x), kThDdThreads,
                                               kThDdConvBytes, s, x, map->jac_pos_rows);
            },
            dep);
      }
      else
      {
        pass(resDF, false);
      }
    }
    else if (precision == GBFEM_PREC_FP32_QUAD)
    {
      pass(
          [&](const ThArgs& x, bool d, bool plain) {
            if (plain)
            {
              jac ? launchMaybeDependent(d, thKernelColour<float, true, true>, gb(x), kThreads,
                                         s, x)
                  : launchMaybeDependent(d, thKernelColour<float, false, true>, gb(x),
                                         kThreads, s, x);
            }
            else
            {
              jac ? launchMaybeDependent(d, thKernel<float, true, true>, gb(x), kThreads, s, x)
                  : launchMaybeDependent(d, thKernel<float, false, true>, gb(x), kThreads, s,
                                         x);
            }
          },
          dep);
    }
    else
    {
      if (jac)
      {
        // MIXED: FP32-quadrature Jacobian, residual in double-float. (Run
        // side by side on two streams they overlapped by 1.5 % only: the
        // residual kernel's 128-register blocks and the Jacobian kernel's
        // 12 blocks per SM do not share SMs.)
        pass(
            [&](const ThArgs& x, bool d, bool plain) {
              plain ? launchMaybeDependent(d, thKernelColour<float, true, false>, gb(x),
                                           kThreads, s, x)
                    : launchMaybeDependent(d, thKernel<float, true, false>, gb(x), kThreads, s,
                                           x);
            },
            dep);
        pass(resDF, false);
      }
      else
      {
        // residual-only calls of the FP64 and MIXED modes: FP64
        pass(res64, false);
      }
    }
    cudaCheck(cudaGetLastError(), "Taylor-Hood assembly launch");
  }
}

} // namespace gbfem

extern "C" int gbfem_assemble_th_ns(const gbfem_assembly_map* map,
                                    int num_p2_nodes, const double* coords,
                                    const int* conn6, double nu,
                                    const double* state, double* res,
                                    double* vals, int precision, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    assembleTaylorHood(map, num_p2_nodes, coords, conn6, nu, state, res, vals, precision,
                       asStream(stream), true);
  });
}

extern "C" int gbfem_vjp_th_ns(const gbfem_assembly_map* map, int num_p2_nodes,
                               const double* coords, const int* conn6, double nu,
                               const double* state, const double* lam, double* g_state,
                               int precision, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(map != nullptr, "AssemblyMap handle is null");
    require(map->num_elems == 0
                || (map->uniform_res == 15 && map->uniform_state == 15),
            "Taylor-Hood element expects 15 DOFs per element");
    require(map->num_res == map->num_states && map->same_dofs,
            "Taylor-Hood assembly expects identical residual and state DOF "
            "tables");
    require(num_p2_nodes >= 0, "Geometry node count must be non-negative");
    require(map->num_elems == 0 || (coords && conn6 && state && lam),
            "VJP inputs must not be null");
    require(g_state != nullptr, "VJP output is null");
    require(g_state != state && g_state != lam, "VJP output must not alias its inputs");
    const bool col = (precision & GBFEM_COLOURED) != 0;
    precision &= ~GBFEM_COLOURED;
    require(precision >= GBFEM_PREC_FP64 && precision <= GBFEM_PREC_DOUBLE_FLOAT,
            "unknown precision mode");
    require(!col || map->num_elems == 0 || map->colour_elems != nullptr,
            "coloured assembly needs gbfem_assembly_map_enable_colouring on the map");
    require((reinterpret_cast<uintptr_t>(coords) & 15) == 0,
            "Geometry coordinates must be 16-byte aligned");
    cudaStream_t s = asStream(stream);
    thPrepareSharedMemory();
    // the VJP kernel is launched as a dependent of this zero fill
    zeroForNext(g_state, map->num_states, nullptr, 0, s);
    if (map->num_elems == 0)
    {
      return;
    }
    ThArgs a{};
    a.ne        = map->num_elems;
    a.num_nodes = num_p2_nodes;
    a.dofs      = map->state_dofs;
    a.conn6     = conn6;
    a.coords    = reinterpret_cast<const double2*>(coords);
    a.nu        = nu;
    a.state     = state;
    a.row_ptr   = map->row_ptr;
    a.jac_map   = map->jac_map;
    a.lam       = lam;
    a.g_state   = g_state;
    a.status    = map->status;
    // MIXED keeps the Jacobian (and so J^T lam) in FP32 quadrature; coloured:
    // one launch per colour, plain adds into g_state
    auto launch = [&](const ThArgs& x, bool d) {
      const unsigned blocks = blocksFor(x.ne, kElemsPerBlock);
      const bool     plain  = x.elems != nullptr;
      if (precision == GBFEM_PREC_FP64)
      {
        // one thread per element (the FP64 Jacobian kernel in VJP mode)
        const unsigned eb = blocksFor(x.ne, 128);
        plain ? launchMaybeDependentSmem(d, thElemKernel64<true, true>, eb, 128, kTh64PresBytes,
                                         s, x, nullptr)
              : launchMaybeDependentSmem(d, thElemKernel64<false, true>, eb, 128,
                                         kTh64PresBytes, s, x, nullptr);
      }
      else if (precision == GBFEM_PREC_DOUBLE_FLOAT)
      {
        // one thread per element (the double-float Jacobian kernel in VJP mode)
        const unsigned eb = blocksFor(x.ne, kThDdThreads);
        plain ? launchMaybeDependentSmem(d, thElemKernelDd<true, true>, eb, kThDdThreads,
                                         kThDdConvBytes, s, x, nullptr)
              : launchMaybeDependentSmem(d, thElemKernelDd<false, true>, eb, kThDdThreads,
                                         kThDdConvBytes, s, x, nullptr);
      }
      else
      {
        plain ? launchMaybeDependent(d, thVjpKernelColour<float, false>, blocks, kThreads, s, x)
              : launchMaybeDependent(d, thVjpKernel<float, false>, blocks, kThreads, s, x);
      }
    };
    if (!col)
    {
      launch(a, true);
    }
    else
    {
      for (int c = 0; c < map->num_colours; ++c)
      {
        ThArgs ac = a;
        ac.elems  = map->colour_elems + map->colour_off_host[c];
        ac.ne     = map->colour_off_host[c + 1] - map->colour_off_host[c];
        if (ac.ne > 0)
        {
          launch(ac, c == 0);
        }
      }
    }
    cudaCheck(cudaGetLastError(), "Taylor-Hood VJP launch");
  });
}
