// th.cu — Taylor-Hood P2/P1 steady Navier-Stokes Newton residual and
// Jacobian through femx's assemble contract (femx/assembly/CudaAssembly.hpp:
// 319-364). The element has 15 local DOFs (12 velocity, 3 pressure) in
// MixedFESpace order (MixedFESpace.cpp:57-84), and uses the published
// 6-point degree-4 triangle rule (Dunavant).
//
// Layout: a 16-lane group owns one element, lane l computes local row l
// (lane 15 helps with the shared stages). Per element, shared memory holds
// the gathered state, the physical shape gradients at the six quadrature
// points and the quadrature-point state (u, grad u, p), computed once per
// element — unlike the reference's row operators, which recompute the
// quadrature-point state for every row (femx/model/ns/Components.hpp:
// 492-495). Each row's 15 Jacobian entries and residual are then scatter-
// added with FP64 reductions at L2.
#include <type_traits>

#include "maps.cuh"

namespace
{
using gbfem::DeviceStatus;

constexpr int kLanes          = 16;
constexpr int kElemsPerBlock  = 8;
constexpr int kThreads        = kLanes * kElemsPerBlock;
constexpr int kNq             = 6;

struct ThTables
{
  double N[kNq][6];      // P2 values
  double P[kNq][3];      // P1 values
  double dNr[kNq][6][2]; // P2 reference gradients
  double w[kNq];         // weights (reference area 1/2)
};

struct ThTablesF
{
  float N[kNq][6];
  float P[kNq][3];
  float dNr[kNq][6][2];
  float w[kNq];
};

constexpr ThTables makeTables()
{
  ThTables   t{};
  const double a1 = 0.445948490915964886, w1 = 0.223381589678011466 * 0.5;
  const double a2 = 0.091576213509770743, w2 = 0.109951743655321868 * 0.5;
  const double q[kNq][3] = {{a1, a1, w1}, {1.0 - 2.0 * a1, a1, w1},
                            {a1, 1.0 - 2.0 * a1, w1}, {a2, a2, w2},
                            {1.0 - 2.0 * a2, a2, w2}, {a2, 1.0 - 2.0 * a2, w2}};
  for (int i = 0; i < kNq; ++i)
  {
    const double r = q[i][0], s = q[i][1];
    const double l0 = 1.0 - r - s, l1 = r, l2 = s;
    const double g0[2] = {-1.0, -1.0}, g1[2] = {1.0, 0.0}, g2[2] = {0.0, 1.0};
    t.N[i][0] = l0 * (2.0 * l0 - 1.0);
    t.N[i][1] = l1 * (2.0 * l1 - 1.0);
    t.N[i][2] = l2 * (2.0 * l2 - 1.0);
    t.N[i][3] = 4.0 * l0 * l1;
    t.N[i][4] = 4.0 * l1 * l2;
    t.N[i][5] = 4.0 * l2 * l0;
    for (int d = 0; d < 2; ++d)
    {
      t.dNr[i][0][d] = (4.0 * l0 - 1.0) * g0[d];
      t.dNr[i][1][d] = (4.0 * l1 - 1.0) * g1[d];
      t.dNr[i][2][d] = (4.0 * l2 - 1.0) * g2[d];
      t.dNr[i][3][d] = 4.0 * (l1 * g0[d] + l0 * g1[d]);
      t.dNr[i][4][d] = 4.0 * (l2 * g1[d] + l1 * g2[d]);
      t.dNr[i][5][d] = 4.0 * (l0 * g2[d] + l2 * g0[d]);
    }
    t.P[i][0] = l0;
    t.P[i][1] = l1;
    t.P[i][2] = l2;
    t.w[i]    = q[i][2];
  }
  return t;
}

constexpr ThTablesF makeTablesF()
{
  const ThTables d = makeTables();
  ThTablesF      f{};
  for (int i = 0; i < kNq; ++i)
  {
    for (int a = 0; a < 6; ++a)
    {
      f.N[i][a]      = static_cast<float>(d.N[i][a]);
      f.dNr[i][a][0] = static_cast<float>(d.dNr[i][a][0]);
      f.dNr[i][a][1] = static_cast<float>(d.dNr[i][a][1]);
    }
    for (int b = 0; b < 3; ++b)
    {
      f.P[i][b] = static_cast<float>(d.P[i][b]);
    }
    f.w[i] = static_cast<float>(d.w[i]);
  }
  return f;
}

__constant__ ThTables  kTab  = makeTables();
__constant__ ThTablesF kTabF = makeTablesF();

__device__ __forceinline__ const ThTables& tables(double)
{
  return kTab;
}
__device__ __forceinline__ const ThTablesF& tables(float)
{
  return kTabF;
}

struct ThArgs
{
  int            ne;
  int            num_nodes;
  const int*     dofs;  // [ne][15]
  const int*     conn6; // [ne][6]
  const double2* coords;
  double         nu;
  const double*  state;
  const int*     jac_map;
  double*        res;
  double*        vals;
  DeviceStatus*  status;
};

template <class T>
struct ElemShared
{
  T   st[16];
  T   invJ[4];
  T   W[kNq];
  T   dN[kNq][6][2];
  T   u[kNq][2];
  T   G[kNq][4];
  T   p[kNq];
  int ok;
};

template <class T, bool kJac>
__global__ void __launch_bounds__(kThreads) thKernel(ThArgs a)
{
  __shared__ ElemShared<T> sh[kElemsPerBlock];
  const int  l   = threadIdx.x & (kLanes - 1);
  const int  le  = threadIdx.x / kLanes;
  const int  e   = blockIdx.x * kElemsPerBlock + le;
  const bool has = e < a.ne;
  ElemShared<T>& S   = sh[le];
  const auto&    tab = tables(T());

  if (has && l < 15)
  {
    S.st[l] = T(a.state[a.dofs[15 * e + l]]);
  }
  bool nodes_ok = true;
  if (has && l == 15)
  {
    for (int k = 0; k < 6; ++k)
    {
      nodes_ok = nodes_ok
                 && static_cast<unsigned>(a.conn6[6 * e + k])
                        < static_cast<unsigned>(a.num_nodes);
    }
    if (!nodes_ok)
    {
      gbfem::devFail(a.status, gbfem::kDevNodeRange, e);
    }
  }
  if (has && l == 15 && !nodes_ok)
  {
    S.ok = 0;
  }
  else if (has && l == 15)
  {
    const double2 x0 = a.coords[a.conn6[6 * e + 0]];
    const double2 x1 = a.coords[a.conn6[6 * e + 1]];
    const double2 x2 = a.coords[a.conn6[6 * e + 2]];
    // J[a][b] = d x_a / d r_b from the vertices (affine element)
    const double j00 = x1.x - x0.x, j01 = x2.x - x0.x;
    const double j10 = x1.y - x0.y, j11 = x2.y - x0.y;
    const double det = j00 * j11 - j01 * j10;
    const double ad  = fabs(det);
    S.ok             = ad >= 1.0e-30 ? 1 : 0;
    if (S.ok)
    {
      const double inv = 1.0 / det;
      S.invJ[0]        = T(j11 * inv);
      S.invJ[1]        = T(-j01 * inv);
      S.invJ[2]        = T(-j10 * inv);
      S.invJ[3]        = T(j00 * inv);
      for (int q = 0; q < kNq; ++q)
      {
        S.W[q] = T(ad * tab.w[q]);
      }
    }
    else
    {
      gbfem::devFail(a.status, gbfem::kDevSingularJacobian, e);
    }
  }
  __syncthreads();
  const bool live = has && S.ok;
  if (live)
  {
    // physical gradients dN[q][i][d] = sum_b dNr[q][i][b] invJ[b][d]
    for (int i = l; i < kNq * 12; i += kLanes)
    {
      const int q = i / 12, s = (i % 12) / 2, d = i % 2;
      S.dN[q][s][d] = T(tab.dNr[q][s][0]) * S.invJ[0 * 2 + d]
                      + T(tab.dNr[q][s][1]) * S.invJ[1 * 2 + d];
    }
  }
  __syncthreads();
  if (live && l < kNq)
  {
    const int q  = l;
    T         u0 = 0, u1 = 0, g00 = 0, g01 = 0, g10 = 0, g11 = 0, p = 0;
#pragma unroll
    for (int s = 0; s < 6; ++s)
    {
      const T v0 = S.st[2 * s], v1 = S.st[2 * s + 1];
      const T n  = T(tab.N[q][s]);
      u0 += n * v0;
      u1 += n * v1;
      g00 += v0 * S.dN[q][s][0];
      g01 += v0 * S.dN[q][s][1];
      g10 += v1 * S.dN[q][s][0];
      g11 += v1 * S.dN[q][s][1];
    }
#pragma unroll
    for (int b = 0; b < 3; ++b)
    {
      p += T(tab.P[q][b]) * S.st[12 + b];
    }
    S.u[q][0] = u0;
    S.u[q][1] = u1;
    S.G[q][0] = g00;
    S.G[q][1] = g01;
    S.G[q][2] = g10;
    S.G[q][3] = g11;
    S.p[q]    = p;
  }
  __syncthreads();
  if (!live || l >= 15)
  {
    return;
  }
  const T nu = T(a.nu);
  // Velocity row (sa, c): jcc[sb] -> column (sb, c), jco[sb] -> (sb, 1-c),
  // jp[b] -> pressure column b. Pressure row b: jcc[sb] -> (sb, 0),
  // jco[sb] -> (sb, 1). Compile-time indices keep everything in registers.
  T jcc[6], jco[6], jp[3];
#pragma unroll
  for (int j = 0; j < 6; ++j)
  {
    jcc[j] = 0;
    jco[j] = 0;
  }
  jp[0] = jp[1] = jp[2] = 0;
  T   r = 0;
  int c = 0;
  if (l < 12)
  {
    const int sa = l >> 1;
    c            = l & 1;
    const int oc = c ^ 1;
    for (int q = 0; q < kNq; ++q)
    {
      const T W   = S.W[q];
      const T Na  = T(tab.N[q][sa]);
      const T dx  = S.dN[q][sa][0], dy = S.dN[q][sa][1];
      const T ux  = S.u[q][0], uy = S.u[q][1];
      const T gcx = S.G[q][2 * c], gcy = S.G[q][2 * c + 1];
      const T gcc = S.G[q][2 * c + c], gco = S.G[q][2 * c + oc];
      const T WNa = W * Na;
      const T dc  = c == 0 ? dx : dy;
      r += W * (nu * (gcx * dx + gcy * dy) - S.p[q] * dc)
           + WNa * (ux * gcx + uy * gcy);
      if (kJac)
      {
        const T Wnu = W * nu;
#pragma unroll
        for (int sb = 0; sb < 6; ++sb)
        {
          const T bx   = S.dN[q][sb][0], by = S.dN[q][sb][1];
          const T diff = bx * dx + by * dy;
          const T adv  = ux * bx + uy * by;
          const T tNb  = WNa * T(tab.N[q][sb]);
          jcc[sb] += Wnu * diff + WNa * adv + tNb * gcc;
          jco[sb] += tNb * gco;
        }
        const T wd = W * dc;
#pragma unroll
        for (int b = 0; b < 3; ++b)
        {
          jp[b] -= wd * T(tab.P[q][b]);
        }
      }
    }
  }
  else
  {
    const int b = l - 12;
    for (int q = 0; q < kNq; ++q)
    {
      const T wp = S.W[q] * T(tab.P[q][b]);
      r -= wp * (S.G[q][0] + S.G[q][3]);
      if (kJac)
      {
#pragma unroll
        for (int sa = 0; sa < 6; ++sa)
        {
          jcc[sa] -= wp * S.dN[q][sa][0];
          jco[sa] -= wp * S.dN[q][sa][1];
        }
      }
    }
  }
  gbfem::redAdd(a.res + a.dofs[15 * e + l], double(r));
  if (kJac)
  {
    const int* jm = a.jac_map + 225 * e + 15 * l;
#pragma unroll
    for (int sb = 0; sb < 6; ++sb)
    {
      gbfem::redAdd(a.vals + jm[2 * sb + c], double(jcc[sb]));
      gbfem::redAdd(a.vals + jm[2 * sb + (c ^ 1)], double(jco[sb]));
    }
#pragma unroll
    for (int b = 0; b < 3; ++b)
    {
      gbfem::redAdd(a.vals + jm[12 + b], double(jp[b]));
    }
  }
}

} // namespace

extern "C" int gbfem_assemble_th_ns(const gbfem_assembly_map* map,
                                    int num_p2_nodes, const double* coords,
                                    const int* conn6, double nu,
                                    const double* state, double* res,
                                    double* vals, int precision, void* stream)
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
    require(map->num_elems == 0 || (coords && conn6 && state),
            "Assembly inputs must not be null");
    require(res != nullptr, "Assembly residual output is null");
    require(res != state && vals != state && (vals == nullptr || res != vals),
            "Assembly state, residual, and matrix values must not alias");
    require(precision == GBFEM_PREC_FP64 || precision == GBFEM_PREC_FP32_QUAD,
            "unknown precision mode");
    require((reinterpret_cast<uintptr_t>(coords) & 15) == 0,
            "Geometry coordinates must be 16-byte aligned");
    cudaStream_t s = asStream(stream);
    cudaCheck(cudaMemsetAsync(res, 0, sizeof(double) * map->num_res, s),
              "residual zero");
    if (vals != nullptr && map->nnz > 0)
    {
      cudaCheck(cudaMemsetAsync(vals, 0, sizeof(double) * map->nnz, s),
                "matrix zero");
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
    a.res     = res;
    a.vals    = vals;
    a.status  = map->status;
    const unsigned blocks = blocksFor(a.ne, kElemsPerBlock);
    const bool     jac    = vals != nullptr;
    if (precision == GBFEM_PREC_FP64)
    {
      jac ? thKernel<double, true><<<blocks, kThreads, 0, s>>>(a)
          : thKernel<double, false><<<blocks, kThreads, 0, s>>>(a);
    }
    else
    {
      jac ? thKernel<float, true><<<blocks, kThreads, 0, s>>>(a)
          : thKernel<float, false><<<blocks, kThreads, 0, s>>>(a);
    }
    cudaCheck(cudaGetLastError(), "Taylor-Hood assembly launch");
  });
}
