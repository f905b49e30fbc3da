// batch.cu — many assembly instances of uneven size in one persistent launch.
//
// Each instance is one femx-style assemble (+ residual VJP) call: a
// kappa-weighted P1 Poisson or a Taylor-Hood P2/P1 Navier-Stokes Newton
// assembly on its own mesh and AssemblyMap. gbfem_batch_run enqueues exactly
// two kernels, so the whole batch can be captured once in a CUDA graph and
// replayed:
//   1. zeroSegments — zeroes every instance's residual, matrix values and
//      state-gradient (the outputs accumulated by FP64 reductions) and
//      resets the work ticket;
//   2. batchKernel  — a persistent grid (blocks_per_sm x SM count blocks of
//      128 threads). Blocks draw work items from one atomic ticket counter
//      (no block ever waits on another); an item is a chunk of consecutive
//      elements of one instance. P1 items run one element per thread, with
//      residual, Jacobian scatter and VJP (K lam, lam^T K u) fused on one
//      evaluation of the element stiffness; Taylor-Hood items run 16-lane
//      element groups with the row-coalesced scatter and the fused state VJP
//      J^T lam (a reduction over the element's rows).
// The item decode (instance prefix of chunk counts) is built by every block
// in shared memory from the descriptor table at kernel start.
#include <algorithm>
#include <vector>

#include "p1_elem.cuh"
#include "th_elem.cuh"

namespace
{

constexpr int kBatchThreads = 128;
constexpr int kMaxInstances = 1024;
constexpr int kZeroTile     = 8192; // doubles zeroed per block

static_assert(kBatchThreads == kThreads, "Taylor-Hood block shape");

struct BatchDesc
{
  int        kind;
  int        num_elems;
  int        num_colours;  // 0 when the instance's map is not coloured
  const int* colour_off;   // [num_colours + 1], device
  const int* colour_elems; // elements colour by colour, device
  P1Args     p1;
  ThArgs     th;
};

constexpr int kMaxRounds = 64; // colours (one launch each) of a coloured run

struct ZeroSeg
{
  double*   ptr;
  long long n;
};

__global__ void zeroSegments(const ZeroSeg* __restrict__ segs,
                             const long long* __restrict__ block_prefix, int nseg,
                             int* __restrict__ ticket)
{
  __shared__ int seg;
  if (threadIdx.x == 0)
  {
    if (blockIdx.x == 0)
    {
      for (int r = 0; r < kMaxRounds; ++r)
      {
        ticket[r] = 0;
      }
    }
    int lo = 0, hi = nseg;
    while (hi - lo > 1)
    {
      const int mid = (lo + hi) >> 1;
      if (block_prefix[mid] <= blockIdx.x)
      {
        lo = mid;
      }
      else
      {
        hi = mid;
      }
    }
    seg = lo;
  }
  __syncthreads();
  const ZeroSeg   s    = segs[seg];
  const long long base = (static_cast<long long>(blockIdx.x) - block_prefix[seg]) * kZeroTile;
  const long long end  = base + kZeroTile < s.n ? base + kZeroTile : s.n;
  for (long long i = base + threadIdx.x; i < end; i += blockDim.x)
  {
    s.ptr[i] = 0.0;
  }
}

// kMode: 0 = FP64, 1 = FP32 quadrature, 2 = MIXED (Jacobian from FP32
// quadrature; residual and the P1 gradients from FP64 element math; the
// Taylor-Hood state VJP J^T lam uses the FP32 Jacobian it transposes).
constexpr int kModeFp64  = 0;
constexpr int kModeFp32  = 1;
constexpr int kModeMixed = 2;

// Elements of an instance in a launch: all of them, or, in a coloured run,
// those of colour `round` (none once the instance's colours are exhausted).
__device__ __forceinline__ int roundElems(const BatchDesc& d, int round)
{
  if (round < 0)
  {
    return d.num_elems;
  }
  return round < d.num_colours ? d.colour_off[round + 1] - d.colour_off[round] : 0;
}

__device__ __forceinline__ int chunksOf(const BatchDesc& d, int p1_chunk, int th_chunk,
                                        int round)
{
  const int c = d.kind == GBFEM_BATCH_P1_KAPPA ? p1_chunk : th_chunk;
  return (roundElems(d, round) + c - 1) / c;
}

// Staging of the next work item (depth 1): the byte ranges of its element
// DOF table and connectivity (and the P1 coefficients) are prefetched into
// L2 while the current item runs, so that its first dependent gathers hit.
__device__ __forceinline__ void prefetchL2(const void* p, long long bytes)
{
  const char* c = static_cast<const char*>(p);
  for (long long off = static_cast<long long>(threadIdx.x) * 128; off < bytes;
       off += static_cast<long long>(blockDim.x) * 128)
  {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(c + off));
  }
}

// MIXED: the Taylor-Hood residuals of every instance (double-float on the
// FP32 pipe) in one flat launch after the persistent kernel, one thread per
// element (inside the persistent kernel its registers would cut the
// occupancy of the other work items).
__global__ void __launch_bounds__(kBatchThreads)
    thResidualBatchKernel(const BatchDesc* __restrict__ descs, const int* __restrict__ th_idx,
                          const long long* __restrict__ th_prefix, int nth)
{
  const long long g = blockIdx.x * static_cast<long long>(kBatchThreads) + threadIdx.x;
  if (g >= th_prefix[nth])
  {
    return;
  }
  int lo = 0, hi = nth;
  while (hi - lo > 1)
  {
    const int mid = (lo + hi) >> 1;
    if (th_prefix[mid] <= g)
    {
      lo = mid;
    }
    else
    {
      hi = mid;
    }
  }
  thResidualDFElem(descs[th_idx[lo]].th, static_cast<int>(g - th_prefix[lo]));
}

// Elements [e0, e1) of an instance, or of its colour list (elems != null:
// coloured run, plain adds).
template <int kMode, bool kSep, bool kLoad, bool kVjp, bool kPlain>
__device__ __forceinline__ void p1Chunk(const P1Args& a, int e0, int e1, const int* elems)
{
  for (int i = e0 + static_cast<int>(threadIdx.x); i < e1; i += kBatchThreads)
  {
    const int e = kPlain ? elems[i] : i;
    if (kMode == kModeFp64)
    {
      p1Element<false, kSep, kLoad, true, true, kVjp, kPlain>(a, e);
    }
    else if (kMode == kModeFp32)
    {
      p1Element<true, kSep, kLoad, true, true, kVjp, kPlain>(a, e);
    }
    else
    {
      p1Element<true, kSep, false, true, false, false, kPlain>(a, e);
      p1Element<false, kSep, kLoad, false, true, kVjp, kPlain>(a, e);
    }
  }
}

template <int kMode, bool kSep, bool kPlain>
__device__ __forceinline__ void p1Dispatch(const P1Args& a, int e0, int e1, const int* elems)
{
  const bool load = a.f != nullptr, vjp = a.lam != nullptr;
  if (load)
  {
    vjp ? p1Chunk<kMode, kSep, true, true, kPlain>(a, e0, e1, elems)
        : p1Chunk<kMode, kSep, true, false, kPlain>(a, e0, e1, elems);
  }
  else
  {
    vjp ? p1Chunk<kMode, kSep, false, true, kPlain>(a, e0, e1, elems)
        : p1Chunk<kMode, kSep, false, false, kPlain>(a, e0, e1, elems);
  }
}

// Taylor-Hood staging of each precision mode.
template <int kMode>
struct BatchSmem;
template <>
struct BatchSmem<kModeFp64>
{
  using type = ThSmem<double>;
};
template <>
struct BatchSmem<kModeFp32>
{
  using type = ThSmem<float>;
};
template <>
struct BatchSmem<kModeMixed>
{
  using type = ThSmem<float>;
};

// Where a work item lies: instance `inst`, its element range [e0, e1) (in
// the instance's colour list for a coloured run).
struct BatchItem
{
  int inst, e0, e1;
};

__device__ __forceinline__ BatchItem decodeItem(const int* prefix, int ni, int it,
                                                const BatchDesc* descs, int p1_chunk,
                                                int th_chunk, int round)
{
  int lo = 0, hi = ni;
  while (hi - lo > 1)
  {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= it)
    {
      lo = mid;
    }
    else
    {
      hi = mid;
    }
  }
  const BatchDesc& d     = descs[lo];
  const int        chunk = d.kind == GBFEM_BATCH_P1_KAPPA ? p1_chunk : th_chunk;
  const int        e0    = (it - prefix[lo]) * chunk;
  return {lo, e0, min(roundElems(d, round), e0 + chunk)};
}

// The next item's element DOF table and connectivity (and P1 coefficients)
// into L2 (the staging of depth 1).
__device__ __forceinline__ void stageItem(const BatchDesc& d, const BatchItem& w, int round)
{
  if (round >= 0)
  {
    return; // coloured runs gather through the colour list
  }
  const long long n = w.e1 - w.e0;
  if (d.kind == GBFEM_BATCH_P1_KAPPA)
  {
    prefetchL2(d.p1.dofs + 3LL * w.e0, 12 * n);
    prefetchL2(d.p1.kappa + w.e0, 8 * n);
    if (d.p1.conn != nullptr)
    {
      prefetchL2(d.p1.conn + 3LL * w.e0, 12 * n);
    }
  }
  else
  {
    prefetchL2(d.th.dofs + 15LL * w.e0, 60 * n);
    prefetchL2(d.th.conn6 + 6LL * w.e0, 24 * n);
  }
}

// FP32 and MIXED: at least six resident blocks per SM (at most 80 registers;
// left free, the compiler takes 128-147 and four blocks fit, and the
// kernel, which waits mostly on its dependent gathers, runs 3 % slower).
// round < 0: every element of every instance, FP64 reductions; round >= 0
// (kPlain): the elements of colour `round` of each instance, plain adds
// (elements of one colour share no DOF), one launch per colour. kStage: work
// items claimed this many ahead, their inputs prefetched into L2 (0 or 1).
template <int kMode, bool kPlain, int kStage>
__global__ void __launch_bounds__(kBatchThreads, kMode == kModeFp64 ? 1 : 6)
    batchKernel(const BatchDesc* __restrict__ descs, int ni, int p1_chunk, int th_chunk,
                int* __restrict__ ticket, int round)
{
  __shared__ typename BatchSmem<kMode>::type sm;
  __shared__ int                             prefix[kMaxInstances + 1];
  __shared__ int                             item[2];
  // every instance reports into the batch's one status word
  DeviceStatus* status = ni > 0 ? (descs[0].kind == GBFEM_BATCH_P1_KAPPA ? descs[0].p1.status
                                                                          : descs[0].th.status)
                                : nullptr;
  thStageRef(sm, status);
  if (threadIdx.x == 0)
  {
    int acc = 0;
    for (int i = 0; i < ni; ++i)
    {
      prefix[i] = acc;
      acc += chunksOf(descs[i], p1_chunk, th_chunk, round);
    }
    prefix[ni] = acc;
    item[0]    = atomicAdd(ticket, 1);
  }
  __syncthreads();
  const int total = prefix[ni];
  for (int k = 0;; k ^= 1)
  {
    const int it = item[k];
    if (it >= total)
    {
      break;
    }
    if (kStage > 0)
    {
      // claim the next item now and stage its inputs while this one runs
      if (threadIdx.x == 0)
      {
        item[k ^ 1] = atomicAdd(ticket, 1);
      }
      __syncthreads();
      const int nx = item[k ^ 1];
      if (nx < total)
      {
        const BatchItem w = decodeItem(prefix, ni, nx, descs, p1_chunk, th_chunk, round);
        stageItem(descs[w.inst], w, round);
      }
    }
    const BatchItem  w  = decodeItem(prefix, ni, it, descs, p1_chunk, th_chunk, round);
    const BatchDesc& d  = descs[w.inst];
    const int*       el = kPlain ? d.colour_elems + d.colour_off[round] : nullptr;
    if (d.kind == GBFEM_BATCH_P1_KAPPA)
    {
      d.p1.conn != nullptr ? p1Dispatch<kMode, true, kPlain>(d.p1, w.e0, w.e1, el)
                           : p1Dispatch<kMode, false, kPlain>(d.p1, w.e0, w.e1, el);
    }
    else
    {
      ThArgs tc; // the coloured run's view of the instance
      if (kPlain)
      {
        tc       = d.th;
        tc.elems = el;
        tc.ne    = roundElems(d, round);
      }
      const ThArgs& ta  = kPlain ? tc : d.th;
      const bool    vjp = ta.lam != nullptr;
      for (int eb = w.e0; eb < w.e1; eb += kElemsPerBlock)
      {
        if constexpr (kMode == kModeFp64)
        {
          vjp ? thBlock<double, true, true, true, false, false, kPlain>(ta, eb, sm)
              : thBlock<double, true, true, false, false, false, kPlain>(ta, eb, sm);
        }
        else if constexpr (kMode == kModeFp32)
        {
          vjp ? thBlock<float, true, true, true, false, false, kPlain>(ta, eb, sm)
              : thBlock<float, true, true, false, false, false, kPlain>(ta, eb, sm);
        }
        else
        {
          vjp ? thBlock<float, true, false, true, false, false, kPlain>(ta, eb, sm)
              : thBlock<float, true, false, false, false, false, kPlain>(ta, eb, sm);
        }
      }
    }
    if (kStage == 0)
    {
      __syncthreads(); // everyone has read item[k] before it is reused
      if (threadIdx.x == 0)
      {
        item[k ^ 1] = atomicAdd(ticket, 1);
      }
      __syncthreads();
    }
    else
    {
      __syncthreads(); // item[k] is free for the claim after next
    }
  }
}

} // namespace

struct gbfem_batch
{
  int                  num_instances = 0;
  int                  sm_count      = 0;
  BatchDesc*           d_descs       = nullptr;
  ZeroSeg*             d_segs        = nullptr;
  long long*           d_block_prefix = nullptr;
  int                  nseg          = 0;
  long long            zero_blocks   = 0;
  int*                 d_ticket      = nullptr;
  gbfem::DeviceStatus* d_status      = nullptr;
  long long            total_elems   = 0;
  int                  nth           = 0;       // Taylor-Hood instances
  long long            th_elems      = 0;
  int*                 d_th_idx      = nullptr; // their descriptor indices
  long long*           d_th_prefix   = nullptr; // [nth + 1] element offsets
  bool                 all_coloured  = false;   // every instance's map coloured at creation
  int                  max_colours   = 0;

  ~gbfem_batch()
  {
    gbfem::deviceFree(d_th_idx);
    gbfem::deviceFree(d_th_prefix);
    gbfem::deviceFree(d_descs);
    gbfem::deviceFree(d_segs);
    gbfem::deviceFree(d_block_prefix);
    gbfem::deviceFree(d_ticket);
    gbfem::deviceFree(d_status);
  }
};

extern "C" int gbfem_batch_create(int n, const gbfem_batch_instance* inst, void* stream,
                                  gbfem_batch** out)
{
  using namespace gbfem;
  return guarded([&] {
    require(out != nullptr, "batch output handle is null");
    *out = nullptr;
    require(n > 0 && n <= kMaxInstances && inst != nullptr,
            "batch instance count must be in 1..1024");
    cudaStream_t s = asStream(stream);
    auto*        b = new gbfem_batch;
    try
    {
      int dev = 0;
      cudaCheck(cudaGetDevice(&dev), "cudaGetDevice");
      cudaCheck(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev),
                "SM count");
      b->num_instances = n;
      b->d_status      = deviceAlloc<DeviceStatus>(1);
      b->d_ticket      = deviceAlloc<int>(kMaxRounds);
      cudaCheck(cudaMemsetAsync(b->d_status, 0, sizeof(DeviceStatus), s), "memset");
      std::vector<BatchDesc> descs(n);
      std::vector<ZeroSeg>   segs;
      for (int i = 0; i < n; ++i)
      {
        const gbfem_batch_instance& x = inst[i];
        const gbfem_assembly_map*   m = x.map;
        require(m != nullptr && x.coords != nullptr && x.state != nullptr && x.res != nullptr,
                "batch instance inputs must not be null");
        require((reinterpret_cast<uintptr_t>(x.coords) & 15) == 0,
                "Geometry coordinates must be 16-byte aligned");
        require(m->num_res == m->num_states && m->same_dofs,
                "batch instances need identical residual and state DOF tables");
        BatchDesc& d   = descs[i];
        d              = BatchDesc{};
        d.kind         = x.kind;
        d.num_elems    = m->num_elems;
        d.num_colours  = m->num_colours;
        d.colour_off   = m->colour_off;
        d.colour_elems = m->colour_elems;
        if (i == 0)
        {
          b->all_coloured = true;
        }
        b->all_coloured = b->all_coloured && (m->num_elems == 0 || m->colour_elems != nullptr);
        b->max_colours  = std::max(b->max_colours, m->num_colours);
        b->total_elems += m->num_elems;
        if (x.kind == GBFEM_BATCH_P1_KAPPA)
        {
          require(m->num_elems == 0 || (m->uniform_res == 3 && m->uniform_state == 3),
                  "KappaPoissonP1 expects three DOFs per element");
          require(x.kappa != nullptr, "batch P1 instance needs kappa");
          require(x.conn != nullptr || x.num_nodes == m->num_states,
                  "Geometry and AssemblyMap have different node counts");
          P1Args& a   = d.p1;
          a.ne        = m->num_elems;
          a.num_nodes = x.num_nodes;
          a.dofs      = m->state_dofs;
          a.conn      = x.conn;
          a.coords    = reinterpret_cast<const double2*>(x.coords);
          a.kappa     = x.kappa;
          a.f         = x.f_nodal;
          a.u         = x.state;
          a.jac_map   = m->jac_map;
          a.row_ptr   = m->row_ptr;
          a.jac_pos   = m->pos_stride == 4 ? reinterpret_cast<const unsigned*>(m->jac_pos)
                                           : nullptr;
          a.res       = x.res;
          a.vals      = x.vals;
          a.lam       = x.lam;
          a.g_u       = x.lam != nullptr ? x.g_state : nullptr;
          a.g_m       = x.lam != nullptr ? x.g_control : nullptr;
          a.status    = b->d_status;
          require(x.vals != nullptr, "batch instance needs matrix values");
        }
        else if (x.kind == GBFEM_BATCH_TH_NS)
        {
          require(m->num_elems == 0 || (m->uniform_res == 15 && m->uniform_state == 15),
                  "Taylor-Hood element expects 15 DOFs per element");
          require(x.conn != nullptr && x.vals != nullptr,
                  "batch Taylor-Hood instance needs conn6 and matrix values");
          require(x.lam == nullptr || x.g_state != nullptr,
                  "batch Taylor-Hood VJP needs a state-gradient output");
          ThArgs& a   = d.th;
          a.ne        = m->num_elems;
          a.num_nodes = x.num_nodes;
          a.dofs      = m->state_dofs;
          a.conn6     = x.conn;
          a.coords    = reinterpret_cast<const double2*>(x.coords);
          a.nu        = x.nu;
          a.state     = x.state;
          a.row_ptr   = m->row_ptr;
          a.jac_pos   = m->pos_stride == 16 ? m->jac_pos : nullptr;
          a.jac_map   = m->jac_map;
          a.res       = x.res;
          a.vals      = x.vals;
          a.lam       = x.lam;
          a.g_state   = x.g_state;
          a.status    = b->d_status;
        }
        else
        {
          throw Error(GBFEM_EINVAL, "unknown batch instance kind");
        }
        segs.push_back({x.res, m->num_res});
        segs.push_back({x.vals, m->nnz});
        if (x.lam != nullptr && x.g_state != nullptr)
        {
          segs.push_back({x.g_state, m->num_states});
        }
      }
      std::vector<ZeroSeg>   nonempty;
      std::vector<long long> prefix;
      long long              acc = 0;
      for (const auto& z : segs)
      {
        if (z.n > 0)
        {
          nonempty.push_back(z);
          prefix.push_back(acc);
          acc += (z.n + kZeroTile - 1) / kZeroTile;
        }
      }
      std::vector<int>       th_idx;
      std::vector<long long> th_prefix{0};
      for (int i = 0; i < n; ++i)
      {
        if (descs[i].kind == GBFEM_BATCH_TH_NS)
        {
          th_idx.push_back(i);
          th_prefix.push_back(th_prefix.back() + descs[i].num_elems);
        }
      }
      b->nth         = static_cast<int>(th_idx.size());
      b->th_elems    = th_prefix.back();
      b->d_th_idx    = deviceAlloc<int>(b->nth);
      b->d_th_prefix = deviceAlloc<long long>(b->nth + 1LL);
      if (b->nth > 0)
      {
        cudaCheck(cudaMemcpyAsync(b->d_th_idx, th_idx.data(), sizeof(int) * b->nth,
                                  cudaMemcpyHostToDevice, s),
                  "batch upload");
      }
      cudaCheck(cudaMemcpyAsync(b->d_th_prefix, th_prefix.data(),
                                sizeof(long long) * (b->nth + 1), cudaMemcpyHostToDevice, s),
                "batch upload");
      cudaCheck(cudaStreamSynchronize(s), "batch upload");
      b->nseg        = static_cast<int>(nonempty.size());
      b->zero_blocks = acc;
      b->d_descs     = deviceAlloc<BatchDesc>(n);
      b->d_segs      = deviceAlloc<ZeroSeg>(b->nseg);
      b->d_block_prefix = deviceAlloc<long long>(b->nseg);
      cudaCheck(cudaMemcpyAsync(b->d_descs, descs.data(), sizeof(BatchDesc) * n,
                                cudaMemcpyHostToDevice, s),
                "batch descriptor upload");
      if (b->nseg > 0)
      {
        cudaCheck(cudaMemcpyAsync(b->d_segs, nonempty.data(), sizeof(ZeroSeg) * b->nseg,
                                  cudaMemcpyHostToDevice, s),
                  "batch segment upload");
        cudaCheck(cudaMemcpyAsync(b->d_block_prefix, prefix.data(),
                                  sizeof(long long) * b->nseg, cudaMemcpyHostToDevice, s),
                  "batch segment upload");
      }
      cudaCheck(cudaStreamSynchronize(s), "batch setup");
    }
    catch (...)
    {
      delete b;
      throw;
    }
    *out = b;
  });
}

extern "C" int gbfem_batch_run(gbfem_batch* b, int precision, int p1_chunk, int th_chunk,
                               int blocks_per_sm, int stage_depth, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(b != nullptr, "batch handle is null");
    const bool col = (precision & GBFEM_COLOURED) != 0;
    precision &= ~GBFEM_COLOURED;
    require(precision >= GBFEM_PREC_FP64 && precision <= GBFEM_PREC_MIXED,
            "unknown precision mode");
    require(!col || b->all_coloured,
            "coloured batch runs need gbfem_assembly_map_enable_colouring on every "
            "instance's map before gbfem_batch_create");
    require(!col || precision != GBFEM_PREC_MIXED,
            "coloured batch runs take FP64 or FP32_QUAD");
    require(p1_chunk >= kBatchThreads && p1_chunk % kBatchThreads == 0,
            "p1_chunk must be a positive multiple of 128");
    require(th_chunk >= kElemsPerBlock && th_chunk % kElemsPerBlock == 0,
            "th_chunk must be a positive multiple of 8");
    require(blocks_per_sm >= 1 && blocks_per_sm <= 32, "blocks_per_sm must be in 1..32");
    require(stage_depth == 0 || stage_depth == 1, "stage_depth must be 0 or 1");
    cudaStream_t s = asStream(stream);
    if (b->zero_blocks > 0)
    {
      zeroSegments<<<static_cast<unsigned>(b->zero_blocks), 256, 0, s>>>(
          b->d_segs, b->d_block_prefix, b->nseg, b->d_ticket);
    }
    else
    {
      cudaCheck(cudaMemsetAsync(b->d_ticket, 0, sizeof(int) * kMaxRounds, s), "ticket reset");
    }
    cudaCheck(cudaGetLastError(), "batch zero launch");
    const unsigned grid = static_cast<unsigned>(b->sm_count * blocks_per_sm);
    const int      nr   = col ? b->max_colours : 1;
    for (int r = 0; r < nr; ++r)
    {
      const int round = col ? r : -1;
      int*      tk    = b->d_ticket + r;
      auto      go    = [&](auto kernel) {
        kernel<<<grid, kBatchThreads, 0, s>>>(b->d_descs, b->num_instances, p1_chunk, th_chunk,
                                              tk, round);
      };
      if (precision == GBFEM_PREC_FP64)
      {
        col ? go(batchKernel<kModeFp64, true, 0>)
            : (stage_depth ? go(batchKernel<kModeFp64, false, 1>)
                           : go(batchKernel<kModeFp64, false, 0>));
      }
      else if (precision == GBFEM_PREC_FP32_QUAD)
      {
        col ? go(batchKernel<kModeFp32, true, 0>)
            : (stage_depth ? go(batchKernel<kModeFp32, false, 1>)
                           : go(batchKernel<kModeFp32, false, 0>));
      }
      else
      {
        stage_depth ? go(batchKernel<kModeMixed, false, 1>)
                    : go(batchKernel<kModeMixed, false, 0>);
      }
      cudaCheck(cudaGetLastError(), "batch launch");
    }
    if (precision == GBFEM_PREC_MIXED && b->th_elems > 0)
    {
      thResidualBatchKernel<<<static_cast<unsigned>((b->th_elems + kBatchThreads - 1)
                                                    / kBatchThreads),
                              kBatchThreads, 0, s>>>(b->d_descs, b->d_th_idx, b->d_th_prefix,
                                                     b->nth);
      cudaCheck(cudaGetLastError(), "batch launch");
    }
  });
}

extern "C" int gbfem_batch_check(const gbfem_batch* b, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(b != nullptr, "batch handle is null");
    cudaStream_t s = asStream(stream);
    try
    {
      checkDeviceStatus(b->d_status, s);
    }
    catch (...)
    {
      cudaMemsetAsync(b->d_status, 0, sizeof(DeviceStatus), s);
      cudaStreamSynchronize(s);
      throw;
    }
  });
}

extern "C" long long gbfem_batch_num_elems(const gbfem_batch* b)
{
  return b != nullptr ? b->total_elems : 0;
}

extern "C" void gbfem_batch_destroy(gbfem_batch* b)
{
  delete b;
}
