// pattern.cu — GPU build of femx's AssemblyMap: element DOF tables in,
// CSR pattern + jac_map out, bit-identical to makeAssemblyMap
// (femx/assembly/AssemblyMap.cpp:54-176).
//
// The reference forms the COO list of every element block, sorts it globally
// and merges duplicates. Here each CSR row owns its candidate columns:
//   1. count, per row, the candidate columns contributed by element blocks;
//   2. bucket every (element, row, col) candidate under its row;
//   3. per row (one warp): mark the first occurrence of each column, count
//      the distinct columns -> row_ptr by scan;
//   4. per row: rank each candidate among the distinct columns; the rank is
//      its CSR slot, written to jac_map at the candidate's local entry.
// The result depends only on the set of (row, col) pairs, so it equals the
// reference's sort-based result exactly, whatever the bucketing order.
#include <algorithm>
#include <atomic>
#include <climits>

#include "maps.cuh"

namespace
{

using gbfem::DeviceStatus;

constexpr int kWarpsPerBlock = 8;
constexpr int kStageCap      = 512; // candidates staged in shared memory per warp
constexpr int kGatherMaxRowEntries = 256; // in-row positions are bytes

// Offsets must start at 0 and be non-decreasing; checked before any DOF
// table is read, so no later kernel can index past the copied tables.
__global__ void validateOffsets(int ne, const int* __restrict__ ro,
                                const int* __restrict__ so, DeviceStatus* st)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne)
  {
    return;
  }
  if (ro[e + 1] < ro[e] || so[e + 1] < so[e] || (e == 0 && (ro[0] != 0 || so[0] != 0)))
  {
    gbfem::devFail(st, gbfem::kDevNegativeLocal, e);
  }
}

__global__ void countCandidates(int ne, int num_res, int num_states,
                                const int* __restrict__ ro,
                                const int* __restrict__ rd,
                                const int* __restrict__ so,
                                const int* __restrict__ sd,
                                long long* __restrict__ elem_jac,
                                int* __restrict__ row_cand,
                                int* __restrict__ stats, DeviceStatus* st)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne)
  {
    return;
  }
  const int r0 = ro[e], r1 = ro[e + 1], s0 = so[e], s1 = so[e + 1];
  const int nr = r1 - r0, nc = s1 - s0;
  elem_jac[e] = static_cast<long long>(nr) * nc;
  atomicMax(&stats[0], nr);
  atomicMax(&stats[1], nc);
  atomicMin(&stats[2], nr);
  atomicMin(&stats[3], nc);
  for (int i = r0; i < r1; ++i)
  {
    const int dof = rd[i];
    if (dof < 0 || dof >= num_res)
    {
      gbfem::devFail(st, gbfem::kDevResDofRange, i);
      continue;
    }
    atomicAdd(&row_cand[dof], nc);
  }
  for (int j = s0; j < s1; ++j)
  {
    const int dof = sd[j];
    if (dof < 0 || dof >= num_states)
    {
      gbfem::devFail(st, gbfem::kDevStateDofRange, j);
    }
  }
}

__global__ void bucketCandidates(int ne, const int* __restrict__ ro,
                                 const int* __restrict__ rd,
                                 const int* __restrict__ so,
                                 const int* __restrict__ sd,
                                 const int* __restrict__ jac_offsets,
                                 const int* __restrict__ cand_off,
                                 int* __restrict__ cursor,
                                 int* __restrict__ cand_col,
                                 int* __restrict__ cand_src)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne)
  {
    return;
  }
  const int r0 = ro[e], nr = ro[e + 1] - r0;
  const int s0 = so[e], nc = so[e + 1] - s0;
  const int j0 = jac_offsets[e];
  for (int i = 0; i < nr; ++i)
  {
    const int row  = rd[r0 + i];
    const int slot = cand_off[row] + atomicAdd(&cursor[row], nc);
    for (int j = 0; j < nc; ++j)
    {
      cand_col[slot + j] = sd[s0 + j];
      cand_src[slot + j] = j0 + i * nc + j;
    }
  }
}

// Phase 3: first-occurrence flags and distinct-column count per row.
__global__ void markDistinct(int num_res, const int* __restrict__ cand_off,
                             const int* __restrict__ cand_col,
                             unsigned char* __restrict__ first,
                             int* __restrict__ row_nnz)
{
  __shared__ int stage[kWarpsPerBlock][kStageCap];
  const int      lane = threadIdx.x & 31;
  const int      w    = threadIdx.x >> 5;
  const int      row  = blockIdx.x * kWarpsPerBlock + w;
  if (row >= num_res)
  {
    return;
  }
  const int  beg    = cand_off[row];
  const int  n      = cand_off[row + 1] - beg;
  const int* src    = cand_col + beg;
  const bool staged = n <= kStageCap;
  if (staged)
  {
    for (int k = lane; k < n; k += 32)
    {
      stage[w][k] = src[k];
    }
    __syncwarp();
    src = stage[w];
  }
  int count = 0;
  for (int k = lane; k < n; k += 32)
  {
    const int c  = src[k];
    bool      fr = true;
    for (int j = 0; j < k; ++j)
    {
      if (src[j] == c)
      {
        fr = false;
        break;
      }
    }
    first[beg + k] = fr ? 1 : 0;
    count += fr ? 1 : 0;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
  {
    count += __shfl_xor_sync(0xffffffffu, count, off);
  }
  if (lane == 0)
  {
    row_nnz[row] = count;
  }
}

// Phase 4: rank among distinct columns -> CSR slot; write col_ind, jac_map.
__global__ void rankColumns(int num_res, const int* __restrict__ cand_off,
                            const int* __restrict__ cand_col,
                            const int* __restrict__ cand_src,
                            const unsigned char* __restrict__ first,
                            const int* __restrict__ row_ptr,
                            int* __restrict__ col_ind,
                            int* __restrict__ jac_map)
{
  __shared__ int stage[kWarpsPerBlock][kStageCap];
  __shared__ unsigned char fstage[kWarpsPerBlock][kStageCap];
  const int                lane = threadIdx.x & 31;
  const int                w    = threadIdx.x >> 5;
  const int                row  = blockIdx.x * kWarpsPerBlock + w;
  if (row >= num_res)
  {
    return;
  }
  const int            beg    = cand_off[row];
  const int            n      = cand_off[row + 1] - beg;
  const int*           src    = cand_col + beg;
  const unsigned char* fl     = first + beg;
  const bool           staged = n <= kStageCap;
  if (staged)
  {
    for (int k = lane; k < n; k += 32)
    {
      stage[w][k]  = src[k];
      fstage[w][k] = fl[k];
    }
    __syncwarp();
    src = stage[w];
    fl  = fstage[w];
  }
  const int base = row_ptr[row];
  for (int k = lane; k < n; k += 32)
  {
    const int c    = src[k];
    int       rank = 0;
    for (int j = 0; j < n; ++j)
    {
      rank += (fl[j] != 0 && src[j] < c) ? 1 : 0;
    }
    const int pos          = base + rank;
    jac_map[cand_src[beg + k]] = pos;
    if (fl[k] != 0)
    {
      col_ind[pos] = c;
    }
  }
}

// Largest in-row position of every local entry (decides the compact map).
__global__ void maxInRowPos(int ne, int nr, int nc, const int* __restrict__ rd,
                            const int* __restrict__ row_ptr,
                            const int* __restrict__ jac_map, int* __restrict__ mx)
{
  const long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<long long>(ne) * nr)
  {
    return;
  }
  const int rs = row_ptr[rd[t]];
  int       m  = 0;
  for (int j = 0; j < nc; ++j)
  {
    m = max(m, jac_map[t * nc + j] - rs);
  }
  atomicMax(mx, m);
}

// Row-major (stride 4): byte j of record (e, i) is entry (i, j).
// Column-major (stride >= 16): byte i of record (e, j) is entry (i, j), so
// the lane that scatters local column j loads all its rows' positions with
// one 16-byte load. Padding bytes are zeroed by the caller.
__global__ void fillInRowPos(int ne, int nr, int nc, int stride, bool col_major,
                             const int* __restrict__ rd,
                             const int* __restrict__ row_ptr,
                             const int* __restrict__ jac_map,
                             unsigned char* __restrict__ pos)
{
  const long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (t >= static_cast<long long>(ne) * nr)
  {
    return;
  }
  const int rs = row_ptr[rd[t]];
  if (col_major)
  {
    const long long e = t / nr;
    const int       i = static_cast<int>(t - e * nr);
    for (int j = 0; j < nc; ++j)
    {
      pos[(e * nc + j) * stride + i] = static_cast<unsigned char>(jac_map[t * nc + j] - rs);
    }
    return;
  }
  for (int j = 0; j < stride; ++j)
  {
    pos[t * stride + j] =
        j < nc ? static_cast<unsigned char>(jac_map[t * nc + j] - rs) : 0;
  }
}

// Row-gather tables: records per residual row, placed, then each row's
// records put in ascending (e, i) order, so the numbering is deterministic.
__global__ void countGatherRows(long long n, const int* __restrict__ rd, int* __restrict__ cnt)
{
  const long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (t < n)
  {
    atomicAdd(cnt + rd[t], 1);
  }
}

__global__ void placeGatherRecords(long long n, const int* __restrict__ rd,
                                   const int* __restrict__ off, int* __restrict__ fill,
                                   int* __restrict__ keys)
{
  const long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (t < n)
  {
    const int r                        = rd[t];
    keys[off[r] + atomicAdd(fill + r, 1)] = static_cast<int>(t);
  }
}

__global__ void sortGatherRows(int num_res, const int* __restrict__ off, int* __restrict__ keys)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= num_res)
  {
    return;
  }
  for (int a = off[r] + 1; a < off[r + 1]; ++a)
  {
    const int v = keys[a];
    int       b = a - 1;
    while (b >= off[r] && keys[b] > v)
    {
      keys[b + 1] = keys[b];
      --b;
    }
    keys[b + 1] = v;
  }
}

__global__ void fillGatherRecords(long long n, int nc, const int* __restrict__ keys,
                                  const int* __restrict__ rd, const int* __restrict__ row_ptr,
                                  const int* __restrict__ jac_map, int* __restrict__ slot,
                                  unsigned char* __restrict__ pos)
{
  const long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (k >= n)
  {
    return;
  }
  const int t  = keys[k];
  slot[t]      = static_cast<int>(k);
  const int rs = row_ptr[rd[t]];
  for (int j = 0; j < 16; ++j)
  {
    pos[k * 16 + j] = j < nc ? static_cast<unsigned char>(jac_map[static_cast<long long>(t) * nc + j] - rs) : 0;
  }
}

__global__ void compareTables(long long n, const int* __restrict__ a,
                              const int* __restrict__ b, int* __restrict__ diff)
{
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < n && a[i] != b[i])
  {
    *diff = 1;
  }
}

template <class T>
void copyIn(T*& dst, const T* src, long long n, cudaStream_t s)
{
  dst = gbfem::deviceAlloc<T>(n);
  if (n > 0)
  {
    gbfem::cudaCheck(cudaMemcpyAsync(dst, src, sizeof(T) * n,
                                     cudaMemcpyDeviceToDevice, s),
                     "AssemblyMap table copy");
  }
}

struct Scratch
{
  void* p[8] = {};
  ~Scratch()
  {
    for (void* q : p)
    {
      gbfem::deviceFree(q);
    }
  }
};

void buildGatherTables(gbfem_assembly_map* m, cudaStream_t s)
{
  using gbfem::blocksFor;
  using gbfem::cudaCheck;
  using gbfem::deviceAlloc;
  const int       nr = m->uniform_res, nc = m->uniform_state;
  const long long n  = static_cast<long long>(m->num_elems) * nr;
  Scratch         tmp;
  int*            cnt  = deviceAlloc<int>(m->num_res + 1LL);
  tmp.p[0]             = cnt;
  int*            keys = deviceAlloc<int>(n);
  tmp.p[1]             = keys;
  cudaCheck(cudaMemsetAsync(cnt, 0, sizeof(int) * (m->num_res + 1LL), s), "memset");
  countGatherRows<<<blocksFor(n, 256), 256, 0, s>>>(n, m->res_dofs, cnt);
  cudaCheck(cudaGetLastError(), "gather count launch");
  m->gather_off = deviceAlloc<int>(m->num_res + 1LL);
  gbfem::exclusiveScan(cnt, m->gather_off, m->num_res, s);
  cudaCheck(cudaMemsetAsync(cnt, 0, sizeof(int) * (m->num_res + 1LL), s), "memset");
  placeGatherRecords<<<blocksFor(n, 256), 256, 0, s>>>(n, m->res_dofs, m->gather_off, cnt, keys);
  sortGatherRows<<<blocksFor(m->num_res, 256), 256, 0, s>>>(m->num_res, m->gather_off, keys);
  m->gather_slot = deviceAlloc<int>(n);
  m->gather_pos  = deviceAlloc<unsigned char>(n * 16);
  fillGatherRecords<<<blocksFor(n, 256), 256, 0, s>>>(n, nc, keys, m->res_dofs, m->row_ptr,
                                                      m->jac_map, m->gather_slot,
                                                      m->gather_pos);
  cudaCheck(cudaGetLastError(), "gather fill launch");
  m->gather_eb      = deviceAlloc<double>(n * 16);
  m->gather_res     = deviceAlloc<double>(n);
  m->gather_records = static_cast<int>(n);
  cudaCheck(cudaStreamSynchronize(s), "gather tables");
}

} // namespace

gbfem_assembly_map::~gbfem_assembly_map()
{
  for (int* p : {res_offsets, res_dofs, state_offsets, state_dofs, jac_offsets,
                 jac_map, row_ptr, col_ind, gather_off, gather_slot, colour_off,
                 colour_elems, tile_row_off, tile_run_off, tile_elem_off, tile_elems,
                 tile_vert_off, tile_vert_dof, tile_vert_node})
  {
    gbfem::deviceFree(p);
  }
  gbfem::deviceFree(tile_row_info);
  gbfem::deviceFree(tile_runs);
  gbfem::deviceFree(tile_conn);
  gbfem::deviceFree(slot_ref);
  gbfem::deviceFree(status);
  gbfem::deviceFree(jac_pos);
  gbfem::deviceFree(jac_pos_rows);
  gbfem::deviceFree(gather_pos);
  gbfem::deviceFree(gather_eb);
  gbfem::deviceFree(gather_res);
}

namespace gbfem
{
unsigned long long nextLayoutId()
{
  static std::atomic<unsigned long long> next{1};
  return next++;
}
} // namespace gbfem

extern "C" int gbfem_assembly_map_create(int num_res, int num_states,
                                         int num_elems, const int* res_offsets,
                                         const int* res_dofs,
                                         const int* state_offsets,
                                         const int* state_dofs, void* stream,
                                         gbfem_assembly_map** out)
{
  using namespace gbfem;
  return guarded([&] {
    require(out != nullptr, "AssemblyMap output handle is null");
    *out = nullptr;
    require(num_res >= 0 && num_states >= 0,
            "AssemblyMap global dimensions must be non-negative");
    require(num_elems >= 0, "AssemblyMap residual/state element counts differ");
    require(num_elems == 0 || (res_offsets && res_dofs && state_offsets && state_dofs),
            "AssemblyMap element tables must not be null");
    cudaStream_t s = asStream(stream);
    auto* m        = new gbfem_assembly_map;
    try
    {
      m->num_elems  = num_elems;
      m->num_res    = num_res;
      m->num_states = num_states;
      m->layout_id  = nextLayoutId();
      m->status     = deviceAlloc<DeviceStatus>(1);
      cudaCheck(cudaMemsetAsync(m->status, 0, sizeof(DeviceStatus), s), "memset");

      int tot[2] = {0, 0};
      if (num_elems > 0)
      {
        cudaCheck(cudaMemcpyAsync(&tot[0], res_offsets + num_elems, sizeof(int),
                                  cudaMemcpyDeviceToHost, s),
                  "AssemblyMap offsets readback");
        cudaCheck(cudaMemcpyAsync(&tot[1], state_offsets + num_elems, sizeof(int),
                                  cudaMemcpyDeviceToHost, s),
                  "AssemblyMap offsets readback");
        cudaCheck(cudaStreamSynchronize(s), "AssemblyMap offsets readback");
        require(tot[0] >= 0 && tot[1] >= 0,
                "AssemblyMap local dimensions must be non-negative");
      }
      copyIn(m->res_offsets, res_offsets, num_elems + 1LL, s);
      copyIn(m->state_offsets, state_offsets, num_elems + 1LL, s);
      copyIn(m->res_dofs, res_dofs, tot[0], s);
      copyIn(m->state_dofs, state_dofs, tot[1], s);
      if (num_elems == 0)
      {
        cudaCheck(cudaMemsetAsync(m->res_offsets, 0, sizeof(int), s), "memset");
        cudaCheck(cudaMemsetAsync(m->state_offsets, 0, sizeof(int), s), "memset");
      }
      m->row_ptr     = deviceAlloc<int>(num_res + 1LL);
      m->jac_offsets = deviceAlloc<int>(num_elems + 1LL);

      Scratch sc;
      auto* status   = deviceAlloc<DeviceStatus>(1);
      sc.p[0]        = status;
      auto* elem_jac = deviceAlloc<long long>(std::max(num_elems, 1));
      sc.p[1]        = elem_jac;
      auto* row_cand = deviceAlloc<int>(num_res + 1LL);
      sc.p[2]        = row_cand;
      auto* cand_off = deviceAlloc<int>(num_res + 1LL);
      sc.p[3]        = cand_off;
      auto* stats    = deviceAlloc<int>(4);
      sc.p[4]        = stats;
      const int stats_init[4] = {0, 0, INT_MAX, INT_MAX};
      cudaCheck(cudaMemcpyAsync(stats, stats_init, sizeof(stats_init),
                                cudaMemcpyHostToDevice, s),
                "stats init");
      cudaCheck(cudaMemsetAsync(status, 0, sizeof(DeviceStatus), s), "memset");
      cudaCheck(cudaMemsetAsync(row_cand, 0, sizeof(int) * (num_res + 1LL), s),
                "memset");
      if (num_elems > 0)
      {
        validateOffsets<<<blocksFor(num_elems, 256), 256, 0, s>>>(
            num_elems, m->res_offsets, m->state_offsets, status);
        cudaCheck(cudaGetLastError(), "AssemblyMap offsets launch");
      }
      checkDeviceStatus(status, s);
      if (num_elems > 0)
      {
        countCandidates<<<blocksFor(num_elems, 256), 256, 0, s>>>(
            num_elems, num_res, num_states, m->res_offsets, m->res_dofs,
            m->state_offsets, m->state_dofs, elem_jac, row_cand, stats, status);
        cudaCheck(cudaGetLastError(), "AssemblyMap count launch");
      }
      checkDeviceStatus(status, s);
      int st_h[4] = {0, 0, 0, 0};
      cudaCheck(cudaMemcpy(st_h, stats, sizeof(st_h), cudaMemcpyDeviceToHost),
                "stats readback");
      if (num_elems > 0)
      {
        m->max_res       = st_h[0];
        m->max_state     = st_h[1];
        m->uniform_res   = st_h[0] == st_h[2] ? st_h[0] : -1;
        m->uniform_state = st_h[1] == st_h[3] ? st_h[1] : -1;
        const long long mj = static_cast<long long>(st_h[0]) * st_h[1];
        require(mj <= INT_MAX, "AssemblyMap local Jacobian is too large");
        m->max_jac = static_cast<int>(mj);
      }
      // jac_offsets = exclusive scan of element block sizes (checked to fit)
      const long long jac_nnz =
          num_elems > 0 ? exclusiveScan64to32(elem_jac, m->jac_offsets, num_elems, s) : 0;
      if (num_elems == 0)
      {
        cudaCheck(cudaMemsetAsync(m->jac_offsets, 0, sizeof(int), s), "memset");
      }
      m->jac_nnz = static_cast<int>(jac_nnz);
      exclusiveScan(row_cand, cand_off, num_res, s);

      m->jac_map    = deviceAlloc<int>(jac_nnz);
      auto* cand_col = deviceAlloc<int>(jac_nnz);
      sc.p[5]        = cand_col;
      auto* cand_src = deviceAlloc<int>(jac_nnz);
      sc.p[6]        = cand_src;
      auto* first    = deviceAlloc<unsigned char>(jac_nnz);
      sc.p[7]        = first;
      cudaCheck(cudaMemsetAsync(row_cand, 0, sizeof(int) * (num_res + 1LL), s),
                "memset");
      if (num_elems > 0)
      {
        bucketCandidates<<<blocksFor(num_elems, 256), 256, 0, s>>>(
            num_elems, m->res_offsets, m->res_dofs, m->state_offsets,
            m->state_dofs, m->jac_offsets, cand_off, row_cand, cand_col,
            cand_src);
        cudaCheck(cudaGetLastError(), "AssemblyMap bucket launch");
      }
      const unsigned rblocks = blocksFor(num_res, kWarpsPerBlock);
      if (num_res > 0)
      {
        markDistinct<<<rblocks, 32 * kWarpsPerBlock, 0, s>>>(
            num_res, cand_off, cand_col, first, row_cand);
        cudaCheck(cudaGetLastError(), "AssemblyMap distinct launch");
      }
      const long long nnz = exclusiveScan(row_cand, m->row_ptr, num_res, s);
      m->nnz              = static_cast<int>(nnz);
      m->col_ind          = deviceAlloc<int>(nnz);
      if (num_res > 0)
      {
        rankColumns<<<rblocks, 32 * kWarpsPerBlock, 0, s>>>(
            num_res, cand_off, cand_col, cand_src, first, m->row_ptr,
            m->col_ind, m->jac_map);
        cudaCheck(cudaGetLastError(), "AssemblyMap rank launch");
      }
      // Identical residual and state tables (square scalar/mixed layouts)
      // let element kernels read one DOF table instead of two.
      if (tot[0] == tot[1])
      {
        int* diff = deviceAlloc<int>(1);
        cudaCheck(cudaMemsetAsync(diff, 0, sizeof(int), s), "memset");
        compareTables<<<blocksFor(num_elems + 1LL, 256), 256, 0, s>>>(
            num_elems + 1LL, m->res_offsets, m->state_offsets, diff);
        if (tot[0] > 0)
        {
          compareTables<<<blocksFor(tot[0], 256), 256, 0, s>>>(
              tot[0], m->res_dofs, m->state_dofs, diff);
        }
        int diff_h = 1;
        cudaCheck(cudaMemcpyAsync(&diff_h, diff, sizeof(int),
                                  cudaMemcpyDeviceToHost, s),
                  "AssemblyMap compare readback");
        cudaCheck(cudaStreamSynchronize(s), "AssemblyMap compare");
        deviceFree(diff);
        m->same_dofs = diff_h == 0;
      }
      // Compact in-row position map (uniform layouts, rows up to 256 wide).
      if (num_elems > 0 && m->uniform_res > 0 && m->uniform_state > 0)
      {
        const long long rows_tot = static_cast<long long>(num_elems) * m->uniform_res;
        int*            mx       = deviceAlloc<int>(1);
        cudaCheck(cudaMemsetAsync(mx, 0, sizeof(int), s), "memset");
        maxInRowPos<<<blocksFor(rows_tot, 256), 256, 0, s>>>(
            num_elems, m->uniform_res, m->uniform_state, m->res_dofs, m->row_ptr,
            m->jac_map, mx);
        int mx_h = 0;
        cudaCheck(cudaMemcpyAsync(&mx_h, mx, sizeof(int), cudaMemcpyDeviceToHost, s),
                  "AssemblyMap position readback");
        cudaCheck(cudaStreamSynchronize(s), "AssemblyMap position scan");
        deviceFree(mx);
        const int nr = m->uniform_res, nc = m->uniform_state;
        if (mx_h < 256 && (nc <= 4 || nr <= 16))
        {
          const bool      col_major = nc > 4;
          const int       stride    = col_major ? 16 * ((max(nr, nc) + 15) / 16) : 4;
          const long long records   = static_cast<long long>(num_elems) * (col_major ? nc : nr);
          m->pos_stride             = stride;
          m->jac_pos                = deviceAlloc<unsigned char>(records * stride);
          cudaCheck(cudaMemsetAsync(m->jac_pos, 0, records * stride, s), "memset");
          fillInRowPos<<<blocksFor(rows_tot, 256), 256, 0, s>>>(
              num_elems, nr, nc, stride, col_major, m->res_dofs, m->row_ptr,
              m->jac_map, m->jac_pos);
          cudaCheck(cudaGetLastError(), "AssemblyMap position launch");
          if (col_major && nc <= 16)
          {
            // the row-major twin for thread-per-element kernels, which
            // stage one element row at a time
            m->jac_pos_rows = deviceAlloc<unsigned char>(rows_tot * 16);
            cudaCheck(cudaMemsetAsync(m->jac_pos_rows, 0, rows_tot * 16, s), "memset");
            fillInRowPos<<<blocksFor(rows_tot, 256), 256, 0, s>>>(
                num_elems, nr, nc, 16, false, m->res_dofs, m->row_ptr, m->jac_map,
                m->jac_pos_rows);
            cudaCheck(cudaGetLastError(), "AssemblyMap position launch");
          }
        }
        m->max_in_row_pos = mx_h;
      }
      cudaCheck(cudaStreamSynchronize(s), "AssemblyMap build");
    }
    catch (...)
    {
      delete m;
      throw;
    }
    *out = m;
  });
}

extern "C" int gbfem_assembly_map_get_view(const gbfem_assembly_map* m,
                                           gbfem_assembly_map_view* info)
{
  using namespace gbfem;
  return guarded([&] {
    require(m != nullptr && info != nullptr, "AssemblyMap handle is null");
    info->num_elems     = m->num_elems;
    info->num_res       = m->num_res;
    info->num_states    = m->num_states;
    info->nnz           = m->nnz;
    info->jac_nnz       = m->jac_nnz;
    info->max_res       = m->max_res;
    info->max_state     = m->max_state;
    info->max_jac       = m->max_jac;
    info->layout_id     = m->layout_id;
    info->res_offsets   = m->res_offsets;
    info->res_dofs      = m->res_dofs;
    info->state_offsets = m->state_offsets;
    info->state_dofs    = m->state_dofs;
    info->jac_offsets   = m->jac_offsets;
    info->jac_map       = m->jac_map;
    info->row_ptr       = m->row_ptr;
    info->col_ind       = m->col_ind;
  });
}

extern "C" int gbfem_assembly_map_enable_gather(gbfem_assembly_map* m, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(m != nullptr, "AssemblyMap handle is null");
    if (m->gather_off != nullptr || m->num_elems == 0)
    {
      return;
    }
    const int nr = m->uniform_res, nc = m->uniform_state;
    require(nr >= 6 && nr <= 16 && nc >= 6 && nc <= 16 && m->max_in_row_pos >= 0
                && m->max_in_row_pos < kGatherMaxRowEntries,
            "AssemblyMap layout does not support deterministic row-gather assembly "
            "(uniform blocks of 6..16 DOFs and rows up to 256 entries)");
    try
    {
      buildGatherTables(m, asStream(stream));
    }
    catch (...)
    {
      for (void* p : {static_cast<void*>(m->gather_off), static_cast<void*>(m->gather_slot),
                      static_cast<void*>(m->gather_pos), static_cast<void*>(m->gather_eb),
                      static_cast<void*>(m->gather_res)})
      {
        deviceFree(p);
      }
      m->gather_off = m->gather_slot = nullptr;
      m->gather_pos                  = nullptr;
      m->gather_eb = m->gather_res = nullptr;
      m->gather_records            = 0;
      throw;
    }
  });
}

extern "C" void gbfem_assembly_map_destroy(gbfem_assembly_map* m)
{
  delete m;
}

// Greedy element colouring (setup, on the host): elements in ascending
// order take the smallest colour that no element sharing one of their
// residual or state DOFs has taken. A DOF remembers the colours of its
// elements as a 64-bit mask, so one pass over the DOF tables suffices.
extern "C" int gbfem_assembly_map_enable_colouring(gbfem_assembly_map* m, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(m != nullptr, "AssemblyMap handle is null");
    if (m->colour_elems != nullptr || m->num_elems == 0)
    {
      return;
    }
    cudaStream_t      s  = asStream(stream);
    const int         ne = m->num_elems;
    std::vector<int>  ro(ne + 1), so(ne + 1);
    cudaCheck(cudaMemcpyAsync(ro.data(), m->res_offsets, sizeof(int) * (ne + 1),
                              cudaMemcpyDeviceToHost, s),
              "colouring readback");
    cudaCheck(cudaMemcpyAsync(so.data(), m->state_offsets, sizeof(int) * (ne + 1),
                              cudaMemcpyDeviceToHost, s),
              "colouring readback");
    cudaCheck(cudaStreamSynchronize(s), "colouring readback");
    std::vector<int> rd(ro[ne]), sd(so[ne]);
    if (ro[ne] > 0)
    {
      cudaCheck(cudaMemcpyAsync(rd.data(), m->res_dofs, sizeof(int) * ro[ne],
                                cudaMemcpyDeviceToHost, s),
                "colouring readback");
    }
    if (so[ne] > 0)
    {
      cudaCheck(cudaMemcpyAsync(sd.data(), m->state_dofs, sizeof(int) * so[ne],
                                cudaMemcpyDeviceToHost, s),
                "colouring readback");
    }
    cudaCheck(cudaStreamSynchronize(s), "colouring readback");
    // residual DOF r and state DOF c are one DOF when the tables are shared
    const long long            nres = m->num_res;
    std::vector<unsigned long long> used(static_cast<size_t>(nres + m->num_states), 0ull);
    std::vector<unsigned char>      colour(ne);
    int                             ncol = 0;
    auto key = [&](bool state, int d) -> size_t {
      return static_cast<size_t>(state && !m->same_dofs ? nres + d : d);
    };
    for (int e = 0; e < ne; ++e)
    {
      unsigned long long forbid = 0ull;
      for (int k = ro[e]; k < ro[e + 1]; ++k)
      {
        forbid |= used[key(false, rd[k])];
      }
      for (int k = so[e]; k < so[e + 1]; ++k)
      {
        forbid |= used[key(true, sd[k])];
      }
      require(forbid != ~0ull, "element colouring needs more than 64 colours");
      int c = 0;
      while ((forbid >> c) & 1ull)
      {
        ++c;
      }
      colour[e] = static_cast<unsigned char>(c);
      ncol      = c + 1 > ncol ? c + 1 : ncol;
      for (int k = ro[e]; k < ro[e + 1]; ++k)
      {
        used[key(false, rd[k])] |= 1ull << c;
      }
      for (int k = so[e]; k < so[e + 1]; ++k)
      {
        used[key(true, sd[k])] |= 1ull << c;
      }
    }
    std::vector<int> off(ncol + 1, 0), elems(ne);
    for (int e = 0; e < ne; ++e)
    {
      ++off[colour[e] + 1];
    }
    for (int c = 0; c < ncol; ++c)
    {
      off[c + 1] += off[c];
    }
    std::vector<int> next(off.begin(), off.end() - 1);
    for (int e = 0; e < ne; ++e)
    {
      elems[next[colour[e]]++] = e;
    }
    int* d_off   = deviceAlloc<int>(ncol + 1);
    int* d_elems = nullptr;
    try
    {
      d_elems = deviceAlloc<int>(ne);
      cudaCheck(cudaMemcpyAsync(d_off, off.data(), sizeof(int) * (ncol + 1),
                                cudaMemcpyHostToDevice, s),
                "colouring upload");
      cudaCheck(cudaMemcpyAsync(d_elems, elems.data(), sizeof(int) * ne,
                                cudaMemcpyHostToDevice, s),
                "colouring upload");
      cudaCheck(cudaStreamSynchronize(s), "colouring upload");
    }
    catch (...)
    {
      deviceFree(d_off);
      deviceFree(d_elems);
      throw;
    }
    m->num_colours     = ncol;
    m->colour_off_host = std::move(off);
    m->colour_off      = d_off;
    m->colour_elems    = d_elems;
  });
}

extern "C" int gbfem_assembly_map_num_colours(const gbfem_assembly_map* m)
{
  return m != nullptr ? m->num_colours : 0;
}
