// hostio.cu — one Newton system per call for a host-resident state: the
// Taylor-Hood residual and Jacobian with Dirichlet rows, from a state in
// host memory to a residual in host memory (femx's Newton iteration,
// femx/solver/Newton.hpp, with the CPU-side vectors of its examples).
//
// The transfers overlap the device work on a side stream:
//   user stream : H2D state ──────────┐ assemble, replaceRes ─┬─ replaceRows ─┐ join
//   side stream : zero fill of res/J ─┘                       └─ D2H residual ┘
// so the call costs max(H2D, zero fill) + assembly + replaceRes +
// max(D2H, replaceRows) instead of their sum. The side stream and its
// events belong to the calling host thread (gbfem::sideStream).
#include <string>

#include "common.cuh"
#include "maps.cuh"

namespace gbfem
{
void assembleTaylorHood(const gbfem_assembly_map* map, int num_p2_nodes, const double* coords,
                        const int* conn6, double nu, const double* state, double* res,
                        double* vals, int precision, cudaStream_t s, bool zero);
}

namespace
{

void checkCode(int code)
{
  if (code != GBFEM_OK)
  {
    throw gbfem::Error(code, gbfem_last_error());
  }
}

} // namespace

extern "C" int gbfem_newton_system_th_ns_host(
    const gbfem_assembly_map* map, const gbfem_boundary_map* bc, int num_p2_nodes,
    const double* coords, const int* conn6, double nu, const double* state_host, double* state,
    const double* bc_vals, double* res, double* vals, double diag, double* res_host,
    int precision, void* stream)
{
  using namespace gbfem;
  return guarded([&] {
    require(map != nullptr && bc != nullptr, "AssemblyMap or BoundaryMap handle is null");
    require(state_host != nullptr && state != nullptr && res != nullptr && res_host != nullptr,
            "Newton system buffers must not be null");
    require(bc->num_rows == map->num_res && bc->num_cols == map->num_states,
            "BoundaryMap does not match the AssemblyMap");
    require(bc->num_bcs == 0 || bc_vals != nullptr, "Dirichlet values are null");
    require(vals == nullptr || bc->layout_id == map->layout_id,
            "BoundaryMap was built for another CSR pattern");
    cudaStream_t s = asStream(stream);
    SideStream&  g_side = sideStream();
    cudaStream_t s2     = g_side.s;
    // fork after the work already queued on the user stream
    cudaCheck(cudaEventRecord(g_side.ev[0], s), "fork");
    cudaCheck(cudaStreamWaitEvent(s2, g_side.ev[0], 0), "fork");
    zeroForNext(vals, vals != nullptr ? map->nnz : 0, res, map->num_res, s2);
    cudaCheck(cudaEventRecord(g_side.ev[1], s2), "zero fill event");
    cudaCheck(cudaMemcpyAsync(state, state_host, sizeof(double) * map->num_states,
                              cudaMemcpyHostToDevice, s),
              "state upload");
    cudaCheck(cudaStreamWaitEvent(s, g_side.ev[1], 0), "join zero fill");
    assembleTaylorHood(map, num_p2_nodes, coords, conn6, nu, state, res, vals, precision, s,
                       false);
    checkCode(gbfem_replace_res(bc, state, bc_vals, res, s));
    // the residual is final: download it while the matrix rows are replaced
    cudaCheck(cudaEventRecord(g_side.ev[2], s), "residual event");
    cudaCheck(cudaStreamWaitEvent(s2, g_side.ev[2], 0), "residual event");
    cudaCheck(cudaMemcpyAsync(res_host, res, sizeof(double) * map->num_res,
                              cudaMemcpyDeviceToHost, s2),
              "residual download");
    cudaCheck(cudaEventRecord(g_side.ev[3], s2), "download event");
    if (vals != nullptr)
    {
      checkCode(gbfem_replace_rows(bc, vals, diag, s));
    }
    cudaCheck(cudaStreamWaitEvent(s, g_side.ev[3], 0), "join download");
  });
}
