// gpu_bar_launch.cpp — launches the reference's own CUDA assembly kernel
// (femx's assembleKernel, compiled from femx's sources into
// oracle/_ref/gpu_bar.cubin by oracle/ref/Makefile) so that the benchmark can
// time it on the same GPU as the product kernels.
//
// Test and measurement infrastructure, not product code: only bench.py's
// reference legs load it. Built on the GPU machine (g++ against the CUDA driver
// API; no femx source is needed there). The kernel arguments are filled by
// the caller from oracle/_ref/gpu_bar_layout.json (byte offsets of femx's
// argument structs, found by the compiler); this file only loads the module,
// finds the kernel by name and launches it on the caller's stream.
#include <cuda.h>

#include <cstring>
#include <string>

namespace
{
CUmodule    g_mod = nullptr;
std::string g_err;

int fail(const char* what, CUresult r)
{
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  g_err = std::string(what) + ": " + (s ? s : "unknown CUDA driver error");
  return 1;
}
} // namespace

extern "C" const char* refbar_last_error()
{
  return g_err.c_str();
}

// Loads `cubin` into the current context (the runtime's primary context)
// once and returns in *func the first kernel whose name contains
// `name_part`; its name is copied to `name_out` (capacity `cap`). 0 on
// success.
extern "C" int refbar_load(const char* cubin, const char* name_part, char* name_out, int cap,
                           void** func)
{
  CUresult r = cuInit(0);
  if (r != CUDA_SUCCESS)
  {
    return fail("cuInit", r);
  }
  if (g_mod == nullptr)
  {
    r = cuModuleLoad(&g_mod, cubin);
    if (r != CUDA_SUCCESS)
    {
      g_mod = nullptr;
      return fail("cuModuleLoad", r);
    }
  }
  unsigned n = 0;
  r          = cuModuleGetFunctionCount(&n, g_mod);
  if (r != CUDA_SUCCESS)
  {
    return fail("cuModuleGetFunctionCount", r);
  }
  CUfunction fs[64];
  if (n > 64)
  {
    n = 64;
  }
  r = cuModuleEnumerateFunctions(fs, n, g_mod);
  if (r != CUDA_SUCCESS)
  {
    return fail("cuModuleEnumerateFunctions", r);
  }
  for (unsigned i = 0; i < n; ++i)
  {
    const char* name = nullptr;
    if (cuFuncGetName(&name, fs[i]) == CUDA_SUCCESS && name != nullptr
        && std::strstr(name, name_part) != nullptr)
    {
      *func = fs[i];
      if (name_out != nullptr && cap > 0)
      {
        std::strncpy(name_out, name, static_cast<size_t>(cap) - 1);
        name_out[cap - 1] = '\0';
      }
      return 0;
    }
  }
  g_err = "no kernel named like the request in the module";
  return 1;
}

// Offset and size of kernel parameter `index` (from the module's own
// parameter table), to cross-check the layout file.
extern "C" int refbar_param(void* func, int index, long long* offset, long long* size)
{
  size_t   o = 0, s = 0;
  CUresult r = cuFuncGetParamInfo(static_cast<CUfunction>(func), static_cast<size_t>(index), &o,
                                  &s);
  if (r != CUDA_SUCCESS)
  {
    return fail("cuFuncGetParamInfo", r);
  }
  *offset = static_cast<long long>(o);
  *size   = static_cast<long long>(s);
  return 0;
}

// Launches `func`: `args[i]` points at the bytes of parameter i.
extern "C" int refbar_launch(void* func, void** args, unsigned grid, unsigned block,
                             unsigned smem, void* stream)
{
  if (func == nullptr)
  {
    g_err = "no kernel loaded";
    return 1;
  }
  const CUresult r = cuLaunchKernel(static_cast<CUfunction>(func), grid, 1, 1, block, 1, 1, smem,
                                    static_cast<CUstream>(stream), args, nullptr);
  return r == CUDA_SUCCESS ? 0 : fail("cuLaunchKernel", r);
}
