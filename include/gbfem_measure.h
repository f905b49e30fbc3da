/*
 * gbfem_measure.h — measurement support for libgbfem's benchmark. Not part
 * of the femx drop-in surface and without a counterpart in the reference:
 * femx publishes no rooflines. It lets the benchmark measure the FP64 FMA
 * ceiling of the GPU it runs on, the roof for the FP64-bound element kernels.
 */
#ifndef GBFEM_MEASURE_H
#define GBFEM_MEASURE_H

#include "gbfem.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Runs `blocks` x `threads` threads, each doing `iters` x 8 independent FP64
 * FMAs; writes one value per thread to `out` (device, blocks*threads
 * doubles) so the work is not elided. FLOPs = 16 * iters * blocks * threads. */
GBFEM_API int gbfem_probe_fp64_fma(int blocks, int threads, int iters,
                                   double* out, void* stream);

/* Test hook for the integer-pipe conversions the FP32 element paths use:
 * out_f[i] = double->float (round to nearest even) of in[i] and
 * out_d[i] = float->double of out_f[i], computed the way the kernels do.
 * The tests compare them with the hardware conversions. */
GBFEM_API int gbfem_probe_convert(int n, const double* in, float* out_f,
                                  double* out_d, void* stream);

/* Test hook for the branch-free float->double conversion of the FP32
 * Jacobian scatter: out[i] = in[i] widened exactly, except that subnormal
 * floats become zeros of the same sign. */
GBFEM_API int gbfem_probe_convert_ftz(int n, const float* in, double* out, void* stream);

/* Test hook for the FP64 reciprocal and reciprocal square root of the FP64
 * kernels (a float seed refined by two Newton-Raphson steps):
 * out[i] = 1 / in[i] (rsqrt == 0) or 1 / sqrt(in[i]) (rsqrt != 0). */
GBFEM_API int gbfem_probe_rcp(int n, const double* in, double* out, int rsqrt, void* stream);

/* Test hook for the integer-pipe double-float conversions of the tiled
 * FP64-accurate assembly: (hi[i], lo[i]) = split of in[i] (hi + lo within
 * 2^-46 |in[i]|), joined[i] = the double nearest below or above
 * jhi[i] + jlo[i] (a normalised pair with |jhi[i]| >= 2^-74; smaller
 * magnitudes count jlo[i] in part), computed the way the kernels do. */
GBFEM_API int gbfem_probe_dd(int n, const double* in, float* hi, float* lo, const float* jhi,
                             const float* jlo, double* joined, void* stream);

#ifdef __cplusplus
}
#endif

#endif
