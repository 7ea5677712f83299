/*
 * TEST INFRASTRUCTURE ONLY.  Host shim that lets the reference's own CUDA
 * sources (src/*.h, src/*.cu) compile with g++ and execute on the CPU.
 *
 *  - __global__/__device__/__host__ become plain functions; __shared__
 *    arrays become function statics (one block runs at a time);
 *  - a kernel launch runs the body once per (block, thread) of the launch
 *    grid; kernels that call __syncthreads run each block's threads as
 *    cooperative fibers that switch at every barrier;
 *  - cudaMalloc/cudaMemcpy/cudaFree become calloc/memcpy/free;
 *  - device printf goes through sevc_ref_printf (silenced unless
 *    SEVC_REF_VERBOSE is set; the two calls at src/topological.h:598,601
 *    that pass ints for "%s" are printed safely);
 *  - the min_grains constant of src/main.cu:49 is read from
 *    SEVC_REF_MIN_GRAINS (default 5000, the reference's value).
 */
#ifndef SEVC_REF_SHIM_H
#define SEVC_REF_SHIM_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdarg>
#include <type_traits>

using std::abs;

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static

struct sevc_dim3 { unsigned int x, y, z; };
extern sevc_dim3 blockIdx, threadIdx, blockDim, gridDim;

static inline double max(double a, double b) { return std::fmax(a, b); }
static inline double min(double a, double b) { return std::fmin(a, b); }
static_assert(std::is_same<decltype(abs(1.0)), double>::value, "abs(double) must be the double overload");

void sevc_syncthreads();
#define __syncthreads() sevc_syncthreads()

typedef int cudaError_t;
#define cudaSuccess 0
enum { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 };
static inline const char *cudaGetErrorString(cudaError_t) { return "no error"; }
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
static inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
static inline cudaError_t cudaMalloc(void **p, size_t n) { *p = calloc(n ? n : 1, 1); return *p ? 0 : 2; }
template <class T> static inline cudaError_t cudaMalloc(T **p, size_t n) { return cudaMalloc((void **)p, n); }
static inline cudaError_t cudaFree(void *p) { free(p); return cudaSuccess; }
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, int) { memmove(d, s, n); return cudaSuccess; }

int sevc_ref_printf(const char *fmt, ...);
#define printf sevc_ref_printf
int sevc_ref_min_grains();

#include <functional>
void sevc_launch(const char *name, unsigned int grid, unsigned int block, const std::function<void()> &body);
#define SEVC_LAUNCH(f, g, b, ...) sevc_launch(#f, (g), (b), [&]() { f(__VA_ARGS__); })

#endif
