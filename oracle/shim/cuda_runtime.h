// Host-only stand-in for the CUDA runtime header, used ONLY to compile the
// reference's VX3 physics sources as plain C++ for the oracle build under
// oracle/_ref/.  "Device" memory is host memory; atomics are plain
// read-modify-write (the oracle runs single-threaded).
#pragma once
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
enum cudaLimit { cudaLimitMallocHeapSize, cudaLimitPrintfFifoSize, cudaLimitStackSize };

inline const char *cudaGetErrorString(int) { return "shim"; }
inline int cudaMalloc(void **p, size_t n) { *p = calloc(1, n ? n : 1); return 0; }
template <class T> inline int cudaMalloc(T **p, size_t n) { *p = (T *)calloc(1, n ? n : 1); return 0; }
inline int cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memcpy(d, s, n); return 0; }
inline int cudaFree(void *p) { free(p); return 0; }
inline int cudaGetLastError() { return 0; }
inline int cudaDeviceSynchronize() { return 0; }

inline int atomicCAS(int *a, int c, int v) { int o = *a; if (o == c) *a = v; return o; }
inline int atomicExch(int *a, int v) { int o = *a; *a = v; return o; }
inline int atomicAdd(int *a, int v) { int o = *a; *a += v; return o; }
inline double normcdf(double x) { return 0.5 * erfc(-x / sqrt(2.0)); }
inline int __isnand(double x) { return std::isnan(x); }
