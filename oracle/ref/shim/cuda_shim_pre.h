/* ORACLE (test infrastructure): host stand-ins for the CUDA runtime names the
 * reference's solver sources use, so those sources compile with g++ for the
 * CPU.  Device qualifiers vanish, device memory is host memory, atomics are
 * plain (one thread), launch geometry is all zeros.  Included first into
 * every reference translation unit by oracle/ref/build_ref.py. */
#pragma once
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>

#define __host__
#define __device__
#define __global__
#define __forceinline__ inline

struct gpsat_shim_dim3 { unsigned x = 0, y = 0, z = 0; };
static gpsat_shim_dim3 threadIdx, blockIdx, blockDim, gridDim;

typedef int cudaError;
typedef int cudaError_t;
enum { cudaSuccess = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3,
       cudaMemcpyHostToHost = 4 };

inline cudaError cudaMalloc(void *p, size_t n) { *(void **)p = std::malloc(n ? n : 1); return 0; }
inline cudaError cudaMallocManaged(void *p, size_t n) { return cudaMalloc(p, n); }
inline cudaError cudaMallocPitch(void **p, size_t *pitch, size_t w, size_t h)
{ *p = std::malloc(w * h ? w * h : 1); *pitch = w; return 0; }
inline cudaError cudaMemcpy(void *d, const void *s, size_t n, int) { std::memcpy(d, s, n); return 0; }
inline cudaError cudaMemset(void *d, int v, size_t n) { std::memset(d, v, n); return 0; }
inline cudaError cudaFree(void *p) { std::free(p); return 0; }
inline const char *cudaGetErrorString(int) { return "host shim"; }
inline cudaError cudaDeviceReset() { return 0; }
inline cudaError cudaDeviceSynchronize() { return 0; }
inline cudaError cudaThreadSynchronize() { return 0; }
#define cudaMemcpyToSymbol(...) 0

inline unsigned atomicInc(unsigned *a, unsigned m) { unsigned o = *a; *a = (o >= m) ? 0 : o + 1; return o; }
inline int atomicExch(int *a, int v) { int o = *a; *a = v; return o; }
template <class T, class U> inline T atomicAdd(T *a, U v) { T o = *a; *a += (T)v; return o; }
inline long long clock64() { return 0; }

/* curand is only reached with the reference's optional VSIDS; a small LCG */
struct curandState { unsigned s; };
inline void curand_init(unsigned long long seed, unsigned long long, unsigned long long, curandState *st)
{ st->s = (unsigned)seed; }
inline unsigned curand(curandState *st) { st->s = st->s * 1664525u + 1013904223u; return st->s; }
inline float curand_uniform(curandState *st) { return (curand(st) >> 8) * (1.0f / 16777216.0f); }

namespace thrust {
template <class T> struct device_ptr { T *p; T *get() const { return p; } };
template <class T> device_ptr<T> device_malloc(size_t n) { return device_ptr<T>{(T *)std::malloc(sizeof(T) * (n ? n : 1))}; }
template <class T> T *raw_pointer_cast(device_ptr<T> d) { return d.p; }
}
