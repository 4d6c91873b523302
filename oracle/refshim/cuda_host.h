// Host stand-ins for the few CUDA runtime names that the VEDAS reference
// sources use outside Thrust, so that they compile with g++ against Thrust's
// OpenMP backend.  Test infrastructure only (the reference-as-oracle build);
// "device" memory is host memory under that backend, so copies are memcpy.
#ifndef VEDAS_ORACLE_CUDA_HOST_H
#define VEDAS_ORACLE_CUDA_HOST_H

#include <cstddef>
#include <cstring>

#ifndef VEDAS_ORACLE_HAVE_INT2
#define VEDAS_ORACLE_HAVE_INT2
struct int2 {
  int x, y;
};
static inline int2 make_int2(int x, int y) {
  int2 r;
  r.x = x;
  r.y = y;
  return r;
}
#endif

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
  cudaMemcpyDefault = 4
};

static inline cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
  if (n) std::memmove(dst, src, n);
  return cudaSuccess;
}
static inline cudaError_t cudaMemcpyPeer(void* dst, int, const void* src, int, size_t n) {
  if (n) std::memmove(dst, src, n);
  return cudaSuccess;
}
static inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
static inline cudaError_t cudaGetDevice(int* d) {
  *d = 0;
  return cudaSuccess;
}
static inline cudaError_t cudaDeviceCanAccessPeer(int* can, int, int) {
  *can = 0;
  return cudaSuccess;
}
static inline cudaError_t cudaDeviceEnablePeerAccess(int, unsigned) { return cudaSuccess; }
static inline const char* cudaGetErrorString(cudaError_t) { return "no error"; }

#endif
