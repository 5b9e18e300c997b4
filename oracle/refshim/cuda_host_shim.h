/* Forced include: the CUDA runtime calls and built-in variables calcIR.cu uses, mapped to
 * host memory.  Kernels run as ordinary functions with one "thread" (blockIdx.x = 0,
 * blockDim.x = gridDim.x = 1), so their grid-stride loops visit every index in order.
 * Test infrastructure only. */
#ifndef REFSHIM_CUDA_HOST_H
#define REFSHIM_CUDA_HOST_H
#include <stdlib.h>
#include <string.h>
#include "shim_types.h"

struct refshim_dim3 { unsigned x, y, z; };
static const refshim_dim3 blockIdx = {0, 0, 0}, threadIdx = {0, 0, 0};
static const refshim_dim3 blockDim = {1, 1, 1}, gridDim = {1, 1, 1};

typedef int cudaError_t;
#define cudaSuccess 0
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
struct cudaDeviceProp { char name[256]; size_t totalGlobalMem; };
static inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp *p, int) {
    strcpy(p->name, "host shim (reference kernels run on the CPU)");
    p->totalGlobalMem = 0;
    return 0;
}
template <class T> static inline cudaError_t cudaMalloc(T **p, size_t n) {
    *p = (T *)calloc(n ? n : 1, 1);
    return *p ? 0 : 2;
}
static inline cudaError_t cudaFree(void *p) { free(p); return 0; }
static inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) { memmove(d, s, n); return 0; }
static inline cudaError_t cudaMemGetInfo(size_t *f, size_t *t) { *f = 0; *t = 0; return 0; }
static inline const char *cudaGetErrorString(cudaError_t) { return "host shim error"; }
#endif
