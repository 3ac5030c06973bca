/*
 * ORACLE test infrastructure: a host-only stand-in for the handful of CUDA
 * runtime names that the reference's src/Tiled-MM/gpu_runtime_api.hpp
 * forwards to.  It lets the reference's own host code (tile policy, tile
 * geometry, the round-robin schedule in tiled_mm.cpp) be compiled with g++
 * and executed on the CPU, with "device memory" in host RAM and every
 * asynchronous operation executed immediately, in issue order (a valid
 * serialisation of the reference's stream/event program).
 *
 * Only declarations needed by that header are provided; the definitions are
 * in fake_cuda.cpp.  This is not a CUDA implementation and is never linked
 * into the product.
 */
#pragma once
#include <stddef.h>

#define CUDART_VERSION 13000

typedef enum cudaError {
  cudaSuccess = 0,
  cudaErrorInvalidValue = 1,
  cudaErrorMemoryAllocation = 2,
  cudaErrorInitializationError = 3,
  cudaErrorLaunchOutOfResources = 7,
  cudaErrorInvalidDevice = 101,
  cudaErrorInvalidMemcpyDirection = 21,
  cudaErrorInvalidDevicePointer = 17,
  cudaErrorNoDevice = 100,
  cudaErrorNotReady = 600,
  cudaErrorUnknown = 999,
  cudaErrorPeerAccessNotEnabled = 705,
  cudaErrorPeerAccessAlreadyEnabled = 704,
  cudaErrorHostMemoryAlreadyRegistered = 712,
  cudaErrorHostMemoryNotRegistered = 713,
  cudaErrorUnsupportedLimit = 215,
  cudaErrorInvalidResourceHandle = 400
} cudaError_t;

typedef struct fake_stream* cudaStream_t;
typedef struct fake_event* cudaEvent_t;

enum cudaMemoryType {
  cudaMemoryTypeUnregistered = 0,
  cudaMemoryTypeHost = 1,
  cudaMemoryTypeDevice = 2,
  cudaMemoryTypeManaged = 3
};

struct cudaPointerAttributes {
  enum cudaMemoryType type;
  int device;
  void* devicePointer;
  void* hostPointer;
};

enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
  cudaMemcpyDefault = 4
};

#define cudaHostRegisterDefault 0x00
#define cudaHostRegisterPortable 0x01
#define cudaHostRegisterMapped 0x02
#define cudaHostRegisterIoMemory 0x04
#define cudaStreamDefault 0x00
#define cudaStreamNonBlocking 0x01
#define cudaEventDefault 0x00
#define cudaEventBlockingSync 0x01
#define cudaEventDisableTiming 0x02
#define cudaEventInterprocess 0x04

cudaError_t cudaHostRegister(void* ptr, size_t size, unsigned int flags);
cudaError_t cudaHostUnregister(void* ptr);
cudaError_t cudaStreamCreateWithFlags(cudaStream_t* s, unsigned int flags);
cudaError_t cudaStreamDestroy(cudaStream_t s);
cudaError_t cudaStreamWaitEvent(cudaStream_t s, cudaEvent_t e, unsigned int flags);
cudaError_t cudaStreamSynchronize(cudaStream_t s);
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned int flags);
cudaError_t cudaEventDestroy(cudaEvent_t e);
cudaError_t cudaEventRecord(cudaEvent_t e, cudaStream_t s);
cudaError_t cudaEventSynchronize(cudaEvent_t e);
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b);
cudaError_t cudaMalloc(void** p, size_t size);
cudaError_t cudaHostAlloc(void** p, size_t size, unsigned int flags);
cudaError_t cudaFree(void* p);
cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, enum cudaMemcpyKind kind);
cudaError_t cudaMemcpyAsync(void* dst, const void* src, size_t n, enum cudaMemcpyKind kind, cudaStream_t s);
cudaError_t cudaMemcpy2D(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                         size_t height, enum cudaMemcpyKind kind);
cudaError_t cudaMemcpy2DAsync(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                              size_t height, enum cudaMemcpyKind kind, cudaStream_t s);
cudaError_t cudaGetDevice(int* d);
cudaError_t cudaSetDevice(int d);
cudaError_t cudaGetDeviceCount(int* n);
cudaError_t cudaMemsetAsync(void* p, int v, size_t n, cudaStream_t s);
cudaError_t cudaPointerGetAttributes(struct cudaPointerAttributes* a, const void* p);
cudaError_t cudaMemGetInfo(size_t* free_b, size_t* total_b);
const char* cudaGetErrorString(cudaError_t e);
cudaError_t cudaGetLastError(void);
cudaError_t cudaDeviceSynchronize(void);
