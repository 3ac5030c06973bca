// Host-link probes on one GB300: copy-engine copies against kernel loads and stores of host
// memory over the C2C link, page-locked and (when the device reports pageable memory
// access through the host page tables) ordinary pageable memory, and the cost of
// page-locking a buffer.  4 GiB per transfer, three transfers per figure.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -o host_link host_link.cu
//   ./host_link        # one JSON line
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>

__global__ void copy_kernel(const double2* __restrict__ x, double2* __restrict__ y, size_t n2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x) y[i] = x[i];
}

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { printf("ERR %s at %d: %s\n", #x, __LINE__, cudaGetErrorString(e_)); return 1; } } while (0)

int main() {
  int dev = 0, pma = 0, pmaHPT = 0, cma = 0, sms = 0;
  CK(cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev));
  CK(cudaDeviceGetAttribute(&pmaHPT, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
  CK(cudaDeviceGetAttribute(&cma, cudaDevAttrConcurrentManagedAccess, dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  printf("{\"pageable_memory_access\": %d, \"uses_host_page_tables\": %d, \"concurrent_managed\": %d", pma, pmaHPT, cma);
  const size_t bytes = (size_t)4 << 30, n2 = bytes / 16;
  double *hp = nullptr, *d = nullptr;
  CK(cudaHostAlloc((void**)&hp, bytes, cudaHostAllocDefault));
  for (size_t i = 0; i < bytes / 8; ++i) hp[i] = 1.0;
  CK(cudaMalloc((void**)&d, bytes));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms = 0.f;
  // copy engine, pinned
  CK(cudaMemcpy(d, hp, bytes, cudaMemcpyHostToDevice));
  cudaEventRecord(e0);
  for (int r = 0; r < 3; ++r) CK(cudaMemcpyAsync(d, hp, bytes, cudaMemcpyHostToDevice));
  cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
  printf(", \"memcpy_h2d_pinned_gbs\": %.1f", 3.0 * bytes / (ms * 1e6));
  cudaEventRecord(e0);
  for (int r = 0; r < 3; ++r) CK(cudaMemcpyAsync(hp, d, bytes, cudaMemcpyDeviceToHost));
  cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
  printf(", \"memcpy_d2h_pinned_gbs\": %.1f", 3.0 * bytes / (ms * 1e6));
  // kernel loads of pinned host memory (mapped through unified addressing)
  for (int blocks_per_sm : {4, 8, 16}) {
    cudaEventRecord(e0);
    for (int r = 0; r < 3; ++r) copy_kernel<<<sms * blocks_per_sm, 256>>>((const double2*)hp, (double2*)d, n2);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); cudaEventElapsedTime(&ms, e0, e1);
    printf(", \"kernel_read_pinned_gbs_%d\": %.1f", blocks_per_sm, 3.0 * bytes / (ms * 1e6));
  }
  // kernel stores into pinned host memory
  cudaEventRecord(e0);
  for (int r = 0; r < 3; ++r) copy_kernel<<<sms * 8, 256>>>((const double2*)d, (double2*)hp, n2);
  cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); cudaEventElapsedTime(&ms, e0, e1);
  printf(", \"kernel_write_pinned_gbs\": %.1f", 3.0 * bytes / (ms * 1e6));
  if (pma) {
    double* pg = (double*)malloc(bytes);
    for (size_t i = 0; i < bytes / 8; ++i) pg[i] = 1.0;
    copy_kernel<<<sms * 8, 256>>>((const double2*)pg, (double2*)d, n2);
    CK(cudaDeviceSynchronize());
    cudaEventRecord(e0);
    for (int r = 0; r < 3; ++r) copy_kernel<<<sms * 8, 256>>>((const double2*)pg, (double2*)d, n2);
    cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); cudaEventElapsedTime(&ms, e0, e1);
    printf(", \"kernel_read_pageable_gbs\": %.1f", 3.0 * bytes / (ms * 1e6));
    cudaEventRecord(e0);
    for (int r = 0; r < 3; ++r) CK(cudaMemcpyAsync(d, pg, bytes, cudaMemcpyHostToDevice));
    cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1);
    printf(", \"memcpy_h2d_pageable_gbs\": %.1f", 3.0 * bytes / (ms * 1e6));
    auto t0 = std::chrono::steady_clock::now();
    CK(cudaHostRegister(pg, bytes, cudaHostRegisterDefault));
    auto t1 = std::chrono::steady_clock::now();
    CK(cudaHostUnregister(pg));
    printf(", \"host_register_4gb_ms\": %.1f", std::chrono::duration<double, std::milli>(t1 - t0).count());
    free(pg);
  }
  printf("}\n");
  return 0;
}
