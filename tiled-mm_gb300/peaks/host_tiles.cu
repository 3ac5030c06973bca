// Host-link bandwidth of the tile copies the out-of-core call makes, on one GB300: three
// page-locked host matrices of 32768 x 32768 doubles (cudaHostAlloc, filled by one thread, as
// the bench fills them), and for each 16384 x 16384 tile of the first one a 2D copy (16384
// columns of 128 KiB at a 256 KiB host pitch) and a 1D copy of the same number of bytes from
// the tile's first column on.  Also prints where the pages of each matrix live
// (/proc/self/numa_maps) and the machine's NUMA nodes.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -o host_tiles host_tiles.cu
//   ./host_tiles
#include <cuda_runtime.h>
#include <sched.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>

#define CK(x)                                                                     \
  do {                                                                            \
    cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess) {                                                      \
      printf("{\"error\": \"%s: %s\"}\n", #x, cudaGetErrorString(e_));            \
      return 1;                                                                   \
    }                                                                             \
  } while (0)

static void print_numa_of(const void* p, const char* tag) {
  std::ifstream f("/proc/self/numa_maps");
  std::string line;
  char key[32];
  snprintf(key, sizeof key, "%lx ", (unsigned long)(uintptr_t)p);
  while (std::getline(f, line)) {
    if (line.rfind(key, 0) == 0) {
      printf("{\"matrix\": \"%s\", \"numa_maps\": \"%s\"}\n", tag, line.substr(0, 200).c_str());
      return;
    }
  }
  printf("{\"matrix\": \"%s\", \"numa_maps\": \"mapping not found at %p\"}\n", tag, p);
}

int main() {
  for (int nd = 0; nd < 8; ++nd) {
    char path[96];
    snprintf(path, sizeof path, "/sys/devices/system/node/node%d/cpulist", nd);
    std::ifstream f(path);
    std::string cpus;
    if (!f || !std::getline(f, cpus)) continue;
    printf("{\"node\": %d, \"cpus\": \"%s\"}\n", nd, cpus.c_str());
  }
  printf("{\"this_thread_cpu\": %d}\n", sched_getcpu());
  const size_t n = 32768, t = 16384, bytes = n * n * 8;
  double* h[3];
  for (int i = 0; i < 3; ++i) {
    CK(cudaHostAlloc((void**)&h[i], bytes, cudaHostAllocDefault));
    for (size_t j = 0; j < n * n; ++j) h[i][j] = (double)(j & 1023);
  }
  const char* names[3] = {"A", "B", "C"};
  for (int i = 0; i < 3; ++i) print_numa_of(h[i], names[i]);
  double* d = nullptr;
  CK(cudaMalloc((void**)&d, t * t * 8));
  cudaStream_t s;
  CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  for (int i = 0; i < 3; ++i) {
    for (int ti = 0; ti < 2; ++ti)
      for (int tj = 0; tj < 2; ++tj) {
        const double* src = h[i] + (size_t)tj * t * n + (size_t)ti * t;  // tile (ti, tj), column-major
        float ms2 = 0.f, ms1 = 0.f;
        CK(cudaEventRecord(e0, s));
        CK(cudaMemcpy2DAsync(d, t * 8, src, n * 8, t * 8, t, cudaMemcpyHostToDevice, s));
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        cudaEventElapsedTime(&ms2, e0, e1);
        CK(cudaEventRecord(e0, s));
        CK(cudaMemcpyAsync(d, src, t * t * 8, cudaMemcpyHostToDevice, s));
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        cudaEventElapsedTime(&ms1, e0, e1);
        printf("{\"matrix\": \"%s\", \"tile\": [%d, %d], \"copy2d_gbs\": %.1f, \"copy1d_same_bytes_gbs\": %.1f}\n", names[i],
               ti, tj, t * t * 8 / (ms2 * 1e6), t * t * 8 / (ms1 * 1e6));
      }
  }
  return 0;
}
