// Host-link bandwidth on one GB300 while a kernel keeps the GPU busy: page-locked 4 GiB
// cudaMemcpyAsync copies (host to device, then device to host) on one stream while another
// stream runs, for longer than the copies take, one of
//   none     nothing
//   hbm      a device-to-device copy kernel streaming 8 GiB buffers (HBM read + write bound)
//   l2       the same kernel over 32 MiB buffers (L2 resident)
//   fma      a register-only FMA loop (SMs busy, no memory traffic)
// Every kernel runs a fixed amount of work (no waits).  Prints one JSON line per case.
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -o link_under_load link_under_load.cu
//   ./link_under_load
#include <cuda_runtime.h>

#include <cstdio>

#define CK(x)                                                                     \
  do {                                                                            \
    cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess) {                                                      \
      printf("{\"error\": \"%s: %s\"}\n", #x, cudaGetErrorString(e_));            \
      return 1;                                                                   \
    }                                                                             \
  } while (0)

__global__ void stream_copy(const double2* __restrict__ x, double2* __restrict__ y, size_t n2, int reps) {
  for (int r = 0; r < reps; ++r)
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x)
      y[i] = x[i];
}

__global__ void fma_spin(float* out, int iters) {
  float a = threadIdx.x * 1e-3f, b = 1.0001f, c = 0.9999f, d = blockIdx.x * 1e-3f;
  for (int i = 0; i < iters; ++i) {
    a = fmaf(a, b, c);
    d = fmaf(d, c, b);
  }
  if (a + d == 12345.0f) out[0] = a + d;  // keeps the loop
}

static float ms_between(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

int main() {
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
  const size_t link_bytes = (size_t)4 << 30;
  const size_t hbm_bytes = (size_t)8 << 30, l2_bytes = (size_t)32 << 20;
  void *hp = nullptr, *dl = nullptr, *x = nullptr, *y = nullptr;
  float* out = nullptr;
  CK(cudaHostAlloc(&hp, link_bytes, cudaHostAllocDefault));
  for (size_t i = 0; i < link_bytes / 8; ++i) ((double*)hp)[i] = 1.0;
  CK(cudaMalloc(&dl, link_bytes));
  CK(cudaMalloc(&x, hbm_bytes));
  CK(cudaMalloc(&y, hbm_bytes));
  CK(cudaMalloc(&out, 4));
  CK(cudaMemset(x, 0, hbm_bytes));
  cudaStream_t sc, sk;
  CK(cudaStreamCreateWithFlags(&sc, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&sk, cudaStreamNonBlocking));
  cudaEvent_t c0, c1, c2, k0, k1;
  for (cudaEvent_t* e : {&c0, &c1, &c2, &k0, &k1}) CK(cudaEventCreate(e));
  CK(cudaMemcpy(dl, hp, link_bytes, cudaMemcpyHostToDevice));  // warm
  const char* names[4] = {"none", "hbm", "l2", "fma"};
  for (int bg = 0; bg < 4; ++bg) {
    for (int rep = 0; rep < 2; ++rep) {
      CK(cudaDeviceSynchronize());
      CK(cudaEventRecord(k0, sk));
      if (bg == 1) stream_copy<<<sms * 4, 256, 0, sk>>>((const double2*)x, (double2*)y, hbm_bytes / 16, 300);
      if (bg == 2) stream_copy<<<sms * 4, 256, 0, sk>>>((const double2*)x, (double2*)y, l2_bytes / 16, 150000);
      if (bg == 3) fma_spin<<<sms * 4, 256, 0, sk>>>(out, 1 << 25);
      CK(cudaGetLastError());
      CK(cudaEventRecord(k1, sk));
      CK(cudaEventRecord(c0, sc));
      CK(cudaMemcpyAsync(dl, hp, link_bytes, cudaMemcpyHostToDevice, sc));
      CK(cudaEventRecord(c1, sc));
      CK(cudaMemcpyAsync(hp, dl, link_bytes, cudaMemcpyDeviceToHost, sc));
      CK(cudaEventRecord(c2, sc));
      CK(cudaDeviceSynchronize());
      if (!rep) continue;
      const float h2d = ms_between(c0, c1), d2h = ms_between(c1, c2), kern = ms_between(k0, k1);
      // the copies count as "under load" only if the kernel ran from before the first copy
      // to after the last
      const float lead = ms_between(k0, c0), tail = ms_between(c2, k1);
      printf("{\"background\": \"%s\", \"h2d_gbs\": %.1f, \"d2h_gbs\": %.1f, \"kernel_ms\": %.1f, "
             "\"copies_ms\": %.1f, \"kernel_started_ms_before\": %.1f, \"kernel_ended_ms_after\": %.1f}\n",
             names[bg], link_bytes / (h2d * 1e6), link_bytes / (d2h * 1e6), kern, h2d + d2h, lead, tail);
    }
  }
  return 0;
}
