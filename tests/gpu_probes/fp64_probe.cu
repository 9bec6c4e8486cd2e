// FP64 facts of the GPU the engine runs on: DADD throughput per SM with 32, 16 or 1
// active lanes, and the dependent-op latency of DADD, log and DDIV in one warp.
// Built and run by tests/test_gpu_fp64_probe.py; the numbers explain why the step
// kernel keeps FP64 work off the common path.
#include <cstdio>
#include <cuda_runtime.h>
__global__ void thr(double *out, int iters, int mode) {
  const int lane = threadIdx.x & 31;
  double a0 = threadIdx.x * 1e-3 + 1.0, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const double b = 1.0000001;
  bool on = mode == 0 ? true : (mode == 1 ? lane == 0 : lane < 16);
  if (on) {
    for (int i = 0; i < iters; i++) {
      a0 = __dadd_rn(a0, b); a1 = __dadd_rn(a1, b); a2 = __dadd_rn(a2, b); a3 = __dadd_rn(a3, b);
      a4 = __dadd_rn(a4, b); a5 = __dadd_rn(a5, b); a6 = __dadd_rn(a6, b); a7 = __dadd_rn(a7, b);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
__global__ void lat(double *out, int iters, int which) {
  double a = 0.5 + threadIdx.x;
  long long t0 = clock64();
  if (which == 0) for (int i = 0; i < iters; i++) a = __dadd_rn(a, 1e-9);
  else if (which == 1) for (int i = 0; i < iters; i++) a = -log(a * 0.999 + 0.5);
  else for (int i = 0; i < iters; i++) a = __ddiv_rn(1.5, a + 1.0);
  long long t1 = clock64();
  out[threadIdx.x] = a;
  if (threadIdx.x == 0) out[32] = (double)(t1 - t0) / iters;
}
int main() {
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  double *out; cudaMalloc(&out, sizeof(double) * blocks * threads);
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  const char *names[3] = {"all 32 lanes", "lane 0 only", "16 lanes"};
  for (int mode = 0; mode < 3; mode++) {
    thr<<<blocks, threads>>>(out, iters, mode);
    cudaEventRecord(e0); thr<<<blocks, threads>>>(out, iters, mode); cudaEventRecord(e1); cudaEventSynchronize(e1);
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    double winst = (double)blocks * threads / 32 * iters * 8;
    printf("DADD throughput %-14s: %.3f ms, %.4g warp-inst/s, %.3f warp-inst/clk/SM (at 2.07 GHz)\n", names[mode], ms, winst / (ms * 1e-3), winst / (ms * 1e-3) / sms / 2.07e9);
  }
  const char *ln[3] = {"DADD", "log", "DDIV"};
  for (int w = 0; w < 3; w++) {
    lat<<<1, 32>>>(out, 1000, w);
    lat<<<1, 32>>>(out, 1000, w);
    double h[33]; cudaMemcpy(h, out, sizeof(h), cudaMemcpyDeviceToHost);
    printf("latency %-5s: %.1f cycles per dependent op (single warp)\n", ln[w], h[32]);
  }
  printf("err=%s\n", cudaGetErrorString(cudaGetLastError()));
  return 0;
}
