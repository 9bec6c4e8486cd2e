// Memory latencies of the GPU the engine runs on, from one warp's dependent loads:
// shared memory, L1-resident, L2-resident and HBM-resident pointer chases, and a global
// store followed by a load of the same word (the pattern of a step that re-reads what
// the previous step wrote).  Built and run by tests/test_gpu_fp64_probe.py.
#include <cstdio>
#include <cuda_runtime.h>

__global__ void chase(const unsigned *next, unsigned start, int iters, unsigned *out, long long *cyc) {
  unsigned p = start;
  long long t0 = clock64();
  for (int i = 0; i < iters; i++) p = next[p];
  long long t1 = clock64();
  if (threadIdx.x == 0) { out[0] = p; cyc[0] = (t1 - t0) / iters; }
}

__global__ void chase_smem(int iters, unsigned *out, long long *cyc) {
  __shared__ unsigned nx[1024];
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) nx[i] = (i * 97 + 13) & 1023;
  __syncthreads();
  unsigned p = threadIdx.x;
  long long t0 = clock64();
  for (int i = 0; i < iters; i++) p = nx[p];
  long long t1 = clock64();
  if (threadIdx.x == 0) { out[0] = p; cyc[0] = (t1 - t0) / iters; }
}

// The same chase through a generic pointer to the shared array (the address space is
// hidden from the compiler by selecting it at run time), as the engine reads a model's
// hot section that may sit in shared or global memory.
__global__ void chase_smem_generic(const unsigned *gbuf, int use_global, int iters, unsigned *out, long long *cyc) {
  __shared__ unsigned nx[1024];
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) nx[i] = (i * 97 + 13) & 1023;
  __syncthreads();
  const unsigned *src = use_global ? gbuf : nx;
  unsigned p = threadIdx.x;
  long long t0 = clock64();
  for (int i = 0; i < iters; i++) p = src[p];
  long long t1 = clock64();
  if (threadIdx.x == 0) { out[0] = p; cyc[0] = (t1 - t0) / iters; }
}

__global__ void store_load(unsigned *buf, int iters, unsigned *out, long long *cyc) {
  unsigned v = threadIdx.x;
  long long t0 = clock64();
  for (int i = 0; i < iters; i++) {
    buf[(v & 255) * 32] = v + 1;       // store, then load the same word
    v = buf[(v & 255) * 32] * 3u + 1u;
  }
  long long t1 = clock64();
  if (threadIdx.x == 0) { out[0] = v; cyc[0] = (t1 - t0) / iters; }
}

// Does a warp barrier wait for global loads still in flight?  Each iteration issues one
// load per lane (independent addresses in a 2 GB buffer, so it misses in L2), then a
// chain of 32 dependent integer ops that does not use it, then uses it.  mode 0: nothing between the
// load and the work; 1: __syncwarp(); 2: __ballot_sync; 3: a shared-memory store and
// __syncwarp (the pattern of the engine's edit rounds).  If a barrier waits for the
// load, its iterations cost the load latency plus the work instead of the larger of the
// two.
__global__ void load_then_sync(const unsigned *buf, size_t n, int iters, int mode, unsigned *out,
                               long long *cyc) {
  __shared__ unsigned sh[32];
  const int lane = threadIdx.x & 31;
  unsigned acc = 0, x = lane;
  size_t idx = (size_t)lane * 4099u;  // < n
  long long t0 = clock64();
  for (int i = 0; i < iters; i++) {
    idx += 1048583u;
    if (idx >= n) idx -= n;  // stays in [0, n): the step is below n
    const unsigned v = buf[idx];
    if (mode == 1) __syncwarp();
    if (mode == 2) x += __ballot_sync(0xffffffffu, x & 1) & 1u;
    if (mode == 3) { sh[lane] = x; __syncwarp(); x += sh[(lane + 1) & 31]; }
#pragma unroll 1
    for (int k = 0; k < 32; k++) x = x * 3u + 1u;
    acc += v;
  }
  long long t1 = clock64();
  const unsigned sum = __reduce_add_sync(0xffffffffu, acc + x);
  if (lane == 0) { out[0] = sum; cyc[0] = (t1 - t0) / iters; }
}

int main() {
  const size_t sizes[3] = {16 << 10, 32 << 20, (size_t)2 << 30};
  const char *names[3] = {"L1-resident (16 KB)", "L2-resident (32 MB)", "HBM (2 GB)"};
  unsigned *out; long long *cyc;
  cudaMalloc(&out, 64); cudaMalloc(&cyc, 64);
  for (int s = 0; s < 3; s++) {
    const size_t n = sizes[s] / 4;
    unsigned *next, *h = new unsigned[n];
    // a random cycle with a 4 KB stride so every step touches another line / page
    const size_t stride = 1031;
    for (size_t i = 0; i < n; i++) h[i] = (unsigned)((i + stride * 16 + 7) % n);
    cudaMalloc(&next, n * 4);
    cudaMemcpy(next, h, n * 4, cudaMemcpyHostToDevice);
    delete[] h;
    chase<<<1, 1>>>(next, 0, 1000, out, cyc);
    chase<<<1, 1>>>(next, 0, 4000, out, cyc);
    long long c; cudaMemcpy(&c, cyc, 8, cudaMemcpyDeviceToHost);
    printf("dependent global load, %-22s: %lld cycles\n", names[s], c);
    cudaFree(next);
  }
  chase_smem<<<1, 32>>>(4000, out, cyc);
  long long c; cudaMemcpy(&c, cyc, 8, cudaMemcpyDeviceToHost);
  printf("dependent shared-memory load           : %lld cycles\n", c);
  chase_smem_generic<<<1, 32>>>(out, 0, 4000, out, cyc);
  cudaMemcpy(&c, cyc, 8, cudaMemcpyDeviceToHost);
  printf("dependent shared-memory load, generic  : %lld cycles\n", c);
  unsigned *buf; cudaMalloc(&buf, 1 << 20);
  store_load<<<1, 32>>>(buf, 100, out, cyc);
  store_load<<<1, 32>>>(buf, 4000, out, cyc);
  cudaMemcpy(&c, cyc, 8, cudaMemcpyDeviceToHost);
  printf("global store then dependent load       : %lld cycles\n", c);
  {
    const size_t n = ((size_t)2 << 30) / 4;
    unsigned *big;
    cudaMalloc(&big, n * 4);
    cudaMemset(big, 1, n * 4);
    const char *modes[4] = {"no barrier", "__syncwarp", "__ballot_sync", "smem store + __syncwarp"};
    for (int m = 0; m < 4; m++) {
      load_then_sync<<<1, 32>>>(big, n, 50, m, out, cyc);
      load_then_sync<<<1, 32>>>(big, n, 2000, m, out, cyc);
      cudaMemcpy(&c, cyc, 8, cudaMemcpyDeviceToHost);
      printf("HBM load, %-24s then 32 int ops, then use: %lld cycles per iteration\n", modes[m], c);
    }
    cudaFree(big);
  }
  printf("err=%s\n", cudaGetErrorString(cudaDeviceSynchronize()));
  return 0;
}
