// philox_curand.cu -- draws blocks of cuRAND's Philox4x32-10 generator (the device
// API of the CUDA toolkit) for a seeded list of (seed, subsequence, offset) and
// prints them, so that tests/test_gpu_philox.py can check the Philox4x32-10
// restatement of the oracle (and the device noise, which the parity tests tie to
// the oracle) against NVIDIA's implementation.
//
// Output, one line per case: seed subsequence offset r0 r1 r2 r3 (hex).
#include <cstdint>
#include <cstdio>
#include <vector>

#include <curand_kernel.h>

__global__ void k_draw(const unsigned long long *seed, const unsigned long long *sub, const unsigned long long *off,
                       uint4 *out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  curandStatePhilox4_32_10_t st;
  curand_init(seed[i], sub[i], off[i], &st);
  out[i] = curand4(&st);
}

int main() {
  const int n = 64;
  std::vector<unsigned long long> seed(n), sub(n), off(n);
  unsigned long long x = 0x2545F4914F6CDD1Dull;  // xorshift64 state
  auto next = [&]() {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return x;
  };
  for (int i = 0; i < n; ++i) {
    seed[i] = i == 0 ? 0ull : next();
    sub[i] = i < 2 ? 0ull : (i % 3 == 0 ? next() : next() & 0xffffffffull);
    off[i] = i < 3 ? 0ull : (next() & 0xffffffffffull) * 4ull;  // whole blocks
  }
  unsigned long long *ds, *dsub, *doff;
  uint4 *dout;
  if (cudaMalloc(&ds, n * 8) || cudaMalloc(&dsub, n * 8) || cudaMalloc(&doff, n * 8) ||
      cudaMalloc(&dout, n * sizeof(uint4))) {
    std::fprintf(stderr, "cudaMalloc failed\n");
    return 1;
  }
  cudaMemcpy(ds, seed.data(), n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(dsub, sub.data(), n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(doff, off.data(), n * 8, cudaMemcpyHostToDevice);
  k_draw<<<1, 64>>>(ds, dsub, doff, dout, n);
  std::vector<uint4> out(n);
  if (cudaMemcpy(out.data(), dout, n * sizeof(uint4), cudaMemcpyDeviceToHost) != cudaSuccess) {
    std::fprintf(stderr, "kernel failed: %s\n", cudaGetErrorString(cudaGetLastError()));
    return 1;
  }
  for (int i = 0; i < n; ++i)
    std::printf("%llx %llx %llx %08x %08x %08x %08x\n", seed[i], sub[i], off[i], out[i].x, out[i].y, out[i].z,
                out[i].w);
  cudaFree(ds);
  cudaFree(dsub);
  cudaFree(doff);
  cudaFree(dout);
  return 0;
}
