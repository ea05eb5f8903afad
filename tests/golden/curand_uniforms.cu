// Test helper (not part of the engine): the uniforms the reference's weighted-MinHash
// sampler consumes (weightedMinHash.cuh:118-126, :151-158).  For hash h (seed
// h*1234 + 92138, createSeedArr :252-262): curand_init(seed, 0, 10000) then T draws of
// curand_uniform.  Writes float32 [H][T] to stdout.
// Usage: curand_uniforms H T
#include <curand_kernel.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

__global__ void draw(int H, int T, float* out) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= H) return;
  int seed = h * 1234 + 92138;
  curandState s;
  curand_init(seed, 0, 10000, &s);
  for (int j = 0; j < T; ++j) out[(size_t)h * T + j] = curand_uniform(&s);
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  int H = atoi(argv[1]), T = atoi(argv[2]);
  if (H <= 0 || T <= 0 || (size_t)H * T > (1u << 28)) return 2;
  float* d = nullptr;
  if (cudaMalloc(&d, (size_t)H * T * sizeof(float)) != cudaSuccess) return 1;
  draw<<<(H + 127) / 128, 128>>>(H, T, d);
  std::vector<float> h((size_t)H * T);
  if (cudaMemcpy(h.data(), d, h.size() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
  cudaFree(d);
  fwrite(h.data(), sizeof(float), h.size(), stdout);
  return 0;
}
