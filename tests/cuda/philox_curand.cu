// Prints cuRAND's Philox4x32-10 outputs and the project's rh_philox4x32_10 for
// the same counter/key, to pin the shared uniform provider against NVIDIA's
// implementation.  Build: nvcc -gencode arch=compute_103a,code=sm_103a
#include <curand_kernel.h>
#include <stdio.h>

#include "rh_philox.h"

__global__ void k(unsigned long long seed, unsigned long long subseq, uint4* out, uint4* mine) {
  curandStatePhilox4_32_10_t st;
  curand_init(seed, subseq, 0, &st);
  out[0] = curand4(&st);
  out[1] = curand4(&st);
  rh_u32x4 a = rh_philox4x32_10(0, 0, (uint32_t)subseq, (uint32_t)(subseq >> 32),
                                (uint32_t)seed, (uint32_t)(seed >> 32));
  rh_u32x4 b = rh_philox4x32_10(1, 0, (uint32_t)subseq, (uint32_t)(subseq >> 32),
                                (uint32_t)seed, (uint32_t)(seed >> 32));
  mine[0] = make_uint4(a.w[0], a.w[1], a.w[2], a.w[3]);
  mine[1] = make_uint4(b.w[0], b.w[1], b.w[2], b.w[3]);
}

int main() {
  unsigned long long cases[][2] = {{0ull, 0ull}, {18ull, 0ull}, {18ull, 977ull},
                                   {1ull, 123456789ull}, {0xdeadbeefcafef00dull, 5ull}};
  uint4 *d, *m;
  cudaMalloc(&d, 2 * sizeof(uint4));
  cudaMalloc(&m, 2 * sizeof(uint4));
  for (auto& c : cases) {
    k<<<1, 1>>>(c[0], c[1], d, m);
    uint4 h[2], hm[2];
    cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaMemcpy(hm, m, sizeof hm, cudaMemcpyDeviceToHost);
    for (int i = 0; i < 2; ++i)
      printf("%llu %llu %d curand %08x %08x %08x %08x mine %08x %08x %08x %08x\n", c[0], c[1], i,
             h[i].x, h[i].y, h[i].z, h[i].w, hm[i].x, hm[i].y, hm[i].z, hm[i].w);
  }
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? 0 : 1;
}
