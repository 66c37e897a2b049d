// mlp.cu — the surrogate network: 4 -> 128 -> 128 -> 128 -> 3, BF16 weights
// and activations, FP32 accumulation and FP32 master weights (Adam).
//
// Outputs: y0 = sigmoid(z0) (EAD probability), y1 = z1 (normalised APD90
// mean), y2 = softplus(z2) (normalised APD90 variance).  Loss per sample:
// BCE(y0, p) + (y1 - m)^2 + (y2 - s)^2, averaged over the batch.
//
// Every GEMM of the handle-based passes (forward Z = A W^T, backward
// dA = dZ W and dW = dZ^T A) runs on Blackwell's 5th-generation tensor cores
// through gemm_tc (tcgen05.mma, BF16 x BF16 -> FP32 accumulator in tensor
// memory).  The no-allocation forward and the GEMM check keep gemm_bf16
// (mma.sync m16n8k16), which also serves as gemm_tc's independent check.
// Padded shapes: layer 1 K = 16 (4 inputs + zeros), layer 4 N = 8 (3
// outputs + zeros; the tcgen05 MMA pads N to 16).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rh_mlp.h"

namespace {

constexpr int H = 128;   // hidden width
constexpr int KIN = 16;  // padded input width
constexpr int NOUT = 8;  // padded output width

// C[M,N] (f32, row-major, ldc) = sum_k A(m,k) B(k,n); A(m,k) = A[m*sam + k*sak],
// B(k,n) = Bm[k*sbk + n*sbn]; out-of-range elements read as zero.
// One warp per 16 x 8 output tile.
__global__ void gemm_bf16(const __nv_bfloat16* __restrict__ A, int sam, int sak,
                          const __nv_bfloat16* __restrict__ Bm, int sbk, int sbn, float* C, int ldc,
                          int M, int N, int K, int accumulate) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int tiles_n = (N + 7) / 8;
  const int tm = warp / tiles_n, tn = warp % tiles_n;
  if (tm * 16 >= M) return;
  const int g = lane >> 2, tq = lane & 3;
  const int m0 = tm * 16, n0 = tn * 8;
  float c[4] = {0.f, 0.f, 0.f, 0.f};
  auto ldA = [&](int m, int k) -> __nv_bfloat16 {
    return (m < M && k < K) ? A[(int64_t)m * sam + (int64_t)k * sak] : __float2bfloat16(0.f);
  };
  auto ldB = [&](int k, int n) -> __nv_bfloat16 {
    return (k < K && n < N) ? Bm[(int64_t)k * sbk + (int64_t)n * sbn] : __float2bfloat16(0.f);
  };
  auto pack = [](__nv_bfloat16 lo, __nv_bfloat16 hi) -> uint32_t {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
  };
  for (int k0 = 0; k0 < K; k0 += 16) {
    const int ka = k0 + tq * 2;
    uint32_t a0 = pack(ldA(m0 + g, ka), ldA(m0 + g, ka + 1));
    uint32_t a1 = pack(ldA(m0 + g + 8, ka), ldA(m0 + g + 8, ka + 1));
    uint32_t a2 = pack(ldA(m0 + g, ka + 8), ldA(m0 + g, ka + 9));
    uint32_t a3 = pack(ldA(m0 + g + 8, ka + 8), ldA(m0 + g + 8, ka + 9));
    uint32_t b0 = pack(ldB(ka, n0 + g), ldB(ka + 1, n0 + g));
    uint32_t b1 = pack(ldB(ka + 8, n0 + g), ldB(ka + 9, n0 + g));
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  const int r0 = m0 + g, r1 = m0 + g + 8, cc = n0 + tq * 2;
  float* out[4] = {C + (int64_t)r0 * ldc + cc, C + (int64_t)r0 * ldc + cc + 1,
                   C + (int64_t)r1 * ldc + cc, C + (int64_t)r1 * ldc + cc + 1};
  const bool ok[4] = {r0 < M && cc < N, r0 < M && cc + 1 < N, r1 < M && cc < N,
                      r1 < M && cc + 1 < N};
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (ok[q]) *out[q] = accumulate ? *out[q] + c[q] : c[q];
}

// ---- the same GEMM on the 5th-generation tensor cores (tcgen05) ----
//
// One CTA of 128 threads per 128-row tile of C, every column of C (N <= 256).
// K is staged in chunks of 128 elements: the threads copy A (128 x 128) and
// B (N x 128, as the MMA's N x K operand) from global memory into shared
// memory in the canonical K-major layout without swizzle (core matrices of 8
// rows x 16 bytes), one elected thread issues eight tcgen05.mma (M = 128,
// N = the padded width, K = 16 each) into an FP32 accumulator in tensor
// memory and commits them to an mbarrier, and the next chunk is staged once
// they have read shared memory.  Each warp then reads its 32 accumulator
// rows with tcgen05.ld and writes C.  Out-of-range elements read as zero.
// Every wait on the mbarrier is bounded: on expiry the CTA sets *err, skips
// the rest of its MMAs and still frees its tensor memory.
namespace tc {

constexpr int kM = 128;   // rows per CTA = tensor-memory lanes
constexpr int kKc = 128;  // K elements per staged chunk
constexpr int kNmax = 128;
constexpr int kSmemA = kM * kKc * 2;      // bytes
constexpr int kSmemB = kNmax * kKc * 2;
constexpr long long kWaitLimit = 1 << 22;  // polls of an mbarrier (a few ms)

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor of tcgen05: start address, the byte
// distance between core matrices adjacent along K (lbo) and along M or N
// (sbo), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Byte offset of element (row, k) of a staged operand with `rows` rows
// (a multiple of 8): core matrix (row / 8, k / 8) at ((k/8) * rows/8 +
// row/8) * 128, row % 8 at 16-byte steps, k % 8 at 2-byte steps.
__device__ __forceinline__ uint32_t core_off(int row, int k, int rows) {
  return (uint32_t)(((k >> 3) * (rows >> 3) + (row >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace tc

// C[M,N] (f32, row-major, ldc) = sum_k A(m,k) B(k,n) (+ C when accumulate),
// with A and B addressed as in gemm_bf16; N <= 128.
__global__ void __launch_bounds__(128, 1)
    gemm_tc(const __nv_bfloat16* __restrict__ A, int sam, int sak,
            const __nv_bfloat16* __restrict__ Bm, int sbk, int sbn, float* C, int ldc, int M,
            int N, int K, int accumulate, int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_base;
  unsigned char* sA = smem;
  unsigned char* sB = smem + tc::kSmemA;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * tc::kM;
  const int Nm = (N + 15) & ~15;                 // MMA width: a multiple of 16
  const uint32_t ncols = Nm <= 32 ? 32u : (Nm <= 64 ? 64u : 128u);  // power of two >= 32
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::saddr(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     tc::saddr(&tmem_base)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = tc::instr_desc(tc::kM, Nm);
  bool ok = true;
  const int nchunks = (K + tc::kKc - 1) / tc::kKc;
  for (int ch = 0; ch < nchunks && ok; ++ch) {
    const int k0 = ch * tc::kKc;
    // stage A (128 x 128) and B (Nm x 128) as 16-byte core-matrix rows
    for (int c = tid; c < tc::kM * (tc::kKc / 8); c += blockDim.x) {
      const int r = c % tc::kM, kg = c / tc::kM;
      uint32_t w[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        __nv_bfloat16 lo = __float2bfloat16(0.f), hi = lo;
        const int m = m0 + r, k = k0 + kg * 8 + 2 * j;
        if (m < M && k < K) lo = A[(int64_t)m * sam + (int64_t)k * sak];
        if (m < M && k + 1 < K) hi = A[(int64_t)m * sam + (int64_t)(k + 1) * sak];
        w[j] = (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
      }
      *reinterpret_cast<uint4*>(sA + tc::core_off(r, kg * 8, tc::kM)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
    for (int c = tid; c < Nm * (tc::kKc / 8); c += blockDim.x) {
      const int n = c % Nm, kg = c / Nm;
      uint32_t w[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        __nv_bfloat16 lo = __float2bfloat16(0.f), hi = lo;
        const int k = k0 + kg * 8 + 2 * j;
        if (n < N && k < K) lo = Bm[(int64_t)k * sbk + (int64_t)n * sbn];
        if (n < N && k + 1 < K) hi = Bm[(int64_t)(k + 1) * sbk + (int64_t)n * sbn];
        w[j] = (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
      }
      *reinterpret_cast<uint4*>(sB + tc::core_off(n, kg * 8, Nm)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
    // the staged operands become visible to the tensor core's (async) proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = tc::saddr(sA), b0 = tc::saddr(sB);
      // K-adjacent core matrices are rows/8 * 128 bytes apart, M/N-adjacent 128
      const uint32_t lbo_a = (tc::kM / 8) * 128, lbo_b = (uint32_t)(Nm / 8) * 128;
#pragma unroll
      for (int s = 0; s < tc::kKc / 16; ++s) {
        const uint64_t ad = tc::smem_desc(a0 + (uint32_t)s * 2 * lbo_a, lbo_a, 128);
        const uint64_t bd = tc::smem_desc(b0 + (uint32_t)s * 2 * lbo_b, lbo_b, 128);
        const uint32_t acc = (ch > 0 || s > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              tc::saddr(&bar))
          : "memory");
    }
    // every thread saw the MMAs finish (or the wait give up) before the next
    // chunk is staged; the outcome is the same in every thread
    ok = __syncthreads_and(tc::mbar_wait(tc::saddr(&bar), (uint32_t)(ch & 1)) ? 1 : 0) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, 1);
  } else {
    // epilogue: warp w reads accumulator rows 32w..32w+31 (its tensor-memory lanes)
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < Nm; c0 += 16) {
      uint32_t v[16];
      const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(ta)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = c0 + j;
          if (col < N) {
            float* o = C + (int64_t)row * ldc + col;
            const float x = __uint_as_float(v[j]);
            *o = accumulate ? *o + x : x;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  __syncwarp();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols)
                 : "memory");
}

// Z += bias (per column); A = relu(Z) in BF16 (hidden layers).
__global__ void bias_relu(float* Z, const float* bias, __nv_bfloat16* Aout, int M, int N) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)M * N) return;
  float z = Z[i] + bias[i % N];
  Z[i] = z;
  Aout[i] = __float2bfloat16(z > 0.f ? z : 0.f);
}

__device__ __forceinline__ float sigmoidf_(float x) { return 1.f / (1.f + expf(-x)); }
__device__ __forceinline__ float softplusf_(float x) { return x > 20.f ? x : log1pf(expf(x)); }

// Output layer: y, loss terms and dZ4 (scaled by 1/B), in FP32 and BF16.
__global__ void output_loss(float* Z4, const float* b4, const float* target, float* y,
                            float* dz4, __nv_bfloat16* dz4b, float* loss_terms, int B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  float z0 = Z4[i * NOUT + 0] + b4[0], z1 = Z4[i * NOUT + 1] + b4[1], z2 = Z4[i * NOUT + 2] + b4[2];
  float y0 = sigmoidf_(z0), y1 = z1, y2 = softplusf_(z2);
  y[i * 3 + 0] = y0;
  y[i * 3 + 1] = y1;
  y[i * 3 + 2] = y2;
  float l = 0.f;
  float g0 = 0.f, g1 = 0.f, g2 = 0.f;
  if (target) {
    const float p = target[i * 3 + 0], m = target[i * 3 + 1], s = target[i * 3 + 2];
    const float e = 1e-7f;
    l = -(p * logf(fmaxf(y0, e)) + (1.f - p) * logf(fmaxf(1.f - y0, e))) + (y1 - m) * (y1 - m) +
        (y2 - s) * (y2 - s);
    const float invB = 1.f / (float)B;
    g0 = (y0 - p) * invB;
    g1 = 2.f * (y1 - m) * invB;
    g2 = 2.f * (y2 - s) * sigmoidf_(z2) * invB;
    loss_terms[i] = l;
  }
  const float gg[NOUT] = {g0, g1, g2, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int q = 0; q < NOUT; ++q) {
    dz4[i * NOUT + q] = gg[q];
    dz4b[i * NOUT + q] = __float2bfloat16(gg[q]);
  }
}

// dZ = dA * relu'(Z) -> BF16
__global__ void relu_backward(const float* dA, const float* Z, __nv_bfloat16* dZb, float* dZf,
                              int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float d = Z[i] > 0.f ? dA[i] : 0.f;
  dZf[i] = d;
  dZb[i] = __float2bfloat16(d);
}

// db[n] = sum over rows of dZ (fixed order per column)
__global__ void bias_grad(const float* dZ, float* db, int M, int N) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += dZ[(int64_t)m * N + n];
  db[n] = s;
}

// Adam step on FP32 masters, refresh the BF16 copies.  Padded entries (mask
// 0) stay zero.
__global__ void adam_update(float* w, const float* g, float* m, float* v, __nv_bfloat16* wb,
                            const float* mask, int n, float lr, float b1, float b2, float eps,
                            float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (mask && mask[i] == 0.f) {
    w[i] = 0.f;
    if (wb) wb[i] = __float2bfloat16(0.f);
    return;
  }
  float gi = g[i];
  float mi = b1 * m[i] + (1.f - b1) * gi;
  float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16(wi);
}

// inputs (B x 4 floats) -> padded BF16 rows of 16
__global__ void pack_inputs(const float* x, __nv_bfloat16* X0, int B) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)B * KIN) return;
  const int r = (int)(i / KIN), c = (int)(i % KIN);
  X0[i] = __float2bfloat16(c < RH_MLP_IN ? x[r * RH_MLP_IN + c] : 0.f);
}

unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------- host side

struct rh_mlp {
  int bmax = 0;
  cudaStream_t st = nullptr;
  // parameters: FP32 masters, BF16 copies, Adam moments, gradients
  float* P = nullptr;  // all FP32 buffers in one allocation
  __nv_bfloat16* Pb = nullptr;
  float *w[4], *b[4], *gw[4], *gb[4], *mw[4], *vw[4], *mb[4], *vb[4], *maskw[4];
  __nv_bfloat16* wb[4];
  int wn[4], wk[4];
  // activations
  __nv_bfloat16 *X0, *A[3], *dZb[4];
  float *Z[4], *dA, *dZf, *y, *target, *xin, *loss;
  int64_t step = 0;
  int* gemm_err = nullptr;  // set by a tcgen05 GEMM whose wait gave up
  std::string err;
};

namespace {

int ck(rh_mlp* m, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return RH_OK;
  if (m) m->err = std::string(what) + ": " + cudaGetErrorString(e);
  return RH_ERR_CUDA;
}
#define MCK(x)                                 \
  do {                                         \
    int r_ = ck(m, (x), #x);                   \
    if (r_) return r_;                         \
  } while (0)

// Every GEMM of the network's handle-based passes runs on the tcgen05
// kernel (the no-allocation forward keeps the mma.sync kernel).
int gemm(rh_mlp* m, const __nv_bfloat16* A, int sam, int sak, const __nv_bfloat16* B, int sbk,
         int sbn, float* C, int ldc, int M, int N, int K, int acc) {
  gemm_tc<<<(M + tc::kM - 1) / tc::kM, 128, tc::kSmemA + tc::kSmemB, m->st>>>(
      A, sam, sak, B, sbk, sbn, C, ldc, M, N, K, acc, m->gemm_err);
  return ck(m, cudaGetLastError(), "gemm");
}

// After a stream synchronisation: RH_ERR_TIMEOUT when a GEMM's wait gave up.
int check_gemm(rh_mlp* m) {
  int h = 0;
  MCK(cudaMemcpy(&h, m->gemm_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    cudaMemset(m->gemm_err, 0, sizeof(int));
    m->err = "a tensor-core GEMM's wait for its MMAs ran out";
    return RH_ERR_TIMEOUT;
  }
  return RH_OK;
}

int forward(rh_mlp* m, int B) {
  // layer l: Z = A_{l-1} W_l^T  (W_l stored n x k, row-major)
  const __nv_bfloat16* in = m->X0;
  int kin = KIN;
  for (int l = 0; l < 3; ++l) {
    int r = gemm(m, in, kin, 1, m->wb[l], 1, kin, m->Z[l], H, B, H, kin, 0);
    if (r) return r;
    bias_relu<<<blocks((int64_t)B * H, 256), 256, 0, m->st>>>(m->Z[l], m->b[l], m->A[l], B, H);
    in = m->A[l];
    kin = H;
  }
  return gemm(m, m->A[2], H, 1, m->wb[3], 1, H, m->Z[3], NOUT, B, NOUT, H, 0);
}

int backward(rh_mlp* m, int B) {
  // output layer gradients were written by output_loss into dZf/dZb[3]
  // dW4 = dZ4^T A3 ; db4 = sum dZ4 ; dA3 = dZ4 W4
  int r;
  const __nv_bfloat16* acts[4] = {m->X0, m->A[0], m->A[1], m->A[2]};
  const int kins[4] = {KIN, H, H, H};
  const int nouts[4] = {H, H, H, NOUT};
  for (int l = 3; l >= 0; --l) {
    const int N = nouts[l], K = kins[l];
    // dW_l (N x K) = dZ_l^T (N x B) * A_{l-1} (B x K)
    if ((r = gemm(m, m->dZb[l], 1, N, acts[l], K, 1, m->gw[l], K, N, K, B, 0))) return r;
    if (l == 3) {
      // dZ4 in FP32 lives in dA's first B*8 entries (written by output_loss)
      bias_grad<<<blocks(N, 128), 128, 0, m->st>>>(m->dA, m->gb[l], B, N);
    } else {
      bias_grad<<<blocks(N, 128), 128, 0, m->st>>>(m->dZf, m->gb[l], B, N);
    }
    if (l == 0) break;
    // dA_{l-1} (B x K) = dZ_l (B x N) * W_l (N x K)
    if ((r = gemm(m, m->dZb[l], N, 1, m->wb[l], K, 1, m->dA, K, B, K, N, 0))) return r;
    relu_backward<<<blocks((int64_t)B * K, 256), 256, 0, m->st>>>(m->dA, m->Z[l - 1], m->dZb[l - 1],
                                                                m->dZf, (int64_t)B * K);
  }
  return ck(m, cudaGetLastError(), "backward");
}

int run_loss(rh_mlp* m, int B, const float* xh, const float* th, float* loss_out) {
  MCK(cudaMemcpyAsync(m->xin, xh, sizeof(float) * RH_MLP_IN * B, cudaMemcpyHostToDevice, m->st));
  if (th)
    MCK(cudaMemcpyAsync(m->target, th, sizeof(float) * 3 * B, cudaMemcpyHostToDevice, m->st));
  pack_inputs<<<blocks((int64_t)B * KIN, 256), 256, 0, m->st>>>(m->xin, m->X0, B);
  int r = forward(m, B);
  if (r) return r;
  output_loss<<<blocks(B, 128), 128, 0, m->st>>>(m->Z[3], m->b[3], th ? m->target : nullptr, m->y,
                                                 m->dA, m->dZb[3], m->loss, B);
  MCK(cudaGetLastError());
  if (loss_out && th) {
    std::vector<float> l(B);
    MCK(cudaMemcpyAsync(l.data(), m->loss, sizeof(float) * B, cudaMemcpyDeviceToHost, m->st));
    MCK(cudaStreamSynchronize(m->st));
    double s = 0;
    for (float v : l) s += v;
    *loss_out = (float)(s / B);
  }
  return RH_OK;
}

}  // namespace

extern "C" {

int rh_mlp_gemm_check(const void* A, int32_t sam, int32_t sak, const void* B, int32_t sbk,
                      int32_t sbn, float* C, int32_t ldc, int32_t M, int32_t N, int32_t K,
                      int32_t tensor_cores) {
  if (!A || !B || !C || M <= 0 || N <= 0 || N > tc::kNmax || K <= 0) return RH_ERR_ARG;
  const __nv_bfloat16* a = static_cast<const __nv_bfloat16*>(A);
  const __nv_bfloat16* b = static_cast<const __nv_bfloat16*>(B);
  if (!tensor_cores) {
    const int tiles = ((M + 15) / 16) * ((N + 7) / 8);
    gemm_bf16<<<blocks((int64_t)tiles * 32, 128), 128>>>(a, sam, sak, b, sbk, sbn, C, ldc, M, N,
                                                         K, 0);
  } else {
    int* err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return RH_ERR_NOMEM;
    cudaMemset(err, 0, sizeof(int));
    const int smem = tc::kSmemA + tc::kSmemB;
    cudaFuncSetAttribute(gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    gemm_tc<<<(M + tc::kM - 1) / tc::kM, 128, smem>>>(a, sam, sak, b, sbk, sbn, C, ldc, M, N, K,
                                                      0, err);
    int h = 0;
    cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(err);
    if (h) return RH_ERR_TIMEOUT;
  }
  if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) return RH_ERR_CUDA;
  return RH_OK;
}

int rh_mlp_create(int32_t batch_max, int32_t device, rh_mlp** out) {
  if (!out || batch_max <= 0) return RH_ERR_ARG;
  *out = nullptr;
  rh_mlp* m = new rh_mlp();
  m->bmax = batch_max;
  const int wn[4] = {H, H, H, NOUT}, wk[4] = {KIN, H, H, H};
  size_t nf = 0, nb = 0;
  for (int l = 0; l < 4; ++l) {
    m->wn[l] = wn[l];
    m->wk[l] = wk[l];
    nf += (size_t)7 * wn[l] * wk[l] + 5 * wn[l];  // w gw mw vw maskw + b gb mb vb
    nb += (size_t)wn[l] * wk[l];
  }
  const size_t B = (size_t)batch_max;
  nf += 4 * B * H + B * H * 2 + B * 3 * 2 + B * RH_MLP_IN + B;  // Z0-2, Z3(8), dA, dZf, y, target, xin, loss
  nb += B * KIN + 3 * B * H + 3 * B * H + B * NOUT;              // X0, A0-2, dZb0-2, dZb3
  int r = RH_OK;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreate(&m->st) != cudaSuccess ||
      cudaMalloc(&m->P, nf * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m->Pb, nb * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc(&m->gemm_err, sizeof(int)) != cudaSuccess ||
      cudaMemset(m->gemm_err, 0, sizeof(int)) != cudaSuccess ||
      cudaFuncSetAttribute(gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           tc::kSmemA + tc::kSmemB) != cudaSuccess) {
    m->err = "allocation failed";
    r = RH_ERR_NOMEM;
  }
  if (r == RH_OK) {
    cudaMemset(m->P, 0, nf * sizeof(float));
    cudaMemset(m->Pb, 0, nb * sizeof(__nv_bfloat16));
    float* p = m->P;
    __nv_bfloat16* pb = m->Pb;
    for (int l = 0; l < 4; ++l) {
      const size_t nw = (size_t)wn[l] * wk[l];
      m->w[l] = p; p += nw;
      m->gw[l] = p; p += nw;
      m->mw[l] = p; p += nw;
      m->vw[l] = p; p += nw;
      m->maskw[l] = p; p += nw;
      m->b[l] = p; p += wn[l];
      m->gb[l] = p; p += wn[l];
      m->mb[l] = p; p += wn[l];
      m->vb[l] = p; p += wn[l];
      p += (size_t)2 * nw;  // spare (keeps the arithmetic above honest)
      p += wn[l];
      m->wb[l] = pb; pb += nw;
    }
    m->Z[0] = p; p += B * H;
    m->Z[1] = p; p += B * H;
    m->Z[2] = p; p += B * H;
    m->Z[3] = p; p += B * H;  // only B*NOUT used
    m->dA = p; p += B * H;
    m->dZf = p; p += B * H;
    m->y = p; p += B * 3;
    m->target = p; p += B * 3;
    m->xin = p; p += B * RH_MLP_IN;
    m->loss = p; p += B;
    m->X0 = pb; pb += B * KIN;
    for (int l = 0; l < 3; ++l) { m->A[l] = pb; pb += B * H; }
    for (int l = 0; l < 3; ++l) { m->dZb[l] = pb; pb += B * H; }
    m->dZb[3] = pb; pb += B * NOUT;
    // masks: real weights 1, padding 0 (layer 1 inputs >= 4, layer 4 outputs >= 3)
    for (int l = 0; l < 4; ++l) {
      std::vector<float> mk((size_t)wn[l] * wk[l], 1.f);
      for (int n = 0; n < wn[l]; ++n)
        for (int k = 0; k < wk[l]; ++k)
          if ((l == 0 && k >= RH_MLP_IN) || (l == 3 && n >= RH_MLP_OUT)) mk[(size_t)n * wk[l] + k] = 0.f;
      cudaMemcpy(m->maskw[l], mk.data(), mk.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
      m->err = "initialisation failed";
      r = RH_ERR_CUDA;
    }
  }
  if (r != RH_OK) {
    rh_mlp_destroy(m);
    return r;
  }
  *out = m;
  return RH_OK;
}

int rh_mlp_destroy(rh_mlp* m) {
  if (!m) return RH_ERR_ARG;
  if (m->st) cudaStreamSynchronize(m->st);
  cudaFree(m->P);
  cudaFree(m->Pb);
  cudaFree(m->gemm_err);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
  return RH_OK;
}

int rh_mlp_param_count(const rh_mlp* m, int32_t* n) {
  if (!m || !n) return RH_ERR_ARG;
  int s = 0;
  for (int l = 0; l < 4; ++l) s += m->wn[l] * m->wk[l] + m->wn[l];
  *n = s;
  return RH_OK;
}

// Parameter order: for each layer, W (n x k row-major, padded) then b (n).
int rh_mlp_set_params(rh_mlp* m, const float* params) {
  if (!m || !params) return RH_ERR_ARG;
  const float* p = params;
  for (int l = 0; l < 4; ++l) {
    const size_t nw = (size_t)m->wn[l] * m->wk[l];
    MCK(cudaMemcpy(m->w[l], p, nw * sizeof(float), cudaMemcpyHostToDevice));
    p += nw;
    MCK(cudaMemcpy(m->b[l], p, m->wn[l] * sizeof(float), cudaMemcpyHostToDevice));
    p += m->wn[l];
    // apply the padding mask and refresh BF16 copies; reset Adam
    adam_update<<<blocks(nw, 256), 256, 0, m->st>>>(m->w[l], m->gw[l], m->mw[l], m->vw[l], m->wb[l],
                                                   m->maskw[l], (int)nw, 0.f, 0.f, 0.f, 1.f, 1.f, 1.f);
    MCK(cudaMemsetAsync(m->mw[l], 0, nw * sizeof(float), m->st));
    MCK(cudaMemsetAsync(m->vw[l], 0, nw * sizeof(float), m->st));
    MCK(cudaMemsetAsync(m->mb[l], 0, m->wn[l] * sizeof(float), m->st));
    MCK(cudaMemsetAsync(m->vb[l], 0, m->wn[l] * sizeof(float), m->st));
  }
  m->step = 0;
  MCK(cudaStreamSynchronize(m->st));
  return RH_OK;
}

int rh_mlp_get_params(rh_mlp* m, float* params) {
  if (!m || !params) return RH_ERR_ARG;
  MCK(cudaStreamSynchronize(m->st));
  float* p = params;
  for (int l = 0; l < 4; ++l) {
    const size_t nw = (size_t)m->wn[l] * m->wk[l];
    MCK(cudaMemcpy(p, m->w[l], nw * sizeof(float), cudaMemcpyDeviceToHost));
    p += nw;
    MCK(cudaMemcpy(p, m->b[l], m->wn[l] * sizeof(float), cudaMemcpyDeviceToHost));
    p += m->wn[l];
  }
  return RH_OK;
}

int rh_mlp_forward(rh_mlp* m, const float* x, int32_t n, float* y) {
  if (!m || !x || !y || n <= 0) return RH_ERR_ARG;
  for (int32_t off = 0; off < n; off += m->bmax) {
    const int B = (int)std::min<int64_t>(m->bmax, n - off);
    int r = run_loss(m, B, x + (size_t)off * RH_MLP_IN, nullptr, nullptr);
    if (r) return r;
    MCK(cudaMemcpyAsync(y + (size_t)off * 3, m->y, sizeof(float) * 3 * B, cudaMemcpyDeviceToHost,
                        m->st));
  }
  MCK(cudaStreamSynchronize(m->st));
  return check_gemm(m);
}

int rh_mlp_gradients(rh_mlp* m, const float* x, const float* target, int32_t n, float* grads,
                     float* loss) {
  if (!m || !x || !target || n <= 0 || n > m->bmax) return RH_ERR_ARG;
  int r = run_loss(m, n, x, target, loss);
  if (r) return r;
  if ((r = backward(m, n))) return r;
  if (grads) {
    MCK(cudaStreamSynchronize(m->st));
    if ((r = check_gemm(m))) return r;
    float* p = grads;
    for (int l = 0; l < 4; ++l) {
      const size_t nw = (size_t)m->wn[l] * m->wk[l];
      MCK(cudaMemcpy(p, m->gw[l], nw * sizeof(float), cudaMemcpyDeviceToHost));
      p += nw;
      MCK(cudaMemcpy(p, m->gb[l], m->wn[l] * sizeof(float), cudaMemcpyDeviceToHost));
      p += m->wn[l];
    }
  }
  return RH_OK;
}

int rh_mlp_train_step(rh_mlp* m, const float* x, const float* target, int32_t n, float lr,
                      float* loss) {
  int r = rh_mlp_gradients(m, x, target, n, nullptr, loss);
  if (r) return r;
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float bc1 = 1.f - powf(b1, (float)m->step), bc2 = 1.f - powf(b2, (float)m->step);
  for (int l = 0; l < 4; ++l) {
    const int nw = m->wn[l] * m->wk[l];
    adam_update<<<blocks(nw, 256), 256, 0, m->st>>>(m->w[l], m->gw[l], m->mw[l], m->vw[l], m->wb[l],
                                                   m->maskw[l], nw, lr, b1, b2, eps, bc1, bc2);
    adam_update<<<blocks(m->wn[l], 128), 128, 0, m->st>>>(m->b[l], m->gb[l], m->mb[l], m->vb[l],
                                                         nullptr, nullptr, m->wn[l], lr, b1, b2, eps,
                                                         bc1, bc2);
  }
  MCK(cudaGetLastError());
  MCK(cudaStreamSynchronize(m->st));
  return check_gemm(m);
}

int rh_mlp_last_error(const rh_mlp* m, char* buf, size_t n) {
  if (!buf || n == 0) return RH_ERR_ARG;
  snprintf(buf, n, "%s", m ? m->err.c_str() : "");
  return RH_OK;
}

}  // extern "C"

// ------------------------------------------------ forward pass without allocation
//
// rh_mlp_forward above works on a handle whose buffers rh_mlp_create obtained
// with cudaMalloc.  Some callers cannot make that call: a host program whose
// device memory is all handed out by its own allocator or pool, a co-simulation
// loop that budgets device memory up front, or a caller that must not pay the
// device-wide synchronisation an allocation can imply.  rh_mlp_forward_noalloc
// serves them: the caller brings the parameters, inputs and outputs in device
// memory, and the intermediate values (BF16 weight copies, packed inputs,
// pre-activations, activations, output-layer terms) live in the fixed array
// below, which is part of the library image on every device that loads it.

static __device__ __align__(256) unsigned char g_forward_scratch[RH_MLP_NOALLOC_SCRATCH_BYTES];

namespace {

// Byte offsets inside the scratch array, each a multiple of 256.
constexpr size_t kNaRows = RH_MLP_NOALLOC_MAX_BATCH;
constexpr size_t kNaWeights = (size_t)H * KIN + 2 * (size_t)H * H + (size_t)NOUT * H;
constexpr size_t round256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kOffW = 0;
constexpr size_t kOffX0 = kOffW + round256(kNaWeights * 2);
constexpr size_t kOffZ = kOffX0 + round256(kNaRows * KIN * 2);
constexpr size_t kOffA = kOffZ + round256(kNaRows * H * 4);
constexpr size_t kOffDz = kOffA + round256(kNaRows * H * 2);
constexpr size_t kOffDzb = kOffDz + round256(kNaRows * NOUT * 4);
constexpr size_t kNaEnd = kOffDzb + round256(kNaRows * NOUT * 2);
static_assert(kNaEnd <= RH_MLP_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the array");

// FP32 weights of one layer -> BF16, padding entries (layer 1 inputs >= 4,
// layer 4 outputs >= 3) forced to zero, as rh_mlp_set_params does.
__global__ void weights_to_bf16(const float* w, __nv_bfloat16* wb, int n, int k, int nvalid,
                                int kvalid) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * k) return;
  const int r = i / k, c = i % k;
  wb[i] = __float2bfloat16(r < nvalid && c < kvalid ? w[i] : 0.f);
}

constexpr int kMaxDevices = 64;
// The device address of the scratch array belongs to one CUDA context.  The
// cache holds it per device together with the id of the context that was
// current when it was looked up; a call from another context on that device
// (a context the caller made current, or the primary context created anew
// after cudaDeviceReset) looks it up again.
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

// Id of the calling thread's current context (cuCtxGetCurrent + cuCtxGetId,
// reached through the runtime's driver entry points so that the library does
// not link the driver library itself); false where it cannot be had.
bool current_context_id(unsigned long long* id) {
  using GetCurrentFn = CUresult (*)(CUcontext*);
  using GetIdFn = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetIdFn>(f);
  });
  CUcontext ctx = nullptr;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

void na_msg(char* err, size_t len, const char* fmt, ...) __attribute__((format(printf, 3, 4)));
void na_msg(char* err, size_t len, const char* fmt, ...) {
  if (!err || len == 0) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(err, len, fmt, ap);
  va_end(ap);
}

bool on_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (a.type == cudaMemoryTypeDevice && a.device == dev) || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" int rh_mlp_forward_noalloc(const float* d_params, const float* d_x, int32_t n,
                                      float* d_y, void* stream, char* err, size_t err_len) {
  if (err && err_len) err[0] = '\0';
  if (!d_params || !d_x || !d_y) {
    na_msg(err, err_len, "rh_mlp_forward_noalloc: params, x and y must be device pointers");
    return RH_ERR_ARG;
  }
  if (n <= 0 || n > RH_MLP_NOALLOC_MAX_BATCH) {
    na_msg(err, err_len,
           "rh_mlp_forward_noalloc: n = %d is outside 1..%d, the largest batch its fixed "
           "%d-byte scratch array holds; split the batch",
           (int)n, RH_MLP_NOALLOC_MAX_BATCH, RH_MLP_NOALLOC_SCRATCH_BYTES);
    return RH_ERR_ARG;
  }
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    na_msg(err, err_len, "rh_mlp_forward_noalloc: no usable current device (%s)",
           cudaGetErrorString(e));
    return RH_ERR_CUDA;
  }
  if (!on_device(d_params, dev) || !on_device(d_x, dev) || !on_device(d_y, dev)) {
    na_msg(err, err_len,
           "rh_mlp_forward_noalloc: params, x and y must be device memory of the current "
           "device %d",
           dev);
    return RH_ERR_ARG;
  }
  // Set-up, once per device (and context), with that device current: the
  // scratch array's device address.  Later calls from the same context reuse
  // the cached address.
  void* base = nullptr;
  {
    // the pointer checks above ran runtime calls on this thread, so its
    // context is current; without a context id the address is looked up
    // on every call
    unsigned long long ctx = 0;
    const bool known_ctx = current_context_id(&ctx);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev] || !known_ctx || g_scratch_ctx[dev] != ctx) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_forward_scratch);
      if (e != cudaSuccess || !p) {
        na_msg(err, err_len, "rh_mlp_forward_noalloc: cudaGetSymbolAddress failed on device %d: %s",
               dev, cudaGetErrorString(e));
        return RH_ERR_CUDA;
      }
      g_scratch_addr[dev] = p;
      g_scratch_ctx[dev] = known_ctx ? ctx : 0;
    }
    base = g_scratch_addr[dev];
  }
  unsigned char* s = static_cast<unsigned char*>(base);
  __nv_bfloat16* wb = reinterpret_cast<__nv_bfloat16*>(s + kOffW);
  __nv_bfloat16* X0 = reinterpret_cast<__nv_bfloat16*>(s + kOffX0);
  float* Z = reinterpret_cast<float*>(s + kOffZ);
  __nv_bfloat16* A = reinterpret_cast<__nv_bfloat16*>(s + kOffA);
  float* dz = reinterpret_cast<float*>(s + kOffDz);
  __nv_bfloat16* dzb = reinterpret_cast<__nv_bfloat16*>(s + kOffDzb);
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  // Every scratch element read below is written earlier in this call, so the
  // previous call's contents never leak into the result and nothing needs
  // clearing.
  const int wn[4] = {H, H, H, NOUT}, wk[4] = {KIN, H, H, H};
  const float* wl[4];
  const float* bl[4];
  __nv_bfloat16* wbl[4];
  {
    const float* p = d_params;
    __nv_bfloat16* q = wb;
    for (int l = 0; l < 4; ++l) {
      const int nw = wn[l] * wk[l];
      wl[l] = p;
      bl[l] = p + nw;
      wbl[l] = q;
      p += nw + wn[l];
      q += nw;
      weights_to_bf16<<<blocks(nw, 256), 256, 0, st>>>(wl[l], wbl[l], wn[l], wk[l],
                                                        l == 3 ? RH_MLP_OUT : wn[l],
                                                        l == 0 ? RH_MLP_IN : wk[l]);
    }
  }
  const int B = n;
  pack_inputs<<<blocks((int64_t)B * KIN, 256), 256, 0, st>>>(d_x, X0, B);
  const __nv_bfloat16* in = X0;
  for (int l = 0; l < 4; ++l) {
    const int kin = wk[l], nout = wn[l];
    const int tiles = ((B + 15) / 16) * ((nout + 7) / 8);
    gemm_bf16<<<blocks((int64_t)tiles * 32, 128), 128, 0, st>>>(in, kin, 1, wbl[l], 1, kin, Z, nout,
                                                                B, nout, kin, 0);
    if (l < 3) {
      bias_relu<<<blocks((int64_t)B * H, 256), 256, 0, st>>>(Z, bl[l], A, B, H);
      in = A;
    }
  }
  output_loss<<<blocks(B, 128), 128, 0, st>>>(Z, bl[3], nullptr, d_y, dz, dzb, nullptr, B);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    na_msg(err, err_len, "rh_mlp_forward_noalloc: launch failed: %s", cudaGetErrorString(e));
    return RH_ERR_CUDA;
  }
  return RH_OK;
}
