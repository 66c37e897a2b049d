/*
 * rh_mlp.h — C ABI of the surrogate network that screens parameter sweeps.
 *
 * No counterpart in the reference (cuda_Cell_Detailed.cu has no learned
 * component); the network is this project's addition: 4 inputs (RyR open-rate
 * scale Ku2, IKr scale, PCL, [Ca]o, each normalised to [0, 1]) -> three
 * hidden layers of 128 ReLU units -> 3 outputs (EAD probability, normalised
 * APD90 mean, normalised APD90 variance).  BF16 weights and activations,
 * FP32 accumulation on the tensor cores, FP32 master weights trained with
 * Adam by the library's own forward and backward kernels.
 *
 * Parameter vector layout (floats): for layers 1..4, W (n x k, row-major)
 * then b (n), with padded shapes W1 128x16 (inputs 4..15 zero), W2 128x128,
 * W3 128x128, W4 8x128 (outputs 3..7 zero), b4 of 8.
 * Status codes are those of rh.h.
 */
#ifndef RH_MLP_H
#define RH_MLP_H

#include <stddef.h>
#include <stdint.h>

#include "rh.h"

#ifdef __cplusplus
extern "C" {
#endif

#define RH_MLP_IN 4
#define RH_MLP_OUT 3

typedef struct rh_mlp rh_mlp;

int rh_mlp_create(int32_t batch_max, int32_t device, rh_mlp** out);
int rh_mlp_destroy(rh_mlp* m);
int rh_mlp_param_count(const rh_mlp* m, int32_t* n);
int rh_mlp_set_params(rh_mlp* m, const float* params);
int rh_mlp_get_params(rh_mlp* m, float* params);
/* y[n x 3] = network(x[n x 4]); any n (processed in batches of batch_max). */
int rh_mlp_forward(rh_mlp* m, const float* x, int32_t n, float* y);
/* Loss and parameter gradients for one batch (n <= batch_max); grads in the
 * parameter layout (may be NULL). */
int rh_mlp_gradients(rh_mlp* m, const float* x, const float* target, int32_t n, float* grads,
                     float* loss);
/* One Adam step (beta 0.9/0.999) on one batch; returns the batch loss. */
int rh_mlp_train_step(rh_mlp* m, const float* x, const float* target, int32_t n, float lr,
                      float* loss);
int rh_mlp_last_error(const rh_mlp* m, char* buf, size_t n);

/* Forward pass that allocates nothing.  It has no counterpart in the
 * reference.  It is for callers that may not call cudaMalloc themselves or
 * have the library call it: programs whose device memory belongs to their own
 * allocator or pool, and loops that cannot take the synchronisation an
 * allocation can bring.
 *
 * d_params: device FP32 parameter vector in the layout above (what
 * rh_mlp_get_params returns); d_x: device [n x 4]; d_y: device [n x 3]; all
 * on the calling thread's current device.  Same kernels and the same result
 * as rh_mlp_forward with those parameters.  The work is queued on `stream`
 * (a cudaStream_t; NULL = the default stream) and the call returns without
 * waiting for it.
 *
 * The intermediate values live in one fixed device array inside the library,
 * RH_MLP_NOALLOC_SCRATCH_BYTES (4 MiB) per device, held from the library's
 * loading until process exit.  n above RH_MLP_NOALLOC_MAX_BATCH is rejected
 * with RH_ERR_ARG and a message in err (err may be NULL).  The first call on
 * a device looks up that array's device address (one-time set-up, repeated
 * when the call comes from another context of that device, e.g. after
 * cudaDeviceReset); make that first call before any stream capture.  All
 * calls on a device share the array: two calls whose work overlaps on the
 * GPU (different streams, or different threads without ordering) race and
 * give wrong results.  Each
 * call writes every scratch value it reads, so nothing left by an earlier
 * call reaches the result. */
/* Check of the network's GEMM kernels (testing aid; synchronous, default
 * stream): C[M x N] (FP32, row-major, leading dimension ldc) = sum over k of
 * A(m, k) B(k, n), with A(m, k) = A[m*sam + k*sak] and B(k, n) =
 * B[k*sbk + n*sbn] BF16 device arrays and C a device array; N <= 128.
 * tensor_cores = 1 runs the tcgen05 kernel (tensor-memory accumulator) the
 * network uses, 0 the mma.sync kernel kept as its independent check. */
int rh_mlp_gemm_check(const void* A, int32_t sam, int32_t sak, const void* B, int32_t sbk,
                      int32_t sbn, float* C, int32_t ldc, int32_t M, int32_t N, int32_t K,
                      int32_t tensor_cores);

#define RH_MLP_NOALLOC_MAX_BATCH 4096
#define RH_MLP_NOALLOC_SCRATCH_BYTES (4 * 1024 * 1024)
int rh_mlp_forward_noalloc(const float* d_params, const float* d_x, int32_t n, float* d_y,
                           void* stream, char* err, size_t err_len);

#ifdef __cplusplus
}
#endif

#endif
