/*
 * ref_shim.h — lets the reference program (cuda_Cell_Detailed.cu and the
 * device files it includes) compile and run on the host CPU, unchanged except
 * for the "fixA" deletion and the launch rewrites done by build_ref.sh.
 *
 * TEST INFRASTRUCTURE ONLY: the result lives in oracle/_ref/ and is used to
 * pin the oracle restatement against the reference's own code.
 *
 *   - __global__/__device__ vanish; a kernel launch runs the kernel body once
 *     per lattice site (i,j,k) with threadIdx = (i,j,k), in parallel over
 *     sites with OpenMP.
 *   - curandState becomes the shared Philox stream (include/rh_philox.h):
 *     key = (seed, REF_CELL_ID), counter = (draw/2, subsequence = pos, step).
 *     The step is the number of Compute launches so far, so every Compute
 *     launch restarts each site's draw index at 0.
 *   - cudaMalloc/cudaMemcpy/cudaFree become calloc/memcpy/free.
 * This header is force-included before the reference source.
 */
#ifndef REF_SHIM_H
#define REF_SHIM_H

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/rh_philox.h"

#ifndef REF_CELL_ID
#define REF_CELL_ID 0u
#endif

#define __global__
#define __device__
#define __host__

struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};

inline thread_local dim3 threadIdx;
inline thread_local dim3 blockIdx(0, 0, 0);
inline thread_local dim3 blockDim(1, 1, 1);
inline uint64_t g_ref_step = 0;
inline long long g_ref_max_steps = -1;

struct curandState {
  rh_stream s;
  uint64_t step_seen;
};

inline void curand_init(unsigned long long seed, unsigned long long subsequence,
                        unsigned long long offset, curandState* st) {
  (void)offset;
  rh_stream_init(&st->s, (uint32_t)seed, (uint32_t)REF_CELL_ID, (uint32_t)subsequence, 0);
  st->step_seen = ~0ull;
}

inline void ref_sync_step(curandState* st) {
  if (st->step_seen != g_ref_step) {
    rh_stream_init(&st->s, st->s.k0, st->s.k1, st->s.pos, g_ref_step);
    st->step_seen = g_ref_step;
  }
}

inline double curand_uniform_double(curandState* st) {
  ref_sync_step(st);
  return rh_uniform_double(&st->s);
}

inline unsigned int curand(curandState* st) {
  ref_sync_step(st);
  return rh_uniform_u32(&st->s);
}

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3
};
inline cudaError_t cudaMalloc(void** p, size_t n) {
  *p = calloc(1, n);
  return *p ? 0 : 2;
}
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, int kind) {
  (void)kind;
  memcpy(d, s, n);
  return 0;
}
inline cudaError_t cudaFree(void* p) {
  free(p);
  return 0;
}
inline cudaError_t cudaSetDevice(int) { return 0; }
inline cudaError_t cudaGetLastError() { return 0; }
inline const char* cudaGetErrorString(cudaError_t) { return "no error"; }

/* One kernel launch: the body runs for every lattice site of the full grid. */
template <class F>
inline void ref_launch_all(int gx, int gy, int gz, F&& body) {
#pragma omp parallel for collapse(3) schedule(static)
  for (int k = 0; k < gz; ++k)
    for (int j = 0; j < gy; ++j)
      for (int i = 0; i < gx; ++i) {
        threadIdx = dim3(i, j, k);
        blockIdx = dim3(0, 0, 0);
        blockDim = dim3(1, 1, 1);
        body();
      }
}

/* Step budget for runs that only need a prefix of the protocol
 * (environment variable REF_MAX_STEPS). */
inline bool ref_continue() {
  if (g_ref_max_steps < 0) {
    const char* e = getenv("REF_MAX_STEPS");
    g_ref_max_steps = e ? atoll(e) : (long long)1 << 62;
  }
  return (long long)g_ref_step < g_ref_max_steps;
}

/* The NCX call of Compute (cuda_Cell_Detailed.cu:1296), rewritten by
 * build_ref.sh to REF_NCX(...): the reference's ncx, or with REF_NCX_OLD the
 * oldncx of its commented alternative call (:1300), or with REF_NCX_NOALLO
 * its ncx_noallo (subroutine_cuda.c:102), which takes no allosteric state. */
#if defined(REF_NCX_NOALLO)
#define REF_NCX(cs, v, tp, na, ancx, dt) ncx_noallo(cs, v, tp, na)
#elif defined(REF_NCX_OLD)
#define REF_NCX oldncx
#else
#define REF_NCX ncx
#endif

/* nx, ny, nz are the reference's lattice macros, visible where these expand. */
#define REF_LAUNCH(...) ref_launch_all(nx, ny, nz, [&]() { __VA_ARGS__; })
#define REF_LAUNCH_STEP(...)                                \
  do {                                                      \
    ref_launch_all(nx, ny, nz, [&]() { __VA_ARGS__; });     \
    ++g_ref_step;                                           \
  } while (0)

#endif
