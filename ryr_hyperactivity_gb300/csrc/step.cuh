// step.cuh — launch interface of the step kernels (step.cu).
#pragma once

#include <cuda_runtime.h>

#include "lattice.cuh"

namespace rh {

// CRUs (threads) per CTA of the step kernel.
template <class R>
__host__ __device__ constexpr int block_of() {
  return 128;
}

// Resident CTAs per SM the register allocation is bounded for: the FP32
// kernel is latency-bound and wants warps (5 x 128 threads at <= 102
// registers measured best); the FP64 kernel is bound by the FP64 pipe and
// wants registers.
template <class R>
__host__ __device__ constexpr int min_blocks() {
  return sizeof(R) == 4 ? 5 : 3;
}

// Basal values of one cell (Init kernel, cuda_Cell_Detailed.cu:1121-1174),
// computed on the host in FP64 and broadcast to every CRU of the cell.
struct InitValues {
  double cp, cs, cjsr, cjsrb, ancx, casar, casarh, casarj, casarhj;
  double ci, cnsr, catf, cats, cacal, casr, camyo, mgmyo;
  int nou, ncu, nob, ncb;
  uint32_t lcc_lo, lcc_hi;
};

template <class R>
cudaError_t launch_step(const StepArgs<R>& a, int ntiles, bool out, cudaStream_t st);

template <class R>
cudaError_t launch_init(const Lattice<R>& L, const CellConst* cells, const InitValues* iv,
                        int ncells, int max_n, cudaStream_t st);

cudaError_t launch_volt_prep(const CellConst* cells, CellDyn* dyn, int ncells, double dt,
                             cudaStream_t st);

}  // namespace rh
