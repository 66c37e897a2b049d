// step.cu — the per-time-step kernels.
//
// Two launches per cell group advance every active cell of the group by one
// time step, with no host round trip:
//   1. step_kernel: each CTA owns a tile of up to B consecutive CRUs of one cell and
//      updates them as the reference's Compute kernel does
//      (cuda_Cell_Detailed.cu:1187-1692, fixA): the tile's own ci/cnsr
//      sub-voxels are staged in shared memory so that in-tile stencil
//      neighbours (+-x always, +-y when the row above/below is in the tile)
//      come from shared memory and only the rest from L1/L2;
//   2. the CTA reduces sum(cs), sum(xicat), sum(xinaca) exactly in 128-bit
//      fixed point (fixedsum.cuh) and adds them to the cell's accumulators
//      with integer atomics; at output steps it also stores the ~30
//      statistics of :839-929 as one FP64 partial row per warp;
//   2. cell_kernel, next on the same stream: one warp per cell reads the
//      sums (and sums the output partials in a fixed order), runs the
//      membrane model and V update (:430-739, the reference's host loop),
//      writes the output record at output steps, and prepares the
//      coefficients of the next step.
#include <cuda_runtime.h>
#include <stdint.h>

#include "tile.cuh"

namespace rh {

template <class R, bool OUT>
__global__ void __launch_bounds__(32, 16) cell_kernel(StepArgs<R> a, int cell0, int nw) {
  __shared__ double scratch[160];
  cell_update<R, OUT, false>(a, cell0 + blockIdx.x, nw, scratch);
}

template <class R, bool OUT, int B, bool OPT, int STG>
__global__ void __launch_bounds__(B, min_blocks_for<R, B>())
    step_kernel(StepArgs<R> a, const __grid_constant__ StageMaps maps) {
  __shared__ TileHeader sh;
  __shared__ StepCoef<R> sk;
  // bulk staging: channel data, halo rows; tensor staging: real planes, pair planes
  __shared__ __align__(8) uint64_t bars[2];
  extern __shared__ __align__(128) unsigned char dsm[];  // tensor copies land 128-byte aligned
  allow_dependent_launch();  // the cell update may start its first part
  if (STG != 0 && threadIdx.x == 0) {  // ordered before the other threads' waits by the header barrier
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tile_update<R, OUT, B, OPT, STG>(a, blockIdx.x, sh, sk, dsm, bars, 0u, &maps);
}

// ------------------------------------------------------------- other kernels

// Fills a cell's CRUs with its basal state (values computed on the host by
// the Init rules, cuda_Cell_Detailed.cu:1108-1182).
template <class R>
__global__ void init_kernel(Lattice<R> L, const CellConst* cells, const InitValues* iv, int ncells) {
  const int cell = blockIdx.y;
  if (cell >= ncells) return;
  const CellConst& c = cells[cell];
  const InitValues& v = iv[cell];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < c.n; q += gridDim.x * blockDim.x) {
    const int64_t g = c.off + q, S = L.stride;
    L.cp[g] = R(v.cp);
    L.cs[0][g] = R(v.cs);
    L.cs[1][g] = R(v.cs);
    L.cjsr[g] = R(v.cjsr);
    L.cjsrb[g] = R(v.cjsrb);
    L.ancx[g] = R(v.ancx);
    L.casar[g] = R(v.casar);
    L.casarh[g] = R(v.casarh);
    L.casarj[g] = R(v.casarj);
    L.casarhj[g] = R(v.casarhj);
    for (int ii = 0; ii < 8; ++ii) {
      const int64_t gi = sub_index(ii, g, S);
      L.ci[0][gi] = R(v.ci);
      L.ci[1][gi] = R(v.ci);
      L.cnsr[0][gi] = R(v.cnsr);
      L.cnsr[1][gi] = R(v.cnsr);
      L.catf[gi] = R(v.catf);
      L.cats[gi] = R(v.cats);
      L.cacal[gi] = R(v.cacal);
      L.casr[gi] = R(v.casr);
      L.camyo[gi] = R(v.camyo);
      L.mgmyo[gi] = R(v.mgmyo);
    }
    L.ryr[g] = (uint32_t)v.nou | ((uint32_t)v.ncu << 8) | ((uint32_t)v.nob << 16) |
               ((uint32_t)v.ncb << 24);
    uint2 lcc = make_uint2(v.lcc_lo, v.lcc_hi);
    if (c.randomlcc) {  // 0..8 channels: curand() % 9 at initialisation (:1150-1151)
      const int x = q % c.lx, y = (q / c.lx) % c.ly, z = q / (c.lx * c.ly);
      const uint32_t pos = (uint32_t)((x + 1) + c.nxf * ((y + 1) + c.nyf * (z + 1)));
      rh_stream rng;
      rh_stream_init(&rng, c.seed, c.cell_id, pos, RH_PHILOX_INIT_STEP);
      const uint32_t nlcc = rh_uniform_u32(&rng) % 9u;
      uint64_t slots = 0;
      for (uint32_t ll = 0; ll < 8; ++ll) slots |= (uint64_t)(ll < nlcc ? 3u : 16u) << (8 * ll);
      lcc = make_uint2((uint32_t)slots, (uint32_t)(slots >> 32));
    }
    L.lcc[g] = lcc;
    L.win[g] = 0;
  }
}

// Coefficients of the next lattice update from the current membrane state
// (after create or a host-side membrane change).
__global__ void coef_prep_kernel(const CellConst* cells, CellDyn* dyn, int ncells, double dt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  StepCoef<double> kd;
  bool active = step_coef(kd, dyn[c].m, cells[c], dt);
  StepCoef<float> kf;
  convert_coef(kf, kd);
  dyn[c].cd = kd;
  dyn[c].cf = kf;
  if (!active) {
    dyn[c].done = 1;
    dyn[c].status |= RH_STATUS_DONE;
  } else {
    dyn[c].done = 0;
    dyn[c].status &= ~RH_STATUS_DONE;
  }
}

// ------------------------------------------------------------- launchers

// Instantiations whose tile needs more than the default 48 KB of dynamic
// shared memory opt in once per device (before any launch or capture).
template <class R, int B, int STG>
cudaError_t opt_in_smem() {
  constexpr size_t smem = STG == 1 ? TileSmem<R, B>::kBytesBulk : TileSmem<R, B>::kBytes;
  if (smem <= 48 * 1024) return cudaSuccess;
  const cudaFuncAttribute attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(step_kernel<R, true, B, false, STG>, attr, (int)smem))) return e;
  if ((e = cudaFuncSetAttribute(step_kernel<R, false, B, false, STG>, attr, (int)smem))) return e;
  if ((e = cudaFuncSetAttribute(step_kernel<R, true, B, true, STG>, attr, (int)smem))) return e;
  return cudaFuncSetAttribute(step_kernel<R, false, B, true, STG>, attr, (int)smem);
}

template <int B>
cudaError_t opt_in_smem_f32() {
  cudaError_t e;
  if ((e = opt_in_smem<float, B, 0>()) != cudaSuccess) return e;
  if ((e = opt_in_smem<float, B, 1>()) != cudaSuccess) return e;
  return opt_in_smem<float, B, 2>();
}

cudaError_t prepare_step_kernels() {
  cudaError_t e;
  if ((e = opt_in_smem_f32<64>()) != cudaSuccess) return e;
  if ((e = opt_in_smem_f32<128>()) != cudaSuccess) return e;
  if ((e = opt_in_smem_f32<256>()) != cudaSuccess) return e;
  if ((e = opt_in_smem<double, 64, 0>()) != cudaSuccess) return e;
  if ((e = opt_in_smem<double, 128, 0>()) != cudaSuccess) return e;
  return opt_in_smem<double, 256, 0>();
}

template <class R, int B, int STG>
void launch_bb(const StepArgs<R>& a, const StageMaps& maps, int ntiles, bool out, bool opt,
               cudaStream_t st) {
  constexpr size_t smem = STG == 1 ? TileSmem<R, B>::kBytesBulk : TileSmem<R, B>::kBytes;
  if (opt) {
    if (out) step_kernel<R, true, B, true, STG><<<ntiles, B, smem, st>>>(a, maps);
    else step_kernel<R, false, B, true, STG><<<ntiles, B, smem, st>>>(a, maps);
  } else {
    if (out) step_kernel<R, true, B, false, STG><<<ntiles, B, smem, st>>>(a, maps);
    else step_kernel<R, false, B, false, STG><<<ntiles, B, smem, st>>>(a, maps);
  }
}

// Bulk and tensor staging are compiled for the FP32 lattice only (the FP64
// kernels read global memory directly).
template <class R, int B>
void launch_b(const StepArgs<R>& a, const StageMaps& maps, int ntiles, bool out, bool opt,
              int staging, cudaStream_t st) {
  if constexpr (sizeof(R) == 4) {
    if (staging == 1) {
      launch_bb<R, B, 1>(a, maps, ntiles, out, opt, st);
      return;
    }
    if (staging == 2) {
      launch_bb<R, B, 2>(a, maps, ntiles, out, opt, st);
      return;
    }
  }
  launch_bb<R, B, 0>(a, maps, ntiles, out, opt, st);
}

template <class R>
cudaError_t launch_step(const StepArgs<R>& a, int ntiles, bool out, bool opt, int tile,
                        int staging, const StageMaps* maps, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  if (staging == 2 && !maps) return cudaErrorInvalidValue;
  static const StageMaps kNoMaps{};
  const StageMaps& m = maps ? *maps : kNoMaps;
  switch (tile) {
    case 64: launch_b<R, 64>(a, m, ntiles, out, opt, staging, st); break;
    case 128: launch_b<R, 128>(a, m, ntiles, out, opt, staging, st); break;
    case 256: launch_b<R, 256>(a, m, ntiles, out, opt, staging, st); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_cells(const StepArgs<R>& a, int cell0, int ncells, bool out, int tile,
                         cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ncells);
  cfg.blockDim = dim3(32);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  // Programmatic serialization after the lattice launch, and the device's
  // highest launch priority: when lattice CTAs of the other groups are also
  // waiting for an SM, the cell warps go first.  Inside a captured window
  // the priority holds because the window's graph is instantiated with
  // per-node priorities.
  int prio_low = 0, prio_high = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
  if (e != cudaSuccess) return e;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  at[1].id = cudaLaunchAttributePriority;
  at[1].val.priority = prio_high;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  const int nw = tile / 32;
  if (out) return cudaLaunchKernelEx(&cfg, cell_kernel<R, true>, a, cell0, nw);
  return cudaLaunchKernelEx(&cfg, cell_kernel<R, false>, a, cell0, nw);
}

template <class R>
cudaError_t launch_init(const Lattice<R>& L, const CellConst* cells, const InitValues* iv,
                        int ncells, int max_n, cudaStream_t st) {
  dim3 grid((max_n + 255) / 256, ncells);
  if (grid.x > 1024) grid.x = 1024;
  init_kernel<R><<<grid, 256, 0, st>>>(L, cells, iv, ncells);
  return cudaGetLastError();
}

cudaError_t launch_volt_prep(const CellConst* cells, CellDyn* dyn, int ncells, double dt,
                             cudaStream_t st) {
  coef_prep_kernel<<<(ncells + 127) / 128, 128, 0, st>>>(cells, dyn, ncells, dt);
  return cudaGetLastError();
}

template cudaError_t launch_step<double>(const StepArgs<double>&, int, bool, bool, int, int,
                                         const StageMaps*, cudaStream_t);
template cudaError_t launch_step<float>(const StepArgs<float>&, int, bool, bool, int, int,
                                        const StageMaps*, cudaStream_t);
template cudaError_t launch_cells<double>(const StepArgs<double>&, int, int, bool, int,
                                          cudaStream_t);
template cudaError_t launch_cells<float>(const StepArgs<float>&, int, int, bool, int,
                                         cudaStream_t);
template cudaError_t launch_init<double>(const Lattice<double>&, const CellConst*,
                                         const InitValues*, int, int, cudaStream_t);
template cudaError_t launch_init<float>(const Lattice<float>&, const CellConst*,
                                        const InitValues*, int, int, cudaStream_t);

}  // namespace rh
