// window.cu — the persistent window kernel: W time steps of every cell in one
// cooperative launch, with per-cell arrival counters, a queue of cell updates
// and bounded waits in place of the launch boundaries of step.cu.
#include <cuda_runtime.h>
#include <stdint.h>

#include "tile.cuh"

namespace rh {

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned int* p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// atomic add with acquire-release semantics at device scope: publishes this
// CTA's writes of the tile (ordered before it by the CTA barrier) and, for
// the thread that learns it arrived last, makes every other arrival's writes
// visible before it queues the cell
__device__ __forceinline__ unsigned int atom_add_acq_rel_u32(unsigned int* p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// ---- the queue of cell updates (the q_* words of WindowCtl) ----
//
// The CTA whose arrival completes a cell's step only enqueues the cell; the
// update is run by a CTA that would otherwise wait.  Had the last arriver run it, the update would make
// that CTA late, so it would again be the last arriver of every later cell it
// shares tiles with: one CTA falls ~25 us per cell behind in every sweep and
// the cells it touches become ready late (measured: 1.5 ms per step against
// 0.52 for the two-launch path, the CTAs waiting for readiness most of the
// time).  A slot is published with a sequence number, so a consumer never
// reads a cell before it is written.

// One thread: appends `cell` to the queue.
__device__ __forceinline__ void enqueue_update(const WindowCtl& w, int cell) {
  const unsigned int pos = atomicAdd(w.q_tail, 1u);
  const unsigned int slot = pos % (unsigned int)w.q_cap;
  w.q_cell[slot] = cell;
  st_release_u32(&w.q_seq[slot], pos + 1u);
}

// One thread: takes the oldest queued cell; -1 when the queue is empty, -2
// when a wait gave up.
__device__ int try_dequeue(const WindowCtl& w) {
  unsigned int h = ld_acquire_u32(w.q_head);
  const unsigned int t = ld_acquire_u32(w.q_tail);
  while (h < t) {
    const unsigned int prev = atomicCAS(w.q_head, h, h + 1u);
    if (prev == h) {  // ticket h is ours: its producer is writing the slot
      const unsigned int slot = h % (unsigned int)w.q_cap;
      for (long long it = 0; ld_acquire_u32(&w.q_seq[slot]) != h + 1u; ++it) {
        if (it >= w.wait_limit || ld_acquire_u32(w.error) != 0u) {
          atomicOr(w.error, 1u);
          return -2;
        }
        __nanosleep(32);
      }
      return __ldcg(&w.q_cell[slot]);
    }
    h = prev;
  }
  return -1;
}

// The cold paths of the window kernel out of line, so that their registers
// (the output-step statistics, the FP64 cell update) do not constrain the
// plain tile update: the lattice update of an output step, and the cell
// update with the publication of the cell's next step.  Their arguments live
// in shared memory.
template <class R, int B, bool OPT>
__device__ __noinline__ bool tile_update_output(const StepArgs<R>& a, int ti, TileHeader& sh,
                                                StepCoef<R>& sk, unsigned char* dsm) {
  return tile_update<R, true, B, OPT>(a, ti, sh, sk, dsm);
}

// One warp: the update of `cell`'s step in progress, then its publication
// (the number of the cell's completed steps, or kReadyDone).
template <class R>
__device__ __noinline__ void cell_update_publish(const StepArgs<R>& a, const WindowCtl& w,
                                                 int cell, int nw, double* scratch) {
  cell_update<R, true, true>(a, cell, nw, scratch);
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    __threadfence();
    const unsigned int next = ld_acquire_u32(&w.sync[cell].ready) + 1u;
    st_release_u32(&w.sync[cell].ready, a.dyn[cell].done ? kReadyDone : next);
  }
}

// Bounded wait of warp 0 for the cell of the CTA's next tile (window step
// `target`), running queued cell updates while it waits: returns 1 when the
// cell's previous step is published, 0 when the cell has finished its
// protocol (the tile is skipped), -1 when the wait gave up (its poll limit
// ran out, or another CTA's did): the cell then carries RH_STATUS_TIMEOUT and
// the launch returns early.
template <class R>
__device__ __noinline__ int wait_or_help(const StepArgs<R>& a, const WindowCtl& w, int cell,
                                         unsigned int target, int nw, double* scratch) {
  const int lane = threadIdx.x & 31;
  CellDyn* dyn = a.dyn + cell;
  for (long long it = 0;;) {
    int st = 0;  // 1 ready, 2 finished, 3 error
    if (lane == 0) {
      const unsigned int r = ld_acquire_u32(&w.sync[cell].ready);
      if (r >= target) st = r == kReadyDone ? 2 : 1;
      else if (__ldcg(&dyn->done)) st = 2;  // finished before the launch: publishes nothing
      else if (ld_acquire_u32(w.error) != 0u) st = 3;
    }
    st = __shfl_sync(0xffffffffu, st, 0);
    if (st == 1) return 1;
    if (st == 2) return 0;
    if (st == 3) return -1;
    int u = lane == 0 ? try_dequeue(w) : 0;
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u == -2) return -1;
    if (u >= 0) {  // another cell's update, while this one is not ready
      cell_update_publish<R>(a, w, u, nw, scratch);
      continue;
    }
    if (++it >= w.wait_limit) {
      if (lane == 0) {
        atomicOr(&dyn->status, (unsigned int)RH_STATUS_TIMEOUT);
        atomicOr(w.error, 1u);
      }
      return -1;
    }
    __nanosleep(128);
  }
}

// Warp 0 after the CTA's last tile of the launch: runs queued updates until
// the queue is empty and every cell this CTA worked on has published its
// last step (the CTAs still working on those cells need nothing more from
// this one).  False when a wait gave up.
template <class R>
__device__ __noinline__ bool drain_updates(const StepArgs<R>& a, const WindowCtl& w, int nw,
                                           double* scratch) {
  const int lane = threadIdx.x & 31;
  for (long long it = 0;;) {
    int u = lane == 0 ? try_dequeue(w) : 0;
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u == -2) return false;
    if (u >= 0) {
      cell_update_publish<R>(a, w, u, nw, scratch);
      continue;
    }
    bool pending = false;
    for (int ti = blockIdx.x + lane * gridDim.x; ti < w.ntiles; ti += 32 * gridDim.x) {
      const int c = __ldg(&a.tiles[ti].x);
      const unsigned int r = ld_acquire_u32(&w.sync[c].ready);
      if (r < (unsigned int)w.steps && !__ldcg(&a.dyn[c].done)) pending = true;
    }
    if (!__any_sync(0xffffffffu, pending)) return true;
    int err = lane == 0 ? (int)ld_acquire_u32(w.error) : 0;
    err = __shfl_sync(0xffffffffu, err, 0);
    if (++it >= w.wait_limit || err) {
      if (lane == 0) atomicOr(w.error, 1u);
      return false;
    }
    __nanosleep(256);
  }
}

// Persistent lattice + cell update of every active cell for w.steps time
// steps in one launch (all CTAs resident: a cooperative launch).  CTA k takes
// tiles k, k + G, k + 2G ... of the tile table, which is ordered by cell, so
// each CTA sweeps the cells in the same order once per step and a cell's
// tiles finish close together in every sweep.  Per tile and step:
//   1. warp 0 waits until the cell's update of the previous step is published
//      (sync[cell].ready counts the cell's completed steps), running queued
//      updates of other cells meanwhile (wait_or_help);
//   2. the CTA updates the tile (tile_update, the same code as step_kernel);
//   3. thread 0 adds one arrival for the cell; the CTA that arrives last
//      queues the cell for its whole-cell update (cell_update, the same code
//      as cell_kernel), which a waiting CTA then runs and publishes.
// Each CTA finishes every tile of step i before any tile of step i + 1, an
// update depends only on arrivals of its own step, and every waiting CTA
// runs queued updates, so the waits cannot form a cycle; every wait is
// bounded all the same.
//
// MINB is the number of resident CTAs per SM the registers are bounded for:
// the step kernel's count, or one less, which gives each thread more
// registers at the cost of fewer resident warps.
template <class R, int B, bool OPT, int MINB>
__global__ void __launch_bounds__(B, MINB) window_kernel(StepArgs<R> a, WindowCtl w) {
  __shared__ TileHeader sh;
  __shared__ StepCoef<R> sk;
  __shared__ double scratch[160];
  __shared__ StepArgs<R> s_a;  // arguments of the out-of-line cold paths
  __shared__ WindowCtl s_w;
  __shared__ int s_go[2];
  extern __shared__ __align__(16) unsigned char dsm[];
  constexpr int NW = B / 32;
  const int tid = threadIdx.x;
  if (tid == 0) {
    s_a = a;
    s_w = w;
  }
  __syncthreads();
  int k = 0;  // double-buffered flag: a slow thread may still read the previous one
  for (int i = 0; i < w.steps; ++i) {
    for (int ti = blockIdx.x; ti < w.ntiles; ti += gridDim.x, k ^= 1) {
      const int cell = __ldg(&a.tiles[ti].x);
      CellDyn* dyn = a.dyn + cell;
      if (tid < 32) {
        const int go = wait_or_help<R>(s_a, s_w, cell, (unsigned int)i + w.wait_offset, NW, scratch);
        if (tid == 0) s_go[k] = go;
      }
      __syncthreads();
      const int go = s_go[k];
      if (go < 0) return;  // no copy is in flight: the tile's staging has not begun
      if (go == 0) continue;
      const bool out = !a.no_output && __ldcg(&coef_ptr<R>(dyn)->output_step) != 0;
      const bool did = out ? tile_update_output<R, B, OPT>(s_a, ti, sh, sk, dsm)
                           : tile_update<R, false, B, OPT>(a, ti, sh, sk, dsm);
      __syncthreads();  // every warp's sums and writes of this tile are issued
      if (tid == 0 && did) {
        const unsigned int prev = atom_add_acq_rel_u32(&w.sync[cell].arrive, 1u);
        if (prev + 1u == (unsigned int)sh.tile_count) {  // every arrival of this step is in
          w.sync[cell].arrive = 0u;
          enqueue_update(w, cell);
        }
      }
    }
  }
  if (tid < 32) drain_updates<R>(s_a, s_w, NW, scratch);
}

// ------------------------------------------------------------- launchers

// The persistent kernel is compiled for tiles of 64 and 128 CRUs (the fastest
// tile lengths of the step kernel; 256-CRU tiles hold too few CTAs per SM),
// each at the step kernel's CTAs per SM and, without the build options, at
// one CTA per SM fewer.
template <class R, int B, bool OPT, int MINB>
cudaError_t window_grid_b(int* ctas) {
  int dev = 0, sms = 0, coop = 0, per = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, window_kernel<R, B, OPT, MINB>, B,
                                                      TileSmem<R, B>::kBytes);
  if (e != cudaSuccess) return e;
  if (!coop || per <= 0) return cudaErrorNotSupported;
  *ctas = per * sms;
  return cudaSuccess;
}

template <class R, int B, bool OPT, int MINB>
cudaError_t launch_window_b(const StepArgs<R>& a, const WindowCtl& w, cudaStream_t st) {
  int ctas = 0;
  cudaError_t e = window_grid_b<R, B, OPT, MINB>(&ctas);
  if (e != cudaSuccess) return e;
  if (ctas > w.ntiles) ctas = w.ntiles;
  if (ctas <= 0 || w.steps <= 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3(B);
  cfg.dynamicSmemBytes = TileSmem<R, B>::kBytes;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, window_kernel<R, B, OPT, MINB>, a, w);
}

// Dispatch on (tile, build options, fewer CTAs per SM); a non-null `grid`
// selects the query of the grid instead of the launch.
template <class R, int B>
cudaError_t window_dispatch(const StepArgs<R>* a, const WindowCtl* w, bool opt, bool fewer,
                            cudaStream_t st, int* grid) {
  constexpr int M = min_blocks_for<R, B>();
  if (opt) {
    if (fewer) return cudaErrorNotSupported;
    return grid ? window_grid_b<R, B, true, M>(grid) : launch_window_b<R, B, true, M>(*a, *w, st);
  }
  if (fewer) {
    if constexpr (M > 1)
      return grid ? window_grid_b<R, B, false, M - 1>(grid)
                  : launch_window_b<R, B, false, M - 1>(*a, *w, st);
    return cudaErrorNotSupported;
  }
  return grid ? window_grid_b<R, B, false, M>(grid) : launch_window_b<R, B, false, M>(*a, *w, st);
}

template <class R>
cudaError_t launch_window(const StepArgs<R>& a, const WindowCtl& w, bool opt, int tile,
                          bool fewer_ctas, cudaStream_t st) {
  switch (tile) {
    case 64: return window_dispatch<R, 64>(&a, &w, opt, fewer_ctas, st, nullptr);
    case 128: return window_dispatch<R, 128>(&a, &w, opt, fewer_ctas, st, nullptr);
    default: return cudaErrorNotSupported;
  }
}

template <class R>
cudaError_t window_grid(int tile, bool opt, bool fewer_ctas, int* ctas) {
  switch (tile) {
    case 64: return window_dispatch<R, 64>(nullptr, nullptr, opt, fewer_ctas, nullptr, ctas);
    case 128: return window_dispatch<R, 128>(nullptr, nullptr, opt, fewer_ctas, nullptr, ctas);
    default: return cudaErrorNotSupported;
  }
}

template cudaError_t launch_window<float>(const StepArgs<float>&, const WindowCtl&, bool, int,
                                          bool, cudaStream_t);
template cudaError_t launch_window<double>(const StepArgs<double>&, const WindowCtl&, bool, int,
                                           bool, cudaStream_t);
template cudaError_t window_grid<float>(int, bool, bool, int*);
template cudaError_t window_grid<double>(int, bool, bool, int*);

}  // namespace rh
