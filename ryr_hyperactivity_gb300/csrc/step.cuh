// step.cuh — launch interface of the step kernels (step.cu).
#pragma once

#include <cuda_runtime.h>

#include "lattice.cuh"

namespace rh {

// Tile lengths (CRUs = threads per CTA) the step kernel is compiled for; the
// autotuner (rh_autotune) picks one per simulator.
constexpr int kNumTileSizes = 3;
constexpr int kTileSizes[kNumTileSizes] = {64, 128, 256};
constexpr int kDefaultTile = 128;

// Cell groups advanced on concurrent streams when the run options leave the
// choice to the library.  Each group's step ends with its cell update, a
// chain of dependent FP64 work that leaves most SMs to the other groups; with
// 16 groups (512 cells, mixed precision) the step took 0.524 ms against
// 0.542 ms with 4 groups.
constexpr int kDefaultGroups = 8;

// Resident CTAs per SM each instantiation's register allocation is bounded
// for.  FP32: about 640 threads per SM at <= ~100 registers (measured best:
// the kernel is latency-bound and wants warps).  FP64: bound by the FP64 pipe,
// so fewer, register-rich threads.
template <class R, int B>
__host__ __device__ constexpr int min_blocks_for() {
  return sizeof(R) == 4 ? (B == 64 ? 10 : (B == 128 ? 5 : 2))
                        : (B == 64 ? 6 : (B == 128 ? 3 : 1));
}

// Basal values of one cell (Init kernel, cuda_Cell_Detailed.cu:1121-1174),
// computed on the host in FP64 and broadcast to every CRU of the cell.
struct InitValues {
  double cp, cs, cjsr, cjsrb, ancx, casar, casarh, casarj, casarhj;
  double ci, cnsr, catf, cats, cacal, casr, camyo, mgmyo;
  int nou, ncu, nob, ncb;
  uint32_t lcc_lo, lcc_hi;
};

// Synchronisation words of one cell inside a persistent window launch,
// zeroed before each launch.
struct CellSync {
  unsigned int arrive;  // tiles of the step in progress that have finished
  unsigned int ready;   // steps of this launch whose cell update is published
};
// `ready` of a cell that finished its protocol: every later wait passes and
// its tiles are skipped.
constexpr unsigned int kReadyDone = 0x7fffffffu;

// Control block of a persistent window launch (window_kernel).
struct WindowCtl {
  CellSync* sync;          // [ncells]
  unsigned int* error;     // set when a wait gave up
  int steps;               // time steps of this launch
  int ntiles;              // tiles of the tile table
  long long wait_limit;    // polls before a wait gives up
  unsigned int wait_offset;  // added to every readiness target; 0 (a test sets a
                             // target that is never published)
  // queue of cells whose step has every arrival in and awaits its update:
  // q_cap slots of (sequence number, cell), consumed in order
  unsigned int* q_head;
  unsigned int* q_tail;
  unsigned int* q_seq;
  int* q_cell;
  int q_cap;
};

// Default poll limit of a wait: about 0.3 s (a poll is an L2 round trip and a
// short sleep), far above the longest legitimate wait (a few cell updates,
// tens of microseconds).
constexpr long long kDefaultWaitLimit = 300000;

// W time steps of every cell in one persistent cooperative launch with tiles
// of `tile` CRUs (64 or 128): the grid is every CTA the device holds at once,
// at the step kernel's CTAs per SM or, with fewer_ctas (plain cells only),
// one fewer with more registers per thread.  Returns cudaErrorNotSupported
// for a combination that is not compiled or a device that cannot launch it
// cooperatively.
template <class R>
cudaError_t launch_window(const StepArgs<R>& a, const WindowCtl& w, bool opt, int tile,
                          bool fewer_ctas, cudaStream_t st);

// Resident CTAs of that persistent window kernel on this device (its grid).
template <class R>
cudaError_t window_grid(int tile, bool opt, bool fewer_ctas, int* ctas);

// One time step with tiles of `tile` CRUs (one of kTileSizes).  `opt` selects
// the kernel variant that handles the per-cell build options of the lattice
// update (perm, iso, slowncxchange, NCX form); without them a cell runs the
// plain variant.
// `staging` selects the FP32 kernels' staging (0 per-thread copies, 1 bulk
// asynchronous copies, 2 tensor copies through `maps`, built for `tile`).
template <class R>
cudaError_t launch_step(const StepArgs<R>& a, int ntiles, bool out, bool opt, int tile,
                        int staging, const StageMaps* maps, cudaStream_t st);

// The whole-cell update of cells [cell0, cell0 + ncells) after their lattice
// launch on the same stream (`tile` is the lattice launch's tile length).
template <class R>
cudaError_t launch_cells(const StepArgs<R>& a, int cell0, int ncells, bool out, int tile,
                         cudaStream_t st);

// Whether a cell's lattice update uses any build option of the `opt` variant.
inline bool cell_uses_options(const CellConst& c) {
  return c.perm || c.iso || c.slowncx || c.ncx_form != RH_NCX_ALLOSTERIC;
}

template <class R>
cudaError_t launch_init(const Lattice<R>& L, const CellConst* cells, const InitValues* iv,
                        int ncells, int max_n, cudaStream_t st);

// Per-device set-up of the step kernels (shared-memory opt-in); call with
// the device current before the first launch.
cudaError_t prepare_step_kernels();

cudaError_t launch_volt_prep(const CellConst* cells, CellDyn* dyn, int ncells, double dt,
                             cudaStream_t st);

}  // namespace rh
