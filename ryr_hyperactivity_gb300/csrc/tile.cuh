// tile.cuh — device code of one time step shared by the kernels of step.cu
// (one launch per step and cell group) and window.cu (the persistent window
// kernel): the lattice update of one tile of CRUs (tile_update) and the
// whole-cell update of one cell by one warp (cell_update).
//
// A lattice update of a cell is the reference's Compute kernel
// (cuda_Cell_Detailed.cu:1187-1692, fixA) over the cell's tiles; a cell update
// is the reference's host loop between two launches (:430-739): the exact
// whole-cell sums, the membrane model and V, the output record, and the
// coefficients of the next step.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "cellmodel.cuh"
#include "cellwarp.cuh"
#include "fixedsum.cuh"
#include "lattice.cuh"
#include "model.cuh"
#include "step.cuh"
#include "async_copy.cuh"

namespace rh {

// ---------------------------------------------------------------- reductions

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}

// ------------------------------------------------------- launch ordering

// Programmatic dependent launch: the cell update of a group is launched with
// programmatic stream serialization after the group's lattice launch, so its
// CTAs may start once every lattice CTA has started (each signals at entry).
// It does the part of the membrane step that needs only the previous step's
// state, then waits in griddepcontrol.wait until the lattice launch has
// completed and its memory is visible.  Without the launch attribute the wait
// returns at once.
__device__ __forceinline__ void allow_dependent_launch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void wait_for_prerequisite_grid() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ------------------------------------------------------------ cell update

// Whole-cell part of the step for cells [cell0, cell0 + gridDim.x): one warp
// per cell, launched on the group's stream right after the group's lattice
// launch.  Before the wait it reads only what the previous step's cell
// update wrote (that launch completed before the lattice launch began): the
// membrane state, the flags of the step just taken, the cell constants.
// After the wait: the exact lattice sums, the output partials, the status
// bits the lattice CTAs set.  Then V and [Na]i (:430-739, the reference's
// host loop), the coefficients of the next step, the output record and the
// per-beat statistics.  A separate launch keeps this FP64 work (tens of
// microseconds of dependent FP64 latency on this GPU) out of the lattice
// CTAs; at <= 128 registers a cell warp fits beside five lattice CTAs.
// `nw` is the number of warps per lattice tile (the rows of output partials
// each tile wrote).
//
// The same update runs inside the persistent window kernel (PERSIST), by one
// warp of a CTA that takes the cell's update from the queue: there is no
// prior launch to wait for, the output step is the cell's own flag (OUT =
// true reads it), and a device-scope fence first makes the cell's state,
// written by other CTAs during the launch, visible to the warp's loads.
template <class R, bool OUT, bool PERSIST>
__device__ __forceinline__ void cell_update(const StepArgs<R>& a, int cell, int nw,
                                            double* scratch) {
  const int lane = threadIdx.x & 31;
  CellDyn* dyn = a.dyn + cell;
  if (PERSIST) __threadfence();
  if (dyn->done) return;  // its lattice CTAs returned at once as well
  // the flags of the step just taken, read before the update replaces them
  const StepCoef<R>* kc = coef_ptr<R>(dyn);
  const bool out_step = OUT && kc->output_step && !a.lattice_only && !a.no_output;
  const bool cadist = out_step && kc->cadist_step && a.out_cd != nullptr;
  const CellConst& cc = a.cells[cell];
  const double dt = a.dt;
  rh_membrane m = dyn->m;
  MembranePre pre;
  double fm[6];
  if (!a.lattice_only) membrane_pre_warp(m, dt, cc, scratch, fm, pre);

  if (!PERSIST) wait_for_prerequisite_grid();

  if (!a.lattice_only) {
    const double* P = a.partials;
    // output-step partials: one row per warp of each of the cell's tiles
    const int t0 = cc.tile_begin * nw, nt = cc.tile_count * nw;
    // the step's exact whole-cell sums, accumulated by the cell's CTAs
    double tot[3];
#pragma unroll
    for (int q = 0; q < 3; ++q)
      tot[q] = fx_to_double(__ldcg(&dyn->acc[2 * q]), __ldcg(&dyn->acc[2 * q + 1]));
    double osum[NOUT];
    if (out_step) {
      for (int q = 0; q < NOUT; ++q) {
        double s = 0.0;
        for (int tl = lane; tl < nt; tl += 32)
          s += __ldcg(P + (size_t)(t0 + tl) * P_COUNT + P_STEP_END + q);
        osum[q] = warp_sum(s);
      }
      // the ci > 1000 flag is a max, not a sum
      double f = 0.0;
      for (int tl = lane; tl < nt; tl += 32)
        f = fmax(f, __ldcg(P + (size_t)(t0 + tl) * P_COUNT + O_CIHIGH));
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) f = fmax(f, __shfl_down_sync(0xffffffffu, f, off));
      osum[O_CIHIGH - P_STEP_END] = f;
    }
    // reduction quotients, [Na]i and V (:447-456, :701-738)
    membrane_post_warp(m, dt, cc, tot, scratch, pre);
    uint32_t status = __ldcg(&dyn->status);
    if (!isfinite(m.v) || !isfinite(m.xnai) || !isfinite(m.csubt) || !isfinite(m.xicatto) ||
        !isfinite(m.xinacato))
      status |= RH_STATUS_NAN;
    const double t_step = m.t;  // the time the output record and statistics carry
    m.t = m.t + dt;             // :1083
    m.step += 1;
    // coefficients of the next lattice update: FP64 for the FP64 lattice
    // (the qks update in spare slots of its rounds), FP32 for the FP32
    // lattice (the qks update in one FP64 division beside it)
    StepCoef<double> kd;
    StepCoef<float> kf;
    bool active;
    if constexpr (sizeof(R) == 8) {
      QksStep qs{m.csubt, m.qks, pre.qks_num, pre.tauqks, 0.0};
      active = step_coef_warp(kd, m, cc, dt, fm + 1, scratch, &qs);
      m.qks = m.qks + qs.dqks;
    } else {
      const double dqks = qks_increment_warp(m.csubt, m.qks, pre.qks_num, pre.tauqks, dt, scratch);
      active = step_coef_warp_f32(kf, m, cc, dt, fm + 1, pre);
      m.qks = m.qks + dqks;
    }
    if (lane == 0) {
      if (a.stats) {  // per-beat detectors on the (t, V) sample of this step
        rh_beat_stats rec;
        if (beat_on_step(dyn->bt, t_step, m.v, cc.pcl, &rec)) {
          a.stats[(size_t)cell * a.stats_cap + dyn->stats_count % a.stats_cap] = rec;
          dyn->stats_count += 1;
        }
      }
      if (out_step) {
        m.sparksum += (long long)osum[O_SPARK - P_STEP_END];
        if (osum[O_CIHIGH - P_STEP_END] > 0) status |= RH_STATUS_CI_HIGH;
        long long slot = dyn->out_count % a.out_cap;
        double* w = a.out_wc + ((size_t)cell * a.out_cap + slot) * RH_WHOLECELL_COLS;
        const double t_next = m.t;
        m.t = t_step;
        wholecell_columns(w, osum, m, cc.n, dt);
        m.t = t_next;
        if (cadist) {  // record header: t and V of this output step (:1005)
          double* h = a.out_cd + cc.cd_off + (dyn->cd_count % a.cd_cap) * (2 + 6 * (long long)cc.n);
          h[0] = t_step;
          h[1] = m.v;
          dyn->cd_count += 1;
        }
        if (a.stats) beat_on_output(dyn->bt, w);
        dyn->out_count += 1;
        m.sparksum = 0;  // :1074-1077
        m.out_ica = 0;
        m.out_ncx = 0;
        m.out_ina = 0;
      }
      if (!active) {
        dyn->done = 1;
        status |= RH_STATUS_DONE;
      }
      dyn->m = m;
      if constexpr (sizeof(R) == 8) {
        dyn->cd = kd;
      } else {
        dyn->cf = kf;
      }
      dyn->status = status;
    }
  }
  __syncwarp();
  if (lane < 6) dyn->acc[lane] = 0ull;  // the next step starts from zero
  if (lane == 0) dyn->parity ^= 1;
}

// ------------------------------------------------------------- step kernel

// Dynamic shared memory of one CTA (tile of B CRUs).  Always the z-pair
// planes of ci and cnsr, which the stencil reads from neighbouring threads.
// FP32 kernels also stage, with asynchronous copies issued at the top of the
// kernel, the tile's per-CRU scalars and integers (their copies overlap the
// cell-header load) and the stencil halo (the neighbours of the tile's CRUs
// along y and z, and one CRU at each end along x), so the sub-voxel loop
// reads no neighbour from global memory.  The FP64 kernels are bound by the
// FP64 pipe, not by memory latency, and read global memory directly.
template <class R, int B>
struct TileSmem {
  using V = typename Vec2<R>::T;
  static constexpr bool kStage = sizeof(R) == 4;
  // The six cytosolic buffer fields (half of the state) are read straight
  // from global memory inside the sub-voxel loop: staging them as well costs
  // more in resident CTAs than it saves in latency.
  static constexpr size_t kPlane = sizeof(V) * B;     // one pair plane
  static constexpr size_t kCi = 0;                     // V[4][B]
  static constexpr size_t kCn = 4 * kPlane;            // V[4][B]
  static constexpr size_t kCs = 8 * kPlane;            // R[B]: cs
  // FP32 kernels stage the per-CRU scalars and integers (8 + 3 fields) too
  static constexpr size_t kSc = kCs + sizeof(R) * B;        // R[8][B]: cp cjsr cjsrb ancx casar casarh casarj casarhj
  static constexpr size_t kLcc = kSc + (kStage ? 8 : 0) * sizeof(R) * B;  // uint2[B]
  static constexpr size_t kRyr = kLcc + (kStage ? 8 : 0) * B;             // u32[B]
  static constexpr size_t kWin = kRyr + (kStage ? 4 : 0) * B;             // u32[B]
  // stencil halo of the tile (ci, cnsr; cs along z):
  //   y: V[dir][j][field][B], dir 1 = +lx (pairs 0, 2), dir 0 = -lx (pairs 1, 3)
  //   z: R[dir][pair][field][B], the pair half that faces the tile: the lower
  //      sub-voxel of the CRU above (dir 1), the upper one of the CRU below
  //   x: V[side][pair][field], side 0 = the CRU before the tile, 1 = after it
  static constexpr size_t kHy = kWin + (kStage ? 4 : 0) * B;
  static constexpr size_t kHz = kHy + 8 * kPlane;
  static constexpr size_t kHcs = kHz + 16 * sizeof(R) * B;  // R[dir][B]
  static constexpr size_t kHx = kHcs + 2 * sizeof(R) * B;  // V[2][4][2]
  static constexpr size_t kBytes = kStage ? kHx + 16 * sizeof(V) : 8 * kPlane;
  // The bulk-copy staging (BULK, FP32 only) keeps the tile's own planes,
  // scalars and integers at the offsets above and moves the halo as whole
  // rows: each of the y and z halo planes holds B + 2 pairs (the row may
  // start one pair before a 16-byte boundary), the cs rows of the z
  // neighbours B + 4 values.
  static constexpr size_t kRowV = sizeof(V) * (B + 2);
  static constexpr size_t kRowR = sizeof(R) * (B + 4);
  static constexpr size_t kHyB = kWin + 4 * B;
  static constexpr size_t kHzB = kHyB + 8 * kRowV;   // V[dir][pair plane][field][B + 2]
  static constexpr size_t kHcsB = kHzB + 16 * kRowV;  // R[dir][B + 4]
  static constexpr size_t kHxB = kHcsB + 2 * kRowR;   // V[2][4][2]
  static constexpr size_t kBytesBulk = kHxB + 16 * sizeof(V);
  static_assert(kRowV % 16 == 0 && kRowR % 16 == 0 && kHyB % 16 == 0, "bulk rows 16-byte aligned");
};

// ---- bulk asynchronous copies (the tensor-memory-access engine's linear
//      mode) into shared memory, completing on an mbarrier ----

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// Bounded wait for the phase with parity `parity`; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// Elements [first, first + n) of a row of `len` elements of `esz` bytes into
// dst (dst[0] <- element first); only the part inside [0, len) moves (the
// rest is never read).  first, n and len are multiples of 16 / esz, the row
// and dst 16-byte aligned, so every copy starts and ends on a 16-byte
// boundary.
__device__ __forceinline__ void bulk_row(void* dst, const void* row, long long first, int n,
                                         int esz, long long len, uint64_t* bar) {
  const long long lo = first > 0 ? first : 0;
  const long long hi = first + n < len ? first + n : len;
  if (hi <= lo) return;
  const uint32_t bytes = (uint32_t)((hi - lo) * esz);
  mbar_expect_tx(bar, bytes);
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(static_cast<char*>(dst) + (lo - first) * esz)),
      "l"(static_cast<const char*>(row) + lo * esz), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// One 2-D tile of a tensor into shared memory (dst 128-byte aligned), its
// bytes counted on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

struct TileHeader {
  int lx, ly, lz, nxf, nyf, tile_count, line_y, line_z;
  uint32_t seed, cell_id;
  long long off, ls_off, step, slot, cd_off, cd_slot;
  int n;
  double t;
  int parity, done;
};

// The lattice update of tile `ti` of the tile table: staging, the channel
// and sub-voxel parts of every CRU, and the per-warp sums into the cell's
// accumulators (no CTA barrier at the end).  `sh`, `sk` and `dsm` are the
// CTA's shared memory; the caller separates two calls by a CTA barrier.
// Returns false, with no work done, when the cell has finished its protocol.
// Per-cell state is read through L2 (__ldcg): inside the persistent window
// kernel other CTAs write it during the launch.
//
// STG selects the staging of the FP32 kernels (the FP64 kernels stage only
// their own pair planes, with plain loads):
//   0: every thread issues cp.async copies of its share of the tile's own
//      data and of its CRU's halo;
//   1: warp 0 issues bulk asynchronous copies (the TMA engine's linear mode)
//      into two mbarriers (`bars`, one arrival each, phase `phase`): the
//      tile's own planes, scalars, integers and the cs of its z neighbours,
//      then the y and z halo rows;
//   2: thread 0 issues 2-D tensor copies (cp.async.bulk.tensor, `maps`) of the
//      tile's eight per-CRU real planes (bars[0], before the cell header
//      arrives) and of its ci and cnsr pair planes (bars[1]); the integers,
//      cs and the halo stay per-thread copies as in 0.
template <class R, bool OUT, int B, bool OPT, int STG = 0>
__device__ __forceinline__ bool tile_update(const StepArgs<R>& a, int ti, TileHeader& sh,
                                            StepCoef<R>& sk, unsigned char* dsm,
                                            uint64_t* bars = nullptr, uint32_t phase = 0,
                                            const StageMaps* maps = nullptr) {
  constexpr int kBlock = B;
  using TS = TileSmem<R, B>;
  constexpr bool kStage = TS::kStage;
  constexpr bool BULK = STG == 1, TMA = STG == 2;
  static_assert(STG == 0 || kStage, "bulk and tensor staging are the FP32 staging");
  using V = typename Vec2<R>::T;
  V(*s_ci2)[kBlock] = reinterpret_cast<V(*)[kBlock]>(dsm + TS::kCi);
  V(*s_cn2)[kBlock] = reinterpret_cast<V(*)[kBlock]>(dsm + TS::kCn);
  R(*s_sc)[kBlock] = reinterpret_cast<R(*)[kBlock]>(dsm + TS::kSc);
  R* s_cs = reinterpret_cast<R*>(dsm + TS::kCs);
  constexpr bool kSS = kStage;  // per-CRU scalars and integers staged
  uint2* s_lcc = reinterpret_cast<uint2*>(dsm + TS::kLcc);
  uint32_t* s_ryr = reinterpret_cast<uint32_t*>(dsm + TS::kRyr);
  uint32_t* s_win = reinterpret_cast<uint32_t*>(dsm + TS::kWin);
  V(*s_hy)[2][2][kBlock] = reinterpret_cast<V(*)[2][2][kBlock]>(dsm + TS::kHy);
  R(*s_hz)[4][2][kBlock] = reinterpret_cast<R(*)[4][2][kBlock]>(dsm + TS::kHz);
  R(*s_hcs)[kBlock] = reinterpret_cast<R(*)[kBlock]>(dsm + TS::kHcs);
  V(*s_hx)[4][2] = reinterpret_cast<V(*)[4][2]>(dsm + TS::kHx);

  const int4 tile = a.tiles[ti];
  const int cell = tile.x;
  const int tid = threadIdx.x;
  const int cpad = (tile.z + 31) & ~31;  // cells are padded to 32 CRUs
  // Arena indices are 32-bit: the arena holds fewer than 2^29 CRUs (checked at
  // creation), so every element index, 8 sub-voxels per CRU included, is
  // below 2^32 and each address is one 32x64 multiply-add.
  const uint32_t gt0 = (uint32_t)tile.w;  // arena index of the tile's first CRU
  if (kStage && !BULK) {
    // Fields updated in place do not depend on the ping-pong parity, so
    // their copies start before the cell header arrives.  16-byte chunks:
    // a pair plane holds 2 CRUs per chunk, a 4-byte plane 4.
    const Lattice<R>& L = a.L;
    constexpr int kTpp = kBlock / 2;  // threads per pair plane
    const int c2 = tid % kTpp, h2 = tid / kTpp;
    if (kSS && h2 == 0 && 2 * c2 < cpad) cp_async16(&s_lcc[2 * c2], L.lcc + gt0 + 2 * c2);
    constexpr int kTpq = kBlock / 4;  // threads per 4-byte plane
    const int c4 = tid % kTpq, h4 = tid / kTpq;
    if (TMA && tid == 0) {  // the eight real planes as one tensor tile
      mbar_expect_tx(&bars[0], 8u * kBlock * sizeof(R));
      tma_load_2d(&s_sc[0][0], &maps->sc, (int)gt0, 0, &bars[0]);
      mbar_arrive(&bars[0]);
    }
    if (kSS && 4 * c4 < cpad) {
#pragma unroll
      for (int f = TMA ? 8 : 0; f < 10; ++f) {  // cp cjsr cjsrb ancx casar casarh casarj casarhj ryr win
        if ((f & 3) != h4) continue;
        const void* src = f == 0 ? (const void*)(L.cp + gt0) : f == 1 ? (const void*)(L.cjsr + gt0)
                        : f == 2 ? (const void*)(L.cjsrb + gt0) : f == 3 ? (const void*)(L.ancx + gt0)
                        : f == 4 ? (const void*)(L.casar + gt0) : f == 5 ? (const void*)(L.casarh + gt0)
                        : f == 6 ? (const void*)(L.casarj + gt0) : f == 7 ? (const void*)(L.casarhj + gt0)
                        : f == 8 ? (const void*)(L.ryr + gt0) : (const void*)(L.win + gt0);
        void* dst = f < 8 ? (void*)&s_sc[f][4 * c4] : f == 8 ? (void*)&s_ryr[4 * c4] : (void*)&s_win[4 * c4];
        cp_async16(dst, static_cast<const char*>(src) + 16 * c4);
      }
    }
  }
  {
    const CellDyn* d = a.dyn + cell;
    const int* src = reinterpret_cast<const int*>(coef_ptr<R>(d));
    int* dst = reinterpret_cast<int*>(&sk);
    for (int w = tid; w < (int)(sizeof(StepCoef<R>) / 4); w += blockDim.x) dst[w] = __ldcg(src + w);
    if (tid == 0) {
      const CellConst& c = a.cells[cell];
      sh.lx = c.lx;
      sh.ly = c.ly;
      sh.lz = c.lz;
      sh.nxf = c.nxf;
      sh.nyf = c.nyf;
      sh.tile_count = c.tile_count;
      sh.line_y = c.line_y;
      sh.line_z = c.line_z;
      sh.seed = c.seed;
      sh.cell_id = c.cell_id;
      sh.off = c.off;
      sh.ls_off = c.ls_off;
      sh.step = __ldcg(&d->m.step);
      sh.t = __ldcg(&d->m.t);
      sh.slot = __ldcg(&d->out_count) % a.out_cap;
      sh.n = c.n;
      sh.cd_off = c.cd_off;
      sh.cd_slot = a.out_cd ? __ldcg(&d->cd_count) % a.cd_cap : 0;
      sh.parity = __ldcg(&d->parity);
      sh.done = __ldcg(&d->done);
    }
  }
  __syncthreads();
  if (sh.done) {
    if (kStage) cp_async_wait_all();  // no copy may still target this CTA's shared memory
    if (TMA) mbar_wait(&bars[0], phase);
    return false;
  }

  const bool out_step = OUT && sk.output_step && !a.lattice_only && !a.no_output;
  const bool cadist_step = out_step && sk.cadist_step && a.out_cd != nullptr;
  const Lattice<R>& L = a.L;
  const uint32_t S = (uint32_t)L.stride;
  const int lx = sh.lx, ly = sh.ly, lz = sh.lz;
  const int lxly = lx * ly;
  const int count = tile.z;
  const int q = tile.y + tid;
  const bool valid = tid < count;
  const int par = sh.parity;
  const uint32_t g = (uint32_t)(sh.off + q);
  const V* ci2 = reinterpret_cast<const V*>(L.ci[par]);
  const V* cn2 = reinterpret_cast<const V*>(L.cnsr[par]);

  // ---- bulk staging: warp 0 issues whole rows ----
  // halo row offsets: a row starts at the 16-byte boundary at or before the
  // first neighbour, `o*` elements before it (gt0 is a multiple of 32)
  const int oy = lx & 1, oz = lxly & 1, ocp = lxly & 3, ocm = (4 - (lxly & 3)) & 3;
  V(*b_hy)[2][2][kBlock + 2] = reinterpret_cast<V(*)[2][2][kBlock + 2]>(dsm + TS::kHyB);
  V(*b_hz)[4][2][kBlock + 2] = reinterpret_cast<V(*)[4][2][kBlock + 2]>(dsm + TS::kHzB);
  R(*b_hcs)[kBlock + 4] = reinterpret_cast<R(*)[kBlock + 4]>(dsm + TS::kHcsB);
  V(*b_hx)[4][2] = reinterpret_cast<V(*)[4][2]>(dsm + TS::kHxB);
  if constexpr (BULK) {
    const int lane = tid & 31;
    if (tid < 32) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // after the last tile's reads
      const long long S64 = (long long)S, g0 = (long long)gt0;
      // group 1 (bars[0]): what the channel part reads
      if (lane < 8) {  // own pair planes: ci, cnsr x 4
        const V* f = (lane >> 2) ? cn2 : ci2;
        const int pl = lane & 3;
        V(*dst)[kBlock] = (lane >> 2) ? s_cn2 : s_ci2;
        bulk_row(dst[pl], f + pl * S64, g0, cpad, 8, S64, &bars[0]);
      } else if (lane < 16) {  // cp cjsr cjsrb ancx casar casarh casarj casarhj
        const int k = lane - 8;
        const R* f = k == 0 ? L.cp : k == 1 ? L.cjsr : k == 2 ? L.cjsrb : k == 3 ? L.ancx
                   : k == 4 ? L.casar : k == 5 ? L.casarh : k == 6 ? L.casarj : L.casarhj;
        bulk_row(s_sc[k], f, g0, cpad, 4, S64, &bars[0]);
      } else if (lane == 16) {
        bulk_row(s_cs, L.cs[par], g0, cpad, 4, S64, &bars[0]);
      } else if (lane == 17) {
        bulk_row(s_lcc, L.lcc, g0, cpad, 8, S64, &bars[0]);
      } else if (lane == 18) {
        bulk_row(s_ryr, L.ryr, g0, cpad, 4, S64, &bars[0]);
      } else if (lane == 19) {
        bulk_row(s_win, L.win, g0, cpad, 4, S64, &bars[0]);
      } else if (lane == 20) {  // cs of the CRUs above (+z)
        bulk_row(b_hcs[1], L.cs[par], g0 + lxly - ocp, (count + ocp + 3) & ~3, 4, S64, &bars[0]);
      } else if (lane == 21) {  // and below (-z)
        bulk_row(b_hcs[0], L.cs[par], g0 - lxly - ocm, (count + ocm + 3) & ~3, 4, S64, &bars[0]);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&bars[0]);
      // group 2 (bars[1]): the y and z halo rows of ci and cnsr
      if (lane < 8) {  // y: dir 1 (+lx) planes 0, 2; dir 0 (-lx) planes 1, 3
        const int dir = lane >> 2, j = (lane >> 1) & 1, fld = lane & 1;
        const int pl = dir ? 2 * j : 2 * j + 1;
        const V* f = (fld ? cn2 : ci2) + pl * S64;
        const long long first = g0 + (dir ? lx : -lx) - oy;
        bulk_row(b_hy[dir][j][fld], f, first, (count + oy + 1) & ~1, 8, S64, &bars[1]);
      } else if (lane < 24) {  // z: whole pairs of the CRUs above (dir 1) and below (dir 0)
        const int k = lane - 8, dir = k >> 3, pl = (k >> 1) & 3, fld = k & 1;
        const V* f = (fld ? cn2 : ci2) + pl * S64;
        const long long first = g0 + (dir ? lxly : -lxly) - oz;
        bulk_row(b_hz[dir][pl][fld], f, first, (count + oz + 1) & ~1, 8, S64, &bars[1]);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&bars[1]);
    }
    // the x halo: one CRU before and one after the tile (two threads)
    if (valid) {
      const int hx = q % lx;
#pragma unroll
      for (int f = 0; f < 2; ++f) {
        const V* src = f ? cn2 : ci2;
#pragma unroll
        for (int pl = 0; pl < 4; ++pl) {
          if (tid == 0 && hx > 0) cp_async8(&b_hx[0][pl][f], src + pl * S + g - 1);
          if (tid == count - 1 && hx + 1 < lx) cp_async8(&b_hx[1][pl][f], src + pl * S + g + 1);
        }
      }
    }
    cp_async_commit();
    if (!mbar_wait(&bars[0], phase)) atomicOr(&a.dyn[cell].status, (unsigned int)RH_STATUS_TIMEOUT);
  }

  // ---- stage the tile's own sub-voxels (z-pairs) ----
  if (kStage && !BULK) {
    constexpr int kTpp = kBlock / 2;
    const int c2 = tid % kTpp, h2 = tid / kTpp;
    if (TMA && tid == 0) {  // ci and cnsr of this parity: one tensor tile each
      mbar_expect_tx(&bars[1], 2u * 4u * kBlock * sizeof(V));
      tma_load_2d(&s_ci2[0][0], &maps->plane[par], (int)gt0, 0, &bars[1]);
      tma_load_2d(&s_cn2[0][0], &maps->plane[2 + par], (int)gt0, 0, &bars[1]);
      mbar_arrive(&bars[1]);
    }
    if (!TMA && 2 * c2 < cpad) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {  // ci and cnsr, 4 pair planes each
        const int pl = 2 * (k & 1) + h2;
        const V* src = (k >> 1) ? cn2 : ci2;
        V(*dst)[kBlock] = (k >> 1) ? s_cn2 : s_ci2;
        cp_async16(&dst[pl][2 * c2], src + pl * S + gt0 + 2 * c2);
      }
    }
    if (4 * tid < cpad) cp_async16(&s_cs[4 * tid], L.cs[par] + gt0 + 4 * tid);
    const int hx = q % lx, hy = (q / lx) % ly, hz = q / lxly;
    if (valid) {  // cs of the z-neighbours (the sub-steps need it first)
      const R* csp = L.cs[par];
      if (hz + 1 < lz) cp_async4(&s_hcs[1][tid], csp + g + lxly);
      if (hz > 0) cp_async4(&s_hcs[0][tid], csp + g - lxly);
    }
    cp_async_commit();  // group 1: everything the channel part reads
    if (valid) {  // the stencil halo: each thread fetches its own CRU's outer neighbours
#pragma unroll
      for (int f = 0; f < 2; ++f) {
        const V* src = f ? cn2 : ci2;
        if (hy + 1 < ly) {
          cp_async8(&s_hy[1][0][f][tid], src + g + lx);
          cp_async8(&s_hy[1][1][f][tid], src + 2 * S + g + lx);
        }
        if (hy > 0) {
          cp_async8(&s_hy[0][0][f][tid], src + S + g - lx);
          cp_async8(&s_hy[0][1][f][tid], src + 3 * S + g - lx);
        }
#pragma unroll
        for (int pl = 0; pl < 4; ++pl) {
          if (hz + 1 < lz)
            cp_async4(&s_hz[1][pl][f][tid], reinterpret_cast<const R*>(src + pl * S + g + lxly));
          if (hz > 0)
            cp_async4(&s_hz[0][pl][f][tid], reinterpret_cast<const R*>(src + pl * S + g - lxly) + 1);
          if (tid == 0 && hx > 0) cp_async8(&s_hx[0][pl][f], src + pl * S + g - 1);
          if (tid == count - 1 && hx + 1 < lx) cp_async8(&s_hx[1][pl][f], src + pl * S + g + 1);
        }
      }
    }
    cp_async_commit();       // group 2: the halo, which only its own thread reads
    cp_async_wait_group<1>();  // group 1 has landed (this thread's part of it)
    if (TMA && !(mbar_wait(&bars[0], phase) && mbar_wait(&bars[1], phase)))
      atomicOr(&a.dyn[cell].status, (unsigned int)RH_STATUS_TIMEOUT);
  } else if (!kStage) {
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      s_ci2[p][tid] = valid ? ci2[p * S + g] : splat2(R(0));
      s_cn2[p][tid] = valid ? cn2[p * S + g] : splat2(R(0));
    }
  }
  __syncthreads();

  R p_cs = R(0), p_xicat = R(0), p_xinaca = R(0);
  uint32_t tstat = 0;  // this thread's status bits
  // output-step statistics of this thread's CRU, in the lattice precision
  // (the integer ones are exact in FP32 too)
  R o[OUT ? NOUT : 1];
  if (OUT) {
#pragma unroll
    for (int k = 0; k < NOUT; ++k) o[k] = R(0);
  }

  if (valid) {
    const StepCoef<R>& k = sk;
    // the cell's build options (perm, iso, slowncxchange, NCX form); the
    // OPT = false variant runs groups whose cells use none of them, with all
    // of this folded away at compile time
    const bool o_perm = OPT && k.perm;
    const bool o_slowncx = OPT && k.slowncx;
    const int o_ncx = OPT ? k.ncx_form : RH_NCX_ALLOSTERIC;
    const R dt = k.dt;
    const int x = q % lx, y = (q / lx) % ly, z = q / lxly;
    const R* cs = L.cs[par];
    V* cinext2 = reinterpret_cast<V*>(L.ci[par ^ 1]);
    V* cnnext2 = reinterpret_cast<V*>(L.cnsr[par ^ 1]);
    R* csnext = L.cs[par ^ 1];

    R cp = kSS ? s_sc[0][tid] : L.cp[g], cjsr = kSS ? s_sc[1][tid] : L.cjsr[g];
    const R cs0 = kStage ? s_cs[tid] : cs[g];
    // ---- dyad/submembrane/JSR coupling terms from the old state (:1309-1314) ----
    const R ci0 = s_ci2[0][tid].x, ci1 = s_ci2[0][tid].y;
    const R cn0 = s_cn2[0][tid].x, cn1 = s_cn2[0][tid].y;
    const R diffpi0 = (cp - ci0) * R(1.0 / TAUPI / 2.);
    const R diffpi1 = (cp - ci1) * R(1.0 / TAUPI / 2.);
    const R diffsi0 = (cs0 - ci0) * R(1.0 / TAUSI / 2.);
    const R diffsi1 = (cs0 - ci1) * R(1.0 / TAUSI / 2.);
    const R diffjn0 = (cjsr - cn0) * R(1.0 / TAUTR / 2.);
    const R diffjn1 = (cjsr - cn1) * R(1.0 / TAUTR / 2.);

    const bool has_zp = z + 1 < lz, has_zm = z > 0;
    // the buffer fields of pair p + 1 load while pair p is computed (those
    // of pair 0 while the channel part runs)
    V nb0, nb1, nb2, nb3, nb4, nb5;
    {
      const V* b2 = reinterpret_cast<const V*>(L.catf);
      nb0 = b2[g];
      nb1 = reinterpret_cast<const V*>(L.cats)[g];
      nb2 = reinterpret_cast<const V*>(L.cacal)[g];
      nb3 = reinterpret_cast<const V*>(L.casr)[g];
      nb4 = reinterpret_cast<const V*>(L.camyo)[g];
      nb5 = reinterpret_cast<const V*>(L.mgmyo)[g];
    }


    // ---- CRU state of the stochastic part ----
    R cjsrb = kSS ? s_sc[2][tid] : L.cjsrb[g], ancx = kSS ? s_sc[3][tid] : L.ancx[g];
    const uint32_t ryr = kSS ? s_ryr[tid] : L.ryr[g];
    uint2 lccw = kSS ? s_lcc[tid] : L.lcc[g];
    const uint32_t win = kSS ? s_win[tid] : L.win[g];
    int nou = ryr & 0xff, ncu = (ryr >> 8) & 0xff, nob = (ryr >> 16) & 0xff, ncb = ryr >> 24;
    int nl = win & 0xffff, nspark = win >> 16;
    if (k.reset_window) {  // :1244-1247
      nl = 0;
      nspark = 0;
    }
    uint32_t status = 0;
    rh_stream rng;
    const uint32_t pos = (uint32_t)((x + 1) + sh.nxf * ((y + 1) + sh.nyf * (z + 1)));
    rh_stream_init(&rng, sh.seed, sh.cell_id, pos, (uint64_t)sh.step);

    // ---- LCC channels (:1248-1263, reesica.h:14-116) ----
    const R cpx = Math<R>::div(cp + cs0 * R(ICAGAMMA), R(1 + ICAGAMMA));
    R bfca;
    {
      R qq = Math<R>::div(R(25), cpx);
      bfca = Math<R>::div(R(0.175), R(1) + qq * qq);
    }
    if (OPT && k.iso_add_lcc) {  // iso: the empty slots 4-7 receive a channel in state 3 (:1213-1218)
      uint32_t hi = lccw.y;
#pragma unroll
      for (int b = 0; b < 32; b += 8)
        if (((hi >> b) & 0xffu) == 16u) hi = (hi & ~(0xffu << b)) | (3u << b);
      lccw.y = hi;
    }
    int nlcp = 0;
    if (!o_perm) {  // a permeabilised cell has no LCC current (:1249-1263 under -Dperm)
      uint64_t slots = ((uint64_t)lccw.y << 32) | lccw.x;
#pragma unroll 1
      for (int ll = 0; ll < 8; ++ll) {
        const int sh8 = ll * 8;
        int st = (int)((slots >> sh8) & 0xff);
        if (st >= 16) break;  // the reference stops at the first empty slot
        R u = Math<R>::uniform(&rng);
        st = lcc_next<R>(st, u * k.rdt, k.alphac, k.betac, k.alphad, k.betad, k.alphaf, k.betaf,
                         R(0.012 / 2.), bfca);
        slots = (slots & ~(0xffull << sh8)) | ((uint64_t)st << sh8);
        if (st == 0) {
          ++nl;
          ++nlcp;
        }
      }
      lccw.x = (uint32_t)slots;
      lccw.y = (uint32_t)(slots >> 32);
    }
    R icat1 = R(0);
    if (!o_perm) {
      R ica = k.lcc_k * (cpx * k.lcc_e2z_k - k.cao);
      if (ica > R(0)) ica = R(0);
      icat1 = k.svica * R(nlcp) * ica;
    }

    // ---- RyR gating, spark flag, release (:1274-1293) ----
    R roo2, mono;
    csqn_mono<R>(cjsr, roo2, mono);
    const int prevsp = nou + nob;
    ryr_gating<R>(&rng, k, cp, cjsr, mono, ncu, nou, ncb, nob, &status);
    if (prevsp < 5 && nou + nob >= 5) nspark = 1;
    const R po = Math<R>::div(R(nou + nob), R(NRYR));
    R xire = R(0.0147 * SVJMAX) * po * (cjsr - cp) * R(1.0 / VP);
    xire = clamp0(xire);

    // ---- NCX (:1296, subroutine_cuda.c:47-120); zero in a permeabilised
    //      cell, whose Ancx keeps its value (:1302) ----
    R xinaca = R(0);
    if (!o_perm) {
      const R csm = cs0 * R(1e-3);
      const R t3 = k.ncx_t3a + csm * R(XNAO * XNAO * XNAO);
      if (o_ncx == RH_NCX_ALLOSTERIC) {  // ncx, :47-75
        const R t2 = R(KMNAO * KMNAO * KMNAO) * csm * (R(1) + csm * R(1.0 / KMCAI));
        const R ka = o_slowncx ? ancx * R(5) : ancx;  // slowncxchange: Ka = 5 Ancx (:59-62)
        const R inaca = Math<R>::div(ka * R(VNACA) * (k.ncx_num_a - k.ncx_num_b * csm),
                                     (k.ncx_t1 + t2 + t3) * k.ncx_den2);
        const R r3 = Math<R>::div(R(0.0003), csm);
        ancx += (Math<R>::div(R(1), R(1) + r3 * r3 * r3) - ancx) * R(1.0 / 150.) * dt;
        xinaca = k.svncx * inaca;
      } else {  // oldncx (:77-100) and ncx_noallo (:102-120)
        R ka = R(1);
        if (k.ncx_ka_hill) {
          const R q = Math<R>::div(R(KDA), csm);
          ka = Math<R>::div(R(1), R(1) + q * q * q);
        }
        const R t2 = R(KMNAO * KMNAO * KMNAO) * csm + k.ncx_t2b * (R(1) + csm * R(1.0 / KMCAI));
        const R inaca = Math<R>::div(ka * R(VNACA) * (k.ncx_num_a - k.ncx_num_b * csm),
                                     (k.ncx_t1 + t2 + t3) * k.ncx_den2);
        if (o_ncx == RH_NCX_OLD) {  // allosteric state from on/off rates, capped
          const R cu = csm * R(1000);
          const R on = R(KNCXON_OLD) * cu * cu;
          R da = on * (R(1) - ancx) - ancx * R(KNCXOFF_OLD);
          if (on * dt > R(0.95)) da = k.rdt95 * (R(1) - ancx) - ancx * R(KNCXOFF_OLD);
          ancx += da * dt;
        }
        xinaca = k.svncx * inaca;
      }
    }
    // slowncxchange background Ca current (:1267-1269), into xicat and the
    // submembrane balance
    R bcgcur = R(0);
    if (o_slowncx) bcgcur = k.bcg_a - k.bcg_b * Math<R>::log(Math<R>::div(R(180000), cs0));

    // ---- CSQN buffering of the JSR (:1316-1317) ----
    const R beta = csqn_beta<R>(cjsr, roo2, mono);
    const R jterm = (-diffjn0 - diffjn1) - xire * R(VP / VJSR);
    const R dotcjsr = beta * jterm;
    cjsrb += (R(1) - beta) * jterm * dt;

    // ---- five sub-steps of cs, cp and the sarcolemmal buffers (:1396-1473) ----
    R casar = kSS ? s_sc[4][tid] : L.casar[g], casarh = kSS ? s_sc[5][tid] : L.casarh[g];
    R casarj = kSS ? s_sc[6][tid] : L.casarj[g], casarhj = kSS ? s_sc[7][tid] : L.casarhj[g];
    R csn = cs0;
    {
      const R dth = k.dth, rdth95 = k.rdth95;
      // z faces: zero flux (the ghost repeats cs), or the permeabilised
      // cell's bath value, which its ghosts keep (:1603-1689 under -Dperm)
      const R cs_face = o_perm ? R(PERM_CI_BASAL) : cs0;
      R csN = cs_face, csS = cs_face;
      if (has_zp) csN = BULK ? b_hcs[1][tid + ocp] : kStage ? s_hcs[1][tid] : __ldg(cs + g + lxly);
      if (has_zm) csS = BULK ? b_hcs[0][tid + ocm] : kStage ? s_hcs[0][tid] : __ldg(cs + g - lxly);
      const R csdiff = (csN + csS - R(2) * cs0) * R(1.0 / TAUST);
      const R cs_const = -R(ICAGAMMA * VP / VS) * icat1 + xinaca -
                         (cs0 - ci0) * R(1.0 / TAUSI / 2.) - (cs0 - ci1) * R(1.0 / TAUSI / 2.) +
                         csdiff - bcgcur;
      const R cp_const =
          (ci0 - cp) * R(1.0 / TAUPI / 2.) + (ci1 - cp) * R(1.0 / TAUPI / 2.) + xire - icat1;
#pragma unroll 1
      for (int it = 0; it < 5; ++it) {
        const R r_sar = buffer_rate<R>(R(KSARON), R(KSAROFF), R(BSAR), casar, csn, dth, rdth95);
        const R r_sarh =
            buffer_rate<R>(R(KSARHON), R(KSARHOFF), R(BSARH), casarh, csn, dth, rdth95);
        R dotcs = R(VP / VS / TAUPS) * (cp - csn) + cs_const - (r_sar + r_sarh);
        if (o_perm) dotcs += (R(PERM_CI_BASAL) - csn) * R(0.2);  // :1409-1411
        const R cpbuff = buffer_rate<R>(R(KSARON), R(KSAROFF), R(BSAR), casarj, cp, dth, rdth95);
        const R cpbuffh =
            buffer_rate<R>(R(KSARHON), R(KSARHOFF), R(BSARH), casarhj, cp, dth, rdth95);
        const R cpdot = (csn - cp) * R(1.0 / TAUPS) + cp_const - cpbuff - cpbuffh;
        casarj = clamp0(casarj + cpbuff * dth);
        casarhj = clamp0(casarhj + cpbuffh * dth);
        cp += cpdot * dth;
        casar = clamp0(casar + r_sar * dth);
        casarh = clamp0(casarh + r_sarh * dth);
        csn += dotcs * dth;
      }
    }
    cp = clamp0(cp);
    if (csn < R(0)) csn = R(1e-6);
    cjsr = cjsr + dotcjsr * dt;

    // ---- stores ----
    L.cp[g] = cp;
    L.cjsr[g] = cjsr;
    L.cjsrb[g] = cjsrb;
    L.ancx[g] = ancx;
    L.casar[g] = casar;
    L.casarh[g] = casarh;
    L.casarj[g] = casarj;
    L.casarhj[g] = casarhj;
    csnext[g] = csn;
    L.ryr[g] = (uint32_t)nou | ((uint32_t)ncu << 8) | ((uint32_t)nob << 16) | ((uint32_t)ncb << 24);
    L.lcc[g] = lccw;
    L.win[g] = (uint32_t)(nl & 0xffff) | ((uint32_t)nspark << 16);
    if (a.diag) {
      a.diag[(int64_t)D_XIRE * S + g] = (double)xire;
      a.diag[(int64_t)D_PO * S + g] = (double)po;
      a.diag[(int64_t)D_XINACA * S + g] = (double)xinaca;
      a.diag[(int64_t)D_XICAT * S + g] = (double)(icat1 + bcgcur * R(VS / VP));
    }
    tstat = status;

    // the channel part above reads no halo; the sub-voxel part below needs
    // this thread's halo copies
    if (kStage) cp_async_wait_group<0>();
    if constexpr (BULK) {
      if (!mbar_wait(&bars[1], phase)) tstat |= RH_STATUS_TIMEOUT;
    }

    // ---- sub-voxel diffusion, SERCA/leak, cytosolic buffers (:1305-1393) ----
    // Processed as four z-pairs p = (sub-voxels 2p, 2p+1).  Along z the pair's
    // halves are each other's neighbour; the outer neighbours are the
    // adjacent CRUs' pair p.  Along y (x) the neighbour pair is p^1 (p^2) of
    // this CRU or of the adjacent CRU in the direction of the pair's y (x)
    // bit.  At a lattice face the zero-flux ghost equals the sub-voxel
    // itself (:1601-1652), so that difference vanishes; a permeabilised
    // cell's ci ghosts instead keep the bath value (:1653-1689).
    const bool has_yp = y + 1 < ly, has_ym = y > 0;
    const bool has_xp = x + 1 < lx, has_xm = x > 0;
    const bool zp_in = tid + lxly < count, zm_in = tid - lxly >= 0;
    const bool yp_in = tid + lx < count, ym_in = tid - lx >= 0;
    const bool xp_in = tid + 1 < count, xm_in = tid - 1 >= 0;
    const V kt_n = splat2(R(1.0 / (TAUNT * XI))), kl_n = splat2(R(1.0 / (TAUNL * XI)));
    const V kt_i = splat2(R(1.0 / (TAUIT * XI))), kl_i = splat2(R(1.0 / (TAUIL * XI)));
    const V dt2 = splat2(dt);
    const V* catf2 = reinterpret_cast<const V*>(L.catf);
    const V* cats2 = reinterpret_cast<const V*>(L.cats);
    const V* cacal2 = reinterpret_cast<const V*>(L.cacal);
    const V* casr2 = reinterpret_cast<const V*>(L.casr);
    const V* camyo2 = reinterpret_cast<const V*>(L.camyo);
    const V* mgmyo2 = reinterpret_cast<const V*>(L.mgmyo);
    V* catf2w = reinterpret_cast<V*>(L.catf);
    V* cats2w = reinterpret_cast<V*>(L.cats);
    V* cacal2w = reinterpret_cast<V*>(L.cacal);
    V* casr2w = reinterpret_cast<V*>(L.casr);
    V* camyo2w = reinterpret_cast<V*>(L.camyo);
    V* mgmyo2w = reinterpret_cast<V*>(L.mgmyo);
    R sum_ci = R(0), sum_cn = R(0), sum_catf = R(0), sum_cats = R(0), sum_casr = R(0);
    R sum_camyo = R(0), sum_cacal = R(0), sum_up = R(0), sum_lk = R(0);
    bool ci_high = false;
#pragma unroll 1
    for (int p = 0; p < 4; ++p) {
      const int by = p & 1, bx = p >> 1;
      const uint32_t gp = p * S + g;
      const V c = s_ci2[p][tid], n = s_cn2[p][tid];
      V catf = nb0, cats = nb1, cacal = nb2, casr = nb3, camyo = nb4, mgmyo = nb5;
      if (p < 3) {
        const uint32_t gq = gp + S;
        nb0 = catf2[gq], nb1 = cats2[gq], nb2 = cacal2[gq], nb3 = casr2[gq], nb4 = camyo2[gq];
        nb5 = mgmyo2[gq];
      }
      // ci a face ghost holds: the sub-voxel's own value, or the bath
      const V cface = o_perm ? splat2(R(PERM_CI_BASAL)) : c;
      // z
      V czp = c, nzp = n, czm = c, nzm = n;
      if (BULK) {
        if (has_zp) {
          czp.x = b_hz[1][p][0][tid + oz].x;
          nzp.x = b_hz[1][p][1][tid + oz].x;
        }
        if (has_zm) {
          czm.y = b_hz[0][p][0][tid + oz].y;
          nzm.y = b_hz[0][p][1][tid + oz].y;
        }
      } else if (kStage) {
        if (has_zp) {
          czp.x = s_hz[1][p][0][tid];
          nzp.x = s_hz[1][p][1][tid];
        }
        if (has_zm) {
          czm.y = s_hz[0][p][0][tid];
          nzm.y = s_hz[0][p][1][tid];
        }
      } else {
      if (has_zp) {
        if (zp_in) {
          czp = s_ci2[p][tid + lxly];
          nzp = s_cn2[p][tid + lxly];
        } else {
          czp = __ldg(ci2 + gp + lxly);
          nzp = __ldg(cn2 + gp + lxly);
        }
      }
      if (has_zm) {
        if (zm_in) {
          czm = s_ci2[p][tid - lxly];
          nzm = s_cn2[p][tid - lxly];
        } else {
          czm = __ldg(ci2 + gp - lxly);
          nzm = __ldg(cn2 + gp - lxly);
        }
      }
      }
      const V ciN = v2(c.y, has_zp ? czp.x : cface.y), cnN = v2(n.y, has_zp ? nzp.x : n.y);
      const V ciS = v2(has_zm ? czm.y : cface.x, c.x), cnS = v2(has_zm ? nzm.y : n.x, n.x);
      // y: pair p^1 of this CRU (inside) and of the CRU on the side of the
      // pair's y bit (outside).  The stencil only sums the two differences,
      // so they need no east/west order.
      V ciy_in, cny_in, ciy_ex, cny_ex;
      {
        const int py = p ^ 1;
        const V ci_in = s_ci2[py][tid], cn_in = s_cn2[py][tid];
        V ci_ex = cface, cn_ex = n;
        const int d = by ? lx : -lx;
        if (by ? has_yp : has_ym) {
          if (BULK) {
            ci_ex = b_hy[by][p >> 1][0][tid + oy];
            cn_ex = b_hy[by][p >> 1][1][tid + oy];
          } else if (kStage) {
            ci_ex = s_hy[by][p >> 1][0][tid];
            cn_ex = s_hy[by][p >> 1][1][tid];
          } else if (by ? yp_in : ym_in) {
            ci_ex = s_ci2[py][tid + d];
            cn_ex = s_cn2[py][tid + d];
          } else {
            ci_ex = __ldg(ci2 + py * S + g + d);
            cn_ex = __ldg(cn2 + py * S + g + d);
          }
        }
        ciy_in = ci_in;
        cny_in = cn_in;
        ciy_ex = ci_ex;
        cny_ex = cn_ex;
      }
      // x: pair p^2, likewise
      V cix_in, cnx_in, cix_ex, cnx_ex;
      {
        const int px = p ^ 2;
        const V ci_in = s_ci2[px][tid], cn_in = s_cn2[px][tid];
        V ci_ex = cface, cn_ex = n;
        const int d = bx ? 1 : -1;
        if (bx ? has_xp : has_xm) {
          if (bx ? xp_in : xm_in) {
            ci_ex = s_ci2[px][tid + d];
            cn_ex = s_cn2[px][tid + d];
          } else if (BULK) {
            ci_ex = b_hx[bx][px][0];
            cn_ex = b_hx[bx][px][1];
          } else if (kStage) {
            ci_ex = s_hx[bx][px][0];
            cn_ex = s_hx[bx][px][1];
          } else {
            ci_ex = __ldg(ci2 + px * S + g + d);
            cn_ex = __ldg(cn2 + px * S + g + d);
          }
        }
        cix_in = ci_in;
        cnx_in = cn_in;
        cix_ex = ci_ex;
        cnx_ex = cn_ex;
      }
      const V coupn =
          vfma(vadd(vadd(vadd(vsub(cnN, n), vsub(cnS, n)), vsub(cny_in, n)), vsub(cny_ex, n)), kt_n,
               vmul(vadd(vsub(cnx_in, n), vsub(cnx_ex, n)), kl_n));
      const V coupi =
          vfma(vadd(vadd(vadd(vsub(ciN, c), vsub(ciS, c)), vsub(ciy_in, c)), vsub(ciy_ex, c)), kt_i,
               vmul(vadd(vsub(cix_in, c), vsub(cix_ex, c)), kl_i));
      // SERCA and leak (subroutine_cuda.c:128-146)
      V up, lk;
      {
        const R pax = serca_pow<0>(c.x), pay = serca_pow<0>(c.y);
        const R pbx = serca_pow<1>(n.x), pby = serca_pow<1>(n.y);
        up = v2(k.sviup * Math<R>::div(R(VUP) * (pax - pbx), R(1) + pax + pbx),
                k.sviup * Math<R>::div(R(VUP) * (pay - pby), R(1) + pay + pby));
        const V n2 = vmul(n, n);
        const V num = vmul(vmul(splat2(R(GLEAK)), vsub(n, c)), n2);
        const V den = vadd(n2, splat2(R(KJSR_LEAK * KJSR_LEAK)));
        lk = v2(Math<R>::div(num.x, den.x), Math<R>::div(num.y, den.y));
      }
      // cytosolic buffers (buffers.c:55-115): on*(B-b) - koff*b, where the
      // saturation guard kon*c*dt > 1 replaces on by 0.95/dt.  Myosin's
      // guard (kon 13.8 per uM ms) trips from c = 2.9 uM on, which the
      // sub-voxels near a releasing dyad pass in most warps of a beating
      // cell: its on-rate is a per-half select.  The other four (kon <= 0.1,
      // from c = 400 uM on) take the slow path.
      const V freemyo = vsub(vsub(splat2(R(BMYO)), camyo), mgmyo);
      V r_tf = vfma(vmul(splat2(R(KTFON)), c), vsub(splat2(R(BTF)), catf), vmul(splat2(R(-KTFOFF)), catf));
      V r_ts = vfma(vmul(splat2(R(KTSON)), c), vsub(splat2(R(BTS)), cats), vmul(splat2(R(-KTSOFF)), cats));
      V r_cal = vfma(vmul(splat2(R(KCALON)), c), vsub(splat2(R(BCAL)), cacal),
                     vmul(splat2(R(-KCALOFF)), cacal));
      V r_sr = vfma(vmul(splat2(R(KSRON)), c), vsub(splat2(R(BSR)), casr), vmul(splat2(R(-KSROFF)), casr));
      V on_mc = vmul(splat2(R(KONMYOCA)), c);
      on_mc.x = (on_mc.x * dt > R(1)) ? k.rdt95 : on_mc.x;
      on_mc.y = (on_mc.y * dt > R(1)) ? k.rdt95 : on_mc.y;
      const V r_mc = vfma(on_mc, freemyo, vmul(splat2(R(-KOFFMYOCA)), camyo));
      static_assert(KTFON <= KSRON && KTSON <= KSRON && KCALON <= KSRON, "SR has the largest on-rate");
      if (fmax(c.x, c.y) * R(KSRON) * dt > R(1)) {  // another buffer saturates
        const R cc[2] = {c.x, c.y};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const R cv = cc[h];
          R& tf = h ? r_tf.y : r_tf.x;
          R& ts = h ? r_ts.y : r_ts.x;
          R& cal = h ? r_cal.y : r_cal.x;
          R& sr = h ? r_sr.y : r_sr.x;
          tf = buffer_rate<R>(R(KTFON), R(KTFOFF), R(BTF), h ? catf.y : catf.x, cv, dt, k.rdt95);
          ts = buffer_rate<R>(R(KTSON), R(KTSOFF), R(BTS), h ? cats.y : cats.x, cv, dt, k.rdt95);
          cal = buffer_rate<R>(R(KCALON), R(KCALOFF), R(BCAL), h ? cacal.y : cacal.x, cv, dt, k.rdt95);
          sr = buffer_rate<R>(R(KSRON), R(KSROFF), R(BSR), h ? casr.y : casr.x, cv, dt, k.rdt95);
        }
      }
      V dotcn = vfma(vsub(up, lk), splat2(R(VI / VNSR)), coupn);
      V dotci = vadd(vsub(vsub(lk, up), vadd(vadd(vadd(vadd(r_tf, r_ts), r_cal), r_sr), r_mc)), coupi);
      if (p == 0) {  // sub-voxels 0 and 1 touch the dyad, submembrane and JSR (:1356-1361)
        dotcn = vfma(v2(diffjn0, diffjn1), splat2(R(VJSR / VNSR)), dotcn);
        dotci = vfma(v2(diffsi0, diffsi1), splat2(R(VS / VI)), dotci);
        dotci = vfma(v2(diffpi0, diffpi1), splat2(R(VP / VI)), dotci);
      }
      const V cinew = vclamp0(vfma(dotci, dt2, c));
      const V cnnew = vfma(dotcn, dt2, n);
      catf = vclamp0(vfma(r_tf, dt2, catf));
      cats = vclamp0(vfma(r_ts, dt2, cats));
      cacal = vclamp0(vfma(r_cal, dt2, cacal));
      casr = vclamp0(vfma(r_sr, dt2, casr));
      camyo = vclamp0(vfma(r_mc, dt2, camyo));
      {
        const V fm = vsub(vsub(splat2(R(BMYO)), camyo), mgmyo);
        V r_mg = vfma(splat2(R(KONMYOMG * MGI)), fm, vmul(splat2(R(-KOFFMYOMG)), mgmyo));
        if (R(KONMYOMG * MGI) * dt > R(1)) {  // guard of myomg (buffers.c:65)
          r_mg = vfma(splat2(k.rdt95), fm, vmul(splat2(R(-KOFFMYOMG)), mgmyo));
        }
        mgmyo = vclamp0(vfma(r_mg, dt2, mgmyo));
      }
      cinext2[gp] = cinew;
      cnnext2[gp] = cnnew;
      catf2w[gp] = catf;
      cats2w[gp] = cats;
      cacal2w[gp] = cacal;
      casr2w[gp] = casr;
      camyo2w[gp] = camyo;
      mgmyo2w[gp] = mgmyo;
      if (a.diag) {
        a.diag[(int64_t)(D_XIUP + 2 * p) * S + g] = (double)up.x;
        a.diag[(int64_t)(D_XIUP + 2 * p + 1) * S + g] = (double)up.y;
        a.diag[(int64_t)(D_XILEAK + 2 * p) * S + g] = (double)lk.x;
        a.diag[(int64_t)(D_XILEAK + 2 * p + 1) * S + g] = (double)lk.y;
      }
      if (OUT && out_step) {
        sum_ci += cinew.x + cinew.y;
        sum_cn += cnnew.x + cnnew.y;
        sum_catf += catf.x + catf.y;
        sum_cats += cats.x + cats.y;
        sum_casr += casr.x + casr.y;
        sum_camyo += camyo.x + camyo.y;
        sum_cacal += cacal.x + cacal.y;
        sum_up += up.x + up.y;
        sum_lk += lk.x + lk.y;
        ci_high |= (cinew.x > R(1000)) || (cinew.y > R(1000));
      }
    }

    p_cs = csn;
    p_xicat = icat1 + bcgcur * R(VS / VP);  // xicat (:1271)
    p_xinaca = xinaca;

    if (OUT && out_step) {
      o[O_CP - P_STEP_END] = cp;
      o[O_CJSR - P_STEP_END] = cjsr;
      o[O_CJSRB - P_STEP_END] = cjsrb;
      o[O_CNSR - P_STEP_END] = sum_cn;
      o[O_CI - P_STEP_END] = sum_ci;
      o[O_PO - P_STEP_END] = po;
      o[O_NCB - P_STEP_END] = ncb;
      o[O_NCXFWD - P_STEP_END] = xinaca < R(0) ? xinaca : R(0);
      o[O_CATF - P_STEP_END] = sum_catf;
      o[O_CATS - P_STEP_END] = sum_cats;
      o[O_CASR - P_STEP_END] = sum_casr;
      o[O_CAMYO - P_STEP_END] = sum_camyo;
      o[O_CACAL - P_STEP_END] = sum_cacal;
      o[O_LEAK - P_STEP_END] = sum_lk;
      o[O_UP - P_STEP_END] = sum_up;
      o[O_XIRE - P_STEP_END] = xire;
      o[O_ANCX - P_STEP_END] = ancx;
      o[O_CASAR - P_STEP_END] = casar;
      o[O_CASARH - P_STEP_END] = casarh;
      o[O_CASARJ - P_STEP_END] = casarj;
      o[O_CASARHJ - P_STEP_END] = casarhj;
      o[O_NOU - P_STEP_END] = nou;
      o[O_NOB - P_STEP_END] = nob;
      o[O_NCU - P_STEP_END] = ncu;
      {
        int tn[7] = {0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int ll = 0; ll < 8; ++ll) {
          int st = ((ll < 4 ? lccw.x : lccw.y) >> ((ll & 3) * 8)) & 0xff;
          if (st < 16) {
            tn[0] += st & 1;
            tn[1] += (st >> 1) & 1;
            tn[2] += (st >> 2) & 1;
            tn[3] += (st >> 3) & 1;
            tn[4] += ((st >> 2) & 3) == 1;
            tn[5] += st <= 1;
            tn[6] += st == 0;
          }
        }
#pragma unroll
        for (int kk = 0; kk < 7; ++kk) o[O_TN1 - P_STEP_END + kk] = tn[kk];
      }
      o[O_SPARK - P_STEP_END] = nspark;
      o[O_CIHIGH - P_STEP_END] = ci_high ? R(1) : R(0);
      if (cadist_step) {  // cadist row (:1009), post-step values in this CRU's slot
        double* r = a.out_cd + sh.cd_off + sh.cd_slot * (2 + 6 * (long long)sh.n) + 2 + 6 * (long long)q;
        r[0] = (double)cinext2[g].x;
        r[1] = (double)csn;
        r[2] = (double)cp;
        r[3] = (double)cjsr;
        r[4] = (double)xinaca;  // scaled on the host as the reference prints it
        r[5] = (double)xire;
      }
      if (a.out_ls && y == sh.line_y && z == sh.line_z) {  // linescan row (:967-989), post-step values
        const uint32_t g0 = g;
        double* r = a.out_ls + ((size_t)sh.ls_off + (size_t)sh.slot * lx + x) * RH_LINESCAN_COLS;
        r[0] = sh.t;
        r[1] = (double)(x + 1);
        r[2] = (double)cinext2[g0].x;
        r[3] = nob;
        r[4] = nou;
        r[5] = ncb;
        r[6] = ncu;
        r[7] = nl;
        r[8] = (double)csn;
        r[9] = (double)cp;
        r[10] = (double)casar;
        r[11] = (double)casarh;
        r[12] = (double)L.camyo[2 * g0];
        r[13] = (double)L.mgmyo[2 * g0];
        r[14] = (double)L.casr[2 * g0];
        r[15] = (double)L.cacal[2 * g0];
        r[16] = (double)L.cats[2 * g0];
        r[17] = (double)L.catf[2 * g0];
        r[18] = (double)xire;
        r[19] = (double)cjsr;
        r[20] = (double)ancx;
        r[21] = (double)xinaca;
      }
    }
  }

  // every thread waits for the halo rows, so no bulk copy is still writing
  // this CTA's shared memory when it finishes
  if constexpr (BULK) {
    if (!valid) mbar_wait(&bars[1], phase);
  }

  // ---- per-warp reduction: the per-step sums exactly (fixedsum.cuh) into
  //      the cell's accumulators, the output-step statistics as one FP64
  //      partial row per warp; no CTA barrier ----
  const int warp = tid >> 5, lane = tid & 31;
  constexpr int NW = kBlock / 32;
  uint64_t qlo = 0, qhi = 0;  // lane q < 3: the warp's sum q
  uint32_t bad = 0;
  {
    const R pv[3] = {p_cs, p_xicat, p_xinaca};
#pragma unroll
    for (int qq = 0; qq < 3; ++qq) {
      uint64_t lo, hi;
      if constexpr (sizeof(R) == 4) {
        fx_warp_sum_f32(pv[qq], lo, hi, bad);  // every lane holds the sum
      } else {
        fx_from(pv[qq], lo, hi, bad);
        fx_warp_sum(lo, hi);
        lo = __shfl_sync(0xffffffffu, lo, 0);
        hi = __shfl_sync(0xffffffffu, hi, 0);
      }
      if (lane == qq) {
        qlo = lo;
        qhi = hi;
      }
    }
  }
  const uint32_t wst = __reduce_or_sync(0xffffffffu, tstat | (bad ? (uint32_t)RH_STATUS_NAN : 0u));
  if (OUT && out_step) {
    double* dst = a.partials + ((size_t)(a.tile_base + ti) * NW + warp) * P_COUNT;
    static_assert(O_CIHIGH - P_STEP_END == NOUT - 1 && NOUT - 1 == 32,
                  "one summed statistic per lane, the ci flag last");
    if constexpr (sizeof(R) == 4) {
      // exact warp sums in 128-bit fixed point (integer adds, no FP64
      // instruction); lane kk keeps statistic kk and converts it once; a
      // non-finite (or out-of-range) value makes the statistic NaN
      uint64_t mlo = 0, mhi = 0;
      bool mbad = false;
#pragma unroll
      for (int kk = 0; kk < NOUT - 1; ++kk) {
        uint64_t lo, hi;
        uint32_t bad = 0;
        fx_warp_sum_f32(o[kk], lo, hi, bad);
        const bool wbad = __any_sync(0xffffffffu, bad != 0u);
        if (lane == kk) {
          mlo = lo;
          mhi = hi;
          mbad = wbad;
        }
      }
      dst[P_STEP_END + lane] = mbad ? __longlong_as_double(0x7ff8000000000000ll) : fx_to_double(mlo, mhi);
      const bool high = __any_sync(0xffffffffu, o[NOUT - 1] > R(0));
      if (lane == 0) dst[P_STEP_END + NOUT - 1] = high ? 1.0 : 0.0;
    } else {
#pragma unroll 1
      for (int kk = 0; kk < NOUT; ++kk) {
        double v = o[kk];
        if (kk == O_CIHIGH - P_STEP_END) {
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, off));
        } else {
          v = warp_sum(v);
        }
        if (lane == 0) dst[P_STEP_END + kk] = v;
      }
    }
  }
  if (lane < 3) {
    fx_atomic_add(&a.dyn[cell].acc[2 * lane], qlo, qhi);
    if (lane == 0 && wst) atomicOr(&a.dyn[cell].status, wst);
  }
  return true;
}


}  // namespace rh
