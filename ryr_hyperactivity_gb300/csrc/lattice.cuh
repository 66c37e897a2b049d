// lattice.cuh — device data layout of the batched simulator.
//
// HBM layout (structure of arrays, all cells concatenated):
//   * a cell owns the CRU index range [off, off + n) of every field, n =
//     (nx-2)(ny-2)(nz-2) interior CRUs, x fastest (q = x + lx*(y + ly*z));
//     ranges are padded to a multiple of 32 so no warp spans two cells;
//   * per-CRU fields are one array of `stride` elements; per-sub-voxel fields
//     hold 8 values per CRU (sub-voxel ii: bit 0 = z, bit 1 = y, bit 2 = x
//     half, as cuda_Cell_Detailed.cu:1322-1327 defines) stored as 4 planes of
//     z-pairs: sub-voxels 2p and 2p+1 of CRU g are adjacent at
//     (p*stride + g)*2 + {0,1} (sub_index), so one 8-byte (FP32) or 16-byte
//     (FP64) coalesced access moves a pair;
//   * ci, cnsr and cs are ping-ponged (two buffers, per-cell parity);
//   * integer state packs into 16 B per CRU: RyR counts (4 x 8 bit), eight
//     LCC slot states (8 x 8 bit) and the window counters nl (16 bit) and
//     nspark (16 bit).
// Ghost CRUs are not stored: the reference's zero-flux ghost copies
// (:1601-1652) make every boundary difference exactly zero, so boundary
// terms are dropped and the z-ghost of cs reads the CRU's own value.
#pragma once

#include <cuda.h>
#include <stdint.h>

#include "../../include/rh.h"
#include "beatstats.cuh"
#include "model.cuh"

namespace rh {

// Element index of sub-voxel ii of CRU g in a per-sub-voxel field.
__host__ __device__ __forceinline__ int64_t sub_index(int ii, int64_t g, int64_t stride) {
  return (((int64_t)(ii >> 1) * stride + g) << 1) | (ii & 1);
}

template <class R>
struct Lattice {
  R* cp;
  R* cjsr;
  R* cjsrb;
  R* ancx;
  R* casar;
  R* casarh;
  R* casarj;
  R* casarhj;
  R* cs[2];
  R* ci[2];    // 4 pair planes each
  R* cnsr[2];  // 4 pair planes each
  R* catf;     // 4 pair planes
  R* cats;
  R* cacal;
  R* casr;
  R* camyo;
  R* mgmyo;
  uint32_t* ryr;  // nou | ncu << 8 | nob << 16 | ncb << 24
  uint2* lcc;     // slot ll in byte ll (x: slots 0-3, y: slots 4-7)
  uint32_t* win;  // nl | nspark << 16
  int64_t stride;
};

// Read-only per-cell constants.
struct CellConst {
  int lx, ly, lz;  // interior extent
  int nxf, nyf;    // full lattice extent (Philox CRU index uses ghosts)
  int n;           // interior CRUs
  long long off;   // first CRU index
  int tile_begin, tile_count;
  int line_y, line_z;  // linescan row (interior coordinates)
  int iso2;
  uint32_t seed, cell_id;
  long long ls_off;  // first linescan row of this cell in the ring
  long long cd_off;  // first double of this cell's cadist records (record_cadist)
  double svica, svncx, sviup_tot, svikr, cao, ku, ku2, kb, pcl, tend;
  int perm;            // permeabilised cell (rh_cell_params.perm)
  int protocol;        // RH_PROTO_*
  double clamp_mv;     // RH_PROTO_VCLAMP holding voltage
  const double* apv;   // RH_PROTO_AP_CLAMP waveform (device), napv samples
  int napv;
  int iso, randomlcc, slowncx, ncx_form;  // build options (rh_cell_params)
  double sviup_iso;    // SERCA prefactor once iso is active (t >= 5.5 PCL)
};

// Mutable per-cell state, owned by the device between host calls.
struct CellDyn {
  rh_membrane m;
  StepCoef<double> cd;  // coefficients of the next lattice update, FP64 path
  StepCoef<float> cf;   // the same in FP32 for the mixed path
  uint32_t status;
  int parity;
  int done;
  unsigned int arrive;  // reserved, always 0 (kept for the exported state layout)
  long long out_count;  // output records produced
  BeatTracker bt;       // per-beat statistics in progress
  long long stats_count;  // beat records produced
  long long cd_count;     // cadist records produced
  // sum cs, xicat, xinaca of the step in progress as 128-bit fixed point
  // (value * 2^64, lo word first), added to by every warp of the cell's
  // lattice CTAs, read and cleared by the cell's update (fixedsum.cuh)
  unsigned long long acc[6];
};

// Quantities each CTA reduces over its CRUs at output steps (:839-929), in
// FP64 partials per tile.  The first three slots are unused: the per-step
// sums (:435-456) go through the fixed-point accumulators of CellDyn.
enum PartialIdx {
  P_CS = 0,      // sum cs (new)           [sum, comp]
  P_XICAT = 2,   // sum xicat              [sum, comp]
  P_XINACA = 4,  // sum xinaca             [sum, comp]
  P_STEP_END = 6,
  O_CP = 6, O_CJSR, O_CJSRB, O_CNSR, O_CI, O_PO, O_NCB, O_NCXFWD, O_CATF, O_CATS, O_CASR,
  O_CAMYO, O_CACAL, O_LEAK, O_UP, O_XIRE, O_ANCX, O_CASAR, O_CASARH, O_CASARJ, O_CASARHJ,
  O_NOU, O_NOB, O_NCU, O_TN1, O_TN2, O_TN3, O_TN4, O_TN5, O_TN6, O_TN7, O_SPARK, O_CIHIGH,
  P_COUNT
};
constexpr int NOUT = P_COUNT - P_STEP_END;

// Diagnostics of the last lattice update (FP64 planes of `stride`), written
// only when requested: xire, po, xinaca, xicat, xiup[8], xileak[8].
enum DiagPlane { D_XIRE = 0, D_PO, D_XINACA, D_XICAT, D_XIUP, D_XILEAK = D_XIUP + 8, D_COUNT = D_XILEAK + 8 };

template <class R>
__device__ __forceinline__ const StepCoef<R>* coef_ptr(const CellDyn* d);
template <>
__device__ __forceinline__ const StepCoef<double>* coef_ptr<double>(const CellDyn* d) {
  return &d->cd;
}
template <>
__device__ __forceinline__ const StepCoef<float>* coef_ptr<float>(const CellDyn* d) {
  return &d->cf;
}

// Tensor maps of the tensor-copy staging (FP32 only): the pair planes of ci
// and cnsr of each ping-pong parity as 2-D tensors of 8-byte pairs (x: arena
// index, y: pair plane; box B x 4), and the eight per-CRU real planes
// cp .. casarhj as a 2-D tensor of floats (box B x 8).  Built on the host per
// tile length, passed to the lattice launch as a grid constant.
struct StageMaps {
  CUtensorMap plane[4];  // ci[0], ci[1], cnsr[0], cnsr[1]
  CUtensorMap sc;
};

template <class R>
struct StepArgs {
  Lattice<R> L;
  const CellConst* cells;
  CellDyn* dyn;
  const int4* tiles;  // x: cell, y: first local CRU, z: CRUs in tile, w: arena index of that CRU
  int tile_base;      // index of tiles[0] in the simulator's tile table (launches of one group)
  double* partials;   // [tile][P_COUNT], by tile-table index
  double* out_wc;     // [cell][cap][45]
  double* out_ls;     // [ls_off + slot*lx + x][22]
  double* out_cd;     // cadist records, optional: [cd_off + slot*(2 + 6n)]: t, v, 6 per CRU
  int cd_cap;         // cadist records kept per cell
  double* diag;       // optional
  rh_beat_stats* stats;  // [cell][stats_cap], optional
  int stats_cap;
  int out_cap;
  int lattice_only;
  int no_output;      // steps write no output records (the autotuner's trials)
  double dt;
};

}  // namespace rh
