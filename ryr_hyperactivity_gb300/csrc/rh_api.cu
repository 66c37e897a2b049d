// rh_api.cu — host implementation of the C ABI in include/rh.h.
//
// Owns all device memory of a batch of cells, launches the lattice update and
// the cell update of each cell group per time step (step.cu), replays windows
// of steps as captured CUDA graphs,
// mirrors each cell's time on the host to know which steps are output steps,
// and moves state and output records between host and device.
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/rh.h"
#include "cellmodel.cuh"
#include "lattice.cuh"
#include "step.cuh"

using namespace rh;

struct rh_sim {
  int ncells = 0;
  rh_run_opts opts{};
  std::vector<rh_cell_params> params;
  std::vector<CellConst> hcells;  // per-cell constants (tile fields of the current set)
  // one tile table per compiled tile length (kTileSizes); `ts` is in use
  struct TileSet {
    int tile = 0;
    int ntiles = 0;
    std::vector<CellConst> hcells;
    std::vector<int4> htiles;
    CellConst* d_cells = nullptr;
    int4* d_tiles = nullptr;
  } sets[kNumTileSizes];
  int ts = 0;
  // Cell groups: contiguous cell ranges of about equal CRU count, each with
  // its own stream.  A window of steps runs as one graph with a branch per
  // group, so one group's end-of-step tail (its last lattice CTAs and its
  // cell update) overlaps the other groups' lattice work.
  int ngroups = 1;
  std::vector<int> group_cell;  // group g holds cells [group_cell[g], group_cell[g+1])
  std::vector<char> group_opt;  // group g has a cell with lattice build options
  std::vector<cudaStream_t> gstreams;
  std::vector<cudaEvent_t> gevents;  // [0] fork, [1..G] join
  int64_t stride = 0;
  int max_n = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  // device memory
  void* arena = nullptr;
  size_t arena_bytes = 0;
  Lattice<double> Ld{};
  Lattice<float> Lf{};
  CellDyn* d_dyn = nullptr;
  double* d_partials = nullptr;
  double* d_out_wc = nullptr;
  double* d_out_ls = nullptr;
  double* d_out_cd = nullptr;  // cadist records (record_cadist), per cell from cd_off
  double* d_diag = nullptr;
  std::vector<double*> d_apv;  // AP-clamp waveforms, per cell (rh_set_ap_clamp)
  rh_beat_stats* d_stats = nullptr;
  int64_t ls_rows_total = 0;
  // host mirror of each cell's clock (same IEEE additions as the device)
  std::vector<double> t_host;
  std::vector<char> active_host;
  std::vector<long long> drained_wc, drained_ls, drained_st, drained_cd;
  // host staging of rh_drain_wholecell_all: record counters and the record ring
  std::vector<long long> h_counts;
  std::vector<double> h_ring;
  // graphs keyed by (window length, output-step bitmask, host buffers of a
  // state import at the head / export at the tail of each group's branch)
  std::map<std::tuple<int, std::vector<bool>, const void*, void*>, cudaGraphExec_t> graphs;
  // persistent window launches (run option persistent): per-cell arrival and
  // readiness words with the update queue, the wait-timeout flag, and whether
  // a window launch can be captured in a graph on this device (else it is
  // launched directly)
  bool persist_ok = false;
  bool persist_graph = true;
  bool fewer_ctas = false;  // persistent launch at one resident CTA per SM fewer
  int staging = 0;          // two-launch path, FP32: 0 per-thread, 1 bulk, 2 tensor copies
  // tensor maps of the tensor-copy staging, one set per tile length (FP32)
  StageMaps maps[kNumTileSizes]{};
  bool maps_ok = false;
  CellSync* d_sync = nullptr;
  unsigned int* d_err = nullptr;
  unsigned int* h_err = nullptr;  // pinned
  long long wait_limit = kDefaultWaitLimit;
  unsigned int wait_offset = 0;
  long long kernels = 0;  // kernel launches issued for time steps
  // timing
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timing_open = false;
  long long launches_pending = 0, launches_total = 0;
  double ms_total = 0.0;
  std::string err;
};

namespace {

int fail(rh_sim* s, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (s) s->err = buf;
  return code;
}

#define CK(call)                                                                           \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(s, RH_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                     \
  } while (0)

bool is_mixed(const rh_sim* s) { return s->opts.precision == RH_MIXED; }

size_t real_size(const rh_sim* s) { return is_mixed(s) ? sizeof(float) : sizeof(double); }

double csqn_bound_ss(double cjsr) {  // subroutine_cuda.c:179-195
  double roo2 = RATEDIMER / (1.0 + pow(KDIMER / cjsr, HILLDIMER));
  double mono = (-1.0 + sqrt(1.0 + 8.0 * CSQBERS * roo2)) / (4.0 * roo2 * CSQBERS);
  double ene = mono * NM + (1.0 - mono) * ND;
  return CSQBERS * ene * cjsr / (KBERS + cjsr);
}

InitValues init_values(const rh_cell_params& p) {  // cuda_Cell_Detailed.cu:1108-1174
  InitValues v{};
  // :87-92 (perm fixes both basal values), :1118-1120 (tapsi overrides the load)
  double cjsr_b = p.tapsi ? 10 : (p.perm ? PERM_CJSR_BASAL : p.cjsr_basal);
  const double cb = p.perm ? PERM_CI_BASAL : CI_BASAL;
  v.cp = cb;
  v.cs = cb;
  v.cjsr = cjsr_b;
  v.cjsrb = csqn_bound_ss(cjsr_b);
  v.ancx = 0.025;
  v.ci = cb;
  v.cnsr = cjsr_b;
  v.catf = KTFON * cb * BTF / (KTFON * cb + KTFOFF);
  v.cats = KTSON * cb * BTS / (KTSON * cb + KTSOFF);
  v.cacal = KCALON * cb * BCAL / (KCALON * cb + KCALOFF);
  v.casr = KSRON * cb * BSR / (KSRON * cb + KSROFF);
  v.camyo = 3.;
  v.mgmyo = 136.209996;
  v.casar = KSARON * cb * BSAR / (KSARON * cb + KSAROFF);
  v.casarh = KSARHON * cb * BSARH / (KSARHON * cb + KSARHOFF);
  v.casarj = v.casar;
  v.casarhj = v.casarh;
  double roo2 = RATEDIMER / (1.0 + pow(KDIMER / (cjsr_b), HILLDIMER));
  double aub = (-1.0 + sqrt(1.0 + 8.0 * CSQBERS * roo2)) / (4.0 * roo2 * CSQBERS) / TAUB;
  double abu = 1.0 / TAUU;
  double fracbound = 1 / (1 + abu / aub);
  v.ncb = (int)(fracbound * NRYR);
  v.ncu = NRYR - (int)(fracbound * NRYR);
  v.nob = 0;
  v.nou = 0;
  v.lcc_lo = 0x03030303u;  // slots 0-3: state 3 (svncp = 4, :1153-1162)
  v.lcc_hi = 0x10101010u;  // slots 4-7: absent (16)
  return v;
}

rh_membrane initial_membrane(const rh_cell_params& p) {  // :346-365
  rh_membrane m{};
  m.t = 0.0;
  m.xnai = 6.1 * ((9000) / (p.pcl_ms + 5000));
  m.v = -80.00;
  m.xm = 0.0010;
  m.xh = 1.00;
  m.xj = 1.00;
  m.xr = 0.00;
  m.xs1 = 0.08433669901;
  m.xs2 = m.xs1;
  m.qks = 0.20;
  m.xtos = 0.010;
  m.ytos = 1.00;
  m.xtof = 0.020;
  m.ytof = 0.80;
  return m;
}

template <class R>
void carve(Lattice<R>& L, char*& p, int64_t S) {
  auto take = [&](size_t count) {
    R* r = reinterpret_cast<R*>(p);
    size_t b = (count * sizeof(R) + 255) & ~size_t(255);
    p += b;
    return r;
  };
  L.stride = S;
  L.cp = take(S);
  L.cjsr = take(S);
  L.cjsrb = take(S);
  L.ancx = take(S);
  L.casar = take(S);
  L.casarh = take(S);
  L.casarj = take(S);
  L.casarhj = take(S);
  L.cs[0] = take(S);
  L.cs[1] = take(S);
  L.ci[0] = take(8 * S);
  L.ci[1] = take(8 * S);
  L.cnsr[0] = take(8 * S);
  L.cnsr[1] = take(8 * S);
  L.catf = take(8 * S);
  L.cats = take(8 * S);
  L.cacal = take(8 * S);
  L.casr = take(8 * S);
  L.camyo = take(8 * S);
  L.mgmyo = take(8 * S);
  auto takeu = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~size_t(255);
    return r;
  };
  L.ryr = reinterpret_cast<uint32_t*>(takeu(S * 4));
  L.lcc = reinterpret_cast<uint2*>(takeu(S * 8));
  L.win = reinterpret_cast<uint32_t*>(takeu(S * 4));
}

// cuTensorMapEncodeTiled from the driver, looked up once per process.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn tensor_map_encoder() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
    else
      cudaGetLastError();
  });
  return fn;
}

// The tensor maps of the FP32 lattice's tensor-copy staging for tiles of
// `tile` CRUs.  The encoder checks the base addresses (256-byte aligned
// planes), the pitches (multiples of 256 bytes) and the boxes (at most 256
// elements a side, B x 8 or B x 4 bytes inner extent); the kernels' x
// coordinate, a tile's first arena index, is a multiple of 32.
bool build_stage_maps(const Lattice<float>& L, int64_t stride, int tile, StageMaps& m) {
  EncodeTiledFn enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t S = (cuuint64_t)stride;
  const cuuint32_t one[2] = {1, 1};
  // pair planes: 8-byte pairs, 4 planes of S pairs, 8 S bytes apart
  const cuuint64_t pdim[2] = {S, 4}, pstride[1] = {8 * S};
  const cuuint32_t pbox[2] = {(cuuint32_t)tile, 4};
  float* planes[4] = {L.ci[0], L.ci[1], L.cnsr[0], L.cnsr[1]};
  for (int i = 0; i < 4; ++i)
    if (enc(&m.plane[i], CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, planes[i], pdim, pstride, pbox, one,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  // the eight real planes cp .. casarhj, equally spaced
  const float* sc[8] = {L.cp, L.cjsr, L.cjsrb, L.ancx, L.casar, L.casarh, L.casarj, L.casarhj};
  const ptrdiff_t pitch = reinterpret_cast<const char*>(sc[1]) - reinterpret_cast<const char*>(sc[0]);
  for (int i = 1; i < 8; ++i)
    if (reinterpret_cast<const char*>(sc[i]) - reinterpret_cast<const char*>(sc[i - 1]) != pitch)
      return false;
  const cuuint64_t sdim[2] = {S, 8}, sstride[1] = {(cuuint64_t)pitch};
  const cuuint32_t sbox[2] = {(cuuint32_t)tile, 8};
  return enc(&m.sc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, L.cp, sdim, sstride, sbox, one,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
             CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t lattice_bytes(size_t rs, int64_t S) {
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  // 10 per-CRU real fields (cs twice), 10 sub-voxel fields (8 values per CRU,
  // ci and cnsr twice), packed integers
  return 10 * al(S * rs) + 10 * al(8 * S * rs) + al(S * 4) + al(S * 8) + al(S * 4);
}

template <class R>
StepArgs<R> make_args(rh_sim* s, const Lattice<R>& L, bool lattice_only) {
  StepArgs<R> a{};
  a.L = L;
  a.cells = s->sets[s->ts].d_cells;
  a.dyn = s->d_dyn;
  a.tiles = s->sets[s->ts].d_tiles;
  a.partials = s->d_partials;
  a.out_wc = s->d_out_wc;
  a.out_ls = s->d_out_ls;
  a.out_cd = s->d_out_cd;
  a.cd_cap = s->opts.cadist_capacity;
  a.diag = (lattice_only || s->opts.keep_diagnostics) ? s->d_diag : nullptr;
  a.stats = s->d_stats;
  a.stats_cap = s->opts.stats_capacity;
  a.out_cap = s->opts.output_capacity;
  a.lattice_only = lattice_only ? 1 : 0;
  a.dt = s->opts.dt_ms;
  return a;
}

// One group's step: the tiles of cells [group_cell[g], group_cell[g+1]),
// then the whole-cell update of those cells.
cudaError_t launch_group(rh_sim* s, int g, bool out, bool lattice_only, cudaStream_t st) {
  const rh_sim::TileSet& t = s->sets[s->ts];
  const int c0 = s->group_cell[g], c1 = s->group_cell[g + 1];
  const int tb = t.hcells[c0].tile_begin;
  const int te = c1 < s->ncells ? t.hcells[c1].tile_begin : t.ntiles;
  cudaError_t e;
  if (is_mixed(s)) {
    StepArgs<float> a = make_args(s, s->Lf, lattice_only);
    a.tiles += tb;
    a.tile_base = tb;
    if ((e = launch_step<float>(a, te - tb, out, s->group_opt[g], t.tile, s->staging,
                                &s->maps[s->ts], st)) != cudaSuccess)
      return e;
    return launch_cells<float>(a, c0, c1 - c0, out, t.tile, st);
  }
  StepArgs<double> a = make_args(s, s->Ld, lattice_only);
  a.tiles += tb;
  a.tile_base = tb;
  if ((e = launch_step<double>(a, te - tb, out, s->group_opt[g], t.tile, 0, nullptr, st)) !=
      cudaSuccess)
    return e;
  return launch_cells<double>(a, c0, c1 - c0, out, t.tile, st);
}

// The state of cells [c0, c1) between the device and a host image in the
// layout rh_export_state writes (the arena, then one CellDyn per cell): from
// `hin` to the device, or from the device to `hout`, on stream `st`.  Cells
// are consecutive in every plane of the arena, so a group's slice is the same
// CRU range of each plane: the 10 per-CRU real planes and the 40 sub-voxel
// pair planes are two strided copies (their planes are equally spaced), the
// packed integers three more, and the group's CellDyn records one.
cudaError_t copy_group_state(rh_sim* s, int c0, int c1, const char* hin, char* hout,
                             cudaStream_t st) {
  const size_t rs = real_size(s), S = (size_t)s->stride;
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t o0 = (size_t)s->hcells[c0].off;
  const size_t o1 = c1 < s->ncells ? (size_t)s->hcells[c1].off : S;
  const size_t sc_pitch = al(S * rs), pair_pitch = 2 * rs * S;
  const size_t sv_base = 10 * sc_pitch;
  const size_t ryr_base = sv_base + 10 * al(8 * S * rs);
  const size_t lcc_base = ryr_base + al(4 * S), win_base = lcc_base + al(8 * S);
  char* dev = reinterpret_cast<char*>(s->arena);
  const cudaMemcpyKind kind = hin ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  auto planes = [&](size_t base, size_t pitch, size_t esz, size_t rows) {
    const size_t off = base + esz * o0, w = esz * (o1 - o0);
    if (hin) return cudaMemcpy2DAsync(dev + off, pitch, hin + off, pitch, w, rows, kind, st);
    return cudaMemcpy2DAsync(hout + off, pitch, dev + off, pitch, w, rows, kind, st);
  };
  cudaError_t e;
  if ((e = planes(0, sc_pitch, rs, 10)) != cudaSuccess) return e;
  if ((e = planes(sv_base, pair_pitch, 2 * rs, 40)) != cudaSuccess) return e;
  if ((e = planes(ryr_base, 4 * S, 4, 1)) != cudaSuccess) return e;
  if ((e = planes(lcc_base, 8 * S, 8, 1)) != cudaSuccess) return e;
  if ((e = planes(win_base, 4 * S, 4, 1)) != cudaSuccess) return e;
  const size_t doff = s->arena_bytes + sizeof(CellDyn) * (size_t)c0;
  const size_t dbytes = sizeof(CellDyn) * (size_t)(c1 - c0);
  char* ddev = reinterpret_cast<char*>(s->d_dyn) + sizeof(CellDyn) * (size_t)c0;
  return hin ? cudaMemcpyAsync(ddev, hin + doff, dbytes, kind, st)
             : cudaMemcpyAsync(hout + doff, ddev, dbytes, kind, st);
}

// Host state image around a run of steps (rh_run_steps_host): imported at
// the head of the first window, exported at the tail of the last.
struct HostIO {
  const char* in = nullptr;
  char* out = nullptr;
};

// `n` steps of every group: group g's launches go to its own stream, forked
// from and joined back to the simulator's stream (inside a capture this
// makes one graph branch per group).  With `io`, group g's branch begins
// with the import of its cells' state and ends with their export, so that
// the copies of one group overlap the other groups' steps.
cudaError_t launch_steps(rh_sim* s, int n, const bool* outs, bool lattice_only,
                         const HostIO* io = nullptr) {
  const char* hin = io ? io->in : nullptr;
  char* hout = io ? io->out : nullptr;
  if (s->ngroups == 1) {
    cudaError_t e = cudaSuccess;
    if (hin) e = copy_group_state(s, 0, s->ncells, hin, nullptr, s->stream);
    for (int i = 0; i < n && e == cudaSuccess; ++i)
      e = launch_group(s, 0, outs[i], lattice_only, s->stream);
    if (hout && e == cudaSuccess) e = copy_group_state(s, 0, s->ncells, nullptr, hout, s->stream);
    return e;
  }
  cudaError_t e = cudaEventRecord(s->gevents[0], s->stream);
  for (int g = 0; g < s->ngroups && e == cudaSuccess; ++g) {
    const int c0 = s->group_cell[g], c1 = s->group_cell[g + 1];
    e = cudaStreamWaitEvent(s->gstreams[g], s->gevents[0], 0);
    if (hin && e == cudaSuccess) e = copy_group_state(s, c0, c1, hin, nullptr, s->gstreams[g]);
    for (int i = 0; i < n && e == cudaSuccess; ++i)
      e = launch_group(s, g, outs[i], lattice_only, s->gstreams[g]);
    if (hout && e == cudaSuccess) e = copy_group_state(s, c0, c1, nullptr, hout, s->gstreams[g]);
    if (e == cudaSuccess) e = cudaEventRecord(s->gevents[1 + g], s->gstreams[g]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->stream, s->gevents[1 + g], 0);
  }
  return e;
}

cudaError_t launch_one(rh_sim* s, bool out, bool lattice_only) {
  return launch_steps(s, 1, &out, lattice_only);
}

// Whether some cell uses a build option of the lattice update (perm, iso,
// slowncxchange, another NCX form).
bool any_options(const rh_sim* s) {
  for (char g : s->group_opt)
    if (g) return true;
  return false;
}

// Bytes of the synchronisation block of a persistent window launch: the
// per-cell words, then the update queue (head, tail and 2 * ncells slots of
// sequence number and cell).
size_t sync_bytes(int ncells) {
  return sizeof(CellSync) * (size_t)ncells + sizeof(unsigned int) * (2 + 4 * (size_t)ncells);
}

// Whether windows of steps run as one persistent launch: the run option, a
// tile length the window kernel is compiled for, and a device that can
// launch it cooperatively.
bool use_persist(const rh_sim* s) {
  const int tile = s->sets[s->ts].tile;
  return s->opts.persistent && s->persist_ok && (tile == 64 || tile == 128);
}

// `n` steps of every cell as one persistent launch: the synchronisation
// block is cleared first (a memset node in a captured window).  With
// no_output the steps write no output records (the autotuner's trials).
cudaError_t launch_persist(rh_sim* s, int n, bool no_output) {
  cudaError_t e = cudaMemsetAsync(s->d_sync, 0, sync_bytes(s->ncells), s->stream);
  if (e != cudaSuccess) return e;
  WindowCtl w{};
  w.sync = s->d_sync;
  w.error = s->d_err;
  w.steps = n;
  w.ntiles = s->sets[s->ts].ntiles;
  w.wait_limit = s->wait_limit;
  w.wait_offset = s->wait_offset;
  unsigned int* q = reinterpret_cast<unsigned int*>(s->d_sync + s->ncells);
  w.q_cap = 2 * s->ncells;
  w.q_head = q;
  w.q_tail = q + 1;
  w.q_seq = q + 2;
  w.q_cell = reinterpret_cast<int*>(q + 2 + w.q_cap);
  const bool opt = any_options(s);
  const int tile = s->sets[s->ts].tile;
  if (is_mixed(s)) {
    StepArgs<float> a = make_args(s, s->Lf, false);
    a.no_output = no_output ? 1 : 0;
    return launch_window<float>(a, w, opt, tile, s->fewer_ctas, s->stream);
  }
  StepArgs<double> a = make_args(s, s->Ld, false);
  a.no_output = no_output ? 1 : 0;
  return launch_window<double>(a, w, opt, tile, s->fewer_ctas, s->stream);
}

// Reads and clears the wait-timeout flag of the persistent launches (the
// stream is synchronised first).
int check_wait_error(rh_sim* s) {
  if (!s->d_err) return RH_OK;
  CK(cudaMemcpyAsync(s->h_err, s->d_err, sizeof(unsigned int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (*s->h_err) {
    *s->h_err = 0;
    CK(cudaMemsetAsync(s->d_err, 0, sizeof(unsigned int), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return fail(s, RH_ERR_TIMEOUT,
                "a wait of the persistent window launch ran out (cells flagged "
                "RH_STATUS_TIMEOUT); the lattice state is left part-way through a step");
  }
  return RH_OK;
}

bool out_step_host(double t, double dt) { return fmod(t + 0.0000001, OUTT) < dt; }

// Splits the cells into `want` groups of about equal CRU count (never more
// groups than cells), each with its own stream for the two-launch path.
int set_groups(rh_sim* s, int want) {
  const int ncells = s->ncells;
  want = std::max(1, std::min(want, ncells));
  for (cudaStream_t st : s->gstreams)
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t ev : s->gevents)
    if (ev) cudaEventDestroy(ev);
  s->gstreams.clear();
  s->gevents.clear();
  int64_t total = 0;
  for (const CellConst& c : s->hcells) total += c.n;
  s->group_cell.assign(1, 0);
  int64_t acc = 0;
  for (int c = 0; c < ncells; ++c) {
    acc += s->hcells[c].n;
    const int g = (int)s->group_cell.size();  // next boundary index
    if (g < want && c + 1 < ncells && acc * want >= total * g) s->group_cell.push_back(c + 1);
  }
  s->ngroups = (int)s->group_cell.size();
  s->group_cell.push_back(ncells);
  s->group_opt.assign(s->ngroups, 0);
  for (int g = 0; g < s->ngroups; ++g)
    for (int c = s->group_cell[g]; c < s->group_cell[g + 1]; ++c)
      if (cell_uses_options(s->hcells[c])) s->group_opt[g] = 1;
  if (s->ngroups > 1) {
    s->gstreams.resize(s->ngroups);
    s->gevents.resize(s->ngroups + 1);
    for (auto& st : s->gstreams) CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    for (auto& ev : s->gevents) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  return RH_OK;
}

int ensure_diag(rh_sim* s) {
  if (s->d_diag) return RH_OK;
  CK(cudaMalloc(&s->d_diag, sizeof(double) * D_COUNT * (size_t)s->stride));
  CK(cudaMemsetAsync(s->d_diag, 0, sizeof(double) * D_COUNT * (size_t)s->stride, s->stream));
  return RH_OK;
}

void timing_begin(rh_sim* s) {
  if (!s->timing_open) {
    cudaEventRecord(s->ev0, s->stream);
    s->timing_open = true;
  }
}

void timing_end(rh_sim* s, long long nl) {
  cudaEventRecord(s->ev1, s->stream);
  s->launches_pending += nl;
}

int check_cell(rh_sim* s, int32_t cell) {
  if (!s) return RH_ERR_ARG;
  if (cell < 0 || cell >= s->ncells) return fail(s, RH_ERR_ARG, "cell %d out of range", cell);
  return RH_OK;
}

// Runs `n` steps in one window: replays (or captures) the graph for this
// window's pattern of output steps.
int run_window(rh_sim* s, int n, const std::vector<bool>& outs, const HostIO* io = nullptr) {
  const bool persist = use_persist(s);
  if (persist) io = nullptr;  // the persistent path imports and exports around the window
  if (persist && !s->persist_graph) {  // this device could not capture it: launch directly
    CK(launch_persist(s, n, false));
    return RH_OK;
  }
  // a persistent window reads its output steps on the device: one graph per length
  const void* kin = io ? io->in : nullptr;
  void* kout = io ? io->out : nullptr;
  auto key = persist ? std::make_tuple(-n, std::vector<bool>(), kin, kout)
                     : std::make_tuple(n, outs, kin, kout);
  auto it = s->graphs.find(key);
  cudaGraphExec_t exec = nullptr;
  if (it == s->graphs.end()) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    std::unique_ptr<bool[]> o(new bool[n]);
    for (int i = 0; i < n; ++i) o[i] = outs[i];
    cudaError_t le = persist ? launch_persist(s, n, false) : launch_steps(s, n, o.get(), false, io);
    cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
    cudaError_t ie = cudaErrorUnknown;
    if (le == cudaSuccess && ce == cudaSuccess) {
      // Per-node priorities: without this flag a graph launch runs every
      // node at the priority of the stream it is launched into, and the
      // cell updates' launch priority is lost (measured on the 512-cell
      // ensemble: 0.510 against 0.520 ms per update of every cell).
      ie = cudaGraphInstantiate(&exec, g, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(g);
      g = nullptr;
    }
    if (persist && ie != cudaSuccess) {
      // the cooperative launch could not be captured here: launch windows directly
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      s->persist_graph = false;
      CK(launch_persist(s, n, false));
      return RH_OK;
    }
    if (le != cudaSuccess) return fail(s, RH_ERR_CUDA, "launch during capture: %s", cudaGetErrorString(le));
    if (ce != cudaSuccess) return fail(s, RH_ERR_CUDA, "capture: %s", cudaGetErrorString(ce));
    CK(ie);
    if (s->graphs.size() > 64) {  // bound the cache
      for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
      s->graphs.clear();
    }
    s->graphs[key] = exec;
  } else {
    exec = it->second;
  }
  CK(cudaGraphLaunch(exec, s->stream));
  return RH_OK;
}

}  // namespace

// ------------------------------------------------------------------ ABI

extern "C" {

void rh_default_cell_params(rh_cell_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->nx = 64;
  p->ny = 28;
  p->nz = 12;
  p->nbeats = 7;
  p->pcl_ms = 4000.0;
  p->clamp_mv = 1.0;
  p->cjsr_basal = 740.0;
  p->ncx_scale = 1.0;
  p->ku = 3.333;
  p->r1 = 0.0;
  p->kb = 18.0;
  p->ica_scale = 0.7;
  p->ku2 = 1.0;
  p->ikr_scale = 1.0;
  p->cao_mM = 1.8;
  p->lqt = 1;
  p->iso2 = 1;
  p->tapsi = 0;
  p->seed = 18;
  p->cell_id = 0;
  p->linescan_jz = -1;
  p->protocol = RH_PROTO_PACED;
  p->perm = 0;
  p->iso = 0;
  p->randomlcc = 0;
  p->slowncx = 0;
  p->ncx_form = RH_NCX_ALLOSTERIC;
}

void rh_default_run_opts(rh_run_opts* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->precision = RH_FP64;
  o->device = 0;
  o->dt_ms = 0.025;
  o->block_size = 0;
  o->output_capacity = 64;
  o->record_linescan = 1;
  o->track_stats = 1;
  o->stats_capacity = 64;
  o->keep_diagnostics = 0;
  o->window_steps = 100;
  o->persistent = 0;
}

static thread_local std::string g_create_error;

static int create_impl(rh_sim* s, const rh_cell_params* cells, int32_t ncells,
                       const rh_run_opts* opts);

int rh_create(const rh_cell_params* cells, int32_t ncells, const rh_run_opts* opts, rh_sim** out) {
  if (!out) return RH_ERR_ARG;
  *out = nullptr;
  g_create_error.clear();
  if (!cells || ncells <= 0) {
    g_create_error = "no cells";
    return RH_ERR_ARG;
  }
  rh_sim* s = new rh_sim();
  int r = create_impl(s, cells, ncells, opts);
  if (r != RH_OK) {
    g_create_error = s->err.empty() ? "invalid argument" : s->err;
    rh_destroy(s);
    return r;
  }
  *out = s;
  return RH_OK;
}

static int create_impl(rh_sim* s, const rh_cell_params* cells, int32_t ncells,
                       const rh_run_opts* opts) {
  if (opts) s->opts = *opts;
  else rh_default_run_opts(&s->opts);
  if (s->opts.output_capacity <= 0) s->opts.output_capacity = 64;
  if (s->opts.window_steps <= 0) s->opts.window_steps = 100;
  if (s->opts.stats_capacity <= 0) s->opts.stats_capacity = 64;
  if (s->opts.cadist_capacity <= 0) s->opts.cadist_capacity = 8;
  if (!(s->opts.dt_ms > 0)) return fail(s, RH_ERR_ARG, "dt_ms must be positive");
  if (s->opts.precision != RH_FP64 && s->opts.precision != RH_MIXED)
    return fail(s, RH_ERR_ARG, "unknown precision %d", s->opts.precision);
  s->ncells = ncells;
  s->params.assign(cells, cells + ncells);
  // layout
  int64_t off = 0;
  int64_t ls_off = 0;
  int64_t cd_off = 0;
  for (int c = 0; c < ncells; ++c) {
    const rh_cell_params& p = cells[c];
    if (p.nx < 3 || p.ny < 3 || p.nz < 3 || p.nx > 4096 || p.ny > 4096 || p.nz > 4096)
      return fail(s, RH_ERR_ARG, "cell %d: lattice %dx%dx%d outside 3..4096", c, p.nx, p.ny, p.nz);
    if (!(p.pcl_ms > 0) || p.nbeats < 0)
      return fail(s, RH_ERR_ARG, "cell %d: bad protocol (pcl %g, beats %d)", c, p.pcl_ms, p.nbeats);
    int64_t n64 = (int64_t)(p.nx - 2) * (p.ny - 2) * (p.nz - 2);
    if (n64 > (1 << 30)) return fail(s, RH_ERR_ARG, "cell %d: lattice too large", c);
    CellConst cc{};
    cc.lx = p.nx - 2;
    cc.ly = p.ny - 2;
    cc.lz = p.nz - 2;
    cc.nxf = p.nx;
    cc.nyf = p.ny;
    cc.n = (int)n64;
    cc.off = off;
    int jz = p.linescan_jz < 0 ? 5 : p.linescan_jz;
    if (jz > p.nz - 2) jz = p.nz / 2;
    if (jz < 1) jz = 1;
    cc.line_z = jz - 1;
    cc.line_y = p.ny / 2 - 1;
    cc.iso2 = p.iso2 ? 1 : 0;
    cc.seed = p.seed;
    cc.cell_id = p.cell_id;
    cc.ls_off = ls_off;
    cc.cd_off = cd_off;
    cc.svica = ((0.666) * (1.2) * (p.ica_scale));
    cc.svncx = (2.5 * p.ncx_scale);
    double sviup = (1.0 + 0.75);
    if (p.iso2) sviup = (1.0 + 0.75) * 1.75;
    if (p.tapsi) sviup = 0;
    double sviup_lqt = (p.lqt && p.tapsi) ? 0.05 : 0.;
    cc.sviup_tot = sviup + sviup_lqt;
    // iso doubles SERCA from 5.5 PCL on; iso2 and tapsi still override (:1220-1238)
    double sviup_iso = p.iso2 ? (1.0 + 0.75) * 1.75 : (1.0 + 0.75) * 2.;
    if (p.tapsi) sviup_iso = 0;
    cc.sviup_iso = sviup_iso + sviup_lqt;
    if (p.ncx_form < RH_NCX_ALLOSTERIC || p.ncx_form > RH_NCX_NOALLO)
      return fail(s, RH_ERR_ARG, "cell %d: unknown NCX form %d", c, p.ncx_form);
    cc.iso = p.iso ? 1 : 0;
    cc.randomlcc = p.randomlcc ? 1 : 0;
    cc.slowncx = p.slowncx ? 1 : 0;
    cc.ncx_form = p.ncx_form;
    cc.svikr = p.lqt ? 0 : 3 * p.ikr_scale;
    cc.cao = p.cao_mM;
    cc.ku = p.ku;
    cc.ku2 = p.ku2;
    cc.kb = p.kb;
    cc.pcl = p.pcl_ms;
    cc.tend = p.nbeats * p.pcl_ms + 2100;
    if (p.protocol < RH_PROTO_PACED || p.protocol > RH_PROTO_LINEAR_AP_CLAMP)
      return fail(s, RH_ERR_ARG, "cell %d: unknown protocol %d", c, p.protocol);
    cc.perm = p.perm ? 1 : 0;
    cc.protocol = p.protocol;
    cc.clamp_mv = p.clamp_mv;
    cc.apv = nullptr;  // rh_set_ap_clamp
    cc.napv = p.protocol == RH_PROTO_AP_CLAMP ? (int)(p.pcl_ms / s->opts.dt_ms + 0.1) : 0;
    if (p.protocol == RH_PROTO_AP_CLAMP && cc.napv < 1)
      return fail(s, RH_ERR_ARG, "cell %d: AP clamp needs pcl_ms >= dt", c);
    off += (n64 + 31) & ~int64_t(31);
    if (s->opts.record_linescan) ls_off += (int64_t)s->opts.output_capacity * cc.lx;
    if (s->opts.record_cadist)
      cd_off += (int64_t)s->opts.cadist_capacity * (2 + RH_CADIST_COLS * n64);
    s->max_n = std::max(s->max_n, cc.n);
    s->hcells.push_back(cc);
  }
  int max_tiles = 0;
  for (int k = 0; k < kNumTileSizes; ++k) {
    rh_sim::TileSet& t = s->sets[k];
    t.tile = kTileSizes[k];
    t.hcells = s->hcells;
    int nt = 0;
    for (int c = 0; c < ncells; ++c) {
      CellConst& cc = t.hcells[c];
      cc.tile_begin = nt;
      cc.tile_count = (cc.n + t.tile - 1) / t.tile;
      for (int q = 0; q < cc.tile_count; ++q)
        t.htiles.push_back(make_int4(c, q * t.tile, std::min(t.tile, cc.n - q * t.tile),
                                     (int)(cc.off + (int64_t)q * t.tile)));
      nt += cc.tile_count;
    }
    t.ntiles = nt;
    max_tiles = std::max(max_tiles, nt * (t.tile / 32));  // partial rows: one per warp
  }
  {
    int want = s->opts.block_size > 0 ? s->opts.block_size : kDefaultTile;
    s->ts = -1;
    for (int k = 0; k < kNumTileSizes; ++k)
      if (kTileSizes[k] == want) s->ts = k;
    if (s->ts < 0) return fail(s, RH_ERR_ARG, "block_size %d is not a compiled tile length", want);
  }
  s->hcells = s->sets[s->ts].hcells;
  // the step kernel indexes the arena with 32-bit element offsets (8 per CRU)
  if (off > ((int64_t)1 << 29))
    return fail(s, RH_ERR_ARG, "ensemble too large (%lld CRUs, at most 2^29)", (long long)off);
  s->stride = off;
  s->ls_rows_total = ls_off;
  s->device = s->opts.device;
  CK(cudaSetDevice(s->device));
  CK(prepare_step_kernels());
  CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  {
    int r = set_groups(s, s->opts.cell_groups > 0 ? s->opts.cell_groups : kDefaultGroups);
    if (r) return r;
  }
  CK(cudaEventCreate(&s->ev0));
  CK(cudaEventCreate(&s->ev1));
  s->arena_bytes = lattice_bytes(real_size(s), s->stride);
  if (cudaMalloc(&s->arena, s->arena_bytes) != cudaSuccess) {
    cudaGetLastError();
    s->arena = nullptr;
    return fail(s, RH_ERR_NOMEM, "cannot allocate %zu bytes of lattice state", s->arena_bytes);
  }
  char* p = reinterpret_cast<char*>(s->arena);
  if (is_mixed(s)) carve(s->Lf, p, s->stride);
  else carve(s->Ld, p, s->stride);
  if (is_mixed(s)) {
    s->maps_ok = true;
    for (int k = 0; k < kNumTileSizes; ++k)
      s->maps_ok = s->maps_ok && build_stage_maps(s->Lf, s->stride, kTileSizes[k], s->maps[k]);
  }
  CK(cudaMalloc(&s->d_dyn, sizeof(CellDyn) * ncells));
  for (int k = 0; k < kNumTileSizes; ++k) {
    rh_sim::TileSet& t = s->sets[k];
    CK(cudaMalloc(&t.d_cells, sizeof(CellConst) * ncells));
    CK(cudaMalloc(&t.d_tiles, sizeof(int4) * t.ntiles));
    CK(cudaMemcpyAsync(t.d_cells, t.hcells.data(), sizeof(CellConst) * ncells,
                       cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(t.d_tiles, t.htiles.data(), sizeof(int4) * t.ntiles,
                       cudaMemcpyHostToDevice, s->stream));
  }
  CK(cudaMalloc(&s->d_partials, sizeof(double) * P_COUNT * (size_t)max_tiles));
  CK(cudaMalloc(&s->d_sync, sync_bytes(ncells)));
  CK(cudaMalloc(&s->d_err, sizeof(unsigned int)));
  CK(cudaMemsetAsync(s->d_err, 0, sizeof(unsigned int), s->stream));
  CK(cudaMallocHost(&s->h_err, sizeof(unsigned int)));
  *s->h_err = 0;
  {  // can this device run the persistent window kernel (cooperatively)?
    int ctas = 0;
    const cudaError_t we = is_mixed(s) ? window_grid<float>(128, false, false, &ctas)
                                       : window_grid<double>(128, false, false, &ctas);
    s->persist_ok = we == cudaSuccess && ctas > 0;
    if (we != cudaSuccess) cudaGetLastError();
  }
  CK(cudaMalloc(&s->d_out_wc, sizeof(double) * RH_WHOLECELL_COLS * (size_t)ncells *
                                  s->opts.output_capacity));
  if (s->opts.record_linescan)  // the reference's outputlinescan switch (:46, :967)
    CK(cudaMalloc(&s->d_out_ls, sizeof(double) * RH_LINESCAN_COLS * (size_t)std::max<int64_t>(ls_off, 1)));
  if (s->opts.record_cadist) {
    if (cudaMalloc(&s->d_out_cd, sizeof(double) * (size_t)cd_off) != cudaSuccess) {
      cudaGetLastError();
      s->d_out_cd = nullptr;
      return fail(s, RH_ERR_NOMEM, "cannot allocate %lld cadist values", (long long)cd_off);
    }
  }
  if (s->opts.track_stats)
    CK(cudaMalloc(&s->d_stats, sizeof(rh_beat_stats) * (size_t)ncells * s->opts.stats_capacity));
  // cells' basal state and membrane initial conditions
  std::vector<InitValues> iv(ncells);
  std::vector<CellDyn> dyn(ncells);
  s->t_host.resize(ncells);
  s->active_host.resize(ncells);
  s->drained_wc.assign(ncells, 0);
  s->drained_ls.assign(ncells, 0);
  s->drained_st.assign(ncells, 0);
  s->drained_cd.assign(ncells, 0);
  for (int c = 0; c < ncells; ++c) {
    iv[c] = init_values(cells[c]);
    memset(&dyn[c], 0, sizeof(CellDyn));
    dyn[c].m = initial_membrane(cells[c]);
    beat_reset(dyn[c].bt);
    s->t_host[c] = dyn[c].m.t;
    s->active_host[c] = dyn[c].m.t < s->hcells[c].tend;
  }
  InitValues* d_iv = nullptr;
  CK(cudaMalloc(&d_iv, sizeof(InitValues) * ncells));
  CK(cudaMemcpyAsync(d_iv, iv.data(), sizeof(InitValues) * ncells, cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemcpyAsync(s->d_dyn, dyn.data(), sizeof(CellDyn) * ncells, cudaMemcpyHostToDevice, s->stream));
  const CellConst* dcells = s->sets[s->ts].d_cells;
  if (is_mixed(s)) CK(launch_init<float>(s->Lf, dcells, d_iv, ncells, s->max_n, s->stream));
  else CK(launch_init<double>(s->Ld, dcells, d_iv, ncells, s->max_n, s->stream));
  CK(launch_volt_prep(dcells, s->d_dyn, ncells, s->opts.dt_ms, s->stream));
  if (s->opts.keep_diagnostics) {
    int r = ensure_diag(s);
    if (r) return r;
  }
  CK(cudaStreamSynchronize(s->stream));
  cudaFree(d_iv);
  return RH_OK;
}

int rh_destroy(rh_sim* s) {
  if (!s) return RH_ERR_ARG;
  if (s->stream) {
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
  }
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  cudaFree(s->arena);
  for (auto& t : s->sets) {
    cudaFree(t.d_cells);
    cudaFree(t.d_tiles);
  }
  cudaFree(s->d_dyn);
  cudaFree(s->d_partials);
  cudaFree(s->d_sync);
  cudaFree(s->d_err);
  if (s->h_err) cudaFreeHost(s->h_err);
  cudaFree(s->d_out_wc);
  cudaFree(s->d_out_ls);
  cudaFree(s->d_out_cd);
  for (double* w : s->d_apv) cudaFree(w);
  cudaFree(s->d_diag);
  cudaFree(s->d_stats);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
  for (cudaStream_t st : s->gstreams)
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t ev : s->gevents)
    if (ev) cudaEventDestroy(ev);
  delete s;
  return RH_OK;
}

namespace {

// Whether `p` is host memory the GPU can copy from asynchronously (pinned or
// registered); NULL counts as such.
bool host_pinned(const void* p) {
  if (!p) return true;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// The strided group copies take the 40 sub-voxel pair planes as equally
// spaced, which holds when a sub-voxel field fills whole 256-byte blocks.
bool group_copies_ok(const rh_sim* s) {
  return ((8 * (size_t)s->stride * real_size(s)) % 256) == 0;
}

// Checks a host state image and points the host mirrors (time, activity,
// drained records) at the state it holds.
int import_mirrors(rh_sim* s, const char* h) {
  const CellDyn* dyn = reinterpret_cast<const CellDyn*>(h + s->arena_bytes);
  for (int c = 0; c < s->ncells; ++c)
    if (dyn[c].arrive != 0) return fail(s, RH_ERR_ARG, "import block is not an exported state");
  for (int c = 0; c < s->ncells; ++c) {
    s->t_host[c] = dyn[c].m.t;
    s->active_host[c] = !dyn[c].done;
    s->drained_wc[c] = std::min(s->drained_wc[c], dyn[c].out_count);
    s->drained_ls[c] = std::min(s->drained_ls[c], dyn[c].out_count);
    s->drained_st[c] = std::min(s->drained_st[c], dyn[c].stats_count);
    s->drained_cd[c] = std::min(s->drained_cd[c], dyn[c].cd_count);
  }
  return RH_OK;
}

cudaError_t copy_state_in(rh_sim* s, const char* h) {
  cudaError_t e = cudaMemcpyAsync(s->arena, h, s->arena_bytes, cudaMemcpyHostToDevice, s->stream);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(s->d_dyn, h + s->arena_bytes, sizeof(CellDyn) * s->ncells,
                         cudaMemcpyHostToDevice, s->stream);
}

cudaError_t copy_state_out(rh_sim* s, char* h) {
  cudaError_t e = cudaMemcpyAsync(h, s->arena, s->arena_bytes, cudaMemcpyDeviceToHost, s->stream);
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(h + s->arena_bytes, s->d_dyn, sizeof(CellDyn) * s->ncells,
                         cudaMemcpyDeviceToHost, s->stream);
}

// rh_run_steps, optionally with the state imported from `hin` first and
// exported to `hout` after (rh_run_steps_host).  On the two-launch path with
// pinned buffers the copies ride in the first and the last window, per cell
// group; otherwise they run before and after the steps.
int run_steps_impl(rh_sim* s, int64_t nsteps, const char* hin, char* hout) {
  if (!s || nsteps < 0) return RH_ERR_ARG;
  if (!s->stream) return fail(s, RH_ERR_STATE, "simulator not initialised");
  CK(cudaSetDevice(s->device));
  const bool pipe = (hin || hout) && !use_persist(s) && group_copies_ok(s) && host_pinned(hin) &&
                    host_pinned(hout);
  if (hin) {
    int r = import_mirrors(s, hin);
    if (r) return r;
  }
  for (int c = 0; c < s->ncells; ++c)
    if (s->active_host[c] && s->hcells[c].protocol == RH_PROTO_AP_CLAMP && !s->hcells[c].apv)
      return fail(s, RH_ERR_STATE, "cell %d: AP-clamp waveform not set (rh_set_ap_clamp)", c);
  if (s->opts.keep_diagnostics) {
    int r = ensure_diag(s);
    if (r) return r;
  }
  if (hin && !pipe) CK(copy_state_in(s, hin));
  bool in_pending = hin && pipe, out_pending = hout != nullptr;
  const double dt = s->opts.dt_ms;
  const int W = s->opts.window_steps;
  int64_t done = 0;
  timing_begin(s);
  long long nlaunch = 0;
  while (done < nsteps) {
    // plan the next window from the host clock mirror
    int n = (int)std::min<int64_t>(W, nsteps - done);
    std::vector<bool> outs;
    outs.reserve(n);
    int k = 0;
    for (; k < n; ++k) {
      bool any_active = false, out = false;
      for (int c = 0; c < s->ncells; ++c) {
        if (!s->active_host[c]) continue;
        any_active = true;
        if (out_step_host(s->t_host[c], dt)) out = true;
      }
      if (!any_active) break;
      outs.push_back(out);
      for (int c = 0; c < s->ncells; ++c) {
        if (!s->active_host[c]) continue;
        s->t_host[c] = s->t_host[c] + dt;
        if (!(s->t_host[c] < s->hcells[c].tend)) s->active_host[c] = 0;
      }
    }
    if (k == 0) break;
    bool any_left = false;
    for (int c = 0; c < s->ncells; ++c) any_left = any_left || s->active_host[c];
    HostIO io;
    if (in_pending) io.in = hin;
    if (pipe && hout && (done + k >= nsteps || !any_left)) io.out = hout;
    const HostIO* iop = (io.in || io.out) ? &io : nullptr;
    int r;
    const bool persist = use_persist(s);
    if (k == W) {
      r = run_window(s, k, outs, iop);
    } else {
      r = RH_OK;
      std::unique_ptr<bool[]> o(new bool[k]);
      for (int i = 0; i < k; ++i) o[i] = outs[i];
      cudaError_t e = persist ? launch_persist(s, k, false) : launch_steps(s, k, o.get(), false, iop);
      if (e != cudaSuccess) return fail(s, RH_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    }
    if (r) return r;
    if (io.in) in_pending = false;
    if (io.out) out_pending = false;
    s->kernels += persist ? 1 : 2LL * s->ngroups * k;
    nlaunch += k;
    done += k;
  }
  if (in_pending) CK(copy_state_in(s, hin));  // no step ran
  if (out_pending) CK(copy_state_out(s, hout));
  timing_end(s, nlaunch);
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaGetLastError());
  return check_wait_error(s);
}

}  // namespace

int rh_run_steps(rh_sim* s, int64_t nsteps) { return run_steps_impl(s, nsteps, nullptr, nullptr); }

int rh_run_steps_host(rh_sim* s, int64_t nsteps, const void* host_in, void* host_out,
                      size_t bytes) {
  if (!s || nsteps < 0) return RH_ERR_ARG;
  if ((host_in || host_out) && bytes != s->arena_bytes + sizeof(CellDyn) * (size_t)s->ncells)
    return fail(s, RH_ERR_ARG, "state buffers must hold rh_state_bytes() bytes");
  return run_steps_impl(s, nsteps, reinterpret_cast<const char*>(host_in),
                        reinterpret_cast<char*>(host_out));
}

int rh_run_to_end(rh_sim* s) {
  if (!s) return RH_ERR_ARG;
  int64_t most = 0;
  for (int c = 0; c < s->ncells; ++c) {
    if (!s->active_host[c]) continue;
    double rem = (s->hcells[c].tend - s->t_host[c]) / s->opts.dt_ms;
    most = std::max<int64_t>(most, (int64_t)rem + 2);
  }
  return rh_run_steps(s, most);
}

int rh_lattice_step(rh_sim* s) {
  if (!s || !s->stream) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  int r = ensure_diag(s);
  if (r) return r;
  CK(launch_one(s, false, true));
  CK(cudaStreamSynchronize(s->stream));
  return RH_OK;
}

int rh_set_ap_clamp(rh_sim* s, int32_t cell, const double* v, int64_t n) {
  int r = check_cell(s, cell);
  if (r) return r;
  const CellConst& cc = s->hcells[cell];
  if (cc.protocol != RH_PROTO_AP_CLAMP)
    return fail(s, RH_ERR_ARG, "cell %d: protocol is not RH_PROTO_AP_CLAMP", cell);
  if (!v || n != cc.napv)
    return fail(s, RH_ERR_ARG, "cell %d: AP-clamp waveform needs %d samples (pcl/dt), got %lld",
                cell, cc.napv, (long long)n);
  for (int64_t k = 0; k < n; ++k)
    if (!std::isfinite(v[k])) return fail(s, RH_ERR_ARG, "cell %d: sample %lld is not finite",
                                          cell, (long long)k);
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  if (s->d_apv.empty()) s->d_apv.assign(s->ncells, nullptr);
  if (!s->d_apv[cell]) CK(cudaMalloc(&s->d_apv[cell], sizeof(double) * (size_t)n));
  CK(cudaMemcpy(s->d_apv[cell], v, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
  // every tile layout's copy of the cell constants points at the waveform
  for (int k = 0; k < kNumTileSizes; ++k) {
    rh_sim::TileSet& t = s->sets[k];
    t.hcells[cell].apv = s->d_apv[cell];
    CK(cudaMemcpy(t.d_cells + cell, &t.hcells[cell], sizeof(CellConst), cudaMemcpyHostToDevice));
  }
  s->hcells[cell].apv = s->d_apv[cell];
  return RH_OK;
}

int rh_num_cells(const rh_sim* s, int32_t* n) {
  if (!s || !n) return RH_ERR_ARG;
  *n = s->ncells;
  return RH_OK;
}

int rh_cell_size(const rh_sim* s, int32_t cell, int32_t* n) {
  if (!s || !n || cell < 0 || cell >= s->ncells) return RH_ERR_ARG;
  *n = s->hcells[cell].n;
  return RH_OK;
}

}  // extern "C"

namespace {

template <class R>
int get_state_t(rh_sim* s, const Lattice<R>& L, int cell, int par, rh_state_f64* d) {
  const CellConst& cc = s->hcells[cell];
  const int n = cc.n;
  const int64_t S = s->stride;
  std::vector<R> buf(8 * (size_t)n);
  // per-CRU fields: one plane; per-sub-voxel fields: 4 pair planes, each a
  // contiguous run of 2n values (sub_index), de-interleaved into 8 planes
  auto pull = [&](const R* src, double* dst, int planes) -> int {
    if (!dst) return RH_OK;
    if (planes == 1) {
      CK(cudaMemcpyAsync(buf.data(), src + cc.off, sizeof(R) * n, cudaMemcpyDeviceToHost,
                         s->stream));
    } else {
      for (int p = 0; p < 4; ++p)
        CK(cudaMemcpyAsync(buf.data() + (size_t)p * 2 * n, src + sub_index(2 * p, cc.off, S),
                           sizeof(R) * 2 * n, cudaMemcpyDeviceToHost, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    if (planes == 1) {
      for (size_t q = 0; q < (size_t)n; ++q) dst[q] = (double)buf[q];
    } else {
      for (int ii = 0; ii < 8; ++ii)
        for (size_t q = 0; q < (size_t)n; ++q)
          dst[(size_t)ii * n + q] = (double)buf[(size_t)(ii >> 1) * 2 * n + 2 * q + (ii & 1)];
    }
    return RH_OK;
  };
  int r;
  if ((r = pull(L.cp, d->cp, 1)) || (r = pull(L.cs[par], d->cs, 1)) ||
      (r = pull(L.cjsr, d->cjsr, 1)) || (r = pull(L.cjsrb, d->cjsrb, 1)) ||
      (r = pull(L.ancx, d->ancx, 1)) || (r = pull(L.casar, d->casar, 1)) ||
      (r = pull(L.casarh, d->casarh, 1)) || (r = pull(L.casarj, d->casarj, 1)) ||
      (r = pull(L.casarhj, d->casarhj, 1)) || (r = pull(L.ci[par], d->ci, 8)) ||
      (r = pull(L.cnsr[par], d->cnsr, 8)) || (r = pull(L.catf, d->catf, 8)) ||
      (r = pull(L.cats, d->cats, 8)) || (r = pull(L.cacal, d->cacal, 8)) ||
      (r = pull(L.casr, d->casr, 8)) || (r = pull(L.camyo, d->camyo, 8)) ||
      (r = pull(L.mgmyo, d->mgmyo, 8)))
    return r;
  std::vector<uint32_t> ryr(n), win(n);
  std::vector<uint2> lcc(n);
  CK(cudaMemcpyAsync(ryr.data(), L.ryr + cc.off, 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaMemcpyAsync(win.data(), L.win + cc.off, 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaMemcpyAsync(lcc.data(), L.lcc + cc.off, 8 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  for (int q = 0; q < n; ++q) {
    if (d->nou) d->nou[q] = ryr[q] & 0xff;
    if (d->ncu) d->ncu[q] = (ryr[q] >> 8) & 0xff;
    if (d->nob) d->nob[q] = (ryr[q] >> 16) & 0xff;
    if (d->ncb) d->ncb[q] = ryr[q] >> 24;
    if (d->nl) d->nl[q] = win[q] & 0xffff;
    if (d->nspark) d->nspark[q] = win[q] >> 16;
    if (d->lcc)
      for (int ll = 0; ll < 8; ++ll)
        d->lcc[(size_t)ll * n + q] = ((ll < 4 ? lcc[q].x : lcc[q].y) >> ((ll & 3) * 8)) & 0xff;
  }
  // diagnostics of the last lattice update
  double* dplanes[D_COUNT];
  for (int k = 0; k < D_COUNT; ++k) dplanes[k] = nullptr;
  if (s->d_diag) {
    std::vector<double> tmp(n);
    auto pd = [&](int plane, double* dst) -> int {
      if (!dst) return RH_OK;
      CK(cudaMemcpy(dst, s->d_diag + (int64_t)plane * S + cc.off, sizeof(double) * n,
                    cudaMemcpyDeviceToHost));
      return RH_OK;
    };
    if ((r = pd(D_XIRE, d->xire)) || (r = pd(D_PO, d->po)) || (r = pd(D_XINACA, d->xinaca)) ||
        (r = pd(D_XICAT, d->xicat)))
      return r;
    for (int ii = 0; ii < 8; ++ii) {
      if ((r = pd(D_XIUP + ii, d->xiup ? d->xiup + (size_t)ii * n : nullptr)) ||
          (r = pd(D_XILEAK + ii, d->xileak ? d->xileak + (size_t)ii * n : nullptr)))
        return r;
    }
  }
  return RH_OK;
}

template <class R>
int set_state_t(rh_sim* s, const Lattice<R>& L, int cell, int par, const rh_state_f64* d) {
  const CellConst& cc = s->hcells[cell];
  const int n = cc.n;
  const int64_t S = s->stride;
  std::vector<R> buf(8 * (size_t)n);
  auto push = [&](R* dst, const double* src, int planes) -> int {
    if (!src) return RH_OK;
    if (planes == 1) {
      for (size_t q = 0; q < (size_t)n; ++q) buf[q] = (R)src[q];
      CK(cudaMemcpyAsync(dst + cc.off, buf.data(), sizeof(R) * n, cudaMemcpyHostToDevice,
                         s->stream));
    } else {
      for (int ii = 0; ii < 8; ++ii)
        for (size_t q = 0; q < (size_t)n; ++q)
          buf[(size_t)(ii >> 1) * 2 * n + 2 * q + (ii & 1)] = (R)src[(size_t)ii * n + q];
      for (int p = 0; p < 4; ++p)
        CK(cudaMemcpyAsync(dst + sub_index(2 * p, cc.off, S), buf.data() + (size_t)p * 2 * n,
                           sizeof(R) * 2 * n, cudaMemcpyHostToDevice, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));
    return RH_OK;
  };
  int r;
  if ((r = push(L.cp, d->cp, 1)) || (r = push(L.cs[par], d->cs, 1)) ||
      (r = push(L.cjsr, d->cjsr, 1)) || (r = push(L.cjsrb, d->cjsrb, 1)) ||
      (r = push(L.ancx, d->ancx, 1)) || (r = push(L.casar, d->casar, 1)) ||
      (r = push(L.casarh, d->casarh, 1)) || (r = push(L.casarj, d->casarj, 1)) ||
      (r = push(L.casarhj, d->casarhj, 1)) || (r = push(L.ci[par], d->ci, 8)) ||
      (r = push(L.cnsr[par], d->cnsr, 8)) || (r = push(L.catf, d->catf, 8)) ||
      (r = push(L.cats, d->cats, 8)) || (r = push(L.cacal, d->cacal, 8)) ||
      (r = push(L.casr, d->casr, 8)) || (r = push(L.camyo, d->camyo, 8)) ||
      (r = push(L.mgmyo, d->mgmyo, 8)))
    return r;
  std::vector<uint32_t> ryr(n), win(n);
  std::vector<uint2> lcc(n);
  CK(cudaMemcpy(ryr.data(), L.ryr + cc.off, 4 * (size_t)n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(win.data(), L.win + cc.off, 4 * (size_t)n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(lcc.data(), L.lcc + cc.off, 8 * (size_t)n, cudaMemcpyDeviceToHost));
  for (int q = 0; q < n; ++q) {
    uint32_t nou = ryr[q] & 0xff, ncu = (ryr[q] >> 8) & 0xff, nob = (ryr[q] >> 16) & 0xff,
             ncb = ryr[q] >> 24;
    if (d->nou) nou = (uint32_t)std::min(std::max(d->nou[q], 0), 255);
    if (d->ncu) ncu = (uint32_t)std::min(std::max(d->ncu[q], 0), 255);
    if (d->nob) nob = (uint32_t)std::min(std::max(d->nob[q], 0), 255);
    if (d->ncb) ncb = (uint32_t)std::min(std::max(d->ncb[q], 0), 255);
    ryr[q] = nou | (ncu << 8) | (nob << 16) | (ncb << 24);
    uint32_t nl = win[q] & 0xffff, ns = win[q] >> 16;
    if (d->nl) nl = (uint32_t)std::min(std::max(d->nl[q], 0), 0xffff);
    if (d->nspark) ns = (uint32_t)std::min(std::max(d->nspark[q], 0), 0xffff);
    win[q] = nl | (ns << 16);
    if (d->lcc) {
      uint32_t lo = 0, hi = 0;
      for (int ll = 0; ll < 8; ++ll) {
        uint32_t st = (uint32_t)std::min(std::max(d->lcc[(size_t)ll * n + q], 0), 16);
        if (ll < 4) lo |= st << ((ll & 3) * 8);
        else hi |= st << ((ll & 3) * 8);
      }
      lcc[q] = make_uint2(lo, hi);
    }
  }
  CK(cudaMemcpy(L.ryr + cc.off, ryr.data(), 4 * (size_t)n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(L.win + cc.off, win.data(), 4 * (size_t)n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(L.lcc + cc.off, lcc.data(), 8 * (size_t)n, cudaMemcpyHostToDevice));
  return RH_OK;
}

int read_dyn(rh_sim* s, int cell, CellDyn* d) {
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMemcpy(d, s->d_dyn + cell, sizeof(CellDyn), cudaMemcpyDeviceToHost));
  return RH_OK;
}

}  // namespace

extern "C" {

int rh_get_state(rh_sim* s, int32_t cell, rh_state_f64* dst) {
  int r = check_cell(s, cell);
  if (r) return r;
  if (!dst || dst->n != s->hcells[cell].n) return fail(s, RH_ERR_ARG, "state view size mismatch");
  CK(cudaSetDevice(s->device));
  CellDyn d;
  if ((r = read_dyn(s, cell, &d))) return r;
  if (is_mixed(s)) return get_state_t<float>(s, s->Lf, cell, d.parity, dst);
  return get_state_t<double>(s, s->Ld, cell, d.parity, dst);
}

int rh_set_state(rh_sim* s, int32_t cell, const rh_state_f64* src) {
  int r = check_cell(s, cell);
  if (r) return r;
  if (!src || src->n != s->hcells[cell].n) return fail(s, RH_ERR_ARG, "state view size mismatch");
  CK(cudaSetDevice(s->device));
  CellDyn d;
  if ((r = read_dyn(s, cell, &d))) return r;
  if (is_mixed(s)) return set_state_t<float>(s, s->Lf, cell, d.parity, src);
  return set_state_t<double>(s, s->Ld, cell, d.parity, src);
}

int rh_get_membrane(rh_sim* s, int32_t cell, rh_membrane* dst) {
  int r = check_cell(s, cell);
  if (r) return r;
  if (!dst) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  CellDyn d;
  if ((r = read_dyn(s, cell, &d))) return r;
  *dst = d.m;
  return RH_OK;
}

int rh_set_membrane(rh_sim* s, int32_t cell, const rh_membrane* src) {
  int r = check_cell(s, cell);
  if (r) return r;
  if (!src) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMemcpy(&s->d_dyn[cell].m, src, sizeof(rh_membrane), cudaMemcpyHostToDevice));
  // the next step's coefficients of this cell only: the others keep theirs
  // (in mixed precision the cell update computes them in FP32)
  CK(launch_volt_prep(s->sets[s->ts].d_cells + cell, s->d_dyn + cell, 1, s->opts.dt_ms, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  s->t_host[cell] = src->t;
  s->active_host[cell] = src->t < s->hcells[cell].tend;
  return RH_OK;
}

int rh_drain_wholecell(rh_sim* s, int32_t cell, double* rows, int32_t max_rec, int32_t* nrec) {
  int r = check_cell(s, cell);
  if (r) return r;
  if (!nrec || max_rec < 0 || (max_rec > 0 && !rows)) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  long long out_count = 0;  // only the record counter of the cell state
  CK(cudaMemcpy(&out_count, reinterpret_cast<const char*>(s->d_dyn + cell) + offsetof(CellDyn, out_count),
                sizeof out_count, cudaMemcpyDeviceToHost));
  const int cap = s->opts.output_capacity;
  long long first = s->drained_wc[cell];
  if (out_count - first > cap) first = out_count - cap;  // overwritten records are lost
  const long long avail = out_count - first;
  const int cnt = (int)std::min<long long>(avail, max_rec);
  // the ring slots [first, first + cnt) in at most two contiguous copies
  const double* ring = s->d_out_wc + (size_t)cell * cap * RH_WHOLECELL_COLS;
  int done = 0;
  while (done < cnt) {
    const int slot = (int)((first + done) % cap);
    const int run = std::min(cnt - done, cap - slot);
    CK(cudaMemcpy(rows + (size_t)done * RH_WHOLECELL_COLS, ring + (size_t)slot * RH_WHOLECELL_COLS,
                  sizeof(double) * RH_WHOLECELL_COLS * run, cudaMemcpyDeviceToHost));
    done += run;
  }
  s->drained_wc[cell] = first + cnt;
  *nrec = cnt;
  return RH_OK;
}

int rh_drain_wholecell_all(rh_sim* s, double* rows, int32_t max_rec, int32_t* nrec) {
  if (!s || !nrec || max_rec < 0 || (max_rec > 0 && !rows)) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  const int n = s->ncells, cap = s->opts.output_capacity;
  const size_t ring_doubles = (size_t)n * cap * RH_WHOLECELL_COLS;
  if (s->h_counts.size() != (size_t)n) s->h_counts.assign(n, 0);
  if (s->h_ring.size() != ring_doubles) s->h_ring.assign(ring_doubles, 0.0);
  // every cell's record counter (a strided copy out of the cell states) and
  // the whole record ring, after the work queued so far
  CK(cudaMemcpy2DAsync(s->h_counts.data(), sizeof(long long),
                       reinterpret_cast<const char*>(s->d_dyn) + offsetof(CellDyn, out_count),
                       sizeof(CellDyn), sizeof(long long), n, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaMemcpyAsync(s->h_ring.data(), s->d_out_wc, sizeof(double) * ring_doubles,
                     cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  for (int c = 0; c < n; ++c) {
    const long long out_count = s->h_counts[c];
    long long first = s->drained_wc[c];
    if (out_count - first > cap) first = out_count - cap;
    const int cnt = (int)std::min<long long>(out_count - first, max_rec);
    double* dst = rows + (size_t)c * max_rec * RH_WHOLECELL_COLS;
    for (int k = 0; k < cnt; ++k) {
      const size_t slot = (size_t)((first + k) % cap);
      memcpy(dst + (size_t)k * RH_WHOLECELL_COLS,
             s->h_ring.data() + ((size_t)c * cap + slot) * RH_WHOLECELL_COLS,
             sizeof(double) * RH_WHOLECELL_COLS);
    }
    s->drained_wc[c] = first + cnt;
    nrec[c] = cnt;
  }
  return RH_OK;
}

int rh_drain_linescan(rh_sim* s, int32_t cell, double* rows, int32_t max_rec, int32_t* nrec) {
  int r = check_cell(s, cell);
  if (r) return r;
  if (!nrec || max_rec < 0 || (max_rec > 0 && !rows)) return RH_ERR_ARG;
  *nrec = 0;
  if (!s->d_out_ls) return RH_OK;  // record_linescan off: no rows
  CK(cudaSetDevice(s->device));
  CellDyn d;
  if ((r = read_dyn(s, cell, &d))) return r;
  const int cap = s->opts.output_capacity;
  const CellConst& cc = s->hcells[cell];
  long long first = s->drained_ls[cell];
  if (d.out_count - first > cap) first = d.out_count - cap;
  long long avail = d.out_count - first;
  int cnt = (int)std::min<long long>(avail, max_rec);
  const size_t blk = (size_t)cc.lx * RH_LINESCAN_COLS;
  for (int k = 0; k < cnt; ++k) {
    long long slot = (first + k) % cap;
    CK(cudaMemcpy(rows + (size_t)k * blk,
                  s->d_out_ls + ((size_t)cc.ls_off + (size_t)slot * cc.lx) * RH_LINESCAN_COLS,
                  sizeof(double) * blk, cudaMemcpyDeviceToHost));
  }
  s->drained_ls[cell] = first + cnt;
  *nrec = cnt;
  return RH_OK;
}

int rh_drain_cadist(rh_sim* s, int32_t cell, double* rec, int32_t max_rec, int32_t* nrec) {
  int r = check_cell(s, cell);
  if (r) return r;
  if (!nrec || max_rec < 0 || (max_rec > 0 && !rec)) return RH_ERR_ARG;
  *nrec = 0;
  if (!s->d_out_cd) return fail(s, RH_ERR_ARG, "cadist records are off (run option record_cadist)");
  CK(cudaSetDevice(s->device));
  CellDyn d;
  if ((r = read_dyn(s, cell, &d))) return r;
  const int cap = s->opts.cadist_capacity;
  const CellConst& cc = s->hcells[cell];
  long long first = s->drained_cd[cell];
  if (d.cd_count - first > cap) first = d.cd_count - cap;
  const int cnt = (int)std::min<long long>(d.cd_count - first, max_rec);
  const size_t len = 2 + (size_t)RH_CADIST_COLS * cc.n;
  std::vector<double> dev(len);
  for (int k = 0; k < cnt; ++k) {
    const long long slot = (first + k) % cap;
    CK(cudaMemcpy(dev.data(), s->d_out_cd + cc.cd_off + (size_t)slot * len, sizeof(double) * len,
                  cudaMemcpyDeviceToHost));
    // device rows are in CRU order (x fastest); the reference prints jx outer,
    // jz inner (:1006-1008) and scales xinaca for print (:1009)
    double* o = rec + (size_t)k * len;
    o[0] = dev[0];
    o[1] = dev[1];
    for (int x = 0; x < cc.lx; ++x)
      for (int y = 0; y < cc.ly; ++y)
        for (int z = 0; z < cc.lz; ++z) {
          const double* src = dev.data() + 2 + RH_CADIST_COLS * ((size_t)(z * cc.ly + y) * cc.lx + x);
          double* dst = o + 2 + RH_CADIST_COLS * ((size_t)(x * cc.ly + y) * cc.lz + z);
          dst[0] = src[0];
          dst[1] = src[1];
          dst[2] = src[2];
          dst[3] = src[3];
          dst[4] = src[4] / CM * 0.0965 * VS * 16120.;
          dst[5] = src[5];
        }
  }
  s->drained_cd[cell] = first + cnt;
  *nrec = cnt;
  return RH_OK;
}

int rh_drain_stats(rh_sim* s, int32_t cell, rh_beat_stats* out, int32_t max_rec, int32_t* nrec) {
  int r = check_cell(s, cell);
  if (r) return r;
  if (!nrec || max_rec < 0 || (max_rec > 0 && !out)) return RH_ERR_ARG;
  *nrec = 0;
  if (!s->d_stats) return RH_OK;
  CK(cudaSetDevice(s->device));
  CellDyn d;
  if ((r = read_dyn(s, cell, &d))) return r;
  const int cap = s->opts.stats_capacity;
  long long first = s->drained_st[cell];
  if (d.stats_count - first > cap) first = d.stats_count - cap;
  int cnt = (int)std::min<long long>(d.stats_count - first, max_rec);
  for (int k = 0; k < cnt; ++k) {
    long long slot = (first + k) % cap;
    CK(cudaMemcpy(out + k, s->d_stats + (size_t)cell * cap + slot, sizeof(rh_beat_stats),
                  cudaMemcpyDeviceToHost));
  }
  s->drained_st[cell] = first + cnt;
  *nrec = cnt;
  return RH_OK;
}

int rh_analyze_trace(double pcl_ms, const double* t, const double* v, int64_t nsteps,
                     const double* wholecell, int32_t nrec, rh_beat_stats* out, int32_t max_rec,
                     int32_t* nbeats) {
  if (!t || !v || !nbeats || nsteps < 0 || nrec < 0 || (nrec > 0 && !wholecell) ||
      !(pcl_ms > 0) || max_rec < 0 || (max_rec > 0 && !out))
    return RH_ERR_ARG;
  BeatTracker b;
  beat_reset(b);
  int32_t nb = 0, rec = 0;
  for (int64_t i = 0; i < nsteps; ++i) {
    rh_beat_stats st;
    if (beat_on_step(b, t[i], v[i], pcl_ms, &st)) {
      if (nb < max_rec) out[nb] = st;
      ++nb;
    }
    // output records carry the step time in column 1
    while (rec < nrec && wholecell[(size_t)rec * RH_WHOLECELL_COLS] <= t[i]) {
      if (wholecell[(size_t)rec * RH_WHOLECELL_COLS] == t[i])
        beat_on_output(b, wholecell + (size_t)rec * RH_WHOLECELL_COLS);
      ++rec;
    }
  }
  *nbeats = std::min(nb, max_rec);
  return RH_OK;
}

int rh_cell_status(rh_sim* s, int32_t cell, uint32_t* status) {
  int r = check_cell(s, cell);
  if (r) return r;
  if (!status) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  CellDyn d;
  if ((r = read_dyn(s, cell, &d))) return r;
  *status = d.status;
  return RH_OK;
}

// Snapshot format: magic, version, precision, ncells, stride, the cells'
// parameters, the whole lattice arena and the per-cell dynamic state.
static const char kMagic[8] = {'R', 'H', 'S', 'N', 'A', 'P', '0', '1'};

int rh_checkpoint(rh_sim* s, const char* path) {
  if (!s || !path) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  FILE* f = fopen(path, "wb");
  if (!f) return fail(s, RH_ERR_IO, "cannot open %s", path);
  std::vector<char> host(s->arena_bytes);
  std::vector<CellDyn> dyn(s->ncells);
  cudaError_t e1 = cudaMemcpy(host.data(), s->arena, s->arena_bytes, cudaMemcpyDeviceToHost);
  cudaError_t e2 = cudaMemcpy(dyn.data(), s->d_dyn, sizeof(CellDyn) * s->ncells, cudaMemcpyDeviceToHost);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    fclose(f);
    return fail(s, RH_ERR_CUDA, "checkpoint copy failed");
  }
  int32_t hdr[4] = {1, s->opts.precision, s->ncells, 0};
  int64_t stride = s->stride;
  uint64_t bytes = s->arena_bytes;
  bool ok = fwrite(kMagic, 1, 8, f) == 8 && fwrite(hdr, sizeof hdr, 1, f) == 1 &&
            fwrite(&stride, 8, 1, f) == 1 && fwrite(&bytes, 8, 1, f) == 1 &&
            fwrite(s->params.data(), sizeof(rh_cell_params), s->ncells, f) == (size_t)s->ncells &&
            fwrite(host.data(), 1, host.size(), f) == host.size() &&
            fwrite(dyn.data(), sizeof(CellDyn), s->ncells, f) == (size_t)s->ncells;
  ok = (fclose(f) == 0) && ok;
  if (!ok) return fail(s, RH_ERR_IO, "write to %s failed", path);
  return RH_OK;
}

int rh_restore(rh_sim* s, const char* path) {
  if (!s || !path) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  FILE* f = fopen(path, "rb");
  if (!f) return fail(s, RH_ERR_IO, "cannot open %s", path);
  char magic[8];
  int32_t hdr[4];
  int64_t stride = 0;
  uint64_t bytes = 0;
  bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, kMagic, 8) == 0 &&
            fread(hdr, sizeof hdr, 1, f) == 1 && fread(&stride, 8, 1, f) == 1 &&
            fread(&bytes, 8, 1, f) == 1;
  if (!ok || hdr[0] != 1 || hdr[1] != s->opts.precision || hdr[2] != s->ncells ||
      stride != s->stride || bytes != s->arena_bytes) {
    fclose(f);
    return fail(s, RH_ERR_IO, "%s is not a snapshot of this simulator layout", path);
  }
  std::vector<rh_cell_params> prm(s->ncells);
  std::vector<char> host(s->arena_bytes);
  std::vector<CellDyn> dyn(s->ncells);
  ok = fread(prm.data(), sizeof(rh_cell_params), s->ncells, f) == (size_t)s->ncells &&
       fread(host.data(), 1, host.size(), f) == host.size() &&
       fread(dyn.data(), sizeof(CellDyn), s->ncells, f) == (size_t)s->ncells;
  fclose(f);
  if (!ok) return fail(s, RH_ERR_IO, "%s is truncated", path);
  if (memcmp(prm.data(), s->params.data(), sizeof(rh_cell_params) * s->ncells) != 0)
    return fail(s, RH_ERR_IO, "%s holds different cell parameters", path);
  CK(cudaMemcpy(s->arena, host.data(), s->arena_bytes, cudaMemcpyHostToDevice));
  for (auto& d : dyn) d.arrive = 0;
  CK(cudaMemcpy(s->d_dyn, dyn.data(), sizeof(CellDyn) * s->ncells, cudaMemcpyHostToDevice));
  for (int c = 0; c < s->ncells; ++c) {
    s->t_host[c] = dyn[c].m.t;
    s->active_host[c] = !dyn[c].done;
    s->drained_wc[c] = dyn[c].out_count;
    s->drained_ls[c] = dyn[c].out_count;
    s->drained_st[c] = dyn[c].stats_count;
    s->drained_cd[c] = dyn[c].cd_count;
  }
  return RH_OK;
}

int rh_state_bytes(const rh_sim* s, size_t* bytes) {
  if (!s || !bytes) return RH_ERR_ARG;
  *bytes = s->arena_bytes + sizeof(CellDyn) * (size_t)s->ncells;
  return RH_OK;
}

int rh_export_state(rh_sim* s, void* host, size_t bytes) {
  if (!s || !host || bytes != s->arena_bytes + sizeof(CellDyn) * (size_t)s->ncells)
    return fail(s, RH_ERR_ARG, "export buffer must hold rh_state_bytes() bytes");
  CK(cudaSetDevice(s->device));
  CK(copy_state_out(s, reinterpret_cast<char*>(host)));
  CK(cudaStreamSynchronize(s->stream));
  return RH_OK;
}

int rh_import_state(rh_sim* s, const void* host, size_t bytes) {
  if (!s || !host || bytes != s->arena_bytes + sizeof(CellDyn) * (size_t)s->ncells)
    return fail(s, RH_ERR_ARG, "import buffer must hold rh_state_bytes() bytes");
  CK(cudaSetDevice(s->device));
  const char* h = reinterpret_cast<const char*>(host);
  int r = import_mirrors(s, h);
  if (r) return r;
  CK(copy_state_in(s, h));
  CK(cudaStreamSynchronize(s->stream));
  return RH_OK;
}

int rh_tile_size(const rh_sim* s, int32_t* tile) {
  if (!s || !tile) return RH_ERR_ARG;
  *tile = s->sets[s->ts].tile;
  return RH_OK;
}

int rh_autotune(rh_sim* s, int32_t steps, int32_t* tile, double* ms_per_step) {
  if (!s || steps <= 0) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  // save the state on the device; every candidate starts from it
  const size_t dyn_bytes = sizeof(CellDyn) * (size_t)s->ncells;
  void* backup = nullptr;
  if (cudaMalloc(&backup, s->arena_bytes + dyn_bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(s, RH_ERR_NOMEM, "autotune: no room for a state copy");
  }
  char* bk = reinterpret_cast<char*>(backup);
  CK(cudaMemcpyAsync(bk, s->arena, s->arena_bytes, cudaMemcpyDeviceToDevice, s->stream));
  CK(cudaMemcpyAsync(bk + s->arena_bytes, s->d_dyn, dyn_bytes, cudaMemcpyDeviceToDevice, s->stream));
  const std::vector<double> t0 = s->t_host;
  const std::vector<char> a0 = s->active_host;
  const int ts0 = s->ts;
  double best = 1e300;
  int best_k = ts0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = RH_OK;
  for (int k = 0; k < kNumTileSizes && rc == RH_OK; ++k) {
    s->ts = k;
    cudaMemcpyAsync(s->arena, bk, s->arena_bytes, cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(s->d_dyn, bk + s->arena_bytes, dyn_bytes, cudaMemcpyDeviceToDevice, s->stream);
    cudaEventRecord(e0, s->stream);
    // the trial steps write no output records, so records still waiting in
    // the output rings are never overwritten (one step in 100 is an output
    // step; its extra stores do not move the choice)
    if (use_persist(s)) {  // one persistent launch of `steps` steps
      cudaError_t e = launch_persist(s, steps, true);
      if (e != cudaSuccess) rc = fail(s, RH_ERR_CUDA, "autotune launch: %s", cudaGetErrorString(e));
    } else {
      for (int i = 0; i < steps; ++i) {  // the output-free kernel variant
        cudaError_t e = launch_one(s, false, false);
        if (e != cudaSuccess) {
          rc = fail(s, RH_ERR_CUDA, "autotune launch: %s", cudaGetErrorString(e));
          break;
        }
      }
    }
    if (rc != RH_OK) break;
    cudaEventRecord(e1, s->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = fail(s, RH_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    if ((rc = check_wait_error(s)) != RH_OK) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    double per = ms / steps;
    if (ms_per_step) ms_per_step[k] = per;
    if (per < best) {
      best = per;
      best_k = k;
    }
  }
  // restore the state and select the winner
  cudaMemcpyAsync(s->arena, bk, s->arena_bytes, cudaMemcpyDeviceToDevice, s->stream);
  cudaMemcpyAsync(s->d_dyn, bk + s->arena_bytes, dyn_bytes, cudaMemcpyDeviceToDevice, s->stream);
  cudaStreamSynchronize(s->stream);
  cudaFree(backup);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s->t_host = t0;
  s->active_host = a0;
  s->ts = rc == RH_OK ? best_k : ts0;
  s->hcells = s->sets[s->ts].hcells;
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  if (tile) *tile = s->sets[s->ts].tile;
  CK(cudaGetLastError());
  return rc;
}

int rh_get_launch_shape(const rh_sim* s, rh_launch_shape* shape) {
  if (!s || !shape) return RH_ERR_ARG;
  shape->persistent = use_persist(s) ? 1 : 0;
  shape->tile_crus = s->sets[s->ts].tile;
  shape->fewer_ctas = (shape->persistent && s->fewer_ctas) ? 1 : 0;
  shape->cell_groups = s->ngroups;
  shape->bulk_staging = shape->persistent ? 0 : s->staging;
  return RH_OK;
}

int rh_set_launch_shape(rh_sim* s, const rh_launch_shape* shape) {
  if (!s || !shape) return RH_ERR_ARG;
  int k = -1;
  for (int i = 0; i < kNumTileSizes; ++i)
    if (kTileSizes[i] == shape->tile_crus) k = i;
  if (k < 0) return fail(s, RH_ERR_NOTBUILT, "no kernel for tiles of %d CRUs", shape->tile_crus);
  if (shape->persistent) {
    if (!s->persist_ok)
      return fail(s, RH_ERR_NOTBUILT, "this device cannot run the persistent launch");
    if (shape->tile_crus != 64 && shape->tile_crus != 128)
      return fail(s, RH_ERR_NOTBUILT, "the persistent launch takes tiles of 64 or 128 CRUs");
    if (shape->fewer_ctas && any_options(s))
      return fail(s, RH_ERR_NOTBUILT, "fewer_ctas is compiled for cells without build options");
    if (shape->bulk_staging)
      return fail(s, RH_ERR_NOTBUILT, "bulk staging is compiled for the two-launch path");
  }
  if (shape->bulk_staging < 0 || shape->bulk_staging > 2)
    return fail(s, RH_ERR_ARG, "bulk_staging is 0, 1 or 2");
  if (shape->bulk_staging && !is_mixed(s))
    return fail(s, RH_ERR_NOTBUILT, "bulk staging is compiled for the FP32 lattice");
  if (shape->bulk_staging == 2 && !s->maps_ok)
    return fail(s, RH_ERR_NOTBUILT, "tensor copies need the driver's tensor-map encoder");
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  s->ts = k;
  s->hcells = s->sets[k].hcells;
  s->opts.persistent = shape->persistent ? 1 : 0;
  s->fewer_ctas = shape->persistent && shape->fewer_ctas;
  s->staging = shape->persistent ? 0 : shape->bulk_staging;
  if (!shape->persistent && shape->cell_groups > 0 && shape->cell_groups != s->ngroups) {
    int r = set_groups(s, shape->cell_groups);
    if (r) return r;
  }
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  return RH_OK;
}

namespace {

// Process-wide cache of rh_autotune_shapes' choices, by device, precision
// and lattice classes.
std::mutex g_shape_mu;
std::map<std::string, rh_launch_shape> g_shape_cache;

std::string workload_key(const rh_sim* s) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, s->device);
  std::map<std::pair<int, int>, int> classes;  // (lx / 16, ly / 16) -> cells
  long long crus = 0;
  for (const CellConst& c : s->hcells) {
    classes[{c.lx / 16, c.ly / 16}] += 1;
    crus += c.n;
  }
  std::string k = std::string(prop.name) + "|sm" + std::to_string(prop.multiProcessorCount) +
                  "|p" + std::to_string(s->opts.precision) + "|opt" +
                  std::to_string(any_options(s) ? 1 : 0) + "|n" + std::to_string(crus);
  for (const auto& kv : classes)
    k += "|" + std::to_string(kv.first.first) + "," + std::to_string(kv.first.second) + ":" +
         std::to_string(kv.second);
  return k;
}

// The file that keeps choices across processes (environment RH_SHAPE_CACHE),
// one line per choice: key, tab, persistent tile fewer groups staging; the
// last line of a key counts.
const char* shape_cache_file() {
  const char* p = getenv("RH_SHAPE_CACHE");
  return (p && *p) ? p : nullptr;
}

bool shape_file_lookup(const std::string& key, rh_launch_shape& out) {
  const char* path = shape_cache_file();
  if (!path) return false;
  FILE* f = fopen(path, "r");
  if (!f) return false;
  bool found = false;
  char line[4096];
  while (fgets(line, sizeof(line), f)) {
    char* tab = strchr(line, '\t');
    if (!tab || (size_t)(tab - line) != key.size() || key.compare(0, key.size(), line, key.size()))
      continue;
    rh_launch_shape sh{};
    if (sscanf(tab + 1, "%d %d %d %d %d", &sh.persistent, &sh.tile_crus, &sh.fewer_ctas,
               &sh.cell_groups, &sh.bulk_staging) == 5) {
      out = sh;
      found = true;
    }
  }
  fclose(f);
  return found;
}

void shape_file_store(const std::string& key, const rh_launch_shape& sh) {
  const char* path = shape_cache_file();
  if (!path) return;
  FILE* f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "%s\t%d %d %d %d %d\n", key.c_str(), sh.persistent, sh.tile_crus, sh.fewer_ctas,
          sh.cell_groups, sh.bulk_staging);
  fclose(f);
}

}  // namespace

int rh_autotune_shapes(rh_sim* s, int32_t steps, rh_launch_shape* best,
                       rh_launch_shape* tried, double* ms_per_step, int32_t max_tried,
                       int32_t* ntried) {
  if (!s || steps <= 0 || max_tried < 0) return RH_ERR_ARG;
  if (ntried) *ntried = 0;
  CK(cudaSetDevice(s->device));
  CK(cudaStreamSynchronize(s->stream));
  const std::string key = workload_key(s);
  {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    auto it = g_shape_cache.find(key);
    rh_launch_shape cached{};
    bool hit = it != g_shape_cache.end();
    if (hit) cached = it->second;
    else if (shape_file_lookup(key, cached)) hit = true;
    if (hit) {
      int r = rh_set_launch_shape(s, &cached);
      if (r == RH_OK) {
        g_shape_cache[key] = cached;
        if (best) *best = cached;
        return r;
      }
      // a stored shape this build cannot run: time the candidates instead
      g_shape_cache.erase(key);
    }
  }
  // candidates
  std::vector<rh_launch_shape> cand;
  if (s->persist_ok)
    for (int tile : {64, 128})
      for (int fewer = 0; fewer < (any_options(s) ? 1 : 2); ++fewer)
        cand.push_back(rh_launch_shape{1, tile, fewer, 0, 0});
  for (int bulk = 0; bulk < (is_mixed(s) ? (s->maps_ok ? 3 : 2) : 1); ++bulk)
    for (int tile : {64, 128, 256})
      for (int g : {8, 12, 16, 24})
        if (g <= s->ncells || g == 8)
          cand.push_back(rh_launch_shape{0, tile, 0, std::min(g, s->ncells), bulk});
  rh_launch_shape orig{};
  rh_get_launch_shape(s, &orig);
  // save the state on the device; every candidate starts from it
  const size_t dyn_bytes = sizeof(CellDyn) * (size_t)s->ncells;
  void* backup = nullptr;
  if (cudaMalloc(&backup, s->arena_bytes + dyn_bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(s, RH_ERR_NOMEM, "autotune: no room for a state copy");
  }
  char* bk = reinterpret_cast<char*>(backup);
  CK(cudaMemcpyAsync(bk, s->arena, s->arena_bytes, cudaMemcpyDeviceToDevice, s->stream));
  CK(cudaMemcpyAsync(bk + s->arena_bytes, s->d_dyn, dyn_bytes, cudaMemcpyDeviceToDevice, s->stream));
  const std::vector<double> t0 = s->t_host;
  const std::vector<char> a0 = s->active_host;
  auto restore = [&]() {
    cudaMemcpyAsync(s->arena, bk, s->arena_bytes, cudaMemcpyDeviceToDevice, s->stream);
    cudaMemcpyAsync(s->d_dyn, bk + s->arena_bytes, dyn_bytes, cudaMemcpyDeviceToDevice, s->stream);
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // the trial steps write no output records (see rh_autotune)
  auto trial = [&](int n) -> cudaError_t {
    if (use_persist(s)) return launch_persist(s, n, true);
    for (int i = 0; i < n; ++i) {
      cudaError_t e = launch_one(s, false, false);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  int rc = RH_OK, nt = 0;
  double best_ms = 1e300;
  rh_launch_shape win = orig;
  for (const rh_launch_shape& c : cand) {
    if (rh_set_launch_shape(s, &c) != RH_OK) continue;
    restore();
    cudaError_t e = trial(std::max(1, steps / 4));  // first launches of this shape, untimed
    restore();
    cudaEventRecord(e0, s->stream);
    if (e == cudaSuccess) e = trial(steps);
    cudaEventRecord(e1, s->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      rc = fail(s, RH_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
      break;
    }
    if ((rc = check_wait_error(s)) != RH_OK) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double per = ms / steps;
    if (nt < max_tried) {
      if (tried) tried[nt] = c;
      if (ms_per_step) ms_per_step[nt] = per;
    }
    ++nt;
    if (per < best_ms) {
      best_ms = per;
      win = c;
    }
  }
  restore();
  cudaStreamSynchronize(s->stream);
  cudaFree(backup);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s->t_host = t0;
  s->active_host = a0;
  if (ntried) *ntried = std::min(nt, max_tried);
  const int r = rh_set_launch_shape(s, rc == RH_OK ? &win : &orig);
  if (rc != RH_OK) return rc;
  if (r != RH_OK) return r;
  {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    g_shape_cache[key] = win;
    shape_file_store(key, win);
  }
  if (best) *best = win;
  CK(cudaGetLastError());
  return RH_OK;
}

int rh_bytes_per_cru_step(const rh_sim* s, double* bytes) {
  if (!s || !bytes) return RH_ERR_ARG;
  // 73 persistent real fields and 16 B of packed integers, each read and
  // written once
  *bytes = 2.0 * (73.0 * (double)real_size(s) + 16.0);
  return RH_OK;
}

int rh_kernel_timing(rh_sim* s, int64_t* launches, double* ms) {
  if (!s || !launches || !ms) return RH_ERR_ARG;
  CK(cudaSetDevice(s->device));
  if (s->timing_open) {
    CK(cudaEventSynchronize(s->ev1));
    float e = 0;
    CK(cudaEventElapsedTime(&e, s->ev0, s->ev1));
    s->ms_total += e;
    s->launches_total += s->launches_pending;
    s->launches_pending = 0;
    s->timing_open = false;
  }
  *launches = s->launches_total;
  *ms = s->ms_total;
  s->launches_total = 0;
  s->ms_total = 0;
  return RH_OK;
}

int rh_num_groups(const rh_sim* s, int32_t* groups) {
  if (!s || !groups) return RH_ERR_ARG;
  *groups = s->ngroups;
  return RH_OK;
}

int rh_kernel_launches(const rh_sim* s, int64_t* launches, int32_t* persistent) {
  if (!s) return RH_ERR_ARG;
  if (launches) *launches = s->kernels;
  if (persistent) *persistent = use_persist(s) ? 1 : 0;
  return RH_OK;
}

int rh_window_ctas(const rh_sim* s, int32_t* ctas) {
  if (!s || !ctas) return RH_ERR_ARG;
  *ctas = 0;
  if (!use_persist(s)) return RH_OK;
  int g = 0;
  const bool opt = any_options(s);
  const int tile = s->sets[s->ts].tile;
  cudaError_t e = is_mixed(s) ? window_grid<float>(tile, opt, s->fewer_ctas, &g)
                              : window_grid<double>(tile, opt, s->fewer_ctas, &g);
  if (e != cudaSuccess) return RH_ERR_CUDA;
  *ctas = std::min(g, s->sets[s->ts].ntiles);
  return RH_OK;
}

int rh_set_wait_limit(rh_sim* s, int64_t polls, uint32_t target_offset) {
  if (!s || polls < 0) return RH_ERR_ARG;
  s->wait_limit = polls == 0 ? kDefaultWaitLimit : polls;
  s->wait_offset = target_offset;
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);  // launch arguments changed
  s->graphs.clear();
  return RH_OK;
}

int rh_last_error(const rh_sim* s, char* buf, size_t n) {
  if (!buf || n == 0) return RH_ERR_ARG;
  const char* m = s ? s->err.c_str() : g_create_error.c_str();
  snprintf(buf, n, "%s", m);
  return RH_OK;
}

int rh_format_wholecell(const double* c, char* buf, size_t n) {
  if (!c || !buf) return RH_ERR_ARG;
  return snprintf(buf, n,
                  "%f %f %f %f %f  %f %f %f %f %f  "
                  "%f %f %f %f %f  %f %f %f %f %f  "
                  "%f %f %f %f %f  %f %i %i %i %i  "
                  "%i %i %i %i %i  %i %i %f %f %f  "
                  "%i %f %f %f %f\n",
                  c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], c[8], c[9], c[10], c[11], c[12],
                  c[13], c[14], c[15], c[16], c[17], c[18], c[19], c[20], c[21], c[22], c[23],
                  c[24], c[25], (int)c[26], (int)c[27], (int)c[28], (int)c[29], (int)c[30],
                  (int)c[31], (int)c[32], (int)c[33], (int)c[34], (int)c[35], (int)c[36], c[37],
                  c[38], c[39], (int)c[40], c[41], c[42], c[43], c[44]);
}

int rh_format_linescan(const double* c, char* buf, size_t n) {
  if (!c || !buf) return RH_ERR_ARG;
  return snprintf(buf, n,
                  "%f %f %f %i %i %i %i %i %f %f %f %f %f %f %f %f %f %f %f %f %f %f\n", c[0],
                  c[1], c[2], (int)c[3], (int)c[4], (int)c[5], (int)c[6], (int)c[7], c[8], c[9],
                  c[10], c[11], c[12], c[13], c[14], c[15], c[16], c[17], c[18], c[19], c[20],
                  c[21]);
}

}  // extern "C"
