/*
 * rh.h — C ABI of the GB300 stochastic myocyte simulator (ryr_hyperactivity_gb300).
 *
 * The simulator advances the CRU lattice of one or many independent cells by
 * one time step per lattice update, then reduces the whole-cell currents and
 * integrates the membrane model, all on the GPU.  It replaces the per-step
 * seam of cuda_Cell_Detailed.cu: the `Compute` launch (cuda_Cell_Detailed.cu:217,
 * :420), the two synchronous device-to-host copies and the host loop that sums
 * xicat/xinaca/cs and integrates V (:427-739), and the output block (:777-1081).
 *
 * Conventions
 *   - Every call returns an int status: 0 = RH_OK, negative = error.  The text
 *     of the last error is available from rh_last_error().
 *   - A handle is single-threaded and not re-entrant; distinct handles may be
 *     used from different host threads.  The library owns all device memory.
 *   - No C++ exceptions cross this boundary; plain C types only.
 *   - Lattice dimensions follow the reference: nx, ny, nz count the ghost
 *     shell, so a cell has (nx-2)(ny-2)(nz-2) interior CRUs.  Host-side state
 *     arrays in rh_state_f64 hold interior CRUs only, x fastest:
 *     index = (i-1) + (nx-2)*((j-1) + (ny-2)*(k-1)); sub-voxel fields are
 *     8 planes: field[sub*n + index].
 */
#ifndef RH_H
#define RH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RH_ABI_VERSION 1

/* status codes */
#define RH_OK 0
#define RH_ERR_ARG -1        /* invalid argument */
#define RH_ERR_CUDA -2       /* CUDA runtime error */
#define RH_ERR_NOMEM -3      /* allocation failed */
#define RH_ERR_NUMERIC -4    /* NaN/Inf detected in a cell (see rh_cell_status) */
#define RH_ERR_TIMEOUT -5    /* a bounded device wait ran out */
#define RH_ERR_IO -6         /* checkpoint file error */
#define RH_ERR_STATE -7      /* call not valid in the current state */
#define RH_ERR_NOTBUILT -8   /* kernel variant not compiled in */

/* precision modes */
#define RH_FP64 0   /* every field and operation in FP64 */
#define RH_MIXED 1  /* lattice fields/rates FP32; V, [Na]i, reductions FP64 */

/* per-cell status bits (rh_cell_status) */
#define RH_STATUS_NAN 0x1u            /* NaN/Inf in V or a reduced quantity */
#define RH_STATUS_GAUSS_RETRY 0x2u    /* a Gaussian RyR draw hit the 200-retry cap
                                         (subroutine_cuda.c:358-361 and siblings) */
#define RH_STATUS_CI_HIGH 0x4u        /* some ci > 1000 uM at an output step
                                         (cuda_Cell_Detailed.cu:878-880) */
#define RH_STATUS_DONE 0x8u           /* the cell reached the end of its protocol */
#define RH_STATUS_RATE_CAP 0x10u      /* an RyR transition probability per step
                                         exceeded 1 (the OB->OU probability pbu of
                                         subroutine_cuda.c:443 is not capped); its
                                         Gaussian draw is then NaN, is redrawn up to
                                         the 200-try cap and counts 0 */

#define RH_STATUS_TIMEOUT 0x20u       /* a bounded device wait of the persistent
                                         window launch ran out (rh_run_steps then
                                         returns RH_ERR_TIMEOUT; the lattice state
                                         is left part-way through a step) */

/* Number of columns of one wholecell record and one linescan row. */
#define RH_WHOLECELL_COLS 45
#define RH_LINESCAN_COLS 22
#define RH_CADIST_COLS 6 /* per interior CRU; a record adds t and V */

/* Membrane-voltage protocols (the reference's compile-time protocol switches,
 * cuda_Cell_Detailed.cu:34, :54-61, :733-773).  The voltage the model computes
 * is replaced after each step by the protocol's value, except for PACED and
 * NOPACING, which only differ in the stimulus. */
#define RH_PROTO_PACED 0           /* default build: 80 uA/uF for 1 ms at t = 100 + k*PCL (:689) */
#define RH_PROTO_NOPACING 1        /* -Dnopacing: no stimulus (:694-696) */
#define RH_PROTO_VCLAMP 2          /* -Dvclamp: -86 mV, clamp_mv after t > 100 ms (:733-739) */
#define RH_PROTO_BROWN_VCLAMP 3    /* -Dbrownvclamp: -86/-10/10/-30/-86 mV steps at 4000, 4200,
                                      6200, 7200 ms (:741-752) */
#define RH_PROTO_AP_CLAMP 4        /* -Dapclamp: V from a recorded waveform of PCL/dt samples,
                                      repeated every PCL (:383-395, :754-757); the waveform is
                                      given with rh_set_ap_clamp */
#define RH_PROTO_LINEAR_AP_CLAMP 5 /* -Dlinearapclamp: piecewise-linear AP (:758-773) */

/* Sarcolemmal Na/Ca exchanger forms (subroutine_cuda.c:47-120). */
#define RH_NCX_ALLOSTERIC 0  /* ncx: Ka = Ancx with its own ODE (the reference's build) */
#define RH_NCX_OLD 1         /* oldncx: Ka = 1/(1+(Kda/cs)^3), Ancx from on/off rates
                                (the commented call at cuda_Cell_Detailed.cu:1300) */
#define RH_NCX_NOALLO 2      /* ncx_noallo: no allosteric state, Ka = 1 above -75 mV */

/* Parameters of one cell.  argv[k] refers to the reference command line
 * (cuda_Cell_Detailed <dev> <name> a3 .. a10). */
typedef struct {
  int32_t nx, ny, nz;   /* lattice incl. ghost shell (cuda_Cell_Detailed.cu:80-82) */
  int32_t nbeats;       /* nbeat (:49) */
  double pcl_ms;        /* tperid, pacing cycle length (:50) */
  double clamp_mv;      /* argv[3], clamp voltage (vclamp builds only, :59) */
  double cjsr_basal;    /* argv[4], initial JSR/NSR load in uM (:92) */
  double ncx_scale;     /* argv[5]: svncx = 2.5*a5 (:109) */
  double ku;            /* argv[6]: RyR cp half-activation (:126,:136,:403) */
  double r1;            /* argv[7]: passed through, unused (reesica.h:14) */
  double kb;            /* argv[8]: bound-RyR opening scale (:402) */
  double ica_scale;     /* argv[9]: svica = 0.666*1.2*a9 (:96) */
  double ku2;           /* argv[10]: RyR CU->OU rate multiplier (:401) */
  double ikr_scale;     /* multiplies the control IKr prefactor svikr=3 (:138);
                           forced to 0 under lqt (:128) */
  double cao_mM;        /* extracellular Ca, Cext (subroutine_cuda.c:24) */
  int32_t lqt;          /* -Dlqt  (Makefile:9): IKr off */
  int32_t iso2;         /* -Diso2 (Makefile:16): SERCA x1.75, LCC shifts */
  int32_t tapsi;        /* -Dtapsi (Makefile:11): SERCA off, cjsr 10 */
  uint32_t seed;        /* Philox key word 0 (reference: curand seed 18, :377) */
  uint32_t cell_id;     /* Philox key word 1 */
  int32_t linescan_jz;  /* z plane of the linescan; -1 = reference's 5 (:972),
                           clamped to nz-2 when the lattice is thinner */
  int32_t protocol;     /* RH_PROTO_* (default RH_PROTO_PACED) */
  int32_t perm;         /* -Dperm (:35): permeabilised cell.  No LCC or NCX flux, no
                           stimulus, [Ca] 0.3 uM held at the lattice faces and
                           leaking into the submembrane space (:1409-1411), initial
                           [Ca]i 0.3 uM and JSR 900 uM (argv[4] unused, :87-93) */
  int32_t iso;          /* -Diso (:32): isoproterenol from t = 5.5 PCL: SERCA x2
                           (x1.75 still wins under iso2), LCC slots 4-7 filled at
                           t = 5.5 PCL (+15.5 PCL ...), stimulus at phase 0 and
                           only while t < 11.9 PCL (:683-687, :1213-1229) */
  int32_t randomlcc;    /* -Drandomlcc (:31): each CRU starts with 0..8 LCCs, one
                           Philox draw per CRU at initialisation (:1150-1155) */
  int32_t slowncx;      /* -Dslowncxchange (:52): background Ca current in the
                           submembrane space, NCX Ka = 5 Ancx, slower IKs Ca
                           dependence (:540-543, :1267-1269, subroutine_cuda.c:59-62) */
  int32_t ncx_form;     /* RH_NCX_* (default RH_NCX_ALLOSTERIC) */
} rh_cell_params;

/* Run-wide options. */
typedef struct {
  int32_t precision;          /* RH_FP64 or RH_MIXED */
  int32_t device;             /* CUDA device ordinal */
  double dt_ms;               /* time step (reference DT 0.025, :51) */
  int32_t block_size;         /* CRUs per CTA (64, 128 or 256); 0 = 128 */
  int32_t output_capacity;    /* wholecell records kept per cell between drains */
  int32_t record_linescan;    /* 1 = keep linescan rows at output steps */
  int32_t track_stats;        /* 1 = per-beat APD90/EAD/peak-ci/SR-load/sparks */
  int32_t stats_capacity;     /* beats kept per cell between drains */
  int32_t keep_diagnostics;   /* 1 = keep xire/po/xinaca/xicat/xiup/xileak of the
                                 last lattice update for rh_get_state */
  int32_t window_steps;       /* steps per captured CUDA graph (0 = 100, one
                                 output period) */
  int32_t cell_groups;        /* cells split into this many groups of about equal
                                 CRU count that advance on concurrent streams
                                 (0 = 8; capped at the number of cells) */
  int32_t record_cadist;      /* 1 = keep cadist records (the reference's
                                 outputcadist build, :1001-1013): every 5 ms in the
                                 first 500 ms of each pacing period, t, V and 6
                                 values per interior CRU */
  int32_t cadist_capacity;    /* cadist records kept per cell between drains
                                 (0 = 8) */
  int32_t persistent;         /* 1 = each window of steps is one persistent
                                 cooperative launch: every cell's lattice and
                                 whole-cell updates, cells synchronised by
                                 per-cell arrival counters, a queue of cell
                                 updates and bounded device waits (tiles of 64
                                 or 128 CRUs; other tile lengths run the 0
                                 path); 0 (default) = two launches per step and
                                 cell group (lattice update, then cell update),
                                 the faster path on GB300 (rh_autotune_shapes
                                 measures both) */
} rh_run_opts;

/* Full FP64 view of one cell's lattice state (caller-owned host arrays of
 * n = (nx-2)(ny-2)(nz-2) interior CRUs; sub-voxel arrays hold 8*n values).
 * xire, po, xinaca, xicat, xiup, xileak are the diagnostics of the last
 * lattice update: written by rh_get_state, ignored by rh_set_state. */
typedef struct {
  int32_t n;
  double *cp, *cs, *cjsr, *cjsrb, *ancx;
  double *casar, *casarh, *casarj, *casarhj;
  double *ci, *cnsr, *catf, *cats, *cacal, *casr, *camyo, *mgmyo; /* [8][n] */
  int32_t *nou, *ncu, *nob, *ncb, *nl, *nspark;
  int32_t *lcc;                                                    /* [8][n] */
  double *xire, *po, *xinaca, *xicat;                              /* [n] */
  double *xiup, *xileak;                                           /* [8][n] */
} rh_state_f64;

/* Whole-cell (membrane) state of one cell, the host scalars of
 * cuda_Cell_Detailed.cu:325-371 plus the currents of the last step. */
typedef struct {
  double t;             /* ms, accumulated by repeated addition of dt (:1083) */
  int64_t step;         /* lattice updates done */
  double v, xnai, xm, xh, xj, xr, xs1, xs2, qks, xtos, ytos, xtof, ytof;
  double out_ica, out_ncx, out_ina;  /* window accumulators (:774-776) */
  int64_t sparksum;
  double csubt, xicatto, xinacato;   /* last reduction (:447-456) */
  double xina, xiks, xikr, xik1, xinak, xitos, xitof;  /* last currents */
} rh_membrane;

/* Per-beat statistics of one cell (project-defined detectors). */
typedef struct {
  int32_t beat;          /* beat index from 0 */
  int32_t ead;           /* 1 if an early afterdepolarisation was detected */
  double apd90_ms;       /* -1 if the AP did not repolarise within the beat */
  double v_peak;         /* mV */
  double ci_peak;        /* peak of mean [Ca]i over the beat's output samples, uM */
  double sr_load;        /* mean cjsr at the last output sample before the stimulus, uM */
  int32_t sparks;        /* spark onsets in the beat (sum of wholecell column 41) */
  int32_t pad;
} rh_beat_stats;

typedef struct rh_sim rh_sim;

/* Defaults: reference's shipped build (cuda_Cell_Detailed.cu:45-145, run.sh:9
 * "hyper" arguments) on a 64x28x12 lattice. */
void rh_default_cell_params(rh_cell_params* p);
void rh_default_run_opts(rh_run_opts* o);

/* Creates a simulator for `ncells` cells and initialises every cell as the
 * reference's Init kernel does (cuda_Cell_Detailed.cu:1108-1182) plus the
 * host initial conditions (:349-365). */
int rh_create(const rh_cell_params* cells, int32_t ncells, const rh_run_opts* opts,
              rh_sim** out);
int rh_destroy(rh_sim* sim);

/* Advances every cell that has not finished its protocol by `nsteps` time
 * steps (one reference loop iteration each, :399-1085).  Cells whose time
 * reached nbeats*pcl + 2100 ms stop and are flagged RH_STATUS_DONE. */
int rh_run_steps(rh_sim* sim, int64_t nsteps);

/* Runs until every cell finished its protocol. */
int rh_run_to_end(rh_sim* sim);

/* Only the lattice update (the Compute kernel, :1187-1692) for every cell,
 * with the cell's current v, t and [Na]i; no reduction, no V update, t does
 * not advance.  For single-step parity checks. */
int rh_lattice_step(rh_sim* sim);

/* Waveform of an RH_PROTO_AP_CLAMP cell: n = (int)(pcl_ms/dt + 0.1) voltages
 * (mV), sample k applied at the steps whose (int)(t/dt + 0.1) is k modulo n
 * (the reference reads them from v_1000.txt, :383-395).  Copied; must be set
 * before such a cell runs (rh_run_steps fails with RH_ERR_STATE otherwise). */
int rh_set_ap_clamp(rh_sim* sim, int32_t cell, const double* v_mV, int64_t n);

/* Number of cells / interior CRUs of a cell. */
int rh_num_cells(const rh_sim* sim, int32_t* ncells);
int rh_cell_size(const rh_sim* sim, int32_t cell, int32_t* n_interior);

/* State transfer (host <-> device) for one cell. */
int rh_get_state(rh_sim* sim, int32_t cell, rh_state_f64* dst);
int rh_set_state(rh_sim* sim, int32_t cell, const rh_state_f64* src);
int rh_get_membrane(rh_sim* sim, int32_t cell, rh_membrane* dst);
int rh_set_membrane(rh_sim* sim, int32_t cell, const rh_membrane* src);

/* Output records produced since the last drain: wholecell rows of 45 columns
 * (:1041-1072) and linescan blocks of (nx-2) rows x 22 columns (:974-989).
 * `*nrec` receives the number of records copied; records beyond `max_rec`
 * stay queued. */
int rh_drain_wholecell(rh_sim* sim, int32_t cell, double* rows, int32_t max_rec,
                       int32_t* nrec);
int rh_drain_linescan(rh_sim* sim, int32_t cell, double* rows, int32_t max_rec,
                      int32_t* nrec);

/* rh_drain_wholecell for every cell in one call (two device-to-host copies
 * in all, instead of one round trip per cell and record): the records of
 * cell c go to rows + c * max_rec * 45 and their number to nrec[c].  Replaces
 * the reference's per-output-step host loop over the wholecell statistics
 * (cuda_Cell_Detailed.cu:777-1072) for a batch of cells. */
int rh_drain_wholecell_all(rh_sim* sim, double* rows, int32_t max_rec, int32_t* nrec);
int rh_drain_stats(rh_sim* sim, int32_t cell, rh_beat_stats* out, int32_t max_rec,
                   int32_t* nrec);

/* cadist records produced since the last drain (run option record_cadist):
 * each is 2 + 6*n doubles (n interior CRUs), t and V, then per CRU in the
 * reference's order (jx outer, jy, jz inner) ci of sub-voxel 0, cs, cp, cjsr,
 * xinaca/Cm*0.0965*Vs*16120 and xire, the values the reference prints
 * (:1005, :1009).  Returns RH_ERR_ARG when record_cadist is off. */
int rh_drain_cadist(rh_sim* sim, int32_t cell, double* rec, int32_t max_rec, int32_t* nrec);

/* Per-beat statistics of a recorded trace, with the same detectors the
 * simulator runs on the GPU (for traces produced elsewhere, e.g. by a CPU
 * model): t and v are the per-step (time, membrane voltage after the step)
 * samples, wholecell the output records of the same run.  Host-only. */
int rh_analyze_trace(double pcl_ms, const double* t, const double* v, int64_t nsteps,
                     const double* wholecell, int32_t nrec, rh_beat_stats* out, int32_t max_rec,
                     int32_t* nbeats);

/* Status bits of a cell (RH_STATUS_*). */
int rh_cell_status(rh_sim* sim, int32_t cell, uint32_t* status);

/* Binary snapshot of every cell's lattice + membrane state and step counter.
 * With counter-based random numbers a restored run continues bit-identically. */
int rh_checkpoint(rh_sim* sim, const char* path);
int rh_restore(rh_sim* sim, const char* path);

/* Bulk state transfer for callers that keep the whole batch on the host
 * between calls: the native lattice state of every cell plus the per-cell
 * dynamic state, as one opaque block of rh_state_bytes() bytes (the same
 * content a checkpoint holds).  Host buffers may be pageable or pinned. */
int rh_state_bytes(const rh_sim* sim, size_t* bytes);
int rh_export_state(rh_sim* sim, void* host, size_t bytes);
int rh_import_state(rh_sim* sim, const void* host, size_t bytes);

/* rh_import_state(host_in) + rh_run_steps(nsteps) + rh_export_state(host_out)
 * in one call, with the same result.  Either buffer may be NULL (no import,
 * no export), both may be the same buffer, and `bytes` is rh_state_bytes().
 * On the two-launch path with pinned (or registered) buffers the copies are
 * split by cell group: each group's import opens its branch of the first
 * window and its export closes its branch of the last window, so one group's
 * copies overlap the other groups' steps.  Otherwise (persistent launch,
 * pageable buffers) the copies run before and after the steps.  The kernel
 * timing (rh_kernel_timing) of such a call includes its copies. */
int rh_run_steps_host(rh_sim* sim, int64_t nsteps, const void* host_in, void* host_out,
                      size_t bytes);

/* CRU-tile autotuner within the simulator's launch mode.  The step kernel is
 * compiled for tiles of 64, 128 and 256 CRUs per CTA (each with its own
 * register/occupancy bound).  Times `steps` lattice updates of the live
 * workload with each candidate, starting every candidate from a device-side
 * copy of the current state and restoring that state afterwards (the
 * simulation does not advance), then keeps the fastest.  ms_per_step (3
 * entries, may be NULL) receives the timings.  rh_autotune_shapes searches
 * the launch mode, CTAs per SM and cell groups as well. */
int rh_autotune(rh_sim* sim, int32_t steps, int32_t* tile_crus, double* ms_per_step);
int rh_tile_size(const rh_sim* sim, int32_t* tile_crus);

/* How the time steps of a simulator are launched: the autotuner's search
 * space.  The reference launches one Compute kernel of 48 CTAs of (16,7,4)
 * threads per step (cuda_Cell_Detailed.cu:155-158, :292-295, :420); here the
 * shape is chosen per device and workload. */
typedef struct {
  int32_t persistent;   /* 1 = one persistent cooperative launch per window,
                           0 = two launches per step and cell group */
  int32_t tile_crus;    /* CRUs (threads) per CTA: 64, 128 or 256; the
                           persistent launch takes 64 or 128 */
  int32_t fewer_ctas;   /* persistent launch only: 1 = one resident CTA per SM
                           fewer than the step kernel holds, with more registers
                           per thread (cells without build options only) */
  int32_t cell_groups;  /* two-launch path: cell groups on concurrent streams */
  int32_t bulk_staging; /* two-launch path, FP32 lattice: 0 = every thread
                           copies its share with cp.async; 1 = a tile's own
                           state and its stencil halo rows arrive by bulk
                           asynchronous copies issued by one warp (completion
                           on mbarriers); 2 = the tile's ci/cnsr pair planes and
                           its eight real planes arrive as 2-D tensor tiles
                           (cp.async.bulk.tensor, one thread), the rest as in 0 */
} rh_launch_shape;

int rh_get_launch_shape(const rh_sim* sim, rh_launch_shape* shape);

/* Switches the simulator to `shape` (state and outputs are unaffected).
 * RH_ERR_NOTBUILT for a shape no kernel is compiled for or the device cannot
 * run (a persistent launch with tiles of 256, or with fewer_ctas when some
 * cell uses a build option). */
int rh_set_launch_shape(rh_sim* sim, const rh_launch_shape* shape);

/* Launch-shape autotuner.  Times `steps` lattice updates of the live
 * workload with every candidate shape (persistent launches with tiles of 64
 * and 128 at both CTA counts; two-launch windows with tiles of 64, 128 and
 * 256 at 8, 12, 16 and 24 cell groups, in mixed precision with each staging),
 * each from a device-side copy of the
 * current state that is restored afterwards (the simulation does not
 * advance), and switches to the fastest.  The choice is cached for the
 * process by device, precision and lattice classes (the cells' interior x
 * and y extents in steps of 16 and their CRU total): a later simulator of
 * the same workload on the same device reuses it without timing (then
 * *ntried = 0).  With the environment variable RH_SHAPE_CACHE naming a
 * file, choices are also appended to it and read from it, so that later
 * processes reuse them too.  tried/ms_per_step (max_tried entries each, may be NULL)
 * receive the candidates and their ms per lattice update of every cell. */
int rh_autotune_shapes(rh_sim* sim, int32_t steps, rh_launch_shape* best,
                       rh_launch_shape* tried, double* ms_per_step, int32_t max_tried,
                       int32_t* ntried);

/* Algorithmic HBM bytes moved per interior CRU per lattice update for the
 * simulator's precision (each persistent field read once, written once). */
int rh_bytes_per_cru_step(const rh_sim* sim, double* bytes);

/* Device time of the lattice updates, accumulated since the last call (CUDA
 * events on the simulator's stream around the work it enqueued); returns the
 * number of lattice updates (time steps) and milliseconds.  Each update is
 * two kernel launches per cell group (rh_num_groups): the lattice step and
 * the cells' whole-cell update. */
int rh_kernel_timing(rh_sim* sim, int64_t* launches, double* ms);

/* Number of cell groups advanced on concurrent streams (run option
 * cell_groups, capped at the number of cells). */
int rh_num_groups(const rh_sim* sim, int32_t* groups);

/* Kernel launches issued for time steps since the simulator was created:
 * one per window with the persistent launch, two per step and cell group
 * otherwise.  *persistent receives whether windows run as persistent
 * launches (the run option, unless the tile length or the device rules it
 * out); either pointer may be NULL. */
int rh_kernel_launches(const rh_sim* sim, int64_t* launches, int32_t* persistent);

/* CTAs of the persistent window launch (its grid: every CTA the device holds
 * at once for the simulator's tile length), 0 when windows do not run
 * persistently. */
int rh_window_ctas(const rh_sim* sim, int32_t* ctas);

/* Testing hook of the persistent launch's bounded waits: `polls` is the
 * number of polls (about 1 us apart) after which a wait gives up (0 = the
 * default, about 0.3 s), `target_offset` is added to the step every wait
 * waits for (0 = normal).  An offset that no cell reaches makes every wait
 * run out: the next rh_run_steps returns RH_ERR_TIMEOUT and the cells carry
 * RH_STATUS_TIMEOUT, with the GPU context intact. */
int rh_set_wait_limit(rh_sim* sim, int64_t polls, uint32_t target_offset);

/* Copies the text of the last error into buf (always NUL-terminated). */
int rh_last_error(const rh_sim* sim, char* buf, size_t n);

/* Formats a wholecell record or one linescan row exactly as the reference's
 * fprintf calls do (:1041-1072, :974-989).  Returns the string length. */
int rh_format_wholecell(const double* cols45, char* buf, size_t n);
int rh_format_linescan(const double* cols22, char* buf, size_t n);

#ifdef __cplusplus
}
#endif

#endif /* RH_H */
