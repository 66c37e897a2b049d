/*
 * rh_oracle.h — CPU oracle for the per-time-step myocyte update.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference's lattice update (cuda_Cell_Detailed.cu `Compute`, :1187-1692,
 * with the "fixA" choice of keeping block A :1356-1473), its Init kernel
 * (:1108-1182), the host whole-cell reduction and membrane model (:427-739)
 * and the output statistics (:777-1081).  Random numbers come from the shared
 * Philox provider (include/rh_philox.h) in the reference's draw order.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
 * as the checker.  The product never links or calls it.
 *
 * The oracle keeps the reference's memory model: the full lattice including
 * the ghost shell, ping-pong ci/cnsr/cs arrays and ghost-face copies.
 */
#ifndef RH_ORACLE_H
#define RH_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/rh.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

orc_sim* orc_create(const rh_cell_params* p, double dt);
void orc_destroy(orc_sim* s);
void orc_set_threads(int nthreads);
int orc_get_threads(void);

/* One iteration of the reference's time loop (:399-1085): lattice update,
 * whole-cell reduction, membrane model, output bookkeeping, t += dt.
 * Returns 1 when this step produced an output record, -1 (nothing done) for an
 * AP-clamp cell without its waveform. */
int orc_step(orc_sim* s);

/* Runs `nsteps` iterations (or until the protocol ends) and copies each
 * output record (45 doubles) and linescan block ((nx-2) x 22 doubles) into the
 * caller's arrays while they have room.  Returns the steps actually run. */
int64_t orc_run(orc_sim* s, int64_t nsteps, double* wholecell, int32_t max_rec,
                int32_t* nrec, double* linescan, int32_t max_blocks, int32_t* nblocks);

/* As orc_run, also recording each step's time (before the step) and
 * membrane voltage (after it): the samples the per-beat detectors use. */
int64_t orc_run_traced(orc_sim* s, int64_t nsteps, double* t_out, double* v_out,
                       double* wholecell, int32_t max_rec, int32_t* nrec);

/* Lattice update only (Compute + ping-pong swap) with the current v, t, xnai. */
void orc_lattice_step(orc_sim* s);

/* Interior-only state exchange in the rh_state_f64 layout of include/rh.h. */
void orc_get_state(const orc_sim* s, rh_state_f64* dst);
void orc_set_state(orc_sim* s, const rh_state_f64* src);
void orc_get_membrane(const orc_sim* s, rh_membrane* dst);
void orc_set_membrane(orc_sim* s, const rh_membrane* src);

/* Last output record / linescan block (valid after orc_step returned 1). */
void orc_last_wholecell(const orc_sim* s, double* cols45);
int32_t orc_last_linescan(const orc_sim* s, double* rows);
/* cadist record of the last step (t, v, then 6 values per interior CRU in the
 * reference's jx-outer order) if that step wrote one: returns the number of
 * CRUs, else 0. */
int32_t orc_last_cadist(const orc_sim* s, double* rec);

int32_t orc_protocol_done(const orc_sim* s);
/* Waveform of an RH_PROTO_AP_CLAMP cell: (int)(pcl/dt + 0.1) voltages, the
 * values the reference reads from v_1000.txt (:383-395).  0 on success. */
int32_t orc_set_ap_clamp(orc_sim* s, const double* v, int64_t n);
uint32_t orc_status(const orc_sim* s);
int32_t orc_interior(const orc_sim* s);

/* Output formatting as the reference's fprintf calls (:1041-1072, :974-989). */
int orc_format_wholecell(const double* cols45, char* buf, size_t n);
int orc_format_linescan(const double* cols22, char* buf, size_t n);

#ifdef __cplusplus
}
#endif

#endif
