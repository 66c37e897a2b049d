// beatstats.cuh — per-beat statistics of one cell from its voltage trace and
// its output records.  The reference defines none of these; the definitions
// below are this project's, and the same code runs on the GPU (in the cell
// update of every step) and on the host (rh_analyze_trace, applied to CPU
// oracle traces).
//
// A beat k starts at the k-th stimulus onset t_k = 100 + k*PCL (the stimulus
// rule of cuda_Cell_Detailed.cu:689-692) and ends at the next one.  From the
// per-step samples (t, V) after each membrane update:
//   v_rest   V at the first sample of the beat;
//   t_act    first time V crosses -40 mV upwards (no crossing: no AP);
//   v_peak   maximum V of the beat;
//   APD90    time of the first fall below v_peak - 0.9 (v_peak - v_rest)
//            after the peak, minus t_act; -1 when the AP does not
//            repolarise within the beat or never fired;
//   EAD      from t_act + 50 ms until the AP has repolarised below -60 mV,
//            V rising 3 mV or more above its running minimum.
// From the output records (every 2.5 ms):
//   ci_peak  maximum of mean [Ca]i (column 2) over the beat's records;
//   sr_load  mean JSR [Ca] (column 8) of the last record before the beat's
//            stimulus (diastolic SR load);
//   sparks   sum of column 41 (spark onsets per window) over the beat.
#pragma once

#include <math.h>

#include "../../include/rh.h"

namespace rh {

constexpr double kStimStart = 100.0;
constexpr double kActThreshold = -40.0;
constexpr double kEadDelay = 50.0;
constexpr double kEadRise = 3.0;
constexpr double kEadRepolarised = -60.0;

struct BeatTracker {
  int beat;        // index of the beat in progress, -1 before the first stimulus
  int fired;       // t_act seen
  int repolarised; // APD90 crossing seen
  int ead;
  int sparks;
  int ead_armed;   // running minimum tracking active
  double t0, v_rest, v_peak, t_peak, t_act, apd90, v_min;
  double ci_peak, sr_load, last_cjsr;
};

__host__ __device__ inline void beat_reset(BeatTracker& b) {
  b.beat = -1;
  b.fired = b.repolarised = b.ead = b.sparks = b.ead_armed = 0;
  b.t0 = b.v_rest = b.v_peak = b.t_peak = b.t_act = 0.0;
  b.apd90 = -1.0;
  b.v_min = 0.0;
  b.ci_peak = 0.0;
  b.sr_load = -1.0;
  b.last_cjsr = -1.0;
}

__host__ __device__ inline void beat_finish(const BeatTracker& b, rh_beat_stats* out) {
  out->beat = b.beat;
  out->ead = b.ead;
  out->apd90_ms = b.repolarised && b.fired ? b.apd90 : -1.0;
  out->v_peak = b.v_peak;
  out->ci_peak = b.ci_peak;
  out->sr_load = b.sr_load;
  out->sparks = b.sparks;
  out->pad = 0;
}

// One per-step sample.  Returns 1 when a beat completed; its statistics are
// written to *out.
__host__ __device__ inline int beat_on_step(BeatTracker& b, double t, double v, double pcl,
                                            rh_beat_stats* out) {
  int done = 0;
  int k = t < kStimStart ? -1 : (int)floor((t - kStimStart) / pcl);
  if (k != b.beat && k >= 0) {
    if (b.beat >= 0) {
      beat_finish(b, out);
      done = 1;
    }
    double sr = b.last_cjsr;
    b.beat = k;
    b.fired = b.repolarised = b.ead = b.sparks = b.ead_armed = 0;
    b.t0 = t;
    b.v_rest = v;
    b.v_peak = v;
    b.t_peak = t;
    b.t_act = t;
    b.apd90 = -1.0;
    b.v_min = v;
    b.ci_peak = 0.0;
    b.sr_load = sr;
  }
  if (b.beat < 0) return done;
  if (!b.fired && v > kActThreshold) {
    b.fired = 1;
    b.t_act = t;
  }
  if (v > b.v_peak && !b.repolarised) {
    b.v_peak = v;
    b.t_peak = t;
  }
  if (b.fired && !b.repolarised && t > b.t_peak) {
    double v90 = b.v_peak - 0.9 * (b.v_peak - b.v_rest);
    if (v < v90) {
      b.repolarised = 1;
      b.apd90 = t - b.t_act;
    }
  }
  if (b.fired && t >= b.t_act + kEadDelay) {
    if (!b.ead_armed) {
      b.ead_armed = 1;
      b.v_min = v;
    }
    if (b.ead_armed && b.v_min > kEadRepolarised) {
      if (v < b.v_min) b.v_min = v;
      if (v >= b.v_min + kEadRise) b.ead = 1;
    }
  }
  return done;
}

// One output record (the 45 wholecell columns).
__host__ __device__ inline void beat_on_output(BeatTracker& b, const double* w) {
  b.last_cjsr = w[7];
  if (b.beat < 0) return;
  if (w[1] > b.ci_peak) b.ci_peak = w[1];
  b.sparks += (int)w[40];
}

}  // namespace rh
