// cellwarp.cuh — the whole-cell FP64 update (membrane_update and step_coef of
// cellmodel.cuh) computed by one full warp.
//
// FP64 runs at a small fraction of the FP32 rate on this GPU, and a warp
// instruction costs the FP64 pipe the same time whether one lane or 32 lanes
// are active.  The serial versions evaluate some 55 exponentials, 60
// divisions, three logarithms and three fmods one after the other in one
// lane; here every group of mutually independent transcendentals and
// divisions is evaluated in one SIMT call, one operand set per lane, through
// a 32-slot shared-memory exchange.  Each operation keeps its operands and
// its order, so the results are bit-identical to the serial versions; only
// the lane that computes each value changes.  The reference's two powers,
// pow(0.28/csubt, 3) and pow(12/xnai, 1), are a product and the quotient
// itself in both versions (the CPU oracle keeps pow; the results differ in
// the last bits).
//
// The membrane step is split at the point where it needs the lattice sums:
// membrane_pre_warp runs while the cell's lattice launch is still finishing,
// membrane_post_warp after it.
//
// All 32 lanes of the calling warp must be active and call with identical
// arguments; every lane returns the same results.
#pragma once

#include <math.h>

#include "cellmodel.cuh"

namespace rh {

// Argument of one exponential of a per-lane table:
//   u = {v, v - ek, XNAO}[src];  t = u + a;
//   w = div ? t / d : t * c;  w = w * c2;  arg = sq ? (-w) * w : w
// Each entry restates one exp() argument of membrane_update (the comment
// gives the original form; (-x)/d equals x/(-d) and x - b equals x + (-b)
// exactly in IEEE arithmetic, and x * 1 = x).
struct ExpArg {
  double a, c, d, c2;
  int src, div, sq, pad;
};

enum { kSrcV = 0, kSrcVek = 1, kSrcNao = 2 };

#define RH_MUL(c_, a_) {a_, c_, 1.0, 1.0, kSrcV, 0, 0, 0}
#define RH_DIV(a_, d_) {a_, 1.0, d_, 1.0, kSrcV, 1, 0, 0}
#define RH_NONE {0.0, 0.0, 1.0, 1.0, kSrcV, 0, 0, 0}

// v < -40 mV (cuda_Cell_Detailed.cu:466-476 branch taken)
__device__ const ExpArg kMemExpLow[32] = {
    RH_MUL(-0.1, 47.13),                        // 0  am: -0.1*(v+47.13)
    RH_DIV(0.0, -11.0),                         // 1  bm: -v/11
    RH_DIV(80.0, -6.8),                         // 2  ah: (80+v)/(-6.8)
    RH_MUL(0.079, 0.0),                         // 3  bh: 0.079*v
    RH_MUL(0.35, 0.0),                          // 4  bh: 0.35*v
    RH_MUL(0.2444, 0.0),                        // 5  aj: 0.2444*v
    RH_MUL(-0.04391, 0.0),                      // 6  aj: -0.04391*v
    RH_MUL(0.311, 79.23),                       // 7  aj: 0.311*(v+79.23)
    RH_MUL(-0.01052, 0.0),                      // 8  bj: -0.01052*v
    RH_MUL(-0.1378, 40.14),                     // 9  bj: -0.1378*(v+40.14)
    RH_MUL(-0.123, 7.00),                       // 10 xkrv1: -0.123*(v+7)
    RH_MUL(0.1450, 10.00),                      // 11 xkrv2: 0.145*(v+10)
    RH_DIV(50.00, -7.50),                       // 12 xkrinf: -(v+50)/7.5
    RH_DIV(33.00, 22.40),                       // 13 rg: (v+33)/22.4
    RH_DIV(-1.500, -16.700),                    // 14 xs1ss: -(v-1.5)/16.7
    RH_MUL(-0.1480, 30.0),                      // 15 tauxs: -0.148*(v+30)
    RH_MUL(0.06870, 30.00),                     // 16 tauxs: 0.0687*(v+30)
    {-59.215, 0.2385, 1.0, 1.0, kSrcVek, 0, 0, 0},   // 17 aki: 0.2385*(v-ek-59.215)
    {5.476, 0.08032, 1.0, 1.0, kSrcVek, 0, 0, 0},    // 18 bki: 0.08032*(v-ek+5.476)
    {-594.31, 0.061750, 1.0, 1.0, kSrcVek, 0, 0, 0}, // 19 bki: 0.06175*(v-ek-594.31)
    {4.753, -0.5143, 1.0, 1.0, kSrcVek, 0, 0, 0},    // 20 bki: -0.5143*(v-ek+4.753)
    RH_DIV(3.0, -15.00),                        // 21 rt1 = -(v+3)/15
    RH_DIV(33.5, 10.00),                        // 22 rt2 = rt5 = (v+33.5)/10
    RH_DIV(3.0, 15.00),                         // 23 -rt1
    RH_DIV(60.00, 10.00),                       // 24 rt3 = (v+60)/10
    {0.0, 1.0, 30.00, 1.0, kSrcV, 1, 1, 0},     // 25 rt4 = -(v/30)*(v/30)
    {0.0, 1.0, 67.30, 1.0, kSrcNao, 1, 0, 0},   // 26 sigma: XNAO/67.3
    {0.0, -0.1, 1.0, FRT, kSrcV, 0, 0, 0},      // 27 fnak: -0.1*v*FRT
    RH_MUL(-FRT, 0.0),                          // 28 fnak: -v*FRT
    RH_NONE, RH_NONE, RH_NONE};

// v >= -40 mV: entries 2-4 are the other branch's, 5-9 unused
__device__ const ExpArg kMemExpHigh[32] = {
    RH_MUL(-0.1, 47.13),
    RH_DIV(0.0, -11.0),
    RH_DIV(10.66, -11.10),                      // 2  bh: (v+10.66)/(-11.1)
    RH_MUL(-0.00000025350, 0.0),                // 3  bj: -2.535e-7*v
    RH_MUL(-0.10, 32.00),                       // 4  bj: -0.1*(v+32)
    RH_NONE, RH_NONE, RH_NONE, RH_NONE, RH_NONE,
    RH_MUL(-0.123, 7.00),
    RH_MUL(0.1450, 10.00),
    RH_DIV(50.00, -7.50),
    RH_DIV(33.00, 22.40),
    RH_DIV(-1.500, -16.700),
    RH_MUL(-0.1480, 30.0),
    RH_MUL(0.06870, 30.00),
    {-59.215, 0.2385, 1.0, 1.0, kSrcVek, 0, 0, 0},
    {5.476, 0.08032, 1.0, 1.0, kSrcVek, 0, 0, 0},
    {-594.31, 0.061750, 1.0, 1.0, kSrcVek, 0, 0, 0},
    {4.753, -0.5143, 1.0, 1.0, kSrcVek, 0, 0, 0},
    RH_DIV(3.0, -15.00),
    RH_DIV(33.5, 10.00),
    RH_DIV(3.0, 15.00),
    RH_DIV(60.00, 10.00),
    {0.0, 1.0, 30.00, 1.0, kSrcV, 1, 1, 0},
    {0.0, 1.0, 67.30, 1.0, kSrcNao, 1, 0, 0},
    {0.0, -0.1, 1.0, FRT, kSrcV, 0, 0, 0},
    RH_MUL(-FRT, 0.0),
    RH_NONE, RH_NONE, RH_NONE};

#undef RH_MUL
#undef RH_DIV
#undef RH_NONE

// 32-slot exchange of one warp: lane 0 deposits operands, every lane
// evaluates its slot, every lane reads back any slot.
struct WarpSlots {
  double* n;  // [32] numerators / first operands
  double* d;  // [32] denominators / second operands
  double* r;  // [32] results
  int lane;

  // operands of slots 0..k-1 come from lane 0; the other slots get n = 0, d = 1
  __device__ __forceinline__ void open(int k) {
    __syncwarp();
    if (lane >= k) {
      n[lane] = 0.0;
      d[lane] = 1.0;
    }
  }
  __device__ __forceinline__ void put(int i, double a, double b) {
    if (lane == 0) {
      n[i] = a;
      d[i] = b;
    }
  }
  // every lane: its slot's quotient n/d, published in r
  __device__ __forceinline__ void divide() {
    __syncwarp();
    const double q = n[lane] / d[lane];
    r[lane] = q;
    __syncwarp();
  }
  __device__ __forceinline__ double get(int i) const { return r[i]; }
};

// Results of the membrane step (membrane_update, cellmodel.cuh) that do not
// depend on the step's lattice sums: the currents of the old state, the
// stimulus and the two constants of the qks update.
struct MembranePre {
  double xina, xikr, xiks, xik1, xitos, xitof, xinak, stim;
  double qks_num, tauqks;  // qks_inf = 0.2 (1 + qks_num / (1 + (0.28/csubt)^3))
  // the time-step constants of StepCoef: 1/dt, dt/5, 0.95/dt, 0.95/(dt/5)
  double rdt, dth, rdt95, rdth95;
};

// The qks update, which needs csubt and nothing downstream of the new
// voltage; step_coef_warp evaluates it in spare slots of its own rounds.
struct QksStep {
  double csubt, qks, qks_num, tauqks;  // in
  double dqks;                          // out: dt (qks_inf - qks) / tauqks
};

// Membrane step by one warp, first part: everything that needs only the
// state of the previous step (:458-700 without the reduction), run before
// the cell update waits for its lattice launch.  Gates are advanced in `m`;
// m.qks, m.xnai, m.v and the reduction quotients are left to
// membrane_post_warp.  `s` is 160 doubles of shared memory owned by the warp;
// fm[0..5] receives the fmods of this step (stimulus phase and the next
// lattice update's window flags: reset, output, the two cadist conditions and
// the iso LCC phase).
__device__ inline void membrane_pre_warp(rh_membrane& m, double dt, const CellConst& c, double* s,
                                         double fm[6], MembranePre& P) {
  const double tperid = c.pcl, svikr = c.svikr;
  const int lane = threadIdx.x & 31;
  WarpSlots w{s, s + 32, s + 64, lane};
  const double t = m.t, v = m.v;
  const double xki = 140.0, xko = 5.40;  // :350-351
  const double xnai = m.xnai;
  const double prnak = 0.0183300;

  // ---- round 0: log arguments and the INaK quotient ----
  w.open(7);
  w.put(0, XNAO, xnai);                                  // ena
  w.put(1, xko, xki);                                    // ek
  w.put(2, xko + prnak * XNAO, xki + prnak * xnai);      // eks
  w.put(3, 12.00, xnai);                                 // INaK base, 12/xnai
  w.put(4, 1.0, dt);                                     // rdt
  w.put(5, dt, 5.0);                                     // dth
  w.put(6, 0.95, dt);                                    // rdt95
  w.divide();
  P.rdt = w.get(4);
  P.dth = w.get(5);
  P.rdt95 = w.get(6);
  // logarithms (lanes 0-2)
  const double lgv = log(w.r[lane]);
  const double ena = (1.0 / FRT) * __shfl_sync(0xffffffffu, lgv, 0);
  const double ek = (1.00 / FRT) * __shfl_sync(0xffffffffu, lgv, 1);
  const double eks = (1.00 / FRT) * __shfl_sync(0xffffffffu, lgv, 2);
  const double pow_nak = w.get(3);  // pow(12/xnai, 1) = 12/xnai
  // fmods: stimulus phase (:689, iso :683) and the next update's window,
  // output, cadist and iso LCC flags (:1244, :777, :1002, :1213)
  {
    const double tn = t + dt;
    const double x = lane == 0 ? (c.iso ? t : t + tperid - 100)
                   : lane == 1 ? tn - dt
                   : lane == 5 ? tn + 10 * tperid
                               : tn + 0.0000001;
    const double y = lane == 0 ? tperid : lane == 3 ? 5.0 : lane == 4 ? tperid
                   : lane == 5 ? 15.5 * tperid : OUTT;
    const double f = fmod(x, y);
#pragma unroll
    for (int i = 0; i < 6; ++i) fm[i] = __shfl_sync(0xffffffffu, f, i);
  }

  // ---- round 1: the voltage exponentials, one per lane ----
  double* const E = s + 96;  // E[i] = exp of table entry i
  {
    const ExpArg* tab = (v < -40.0) ? kMemExpLow : kMemExpHigh;
    const ExpArg ea = tab[lane];
    const double vek = v - ek;
    const double u = ea.src == kSrcV ? v : (ea.src == kSrcVek ? vek : XNAO);
    const double tt = u + ea.a;
    const double q = tt / ea.d;
    double z = ea.div ? q : tt * ea.c;
    z = z * ea.c2;
    const double arg = ea.sq ? (-z) * z : z;
    const double ex = exp(arg);
    __syncwarp();
    E[lane] = ex;
    __syncwarp();
  }
  const bool low = v < -40.0;

  // ---- round 2: first-level divisions ----
  const double bm = 0.08 * E[1];
  double ah, bh, aj, bj, am;
  w.open(20);
  w.put(0, 0.32 * (v + 47.13), 1.0 - E[0]);                    // am
  if (low) {
    w.put(1, v + 37.78, 1.0 + E[7]);                           // aj factor
    w.put(2, 0.1212 * E[8], 1.0 + E[9]);                       // bj
  } else {
    w.put(1, 1.00, 0.130 * (1.00 + E[2]));                     // bh
    w.put(2, 0.3 * E[3], 1.0 + E[4]);                          // bj
  }
  w.put(3, 0.001380 * (v + 7.00), 1.0 - E[10]);                // xkrv1
  w.put(4, 0.000610 * (v + 10.00), E[11] - 1.00);              // xkrv2
  w.put(5, 1.00, 1.00 + E[12]);                                // xkrinf
  w.put(6, 1.00, 1.00 + E[13]);                                // rg
  w.put(7, 1.0, 1.0 + pow_nak);                                // INaK factor
  w.put(8, 1.0, 1.0 + E[14]);                                  // xs1ss
  w.put(9, 0.0000719 * (v + 30.00), 1.00 - E[15]);             // tauxs term 1
  w.put(10, 0.0001310 * (v + 30.00), E[16] - 1.00);            // tauxs term 2
  w.put(11, 1.02, 1.0 + E[17]);                                // aki
  w.put(12, 0.49124 * E[18] + E[19], 1.0 + E[20]);             // bki
  w.put(13, 1.00, 1.0 + E[21]);                                // xtos_inf
  w.put(14, 1.00, 1.00 + E[22]);                               // ytos_inf = rs_inf
  w.put(15, 9.00, 1.00 + E[23]);                               // txs
  w.put(16, 3000.00, 1.0 + E[24]);                             // tys
  w.put(17, 20.0, 1.0 + E[22]);                                // tyf
  w.put(18, E[26] - 1.00, 7.00);                               // sigma
  w.put(19, 0.95, P.dth);                                      // rdth95
  w.divide();
  P.rdth95 = w.get(19);
  am = w.get(0);
  if (low) {
    ah = 0.135 * E[2];
    bh = 3.56 * E[3] + 310000.0 * E[4];
    aj = (-127140.0 * E[5] - 0.00003474 * E[6]) * w.get(1);
    bj = w.get(2);
  } else {
    ah = 0.00;
    bh = w.get(1);
    aj = 0.00;
    bj = w.get(2);
  }
  const double xkrv1 = w.get(3), xkrv2 = w.get(4), xkrinf = w.get(5), rg = w.get(6);
  const double nak_f = w.get(7);
  const double xs1ss = w.get(8);
  const double aki = w.get(11), bki = w.get(12);
  const double xtos_inf = w.get(13), ytos_inf = w.get(14), rs_inf = w.get(14);
  const double txs = w.get(15) + 0.50, tys = w.get(16) + 30.00;
  const double txf = 3.50 * E[25] + 1.50, tyf = w.get(17) + 20.00;
  const double sigma = w.get(18);
  const double tauxs_sum = w.get(9) + w.get(10);

  // ---- round 3: second-level divisions ----
  w.open(10);
  w.put(0, 1.00, ah + bh);                                     // tauh
  w.put(1, 1.00, aj + bj);                                     // tauj
  w.put(2, 1.00, am + bm);                                     // taum
  w.put(3, ah, ah + bh);
  w.put(4, aj, aj + bj);
  w.put(5, am, am + bm);
  w.put(6, 1.00, xkrv1 + xkrv2);                               // taukr
  w.put(7, 1.00, tauxs_sum);                                   // tauxs
  w.put(8, aki, aki + bki);                                    // xkin
  w.put(9, 1.00, 1.0 + 0.1245 * E[27] + 0.0365 * sigma * E[28]);  // fnak
  w.divide();
  const double tauh = w.get(0), tauj = w.get(1), taum = w.get(2);
  const double rh_ = w.get(3), rj_ = w.get(4), rm_ = w.get(5);
  const double taukr = w.get(6);
  const double tauxs = 0.95 * w.get(7);
  const double xkin = w.get(8), fnak = w.get(9);

  // ---- round 4: gate exponent arguments and INaK ----
  w.open(10);
  w.put(0, -dt, tauh);
  w.put(1, -dt, tauj);
  w.put(2, -dt, taum);
  w.put(3, -dt, taukr);
  w.put(4, -dt, tauxs);
  w.put(5, -dt, txs);
  w.put(6, -dt, tys);
  w.put(7, -dt, txf);
  w.put(8, -dt, tyf);
  w.put(9, 1. * 1.5000 * fnak * nak_f * xko, xko + 1.50);      // xinak
  w.divide();
  P.xinak = w.get(9);
  double* const G = s + 128;  // exp(-dt/tau) of the nine gates
  {
    const double ge = exp(lane < 9 ? w.r[lane] : 0.0);
    G[lane] = ge;
    __syncwarp();
  }

  // ---- currents of the old state and the gate updates (identical in
  //      every lane) ----
  const double gna = 15;
  const double gnaleak = 0.3e-3 * 5;
  P.xina = gna * m.xh * m.xj * m.xm * m.xm * m.xm * (v - ena) + gnaleak * (v - ena);
  m.xh = rh_ - (rh_ - m.xh) * G[0];
  m.xj = rj_ - (rj_ - m.xj) * G[1];
  m.xm = rm_ - (rm_ - m.xm) * G[2];
  const double gss = sqrt(xko / 5.40);
  const double gkr = 0.0078360;
  P.xikr = svikr * gkr * gss * m.xr * rg * (v - ek);
  m.xr = xkrinf - (xkrinf - m.xr) * G[3];
  const double gksx = 0.2000;
  P.xiks = 1.0 * 1. * gksx * m.qks * m.xs1 * m.xs2 * (v - eks);
  m.xs1 = xs1ss - (xs1ss - m.xs1) * G[4];
  m.xs2 = xs1ss - (xs1ss - m.xs2) * G[4];
  P.qks_num = c.slowncx ? 1.6 : 0.8;         // :537, :541
  P.tauqks = c.slowncx ? 2000 : 1000.00;     // :538, :542
  const double gki = 0.600 * (sqrt(xko / 5.4));
  P.xik1 = (1.0) * gki * xkin * (v - ek);
  P.xitos = 1.0 * 0.040 * m.xtos * (m.ytos + 0.50 * rs_inf) * (v - ek);
  m.xtos = xtos_inf - (xtos_inf - m.xtos) * G[5];
  m.ytos = ytos_inf - (ytos_inf - m.ytos) * G[6];
  P.xitof = 1.0 * 0.10 * m.xtof * m.ytof * (v - ek);
  m.xtof = xtos_inf - (xtos_inf - m.xtof) * G[7];
  m.ytof = ytos_inf - (ytos_inf - m.ytof) * G[8];
  P.stim = stimulus(c, t, fm[0]);
}

// Membrane step by one warp, second part, once the lattice sums tot (sum cs,
// sum xicat, sum xinaca over the cell's CRUs, :447-456) are in: the
// reduction quotients, [Na]i and V (:701-738), and the currents into `m`.
// m.t and m.v still hold the old step's time and voltage.
__device__ inline void membrane_post_warp(rh_membrane& m, double dt, const CellConst& c,
                                          const double tot[3], double* s, const MembranePre& P) {
  const int lane = threadIdx.x & 31;
  WarpSlots w{s, s + 32, s + 64, lane};
  const double t = m.t, v = m.v;
  const double xnai = m.xnai;
  w.open(3);
  w.put(0, tot[0], (double)c.n);                         // csubt (:447)
  w.put(1, tot[1], CM);                                  // xicatto (:452)
  w.put(2, tot[2], CM);                                  // xinacato (:456)
  w.divide();
  m.csubt = w.get(0);
  m.xicatto = w.get(1) * 0.0965 * VP * 2.0 * (ICAGAMMA + 1.);
  m.xinacato = w.get(2) * 0.0965 * VS;
  const double wcainv = 1.0 / 50.0;
  const double conv = 0.18 * 12500;
  const double xrr = 1.0 * (1.0 / wcainv / conv) / 1000.0;
  const double dnai = -xrr * (P.xina + 3.0 * P.xinak + 3.0 * m.xinacato);
  m.xnai = xnai + dnai * dt;
  const double dvh = -(P.xina + P.xik1 + 1 * P.xikr + 1 * P.xiks + P.xitos + 1 * P.xitof +
                       1. * m.xinacato + 1 * m.xicatto + P.xinak) +
                     P.stim;
  m.v = protocol_voltage(c, t, dt, v + dvh * dt);
  m.out_ica += m.xicatto;
  m.out_ncx += m.xinacato;
  m.out_ina += P.xina;
  m.xina = P.xina;
  m.xiks = P.xiks;
  m.xikr = P.xikr;
  m.xik1 = P.xik1;
  m.xinak = P.xinak;
  m.xitos = P.xitos;
  m.xitof = P.xitof;
}

// Coefficients of the next lattice update (step_coef, cellmodel.cuh) by one
// warp; fm holds fmod(t - dt, OUTT), fmod(t + 1e-7, OUTT), fmod(t + 1e-7, 5),
// fmod(t + 1e-7, PCL) and fmod(t + 10 PCL, 15.5 PCL) for the state's time t
// (entries 1..5 of membrane_update_warp's fm); `s` is 96 doubles of shared
// memory owned by the warp.  Returns whether the cell is inside its protocol.
__device__ inline bool step_coef_warp(StepCoef<double>& k, const rh_membrane& m,
                                      const CellConst& c, double dt, const double* fm,
                                      double* s, QksStep* qs = nullptr) {
  const double fm1 = fm[0], fm2 = fm[1];
  const int lane = threadIdx.x & 31;
  WarpSlots w{s, s + 32, s + 64, lane};
  const double v = m.v, xnai = m.xnai, t = m.t;
  double dv5 = 5, dvk = 8, fv5 = -22.8, fvk = 9.1;
  k.alphac = 0.22;
  k.betac = 4;
  if (c.iso2) {
    k.betac = 2;
    dv5 = 0;
    fv5 = -28;
    fvk = 8.5;
  }
  // ---- round 1: quotients that do not need za ----
  w.open(qs ? 9 : 8);
  w.put(0, v * FARAD, XRGAS);                  // za, first division
  w.put(1, xnai, KMNAI);                       // r
  w.put(2, 1.0, dt);                           // rdt
  w.put(3, dt, 5.0);                           // dth
  w.put(4, 0.95, dt);                          // rdt95
  w.put(5, -(v - dv5), dvk);                   // dinf / taudin exponent
  w.put(6, -(v - fv5), fvk);                   // finf exponent 1
  w.put(7, (v - 60), 12.);                     // finf exponent 2
  if (qs) w.put(8, 0.28, qs->csubt);           // qks: 0.28/csubt
  w.divide();
  const double za1 = w.get(0), r = w.get(1);
  k.rdt = w.get(2);
  k.dth = w.get(3);
  k.rdt95 = w.get(4);
  const double x_d = w.get(5), x_f1 = w.get(6), x_f2 = w.get(7);
  // ---- round 2: za, rdth95 ----
  double q28 = 0.0;
  if (qs) q28 = w.get(8);
  w.open(qs ? 3 : 2);
  w.put(0, za1, TEMPER);
  w.put(1, 0.95, k.dth);
  if (qs) w.put(2, qs->qks_num, 1 + q28 * q28 * q28);  // pow(0.28/csubt, 3) as a product
  w.divide();
  const double za = w.get(0);
  k.rdth95 = w.get(1);
  double qks_inf = 0.0;
  if (qs) qks_inf = 0.2 * (1 + w.get(2));
  // ---- round 3: exponentials ----
  const double tq = 0.0337 * (v + 10.5);
  double X[7];
  {
    const double arg = lane == 0 ? x_d
                     : lane == 1 ? x_f1
                     : lane == 2 ? x_f2
                     : lane == 3 ? -tq * tq
                     : lane == 4 ? 2.0 * za
                     : lane == 5 ? ETA * za
                     : lane == 6 ? (ETA - 1.0) * za
                                 : 0.0;
    const double ex = exp(arg);
#pragma unroll
    for (int i = 0; i < 7; ++i) X[i] = __shfl_sync(0xffffffffu, ex, i);
  }
  const double e2z = X[4], e1 = X[5], e2 = X[6];
  const bool za_small = fabs(za) < 0.001;
  // ---- round 4 ----
  w.open(qs ? 6 : 5);
  w.put(0, 1.0, 1.0 + X[0]);                                   // dinf
  w.put(1, 1.0, 1.0 + X[1]);                                   // finf term
  w.put(2, 1.0 - X[0], 0.035 * (v - dv5));                     // taudin inner
  w.put(3, 4.0 * PCA * za * FARAD * GAMMAI, e2z - 1.0);        // lcc_k
  w.put(4, e2z, 1000.0);                                       // lcc_e2z_k
  if (qs) w.put(5, dt * (qks_inf - qs->qks), qs->tauqks);  // qks increment
  w.divide();
  if (qs) qs->dqks = w.get(5);
  const double dinf = w.get(0);
  const double f_a = w.get(1), td_in = w.get(2);
  k.lcc_k = za_small ? 2.0 * PCA * FARAD * GAMMAI : w.get(3);
  k.lcc_e2z_k = w.get(4);
  const bool v_tiny = (v < 0.0001) && (v > -0.0001);
  // ---- round 5 ----
  w.open(3);
  w.put(0, f_a, 1. + X[2]);                                    // finf
  w.put(1, 1.0, td_in * dinf);                                 // taudin
  w.put(2, 0.035 * dvk, dinf);                                 // taudin near v = 0
  w.divide();
  const double finf = 1. - w.get(0);
  const double taudin = v_tiny ? w.get(2) : w.get(1);
  const double taufin = (0.02 - 0.007 * X[3]);
  k.alphad = dinf * taudin;
  k.betad = (1 - dinf) * taudin;
  k.alphaf = finf * taufin;
  k.betaf = (1 - finf) * taufin;
  // NCX (subroutine_cuda.c:56-67)
  const double xn3 = xnai * xnai * xnai;
  k.ncx_num_a = e1 * xn3 * c.cao;
  k.ncx_num_b = e2 * (XNAO * XNAO * XNAO);
  k.ncx_t1 = KMCAI * (XNAO * XNAO * XNAO) * (1.0 + r * r * r);
  k.ncx_t3a = (KMCAO + c.cao) * xn3;
  k.ncx_den2 = 1.0 + KSAT * e2;
  k.svica = c.svica;
  k.svncx = c.svncx;
  option_coef(k, c, v, t, dt, fm[4]);
  k.cao = c.cao;
  k.ku = c.ku;
  k.ku2 = c.ku2;
  k.kb = c.kb;
  k.dt = dt;
  k.reset_window = fm1 < dt;
  k.output_step = fm2 < dt;
  k.perm = c.perm;
  k.cadist_step = k.output_step && fm[2] < dt && fm[3] < 500;
  return t < c.tend;
}

// The qks update of the mixed path in one division: with c3 = csubt^3 and
// K = 0.28^3, qks_inf = 0.2 (c3 + K + num c3) / (c3 + K), so
//   dqks = dt (0.2 (c3 + K + num c3) - qks (c3 + K)) / ((c3 + K) tauqks),
// the reference's three quotients (q28, qks_inf, the increment) folded into
// one (equal in exact arithmetic; the last bits differ).  `s` as in
// membrane_post_warp; all lanes return the increment.
__device__ inline double qks_increment_warp(double csubt, double qks, double num, double tauqks,
                                            double dt, double* s) {
  const int lane = threadIdx.x & 31;
  WarpSlots w{s, s + 32, s + 64, lane};
  constexpr double K = 0.28 * 0.28 * 0.28;
  const double c3 = csubt * csubt * csubt;
  const double d = c3 + K;
  w.open(1);
  w.put(0, dt * (0.2 * (d + num * c3) - qks * d), d * tauqks);
  w.divide();
  return w.get(0);
}

// Coefficients of the next lattice update for the FP32 lattice, computed in
// FP32 from the FP64 membrane state (step_coef, cellmodel.cuh, restated): the
// gating rates and the LCC/NCX factors are FP32 quantities of the mixed
// path, and FP32 arithmetic keeps them off the long FP64 latency chain of the
// cell update.  Where the FP64 form subtracts nearly equal values, the FP32
// form avoids it: 1 - exp(x) and exp(2 za) - 1 as -expm1(x) and expm1(2 za),
// 1 - dinf as exp(x) dinf, 1 - finf as the quotient it subtracts.  The flags
// come from the FP64 fmods in fm (as step_coef_warp takes them) and the time
// step constants from P.  Every lane returns the same coefficients.
__device__ inline bool step_coef_warp_f32(StepCoef<float>& k, const rh_membrane& m,
                                          const CellConst& c, double dt, const double* fm,
                                          const MembranePre& P) {
  const int lane = threadIdx.x & 31;
  const double vd = m.v;
  const float v = (float)vd, xnai = (float)m.xnai;
  float dv5 = 5.f, dvk = 8.f, fv5 = -22.8f, fvk = 9.1f;
  k.alphac = 0.22f;
  k.betac = 4.f;
  if (c.iso2) {
    k.betac = 2.f;
    dv5 = 0.f;
    fv5 = -28.f;
    fvk = 8.5f;
  }
  const float za = v * (float)(FARAD / XRGAS / TEMPER);
  const float tq = 0.0337f * (v + 10.5f);
  // one exponential per lane: lanes 0-6 the arguments of step_coef
  const float arg = lane == 0 ? -(v - dv5) / dvk
                  : lane == 1 ? -(v - fv5) / fvk
                  : lane == 2 ? (v - 60.f) / 12.f
                  : lane == 3 ? -tq * tq
                  : lane == 4 ? 2.f * za
                  : lane == 5 ? (float)ETA * za
                  : lane == 6 ? (float)(ETA - 1.0) * za
                              : 0.f;
  const float ex = expf(arg);
  const float em = (lane == 0 || lane == 4) ? expm1f(arg) : 0.f;
  const float ed = __shfl_sync(0xffffffffu, ex, 0), emd = __shfl_sync(0xffffffffu, em, 0);
  const float ef1 = __shfl_sync(0xffffffffu, ex, 1), ef2 = __shfl_sync(0xffffffffu, ex, 2);
  const float eq = __shfl_sync(0xffffffffu, ex, 3);
  const float e2z = __shfl_sync(0xffffffffu, ex, 4), em2z = __shfl_sync(0xffffffffu, em, 4);
  const float e1 = __shfl_sync(0xffffffffu, ex, 5), e2 = __shfl_sync(0xffffffffu, ex, 6);
  // LCC gates (reesica.h:21-63)
  const float dinf = 1.f / (1.f + ed);
  float taudin = 1.f / ((-emd) / (0.035f * (v - dv5)) * dinf);
  if ((vd < 0.0001) && (vd > -0.0001)) taudin = 0.035f * dvk / dinf;
  const float fq = 1.f / (1.f + ef1) / (1.f + ef2);  // 1 - finf
  const float finf = 1.f - fq;
  const float taufin = 0.02f - 0.007f * eq;
  k.alphad = dinf * taudin;
  k.betad = (ed * dinf) * taudin;
  k.alphaf = finf * taufin;
  k.betaf = fq * taufin;
  // ICaL (subroutine_cuda.c:231-247)
  k.lcc_k = fabsf(za) < 0.001f ? (float)(2.0 * PCA * FARAD * GAMMAI)
                               : (float)(4.0 * PCA * FARAD * GAMMAI) * za / em2z;
  k.lcc_e2z_k = e2z / 1000.f;
  // NCX (subroutine_cuda.c:56-67)
  const float xn3 = xnai * xnai * xnai;
  const float r = xnai / (float)KMNAI;
  k.ncx_num_a = e1 * xn3 * (float)c.cao;
  k.ncx_num_b = e2 * (float)(XNAO * XNAO * XNAO);
  k.ncx_t1 = (float)(KMCAI * (XNAO * XNAO * XNAO)) * (1.f + r * r * r);
  k.ncx_t3a = (float)(KMCAO + c.cao) * xn3;
  k.ncx_den2 = 1.f + (float)KSAT * e2;
  k.svica = (float)c.svica;
  k.svncx = (float)c.svncx;
  // build options (option_coef)
  const double t = m.t;
  k.sviup = (float)((c.iso && t >= 5.5 * c.pcl) ? c.sviup_iso : c.sviup_tot);
  k.iso_add_lcc = c.iso && fm[4] < dt;
  k.ncx_form = c.ncx_form;
  k.ncx_ka_hill = c.ncx_form == RH_NCX_OLD || (c.ncx_form == RH_NCX_NOALLO && vd < -75);
  k.ncx_t2b = (float)((KMNAI * KMNAI * KMNAI) * c.cao);
  k.slowncx = c.slowncx;
  k.bcg_a = (float)(BCG_G * vd);
  k.bcg_b = (float)(BCG_G / 2. / FRT);
  k.cao = (float)c.cao;
  k.ku = (float)c.ku;
  k.ku2 = (float)c.ku2;
  k.kb = (float)c.kb;
  k.dt = (float)dt;
  k.rdt = (float)P.rdt;
  k.dth = (float)P.dth;
  k.rdt95 = (float)P.rdt95;
  k.rdth95 = (float)P.rdth95;
  k.reset_window = fm[0] < dt;
  k.output_step = fm[1] < dt;
  k.perm = c.perm;
  k.cadist_step = k.output_step && fm[2] < dt && fm[3] < 500;
  return t < c.tend;
}

}  // namespace rh
