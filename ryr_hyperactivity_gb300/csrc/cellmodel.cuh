// cellmodel.cuh — whole-cell part of a time step, FP64: the membrane
// currents, gates, [Na]i and V (cuda_Cell_Detailed.cu:458-739, run on the
// host every step in the reference, here by the cell update on the GPU), the
// per-cell voltage coefficients of the next lattice update, and the 45
// wholecell output columns (:1031-1072).
#pragma once

#include <math.h>

#include "lattice.cuh"

namespace rh {

// Voltage a clamp protocol sets after the step that starts at time t
// (cuda_Cell_Detailed.cu:733-773); `v` is the voltage the membrane model
// computed, returned unchanged by the paced protocols.
__host__ __device__ inline double protocol_voltage(const CellConst& c, double t, double dt,
                                                   double v) {
  switch (c.protocol) {
    case RH_PROTO_VCLAMP:  // :733-739
      return t > 100 ? c.clamp_mv : -86;
    case RH_PROTO_BROWN_VCLAMP:  // :741-752
      if (t < 4000) return -86;
      if (t < 4200) return -10;
      if (t < 6200) return 10;
      if (t < 7200) return -30;
      return -86;
    case RH_PROTO_AP_CLAMP:  // :754-757, one PCL of samples repeated
      return c.apv[((int)(t / dt + 0.1)) % c.napv];
    case RH_PROTO_LINEAR_AP_CLAMP:  // :758-773
      if (t < 100) return -86;
      if (t < 101.865) return 68 * (t - 100) - 80;
      if (t < 119.1) return -(t - 100) + 48;
      if (t < 138.9) return 27 + 0.1 * (t - 100);
      if (t < 364.43) return 43 - (t - 100) / 3.2;
      if (t < 395.43) return -1.5 * (t - 100) + 357;
      return -86;
    default:
      return v;
  }
}

// Stimulus current of the step that starts at time t (:683-699): 80 uA/uF
// in the first ms of each period, none for unpaced and permeabilised cells.
// `phase` is fmod(t + PCL - 100, PCL), or fmod(t, PCL) for an iso cell,
// which is paced only while t < 11.9 PCL.
__host__ __device__ inline double stimulus(const CellConst& c, double t, double phase) {
  if (c.perm || c.protocol == RH_PROTO_NOPACING) return 0.0;
  if (c.iso) return (phase < 1.0 && t < c.pcl * 11.9) ? 80.0 : 0.0;
  return phase < 1.0 ? 80.0 : 0.0;
}

// Coefficients of the build options for the lattice update at time t with
// voltage v: iso's SERCA boost and LCC insertion (:1213-1229; iso_phase =
// fmod(t + 10 PCL, 15.5 PCL)), the NCX form, slowncxchange's background
// current (:1267-1269).
__host__ __device__ inline void option_coef(StepCoef<double>& k, const CellConst& c, double v,
                                            double t, double dt, double iso_phase) {
  k.sviup = (c.iso && t >= 5.5 * c.pcl) ? c.sviup_iso : c.sviup_tot;
  k.iso_add_lcc = c.iso && iso_phase < dt;
  k.ncx_form = c.ncx_form;
  k.ncx_ka_hill = c.ncx_form == RH_NCX_OLD || (c.ncx_form == RH_NCX_NOALLO && v < -75);
  k.ncx_t2b = (KMNAI * KMNAI * KMNAI) * c.cao;
  k.slowncx = c.slowncx;
  k.bcg_a = BCG_G * v;
  k.bcg_b = BCG_G / 2. / FRT;
}

// Membrane model step.  Expression order follows the reference so that the
// device result agrees with it to the last few ulps.
__host__ __device__ inline void membrane_update(rh_membrane& m, double dt, const CellConst& c) {
  const double tperid = c.pcl, svikr = c.svikr;
  const double t = m.t, v = m.v;
  const double xki = 140.0, xko = 5.40;  // :350-351
  const double csubt = m.csubt;
  const double xnai = m.xnai;
  // INa (:460-502)
  double ena = (1.0 / FRT) * log(XNAO / xnai);
  double am = 0.32 * (v + 47.13) / (1.0 - exp(-0.1 * (v + 47.13)));
  double bm = 0.08 * exp(-v / 11.0);
  double ah, bh, aj, bj;
  if (v < -40.0) {
    ah = 0.135 * exp((80.0 + v) / (-6.8));
    bh = 3.56 * exp(0.079 * v) + 310000.0 * exp(0.35 * v);
    aj = (-127140.0 * exp(0.2444 * v) - 0.00003474 * exp(-0.04391 * v)) *
         ((v + 37.78) / (1.0 + exp(0.311 * (v + 79.23))));
    bj = (0.1212 * exp(-0.01052 * v)) / (1.0 + exp(-0.1378 * (v + 40.14)));
  } else {
    ah = 0.00;
    bh = 1.00 / (0.130 * (1.00 + exp((v + 10.66) / (-11.10))));
    aj = 0.00;
    bj = (0.3 * exp(-0.00000025350 * v)) / (1.0 + exp(-0.10 * (v + 32.00)));
  }
  double tauh = 1.00 / (ah + bh);
  double tauj = 1.00 / (aj + bj);
  double taum = 1.00 / (am + bm);
  double gna = 15;
  double gnaleak = 0.3e-3 * 5;
  double xina = gna * m.xh * m.xj * m.xm * m.xm * m.xm * (v - ena) + gnaleak * (v - ena);
  m.xh = ah / (ah + bh) - ((ah / (ah + bh)) - m.xh) * exp(-dt / tauh);
  m.xj = aj / (aj + bj) - ((aj / (aj + bj)) - m.xj) * exp(-dt / tauj);
  m.xm = am / (am + bm) - ((am / (am + bm)) - m.xm) * exp(-dt / taum);
  // IKr (:507-529)
  double ek = (1.00 / FRT) * log(xko / xki);
  double gss = sqrt(xko / 5.40);
  double xkrv1 = 0.001380 * (v + 7.00) / (1.0 - exp(-0.123 * (v + 7.00)));
  double xkrv2 = 0.000610 * (v + 10.00) / (exp(0.1450 * (v + 10.00)) - 1.00);
  double taukr = 1.00 / (xkrv1 + xkrv2);
  double xkrinf = 1.00 / (1.00 + exp(-(v + 50.00) / 7.50));
  double rg = 1.00 / (1.00 + exp((v + 33.00) / 22.40));
  double gkr = 0.0078360;
  double xikr = svikr * gkr * gss * m.xr * rg * (v - ek);
  m.xr = xkrinf - (xkrinf - m.xr) * exp(-dt / taukr);
  // IKs (:534-559)
  double prnak = 0.0183300;
  // pow((0.28 / csubt), 3) and, below, pow(12 / xnai, 1) of the reference are
  // evaluated as the product and the quotient itself
  const double q28 = 0.28 / csubt;
  double qks_inf = 0.2 * (1 + (c.slowncx ? 1.6 : 0.8) / (1 + q28 * q28 * q28));
  double tauqks = c.slowncx ? 2000 : 1000.00;  // :540-543
  double eks = (1.00 / FRT) * log((xko + prnak * XNAO) / (xki + prnak * xnai));
  double xs1ss = 1.0 / (1.0 + exp(-(v - 1.500) / 16.700));
  double tauxs = 1.00 / (0.0000719 * (v + 30.00) / (1.00 - exp(-0.1480 * (v + 30.0))) +
                         0.0001310 * (v + 30.00) / (exp(0.06870 * (v + 30.00)) - 1.00));
  tauxs = 0.95 * tauxs;
  double gksx = 0.2000;
  double xiks = 1.0 * 1. * gksx * m.qks * m.xs1 * m.xs2 * (v - eks);
  m.xs1 = xs1ss - (xs1ss - m.xs1) * exp(-dt / tauxs);
  m.xs2 = xs1ss - (xs1ss - m.xs2) * exp(-dt / tauxs);
  m.qks = m.qks + dt * (qks_inf - m.qks) / tauqks;
  // IK1 (:590-600)
  double gki = 0.600 * (sqrt(xko / 5.4));
  double aki = 1.02 / (1.0 + exp(0.2385 * (v - ek - 59.215)));
  double bki = (0.49124 * exp(0.08032 * (v - ek + 5.476)) + exp(0.061750 * (v - ek - 594.31))) /
               (1.0 + exp(-0.5143 * (v - ek + 4.753)));
  double xkin = aki / (aki + bki);
  double xik1 = (1.0) * gki * xkin * (v - ek);
  // Ito,s (:604-629)
  double rt1 = -(v + 3.0) / 15.00;
  double rt2 = (v + 33.5) / 10.00;
  double rt3 = (v + 60.00) / 10.00;
  double xtos_inf = 1.00 / (1.0 + exp(rt1));
  double ytos_inf = 1.00 / (1.00 + exp(rt2));
  double rs_inf = 1.00 / (1.00 + exp(rt2));
  double txs = 9.00 / (1.00 + exp(-rt1)) + 0.50;
  double tys = 3000.00 / (1.0 + exp(rt3)) + 30.00;
  double xitos = 1.0 * 0.040 * m.xtos * (m.ytos + 0.50 * rs_inf) * (v - ek);
  m.xtos = xtos_inf - (xtos_inf - m.xtos) * exp(-dt / txs);
  m.ytos = ytos_inf - (ytos_inf - m.ytos) * exp(-dt / tys);
  // Ito,f (:633-659)
  double rt4 = -(v / 30.00) * (v / 30.00);
  double rt5 = (v + 33.50) / 10.00;
  double txf = 3.50 * exp(rt4) + 1.50;
  double tyf = 20.0 / (1.0 + exp(rt5)) + 20.00;
  double xitof = 1.0 * 0.10 * m.xtof * m.ytof * (v - ek);
  m.xtof = xtos_inf - (xtos_inf - m.xtof) * exp(-dt / txf);
  m.ytof = ytos_inf - (ytos_inf - m.ytof) * exp(-dt / tyf);
  // INaK (:665-676)
  double sigma = (exp(XNAO / 67.30) - 1.00) / 7.00;
  double fnak = 1.00 / (1.0 + 0.1245 * exp(-0.1 * v * FRT) + 0.0365 * sigma * exp(-v * FRT));
  double xinak = 1. * 1.5000 * fnak * (1.0 / (1.0 + (12.00 / xnai))) * xko / (xko + 1.50);
  // stimulus (:689-692)
  double stim = stimulus(c, t, c.iso ? fmod(t, tperid) : fmod(t + tperid - 100, tperid));
  // [Na]i and V (:701-738)
  double wcainv = 1.0 / 50.0;
  double conv = 0.18 * 12500;
  double xrr = 1.0 * (1.0 / wcainv / conv) / 1000.0;
  double dnai = -xrr * (xina + 3.0 * xinak + 3.0 * m.xinacato);
  m.xnai = xnai + dnai * dt;
  double dvh = -(xina + xik1 + 1 * xikr + 1 * xiks + xitos + 1 * xitof + 1. * m.xinacato +
                 1 * m.xicatto + xinak) +
               stim;
  m.v = protocol_voltage(c, t, dt, v + dvh * dt);
  m.out_ica += m.xicatto;  // :774-776
  m.out_ncx += m.xinacato;
  m.out_ina += xina;
  m.xina = xina;
  m.xiks = xiks;
  m.xikr = xikr;
  m.xik1 = xik1;
  m.xinak = xinak;
  m.xitos = xitos;
  m.xitof = xitof;
}

// Coefficients of the next lattice update for the membrane state m.
// Returns whether the cell is still inside its protocol (t < tend, :399).
__host__ __device__ inline bool step_coef(StepCoef<double>& k, const rh_membrane& m,
                                          const CellConst& c, double dt) {
  const double v = m.v, xnai = m.xnai, t = m.t;
  // LCC gates (reesica.h:21-63)
  double dv5 = 5, dvk = 8, fv5 = -22.8, fvk = 9.1;
  k.alphac = 0.22;
  k.betac = 4;
  if (c.iso2) {
    k.betac = 2;
    dv5 = 0;
    fv5 = -28;
    fvk = 8.5;
  }
  double dinf = 1.0 / (1.0 + exp(-(v - dv5) / dvk));
  double taudin = 1.0 / ((1.0 - exp(-(v - dv5) / dvk)) / (0.035 * (v - dv5)) * dinf);
  if ((v < 0.0001) && (v > -0.0001)) taudin = 0.035 * dvk / dinf;
  double finf = 1. - 1.0 / (1.0 + exp(-(v - fv5) / fvk)) / (1. + exp((v - 60) / 12.));
  double taufin = (0.02 - 0.007 * exp(-(0.0337 * (v + 10.5)) * (0.0337 * (v + 10.5))));
  k.alphad = dinf * taudin;
  k.betad = (1 - dinf) * taudin;
  k.alphaf = finf * taufin;
  k.betaf = (1 - finf) * taufin;
  // ICaL (subroutine_cuda.c:231-247)
  double za = v * FARAD / XRGAS / TEMPER;
  double e2z = exp(2.0 * za);
  if (fabs(za) < 0.001)
    k.lcc_k = 2.0 * PCA * FARAD * GAMMAI;
  else
    k.lcc_k = 4.0 * PCA * za * FARAD * GAMMAI / (e2z - 1.0);
  k.lcc_e2z_k = e2z / 1000.0;
  // NCX (subroutine_cuda.c:56-67)
  double e1 = exp(ETA * za), e2 = exp((ETA - 1.0) * za);
  double xn3 = xnai * xnai * xnai;
  double r = xnai / KMNAI;
  k.ncx_num_a = e1 * xn3 * c.cao;
  k.ncx_num_b = e2 * (XNAO * XNAO * XNAO);
  k.ncx_t1 = KMCAI * (XNAO * XNAO * XNAO) * (1.0 + r * r * r);
  k.ncx_t3a = (KMCAO + c.cao) * xn3;
  k.ncx_den2 = 1.0 + KSAT * e2;
  k.svica = c.svica;
  k.svncx = c.svncx;
  option_coef(k, c, v, t, dt, fmod(t + 10 * c.pcl, 15.5 * c.pcl));
  k.cao = c.cao;
  k.ku = c.ku;
  k.ku2 = c.ku2;
  k.kb = c.kb;
  k.dt = dt;
  k.rdt = 1.0 / dt;
  k.dth = dt / 5.0;
  k.rdt95 = 0.95 / dt;
  k.rdth95 = 0.95 / (dt / 5.0);
  k.reset_window = fmod(t - dt, OUTT) < dt;
  k.output_step = fmod(t + 0.0000001, OUTT) < dt;
  k.perm = c.perm;
  k.cadist_step = k.output_step && fmod(t + 0.0000001, 5.0) < dt &&
                  fmod(t + 0.0000001, c.pcl) < 500.0;  // :1002
  return t < c.tend;
}

// Output-step reductions -> the 45 wholecell columns (:931-1072).
__host__ __device__ inline void wholecell_columns(double* w, const double* o, const rh_membrane& m,
                                                  int nin, double dt) {
  const double N = nin;
  double cit = o[O_CI - P_STEP_END] / 8. / N;
  double cproxit = o[O_CP - P_STEP_END] / N;
  double cjsrt = o[O_CJSR - P_STEP_END] / N;
  double csqnbt = o[O_CJSRB - P_STEP_END] / N;
  double cnsrt = o[O_CNSR - P_STEP_END] / 8. / N;
  double poto = o[O_PO - P_STEP_END] / N;
  double pbcto = o[O_NCB - P_STEP_END] / N / 100.;
  double catft = o[O_CATF - P_STEP_END] / 8. / N;
  double catst = o[O_CATS - P_STEP_END] / 8. / N;
  double casrt = o[O_CASR - P_STEP_END] / 8. / N;
  double camyot = o[O_CAMYO - P_STEP_END] / 8. / N;
  double cacalt = o[O_CACAL - P_STEP_END] / 8. / N;
  double leakt = o[O_LEAK - P_STEP_END] / 8. / N;
  double upt = o[O_UP - P_STEP_END] / 8. / N;
  double ire = o[O_XIRE - P_STEP_END] / N;
  double ncxfwd = o[O_NCXFWD - P_STEP_END] / N;
  double outancx = o[O_ANCX - P_STEP_END] / N;
  double casart = o[O_CASAR - P_STEP_END] / N;
  double casarht = o[O_CASARH - P_STEP_END] / N;
  double casarjt = o[O_CASARJ - P_STEP_END] / N;
  double casarhjt = o[O_CASARHJ - P_STEP_END] / N;
  const double csubt = m.csubt;
  double total_ca = (cit + catft + catst + casrt + camyot + cacalt) * VI * 8. +
                    (csubt + casart + casarht) * VS + (cproxit + casarjt + casarhjt) * VP +
                    (cnsrt)*VNSR * 8. + (cjsrt + csqnbt) * VJSR;
  double total_ci = (cit + catft + catst + casrt + camyot + cacalt) * VI * 8. +
                    (csubt + casart + casarht) * VS + (cproxit + casarjt + casarhjt) * VP;
  w[0] = m.t;
  w[1] = cit;
  w[2] = m.v;
  w[3] = m.out_ncx / (OUTT / dt);
  w[4] = m.out_ica / (OUTT / dt);
  w[5] = cproxit;
  w[6] = csubt;
  w[7] = cjsrt;
  w[8] = cnsrt;
  w[9] = poto;
  w[10] = m.xnai;
  w[11] = m.xiks;
  w[12] = m.xikr;
  w[13] = m.xik1;
  w[14] = m.xinak;
  w[15] = m.xitos;
  w[16] = m.xitof;
  w[17] = m.out_ina / (OUTT / dt);
  w[18] = m.xr;
  w[19] = ncxfwd * (VS / VP);
  w[20] = pbcto;
  w[21] = cacalt;
  w[22] = catft;
  w[23] = leakt;
  w[24] = upt;
  w[25] = ire;
  w[26] = o[O_NOU - P_STEP_END];
  w[27] = o[O_NOB - P_STEP_END];
  w[28] = o[O_NCU - P_STEP_END];
  w[29] = o[O_NCB - P_STEP_END];
  for (int q = 0; q < 7; ++q) w[30 + q] = o[O_TN1 - P_STEP_END + q];
  w[37] = outancx;
  w[38] = m.xs1;
  w[39] = m.qks;
  w[40] = (double)m.sparksum;
  w[41] = catst;
  w[42] = csqnbt;
  w[43] = total_ci;
  w[44] = total_ca;
}

}  // namespace rh
