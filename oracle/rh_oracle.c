/*
 * rh_oracle.c — CPU oracle (FP64) for the per-time-step myocyte update.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker.  Never linked by the product.
 *
 * Each function restates one part of the reference and cites the lines it
 * follows (paths relative to the reference project).  Arithmetic keeps the
 * reference's expression order so that, compiled with -ffp-contract=off, the
 * oracle reproduces the reference's own routines bit for bit on the same
 * uniforms (checked against the reference compiled for the host, oracle/_ref).
 */
#include "rh_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/rh_philox.h"

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------------
 * Constants: cuda_Cell_Detailed.cu:63-145, subroutine_cuda.c:7-39,
 * buffers.c:16-52.  Multi-token definitions keep the reference's grouping so
 * that constant folding yields the same doubles.
 * ------------------------------------------------------------------------- */
#define OUTT 2.5                 /* :63 */
#define PI_TRUNC 3.1415926       /* :65, truncated pi used by Box-Muller */
#define VP 0.00126               /* :66 */
#define VJSR (0.02 * 1)          /* :67 */
#define VI (0.5 / 8.)            /* :68 */
#define VNSR (0.025 / 8.)        /* :69 */
#define NRYR 100                 /* :70 */
#define TAUPS 0.0283             /* :71 */
#define TAUPI 0.1                /* :72 */
#define TAUSI 0.04               /* :73 */
#define TAUTR (25.0 * 1.0 / 4.)  /* :74 */
#define TAUNL 6.                 /* :75 */
#define TAUNT 1.8                /* :76 */
#define TAUIL (0.7 * 2.)         /* :77 */
#define TAUIT (0.33 * 2.)        /* :78 */
#define TAUST 1.42               /* :79 */
#define FRT (96.485 / 8.314 / 308.0) /* :83 */
#define XI 0.7                   /* :84 */
#define CI_BASAL 0.0944          /* :91 */
#define PERM_CI_BASAL 0.3        /* :88, the perm build */
#define PERM_CJSR_BASAL 900      /* :89, the perm build */
#define VS 0.025                 /* :95 */
#define ICAGAMMA 0.5             /* :99 */
#define CM 45                    /* :100 */
#define SVNCP 4                  /* :102 */
#define TAUCB 1.                 /* :104 */
#define TAUCU 1.                 /* :105 */
#define SV_IUP (1.0 + 0.75)      /* :107 */
#define SVJMAX 11.5              /* :111 */
#define TAUU (0.2 * 5 * 220.)    /* :113 */
#define TAUB 1.0                 /* :114 */
#define SVILEAK 1.0              /* :116 */
#define SVTAUXS 0.95             /* :117 */
#define XNAO 140.0               /* :145 */

/* NCX, CSQN, LCC (subroutine_cuda.c:7-39) */
#define VNACA (21.0 / 1.0)
#define KMCAI 0.00359
#define KMCAO 1.3
#define KMNAI 12.3
#define KMNAO 87.5
#define KDA 0.0003
#define KSAT 0.27
#define ETA 0.35
#define FARAD 96.485
#define XRGAS 8.314
#define TEMPER 308
#define NM 20
#define ND 30
#define RATEDIMER 5000.0
#define KDIMER 850.0
#define HILLDIMER 23.0
#define CSQBERS 460.0
#define KBERS 600.0
#define PCA 11.9
#define GAMMAI 0.341

/* Buffers (buffers.c:16-52) */
#define KTSON 0.00254
#define KTSOFF 0.000033
#define BTS 134.
#define KTFON 0.0327
#define KTFOFF 0.0196
#define BTF 70.
#define KCALON 0.0543
#define KCALOFF 0.238
#define BCAL 24.
#define KDYEON 0.256
#define KDYEOFF 0.1
#define BDYE 50.
#define KSRON 0.1
#define KSROFF 0.06
#define BSR 19.
#define KSARON 0.1
#define KSAROFF 1.3
#define BSAR (42 * (VI * 8.0 / VS))
#define KSARHON 0.1
#define KSARHOFF 0.03
#define BSARH (15. * (VI * 8.0 / VS))
#define BMYO 140
#define KONMYOMG 0.0157
#define KOFFMYOMG 0.057
#define KONMYOCA 13.8
#define KOFFMYOCA 0.46
#define MGI 500

#define SQ(x) ((x) * (x))
#define CUBE(x) ((x) * (x) * (x))

static int g_threads = 0;

void orc_set_threads(int nthreads) { g_threads = nthreads; }

int orc_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---------------------------------------------------------------------------
 * Simulator state: the reference's arrays (cuda_Cell_Detailed.cu:164-212,
 * :259-320) as separate arrays over the full lattice including ghosts.
 * ------------------------------------------------------------------------- */
struct orc_sim {
  rh_cell_params p;
  int nx, ny, nz, ntot, nin;
  double dt;
  /* run constants derived from the parameters */
  double svica, svncx, sviup_tot, svikr, cao, tend;
  double sviup_iso; /* SERCA prefactor once iso is active (t >= 5.5 PCL) */
  double sviup_now; /* the prefactor of the lattice update in progress */
  int jz_line;
  /* per CRU */
  double *cp, *cjsr, *cjsrb, *ancx, *xire, *po, *xinaca, *xicat;
  double *casar, *casarh, *casarj, *casarhj;
  int *lcc; /* [ntot*8], slot ll of CRU ac at ac*8+ll */
  int *nl, *nou, *ncu, *nob, *ncb, *nspark;
  /* per sub-voxel, index ac*8+ii */
  double *xiup, *xileak, *catf, *cats, *cacal, *casr, *camyo, *mgmyo, *cadye;
  /* ping-pong pairs */
  double *ci[2], *cnsr[2], *cs[2];
  int cur;
  uint32_t status;
  rh_membrane m;
  double wc[RH_WHOLECELL_COLS];
  double* ls; /* (nx-2) x 22 */
  double* cd; /* cadist record: t, v, then 6 values per interior CRU */
  int cd_valid;
  double* apv; /* AP-clamp waveform (orc_set_ap_clamp), napv samples */
  int napv;
};

static inline int opos(const orc_sim* s, int i, int j, int k) {
  return s->nx * s->ny * k + s->nx * j + i; /* cuda_Cell_Detailed.cu:160-162 */
}

/* ------------------------------- buffers.c ------------------------------- */

/* Mass-action buffer rate with the saturation guard shared by tropf, trops,
 * bucal, budye, busr, busar, busarh, busarj, busarhj (buffers.c:72-155; the
 * `ba`=1 factors of busarj/busarhj are exact no-ops). */
static inline double buffer_rate(double kon, double koff, double total, double bound,
                                 double c, double dt) {
  if (kon * c * dt > 1) return 0.95 / dt * (total - bound) - koff * bound;
  return kon * c * (total - bound) - koff * bound;
}

/* Myosin Ca site, competing with Mg (buffers.c:55-62). */
static inline double myo_ca_rate(double camyo, double mgmyo, double c, double dt) {
  if (KONMYOCA * c * dt > 1) return 0.95 / dt * (BMYO - camyo - mgmyo) - KOFFMYOCA * camyo;
  return KONMYOCA * c * (BMYO - camyo - mgmyo) - KOFFMYOCA * camyo;
}

/* Myosin Mg site (buffers.c:63-70). */
static inline double myo_mg_rate(double camyo, double mgmyo, double dt) {
  if (KONMYOMG * MGI * dt > 1) return 0.95 / dt * (BMYO - camyo - mgmyo) - KOFFMYOMG * mgmyo;
  return KONMYOMG * MGI * (BMYO - camyo - mgmyo) - KOFFMYOMG * mgmyo;
}

/* --------------------------- subroutine_cuda.c --------------------------- */

/* Allosteric NCX with its activation state (subroutine_cuda.c:47-75); the
 * slowncxchange build scales Ka by 5 (:59-62). */
static double ncx_flux(double cs, double v, double xnai, double* ancx, double dt, double cext,
                       int slowncx) {
  double za = v * FARAD / XRGAS / TEMPER;
  double ka = *ancx;
  if (slowncx) ka = *ancx * 5;
  double t1 = KMCAI * CUBE(XNAO) * (1.0 + CUBE(xnai / KMNAI));
  double t2 = CUBE(KMNAO) * cs * (1.0 + cs / KMCAI);
  double t3 = (KMCAO + cext) * CUBE(xnai) + cs * CUBE(XNAO);
  double inaca = ka * VNACA *
                 (exp(ETA * za) * CUBE(xnai) * cext - exp((ETA - 1.0) * za) * CUBE(XNAO) * cs) /
                 ((t1 + t2 + t3) * (1.0 + KSAT * exp((ETA - 1.0) * za)));
  double ancxdot = (1.0 / (1.0 + CUBE(0.0003 / cs)) - *ancx) / 150.;
  *ancx += ancxdot * dt;
  return inaca;
}

/* NCX with the Ca-dependent Ka and the Mahajan t2, and the allosteric state
 * from on/off rates (oldncx, subroutine_cuda.c:77-100). */
static double ncx_old_flux(double cs, double v, double xnai, double* ancx, double dt,
                           double cext) {
  const double kncxoff = 0.00005;
  const double kncxon = 2.53e-3 * 0.05;
  double za = v * FARAD / XRGAS / TEMPER;
  double ka = 1.0 / (1.0 + CUBE(KDA / cs));
  double t1 = KMCAI * CUBE(XNAO) * (1.0 + CUBE(xnai / KMNAI));
  double t2 = CUBE(KMNAO) * cs + CUBE(KMNAI) * cext * (1.0 + cs / KMCAI);
  double t3 = (KMCAO + cext) * CUBE(xnai) + cs * CUBE(XNAO);
  double inaca = ka * VNACA *
                 (exp(ETA * za) * CUBE(xnai) * cext - exp((ETA - 1.0) * za) * CUBE(XNAO) * cs) /
                 ((t1 + t2 + t3) * (1.0 + KSAT * exp((ETA - 1.0) * za)));
  double ancxdot = (kncxon * SQ(cs * 1000) * (1 - *ancx) - *ancx * kncxoff);
  if (kncxon * SQ(cs * 1000) * dt > 0.95) ancxdot = 0.95 / dt * (1 - *ancx) - *ancx * kncxoff;
  *ancx += ancxdot * dt;
  return inaca;
}

/* NCX without an allosteric state (ncx_noallo, subroutine_cuda.c:102-120). */
static double ncx_noallo_flux(double cs, double v, double xnai, double cext) {
  double za = v * FARAD / XRGAS / TEMPER;
  double ka = 1.;
  if (v < -75) ka = 1.0 / (1.0 + CUBE(KDA / cs));
  double t1 = KMCAI * CUBE(XNAO) * (1.0 + CUBE(xnai / KMNAI));
  double t2 = CUBE(KMNAO) * cs + CUBE(KMNAI) * cext * (1.0 + cs / KMCAI);
  double t3 = (KMCAO + cext) * CUBE(xnai) + cs * CUBE(XNAO);
  return ka * VNACA *
         (exp(ETA * za) * CUBE(xnai) * cext - exp((ETA - 1.0) * za) * CUBE(XNAO) * cs) /
         ((t1 + t2 + t3) * (1.0 + KSAT * exp((ETA - 1.0) * za)));
}

/* SERCA uptake (subroutine_cuda.c:128-137). */
static inline double serca(double ci, double cnsr) {
  const double vup = 0.3, ki = 0.123, knsr = 1700.0, hh = 1.787, upfactor = 1.0;
  double a = pow(ci / ki, hh), b = pow(cnsr / knsr, hh);
  return upfactor * vup * (a - b) / (1.0 + a + b);
}

/* NSR leak (subroutine_cuda.c:139-146). */
static inline double sr_leak(double cnsr, double ci) {
  const double gleak = 0.00001035, kjsr = 500.0;
  return gleak * (cnsr - ci) * SQ(cnsr) / (SQ(cnsr) + SQ(kjsr));
}

/* CSQN monomer/dimer luminal buffering factor (subroutine_cuda.c:161-177). */
static double csqn_beta(double cjsr) {
  double roo2 = RATEDIMER / (1.0 + pow(KDIMER / cjsr, HILLDIMER));
  double mono = (-1.0 + sqrt(1.0 + 8.0 * CSQBERS * roo2)) / (4.0 * roo2 * CSQBERS);
  double ene = mono * NM + (1.0 - mono) * ND;
  double enedot = (NM - ND) * (-mono + 1.0 / (4.0 * CSQBERS * mono * roo2 + 1.0)) *
                  (HILLDIMER / cjsr) * (1.0 - roo2 / RATEDIMER);
  return 1.0 / (1.0 + (CSQBERS * KBERS * ene + CSQBERS * enedot * cjsr * (cjsr + KBERS)) /
                          SQ((KBERS + cjsr)));
}

/* Steady-state CSQN-bound Ca (subroutine_cuda.c:179-195). */
static double csqn_bound_ss(double cjsr) {
  double roo2 = RATEDIMER / (1.0 + pow(KDIMER / cjsr, HILLDIMER));
  double mono = (-1.0 + sqrt(1.0 + 8.0 * CSQBERS * roo2)) / (4.0 * roo2 * CSQBERS);
  double ene = mono * NM + (1.0 - mono) * ND;
  return CSQBERS * ene * cjsr / (KBERS + cjsr);
}

/* RyR release flux (subroutine_cuda.c:222-228). */
static inline double jsr_release(double po, double cjsr, double cp) {
  double jmax = (0.0147 * SVJMAX);
  return 1.0 * jmax * po * (cjsr - cp) / VP;
}

/* GHK single-LCC flux, clamped at 0 (subroutine_cuda.c:231-247). */
static double lcc_flux(double v, double cp, double cext) {
  double za = v * FARAD / XRGAS / TEMPER;
  double ica;
  if (fabs(za) < 0.001)
    ica = 2.0 * PCA * FARAD * GAMMAI * (cp / 1000.0 * exp(2.0 * za) - cext);
  else
    ica = 4.0 * PCA * za * FARAD * GAMMAI * (cp / 1000.0 * exp(2.0 * za) - cext) /
          (exp(2.0 * za) - 1.0);
  if (ica > 0.0) ica = 0.0;
  return ica;
}

/* 1 - u for the Box-Muller radius.  Uniforms lie in (0,1], so 1-u can be 0
 * (log -> -inf in subroutine_cuda.c:356); the smallest uniform step 2^-53 is
 * used instead.  Only u == 1 exactly is affected. */
static inline double one_minus_uniform(double u) {
  double r = 1.0 - u;
  return r > 0.0 ? r : 0x1.0p-53;
}

/* Double -> int of the Gaussian draw, spelled out because C leaves NaN and
 * out-of-range conversions undefined (x86 and aarch64 hosts disagree).  The
 * value follows the reference's own platform: on the GB300 the conversion of
 * NaN gives a negative integer (INT_MIN), so the draw is repeated until the
 * 200-try cap of subroutine_cuda.c:358-361 forces 0.  NaN arises when a
 * transition probability per step exceeds 1 (pbu, subroutine_cuda.c:443, is
 * not capped), making n*p*(1-p) negative.  Out-of-range values saturate. */
static inline int cuda_cvt_int(double x, uint32_t* status) {
  if (x != x) {
    *status |= RH_STATUS_RATE_CAP;
    return (-2147483647 - 1);
  }
  if (x >= 2147483647.0) return 2147483647;
  if (x <= -2147483648.0) return (-2147483647 - 1);
  return (int)x;
}

/* One RyR transition count (the pattern of subroutine_cuda.c:332-363, repeated
 * for all eight transitions): Poisson by Knuth's product of uniforms, capped
 * at 195 draws, when n<=1, p<0.2 or (n<=5 and p<0.3); otherwise a Gaussian
 * by Box-Muller, floored and dithered by one random bit, redrawn while
 * negative and forced to 0 after 200 tries (the reference's error return). */
static int ryr_transition(rh_stream* rng, int n, double p, double lam, uint32_t* status) {
  int kk;
  if (n <= 1 || p < 0.2 || (n <= 5 && p < 0.3)) {
    double puu = 1.0;
    kk = 0;
    while (puu >= lam && kk < 195) {
      kk++;
      double re = rh_uniform_double(rng);
      puu = puu * re;
    }
    return kk - 1;
  }
  int m = -1;
  kk = 0;
  while (m < 0) {
    double u1 = rh_uniform_double(rng);
    double u2 = rh_uniform_double(rng);
    unsigned int bit = rh_uniform_u32(rng);
    m = cuda_cvt_int(floor(n * p + sqrt(n * p * (1.0 - p)) * sqrt(-2.0 * log(one_minus_uniform(u1))) *
                                     cos(2.0 * PI_TRUNC * u2)) +
                         bit % 2,
                     status);
    kk++;
    if (kk > 200) {
      m = 0;
      *status |= RH_STATUS_GAUSS_RETRY;
    }
  }
  return m;
}

/* Four-state RyR cluster update (subroutine_cuda.c:251-669). */
static void ryr_gating(rh_stream* rng, double Ku, double Ku2, double Kb, double cp, double cjsr,
                       int* ncu, int* nou, int* ncb, int* nob, double dt, uint32_t* status) {
  double ryrpref = 4.5 * 1.5;
  double cygatek = Ku;
  double ryrhill = 2;
  double pku = ryrpref * Ku2 * 1 / (1 + SQ(5000 / cjsr)) * 1 / (1 + pow(cygatek / cp, ryrhill));
  double pkb =
      ryrpref / 36. * Kb * 1 / (1 + SQ(5000 / cjsr)) * 1 / (1 + pow(cygatek / cp, ryrhill));
  double pkuminus = 1. / TAUCU;
  double pkbminus = 1. / TAUCB;
  if (pku * dt > 1.0) pku = 1.0 / dt;
  if (pkb * dt > 1.0) pkb = 1.0 / dt;
  if (pkuminus * dt > 1.0) pkuminus = 1.0 / dt;
  if (pkbminus * dt > 1.0) pkbminus = 1.0 / dt;

  double roo2 = RATEDIMER / (1.0 + pow(KDIMER / (cjsr), HILLDIMER));
  double aub = (-1.0 + sqrt(1.0 + 8.0 * CSQBERS * roo2)) / (4.0 * roo2 * CSQBERS) / TAUB;
  double abu = 1.0 / TAUU;

  /* OU -> CU (:332-364) */
  double pkuh = pkuminus * dt;
  int n_ou_cu = ryr_transition(rng, *nou, pkuh, exp(-(*nou) * pkuh), status);
  if (n_ou_cu > NRYR) n_ou_cu = NRYR;
  /* CU -> OU (:366-397) */
  double pkum = pku * dt;
  int n_cu_ou = ryr_transition(rng, *ncu, pkum, exp(-(*ncu) * pkum), status);
  if (n_cu_ou > NRYR) n_cu_ou = NRYR;
  /* OU -> OB (:401-436) */
  double pau = (pkb < 1e-16) ? 0 : aub * dt;
  int n_ou_ob = ryr_transition(rng, *nou, pau, exp(-(*nou) * pau), status);
  if (n_ou_ob > NRYR) n_ou_ob = NRYR;
  /* OB -> OU (:439-476) */
  double pbu = (pkb < 1e-16) ? abu * dt * 36 : abu * dt * (pku / pkb);
  int n_ob_ou = ryr_transition(rng, *nob, pbu, exp(-(*nob) * pbu), status);
  if (n_ob_ou > NRYR) n_ob_ou = NRYR;
  /* CB -> CU (:480-511) */
  double pcb = abu * dt;
  int n_cb_cu = ryr_transition(rng, *ncb, pcb, exp(-(*ncb) * pcb), status);
  if (n_cb_cu > NRYR) n_cb_cu = NRYR;
  /* CU -> CB (:513-544) */
  double pcub = aub * dt;
  int n_cu_cb = ryr_transition(rng, *ncu, pcub, exp(-*ncu * pcub), status);
  if (n_cu_cb > NRYR) n_cu_cb = NRYR;
  /* OB -> CB (:548-579), no cap in the reference */
  double pkbh = pkbminus * dt;
  int n_ob_cb = ryr_transition(rng, *nob, pkbh, exp(-(*nob) * pkbh), status);
  /* CB -> OB (:581-613) */
  double pkbm = pkb * dt;
  int n_cb_ob = ryr_transition(rng, *ncb, pkbm, exp(-(*ncb) * pkbm), status);
  if (n_cb_ob > NRYR) n_cb_ob = NRYR;

  /* conflict resolution (:617-639) */
  if (n_ou_ob + n_ou_cu > *nou) {
    if (n_ou_cu >= n_ou_ob) n_ou_cu = 0;
    else n_ou_ob = 0;
    if (n_ou_ob > *nou) n_ou_ob = 0;
    else if (n_ou_cu > *nou) n_ou_cu = 0;
  }
  if (n_ob_ou + n_ob_cb > *nob) {
    if (n_ob_ou >= n_ob_cb) n_ob_ou = 0;
    else n_ob_cb = 0;
    if (n_ob_cb > *nob) n_ob_cb = 0;
    else if (n_ob_ou > *nob) n_ob_ou = 0;
  }
  if (n_cu_ou + n_cu_cb > *ncu) {
    if (n_cu_cb >= n_cu_ou) n_cu_cb = 0;
    else n_cu_ou = 0;
    if (n_cu_ou > *ncu) n_cu_ou = 0;
    else if (n_cu_cb > *ncu) n_cu_cb = 0;
  }
  /* updates and clamps (:642-665) */
  *nou += -n_ou_ob - n_ou_cu + n_ob_ou + n_cu_ou;
  if (*nou < 0) *nou = 0;
  if (*nou > NRYR) *nou = NRYR;
  *nob += -n_ob_ou - n_ob_cb + n_ou_ob + n_cb_ob;
  if (*nob < 0) *nob = 0;
  if (*nob > NRYR) *nob = NRYR;
  *ncu += -n_cu_ou - n_cu_cb + n_ou_cu + n_cb_cu;
  if (*ncu < 0) *ncu = 0;
  if (*ncu > NRYR) *ncu = NRYR;
  *ncb = NRYR - *nou - *nob - *ncu;
  if (*ncb < 0) *ncb = 0;
  if (*ncb > NRYR) *ncb = NRYR;
}

/* -------------------------------- reesica.h ------------------------------ */

/* Per-CRU LCC gate rates.  reesica.h:14-63 computes them inside every
 * lcc_markov call; they depend only on v and cpx, which all slots of a CRU
 * share, so they are evaluated once per CRU (same values). */
typedef struct {
  double alphac, betac, alphad, betad, alphaf, betaf, alphafca, betafca;
} lcc_rates;

static lcc_rates lcc_rates_at(double cpx, double v, int iso2) {
  lcc_rates r;
  double dv5 = 5, dvk = 8, fv5 = -22.8, fvk = 9.1;
  r.alphac = 0.22;
  r.betac = 4;
  if (iso2) { /* reesica.h:30-35 */
    r.betac = 2;
    dv5 = 0;
    fv5 = -28;
    fvk = 8.5;
  }
  double dinf = 1.0 / (1.0 + exp(-(v - dv5) / dvk));
  double taudin = 1.0 / ((1.0 - exp(-(v - dv5) / dvk)) / (0.035 * (v - dv5)) * dinf);
  if ((v < 0.0001) && (v > -0.0001)) taudin = 0.035 * dvk / dinf;
  double finf = 1. - 1.0 / (1.0 + exp(-(v - fv5) / fvk)) / (1. + exp((v - 60) / 12.));
  double taufin = (0.02 - 0.007 * exp(-SQ(0.0337 * (v + 10.5))));
  r.alphad = dinf * taudin;
  r.betad = (1 - dinf) * taudin;
  r.alphaf = (finf)*taufin;
  r.betaf = (1 - finf) * taufin;
  r.alphafca = 0.012 / 2.;
  r.betafca = 0.175 / (1 + SQ(25 / cpx));
  return r;
}

/* One LCC slot: a single uniform selects at most one gate flip by first
 * passage over the cumulative rates (reesica.h:65-115).  Bit 0 = c gate,
 * bit 1 = d, bit 2 = f, bit 3 = fCa; state 0 is open. */
static int lcc_next(int st, double u, double dt, const lcc_rates* r) {
  double rig = u / dt;
  if ((st % 2)) {
    if (rig < r->alphac) return st - 1;
    rig -= r->alphac;
  } else {
    if (rig < r->betac) return st + 1;
    rig -= r->betac;
  }
  if (((st / 2) % 2)) {
    if (rig < r->alphad) return st - 2;
    rig -= r->alphad;
  } else {
    if (rig < r->betad) return st + 2;
    rig -= r->betad;
  }
  if (((st / 4) % 2)) {
    if (rig < r->alphaf) return st - 4;
    rig -= r->alphaf;
  } else {
    if (rig < r->betaf) return st + 4;
    rig -= r->betaf;
  }
  if (((st / 8) % 2)) {
    if (rig < r->alphafca) return st - 8;
  } else {
    if (rig < r->betafca) return st + 8;
  }
  return st;
}

/* ------------------------------ Init kernel ------------------------------ */

/* Basal state of every CRU incl. ghosts (cuda_Cell_Detailed.cu:1108-1182). */
static void init_lattice(orc_sim* s) {
  /* ci_basal and cjsr_basal are fixed in the perm build (:87-92); tapsi then
   * overrides the load (:1118-1120) */
  const double CI_B = s->p.perm ? PERM_CI_BASAL : CI_BASAL;
  double cjsr_b = s->p.tapsi ? 10 : (s->p.perm ? PERM_CJSR_BASAL : s->p.cjsr_basal);
  for (int ac = 0; ac < s->ntot; ++ac) {
    s->cp[ac] = CI_B;
    s->cs[0][ac] = CI_B;
    s->cs[1][ac] = CI_B;
    s->cjsr[ac] = cjsr_b;
    s->cjsrb[ac] = csqn_bound_ss(cjsr_b);
    s->nspark[ac] = 0;
    s->nl[ac] = 0; /* not set by the reference's Init; reset at step 0 anyway (:1244) */
    s->ancx[ac] = 0.025;
    s->xire[ac] = 0;
    s->po[ac] = 0;
    s->xinaca[ac] = 0;
    s->xicat[ac] = 0;
    for (int ii = 0; ii < 8; ++ii) {
      int a8 = ac * 8 + ii;
      s->ci[0][a8] = CI_B;
      s->ci[1][a8] = CI_B;
      s->cnsr[0][a8] = cjsr_b;
      s->cnsr[1][a8] = cjsr_b;
      s->catf[a8] = KTFON * CI_B * BTF / (KTFON * CI_B + KTFOFF);
      s->cats[a8] = KTSON * CI_B * BTS / (KTSON * CI_B + KTSOFF);
      s->cacal[a8] = KCALON * CI_B * BCAL / (KCALON * CI_B + KCALOFF);
      s->cadye[a8] = KDYEON * CI_B * BDYE / (KDYEON * CI_B + KDYEOFF);
      s->casr[a8] = KSRON * CI_B * BSR / (KSRON * CI_B + KSROFF);
      s->camyo[a8] = 3.;
      s->mgmyo[a8] = 136.209996;
      s->xiup[a8] = 0;
      s->xileak[a8] = 0;
    }
    s->casar[ac] = KSARON * CI_B * BSAR / (KSARON * CI_B + KSAROFF);
    s->casarh[ac] = KSARHON * CI_B * BSARH / (KSARHON * CI_B + KSARHOFF);
    s->casarj[ac] = KSARON * CI_B * BSAR / (KSARON * CI_B + KSAROFF);
    s->casarhj[ac] = KSARHON * CI_B * BSARH / (KSARHON * CI_B + KSARHOFF);
    int randpoint = SVNCP; /* :1150-1155 */
    if (s->p.randomlcc) {
      rh_stream st;
      rh_stream_init(&st, s->p.seed, s->p.cell_id, (uint32_t)ac, RH_PHILOX_INIT_STEP);
      randpoint = (int)(rh_uniform_u32(&st) % 9u);
    }
    for (int ll = 0; ll < 8; ++ll) s->lcc[ac * 8 + ll] = (ll < randpoint) ? 3 : 16;
    double roo2 = RATEDIMER / (1.0 + pow(KDIMER / (cjsr_b), HILLDIMER));
    double aub = (-1.0 + sqrt(1.0 + 8.0 * CSQBERS * roo2)) / (4.0 * roo2 * CSQBERS) / TAUB;
    double abu = 1.0 / TAUU;
    double fracbound = 1 / (1 + abu / aub);
    s->ncb[ac] = (int)(fracbound * NRYR);
    s->ncu[ac] = NRYR - (int)(fracbound * NRYR);
    s->nob[ac] = 0;
    s->nou[ac] = 0;
  }
  s->cur = 0;
}

/* ---------------------------- Compute kernel ----------------------------- */

/* Interior CRU update (cuda_Cell_Detailed.cu:1242-1473, block A). */
static void update_cru(orc_sim* s, int i, int j, int k, double v, double t, double xnai,
                       uint32_t* status) {
  const double dt = s->dt;
  const int ac = opos(s, i, j, k);
  const double* ci = s->ci[s->cur];
  const double* cnsr = s->cnsr[s->cur];
  const double* cs = s->cs[s->cur];
  double* cinext = s->ci[1 - s->cur];
  double* cnsrnext = s->cnsr[1 - s->cur];
  double* csnext = s->cs[1 - s->cur];
  const double randomi = 1.0; /* CRU2.randomi, set to 1 by Init (:1121) */

  rh_stream rng;
  rh_stream_init(&rng, s->p.seed, s->p.cell_id, (uint32_t)ac, (uint64_t)s->m.step);

  if (s->p.iso && fmod(t + 10 * s->p.pcl_ms, 15.5 * s->p.pcl_ms) < dt) { /* :1213-1218 */
    for (int ll = 4; ll < 8; ++ll)
      if (s->lcc[ac * 8 + ll] == 16) s->lcc[ac * 8 + ll] = 3;
  }
  if (fmod(t - dt, OUTT) < dt) { /* window reset (:1244-1247) */
    s->nspark[ac] = 0;
    s->nl[ac] = 0;
  }
  /* LCC channels (:1248-1263); none in the perm build (:1249) */
  double icat1 = 0;
  if (!s->p.perm) {
    double cpx = (s->cp[ac] + cs[ac] * ICAGAMMA) / (1 + ICAGAMMA);
    lcc_rates lr = lcc_rates_at(cpx, v, s->p.iso2);
    int nlcp = 0;
    for (int ll = 0; ll < 8 && s->lcc[ac * 8 + ll] < 16; ll++) {
      double u = rh_uniform_double(&rng);
      int jj = lcc_next(s->lcc[ac * 8 + ll], u, dt, &lr);
      s->lcc[ac * 8 + ll] = jj;
      if (jj == 0) {
        ++s->nl[ac];
        ++nlcp;
      }
    }
    icat1 = s->svica * (double)(nlcp)*lcc_flux(v, cpx, s->cao);
  }
  const double pmca = 0; /* :1265 */
  double bcgcur = 0;
  if (s->p.slowncx) bcgcur = 1.0 * 0.003016 / 32. * (v - log(180000 / cs[ac]) / 2. / FRT); /* :1268 */
  s->xicat[ac] = icat1 + pmca + bcgcur * (VS / VP);

  /* RyR gating and release (:1274-1293) */
  int prevsp = s->nou[ac] + s->nob[ac];
  ryr_gating(&rng, s->p.ku, s->p.ku2, s->p.kb, s->cp[ac], s->cjsr[ac], &s->ncu[ac], &s->nou[ac],
             &s->ncb[ac], &s->nob[ac], dt, status);
  if (prevsp < 5 && (s->nou[ac] + s->nob[ac]) >= 5) s->nspark[ac] = 1;
  s->po[ac] = (double)(s->nou[ac] + s->nob[ac]) / (double)(NRYR);
  s->xire[ac] = jsr_release(s->po[ac], s->cjsr[ac], s->cp[ac]) / randomi;
  if (s->xire[ac] < 0) s->xire[ac] = 0;

  /* NCX (:1296); zero in the perm build, Ancx then keeps its value (:1302) */
  if (s->p.perm)
    s->xinaca[ac] = 0;
  else if (s->p.ncx_form == RH_NCX_OLD) /* the commented alternative call, :1300 */
    s->xinaca[ac] = s->svncx * 1.0 * ncx_old_flux(cs[ac] / 1000.0, v, xnai, &s->ancx[ac], dt, s->cao);
  else if (s->p.ncx_form == RH_NCX_NOALLO)
    s->xinaca[ac] = s->svncx * 1.0 * ncx_noallo_flux(cs[ac] / 1000.0, v, xnai, s->cao);
  else
    s->xinaca[ac] = s->svncx * 1.0 *
                    ncx_flux(cs[ac] / 1000.0, v, xnai, &s->ancx[ac], dt, s->cao, s->p.slowncx);

  /* SERCA and leak per sub-voxel (:1305-1308) */
  for (int ii = 0; ii < 8; ++ii) {
    int a8 = ac * 8 + ii;
    s->xiup[a8] = s->sviup_now * serca(ci[a8], cnsr[a8]);
    s->xileak[a8] = SVILEAK * sr_leak(cnsr[a8], ci[a8]);
  }
  /* dyad / submembrane / JSR couplings (:1309-1317) */
  double diffpi0 = (s->cp[ac] - ci[ac * 8]) / TAUPI / 2.;
  double diffpi1 = (s->cp[ac] - ci[ac * 8 + 1]) / TAUPI / 2.;
  double diffsi0 = (cs[ac] - ci[ac * 8]) / TAUSI / 2.;
  double diffsi1 = (cs[ac] - ci[ac * 8 + 1]) / TAUSI / 2.;
  double diffjn0 = (s->cjsr[ac] - cnsr[ac * 8]) / TAUTR / 2.;
  double diffjn1 = (s->cjsr[ac] - cnsr[ac * 8 + 1]) / TAUTR / 2.;
  double beta = csqn_beta(s->cjsr[ac]);
  double dotcjsr = beta * ((-diffjn0 - diffjn1) - s->xire[ac] * VP * randomi / VJSR);
  s->cjsrb[ac] += (1 - beta) * ((-diffjn0 - diffjn1) - s->xire[ac] * VP * randomi / VJSR) * dt;

  /* sub-voxel diffusion and cytosolic buffers (:1320-1355) */
  double dotci[8], dotcnsr[8];
  for (int ii = 0; ii < 8; ++ii) {
    int act = ac * 8 + ii;
    int north = (ii % 2) ? (opos(s, i, j, k + 1) * 8 + ii - 1) : (ac * 8 + ii + 1);
    int south = (ii % 2) ? (ac * 8 + ii - 1) : (opos(s, i, j, k - 1) * 8 + ii + 1);
    int east = ((ii / 2) % 2) ? (opos(s, i, j + 1, k) * 8 + ii - 2) : (ac * 8 + ii + 2);
    int west = ((ii / 2) % 2) ? (ac * 8 + ii - 2) : (opos(s, i, j - 1, k) * 8 + ii + 2);
    int top = ((ii / 4) % 2) ? (opos(s, i + 1, j, k) * 8 + ii - 4) : (ac * 8 + ii + 4);
    int bottom = ((ii / 4) % 2) ? (ac * 8 + ii - 4) : (opos(s, i - 1, j, k) * 8 + ii + 4);
    double coupn = ((cnsr[north] - cnsr[act]) / (TAUNT * XI) +
                    (cnsr[south] - cnsr[act]) / (TAUNT * XI) +
                    (cnsr[east] - cnsr[act]) / (TAUNT * XI) +
                    (cnsr[west] - cnsr[act]) / (TAUNT * XI) +
                    (cnsr[top] - cnsr[act]) / (TAUNL * XI) +
                    (cnsr[bottom] - cnsr[act]) / (TAUNL * XI));
    double coupi = ((ci[north] - ci[act]) / (TAUIT * XI) + (ci[south] - ci[act]) / (TAUIT * XI) +
                    (ci[east] - ci[act]) / (TAUIT * XI) + (ci[west] - ci[act]) / (TAUIT * XI) +
                    (ci[top] - ci[act]) / (TAUIL * XI) + (ci[bottom] - ci[act]) / (TAUIL * XI));
    dotcnsr[ii] = (s->xiup[act] - s->xileak[act]) * VI / VNSR + coupn;
    double c = ci[act];
    double buffers = (buffer_rate(KTFON, KTFOFF, BTF, s->catf[act], c, dt) +
                      buffer_rate(KTSON, KTSOFF, BTS, s->cats[act], c, dt) +
                      buffer_rate(KCALON, KCALOFF, BCAL, s->cacal[act], c, dt) +
                      buffer_rate(KSRON, KSROFF, BSR, s->casr[act], c, dt) +
                      myo_ca_rate(s->camyo[act], s->mgmyo[act], c, dt));
    dotci[ii] = (-s->xiup[act] + s->xileak[act]) - buffers + coupi;
  }
  dotcnsr[0] += diffjn0 * VJSR / VNSR; /* :1356-1361 */
  dotcnsr[1] += diffjn1 * VJSR / VNSR;
  dotci[0] += diffsi0 * (VS / VI);
  dotci[1] += diffsi1 * (VS / VI);
  dotci[0] += diffpi0 * (VP / VI);
  dotci[1] += diffpi1 * (VP / VI);

  /* explicit Euler of ci, cnsr and the cytosolic buffers (:1364-1393) */
  for (int ii = 0; ii < 8; ++ii) {
    int act = ac * 8 + ii;
    double c = ci[act];
    cinext[act] = ci[act] + dotci[ii] * dt;
    if (cinext[act] < 0) cinext[act] = 0;
    cnsrnext[act] = cnsr[act] + dotcnsr[ii] * dt;
    s->catf[act] += buffer_rate(KTFON, KTFOFF, BTF, s->catf[act], c, dt) * dt;
    if (s->catf[act] < 0) s->catf[act] = 0;
    s->cats[act] += buffer_rate(KTSON, KTSOFF, BTS, s->cats[act], c, dt) * dt;
    if (s->cats[act] < 0) s->cats[act] = 0;
    s->cacal[act] += buffer_rate(KCALON, KCALOFF, BCAL, s->cacal[act], c, dt) * dt;
    if (s->cacal[act] < 0) s->cacal[act] = 0;
    s->casr[act] += buffer_rate(KSRON, KSROFF, BSR, s->casr[act], c, dt) * dt;
    if (s->casr[act] < 0) s->casr[act] = 0;
    s->camyo[act] += myo_ca_rate(s->camyo[act], s->mgmyo[act], c, dt) * dt;
    if (s->camyo[act] < 0) s->camyo[act] = 0;
    s->mgmyo[act] += myo_mg_rate(s->camyo[act], s->mgmyo[act], dt) * dt;
    if (s->mgmyo[act] < 0) s->mgmyo[act] = 0;
    s->cadye[act] += buffer_rate(KDYEON, KDYEOFF, BDYE, s->cadye[act], c, dt) * dt;
    if (s->cadye[act] < 0) s->cadye[act] = 0;
  }

  /* five sub-steps of cs, cp and the sarcolemmal buffers (:1396-1464) */
  csnext[ac] = cs[ac];
  double cpstart = s->cp[ac];
  int finestep = 5;
  double dth = dt / finestep;
  int kz_up = opos(s, i, j, k + 1), kz_dn = opos(s, i, j, k - 1);
  for (int iii = 0; iii < finestep; ++iii) {
    double csbuffers = (buffer_rate(KSARON, KSAROFF, BSAR, s->casar[ac], csnext[ac], dth) +
                        buffer_rate(KSARHON, KSARHOFF, BSARH, s->casarh[ac], csnext[ac], dth));
    double csdiff = (cs[kz_up] + cs[kz_dn] - 2 * cs[ac]) / (TAUST);
    if (s->p.perm) csdiff += (PERM_CI_BASAL - csnext[ac]) / 5; /* :1409-1411 */
    double dotcs = VP / VS * (s->cp[ac] - csnext[ac]) / (TAUPS) - ICAGAMMA * icat1 * VP / VS +
                   s->xinaca[ac] - (cs[ac] - ci[ac * 8]) / TAUSI / 2. -
                   (cs[ac] - ci[ac * 8 + 1]) / TAUSI / 2. + csdiff - csbuffers - bcgcur;
    double cpbuff = buffer_rate(KSARON, KSAROFF, BSAR, s->casarj[ac], s->cp[ac], dth);
    double cpbuffh = buffer_rate(KSARHON, KSARHOFF, BSARH, s->casarhj[ac], s->cp[ac], dth);
    double cpdot = ((csnext[ac] - s->cp[ac]) / TAUPS + (ci[ac * 8] - cpstart) / TAUPI / 2. +
                    (ci[ac * 8 + 1] - cpstart) / TAUPI / 2. + s->xire[ac] - icat1 - cpbuff -
                    cpbuffh);
    s->casarj[ac] += cpbuff * dt / finestep;
    if (s->casarj[ac] < 0) s->casarj[ac] = 0;
    s->casarhj[ac] += cpbuffh * dt / finestep;
    if (s->casarhj[ac] < 0) s->casarhj[ac] = 0;
    s->cp[ac] += cpdot * dt / finestep;
    s->casar[ac] +=
        buffer_rate(KSARON, KSAROFF, BSAR, s->casar[ac], csnext[ac], dt / finestep) * dt / finestep;
    if (s->casar[ac] < 0) s->casar[ac] = 0;
    s->casarh[ac] += buffer_rate(KSARHON, KSARHOFF, BSARH, s->casarh[ac], csnext[ac],
                                 dt / finestep) * dt / finestep;
    if (s->casarh[ac] < 0) s->casarh[ac] = 0;
    csnext[ac] += (dotcs)*dth;
  }
  if (s->cp[ac] < 0) s->cp[ac] = 0; /* :1466-1473 */
  if (csnext[ac] < 0) csnext[ac] = 1e-6;
  s->cjsr[ac] = s->cjsr[ac] + dotcjsr * dt;
}

/* Zero-flux boundaries: ghost faces copy the facing interior sub-voxels
 * (cuda_Cell_Detailed.cu:1603-1652).  Only face ghosts are written, which are
 * the only ghosts the stencil reads.  The perm build copies only cnsr
 * (:1653-1689): the ci and cs ghosts keep their initial bath value. */
static void apply_ghost_faces(orc_sim* s) {
  const int perm = s->p.perm;
  double* ci = s->ci[1 - s->cur];
  double* cn = s->cnsr[1 - s->cur];
  double* cs = s->cs[1 - s->cur];
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  for (int k = 1; k < nz - 1; ++k)
    for (int j = 1; j < ny - 1; ++j) {
      int g0 = opos(s, 0, j, k) * 8, i1 = opos(s, 1, j, k) * 8;
      int g1 = opos(s, nx - 1, j, k) * 8, i2 = opos(s, nx - 2, j, k) * 8;
      for (int ii = 4; ii < 8; ++ii) {
        if (!perm) ci[g0 + ii] = ci[i1 + ii - 4];
        cn[g0 + ii] = cn[i1 + ii - 4];
      }
      for (int ii = 0; ii < 4; ++ii) {
        if (!perm) ci[g1 + ii] = ci[i2 + ii + 4];
        cn[g1 + ii] = cn[i2 + ii + 4];
      }
    }
  for (int k = 1; k < nz - 1; ++k)
    for (int i = 1; i < nx - 1; ++i) {
      int g0 = opos(s, i, 0, k) * 8, i1 = opos(s, i, 1, k) * 8;
      int g1 = opos(s, i, ny - 1, k) * 8, i2 = opos(s, i, ny - 2, k) * 8;
      for (int ii = 2; ii < 8; ii += 4) {
        if (!perm) {
          ci[g0 + ii] = ci[i1 + ii - 2];
          ci[g0 + ii + 1] = ci[i1 + ii - 1];
        }
        cn[g0 + ii] = cn[i1 + ii - 2];
        cn[g0 + ii + 1] = cn[i1 + ii - 1];
      }
      for (int ii = 0; ii < 8; ii += 4) {
        if (!perm) {
          ci[g1 + ii] = ci[i2 + ii + 2];
          ci[g1 + ii + 1] = ci[i2 + ii + 3];
        }
        cn[g1 + ii] = cn[i2 + ii + 2];
        cn[g1 + ii + 1] = cn[i2 + ii + 3];
      }
    }
  for (int j = 1; j < ny - 1; ++j)
    for (int i = 1; i < nx - 1; ++i) {
      int g0 = opos(s, i, j, 0), i1 = opos(s, i, j, 1);
      int g1 = opos(s, i, j, nz - 1), i2 = opos(s, i, j, nz - 2);
      for (int ii = 1; ii < 8; ii += 2) {
        if (!perm) ci[g0 * 8 + ii] = ci[i1 * 8 + ii - 1];
        cn[g0 * 8 + ii] = cn[i1 * 8 + ii - 1];
      }
      for (int ii = 0; ii < 8; ii += 2) {
        if (!perm) ci[g1 * 8 + ii] = ci[i2 * 8 + ii + 1];
        cn[g1 * 8 + ii] = cn[i2 * 8 + ii + 1];
      }
      if (!perm) {
        cs[g0] = cs[i1];
        cs[g1] = cs[i2];
      }
    }
}

void orc_lattice_step(orc_sim* s) {
  const double v = s->m.v, t = s->m.t, xnai = s->m.xnai;
  s->sviup_now = (s->p.iso && t >= 5.5 * s->p.pcl_ms) ? s->sviup_iso : s->sviup_tot; /* :1219 */
  const int lx = s->nx - 2, ly = s->ny - 2, lz = s->nz - 2;
  const int n = lx * ly * lz;
  uint32_t st = 0;
#ifdef _OPENMP
  int nt = orc_get_threads();
#pragma omp parallel for num_threads(nt) schedule(static) reduction(| : st)
#endif
  for (int q = 0; q < n; ++q) {
    int i = 1 + q % lx, j = 1 + (q / lx) % ly, k = 1 + q / (lx * ly);
    update_cru(s, i, j, k, v, t, xnai, &st);
  }
  s->status |= st;
  apply_ghost_faces(s);
  s->cur = 1 - s->cur; /* ping-pong swap (:422-425) */
}

/* --------------------- host whole-cell model (:427-739) ------------------- */

static void wholecell_reduce(orc_sim* s) {
  const double* cs = s->cs[s->cur];
  double csubt = 0, xicatto = 0, xinacato = 0;
  for (int jz = 1; jz < s->nz - 1; jz++)
    for (int jy = 1; jy < s->ny - 1; jy++)
      for (int jx = 1; jx < s->nx - 1; jx++) {
        int ac = opos(s, jx, jy, jz);
        csubt += cs[ac];
        xicatto = xicatto + s->xicat[ac];
        xinacato = xinacato + s->xinaca[ac];
      }
  csubt = csubt / ((s->nx - 2) * (s->ny - 2) * (s->nz - 2));
  xicatto = xicatto / CM * 0.0965 * VP * 2.0 * (ICAGAMMA + 1.);
  xinacato = xinacato / CM * 0.0965 * VS;
  s->m.csubt = csubt;
  s->m.xicatto = xicatto;
  s->m.xinacato = xinacato;
}

/* Membrane currents, gates, [Na]i and V (cuda_Cell_Detailed.cu:458-739). */
static void membrane_update(orc_sim* s) {
  rh_membrane* m = &s->m;
  const double dt = s->dt, t = m->t, v = m->v, tperid = s->p.pcl_ms;
  const double xki = 140.0, xko = 5.40; /* :350-351 */
  const double csubt = m->csubt;
  double xnai = m->xnai;
  /* INa (:460-502) */
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
  double xina = gna * m->xh * m->xj * m->xm * m->xm * m->xm * (v - ena) + gnaleak * (v - ena);
  m->xh = ah / (ah + bh) - ((ah / (ah + bh)) - m->xh) * exp(-dt / tauh);
  m->xj = aj / (aj + bj) - ((aj / (aj + bj)) - m->xj) * exp(-dt / tauj);
  m->xm = am / (am + bm) - ((am / (am + bm)) - m->xm) * exp(-dt / taum);
  /* IKr (:507-529) */
  double ek = (1.00 / FRT) * log(xko / xki);
  double gss = sqrt(xko / 5.40);
  double xkrv1 = 0.001380 * (v + 7.00) / (1.0 - exp(-0.123 * (v + 7.00)));
  double xkrv2 = 0.000610 * (v + 10.00) / (exp(0.1450 * (v + 10.00)) - 1.00);
  double taukr = 1.00 / (xkrv1 + xkrv2);
  double xkrinf = 1.00 / (1.00 + exp(-(v + 50.00) / 7.50));
  double rg = 1.00 / (1.00 + exp((v + 33.00) / 22.40));
  double gkr = 0.0078360;
  double xikr = s->svikr * gkr * gss * m->xr * rg * (v - ek);
  m->xr = xkrinf - (xkrinf - m->xr) * exp(-dt / taukr);
  /* IKs (:534-559) */
  double prnak = 0.0183300;
  double qks_inf = 0.2 * (1 + 0.8 / (1 + pow((0.28 / csubt), 3)));
  double tauqks = 1000.00;
  if (s->p.slowncx) { /* :540-543 */
    qks_inf = 0.2 * (1 + 1.6 / (1 + pow((0.28 / csubt), 3)));
    tauqks = 2000;
  }
  double eks = (1.00 / FRT) * log((xko + prnak * XNAO) / (xki + prnak * xnai));
  double xs1ss = 1.0 / (1.0 + exp(-(v - 1.500) / 16.700));
  double tauxs = 1.00 / (0.0000719 * (v + 30.00) / (1.00 - exp(-0.1480 * (v + 30.0))) +
                         0.0001310 * (v + 30.00) / (exp(0.06870 * (v + 30.00)) - 1.00));
  tauxs = SVTAUXS * tauxs;
  double gksx = 0.2000;
  double sviks = 1.0, sviks_iso = 1.;
  double xiks = sviks * sviks_iso * gksx * m->qks * m->xs1 * m->xs2 * (v - eks);
  m->xs1 = xs1ss - (xs1ss - m->xs1) * exp(-dt / tauxs);
  m->xs2 = xs1ss - (xs1ss - m->xs2) * exp(-dt / tauxs);
  m->qks = m->qks + dt * (qks_inf - m->qks) / tauqks;
  /* IK1 (:590-600) */
  double gkix = 0.600;
  double gki = gkix * (sqrt(xko / 5.4));
  double aki = 1.02 / (1.0 + exp(0.2385 * (v - ek - 59.215)));
  double bki = (0.49124 * exp(0.08032 * (v - ek + 5.476)) + exp(0.061750 * (v - ek - 594.31))) /
               (1.0 + exp(-0.5143 * (v - ek + 4.753)));
  double xkin = aki / (aki + bki);
  double svk1 = (1.0);
  double xik1 = svk1 * gki * xkin * (v - ek);
  /* Ito,s (:604-629) */
  double rt1 = -(v + 3.0) / 15.00;
  double rt2 = (v + 33.5) / 10.00;
  double rt3 = (v + 60.00) / 10.00;
  double xtos_inf = 1.00 / (1.0 + exp(rt1));
  double ytos_inf = 1.00 / (1.00 + exp(rt2));
  double rs_inf = 1.00 / (1.00 + exp(rt2));
  double txs = 9.00 / (1.00 + exp(-rt1)) + 0.50;
  double tys = 3000.00 / (1.0 + exp(rt3)) + 30.00;
  double gtos = 0.040;
  double svtos = 1.0, svtof = 1.0;
  double xitos = svtos * gtos * m->xtos * (m->ytos + 0.50 * rs_inf) * (v - ek);
  m->xtos = xtos_inf - (xtos_inf - m->xtos) * exp(-dt / txs);
  m->ytos = ytos_inf - (ytos_inf - m->ytos) * exp(-dt / tys);
  /* Ito,f (:633-659) */
  double xtof_inf = xtos_inf;
  double ytof_inf = ytos_inf;
  double rt4 = -(v / 30.00) * (v / 30.00);
  double rt5 = (v + 33.50) / 10.00;
  double txf = 3.50 * exp(rt4) + 1.50;
  double tyf = 20.0 / (1.0 + exp(rt5)) + 20.00;
  double gtof = 0.10;
  double xitof = svtof * gtof * m->xtof * m->ytof * (v - ek);
  m->xtof = xtof_inf - (xtof_inf - m->xtof) * exp(-dt / txf);
  m->ytof = ytof_inf - (ytof_inf - m->ytof) * exp(-dt / tyf);
  /* INaK (:665-676) */
  double xkmko = 1.50, xkmnai = 12.00, xibarnak = 1.5000, hh = 1.00, svnak = 1.;
  double sigma = (exp(XNAO / 67.30) - 1.00) / 7.00;
  double fnak = 1.00 / (1.0 + 0.1245 * exp(-0.1 * v * FRT) + 0.0365 * sigma * exp(-v * FRT));
  double xinak =
      svnak * xibarnak * fnak * (1.0 / (1.0 + pow((xkmnai / xnai), hh))) * xko / (xko + xkmko);
  /* stimulus (:689-692; iso :683-687); none in the nopacing and perm builds
   * (:694-699) */
  double stim;
  if (s->p.iso) {
    if (fmod(t, tperid) < 1.0 && (t < tperid * 11.9)) stim = 80.0;
    else stim = 0.0;
  } else if (fmod(t + tperid - 100, tperid) < 1.0) stim = 80.0;
  else stim = 0.0;
  if (s->p.protocol == RH_PROTO_NOPACING || s->p.perm) stim = 0.0;
  /* [Na]i and V (:701-738) */
  double wcainv = 1.0 / 50.0;
  double conv = 0.18 * 12500;
  double xinaca = m->xinacato;
  double trick = 1.0;
  double xrr = trick * (1.0 / wcainv / conv) / 1000.0;
  double dnai = -xrr * (xina + 3.0 * xinak + 3.0 * xinaca);
  m->xnai = xnai + dnai * dt;
  double dvh = -(xina + xik1 + 1 * xikr + 1 * xiks + xitos + 1 * xitof + 1. * m->xinacato +
                 1 * m->xicatto + xinak) +
               stim;
  m->v = v + dvh * dt;
  /* voltage protocols (:733-773): the clamp replaces the integrated V */
  switch (s->p.protocol) {
    case RH_PROTO_VCLAMP: /* :733-739 */
      m->v = -86;
      if (t > 100) m->v = s->p.clamp_mv;
      break;
    case RH_PROTO_BROWN_VCLAMP: /* :741-752 */
      if (t < 4000) m->v = -86;
      else if (t < 4200) m->v = -10;
      else if (t < 6200) m->v = 10;
      else if (t < 7200) m->v = -30;
      else m->v = -86;
      break;
    case RH_PROTO_AP_CLAMP: /* :754-757 */
      m->v = s->apv[((int)(t / dt + 0.1)) % ((int)(tperid / dt + 0.1))];
      break;
    case RH_PROTO_LINEAR_AP_CLAMP: /* :758-773 */
      if (t < 100) m->v = -86;
      else if (t < 101.865) m->v = 68 * (t - 100) - 80;
      else if (t < 119.1) m->v = -(t - 100) + 48;
      else if (t < 138.9) m->v = 27 + 0.1 * (t - 100);
      else if (t < 364.43) m->v = 43 - (t - 100) / 3.2;
      else if (t < 395.43) m->v = -1.5 * (t - 100) + 357;
      else m->v = -86;
      break;
    default:
      break;
  }
  m->out_ica += m->xicatto; /* :774-776 */
  m->out_ncx += m->xinacato;
  m->out_ina += xina;
  m->xina = xina;
  m->xiks = xiks;
  m->xikr = xikr;
  m->xik1 = xik1;
  m->xinak = xinak;
  m->xitos = xitos;
  m->xitof = xitof;
}

/* Output statistics at an output step (cuda_Cell_Detailed.cu:788-1079). */
/* cadist record (cuda_Cell_Detailed.cu:1001-1013, the outputcadist build):
 * every 5 ms during the first 500 ms of each pacing period, "0 header t v"
 * and per interior CRU (jx outer, jz inner) ci of sub-voxel 0, cs, cp, cjsr,
 * xinaca/Cm*0.0965*Vs*16120 and xire. */
static void cadist_record(orc_sim* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double* ci = s->ci[s->cur];
  const double* cs = s->cs[s->cur];
  double* r = s->cd;
  *r++ = s->m.t;
  *r++ = s->m.v;
  for (int jx = 1; jx < nx - 1; jx++)
    for (int jy = 1; jy < ny - 1; jy++)
      for (int jz = 1; jz < nz - 1; jz++) {
        const int ac = opos(s, jx, jy, jz);
        *r++ = ci[ac * 8];
        *r++ = cs[ac];
        *r++ = s->cp[ac];
        *r++ = s->cjsr[ac];
        *r++ = s->xinaca[ac] / CM * 0.0965 * VS * 16120.;
        *r++ = s->xire[ac];
      }
  s->cd_valid = 1;
}

static void output_record(orc_sim* s) {
  const int nx = s->nx, ny = s->ny, nz = s->nz;
  const double* ci = s->ci[s->cur];
  const double* cnsr = s->cnsr[s->cur];
  const double* cs = s->cs[s->cur];
  rh_membrane* m = &s->m;
  const double dt = s->dt;
  double cproxit = 0, cjsrt = 0, csqnbt = 0, cnsrt = 0, poto = 0, pbcto = 0, ncxfwd = 0;
  double catft = 0, catst = 0, casrt = 0, camyot = 0, mgmyot = 0, cacalt = 0, cadyet = 0;
  double casart = 0, casarht = 0, casarjt = 0, casarhjt = 0, leakt = 0, upt = 0, ire = 0;
  double icaflux = 0, ncxflux = 0, outancx = 0, cit = 0;
  int tn1 = 0, tn2 = 0, tn3 = 0, tn4 = 0, tn5 = 0, tn6 = 0, tn7 = 0;
  int tnou = 0, tnob = 0, tncu = 0, tncb = 0;
  for (int jz = 1; jz < nz - 1; jz++)
    for (int jy = 1; jy < ny - 1; jy++)
      for (int jx = 1; jx < nx - 1; jx++) {
        int ac = opos(s, jx, jy, jz);
        icaflux = icaflux + s->xicat[ac];
        ncxflux = ncxflux + s->xinaca[ac];
        if (s->xinaca[ac] < 0) ncxfwd = ncxfwd + s->xinaca[ac];
        outancx += s->ancx[ac];
        cproxit = cproxit + s->cp[ac];
        cjsrt = cjsrt + s->cjsr[ac];
        csqnbt = csqnbt + s->cjsrb[ac];
        poto = poto + s->po[ac];
        pbcto = pbcto + s->ncb[ac];
        casart += s->casar[ac];
        casarht += s->casarh[ac];
        casarjt += s->casarj[ac];
        casarhjt += s->casarhj[ac];
        for (int ii = 0; ii < 8; ++ii) {
          int a8 = ac * 8 + ii;
          cit += ci[a8] / 8.;
          cnsrt = cnsrt + cnsr[a8] / 8.;
          catft = catft + s->catf[a8] / 8.;
          catst = catst + s->cats[a8] / 8.;
          casrt = casrt + s->casr[a8] / 8.;
          camyot = camyot + s->camyo[a8] / 8.;
          mgmyot = mgmyot + s->mgmyo[a8] / 8.;
          cacalt = cacalt + s->cacal[a8] / 8.;
          cadyet = cadyet + s->cadye[a8] / 8.;
          leakt = leakt + s->xileak[a8] / 8.;
          upt = upt + s->xiup[a8] / 8.;
          if (ci[a8] > 1000) s->status |= RH_STATUS_CI_HIGH;
        }
        ire += s->xire[ac];
        tnou += s->nou[ac];
        tnob += s->nob[ac];
        tncu += s->ncu[ac];
        tncb += s->ncb[ac];
        m->sparksum += s->nspark[ac];
        for (int jj = 0; jj < 8; ++jj) {
          switch (s->lcc[ac * 8 + jj]) { /* gate-bit counts (:904-923) */
            case 1: ++tn1; ++tn6; break;
            case 2: ++tn2; break;
            case 3: ++tn1; ++tn2; break;
            case 4: ++tn3; ++tn5; break;
            case 5: ++tn1; ++tn3; ++tn5; break;
            case 6: ++tn2; ++tn3; ++tn5; break;
            case 7: ++tn1; ++tn2; ++tn3; ++tn5; break;
            case 8: ++tn4; break;
            case 9: ++tn1; ++tn4; break;
            case 10: ++tn2; ++tn4; break;
            case 11: ++tn1; ++tn2; ++tn4; break;
            case 12: ++tn3; ++tn4; break;
            case 13: ++tn1; ++tn3; ++tn4; break;
            case 14: ++tn2; ++tn3; ++tn4; break;
            case 15: ++tn1; ++tn2; ++tn3; ++tn4; break;
            case 0: ++tn7; ++tn6; break;
          }
        }
      }
  const int nin = (nx - 2) * (ny - 2) * (nz - 2);
  cproxit = cproxit / nin;
  cjsrt = cjsrt / nin;
  csqnbt = csqnbt / nin;
  cnsrt = cnsrt / nin;
  cit /= nin;
  poto = poto / nin;
  pbcto = pbcto / nin / 100.;
  catft = catft / nin;
  catst = catst / nin;
  casrt = casrt / nin;
  camyot /= nin;
  mgmyot /= nin;
  cacalt = cacalt / nin;
  leakt = leakt / nin;
  upt = upt / nin;
  ire = ire / nin;
  ncxfwd /= nin;
  outancx /= nin;
  casart /= nin;
  casarht /= nin;
  casarjt /= nin;
  casarhjt /= nin;
  const double csubt = m->csubt;
  /* linescan (:967-998) */
  {
    int jz = s->jz_line, jy = ny / 2;
    for (int jx = 1; jx < nx - 1; jx++) {
      int ac = opos(s, jx, jy, jz);
      double* r = s->ls + (size_t)(jx - 1) * RH_LINESCAN_COLS;
      r[0] = m->t;
      r[1] = (double)jx;
      r[2] = ci[ac * 8];
      r[3] = s->nob[ac];
      r[4] = s->nou[ac];
      r[5] = s->ncb[ac];
      r[6] = s->ncu[ac];
      r[7] = s->nl[ac];
      r[8] = cs[ac];
      r[9] = s->cp[ac];
      r[10] = s->casar[ac];
      r[11] = s->casarh[ac];
      r[12] = s->camyo[ac * 8];
      r[13] = s->mgmyo[ac * 8];
      r[14] = s->casr[ac * 8];
      r[15] = s->cacal[ac * 8];
      r[16] = s->cats[ac * 8];
      r[17] = s->catf[ac * 8];
      r[18] = s->xire[ac];
      r[19] = s->cjsr[ac];
      r[20] = s->ancx[ac];
      r[21] = s->xinaca[ac];
    }
  }
  /* Total Ca bookkeeping (:1031-1039) */
  double total_ca = (cit + catft + catst + casrt + camyot + cacalt) * VI * 8. +
                    (csubt + casart + casarht) * VS + (cproxit + casarjt + casarhjt) * VP +
                    (cnsrt)*VNSR * 8. + (cjsrt + csqnbt) * VJSR;
  double total_ci = (cit + catft + catst + casrt + camyot + cacalt) * VI * 8. +
                    (csubt + casart + casarht) * VS + (cproxit + casarjt + casarhjt) * VP;
  double* w = s->wc;
  w[0] = m->t;
  w[1] = cit;
  w[2] = m->v;
  w[3] = m->out_ncx / (OUTT / dt);
  w[4] = m->out_ica / (OUTT / dt);
  w[5] = cproxit;
  w[6] = csubt;
  w[7] = cjsrt;
  w[8] = cnsrt;
  w[9] = poto;
  w[10] = m->xnai;
  w[11] = m->xiks;
  w[12] = m->xikr;
  w[13] = m->xik1;
  w[14] = m->xinak;
  w[15] = m->xitos;
  w[16] = m->xitof;
  w[17] = m->out_ina / (OUTT / dt);
  w[18] = m->xr;
  w[19] = ncxfwd * (VS / VP);
  w[20] = pbcto;
  w[21] = cacalt;
  w[22] = catft;
  w[23] = leakt;
  w[24] = upt;
  w[25] = ire;
  w[26] = tnou;
  w[27] = tnob;
  w[28] = tncu;
  w[29] = tncb;
  w[30] = tn1;
  w[31] = tn2;
  w[32] = tn3;
  w[33] = tn4;
  w[34] = tn5;
  w[35] = tn6;
  w[36] = tn7;
  w[37] = outancx;
  w[38] = m->xs1;
  w[39] = m->qks;
  w[40] = (double)m->sparksum;
  w[41] = catst;
  w[42] = csqnbt;
  w[43] = total_ci;
  w[44] = total_ca;
  (void)icaflux;
  (void)ncxflux;
  (void)mgmyot;
  (void)cadyet;
  m->sparksum = 0; /* :1074-1077 */
  m->out_ica = 0;
  m->out_ncx = 0;
  m->out_ina = 0;
}

int orc_step(orc_sim* s) {
  if (s->p.protocol == RH_PROTO_AP_CLAMP && !s->apv) return -1; /* no waveform */
  orc_lattice_step(s);
  s->m.step += 1;
  wholecell_reduce(s);
  membrane_update(s);
  int out = 0;
  s->cd_valid = 0;
  if (fmod(s->m.t + 0.0000001, OUTT) < s->dt) { /* :777 */
    output_record(s);
    out = 1;
    if (fmod(s->m.t + 0.0000001, 5) < s->dt && fmod(s->m.t + 0.0000001, s->p.pcl_ms) < 500)
      cadist_record(s); /* :1002 */
  }
  s->m.t = s->m.t + s->dt; /* :1083 */
  return out;
}

int32_t orc_protocol_done(const orc_sim* s) { return !(s->m.t < s->tend); }

int32_t orc_set_ap_clamp(orc_sim* s, const double* v, int64_t n) {
  const int need = (int)(s->p.pcl_ms / s->dt + 0.1); /* numsteps, :384 */
  if (s->p.protocol != RH_PROTO_AP_CLAMP || !v || n != need) return -1;
  double* w = (double*)malloc(sizeof(double) * (size_t)n);
  if (!w) return -1;
  memcpy(w, v, sizeof(double) * (size_t)n);
  free(s->apv);
  s->apv = w;
  s->napv = need;
  return 0;
}

int64_t orc_run(orc_sim* s, int64_t nsteps, double* wholecell, int32_t max_rec, int32_t* nrec,
                double* linescan, int32_t max_blocks, int32_t* nblocks) {
  int64_t done = 0;
  int32_t nr = 0, nb = 0;
  const int lrows = s->nx - 2;
  while (done < nsteps && s->m.t < s->tend) { /* :399 */
    const int out = orc_step(s);
    if (out < 0) break;
    if (out) {
      if (wholecell && nr < max_rec)
        memcpy(wholecell + (size_t)nr * RH_WHOLECELL_COLS, s->wc, sizeof(s->wc));
      if (nr < max_rec) nr++;
      if (linescan && nb < max_blocks) {
        memcpy(linescan + (size_t)nb * lrows * RH_LINESCAN_COLS, s->ls,
               sizeof(double) * lrows * RH_LINESCAN_COLS);
        nb++;
      }
    }
    done++;
  }
  if (nrec) *nrec = nr;
  if (nblocks) *nblocks = nb;
  return done;
}

int64_t orc_run_traced(orc_sim* s, int64_t nsteps, double* t_out, double* v_out,
                       double* wholecell, int32_t max_rec, int32_t* nrec) {
  int64_t done = 0;
  int32_t nr = 0;
  while (done < nsteps && s->m.t < s->tend) {
    double t0 = s->m.t;
    int out = orc_step(s);
    if (out < 0) break;
    if (t_out) t_out[done] = t0;
    if (v_out) v_out[done] = s->m.v;
    if (out && wholecell && nr < max_rec) {
      memcpy(wholecell + (size_t)nr * RH_WHOLECELL_COLS, s->wc, sizeof(s->wc));
      nr++;
    }
    done++;
  }
  if (nrec) *nrec = nr;
  return done;
}

/* ------------------------------ construction ----------------------------- */

orc_sim* orc_create(const rh_cell_params* p, double dt) {
  if (!p || p->nx < 3 || p->ny < 3 || p->nz < 3 || !(dt > 0)) return NULL;
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  if (!s) return NULL;
  s->p = *p;
  s->nx = p->nx;
  s->ny = p->ny;
  s->nz = p->nz;
  s->ntot = p->nx * p->ny * p->nz;
  s->nin = (p->nx - 2) * (p->ny - 2) * (p->nz - 2);
  s->dt = dt;
  s->svica = ((0.666) * (1.2) * (p->ica_scale)); /* :96 */
  s->svncx = (2.5 * p->ncx_scale);               /* :109 */
  double sviup = SV_IUP;                         /* :1205, :1230-1238 */
  if (p->iso2) sviup = SV_IUP * 1.75;
  if (p->tapsi) sviup = 0;
  double sviup_lqt = (p->lqt && p->tapsi) ? 0.05 : 0.; /* :121-125, :135 */
  s->sviup_tot = sviup + sviup_lqt;
  /* the iso block sets sv_iup*2 from 5.5 PCL on, then iso2 and tapsi
   * override it as before (:1219-1238) */
  double sviup_iso = SV_IUP * 2.;
  if (p->iso2) sviup_iso = SV_IUP * 1.75;
  if (p->tapsi) sviup_iso = 0;
  s->sviup_iso = sviup_iso + sviup_lqt;
  s->svikr = p->lqt ? 0 : 3 * p->ikr_scale; /* :128, :138 */
  s->cao = p->cao_mM;
  s->tend = p->nbeats * p->pcl_ms + 2100; /* :399 */
  int jz = p->linescan_jz < 0 ? 5 : p->linescan_jz;
  if (jz > p->nz - 2) jz = p->nz / 2;
  if (jz < 1) jz = 1;
  s->jz_line = jz;
  size_t n1 = (size_t)s->ntot, n8 = n1 * 8;
#define ALLOC(ptr, cnt) ptr = calloc((cnt), sizeof(*(ptr)))
  ALLOC(s->cp, n1); ALLOC(s->cjsr, n1); ALLOC(s->cjsrb, n1); ALLOC(s->ancx, n1);
  ALLOC(s->xire, n1); ALLOC(s->po, n1); ALLOC(s->xinaca, n1); ALLOC(s->xicat, n1);
  ALLOC(s->casar, n1); ALLOC(s->casarh, n1); ALLOC(s->casarj, n1); ALLOC(s->casarhj, n1);
  ALLOC(s->lcc, n8); ALLOC(s->nl, n1); ALLOC(s->nou, n1); ALLOC(s->ncu, n1);
  ALLOC(s->nob, n1); ALLOC(s->ncb, n1); ALLOC(s->nspark, n1);
  ALLOC(s->xiup, n8); ALLOC(s->xileak, n8); ALLOC(s->catf, n8); ALLOC(s->cats, n8);
  ALLOC(s->cacal, n8); ALLOC(s->casr, n8); ALLOC(s->camyo, n8); ALLOC(s->mgmyo, n8);
  ALLOC(s->cadye, n8);
  ALLOC(s->ci[0], n8); ALLOC(s->ci[1], n8); ALLOC(s->cnsr[0], n8); ALLOC(s->cnsr[1], n8);
  ALLOC(s->cs[0], n1); ALLOC(s->cs[1], n1);
  ALLOC(s->ls, (size_t)(p->nx - 2) * RH_LINESCAN_COLS);
  ALLOC(s->cd, 2 + (size_t)s->nin * 6);
#undef ALLOC
  if (!s->ls || !s->cs[1] || !s->cd) {
    orc_destroy(s);
    return NULL;
  }
  init_lattice(s);
  /* host initial conditions (:346-365) */
  rh_membrane* m = &s->m;
  memset(m, 0, sizeof(*m));
  m->t = 0.0;
  m->xnai = 6.1 * ((9000) / (p->pcl_ms + 5000));
  m->v = -80.00;
  m->xm = 0.0010;
  m->xh = 1.00;
  m->xj = 1.00;
  m->xr = 0.00;
  m->xs1 = 0.08433669901;
  m->xs2 = m->xs1;
  m->qks = 0.20;
  m->xtos = 0.010;
  m->ytos = 1.00;
  m->xtof = 0.020;
  m->ytof = 0.80;
  return s;
}

void orc_destroy(orc_sim* s) {
  if (!s) return;
  double* dp[] = {s->cp, s->cjsr, s->cjsrb, s->ancx, s->xire, s->po, s->xinaca, s->xicat,
                  s->casar, s->casarh, s->casarj, s->casarhj, s->xiup, s->xileak, s->catf,
                  s->cats, s->cacal, s->casr, s->camyo, s->mgmyo, s->cadye, s->ci[0], s->ci[1],
                  s->cnsr[0], s->cnsr[1], s->cs[0], s->cs[1], s->ls, s->cd};
  for (size_t q = 0; q < sizeof(dp) / sizeof(dp[0]); ++q) free(dp[q]);
  free(s->apv);
  int* ip[] = {s->lcc, s->nl, s->nou, s->ncu, s->nob, s->ncb, s->nspark};
  for (size_t q = 0; q < sizeof(ip) / sizeof(ip[0]); ++q) free(ip[q]);
  free(s);
}

/* ---------------------------- state exchange ----------------------------- */

void orc_get_state(const orc_sim* s, rh_state_f64* d) {
  const int lx = s->nx - 2, ly = s->ny - 2, lz = s->nz - 2, n = lx * ly * lz;
  const double* ci = s->ci[s->cur];
  const double* cn = s->cnsr[s->cur];
  const double* cs = s->cs[s->cur];
  for (int q = 0; q < n; ++q) {
    int ac = opos(s, 1 + q % lx, 1 + (q / lx) % ly, 1 + q / (lx * ly));
#define PUT(f, src) if (d->f) d->f[q] = src
    PUT(cp, s->cp[ac]); PUT(cs, cs[ac]); PUT(cjsr, s->cjsr[ac]); PUT(cjsrb, s->cjsrb[ac]);
    PUT(ancx, s->ancx[ac]); PUT(casar, s->casar[ac]); PUT(casarh, s->casarh[ac]);
    PUT(casarj, s->casarj[ac]); PUT(casarhj, s->casarhj[ac]);
    PUT(nou, s->nou[ac]); PUT(ncu, s->ncu[ac]); PUT(nob, s->nob[ac]); PUT(ncb, s->ncb[ac]);
    PUT(nl, s->nl[ac]); PUT(nspark, s->nspark[ac]);
    PUT(xire, s->xire[ac]); PUT(po, s->po[ac]); PUT(xinaca, s->xinaca[ac]);
    PUT(xicat, s->xicat[ac]);
#undef PUT
    for (int ii = 0; ii < 8; ++ii) {
      int a8 = ac * 8 + ii;
      size_t o = (size_t)ii * n + q;
#define PUT8(f, src) if (d->f) d->f[o] = src
      PUT8(ci, ci[a8]); PUT8(cnsr, cn[a8]); PUT8(catf, s->catf[a8]); PUT8(cats, s->cats[a8]);
      PUT8(cacal, s->cacal[a8]); PUT8(casr, s->casr[a8]); PUT8(camyo, s->camyo[a8]);
      PUT8(mgmyo, s->mgmyo[a8]); PUT8(lcc, s->lcc[ac * 8 + ii]); PUT8(xiup, s->xiup[a8]);
      PUT8(xileak, s->xileak[a8]);
#undef PUT8
    }
  }
}

void orc_set_state(orc_sim* s, const rh_state_f64* d) {
  const int lx = s->nx - 2, ly = s->ny - 2, lz = s->nz - 2, n = lx * ly * lz;
  double* ci = s->ci[s->cur];
  double* cn = s->cnsr[s->cur];
  double* cs = s->cs[s->cur];
  for (int q = 0; q < n; ++q) {
    int ac = opos(s, 1 + q % lx, 1 + (q / lx) % ly, 1 + q / (lx * ly));
#define GET(f, dst) if (d->f) dst = d->f[q]
    GET(cp, s->cp[ac]); GET(cs, cs[ac]); GET(cjsr, s->cjsr[ac]); GET(cjsrb, s->cjsrb[ac]);
    GET(ancx, s->ancx[ac]); GET(casar, s->casar[ac]); GET(casarh, s->casarh[ac]);
    GET(casarj, s->casarj[ac]); GET(casarhj, s->casarhj[ac]);
    GET(nou, s->nou[ac]); GET(ncu, s->ncu[ac]); GET(nob, s->nob[ac]); GET(ncb, s->ncb[ac]);
    GET(nl, s->nl[ac]); GET(nspark, s->nspark[ac]);
#undef GET
    for (int ii = 0; ii < 8; ++ii) {
      int a8 = ac * 8 + ii;
      size_t o = (size_t)ii * n + q;
#define GET8(f, dst) if (d->f) dst = d->f[o]
      GET8(ci, ci[a8]); GET8(cnsr, cn[a8]); GET8(catf, s->catf[a8]); GET8(cats, s->cats[a8]);
      GET8(cacal, s->cacal[a8]); GET8(casr, s->casr[a8]); GET8(camyo, s->camyo[a8]);
      GET8(mgmyo, s->mgmyo[a8]); GET8(lcc, s->lcc[ac * 8 + ii]);
#undef GET8
    }
  }
  /* ghost faces consistent with the imported interior (what the reference's
   * end-of-step copy would have left) */
  s->cur = 1 - s->cur;
  apply_ghost_faces(s);
  s->cur = 1 - s->cur;
}

void orc_get_membrane(const orc_sim* s, rh_membrane* d) { *d = s->m; }
void orc_set_membrane(orc_sim* s, const rh_membrane* d) { s->m = *d; }

void orc_last_wholecell(const orc_sim* s, double* cols45) {
  memcpy(cols45, s->wc, sizeof(s->wc));
}

int32_t orc_last_linescan(const orc_sim* s, double* rows) {
  if (rows) memcpy(rows, s->ls, sizeof(double) * (s->nx - 2) * RH_LINESCAN_COLS);
  return s->nx - 2;
}

int32_t orc_last_cadist(const orc_sim* s, double* rec) {
  if (!s->cd_valid) return 0;
  if (rec) memcpy(rec, s->cd, sizeof(double) * (2 + (size_t)s->nin * 6));
  return s->nin;
}

uint32_t orc_status(const orc_sim* s) { return s->status; }
int32_t orc_interior(const orc_sim* s) { return s->nin; }

/* --------------------------- output formatting --------------------------- */

int orc_format_wholecell(const double* c, char* buf, size_t n) {
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

int orc_format_linescan(const double* c, char* buf, size_t n) {
  return snprintf(buf, n,
                  "%f %f %f %i %i "
                  "%i %i %i %f %f "
                  "%f %f %f %f %f "
                  "%f %f %f %f %f "
                  "%f %f\n",
                  c[0], c[1], c[2], (int)c[3], (int)c[4], (int)c[5], (int)c[6], (int)c[7], c[8],
                  c[9], c[10], c[11], c[12], c[13], c[14], c[15], c[16], c[17], c[18], c[19],
                  c[20], c[21]);
}
