// model.cuh — device physics of one CRU time step, templated on the real type
// R (double for the FP64 path, float for the mixed path).
//
// Physics follows the reference (subroutine_cuda.c, reesica.h, buffers.c and
// the Compute kernel of cuda_Cell_Detailed.cu); the line citations are on each
// function.  Arithmetic is arranged for sm_103a rather than copied: constant
// divisors become reciprocal multiplies, pow(x, 23) is a product chain,
// pow(x, 1.787) is exp(1.787 log x), and every quantity that depends only on
// the membrane voltage is computed once per cell and step (StepCoef), not per
// CRU or per channel.
#pragma once

#include <limits.h>
#include <stdint.h>

#include "../../include/rh_philox.h"

namespace rh {

// ---- constants (cuda_Cell_Detailed.cu:63-145, subroutine_cuda.c:7-39,
//      buffers.c:16-52); same expressions, folded at compile time ----
constexpr double OUTT = 2.5;
constexpr double PI_TRUNC = 3.1415926;  // :65 (truncated pi of Box-Muller)
constexpr double VP = 0.00126;
constexpr double VJSR = (0.02 * 1);
constexpr double VI = (0.5 / 8.);
constexpr double VNSR = (0.025 / 8.);
constexpr int NRYR = 100;
constexpr double TAUPS = 0.0283;
constexpr double TAUPI = 0.1;
constexpr double TAUSI = 0.04;
constexpr double TAUTR = (25.0 * 1.0 / 4.);
constexpr double TAUNL = 6.;
constexpr double TAUNT = 1.8;
constexpr double TAUIL = (0.7 * 2.);
constexpr double TAUIT = (0.33 * 2.);
constexpr double TAUST = 1.42;
constexpr double FRT = (96.485 / 8.314 / 308.0);
constexpr double XI = 0.7;
constexpr double CI_BASAL = 0.0944;
// permeabilised cell (-Dperm, :87-89): basal [Ca]i held at the lattice faces
// and in the submembrane leak; initial JSR/NSR load
constexpr double PERM_CI_BASAL = 0.3;
constexpr double PERM_CJSR_BASAL = 900;
constexpr double VS = 0.025;
constexpr double ICAGAMMA = 0.5;
constexpr double CM = 45;
constexpr double TAUU = (0.2 * 5 * 220.);
constexpr double TAUB = 1.0;
constexpr double XNAO = 140.0;
constexpr double SVJMAX = 11.5;
// NCX / CSQN / LCC
constexpr double VNACA = (21.0 / 1.0);
constexpr double KMCAI = 0.00359;
constexpr double KMCAO = 1.3;
constexpr double KMNAI = 12.3;
constexpr double KMNAO = 87.5;
constexpr double KSAT = 0.27;
constexpr double ETA = 0.35;
constexpr double KDA = 0.0003;  // mM, Ka of oldncx and ncx_noallo (subroutine_cuda.c:12)
// oldncx allosteric on/off rates (subroutine_cuda.c:79-80)
constexpr double KNCXOFF_OLD = 0.00005;
constexpr double KNCXON_OLD = 2.53e-3 * 0.05;
// slowncxchange background current, cuda_Cell_Detailed.cu:1268:
//   bcgcur = BCG_G * (v - log(180000 / cs) / 2 / frt)
constexpr double BCG_G = 1.0 * 0.003016 / 32.;
constexpr double FARAD = 96.485;
constexpr double XRGAS = 8.314;
constexpr double TEMPER = 308;
constexpr double NM = 20;
constexpr double ND = 30;
constexpr double RATEDIMER = 5000.0;
constexpr double KDIMER = 850.0;
constexpr double HILLDIMER = 23.0;
constexpr double CSQBERS = 460.0;
constexpr double KBERS = 600.0;
constexpr double PCA = 11.9;
constexpr double GAMMAI = 0.341;
// buffers
constexpr double KTSON = 0.00254, KTSOFF = 0.000033, BTS = 134.;
constexpr double KTFON = 0.0327, KTFOFF = 0.0196, BTF = 70.;
constexpr double KCALON = 0.0543, KCALOFF = 0.238, BCAL = 24.;
constexpr double KSRON = 0.1, KSROFF = 0.06, BSR = 19.;
constexpr double KSARON = 0.1, KSAROFF = 1.3, BSAR = (42 * (VI * 8.0 / VS));
constexpr double KSARHON = 0.1, KSARHOFF = 0.03, BSARH = (15. * (VI * 8.0 / VS));
constexpr double BMYO = 140;
constexpr double KONMYOMG = 0.0157, KOFFMYOMG = 0.057;
constexpr double KONMYOCA = 13.8, KOFFMYOCA = 0.46;
constexpr double MGI = 500;
// SERCA / leak (subroutine_cuda.c:128-146)
constexpr double VUP = 0.3, KI_UP = 0.123, KNSR_UP = 1700.0, HH_UP = 1.787;
constexpr double GLEAK = 0.00001035, KJSR_LEAK = 500.0;

// ---- math of each precision ----
template <class R>
struct Math;

template <>
struct Math<double> {
  static __device__ __forceinline__ double exp(double x) { return ::exp(x); }
  static __device__ __forceinline__ double log(double x) { return ::log(x); }
  static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
  static __device__ __forceinline__ double cos(double x) { return ::cos(x); }
  static __device__ __forceinline__ double floor(double x) { return ::floor(x); }
  // x^y for x >= 0: exp(y log x) keeps ~1e-15 relative error here (|y log x| < 20)
  static __device__ __forceinline__ double powpos(double x, double y) {
    return ::exp(y * ::log(x));
  }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ int to_int(double x) { return __double2int_rz(x); }
  static __device__ __forceinline__ double uniform(rh_stream* s) { return rh_uniform_double(s); }
  static constexpr double TINY_UNIFORM = 0x1.0p-53;
};

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// FP32: the SFU forms (ex2/lg2/cos approximations, reciprocal division).
// Their relative errors (~1e-6 for the arguments met here) stay well inside
// the mixed path's 1e-5 single-step tolerance.
template <>
struct Math<float> {
  static __device__ __forceinline__ float exp(float x) { return __expf(x); }
  static __device__ __forceinline__ float log(float x) { return __logf(x); }
  static __device__ __forceinline__ float sqrt(float x) { return ::sqrtf(x); }
  static __device__ __forceinline__ float cos(float x) { return __cosf(x); }
  static __device__ __forceinline__ float floor(float x) { return ::floorf(x); }
  static __device__ __forceinline__ float powpos(float x, float y) {
    return ex2_approx(y * __log2f(x));
  }
  static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
  static __device__ __forceinline__ int to_int(float x) { return __float2int_rz(x); }
  static __device__ __forceinline__ float uniform(rh_stream* s) { return rh_uniform_float(s); }
  static constexpr float TINY_UNIFORM = 0x1.0p-24f;
};

// ---- z-pairs of sub-voxels: (lower, upper) half of a CRU in z, handled as
//      one 2-vector.  FP32 pairs use Blackwell's packed FP32x2 instructions
//      (add/mul/fma .f32x2); FP64 pairs are plain component-wise code. ----
template <class R>
struct Vec2;
template <>
struct Vec2<float> {
  using T = float2;
};
template <>
struct Vec2<double> {
  using T = double2;
};

__device__ __forceinline__ float2 v2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 v2(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 splat2(float a) { return make_float2(a, a); }
__device__ __forceinline__ double2 splat2(double a) { return make_double2(a, a); }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 vmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as fma(b, -1, a): exact product, one rounding, one packed instruction
__device__ __forceinline__ float2 vsub(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}
__device__ __forceinline__ double2 vadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 vmul(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ double2 vfma(double2 a, double2 b, double2 c) {
  return make_double2(a.x * b.x + c.x, a.y * b.y + c.y);
}
__device__ __forceinline__ double2 vsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// x < 0 ? 0 : x, NaN staying NaN.  In FP32 one max.NaN instruction (its
// max(-0, +0) is +0 where the comparison keeps -0, which no later FP32 result
// tells apart); in FP64 the comparison itself, as the oracle has it.
__device__ __forceinline__ float clamp0(float x) {
  float r;
  asm("max.NaN.f32 %0, %1, 0f00000000;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ double clamp0(double x) { return x < 0.0 ? 0.0 : x; }
template <class V>
__device__ __forceinline__ V vclamp0(V a) {
  a.x = clamp0(a.x);
  a.y = clamp0(a.y);
  return a;
}

// SERCA's (x / K)^1.787 for x >= 0 (subroutine_cuda.c:128-146), K = KI_UP
// for the cytosol (SIDE 0) and KNSR_UP for the network SR (SIDE 1).  FP64 as
// exp(1.787 log(x / K)); FP32 as ex2(1.787 lg2(x) - 1.787 lg2(K)), the
// division folded into the constant (lg2(0.123) = -3.0232697793228470,
// lg2(1700) = 10.731319031025064).
template <int SIDE>
__device__ __forceinline__ double serca_pow(double x) {
  return Math<double>::powpos(x * (1.0 / (SIDE ? KNSR_UP : KI_UP)), HH_UP);
}
template <int SIDE>
__device__ __forceinline__ float serca_pow(float x) {
  constexpr double lg2k = SIDE ? 10.731319031025064 : -3.0232697793228470;
  return ex2_approx(fmaf((float)HH_UP, __log2f(x), (float)(-HH_UP * lg2k)));
}

template <class R>
__device__ __forceinline__ R pow23(R x) {  // x^23 = x^16 x^4 x^2 x
  R x2 = x * x, x4 = x2 * x2, x8 = x4 * x4, x16 = x8 * x8;
  return x16 * x4 * x2 * x;
}

// ---- buffers (buffers.c:55-155) ----

// Mass-action rate with the reference's saturation guard kon*c*dt > 1, which
// replaces the on-rate kon*c by 0.95/dt: the guard selects the factor, one
// expression computes the rate.
template <class R>
__device__ __forceinline__ R buffer_rate(R kon, R koff, R total, R bound, R c, R dt, R rdt95) {
  R on = kon * c;
  on = (on * dt > R(1)) ? rdt95 : on;
  return on * (total - bound) - koff * bound;
}

// ---- CSQN (subroutine_cuda.c:161-195) ----

// Dimerisation fraction shared by luminal(), luminal_SS() and ryrgating().
// FP64 keeps the reference's form (-1 + sqrt(1+z))/(z/2), z = 8 C roo2,
// including its collapse to 0 when 1+z rounds to 1.  FP32 uses the
// rationalised form 2/(1+sqrt(1+z)), which is stable, and reproduces the FP64
// collapse for z < 2^-53.
template <class R>
__device__ __forceinline__ void csqn_mono(R cjsr, R& roo2, R& mono);

template <>
__device__ __forceinline__ void csqn_mono<double>(double cjsr, double& roo2, double& mono) {
  roo2 = RATEDIMER / (1.0 + pow23(KDIMER / cjsr));
  mono = (-1.0 + ::sqrt(1.0 + 8.0 * CSQBERS * roo2)) / (4.0 * roo2 * CSQBERS);
}

template <>
__device__ __forceinline__ void csqn_mono<float>(float cjsr, float& roo2, float& mono) {
  roo2 = __fdividef(float(RATEDIMER), 1.0f + pow23(__fdividef(float(KDIMER), cjsr)));
  float z = float(8.0 * CSQBERS) * roo2;
  mono = (z < 0x1.0p-53f) ? 0.0f : __fdividef(2.0f, 1.0f + ::sqrtf(1.0f + z));
}

// luminal buffering factor beta(cjsr) (subroutine_cuda.c:161-177)
template <class R>
__device__ __forceinline__ R csqn_beta(R cjsr, R roo2, R mono) {
  R ene = mono * R(NM) + (R(1) - mono) * R(ND);
  R enedot = R(NM - ND) * (-mono + Math<R>::div(R(1), R(4.0 * CSQBERS) * mono * roo2 + R(1))) *
             Math<R>::div(R(HILLDIMER), cjsr) * (R(1) - roo2 * R(1.0 / RATEDIMER));
  R kc = R(KBERS) + cjsr;
  return Math<R>::div(R(1), R(1) + Math<R>::div(R(CSQBERS * KBERS) * ene +
                                                    R(CSQBERS) * enedot * cjsr * kc,
                                                kc * kc));
}

// ---- per-cell coefficients of one lattice update: everything that depends
//      only on the membrane voltage, [Na]i, time and the cell's parameters,
//      computed once per cell and step in FP64 and stored in the kernel's
//      precision R ----
template <class R>
struct StepCoef {
  // LCC gates (reesica.h:21-63): c, d and f rates are voltage-only
  R alphac, betac, alphad, betad, alphaf, betaf;
  // ICaL GHK (subroutine_cuda.c:231-247): ica = lcc_k * (cpx*lcc_e2z_k - cao)
  R lcc_e2z_k, lcc_k;
  // NCX (subroutine_cuda.c:47-75) with za and [Na]i fixed:
  //   Inaca = Ka * (num_a - num_b cs) / ((t1 + t2(cs) + t3a + cs XNAO^3) den2)
  // t2 = KMNAO^3 cs (1 + cs/KMCAI), or in oldncx/ncx_noallo
  // KMNAO^3 cs + ncx_t2b (1 + cs/KMCAI) with ncx_t2b = KMNAI^3 Cext (:91, :116)
  R ncx_num_a, ncx_num_b, ncx_t1, ncx_t3a, ncx_den2, ncx_t2b;
  // slowncxchange background current: bcgcur = bcg_a - bcg_b log(180000/cs)
  R bcg_a, bcg_b;
  // cell parameters
  R svica, svncx, sviup, cao, ku, ku2, kb;
  // time step constants
  R dt, rdt, dth, rdt95, rdth95;
  int reset_window;  // fmod(t-dt, outt) < dt (cuda_Cell_Detailed.cu:1244)
  int output_step;   // fmod(t+1e-7, outt) < dt (:777)
  int cadist_step;   // output step that also writes a cadist record (:1002)
  int perm;          // permeabilised cell: no LCC/NCX, [Ca] faces held (-Dperm)
  int ncx_form;      // RH_NCX_*
  int ncx_ka_hill;   // ncx_noallo below -75 mV: Ka = 1/(1+(Kda/cs)^3), else 1 (:110-112)
  int slowncx;       // slowncxchange: bcgcur on, allosteric Ka = 5 Ancx
  int iso_add_lcc;   // iso: fill the empty LCC slots 4-7 this step (:1213-1218)
};

template <class R, class Q>
__host__ __device__ inline void convert_coef(StepCoef<R>& d, const StepCoef<Q>& s) {
  d.alphac = R(s.alphac); d.betac = R(s.betac); d.alphad = R(s.alphad); d.betad = R(s.betad);
  d.alphaf = R(s.alphaf); d.betaf = R(s.betaf); d.lcc_e2z_k = R(s.lcc_e2z_k); d.lcc_k = R(s.lcc_k);
  d.ncx_num_a = R(s.ncx_num_a); d.ncx_num_b = R(s.ncx_num_b); d.ncx_t1 = R(s.ncx_t1);
  d.ncx_t3a = R(s.ncx_t3a); d.ncx_den2 = R(s.ncx_den2); d.ncx_t2b = R(s.ncx_t2b);
  d.bcg_a = R(s.bcg_a); d.bcg_b = R(s.bcg_b); d.svica = R(s.svica); d.svncx = R(s.svncx);
  d.sviup = R(s.sviup); d.cao = R(s.cao); d.ku = R(s.ku); d.ku2 = R(s.ku2); d.kb = R(s.kb);
  d.dt = R(s.dt); d.rdt = R(s.rdt); d.dth = R(s.dth); d.rdt95 = R(s.rdt95); d.rdth95 = R(s.rdth95);
  d.reset_window = s.reset_window;
  d.output_step = s.output_step;
  d.cadist_step = s.cadist_step;
  d.perm = s.perm;
  d.ncx_form = s.ncx_form;
  d.ncx_ka_hill = s.ncx_ka_hill;
  d.slowncx = s.slowncx;
  d.iso_add_lcc = s.iso_add_lcc;
}

// ---- RyR transition draw (subroutine_cuda.c:332-363 and siblings) ----
template <class R>
__device__ __forceinline__ int ryr_transition(rh_stream* rng, int n, R p, R lam,
                                              uint32_t* status) {
  int kk = 0;
  if (n <= 1 || p < R(0.2) || (n <= 5 && p < R(0.3))) {
    R puu = R(1);
    while (puu >= lam && kk < 195) {
      ++kk;
      puu = puu * Math<R>::uniform(rng);
    }
    return kk - 1;
  }
  int m = -1;
  const R np = R(n) * p;
  const R sd = Math<R>::sqrt(np * (R(1) - p));
  while (m < 0) {
    R u1 = Math<R>::uniform(rng);
    R u2 = Math<R>::uniform(rng);
    uint32_t bit = rh_uniform_u32(rng);
    R om = R(1) - u1;
    if (!(om > R(0))) om = Math<R>::TINY_UNIFORM;  // u1 == 1: log(0) in the reference
    R g = sd * Math<R>::sqrt(R(-2) * Math<R>::log(om)) * Math<R>::cos(R(2.0 * PI_TRUNC) * u2);
    R xm = Math<R>::floor(np + g) + R(bit % 2u);
    // p > 1 makes the variance negative and the draw NaN; it converts to a
    // negative count (as the hardware conversion does), so the draw repeats
    // until the 200-try cap; out-of-range values saturate
    if (xm != xm) {
      *status |= 0x10u;  // RH_STATUS_RATE_CAP
      m = INT_MIN;
    } else {
      m = Math<R>::to_int(xm);
    }
    ++kk;
    if (kk > 200) {
      m = 0;
      *status |= 0x2u;  // RH_STATUS_GAUSS_RETRY
    }
  }
  return m;
}

// Four-state RyR cluster step (subroutine_cuda.c:251-669).  roo2/mono come
// from csqn_mono (the same expression the reference evaluates at :328-329).
// The eight transitions run in source order (so do their draws), unrolled:
// each transition's count and rates are then fixed at compile time, which
// measured 1% faster than the rolled loop despite the larger code; each count
// is packed into a byte (counts are <= 195 before clamping).
template <class R>
__device__ __forceinline__ void ryr_gating(rh_stream* rng, const StepCoef<R>& k, R cp, R cjsr,
                                           R mono, int& ncu, int& nou, int& ncb, int& nob,
                                           uint32_t* status) {
  const R dt = k.dt;
  R q = Math<R>::div(R(5000), cjsr);
  R a = Math<R>::div(k.ku, cp);
  R common = Math<R>::div(R(1), (R(1) + q * q) * (R(1) + a * a));
  R pku = R(4.5 * 1.5) * k.ku2 * common;
  R pkb = R(4.5 * 1.5 / 36.) * k.kb * common;
  R pkuminus = R(1);  // 1/taucu
  R pkbminus = R(1);  // 1/taucb
  if (pku * dt > R(1)) pku = k.rdt;
  if (pkb * dt > R(1)) pkb = k.rdt;
  if (pkuminus * dt > R(1)) pkuminus = k.rdt;
  if (pkbminus * dt > R(1)) pkbminus = k.rdt;
  const R aub = mono * R(1.0 / TAUB);
  const R abu = R(1.0 / TAUU);
  const int nou0 = nou, ncu0 = ncu, nob0 = nob, ncb0 = ncb;
  const R pbu = (pkb < R(1e-16)) ? abu * dt * R(36) : abu * dt * Math<R>::div(pku, pkb);
  const R pau = (pkb < R(1e-16)) ? R(0) : aub * dt;
  uint32_t packed0 = 0u, packed1 = 0u;
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    int n;
    R p;
    switch (t) {
      case 0: n = nou0; p = pkuminus * dt; break;  // OU -> CU (:332-364)
      case 1: n = ncu0; p = pku * dt; break;       // CU -> OU (:366-397)
      case 2: n = nou0; p = pau; break;            // OU -> OB (:401-436)
      case 3: n = nob0; p = pbu; break;            // OB -> OU (:439-476)
      case 4: n = ncb0; p = abu * dt; break;       // CB -> CU (:480-511)
      case 5: n = ncu0; p = aub * dt; break;       // CU -> CB (:513-544)
      case 6: n = nob0; p = pkbminus * dt; break;  // OB -> CB (:548-579)
      default: n = ncb0; p = pkb * dt; break;      // CB -> OB (:581-613)
    }
    int r = ryr_transition<R>(rng, n, p, Math<R>::exp(-R(n) * p), status);
    if (t != 6) r = min(r, NRYR);  // the reference does not cap OB -> CB
    r = min(r, 255);
    if (t < 4) packed0 |= (uint32_t)r << (t * 8);
    else packed1 |= (uint32_t)r << ((t - 4) * 8);
  }
  int n_ou_cu = packed0 & 0xff, n_cu_ou = (packed0 >> 8) & 0xff;
  int n_ou_ob = (packed0 >> 16) & 0xff, n_ob_ou = packed0 >> 24;
  int n_cb_cu = packed1 & 0xff, n_cu_cb = (packed1 >> 8) & 0xff;
  int n_ob_cb = (packed1 >> 16) & 0xff, n_cb_ob = packed1 >> 24;

  // conflict resolution (:617-639)
  if (n_ou_ob + n_ou_cu > nou0) {
    if (n_ou_cu >= n_ou_ob) n_ou_cu = 0;
    else n_ou_ob = 0;
    if (n_ou_ob > nou0) n_ou_ob = 0;
    else if (n_ou_cu > nou0) n_ou_cu = 0;
  }
  if (n_ob_ou + n_ob_cb > nob0) {
    if (n_ob_ou >= n_ob_cb) n_ob_ou = 0;
    else n_ob_cb = 0;
    if (n_ob_cb > nob0) n_ob_cb = 0;
    else if (n_ob_ou > nob0) n_ob_ou = 0;
  }
  if (n_cu_ou + n_cu_cb > ncu0) {
    if (n_cu_cb >= n_cu_ou) n_cu_cb = 0;
    else n_cu_ou = 0;
    if (n_cu_ou > ncu0) n_cu_ou = 0;
    else if (n_cu_cb > ncu0) n_cu_cb = 0;
  }
  // updates and clamps (:642-665)
  nou = min(max(nou0 - n_ou_ob - n_ou_cu + n_ob_ou + n_cu_ou, 0), NRYR);
  nob = min(max(nob0 - n_ob_ou - n_ob_cb + n_ou_ob + n_cb_ob, 0), NRYR);
  ncu = min(max(ncu0 - n_cu_ou - n_cu_cb + n_ou_cu + n_cb_cu, 0), NRYR);
  ncb = min(max(NRYR - nou - nob - ncu, 0), NRYR);
}

// One LCC slot (reesica.h:65-115): a single uniform picks at most one gate
// flip by first passage over the cumulative rates.
// Gate b flips from open to closed (st - 2^b) or back (st + 2^b), i.e.
// st ^ 2^b.  The comparisons keep the reference's order and its running
// subtraction, so the chosen gate is the same; they are evaluated without
// branches, which keeps the warp's lanes together.
template <class R>
__device__ __forceinline__ int lcc_next(int st, R rig, R ac, R bc, R ad, R bd, R af, R bf,
                                        R afca, R bfca) {
  const R r0 = (st & 1) ? ac : bc;
  const R r1 = (st & 2) ? ad : bd;
  const R r2 = (st & 4) ? af : bf;
  const R r3 = (st & 8) ? afca : bfca;
  const R g1 = rig - r0, g2 = g1 - r1, g3 = g2 - r2;
  const int flip = rig < r0 ? 1 : g1 < r1 ? 2 : g2 < r2 ? 4 : g3 < r3 ? 8 : 0;
  return st ^ flip;
}

}  // namespace rh
