// step.cu — the fused per-time-step kernel.
//
// One launch advances every active cell by one time step:
//   1. each CTA updates a tile of up to kBlock CRUs of one cell (the
//      reference's Compute kernel, cuda_Cell_Detailed.cu:1187-1692, fixA),
//      reading the previous ci/cnsr/cs buffers and writing the next ones;
//   2. the CTA reduces sum(cs), sum(xicat), sum(xinaca) (and at output steps
//      the ~30 statistics of :839-929) with warp shuffles, compensated, and
//      stores one partial per tile;
//   3. the last CTA of a cell to finish (atomic arrival counter) sums the
//      cell's partials in a fixed order, runs the membrane model and V update
//      (:430-739, the reference's host loop), writes the output record at
//      output steps, and prepares the voltage coefficients of the next step.
// So the per-step device-to-host copies and host loop of the reference
// (:427-456) disappear; a step is one kernel launch.
#include <cuda_runtime.h>
#include <stdint.h>

#include "cellmodel.cuh"
#include "lattice.cuh"
#include "model.cuh"
#include "step.cuh"

namespace rh {

// ---------------------------------------------------------------- reductions

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Compensated warp sum of one value per lane; returns (sum, comp) in lane 0.
__device__ __forceinline__ void warp_sum_comp(double v, double& s, double& c) {
  s = v;
  c = 0.0;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    double so = __shfl_down_sync(0xffffffffu, s, off);
    double co = __shfl_down_sync(0xffffffffu, c, off);
    double e;
    two_sum(s, so, s, e);
    c = c + co + e;
  }
}

// Same for float lane values: error-free in FP32, widened to FP64 at the end.
__device__ __forceinline__ void warp_sum_comp(float v, double& s, double& c) {
  float fs = v, fc = 0.0f;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    float so = __shfl_down_sync(0xffffffffu, fs, off);
    float co = __shfl_down_sync(0xffffffffu, fc, off);
    float e;
    two_sum_f(fs, so, fs, e);
    fc = fc + co + e;
  }
  s = (double)fs;
  c = (double)fc;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}

template <class R>
__device__ __forceinline__ R clamp0(R x) {
  return x < R(0) ? R(0) : x;
}

// ------------------------------------------------------------ cell update

// Whole-cell part of the step, run by warp 0 of the last CTA of the cell.
template <class R>
__device__ void cell_update(const StepArgs<R>& a, int cell, const CellConst& cc, bool out_step) {
  const int lane = threadIdx.x & 31;
  CellDyn* dyn = a.dyn + cell;
  const double* P = a.partials;
  const int t0 = cc.tile_begin, nt = cc.tile_count;
  // fixed-order sums over the cell's tiles: lane l takes tiles l, l+32, ...
  double tot[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    double s = 0.0, c = 0.0;
    for (int tl = lane; tl < nt; tl += 32) {
      const double* p = P + (size_t)(t0 + tl) * P_COUNT + 2 * q;
      double e;
      two_sum(s, __ldcg(p), s, e);
      c += e + __ldcg(p + 1);
    }
    double ws, wc;
    warp_sum_comp(s, ws, wc);
    double wc2 = warp_sum(c);
    tot[q] = ws + (wc + wc2);
  }
  double osum[NOUT];
  if (out_step) {
    for (int q = 0; q < NOUT; ++q) {
      double s = 0.0;
      for (int tl = lane; tl < nt; tl += 32) s += __ldcg(P + (size_t)(t0 + tl) * P_COUNT + P_STEP_END + q);
      s = warp_sum(s);
      osum[q] = s;
    }
    // the ci>1000 flag is a max, not a sum
    double f = 0.0;
    for (int tl = lane; tl < nt; tl += 32) f = fmax(f, __ldcg(P + (size_t)(t0 + tl) * P_COUNT + O_CIHIGH));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) f = fmax(f, __shfl_down_sync(0xffffffffu, f, off));
    osum[O_CIHIGH - P_STEP_END] = f;
  }
  if (lane != 0) return;
  rh_membrane m = dyn->m;
  const double dt = a.dt;
  // reduction (:447-456)
  m.csubt = tot[0] / cc.n;
  m.xicatto = tot[1] / CM * 0.0965 * VP * 2.0 * (ICAGAMMA + 1.);
  m.xinacato = tot[2] / CM * 0.0965 * VS;
  membrane_update(m, dt, cc.pcl, cc.svikr);
  uint32_t status = dyn->status;
  if (!isfinite(m.v) || !isfinite(m.xnai) || !isfinite(m.csubt) || !isfinite(m.xicatto) ||
      !isfinite(m.xinacato))
    status |= RH_STATUS_NAN;
  if (out_step) {
    m.sparksum += (long long)osum[O_SPARK - P_STEP_END];
    if (osum[O_CIHIGH - P_STEP_END] > 0) status |= RH_STATUS_CI_HIGH;
    long long slot = dyn->out_count % a.out_cap;
    double* w = a.out_wc + ((size_t)cell * a.out_cap + slot) * RH_WHOLECELL_COLS;
    wholecell_columns(w, osum, m, cc.n, dt);
    dyn->out_count += 1;
    m.sparksum = 0;  // :1074-1077
    m.out_ica = 0;
    m.out_ncx = 0;
    m.out_ina = 0;
  }
  m.t = m.t + dt;  // :1083
  m.step += 1;
  VoltCoef vc;
  volt_coef(vc, m, cc, dt);
  if (!vc.active) {
    dyn->done = 1;
    status |= RH_STATUS_DONE;
  }
  dyn->m = m;
  dyn->vc = vc;
  dyn->status = status;
}

// ------------------------------------------------------------- step kernel

template <class R, bool OUT>
__global__ void __launch_bounds__(kBlock) step_kernel(StepArgs<R> a) {
  __shared__ CellConst sc;
  __shared__ VoltCoef sv;
  __shared__ int s_parity, s_done, s_last;
  __shared__ long long s_step, s_slot;
  __shared__ double s_red[kBlock / 32][P_COUNT];
  __shared__ uint32_t s_status;

  const int4 tile = a.tiles[blockIdx.x];
  const int cell = tile.x;
  {
    // cooperative copy of the cell's constants and coefficients
    const int* src = reinterpret_cast<const int*>(a.cells + cell);
    int* dst = reinterpret_cast<int*>(&sc);
    for (int w = threadIdx.x; w < (int)(sizeof(CellConst) / 4); w += blockDim.x) dst[w] = src[w];
    const int* src2 = reinterpret_cast<const int*>(&a.dyn[cell].vc);
    int* dst2 = reinterpret_cast<int*>(&sv);
    for (int w = threadIdx.x; w < (int)(sizeof(VoltCoef) / 4); w += blockDim.x) dst2[w] = src2[w];
    if (threadIdx.x == 0) {
      s_parity = a.dyn[cell].parity;
      s_done = a.dyn[cell].done;
      s_step = a.dyn[cell].m.step;
      s_slot = a.dyn[cell].out_count % a.out_cap;
      s_status = 0;
    }
  }
  __syncthreads();
  if (s_done) return;

  const bool out_step = OUT && sv.output_step && !a.lattice_only;
  const Lattice<R>& L = a.L;
  const int64_t S = L.stride;
  const int lx = sc.lx, ly = sc.ly, lz = sc.lz;
  const int lxly = lx * ly;
  const int q = tile.y + threadIdx.x;
  const bool valid = threadIdx.x < tile.z;
  const int par = s_parity;
  const R dt = R(a.dt);
  const R dth = R(a.dt / 5.0);

  // per-thread partials
  R p_cs = R(0), p_xicat = R(0), p_xinaca = R(0);
  double o[NOUT];
  if (OUT) {
#pragma unroll
    for (int k = 0; k < NOUT; ++k) o[k] = 0.0;
  }

  if (valid) {
    const int64_t g = sc.off + q;
    const int x = q % lx, y = (q / lx) % ly, z = q / lxly;
    const R* ci = L.ci[par];
    const R* cn = L.cnsr[par];
    const R* cs = L.cs[par];
    R* cinext = L.ci[par ^ 1];
    R* cnnext = L.cnsr[par ^ 1];
    R* csnext = L.cs[par ^ 1];

    R cp = L.cp[g], cjsr = L.cjsr[g], cjsrb = L.cjsrb[g], ancx = L.ancx[g];
    const R cs0 = cs[g];
    uint32_t ryr = L.ryr[g];
    uint2 lccw = L.lcc[g];
    uint32_t win = L.win[g];
    int nou = ryr & 0xff, ncu = (ryr >> 8) & 0xff, nob = (ryr >> 16) & 0xff, ncb = ryr >> 24;
    int nl = win & 0xffff, nspark = win >> 16;
    if (sv.reset_window) {  // :1244-1247
      nl = 0;
      nspark = 0;
    }
    uint32_t status = 0;
    rh_stream rng;
    const uint32_t pos = (uint32_t)((x + 1) + sc.nxf * ((y + 1) + sc.nyf * (z + 1)));
    rh_stream_init(&rng, sc.seed, sc.cell_id, pos, (uint64_t)s_step);

    // ---- LCC channels (:1248-1263, reesica.h:14-116) ----
    const R cpx = (cp + cs0 * R(ICAGAMMA)) / R(1 + ICAGAMMA);
    const R rdt = R(1.0 / a.dt);
    R bfca;
    {
      R qq = R(25) / cpx;
      bfca = R(0.175) / (R(1) + qq * qq);
    }
    int nlcp = 0;
    {
      const R ac = R(sv.alphac), bc = R(sv.betac), ad = R(sv.alphad), bd = R(sv.betad);
      const R af = R(sv.alphaf), bf = R(sv.betaf), afca = R(0.012 / 2.);
      uint32_t w0 = lccw.x, w1 = lccw.y;
      bool stop = false;
#pragma unroll
      for (int ll = 0; ll < 8; ++ll) {
        uint32_t& wd = (ll < 4) ? w0 : w1;
        const int sh = (ll & 3) * 8;
        int st = (wd >> sh) & 0xff;
        if (!stop && st < 16) {
          R u = Math<R>::uniform(&rng);
          st = lcc_next<R>(st, u * rdt, ac, bc, ad, bd, af, bf, afca, bfca);
          wd = (wd & ~(0xffu << sh)) | ((uint32_t)st << sh);
          if (st == 0) {
            ++nl;
            ++nlcp;
          }
        } else {
          stop = true;
        }
      }
      lccw.x = w0;
      lccw.y = w1;
    }
    R icat1;
    {
      R ica = R(sv.lcc_k) * (cpx * R(sv.lcc_e2z_k) - R(sc.cao));
      if (ica > R(0)) ica = R(0);
      icat1 = R(sc.svica) * R(nlcp) * ica;
    }

    // ---- RyR gating, spark flag, release (:1274-1293) ----
    R roo2, mono;
    csqn_mono<R>(cjsr, roo2, mono);
    const int prevsp = nou + nob;
    ryr_gating<R>(&rng, R(sc.ku), R(sc.ku2), R(sc.kb), cp, cjsr, mono, dt, ncu, nou, ncb, nob,
                  &status);
    if (prevsp < 5 && nou + nob >= 5) nspark = 1;
    const R po = R(nou + nob) / R(NRYR);
    R xire = R(0.0147 * SVJMAX) * po * (cjsr - cp) * R(1.0 / VP);
    if (xire < R(0)) xire = R(0);

    // ---- NCX (:1296, subroutine_cuda.c:47-75) ----
    R xinaca;
    {
      const R csm = cs0 / R(1000);
      const R t2 = R(KMNAO * KMNAO * KMNAO) * csm * (R(1) + csm * R(1.0 / KMCAI));
      const R t3 = R(sv.ncx_t3a) + csm * R(XNAO * XNAO * XNAO);
      const R inaca = ancx * R(VNACA) * (R(sv.ncx_num_a) - R(sv.ncx_num_b) * csm) /
                      ((R(sv.ncx_t1) + t2 + t3) * R(sv.ncx_den2));
      const R r3 = R(0.0003) / csm;
      ancx += (R(1) / (R(1) + r3 * r3 * r3) - ancx) * R(1.0 / 150.) * dt;
      xinaca = R(sc.svncx) * inaca;
    }

    // ---- own sub-voxels (old values) ----
    R cio[8], cno[8];
#pragma unroll
    for (int ii = 0; ii < 8; ++ii) {
      cio[ii] = ci[ii * S + g];
      cno[ii] = cn[ii * S + g];
    }

    // ---- dyad/submembrane/JSR couplings and CSQN (:1309-1317) ----
    const R diffpi0 = (cp - cio[0]) * R(1.0 / TAUPI / 2.);
    const R diffpi1 = (cp - cio[1]) * R(1.0 / TAUPI / 2.);
    const R diffsi0 = (cs0 - cio[0]) * R(1.0 / TAUSI / 2.);
    const R diffsi1 = (cs0 - cio[1]) * R(1.0 / TAUSI / 2.);
    const R diffjn0 = (cjsr - cno[0]) * R(1.0 / TAUTR / 2.);
    const R diffjn1 = (cjsr - cno[1]) * R(1.0 / TAUTR / 2.);
    const R beta = csqn_beta<R>(cjsr, roo2, mono);
    const R jterm = (-diffjn0 - diffjn1) - xire * R(VP / VJSR);
    const R dotcjsr = beta * jterm;
    cjsrb += (R(1) - beta) * jterm * dt;

    // ---- sub-voxel diffusion, SERCA/leak, cytosolic buffers (:1305-1393) ----
    const bool has_zp = z + 1 < lz, has_zm = z > 0;
    const bool has_yp = y + 1 < ly, has_ym = y > 0;
    const bool has_xp = x + 1 < lx, has_xm = x > 0;
    const R kt_n = R(1.0 / (TAUNT * XI)), kl_n = R(1.0 / (TAUNL * XI));
    const R kt_i = R(1.0 / (TAUIT * XI)), kl_i = R(1.0 / (TAUIL * XI));
    const R sviup = R(sc.sviup_tot);
    const R rdt95 = R(0.95 / a.dt);
    R sum_ci = R(0), sum_cn = R(0), sum_catf = R(0), sum_cats = R(0), sum_casr = R(0);
    R sum_camyo = R(0), sum_cacal = R(0), sum_up = R(0), sum_lk = R(0);
    R ci_sub0 = R(0), camyo0 = R(0), mgmyo0 = R(0), casr0 = R(0), cacal0 = R(0), cats0 = R(0),
      catf0 = R(0);
    bool ci_high = false;
#pragma unroll
    for (int ii = 0; ii < 8; ++ii) {
      const int bz = ii & 1, by = (ii >> 1) & 1, bx = (ii >> 2) & 1;
      const R c = cio[ii], n = cno[ii];
      // +z / -z
      R ciN, cnN, ciS, cnS;
      if (bz) {
        ciS = cio[ii - 1];
        cnS = cno[ii - 1];
        if (has_zp) {
          ciN = __ldg(ci + (ii - 1) * S + g + lxly);
          cnN = __ldg(cn + (ii - 1) * S + g + lxly);
        } else {
          ciN = c;
          cnN = n;
        }
      } else {
        ciN = cio[ii + 1];
        cnN = cno[ii + 1];
        if (has_zm) {
          ciS = __ldg(ci + (ii + 1) * S + g - lxly);
          cnS = __ldg(cn + (ii + 1) * S + g - lxly);
        } else {
          ciS = c;
          cnS = n;
        }
      }
      // +y / -y
      R ciE, cnE, ciW, cnW;
      if (by) {
        ciW = cio[ii - 2];
        cnW = cno[ii - 2];
        if (has_yp) {
          ciE = __ldg(ci + (ii - 2) * S + g + lx);
          cnE = __ldg(cn + (ii - 2) * S + g + lx);
        } else {
          ciE = c;
          cnE = n;
        }
      } else {
        ciE = cio[ii + 2];
        cnE = cno[ii + 2];
        if (has_ym) {
          ciW = __ldg(ci + (ii + 2) * S + g - lx);
          cnW = __ldg(cn + (ii + 2) * S + g - lx);
        } else {
          ciW = c;
          cnW = n;
        }
      }
      // +x / -x
      R ciT, cnT, ciB, cnB;
      if (bx) {
        ciB = cio[ii - 4];
        cnB = cno[ii - 4];
        if (has_xp) {
          ciT = __ldg(ci + (ii - 4) * S + g + 1);
          cnT = __ldg(cn + (ii - 4) * S + g + 1);
        } else {
          ciT = c;
          cnT = n;
        }
      } else {
        ciT = cio[ii + 4];
        cnT = cno[ii + 4];
        if (has_xm) {
          ciB = __ldg(ci + (ii + 4) * S + g - 1);
          cnB = __ldg(cn + (ii + 4) * S + g - 1);
        } else {
          ciB = c;
          cnB = n;
        }
      }
      const R coupn = ((cnN - n) + (cnS - n) + (cnE - n) + (cnW - n)) * kt_n +
                      ((cnT - n) + (cnB - n)) * kl_n;
      const R coupi = ((ciN - c) + (ciS - c) + (ciE - c) + (ciW - c)) * kt_i +
                      ((ciT - c) + (ciB - c)) * kl_i;
      // SERCA and leak (subroutine_cuda.c:128-146)
      const R pa = Math<R>::powpos(c * R(1.0 / KI_UP), R(HH_UP));
      const R pb = Math<R>::powpos(n * R(1.0 / KNSR_UP), R(HH_UP));
      const R up = sviup * (R(VUP) * (pa - pb) / (R(1) + pa + pb));
      const R n2 = n * n;
      const R lk = R(GLEAK) * (n - c) * n2 / (n2 + R(KJSR_LEAK * KJSR_LEAK));
      // buffers (buffers.c:55-115)
      const int64_t gi = ii * S + g;
      R catf = L.catf[gi], cats = L.cats[gi], cacal = L.cacal[gi], casr = L.casr[gi];
      R camyo = L.camyo[gi], mgmyo = L.mgmyo[gi];
      const R r_tf = buffer_rate<R>(R(KTFON), R(KTFOFF), R(BTF), catf, c, dt, rdt95);
      const R r_ts = buffer_rate<R>(R(KTSON), R(KTSOFF), R(BTS), cats, c, dt, rdt95);
      const R r_cal = buffer_rate<R>(R(KCALON), R(KCALOFF), R(BCAL), cacal, c, dt, rdt95);
      const R r_sr = buffer_rate<R>(R(KSRON), R(KSROFF), R(BSR), casr, c, dt, rdt95);
      const R freemyo = R(BMYO) - camyo - mgmyo;
      const R onmc = R(KONMYOCA) * c;
      const R r_mc = (onmc * dt > R(1)) ? rdt95 * freemyo - R(KOFFMYOCA) * camyo
                                        : onmc * freemyo - R(KOFFMYOCA) * camyo;
      R dotcn = (up - lk) * R(VI / VNSR) + coupn;
      R dotci = (-up + lk) - (r_tf + r_ts + r_cal + r_sr + r_mc) + coupi;
      if (ii == 0) {
        dotcn += diffjn0 * R(VJSR / VNSR);
        dotci += diffsi0 * R(VS / VI);
        dotci += diffpi0 * R(VP / VI);
      } else if (ii == 1) {
        dotcn += diffjn1 * R(VJSR / VNSR);
        dotci += diffsi1 * R(VS / VI);
        dotci += diffpi1 * R(VP / VI);
      }
      const R cinew = clamp0(c + dotci * dt);
      const R cnnew = n + dotcn * dt;
      catf = clamp0(catf + r_tf * dt);
      cats = clamp0(cats + r_ts * dt);
      cacal = clamp0(cacal + r_cal * dt);
      casr = clamp0(casr + r_sr * dt);
      camyo = clamp0(camyo + r_mc * dt);
      {
        const R fm = R(BMYO) - camyo - mgmyo;
        const R onmg = R(KONMYOMG * MGI);
        const R r_mg = (onmg * dt > R(1)) ? rdt95 * fm - R(KOFFMYOMG) * mgmyo
                                          : onmg * fm - R(KOFFMYOMG) * mgmyo;
        mgmyo = clamp0(mgmyo + r_mg * dt);
      }
      cinext[gi] = cinew;
      cnnext[gi] = cnnew;
      L.catf[gi] = catf;
      L.cats[gi] = cats;
      L.cacal[gi] = cacal;
      L.casr[gi] = casr;
      L.camyo[gi] = camyo;
      L.mgmyo[gi] = mgmyo;
      if (a.diag) {
        a.diag[(int64_t)(D_XIUP + ii) * S + g] = (double)up;
        a.diag[(int64_t)(D_XILEAK + ii) * S + g] = (double)lk;
      }
      if (out_step) {
        sum_ci += cinew;
        sum_cn += cnnew;
        sum_catf += catf;
        sum_cats += cats;
        sum_casr += casr;
        sum_camyo += camyo;
        sum_cacal += cacal;
        sum_up += up;
        sum_lk += lk;
        ci_high |= cinew > R(1000);
        if (ii == 0) {
          ci_sub0 = cinew;
          camyo0 = camyo;
          mgmyo0 = mgmyo;
          casr0 = casr;
          cacal0 = cacal;
          cats0 = cats;
          catf0 = catf;
        }
      }
    }

    // ---- five sub-steps of cs, cp and the sarcolemmal buffers (:1396-1473) ----
    R casar = L.casar[g], casarh = L.casarh[g], casarj = L.casarj[g], casarhj = L.casarhj[g];
    R csn = cs0;
    {
      const R csN = has_zp ? __ldg(cs + g + lxly) : cs0;
      const R csS = has_zm ? __ldg(cs + g - lxly) : cs0;
      const R csdiff = (csN + csS - R(2) * cs0) * R(1.0 / TAUST);
      const R cs_const = -R(ICAGAMMA * VP / VS) * icat1 + xinaca -
                         (cs0 - cio[0]) * R(1.0 / TAUSI / 2.) -
                         (cs0 - cio[1]) * R(1.0 / TAUSI / 2.) + csdiff;
      const R cp_const = (cio[0] - cp) * R(1.0 / TAUPI / 2.) + (cio[1] - cp) * R(1.0 / TAUPI / 2.) +
                         xire - icat1;
      const R rdth95 = R(0.95 * 5.0 / a.dt);
#pragma unroll 1
      for (int it = 0; it < 5; ++it) {
        const R r_sar = buffer_rate<R>(R(KSARON), R(KSAROFF), R(BSAR), casar, csn, dth, rdth95);
        const R r_sarh = buffer_rate<R>(R(KSARHON), R(KSARHOFF), R(BSARH), casarh, csn, dth, rdth95);
        const R dotcs = R(VP / VS / TAUPS) * (cp - csn) + cs_const - (r_sar + r_sarh);
        const R cpbuff = buffer_rate<R>(R(KSARON), R(KSAROFF), R(BSAR), casarj, cp, dth, rdth95);
        const R cpbuffh = buffer_rate<R>(R(KSARHON), R(KSARHOFF), R(BSARH), casarhj, cp, dth, rdth95);
        const R cpdot = (csn - cp) * R(1.0 / TAUPS) + cp_const - cpbuff - cpbuffh;
        casarj = clamp0(casarj + cpbuff * dth);
        casarhj = clamp0(casarhj + cpbuffh * dth);
        cp += cpdot * dth;
        casar = clamp0(casar + r_sar * dth);
        casarh = clamp0(casarh + r_sarh * dth);
        csn += dotcs * dth;
      }
    }
    if (cp < R(0)) cp = R(0);
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
      a.diag[(int64_t)D_XICAT * S + g] = (double)icat1;
    }
    if (status) atomicOr(&s_status, status);

    p_cs = csn;
    p_xicat = icat1;
    p_xinaca = xinaca;

    if (out_step) {
      o[O_CP - P_STEP_END] = (double)cp;
      o[O_CJSR - P_STEP_END] = (double)cjsr;
      o[O_CJSRB - P_STEP_END] = (double)cjsrb;
      o[O_CNSR - P_STEP_END] = (double)sum_cn;
      o[O_CI - P_STEP_END] = (double)sum_ci;
      o[O_PO - P_STEP_END] = (double)po;
      o[O_NCB - P_STEP_END] = (double)ncb;
      o[O_NCXFWD - P_STEP_END] = xinaca < R(0) ? (double)xinaca : 0.0;
      o[O_CATF - P_STEP_END] = (double)sum_catf;
      o[O_CATS - P_STEP_END] = (double)sum_cats;
      o[O_CASR - P_STEP_END] = (double)sum_casr;
      o[O_CAMYO - P_STEP_END] = (double)sum_camyo;
      o[O_CACAL - P_STEP_END] = (double)sum_cacal;
      o[O_LEAK - P_STEP_END] = (double)sum_lk;
      o[O_UP - P_STEP_END] = (double)sum_up;
      o[O_XIRE - P_STEP_END] = (double)xire;
      o[O_ANCX - P_STEP_END] = (double)ancx;
      o[O_CASAR - P_STEP_END] = (double)casar;
      o[O_CASARH - P_STEP_END] = (double)casarh;
      o[O_CASARJ - P_STEP_END] = (double)casarj;
      o[O_CASARHJ - P_STEP_END] = (double)casarhj;
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
        for (int k = 0; k < 7; ++k) o[O_TN1 - P_STEP_END + k] = tn[k];
      }
      o[O_SPARK - P_STEP_END] = nspark;
      o[O_CIHIGH - P_STEP_END] = ci_high ? 1.0 : 0.0;
      if (y == sc.line_y && z == sc.line_z) {  // linescan row (:967-989)
        double* r = a.out_ls + ((size_t)sc.ls_off + (size_t)s_slot * lx + x) * RH_LINESCAN_COLS;
        r[0] = sv.t;
        r[1] = (double)(x + 1);
        r[2] = (double)ci_sub0;
        r[3] = nob;
        r[4] = nou;
        r[5] = ncb;
        r[6] = ncu;
        r[7] = nl;
        r[8] = (double)csn;
        r[9] = (double)cp;
        r[10] = (double)casar;
        r[11] = (double)casarh;
        r[12] = (double)camyo0;
        r[13] = (double)mgmyo0;
        r[14] = (double)casr0;
        r[15] = (double)cacal0;
        r[16] = (double)cats0;
        r[17] = (double)catf0;
        r[18] = (double)xire;
        r[19] = (double)cjsr;
        r[20] = (double)ancx;
        r[21] = (double)xinaca;
      }
    }
  }

  // ---- CTA reduction of the partials ----
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  {
    double s, c;
    warp_sum_comp(p_cs, s, c);
    if (lane == 0) {
      s_red[warp][P_CS] = s;
      s_red[warp][P_CS + 1] = c;
    }
    warp_sum_comp(p_xicat, s, c);
    if (lane == 0) {
      s_red[warp][P_XICAT] = s;
      s_red[warp][P_XICAT + 1] = c;
    }
    warp_sum_comp(p_xinaca, s, c);
    if (lane == 0) {
      s_red[warp][P_XINACA] = s;
      s_red[warp][P_XINACA + 1] = c;
    }
    if (out_step) {
#pragma unroll 1
      for (int k = 0; k < NOUT; ++k) {
        double v = o[k];
        if (k == O_CIHIGH - P_STEP_END) {
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, off));
        } else {
          v = warp_sum(v);
        }
        if (lane == 0) s_red[warp][P_STEP_END + k] = v;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    constexpr int NW = kBlock / 32;
    double* dst = a.partials + (size_t)blockIdx.x * P_COUNT;
    if (lane < 3) {
      // compensated sum over warps in fixed order
      double s = 0.0, c = 0.0;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        double e;
        two_sum(s, s_red[w][2 * lane], s, e);
        c += e + s_red[w][2 * lane + 1];
      }
      dst[2 * lane] = s;
      dst[2 * lane + 1] = c;
    }
    if (out_step) {
      for (int k = lane; k < NOUT; k += 32) {
        double v = 0.0;
        if (k == O_CIHIGH - P_STEP_END) {
          for (int w = 0; w < NW; ++w) v = fmax(v, s_red[w][P_STEP_END + k]);
        } else {
          for (int w = 0; w < NW; ++w) v += s_red[w][P_STEP_END + k];
        }
        dst[P_STEP_END + k] = v;
      }
    }
    if (lane == 0) {
      if (s_status) atomicOr(&a.dyn[cell].status, s_status);
      __threadfence();
      unsigned int prev = atomicAdd(&a.dyn[cell].arrive, 1u);
      s_last = (prev == (unsigned)(sc.tile_count - 1));
    }
    __syncwarp();
  }
  __syncthreads();
  if (!s_last) return;
  // ---- last CTA of the cell: whole-cell update ----
  if (threadIdx.x < 32) {
    __threadfence();
    if (a.lattice_only) {
      if (threadIdx.x == 0) {
        a.dyn[cell].parity = par ^ 1;
        a.dyn[cell].arrive = 0;
      }
    } else {
      cell_update<R>(a, cell, sc, out_step);
      if (threadIdx.x == 0) {
        a.dyn[cell].parity = par ^ 1;
        a.dyn[cell].arrive = 0;
      }
    }
  }
}

// ------------------------------------------------------------- other kernels

// Fills a cell's CRUs with its basal state (values computed on the host by
// the Init rules, cuda_Cell_Detailed.cu:1108-1182).
template <class R>
__global__ void init_kernel(Lattice<R> L, const CellConst* cells, const InitValues* iv, int ncells) {
  const int cell = blockIdx.y;
  if (cell >= ncells) return;
  const CellConst& c = cells[cell];
  const InitValues& v = iv[cell];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < c.n; q += gridDim.x * blockDim.x) {
    const int64_t g = c.off + q, S = L.stride;
    L.cp[g] = R(v.cp);
    L.cs[0][g] = R(v.cs);
    L.cs[1][g] = R(v.cs);
    L.cjsr[g] = R(v.cjsr);
    L.cjsrb[g] = R(v.cjsrb);
    L.ancx[g] = R(v.ancx);
    L.casar[g] = R(v.casar);
    L.casarh[g] = R(v.casarh);
    L.casarj[g] = R(v.casarj);
    L.casarhj[g] = R(v.casarhj);
    for (int ii = 0; ii < 8; ++ii) {
      const int64_t gi = ii * S + g;
      L.ci[0][gi] = R(v.ci);
      L.ci[1][gi] = R(v.ci);
      L.cnsr[0][gi] = R(v.cnsr);
      L.cnsr[1][gi] = R(v.cnsr);
      L.catf[gi] = R(v.catf);
      L.cats[gi] = R(v.cats);
      L.cacal[gi] = R(v.cacal);
      L.casr[gi] = R(v.casr);
      L.camyo[gi] = R(v.camyo);
      L.mgmyo[gi] = R(v.mgmyo);
    }
    L.ryr[g] = (uint32_t)v.nou | ((uint32_t)v.ncu << 8) | ((uint32_t)v.nob << 16) |
               ((uint32_t)v.ncb << 24);
    L.lcc[g] = make_uint2(v.lcc_lo, v.lcc_hi);
    L.win[g] = 0;
  }
}

// Voltage coefficients from the current membrane state (after create or a
// host-side membrane change).
__global__ void volt_prep_kernel(const CellConst* cells, CellDyn* dyn, int ncells, double dt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  VoltCoef vc;
  volt_coef(vc, dyn[c].m, cells[c], dt);
  dyn[c].vc = vc;
  if (!vc.active) {
    dyn[c].done = 1;
    dyn[c].status |= RH_STATUS_DONE;
  } else {
    dyn[c].done = 0;
    dyn[c].status &= ~RH_STATUS_DONE;
  }
}

// ------------------------------------------------------------- launchers

template <class R>
cudaError_t launch_step(const StepArgs<R>& a, int ntiles, bool out, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  if (out)
    step_kernel<R, true><<<ntiles, kBlock, 0, st>>>(a);
  else
    step_kernel<R, false><<<ntiles, kBlock, 0, st>>>(a);
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_init(const Lattice<R>& L, const CellConst* cells, const InitValues* iv,
                        int ncells, int max_n, cudaStream_t st) {
  dim3 grid((max_n + 255) / 256, ncells);
  if (grid.x > 1024) grid.x = 1024;
  init_kernel<R><<<grid, 256, 0, st>>>(L, cells, iv, ncells);
  return cudaGetLastError();
}

cudaError_t launch_volt_prep(const CellConst* cells, CellDyn* dyn, int ncells, double dt,
                             cudaStream_t st) {
  volt_prep_kernel<<<(ncells + 127) / 128, 128, 0, st>>>(cells, dyn, ncells, dt);
  return cudaGetLastError();
}

template cudaError_t launch_step<double>(const StepArgs<double>&, int, bool, cudaStream_t);
template cudaError_t launch_step<float>(const StepArgs<float>&, int, bool, cudaStream_t);
template cudaError_t launch_init<double>(const Lattice<double>&, const CellConst*,
                                         const InitValues*, int, int, cudaStream_t);
template cudaError_t launch_init<float>(const Lattice<float>&, const CellConst*,
                                        const InitValues*, int, int, cudaStream_t);

}  // namespace rh
