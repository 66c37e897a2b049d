/*
 * rh_philox.h — counter-based uniform provider shared by the CUDA kernels and
 * the CPU oracle.
 *
 * Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3" (SC'11): a 4x32-bit counter, a 2x32-bit
 * key, ten rounds of two 32x32->64 multiplies with the Weyl key schedule.
 *
 * Stream layout (the "draw index" spec both sides follow):
 *   key     = (seed, cell)
 *   counter = (draw >> 1, pos, step_lo, step_hi)
 * where `pos` is the CRU's linear index in the full lattice including the
 * ghost shell (pos = nx*ny*k + nx*j + i, as cuda_Cell_Detailed.cu:160-162
 * defines it), `step` is the number of lattice updates done before this one,
 * and `draw` counts the uniforms this CRU has consumed in this step, in the
 * order the reference calls curand: LCC slots first (reesica.h:65, one per
 * populated slot, cuda_Cell_Detailed.cu:1253-1261), then the eight RyR
 * transitions of subroutine_cuda.c:332-613 in source order.
 *
 * One Philox block (4 words) serves two draws: draw d uses the 64-bit half
 *   x = w[2h+1]:w[2h],  h = d & 1.
 *   double  u = ((x >> 11) + 1) * 2^-53          in (0, 1]
 *   float   u = ((w[2h+1] >> 8) + 1) * 2^-24     in (0, 1]  (the top 24 bits
 *                                                of the same draw)
 *   uint32    = w[2h]                           (the reference's curand())
 * The (0,1] range is the one curand_uniform_double has.
 *
 * Draws made while the lattice is initialised (the LCC count of a randomlcc
 * cell, cuda_Cell_Detailed.cu:1150-1151) use step = RH_PHILOX_INIT_STEP, a
 * value no lattice update reaches.
 */
#ifndef RH_PHILOX_H
#define RH_PHILOX_H

#include <stdint.h>

#if defined(__CUDACC__)
#define RH_HD __host__ __device__ __forceinline__
#else
#define RH_HD static inline
#endif

#define RH_PHILOX_INIT_STEP 0xFFFFFFFFFFFFFFFFull

#define RH_PHILOX_M0 0xD2511F53u
#define RH_PHILOX_M1 0xCD9E8D57u
#define RH_PHILOX_W0 0x9E3779B9u
#define RH_PHILOX_W1 0xBB67AE85u

typedef struct {
  uint32_t w[4];
} rh_u32x4;

/* One 32x32 -> 64-bit product (a single wide multiply on the GPU). */
RH_HD void rh_mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

/* Philox4x32 with 10 rounds: counter (c0..c3), key (k0, k1). */
RH_HD rh_u32x4 rh_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                uint32_t c3, uint32_t k0, uint32_t k1) {
  rh_u32x4 r;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int round = 0; round < 10; ++round) {
    uint32_t hi0, lo0, hi1, lo1;
    rh_mulhilo32(RH_PHILOX_M0, c0, &hi0, &lo0);
    rh_mulhilo32(RH_PHILOX_M1, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += RH_PHILOX_W0;
    k1 += RH_PHILOX_W1;
  }
  r.w[0] = c0;
  r.w[1] = c1;
  r.w[2] = c2;
  r.w[3] = c3;
  return r;
}

/* Per-CRU, per-step draw stream.  `buf` caches the second half of the last
 * block so that each Philox evaluation serves two draws. */
typedef struct {
  uint32_t k0, k1;       /* seed, cell */
  uint32_t pos;          /* CRU index in the full lattice (ghosts included) */
  uint32_t step_lo, step_hi;
  uint32_t draw;         /* next draw index */
  uint32_t buf_lo, buf_hi;
} rh_stream;

RH_HD void rh_stream_init(rh_stream* s, uint32_t seed, uint32_t cell,
                          uint32_t pos, uint64_t step) {
  s->k0 = seed;
  s->k1 = cell;
  s->pos = pos;
  s->step_lo = (uint32_t)step;
  s->step_hi = (uint32_t)(step >> 32);
  s->draw = 0;
  s->buf_lo = 0;
  s->buf_hi = 0;
}

/* Raw 64-bit draw as (hi, lo) words. */
RH_HD void rh_stream_next(rh_stream* s, uint32_t* hi, uint32_t* lo) {
  uint32_t d = s->draw++;
  if ((d & 1u) == 0u) {
    rh_u32x4 b = rh_philox4x32_10(d >> 1, s->pos, s->step_lo, s->step_hi,
                                  s->k0, s->k1);
    *lo = b.w[0];
    *hi = b.w[1];
    s->buf_lo = b.w[2];
    s->buf_hi = b.w[3];
  } else {
    *lo = s->buf_lo;
    *hi = s->buf_hi;
  }
}

RH_HD double rh_bits_to_double(uint32_t hi, uint32_t lo) {
  uint64_t x = ((uint64_t)hi << 32) | (uint64_t)lo;
  return (double)((x >> 11) + 1u) * 0x1.0p-53;
}

RH_HD float rh_bits_to_float(uint32_t hi) {
  return (float)((hi >> 8) + 1u) * 0x1.0p-24f;
}

RH_HD double rh_uniform_double(rh_stream* s) {
  uint32_t hi, lo;
  rh_stream_next(s, &hi, &lo);
  return rh_bits_to_double(hi, lo);
}

RH_HD float rh_uniform_float(rh_stream* s) {
  uint32_t hi, lo;
  rh_stream_next(s, &hi, &lo);
  return rh_bits_to_float(hi);
}

RH_HD uint32_t rh_uniform_u32(rh_stream* s) {
  uint32_t hi, lo;
  rh_stream_next(s, &hi, &lo);
  return lo;
}

#endif /* RH_PHILOX_H */
