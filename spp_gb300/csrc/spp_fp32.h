/*
 * spp_fp32.h -- the arithmetic contract shared by the sm_103a kernels and any
 * CPU code that must reproduce them bit for bit.
 *
 * Everything here is a pure function of its arguments and compiles both as
 * CUDA device code (nvcc, -fmad=false) and as plain C99 (gcc,
 * -ffp-contract=off).  Fused multiply-adds appear only where written as
 * fmaf(), division and sqrtf() are IEEE correctly rounded on both sides, so
 * a CPU build of these functions returns the same bits as the GPU.
 *
 * Contents
 *   - Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
 *     "Parallel random numbers: as easy as 1, 2, 3", SC'11).  It replaces
 *     the single global GSL generator of the reference (shared/c2dvector.h:
 *     15-25, 134-144): a draw is a function of (seed, system, particle id,
 *     step, stream), so it does not depend on the order particles are
 *     visited in.
 *   - uniform / Gaussian mappings standing in for gsl_ran_flat and
 *     gsl_ran_gaussian (shared/particle.h:154, 568).
 *   - FP32 sin/cos/atan2/log/exp: Cody-Waite range reduction plus
 *     polynomials fitted by gen_fp32_poly.py (this directory).
 *   - periodic wrap of angles and coordinates (shared/c2dvector.h:67-73,
 *     shared/particle.h:599).
 *   - exact fixed-point accumulation (2^-27 resolution) in two int32 parts,
 *     which makes the neighbour sums independent of summation order.
 */
#ifndef SPP_FP32_H
#define SPP_FP32_H

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define SPP_HD __host__ __device__ __forceinline__
#else
#define SPP_HD static inline
#include <string.h>
#endif

/* ------------------------------------------------------------------ */
/* bit casts                                                           */
/* ------------------------------------------------------------------ */
SPP_HD uint32_t spp_f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
SPP_HD float spp_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f; memcpy(&f, &u, 4); return f;
#endif
}

/* ------------------------------------------------------------------ */
/* Philox4x32-10                                                       */
/* ------------------------------------------------------------------ */
#define SPP_PHILOX_M0 0xD2511F53u
#define SPP_PHILOX_M1 0xCD9E8D57u
#define SPP_PHILOX_W0 0x9E3779B9u
#define SPP_PHILOX_W1 0xBB67AE85u

/* Stream tags: the third counter word separates independent uses. */
#define SPP_RNG_ROT_NOISE   1u  /* rotational Gaussian noise, one per particle-step */
#define SPP_RNG_VICSEK      2u  /* Vicsek angular noise xi ~ U[-pi,pi) */
#define SPP_RNG_INIT_POS    3u  /* initial positions */
#define SPP_RNG_INIT_ANGLE  4u  /* initial headings */
#define SPP_RNG_TANGENT     5u  /* tangent-vector initialisation */
#define SPP_RNG_TRANS_NOISE 6u  /* translational noise (ContinuousParticle Kamp) */
#define SPP_RNG_SWEEP       7u  /* sweep parameter sampling */
/* Run and tumble: the start test and the direction of a tumble, the first
 * and second draw of RTPChain::Noise_Gen (shared/particle.h:1089, 1092) in
 * the per-(particle, step) stream order the tests' GSL stand-in uses. */
#define SPP_RNG_TUMBLE      SPP_RNG_VICSEK
#define SPP_RNG_TUMBLE_SIGN 101u

typedef struct { uint32_t v[4]; } spp_u32x4;

SPP_HD void spp_mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
#if defined(__CUDA_ARCH__)
  *hi = __umulhi(a, b);
  *lo = a * b;
#else
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
#endif
}

SPP_HD spp_u32x4 spp_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                   uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    spp_mulhilo(SPP_PHILOX_M0, c0, &hi0, &lo0);
    spp_mulhilo(SPP_PHILOX_M1, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += SPP_PHILOX_W0;
    k1 += SPP_PHILOX_W1;
  }
  spp_u32x4 o; o.v[0] = c0; o.v[1] = c1; o.v[2] = c2; o.v[3] = c3;
  return o;
}

/* The round keys of key (k0, k1) = (seed low, seed high): round r uses
 * (k0 + r W0, k1 + r W1) mod 2^32, ks[2r] and ks[2r + 1].  Kernels that
 * draw for many particles take them precomputed (spp_philox4x32_10_ks)
 * instead of advancing the key in every draw; the words are the same. */
SPP_HD void spp_philox_round_keys(uint64_t seed, uint32_t* ks) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    ks[2 * r] = k0;
    ks[2 * r + 1] = k1;
    k0 += SPP_PHILOX_W0;
    k1 += SPP_PHILOX_W1;
  }
}

SPP_HD spp_u32x4 spp_philox4x32_10_ks(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                      const uint32_t* ks) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    spp_mulhilo(SPP_PHILOX_M0, c0, &hi0, &lo0);
    spp_mulhilo(SPP_PHILOX_M1, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ ks[2 * r];
    uint32_t n2 = hi0 ^ c3 ^ ks[2 * r + 1];
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  spp_u32x4 o; o.v[0] = c0; o.v[1] = c1; o.v[2] = c2; o.v[3] = c3;
  return o;
}

/* Draw for (seed, system, particle id, step, stream). */
SPP_HD spp_u32x4 spp_draw(uint64_t seed, uint32_t system, uint32_t pid, uint32_t step,
                          uint32_t stream) {
  return spp_philox4x32_10(pid, step, stream, system, (uint32_t)seed,
                           (uint32_t)(seed >> 32));
}

/* 24-bit uniforms; both are exact in float and in double. */
SPP_HD float spp_u01_f(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-08f; }       /* [0,1)  */
SPP_HD float spp_u01_open0_f(uint32_t x) { return (float)((x >> 8) + 1u) * 5.9604644775390625e-08f; } /* (0,1] */
SPP_HD double spp_u01_d(uint32_t x) { return (double)(x >> 8) * 5.9604644775390625e-08; }
SPP_HD double spp_u01_open0_d(uint32_t x) { return (double)((x >> 8) + 1u) * 5.9604644775390625e-08; }

/* ------------------------------------------------------------------ */
/* constants and fitted coefficients (gen_fp32_poly.py)                */
/* ------------------------------------------------------------------ */
#define SPP_PI_F       3.14159265358979323846f
#define SPP_TWO_PI_F   6.28318530717958647692f
#define SPP_PIO2_F     1.57079632679489661923f
#define SPP_PIO4_F     0.78539816339744830962f
#define SPP_INV_2PI_F  0.15915494309189533577f
#define SPP_2_OVER_PI_F 0.63661977236758134308f
#define SPP_LOG2E_F    1.44269504088896340736f

#define SPP_SIN_C0      -0.1666666716337204f
#define SPP_SIN_C1     0.008333329111337662f
#define SPP_SIN_C2  -0.00019839353626593947f
#define SPP_SIN_C3    2.718452151384554e-06f
#define SPP_COS_C0       0.0416666679084301f
#define SPP_COS_C1   -0.0013888883404433727f
#define SPP_COS_C2   2.4799463062663563e-05f
#define SPP_COS_C3   -2.720596512517659e-07f
#define SPP_ATAN_C0      -0.3333333432674408f
#define SPP_ATAN_C1      0.19999994337558746f
#define SPP_ATAN_C2     -0.14285436272621155f
#define SPP_ATAN_C3       0.1110420972108841f
#define SPP_ATAN_C4      -0.0899854525923729f
#define SPP_ATAN_C5      0.06998246908187866f
#define SPP_ATAN_C6    -0.038038525730371475f
#define SPP_LOG_C0       0.6666666865348816f
#define SPP_LOG_C1      0.40000319480895996f
#define SPP_LOG_C2      0.28538140654563904f
#define SPP_LOG_C3      0.23567897081375122f
#define SPP_EXP_C0                      0.5f
#define SPP_EXP_C1       0.1666666567325592f
#define SPP_EXP_C2     0.041666269302368164f
#define SPP_EXP_C3      0.00833342969417572f
#define SPP_EXP_C4    0.0013946021208539605f
#define SPP_EXP_C5   0.00019826495554298162f
#define SPP_PIO2_HI 1.57080078125f
#define SPP_PIO2_MID -4.453584551811218e-06f
#define SPP_PIO2_LO -8.705516307827565e-10f
#define SPP_LN2_HI 0.693115234375f
#define SPP_LN2_LO 3.194618329871446e-05f

/* ------------------------------------------------------------------ */
/* sin / cos                                                           */
/* ------------------------------------------------------------------ */
/* Valid for |x| up to ~1e4 (three-part Cody-Waite reduction by pi/2). */
SPP_HD void spp_sincosf(float x, float* s_out, float* c_out) {
  float k = rintf(x * SPP_2_OVER_PI_F);
  float r = fmaf(-k, SPP_PIO2_HI, x);
  r = fmaf(-k, SPP_PIO2_MID, r);
  r = fmaf(-k, SPP_PIO2_LO, r);
  float z = r * r;
  float ps = fmaf(fmaf(fmaf(SPP_SIN_C3, z, SPP_SIN_C2), z, SPP_SIN_C1), z, SPP_SIN_C0);
  float s = fmaf(r * z, ps, r);
  float pc = fmaf(fmaf(fmaf(SPP_COS_C3, z, SPP_COS_C2), z, SPP_COS_C1), z, SPP_COS_C0);
  float c = fmaf(z * z, pc, fmaf(-0.5f, z, 1.0f));
  int q = ((int)k) & 3;
  float so, co;
  if (q == 0) { so = s; co = c; }
  else if (q == 1) { so = c; co = -s; }
  else if (q == 2) { so = -s; co = -c; }
  else { so = -c; co = s; }
  *s_out = so;
  *c_out = co;
}
SPP_HD float spp_cosf(float x) { float s, c; spp_sincosf(x, &s, &c); return c; }
SPP_HD float spp_sinf(float x) { float s, c; spp_sincosf(x, &s, &c); return s; }

/* ------------------------------------------------------------------ */
/* atan2                                                               */
/* ------------------------------------------------------------------ */
/* Returns a value in [-pi, pi]; atan2(0, 0) returns 0. */
SPP_HD float spp_atan2f(float y, float x) {
  float ax = fabsf(x), ay = fabsf(y);
  float mx = ax > ay ? ax : ay;
  float mn = ax > ay ? ay : ax;
  if (mx == 0.0f) return 0.0f;
  float a = mn / mx;
  float t, base;
  if (a > 0.41421356237309503f) { t = (a - 1.0f) / (a + 1.0f); base = SPP_PIO4_F; }
  else { t = a; base = 0.0f; }
  float u = t * t;
  float p = SPP_ATAN_C6;
  p = fmaf(p, u, SPP_ATAN_C5);
  p = fmaf(p, u, SPP_ATAN_C4);
  p = fmaf(p, u, SPP_ATAN_C3);
  p = fmaf(p, u, SPP_ATAN_C2);
  p = fmaf(p, u, SPP_ATAN_C1);
  p = fmaf(p, u, SPP_ATAN_C0);
  float r = fmaf(t * u, p, t) + base;
  if (ay > ax) r = SPP_PIO2_F - r;
  if (x < 0.0f) r = SPP_PI_F - r;
  if (y < 0.0f) r = -r;
  return r;
}

/* ------------------------------------------------------------------ */
/* log (argument > 0, normal) and exp (|x| < 80)                       */
/* ------------------------------------------------------------------ */
SPP_HD float spp_logf(float u) {
  uint32_t b = spp_f2u(u);
  int e = (int)(b >> 23) - 127;
  float m = spp_u2f((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421356237309505f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float w = s * s;
  float R = fmaf(fmaf(fmaf(SPP_LOG_C3, w, SPP_LOG_C2), w, SPP_LOG_C1), w, SPP_LOG_C0);
  float lm = fmaf(s * w, R, 2.0f * s);
  float fe = (float)e;
  return fmaf(fe, SPP_LN2_HI, fmaf(fe, SPP_LN2_LO, lm));
}

SPP_HD float spp_expf(float x) {
  float k = rintf(x * SPP_LOG2E_F);
  float r = fmaf(-k, SPP_LN2_HI, x);
  r = fmaf(-k, SPP_LN2_LO, r);
  float p = SPP_EXP_C5;
  p = fmaf(p, r, SPP_EXP_C4);
  p = fmaf(p, r, SPP_EXP_C3);
  p = fmaf(p, r, SPP_EXP_C2);
  p = fmaf(p, r, SPP_EXP_C1);
  p = fmaf(p, r, SPP_EXP_C0);
  float e = fmaf(r * r, p, r) + 1.0f;
  int ki = (int)k;
  return e * spp_u2f((uint32_t)(ki + 127) << 23);
}

/* 1/sqrt(x) for normal x > 0: the bit-level initial estimate of Lomont
 * ("Fast inverse square root", 2003; constant 0x5f375a86, ~3.4% error)
 * refined by three Newton-Raphson steps y <- y (3/2 - (x/2) y^2) written with
 * fused multiply-adds; within 2 ulp over the normal range.  One such call
 * replaces the sqrtf + division of a pair force. */
SPP_HD float spp_rsqrtf(float x) {
  float y = spp_u2f(0x5f375a86u - (spp_f2u(x) >> 1));
  const float h = 0.5f * x;
  y = y * fmaf(-h * y, y, 1.5f);
  y = y * fmaf(-h * y, y, 1.5f);
  y = y * fmaf(-h * y, y, 1.5f);
  return y;
}

/* ------------------------------------------------------------------ */
/* noise mappings                                                      */
/* ------------------------------------------------------------------ */
/* xi ~ U[-pi, pi): (2u-1) is exact, then one rounding for the product. */
SPP_HD float spp_uniform_pm_pi_f(uint32_t x) {
  float u = spp_u01_f(x);
  return (2.0f * u - 1.0f) * SPP_PI_F;
}
/* Box-Muller: z = sqrt(-2 ln u1) cos(2 pi u2), u1 in (0,1], u2 in [0,1). */
SPP_HD float spp_normal_f(uint32_t x0, uint32_t x1) {
  float u1 = spp_u01_open0_f(x0);
  float u2 = spp_u01_f(x1);
  float rad = sqrtf(-2.0f * spp_logf(u1));
  return rad * spp_cosf(u2 * SPP_TWO_PI_F);
}

/* ------------------------------------------------------------------ */
/* two-lane FP32 operations                                            */
/* ------------------------------------------------------------------ */
/* A pair of floats handled together.  On sm_103a one packed instruction
 * (add / sub / fma .rn.f32x2) performs both lanes, each lane correctly
 * rounded exactly as the scalar operation, so the CPU's two scalar
 * operations return the same bits. */
typedef struct { float x, y; } spp_f2;

SPP_HD spp_f2 spp_f2_make(float x, float y) { spp_f2 r; r.x = x; r.y = y; return r; }
#if defined(__CUDA_ARCH__)
SPP_HD unsigned long long spp_f2_pack(spp_f2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
SPP_HD spp_f2 spp_f2_unpack(unsigned long long r) {
  spp_f2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
/* a - b */
SPP_HD spp_f2 spp_sub2(spp_f2 a, spp_f2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(spp_f2_pack(a)), "l"(spp_f2_pack(b)));
  return spp_f2_unpack(r);
}
/* a + b */
SPP_HD spp_f2 spp_add2(spp_f2 a, spp_f2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(spp_f2_pack(a)), "l"(spp_f2_pack(b)));
  return spp_f2_unpack(r);
}
/* fmaf(t, b, c) in both lanes */
SPP_HD spp_f2 spp_fma2s(float t, spp_f2 b, spp_f2 c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(spp_f2_pack(spp_f2_make(t, t))),
      "l"(spp_f2_pack(b)), "l"(spp_f2_pack(c)));
  return spp_f2_unpack(r);
}
/* a * b */
SPP_HD spp_f2 spp_mul2(spp_f2 a, spp_f2 b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(spp_f2_pack(a)), "l"(spp_f2_pack(b)));
  return spp_f2_unpack(r);
}
/* fmaf(a, b, c) lane by lane */
SPP_HD spp_f2 spp_fma2(spp_f2 a, spp_f2 b, spp_f2 c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(spp_f2_pack(a)), "l"(spp_f2_pack(b)),
      "l"(spp_f2_pack(c)));
  return spp_f2_unpack(r);
}
#else
SPP_HD spp_f2 spp_sub2(spp_f2 a, spp_f2 b) { return spp_f2_make(a.x - b.x, a.y - b.y); }
SPP_HD spp_f2 spp_add2(spp_f2 a, spp_f2 b) { return spp_f2_make(a.x + b.x, a.y + b.y); }
SPP_HD spp_f2 spp_fma2s(float t, spp_f2 b, spp_f2 c) {
  return spp_f2_make(fmaf(t, b.x, c.x), fmaf(t, b.y, c.y));
}
SPP_HD spp_f2 spp_mul2(spp_f2 a, spp_f2 b) { return spp_f2_make(a.x * b.x, a.y * b.y); }
SPP_HD spp_f2 spp_fma2(spp_f2 a, spp_f2 b, spp_f2 c) {
  return spp_f2_make(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
}
#endif

/* spp_rsqrtf of two values at once: the same steps lane by lane, so each
 * lane returns the bits of the scalar call.  (-0.5) x equals -(0.5 x)
 * exactly (scaling by a power of two, rounding symmetric about zero), which
 * is the scalar form's -h. */
SPP_HD spp_f2 spp_rsqrtf2(spp_f2 x) {
  spp_f2 y = spp_f2_make(spp_u2f(0x5f375a86u - (spp_f2u(x.x) >> 1)),
                         spp_u2f(0x5f375a86u - (spp_f2u(x.y) >> 1)));
  const spp_f2 nh = spp_mul2(spp_f2_make(-0.5f, -0.5f), x);
  const spp_f2 c15 = spp_f2_make(1.5f, 1.5f);
  y = spp_mul2(y, spp_fma2(spp_mul2(nh, y), y, c15));
  y = spp_mul2(y, spp_fma2(spp_mul2(nh, y), y, c15));
  y = spp_mul2(y, spp_fma2(spp_mul2(nh, y), y, c15));
  return y;
}

/* ------------------------------------------------------------------ */
/* periodic wraps                                                      */
/* ------------------------------------------------------------------ */
/* theta -> theta - 2 pi floor(theta / 2 pi + 1/2), as shared/particle.h:599. */
SPP_HD float spp_wrap_angle_f(float th) {
  float q = floorf(fmaf(th, SPP_INV_2PI_F, 0.5f));
  return fmaf(-q, SPP_TWO_PI_F, th);
}
/* Coordinate in [-L, L) after a move of less than one box length.  The
 * subtractions are exact (Sterbenz), so wrapping loses no bits; *img counts
 * box crossings so that the unwrapped position is x + 2L * img. */
SPP_HD float spp_wrap_coord_f(float x, float L, float L2, int* img) {
  if (x >= L) { x -= L2; *img += 1; }
  else if (x < -L) { x += L2; *img -= 1; }
  return x;
}
/* Minimum image of a separation of two wrapped coordinates. */
SPP_HD float spp_min_image_f(float d, float L, float L2) {
  if (d >= L) d -= L2;
  else if (d < -L) d += L2;
  return d;
}

/* ------------------------------------------------------------------ */
/* fixed-point accumulation                                            */
/* ------------------------------------------------------------------ */
/* A term x (|x| < 2^16) is split exactly into a coarse part, x rounded to a
 * multiple of 2^-5, and a fine remainder rounded to a multiple of 2^-27; the
 * integer counts of both parts go to two int32 accumulators.  Integer sums
 * are exact, so the total does not depend on the order of the terms.  The
 * split uses only FP32 adds/multiplies and integer subtracts of bit patterns
 * (the "magic number" rounding: adding 1.5 * 2^k moves x into a binade whose
 * ulp is the desired grid, and the bit-pattern difference is the integer
 * count).  Conversions to or from 64-bit integers are avoided on purpose: on
 * this GPU they execute on the FP64 pipe, which is a small fraction of the
 * FP32 rate.  Bounds: |x| < 2^16 per term (spp_fx_ok), up to 1024 terms per
 * accumulator. */
#define SPP_FX_HI_MAGIC  393216.0f      /* 1.5 * 2^18, ulp 2^-5 */
#define SPP_FX_LO_MAGIC  12582912.0f    /* 1.5 * 2^23, ulp 1    */
#define SPP_FX_LO_SCALE  134217728.0f   /* 2^27 */
#define SPP_FX_INV_LO    7.450580596923828125e-09f /* 2^-27 */
#define SPP_FX_INV_HI    0.03125f       /* 2^-5 */
#define SPP_FX_RANGE     65536.0f       /* |term| < 2^16 */

typedef struct { int32_t hi, lo; } spp_fx;

SPP_HD int spp_fx_ok(float x) { return fabsf(x) < SPP_FX_RANGE; }

SPP_HD void spp_fx_add(spp_fx* a, float x) {
  const float t = x + SPP_FX_HI_MAGIC;          /* x rounded to a multiple of 2^-5 */
  const float h = t - SPP_FX_HI_MAGIC;          /* exact */
  const float l = x - h;                        /* exact, |l| <= 2^-6 */
  const float u = l * SPP_FX_LO_SCALE + SPP_FX_LO_MAGIC; /* round(l * 2^27) */
  a->hi += (int32_t)(spp_f2u(t) - spp_f2u(SPP_FX_HI_MAGIC));
  a->lo += (int32_t)(spp_f2u(u) - spp_f2u(SPP_FX_LO_MAGIC));
}

SPP_HD float spp_fx_value(spp_fx a) {
  return fmaf((float)a.lo, SPP_FX_INV_LO, (float)a.hi * SPP_FX_INV_HI);
}

/* The exact sum in units of 2^-27 (for reductions across particles). */
SPP_HD int64_t spp_fx_units(spp_fx a) { return (int64_t)a.hi * 4194304 + (int64_t)a.lo; }

#endif /* SPP_FP32_H */
