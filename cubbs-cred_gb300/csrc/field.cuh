// BLS12-381 field tower on sm_103a: Fp (12 x 32-bit limbs, Montgomery,
// R = 2^384), Fr (8 x 32-bit limbs, R = 2^256), Fp2 = Fp[u]/(u^2+1),
// Fp6 = Fp2[v]/(v^3 - (1+u)), Fp12 = Fp6[w]/(w^2 - v).
//
// The tower and encodings follow the curve arithmetic the reference protocol
// delegates to (bls12_381_plus 0.8.18; reference device types are SPPARK
// fp_t/fr_t/fp2_t, prepare_b_msm.cu:40-49, pairing.cuh:3-321).  Multiplication
// is CIOS over inline-PTX carry chains generated by gen_field_ptx.py.
#pragma once
#include <stdint.h>

#include "curve_constants.cuh"
#include "field_ptx.cuh"

#define DEV __device__ __forceinline__
#define DEVNI static __device__ __noinline__

struct fp { uint32_t w[12]; };
struct fr { uint32_t w[8]; };
struct fp2 { fp c0, c1; };
struct fp6 { fp2 c0, c1, c2; };
struct fp12 { fp6 c0, c1; };

// Bit i of |z| = 0xd201000000010000 (the BLS parameter), from two 32-bit halves.
DEV uint32_t zabs_bit(int i) { return i >= 32 ? (0xd2010000u >> (i - 32)) & 1u : (0x00010000u >> i) & 1u; }

// ------------------------------------------------------------------ Fp
DEV fp fp_zero() { fp r; _Pragma("unroll") for (int i = 0; i < 12; i++) r.w[i] = 0; return r; }
DEV fp fp_one() { const fp r = C_FP_ONE; return r; }
DEV bool fp_is_zero(const fp &a) {
  uint32_t x = 0;
  _Pragma("unroll") for (int i = 0; i < 12; i++) x |= a.w[i];
  return x == 0;
}
DEV bool fp_eq(const fp &a, const fp &b) {
  uint32_t x = 0;
  _Pragma("unroll") for (int i = 0; i < 12; i++) x |= a.w[i] ^ b.w[i];
  return x == 0;
}
DEV fp fp_add(const fp &a, const fp &b) { fp r; fp_add_raw(r.w, a.w, b.w); return r; }
DEV fp fp_sub(const fp &a, const fp &b) { fp r; fp_sub_raw(r.w, a.w, b.w); return r; }
DEV fp fp_dbl(const fp &a) { return fp_add(a, a); }
DEV fp fp_neg(const fp &a) { return fp_sub(fp_zero(), a); }
// CIOS Montgomery product over the carry chains of field_ptx.cuh (one row per
// limb of b; every row is a dependent carry chain).
DEV fp fp_mul_cios_inl(const fp &a, const fp &b) {
  uint32_t t[25];
  _Pragma("unroll") for (int i = 0; i < 13; i++) t[i] = 0;
  _Pragma("unroll") for (int i = 0; i < 12; i++) {
    t[i + 12] = 0;
    fp_cios_row(&t[i], a.w, b.w[i]);
  }
  fp r;
  fp_reduce_once(r.w, &t[12]);
  return r;
}

// The Montgomery product a b / 2^384 mod p (fully reduced) used everywhere:
// carry-save accumulation instead of carry chains.  T_j = (hi_j : lo_j) are
// 64-bit partial sums of limb position j; each row adds a_j b_i to every T_j
// (a mad.lo.cc / madc.hi pair), splits every sum into its low word and the
// high word of its right neighbour (N_j = lo(T_j) + hi(T_{j-1}) <= 2^33 - 2,
// an add.cc / addc pair, so the next 32 x 32-bit product cannot overflow 64
// bits), adds m p_j, and splits again while shifting one limb down.  No step
// depends on a carry from another limb, so the twelve products of a row
// issue back to back.  One carry pass at the end and one conditional
// subtraction of p finish it.
// Bounds: a, b < p; every partial sum stays below 2^64 (the worst case is
// (2^33 - 2) + (2^32 - 1)^2 = 2^64 - 1) and the final value is below 2p.
// Written in PTX: from the same arithmetic in C++ 64-bit integers the
// compiler put many of the splits' carry additions on the FMA pipe, beside
// the multiplies (522 FMA-pipe and 511 ALU instructions a product); here 324
// and 587.  Measured on GB300, one warp, chains of dependent products: 1965
// cycles a product against 2316 for the C++ form (and 2802 for CIOS); about
// the same with two warps per SM sub-partition (1830 vs 1860 cycles of the
// sub-partition a product) and 3 % slower with four (1813 vs 1753).  Every
// carry flag lives inside one asm statement.
DEV fp fp_mul_inl(const fp &a, const fp &b) {
  const fp pm = FP_MOD_INIT;
  uint32_t lo[12], hi[12];  // T_j = hi_j : lo_j
#pragma unroll
  for (int j = 0; j < 12; j++) lo[j] = hi[j] = 0;
#pragma unroll
  for (int i = 0; i < 12; i++) {
    const uint32_t bi = b.w[i];
#pragma unroll
    for (int j = 0; j < 12; j++)
      asm("mad.lo.cc.u32 %0, %2, %3, %0;\n\tmadc.hi.u32 %1, %2, %3, %1;"
          : "+r"(lo[j]), "+r"(hi[j])
          : "r"(a.w[j]), "r"(bi));
    uint32_t nl[12], nh[12];  // N_j = nh_j : nl_j
    nl[0] = lo[0];
    nh[0] = 0;
#pragma unroll
    for (int j = 1; j < 12; j++)
      asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=r"(nl[j]), "=r"(nh[j]) : "r"(lo[j]), "r"(hi[j - 1]));
    const uint32_t n12 = hi[11];
    const uint32_t m = nl[0] * FP_PINV;
#pragma unroll
    for (int j = 0; j < 12; j++)
      asm("mad.lo.cc.u32 %0, %2, %3, %0;\n\tmadc.hi.u32 %1, %2, %3, %1;"
          : "+r"(nl[j]), "+r"(nh[j])
          : "r"(m), "r"(pm.w[j]));
#pragma unroll
    for (int j = 0; j < 11; j++)
      asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=r"(lo[j]), "=r"(hi[j]) : "r"(nl[j + 1]), "r"(nh[j]));
    asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=r"(lo[11]), "=r"(hi[11]) : "r"(n12), "r"(nh[11]));
  }
  // t = sum_j T_j 2^(32 j): t_j = lo_j + hi_(j-1) + carry (the value is below 2p < 2^384)
  uint32_t t[12];
  asm("add.cc.u32 %0, %12, 0;\n\taddc.cc.u32 %1, %13, %24;\n\taddc.cc.u32 %2, %14, %25;\n\t"
      "addc.cc.u32 %3, %15, %26;\n\taddc.cc.u32 %4, %16, %27;\n\taddc.cc.u32 %5, %17, %28;\n\t"
      "addc.cc.u32 %6, %18, %29;\n\taddc.cc.u32 %7, %19, %30;\n\taddc.cc.u32 %8, %20, %31;\n\t"
      "addc.cc.u32 %9, %21, %32;\n\taddc.cc.u32 %10, %22, %33;\n\taddc.u32 %11, %23, %34;"
      : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7]), "=r"(t[8]),
        "=r"(t[9]), "=r"(t[10]), "=r"(t[11])
      : "r"(lo[0]), "r"(lo[1]), "r"(lo[2]), "r"(lo[3]), "r"(lo[4]), "r"(lo[5]), "r"(lo[6]), "r"(lo[7]), "r"(lo[8]),
        "r"(lo[9]), "r"(lo[10]), "r"(lo[11]), "r"(hi[0]), "r"(hi[1]), "r"(hi[2]), "r"(hi[3]), "r"(hi[4]), "r"(hi[5]),
        "r"(hi[6]), "r"(hi[7]), "r"(hi[8]), "r"(hi[9]), "r"(hi[10]));
  fp r;
  fp_reduce_once(r.w, t);
  return r;
}
// One out-of-line copy of the product per translation unit: with the body
// inlined at every call site the straight-line code of a point or Fp12
// operation overflows the instruction cache, which a lone warp per SM
// sub-partition cannot hide (measured 2.6x slower G1 doubling).
DEVNI fp fp_mul(fp a, fp b) { return fp_mul_inl(a, b); }
DEVNI fp fp_mul_cios(fp a, fp b) { return fp_mul_cios_inl(a, b); }
DEV fp fp_sqr(const fp &a) { return fp_mul(a, a); }

// raw canonical limbs (little-endian words) -> Montgomery
DEV fp fp_to_mont(const fp &a) { const fp r2 = FP_R2_INIT; return fp_mul(a, r2); }
DEV fp fp_from_mont(const fp &a) { fp one = fp_zero(); one.w[0] = 1; return fp_mul(a, one); }
DEV bool fp_lt_mod(const fp &a) {  // canonical a < p ?
  const fp m = FP_MOD_INIT;
  _Pragma("unroll") for (int i = 11; i >= 0; i--) {
    if (a.w[i] != m.w[i]) return a.w[i] < m.w[i];
  }
  return false;
}
// square-and-multiply by a 12-word exponent (most significant word first scan)
DEV fp fp_pow(const fp &a, const uint32_t *e, int nwords) {
  fp r = fp_one();
  #pragma unroll 1
  for (int i = nwords * 32 - 1; i >= 0; i--) {
    r = fp_sqr(r);
    if ((e[i >> 5] >> (i & 31)) & 1) r = fp_mul(r, a);
  }
  return r;
}
// a^(p-2) via 4-bit fixed windows
DEVNI fp fp_pow_window(fp a, const uint32_t *e) {
  fp tab[16];
  tab[0] = fp_one();
  tab[1] = a;
  #pragma unroll 1
  for (int i = 2; i < 16; i++) tab[i] = fp_mul(tab[i - 1], a);
  fp r = fp_one();
  #pragma unroll 1
  for (int i = 95; i >= 0; i--) {
    r = fp_sqr(r); r = fp_sqr(r); r = fp_sqr(r); r = fp_sqr(r);
    uint32_t nib = (e[i >> 3] >> ((i & 7) * 4)) & 15;
    if (nib) r = fp_mul(r, tab[nib]);
  }
  return r;
}
DEV fp fp_inv(fp a) {
  // p - 2
  const uint32_t e[12] = {0xffffaaa9u, 0xb9feffffu, 0xb153ffffu, 0x1eabfffeu, 0xf6b0f624u, 0x6730d2a0u,
                          0xf38512bfu, 0x64774b84u, 0x434bacd7u, 0x4b1ba7b6u, 0x397fe69au, 0x1a0111eau};
  return fp_pow_window(a, e);
}
// Variable-time inverse for public values: the optimized binary GCD of
// T. Pornin, "Optimized Binary GCD for Modular Inversion" (IACR ePrint
// 2020/972).  Each outer iteration runs 30 binary-GCD divsteps on 64-bit
// approximations of (a, b) (the low 31 bits and the top 33 bits of the longer
// value's length), then applies the resulting 2x2 matrix of factors in
// [-2^30, 2^30] to the full 381-bit a, b (exact division by 2^30) and to the
// companions u, v (Montgomery division by 2^30 mod p).  The invariants
// a c = y u and b c = y v (mod p), with u = c = R^2 mod p at the start, end at
// b = 1, v = R^2 / y; for the Montgomery residue y = aR that is a^-1 R, the
// Montgomery form of the inverse.  2 * 381 - 1 divsteps suffice (Pornin,
// section 3), so at most 26 outer iterations run; 32 only bound the loop.
// The accumulators stay inside int64: |a_i f| + |b_i g| < 2^63, and with the
// Montgomery term k p_i < 2^62 added, |u_i f| + |v_i g| + k p_i < 3 * 2^62.
namespace inv_detail {
constexpr uint32_t FP_NEG_PINV = 0xfffcfffdu;  // -p^-1 mod 2^32

// out = (a f + b g) / 2^30, exact; returns true when that was negative, in
// which case out holds its absolute value.
DEV bool lin_div30(const uint32_t *a, const uint32_t *b, int32_t f, int32_t g, uint32_t *out) {
  uint32_t r[13];
  int64_t c = 0;
#pragma unroll
  for (int i = 0; i < 12; i++) {
    const int64_t acc = c + (int64_t)a[i] * f + (int64_t)b[i] * g;
    r[i] = (uint32_t)acc;
    c = acc >> 32;
  }
  r[12] = (uint32_t)c;
#pragma unroll
  for (int i = 0; i < 12; i++) out[i] = __funnelshift_r(r[i], r[i + 1], 30);
  const bool neg = c < 0;
  if (neg) {
    uint64_t t = 1;
#pragma unroll
    for (int i = 0; i < 12; i++) {
      t += (uint32_t)~out[i];
      out[i] = (uint32_t)t;
      t >>= 32;
    }
  }
  return neg;
}

// out = (u f + v g) / 2^30 mod p, for u, v in [0, p); out in [0, p).
DEV void mod_div30(const uint32_t *u, const uint32_t *v, int32_t f, int32_t g, uint32_t *out) {
  const fp pm = FP_MOD_INIT;
  const uint32_t k = ((u[0] * (uint32_t)f + v[0] * (uint32_t)g) * FP_NEG_PINV) & 0x3fffffffu;
  uint32_t r[13];
  int64_t c = 0;
#pragma unroll
  for (int i = 0; i < 12; i++) {
    const int64_t acc = c + (int64_t)u[i] * f + (int64_t)v[i] * g + (int64_t)((uint64_t)k * pm.w[i]);
    r[i] = (uint32_t)acc;
    c = acc >> 32;
  }
  r[12] = (uint32_t)c;
#pragma unroll
  for (int i = 0; i < 12; i++) out[i] = __funnelshift_r(r[i], r[i + 1], 30);
  // out is in (-2p, 3p), as a 384-bit two's complement value: at most two
  // additions or two subtractions of p bring it into [0, p)
#pragma unroll 1
  for (int rep = 0; rep < 2 && (int32_t)out[11] < 0; rep++) {
    uint64_t t = 0;
#pragma unroll
    for (int i = 0; i < 12; i++) {
      t += (uint64_t)out[i] + pm.w[i];
      out[i] = (uint32_t)t;
      t >>= 32;
    }
  }
#pragma unroll 1
  for (int rep = 0; rep < 2; rep++) {
    uint32_t d[12];
    int64_t t = 0;
#pragma unroll
    for (int i = 0; i < 12; i++) {
      t += (int64_t)out[i] - pm.w[i];
      d[i] = (uint32_t)t;
      t >>= 32;
    }
    if (t < 0) break;
#pragma unroll
    for (int i = 0; i < 12; i++) out[i] = d[i];
  }
}
}  // namespace inv_detail

DEVNI fp fp_inv_vartime(fp y) {
  if (fp_is_zero(y)) return y;
  const fp pm = FP_MOD_INIT, r2 = FP_R2_INIT;
  uint32_t a[12], b[12], u[12], v[12];
#pragma unroll
  for (int i = 0; i < 12; i++) {
    a[i] = y.w[i];
    b[i] = pm.w[i];
    u[i] = r2.w[i];
    v[i] = 0;
  }
#pragma unroll 1
  for (int it = 0; it < 32; it++) {
    uint32_t any = 0;
#pragma unroll
    for (int i = 0; i < 12; i++) any |= a[i];
    if (any == 0) break;
    // n = max(bit length of a, of b, 64); s = n - 33
    int top = 1;
    uint32_t mt = a[1] | b[1];
#pragma unroll
    for (int i = 2; i < 12; i++) {
      const uint32_t m = a[i] | b[i];
      if (m) {
        top = i;
        mt = m;
      }
    }
    const int n = max(32 * top + 32 - __clz(mt), 64), s = n - 33, q = s >> 5, sh = s & 31;
    uint32_t a0 = 0, a1 = 0, a2 = 0, b0 = 0, b1 = 0, b2 = 0;
#pragma unroll
    for (int i = 0; i < 12; i++) {
      if (i == q) { a0 = a[i]; b0 = b[i]; }
      if (i == q + 1) { a1 = a[i]; b1 = b[i]; }
      if (i == q + 2) { a2 = a[i]; b2 = b[i]; }
    }
    // top 33 bits (bits s .. s+32) above the low 31 bits
    const uint32_t ta = __funnelshift_r(a0, a1, sh), tb = __funnelshift_r(b0, b1, sh);
    const uint32_t ha = __funnelshift_r(a1, a2, sh) & 1u, hb = __funnelshift_r(b1, b2, sh) & 1u;
    uint64_t xa = ((uint64_t)((ta >> 1) | (ha << 31)) << 32) | ((ta << 31) | (a[0] & 0x7fffffffu));
    uint64_t xb = ((uint64_t)((tb >> 1) | (hb << 31)) << 32) | ((tb << 31) | (b[0] & 0x7fffffffu));
    int32_t f0 = 1, g0 = 0, f1 = 0, g1 = 1;
#pragma unroll
    for (int j = 0; j < 30; j++) {
      if (xa & 1) {
        if (xa < xb) {
          const uint64_t tx = xa; xa = xb; xb = tx;
          const int32_t tf = f0; f0 = f1; f1 = tf;
          const int32_t tg = g0; g0 = g1; g1 = tg;
        }
        xa -= xb;
        f0 -= f1;
        g0 -= g1;
      }
      xa >>= 1;
      f1 += f1;
      g1 += g1;
    }
    uint32_t na[12], nb[12];
    if (inv_detail::lin_div30(a, b, f0, g0, na)) { f0 = -f0; g0 = -g0; }
    if (inv_detail::lin_div30(a, b, f1, g1, nb)) { f1 = -f1; g1 = -g1; }
    uint32_t nu[12], nv[12];
    inv_detail::mod_div30(u, v, f0, g0, nu);
    inv_detail::mod_div30(u, v, f1, g1, nv);
#pragma unroll
    for (int i = 0; i < 12; i++) {
      a[i] = na[i];
      b[i] = nb[i];
      u[i] = nu[i];
      v[i] = nv[i];
    }
  }
  fp r;
#pragma unroll
  for (int i = 0; i < 12; i++) r.w[i] = v[i];
  return r;
}
// sqrt for p = 3 mod 4: s = a^((p+1)/4); returns false if a is not a square.
DEV bool fp_sqrt(fp a, fp &out) {
  const uint32_t e[12] = {0xffffeaabu, 0xee7fbfffu, 0xac54ffffu, 0x07aaffffu, 0x3dac3d89u, 0xd9cc34a8u,
                          0x3ce144afu, 0xd91dd2e1u, 0x90d2eb35u, 0x92c6e9edu, 0x8e5ff9a6u, 0x0680447au};
  fp s = fp_pow_window(a, e);
  out = s;
  return fp_eq(fp_sqr(s), a);
}
// canonical value > (p-1)/2 ?
DEVNI bool fp_lex_largest(fp a) {
  fp c = fp_from_mont(a);
  // (p-1)/2
  const uint32_t h[12] = {0xffffd555u, 0xdcff7fffu, 0x58a9ffffu, 0x0f55ffffu, 0x7b587b12u, 0xb3986950u,
                          0x79c2895fu, 0xb23ba5c2u, 0x21a5d66bu, 0x258dd3dbu, 0x1cbff34du, 0x0d0088f5u};
  _Pragma("unroll") for (int i = 11; i >= 0; i--) {
    if (c.w[i] != h[i]) return c.w[i] > h[i];
  }
  return false;
}
DEV bool fp_parity(const fp &a) { return fp_from_mont(a).w[0] & 1; }
// 48-byte big-endian canonical encoding (flag bits must be cleared by the caller)
DEVNI bool fp_from_be48(const uint8_t *b, fp &out) {
  fp c;
  _Pragma("unroll") for (int i = 0; i < 12; i++) {
    const uint8_t *q = b + (11 - i) * 4;
    c.w[i] = ((uint32_t)q[0] << 24) | ((uint32_t)q[1] << 16) | ((uint32_t)q[2] << 8) | q[3];
  }
  if (!fp_lt_mod(c)) return false;
  out = fp_to_mont(c);
  return true;
}
DEVNI void fp_to_be48(fp a, uint8_t *b) {
  fp c = fp_from_mont(a);
  _Pragma("unroll") for (int i = 0; i < 12; i++) {
    uint8_t *q = b + (11 - i) * 4;
    q[0] = (uint8_t)(c.w[i] >> 24); q[1] = (uint8_t)(c.w[i] >> 16);
    q[2] = (uint8_t)(c.w[i] >> 8); q[3] = (uint8_t)c.w[i];
  }
}
// OS2IP(64 bytes) mod p: value = hi*2^384 + lo, hi < 2^128
DEVNI fp fp_from_be64_mod(const uint8_t *b) {
  fp lo, hi = fp_zero();
  _Pragma("unroll") for (int i = 0; i < 12; i++) {
    const uint8_t *q = b + 16 + (11 - i) * 4;
    lo.w[i] = ((uint32_t)q[0] << 24) | ((uint32_t)q[1] << 16) | ((uint32_t)q[2] << 8) | q[3];
  }
  _Pragma("unroll") for (int i = 0; i < 4; i++) {
    const uint8_t *q = b + (3 - i) * 4;
    hi.w[i] = ((uint32_t)q[0] << 24) | ((uint32_t)q[1] << 16) | ((uint32_t)q[2] << 8) | q[3];
  }
  // lo < 2^384 < 10p: subtract p while lo >= p
  const fp m = FP_MOD_INIT;
  #pragma unroll 1
  for (int k = 0; k < 10 && !fp_lt_mod(lo); k++) {
    uint32_t borrow = 0;
    _Pragma("unroll") for (int i = 0; i < 12; i++) {
      uint64_t d = (uint64_t)lo.w[i] - m.w[i] - borrow;
      lo.w[i] = (uint32_t)d;
      borrow = (uint32_t)(d >> 63);
    }
  }
  // hi*2^384 mod p = mont(hi * R^2) (a canonical value); both terms canonical -> add in canonical domain
  const fp r2 = FP_R2_INIT;
  fp h = fp_mul(hi, r2);
  fp s = fp_add(h, lo);
  return fp_to_mont(s);
}
DEV fp fp_select(bool c, const fp &a, const fp &b) {
  fp r;
  _Pragma("unroll") for (int i = 0; i < 12; i++) r.w[i] = c ? a.w[i] : b.w[i];
  return r;
}

// ------------------------------------------------------------------ Fr
DEV fr fr_zero() { fr r; _Pragma("unroll") for (int i = 0; i < 8; i++) r.w[i] = 0; return r; }
DEV fr fr_one() { const fr r = FR_ONE_INIT; return r; }
DEV bool fr_is_zero(const fr &a) {
  uint32_t x = 0;
  _Pragma("unroll") for (int i = 0; i < 8; i++) x |= a.w[i];
  return x == 0;
}
DEV bool fr_eq(const fr &a, const fr &b) {
  uint32_t x = 0;
  _Pragma("unroll") for (int i = 0; i < 8; i++) x |= a.w[i] ^ b.w[i];
  return x == 0;
}
DEV fr fr_add(const fr &a, const fr &b) { fr r; fr_add_raw(r.w, a.w, b.w); return r; }
DEV fr fr_sub(const fr &a, const fr &b) { fr r; fr_sub_raw(r.w, a.w, b.w); return r; }
// Montgomery product mod r (R = 2^256, fully reduced): the carry-save rows of
// fp_mul_inl over 8 limbs, in PTX for the same reason (the carry additions stay
// on the ALU pipe).  Bounds: a, b < r; partial sums below 2^64; result below 2r.
DEV fr fr_mul_inl(const fr &a, const fr &b) {
  const fr rm = FR_MOD_INIT;
  uint32_t lo[8], hi[8];
#pragma unroll
  for (int j = 0; j < 8; j++) lo[j] = hi[j] = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint32_t bi = b.w[i];
#pragma unroll
    for (int j = 0; j < 8; j++)
      asm("mad.lo.cc.u32 %0, %2, %3, %0;\n\tmadc.hi.u32 %1, %2, %3, %1;"
          : "+r"(lo[j]), "+r"(hi[j])
          : "r"(a.w[j]), "r"(bi));
    uint32_t nl[8], nh[8];
    nl[0] = lo[0];
    nh[0] = 0;
#pragma unroll
    for (int j = 1; j < 8; j++)
      asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=r"(nl[j]), "=r"(nh[j]) : "r"(lo[j]), "r"(hi[j - 1]));
    const uint32_t n8 = hi[7];
    const uint32_t m = nl[0] * FR_PINV;
#pragma unroll
    for (int j = 0; j < 8; j++)
      asm("mad.lo.cc.u32 %0, %2, %3, %0;\n\tmadc.hi.u32 %1, %2, %3, %1;"
          : "+r"(nl[j]), "+r"(nh[j])
          : "r"(m), "r"(rm.w[j]));
#pragma unroll
    for (int j = 0; j < 7; j++)
      asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=r"(lo[j]), "=r"(hi[j]) : "r"(nl[j + 1]), "r"(nh[j]));
    asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=r"(lo[7]), "=r"(hi[7]) : "r"(n8), "r"(nh[7]));
  }
  uint32_t t[8];
  asm("add.cc.u32 %0, %8, 0;\n\taddc.cc.u32 %1, %9, %16;\n\taddc.cc.u32 %2, %10, %17;\n\taddc.cc.u32 %3, %11, %18;\n\t"
      "addc.cc.u32 %4, %12, %19;\n\taddc.cc.u32 %5, %13, %20;\n\taddc.cc.u32 %6, %14, %21;\n\taddc.u32 %7, %15, %22;"
      : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]), "=r"(t[7])
      : "r"(lo[0]), "r"(lo[1]), "r"(lo[2]), "r"(lo[3]), "r"(lo[4]), "r"(lo[5]), "r"(lo[6]), "r"(lo[7]),
        "r"(hi[0]), "r"(hi[1]), "r"(hi[2]), "r"(hi[3]), "r"(hi[4]), "r"(hi[5]), "r"(hi[6]));
  fr r;
  fr_reduce_once(r.w, t);
  return r;
}
// The CIOS form it replaced (carry chains of field_ptx.cuh), kept for the tests.
DEV fr fr_mul_cios_inl(const fr &a, const fr &b) {
  uint32_t t[17];
  _Pragma("unroll") for (int i = 0; i < 9; i++) t[i] = 0;
  _Pragma("unroll") for (int i = 0; i < 8; i++) {
    t[i + 8] = 0;
    fr_cios_row(&t[i], a.w, b.w[i]);
  }
  fr r;
  fr_reduce_once(r.w, &t[8]);
  return r;
}
DEVNI fr fr_mul(fr a, fr b) { return fr_mul_inl(a, b); }
DEV fr fr_to_mont(const fr &a) { const fr r2 = FR_R2_INIT; return fr_mul(a, r2); }
DEV fr fr_from_mont(const fr &a) { fr one = fr_zero(); one.w[0] = 1; return fr_mul(a, one); }
DEV bool fr_lt_mod(const fr &a) {
  const fr m = FR_MOD_INIT;
  _Pragma("unroll") for (int i = 7; i >= 0; i--) {
    if (a.w[i] != m.w[i]) return a.w[i] < m.w[i];
  }
  return false;
}
DEVNI fr fr_inv(fr a) {
  // r - 2
  const uint32_t e[8] = {0xffffffffu, 0xfffffffeu, 0xfffe5bfeu, 0x53bda402u,
                         0x09a1d805u, 0x3339d808u, 0x299d7d48u, 0x73eda753u};
  fr tab[16];
  tab[0] = fr_one();
  tab[1] = a;
  #pragma unroll 1
  for (int i = 2; i < 16; i++) tab[i] = fr_mul(tab[i - 1], a);
  fr r = fr_one();
  #pragma unroll 1
  for (int i = 63; i >= 0; i--) {
    r = fr_mul(r, r); r = fr_mul(r, r); r = fr_mul(r, r); r = fr_mul(r, r);
    uint32_t nib = (e[i >> 3] >> ((i & 7) * 4)) & 15;
    if (nib) r = fr_mul(r, tab[nib]);
  }
  return r;
}
// canonical 32-byte big-endian -> raw canonical words; false if >= r
DEV bool fr_raw_from_be32(const uint8_t *b, fr &out) {
  _Pragma("unroll") for (int i = 0; i < 8; i++) {
    const uint8_t *q = b + (7 - i) * 4;
    out.w[i] = ((uint32_t)q[0] << 24) | ((uint32_t)q[1] << 16) | ((uint32_t)q[2] << 8) | q[3];
  }
  return fr_lt_mod(out);
}
DEV void fr_raw_to_be32(const fr &c, uint8_t *b) {
  _Pragma("unroll") for (int i = 0; i < 8; i++) {
    uint8_t *q = b + (7 - i) * 4;
    q[0] = (uint8_t)(c.w[i] >> 24); q[1] = (uint8_t)(c.w[i] >> 16);
    q[2] = (uint8_t)(c.w[i] >> 8); q[3] = (uint8_t)c.w[i];
  }
}
// OS2IP(48 bytes) mod r (Scalar::from_okm): value = hi*2^256 + lo, hi < 2^128.  Returns
// the CANONICAL (non-Montgomery) residue.
DEVNI fr fr_raw_from_okm(const uint8_t *b) {
  fr lo, hi = fr_zero();
  _Pragma("unroll") for (int i = 0; i < 8; i++) {
    const uint8_t *q = b + 16 + (7 - i) * 4;
    lo.w[i] = ((uint32_t)q[0] << 24) | ((uint32_t)q[1] << 16) | ((uint32_t)q[2] << 8) | q[3];
  }
  _Pragma("unroll") for (int i = 0; i < 4; i++) {
    const uint8_t *q = b + (3 - i) * 4;
    hi.w[i] = ((uint32_t)q[0] << 24) | ((uint32_t)q[1] << 16) | ((uint32_t)q[2] << 8) | q[3];
  }
  const fr m = FR_MOD_INIT;
  #pragma unroll 1
  for (int k = 0; k < 3 && !fr_lt_mod(lo); k++) {
    uint32_t borrow = 0;
    _Pragma("unroll") for (int i = 0; i < 8; i++) {
      uint64_t d = (uint64_t)lo.w[i] - m.w[i] - borrow;
      lo.w[i] = (uint32_t)d;
      borrow = (uint32_t)(d >> 63);
    }
  }
  const fr r2 = FR_R2_INIT;
  fr h = fr_mul(hi, r2);  // hi * 2^256 mod r, canonical
  return fr_add(h, lo);
}

// ------------------------------------------------------------------ Fp2
DEV fp2 fp2_zero() { return {fp_zero(), fp_zero()}; }
DEV fp2 fp2_one() { return {fp_one(), fp_zero()}; }
DEV bool fp2_is_zero(const fp2 &a) { return fp_is_zero(a.c0) && fp_is_zero(a.c1); }
DEV bool fp2_eq(const fp2 &a, const fp2 &b) { return fp_eq(a.c0, b.c0) && fp_eq(a.c1, b.c1); }
DEV fp2 fp2_add(const fp2 &a, const fp2 &b) { return {fp_add(a.c0, b.c0), fp_add(a.c1, b.c1)}; }
DEV fp2 fp2_sub(const fp2 &a, const fp2 &b) { return {fp_sub(a.c0, b.c0), fp_sub(a.c1, b.c1)}; }
DEV fp2 fp2_dbl(const fp2 &a) { return fp2_add(a, a); }
DEV fp2 fp2_neg(const fp2 &a) { return {fp_neg(a.c0), fp_neg(a.c1)}; }
DEV fp2 fp2_conj(const fp2 &a) { return {a.c0, fp_neg(a.c1)}; }
DEV fp2 fp2_mul_inl(fp2 a, fp2 b) {
  fp t0 = fp_mul(a.c0, b.c0), t1 = fp_mul(a.c1, b.c1);
  fp t2 = fp_mul(fp_add(a.c0, a.c1), fp_add(b.c0, b.c1));
  return {fp_sub(t0, t1), fp_sub(fp_sub(t2, t0), t1)};
}
DEV fp2 fp2_sqr_inl(fp2 a) {
  // (a0 + a1)(a0 - a1) + 2 a0 a1 u
  fp t = fp_mul(a.c0, a.c1);
  return {fp_mul(fp_add(a.c0, a.c1), fp_sub(a.c0, a.c1)), fp_dbl(t)};
}
DEVNI fp2 fp2_mul(fp2 a, fp2 b) { return fp2_mul_inl(a, b); }
DEVNI fp2 fp2_sqr(fp2 a) { return fp2_sqr_inl(a); }
DEV fp2 fp2_mul_fp(const fp2 &a, const fp &s) { return {fp_mul(a.c0, s), fp_mul(a.c1, s)}; }
DEV fp2 fp2_mul_xi(const fp2 &a) { return {fp_sub(a.c0, a.c1), fp_add(a.c0, a.c1)}; }  // *(1+u)
DEV fp2 fp2_inv(fp2 a) {
  fp n = fp_inv(fp_add(fp_sqr(a.c0), fp_sqr(a.c1)));
  return {fp_mul(a.c0, n), fp_neg(fp_mul(a.c1, n))};
}
DEV bool fp2_lex_largest(const fp2 &a) {
  if (!fp_is_zero(a.c1)) return fp_lex_largest(a.c1);
  return fp_lex_largest(a.c0);
}
// square root in Fp2 via the norm: for a = a0 + a1 u, sqrt(a) = x0 + x1 u with
// x0^2 = (a0 +- sqrt(a0^2+a1^2))/2, x1 = a1/(2 x0).
DEV bool fp2_sqrt(fp2 a, fp2 &out) {
  if (fp_is_zero(a.c1)) {
    fp s;
    if (fp_sqrt(a.c0, s)) { out = {s, fp_zero()}; return true; }
    if (fp_sqrt(fp_neg(a.c0), s)) { out = {fp_zero(), s}; return true; }
    return false;
  }
  fp n = fp_add(fp_sqr(a.c0), fp_sqr(a.c1)), s;
  if (!fp_sqrt(n, s)) return false;
  const fp inv2 = C_FP_INV2;
  fp t = fp_mul(fp_add(a.c0, s), inv2), x0;
  if (!fp_sqrt(t, x0)) {
    t = fp_mul(fp_sub(a.c0, s), inv2);
    if (!fp_sqrt(t, x0)) return false;
  }
  fp x1 = fp_mul(a.c1, fp_inv(fp_dbl(x0)));
  fp2 r = {x0, x1};
  if (!fp2_eq(fp2_sqr(r), a)) return false;
  out = r;
  return true;
}

// ------------------------------------------------------------------ Fp6
DEV fp6 fp6_zero() { return {fp2_zero(), fp2_zero(), fp2_zero()}; }
DEV fp6 fp6_one() { return {fp2_one(), fp2_zero(), fp2_zero()}; }
DEV fp6 fp6_add(const fp6 &a, const fp6 &b) { return {fp2_add(a.c0, b.c0), fp2_add(a.c1, b.c1), fp2_add(a.c2, b.c2)}; }
DEV fp6 fp6_sub(const fp6 &a, const fp6 &b) { return {fp2_sub(a.c0, b.c0), fp2_sub(a.c1, b.c1), fp2_sub(a.c2, b.c2)}; }
DEV fp6 fp6_neg(const fp6 &a) { return {fp2_neg(a.c0), fp2_neg(a.c1), fp2_neg(a.c2)}; }
DEV bool fp6_eq(const fp6 &a, const fp6 &b) { return fp2_eq(a.c0, b.c0) && fp2_eq(a.c1, b.c1) && fp2_eq(a.c2, b.c2); }
DEV fp6 fp6_mul(fp6 a, fp6 b) {
  fp2 a0 = fp2_mul(a.c0, b.c0), a1 = fp2_mul(a.c1, b.c1), a2 = fp2_mul(a.c2, b.c2);
  fp2 t0 = fp2_add(fp2_mul_xi(fp2_sub(fp2_sub(fp2_mul(fp2_add(a.c1, a.c2), fp2_add(b.c1, b.c2)), a1), a2)), a0);
  fp2 t1 = fp2_add(fp2_sub(fp2_sub(fp2_mul(fp2_add(a.c0, a.c1), fp2_add(b.c0, b.c1)), a0), a1), fp2_mul_xi(a2));
  fp2 t2 = fp2_add(fp2_sub(fp2_sub(fp2_mul(fp2_add(a.c0, a.c2), fp2_add(b.c0, b.c2)), a0), a2), a1);
  return {t0, t1, t2};
}
DEV fp6 fp6_mul_v(const fp6 &a) { return {fp2_mul_xi(a.c2), a.c0, a.c1}; }
DEV fp6 fp6_inv(fp6 a) {
  fp2 t0 = fp2_sub(fp2_sqr(a.c0), fp2_mul_xi(fp2_mul(a.c1, a.c2)));
  fp2 t1 = fp2_sub(fp2_mul_xi(fp2_sqr(a.c2)), fp2_mul(a.c0, a.c1));
  fp2 t2 = fp2_sub(fp2_sqr(a.c1), fp2_mul(a.c0, a.c2));
  fp2 d = fp2_add(fp2_mul(a.c0, t0), fp2_mul_xi(fp2_add(fp2_mul(a.c2, t1), fp2_mul(a.c1, t2))));
  d = fp2_inv(d);
  return {fp2_mul(t0, d), fp2_mul(t1, d), fp2_mul(t2, d)};
}

// ------------------------------------------------------------------ Fp12
DEV fp12 fp12_one() { return {fp6_one(), fp6_zero()}; }
DEV bool fp12_eq(const fp12 &a, const fp12 &b) { return fp6_eq(a.c0, b.c0) && fp6_eq(a.c1, b.c1); }
DEV bool fp12_is_one(const fp12 &a) { return fp12_eq(a, fp12_one()); }
DEV fp12 fp12_mul(fp12 a, fp12 b) {
  fp6 t0 = fp6_mul(a.c0, b.c0), t1 = fp6_mul(a.c1, b.c1);
  fp6 t2 = fp6_sub(fp6_sub(fp6_mul(fp6_add(a.c0, a.c1), fp6_add(b.c0, b.c1)), t0), t1);
  return {fp6_add(t0, fp6_mul_v(t1)), t2};
}
DEV fp12 fp12_sqr(fp12 a) {
  // (a0 + a1 w)^2 = (a0^2 + v a1^2) + 2 a0 a1 w ; via (a0+a1)(a0+v a1) - a0a1 - v a0a1
  fp6 ab = fp6_mul(a.c0, a.c1);
  fp6 t = fp6_mul(fp6_add(a.c0, a.c1), fp6_add(a.c0, fp6_mul_v(a.c1)));
  fp6 c0 = fp6_sub(fp6_sub(t, ab), fp6_mul_v(ab));
  return {c0, fp6_add(ab, ab)};
}
DEV fp12 fp12_conj(const fp12 &a) { return {a.c0, fp6_neg(a.c1)}; }
DEV fp12 fp12_inv(fp12 a) {
  fp6 t = fp6_inv(fp6_sub(fp6_mul(a.c0, a.c0), fp6_mul_v(fp6_mul(a.c1, a.c1))));
  return {fp6_mul(a.c0, t), fp6_neg(fp6_mul(a.c1, t))};
}
// Frobenius x -> x^p: conjugate each Fp2 coefficient and scale the basis
// element w^k by gamma_k = xi^(k(p-1)/6).
DEV fp12 fp12_frobenius(fp12 a) {
  const fp2 g[6] = C_FROB_GAMMA;
  fp12 r;
  r.c0.c0 = fp2_conj(a.c0.c0);
  r.c0.c1 = fp2_mul(fp2_conj(a.c0.c1), g[2]);
  r.c0.c2 = fp2_mul(fp2_conj(a.c0.c2), g[4]);
  r.c1.c0 = fp2_mul(fp2_conj(a.c1.c0), g[1]);
  r.c1.c1 = fp2_mul(fp2_conj(a.c1.c1), g[3]);
  r.c1.c2 = fp2_mul(fp2_conj(a.c1.c2), g[5]);
  return r;
}
