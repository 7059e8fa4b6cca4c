// hash_to_curve for G1, suite BLS12381G1_XMD:SHA-256_SSWU_RO_ (RFC 9380),
// used to build the BBS message generators on the device
// (create_generators, crates/cubbs-bbs-protocol/src/bbsplus/generators.rs:119-146).
// The 11-isogeny coefficients come from gen_curve_constants.py, which derives
// them from the curve (Velu on the rational 11-torsion kernel of E').
#pragma once
#include "curve.cuh"
#include "suite.cuh"

DEV fp poly_eval(const fp *c, int n, const fp &x) {
  fp r = c[n - 1];
  #pragma unroll 1
  for (int i = n - 2; i >= 0; i--) r = fp_add(fp_mul(r, x), c[i]);
  return r;
}

// simplified SWU onto E': y^2 = x^3 + A'x + B' (RFC 9380 6.6.2), then the isogeny onto E.
DEV g1a map_to_curve_g1(fp u) {
  const fp A = C_SSWU_A, B = C_SSWU_B, Z = C_SSWU_Z;
  const fp mBA = C_SSWU_MINUS_B_OVER_A, BZA = C_SSWU_B_OVER_ZA;
  fp u2 = fp_sqr(u);
  fp zu2 = fp_mul(Z, u2);
  fp tv1 = fp_add(fp_sqr(zu2), zu2);
  fp x1 = fp_is_zero(tv1) ? BZA : fp_mul(mBA, fp_add(fp_one(), fp_inv(tv1)));
  fp gx1 = fp_add(fp_mul(fp_add(fp_sqr(x1), A), x1), B);
  fp x, y;
  if (fp_sqrt(gx1, y)) {
    x = x1;
  } else {
    x = fp_mul(zu2, x1);
    fp gx2 = fp_add(fp_mul(fp_add(fp_sqr(x), A), x), B);
    fp_sqrt(gx2, y);
  }
  if (fp_parity(u) != fp_parity(y)) y = fp_neg(y);
  const fp xnum[C_ISO_XNUM_LEN] = C_ISO_XNUM;
  const fp xden[C_ISO_XDEN_LEN] = C_ISO_XDEN;
  const fp ynum[C_ISO_YNUM_LEN] = C_ISO_YNUM;
  const fp yden[C_ISO_YDEN_LEN] = C_ISO_YDEN;
  fp xn = poly_eval(xnum, C_ISO_XNUM_LEN, x), xd = poly_eval(xden, C_ISO_XDEN_LEN, x);
  fp yn = poly_eval(ynum, C_ISO_YNUM_LEN, x), yd = poly_eval(yden, C_ISO_YDEN_LEN, x);
  // one inversion for both denominators
  fp inv = fp_inv(fp_mul(xd, yd));
  g1a r;
  r.x = fp_mul(xn, fp_mul(inv, yd));
  r.y = fp_mul(fp_mul(y, yn), fp_mul(inv, xd));
  return r;
}

// hash_to_curve(msg, dst) with the expander of suite S (expand_message_xmd /
// expand_message_xof, 128 bytes): returns an XYZZ point (cofactor cleared with
// h_eff = |z| + 1).
template <int S = SUITE_SHA256>
DEV g1 hash_to_curve_g1(const uint8_t *msg, uint32_t len, const uint8_t *dst, uint32_t dlen) {
  hash_ctx<S> c;
  msg_begin(c);
  msg_bytes(c, msg, len);
  uint8_t ub[128];
  msg_finish(c, dst, dlen, 128, ub);
  g1a q0 = map_to_curve_g1(fp_from_be64_mod(ub));
  g1a q1 = map_to_curve_g1(fp_from_be64_mod(ub + 64));
  g1 r = g1_add_aff(g1_from_aff(q0), q1);
  return g1_add(g1_mul_zabs(r), r);
}
