// Team-parallel pairing check: 16 lanes (half a warp) evaluate one
//     e(P_a, Q_a) * e(P_b, Q_b) == 1
// with the Miller loop over precomputed lines and the final exponentiation
// of pairing.cuh, split at Fp2 granularity.  The Fp12 value lives in shared
// memory as six Fp2 slots
//     slot 0..2 = c0.c0, c0.c1, c0.c2   slot 3..5 = c1.c0, c1.c1, c1.c2
// and each operation runs as rounds:  every busy lane forms its operands
// from the slots and computes one Fp2 product; then a few lanes assemble the
// result slots from the products.  A lone warp already fills its SM
// sub-partition's multiply issue with one Fp product at a time, so spreading
// one pairing over 16 lanes divides its latency by roughly the number of
// independent Fp2 products per operation (12 for a squaring, 13 for a line,
// 9 for a cyclotomic squaring, 18 for a product).
//
// Formulas: Fp6/Fp12 Karatsuba as in field.cuh; the line product as
// fp12_mul_line; the cyclotomic squaring is Granger-Scott (compressed Fp4
// squarings, "Faster squaring in the cyclotomic subgroup of sixth degree
// extensions", PKC 2010); the final exponentiation is final_exponentiation of
// pairing.cuh with every exp-by-z squaring replaced by the cyclotomic one.
// Results equal the single-thread kernel exactly (all values fully reduced).
#pragma once
#include "pairing.cuh"

#define PT_LANES 16

// Per-team shared memory.
struct PtShared {
  fp2 S[6][6];   // six Fp12 slots: F, T, A, X, R, U
  fp2 Z[18];     // products of the current round
  fp2 W[9];      // assembled Fp6 coefficients
  fp Wf[6];      // Fp-level products
  fp2 BX[2];     // B * xP of the doubling line of each pair
  fp2 BXA[2];    // B * xP of the addition line of each pair
  fp PX[2], PY[2];
};

enum { PT_F = 0, PT_T = 1, PT_A = 2, PT_X = 3, PT_R = 4, PT_U = 5 };

struct PtCtx {
  int lane;
  unsigned mask;
  PtShared *sm;
  DEV void sync() const { __syncwarp(mask); }
};

// Karatsuba Fp6 product list: for a*b the products are
//   P0 = a0 b0, P1 = a1 b1, P2 = a2 b2, P3 = (a1+a2)(b1+b2), P4 = (a0+a1)(b0+b1), P5 = (a0+a2)(b0+b2)
DEV void pt_kara_pick(int j, const fp2 &a0, const fp2 &a1, const fp2 &a2, const fp2 &b0, const fp2 &b1,
                      const fp2 &b2, fp2 &x, fp2 &y) {
  switch (j) {
    case 0: x = a0; y = b0; break;
    case 1: x = a1; y = b1; break;
    case 2: x = a2; y = b2; break;
    case 3: x = fp2_add(a1, a2); y = fp2_add(b1, b2); break;
    case 4: x = fp2_add(a0, a1); y = fp2_add(b0, b1); break;
    default: x = fp2_add(a0, a2); y = fp2_add(b0, b2); break;
  }
}
// coefficient k of the Fp6 product from its six Karatsuba products
DEV fp2 pt_kara_assemble(int k, const fp2 *P) {
  if (k == 0) return fp2_add(P[0], fp2_mul_xi(fp2_sub(fp2_sub(P[3], P[1]), P[2])));
  if (k == 1) return fp2_add(fp2_sub(fp2_sub(P[4], P[0]), P[1]), fp2_mul_xi(P[2]));
  return fp2_add(fp2_sub(fp2_sub(P[5], P[0]), P[2]), P[1]);
}

DEVNI void pt_set_one(PtCtx c, int slot) {
  if (c.lane < 6) c.sm->S[slot][c.lane] = c.lane == 0 ? fp2_one() : fp2_zero();
  c.sync();
}
DEVNI void pt_copy(PtCtx c, int dst, int src) {
  if (c.lane < 6) c.sm->S[dst][c.lane] = c.sm->S[src][c.lane];
  c.sync();
}
DEVNI void pt_conj(PtCtx c, int dst, int src) {
  if (c.lane < 6) {
    fp2 v = c.sm->S[src][c.lane];
    c.sm->S[dst][c.lane] = c.lane < 3 ? v : fp2_neg(v);
  }
  c.sync();
}
// dst = src^p: conjugate every coefficient, scale slot k by its gamma
// (each lane reads and writes only its own slot, so dst may alias src)
DEVNI void pt_frob(PtCtx c, int dst, int src) {
  if (c.lane < 6) {
    const fp2 g[6] = C_FROB_GAMMA;
    const int gi[6] = {0, 2, 4, 1, 3, 5};
    fp2 v = fp2_conj(c.sm->S[src][c.lane]);
    if (c.lane > 0) v = fp2_mul(v, g[gi[c.lane]]);
    c.sm->S[dst][c.lane] = v;
  }
  c.sync();
}

// Every lane of a round selects its operands (cheap, divergent) and then all
// lanes make the same fp2_mul call, so the products of a round run as one
// SIMT instruction stream.  `side(s, x, y)` lets the lanes beyond the
// operation's own products compute other Fp2 products (the B * xP factors of
// the next lines) in the same call: it sets the operands and returns where to
// store the product, or nullptr.

// S = S^2 (general Fp12 squaring, Miller loop); side lanes 12..15.
template <typename Side>
DEV void pt_sqr(const PtCtx &c, int s, Side side) {
  fp2 *S = c.sm->S[s];
  const int l = c.lane;
  fp2 x = fp2_zero(), y = fp2_zero();
  fp2 *dst = nullptr;
  if (l < 6) {  // ab = c0 * c1
    pt_kara_pick(l, S[0], S[1], S[2], S[3], S[4], S[5], x, y);
    dst = &c.sm->Z[l];
  } else if (l < 12) {  // (c0 + c1) * (c0 + v c1),  v c1 = (xi c12, c10, c11)
    fp2 a0 = fp2_add(S[0], S[3]), a1 = fp2_add(S[1], S[4]), a2 = fp2_add(S[2], S[5]);
    fp2 b0 = fp2_add(S[0], fp2_mul_xi(S[5])), b1 = fp2_add(S[1], S[3]), b2 = fp2_add(S[2], S[4]);
    pt_kara_pick(l - 6, a0, a1, a2, b0, b1, b2, x, y);
    dst = &c.sm->Z[l];
  } else {
    dst = side(l - 12, x, y);
  }
  const fp2 z = fp2_mul(x, y);
  if (dst) *dst = z;
  c.sync();
  if (l < 6) c.sm->W[l] = pt_kara_assemble(l % 3, c.sm->Z + (l < 3 ? 0 : 6));  // r = ab, t
  c.sync();
  if (l < 6) {
    const fp2 *r = c.sm->W, *t = c.sm->W + 3;
    fp2 o;
    switch (l) {
      case 0: o = fp2_sub(fp2_sub(t[0], r[0]), fp2_mul_xi(r[2])); break;
      case 1: o = fp2_sub(fp2_sub(t[1], r[1]), r[0]); break;
      case 2: o = fp2_sub(fp2_sub(t[2], r[2]), r[1]); break;
      default: o = fp2_dbl(r[l - 3]); break;
    }
    S[l] = o;
  }
  c.sync();
}

// S *= A + (B xP) v + yP v w  with Bx = B xP from shared memory; side lanes 13..15.
template <typename Side>
DEV void pt_line(const PtCtx &c, int s, const fp2 &A, const fp2 *Bxp, const fp *yPp, Side side) {
  fp2 *S = c.sm->S[s];
  const int l = c.lane;
  fp2 x = fp2_zero(), y = fp2_zero();
  fp2 *dst = l < 13 ? &c.sm->Z[l] : nullptr;
  if (l < 5) {  // t0 = f0 * (A, Bx, 0)
    const fp2 Bx = *Bxp;
    switch (l) {
      case 0: x = S[0]; y = A; break;
      case 1: x = S[1]; y = Bx; break;
      case 2: x = S[2]; y = Bx; break;
      case 3: x = fp2_add(S[0], S[1]); y = fp2_add(A, Bx); break;
      default: x = S[2]; y = A; break;
    }
  } else if (l < 8) {  // t1 = f1 * yP v : products f12 yP, f10 yP, f11 yP
    const int src[3] = {5, 3, 4};
    x = S[src[l - 5]];
    y.c0 = *yPp;
  } else if (l < 13) {  // t2 = (f0 + f1) * (A, Bx + yP, 0)
    fp2 B2 = *Bxp;
    B2.c0 = fp_add(B2.c0, *yPp);
    switch (l) {
      case 8: x = fp2_add(S[0], S[3]); y = A; break;
      case 9: x = fp2_add(S[1], S[4]); y = B2; break;
      case 10: x = fp2_add(S[2], S[5]); y = B2; break;
      case 11: x = fp2_add(fp2_add(S[0], S[3]), fp2_add(S[1], S[4])); y = fp2_add(A, B2); break;
      default: x = fp2_add(S[2], S[5]); y = A; break;
    }
  } else {
    dst = side(l - 13, x, y);
  }
  const fp2 z = fp2_mul(x, y);
  if (dst) *dst = z;
  c.sync();
  if (l < 6) {
    const fp2 *Z = c.sm->Z;
    fp2 o;
    switch (l) {
      case 0: o = fp2_add(Z[0], fp2_mul_xi(fp2_add(Z[2], Z[7]))); break;
      case 1: o = fp2_add(fp2_sub(fp2_sub(Z[3], Z[0]), Z[1]), fp2_mul_xi(Z[5])); break;
      case 2: o = fp2_add(fp2_add(Z[1], Z[4]), Z[6]); break;
      case 3: o = fp2_sub(fp2_sub(fp2_add(Z[8], fp2_mul_xi(Z[10])), fp2_add(Z[0], fp2_mul_xi(Z[2]))), fp2_mul_xi(Z[5])); break;
      case 4: o = fp2_sub(fp2_sub(fp2_sub(fp2_sub(Z[11], Z[8]), Z[9]), fp2_sub(fp2_sub(Z[3], Z[0]), Z[1])), Z[6]); break;
      default: o = fp2_sub(fp2_sub(fp2_add(Z[9], Z[12]), fp2_add(Z[1], Z[4])), Z[7]); break;
    }
    S[l] = o;
  }
  c.sync();
}

// S = S^2 for S in the cyclotomic subgroup (Granger-Scott).
DEVNI void pt_cyclo_sqr(PtCtx c, int s) {
  fp2 *S = c.sm->S[s];
  const int l = c.lane;
  // Fp4 pairs (z0, z1) = (S0, S4), (z2, z3) = (S3, S2), (z4, z5) = (S1, S5)
  if (l < 9) {
    const int pa[3] = {0, 3, 1}, pb[3] = {4, 2, 5};
    const int g = l / 3, k = l % 3;
    fp2 x = k == 0 ? S[pa[g]] : k == 1 ? S[pb[g]] : fp2_add(S[pa[g]], S[pb[g]]);
    c.sm->Z[l] = fp2_sqr(x);
  }
  c.sync();
  fp2 o;
  if (l < 6) {
    const fp2 *Z = c.sm->Z;
    fp2 v = S[l];
    switch (l) {
      case 0: {  // 3 A0 - 2 z0,  A0 = xi z1^2 + z0^2
        fp2 t = fp2_add(fp2_mul_xi(Z[1]), Z[0]);
        o = fp2_add(fp2_dbl(fp2_sub(t, v)), t);
        break;
      }
      case 4: {  // 3 A1 + 2 z1,  A1 = (z0+z1)^2 - z0^2 - z1^2
        fp2 t = fp2_sub(fp2_sub(Z[2], Z[0]), Z[1]);
        o = fp2_add(fp2_dbl(fp2_add(t, v)), t);
        break;
      }
      case 1: {  // z4: 3 B0 - 2 z4,  B0 = xi z3^2 + z2^2
        fp2 t = fp2_add(fp2_mul_xi(Z[4]), Z[3]);
        o = fp2_add(fp2_dbl(fp2_sub(t, v)), t);
        break;
      }
      case 5: {  // z5: 3 B1 + 2 z5,  B1 = (z2+z3)^2 - z2^2 - z3^2
        fp2 t = fp2_sub(fp2_sub(Z[5], Z[3]), Z[4]);
        o = fp2_add(fp2_dbl(fp2_add(t, v)), t);
        break;
      }
      case 3: {  // z2: 3 xi C1 + 2 z2,  C1 = (z4+z5)^2 - z4^2 - z5^2
        fp2 t = fp2_mul_xi(fp2_sub(fp2_sub(Z[8], Z[6]), Z[7]));
        o = fp2_add(fp2_dbl(fp2_add(t, v)), t);
        break;
      }
      default: {  // z3: 3 C0 - 2 z3,  C0 = xi z5^2 + z4^2
        fp2 t = fp2_add(fp2_mul_xi(Z[7]), Z[6]);
        o = fp2_add(fp2_dbl(fp2_sub(t, v)), t);
        break;
      }
    }
  }
  c.sync();
  if (l < 6) S[l] = o;
  c.sync();
}

// dst = a * b (dst may alias a or b).  18 Fp2 products: 16 in the first
// round, the last two as six Fp products in the second.
DEVNI void pt_mul(PtCtx c, int dst, int sa, int sb) {
  const fp2 *a = c.sm->S[sa], *b = c.sm->S[sb];
  const int l = c.lane;
  auto operands = [&](int q, fp2 &x, fp2 &y) {
    const int g = q / 6, j = q % 6;
    if (g == 0) {
      pt_kara_pick(j, a[0], a[1], a[2], b[0], b[1], b[2], x, y);
    } else if (g == 1) {
      pt_kara_pick(j, a[3], a[4], a[5], b[3], b[4], b[5], x, y);
    } else {
      pt_kara_pick(j, fp2_add(a[0], a[3]), fp2_add(a[1], a[4]), fp2_add(a[2], a[5]), fp2_add(b[0], b[3]),
                   fp2_add(b[1], b[4]), fp2_add(b[2], b[5]), x, y);
    }
  };
  {
    fp2 x, y;
    operands(l, x, y);
    c.sm->Z[l] = fp2_mul(x, y);
  }
  if (l < 6) {  // products 16, 17 at Fp level: x0 y0, x1 y1, (x0 + x1)(y0 + y1)
    fp2 x, y;
    operands(16 + l / 3, x, y);
    const int k = l % 3;
    fp u = k == 0 ? x.c0 : k == 1 ? x.c1 : fp_add(x.c0, x.c1);
    fp v = k == 0 ? y.c0 : k == 1 ? y.c1 : fp_add(y.c0, y.c1);
    c.sm->Wf[l] = fp_mul(u, v);
  }
  c.sync();
  if (l < 2) {
    const fp *w = c.sm->Wf + 3 * l;
    fp2 z;
    z.c0 = fp_sub(w[0], w[1]);
    z.c1 = fp_sub(fp_sub(w[2], w[0]), w[1]);
    c.sm->Z[16 + l] = z;
  }
  c.sync();
  if (l < 9) c.sm->W[l] = pt_kara_assemble(l % 3, c.sm->Z + 6 * (l / 3));  // T0, T1, T2'
  c.sync();
  if (l < 6) {
    const fp2 *T0 = c.sm->W, *T1 = c.sm->W + 3, *T2 = c.sm->W + 6;
    fp2 o;
    switch (l) {  // c0 = T0 + v T1,  c1 = T2' - T0 - T1
      case 0: o = fp2_add(T0[0], fp2_mul_xi(T1[2])); break;
      case 1: o = fp2_add(T0[1], T1[0]); break;
      case 2: o = fp2_add(T0[2], T1[1]); break;
      default: o = fp2_sub(fp2_sub(T2[l - 3], T0[l - 3]), T1[l - 3]); break;
    }
    c.sm->S[dst][l] = o;
  }
  c.sync();
}

// dst = src^-1 (general Fp12): (c0 - c1 w) / (c0^2 - v c1^2)
DEVNI void pt_inv(PtCtx c, int dst, int src) {
  const fp2 *a = c.sm->S[src];
  const int l = c.lane;
  fp2 *Z = c.sm->Z, *W = c.sm->W;
  if (l < 12) {  // c0^2 (products 0..5), c1^2 (6..11)
    fp2 x, y;
    const int o = l < 6 ? 0 : 3;
    pt_kara_pick(l % 6, a[o], a[o + 1], a[o + 2], a[o], a[o + 1], a[o + 2], x, y);
    Z[l] = fp2_mul(x, y);
  }
  c.sync();
  fp2 d;
  if (l < 3) {  // D = c0^2 - v c1^2,  v (e0, e1, e2) = (xi e2, e0, e1)
    fp2 s0 = pt_kara_assemble(l, Z);
    fp2 s1 = pt_kara_assemble(l == 0 ? 2 : l - 1, Z + 6);
    d = fp2_sub(s0, l == 0 ? fp2_mul_xi(s1) : s1);
  }
  c.sync();
  if (l < 3) W[l] = d;  // D0, D1, D2
  c.sync();
  if (l < 6) {  // D0^2, D1 D2, D2^2, D0 D1, D1^2, D0 D2
    const int xa[6] = {0, 1, 2, 0, 1, 0}, xb[6] = {0, 2, 2, 1, 1, 2};
    Z[l] = fp2_mul(W[xa[l]], W[xb[l]]);
  }
  c.sync();
  if (l < 3) {  // t0 = D0^2 - xi D1 D2, t1 = xi D2^2 - D0 D1, t2 = D1^2 - D0 D2
    fp2 t;
    if (l == 0) t = fp2_sub(Z[0], fp2_mul_xi(Z[1]));
    else if (l == 1) t = fp2_sub(fp2_mul_xi(Z[2]), Z[3]);
    else t = fp2_sub(Z[4], Z[5]);
    W[3 + l] = t;
  }
  c.sync();
  if (l < 3) {  // D0 t0, D2 t1, D1 t2
    const int xd[3] = {0, 2, 1};
    Z[l] = fp2_mul(W[xd[l]], W[3 + l]);
  }
  c.sync();
  if (l == 0) {  // 1 / (D0 t0 + xi (D2 t1 + D1 t2)) on one lane, variable time
    fp2 n = fp2_add(Z[0], fp2_mul_xi(fp2_add(Z[1], Z[2])));
    fp ni = fp_inv_vartime(fp_add(fp_sqr(n.c0), fp_sqr(n.c1)));
    fp2 r;
    r.c0 = fp_mul(n.c0, ni);
    r.c1 = fp_neg(fp_mul(n.c1, ni));
    W[6] = r;
  }
  c.sync();
  if (l < 3) W[l] = fp2_mul(W[3 + l], W[6]);  // D^-1 = (t0, t1, t2) / d
  c.sync();
  if (l < 12) {  // c0 * D^-1 (0..5), c1 * D^-1 (6..11)
    fp2 x, y;
    const int o = l < 6 ? 0 : 3;
    pt_kara_pick(l % 6, a[o], a[o + 1], a[o + 2], W[0], W[1], W[2], x, y);
    Z[l] = fp2_mul(x, y);
  }
  c.sync();
  fp2 o;
  if (l < 6) {
    o = pt_kara_assemble(l % 3, Z + (l < 3 ? 0 : 6));
    if (l >= 3) o = fp2_neg(o);
  }
  c.sync();
  if (l < 6) c.sm->S[dst][l] = o;
  c.sync();
}

// dst = base^z (z < 0) for base in the cyclotomic subgroup; dst != base
DEVNI void pt_exp_by_z(PtCtx c, int dst, int base) {
  pt_copy(c, dst, base);
#pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    pt_cyclo_sqr(c, dst);
    if (zabs_bit(i)) pt_mul(c, dst, dst, base);
  }
  pt_conj(c, dst, dst);
}

// Final exponentiation of slot F; returns (on every lane) whether it is 1.
DEVNI bool pt_final_exp_is_one(PtCtx c) {
  // easy part: t = conj(f) / f, t = t^(p^2) * t
  pt_inv(c, PT_U, PT_F);
  pt_conj(c, PT_X, PT_F);
  pt_mul(c, PT_T, PT_X, PT_U);
  pt_frob(c, PT_X, PT_T);
  pt_frob(c, PT_X, PT_X);
  pt_mul(c, PT_T, PT_X, PT_T);
  // hard part: (z-1)^2 (z+p)(z^2+p^2-1) + 3
  pt_exp_by_z(c, PT_R, PT_T);  // a = t^z * conj(t)
  pt_conj(c, PT_X, PT_T);
  pt_mul(c, PT_A, PT_R, PT_X);
  pt_exp_by_z(c, PT_R, PT_A);  // a = a^z * conj(a)
  pt_conj(c, PT_X, PT_A);
  pt_mul(c, PT_A, PT_R, PT_X);
  pt_exp_by_z(c, PT_R, PT_A);  // b = a^z * a^p
  pt_frob(c, PT_X, PT_A);
  pt_mul(c, PT_A, PT_R, PT_X);
  pt_exp_by_z(c, PT_R, PT_A);  // c = (b^z)^z * b^(p^2) * conj(b)
  pt_copy(c, PT_X, PT_R);
  pt_exp_by_z(c, PT_R, PT_X);
  pt_frob(c, PT_X, PT_A);
  pt_frob(c, PT_X, PT_X);
  pt_mul(c, PT_R, PT_R, PT_X);
  pt_conj(c, PT_X, PT_A);
  pt_mul(c, PT_R, PT_R, PT_X);
  pt_mul(c, PT_R, PT_R, PT_T);  // c * t^3
  pt_mul(c, PT_R, PT_R, PT_T);
  pt_mul(c, PT_R, PT_R, PT_T);
  bool mine = true;
  if (c.lane < 6) mine = fp2_eq(c.sm->S[PT_R][c.lane], c.lane == 0 ? fp2_one() : fp2_zero());
  unsigned bad = __ballot_sync(c.mask, !mine);
  return bad == 0;
}
