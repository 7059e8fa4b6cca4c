// Optimal-ate pairing for BLS12-381 on sm_103a.
//
// A G2 point that is fixed across requests (a public key, -P2) is turned once
// into its 68 Miller-loop lines (63 doubling steps + 5 addition steps over the
// bits of |z| = 0xd201000000010000).  A line through T on the twist, pulled
// back to E and scaled by an Fp2 factor (removed by the final exponentiation),
// evaluates at P = (xP, yP) as
//     l(P) = A + (B * xP) v + yP * v w,
// so a line is stored as the pair (A, B) in Fp2 (2 x 96 bytes).  The product
// of the pairs' Miller functions shares one Fp12 squaring per step (the
// reference runs two separate Miller loops: pairing.cuh:376-478).  The final
// exponentiation raises to (p^6-1)(p^2+1) * 3(p^4-p^2+1)/r using
// 3(p^4-p^2+1)/r = (z-1)^2 (z+p)(z^2+p^2-1) + 3, which preserves "== 1".
#pragma once
#include "curve.cuh"

#define MILLER_LINES 68
struct line2 { fp2 a, b; };

// Lines of the Miller loop for Q (affine, not infinity), written to out[0..67].
DEV void g2_precompute_lines(g2a q, line2 *out) {
  g2j T = g2j_from_aff(q);
  int idx = 0;
  #pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    {  // tangent at T: (3X^3 - 2Y^2) + (-3 X^2 Z^2) xP v + (2 Y Z^3) yP v w
      fp2 X2 = fp2_sqr(T.X), Z2 = fp2_sqr(T.Z);
      fp2 X3 = fp2_mul(X2, T.X);
      fp2 a = fp2_sub(fp2_add(fp2_dbl(X3), X3), fp2_dbl(fp2_sqr(T.Y)));
      fp2 b = fp2_neg(fp2_mul(fp2_add(fp2_dbl(X2), X2), Z2));
      fp2 c = fp2_dbl(fp2_mul(fp2_mul(T.Y, Z2), T.Z));
      fp2 ci = fp2_inv(c);
      out[idx].a = fp2_mul(a, ci);
      out[idx].b = fp2_mul(b, ci);
      idx++;
      T = g2j_dbl(T);
    }
    if (zabs_bit(i)) {  // chord through T and Q
      fp2 Z2 = fp2_sqr(T.Z);
      fp2 N = fp2_sub(fp2_mul(fp2_mul(q.y, Z2), T.Z), T.Y);
      fp2 D = fp2_mul(T.Z, fp2_sub(fp2_mul(q.x, Z2), T.X));
      fp2 a = fp2_sub(fp2_mul(N, q.x), fp2_mul(q.y, D));
      fp2 b = fp2_neg(N);
      fp2 ci = fp2_inv(D);
      out[idx].a = fp2_mul(a, ci);
      out[idx].b = fp2_mul(b, ci);
      idx++;
      T = g2j_add(T, g2j_from_aff(q));
    }
  }
}

// f *= (A + (B xP) v + yP v w)
DEV fp12 fp12_mul_line(fp12 f, fp2 A, fp2 Bx, fp yP) {
  // l0 = (A, Bx, 0) in Fp6, l1 = (0, yP, 0) in Fp6 (coefficient of w)
  // f0*l0 (sparse)
  const fp6 &f0 = f.c0, &f1 = f.c1;
  fp6 t0;
  {
    fp2 a0 = fp2_mul(f0.c0, A), a1 = fp2_mul(f0.c1, Bx);
    t0.c0 = fp2_add(a0, fp2_mul_xi(fp2_mul(f0.c2, Bx)));
    t0.c1 = fp2_sub(fp2_sub(fp2_mul(fp2_add(f0.c0, f0.c1), fp2_add(A, Bx)), a0), a1);
    t0.c2 = fp2_add(a1, fp2_mul(f0.c2, A));
  }
  // f1*l1 = f1 * (yP v) = mul_v(f1 * yP)
  fp6 t1;
  t1.c0 = fp2_mul_xi(fp2_mul_fp(f1.c2, yP));
  t1.c1 = fp2_mul_fp(f1.c0, yP);
  t1.c2 = fp2_mul_fp(f1.c1, yP);
  // (f0 + f1) * (l0 + l1) with l0 + l1 = (A, Bx + yP, 0)
  fp6 s = fp6_add(f0, f1);
  fp2 B2 = Bx;
  B2.c0 = fp_add(B2.c0, yP);
  fp6 t2;
  {
    fp2 a0 = fp2_mul(s.c0, A), a1 = fp2_mul(s.c1, B2);
    t2.c0 = fp2_add(a0, fp2_mul_xi(fp2_mul(s.c2, B2)));
    t2.c1 = fp2_sub(fp2_sub(fp2_mul(fp2_add(s.c0, s.c1), fp2_add(A, B2)), a0), a1);
    t2.c2 = fp2_add(a1, fp2_mul(s.c2, A));
  }
  fp12 r;
  r.c0 = fp6_add(t0, fp6_mul_v(t1));
  r.c1 = fp6_sub(fp6_sub(t2, t0), t1);
  return r;
}

// Miller loop over npairs (P_i affine in G1, lines of Q_i); skip[i] drops a pair
// whose point is the identity.
template <int NP>
DEV fp12 miller_loop_lines(const g1a *P, const line2 *const *lines, const bool *skip) {
  fp12 f = fp12_one();
  int idx = 0;
  #pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    f = fp12_sqr(f);
    #pragma unroll 1
    for (int k = 0; k < NP; k++) {
      if (skip[k]) continue;
      const line2 l = lines[k][idx];
      f = fp12_mul_line(f, l.a, fp2_mul_fp(l.b, P[k].x), P[k].y);
    }
    idx++;
    if (zabs_bit(i)) {
      #pragma unroll 1
      for (int k = 0; k < NP; k++) {
        if (skip[k]) continue;
        const line2 l = lines[k][idx];
        f = fp12_mul_line(f, l.a, fp2_mul_fp(l.b, P[k].x), P[k].y);
      }
      idx++;
    }
  }
  return fp12_conj(f);  // z < 0
}

DEV fp12 fp12_exp_by_zabs(fp12 f) {
  fp12 r = f;
  #pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    r = fp12_sqr(r);
    if (zabs_bit(i)) r = fp12_mul(r, f);
  }
  return r;
}
// f^z for unitary f (z < 0)
DEV fp12 fp12_exp_by_z(const fp12 &f) { return fp12_conj(fp12_exp_by_zabs(f)); }

DEV fp12 final_exponentiation(fp12 f) {
  fp12 t = fp12_mul(fp12_conj(f), fp12_inv(f));
  t = fp12_mul(fp12_frobenius(fp12_frobenius(t)), t);
  fp12 a = fp12_mul(fp12_exp_by_z(t), fp12_conj(t));
  a = fp12_mul(fp12_exp_by_z(a), fp12_conj(a));
  fp12 b = fp12_mul(fp12_exp_by_z(a), fp12_frobenius(a));
  fp12 c = fp12_mul(fp12_mul(fp12_exp_by_z(fp12_exp_by_z(b)), fp12_frobenius(fp12_frobenius(b))),
                    fp12_conj(b));
  return fp12_mul(fp12_mul(fp12_mul(c, t), t), t);
}
