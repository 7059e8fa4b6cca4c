// G1 / G2 group law, encodings and scalar multiplication on sm_103a.
//
// G1 accumulators use XYZZ coordinates (x = X/ZZ, y = Y/ZZZ; EFD formulas
// madd-2008-s, add-2008-s, dbl-2008-s-1, mdbl-2008-s-1).  G2 uses Jacobian
// coordinates over Fp2.  Encodings follow the zkcrypto/bls12_381_plus
// compressed format used by the reference (G1 48 B, G2 96 B with x.c1 first;
// flag bits: 0x80 compressed, 0x40 infinity, 0x20 y lexicographically largest;
// reference decode/encode: native/cuda/src/g1_msm_blst.cpp:614-732).
#pragma once
#include "field.cuh"

struct g1a { fp x, y; };               // affine, no infinity
struct g1 { fp X, Y, ZZ, ZZZ; };       // XYZZ, ZZ == 0 is infinity

DEV g1 g1_inf() { g1 r; r.X = fp_one(); r.Y = fp_one(); r.ZZ = fp_zero(); r.ZZZ = fp_zero(); return r; }
DEV bool g1_is_inf(const g1 &p) { return fp_is_zero(p.ZZ); }
DEV g1 g1_from_aff(const g1a &a) { g1 r; r.X = a.x; r.Y = a.y; r.ZZ = fp_one(); r.ZZZ = fp_one(); return r; }
DEV g1 g1_neg(const g1 &p) { g1 r = p; r.Y = fp_neg(p.Y); return r; }
DEV g1a g1a_neg(const g1a &p) { g1a r = p; r.y = fp_neg(p.y); return r; }

DEVNI g1 g1_dbl(g1 p);
DEVNI g1 g1_dbl_aff(g1a p);

DEV g1 g1_dbl_inl(g1 p) {
  if (g1_is_inf(p)) return p;
  fp U = fp_dbl(p.Y);
  fp V = fp_sqr(U);
  fp W = fp_mul(U, V);
  fp S = fp_mul(p.X, V);
  fp X2 = fp_sqr(p.X);
  fp M = fp_add(fp_dbl(X2), X2);
  g1 r;
  r.X = fp_sub(fp_sub(fp_sqr(M), S), S);
  r.Y = fp_sub(fp_mul(M, fp_sub(S, r.X)), fp_mul(W, p.Y));
  r.ZZ = fp_mul(V, p.ZZ);
  r.ZZZ = fp_mul(W, p.ZZZ);
  return r;
}
DEV g1 g1_dbl_aff_inl(g1a p) {
  fp U = fp_dbl(p.y);
  fp V = fp_sqr(U);
  fp W = fp_mul(U, V);
  fp S = fp_mul(p.x, V);
  fp X2 = fp_sqr(p.x);
  fp M = fp_add(fp_dbl(X2), X2);
  g1 r;
  r.X = fp_sub(fp_sub(fp_sqr(M), S), S);
  r.Y = fp_sub(fp_mul(M, fp_sub(S, r.X)), fp_mul(W, p.y));
  r.ZZ = V;
  r.ZZZ = W;
  return r;
}
// p + q with q affine
DEV g1 g1_add_aff_inl(g1 p, g1a q) {
  if (g1_is_inf(p)) return g1_from_aff(q);
  fp U2 = fp_mul(q.x, p.ZZ);
  fp S2 = fp_mul(q.y, p.ZZZ);
  fp P = fp_sub(U2, p.X);
  fp R = fp_sub(S2, p.Y);
  if (fp_is_zero(P)) {
    if (fp_is_zero(R)) return g1_dbl_aff(q);
    return g1_inf();
  }
  fp PP = fp_sqr(P);
  fp PPP = fp_mul(P, PP);
  fp Q = fp_mul(p.X, PP);
  g1 r;
  r.X = fp_sub(fp_sub(fp_sqr(R), PPP), fp_dbl(Q));
  r.Y = fp_sub(fp_mul(R, fp_sub(Q, r.X)), fp_mul(p.Y, PPP));
  r.ZZ = fp_mul(p.ZZ, PP);
  r.ZZZ = fp_mul(p.ZZZ, PPP);
  return r;
}
DEV g1 g1_add_inl(g1 p, g1 q) {
  if (g1_is_inf(p)) return q;
  if (g1_is_inf(q)) return p;
  fp U1 = fp_mul(p.X, q.ZZ);
  fp U2 = fp_mul(q.X, p.ZZ);
  fp S1 = fp_mul(p.Y, q.ZZZ);
  fp S2 = fp_mul(q.Y, p.ZZZ);
  fp P = fp_sub(U2, U1);
  fp R = fp_sub(S2, S1);
  if (fp_is_zero(P)) {
    if (fp_is_zero(R)) return g1_dbl(p);
    return g1_inf();
  }
  fp PP = fp_sqr(P);
  fp PPP = fp_mul(P, PP);
  fp Q = fp_mul(U1, PP);
  g1 r;
  r.X = fp_sub(fp_sub(fp_sqr(R), PPP), fp_dbl(Q));
  r.Y = fp_sub(fp_mul(R, fp_sub(Q, r.X)), fp_mul(S1, PPP));
  r.ZZ = fp_mul(fp_mul(p.ZZ, q.ZZ), PP);
  r.ZZZ = fp_mul(fp_mul(p.ZZZ, q.ZZZ), PPP);
  return r;
}
// Out-of-line entry points (one copy per translation unit keeps compile
// times bounded); hot loops call the _inl forms directly.
DEVNI g1 g1_dbl(g1 p) { return g1_dbl_inl(p); }
DEVNI g1 g1_dbl_aff(g1a p) { return g1_dbl_aff_inl(p); }
DEVNI g1 g1_add_aff(g1 p, g1a q) { return g1_add_aff_inl(p, q); }
DEVNI g1 g1_add(g1 p, g1 q) { return g1_add_inl(p, q); }
// affine conversion with a single inversion; returns false for infinity.  The
// points converted are public (proof and signature components, MSM outputs),
// so the inverse is the variable-time one.
DEV bool g1_to_aff(g1 p, g1a &out) {
  if (g1_is_inf(p)) return false;
  fp t = fp_inv_vartime(fp_mul(p.ZZ, p.ZZZ));
  out.x = fp_mul(p.X, fp_mul(t, p.ZZZ));  // X / ZZ
  out.y = fp_mul(p.Y, fp_mul(t, p.ZZ));   // Y / ZZZ
  return true;
}
// Fp value of another lane (full-warp shuffles).
DEV fp shfl_fp(const fp &a, int src) {
  fp r;
#pragma unroll
  for (int i = 0; i < 12; i++) r.w[i] = __shfl_sync(0xffffffffu, a.w[i], src);
  return r;
}
DEV fp shfl_up_fp(const fp &a, int d) {
  fp r;
#pragma unroll
  for (int i = 0; i < 12; i++) r.w[i] = __shfl_up_sync(0xffffffffu, a.w[i], d);
  return r;
}
DEV fp shfl_down_fp(const fp &a, int d) {
  fp r;
#pragma unroll
  for (int i = 0; i < 12; i++) r.w[i] = __shfl_down_sync(0xffffffffu, a.w[i], d);
  return r;
}
// v^-1 for one value per lane of a full warp (Montgomery's simultaneous
// inversion): inclusive prefix and suffix products by shuffles (5 products
// each), one variable-time inverse of the whole product on lane 31, then
// v_l^-1 = (v_0 .. v_{l-1}) (v_{l+1} .. v_31) / (v_0 .. v_31).  A zero value
// counts as 1 and gets 0.  Every lane of the warp must call it.
DEV fp warp_batch_inv(const fp &v_in) {
  const int lane = threadIdx.x & 31;
  const bool zero = fp_is_zero(v_in);
  const fp one = fp_one();
  const fp v = zero ? one : v_in;
  fp pre = v, suf = v;
#pragma unroll 1
  for (int d = 1; d < 32; d *= 2) {
    fp o = shfl_up_fp(pre, d);
    pre = fp_mul(pre, lane >= d ? o : one);
    fp q = shfl_down_fp(suf, d);
    suf = fp_mul(suf, lane + d < 32 ? q : one);
  }
  fp inv_all = fp_zero();
  if (lane == 31) inv_all = fp_inv_vartime(pre);
  inv_all = shfl_fp(inv_all, 31);
  fp before = shfl_up_fp(pre, 1), after = shfl_down_fp(suf, 1);
  if (lane == 0) before = one;
  if (lane == 31) after = one;
  const fp r = fp_mul(fp_mul(before, after), inv_all);
  return zero ? fp_zero() : r;
}
// Affine forms of N points per lane with one warp-batched inversion (the
// inverses of the lane's N values ZZ ZZZ come from the inverse of their
// product and in-lane prefix / suffix products); fin[k] is false for infinity.
// Every lane of the warp must call it.
template <int N> DEV void warp_to_aff(const g1 *p, g1a *a, bool *fin) {
  const fp one = fp_one();
  fp z[N], pre[N], suf[N];
#pragma unroll
  for (int k = 0; k < N; k++) {
    fin[k] = !g1_is_inf(p[k]);
    z[k] = fin[k] ? fp_mul(p[k].ZZ, p[k].ZZZ) : one;
  }
  pre[0] = z[0];
#pragma unroll
  for (int k = 1; k < N; k++) pre[k] = fp_mul(pre[k - 1], z[k]);
  suf[N - 1] = z[N - 1];
#pragma unroll
  for (int k = N - 2; k >= 0; k--) suf[k] = fp_mul(suf[k + 1], z[k]);
  const fp t = warp_batch_inv(pre[N - 1]);
#pragma unroll
  for (int k = 0; k < N; k++) {
    fp ik = t;  // 1 / (ZZ_k ZZZ_k) = t * prod_{j != k} z_j
    if (k > 0) ik = fp_mul(ik, pre[k - 1]);
    if (k < N - 1) ik = fp_mul(ik, suf[k + 1]);
    a[k].x = fp_mul(p[k].X, fp_mul(ik, p[k].ZZZ));
    a[k].y = fp_mul(p[k].Y, fp_mul(ik, p[k].ZZ));
  }
}
DEV void g1_compress_aff_or_inf(const g1a &a, bool finite, uint8_t out[48]);

DEV bool g1_eq(const g1 &p, const g1 &q) {
  bool pi = g1_is_inf(p), qi = g1_is_inf(q);
  if (pi || qi) return pi && qi;
  return fp_eq(fp_mul(p.X, q.ZZ), fp_mul(q.X, p.ZZ)) && fp_eq(fp_mul(p.Y, q.ZZZ), fp_mul(q.Y, p.ZZZ));
}
// GLV endomorphism image of an XYZZ point: [z^2]P = (beta x, -y)
DEV g1 g1_endo(const g1 &p) {
  const fp beta = C_GLV_BETA;
  g1 r = p;
  r.X = fp_mul(p.X, beta);
  r.Y = fp_neg(p.Y);
  return r;
}

// ---- encodings
DEV void g1_compress_aff(const g1a &a, uint8_t out[48]) {
  fp_to_be48(a.x, out);
  out[0] |= 0x80;
  if (fp_lex_largest(a.y)) out[0] |= 0x20;
}
DEV void g1_compress_aff_or_inf(const g1a &a, bool finite, uint8_t out[48]) {
  if (!finite) {
    out[0] = 0xc0;
    #pragma unroll 1
    for (int i = 1; i < 48; i++) out[i] = 0;
    return;
  }
  g1_compress_aff(a, out);
}
DEV void g1_compress(g1 p, uint8_t out[48]) {
  g1a a;
  if (!g1_to_aff(p, a)) {
    out[0] = 0xc0;
    #pragma unroll 1
    for (int i = 1; i < 48; i++) out[i] = 0;
    return;
  }
  g1_compress_aff(a, out);
}

// [|z|]P for |z| = 0xd201000000010000 (bits 63,62,60,57,48,16)
DEV g1 g1_mul_zabs(g1 p) {
  g1 acc = p;
  #pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    acc = g1_dbl(acc);
    if (zabs_bit(i)) acc = g1_add(acc, p);
  }
  return acc;
}
// G1 membership for a curve point: phi(P) == -[z^2]P  <=>  [z^2]P == (beta x, -y)
DEV bool g1_in_subgroup(g1a a) {
  g1 t = g1_mul_zabs(g1_mul_zabs(g1_from_aff(a)));
  if (g1_is_inf(t)) return false;
  const fp beta = C_GLV_BETA;
  fp bx = fp_mul(a.x, beta);
  fp ny = fp_neg(a.y);
  return fp_eq(t.X, fp_mul(bx, t.ZZ)) && fp_eq(t.Y, fp_mul(ny, t.ZZZ));
}

// ---- point arithmetic on a lane pair
// Lanes 2k and 2k+1 hold the same operands and split every formula's
// independent Fp products between them: in each round each lane computes one
// product and the two results are exchanged with one pair-masked shuffle, so
// a doubling takes 5 product latencies instead of 9, a mixed addition 5
// instead of 10 and an XYZZ addition 7 instead of 14.  Both lanes take the
// same branches (they hold the same values), and the shuffles name only the
// pair, so pairs may diverge from one another.  Results equal the one-lane
// formulas above exactly.
struct LanePair {
  unsigned mask;  // the two lanes of the pair
  int role;       // 0 or 1
  DEV static LanePair here() {
    const int lane = threadIdx.x & 31;
    LanePair p;
    p.mask = 3u << (lane & ~1);
    p.role = lane & 1;
    return p;
  }
};
DEV fp pair_swap(const LanePair &lp, const fp &a) {
  fp r;
#pragma unroll
  for (int i = 0; i < 12; i++) r.w[i] = __shfl_xor_sync(lp.mask, a.w[i], 1);
  return r;
}
DEV fp pair_sel(const LanePair &lp, const fp &a, const fp &b) {
  fp r;
#pragma unroll
  for (int i = 0; i < 12; i++) r.w[i] = lp.role ? b.w[i] : a.w[i];
  return r;
}
// r0 = a0 b0 (computed by role 0), r1 = a1 b1 (role 1); both lanes get both.
DEV void pair_mul(const LanePair &lp, const fp &a0, const fp &b0, const fp &a1, const fp &b1, fp &r0, fp &r1) {
  const fp r = fp_mul(pair_sel(lp, a0, a1), pair_sel(lp, b0, b1));
  const fp o = pair_swap(lp, r);
  r0 = pair_sel(lp, r, o);
  r1 = pair_sel(lp, o, r);
}
DEV g1 g1_dbl_pair(const LanePair &lp, const g1 &p) {
  if (g1_is_inf(p)) return p;
  const fp U = fp_dbl(p.Y);
  fp V, X2, W, S, ZZ3, M2, WY, ZZZ3;
  pair_mul(lp, U, U, p.X, p.X, V, X2);
  const fp M = fp_add(fp_dbl(X2), X2);
  pair_mul(lp, U, V, p.X, V, W, S);
  pair_mul(lp, V, p.ZZ, M, M, ZZ3, M2);
  pair_mul(lp, W, p.Y, W, p.ZZZ, WY, ZZZ3);
  g1 r;
  r.X = fp_sub(fp_sub(M2, S), S);
  r.Y = fp_sub(fp_mul(M, fp_sub(S, r.X)), WY);  // same product on both lanes
  r.ZZ = ZZ3;
  r.ZZZ = ZZZ3;
  return r;
}
// p + q with q affine
DEV g1 g1_add_aff_pair(const LanePair &lp, const g1 &p, const g1a &q) {
  if (g1_is_inf(p)) return g1_from_aff(q);
  fp U2, S2;
  pair_mul(lp, q.x, p.ZZ, q.y, p.ZZZ, U2, S2);
  const fp P = fp_sub(U2, p.X), R = fp_sub(S2, p.Y);
  if (fp_is_zero(P)) {
    if (fp_is_zero(R)) return g1_dbl_pair(lp, g1_from_aff(q));
    return g1_inf();
  }
  fp PP, RR, PPP, Q, ZZ3, YP, ZZZ3, T;
  pair_mul(lp, P, P, R, R, PP, RR);
  pair_mul(lp, P, PP, p.X, PP, PPP, Q);
  g1 r;
  r.X = fp_sub(fp_sub(RR, PPP), fp_dbl(Q));
  pair_mul(lp, p.ZZ, PP, p.Y, PPP, ZZ3, YP);
  pair_mul(lp, p.ZZZ, PPP, R, fp_sub(Q, r.X), ZZZ3, T);
  r.Y = fp_sub(T, YP);
  r.ZZ = ZZ3;
  r.ZZZ = ZZZ3;
  return r;
}
DEV g1 g1_add_pair(const LanePair &lp, const g1 &p, const g1 &q) {
  if (g1_is_inf(p)) return q;
  if (g1_is_inf(q)) return p;
  fp U1, U2, S1, S2;
  pair_mul(lp, p.X, q.ZZ, q.X, p.ZZ, U1, U2);
  pair_mul(lp, p.Y, q.ZZZ, q.Y, p.ZZZ, S1, S2);
  const fp P = fp_sub(U2, U1), R = fp_sub(S2, S1);
  if (fp_is_zero(P)) {
    if (fp_is_zero(R)) return g1_dbl_pair(lp, p);
    return g1_inf();
  }
  fp PP, RR, PPP, Q, Z1, Z2, ZZ3, ZZZ3, SP, T;
  pair_mul(lp, P, P, R, R, PP, RR);
  pair_mul(lp, P, PP, U1, PP, PPP, Q);
  g1 r;
  r.X = fp_sub(fp_sub(RR, PPP), fp_dbl(Q));
  pair_mul(lp, p.ZZ, q.ZZ, p.ZZZ, q.ZZZ, Z1, Z2);
  pair_mul(lp, Z1, PP, Z2, PPP, ZZ3, ZZZ3);
  pair_mul(lp, S1, PPP, R, fp_sub(Q, r.X), SP, T);
  r.Y = fp_sub(T, SP);
  r.ZZ = ZZ3;
  r.ZZZ = ZZZ3;
  return r;
}

// [|z|]P on a lane pair.
DEV g1 g1_mul_zabs_pair(const LanePair &lp, const g1 &p) {
  g1 acc = p;
  #pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    acc = g1_dbl_pair(lp, acc);
    if (zabs_bit(i)) acc = g1_add_pair(lp, acc, p);
  }
  return acc;
}
// g1_in_subgroup on a lane pair.
DEV bool g1_in_subgroup_pair(const LanePair &lp, g1a a) {
  g1 t = g1_mul_zabs_pair(lp, g1_mul_zabs_pair(lp, g1_from_aff(a)));
  if (g1_is_inf(t)) return false;
  const fp beta = C_GLV_BETA;
  fp bx = fp_mul(a.x, beta);
  fp ny = fp_neg(a.y);
  return fp_eq(t.X, fp_mul(bx, t.ZZ)) && fp_eq(t.Y, fp_mul(ny, t.ZZZ));
}
// ---- point arithmetic on a lane quad
// Lanes 4k .. 4k+3 hold the same operands and split each formula's
// independent products four ways: a doubling takes 3 product latencies
// (instead of 5 on a pair, 9 on one lane), a mixed or an XYZZ addition 4
// (5 / 7 on a pair).  In each round lane k of the quad computes product k and
// every lane receives all of them by quad-masked shuffles; the four lanes take
// the same branches, quads may diverge from one another.  Results equal the
// one-lane formulas exactly (same products, same order of the sums).
struct LaneQuad {
  unsigned mask;  // the four lanes of the quad
  int role;       // 0..3
  int base;       // lane of role 0
  DEV static LaneQuad here() {
    const int lane = threadIdx.x & 31;
    LaneQuad q;
    q.base = lane & ~3;
    q.mask = 0xFu << q.base;
    q.role = lane & 3;
    return q;
  }
};
DEV fp quad_from(const LaneQuad &q, const fp &a, int src) {
  fp r;
#pragma unroll
  for (int i = 0; i < 12; i++) r.w[i] = __shfl_sync(q.mask, a.w[i], q.base + src);
  return r;
}
DEV fp quad_pick(const LaneQuad &q, const fp &a0, const fp &a1, const fp &a2, const fp &a3) {
  fp r;
#pragma unroll
  for (int i = 0; i < 12; i++) r.w[i] = q.role == 0 ? a0.w[i] : q.role == 1 ? a1.w[i] : q.role == 2 ? a2.w[i] : a3.w[i];
  return r;
}
// r_k = a_k b_k for k < N (2..4), product k computed by role k (a role >= N
// repeats product 0); every lane gets every r_k.
template <int N>
DEV void quad_mul(const LaneQuad &q, const fp &a0, const fp &b0, const fp &a1, const fp &b1, const fp &a2,
                  const fp &b2, const fp &a3, const fp &b3, fp &r0, fp &r1, fp &r2, fp &r3) {
  const fp mine = fp_mul(quad_pick(q, a0, a1, N > 2 ? a2 : a0, N > 3 ? a3 : a0),
                         quad_pick(q, b0, b1, N > 2 ? b2 : b0, N > 3 ? b3 : b0));
  r0 = quad_from(q, mine, 0);
  r1 = quad_from(q, mine, 1);
  if (N > 2) r2 = quad_from(q, mine, 2);
  if (N > 3) r3 = quad_from(q, mine, 3);
}
DEV g1 g1_dbl_quad(const LaneQuad &q, const g1 &p) {
  if (g1_is_inf(p)) return p;
  const fp U = fp_dbl(p.Y);
  fp V, X2, W, S, ZZ3, M2, T, WY, ZZZ3, unused;
  quad_mul<2>(q, U, U, p.X, p.X, U, U, U, U, V, X2, unused, unused);
  const fp M = fp_add(fp_dbl(X2), X2);
  quad_mul<4>(q, U, V, p.X, V, V, p.ZZ, M, M, W, S, ZZ3, M2);
  g1 r;
  r.X = fp_sub(fp_sub(M2, S), S);
  quad_mul<3>(q, M, fp_sub(S, r.X), W, p.Y, W, p.ZZZ, M, M, T, WY, ZZZ3, unused);
  r.Y = fp_sub(T, WY);
  r.ZZ = ZZ3;
  r.ZZZ = ZZZ3;
  return r;
}
// p + q with q affine
DEV g1 g1_add_aff_quad(const LaneQuad &lq, const g1 &p, const g1a &q) {
  if (g1_is_inf(p)) return g1_from_aff(q);
  fp U2, S2, PP, RR, PPP, Q, ZZ3, T, YP, ZZZ3, unused;
  quad_mul<2>(lq, q.x, p.ZZ, q.y, p.ZZZ, q.x, q.x, q.x, q.x, U2, S2, unused, unused);
  const fp P = fp_sub(U2, p.X), R = fp_sub(S2, p.Y);
  if (fp_is_zero(P)) {
    if (fp_is_zero(R)) return g1_dbl_quad(lq, g1_from_aff(q));
    return g1_inf();
  }
  quad_mul<2>(lq, P, P, R, R, P, P, P, P, PP, RR, unused, unused);
  quad_mul<3>(lq, P, PP, p.X, PP, p.ZZ, PP, P, P, PPP, Q, ZZ3, unused);
  g1 r;
  r.X = fp_sub(fp_sub(RR, PPP), fp_dbl(Q));
  quad_mul<3>(lq, R, fp_sub(Q, r.X), p.Y, PPP, p.ZZZ, PPP, P, P, T, YP, ZZZ3, unused);
  r.Y = fp_sub(T, YP);
  r.ZZ = ZZ3;
  r.ZZZ = ZZZ3;
  return r;
}
DEV g1 g1_add_quad(const LaneQuad &lq, const g1 &p, const g1 &q) {
  if (g1_is_inf(p)) return q;
  if (g1_is_inf(q)) return p;
  fp U1, U2, S1, S2, PP, RR, Z1, Z2, PPP, Q, ZZ3, T, SP, ZZZ3, unused;
  quad_mul<4>(lq, p.X, q.ZZ, q.X, p.ZZ, p.Y, q.ZZZ, q.Y, p.ZZZ, U1, U2, S1, S2);
  const fp P = fp_sub(U2, U1), R = fp_sub(S2, S1);
  if (fp_is_zero(P)) {
    if (fp_is_zero(R)) return g1_dbl_quad(lq, p);
    return g1_inf();
  }
  quad_mul<4>(lq, P, P, R, R, p.ZZ, q.ZZ, p.ZZZ, q.ZZZ, PP, RR, Z1, Z2);
  quad_mul<3>(lq, P, PP, U1, PP, Z1, PP, P, P, PPP, Q, ZZ3, unused);
  g1 r;
  r.X = fp_sub(fp_sub(RR, PPP), fp_dbl(Q));
  quad_mul<3>(lq, R, fp_sub(Q, r.X), S1, PPP, Z2, PPP, P, P, T, SP, ZZZ3, unused);
  r.Y = fp_sub(T, SP);
  r.ZZ = ZZ3;
  r.ZZZ = ZZZ3;
  return r;
}
// [|z|]P and the G1 membership test on a lane quad.
DEV g1 g1_mul_zabs_quad(const LaneQuad &q, const g1 &p) {
  g1 acc = p;
  #pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    acc = g1_dbl_quad(q, acc);
    if (zabs_bit(i)) acc = g1_add_quad(q, acc, p);
  }
  return acc;
}
DEV bool g1_in_subgroup_quad(const LaneQuad &q, g1a a) {
  g1 t = g1_mul_zabs_quad(q, g1_mul_zabs_quad(q, g1_from_aff(a)));
  if (g1_is_inf(t)) return false;
  const fp beta = C_GLV_BETA;
  fp bx = fp_mul(a.x, beta);
  fp ny = fp_neg(a.y);
  return fp_eq(t.X, fp_mul(bx, t.ZZ)) && fp_eq(t.Y, fp_mul(ny, t.ZZZ));
}

// Warp-wide sum of one XYZZ point per lane (the result is valid on lane 0).
DEV g1 shfl_down_g1(const g1 &p, int delta) {
  g1 r;
#pragma unroll
  for (int i = 0; i < 12; i++) {
    r.X.w[i] = __shfl_down_sync(0xffffffffu, p.X.w[i], delta);
    r.Y.w[i] = __shfl_down_sync(0xffffffffu, p.Y.w[i], delta);
    r.ZZ.w[i] = __shfl_down_sync(0xffffffffu, p.ZZ.w[i], delta);
    r.ZZZ.w[i] = __shfl_down_sync(0xffffffffu, p.ZZZ.w[i], delta);
  }
  return r;
}
DEV g1 warp_sum_g1(g1 acc) {
  #pragma unroll 1
  for (int d = 16; d > 0; d >>= 1) {
    g1 o = shfl_down_g1(acc, d);
    acc = g1_add(acc, o);
  }
  return acc;
}

// Decode status values
#define DEC_OK 0
#define DEC_INF 1
#define DEC_BAD 2
// G1Affine::from_compressed (unchecked decode + torsion check).  Returns DEC_OK
// with the affine point, DEC_INF for the canonical identity encoding, DEC_BAD otherwise.
DEV int g1_decompress(const uint8_t in[48], g1a &out, bool check_subgroup = true) {
  uint8_t f = in[0];
  bool comp = f & 0x80, inf = f & 0x40, sort = f & 0x20;
  uint8_t t[48];
  t[0] = f & 0x1f;
  #pragma unroll 1
  for (int i = 1; i < 48; i++) t[i] = in[i];
  fp x;
  if (!fp_from_be48(t, x)) return DEC_BAD;
  if (inf) return (comp && !sort && fp_is_zero(x)) ? DEC_INF : DEC_BAD;
  if (!comp) return DEC_BAD;
  const fp four = C_FP_FOUR;
  fp y;
  if (!fp_sqrt(fp_add(fp_mul(fp_sqr(x), x), four), y)) return DEC_BAD;
  if (fp_lex_largest(y) != sort) y = fp_neg(y);
  out.x = x;
  out.y = y;
  if (check_subgroup && !g1_in_subgroup(out)) return DEC_BAD;
  return DEC_OK;
}

// ---- scalar multiplication (variable base, GLV + signed 4-bit windows)
// Split k (canonical, < r) as k = q * lambda + s with lambda = z^2 (128-bit),
// so k P = s P + q [lambda]P with [lambda]P = g1_endo(P).  Both halves are
// below 2^128 (q < r / lambda < 2^128).
DEVNI void glv_split(fr k, uint32_t s[4], uint32_t q[4]) {
  // schoolbook shift-subtract long division of a 256-bit k by the 128-bit lambda
  const uint64_t lam_lo = C_GLV_LAMBDA_LO, lam_hi = C_GLV_LAMBDA_HI;
  // After the steps over bits 255..128 the remainder is k >> 128 and no step
  // has subtracted as long as k >> 128 < lambda, which holds for every k < r
  // (r >> 128 < lambda): start from there.  Larger k take all 256 steps.
  uint64_t rem_lo = ((uint64_t)k.w[5] << 32) | k.w[4], rem_hi = ((uint64_t)k.w[7] << 32) | k.w[6];
  int top = 127;
  if (rem_hi > lam_hi || (rem_hi == lam_hi && rem_lo >= lam_lo)) { rem_lo = rem_hi = 0; top = 255; }
  uint64_t q_lo = 0, q_hi = 0;
  #pragma unroll 1
  for (int i = top; i >= 0; i--) {
    uint32_t bit = (k.w[i >> 5] >> (i & 31)) & 1;
    // rem = rem*2 + bit (rem < 2^128 so rem*2 < 2^129: track the carry)
    uint64_t carry = rem_hi >> 63;
    rem_hi = (rem_hi << 1) | (rem_lo >> 63);
    rem_lo = (rem_lo << 1) | bit;
    bool ge = carry || rem_hi > lam_hi || (rem_hi == lam_hi && rem_lo >= lam_lo);
    if (ge) {
      uint64_t nlo = rem_lo - lam_lo;
      uint64_t borrow = rem_lo < lam_lo ? 1 : 0;
      rem_hi = rem_hi - lam_hi - borrow;
      rem_lo = nlo;
    }
    // q = q*2 + ge  (q < 2^128)
    q_hi = (q_hi << 1) | (q_lo >> 63);
    q_lo = (q_lo << 1) | (ge ? 1 : 0);
  }
  s[0] = (uint32_t)rem_lo; s[1] = (uint32_t)(rem_lo >> 32); s[2] = (uint32_t)rem_hi; s[3] = (uint32_t)(rem_hi >> 32);
  q[0] = (uint32_t)q_lo; q[1] = (uint32_t)(q_lo >> 32); q[2] = (uint32_t)q_hi; q[3] = (uint32_t)(q_hi >> 32);
}
// signed 4-bit digits of a 128-bit value: 33 digits in [-7, 8]
DEV void recode_w4(const uint32_t v[4], int8_t d[33]) {
  int carry = 0;
  for (int i = 0; i < 32; i++) {
    int x = (int)((v[i >> 3] >> ((i & 7) * 4)) & 15) + carry;
    if (x > 8) { x -= 16; carry = 1; } else { carry = 0; }
    d[i] = (int8_t)x;
  }
  d[32] = (int8_t)carry;
}
// k * P (P affine, k canonical raw Fr).  Returns XYZZ.
DEV g1 g1_mul_glv(g1a p, fr k) {
  uint32_t s[4], q[4];
  glv_split(k, s, q);
  int8_t ds[33], dq[33];
  recode_w4(s, ds);
  recode_w4(q, dq);
  g1 tab[8];
  tab[0] = g1_from_aff(p);
  tab[1] = g1_dbl_aff(p);
  #pragma unroll 1
  for (int i = 2; i < 8; i++) tab[i] = g1_add_aff(tab[i - 1], p);
  g1 acc = g1_inf();
  #pragma unroll 1
  for (int i = 32; i >= 0; i--) {
    if (i != 32) {
      acc = g1_dbl(acc); acc = g1_dbl(acc); acc = g1_dbl(acc); acc = g1_dbl(acc);
    }
    int a = ds[i];
    if (a) {
      g1 t = tab[(a > 0 ? a : -a) - 1];
      acc = g1_add(acc, a > 0 ? t : g1_neg(t));
    }
    int b = dq[i];
    if (b) {
      g1 t = g1_endo(tab[(b > 0 ? b : -b) - 1]);
      acc = g1_add(acc, b > 0 ? t : g1_neg(t));
    }
  }
  return acc;
}

// g1_mul_glv on a lane pair (both lanes return k * P).  The multiples
// 1P..8P are brought to one common denominator, Z_c^2 = prod ZZ_j and
// Z_c^3 = prod ZZZ_j, by suffix and prefix products (no inversion): entry k
// becomes (X_k', Y_k') = (X_k prod_{j != k} ZZ_j, Y_k prod_{j != k} ZZZ_j), the
// affine point (x Z_c^2, y Z_c^3) of the isomorphic curve y^2 = x^3 + 4 Z_c^6.
// The doubling and mixed-addition formulas do not involve the curve's b, so
// the ladder runs on that curve with mixed additions (5 product rounds on a
// pair instead of 7 for an XYZZ addition) and precomputed phi-images
// (beta X_k', -Y_k'); the sum comes back with ZZ *= Z_c^2, ZZZ *= Z_c^3.  A
// point of small order (not in G1: rejected by the subgroup check) can make
// a multiple the identity, Z_c = 0 and the result meaningless, never a fault.
DEV g1 g1_mul_glv_pair(const LanePair &lp, g1a p, fr k) {
  uint32_t s[4], q[4];
  glv_split(k, s, q);
  int8_t ds[33], dq[33];
  recode_w4(s, ds);
  recode_w4(q, dq);
  g1 t[8];
  t[0] = g1_from_aff(p);
  t[1] = g1_dbl_pair(lp, t[0]);
  #pragma unroll 1
  for (int i = 2; i < 8; i++) t[i] = g1_add_aff_pair(lp, t[i - 1], p);
  // suffix products sz[k] = prod_{j > k} ZZ_j, szz[k] = prod_{j > k} ZZZ_j
  fp sz[8], szz[8];
  sz[7] = szz[7] = fp_one();
  sz[6] = t[7].ZZ;
  szz[6] = t[7].ZZZ;
  #pragma unroll 1
  for (int i = 5; i >= 0; i--) pair_mul(lp, sz[i + 1], t[i + 1].ZZ, szz[i + 1], t[i + 1].ZZZ, sz[i], szz[i]);
  const fp zc2 = sz[0], zc3 = szz[0];  // ZZ_0 = ZZZ_0 = 1
  // forward: pz = prod_{j < k} ZZ_j; X_k' = X_k pz sz[k], Y_k' = Y_k pzz szz[k] (in place)
  fp pz = fp_one(), pzz = fp_one();
  #pragma unroll 1
  for (int i = 0; i < 8; i++) {
    fp f = sz[i], g = szz[i];
    if (i > 0) pair_mul(lp, pz, sz[i], pzz, szz[i], f, g);
    if (i > 0 && i < 7) pair_mul(lp, pz, t[i].ZZ, pzz, t[i].ZZZ, pz, pzz);
    else if (i == 0) { pz = t[0].ZZ; pzz = t[0].ZZZ; }
    pair_mul(lp, t[i].X, f, t[i].Y, g, t[i].X, t[i].Y);
  }
  // phi-images: X of phi(entry k) in t[k].ZZ
  const fp beta = C_GLV_BETA;
  #pragma unroll 1
  for (int i = 0; i < 8; i += 2) pair_mul(lp, t[i].X, beta, t[i + 1].X, beta, t[i].ZZ, t[i + 1].ZZ);
  g1 acc = g1_inf();
  #pragma unroll 1
  for (int i = 32; i >= 0; i--) {
    if (i != 32) {
      acc = g1_dbl_pair(lp, acc); acc = g1_dbl_pair(lp, acc); acc = g1_dbl_pair(lp, acc); acc = g1_dbl_pair(lp, acc);
    }
    const int a = ds[i];
    if (a) {
      const g1 &e = t[(a > 0 ? a : -a) - 1];
      g1a pt;
      pt.x = e.X;
      pt.y = a > 0 ? e.Y : fp_neg(e.Y);
      acc = g1_add_aff_pair(lp, acc, pt);
    }
    const int b = dq[i];
    if (b) {
      const g1 &e = t[(b > 0 ? b : -b) - 1];
      g1a pt;
      pt.x = e.ZZ;  // beta X'
      pt.y = b > 0 ? fp_neg(e.Y) : e.Y;
      acc = g1_add_aff_pair(lp, acc, pt);
    }
  }
  pair_mul(lp, acc.ZZ, zc2, acc.ZZZ, zc3, acc.ZZ, acc.ZZZ);  // back to y^2 = x^3 + 4 (identity stays ZZ = 0)
  return acc;
}

// g1_mul_glv on a lane quad (all four lanes return k * P).
DEV g1 g1_mul_glv_quad(const LaneQuad &lq, g1a p, fr k) {
  uint32_t s[4], q[4];
  glv_split(k, s, q);
  int8_t ds[33], dq[33];
  recode_w4(s, ds);
  recode_w4(q, dq);
  g1 tab[8];
  tab[0] = g1_from_aff(p);
  tab[1] = g1_dbl_quad(lq, g1_from_aff(p));
  #pragma unroll 1
  for (int i = 2; i < 8; i++) tab[i] = g1_add_aff_quad(lq, tab[i - 1], p);
  g1 acc = g1_inf();
  #pragma unroll 1
  for (int i = 32; i >= 0; i--) {
    if (i != 32) {
      acc = g1_dbl_quad(lq, acc); acc = g1_dbl_quad(lq, acc); acc = g1_dbl_quad(lq, acc); acc = g1_dbl_quad(lq, acc);
    }
    int a = ds[i];
    if (a) {
      g1 t = tab[(a > 0 ? a : -a) - 1];
      acc = g1_add_quad(lq, acc, a > 0 ? t : g1_neg(t));
    }
    int b = dq[i];
    if (b) {
      g1 t = g1_endo(tab[(b > 0 ? b : -b) - 1]);
      acc = g1_add_quad(lq, acc, b > 0 ? t : g1_neg(t));
    }
  }
  return acc;
}

// k * P on eight lanes: the quad of lanes 8j .. 8j+3 computes s P and the quad
// of lanes 8j+4 .. 8j+7 computes q [lambda]P = q phi(P) (k = q lambda + s),
// each with its own doubling chain (half the additions of the shared chain
// each); the first quad adds the second quad's sum.  Lanes of the first quad
// return k * P.  All eight lanes must call it.
DEV g1 g1_mul_glv_octet(const LaneQuad &lq, g1a p, fr k) {
  uint32_t s[4], q[4];
  glv_split(k, s, q);
  const int half = (threadIdx.x >> 2) & 1;
  int8_t d[33];
  recode_w4(half ? q : s, d);
  if (half) {
    const fp beta = C_GLV_BETA;
    p.x = fp_mul(p.x, beta);  // phi(P) = (beta x, -y) = [lambda]P
    p.y = fp_neg(p.y);
  }
  g1 tab[8];
  tab[0] = g1_from_aff(p);
  tab[1] = g1_dbl_quad(lq, g1_from_aff(p));
  #pragma unroll 1
  for (int i = 2; i < 8; i++) tab[i] = g1_add_aff_quad(lq, tab[i - 1], p);
  g1 acc = g1_inf();
  #pragma unroll 1
  for (int i = 32; i >= 0; i--) {
    if (i != 32) {
      acc = g1_dbl_quad(lq, acc); acc = g1_dbl_quad(lq, acc); acc = g1_dbl_quad(lq, acc); acc = g1_dbl_quad(lq, acc);
    }
    const int a = d[i];
    if (a) {
      g1 t = tab[(a > 0 ? a : -a) - 1];
      acc = g1_add_quad(lq, acc, a > 0 ? t : g1_neg(t));
    }
  }
  // both quads meet here: the first takes the second's sum
  const unsigned oct = 0xFFu << (threadIdx.x & 24);
  g1 other;
#pragma unroll
  for (int i = 0; i < 12; i++) {
    other.X.w[i] = __shfl_xor_sync(oct, acc.X.w[i], 4);
    other.Y.w[i] = __shfl_xor_sync(oct, acc.Y.w[i], 4);
    other.ZZ.w[i] = __shfl_xor_sync(oct, acc.ZZ.w[i], 4);
    other.ZZZ.w[i] = __shfl_xor_sync(oct, acc.ZZZ.w[i], 4);
  }
  if (half) return acc;
  return g1_add_quad(lq, acc, other);
}

// ------------------------------------------------------------------ G2 (Jacobian over Fp2)
struct g2a { fp2 x, y; };
struct g2j { fp2 X, Y, Z; };

DEV fp2 g2_b() { const fp four = C_FP_FOUR; return {four, four}; }
DEV bool g2j_is_inf(const g2j &p) { return fp2_is_zero(p.Z); }
DEV g2j g2j_inf() { return {fp2_one(), fp2_one(), fp2_zero()}; }
DEV g2j g2j_from_aff(const g2a &a) { return {a.x, a.y, fp2_one()}; }
DEV g2j g2j_dbl(g2j p) {
  if (g2j_is_inf(p)) return p;
  fp2 A = fp2_sqr(p.X), B = fp2_sqr(p.Y), C = fp2_sqr(B);
  fp2 D = fp2_dbl(fp2_sub(fp2_sub(fp2_sqr(fp2_add(p.X, B)), A), C));
  fp2 E = fp2_add(fp2_dbl(A), A), F = fp2_sqr(E);
  g2j r;
  r.X = fp2_sub(F, fp2_dbl(D));
  fp2 C8 = fp2_dbl(fp2_dbl(fp2_dbl(C)));
  r.Y = fp2_sub(fp2_mul(E, fp2_sub(D, r.X)), C8);
  r.Z = fp2_dbl(fp2_mul(p.Y, p.Z));
  return r;
}
DEV g2j g2j_add(g2j p, g2j q) {
  if (g2j_is_inf(p)) return q;
  if (g2j_is_inf(q)) return p;
  fp2 Z1Z1 = fp2_sqr(p.Z), Z2Z2 = fp2_sqr(q.Z);
  fp2 U1 = fp2_mul(p.X, Z2Z2), U2 = fp2_mul(q.X, Z1Z1);
  fp2 S1 = fp2_mul(fp2_mul(p.Y, q.Z), Z2Z2), S2 = fp2_mul(fp2_mul(q.Y, p.Z), Z1Z1);
  if (fp2_eq(U1, U2)) {
    if (fp2_eq(S1, S2)) return g2j_dbl(p);
    return g2j_inf();
  }
  fp2 H = fp2_sub(U2, U1), I = fp2_sqr(fp2_dbl(H)), J = fp2_mul(H, I);
  fp2 rr = fp2_dbl(fp2_sub(S2, S1));
  fp2 V = fp2_mul(U1, I);
  g2j r;
  r.X = fp2_sub(fp2_sub(fp2_sqr(rr), J), fp2_dbl(V));
  r.Y = fp2_sub(fp2_mul(rr, fp2_sub(V, r.X)), fp2_dbl(fp2_mul(S1, J)));
  r.Z = fp2_mul(fp2_sub(fp2_sub(fp2_sqr(fp2_add(p.Z, q.Z)), Z1Z1), Z2Z2), H);
  return r;
}
DEV g2j g2j_neg(const g2j &p) { return {p.X, fp2_neg(p.Y), p.Z}; }
DEV bool g2j_to_aff(g2j p, g2a &out) {
  if (g2j_is_inf(p)) return false;
  fp2 zi = fp2_inv(p.Z), zi2 = fp2_sqr(zi);
  out.x = fp2_mul(p.X, zi2);
  out.y = fp2_mul(fp2_mul(p.Y, zi2), zi);
  return true;
}
// [r]P == O (naive membership test, used once per public key)
DEV bool g2_in_subgroup(g2a a) {
  const fr rm = FR_MOD_INIT;
  g2j p = g2j_from_aff(a), acc = g2j_inf();
  #pragma unroll 1
  for (int i = 254; i >= 0; i--) {
    acc = g2j_dbl(acc);
    if ((rm.w[i >> 5] >> (i & 31)) & 1) acc = g2j_add(acc, p);
  }
  return g2j_is_inf(acc);
}
DEV g2j g2j_mul_raw(g2a a, fr k) {
  g2j p = g2j_from_aff(a), acc = g2j_inf();
  #pragma unroll 1
  for (int i = 255; i >= 0; i--) {
    acc = g2j_dbl(acc);
    if ((k.w[i >> 5] >> (i & 31)) & 1) acc = g2j_add(acc, p);
  }
  return acc;
}
DEV int g2_decompress(const uint8_t in[96], g2a &out) {
  uint8_t f = in[0];
  bool comp = f & 0x80, inf = f & 0x40, sort = f & 0x20;
  uint8_t t[48];
  t[0] = f & 0x1f;
  #pragma unroll 1
  for (int i = 1; i < 48; i++) t[i] = in[i];
  fp2 x;
  if (!fp_from_be48(t, x.c1) || !fp_from_be48(in + 48, x.c0)) return DEC_BAD;
  if (inf) return (comp && !sort && fp2_is_zero(x)) ? DEC_INF : DEC_BAD;
  if (!comp) return DEC_BAD;
  fp2 y;
  if (!fp2_sqrt(fp2_add(fp2_mul(fp2_sqr(x), x), g2_b()), y)) return DEC_BAD;
  if (fp2_lex_largest(y) != sort) y = fp2_neg(y);
  out.x = x;
  out.y = y;
  if (!g2_in_subgroup(out)) return DEC_BAD;
  return DEC_OK;
}
DEV void g2_compress_aff(const g2a &a, uint8_t out[96]) {
  fp_to_be48(a.x.c1, out);
  fp_to_be48(a.x.c0, out + 48);
  out[0] |= 0x80;
  if (fp2_lex_largest(a.y)) out[0] |= 0x20;
}
DEV g2a g2_generator() {
  g2a g;
  const fp x0 = C_G2_GEN_X0, x1 = C_G2_GEN_X1, y0 = C_G2_GEN_Y0, y1 = C_G2_GEN_Y1;
  g.x = {x0, x1};
  g.y = {y0, y1};
  return g;
}
