// Warp-per-check pairing: one warp evaluates
//     e(P_a, Q_a) * e(P_b, Q_b) == 1
// with the Miller loop over the precomputed lines of pairing.cuh and the same
// final exponentiation, as a sequence of table-driven programs
// (pairing_program.cuh, generated and checked by gen_pairing_program.py).
//
// The check's state is an array of Fp slots in shared memory: six Fp12
// registers F, T, A, X, R, U (12 slots each), the current lines of both
// pairs, the two points, the Frobenius constants, a zero slot and the
// temporaries of the programs.  A program is a list of phases; in a phase
// every lane reads its table entry and either computes one Fp product of two
// short weighted sums of slots (MUL), one weighted sum of at most 14 slots
// (LIN), or, on lane 0, one Fp inverse (INV).  All lanes run the same
// instruction stream, the products of an Fp12 operation run side by side (up
// to 32 per phase), and results are written only after every lane of the
// phase has read its operands, so a program may overwrite its own input
// register.
//
// Compared with a 16-lane team working at Fp2 granularity, a phase costs one
// Fp product instead of three in a row, and the assembly of Karatsuba terms
// is a few multiply-adds per lane instead of divergent per-lane code.
//
// A team is one warp or two: the programs are compiled for both widths, and a
// two-warp team runs phases of up to 64 entries between named barriers, so an
// Fp12 product or a Miller step's squaring (36..54 products) takes one round of
// products instead of two.  Latency-bound checks (the group checks of an
// aggregated batch, small batches) use two-warp teams.
#pragma once
#include "pairing.cuh"
#include "pairing_program.cuh"

namespace pp {

DEV fp ld(const fp *sl, uint32_t i) {
  const uint4 *p = reinterpret_cast<const uint4 *>(sl + i);
  const uint4 a = p[0], b = p[1], c = p[2];
  fp r;
  r.w[0] = a.x; r.w[1] = a.y; r.w[2] = a.z; r.w[3] = a.w;
  r.w[4] = b.x; r.w[5] = b.y; r.w[6] = b.z; r.w[7] = b.w;
  r.w[8] = c.x; r.w[9] = c.y; r.w[10] = c.z; r.w[11] = c.w;
  return r;
}
DEV void st(fp *sl, uint32_t i, const fp &r) {
  uint4 *p = reinterpret_cast<uint4 *>(sl + i);
  p[0] = make_uint4(r.w[0], r.w[1], r.w[2], r.w[3]);
  p[1] = make_uint4(r.w[4], r.w[5], r.w[6], r.w[7]);
  p[2] = make_uint4(r.w[8], r.w[9], r.w[10], r.w[11]);
}

constexpr uint32_t PP_SLOT_MASK = 0x1ffu;  // term = slot | signed 7-bit coefficient << 9

DEV uint32_t term(const uint4 &e, int t) {
  const uint32_t w = t < 2 ? e.y : t < 4 ? e.z : e.w;
  return (t & 1) ? w >> 16 : w & 0xffffu;
}

// Signed sum of N reduced slots with coefficients +-1 (N is the same on every
// lane of a phase): a subtracted term x enters as p - x, every term is loaded
// and prepared before the sums, and the terms are added as a pairwise tree of
// plain 12-limb additions (every partial sum stays below N p <= 6p < 2^384);
// conditional subtractions of 4p, 2p and p, as many as N needs, reduce the
// result once.  No branch depends on the lane.
template <int N> DEV fp lin_n(const fp *sl, const uint4 &e) {
  fp v[N];
#pragma unroll
  for (int t = 0; t < N; t++) {
    const uint32_t tv = term(e, t);
    const fp x = ld(sl, tv & PP_SLOT_MASK);
    fp y;
    fp_from_mod(y.w, x.w);
    const bool neg = (tv & 0x8000u) != 0;
#pragma unroll
    for (int k = 0; k < 12; k++) v[t].w[k] = neg ? y.w[k] : x.w[k];
  }
#pragma unroll
  for (int w = 1; w < N; w *= 2) {
#pragma unroll
    for (int t = 0; t + w < N; t += 2 * w) fp_acc_add(v[t].w, v[t].w, v[t + w].w);
  }
  if (N >= 4) fp_csub4(v[0].w, v[0].w);
  if (N >= 2) fp_csub2(v[0].w, v[0].w);
  fp_csub1(v[0].w, v[0].w);
  return v[0];
}
DEV fp lin(const fp *sl, const uint4 &e, int n) {
  switch (n) {
    case 1: return lin_n<1>(sl, e);
    case 2: return lin_n<2>(sl, e);
    case 3: return lin_n<3>(sl, e);
    case 4: return lin_n<4>(sl, e);
    case 5: return lin_n<5>(sl, e);
    default: return lin_n<6>(sl, e);
  }
}

// Up to 14 terms of an entry as a shift register: term t in bits 16 t .. 16 t + 15.
struct Terms {
  uint32_t w[7];
};
DEV Terms terms_lo(const uint4 &e0, const uint4 &e1) {  // terms 0..13
  return {{e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w}};
}
DEV Terms terms_hi(const uint4 &e1) {  // terms 7..13
  return {{__funnelshift_r(e1.x, e1.y, 16), __funnelshift_r(e1.y, e1.z, 16), __funnelshift_r(e1.z, e1.w, 16),
           e1.w >> 16, 0u, 0u, 0u}};
}

// sum_t k_t slot[s_t] mod p over the first n terms of q (n is the same on
// every lane of a phase; |k_t| <= 64, n <= 14).  A term with k < 0 enters as
// |k| (p - x).  The products accumulate per limb in 64 bits (at most
// 14 * 64 * 2^32 < 2^42 each), so S = sum_j acc_j 2^(32 j) < 896 p < 2^391.
// Before any carry, q = floor(S / p) - (0..3) comes from the top of S,
// acc_11 + floor(acc_10 / 2^32) (S / 2^352 less at most 1), times
// 1 / (floor(p / 2^352) + 1) in single precision (relative error below 2^-22
// on a quotient below 2^10), minus one; q p is taken off limb by limb and one
// signed carry pass leaves S - q p in [0, 4p).  Two conditional subtractions
// finish the reduction.
DEVNI fp wsum(const fp *sl, Terms q, int n) {
  const fp pm = FP_MOD_INIT;
  uint64_t acc[12];
#pragma unroll
  for (int j = 0; j < 12; j++) acc[j] = 0;
#pragma unroll 1
  for (int t = 0; t < n; t++) {
    const uint32_t v = q.w[0] & 0xffffu;
#pragma unroll
    for (int i = 0; i < 6; i++) q.w[i] = __funnelshift_r(q.w[i], q.w[i + 1], 16);
    q.w[6] >>= 16;
    const fp x = ld(sl, v & PP_SLOT_MASK);
    fp y;
    fp_from_mod(y.w, x.w);
    const int k = (int32_t)(v << 16) >> 25;
    const bool neg = k < 0;
    const uint32_t m = (uint32_t)(neg ? -k : k);
#pragma unroll
    for (int j = 0; j < 12; j++) acc[j] += (uint64_t)(neg ? y.w[j] : x.w[j]) * m;
  }
  constexpr float INV_PTOP = 1.0f / 436277739.0f;  // 1 / (floor(p / 2^352) + 1)
  const uint64_t top = acc[11] + (acc[10] >> 32);
  uint32_t qq = (uint32_t)(__ull2float_rn(top) * INV_PTOP);
  qq = qq ? qq - 1 : 0;
  int64_t c = 0;
  fp out;
#pragma unroll
  for (int j = 0; j < 12; j++) {
    c += (int64_t)acc[j] - (int64_t)((uint64_t)qq * pm.w[j]);
    out.w[j] = (uint32_t)c;
    c >>= 32;
  }
  fp_csub2(out.w, out.w);
  fp_csub1(out.w, out.w);
  return out;
}

// Synchronisation of a team of W lanes: one warp (W = 32), or two consecutive
// warps (W = 64) on named barrier `bar` (1..15; barrier 0 is __syncthreads),
// which also orders their shared-memory accesses.
template <int W> DEV void team_sync(int bar) {
  if constexpr (W == 32) {
    __syncwarp();
  } else {
    static_assert(W == 64, "teams are one or two warps");
    asm volatile("bar.sync %0, 64;" ::"r"(bar) : "memory");
  }
}

// Runs program `prog` on the slot array of this team's check, from the phase
// tables of its width (PP_ENTRY: one warp; PP_ENTRY_W: two warps, whose
// phases hold up to 64 entries, so an Fp12 product takes one round of
// products instead of two).  The table entry of the next phase is fetched
// while the current one computes.
template <int W = 32> DEVNI void run(fp *sl, int lane, int prog, int bar = 0) {
  const uint16_t *first = W == 32 ? PP_PROG_FIRST : PP_PROG_FIRST_W;
  const int ph0 = first[prog], ph1 = first[prog + 1];
  const uint4 *tab = (W == 32 ? PP_ENTRY : PP_ENTRY_W) + 2 * lane;
  uint4 e0 = __ldg(&tab[2 * W * ph0]), e1 = __ldg(&tab[2 * W * ph0 + 1]);
#pragma unroll 1
  for (int ph = ph0; ph < ph1; ph++) {
    const int nx = min(ph + 1, ph1 - 1);
    const uint4 n0 = __ldg(&tab[2 * W * nx]), n1 = __ldg(&tab[2 * W * nx + 1]);
    const uint32_t out = e0.x & 0xffffu, tw = e0.x >> 16, type = tw >> 12;
    const int na = (int)(tw & 15u), nb = (int)((tw >> 4) & 15u);
    const bool act = out != PP_NONE;
    fp r = fp_zero();
    if (act) {
      if (type == PP_MUL) {
        const fp x = (tw & PP_F_PLAIN_A) ? ld(sl, e0.y & PP_SLOT_MASK) : wsum(sl, terms_lo(e0, e1), na);
        const fp y = (tw & PP_F_PLAIN_B) ? ld(sl, (e1.x >> 16) & PP_SLOT_MASK) : wsum(sl, terms_hi(e1), nb);
        // one dependent product per lane, inlined: the PTX carry-save form
        // (1965 cycles a product on one warp against 2802 for the CIOS form
        // this replaced; the aggregated check 1.88 -> 1.73 ms, C1 Verify
        // 17.2k -> 18.1k ops/s on GB300)
        r = fp_mul_inl(x, y);
      } else if (type == PP_LIN) {
        r = (tw & PP_F_UNIT) ? lin(sl, e0, na) : wsum(sl, terms_lo(e0, e1), na);
      } else {
        r = fp_inv_vartime(ld(sl, e0.y & PP_SLOT_MASK));  // PP_INV: public value, variable time
      }
    }
    team_sync<W>(bar);
    if (act) st(sl, out, r);
    team_sync<W>(bar);
    e0 = n0;
    e1 = n1;
  }
}

// dst = base^|z| for base in the cyclotomic subgroup (dst register R).
template <int W = 32> DEV void exp_by_zabs(fp *sl, int lane, int copy_prog, int mul_prog, int bar = 0) {
  run<W>(sl, lane, copy_prog, bar);
#pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    run<W>(sl, lane, PP_CYCLO_R, bar);
    if (zabs_bit(i)) run<W>(sl, lane, mul_prog, bar);
  }
}

// Final exponentiation of register F; true (on every lane) when the result is 1.
// Same steps as final_exponentiation of pairing.cuh:
//   t = conj(f) f^-1, t = t^(p^2) t;  a = t^z conj(t);  a = a^z conj(a);
//   b = a^z a^p;  c = (b^z)^z b^(p^2) conj(b);  result c t^3.
template <int W = 32> DEV bool final_exp_is_one(fp *sl, int lane, int bar = 0) {
  run<W>(sl, lane, PP_INV_U_F, bar);
  run<W>(sl, lane, PP_EASY1_T, bar);
  run<W>(sl, lane, PP_EASY2_T, bar);
  exp_by_zabs<W>(sl, lane, PP_COPY_R_T, PP_MUL_R_R_T, bar);
  run<W>(sl, lane, PP_S1_A, bar);  // a = conj(t^|z|) conj(t)
  exp_by_zabs<W>(sl, lane, PP_COPY_R_A, PP_MUL_R_R_A, bar);
  run<W>(sl, lane, PP_S2_A, bar);  // a = conj(a^|z|) conj(a)
  exp_by_zabs<W>(sl, lane, PP_COPY_R_A, PP_MUL_R_R_A, bar);
  run<W>(sl, lane, PP_S3_A, bar);  // b = conj(a^|z|) a^p
  exp_by_zabs<W>(sl, lane, PP_COPY_R_A, PP_MUL_R_R_A, bar);
  run<W>(sl, lane, PP_S4_X, bar);  // x = b^z
  exp_by_zabs<W>(sl, lane, PP_COPY_R_X, PP_MUL_R_R_X, bar);
  run<W>(sl, lane, PP_S5_R, bar);  // r = (b^z)^z b^(p^2)
  run<W>(sl, lane, PP_MUL_R_R_CA, bar);  // r = r conj(b)
  run<W>(sl, lane, PP_MUL_R_R_T, bar);
  run<W>(sl, lane, PP_MUL_R_R_T, bar);
  run<W>(sl, lane, PP_MUL_R_R_T, bar);
  if constexpr (W == 32) {
    bool mine = true;
    if (lane < 12) {
      const fp v = ld(sl, PP_REG(PP_REG_R) + lane);
      mine = lane == 0 ? fp_eq(v, fp_one()) : fp_is_zero(v);
    }
    return __ballot_sync(0xffffffffu, !mine) == 0;
  } else {
    // every lane reads the result register (written before the last team_sync)
    bool one = fp_eq(ld(sl, PP_REG(PP_REG_R)), fp_one());
#pragma unroll 1
    for (int k = 1; k < 12; k++) one = one && fp_is_zero(ld(sl, PP_REG(PP_REG_R) + k));
    return one;
  }
}

// Lines idx of both pairs into the line slots (lanes 0..7); a skipped pair
// gets the line 1 (A = 1, B = 0).
DEV void load_lines(fp *sl, int lane, const line2 *const *L, const bool *skip, int idx) {
  if (lane < 8) {
    const int p = lane >> 2, c = lane & 3;
    fp v;
    if (skip[p]) {
      v = c == 0 ? fp_one() : fp_zero();
    } else {
      const line2 &l = L[p][idx];
      v = c == 0 ? l.a.c0 : c == 1 ? l.a.c1 : c == 2 ? l.b.c0 : l.b.c1;
    }
    st(sl, PP_LINE_BASE + lane, v);
  }
  __syncwarp();
}

// The whole check for one warp.  P[p] affine (ignored when skip[p]).
DEV bool pairing_check(fp *sl, int lane, const g1a *P, const line2 *const *L, const bool *skip) {
  if (lane < 10) {
    const fp2 g[6] = C_FROB_GAMMA;
    const fp2 &ge = g[1 + (lane >> 1)];
    st(sl, PP_GAMMA_BASE + lane, (lane & 1) ? ge.c1 : ge.c0);
  } else if (lane < 14) {
    const int p = (lane - 10) >> 1;
    st(sl, PP_PT_BASE + lane - 10, skip[p] ? fp_zero() : ((lane & 1) ? P[p].y : P[p].x));
  } else if (lane == 14) {
    st(sl, PP_ZERO_SLOT, fp_zero());
  } else if (lane >= 16 && lane < 28) {
    st(sl, PP_REG(PP_REG_F) + lane - 16, lane == 16 ? fp_one() : fp_zero());
  }
  __syncwarp();
  int idx = 0;
#pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    load_lines(sl, lane, L, skip, idx++);
    run(sl, lane, PP_DBL);
    if (zabs_bit(i)) {
      load_lines(sl, lane, L, skip, idx++);
      run(sl, lane, PP_ADD);
    }
  }
  run(sl, lane, PP_CONJ_F);  // z < 0
  return final_exp_is_one(sl, lane);
}

// ---- one pair per warp
// The Miller loop of a single pair (P, lines L) into register F of this warp's
// slot array; a skipped pair leaves F = 1.  Also loads the Frobenius constants
// and the zero slot, so the warp can run the final exponentiation after.
template <int W = 32> DEV void miller_one(fp *sl, int lane, const g1a &P, const line2 *L, bool skip, int bar = 0) {
  if (lane < 10) {
    const fp2 g[6] = C_FROB_GAMMA;
    const fp2 &ge = g[1 + (lane >> 1)];
    st(sl, PP_GAMMA_BASE + lane, (lane & 1) ? ge.c1 : ge.c0);
  } else if (lane < 12) {
    st(sl, PP_PT_BASE + lane - 10, skip ? fp_zero() : ((lane & 1) ? P.y : P.x));
  } else if (lane == 14) {
    st(sl, PP_ZERO_SLOT, fp_zero());
  } else if (lane >= 16 && lane < 28) {
    st(sl, PP_REG(PP_REG_F) + lane - 16, lane == 16 ? fp_one() : fp_zero());
  }
  team_sync<W>(bar);
  int idx = 0;
#pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    if (lane < 4) {
      fp v;
      if (skip) v = lane == 0 ? fp_one() : fp_zero();
      else {
        const line2 &l = L[idx];
        v = lane == 0 ? l.a.c0 : lane == 1 ? l.a.c1 : lane == 2 ? l.b.c0 : l.b.c1;
      }
      st(sl, PP_LINE_BASE + lane, v);
    }
    team_sync<W>(bar);
    idx++;
    run<W>(sl, lane, PP_DBL1, bar);
    if (zabs_bit(i)) {
      if (lane < 4) {
        fp v;
        if (skip) v = lane == 0 ? fp_one() : fp_zero();
        else {
          const line2 &l = L[idx];
          v = lane == 0 ? l.a.c0 : lane == 1 ? l.a.c1 : lane == 2 ? l.b.c0 : l.b.c1;
        }
        st(sl, PP_LINE_BASE + lane, v);
      }
      team_sync<W>(bar);
      idx++;
      run<W>(sl, lane, PP_ADD1, bar);
    }
  }
}

}  // namespace pp
