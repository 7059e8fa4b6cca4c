// The four BBS operations, fully on the device, behind the required ABI
// symbols (reference stubs: native/cuda/src/cubbs_bbs_cuda.cu:826-835,1169-1200).
//
// Protocol steps follow crates/cubbs-bbs-protocol/src/bbsplus/signature.rs:
// 544-728 (Sign, Verify) and proof.rs:1568-1867, 2155-2426, 3015-3078
// (ProofGen, ProofVerify); Verify uses the fixed-G2 rewrite
// e(A, PK) * e(B - e A, -P2) == 1 (crates/cubbs-bbs/src/execution.rs:390-430)
// so both G2 arguments have resident Miller lines.
//
// Pipeline per batch (one stream): hash messages -> decode points -> domain ->
// per-item scalar prep (Fr) -> fixed-base MSM against the generator tables +
// GLV variable-base terms -> per-item finish (compress, challenge hash) ->
// 2-pair pairing check.  The host only validates argument shapes, sorts
// disclosed indexes, packs bytes and copies results back.
#include <sys/random.h>

#include <algorithm>
#include <chrono>
#include <thread>
#include <mutex>
#include <condition_variable>
#include <functional>
#include <cstdio>
#include <cstring>

#include "bbs_dst.cuh"
#include "runtime.cuh"
#include "suite.cuh"

namespace cubbs {

// ----------------------------------------------------------------------------- raw Fr helpers
DEVNI fr frr_mul(fr a, fr b) { return fr_mul(a, fr_to_mont(b)); }
DEV fr frr_inv(fr a) { return fr_from_mont(fr_inv(fr_to_mont(a))); }
DEV fr frr_neg(const fr &a) { return fr_sub(fr_zero(), a); }
DEV fr frr_one() { fr r = fr_zero(); r.w[0] = 1; return r; }

DEV void sha_fr_be(sha_ctx &c, const fr &raw) {
  uint8_t b[32];
  fr_raw_to_be32(raw, b);
  sha_bytes(c, b, 32);
}

// Debug record of item 0 of the last ProofGen / ProofVerify finish kernel:
// [0,48) T1, [48,96) T2, [96,128) domain BE, [128,160) challenge BE,
// [160,164) R, [164,180) first four disclosed indexes, [180,212) first disclosed scalar BE.
__device__ uint8_t g_debug_record[256];
DEV void debug_record(const uint8_t *t1c, const uint8_t *t2c, const fr &dom, const fr &ch, uint32_t R,
                      const uint32_t *idx, const fr *m0) {
  for (int k = 0; k < 48; k++) { g_debug_record[k] = t1c[k]; g_debug_record[48 + k] = t2c[k]; }
  fr_raw_to_be32(dom, g_debug_record + 96);
  fr_raw_to_be32(ch, g_debug_record + 128);
  for (int k = 0; k < 4; k++) g_debug_record[160 + k] = (uint8_t)(R >> (8 * k));
  for (uint32_t j = 0; j < 4; j++) {
    uint32_t v = j < R ? idx[j] : 0xffffffffu;
    for (int k = 0; k < 4; k++) g_debug_record[164 + 4 * j + k] = (uint8_t)(v >> (8 * k));
  }
  if (R && m0) fr_raw_to_be32(*m0, g_debug_record + 180);
}

// Item status codes kept on the device
#define ST_OK 0
#define ST_INVALID 1      // verification input does not decode: value 0
#define ST_ERROR 2        // per-item error (code INVALID_INPUT)

// ============================================================================ ProofVerify
struct PvItem {
  uint32_t proof_off, U, hdr_off, hdr_len, ph_off, ph_len, idx_off, R, msg_base, L;
  int32_t pk_slot, pk_status;
  int32_t status;  // host-side status
};

// Parse the scalars of the proof and build its T2 fixed-base row.  Needs no
// decoded point, so the fixed-base MSM can run while the points decode.
__global__ void __launch_bounds__(128) k_pv_rows(PvItem *items, uint32_t n, const uint8_t *blob, const fr *msc,
                                                 const fr *domain, fr *rows, uint32_t stride, uint32_t *nterms) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  PvItem it = items[i];
  bool ok = it.status == ST_OK && it.pk_status != DEC_BAD;
  const uint8_t *pr = blob + it.proof_off;
  fr ecap, r1cap, r3cap, c;
  if (ok) ok = fr_raw_from_be32(pr + 144, ecap) && fr_raw_from_be32(pr + 176, r1cap) &&
               fr_raw_from_be32(pr + 208, r3cap) && fr_raw_from_be32(pr + 240 + 32 * it.U, c);
  #pragma unroll 1
  for (uint32_t j = 0; j < it.U && ok; j++) {
    fr t;
    ok = fr_raw_from_be32(pr + 240 + 32 * j, t);
  }
  fr *row = rows + (size_t)i * stride;
  if (!ok) {
    items[i].status = ST_INVALID;
    nterms[i] = 0;
    return;
  }
  nterms[i] = it.L + 2;
  row[0] = c;
  row[1] = frr_mul(domain[i], c);
  const uint32_t *idx = reinterpret_cast<const uint32_t *>(blob + it.idx_off);
  uint32_t k = 0, u = 0;
  #pragma unroll 1
  for (uint32_t m = 0; m < it.L; m++) {
    if (k < it.R && idx[k] == m) {
      row[2 + m] = frr_mul(msc[it.msg_base + k], c);
      k++;
    } else {
      fr t;
      fr_raw_from_be32(pr + 240 + 32 * u, t);
      row[2 + m] = t;
      u++;
    }
  }
}

// The four variable-base jobs of each proof, from the untouched input items
// and the decoded points: the terms of T1 (Bbar*c, Abar*e^, D*r1^) as jobs
// 3i .. 3i+2 and D*r3^ as job 3n + i; a proof whose points or scalars do not
// decode gets jobs at infinity (k_pv_rows and k_pv_finish mark it invalid).
__global__ void __launch_bounds__(128) k_pv_jobs(const PvItem *items0, uint32_t n, const uint8_t *blob,
                                                 const int32_t *dec_status, VarJob *jobs, fr *jscal) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PvItem it = items0[i];
  bool ok = it.status == ST_OK && it.pk_status != DEC_BAD;
  #pragma unroll 1
  for (int k = 0; k < 3 && ok; k++) ok = dec_status[3 * i + k] != DEC_BAD;
  const uint8_t *pr = blob + it.proof_off;
  fr ecap, r1cap, r3cap, c;
  if (ok) ok = fr_raw_from_be32(pr + 144, ecap) && fr_raw_from_be32(pr + 176, r1cap) &&
               fr_raw_from_be32(pr + 208, r3cap) && fr_raw_from_be32(pr + 240 + 32 * it.U, c);
  if (!ok) {
    for (int k = 0; k < 3; k++) jobs[3 * i + k] = {0, 1};
    jobs[3 * n + i] = {0, 1};
    return;
  }
  // points: 3i+0 Abar, 3i+1 Bbar, 3i+2 D
  uint32_t fa = dec_status[3 * i] == DEC_INF, fb = dec_status[3 * i + 1] == DEC_INF, fd = dec_status[3 * i + 2] == DEC_INF;
  jobs[3 * i + 0] = {3 * i + 1, fb};
  jscal[3 * i + 0] = c;
  jobs[3 * i + 1] = {3 * i + 0, fa};
  jscal[3 * i + 1] = ecap;
  jobs[3 * i + 2] = {3 * i + 2, fd};
  jscal[3 * i + 2] = r1cap;
  jobs[3 * n + i] = {3 * i + 2, fd};
  jscal[3 * n + i] = r3cap;
}

// Pairing job of each proof, built from the untouched input items and the
// decoded points alone, so that the pairing can run beside the MSMs and the
// challenge (the item is valid only if both checks pass).
__global__ void __launch_bounds__(128) k_pv_pairjobs(const PvItem *items0, uint32_t n, const g1a *pts,
                                                     const int32_t *dec_status, PairJob *pj) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PvItem it = items0[i];
  PairJob job;
  job.slot_a = it.pk_slot < 0 ? 0 : it.pk_slot;
  job.slot_b = 0;
  job.pa = pts[3 * i];
  job.pb = pts[3 * i + 1];
  job.flags = 0;
  bool ok = it.status == ST_OK && it.pk_status != DEC_BAD;
  #pragma unroll 1
  for (int k = 0; k < 3; k++) ok = ok && dec_status[3 * i + k] != DEC_BAD;
  job.active = ok ? 1 : 0;
  if (dec_status[3 * i] == DEC_INF || it.pk_status == DEC_INF) job.flags |= 1;
  if (dec_status[3 * i + 1] == DEC_INF) job.flags |= 2;
  pj[i] = job;
}

// ---------------------------------------------------------------- aggregated pairing checks
// Proofs under one public key are checked together, as the reference's GPU
// engine does for ProofVerify batches of 128 or more
// (crates/cubbs-bbs/src/gpu_engine.rs:2095-2108, execution.rs:3797-3801;
// protocol form core_proof_pairing_verify_batch, proof.rs:2656-2710): with
// random coefficients rho_i,
//     e(sum rho_i Abar_i, PK) * e(sum rho_i Bbar_i, -P2) == 1
// holds for a group whose items all pass their own check, and fails with
// probability at least 1 - 2^-63 when one item of the group fails its own
// check.  rho_i = a_i + b_i lambda with a_i in [2^31, 2^32), b_i in [0, 2^32)
// drawn per call from OS randomness (lambda = z^2 is the eigenvalue of the GLV
// endomorphism, so the 2^63 values are distinct below r, and
// rho_i P = a_i P + b_i phi(P) needs only 32-bit scalars); every pairing value lies in
// the order-r subgroup of Fp12*.  A group that fails is checked item by item,
// so every item's result equals its own check.
struct AggSeed {
  uint32_t w[8];
};

// (a_i, b_i) = the first 8 bytes of SHA-256(seed || I2OSP(i, 4)), big-endian,
// with the top bit of a_i set.
DEV void agg_rho(const AggSeed &seed, uint32_t i, uint32_t &a, uint32_t &b) {
  sha_ctx c;
  sha_init(c);
  uint8_t m[36];
  for (int k = 0; k < 8; k++)
    for (int j = 0; j < 4; j++) m[4 * k + j] = (uint8_t)(seed.w[k] >> (8 * j));
  for (int j = 0; j < 4; j++) m[32 + j] = (uint8_t)(i >> (24 - 8 * j));
  sha_bytes(c, m, 36);
  uint8_t h[32];
  sha_final(c, h);
  a = ((uint32_t)h[0] << 24 | (uint32_t)h[1] << 16 | (uint32_t)h[2] << 8 | h[3]) | 0x80000000u;
  b = (uint32_t)h[4] << 24 | (uint32_t)h[5] << 16 | (uint32_t)h[6] << 8 | h[7];
}

// The sums of a group, R_s = sum_i rho_i P_{i,s} (set 0: Abar_i or A_i, set 1:
// Bbar_i or B_i - e_i A_i), as one bucket MSM per (group, set).  With
// rho_i P = a_i P + b_i phi(P), a group of n_g items is an MSM of 2 n_g points
// with 32-bit scalars, cut into four 8-bit windows:
//   k_agg_prep_*   one thread per item: rho_i, phi of its two points;
//   k_agg_sort     per (group, set, window): counting sort of the entries by
//                  digit (bucket), offsets in boff;
//   k_agg_buckets  one lane pair per bucket j: the sum of its points (mixed
//                  additions), times j; the 16 pairs of a warp add theirs;
//   k_agg_combine  per (group, set): one warp per window adds its 16 warp sums
//                  and doubles 8 w times (lane quad); the four windows are
//                  added and written, affine, into the group's pairing job.
// About a fifth of the work of one 31-step ladder per point, and the depth of
// the chain is a few bucket additions, one 8-bit multiple and 24 doublings.
// The order of the additions inside a bucket is not fixed (the sort places
// entries by atomics), but the sum is a group element and its affine form is
// unique, so the pairing input and every verdict are deterministic.
constexpr uint32_t AGG_SLAB = 8;  // (set, window) slabs per group: 2 sets x 4 windows

// pts4[4i + 2s] = P_{i,s}, pts4[4i + 2s + 1] = phi(P_{i,s}) = (beta x, -y) =
// [lambda]P; sc[2i + s] = (a_i, b_i), or (0, 0) when the point takes no part
// (every digit 0: bucket 0 collects it and is never summed).
DEV void agg_put(uint32_t i, uint32_t s, bool use, const g1a &p, uint32_t a, uint32_t b, g1a *pts4, uint2 *sc) {
  g1a e = p;
  if (use) {
    const fp beta = C_GLV_BETA;
    e.x = fp_mul(p.x, beta);
    e.y = fp_neg(p.y);
  }
  pts4[4 * i + 2 * s] = p;
  pts4[4 * i + 2 * s + 1] = e;
  sc[2 * i + s] = use ? make_uint2(a, b) : make_uint2(0u, 0u);
}
// ProofVerify: items of an aggregated group whose three points decoded take
// part; an identity Abar or Bbar adds nothing (rho O = O).
__global__ void __launch_bounds__(128) k_agg_prep_pv(const PvItem *items0, uint32_t n, const g1a *pts,
                                                     const int32_t *dec, const int32_t *group_of, AggSeed seed,
                                                     g1a *pts4, uint2 *sc) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || group_of[i] < 0) return;
  const PvItem it = items0[i];
  bool use = it.status == ST_OK && it.pk_status == DEC_OK;
  #pragma unroll 1
  for (int k = 0; k < 3 && use; k++) use = dec[3 * i + k] != DEC_BAD;
  uint32_t a, b;
  agg_rho(seed, i, a, b);
  agg_put(i, 0, use && dec[3 * i] == DEC_OK, pts[3 * i], a, b, pts4, sc);
  agg_put(i, 1, use && dec[3 * i + 1] == DEC_OK, pts[3 * i + 1], a, b, pts4, sc);
}
// Verify: the two points of the item's own pairing job (A and B - e A); a job
// that is not evaluated, or a point the job skips (the identity), adds nothing.
__global__ void __launch_bounds__(128) k_agg_prep_vf(const PairJob *pj, uint32_t n, const int32_t *group_of,
                                                     AggSeed seed, g1a *pts4, uint2 *sc) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || group_of[i] < 0) return;
  const PairJob j = pj[i];
  const bool use = j.active == 1;
  uint32_t a, b;
  agg_rho(seed, i, a, b);
  agg_put(i, 0, use && !(j.flags & 1u), j.pa, a, b, pts4, sc);
  agg_put(i, 1, use && !(j.flags & 2u), j.pb, a, b, pts4, sc);
}

// Grid (groups, 8): block (g, 4 s + w) sorts the 2 n_g entries of set s,
// window w of group g (entry 2m + h: item perm[goff[g] + m], h = 0 for a_i P,
// 1 for b_i phi(P)) by their digit d = byte w of the scalar.  The indexes into
// pts4 go to ent[(4 s + w) * 2 M + 2 goff[g] ..] bucket by bucket (M = number
// of grouped items); bucket d spans [bo[d], bo[d + 1]) of that slab, with
// bo = boff + (8 g + 4 s + w) * 257.
__global__ void __launch_bounds__(256) k_agg_sort(const uint32_t *perm, const uint32_t *goff, const uint2 *sc,
                                                  uint32_t M, uint32_t *ent, uint32_t *boff) {
  __shared__ uint32_t cnt[256], wsum[8];
  const uint32_t g = blockIdx.x, sw = blockIdx.y, s = sw >> 2, w = sw & 3, t = threadIdx.x;
  const uint32_t lane = t & 31, warp = t >> 5;
  const uint32_t g0 = goff[g], ng = goff[g + 1] - g0;
  cnt[t] = 0;
  __syncthreads();
  #pragma unroll 1
  for (uint32_t k = t; k < 2 * ng; k += 256) {
    const uint2 v = sc[2 * perm[g0 + (k >> 1)] + s];
    atomicAdd(&cnt[(((k & 1) ? v.y : v.x) >> (8 * w)) & 255u], 1u);
  }
  __syncthreads();
  const uint32_t c = cnt[t];
  uint32_t incl = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= (uint32_t)d) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  uint32_t base = 2 * g0;
  for (uint32_t k = 0; k < warp; k++) base += wsum[k];
  const uint32_t excl = base + incl - c;
  uint32_t *bo = boff + (size_t)(AGG_SLAB * g + sw) * 257;
  bo[t] = excl;
  if (t == 255) bo[256] = excl + c;
  __syncthreads();  // every thread has read cnt[t]
  cnt[t] = excl;
  __syncthreads();
  uint32_t *e = ent + (size_t)sw * 2 * M;
  #pragma unroll 1
  for (uint32_t k = t; k < 2 * ng; k += 256) {
    const uint32_t i = perm[g0 + (k >> 1)];
    const uint2 v = sc[2 * i + s];
    const uint32_t d = (((k & 1) ? v.y : v.x) >> (8 * w)) & 255u;
    e[atomicAdd(&cnt[d], 1u)] = 4 * i + 2 * s + (k & 1);
  }
}

// Sum of the 16 pairs' points of a warp (valid on lanes 0 and 1).
DEV g1 shfl_down_g1_all(const g1 &p, int delta) {
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
DEV g1 warp_sum_pairs(const LanePair &lp, g1 acc) {
#pragma unroll 1
  for (int d = 2; d < 32; d *= 2) {
    const g1 o = shfl_down_g1_all(acc, d);
    const bool has = ((threadIdx.x & 31) + d) < 32;
    const g1 sum = g1_add_pair(lp, acc, o);
    if (has) acc = sum;
  }
  return acc;
}

// 64 blocks of 64 threads per group: block 8 q + c (q = 8 g + 4 s + w) gives
// buckets 32 c .. 32 c + 31 of slab q one lane pair each.  A pair adds the
// points of its bucket j (mixed additions) and multiplies the sum by j (from
// its top bit down; the additions are kept by a select, and the pairs of a
// warp share every bit but the low four, so they stay together); the 16 pairs
// of each warp add their products, and lanes 0 and 1 write the warp's sum to
// part[16 q + 2 c + warp].
__global__ void __launch_bounds__(64) k_agg_buckets(const g1a *pts4, const uint32_t *ent, const uint32_t *boff,
                                                    uint32_t M, g1 *part) {
  const uint32_t q = blockIdx.x >> 3, c = blockIdx.x & 7, sw = q % AGG_SLAB;
  const LanePair lp = LanePair::here();
  const uint32_t j = 32 * c + (threadIdx.x >> 1);
  const uint32_t *bo = boff + (size_t)q * 257;
  const uint32_t *e = ent + (size_t)sw * 2 * M;
  g1 sum = g1_inf();
  if (j) {
    const uint32_t k1 = bo[j + 1];
    #pragma unroll 1
    for (uint32_t k = bo[j]; k < k1; k++) sum = g1_add_aff_pair(lp, sum, pts4[e[k]]);
  }
  g1 r = sum;
  #pragma unroll 1
  for (int bit = j ? 30 - __clz(j) : -1; bit >= 0; bit--) {
    r = g1_dbl_pair(lp, r);
    const g1 t = g1_add_pair(lp, r, sum);
    if ((j >> bit) & 1) r = t;
  }
  r = warp_sum_pairs(lp, r);
  if ((threadIdx.x & 31) == 0) part[(size_t)q * 16 + 2 * c + (threadIdx.x >> 5)] = r;
}

// Grid (groups, 2), 128 threads: warp w adds the 16 warp sums of window w of
// set s (one per lane pair), then every quad of the warp doubles that sum 8 w
// times; the four windows are added by warp 0, and lane 0 writes the affine
// result as half of group g's pairing job (the jobs start zeroed): set 0 is
// pa (with the key's slot), set 1 pb; an identity sum sets the job's flag.
DEV g1 shfl_g1(const g1 &p, int src) {
  g1 r;
#pragma unroll
  for (int i = 0; i < 12; i++) {
    r.X.w[i] = __shfl_sync(0xffffffffu, p.X.w[i], src);
    r.Y.w[i] = __shfl_sync(0xffffffffu, p.Y.w[i], src);
    r.ZZ.w[i] = __shfl_sync(0xffffffffu, p.ZZ.w[i], src);
    r.ZZZ.w[i] = __shfl_sync(0xffffffffu, p.ZZZ.w[i], src);
  }
  return r;
}
// Set s's half of group g's pairing job, affine: set 0 is pa (with the key's
// slot), set 1 pb; an identity sum sets the job's flag.
DEV void agg_write_job(const g1 &a, uint32_t g, uint32_t s, const int32_t *gslot, PairJob *gjobs) {
  g1a aff;
  const bool finite = g1_to_aff(a, aff);
  if (!finite) aff.x = aff.y = fp_zero();
  PairJob &jb = gjobs[g];
  if (s == 0) {
    jb.pa = aff;
    jb.slot_a = gslot[g];
    jb.slot_b = 0;
    jb.active = 1;
  } else {
    jb.pb = aff;
  }
  if (!finite) atomicOr(&jb.flags, s == 0 ? 1u : 2u);
}
__global__ void __launch_bounds__(128) k_agg_combine(const g1 *part, const int32_t *gslot, PairJob *gjobs) {
  __shared__ g1 win[4];
  const uint32_t g = blockIdx.x, s = blockIdx.y, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const LanePair lp = LanePair::here();
  g1 a = part[(size_t)(AGG_SLAB * g + 4 * s + w) * 16 + (lane >> 1)];
  a = shfl_g1(warp_sum_pairs(lp, a), 0);
  const LaneQuad lq = LaneQuad::here();
  #pragma unroll 1
  for (uint32_t k = 0; k < 8 * w; k++) a = g1_dbl_quad(lq, a);
  if (lane == 0) win[w] = a;
  __syncthreads();
  if (w != 0) return;
  a = warp_sum_pairs(lp, lane < 8 ? win[lane >> 1] : g1_inf());
  if (lane == 0) agg_write_job(a, g, s, gslot, gjobs);
}
// Small groups: one ladder per point instead of the bucket MSM, whose
// 255 bucket weights per (set, window) cost the same whatever the group size
// (per group about 16 n mixed additions plus 8 x 255 x 15 point operations,
// against 2 n x 62 for the ladders: the buckets win from about 280 items).
// k_agg_ladder: one lane pair per (item, set) of a grouped item,
// scaled[2i + s] = a P + b phi(P) from the prepared pts4 / sc (Shamir's trick
// over the 32 bits of a and b; every step adds one of {P, phi(P), P + phi(P)}
// or nothing and keeps the sum by a select, so pairs never diverge).
__global__ void __launch_bounds__(32) k_agg_ladder(const g1a *pts4, const uint2 *sc, const int32_t *group_of,
                                                   uint32_t n, g1 *scaled) {
  const uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 1;
  if (t >= 2 * n) return;  // both lanes of a pair leave together
  const LanePair lp = LanePair::here();
  const uint32_t i = t >> 1, s = t & 1;
  g1 acc = g1_inf();
  const uint2 v = group_of[i] >= 0 ? sc[2 * i + s] : make_uint2(0u, 0u);
  if (v.x) {  // a_i has its top bit set when the point takes part
    const uint32_t a = v.x, b = v.y;
    const g1 P = g1_from_aff(pts4[4 * i + 2 * s]), E = g1_from_aff(pts4[4 * i + 2 * s + 1]);
    const g1 PE = g1_add_pair(lp, P, E);
    acc = (b >> 31) ? PE : P;
    #pragma unroll 1
    for (int k = 30; k >= 0; k--) {
      acc = g1_dbl_pair(lp, acc);
      const uint32_t sel = ((a >> k) & 1) | (((b >> k) & 1) << 1);
      const g1 q = sel == 1 ? P : sel == 2 ? E : PE;
      const g1 sum = g1_add_pair(lp, acc, q);
      if (sel) acc = sum;
    }
  }
  if (lp.role == 0) scaled[t] = acc;
}
// Grid (groups, 2): block (g, s) sums scaled[2 i + s] over group g's items
// (perm[goff[g] .. goff[g+1])) and writes its half of the group's pairing job
// in affine form (the jobs start zeroed).  256 threads = 128 lane pairs: every
// pair sums a strided share of the items, then the pairs' sums are added by
// shuffles within each warp and through shared memory across the 8 warps.
__global__ void __launch_bounds__(256) k_agg_sum(const g1 *scaled, const uint32_t *perm, const uint32_t *goff,
                                                 const int32_t *gslot, PairJob *gjobs) {
  __shared__ g1 part[8];
  const uint32_t g = blockIdx.x, s = blockIdx.y, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const LanePair lp = LanePair::here();
  g1 a = g1_inf();
  #pragma unroll 1
  for (uint32_t k = goff[g] + (threadIdx.x >> 1); k < goff[g + 1]; k += blockDim.x >> 1)
    a = g1_add_pair(lp, a, scaled[2 * perm[k] + s]);
  a = warp_sum_pairs(lp, a);
  if (lane == 0) part[warp] = a;
  __syncthreads();
  if (warp == 0) {
    a = warp_sum_pairs(lp, lane < 16 ? part[lane >> 1] : g1_inf());
    if (lane == 0) agg_write_job(a, g, s, gslot, gjobs);
  }
}

// Per-item pairing jobs after the group checks: an item of a group whose check
// passed is valid for the pairing (ok = 1, job skipped); any other item that
// decoded gets its own check.
__global__ void __launch_bounds__(128) k_pv_pairjobs_agg(const PvItem *items0, uint32_t n, const g1a *pts,
                                                         const int32_t *dec_status, const int32_t *group_of,
                                                         const uint8_t *group_ok, PairJob *pj, uint8_t *ok) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PvItem it = items0[i];
  PairJob job;
  job.slot_a = it.pk_slot < 0 ? 0 : it.pk_slot;
  job.slot_b = 0;
  job.pa = pts[3 * i];
  job.pb = pts[3 * i + 1];
  job.flags = 0;
  bool valid = it.status == ST_OK && it.pk_status != DEC_BAD;
  #pragma unroll 1
  for (int k = 0; k < 3; k++) valid = valid && dec_status[3 * i + k] != DEC_BAD;
  job.active = valid ? 1 : 0;
  if (valid && group_of[i] >= 0 && group_ok[group_of[i]]) {
    job.active = 2;
    ok[i] = 1;
  }
  if (dec_status[3 * i] == DEC_INF || it.pk_status == DEC_INF) job.flags |= 1;
  if (dec_status[3 * i + 1] == DEC_INF) job.flags |= 2;
  pj[i] = job;
}

// Verify: items of groups whose check passed are settled (ok = 1, job
// skipped); the others keep their own job.
__global__ void __launch_bounds__(128) k_vf_pairjobs_agg(uint32_t n, const int32_t *group_of,
                                                         const uint8_t *group_ok, PairJob *pj, uint8_t *ok) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (pj[i].active == 1 && group_of[i] >= 0 && group_ok[group_of[i]]) {
    pj[i].active = 2;
    ok[i] = 1;
  }
}

// The part of the challenge hash that comes before T1 and T2 (R, the disclosed
// indexes and message scalars, Abar || Bbar || D: about 34 SHA-256 blocks at
// 50 disclosed messages) needs no point arithmetic, so it is absorbed early,
// beside the MSMs, and the expander's state is kept per item for k_pv_finish.
// It reads the input items as packed (items0): an item the host rejected is
// skipped, and k_pv_finish skips it as well (a status never returns to ST_OK).
template <int S>
__global__ void __launch_bounds__(64) k_pv_chal_prefix(const PvItem *items0, uint32_t n, const uint8_t *blob,
                                                       const fr *msc, hash_ctx<S> *chal) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PvItem it = items0[i];
  if (it.status != ST_OK) return;
  const uint32_t *idx = reinterpret_cast<const uint32_t *>(blob + it.idx_off);
  hash_ctx<S> c;
  msg_begin(c);
  msg_u64be(c, it.R, 8);
  #pragma unroll 1
  for (uint32_t k = 0; k < it.R; k++) {
    msg_u64be(c, idx[k], 8);
    msg_fr_be(c, msc[it.msg_base + k]);
  }
  msg_bytes(c, blob + it.proof_off, 144);
  chal[i] = c;
}

// T1, T2 -> compressed; finish the challenge from the state k_pv_chal_prefix
// kept (a mismatch marks the item invalid).
template <int S>
__global__ void __launch_bounds__(64) k_pv_finish(PvItem *items, uint32_t n, const uint8_t *blob, const fr *msc,
                                                  const fr *domain, const int32_t *dec_status,
                                                  const int32_t *outside_g1, const g1 *t2fix, const g1 *v,
                                                  const hash_ctx<S> *chal) {
  // every lane of the warp reaches the shared affine conversion below
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool act = i < n;
  PvItem it;
  if (act) {
    it = items[i];
    act = it.status == ST_OK;
    if (act && (dec_status[3 * i] == DEC_BAD || dec_status[3 * i + 1] == DEC_BAD ||
                dec_status[3 * i + 2] == DEC_BAD || outside_g1[3 * i] || outside_g1[3 * i + 1] ||
                outside_g1[3 * i + 2])) {
      items[i].status = ST_INVALID;
      act = false;
    }
  }
  g1 T1 = g1_inf(), T2 = g1_inf();
  if (act) {
    T1 = g1_add(g1_add(v[3 * i], v[3 * i + 1]), v[3 * i + 2]);
    T2 = g1_add(t2fix[i], v[3 * n + i]);
  }
  const g1 T[2] = {T1, T2};
  g1a aff[2];
  bool fin[2];
  warp_to_aff<2>(T, aff, fin);
  if (!act) return;
  uint8_t t1c[48], t2c[48];
  g1_compress_aff_or_inf(aff[0], fin[0], t1c);
  g1_compress_aff_or_inf(aff[1], fin[1], t2c);
  const uint8_t *pr = blob + it.proof_off;
  const uint32_t *idx = reinterpret_cast<const uint32_t *>(blob + it.idx_off);
  hash_ctx<S> c = chal[i];
  msg_bytes(c, t1c, 48);
  msg_bytes(c, t2c, 48);
  msg_fr_be(c, domain[i]);
  msg_u64be(c, it.ph_len, 8);
  msg_bytes(c, blob + it.ph_off, it.ph_len);
  fr ch = h2s_api<S>(c);
  if (i == 0) debug_record(t1c, t2c, domain[i], ch, it.R, idx, it.R ? &msc[it.msg_base] : nullptr);
  fr cp;
  fr_raw_from_be32(pr + 240 + 32 * it.U, cp);
  if (!fr_eq(ch, cp)) items[i].status = ST_INVALID;
}

// ============================================================================ Sign
struct SignItem {
  uint32_t sk_off, pk_off, hdr_off, hdr_len, msg_base, L;
  int32_t pk_status;
  int32_t status;
};

template <int S>
__global__ void __launch_bounds__(64) k_sign_prep(SignItem *items, uint32_t n, const uint8_t *blob, const fr *msc,
                                                  const fr *domain, fr *rows, uint32_t stride, uint32_t *nterms,
                                                  fr *e_out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  SignItem it = items[i];
  fr sk;
  bool ok = it.status == ST_OK && it.pk_status != DEC_BAD && fr_raw_from_be32(blob + it.sk_off, sk);
  if (!ok) {
    items[i].status = ST_ERROR;
    nterms[i] = 0;
    return;
  }
  // e = hash_to_scalar(sk || m_1..m_L || domain, api_id || "H2S_")  (signature.rs:564-577)
  hash_ctx<S> c;
  msg_begin(c);
  msg_fr_be(c, sk);
  #pragma unroll 1
  for (uint32_t k = 0; k < it.L; k++) msg_fr_be(c, msc[it.msg_base + k]);
  msg_fr_be(c, domain[i]);
  fr e = h2s_api<S>(c);
  e_out[i] = e;
  fr ske = fr_add(sk, e);
  if (fr_is_zero(ske)) {
    items[i].status = ST_ERROR;
    nterms[i] = 0;
    return;
  }
  // A = B / (sk + e) = sum_g (s_g / (sk + e)) G_g: scale the B row (execution.rs:3400-3447)
  fr inv = frr_inv(ske);
  fr *row = rows + (size_t)i * stride;
  nterms[i] = it.L + 2;
  row[0] = inv;
  row[1] = frr_mul(domain[i], inv);
  #pragma unroll 1
  for (uint32_t k = 0; k < it.L; k++) row[2 + k] = frr_mul(msc[it.msg_base + k], inv);
}

__global__ void __launch_bounds__(64) k_sign_finish(SignItem *items, uint32_t n, const g1 *A, const fr *e,
                                                    uint8_t *sig) {
  // every lane of the warp reaches the shared affine conversion below
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool act = i < n && items[i].status == ST_OK;
  if (act && g1_is_inf(A[i])) {  // "A == Identity_G1" (signature.rs:653-657)
    items[i].status = ST_ERROR;
    act = false;
  }
  const g1 p = act ? A[i] : g1_inf();
  g1a a[1];
  bool fin[1];
  warp_to_aff<1>(&p, a, fin);
  if (!act) return;
  g1_compress_aff_or_inf(a[0], fin[0], sig + 80 * (size_t)i);
  fr_raw_to_be32(e[i], sig + 80 * (size_t)i + 48);
}

// ============================================================================ Verify
struct VerifyItem {
  uint32_t sig_off, hdr_off, hdr_len, msg_base, L;
  int32_t pk_slot, pk_status;
  int32_t status;
};

// B-MSM row of each signature (needs no decoded point, so the fixed-base MSM
// runs while the signature's A decodes).
__global__ void __launch_bounds__(128) k_verify_rows(VerifyItem *items, uint32_t n, const uint8_t *blob,
                                                     const fr *msc, const fr *domain, fr *rows, uint32_t stride,
                                                     uint32_t *nterms) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  VerifyItem it = items[i];
  fr e;
  bool ok = it.status == ST_OK && it.pk_status != DEC_BAD && fr_raw_from_be32(blob + it.sig_off + 48, e);
  if (!ok) {
    if (items[i].status == ST_OK) items[i].status = ST_INVALID;
    nterms[i] = 0;
    return;
  }
  fr *row = rows + (size_t)i * stride;
  nterms[i] = it.L + 2;
  row[0] = frr_one();
  row[1] = domain[i];
  #pragma unroll 1
  for (uint32_t k = 0; k < it.L; k++) row[2 + k] = msc[it.msg_base + k];
}

// The variable-base job -e * A of each signature, from the untouched input
// items and the decoded A (a signature that does not decode gets a job at
// infinity; k_verify_finish rejects it).
__global__ void __launch_bounds__(128) k_verify_jobs(const VerifyItem *items0, uint32_t n, const uint8_t *blob,
                                                     const int32_t *dec_status, VarJob *jobs, fr *jscal) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const VerifyItem it = items0[i];
  fr e;
  const bool ok = it.status == ST_OK && dec_status[i] != DEC_BAD && fr_raw_from_be32(blob + it.sig_off + 48, e);
  jobs[i] = {i, (!ok || dec_status[i] == DEC_INF) ? 1u : 0u};
  jscal[i] = ok ? frr_neg(e) : fr_zero();
}

// Pairing job of each signature: e(A, PK) * e(B - e A, -P2) == 1; every lane
// of the warp reaches the shared affine conversion.
__global__ void __launch_bounds__(64) k_verify_finish(VerifyItem *items, uint32_t n, const g1 *B, const g1 *v,
                                                      const g1a *A, const int32_t *dec_status,
                                                      const int32_t *outside_g1, PairJob *pj) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool act = i < n;
  VerifyItem it;
  if (act) {
    it = items[i];
    act = it.status == ST_OK;
    if (act && (dec_status[i] == DEC_BAD || outside_g1[i])) {
      items[i].status = ST_INVALID;
      act = false;
    }
  }
  g1 C = g1_inf();
  if (act) C = g1_add(B[i], v[i]);  // B - e A
  g1a ca[1];
  bool fin[1];
  warp_to_aff<1>(&C, ca, fin);
  if (i >= n) return;
  PairJob job;
  job.active = 0;
  job.flags = 0;
  job.slot_a = it.pk_slot < 0 ? 0 : it.pk_slot;
  job.slot_b = 0;
  job.pa = A[i];
  job.pb = A[i];
  if (act) {
    if (fin[0]) job.pb = ca[0];
    else job.flags |= 2;
    if (dec_status[i] == DEC_INF || it.pk_status == DEC_INF) job.flags |= 1;
    job.active = 1;
  }
  pj[i] = job;
}

// ============================================================================ ProofGen
struct PgItem {
  uint32_t sig_off, hdr_off, hdr_len, ph_off, ph_len, idx_off, R, U, msg_base, L, seed_off, out_off;
  int32_t pk_status;
  int32_t status;
};

// seeded_random_scalars(5+U, seed, api_id || "MOCK_RANDOM_SCALARS_DST_") (util.rs:329-358);
// with expand_message_xmd more than 170 scalars are drawn in chunks keyed by
// seed || I2OSP(chunk, 2); with expand_message_xof one call covers up to 1365
// (65535 bytes) and larger counts are chunked the same way.
template <int S>
__global__ void __launch_bounds__(64) k_pg_random(const PgItem *items, uint32_t n, const uint8_t *blob,
                                                  fr *rs, uint32_t rs_stride) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  PgItem it = items[i];
  if (it.status != ST_OK) return;
  if constexpr (S == SUITE_SHAKE256) {
    const uint32_t count = 5 + it.U, CH = 1365;
    fr *out = rs + (size_t)i * rs_stride;
#pragma unroll 1
    for (uint32_t c0 = 0; c0 < count; c0 += CH) {
      const uint32_t m = min(CH, count - c0);
      shake_ctx c;
      xof_begin(c);
      shake_bytes(c, blob + it.seed_off, 32);
      if (count > CH) {
        shake_byte(c, (uint8_t)((c0 / CH) >> 8));
        shake_byte(c, (uint8_t)(c0 / CH));
      }
      xof_start_output(c, SuiteDst<S>::dst_mock(), SuiteDst<S>::dst_mock_len, 48 * m);
#pragma unroll 1
      for (uint32_t k = 0; k < m; k++) {
        uint8_t okm[48];
        shake_squeeze(c, okm, 48);
        out[c0 + k] = fr_raw_from_okm(okm);
      }
    }
    return;
  }
  const uint8_t *dst = DST_MOCK;
  uint32_t count = 5 + it.U;
  const uint32_t CH = 170;
  fr *out = rs + (size_t)i * rs_stride;
  #pragma unroll 1
  for (uint32_t c0 = 0; c0 < count; c0 += CH) {
    uint32_t m = min(CH, count - c0);
    sha_ctx c;
    xmd_begin(c);
    sha_bytes(c, blob + it.seed_off, 32);
    if (count > CH) {
      uint32_t chunk = c0 / CH;
      sha_byte(c, (uint8_t)(chunk >> 8));
      sha_byte(c, (uint8_t)chunk);
    }
    // expand 48*m bytes, one 32-byte block at a time, reducing every 48 bytes
    // (xmd_finish into a per-thread buffer of at most 8160 bytes would not fit in
    // registers; stream the b_i blocks instead)
    uint32_t nbytes = 48 * m;
    sha_byte(c, (uint8_t)(nbytes >> 8));
    sha_byte(c, (uint8_t)nbytes);
    sha_byte(c, 0);
    sha_bytes(c, dst, DST_MOCK_LEN);
    sha_byte(c, DST_MOCK_LEN);
    uint8_t b0[32];
    sha_final(c, b0);
    // b_i = SHA-256((b_0 xor b_(i-1)) || I2OSP(i, 1) || DST || I2OSP(68, 1)): 102 bytes
    // in two blocks.  Block 1 is 8 words of b_0 xor b_(i-1), then i and DST[0..30];
    // block 2 (DST[31..67], the DST length, the padding, the bit length 816) is the
    // same for every i.
    uint32_t x0[8], bi[8] = {0, 0, 0, 0, 0, 0, 0, 0}, tail1[7], blk2[16];
    for (int k = 0; k < 8; k++)
      x0[k] = (uint32_t)b0[4 * k] << 24 | (uint32_t)b0[4 * k + 1] << 16 | (uint32_t)b0[4 * k + 2] << 8 | b0[4 * k + 3];
    const uint32_t dst3 = (uint32_t)dst[0] << 16 | (uint32_t)dst[1] << 8 | dst[2];
    for (int k = 0; k < 7; k++)
      tail1[k] = (uint32_t)dst[3 + 4 * k] << 24 | (uint32_t)dst[4 + 4 * k] << 16 | (uint32_t)dst[5 + 4 * k] << 8 |
                 dst[6 + 4 * k];
    {
      uint8_t t[64];
      for (int k = 0; k < 37; k++) t[k] = dst[31 + k];
      t[37] = DST_MOCK_LEN;
      t[38] = 0x80;
      for (int k = 39; k < 64; k++) t[k] = 0;
      t[62] = (uint8_t)((102 * 8) >> 8);
      t[63] = (uint8_t)(102 * 8);
      for (int k = 0; k < 16; k++)
        blk2[k] = (uint32_t)t[4 * k] << 24 | (uint32_t)t[4 * k + 1] << 16 | (uint32_t)t[4 * k + 2] << 8 | t[4 * k + 3];
    }
    uint8_t okm[48];
    uint32_t fill = 0, produced = 0;
    uint32_t ell = (nbytes + 31) / 32;
    #pragma unroll 1
    for (uint32_t b = 1; b <= ell; b++) {
      uint32_t h[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                       0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
      uint32_t w[16];
      for (int k = 0; k < 8; k++) w[k] = x0[k] ^ bi[k];  // bi = 0 before b_1
      w[8] = b << 24 | dst3;
      for (int k = 0; k < 7; k++) w[9 + k] = tail1[k];
      sha256_compress(h, w);
      for (int k = 0; k < 16; k++) w[k] = blk2[k];
      sha256_compress(h, w);
      for (int k = 0; k < 8; k++) bi[k] = h[k];
      for (int j = 0; j < 32; j++) {
        okm[fill++] = (uint8_t)(bi[j >> 2] >> (24 - 8 * (j & 3)));
        if (fill == 48) {
          out[c0 + produced] = fr_raw_from_okm(okm);
          produced++;
          fill = 0;
        }
      }
    }
  }
}

// Row i: B = P1 + Q1 domain + sum H_i m_i.  Needs neither the decoded signature
// point (k_pg_vars rejects a signature whose A does not decode) nor the blinding
// scalars, so the B-MSM starts as soon as the messages are hashed.
__global__ void __launch_bounds__(128) k_pg_rows_b(PgItem *items, uint32_t n, const uint8_t *blob, const fr *msc,
                                                   const fr *domain, fr *rows, uint32_t stride, uint32_t *nterms) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  PgItem it = items[i];
  fr e;
  bool ok = it.status == ST_OK && it.pk_status != DEC_BAD && fr_raw_from_be32(blob + it.sig_off + 48, e);
  if (!ok) {
    items[i].status = ST_ERROR;
    nterms[i] = 0;
    return;
  }
  fr *rb = rows + (size_t)i * stride;
  nterms[i] = it.L + 2;
  rb[0] = frr_one();
  rb[1] = domain[i];
  #pragma unroll 1
  for (uint32_t m = 0; m < it.L; m++) rb[2 + m] = msc[it.msg_base + m];
}

// Row n + i: the fixed part of T2, sum_{j not disclosed} H_j m~_j, from the
// untouched input items and the blinding scalars.
__global__ void __launch_bounds__(128) k_pg_rows_t2(const PgItem *items0, uint32_t n, const uint8_t *blob,
                                                    const fr *rs, uint32_t rs_stride, fr *rows, uint32_t stride,
                                                    uint32_t *nterms) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PgItem it = items0[i];
  if (it.status != ST_OK) {
    nterms[n + i] = 0;
    return;
  }
  fr *rt = rows + (size_t)(n + i) * stride;
  nterms[n + i] = it.L + 2;
  rt[0] = fr_zero();
  rt[1] = fr_zero();
  const uint32_t *idx = reinterpret_cast<const uint32_t *>(blob + it.idx_off);
  const fr *r = rs + (size_t)i * rs_stride;
  uint32_t k = 0, u = 0;
  #pragma unroll 1
  for (uint32_t m = 0; m < it.L; m++) {
    if (k < it.R && idx[k] == m) {
      rt[2 + m] = fr_zero();
      k++;
    } else {
      rt[2 + m] = r[5 + u];
      u++;
    }
  }
}

// Variable-base jobs on B (affine) and A: D = r2 B, Abar = r1r2 A,
// Bbar = r1r2 B - e r1r2 A, T1 = r1~ r2 B + e~ r1r2 A, T2 += r3~ r2 B.
__global__ void __launch_bounds__(64) k_pg_vars(PgItem *items, uint32_t n, const uint8_t *blob, const g1 *Bx,
                                                const g1a *A, const int32_t *dec_status, const int32_t *outside_g1,
                                                const fr *rs, uint32_t rs_stride, g1a *pts, VarJob *jobs, fr *jscal) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  PgItem it = items[i];
  for (int k = 0; k < 7; k++) jobs[7 * i + k] = {2 * i, 1};
  if (it.status != ST_OK) return;
  if (dec_status[i] == DEC_BAD || outside_g1[i]) {  // signature A does not decode to a point of G1
    items[i].status = ST_ERROR;
    return;
  }
  g1a b;
  bool binf = !g1_to_aff(Bx[i], b);
  pts[2 * i] = A[i];
  pts[2 * i + 1] = binf ? A[i] : b;
  uint32_t fa = dec_status[i] == DEC_INF ? 1 : 0, fb = binf ? 1 : 0;
  fr e;
  fr_raw_from_be32(blob + it.sig_off + 48, e);
  const fr *r = rs + (size_t)i * rs_stride;
  fr r1 = r[0], r2 = r[1], et = r[2], r1t = r[3], r3t = r[4];
  fr r1r2 = frr_mul(r1, r2);
  jobs[7 * i + 0] = {2 * i + 1, fb}; jscal[7 * i + 0] = r2;
  jobs[7 * i + 1] = {2 * i, fa};     jscal[7 * i + 1] = r1r2;
  jobs[7 * i + 2] = {2 * i + 1, fb}; jscal[7 * i + 2] = r1r2;
  jobs[7 * i + 3] = {2 * i, fa};     jscal[7 * i + 3] = frr_neg(frr_mul(e, r1r2));
  jobs[7 * i + 4] = {2 * i + 1, fb}; jscal[7 * i + 4] = frr_mul(r1t, r2);
  jobs[7 * i + 5] = {2 * i, fa};     jscal[7 * i + 5] = frr_mul(et, r1r2);
  jobs[7 * i + 6] = {2 * i + 1, fb}; jscal[7 * i + 6] = frr_mul(r3t, r2);
}

template <int S>
__global__ void __launch_bounds__(64) k_pg_finish(PgItem *items, uint32_t n, const uint8_t *blob, const fr *msc,
                                                  const fr *domain, const fr *rs, uint32_t rs_stride,
                                                  const g1 *t2fix, const g1 *v, uint8_t *out, const hash_ctx<S> *chal,
                                                  const fr *r3inv) {
  // every lane of the warp reaches the shared affine conversion below
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = i < n && items[i].status == ST_OK;
  g1 P[5] = {g1_inf(), g1_inf(), g1_inf(), g1_inf(), g1_inf()};  // Abar, Bbar, D, T1, T2
  if (act) {
    const g1 *vi = v + 7 * (size_t)i;
    P[0] = vi[1];
    P[1] = g1_add(vi[2], vi[3]);
    P[2] = vi[0];
    P[3] = g1_add(vi[4], vi[5]);
    P[4] = g1_add(t2fix[i], vi[6]);
  }
  g1a aff[5];
  bool fin[5];
  warp_to_aff<5>(P, aff, fin);
  if (!act) return;
  const PgItem it = items[i];
  uint8_t *o = out + it.out_off;
  g1_compress_aff_or_inf(aff[0], fin[0], o);
  g1_compress_aff_or_inf(aff[1], fin[1], o + 48);
  g1_compress_aff_or_inf(aff[2], fin[2], o + 96);
  uint8_t t1c[48], t2c[48];
  g1_compress_aff_or_inf(aff[3], fin[3], t1c);
  g1_compress_aff_or_inf(aff[4], fin[4], t2c);
  const uint32_t *idx = reinterpret_cast<const uint32_t *>(blob + it.idx_off);
  hash_ctx<S> c = chal[i];  // R and the disclosed messages, absorbed by k_pg_early
  msg_bytes(c, o, 144);
  msg_bytes(c, t1c, 48);
  msg_bytes(c, t2c, 48);
  msg_fr_be(c, domain[i]);
  msg_u64be(c, it.ph_len, 8);
  msg_bytes(c, blob + it.ph_off, it.ph_len);
  fr ch = h2s_api<S>(c);
  if (i == 0) debug_record(t1c, t2c, domain[i], ch, it.R, idx, it.R ? &msc[it.msg_base + idx[0]] : nullptr);
  const fr *r = rs + (size_t)i * rs_stride;
  fr r1 = r[0], r2 = r[1], et = r[2], r1t = r[3], r3t = r[4];
  if (fr_is_zero(r2)) {  // "Invert scalar failed" (proof.rs:2340-2341)
    items[i].status = ST_ERROR;
    return;
  }
  fr e;
  fr_raw_from_be32(blob + it.sig_off + 48, e);
  const fr r3 = r3inv[i];
  fr_raw_to_be32(fr_add(et, frr_mul(e, ch)), o + 144);
  fr_raw_to_be32(fr_sub(r1t, frr_mul(r1, ch)), o + 176);
  fr_raw_to_be32(fr_sub(r3t, frr_mul(r3, ch)), o + 208);
  uint32_t k = 0, u = 0;
  #pragma unroll 1
  for (uint32_t m = 0; m < it.L; m++) {
    if (k < it.R && idx[k] == m) {
      k++;
      continue;
    }
    fr_raw_to_be32(fr_add(r[5 + u], frr_mul(msc[it.msg_base + m], ch)), o + 240 + 32 * u);
    u++;
  }
  fr_raw_to_be32(ch, o + 240 + 32 * it.U);
}

// Work of k_pg_finish that needs neither the MSMs nor the proof's points, done
// beside them: the challenge hash's leading part (R, the disclosed indexes and
// message scalars: about 31 SHA-256 blocks at 50 disclosed messages), kept as
// the expander's state per item, and r3 = r2^-1 (a Fermat inversion in Fr).
// It reads the input items as packed; an item the host rejected is skipped
// (k_pg_finish skips it as well).
template <int S>
__global__ void __launch_bounds__(64) k_pg_early(const PgItem *items0, uint32_t n, const uint8_t *blob,
                                                 const fr *msc, const fr *rs, uint32_t rs_stride, hash_ctx<S> *chal,
                                                 fr *r3inv) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PgItem it = items0[i];
  if (it.status != ST_OK) return;
  const uint32_t *idx = reinterpret_cast<const uint32_t *>(blob + it.idx_off);
  hash_ctx<S> c;
  msg_begin(c);
  msg_u64be(c, it.R, 8);
  #pragma unroll 1
  for (uint32_t k = 0; k < it.R; k++) {
    msg_u64be(c, idx[k], 8);
    msg_fr_be(c, msc[it.msg_base + idx[k]]);
  }
  chal[i] = c;
  r3inv[i] = frr_inv(rs[(size_t)i * rs_stride + 1]);  // r2 == 0 gives 0; k_pg_finish reports it
}

// ============================================================================ host side
namespace {

bool abi_ok(uint32_t v) { return v == CUBBS_BBS_GPU_ABI_VERSION; }
const size_t MAX_MESSAGES = 16384;  // generators kept resident: L + 2 <= 16386

// Growable host byte blob (packed inputs for one batch).
// Packed bytes of a batch, written straight into pinned host memory (the
// workspace's pack buffer) so that one DMA moves them to the device.
struct PinnedBytes {
  uint8_t *base = nullptr;
  size_t used = 0, cap = 0;
  void bind(HostStaging &pack, size_t bytes) {
    base = pack.alloc(bytes ? bytes : 16);
    cap = bytes;
    used = 0;
  }
  uint8_t *grab(size_t n) {
    if (used + n > cap) throw CudaError(cudaErrorMemoryAllocation, "packed batch larger than planned");
    uint8_t *p = base + used;
    used += n;
    return p;
  }
  size_t size() const { return used; }
  const uint8_t *data() const { return base; }
};

struct Blob {
  PinnedBytes b;
  uint32_t put(const uint8_t *p, size_t n) {
    uint32_t off = (uint32_t)b.size();
    if (n) std::memcpy(b.grab(n), p, n);
    return off;
  }
  uint32_t put_u32s(const std::vector<uint32_t> &v) {
    if (b.size() & 3) std::memset(b.grab(4 - (b.size() & 3)), 0, 4 - (b.size() & 3));
    uint32_t off = (uint32_t)b.size();
    if (!v.empty()) std::memcpy(b.grab(4 * v.size()), v.data(), 4 * v.size());
    return off;
  }
  // bytes that put() / put_u32s() of n bytes may take (alignment included)
  static size_t room(size_t n) { return n + 4; }
};

// Flat message list: [offsets u32 * n][lengths u32 * n][bytes]; the bytes are pinned.
struct MsgList {
  std::vector<uint32_t> offs, lens;
  PinnedBytes bytes;
  uint32_t add(const uint8_t *p, size_t n) {
    offs.push_back((uint32_t)bytes.size());
    lens.push_back((uint32_t)n);
    if (n) std::memcpy(bytes.grab(n), p, n);
    return (uint32_t)(offs.size() - 1);
  }
  size_t count() const { return offs.size(); }
};

// Host workers that pack large batches: created once, they wait for work
// between calls.  One parallel_for runs at a time; a call that finds the pool
// busy (another host thread is packing) runs its ranges on its own thread.
class PackPool {
 public:
  static PackPool &get() {
    static PackPool pool;
    return pool;
  }
  // Runs fn(r) for r = 0..ranges-1 on the workers and the calling thread.
  void parallel_for(size_t ranges, const std::function<void(size_t)> &fn) {
    std::unique_lock<std::mutex> owner(run_mu_, std::try_to_lock);
    if (!owner.owns_lock() || workers_.empty()) {
      for (size_t r = 0; r < ranges; r++) fn(r);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &fn;
      ranges_ = ranges;
      next_ = 0;
      done_ = 0;
      gen_++;
    }
    cv_.notify_all();
    drain();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return done_ == ranges_; });
    fn_ = nullptr;
  }

 private:
  PackPool() {
    const unsigned hw = std::thread::hardware_concurrency();
    const unsigned n = hw > 1 ? std::min(7u, hw - 1) : 0;
    for (unsigned k = 0; k < n; k++) workers_.emplace_back([this] { worker(); });
  }
  ~PackPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto &t : workers_) t.join();
  }
  // Takes ranges until none are left.
  void drain() {
    for (;;) {
      size_t r;
      const std::function<void(size_t)> *fn;
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (!fn_ || next_ >= ranges_) return;
        r = next_++;
        fn = fn_;
      }
      (*fn)(r);
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (++done_ == ranges_) done_cv_.notify_all();
      }
    }
  }
  void worker() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
      }
      drain();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(size_t)> *fn_ = nullptr;
  size_t ranges_ = 0, next_ = 0, done_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// Sorted, de-duplicated disclosed indexes (proof.rs:961-963); callers
// usually pass them sorted already, which needs no sort.
void sort_dedup(const size_t *p, size_t n, std::vector<size_t> &out) {
  out.assign(p, p + n);
  bool strictly_increasing = true;
  for (size_t k = 1; k < n && strictly_increasing; k++) strictly_increasing = p[k - 1] < p[k];
  if (strictly_increasing) return;
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
}

enum Op { OP_SIGN = 0, OP_VERIFY = 1, OP_PGEN = 2, OP_PVERIFY = 3 };

// One packed batch of a four-operation call.  plan_*() packs on the host,
// upload() moves everything to the device once, run() replays the whole device
// pipeline (this is the timed step of the benchmark), download() maps results.
struct OpBatch {
  explicit OpBatch(Runtime &rt) : pack(&rt.pack) {}
  HostStaging *pack;  // pinned buffer the blob and the message bytes are packed into
  // Binds the blob and the message bytes to the pack buffer (called by the
  // planners once they know the sizes, before packing).
  void bind(size_t blob_bytes, size_t msg_bytes, size_t msg_count) {
    pack->reserve(blob_bytes + msg_bytes + 64);
    blob.b.bind(*pack, blob_bytes);
    ml.bytes.bind(*pack, msg_bytes);
    ml.offs.reserve(msg_count);
    ml.lens.reserve(msg_count);
  }
  Op op;
  size_t n = 0, maxL = 0, maxU = 0, stride = 0, rs_stride = 0, out_total = 0;
  Blob blob;
  MsgList ml;
  std::vector<uint8_t> pts48;       // points to decode (48 B each), npts per item
  size_t npts_per_item = 0;
  std::vector<DomainJob> dj;
  std::vector<uint8_t> items;       // host copy of the per-item device structs
  size_t item_size = 0;
  std::vector<const uint8_t *> pks;
  std::vector<int32_t> code;        // host-side per-item result codes
  // device buffers
  uint8_t *dblob = nullptr, *dmsg = nullptr, *dpts48 = nullptr, *ditems0 = nullptr, *ditems = nullptr;
  DomainJob *ddj = nullptr;
  fr *msc = nullptr, *domain = nullptr, *rows = nullptr, *jscal = nullptr, *rs = nullptr, *e = nullptr;
  uint32_t *nterms = nullptr;
  VarJob *jobs = nullptr;
  g1a *pts = nullptr, *vpts = nullptr;
  int32_t *dec = nullptr, *sub = nullptr;  // decode status; 1 = decoded outside G1 (ProofVerify)
  // ProofVerify pairing groups (items under one public key, checked together)
  std::vector<int32_t> h_group_of, h_gslot;
  std::vector<uint32_t> h_perm, h_goff;
  int32_t *group_of = nullptr, *gslot = nullptr;
  uint32_t *perm = nullptr, *goff = nullptr;
  PairJob *gjobs = nullptr;
  uint8_t *gok = nullptr;
  // bucket MSM of the group sums (k_agg_*)
  g1a *agg_pts = nullptr;
  uint2 *agg_sc = nullptr;
  uint32_t *agg_ent = nullptr, *agg_boff = nullptr;
  g1 *agg_part = nullptr;
  g1 *scaled = nullptr;  // per-point ladders of small groups
  uint8_t *chal = nullptr;  // ProofVerify, ProofGen: challenge-hash state per item (hash_ctx of the suite)
  fr *r3inv = nullptr;      // ProofGen: r2^-1 per item
  g1 *fixed = nullptr, *v = nullptr;
  PairJob *pj = nullptr;
  uint8_t *ok = nullptr, *out = nullptr;
  size_t launches_per_run = 0;
};

thread_local size_t g_h2d_bytes = 0, g_d2h_bytes = 0;  // bytes moved by this thread's last four-operation call

template <typename T> T *upload_to(Runtime &rt, T *d, const T *h, size_t n) {
  if (n) {
    g_h2d_bytes += n * sizeof(T);
    uint8_t *st = rt.staging.alloc(n * sizeof(T));
    std::memcpy(st, h, n * sizeof(T));
    CUBBS_CHECK(cudaMemcpyAsync(d, st, n * sizeof(T), cudaMemcpyHostToDevice, rt.stream));
  }
  return d;
}
template <typename T> T *upload(Runtime &rt, const T *h, size_t n) {
  return upload_to(rt, rt.arena.alloc<T>(n ? n : 1), h, n);
}

size_t vars_per_item(Op op) { return op == OP_PVERIFY ? 4 : op == OP_VERIFY ? 1 : op == OP_PGEN ? 7 : 0; }
size_t fixed_rows_per_item(Op op) { return op == OP_PGEN ? 2 : 1; }

// Pairing groups of a ProofVerify batch: the items that are well formed so far,
// by public-key slot; a batch of at least 128 items checks every key with at
// least 16 items as one group (the reference aggregates batches of 128 or more:
// crates/cubbs-bbs/src/execution.rs:3797-3801).  Other items are checked alone.
const size_t AGG_MIN_BATCH = 128, AGG_MIN_GROUP = 16;
// Verify batches group the same way (the reference's GPU engine aggregates
// Verify pairings of 128 or more items too: crates/cubbs-bbs/src/execution.rs:
// 3797-3801, gpu_engine.rs:1756-1781).
template <typename ItemT> void plan_groups_of(Runtime &rt, OpBatch &b) {
  const size_t n = b.n;
  b.h_group_of.assign(n, -1);
  b.h_perm.clear();
  b.h_goff.assign(1, 0);
  b.h_gslot.clear();
  if (n >= AGG_MIN_BATCH) {
    std::unordered_map<int32_t, std::vector<uint32_t>> by_slot;
    std::vector<int32_t> order;
    for (size_t i = 0; i < n; i++) {
      const ItemT &p = reinterpret_cast<const ItemT *>(b.items.data())[i];
      if (p.status != ST_OK || p.pk_status != DEC_OK) continue;
      auto &v = by_slot[p.pk_slot];
      if (v.empty()) order.push_back(p.pk_slot);
      v.push_back((uint32_t)i);
    }
    for (int32_t slot : order) {
      const auto &v = by_slot[slot];
      if (v.size() < AGG_MIN_GROUP) continue;
      for (uint32_t i : v) {
        b.h_group_of[i] = (int32_t)b.h_gslot.size();
        b.h_perm.push_back(i);
      }
      b.h_gslot.push_back(slot);
      b.h_goff.push_back((uint32_t)b.h_perm.size());
    }
  }
  const size_t G = b.h_gslot.size();
  b.group_of = upload(rt, b.h_group_of.data(), n);
  if (G) {
    b.perm = upload(rt, b.h_perm.data(), b.h_perm.size());
    b.goff = upload(rt, b.h_goff.data(), G + 1);
    b.gslot = upload(rt, b.h_gslot.data(), G);
    b.gjobs = rt.arena.alloc<PairJob>(G);
    b.gok = rt.arena.alloc<uint8_t>(G);
    const size_t M = b.h_perm.size();
    b.agg_pts = rt.arena.alloc<g1a>(4 * n);
    b.agg_sc = rt.arena.alloc<uint2>(2 * n);
    b.agg_ent = rt.arena.alloc<uint32_t>(2 * AGG_SLAB * M);
    b.agg_boff = rt.arena.alloc<uint32_t>(AGG_SLAB * G * 257);
    b.agg_part = rt.arena.alloc<g1>(AGG_SLAB * G * 16);
    b.scaled = rt.arena.alloc<g1>(2 * n);
  }
}

void upload(Runtime &rt, OpBatch &b) {
  size_t n = b.n, nm = b.ml.count();
  b.stride = b.maxL + 2;
  b.rs_stride = b.maxU + 5;
  size_t fr_rows = fixed_rows_per_item(b.op) * n * b.stride, nv = vars_per_item(b.op) * n;
  size_t need = 65536 + 2 * b.blob.b.size() + b.ml.bytes.size() + 8 * nm + nm * sizeof(fr) + b.pts48.size() +
                n * (b.item_size * 2 + sizeof(DomainJob) + 2 * sizeof(fr) + sizeof(PairJob) + 256) +
                fr_rows * sizeof(fr) + 2 * n * sizeof(uint32_t) + nv * (sizeof(VarJob) + sizeof(fr) + sizeof(g1)) +
                (b.pts48.size() / 48) * (sizeof(g1a) + 8) + 2 * n * sizeof(g1) + 2 * n * sizeof(g1a) +
                n * b.rs_stride * sizeof(fr) + b.out_total + n * (2 * sizeof(g1) + 16 + sizeof(PairJob) + 8) +
                n * (4 * sizeof(g1a) + 2 * sizeof(uint2) + 4 * 2 * AGG_SLAB) +
                (n / AGG_MIN_GROUP + 1) * AGG_SLAB * (257 * 4 + 16 * sizeof(g1)) +
                n * std::max(sizeof(sha_ctx), sizeof(shake_ctx)) + 64 * 256;
  rt.arena.reserve(need);
  rt.staging.reserve(65536 + 8 * nm + b.pts48.size() + n * (b.item_size + sizeof(DomainJob) + 96));
  // the blob and the message bytes are already pinned: DMA them directly
  b.dblob = rt.arena.alloc<uint8_t>(b.blob.b.size() ? b.blob.b.size() : 1);
  if (b.blob.b.size()) {
    CUBBS_CHECK(cudaMemcpyAsync(b.dblob, b.blob.b.data(), b.blob.b.size(), cudaMemcpyHostToDevice, rt.stream));
    g_h2d_bytes += b.blob.b.size();
  }
  b.dmsg = rt.arena.alloc<uint8_t>(8 * nm + b.ml.bytes.size() + 1);
  if (nm) {
    upload_to(rt, reinterpret_cast<uint32_t *>(b.dmsg), b.ml.offs.data(), nm);
    upload_to(rt, reinterpret_cast<uint32_t *>(b.dmsg) + nm, b.ml.lens.data(), nm);
    if (b.ml.bytes.size()) {
      CUBBS_CHECK(cudaMemcpyAsync(b.dmsg + 8 * nm, b.ml.bytes.data(), b.ml.bytes.size(), cudaMemcpyHostToDevice,
                                  rt.stream));
      g_h2d_bytes += b.ml.bytes.size();
    }
  }
  b.msc = rt.arena.alloc<fr>(nm ? nm : 1);
  b.dpts48 = upload(rt, b.pts48.data(), b.pts48.size());
  size_t npts = b.pts48.size() / 48;
  b.pts = rt.arena.alloc<g1a>(npts ? npts : 1);
  b.dec = rt.arena.alloc<int32_t>(npts ? npts : 1);
  b.sub = rt.arena.alloc<int32_t>(npts ? npts : 1);
  b.ddj = upload(rt, b.dj.data(), n);
  b.domain = rt.arena.alloc<fr>(n);
  b.ditems0 = upload(rt, b.items.data(), b.items.size());
  b.ditems = rt.arena.alloc<uint8_t>(b.items.size());
  b.rows = rt.arena.alloc<fr>(fr_rows ? fr_rows : 1);
  b.nterms = rt.arena.alloc<uint32_t>(fixed_rows_per_item(b.op) * n);
  b.jobs = rt.arena.alloc<VarJob>(nv ? nv : 1);
  b.jscal = rt.arena.alloc<fr>(nv ? nv : 1);
  b.v = rt.arena.alloc<g1>(nv ? nv : 1);
  b.fixed = rt.arena.alloc<g1>(fixed_rows_per_item(b.op) * n);
  b.pj = rt.arena.alloc<PairJob>(n);
  b.ok = rt.arena.alloc<uint8_t>(n);
  b.e = rt.arena.alloc<fr>(n);
  b.vpts = rt.arena.alloc<g1a>(2 * n);
  if (b.op == OP_PGEN) {
    b.rs = rt.arena.alloc<fr>(n * b.rs_stride);
    b.chal = rt.arena.alloc<uint8_t>(n * std::max(sizeof(sha_ctx), sizeof(shake_ctx)));
    b.r3inv = rt.arena.alloc<fr>(n);
  }
  if (b.op == OP_PVERIFY) {
    plan_groups_of<PvItem>(rt, b);
    b.chal = rt.arena.alloc<uint8_t>(n * std::max(sizeof(sha_ctx), sizeof(shake_ctx)));
  }
  if (b.op == OP_VERIFY) plan_groups_of<VerifyItem>(rt, b);
  b.out = rt.arena.alloc<uint8_t>(b.out_total + 1);
}

// api_id || "MAP_MSG_TO_SCALAR_AS_HASH_" of each suite (ciphersuites.rs:21-79)
static const char *const MAP_DST_H[SUITE_COUNT] = {
    "BBS_BLS12381G1_XMD:SHA-256_SSWU_RO_H2G_HM2S_MAP_MSG_TO_SCALAR_AS_HASH_",
    "BBS_BLS12381G1_XOF:SHAKE-256_SSWU_RO_H2G_HM2S_MAP_MSG_TO_SCALAR_AS_HASH_"};
uint32_t map_dst_len(const Runtime &rt) { return (uint32_t)std::strlen(MAP_DST_H[rt.suite]); }

// Optional per-kernel spans (benchmark breakdown): span k runs from a[k] to
// b[k], both recorded on the stream the kernel is launched on, so kernels that
// run side by side on different streams are timed each on its own stream.
struct StageEvents {
  cudaEvent_t a[16], b[16];
  const char *name[16];
  int used = 0;
};
thread_local StageEvents *g_stages = nullptr;
int span_begin(cudaStream_t s) {
  if (!g_stages || g_stages->used >= 16) return -1;
  CUBBS_CHECK(cudaEventRecord(g_stages->a[g_stages->used], s));
  return g_stages->used++;
}
void span_end(cudaStream_t s, int k, const char *name) {
  if (!g_stages || k < 0) return;
  CUBBS_CHECK(cudaEventRecord(g_stages->b[k], s));
  g_stages->name[k] = name;
}
#define SPAN(stream, label, ...)          \
  do {                                    \
    const int _k = span_begin(stream);    \
    __VA_ARGS__;                          \
    span_end(stream, _k, label);          \
  } while (0)

// The group sums of a batch (k_agg_prep_* has filled agg_pts / agg_sc): the
// bucket MSM when a group has AGG_BUCKET_MIN items or more, else the ladders.
const size_t AGG_BUCKET_MIN = 256;
bool agg_by_buckets(const OpBatch &b) {
  for (size_t g = 0; g + 1 < b.h_goff.size(); g++)
    if (b.h_goff[g + 1] - b.h_goff[g] >= AGG_BUCKET_MIN) return true;
  return false;
}
void launch_agg_buckets(cudaStream_t s, OpBatch &b, uint32_t G) {
  const uint32_t M = (uint32_t)b.h_perm.size();
  if (agg_by_buckets(b)) {
    k_agg_sort<<<dim3(G, AGG_SLAB), 256, 0, s>>>(b.perm, b.goff, b.agg_sc, M, b.agg_ent, b.agg_boff);
    k_agg_buckets<<<AGG_SLAB * G * 8, 64, 0, s>>>(b.agg_pts, b.agg_ent, b.agg_boff, M, b.agg_part);
  } else {
    k_agg_ladder<<<blocks_for(4 * b.n, 32), 32, 0, s>>>(b.agg_pts, b.agg_sc, b.group_of, (uint32_t)b.n, b.scaled);
  }
}
void launch_agg_combine(cudaStream_t s, OpBatch &b, uint32_t G) {
  CUBBS_CHECK(cudaMemsetAsync(b.gjobs, 0, G * sizeof(PairJob), s));
  if (agg_by_buckets(b))
    k_agg_combine<<<dim3(G, 2), 128, 0, s>>>(b.agg_part, b.gslot, b.gjobs);
  else
    k_agg_sum<<<dim3(G, 2), 256, 0, s>>>(b.scaled, b.perm, b.goff, b.gslot, b.gjobs);
}

// ProofVerify on four streams.  Decoding Abar, Bbar, D (stream2) is
// independent of the message hash, the domain and the T2 fixed-base MSM
// (stream); the variable-base terms follow the decode on stream2 and the
// pairing follows it on stream3.  The decode leaves out the subgroup check,
// which runs on stream4 beside the pairing and the variable-base terms: those
// need only the affine points, and the challenge kernel rejects every proof
// with a point outside G1 before any result is read.  Each of these kernels
// fills only part of the GPU, so running them side by side shortens the step.
// The SM partition is used when the batch's key groups fit its small part
// two to an SM: the four streams are then those of the larger partition and
// the aggregated pairing chain (the group sums and one check per key group,
// made of kernels that fill only a few SMs) runs alone on the smaller one;
// sharing SMs with the MSM kernels stretched that chain from about 3.5 ms to
// 5 ms.  With the third partition, stream2 (the decode and the variable-base
// terms) runs on it and the other three streams on the SMs left.  A batch with
// more groups runs on the plain streams (64 keys of 16 proofs: 1.5 % faster on
// the whole GPU than with the chain beside the MSM kernels on the larger part).
void run_pverify(Runtime &rt, OpBatch &b, uint8_t *dmapdst) {
  const bool part = !b.h_gslot.empty() && rt.use_partition() && b.h_gslot.size() <= 2 * (size_t)rt.sh.small_sms;
  cudaStream_t s0 = rt.stream;
  cudaStream_t s = part ? rt.part[0] : rt.stream, s2 = part ? rt.part[1] : rt.stream2;
  cudaStream_t s3 = part ? rt.part[2] : rt.stream3, s4 = part ? rt.part[3] : rt.stream4;
  size_t n = b.n, nm = b.ml.count(), npts = b.pts48.size() / 48;
  uint32_t N = (uint32_t)n, stride = (uint32_t)b.stride;
  PvItem *it = reinterpret_cast<PvItem *>(b.ditems);
  const PvItem *it0 = reinterpret_cast<const PvItem *>(b.ditems0);
  CUBBS_CHECK(cudaEventRecord(rt.ev_fork, s0));
  if (part) CUBBS_CHECK(cudaStreamWaitEvent(s, rt.ev_fork, 0));
  CUBBS_CHECK(cudaStreamWaitEvent(s2, rt.ev_fork, 0));
  if (nm)
    SPAN(s, "hash_messages",
         launch_h2s_flat(s, b.dmsg + 8 * nm, reinterpret_cast<uint32_t *>(b.dmsg),
                         reinterpret_cast<uint32_t *>(b.dmsg) + nm, (uint32_t)nm, dmapdst, map_dst_len(rt), b.msc, rt.suite));
  CUBBS_CHECK(cudaEventRecord(rt.ev_hash, s));
  SPAN(s2, "g1_decode", launch_g1_decode(s2, b.dpts48, 48, (uint32_t)npts, b.pts, b.dec, false));
  CUBBS_CHECK(cudaEventRecord(rt.ev_mid, s2));
  // stream4: the challenge-hash prefix (needs the message scalars), then the
  // subgroup check (needs the decoded points)
  CUBBS_CHECK(cudaStreamWaitEvent(s4, rt.ev_hash, 0));
  SPAN(s4, "challenge_prefix",
       CUBBS_SUITE_DISPATCH(rt.suite, k_pv_chal_prefix<S><<<blocks_for(n, 64), 64, 0, s4>>>(
                                          it0, N, b.dblob, b.msc, reinterpret_cast<hash_ctx<S> *>(b.chal))));
  CUBBS_CHECK(cudaStreamWaitEvent(s4, rt.ev_mid, 0));
  SPAN(s4, "g1_subgroup", launch_g1_subgroup(s4, b.pts, b.dec, (uint32_t)npts, b.sub));
  CUBBS_CHECK(cudaEventRecord(rt.ev_sub, s4));
  CUBBS_CHECK(cudaStreamWaitEvent(s3, rt.ev_mid, 0));
  const uint32_t G = (uint32_t)b.h_gslot.size();
  if (G) {
    AggSeed seed;
    size_t got = 0;
    while (got < sizeof(seed)) {
      ssize_t r = getrandom(reinterpret_cast<uint8_t *>(&seed) + got, sizeof(seed) - got, 0);
      if (r <= 0) throw CudaError(cudaErrorUnknown, "getrandom");
      got += (size_t)r;
    }
    // the group sums and the group checks run on the small partition
    cudaStream_t sa = part ? rt.part_check : s3;
    if (part) {
      CUBBS_CHECK(cudaEventRecord(rt.ev_gc, s3));
      CUBBS_CHECK(cudaStreamWaitEvent(sa, rt.ev_gc, 0));
    }
    SPAN(sa, "agg_buckets",
         k_agg_prep_pv<<<blocks_for(n, 128), 128, 0, sa>>>(it0, N, b.pts, b.dec, b.group_of, seed, b.agg_pts,
                                                            b.agg_sc);
         launch_agg_buckets(sa, b, G));
    SPAN(sa, "agg_sum", launch_agg_combine(sa, b, G));
    SPAN(sa, "pairing_check", launch_pairing_check_split(sa, b.gjobs, G, rt.d_lines, b.gok));
    if (part) {
      CUBBS_CHECK(cudaEventRecord(rt.ev_gc2, sa));
      CUBBS_CHECK(cudaStreamWaitEvent(s3, rt.ev_gc2, 0));
    }
    SPAN(s3, "pairing_kernel",
         k_pv_pairjobs_agg<<<blocks_for(n, 128), 128, 0, s3>>>(it0, N, b.pts, b.dec, b.group_of, b.gok, b.pj,
                                                                b.ok);
         launch_pairing_check(s3, b.pj, N, rt.d_lines, b.ok));
  } else {
    SPAN(s3, "pairing_kernel",
         k_pv_pairjobs<<<blocks_for(n, 128), 128, 0, s3>>>(it0, N, b.pts, b.dec, b.pj);
         launch_pairing_check(s3, b.pj, N, rt.d_lines, b.ok));
  }
  CUBBS_CHECK(cudaEventRecord(rt.ev_join, s3));
  SPAN(s2, "var_mul",
       k_pv_jobs<<<blocks_for(n, 128), 128, 0, s2>>>(it0, N, b.dblob, b.dec, b.jobs, b.jscal);
       launch_var_mul(s2, b.pts, b.jobs, b.jscal, 4 * N, b.v));
  CUBBS_CHECK(cudaEventRecord(rt.ev_side, s2));
  SPAN(s, "domain", launch_domain(s, b.ddj, N, b.dblob, rt.d_gens_c(), rt.ss().d_dom_prefix, b.domain, rt.suite));
  SPAN(s, "scalar_prep",
       k_pv_rows<<<blocks_for(n, 128), 128, 0, s>>>(it, N, b.dblob, b.msc, b.domain, b.rows, stride, b.nterms));
  SPAN(s, "fixed_msm", launch_fixed_msm(s, rt.table(), b.rows, stride, b.nterms, N, b.fixed));
  CUBBS_CHECK(cudaStreamWaitEvent(s, rt.ev_side, 0));
  CUBBS_CHECK(cudaStreamWaitEvent(s, rt.ev_sub, 0));
  SPAN(s, "challenge",
       CUBBS_SUITE_DISPATCH(rt.suite, k_pv_finish<S><<<blocks_for(n, 64), 64, 0, s>>>(it, N, b.dblob, b.msc, b.domain, b.dec, b.sub, b.fixed, b.v,
                                                                                      reinterpret_cast<const hash_ctx<S> *>(b.chal))));
  CUBBS_CHECK(cudaStreamWaitEvent(s, rt.ev_join, 0));
  if (part) {
    CUBBS_CHECK(cudaEventRecord(rt.ev_done, s));
    CUBBS_CHECK(cudaStreamWaitEvent(s0, rt.ev_done, 0));
  }
  b.launches_per_run = (nm ? 1 : 0) + (npts ? 2 : 0) + 9 + (G ? (agg_by_buckets(b) ? 5 : 4) : 0);
}

// ProofGen on three streams: the signature decode (stream3) runs beside
// everything before the variable-base terms; the B-MSM follows the message hash
// and the domain (stream) while the blinding scalars and the T2 fixed-base MSM
// run on stream2; the variable-base terms need all of them.
void run_pgen(Runtime &rt, OpBatch &b, uint8_t *dmapdst) {
  cudaStream_t s = rt.stream, s2 = rt.stream2, s3 = rt.stream3;
  size_t n = b.n, nm = b.ml.count(), npts = b.pts48.size() / 48;
  uint32_t N = (uint32_t)n, stride = (uint32_t)b.stride, rss = (uint32_t)b.rs_stride;
  PgItem *it = reinterpret_cast<PgItem *>(b.ditems);
  const PgItem *it0 = reinterpret_cast<const PgItem *>(b.ditems0);
  CUBBS_CHECK(cudaEventRecord(rt.ev_fork, s));
  CUBBS_CHECK(cudaStreamWaitEvent(s2, rt.ev_fork, 0));
  CUBBS_CHECK(cudaStreamWaitEvent(s3, rt.ev_fork, 0));
  SPAN(s3, "g1_decode", launch_g1_decode(s3, b.dpts48, 48, (uint32_t)npts, b.pts, b.dec, false));
  SPAN(s3, "g1_subgroup", launch_g1_subgroup(s3, b.pts, b.dec, (uint32_t)npts, b.sub));
  CUBBS_CHECK(cudaEventRecord(rt.ev_join, s3));
  SPAN(s2, "random_scalars", CUBBS_SUITE_DISPATCH(rt.suite, k_pg_random<S><<<blocks_for(n, 64), 64, 0, s2>>>(it0, N, b.dblob, b.rs, rss)));
  CUBBS_CHECK(cudaEventRecord(rt.ev_mid, s2));
  SPAN(s2, "fixed_msm_t2",
       k_pg_rows_t2<<<blocks_for(n, 128), 128, 0, s2>>>(it0, N, b.dblob, b.rs, rss, b.rows, stride, b.nterms);
       launch_fixed_msm(s2, rt.table(), b.rows + (size_t)n * stride, stride, b.nterms + n, N, b.fixed + n));
  CUBBS_CHECK(cudaEventRecord(rt.ev_side, s2));
  if (nm)
    SPAN(s, "hash_messages",
         launch_h2s_flat(s, b.dmsg + 8 * nm, reinterpret_cast<uint32_t *>(b.dmsg),
                         reinterpret_cast<uint32_t *>(b.dmsg) + nm, (uint32_t)nm, dmapdst, map_dst_len(rt), b.msc, rt.suite));
  SPAN(s, "domain", launch_domain(s, b.ddj, N, b.dblob, rt.d_gens_c(), rt.ss().d_dom_prefix, b.domain, rt.suite));
  SPAN(s, "fixed_msm",
       k_pg_rows_b<<<blocks_for(n, 128), 128, 0, s>>>(it, N, b.dblob, b.msc, b.domain, b.rows, stride, b.nterms);
       launch_fixed_msm(s, rt.table(), b.rows, stride, b.nterms, N, b.fixed));
  CUBBS_CHECK(cudaStreamWaitEvent(s, rt.ev_mid, 0));  // the blinding scalars
  SPAN(s, "finish_early",
       CUBBS_SUITE_DISPATCH(rt.suite, k_pg_early<S><<<blocks_for(n, 64), 64, 0, s>>>(
                                          it0, N, b.dblob, b.msc, b.rs, rss, reinterpret_cast<hash_ctx<S> *>(b.chal),
                                          b.r3inv)));
  CUBBS_CHECK(cudaStreamWaitEvent(s, rt.ev_side, 0));
  CUBBS_CHECK(cudaStreamWaitEvent(s, rt.ev_join, 0));
  SPAN(s, "var_prep",
       k_pg_vars<<<blocks_for(n, 64), 64, 0, s>>>(it, N, b.dblob, b.fixed, b.pts, b.dec, b.sub, b.rs, rss, b.vpts,
                                                  b.jobs, b.jscal));
  SPAN(s, "var_mul", launch_var_mul(s, b.vpts, b.jobs, b.jscal, 7 * N, b.v));
  SPAN(s, "finish",
       CUBBS_SUITE_DISPATCH(rt.suite, k_pg_finish<S><<<blocks_for(n, 64), 64, 0, s>>>(it, N, b.dblob, b.msc, b.domain, b.rs, rss, b.fixed + n, b.v,
                                                    b.out, reinterpret_cast<const hash_ctx<S> *>(b.chal), b.r3inv)));
  b.launches_per_run = (nm ? 1 : 0) + (npts ? 2 : 0) + 10;
}

// Verify on three streams, as ProofVerify: the signature decode (stream2, no
// subgroup check) and its GLV term run beside the message hash, the domain and
// the B-MSM (stream); the subgroup check runs on stream4; the pairing checks
// follow the finish kernel.  Small batches take the two-warp pairing kernel
// (lower latency per check).
void run_verify(Runtime &rt, OpBatch &b, uint8_t *dmapdst) {
  cudaStream_t s = rt.stream, s2 = rt.stream2, s4 = rt.stream4;
  size_t n = b.n, nm = b.ml.count(), npts = b.pts48.size() / 48;
  uint32_t N = (uint32_t)n, stride = (uint32_t)b.stride;
  VerifyItem *it = reinterpret_cast<VerifyItem *>(b.ditems);
  const VerifyItem *it0 = reinterpret_cast<const VerifyItem *>(b.ditems0);
  CUBBS_CHECK(cudaEventRecord(rt.ev_fork, s));
  CUBBS_CHECK(cudaStreamWaitEvent(s2, rt.ev_fork, 0));
  SPAN(s2, "g1_decode", launch_g1_decode(s2, b.dpts48, 48, (uint32_t)npts, b.pts, b.dec, false));
  CUBBS_CHECK(cudaEventRecord(rt.ev_mid, s2));
  CUBBS_CHECK(cudaStreamWaitEvent(s4, rt.ev_mid, 0));
  SPAN(s4, "g1_subgroup", launch_g1_subgroup(s4, b.pts, b.dec, (uint32_t)npts, b.sub));
  CUBBS_CHECK(cudaEventRecord(rt.ev_sub, s4));
  SPAN(s2, "var_mul",
       k_verify_jobs<<<blocks_for(n, 128), 128, 0, s2>>>(it0, N, b.dblob, b.dec, b.jobs, b.jscal);
       launch_var_mul(s2, b.pts, b.jobs, b.jscal, N, b.v));
  CUBBS_CHECK(cudaEventRecord(rt.ev_side, s2));
  if (nm)
    SPAN(s, "hash_messages",
         launch_h2s_flat(s, b.dmsg + 8 * nm, reinterpret_cast<uint32_t *>(b.dmsg),
                         reinterpret_cast<uint32_t *>(b.dmsg) + nm, (uint32_t)nm, dmapdst, map_dst_len(rt), b.msc, rt.suite));
  SPAN(s, "domain", launch_domain(s, b.ddj, N, b.dblob, rt.d_gens_c(), rt.ss().d_dom_prefix, b.domain, rt.suite));
  SPAN(s, "scalar_prep",
       k_verify_rows<<<blocks_for(n, 128), 128, 0, s>>>(it, N, b.dblob, b.msc, b.domain, b.rows, stride, b.nterms));
  SPAN(s, "fixed_msm", launch_fixed_msm(s, rt.table(), b.rows, stride, b.nterms, N, b.fixed));
  CUBBS_CHECK(cudaStreamWaitEvent(s, rt.ev_side, 0));
  CUBBS_CHECK(cudaStreamWaitEvent(s, rt.ev_sub, 0));
  SPAN(s, "finish",
       k_verify_finish<<<blocks_for(n, 64), 64, 0, s>>>(it, N, b.fixed, b.v, b.pts, b.dec, b.sub, b.pj));
  const uint32_t G = (uint32_t)b.h_gslot.size();
  if (G) {
    // random-coefficient group checks per key, then the per-item checks of the
    // items outside passing groups (as ProofVerify does; see k_agg_prep_pv)
    AggSeed seed;
    size_t got = 0;
    while (got < sizeof(seed)) {
      ssize_t r = getrandom(reinterpret_cast<uint8_t *>(&seed) + got, sizeof(seed) - got, 0);
      if (r <= 0) throw CudaError(cudaErrorUnknown, "getrandom");
      got += (size_t)r;
    }
    SPAN(s, "agg_buckets",
         k_agg_prep_vf<<<blocks_for(n, 128), 128, 0, s>>>(b.pj, N, b.group_of, seed, b.agg_pts, b.agg_sc);
         launch_agg_buckets(s, b, G));
    SPAN(s, "agg_sum", launch_agg_combine(s, b, G));
    SPAN(s, "pairing_check", launch_pairing_check_split(s, b.gjobs, G, rt.d_lines, b.gok));
    SPAN(s, "pairing",
         k_vf_pairjobs_agg<<<blocks_for(n, 128), 128, 0, s>>>(N, b.group_of, b.gok, b.pj, b.ok);
         launch_pairing_check_split(s, b.pj, N, rt.d_lines, b.ok));
  } else if (n <= 256) {
    SPAN(s, "pairing", launch_pairing_check_split(s, b.pj, N, rt.d_lines, b.ok));
  } else {
    SPAN(s, "pairing", launch_pairing_check(s, b.pj, N, rt.d_lines, b.ok));
  }
  b.launches_per_run = (nm ? 1 : 0) + (npts ? 2 : 0) + 7 + (G ? (agg_by_buckets(b) ? 6 : 5) : 0);
}

// The whole device pipeline of one batch (no host work, no transfers).
void run(Runtime &rt, OpBatch &b, uint8_t *dmapdst) {
  cudaStream_t s = rt.stream;
  size_t n = b.n, nm = b.ml.count();
  uint32_t N = (uint32_t)n, stride = (uint32_t)b.stride;
  CUBBS_CHECK(cudaMemcpyAsync(b.ditems, b.ditems0, b.items.size(), cudaMemcpyDeviceToDevice, s));
  if (b.op == OP_PVERIFY || b.op == OP_PGEN || b.op == OP_VERIFY) {
    if (b.op == OP_PVERIFY) run_pverify(rt, b, dmapdst);
    else if (b.op == OP_PGEN) run_pgen(rt, b, dmapdst);
    else run_verify(rt, b, dmapdst);
    CUBBS_CHECK(cudaGetLastError());
    return;
  }
  size_t launches = 0;
  if (nm) {
    SPAN(s, "hash_messages",
         launch_h2s_flat(s, b.dmsg + 8 * nm, reinterpret_cast<uint32_t *>(b.dmsg),
                         reinterpret_cast<uint32_t *>(b.dmsg) + nm, (uint32_t)nm, dmapdst, map_dst_len(rt), b.msc, rt.suite));
    launches++;
  }
  size_t npts = b.pts48.size() / 48;
  if (npts) {
    SPAN(s, "g1_decode", launch_g1_decode(s, b.dpts48, 48, (uint32_t)npts, b.pts, b.dec, true));
    launches++;
  }
  SPAN(s, "domain", launch_domain(s, b.ddj, N, b.dblob, rt.d_gens_c(), rt.ss().d_dom_prefix, b.domain, rt.suite));
  launches++;
  switch (b.op) {
    case OP_PVERIFY:
      break;
    case OP_SIGN: {
      SignItem *it = reinterpret_cast<SignItem *>(b.ditems);
      SPAN(s, "scalar_prep",
           CUBBS_SUITE_DISPATCH(rt.suite, k_sign_prep<S><<<blocks_for(n, 64), 64, 0, s>>>(it, N, b.dblob, b.msc, b.domain, b.rows, stride, b.nterms,
                                                        b.e)));
      SPAN(s, "fixed_msm", launch_fixed_msm(s, rt.table(), b.rows, stride, b.nterms, N, b.fixed));
      SPAN(s, "finish", k_sign_finish<<<blocks_for(n, 64), 64, 0, s>>>(it, N, b.fixed, b.e, b.out));
      launches += 3;
      break;
    }
    case OP_VERIFY:
      break;
    case OP_PGEN:
      break;
  }
  CUBBS_CHECK(cudaGetLastError());
  b.launches_per_run = launches;
}

uint8_t *upload_mapdst(Runtime &rt) {
  return upload(rt, reinterpret_cast<const uint8_t *>(MAP_DST_H[rt.suite]), map_dst_len(rt));
}

// Points every item whose key resolved to a slot at the resident domain-hash
// prefix of its (key slot, L), building the prefixes a batch meets for the
// first time (under the exclusive lock, like the keys' Miller lines).  Items
// keep the full hash when the generators do not cover their L yet.
void attach_domain_prefixes(Runtime &rt, OpBatch &b, const std::vector<int> &slots) {
  if (rt.suite != SUITE_SHA256) return;  // the SHAKE-256 domain hashes its whole input
  SharedState &sh = rt.sh;
  SuiteState &ss = rt.ss();
  std::vector<uint64_t> key(b.n, UINT64_MAX);
  std::vector<std::pair<uint64_t, const uint8_t *>> fresh;
  uint64_t last = UINT64_MAX;
  for (size_t i = 0; i < b.n; i++) {
    const uint32_t L = b.dj[i].L;
    if (slots[i] < 0 || (int)L + 2 > ss.gen_count) continue;
    key[i] = (uint64_t)(uint32_t)slots[i] << 32 | L;
    if (key[i] != last && !ss.dom_prefix.count(key[i])) fresh.emplace_back(key[i], b.pks[i]);
    last = key[i];
  }
  if (!fresh.empty()) {
    rt.lock->unlock();
    {
      std::unique_lock<std::shared_mutex> ex(sh.mu);
      sh.add_domain_prefixes(rt.suite, fresh);
    }
    rt.lock->lock();
  }
  for (size_t i = 0; i < b.n; i++)
    if (key[i] != UINT64_MAX) b.dj[i].prefix = ss.dom_prefix.at(key[i]);
}

void finish_pks(Runtime &rt, OpBatch &b, bool need_table = true) {
  std::vector<int> slots, st;
  rt.resolve_pks(b.pks, slots, st);
  for (size_t i = 0; i < b.n; i++) {
    uint8_t *raw = b.items.data() + i * b.item_size;
    switch (b.op) {
      case OP_PVERIFY: {
        PvItem *p = reinterpret_cast<PvItem *>(raw);
        p->pk_slot = slots[i];
        p->pk_status = st[i];
        if (st[i] == DEC_BAD) p->status = ST_ERROR;
        break;
      }
      case OP_VERIFY: {
        VerifyItem *p = reinterpret_cast<VerifyItem *>(raw);
        p->pk_slot = slots[i];
        p->pk_status = st[i];
        if (st[i] == DEC_BAD) p->status = ST_ERROR;
        break;
      }
      case OP_SIGN:
        reinterpret_cast<SignItem *>(raw)->pk_status = st[i];
        break;
      case OP_PGEN: {
        PgItem *p = reinterpret_cast<PgItem *>(raw);
        p->pk_status = st[i];
        if (st[i] == DEC_BAD && p->status == ST_OK) {
          p->status = ST_ERROR;
          b.code[i] = CUBBS_BBS_GPU_ERR_INVALID_INPUT;
        }
        break;
      }
    }
  }
  if (need_table) rt.ensure_table((int)b.maxL + 2);
  attach_domain_prefixes(rt, b, slots);
}

// --------------------------------------------------------------------------- planners (host packing)
int32_t plan_pverify(const CuBbsBbsGpuProofVerifyItem *items, size_t n, OpBatch &b) {
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if (it.public_key.data == nullptr || it.public_key.len != 96 || (it.proof.len && !it.proof.data) ||
        (it.header.len && !it.header.data) || (it.presentation_header.len && !it.presentation_header.data) ||
        (it.disclosed_count && !it.disclosed_messages) || (it.disclosed_indexes.len && !it.disclosed_indexes.data))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < it.disclosed_count; k++)
      if (it.disclosed_messages[k].len && !it.disclosed_messages[k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  // Every item gets a fixed slot of the blob ([PK][proof][header][ph][pad][indexes u32])
  // and of the message list, from prefix sums of its sizes, so that worker
  // threads can pack disjoint items straight into the pinned buffer.  An item
  // rejected by the shape checks keeps its message slots as empty messages.
  std::vector<size_t> blob_at(n + 1), msg_at(n + 1), byte_at(n + 1);
  blob_at[0] = msg_at[0] = byte_at[0] = 0;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    const size_t slot = 96 + it.proof.len + it.header.len + it.presentation_header.len + 3 + 4 * it.disclosed_indexes.len;
    blob_at[i + 1] = blob_at[i] + ((slot + 3) & ~(size_t)3);
    msg_at[i + 1] = msg_at[i] + it.disclosed_count;
    size_t bytes = 0;
    for (size_t k = 0; k < it.disclosed_count; k++) bytes += it.disclosed_messages[k].len;
    byte_at[i + 1] = byte_at[i] + bytes;
  }
  if (blob_at[n] >= 0xffffffffull || byte_at[n] >= 0xffffffffull) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  b.bind(blob_at[n], byte_at[n], msg_at[n]);
  b.blob.b.used = blob_at[n];
  b.ml.bytes.used = byte_at[n];
  b.ml.offs.resize(msg_at[n]);
  b.ml.lens.resize(msg_at[n]);
  b.op = OP_PVERIFY;
  b.n = n;
  b.item_size = sizeof(PvItem);
  b.items.assign(n * sizeof(PvItem), 0);
  b.pts48.assign(144 * n, 0);
  b.npts_per_item = 3;
  b.pks.resize(n);
  b.code.assign(n, CUBBS_BBS_GPU_SUCCESS);
  b.dj.resize(n);
  auto pack_range = [&](size_t i0, size_t i1, size_t &maxL) {
    std::vector<size_t> di;
    uint8_t *blob = b.blob.b.base;
    for (size_t i = i0; i < i1; i++) {
      const auto &it = items[i];
      PvItem &p = reinterpret_cast<PvItem *>(b.items.data())[i];
      b.pks[i] = it.public_key.data;
      p.status = ST_OK;
      const size_t plen = it.proof.len;
      sort_dedup(it.disclosed_indexes.data, it.disclosed_indexes.len, di);
      const size_t U = plen >= 272 ? (plen - 240) / 32 - 1 : 0;
      const size_t R = di.size(), L = U + R;
      bool ok = plen >= 272 && it.disclosed_count == R && L <= MAX_MESSAGES;
      for (size_t k = 0; k < R && ok; k++) ok = di[k] < L;
      p.msg_base = (uint32_t)msg_at[i];
      size_t at = blob_at[i];
      const uint32_t pk_off = (uint32_t)at;
      std::memcpy(blob + at, it.public_key.data, 96);
      at += 96;
      if (!ok) {
        p.status = ST_INVALID;
        p.proof_off = (uint32_t)at;
        b.dj[i] = {pk_off, 0, 0, 0};
        for (size_t k = msg_at[i]; k < msg_at[i + 1]; k++) {
          b.ml.offs[k] = (uint32_t)byte_at[i];
          b.ml.lens[k] = 0;
        }
        continue;
      }
      size_t bat = byte_at[i];
      for (size_t k = 0; k < it.disclosed_count; k++) {
        const size_t ln = it.disclosed_messages[k].len;
        b.ml.offs[msg_at[i] + k] = (uint32_t)bat;
        b.ml.lens[msg_at[i] + k] = (uint32_t)ln;
        if (ln) std::memcpy(b.ml.bytes.base + bat, it.disclosed_messages[k].data, ln);
        bat += ln;
      }
      p.U = (uint32_t)U;
      p.R = (uint32_t)R;
      p.L = (uint32_t)L;
      const size_t used = 240 + 32 * (U + 1);
      p.proof_off = (uint32_t)at;
      std::memcpy(blob + at, it.proof.data, used);
      at += used;
      p.hdr_off = (uint32_t)at;
      p.hdr_len = (uint32_t)it.header.len;
      if (it.header.len) std::memcpy(blob + at, it.header.data, it.header.len);
      at += it.header.len;
      p.ph_off = (uint32_t)at;
      p.ph_len = (uint32_t)it.presentation_header.len;
      if (it.presentation_header.len) std::memcpy(blob + at, it.presentation_header.data, it.presentation_header.len);
      at += it.presentation_header.len;
      at = (at + 3) & ~(size_t)3;
      p.idx_off = (uint32_t)at;
      for (size_t k = 0; k < R; k++) {
        const uint32_t v = (uint32_t)di[k];
        std::memcpy(blob + at + 4 * k, &v, 4);
      }
      std::memcpy(&b.pts48[144 * i], it.proof.data, 144);
      b.dj[i] = {pk_off, p.hdr_off, p.hdr_len, p.L};
      maxL = std::max(maxL, L);
    }
  };
  const size_t ranges = n >= 256 ? std::min<size_t>(16, n / 64) : 1;
  std::vector<size_t> maxLs(ranges, 0);
  if (ranges == 1) pack_range(0, n, maxLs[0]);
  else PackPool::get().parallel_for(ranges, [&](size_t r) { pack_range(n * r / ranges, n * (r + 1) / ranges, maxLs[r]); });
  for (size_t m : maxLs) b.maxL = std::max(b.maxL, m);
  return CUBBS_BBS_GPU_SUCCESS;
}

int32_t plan_sign(CuBbsBbsGpuSignItem *items, size_t n, OpBatch &b) {
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if (it.secret_key.data == nullptr || it.public_key.data == nullptr || (it.header.len && !it.header.data) ||
        (it.message_count && !it.messages) || it.signature_out.data == nullptr)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < it.message_count; k++)
      if (it.messages[k].len && !it.messages[k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  {
    size_t blob = 0, msg = 0, count = 0;
    for (size_t i = 0; i < n; i++) {
      const auto &it = items[i];
      blob += Blob::room(32) + Blob::room(96) + Blob::room(it.header.len);
      for (size_t k = 0; k < it.message_count; k++) msg += it.messages[k].len;
      count += it.message_count;
    }
    b.bind(blob, msg, count);
  }
  static const uint8_t zero96[96] = {0};
  b.op = OP_SIGN;
  b.n = n;
  b.item_size = sizeof(SignItem);
  b.items.assign(n * sizeof(SignItem), 0);
  b.pks.resize(n);
  b.code.assign(n, CUBBS_BBS_GPU_SUCCESS);
  b.dj.resize(n);
  b.out_total = 80 * n;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    SignItem &p = reinterpret_cast<SignItem *>(b.items.data())[i];
    bool shape = it.secret_key.len == 32 && it.public_key.len == 96 && it.message_count <= MAX_MESSAGES;
    if (shape && it.signature_out.capacity < 80) b.code[i] = CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT;
    else if (!shape) b.code[i] = CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    bool ok = b.code[i] == CUBBS_BBS_GPU_SUCCESS;
    p.status = ok ? ST_OK : ST_ERROR;
    b.pks[i] = it.public_key.len == 96 ? it.public_key.data : zero96;
    p.sk_off = b.blob.put(ok ? it.secret_key.data : zero96, 32);
    p.pk_off = b.blob.put(b.pks[i], 96);
    p.hdr_off = b.blob.put(it.header.data, it.header.len);
    p.hdr_len = (uint32_t)it.header.len;
    p.msg_base = (uint32_t)b.ml.count();
    p.L = ok ? (uint32_t)it.message_count : 0;
    if (ok)
      for (size_t k = 0; k < it.message_count; k++) b.ml.add(it.messages[k].data, it.messages[k].len);
    b.dj[i] = {p.pk_off, p.hdr_off, p.hdr_len, p.L};
    b.maxL = std::max(b.maxL, (size_t)p.L);
  }
  return CUBBS_BBS_GPU_SUCCESS;
}

int32_t plan_verify(const CuBbsBbsGpuVerifyItem *items, size_t n, OpBatch &b) {
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if (it.public_key.data == nullptr || it.public_key.len != 96 || (it.signature.len && !it.signature.data) ||
        (it.header.len && !it.header.data) || (it.message_count && !it.messages))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < it.message_count; k++)
      if (it.messages[k].len && !it.messages[k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  {
    size_t blob = 0, msg = 0, count = 0;
    for (size_t i = 0; i < n; i++) {
      const auto &it = items[i];
      blob += Blob::room(80) + Blob::room(96) + Blob::room(it.header.len);
      for (size_t k = 0; k < it.message_count; k++) msg += it.messages[k].len;
      count += it.message_count;
    }
    b.bind(blob, msg, count);
  }
  static const uint8_t zeros[80] = {0};
  b.op = OP_VERIFY;
  b.n = n;
  b.item_size = sizeof(VerifyItem);
  b.items.assign(n * sizeof(VerifyItem), 0);
  b.pks.resize(n);
  b.code.assign(n, CUBBS_BBS_GPU_SUCCESS);
  b.dj.resize(n);
  b.pts48.assign(48 * n, 0);
  b.npts_per_item = 1;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    VerifyItem &p = reinterpret_cast<VerifyItem *>(b.items.data())[i];
    b.pks[i] = it.public_key.data;
    bool ok = it.signature.len == 80 && it.message_count <= MAX_MESSAGES;
    p.status = ok ? ST_OK : ST_INVALID;
    p.sig_off = b.blob.put(ok ? it.signature.data : zeros, 80);
    if (ok) std::memcpy(&b.pts48[48 * i], it.signature.data, 48);
    uint32_t pk_off = b.blob.put(it.public_key.data, 96);
    p.hdr_off = b.blob.put(it.header.data, it.header.len);
    p.hdr_len = (uint32_t)it.header.len;
    p.msg_base = (uint32_t)b.ml.count();
    p.L = ok ? (uint32_t)it.message_count : 0;
    if (ok)
      for (size_t k = 0; k < it.message_count; k++) b.ml.add(it.messages[k].data, it.messages[k].len);
    b.dj[i] = {pk_off, p.hdr_off, p.hdr_len, p.L};
    b.maxL = std::max(b.maxL, (size_t)p.L);
  }
  return CUBBS_BBS_GPU_SUCCESS;
}

int32_t plan_pgen(CuBbsBbsGpuProofGenItem *items, size_t n, const uint8_t (*seeds)[32], OpBatch &b,
                  std::vector<uint8_t> &os_seeds) {
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if (it.public_key.data == nullptr || it.public_key.len != 96 || (it.signature.len && !it.signature.data) ||
        (it.header.len && !it.header.data) || (it.presentation_header.len && !it.presentation_header.data) ||
        (it.message_count && !it.messages) || (it.disclosed_indexes.len && !it.disclosed_indexes.data) ||
        it.proof_out.data == nullptr)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < it.message_count; k++)
      if (it.messages[k].len && !it.messages[k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  if (seeds == nullptr) {  // production blinding: 32 bytes of OS randomness per item
    os_seeds.resize(32 * n);
    size_t got = 0;
    while (got < os_seeds.size()) {
      ssize_t r = getrandom(os_seeds.data() + got, os_seeds.size() - got, 0);
      if (r <= 0) return CUBBS_BBS_GPU_ERR_INTERNAL;
      got += (size_t)r;
    }
  }
  {
    size_t blob = 0, msg = 0, count = 0;
    for (size_t i = 0; i < n; i++) {
      const auto &it = items[i];
      blob += Blob::room(80) + Blob::room(96) + Blob::room(it.header.len) + Blob::room(it.presentation_header.len) +
              Blob::room(4 * it.disclosed_indexes.len) + Blob::room(32);
      for (size_t k = 0; k < it.message_count; k++) msg += it.messages[k].len;
      count += it.message_count;
    }
    b.bind(blob, msg, count);
  }
  static const uint8_t zeros[80] = {0};
  b.op = OP_PGEN;
  b.n = n;
  b.item_size = sizeof(PgItem);
  b.items.assign(n * sizeof(PgItem), 0);
  b.pks.resize(n);
  b.code.assign(n, CUBBS_BBS_GPU_SUCCESS);
  b.dj.resize(n);
  b.pts48.assign(48 * n, 0);
  b.npts_per_item = 1;
  std::vector<size_t> di;
  std::vector<uint32_t> d32;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    PgItem &p = reinterpret_cast<PgItem *>(b.items.data())[i];
    b.pks[i] = it.public_key.data;
    sort_dedup(it.disclosed_indexes.data, it.disclosed_indexes.len, di);
    size_t L = it.message_count, R = di.size();
    bool ok = it.signature.len == 80 && L <= MAX_MESSAGES && R <= L;
    for (size_t k = 0; k < R && ok; k++) ok = di[k] < L;
    size_t U = ok ? L - R : 0;
    size_t need = 272 + 32 * U;
    if (ok && it.proof_out.capacity < need) {
      b.code[i] = CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT;
      ok = false;
    } else if (!ok) {
      b.code[i] = CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    }
    p.status = ok ? ST_OK : ST_ERROR;
    p.sig_off = b.blob.put(ok ? it.signature.data : zeros, 80);
    if (ok) std::memcpy(&b.pts48[48 * i], it.signature.data, 48);
    uint32_t pk_off = b.blob.put(it.public_key.data, 96);
    p.hdr_off = b.blob.put(it.header.data, it.header.len);
    p.hdr_len = (uint32_t)it.header.len;
    p.ph_off = b.blob.put(it.presentation_header.data, it.presentation_header.len);
    p.ph_len = (uint32_t)it.presentation_header.len;
    d32.assign(di.begin(), di.end());
    p.idx_off = b.blob.put_u32s(d32);
    p.seed_off = b.blob.put(seeds ? seeds[i] : &os_seeds[32 * i], 32);
    p.msg_base = (uint32_t)b.ml.count();
    p.L = ok ? (uint32_t)L : 0;
    p.R = ok ? (uint32_t)R : 0;
    p.U = (uint32_t)U;
    p.out_off = (uint32_t)b.out_total;
    if (ok) {
      b.out_total += need;
      for (size_t k = 0; k < L; k++) b.ml.add(it.messages[k].data, it.messages[k].len);
    }
    b.dj[i] = {pk_off, p.hdr_off, p.hdr_len, p.L};
    b.maxL = std::max(b.maxL, (size_t)p.L);
    b.maxU = std::max(b.maxU, U);
  }
  return CUBBS_BBS_GPU_SUCCESS;
}

// --------------------------------------------------------------------------- result mapping
template <typename ItemT> void fetch_items(Runtime &rt, OpBatch &b, std::vector<ItemT> &out) {
  out.resize(b.n);
  g_d2h_bytes += b.n * sizeof(ItemT);
  CUBBS_CHECK(cudaMemcpyAsync(out.data(), b.ditems, b.n * sizeof(ItemT), cudaMemcpyDeviceToHost, rt.stream));
}

void download_bool(Runtime &rt, OpBatch &b, CuBbsBbsGpuResult *results) {
  std::vector<uint8_t> hok(b.n);
  std::vector<int32_t> st(b.n);
  CUBBS_CHECK(cudaMemcpyAsync(hok.data(), b.ok, b.n, cudaMemcpyDeviceToHost, rt.stream));
  g_d2h_bytes += b.n;
  if (b.op == OP_PVERIFY) {
    std::vector<PvItem> h;
    fetch_items(rt, b, h);
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    for (size_t i = 0; i < b.n; i++) st[i] = h[i].status;
  } else {
    std::vector<VerifyItem> h;
    fetch_items(rt, b, h);
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    for (size_t i = 0; i < b.n; i++) st[i] = h[i].status;
  }
  for (size_t i = 0; i < b.n; i++) {
    if (st[i] == ST_ERROR) results[i] = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
    else results[i] = {CUBBS_BBS_GPU_SUCCESS, (uint8_t)(st[i] == ST_OK && hok[i] ? 1 : 0), 0};
  }
}

}  // namespace

// Runs one packed batch through upload + pipeline (used by the ABI entries and the bench).
static void execute(Runtime &rt, OpBatch &b) {
  g_h2d_bytes = g_d2h_bytes = 0;
  upload(rt, b);
  uint8_t *mapdst = upload_mapdst(rt);
  run(rt, b, mapdst);
}

}  // namespace cubbs

using namespace cubbs;

static bool suite_ok(uint32_t suite) { return suite == CUBBS_BBS_CIPHERSUITE_SHA256 || suite == CUBBS_BBS_CIPHERSUITE_SHAKE256; }

// ----------------------------------------------------------------------------- ProofVerify
static int32_t proof_verify_impl(int suite, const CuBbsBbsGpuProofVerifyItem *items, size_t n,
                                 CuBbsBbsGpuResult *results) {
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    rt.suite = suite;
    OpBatch b(rt);
    int32_t st = plan_pverify(items, n, b);
    if (st != CUBBS_BBS_GPU_SUCCESS) return st;
    finish_pks(rt, b);
    execute(rt, b);
    download_bool(rt, b, results);
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

extern "C" int32_t cubbs_bbs_gpu_proof_verify_batch_v2(uint32_t abi, const CuBbsBbsGpuProofVerifyItem *items,
                                                       size_t n, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return proof_verify_impl(CUBBS_BBS_CIPHERSUITE_SHA256, items, n, results);
}

extern "C" int32_t cubbs_bbs_gpu_proof_verify_batch_cs_v2(uint32_t abi, uint32_t suite,
                                                          const CuBbsBbsGpuProofVerifyItem *items, size_t n,
                                                          CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || !suite_ok(suite) || (n > 0 && (items == nullptr || results == nullptr)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return proof_verify_impl((int)suite, items, n, results);
}

// Test export: host-side phase times (ms) of one ProofVerify call, in order:
// workspace, plan, public keys, upload, device pipeline, results.
extern "C" int32_t cubbs_bbs_gpu_proof_verify_phases_for_test_v2(const CuBbsBbsGpuProofVerifyItem *items, size_t n,
                                                                 CuBbsBbsGpuResult *results, double *ms6) {
  if (!items || !results || !ms6 || n == 0) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  using clk = std::chrono::steady_clock;
  try {
    auto t0 = clk::now();
    CallScope scope;
    Runtime &rt = scope.rt;
    auto t1 = clk::now();
    OpBatch b(rt);
    int32_t st = plan_pverify(items, n, b);
    if (st != CUBBS_BBS_GPU_SUCCESS) return st;
    auto t2 = clk::now();
    finish_pks(rt, b);
    auto t3 = clk::now();
    g_h2d_bytes = g_d2h_bytes = 0;
    upload(rt, b);
    uint8_t *mapdst = upload_mapdst(rt);
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    auto t4 = clk::now();
    run(rt, b, mapdst);
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    auto t5 = clk::now();
    download_bool(rt, b, results);
    auto t6 = clk::now();
    const clk::time_point t[7] = {t0, t1, t2, t3, t4, t5, t6};
    for (int k = 0; k < 6; k++) ms6[k] = std::chrono::duration<double, std::milli>(t[k + 1] - t[k]).count();
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// ----------------------------------------------------------------------------- Verify
static int32_t verify_impl(int suite, const CuBbsBbsGpuVerifyItem *items, size_t n, CuBbsBbsGpuResult *results) {
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    rt.suite = suite;
    OpBatch b(rt);
    int32_t st = plan_verify(items, n, b);
    if (st != CUBBS_BBS_GPU_SUCCESS) return st;
    finish_pks(rt, b);
    execute(rt, b);
    download_bool(rt, b, results);
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

extern "C" int32_t cubbs_bbs_gpu_verify_batch_v2(uint32_t abi, const CuBbsBbsGpuVerifyItem *items, size_t n,
                                                 CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return verify_impl(CUBBS_BBS_CIPHERSUITE_SHA256, items, n, results);
}

extern "C" int32_t cubbs_bbs_gpu_verify_batch_cs_v2(uint32_t abi, uint32_t suite, const CuBbsBbsGpuVerifyItem *items,
                                                    size_t n, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || !suite_ok(suite) || (n > 0 && (items == nullptr || results == nullptr)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return verify_impl((int)suite, items, n, results);
}

// ----------------------------------------------------------------------------- Sign
static int32_t sign_impl(int suite, CuBbsBbsGpuSignItem *items, size_t n, CuBbsBbsGpuResult *results) {
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    rt.suite = suite;
    OpBatch b(rt);
    int32_t st = plan_sign(items, n, b);
    if (st != CUBBS_BBS_GPU_SUCCESS) return st;
    finish_pks(rt, b);
    execute(rt, b);
    std::vector<uint8_t> hsig(80 * n);
    std::vector<SignItem> h;
    CUBBS_CHECK(cudaMemcpyAsync(hsig.data(), b.out, 80 * n, cudaMemcpyDeviceToHost, rt.stream));
    g_d2h_bytes += 80 * n;
    fetch_items(rt, b, h);
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    for (size_t i = 0; i < n; i++) {
      if (b.code[i] != CUBBS_BBS_GPU_SUCCESS) {
        results[i] = {b.code[i], 0, 0};
      } else if (h[i].status != ST_OK) {
        results[i] = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
      } else {
        std::memcpy(items[i].signature_out.data, &hsig[80 * i], 80);
        items[i].signature_out.len = 80;
        results[i] = {CUBBS_BBS_GPU_SUCCESS, 0, 80};
      }
    }
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

extern "C" int32_t cubbs_bbs_gpu_sign_batch_v2(uint32_t abi, CuBbsBbsGpuSignItem *items, size_t n,
                                               CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return sign_impl(CUBBS_BBS_CIPHERSUITE_SHA256, items, n, results);
}

extern "C" int32_t cubbs_bbs_gpu_sign_batch_cs_v2(uint32_t abi, uint32_t suite, CuBbsBbsGpuSignItem *items, size_t n,
                                                  CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || !suite_ok(suite) || (n > 0 && (items == nullptr || results == nullptr)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return sign_impl((int)suite, items, n, results);
}

// ----------------------------------------------------------------------------- ProofGen
static int32_t proof_gen_impl(int suite, CuBbsBbsGpuProofGenItem *items, size_t n, const uint8_t (*seeds)[32],
                              CuBbsBbsGpuResult *results) {
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    rt.suite = suite;
    OpBatch b(rt);
    std::vector<uint8_t> os_seeds;
    int32_t st = plan_pgen(items, n, seeds, b, os_seeds);
    if (st != CUBBS_BBS_GPU_SUCCESS) return st;
    finish_pks(rt, b);
    execute(rt, b);
    std::vector<uint8_t> hout(b.out_total + 1);
    std::vector<PgItem> h;
    CUBBS_CHECK(cudaMemcpyAsync(hout.data(), b.out, b.out_total + 1, cudaMemcpyDeviceToHost, rt.stream));
    g_d2h_bytes += b.out_total + 1;
    fetch_items(rt, b, h);
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    const PgItem *hp = reinterpret_cast<const PgItem *>(b.items.data());
    for (size_t i = 0; i < n; i++) {
      if (b.code[i] != CUBBS_BBS_GPU_SUCCESS) {
        results[i] = {b.code[i], 0, 0};
      } else if (h[i].status != ST_OK) {
        results[i] = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
      } else {
        size_t need = 272 + 32 * (size_t)hp[i].U;
        std::memcpy(items[i].proof_out.data, &hout[hp[i].out_off], need);
        items[i].proof_out.len = need;
        results[i] = {CUBBS_BBS_GPU_SUCCESS, 0, need};
      }
    }
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

extern "C" int32_t cubbs_bbs_gpu_proof_gen_batch_v2(uint32_t abi, CuBbsBbsGpuProofGenItem *items, size_t n,
                                                    CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  return proof_gen_impl(CUBBS_BBS_CIPHERSUITE_SHA256, items, n, nullptr, results);
}

extern "C" int32_t cubbs_bbs_gpu_proof_gen_batch_cs_v2(uint32_t abi, uint32_t suite, CuBbsBbsGpuProofGenItem *items,
                                                       size_t n, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || !suite_ok(suite) || (n > 0 && (items == nullptr || results == nullptr)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  return proof_gen_impl((int)suite, items, n, nullptr, results);
}

extern "C" int32_t cubbs_bbs_gpu_proof_gen_seeded_batch_v2(uint32_t abi, CuBbsBbsGpuProofGenItem *items, size_t n,
                                                           const uint8_t (*seeds)[32], CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr || seeds == nullptr)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  return proof_gen_impl(CUBBS_BBS_CIPHERSUITE_SHA256, items, n, seeds, results);
}

extern "C" int32_t cubbs_bbs_gpu_proof_gen_seeded_batch_cs_v2(uint32_t abi, uint32_t suite,
                                                              CuBbsBbsGpuProofGenItem *items, size_t n,
                                                              const uint8_t (*seeds)[32], CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || !suite_ok(suite) || (n > 0 && (items == nullptr || results == nullptr || seeds == nullptr)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  return proof_gen_impl((int)suite, items, n, seeds, results);
}

// ----------------------------------------------------------------------------- device-resident timing
// Benchmark entry (outside the reference ABI): packs and uploads one batch of
// the given operation once, then replays the whole device pipeline warmup +
// steps times on the library's stream.  Each timed step is bracketed by CUDA
// events on that stream; between steps a 256 MiB buffer is rewritten to evict
// L2 (outside the events).  op: 0 Sign, 1 Verify, 2 ProofGen (items seeded by
// seeds), 3 ProofVerify.  ms_out[k] = duration of step k; *launches = kernels
// per step.  The results of the last step are returned in results as the ABI
// call would.
static char g_stage_names[16][32];
static float g_stage_ms[16];
static int g_stage_count = 0;

extern "C" int32_t cubbs_bbs_gpu_bench_device_steps_v2(uint32_t abi, int32_t op, void *items, size_t n,
                                                       const uint8_t (*seeds)[32], int32_t warmup, int32_t steps,
                                                       float *ms_out, int32_t *launches, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || !items || n == 0 || !ms_out || !launches || !results || steps <= 0 || warmup < 0)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    OpBatch b(rt);
    std::vector<uint8_t> os_seeds;
    int32_t st;
    switch (op) {
      case 0: st = plan_sign(static_cast<CuBbsBbsGpuSignItem *>(items), n, b); break;
      case 1: st = plan_verify(static_cast<const CuBbsBbsGpuVerifyItem *>(items), n, b); break;
      case 2: st = plan_pgen(static_cast<CuBbsBbsGpuProofGenItem *>(items), n, seeds, b, os_seeds); break;
      case 3: st = plan_pverify(static_cast<const CuBbsBbsGpuProofVerifyItem *>(items), n, b); break;
      default: return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    }
    if (st != CUBBS_BBS_GPU_SUCCESS) return st;
    finish_pks(rt, b);
    upload(rt, b);
    uint8_t *mapdst = upload_mapdst(rt);
    static uint8_t *flush = nullptr;
    const size_t FLUSH = (size_t)256 << 20;
    if (!flush) CUBBS_CHECK(cudaMalloc(&flush, FLUSH));
    cudaEvent_t e0, e1;
    CUBBS_CHECK(cudaEventCreate(&e0));
    CUBBS_CHECK(cudaEventCreate(&e1));
    for (int k = 0; k < warmup + steps; k++) {
      CUBBS_CHECK(cudaMemsetAsync(flush, k & 0xff, FLUSH, rt.stream));
      CUBBS_CHECK(cudaEventRecord(e0, rt.stream));
      run(rt, b, mapdst);
      CUBBS_CHECK(cudaEventRecord(e1, rt.stream));
      CUBBS_CHECK(cudaEventSynchronize(e1));
      float ms = 0;
      CUBBS_CHECK(cudaEventElapsedTime(&ms, e0, e1));
      if (k >= warmup) ms_out[k - warmup] = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *launches = (int32_t)b.launches_per_run;
    // one extra untimed replay with per-kernel spans for the breakdown
    StageEvents se;
    for (int k = 0; k < 16; k++) {
      CUBBS_CHECK(cudaEventCreate(&se.a[k]));
      CUBBS_CHECK(cudaEventCreate(&se.b[k]));
    }
    g_stages = &se;
    CUBBS_CHECK(cudaMemsetAsync(flush, 0x5a, FLUSH, rt.stream));
    run(rt, b, mapdst);
    g_stages = nullptr;
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    g_stage_count = se.used;
    for (int k = 0; k < se.used; k++) {
      float ms = 0;
      CUBBS_CHECK(cudaEventElapsedTime(&ms, se.a[k], se.b[k]));
      g_stage_ms[k] = ms;
      std::snprintf(g_stage_names[k], 32, "%s", se.name[k]);
    }
    for (int k = 0; k < 16; k++) {
      cudaEventDestroy(se.a[k]);
      cudaEventDestroy(se.b[k]);
    }
    if (op == 1 || op == 3) {
      download_bool(rt, b, results);
    } else {
      std::vector<uint8_t> codes(n);
      if (op == 0) {
        std::vector<SignItem> h;
        fetch_items(rt, b, h);
        CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
        for (size_t i = 0; i < n; i++) results[i] = {h[i].status == ST_OK ? 0 : 1, 0, 80};
      } else {
        std::vector<PgItem> h;
        fetch_items(rt, b, h);
        CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
        for (size_t i = 0; i < n; i++) results[i] = {h[i].status == ST_OK ? 0 : 1, 0, 0};
      }
    }
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// Test export: H2S(s_0 || ... || s_{n-1}, api_id || "H2S_") over canonical scalars,
// absorbed exactly as the Sign e-hash and the challenge hash do (parse -> raw -> BE).
__global__ void k_h2s_scalars_test(const uint8_t *be, uint32_t n, fr *out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  sha_ctx c;
  xmd_begin(c);
  for (uint32_t k = 0; k < n; k++) {
    fr s;
    fr_raw_from_be32(be + 32 * k, s);
    sha_fr_be(c, s);
  }
  out[0] = h2s_finish(c, DST_H2S, DST_H2S_LEN);
}

extern "C" int32_t cubbs_bbs_gpu_h2s_scalars_for_test_v2(uint32_t abi, const uint8_t *be, size_t n, uint8_t *out32) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || !be || !out32 || n == 0) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    uint8_t *d = rt.arena.alloc<uint8_t>(32 * n);
    fr *o = rt.arena.alloc<fr>(1);
    CUBBS_CHECK(cudaMemcpy(d, be, 32 * n, cudaMemcpyHostToDevice));
    k_h2s_scalars_test<<<1, 32, 0, rt.stream>>>(d, (uint32_t)n, o);
    CUBBS_CHECK(cudaGetLastError());
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    uint32_t raw[8];
    CUBBS_CHECK(cudaMemcpy(raw, o, 32, cudaMemcpyDeviceToHost));
    for (int w = 0; w < 8; w++)
      for (int b = 0; b < 4; b++) out32[(7 - w) * 4 + (3 - b)] = (uint8_t)(raw[w] >> (8 * b));
    return 0;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// Test export: the disclosed-pair part of the challenge, H2S(I2OSP(R,8) || (I2OSP(i_k,8) || m_k)...),
// with the indexes read as uint32 from a byte blob at offset idx_off (as the proof kernels do).
__global__ void k_pairs_test(const uint8_t *blob, uint32_t idx_off, uint32_t R, const uint8_t *mbe, fr *out,
                             uint32_t *echo) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const uint32_t *idx = reinterpret_cast<const uint32_t *>(blob + idx_off);
  sha_ctx c;
  xmd_begin(c);
  sha_u64be(c, R, 8);
  for (uint32_t k = 0; k < R; k++) {
    echo[k] = idx[k];
    sha_u64be(c, idx[k], 8);
    fr m;
    fr_raw_from_be32(mbe + 32 * k, m);
    sha_fr_be(c, m);
  }
  out[0] = h2s_finish(c, DST_H2S, DST_H2S_LEN);
}

extern "C" int32_t cubbs_bbs_gpu_pairs_h2s_for_test_v2(uint32_t abi, const uint8_t *blob, size_t blob_len,
                                                       uint32_t idx_off, uint32_t R, const uint8_t *mbe,
                                                       uint8_t *out32, uint32_t *echo) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    uint8_t *d = rt.arena.alloc<uint8_t>(blob_len + 1);
    uint8_t *dm = rt.arena.alloc<uint8_t>(32 * R + 1);
    uint32_t *de = rt.arena.alloc<uint32_t>(R + 1);
    fr *o = rt.arena.alloc<fr>(1);
    CUBBS_CHECK(cudaMemcpy(d, blob, blob_len, cudaMemcpyHostToDevice));
    if (R) CUBBS_CHECK(cudaMemcpy(dm, mbe, 32 * R, cudaMemcpyHostToDevice));
    k_pairs_test<<<1, 32, 0, rt.stream>>>(d, idx_off, R, dm, o, de);
    CUBBS_CHECK(cudaGetLastError());
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    uint32_t raw[8];
    CUBBS_CHECK(cudaMemcpy(raw, o, 32, cudaMemcpyDeviceToHost));
    if (R) CUBBS_CHECK(cudaMemcpy(echo, de, 4 * R, cudaMemcpyDeviceToHost));
    for (int w = 0; w < 8; w++)
      for (int b = 0; b < 4; b++) out32[(7 - w) * 4 + (3 - b)] = (uint8_t)(raw[w] >> (8 * b));
    return 0;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

extern "C" int32_t cubbs_bbs_gpu_last_debug_record_for_test_v2(uint8_t *out256) {
  if (!out256) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return cudaMemcpyFromSymbol(out256, g_debug_record, 256) == cudaSuccess ? 0 : CUBBS_BBS_GPU_ERR_INTERNAL;
}

// Stage breakdown of the last bench_device_steps call: returns the number of
// stages; names are written as 32-byte NUL-padded strings.
extern "C" int32_t cubbs_bbs_gpu_bench_stages_v2(char *names32, float *ms, int32_t cap) {
  int k = 0;
  for (; k < g_stage_count && k < cap; k++) {
    std::memcpy(names32 + 32 * k, g_stage_names[k], 32);
    ms[k] = g_stage_ms[k];
  }
  return k;
}

extern "C" int32_t cubbs_bbs_gpu_last_transfer_bytes_v2(uint64_t *h2d, uint64_t *d2h) {
  if (!h2d || !d2h) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  *h2d = g_h2d_bytes;
  *d2h = g_d2h_bytes;
  return 0;
}
