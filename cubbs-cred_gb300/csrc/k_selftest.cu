// Test-only exports (outside the ABI header, like the reference's
// *_for_test_v2 symbols): raw device field and curve operations so that parity
// tests can localise a mismatch to one layer (Fp, decode, scalar mul, encode).
#include <cstring>
#include <vector>

#include "runtime.cuh"

namespace cubbs {

// variants of [|z|]P used to localise a miscompare
DEV g1 zabs_inline(const g1 &p) {
  g1 acc = p;
#pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    acc = g1_dbl(acc);
    if (zabs_bit(i)) acc = g1_add(acc, p);
  }
  return acc;
}
DEV g1 zabs_local(g1 p) {
  volatile g1 keep[1];
  for (int k = 0; k < 12; k++) {
    keep[0].X.w[k] = p.X.w[k]; keep[0].Y.w[k] = p.Y.w[k];
    keep[0].ZZ.w[k] = p.ZZ.w[k]; keep[0].ZZZ.w[k] = p.ZZZ.w[k];
  }
  g1 acc = p;
#pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    acc = g1_dbl(acc);
    if (zabs_bit(i)) {
      g1 b;
      for (int k = 0; k < 12; k++) {
        b.X.w[k] = keep[0].X.w[k]; b.Y.w[k] = keep[0].Y.w[k];
        b.ZZ.w[k] = keep[0].ZZ.w[k]; b.ZZZ.w[k] = keep[0].ZZZ.w[k];
      }
      acc = g1_add(acc, b);
    }
  }
  return acc;
}
DEV g1 zabs_unrolled_bits(g1 p) {
  // |z| = 2^63 + 2^62 + 2^60 + 2^57 + 2^48 + 2^16, Horner over the set bits
  g1 acc = p;
  const int gaps[5] = {1, 2, 3, 9, 32};
  for (int j = 0; j < 5; j++) {
#pragma unroll 1
    for (int d = 0; d < gaps[j]; d++) acc = g1_dbl(acc);
    acc = g1_add(acc, p);
  }
#pragma unroll 1
  for (int d = 0; d < 16; d++) acc = g1_dbl(acc);
  return acc;
}

// op 0: Fp product of canonical BE inputs; op 1: Fp inverse; op 2: Fp sqrt (0 if none);
// op 3: variable-time Fp inverse; op 4: Fp product by CIOS carry chains
__global__ void k_fp_test(const uint8_t *a, const uint8_t *b, uint32_t n, int op, uint8_t *out, int32_t *st) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fp x, y, r = fp_zero();
  bool ok = fp_from_be48(a + 48 * (size_t)i, x) && fp_from_be48(b + 48 * (size_t)i, y);
  if (ok) {
    if (op == 0) r = fp_mul(x, y);
    else if (op == 4) r = fp_mul_cios(x, y);
    else if (op == 1) r = fp_inv(x);
    else if (op == 3) r = fp_inv_vartime(x);
    else ok = fp_sqrt(x, r);
  }
  st[i] = ok ? 0 : 1;
  fp_to_be48(r, out + 48 * (size_t)i);
}

// decode (subgroup-checked) then re-encode; also k*P via GLV when k given
__global__ void k_g1_test(const uint8_t *pts, const uint8_t *ks, uint32_t n, uint8_t *xy, uint8_t *kp,
                          int32_t *st) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint8_t b[48];
  for (int k = 0; k < 48; k++) b[k] = pts[48 * (size_t)i + k];
  g1a a;
  int s = g1_decompress(b, a, false);  // unchecked decode first
  st[i] = s * 16;
  if (s != DEC_OK) return;
  st[i] = g1_decompress(b, a, true);
  // diagnostics in kp slots beyond n: 2P, 3P, [|z|]P, [z^2]P compressed
  g1 P = g1_from_aff(a);
  g1 d = g1_dbl(P);
  uint8_t *o = kp + 48 * (size_t)(n + 12 * i);
  g1_compress(d, o);                                  // 2P
  g1_compress(g1_add(d, P), o + 48);                  // 3P
  g1_compress(g1_add_aff(d, a), o + 96);              // 3P
  g1 q = g1_dbl(d);
  g1_compress(q, o + 144);                            // 4P
  g1_compress(g1_add(q, P), o + 192);                 // 5P
  g1_compress(g1_add(d, d), o + 240);                 // 4P via add
  g1 t = g1_add(q, d);                                // 6P
  g1_compress(g1_add(t, g1_dbl(t)), o + 288);         // 18P
  g1_compress(g1_mul_zabs(P), o + 336);               // [|z|]P
  g1_compress(zabs_inline(P), o + 48 * 9);
  g1_compress(zabs_local(P), o + 48 * 10);
  g1_compress(zabs_unrolled_bits(P), o + 48 * 11);
  // doubling chain 2^k P, k = 1..64
  g1 c = P;
  uint8_t *oc = kp + 48 * (size_t)(13 * n + 64 * i);
  #pragma unroll 1
  for (int k = 0; k < 64; k++) {
    c = g1_dbl(c);
    g1_compress(c, oc + 48 * k);
  }
  fp_to_be48(a.x, xy + 96 * (size_t)i);
  fp_to_be48(a.y, xy + 96 * (size_t)i + 48);
  fr k;
  fr_raw_from_be32(ks + 32 * (size_t)i, k);
  g1_compress(g1_mul_glv(a, k), kp + 48 * (size_t)i);
}

}  // namespace cubbs

using namespace cubbs;

static int32_t run_test(int kind, int op, const uint8_t *a, const uint8_t *b, size_t n, uint8_t *out, uint8_t *out2,
                        int32_t *status) {
  if (n == 0) return 0;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    size_t asz = kind == 0 ? 48 : 48, bsz = kind == 0 ? 48 : 32;
    uint8_t *da = rt.arena.alloc<uint8_t>(asz * n), *db = rt.arena.alloc<uint8_t>(bsz * n);
    uint8_t *d1 = rt.arena.alloc<uint8_t>(96 * n), *d2 = rt.arena.alloc<uint8_t>(48 * (13 + 64) * n);
    int32_t *ds = rt.arena.alloc<int32_t>(n);
    CUBBS_CHECK(cudaMemcpy(da, a, asz * n, cudaMemcpyHostToDevice));
    CUBBS_CHECK(cudaMemcpy(db, b, bsz * n, cudaMemcpyHostToDevice));
    if (kind == 0) k_fp_test<<<blocks_for(n, 64), 64, 0, rt.stream>>>(da, db, (uint32_t)n, op, d1, ds);
    else k_g1_test<<<blocks_for(n, 64), 64, 0, rt.stream>>>(da, db, (uint32_t)n, d1, d2, ds);
    CUBBS_CHECK(cudaGetLastError());
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    CUBBS_CHECK(cudaMemcpy(out, d1, (kind == 0 ? 48 : 96) * n, cudaMemcpyDeviceToHost));
    if (out2) CUBBS_CHECK(cudaMemcpy(out2, d2, 48 * (13 + 64) * n, cudaMemcpyDeviceToHost));
    CUBBS_CHECK(cudaMemcpy(status, ds, 4 * n, cudaMemcpyDeviceToHost));
    return 0;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// op: 0 mul, 1 inverse, 2 sqrt, 3 variable-time inverse.  Inputs and outputs are 48-byte
// big-endian canonical.
extern "C" int32_t cubbs_bbs_gpu_fp_op_for_test_v2(uint32_t abi, int32_t op, const uint8_t *a, const uint8_t *b,
                                                   size_t n, uint8_t *out, int32_t *status) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (n && (!a || !b || !out || !status))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return run_test(0, op, a, b, n, out, nullptr, status);
}

// Decodes points (status DEC_*, or 16*DEC_* when the unchecked decode fails), writes affine
// x||y (96 B BE), k*P compressed, then per point 2P, 3P (add), 3P (mixed add), [|z|]P.
extern "C" int32_t cubbs_bbs_gpu_g1_op_for_test_v2(uint32_t abi, const uint8_t *pts48, const uint8_t *k32, size_t n,
                                                   uint8_t *xy96, uint8_t *kp48, int32_t *status) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (n && (!pts48 || !k32 || !xy96 || !kp48 || !status)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  return run_test(1, 0, pts48, k32, n, xy96, kp48, status);
}

// Decode without the subgroup check, then the separate subgroup kernel (the
// ProofVerify split): status[i] = decode status, outside[i] = 1 when point i
// decoded to a point outside G1.
extern "C" int32_t cubbs_bbs_gpu_g1_subgroup_for_test_v2(uint32_t abi, const uint8_t *pts48, size_t n,
                                                         int32_t *status, int32_t *outside) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || n == 0 || !pts48 || !status || !outside)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    uint8_t *d = rt.arena.alloc<uint8_t>(48 * n);
    g1a *pts = rt.arena.alloc<g1a>(n);
    int32_t *st = rt.arena.alloc<int32_t>(n), *bad = rt.arena.alloc<int32_t>(n);
    CUBBS_CHECK(cudaMemcpyAsync(d, pts48, 48 * n, cudaMemcpyHostToDevice, rt.stream));
    launch_g1_decode(rt.stream, d, 48, (uint32_t)n, pts, st, false);
    launch_g1_subgroup(rt.stream, pts, st, (uint32_t)n, bad);
    CUBBS_CHECK(cudaGetLastError());
    CUBBS_CHECK(cudaMemcpyAsync(status, st, 4 * n, cudaMemcpyDeviceToHost, rt.stream));
    CUBBS_CHECK(cudaMemcpyAsync(outside, bad, 4 * n, cudaMemcpyDeviceToHost, rt.stream));
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    return 0;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// ------------------------------------------------------------------------- integer-pipe peak
// Peak 32-bit multiply-add throughput: every thread runs 16 independent
// mad.lo chains (no carries), so issue rate, not latency, bounds the kernel.
__global__ void __launch_bounds__(256) k_imad_peak(uint32_t *out, uint32_t iters, uint32_t seed) {
  uint32_t a[16];
#pragma unroll
  for (int k = 0; k < 16; k++) a[k] = seed + threadIdx.x * 16 + k;
  const uint32_t m = 0x9e3779b9u + blockIdx.x;
#pragma unroll 1
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int r = 0; r < 8; r++) {
#pragma unroll
      for (int k = 0; k < 16; k++) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[k]) : "r"(m), "r"(k + 1));
    }
  }
  uint32_t x = 0;
#pragma unroll
  for (int k = 0; k < 16; k++) x ^= a[k];
  if (x == 0x12345678u) out[0] = x;  // keeps the chains live
}

// Fp Montgomery products per second at full occupancy (4 independent products per thread).
__global__ void __launch_bounds__(256) k_fpmul_rate(fp *out, uint32_t iters) {
  fp a = fp_one(), b = fp_one(), c = fp_one(), d = fp_one();
  a.w[0] += threadIdx.x; b.w[1] += blockIdx.x; c.w[2] += 3; d.w[3] += 5;
  fp k = fp_one();
  k.w[4] ^= threadIdx.x * 7u;
#pragma unroll 1
  for (uint32_t it = 0; it < iters; it++) {
    a = fp_mul(a, k);
    b = fp_mul(b, k);
    c = fp_mul(c, k);
    d = fp_mul(d, k);
  }
  if (fp_is_zero(a) && fp_is_zero(b) && fp_is_zero(c) && fp_is_zero(d)) out[0] = a;
}

// CIOS products per second (same shape as k_fpmul_rate).
__global__ void __launch_bounds__(256) k_fpmul_cios_rate(fp *out, uint32_t iters) {
  fp a = fp_one(), b = fp_one(), c = fp_one(), d = fp_one();
  a.w[0] += threadIdx.x; b.w[1] += blockIdx.x; c.w[2] += 3; d.w[3] += 5;
  fp k = fp_one();
  k.w[4] ^= threadIdx.x * 7u;
#pragma unroll 1
  for (uint32_t it = 0; it < iters; it++) {
    a = fp_mul_cios(a, k);
    b = fp_mul_cios(b, k);
    c = fp_mul_cios(c, k);
    d = fp_mul_cios(d, k);
  }
  if (fp_is_zero(a) && fp_is_zero(b) && fp_is_zero(c) && fp_is_zero(d)) out[0] = a;
}

// Code-size variants of the Fp product for the latency probe.
DEVNI fp fp_mul_call(fp a, fp b) { return fp_mul_inl(a, b); }
DEV fp fp_mul_rolled(const fp &a, fp b) {
  uint32_t t[13];
#pragma unroll
  for (int j = 0; j < 13; j++) t[j] = 0;
#pragma unroll 1
  for (int i = 0; i < 12; i++) {
    fp_cios_row(t, a.w, b.w[0]);
#pragma unroll
    for (int j = 0; j < 12; j++) t[j] = t[j + 1];
    t[12] = 0;
#pragma unroll
    for (int j = 0; j < 11; j++) b.w[j] = b.w[j + 1];
  }
  fp r;
  fp_reduce_once(r.w, t);
  return r;
}
#define G1_DBL_WITH(NAME, MUL)                                   \
  DEVNI g1 NAME(g1 p) {                                          \
    if (g1_is_inf(p)) return p;                                  \
    fp U = fp_dbl(p.Y);                                          \
    fp V = MUL(U, U);                                            \
    fp W = MUL(U, V);                                            \
    fp S = MUL(p.X, V);                                          \
    fp X2 = MUL(p.X, p.X);                                       \
    fp M = fp_add(fp_dbl(X2), X2);                               \
    g1 r;                                                        \
    r.X = fp_sub(fp_sub(MUL(M, M), S), S);                       \
    r.Y = fp_sub(MUL(M, fp_sub(S, r.X)), MUL(W, p.Y));           \
    r.ZZ = MUL(V, p.ZZ);                                         \
    r.ZZZ = MUL(W, p.ZZZ);                                       \
    return r;                                                    \
  }
G1_DBL_WITH(g1_dbl_call, fp_mul_call)
G1_DBL_WITH(g1_dbl_rolled, fp_mul_rolled)
G1_DBL_WITH(g1_dbl_cios, fp_mul_cios)

// Single-warp latency of dependent chains, in SM cycles per operation
// (clock64 around n iterations; every lane runs the same chain).
//   0 fp_mul (out of line)   1 three independent fp_mul chains (cycles per iteration)
//   2 fp_add   3 fp2_mul   4 fp2_sqr   5 fp12_sqr   6 fp12_mul
//   7 fp12_mul_line   8 g1_dbl   9 g1_add_aff   10 g1_add   11 fr_mul
//   12 g1_dbl_inl   13 g1_add_aff_inl   14 fp2_mul_inl   15 fp_sqr chain of 64 (one fp_pow step)
//   16 inlined fp_mul   17 three independent inlined fp_mul chains
//   18/19 out-of-line fp_mul (1 / 3 chains)   20/21 rolled-loop fp_mul (1 / 3 chains)
//   22 g1_dbl over out-of-line fp_mul   23 g1_dbl over rolled fp_mul
//   24/25 CIOS fp_mul out of line (1 / 3 chains)   26 CIOS inlined
//   27 g1_dbl over CIOS fp_mul   28 fp_inv_vartime
__global__ void __launch_bounds__(32) k_latency_probe(double *cyc, fp *sink, uint32_t n) {
  fp a = fp_one(), b = fp_one(), c = fp_one(), k = fp_one();
  a.w[0] += threadIdx.x + 3;
  b.w[1] += 7;
  c.w[2] += 11;
  k.w[3] ^= 0x55u;
  fp2 x2 = {a, b}, k2 = {b, c};
  fp12 f, g;
  f.c0 = {x2, k2, x2};
  f.c1 = {k2, x2, k2};
  g = f;
  g1 P = {a, b, fp_one(), fp_one()};
  g1a Q = {c, k};
  g1 Rr = {k, c, fp_one(), fp_one()};
  fr s = fr_one(), sk = fr_one();
  sk.w[1] ^= 0x1234u;
  long long t0, t1;
  const int R = 29;
  double res[R];
#define LAT(IDX, ITERS, BODY)                          \
  t0 = clock64();                                      \
  _Pragma("unroll 1") for (uint32_t it = 0; it < (ITERS); it++) { BODY; } \
  t1 = clock64();                                      \
  res[IDX] = (double)(t1 - t0) / (ITERS);
  LAT(0, n, a = fp_mul(a, k));
  LAT(1, n, a = fp_mul(a, k); b = fp_mul(b, k); c = fp_mul(c, k));
  LAT(2, n, a = fp_add(a, k));
  LAT(3, n, x2 = fp2_mul(x2, k2));
  LAT(4, n, x2 = fp2_sqr(x2));
  LAT(5, n / 8, f = fp12_sqr(f));
  LAT(6, n / 8, f = fp12_mul(f, g));
  LAT(7, n / 8, f = fp12_mul_line(f, k2, x2, c));
  LAT(8, n / 4, P = g1_dbl(P));
  LAT(9, n / 4, P = g1_add_aff(P, Q));
  LAT(10, n / 4, P = g1_add(P, Rr));
  LAT(11, n, s = fr_mul(s, sk));
  LAT(12, n / 4, P = g1_dbl_inl(P));
  LAT(13, n / 4, P = g1_add_aff_inl(P, Q));
  LAT(14, n, x2 = fp2_mul_inl(x2, k2));
  LAT(15, n / 64, _Pragma("unroll 1") for (int q = 0; q < 64; q++) b = fp_sqr(b));
  LAT(16, n, a = fp_mul_inl(a, k));
  LAT(17, n, a = fp_mul_inl(a, k); b = fp_mul_inl(b, k); c = fp_mul_inl(c, k));
  LAT(18, n, a = fp_mul_call(a, k));
  LAT(19, n, a = fp_mul_call(a, k); b = fp_mul_call(b, k); c = fp_mul_call(c, k));
  LAT(20, n, a = fp_mul_rolled(a, k));
  LAT(21, n, a = fp_mul_rolled(a, k); b = fp_mul_rolled(b, k); c = fp_mul_rolled(c, k));
  LAT(22, n / 4, P = g1_dbl_call(P));
  LAT(23, n / 4, P = g1_dbl_rolled(P));
  LAT(24, n, a = fp_mul_cios(a, k));
  LAT(25, n, a = fp_mul_cios(a, k); b = fp_mul_cios(b, k); c = fp_mul_cios(c, k));
  LAT(26, n, a = fp_mul_cios_inl(a, k));
  LAT(27, n / 4, P = g1_dbl_cios(P));
  LAT(28, n / 64, a = fp_inv_vartime(a));
#undef LAT
  if (threadIdx.x == 0)
    for (int i = 0; i < R; i++) cyc[i] = res[i];
  fp acc = fp_add(fp_add(a, b), fp_add(c, x2.c0));
  acc = fp_add(acc, fp_add(f.c0.c0.c0, P.X));
  acc.w[0] ^= s.w[0];
  sink[threadIdx.x] = acc;
}

// Fills cycles[0..cap) with the per-operation latencies of k_latency_probe;
// returns how many were written.
extern "C" int32_t cubbs_bbs_gpu_latency_probe_for_test_v2(double *cycles, int32_t cap) {
  if (!cycles || cap < 29) return -1;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    double *d = rt.arena.alloc<double>(29);
    fp *sink = rt.arena.alloc<fp>(32);
    k_latency_probe<<<1, 32, 0, rt.stream>>>(d, sink, 64);  // warm-up
    k_latency_probe<<<1, 32, 0, rt.stream>>>(d, sink, 512);
    CUBBS_CHECK(cudaGetLastError());
    CUBBS_CHECK(cudaMemcpyAsync(cycles, d, 29 * sizeof(double), cudaMemcpyDeviceToHost, rt.stream));
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    return 29;
  } catch (const CudaError &) {
    return -2;
  }
}

// Fp products per second (1e9) of the carry-save product (fp_mul) and the
// CIOS product with `wps[k]` warps per SM (blocks of 32 threads,
// sm_count * wps[k] blocks): rates[2k] carry-save, rates[2k + 1] CIOS.
extern "C" int32_t cubbs_bbs_gpu_fpmul_rates_for_test_v2(const int32_t *wps, int32_t n, double *rates) {
  if (!wps || !rates || n <= 0 || n > 8) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (int k = 0; k < n; k++)
    if (wps[k] < 1 || wps[k] > 64) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    fp *of = rt.arena.alloc<fp>(1);
    cudaEvent_t e0, e1;
    CUBBS_CHECK(cudaEventCreate(&e0));
    CUBBS_CHECK(cudaEventCreate(&e1));
    const uint32_t iters = 128;
    for (int k = 0; k < n; k++) {
      const int blocks = rt.sm_count * wps[k];
      for (int v = 0; v < 2; v++) {
        for (int rep = 0; rep < 2; rep++) {  // the first run is a warm-up
          CUBBS_CHECK(cudaEventRecord(e0, rt.stream));
          if (v == 0) k_fpmul_rate<<<blocks, 32, 0, rt.stream>>>(of, iters);
          else k_fpmul_cios_rate<<<blocks, 32, 0, rt.stream>>>(of, iters);
          CUBBS_CHECK(cudaEventRecord(e1, rt.stream));
          CUBBS_CHECK(cudaEventSynchronize(e1));
        }
        float ms = 0;
        CUBBS_CHECK(cudaEventElapsedTime(&ms, e0, e1));
        rates[2 * k + v] = (double)blocks * 32 * iters * 4 / (ms * 1e-3) / 1e9;
      }
    }
    CUBBS_CHECK(cudaGetLastError());
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// Returns the measured IMAD rate (1e12 multiply-adds per second) and the Fp
// Montgomery product rate (1e9 products per second) on the current device.
extern "C" int32_t cubbs_bbs_gpu_int_peaks_v2(double *tera_imad, double *giga_fpmul) {
  if (!tera_imad || !giga_fpmul) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    uint32_t *o = rt.arena.alloc<uint32_t>(4);
    fp *of = rt.arena.alloc<fp>(1);
    int blocks = rt.sm_count * 8;
    cudaEvent_t e0, e1;
    CUBBS_CHECK(cudaEventCreate(&e0));
    CUBBS_CHECK(cudaEventCreate(&e1));
    const uint32_t iters = 4096;
    k_imad_peak<<<blocks, 256, 0, rt.stream>>>(o, 64, 1);  // warm-up
    CUBBS_CHECK(cudaEventRecord(e0, rt.stream));
    k_imad_peak<<<blocks, 256, 0, rt.stream>>>(o, iters, 2);
    CUBBS_CHECK(cudaEventRecord(e1, rt.stream));
    CUBBS_CHECK(cudaEventSynchronize(e1));
    float ms = 0;
    CUBBS_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    *tera_imad = (double)blocks * 256 * iters * 8 * 16 / (ms * 1e-3) / 1e12;
    const uint32_t fiters = 256;
    k_fpmul_rate<<<blocks, 256, 0, rt.stream>>>(of, 8);
    CUBBS_CHECK(cudaEventRecord(e0, rt.stream));
    k_fpmul_rate<<<blocks, 256, 0, rt.stream>>>(of, fiters);
    CUBBS_CHECK(cudaEventRecord(e1, rt.stream));
    CUBBS_CHECK(cudaEventSynchronize(e1));
    CUBBS_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    *giga_fpmul = (double)blocks * 256 * fiters * 4 / (ms * 1e-3) / 1e9;
    CUBBS_CHECK(cudaGetLastError());
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}
