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

// op 0: Fp product of canonical BE inputs; op 1: Fp inverse; op 2: Fp sqrt (0 if none)
__global__ void k_fp_test(const uint8_t *a, const uint8_t *b, uint32_t n, int op, uint8_t *out, int32_t *st) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fp x, y, r = fp_zero();
  bool ok = fp_from_be48(a + 48 * (size_t)i, x) && fp_from_be48(b + 48 * (size_t)i, y);
  if (ok) {
    if (op == 0) r = fp_mul(x, y);
    else if (op == 1) r = fp_inv(x);
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
    Runtime &rt = Runtime::get();
    CallScope scope(rt);
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

// op: 0 mul, 1 inverse, 2 sqrt.  Inputs and outputs are 48-byte big-endian canonical.
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

// Returns the measured IMAD rate (1e12 multiply-adds per second) and the Fp
// Montgomery product rate (1e9 products per second) on the current device.
extern "C" int32_t cubbs_bbs_gpu_int_peaks_v2(double *tera_imad, double *giga_fpmul) {
  if (!tera_imad || !giga_fpmul) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    Runtime &rt = Runtime::get();
    CallScope scope(rt);
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
