// SHA-256 (FIPS 180-4), expand_message_xmd (RFC 9380 5.3.1, b = 32, s = 64)
// and BBS hash_to_scalar on sm_103a, one message per thread.
// Reference kernels: native/cuda/src/sha256.cuh:26-364 (xmd :242-272,
// bit-serial mod-r reduction :317-364; here the 384-bit OKM is reduced with
// two Montgomery products, fr_raw_from_okm).
#pragma once
#include "field.cuh"

__device__ __constant__ static const uint32_t SHA256_K[64] = {
    0x428a2f98u, 0x71374491u, 0xb5c0fbcfu, 0xe9b5dba5u, 0x3956c25bu, 0x59f111f1u, 0x923f82a4u,
    0xab1c5ed5u, 0xd807aa98u, 0x12835b01u, 0x243185beu, 0x550c7dc3u, 0x72be5d74u, 0x80deb1feu,
    0x9bdc06a7u, 0xc19bf174u, 0xe49b69c1u, 0xefbe4786u, 0x0fc19dc6u, 0x240ca1ccu, 0x2de92c6fu,
    0x4a7484aau, 0x5cb0a9dcu, 0x76f988dau, 0x983e5152u, 0xa831c66du, 0xb00327c8u, 0xbf597fc7u,
    0xc6e00bf3u, 0xd5a79147u, 0x06ca6351u, 0x14292967u, 0x27b70a85u, 0x2e1b2138u, 0x4d2c6dfcu,
    0x53380d13u, 0x650a7354u, 0x766a0abbu, 0x81c2c92eu, 0x92722c85u, 0xa2bfe8a1u, 0xa81a664bu,
    0xc24b8b70u, 0xc76c51a3u, 0xd192e819u, 0xd6990624u, 0xf40e3585u, 0x106aa070u, 0x19a4c116u,
    0x1e376c08u, 0x2748774cu, 0x34b0bcb5u, 0x391c0cb3u, 0x4ed8aa4au, 0x5b9cca4fu, 0x682e6ff3u,
    0x748f82eeu, 0x78a5636fu, 0x84c87814u, 0x8cc70208u, 0x90befffau, 0xa4506cebu, 0xbef9a3f7u,
    0xc67178f2u};

DEV uint32_t sha_rotr(uint32_t x, int n) { return __funnelshift_r(x, x, n); }

DEVNI void sha256_compress(uint32_t h[8], uint32_t w[16]) {
  uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
#pragma unroll
  for (int i = 0; i < 64; i++) {
    uint32_t wi;
    if (i < 16) {
      wi = w[i];
    } else {
      uint32_t w15 = w[(i - 15) & 15], w2 = w[(i - 2) & 15];
      uint32_t s0 = sha_rotr(w15, 7) ^ sha_rotr(w15, 18) ^ (w15 >> 3);
      uint32_t s1 = sha_rotr(w2, 17) ^ sha_rotr(w2, 19) ^ (w2 >> 10);
      wi = w[i & 15] + s0 + w[(i - 7) & 15] + s1;
      w[i & 15] = wi;
    }
    uint32_t S1 = sha_rotr(e, 6) ^ sha_rotr(e, 11) ^ sha_rotr(e, 25);
    uint32_t ch = (e & f) ^ (~e & g);
    uint32_t t1 = hh + S1 + ch + SHA256_K[i] + wi;
    uint32_t S0 = sha_rotr(a, 2) ^ sha_rotr(a, 13) ^ sha_rotr(a, 22);
    uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
    hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + S0 + mj;
  }
  h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
}

struct sha_ctx {
  uint32_t h[8];
  uint32_t w[16];
  uint32_t fill;    // bytes in the current block
  uint32_t total;   // total bytes absorbed (< 2^32 here)
};

DEV void sha_init(sha_ctx &c) {
  c.h[0] = 0x6a09e667u; c.h[1] = 0xbb67ae85u; c.h[2] = 0x3c6ef372u; c.h[3] = 0xa54ff53au;
  c.h[4] = 0x510e527fu; c.h[5] = 0x9b05688cu; c.h[6] = 0x1f83d9abu; c.h[7] = 0x5be0cd19u;
  for (int i = 0; i < 16; i++) c.w[i] = 0;
  c.fill = 0;
  c.total = 0;
}
DEV void sha_byte(sha_ctx &c, uint8_t b) {
  c.w[c.fill >> 2] |= (uint32_t)b << (24 - 8 * (c.fill & 3));
  c.fill++;
  c.total++;
  if (c.fill == 64) {
    sha256_compress(c.h, c.w);
    for (int i = 0; i < 16; i++) c.w[i] = 0;
    c.fill = 0;
  }
}
DEV void sha_bytes(sha_ctx &c, const uint8_t *p, uint32_t n) {
  // word-at-a-time when the block position is 4-aligned (bytes are assembled
  // individually: the source may be a byte array just written by this thread)
  uint32_t i = 0;
  if ((c.fill & 3) == 0) {
#pragma unroll 1
    while (i + 4 <= n) {
      c.w[c.fill >> 2] = ((uint32_t)p[i] << 24) | ((uint32_t)p[i + 1] << 16) | ((uint32_t)p[i + 2] << 8) | p[i + 3];
      c.fill += 4;
      c.total += 4;
      i += 4;
      if (c.fill == 64) {
        sha256_compress(c.h, c.w);
        for (int k = 0; k < 16; k++) c.w[k] = 0;
        c.fill = 0;
      }
    }
  }
#pragma unroll 1
  for (; i < n; i++) sha_byte(c, p[i]);
}
DEV void sha_u64be(sha_ctx &c, uint64_t x, int nbytes) {
  #pragma unroll 1
  for (int i = nbytes - 1; i >= 0; i--) sha_byte(c, (uint8_t)(x >> (8 * i)));
}
DEV void sha_final(sha_ctx &c, uint8_t out[32]) {
  uint64_t bits = (uint64_t)c.total * 8;
  sha_byte(c, 0x80);
  while (c.fill != 56) sha_byte(c, 0);
  c.w[14] = (uint32_t)(bits >> 32);
  c.w[15] = (uint32_t)bits;
  sha256_compress(c.h, c.w);
  for (int i = 0; i < 8; i++) {
    out[4 * i] = (uint8_t)(c.h[i] >> 24); out[4 * i + 1] = (uint8_t)(c.h[i] >> 16);
    out[4 * i + 2] = (uint8_t)(c.h[i] >> 8); out[4 * i + 3] = (uint8_t)c.h[i];
  }
}

// expand_message_xmd: the caller absorbs msg into ctx after xmd_begin().
DEV void xmd_begin(sha_ctx &c) {
  sha_init(c);
  // Z_pad: one all-zero 64-byte block (the compression overwrites w with the
  // message schedule, so clear it again)
  sha256_compress(c.h, c.w);
  for (int i = 0; i < 16; i++) c.w[i] = 0;
  c.total = 64;
}
// Finishes b_0 and writes n output bytes (n <= 255*32).
DEV void xmd_finish(sha_ctx &c, const uint8_t *dst, uint32_t dlen, uint32_t n, uint8_t *out) {
  sha_byte(c, (uint8_t)(n >> 8));
  sha_byte(c, (uint8_t)n);
  sha_byte(c, 0);
  sha_bytes(c, dst, dlen);
  sha_byte(c, (uint8_t)dlen);
  uint8_t b0[32], bi[32];
  sha_final(c, b0);
  uint32_t ell = (n + 31) / 32;
  #pragma unroll 1
  for (uint32_t i = 1; i <= ell; i++) {
    sha_ctx s;
    sha_init(s);
    for (int j = 0; j < 32; j++) sha_byte(s, i == 1 ? b0[j] : (uint8_t)(b0[j] ^ bi[j]));
    sha_byte(s, (uint8_t)i);
    sha_bytes(s, dst, dlen);
    sha_byte(s, (uint8_t)dlen);
    sha_final(s, bi);
    uint32_t off = (i - 1) * 32;
    #pragma unroll 1
    for (uint32_t j = 0; j < 32 && off + j < n; j++) out[off + j] = bi[j];
  }
}
// hash_to_scalar (util.rs:104-129): OS2IP(expand_message_xmd(msg, dst, 48)) mod r,
// returned as the canonical raw residue.
DEV fr h2s_finish(sha_ctx &c, const uint8_t *dst, uint32_t dlen) {
  uint8_t okm[48];
  xmd_finish(c, dst, dlen, 48, okm);
  return fr_raw_from_okm(okm);
}

// The suite-generic names used by the kernels (the SHAKE-256 forms are in keccak.cuh).
DEV void msg_begin(sha_ctx &c) { xmd_begin(c); }
DEV void msg_byte(sha_ctx &c, uint8_t b) { sha_byte(c, b); }
DEV void msg_bytes(sha_ctx &c, const uint8_t *p, uint32_t n) { sha_bytes(c, p, n); }
DEV void msg_u64be(sha_ctx &c, uint64_t x, int nbytes) { sha_u64be(c, x, nbytes); }
DEV void msg_finish(sha_ctx &c, const uint8_t *dst, uint32_t dlen, uint32_t n, uint8_t *out) {
  xmd_finish(c, dst, dlen, n, out);
}
