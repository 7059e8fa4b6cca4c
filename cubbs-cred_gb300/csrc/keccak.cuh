// SHAKE-256 (FIPS 202) and expand_message_xof (RFC 9380 5.3.2, k = 128) on
// sm_103a, one message per thread: the expander of the BLS12-381-SHAKE-256
// ciphersuite (crates/cubbs-bbs-protocol/src/bbsplus/ciphersuites.rs:49-63,
// ExpandMsgXof<Shake256>).
//
// The sponge state is 25 64-bit lanes (lane x + 5 y holds bytes 8 (x + 5 y) ..
// of the state, little-endian).  Bytes are gathered into a 136-byte rate block
// and XORed into the state a block at a time, so the permutation indexes the
// state with constants only.  The round constants and the rho offsets are
// computed at compile time from FIPS 202's definitions (rc(t) LFSR,
// Algorithm 5; the (x, y) -> (y, 2x + 3y) walk, Algorithm 2).
#pragma once
#include <stdint.h>

#include "field.cuh"

__host__ __device__ constexpr bool keccak_rc_bit(int t) {
  if (t % 255 == 0) return true;
  uint32_t r = 0x80;  // R[0] is bit 7 of the byte
  for (int i = 1; i <= t % 255; i++) {
    const uint32_t r8 = r & 1;
    r >>= 1;
    if (r8) r ^= 0x80 | 0x08 | 0x04 | 0x02;  // R[0], R[4], R[5], R[6] ^= R[8]
  }
  return (r & 0x80) != 0;
}
// rho offset of lane (x, y): ((t + 1)(t + 2) / 2) mod 64 where step t of the
// walk from (1, 0) reaches (x, y); 0 for (0, 0)
__host__ __device__ constexpr int keccak_rot(int x, int y) {
  int cx = 1, cy = 0;
  for (int t = 0; t < 24; t++) {
    if (cx == x && cy == y) return ((t + 1) * (t + 2) / 2) % 64;
    const int nx = cy, ny = (2 * cx + 3 * cy) % 5;
    cx = nx;
    cy = ny;
  }
  return 0;
}
struct KeccakRoundConstants {
  uint64_t rc[24];
  constexpr KeccakRoundConstants() : rc() {
    for (int ir = 0; ir < 24; ir++) {
      uint64_t v = 0;
      for (int j = 0; j <= 6; j++)
        if (keccak_rc_bit(j + 7 * ir)) v |= 1ull << ((1 << j) - 1);
      rc[ir] = v;
    }
  }
};
__device__ __constant__ static const KeccakRoundConstants KECCAK_RC = KeccakRoundConstants();
static_assert(KeccakRoundConstants().rc[1] == 0x8082ull && keccak_rot(1, 0) == 1 && keccak_rot(0, 1) == 36,
              "Keccak constants");

DEV uint64_t keccak_rol(uint64_t v, int n) { return n ? (v << n) | (v >> (64 - n)) : v; }

DEVNI void keccak_f1600(uint64_t a[25]) {
#pragma unroll 1
  for (int ir = 0; ir < 24; ir++) {
    uint64_t c[5], b[25];
#pragma unroll
    for (int x = 0; x < 5; x++) c[x] = a[x] ^ a[x + 5] ^ a[x + 10] ^ a[x + 15] ^ a[x + 20];
#pragma unroll
    for (int x = 0; x < 5; x++) {
      const uint64_t d = c[(x + 4) % 5] ^ keccak_rol(c[(x + 1) % 5], 1);
#pragma unroll
      for (int y = 0; y < 5; y++) a[x + 5 * y] ^= d;
    }
    // rho and pi: B[y, 2x + 3y] = rot(A[x, y], r[x, y])
#pragma unroll
    for (int x = 0; x < 5; x++)
#pragma unroll
      for (int y = 0; y < 5; y++) b[y + 5 * ((2 * x + 3 * y) % 5)] = keccak_rol(a[x + 5 * y], keccak_rot(x, y));
#pragma unroll
    for (int y = 0; y < 5; y++)
#pragma unroll
      for (int x = 0; x < 5; x++)
        a[x + 5 * y] = b[x + 5 * y] ^ (~b[(x + 1) % 5 + 5 * y] & b[(x + 2) % 5 + 5 * y]);
    a[0] ^= KECCAK_RC.rc[ir];
  }
}

constexpr uint32_t SHAKE256_RATE = 136;

struct shake_ctx {
  uint64_t a[25];
  uint64_t blk[17];  // the rate block being gathered
  uint32_t fill;     // bytes in blk (absorbing) or bytes used of the current output block (squeezing)
  uint32_t total;
};

DEV void shake_init(shake_ctx &c) {
#pragma unroll
  for (int i = 0; i < 25; i++) c.a[i] = 0;
#pragma unroll
  for (int i = 0; i < 17; i++) c.blk[i] = 0;
  c.fill = 0;
  c.total = 0;
}
DEV void shake_absorb_block(shake_ctx &c) {
#pragma unroll
  for (int i = 0; i < 17; i++) {
    c.a[i] ^= c.blk[i];
    c.blk[i] = 0;
  }
  keccak_f1600(c.a);
  c.fill = 0;
}
DEV void shake_byte(shake_ctx &c, uint8_t b) {
  c.blk[c.fill >> 3] |= (uint64_t)b << (8 * (c.fill & 7));
  c.fill++;
  c.total++;
  if (c.fill == SHAKE256_RATE) shake_absorb_block(c);
}
DEV void shake_bytes(shake_ctx &c, const uint8_t *p, uint32_t n) {
  uint32_t i = 0;
#pragma unroll 1
  for (; i < n && (c.fill & 7); i++) shake_byte(c, p[i]);
  // whole 8-byte words while the block position is word-aligned
#pragma unroll 1
  while (i + 8 <= n) {
    uint64_t w = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) w |= (uint64_t)p[i + k] << (8 * k);
    c.blk[c.fill >> 3] = w;
    c.fill += 8;
    c.total += 8;
    i += 8;
    if (c.fill == SHAKE256_RATE) shake_absorb_block(c);
  }
#pragma unroll 1
  for (; i < n; i++) shake_byte(c, p[i]);
}
// Pads (0x1F ... 0x80), permutes and starts squeezing.
DEV void shake_pad(shake_ctx &c) {
  c.blk[c.fill >> 3] ^= (uint64_t)0x1F << (8 * (c.fill & 7));
  c.blk[16] ^= (uint64_t)0x80 << 56;
  shake_absorb_block(c);  // fill = 0: no output byte used yet
}
DEV void shake_squeeze(shake_ctx &c, uint8_t *out, uint32_t n) {
#pragma unroll 1
  for (uint32_t k = 0; k < n; k++) {
    if (c.fill == SHAKE256_RATE) {
      keccak_f1600(c.a);
      c.fill = 0;
    }
    uint64_t lane = 0;
#pragma unroll
    for (int q = 0; q < 17; q++)
      if (q == (int)(c.fill >> 3)) lane = c.a[q];
    out[k] = (uint8_t)(lane >> (8 * (c.fill & 7)));
    c.fill++;
  }
}

// expand_message_xof: msg_prime = msg || I2OSP(n, 2) || DST || I2OSP(len(DST), 1);
// the caller absorbs msg after xof_begin.  xof_start_output absorbs the rest and
// pads; the n output bytes then come from shake_squeeze (in pieces if wanted).
DEV void xof_begin(shake_ctx &c) { shake_init(c); }
DEV void xof_start_output(shake_ctx &c, const uint8_t *dst, uint32_t dlen, uint32_t n) {
  shake_byte(c, (uint8_t)(n >> 8));
  shake_byte(c, (uint8_t)n);
  shake_bytes(c, dst, dlen);
  shake_byte(c, (uint8_t)dlen);
  shake_pad(c);
}
DEV void xof_finish(shake_ctx &c, const uint8_t *dst, uint32_t dlen, uint32_t n, uint8_t *out) {
  xof_start_output(c, dst, dlen, n);
  shake_squeeze(c, out, n);
}

// The suite-generic names used by the kernels (the SHA-256 forms are in sha256.cuh).
DEV void msg_begin(shake_ctx &c) { xof_begin(c); }
DEV void msg_byte(shake_ctx &c, uint8_t b) { shake_byte(c, b); }
DEV void msg_bytes(shake_ctx &c, const uint8_t *p, uint32_t n) { shake_bytes(c, p, n); }
DEV void msg_u64be(shake_ctx &c, uint64_t x, int nbytes) {
#pragma unroll 1
  for (int i = nbytes - 1; i >= 0; i--) shake_byte(c, (uint8_t)(x >> (8 * i)));
}
DEV void msg_finish(shake_ctx &c, const uint8_t *dst, uint32_t dlen, uint32_t n, uint8_t *out) {
  xof_finish(c, dst, dlen, n, out);
}
DEV fr h2s_finish(shake_ctx &c, const uint8_t *dst, uint32_t dlen) {
  uint8_t okm[48];
  xof_finish(c, dst, dlen, 48, okm);
  return fr_raw_from_okm(okm);
}

