// CPU oracle for the BBS BLS12-381-SHA-256 hot path.  TEST INFRASTRUCTURE:
// loaded only by tests/, the smoke entry and the CPU-baseline leg of bench.py,
// always as the checker.  The GPU library never links or calls this file.
//
// Restates, in portable C++17 (6x64-bit limb Montgomery arithmetic, no
// platform intrinsics), the reference protocol crate:
//   crates/cubbs-bbs-protocol/src/bbsplus/ciphersuites.rs:21-79  (DSTs, P1)
//   crates/cubbs-bbs-protocol/src/utils/util.rs:78-189           (i2osp, hash_to_scalar, calculate_domain)
//   crates/cubbs-bbs-protocol/src/utils/util.rs:329-358          (seeded_random_scalars)
//   crates/cubbs-bbs-protocol/src/utils/message.rs:54-62         (messages_to_scalar)
//   crates/cubbs-bbs-protocol/src/bbsplus/generators.rs:71-146   (create_generators)
//   crates/cubbs-bbs-protocol/src/bbsplus/keys.rs:214-261        (KeyGen, SkToPk)
//   crates/cubbs-bbs-protocol/src/bbsplus/signature.rs:544-728   (core_sign, core_verify)
//   crates/cubbs-bbs-protocol/src/bbsplus/proof.rs:173-225,1568-1867,2155-2426,3015-3078
// and the third-party arithmetic it calls (bls12_381_plus 0.8.18 field/curve/
// pairing and point encodings; elliptic-curve 0.13.8 ExpandMsgXmd and
// ExpandMsgXof; sha2 0.10.9; sha3 SHAKE-256; RFC 9380
// BLS12381G1_XMD:SHA-256_SSWU_RO_ and BLS12381G1_XOF:SHAKE-256_SSWU_RO_).
// Both ciphersuites of ciphersuites.rs:49-79 are restated: the suite of the
// calling thread (oracle_set_suite) selects API_ID, P1 and the expander.
// Parity is pinned by the CFRG fixtures of both suites.
#include "bbs_oracle.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

typedef uint64_t u64;
typedef unsigned __int128 u128;
typedef std::vector<uint8_t> Bytes;

// ============================================================ SHA-256 (FIPS 180-4)
namespace {
const uint32_t SHA_K[64] = {
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
const uint32_t SHA_H0[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                            0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};

inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

struct Sha256 {
  uint32_t h[8];
  uint8_t buf[64];
  size_t buf_len = 0;
  uint64_t total = 0;
  Sha256() { std::memcpy(h, SHA_H0, sizeof h); }
  void block(const uint8_t *p) {
    uint32_t w[64];
    for (int i = 0; i < 16; i++)
      w[i] = (uint32_t)p[4 * i] << 24 | (uint32_t)p[4 * i + 1] << 16 |
             (uint32_t)p[4 * i + 2] << 8 | p[4 * i + 3];
    for (int i = 16; i < 64; i++) {
      uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
      uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
      w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
    for (int i = 0; i < 64; i++) {
      uint32_t S1 = rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
      uint32_t ch = (e & f) ^ (~e & g);
      uint32_t t1 = hh + S1 + ch + SHA_K[i] + w[i];
      uint32_t S0 = rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
      uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
      uint32_t t2 = S0 + mj;
      hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
  }
  void update(const uint8_t *p, size_t n) {
    total += n;
    while (n > 0) {
      size_t take = std::min(n, (size_t)64 - buf_len);
      std::memcpy(buf + buf_len, p, take);
      buf_len += take; p += take; n -= take;
      if (buf_len == 64) { block(buf); buf_len = 0; }
    }
  }
  void update(const Bytes &b) { if (!b.empty()) update(b.data(), b.size()); }
  void final(uint8_t out[32]) {
    uint64_t bits = total * 8;
    uint8_t pad = 0x80;
    update(&pad, 1);
    uint8_t z = 0;
    while (buf_len != 56) update(&z, 1);
    uint8_t len[8];
    for (int i = 0; i < 8; i++) len[i] = (uint8_t)(bits >> (56 - 8 * i));
    update(len, 8);
    for (int i = 0; i < 8; i++) {
      out[4 * i] = (uint8_t)(h[i] >> 24); out[4 * i + 1] = (uint8_t)(h[i] >> 16);
      out[4 * i + 2] = (uint8_t)(h[i] >> 8); out[4 * i + 3] = (uint8_t)h[i];
    }
  }
};

// RFC 9380 section 5.3.1 expand_message_xmd with SHA-256 (b=32, s=64).
bool expand_xmd(const uint8_t *msg, size_t len, const uint8_t *dst, size_t dlen, uint8_t *out,
                size_t n) {
  if (dlen > 255 || n == 0 || n > 255 * 32 || n > 65535) return false;
  size_t ell = (n + 31) / 32;
  uint8_t dl = (uint8_t)dlen;
  uint8_t zpad[64] = {0};
  uint8_t lib[3] = {(uint8_t)(n >> 8), (uint8_t)n, 0};
  uint8_t b0[32], bi[32];
  Sha256 s0;
  s0.update(zpad, 64);
  if (len) s0.update(msg, len);
  s0.update(lib, 3);
  if (dlen) s0.update(dst, dlen);
  s0.update(&dl, 1);
  s0.final(b0);
  for (size_t i = 1; i <= ell; i++) {
    uint8_t x[32];
    for (int j = 0; j < 32; j++) x[j] = (i == 1) ? b0[j] : (uint8_t)(b0[j] ^ bi[j]);
    uint8_t ib = (uint8_t)i;
    Sha256 s;
    s.update(x, 32);
    s.update(&ib, 1);
    if (dlen) s.update(dst, dlen);
    s.update(&dl, 1);
    s.final(bi);
    size_t off = (i - 1) * 32;
    std::memcpy(out + off, bi, std::min((size_t)32, n - off));
  }
  return true;
}

// ============================================================ SHAKE-256 (FIPS 202)
// Keccak-f[1600] on 25 64-bit lanes (state index x + 5 y), 24 rounds; the
// round constants are those of FIPS 202 section 3.2.5, computed here from its
// rc(t) LFSR rather than tabulated.
struct Keccak {
  uint64_t a[25];
  static uint64_t rol(uint64_t x, int n) { return n ? (x << n) | (x >> (64 - n)) : x; }
  static bool rc_bit(int t) {  // FIPS 202 Algorithm 5
    if (t % 255 == 0) return true;
    uint32_t r = 0x80;  // bits R[0..7], R[0] the most significant of the byte
    for (int i = 1; i <= t % 255; i++) {
      uint32_t r8 = r & 1;  // R[7] before the shift
      r >>= 1;
      if (r8) r ^= 0x80 | 0x08 | 0x04 | 0x02;  // R[0], R[4], R[5], R[6] ^= R[8]
    }
    return (r & 0x80) != 0;
  }
  static uint64_t round_constant(int ir) {
    uint64_t rc = 0;
    for (int j = 0; j <= 6; j++)
      if (rc_bit(j + 7 * ir)) rc |= 1ull << ((1 << j) - 1);
    return rc;
  }
  void permute() {
    static uint64_t RC[24];
    static int ROT[25];
    static std::once_flag once;
    std::call_once(once, [] {
      for (int i = 0; i < 24; i++) RC[i] = round_constant(i);
      // rho offsets (FIPS 202 Algorithm 2): walk (x, y) -> (y, 2x + 3y)
      ROT[0] = 0;
      int x = 1, y = 0;
      for (int t = 0; t < 24; t++) {
        ROT[x + 5 * y] = ((t + 1) * (t + 2) / 2) % 64;
        int nx = y, ny = (2 * x + 3 * y) % 5;
        x = nx;
        y = ny;
      }
    });
    for (int ir = 0; ir < 24; ir++) {
      uint64_t c[5], d[5], b[25];
      for (int x = 0; x < 5; x++) c[x] = a[x] ^ a[x + 5] ^ a[x + 10] ^ a[x + 15] ^ a[x + 20];
      for (int x = 0; x < 5; x++) d[x] = c[(x + 4) % 5] ^ rol(c[(x + 1) % 5], 1);
      for (int i = 0; i < 25; i++) a[i] ^= d[i % 5];
      // rho and pi: B[y, 2x + 3y] = rot(A[x, y])
      for (int x = 0; x < 5; x++)
        for (int y = 0; y < 5; y++) b[y + 5 * ((2 * x + 3 * y) % 5)] = rol(a[x + 5 * y], ROT[x + 5 * y]);
      for (int x = 0; x < 5; x++)
        for (int y = 0; y < 5; y++)
          a[x + 5 * y] = b[x + 5 * y] ^ (~b[(x + 1) % 5 + 5 * y] & b[(x + 2) % 5 + 5 * y]);
      a[0] ^= RC[ir];
    }
  }
};

// SHAKE-256: rate 136 bytes, domain padding 0x1F ... 0x80.
struct Shake256 {
  Keccak k;
  size_t pos = 0;
  Shake256() { std::memset(k.a, 0, sizeof k.a); }
  void xor_byte(size_t i, uint8_t b) { k.a[i / 8] ^= (uint64_t)b << (8 * (i % 8)); }
  void update(const uint8_t *p, size_t n) {
    for (size_t i = 0; i < n; i++) {
      xor_byte(pos++, p[i]);
      if (pos == 136) {
        k.permute();
        pos = 0;
      }
    }
  }
  void squeeze(uint8_t *out, size_t n) {
    xor_byte(pos, 0x1F);
    xor_byte(135, 0x80);
    k.permute();
    size_t off = 0;
    while (n) {
      size_t take = std::min(n, (size_t)136 - off);
      for (size_t i = 0; i < take; i++) *out++ = (uint8_t)(k.a[(off + i) / 8] >> (8 * ((off + i) % 8)));
      n -= take;
      off += take;
      if (off == 136 && n) {
        k.permute();
        off = 0;
      }
    }
  }
};

// RFC 9380 section 5.3.2 expand_message_xof with SHAKE-256 (k = 128):
// SHAKE256(msg || I2OSP(n, 2) || DST || I2OSP(len(DST), 1), n).
bool expand_xof(const uint8_t *msg, size_t len, const uint8_t *dst, size_t dlen, uint8_t *out, size_t n) {
  if (dlen > 255 || n == 0 || n > 65535) return false;
  Shake256 h;
  if (len) h.update(msg, len);
  uint8_t lib[2] = {(uint8_t)(n >> 8), (uint8_t)n};
  h.update(lib, 2);
  if (dlen) h.update(dst, dlen);
  uint8_t dl = (uint8_t)dlen;
  h.update(&dl, 1);
  h.squeeze(out, n);
  return true;
}

// Ciphersuite of the calling thread: 0 BLS12-381-SHA-256 (expand_message_xmd),
// 1 BLS12-381-SHAKE-256 (expand_message_xof).
thread_local int SUITE = 0;
bool expand_message(const uint8_t *msg, size_t len, const uint8_t *dst, size_t dlen, uint8_t *out, size_t n) {
  return SUITE == 1 ? expand_xof(msg, len, dst, dlen, out, n) : expand_xmd(msg, len, dst, dlen, out, n);
}

// ============================================================ Montgomery fields
template <int N> struct Modulus {
  u64 m[N];
  u64 inv;   // -m^{-1} mod 2^64
  u64 one[N];  // R mod m
  u64 r2[N];   // R^2 mod m
};

template <int N> inline bool geq(const u64 *a, const u64 *b) {
  for (int i = N - 1; i >= 0; i--) {
    if (a[i] != b[i]) return a[i] > b[i];
  }
  return true;
}
template <int N> inline u64 sub_n(u64 *out, const u64 *a, const u64 *b) {
  u64 borrow = 0;
  for (int i = 0; i < N; i++) {
    u128 x = (u128)a[i] - b[i] - borrow;
    out[i] = (u64)x;
    borrow = (u64)(x >> 64) & 1;
  }
  return borrow;
}
template <int N> inline u64 add_n(u64 *out, const u64 *a, const u64 *b) {
  u64 carry = 0;
  for (int i = 0; i < N; i++) {
    u128 x = (u128)a[i] + b[i] + carry;
    out[i] = (u64)x;
    carry = (u64)(x >> 64);
  }
  return carry;
}

template <int N> inline void mont_mul(u64 *out, const u64 *a, const u64 *b, const Modulus<N> &M) {
  u64 t[N + 2] = {0};
  for (int i = 0; i < N; i++) {
    u128 c = 0;
    for (int j = 0; j < N; j++) {
      c += (u128)a[j] * b[i] + t[j];
      t[j] = (u64)c;
      c >>= 64;
    }
    u128 s = (u128)t[N] + (u64)c;
    t[N] = (u64)s;
    t[N + 1] = (u64)(s >> 64);
    u64 q = t[0] * M.inv;
    c = (u128)q * M.m[0] + t[0];
    c >>= 64;
    for (int j = 1; j < N; j++) {
      c += (u128)q * M.m[j] + t[j];
      t[j - 1] = (u64)c;
      c >>= 64;
    }
    s = (u128)t[N] + (u64)c;
    t[N - 1] = (u64)s;
    t[N] = t[N + 1] + (u64)(s >> 64);
  }
  u64 d[N];
  u64 borrow = sub_n<N>(d, t, M.m);
  bool use_d = t[N] != 0 || borrow == 0;
  for (int j = 0; j < N; j++) out[j] = use_d ? d[j] : t[j];
}

template <int N> void init_modulus(Modulus<N> &M, const char *hex) {
  std::memset(&M, 0, sizeof M);
  // parse hex big-endian into little-endian limbs
  size_t len = std::strlen(hex);
  for (size_t i = 0; i < len; i++) {
    char ch = hex[len - 1 - i];
    u64 v = (ch >= '0' && ch <= '9') ? ch - '0' : (ch >= 'a' && ch <= 'f') ? ch - 'a' + 10 : ch - 'A' + 10;
    M.m[i / 16] |= v << (4 * (i % 16));
  }
  u64 inv = 1;  // Newton iteration for m^{-1} mod 2^64
  for (int i = 0; i < 6; i++) inv *= 2 - M.m[0] * inv;
  M.inv = (u64)0 - inv;
  // one = 2^(64N) mod m by repeated doubling of 1
  u64 x[N] = {1};
  for (int i = 0; i < 64 * N; i++) {
    u64 c = add_n<N>(x, x, x);
    if (c || geq<N>(x, M.m)) sub_n<N>(x, x, M.m);
  }
  std::memcpy(M.one, x, sizeof x);
  for (int i = 0; i < 64 * N; i++) {
    u64 c = add_n<N>(x, x, x);
    if (c || geq<N>(x, M.m)) sub_n<N>(x, x, M.m);
  }
  std::memcpy(M.r2, x, sizeof x);
}

Modulus<6> PM;  // base field p
Modulus<4> RM;  // scalar field r

const char *P_HEX =
    "1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab";
const char *R_HEX = "73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001";

struct Fp {
  u64 v[6];
  static Fp zero() { Fp r; std::memset(r.v, 0, sizeof r.v); return r; }
  static Fp one() { Fp r; std::memcpy(r.v, PM.one, sizeof r.v); return r; }
  bool is_zero() const { for (int i = 0; i < 6; i++) if (v[i]) return false; return true; }
  bool operator==(const Fp &o) const { return std::memcmp(v, o.v, sizeof v) == 0; }
  bool operator!=(const Fp &o) const { return !(*this == o); }
  Fp operator+(const Fp &o) const {
    Fp r; u64 c = add_n<6>(r.v, v, o.v);
    if (c || geq<6>(r.v, PM.m)) sub_n<6>(r.v, r.v, PM.m);
    return r;
  }
  Fp operator-(const Fp &o) const {
    Fp r; u64 b = sub_n<6>(r.v, v, o.v);
    if (b) add_n<6>(r.v, r.v, PM.m);
    return r;
  }
  Fp operator-() const { return zero() - *this; }
  Fp operator*(const Fp &o) const { Fp r; mont_mul<6>(r.v, v, o.v, PM); return r; }
  Fp sq() const { return *this * *this; }
  Fp dbl() const { return *this + *this; }
  // canonical (non-Montgomery) little-endian limbs
  void to_canon(u64 out[6]) const { u64 one[6] = {1}; mont_mul<6>(out, v, one, PM); }
  static Fp from_canon(const u64 in[6]) { Fp r; mont_mul<6>(r.v, in, PM.r2, PM); return r; }
  static Fp from_u64(u64 x) { u64 t[6] = {x}; return from_canon(t); }
  Fp pow(const u64 *e, int nlimbs) const {
    Fp r = one();
    for (int i = nlimbs * 64 - 1; i >= 0; i--) {
      r = r.sq();
      if ((e[i / 64] >> (i % 64)) & 1) r = r * *this;
    }
    return r;
  }
  Fp inv() const {  // Fermat
    u64 e[6]; std::memcpy(e, PM.m, sizeof e);
    u64 two[6] = {2}; sub_n<6>(e, e, two);
    return pow(e, 6);
  }
  bool sqrt(Fp &out) const {  // p = 3 mod 4
    u64 e[6]; std::memcpy(e, PM.m, sizeof e);
    u64 one_[6] = {1};
    add_n<6>(e, e, one_);
    for (int i = 0; i < 6; i++) e[i] = (e[i] >> 2) | (i < 5 ? e[i + 1] << 62 : 0);
    Fp s = pow(e, 6);
    if (s.sq() != *this) return false;
    out = s;
    return true;
  }
  bool lexicographically_largest() const {
    // canonical value > (p-1)/2
    u64 c[6]; to_canon(c);
    u64 h[6]; std::memcpy(h, PM.m, sizeof h);
    for (int i = 0; i < 6; i++) h[i] = (h[i] >> 1) | (i < 5 ? h[i + 1] << 63 : 0);  // (p-1)/2 since p odd
    // c > h  <=>  !(h >= c)
    return !geq<6>(h, c);
  }
  bool parity() const { u64 c[6]; to_canon(c); return c[0] & 1; }
  // 48-byte big-endian canonical; returns false if >= p
  static bool from_be48(const uint8_t *b, Fp &out) {
    u64 c[6];
    for (int i = 0; i < 6; i++) {
      u64 x = 0;
      for (int j = 0; j < 8; j++) x = (x << 8) | b[(5 - i) * 8 + j];
      c[i] = x;
    }
    if (geq<6>(c, PM.m)) return false;
    out = from_canon(c);
    return true;
  }
  void to_be48(uint8_t *b) const {
    u64 c[6]; to_canon(c);
    for (int i = 0; i < 6; i++)
      for (int j = 0; j < 8; j++) b[(5 - i) * 8 + j] = (uint8_t)(c[i] >> (56 - 8 * j));
  }
  // OS2IP(64 bytes) mod p
  static Fp from_be64_mod(const uint8_t *b) {
    u64 lo[6], hi[6] = {0};
    for (int i = 0; i < 6; i++) {
      u64 x = 0;
      for (int j = 0; j < 8; j++) x = (x << 8) | b[16 + (5 - i) * 8 + j];
      lo[i] = x;
    }
    for (int i = 0; i < 2; i++) {
      u64 x = 0;
      for (int j = 0; j < 8; j++) x = (x << 8) | b[(1 - i) * 8 + j];
      hi[i] = x;
    }
    while (geq<6>(lo, PM.m)) sub_n<6>(lo, lo, PM.m);
    // value = hi * 2^384 + lo ; hi*2^384 mod p = mont_mul(hi, R^2) (as a canonical number)
    u64 t[6]; mont_mul<6>(t, hi, PM.r2, PM);
    u64 s[6]; u64 c = add_n<6>(s, t, lo);
    if (c || geq<6>(s, PM.m)) sub_n<6>(s, s, PM.m);
    return from_canon(s);
  }
};

struct Fr {
  u64 v[4];
  static Fr zero() { Fr r; std::memset(r.v, 0, sizeof r.v); return r; }
  static Fr one() { Fr r; std::memcpy(r.v, RM.one, sizeof r.v); return r; }
  bool is_zero() const { return !(v[0] | v[1] | v[2] | v[3]); }
  bool operator==(const Fr &o) const { return std::memcmp(v, o.v, sizeof v) == 0; }
  bool operator!=(const Fr &o) const { return !(*this == o); }
  Fr operator+(const Fr &o) const {
    Fr r; u64 c = add_n<4>(r.v, v, o.v);
    if (c || geq<4>(r.v, RM.m)) sub_n<4>(r.v, r.v, RM.m);
    return r;
  }
  Fr operator-(const Fr &o) const {
    Fr r; u64 b = sub_n<4>(r.v, v, o.v);
    if (b) add_n<4>(r.v, r.v, RM.m);
    return r;
  }
  Fr operator*(const Fr &o) const { Fr r; mont_mul<4>(r.v, v, o.v, RM); return r; }
  void to_canon(u64 out[4]) const { u64 one[4] = {1}; mont_mul<4>(out, v, one, RM); }
  static Fr from_canon(const u64 in[4]) { Fr r; mont_mul<4>(r.v, in, RM.r2, RM); return r; }
  Fr inv() const {
    u64 e[4]; std::memcpy(e, RM.m, sizeof e);
    u64 two[4] = {2}; sub_n<4>(e, e, two);
    Fr r = one();
    for (int i = 255; i >= 0; i--) {
      r = r * r;
      if ((e[i / 64] >> (i % 64)) & 1) r = r * *this;
    }
    return r;
  }
  // canonical 32-byte big-endian; false if >= r (ScalarExt::from_bytes_be, util.rs:203-213)
  static bool from_be32(const uint8_t *b, Fr &out) {
    u64 c[4];
    for (int i = 0; i < 4; i++) {
      u64 x = 0;
      for (int j = 0; j < 8; j++) x = (x << 8) | b[(3 - i) * 8 + j];
      c[i] = x;
    }
    if (geq<4>(c, RM.m)) return false;
    out = from_canon(c);
    return true;
  }
  void to_be32(uint8_t *b) const {
    u64 c[4]; to_canon(c);
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 8; j++) b[(3 - i) * 8 + j] = (uint8_t)(c[i] >> (56 - 8 * j));
  }
  // OS2IP(48 bytes) mod r  (Scalar::from_okm)
  static Fr from_okm(const uint8_t *b) {
    u64 lo[4], hi[4] = {0};
    for (int i = 0; i < 4; i++) {
      u64 x = 0;
      for (int j = 0; j < 8; j++) x = (x << 8) | b[16 + (3 - i) * 8 + j];
      lo[i] = x;
    }
    for (int i = 0; i < 2; i++) {
      u64 x = 0;
      for (int j = 0; j < 8; j++) x = (x << 8) | b[(1 - i) * 8 + j];
      hi[i] = x;
    }
    while (geq<4>(lo, RM.m)) sub_n<4>(lo, lo, RM.m);
    u64 t[4]; mont_mul<4>(t, hi, RM.r2, RM);  // hi * 2^256 mod r
    u64 s[4]; u64 c = add_n<4>(s, t, lo);
    if (c || geq<4>(s, RM.m)) sub_n<4>(s, s, RM.m);
    return from_canon(s);
  }
};

// ============================================================ extension tower
struct Fp2 {
  Fp c0, c1;  // c0 + c1*u, u^2 = -1
  static Fp2 zero() { return {Fp::zero(), Fp::zero()}; }
  static Fp2 one() { return {Fp::one(), Fp::zero()}; }
  bool is_zero() const { return c0.is_zero() && c1.is_zero(); }
  bool operator==(const Fp2 &o) const { return c0 == o.c0 && c1 == o.c1; }
  bool operator!=(const Fp2 &o) const { return !(*this == o); }
  Fp2 operator+(const Fp2 &o) const { return {c0 + o.c0, c1 + o.c1}; }
  Fp2 operator-(const Fp2 &o) const { return {c0 - o.c0, c1 - o.c1}; }
  Fp2 operator-() const { return {-c0, -c1}; }
  Fp2 operator*(const Fp2 &o) const {
    Fp a = c0 * o.c0, b = c1 * o.c1;
    Fp c = (c0 + c1) * (o.c0 + o.c1);
    return {a - b, c - a - b};
  }
  Fp2 operator*(const Fp &s) const { return {c0 * s, c1 * s}; }
  Fp2 sq() const { return *this * *this; }
  Fp2 dbl() const { return *this + *this; }
  Fp2 conj() const { return {c0, -c1}; }
  Fp2 mul_xi() const { return {c0 - c1, c0 + c1}; }  // * (1 + u)
  Fp2 inv() const {
    Fp n = (c0.sq() + c1.sq()).inv();
    return {c0 * n, -(c1 * n)};
  }
  Fp2 pow(const u64 *e, int nlimbs) const {
    Fp2 r = one();
    for (int i = nlimbs * 64 - 1; i >= 0; i--) {
      r = r.sq();
      if ((e[i / 64] >> (i % 64)) & 1) r = r * *this;
    }
    return r;
  }
  bool sqrt(Fp2 &out) const {
    if (c1.is_zero()) {
      Fp s;
      if (c0.sqrt(s)) { out = {s, Fp::zero()}; return true; }
      if ((-c0).sqrt(s)) { out = {Fp::zero(), s}; return true; }
      return false;
    }
    Fp n = c0.sq() + c1.sq(), s;
    if (!n.sqrt(s)) return false;
    Fp half = Fp::from_u64(2).inv();
    Fp t = (c0 + s) * half, x0;
    if (!t.sqrt(x0)) {
      t = (c0 - s) * half;
      if (!t.sqrt(x0)) return false;
    }
    Fp x1 = c1 * (x0.dbl()).inv();
    Fp2 r = {x0, x1};
    if (r.sq() != *this) return false;
    out = r;
    return true;
  }
  bool lexicographically_largest() const {
    if (!c1.is_zero()) return c1.lexicographically_largest();
    return c0.lexicographically_largest();
  }
};

struct Fp6 {
  Fp2 c0, c1, c2;  // c0 + c1 v + c2 v^2, v^3 = xi
  static Fp6 zero() { return {Fp2::zero(), Fp2::zero(), Fp2::zero()}; }
  static Fp6 one() { return {Fp2::one(), Fp2::zero(), Fp2::zero()}; }
  bool operator==(const Fp6 &o) const { return c0 == o.c0 && c1 == o.c1 && c2 == o.c2; }
  Fp6 operator+(const Fp6 &o) const { return {c0 + o.c0, c1 + o.c1, c2 + o.c2}; }
  Fp6 operator-(const Fp6 &o) const { return {c0 - o.c0, c1 - o.c1, c2 - o.c2}; }
  Fp6 operator-() const { return {-c0, -c1, -c2}; }
  Fp6 operator*(const Fp6 &o) const {
    Fp2 a0 = c0 * o.c0, a1 = c1 * o.c1, a2 = c2 * o.c2;
    Fp2 t0 = ((c1 + c2) * (o.c1 + o.c2) - a1 - a2).mul_xi() + a0;
    Fp2 t1 = (c0 + c1) * (o.c0 + o.c1) - a0 - a1 + a2.mul_xi();
    Fp2 t2 = (c0 + c2) * (o.c0 + o.c2) - a0 - a2 + a1;
    return {t0, t1, t2};
  }
  Fp6 mul_v() const { return {c2.mul_xi(), c0, c1}; }
  Fp6 inv() const {
    Fp2 t0 = c0.sq() - (c1 * c2).mul_xi();
    Fp2 t1 = c2.sq().mul_xi() - c0 * c1;
    Fp2 t2 = c1.sq() - c0 * c2;
    Fp2 d = (c0 * t0 + (c2 * t1).mul_xi() + (c1 * t2).mul_xi()).inv();
    return {t0 * d, t1 * d, t2 * d};
  }
};

struct Fp12 {
  Fp6 c0, c1;  // c0 + c1 w, w^2 = v
  static Fp12 one() { return {Fp6::one(), Fp6::zero()}; }
  bool operator==(const Fp12 &o) const { return c0 == o.c0 && c1 == o.c1; }
  Fp12 operator*(const Fp12 &o) const {
    Fp6 a = c0 * o.c0, b = c1 * o.c1;
    Fp6 c = (c0 + c1) * (o.c0 + o.c1) - a - b;
    return {a + b.mul_v(), c};
  }
  Fp12 sq() const { return *this * *this; }
  Fp12 conj() const { return {c0, -c1}; }
  Fp12 inv() const {
    Fp6 t = (c0 * c0 - (c1 * c1).mul_v()).inv();
    return {c0 * t, -(c1 * t)};
  }
};

// Frobenius coefficients gamma_k = xi^{k(p-1)/6}, derived at init.
Fp2 FROB_GAMMA[6];

Fp12 frobenius(const Fp12 &a) {
  // basis w^k: c0 = (w^0, w^2, w^4), c1 = (w^1, w^3, w^5)
  Fp12 r;
  r.c0.c0 = a.c0.c0.conj() * FROB_GAMMA[0];
  r.c0.c1 = a.c0.c1.conj() * FROB_GAMMA[2];
  r.c0.c2 = a.c0.c2.conj() * FROB_GAMMA[4];
  r.c1.c0 = a.c1.c0.conj() * FROB_GAMMA[1];
  r.c1.c1 = a.c1.c1.conj() * FROB_GAMMA[3];
  r.c1.c2 = a.c1.c2.conj() * FROB_GAMMA[5];
  return r;
}

// ============================================================ curves
template <typename F> struct Jac {
  F X, Y, Z;  // x = X/Z^2, y = Y/Z^3 ; Z = 0 is infinity
};

template <typename F> struct CurveOps {
  static F B;
  static Jac<F> infinity() { return {F::one(), F::one(), F::zero()}; }
  static bool is_inf(const Jac<F> &p) { return p.Z.is_zero(); }
  static Jac<F> from_affine(const F &x, const F &y) { return {x, y, F::one()}; }
  static Jac<F> dbl(const Jac<F> &p) {
    if (is_inf(p)) return p;
    // dbl-2009-l (a = 0)
    F A = p.X.sq(), Bv = p.Y.sq(), C = Bv.sq();
    F D = ((p.X + Bv).sq() - A - C).dbl();
    F E = A.dbl() + A, Fv = E.sq();
    F X3 = Fv - D.dbl();
    F C8 = C.dbl().dbl().dbl();
    F Y3 = E * (D - X3) - C8;
    F Z3 = (p.Y * p.Z).dbl();
    return {X3, Y3, Z3};
  }
  static Jac<F> add(const Jac<F> &p, const Jac<F> &q) {
    if (is_inf(p)) return q;
    if (is_inf(q)) return p;
    // add-2007-bl
    F Z1Z1 = p.Z.sq(), Z2Z2 = q.Z.sq();
    F U1 = p.X * Z2Z2, U2 = q.X * Z1Z1;
    F S1 = p.Y * q.Z * Z2Z2, S2 = q.Y * p.Z * Z1Z1;
    if (U1 == U2) {
      if (S1 == S2) return dbl(p);
      return infinity();
    }
    F H = U2 - U1, I = H.dbl().sq(), J = H * I;
    F r = (S2 - S1).dbl();
    F V = U1 * I;
    F X3 = r.sq() - J - V.dbl();
    F Y3 = r * (V - X3) - (S1 * J).dbl();
    F Z3 = ((p.Z + q.Z).sq() - Z1Z1 - Z2Z2) * H;
    return {X3, Y3, Z3};
  }
  static Jac<F> neg(const Jac<F> &p) { return {p.X, -p.Y, p.Z}; }
  static void to_affine(const Jac<F> &p, F &x, F &y) {
    F zi = p.Z.inv(), zi2 = zi.sq();
    x = p.X * zi2;
    y = p.Y * zi2 * zi;
  }
  static bool eq(const Jac<F> &p, const Jac<F> &q) {
    if (is_inf(p) || is_inf(q)) return is_inf(p) && is_inf(q);
    F Z1Z1 = p.Z.sq(), Z2Z2 = q.Z.sq();
    return p.X * Z2Z2 == q.X * Z1Z1 && p.Y * q.Z * Z2Z2 == q.Y * p.Z * Z1Z1;
  }
  static Jac<F> mul_limbs(const Jac<F> &p, const u64 *k, int nlimbs) {
    Jac<F> r = infinity();
    for (int i = nlimbs * 64 - 1; i >= 0; i--) {
      r = dbl(r);
      if ((k[i / 64] >> (i % 64)) & 1) r = add(r, p);
    }
    return r;
  }
  static Jac<F> mul(const Jac<F> &p, const Fr &k) {
    u64 c[4]; k.to_canon(c);
    return mul_limbs(p, c, 4);
  }
  static bool on_curve_affine(const F &x, const F &y) { return y.sq() == x.sq() * x + B; }
  static bool in_subgroup(const Jac<F> &p) { return is_inf(mul_limbs(p, RM.m, 4)); }
};
template <> Fp CurveOps<Fp>::B = Fp();
template <> Fp2 CurveOps<Fp2>::B = Fp2();
typedef CurveOps<Fp> G1;
typedef CurveOps<Fp2> G2;
typedef Jac<Fp> G1P;
typedef Jac<Fp2> G2P;

G1P G1_GEN, P1_POINTS[2];
#define P1_POINT (P1_POINTS[SUITE])
G2P G2_GEN;

// --- encodings (bls12_381 zkcrypto format: flags in the top 3 bits of byte 0)
void g1_compress(const G1P &p, uint8_t out[48]) {
  if (G1::is_inf(p)) {
    std::memset(out, 0, 48);
    out[0] = 0xc0;
    return;
  }
  Fp x, y;
  G1::to_affine(p, x, y);
  x.to_be48(out);
  out[0] |= 0x80;
  if (y.lexicographically_largest()) out[0] |= 0x20;
}
// G1Affine::from_compressed: unchecked decode + torsion check.
bool g1_decompress(const uint8_t in[48], G1P &out, bool check_subgroup = true) {
  bool comp = in[0] & 0x80, inf = in[0] & 0x40, sort = in[0] & 0x20;
  uint8_t t[48];
  std::memcpy(t, in, 48);
  t[0] &= 0x1f;
  Fp x;
  if (!Fp::from_be48(t, x)) return false;
  if (inf) {
    if (comp && !sort && x.is_zero()) { out = G1::infinity(); return true; }
    return false;
  }
  if (!comp) return false;
  Fp y;
  if (!(x.sq() * x + G1::B).sqrt(y)) return false;
  if (y.lexicographically_largest() != sort) y = -y;
  out = G1::from_affine(x, y);
  if (check_subgroup && !G1::in_subgroup(out)) return false;
  return true;
}
void g2_compress(const G2P &p, uint8_t out[96]) {
  if (G2::is_inf(p)) {
    std::memset(out, 0, 96);
    out[0] = 0xc0;
    return;
  }
  Fp2 x, y;
  G2::to_affine(p, x, y);
  x.c1.to_be48(out);
  x.c0.to_be48(out + 48);
  out[0] |= 0x80;
  if (y.lexicographically_largest()) out[0] |= 0x20;
}
bool g2_decompress(const uint8_t in[96], G2P &out) {
  bool comp = in[0] & 0x80, inf = in[0] & 0x40, sort = in[0] & 0x20;
  uint8_t t[48];
  std::memcpy(t, in, 48);
  t[0] &= 0x1f;
  Fp2 x;
  if (!Fp::from_be48(t, x.c1) || !Fp::from_be48(in + 48, x.c0)) return false;
  if (inf) {
    if (comp && !sort && x.is_zero()) { out = G2::infinity(); return true; }
    return false;
  }
  if (!comp) return false;
  Fp2 y;
  if (!(x.sq() * x + G2::B).sqrt(y)) return false;
  if (y.lexicographically_largest() != sort) y = -y;
  out = G2::from_affine(x, y);
  return G2::in_subgroup(out);
}

// ============================================================ pairing
const u64 Z_ABS = 0xd201000000010000ull;  // |z|, z < 0

// Line functions evaluated at P (affine), scaled by Fp2 factors that the
// final exponentiation removes.  Returns the sparse element
// l = a + b*v + c*v*w  (positions c0.c0, c0.c1, c1.c1).
struct Line { Fp2 a, b, c; };

Fp12 mul_by_line(const Fp12 &f, const Line &l) {
  Fp12 e;
  e.c0 = {l.a, l.b, Fp2::zero()};
  e.c1 = {Fp2::zero(), l.c, Fp2::zero()};
  return f * e;
}

Line line_dbl(G2P &T, const Fp &xP, const Fp &yP) {
  // tangent at T (Jacobian); see derivation: (3X^3 - 2Y^2) + (-3X^2 Z^2 xP) v + (2 Y Z^3 yP) v w
  Fp2 X2 = T.X.sq(), Z2 = T.Z.sq();
  Fp2 X3 = X2 * T.X;
  Line l;
  l.a = X3 + X3 + X3 - T.Y.sq().dbl();
  l.b = -((X2 + X2 + X2) * Z2 * xP);
  l.c = (T.Y * Z2 * T.Z).dbl() * yP;
  T = G2::dbl(T);
  return l;
}
Line line_add(G2P &T, const Fp2 &xQ, const Fp2 &yQ, const Fp &xP, const Fp &yP) {
  Fp2 Z2 = T.Z.sq();
  Fp2 N = yQ * Z2 * T.Z - T.Y;
  Fp2 D = T.Z * (xQ * Z2 - T.X);
  Line l;
  l.a = N * xQ - yQ * D;
  l.b = -(N * xP);
  l.c = D * yP;
  T = G2::add(T, G2::from_affine(xQ, yQ));
  return l;
}

// Multi-Miller loop over pairs (P_i affine in G1, Q_i in G2), shared squarings.
Fp12 miller_loop(const std::vector<std::pair<G1P, G2P>> &pairs) {
  struct St { Fp xP, yP; Fp2 xQ, yQ; G2P T; bool skip; };
  std::vector<St> st;
  for (auto &pr : pairs) {
    St s;
    s.skip = G1::is_inf(pr.first) || G2::is_inf(pr.second);
    if (!s.skip) {
      G1::to_affine(pr.first, s.xP, s.yP);
      G2::to_affine(pr.second, s.xQ, s.yQ);
      s.T = G2::from_affine(s.xQ, s.yQ);
    }
    st.push_back(s);
  }
  Fp12 f = Fp12::one();
  for (int i = 62; i >= 0; i--) {
    f = f.sq();
    for (auto &s : st) {
      if (s.skip) continue;
      f = mul_by_line(f, line_dbl(s.T, s.xP, s.yP));
    }
    if ((Z_ABS >> i) & 1) {
      for (auto &s : st) {
        if (s.skip) continue;
        f = mul_by_line(f, line_add(s.T, s.xQ, s.yQ, s.xP, s.yP));
      }
    }
  }
  return f.conj();  // z < 0
}

Fp12 exp_by_z(const Fp12 &f) {  // f^z for unitary f, z < 0
  Fp12 r = Fp12::one();
  for (int i = 63; i >= 0; i--) {
    r = r.sq();
    if ((Z_ABS >> i) & 1) r = r * f;
  }
  return r.conj();
}

// Final exponentiation up to a fixed power coprime to r:
// easy part (p^6-1)(p^2+1), then 3*(p^4-p^2+1)/r = (z-1)^2 (z+p)(z^2+p^2-1) + 3.
Fp12 final_exp(const Fp12 &f) {
  Fp12 t = f.conj() * f.inv();
  t = frobenius(frobenius(t)) * t;
  Fp12 a = exp_by_z(t) * t.conj();      // t^(z-1)
  a = exp_by_z(a) * a.conj();           // t^((z-1)^2)
  Fp12 b = exp_by_z(a) * frobenius(a);  // a^(z+p)
  Fp12 c = exp_by_z(exp_by_z(b)) * frobenius(frobenius(b)) * b.conj();  // b^(z^2+p^2-1)
  return c * t * t * t;
}

bool pairing_product_is_one(const std::vector<std::pair<G1P, G2P>> &pairs) {
  return final_exp(miller_loop(pairs)) == Fp12::one();
}

// ============================================================ hash_to_curve G1 (RFC 9380)
// E': y^2 = x^3 + A'x + B' is 11-isogenous to E.  The isogeny is built at
// init by Velu's formulas from the kernel polynomial of its unique Fp-rational
// 11-torsion subgroup, then composed with the isomorphism (x,y)->(u^2 x,u^3 y)
// that lands on y^2 = x^3 + 4.  (The kernel polynomial and u are derived from
// the curve parameters; the resulting map reproduces the CFRG generator
// vectors bit for bit.)
const char *SSWU_A_HEX =
    "144698a3b8e9433d693a02c96d4982b0ea985383ee66a8d8e8981aefd881ac98936f8da0e0f97f5cf428082d584c1d";
const char *SSWU_B_HEX =
    "12e2908d11688030018b12e8753eee3b2016c1f0f24f4070a0b9c14fcef35ef55a23215a316ceaa5d1cc48e98e172be0";
const char *ISO_KERNEL_HEX[5] = {
    "133341fb0962a34cb0504a9c4fada0a5090d38679b4c040d5d1c3afb023a3409fcc0815fea66d8b02bbef9c8b5a66e07",
    "264908af037bcede00d054cf5d4775e83eb6cf63c76b969f8ed174fb59fcff78d201f46f6cfc4ed6552e59ce75177b0",
    "1335c502c1f54c49aceea65e87fd7203ba0f626f305fc0cfd606a5dae9f3c8e81a4b3b69600129fabd307c69bf319d39",
    "94440f65f408a6e930e16e3e92dd17bf60d6e9679a8d3d58593de55ac23703042d609537eb3549aac234d896ca82944",
    "4afe09d5cf4956a23b6b71f59d2b3407b415a774b7be81bbb6fa99cbc798e0ac98ba725a5bc328016b1c268b4766e85"};
const char *ISO_U_HEX =
    "17a3e1bda8a2d1a38a19241a0ea1e2f25b552d6197903f96bae690ef6be6b1381be22e8a72a9745cd7a1ffffffffb26d";

Fp fp_from_hex(const char *hex) {
  u64 c[6] = {0};
  size_t len = std::strlen(hex);
  for (size_t i = 0; i < len; i++) {
    char ch = hex[len - 1 - i];
    u64 v = (ch >= '0' && ch <= '9') ? ch - '0' : ch - 'a' + 10;
    c[i / 16] |= v << (4 * (i % 16));
  }
  return Fp::from_canon(c);
}

typedef std::vector<Fp> Poly;  // low -> high
Poly pmul(const Poly &a, const Poly &b) {
  Poly r(a.size() + b.size() - 1, Fp::zero());
  for (size_t i = 0; i < a.size(); i++)
    for (size_t j = 0; j < b.size(); j++) r[i + j] = r[i + j] + a[i] * b[j];
  return r;
}
Poly padd(const Poly &a, const Poly &b) {
  Poly r(std::max(a.size(), b.size()), Fp::zero());
  for (size_t i = 0; i < a.size(); i++) r[i] = r[i] + a[i];
  for (size_t i = 0; i < b.size(); i++) r[i] = r[i] + b[i];
  return r;
}
Poly pscale(const Poly &a, const Fp &s) {
  Poly r = a;
  for (auto &c : r) c = c * s;
  return r;
}
Poly pderiv(const Poly &a) {
  Poly r;
  for (size_t i = 1; i < a.size(); i++) r.push_back(a[i] * Fp::from_u64(i));
  if (r.empty()) r.push_back(Fp::zero());
  return r;
}
Poly pmod_monic(Poly a, const Poly &m) {  // m monic
  size_t dm = m.size() - 1;
  for (size_t i = a.size(); i-- > dm;) {
    Fp c = a[i];
    if (c.is_zero()) continue;
    for (size_t j = 0; j <= dm; j++) a[i - dm + j] = a[i - dm + j] - c * m[j];
  }
  a.resize(dm);
  return a;
}
Fp peval(const Poly &a, const Fp &x) {
  Fp r = Fp::zero();
  for (size_t i = a.size(); i-- > 0;) r = r * x + a[i];
  return r;
}

Fp SSWU_A, SSWU_B, SSWU_Z;
Poly ISO_XNUM, ISO_XDEN, ISO_YNUM, ISO_YDEN;

void init_isogeny() {
  SSWU_A = fp_from_hex(SSWU_A_HEX);
  SSWU_B = fp_from_hex(SSWU_B_HEX);
  SSWU_Z = Fp::from_u64(11);
  Poly D;
  for (int i = 0; i < 5; i++) D.push_back(fp_from_hex(ISO_KERNEL_HEX[i]));
  D.push_back(Fp::one());
  const Fp &a = SSWU_A, &b = SSWU_B;
  Poly Dp = pderiv(D);
  // Velu: X = x + sum v_P/(x-x_P) + u_P/(x-x_P)^2, v = 2(3t^2+a), u = 4(t^3+at+b)
  Poly vpoly = {a.dbl(), Fp::zero(), Fp::from_u64(6)};
  Poly upoly = {b.dbl().dbl(), a.dbl().dbl(), Fp::zero(), Fp::from_u64(4)};
  Poly Rv = pmod_monic(pmul(vpoly, Dp), D);
  Poly Ru = pmod_monic(pmul(upoly, Dp), D);
  Poly D2 = pmul(D, D);
  Poly N = padd(padd(pmul({Fp::zero(), Fp::one()}, D2), pmul(Rv, D)),
                padd(pmul(Ru, Dp), pscale(pmul(pderiv(Ru), D), -Fp::one())));
  Poly Yn = padd(pmul(pderiv(N), D), pscale(pmul(N, Dp), -Fp::from_u64(2)));
  Fp u = fp_from_hex(ISO_U_HEX);
  ISO_XNUM = pscale(N, u.sq());
  ISO_XDEN = D2;
  ISO_YNUM = pscale(Yn, u.sq() * u);
  ISO_YDEN = pmul(D2, D);
}

void sswu(const Fp &u, Fp &x, Fp &y) {
  const Fp &A = SSWU_A, &B = SSWU_B, &Z = SSWU_Z;
  Fp u2 = u.sq();
  Fp tv1 = Z.sq() * u2.sq() + Z * u2;
  Fp x1;
  if (tv1.is_zero()) x1 = B * (Z * A).inv();
  else x1 = (-B) * A.inv() * (Fp::one() + tv1.inv());
  Fp gx1 = x1.sq() * x1 + A * x1 + B;
  if (gx1.sqrt(y)) {
    x = x1;
  } else {
    x = Z * u2 * x1;
    Fp gx2 = x.sq() * x + A * x + B;
    gx2.sqrt(y);
  }
  if (u.parity() != y.parity()) y = -y;
}

G1P iso_map(const Fp &x, const Fp &y) {
  Fp xd = peval(ISO_XDEN, x), yd = peval(ISO_YDEN, x);
  if (xd.is_zero() || yd.is_zero()) return G1::infinity();
  return G1::from_affine(peval(ISO_XNUM, x) * xd.inv(), y * peval(ISO_YNUM, x) * yd.inv());
}

G1P hash_to_curve(const uint8_t *msg, size_t len, const uint8_t *dst, size_t dlen) {
  uint8_t ub[128];
  expand_message(msg, len, dst, dlen, ub, 128);
  Fp u0 = Fp::from_be64_mod(ub), u1 = Fp::from_be64_mod(ub + 64);
  Fp x, y;
  sswu(u0, x, y);
  G1P q0 = iso_map(x, y);
  sswu(u1, x, y);
  G1P q1 = iso_map(x, y);
  u64 heff[1] = {0xd201000000010001ull};
  return G1::mul_limbs(G1::add(q0, q1), heff, 1);
}

// ============================================================ init
std::once_flag INIT_FLAG;
void init_all() {
  init_modulus<6>(PM, P_HEX);
  init_modulus<4>(RM, R_HEX);
  G1::B = Fp::from_u64(4);
  G2::B = Fp2{Fp::from_u64(4), Fp::from_u64(4)};
  G1_GEN = G1::from_affine(
      fp_from_hex("17f1d3a73197d7942695638c4fa9ac0fc3688c4f9774b905a14e3a3f171bac586c55e83ff97a1aeffb3af00adb22c6bb"),
      fp_from_hex("08b3f481e3aaa0f1a09e30ed741d8ae4fcf5e095d5d00af600db18cb2c04b3edd03cc744a2888ae40caa232946c5e7e1"));
  G2_GEN = G2::from_affine(
      Fp2{fp_from_hex("024aa2b2f08f0a91260805272dc51051c6e47ad4fa403b02b4510b647ae3d1770bac0326a805bbefd48056c8c121bdb8"),
          fp_from_hex("13e02b6052719f607dacd3a088274f65596bd0d09920b61ab5da61bbdc7f5049334cf11213945d57e5ac7d055d042b7e")},
      Fp2{fp_from_hex("0ce5d527727d6e118cc9cdc6da2e351aadfd9baa8cbdd3a76d429a695160d12c923ac9cc3baca289e193548608b82801"),
          fp_from_hex("0606c4a02ea734cc32acd2b02bc28b99cb3e287e85a763af267492ab572e99ab3f370d275cec1da1aaa9075ff05f79be")});
  // gamma_k = xi^{k(p-1)/6}
  u64 e[6];
  std::memcpy(e, PM.m, sizeof e);
  e[0] -= 1;  // p - 1 (p is odd, no borrow)
  // divide by 6
  u128 rem = 0;
  for (int i = 5; i >= 0; i--) {
    u128 cur = (rem << 64) | e[i];
    e[i] = (u64)(cur / 6);
    rem = cur % 6;
  }
  Fp2 xi = {Fp::one(), Fp::one()};
  Fp2 g = xi.pow(e, 6);
  FROB_GAMMA[0] = Fp2::one();
  for (int k = 1; k < 6; k++) FROB_GAMMA[k] = FROB_GAMMA[k - 1] * g;
  init_isogeny();
  // P1 of each suite (ciphersuites.rs:62 SHAKE-256, :78 SHA-256)
  const char *P1_HEX[2] = {
      "a8ce256102840821a3e94ea9025e4662b205762f9776b3a766c872b948f1fd225e7c59698588e70d11406d161b4e28c9",
      "8929dfbc7e6642c4ed9cba0856e493f8b9d7d5fcb0c31ef8fdcd34d50648a56c795e106e9eada6e0bda386b414150755"};
  for (int su = 0; su < 2; su++) {
    uint8_t p1[48];
    for (int i = 0; i < 48; i++) {
      auto hv = [](char c) { return (c >= '0' && c <= '9') ? c - '0' : c - 'a' + 10; };
      p1[i] = (uint8_t)(hv(P1_HEX[su][2 * i]) << 4 | hv(P1_HEX[su][2 * i + 1]));
    }
    g1_decompress(p1, P1_POINTS[su]);
  }
}
inline void ensure_init() { std::call_once(INIT_FLAG, init_all); }

// ============================================================ BBS protocol
const std::string API_IDS[2] = {"BBS_BLS12381G1_XMD:SHA-256_SSWU_RO_H2G_HM2S_",
                                "BBS_BLS12381G1_XOF:SHAKE-256_SSWU_RO_H2G_HM2S_"};
#define API_ID (API_IDS[SUITE])

Bytes str_bytes(const std::string &s) { return Bytes(s.begin(), s.end()); }
void i2osp(Bytes &out, u64 x, int n) {
  for (int i = n - 1; i >= 0; i--) out.push_back((uint8_t)(x >> (8 * i)));
}

bool hash_to_scalar(const uint8_t *msg, size_t len, const Bytes &dst, Fr &out) {
  if (dst.size() > 255) return false;
  uint8_t ub[48];
  if (!expand_message(msg, len, dst.data(), dst.size(), ub, 48)) return false;
  out = Fr::from_okm(ub);
  return true;
}
bool hash_to_scalar(const Bytes &msg, const Bytes &dst, Fr &out) {
  return hash_to_scalar(msg.data(), msg.size(), dst, out);
}

// Generators cache: prefix-stable chain (generators.rs:119-146)
std::mutex GEN_MU;
std::vector<G1P> GEN_CACHES[2];    // Q1, H1, H2, ... per suite
std::vector<Bytes> GEN_CACHES_C[2];  // compressed
Bytes GEN_VS[2];                   // chain state after GEN_CACHE.size() steps

void generators(size_t count, std::vector<G1P> &out, std::vector<Bytes> *comp = nullptr) {
  std::lock_guard<std::mutex> g(GEN_MU);
  std::vector<G1P> &GEN_CACHE = GEN_CACHES[SUITE];
  std::vector<Bytes> &GEN_CACHE_C = GEN_CACHES_C[SUITE];
  Bytes &GEN_V = GEN_VS[SUITE];
  Bytes seed_dst = str_bytes(API_ID + "SIG_GENERATOR_SEED_");
  Bytes gen_dst = str_bytes(API_ID + "SIG_GENERATOR_DST_");
  if (GEN_CACHE.empty()) {
    Bytes seed = str_bytes(API_ID + "MESSAGE_GENERATOR_SEED");
    GEN_V.assign(48, 0);
    expand_message(seed.data(), seed.size(), seed_dst.data(), seed_dst.size(), GEN_V.data(), 48);
  }
  while (GEN_CACHE.size() < count) {
    Bytes v = GEN_V;
    i2osp(v, GEN_CACHE.size() + 1, 8);
    Bytes nv(48);
    expand_message(v.data(), v.size(), seed_dst.data(), seed_dst.size(), nv.data(), 48);
    GEN_V = nv;
    G1P gpt = hash_to_curve(nv.data(), 48, gen_dst.data(), gen_dst.size());
    GEN_CACHE.push_back(gpt);
    Bytes c(48);
    g1_compress(gpt, c.data());
    GEN_CACHE_C.push_back(c);
  }
  out.assign(GEN_CACHE.begin(), GEN_CACHE.begin() + count);
  if (comp) comp->assign(GEN_CACHE_C.begin(), GEN_CACHE_C.begin() + count);
}

// calculate_domain (util.rs:147-189)
bool calculate_domain(const uint8_t pk[96], const std::vector<Bytes> &gens_c, size_t L,
                      const uint8_t *header, size_t hlen, Fr &out) {
  Bytes in(pk, pk + 96);
  i2osp(in, L, 8);
  for (size_t i = 0; i <= L; i++) in.insert(in.end(), gens_c[i].begin(), gens_c[i].end());
  in.insert(in.end(), API_ID.begin(), API_ID.end());
  i2osp(in, hlen, 8);
  if (hlen) in.insert(in.end(), header, header + hlen);
  return hash_to_scalar(in, str_bytes(API_ID + "H2S_"), out);
}

bool messages_to_scalars(const uint8_t *msgs, const size_t *lens, size_t L, std::vector<Fr> &out) {
  Bytes dst = str_bytes(API_ID + "MAP_MSG_TO_SCALAR_AS_HASH_");
  out.resize(L);
  size_t off = 0;
  for (size_t i = 0; i < L; i++) {
    if (!hash_to_scalar(msgs + off, lens[i], dst, out[i])) return false;
    off += lens[i];
  }
  return true;
}

G1P compute_b(const std::vector<G1P> &gens, const std::vector<Fr> &m, const Fr &domain) {
  // B = P1 + Q1*domain + sum H_i*m_i (signature.rs:620-640)
  G1P B = G1::add(P1_POINT, G1::mul(gens[0], domain));
  for (size_t i = 0; i < m.size(); i++) B = G1::add(B, G1::mul(gens[i + 1], m[i]));
  return B;
}

// seeded_random_scalars (util.rs:329-358).  With expand_message_xmd a single
// call covers at most 170 scalars (255*32 bytes); larger counts are derived in
// chunks of 170 with seed || I2OSP(chunk, 2) (build-defined extension).  With
// expand_message_xof one call covers up to 1365 scalars (65535 bytes).
bool seeded_random_scalars(const uint8_t *seed, size_t slen, const uint8_t *dst, size_t dlen,
                           size_t count, std::vector<Fr> &out) {
  out.clear();
  const size_t CHUNK = SUITE == 1 ? 1365 : 170;
  if (count <= CHUNK) {
    Bytes v(48 * count);
    if (count && !expand_message(seed, slen, dst, dlen, v.data(), v.size())) return false;
    for (size_t i = 0; i < count; i++) out.push_back(Fr::from_okm(v.data() + 48 * i));
    return true;
  }
  for (size_t c = 0; c * CHUNK < count; c++) {
    size_t n = std::min(CHUNK, count - c * CHUNK);
    Bytes s(seed, seed + slen);
    i2osp(s, c, 2);
    Bytes v(48 * n);
    if (!expand_message(s.data(), s.size(), dst, dlen, v.data(), v.size())) return false;
    for (size_t i = 0; i < n; i++) out.push_back(Fr::from_okm(v.data() + 48 * i));
  }
  return true;
}

}  // namespace

// ============================================================ C API
extern "C" {

int oracle_sha256(const uint8_t *msg, size_t len, uint8_t out[32]) {
  Sha256 s;
  if (len) s.update(msg, len);
  s.final(out);
  return 0;
}

int oracle_expand_message_xmd(const uint8_t *msg, size_t len, const uint8_t *dst, size_t dst_len,
                              uint8_t *out, size_t out_len) {
  return expand_xmd(msg, len, dst, dst_len, out, out_len) ? 0 : 1;
}

int oracle_expand_message_xof(const uint8_t *msg, size_t len, const uint8_t *dst, size_t dst_len,
                              uint8_t *out, size_t out_len) {
  return expand_xof(msg, len, dst, dst_len, out, out_len) ? 0 : 1;
}

int oracle_shake256(const uint8_t *msg, size_t len, uint8_t *out, size_t out_len) {
  Shake256 h;
  if (len) h.update(msg, len);
  h.squeeze(out, out_len);
  return 0;
}

// Selects the calling thread's ciphersuite (0 SHA-256, 1 SHAKE-256) for every
// later call on this thread; returns the previous one (-1 for an unknown suite).
int oracle_set_suite(int suite) {
  if (suite != 0 && suite != 1) return -1;
  int prev = SUITE;
  SUITE = suite;
  return prev;
}

int oracle_hash_to_scalar(const uint8_t *msg, size_t len, const uint8_t *dst, size_t dst_len,
                          uint8_t out[32]) {
  ensure_init();
  Fr s;
  if (!hash_to_scalar(msg, len, Bytes(dst, dst + dst_len), s)) return 1;
  s.to_be32(out);
  return 0;
}

int oracle_keygen(const uint8_t *km, size_t km_len, const uint8_t *ki, size_t ki_len,
                  const uint8_t *kd, size_t kd_len, uint8_t sk_out[32]) {
  ensure_init();
  if (km_len < 32 || ki_len > 65535) return 1;
  Bytes in(km, km + km_len);
  i2osp(in, ki_len, 2);
  if (ki_len) in.insert(in.end(), ki, ki + ki_len);
  Bytes dst = kd ? Bytes(kd, kd + kd_len) : str_bytes(API_ID + "KEYGEN_DST_");
  Fr sk;
  if (!hash_to_scalar(in, dst, sk)) return 1;
  sk.to_be32(sk_out);
  return 0;
}

int oracle_sk_to_pk(const uint8_t sk[32], uint8_t pk_out[96]) {
  ensure_init();
  Fr s;
  if (!Fr::from_be32(sk, s)) return 1;
  g2_compress(G2::mul(G2_GEN, s), pk_out);
  return 0;
}

int oracle_generators(size_t count, uint8_t *out, uint8_t *p1_out) {
  ensure_init();
  std::vector<G1P> g;
  std::vector<Bytes> c;
  generators(count, g, &c);
  for (size_t i = 0; i < count; i++) std::memcpy(out + 48 * i, c[i].data(), 48);
  if (p1_out) g1_compress(P1_POINT, p1_out);
  return 0;
}

int oracle_hash_to_curve_g1(const uint8_t *msg, size_t len, const uint8_t *dst, size_t dst_len,
                            uint8_t out[48]) {
  ensure_init();
  g1_compress(hash_to_curve(msg, len, dst, dst_len), out);
  return 0;
}

int oracle_seeded_random_scalars(const uint8_t *seed, size_t seed_len, const uint8_t *dst,
                                 size_t dst_len, size_t count, uint8_t *out) {
  ensure_init();
  std::vector<Fr> s;
  if (!seeded_random_scalars(seed, seed_len, dst, dst_len, count, s)) return 1;
  for (size_t i = 0; i < count; i++) s[i].to_be32(out + 32 * i);
  return 0;
}

// Sign (signature.rs:101-135 -> core_sign :544-580 -> :642-660)
int oracle_sign(const uint8_t sk[32], const uint8_t pk[96], const uint8_t *header, size_t hlen,
                const uint8_t *msgs, const size_t *lens, size_t L, uint8_t sig_out[80],
                uint8_t b_trace[48], uint8_t domain_trace[32]) {
  ensure_init();
  Fr s;
  if (!Fr::from_be32(sk, s)) return 1;
  G2P pkp;
  if (!g2_decompress(pk, pkp)) return 1;
  std::vector<Fr> m;
  if (!messages_to_scalars(msgs, lens, L, m)) return 1;
  std::vector<G1P> gens;
  std::vector<Bytes> gc;
  generators(L + 1, gens, &gc);
  Fr domain;
  if (!calculate_domain(pk, gc, L, header, hlen, domain)) return 1;
  Bytes ein;
  uint8_t tmp[32];
  s.to_be32(tmp);
  ein.insert(ein.end(), tmp, tmp + 32);
  for (auto &x : m) { x.to_be32(tmp); ein.insert(ein.end(), tmp, tmp + 32); }
  domain.to_be32(tmp);
  ein.insert(ein.end(), tmp, tmp + 32);
  Fr e;
  if (!hash_to_scalar(ein, str_bytes(API_ID + "H2S_"), e)) return 1;
  G1P B = compute_b(gens, m, domain);
  Fr ske = s + e;
  if (ske.is_zero()) return 1;
  G1P A = G1::mul(B, ske.inv());
  if (G1::is_inf(A)) return 1;
  g1_compress(A, sig_out);
  e.to_be32(sig_out + 48);
  if (b_trace) g1_compress(B, b_trace);
  if (domain_trace) domain.to_be32(domain_trace);
  return 0;
}

// Verify (signature.rs:264-292 -> core_verify :676-728)
int oracle_verify(const uint8_t pk[96], const uint8_t *sig, size_t sig_len, const uint8_t *header,
                  size_t hlen, const uint8_t *msgs, const size_t *lens, size_t L) {
  ensure_init();
  G2P pkp;
  if (!g2_decompress(pk, pkp)) return 1;
  if (sig_len != 80) return 1;
  G1P A;
  Fr e;
  if (!g1_decompress(sig, A) || !Fr::from_be32(sig + 48, e)) return 1;
  std::vector<Fr> m;
  if (!messages_to_scalars(msgs, lens, L, m)) return 1;
  std::vector<G1P> gens;
  std::vector<Bytes> gc;
  generators(L + 1, gens, &gc);
  Fr domain;
  if (!calculate_domain(pk, gc, L, header, hlen, domain)) return 1;
  G1P B = compute_b(gens, m, domain);
  G2P A2 = G2::add(pkp, G2::mul(G2_GEN, e));
  std::vector<std::pair<G1P, G2P>> pairs = {{A, A2}, {B, G2::neg(G2_GEN)}};
  return pairing_product_is_one(pairs) ? 0 : 2;
}

// ProofGen (proof.rs:1634-1680 -> core_proof_gen :1568-1650, proof_init :1754-1820,
// proof_challenge_calculate :2165-2282, proof_finalize_parts :2317-2359, to_bytes :173-187)
int oracle_proof_gen(const uint8_t pk[96], const uint8_t *sig, size_t sig_len,
                     const uint8_t *header, size_t hlen, const uint8_t *ph, size_t phlen,
                     const uint8_t *msgs, const size_t *lens, size_t L, const size_t *disclosed,
                     size_t R_in, const uint8_t *seed, size_t seed_len, const uint8_t *dst,
                     size_t dst_len, uint8_t *proof_out, size_t proof_cap, size_t *proof_len) {
  ensure_init();
  G2P pkp;
  if (!g2_decompress(pk, pkp)) return 1;
  if (sig_len != 80) return 1;
  G1P A;
  Fr e;
  if (!g1_decompress(sig, A) || !Fr::from_be32(sig + 48, e)) return 1;
  std::vector<Fr> m;
  if (!messages_to_scalars(msgs, lens, L, m)) return 1;
  std::vector<size_t> di(disclosed, disclosed + R_in);
  std::sort(di.begin(), di.end());
  di.erase(std::unique(di.begin(), di.end()), di.end());
  size_t R = di.size();
  if (R > L) return 1;
  for (size_t i : di)
    if (L == 0 || i > L - 1) return 1;
  size_t U = L - R;
  std::vector<size_t> ui;
  for (size_t i = 0, k = 0; i < L; i++) {
    if (k < R && di[k] == i) { k++; continue; }
    ui.push_back(i);
  }
  std::vector<Fr> rs;
  if (!seeded_random_scalars(seed, seed_len, dst, dst_len, 5 + U, rs)) return 1;
  std::vector<G1P> gens;
  std::vector<Bytes> gc;
  generators(L + 1, gens, &gc);
  Fr domain;
  if (!calculate_domain(pk, gc, L, header, hlen, domain)) return 1;
  G1P B = compute_b(gens, m, domain);
  const Fr &r1 = rs[0], &r2 = rs[1], &et = rs[2], &r1t = rs[3], &r3t = rs[4];
  G1P D = G1::mul(B, r2);
  G1P Abar = G1::mul(A, r1 * r2);
  G1P Bbar = G1::add(G1::mul(D, r1), G1::neg(G1::mul(Abar, e)));
  G1P T1 = G1::add(G1::mul(Abar, et), G1::mul(D, r1t));
  G1P T2 = G1::mul(D, r3t);
  for (size_t j = 0; j < U; j++) T2 = G1::add(T2, G1::mul(gens[1 + ui[j]], rs[5 + j]));
  // challenge
  Bytes c;
  i2osp(c, R, 8);
  uint8_t tmp[48];
  for (size_t i = 0; i < R; i++) {
    i2osp(c, di[i], 8);
    m[di[i]].to_be32(tmp);
    c.insert(c.end(), tmp, tmp + 32);
  }
  for (const G1P *pt : {&Abar, &Bbar, &D, &T1, &T2}) {
    g1_compress(*pt, tmp);
    c.insert(c.end(), tmp, tmp + 48);
  }
  domain.to_be32(tmp);
  c.insert(c.end(), tmp, tmp + 32);
  i2osp(c, phlen, 8);
  if (phlen) c.insert(c.end(), ph, ph + phlen);
  Fr ch;
  if (!hash_to_scalar(c, str_bytes(API_ID + "H2S_"), ch)) return 1;
  if (r2.is_zero()) return 1;
  Fr r3 = r2.inv();
  Fr ecap = et + e * ch, r1cap = r1t - r1 * ch, r3cap = r3t - r3 * ch;
  size_t need = 3 * 48 + (U + 4) * 32;
  if (proof_cap < need) return 2;
  uint8_t *o = proof_out;
  g1_compress(Abar, o); o += 48;
  g1_compress(Bbar, o); o += 48;
  g1_compress(D, o); o += 48;
  ecap.to_be32(o); o += 32;
  r1cap.to_be32(o); o += 32;
  r3cap.to_be32(o); o += 32;
  for (size_t j = 0; j < U; j++) {
    (rs[5 + j] + m[ui[j]] * ch).to_be32(o);
    o += 32;
  }
  ch.to_be32(o);
  *proof_len = need;
  return 0;
}

// ProofVerify (proof.rs:948-985 -> core_proof_verify :2382-2426, proof_verify_init :3015-3078,
// from_bytes :189-225)
int oracle_proof_verify(const uint8_t pk[96], const uint8_t *proof, size_t proof_len,
                        const uint8_t *header, size_t hlen, const uint8_t *ph, size_t phlen,
                        const uint8_t *dmsgs, const size_t *dlens, size_t R_in,
                        const size_t *disclosed) {
  ensure_init();
  G2P pkp;
  if (!g2_decompress(pk, pkp)) return 1;
  if (proof_len < 240 + 32) return 2;
  G1P Abar, Bbar, D;
  if (!g1_decompress(proof, Abar) || !g1_decompress(proof + 48, Bbar) ||
      !g1_decompress(proof + 96, D))
    return 2;
  Fr ecap, r1cap, r3cap;
  if (!Fr::from_be32(proof + 144, ecap) || !Fr::from_be32(proof + 176, r1cap) ||
      !Fr::from_be32(proof + 208, r3cap))
    return 2;
  size_t nchunks = (proof_len - 240) / 32;  // chunks_exact ignores a remainder
  std::vector<Fr> mcap(nchunks);
  for (size_t i = 0; i < nchunks; i++)
    if (!Fr::from_be32(proof + 240 + 32 * i, mcap[i])) return 2;
  Fr ch = mcap.back();
  mcap.pop_back();
  std::vector<size_t> di(disclosed, disclosed + R_in);
  std::sort(di.begin(), di.end());
  di.erase(std::unique(di.begin(), di.end()), di.end());
  size_t U = mcap.size(), R = di.size(), L = U + R;
  std::vector<Fr> dm;
  if (!messages_to_scalars(dmsgs, dlens, R_in, dm)) return 1;
  for (size_t i : di)
    if (L == 0 || i > L - 1) return 2;
  if (dm.size() != R) return 2;
  std::vector<G1P> gens;
  std::vector<Bytes> gc;
  generators(L + 1, gens, &gc);
  std::vector<size_t> ui;
  for (size_t i = 0, k = 0; i < L; i++) {
    if (k < R && di[k] == i) { k++; continue; }
    ui.push_back(i);
  }
  Fr domain;
  if (!calculate_domain(pk, gc, L, header, hlen, domain)) return 1;
  G1P T1 = G1::add(G1::add(G1::mul(Bbar, ch), G1::mul(Abar, ecap)), G1::mul(D, r1cap));
  G1P Bv = G1::add(P1_POINT, G1::mul(gens[0], domain));
  for (size_t i = 0; i < R; i++) Bv = G1::add(Bv, G1::mul(gens[1 + di[i]], dm[i]));
  G1P T2 = G1::add(G1::mul(Bv, ch), G1::mul(D, r3cap));
  for (size_t j = 0; j < U; j++) T2 = G1::add(T2, G1::mul(gens[1 + ui[j]], mcap[j]));
  Bytes c;
  i2osp(c, R, 8);
  uint8_t tmp[48];
  for (size_t i = 0; i < R; i++) {
    i2osp(c, di[i], 8);
    dm[i].to_be32(tmp);
    c.insert(c.end(), tmp, tmp + 32);
  }
  for (const G1P *pt : {&Abar, &Bbar, &D, &T1, &T2}) {
    g1_compress(*pt, tmp);
    c.insert(c.end(), tmp, tmp + 48);
  }
  domain.to_be32(tmp);
  c.insert(c.end(), tmp, tmp + 32);
  i2osp(c, phlen, 8);
  if (phlen) c.insert(c.end(), ph, ph + phlen);
  Fr ch2;
  if (!hash_to_scalar(c, str_bytes(API_ID + "H2S_"), ch2)) return 1;
  if (ch2 != ch) return 2;
  std::vector<std::pair<G1P, G2P>> pairs = {{Abar, pkp}, {Bbar, G2::neg(G2_GEN)}};
  return pairing_product_is_one(pairs) ? 0 : 2;
}

int oracle_calculate_domain(const uint8_t pk[96], const uint8_t *header, size_t hlen, size_t L,
                            uint8_t out32[32]) {
  ensure_init();
  std::vector<G1P> gens;
  std::vector<Bytes> gc;
  generators(L + 1, gens, &gc);
  Fr d;
  if (!calculate_domain(pk, gc, L, header, hlen, d)) return 1;
  d.to_be32(out32);
  return 0;
}

int oracle_g1_msm(const uint8_t *points48, const uint8_t *scalars32_be, size_t n, uint8_t out48[48]) {
  ensure_init();
  G1P acc = G1::infinity();
  for (size_t i = 0; i < n; i++) {
    G1P p;
    Fr k;
    if (!g1_decompress(points48 + 48 * i, p) || !Fr::from_be32(scalars32_be + 32 * i, k)) return 1;
    acc = G1::add(acc, G1::mul(p, k));
  }
  g1_compress(acc, out48);
  return 0;
}

int oracle_g1_add(const uint8_t a48[48], const uint8_t b48[48], uint8_t out48[48]) {
  ensure_init();
  G1P a, b;
  if (!g1_decompress(a48, a) || !g1_decompress(b48, b)) return 1;
  g1_compress(G1::add(a, b), out48);
  return 0;
}

int oracle_g1_decompress(const uint8_t in48[48], uint8_t out_xy_be[96]) {
  ensure_init();
  G1P p;
  if (!g1_decompress(in48, p)) return 1;
  if (G1::is_inf(p)) {
    std::memset(out_xy_be, 0, 96);
    return 0;
  }
  Fp x, y;
  G1::to_affine(p, x, y);
  x.to_be48(out_xy_be);
  y.to_be48(out_xy_be + 48);
  return 0;
}

int oracle_g1_mul(const uint8_t p48[48], const uint8_t k32_be[32], uint8_t out48[48]) {
  ensure_init();
  G1P p;
  Fr k;
  if (!g1_decompress(p48, p) || !Fr::from_be32(k32_be, k)) return 1;
  g1_compress(G1::mul(p, k), out48);
  return 0;
}

int oracle_g2_decompress(const uint8_t in96[96]) {
  ensure_init();
  G2P p;
  return g2_decompress(in96, p) ? 0 : 1;
}

int oracle_pairing_eq(const uint8_t a48[48], const uint8_t b96[96], const uint8_t c48[48],
                      const uint8_t d96[96]) {
  ensure_init();
  G1P a, c;
  G2P b, d;
  if (!g1_decompress(a48, a) || !g1_decompress(c48, c) || !g2_decompress(b96, b) ||
      !g2_decompress(d96, d))
    return 1;
  std::vector<std::pair<G1P, G2P>> pairs = {{a, b}, {c, G2::neg(d)}};
  return pairing_product_is_one(pairs) ? 0 : 2;
}

int oracle_fp_mul(const uint8_t a48[48], const uint8_t b48[48], uint8_t out48[48]) {
  ensure_init();
  Fp a, b;
  if (!Fp::from_be48(a48, a) || !Fp::from_be48(b48, b)) return 1;
  (a * b).to_be48(out48);
  return 0;
}

int oracle_fr_mul(const uint8_t a32[32], const uint8_t b32[32], uint8_t out32[32]) {
  ensure_init();
  Fr a, b;
  if (!Fr::from_be32(a32, a) || !Fr::from_be32(b32, b)) return 1;
  (a * b).to_be32(out32);
  return 0;
}

int oracle_fr_inv(const uint8_t a32[32], uint8_t out32[32]) {
  ensure_init();
  Fr a;
  if (!Fr::from_be32(a32, a)) return 1;
  a.inv().to_be32(out32);
  return 0;
}

}  // extern "C"
