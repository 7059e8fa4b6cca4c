// W3C bbs-2023 input producers and lowering (host code): the steps between
// RDF canonicalisation of a credential and the BBS operations, as
// crates/cubbs-vc-di-bbs/src/{hashing,hmac_label,canonical,key,prepared}.rs
// take them.
//
//   * HMAC-SHA256 blank-node label map (hmac_label.rs:26-50): each canonical
//     label c14nN is HMAC'd under the credential's HMAC key and written as
//     'u' || base64url-no-pad(HMAC); the identifiers are sorted and each input
//     label becomes b<rank>.
//   * Relabel and sort (canonical.rs:64-92,130-150): every "_:label" of a
//     canonical N-Quad is replaced through the map (a label runs to the next
//     Unicode whitespace), then the lines are sorted bytewise.
//   * The 64-byte bbs-2023 header (hashing.rs:7-31): SHA-256 of the canonical
//     proof configuration lines, joined with no separator, then SHA-256 of the
//     mandatory lines likewise.
//   * The BLS12-381 G2 public key as a Multikey (key.rs:25-80): 'z' ||
//     base58btc(0xeb 0x01 || key), did:key and verification-method forms.
//   * Issue and verify of a base proof lowered to the BBS operations
//     (prepared.rs:335-513): the header from the proof hash and the mandatory
//     lines, the non-mandatory lines as the messages, Sign or Verify on the
//     device, and the proofValue codec.
//
// JSON-LD expansion and RDFC-1.0 canonicalisation come before these steps;
// the reference takes them from third-party crates (json-ld, rdf-canon).
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/cubbs_bbs_gpu_abi.h"

namespace {

// ------------------------------------------------------------------ SHA-256 (FIPS 180-4), host
// The round constants and the initial hash value are derived as FIPS 180-4
// defines them: the first 32 bits of the fractional parts of the cube roots
// (K) and square roots (H0) of the first primes, found exactly with integer
// roots of p * 2^96 and p * 2^64.
struct Sha256Constants {
  uint32_t k[64], h0[8];
  Sha256Constants() {
    int primes[64], np = 0;
    for (int c = 2; np < 64; c++) {
      bool prime = true;
      for (int d = 2; d * d <= c; d++) prime = prime && c % d;
      if (prime) primes[np++] = c;
    }
    for (int i = 0; i < 64; i++) k[i] = (uint32_t)iroot(primes[i], 3);
    for (int i = 0; i < 8; i++) h0[i] = (uint32_t)iroot(primes[i], 2);
  }
  // largest x with x^e <= p * 2^(32 e): x = floor(p^(1/e) 2^32) < 2^35
  static uint64_t iroot(int p, int e) {
    const unsigned __int128 target = (unsigned __int128)p << (32 * e);
    uint64_t lo = 0, hi = (uint64_t)1 << 36;
    while (hi - lo > 1) {
      const uint64_t mid = lo + (hi - lo) / 2;
      unsigned __int128 v = 1;
      for (int j = 0; j < e; j++) v *= mid;
      if (v <= target) lo = mid;
      else hi = mid;
    }
    return lo;
  }
};
const Sha256Constants &sha_consts() {
  static const Sha256Constants c;
  return c;
}

struct Sha256 {
  uint32_t h[8];
  uint8_t buf[64];
  size_t fill = 0;
  uint64_t total = 0;
  Sha256() { std::memcpy(h, sha_consts().h0, sizeof h); }
  static uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }
  void block(const uint8_t *p) {
    const uint32_t *K = sha_consts().k;
    uint32_t w[64];
    for (int i = 0; i < 16; i++) w[i] = (uint32_t)p[4 * i] << 24 | (uint32_t)p[4 * i + 1] << 16 | p[4 * i + 2] << 8 | p[4 * i + 3];
    for (int i = 16; i < 64; i++) {
      const uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
      const uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
      w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
    for (int i = 0; i < 64; i++) {
      const uint32_t t1 = hh + (rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25)) + ((e & f) ^ (~e & g)) + K[i] + w[i];
      const uint32_t t2 = (rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
      hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
  }
  void update(const uint8_t *p, size_t n) {
    total += n;
    while (n) {
      const size_t take = std::min(n, 64 - fill);
      std::memcpy(buf + fill, p, take);
      fill += take;
      p += take;
      n -= take;
      if (fill == 64) {
        block(buf);
        fill = 0;
      }
    }
  }
  void final(uint8_t out[32]) {
    const uint64_t bits = total * 8;
    const uint8_t one = 0x80, zero = 0;
    update(&one, 1);
    while (fill != 56) update(&zero, 1);
    uint8_t len[8];
    for (int i = 0; i < 8; i++) len[i] = (uint8_t)(bits >> (56 - 8 * i));
    update(len, 8);
    for (int i = 0; i < 8; i++)
      for (int j = 0; j < 4; j++) out[4 * i + j] = (uint8_t)(h[i] >> (24 - 8 * j));
  }
};

// HMAC-SHA256 (RFC 2104, block 64 bytes; a key longer than a block is hashed first).
void hmac_sha256(const uint8_t *key, size_t klen, const uint8_t *msg, size_t mlen, uint8_t out[32]) {
  uint8_t k[64] = {0};
  if (klen > 64) {
    Sha256 s;
    s.update(key, klen);
    s.final(k);
  } else if (klen) {
    std::memcpy(k, key, klen);
  }
  uint8_t pad[64], inner[32];
  for (int i = 0; i < 64; i++) pad[i] = k[i] ^ 0x36;
  Sha256 si;
  si.update(pad, 64);
  si.update(msg, mlen);
  si.final(inner);
  for (int i = 0; i < 64; i++) pad[i] = k[i] ^ 0x5c;
  Sha256 so;
  so.update(pad, 64);
  so.update(inner, 32);
  so.final(out);
}

std::string b64url(const uint8_t *p, size_t n) {
  static const char A[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789-_";
  std::string o;
  size_t i = 0;
  for (; i + 3 <= n; i += 3) {
    const uint32_t v = (uint32_t)p[i] << 16 | p[i + 1] << 8 | p[i + 2];
    for (int s = 18; s >= 0; s -= 6) o.push_back(A[(v >> s) & 63]);
  }
  if (n - i == 1) {
    const uint32_t v = (uint32_t)p[i] << 16;
    o.push_back(A[(v >> 18) & 63]);
    o.push_back(A[(v >> 12) & 63]);
  } else if (n - i == 2) {
    const uint32_t v = (uint32_t)p[i] << 16 | p[i + 1] << 8;
    for (int s = 18; s >= 6; s -= 6) o.push_back(A[(v >> s) & 63]);
  }
  return o;
}

// ------------------------------------------------------------------ base58btc (Bitcoin alphabet)
const char B58[] = "123456789ABCDEFGHJKLMNPQRSTUVWXYZabcdefghijkmnopqrstuvwxyz";

std::string b58_encode(const uint8_t *p, size_t n) {
  size_t zeros = 0;
  while (zeros < n && p[zeros] == 0) zeros++;
  std::vector<uint8_t> digits;  // base-58 digits, least significant first
  for (size_t i = zeros; i < n; i++) {
    uint32_t carry = p[i];
    for (auto &d : digits) {
      carry += (uint32_t)d << 8;
      d = (uint8_t)(carry % 58);
      carry /= 58;
    }
    while (carry) {
      digits.push_back((uint8_t)(carry % 58));
      carry /= 58;
    }
  }
  std::string o(zeros, '1');
  for (auto it = digits.rbegin(); it != digits.rend(); ++it) o.push_back(B58[*it]);
  return o;
}

bool b58_decode(const char *s, size_t n, std::vector<uint8_t> &out) {
  size_t ones = 0;
  while (ones < n && s[ones] == '1') ones++;
  std::vector<uint8_t> bytes;  // least significant first
  for (size_t i = ones; i < n; i++) {
    const char *f = (unsigned char)s[i] < 0x80 ? std::strchr(B58, s[i]) : nullptr;
    if (!f || !s[i]) return false;
    uint32_t carry = (uint32_t)(f - B58);
    for (auto &b : bytes) {
      carry += (uint32_t)b * 58;
      b = (uint8_t)carry;
      carry >>= 8;
    }
    while (carry) {
      bytes.push_back((uint8_t)carry);
      carry >>= 8;
    }
  }
  out.assign(ones, 0);
  out.insert(out.end(), bytes.rbegin(), bytes.rend());
  return true;
}

const uint8_t MULTICODEC_G2[2] = {0xeb, 0x01};
const size_t PK_LEN = CUBBS_BBS_PUBLIC_KEY_LEN;

int32_t key_from_multibase(const char *s, size_t n, uint8_t *pk) {
  if (n == 0 || s[0] != 'z') return CUBBS_BBS2023_ERR_MULTIBASE_PREFIX;
  std::vector<uint8_t> raw;
  if (!b58_decode(s + 1, n - 1, raw)) return CUBBS_BBS2023_ERR_BASE58;
  if (raw.size() < 2 || raw[0] != MULTICODEC_G2[0] || raw[1] != MULTICODEC_G2[1])
    return CUBBS_BBS2023_ERR_MULTICODEC_HEADER;
  if (raw.size() - 2 != PK_LEN) return CUBBS_BBS2023_ERR_PUBLIC_KEY_LENGTH;
  std::memcpy(pk, raw.data() + 2, PK_LEN);
  return CUBBS_BBS_GPU_SUCCESS;
}

int32_t text_out(const std::string &t, char *out, size_t cap, size_t *len_out) {
  *len_out = t.size();
  if (!out || cap < t.size()) return CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT;
  std::memcpy(out, t.data(), t.size());
  return CUBBS_BBS_GPU_SUCCESS;
}

// ------------------------------------------------------------------ N-Quads relabelling
// Rust's char::is_whitespace (the Unicode White_Space property) at s[i] (UTF-8);
// *len gets the byte length of the character there.
bool ws_at(const std::string &s, size_t i, size_t *len) {
  const uint8_t c = (uint8_t)s[i];
  if (c < 0x80) {
    *len = 1;
    return c == ' ' || (c >= 0x09 && c <= 0x0d);
  }
  const int n = (c >> 5) == 6 ? 2 : (c >> 4) == 14 ? 3 : (c >> 3) == 30 ? 4 : 1;
  *len = std::min<size_t>(n, s.size() - i);
  if (n == 1 || i + n > s.size()) return false;
  uint32_t cp = n == 2 ? (c & 0x1f) : n == 3 ? (c & 0x0f) : (c & 0x07);
  for (int k = 1; k < n; k++) cp = cp << 6 | ((uint8_t)s[i + k] & 0x3f);
  return cp == 0x85 || cp == 0xa0 || cp == 0x1680 || (cp >= 0x2000 && cp <= 0x200a) || cp == 0x2028 ||
         cp == 0x2029 || cp == 0x202f || cp == 0x205f || cp == 0x3000;
}

std::string relabel_line(const std::string &line, const std::map<std::string, std::string> &m) {
  std::string out;
  size_t at = 0;
  for (;;) {
    const size_t pos = line.find("_:", at);
    if (pos == std::string::npos) break;
    out.append(line, at, pos + 2 - at);
    size_t end = pos + 2, step = 1;
    while (end < line.size() && !ws_at(line, end, &step)) end += step;
    if (end > line.size()) end = line.size();
    const std::string label = line.substr(pos + 2, end - pos - 2);
    const auto it = m.find(label);
    out += it == m.end() ? label : it->second;
    at = end;
  }
  out.append(line, at, std::string::npos);
  return out;
}

std::string str(const CuBbsBbsGpuByteSlice &b) { return std::string(reinterpret_cast<const char *>(b.data), b.len); }

void header_of(const uint8_t proof_hash[32], const CuBbsBbsGpuByteSlice *mandatory, size_t count, uint8_t out[64]) {
  std::memcpy(out, proof_hash, 32);
  Sha256 s;
  for (size_t i = 0; i < count; i++) s.update(mandatory[i].data, mandatory[i].len);
  s.final(out + 32);
}

bool slices_ok(const CuBbsBbsGpuByteSlice *p, size_t n) {
  if (n && !p) return false;
  for (size_t i = 0; i < n; i++)
    if (p[i].len && !p[i].data) return false;
  return true;
}

}  // namespace

extern "C" int32_t cubbs_bbs2023_hmac_sha256_v2(uint32_t abi, const uint8_t *key, size_t key_len, const uint8_t *data,
                                                size_t len, uint8_t *out32) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (key_len && !key) || (len && !data) || !out32)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  hmac_sha256(key, key_len, data, len, out32);
  return CUBBS_BBS_GPU_SUCCESS;
}

extern "C" int32_t cubbs_bbs2023_shuffled_label_map_v2(uint32_t abi, const CuBbsBbs2023LabelEntry *map, size_t count,
                                                       const uint8_t *hmac_key, size_t key_len,
                                                       uint32_t *b_index_out) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (count && (!map || !b_index_out)) || (key_len && !hmac_key))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  std::vector<std::string> ids(count);
  for (size_t i = 0; i < count; i++) {
    if (map[i].canonical.len && !map[i].canonical.data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    uint8_t d[32];
    hmac_sha256(hmac_key, key_len, map[i].canonical.data, map[i].canonical.len, d);
    ids[i] = "u" + b64url(d, 32);
  }
  std::vector<std::string> sorted = ids;
  std::sort(sorted.begin(), sorted.end());
  for (size_t i = 0; i < count; i++)
    b_index_out[i] = (uint32_t)(std::lower_bound(sorted.begin(), sorted.end(), ids[i]) - sorted.begin());
  return CUBBS_BBS_GPU_SUCCESS;
}

extern "C" int32_t cubbs_bbs2023_relabel_sort_v2(uint32_t abi, const CuBbsBbsGpuByteSlice *lines, size_t line_count,
                                                 const CuBbsBbs2023LabelEntry *label_map, size_t map_count,
                                                 uint8_t *arena, size_t arena_cap, CuBbsBbsGpuByteSlice *lines_out,
                                                 size_t *arena_used) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || !slices_ok(lines, line_count) || (map_count && !label_map) ||
      (line_count && !lines_out) || !arena_used)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  std::map<std::string, std::string> m;
  for (size_t i = 0; i < map_count; i++) m[str(label_map[i].input)] = str(label_map[i].canonical);
  std::vector<std::string> out(line_count);
  size_t need = 0;
  for (size_t i = 0; i < line_count; i++) {
    out[i] = relabel_line(str(lines[i]), m);
    need += out[i].size();
  }
  std::sort(out.begin(), out.end());
  *arena_used = need;
  if (need > arena_cap || (need && !arena)) return CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT;
  size_t at = 0;
  for (size_t i = 0; i < line_count; i++) {
    std::memcpy(arena + at, out[i].data(), out[i].size());
    lines_out[i] = {arena + at, out[i].size()};
    at += out[i].size();
  }
  return CUBBS_BBS_GPU_SUCCESS;
}

extern "C" int32_t cubbs_bbs2023_header_v2(uint32_t abi, const CuBbsBbsGpuByteSlice *proof_lines, size_t proof_count,
                                           const CuBbsBbsGpuByteSlice *mandatory, size_t mandatory_count,
                                           uint8_t *header64) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || !slices_ok(proof_lines, proof_count) ||
      !slices_ok(mandatory, mandatory_count) || !header64)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  uint8_t ph[32];
  Sha256 s;
  for (size_t i = 0; i < proof_count; i++) s.update(proof_lines[i].data, proof_lines[i].len);
  s.final(ph);
  header_of(ph, mandatory, mandatory_count, header64);
  return CUBBS_BBS_GPU_SUCCESS;
}

extern "C" int32_t cubbs_bbs2023_public_key_to_multibase_v2(uint32_t abi, int32_t form, const uint8_t *pk,
                                                            size_t pk_len, char *out, size_t cap, size_t *len_out) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (pk_len && !pk) || !len_out || form < 0 || form > 2)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (pk_len != PK_LEN) return CUBBS_BBS2023_ERR_PUBLIC_KEY_LENGTH;
  uint8_t raw[2 + PK_LEN];
  std::memcpy(raw, MULTICODEC_G2, 2);
  std::memcpy(raw + 2, pk, PK_LEN);
  const std::string mb = "z" + b58_encode(raw, sizeof raw);
  const std::string t = form == 0 ? mb : form == 1 ? "did:key:" + mb : "did:key:" + mb + "#" + mb;
  return text_out(t, out, cap, len_out);
}

extern "C" int32_t cubbs_bbs2023_public_key_from_multibase_v2(uint32_t abi, int32_t form, const char *text,
                                                              size_t len, uint8_t *pk96) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (len && !text) || !pk96 || form < 0 || form > 2)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  const std::string s(text ? text : "", len);
  if (form == 0) return key_from_multibase(s.data(), s.size(), pk96);
  if (form == 2) {  // a verification method: the multibase after '#', else a did:key
    const size_t h = s.find('#');
    if (h != std::string::npos) return key_from_multibase(s.data() + h + 1, s.size() - h - 1, pk96);
  }
  if (s.compare(0, 8, "did:key:") != 0) return CUBBS_BBS2023_ERR_VERIFICATION_METHOD;
  return key_from_multibase(s.data() + 8, s.size() - 8, pk96);
}

// Issue: per item, the header from the proof hash and the mandatory lines,
// Sign of the non-mandatory lines on the device (one batch), then the base
// proofValue.  results[i]: code 0 and bytes_written = text length; an HMAC key
// other than 32 bytes is CUBBS_BBS2023_ERR_HMAC_KEY_LENGTH (prepared.rs:
// 849-854); Sign's own per-item codes otherwise.
extern "C" int32_t cubbs_bbs2023_issue_base_proof_batch_v2(uint32_t abi, CuBbs2023IssueItem *items, size_t n,
                                                           CuBbsBbsGpuResult *results) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (n && (!items || !results))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++) {
    const CuBbs2023IssueItem &it = items[i];
    if (!slices_ok(it.mandatory, it.mandatory_count) || !slices_ok(it.non_mandatory, it.non_mandatory_count) ||
        !slices_ok(it.mandatory_pointers, it.mandatory_pointer_count) || it.proof_hash.len != 32 ||
        !it.proof_hash.data || (it.hmac_key.len && !it.hmac_key.data))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  std::vector<uint8_t> headers(64 * n), sigs(80 * n);
  std::vector<CuBbsBbsGpuSignItem> sign;
  std::vector<size_t> of;
  for (size_t i = 0; i < n; i++) {
    const CuBbs2023IssueItem &it = items[i];
    results[i] = {CUBBS_BBS_GPU_SUCCESS, 0, 0};
    if (it.hmac_key.len != 32) {
      results[i].code = CUBBS_BBS2023_ERR_HMAC_KEY_LENGTH;
      continue;
    }
    header_of(it.proof_hash.data, it.mandatory, it.mandatory_count, &headers[64 * i]);
    CuBbsBbsGpuSignItem s{};
    s.secret_key = it.secret_key;
    s.public_key = it.public_key;
    s.header = {&headers[64 * i], 64};
    s.messages = it.non_mandatory;
    s.message_count = it.non_mandatory_count;
    s.signature_out = {&sigs[80 * i], 80, 0};
    sign.push_back(s);
    of.push_back(i);
  }
  std::vector<CuBbsBbsGpuResult> sr(sign.size());
  if (!sign.empty()) {
    const int32_t rc = cubbs_bbs_gpu_sign_batch_v2(abi, sign.data(), sign.size(), sr.data());
    if (rc) return rc;
  }
  for (size_t k = 0; k < sign.size(); k++) {
    const size_t i = of[k];
    CuBbs2023IssueItem &it = items[i];
    if (sr[k].code != CUBBS_BBS_GPU_SUCCESS) {
      results[i] = sr[k];
      continue;
    }
    CuBbsBbsProofValueBase pv{};
    pv.bbs_signature = {&sigs[80 * i], sign[k].signature_out.len};
    pv.bbs_header = {&headers[64 * i], 64};
    pv.public_key = it.public_key;
    pv.hmac_key = it.hmac_key;
    pv.mandatory_pointers = it.mandatory_pointers;
    pv.mandatory_pointer_count = it.mandatory_pointer_count;
    size_t len = 0;
    const int32_t rc = cubbs_bbs_proofvalue_serialize_base_v2(abi, &pv, reinterpret_cast<char *>(it.proof_value_out.data),
                                                              it.proof_value_out.capacity, &len);
    it.proof_value_out.len = rc == CUBBS_BBS_GPU_SUCCESS ? len : 0;
    results[i] = {rc, 0, len};
  }
  return CUBBS_BBS_GPU_SUCCESS;
}

// Verify a base proof: parse the proofValue, compare its public key and header
// with the item's (a mismatch is value 0, prepared.rs:489-509), then Verify of
// the non-mandatory lines on the device (one batch).  results[i]: code 0 with
// value 1 / 0, or the proofValue codec's error code.
extern "C" int32_t cubbs_bbs2023_verify_base_proof_batch_v2(uint32_t abi, const CuBbs2023VerifyBaseItem *items,
                                                            size_t n, CuBbsBbsGpuResult *results) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (n && (!items || !results))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++) {
    const CuBbs2023VerifyBaseItem &it = items[i];
    if (!slices_ok(it.mandatory, it.mandatory_count) || !slices_ok(it.non_mandatory, it.non_mandatory_count) ||
        it.proof_hash.len != 32 || !it.proof_hash.data || (it.proof_value.len && !it.proof_value.data) ||
        (it.public_key.len && !it.public_key.data))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  std::vector<uint8_t> headers(64 * n);
  std::vector<std::vector<uint8_t>> arenas(n);
  std::vector<CuBbsBbsGpuVerifyItem> ver;
  std::vector<size_t> of;
  for (size_t i = 0; i < n; i++) {
    const CuBbs2023VerifyBaseItem &it = items[i];
    results[i] = {CUBBS_BBS_GPU_SUCCESS, 0, 0};
    CuBbsBbsProofValueBase pv{};
    size_t used = 0;
    arenas[i].resize(it.proof_value.len + 64);
    const int32_t rc = cubbs_bbs_proofvalue_parse_base_v2(abi, reinterpret_cast<const char *>(it.proof_value.data),
                                                          it.proof_value.len, arenas[i].data(), arenas[i].size(), &pv,
                                                          &used);
    if (rc != CUBBS_BBS_GPU_SUCCESS) {
      results[i].code = rc;
      continue;
    }
    header_of(it.proof_hash.data, it.mandatory, it.mandatory_count, &headers[64 * i]);
    if (pv.public_key.len != it.public_key.len ||
        std::memcmp(pv.public_key.data, it.public_key.data, it.public_key.len) != 0 ||
        std::memcmp(pv.bbs_header.data, &headers[64 * i], 64) != 0)
      continue;  // value 0
    CuBbsBbsGpuVerifyItem v{};
    v.public_key = it.public_key;
    v.signature = pv.bbs_signature;
    v.header = {&headers[64 * i], 64};
    v.messages = it.non_mandatory;
    v.message_count = it.non_mandatory_count;
    ver.push_back(v);
    of.push_back(i);
  }
  std::vector<CuBbsBbsGpuResult> vr(ver.size());
  if (!ver.empty()) {
    const int32_t rc = cubbs_bbs_gpu_verify_batch_v2(abi, ver.data(), ver.size(), vr.data());
    if (rc) return rc;
  }
  for (size_t k = 0; k < ver.size(); k++) results[of[k]] = vr[k];
  return CUBBS_BBS_GPU_SUCCESS;
}
