// W3C bbs-2023 proofValue wire format (host code): the multibase
// base64url-no-pad string 'u' || base64url(prefix || CBOR(payload)) of a base
// proof (prefix d9 5d 02) or a derived proof (prefix d9 5d 03).  Restates the
// codec of crates/cubbs-bbs-proofvalue/src/lib.rs:1-220:
//   base payload    = [bstr signature(80), bstr header(64), bstr public key(96),
//                      bstr hmac key(32), [tstr mandatory pointer, ...]]
//   derived payload = [bstr proof (non-empty), {uint c14n label: uint b label},
//                      [uint mandatory index], [uint selective index],
//                      bstr presentation header]
// Encoding follows the reference's serializer (serde_cbor): definite lengths,
// every length and integer in its shortest form, the label map in ascending
// key order.  Decoding takes definite-length items with any integer width,
// rejects trailing bytes, and keeps the last value of a repeated map key.
// The label map crosses the C boundary in its compressed numeric form
// (c14n<k> -> b<v> as k -> v, lib.rs:177-206).
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/cubbs_bbs_gpu_abi.h"

namespace {

const uint8_t PREFIX_BASE[3] = {0xd9, 0x5d, 0x02};
const uint8_t PREFIX_DERIVED[3] = {0xd9, 0x5d, 0x03};

// ------------------------------------------------------------------ CBOR writer
void put_head(std::vector<uint8_t> &o, int major, uint64_t v) {
  const uint8_t m = (uint8_t)(major << 5);
  if (v < 24) {
    o.push_back(m | (uint8_t)v);
  } else if (v <= 0xff) {
    o.push_back(m | 24);
    o.push_back((uint8_t)v);
  } else if (v <= 0xffff) {
    o.push_back(m | 25);
    for (int s = 8; s >= 0; s -= 8) o.push_back((uint8_t)(v >> s));
  } else if (v <= 0xffffffffull) {
    o.push_back(m | 26);
    for (int s = 24; s >= 0; s -= 8) o.push_back((uint8_t)(v >> s));
  } else {
    o.push_back(m | 27);
    for (int s = 56; s >= 0; s -= 8) o.push_back((uint8_t)(v >> s));
  }
}
void put_bytes(std::vector<uint8_t> &o, int major, const uint8_t *p, size_t n) {
  put_head(o, major, n);
  if (n) o.insert(o.end(), p, p + n);
}

// RFC 3629 UTF-8 (a text string must hold it, as the reference's String does).
bool utf8_ok(const std::string &s) {
  size_t i = 0;
  const size_t n = s.size();
  while (i < n) {
    const uint8_t c = (uint8_t)s[i];
    int len = c < 0x80 ? 1 : (c >> 5) == 6 ? 2 : (c >> 4) == 14 ? 3 : (c >> 3) == 30 ? 4 : 0;
    if (!len || i + len > n) return false;
    uint32_t cp = len == 1 ? c : len == 2 ? (c & 0x1f) : len == 3 ? (c & 0x0f) : (c & 0x07);
    for (int k = 1; k < len; k++) {
      const uint8_t d = (uint8_t)s[i + k];
      if ((d >> 6) != 2) return false;
      cp = cp << 6 | (d & 0x3f);
    }
    const uint32_t min[5] = {0, 0, 0x80, 0x800, 0x10000};
    if (cp < min[len] || cp > 0x10ffff || (cp >= 0xd800 && cp <= 0xdfff)) return false;
    i += len;
  }
  return true;
}

// ------------------------------------------------------------------ CBOR reader
struct Reader {
  const uint8_t *p;
  size_t n, at = 0;
  bool ok = true;
  // head of the next item: major type and argument (definite lengths only)
  bool head(int &major, uint64_t &v) {
    if (at >= n) return ok = false;
    const uint8_t b = p[at++];
    major = b >> 5;
    const int ai = b & 31;
    if (ai < 24) {
      v = (uint64_t)ai;
      return true;
    }
    const int len = ai == 24 ? 1 : ai == 25 ? 2 : ai == 26 ? 4 : ai == 27 ? 8 : 0;
    if (!len || at + len > n) return ok = false;  // indefinite lengths and reserved values
    v = 0;
    for (int k = 0; k < len; k++) v = v << 8 | p[at++];
    return true;
  }
  bool expect(int major, uint64_t &v) {
    int m;
    if (!head(m, v) || m != major) return ok = false;
    return true;
  }
  bool bytes(int major, std::string &out) {
    uint64_t len;
    if (!expect(major, len) || len > n - at) return ok = false;
    out.assign(reinterpret_cast<const char *>(p + at), (size_t)len);
    at += (size_t)len;
    if (major == 3 && !utf8_ok(out)) return ok = false;
    return true;
  }
  bool uint_array(std::vector<uint64_t> &out) {
    uint64_t cnt;
    if (!expect(4, cnt) || cnt > n - at) return ok = false;
    out.clear();
    for (uint64_t k = 0; k < cnt; k++) {
      uint64_t v;
      if (!expect(0, v)) return false;
      out.push_back(v);
    }
    return true;
  }
};

// ------------------------------------------------------------------ base64url, no padding
const char B64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789-_";
std::string b64url(const std::vector<uint8_t> &in) {
  std::string o;
  size_t i = 0;
  for (; i + 3 <= in.size(); i += 3) {
    const uint32_t v = (uint32_t)in[i] << 16 | (uint32_t)in[i + 1] << 8 | in[i + 2];
    for (int s = 18; s >= 0; s -= 6) o.push_back(B64[(v >> s) & 63]);
  }
  const size_t rest = in.size() - i;
  if (rest == 1) {
    const uint32_t v = (uint32_t)in[i] << 16;
    o.push_back(B64[(v >> 18) & 63]);
    o.push_back(B64[(v >> 12) & 63]);
  } else if (rest == 2) {
    const uint32_t v = (uint32_t)in[i] << 16 | (uint32_t)in[i + 1] << 8;
    o.push_back(B64[(v >> 18) & 63]);
    o.push_back(B64[(v >> 12) & 63]);
    o.push_back(B64[(v >> 6) & 63]);
  }
  return o;
}
int b64val(char c) {
  if (c >= 'A' && c <= 'Z') return c - 'A';
  if (c >= 'a' && c <= 'z') return c - 'a' + 26;
  if (c >= '0' && c <= '9') return c - '0' + 52;
  if (c == '-') return 62;
  if (c == '_') return 63;
  return -1;
}
// Strict: the URL-safe alphabet, no padding, no length of 1 mod 4, and zero
// bits after the last byte.
bool unb64url(const char *s, size_t n, std::vector<uint8_t> &out) {
  if (n % 4 == 1) return false;
  out.clear();
  uint32_t acc = 0;
  int bits = 0;
  for (size_t i = 0; i < n; i++) {
    const int v = b64val(s[i]);
    if (v < 0) return false;
    acc = acc << 6 | (uint32_t)v;
    bits += 6;
    if (bits >= 8) {
      bits -= 8;
      out.push_back((uint8_t)(acc >> bits));
      acc &= (1u << bits) - 1;
    }
  }
  return acc == 0;
}

int32_t finish_text(const std::vector<uint8_t> &bytes, char *out, size_t cap, size_t *len_out) {
  const std::string t = "u" + b64url(bytes);
  *len_out = t.size();
  if (cap < t.size()) return CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT;
  std::memcpy(out, t.data(), t.size());
  return CUBBS_BBS_GPU_SUCCESS;
}

int32_t decode_text(const char *text, size_t len, const uint8_t prefix[3], std::vector<uint8_t> &payload) {
  if (len == 0 || text[0] != 'u') return CUBBS_BBS_PROOFVALUE_ERR_MULTIBASE_PREFIX;
  std::vector<uint8_t> raw;
  if (!unb64url(text + 1, len - 1, raw)) return CUBBS_BBS_PROOFVALUE_ERR_BASE64;
  if (raw.size() < 3 || std::memcmp(raw.data(), prefix, 3) != 0) return CUBBS_BBS_PROOFVALUE_ERR_CBOR_PREFIX;
  payload.assign(raw.begin() + 3, raw.end());
  return CUBBS_BBS_GPU_SUCCESS;
}

// Bump allocation of parse outputs in the caller's arena.
struct Arena {
  uint8_t *base;
  size_t cap, used = 0;
  bool ok = true;
  void *take(size_t bytes, size_t align) {
    const size_t at = (used + align - 1) & ~(align - 1);
    if (at + bytes > cap) {
      ok = false;
      return nullptr;
    }
    used = at + bytes;
    return base + at;
  }
  CuBbsBbsGpuByteSlice copy(const std::string &s) {
    uint8_t *d = static_cast<uint8_t *>(take(s.size() ? s.size() : 1, 1));
    if (!d) return {nullptr, 0};
    if (!s.empty()) std::memcpy(d, s.data(), s.size());
    return {d, s.size()};
  }
  const uint64_t *copy(const std::vector<uint64_t> &v) {
    uint64_t *d = static_cast<uint64_t *>(take(8 * (v.size() ? v.size() : 1), 8));
    if (d && !v.empty()) std::memcpy(d, v.data(), 8 * v.size());
    return d;
  }
};

bool slice_ok(const CuBbsBbsGpuByteSlice &s) { return s.len == 0 || s.data != nullptr; }

}  // namespace

extern "C" int32_t cubbs_bbs_proofvalue_serialize_base_v2(uint32_t abi, const CuBbsBbsProofValueBase *in, char *out,
                                                          size_t cap, size_t *len_out) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || !in || !len_out || (cap && !out) || !slice_ok(in->bbs_signature) ||
      !slice_ok(in->bbs_header) || !slice_ok(in->public_key) || !slice_ok(in->hmac_key) ||
      (in->mandatory_pointer_count && !in->mandatory_pointers))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t k = 0; k < in->mandatory_pointer_count; k++)
    if (!slice_ok(in->mandatory_pointers[k])) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (in->bbs_signature.len != 80 || in->bbs_header.len != 64 || in->public_key.len != 96 || in->hmac_key.len != 32)
    return CUBBS_BBS_PROOFVALUE_ERR_INVALID_BASE;
  std::vector<uint8_t> b(PREFIX_BASE, PREFIX_BASE + 3);
  put_head(b, 4, 5);
  for (const CuBbsBbsGpuByteSlice *s : {&in->bbs_signature, &in->bbs_header, &in->public_key, &in->hmac_key})
    put_bytes(b, 2, s->data, s->len);
  put_head(b, 4, in->mandatory_pointer_count);
  for (size_t k = 0; k < in->mandatory_pointer_count; k++)
    put_bytes(b, 3, in->mandatory_pointers[k].data, in->mandatory_pointers[k].len);
  return finish_text(b, out, cap, len_out);
}

extern "C" int32_t cubbs_bbs_proofvalue_parse_base_v2(uint32_t abi, const char *text, size_t len, uint8_t *arena,
                                                      size_t arena_cap, CuBbsBbsProofValueBase *out,
                                                      size_t *arena_used) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (len && !text) || (arena_cap && !arena) || !out || !arena_used)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  std::vector<uint8_t> payload;
  int32_t st = decode_text(text, len, PREFIX_BASE, payload);
  if (st) return st;
  Reader r{payload.data(), payload.size()};
  uint64_t cnt = 0;
  std::string f[4];
  std::vector<std::string> ptrs;
  if (r.expect(4, cnt) && cnt == 5) {
    for (auto &x : f) r.bytes(2, x);
    uint64_t np = 0;
    if (r.ok && r.expect(4, np) && np <= payload.size()) {
      for (uint64_t k = 0; k < np && r.ok; k++) {
        std::string s;
        if (r.bytes(3, s)) ptrs.push_back(s);
      }
    }
  } else {
    r.ok = false;
  }
  if (!r.ok || r.at != payload.size()) return CUBBS_BBS_PROOFVALUE_ERR_CBOR;
  if (f[0].size() != 80 || f[1].size() != 64 || f[2].size() != 96 || f[3].size() != 32)
    return CUBBS_BBS_PROOFVALUE_ERR_INVALID_BASE;
  Arena a{arena, arena_cap};
  out->bbs_signature = a.copy(f[0]);
  out->bbs_header = a.copy(f[1]);
  out->public_key = a.copy(f[2]);
  out->hmac_key = a.copy(f[3]);
  auto *list = static_cast<CuBbsBbsGpuByteSlice *>(
      a.take(sizeof(CuBbsBbsGpuByteSlice) * (ptrs.size() ? ptrs.size() : 1), alignof(CuBbsBbsGpuByteSlice)));
  for (size_t k = 0; k < ptrs.size() && list; k++) list[k] = a.copy(ptrs[k]);
  out->mandatory_pointers = list;
  out->mandatory_pointer_count = ptrs.size();
  *arena_used = a.used;
  return a.ok ? CUBBS_BBS_GPU_SUCCESS : CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT;
}

extern "C" int32_t cubbs_bbs_proofvalue_serialize_derived_v2(uint32_t abi, const CuBbsBbsProofValueDerived *in,
                                                             char *out, size_t cap, size_t *len_out) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || !in || !len_out || (cap && !out) || !slice_ok(in->bbs_proof) ||
      !slice_ok(in->presentation_header) || (in->label_count && (!in->label_keys || !in->label_values)) ||
      (in->mandatory_count && !in->mandatory_indexes) || (in->selective_count && !in->selective_indexes))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (in->bbs_proof.len == 0) return CUBBS_BBS_PROOFVALUE_ERR_INVALID_DERIVED;
  // the label map as the reference holds it: ascending keys, one value each
  std::map<uint64_t, uint64_t> labels;
  for (size_t k = 0; k < in->label_count; k++) labels[in->label_keys[k]] = in->label_values[k];
  if (labels.size() != in->label_count) return CUBBS_BBS_PROOFVALUE_ERR_INVALID_DERIVED;  // repeated c14n label
  std::vector<uint8_t> b(PREFIX_DERIVED, PREFIX_DERIVED + 3);
  put_head(b, 4, 5);
  put_bytes(b, 2, in->bbs_proof.data, in->bbs_proof.len);
  put_head(b, 5, labels.size());
  for (const auto &kv : labels) {
    put_head(b, 0, kv.first);
    put_head(b, 0, kv.second);
  }
  put_head(b, 4, in->mandatory_count);
  for (size_t k = 0; k < in->mandatory_count; k++) put_head(b, 0, in->mandatory_indexes[k]);
  put_head(b, 4, in->selective_count);
  for (size_t k = 0; k < in->selective_count; k++) put_head(b, 0, in->selective_indexes[k]);
  put_bytes(b, 2, in->presentation_header.data, in->presentation_header.len);
  return finish_text(b, out, cap, len_out);
}

extern "C" int32_t cubbs_bbs_proofvalue_parse_derived_v2(uint32_t abi, const char *text, size_t len, uint8_t *arena,
                                                         size_t arena_cap, CuBbsBbsProofValueDerived *out,
                                                         size_t *arena_used) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || (len && !text) || (arena_cap && !arena) || !out || !arena_used)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  std::vector<uint8_t> payload;
  int32_t st = decode_text(text, len, PREFIX_DERIVED, payload);
  if (st) return st;
  Reader r{payload.data(), payload.size()};
  uint64_t cnt = 0;
  std::string proof, ph;
  std::map<uint64_t, uint64_t> labels;
  std::vector<uint64_t> mand, sel;
  if (r.expect(4, cnt) && cnt == 5) {
    r.bytes(2, proof);
    uint64_t nl = 0;
    if (r.ok && r.expect(5, nl) && nl <= payload.size()) {
      for (uint64_t k = 0; k < nl && r.ok; k++) {
        uint64_t key, val;
        if (r.expect(0, key) && r.expect(0, val)) labels[key] = val;  // a repeated key keeps its last value
      }
    }
    if (r.ok) r.uint_array(mand);
    if (r.ok) r.uint_array(sel);
    if (r.ok) r.bytes(2, ph);
  } else {
    r.ok = false;
  }
  if (!r.ok || r.at != payload.size()) return CUBBS_BBS_PROOFVALUE_ERR_CBOR;
  if (proof.empty()) return CUBBS_BBS_PROOFVALUE_ERR_INVALID_DERIVED;
  Arena a{arena, arena_cap};
  out->bbs_proof = a.copy(proof);
  std::vector<uint64_t> keys, vals;
  for (const auto &kv : labels) {
    keys.push_back(kv.first);
    vals.push_back(kv.second);
  }
  out->label_keys = a.copy(keys);
  out->label_values = a.copy(vals);
  out->label_count = keys.size();
  out->mandatory_indexes = a.copy(mand);
  out->mandatory_count = mand.size();
  out->selective_indexes = a.copy(sel);
  out->selective_count = sel.size();
  out->presentation_header = a.copy(ph);
  *arena_used = a.used;
  return a.ok ? CUBBS_BBS_GPU_SUCCESS : CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT;
}
