// The two BBS ciphersuites on the device (ciphersuites.rs:49-79):
// suite 0 BLS12-381-SHA-256 (expand_message_xmd over SHA-256, sha256.cuh),
// suite 1 BLS12-381-SHAKE-256 (expand_message_xof over SHAKE-256, keccak.cuh).
// Kernels that hash take the suite as a template parameter S: hash_ctx<S> is
// the expander's streaming state, the msg_* overloads absorb into it and
// SuiteDst<S> (bbs_dst.cuh) holds the suite's strings and P1.
#pragma once
#include "bbs_dst.cuh"
#include "keccak.cuh"
#include "sha256.cuh"

constexpr int SUITE_SHA256 = 0, SUITE_SHAKE256 = 1, SUITE_COUNT = 2;

template <int S> struct HashCtxOf { using type = sha_ctx; };
template <> struct HashCtxOf<SUITE_SHAKE256> { using type = shake_ctx; };
template <int S> using hash_ctx = typename HashCtxOf<S>::type;

template <class C> DEV void msg_fr_be(C &c, const fr &raw) {
  uint8_t b[32];
  fr_raw_to_be32(raw, b);
  msg_bytes(c, b, 32);
}

// hash_to_scalar(msg absorbed into c, api_id || "H2S_")
template <int S> DEV fr h2s_api(hash_ctx<S> &c) { return h2s_finish(c, SuiteDst<S>::dst_h2s(), SuiteDst<S>::dst_h2s_len); }

// Launch helper: calls f(std::integral_constant<int, S>) for the runtime suite.
#define CUBBS_SUITE_DISPATCH(suite, ...)                                  \
  do {                                                                    \
    if ((suite) == SUITE_SHAKE256) {                                      \
      constexpr int S = SUITE_SHAKE256;                                   \
      __VA_ARGS__;                                                        \
    } else {                                                              \
      constexpr int S = SUITE_SHA256;                                     \
      __VA_ARGS__;                                                        \
    }                                                                     \
  } while (0)
