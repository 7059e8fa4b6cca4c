/*
 * CPU oracle for the BBS (BLS12-381-SHA-256) hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain C++ restatement of the
 * reference protocol crate (crates/cubbs-bbs-protocol/src/bbsplus (all .rs files) and
 * utils/util.rs) and of the curve arithmetic it delegates to
 * (bls12_381_plus 0.8.18, elliptic-curve 0.13.8 ExpandMsgXmd, sha2 0.10.9;
 * RFC 9380 hash_to_curve BLS12381G1_XMD:SHA-256_SSWU_RO_).  Only the test
 * suite, the smoke entry and the benchmark's CPU-baseline leg load it, and
 * only as a checker.  The GPU product never links or calls it.
 *
 * Parity is pinned by the CFRG fixture vectors (h2s, map-to-scalar,
 * generators, mocked RNG, keypair, signature001-010, proof001-015) committed
 * under tests/golden/.
 *
 * All functions are reentrant.  Return codes: 0 = ok / valid,
 * 1 = invalid input (decode failure, bad length, out-of-range index),
 * 2 = verification failed (for verify functions), negative = internal error.
 */
#ifndef CUBBS_BBS_ORACLE_H
#define CUBBS_BBS_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

int oracle_sha256(const uint8_t *msg, size_t len, uint8_t out[32]);
int oracle_expand_message_xmd(const uint8_t *msg, size_t len, const uint8_t *dst,
                              size_t dst_len, uint8_t *out, size_t out_len);
int oracle_hash_to_scalar(const uint8_t *msg, size_t len, const uint8_t *dst,
                          size_t dst_len, uint8_t out[32]);
int oracle_keygen(const uint8_t *key_material, size_t km_len, const uint8_t *key_info,
                  size_t ki_len, const uint8_t *key_dst, size_t kd_len, uint8_t sk_out[32]);
int oracle_sk_to_pk(const uint8_t sk[32], uint8_t pk_out[96]);
/* Q1, H1..H_{count-1} compressed (count*48 bytes), plus P1 in p1_out (may be NULL). */
int oracle_generators(size_t count, uint8_t *out, uint8_t *p1_out);
int oracle_hash_to_curve_g1(const uint8_t *msg, size_t len, const uint8_t *dst, size_t dst_len,
                            uint8_t out[48]);
int oracle_seeded_random_scalars(const uint8_t *seed, size_t seed_len, const uint8_t *dst,
                                 size_t dst_len, size_t count, uint8_t *out);

/* Messages are passed packed: msgs = concatenation, lens[i] = length of message i. */
int oracle_sign(const uint8_t sk[32], const uint8_t pk[96], const uint8_t *header, size_t hlen,
                const uint8_t *msgs, const size_t *lens, size_t L, uint8_t sig_out[80],
                uint8_t b_trace[48], uint8_t domain_trace[32]);
int oracle_verify(const uint8_t pk[96], const uint8_t *sig, size_t sig_len, const uint8_t *header,
                  size_t hlen, const uint8_t *msgs, const size_t *lens, size_t L);
/* seed/dst select seeded_random_scalars (spec mocked RNG; chunked past 170 scalars). */
int oracle_proof_gen(const uint8_t pk[96], const uint8_t *sig, size_t sig_len,
                     const uint8_t *header, size_t hlen, const uint8_t *ph, size_t phlen,
                     const uint8_t *msgs, const size_t *lens, size_t L, const size_t *disclosed,
                     size_t R, const uint8_t *seed, size_t seed_len, const uint8_t *dst,
                     size_t dst_len, uint8_t *proof_out, size_t proof_cap, size_t *proof_len);
int oracle_proof_verify(const uint8_t pk[96], const uint8_t *proof, size_t proof_len,
                        const uint8_t *header, size_t hlen, const uint8_t *ph, size_t phlen,
                        const uint8_t *dmsgs, const size_t *dlens, size_t R,
                        const size_t *disclosed);

/* calculate_domain (util.rs:147-189) for L messages */
int oracle_calculate_domain(const uint8_t pk[96], const uint8_t *header, size_t hlen, size_t L,
                            uint8_t out32[32]);
/* Primitive checkers used by kernel-level parity tests. */
int oracle_g1_msm(const uint8_t *points48, const uint8_t *scalars32_be, size_t n, uint8_t out48[48]);
int oracle_g1_add(const uint8_t a48[48], const uint8_t b48[48], uint8_t out48[48]);
/* 0 = valid point in G1, 1 = rejected */
int oracle_g1_decompress(const uint8_t in48[48], uint8_t out_xy_be[96]);
int oracle_g1_mul(const uint8_t p48[48], const uint8_t k32_be[32], uint8_t out48[48]);
int oracle_g2_decompress(const uint8_t in96[96]);
/* e(a, b) == e(c, d): returns 0 if equal, 2 if not, 1 on decode failure */
int oracle_pairing_eq(const uint8_t a48[48], const uint8_t b96[96], const uint8_t c48[48],
                      const uint8_t d96[96]);
int oracle_fp_mul(const uint8_t a48[48], const uint8_t b48[48], uint8_t out48[48]);
int oracle_fr_mul(const uint8_t a32[32], const uint8_t b32[32], uint8_t out32[32]);
int oracle_fr_inv(const uint8_t a32[32], uint8_t out32[32]);

#ifdef __cplusplus
}
#endif
#endif
