/*
 * cubbs_bbs_gpu_abi.h -- C ABI v2 of the GB300 BBS (BLS12-381-SHA-256) library
 * libcubbs_bbs_cuda.so.
 *
 * The structs and entry points keep the exact layout and calling convention
 * of the reference ABI (native/cuda/include/cubbs_bbs_gpu_abi.h:1-314) so the
 * library drops in under the Rust loader (crates/cubbs-bbs/src/gpu_runtime.rs:
 * 269-497), which resolves the four required symbols and probes the optional
 * ones.  Each declaration cites the reference declaration it replaces.
 *
 * Conventions (reference cubbs_bbs_gpu_abi.h:25-59; docs/gpu-bbs-backend-design.md:
 * 145-169):
 *   - every call returns 0 (success), 1 (invalid input), 2 (insufficient
 *     output) or 3 (internal); a call-level error means malformed arguments;
 *   - per-item results[i] = {code, value, bytes_written}; value is the
 *     verification boolean (1/0) or an MSM route id;
 *   - an invalid signature or proof is code 0 with value 0, not an error;
 *   - buffers are caller-owned and must stay valid until the call returns;
 *     every call is synchronous and thread-safe.
 * Encodings: Fr scalars 32-byte big-endian canonical (< r); G1 48-byte and G2
 * 96-byte compressed (zkcrypto / ZCash flag bits); signature A || e (80 B);
 * proof Abar || Bbar || D || e^ || r1^ || r3^ || m^_j... || c.
 *
 * All BBS work runs on the GPU; there is no CPU fallback.
 */
#ifndef CUBBS_BBS_GPU_ABI_H
#define CUBBS_BBS_GPU_ABI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CUBBS_BBS_GPU_ABI_VERSION 2u

/* MSM route ids reported in CuBbsBbsGpuResult.value (reference :13-23).
 * This library uses route 2 for fixed-base (common point) MSMs against the
 * resident generator tables and route 4 for general variable-base MSMs. */
#define CUBBS_BBS_MSM_ROUTE_CUBBS_ITEM 1u
#define CUBBS_BBS_MSM_ROUTE_CUBBS_COMMON_POINTS 2u
#define CUBBS_BBS_MSM_ROUTE_CUBBS_LARGE 3u
#define CUBBS_BBS_MSM_ROUTE_CUBBS_UNIVERSAL 4u
#define CUBBS_BBS_MSM_ROUTE_BLST_ITEM 5u
#define CUBBS_BBS_MSM_ROUTE_BLST_COMMON_POINTS 6u
#define CUBBS_BBS_MSM_ROUTE_SPPARK_ITEM_REFERENCE 7u
#define CUBBS_BBS_MSM_ROUTE_SPPARK_COMMON_POINTS_REFERENCE 8u

#define CUBBS_BBS_GPU_SUCCESS 0
#define CUBBS_BBS_GPU_ERR_INVALID_INPUT 1
#define CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT 2
#define CUBBS_BBS_GPU_ERR_INTERNAL 3

#define CUBBS_BBS_GPU_BACKEND_KIND_UNKNOWN 0u
#define CUBBS_BBS_GPU_BACKEND_KIND_CUDA 1u
#define CUBBS_BBS_GPU_BACKEND_KIND_CPU_ABI_TEST 2u

#define CUBBS_BBS_SECRET_KEY_LEN 32u
#define CUBBS_BBS_PUBLIC_KEY_LEN 96u
#define CUBBS_BBS_SIGNATURE_LEN 80u
#define CUBBS_BBS_2023_HEADER_LEN 64u

/* Byte and index views (reference :34-53). */
typedef struct CuBbsBbsGpuByteSlice {
  const uint8_t *data;
  size_t len;
} CuBbsBbsGpuByteSlice;

typedef struct CuBbsBbsGpuByteBuffer {
  uint8_t *data;
  size_t capacity;
  size_t len;
} CuBbsBbsGpuByteBuffer;

typedef struct CuBbsBbsGpuIndexSlice {
  const size_t *data;
  size_t len;
} CuBbsBbsGpuIndexSlice;

typedef struct CuBbsBbsGpuResult {
  int32_t code;
  uint8_t value;
  size_t bytes_written;
} CuBbsBbsGpuResult;

typedef struct CuBbsBbsGpuBackendInfo {
  uint32_t backend_kind;
  uint8_t hardware_acceleration;
} CuBbsBbsGpuBackendInfo;

/* Four-operation items (reference :66-103). */
typedef struct CuBbsBbsGpuSignItem {
  CuBbsBbsGpuByteSlice secret_key;
  CuBbsBbsGpuByteSlice public_key;
  CuBbsBbsGpuByteSlice header;
  const CuBbsBbsGpuByteSlice *messages;
  size_t message_count;
  CuBbsBbsGpuByteBuffer signature_out;
} CuBbsBbsGpuSignItem;

typedef struct CuBbsBbsGpuVerifyItem {
  CuBbsBbsGpuByteSlice public_key;
  CuBbsBbsGpuByteSlice signature;
  CuBbsBbsGpuByteSlice header;
  const CuBbsBbsGpuByteSlice *messages;
  size_t message_count;
} CuBbsBbsGpuVerifyItem;

typedef struct CuBbsBbsGpuProofGenItem {
  CuBbsBbsGpuByteSlice public_key;
  CuBbsBbsGpuByteSlice signature;
  CuBbsBbsGpuByteSlice header;
  CuBbsBbsGpuByteSlice presentation_header;
  const CuBbsBbsGpuByteSlice *messages;
  size_t message_count;
  CuBbsBbsGpuIndexSlice disclosed_indexes;
  CuBbsBbsGpuByteBuffer proof_out;
} CuBbsBbsGpuProofGenItem;

typedef struct CuBbsBbsGpuProofVerifyItem {
  CuBbsBbsGpuByteSlice public_key;
  CuBbsBbsGpuByteSlice proof;
  CuBbsBbsGpuByteSlice header;
  CuBbsBbsGpuByteSlice presentation_header;
  const CuBbsBbsGpuByteSlice *disclosed_messages;
  size_t disclosed_count;
  CuBbsBbsGpuIndexSlice disclosed_indexes;
  size_t total_message_count;
} CuBbsBbsGpuProofVerifyItem;

/* Primitive items (reference :105-225). */
typedef struct CuBbsBbsGpuMessagesToScalarItem {
  CuBbsBbsGpuByteSlice message;
  CuBbsBbsGpuByteSlice dst;
  CuBbsBbsGpuByteBuffer scalar_out;
} CuBbsBbsGpuMessagesToScalarItem;

typedef struct CuBbsBbsGpuSignEFromResidentScalarsItem {
  CuBbsBbsGpuByteSlice secret_key;
  CuBbsBbsGpuByteSlice domain;
  const CuBbsBbsGpuByteSlice *messages;
  size_t message_scalar_offset;
  size_t message_count;
  CuBbsBbsGpuByteBuffer message_scalars_out;
  CuBbsBbsGpuByteBuffer scalar_out;
} CuBbsBbsGpuSignEFromResidentScalarsItem;

typedef struct CuBbsBbsGpuPrepareBItem {
  CuBbsBbsGpuByteSlice public_key;
  CuBbsBbsGpuByteSlice header;
  const CuBbsBbsGpuByteSlice *message_scalars;
  size_t message_count;
  CuBbsBbsGpuByteBuffer b_out;
} CuBbsBbsGpuPrepareBItem;

typedef struct CuBbsBbsGpuG1MsmItem {
  const CuBbsBbsGpuByteSlice *points;
  const CuBbsBbsGpuByteSlice *scalars;
  size_t term_count;
  CuBbsBbsGpuByteBuffer point_out;
} CuBbsBbsGpuG1MsmItem;

typedef struct CuBbsBbsGpuG1MsmCommonPointsBatchItem {
  const CuBbsBbsGpuByteSlice *points;
  size_t term_count;
  const CuBbsBbsGpuByteSlice *scalar_rows;
  const uint8_t *scalar_rows_be;
  size_t scalar_row_stride;
  size_t output_count;
  CuBbsBbsGpuByteBuffer *point_outs;
} CuBbsBbsGpuG1MsmCommonPointsBatchItem;

typedef struct CuBbsBbsGpuG1MsmCommonPointsPlusVariableItem {
  const CuBbsBbsGpuByteSlice *points;
  size_t term_count;
  const CuBbsBbsGpuByteSlice *scalar_rows;
  const CuBbsBbsGpuByteSlice *variable_points;
  const CuBbsBbsGpuByteSlice *variable_scalars;
  size_t output_count;
  CuBbsBbsGpuByteBuffer *point_outs;
} CuBbsBbsGpuG1MsmCommonPointsPlusVariableItem;

/* T1 = challenge*Bbar + e_cap*Abar + r1_cap*D ;
 * T2 = MSM(common_points, common_scalars) + r3_cap*D ;
 * proof_points rows [Bbar, Abar, D], proof_scalars rows [challenge, e_cap, r1_cap, r3_cap]. */
typedef struct CuBbsBbsGpuProofVerifyMsmPairItem {
  const CuBbsBbsGpuByteSlice *common_points;
  size_t common_term_count;
  const CuBbsBbsGpuByteSlice *common_scalar_rows;
  const CuBbsBbsGpuByteSlice *proof_points;
  const CuBbsBbsGpuByteSlice *proof_scalars;
  size_t output_count;
  CuBbsBbsGpuByteBuffer *t1_outs;
  CuBbsBbsGpuByteBuffer *t2_outs;
} CuBbsBbsGpuProofVerifyMsmPairItem;

typedef struct CuBbsBbsGpuG1DualMsmSamePointsItem {
  const CuBbsBbsGpuByteSlice *points;
  const CuBbsBbsGpuByteSlice *lhs_scalars;
  const CuBbsBbsGpuByteSlice *rhs_scalars;
  size_t term_count;
  CuBbsBbsGpuByteBuffer lhs_out;
  CuBbsBbsGpuByteBuffer rhs_out;
} CuBbsBbsGpuG1DualMsmSamePointsItem;

typedef struct CuBbsBbsGpuG1DualMsmSamePointsLanesItem {
  const CuBbsBbsGpuByteSlice *points;
  const CuBbsBbsGpuByteSlice *lhs_scalars;
  const CuBbsBbsGpuByteSlice *rhs_scalars;
  size_t term_count;
  size_t lane_count;
  CuBbsBbsGpuByteBuffer lhs_outs;
  CuBbsBbsGpuByteBuffer rhs_outs;
} CuBbsBbsGpuG1DualMsmSamePointsLanesItem;

typedef struct CuBbsBbsGpuG1AddItem {
  CuBbsBbsGpuByteSlice lhs;
  CuBbsBbsGpuByteSlice rhs;
  CuBbsBbsGpuByteBuffer point_out;
} CuBbsBbsGpuG1AddItem;

typedef struct CuBbsBbsGpuPairingEqItem {
  CuBbsBbsGpuByteSlice lhs_g1;
  CuBbsBbsGpuByteSlice lhs_g2;
  CuBbsBbsGpuByteSlice rhs_g1;
  CuBbsBbsGpuByteSlice rhs_g2;
} CuBbsBbsGpuPairingEqItem;

typedef struct CuBbsBbsGpuPairingEqScaledItem {
  CuBbsBbsGpuByteSlice lhs_g1;
  CuBbsBbsGpuByteSlice lhs_g2;
  CuBbsBbsGpuByteSlice rhs_g1;
  CuBbsBbsGpuByteSlice rhs_g2;
  CuBbsBbsGpuByteSlice coefficient;
} CuBbsBbsGpuPairingEqScaledItem;

/* d = B*r2, abar = A*(r1 r2), bbar = d*r1 - abar*e, t1 = abar*e~ + d*r1~
 * from 7 host-supplied multipliers r2, r1r2, r1r2, r1r2e, r1r2e~, r2r1~, r3~. */
typedef struct CuBbsBbsGpuProofGenT2PrepareItem {
  CuBbsBbsGpuByteSlice compressed_b;
  CuBbsBbsGpuByteSlice signature_a;
  CuBbsBbsGpuByteSlice scalars_be[7];
  CuBbsBbsGpuByteSlice seed;
  CuBbsBbsGpuByteBuffer d_out;
  CuBbsBbsGpuByteBuffer abar_out;
  CuBbsBbsGpuByteBuffer bbar_out;
  CuBbsBbsGpuByteBuffer t1_out;
} CuBbsBbsGpuProofGenT2PrepareItem;

/* reference :227-228 (the reference always reports hardware_acceleration=0,
 * cubbs_bbs_cuda.cu:822; this library reports 1: the four operations run on
 * the GPU). */
int32_t cubbs_bbs_gpu_backend_info_v2(uint32_t abi_version, CuBbsBbsGpuBackendInfo *info_out);

/* reference :230-247 -- required symbols; stubs in the reference
 * (cubbs_bbs_cuda.cu:826-835,1169-1200), implemented here fully on device. */
int32_t cubbs_bbs_gpu_sign_batch_v2(uint32_t abi_version, CuBbsBbsGpuSignItem *items,
                                    size_t item_count, CuBbsBbsGpuResult *results);
int32_t cubbs_bbs_gpu_verify_batch_v2(uint32_t abi_version, const CuBbsBbsGpuVerifyItem *items,
                                      size_t item_count, CuBbsBbsGpuResult *results);
/* Blinding scalars come from a per-item 32-byte seed drawn from the OS
 * (getrandom) and expanded on the device. */
int32_t cubbs_bbs_gpu_proof_gen_batch_v2(uint32_t abi_version, CuBbsBbsGpuProofGenItem *items,
                                         size_t item_count, CuBbsBbsGpuResult *results);
int32_t cubbs_bbs_gpu_proof_verify_batch_v2(uint32_t abi_version,
                                            const CuBbsBbsGpuProofVerifyItem *items,
                                            size_t item_count, CuBbsBbsGpuResult *results);

/* ABI-compatible addition: ProofGen with caller-chosen blinding.  Item i draws
 * its 5+U scalars with seeded_random_scalars(seed_i, api_id ||
 * "MOCK_RANDOM_SCALARS_DST_") (crates/cubbs-bbs-protocol/src/utils/util.rs:
 * 329-358); with seed "3.141592653589793238462643383279" this reproduces the
 * CFRG proof fixtures.  Past 170 scalars the expansion runs in chunks of 170
 * keyed by seed || I2OSP(chunk, 2). */
int32_t cubbs_bbs_gpu_proof_gen_seeded_batch_v2(uint32_t abi_version,
                                                CuBbsBbsGpuProofGenItem *items, size_t item_count,
                                                const uint8_t (*seeds)[32],
                                                CuBbsBbsGpuResult *results);

/* ABI-compatible addition: the four operations under a chosen ciphersuite.
 * The reference protocol crate defines two (crates/cubbs-bbs-protocol/src/
 * bbsplus/ciphersuites.rs:49-79): Bls12381Sha256 (API_ID
 * "BBS_BLS12381G1_XMD:SHA-256_SSWU_RO_H2G_HM2S_", expand_message_xmd over
 * SHA-256) and Bls12381Shake256 (API_ID
 * "BBS_BLS12381G1_XOF:SHAKE-256_SSWU_RO_H2G_HM2S_", expand_message_xof over
 * SHAKE-256); its C ABI exposes only the first, which the *_batch_v2 entries
 * above keep.  These take the suite as a second argument and the same item
 * structs; an unknown suite is a call-level CUBBS_BBS_GPU_ERR_INVALID_INPUT.
 * Each suite has its own generators (and P1), so keys, signatures and proofs
 * of one suite do not verify under the other.  The seeded ProofGen of the
 * SHAKE-256 suite draws up to 1365 scalars in one expansion (65535 bytes)
 * and chunks past that as above. */
#define CUBBS_BBS_CIPHERSUITE_SHA256 0u
#define CUBBS_BBS_CIPHERSUITE_SHAKE256 1u
int32_t cubbs_bbs_gpu_sign_batch_cs_v2(uint32_t abi_version, uint32_t suite, CuBbsBbsGpuSignItem *items,
                                       size_t item_count, CuBbsBbsGpuResult *results);
int32_t cubbs_bbs_gpu_verify_batch_cs_v2(uint32_t abi_version, uint32_t suite, const CuBbsBbsGpuVerifyItem *items,
                                         size_t item_count, CuBbsBbsGpuResult *results);
int32_t cubbs_bbs_gpu_proof_gen_batch_cs_v2(uint32_t abi_version, uint32_t suite, CuBbsBbsGpuProofGenItem *items,
                                            size_t item_count, CuBbsBbsGpuResult *results);
int32_t cubbs_bbs_gpu_proof_gen_seeded_batch_cs_v2(uint32_t abi_version, uint32_t suite,
                                                   CuBbsBbsGpuProofGenItem *items, size_t item_count,
                                                   const uint8_t (*seeds)[32], CuBbsBbsGpuResult *results);
int32_t cubbs_bbs_gpu_proof_verify_batch_cs_v2(uint32_t abi_version, uint32_t suite,
                                               const CuBbsBbsGpuProofVerifyItem *items, size_t item_count,
                                               CuBbsBbsGpuResult *results);

/* reference :249-251 */
int32_t cubbs_bbs_gpu_messages_to_scalar_batch_v2(uint32_t abi_version,
                                                  CuBbsBbsGpuMessagesToScalarItem *items,
                                                  size_t item_count, CuBbsBbsGpuResult *results);
/* reference :253-256 ("resident" reuses the previous call's device scalars,
 * cubbs_bbs_cuda.cu:523-534) */
int32_t cubbs_bbs_gpu_sign_e_from_resident_scalars_batch_v2(
    uint32_t abi_version, CuBbsBbsGpuSignEFromResidentScalarsItem *items, size_t item_count,
    CuBbsBbsGpuByteSlice message_dst, CuBbsBbsGpuByteSlice e_dst, CuBbsBbsGpuResult *results);
/* reference :258-261 (B = P1 + Q1*domain + sum H_i*m_i, header 64 bytes) */
int32_t cubbs_bbs_gpu_prepare_b_batch_v2(uint32_t abi_version, CuBbsBbsGpuPrepareBItem *items,
                                         size_t item_count, CuBbsBbsGpuResult *results);
/* reference :263-266 */
int32_t cubbs_bbs_gpu_g1_msm_batch_v2(uint32_t abi_version, CuBbsBbsGpuG1MsmItem *items,
                                      size_t item_count, CuBbsBbsGpuResult *results);

/* Addition with no counterpart in the reference: one G1 MSM that allocates
 * nothing.  out = sum_k scalar_k * point_k over term_count terms, given as
 * contiguous 48-byte compressed points and 32-byte big-endian scalars; same
 * result and per-item codes as one item of cubbs_bbs_gpu_g1_msm_batch_v2
 * (result.value = route 4).  Every device buffer is a slice of one fixed
 * scratch array in the library (under 2 MiB, held by every device that loads
 * the library until exit), so the call makes no device or pinned allocation:
 * for callers that must not allocate while they run (a process that has
 * reserved all free device memory up front, code inside an allocator, where
 * an allocation would re-enter it).  Limits: term_count <=
 * CUBBS_BBS_GPU_NOALLOC_MSM_MAX_TERMS, else CUBBS_BBS_GPU_ERR_NOALLOC_LIMIT
 * (returned and in result.code) with no CUDA call made.  The first call on a
 * device does one-time set-up with that device current (looks up the scratch
 * address and loads the kernels it launches).  The call is synchronous (it
 * copies on the legacy default stream and returns with the result on the
 * host): do not make it while any stream capture is active.  All calls share
 * the scratch array, so overlapping calls would race; the library
 * serialises them with a lock. */
#define CUBBS_BBS_GPU_NOALLOC_MSM_MAX_TERMS 4096u
#define CUBBS_BBS_GPU_ERR_NOALLOC_LIMIT 4
int32_t cubbs_bbs_gpu_g1_msm_noalloc_v2(uint32_t abi_version, const uint8_t *points48,
                                        const uint8_t *scalars32, size_t term_count,
                                        uint8_t *point_out48, CuBbsBbsGpuResult *result);
/* Addition with no counterpart in the reference: an uneven batch of G1 MSMs
 * (items as in cubbs_bbs_gpu_g1_msm_batch_v2) and of pairing equality checks
 * (items as in cubbs_bbs_gpu_pairing_eq_batch_v2) evaluated by one persistent
 * launch whose warps take MSM and pairing work from one queue.  Each result
 * array gets what the separate entry point would return. */
int32_t cubbs_bbs_gpu_g1_msm_pairing_batch_v2(uint32_t abi_version, CuBbsBbsGpuG1MsmItem *msm_items,
                                              size_t msm_count, const CuBbsBbsGpuPairingEqItem *pairing_items,
                                              size_t pairing_count, CuBbsBbsGpuResult *msm_results,
                                              CuBbsBbsGpuResult *pairing_results);
/* Addition with no counterpart in the reference C ABI: the W3C bbs-2023
 * proofValue codec of the reference's crates/cubbs-bbs-protocol callers
 * (crates/cubbs-bbs-proofvalue/src/lib.rs:1-220), host code, no GPU work.
 * A proofValue is 'u' || base64url-no-pad(prefix || CBOR payload): prefix
 * d9 5d 02 and [bstr signature(80), bstr header(64), bstr public key(96),
 * bstr hmac key(32), [tstr mandatory pointer...]] for a base proof; prefix
 * d9 5d 03 and [bstr proof, {uint: uint} label map, [uint mandatory index],
 * [uint selective index], bstr presentation header] for a derived proof.  The
 * label map is given in numeric form: label_keys[k] = n of "c14n<n>",
 * label_values[k] = m of "b<m>".  Serialize writes the text to out (cap
 * bytes; *len_out is the length needed); parse copies every field into the
 * caller's arena and points the output struct into it (*arena_used bytes).
 * Returns 0, CUBBS_BBS_GPU_ERR_INVALID_INPUT for malformed arguments,
 * CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT when out or the arena is too small,
 * or one of the CUBBS_BBS_PROOFVALUE_ERR_* codes (the reference's error
 * kinds, lib.rs:17-36). */
#define CUBBS_BBS_PROOFVALUE_ERR_MULTIBASE_PREFIX 10
#define CUBBS_BBS_PROOFVALUE_ERR_CBOR_PREFIX 11
#define CUBBS_BBS_PROOFVALUE_ERR_INVALID_BASE 12
#define CUBBS_BBS_PROOFVALUE_ERR_INVALID_DERIVED 13
#define CUBBS_BBS_PROOFVALUE_ERR_BASE64 14
#define CUBBS_BBS_PROOFVALUE_ERR_CBOR 15
typedef struct CuBbsBbsProofValueBase {
  CuBbsBbsGpuByteSlice bbs_signature;
  CuBbsBbsGpuByteSlice bbs_header;
  CuBbsBbsGpuByteSlice public_key;
  CuBbsBbsGpuByteSlice hmac_key;
  const CuBbsBbsGpuByteSlice *mandatory_pointers;
  size_t mandatory_pointer_count;
} CuBbsBbsProofValueBase;
typedef struct CuBbsBbsProofValueDerived {
  CuBbsBbsGpuByteSlice bbs_proof;
  const uint64_t *label_keys;
  const uint64_t *label_values;
  size_t label_count;
  const uint64_t *mandatory_indexes;
  size_t mandatory_count;
  const uint64_t *selective_indexes;
  size_t selective_count;
  CuBbsBbsGpuByteSlice presentation_header;
} CuBbsBbsProofValueDerived;
int32_t cubbs_bbs_proofvalue_serialize_base_v2(uint32_t abi_version, const CuBbsBbsProofValueBase *value,
                                               char *out, size_t cap, size_t *len_out);
int32_t cubbs_bbs_proofvalue_parse_base_v2(uint32_t abi_version, const char *text, size_t len, uint8_t *arena,
                                           size_t arena_cap, CuBbsBbsProofValueBase *out, size_t *arena_used);
int32_t cubbs_bbs_proofvalue_serialize_derived_v2(uint32_t abi_version, const CuBbsBbsProofValueDerived *value,
                                                  char *out, size_t cap, size_t *len_out);
int32_t cubbs_bbs_proofvalue_parse_derived_v2(uint32_t abi_version, const char *text, size_t len, uint8_t *arena,
                                              size_t arena_cap, CuBbsBbsProofValueDerived *out,
                                              size_t *arena_used);

/* Addition with no counterpart in the reference C ABI: the W3C bbs-2023 input
 * producers between RDF canonicalisation and the BBS operations, host code
 * (crates/cubbs-vc-di-bbs/src/{hashing,hmac_label,canonical,key,prepared}.rs).
 * JSON-LD expansion and RDFC-1.0 canonicalisation come first and are the
 * caller's.  Returns 0, CUBBS_BBS_GPU_ERR_INVALID_INPUT for malformed
 * arguments, CUBBS_BBS_GPU_ERR_INSUFFICIENT_OUTPUT (with the size needed),
 * or one of the codes below (the reference's error kinds). */
#define CUBBS_BBS2023_ERR_HMAC_KEY_LENGTH 20    /* InvalidHmacKeyLength: not 32 bytes */
#define CUBBS_BBS2023_ERR_PUBLIC_KEY_LENGTH 21  /* InvalidPublicKeyLength: not 96 bytes */
#define CUBBS_BBS2023_ERR_MULTIBASE_PREFIX 22   /* InvalidMultibasePrefix: no leading 'z' */
#define CUBBS_BBS2023_ERR_MULTICODEC_HEADER 23  /* InvalidMulticodecHeader: not 0xeb 0x01 */
#define CUBBS_BBS2023_ERR_BASE58 24             /* Base58: not base58btc */
#define CUBBS_BBS2023_ERR_VERIFICATION_METHOD 25 /* InvalidVerificationMethod: no did:key */

/* A blank-node label map entry: input label -> canonical label (c14nN), both
 * without the "_:" prefix. */
typedef struct CuBbsBbs2023LabelEntry {
  CuBbsBbsGpuByteSlice input;
  CuBbsBbsGpuByteSlice canonical;
} CuBbsBbs2023LabelEntry;

/* HMAC-SHA256 (hmac_label.rs:11-16). */
int32_t cubbs_bbs2023_hmac_sha256_v2(uint32_t abi_version, const uint8_t *key, size_t key_len,
                                     const uint8_t *data, size_t len, uint8_t *out32);
/* shuffled_bnode_label_map (hmac_label.rs:26-50): map[k].input gets the label
 * "b" + b_index_out[k], the rank of 'u' || base64url(HMAC(key, canonical)). */
int32_t cubbs_bbs2023_shuffled_label_map_v2(uint32_t abi_version, const CuBbsBbs2023LabelEntry *map,
                                            size_t count, const uint8_t *hmac_key, size_t key_len,
                                            uint32_t *b_index_out);
/* relabel_and_sort_canonical_nquads (canonical.rs:64-92,130-150): each
 * "_:label" of each line is replaced through label_map (entry input -> entry
 * canonical; a label runs to the next Unicode whitespace; labels not in the
 * map stay), and the lines are sorted bytewise.  The new lines are copied to
 * arena (*arena_used bytes) and lines_out[0..line_count) points into it. */
int32_t cubbs_bbs2023_relabel_sort_v2(uint32_t abi_version, const CuBbsBbsGpuByteSlice *lines,
                                      size_t line_count, const CuBbsBbs2023LabelEntry *label_map,
                                      size_t map_count, uint8_t *arena, size_t arena_cap,
                                      CuBbsBbsGpuByteSlice *lines_out, size_t *arena_used);
/* bbs_header (hashing.rs:7-31): SHA-256 of the canonical proof configuration
 * lines joined without separators, then SHA-256 of the mandatory lines. */
int32_t cubbs_bbs2023_header_v2(uint32_t abi_version, const CuBbsBbsGpuByteSlice *proof_lines,
                                size_t proof_count, const CuBbsBbsGpuByteSlice *mandatory,
                                size_t mandatory_count, uint8_t *header64);
/* Multikey forms of a BLS12-381 G2 public key (key.rs:25-80): form 0 the
 * multibase 'z' || base58btc(0xeb 0x01 || key); 1 "did:key:" + multibase;
 * 2 the verification method "did:key:" + multibase + "#" + multibase.
 * Parsing form 2 takes the part after the first '#' when there is one, else
 * a did:key. */
int32_t cubbs_bbs2023_public_key_to_multibase_v2(uint32_t abi_version, int32_t form, const uint8_t *public_key,
                                                 size_t key_len, char *out, size_t cap, size_t *len_out);
int32_t cubbs_bbs2023_public_key_from_multibase_v2(uint32_t abi_version, int32_t form, const char *text,
                                                   size_t len, uint8_t *public_key96);

/* A base proof to issue (IssueBaseProofRequest, prepared.rs:52-60): the BBS
 * messages are the non-mandatory canonical N-Quads, the header is
 * proof_hash || SHA-256(mandatory lines joined); proof_value_out receives the
 * base proofValue text. */
typedef struct CuBbs2023IssueItem {
  CuBbsBbsGpuByteSlice secret_key;
  CuBbsBbsGpuByteSlice public_key;
  CuBbsBbsGpuByteSlice proof_hash; /* 32 bytes */
  const CuBbsBbsGpuByteSlice *mandatory;
  size_t mandatory_count;
  const CuBbsBbsGpuByteSlice *non_mandatory;
  size_t non_mandatory_count;
  CuBbsBbsGpuByteSlice hmac_key; /* 32 bytes */
  const CuBbsBbsGpuByteSlice *mandatory_pointers;
  size_t mandatory_pointer_count;
  CuBbsBbsGpuByteBuffer proof_value_out;
} CuBbs2023IssueItem;
/* A base proof to verify (PreparedBaseVerification, prepared.rs:83-89). */
typedef struct CuBbs2023VerifyBaseItem {
  CuBbsBbsGpuByteSlice public_key;
  CuBbsBbsGpuByteSlice proof_hash; /* 32 bytes */
  const CuBbsBbsGpuByteSlice *mandatory;
  size_t mandatory_count;
  const CuBbsBbsGpuByteSlice *non_mandatory;
  size_t non_mandatory_count;
  CuBbsBbsGpuByteSlice proof_value; /* the proofValue text */
} CuBbs2023VerifyBaseItem;
/* issue_base_proof_batch / verify_base_proof_batch (prepared.rs:335-513) with
 * Sign / Verify as one device batch.  Issue: results[i] = {0, 0, text length},
 * CUBBS_BBS2023_ERR_HMAC_KEY_LENGTH, or Sign's per-item code.  Verify:
 * {0, 1 / 0, 0} (a proofValue whose key or header differs is value 0), or the
 * proofValue codec's error code. */
int32_t cubbs_bbs2023_issue_base_proof_batch_v2(uint32_t abi_version, CuBbs2023IssueItem *items,
                                                size_t item_count, CuBbsBbsGpuResult *results);
int32_t cubbs_bbs2023_verify_base_proof_batch_v2(uint32_t abi_version, const CuBbs2023VerifyBaseItem *items,
                                                 size_t item_count, CuBbsBbsGpuResult *results);

/* reference :268-271 */
int32_t cubbs_bbs_gpu_g1_msm_common_points_batch_v2(uint32_t abi_version,
                                                    CuBbsBbsGpuG1MsmCommonPointsBatchItem *items,
                                                    size_t group_count,
                                                    CuBbsBbsGpuResult *results);
/* reference :273-275 */
int32_t cubbs_bbs_gpu_g1_msm_fused_common_points_batch_v2(
    uint32_t abi_version, CuBbsBbsGpuG1MsmCommonPointsBatchItem *items, size_t group_count,
    CuBbsBbsGpuResult *results);
/* reference :277-280 */
int32_t cubbs_bbs_gpu_g1_msm_common_points_plus_variable_batch_v2(
    uint32_t abi_version, CuBbsBbsGpuG1MsmCommonPointsPlusVariableItem *items, size_t group_count,
    CuBbsBbsGpuResult *results);
/* reference :282-284 */
int32_t cubbs_bbs_gpu_proof_verify_msm_pair_batch_v2(uint32_t abi_version,
                                                     CuBbsBbsGpuProofVerifyMsmPairItem *items,
                                                     size_t group_count,
                                                     CuBbsBbsGpuResult *results);
/* reference :286-288 */
int32_t cubbs_bbs_gpu_g1_dual_msm_same_points_batch_v2(uint32_t abi_version,
                                                       CuBbsBbsGpuG1DualMsmSamePointsItem *items,
                                                       size_t item_count,
                                                       CuBbsBbsGpuResult *results);
/* reference :290-292 */
int32_t cubbs_bbs_gpu_g1_dual_msm_same_points_lanes_batch_v2(
    uint32_t abi_version, CuBbsBbsGpuG1DualMsmSamePointsLanesItem *items, size_t item_count,
    CuBbsBbsGpuResult *results);
/* reference :294-297 */
int32_t cubbs_bbs_gpu_g1_add_batch_v2(uint32_t abi_version, CuBbsBbsGpuG1AddItem *items,
                                      size_t item_count, CuBbsBbsGpuResult *results);
/* reference :299-301: value = e(lhs_g1, lhs_g2) == e(rhs_g1, rhs_g2) */
int32_t cubbs_bbs_gpu_pairing_eq_batch_v2(uint32_t abi_version,
                                          const CuBbsBbsGpuPairingEqItem *items,
                                          size_t item_count, CuBbsBbsGpuResult *results);
/* reference :303-305: one result for the whole batch,
 * value = prod_i (e(lhs_i, lhs2_i) / e(rhs_i, rhs2_i))^{coef_i} == 1 */
int32_t cubbs_bbs_gpu_pairing_eq_aggregate_v2(uint32_t abi_version,
                                              const CuBbsBbsGpuPairingEqScaledItem *items,
                                              size_t item_count, CuBbsBbsGpuResult *result);
/* reference :307-309 */
int32_t cubbs_bbs_gpu_proof_gen_t2_prepare_batch_v2(uint32_t abi_version,
                                                    CuBbsBbsGpuProofGenT2PrepareItem *items,
                                                    size_t item_count,
                                                    CuBbsBbsGpuResult *results);

/* Serving queue (no counterpart in the reference ABI): continuous batching of
 * single requests of the four operations.  Up to max_inflight batches run at
 * once on separate device workspaces; a free slot takes the operation whose
 * oldest request waited longest, as many of its requests as fit in
 * max_batch_items and in the device-memory budget left by the running batches.
 * Items and their buffers are caller-owned and must stay alive until the
 * request's wait returns.  op: 0 Sign, 1 Verify, 2 ProofGen, 3 ProofVerify
 * under BLS12-381-SHA-256, 4..7 the same under BLS12-381-SHAKE-256 (op & 3 is
 * the operation, op >> 2 the CUBBS_BBS_CIPHERSUITE_* value), each its own
 * queue; seed32 (ProofGen only, nullable) selects seeded blinding as in
 * cubbs_bbs_gpu_proof_gen_seeded_batch_v2, else OS randomness.  The result of
 * a request equals the result of the same request in a batch of its own. */
typedef struct CuBbsBbsGpuServeConfig {
  uint32_t max_inflight;     /* 0: one per device workspace (CUBBS_BBS_WORKSPACES, default 4) */
  uint32_t max_batch_items;  /* 0: 1024 */
  uint64_t hbm_budget_bytes; /* device bytes admitted across running batches; 0: 1 GiB */
} CuBbsBbsGpuServeConfig;

int32_t cubbs_bbs_gpu_serve_create(uint32_t abi_version, const CuBbsBbsGpuServeConfig *config,
                                   void **server);
int32_t cubbs_bbs_gpu_serve_submit(void *server, int32_t op, void *item, const uint8_t *seed32,
                                   uint64_t *ticket);
int32_t cubbs_bbs_gpu_serve_wait(void *server, uint64_t ticket, CuBbsBbsGpuResult *result);
/* Stops taking requests, serves every request still queued (their waits and
 * callbacks complete), then frees the server. */
int32_t cubbs_bbs_gpu_serve_destroy(void *server);

/* Batcher settings of one queue, the per-operation BatcherConfig of the
 * reference W3C service (crates/cubbs-w3c-service/src/batcher.rs:21-60):
 *   max_batch_items <- max_batch_size (0: the server's max_batch_items);
 *   max_inflight    <- pipelines, running batches of this queue, under the
 *                      server's max_inflight slots shared by all queues
 *                      (spawn_with_slots, batcher.rs:142-167) (0: no limit);
 *   coalesce_us     <- interval_ms * 1000: a free slot that finds a partial
 *                      batch waits up to this long for it to fill; a full
 *                      batch leaves at once (batcher.rs:254-268) (0: none);
 *   queue_capacity  <- queue_capacity: submit waits while the queue holds
 *                      this many requests, like the batcher's bounded channel
 *                      (0: unbounded).
 * A new server's queues have {server max_batch_items, 0, 0, 0}. */
#define CUBBS_BBS_GPU_SERVE_MAX_QUEUES 8
typedef struct CuBbsBbsGpuServeQueueConfig {
  uint32_t max_batch_items;
  uint32_t max_inflight;
  uint32_t coalesce_us;
  uint32_t queue_capacity;
} CuBbsBbsGpuServeQueueConfig;

/* BatcherSnapshot (batcher.rs:86-97) of one queue, or of all with queue -1:
 * queued = submitted and not yet dispatched; last_batch_size of all queues is
 * the most recent dispatch of any queue; queue wait = submit to dispatch. */
typedef struct CuBbsBbsGpuServeSnapshot {
  uint64_t queued;
  uint64_t dispatches;
  uint64_t dispatched_items;
  uint64_t max_observed_batch;
  uint64_t last_batch_size;
  uint64_t inflight_batches;
  double total_queue_wait_ms;
  double average_queue_wait_ms;
} CuBbsBbsGpuServeSnapshot;

/* Completion callback of cubbs_bbs_gpu_serve_submit_notify, called once per
 * request on a dispatch thread, outside the server's lock (it may submit
 * again); *result is valid only during the call. */
typedef void (*CuBbsBbsGpuServeDone)(void *ctx, uint64_t ticket, const CuBbsBbsGpuResult *result);
/* Batch processor of a server made by cubbs_bbs_gpu_serve_create_with_processor:
 * processes items[0..count) of one queue and fills results[0..count); a
 * nonzero return fails every request of the batch with that code. */
typedef int32_t (*CuBbsBbsGpuServeProcessor)(void *ctx, int32_t queue, void *const *items, size_t count,
                                             CuBbsBbsGpuResult *results);

/* queue selects the operation queue (as op above); config NULL only reads the
 * settings in force into *effective (nullable), which mirrors
 * BatchQueue::config (batcher.rs:196-198). */
int32_t cubbs_bbs_gpu_serve_configure_queue(void *server, int32_t queue,
                                            const CuBbsBbsGpuServeQueueConfig *config,
                                            CuBbsBbsGpuServeQueueConfig *effective);
/* Like cubbs_bbs_gpu_serve_submit, but the result is delivered to done(ctx,
 * ticket, result) instead of a wait (BatchQueue::enqueue and its oneshot
 * reply, batcher.rs:171-190).  *ticket (nullable) is set before return; the
 * ticket is not waitable. */
int32_t cubbs_bbs_gpu_serve_submit_notify(void *server, int32_t op, void *item, const uint8_t *seed32,
                                          CuBbsBbsGpuServeDone done, void *ctx, uint64_t *ticket);
/* batch_size_counts[k] (k < counts_len; nullable when counts_len is 0) =
 * batches of k requests dispatched, as BatcherSnapshot::batch_size_counts. */
int32_t cubbs_bbs_gpu_serve_snapshot(void *server, int32_t queue, CuBbsBbsGpuServeSnapshot *out,
                                     uint64_t *batch_size_counts, size_t counts_len);
/* A server whose batches go to `processor` instead of the device: the
 * reference's BatchQueue::spawn(config, processor) (batcher.rs:130-140) for
 * callers that batch their own items (the service's JSON-LD stages).  Queues
 * 0..CUBBS_BBS_GPU_SERVE_MAX_QUEUES-1; no device-memory admission; max_inflight
 * 0 means 1.  No CUDA call is made on this server's behalf. */
int32_t cubbs_bbs_gpu_serve_create_with_processor(uint32_t abi_version,
                                                  const CuBbsBbsGpuServeConfig *config,
                                                  CuBbsBbsGpuServeProcessor processor, void *ctx,
                                                  void **server);
/* Load replay for benchmarks and tests: request i arrives arrival_ns[i] after
 * the start (non-decreasing); mode 0 serves through the queue, mode 1 through
 * plain fixed-size batches (plain_batch requests, flushed after
 * plain_timeout_us, one batch at a time).  latency_ns[i] = completion minus
 * scheduled arrival; wall_s = start to last completion. */
int32_t cubbs_bbs_gpu_serve_replay(uint32_t abi_version, int32_t mode,
                                   const CuBbsBbsGpuServeConfig *config, const int32_t *ops,
                                   void *const *items, const uint8_t (*seeds)[32],
                                   const uint64_t *arrival_ns, size_t count, uint32_t plain_batch,
                                   uint32_t plain_timeout_us, uint64_t *latency_ns,
                                   CuBbsBbsGpuResult *results, double *wall_s);

/* Test exports outside the reference header (reference cubbs_bbs_cuda.cu:53,117,230). */
int32_t cubbs_bbs_gpu_sha256_batch_for_test_v2(uint32_t abi_version, const uint8_t *messages,
                                               const size_t *offsets, const size_t *lengths,
                                               size_t item_count, uint8_t *digests);
int32_t cubbs_bbs_gpu_expand_xmd_sha256_48_batch_for_test_v2(
    uint32_t abi_version, const uint8_t *messages, const size_t *offsets, const size_t *lengths,
    size_t item_count, const uint8_t *dst, size_t dst_len, uint8_t *outputs);
int32_t cubbs_bbs_gpu_hash_to_scalar_sha256_batch_for_test_v2(
    uint32_t abi_version, const uint8_t *messages, const size_t *offsets, const size_t *lengths,
    size_t item_count, const uint8_t *dst, size_t dst_len, uint8_t *scalars);

#ifdef __cplusplus
}
#endif

#endif
