/*
 * cubbs_bbs_gpu_test.h -- test, benchmark and tuning exports of
 * libcubbs_bbs_cuda.so that are not part of the drop-in ABI.
 *
 * None of these has a counterpart in the reference header: the Rust loader
 * never binds them.  The parity tests, the benchmark and the profiling runs
 * call them (through ctypes); a production caller needs only
 * cubbs_bbs_gpu_abi.h.  They follow the same conventions: 0 success,
 * 1 invalid input, 3 internal error; synchronous; thread-safe.
 */
#ifndef CUBBS_BBS_GPU_TEST_H
#define CUBBS_BBS_GPU_TEST_H

#include "cubbs_bbs_gpu_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- tuning and state queries */

/* Window width of the resident fixed-base table (0 before the first table). */
int32_t cubbs_bbs_gpu_table_window_v2(int32_t *w);

/* SM counts of the ProofVerify partition and why it is off (status 0: on;
 * 1: turned off; 2: off under an injected profiler; 200 + k: driver entry
 * point k missing; else 1000 * failed step + driver result).  Makes the
 * partition on first use. */
int32_t cubbs_bbs_gpu_sm_partition_v2(int32_t *small_sms, int32_t *rest_sms, int32_t *status);

/* SMs of the third ProofVerify partition (point decode and variable-base
 * terms), split off rest_sms; 0 when off (CUBBS_BBS_VAR_SMS=0 or refused),
 * with the reason in *status (0: on; 1: not asked for; -1: no partition;
 * else failed step * 1000 + driver result). */
int32_t cubbs_bbs_gpu_sm_partition_var_v2(int32_t *var_sms, int32_t *status);

/* Fixed-base table width sweep w_lo..w_hi (4..20) over rows x terms scalars
 * against the first `terms` generators [P1, Q1, H1, ...]: each width's first
 * 64 rows are compared with a table-free recomputation (ms_per_w = -1 and
 * *mismatched counts the width when they differ); the fastest agreeing width
 * stays in use (*best_w).  A width whose table does not fit the table budget
 * is narrowed to one that does (the table in use then reports the width). */
int32_t cubbs_bbs_gpu_fixed_msm_autotune_v2(uint32_t abi_version, const uint8_t *scalars_be, size_t rows,
                                            size_t terms, int32_t w_lo, int32_t w_hi, int32_t steps,
                                            float *ms_per_w, int32_t *best_w, int32_t *mismatched);

/* Uneven-MSM engine settings per size class (K <= 8, <= 32, <= 96, larger):
 * mode (0: thread per chunk of `chunk` terms, window 4..7; 1: warp per MSM,
 * window 4..12), chunk length and window width; non-null inputs replace them,
 * non-null outputs receive the settings in force. */
int32_t cubbs_bbs_gpu_msm_tuning_v2(const uint32_t *chunk_in, const uint32_t *window_in, const uint32_t *mode_in,
                                    uint32_t *chunk_out, uint32_t *window_out, uint32_t *mode_out);

/* ---- benchmarks */

/* Uneven variable-base MSM benchmark: n_msms MSMs with K ~ U{k_min..k_max}
 * generated on the device from `seed`; optional autotuning (tuning_out: 12
 * values, chunk / window / mode per size class); CUDA-graph replays
 * (ms_out[steps]); decode cost; the first 64 MSMs rechecked. */
int32_t cubbs_bbs_gpu_msm_uneven_bench_v2(uint32_t abi_version, size_t n_msms, uint32_t k_min, uint32_t k_max,
                                         uint64_t seed, int32_t tune, int32_t warmup, int32_t steps, float *ms_out,
                                         float *decode_ms, uint32_t *tuning_out, uint32_t *checked,
                                         uint32_t *mismatch);

/* One operation's batch (op 0..3: Sign, Verify, ProofGen, ProofVerify) packed
 * and uploaded once, then its device pipeline timed warmup + steps times
 * (ms_out[steps], CUDA events, L2 flushed between steps). */
int32_t cubbs_bbs_gpu_bench_device_steps_v2(uint32_t abi_version, int32_t op, void *items, size_t n,
                                            const uint8_t (*seeds)[32], int32_t warmup, int32_t steps,
                                            float *ms_out, int32_t *launches, CuBbsBbsGpuResult *results);

/* Per-kernel spans of the last timed step (names32: cap x 32-byte names). */
int32_t cubbs_bbs_gpu_bench_stages_v2(char *names32, float *ms, int32_t cap);

/* Bytes copied host-to-device and device-to-host by the calling thread's last call. */
int32_t cubbs_bbs_gpu_last_transfer_bytes_v2(uint64_t *h2d, uint64_t *d2h);

/* Measured integer peaks: T IMAD/s (independent mad.lo chains) and G Fp products/s. */
int32_t cubbs_bbs_gpu_int_peaks_v2(double *tera_imad, double *giga_fpmul);

/* ---- probes (SM cycles of single programs) */
int32_t cubbs_bbs_gpu_latency_probe_for_test_v2(double *cycles, int32_t cap);
int32_t cubbs_bbs_gpu_pairing_probe_for_test_v2(double *cycles, int32_t cap);
/* the same for two-warp teams (the 64-lane phase tables) */
int32_t cubbs_bbs_gpu_pairing_probe_wide_for_test_v2(double *cycles, int32_t cap);
int32_t cubbs_bbs_gpu_fpmul_rates_for_test_v2(const int32_t *warps_per_sm, int32_t n, double *rates);

/* ---- arithmetic test exports (compared with the oracle by the tests) */
int32_t cubbs_bbs_gpu_fp_op_for_test_v2(uint32_t abi_version, int32_t op, const uint8_t *a, const uint8_t *b,
                                        size_t n, uint8_t *out, int32_t *status);
int32_t cubbs_bbs_gpu_g1_op_for_test_v2(uint32_t abi_version, const uint8_t *pts48, const uint8_t *k32, size_t n,
                                        uint8_t *xy96, uint8_t *kp48, int32_t *status);
int32_t cubbs_bbs_gpu_g1_subgroup_for_test_v2(uint32_t abi_version, const uint8_t *pts48, size_t n,
                                              int32_t *status, int32_t *outside);
int32_t cubbs_bbs_gpu_h2s_scalars_for_test_v2(uint32_t abi_version, const uint8_t *be, size_t n, uint8_t *out32);
int32_t cubbs_bbs_gpu_pairs_h2s_for_test_v2(uint32_t abi_version, const uint8_t *blob, size_t blob_len,
                                            uint32_t idx_off, uint32_t R, const uint8_t *mbe, uint8_t *out32,
                                            uint32_t *echo);
int32_t cubbs_bbs_gpu_last_debug_record_for_test_v2(uint8_t *out256);
/* expand_message_xof over SHAKE-256 (48 bytes per message) and hash_to_scalar
 * over it (the SHAKE-256 suite's expander), one message per thread. */
int32_t cubbs_bbs_gpu_expand_xof_shake256_48_batch_for_test_v2(uint32_t abi_version, const uint8_t *messages,
                                                               const size_t *offsets, const size_t *lengths,
                                                               size_t count, const uint8_t *dst, size_t dst_len,
                                                               uint8_t *outputs);
int32_t cubbs_bbs_gpu_hash_to_scalar_shake256_batch_for_test_v2(uint32_t abi_version, const uint8_t *messages,
                                                                const size_t *offsets, const size_t *lengths,
                                                                size_t count, const uint8_t *dst, size_t dst_len,
                                                                uint8_t *scalars);
/* Host phase times (ms6: workspace, plan, public keys, upload, device pipeline, results) of one
 * ProofVerify call. */
int32_t cubbs_bbs_gpu_proof_verify_phases_for_test_v2(const CuBbsBbsGpuProofVerifyItem *items, size_t n,
                                                      CuBbsBbsGpuResult *results, double *ms6);

#ifdef __cplusplus
}
#endif

#endif /* CUBBS_BBS_GPU_TEST_H */
