// Host runtime shared by the translation units of libcubbs_bbs_cuda.so:
// device arena, pinned staging, the resident prepared state (generators,
// fixed-base window tables, public-key Miller lines) and launch helpers.
#pragma once
#include <cuda.h>  // driver types of the SM partition (entry points come through the runtime)
#include <cuda_runtime.h>
#include <stdint.h>

#include <condition_variable>
#include <memory>
#include <mutex>
#include <shared_mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/cubbs_bbs_gpu_abi.h"
#include "../../include/cubbs_bbs_gpu_test.h"  // the definitions are checked against these declarations
#include "pairing.cuh"
#include "suite.cuh"

namespace cubbs {

#define CUBBS_CHECK(expr)                                 \
  do {                                                    \
    cudaError_t _e = (expr);                              \
    if (_e != cudaSuccess) throw CudaError(_e, #expr);    \
  } while (0)

struct CudaError {
  cudaError_t code;
  const char *what;
  CudaError(cudaError_t c, const char *w) : code(c), what(w) {}
};

// Bump allocator over one growable device allocation.  Reset at the start of
// every ABI call (calls are serialised by Runtime::mu).
struct DeviceArena {
  uint8_t *base = nullptr;
  size_t cap = 0, used = 0;
  void reset() { used = 0; }
  void reserve(size_t bytes);
  template <typename T> T *alloc(size_t n) {
    size_t bytes = (n * sizeof(T) + 255) & ~(size_t)255;
    if (used + bytes > cap) throw CudaError(cudaErrorMemoryAllocation, "arena exhausted");
    T *p = reinterpret_cast<T *>(base + used);
    used += bytes;
    return p;
  }
};

// Pinned host staging buffer (one per runtime).
struct HostStaging {
  uint8_t *base = nullptr;
  size_t cap = 0, used = 0;
  void reset() { used = 0; }
  void reserve(size_t bytes);
  uint8_t *alloc(size_t bytes) {
    bytes = (bytes + 15) & ~(size_t)15;
    if (used + bytes > cap) throw CudaError(cudaErrorMemoryAllocation, "staging exhausted");
    uint8_t *p = base + used;
    used += bytes;
    return p;
  }
};

// Fixed-base window table over the generator list [P1, Q1, H1, ...]:
// entry (g, k, d-1) = d * 2^(w k) * G_g (affine), d = 1..2^(w-1).
constexpr int MAX_TABLE_WINDOW = 20;  // widest fixed-base window (13 windows, 654 MB per generator)

struct FixedTable {
  int w = 0, nwin = 0, half = 0, gens = 0;
  int req_w = 0;  // the width setting it was built under (0: automatic)
  g1a *entries = nullptr;
};
// Bytes of a fixed-base table over `gens` generators at window width w.
inline size_t table_bytes(int gens, int w) {
  return (size_t)gens * (size_t)(255 / w + 1) * ((size_t)1 << (w - 1)) * sizeof(g1a);
}

struct PkSlot {
  int status = DEC_BAD;  // DEC_OK / DEC_INF / DEC_BAD
};

// Uneven variable-base MSMs (k_msm.cu), per size class of the term count K:
// thread mode (chunks of t terms per lane, each lane a bucket method of window
// c <= 7 with its own buckets) or warp mode (one warp per MSM, window c in
// 4..12, buckets shared by the warp's lanes).
#define MSM_CLASSES 4  // K <= 8, <= 32, <= 96, larger
#define MSM_MODE_THREAD 0u
#define MSM_MODE_WARP 1u
#define MSM_THREAD_C_MAX 7
#define MSM_WARP_C_MAX 12
#define MSM_WARP_SMEM_C_MAX 10  // warp-mode buckets in shared memory up to this window, global memory beyond
struct MsmTuning {
  // measured on GB300 over 16384 MSMs with K ~ U{2..257}: 120.7k MSMs/s
  uint32_t chunk[MSM_CLASSES] = {8, 16, 32, 32};
  uint32_t window[MSM_CLASSES] = {4, 4, 4, 4};
  uint32_t mode[MSM_CLASSES] = {MSM_MODE_THREAD, MSM_MODE_THREAD, MSM_MODE_THREAD, MSM_MODE_THREAD};
};
struct MsmChunk {
  uint32_t first, count;  // term range
  uint32_t slot;          // partial index (0xffffffff: padding)
  uint32_t pad;
};
// Work unit of the persistent engine (one warp): kind << 8 | window, and the
// first of 32 chunks (thread mode), the MSM (warp mode) or the pairing job.
enum : uint32_t { MSM_UNIT_THREAD = 0, MSM_UNIT_WARP = 1, MSM_UNIT_PAIR = 2 };
struct MsmUnit {
  uint32_t kind_c;
  uint32_t index;
};
int msm_size_class(uint32_t K);
struct MsmPlan {
  std::vector<uint32_t> start;    // term offsets of the MSMs (n + 1)
  uint32_t terms = 0;
  std::vector<uint8_t> term_c;    // window width per term
  std::vector<MsmChunk> chunks;   // thread-mode chunks, 32 per unit
  std::vector<MsmUnit> units;     // pairing units first, then the largest MSMs first
  std::vector<uint32_t> pstart;   // partial offsets of the MSMs (n + 1)
  uint32_t nparts = 0;
  uint32_t max_warp_c = 0;        // widest warp-mode window (0: no warp units)
  uint32_t max_warp_smem_c = 0;   // widest warp-mode window with buckets in shared memory (0: none)
  uint32_t pair_units = 0;
  void build(const std::vector<uint32_t> &K, const MsmTuning &tune, uint32_t pairings = 0);
};
// Prepared state of one ciphersuite (the generators and everything built on
// them differ between BLS12-381-SHA-256 and BLS12-381-SHAKE-256).
struct SuiteState {
  // generators: d_gens[0] = P1, d_gens[1] = Q1, d_gens[1 + i] = H_i
  int gen_count = 0;            // entries of d_gens built (P1 included)
  int gen_capacity = 0;
  g1a *d_gens = nullptr;
  uint8_t *d_gens_c = nullptr;  // compressed, same indexing as d_gens
  std::vector<uint8_t> h_gens_c;  // host copy of d_gens_c[0..gen_count)
  uint8_t *d_seed_state = nullptr;  // generator seed chain after gen_count - 1 steps
  FixedTable table;
  // Resident domain-hash prefixes (DomainJob::prefix), one per (key slot, L):
  // key slot << 32 | L -> index into d_dom_prefix (DOMAIN_PREFIX_BYTES each).
  // SHA-256 suite only.
  std::unordered_map<uint64_t, uint32_t> dom_prefix;
  uint8_t *d_dom_prefix = nullptr;
  uint32_t dom_prefix_cap = 0;
};

// Process-wide prepared state shared by every call: generators, the
// fixed-base window table (per ciphersuite) and the Miller lines of -P2, P2
// and every public key seen.  Calls hold `mu` shared while their kernels may
// read the state; growing it (more generators, a wider table, new keys) takes
// `mu` exclusive, so nothing is reallocated under a running call.
struct SharedState {
  std::shared_mutex mu;
  std::mutex init_mu;
  bool initialised = false;
  int device = 0;
  int sm_count = 0;
  cudaStream_t prep = nullptr;  // stream that builds prepared state
  SuiteState suites[SUITE_COUNT];
  int table_w = 0;              // fixed-base window width; 0 = fewest windows within the table budget
  // Miller lines: slot 0 = -P2, slot 1 = P2, slots >= 2 = public keys
  line2 *d_lines = nullptr;
  g2a *d_pk_aff = nullptr;
  int line_capacity = 0, line_used = 0;
  std::unordered_map<std::string, int> pk_slots;
  std::vector<PkSlot> slot_info;
  int workspaces = 4;           // concurrent calls (CUBBS_BBS_WORKSPACES)
  MsmTuning msm_tuning;         // uneven-MSM chunk length / window per size class
  // SM partition of ProofVerify (green contexts): a few SMs for the
  // aggregated pairing chain (scaling, group sums, single-block checks), the
  // rest for every other kernel of the call, so that the chain's few warps do
  // not share their SMs with the MSM kernels.  Null when the driver offers no
  // partition or CUBBS_BBS_SM_PARTITION is 0.
  CUgreenCtx green_small = nullptr, green_rest = nullptr;
  int small_sms = 0, rest_sms = 0;
  // green_rest split once more (CUBBS_BBS_VAR_SMS): green_var for the decode
  // and the variable-base terms, green_rest2 for the other kernels (null when
  // the split is off or failed; green_rest is then used whole)
  CUgreenCtx green_var = nullptr, green_rest2 = nullptr;
  int var_sms = 0;
  int var_status = -1;  // 0: on; 1: not asked for; else the step that failed (* 1000 + driver result)
  int partition_status = -1;  // 0: on; -1: not tried yet; else why it is off (step * 1000 + driver result)
  bool partition_tried = false;
  CUresult (*green_stream_create)(CUstream *, CUgreenCtx, unsigned, int) = nullptr;

  static SharedState &get();
  void init();                              // device, prep stream, -P2/P2 lines
  // green_small / green_rest, made on first use (the first ProofVerify batch
  // with a key group, or a partition query), not at library start: small
  // calls then never launch on a green context
  void ensure_partition();
  void init_partition();
  // the following run with mu held exclusively
  void grow_generators(int suite, int count);
  void grow_table(int suite, int gens);
  int table_window_for(int suite, int gens) const;
  size_t table_budget = 0;  // device bytes for the tables of all suites
  bool table_covers(int suite, int gens) const;
  void add_pks(const std::vector<std::string> &fresh);
  void add_domain_prefixes(int suite, const std::vector<std::pair<uint64_t, const uint8_t *>> &fresh);
};

// One call's workspace: arena, pinned staging, two streams and the events
// that fork and join them.  Workspaces come from a pool (CallScope), so calls
// from several host threads run concurrently on the device.  The prepared
// state is reached through the reference members below.
struct Runtime {
  SharedState &sh;
  int &device;
  int &sm_count;
  int &table_w;
  line2 *&d_lines;
  int suite = SUITE_SHA256;  // ciphersuite of the running call (set by the entry point)
  SuiteState &ss() const { return sh.suites[suite]; }
  const FixedTable &table() const { return ss().table; }
  g1a *d_gens() const { return ss().d_gens; }
  uint8_t *d_gens_c() const { return ss().d_gens_c; }
  cudaStream_t stream = nullptr, stream2 = nullptr, stream3 = nullptr, stream4 = nullptr;
  // stream -> stream2 (ev_fork), stream2 -> stream3, stream4 (ev_mid), back to stream
  // (ev_side, ev_join, ev_sub)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_mid = nullptr, ev_side = nullptr, ev_sub = nullptr;
  cudaEvent_t ev_hash = nullptr;  // ProofVerify: message scalars ready (stream -> stream4)
  // ProofVerify on the SM partition: part[0..3] play stream..stream4 on the
  // larger partition, part_check runs the aggregated pairing chain on the
  // smaller one (all null without a partition)
  cudaStream_t part[4] = {nullptr, nullptr, nullptr, nullptr}, part_check = nullptr;
  cudaEvent_t ev_gc = nullptr, ev_gc2 = nullptr, ev_done = nullptr;
  bool part_tried = false;
  // CUDA graphs of the uneven-MSM engine, keyed by plan shape and buffers (k_prims.cu)
  std::unordered_map<uint64_t, cudaGraphExec_t> msm_graphs;
  DeviceArena arena;
  HostStaging staging;
  HostStaging pack;  // pinned: the packed batch bytes, copied to the device without a host copy
  std::shared_lock<std::shared_mutex> *lock = nullptr;  // the running call's shared hold

  explicit Runtime(SharedState &s);
  // true when part[] / part_check exist (makes the shared partition and this
  // workspace's streams on it the first time)
  bool use_partition();
  void ensure_generators(int count);  // d_gens[0..count) (P1 + count-1 generators)
  void ensure_table(int gens);        // fixed-base table covering d_gens[0..gens)
  void set_table_window(int w, int gens);  // rebuild the table with window width w (0: automatic)
  void set_msm_tuning(const MsmTuning &t);
  // Resolve public keys to line slots (decoding + subgroup check + lines on the
  // device for new keys).  pk_ptrs[i] -> slot index; status per key.
  void resolve_pks(const std::vector<const uint8_t *> &pk_ptrs, std::vector<int> &slots,
                   std::vector<int> &status);
  const std::vector<uint8_t> &host_gens_c() const { return ss().h_gens_c; }
};

// Takes a free workspace from the pool (waiting while all are busy), makes the
// device current on the calling thread, holds the prepared state shared and
// resets the workspace's arena and staging.  Released on destruction.
struct CallScope {
  Runtime &rt;
  std::shared_lock<std::shared_mutex> lock;
  CallScope();
  ~CallScope();
  CallScope(const CallScope &) = delete;
  CallScope &operator=(const CallScope &) = delete;
};

inline unsigned blocks_for(size_t n, unsigned tpb) { return (unsigned)((n + tpb - 1) / tpb); }

// Launchers implemented in the kernel translation units.
void launch_h2s_flat(cudaStream_t s, const uint8_t *msgs, const uint32_t *offs, const uint32_t *lens,
                     uint32_t n, const uint8_t *dst, uint32_t dlen, fr *out_raw, int suite = SUITE_SHA256);
void launch_sha256_flat(cudaStream_t s, const uint8_t *msgs, const uint32_t *offs, const uint32_t *lens,
                        uint32_t n, uint8_t *digests);
void launch_expand48_flat(cudaStream_t s, const uint8_t *msgs, const uint32_t *offs, const uint32_t *lens,
                          uint32_t n, const uint8_t *dst, uint32_t dlen, uint8_t *out, int suite);
// domain = H2S(PK || I2OSP(L,8) || Q1..H_L || api_id || I2OSP(hlen,8) || header)
// `prefix` indexes the resident SHA-256 state after Z_pad || PK || I2OSP(L,8) ||
// Q1..H_L of the item's (key, L) (DOMAIN_NO_PREFIX: hash the whole input).
constexpr uint32_t DOMAIN_NO_PREFIX = 0xffffffffu;
struct DomainJob {
  uint32_t pk_off, hdr_off, hdr_len, L;
  uint32_t prefix = DOMAIN_NO_PREFIX;
};
constexpr size_t DOMAIN_PREFIX_BYTES = 104;  // one SHA-256 context (sha_ctx)
struct DomainPrefixJob {
  uint8_t pk[96];
  uint32_t L, index;  // index: the context's place in the resident array
};
void launch_domain(cudaStream_t s, const DomainJob *jobs, uint32_t n, const uint8_t *blob,
                   const uint8_t *gens_c, const uint8_t *prefixes, fr *out_raw, int suite = SUITE_SHA256);
void launch_domain_prefix(cudaStream_t s, const DomainPrefixJob *jobs, uint32_t n, const uint8_t *gens_c,
                          uint8_t *prefixes);
void launch_make_generator_seeds(cudaStream_t s, int first, int count, uint8_t *seeds_state,
                                 uint8_t *seeds_out, int suite);
void launch_hash_generators(cudaStream_t s, int first, int count, const uint8_t *seeds, g1a *gens,
                            uint8_t *gens_c, int suite);
void launch_decode_p1(cudaStream_t s, g1a *gens, uint8_t *gens_c, int suite);
void launch_build_table(cudaStream_t s, const g1a *gens, int g0, int g1n, FixedTable t, g1a *bases,
                        g1 *scratch_xyzz, fp *scratch_prod);
// decode N compressed G1 points: status DEC_*; affine out
// lanes per point: 1, 2 or 4 (0: chosen by the point count or CUBBS_BBS_VAR_LANES)
void launch_g1_subgroup(cudaStream_t s, const g1a *pts, const int32_t *status, uint32_t n, int32_t *bad,
                        int lanes = 0);
int var_lanes_setting();
void launch_g1_decode(cudaStream_t s, const uint8_t *pts48, uint32_t stride, uint32_t n, g1a *out,
                      int32_t *status, bool check_subgroup);
// fixed-base MSM rows: scalars raw Fr [row * stride + g] for g < nterms[row]
void launch_fixed_msm(cudaStream_t s, const FixedTable &t, const fr *scalars, uint32_t stride,
                      const uint32_t *nterms, uint32_t rows, g1 *out);
// variable-base jobs: out[i] = k[i] * P[i]; P given as affine points
struct VarJob {
  uint32_t point;  // index into the point array
  uint32_t flags;  // bit0: point is infinity (result infinity)
};
// lanes per job: 1, 2, 4 or 8 (0: chosen by the job count or CUBBS_BBS_VAR_LANES)
void launch_var_mul(cudaStream_t s, const g1a *points, const VarJob *jobs, const fr *scalars, uint32_t n,
                    g1 *out, int lanes = 0);
void launch_g1_compress(cudaStream_t s, const g1 *pts, uint32_t n, uint8_t *out48);
// Launches k_g1_decode and every variable-base kernel over zero items on the
// legacy default stream of the current device (module load and local-memory
// sizing ahead of real work; nothing is read or written).
cudaError_t warm_decode_and_var_mul_kernels(uint8_t *any_device_buffer);
struct PairJob;
struct MsmDevice {
  uint32_t n = 0, nterms = 0, nchunks = 0, nunits = 0;
  uint8_t *term_c = nullptr;
  MsmChunk *chunks = nullptr;
  MsmUnit *units = nullptr;
  uint32_t *pstart = nullptr, *start = nullptr, *koff = nullptr, *counter = nullptr;
  g1a *phi = nullptr;
  g1 *partials = nullptr;
  g1 *gbuckets = nullptr;  // global buckets of warp units whose window exceeds MSM_WARP_SMEM_C_MAX
  uint32_t warps_per_block = 4, smem_per_warp = 0, grid = 0, gbucket_stride = 0;
  // pairing units: e(pa, Q_slot_a) e(pb, Q_slot_b) == 1 for pjobs[0 .. pair_units)
  const PairJob *pjobs = nullptr;
  const line2 *lines = nullptr;
  uint8_t *pok = nullptr;
  void upload(Runtime &rt, const MsmPlan &p, cudaStream_t s);
  static size_t arena_bytes(const MsmPlan &p, int sm_count);
};
// term j of the flat term list uses point jobs[j].point (skipped when flags & 1)
// and scalar scalars[j]; MSM i owns terms [start[i], start[i+1]).
void launch_msm_prep(cudaStream_t s, const MsmDevice &d, const g1a *pts, const VarJob *jobs, const fr *scalars);
// One persistent launch over all units (thread chunks, warp MSMs, pairing
// checks), then the per-MSM reduction of the partials.
void launch_msm_main(cudaStream_t s, const MsmDevice &d, const g1a *pts, const VarJob *jobs, int sm_count, g1 *out,
                     uint8_t *out48);
void launch_pk_prepare(cudaStream_t s, const uint8_t *pks96, uint32_t n, int slot0, g2a *pk_aff,
                       line2 *lines, int32_t *status);
void launch_p2_lines(cudaStream_t s, line2 *lines);
// Pairing check job: e(pa, Q_slot_a) * e(pb, Q_slot_b) == 1.  flags bit0/bit1:
// pair a / pair b is skipped (its G1 or G2 side is the identity).
struct PairJob {
  g1a pa, pb;
  int32_t slot_a, slot_b;
  uint32_t flags;
  uint32_t active;  // 1: evaluate; 0: not evaluated (result 0); 2: result already written
};
void launch_pairing_check(cudaStream_t s, const PairJob *jobs, uint32_t n, const line2 *lines, uint8_t *ok);
// the same check with one warp per pair (lower latency for a few checks)
void launch_pairing_check_split(cudaStream_t s, const PairJob *jobs, uint32_t n, const line2 *lines, uint8_t *ok);

}  // namespace cubbs
