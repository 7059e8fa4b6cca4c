// Hash kernels (one message per thread) and the hash-only ABI entry points:
// messages_to_scalar (reference cubbs_bbs_cuda.cu:353-439), the test exports
// sha256 / expand_xmd / hash_to_scalar (reference cubbs_bbs_cuda.cu:53-351) and
// sign_e_from_resident_scalars (reference cubbs_bbs_cuda.cu:476-717).
#include <cstring>

#include "h2c.cuh"
#include "bbs_dst.cuh"
#include "runtime.cuh"

namespace cubbs {


__global__ void k_sha256_flat(const uint8_t *msgs, const uint32_t *offs, const uint32_t *lens, uint32_t n,
                              uint8_t *digests) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  sha_ctx c;
  sha_init(c);
  sha_bytes(c, msgs + offs[i], lens[i]);
  sha_final(c, digests + 32 * (size_t)i);
}

template <int S>
__global__ void k_expand48_flat(const uint8_t *msgs, const uint32_t *offs, const uint32_t *lens, uint32_t n,
                                const uint8_t *dst, uint32_t dlen, uint8_t *out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  hash_ctx<S> c;
  msg_begin(c);
  msg_bytes(c, msgs + offs[i], lens[i]);
  msg_finish(c, dst, dlen, 48, out + 48 * (size_t)i);
}

template <int S>
__global__ void k_h2s_flat(const uint8_t *msgs, const uint32_t *offs, const uint32_t *lens, uint32_t n,
                           const uint8_t *dst, uint32_t dlen, fr *out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  hash_ctx<S> c;
  msg_begin(c);
  msg_bytes(c, msgs + offs[i], lens[i]);
  out[i] = h2s_finish(c, dst, dlen);
}

static_assert(sizeof(sha_ctx) == DOMAIN_PREFIX_BYTES, "domain prefix size");

// calculate_domain (crates/cubbs-bbs-protocol/src/utils/util.rs:147-189).  The
// input starts with Z_pad || PK || I2OSP(L, 8) || Q1 .. H_L (78 of its 80
// SHA-256 blocks at L = 100), the same for every item of a key and message
// count: an item whose (key, L) has a resident prefix starts from that state
// (suite 0 only; the SHAKE-256 suite hashes the whole input).
template <int S>
__global__ void k_domain(const DomainJob *jobs, uint32_t n, const uint8_t *blob, const uint8_t *gens_c,
                         const sha_ctx *prefixes, fr *out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  DomainJob j = jobs[i];
  hash_ctx<S> c;
  bool resumed = false;
  if constexpr (S == SUITE_SHA256) {
    if (prefixes && j.prefix != DOMAIN_NO_PREFIX) {
      c = prefixes[j.prefix];
      resumed = true;
    }
  }
  if (!resumed) {
    msg_begin(c);
    msg_bytes(c, blob + j.pk_off, 96);
    msg_u64be(c, j.L, 8);
    // Q1, H1..H_L are d_gens_c[1 .. L+1]
    msg_bytes(c, gens_c + 48, 48 * (j.L + 1));
  }
  msg_bytes(c, SuiteDst<S>::api_id(), SuiteDst<S>::api_id_len);
  msg_u64be(c, j.hdr_len, 8);
  msg_bytes(c, blob + j.hdr_off, j.hdr_len);
  out[i] = h2s_api<S>(c);
}

// Generator seed chain (generators.rs:131-144): v_0 = expand(seed, seed_dst),
// v_i = expand(v_{i-1} || I2OSP(i, 8), seed_dst).  Sequential, one thread.
// state holds v_{first-1} (48 bytes) on entry and v_{first+count-1} on exit.
template <int S> __global__ void k_generator_seeds(int first, int count, uint8_t *state, uint8_t *seeds) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const uint8_t *dst = SuiteDst<S>::dst_gen_seed();
  constexpr uint32_t dlen = SuiteDst<S>::dst_gen_seed_len;
  uint8_t v[48];
  if (first == 1) {
    hash_ctx<S> c;
    msg_begin(c);
    msg_bytes(c, SuiteDst<S>::gen_seed(), SuiteDst<S>::gen_seed_len);
    msg_finish(c, dst, dlen, 48, v);
  } else {
    for (int k = 0; k < 48; k++) v[k] = state[k];
  }
  #pragma unroll 1
  for (int i = first; i < first + count; i++) {
    hash_ctx<S> c;
    msg_begin(c);
    msg_bytes(c, v, 48);
    msg_u64be(c, (uint64_t)i, 8);
    msg_finish(c, dst, dlen, 48, v);
    for (int k = 0; k < 48; k++) seeds[48 * (size_t)(i - first) + k] = v[k];
  }
  for (int k = 0; k < 48; k++) state[k] = v[k];
}

// generator i (1-based: Q1 = 1, H_j = j + 1) = hash_to_curve(v_i, api_id || "SIG_GENERATOR_DST_")
template <int S>
__global__ void k_hash_generators(int first, int count, const uint8_t *seeds, g1a *gens, uint8_t *gens_c) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  g1 p = hash_to_curve_g1<S>(seeds + 48 * (size_t)t, 48, SuiteDst<S>::dst_gen(), SuiteDst<S>::dst_gen_len);
  g1a a;
  g1_to_aff(p, a);
  int idx = first + t;  // d_gens index: P1 at 0, Q1 at 1
  gens[idx] = a;
  g1_compress_aff(a, gens_c + 48 * (size_t)idx);
}

// e = hash_to_scalar(sk || m_1..m_L || domain, e_dst) over resident message scalars
// (reference cubbs_bbs_cuda.cu:449-474 packs the same input on the device).
struct SignEJob {
  uint32_t blob_off;  // sk (32) then domain (32)
  uint32_t scalar_off, count;
};
__global__ void k_sign_e(const SignEJob *jobs, uint32_t n, const uint8_t *blob, const fr *scalars,
                         const uint8_t *dst, uint32_t dlen, fr *out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  SignEJob j = jobs[i];
  sha_ctx c;
  xmd_begin(c);
  sha_bytes(c, blob + j.blob_off, 32);
  #pragma unroll 1
  for (uint32_t k = 0; k < j.count; k++) {
    uint8_t b[32];
    fr_raw_to_be32(scalars[j.scalar_off + k], b);
    sha_bytes(c, b, 32);
  }
  sha_bytes(c, blob + j.blob_off + 32, 32);
  out[i] = h2s_finish(c, dst, dlen);
}

template <int S> __global__ void k_decode_p1(g1a *gens, uint8_t *gens_c) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  uint8_t p1[48];
  for (int k = 0; k < 48; k++) p1[k] = SuiteDst<S>::p1_compressed()[k];
  g1a a;
  g1_decompress(p1, a, false);
  gens[0] = a;
  for (int k = 0; k < 48; k++) gens_c[k] = p1[k];
}

void launch_sha256_flat(cudaStream_t s, const uint8_t *msgs, const uint32_t *offs, const uint32_t *lens,
                        uint32_t n, uint8_t *digests) {
  if (n) k_sha256_flat<<<blocks_for(n, 128), 128, 0, s>>>(msgs, offs, lens, n, digests);
}
void launch_expand48_flat(cudaStream_t s, const uint8_t *msgs, const uint32_t *offs, const uint32_t *lens,
                          uint32_t n, const uint8_t *dst, uint32_t dlen, uint8_t *out, int suite) {
  if (n)
    CUBBS_SUITE_DISPATCH(suite, k_expand48_flat<S><<<blocks_for(n, 128), 128, 0, s>>>(msgs, offs, lens, n, dst,
                                                                                       dlen, out));
}
void launch_h2s_flat(cudaStream_t s, const uint8_t *msgs, const uint32_t *offs, const uint32_t *lens,
                     uint32_t n, const uint8_t *dst, uint32_t dlen, fr *out, int suite) {
  if (n)
    CUBBS_SUITE_DISPATCH(suite, k_h2s_flat<S><<<blocks_for(n, 128), 128, 0, s>>>(msgs, offs, lens, n, dst, dlen,
                                                                                  out));
}
void launch_domain(cudaStream_t s, const DomainJob *jobs, uint32_t n, const uint8_t *blob,
                   const uint8_t *gens_c, const uint8_t *prefixes, fr *out, int suite) {
  if (n)
    CUBBS_SUITE_DISPATCH(suite, k_domain<S><<<blocks_for(n, 64), 64, 0, s>>>(
                                    jobs, n, blob, gens_c, reinterpret_cast<const sha_ctx *>(prefixes), out));
}

// The domain-hash prefix of each job's (key, L): the SHA-256 state after
// Z_pad || PK || I2OSP(L, 8) || Q1 .. H_L, stored at prefixes[index].
__global__ void k_domain_prefix(const DomainPrefixJob *jobs, uint32_t n, const uint8_t *gens_c, sha_ctx *out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const DomainPrefixJob &j = jobs[i];
  sha_ctx c;
  xmd_begin(c);
  sha_bytes(c, j.pk, 96);
  sha_u64be(c, j.L, 8);
  sha_bytes(c, gens_c + 48, 48 * (j.L + 1));
  out[j.index] = c;
}
void launch_domain_prefix(cudaStream_t s, const DomainPrefixJob *jobs, uint32_t n, const uint8_t *gens_c,
                          uint8_t *prefixes) {
  if (n)
    k_domain_prefix<<<blocks_for(n, 64), 64, 0, s>>>(jobs, n, gens_c, reinterpret_cast<sha_ctx *>(prefixes));
}
void launch_make_generator_seeds(cudaStream_t s, int first, int count, uint8_t *state, uint8_t *seeds, int suite) {
  CUBBS_SUITE_DISPATCH(suite, k_generator_seeds<S><<<1, 1, 0, s>>>(first, count, state, seeds));
}
void launch_hash_generators(cudaStream_t s, int first, int count, const uint8_t *seeds, g1a *gens,
                            uint8_t *gens_c, int suite) {
  if (count)
    CUBBS_SUITE_DISPATCH(suite, k_hash_generators<S><<<blocks_for(count, 32), 32, 0, s>>>(first, count, seeds,
                                                                                           gens, gens_c));
}
void launch_decode_p1(cudaStream_t s, g1a *gens, uint8_t *gens_c, int suite) {
  CUBBS_SUITE_DISPATCH(suite, k_decode_p1<S><<<1, 1, 0, s>>>(gens, gens_c));
}

// ----------------------------------------------------------------------------- ABI: hashing
namespace {
bool abi_ok(uint32_t v) { return v == CUBBS_BBS_GPU_ABI_VERSION; }

// Stage a packed message list: returns device pointers to bytes/offsets/lengths.
struct FlatMsgs {
  uint8_t *bytes;
  uint32_t *offs, *lens;
};
FlatMsgs stage_flat(Runtime &rt, const uint8_t *const *ptrs, const size_t *lens, size_t n) {
  size_t total = 0;
  #pragma unroll 1
  for (size_t i = 0; i < n; i++) total += lens[i];
  uint8_t *h = rt.staging.alloc(total + 8 * n + 16);
  uint32_t *ho = reinterpret_cast<uint32_t *>(h);
  uint32_t *hl = ho + n;
  uint8_t *hb = h + 8 * n;
  size_t cur = 0;
  #pragma unroll 1
  for (size_t i = 0; i < n; i++) {
    ho[i] = (uint32_t)cur;
    hl[i] = (uint32_t)lens[i];
    if (lens[i]) std::memcpy(hb + cur, ptrs[i], lens[i]);
    cur += lens[i];
  }
  uint8_t *d = rt.arena.alloc<uint8_t>(total + 8 * n + 16);
  CUBBS_CHECK(cudaMemcpyAsync(d, h, total + 8 * n, cudaMemcpyHostToDevice, rt.stream));
  return {d + 8 * n, reinterpret_cast<uint32_t *>(d), reinterpret_cast<uint32_t *>(d) + n};
}
uint8_t *stage_bytes(Runtime &rt, const uint8_t *p, size_t n) {
  uint8_t *d = rt.arena.alloc<uint8_t>(n + 1);
  if (n) CUBBS_CHECK(cudaMemcpyAsync(d, p, n, cudaMemcpyHostToDevice, rt.stream));
  return d;
}
}  // namespace

}  // namespace cubbs

using namespace cubbs;

static int32_t flat_test_call(uint32_t abi, const uint8_t *messages, const size_t *offsets, const size_t *lengths,
                              size_t n, const uint8_t *dst, size_t dst_len, uint8_t *out, int mode) {
  if (!abi_ok(abi) || (n > 0 && (messages == nullptr || offsets == nullptr || lengths == nullptr || out == nullptr)) ||
      dst_len > 255 || (dst_len > 0 && dst == nullptr) || n > 0xffffffffu)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    std::vector<const uint8_t *> ptrs(n);
    size_t total = 0;
    #pragma unroll 1
    for (size_t i = 0; i < n; i++) {
      ptrs[i] = messages + offsets[i];
      total += lengths[i];
    }
    rt.staging.reserve(total + 16 * n + 4096);
    rt.arena.reserve(total + 16 * n + 64 * n + 4096);
    FlatMsgs f = stage_flat(rt, ptrs.data(), lengths, n);
    uint8_t *ddst = stage_bytes(rt, dst, dst_len);
    // mode: 0 SHA-256, 1 expand_message_xmd (48 B), 2 hash_to_scalar over xmd,
    // 3 expand_message_xof (48 B), 4 hash_to_scalar over xof
    const bool expand = mode == 1 || mode == 3, h2s = mode == 2 || mode == 4;
    const int suite = mode >= 3 ? SUITE_SHAKE256 : SUITE_SHA256;
    size_t out_sz = expand ? 48 : 32;
    uint8_t *dout = rt.arena.alloc<uint8_t>(n * 48);
    if (mode == 0) {
      launch_sha256_flat(rt.stream, f.bytes, f.offs, f.lens, (uint32_t)n, dout);
    } else if (expand) {
      launch_expand48_flat(rt.stream, f.bytes, f.offs, f.lens, (uint32_t)n, ddst, (uint32_t)dst_len, dout, suite);
    } else {
      launch_h2s_flat(rt.stream, f.bytes, f.offs, f.lens, (uint32_t)n, ddst, (uint32_t)dst_len,
                      reinterpret_cast<fr *>(dout), suite);
    }
    CUBBS_CHECK(cudaGetLastError());
    if (h2s) {
      std::vector<uint32_t> raw(8 * n);
      CUBBS_CHECK(cudaMemcpyAsync(raw.data(), dout, 32 * n, cudaMemcpyDeviceToHost, rt.stream));
      CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
      #pragma unroll 1
      for (size_t i = 0; i < n; i++)
        #pragma unroll 1
        for (int w = 0; w < 8; w++)
          #pragma unroll 1
          for (int b = 0; b < 4; b++) out[32 * i + (7 - w) * 4 + (3 - b)] = (uint8_t)(raw[8 * i + w] >> (8 * b));
    } else {
      CUBBS_CHECK(cudaMemcpyAsync(out, dout, out_sz * n, cudaMemcpyDeviceToHost, rt.stream));
      CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    }
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

extern "C" int32_t cubbs_bbs_gpu_sha256_batch_for_test_v2(uint32_t abi, const uint8_t *messages,
                                                          const size_t *offsets, const size_t *lengths,
                                                          size_t n, uint8_t *digests) {
  return flat_test_call(abi, messages, offsets, lengths, n, nullptr, 0, digests, 0);
}
extern "C" int32_t cubbs_bbs_gpu_expand_xmd_sha256_48_batch_for_test_v2(
    uint32_t abi, const uint8_t *messages, const size_t *offsets, const size_t *lengths, size_t n,
    const uint8_t *dst, size_t dst_len, uint8_t *outputs) {
  return flat_test_call(abi, messages, offsets, lengths, n, dst, dst_len, outputs, 1);
}
extern "C" int32_t cubbs_bbs_gpu_expand_xof_shake256_48_batch_for_test_v2(
    uint32_t abi, const uint8_t *messages, const size_t *offsets, const size_t *lengths, size_t n,
    const uint8_t *dst, size_t dst_len, uint8_t *outputs) {
  return flat_test_call(abi, messages, offsets, lengths, n, dst, dst_len, outputs, 3);
}
extern "C" int32_t cubbs_bbs_gpu_hash_to_scalar_shake256_batch_for_test_v2(
    uint32_t abi, const uint8_t *messages, const size_t *offsets, const size_t *lengths, size_t n,
    const uint8_t *dst, size_t dst_len, uint8_t *scalars) {
  return flat_test_call(abi, messages, offsets, lengths, n, dst, dst_len, scalars, 4);
}
extern "C" int32_t cubbs_bbs_gpu_hash_to_scalar_sha256_batch_for_test_v2(
    uint32_t abi, const uint8_t *messages, const size_t *offsets, const size_t *lengths, size_t n,
    const uint8_t *dst, size_t dst_len, uint8_t *scalars) {
  return flat_test_call(abi, messages, offsets, lengths, n, dst, dst_len, scalars, 2);
}

// messages_to_scalar: one DST per batch (reference cubbs_bbs_cuda.cu:398-410 rejects mixed DSTs).
extern "C" int32_t cubbs_bbs_gpu_messages_to_scalar_batch_v2(uint32_t abi,
                                                             CuBbsBbsGpuMessagesToScalarItem *items,
                                                             size_t n, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  #pragma unroll 1
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if ((it.message.len > 0 && it.message.data == nullptr) || it.dst.len > 255 ||
        (it.dst.len > 0 && it.dst.data == nullptr) || it.scalar_out.data == nullptr || it.scalar_out.capacity < 32)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    if (it.dst.len != items[0].dst.len ||
        (it.dst.len > 0 && std::memcmp(it.dst.data, items[0].dst.data, it.dst.len) != 0))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  std::vector<size_t> offs(n), lens(n);
  // Build a contiguous view through pointers: stage_flat copies each message.
  std::vector<const uint8_t *> ptrs(n);
  size_t total = 0;
  #pragma unroll 1
  for (size_t i = 0; i < n; i++) {
    ptrs[i] = items[i].message.data;
    lens[i] = items[i].message.len;
    total += lens[i];
  }
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    rt.staging.reserve(total + 16 * n + 4096);
    rt.arena.reserve(total + 64 * n + 4096);
    FlatMsgs f = stage_flat(rt, ptrs.data(), lens.data(), n);
    uint8_t *ddst = stage_bytes(rt, items[0].dst.data, items[0].dst.len);
    fr *dout = rt.arena.alloc<fr>(n);
    launch_h2s_flat(rt.stream, f.bytes, f.offs, f.lens, (uint32_t)n, ddst, (uint32_t)items[0].dst.len, dout);
    CUBBS_CHECK(cudaGetLastError());
    std::vector<uint32_t> raw(8 * n);
    CUBBS_CHECK(cudaMemcpyAsync(raw.data(), dout, 32 * n, cudaMemcpyDeviceToHost, rt.stream));
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    #pragma unroll 1
    for (size_t i = 0; i < n; i++) {
      uint8_t *o = items[i].scalar_out.data;
      #pragma unroll 1
      for (int w = 0; w < 8; w++)
        #pragma unroll 1
        for (int b = 0; b < 4; b++) o[(7 - w) * 4 + (3 - b)] = (uint8_t)(raw[8 * i + w] >> (8 * b));
      items[i].scalar_out.len = 32;
      results[i] = {CUBBS_BBS_GPU_SUCCESS, 0, 32};
    }
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// Resident message scalars for sign_e_from_resident_scalars: the last raw-pipeline
// call's scalars stay on the device for later resident calls.
static fr *g_resident = nullptr;
static size_t g_resident_cap = 0, g_resident_count = 0;
static std::mutex g_resident_mu;  // one resident set per process

static void be_from_raw(const uint32_t *raw, uint8_t *o) {
  for (int w = 0; w < 8; w++)
    for (int b = 0; b < 4; b++) o[(7 - w) * 4 + (3 - b)] = (uint8_t)(raw[w] >> (8 * b));
}

extern "C" int32_t cubbs_bbs_gpu_sign_e_from_resident_scalars_batch_v2(
    uint32_t abi, CuBbsBbsGpuSignEFromResidentScalarsItem *items, size_t n, CuBbsBbsGpuByteSlice message_dst,
    CuBbsBbsGpuByteSlice e_dst, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || message_dst.len > 255 || e_dst.len > 255 || (message_dst.len && !message_dst.data) ||
      (e_dst.len && !e_dst.data) || (n > 0 && (items == nullptr || results == nullptr)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  const bool raw = items[0].messages != nullptr;
  size_t total = 0, bytes = 0;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    size_t cnt = it.message_count;
    if (cnt == 0 || !it.secret_key.data || it.secret_key.len != 32 || !it.domain.data || it.domain.len != 32 ||
        !it.scalar_out.data || it.scalar_out.capacity < 32 || (it.messages != nullptr) != raw ||
        it.message_scalar_offset + cnt < it.message_scalar_offset)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    if (raw) {
      if (it.message_scalar_offset != total || !it.message_scalars_out.data ||
          it.message_scalars_out.capacity < 32 * cnt)
        return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
      for (size_t k = 0; k < cnt; k++) {
        if (it.messages[k].len && !it.messages[k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
        bytes += it.messages[k].len;
      }
      total += cnt;
    }
  }
  try {
    std::lock_guard<std::mutex> resident_lock(g_resident_mu);
    CallScope scope;
    Runtime &rt = scope.rt;
    if (!raw) {
      for (size_t i = 0; i < n; i++)
        if (items[i].message_scalar_offset + items[i].message_count > g_resident_count)
          return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    }
    rt.staging.reserve(bytes + 16 * total + 64 * n + 65536);
    rt.arena.reserve(bytes + 64 * total + 128 * n + 65536);
    if (raw) {
      std::vector<const uint8_t *> ptrs;
      std::vector<size_t> lens;
      for (size_t i = 0; i < n; i++)
        for (size_t k = 0; k < items[i].message_count; k++) {
          ptrs.push_back(items[i].messages[k].data);
          lens.push_back(items[i].messages[k].len);
        }
      if (g_resident_cap < total) {
        if (g_resident) cudaFree(g_resident);
        g_resident = nullptr;
        g_resident_cap = 0;
        CUBBS_CHECK(cudaMalloc(&g_resident, total * sizeof(fr)));
        g_resident_cap = total;
      }
      FlatMsgs f = stage_flat(rt, ptrs.data(), lens.data(), total);
      uint8_t *md = stage_bytes(rt, message_dst.data, message_dst.len);
      launch_h2s_flat(rt.stream, f.bytes, f.offs, f.lens, (uint32_t)total, md, (uint32_t)message_dst.len, g_resident);
      g_resident_count = total;
    }
    std::vector<uint8_t> blob(64 * n);
    std::vector<SignEJob> jobs(n);
    for (size_t i = 0; i < n; i++) {
      std::memcpy(&blob[64 * i], items[i].secret_key.data, 32);
      std::memcpy(&blob[64 * i + 32], items[i].domain.data, 32);
      jobs[i] = {(uint32_t)(64 * i), (uint32_t)items[i].message_scalar_offset, (uint32_t)items[i].message_count};
    }
    uint8_t *dblob = stage_bytes(rt, blob.data(), blob.size());
    SignEJob *dj = reinterpret_cast<SignEJob *>(stage_bytes(rt, reinterpret_cast<uint8_t *>(jobs.data()),
                                                            jobs.size() * sizeof(SignEJob)));
    uint8_t *ed = stage_bytes(rt, e_dst.data, e_dst.len);
    fr *e = rt.arena.alloc<fr>(n);
    k_sign_e<<<blocks_for(n, 64), 64, 0, rt.stream>>>(dj, (uint32_t)n, dblob, g_resident, ed, (uint32_t)e_dst.len, e);
    CUBBS_CHECK(cudaGetLastError());
    std::vector<uint32_t> he(8 * n), hm(raw ? 8 * total : 0);
    CUBBS_CHECK(cudaMemcpyAsync(he.data(), e, 32 * n, cudaMemcpyDeviceToHost, rt.stream));
    if (raw) CUBBS_CHECK(cudaMemcpyAsync(hm.data(), g_resident, 32 * total, cudaMemcpyDeviceToHost, rt.stream));
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    for (size_t i = 0; i < n; i++) {
      if (raw) {
        for (size_t k = 0; k < items[i].message_count; k++)
          be_from_raw(&hm[8 * (items[i].message_scalar_offset + k)], items[i].message_scalars_out.data + 32 * k);
        items[i].message_scalars_out.len = 32 * items[i].message_count;
      }
      be_from_raw(&he[8 * i], items[i].scalar_out.data);
      items[i].scalar_out.len = 32;
      results[i] = {CUBBS_BBS_GPU_SUCCESS, 0, 32};
    }
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    g_resident_count = 0;
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}
