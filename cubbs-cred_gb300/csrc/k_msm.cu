// Uneven variable-base G1 MSMs: many independent MSMs of different term
// counts (config 4 of the benchmark plan: 16384 MSMs, K ~ U{2..257}) in one
// persistent launch.
//
// Every term k_j * P_j is GLV-split as k_j = q_j * lambda + s_j (lambda = z^2,
// so k_j P_j = s_j P_j + q_j phi(P_j) with phi(x, y) = (beta x, -y)), which
// turns an MSM of K terms into one of 2K terms with 128-bit scalars.  The
// terms of an MSM are cut into chunks of t terms; one lane evaluates a chunk
// with the bucket (Pippenger) method of window c: per window, each nonzero
// signed digit adds its point into bucket |d| (mixed addition), a running sum
// folds the buckets into sum_b b * B_b, and Horner doubling joins the windows.
// Signed digits come from k' = k + sum_w 2^(c-1) 2^(wc): digit_w =
// field_w(k') - 2^(c-1) in [-2^(c-1), 2^(c-1)).
//
// Work is grouped into units of 32 chunks with the same window width; the
// persistent kernel's warps take units from an atomic counter until none are
// left.  A second kernel sums the chunk partials of each MSM (one warp per
// MSM) and compresses the result.  Chunk length t and window c are chosen per
// size class of K by an autotuner (t >= K: one lane per MSM; t < K: the MSM is
// spread over several lanes and joined by the reduction).
//
// Reference counterpart: route 4 (native/cuda/src/kernels/variable_base_universal.cuh:
// 337-644) and the Pippenger kernel (kernels/large_msm.cuh:322-416).
#include <algorithm>
#include <cstring>
#include <vector>

#include "runtime.cuh"

namespace cubbs {

#define MSM_C_MAX 7  // buckets live in per-lane local memory: 64 XYZZ points (12 KB)

// Per term: phi(P) and the offset forms k' = k + M of the two 128-bit GLV
// halves for the window width c of the term's MSM (5 words each; with
// nwin = ceil(130 / c) windows, k' < 2^(nwin c) <= 2^136).  An identity
// point gets all-zero offset forms, which the chunk kernel skips.
__global__ void __launch_bounds__(128) k_msm_prep(const g1a *pts, const VarJob *jobs,
                                                  const fr *scalars, const uint8_t *term_c, uint32_t n, g1a *phi,
                                                  uint32_t *koff) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  uint32_t *o = koff + 10 * (size_t)j;
  const VarJob jb = jobs[j];
  if (jb.flags & 1) {  // identity point: the term contributes nothing
    for (int k = 0; k < 10; k++) o[k] = 0;
    return;
  }
  const g1a p = pts[jb.point];
  const fp beta = C_GLV_BETA;
  g1a f;
  f.x = fp_mul(p.x, beta);
  f.y = fp_neg(p.y);
  phi[j] = f;
  uint32_t s[4], q[4];
  glv_split(scalars[j], s, q);
  const int c = term_c[j];
  // M = sum_{w < nwin} 2^(c-1) 2^(wc); nwin c >= 130 keeps k + M below 2^(nwin c)
  uint32_t m[5] = {0, 0, 0, 0, 0};
  const int nwin = (130 + c - 1) / c;
  for (int w = 0; w < nwin; w++) {
    const int pos = c - 1 + w * c;
    m[pos >> 5] |= 1u << (pos & 31);
  }
  const uint32_t *halves[2] = {s, q};
  for (int h = 0; h < 2; h++) {
    uint64_t carry = 0;
    for (int k = 0; k < 5; k++) {
      uint64_t v = (uint64_t)(k < 4 ? halves[h][k] : 0) + m[k] + carry;
      o[5 * h + k] = (uint32_t)v;
      carry = v >> 32;
    }
  }
}

DEV int msm_digit(const uint32_t *k5, int w, int c) {
  const int pos = w * c;
  const int wi = pos >> 5, sh = pos & 31;
  uint64_t v = (uint64_t)k5[wi] | ((uint64_t)(wi + 1 < 5 ? k5[wi + 1] : 0) << 32);
  return (int)((v >> sh) & ((1u << c) - 1)) - (1 << (c - 1));
}

// One chunk by the bucket method; returns XYZZ.
DEV g1 msm_chunk(const g1a *pts, const VarJob *jobs, const g1a *phi,
                 const uint32_t *koff, uint32_t first, uint32_t count, int c) {
  g1 buckets[1 << (MSM_C_MAX - 1)];
  const int nb = 1 << (c - 1);
  const int nwin = (130 + c - 1) / c;
  // highest window with a nonzero digit anywhere in the chunk
  int top = 0;
#pragma unroll 1
  for (uint32_t j = first; j < first + count; j++) {
    if (jobs[j].flags & 1) continue;
    const uint32_t *k = koff + 10 * (size_t)j;
#pragma unroll 1
    for (int w = nwin - 1; w > top; w--)
      if (msm_digit(k, w, c) != 0 || msm_digit(k + 5, w, c) != 0) {
        top = w;
        break;
      }
  }
  g1 acc = g1_inf();
#pragma unroll 1
  for (int w = top; w >= 0; w--) {
    if (w != top) {
#pragma unroll 1
      for (int d = 0; d < c; d++) acc = g1_dbl(acc);
    }
#pragma unroll 1
    for (int b = 0; b < nb; b++) buckets[b] = g1_inf();
#pragma unroll 1
    for (uint32_t j = first; j < first + count; j++) {
      const VarJob jb = jobs[j];
      if (jb.flags & 1) continue;
      const uint32_t *k = koff + 10 * (size_t)j;
#pragma unroll 1
      for (int h = 0; h < 2; h++) {
        const int d = msm_digit(k + 5 * h, w, c);
        if (d == 0) continue;
        g1a p = h ? phi[j] : pts[jb.point];
        if (d < 0) p.y = fp_neg(p.y);
        const int b = (d < 0 ? -d : d) - 1;
        buckets[b] = g1_add_aff(buckets[b], p);
      }
    }
    g1 run = g1_inf(), sum = g1_inf();
#pragma unroll 1
    for (int b = nb - 1; b >= 0; b--) {
      run = g1_add(run, buckets[b]);
      sum = g1_add(sum, run);
    }
    acc = g1_add(acc, sum);
  }
  return acc;
}

// Persistent: warps take units of 32 chunks until the counter runs out.
__global__ void __launch_bounds__(128) k_msm_chunks(const g1a *pts, const VarJob *jobs,
                                                    const g1a *phi, const uint32_t *koff, const MsmChunk *chunks,
                                                    uint32_t nchunks, const uint8_t *unit_c, uint32_t nunits,
                                                    uint32_t *counter, g1 *partials) {
  const int lane = threadIdx.x & 31;
#pragma unroll 1
  for (;;) {
    uint32_t unit = 0;
    if (lane == 0) unit = atomicAdd(counter, 1u);
    unit = __shfl_sync(0xffffffffu, unit, 0);
    if (unit >= nunits) break;
    const uint32_t ci = unit * 32 + lane;
    if (ci < nchunks) {
      const MsmChunk ch = chunks[ci];
      if (ch.slot != 0xffffffffu)  // padding of a unit's last lanes
        partials[ch.slot] = msm_chunk(pts, jobs, phi, koff, ch.first, ch.count, unit_c[unit]);
    }
  }
}

// One warp per MSM: sum its chunk partials [pstart[i], pstart[i+1]), compress.
__global__ void __launch_bounds__(128) k_msm_reduce(const g1 *partials, const uint32_t *pstart, uint32_t n,
                                                    g1 *out, uint8_t *out48) {
  const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  g1 acc = g1_inf();
#pragma unroll 1
  for (uint32_t k = pstart[i] + lane; k < pstart[i + 1]; k += 32) acc = g1_add(acc, partials[k]);
#pragma unroll 1
  for (int d = 16; d > 0; d >>= 1) {
    g1 o;
#pragma unroll
    for (int k = 0; k < 12; k++) {
      o.X.w[k] = __shfl_down_sync(0xffffffffu, acc.X.w[k], d);
      o.Y.w[k] = __shfl_down_sync(0xffffffffu, acc.Y.w[k], d);
      o.ZZ.w[k] = __shfl_down_sync(0xffffffffu, acc.ZZ.w[k], d);
      o.ZZZ.w[k] = __shfl_down_sync(0xffffffffu, acc.ZZZ.w[k], d);
    }
    acc = g1_add(acc, o);
  }
  if (lane != 0) return;
  if (out) out[i] = acc;
  if (out48) {
    uint8_t b[48];
    g1_compress(acc, b);
    for (int k = 0; k < 48; k++) out48[48 * (size_t)i + k] = b[k];
  }
}

// ------------------------------------------------------------------ host plan
int msm_size_class(uint32_t K) { return K <= 8 ? 0 : K <= 32 ? 1 : K <= 96 ? 2 : 3; }

void MsmPlan::build(const std::vector<uint32_t> &K, const MsmTuning &tune) {
  const size_t n = K.size();
  start.assign(n + 1, 0);
  for (size_t i = 0; i < n; i++) start[i + 1] = start[i] + K[i];
  terms = start[n];
  term_c.assign(terms, 0);
  pstart.assign(n + 1, 0);
  // chunks per class, longest first inside a class so that a unit's lanes finish together
  std::vector<MsmChunk> per_class[MSM_CLASSES];
  for (size_t i = 0; i < n; i++) {
    const int cls = msm_size_class(K[i]);
    const uint32_t t = std::max<uint32_t>(1, tune.chunk[cls]);
    const uint32_t nch = K[i] == 0 ? 0 : (K[i] + t - 1) / t;
    pstart[i + 1] = pstart[i] + nch;
    for (uint32_t k = 0; k < nch; k++) {
      const uint32_t first = start[i] + k * t;
      const uint32_t cnt = std::min(t, start[i] + K[i] - first);
      per_class[cls].push_back({first, cnt, pstart[i] + k, 0});
    }
    for (uint32_t j = start[i]; j < start[i + 1]; j++) term_c[j] = (uint8_t)tune.window[cls];
  }
  chunks.clear();
  unit_c.clear();
  for (int cls = 0; cls < MSM_CLASSES; cls++) {
    auto &v = per_class[cls];
    std::stable_sort(v.begin(), v.end(), [](const MsmChunk &a, const MsmChunk &b) { return a.count > b.count; });
    for (size_t u = 0; u < v.size(); u += 32) {
      for (size_t k = u; k < std::min(v.size(), u + 32); k++) chunks.push_back(v[k]);
      for (size_t k = std::min(v.size(), u + 32); k < u + 32; k++) chunks.push_back({0, 0, 0xffffffffu, 0});
      unit_c.push_back((uint8_t)tune.window[cls]);
    }
  }
  nparts = pstart[n];
}

// Device buffers for one plan (arena-allocated, valid for the current call).
void MsmDevice::upload(Runtime &rt, const MsmPlan &p, cudaStream_t s) {
  auto put = [&](const void *h, size_t bytes) {
    uint8_t *d = rt.arena.alloc<uint8_t>(bytes ? bytes : 1);
    if (bytes) {
      uint8_t *st = rt.staging.alloc(bytes);
      std::memcpy(st, h, bytes);
      CUBBS_CHECK(cudaMemcpyAsync(d, st, bytes, cudaMemcpyHostToDevice, s));
    }
    return d;
  };
  n = (uint32_t)(p.pstart.size() - 1);
  nterms = p.terms;
  nchunks = (uint32_t)p.chunks.size();
  nunits = (uint32_t)p.unit_c.size();
  term_c = put(p.term_c.data(), p.term_c.size());
  chunks = reinterpret_cast<MsmChunk *>(put(p.chunks.data(), p.chunks.size() * sizeof(MsmChunk)));
  unit_c = put(p.unit_c.data(), p.unit_c.size());
  pstart = reinterpret_cast<uint32_t *>(put(p.pstart.data(), p.pstart.size() * 4));
  phi = rt.arena.alloc<g1a>(nterms ? nterms : 1);
  koff = rt.arena.alloc<uint32_t>(10 * (size_t)(nterms ? nterms : 1));
  partials = rt.arena.alloc<g1>(p.nparts ? p.nparts : 1);
  counter = rt.arena.alloc<uint32_t>(1);
}

size_t MsmDevice::arena_bytes(const MsmPlan &p) {
  return p.term_c.size() + p.chunks.size() * sizeof(MsmChunk) + p.unit_c.size() + p.pstart.size() * 4 +
         (size_t)p.terms * (sizeof(g1a) + 40) + (size_t)p.nparts * sizeof(g1) + 8 * 256;
}

void launch_msm_prep(cudaStream_t s, const MsmDevice &d, const g1a *pts, const VarJob *jobs, const fr *scalars) {
  if (d.nterms)
    k_msm_prep<<<blocks_for(d.nterms, 128), 128, 0, s>>>(pts, jobs, scalars, d.term_c, d.nterms, d.phi, d.koff);
}

void launch_msm_main(cudaStream_t s, const MsmDevice &d, const g1a *pts, const VarJob *jobs, int sm_count, g1 *out,
                     uint8_t *out48) {
  CUBBS_CHECK(cudaMemsetAsync(d.counter, 0, 4, s));
  if (d.nunits)
    k_msm_chunks<<<sm_count * 4, 128, 0, s>>>(pts, jobs, d.phi, d.koff, d.chunks, d.nchunks, d.unit_c, d.nunits,
                                              d.counter, d.partials);
  if (d.n) k_msm_reduce<<<blocks_for((size_t)d.n * 32, 128), 128, 0, s>>>(d.partials, d.pstart, d.n, out, out48);
}


// ------------------------------------------------------------------ benchmark workload
DEV uint64_t splitmix64(uint64_t &x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
uint64_t splitmix64_host(uint64_t &x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Term j: scalar uniform mod r and point u_j * P1 (u_j uniform mod r) from the
// fixed-base table of generator 0, both from a splitmix64 stream of (seed, j).
__global__ void __launch_bounds__(128) k_msm_gen(uint64_t seed, uint32_t n, FixedTable t, fr *scalars, g1a *pts,
                                                 VarJob *jobs) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  uint64_t x = seed ^ (0xd1b54a32d192ed03ull * (uint64_t)(j + 1));
  uint8_t b[48];
  for (int r = 0; r < 2; r++) {
    for (int k = 0; k < 6; k++) {
      uint64_t v = splitmix64(x);
      for (int q = 0; q < 8; q++) b[8 * k + q] = (uint8_t)(v >> (8 * q));
    }
    fr s = fr_raw_from_okm(b);
    if (r == 0) {
      scalars[j] = s;
      continue;
    }
    g1 acc = g1_inf();
    uint32_t carry = 0;
    const uint32_t full = 1u << t.w;
#pragma unroll 1
    for (int k = 0; k < t.nwin; k++) {
      const int pos = k * t.w;
      uint32_t d = carry;
      if (pos < 256) {
        const int wi = pos >> 5, sh = pos & 31;
        uint64_t v = (uint64_t)s.w[wi] | ((uint64_t)(wi + 1 < 8 ? s.w[wi + 1] : 0) << 32);
        d += (uint32_t)((v >> sh) & (full - 1));
      }
      bool neg = false;
      if (d > (uint32_t)t.half) {
        d = full - d;
        neg = true;
        carry = 1;
      } else {
        carry = 0;
      }
      if (d) {
        g1a e = t.entries[(size_t)k * t.half + d - 1];  // generator 0 (P1)
        if (neg) e.y = fp_neg(e.y);
        acc = g1_add_aff(acc, e);
      }
    }
    g1a a;
    g1_to_aff(acc, a);
    pts[j] = a;
    jobs[j] = {j, 0};
  }
}

__global__ void __launch_bounds__(128) k_msm_compress_aff(const g1a *pts, uint32_t n, uint8_t *out48) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  uint8_t b[48];
  g1_compress_aff(pts[j], b);
  for (int k = 0; k < 48; k++) out48[48 * (size_t)j + k] = b[k];
}

__global__ void k_count_nonzero(const int32_t *st, uint32_t n, uint32_t *bad) {
  uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n && st[j] != DEC_OK) atomicAdd(bad, 1u);
}

namespace {
std::vector<uint32_t> draw_k(uint64_t seed, size_t n, uint32_t kmin, uint32_t kmax) {
  std::vector<uint32_t> K(n);
  uint64_t x = seed;
  for (size_t i = 0; i < n; i++) K[i] = kmin + (uint32_t)(splitmix64_host(x) % (uint64_t)(kmax - kmin + 1));
  return K;
}

struct MsmWork {
  std::vector<uint32_t> K;
  uint32_t terms = 0;
  fr *sc = nullptr;
  g1a *pts = nullptr;
  VarJob *jobs = nullptr;
};

MsmWork make_work(Runtime &rt, cudaStream_t s, uint64_t seed, const std::vector<uint32_t> &K) {
  MsmWork w;
  w.K = K;
  for (uint32_t k : K) w.terms += k;
  w.sc = rt.arena.alloc<fr>(w.terms);
  w.pts = rt.arena.alloc<g1a>(w.terms);
  w.jobs = rt.arena.alloc<VarJob>(w.terms);
  if (w.terms) k_msm_gen<<<blocks_for(w.terms, 128), 128, 0, s>>>(seed, w.terms, rt.table(), w.sc, w.pts, w.jobs);
  CUBBS_CHECK(cudaGetLastError());
  return w;
}

// mean ms of `reps` engine runs (prep + persistent launch + reduction) on `w` with `tune`;
// the kernels are the same for every candidate, so no warm-up run is needed
float time_engine(Runtime &rt, cudaStream_t s, const MsmWork &w, const MsmTuning &tune, int reps, uint8_t *out48,
                  cudaEvent_t e0, cudaEvent_t e1) {
  MsmPlan p;
  p.build(w.K, tune);
  size_t mark = rt.arena.used;
  MsmDevice d;
  d.upload(rt, p, s);
  CUBBS_CHECK(cudaEventRecord(e0, s));
  for (int r = 0; r < reps; r++) {
    launch_msm_prep(s, d, w.pts, w.jobs, w.sc);
    launch_msm_main(s, d, w.pts, w.jobs, rt.sm_count, nullptr, out48);
  }
  CUBBS_CHECK(cudaEventRecord(e1, s));
  CUBBS_CHECK(cudaEventSynchronize(e1));
  float ms = 0;
  CUBBS_CHECK(cudaEventElapsedTime(&ms, e0, e1));
  rt.arena.used = mark;  // the plan's buffers are free again
  rt.staging.reset();
  return ms / reps;
}
}  // namespace

}  // namespace cubbs

using namespace cubbs;

// Uneven MSM benchmark (config 4): n_msms MSMs with K ~ U{k_min..k_max} drawn
// from `seed`, points u * P1 and scalars uniform mod r generated on the
// device.  With tune != 0 the chunk length and window of each size class are
// chosen by timing candidates on a 1024-MSM sample of that class, and kept for
// later g1_msm_batch_v2 calls.  The engine (prep + persistent launch +
// reduction) is captured in a CUDA graph and replayed warmup + steps times
// with a 256 MiB L2 flush before each; ms_out gets the timed replays.
// decode_ms: decompression with subgroup check of all points (the work the
// ABI path adds).  checked/mismatch: the first 64 MSMs recomputed with one GLV
// multiplication per term and compared.  tuning_out[2 * MSM_CLASSES]: chunk
// lengths, then windows.
extern "C" int32_t cubbs_bbs_gpu_msm_uneven_bench_v2(uint32_t abi, size_t n_msms, uint32_t k_min, uint32_t k_max,
                                                    uint64_t seed, int32_t tune, int32_t warmup, int32_t steps,
                                                    float *ms_out, float *decode_ms, uint32_t *tuning_out,
                                                    uint32_t *checked, uint32_t *mismatch) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || n_msms == 0 || n_msms > (1u << 20) || k_min == 0 || k_max < k_min ||
      k_max > 4096 || steps <= 0 || warmup < 0 || !ms_out || !decode_ms || !tuning_out || !checked || !mismatch)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    cudaStream_t s = rt.stream;
    rt.ensure_table(2);
    const std::vector<uint32_t> K = draw_k(seed, n_msms, k_min, k_max);
    size_t terms = 0;
    for (uint32_t k : K) terms += k;
    rt.arena.reserve(terms * (sizeof(fr) + 2 * sizeof(g1a) + sizeof(VarJob) + 48 + 4 + 40 + sizeof(g1)) +
                     n_msms * (sizeof(g1) * 4 + 64) + ((size_t)64 << 20));
    rt.staging.reserve(((size_t)64 << 20) + n_msms * 64 + terms * 8);
    cudaEvent_t e0, e1;
    CUBBS_CHECK(cudaEventCreate(&e0));
    CUBBS_CHECK(cudaEventCreate(&e1));
    // ---- autotune: coordinate descent over the size classes on a sample with the
    // workload's own K distribution (all classes share the device, as in the run)
    MsmTuning best = rt.sh.msm_tuning;
    if (tune) {
      const uint32_t lo[MSM_CLASSES] = {2, 9, 33, 97}, hi[MSM_CLASSES] = {8, 32, 96, 0xffffffffu};
      const uint32_t chunks[] = {2, 4, 8, 16, 32, 64};
      const size_t ns = std::min<size_t>(n_msms, 4096);
      size_t mark = rt.arena.used;
      MsmWork w = make_work(rt, s, seed ^ 0x77ull, draw_k(seed + 99, ns, k_min, k_max));
      uint8_t *o = rt.arena.alloc<uint8_t>(48 * ns);
      time_engine(rt, s, w, best, 1, o, e0, e1);  // first launch of the kernels, untimed
      float cur = time_engine(rt, s, w, best, 1, o, e0, e1);
      for (int cls = 0; cls < MSM_CLASSES; cls++) {
        const uint32_t a = std::max(lo[cls], k_min), b = std::min(hi[cls], k_max);
        if (a > b) continue;
        for (uint32_t t : chunks) {
          if (t > 2 * b) continue;
          for (int c = 4; c <= 6; c++) {
            MsmTuning cand = best;
            cand.chunk[cls] = t;
            cand.window[cls] = (uint32_t)c;
            const float ms = time_engine(rt, s, w, cand, 1, o, e0, e1);
            if (ms < cur) {
              cur = ms;
              best = cand;
            }
          }
        }
      }
      rt.arena.used = mark;
      rt.set_msm_tuning(best);
    }
    for (int c = 0; c < MSM_CLASSES; c++) {
      tuning_out[c] = best.chunk[c];
      tuning_out[MSM_CLASSES + c] = best.window[c];
    }
    // ---- the workload
    MsmWork w = make_work(rt, s, seed, K);
    // decode cost of the same points (compress, then decompress + subgroup check)
    uint8_t *p48 = rt.arena.alloc<uint8_t>(48 * (size_t)w.terms);
    g1a *dec = rt.arena.alloc<g1a>(w.terms);
    int32_t *dst = rt.arena.alloc<int32_t>(w.terms);
    uint32_t *bad = rt.arena.alloc<uint32_t>(1);
    k_msm_compress_aff<<<blocks_for(w.terms, 128), 128, 0, s>>>(w.pts, w.terms, p48);
    CUBBS_CHECK(cudaEventRecord(e0, s));
    launch_g1_decode(s, p48, 48, w.terms, dec, dst, true);
    CUBBS_CHECK(cudaEventRecord(e1, s));
    CUBBS_CHECK(cudaMemsetAsync(bad, 0, 4, s));
    k_count_nonzero<<<blocks_for(w.terms, 256), 256, 0, s>>>(dst, w.terms, bad);
    CUBBS_CHECK(cudaEventSynchronize(e1));
    CUBBS_CHECK(cudaEventElapsedTime(decode_ms, e0, e1));
    uint32_t hbad = 0;
    CUBBS_CHECK(cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, s));
    // ---- plan, graph capture, timed replays
    MsmPlan p;
    p.build(K, best);
    MsmDevice d;
    d.upload(rt, p, s);
    uint8_t *out48 = rt.arena.alloc<uint8_t>(48 * n_msms);
    CUBBS_CHECK(cudaStreamSynchronize(s));
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    CUBBS_CHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    launch_msm_prep(s, d, w.pts, w.jobs, w.sc);
    launch_msm_main(s, d, w.pts, w.jobs, rt.sm_count, nullptr, out48);
    CUBBS_CHECK(cudaStreamEndCapture(s, &graph));
    CUBBS_CHECK(cudaGraphInstantiate(&exec, graph, 0));
    static uint8_t *flush = nullptr;
    const size_t FLUSH = (size_t)256 << 20;
    if (!flush) CUBBS_CHECK(cudaMalloc(&flush, FLUSH));
    for (int k = 0; k < warmup + steps; k++) {
      CUBBS_CHECK(cudaMemsetAsync(flush, k & 0xff, FLUSH, s));
      CUBBS_CHECK(cudaEventRecord(e0, s));
      CUBBS_CHECK(cudaGraphLaunch(exec, s));
      CUBBS_CHECK(cudaEventRecord(e1, s));
      CUBBS_CHECK(cudaEventSynchronize(e1));
      float ms = 0;
      CUBBS_CHECK(cudaEventElapsedTime(&ms, e0, e1));
      if (k >= warmup) ms_out[k - warmup] = ms;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    // ---- check: first 64 MSMs with one GLV multiplication per term
    const uint32_t nchk = (uint32_t)std::min<size_t>(64, n_msms);
    const uint32_t tchk = p.start[nchk];
    g1 *v = rt.arena.alloc<g1>(tchk);
    launch_var_mul(s, w.pts, w.jobs, w.sc, tchk, v);
    uint32_t *dstart = rt.arena.alloc<uint32_t>(nchk + 1);
    CUBBS_CHECK(cudaMemcpyAsync(dstart, p.start.data(), 4 * (nchk + 1), cudaMemcpyHostToDevice, s));
    uint8_t *ref48 = rt.arena.alloc<uint8_t>(48 * nchk);
    k_msm_reduce<<<blocks_for((size_t)nchk * 32, 128), 128, 0, s>>>(v, dstart, nchk, nullptr, ref48);
    std::vector<uint8_t> a(48 * nchk), b(48 * nchk);
    CUBBS_CHECK(cudaMemcpyAsync(a.data(), out48, a.size(), cudaMemcpyDeviceToHost, s));
    CUBBS_CHECK(cudaMemcpyAsync(b.data(), ref48, b.size(), cudaMemcpyDeviceToHost, s));
    CUBBS_CHECK(cudaStreamSynchronize(s));
    CUBBS_CHECK(cudaGetLastError());
    uint32_t mm = 0;
    for (uint32_t i = 0; i < nchk; i++) mm += std::memcmp(&a[48 * i], &b[48 * i], 48) != 0;
    *checked = nchk;
    *mismatch = mm + hbad;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// Uneven-MSM engine settings per size class of K (K <= 8, <= 32, <= 96,
// larger): chunk length (terms per lane, 1..256) and window width
// (4..MSM_C_MAX).  Non-null chunk_in / window_in replace the process's
// settings (both or neither; out-of-range values are rejected), then the
// settings in force are written to chunk_out / window_out when non-null.
extern "C" int32_t cubbs_bbs_gpu_msm_tuning_v2(const uint32_t *chunk_in, const uint32_t *window_in,
                                               uint32_t *chunk_out, uint32_t *window_out) {
  if ((chunk_in == nullptr) != (window_in == nullptr)) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (chunk_in)
    for (int c = 0; c < MSM_CLASSES; c++)
      if (chunk_in[c] < 1 || chunk_in[c] > 256 || window_in[c] < 4 || window_in[c] > MSM_C_MAX)
        return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    if (chunk_in) {
      MsmTuning t;
      for (int c = 0; c < MSM_CLASSES; c++) {
        t.chunk[c] = chunk_in[c];
        t.window[c] = window_in[c];
      }
      rt.set_msm_tuning(t);
    }
    for (int c = 0; c < MSM_CLASSES; c++) {
      if (chunk_out) chunk_out[c] = rt.sh.msm_tuning.chunk[c];
      if (window_out) window_out[c] = rt.sh.msm_tuning.window[c];
    }
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}
