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
// Work is grouped into units: 32 chunks of the same window width (thread
// mode), one whole MSM (warp mode: the warp's lanes share the MSM's buckets,
// each lane owning the buckets of its index mod 32; windows 4..12), or one
// pairing check.  The persistent kernel's warps take units from an atomic
// counter until none are left, so uneven MSMs and pairing checks share one
// launch.  A second kernel sums the partials of each MSM (one warp per MSM)
// and compresses the result.  Mode, chunk length t and window c are chosen
// per size class of K by an autotuner (t >= K: one lane per MSM; t < K: the
// MSM is spread over several lanes and joined by the reduction).  The
// general MSM entry point replays the engine's kernels from captured CUDA
// graphs (k_prims.cu).
//
// Reference counterpart: route 4 (native/cuda/src/kernels/variable_base_universal.cuh:
// 337-644) and the Pippenger kernel (kernels/large_msm.cuh:322-416).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "pairing_team.cuh"
#include "runtime.cuh"

namespace cubbs {

#define MSM_C_MAX MSM_THREAD_C_MAX  // thread-mode buckets live in per-lane local memory: 64 XYZZ points (12 KB)

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

// One chunk by the bucket method; returns XYZZ.  Out of line: the engine
// kernel's three unit kinds then get register allocations of their own.
static __device__ __noinline__ g1 msm_chunk(const g1a *pts, const VarJob *jobs, const g1a *phi,
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

// ---------------------------------------------------------------- warp mode
// One MSM on one warp, windows from the top (Horner).  Per window: the lanes
// compute the signed digits of the MSM's 2K half-terms into shared memory and
// sort the nonzero ones by owner lane (bucket index mod 32) with a
// shared-memory counting sort; every lane then adds its own terms into the
// buckets it owns (no two lanes touch one bucket, so no locks), in step with
// the other lanes.  The weighted bucket sum sum_b b B_b comes from the lanes'
// own running sums plus a suffix scan across the lanes.  All lanes return the
// MSM's sum.
constexpr uint32_t MSM_WARP_MAX_TERMS = 512;  // larger MSMs of a warp-mode class run in thread mode
constexpr uint32_t MSM_WARP_MAX_HALVES = 2 * MSM_WARP_MAX_TERMS;
// per-warp scratch ahead of the buckets: digits and sorted order (int16 each),
// owner counts and positions
struct WarpMsmScratch {
  int16_t dig[MSM_WARP_MAX_HALVES];
  int16_t order[MSM_WARP_MAX_HALVES];
  int32_t cnt[32], pos[32];
};
DEV g1 shfl_g1(const g1 &p, int delta, bool xor_mode) {
  g1 r;
#pragma unroll
  for (int i = 0; i < 12; i++) {
    if (xor_mode) {
      r.X.w[i] = __shfl_xor_sync(0xffffffffu, p.X.w[i], delta);
      r.Y.w[i] = __shfl_xor_sync(0xffffffffu, p.Y.w[i], delta);
      r.ZZ.w[i] = __shfl_xor_sync(0xffffffffu, p.ZZ.w[i], delta);
      r.ZZZ.w[i] = __shfl_xor_sync(0xffffffffu, p.ZZZ.w[i], delta);
    } else {
      r.X.w[i] = __shfl_down_sync(0xffffffffu, p.X.w[i], delta);
      r.Y.w[i] = __shfl_down_sync(0xffffffffu, p.Y.w[i], delta);
      r.ZZ.w[i] = __shfl_down_sync(0xffffffffu, p.ZZ.w[i], delta);
      r.ZZZ.w[i] = __shfl_down_sync(0xffffffffu, p.ZZZ.w[i], delta);
    }
  }
  return r;
}
// every lane gets the sum of the 32 lanes' points
DEV g1 warp_sum_all(g1 a) {
#pragma unroll 1
  for (int d = 16; d > 0; d >>= 1) a = g1_add(a, shfl_g1(a, d, true));
  return a;
}
static __device__ __noinline__ g1 msm_warp(const g1a *pts, const VarJob *jobs, const g1a *phi, const uint32_t *koff, uint32_t first,
                uint32_t count, int c, g1 *bk, WarpMsmScratch *ws, int lane) {
  const int nb = 1 << (c - 1);
  const int m = nb >= 32 ? nb / 32 : 1;  // buckets per lane; with nb < 32 lanes >= nb own none
  const int nwin = (130 + c - 1) / c;
  const uint32_t nh = 2 * count;
  g1 acc = g1_inf();
#pragma unroll 1
  for (int w = nwin - 1; w >= 0; w--) {
    if (w != nwin - 1) {
#pragma unroll 1
      for (int k = 0; k < c; k++) acc = g1_dbl(acc);
    }
    ws->cnt[lane] = 0;
    __syncwarp();
    bool any = false;
#pragma unroll 1
    for (uint32_t h = lane; h < nh; h += 32) {
      const uint32_t j = first + (h >> 1);
      int d = 0;
      if (!(jobs[j].flags & 1)) d = msm_digit(koff + 10 * (size_t)j + 5 * (h & 1), w, c);
      ws->dig[h] = (int16_t)d;
      if (d) {
        any = true;
        atomicAdd(&ws->cnt[((d < 0 ? -d : d) - 1) & 31], 1);
      }
    }
    if (!__any_sync(0xffffffffu, any)) continue;
    __syncwarp();
    // exclusive prefix of the owner counts -> each owner's run in order[]
    const int mine = ws->cnt[lane];
    int incl = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int o = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += o;
    }
    const int off = incl - mine;
    ws->pos[lane] = off;
    const int most = __reduce_max_sync(0xffffffffu, (unsigned)mine);
    __syncwarp();
#pragma unroll 1
    for (uint32_t h = lane; h < nh; h += 32) {
      const int d = ws->dig[h];
      if (d) ws->order[atomicAdd(&ws->pos[((d < 0 ? -d : d) - 1) & 31], 1)] = (int16_t)h;
    }
#pragma unroll 1
    for (int k = 0; k < m; k++) {
      const int b = lane + 32 * k;
      if (b < nb) bk[b] = g1_inf();
    }
    __syncwarp();
    // the owners add their terms in step
#pragma unroll 1
    for (int k = 0; k < most; k++) {
      if (k < mine) {
        const uint32_t h = (uint32_t)ws->order[off + k];
        const int d = ws->dig[h];
        const uint32_t j = first + (h >> 1);
        g1a pt = (h & 1) ? phi[j] : pts[jobs[j].point];
        if (d < 0) pt.y = fp_neg(pt.y);
        const int b = (d < 0 ? -d : d) - 1;
        bk[b] = g1_add_aff(bk[b], pt);
      }
    }
    __syncwarp();
    // sum_b b B_b: lane l owns b = l + 1 + 32k (k < m).  C_l = sum_k B, E_l = sum_k k B
    g1 run = g1_inf(), E = g1_inf();
#pragma unroll 1
    for (int k = m - 1; k >= 1; k--) {
      run = g1_add(run, bk[lane + 32 * k]);
      E = g1_add(E, run);
    }
    g1 C = lane < nb ? g1_add(run, bk[lane]) : g1_inf();
    // inclusive suffix scan S_l = sum_{l' >= l} C_l'; sum_l S_l = sum_l (l + 1) C_l
#pragma unroll 1
    for (int d = 1; d < 32; d <<= 1) {
      const g1 o = shfl_g1(C, d, false);
      const g1 t = g1_add(C, o);
      if (lane + d < 32) C = t;
    }
    g1 W = warp_sum_all(C);
    if (m > 1) {
      g1 T = warp_sum_all(E);
#pragma unroll 1
      for (int k = 0; k < 5; k++) T = g1_dbl(T);  // 32 sum_l E_l
      W = g1_add(W, T);
    }
    acc = g1_add(acc, W);
    __syncwarp();
  }
  return acc;
}

// ---------------------------------------------------------------- persistent engine
// Warps take units from an atomic counter until none are left: 32 thread-mode
// chunks, one warp-mode MSM, or one pairing check (pp::pairing_check over the
// warp's shared-memory slots), so uneven MSMs and pairings share one launch.
// Dynamic shared memory per warp: smem_per_warp bytes (the warp-mode scratch
// and buckets, or the pairing slots, whichever is larger).
struct EngineArgs {
  const g1a *pts;
  const VarJob *jobs;
  const g1a *phi;
  const uint32_t *koff;
  const MsmChunk *chunks;
  uint32_t nchunks;
  const MsmUnit *units;
  uint32_t nunits;
  const uint32_t *start;  // term offsets of the MSMs (warp units)
  uint32_t *counter;
  g1 *partials;
  const uint32_t *pstart;
  g1 *gbuckets;
  uint32_t gbucket_stride;  // XYZZ points per warp slot of gbuckets
  uint32_t smem_per_warp;
  const PairJob *pjobs;
  const line2 *lines;
  uint8_t *pok;
};
static __device__ __noinline__ bool engine_pairing(fp *sl, int lane, const PairJob &j, const line2 *lines) {
  const bool skip[2] = {(j.flags & 1) != 0, (j.flags & 2) != 0};
  const line2 *L[2] = {lines + (size_t)j.slot_a * MILLER_LINES, lines + (size_t)j.slot_b * MILLER_LINES};
  const g1a P[2] = {j.pa, j.pb};
  return pp::pairing_check(sl, lane, P, L, skip);
}
__global__ void __launch_bounds__(128) k_msm_engine(EngineArgs a) {
  extern __shared__ __align__(16) uint8_t eng_smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint8_t *mine = eng_smem + (size_t)warp * a.smem_per_warp;
  const uint32_t gslot = blockIdx.x * (blockDim.x >> 5) + warp;
#pragma unroll 1
  for (;;) {
    uint32_t unit = 0;
    if (lane == 0) unit = atomicAdd(a.counter, 1u);
    unit = __shfl_sync(0xffffffffu, unit, 0);
    if (unit >= a.nunits) break;
    const MsmUnit u = a.units[unit];
    const uint32_t kind = u.kind_c >> 8, c = u.kind_c & 0xff;
    if (kind == MSM_UNIT_THREAD) {
      const uint32_t ci = u.index + lane;
      if (ci < a.nchunks) {
        const MsmChunk ch = a.chunks[ci];
        if (ch.slot != 0xffffffffu)  // padding of a unit's last lanes
          a.partials[ch.slot] = msm_chunk(a.pts, a.jobs, a.phi, a.koff, ch.first, ch.count, (int)c);
      }
    } else if (kind == MSM_UNIT_WARP) {
      WarpMsmScratch *ws = reinterpret_cast<WarpMsmScratch *>(mine);
      const uint32_t nb = 1u << (c - 1);
      const bool in_smem = c <= MSM_WARP_SMEM_C_MAX;
      const uint32_t first = a.start[u.index], count = a.start[u.index + 1] - first;
      // a unit the launch has no room for is skipped and reported (counter[1])
      const bool fits = 2 * count <= MSM_WARP_MAX_HALVES &&
                        (in_smem ? sizeof(WarpMsmScratch) + (size_t)nb * sizeof(g1) <= a.smem_per_warp
                                 : (a.gbuckets != nullptr && nb <= a.gbucket_stride));
      if (!fits) {
        if (lane == 0) atomicOr(a.counter + 1, 1u);
        continue;
      }
      g1 *bk = in_smem ? reinterpret_cast<g1 *>(mine + sizeof(WarpMsmScratch))
                       : a.gbuckets + (size_t)gslot * a.gbucket_stride;
      const g1 r = msm_warp(a.pts, a.jobs, a.phi, a.koff, first, count, (int)c, bk, ws, lane);
      if (lane == 0) a.partials[a.pstart[u.index]] = r;
    } else {
      const PairJob &j = a.pjobs[u.index];
      if ((size_t)PP_SLOTS * sizeof(fp) > a.smem_per_warp) {
        if (lane == 0) atomicOr(a.counter + 1, 2u);
        continue;
      }
      if (j.active != 1) {
        if (lane == 0 && j.active == 0) a.pok[u.index] = 0;
      } else {
        const bool one = engine_pairing(reinterpret_cast<fp *>(mine), lane, j, a.lines);
        if (lane == 0) a.pok[u.index] = one ? 1 : 0;
      }
    }
    __syncwarp();
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

void MsmPlan::build(const std::vector<uint32_t> &K, const MsmTuning &tune, uint32_t pairings) {
  const size_t n = K.size();
  start.assign(n + 1, 0);
  for (size_t i = 0; i < n; i++) start[i + 1] = start[i] + K[i];
  terms = start[n];
  term_c.assign(terms, 0);
  pstart.assign(n + 1, 0);
  max_warp_c = 0;
  max_warp_smem_c = 0;
  pair_units = pairings;
  units.clear();
  chunks.clear();
  // pairing checks first: each takes a warp for milliseconds, so they must
  // not be the launch's tail
  for (uint32_t k = 0; k < pairings; k++) units.push_back({MSM_UNIT_PAIR << 8, k});
  // thread-mode chunks per class, longest first inside a class so that a
  // unit's lanes finish together; warp-mode MSMs one unit each
  std::vector<MsmChunk> per_class[MSM_CLASSES];
  std::vector<std::pair<uint32_t, uint32_t>> warp_msms;  // (K, MSM)
  for (size_t i = 0; i < n; i++) {
    const int cls = msm_size_class(K[i]);
    const bool warp = tune.mode[cls] == MSM_MODE_WARP && K[i] <= MSM_WARP_MAX_TERMS;
    const uint32_t c = warp ? tune.window[cls] : std::min<uint32_t>(tune.window[cls], MSM_THREAD_C_MAX);
    for (uint32_t j = start[i]; j < start[i + 1]; j++) term_c[j] = (uint8_t)c;
    if (warp) {
      pstart[i + 1] = pstart[i] + (K[i] ? 1 : 0);
      if (K[i]) warp_msms.emplace_back(K[i], (uint32_t)i);
      continue;
    }
    const uint32_t t = std::max<uint32_t>(1, tune.chunk[cls]);
    const uint32_t nch = K[i] == 0 ? 0 : (K[i] + t - 1) / t;
    pstart[i + 1] = pstart[i] + nch;
    for (uint32_t k = 0; k < nch; k++) {
      const uint32_t first = start[i] + k * t;
      const uint32_t cnt = std::min(t, start[i] + K[i] - first);
      per_class[cls].push_back({first, cnt, pstart[i] + k, 0});
    }
  }
  std::stable_sort(warp_msms.begin(), warp_msms.end(), [](auto &x, auto &y) { return x.first > y.first; });
  for (const auto &wm : warp_msms) {
    const uint32_t c = tune.window[msm_size_class(wm.first)];
    units.push_back({MSM_UNIT_WARP << 8 | c, wm.second});
    max_warp_c = std::max(max_warp_c, c);
    if (c <= MSM_WARP_SMEM_C_MAX) max_warp_smem_c = std::max(max_warp_smem_c, c);
  }
  // (largest class first; small-first measured the same on GB300)
  for (int cls = MSM_CLASSES - 1; cls >= 0; cls--) {
    auto &v = per_class[cls];
    std::stable_sort(v.begin(), v.end(), [](const MsmChunk &a, const MsmChunk &b) { return a.count > b.count; });
    const uint32_t c = std::min<uint32_t>(tune.window[cls], MSM_THREAD_C_MAX);
    for (size_t u = 0; u < v.size(); u += 32) {
      units.push_back({MSM_UNIT_THREAD << 8 | c, (uint32_t)chunks.size()});
      for (size_t k = u; k < std::min(v.size(), u + 32); k++) chunks.push_back(v[k]);
      for (size_t k = std::min(v.size(), u + 32); k < u + 32; k++) chunks.push_back({0, 0, 0xffffffffu, 0});
    }
  }
  nparts = pstart[n];
}

namespace {
// Launch shape of the engine for a plan: warps per block and shared memory per
// warp (warp-mode scratch and buckets, pairing slots), blocks from the
// occupancy the device reports.
void engine_shape(const MsmPlan &p, int sm_count, uint32_t &wpb, uint32_t &smem_per_warp, uint32_t &grid,
                  uint32_t &gstride) {
  // A warp unit keeps its buckets in shared memory when its window is at most
  // MSM_WARP_SMEM_C_MAX, in its warp's slot of the global buckets otherwise;
  // one plan may hold both kinds (windows differ between size classes).
  size_t per = 0;
  gstride = 0;
  if (p.max_warp_c) {
    per = sizeof(WarpMsmScratch);
    if (p.max_warp_smem_c) per += ((size_t)1 << (p.max_warp_smem_c - 1)) * sizeof(g1);
    if (p.max_warp_c > MSM_WARP_SMEM_C_MAX) gstride = 1u << (p.max_warp_c - 1);
  }
  if (p.pair_units) per = std::max(per, (size_t)PP_SLOTS * sizeof(fp));
  per = (per + 15) & ~(size_t)15;
  const size_t budget = (size_t)200 << 10;
  wpb = per * 4 <= budget ? 4 : per * 2 <= budget ? 2 : 1;
  smem_per_warp = (uint32_t)per;
  static const bool attr = [] {
    CUBBS_CHECK(cudaFuncSetAttribute(k_msm_engine, cudaFuncAttributeMaxDynamicSharedMemorySize, 210 << 10));
    return true;
  }();
  (void)attr;
  int per_sm = 0;
  CUBBS_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_msm_engine, (int)(32 * wpb),
                                                             wpb * smem_per_warp));
  if (per_sm < 1) per_sm = 1;
  grid = (uint32_t)(sm_count * per_sm);
}
}  // namespace

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
  nunits = (uint32_t)p.units.size();
  term_c = put(p.term_c.data(), p.term_c.size());
  chunks = reinterpret_cast<MsmChunk *>(put(p.chunks.data(), p.chunks.size() * sizeof(MsmChunk)));
  units = reinterpret_cast<MsmUnit *>(put(p.units.data(), p.units.size() * sizeof(MsmUnit)));
  pstart = reinterpret_cast<uint32_t *>(put(p.pstart.data(), p.pstart.size() * 4));
  start = reinterpret_cast<uint32_t *>(put(p.start.data(), p.start.size() * 4));
  phi = rt.arena.alloc<g1a>(nterms ? nterms : 1);
  koff = rt.arena.alloc<uint32_t>(10 * (size_t)(nterms ? nterms : 1));
  partials = rt.arena.alloc<g1>(p.nparts ? p.nparts : 1);
  counter = rt.arena.alloc<uint32_t>(2);  // [0] next unit, [1] units skipped for want of room
  engine_shape(p, rt.sm_count, warps_per_block, smem_per_warp, grid, gbucket_stride);
  gbuckets = gbucket_stride ? rt.arena.alloc<g1>((size_t)grid * warps_per_block * gbucket_stride) : nullptr;
}

size_t MsmDevice::arena_bytes(const MsmPlan &p, int sm_count) {
  uint32_t wpb, per, grid, gstride;
  engine_shape(p, sm_count, wpb, per, grid, gstride);
  const size_t g = (size_t)grid * wpb * gstride * sizeof(g1) + 256;
  return p.term_c.size() + p.chunks.size() * sizeof(MsmChunk) + p.units.size() * sizeof(MsmUnit) +
         p.pstart.size() * 4 + p.start.size() * 4 + (size_t)p.terms * (sizeof(g1a) + 40) +
         (size_t)p.nparts * sizeof(g1) + g + 10 * 256;
}

void launch_msm_prep(cudaStream_t s, const MsmDevice &d, const g1a *pts, const VarJob *jobs, const fr *scalars) {
  if (d.nterms)
    k_msm_prep<<<blocks_for(d.nterms, 128), 128, 0, s>>>(pts, jobs, scalars, d.term_c, d.nterms, d.phi, d.koff);
}

void launch_msm_main(cudaStream_t s, const MsmDevice &d, const g1a *pts, const VarJob *jobs, int sm_count, g1 *out,
                     uint8_t *out48) {
  (void)sm_count;
  CUBBS_CHECK(cudaMemsetAsync(d.counter, 0, 8, s));
  if (d.nunits) {
    EngineArgs a{pts, jobs, d.phi, d.koff, d.chunks, d.nchunks, d.units, d.nunits, d.start, d.counter, d.partials,
                 d.pstart, d.gbuckets, d.gbucket_stride, d.smem_per_warp, d.pjobs, d.lines, d.pok};
    k_msm_engine<<<d.grid, 32 * d.warps_per_block, d.warps_per_block * d.smem_per_warp, s>>>(a);
  }
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
  uint32_t herr = 0;
  CUBBS_CHECK(cudaMemcpy(&herr, d.counter + 1, 4, cudaMemcpyDeviceToHost));
  if (herr) throw CudaError(cudaErrorInvalidValue, "uneven-MSM engine: a unit had no room in its launch");
  rt.arena.used = mark;  // the plan's buffers are free again
  rt.staging.reset();
  return ms / reps;
}
}  // namespace

}  // namespace cubbs

using namespace cubbs;

// Uneven MSM benchmark (config 4): n_msms MSMs with K ~ U{k_min..k_max} drawn
// from `seed`, points u * P1 and scalars uniform mod r generated on the
// device.  With tune != 0 the mode, chunk length and window of each size
// class are chosen by timing candidates on a sample of the same size and K
// distribution (coordinate descent, largest class first), and kept for later
// g1_msm_batch_v2 calls.  The engine (prep + persistent launch +
// reduction) is captured in a CUDA graph and replayed warmup + steps times
// with a 256 MiB L2 flush before each; ms_out gets the timed replays.
// decode_ms: decompression with subgroup check of all points (the work the
// ABI path adds).  checked/mismatch: the first 64 MSMs recomputed with one GLV
// multiplication per term and compared.  tuning_out[3 * MSM_CLASSES]: chunk
// lengths, windows, then modes (0 thread, 1 warp) per size class.  The
// autotuner tries thread mode (chunks of 4..64 terms, windows 4..7) and warp
// mode (windows 4..12) for every class.
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
    // room for the widest warp-mode candidate's global buckets (window 12)
    MsmPlan widest;
    {
      MsmTuning t;
      for (int c = 0; c < MSM_CLASSES; c++) {
        t.mode[c] = MSM_MODE_WARP;
        t.window[c] = MSM_WARP_C_MAX;
      }
      widest.build(std::vector<uint32_t>(1, 2), t);
    }
    rt.arena.reserve(terms * (sizeof(fr) + 2 * sizeof(g1a) + sizeof(VarJob) + 48 + 4 + 40 + sizeof(g1)) +
                     n_msms * (sizeof(g1) * 4 + 64) + ((size_t)64 << 20) +
                     MsmDevice::arena_bytes(widest, rt.sm_count));
    rt.staging.reserve(((size_t)64 << 20) + n_msms * 64 + terms * 8);
    cudaEvent_t e0, e1;
    CUBBS_CHECK(cudaEventCreate(&e0));
    CUBBS_CHECK(cudaEventCreate(&e1));
    // ---- autotune: coordinate descent over the size classes, largest first, on
    // a sample of the workload's own size and K distribution: the launch shape
    // a candidate implies (warps and shared memory per block) only costs time
    // once the units fill the GPU, which a smaller sample would hide
    MsmTuning best = rt.sh.msm_tuning;
    if (tune) {
      const uint32_t lo[MSM_CLASSES] = {2, 9, 33, 97}, hi[MSM_CLASSES] = {8, 32, 96, 0xffffffffu};
      const uint32_t chunks[] = {4, 8, 16, 32, 64};
      const size_t ns = std::min<size_t>(n_msms, 16384);
      size_t mark = rt.arena.used;
      MsmWork w = make_work(rt, s, seed ^ 0x77ull, draw_k(seed + 99, ns, k_min, k_max));
      uint8_t *o = rt.arena.alloc<uint8_t>(48 * ns);
      time_engine(rt, s, w, best, 1, o, e0, e1);  // first launch of the kernels, untimed
      float cur = time_engine(rt, s, w, best, 1, o, e0, e1);
      for (int cls = MSM_CLASSES - 1; cls >= 0; cls--) {
        const uint32_t a = std::max(lo[cls], k_min), b = std::min(hi[cls], k_max);
        if (a > b) continue;
        for (uint32_t t : chunks) {
          if (t > 2 * b) continue;
          for (int c = 4; c <= MSM_THREAD_C_MAX; c++) {
            MsmTuning cand = best;
            cand.mode[cls] = MSM_MODE_THREAD;
            cand.chunk[cls] = t;
            cand.window[cls] = (uint32_t)c;
            const float ms = time_engine(rt, s, w, cand, 1, o, e0, e1);
            if (ms < cur) {
              cur = ms;
              best = cand;
            }
          }
        }
        // one warp per MSM, buckets shared by the warp's lanes
        for (int c = 4; c <= MSM_WARP_C_MAX; c++) {
          MsmTuning cand = best;
          cand.mode[cls] = MSM_MODE_WARP;
          cand.window[cls] = (uint32_t)c;
          const float ms = time_engine(rt, s, w, cand, 1, o, e0, e1);
          if (ms < cur) {
            cur = ms;
            best = cand;
          }
        }
      }
      rt.arena.used = mark;
      rt.set_msm_tuning(best);
    }
    for (int c = 0; c < MSM_CLASSES; c++) {
      tuning_out[c] = best.chunk[c];
      tuning_out[MSM_CLASSES + c] = best.window[c];
      tuning_out[2 * MSM_CLASSES + c] = best.mode[c];
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
// larger): mode (0 thread, 1 warp), chunk length (terms per lane, 1..256;
// thread mode) and window width (4..7 in thread mode, 4..12 in warp mode).
// Non-null chunk_in / window_in / mode_in replace the process's settings (all
// three or none; out-of-range values are rejected), then the settings in
// force are written to the non-null outputs.
extern "C" int32_t cubbs_bbs_gpu_msm_tuning_v2(const uint32_t *chunk_in, const uint32_t *window_in,
                                               const uint32_t *mode_in, uint32_t *chunk_out, uint32_t *window_out,
                                               uint32_t *mode_out) {
  if ((chunk_in == nullptr) != (window_in == nullptr) || (chunk_in == nullptr) != (mode_in == nullptr))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (chunk_in)
    for (int c = 0; c < MSM_CLASSES; c++) {
      const uint32_t cmax = mode_in[c] == MSM_MODE_WARP ? MSM_WARP_C_MAX : MSM_THREAD_C_MAX;
      if (mode_in[c] > MSM_MODE_WARP || chunk_in[c] < 1 || chunk_in[c] > 256 || window_in[c] < 4 ||
          window_in[c] > cmax)
        return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    }
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    if (chunk_in) {
      MsmTuning t;
      for (int c = 0; c < MSM_CLASSES; c++) {
        t.chunk[c] = chunk_in[c];
        t.window[c] = window_in[c];
        t.mode[c] = mode_in[c];
      }
      rt.set_msm_tuning(t);
    }
    for (int c = 0; c < MSM_CLASSES; c++) {
      if (chunk_out) chunk_out[c] = rt.sh.msm_tuning.chunk[c];
      if (window_out) window_out[c] = rt.sh.msm_tuning.window[c];
      if (mode_out) mode_out[c] = rt.sh.msm_tuning.mode[c];
    }
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}
