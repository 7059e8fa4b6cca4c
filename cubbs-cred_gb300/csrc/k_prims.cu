// Primitive ABI entry points the Rust engine probes as optional symbols
// (crates/cubbs-bbs/src/gpu_runtime.rs:300-428): generic and common-point G1
// MSMs, MSM + variable term, the ProofVerify T1/T2 pair, dual MSMs, G1 add,
// prepare-B, ProofGen T2-prepare and the pairing equality checks.
//
// All of them share one device plan: user points are decoded on the device
// (decompress + subgroup check), scalars are parsed on the device (canonical
// check), fixed-base rows run against the resident generator tables when the
// common points are a prefix of [P1, Q1, H1, ...] (route 2), every other term
// is a GLV variable-base job (route 4), and a warp per output row sums the
// terms before compression.
#include <algorithm>
#include <cstring>

#include "runtime.cuh"
#include "sha256.cuh"

namespace cubbs {

// BE canonical scalars -> raw Fr; status 0 ok / 1 non-canonical
__global__ void k_parse_scalars(const uint8_t *be, uint32_t n, fr *out, int32_t *status) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fr s;
  bool ok = fr_raw_from_be32(be + 32 * (size_t)i, s);
  out[i] = ok ? s : fr_zero();
  status[i] = ok ? 0 : 1;
}

// optional row scale: out[row*stride + g] = in[row*stride + g] * scale[row]  (raw Fr)
__global__ void k_scale_rows(fr *rows, uint32_t stride, const uint32_t *nterms, const fr *scale, uint32_t nrows) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t row = i / stride, g = i % stride;
  if (row >= nrows || g >= nterms[row]) return;
  fr sm = fr_to_mont(scale[row]);
  rows[i] = fr_mul(rows[i], sm);
}

// row r = fixed[r] (if has_fixed) + sum_{j in [start[r], start[r+1])} var[j]; warp per row.
__global__ void __launch_bounds__(128) k_row_sum(const g1 *fixed, const g1 *var, const uint32_t *start,
                                                 uint32_t rows, g1 *out) {
  uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= rows) return;
  g1 acc = g1_inf();
  uint32_t a = start[row], b = start[row + 1];
#pragma unroll 1
  for (uint32_t j = a + lane; j < b; j += 32) acc = g1_add(acc, var[j]);
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
  if (lane == 0) out[row] = fixed ? g1_add(acc, fixed[row]) : acc;
}

// negate the second G1 point of pairing jobs (e(a,b) == e(c,d) <=> e(a,b) e(-c,d) == 1)
__global__ void k_negate_pb(PairJob *j, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(j[i].flags & 2)) j[i].pb.y = fp_neg(j[i].pb.y);
}

// ---------------------------------------------------------------------------- generic multi-pairing
// prod_k e(P_k, Q_k) == 1 over K pairs with precomputed lines (one thread).
__global__ void k_multi_pairing(const g1a *P, const int32_t *slots, const uint8_t *skip, uint32_t K,
                                const line2 *lines, uint8_t *ok) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  fp12 f = fp12_one();
  int idx = 0;
#pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    f = fp12_sqr(f);
#pragma unroll 1
    for (int step = 0; step < (zabs_bit(i) ? 2 : 1); step++) {
#pragma unroll 1
      for (uint32_t k = 0; k < K; k++) {
        if (skip[k]) continue;
        line2 l = lines[(size_t)slots[k] * MILLER_LINES + idx];
        f = fp12_mul_line(f, l.a, fp2_mul_fp(l.b, P[k].x), P[k].y);
      }
      idx++;
    }
  }
  f = fp12_conj(f);
  ok[0] = fp12_is_one(final_exponentiation(f)) ? 1 : 0;
}

namespace {
bool abi_ok(uint32_t v) { return v == CUBBS_BBS_GPU_ABI_VERSION; }

template <typename T> T *upload(Runtime &rt, const T *h, size_t n) {
  T *d = rt.arena.alloc<T>(n ? n : 1);
  if (n) {
    uint8_t *st = rt.staging.alloc(n * sizeof(T));
    std::memcpy(st, h, n * sizeof(T));
    CUBBS_CHECK(cudaMemcpyAsync(d, st, n * sizeof(T), cudaMemcpyHostToDevice, rt.stream));
  }
  return d;
}

// Host copy of the compressed generators [P1, Q1, H1, ...] for prefix detection.
const std::vector<uint8_t> &host_gens_c(Runtime &rt, int count) {
  rt.ensure_generators(count);
  return rt.host_gens_c();
}

// Plan of output rows made of (a) an optional fixed-base part over a prefix of
// the generators and (b) variable-base terms over user points.
struct Plan {
  size_t rows = 0;
  // fixed part
  bool has_fixed = false;
  uint32_t fixed_stride = 0;
  std::vector<uint32_t> fixed_nterms;
  std::vector<uint8_t> fixed_scalars_be;  // rows * stride * 32
  std::vector<uint8_t> fixed_scale_be;    // optional per-row scale (rows * 32)
  // variable part
  std::vector<uint8_t> points_be;   // user points, 48 B each
  std::vector<uint32_t> var_point;  // per var job: index into points
  std::vector<uint8_t> var_scalars_be;
  std::vector<uint32_t> var_start;  // rows + 1
  uint32_t add_point(const uint8_t *p) {
    points_be.insert(points_be.end(), p, p + 48);
    return (uint32_t)(points_be.size() / 48 - 1);
  }
  void add_var(uint32_t point, const uint8_t *scalar) {
    var_point.push_back(point);
    var_scalars_be.insert(var_scalars_be.end(), scalar, scalar + 32);
  }
};

// Pairing checks that share the engine's persistent launch with the plan's
// MSMs: the items in, per-item verdicts and decode failures out.
struct PairRequest {
  const CuBbsBbsGpuPairingEqItem *items = nullptr;
  size_t n = 0;
  std::vector<int> bad;
  std::vector<uint8_t> ok;
};
bool pairing_items_ok(const CuBbsBbsGpuPairingEqItem *items, size_t n) {
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if (it.lhs_g1.len != 48 || !it.lhs_g1.data || it.rhs_g1.len != 48 || !it.rhs_g1.data || it.lhs_g2.len != 96 ||
        !it.lhs_g2.data || it.rhs_g2.len != 96 || !it.rhs_g2.data)
      return false;
  }
  return true;
}

// Device pairing jobs e(lhs_g1, lhs_g2) * e(-rhs_g1, rhs_g2) == 1 of the items
// (G2 points resolved to resident line slots, G1 points decoded with the
// subgroup check); bad[i] = 1 for an item with an undecodable point.
PairJob *prepare_pair_jobs(Runtime &rt, const CuBbsBbsGpuPairingEqItem *items, size_t n,
                                  std::vector<int> &bad) {
  std::vector<const uint8_t *> g2(2 * n);
  for (size_t i = 0; i < n; i++) {
    g2[2 * i] = items[i].lhs_g2.data;
    g2[2 * i + 1] = items[i].rhs_g2.data;
  }
  std::vector<int> slots, st;
  rt.resolve_pks(g2, slots, st);
  std::vector<uint8_t> g1b(96 * n);
  for (size_t i = 0; i < n; i++) {
    std::memcpy(&g1b[96 * i], items[i].lhs_g1.data, 48);
    std::memcpy(&g1b[96 * i + 48], items[i].rhs_g1.data, 48);
  }
  uint8_t *d = upload(rt, g1b.data(), g1b.size());
  g1a *pts = rt.arena.alloc<g1a>(2 * n);
  int32_t *pst = rt.arena.alloc<int32_t>(2 * n);
  launch_g1_decode(rt.stream, d, 48, (uint32_t)(2 * n), pts, pst, true);
  std::vector<g1a> hp(2 * n);
  std::vector<int32_t> hst(2 * n);
  CUBBS_CHECK(cudaMemcpyAsync(hp.data(), pts, sizeof(g1a) * 2 * n, cudaMemcpyDeviceToHost, rt.stream));
  CUBBS_CHECK(cudaMemcpyAsync(hst.data(), pst, 8 * n, cudaMemcpyDeviceToHost, rt.stream));
  CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
  std::vector<PairJob> jobs(n);
  bad.assign(n, 0);
  for (size_t i = 0; i < n; i++) {
    PairJob &j = jobs[i];
    j.pa = hp[2 * i];
    j.pb = hp[2 * i + 1];
    j.slot_a = slots[2 * i];
    j.slot_b = slots[2 * i + 1];
    j.flags = 0;
    j.active = 1;
    if (hst[2 * i] == DEC_BAD || hst[2 * i + 1] == DEC_BAD || st[2 * i] == DEC_BAD || st[2 * i + 1] == DEC_BAD) {
      bad[i] = 1;
      j.active = 0;
    }
    if (hst[2 * i] == DEC_INF || st[2 * i] == DEC_INF) j.flags |= 1;
    if (hst[2 * i + 1] == DEC_INF || st[2 * i + 1] == DEC_INF) j.flags |= 2;
  }
  PairJob *dj = upload(rt, jobs.data(), n);
  k_negate_pb<<<blocks_for(n, 128), 128, 0, rt.stream>>>(dj, (uint32_t)n);
  return dj;
}

// The engine's kernels (prep, persistent launch, reduction) for a plan, from a
// CUDA graph: one is captured the first time a workspace meets the plan's
// shape and device buffers (the arena hands out the same addresses to the same
// sequence of allocations) and replayed afterwards.  At most 32 graphs per
// workspace are kept.
void run_engine_graph(Runtime &rt, cudaStream_t s, const MsmPlan &mp, MsmDevice &md, const g1a *pts,
                      const VarJob *djobs, const fr *vsc, uint8_t *dout) {
  uint64_t key = 1469598103934665603ull;
  auto mix = [&key](uint64_t v) { key = (key ^ v) * 1099511628211ull; };
  for (const MsmUnit &u : mp.units) {
    mix(u.kind_c);
    mix(u.index);
  }
  for (const MsmChunk &c : mp.chunks) mix((uint64_t)c.first << 32 | c.count);
  for (uint32_t v : mp.start) mix(v);
  for (uint32_t v : mp.pstart) mix(v);
  const void *ptrs[] = {pts, djobs, vsc, dout, md.term_c, md.chunks, md.units, md.pstart, md.start, md.koff,
                        md.counter, md.phi, md.partials, md.gbuckets, md.pjobs, md.lines, md.pok};
  for (const void *q : ptrs) mix((uint64_t)(uintptr_t)q);
  mix((uint64_t)md.grid << 32 | md.warps_per_block);
  mix(md.smem_per_warp);
  auto it = rt.msm_graphs.find(key);
  if (it == rt.msm_graphs.end()) {
    if (rt.msm_graphs.size() >= 32) {
      for (auto &g : rt.msm_graphs) cudaGraphExecDestroy(g.second);
      rt.msm_graphs.clear();
    }
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    CUBBS_CHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    launch_msm_prep(s, md, pts, djobs, vsc);
    launch_msm_main(s, md, pts, djobs, rt.sm_count, nullptr, dout);
    CUBBS_CHECK(cudaStreamEndCapture(s, &graph));
    const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    CUBBS_CHECK(e);
    it = rt.msm_graphs.emplace(key, exec).first;
  }
  CUBBS_CHECK(cudaGraphLaunch(it->second, s));
}

// Runs the plan; returns per-row compressed outputs and per-row ok flags.
// With pairs (or force_engine) the MSMs take the persistent engine, and the
// pairing checks run as units of the same launch.
void run_plan(Runtime &rt, Plan &pl, std::vector<uint8_t> &out48, std::vector<uint8_t> &row_ok,
              PairRequest *pairs = nullptr) {
  cudaStream_t s = rt.stream;
  size_t R = pl.rows, npts = pl.points_be.size() / 48, nvar = pl.var_point.size();
  size_t nfix = pl.has_fixed ? R * pl.fixed_stride : 0;
  // Many variable-only rows: the persistent bucket-method engine (k_msm.cu)
  // instead of one GLV multiplication per term plus a row sum.
  const bool engine = (pairs && pairs->n && !pl.has_fixed) || (!pl.has_fixed && R >= 32 && nvar >= 8 * R);
  MsmPlan mp;
  if (engine) {
    std::vector<uint32_t> K(R);
    for (size_t r = 0; r < R; r++) K[r] = pl.var_start[r + 1] - pl.var_start[r];
    mp.build(K, rt.sh.msm_tuning, pairs ? pairs->n : 0);
  }
  const size_t eng_bytes = engine ? MsmDevice::arena_bytes(mp, rt.sm_count) : 0;
  const size_t np = pairs ? pairs->n : 0;
  rt.arena.reserve(8192 + npts * (sizeof(g1a) + 64) + nvar * (sizeof(g1) + sizeof(fr) + 48) +
                   nfix * (sizeof(fr) + 40) + R * (2 * sizeof(g1) + 128) + eng_bytes + 65536 + np * 512);
  rt.staging.reserve(65536 + pl.points_be.size() + pl.var_scalars_be.size() + pl.fixed_scalars_be.size() +
                     R * 128 + nvar * 16 + eng_bytes + 65536 + np * 256);
  const PairJob *pjobs = nullptr;
  uint8_t *pok = nullptr;
  if (np) {
    pjobs = prepare_pair_jobs(rt, pairs->items, np, pairs->bad);
    pok = rt.arena.alloc<uint8_t>(np);
  }
  if (pl.has_fixed) rt.ensure_table((int)pl.fixed_stride);
  // decode points
  uint8_t *dpb = upload(rt, pl.points_be.data(), pl.points_be.size());
  g1a *pts = rt.arena.alloc<g1a>(npts);
  int32_t *pst = rt.arena.alloc<int32_t>(npts);
  launch_g1_decode(s, dpb, 48, (uint32_t)npts, pts, pst, true);
  // var scalars
  uint8_t *dvs = upload(rt, pl.var_scalars_be.data(), pl.var_scalars_be.size());
  fr *vsc = rt.arena.alloc<fr>(nvar);
  int32_t *vst = rt.arena.alloc<int32_t>(nvar);
  if (nvar) k_parse_scalars<<<blocks_for(nvar, 128), 128, 0, s>>>(dvs, (uint32_t)nvar, vsc, vst);
  // host needs point statuses to build job flags: fetch them
  std::vector<int32_t> hpst(npts);
  if (npts) CUBBS_CHECK(cudaMemcpyAsync(hpst.data(), pst, 4 * npts, cudaMemcpyDeviceToHost, s));
  std::vector<int32_t> hvst(nvar);
  if (nvar) CUBBS_CHECK(cudaMemcpyAsync(hvst.data(), vst, 4 * nvar, cudaMemcpyDeviceToHost, s));
  // fixed scalars
  g1 *fixed = nullptr;
  std::vector<int32_t> hfst;
  if (pl.has_fixed) {
    uint8_t *dfs = upload(rt, pl.fixed_scalars_be.data(), pl.fixed_scalars_be.size());
    fr *fsc = rt.arena.alloc<fr>(nfix);
    int32_t *fst = rt.arena.alloc<int32_t>(nfix);
    k_parse_scalars<<<blocks_for(nfix, 128), 128, 0, s>>>(dfs, (uint32_t)nfix, fsc, fst);
    hfst.resize(nfix);
    CUBBS_CHECK(cudaMemcpyAsync(hfst.data(), fst, 4 * nfix, cudaMemcpyDeviceToHost, s));
    uint32_t *dnt = upload(rt, pl.fixed_nterms.data(), R);
    if (!pl.fixed_scale_be.empty()) {
      uint8_t *dsc = upload(rt, pl.fixed_scale_be.data(), pl.fixed_scale_be.size());
      fr *scale = rt.arena.alloc<fr>(R);
      int32_t *sst = rt.arena.alloc<int32_t>(R);
      k_parse_scalars<<<blocks_for(R, 128), 128, 0, s>>>(dsc, (uint32_t)R, scale, sst);
      k_scale_rows<<<blocks_for(nfix, 128), 128, 0, s>>>(fsc, pl.fixed_stride, dnt, scale, (uint32_t)R);
      std::vector<int32_t> hs(R);
      CUBBS_CHECK(cudaMemcpyAsync(hs.data(), sst, 4 * R, cudaMemcpyDeviceToHost, s));
      CUBBS_CHECK(cudaStreamSynchronize(s));
      for (size_t r = 0; r < R; r++)
        if (hs[r]) hfst[r * pl.fixed_stride] |= 1;
    }
    fixed = rt.arena.alloc<g1>(R);
    launch_fixed_msm(s, rt.table(), fsc, pl.fixed_stride, dnt, (uint32_t)R, fixed);
  }
  CUBBS_CHECK(cudaStreamSynchronize(s));
  std::vector<VarJob> jobs(nvar);
  for (size_t j = 0; j < nvar; j++) {
    uint32_t p = pl.var_point[j];
    jobs[j] = {p, (uint32_t)(hpst[p] != DEC_OK ? 1 : 0)};
  }
  VarJob *djobs = upload(rt, jobs.data(), nvar);
  uint8_t *dout = rt.arena.alloc<uint8_t>(48 * R);
  uint32_t *engine_err = nullptr, herr = 0;
  if (engine) {
    MsmDevice md;
    md.upload(rt, mp, s);
    if (np) {
      md.pjobs = pjobs;
      md.lines = rt.d_lines;
      md.pok = pok;
    }
    run_engine_graph(rt, s, mp, md, pts, djobs, vsc, dout);
    engine_err = md.counter + 1;
  } else {
    g1 *v = rt.arena.alloc<g1>(nvar);
    launch_var_mul(s, pts, djobs, vsc, (uint32_t)nvar, v);
    uint32_t *dstart = upload(rt, pl.var_start.data(), R + 1);
    g1 *res = rt.arena.alloc<g1>(R);
    if (R) k_row_sum<<<blocks_for(R * 32, 128), 128, 0, s>>>(fixed, v, dstart, (uint32_t)R, res);
    launch_g1_compress(s, res, (uint32_t)R, dout);
  }
  CUBBS_CHECK(cudaGetLastError());
  out48.resize(48 * R);
  if (R) CUBBS_CHECK(cudaMemcpyAsync(out48.data(), dout, 48 * R, cudaMemcpyDeviceToHost, s));
  if (np) {
    pairs->ok.resize(np);
    CUBBS_CHECK(cudaMemcpyAsync(pairs->ok.data(), pok, np, cudaMemcpyDeviceToHost, s));
  }
  if (engine_err) CUBBS_CHECK(cudaMemcpyAsync(&herr, engine_err, 4, cudaMemcpyDeviceToHost, s));
  CUBBS_CHECK(cudaStreamSynchronize(s));
  if (herr) throw CudaError(cudaErrorInvalidValue, "uneven-MSM engine: a unit had no room in its launch");
  row_ok.assign(R, 1);
  for (size_t r = 0; r < R; r++) {
    for (uint32_t j = pl.var_start[r]; j < pl.var_start[r + 1]; j++)
      if (hpst[pl.var_point[j]] == DEC_BAD || hvst[j]) row_ok[r] = 0;
    if (pl.has_fixed)
      for (uint32_t g = 0; g < pl.fixed_nterms[r]; g++)
        if (hfst[r * pl.fixed_stride + g]) row_ok[r] = 0;
  }
}

// Is points[0..K) == [P1, Q1, H1, ...][0..K)?
bool is_generator_prefix(Runtime &rt, const CuBbsBbsGpuByteSlice *points, size_t K) {
  if (K == 0 || K > 16386) return false;
  const std::vector<uint8_t> &g = host_gens_c(rt, (int)K);
  for (size_t k = 0; k < K; k++)
    if (points[k].len != 48 || std::memcmp(points[k].data, &g[48 * k], 48) != 0) return false;
  return true;
}

int32_t finish_rows(const std::vector<uint8_t> &out, const std::vector<uint8_t> &ok, CuBbsBbsGpuByteBuffer *outs,
                    CuBbsBbsGpuResult *results, size_t R, uint8_t route) {
  for (size_t r = 0; r < R; r++) {
    if (!ok[r]) {
      results[r] = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
      continue;
    }
    std::memcpy(outs[r].data, &out[48 * r], 48);
    outs[r].len = 48;
    results[r] = {CUBBS_BBS_GPU_SUCCESS, route, 48};
  }
  return CUBBS_BBS_GPU_SUCCESS;
}

// Common-points matrix (shared by the common / fused / plus-variable entries).
int32_t common_points_group(Runtime &rt, const CuBbsBbsGpuByteSlice *points, size_t K,
                            const CuBbsBbsGpuByteSlice *scalar_rows, const uint8_t *rows_be, size_t stride,
                            size_t R, const CuBbsBbsGpuByteSlice *var_points, const CuBbsBbsGpuByteSlice *var_scalars,
                            CuBbsBbsGpuByteBuffer *outs, CuBbsBbsGpuResult *results) {
  Plan pl;
  pl.rows = R;
  bool fixed = is_generator_prefix(rt, points, K);
  bool scaled = rows_be && stride == (K + 1) * 32;
  auto scalar_at = [&](size_t r, size_t k) -> const uint8_t * {
    if (rows_be) return rows_be + r * stride + (scaled ? 32 : 0) + 32 * k;
    return scalar_rows[r * K + k].data;
  };
  std::vector<uint32_t> common_idx;
  if (!fixed)
    for (size_t k = 0; k < K; k++) common_idx.push_back(pl.add_point(points[k].data));
  if (fixed) {
    pl.has_fixed = true;
    pl.fixed_stride = (uint32_t)K;
    pl.fixed_nterms.assign(R, (uint32_t)K);
    pl.fixed_scalars_be.resize(R * K * 32);
    for (size_t r = 0; r < R; r++)
      for (size_t k = 0; k < K; k++) std::memcpy(&pl.fixed_scalars_be[(r * K + k) * 32], scalar_at(r, k), 32);
    if (scaled) {
      pl.fixed_scale_be.resize(R * 32);
      for (size_t r = 0; r < R; r++) std::memcpy(&pl.fixed_scale_be[32 * r], rows_be + r * stride, 32);
    }
  }
  std::vector<uint8_t> scaled_tmp;
  for (size_t r = 0; r < R; r++) {
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    if (!fixed) {
      for (size_t k = 0; k < K; k++) pl.add_var(common_idx[k], scalar_at(r, k));
    }
    if (var_points) pl.add_var(pl.add_point(var_points[r].data), var_scalars[r].data);
  }
  pl.var_start.push_back((uint32_t)pl.var_point.size());
  if (!fixed && scaled) return -1;  // handled by the caller
  std::vector<uint8_t> out, ok;
  run_plan(rt, pl, out, ok);
  return finish_rows(out, ok, outs, results, R, fixed ? CUBBS_BBS_MSM_ROUTE_CUBBS_COMMON_POINTS
                                                      : CUBBS_BBS_MSM_ROUTE_CUBBS_UNIVERSAL);
}

}  // namespace
}  // namespace cubbs

using namespace cubbs;

#define ABI_GUARD_BEGIN try {
#define ABI_GUARD_END                      \
  }                                        \
  catch (const CudaError &) {              \
    return CUBBS_BBS_GPU_ERR_INTERNAL;     \
  }

// ----------------------------------------------------------------------------- g1_msm_batch (route 4)
extern "C" int32_t cubbs_bbs_gpu_g1_msm_batch_v2(uint32_t abi, CuBbsBbsGpuG1MsmItem *items, size_t n,
                                                 CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if ((it.term_count > 0 && (!it.points || !it.scalars)) || !it.point_out.data || it.point_out.capacity < 48)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < it.term_count; k++)
      if (it.points[k].len != 48 || !it.points[k].data || it.scalars[k].len != 32 || !it.scalars[k].data)
        return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  Plan pl;
  pl.rows = n;
  for (size_t i = 0; i < n; i++) {
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    for (size_t k = 0; k < items[i].term_count; k++)
      pl.add_var(pl.add_point(items[i].points[k].data), items[i].scalars[k].data);
  }
  pl.var_start.push_back((uint32_t)pl.var_point.size());
  std::vector<uint8_t> out, ok;
  run_plan(rt, pl, out, ok);
  std::vector<CuBbsBbsGpuByteBuffer> outs(n);
  for (size_t i = 0; i < n; i++) outs[i] = items[i].point_out;
  finish_rows(out, ok, outs.data(), results, n, CUBBS_BBS_MSM_ROUTE_CUBBS_UNIVERSAL);
  for (size_t i = 0; i < n; i++) items[i].point_out.len = outs[i].len;
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// ----------------------------------------------------------------------------- MSMs and pairings in one launch
// An uneven batch of G1 MSMs (the items of g1_msm_batch_v2) and of pairing
// equality checks (the items of pairing_eq_batch_v2) evaluated by one
// persistent engine launch: its warps take MSM units and pairing units from
// one queue, pairing units first.  Results as the two separate entry points
// give them.
extern "C" int32_t cubbs_bbs_gpu_g1_msm_pairing_batch_v2(uint32_t abi, CuBbsBbsGpuG1MsmItem *msm_items,
                                                         size_t msm_count,
                                                         const CuBbsBbsGpuPairingEqItem *pairing_items,
                                                         size_t pairing_count, CuBbsBbsGpuResult *msm_results,
                                                         CuBbsBbsGpuResult *pairing_results) {
  if (!abi_ok(abi) || (msm_count > 0 && (msm_items == nullptr || msm_results == nullptr)) ||
      (pairing_count > 0 && (pairing_items == nullptr || pairing_results == nullptr)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < msm_count; i++) {
    const auto &it = msm_items[i];
    if ((it.term_count > 0 && (!it.points || !it.scalars)) || !it.point_out.data || it.point_out.capacity < 48)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < it.term_count; k++)
      if (it.points[k].len != 48 || !it.points[k].data || it.scalars[k].len != 32 || !it.scalars[k].data)
        return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  if (!pairing_items_ok(pairing_items, pairing_count)) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (msm_count == 0 && pairing_count == 0) return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  Plan pl;
  pl.rows = msm_count;
  for (size_t i = 0; i < msm_count; i++) {
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    for (size_t k = 0; k < msm_items[i].term_count; k++)
      pl.add_var(pl.add_point(msm_items[i].points[k].data), msm_items[i].scalars[k].data);
  }
  pl.var_start.push_back((uint32_t)pl.var_point.size());
  PairRequest pr;
  pr.items = pairing_items;
  pr.n = pairing_count;
  std::vector<uint8_t> out, ok;
  run_plan(rt, pl, out, ok, &pr);
  std::vector<CuBbsBbsGpuByteBuffer> outs(msm_count);
  for (size_t i = 0; i < msm_count; i++) outs[i] = msm_items[i].point_out;
  finish_rows(out, ok, outs.data(), msm_results, msm_count, CUBBS_BBS_MSM_ROUTE_CUBBS_UNIVERSAL);
  for (size_t i = 0; i < msm_count; i++) msm_items[i].point_out.len = outs[i].len;
  for (size_t i = 0; i < pairing_count; i++)
    pairing_results[i] = pr.bad[i] ? CuBbsBbsGpuResult{CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0}
                                   : CuBbsBbsGpuResult{CUBBS_BBS_GPU_SUCCESS, pr.ok[i], 0};
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// ----------------------------------------------------------------------------- common points (route 2 / 4)
static int32_t common_points_entry(uint32_t abi, CuBbsBbsGpuG1MsmCommonPointsBatchItem *items, size_t groups,
                                   CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (groups > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t g = 0; g < groups; g++) {
    const auto &it = items[g];
    bool packed = it.scalar_rows_be != nullptr;
    if ((it.term_count > 0 && !it.points) ||
        (it.output_count > 0 && ((!packed && !it.scalar_rows) || !it.point_outs)) ||
        (packed && it.scalar_row_stride < it.term_count * 32))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < it.term_count; k++)
      if (it.points[k].len != 48 || !it.points[k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t r = 0; r < it.output_count; r++) {
      if (!it.point_outs[r].data || it.point_outs[r].capacity < 48) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
      if (!packed)
        for (size_t k = 0; k < it.term_count; k++)
          if (it.scalar_rows[r * it.term_count + k].len != 32 || !it.scalar_rows[r * it.term_count + k].data)
            return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    }
  }
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  size_t cursor = 0;
  for (size_t g = 0; g < groups; g++) {
    auto &it = items[g];
    size_t K = it.term_count, R = it.output_count;
    if (R == 0) continue;
    const uint8_t *rows_be = it.scalar_rows_be;
    size_t stride = it.scalar_row_stride;
    std::vector<uint8_t> unscaled;
    if (rows_be && stride == (K + 1) * 32 && !is_generator_prefix(rt, it.points, K)) {
      // row-scale prefix with arbitrary points: fold the scale into each term as a
      // separate variable-base term product (points * (s_k * scale)) via two passes
      // is not needed; instead expand to K variable terms per row with scaled
      // scalars computed on the device by the fixed path's scaler.
      Plan pl;
      pl.rows = R;
      std::vector<uint32_t> idx;
      for (size_t k = 0; k < K; k++) idx.push_back(pl.add_point(it.points[k].data));
      pl.has_fixed = false;
      for (size_t r = 0; r < R; r++) {
        pl.var_start.push_back((uint32_t)pl.var_point.size());
        for (size_t k = 0; k < K; k++) pl.add_var(idx[k], rows_be + r * stride + 32 + 32 * k);
      }
      pl.var_start.push_back((uint32_t)pl.var_point.size());
      // scale the var scalars on the device: reuse the fixed-path scaler by
      // treating the var scalar list as R rows of K
      // (done below by running the plan on pre-scaled scalars)
      rt.arena.reserve(65536 + R * K * 80);
      rt.staging.reserve(65536 + R * K * 40 + R * 40);
      uint8_t *dvs = upload(rt, pl.var_scalars_be.data(), pl.var_scalars_be.size());
      fr *vs = rt.arena.alloc<fr>(R * K);
      int32_t *vst = rt.arena.alloc<int32_t>(R * K);
      k_parse_scalars<<<blocks_for(R * K, 128), 128, 0, rt.stream>>>(dvs, (uint32_t)(R * K), vs, vst);
      std::vector<uint8_t> sc(R * 32);
      for (size_t r = 0; r < R; r++) std::memcpy(&sc[32 * r], rows_be + r * stride, 32);
      uint8_t *dsc = upload(rt, sc.data(), sc.size());
      fr *scale = rt.arena.alloc<fr>(R);
      int32_t *sst = rt.arena.alloc<int32_t>(R);
      k_parse_scalars<<<blocks_for(R, 128), 128, 0, rt.stream>>>(dsc, (uint32_t)R, scale, sst);
      std::vector<uint32_t> nt(R, (uint32_t)K);
      uint32_t *dnt = upload(rt, nt.data(), R);
      k_scale_rows<<<blocks_for(R * K, 128), 128, 0, rt.stream>>>(vs, (uint32_t)K, dnt, scale, (uint32_t)R);
      std::vector<uint32_t> raw(8 * R * K);
      CUBBS_CHECK(cudaMemcpyAsync(raw.data(), vs, 32 * R * K, cudaMemcpyDeviceToHost, rt.stream));
      CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
      for (size_t j = 0; j < R * K; j++)
        for (int w = 0; w < 8; w++)
          for (int b = 0; b < 4; b++) pl.var_scalars_be[32 * j + (7 - w) * 4 + (3 - b)] = (uint8_t)(raw[8 * j + w] >> (8 * b));
      rt.arena.reset();
      rt.staging.reset();
      std::vector<uint8_t> out, ok;
      run_plan(rt, pl, out, ok);
      finish_rows(out, ok, it.point_outs, results + cursor, R, CUBBS_BBS_MSM_ROUTE_CUBBS_UNIVERSAL);
    } else {
      common_points_group(rt, it.points, K, it.scalar_rows, rows_be, stride, R, nullptr, nullptr, it.point_outs,
                          results + cursor);
    }
    rt.arena.reset();
    rt.staging.reset();
    cursor += R;
  }
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

extern "C" int32_t cubbs_bbs_gpu_g1_msm_common_points_batch_v2(uint32_t abi,
                                                               CuBbsBbsGpuG1MsmCommonPointsBatchItem *items,
                                                               size_t groups, CuBbsBbsGpuResult *results) {
  return common_points_entry(abi, items, groups, results);
}
extern "C" int32_t cubbs_bbs_gpu_g1_msm_fused_common_points_batch_v2(uint32_t abi,
                                                                     CuBbsBbsGpuG1MsmCommonPointsBatchItem *items,
                                                                     size_t groups, CuBbsBbsGpuResult *results) {
  return common_points_entry(abi, items, groups, results);
}

extern "C" int32_t cubbs_bbs_gpu_g1_msm_common_points_plus_variable_batch_v2(
    uint32_t abi, CuBbsBbsGpuG1MsmCommonPointsPlusVariableItem *items, size_t groups, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (groups > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t g = 0; g < groups; g++) {
    const auto &it = items[g];
    if ((it.term_count > 0 && (!it.points || !it.scalar_rows)) ||
        (it.output_count > 0 && (!it.variable_points || !it.variable_scalars || !it.point_outs)))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t r = 0; r < it.output_count; r++) {
      if (!it.point_outs[r].data || it.point_outs[r].capacity < 48 || it.variable_points[r].len != 48 ||
          !it.variable_points[r].data || it.variable_scalars[r].len != 32 || !it.variable_scalars[r].data)
        return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
      for (size_t k = 0; k < it.term_count; k++)
        if (it.scalar_rows[r * it.term_count + k].len != 32 || !it.scalar_rows[r * it.term_count + k].data)
          return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    }
    for (size_t k = 0; k < it.term_count; k++)
      if (it.points[k].len != 48 || !it.points[k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  size_t cursor = 0;
  for (size_t g = 0; g < groups; g++) {
    auto &it = items[g];
    if (it.output_count == 0) continue;
    common_points_group(rt, it.points, it.term_count, it.scalar_rows, nullptr, 0, it.output_count,
                        it.variable_points, it.variable_scalars, it.point_outs, results + cursor);
    rt.arena.reset();
    rt.staging.reset();
    cursor += it.output_count;
  }
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// T1 = c Bbar + e^ Abar + r1^ D ;  T2 = MSM(common) + r3^ D
extern "C" int32_t cubbs_bbs_gpu_proof_verify_msm_pair_batch_v2(uint32_t abi, CuBbsBbsGpuProofVerifyMsmPairItem *items,
                                                                size_t groups, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (groups > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t g = 0; g < groups; g++) {
    const auto &it = items[g];
    size_t K = it.common_term_count, R = it.output_count;
    if ((K && (!it.common_points || !it.common_scalar_rows)) ||
        (R && (!it.proof_points || !it.proof_scalars || !it.t1_outs || !it.t2_outs)))
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < K; k++)
      if (it.common_points[k].len != 48 || !it.common_points[k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t r = 0; r < R; r++) {
      if (!it.t1_outs[r].data || it.t1_outs[r].capacity < 48 || !it.t2_outs[r].data || it.t2_outs[r].capacity < 48)
        return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
      for (size_t k = 0; k < 3; k++)
        if (it.proof_points[3 * r + k].len != 48 || !it.proof_points[3 * r + k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
      for (size_t k = 0; k < 4; k++)
        if (it.proof_scalars[4 * r + k].len != 32 || !it.proof_scalars[4 * r + k].data)
          return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
      for (size_t k = 0; k < K; k++)
        if (it.common_scalar_rows[r * K + k].len != 32 || !it.common_scalar_rows[r * K + k].data)
          return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    }
  }
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  size_t cursor = 0;
  for (size_t g = 0; g < groups; g++) {
    auto &it = items[g];
    size_t K = it.common_term_count, R = it.output_count;
    if (R == 0) continue;
    // T1 rows: 3 variable terms each
    Plan p1;
    p1.rows = R;
    for (size_t r = 0; r < R; r++) {
      p1.var_start.push_back((uint32_t)p1.var_point.size());
      for (int k = 0; k < 3; k++) p1.add_var(p1.add_point(it.proof_points[3 * r + k].data), it.proof_scalars[4 * r + k].data);
    }
    p1.var_start.push_back((uint32_t)p1.var_point.size());
    std::vector<uint8_t> o1, ok1;
    run_plan(rt, p1, o1, ok1);
    rt.arena.reset();
    rt.staging.reset();
    // T2 rows: common MSM + r3^ D
    std::vector<CuBbsBbsGpuByteSlice> vp(R), vs(R);
    for (size_t r = 0; r < R; r++) {
      vp[r] = it.proof_points[3 * r + 2];
      vs[r] = it.proof_scalars[4 * r + 3];
    }
    std::vector<CuBbsBbsGpuResult> r2(R);
    common_points_group(rt, it.common_points, K, it.common_scalar_rows, nullptr, 0, R, vp.data(), vs.data(),
                        it.t2_outs, r2.data());
    rt.arena.reset();
    rt.staging.reset();
    for (size_t r = 0; r < R; r++) {
      if (!ok1[r] || r2[r].code != CUBBS_BBS_GPU_SUCCESS) {
        results[cursor + r] = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
        continue;
      }
      std::memcpy(it.t1_outs[r].data, &o1[48 * r], 48);
      it.t1_outs[r].len = 48;
      it.t2_outs[r].len = 48;
      results[cursor + r] = {CUBBS_BBS_GPU_SUCCESS, r2[r].value, 96};
    }
    cursor += R;
  }
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// ----------------------------------------------------------------------------- dual MSMs over the same points
extern "C" int32_t cubbs_bbs_gpu_g1_dual_msm_same_points_lanes_batch_v2(uint32_t abi,
                                                                        CuBbsBbsGpuG1DualMsmSamePointsLanesItem *items,
                                                                        size_t n, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    size_t ob = it.lane_count * 48;
    if (it.term_count == 0 || it.lane_count == 0 || it.lane_count > it.term_count || !it.points || !it.lhs_scalars ||
        !it.rhs_scalars || !it.lhs_outs.data || it.lhs_outs.capacity < ob || !it.rhs_outs.data ||
        it.rhs_outs.capacity < ob)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < it.term_count; k++)
      if (it.points[k].len != 48 || !it.points[k].data || it.lhs_scalars[k].len != 32 || !it.lhs_scalars[k].data ||
          it.rhs_scalars[k].len != 32 || !it.rhs_scalars[k].data)
        return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  for (size_t i = 0; i < n; i++) {
    auto &it = items[i];
    // rows: lane j of lhs = row j, lane j of rhs = row lanes + j; lane j sums terms k = j (mod lanes)
    Plan pl;
    size_t lanes = it.lane_count;
    pl.rows = 2 * lanes;
    std::vector<uint32_t> idx;
    for (size_t k = 0; k < it.term_count; k++) idx.push_back(pl.add_point(it.points[k].data));
    for (int side = 0; side < 2; side++)
      for (size_t j = 0; j < lanes; j++) {
        pl.var_start.push_back((uint32_t)pl.var_point.size());
        for (size_t k = j; k < it.term_count; k += lanes)
          pl.add_var(idx[k], side == 0 ? it.lhs_scalars[k].data : it.rhs_scalars[k].data);
      }
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    std::vector<uint8_t> out, ok;
    run_plan(rt, pl, out, ok);
    rt.arena.reset();
    rt.staging.reset();
    bool all = true;
    for (auto o : ok) all = all && o;
    if (!all) {
      results[i] = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
      continue;
    }
    std::memcpy(it.lhs_outs.data, out.data(), 48 * lanes);
    std::memcpy(it.rhs_outs.data, out.data() + 48 * lanes, 48 * lanes);
    it.lhs_outs.len = 48 * lanes;
    it.rhs_outs.len = 48 * lanes;
    results[i] = {CUBBS_BBS_GPU_SUCCESS, CUBBS_BBS_MSM_ROUTE_BLST_COMMON_POINTS, 96 * lanes};
  }
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

extern "C" int32_t cubbs_bbs_gpu_g1_dual_msm_same_points_batch_v2(uint32_t abi, CuBbsBbsGpuG1DualMsmSamePointsItem *items,
                                                                  size_t n, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++) {
    auto &it = items[i];
    if (it.term_count == 0 || !it.points || !it.lhs_scalars || !it.rhs_scalars || !it.lhs_out.data ||
        it.lhs_out.capacity < 48 || !it.rhs_out.data || it.rhs_out.capacity < 48)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    CuBbsBbsGpuG1DualMsmSamePointsLanesItem l = {it.points, it.lhs_scalars, it.rhs_scalars, it.term_count, 1,
                                                 it.lhs_out, it.rhs_out};
    int32_t st = cubbs_bbs_gpu_g1_dual_msm_same_points_lanes_batch_v2(abi, &l, 1, &results[i]);
    if (st != CUBBS_BBS_GPU_SUCCESS) return st;
    it.lhs_out.len = l.lhs_outs.len;
    it.rhs_out.len = l.rhs_outs.len;
  }
  return CUBBS_BBS_GPU_SUCCESS;
}

// ----------------------------------------------------------------------------- G1 add
extern "C" int32_t cubbs_bbs_gpu_g1_add_batch_v2(uint32_t abi, CuBbsBbsGpuG1AddItem *items, size_t n,
                                                 CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if (it.lhs.len != 48 || !it.lhs.data || it.rhs.len != 48 || !it.rhs.data || !it.point_out.data ||
        it.point_out.capacity < 48)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  // lhs + rhs as a 2-term MSM with unit scalars
  Plan pl;
  pl.rows = n;
  uint8_t one[32] = {0};
  one[31] = 1;
  for (size_t i = 0; i < n; i++) {
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    pl.add_var(pl.add_point(items[i].lhs.data), one);
    pl.add_var(pl.add_point(items[i].rhs.data), one);
  }
  pl.var_start.push_back((uint32_t)pl.var_point.size());
  std::vector<uint8_t> out, ok;
  run_plan(rt, pl, out, ok);
  std::vector<CuBbsBbsGpuByteBuffer> outs(n);
  for (size_t i = 0; i < n; i++) outs[i] = items[i].point_out;
  finish_rows(out, ok, outs.data(), results, n, 0);
  for (size_t i = 0; i < n; i++) items[i].point_out.len = outs[i].len;
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// ----------------------------------------------------------------------------- prepare B
// B = P1 + Q1 domain + sum H_i m_i with domain from (PK, 64-byte header, L).
extern "C" int32_t cubbs_bbs_gpu_prepare_b_batch_v2(uint32_t abi, CuBbsBbsGpuPrepareBItem *items, size_t n,
                                                    CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if (it.public_key.len != 96 || !it.public_key.data || it.header.len != 64 || !it.header.data ||
        (it.message_count && !it.message_scalars) || !it.b_out.data || it.b_out.capacity < 48 ||
        it.message_count > 16384)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    for (size_t k = 0; k < it.message_count; k++)
      if (it.message_scalars[k].len != 32 || !it.message_scalars[k].data) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  size_t maxL = 0;
  for (size_t i = 0; i < n; i++) maxL = std::max(maxL, items[i].message_count);
  rt.ensure_table((int)maxL + 2);
  rt.arena.reserve(65536 + n * 256);
  rt.staging.reserve(65536 + n * 256);
  // domains on the device
  std::vector<uint8_t> blob(160 * n);
  std::vector<DomainJob> dj(n);
  for (size_t i = 0; i < n; i++) {
    std::memcpy(&blob[160 * i], items[i].public_key.data, 96);
    std::memcpy(&blob[160 * i + 96], items[i].header.data, 64);
    dj[i] = {(uint32_t)(160 * i), (uint32_t)(160 * i + 96), 64, (uint32_t)items[i].message_count};
  }
  uint8_t *dblob = upload(rt, blob.data(), blob.size());
  DomainJob *ddj = upload(rt, dj.data(), n);
  fr *domain = rt.arena.alloc<fr>(n);
  launch_domain(rt.stream, ddj, (uint32_t)n, dblob, rt.d_gens_c(), nullptr, domain);
  std::vector<uint32_t> raw(8 * n);
  CUBBS_CHECK(cudaMemcpyAsync(raw.data(), domain, 32 * n, cudaMemcpyDeviceToHost, rt.stream));
  CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
  rt.arena.reset();
  rt.staging.reset();
  Plan pl;
  pl.rows = n;
  pl.has_fixed = true;
  pl.fixed_stride = (uint32_t)(maxL + 2);
  pl.fixed_nterms.resize(n);
  pl.fixed_scalars_be.assign(n * pl.fixed_stride * 32, 0);
  for (size_t i = 0; i < n; i++) {
    uint8_t *row = &pl.fixed_scalars_be[i * pl.fixed_stride * 32];
    pl.fixed_nterms[i] = (uint32_t)items[i].message_count + 2;
    row[31] = 1;
    for (int w = 0; w < 8; w++)
      for (int b = 0; b < 4; b++) row[32 + (7 - w) * 4 + (3 - b)] = (uint8_t)(raw[8 * i + w] >> (8 * b));
    for (size_t k = 0; k < items[i].message_count; k++) std::memcpy(row + 64 + 32 * k, items[i].message_scalars[k].data, 32);
    pl.var_start.push_back(0);
  }
  pl.var_start.push_back(0);
  std::vector<uint8_t> out, ok;
  run_plan(rt, pl, out, ok);
  std::vector<CuBbsBbsGpuByteBuffer> outs(n);
  for (size_t i = 0; i < n; i++) outs[i] = items[i].b_out;
  finish_rows(out, ok, outs.data(), results, n, CUBBS_BBS_MSM_ROUTE_CUBBS_COMMON_POINTS);
  for (size_t i = 0; i < n; i++) items[i].b_out.len = outs[i].len;
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// ----------------------------------------------------------------------------- ProofGen T2-prepare
extern "C" int32_t cubbs_bbs_gpu_proof_gen_t2_prepare_batch_v2(uint32_t abi, CuBbsBbsGpuProofGenT2PrepareItem *items,
                                                               size_t n, CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    bool ok = it.compressed_b.len == 48 && it.compressed_b.data && it.signature_a.len == 48 && it.signature_a.data &&
              it.d_out.data && it.d_out.capacity >= 48 && it.abar_out.data && it.abar_out.capacity >= 48 &&
              it.bbar_out.data && it.bbar_out.capacity >= 48 && it.t1_out.data && it.t1_out.capacity >= 48;
    for (int s = 0; s < 7 && ok; s++) ok = it.scalars_be[s].len == 32 && it.scalars_be[s].data;
    if (!ok) {
      results[i] = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
    }
  }
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  // rows per item: d = B s0 ; abar = A s1 ; bbar = B s2 - A s3 ; t1 = A s4 + B s5
  Plan pl;
  pl.rows = 4 * n;
  std::vector<uint8_t> neg(32 * n);
  // -s3 mod r is formed on the device: bbar = B s2 + (-A) s3, with -A by negating the encoding's sign bit
  std::vector<uint8_t> negA(48 * n);
  for (size_t i = 0; i < n; i++) {
    std::memcpy(&negA[48 * i], items[i].signature_a.data, 48);
    uint8_t f = negA[48 * i];
    if ((f & 0x40) == 0) negA[48 * i] = f ^ 0x20;  // flip y sign (identity unchanged)
  }
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    uint32_t B = pl.add_point(it.compressed_b.data), A = pl.add_point(it.signature_a.data);
    uint32_t nA = pl.add_point(&negA[48 * i]);
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    pl.add_var(B, it.scalars_be[0].data);
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    pl.add_var(A, it.scalars_be[1].data);
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    pl.add_var(B, it.scalars_be[2].data);
    pl.add_var(nA, it.scalars_be[3].data);
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    pl.add_var(A, it.scalars_be[4].data);
    pl.add_var(B, it.scalars_be[5].data);
  }
  pl.var_start.push_back((uint32_t)pl.var_point.size());
  std::vector<uint8_t> out, ok;
  run_plan(rt, pl, out, ok);
  for (size_t i = 0; i < n; i++) {
    bool good = ok[4 * i] && ok[4 * i + 1] && ok[4 * i + 2] && ok[4 * i + 3];
    if (!good) {
      results[i] = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
      continue;
    }
    CuBbsBbsGpuByteBuffer *dst[4] = {&items[i].d_out, &items[i].abar_out, &items[i].bbar_out, &items[i].t1_out};
    for (int k = 0; k < 4; k++) {
      std::memcpy(dst[k]->data, &out[48 * (4 * i + k)], 48);
      dst[k]->len = 48;
    }
    results[i] = {CUBBS_BBS_GPU_SUCCESS, 0, 192};
  }
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// ----------------------------------------------------------------------------- pairing equality
// value = e(lhs_g1, lhs_g2) == e(rhs_g1, rhs_g2), via e(lhs, lhs2) * e(-rhs, rhs2) == 1

extern "C" int32_t cubbs_bbs_gpu_pairing_eq_batch_v2(uint32_t abi, const CuBbsBbsGpuPairingEqItem *items, size_t n,
                                                     CuBbsBbsGpuResult *results) {
  if (!abi_ok(abi) || (n > 0 && (items == nullptr || results == nullptr))) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (!pairing_items_ok(items, n)) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (n == 0) return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  rt.arena.reserve(65536 + n * 512);
  rt.staging.reserve(65536 + n * 256);
  std::vector<int> bad;
  PairJob *dj = prepare_pair_jobs(rt, items, n, bad);
  uint8_t *ok = rt.arena.alloc<uint8_t>(n);
  launch_pairing_check(rt.stream, dj, (uint32_t)n, rt.d_lines, ok);
  CUBBS_CHECK(cudaGetLastError());
  std::vector<uint8_t> hok(n);
  CUBBS_CHECK(cudaMemcpyAsync(hok.data(), ok, n, cudaMemcpyDeviceToHost, rt.stream));
  CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
  for (size_t i = 0; i < n; i++)
    results[i] = bad[i] ? CuBbsBbsGpuResult{CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0}
                        : CuBbsBbsGpuResult{CUBBS_BBS_GPU_SUCCESS, hok[i], 0};
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// One result for the batch: prod_i (e(lhs_i, lhs2_i) / e(rhs_i, rhs2_i))^{coef_i} == 1.
// The coefficient scales the G1 sides; pairs that share a G2 point are merged
// by summing their scaled G1 points, then one multi-Miller loop and one final
// exponentiation run on the device.
extern "C" int32_t cubbs_bbs_gpu_pairing_eq_aggregate_v2(uint32_t abi, const CuBbsBbsGpuPairingEqScaledItem *items,
                                                         size_t n, CuBbsBbsGpuResult *result) {
  if (!abi_ok(abi) || result == nullptr || (n > 0 && items == nullptr)) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  for (size_t i = 0; i < n; i++) {
    const auto &it = items[i];
    if (it.lhs_g1.len != 48 || !it.lhs_g1.data || it.rhs_g1.len != 48 || !it.rhs_g1.data || it.lhs_g2.len != 96 ||
        !it.lhs_g2.data || it.rhs_g2.len != 96 || !it.rhs_g2.data || it.coefficient.len != 32 || !it.coefficient.data)
      return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  }
  if (n == 0) {
    *result = {CUBBS_BBS_GPU_SUCCESS, 1, 0};
    return CUBBS_BBS_GPU_SUCCESS;
  }
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  // group G1 terms by G2 point: for lhs pair, (coef, lhs_g1); for rhs pair, (coef, -rhs_g1)
  std::vector<std::string> keys;
  std::unordered_map<std::string, size_t> key_idx;
  std::vector<std::vector<std::pair<const uint8_t *, std::pair<const uint8_t *, bool>>>> groups;
  auto add = [&](const uint8_t *g2, const uint8_t *g1p, const uint8_t *coef, bool neg) {
    std::string k(reinterpret_cast<const char *>(g2), 96);
    auto f = key_idx.find(k);
    size_t gi;
    if (f == key_idx.end()) {
      gi = keys.size();
      key_idx[k] = gi;
      keys.push_back(k);
      groups.emplace_back();
    } else {
      gi = f->second;
    }
    groups[gi].push_back({g1p, {coef, neg}});
  };
  for (size_t i = 0; i < n; i++) {
    add(items[i].lhs_g2.data, items[i].lhs_g1.data, items[i].coefficient.data, false);
    add(items[i].rhs_g2.data, items[i].rhs_g1.data, items[i].coefficient.data, true);
  }
  std::vector<const uint8_t *> g2p;
  for (auto &k : keys) g2p.push_back(reinterpret_cast<const uint8_t *>(k.data()));
  std::vector<int> slots, st;
  rt.resolve_pks(g2p, slots, st);
  for (size_t g = 0; g < keys.size(); g++)
    if (st[g] == DEC_BAD) {
      *result = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
      return CUBBS_BBS_GPU_SUCCESS;
    }
  Plan pl;
  pl.rows = keys.size();
  std::vector<uint8_t> negbuf;
  negbuf.reserve(48 * 2 * n);
  for (size_t g = 0; g < keys.size(); g++) {
    pl.var_start.push_back((uint32_t)pl.var_point.size());
    for (auto &t : groups[g]) {
      uint8_t b[48];
      std::memcpy(b, t.first, 48);
      if (t.second.second && (b[0] & 0x40) == 0) b[0] ^= 0x20;  // -P by flipping the y sign flag
      pl.add_var(pl.add_point(b), t.second.first);
    }
  }
  pl.var_start.push_back((uint32_t)pl.var_point.size());
  std::vector<uint8_t> out, ok;
  run_plan(rt, pl, out, ok);
  for (auto o : ok)
    if (!o) {
      *result = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
      return CUBBS_BBS_GPU_SUCCESS;
    }
  rt.arena.reset();
  rt.staging.reset();
  size_t K = keys.size();
  rt.arena.reserve(65536 + K * 256);
  rt.staging.reserve(65536 + K * 256);
  uint8_t *d = upload(rt, out.data(), out.size());
  g1a *pts = rt.arena.alloc<g1a>(K);
  int32_t *pst = rt.arena.alloc<int32_t>(K);
  launch_g1_decode(rt.stream, d, 48, (uint32_t)K, pts, pst, false);
  std::vector<int32_t> hst(K);
  CUBBS_CHECK(cudaMemcpyAsync(hst.data(), pst, 4 * K, cudaMemcpyDeviceToHost, rt.stream));
  CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
  std::vector<uint8_t> skip(K);
  std::vector<int32_t> sl(K);
  for (size_t g = 0; g < K; g++) {
    skip[g] = (hst[g] != DEC_OK || st[g] == DEC_INF) ? 1 : 0;
    sl[g] = slots[g];
  }
  uint8_t *dskip = upload(rt, skip.data(), K);
  int32_t *dsl = upload(rt, sl.data(), K);
  uint8_t *dok = rt.arena.alloc<uint8_t>(1);
  k_multi_pairing<<<1, 32, 0, rt.stream>>>(pts, dsl, dskip, (uint32_t)K, rt.d_lines, dok);
  CUBBS_CHECK(cudaGetLastError());
  uint8_t hok = 0;
  CUBBS_CHECK(cudaMemcpyAsync(&hok, dok, 1, cudaMemcpyDeviceToHost, rt.stream));
  CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
  *result = {CUBBS_BBS_GPU_SUCCESS, hok, 0};
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// ----------------------------------------------------------------------------- fixed-base MSM autotuner
// Batched fixed-base MSMs over the first `terms` resident generators
// [P1, Q1, H1, ...]: rows x terms canonical big-endian scalars.  For every
// window width w in [w_lo, w_hi] the table is rebuilt with width w and the
// MSM kernel is timed with CUDA events over `steps` launches (256 MiB L2
// flush before each); ms_per_w[w - w_lo] gets the mean.  Each width's output
// rows (the first 64, compressed) are compared with the same rows computed
// without any table (GLV variable-base terms over the affine generators plus
// a row sum); a width that disagrees gets ms_per_w = -1, counts in
// *mismatched and is never chosen.  The fastest agreeing width stays as the
// process's table width (*best_w; 0 and ERR_INTERNAL if none agreed).  The
// reference sweeps its comb width by term count (prepare_b_msm.cu:315-329).
extern "C" int32_t cubbs_bbs_gpu_fixed_msm_autotune_v2(uint32_t abi, const uint8_t *scalars_be, size_t rows,
                                                       size_t terms, int32_t w_lo, int32_t w_hi, int32_t steps,
                                                       float *ms_per_w, int32_t *best_w, int32_t *mismatched) {
  if (!abi_ok(abi) || !scalars_be || rows == 0 || terms == 0 || terms > 1024 || w_lo < 4 || w_hi > MAX_TABLE_WINDOW ||
      w_lo > w_hi || steps <= 0 || !ms_per_w || !best_w || !mismatched)
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  ABI_GUARD_BEGIN
  CallScope scope;
  Runtime &rt = scope.rt;
  cudaStream_t s = rt.stream;
  const size_t n = rows * terms;
  rt.arena.reserve(n * (32 + sizeof(fr) + 4) + rows * (sizeof(g1) + 4) + 65536);
  rt.staging.reserve(n * 32 + rows * 4 + 65536);
  uint8_t *dbe = upload(rt, scalars_be, n * 32);
  fr *sc = rt.arena.alloc<fr>(n);
  int32_t *st = rt.arena.alloc<int32_t>(n);
  k_parse_scalars<<<blocks_for(n, 128), 128, 0, s>>>(dbe, (uint32_t)n, sc, st);
  std::vector<uint32_t> nt(rows, (uint32_t)terms);
  uint32_t *dnt = upload(rt, nt.data(), rows);
  g1 *out = rt.arena.alloc<g1>(rows);
  // check rows: the first min(rows, 64), recomputed without the table
  const size_t RC = std::min<size_t>(rows, 64);
  std::vector<VarJob> cj(RC * terms);
  std::vector<uint32_t> cstart(RC + 1);
  for (size_t r = 0; r <= RC; r++) cstart[r] = (uint32_t)(r * terms);
  for (size_t j = 0; j < RC * terms; j++) cj[j] = {(uint32_t)(j % terms), 0u};
  VarJob *dcj = upload(rt, cj.data(), cj.size());
  uint32_t *dcs = upload(rt, cstart.data(), RC + 1);
  g1 *cv = rt.arena.alloc<g1>(RC * terms);
  g1 *cref = rt.arena.alloc<g1>(RC);
  uint8_t *dref48 = rt.arena.alloc<uint8_t>(48 * RC), *dout48 = rt.arena.alloc<uint8_t>(48 * RC);
  std::vector<uint8_t> href(48 * RC), hout(48 * RC);
  static std::once_flag flush_once;
  static uint8_t *flush = nullptr;
  static cudaError_t flush_err = cudaSuccess;
  const size_t FLUSH = (size_t)256 << 20;
  std::call_once(flush_once, [&] { flush_err = cudaMalloc(&flush, FLUSH); });
  CUBBS_CHECK(flush_err);
  cudaEvent_t e0, e1;
  CUBBS_CHECK(cudaEventCreate(&e0));
  CUBBS_CHECK(cudaEventCreate(&e1));
  float best = 0;
  int bw = 0;
  *mismatched = 0;
  for (int w = w_lo; w <= w_hi; w++) {
    rt.set_table_window(w, (int)terms);
    if (w == w_lo) {
      // the generators now cover `terms` (the table build grew them) and stay put
      launch_var_mul(s, rt.d_gens(), dcj, sc, (uint32_t)(RC * terms), cv);
      k_row_sum<<<blocks_for(RC * 32, 128), 128, 0, s>>>(nullptr, cv, dcs, (uint32_t)RC, cref);
      launch_g1_compress(s, cref, (uint32_t)RC, dref48);
      CUBBS_CHECK(cudaMemcpyAsync(href.data(), dref48, href.size(), cudaMemcpyDeviceToHost, s));
    }
    launch_fixed_msm(s, rt.table(), sc, (uint32_t)terms, dnt, (uint32_t)rows, out);  // warm-up and check
    launch_g1_compress(s, out, (uint32_t)RC, dout48);
    CUBBS_CHECK(cudaMemcpyAsync(hout.data(), dout48, hout.size(), cudaMemcpyDeviceToHost, s));
    CUBBS_CHECK(cudaStreamSynchronize(s));
    const bool agree = std::memcmp(href.data(), hout.data(), href.size()) == 0;
    float total = 0;
    for (int k = 0; k < steps; k++) {
      CUBBS_CHECK(cudaMemsetAsync(flush, k & 0xff, FLUSH, s));
      CUBBS_CHECK(cudaEventRecord(e0, s));
      launch_fixed_msm(s, rt.table(), sc, (uint32_t)terms, dnt, (uint32_t)rows, out);
      CUBBS_CHECK(cudaEventRecord(e1, s));
      CUBBS_CHECK(cudaEventSynchronize(e1));
      float ms = 0;
      CUBBS_CHECK(cudaEventElapsedTime(&ms, e0, e1));
      total += ms;
    }
    ms_per_w[w - w_lo] = agree ? total / steps : -1.0f;
    if (!agree) {
      ++*mismatched;
      continue;
    }
    if (bw == 0 || ms_per_w[w - w_lo] < best) {
      best = ms_per_w[w - w_lo];
      bw = w;
    }
  }
  CUBBS_CHECK(cudaGetLastError());
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *best_w = bw;
  if (bw == 0) {
    rt.set_table_window(0, (int)terms);  // back to the automatic width
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
  rt.set_table_window(bw, (int)terms);
  return CUBBS_BBS_GPU_SUCCESS;
  ABI_GUARD_END
}

// SM counts of the ProofVerify partition (small: the aggregated pairing
// check; rest: every other kernel of the call); both 0 when it is off, and
// *status tells why (0: on; 1: turned off; 2: off under an injected profiler;
// 200 + k: driver entry point k missing; else 1000 * failed step + driver or
// runtime result).  The partition is made on first use: by this query or by
// the first ProofVerify batch with a key group.
extern "C" int32_t cubbs_bbs_gpu_sm_partition_v2(int32_t *small_sms, int32_t *rest_sms, int32_t *status) {
  if (!small_sms || !rest_sms || !status) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    const bool on = scope.rt.use_partition();
    *small_sms = on ? scope.rt.sh.small_sms : 0;
    *rest_sms = on ? scope.rt.sh.rest_sms : 0;
    *status = on ? 0 : (scope.rt.sh.partition_status ? scope.rt.sh.partition_status : 99);
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// SMs of the third ProofVerify partition (the point decode and the
// variable-base terms), split off the rest; 0 when it is off
// (CUBBS_BBS_VAR_SMS=0, the driver refused the split, or no partition), and
// *status tells why (0: on; 1: not asked for; -1: no partition; else the step
// that failed * 1000 + driver result).
extern "C" int32_t cubbs_bbs_gpu_sm_partition_var_v2(int32_t *var_sms, int32_t *status) {
  if (!var_sms || !status) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    const bool on = scope.rt.use_partition();
    *var_sms = on ? scope.rt.sh.var_sms : 0;
    *status = scope.rt.sh.var_status;
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}

// Window width of the resident fixed-base table (0 before the first table is built).
extern "C" int32_t cubbs_bbs_gpu_table_window_v2(int32_t *w) {
  if (!w) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  try {
    CallScope scope;
    *w = scope.rt.table().entries ? scope.rt.table().w : 0;
    return CUBBS_BBS_GPU_SUCCESS;
  } catch (const CudaError &) {
    return CUBBS_BBS_GPU_ERR_INTERNAL;
  }
}
