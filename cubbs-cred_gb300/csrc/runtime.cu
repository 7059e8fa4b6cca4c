// Runtime singleton: device selection, streams, arena, the resident prepared
// state (generators built on the device by hash_to_curve, fixed-base window
// tables, Miller lines of +-P2 and of every public key seen) and
// backend_info.  Reference: host pools/caches in prepare_b_msm.cu:165-301,
// kernels/common_cache.cuh:112-486 and the canary probe cubbs_bbs_cuda.cu:719-824.
#include <cstdlib>
#include <cstring>

#include "runtime.cuh"

namespace cubbs {

void DeviceArena::reserve(size_t bytes) {
  if (bytes <= cap) return;
  size_t ncap = cap ? cap : ((size_t)64 << 20);
  while (ncap < bytes) ncap *= 2;
  if (base) CUBBS_CHECK(cudaFree(base));
  base = nullptr;
  cap = 0;
  CUBBS_CHECK(cudaMalloc(&base, ncap));
  cap = ncap;
  used = 0;
}

void HostStaging::reserve(size_t bytes) {
  if (bytes <= cap) return;
  size_t ncap = cap ? cap : ((size_t)16 << 20);
  while (ncap < bytes) ncap *= 2;
  if (base) CUBBS_CHECK(cudaFreeHost(base));
  base = nullptr;
  cap = 0;
  CUBBS_CHECK(cudaMallocHost(&base, ncap));
  cap = ncap;
  used = 0;
}

SharedState &SharedState::get() {
  static SharedState s;
  return s;
}

static int env_int(const char *name, int dflt) {
  const char *v = std::getenv(name);
  if (!v || !*v) return dflt;
  return std::atoi(v);
}

void SharedState::init() {
  std::lock_guard<std::mutex> g(init_mu);
  if (initialised) return;
  int ndev = 0;
  CUBBS_CHECK(cudaGetDeviceCount(&ndev));
  if (ndev <= 0) throw CudaError(cudaErrorNoDevice, "no CUDA device");
  device = env_int("CUBBS_BBS_DEVICE", 0);
  CUBBS_CHECK(cudaSetDevice(device));
  CUBBS_CHECK(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));
  CUBBS_CHECK(cudaStreamCreateWithFlags(&prep, cudaStreamNonBlocking));
  // The kernels are register heavy; give them room for local-memory spills.
  CUBBS_CHECK(cudaDeviceSetLimit(cudaLimitStackSize, 16384));
  table_w = env_int("CUBBS_BBS_TABLE_WINDOW", 0);  // 0: chosen by table_window_for
  if (table_w != 0 && (table_w < 4 || table_w > MAX_TABLE_WINDOW)) table_w = 0;
  {
    size_t free_b = 0, total_b = 0;
    CUBBS_CHECK(cudaMemGetInfo(&free_b, &total_b));
    const int gib = env_int("CUBBS_BBS_TABLE_BUDGET_GIB", 0);
    table_budget = gib > 0 ? (size_t)gib << 30 : total_b / 100 * 35;
  }
  workspaces = env_int("CUBBS_BBS_WORKSPACES", 4);
  if (workspaces < 1 || workspaces > 64) workspaces = 4;
  line_capacity = 2 + 1024;
  CUBBS_CHECK(cudaMalloc(&d_lines, (size_t)line_capacity * MILLER_LINES * sizeof(line2)));
  CUBBS_CHECK(cudaMalloc(&d_pk_aff, (size_t)line_capacity * sizeof(g2a)));
  launch_p2_lines(prep, d_lines);
  CUBBS_CHECK(cudaGetLastError());
  CUBBS_CHECK(cudaStreamSynchronize(prep));
  line_used = 2;
  slot_info.assign(2, PkSlot{DEC_OK});
  initialised = true;
}

void SharedState::ensure_partition() {
  std::lock_guard<std::mutex> g(init_mu);
  if (partition_tried) return;
  partition_tried = true;
  init_partition();
}

namespace {
__global__ void k_partition_probe(int *flag) {
  if (threadIdx.x == 0) atomicAdd(flag, 1);
}
template <class F> F driver_fn(const char *name) {
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion(name, &fn, CUDART_VERSION, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess)
    return nullptr;
  return reinterpret_cast<F>(fn);
}
}  // namespace

// Splits the device's SMs into a partition of CUBBS_BBS_SM_PARTITION SMs
// (default 16, where ProofVerify at 1024 proofs ran fastest on GB300: 8 SMs
// slow the scaling kernel, 24 gain nothing; the driver rounds to multiples of
// 8; 0 turns the partition off) and the rest, as two green contexts (CUDA driver API,
// entry points looked up through the runtime).  A self-test launches a kernel
// on each and hands an event from one to the other; if any step fails the
// partition stays off and ProofVerify runs on the plain streams.
// Under a profiler that injects itself the partition stays off unless
// CUBBS_BBS_SM_PARTITION asks for it: such tools may stop listing kernels at
// the first green-context launch.  Nsight Compute marks its target process
// with NV_NSIGHT_INJECTION_TRANSPORT_TYPE, NV_COMPUTE_PROFILER_PERFWORKS_DIR
// and NV_TPS_LAUNCH_TOKEN; other injecting tools set CUDA_INJECTION64_PATH.
static bool profiler_injected() {
  for (const char *name : {"CUDA_INJECTION64_PATH", "NV_NSIGHT_INJECTION_TRANSPORT_TYPE",
                           "NV_COMPUTE_PROFILER_PERFWORKS_DIR", "NV_TPS_LAUNCH_TOKEN"}) {
    const char *v = std::getenv(name);
    if (v && *v) return true;
  }
  return false;
}

// A probe kernel on a stream of each of two green contexts, ordered by an
// event; true when both ran.
static bool partition_probe(CUresult (*stream_create)(CUstream *, CUgreenCtx, unsigned, int), CUgreenCtx x,
                            CUgreenCtx y) {
  CUstream a = nullptr, b = nullptr;
  cudaEvent_t ev = nullptr;
  int *flag = nullptr, got = 0;
  bool ok = stream_create(&a, x, CU_STREAM_NON_BLOCKING, 0) == CUDA_SUCCESS &&
            stream_create(&b, y, CU_STREAM_NON_BLOCKING, 0) == CUDA_SUCCESS &&
            cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess &&
            cudaMalloc(&flag, sizeof(int)) == cudaSuccess && cudaMemsetAsync(flag, 0, sizeof(int), b) == cudaSuccess;
  if (ok) {
    k_partition_probe<<<1, 32, 0, b>>>(flag);
    ok = cudaGetLastError() == cudaSuccess && cudaEventRecord(ev, b) == cudaSuccess &&
         cudaStreamWaitEvent(a, ev, 0) == cudaSuccess;
  }
  if (ok) {
    k_partition_probe<<<1, 32, 0, a>>>(flag);
    ok = cudaGetLastError() == cudaSuccess &&
         cudaMemcpyAsync(&got, flag, sizeof(int), cudaMemcpyDeviceToHost, a) == cudaSuccess &&
         cudaStreamSynchronize(a) == cudaSuccess && got == 2;
  }
  (void)cudaGetLastError();
  if (a) cudaStreamDestroy(a);
  if (b) cudaStreamDestroy(b);
  if (ev) cudaEventDestroy(ev);
  if (flag) cudaFree(flag);
  return ok;
}

void SharedState::init_partition() {
  const char *setting = std::getenv("CUBBS_BBS_SM_PARTITION");
  if (profiler_injected() && !(setting && *setting)) {
    partition_status = 2;
    return;
  }
  const int want = env_int("CUBBS_BBS_SM_PARTITION", 16);
  if (want <= 0 || want >= sm_count) {
    partition_status = 1;
    return;
  }
  using GetDevice = CUresult (*)(CUdevice *, int);
  using GetRes = CUresult (*)(CUdevice, CUdevResource *, CUdevResourceType);
  using Split = CUresult (*)(CUdevResource *, unsigned *, const CUdevResource *, CUdevResource *, unsigned, unsigned);
  using GenDesc = CUresult (*)(CUdevResourceDesc *, CUdevResource *, unsigned);
  using Create = CUresult (*)(CUgreenCtx *, CUdevResourceDesc, CUdevice, unsigned);
  using Destroy = CUresult (*)(CUgreenCtx);
  using StreamCreate = CUresult (*)(CUstream *, CUgreenCtx, unsigned, int);
  auto get_device = driver_fn<GetDevice>("cuDeviceGet");
  auto get_res = driver_fn<GetRes>("cuDeviceGetDevResource");
  auto split = driver_fn<Split>("cuDevSmResourceSplitByCount");
  auto gen_desc = driver_fn<GenDesc>("cuDevResourceGenerateDesc");
  auto create = driver_fn<Create>("cuGreenCtxCreate");
  auto destroy = driver_fn<Destroy>("cuGreenCtxDestroy");
  auto stream_create = driver_fn<StreamCreate>("cuGreenCtxStreamCreate");
  const void *fns[] = {(void *)get_device, (void *)get_res, (void *)split, (void *)gen_desc,
                       (void *)create, (void *)destroy, (void *)stream_create};
  for (int k = 0; k < 7; k++)
    if (!fns[k]) {
      partition_status = 200 + k;  // entry point k of the list above is missing
      return;
    }
  // partition_status: 1000 * step + CUresult of the step that failed
  auto fail = [this](int step, CUresult r) {
    partition_status = 1000 * step + (int)r;
    return false;
  };
  CUdevice dev;
  CUdevResource all{}, small{}, rest{};
  unsigned groups = 1;
  CUresult r;
  if ((r = get_device(&dev, device)) != CUDA_SUCCESS) return (void)fail(3, r);
  if ((r = get_res(dev, &all, CU_DEV_RESOURCE_TYPE_SM)) != CUDA_SUCCESS) return (void)fail(4, r);
  if ((r = split(&small, &groups, &all, &rest, 0, (unsigned)want)) != CUDA_SUCCESS) return (void)fail(5, r);
  if (groups != 1 || small.sm.smCount == 0 || rest.sm.smCount == 0) return (void)fail(6, CUDA_SUCCESS);
  CUdevResourceDesc dsmall, drest;
  if ((r = gen_desc(&dsmall, &small, 1)) != CUDA_SUCCESS) return (void)fail(7, r);
  if ((r = gen_desc(&drest, &rest, 1)) != CUDA_SUCCESS) return (void)fail(8, r);
  CUgreenCtx gs = nullptr, gr = nullptr;
  if ((r = create(&gs, dsmall, dev, CU_GREEN_CTX_DEFAULT_STREAM)) != CUDA_SUCCESS) return (void)fail(9, r);
  if ((r = create(&gr, drest, dev, CU_GREEN_CTX_DEFAULT_STREAM)) != CUDA_SUCCESS) {
    destroy(gs);
    return (void)fail(10, r);
  }
  // Optionally a third partition: CUBBS_BBS_VAR_SMS SMs (default 32; 0:
  // none) taken from the larger one for the point decode and the
  // variable-base terms of ProofVerify, whose lane pairs then stop sharing
  // issue slots with the fixed-base MSM and the subgroup check.  Measured on
  // GB300 (1024 proofs, L = 100): 32 SMs 3.87 ms per step, 48 / 56 SMs 3.9 ms,
  // 64 SMs 4.2 ms (the terms at one warp per SM sub-partition take 1.9 ms
  // instead of 2.8, but the subgroup check on the 72 SMs left takes 3.2 ms),
  // no third partition 4.2 ms.  The device's SMs are split into groups of 8
  // in one call and the groups are joined into the three partitions (the
  // chain's partition then holds the first groups, as many SMs as the two-way
  // split gave it, and replaces that split's own small partition so that the
  // three come from one split and do not overlap).  var_status records why it
  // is off; any failure here leaves the two-way split as it is.
  CUgreenCtx gv = nullptr, gr2 = nullptr, gs3 = nullptr;
  int var_count = 0, small3 = 0;
  const int var_want = env_int("CUBBS_BBS_VAR_SMS", 32);
  var_status = 1;
  if (var_want > 0 && var_want + 16 <= (int)rest.sm.smCount) {
    constexpr unsigned GMAX = 64;
    CUdevResource grp[GMAX], left{};
    unsigned ng = GMAX;
    var_status = 2;
    r = split(grp, &ng, &all, &left, 0, 8u);
    if (r != CUDA_SUCCESS) var_status = 3000 + (int)r;
    if (r == CUDA_SUCCESS) {
      // groups [0, k0): the chain's SMs; [k0, k1): the variable-base terms; the rest
      unsigned k0 = 0, k1 = 0;
      while (k0 < ng && small3 < (int)small.sm.smCount) small3 += (int)grp[k0++].sm.smCount;
      k1 = k0;
      while (k1 < ng && var_count < var_want) var_count += (int)grp[k1++].sm.smCount;
      CUdevResource rest_parts[GMAX + 1];
      unsigned nr = 0;
      for (unsigned k = k1; k < ng; k++) rest_parts[nr++] = grp[k];
      if (left.sm.smCount) rest_parts[nr++] = left;
      CUdevResourceDesc dvar, drest2, dsmall3;
      if (k0 == 0 || k1 == k0 || nr == 0) {
        var_status = 4;
      } else if ((r = gen_desc(&dsmall3, grp, k0)) != CUDA_SUCCESS) {
        var_status = 4000 + (int)r;
      } else if ((r = gen_desc(&dvar, grp + k0, k1 - k0)) != CUDA_SUCCESS) {
        var_status = 5000 + (int)r;
      } else if ((r = gen_desc(&drest2, rest_parts, nr)) != CUDA_SUCCESS) {
        var_status = 6000 + (int)r;
      } else if ((r = create(&gv, dvar, dev, CU_GREEN_CTX_DEFAULT_STREAM)) != CUDA_SUCCESS) {
        var_status = 7000 + (int)r;
        gv = nullptr;
      } else if ((r = create(&gr2, drest2, dev, CU_GREEN_CTX_DEFAULT_STREAM)) != CUDA_SUCCESS) {
        var_status = 8000 + (int)r;
        destroy(gv);
        gv = gr2 = nullptr;
      } else if ((r = create(&gs3, dsmall3, dev, CU_GREEN_CTX_DEFAULT_STREAM)) != CUDA_SUCCESS) {
        var_status = 10000 + (int)r;
        destroy(gv);
        destroy(gr2);
        gv = gr2 = gs3 = nullptr;
      }
    }
  }
  // self-test: a kernel on each partition, ordered by an event
  CUstream a = nullptr, b = nullptr;
  cudaEvent_t ev = nullptr;
  int *flag = nullptr;
  int step = 11;
  bool ok = stream_create(&a, gs, CU_STREAM_NON_BLOCKING, 0) == CUDA_SUCCESS &&
            stream_create(&b, gr, CU_STREAM_NON_BLOCKING, 0) == CUDA_SUCCESS;
  if (ok) {
    step = 12;
    ok = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess &&
         cudaMalloc(&flag, sizeof(int)) == cudaSuccess && cudaMemsetAsync(flag, 0, sizeof(int), b) == cudaSuccess;
  }
  int got = 0;
  if (ok) {
    step = 13;
    k_partition_probe<<<1, 32, 0, b>>>(flag);
    ok = cudaGetLastError() == cudaSuccess && cudaEventRecord(ev, b) == cudaSuccess &&
         cudaStreamWaitEvent(a, ev, 0) == cudaSuccess;
  }
  if (ok) {
    step = 14;
    k_partition_probe<<<1, 32, 0, a>>>(flag);
    ok = cudaGetLastError() == cudaSuccess &&
         cudaMemcpyAsync(&got, flag, sizeof(int), cudaMemcpyDeviceToHost, a) == cudaSuccess &&
         cudaStreamSynchronize(a) == cudaSuccess && got == 2;
  }
  const cudaError_t last = cudaGetLastError();  // a failed probe leaves no sticky error behind
  if (a) cudaStreamDestroy(a);
  if (b) cudaStreamDestroy(b);
  if (ev) cudaEventDestroy(ev);
  if (flag) cudaFree(flag);
  if (!ok) {
    destroy(gs);
    destroy(gr);
    if (gv) destroy(gv);
    if (gr2) destroy(gr2);
    if (gs3) destroy(gs3);
    partition_status = 1000 * step + (int)last;
    return;
  }
  green_small = gs;
  green_rest = gr;
  small_sms = (int)small.sm.smCount;
  rest_sms = (int)rest.sm.smCount;
  if (gv && partition_probe(stream_create, gv, gr2) && partition_probe(stream_create, gs3, gv)) {
    destroy(gs);
    green_small = gs3;
    small_sms = small3;
    green_var = gv;
    green_rest2 = gr2;
    var_sms = var_count;
    var_status = 0;
  } else if (gv) {
    var_status = 9;
    destroy(gv);
    destroy(gr2);
    destroy(gs3);
  }
  green_stream_create = stream_create;
  partition_status = 0;
}

// Build generators of `suite` up to d_gens[count) on the device: P1 is decoded
// from its published encoding; Q1, H1, ... come from the seed chain +
// hash_to_curve with the suite's expander.
void SharedState::grow_generators(int suite, int count) {
  SuiteState &g = suites[suite];
  if (count <= g.gen_count) return;
  int ncap = g.gen_capacity ? g.gen_capacity : 256;
  while (ncap < count) ncap *= 2;
  if (ncap != g.gen_capacity) {
    g1a *ng = nullptr;
    uint8_t *nc = nullptr;
    CUBBS_CHECK(cudaMalloc(&ng, (size_t)ncap * sizeof(g1a)));
    CUBBS_CHECK(cudaMalloc(&nc, (size_t)ncap * 48 + 48));
    if (g.gen_count) {
      CUBBS_CHECK(cudaDeviceSynchronize());  // no call may still read the old arrays
      CUBBS_CHECK(cudaMemcpy(ng, g.d_gens, (size_t)g.gen_count * sizeof(g1a), cudaMemcpyDeviceToDevice));
      CUBBS_CHECK(cudaMemcpy(nc, g.d_gens_c, (size_t)g.gen_count * 48 + 48, cudaMemcpyDeviceToDevice));
      cudaFree(g.d_gens);
      cudaFree(g.d_gens_c);
    }
    g.d_gens = ng;
    g.d_gens_c = nc;
    g.gen_capacity = ncap;
  }
  if (!g.d_seed_state) CUBBS_CHECK(cudaMalloc(&g.d_seed_state, 64));
  if (g.gen_count == 0) {
    launch_decode_p1(prep, g.d_gens, g.d_gens_c, suite);
    g.gen_count = 1;
  }
  int first = g.gen_count;  // 1-based generator number == d_gens index
  int n = count - g.gen_count;
  uint8_t *seeds = nullptr;
  CUBBS_CHECK(cudaMalloc(&seeds, (size_t)n * 48));
  launch_make_generator_seeds(prep, first, n, g.d_seed_state, seeds, suite);
  launch_hash_generators(prep, first, n, seeds, g.d_gens, g.d_gens_c, suite);
  CUBBS_CHECK(cudaGetLastError());
  CUBBS_CHECK(cudaStreamSynchronize(prep));
  cudaFree(seeds);
  g.gen_count = count;
  g.h_gens_c.resize((size_t)g.gen_count * 48);
  CUBBS_CHECK(cudaMemcpy(g.h_gens_c.data(), g.d_gens_c, g.h_gens_c.size(), cudaMemcpyDeviceToHost));
}

// Fixed-base window table over d_gens[0..gens) of a suite.  Rebuilt (all
// generators) when it must grow; built in generator chunks to bound the scratch.
// Window width of a suite's table over `gens` generators.  The tables of all
// suites share the table budget (CUBBS_BBS_TABLE_BUDGET_GIB, default 35 % of
// the device memory: 91 GiB on GB300).  Automatic: the width in
// 8..MAX_TABLE_WINDOW with the fewest windows (ceil(256 / w), the mixed
// additions per term) whose table fits what the other suites leave, the
// narrowest of equals (w = 20 up to 128 generators on GB300: 13 additions per
// term instead of 16 at w = 16).  An explicit width (CUBBS_BBS_TABLE_WINDOW,
// the fixed-base autotuner) is narrowed until the table fits.  The entries are
// read at random, one 96-byte point per addition, from HBM.
int SharedState::table_window_for(int suite, int gens) const {
  size_t others = 0;
  for (int s = 0; s < SUITE_COUNT; s++)
    if (s != suite && suites[s].table.entries) others += table_bytes(suites[s].table.gens, suites[s].table.w);
  const size_t budget = table_budget > others ? table_budget - others : 0;
  if (table_w) {
    for (int w = table_w; w > 4; w--)
      if (table_bytes(gens, w) <= budget) return w;
    return 4;
  }
  int best = 8;
  for (int w = 8; w <= MAX_TABLE_WINDOW; w++)
    if (table_bytes(gens, w) <= budget && 255 / w < 255 / best) best = w;
  return best;
}

bool SharedState::table_covers(int suite, int gens) const {
  const FixedTable &t = suites[suite].table;
  return t.entries && t.gens >= gens && t.req_w == table_w;
}

void SharedState::grow_table(int suite, int gens) {
  if (table_covers(suite, gens)) return;
  SuiteState &g = suites[suite];
  int want = 1;
  while (want < gens) want *= 2;
  if (want < 64) want = 64;
  grow_generators(suite, want);
  // the caller holds the prepared state exclusively (no call is in flight), so
  // the old table goes first and the two never occupy the device together
  if (g.table.entries) {
    CUBBS_CHECK(cudaDeviceSynchronize());
    cudaFree(g.table.entries);
    g.table = FixedTable{};
  }
  FixedTable t;
  t.req_w = table_w;
  t.w = table_window_for(suite, want);
  t.nwin = 255 / t.w + 1;
  t.half = 1 << (t.w - 1);
  t.gens = want;
  size_t per_gen = (size_t)t.nwin * t.half;
  g1a *entries = nullptr;
  CUBBS_CHECK(cudaMalloc(&entries, (size_t)want * per_gen * sizeof(g1a)));
  t.entries = entries;
  // chunk so that the XYZZ + prefix scratch stays below ~8 GiB
  size_t per_gen_scratch = per_gen * (sizeof(g1) + sizeof(fp));
  int chunk = (int)std::max<size_t>(1, ((size_t)8 << 30) / per_gen_scratch);
  if (chunk > want) chunk = want;
  g1 *scratch = nullptr;
  fp *prod = nullptr;
  g1a *bases = nullptr;
  try {
    CUBBS_CHECK(cudaMalloc(&scratch, (size_t)chunk * per_gen * sizeof(g1)));
    CUBBS_CHECK(cudaMalloc(&prod, (size_t)chunk * per_gen * sizeof(fp)));
    CUBBS_CHECK(cudaMalloc(&bases, (size_t)chunk * t.nwin * sizeof(g1a)));
    for (int g0 = 0; g0 < want; g0 += chunk) {
      int g1n = std::min(want, g0 + chunk);
      // the kernels index bases and scratch from generator g0
      launch_build_table(prep, g.d_gens, g0, g1n, t, bases, scratch, prod);
      CUBBS_CHECK(cudaGetLastError());
      CUBBS_CHECK(cudaStreamSynchronize(prep));
    }
  } catch (const CudaError &) {
    cudaFree(scratch);
    cudaFree(prod);
    cudaFree(bases);
    cudaFree(entries);
    throw;
  }
  cudaFree(scratch);
  cudaFree(prod);
  cudaFree(bases);
  g.table = t;
}

// Decode, check and line-precompute public keys not seen before.
void SharedState::add_pks(const std::vector<std::string> &keys) {
  std::vector<std::string> fresh;
  for (const auto &k : keys)
    if (!pk_slots.count(k)) fresh.push_back(k);
  if (fresh.empty()) return;
  if (line_used + (int)fresh.size() > line_capacity) {
    int ncap = line_capacity;
    while (ncap < line_used + (int)fresh.size()) ncap *= 2;
    line2 *nl = nullptr;
    g2a *na = nullptr;
    CUBBS_CHECK(cudaMalloc(&nl, (size_t)ncap * MILLER_LINES * sizeof(line2)));
    CUBBS_CHECK(cudaMalloc(&na, (size_t)ncap * sizeof(g2a)));
    CUBBS_CHECK(cudaDeviceSynchronize());
    CUBBS_CHECK(cudaMemcpy(nl, d_lines, (size_t)line_used * MILLER_LINES * sizeof(line2), cudaMemcpyDeviceToDevice));
    CUBBS_CHECK(cudaMemcpy(na, d_pk_aff, (size_t)line_used * sizeof(g2a), cudaMemcpyDeviceToDevice));
    cudaFree(d_lines);
    cudaFree(d_pk_aff);
    d_lines = nl;
    d_pk_aff = na;
    line_capacity = ncap;
  }
  std::vector<uint8_t> h(96 * fresh.size());
  for (size_t i = 0; i < fresh.size(); i++) std::memcpy(h.data() + 96 * i, fresh[i].data(), 96);
  uint8_t *d = nullptr;
  int32_t *dst = nullptr;
  CUBBS_CHECK(cudaMalloc(&d, h.size()));
  CUBBS_CHECK(cudaMalloc(&dst, 4 * fresh.size()));
  CUBBS_CHECK(cudaMemcpyAsync(d, h.data(), h.size(), cudaMemcpyHostToDevice, prep));
  launch_pk_prepare(prep, d, (uint32_t)fresh.size(), line_used, d_pk_aff, d_lines, dst);
  CUBBS_CHECK(cudaGetLastError());
  std::vector<int32_t> st(fresh.size());
  CUBBS_CHECK(cudaMemcpyAsync(st.data(), dst, 4 * fresh.size(), cudaMemcpyDeviceToHost, prep));
  CUBBS_CHECK(cudaStreamSynchronize(prep));
  cudaFree(d);
  cudaFree(dst);
  for (size_t i = 0; i < fresh.size(); i++) {
    pk_slots[fresh[i]] = line_used + (int)i;
    slot_info.push_back(PkSlot{st[i]});
  }
  line_used += (int)fresh.size();
}

Runtime::Runtime(SharedState &s)
    : sh(s), device(s.device), sm_count(s.sm_count), table_w(s.table_w), d_lines(s.d_lines) {
  CUBBS_CHECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  CUBBS_CHECK(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
  CUBBS_CHECK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
  CUBBS_CHECK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
  {
    // stream3 carries the ProofVerify pairing chain, the step's critical path:
    // its blocks go first when the block scheduler picks between streams
    int lo = 0, hi = 0;
    CUBBS_CHECK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    CUBBS_CHECK(cudaStreamCreateWithPriority(&stream3, cudaStreamNonBlocking, hi));
  }
  CUBBS_CHECK(cudaEventCreateWithFlags(&ev_mid, cudaEventDisableTiming));
  CUBBS_CHECK(cudaEventCreateWithFlags(&ev_side, cudaEventDisableTiming));
  CUBBS_CHECK(cudaStreamCreateWithFlags(&stream4, cudaStreamNonBlocking));
  CUBBS_CHECK(cudaEventCreateWithFlags(&ev_sub, cudaEventDisableTiming));
  CUBBS_CHECK(cudaEventCreateWithFlags(&ev_hash, cudaEventDisableTiming));
  arena.reserve((size_t)256 << 20);
  staging.reserve((size_t)64 << 20);
  pack.reserve((size_t)64 << 20);
}

// The workspace's streams on the SM partition, made the first time a call on
// this workspace can use them (the workspace belongs to one call at a time).
bool Runtime::use_partition() {
  if (part[0]) return true;
  if (part_tried) return false;
  part_tried = true;
  sh.ensure_partition();
  if (!sh.green_rest) return false;
  int lo = 0, hi = 0;
  CUBBS_CHECK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  cudaStream_t p[4] = {nullptr, nullptr, nullptr, nullptr}, pc = nullptr;
  bool ok = true;
  // with the third partition, part[1] (decode, variable-base terms) runs on it
  // and the other three on the remaining SMs
  for (int k = 0; k < 4 && ok; k++) {
    CUgreenCtx where = sh.green_var ? (k == 1 ? sh.green_var : sh.green_rest2) : sh.green_rest;
    ok = sh.green_stream_create(&p[k], where, CU_STREAM_NON_BLOCKING, k == 2 ? hi : 0) == CUDA_SUCCESS;
  }
  ok = ok && sh.green_stream_create(&pc, sh.green_small, CU_STREAM_NON_BLOCKING, hi) == CUDA_SUCCESS;
  if (!ok) {
    for (auto q : p)
      if (q) cudaStreamDestroy(q);
    if (pc) cudaStreamDestroy(pc);
    return false;
  }
  CUBBS_CHECK(cudaEventCreateWithFlags(&ev_gc, cudaEventDisableTiming));
  CUBBS_CHECK(cudaEventCreateWithFlags(&ev_gc2, cudaEventDisableTiming));
  CUBBS_CHECK(cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming));
  for (int k = 0; k < 4; k++) part[k] = p[k];
  part_check = pc;
  return true;
}

// Growth from inside a call: drop the shared hold, grow under the exclusive
// lock (the grow functions re-check), take the shared hold again.
void Runtime::ensure_generators(int count) {
  if (count <= ss().gen_count) return;
  lock->unlock();
  {
    std::unique_lock<std::shared_mutex> ex(sh.mu);
    sh.grow_generators(suite, count);
  }
  lock->lock();
}

void Runtime::ensure_table(int gens) {
  if (sh.table_covers(suite, gens)) return;
  lock->unlock();
  {
    std::unique_lock<std::shared_mutex> ex(sh.mu);
    sh.grow_table(suite, gens);
  }
  lock->lock();
}

void Runtime::set_table_window(int w, int gens) {
  lock->unlock();
  {
    std::unique_lock<std::shared_mutex> ex(sh.mu);
    sh.table_w = w;
    sh.grow_table(suite, std::max(gens, ss().table.gens));
  }
  lock->lock();
}

void Runtime::set_msm_tuning(const MsmTuning &t) {
  lock->unlock();
  {
    std::unique_lock<std::shared_mutex> ex(sh.mu);
    sh.msm_tuning = t;
  }
  lock->lock();
}

void Runtime::resolve_pks(const std::vector<const uint8_t *> &pk_ptrs, std::vector<int> &slots,
                          std::vector<int> &status) {
  std::vector<std::string> keys(pk_ptrs.size());
  bool missing = false;
  for (size_t i = 0; i < pk_ptrs.size(); i++) {
    keys[i].assign(reinterpret_cast<const char *>(pk_ptrs[i]), 96);
    if (!missing && !sh.pk_slots.count(keys[i])) missing = true;
  }
  if (missing) {
    lock->unlock();
    {
      std::unique_lock<std::shared_mutex> ex(sh.mu);
      sh.add_pks(keys);
    }
    lock->lock();
  }
  slots.assign(pk_ptrs.size(), -1);
  status.assign(pk_ptrs.size(), DEC_BAD);
  for (size_t i = 0; i < keys.size(); i++) {
    int s = sh.pk_slots.at(keys[i]);
    slots[i] = s;
    status[i] = sh.slot_info[s].status;
  }
}

// Builds the domain-hash prefixes of (key slot << 32 | L, key bytes) pairs not
// resident yet (the generators already cover each L).  Growing the array
// waits for the device first: no call may still read the old one.
void SharedState::add_domain_prefixes(int suite, const std::vector<std::pair<uint64_t, const uint8_t *>> &fresh) {
  SuiteState &g = suites[suite];
  auto &dom_prefix = g.dom_prefix;
  auto &d_dom_prefix = g.d_dom_prefix;
  auto &dom_prefix_cap = g.dom_prefix_cap;
  std::vector<DomainPrefixJob> jobs;
  for (const auto &f : fresh) {
    if (dom_prefix.count(f.first)) continue;
    const uint32_t index = (uint32_t)dom_prefix.size();
    dom_prefix.emplace(f.first, index);
    DomainPrefixJob j;
    std::memcpy(j.pk, f.second, 96);
    j.L = (uint32_t)(f.first & 0xffffffffu);
    j.index = index;
    jobs.push_back(j);
  }
  if (jobs.empty()) return;
  const uint32_t need = (uint32_t)dom_prefix.size();
  if (need > dom_prefix_cap) {
    uint32_t ncap = dom_prefix_cap ? dom_prefix_cap : 64;
    while (ncap < need) ncap *= 2;
    uint8_t *np = nullptr;
    CUBBS_CHECK(cudaMalloc(&np, (size_t)ncap * DOMAIN_PREFIX_BYTES));
    if (d_dom_prefix) {
      CUBBS_CHECK(cudaDeviceSynchronize());
      CUBBS_CHECK(cudaMemcpy(np, d_dom_prefix, (size_t)dom_prefix_cap * DOMAIN_PREFIX_BYTES,
                             cudaMemcpyDeviceToDevice));
      cudaFree(d_dom_prefix);
    }
    d_dom_prefix = np;
    dom_prefix_cap = ncap;
  }
  DomainPrefixJob *dj = nullptr;
  CUBBS_CHECK(cudaMalloc(&dj, jobs.size() * sizeof(DomainPrefixJob)));
  CUBBS_CHECK(cudaMemcpyAsync(dj, jobs.data(), jobs.size() * sizeof(DomainPrefixJob), cudaMemcpyHostToDevice, prep));
  launch_domain_prefix(prep, dj, (uint32_t)jobs.size(), g.d_gens_c, d_dom_prefix);
  CUBBS_CHECK(cudaGetLastError());
  CUBBS_CHECK(cudaStreamSynchronize(prep));
  cudaFree(dj);
}

// ---------------------------------------------------------------- workspace pool
namespace {
std::mutex g_pool_mu;
std::condition_variable g_pool_cv;
std::vector<std::unique_ptr<Runtime>> g_pool;
std::vector<bool> g_busy;

Runtime &acquire_workspace() {
  SharedState &sh = SharedState::get();
  sh.init();
  CUBBS_CHECK(cudaSetDevice(sh.device));
  std::unique_lock<std::mutex> lk(g_pool_mu);
  for (;;) {
    for (size_t i = 0; i < g_pool.size(); i++)
      if (!g_busy[i]) {
        g_busy[i] = true;
        return *g_pool[i];
      }
    if ((int)g_pool.size() < sh.workspaces) {
      g_pool.emplace_back(new Runtime(sh));
      g_busy.push_back(true);
      return *g_pool.back();
    }
    g_pool_cv.wait(lk);
  }
}

void release_workspace(Runtime &rt) {
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (size_t i = 0; i < g_pool.size(); i++)
      if (g_pool[i].get() == &rt) g_busy[i] = false;
  }
  g_pool_cv.notify_one();
}
}  // namespace

CallScope::CallScope() : rt(acquire_workspace()), lock(rt.sh.mu) {
  rt.lock = &lock;
  rt.suite = SUITE_SHA256;
  rt.arena.reset();
  rt.staging.reset();
  rt.pack.reset();
}

CallScope::~CallScope() {
  rt.lock = nullptr;
  lock.unlock();
  release_workspace(rt);
}

}  // namespace cubbs

using namespace cubbs;

__global__ void k_canary(uint32_t *out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *out = 0x0BB52023u;
}

extern "C" int32_t cubbs_bbs_gpu_backend_info_v2(uint32_t abi, CuBbsBbsGpuBackendInfo *info) {
  if (abi != CUBBS_BBS_GPU_ABI_VERSION || info == nullptr) return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  info->backend_kind = CUBBS_BBS_GPU_BACKEND_KIND_UNKNOWN;
  info->hardware_acceleration = 0;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    uint32_t *d = rt.arena.alloc<uint32_t>(1);
    k_canary<<<1, 1, 0, rt.stream>>>(d);
    CUBBS_CHECK(cudaGetLastError());
    uint32_t h = 0;
    CUBBS_CHECK(cudaMemcpyAsync(&h, d, 4, cudaMemcpyDeviceToHost, rt.stream));
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    if (h == 0x0BB52023u) {
      info->backend_kind = CUBBS_BBS_GPU_BACKEND_KIND_CUDA;
      info->hardware_acceleration = 1;
    }
  } catch (const CudaError &) {
  }
  return CUBBS_BBS_GPU_SUCCESS;
}
