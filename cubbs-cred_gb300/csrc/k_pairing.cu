// Pairing kernels: G2 public-key preparation (decompress, subgroup check,
// 68 Miller lines kept resident per key), the lines of +-P2, and the 2-pair
// pairing check  e(P_a, Q_a) * e(P_b, Q_b) == 1  with a shared Miller loop
// and one final exponentiation per check, run by one warp per check.
//
// Reference: G2 line precompute by BLST on the host (g1_msm_blst.cpp:441-486),
// Miller loop over precomputed lines and final-verify kernels
// (native/cuda/src/kernels/pairing.cuh:376-478, host :579-737).
#include <cstdlib>

#include "pairing_team.cuh"
#include "runtime.cuh"

namespace cubbs {

__global__ void k_p2_lines(line2 *lines) {
  if (blockIdx.x != 0 || threadIdx.x > 1) return;
  g2a g = g2_generator();
  if (threadIdx.x == 0) g.y = fp2_neg(g.y);  // slot 0: -P2
  g2_precompute_lines(g, lines + (size_t)threadIdx.x * MILLER_LINES);
}

__global__ void k_pk_prepare(const uint8_t *pks, uint32_t n, int slot0, g2a *pk_aff, line2 *lines,
                             int32_t *status) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint8_t b[96];
  for (int k = 0; k < 96; k++) b[k] = pks[96 * (size_t)i + k];
  g2a a;
  int st = g2_decompress(b, a);
  status[i] = st;
  if (st != DEC_OK) return;
  pk_aff[slot0 + i] = a;
  g2_precompute_lines(a, lines + (size_t)(slot0 + i) * MILLER_LINES);
}

void launch_p2_lines(cudaStream_t s, line2 *lines) { k_p2_lines<<<1, 32, 0, s>>>(lines); }
void launch_pk_prepare(cudaStream_t s, const uint8_t *pks96, uint32_t n, int slot0, g2a *pk_aff, line2 *lines,
                       int32_t *status) {
  if (n) k_pk_prepare<<<blocks_for(n, 32), 32, 0, s>>>(pks96, n, slot0, pk_aff, lines, status);
}

// One pairing check per warp (one warp per block); see pairing_team.cuh.
// Dynamic shared memory: PP_SLOTS Fp slots.
__global__ void __launch_bounds__(32) k_pairing_check_warp(const PairJob *jobs, uint32_t n, const line2 *lines,
                                                           uint8_t *ok) {
  extern __shared__ __align__(16) uint8_t pp_smem[];
  fp *sl = reinterpret_cast<fp *>(pp_smem);
  const int lane = threadIdx.x;
  const uint32_t item = blockIdx.x;
  if (item >= n) return;
  const PairJob &j = jobs[item];
  if (j.active != 1) {  // 0: not evaluated (result 0); 2: settled before the launch (ok[item] kept)
    if (lane == 0 && j.active == 0) ok[item] = 0;
    return;
  }
  const bool skip[2] = {(j.flags & 1) != 0, (j.flags & 2) != 0};
  const line2 *L[2] = {lines + (size_t)j.slot_a * MILLER_LINES, lines + (size_t)j.slot_b * MILLER_LINES};
  const g1a P[2] = {j.pa, j.pb};
  const bool one = pp::pairing_check(sl, lane, P, L, skip);
  if (lane == 0) ok[item] = one ? 1 : 0;
}

// One pairing check per block of two warps (for the few group checks of an
// aggregated batch, where one check's latency is the step's critical path):
// warp w runs the Miller loop of pair w, then warp 0 multiplies the two values
// and runs the final exponentiation.  Dynamic shared memory: 2 * PP_SLOTS Fp slots.
__global__ void __launch_bounds__(64) k_pairing_check_split(const PairJob *jobs, uint32_t n, const line2 *lines,
                                                            uint8_t *ok) {
  extern __shared__ __align__(16) uint8_t pp_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  fp *sl = reinterpret_cast<fp *>(pp_smem) + warp * PP_SLOTS;
  const uint32_t item = blockIdx.x;
  if (item >= n) return;
  const PairJob &j = jobs[item];
  if (j.active != 1) {  // 0: not evaluated (result 0); 2: settled before the launch (ok[item] kept)
    if (threadIdx.x == 0 && j.active == 0) ok[item] = 0;
    return;
  }
  const bool skip = (j.flags >> warp) & 1;
  const line2 *L = lines + (size_t)(warp ? j.slot_b : j.slot_a) * MILLER_LINES;
  pp::miller_one(sl, lane, warp ? j.pb : j.pa, L, skip);
  __syncthreads();
  if (warp != 0) return;
  if (lane < 12) pp::st(sl, PP_REG(PP_REG_X) + lane, pp::ld(sl + PP_SLOTS, PP_REG(PP_REG_F) + lane));
  __syncwarp();
  pp::run(sl, lane, PP_MUL_F_F_X);
  pp::run(sl, lane, PP_CONJ_F);  // z < 0
  const bool one = pp::final_exp_is_one(sl, lane);
  if (lane == 0) ok[item] = one ? 1 : 0;
}

// The same with a two-warp team per pair (four warps per check): team t runs
// the Miller loop of pair t on named barrier 1 + t, then team 0 multiplies
// the two values and runs the final exponentiation.  Phases of up to 64
// products take one round (pairing_team.cuh).
__global__ void __launch_bounds__(128) k_pairing_check_split_wide(const PairJob *jobs, uint32_t n,
                                                                  const line2 *lines, uint8_t *ok) {
  extern __shared__ __align__(16) uint8_t pp_smem[];
  const int team = threadIdx.x >> 6, lane = threadIdx.x & 63, bar = 1 + team;
  fp *sl = reinterpret_cast<fp *>(pp_smem) + team * PP_SLOTS;
  const uint32_t item = blockIdx.x;
  if (item >= n) return;
  const PairJob &j = jobs[item];
  if (j.active != 1) {  // 0: not evaluated (result 0); 2: settled before the launch (ok[item] kept)
    if (threadIdx.x == 0 && j.active == 0) ok[item] = 0;
    return;
  }
  const bool skip = (j.flags >> team) & 1;
  const line2 *L = lines + (size_t)(team ? j.slot_b : j.slot_a) * MILLER_LINES;
  pp::miller_one<64>(sl, lane, team ? j.pb : j.pa, L, skip, bar);
  __syncthreads();
  if (team != 0) return;
  if (lane < 12) pp::st(sl, PP_REG(PP_REG_X) + lane, pp::ld(sl + PP_SLOTS, PP_REG(PP_REG_F) + lane));
  pp::team_sync<64>(bar);
  pp::run<64>(sl, lane, PP_MUL_F_F_X, bar);
  pp::run<64>(sl, lane, PP_CONJ_F, bar);  // z < 0
  const bool one = pp::final_exp_is_one<64>(sl, lane, bar);
  if (lane == 0) ok[item] = one ? 1 : 0;
}

// Two-warp teams unless CUBBS_BBS_PAIR_TEAM=32 (one warp per pair).
static bool wide_pair_teams() {
  static const bool v = [] {
    const char *e = std::getenv("CUBBS_BBS_PAIR_TEAM");
    return !(e && std::atoi(e) == 32);
  }();
  return v;
}

void launch_pairing_check_split(cudaStream_t s, const PairJob *jobs, uint32_t n, const line2 *lines, uint8_t *ok) {
  const size_t smem = 2 * (size_t)PP_SLOTS * sizeof(fp);
  static const bool attr = [smem] {
    CUBBS_CHECK(cudaFuncSetAttribute(k_pairing_check_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CUBBS_CHECK(
        cudaFuncSetAttribute(k_pairing_check_split_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return true;
  }();
  (void)attr;
  if (!n) return;
  if (wide_pair_teams()) k_pairing_check_split_wide<<<n, 128, smem, s>>>(jobs, n, lines, ok);
  else k_pairing_check_split<<<n, 64, smem, s>>>(jobs, n, lines, ok);
}

// Latency probe: SM cycles of one run of each pairing program on a lone warp
// (slots filled with Montgomery one; the values do not change the path).
__global__ void __launch_bounds__(32) k_pp_probe(double *cycles, int reps) {
  extern __shared__ __align__(16) uint8_t pp_smem[];
  fp *sl = reinterpret_cast<fp *>(pp_smem);
  const int lane = threadIdx.x;
  for (int i = lane; i < PP_SLOTS; i += 32) pp::st(sl, i, fp_one());
  __syncwarp();
  for (int prog = 0; prog < PP_NPROG; prog++) {
    const long long t0 = clock64();
#pragma unroll 1
    for (int r = 0; r < reps; r++) pp::run(sl, lane, prog);
    const long long t1 = clock64();
    if (lane == 0) cycles[prog] = (double)(t1 - t0) / reps;
  }
}

// The same for two-warp teams (one block of 64 threads, the PP_ENTRY_W tables).
__global__ void __launch_bounds__(64) k_pp_probe_wide(double *cycles, int reps) {
  extern __shared__ __align__(16) uint8_t pp_smem[];
  fp *sl = reinterpret_cast<fp *>(pp_smem);
  const int lane = threadIdx.x;
  for (int i = lane; i < PP_SLOTS; i += 64) pp::st(sl, i, fp_one());
  __syncthreads();
  for (int prog = 0; prog < PP_NPROG; prog++) {
    const long long t0 = clock64();
#pragma unroll 1
    for (int r = 0; r < reps; r++) pp::run<64>(sl, lane, prog, 1);
    const long long t1 = clock64();
    if (lane == 0) cycles[prog] = (double)(t1 - t0) / reps;
  }
}

extern "C" int32_t cubbs_bbs_gpu_pairing_probe_wide_for_test_v2(double *cycles, int32_t cap) {
  if (!cycles || cap < PP_NPROG) return -1;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    double *d = rt.arena.alloc<double>(PP_NPROG);
    const size_t smem = (size_t)PP_SLOTS * sizeof(fp);
    k_pp_probe_wide<<<1, 64, smem, rt.stream>>>(d, 2);  // warm-up
    k_pp_probe_wide<<<1, 64, smem, rt.stream>>>(d, 16);
    CUBBS_CHECK(cudaGetLastError());
    CUBBS_CHECK(cudaMemcpyAsync(cycles, d, PP_NPROG * sizeof(double), cudaMemcpyDeviceToHost, rt.stream));
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    return PP_NPROG;
  } catch (const CudaError &) {
    return -2;
  }
}

extern "C" int32_t cubbs_bbs_gpu_pairing_probe_for_test_v2(double *cycles, int32_t cap) {
  if (!cycles || cap < PP_NPROG) return -1;
  try {
    CallScope scope;
    Runtime &rt = scope.rt;
    double *d = rt.arena.alloc<double>(PP_NPROG);
    const size_t smem = (size_t)PP_SLOTS * sizeof(fp);
    k_pp_probe<<<1, 32, smem, rt.stream>>>(d, 2);  // warm-up
    k_pp_probe<<<1, 32, smem, rt.stream>>>(d, 16);
    CUBBS_CHECK(cudaGetLastError());
    CUBBS_CHECK(cudaMemcpyAsync(cycles, d, PP_NPROG * sizeof(double), cudaMemcpyDeviceToHost, rt.stream));
    CUBBS_CHECK(cudaStreamSynchronize(rt.stream));
    return PP_NPROG;
  } catch (const CudaError &) {
    return -2;
  }
}

void launch_pairing_check(cudaStream_t s, const PairJob *jobs, uint32_t n, const line2 *lines, uint8_t *ok) {
  const size_t smem = (size_t)PP_SLOTS * sizeof(fp);
  static const bool attr = [smem] {  // once per process, on the library's device
    CUBBS_CHECK(cudaFuncSetAttribute(k_pairing_check_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return true;
  }();
  (void)attr;
  if (n) k_pairing_check_warp<<<n, 32, smem, s>>>(jobs, n, lines, ok);
}

}  // namespace cubbs
