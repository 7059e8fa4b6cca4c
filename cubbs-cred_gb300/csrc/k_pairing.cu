// Pairing kernels: G2 public-key preparation (decompress, subgroup check,
// 68 Miller lines kept resident per key), the lines of +-P2, and the 2-pair
// pairing check  e(P_a, Q_a) * e(P_b, Q_b) == 1  with a shared Miller loop
// and one final exponentiation per check, run by a 16-lane team per check.
//
// Reference: G2 line precompute by BLST on the host (g1_msm_blst.cpp:441-486),
// Miller loop over precomputed lines and final-verify kernels
// (native/cuda/src/kernels/pairing.cuh:376-478, host :579-737).
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

// One pairing check per 16-lane team (4 teams per 64-thread block); see
// pairing_team.cuh.  The B * xP factors of the lines are computed by lanes
// that have no product of their own in the preceding round.
__global__ void __launch_bounds__(64) k_pairing_check_team(const PairJob *jobs, uint32_t n, const line2 *lines,
                                                           uint8_t *ok) {
  __shared__ PtShared smem[64 / PT_LANES];
  const int team = threadIdx.x / PT_LANES;
  PtCtx c;
  c.lane = threadIdx.x % PT_LANES;
  c.mask = 0xFFFFu << (threadIdx.x & 16);
  c.sm = &smem[team];
  const uint32_t item = blockIdx.x * (64 / PT_LANES) + team;
  if (item >= n) return;  // the whole team leaves together
  const PairJob &j = jobs[item];
  if (!j.active) {
    if (c.lane == 0) ok[item] = 0;
    return;
  }
  const bool skip[2] = {(j.flags & 1) != 0, (j.flags & 2) != 0};
  const line2 *L[2] = {lines + (size_t)j.slot_a * MILLER_LINES, lines + (size_t)j.slot_b * MILLER_LINES};
  if (c.lane == 0) {
    c.sm->PX[0] = j.pa.x;
    c.sm->PY[0] = j.pa.y;
    c.sm->PX[1] = j.pb.x;
    c.sm->PY[1] = j.pb.y;
  }
  pt_set_one(c, PT_F);
  int idx = 0;
#pragma unroll 1
  for (int i = 62; i >= 0; i--) {
    const bool bit = zabs_bit(i) != 0;
    pt_sqr(c, PT_F, [&](int s, fp2 &x, fp2 &y) -> fp2 * {  // B * xP of this step's doubling lines
      if (s >= 2 || skip[s]) return nullptr;
      x = L[s][idx].b;
      y.c0 = c.sm->PX[s];
      return &c.sm->BX[s];
    });
#pragma unroll 1
    for (int p = 0; p < 2; p++) {
      if (skip[p]) continue;
      const fp2 A = L[p][idx].a;
      pt_line(c, PT_F, A, &c.sm->BX[p], &c.sm->PY[p], [&](int s, fp2 &x, fp2 &y) -> fp2 * {
        if (!bit || s != 0) return nullptr;  // B * xP of the addition line
        x = L[p][idx + 1].b;
        y.c0 = c.sm->PX[p];
        return &c.sm->BXA[p];
      });
    }
    idx++;
    if (bit) {
#pragma unroll 1
      for (int p = 0; p < 2; p++) {
        if (skip[p]) continue;
        const fp2 A = L[p][idx].a;
        pt_line(c, PT_F, A, &c.sm->BXA[p], &c.sm->PY[p], [](int, fp2 &, fp2 &) -> fp2 * { return nullptr; });
      }
      idx++;
    }
  }
  pt_conj(c, PT_F, PT_F);  // z < 0
  const bool one = pt_final_exp_is_one(c);
  if (c.lane == 0) ok[item] = one ? 1 : 0;
}

void launch_pairing_check(cudaStream_t s, const PairJob *jobs, uint32_t n, const line2 *lines, uint8_t *ok) {
  if (n) k_pairing_check_team<<<blocks_for((size_t)n * PT_LANES, 64), 64, 0, s>>>(jobs, n, lines, ok);
}

}  // namespace cubbs
