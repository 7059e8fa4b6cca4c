// G1 kernels: point decoding (decompress + subgroup check), fixed-base window
// tables over the resident generators, the fixed-base MSM (one warp per MSM
// row, signed w-bit windows, affine table entries, mixed XYZZ additions),
// GLV variable-base multiplication and point compression.
//
// Reference counterparts: comb tables and comb MSMs
// (native/cuda/src/kernels/comb_precompute.cuh:8-268, comb_msm.cuh:3-363),
// GLV variable base (kernels/variable_base_universal.cuh:25-331), BLST decode
// and compress on the host (native/cuda/src/g1_msm_blst.cpp:614-732).  Here
// decode and compress run on the device.
#include <cstdlib>

#include "runtime.cuh"

namespace cubbs {

__global__ void __launch_bounds__(128) k_g1_decode(const uint8_t *pts, uint32_t stride, uint32_t n, g1a *out,
                                                   int32_t *status, bool check_subgroup) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint8_t b[48];
  for (int k = 0; k < 48; k++) b[k] = pts[(size_t)i * stride + k];
  g1a a;
  int st = g1_decompress(b, a, check_subgroup);
  if (st != DEC_OK) {
    a.x = fp_zero();
    a.y = fp_zero();
  }
  out[i] = a;
  status[i] = st;
}

// Window bases of a table chunk: bases[(g - g0) * nwin + k] = 2^(w k) G_g in
// affine form, one thread per (generator, window).
__global__ void __launch_bounds__(64) k_table_bases(const g1a *gens, int g0, int g1n, FixedTable t, g1a *bases) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (g1n - g0) * t.nwin) return;
  const int g = g0 + tid / t.nwin, k = tid % t.nwin;
  g1 B = g1_from_aff(gens[g]);
  #pragma unroll 1
  for (int i = 0; i < t.w * k; i++) B = g1_dbl(B);
  g1_to_aff(B, bases[tid]);
}

// Table entries d * B for d = 1..half of every window base B, one thread per
// run of `run` consecutive entries: the thread reaches (d0 + 1) B by double-
// and-add from B, adds B for each further entry and normalises its run to
// affine with one batched inversion.  The runs keep the build parallel at
// wide windows (2^19 entries per window at w = 20).
__global__ void __launch_bounds__(64) k_table_build(const g1a *bases, int g0, int g1n, FixedTable t, int run,
                                                    g1 *scratch, fp *prod) {
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int runs = t.half / run;
  if (tid >= (size_t)(g1n - g0) * t.nwin * runs) return;
  const size_t base_i = tid / runs;
  const int d0 = (int)(tid % runs) * run;
  const g1a Ba = bases[base_i];
  g1 e = g1_from_aff(Ba);
  const uint32_t m = (uint32_t)d0 + 1;  // e = m * B
  #pragma unroll 1
  for (int b = 30 - __clz(m); b >= 0; b--) {
    e = g1_dbl(e);
    if ((m >> b) & 1) e = g1_add_aff(e, Ba);
  }
  g1 *E = scratch + tid * run;
  fp *Pp = prod + tid * run;
  fp acc = fp_one();
  #pragma unroll 1
  for (int j = 0; j < run; j++) {
    if (j > 0) e = g1_add_aff(e, Ba);
    E[j] = e;
    acc = fp_mul(acc, fp_mul(e.ZZ, e.ZZZ));
    Pp[j] = acc;
  }
  fp inv = fp_inv(acc);  // inverse of prod_j ZZ_j ZZZ_j
  g1a *dst = t.entries + ((size_t)g0 * t.nwin + base_i) * t.half + d0;
  #pragma unroll 1
  for (int j = run - 1; j >= 0; j--) {
    fp zinv = j > 0 ? fp_mul(inv, Pp[j - 1]) : inv;  // 1 / (ZZ_j ZZZ_j)
    g1 ej = E[j];
    inv = fp_mul(inv, fp_mul(ej.ZZ, ej.ZZZ));
    g1a a;
    a.x = fp_mul(ej.X, fp_mul(zinv, ej.ZZZ));
    a.y = fp_mul(ej.Y, fp_mul(zinv, ej.ZZ));
    dst[j] = a;
  }
}

// w-bit field of a raw 256-bit scalar starting at bit pos
DEV uint32_t scalar_bits(const fr &s, int pos, int w) {
  if (pos >= 256) return 0;
  int wi = pos >> 5, sh = pos & 31;
  uint64_t lo = s.w[wi];
  uint64_t hi = wi + 1 < 8 ? s.w[wi + 1] : 0;
  uint64_t v = (lo | (hi << 32)) >> sh;
  return (uint32_t)(v & ((1u << w) - 1));
}

// One MSM row on one warp (all lanes call it): lane l takes generators
// l, l+32, ...; per generator the scalar is recoded into signed w-bit digits
// on the fly and each nonzero digit costs one table lookup and one mixed
// addition; the lanes' sums are added by shuffles.
DEV void fixed_msm_row(const FixedTable &t, const fr *scalars, uint32_t stride, const uint32_t *nterms, uint32_t row,
                       int lane, g1 *out) {
  uint32_t n = nterms[row];
  g1 acc = g1_inf();
  const uint32_t full = 1u << t.w;
  #pragma unroll 1
  for (uint32_t g = lane; g < n; g += 32) {
    fr s = scalars[(size_t)row * stride + g];
    uint32_t carry = 0;
    const g1a *base = t.entries + (size_t)g * t.nwin * t.half;
    #pragma unroll 1
    for (int k = 0; k < t.nwin; k++) {
      uint32_t d = scalar_bits(s, k * t.w, t.w) + carry;
      bool neg = false;
      if (d > (uint32_t)t.half) {
        d = full - d;
        neg = true;
        carry = 1;
      } else {
        carry = 0;
      }
      if (d) {
        g1a e = base[(size_t)k * t.half + d - 1];
        if (neg) e.y = fp_neg(e.y);
        acc = g1_add_aff(acc, e);
      }
    }
  }
  acc = warp_sum_g1(acc);
  if (lane == 0) out[row] = acc;
}

// Fixed-base MSM: row r = sum_g scalars[r*stride + g] * G_g, g < nterms[r]; the
// grid's warps take rows in a grid-stride loop.
__global__ void __launch_bounds__(128) k_fixed_msm(FixedTable t, const fr *scalars, uint32_t stride,
                                                   const uint32_t *nterms, uint32_t rows, g1 *out) {
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  #pragma unroll 1
  for (uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < rows; row += warps)  // per warp
    fixed_msm_row(t, scalars, stride, nterms, row, lane, out);
}

// One lane pair per job (g1_mul_glv_pair): the pair splits each point
// operation's products, halving the latency of a job.
__global__ void __launch_bounds__(128) k_var_mul_pair(const g1a *points, const VarJob *jobs, const fr *scalars,
                                                      uint32_t n, g1 *out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t >> 1;
  if (i >= n) return;  // both lanes of a pair leave together
  const LanePair lp = LanePair::here();
  const VarJob j = jobs[i];
  if (j.flags & 1) {
    if (lp.role == 0) out[i] = g1_inf();
    return;
  }
  const g1 r = g1_mul_glv_pair(lp, points[j.point], scalars[i]);
  if (lp.role == 0) out[i] = r;
}
// One lane quad per job (g1_mul_glv_quad).
__global__ void __launch_bounds__(128) k_var_mul_quad(const g1a *points, const VarJob *jobs, const fr *scalars,
                                                      uint32_t n, g1 *out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t >> 2;
  if (i >= n) return;  // the four lanes of a quad leave together
  const LaneQuad lq = LaneQuad::here();
  const VarJob j = jobs[i];
  if (j.flags & 1) {
    if (lq.role == 0) out[i] = g1_inf();
    return;
  }
  const g1 r = g1_mul_glv_quad(lq, points[j.point], scalars[i]);
  if (lq.role == 0) out[i] = r;
}
// Eight lanes per job (g1_mul_glv_octet): one quad per GLV half.
__global__ void __launch_bounds__(128) k_var_mul_octet(const g1a *points, const VarJob *jobs, const fr *scalars,
                                                       uint32_t n, g1 *out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = t >> 3;
  if (i >= n) return;  // the eight lanes of a job leave together
  const LaneQuad lq = LaneQuad::here();
  const VarJob j = jobs[i];
  if (j.flags & 1) {
    if ((t & 7) == 0) out[i] = g1_inf();
    return;
  }
  const g1 r = g1_mul_glv_octet(lq, points[j.point], scalars[i]);
  if ((t & 7) == 0) out[i] = r;
}
__global__ void __launch_bounds__(128) k_var_mul(const g1a *points, const VarJob *jobs, const fr *scalars,
                                                 uint32_t n, g1 *out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  VarJob j = jobs[i];
  if (j.flags & 1) {
    out[i] = g1_inf();
    return;
  }
  out[i] = g1_mul_glv(points[j.point], scalars[i]);
}

__global__ void __launch_bounds__(128) k_g1_compress(const g1 *pts, uint32_t n, uint8_t *out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint8_t b[48];
  g1_compress(pts[i], b);
  for (int k = 0; k < 48; k++) out[48 * (size_t)i + k] = b[k];
}

// Subgroup check of points decoded without it: bad[i] = 1 when point i
// decoded to an affine point outside G1 (status DEC_OK), else 0.
__global__ void __launch_bounds__(32) k_g1_subgroup_lane(const g1a *pts, const int32_t *status, uint32_t n,
                                                          int32_t *bad) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  bad[i] = (status[i] == DEC_OK && !g1_in_subgroup(pts[i])) ? 1 : 0;
}
// One lane pair per point.
__global__ void __launch_bounds__(32) k_g1_subgroup(const g1a *pts, const int32_t *status, uint32_t n, int32_t *bad) {
  const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 1;
  if (i >= n) return;  // both lanes of a pair leave together
  const LanePair lp = LanePair::here();
  const bool outside = status[i] == DEC_OK && !g1_in_subgroup_pair(lp, pts[i]);
  if (lp.role == 0) bad[i] = outside ? 1 : 0;
}
// One lane quad per point.
__global__ void __launch_bounds__(64) k_g1_subgroup_quad(const g1a *pts, const int32_t *status, uint32_t n,
                                                         int32_t *bad) {
  const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 2;
  if (i >= n) return;  // the four lanes of a quad leave together
  const LaneQuad lq = LaneQuad::here();
  const bool outside = status[i] == DEC_OK && !g1_in_subgroup_quad(lq, pts[i]);
  if (lq.role == 0) bad[i] = outside ? 1 : 0;
}

// CUBBS_BBS_VAR_LANES (1, 2, 4 or 8; else 0: chosen by launch size).
int var_lanes_setting() {
  static const int v = [] {
    const char *e = std::getenv("CUBBS_BBS_VAR_LANES");
    const int x = e && *e ? std::atoi(e) : 0;
    return (x == 1 || x == 2 || x == 4 || x == 8) ? x : 0;
  }();
  return v;
}
// Lanes per job for a launch of n jobs: the CUBBS_BBS_VAR_LANES setting, else
// by size.  A few jobs leave the GPU idle, so each job's chain of products is
// spread over more lanes (8: the two GLV halves on a quad each); thousands of
// jobs fill the GPU, where lane pairs spend the fewest instructions per job.
// Measured on GB300: in the 1024-proof ProofVerify step (4096 jobs) 2 lanes
// 4.47 ms, 4 lanes 5.08, 8 lanes 5.40; Verify of 64 signatures (64 jobs) 8
// lanes 12 % faster than 2.
static int lanes_for(uint32_t n, int max_lanes) {
  int l = var_lanes_setting();
  if (l == 0) l = n <= 1024 ? 8 : n <= 2048 ? 4 : 2;
  return l > max_lanes ? max_lanes : l;
}

void launch_g1_subgroup(cudaStream_t s, const g1a *pts, const int32_t *status, uint32_t n, int32_t *bad, int lanes) {
  if (!n) return;
  if (lanes == 0) lanes = lanes_for(n, 4);
  if (lanes >= 4) k_g1_subgroup_quad<<<blocks_for(4 * (size_t)n, 64), 64, 0, s>>>(pts, status, n, bad);
  else if (lanes == 2) k_g1_subgroup<<<blocks_for(2 * (size_t)n, 32), 32, 0, s>>>(pts, status, n, bad);
  else k_g1_subgroup_lane<<<blocks_for(n, 32), 32, 0, s>>>(pts, status, n, bad);
}
void launch_g1_decode(cudaStream_t s, const uint8_t *pts48, uint32_t stride, uint32_t n, g1a *out, int32_t *status,
                      bool check_subgroup) {
  if (n) k_g1_decode<<<blocks_for(n, 128), 128, 0, s>>>(pts48, stride, n, out, status, check_subgroup);
}
void launch_build_table(cudaStream_t s, const g1a *gens, int g0, int g1n, FixedTable t, g1a *bases, g1 *scratch,
                        fp *prod) {
  const int nb = (g1n - g0) * t.nwin;
  if (nb <= 0) return;
  k_table_bases<<<blocks_for(nb, 64), 64, 0, s>>>(gens, g0, g1n, t, bases);
  const int run = std::min(t.half, 256);
  k_table_build<<<blocks_for((size_t)nb * (t.half / run), 64), 64, 0, s>>>(bases, g0, g1n, t, run, scratch, prod);
}
void launch_fixed_msm(cudaStream_t s, const FixedTable &t, const fr *scalars, uint32_t stride,
                      const uint32_t *nterms, uint32_t rows, g1 *out) {
  // one warp per row: fewer warps with several rows each lengthen the MSM more than they
  // relieve the kernels that share its SMs (measured in the ProofVerify step)
  if (rows) k_fixed_msm<<<blocks_for((size_t)rows * 32, 128), 128, 0, s>>>(t, scalars, stride, nterms, rows, out);
}
void launch_var_mul(cudaStream_t s, const g1a *points, const VarJob *jobs, const fr *scalars, uint32_t n, g1 *out,
                    int lanes) {
  if (!n) return;
  if (lanes == 0) lanes = lanes_for(n, 8);
  if (lanes == 8) k_var_mul_octet<<<blocks_for(8 * (size_t)n, 128), 128, 0, s>>>(points, jobs, scalars, n, out);
  else if (lanes == 4) k_var_mul_quad<<<blocks_for(4 * (size_t)n, 128), 128, 0, s>>>(points, jobs, scalars, n, out);
  else if (lanes == 2) k_var_mul_pair<<<blocks_for(2 * (size_t)n, 128), 128, 0, s>>>(points, jobs, scalars, n, out);
  else k_var_mul<<<blocks_for(n, 128), 128, 0, s>>>(points, jobs, scalars, n, out);
}
cudaError_t warm_decode_and_var_mul_kernels(uint8_t *any_device_buffer) {
  // n = 0: every thread returns before touching memory
  k_g1_decode<<<1, 128>>>(any_device_buffer, 48, 0, nullptr, nullptr, true);
  k_var_mul<<<1, 128>>>(nullptr, nullptr, nullptr, 0, nullptr);
  k_var_mul_pair<<<1, 128>>>(nullptr, nullptr, nullptr, 0, nullptr);
  k_var_mul_quad<<<1, 128>>>(nullptr, nullptr, nullptr, 0, nullptr);
  k_var_mul_octet<<<1, 128>>>(nullptr, nullptr, nullptr, 0, nullptr);
  return cudaGetLastError();
}
void launch_g1_compress(cudaStream_t s, const g1 *pts, uint32_t n, uint8_t *out48) {
  if (n) k_g1_compress<<<blocks_for(n, 128), 128, 0, s>>>(pts, n, out48);
}

}  // namespace cubbs
