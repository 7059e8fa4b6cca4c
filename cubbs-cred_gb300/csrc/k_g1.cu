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

// Signed w-bit digit of window k of scalar s (digits in (-half, half], a
// digit above half becomes d - 2^w with a carry into the next window).  The
// carry into window k is recomputed from the windows below it, so any window
// can be taken alone; the work is a few integer operations per window, next
// to the mixed addition the digit costs.
DEV uint32_t fixed_digit(const fr &s, int k, int w, uint32_t half, bool &neg) {
  uint32_t carry = 0;
  #pragma unroll 1
  for (int i = 0; i < k; i++) carry = scalar_bits(s, i * w, w) + carry > half ? 1u : 0u;
  uint32_t d = scalar_bits(s, k * w, w) + carry;
  neg = d > half;
  return neg ? (1u << w) - d : d;  // 2^w - d is 0 for d = 2^w (the carry alone)
}
// Sum of the points of the L-lane groups of a warp (valid on each group's first lane).
template <int L> DEV g1 group_sum_g1(g1 acc) {
  #pragma unroll 1
  for (int d = L / 2; d > 0; d >>= 1) {
    g1 o;
#pragma unroll
    for (int i = 0; i < 12; i++) {
      o.X.w[i] = __shfl_down_sync(0xffffffffu, acc.X.w[i], d, L);
      o.Y.w[i] = __shfl_down_sync(0xffffffffu, acc.Y.w[i], d, L);
      o.ZZ.w[i] = __shfl_down_sync(0xffffffffu, acc.ZZ.w[i], d, L);
      o.ZZZ.w[i] = __shfl_down_sync(0xffffffffu, acc.ZZZ.w[i], d, L);
    }
    acc = g1_add(acc, o);
  }
  return acc;
}

// Fixed-base MSM: row r = sum_g scalars[r*stride + g] * G_g, g < nterms[r].
// A row runs on a group of L lanes (L = 4 .. 32): its (generator, window)
// units g * nwin + k are dealt round robin to the group's lanes, so every lane
// does the same number of mixed additions whatever the row's length (give or
// take one); each nonzero digit costs one table lookup and one mixed addition,
// and the lanes' sums are added by shuffles within the group.  The warps take
// rows in a grid-stride loop, a warp 32 / L rows at a time (every lane of a
// warp runs the same iterations, as the shuffles need).
template <int L>
__global__ void __launch_bounds__(128) k_fixed_msm(FixedTable t, const fr *scalars, uint32_t stride,
                                                   const uint32_t *nterms, uint32_t rows, g1 *out) {
  constexpr uint32_t PER_WARP = 32 / L;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t lane = threadIdx.x & 31, sub = lane % L, grp = lane / L;
  const uint32_t half = (uint32_t)t.half, nwin = (uint32_t)t.nwin;
  #pragma unroll 1
  for (uint32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * PER_WARP; base < rows;
       base += warps * PER_WARP) {
    const uint32_t row = base + grp;
    const uint32_t units = row < rows ? nterms[row] * nwin : 0;
    g1 acc = g1_inf();
    #pragma unroll 1
    for (uint32_t u = sub; u < units; u += L) {
      const uint32_t g = u / nwin, k = u - g * nwin;
      const fr sc = scalars[(size_t)row * stride + g];
      bool neg;
      const uint32_t d = fixed_digit(sc, (int)k, t.w, half, neg);
      if (d) {
        g1a e = t.entries[((size_t)g * nwin + k) * half + d - 1];
        if (neg) e.y = fp_neg(e.y);
        acc = g1_add_aff_inl(acc, e);  // inlined: no struct arguments through the stack
      }
    }
    acc = group_sum_g1<L>(acc);
    if (sub == 0 && row < rows) out[row] = acc;
  }
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
// Lanes per row (CUBBS_BBS_FIXED_LANES forces 4, 8, 16 or 32): a launch whose
// rows give at most two warps per SM sub-partition at 32 lanes a row is bound
// by one row's latency, so a row gets the whole warp; a larger launch is bound
// by issue, where the shuffle reduction (log2 L full additions on every lane)
// outweighs a shorter chain, so short rows share a warp: 16 lanes for rows of
// 256 units or more, else 8.
static int fixed_lanes_for(uint32_t rows, uint32_t stride, int nwin) {
  static const int forced = [] {
    const char *e = std::getenv("CUBBS_BBS_FIXED_LANES");
    const int x = e && *e ? std::atoi(e) : 0;
    return (x == 4 || x == 8 || x == 16 || x == 32) ? x : 0;
  }();
  if (forced) return forced;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if ((size_t)rows <= (size_t)sms * 8) return 32;
  return (size_t)stride * nwin >= 256 ? 16 : 8;
}
void launch_fixed_msm(cudaStream_t s, const FixedTable &t, const fr *scalars, uint32_t stride,
                      const uint32_t *nterms, uint32_t rows, g1 *out) {
  if (!rows) return;
  const int L = fixed_lanes_for(rows, stride, t.nwin);
  const size_t threads = (size_t)(rows + 32 / L - 1) / (32 / L) * 32;
  const unsigned blocks = blocks_for(threads, 128);
  if (L == 32) k_fixed_msm<32><<<blocks, 128, 0, s>>>(t, scalars, stride, nterms, rows, out);
  else if (L == 16) k_fixed_msm<16><<<blocks, 128, 0, s>>>(t, scalars, stride, nterms, rows, out);
  else if (L == 8) k_fixed_msm<8><<<blocks, 128, 0, s>>>(t, scalars, stride, nterms, rows, out);
  else k_fixed_msm<4><<<blocks, 128, 0, s>>>(t, scalars, stride, nterms, rows, out);
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
