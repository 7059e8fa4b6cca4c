// Allocation-free single G1 MSM: out = sum_k scalars[k] * points[k].
//
// Same arithmetic and result as one item of cubbs_bbs_gpu_g1_msm_batch_v2
// (route 4: device decode with subgroup check, canonical scalar parse, GLV
// variable-base terms, sum, compress), but every device buffer lives in one
// file-scope scratch array instead of the library's growable arena, and the
// call makes no cudaMalloc / cudaFree / cudaHostAlloc and takes no library
// runtime state.  It exists for callers that must not allocate device or
// pinned memory while they run: callers on a hard memory budget that have
// reserved all free device memory up front (a cudaMalloc would fail or evict
// their reservation), and callers inside a custom allocator's own code path,
// where a nested allocation would re-enter that allocator.
//
// Limits and rules (also stated beside the declaration in the header):
//  * at most CUBBS_BBS_GPU_NOALLOC_MSM_MAX_TERMS terms per call; a larger
//    term_count is rejected with CUBBS_BBS_GPU_ERR_NOALLOC_LIMIT before any
//    CUDA call;
//  * the first call on a device does set-up with that device current: it
//    looks up the scratch array's device address (cudaGetSymbolAddress) and
//    launches every kernel the call uses once over zero terms, so that module
//    loading, and the growth of the local memory the driver reserves for the
//    kernels it launches, happen then and not in a later call;
//  * the call is synchronous: it copies with cudaMemcpy on the legacy default
//    stream and returns after the result is on the host.  It cannot be
//    captured into a CUDA graph, and it must not be made while any stream
//    capture is active in the process (a legacy-stream copy would invalidate
//    a capture in global mode);
//  * every call on a device shares the one scratch array.  Overlapping calls
//    would race on it, so calls are serialised by a process-wide lock; work
//    that the caller runs against the same library in other ways does not
//    touch this array;
//  * the status word that the kernels OR flags into is cleared on the device
//    at the start of every call; every other region is fully written before
//    it is read.
//
// No counterpart in the reference ABI.
#include <mutex>

#include "runtime.cuh"

namespace cubbs {
namespace {

constexpr uint32_t kMaxTerms = CUBBS_BBS_GPU_NOALLOC_MSM_MAX_TERMS;
constexpr int kMaxDevices = 64;
constexpr uint32_t kReduceThreads = 256;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Scratch layout (byte offsets into the array).  The host copies the inputs
// into [OFF_POINTS_BE, OFF_SCALARS_BE + 32 * n) and reads back the 64-byte
// result block at OFF_RESULT (48-byte compressed point, then the status word).
constexpr size_t OFF_POINTS_BE = 0;
constexpr size_t OFF_SCALARS_BE = OFF_POINTS_BE + align256(48 * (size_t)kMaxTerms);
constexpr size_t OFF_POINTS = OFF_SCALARS_BE + align256(32 * (size_t)kMaxTerms);
constexpr size_t OFF_POINT_STATUS = OFF_POINTS + align256(sizeof(g1a) * (size_t)kMaxTerms);
constexpr size_t OFF_SCALARS = OFF_POINT_STATUS + align256(4 * (size_t)kMaxTerms);
constexpr size_t OFF_JOBS = OFF_SCALARS + align256(sizeof(fr) * (size_t)kMaxTerms);
constexpr size_t OFF_TERMS = OFF_JOBS + align256(sizeof(VarJob) * (size_t)kMaxTerms);
constexpr size_t OFF_RESULT = OFF_TERMS + align256(sizeof(g1) * (size_t)kMaxTerms);
constexpr size_t RESULT_BYTES = 64;
constexpr size_t SCRATCH_BYTES = OFF_RESULT + align256(RESULT_BYTES);
static_assert(SCRATCH_BYTES < 2u * 1024 * 1024, "scratch array stays under 2 MiB");

static __device__ __align__(256) uint8_t g_msm_scratch[SCRATCH_BYTES];

// Per-device scratch address, filled by the first call on that device.
std::mutex g_mu;
uint8_t *g_scratch_ptr[kMaxDevices] = {};

// Result block: compressed point, then status bits (bit0: a point failed to
// decode or is outside G1, bit1: a scalar is not canonical).
struct ResultBlock {
  uint8_t point[48];
  uint32_t status;
  uint32_t pad[3];
};
static_assert(sizeof(ResultBlock) == RESULT_BYTES, "result block layout");

// Scalar parse + per-term job flags; a bad input ORs a status bit.
__global__ void __launch_bounds__(128) k_na_prepare(uint8_t *scratch, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint8_t *sbe = scratch + OFF_SCALARS_BE;
  const int32_t *pst = reinterpret_cast<const int32_t *>(scratch + OFF_POINT_STATUS);
  fr *sc = reinterpret_cast<fr *>(scratch + OFF_SCALARS);
  VarJob *jobs = reinterpret_cast<VarJob *>(scratch + OFF_JOBS);
  ResultBlock *res = reinterpret_cast<ResultBlock *>(scratch + OFF_RESULT);
  fr s;
  bool ok = fr_raw_from_be32(sbe + 32 * (size_t)i, s);
  sc[i] = ok ? s : fr_zero();
  int st = pst[i];
  jobs[i] = {i, (uint32_t)(st != DEC_OK ? 1 : 0)};  // identity points contribute nothing
  uint32_t bad = (st == DEC_BAD ? 1u : 0u) | (ok ? 0u : 2u);
  if (bad) atomicOr(&res->status, bad);
}

DEV g1 shfl_down_point(const g1 &p, int delta) {
  g1 r;
#pragma unroll
  for (int k = 0; k < 12; k++) {
    r.X.w[k] = __shfl_down_sync(0xffffffffu, p.X.w[k], delta);
    r.Y.w[k] = __shfl_down_sync(0xffffffffu, p.Y.w[k], delta);
    r.ZZ.w[k] = __shfl_down_sync(0xffffffffu, p.ZZ.w[k], delta);
    r.ZZZ.w[k] = __shfl_down_sync(0xffffffffu, p.ZZZ.w[k], delta);
  }
  return r;
}

// One block sums the n terms (strided per thread, warp shuffles, then the
// warp partials through shared memory) and compresses the sum.
__global__ void __launch_bounds__(kReduceThreads) k_na_sum_compress(uint8_t *scratch, uint32_t n) {
  __shared__ g1 partial[kReduceThreads / 32];
  const g1 *terms = reinterpret_cast<const g1 *>(scratch + OFF_TERMS);
  ResultBlock *res = reinterpret_cast<ResultBlock *>(scratch + OFF_RESULT);
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  g1 acc = g1_inf();
#pragma unroll 1
  for (uint32_t j = threadIdx.x; j < n; j += kReduceThreads) acc = g1_add(acc, terms[j]);
#pragma unroll 1
  for (int d = 16; d > 0; d >>= 1) acc = g1_add(acc, shfl_down_point(acc, d));
  if (lane == 0) partial[warp] = acc;
  __syncthreads();
  if (threadIdx.x != 0) return;
  acc = partial[0];
#pragma unroll 1
  for (uint32_t w = 1; w < kReduceThreads / 32; w++) acc = g1_add(acc, partial[w]);
  uint8_t b[48];
  g1_compress(acc, b);
  for (int k = 0; k < 48; k++) res->point[k] = b[k];
}

// Device address of the scratch array for the current device.  Set-up on the
// first call per device: the address, then one launch over zero terms of every
// kernel a call uses (whatever the first call's term count), which loads them
// and lets the driver grow its local-memory reservation for them now rather
// than in a later call.  Caller holds g_mu.
cudaError_t scratch_for_current_device(uint8_t **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_msm_scratch);
    if (e != cudaSuccess) return e;
    uint8_t *scratch = static_cast<uint8_t *>(p);
    k_na_prepare<<<1, 128>>>(scratch, 0);
    k_na_sum_compress<<<1, kReduceThreads>>>(scratch, 0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = warm_decode_and_var_mul_kernels(scratch)) != cudaSuccess) return e;
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return e;
    g_scratch_ptr[dev] = scratch;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

cudaError_t run_noalloc_msm(const uint8_t *points48, const uint8_t *scalars32, uint32_t n, ResultBlock *host_res) {
  uint8_t *scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess) return e;
  cudaStream_t s = 0;  // legacy default stream; every copy below is synchronous
  if (n) {
    if ((e = cudaMemcpy(scratch + OFF_POINTS_BE, points48, 48 * (size_t)n, cudaMemcpyHostToDevice)) != cudaSuccess)
      return e;
    if ((e = cudaMemcpy(scratch + OFF_SCALARS_BE, scalars32, 32 * (size_t)n, cudaMemcpyHostToDevice)) !=
        cudaSuccess)
      return e;
  }
  if ((e = cudaMemsetAsync(scratch + OFF_RESULT, 0, RESULT_BYTES, s)) != cudaSuccess) return e;
  if (n) {
    launch_g1_decode(s, scratch + OFF_POINTS_BE, 48, n, reinterpret_cast<g1a *>(scratch + OFF_POINTS),
                     reinterpret_cast<int32_t *>(scratch + OFF_POINT_STATUS), true);
    k_na_prepare<<<blocks_for(n, 128), 128, 0, s>>>(scratch, n);
    launch_var_mul(s, reinterpret_cast<const g1a *>(scratch + OFF_POINTS),
                   reinterpret_cast<const VarJob *>(scratch + OFF_JOBS),
                   reinterpret_cast<const fr *>(scratch + OFF_SCALARS), n, reinterpret_cast<g1 *>(scratch + OFF_TERMS));
  }
  k_na_sum_compress<<<1, kReduceThreads, 0, s>>>(scratch, n);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  return cudaMemcpy(host_res, scratch + OFF_RESULT, RESULT_BYTES, cudaMemcpyDeviceToHost);
}

}  // namespace
}  // namespace cubbs

using namespace cubbs;

extern "C" int32_t cubbs_bbs_gpu_g1_msm_noalloc_v2(uint32_t abi_version, const uint8_t *points48,
                                                   const uint8_t *scalars32, size_t term_count,
                                                   uint8_t *point_out48, CuBbsBbsGpuResult *result) {
  if (abi_version != CUBBS_BBS_GPU_ABI_VERSION || result == nullptr || point_out48 == nullptr ||
      (term_count > 0 && (points48 == nullptr || scalars32 == nullptr)))
    return CUBBS_BBS_GPU_ERR_INVALID_INPUT;
  if (term_count > kMaxTerms) {
    *result = {CUBBS_BBS_GPU_ERR_NOALLOC_LIMIT, 0, 0};
    return CUBBS_BBS_GPU_ERR_NOALLOC_LIMIT;
  }
  ResultBlock host_res;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (run_noalloc_msm(points48, scalars32, (uint32_t)term_count, &host_res) != cudaSuccess) {
      *result = {CUBBS_BBS_GPU_ERR_INTERNAL, 0, 0};
      return CUBBS_BBS_GPU_ERR_INTERNAL;
    }
  }
  if (host_res.status) {
    *result = {CUBBS_BBS_GPU_ERR_INVALID_INPUT, 0, 0};
    return CUBBS_BBS_GPU_SUCCESS;
  }
  for (int k = 0; k < 48; k++) point_out48[k] = host_res.point[k];
  *result = {CUBBS_BBS_GPU_SUCCESS, CUBBS_BBS_MSM_ROUTE_CUBBS_UNIVERSAL, 48};
  return CUBBS_BBS_GPU_SUCCESS;
}
