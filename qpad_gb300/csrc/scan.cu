// scan.cu -- device-wide exclusive prefix sum of int32 counts (reduce / scan / downsweep),
// used by particle compaction and by the counting sort.
#include "particles.cuh"

namespace qpad {

static constexpr int kScanThreads = 1024;
static constexpr int kScanPerThread = 4;
static constexpr int kScanTile = kScanThreads * kScanPerThread;

__device__ __forceinline__ int block_excl_scan(int v, int* sh, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int o = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += o;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < nw ? sh[lane] : 0;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int o = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += o;
    }
    sh[32 + lane] = w;
  }
  __syncthreads();
  total = sh[32 + nw - 1];
  const int before = warp > 0 ? sh[32 + warp - 1] : 0;
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int32_t* __restrict__ in, int64_t n,
                                                              int32_t* __restrict__ sums) {
  __shared__ int sh[64];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPerThread;
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k)
    if (base + k < n) s += in[base + k];
  int total;
  block_excl_scan(s, sh, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// single CTA: exclusive scan of the block sums in place, total to *total
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int32_t* sums, int nb, int64_t* total) {
  __shared__ int sh[64];
  int carry = 0;
  for (int base = 0; base < nb; base += kScanThreads) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? sums[i] : 0;
    int tot;
    const int ex = block_excl_scan(v, sh, tot);
    if (i < nb) sums[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(const int32_t* __restrict__ in, int64_t n,
                                                            const int32_t* __restrict__ sums, int32_t* __restrict__ out) {
  __shared__ int sh[64];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPerThread;
  int v[kScanPerThread];
  int s = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  int total;
  int run = block_excl_scan(s, sh, total) + sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

int64_t scan_tmp_elems(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

int scan_i32(qpad_ctx* ctx, const int32_t* in, int32_t* out, int64_t n, int32_t* tmp, int64_t* total) {
  const int nb = (int)((n + kScanTile - 1) / kScanTile);
  if (nb == 0) {
    if (total) {
      cudaMemsetAsync(total, 0, sizeof(int64_t), ctx->stream);
      return check_launch(ctx, "scan(empty)", 0);
    }
    return 0;
  }
  k_scan_reduce<<<nb, kScanThreads, 0, ctx->stream>>>(in, n, tmp);
  k_scan_sums<<<1, kScanThreads, 0, ctx->stream>>>(tmp, nb, total);
  k_scan_down<<<nb, kScanThreads, 0, ctx->stream>>>(in, n, tmp, out);
  return check_launch(ctx, "scan_i32", 3);
}

}  // namespace qpad
