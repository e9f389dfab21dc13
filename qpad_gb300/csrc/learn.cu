// learn.cu -- the learned predictor-corrector guess: a radial 1D conv net per azimuthal
// mode, trained and evaluated on the GPU by this file's own kernels.
//
// Network (per mode): L layers of conv1d(kernel K, zero padding K/2) over the radial nodes,
// widths cin -> W -> ... -> W -> cout, GELU after every layer but the last.  Activations
// are channel-major [C][N] with N = samples * nr (sample-major, radial node fastest).
//
// Every convolution is an im2col GEMM on BF16 tensor cores (mma.sync m16n8k16, FP32
// accumulation) with FP32 master weights:
//   forward       Y[co][n]  = b[co] + sum_k Wt[co][k] * cols[k][n]        (k = ci*K + tap)
//   weight grad   dW[co][k] = sum_n dY[co][n] * cols[k][n]                  (split over n)
//   data grad     dcols[k][n] = sum_co Wt[co][k] * dY[co][n], then col2im
// Training is Adam on the mean squared error.  Everything here is FP32 outside the MMA.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "qpad_internal.cuh"

namespace qpad {

static constexpr int kGT = 64;       // GEMM CTA tile (M and N)
static constexpr int kGK = 32;       // GEMM K step

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat16 l = __float2bfloat16_rn(lo), h = __float2bfloat16_rn(hi);
  return (uint32_t)(*(const uint16_t*)&l) | ((uint32_t)(*(const uint16_t*)&h) << 16);
}

// D = A(16x16, row) * B(16x8, col) + C, bf16 inputs, f32 accumulate
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[M][N] (+)= sum_k A(m,k) B(k,n) over k in [k_begin, k_end), FP32 in global memory.
// A(m,k) = TA ? A[k*lda + m] : A[m*lda + k];  B(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n].
// accumulate: atomicAdd into C (split-K), else C = result (+ bias[m] when bias).
// CTA: 4 warps, tile 64x64; warp w takes rows 32*(w/2).. and columns 32*(w%2)..
template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int N, int Kdim, const float* __restrict__ A, int lda,
                                                   const float* __restrict__ B, int ldb, float* __restrict__ C,
                                                   int ldc, const float* __restrict__ bias, int accumulate,
                                                   int k_chunk) {
  __shared__ float As[kGT][kGK + 1];   // [m][k]
  __shared__ float Bs[kGK][kGT + 1];   // [k][n]
  const int m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  const int kb = blockIdx.z * k_chunk, ke = min(Kdim, kb + k_chunk);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0f;
  for (int k0 = kb; k0 < ke; k0 += kGK) {
    for (int q = t; q < kGT * kGK; q += 128) {
      const int mm = TA ? q % kGT : q / kGK, kk = TA ? q / kGT : q % kGK;
      const int gm = m0 + mm, gk = k0 + kk;
      As[mm][kk] = (gm < M && gk < ke) ? (TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk]) : 0.0f;
    }
    for (int q = t; q < kGK * kGT; q += 128) {
      const int kk = TB ? q % kGK : q / kGT, nn = TB ? q / kGK : q % kGT;
      const int gk = k0 + kk, gn = n0 + nn;
      Bs[kk][nn] = (gk < ke && gn < N) ? (TB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn]) : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < kGK; ks += 16) {
      const int r = lane >> 2, c = (lane & 3) * 2;
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int mr = wm + i * 16 + r;
        af[i][0] = pack_bf16(As[mr][ks + c], As[mr][ks + c + 1]);
        af[i][1] = pack_bf16(As[mr + 8][ks + c], As[mr + 8][ks + c + 1]);
        af[i][2] = pack_bf16(As[mr][ks + c + 8], As[mr][ks + c + 9]);
        af[i][3] = pack_bf16(As[mr + 8][ks + c + 8], As[mr + 8][ks + c + 9]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int nc = wn + j * 8 + r;
        bf[j][0] = pack_bf16(Bs[ks + c][nc], Bs[ks + c + 1][nc]);
        bf[j][1] = pack_bf16(Bs[ks + c + 8][nc], Bs[ks + c + 9][nc]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }
  const int r = lane >> 2, c = (lane & 3) * 2;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const int gm = m0 + wm + i * 16 + r + (h >= 2 ? 8 : 0);
        const int gn = n0 + wn + j * 8 + c + (h & 1);
        if (gm >= M || gn >= N) continue;
        float* dst = C + (size_t)gm * ldc + gn;
        if (accumulate) atomicAdd(dst, acc[i][j][h]);
        else *dst = acc[i][j][h] + (bias ? bias[gm] : 0.0f);
      }
}

// cols[(ci*K + tap)][n] = X[ci][n + tap - K/2] within the same sample, else 0
__global__ void k_im2col(const float* __restrict__ X, int C, int N, int nr, int K, float* __restrict__ cols) {
  const int64_t total = (int64_t)C * K * N;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(q % N);
    const int row = (int)(q / N);
    const int ci = row / K, tap = row % K;
    const int x = n % nr, xs = x + tap - K / 2;
    cols[q] = (xs >= 0 && xs < nr) ? X[(size_t)ci * N + n - x + xs] : 0.0f;
  }
}

// dX[ci][n] = sum_tap dcols[(ci*K + tap)][n - tap + K/2] within the same sample
__global__ void k_col2im(const float* __restrict__ dcols, int C, int N, int nr, int K, float* __restrict__ dX) {
  const int64_t total = (int64_t)C * N;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(q % N), ci = (int)(q / N);
    const int x = n % nr;
    float s = 0.0f;
    for (int tap = 0; tap < K; ++tap) {
      const int xo = x - tap + K / 2;
      if (xo >= 0 && xo < nr) s += dcols[((size_t)ci * K + tap) * N + n - x + xo];
    }
    dX[q] = s;
  }
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__global__ void k_gelu(const float* __restrict__ pre, float* __restrict__ out, int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    out[q] = gelu(pre[q]);
}

// dpre = dout * gelu'(pre)
__global__ void k_gelu_back(const float* pre, const float* dout, float* dpre, int64_t n) {   // dout may be dpre
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    dpre[q] = dout[q] * gelu_grad(pre[q]);
}

// mean squared error over [C][N]: loss partial sums and dY = 2 (Y - T) / (C N)
__global__ void k_mse(const float* __restrict__ Y, const float* __restrict__ T, float* __restrict__ dY, int64_t n,
                      double* __restrict__ loss) {
  double s = 0.0;
  const float sc = 2.0f / (float)n;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const float d = Y[q] - T[q];
    dY[q] = sc * d;
    s += (double)d * d;
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

// db[co] = sum_n dY[co][n]
__global__ void k_bias_grad(const float* __restrict__ dY, int C, int N, float* __restrict__ db) {
  const int co = blockIdx.x;
  float s = 0.0f;
  for (int n = threadIdx.x; n < N; n += blockDim.x) s += dY[(size_t)co * N + n];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  __shared__ float red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float tot = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    db[co] += tot;
  }
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1, float* __restrict__ m2,
                       int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const float gq = g[q];
    const float a = b1 * m1[q] + (1.0f - b1) * gq;
    const float b = b2 * m2[q] + (1.0f - b2) * gq * gq;
    m1[q] = a;
    m2[q] = b;
    w[q] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
  }
}

static int egrid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

}  // namespace qpad

using namespace qpad;

// Work buffers of one forward (and backward) pass over up to `cap` columns.
struct LearnBufs {
  int64_t cap = 0;
  float* act = nullptr;            // layer inputs [layers+1][maxC][cap]
  float* pre = nullptr;            // pre-activations [layers][maxC][cap]
  float* cols = nullptr;           // [maxC*K][cap]
  float* dcur = nullptr;           // [maxC][cap]
  float* dnext = nullptr;          // [maxC][cap]
  float* target = nullptr;         // [cout][cap]
};

struct qpad_learn {
  int cin, cout, width, layers, ksize;
  std::vector<int> ci, co;         // channels in / out per layer
  std::vector<size_t> woff, boff;  // offsets of each layer's weights / biases in the parameter block
  size_t nparam = 0;
  float* param = nullptr;          // FP32 master weights [co][ci*K] then biases, layer by layer
  float* grad = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  int64_t step = 0;
  LearnBufs B;                     // training / prediction buffers
  double* loss = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  int maxc = 0;
};

namespace {
int lerr(qpad_learn* L, int code, const std::string& m) {
  if (L) L->err = m;
  return code;
}
int lcheck(qpad_learn* L, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return QPAD_OK;
  return lerr(L, QPAD_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void free_bufs(LearnBufs& B) {
  for (float** p : {&B.act, &B.pre, &B.cols, &B.dcur, &B.dnext, &B.target})
    if (*p) { cudaFree(*p); *p = nullptr; }
  B.cap = 0;
}

int alloc_bufs(const qpad_learn* L, LearnBufs& B, int64_t cols, bool train) {
  free_bufs(B);
  const size_t mc = (size_t)L->maxc;
  cudaError_t e = cudaMalloc(&B.act, sizeof(float) * (L->layers + 1) * mc * cols);
  if (e == cudaSuccess) e = cudaMalloc(&B.pre, sizeof(float) * L->layers * mc * cols);
  if (e == cudaSuccess) e = cudaMalloc(&B.cols, sizeof(float) * mc * L->ksize * cols);
  if (train) {
    if (e == cudaSuccess) e = cudaMalloc(&B.dcur, sizeof(float) * mc * cols);
    if (e == cudaSuccess) e = cudaMalloc(&B.dnext, sizeof(float) * mc * cols);
    if (e == cudaSuccess) e = cudaMalloc(&B.target, sizeof(float) * L->cout * cols);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    free_bufs(B);
    return QPAD_E_NOMEM;
  }
  B.cap = cols;
  return 0;
}

int ensure_cap(qpad_learn* L, int64_t cols) {
  if (cols <= L->B.cap) return 0;
  if (alloc_bufs(L, L->B, cols, true)) return lerr(L, QPAD_E_NOMEM, "learn work buffers");
  return 0;
}

template <bool TA, bool TB>
void gemm(cudaStream_t st, int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
          const float* bias, bool accumulate, int ksplit = 1) {
  const int k_chunk = ((K + ksplit - 1) / ksplit + kGK - 1) / kGK * kGK;
  dim3 grid((N + kGT - 1) / kGT, (M + kGT - 1) / kGT, (K + k_chunk - 1) / k_chunk);
  k_gemm_bf16<TA, TB><<<grid, 128, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, accumulate ? 1 : 0, k_chunk);
}

float* act_of(const qpad_learn* L, const LearnBufs& B, int layer) { return B.act + (size_t)layer * L->maxc * B.cap; }
float* pre_of(const qpad_learn* L, const LearnBufs& B, int layer) { return B.pre + (size_t)layer * L->maxc * B.cap; }

}  // namespace

// forward pass over N columns already in act layer 0 of B; output in act[layers]
int learn_forward(const qpad_learn* L, const LearnBufs& B, cudaStream_t st, int N, int nr) {
  for (int l = 0; l < L->layers; ++l) {
    const int ci = L->ci[l], co = L->co[l], K = L->ksize;
    k_im2col<<<egrid((int64_t)ci * K * N), 256, 0, st>>>(act_of(L, B, l), ci, N, nr, K, B.cols);
    float* out = (l == L->layers - 1) ? act_of(L, B, l + 1) : pre_of(L, B, l);
    gemm<false, false>(st, co, N, ci * K, L->param + L->woff[l], ci * K, B.cols, N, out, N, L->param + L->boff[l],
                       false);
    if (l < L->layers - 1) k_gelu<<<egrid((int64_t)co * N), 256, 0, st>>>(out, act_of(L, B, l + 1), (int64_t)co * N);
  }
  return 3 * L->layers - 1;   // kernels launched
}

namespace {
// backward from dY (in B.dcur) to the parameter gradients (accumulated into grad)
void backward(qpad_learn* L, int N, int nr) {
  LearnBufs& B = L->B;
  for (int l = L->layers - 1; l >= 0; --l) {
    const int ci = L->ci[l], co = L->co[l], K = L->ksize;
    if (l < L->layers - 1)   // through the GELU of this layer's output
      k_gelu_back<<<egrid((int64_t)co * N), 256, 0, L->stream>>>(pre_of(L, B, l), B.dcur, B.dcur, (int64_t)co * N);
    k_bias_grad<<<co, 256, 0, L->stream>>>(B.dcur, co, N, L->grad + L->boff[l]);
    k_im2col<<<egrid((int64_t)ci * K * N), 256, 0, L->stream>>>(act_of(L, B, l), ci, N, nr, K, B.cols);
    const int ksplit = std::max(1, std::min(64, N / 2048));
    gemm<false, true>(L->stream, co, ci * K, N, B.dcur, N, B.cols, N, L->grad + L->woff[l], ci * K, nullptr, true,
                      ksplit);
    if (l > 0) {
      gemm<true, false>(L->stream, ci * K, N, co, L->param + L->woff[l], ci * K, B.dcur, N, B.cols, N, nullptr, false);
      k_col2im<<<egrid((int64_t)ci * N), 256, 0, L->stream>>>(B.cols, ci, N, nr, K, B.dnext);
      std::swap(B.dcur, B.dnext);
    }
  }
}
}  // namespace

extern "C" int qpad_learn_create(int cin, int cout, int width, int layers, int ksize, uint64_t seed, int device,
                                 qpad_learn** out) {
  if (!out || cin < 1 || cout < 1 || width < 1 || layers < 1 || ksize < 1 || ksize % 2 == 0 || layers > 16)
    return QPAD_E_ARG;
  *out = nullptr;
  qpad_learn* L = new (std::nothrow) qpad_learn();
  if (!L) return QPAD_E_NOMEM;
  L->cin = cin; L->cout = cout; L->width = width; L->layers = layers; L->ksize = ksize;
  L->maxc = std::max(std::max(cin, cout), width);
  size_t off = 0;
  for (int l = 0; l < layers; ++l) {
    L->ci.push_back(l == 0 ? cin : width);
    L->co.push_back(l == layers - 1 ? cout : width);
    L->woff.push_back(off);
    off += (size_t)L->co[l] * L->ci[l] * ksize;
    L->boff.push_back(off);
    off += (size_t)L->co[l];
  }
  L->nparam = off;
  int r = lcheck(L, cudaSetDevice(device), "cudaSetDevice");
  if (!r) r = lcheck(L, cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking), "stream");
  for (float** p : {&L->param, &L->grad, &L->m1, &L->m2})
    if (!r) r = lcheck(L, cudaMalloc(p, sizeof(float) * L->nparam), "cudaMalloc(params)");
  if (!r) r = lcheck(L, cudaMalloc(&L->loss, sizeof(double)), "cudaMalloc(loss)");
  if (!r) {
    // He-style initialisation, last layer scaled down so that the initial guess is ~0
    std::mt19937_64 g(seed);
    std::vector<float> h(L->nparam, 0.0f);
    for (int l = 0; l < layers; ++l) {
      const size_t nw = (size_t)L->co[l] * L->ci[l] * ksize;
      const double sd = std::sqrt(2.0 / (double)(L->ci[l] * ksize)) * (l == layers - 1 ? 0.1 : 1.0);
      std::normal_distribution<double> nd(0.0, sd);
      for (size_t q = 0; q < nw; ++q) h[L->woff[l] + q] = (float)nd(g);
    }
    r = lcheck(L, cudaMemcpy(L->param, h.data(), sizeof(float) * L->nparam, cudaMemcpyHostToDevice), "upload params");
    if (!r) r = lcheck(L, cudaMemset(L->m1, 0, sizeof(float) * L->nparam), "memset");
    if (!r) r = lcheck(L, cudaMemset(L->m2, 0, sizeof(float) * L->nparam), "memset");
  }
  if (r) {
    qpad_learn_destroy(L);
    return r;
  }
  *out = L;
  return QPAD_OK;
}

extern "C" int qpad_learn_destroy(qpad_learn* L) {
  if (!L) return QPAD_OK;
  for (float* p : {L->param, L->grad, L->m1, L->m2})
    if (p) cudaFree(p);
  free_bufs(L->B);
  if (L->loss) cudaFree(L->loss);
  if (L->stream) cudaStreamDestroy(L->stream);
  delete L;
  return QPAD_OK;
}

extern "C" const char* qpad_learn_last_error(const qpad_learn* L) { return L ? L->err.c_str() : "null net"; }

extern "C" int qpad_learn_param_count(const qpad_learn* L, int64_t* n) {
  if (!L || !n) return QPAD_E_ARG;
  *n = (int64_t)L->nparam;
  return QPAD_OK;
}

extern "C" int qpad_learn_get_params(qpad_learn* L, float* host) {
  if (!L || !host) return QPAD_E_ARG;
  return lcheck(L, cudaMemcpy(host, L->param, sizeof(float) * L->nparam, cudaMemcpyDeviceToHost), "download params");
}

extern "C" int qpad_learn_set_params(qpad_learn* L, const float* host) {
  if (!L || !host) return QPAD_E_ARG;
  return lcheck(L, cudaMemcpy(L->param, host, sizeof(float) * L->nparam, cudaMemcpyHostToDevice), "upload params");
}

// Y[s][cout][nr] = net(X[s][cin][nr]) for ns samples (host arrays, sample-major)
extern "C" int qpad_learn_predict(qpad_learn* L, const float* X, int64_t ns, int nr, float* Y) {
  if (!L || !X || !Y || ns < 1 || nr < 1) return QPAD_E_ARG;
  const int64_t N = ns * nr;
  if (N > INT32_MAX / 8) return lerr(L, QPAD_E_CAPACITY, "too many columns");
  if (int r = ensure_cap(L, N)) return r;
  // host [s][c][x] -> device channel-major [c][s*nr + x]
  for (int c = 0; c < L->cin; ++c)
    for (int64_t s = 0; s < ns; ++s)
      if (int r = lcheck(L, cudaMemcpyAsync(act_of(L, L->B, 0) + (size_t)c * N + s * nr, X + ((size_t)s * L->cin + c) * nr,
                                            sizeof(float) * nr, cudaMemcpyHostToDevice, L->stream), "upload X"))
        return r;
  learn_forward(L, L->B, L->stream, (int)N, nr);
  for (int c = 0; c < L->cout; ++c)
    for (int64_t s = 0; s < ns; ++s)
      if (int r = lcheck(L, cudaMemcpyAsync(Y + ((size_t)s * L->cout + c) * nr, act_of(L, L->B, L->layers) + (size_t)c * N + s * nr,
                                            sizeof(float) * nr, cudaMemcpyDeviceToHost, L->stream), "download Y"))
        return r;
  return lcheck(L, cudaStreamSynchronize(L->stream), "predict");
}

namespace {
int upload_batch(qpad_learn* L, const float* X, const float* T, const int64_t* idx, int64_t nb, int nr) {
  const int64_t N = nb * nr;
  std::vector<float> hx((size_t)L->cin * N), ht((size_t)L->cout * N);
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t s = idx ? idx[b] : b;
    for (int c = 0; c < L->cin; ++c)
      std::memcpy(&hx[(size_t)c * N + b * nr], X + ((size_t)s * L->cin + c) * nr, sizeof(float) * nr);
    for (int c = 0; c < L->cout; ++c)
      std::memcpy(&ht[(size_t)c * N + b * nr], T + ((size_t)s * L->cout + c) * nr, sizeof(float) * nr);
  }
  int r = lcheck(L, cudaMemcpyAsync(act_of(L, L->B, 0), hx.data(), sizeof(float) * hx.size(), cudaMemcpyHostToDevice,
                                    L->stream), "upload batch");
  if (!r) r = lcheck(L, cudaMemcpyAsync(L->B.target, ht.data(), sizeof(float) * ht.size(), cudaMemcpyHostToDevice,
                                        L->stream), "upload target");
  if (!r) r = lcheck(L, cudaStreamSynchronize(L->stream), "batch sync");
  return r;
}

// loss and gradient (into L->grad, zeroed first) of one uploaded batch of N columns
int loss_grad(qpad_learn* L, int64_t N, int nr, double* loss_out) {
  if (int r = lcheck(L, cudaMemsetAsync(L->grad, 0, sizeof(float) * L->nparam, L->stream), "zero grad")) return r;
  if (int r = lcheck(L, cudaMemsetAsync(L->loss, 0, sizeof(double), L->stream), "zero loss")) return r;
  learn_forward(L, L->B, L->stream, (int)N, nr);
  const int64_t ny = (int64_t)L->cout * N;
  k_mse<<<egrid(ny), 256, 0, L->stream>>>(act_of(L, L->B, L->layers), L->B.target, L->B.dcur, ny, L->loss);
  backward(L, (int)N, nr);
  double h = 0.0;
  if (int r = lcheck(L, cudaMemcpyAsync(&h, L->loss, sizeof(double), cudaMemcpyDeviceToHost, L->stream), "loss"))
    return r;
  if (int r = lcheck(L, cudaStreamSynchronize(L->stream), "loss sync")) return r;
  if (loss_out) *loss_out = h / (double)ny;
  return 0;
}
}  // namespace

// Mean squared error of the first ns samples and its gradient with respect to every
// parameter (host arrays; grad has qpad_learn_param_count entries).
extern "C" int qpad_learn_grad(qpad_learn* L, const float* X, const float* T, int64_t ns, int nr, double* loss,
                               float* grad) {
  if (!L || !X || !T || ns < 1 || nr < 1) return QPAD_E_ARG;
  const int64_t N = ns * nr;
  if (int r = ensure_cap(L, N)) return r;
  if (int r = upload_batch(L, X, T, nullptr, ns, nr)) return r;
  if (int r = loss_grad(L, N, nr, loss)) return r;
  if (grad)
    return lcheck(L, cudaMemcpy(grad, L->grad, sizeof(float) * L->nparam, cudaMemcpyDeviceToHost), "download grad");
  return 0;
}

// Adam training on ns samples: `epochs` passes in shuffled mini-batches of `batch` samples.
// losses[e] receives the mean training loss of epoch e.
extern "C" int qpad_learn_train(qpad_learn* L, const float* X, const float* T, int64_t ns, int nr, int epochs,
                                int batch, float lr, uint64_t seed, double* losses) {
  if (!L || !X || !T || ns < 1 || nr < 1 || epochs < 1 || batch < 1 || !(lr > 0.0f)) return QPAD_E_ARG;
  const int64_t nb = std::min<int64_t>(batch, ns);
  if (int r = ensure_cap(L, nb * nr)) return r;
  std::mt19937_64 g(seed);
  std::vector<int64_t> perm(ns);
  for (int64_t i = 0; i < ns; ++i) perm[i] = i;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int e = 0; e < epochs; ++e) {
    std::shuffle(perm.begin(), perm.end(), g);
    double tot = 0.0;
    int64_t cnt = 0;
    for (int64_t b0 = 0; b0 + nb <= ns; b0 += nb) {
      if (int r = upload_batch(L, X, T, perm.data() + b0, nb, nr)) return r;
      double l = 0.0;
      if (int r = loss_grad(L, nb * nr, nr, &l)) return r;
      ++L->step;
      const float c1 = 1.0f - std::pow(b1, (float)L->step), c2 = 1.0f - std::pow(b2, (float)L->step);
      k_adam<<<egrid((int64_t)L->nparam), 256, 0, L->stream>>>(L->param, L->grad, L->m1, L->m2, (int64_t)L->nparam,
                                                                lr, b1, b2, eps, c1, c2);
      if (int r = lcheck(L, cudaGetLastError(), "adam")) return r;
      tot += l;
      ++cnt;
    }
    if (losses) losses[e] = cnt ? tot / (double)cnt : 0.0;
  }
  return lcheck(L, cudaStreamSynchronize(L->stream), "train sync");
}

// =====================================================================================
// The guess hook of the slice loop
// =====================================================================================
// Inputs of mode m at slice j: the previous two slices' B-perp, J-perp and rho - Jz from the
// 3D stores (b_spe, cu, q_spe), channel (d-1)*5*nh + q*nh + h for slice j-d, quantity q in
// {B_r, B_phi, J_r, J_phi, rho-Jz} and part h (Re, Im; m = 0 has Re only), over nodes
// 1..nr, divided by their root mean square s.  Outputs (and training targets), channel
// q*nh + h: q in {dB_r, dB_phi} = B-perp(j) - (2 B-perp(j-1) - B-perp(j-2)), what the linear
// extrapolation from the two previous slices misses, and q in {dJ_r, dJ_phi} =
// (J-perp(j) - J-perp(j-1)) / dxi, also in units of s.  The guess for slice j is then
// b_spe = 2 B-perp(j-1) - B-perp(j-2) + s dB and J-perp = J-perp(j-1) + dxi s dJ (the latter
// replaces the carried predictor J-perp(j-1) + dxi dcu(j-1); off by default).
namespace qpad {

struct GuessStores {
  const double* b2;
  const double* cu2;
  const double* q2;
};

__device__ __forceinline__ double st2(const GridDev& G, const double* f2, int nc, int s, int p, int c, int i) {
  return f2[((((size_t)(s - 1) * G.P + p) * nc + c) * G.ld) + i];
}

__device__ __forceinline__ double guess_raw_in(const GridDev& G, const GuessStores& S, int j, int m, int ch, int i) {
  const int nh = m == 0 ? 1 : 2;
  const int d = ch / (5 * nh) + 1, q = (ch / nh) % 5, h = ch % nh;
  const int p = h == 0 ? part_re(m) : part_im(m), s = j - d;
  if (q < 2) return st2(G, S.b2, 3, s, p, q, i);
  if (q < 4) return st2(G, S.cu2, 3, s, p, q - 2, i);
  return st2(G, S.q2, 1, s, p, 0, i) - st2(G, S.cu2, 3, s, p, 2, i);
}

// One CTA per mode (blockIdx.x = m, or m_fixed >= 0 for a single mode).  X rows have
// length ldx (columns), mode m writes at column (m - 1) * nr of X1 (m >= 1) or at 0 of X0.
__global__ void __launch_bounds__(256) k_guess_in(GridDev G, GuessStores S, const int* __restrict__ jp, int j_fixed,
                                                  int m_fixed, float* __restrict__ X0, float* __restrict__ X1, int ldx1,
                                                  float* __restrict__ scale, float* __restrict__ T) {
  const int j = jp ? *jp : j_fixed;
  const int m = m_fixed >= 0 ? m_fixed : (int)blockIdx.x;
  if (j < 3) return;
  const int nr = G.nr, nh = m == 0 ? 1 : 2, cin = 10 * nh;
  float* X = m == 0 ? X0 : X1 + (size_t)(m_fixed >= 0 ? 0 : (m - 1) * nr);
  const int ldx = m == 0 ? nr : ldx1;
  double ss = 0.0;
  for (int q = threadIdx.x; q < cin * nr; q += blockDim.x) {
    const int ch = q / nr, x = q % nr;
    const double v = guess_raw_in(G, S, j, m, ch, x + 1);
    ss += v * v;
    X[(size_t)ch * ldx + x] = (float)v;
  }
  __shared__ double red[8];
  for (int off = 16; off > 0; off >>= 1) ss += __shfl_down_sync(0xffffffffu, ss, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
  __syncthreads();
  __shared__ float s_inv;
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    const double sc = sqrt(tot / (double)(cin * nr)) + 1e-30;
    scale[m_fixed >= 0 ? 0 : m] = (float)sc;
    s_inv = (float)(1.0 / sc);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < cin * nr; q += blockDim.x) X[(size_t)(q / nr) * ldx + q % nr] *= s_inv;
  if (!T) return;
  for (int q = threadIdx.x; q < 4 * nh * nr; q += blockDim.x) {   // training targets of slice j
    const int ch = q / nr, x = q % nr, i = x + 1;
    const int qq = ch / nh, h = ch % nh, p = h == 0 ? part_re(m) : part_im(m);
    double v;
    if (qq < 2)
      v = st2(G, S.b2, 3, j, p, qq, i) - (2.0 * st2(G, S.b2, 3, j - 1, p, qq, i) - st2(G, S.b2, 3, j - 2, p, qq, i));
    else v = (st2(G, S.cu2, 3, j, p, qq - 2, i) - st2(G, S.cu2, 3, j - 1, p, qq - 2, i)) / G.dxi;
    T[(size_t)ch * nr + x] = (float)(v * s_inv);
  }
}

// Applies the net's outputs of every mode (blockIdx.x = m) as the guess of slice j.
__global__ void __launch_bounds__(256) k_guess_out(GridDev G, GuessStores S, const int* __restrict__ jp,
                                                   const float* __restrict__ Y0, const float* __restrict__ Y1, int ldy1,
                                                   const float* __restrict__ scale, double* __restrict__ b_spe,
                                                   double* __restrict__ cu, int apply, double weight) {
  const int j = *jp;
  const int m = blockIdx.x;
  if (j < 3) return;
  const int nr = G.nr, nh = m == 0 ? 1 : 2;
  const float* Y = m == 0 ? Y0 : Y1 + (size_t)(m - 1) * nr;
  const int ldy = m == 0 ? nr : ldy1;
  const double s = (double)scale[m];
  for (int q = threadIdx.x; q < 2 * nh * nr; q += blockDim.x) {
    const int ch = q / nr, x = q % nr, i = x + 1;
    const int c = ch / nh, h = ch % nh, p = h == 0 ? part_re(m) : part_im(m);
    // the axis node takes the extrapolation alone
    if (apply & 1)
      b_spe[fidx(G.ld, 3, p, c, i)] = 2.0 * st2(G, S.b2, 3, j - 1, p, c, i) - st2(G, S.b2, 3, j - 2, p, c, i) +
                                      (i == 1 ? 0.0 : weight * s * (double)Y[(size_t)ch * ldy + x]);
    if (i == 1) continue;
    if (apply & 2) {     // a blend of the carried predictor and the net's dJ-perp/dxi
      const double carried = cu[fidx(G.ld, 3, p, c, i)];
      const double net = st2(G, S.cu2, 3, j - 1, p, c, i) + G.dxi * s * (double)Y[(size_t)(2 * nh + ch) * ldy + x];
      cu[fidx(G.ld, 3, p, c, i)] = carried + weight * (net - carried);
    }
  }
}

// Inputs of the fused guess: every mode's raw (unnormalised) input channels X[ch][x], one
// CTA per (mode, channel, block of kInNodes nodes) with four nodes per thread, and per CTA
// the partial sum of squares of its inputs (the RMS scale of a mode is formed from its
// 20 x nxb partials, in order, where the net reads them; m = 0 has 10 channels and the
// CTAs of channels 10..19 write a zero partial).
static constexpr int kInNodes = 1024;
__global__ void __launch_bounds__(256) k_guess_in_raw(GridDev G, GuessStores S, const int* __restrict__ jp, int nxb,
                                                      float* __restrict__ X0, float* __restrict__ X1, int ldx1,
                                                      double* __restrict__ part) {
  const int j = *jp;
  if (j < 3) return;
  const int xb = blockIdx.x % nxb, ch = (blockIdx.x / nxb) % 20, m = blockIdx.x / (20 * nxb);
  const int nr = G.nr, nh = m == 0 ? 1 : 2, cin = 10 * nh;
  double ss = 0.0;
  if (ch < cin) {
    float* X = m == 0 ? X0 : X1 + (size_t)(m - 1) * nr;
    const int ldx = m == 0 ? nr : ldx1;
    double v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int x = xb * kInNodes + k * 256 + (int)threadIdx.x;
      v[k] = x < nr ? guess_raw_in(G, S, j, m, ch, x + 1) : 0.0;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int x = xb * kInNodes + k * 256 + (int)threadIdx.x;
      if (x < nr) X[(size_t)ch * ldx + x] = (float)v[k];
      ss += v[k] * v[k];
    }
  }
  __shared__ double red[8];
  for (int off = 16; off > 0; off >>= 1) ss += __shfl_down_sync(0xffffffffu, ss, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    part[blockIdx.x] = tot;
  }
}

// ---- fused inference: the whole net over one radial tile in shared memory ---------------
// One CTA takes a tile of kNetTile output nodes of one mode at a time (net0 for m = 0, net1
// for m >= 1, each CTA staging one net's weights once) and keeps every layer's activations
// in shared memory: the input channels on the tile and a halo of 2 nodes per layer on each
// side (rows outside the radial grid are zero, as the zero padding of every convolution),
// four BF16 tensor-core GEMMs (mma.sync m16n8k16, FP32 accumulation) with bias and GELU in
// their epilogues, and the guess applied to b_spe / cu as k_guess_out does.  The weights are
// BF16 copies of the FP32 master weights, packed once per attach (k_pack_net) as
// [co][tap * cin_pad + ci], so that a 16-wide K step is 16 channels of one tap.
static constexpr int kNetTile = 64;                 // output nodes per tile
static constexpr int kNetRows = kNetTile + 32;      // bound on the rows a layer computes (net_tiles)
static constexpr int kNetBuf = kNetTile + 40;       // rows of an activation buffer
static constexpr int kNetWidth = 64, kNetLayers = 4, kNetK = 5;
static constexpr int kActStride = kNetWidth + 8;    // BF16 per activation row (+8: banks spread)
static constexpr int kNetThreads = 512;
static constexpr int kNetPairs = (4 * (kNetRows / 8) + kNetThreads / 32 - 1) / (kNetThreads / 32);   // MMA tiles per warp
static constexpr int kNetInPer = (kNetBuf * 32 + kNetThreads - 1) / kNetThreads;   // input loads per thread
static constexpr int kMaxGuessParts = 256;                                      // k_guess_in_raw CTAs per mode

struct NetBlock {                   // one net's packed weights
  const __nv_bfloat16* w[kNetLayers];  // [co_pad][kp], k = tap * cin_pad + ci
  const float* b[kNetLayers];          // [co_pad]
  int cin_pad[kNetLayers], co_pad[kNetLayers], kp[kNetLayers];
  int cin, cout;
};

__host__ __device__ inline int net_cin_pad(int c) { return (c + 15) / 16 * 16; }

// packs layer l of an FP32 parameter block (W [co][ci * K + tap], then b [co]) into the
// BF16 layout of NetBlock (zero in the padding), with the rounding of the unfused GEMMs
__global__ void k_pack_net(const float* __restrict__ W, const float* __restrict__ bias, int ci, int co, int K,
                           int cin_pad, int co_pad, int kp, __nv_bfloat16* __restrict__ w16, float* __restrict__ b32) {
  const int n = co_pad * kp;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int o = q / kp, k = q % kp, tap = k / cin_pad, c = k % cin_pad;
    const float v = (o < co && tap < K && c < ci) ? W[(size_t)o * ci * K + c * K + tap] : 0.0f;
    w16[q] = __float2bfloat16_rn(v);
  }
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < co_pad; q += gridDim.x * blockDim.x)
    b32[q] = q < co ? bias[q] : 0.0f;
}

__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// n8 row tiles layer l computes: the rows the layers after it read (kNetTile + 4 (3 - l)),
// rounded up to whole tiles.  Rows past them hold values of an earlier tile (finite), which
// reach only rows the next layer does not need.
__host__ __device__ constexpr int net_tiles(int l) { return (kNetTile + 4 * (kNetLayers - 1 - l) + 7) / 8; }

// One layer: out rows r (0 .. kNetRows) from in rows r .. r + 4.  The (m16 channel tile, n8
// row tile) pairs go round-robin to the warps; with 1 or 4 channel tiles and 16 warps a warp
// keeps one channel tile (its A fragments serve all its pairs).
template <bool kLast>
__device__ __forceinline__ void net_layer(const __nv_bfloat16* in, const __nv_bfloat16* w, const float* bias,
                                          int cin_pad, int co_pad, int kp, int cout, __nv_bfloat16* out,
                                          float* ys, int row_node0, int nr, int nnt) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, q = lane & 3;
  const int nmt = co_pad / 16;
  const int npair = nmt * nnt, nw = kNetThreads / 32;
  const int mt = warp % nmt;
  // this warp's row tiles and their B-fragment rows (fixed for the layer)
  int np = 0;
  const __nv_bfloat16* brow[kNetPairs];
  int ntile[kNetPairs];
#pragma unroll
  for (int k = 0; k < kNetPairs; ++k) {
    const int pr = warp + k * nw;
    ntile[k] = pr < npair ? pr / nmt : 0;
    np += pr < npair ? 1 : 0;
    brow[k] = in + (size_t)(ntile[k] * 8 + g) * kActStride + 2 * q;
  }
  float acc[kNetPairs][4];
#pragma unroll
  for (int k = 0; k < kNetPairs; ++k)
#pragma unroll
    for (int h = 0; h < 4; ++h) acc[k][h] = 0.0f;
  const __nv_bfloat16* wr0 = w + (size_t)(mt * 16 + g) * kp + 2 * q;
  const __nv_bfloat16* wr1 = wr0 + 8 * kp;
  for (int tap = 0; tap < kNetK; ++tap) {
#pragma unroll 2
    for (int c0 = 0; c0 < cin_pad; c0 += 16) {
      const int k0 = tap * cin_pad + c0, boff = tap * kActStride + c0;
      uint32_t af[4];
      af[0] = lds32(wr0 + k0);
      af[1] = lds32(wr1 + k0);
      af[2] = lds32(wr0 + k0 + 8);
      af[3] = lds32(wr1 + k0 + 8);
#pragma unroll
      for (int k = 0; k < kNetPairs; ++k) {
        if (k >= np) break;
        uint32_t bf[2];
        bf[0] = lds32(brow[k] + boff);
        bf[1] = lds32(brow[k] + boff + 8);
        mma_bf16(acc[k], af, bf);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kNetPairs; ++k) {
    if (k >= np) break;
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int co = mt * 16 + g + (h >= 2 ? 8 : 0), r = ntile[k] * 8 + 2 * q + (h & 1);
      const float v = acc[k][h] + bias[co];
      if (kLast) {
        if (co < cout && r < kNetTile) ys[co * kNetTile + r] = v;
      } else {
        const int x = row_node0 + r;                     // radial node (0-based) of this row
        out[(size_t)r * kActStride + co] = __float2bfloat16_rn((x >= 0 && x < nr) ? gelu(v) : 0.0f);
      }
    }
  }
}

__global__ void __launch_bounds__(kNetThreads, 1) k_guess_net(GridDev G, GuessStores S, const int* __restrict__ jp,
                                                             NetBlock n0, NetBlock n1, int g0,
                                                             const float* __restrict__ X0, const float* __restrict__ X1,
                                                             int ldx1, const double* __restrict__ part, int nb,
                                                             double* __restrict__ b_spe, double* __restrict__ cu,
                                                             int apply, double weight) {
  const int j = *jp;
  if (j < 3) return;
  extern __shared__ __align__(16) unsigned char nsm[];
  const bool first = (int)blockIdx.x < g0;
  const NetBlock& N = first ? n0 : n1;
  const int nr = G.nr, T = (nr + kNetTile - 1) / kNetTile;
  const int ntiles = first ? T : G.M * T;
  const int cta = first ? (int)blockIdx.x : (int)blockIdx.x - g0, ncta = first ? g0 : (int)gridDim.x - g0;
  // shared memory: the layers' weights and biases, two activation buffers, the outputs
  __nv_bfloat16* wl[kNetLayers];
  float* bl[kNetLayers];
  size_t off = 0;
#pragma unroll
  for (int l = 0; l < kNetLayers; ++l) {
    wl[l] = reinterpret_cast<__nv_bfloat16*>(nsm + off);
    off += (size_t)N.co_pad[l] * N.kp[l] * 2;
    bl[l] = reinterpret_cast<float*>(nsm + off);
    off += (size_t)N.co_pad[l] * 4;
  }
  __nv_bfloat16* act[2];
  act[0] = reinterpret_cast<__nv_bfloat16*>(nsm + off);
  off += (size_t)kNetBuf * kActStride * 2;
  act[1] = reinterpret_cast<__nv_bfloat16*>(nsm + off);
  off += (size_t)kNetBuf * kActStride * 2;
  float* ys = reinterpret_cast<float*>(nsm + off);   // [cout][kNetTile]
  __shared__ double s_part[kMaxGuessParts];
  __shared__ float s_scale[2];                        // 1 / RMS and RMS of the current tile's mode
  // the weights by 16-byte asynchronous copies, all in flight together (every block is a
  // multiple of 16 bytes at a 16-byte aligned offset)
#pragma unroll
  for (int l = 0; l < kNetLayers; ++l) {
    const int nv = N.co_pad[l] * N.kp[l] / 8;
    const char* src = reinterpret_cast<const char*>(N.w[l]);
    const unsigned dst = (unsigned)__cvta_generic_to_shared(wl[l]);
    for (int v = threadIdx.x; v < nv; v += blockDim.x)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst + 16u * v), "l"(src + 16 * (size_t)v)
                   : "memory");
    for (int v = threadIdx.x; v < N.co_pad[l]; v += blockDim.x) bl[l][v] = N.b[l][v];
  }
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
  for (int v = threadIdx.x; v < 2 * kNetBuf * kActStride / 8; v += blockDim.x)   // rows never written stay 0
    reinterpret_cast<uint4*>(act[0])[v] = make_uint4(0u, 0u, 0u, 0u);
  __syncthreads();
  for (int tile = cta; tile < ntiles; tile += ncta) {
    const int m = first ? 0 : 1 + tile / T, x0 = (tile % T) * kNetTile;
    const int nh = m == 0 ? 1 : 2;
    const float* X = m == 0 ? X0 : X1 + (size_t)(m - 1) * nr;
    const int ldx = m == 0 ? nr : ldx1;
    // the inputs' RMS over the mode (k_guess_in's scale, from the partial sums, loaded
    // together and added in order)
    if ((int)threadIdx.x < nb) s_part[threadIdx.x] = part[m * nb + threadIdx.x];
    // input rows r <-> node x0 - 8 + r, channels ci < cin (zero beyond, and off the grid):
    // every thread's loads in flight together
    const int cp0 = N.cin_pad[0], nin = kNetBuf * cp0;
    float xin[kNetInPer];
#pragma unroll
    for (int k = 0; k < kNetInPer; ++k) {
      const int q = (int)threadIdx.x + k * kNetThreads, r = q / cp0, c = q % cp0, x = x0 - 8 + r;
      xin[k] = (q < nin && c < N.cin && x >= 0 && x < nr) ? X[(size_t)c * ldx + x] : 0.0f;
    }
    __syncthreads();
    // one warp folds the partials (a fixed order: lane-strided sums, then a shuffle tree) and
    // forms the scale once; FP64 work repeated by every thread would occupy the SM's few
    // FP64 units for microseconds
    if (threadIdx.x < 32) {
      double tot = 0.0;
      for (int b = (int)threadIdx.x; b < nb; b += 32) tot += s_part[b];
      for (int off = 16; off > 0; off >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, off);
      if (threadIdx.x == 0) {
        const double scd = sqrt(tot / (double)(10 * nh * nr)) + 1e-30;
        s_scale[0] = (float)(1.0 / scd);
        s_scale[1] = (float)scd;
      }
    }
    __syncthreads();
    const float s_inv = s_scale[0];
#pragma unroll
    for (int k = 0; k < kNetInPer; ++k) {
      const int q = (int)threadIdx.x + k * kNetThreads;
      if (q < nin) act[0][(size_t)(q / cp0) * kActStride + q % cp0] = __float2bfloat16_rn(xin[k] * s_inv);
    }
    __syncthreads();
#pragma unroll
    for (int l = 0; l < kNetLayers - 1; ++l) {
      net_layer<false>(act[l & 1], wl[l], bl[l], N.cin_pad[l], N.co_pad[l], N.kp[l], N.co_pad[l], act[(l + 1) & 1],
                       nullptr, x0 - 8 + 2 * (l + 1), nr, net_tiles(l));
      __syncthreads();
    }
    net_layer<true>(act[1], wl[3], bl[3], N.cin_pad[3], N.co_pad[3], N.kp[3], N.cout, nullptr, ys, x0, nr, net_tiles(3));
    __syncthreads();
    // the guess of slice j on this tile's nodes (k_guess_out's rule)
    const double sc = (double)s_scale[1];
    for (int q = threadIdx.x; q < 2 * nh * kNetTile; q += blockDim.x) {
      const int ch = q / kNetTile, xl = q % kNetTile, x = x0 + xl, i = x + 1;
      if (x >= nr) continue;
      const int c = ch / nh, h = ch % nh, p = h == 0 ? part_re(m) : part_im(m);
      if (apply & 1)
        b_spe[fidx(G.ld, 3, p, c, i)] = 2.0 * st2(G, S.b2, 3, j - 1, p, c, i) - st2(G, S.b2, 3, j - 2, p, c, i) +
                                        (i == 1 ? 0.0 : weight * sc * (double)ys[ch * kNetTile + xl]);
      if (i == 1) continue;
      if (apply & 2) {
        const double carried = cu[fidx(G.ld, 3, p, c, i)];
        const double net = st2(G, S.cu2, 3, j - 1, p, c, i) + G.dxi * sc * (double)ys[(2 * nh + ch) * kNetTile + xl];
        cu[fidx(G.ld, 3, p, c, i)] = carried + weight * (net - carried);
      }
    }
    __syncthreads();                                 // before the next tile overwrites the buffers
  }
}

size_t net_smem_bytes(const NetBlock& N) {
  size_t off = 0;
  for (int l = 0; l < kNetLayers; ++l) off += (size_t)N.co_pad[l] * N.kp[l] * 2 + (size_t)N.co_pad[l] * 4;
  return off + 2 * (size_t)kNetBuf * kActStride * 2 + (size_t)N.cout * kNetTile * 4;
}

}  // namespace qpad

struct qpad_guess_state {
  qpad_learn* net0 = nullptr;     // m = 0
  qpad_learn* net1 = nullptr;     // m >= 1, all modes as one batch
  LearnBufs b0, b1;
  float* scale = nullptr;         // [M+1]
  int apply = 1;                  // bit 0: B-perp guess, bit 1: J-perp predictor
  double weight = 1.0;            // fraction of the net's correction that is applied
  bool fused = false;             // nets of the fused kernel's shape: one k_guess_net launch
  void* packed = nullptr;         // both nets' BF16 weights and biases (NetBlock layout)
  qpad::NetBlock nets[2];
  size_t smem = 0;                // k_guess_net's dynamic shared memory
  int nsm = 0;                    // SMs of the device
  double* part = nullptr;         // k_guess_in_raw's partial sums [M+1][nb]
  int nb = 1;                     // its CTAs per mode
};

namespace qpad {

static GuessStores guess_stores(const qpad_ctx* ctx) {
  return GuessStores{ctx->f2[QPAD_F_B_SPE], ctx->f2[QPAD_F_CU], ctx->f2[QPAD_F_Q_SPE]};
}

void guess_free(qpad_ctx* ctx) {
  if (!ctx->guess) return;
  free_bufs(ctx->guess->b0);
  free_bufs(ctx->guess->b1);
  if (ctx->guess->scale) cudaFree(ctx->guess->scale);
  if (ctx->guess->packed) cudaFree(ctx->guess->packed);
  if (ctx->guess->part) cudaFree(ctx->guess->part);
  delete ctx->guess;
  ctx->guess = nullptr;
}

// Polynomial extrapolation of the initial B-perp guess of slice j (every mode part, nodes
// 1..nr) from the stored B-perp of slices j-1, j-2 (, j-3): order 1 is 2 B1 - B2, order 2 is
// 3 B1 - 3 B2 + B3.  Slices without enough history keep the carried value B(j-1).
__global__ void __launch_bounds__(256) k_guess_extrap(GridDev G, const double* __restrict__ b2,
                                                      const int* __restrict__ jp, double* __restrict__ b_spe,
                                                      int order, double w) {
  const int j = *jp;
  if (j <= order + 1) return;
  const int n = G.P * 2 * G.nr;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int p = q / (2 * G.nr), c = (q / G.nr) % 2, i = q % G.nr + 1;
    const double b1 = st2(G, b2, 3, j - 1, p, c, i), bb = st2(G, b2, 3, j - 2, p, c, i);
    double v;
    if (order == 1) {
      v = 2.0 * b1 - bb;
    } else {
      const double b3 = st2(G, b2, 3, j - 3, p, c, i);
      v = 3.0 * (b1 - bb) + b3;
    }
    b_spe[fidx(G.ld, 3, p, c, i)] = w == 1.0 ? v : b1 + w * (v - b1);
  }
}

// Graph-capturable: the guess of the slice in ctx->d_j (slices 1 and 2 keep the carried one).
int guess_enqueue(qpad_ctx* ctx) {
  qpad_guess_state* g = ctx->guess;
  if (!g && ctx->extrap > 0) {
    const int n = ctx->g.P * 2 * ctx->g.nr;
    k_guess_extrap<<<(n + 255) / 256, 256, 0, ctx->stream>>>(ctx->g, ctx->f2[QPAD_F_B_SPE], ctx->d_j,
                                                             ctx->f[QPAD_F_B_SPE], ctx->extrap, ctx->extrap_w);
    return check_launch(ctx, "k_guess_extrap");
  }
  if (!g) return 0;
  const GridDev& G = ctx->g;
  const int nr = G.nr, M = G.M;
  if (g->fused) {
    prof_begin(ctx, "guess_in");
    k_guess_in_raw<<<(M + 1) * g->nb, 256, 0, ctx->stream>>>(G, guess_stores(ctx), ctx->d_j, g->nb / 20, g->b0.act,
                                                              g->b1.act, M * nr, g->part);
    prof_end(ctx, "guess_in");
    // net0's tiles and net1's (M per radial tile) over at most one CTA per SM, split in
    // proportion to their tile counts
    const int T = (nr + kNetTile - 1) / kNetTile, tot = T * (M + 1);
    const int nsm = g->nsm;
    const int grid = std::max(2, std::min(tot, std::max(nsm, 2)));
    int g0 = M >= 1 ? std::max(1, std::min(T, (int)((int64_t)grid * T / tot))) : grid;
    if (M >= 1 && g0 >= grid) g0 = grid - 1;
    prof_begin(ctx, "guess_net");
    k_guess_net<<<M >= 1 ? grid : g0, kNetThreads, g->smem, ctx->stream>>>(
        G, guess_stores(ctx), ctx->d_j, g->nets[0], g->nets[M >= 1 ? 1 : 0], g0, g->b0.act, g->b1.act, M * nr,
        g->part, g->nb, ctx->f[QPAD_F_B_SPE], ctx->f[QPAD_F_CU], g->apply, g->weight);
    prof_end(ctx, "guess_net");
    return check_launch(ctx, "guess", 2);
  }
  k_guess_in<<<M + 1, 256, 0, ctx->stream>>>(G, guess_stores(ctx), ctx->d_j, 0, -1, g->b0.act, g->b1.act,
                                             M * nr, g->scale, nullptr);
  int n = 1;
  n += learn_forward(g->net0, g->b0, ctx->stream, nr, nr);
  if (M >= 1) n += learn_forward(g->net1, g->b1, ctx->stream, M * nr, nr);
  const float* y0 = g->b0.act + (size_t)g->net0->layers * g->net0->maxc * g->b0.cap;
  const float* y1 = M >= 1 ? g->b1.act + (size_t)g->net1->layers * g->net1->maxc * g->b1.cap : nullptr;
  k_guess_out<<<M + 1, 256, 0, ctx->stream>>>(G, guess_stores(ctx), ctx->d_j, y0, y1, M * nr, g->scale,
                                              ctx->f[QPAD_F_B_SPE], ctx->f[QPAD_F_CU], g->apply, g->weight);
  return check_launch(ctx, "guess", n + 1);
}

}  // namespace qpad

namespace {
// BF16 copies of the attached nets for k_guess_net when both have its shape (width 64, 4
// layers, kernel 5); otherwise the guess runs the per-layer kernels.
int pack_nets(qpad_ctx* ctx, qpad_guess_state* g) {
  const qpad_learn* nets[2] = {g->net0, g->net1 ? g->net1 : g->net0};
  for (const qpad_learn* L : nets)
    if (L->width != kNetWidth || L->layers != kNetLayers || L->ksize != kNetK || L->cout > 16) return 0;
  size_t bytes = 0;
  for (int k = 0; k < 2; ++k) {
    NetBlock& N = g->nets[k];
    N.cin = nets[k]->cin;
    N.cout = nets[k]->cout;
    for (int l = 0; l < kNetLayers; ++l) {
      N.cin_pad[l] = net_cin_pad(nets[k]->ci[l]);
      N.co_pad[l] = nets[k]->co[l] > 16 ? net_cin_pad(nets[k]->co[l]) : 16;
      N.kp[l] = kNetK * N.cin_pad[l] + 8;
      if (N.co_pad[l] != 16 && N.co_pad[l] != 64) return 0;
      bytes += (size_t)N.co_pad[l] * N.kp[l] * 2 + (size_t)N.co_pad[l] * 4;
    }
  }
  if (int r = cuda_check(ctx, cudaMalloc(&g->packed, bytes), "packed guess nets")) return r;
  g->nb = 20 * ((ctx->g.nr + kInNodes - 1) / kInNodes);       // k_guess_in_raw's partials per mode
  if (g->nb > kMaxGuessParts) {                                 // (radial grids above 12800 nodes)
    cudaFree(g->packed);
    g->packed = nullptr;
    return 0;
  }
  if (int r = cuda_check(ctx, cudaMalloc(&g->part, sizeof(double) * (ctx->g.M + 1) * g->nb), "guess partials"))
    return r;
  size_t off = 0;
  for (int k = 0; k < 2; ++k) {
    NetBlock& N = g->nets[k];
    for (int l = 0; l < kNetLayers; ++l) {
      __nv_bfloat16* w = reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(g->packed) + off);
      off += (size_t)N.co_pad[l] * N.kp[l] * 2;
      float* b = reinterpret_cast<float*>(static_cast<char*>(g->packed) + off);
      off += (size_t)N.co_pad[l] * 4;
      k_pack_net<<<64, 256, 0, ctx->stream>>>(nets[k]->param + nets[k]->woff[l], nets[k]->param + nets[k]->boff[l],
                                                nets[k]->ci[l], nets[k]->co[l], kNetK, N.cin_pad[l], N.co_pad[l],
                                                N.kp[l], w, b);
      N.w[l] = w;
      N.b[l] = b;
    }
  }
  if (int r = check_launch(ctx, "k_pack_net", 2 * kNetLayers)) return r;
  g->smem = std::max(net_smem_bytes(g->nets[0]), net_smem_bytes(g->nets[1]));
  if (int r = raise_dyn_smem(ctx, (const void*)k_guess_net, g->smem)) return r;
  if (int r = cuda_check(ctx, cudaDeviceGetAttribute(&g->nsm, cudaDevAttrMultiProcessorCount, ctx->device), "SMs"))
    return r;
  // the nets' parameters are read on their own streams: finish the copies before returning
  if (int r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "pack guess nets")) return r;
  g->fused = true;
  return 0;
}
}  // namespace

extern "C" int qpad_guess_attach(qpad_ctx* ctx, qpad_learn* net0, qpad_learn* net1) {
  if (!ctx) return QPAD_E_ARG;
  guess_free(ctx);
  ctx->step_key.clear();                       // the step graph is rebuilt with or without the guess
  if (ctx->step_exec) {
    cudaGraphExecDestroy(ctx->step_exec);
    ctx->step_exec = nullptr;
  }
  if (!net0) return QPAD_OK;                   // detached
  const int M = ctx->g.M, nr = ctx->g.nr;
  if (net0->cin != 10 || net0->cout != 4 || (M >= 1 && (!net1 || net1->cin != 20 || net1->cout != 8)))
    return set_err(ctx, QPAD_E_ARG, "guess nets: m=0 needs 10 -> 4 channels, m>=1 needs 20 -> 8");
  qpad_guess_state* g = new (std::nothrow) qpad_guess_state();
  if (!g) return set_err(ctx, QPAD_E_NOMEM, "guess state");
  ctx->guess = g;
  g->net0 = net0;
  g->net1 = M >= 1 ? net1 : nullptr;
  int r = alloc_bufs(net0, g->b0, nr, false) ? set_err(ctx, QPAD_E_NOMEM, "guess buffers") : 0;
  if (!r && M >= 1 && alloc_bufs(net1, g->b1, (int64_t)M * nr, false)) r = set_err(ctx, QPAD_E_NOMEM, "guess buffers");
  if (!r) r = cuda_check(ctx, cudaMalloc(&g->scale, sizeof(float) * (M + 1)), "guess scale");
  if (!r) r = pack_nets(ctx, g);
  if (r) guess_free(ctx);
  return r;
}

extern "C" int qpad_guess_sample(qpad_ctx* ctx, int j, int m, float* x, float* t, float* scale) {
  if (!ctx || !x || !t || m < 0 || m > ctx->g.M || j < 3 || j > ctx->g.nz)
    return ctx ? set_err(ctx, QPAD_E_ARG, "guess sample: needs 3 <= j <= nz, 0 <= m <= max_mode") : QPAD_E_ARG;
  const int nr = ctx->g.nr, nh = m == 0 ? 1 : 2;
  const size_t nx = (size_t)10 * nh * nr, nt = (size_t)4 * nh * nr;
  float* d = nullptr;
  if (int r = cuda_check(ctx, cudaMalloc(&d, sizeof(float) * (nx + nt + 1)), "guess sample buffer")) return r;
  k_guess_in<<<1, 256, 0, ctx->stream>>>(ctx->g, guess_stores(ctx), nullptr, j, m, d, d, nr, d + nx + nt, d + nx);
  int r = check_launch(ctx, "k_guess_in");
  if (!r) r = cuda_check(ctx, cudaMemcpyAsync(x, d, sizeof(float) * nx, cudaMemcpyDeviceToHost, ctx->stream), "x");
  if (!r) r = cuda_check(ctx, cudaMemcpyAsync(t, d + nx, sizeof(float) * nt, cudaMemcpyDeviceToHost, ctx->stream), "t");
  if (!r && scale)
    r = cuda_check(ctx, cudaMemcpyAsync(scale, d + nx + nt, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream), "s");
  if (!r) r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "guess sample");
  cudaFree(d);
  return r;
}

extern "C" int qpad_guess_samples(qpad_ctx* ctx, int j_lo, int j_hi, int m, float* x, float* t, float* scale) {
  if (!ctx || !x || !t || m < 0 || m > ctx->g.M || j_lo < 3 || j_hi > ctx->g.nz || j_hi < j_lo)
    return ctx ? set_err(ctx, QPAD_E_ARG, "guess samples: needs 3 <= j_lo <= j_hi <= nz, 0 <= m <= max_mode")
               : QPAD_E_ARG;
  const int nr = ctx->g.nr, nh = m == 0 ? 1 : 2, ns = j_hi - j_lo + 1;
  const size_t nx = (size_t)10 * nh * nr, nt = (size_t)4 * nh * nr;
  float* d = nullptr;
  if (int r = cuda_check(ctx, cudaMalloc(&d, sizeof(float) * (nx + nt + 1) * ns), "guess samples buffer")) return r;
  float* dx = d;
  float* dt = d + nx * ns;
  float* ds = dt + nt * ns;
  int r = 0;
  for (int k = 0; k < ns && !r; ++k) {
    k_guess_in<<<1, 256, 0, ctx->stream>>>(ctx->g, guess_stores(ctx), nullptr, j_lo + k, m, dx + nx * k, dx + nx * k,
                                           nr, ds + k, dt + nt * k);
    r = check_launch(ctx, "k_guess_in");
  }
  if (!r) r = cuda_check(ctx, cudaMemcpyAsync(x, dx, sizeof(float) * nx * ns, cudaMemcpyDeviceToHost, ctx->stream), "x");
  if (!r) r = cuda_check(ctx, cudaMemcpyAsync(t, dt, sizeof(float) * nt * ns, cudaMemcpyDeviceToHost, ctx->stream), "t");
  if (!r && scale)
    r = cuda_check(ctx, cudaMemcpyAsync(scale, ds, sizeof(float) * ns, cudaMemcpyDeviceToHost, ctx->stream), "s");
  if (!r) r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "guess samples");
  cudaFree(d);
  return r;
}

extern "C" int qpad_guess_apply(qpad_ctx* ctx, int j) {
  if (!ctx || j < 3 || j > ctx->g.nz)
    return ctx ? set_err(ctx, QPAD_E_ARG, "guess apply: needs 3 <= j <= nz") : QPAD_E_ARG;
  if (!ctx->guess && ctx->extrap == 0) return set_err(ctx, QPAD_E_STATE, "guess apply: no guess configured");
  if (int r = launch_set_slice(ctx, j)) return r;
  if (int r = guess_enqueue(ctx)) return r;
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "guess apply");
}

extern "C" int qpad_set_guess_extrapolation(qpad_ctx* ctx, int order, double weight) {
  if (!ctx || order < 0 || order > 2 || !(weight >= 0.0 && weight <= 2.0))
    return ctx ? set_err(ctx, QPAD_E_ARG, "guess extrapolation: order 0, 1 or 2, weight in [0, 2]") : QPAD_E_ARG;
  ctx->extrap = order;
  ctx->extrap_w = weight;
  return 0;
}

extern "C" int qpad_guess_config(qpad_ctx* ctx, int apply, double weight) {
  if (!ctx || apply < 0 || apply > 3 || !(weight >= 0.0 && weight <= 1.0))
    return ctx ? set_err(ctx, QPAD_E_ARG, "guess config: apply in 0..3, weight in [0, 1]") : QPAD_E_ARG;
  if (!ctx->guess) return set_err(ctx, QPAD_E_STATE, "guess config: no nets attached");
  ctx->guess->apply = apply;
  ctx->guess->weight = weight;
  return QPAD_OK;
}
