// fields.cu -- per-mode radial field solves of the quasi-static slice loop (FP64).
//
// Every solve of the reference goes through HYPRE's struct cyclic-reduction solver with a
// tridiagonal matrix that is analytic in (kind, mode) (field_solver_class.f03:256-561).
// Here the matrices are factorised once per context (Thomas LU, host, FP64) and each
// solve is a forward and a backward substitution.  Both substitutions are first-order
// affine recurrences, evaluated by one CTA as a parallel scan of affine maps
// (y_k = a_k + b_k * y_{k-1}): each thread composes a contiguous chunk of rows, a warp
// shuffle scan plus a cross-warp scan combine the chunks, and each thread then replays
// its chunk.  One CTA owns one azimuthal mode, so the Re/Im right-hand sides of that mode
// (which share the matrix) are solved together, and the source construction
// (set_source_*), the solve and the recovery of the field (get_solution_*) are fused into
// the same kernel with the radial lines held in shared memory.
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "stencils.cuh"

namespace qpad {

#define FULLMASK 0xffffffffu
static constexpr int kFieldThreads = 256;

int field_ncomp(int field) {
  switch (field) {
    case QPAD_F_PSI: case QPAD_F_Q_SPE: case QPAD_F_Q_BEAM: return 1;
    case QPAD_F_ACU: case QPAD_F_DCU: return 2;
    default: return 3;
  }
}

// ------------------------------------------------------------------------------------
// Host: tridiagonal matrices (field_solver_class.f03:256-561) and their factorisation
// ------------------------------------------------------------------------------------
static void build_matrix(const GridDev& g, int kind, int m, double* a, double* b, double* c) {
  const int nr = g.nr;
  const double dr = g.dr, dr2 = dr * dr, m2 = (double)(m * m), rf = g.relax_fac;
  for (int k = 2; k <= nr; ++k) {                      // rows 2..nr, j = row - 1
    double j = (double)(k - 1);
    a[k - 1] = 1.0 - 0.5 / j;
    c[k - 1] = 1.0 + 0.5 / j;
    if (kind == OK_BPLUS) {
      double t = (double)(m + 1) / j;
      b[k - 1] = -2.0 - t * t - rf;
    } else if (kind == OK_BMINUS) {
      double t = (double)(m - 1) / j;
      b[k - 1] = -2.0 - t * t - rf;
    } else {
      b[k - 1] = -2.0 - m2 / (j * j);
    }
  }
  bool identity_axis = true;                           // axis row
  if (kind == OK_BMINUS && m == 1) {
    a[0] = 0.0; b[0] = -4.0 - rf; c[0] = 4.0; identity_axis = false;
  } else if ((kind == OK_GEN || kind == OK_BT) && m == 0) {
    a[0] = 0.0; b[0] = -4.0; c[0] = 4.0; identity_axis = false;
  }
  if (identity_axis) {
    a[0] = 0.0; b[0] = 1.0; c[0] = 0.0;
    if (nr >= 2) a[1] = 0.0;
  }
  if (g.bnd == QPAD_BND_ZERO) {                        // outer row
    c[nr - 1] = 0.0;
  } else {
    const double jmax = (double)nr;
    bool dirichlet = false;
    double fac = 0.0;
    if (kind == OK_GEN) {
      if (m == 0) dirichlet = true; else fac = 1.0 - (double)m / jmax;
    } else if (kind == OK_BT) {
      fac = (m == 0) ? 1.0 + 1.0 / (jmax * std::log(jmax * dr)) : 1.0 - (double)m / jmax;
    } else {
      fac = 1.0 - (double)(m + 1) / jmax;              // B+ and B- both use (m+1)
    }
    if (!dirichlet) b[nr - 1] = b[nr - 1] + fac * c[nr - 1];
    c[nr - 1] = 0.0;
  }
  for (int k = 0; k < nr; ++k) { a[k] /= dr2; b[k] /= dr2; c[k] /= dr2; }
}

int build_factors(qpad_ctx* ctx) {
  const GridDev& g = ctx->g;
  const int nr = g.nr, M = g.M;
  std::vector<double> h((size_t)OK_NKINDS * (M + 1) * 3 * nr);
  std::vector<double> a(nr), b(nr), c(nr);
  for (int kind = 0; kind < OK_NKINDS; ++kind)
    for (int m = 0; m <= M; ++m) {
      build_matrix(g, kind, m, a.data(), b.data(), c.data());
      double* w = h.data() + fac_off(nr, M, kind, m);
      double* ib = w + nr;
      double* gg = ib + nr;
      double piv = b[0];
      w[0] = 0.0;
      ib[0] = 1.0 / piv;
      for (int k = 1; k < nr; ++k) {
        w[k] = a[k] / piv;
        piv = b[k] - w[k] * c[k - 1];
        ib[k] = 1.0 / piv;
      }
      for (int k = 0; k < nr; ++k) gg[k] = c[k] * ib[k];
      for (int k = 0; k < nr; ++k)
        if (!std::isfinite(ib[k]) || !std::isfinite(w[k]))
          return set_err(ctx, QPAD_E_ARG, "singular tridiagonal operator (check nr, dr, relax_fac)");
    }
  // node tables of the finite-difference factors (same FP64 expressions as the reference)
  std::vector<double> rt(2 * (size_t)g.ld, 0.0);
  for (int i = 2; i < g.ld; ++i) {
    rt[i] = g.idr / (double)(i - 1);
    rt[g.ld + i] = 1.0 / (double)(i - 1);
  }
  cudaError_t e = cudaMalloc(&ctx->rtab, rt.size() * sizeof(double));
  if (e != cudaSuccess) return cuda_check(ctx, e, "cudaMalloc(node tables)");
  e = cudaMemcpy(ctx->rtab, rt.data(), rt.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_check(ctx, e, "upload node tables");
  ctx->g.ir = ctx->rtab;
  ctx->g.inv = ctx->rtab + g.ld;
  e = cudaMalloc(&ctx->fac, h.size() * sizeof(double));
  if (e != cudaSuccess) return cuda_check(ctx, e, "cudaMalloc(factors)");
  return cuda_check(ctx, cudaMemcpy(ctx->fac, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice),
                    "upload factors");
}

// ------------------------------------------------------------------------------------
// Device: CTA-wide scan of affine maps and the substitution passes
// ------------------------------------------------------------------------------------
// Composition convention: map (B, A) sends y -> A + B*y.  Later-after-earlier composes as
// (B_l*B_e, A_l + B_l*A_e).  `reverse` walks the threads (and their chunks) downward.
template <int NV>
__device__ __forceinline__ void affine_scan(double& B, double (&A)[NV], bool reverse, double* sc) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    double Bo = reverse ? __shfl_down_sync(FULLMASK, B, off) : __shfl_up_sync(FULLMASK, B, off);
    double Ao[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
      Ao[v] = reverse ? __shfl_down_sync(FULLMASK, A[v], off) : __shfl_up_sync(FULLMASK, A[v], off);
    const bool valid = reverse ? (lane + off < 32) : (lane >= off);
    if (valid) {
#pragma unroll
      for (int v = 0; v < NV; ++v) A[v] = A[v] + B * Ao[v];
      B = B * Bo;
    }
  }
  double Be = reverse ? __shfl_down_sync(FULLMASK, B, 1) : __shfl_up_sync(FULLMASK, B, 1);
  double Ae[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v)
    Ae[v] = reverse ? __shfl_down_sync(FULLMASK, A[v], 1) : __shfl_up_sync(FULLMASK, A[v], 1);
  if (reverse ? (lane == 31) : (lane == 0)) {
    Be = 1.0;
#pragma unroll
    for (int v = 0; v < NV; ++v) Ae[v] = 0.0;
  }
  double* tot = sc;
  double* pre = sc + 32 * (NV + 1);
  if (reverse ? (lane == 0) : (lane == 31)) {
    tot[warp * (NV + 1)] = B;
#pragma unroll
    for (int v = 0; v < NV; ++v) tot[warp * (NV + 1) + 1 + v] = A[v];
  }
  __syncthreads();
  if (t == 0) {
    double Bc = 1.0, Ac[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) Ac[v] = 0.0;
    for (int k = 0; k < nw; ++k) {
      const int w = reverse ? nw - 1 - k : k;
      pre[w * (NV + 1)] = Bc;
#pragma unroll
      for (int v = 0; v < NV; ++v) pre[w * (NV + 1) + 1 + v] = Ac[v];
      const double Bw = tot[w * (NV + 1)];
#pragma unroll
      for (int v = 0; v < NV; ++v) Ac[v] = tot[w * (NV + 1) + 1 + v] + Bw * Ac[v];
      Bc = Bw * Bc;
    }
  }
  __syncthreads();
  const double Bp = pre[warp * (NV + 1)];
#pragma unroll
  for (int v = 0; v < NV; ++v) A[v] = Ae[v] + Be * pre[warp * (NV + 1) + 1 + v];
  B = Be * Bp;
  __syncthreads();
}

// Solve the factored system in place for NV right-hand sides d0 (and d1) of length n.
template <int NV>
__device__ void tri_solve(int n, const double* __restrict__ fw, const double* __restrict__ fib,
                          const double* __restrict__ fg, double* d0, double* d1, double* sc) {
  const int T = blockDim.x, t = threadIdx.x;
  const int C = (n + T - 1) / T;
  const int k0 = min(t * C, n), k1 = min(k0 + C, n);
  double* d[2] = {d0, d1};
  double B = 1.0, A[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) A[v] = 0.0;
  for (int k = k0; k < k1; ++k) {                       // forward: y_k = d_k - w_k y_{k-1}
    const double beta = -fw[k];
#pragma unroll
    for (int v = 0; v < NV; ++v) A[v] = d[v][k] + beta * A[v];
    B = B * beta;
  }
  affine_scan<NV>(B, A, false, sc);
  for (int k = k0; k < k1; ++k) {
    const double wk = fw[k];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      A[v] = d[v][k] - wk * A[v];
      d[v][k] = A[v];
    }
  }
  __syncthreads();
  B = 1.0;
#pragma unroll
  for (int v = 0; v < NV; ++v) A[v] = 0.0;
  for (int k = k1 - 1; k >= k0; --k) {                  // backward: x_k = y_k ib_k - g_k x_{k+1}
    const double beta = -fg[k], ibk = fib[k];
#pragma unroll
    for (int v = 0; v < NV; ++v) A[v] = d[v][k] * ibk + beta * A[v];
    B = B * beta;
  }
  affine_scan<NV>(B, A, true, sc);
  for (int k = k1 - 1; k >= k0; --k) {
    const double ibk = fib[k], gk = fg[k];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      A[v] = d[v][k] * ibk - gk * A[v];
      d[v][k] = A[v];
    }
  }
  __syncthreads();
}

__device__ __forceinline__ void solve_mode(const GridDev& G, const double* fac, int kind, int m,
                                           double* d0, double* d1, double* sc) {
  const double* w = fac + fac_off(G.nr, G.M, kind, m);
  if (m == 0 && d1 == nullptr)
    tri_solve<1>(G.nr, w, w + G.nr, w + 2 * G.nr, d0, d0, sc);
  else
    tri_solve<2>(G.nr, w, w + G.nr, w + 2 * G.nr, d0, d1, sc);
}

// ------------------------------------------------------------------------------------
// Device: per-mode operations.  Shared-memory vectors are 1-based (index i = node i).
// Each op is executed by a whole CTA for one mode m and ends with __syncthreads().
// ------------------------------------------------------------------------------------
#define FLD(f, nc, p, c, i) (f)[fidx(G.ld, nc, p, c, i)]

// psi: field_psi_class.f03:131-254
__device__ void op_psi(const GridDev& G, int m, const double* fac, double* sm, double* sc,
                       const double* __restrict__ q, double* __restrict__ psi) {
  const int nr = G.nr, pr = part_re(m), pi = part_im(m);
  double* d0 = sm;
  double* d1 = sm + (nr + 2);
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    d0[i] = -1.0 * FLD(q, 1, pr, 0, i);
    if (m > 0) d1[i] = -1.0 * FLD(q, 1, pi, 0, i);
  }
  __syncthreads();
  solve_mode(G, fac, OK_GEN, m, d0 + 1, m > 0 ? d1 + 1 : nullptr, sc);
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    FLD(psi, 1, pr, 0, i) = (m > 0 && i == 1) ? 0.0 : d0[i];
    if (m > 0) FLD(psi, 1, pi, 0, i) = (i == 1) ? 0.0 : d1[i];
  }
  __syncthreads();
}

// Bz: field_b_class.f03:508-543, 760-796
__device__ void op_bz(const GridDev& G, int m, const double* fac, double* sm, double* sc,
                      const double* __restrict__ cu, double* __restrict__ b) {
  const int nr = G.nr, pr = part_re(m), pi = part_im(m);
  double* d0 = sm;
  double* d1 = sm + (nr + 2);
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    double re, im;
    row_bz_src(G, m, i, GlobalF{cu, G.ld, 3}, re, im);
    d0[i] = re;
    d1[i] = im;
  }
  __syncthreads();
  solve_mode(G, fac, OK_GEN, m, d0 + 1, m > 0 ? d1 + 1 : nullptr, sc);
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    FLD(b, 3, pr, 2, i) = (m > 0 && i == 1) ? 0.0 : d0[i];
    if (m > 0) FLD(b, 3, pi, 2, i) = (i == 1) ? 0.0 : d1[i];
  }
  __syncthreads();
}

// Beam B-perp: field_b_class.f03:309-358, 545-701, 798-834 (q read from q, which may be
// a slice of a 3D store with the same per-slice layout)
__device__ void op_bt_beam(const GridDev& G, int m, const double* fac, double* sm, double* sc,
                           const double* __restrict__ q, double* __restrict__ b) {
  const int nr = G.nr, pr = part_re(m), pi = part_im(m);
  const double idr = G.idr, idrh = 0.5 * idr, dm = (double)m;
  double* d0 = sm;
  double* d1 = sm + (nr + 2);
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    d0[i] = -1.0 * FLD(q, 1, pr, 0, i);
    if (m > 0) d1[i] = -1.0 * FLD(q, 1, pi, 0, i);
  }
  __syncthreads();
  solve_mode(G, fac, OK_BT, m, d0 + 1, m > 0 ? d1 + 1 : nullptr, sc);
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    if (m == 0) {
      double br = 0.0, bp;
      if (i == 1) bp = 0.0;
      else if (i == nr) bp = -idrh * (3.0 * d0[nr] - 4.0 * d0[nr - 1] + d0[nr - 2]);
      else bp = -idrh * (d0[i + 1] - d0[i - 1]);
      FLD(b, 3, 0, 0, i) = br;
      FLD(b, 3, 0, 1, i) = bp;
    } else {
      double rr, ri, pr_, pi_;
      if (i == 1) {
        if (m == 1) {
          rr = -idr * dm * d1[2];
          ri = idr * dm * d0[2];
          pr_ = -idr * d0[2];
          pi_ = -idr * d1[2];
        } else {
          rr = ri = pr_ = pi_ = 0.0;
        }
      } else if (i == nr) {
        const double ir = G.ir[nr];
        rr = -ir * dm * d1[nr];
        ri = ir * dm * d0[nr];
        pr_ = -idrh * (3.0 * d0[nr] - 4.0 * d0[nr - 1] + d0[nr - 2]);
        pi_ = -idrh * (3.0 * d1[nr] - 4.0 * d1[nr - 1] + d1[nr - 2]);
      } else {
        const double ir = G.ir[i];
        rr = -ir * dm * d1[i];
        ri = ir * dm * d0[i];
        pr_ = -idrh * (d0[i + 1] - d0[i - 1]);
        pi_ = -idrh * (d1[i + 1] - d1[i - 1]);
      }
      FLD(b, 3, pr, 0, i) = rr;
      FLD(b, 3, pi, 0, i) = ri;
      FLD(b, 3, pr, 1, i) = pr_;
      FLD(b, 3, pi, 1, i) = pi_;
    }
  }
  __syncthreads();
}

// Plasma B-perp predictor-corrector: field_b_class.f03:360-506, 703-758, 836-879.
// b holds B_old in components 1:2 on entry.
__device__ void op_bt_iter(const GridDev& G, int m, const double* fac, double* sm, double* sc,
                           const double* __restrict__ dcu, const double* __restrict__ cu, double* __restrict__ b) {
  const int nr = G.nr;
  double* b1re = sm;
  double* b1im = sm + (nr + 2);
  double* b2re = sm + 2 * (nr + 2);
  double* b2im = sm + 3 * (nr + 2);
  const GlobalF DC{dcu, G.ld, 2}, CU{cu, G.ld, 3}, BO{b, G.ld, 3};
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    double o[4];
    row_btiter_src(G, m, i, DC, CU, BO, o);
    if (m == 0) {
      b1re[i] = o[0];
      b2re[i] = o[1];
    } else {
      b1re[i] = o[0];
      b1im[i] = o[1];
      b2re[i] = o[2];
      b2im[i] = o[3];
    }
  }
  __syncthreads();
  if (m == 0) {
    const double* w = fac + fac_off(nr, G.M, OK_BPLUS, 0);
    tri_solve<1>(nr, w, w + nr, w + 2 * nr, b1re + 1, b1re + 1, sc);
    w = fac + fac_off(nr, G.M, OK_BMINUS, 0);
    tri_solve<1>(nr, w, w + nr, w + 2 * nr, b2re + 1, b2re + 1, sc);
    for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
      FLD(b, 3, 0, 0, i) = (i == 1) ? 0.0 : b1re[i];
      FLD(b, 3, 0, 1, i) = (i == 1) ? 0.0 : b2re[i];
    }
    __syncthreads();
    return;
  }
  const int pr = part_re(m), pi = part_im(m);
  const double* w = fac + fac_off(nr, G.M, OK_BPLUS, m);
  tri_solve<2>(nr, w, w + nr, w + 2 * nr, b1re + 1, b1im + 1, sc);
  w = fac + fac_off(nr, G.M, OK_BMINUS, m);
  tri_solve<2>(nr, w, w + nr, w + 2 * nr, b2re + 1, b2im + 1, sc);
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    const bool zero = (i == 1 && m != 1);
    FLD(b, 3, pr, 0, i) = zero ? 0.0 : 0.5 * (b1re[i] + b2re[i]);
    FLD(b, 3, pi, 0, i) = zero ? 0.0 : 0.5 * (b1im[i] + b2im[i]);
    FLD(b, 3, pr, 1, i) = zero ? 0.0 : 0.5 * (b1im[i] - b2im[i]);
    FLD(b, 3, pi, 1, i) = zero ? 0.0 : 0.5 * (-b1re[i] + b2re[i]);
  }
  __syncthreads();
}

// CTA-wide sum (all threads return the total)
__device__ double block_sum(double v, double* sc) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULLMASK, v, off);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) sc[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < nw; ++w) s += sc[w];
    sc[32] = s;
  }
  __syncthreads();
  s = sc[32];
  __syncthreads();
  return s;
}

// Ez: field_e_class.f03:148-259, 261-296, 298-334
__device__ void op_ez(const GridDev& G, int m, const double* fac, double* sm, double* sc,
                      const double* __restrict__ cu, double* __restrict__ e) {
  const int nr = G.nr, pr = part_re(m), pi = part_im(m);
  double* d0 = sm;
  double* d1 = sm + (nr + 2);
  const GlobalF CU{cu, G.ld, 3};
  double div = 0.0;
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    double re, im;
    bool in_div;
    row_ez_src(G, m, i, CU, re, im, in_div);
    if (in_div) div += re * (double)(i - 1);
    d0[i] = re;
    if (m > 0) d1[i] = im;
  }
  if (m == 0) {
    div = block_sum(div, sc);
    if (threadIdx.x == 0) d0[1] = ez_axis_row(G, div, CU);
  }
  __syncthreads();
  solve_mode(G, fac, OK_GEN, m, d0 + 1, m > 0 ? d1 + 1 : nullptr, sc);
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) {
    FLD(e, 3, pr, 2, i) = (m > 0 && i == 1) ? 0.0 : d0[i];
    if (m > 0) FLD(e, 3, pi, 2, i) = (i == 1) ? 0.0 : d1[i];
  }
  __syncthreads();
}

// E-perp from B and psi: field_e_class.f03:412-514 (no solve)
__device__ void op_et(const GridDev& G, int m, const double* __restrict__ b, const double* __restrict__ psi,
                      double* __restrict__ e) {
  const GlobalF B{b, G.ld, 3}, PS{psi, G.ld, 1};
  const int pr = part_re(m), pi = part_im(m);
  for (int i = 1 + threadIdx.x; i <= G.nr; i += blockDim.x) {
    double o[4];
    row_et(G, m, i, B, PS, o);
    if (m == 0) {
      FLD(e, 3, 0, 0, i) = o[0];
      FLD(e, 3, 0, 1, i) = o[1];
    } else {
      FLD(e, 3, pr, 0, i) = o[0];
      FLD(e, 3, pi, 0, i) = o[1];
      FLD(e, 3, pr, 1, i) = o[2];
      FLD(e, 3, pi, 1, i) = o[3];
    }
  }
  __syncthreads();
}

// dJ_perp/dxi: field_src_class.f03:273-405 (no solve)
__device__ void op_djdxi(const GridDev& G, int m, const double* __restrict__ acu, const double* __restrict__ amu,
                         double* __restrict__ dcu) {
  const GlobalF A{acu, G.ld, 2}, U{amu, G.ld, 3};
  const int pr = part_re(m), pi = part_im(m);
  for (int i = 1 + threadIdx.x; i <= G.nr; i += blockDim.x) {
    double o[4];
    row_djdxi(G, m, i, A, U, o);
    FLD(dcu, 2, pr, 0, i) = o[0];
    FLD(dcu, 2, pr, 1, i) = o[1];
    if (m > 0) {
      FLD(dcu, 2, pi, 0, i) = o[2];
      FLD(dcu, 2, pi, 1, i) = o[3];
    }
  }
  __syncthreads();
}

// Raw charge deposit -> density (part2d_class.f03:314-335): axis guard 0, axis x8 for
// m=0 and 0 for m>0, 1/(j-1) beyond.  out = raw finished (+ qn when add_qn, which is the
// species2d::qdp accumulation q_spe = 0 + q_species + qn).
// smooth > 0: the finished charge takes that many binomial smoothing passes before qn is
// added (qdp_species2d, species2d_class.f03:198-203); sm holds 4 (nr + 2) doubles.
__device__ void op_finish_q(const GridDev& G, int m, const double* __restrict__ raw, const double* __restrict__ qn,
                            double* __restrict__ out, int smooth, double* sm) {
  const int np_ = m == 0 ? 1 : 2;
  if (smooth > 0) {
    const int ld = G.ld;
    for (int h = 0; h < np_; ++h) {
      const int p = h == 0 ? part_re(m) : part_im(m);
      for (int i = threadIdx.x; i <= G.nr + 1; i += blockDim.x) {
        const double r = FLD(raw, 1, p, 0, i);
        sm[h * ld + i] = i == 0 ? 0.0 : (i == 1 ? ((m == 0) ? 8.0 * r : 0.0) : r * G.inv[i]);
      }
    }
    __syncthreads();
    for (int pass = 0; pass < smooth; ++pass) {
      for (int h = 0; h < np_; ++h)
        for (int i = 1 + threadIdx.x; i <= G.nr; i += blockDim.x) {
          const double* v = sm + h * ld;
          sm[(2 + h) * ld + i] = smooth_node(G, i, smooth_ax(0, m, 0), v[i - 1], v[i], v[i + 1]);
        }
      __syncthreads();
      for (int h = 0; h < np_; ++h)
        for (int i = 1 + threadIdx.x; i <= G.nr; i += blockDim.x) sm[h * ld + i] = sm[(2 + h) * ld + i];
      __syncthreads();
    }
    for (int h = 0; h < np_; ++h) {
      const int p = h == 0 ? part_re(m) : part_im(m);
      for (int i = threadIdx.x; i <= G.nr + 1; i += blockDim.x) {
        double v = sm[h * ld + i];
        if (qn) v = (0.0 + v) + FLD(qn, 1, p, 0, i);
        FLD(out, 1, p, 0, i) = v;
      }
    }
    __syncthreads();
    return;
  }
  for (int h = 0; h < np_; ++h) {
    const int p = h == 0 ? part_re(m) : part_im(m);
    for (int i = threadIdx.x; i <= G.nr + 1; i += blockDim.x) {
      const double r = FLD(raw, 1, p, 0, i);
      double v;
      if (i == 0) v = 0.0;
      else if (i == 1) v = (m == 0) ? 8.0 * r : 0.0;
      else v = r * G.inv[i];
      if (qn) v = (0.0 + v) + FLD(qn, 1, p, 0, i);
      FLD(out, 1, p, 0, i) = v;
    }
  }
  __syncthreads();
}

// Axis fixes and 1/(j-1) scaling of the current, momentum-flux and acceleration deposits,
// in place (part2d_class.f03:914-1005).
// smooth > 0: then that many binomial smoothing passes of each of them
// (amjdp_species2d, species2d_class.f03:270-272); sm holds 4 (nr + 2) doubles.
__device__ void op_finish_amj(const GridDev& G, int m, double* __restrict__ cu, double* __restrict__ amu,
                              double* __restrict__ acu, int smooth, double* sm) {
  const int np_ = m == 0 ? 1 : 2;
  for (int h = 0; h < np_; ++h) {
    const int p = h == 0 ? part_re(m) : part_im(m);
    for (int i = threadIdx.x; i <= G.nr + 1; i += blockDim.x) {
      for (int c = 0; c < 3; ++c) {
        FLD(cu, 3, p, c, i) = finish_amj(G, m, 0, c, i, FLD(cu, 3, p, c, i));
        FLD(amu, 3, p, c, i) = finish_amj(G, m, 1, c, i, FLD(amu, 3, p, c, i));
      }
      for (int c = 0; c < 2; ++c) FLD(acu, 2, p, c, i) = finish_amj(G, m, 2, c, i, FLD(acu, 2, p, c, i));
    }
  }
  __syncthreads();
  if (smooth <= 0) return;
  const int ld = G.ld;
  for (int h = 0; h < np_; ++h) {
    const int p = h == 0 ? part_re(m) : part_im(m);
    for (int row = 0; row < 8; ++row) {              // cu 0..2, amu 0..2, acu 0..1
      double* f = row < 3 ? &FLD(cu, 3, p, row, 0) : (row < 6 ? &FLD(amu, 3, p, row - 3, 0) : &FLD(acu, 2, p, row - 6, 0));
      const int kind = row < 6 ? 1 : 2, comp = row < 3 ? row : (row < 6 ? row - 3 : row - 6);
      for (int i = threadIdx.x; i <= G.nr + 1; i += blockDim.x) sm[i] = f[i];
      __syncthreads();
      for (int pass = 0; pass < smooth; ++pass) {
        for (int i = 1 + threadIdx.x; i <= G.nr; i += blockDim.x)
          sm[ld + i] = smooth_node(G, i, smooth_ax(kind, m, comp), sm[i - 1], sm[i], sm[i + 1]);
        __syncthreads();
        for (int i = 1 + threadIdx.x; i <= G.nr; i += blockDim.x) sm[i] = sm[ld + i];
        __syncthreads();
      }
      for (int i = 1 + threadIdx.x; i <= G.nr; i += blockDim.x) f[i] = sm[i];
      __syncthreads();
    }
  }
}

// FP32 gather table of the mixed-precision particle path: T[(node*P + part)*6 + c],
// c = 0..2 the E components, 3..5 the B components, nodes 0..nr+1.
__device__ void op_write_gtab(const GridDev& G, int m, const double* __restrict__ e, const double* __restrict__ b,
                              float* __restrict__ T) {
  const int np_ = m == 0 ? 1 : 2;
  for (int h = 0; h < np_; ++h) {
    const int p = h == 0 ? part_re(m) : part_im(m);
    for (int k = threadIdx.x; k < 6 * G.ld; k += blockDim.x) {
      const int i = k / 6, c = k % 6;
      const double v = c < 3 ? FLD(e, 3, p, c, i) : FLD(b, 3, p, c - 3, i);
      T[((size_t)i * G.P + p) * 6 + c] = (float)v;
    }
  }
  __syncthreads();
}

// c = a + b over all components and nodes of mode m (add_f1_binary)
__device__ void op_add(const GridDev& G, int m, int nc, const double* a, const double* b, double* c) {
  const int np_ = m == 0 ? 1 : 2;
  for (int h = 0; h < np_; ++h) {
    const int p = h == 0 ? part_re(m) : part_im(m);
    for (int k = threadIdx.x; k < nc * G.ld; k += blockDim.x) {
      const size_t o = (size_t)p * nc * G.ld + k;
      c[o] = a[o] + b[o];
    }
  }
  __syncthreads();
}

__device__ void op_fill(const GridDev& G, int m, int nc, double* a, double v) {
  const int np_ = m == 0 ? 1 : 2;
  for (int h = 0; h < np_; ++h) {
    const int p = h == 0 ? part_re(m) : part_im(m);
    for (int k = threadIdx.x; k < nc * G.ld; k += blockDim.x) a[(size_t)p * nc * G.ld + k] = v;
  }
  __syncthreads();
}

__device__ void op_copy(const GridDev& G, int m, int nc, const double* a, double* b) {
  const int np_ = m == 0 ? 1 : 2;
  for (int h = 0; h < np_; ++h) {
    const int p = h == 0 ? part_re(m) : part_im(m);
    for (int k = threadIdx.x; k < nc * G.ld; k += blockDim.x) {
      const size_t o = (size_t)p * nc * G.ld + k;
      b[o] = a[o];
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------------------------
// Kernels
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kFieldThreads) k_field_op(GridDev G, int op, const double* __restrict__ fac,
                                                            FieldArgs a) {
  extern __shared__ double sm[];
  __shared__ double sc[6 * 32 + 8];
  const int m = blockIdx.x;
  switch (op) {
    case FOP_PSI: op_psi(G, m, fac, sm, sc, a.in0, a.out); break;
    case FOP_BZ: op_bz(G, m, fac, sm, sc, a.in0, a.out); break;
    case FOP_BT_BEAM: op_bt_beam(G, m, fac, sm, sc, a.in0, a.out); break;
    case FOP_BT_ITER: op_bt_iter(G, m, fac, sm, sc, a.in0, a.in1, a.out); break;
    case FOP_EZ: op_ez(G, m, fac, sm, sc, a.in0, a.out); break;
    case FOP_ET: op_et(G, m, a.in0, a.in1, a.out); break;
    case FOP_DJDXI: op_djdxi(G, m, a.in0, a.in1, a.out); break;
  }
}

struct SliceFields {
  double* f[QPAD_NFIELDS];
  double* f2[QPAD_NFIELDS];
  const double* qraw;
  const double* qn;
  float* gtab;   // FP32 gather table, written when the mixed path is active
};

static SliceFields slice_fields(qpad_ctx* ctx) {
  SliceFields s;
  for (int k = 0; k < QPAD_NFIELDS; ++k) { s.f[k] = ctx->f[k]; s.f2[k] = ctx->f2[k]; }
  s.qraw = ctx->qraw;
  s.qn = ctx->qbg ? ctx->qbg : ctx->qn;          // with a neutral gas: qn + its ions
  s.gtab = ctx->precision == QPAD_PREC_MIXED ? ctx->gtab : nullptr;
  return s;
}

__global__ void __launch_bounds__(kFieldThreads) k_gtab(GridDev G, const double* e, const double* b, float* T) {
  op_write_gtab(G, blockIdx.x, e, b, T);
}

int launch_gtab(qpad_ctx* ctx, const double* e, const double* b) {
  k_gtab<<<ctx->g.M + 1, kFieldThreads, 0, ctx->stream>>>(ctx->g, e, b, ctx->gtab);
  return check_launch(ctx, "k_gtab");
}

__device__ __forceinline__ double* store_slice(const GridDev& G, double* f2, int nc, int j) {
  return f2 + (size_t)(j - 1) * G.P * nc * G.ld;
}

// Start of slice j (simulation_class.f03:344-360): beam B-perp from the stored beam
// charge; species charge (+ background) and psi; Bz from the carried current; and the Ez
// of the first iteration (:375-378), which also depends only on the carried current.
// One CTA per (job, mode).
__global__ void __launch_bounds__(kFieldThreads) k_slice_begin(GridDev G, const double* __restrict__ fac,
                                                               SliceFields F, const int* __restrict__ jp,
                                                               int use_qn) {
  extern __shared__ double sm[];
  __shared__ double sc[6 * 32 + 8];
  const int j = *jp;
  const int job = blockIdx.x / (G.M + 1), m = blockIdx.x % (G.M + 1);
  if (job == 0) {
    const double* qs = store_slice(G, F.f2[QPAD_F_Q_BEAM], 1, j);
    op_copy(G, m, 1, qs, F.f[QPAD_F_Q_BEAM]);                      // q_beam%copy_slice(j, 2->1)
    op_bt_beam(G, m, fac, sm, sc, F.f[QPAD_F_Q_BEAM], F.f[QPAD_F_B_BEAM]);
  } else if (job == 1) {
    op_finish_q(G, m, F.qraw, use_qn ? F.qn : nullptr, F.f[QPAD_F_Q_SPE], G.smooth, sm);
    op_psi(G, m, fac, sm, sc, F.f[QPAD_F_Q_SPE], F.f[QPAD_F_PSI]);
  } else if (job == 2) {
    op_bz(G, m, fac, sm, sc, F.f[QPAD_F_CU], F.f[QPAD_F_B_SPE]);
  } else {
    op_ez(G, m, fac, sm, sc, F.f[QPAD_F_CU], F.f[QPAD_F_E]);
  }
}

// Rest of the first iteration's phase 1 (simulation_class.f03:375-380), one thread per
// (mode, node): b = b_spe + b_beam, E-perp(b, psi), the FP32 gather table; then
// cu = acu = amu = 0 for the deposit that follows.  Ez came from k_slice_begin.
__global__ void __launch_bounds__(256) k_iter_e(GridDev G, SliceFields F) {
  const int ld = G.ld;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (G.M + 1) * ld) return;
  const int m = q / ld, i = q % ld;
  const int nh = m == 0 ? 1 : 2;
  const int pr = part_re(m), pi = part_im(m);
  const double* bs = F.f[QPAD_F_B_SPE];
  const double* bb = F.f[QPAD_F_B_BEAM];
  double* b = F.f[QPAD_F_B];
  double* e = F.f[QPAD_F_E];
  double bv[2][3];
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int p = h == 0 ? pr : pi;
      bv[h][c] = h < nh ? FLD(bs, 3, p, c, i) + FLD(bb, 3, p, c, i) : 0.0;
    }
  double ev[2][3];
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int c = 0; c < 3; ++c) ev[h][c] = h < nh ? FLD(e, 3, h == 0 ? pr : pi, c, i) : 0.0;
  if (i >= 1 && i <= G.nr) {
    const auto B = [&](int p, int c, int) { return p == pr ? bv[0][c] : bv[1][c]; };
    double o[4];
    row_et(G, m, i, B, GlobalF{F.f[QPAD_F_PSI], ld, 1}, o);
    if (m == 0) {
      ev[0][0] = o[0];
      ev[0][1] = o[1];
    } else {
      ev[0][0] = o[0];
      ev[1][0] = o[1];
      ev[0][1] = o[2];
      ev[1][1] = o[3];
    }
  }
  for (int h = 0; h < nh; ++h) {
    const int p = h == 0 ? pr : pi;
    for (int c = 0; c < 3; ++c) FLD(b, 3, p, c, i) = bv[h][c];
    if (i >= 1 && i <= G.nr)
      for (int c = 0; c < 2; ++c) FLD(e, 3, p, c, i) = ev[h][c];
    if (F.gtab) {
      float* T = F.gtab + ((size_t)i * G.P + p) * 6;
      for (int c = 0; c < 3; ++c) {
        T[c] = (float)ev[h][c];
        T[3 + c] = (float)bv[h][c];
      }
    }
    for (int c = 0; c < 3; ++c) {
      FLD(F.f[QPAD_F_CU], 3, p, c, i) = 0.0;
      FLD(F.f[QPAD_F_AMU], 3, p, c, i) = 0.0;
    }
    for (int c = 0; c < 2; ++c) FLD(F.f[QPAD_F_ACU], 2, p, c, i) = 0.0;
  }
}

// Iteration phase 2 (simulation_class.f03:386-392): finish the deposits, dJ/dxi, B-perp
// predictor-corrector solve and Bz.
__global__ void __launch_bounds__(kFieldThreads) k_iter_b(GridDev G, const double* __restrict__ fac, SliceFields F) {
  extern __shared__ double sm[];
  __shared__ double sc[6 * 32 + 8];
  const int m = blockIdx.x;
  op_finish_amj(G, m, F.f[QPAD_F_CU], F.f[QPAD_F_AMU], F.f[QPAD_F_ACU], G.smooth, sm);
  op_djdxi(G, m, F.f[QPAD_F_ACU], F.f[QPAD_F_AMU], F.f[QPAD_F_DCU]);
  op_bt_iter(G, m, fac, sm, sc, F.f[QPAD_F_DCU], F.f[QPAD_F_CU], F.f[QPAD_F_B_SPE]);
  op_bz(G, m, fac, sm, sc, F.f[QPAD_F_CU], F.f[QPAD_F_B_SPE]);
}

// End of slice j (simulation_class.f03:403-456 without the particle push), one thread per
// (mode part, node): cbq (rho = (rho - Jz) + Jz), the stores of cu, rho, E, B, psi, b_spe
// and e_spe = E-perp(b_spe, psi), then the J-perp predictor dcu *= dxi, cu += dcu.  E and B
// of the slice, b = b_spe + b_beam and the FP32 gather table are those the last
// predictor-corrector iteration (k_iterate) left: the reference's e%solve(cu) and
// e%solve(b, psi) at the slice end see the same inputs.
__global__ void __launch_bounds__(256) k_slice_end(GridDev G, SliceFields F, const int* __restrict__ jp) {
  const int j = *jp;
  const int ld = G.ld;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= G.P * ld) return;
  const int p = q / ld, i = q % ld;
  const int m = (p + 1) / 2;
  double* cu = F.f[QPAD_F_CU];
  double* qs = F.f[QPAD_F_Q_SPE];
  const size_t s1 = (size_t)(j - 1) * G.P;      // slice block of the 3D stores
  // q_spe(1,:) += cu(3,:), then the stores of cu and q_spe
  const double qv = FLD(qs, 1, p, 0, i) + FLD(cu, 3, p, 2, i);
  FLD(qs, 1, p, 0, i) = qv;
  F.f2[QPAD_F_Q_SPE][(s1 + p) * ld + i] = qv;
  for (int c = 0; c < 3; ++c) {
    F.f2[QPAD_F_CU][((s1 + p) * 3 + c) * ld + i] = FLD(cu, 3, p, c, i);
    F.f2[QPAD_F_E][((s1 + p) * 3 + c) * ld + i] = FLD(F.f[QPAD_F_E], 3, p, c, i);
    F.f2[QPAD_F_B][((s1 + p) * 3 + c) * ld + i] = FLD(F.f[QPAD_F_B], 3, p, c, i);
    F.f2[QPAD_F_B_SPE][((s1 + p) * 3 + c) * ld + i] = FLD(F.f[QPAD_F_B_SPE], 3, p, c, i);
  }
  F.f2[QPAD_F_PSI][(s1 + p) * ld + i] = FLD(F.f[QPAD_F_PSI], 1, p, 0, i);
  // e_spe = E-perp(b_spe, psi) on nodes 1..nr (field_e_class.f03:412-514)
  double* es = F.f[QPAD_F_E_SPE];
  if (i >= 1 && i <= G.nr && (m == 0 || p == part_re(m))) {
    double o[4];
    row_et(G, m, i, GlobalF{F.f[QPAD_F_B_SPE], ld, 3}, GlobalF{F.f[QPAD_F_PSI], ld, 1}, o);
    if (m == 0) {
      FLD(es, 3, 0, 0, i) = o[0];
      FLD(es, 3, 0, 1, i) = o[1];
    } else {
      FLD(es, 3, part_re(m), 0, i) = o[0];
      FLD(es, 3, part_im(m), 0, i) = o[1];
      FLD(es, 3, part_re(m), 1, i) = o[2];
      FLD(es, 3, part_im(m), 1, i) = o[3];
    }
  }
  // dcu *= dxi ; cu(1:2) += dcu(1:2)   (simulation_class.f03:425-426)
  double* dcu = F.f[QPAD_F_DCU];
  for (int c = 0; c < 2; ++c) {
    const double d = FLD(dcu, 2, p, c, i) * G.dxi;
    FLD(dcu, 2, p, c, i) = d;
    FLD(cu, 3, p, c, i) = FLD(cu, 3, p, c, i) + d;
  }
}

// e_spe of the slice into its store; needs every part of e_spe, so it follows k_slice_end
__global__ void __launch_bounds__(256) k_store_espe(GridDev G, SliceFields F, const int* __restrict__ jp) {
  const int j = *jp;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= G.P * 3 * G.ld) return;
  F.f2[QPAD_F_E_SPE][(size_t)(j - 1) * G.P * 3 * G.ld + q] = F.f[QPAD_F_E_SPE][q];
}

__global__ void __launch_bounds__(kFieldThreads) k_finish_q(GridDev G, const double* raw, const double* qn,
                                                            double* out, int smooth) {
  extern __shared__ double sm[];
  op_finish_q(G, blockIdx.x, raw, qn, out, smooth, sm);
}

__global__ void __launch_bounds__(kFieldThreads) k_finish_amj(GridDev G, double* cu, double* amu, double* acu) {
  extern __shared__ double sm[];
  op_finish_amj(G, blockIdx.x, cu, amu, acu, G.smooth, sm);
}

// convergence_tester (simulation_class.f03:522-606) on component `comp` of b:
// op 0 records s_re/s_im; op 1 compares against the record, writes rel/abs/converged
// into res and records the new sums for the next iteration.  With a loop state, op 1 also
// counts the iteration, stores the slice's statistics and, inside a CUDA graph, sets the
// condition of the predictor-corrector WHILE node (continue while not converged and
// below iter_max, simulation_class.f03:370-398).
__global__ void __launch_bounds__(1024) k_conv(GridDev G, const double* __restrict__ b, int comp, int op,
                                               double* __restrict__ st, double reltol, double abstol, ConvLoop L) {
  __shared__ double red[33];
  __shared__ double red2[33];
  const int nr = G.nr;
  double* s_re = st;
  double* s_im = st + nr;
  double* res = st + 2 * nr;
  const GlobalF B{b, G.ld, 3};
  double mx_old = 0.0, mx_new = 0.0;
  for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) conv_node(G, B, comp, i, s_re, s_im, op == 1, mx_old, mx_new);
  if (op == 0) {
    // 'record' opens the iteration loop of a new slice: re-arm its WHILE condition (a
    // nested conditional keeps its last value between entries within one graph launch)
    if (L.use_h && threadIdx.x == 0) cudaGraphSetConditional(L.h, 1u);
    return;
  }
  // max-reductions (order independent, exact)
  for (int off = 16; off > 0; off >>= 1) {
    mx_old = fmax(mx_old, __shfl_down_sync(FULLMASK, mx_old, off));
    mx_new = fmax(mx_new, __shfl_down_sync(FULLMASK, mx_new, off));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { red[warp] = mx_old; red2[warp] = mx_new; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, c = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a = fmax(a, red[w]); c = fmax(c, red2[w]); }
    conv_decide(a, c, reltol, abstol, res, L);
  }
}

// Advances the slice counter and sets the condition of the slice WHILE node.
__global__ void k_advance(int* __restrict__ jp, int nz, cudaGraphConditionalHandle hs, cudaGraphConditionalHandle hi) {
  const int j = *jp + 1;
  *jp = j;
  cudaGraphSetConditional(hs, j <= nz ? 1u : 0u);
  // re-arm the iteration WHILE node for the next slice (a nested conditional keeps its
  // last value between entries within one graph launch)
  cudaGraphSetConditional(hi, 1u);
}

// ------------------------------------------------------------------------------------
// Host launchers
// ------------------------------------------------------------------------------------
static size_t field_smem(const qpad_ctx* ctx) { return (size_t)4 * (ctx->g.nr + 2) * sizeof(double); }

// The dynamic shared-memory limit is an attribute of the kernel (per device), shared by
// every context in the process: it is only ever raised, so that a context with a shorter
// radial line never lowers the limit another context's launches rely on.
int raise_dyn_smem(qpad_ctx* ctx, const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> cur;
  std::lock_guard<std::mutex> lock(mu);
  size_t& have = cur[{func, ctx->device}];
  if (bytes <= have) return 0;
  cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return cuda_check(ctx, e, "cudaFuncSetAttribute(smem)");
  have = bytes;
  return 0;
}

static int ensure_smem_attr(qpad_ctx* ctx) {
  if (ctx->field_attr_done) return 0;
  const size_t need = field_smem(ctx);
  const void* ks[] = {(const void*)k_field_op, (const void*)k_slice_begin, (const void*)k_iter_b,
                      (const void*)k_finish_q, (const void*)k_finish_amj};
  for (const void* k : ks)
    if (int r = raise_dyn_smem(ctx, k, need)) return r;
  ctx->field_attr_done = true;
  return 0;
}

int launch_field_op(qpad_ctx* ctx, int op, FieldArgs a) {
  if (int r = ensure_smem_attr(ctx)) return r;
  k_field_op<<<ctx->g.M + 1, kFieldThreads, field_smem(ctx), ctx->stream>>>(ctx->g, op, ctx->fac, a);
  return check_launch(ctx, "k_field_op");
}

int launch_conv(qpad_ctx* ctx, const double* b, int comp, int op, int loop_state, cudaGraphConditionalHandle h,
                int use_h) {
  ConvLoop L{};
  if (loop_state) {
    L.iter_ctr = ctx->d_iter;
    L.stats = ctx->d_stats;
    L.jp = ctx->d_j;
    L.iter_max = ctx->iter_max;
    L.h = h;
    L.use_h = use_h;
  }
  prof_begin(ctx, "conv");
  k_conv<<<1, 1024, 0, ctx->stream>>>(ctx->g, b, comp, op, ctx->conv, ctx->reltol, ctx->abstol, L);
  prof_end(ctx, "conv");
  return check_launch(ctx, "k_conv");
}

__global__ void k_set_slice(int* __restrict__ jp, int j) { *jp = j; }

int launch_set_slice(qpad_ctx* ctx, int j) {
  k_set_slice<<<1, 1, 0, ctx->stream>>>(ctx->d_j, j);
  return check_launch(ctx, "k_set_slice");
}

int launch_advance(qpad_ctx* ctx, cudaGraphConditionalHandle hs, cudaGraphConditionalHandle hi) {
  k_advance<<<1, 1, 0, ctx->stream>>>(ctx->d_j, ctx->g.nz, hs, hi);
  return check_launch(ctx, "k_advance");
}

int launch_slice_begin(qpad_ctx* ctx, int use_qn) {
  if (int r = ensure_smem_attr(ctx)) return r;
  prof_begin(ctx, "slice_begin");
  k_slice_begin<<<4 * (ctx->g.M + 1), kFieldThreads, field_smem(ctx), ctx->stream>>>(ctx->g, ctx->fac,
                                                                                     slice_fields(ctx), ctx->d_j, use_qn);
  prof_end(ctx, "slice_begin");
  return check_launch(ctx, "k_slice_begin");
}

int launch_iter_e(qpad_ctx* ctx) {
  const int n = (ctx->g.M + 1) * ctx->g.ld;
  prof_begin(ctx, "iter_e");
  k_iter_e<<<(n + 255) / 256, 256, 0, ctx->stream>>>(ctx->g, slice_fields(ctx));
  prof_end(ctx, "iter_e");
  return check_launch(ctx, "k_iter_e");
}

int launch_iter_b(qpad_ctx* ctx) {
  if (int r = ensure_smem_attr(ctx)) return r;
  k_iter_b<<<ctx->g.M + 1, kFieldThreads, field_smem(ctx), ctx->stream>>>(ctx->g, ctx->fac, slice_fields(ctx));
  return check_launch(ctx, "k_iter_b");
}

int launch_slice_end(qpad_ctx* ctx) {
  const int n = ctx->g.P * ctx->g.ld;
  prof_begin(ctx, "slice_end");
  k_slice_end<<<(n + 255) / 256, 256, 0, ctx->stream>>>(ctx->g, slice_fields(ctx), ctx->d_j);
  k_store_espe<<<(3 * n + 255) / 256, 256, 0, ctx->stream>>>(ctx->g, slice_fields(ctx), ctx->d_j);
  prof_end(ctx, "slice_end");
  return check_launch(ctx, "k_slice_end", 2);
}

int launch_finish_q(qpad_ctx* ctx, const double* raw, double* out, int add_qn, int smooth) {
  if (int r = ensure_smem_attr(ctx)) return r;
  k_finish_q<<<ctx->g.M + 1, kFieldThreads, smooth > 0 ? field_smem(ctx) : 0, ctx->stream>>>(
      ctx->g, raw, add_qn ? ctx->qn : nullptr, out, smooth);
  return check_launch(ctx, "k_finish_q");
}

int launch_finish_amj(qpad_ctx* ctx, double* cu, double* amu, double* acu) {
  if (int r = ensure_smem_attr(ctx)) return r;
  k_finish_amj<<<ctx->g.M + 1, kFieldThreads, ctx->g.smooth > 0 ? field_smem(ctx) : 0, ctx->stream>>>(ctx->g, cu, amu,
                                                                                                      acu);
  return check_launch(ctx, "k_finish_amj");
}

}  // namespace qpad
