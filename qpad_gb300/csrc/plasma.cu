// plasma.cu -- plasma particle kernels of the slice loop (FP64 reference arithmetic).
//
//   k_qdeposit   part2d::qdeposit          (part2d_class.f03:231-359)
//   k_amjdp      part2d::amjdeposit_robust / _std (part2d_class.f03:746-1010, 478-744)
//   k_push       part2d::push_u_robust / _std + push_x + the edge test of update_bound
//                (part2d_class.f03:1879-1965, 1790-1877, 2221-2262, 2307-2353)
//   compaction   update_bound's removal (order-preserving, count bit-exact)
//   sort         part2d::sort + generate_sort_idx_1d (part2d_class.f03:2498-2579,
//                sort_module.f03:10-41), reproducing the reference permutation
//   k_interp_psi part2d::interp_psi        (part2d_class.f03:2264-2305)
//
// One thread per particle; the particle count is read from device memory so that a
// whole slice can be enqueued without a host round trip (compaction only shrinks it).
// Deposits go straight to the FP64 mode arrays with atomicAdd; the axis corrections and
// the 1/(j-1) scaling are applied afterwards by the field kernels.
#include <algorithm>

#include "particles.cuh"

namespace qpad {

static constexpr int kPartThreads = 256;

static int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > (1 << 30)) b = 1 << 30;
  return (int)b;
}

__global__ void __launch_bounds__(kPartThreads) k_qdeposit(GridDev G, const int64_t* __restrict__ n_ptr,
                                                           const double* __restrict__ x, const double* __restrict__ y,
                                                           const double* __restrict__ q, double* __restrict__ qraw) {
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const double xx = x[pp], yy = y[pp];
  double pos = __dmul_rn(radius_rn(xx, yy), G.idr);
  const double ph0r = xx / pos * G.idr, ph0i = -yy / pos * G.idr;
  if (!(pos >= 0.0 && pos < (double)G.nr)) return;
  const int nn0 = (int)floor(pos);
  pos = __dsub_rn(pos, (double)nn0);
  const int nn = nn0 + 1;
  const double wt0 = 1.0 - pos, wt1 = pos;
  double phr = 1.0 * q[pp], phi = 0.0;
  const size_t ld = G.ld;
  atomicAdd(qraw + nn, wt0 * phr);
  atomicAdd(qraw + nn + 1, wt1 * phr);
  for (int m = 1; m <= G.M; ++m) {
    const double t = phr * ph0r - phi * ph0i;
    phi = phr * ph0i + phi * ph0r;
    phr = t;
    double* qr = qraw + (size_t)(2 * m - 1) * ld;
    double* qi = qraw + (size_t)(2 * m) * ld;
    atomicAdd(qr + nn, wt0 * phr);
    atomicAdd(qi + nn, wt0 * phi);
    atomicAdd(qr + nn + 1, wt1 * phr);
    atomicAdd(qi + nn + 1, wt1 * phi);
  }
}

__global__ void __launch_bounds__(kPartThreads) k_amjdp(GridDev G, int push_type, double qbm, double dt,
                                                        const int64_t* __restrict__ n_ptr,
                                                        const double* __restrict__ x, const double* __restrict__ y,
                                                        const double* __restrict__ px, const double* __restrict__ py,
                                                        const double* __restrict__ pz, const double* __restrict__ q,
                                                        double* __restrict__ gamma, double* __restrict__ psi,
                                                        const double* __restrict__ ef, const double* __restrict__ bf,
                                                        double* __restrict__ cu, double* __restrict__ amu,
                                                        double* __restrict__ acu, const int* __restrict__ guard) {
  if (guard && *guard) return;                 // a part of an unrolled loop body after the loop ended
  // the field iteration launched after this kernel may start its own staging now
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const double idt = 1.0 / dt, qtmh = 0.5 * qbm * dt;
  const Interp ii = gen_interp(x[pp], y[pp], G.idr, G.nr);
  double ep[3], bp[3], wp[3], u0[3], u[3], ut[3];
  gather3(G, ef, ii, ep);
  gather3(G, bf, ii, bp);
  wp[0] = ep[0] - bp[1];
  wp[1] = ep[1] + bp[0];
  wp[2] = ep[2];
  const double p1 = px[pp], p2 = py[pp];
  u0[0] = p1 * ii.pcos + p2 * ii.psin;
  u0[1] = p2 * ii.pcos - p1 * ii.psin;
  u0[2] = pz[pp];
  const double psi_in = psi[pp];
  if (push_type == QPAD_PUSH2_ROBUST) {
    double gam = sqrt(1.0 + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]);
    const double qtmh1 = qtmh * gam / (gam - u0[2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh1; ut[c] = u0[c] + ep[c]; }
    gam = sqrt(1.0 + ut[0] * ut[0] + ut[1] * ut[1] + ut[2] * ut[2]);
    const double qtmh2 = qtmh / (gam - ut[2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) bp[c] = bp[c] * qtmh2;
  } else {
    const double gam = sqrt(1.0 + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]);
    const double qtmh2 = qtmh / (1.0 - qbm * psi_in);
    const double qtmh1 = qtmh2 * gam;
#pragma unroll
    for (int c = 0; c < 3; ++c) { bp[c] = bp[c] * qtmh2; ut[c] = u0[c] + ep[c] * qtmh1; }
  }
  u[0] = ut[0] + ut[1] * bp[2] - ut[2] * bp[1];
  u[1] = ut[1] + ut[2] * bp[0] - ut[0] * bp[2];
  u[2] = ut[2] + ut[0] * bp[1] - ut[1] * bp[0];
  const double ostq = 2.0 / (1.0 + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c) bp[c] = bp[c] * ostq;
  {
    const double t0 = ut[0] + u[1] * bp[2] - u[2] * bp[1];
    const double t1 = ut[1] + u[2] * bp[0] - u[0] * bp[2];
    const double t2 = ut[2] + u[0] * bp[1] - u[1] * bp[0];
    ut[0] = t0; ut[1] = t1; ut[2] = t2;
  }
  if (push_type == QPAD_PUSH2_ROBUST) {
#pragma unroll
    for (int c = 0; c < 3; ++c) u[c] = ut[c] + ep[c];
  } else {
    const double gam = sqrt(1.0 + ut[0] * ut[0] + ut[1] * ut[1] + ut[2] * ut[2]);
    const double qtmh1 = qtmh / (1.0 - qbm * psi_in) * gam;
#pragma unroll
    for (int c = 0; c < 3; ++c) u[c] = ut[c] + ep[c] * qtmh1;
  }
  // time-centred values and deposit
  double du0 = idt * (u[0] - u0[0]);
  double du1 = idt * (u[1] - u0[1]);
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = 0.5 * (u[c] + u0[c]);
  const double g = sqrt(1.0 + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  gamma[pp] = g;
  double ipsi;
  if (push_type == QPAD_PUSH2_ROBUST) {
    ipsi = 1.0 / (g - u[2]);
    psi[pp] = (1.0 - 1.0 / ipsi) / qbm;
  } else {
    ipsi = 1.0 / (1.0 - qbm * psi_in);
  }
  if (!ii.ok) return;
  const double dpsi = qbm * (wp[2] - (wp[0] * u[0] + wp[1] * u[1]) * ipsi);
  du0 = du0 + u[0] * dpsi * ipsi;
  du1 = du1 + u[1] * dpsi * ipsi;
  const double a0 = u[0] * u[0] * ipsi, a1 = u[0] * u[1] * ipsi, a2 = u[1] * u[1] * ipsi;
  const double ph0r = ii.pcos, ph0i = -ii.psin;
  double phr = q[pp] * ipsi, phi = 0.0;
  const size_t ld = G.ld;
  const int n0 = ii.idx;
  const double wj[2] = {ii.w0, ii.w1};
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const double w = wj[j] * phr;
    const int nn = n0 + j;
    atomicAdd(cu + nn, w * u[0]);
    atomicAdd(cu + ld + nn, w * u[1]);
    atomicAdd(cu + 2 * ld + nn, w * u[2]);
    atomicAdd(acu + nn, w * du0);
    atomicAdd(acu + ld + nn, w * du1);
    atomicAdd(amu + nn, w * a0);
    atomicAdd(amu + ld + nn, w * a1);
    atomicAdd(amu + 2 * ld + nn, w * a2);
  }
  for (int m = 1; m <= G.M; ++m) {
    const double t = phr * ph0r - phi * ph0i;
    phi = phr * ph0i + phi * ph0r;
    phr = t;
    const int pr = 2 * m - 1, pi = 2 * m;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int nn = n0 + j;
      const double wr = wj[j] * phr, wi = wj[j] * phi;
      double* c_r = cu + (size_t)pr * 3 * ld + nn;
      double* c_i = cu + (size_t)pi * 3 * ld + nn;
      double* a_r = acu + (size_t)pr * 2 * ld + nn;
      double* a_i = acu + (size_t)pi * 2 * ld + nn;
      double* m_r = amu + (size_t)pr * 3 * ld + nn;
      double* m_i = amu + (size_t)pi * 3 * ld + nn;
      atomicAdd(c_r, wr * u[0]);
      atomicAdd(c_r + ld, wr * u[1]);
      atomicAdd(c_r + 2 * ld, wr * u[2]);
      atomicAdd(a_r, wr * du0);
      atomicAdd(a_r + ld, wr * du1);
      atomicAdd(m_r, wr * a0);
      atomicAdd(m_r + ld, wr * a1);
      atomicAdd(m_r + 2 * ld, wr * a2);
      atomicAdd(c_i, wi * u[0]);
      atomicAdd(c_i + ld, wi * u[1]);
      atomicAdd(c_i + 2 * ld, wi * u[2]);
      atomicAdd(a_i, wi * du0);
      atomicAdd(a_i + ld, wi * du1);
      atomicAdd(m_i, wi * a0);
      atomicAdd(m_i + ld, wi * a1);
      atomicAdd(m_i + 2 * ld, wi * a2);
    }
  }
}

// push_u (+ optionally push_x and the edge test).  alive[pp] = 1 if the particle stays.
__global__ void __launch_bounds__(kPartThreads) k_push(GridDev G, int push_type, double qbm, double dt,
                                                       const int64_t* __restrict__ n_ptr, double* __restrict__ x,
                                                       double* __restrict__ y, double* __restrict__ px,
                                                       double* __restrict__ py, double* __restrict__ pz,
                                                       double* __restrict__ gamma, const double* __restrict__ psi,
                                                       const double* __restrict__ ef, const double* __restrict__ bf,
                                                       int fuse_x, double edge, int32_t* __restrict__ alive) {
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const double qtmh = qbm * dt * 0.5;
  double xx = x[pp], yy = y[pp];
  const Interp ii = gen_interp(xx, yy, G.idr, G.nr);
  double ep[3], bp[3], ut[3], p[3];
  gather3(G, ef, ii, ep);
  gather3(G, bf, ii, bp);
  double t = ep[0] * ii.pcos - ep[1] * ii.psin;       // transform_to_cartesian
  ep[1] = ep[0] * ii.psin + ep[1] * ii.pcos;
  ep[0] = t;
  t = bp[0] * ii.pcos - bp[1] * ii.psin;
  bp[1] = bp[0] * ii.psin + bp[1] * ii.pcos;
  bp[0] = t;
  p[0] = px[pp]; p[1] = py[pp]; p[2] = pz[pp];
  double qtmh1, qtmh2;
  if (push_type == QPAD_PUSH2_ROBUST) {
    const double gam = sqrt(1.0 + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    qtmh1 = qtmh / (gam - p[2]);
    qtmh2 = qtmh1 * gam;
  } else {
    qtmh1 = qtmh / (1.0 - qbm * psi[pp]);
    qtmh2 = qtmh1 * gamma[pp];
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh2; bp[c] = bp[c] * qtmh1; ut[c] = p[c] + ep[c]; }
  p[0] = ut[0] + ut[1] * bp[2] - ut[2] * bp[1];
  p[1] = ut[1] + ut[2] * bp[0] - ut[0] * bp[2];
  p[2] = ut[2] + ut[0] * bp[1] - ut[1] * bp[0];
  const double ostq = 2.0 / (1.0 + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c) bp[c] = bp[c] * ostq;
  {
    const double t0 = ut[0] + p[1] * bp[2] - p[2] * bp[1];
    const double t1 = ut[1] + p[2] * bp[0] - p[0] * bp[2];
    const double t2 = ut[2] + p[0] * bp[1] - p[1] * bp[0];
    p[0] = t0 + ep[0]; p[1] = t1 + ep[1]; p[2] = t2 + ep[2];
  }
  const double g = sqrt(1.0 + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
  px[pp] = p[0]; py[pp] = p[1]; pz[pp] = p[2];
  gamma[pp] = g;
  if (fuse_x) {
    const double dtc = dt / (g - p[2]);
    xx = xx + p[0] * dtc;
    yy = yy + p[1] * dtc;
    x[pp] = xx;
    y[pp] = yy;
    alive[pp] = radius_rn(xx, yy) >= edge ? 0 : 1;
  }
}

__global__ void __launch_bounds__(kPartThreads) k_push_x(const int64_t* __restrict__ n_ptr, double dt,
                                                         double* __restrict__ x, double* __restrict__ y,
                                                         const double* __restrict__ px, const double* __restrict__ py,
                                                         const double* __restrict__ pz, const double* __restrict__ gamma,
                                                         double edge, int32_t* __restrict__ alive) {
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const double dtc = dt / (gamma[pp] - pz[pp]);
  const double xx = x[pp] + px[pp] * dtc, yy = y[pp] + py[pp] * dtc;
  x[pp] = xx;
  y[pp] = yy;
  alive[pp] = radius_rn(xx, yy) >= edge ? 0 : 1;
}

__global__ void __launch_bounds__(kPartThreads) k_interp_psi(GridDev G, const int64_t* __restrict__ n_ptr,
                                                             const double* __restrict__ x, const double* __restrict__ y,
                                                             const double* __restrict__ psif, double* __restrict__ psi) {
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const Interp ii = gen_interp(x[pp], y[pp], G.idr, G.nr);
  psi[pp] = gather1(G, psif, ii);
}

// ---- compaction: keep particles with flag[i] != 0, preserving order ------------------

__global__ void __launch_bounds__(kPartThreads) k_flags_to_i32(const int64_t* __restrict__ n_ptr, int64_t cap,
                                                               int32_t* __restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cap) return;
  if (i >= *n_ptr) flag[i] = 0;
}

__global__ void __launch_bounds__(kPartThreads) k_compact_scatter(const int64_t* __restrict__ n_ptr,
                                                                  const int32_t* __restrict__ flag,
                                                                  const int32_t* __restrict__ pos, PArrays src,
                                                                  PArrays dst, int na) {
  const int64_t n = *n_ptr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flag[i]) return;
  const int32_t d = pos[i];
  for (int k = 0; k < na; ++k) dst.a[k][d] = src.a[k][i];
}

__global__ void k_set_count(int64_t* __restrict__ n_ptr, const int64_t* __restrict__ total) { *n_ptr = *total; }

// ---- counting sort with the reference permutation ---------------------------------------
static constexpr int kSortTile = 1024;

__global__ void __launch_bounds__(kPartThreads) k_sort_keys(GridDev G, const int64_t* __restrict__ n_ptr,
                                                            const double* __restrict__ x, const double* __restrict__ y,
                                                            int32_t* __restrict__ key) {
  const int64_t n = *n_ptr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double pos = __dmul_rn(radius_rn(x[i], y[i]), G.idr);
  int k = (pos >= 0.0 && pos < (double)G.nr) ? (int)floor(pos) + 1 : G.nr;   // 1..nr (clamped)
  key[i] = k;
}

// Per tile of 1024 particles: rank of each particle among the earlier particles of the
// tile with the same key (warps taken in order, match_any inside a warp), and the
// tile histogram written key-major: hist[(key-1)*ntiles + tile].
__global__ void __launch_bounds__(kSortTile) k_sort_tile(GridDev G, const int64_t* __restrict__ n_ptr,
                                                         const int32_t* __restrict__ key, int32_t* __restrict__ rank,
                                                         int32_t* __restrict__ hist, int ntiles) {
  extern __shared__ int cnt[];
  const int64_t n = *n_ptr;
  const int tile = blockIdx.x;
  for (int k = threadIdx.x; k < G.nr; k += blockDim.x) cnt[k] = 0;
  __syncthreads();
  const int64_t i = (int64_t)tile * kSortTile + threadIdx.x;
  const bool valid = i < n;
  const int k = valid ? key[i] - 1 : -1 - (int)threadIdx.x;   // invalid lanes: unique keys
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int r = 0;
  for (int w = 0; w < kSortTile / 32; ++w) {
    if (warp == w) {
      const unsigned mask = __match_any_sync(0xffffffffu, k);
      const unsigned lt = (1u << lane) - 1u;
      const int base = valid ? cnt[k] : 0;
      __syncwarp();
      if (valid) {
        r = base + __popc(mask & lt);
        if ((mask & lt) == 0) cnt[k] = base + __popc(mask);
      }
    }
    __syncthreads();
  }
  if (valid) rank[i] = r;
  for (int kk = threadIdx.x; kk < G.nr; kk += blockDim.x) hist[(int64_t)kk * ntiles + tile] = cnt[kk];
}

// dest = end(key) - 1 - (#earlier particles with the same key), end = inclusive count
__global__ void __launch_bounds__(kPartThreads) k_sort_scatter(GridDev G, const int64_t* __restrict__ n_ptr,
                                                               const int32_t* __restrict__ key,
                                                               const int32_t* __restrict__ rank,
                                                               const int32_t* __restrict__ excl, int ntiles,
                                                               PArrays src, PArrays dst, int32_t* __restrict__ dest_out) {
  const int64_t n = *n_ptr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = key[i] - 1;
  const int tile = (int)(i / kSortTile);
  const int64_t start = excl[(int64_t)k * ntiles];
  const int64_t end = (k + 1 < G.nr) ? (int64_t)excl[(int64_t)(k + 1) * ntiles] : n;
  const int64_t before = (int64_t)excl[(int64_t)k * ntiles + tile] - start + rank[i];
  const int64_t d = end - 1 - before;
  for (int a = 0; a < 8; ++a) dst.a[a][d] = src.a[a][i];
  if (dest_out) dest_out[i] = (int32_t)(d + 1);
}

// ------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------
static PArrays arrays_of(qpad_species* sp, int b) {
  PArrays a;
  a.a[0] = sp->x[b]; a.a[1] = sp->y[b]; a.a[2] = sp->px[b]; a.a[3] = sp->py[b];
  a.a[4] = sp->pz[b]; a.a[5] = sp->gamma[b]; a.a[6] = sp->psi[b]; a.a[7] = sp->q[b];
  return a;
}

// The scatter target [1] is copied back into [0] (one contiguous block of 8 x npmax
// doubles) instead of swapping pointers, so that kernels captured in a CUDA graph keep
// valid arguments from slice to slice.
static int copy_back(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  return cuda_check(ctx, cudaMemcpyAsync(sp->x[0], sp->x[1], sizeof(double) * 8 * (size_t)sp->npmax,
                                         cudaMemcpyDeviceToDevice, ctx->stream), "copy back");
}

int species_qdeposit_raw(qpad_species* sp, double* qraw) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  prof_begin(ctx, "qdeposit");
  k_qdeposit<<<grid_for(sp->np, kPartThreads), kPartThreads, 0, ctx->stream>>>(ctx->g, sp->d_count, sp->x[0], sp->y[0],
                                                                              sp->q[0], qraw);
  prof_end(ctx, "qdeposit");
  return check_launch(ctx, "k_qdeposit");
}

// The charge deposit of arbitrary particle arrays (count on the device, at most n_bound).
int qdeposit_arrays(qpad_ctx* ctx, const int64_t* d_count, int64_t n_bound, const double* x, const double* y,
                    const double* q, double* qraw) {
  if (n_bound <= 0) return 0;
  k_qdeposit<<<grid_for(n_bound, kPartThreads), kPartThreads, 0, ctx->stream>>>(ctx->g, d_count, x, y, q, qraw);
  return check_launch(ctx, "k_qdeposit (arrays)");
}

int species_amjdp_raw(qpad_species* sp, const double* ef, const double* bf, double* cu, double* amu, double* acu,
                      double dt) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  if (is_pgc(sp->push_type)) return laser_amjdp_raw(sp, ef, bf, cu, amu, acu, dt);
  prof_begin(ctx, "amjdp");
  k_amjdp<<<grid_for(sp->np, kPartThreads), kPartThreads, 0, ctx->stream>>>(
      ctx->g, sp->push_type, sp->qbm, dt, sp->d_count, sp->x[0], sp->y[0], sp->px[0], sp->py[0], sp->pz[0], sp->q[0],
      sp->gamma[0], sp->psi[0], ef, bf, cu, amu, acu, iter_guard(ctx));
  prof_end(ctx, "amjdp");
  return check_launch(ctx, "k_amjdp");
}

int species_push_u(qpad_species* sp, const double* ef, const double* bf, double dt, int fuse_x) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  if (is_pgc(sp->push_type)) return laser_push_u(sp, ef, bf, dt, fuse_x);
  const double edge = (double)ctx->g.nr * ctx->g.dr;
  prof_begin(ctx, "push");
  k_push<<<grid_for(sp->np, kPartThreads), kPartThreads, 0, ctx->stream>>>(
      ctx->g, sp->push_type, sp->qbm, dt, sp->d_count, sp->x[0], sp->y[0], sp->px[0], sp->py[0], sp->pz[0],
      sp->gamma[0], sp->psi[0], ef, bf, fuse_x, edge, sp->key);
  prof_end(ctx, "push");
  if (int r = check_launch(ctx, "k_push")) return r;
  return fuse_x ? species_compact(sp) : 0;
}

int species_push_x(qpad_species* sp, double dt) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  const double edge = (double)ctx->g.nr * ctx->g.dr;
  k_push_x<<<grid_for(sp->np, kPartThreads), kPartThreads, 0, ctx->stream>>>(
      sp->d_count, dt, sp->x[0], sp->y[0], sp->px[0], sp->py[0], sp->pz[0], sp->gamma[0], edge, sp->key);
  if (int r = check_launch(ctx, "k_push_x")) return r;
  return species_compact(sp);
}

// Removes particles whose sp->key flag is 0; the new count lands in sp->d_count.
int species_compact(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  const int64_t n = sp->np;
  if (n == 0) return 0;
  int32_t* pos = sp->aux;
  int32_t* tmp = sp->blk;
  k_flags_to_i32<<<grid_for(n, kPartThreads), kPartThreads, 0, ctx->stream>>>(sp->d_count, n, sp->key);
  if (int r = scan_i32(ctx, sp->key, pos, n, tmp, sp->d_total)) return r;
  k_compact_scatter<<<grid_for(n, kPartThreads), kPartThreads, 0, ctx->stream>>>(sp->d_count, sp->key, pos,
                                                                                 arrays_of(sp, 0), arrays_of(sp, 1), 8);
  k_set_count<<<1, 1, 0, ctx->stream>>>(sp->d_count, sp->d_total);
  if (int r = check_launch(ctx, "compact", 3)) return r;
  return copy_back(sp);
}

int species_sort(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  const int64_t n = sp->np;
  if (n == 0) return 0;
  const int ntiles = (int)((n + kSortTile - 1) / kSortTile);
  const int64_t nh = (int64_t)ntiles * ctx->g.nr;
  // scratch: hist (nh) and its scan (nh) + scan temporaries live in sp->blk
  int32_t* hist = sp->blk;
  int32_t* excl = hist + nh;
  int32_t* tmp = excl + nh;
  k_sort_keys<<<grid_for(n, kPartThreads), kPartThreads, 0, ctx->stream>>>(ctx->g, sp->d_count, sp->x[0], sp->y[0],
                                                                           sp->key);
  k_sort_tile<<<ntiles, kSortTile, ctx->g.nr * sizeof(int), ctx->stream>>>(ctx->g, sp->d_count, sp->key, sp->aux, hist,
                                                                          ntiles);
  if (int r = scan_i32(ctx, hist, excl, nh, tmp, nullptr)) return r;
  k_sort_scatter<<<grid_for(n, kPartThreads), kPartThreads, 0, ctx->stream>>>(
      ctx->g, sp->d_count, sp->key, sp->aux, excl, ntiles, arrays_of(sp, 0), arrays_of(sp, 1), nullptr);
  if (int r = check_launch(ctx, "sort", 3)) return r;
  return copy_back(sp);
}

int species_interp_psi(qpad_species* sp, const double* psif) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  k_interp_psi<<<grid_for(sp->np, kPartThreads), kPartThreads, 0, ctx->stream>>>(ctx->g, sp->d_count, sp->x[0],
                                                                                 sp->y[0], psif, sp->psi[0]);
  return check_launch(ctx, "k_interp_psi");
}

int species_sync_count(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  cudaError_t e = cudaMemcpyAsync(sp->h_count, sp->d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "count readback");
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "count sync");
  sp->np = sp->neut ? sp->npmax : *sp->h_count;   // (a neutral gas's launches cover its capacity)
  return 0;
}

}  // namespace qpad
