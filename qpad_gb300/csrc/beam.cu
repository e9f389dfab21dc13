// beam.cu -- beam (3D) particle kernels (FP64 reference arithmetic).
//
//   k_beam_qdeposit   part3d::qdeposit (part3d_class.f03:221-356) into the q_beam 3D store
//   k_beam_finish_q   its axis corrections and 1/(j-1) scaling for slices 1..nz
//   k_beam_push       part3d::push_reduced / push_boris with interp_emf_part3d
//                     (part3d_class.f03:477-576, 358-475, 691-790) and the edge test of
//                     update_bound (:640-689); removal by order-preserving compaction.
#include <algorithm>

#include "particles.cuh"

namespace qpad {

static constexpr int kBeamThreads = 256;

static int grid_for(int64_t n) {
  int64_t b = (n + kBeamThreads - 1) / kBeamThreads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 1 << 30));
}

__device__ __forceinline__ double* q2_at(const GridDev& G, double* q2, int s, int p) {
  return q2 + ((size_t)(s - 1) * G.P + p) * G.ld;
}

__global__ void __launch_bounds__(kBeamThreads) k_beam_qdeposit(GridDev G, const int64_t* __restrict__ n_ptr,
                                                                const double* __restrict__ x,
                                                                const double* __restrict__ y,
                                                                const double* __restrict__ z,
                                                                const double* __restrict__ q, double* __restrict__ q2) {
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const double xx = x[pp], yy = y[pp];
  double pr = __dmul_rn(radius_rn(xx, yy), G.idr);
  double pzs = __dmul_rn(z[pp], 1.0 / G.dxi);
  const double ph0r = xx / pr * G.idr, ph0i = -yy / pr * G.idr;
  if (!(pr >= 0.0 && pr < (double)G.nr && pzs >= 0.0 && pzs < (double)G.nz)) return;
  const int nn0 = (int)floor(pr), mm0 = (int)floor(pzs);
  pr = __dsub_rn(pr, (double)nn0);
  pzs = __dsub_rn(pzs, (double)mm0);
  const int nn = nn0 + 1, mm = mm0 + 1;
  const double wr[2] = {1.0 - pr, pr}, wz[2] = {1.0 - pzs, pzs};
  double phr = 1.0 * q[pp], phi = 0.0;
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int j = 0; j < 2; ++j) atomicAdd(q2_at(G, q2, mm + k, 0) + nn + j, wr[j] * wz[k] * phr);
  for (int m = 1; m <= G.M; ++m) {
    const double t = phr * ph0r - phi * ph0i;
    phi = phr * ph0i + phi * ph0r;
    phr = t;
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const double w = wr[j] * wz[k];
        atomicAdd(q2_at(G, q2, mm + k, 2 * m - 1) + nn + j, w * phr);
        atomicAdd(q2_at(G, q2, mm + k, 2 * m) + nn + j, w * phi);
      }
  }
}

// slices 1..nz: node 0 -> 0; node 1: x8 (m=0) / 0 (m>0); nodes 2..nr+1: x 1/(j-1)
__global__ void k_beam_finish_q(GridDev G, double* __restrict__ q2) {
  const int s = blockIdx.x + 1, p = blockIdx.y;
  double* row = q2_at(G, q2, s, p);
  for (int i = threadIdx.x; i <= G.nr + 1; i += blockDim.x) {
    const double v = row[i];
    double o;
    if (i == 0) o = 0.0;
    else if (i == 1) o = (p == 0) ? 8.0 * v : 0.0;
    else o = v * G.inv[i];
    row[i] = o;
  }
}

// interp_emf_part3d (part3d_class.f03:691-790); e2/b2 stores hold 3 components
__device__ __forceinline__ void beam_gather(const GridDev& G, const double* __restrict__ e2,
                                            const double* __restrict__ b2, double x, double y, double z,
                                            double ep[3], double bp[3]) {
  ep[0] = ep[1] = ep[2] = 0.0;
  bp[0] = bp[1] = bp[2] = 0.0;
  double pr = __dmul_rn(radius_rn(x, y), G.idr);
  double pzs = __dmul_rn(z, 1.0 / G.dxi);
  const double cc = x / pr * G.idr, ss = y / pr * G.idr;
  if (!(pr >= 0.0 && pr < (double)G.nr && pzs > -1.0 && pzs < (double)G.nz)) return;
  const int nn0 = (int)pr, mm0 = (int)pzs;   // truncation, as int() in the reference
  pr = __dsub_rn(pr, (double)nn0);
  pzs = __dsub_rn(pzs, (double)mm0);
  const int nn = nn0 + 1, mm = mm0 + 1;
  const double wr[2] = {1.0 - pr, pr}, wz[2] = {1.0 - pzs, pzs};
  const size_t ld = G.ld, slab = (size_t)G.P * 3 * ld;
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const double wt = wr[j] * wz[k];
      const size_t o = (size_t)(mm + k - 1) * slab + nn + j;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ep[c] = ep[c] + __ldg(e2 + o + c * ld) * wt;
        bp[c] = bp[c] + __ldg(b2 + o + c * ld) * wt;
      }
    }
  double phr = 1.0, phi = 0.0;
  for (int m = 1; m <= G.M; ++m) {
    const double t = phr * cc - phi * ss;
    phi = phr * ss + phi * cc;
    phr = t;
    const double ph_r = 2.0 * phr, ph_i = 2.0 * phi;
    const size_t orr = (size_t)(2 * m - 1) * 3 * ld, oi = (size_t)(2 * m) * 3 * ld;
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const double wt = wr[j] * wz[k];
        const size_t o = (size_t)(mm + k - 1) * slab + nn + j;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          ep[c] = ep[c] + (__ldg(e2 + o + orr + c * ld) * ph_r - __ldg(e2 + o + oi + c * ld) * ph_i) * wt;
          bp[c] = bp[c] + (__ldg(b2 + o + orr + c * ld) * ph_r - __ldg(b2 + o + oi + c * ld) * ph_i) * wt;
        }
      }
  }
  double a = ep[0] * cc - ep[1] * ss, b = ep[0] * ss + ep[1] * cc;
  ep[0] = a; ep[1] = b;
  a = bp[0] * cc - bp[1] * ss; b = bp[0] * ss + bp[1] * cc;
  bp[0] = a; bp[1] = b;
}

__global__ void __launch_bounds__(kBeamThreads) k_beam_push(GridDev G, int push_type, double qbm, double dt,
                                                            const int64_t* __restrict__ n_ptr, double* __restrict__ x,
                                                            double* __restrict__ y, double* __restrict__ z,
                                                            double* __restrict__ px, double* __restrict__ py,
                                                            double* __restrict__ pz, const double* __restrict__ e2,
                                                            const double* __restrict__ b2, double edge_r, double edge_z,
                                                            int32_t* __restrict__ alive) {
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const double qtmh = qbm * dt * 0.5;
  double ep[3], bp[3], p[3] = {px[pp], py[pp], pz[pp]};
  beam_gather(G, e2, b2, x[pp], y[pp], z[pp], ep, bp);
  if (push_type == QPAD_PUSH3_REDUCED) {
    double wp[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh; bp[c] = bp[c] * qtmh; }
    wp[0] = ep[0] - bp[1];
    wp[1] = ep[1] + bp[0];
    wp[2] = ep[2];
#pragma unroll
    for (int c = 0; c < 3; ++c) p[c] = p[c] + wp[c];
#pragma unroll
    for (int c = 0; c < 3; ++c) p[c] = p[c] + wp[c];
  } else {
    double ut[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh; ut[c] = p[c] + ep[c]; }
    const double gam = sqrt(1.0 + (ut[0] * ut[0] + ut[1] * ut[1] + ut[2] * ut[2]));
    const double gq = qtmh / gam;
#pragma unroll
    for (int c = 0; c < 3; ++c) bp[c] = bp[c] * gq;
    p[0] = ut[0] + ut[1] * bp[2] - ut[2] * bp[1];
    p[1] = ut[1] + ut[2] * bp[0] - ut[0] * bp[2];
    p[2] = ut[2] + ut[0] * bp[1] - ut[1] * bp[0];
    const double ostq = 2.0 / (1.0 + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) bp[c] = bp[c] * ostq;
    const double t0 = ut[0] + p[1] * bp[2] - p[2] * bp[1];
    const double t1 = ut[1] + p[2] * bp[0] - p[0] * bp[2];
    const double t2 = ut[2] + p[0] * bp[1] - p[1] * bp[0];
    p[0] = t0 + ep[0]; p[1] = t1 + ep[1]; p[2] = t2 + ep[2];
  }
  const double dt_gam = dt / sqrt(1.0 + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
  const double xx = x[pp] + p[0] * dt_gam, yy = y[pp] + p[1] * dt_gam;
  const double zz = z[pp] - p[2] * dt_gam + dt;
  x[pp] = xx; y[pp] = yy; z[pp] = zz;
  px[pp] = p[0]; py[pp] = p[1]; pz[pp] = p[2];
  alive[pp] = (radius_rn(xx, yy) >= edge_r || zz >= edge_z) ? 0 : 1;
}

__global__ void k_beam_flags(const int64_t* __restrict__ n_ptr, int64_t cap, int32_t* __restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cap && i >= *n_ptr) flag[i] = 0;
}

__global__ void k_beam_scatter(const int64_t* __restrict__ n_ptr, const int32_t* __restrict__ flag,
                               const int32_t* __restrict__ pos, PArrays src, PArrays dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *n_ptr || !flag[i]) return;
  const int32_t d = pos[i];
#pragma unroll
  for (int k = 0; k < 7; ++k) dst.a[k][d] = src.a[k][i];
}

__global__ void k_beam_set_count(int64_t* __restrict__ n_ptr, const int64_t* __restrict__ total) { *n_ptr = *total; }

static PArrays beam_arrays(qpad_beam* bm, int b) {
  PArrays a;
  a.a[0] = bm->x[b]; a.a[1] = bm->y[b]; a.a[2] = bm->z[b]; a.a[3] = bm->px[b];
  a.a[4] = bm->py[b]; a.a[5] = bm->pz[b]; a.a[6] = bm->q[b]; a.a[7] = nullptr;
  return a;
}

int beam_qdeposit(qpad_beam* bm, double* q2) {
  qpad_ctx* ctx = bm->ctx;
  if (bm->nb == 0) return 0;
  prof_begin(ctx, "beam_qdeposit");
  k_beam_qdeposit<<<grid_for(bm->nb), kBeamThreads, 0, ctx->stream>>>(ctx->g, bm->d_count, bm->x[0], bm->y[0],
                                                                       bm->z[0], bm->q[0], q2);
  prof_end(ctx, "beam_qdeposit");
  return check_launch(ctx, "k_beam_qdeposit");
}

int beam_finish_q(qpad_ctx* ctx, double* q2) {
  dim3 grid(ctx->g.nz, ctx->g.P);
  k_beam_finish_q<<<grid, 256, 0, ctx->stream>>>(ctx->g, q2);
  return check_launch(ctx, "k_beam_finish_q");
}

int beam_push(qpad_beam* bm, const double* e2, const double* b2) {
  qpad_ctx* ctx = bm->ctx;
  if (bm->nb == 0 || !bm->evolution) return 0;
  const int64_t n = bm->nb;
  const double er = (double)ctx->g.nr * ctx->g.dr, ez = (double)ctx->g.nz * ctx->g.dxi;
  prof_begin(ctx, "beam_push");
  k_beam_push<<<grid_for(n), kBeamThreads, 0, ctx->stream>>>(ctx->g, bm->push_type, bm->qbm, ctx->dt, bm->d_count,
                                                             bm->x[0], bm->y[0], bm->z[0], bm->px[0], bm->py[0],
                                                             bm->pz[0], e2, b2, er, ez, bm->key);
  prof_end(ctx, "beam_push");
  k_beam_flags<<<grid_for(n), kBeamThreads, 0, ctx->stream>>>(bm->d_count, n, bm->key);
  if (int r = scan_i32(ctx, bm->key, bm->aux, n, bm->blk, bm->d_total)) return r;
  k_beam_scatter<<<grid_for(n), kBeamThreads, 0, ctx->stream>>>(bm->d_count, bm->key, bm->aux, beam_arrays(bm, 0),
                                                                beam_arrays(bm, 1));
  k_beam_set_count<<<1, 1, 0, ctx->stream>>>(bm->d_count, bm->d_total);
  std::swap(bm->x[0], bm->x[1]); std::swap(bm->y[0], bm->y[1]); std::swap(bm->z[0], bm->z[1]);
  std::swap(bm->px[0], bm->px[1]); std::swap(bm->py[0], bm->py[1]); std::swap(bm->pz[0], bm->pz[1]);
  std::swap(bm->q[0], bm->q[1]);
  return check_launch(ctx, "beam_push", 4);
}

}  // namespace qpad
