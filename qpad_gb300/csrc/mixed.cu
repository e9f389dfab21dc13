// mixed.cu -- mixed-precision plasma particle path (QPAD_PREC_MIXED).
//
// Particles: each Cartesian coordinate is an integer cell plus an FP32 offset in [0,1)
// (x = (cell + offset) * dr), so positions do not lose precision as they are advanced
// slice after slice; momenta, charge, gamma and psi are FP32.  The particles are kept
// sorted by radial cell (counting sort after every push).
//
// Gather: E and B are read from an FP32 table [node][part][E0,E1,E2,B0,B1,B2] written by
// the field kernels after every FP64 solve, so one particle reads two contiguous records.
//
// Deposit: the counting sort after every push also writes deposit work items, each at most
// one warp's worth of particles (32 x PPL, PPL = 1, 2 or 4) of a single radial cell.  A warp
// takes an item: every particle of it deposits to the same two nodes, so each lane
// accumulates its particles' contributions to the 2 nodes x Re/Im x 8 quantities of a mode
// in registers, one transposing butterfly (31 shuffles) leaves each lane one total, and each
// lane adds that total into the FP64 global mode arrays with one atomic.  The field solves
// that follow stay FP64.
//
// Reference routines: part2d::qdeposit (part2d_class.f03:231-359), amjdeposit_robust /
// _std (:746-1010, 478-744), push_u_robust / _std (:1879-1965, 1790-1877), push_x
// (:2221-2262), update_bound (:2307-2353), sort (:2498-2579), interp_psi (:2264-2305).
#include <algorithm>

#include "particles.cuh"

namespace qpad {

static constexpr int kMixThreads = 256;
// A deposit work item is one warp's worth of particles of one cell: 32 * PPL of them,
// PPL = ctx->item_ppl in {1, 2, 4} (chosen by qpad_autotune, 4 by default).
static constexpr int kMinItem = 32;                       // smallest work item (sizes the item list)
static constexpr int kItemThreads = 128;                  // four work items per CTA
#define FULL 0xffffffffu

struct MArr {
  int32_t* cxy;
  float *fx, *fy, *px, *py, *pz, *q, *gam, *psi;
  int32_t* key;
};

static MArr marr(qpad_species* sp, int b) {
  return MArr{sp->cxy[b], sp->fx[b], sp->fy[b], sp->mpx[b], sp->mpy[b], sp->mpz[b],
              sp->mq[b],  sp->mgam[b], sp->mpsi[b], sp->mkey[b]};
}

static int mgrid(int64_t n, int per) {
  int64_t b = (n + per - 1) / per;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 1 << 30));
}

__device__ __forceinline__ void unpack_cell(int32_t c, int& ix, int& iy) {
  ix = (int)(int16_t)(uint16_t)((uint32_t)c & 0xffffu);
  iy = (int)(int16_t)(uint16_t)((uint32_t)c >> 16);
}

__device__ __forceinline__ int32_t pack_cell(int ix, int iy) {
  return (int32_t)(((uint32_t)(uint16_t)(int16_t)ix) | ((uint32_t)(uint16_t)(int16_t)iy << 16));
}

// gamma - u_z of a momentum u with gamma = sqrt(1 + |u|^2), without the cancellation of
// the difference for u_z > 0: (gamma - u_z)(gamma + u_z) = 1 + u_x^2 + u_y^2.  In FP32 the
// plain difference loses about log2(2 u_z^2 / (1 + u_perp^2)) bits for a relativistic
// particle moving forward (sheath electrons of a blowout), which the FP64 reference does
// not notice but an FP32 push would.
__device__ __forceinline__ float gamma_minus_uz(float ux, float uy, float uz, float gam) {
  return uz > 0.0f ? (1.0f + ux * ux + uy * uy) / (gam + uz) : gam - uz;
}

// Radial cell K = floor(r) and fraction d = r - K of a particle at (ix + fx, iy + fy) cells,
// to the FP32 precision of d itself.  X = ix + fx rounded to FP32 keeps only
// 24 - log2|X| bits of the offset (about 1e-5 of a cell at X = 500), so away from the axis
// r is not formed from X: r - K = (r^2 - K^2) / (r + K), whose numerator splits into the
// exact integer ix^2 + iy^2 - K^2 and 2 (ix fx + iy fy) + fx^2 + fy^2, both small next to
// r + K.  Within 4 cells of the axis X and Y are nearly exact and the plain radius is the
// more precise.  r_est: sqrtf(X^2 + Y^2).
__device__ __forceinline__ void cell_radius(int ix, int iy, float fx, float fy, float r_est, int& K, float& d) {
  K = (int)r_est;
  d = r_est - (float)K;
  if (r_est < 4.0f) return;
  const float B = 2.0f * ((float)ix * fx + (float)iy * fy) + (fx * fx + fy * fy);
  const long long s2 = (long long)ix * ix + (long long)iy * iy;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    d = ((float)(s2 - (long long)K * K) + B) / (r_est + (float)K);
    if (d < 0.0f) {
      --K;
    } else if (d >= 1.0f) {
      ++K;
    } else {
      return;
    }
  }
  d = fminf(fmaxf(d, 0.0f), 0.99999994f);   // (a third step is never needed: |r_est - r| << 1)
}

// Radial interpolation data in cell units (FP32).
struct MInterp {
  float w0, w1, pcos, psin;
  int idx;
  bool ok;
};

__device__ __forceinline__ MInterp minterp(int32_t c, float fx, float fy, int nr) {
  int ix, iy;
  unpack_cell(c, ix, iy);
  const float X = (float)ix + fx, Y = (float)iy + fy;
  const float r = sqrtf(X * X + Y * Y);
  int K;
  float d;
  cell_radius(ix, iy, fx, fy, r, K, d);
  MInterp m;
  m.pcos = X / r;
  m.psin = Y / r;
  m.ok = K >= 0 && K < nr;
  m.idx = (m.ok ? K : 0) + 1;
  m.w1 = m.ok ? d : 0.0f;
  m.w0 = m.ok ? 1.0f - d : 0.0f;
  return m;
}

// Instances of the particle kernels: kM >= 0 is the highest azimuthal mode known at compile
// time (every mode loop unrolls, every table offset is a constant); kM = -1 takes it from
// the grid at run time (at most QPAD_MAX_MODE).
template <int kM>
struct ModeLoop {
  static constexpr int kLast = kM >= 0 ? kM : QPAD_MAX_MODE;
  __device__ __forceinline__ static bool past(int m, int M) { return kM < 0 && m > M; }
  __device__ __forceinline__ static int modes(int M) { return kM >= 0 ? kM : M; }
};

// E and B gathered from the FP32 table (interp_field, interp_part2d.f03:67-109)
// t0: the records of node ii.idx (in the table, or a copy of the two nodes' records)
template <int kM>
__device__ __forceinline__ void mgather_at(const float* t0, int Prt, int Mrt, const MInterp& ii, float ep[3],
                                           float bp[3]) {
  const int M = ModeLoop<kM>::modes(Mrt), P = kM >= 0 ? 2 * kM + 1 : Prt;
#pragma unroll
  for (int c = 0; c < 3; ++c) { ep[c] = 0.0f; bp[c] = 0.0f; }
  if (!ii.ok) return;
  const float* t1 = t0 + (size_t)P * 6;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    ep[c] = t0[c] * ii.w0 + t1[c] * ii.w1;
    bp[c] = t0[3 + c] * ii.w0 + t1[3 + c] * ii.w1;
  }
  float phr = 1.0f, phi = 0.0f;
#pragma unroll
  for (int m = 1; m <= ModeLoop<kM>::kLast; ++m) {
    if (ModeLoop<kM>::past(m, M)) break;
    const float t = phr * ii.pcos - phi * ii.psin;
    phi = phr * ii.psin + phi * ii.pcos;
    phr = t;
    const float pre = 2.0f * phr, pim = 2.0f * phi;
    const float* r0 = t0 + (2 * m - 1) * 6;
    const float* i0 = t0 + (2 * m) * 6;
    const float* r1 = t1 + (2 * m - 1) * 6;
    const float* i1 = t1 + (2 * m) * 6;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      ep[c] += (r0[c] * pre - i0[c] * pim) * ii.w0 + (r1[c] * pre - i1[c] * pim) * ii.w1;
      bp[c] += (r0[3 + c] * pre - i0[3 + c] * pim) * ii.w0 +
               (r1[3 + c] * pre - i1[3 + c] * pim) * ii.w1;
    }
  }
}

template <int kM>
__device__ __forceinline__ void mgather(const float* __restrict__ T, int P, int M, const MInterp& ii, float ep[3],
                                        float bp[3]) {
  mgather_at<kM>(T + (size_t)(ii.ok ? ii.idx : 0) * P * 6, P, M, ii, ep, bp);
}

// The same gather from one cell's records staged as pairs tp[part * 6 + comp] =
// (value at the inner node, outer minus inner): each value at the particle is one FMA.
template <int kM>
__device__ __forceinline__ void mgather_pair(const float2* tp, int Mrt, const MInterp& ii, float ep[3], float bp[3]) {
  const int M = ModeLoop<kM>::modes(Mrt);
  const float w1 = ii.w1;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float2 e = tp[c], b = tp[3 + c];
    ep[c] = ii.ok ? fmaf(w1, e.y, e.x) : 0.0f;
    bp[c] = ii.ok ? fmaf(w1, b.y, b.x) : 0.0f;
  }
  if (!ii.ok) return;
  float phr = 1.0f, phi = 0.0f;
#pragma unroll
  for (int m = 1; m <= ModeLoop<kM>::kLast; ++m) {
    if (ModeLoop<kM>::past(m, M)) break;
    const float t = phr * ii.pcos - phi * ii.psin;
    phi = phr * ii.psin + phi * ii.pcos;
    phr = t;
    const float pre = 2.0f * phr, pim = 2.0f * phi;
    const float2* re = tp + (2 * m - 1) * 6;
    const float2* im = tp + (2 * m) * 6;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float er = fmaf(w1, re[c].y, re[c].x), ei = fmaf(w1, im[c].y, im[c].x);
      const float br = fmaf(w1, re[3 + c].y, re[3 + c].x), bi = fmaf(w1, im[3 + c].y, im[3 + c].x);
      ep[c] = fmaf(er, pre, fmaf(-ei, pim, ep[c]));
      bp[c] = fmaf(br, pre, fmaf(-bi, pim, bp[c]));
    }
  }
}

// Sum over the 32 lanes of each of 32 values: after the exchange, lane l holds in a[0]
// the total of value l (a transposing butterfly, 31 shuffles for 32 sums).
__device__ __forceinline__ void butterfly32(float (&a)[32], int lane) {
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool up = (lane & s) != 0;
#pragma unroll
    for (int k = 0; k < s; ++k) {
      const float send = up ? a[k] : a[k + s];
      const float keep = up ? a[k + s] : a[k];
      a[k] = keep + __shfl_xor_sync(FULL, send, s);
    }
  }
}

// ------------------------------------------------------------------------------------
// charge deposit (rho - Jz), one warp per work item (kItem particles of one cell)
// ------------------------------------------------------------------------------------
template <int kPPL, int kM>
__global__ void __launch_bounds__(kItemThreads) k_mqdeposit(GridDev G, const int4* __restrict__ items,
                                                            const int* __restrict__ n_items, MArr A,
                                                            double* __restrict__ qraw) {
  const int lane = threadIdx.x & 31;
  const int it = blockIdx.x * (kItemThreads / 32) + (threadIdx.x >> 5);
  if (it >= *n_items) return;                          // warp-uniform
  const int4 item = items[it];
  const int key = item.x, start = item.y, cnt = item.z;
  float wq[kPPL][2], pc[kPPL][2];
#pragma unroll
  for (int j = 0; j < kPPL; ++j) {
    const int o = j * 32 + lane;
    wq[j][0] = wq[j][1] = 0.0f;
    pc[j][0] = 1.0f;
    pc[j][1] = 0.0f;
    if (o < cnt) {
      const int i = start + o;
      const MInterp ii = minterp(A.cxy[i], A.fx[i], A.fy[i], G.nr);
      if (ii.ok) {
        const float q = A.q[i];
        wq[j][0] = q * ii.w0;
        wq[j][1] = q * ii.w1;
        pc[j][0] = ii.pcos;
        pc[j][1] = -ii.psin;
      }
    }
  }
  float ph[kPPL][2];
#pragma unroll
  for (int j = 0; j < kPPL; ++j) { ph[j][0] = 1.0f; ph[j][1] = 0.0f; }
#pragma unroll
  for (int m = 0; m <= ModeLoop<kM>::kLast; ++m) {
    if (ModeLoop<kM>::past(m, G.M)) break;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};          // [node 0/1][re, im]
#pragma unroll
    for (int j = 0; j < kPPL; ++j) {
      if (m > 0) {
        const float t = ph[j][0] * pc[j][0] - ph[j][1] * pc[j][1];
        ph[j][1] = ph[j][0] * pc[j][1] + ph[j][1] * pc[j][0];
        ph[j][0] = t;
      }
#pragma unroll
      for (int jn = 0; jn < 2; ++jn) {
        acc[2 * jn] += wq[j][jn] * ph[j][0];
        acc[2 * jn + 1] += wq[j][jn] * ph[j][1];
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(FULL, acc[k], off);
    if (lane < 4) {
      const int jn = lane >> 1, h = lane & 1;
      float v = acc[0];
#pragma unroll
      for (int k = 1; k < 4; ++k)
        if (lane == k) v = acc[k];
      if (!(m == 0 && h == 1) && v != 0.0f) {
        const int p = m == 0 ? 0 : 2 * m - 1 + h;
        atomicAdd(qraw + (size_t)p * G.ld + key + jn, (double)v);
      }
    }
  }
}

// Predictor push of one particle (amjdeposit_robust / _std): the deposit values
// v = {u0, u1, u2, du0, du1, u0 u0 / (g - u2) .. } and the charge factor qq = q / (g - u2).
// pv: the particle's px, py, pz, psi, q (loaded by the caller); ep, bp: E and B gathered at
// the particle (overwritten)
__device__ __forceinline__ void mpredict(int push_type, float qbm, float dt, const MArr& A, int64_t i,
                                         int write_back, const MInterp& ii, float ep[3], float bp[3],
                                         const float pv[5], float v[8], float& qq) {
  const float idt = 1.0f / dt, qtmh = 0.5f * qbm * dt;
  float wp[3], u0[3], u[3], ut[3];
  wp[0] = ep[0] - bp[1];
  wp[1] = ep[1] + bp[0];
  wp[2] = ep[2];
  const float p1 = pv[0], p2 = pv[1];
  u0[0] = p1 * ii.pcos + p2 * ii.psin;
  u0[1] = p2 * ii.pcos - p1 * ii.psin;
  u0[2] = pv[2];
  const float psi_in = pv[3];
  if (push_type == QPAD_PUSH2_ROBUST) {
    float gam = sqrtf(1.0f + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]);
    const float qtmh1 = qtmh * gam / gamma_minus_uz(u0[0], u0[1], u0[2], gam);
#pragma unroll
    for (int c = 0; c < 3; ++c) { ep[c] *= qtmh1; ut[c] = u0[c] + ep[c]; }
    gam = sqrtf(1.0f + ut[0] * ut[0] + ut[1] * ut[1] + ut[2] * ut[2]);
    const float qtmh2 = qtmh / gamma_minus_uz(ut[0], ut[1], ut[2], gam);
#pragma unroll
    for (int c = 0; c < 3; ++c) bp[c] *= qtmh2;
  } else {
    const float gam = sqrtf(1.0f + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2]);
    const float qtmh2 = qtmh / (1.0f - qbm * psi_in);
    const float qtmh1 = qtmh2 * gam;
#pragma unroll
    for (int c = 0; c < 3; ++c) { bp[c] *= qtmh2; ut[c] = u0[c] + ep[c] * qtmh1; }
  }
  u[0] = ut[0] + ut[1] * bp[2] - ut[2] * bp[1];
  u[1] = ut[1] + ut[2] * bp[0] - ut[0] * bp[2];
  u[2] = ut[2] + ut[0] * bp[1] - ut[1] * bp[0];
  const float ostq = 2.0f / (1.0f + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c) bp[c] *= ostq;
  {
    const float t0 = ut[0] + u[1] * bp[2] - u[2] * bp[1];
    const float t1 = ut[1] + u[2] * bp[0] - u[0] * bp[2];
    const float t2 = ut[2] + u[0] * bp[1] - u[1] * bp[0];
    ut[0] = t0; ut[1] = t1; ut[2] = t2;
  }
  if (push_type == QPAD_PUSH2_ROBUST) {
#pragma unroll
    for (int c = 0; c < 3; ++c) u[c] = ut[c] + ep[c];
  } else {
    const float gam = sqrtf(1.0f + ut[0] * ut[0] + ut[1] * ut[1] + ut[2] * ut[2]);
    const float qtmh1 = qtmh / (1.0f - qbm * psi_in) * gam;
#pragma unroll
    for (int c = 0; c < 3; ++c) u[c] = ut[c] + ep[c] * qtmh1;
  }
  float du0 = idt * (u[0] - u0[0]);
  float du1 = idt * (u[1] - u0[1]);
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = 0.5f * (u[c] + u0[c]);
  const float g = sqrtf(1.0f + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  float ipsi;
  if (push_type == QPAD_PUSH2_ROBUST) {
    ipsi = 1.0f / gamma_minus_uz(u[0], u[1], u[2], g);
    // psi = (1 - gamma + u_z) / qbm with gamma - 1 = |u|^2 / (gamma + 1): no cancellation
    if (write_back) {
      A.gam[i] = g;
      A.psi[i] = (u[2] - (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) / (g + 1.0f)) / qbm;
    }
  } else {
    ipsi = 1.0f / (1.0f - qbm * psi_in);
    A.gam[i] = g;
  }
  const float dpsi = qbm * (wp[2] - (wp[0] * u[0] + wp[1] * u[1]) * ipsi);
  du0 += u[0] * dpsi * ipsi;
  du1 += u[1] * dpsi * ipsi;
  v[0] = u[0]; v[1] = u[1]; v[2] = u[2]; v[3] = du0; v[4] = du1;
  v[5] = u[0] * u[0] * ipsi; v[6] = u[0] * u[1] * ipsi; v[7] = u[1] * u[1] * ipsi;
  qq = pv[4] * ipsi;
}

// ------------------------------------------------------------------------------------
// current / acceleration / momentum-flux deposit with the predictor push, one warp per
// work item.  Every particle of an item sits in the same cell, so all of them deposit to
// the same two nodes: per mode, each lane accumulates its particles' 32 values
// [node 0/1][Re/Im][cu 0..2, acu 3..4, amu 5..7] in registers, one butterfly sums them
// over the warp, and each lane adds one total into the FP64 arrays.
// ------------------------------------------------------------------------------------
template <int kPPL, int kM>
__global__ void __launch_bounds__(kItemThreads) k_mamjdp(GridDev G, int push_type, float qbm, float dt,
                                                         const int4* __restrict__ items, const int* __restrict__ n_items,
                                                         MArr A, const float* __restrict__ T, double* __restrict__ cu,
                                                         double* __restrict__ amu, double* __restrict__ acu,
                                                         int write_back, const int* __restrict__ guard) {
  if (guard && *guard) return;                         // a part of an unrolled loop body after the loop ended
  // the field iteration launched after this kernel may start its own staging now
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int it = blockIdx.x * (kItemThreads / 32) + w;
  // the item and the item count in flight together (the item list holds whole CTAs' worth)
  const int n_it = *n_items;
  const int4 item = items[it];
  if (it >= n_it) return;                              // warp-uniform
  const int key = item.x, start = item.y, cnt = item.z;
  const int ld = G.ld;
  // every particle of an item sits in radial cell `key`: the two gather records (nodes key,
  // key + 1) load with the particles, then go to this warp's shared slot
  constexpr int kTV = (12 * QPAD_MAX_PARTS + 31) / 32;
  __shared__ float tsm[kItemThreads / 32][12 * QPAD_MAX_PARTS];
  __shared__ float2 tpair[kItemThreads / 32][6 * QPAD_MAX_PARTS];
  const int PP = kM >= 0 ? 2 * kM + 1 : G.P;
  const int nt = 12 * PP;
  const float* tb = T + (size_t)min(key, G.nr) * G.P * 6;
  float tv[kTV];
#pragma unroll
  for (int q = 0; q < kTV; ++q) tv[q] = lane + 32 * q < nt ? __ldg(tb + lane + 32 * q) : 0.0f;
  int32_t pcx[kPPL];
  float pf[kPPL][2], pv[kPPL][5];
#pragma unroll
  for (int j = 0; j < kPPL; ++j) {
    const int o = j * 32 + lane;
    const bool in = o < cnt;
    const int i = start + (in ? o : 0);
    pcx[j] = in ? A.cxy[i] : 0;
    pf[j][0] = in ? A.fx[i] : 0.0f;
    pf[j][1] = in ? A.fy[i] : 0.0f;
    pv[j][0] = in ? A.px[i] : 0.0f;
    pv[j][1] = in ? A.py[i] : 0.0f;
    pv[j][2] = in ? A.pz[i] : 0.0f;
    pv[j][3] = in ? A.psi[i] : 0.0f;
    pv[j][4] = in ? A.q[i] : 0.0f;
  }
#pragma unroll
  for (int q = 0; q < kTV; ++q)
    if (lane + 32 * q < nt) tsm[w][lane + 32 * q] = tv[q];
  __syncwarp();
  for (int l = lane; l < 6 * PP; l += 32) {
    const float a = tsm[w][l], b = tsm[w][6 * PP + l];
    tpair[w][l] = make_float2(a, b - a);
  }
  __syncwarp();
  float v[kPPL][8], wq[kPPL][2], pc[kPPL][2];
#pragma unroll
  for (int j = 0; j < kPPL; ++j) {
    const int o = j * 32 + lane;
    wq[j][0] = wq[j][1] = 0.0f;
    pc[j][0] = 1.0f;
    pc[j][1] = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; ++c) v[j][c] = 0.0f;
    if (o < cnt) {
      const int i = start + o;
      const MInterp ii = minterp(pcx[j], pf[j][0], pf[j][1], G.nr);
      if (ii.ok) {
        float qq, ep[3], bp[3];
        if (ii.idx == key)
          mgather_pair<kM>(&tpair[w][0], G.M, ii, ep, bp);
        else      // (not reached: the sort key and the gather use the same cell_radius)
          mgather_at<kM>(T + (size_t)ii.idx * G.P * 6, G.P, G.M, ii, ep, bp);
        mpredict(push_type, qbm, dt, A, i, write_back, ii, ep, bp, pv[j], v[j], qq);
        wq[j][0] = qq * ii.w0;
        wq[j][1] = qq * ii.w1;
        pc[j][0] = ii.pcos;
        pc[j][1] = -ii.psin;
      }
    }
  }
  float ph[kPPL][2];
#pragma unroll
  for (int j = 0; j < kPPL; ++j) { ph[j][0] = 1.0f; ph[j][1] = 0.0f; }
  const int jn = lane >> 4, h = (lane >> 3) & 1, c = lane & 7;
  double* dst = c < 3 ? cu + (size_t)c * ld : (c < 5 ? acu + (size_t)(c - 3) * ld : amu + (size_t)(c - 5) * ld);
  const int ncomp = c < 3 ? 3 : (c < 5 ? 2 : 3);
  // the mode loop is not unrolled: one copy of the accumulation and butterfly keeps the
  // kernel's code small enough for the instruction cache (measured on the c5 shape: 3.5 %
  // shorter 3D step with two particles per lane, whose tuning this makes the fastest)
  const int mlast = kM >= 0 ? kM : G.M;
#pragma unroll 1
  for (int m = 0; m <= mlast; ++m) {
    float acc[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) acc[k] = 0.0f;
#pragma unroll
    for (int j = 0; j < kPPL; ++j) {
      if (m > 0) {
        const float t = ph[j][0] * pc[j][0] - ph[j][1] * pc[j][1];
        ph[j][1] = ph[j][0] * pc[j][1] + ph[j][1] * pc[j][0];
        ph[j][0] = t;
      }
#pragma unroll
      for (int n = 0; n < 2; ++n) {
        const float cre = wq[j][n] * ph[j][0], cim = wq[j][n] * ph[j][1];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          acc[n * 16 + k] += cre * v[j][k];
          acc[n * 16 + 8 + k] += cim * v[j][k];
        }
      }
    }
    butterfly32(acc, lane);
    if (!(m == 0 && h == 1) && acc[0] != 0.0f) {
      const int p = m == 0 ? 0 : 2 * m - 1 + h;
      atomicAdd(dst + (size_t)p * ncomp * ld + key + jn, (double)acc[0]);
    }
  }
}

// ------------------------------------------------------------------------------------
// push_u + push_x + edge test + new cell key
// ------------------------------------------------------------------------------------
template <int kM>
__global__ void __launch_bounds__(kMixThreads) k_mpush(GridDev G, int push_type, float qbm, float dt,
                                                       const int64_t* __restrict__ n_ptr, MArr A,
                                                       const float* __restrict__ T, int do_u, int do_x) {
  const int64_t n = *n_ptr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float qtmh = qbm * dt * 0.5f;
  int ix, iy;
  unpack_cell(A.cxy[i], ix, iy);
  float fx = A.fx[i], fy = A.fy[i];
  float p[3] = {A.px[i], A.py[i], A.pz[i]};
  float g = A.gam[i];
  if (do_u) {
  const MInterp ii = minterp(A.cxy[i], fx, fy, G.nr);
  float ep[3], bp[3], ut[3];
  mgather<kM>(T, G.P, G.M, ii, ep, bp);
  float t = ep[0] * ii.pcos - ep[1] * ii.psin;
  ep[1] = ep[0] * ii.psin + ep[1] * ii.pcos;
  ep[0] = t;
  t = bp[0] * ii.pcos - bp[1] * ii.psin;
  bp[1] = bp[0] * ii.psin + bp[1] * ii.pcos;
  bp[0] = t;
  float qtmh1, qtmh2;
  if (push_type == QPAD_PUSH2_ROBUST) {
    const float gam = sqrtf(1.0f + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    qtmh1 = qtmh / gamma_minus_uz(p[0], p[1], p[2], gam);
    qtmh2 = qtmh1 * gam;
  } else {
    qtmh1 = qtmh / (1.0f - qbm * A.psi[i]);
    qtmh2 = qtmh1 * g;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) { ep[c] *= qtmh2; bp[c] *= qtmh1; ut[c] = p[c] + ep[c]; }
  p[0] = ut[0] + ut[1] * bp[2] - ut[2] * bp[1];
  p[1] = ut[1] + ut[2] * bp[0] - ut[0] * bp[2];
  p[2] = ut[2] + ut[0] * bp[1] - ut[1] * bp[0];
  const float ostq = 2.0f / (1.0f + bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
#pragma unroll
  for (int c = 0; c < 3; ++c) bp[c] *= ostq;
  {
    const float t0 = ut[0] + p[1] * bp[2] - p[2] * bp[1];
    const float t1 = ut[1] + p[2] * bp[0] - p[0] * bp[2];
    const float t2 = ut[2] + p[0] * bp[1] - p[1] * bp[0];
    p[0] = t0 + ep[0]; p[1] = t1 + ep[1]; p[2] = t2 + ep[2];
  }
  g = sqrtf(1.0f + p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
  A.px[i] = p[0]; A.py[i] = p[1]; A.pz[i] = p[2];
  A.gam[i] = g;
  }
  if (!do_x) return;
  // x += p dt / (gamma - pz), in cell units, renormalising the offset into [0,1)
  const float dtc = dt / gamma_minus_uz(p[0], p[1], p[2], g) * (float)G.idr;
  fx += p[0] * dtc;
  fy += p[1] * dtc;
  const float sx = floorf(fx), sy = floorf(fy);
  ix += (int)sx; fx -= sx;
  iy += (int)sy; fy -= sy;
  if (fx >= 1.0f) { fx -= 1.0f; ix += 1; }
  if (fy >= 1.0f) { fy -= 1.0f; iy += 1; }
  const bool inside = ix > -32000 && ix < 32000 && iy > -32000 && iy < 32000;
  const float X = (float)ix + fx, Y = (float)iy + fy;
  int K = G.nr;
  float d;
  if (inside) cell_radius(ix, iy, fx, fy, sqrtf(X * X + Y * Y), K, d);
  const bool alive = inside && K < G.nr;
  A.cxy[i] = pack_cell(alive ? ix : 0, alive ? iy : 0);
  A.fx[i] = fx;
  A.fy[i] = fy;
  A.key[i] = alive ? K + 1 : G.nr + 1;
}

// ------------------------------------------------------------------------------------
// counting sort by key (1..nr, nr+1 = removed); order inside a cell is not kept
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kMixThreads) k_mhist(const int64_t* __restrict__ n_ptr, const int32_t* __restrict__ key,
                                                       int32_t* __restrict__ hist) {
  const int64_t n = *n_ptr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  const int k = valid ? key[i] : -1;
  const unsigned grp = __match_any_sync(FULL, k);
  const int lane = threadIdx.x & 31;
  if (valid && (grp & ((1u << lane) - 1u)) == 0) atomicAdd(hist + k, __popc(grp));
}

// Exclusive scan of the cell histogram into the scatter cursors and the cell starts, and
// the deposit work items: cell k (1..nr) of n_k particles becomes ceil(n_k / kItem) items
// {k, first particle, count}.  One CTA.
__global__ void __launch_bounds__(1024) k_mscan(int nk, int nr, const int32_t* __restrict__ hist,
                                                int32_t* __restrict__ cursor, int64_t* __restrict__ n_ptr,
                                                int dead_key, int4* __restrict__ items, int* __restrict__ n_items,
                                                int kItem) {
  __shared__ int sh[64], shi[64];
  int carry = 0, carry_i = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int base = 0; base < nk; base += blockDim.x) {
    const int k = base + threadIdx.x;
    const int v = k < nk ? hist[k] : 0;
    const int ni = (k >= 1 && k <= nr) ? (v + kItem - 1) / kItem : 0;
    int x = v, xi = ni;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int o = __shfl_up_sync(FULL, x, off), oi = __shfl_up_sync(FULL, xi, off);
      if (lane >= off) { x += o; xi += oi; }
    }
    if (lane == 31) { sh[warp] = x; shi[warp] = xi; }
    __syncthreads();
    if (warp == 0) {
      int w = lane < nw ? sh[lane] : 0, wi = lane < nw ? shi[lane] : 0;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int o = __shfl_up_sync(FULL, w, off), oi = __shfl_up_sync(FULL, wi, off);
        if (lane >= off) { w += o; wi += oi; }
      }
      sh[32 + lane] = w;
      shi[32 + lane] = wi;
    }
    __syncthreads();
    const int before = warp > 0 ? sh[32 + warp - 1] : 0, before_i = warp > 0 ? shi[32 + warp - 1] : 0;
    const int tot = sh[32 + nw - 1], tot_i = shi[32 + nw - 1];
    const int ex = carry + before + x - v, exi = carry_i + before_i + xi - ni;
    if (k < nk) cursor[k] = ex;
    if (k == dead_key) *n_ptr = ex;                   // particles before the removed bucket
    for (int j = 0; j < ni; ++j) items[exi + j] = make_int4(k, ex + j * kItem, min(kItem, v - j * kItem), 0);
    carry += tot;
    carry_i += tot_i;
    __syncthreads();
  }
  if (threadIdx.x == 0) *n_items = carry_i;
}

__global__ void __launch_bounds__(kMixThreads) k_mscatter(const int64_t* __restrict__ n_old, MArr S, MArr D,
                                                          int32_t* __restrict__ cursor) {
  const int64_t n = *n_old;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  const int k = valid ? S.key[i] : -1;
  const unsigned grp = __match_any_sync(FULL, k);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(grp) - 1;
  int base = 0;
  if (valid && lane == leader) base = atomicAdd(cursor + k, __popc(grp));
  base = __shfl_sync(FULL, base, leader);
  if (!valid) return;
  const int d = base + __popc(grp & ((1u << lane) - 1u));
  D.cxy[d] = S.cxy[i]; D.fx[d] = S.fx[i]; D.fy[d] = S.fy[i];
  D.px[d] = S.px[i]; D.py[d] = S.py[i]; D.pz[d] = S.pz[i];
  D.q[d] = S.q[i]; D.gam[d] = S.gam[i]; D.psi[d] = S.psi[i];
  D.key[d] = k;
}

__global__ void k_copy_count(const int64_t* __restrict__ a, int64_t* __restrict__ b) { *b = *a; }

// ------------------------------------------------------------------------------------
// conversions
// ------------------------------------------------------------------------------------
__global__ void k_to_mixed(GridDev G, const int64_t* __restrict__ n_ptr, const double* __restrict__ x,
                           const double* __restrict__ y, const double* __restrict__ px, const double* __restrict__ py,
                           const double* __restrict__ pz, const double* __restrict__ gam,
                           const double* __restrict__ psi, const double* __restrict__ q, MArr A) {
  const int64_t n = *n_ptr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double tx = x[i] * G.idr, ty = y[i] * G.idr;
  const double sx = floor(tx), sy = floor(ty);
  float fx = (float)(tx - sx), fy = (float)(ty - sy);
  int ix = (int)sx, iy = (int)sy;
  if (fx >= 1.0f) { fx -= 1.0f; ix += 1; }
  if (fy >= 1.0f) { fy -= 1.0f; iy += 1; }
  A.cxy[i] = pack_cell(ix, iy);
  A.fx[i] = fx;
  A.fy[i] = fy;
  A.px[i] = (float)px[i]; A.py[i] = (float)py[i]; A.pz[i] = (float)pz[i];
  A.gam[i] = (float)gam[i]; A.psi[i] = (float)psi[i]; A.q[i] = (float)q[i];
  const float X = (float)ix + fx, Y = (float)iy + fy;
  int K;
  float d;
  cell_radius(ix, iy, fx, fy, sqrtf(X * X + Y * Y), K, d);
  // a particle handed in beyond the edge is kept (the reference removes particles only in
  // update_bound after a push); it sorts into the last cell and deposits nothing
  A.key[i] = K < G.nr ? K + 1 : G.nr;
}

__global__ void k_to_fp64(GridDev G, const int64_t* __restrict__ n_ptr, MArr A, double* __restrict__ x,
                          double* __restrict__ y, double* __restrict__ px, double* __restrict__ py,
                          double* __restrict__ pz, double* __restrict__ gam, double* __restrict__ psi,
                          double* __restrict__ q) {
  const int64_t n = *n_ptr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int ix, iy;
  unpack_cell(A.cxy[i], ix, iy);
  x[i] = ((double)ix + (double)A.fx[i]) * G.dr;
  y[i] = ((double)iy + (double)A.fy[i]) * G.dr;
  px[i] = A.px[i]; py[i] = A.py[i]; pz[i] = A.pz[i];
  gam[i] = A.gam[i]; psi[i] = A.psi[i]; q[i] = A.q[i];
}

__global__ void __launch_bounds__(kMixThreads) k_minterp_psi(GridDev G, const int64_t* __restrict__ n_ptr, MArr A,
                                                             const double* __restrict__ psif) {
  const int64_t n = *n_ptr;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const MInterp ii = minterp(A.cxy[i], A.fx[i], A.fy[i], G.nr);
  if (!ii.ok) { A.psi[i] = 0.0f; return; }
  const int i0 = ii.idx;
  float v = (float)psif[i0] * ii.w0 + (float)psif[i0 + 1] * ii.w1;
  float phr = 1.0f, phi = 0.0f;
  for (int m = 1; m <= G.M; ++m) {
    const float t = phr * ii.pcos - phi * ii.psin;
    phi = phr * ii.psin + phi * ii.pcos;
    phr = t;
    const double* fr = psif + (size_t)(2 * m - 1) * G.ld + i0;
    const double* fi = psif + (size_t)(2 * m) * G.ld + i0;
    v += ((float)fr[0] * 2.0f * phr - (float)fi[0] * 2.0f * phi) * ii.w0 +
         ((float)fr[1] * 2.0f * phr - (float)fi[1] * 2.0f * phi) * ii.w1;
  }
  A.psi[i] = v;
}

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
// the instance for the grid's highest mode: compile-time M for 0..4, run-time M above
#define QPAD_MIXED_BY_MODE(M, LAUNCH) \
  do {                                \
    switch (M) {                      \
      case 0: LAUNCH(0); break;       \
      case 1: LAUNCH(1); break;       \
      case 2: LAUNCH(2); break;       \
      case 3: LAUNCH(3); break;       \
      case 4: LAUNCH(4); break;       \
      default: LAUNCH(-1); break;     \
    }                                 \
  } while (0)
int mixed_alloc(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  const size_t cap = (size_t)sp->npmax;
  const size_t per = cap * (sizeof(int32_t) * 2 + sizeof(float) * 8);   // cxy, key, 8 floats
  void* blk = nullptr;
  cudaError_t e = cudaMalloc(&blk, 2 * per + 256);
  if (e != cudaSuccess) { cudaGetLastError(); return set_err(ctx, QPAD_E_NOMEM, "cudaMalloc(mixed particles)"); }
  sp->mixed_block = blk;
  char* p = (char*)blk;
  for (int b = 0; b < 2; ++b) {
    sp->cxy[b] = (int32_t*)p; p += cap * sizeof(int32_t);
    sp->mkey[b] = (int32_t*)p; p += cap * sizeof(int32_t);
    float** fs[8] = {&sp->fx[b], &sp->fy[b], &sp->mpx[b], &sp->mpy[b], &sp->mpz[b], &sp->mq[b], &sp->mgam[b],
                     &sp->mpsi[b]};
    for (int a = 0; a < 8; ++a) { *fs[a] = (float*)p; p += cap * sizeof(float); }
  }
  e = cudaMalloc(&sp->mixed_pristine, per + 256);
  if (e != cudaSuccess) { cudaGetLastError(); return set_err(ctx, QPAD_E_NOMEM, "cudaMalloc(mixed pristine)"); }
  e = cudaMalloc(&sp->hist, sizeof(int32_t) * (ctx->g.nr + 4));
  if (e == cudaSuccess) e = cudaMalloc(&sp->cursor, sizeof(int32_t) * (ctx->g.nr + 4));
  sp->items_cap = ((int64_t)(cap / kMinItem) + ctx->g.nr + 2 + kItemThreads / 32 - 1) / (kItemThreads / 32) *
                  (kItemThreads / 32);                  // whole CTAs: every warp may load its item
  if (e == cudaSuccess) e = cudaMalloc(&sp->items, sizeof(int4) * (size_t)sp->items_cap);
  if (e == cudaSuccess) e = cudaMalloc(&sp->d_nitems, sizeof(int) * 2);
  if (e == cudaSuccess) e = cudaMemset(sp->d_nitems, 0, sizeof(int) * 2);
  if (e != cudaSuccess) { cudaGetLastError(); return set_err(ctx, QPAD_E_NOMEM, "cudaMalloc(mixed sort)"); }
  return 0;
}

void mixed_free(qpad_species* sp) {
  if (sp->mixed_block) cudaFree(sp->mixed_block);
  if (sp->mixed_pristine) cudaFree(sp->mixed_pristine);
  if (sp->hist) cudaFree(sp->hist);
  if (sp->cursor) cudaFree(sp->cursor);
  if (sp->items) cudaFree(sp->items);
  if (sp->d_nitems) cudaFree(sp->d_nitems);
  sp->mixed_block = sp->mixed_pristine = nullptr;
  sp->hist = sp->cursor = nullptr;
  sp->items = nullptr;
  sp->d_nitems = nullptr;
}


// sorts the mixed state by key; the new count (without removed particles) lands in d_count
static int mixed_sort(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  const int64_t n = sp->np;
  if (n == 0) return 0;
  const int nk = ctx->g.nr + 2;
  if (cudaMemsetAsync(sp->hist, 0, sizeof(int32_t) * nk, ctx->stream) != cudaSuccess) return check_launch(ctx, "hist0", 0);
  k_mhist<<<mgrid(n, kMixThreads), kMixThreads, 0, ctx->stream>>>(sp->d_count, sp->mkey[0], sp->hist);
  k_copy_count<<<1, 1, 0, ctx->stream>>>(sp->d_count, sp->d_total);      // old count for the scatter
  k_mscan<<<1, 1024, 0, ctx->stream>>>(nk, ctx->g.nr, sp->hist, sp->cursor, sp->d_count, ctx->g.nr + 1, sp->items,
                                       sp->d_nitems, 32 * ctx->item_ppl);
  k_mscatter<<<mgrid(n, kMixThreads), kMixThreads, 0, ctx->stream>>>(sp->d_total, marr(sp, 0), marr(sp, 1),
                                                                      sp->cursor);
  if (int r = check_launch(ctx, "mixed sort", 4)) return r;
  // copy the sorted half back into place (the two halves are contiguous blocks of 10
  // arrays), so that kernels captured in a CUDA graph keep valid arguments
  return cuda_check(ctx, cudaMemcpyAsync(sp->cxy[0], sp->cxy[1], (size_t)sp->npmax * 40, cudaMemcpyDeviceToDevice,
                                         ctx->stream), "mixed copy back");
}

// Rebuilds the deposit work items of a state that is already sorted by cell.
int mixed_index(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  const int64_t n = sp->np;
  if (n == 0) return 0;
  const int nk = ctx->g.nr + 2;
  if (cudaMemsetAsync(sp->hist, 0, sizeof(int32_t) * nk, ctx->stream) != cudaSuccess) return check_launch(ctx, "hist0", 0);
  k_mhist<<<mgrid(n, kMixThreads), kMixThreads, 0, ctx->stream>>>(sp->d_count, sp->mkey[0], sp->hist);
  k_mscan<<<1, 1024, 0, ctx->stream>>>(nk, ctx->g.nr, sp->hist, sp->cursor, sp->d_count, ctx->g.nr + 1, sp->items,
                                       sp->d_nitems, 32 * ctx->item_ppl);
  return check_launch(ctx, "mixed index", 2);
}

static int item_blocks(const qpad_species* sp) {
  const int64_t bound = sp->np / (32 * sp->ctx->item_ppl) + sp->ctx->g.nr + 2;   // >= sum over cells of ceil(n_k / item)
  return (int)((std::min<int64_t>(bound, sp->items_cap) + kItemThreads / 32 - 1) / (kItemThreads / 32));
}

int mixed_from_fp64(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  k_to_mixed<<<mgrid(sp->np, kMixThreads), kMixThreads, 0, ctx->stream>>>(
      ctx->g, sp->d_count, sp->x[0], sp->y[0], sp->px[0], sp->py[0], sp->pz[0], sp->gamma[0], sp->psi[0], sp->q[0],
      marr(sp, 0));
  if (int r = check_launch(ctx, "to mixed")) return r;
  return mixed_sort(sp);
}

int mixed_to_fp64(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  k_to_fp64<<<mgrid(sp->np, kMixThreads), kMixThreads, 0, ctx->stream>>>(
      ctx->g, sp->d_count, marr(sp, 0), sp->x[0], sp->y[0], sp->px[0], sp->py[0], sp->pz[0], sp->gamma[0],
      sp->psi[0], sp->q[0]);
  return check_launch(ctx, "to fp64");
}

int mixed_save_pristine(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  const size_t cap = (size_t)sp->npmax;
  char* p = (char*)sp->mixed_pristine;
  const void* src[10] = {sp->cxy[0], sp->mkey[0], sp->fx[0], sp->fy[0], sp->mpx[0], sp->mpy[0],
                         sp->mpz[0], sp->mq[0],   sp->mgam[0], sp->mpsi[0]};
  for (int a = 0; a < 10; ++a) {
    if (cudaMemcpyAsync(p + a * cap * 4, src[a], cap * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
      return check_launch(ctx, "mixed pristine", 0);
  }
  return 0;
}

int mixed_restore_pristine(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  const size_t cap = (size_t)sp->npmax;
  const char* p = (const char*)sp->mixed_pristine;
  void* dst[10] = {sp->cxy[0], sp->mkey[0], sp->fx[0], sp->fy[0], sp->mpx[0], sp->mpy[0],
                   sp->mpz[0], sp->mq[0],   sp->mgam[0], sp->mpsi[0]};
  for (int a = 0; a < 10; ++a) {
    if (cudaMemcpyAsync(dst[a], p + a * cap * 4, cap * 4, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
      return check_launch(ctx, "mixed restore", 0);
  }
  return 0;
}

int mixed_qdeposit_raw(qpad_species* sp, double* qraw) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  prof_begin(ctx, "qdeposit");
#define QPAD_MQDEP(PPL, MM) \
  k_mqdeposit<PPL, MM><<<item_blocks(sp), kItemThreads, 0, ctx->stream>>>(ctx->g, sp->items, sp->d_nitems, marr(sp, 0), qraw)
#define QPAD_MQDEP_M(MM) \
  do { if (ctx->item_ppl == 1) QPAD_MQDEP(1, MM); else if (ctx->item_ppl == 2) QPAD_MQDEP(2, MM); else QPAD_MQDEP(4, MM); } while (0)
  QPAD_MIXED_BY_MODE(ctx->g.M, QPAD_MQDEP_M);
#undef QPAD_MQDEP_M
#undef QPAD_MQDEP
  prof_end(ctx, "qdeposit");
  return check_launch(ctx, "k_mqdeposit");
}

int mixed_amjdp_raw(qpad_species* sp, const float* gtab, double* cu, double* amu, double* acu, double dt) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  prof_begin(ctx, "amjdp");
#define QPAD_MAMJ(PPL, MM)                                                                                        \
  k_mamjdp<PPL, MM><<<item_blocks(sp), kItemThreads, 0, ctx->stream>>>(ctx->g, sp->push_type, (float)sp->qbm,     \
                                                                      (float)dt, sp->items, sp->d_nitems,         \
                                                                      marr(sp, 0), gtab, cu, amu, acu, 0,         \
                                                                      iter_guard(ctx))
#define QPAD_MAMJ_M(MM) \
  do { if (ctx->item_ppl == 1) QPAD_MAMJ(1, MM); else if (ctx->item_ppl == 2) QPAD_MAMJ(2, MM); else QPAD_MAMJ(4, MM); } while (0)
  QPAD_MIXED_BY_MODE(ctx->g.M, QPAD_MAMJ_M);
#undef QPAD_MAMJ_M
#undef QPAD_MAMJ
  prof_end(ctx, "amjdp");
  return check_launch(ctx, "k_mamjdp");
}

int mixed_push(qpad_species* sp, const float* gtab, double dt, int do_u, int do_x) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  prof_begin(ctx, "push");
#define QPAD_MPUSH(MM)                                                                                 \
  k_mpush<MM><<<mgrid(sp->np, kMixThreads), kMixThreads, 0, ctx->stream>>>(                            \
      ctx->g, sp->push_type, (float)sp->qbm, (float)dt, sp->d_count, marr(sp, 0), gtab, do_u, do_x)
  QPAD_MIXED_BY_MODE(ctx->g.M, QPAD_MPUSH);
#undef QPAD_MPUSH
  prof_end(ctx, "push");
  if (int r = check_launch(ctx, "k_mpush")) return r;
  return do_x ? mixed_sort(sp) : 0;
}

int mixed_sort_public(qpad_species* sp) { return mixed_sort(sp); }

int mixed_interp_psi(qpad_species* sp, const double* psif) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  k_minterp_psi<<<mgrid(sp->np, kMixThreads), kMixThreads, 0, ctx->stream>>>(ctx->g, sp->d_count, marr(sp, 0), psif);
  return check_launch(ctx, "k_minterp_psi");
}

}  // namespace qpad
