// laser.cu -- laser envelopes and the plasma pushers that see them, FP64 path.
//
// The reference models a laser pulse by the envelope a = a_r + i a_i of its vector
// potential (ponderomotive guiding centre, "PGC"; laser/field_laser_class.f03,
// sim_lasers_class.f03):
//   * per slice, the sum of every laser's envelope and of its gradients (r, phi, xi) is
//     formed (copy_slice, set_grad :637-750, gather :929-946) and the PGC species gather
//     them: |a|^2 raises gamma and its gradient adds the ponderomotive force
//     (amjdeposit_robust_pgc / _std_pgc, part2d_class.f03:1012-1602; push_u_*_pgc
//     :1967-2219);
//   * after the iteration of every slice the plasma susceptibility chi = -qbm q / (1 - qbm psi)
//     of each species is deposited into a store (deposit_chi, part2d_class.f03:361-476);
//   * after the slice loop the envelope advances by one 3D step: an explicit half for every
//     slice (set_rhs :393-635), then slice by slice from the front of the box an implicit half
//     per mode and Re / Im part, a penta-diagonal system of the 2 nr unknowns (a_r, a_i) of the
//     nodes, solved by parallel cyclic reduction with precomputed coefficients
//     (solve :752-927; fpcr_penta_class.f03).
//
// Layouts: envelope store lr2 / li2 [(nz + 3)][P][ld], slice j (-1..nz+1) at index j + 1 (the
// two slices ahead of the box stay zero); explicit half sr / si [nz][P][ld]; the slice sum
// la = [a_r | a_i | grad a_r (3 comps) | grad a_i (3 comps)], each [P][ld] per component;
// chi [P][ld], its store chi2 [nz][P][ld]; PCR tables per mode m [cm1 | cm2 | cp1 | cp2 |
// cfin], the first four [steps][n] and cfin [n], n = 2 nr, row 2i-1 / 2i the a_r / a_i of
// node i.
//
// The implicit half runs as one thread-block cluster per laser with one CTA per mode: each
// iteration of a slice first forms every mode's coupling through chi (which reads all modes'
// envelope), then, after a cluster barrier, each CTA solves its mode's systems and writes
// its envelope; a second barrier precedes the next coupling.  Cluster barriers are hardware
// barriers of co-scheduled CTAs: the kernel has no spin-waits.
#include <cooperative_groups.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "particles.cuh"
#include "qpad_internal.cuh"

namespace cg = cooperative_groups;

struct qpad_laser {
  qpad_ctx* ctx = nullptr;
  double k0 = 10.0;
  int iter = 1, steps = 0, n = 0;
  double* lr2 = nullptr;
  double* li2 = nullptr;
  double* sr = nullptr;
  double* si = nullptr;
  double* coef = nullptr;
};

namespace qpad {

static constexpr int kSolveThreads = 512;
static constexpr int kMaxLasers = 4;
static constexpr int kPartThreads = 256;

// ---- host: the penta-diagonal operator and its reduction tables ---------------------------
// init_solver (field_laser_class.f03:269-391) on one rank, with set_values_matrix_byrow's
// machine-epsilon entries at the couplings that leave the system (fpcr_penta_class.f03:570-595).
static void laser_matrix(int nr, int m, double k0, double ds, double dr, double dz, double* a, double* b, double* c,
                         double* d, double* e) {
  const int n = 2 * nr;
  const double eps = 2.220446049250313e-16;
  const double ds_qtr = 0.25 * ds, dr2_idz_1hf = 1.5 * (dr * dr) / dz, kap = k0 * (dr * dr);
  const double m2 = (double)(m * m);
  auto set = [&](int r, double A, double B, double C, double D, double E) {
    a[r - 1] = A; b[r - 1] = B; c[r - 1] = C; d[r - 1] = D; e[r - 1] = E;
    if (r == 1) { a[0] = eps; b[0] = eps; }
    else if (r == 2) a[1] = eps;
    if (r == n) { e[n - 1] = eps; d[n - 1] = eps; }
    else if (r == n - 1) e[n - 2] = eps;
  };
  for (int i = 3; i <= n - 1; i += 2) {
    const int j = (i + 1) / 2 - 1;
    const double j2 = (double)(j * j);
    const double av = -(ds_qtr * (1.0 - 0.5 / (double)j));
    const double cv = ds_qtr * (2.0 + m2 / j2) + dr2_idz_1hf;
    const double ev = -(ds_qtr * (1.0 + 0.5 / (double)j));
    set(i, av, 0.0, cv, -kap, ev);
    set(i + 1, av, kap, cv, 0.0, ev);
  }
  if (m == 0) {
    set(1, 0.0, eps, ds + dr2_idz_1hf, -kap, -ds);
    set(2, eps, kap, ds + dr2_idz_1hf, 0.0, -ds);
  } else {
    set(1, eps, eps, 1.0, eps, eps);
    set(2, eps, eps, 1.0, eps, eps);
  }
  const int j = nr - 1;
  const double j2 = (double)(j * j);
  const double av = -(ds_qtr * (1.0 - 0.5 / (double)j));
  const double cv = ds_qtr * (2.0 + m2 / j2) + dr2_idz_1hf;
  set(n - 1, av, 0.0, cv, -kap, 0.0);
  set(n, av, kap, cv, 0.0, 0.0);
}

// generate_cr_coef (fpcr_penta_class.f03:288-527) on one rank.  The reduction of the m >= 1
// systems divides by quantities of the order of the epsilon entries, so its tables carry
// large coefficients: they are computed here in the reference's operation order without
// contraction (the library's host code is compiled with -ffp-contract=off), so that the
// device solve applies exactly the reference's reduction.
static void pcr_coef(int n, int steps, std::vector<double>& A5, double* out) {
  double *a = A5.data(), *b = a + n, *c = b + n, *d = c + n, *e = d + n;
  std::vector<double> nw(5 * (size_t)n);
  double *na = nw.data(), *nb = na + n, *nc = nb + n, *nd = nc + n, *ne = nd + n;
  auto row = [&](const double* arr, int k, double pad) { return k >= 1 && k <= n ? arr[k - 1] : pad; };
  for (int s = 1; s <= steps; ++s) {
    const int cs = 1 << (s - 1);
    double* m1 = out + (size_t)(s - 1) * n;
    double* m2 = out + ((size_t)steps + s - 1) * n;
    double* p1 = out + (2 * (size_t)steps + s - 1) * n;
    double* p2 = out + (3 * (size_t)steps + s - 1) * n;
    for (int i = 1; i <= n; ++i) {
      const int im1 = i - cs, ip1 = i + cs, im2 = i - 2 * cs, ip2 = i + 2 * cs;
      const double am1 = row(a, im1, 0.0), bm1 = row(b, im1, 1.0), cm1 = row(c, im1, 2.0), dm1 = row(d, im1, 1.0),
                   em1 = row(e, im1, 0.0);
      const double am2 = row(a, im2, 0.0), bm2 = row(b, im2, 1.0), cm2 = row(c, im2, 2.0), dm2 = row(d, im2, 1.0),
                   em2 = row(e, im2, 0.0);
      const double ap1 = row(a, ip1, 0.0), bp1 = row(b, ip1, 1.0), cp1 = row(c, ip1, 2.0), dp1 = row(d, ip1, 1.0),
                   ep1 = row(e, ip1, 0.0);
      const double ap2 = row(a, ip2, 0.0), bp2 = row(b, ip2, 1.0), cp2 = row(c, ip2, 2.0), dp2 = row(d, ip2, 1.0),
                   ep2 = row(e, ip2, 0.0);
      const double a0 = a[i - 1], b0 = b[i - 1], c0 = c[i - 1], d0 = d[i - 1], e0 = e[i - 1];
      double tmp = am1 * cp1 * dm2 * dp2 - am1 * bp2 * dm2 * ep1 + ap1 * bm2 * dp2 * em1 + bm2 * bp2 * cm1 * ep1 -
                   bm2 * cm1 * cp1 * dp2;
      double km2 = 0.0, km1 = 0.0, kp1 = 0.0, kp2 = 0.0;
      if (std::fabs(tmp) > 1e-40) {
        tmp = 1.0 / tmp;
        km2 = am1 * (ap1 * d0 * dp2 + b0 * bp2 * ep1 - b0 * cp1 * dp2) * tmp;
        km1 = -(bm2 * (ap1 * d0 * dp2 + b0 * bp2 * ep1 - b0 * cp1 * dp2) * tmp);
        kp1 = -(dp2 * (am1 * d0 * dm2 + b0 * bm2 * em1 - d0 * bm2 * cm1) * tmp);
        kp2 = ep1 * (am1 * d0 * dm2 + b0 * bm2 * em1 - d0 * bm2 * cm1) * tmp;
      }
      m1[i - 1] = km1; m2[i - 1] = km2; p1[i - 1] = kp1; p2[i - 1] = kp2;
      na[i - 1] = km2 * am2;
      nb[i - 1] = km2 * cm2 + km1 * bm1 + a0;
      nc[i - 1] = km2 * em2 + km1 * dm1 + c0 + kp1 * bp1 + kp2 * ap2;
      nd[i - 1] = e0 + kp1 * dp1 + kp2 * cp2;
      ne[i - 1] = kp2 * ep2;
    }
    std::memcpy(a, nw.data(), sizeof(double) * 5 * (size_t)n);
  }
  std::memcpy(out + 4 * (size_t)steps * n, c, sizeof(double) * n);
}

// ---- device -------------------------------------------------------------------------------
struct LaserSet {
  const double* lr[kMaxLasers];
  const double* li[kMaxLasers];
  int n;
};

__device__ __forceinline__ int part_of(int m, int im) { return m == 0 ? 0 : (im ? 2 * m : 2 * m - 1); }

// copy_slice + set_grad + gather of slice j (field_laser_class.f03:637-750, 929-946): one
// thread per (part, node).  For m >= 1 the reference's axis branch runs with its loop index
// left at nr + 1, so it writes the upper guard node and leaves node 1's r and phi components
// zero; reproduced for identical results.
__global__ void k_laser_slice(GridDev G, const int* __restrict__ d_j, LaserSet L, double* __restrict__ la) {
  const int P = G.P, ld = G.ld, nr = G.nr;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P * ld) return;
  const int p = t / ld, i = t - p * ld;
  const int j = *d_j;
  const size_t sl = (size_t)P * ld;
  const int m = (p + 1) / 2;
  const bool im = p > 0 && (p % 2) == 0;
  const double idrh = 0.5 / G.dr, idzh = 0.5 / G.dxi;
  double val[2] = {0.0, 0.0}, gr[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
  for (int k = 0; k < L.n; ++k) {
    const double* src[2] = {L.lr[k], L.li[k]};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const double* a = src[h] + (size_t)(j + 1) * sl;
      const double* a1 = a - sl;
      const double* a2 = a1 - sl;
      const size_t o = (size_t)p * ld + i;
      val[h] = val[h] + a[o];
      double c1 = 0.0, c2 = 0.0, c3 = 0.0;
      if (i >= 1 && i <= nr) c3 = idzh * (3.0 * a[o] - 4.0 * a1[o] + a2[o]);
      if (m == 0) {
        if (i >= 2 && i <= nr) c1 = idrh * (a[o + 1] - a[o - 1]);
      } else {
        const size_t pr = (size_t)(2 * m - 1) * ld, pi = (size_t)(2 * m) * ld;
        if (i >= 2 && i <= nr) {
          const double ir = 1.0 / ((double)(i - 1) * G.dr);
          if (!im) {
            c1 = idrh * (a[pr + i + 1] - a[pr + i - 1]);
            c2 = -ir * (double)m * a[pi + i];
          } else {
            c1 = idrh * (a[pi + i + 1] - a[pi + i - 1]);
            c2 = ir * (double)m * a[pr + i];
          }
        } else if (i == nr + 1 && (m & 1)) {
          const double gre = 2.0 * idrh * a[pr + 2], gim = 2.0 * idrh * a[pi + 2];
          c1 = im ? gim : gre;
          c2 = im ? (double)m * gre : -((double)m * gim);
        }
      }
      gr[h][0] = gr[h][0] + c1;
      gr[h][1] = gr[h][1] + c2;
      gr[h][2] = gr[h][2] + c3;
    }
  }
  la[(size_t)p * ld + i] = val[0];
  la[sl + (size_t)p * ld + i] = val[1];
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int c = 0; c < 3; ++c) la[(2 + 3 * h) * sl + ((size_t)p * 3 + c) * ld + i] = gr[h][c];
}

struct LaserF1 {
  const double *ar, *ai, *gr, *gi;
};

__host__ __device__ inline LaserF1 laser_f1(const double* la, const GridDev& G) {
  const size_t sl = (size_t)G.P * G.ld;
  return LaserF1{la, la + sl, la + 2 * sl, la + 5 * sl};
}

// amjdeposit_robust_pgc / _std_pgc (part2d_class.f03:1310-1602, 1012-1308) into the raw
// deposit arrays (finished like the plain deposit).
__global__ void __launch_bounds__(kPartThreads) k_amjdp_pgc(GridDev G, int push_type, double qbm, double dt,
                                                            const int64_t* __restrict__ n_ptr,
                                                            const double* __restrict__ x, const double* __restrict__ y,
                                                            const double* __restrict__ px, const double* __restrict__ py,
                                                            const double* __restrict__ pz, const double* __restrict__ q,
                                                            double* __restrict__ gamma, double* __restrict__ psi,
                                                            const double* __restrict__ ef, const double* __restrict__ bf,
                                                            LaserF1 L, double* __restrict__ cu, double* __restrict__ amu,
                                                            double* __restrict__ acu, const int* __restrict__ guard) {
  if (guard && *guard) return;                 // a part of an unrolled loop body after the loop ended
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const double idt = 1.0 / dt, qtmh = 0.5 * qbm * dt;
  const Interp ii = gen_interp(x[pp], y[pp], G.idr, G.nr);
  double ep[3], bp[3], wp[3], u0[3], u[3], ut[3], gr[3], gi[3];
  gather3(G, ef, ii, ep);
  gather3(G, bf, ii, bp);
  const double apr = gather1(G, L.ar, ii), api = gather1(G, L.ai, ii);
  gather3(G, L.gr, ii, gr);
  gather3(G, L.gi, ii, gi);
  const double gam_corr = 0.5 * (qbm * qbm) * (apr * apr + api * api);
  const double p1 = px[pp], p2 = py[pp];
  u0[0] = p1 * ii.pcos + p2 * ii.psin;
  u0[1] = p2 * ii.pcos - p1 * ii.psin;
  u0[2] = pz[pp];
  const double psi_in = psi[pp];
  double gam = sqrt(1.0 + u0[0] * u0[0] + u0[1] * u0[1] + u0[2] * u0[2] + gam_corr);
  wp[0] = ep[0] - bp[1];
  wp[1] = ep[1] + bp[0];
  wp[2] = ep[2];
  const double tmp = 0.5 * qbm / gam;
  ep[0] = ep[0] - tmp * (apr * gr[0] + api * gi[0]);
  ep[1] = ep[1] - tmp * (apr * gr[1] + api * gi[1]);
  ep[2] = ep[2] + tmp * (apr * gr[2] + api * gi[2]);
  const bool robust = push_type == QPAD_PUSH2_ROBUST_PGC;
  double qtmh_e, qtmh_b;
  if (robust) {
    qtmh_e = qtmh * gam / (gam - u0[2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) ut[c] = u0[c] + ep[c] * qtmh_e;
    gam = sqrt(1.0 + ut[0] * ut[0] + ut[1] * ut[1] + ut[2] * ut[2] + gam_corr);
    qtmh_b = qtmh / (gam - ut[2]);
  } else {
    qtmh_b = qtmh / (1.0 - qbm * psi_in);
    qtmh_e = qtmh_b * gam;
#pragma unroll
    for (int c = 0; c < 3; ++c) ut[c] = u0[c] + ep[c] * qtmh_e;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) bp[c] = bp[c] * qtmh_b;
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
  gam = sqrt(1.0 + ut[0] * ut[0] + ut[1] * ut[1] + ut[2] * ut[2] + gam_corr);
  qtmh_e = robust ? qtmh * gam / (gam - ut[2]) : qtmh_b * gam;
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = ut[c] + ep[c] * qtmh_e;
  double du0 = idt * (u[0] - u0[0]);
  double du1 = idt * (u[1] - u0[1]);
#pragma unroll
  for (int c = 0; c < 3; ++c) u[c] = 0.5 * (u[c] + u0[c]);
  const double g = sqrt(1.0 + u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + gam_corr);
  gamma[pp] = g;
  double ipsi;
  if (robust) {
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
  for (int m = 0; m <= G.M; ++m) {
    if (m > 0) {
      const double t = phr * ph0r - phi * ph0i;
      phi = phr * ph0i + phi * ph0r;
      phr = t;
    }
    const int nh = m == 0 ? 1 : 2;
    for (int h = 0; h < nh; ++h) {
      const int p = part_of(m, h);
      const double ph = h == 0 ? phr : phi;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int nn = n0 + j;
        const double w = wj[j] * ph;
        double* c_ = cu + (size_t)p * 3 * ld + nn;
        double* a_ = acu + (size_t)p * 2 * ld + nn;
        double* m_ = amu + (size_t)p * 3 * ld + nn;
        atomicAdd(c_, w * u[0]);
        atomicAdd(c_ + ld, w * u[1]);
        atomicAdd(c_ + 2 * ld, w * u[2]);
        atomicAdd(a_, w * du0);
        atomicAdd(a_ + ld, w * du1);
        atomicAdd(m_, w * a0);
        atomicAdd(m_ + ld, w * a1);
        atomicAdd(m_ + 2 * ld, w * a2);
      }
    }
  }
}

// push_u_robust_pgc / push_u_std_pgc (part2d_class.f03:1967-2219, the same arithmetic) + push_x
// and the edge test of update_bound.
__global__ void __launch_bounds__(kPartThreads) k_push_pgc(GridDev G, double qbm, double dt,
                                                           const int64_t* __restrict__ n_ptr, double* __restrict__ x,
                                                           double* __restrict__ y, double* __restrict__ px,
                                                           double* __restrict__ py, double* __restrict__ pz,
                                                           double* __restrict__ gamma, const double* __restrict__ psi,
                                                           const double* __restrict__ ef, const double* __restrict__ bf,
                                                           LaserF1 L, int fuse_x, double edge,
                                                           int32_t* __restrict__ alive) {
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const double qtmh = qbm * dt * 0.5, qbm2_hf = (qbm * qbm) * 0.5;
  double xx = x[pp], yy = y[pp];
  const Interp ii = gen_interp(xx, yy, G.idr, G.nr);
  double ep[3], bp[3], gr[3], gi[3], ut[3], p[3];
  gather3(G, ef, ii, ep);
  gather3(G, bf, ii, bp);
  const double apr = gather1(G, L.ar, ii), api = gather1(G, L.ai, ii);
  gather3(G, L.gr, ii, gr);
  gather3(G, L.gi, ii, gi);
  double* vs[4] = {ep, bp, gr, gi};                       // transform_to_cartesian
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double t = vs[k][0] * ii.pcos - vs[k][1] * ii.psin;
    vs[k][1] = vs[k][0] * ii.psin + vs[k][1] * ii.pcos;
    vs[k][0] = t;
  }
  double gam_corr = qbm2_hf * (apr * apr + api * api);
  const double g0 = gamma[pp];
  double tmp = 0.5 * qbm / g0;
  ep[0] = ep[0] - tmp * (apr * gr[0] + api * gi[0]);
  ep[1] = ep[1] - tmp * (apr * gr[1] + api * gi[1]);
  ep[2] = ep[2] + tmp * (apr * gr[2] + api * gi[2]);
  const double qtmh_b = qtmh / (1.0 - qbm * psi[pp]);
  const double qtmh_e = qtmh_b * g0;
  p[0] = px[pp]; p[1] = py[pp]; p[2] = pz[pp];
#pragma unroll
  for (int c = 0; c < 3; ++c) { ep[c] = ep[c] * qtmh_e; ut[c] = p[c] + ep[c]; bp[c] = bp[c] * qtmh_b; }
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
  tmp = gr[2] * dt;
  gam_corr = gam_corr + qbm2_hf * (apr + 0.25 * tmp) * tmp;
  tmp = gi[2] * dt;
  gam_corr = gam_corr + qbm2_hf * (api + 0.25 * tmp) * tmp;
  const double g = sqrt(1.0 + p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + gam_corr);
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

// deposit_chi (part2d_class.f03:361-476): -qbm q / (1 - qbm psi) of every particle into the
// modes of chi with the particle's phase (x - i y) / r; particles beyond the outer edge
// deposit nothing.
__global__ void __launch_bounds__(kPartThreads) k_deposit_chi(GridDev G, double qbm, const int64_t* __restrict__ n_ptr,
                                                              const double* __restrict__ x, const double* __restrict__ y,
                                                              const double* __restrict__ q,
                                                              const double* __restrict__ psi, double* __restrict__ chi) {
  const int64_t n = *n_ptr;
  const int64_t pp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pp >= n) return;
  const double xx = x[pp], yy = y[pp];
  double pos = __dmul_rn(radius_rn(xx, yy), G.idr);
  const double p0r = xx / pos * G.idr, p0i = -yy / pos * G.idr;
  if (!(pos >= 0.0 && pos < (double)G.nr)) return;
  const int nn0 = (int)pos;
  pos = __dsub_rn(pos, (double)nn0);
  const int nn = nn0 + 1;
  const double wt[2] = {1.0 - pos, pos};
  double phr = -(qbm * q[pp] / (1.0 - qbm * psi[pp])), phi = 0.0;
  const size_t ld = G.ld;
  atomicAdd(chi + nn, wt[0] * phr);
  atomicAdd(chi + nn + 1, wt[1] * phr);
  for (int m = 1; m <= G.M; ++m) {
    const double t = phr * p0r - phi * p0i;
    phi = phr * p0i + phi * p0r;
    phr = t;
    double* cr = chi + (size_t)(2 * m - 1) * ld + nn;
    double* ci = chi + (size_t)(2 * m) * ld + nn;
    atomicAdd(cr, wt[0] * phr);
    atomicAdd(cr + 1, wt[1] * phr);
    atomicAdd(ci, wt[0] * phi);
    atomicAdd(ci + 1, wt[1] * phi);
  }
}

// the axis rule and 1/(i-1) of deposit_chi over the whole array; with store, also chi2's slice j
__global__ void k_chi_finish(GridDev G, double corr, double* __restrict__ chi, int store, const int* __restrict__ d_j,
                             double* __restrict__ chi2) {
  const int P = G.P, ld = G.ld;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P * ld) return;
  const int p = t / ld, i = t - p * ld;
  double v = chi[t];
  if (i == 0) v = 0.0;
  else if (i == 1) v = p == 0 ? v * corr : 0.0;
  else v = v * (1.0 / (double)(i - 1));
  chi[t] = v;
  if (store) chi2[(size_t)(*d_j - 1) * P * ld + t] = v;
}

struct LaserDev {
  double* lr2;
  double* li2;
  const double* sr;
  const double* si;
  const double* coef;
  int iter, steps;
  double k0, ds;
};

// the susceptibility coupling of part (m, h) at node i of slice j: the two terms (a_r, a_i)
// added to it, in the reference's order (set_rhs :558-631, solve :795-862)
template <bool kCoherent>
__device__ __forceinline__ void chi_terms(const GridDev& G, const double* chi2, const double* lr2, const double* li2,
                                          int j, int m, int h, int i, double cq, double& tr, double& ti) {
  const int M = G.M, ld = G.ld;
  const size_t sl = (size_t)G.P * ld;
  const double* ch = chi2 + (size_t)(j - 1) * sl + i;
  const double* ar = lr2 + (size_t)(j + 1) * sl + i;
  const double* ai = li2 + (size_t)(j + 1) * sl + i;
  auto ld_ = [](const double* p) { return kCoherent ? __ldcg(p) : *p; };
  if (h == 0) {
    for (int k = m - M; k <= M; ++k) {
      const int ak = k < 0 ? -k : k, amk = m - k < 0 ? k - m : m - k;
      const double sg = (k >= 0 && k <= m) ? 1.0 : -1.0;
      const double cr = ch[(size_t)part_of(ak, 0) * ld];
      tr = tr + cq * cr * ld_(ar + (size_t)part_of(amk, 0) * ld);
      ti = ti + cq * cr * ld_(ai + (size_t)part_of(amk, 0) * ld);
      if (k == 0 || k == m) continue;
      const double ci = ch[(size_t)(2 * ak) * ld];
      tr = tr - cq * sg * ci * ld_(ar + (size_t)(2 * amk) * ld);
      ti = ti - cq * sg * ci * ld_(ai + (size_t)(2 * amk) * ld);
    }
  } else {
    for (int k = m - M; k <= M; ++k) {
      const int ak = k < 0 ? -k : k, amk = m - k < 0 ? k - m : m - k;
      if (k != 0) {
        const double sg = k < 0 ? -1.0 : 1.0;
        const double ci = ch[(size_t)(2 * ak) * ld];
        tr = tr + cq * sg * ci * ld_(ar + (size_t)part_of(amk, 0) * ld);
        ti = ti + cq * sg * ci * ld_(ai + (size_t)part_of(amk, 0) * ld);
      }
      if (k != m) {
        const double sg = k > m ? -1.0 : 1.0;
        const double cr = ch[(size_t)part_of(ak, 0) * ld];
        tr = tr + cq * sg * cr * ld_(ar + (size_t)(2 * amk) * ld);
        ti = ti + cq * sg * cr * ld_(ai + (size_t)(2 * amk) * ld);
      }
    }
  }
}

// set_rhs (field_laser_class.f03:393-635): one thread per (slice, part, node 1..nr)
__global__ void k_laser_rhs(GridDev G, LaserDev L, const double* __restrict__ chi2, double* __restrict__ sr,
                            double* __restrict__ si) {
  const int P = G.P, ld = G.ld, nr = G.nr;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)G.nz * P * nr) return;
  const int i = (int)(t % nr) + 1;
  const int p = (int)((t / nr) % P);
  const int j = (int)(t / ((int64_t)nr * P)) + 1;
  const int m = (p + 1) / 2, h = (p > 0 && p % 2 == 0) ? 1 : 0;
  const double dr = G.dr, dz = G.dxi;
  const double dr2_idzh = 0.5 * (dr * dr) / dz, kap = L.k0 * (dr * dr), ds_qtr = 0.25 * L.ds, cq = ds_qtr * (dr * dr);
  const size_t sl = (size_t)P * ld;
  const double* ar = L.lr2 + (size_t)(j + 1) * sl + (size_t)p * ld;
  const double* ai = L.li2 + (size_t)(j + 1) * sl + (size_t)p * ld;
  double vr = 0.0, vi = 0.0;
  bool stencil = true;
  double bm = 0.0, bp = 0.0, al = 0.0;
  if (i == 1) {
    if (m > 0) stencil = false;
    else { bm = 0.0; bp = L.ds; al = -L.ds; }
  } else {
    const double ik = 1.0 / (double)(i - 1);
    bm = ds_qtr * (1.0 - 0.5 * ik);
    bp = i == nr ? 0.0 : ds_qtr * (1.0 + 0.5 * ik);
    al = m == 0 ? -ds_qtr * 2.0 : -(ds_qtr * (2.0 + (double)(m * m) * ik * ik));
  }
  if (stencil) {
    vr = dr2_idzh * (3.0 * ar[i] - 4.0 * ar[i - sl] + ar[i - 2 * sl]) - kap * ai[i] + bm * ar[i - 1] + al * ar[i] +
         bp * ar[i + 1];
    vi = dr2_idzh * (3.0 * ai[i] - 4.0 * ai[i - sl] + ai[i - 2 * sl]) + kap * ar[i] + bm * ai[i - 1] + al * ai[i] +
         bp * ai[i + 1];
  }
  chi_terms<false>(G, chi2, L.lr2, L.li2, j, m, h, i, cq, vr, vi);
  sr[(size_t)(j - 1) * sl + (size_t)p * ld + i] = vr;
  si[(size_t)(j - 1) * sl + (size_t)p * ld + i] = vi;
}

// solve (field_laser_class.f03:752-927): one cluster per laser, CTA m solves mode m.
// tbuf [M + 1][4][nr]: the coupling terms of the current iteration (phase A), read back by
// the same CTA in phase B.  Shared memory: two rows of n = 2 nr doubles.
__global__ void __launch_bounds__(kSolveThreads) k_laser_solve(GridDev G, LaserDev L, const double* __restrict__ chi2,
                                                               double* __restrict__ tbuf) {
  extern __shared__ double sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int m = (int)cl.block_rank();
  const int nr = G.nr, n = 2 * nr, P = G.P, ld = G.ld, steps = L.steps;
  const size_t sl = (size_t)P * ld;
  const double dr = G.dr, dz = G.dxi;
  const double dr2_idzh = 0.5 * (dr * dr) / dz, cq = 0.25 * L.ds * (dr * dr);
  double* xa = sm;
  double* xb = sm + n;
  double* tb = tbuf + (size_t)m * 4 * nr;
  const double* cf = L.coef + (size_t)m * (4 * (size_t)steps + 1) * n;
  const int nh = m == 0 ? 1 : 2;
  for (int j = 1; j <= G.nz; ++j) {
    for (int l = 1; l <= L.iter; ++l) {
      // phase A: the coupling through chi with every mode's current envelope of slice j
      for (int i = threadIdx.x + 1; i <= nr; i += blockDim.x)
        for (int h = 0; h < nh; ++h) {
          double tr = 0.0, ti = 0.0;
          chi_terms<true>(G, chi2, L.lr2, L.li2, j, m, h, i, cq, tr, ti);
          tb[(2 * h) * nr + i - 1] = tr;
          tb[(2 * h + 1) * nr + i - 1] = ti;
        }
      __threadfence();
      cl.sync();
      // phase B: this mode's systems, Re part then Im part
      for (int h = 0; h < nh; ++h) {
        const int p = part_of(m, h);
        double* ar = L.lr2 + (size_t)(j + 1) * sl + (size_t)p * ld;
        double* ai = L.li2 + (size_t)(j + 1) * sl + (size_t)p * ld;
        const double* srj = L.sr + (size_t)(j - 1) * sl + (size_t)p * ld;
        const double* sij = L.si + (size_t)(j - 1) * sl + (size_t)p * ld;
        for (int i = threadIdx.x + 1; i <= nr; i += blockDim.x) {
          xa[2 * i - 2] = srj[i] + tb[(2 * h) * nr + i - 1] + dr2_idzh * (4.0 * __ldcg(ar + i - sl) - __ldcg(ar + i - 2 * sl));
          xa[2 * i - 1] = sij[i] + tb[(2 * h + 1) * nr + i - 1] +
                          dr2_idzh * (4.0 * __ldcg(ai + i - sl) - __ldcg(ai + i - 2 * sl));
        }
        __syncthreads();
        double* src = xa;
        double* dst = xb;
        for (int s = 0; s < steps; ++s) {
          const int cs = 1 << s;
          const double* k1 = cf + (size_t)s * n;
          const double* k2 = cf + ((size_t)steps + s) * n;
          const double* k3 = cf + (2 * (size_t)steps + s) * n;
          const double* k4 = cf + (3 * (size_t)steps + s) * n;
          for (int i = threadIdx.x; i < n; i += blockDim.x) {
            // the reference's order and rounding (no contraction): the m >= 1 tables hold
            // large coefficients
            double v = src[i];
            v = __dadd_rn(v, __dmul_rn(k1[i], i - cs >= 0 ? src[i - cs] : 0.0));
            v = __dadd_rn(v, __dmul_rn(k2[i], i - 2 * cs >= 0 ? src[i - 2 * cs] : 0.0));
            v = __dadd_rn(v, __dmul_rn(k3[i], i + cs < n ? src[i + cs] : 0.0));
            v = __dadd_rn(v, __dmul_rn(k4[i], i + 2 * cs < n ? src[i + 2 * cs] : 0.0));
            dst[i] = v;
          }
          __syncthreads();
          double* tsw = src; src = dst; dst = tsw;
        }
        const double* cfin = cf + 4 * (size_t)steps * n;
        for (int i = threadIdx.x + 1; i <= nr; i += blockDim.x) {
          ar[i] = __ddiv_rn(src[2 * i - 2], cfin[2 * i - 2]);
          ai[i] = __ddiv_rn(src[2 * i - 1], cfin[2 * i - 1]);
        }
        __syncthreads();
      }
      if (m > 0 && threadIdx.x == 0) {       // on-axis values of m >= 1 are zero
        double* base_r = L.lr2 + (size_t)(j + 1) * sl;
        double* base_i = L.li2 + (size_t)(j + 1) * sl;
        base_r[(size_t)(2 * m - 1) * ld + 1] = 0.0;
        base_i[(size_t)(2 * m - 1) * ld + 1] = 0.0;
        base_r[(size_t)(2 * m) * ld + 1] = 0.0;
        base_i[(size_t)(2 * m) * ld + 1] = 0.0;
      }
      __threadfence();
      cl.sync();
    }
  }
}

static int lmalloc(qpad_ctx* ctx, void** p, size_t bytes, const char* what) {
  if (cudaMalloc(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return set_err(ctx, QPAD_E_NOMEM, what);
  }
  return cuda_check(ctx, cudaMemsetAsync(*p, 0, bytes, ctx->stream), what);
}

static inline int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

// ---- driver hooks ---------------------------------------------------------------------------
int laser_state_ensure(qpad_ctx* ctx) {
  const size_t n1 = (size_t)ctx->g.P * ctx->g.ld;
  if (!ctx->la) {
    if (int r = lmalloc(ctx, (void**)&ctx->la, 8 * n1 * sizeof(double), "laser slice fields")) return r;
  }
  return 0;
}

int laser_slice_prologue(qpad_ctx* ctx) {
  if (ctx->lasers.empty()) return 0;
  LaserSet L{};
  L.n = (int)ctx->lasers.size();
  for (int k = 0; k < L.n; ++k) { L.lr[k] = ctx->lasers[k]->lr2; L.li[k] = ctx->lasers[k]->li2; }
  const int nt = ctx->g.P * ctx->g.ld;
  k_laser_slice<<<blocks_for(nt, 256), 256, 0, ctx->stream>>>(ctx->g, ctx->d_j, L, ctx->la);
  return check_launch(ctx, "k_laser_slice");
}

int laser_amjdp_raw(qpad_species* sp, const double* ef, const double* bf, double* cu, double* amu, double* acu,
                    double dt) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  k_amjdp_pgc<<<blocks_for(sp->np, kPartThreads), kPartThreads, 0, ctx->stream>>>(
      ctx->g, sp->push_type, sp->qbm, dt, sp->d_count, sp->x[0], sp->y[0], sp->px[0], sp->py[0], sp->pz[0], sp->q[0],
      sp->gamma[0], sp->psi[0], ef, bf, laser_f1(ctx->la, ctx->g), cu, amu, acu, iter_guard(ctx));
  return check_launch(ctx, "k_amjdp_pgc");
}

int laser_push_u(qpad_species* sp, const double* ef, const double* bf, double dt, int fuse_x) {
  qpad_ctx* ctx = sp->ctx;
  if (sp->np == 0) return 0;
  const double edge = (double)ctx->g.nr * ctx->g.dr;
  k_push_pgc<<<blocks_for(sp->np, kPartThreads), kPartThreads, 0, ctx->stream>>>(
      ctx->g, sp->qbm, dt, sp->d_count, sp->x[0], sp->y[0], sp->px[0], sp->py[0], sp->pz[0], sp->gamma[0], sp->psi[0],
      ef, bf, laser_f1(ctx->la, ctx->g), fuse_x, edge, sp->key);
  if (int r = check_launch(ctx, "k_push_pgc")) return r;
  return fuse_x ? species_compact(sp) : 0;
}

// lasers%deposit_chi (sim_lasers_class.f03:176-200) for the slice the device index names
int laser_deposit_chi(qpad_ctx* ctx) {
  if (ctx->lasers.empty()) return 0;
  const size_t n1 = (size_t)ctx->g.P * ctx->g.ld;
  if (cudaMemsetAsync(ctx->chi, 0, n1 * sizeof(double), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "chi zero", 0);
  std::vector<qpad_species*> dep;
  for (auto* s : ctx->species)
    if (!s->neut) dep.push_back(s);
  const int nt = (int)n1;
  for (size_t k = 0; k < dep.size(); ++k) {
    qpad_species* s = dep[k];
    if (s->np > 0)
      k_deposit_chi<<<blocks_for(s->np, kPartThreads), kPartThreads, 0, ctx->stream>>>(
          ctx->g, s->qbm, s->d_count, s->x[0], s->y[0], s->q[0], s->psi[0], ctx->chi);
    const double pr = (double)(s->ppc_r * s->ppc_r);
    const double corr = (12.0 * pr) / (1.0 + 2.0 * pr);       // get_deposit_ax_corr, part2d_class.f03:2581-2586
    k_chi_finish<<<blocks_for(nt, 256), 256, 0, ctx->stream>>>(ctx->g, corr, ctx->chi, k + 1 == dep.size() ? 1 : 0,
                                                               ctx->d_j, ctx->chi2);
  }
  if (dep.empty()) {
    k_chi_finish<<<blocks_for(nt, 256), 256, 0, ctx->stream>>>(ctx->g, 0.0, ctx->chi, 1, ctx->d_j, ctx->chi2);
  }
  return check_launch(ctx, "deposit chi", (int)(2 * dep.size() + (dep.empty() ? 1 : 0)));
}

// lasers%advance (sim_lasers_class.f03:202-223) after the slice loop
int lasers_advance(qpad_ctx* ctx) {
  const GridDev& G = ctx->g;
  for (auto* L : ctx->lasers) {
    LaserDev D{L->lr2, L->li2, L->sr, L->si, L->coef, L->iter, L->steps, L->k0, ctx->dt};
    const int64_t nt = (int64_t)G.nz * G.P * G.nr;
    k_laser_rhs<<<(unsigned)((nt + 255) / 256), 256, 0, ctx->stream>>>(G, D, ctx->chi2, L->sr, L->si);
    if (int r = check_launch(ctx, "k_laser_rhs")) return r;
    if (L->iter < 1) continue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(G.M + 1);
    cfg.blockDim = dim3(kSolveThreads);
    cfg.dynamicSmemBytes = 2 * (size_t)L->n * sizeof(double);
    cfg.stream = ctx->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = G.M + 1;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (int r = cuda_check(ctx, cudaLaunchKernelEx(&cfg, k_laser_solve, G, D, (const double*)ctx->chi2, ctx->ltbuf),
                           "k_laser_solve"))
      return r;
    ++ctx->launches;
  }
  return 0;
}

void lasers_free(qpad_ctx* ctx) {
  for (auto* L : ctx->lasers) {
    if (L->lr2) cudaFree(L->lr2);
    if (L->li2) cudaFree(L->li2);
    if (L->sr) cudaFree(L->sr);
    if (L->si) cudaFree(L->si);
    if (L->coef) cudaFree(L->coef);
    delete L;
  }
  ctx->lasers.clear();
  if (ctx->la) cudaFree(ctx->la);
  if (ctx->chi) cudaFree(ctx->chi);
  if (ctx->chi2) cudaFree(ctx->chi2);
  if (ctx->ltbuf) cudaFree(ctx->ltbuf);
  ctx->la = ctx->chi = ctx->chi2 = ctx->ltbuf = nullptr;
}

}  // namespace qpad

using namespace qpad;

extern "C" int qpad_laser_create(qpad_ctx* ctx, const qpad_laser_desc* d, const double* ar, const double* ai,
                                 qpad_laser** out) {
  if (!ctx || !d || !out || !ar || !ai) return QPAD_E_ARG;
  *out = nullptr;
  const GridDev& G = ctx->g;
  if (ctx->precision != QPAD_PREC_FP64) return set_err(ctx, QPAD_E_ARG, "laser: built on the FP64 path only");
  if ((int)ctx->lasers.size() >= kMaxLasers) return set_err(ctx, QPAD_E_CAPACITY, "laser: at most 4 lasers");
  if (G.nr < 4 || (G.nr & (G.nr - 1)) != 0)
    return set_err(ctx, QPAD_E_ARG, "laser: nr must be a power of two (the reduction solves 2 nr unknowns)");
  if (G.M + 1 > 8) return set_err(ctx, QPAD_E_ARG, "laser: at most 7 azimuthal modes");
  if (2 * (size_t)2 * G.nr * sizeof(double) > 200 * 1024) return set_err(ctx, QPAD_E_ARG, "laser: nr too large");
  if (!(d->k0 > 0.0) || d->iter < 0 || d->iter > 64) return set_err(ctx, QPAD_E_ARG, "invalid laser descriptor");
  qpad_laser* L = new (std::nothrow) qpad_laser();
  if (!L) return set_err(ctx, QPAD_E_NOMEM, "laser");
  L->ctx = ctx;
  L->k0 = d->k0;
  L->iter = d->iter;
  L->n = 2 * G.nr;
  while ((1 << L->steps) < L->n) ++L->steps;
  const size_t sl = (size_t)G.P * G.ld;
  const size_t ncoef = (size_t)(G.M + 1) * (4 * (size_t)L->steps + 1) * L->n;
  int r = lmalloc(ctx, (void**)&L->lr2, sizeof(double) * (G.nz + 3) * sl, "laser envelope");
  if (!r) r = lmalloc(ctx, (void**)&L->li2, sizeof(double) * (G.nz + 3) * sl, "laser envelope");
  if (!r) r = lmalloc(ctx, (void**)&L->sr, sizeof(double) * G.nz * sl, "laser right-hand side");
  if (!r) r = lmalloc(ctx, (void**)&L->si, sizeof(double) * G.nz * sl, "laser right-hand side");
  if (!r) r = lmalloc(ctx, (void**)&L->coef, sizeof(double) * ncoef, "laser reduction tables");
  if (!r) r = laser_state_ensure(ctx);
  if (!r && !ctx->chi) r = lmalloc(ctx, (void**)&ctx->chi, sizeof(double) * sl, "chi");
  if (!r && !ctx->chi2) r = lmalloc(ctx, (void**)&ctx->chi2, sizeof(double) * G.nz * sl, "chi store");
  if (!r && !ctx->ltbuf) r = lmalloc(ctx, (void**)&ctx->ltbuf, sizeof(double) * 4 * (G.M + 1) * G.nr, "laser coupling");
  if (!r) {
    // the reduction tables of every mode, and the envelope (slices 1..nz, nodes 1..nr; the
    // on-axis values of m >= 1 are zero, as every solve leaves them)
    std::vector<double> tab(ncoef), A5(5 * (size_t)L->n), env(2 * (G.nz + 3) * sl, 0.0);
    for (int m = 0; m <= G.M; ++m) {
      double* a = A5.data();
      laser_matrix(G.nr, m, d->k0, ctx->dt, G.dr, G.dxi, a, a + L->n, a + 2 * L->n, a + 3 * L->n, a + 4 * L->n);
      pcr_coef(L->n, L->steps, A5, tab.data() + (size_t)m * (4 * (size_t)L->steps + 1) * L->n);
    }
    for (int j = 1; j <= G.nz; ++j)
      for (int p = 0; p < G.P; ++p)
        for (int i = 1; i <= G.nr; ++i) {
          const size_t o = ((size_t)(j - 1) * G.P + p) * G.nr + (i - 1);
          const size_t t = (size_t)(j + 1) * sl + (size_t)p * G.ld + i;
          const bool axis0 = p > 0 && i == 1;
          env[t] = axis0 ? 0.0 : ar[o];
          env[(G.nz + 3) * sl + t] = axis0 ? 0.0 : ai[o];
        }
    r = cuda_check(ctx, cudaMemcpyAsync(L->coef, tab.data(), sizeof(double) * ncoef, cudaMemcpyHostToDevice, ctx->stream),
                   "laser tables");
    if (!r) r = cuda_check(ctx, cudaMemcpyAsync(L->lr2, env.data(), sizeof(double) * (G.nz + 3) * sl,
                                                cudaMemcpyHostToDevice, ctx->stream), "laser envelope");
    if (!r) r = cuda_check(ctx, cudaMemcpyAsync(L->li2, env.data() + (G.nz + 3) * sl, sizeof(double) * (G.nz + 3) * sl,
                                                cudaMemcpyHostToDevice, ctx->stream), "laser envelope");
    if (!r) {
      static bool attr = false;
      if (!attr) {
        r = cuda_check(ctx, cudaFuncSetAttribute(k_laser_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024),
                       "laser solve attribute");
        attr = !r;
      }
    }
    if (!r) r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "laser create");
  }
  if (r) {
    if (L->lr2) cudaFree(L->lr2);
    if (L->li2) cudaFree(L->li2);
    if (L->sr) cudaFree(L->sr);
    if (L->si) cudaFree(L->si);
    if (L->coef) cudaFree(L->coef);
    delete L;
    return r;
  }
  ctx->lasers.push_back(L);
  ctx->step_key.clear();
  *out = L;
  return QPAD_OK;
}

extern "C" int qpad_laser_download(qpad_laser* L, double* ar, double* ai) {
  if (!L || !ar || !ai) return L ? set_err(L->ctx, QPAD_E_ARG, "laser download: null buffer") : QPAD_E_ARG;
  qpad_ctx* ctx = L->ctx;
  const size_t sl = (size_t)ctx->g.P * ctx->g.ld, bytes = sizeof(double) * ctx->g.nz * sl;
  int r = cuda_check(ctx, cudaMemcpyAsync(ar, L->lr2 + 2 * sl, bytes, cudaMemcpyDeviceToHost, ctx->stream), "laser download");
  if (!r) r = cuda_check(ctx, cudaMemcpyAsync(ai, L->li2 + 2 * sl, bytes, cudaMemcpyDeviceToHost, ctx->stream), "laser download");
  if (!r) r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "laser download");
  return r;
}

extern "C" int qpad_laser_chi_download(qpad_ctx* ctx, double* chi2) {
  if (!ctx || !chi2) return QPAD_E_ARG;
  if (!ctx->chi2) return set_err(ctx, QPAD_E_ARG, "no laser: no susceptibility store");
  const size_t bytes = sizeof(double) * ctx->g.nz * ctx->g.P * ctx->g.ld;
  int r = cuda_check(ctx, cudaMemcpyAsync(chi2, ctx->chi2, bytes, cudaMemcpyDeviceToHost, ctx->stream), "chi download");
  if (!r) r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "chi download");
  return r;
}

extern "C" int qpad_lasers_advance(qpad_ctx* ctx) {
  if (!ctx) return QPAD_E_ARG;
  if (int r = lasers_advance(ctx)) return r;
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "lasers advance");
}

extern "C" int qpad_species_set_radial_ppc(qpad_species* sp, int ppc_r) {
  if (!sp) return QPAD_E_ARG;
  if (ppc_r < 1) return set_err(sp->ctx, QPAD_E_ARG, "radial particles per cell must be >= 1");
  sp->ppc_r = ppc_r;
  return QPAD_OK;
}
