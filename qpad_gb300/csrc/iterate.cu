// iterate.cu -- one predictor-corrector iteration of a slice as one cluster kernel.
//
// GB300 executes FP64 at 1/64 of its FP32 rate, so the FP64 field work of an iteration
// has to be spread over many SMs instead of one CTA per mode.  Here each azimuthal mode m
// is two thread-block clusters of CL CTAs: group 0 solves B+ / B- (B-perp, E-perp and
// the convergence test), group 1 solves Bz and Ez; they read and write disjoint
// components.  CTA `rank` of a cluster owns the radial rows [rank*R, (rank+1)*R) of the
// mode (row k = node k+1).  After the plasma deposit the kernel does, per node it owns:
//
//   finish the raw deposits (axis rule, 1/(i-1)), dJ/dxi, and the right-hand sides of
//   B+ / B- (the B-perp predictor-corrector), Bz and Ez (simulation_class.f03:386-392,
//   and the Ez of the next iteration, :375-378, which depends only on the same current);
//   the tridiagonal solves of the group's systems, split across the cluster;
//   B-perp, Bz, Ez, b = b_spe + b_beam, E-perp, the FP32 gather table; and the
//   convergence test (:394-396, simulation_class.f03:522-606).
//
// Staging.  A CTA's inputs are rows on an even-aligned node window; warp 0 issues one
// bulk copy per row onto an mbarrier when every row is 16-byte aligned (even nr and R),
// otherwise every thread issues 8-byte cp.async copies.  The wait is bounded; a CTA whose
// wait gives up sets an error word that the host reads after the step, keeps taking part in
// the cluster barriers and the convergence tickets (so that nothing else waits on it) but
// writes no field, deposit or record to global memory, ends the slice's iteration loop, and
// waits once more, bounded, for its own copies in flight before it retires.
//
// Solves.  Both substitutions of a factored tridiagonal system are first-order affine
// recurrences.  Within a CTA, each right-hand side is taken by a group of gw lanes,
// each composing a contiguous run of rows, combined by a shuffle scan inside the group;
// the CTA's composite map is published in shared memory, and after a cluster barrier
// every CTA composes the maps of the CTAs before it (after it, for the back
// substitution) through distributed shared memory and replays its rows.
//
// Convergence.  The record is a per-node sum over all modes, so it cannot be formed
// inside one cluster.  Each group-0 CTA takes its node range's ticket after writing its
// B-perp; the last of the M+1 CTAs of a range evaluates the record there and folds its
// maxima into two global words (max on the bit patterns of non-negative doubles, which is
// exact and order independent); the last range to finish takes the decision, drives the
// loop state and resets the tickets.  No CTA waits on another.
#include <cooperative_groups.h>

#include <algorithm>

#include "stencils.cuh"

namespace cg = cooperative_groups;

namespace qpad {

static constexpr int kIterThreads = 256;
static constexpr int kMaxRL = 8;           // rows per lane in the solves, at most
static constexpr int kMaxRhs = 8;          // B+ (re, im), B- (re, im), Bz (re, im), Ez (re, im)
static constexpr int kCompConv = 1;        // convergence on B_phi

struct IterArgs {
  GridDev G;
  const double* fac;
  double* raw;            // raw deposits [cu 3 | amu 3 | acu 2] x P x ld, zeroed after use
  double *cu, *amu, *acu, *dcu;
  double* b_spe;
  const double* b_beam;
  double *b, *e;
  const double* psi;
  float* gtab;            // FP32 gather table (mixed path) or null
  double* conv;           // s_re[nr], s_im[nr], res[..]
  unsigned int* tickets;  // [0, CL): modes through each node range; [CL]: node ranges through the test
  unsigned long long* maxima;  // the test's two maxima (bit patterns of non-negative doubles)
  ConvLoop L;
  double reltol, abstol;
  int R;                  // rows per CTA
  int gw;                 // lanes per right-hand side in the solves
  int tma;                // stage with bulk copies (even nr and R: every row 16-byte aligned)
  unsigned int* err;      // device error word: 1 = a bulk-copy wait gave up
  int prefinished;        // the raw deposits were already finished (and smoothed) by k_smooth_raw
  const int* guard;       // part of an unrolled loop body: return at once if *guard (the loop has ended)
  int* skip_out;          // ... and then set this part's flag for the part after it
};

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;\n" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
// Programmatic dependent launch: wait for the grid this one depends on (no-op when the
// launch carried no programmatic dependency).
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

__device__ __forceinline__ void red_max_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.max.u64 [%0], %1;\n" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release;\n" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory"); }

// Raw deposit of component c of `which` (0 cu, 1 amu, 2 acu), finished on the fly.
struct RawFin {
  const GridDev* G;
  const double* raw;
  int m, which, nc;
  int prefinished;
  __device__ __forceinline__ double operator()(int p, int c, int i) const {
    const double v = raw[fidx(G->ld, nc, p, c, i)];
    return prefinished ? v : finish_amj(*G, m, which, c, i, v);
  }
};

// Composite of the per-CTA maps (B, A) published in maps[rhs] by the other CTAs of the
// cluster, applied to 0: forward, the CTAs before `rank` in increasing order; backward,
// the CTAs after it in decreasing order.  Lane l of the right-hand side's group (gw lanes)
// composes a block of up to kMaxQB consecutive maps (their remote loads all in flight
// together) and a shuffle scan over the group joins the blocks.  Every lane of the warp
// must call it.
static constexpr int kMaxQB = 4;
__device__ __forceinline__ double compose_maps(const cg::cluster_group& cluster, double* maps, int rhs, bool act,
                                               int l, int gw, int rank, int CL, bool forward) {
  const int qb = (CL + gw - 1) / gw;                   // <= kMaxQB for CL <= 16, gw >= 4
  double cA = 0.0, cB = 1.0;
#pragma unroll
  for (int j = 0; j < kMaxQB; ++j) {
    const int n = l * qb + j;                          // position in the composition order
    const int q = forward ? n : CL - 1 - n;
    if (act && j < qb && (forward ? q < rank : (q > rank && q >= 0))) {
      const double* mq = cluster.map_shared_rank(maps + 2 * rhs, q);
      const double Bq = mq[0], Aq = mq[1];
      cA = Aq + Bq * cA;
      cB = Bq * cB;
    }
  }
  for (int off = 1; off < gw; off <<= 1) {
    const double Ao = __shfl_up_sync(0xffffffffu, cA, off, gw);
    const double Bo = __shfl_up_sync(0xffffffffu, cB, off, gw);
    if (l >= off) {
      cA = cA + cB * Ao;
      cB = cB * Bo;
    }
  }
  return __shfl_sync(0xffffffffu, cA, gw - 1, gw);
}

// Shared-memory view of a staged node window: component `c0 + c` of part p (the Re or
// the Im part of this CTA's mode) at node i.
struct WinF {
  const double* w;
  int W, wb, pr, c0;
  __device__ __forceinline__ double operator()(int p, int c, int i) const {
    return w[((c0 + c) * 2 + (p == pr ? 0 : 1)) * W + (i - wb)];
  }
};

// Shared-memory staging of one CTA (doubles): the finished deposits on the node window
// [r0-1, r1+2] (cu 0..2, amu 3..5, acu 6..7), b_spe components 0..1 and b_beam on the owned
// nodes, psi on the window, the factor rows of the three matrices, the right-hand sides.
// Smoothing orders up to this many passes run inside k_iterate's node window (a +-2-node
// halo); higher orders run as a pass of their own before it (k_smooth_raw).
static constexpr int kWindowSmooth = 2;

__host__ __device__ inline size_t iterate_smem_doubles(int R, int ld, int smooth) {
  const size_t W = (size_t)R + 6;                // node window [r0-2, r0+R+4)
  (void)ld;
  const bool in_window = smooth > 0 && smooth <= kWindowSmooth;
  return 30 * W + 21 * (size_t)R + (in_window ? 12 * W : 0);   // + the smoothing scratch rows
}

// Bulk (TMA) copy global -> this CTA's shared memory, completing on an mbarrier.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(mbar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, unsigned parity) {
  unsigned ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(ok) : "r"(smem_u32(mbar)), "r"(parity) : "memory");
  return ok != 0;
}

// 8-byte asynchronous copy global -> shared (cp.async), and the wait for all of them
__device__ __forceinline__ void cp_async8(double* dst, const double* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// kSmooth: the instance with the deposit smoothing (the other one carries none of its code)
template <bool kSmooth>
__global__ void __launch_bounds__(kIterThreads) k_iterate(IterArgs a) {
  // a later part of an unrolled loop body after the loop has ended: nothing to do (every CTA
  // reads the flag, written by a kernel that completed before this one began, and leaves
  // before any barrier)
  if (a.guard && __ldcg(a.guard) != 0) {
    if (a.skip_out && blockIdx.x == 0 && threadIdx.x == 0) *a.skip_out = 1;
    return;
  }
  extern __shared__ __align__(16) double smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ double fwd[kMaxRhs][2], bwd[kMaxRhs][2];
  __shared__ double wpart[kIterThreads / 32];
  __shared__ double divp;
  __shared__ unsigned int s_ticket;
  __shared__ int s_gaveup;
  cg::cluster_group cluster = cg::this_cluster();
  const int CL = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  // two clusters per mode: group 0 solves B+ / B- (B-perp, E-perp, the convergence test),
  // group 1 solves Bz and Ez; they read and write disjoint components
  const int m = blockIdx.x / (2 * CL), grp = (blockIdx.x / CL) % 2;
  const int nr = a.G.nr, ld = a.G.ld, P = a.G.P;
  const int pr = part_re(m), pi = part_im(m);
  const int nh = m == 0 ? 1 : 2;                 // parts of this mode
  const int nrhs = m == 0 ? 2 : 4;               // right-hand sides of this group
  const int R = a.R;
  const int r0 = min(rank * R, nr), r1 = min(r0 + R, nr);
  const int Rc = r1 - r0;
  const int t = threadIdx.x;
  const int W = R + 6, wb = r0 - 2;              // node window [wb, wb + W): even start for 16-byte rows
  const size_t P1 = (size_t)P * ld;
  double* raw_cu = a.raw;
  double* raw_amu = a.raw + 3 * P1;
  double* raw_acu = a.raw + 6 * P1;
  double* win = smem;                            // [8][2][W]
  double* bo = win + 16 * W;                     // [2][2][W]
  double* bbm = bo + 4 * W;                      // [3][2][W]
  double* psw = bbm + 6 * W;                     // [2][W]
  double* facs = psw + 2 * W;                    // [3 kinds][w, ib, g][R]
  double* dsm = facs + 9 * R;                    // [kMaxRhs][R]
  double* tab = dsm + kMaxRhs * R;               // node tables ir, inv on the window
  double* djs = tab + 2 * W;                     // dJ/dxi of the owned nodes [4][R]
  double* sms = djs + 4 * R;                     // smoothing scratch [up to 12 rows][W] (smooth > 0)
  GridDev G = a.G;                               // the node tables read from shared memory
  G.ir = tab;
  G.inv = tab + W;
  G.toff = wb;

  // ---- staging: every copy of the iteration's inputs in flight at once --------------------
  // Rows on the node window: the node tables, the group's raw deposit components, psi
  // (group 0), B_old (group 0) and b_beam; then the factor rows of the group's matrices.
  // With even nr and R every row is 16-byte aligned and one thread issues one bulk (TMA)
  // copy per row onto an mbarrier; otherwise each thread issues 8-byte cp.async copies.
  const int c8_lo = grp == 0 ? 2 : 0, c8_n = grp == 0 ? 6 : 2;   // cu_z, amu, acu | cu_r, cu_phi
  const int c5_lo = grp == 0 ? 0 : 4, c5_n = grp == 0 ? 4 : 1;   // B_old r, phi and b_beam r, phi | b_beam z
  const int n0 = max(0, wb), n1 = min(ld, wb + W);               // window nodes that exist
  const int nwin = 2 + c8_n * nh + (grp == 0 ? nh : 0) + c5_n * nh;   // window rows of this CTA
  const int fr0 = grp == 0 ? 0 : 6, fr1 = grp == 0 ? 6 : 9;      // factor rows of this CTA
  // window row k: (destination, source row base at node 0)
  const auto win_row = [&](int k, double*& dst, const double*& src) {
    if (k < 2) {
      dst = tab + k * W;
      src = k == 0 ? a.G.ir : a.G.inv;
      return;
    }
    k -= 2;
    if (k < c8_n * nh) {
      const int c8 = c8_lo + k / nh, h = k % nh, p = h == 0 ? pr : pi;
      dst = win + (c8 * 2 + h) * W;
      src = c8 < 3 ? raw_cu + fidx(ld, 3, p, c8, 0)
                   : (c8 < 6 ? raw_amu + fidx(ld, 3, p, c8 - 3, 0) : raw_acu + fidx(ld, 2, p, c8 - 6, 0));
      return;
    }
    k -= c8_n * nh;
    if (grp == 0 && k < nh) {
      dst = psw + k * W;
      src = a.psi + fidx(ld, 1, k == 0 ? pr : pi, 0, 0);
      return;
    }
    if (grp == 0) k -= nh;
    const int c5 = c5_lo + k / nh, h = k % nh, p = h == 0 ? pr : pi;
    dst = c5 < 2 ? bo + (c5 * 2 + h) * W : bbm + ((c5 - 2) * 2 + h) * W;
    src = c5 < 2 ? a.b_spe + fidx(ld, 3, p, c5, 0) : a.b_beam + fidx(ld, 3, p, c5 - 2, 0);
  };
  const auto fac_src = [&](int row) {
    const int ka = row / 3, arr = row % 3;
    const int kind = ka == 0 ? OK_BPLUS : ka == 1 ? OK_BMINUS : OK_GEN;
    return a.fac + fac_off(nr, a.G.M, kind, m) + (size_t)arr * nr + r0;
  };
  const auto is_raw_row = [&](int k) { return k >= 2 && k < 2 + c8_n * nh; };   // written by the deposit
  // window slots outside the grid are zero
  for (int q = t; q < nwin * W; q += blockDim.x) {
    const int k = q / W, x = q % W;
    if (x >= n0 - wb && x < n1 - wb) continue;
    double* dst;
    const double* src;
    win_row(k, dst, src);
    dst[x] = 0.0;
  }
  __shared__ int s_bulk;
  if (t < 32) {
    // warp 0 issues one bulk copy per row (lane k: rows k, k + 32, ...), only when every
    // copy is 16-byte aligned (each lane checks its rows before any copy is issued)
    const int nf = fr1 - fr0, ncp = nwin + nf;
    const unsigned wbytes = (unsigned)(n1 - n0) * 8u, fbytes = (unsigned)Rc * 8u;
    const auto row_copy = [&](int k, void*& dst, const void*& src, unsigned& bytes) {
      if (k < nwin) {
        double* d;
        const double* sr;
        win_row(k, d, sr);
        dst = d + (n0 - wb);
        src = sr + n0;
        bytes = wbytes;
      } else {
        dst = facs + (fr0 + k - nwin) * R;
        src = fac_src(fr0 + k - nwin);
        bytes = fbytes;
      }
    };
    bool mine = true;
    for (int k = t; k < ncp; k += 32) {
      void* dst;
      const void* src;
      unsigned bytes;
      row_copy(k, dst, src, bytes);
      mine &= (((uintptr_t)src | (uintptr_t)smem_u32(dst) | bytes) & 15u) == 0;
    }
    const bool ok = __all_sync(0xffffffffu, mine) && a.tma;
    if (ok && t == 0) {
      const unsigned total = (unsigned)nwin * wbytes + (unsigned)nf * fbytes;
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&mbar)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(&mbar)), "r"(total)
                   : "memory");
    }
    __syncwarp();
    // rows that the deposit before this kernel does not write first; the raw deposit rows
    // after the programmatic wait (a no-op unless launched as a dependent of the deposit)
    for (int pass = 0; pass < 2; ++pass) {
      if (pass == 1) griddep_wait();
      if (ok)
        for (int k = t; k < ncp; k += 32) {
          if (is_raw_row(k) != (pass == 1)) continue;
          void* dst;
          const void* src;
          unsigned bytes;
          row_copy(k, dst, src, bytes);
          if (bytes) bulk_g2s(dst, src, bytes, &mbar);
        }
    }
    if (t == 0) {
      s_bulk = ok;
      s_gaveup = 0;
    }
  }
  __syncthreads();                                    // s_bulk, s_gaveup and the mbarrier are set up
  griddep_wait();                                     // nothing below runs before the deposit is complete
  if (s_bulk) {
    int spins = 0;
    while (!mbar_try_wait(&mbar, 0u))
      if (++spins > (1 << 20)) {                     // bounded wait: give up (see below)
        s_gaveup = 1;
        break;
      }
  } else {
    for (int k = 0; k < nwin; ++k) {
      double* dst;
      const double* src;
      win_row(k, dst, src);
      for (int x = n0 - wb + t; x < n1 - wb; x += blockDim.x) cp_async8(dst + x, src + wb + x);
    }
    // (this path issues every row after the programmatic wait)
    for (int row = fr0; row < fr1; ++row) {
      const double* src = fac_src(row);
      for (int k = t; k < Rc; k += blockDim.x) cp_async8(facs + row * R + k, src + k);
    }
    cp_async_wait_all();
  }
  __syncthreads();
  // A wait that gave up: the host reads the error word after the step and reports its
  // results as invalid.  The CTA still takes part in every cluster barrier and in the
  // convergence tickets, so that its peers and the loop state finish, but from here on it
  // writes nothing to global memory except that control state, and before it retires it
  // waits (again bounded) for its own bulk copies still in flight.
  const bool gave_up = s_gaveup != 0;
  if (gave_up && t == 0) atomicExch(a.err, 1u);
  // finish the deposits in place, one window node per thread (W <= blockDim.x for the
  // row counts the host allows; the loop covers any W): every row of a node from the
  // second on takes the same factor 1/(i-1)
  if (!a.prefinished)
    for (int x = t; x < W; x += blockDim.x) {
      const int node = wb + x;
      if (node < 0 || node > nr + 1) continue;
      if (node >= 2) {
        const double f = G.inv[node - G.toff];
        for (int c = 0; c < c8_n; ++c)
          for (int h = 0; h < nh; ++h) win[((c8_lo + c) * 2 + h) * W + x] *= f;
        continue;
      }
      for (int c = 0; c < c8_n; ++c)
        for (int h = 0; h < nh; ++h) {
          const int c8 = c8_lo + c;
          double& v = win[(c8 * 2 + h) * W + x];
          v = c8 < 3 ? finish_amj(G, m, 0, c8, node, v) : (c8 < 6 ? finish_amj(G, m, 1, c8 - 3, node, v)
                                                                      : finish_amj(G, m, 2, c8 - 6, node, v));
        }
    }
  __syncthreads();
  // binomial smoothing of the finished deposits (amjdp_species2d, species2d_class.f03:270-272):
  // pass k is exact on window nodes [wb + k, wb + W - 1 - k], which covers the owned nodes and
  // their neighbours for k <= 2
  if constexpr (kSmooth)
  for (int pass = 1; pass <= G.smooth; ++pass) {
    for (int q = t; q < c8_n * nh * W; q += blockDim.x) {
      const int row = q / W, x = q % W, c8 = c8_lo + row / nh, node = wb + x;
      const double* v = win + (c8 * 2 + row % nh) * W;
      double out = v[x];
      if (x >= pass && x <= W - 1 - pass && node >= 1 && node <= nr) {
        const int kind = c8 < 6 ? 1 : 2, comp = c8 < 3 ? c8 : (c8 < 6 ? c8 - 3 : c8 - 6);
        out = smooth_node(G, node, smooth_ax(kind, m, comp), v[x - 1], v[x], v[x + 1]);
      }
      sms[q] = out;
    }
    __syncthreads();
    for (int q = t; q < c8_n * nh * W; q += blockDim.x) {
      const int row = q / W, c8 = c8_lo + row / nh;
      win[(c8 * 2 + row % nh) * W + q % W] = sms[q];
    }
    __syncthreads();
  }
  const WinF CU{win, W, wb, pr, 0}, AMU{win, W, wb, pr, 3}, ACU{win, W, wb, pr, 6};
  const WinF PS{psw, W, wb, pr, 0};
  const auto BO = [&](int p, int c, int i) { return bo[(c * 2 + (p == pr ? 0 : 1)) * W + (i - wb)]; };

  // ---- sources: (node, equation group) per thread ---------------------------------------
  // group 0: dJ/dxi and the B+ / B- right-hand sides; group 1: Bz; group 2: Ez
  double div = 0.0;
  // rows 1, 2 and nr take boundary stencils: they go to the last warp's threads so that
  // the other warps do not wait out their branch
  const auto special = [&](int i) { return i <= 2 || i == nr; };
  const int njob = grp == 0 ? 1 : 2;
  const auto source_row = [&](int job, int k) {
    const int i = r0 + k + 1;
    if (job == 0) {
      double dj[4];
      row_djdxi(G, m, i, ACU, AMU, dj);
      const auto DC = [&](int p, int c, int) { return p == pr ? dj[c] : dj[2 + c]; };
      double bt[4];
      row_btiter_src(G, m, i, DC, CU, BO, bt);
      if (m == 0) {
        dsm[0 * R + k] = bt[0];
        dsm[1 * R + k] = bt[1];
      } else {
        dsm[0 * R + k] = bt[0];
        dsm[1 * R + k] = bt[2];
        dsm[4 * R + k] = bt[1];
        dsm[5 * R + k] = bt[3];
      }
      for (int c = 0; c < 4; ++c) djs[c * R + k] = dj[c];
    } else if (job == 1) {
      double zr, zi;
      row_bz_src(G, m, i, CU, zr, zi);
      dsm[2 * R + k] = zr;
      if (m > 0) dsm[6 * R + k] = zi;
    } else {
      double er, ei;
      bool in_div;
      row_ez_src(G, m, i, CU, er, ei, in_div);
      if (in_div) div += er * (double)(i - 1);
      dsm[3 * R + k] = er;
      if (m > 0) dsm[7 * R + k] = ei;
    }
  };
  for (int q = t; q < njob * Rc; q += blockDim.x) {
    const int job = (grp == 0 ? 0 : 1) + q / Rc, k = q % Rc;
    if (!special(r0 + k + 1)) source_row(job, k);
  }
  {
    // this CTA's boundary rows: candidates k = 0, 1, Rc - 1
    const bool v0 = Rc > 0 && special(r0 + 1), v1 = Rc > 1 && special(r0 + 2), v2 = Rc > 2 && special(r0 + Rc);
    const int ns = (int)v0 + (int)v1 + (int)v2;
    const int sidx = (int)blockDim.x - 1 - t;
    if (sidx < njob * ns) {
      int w = sidx % ns, k = -1;
      if (v0) k = w-- == 0 ? 0 : k;
      if (v1 && k < 0) k = w-- == 0 ? 1 : k;
      if (v2 && k < 0) k = w == 0 ? Rc - 1 : k;
      source_row((grp == 0 ? 0 : 1) + sidx / ns, k);
    }
  }
  // the m = 0 axis row of Ez needs the weighted sum over the whole line
  if (m == 0 && grp == 1) {
    for (int off = 16; off > 0; off >>= 1) div += __shfl_down_sync(0xffffffffu, div, off);
    if ((t & 31) == 0) wpart[t >> 5] = div;
    __syncthreads();
    if (t == 0) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += wpart[w];
      divp = s;
    }
    cluster.sync();
    if (rank == 0 && t == 0) {
      double s = 0.0;
      for (int q = 0; q < CL; ++q) s += *cluster.map_shared_rank(&divp, q);
      const RawFin CUg{&a.G, raw_cu, 0, 0, 3, a.prefinished};   // nodes nr-2, nr-1 lie outside this window
      if constexpr (kSmooth) {
        const auto CUs = [&](int p, int c, int i) { return smoothed_at(a.G, CUg, 1, 0, p, c, i, a.G.smooth); };
        dsm[3 * R + 0] = ez_axis_row(a.G, s, CUs);
      } else {
        dsm[3 * R + 0] = ez_axis_row(a.G, s, CUg);
      }
    }
  }
  __syncthreads();

  // ---- forward substitution y_k = d_k - w_k y_{k-1} ------------------------------------
  // gw lanes per right-hand side (a power of two, host-chosen so that RL <= kMaxRL); a
  // lane's rows and factors are read into registers before its dependent FP64 chain
  const int gw = a.gw;
  const int rl = t / gw, l = t % gw;
  // slot of local right-hand side rl: group 0 {B+ re, B- re, B+ im, B- im} = {0, 1, 4, 5},
  // group 1 {Bz re, Ez re, Bz im, Ez im} = {2, 3, 6, 7}
  const int rhs = ((rl & 1) | ((rl >> 1) << 2)) + 2 * grp;
  const bool solver = t < 32 * ((kMaxRhs / 2 * gw + 31) / 32);   // whole warps take part in the shuffles
  const bool act = rl < nrhs;
  const int RL = (Rc + gw - 1) / gw;
  const int k0 = min(l * RL, Rc), cnt = min(RL, Rc - k0);
  const int ka = (rhs & 3) < 2 ? (rhs & 3) : 2;          // B+, B-, then the shared Bz / Ez matrix
  const double* fw = facs + ka * 3 * R + k0;
  const double* fib = facs + ka * 3 * R + R + k0;
  const double* fg = facs + ka * 3 * R + 2 * R + k0;
  double* d = dsm + (size_t)(act ? rhs : 2 * grp) * R + k0;
  double dv[kMaxRL], cv[kMaxRL];
#pragma unroll
  for (int j = 0; j < kMaxRL; ++j) {
    const bool in = act && j < cnt;
    dv[j] = in ? d[j] : 0.0;
    cv[j] = in ? fw[j] : 0.0;
  }
  double Aex = 0.0, Bex = 1.0;
  if (solver) {
    double A = 0.0, B = 1.0;
#pragma unroll
    for (int j = 0; j < kMaxRL; ++j)
      if (j < cnt) {
        A = dv[j] - cv[j] * A;
        B = -cv[j] * B;
      }
    for (int off = 1; off < gw; off <<= 1) {
      const double Ao = __shfl_up_sync(0xffffffffu, A, off, gw);
      const double Bo = __shfl_up_sync(0xffffffffu, B, off, gw);
      if (l >= off) {
        A = A + B * Ao;
        B = B * Bo;
      }
    }
    Aex = __shfl_up_sync(0xffffffffu, A, 1, gw);
    Bex = __shfl_up_sync(0xffffffffu, B, 1, gw);
    if (l == 0) {
      Aex = 0.0;
      Bex = 1.0;
    }
    if (act && l == gw - 1) {
      fwd[rhs][0] = B;
      fwd[rhs][1] = A;
    }
  }
  cluster.sync();
  double carry = 0.0;                                 // y at the row before this CTA
  if (solver) carry = compose_maps(cluster, &fwd[0][0], rhs, act, l, gw, rank, CL, true);
  if (solver && act) {
    double y = Aex + Bex * carry;
#pragma unroll
    for (int j = 0; j < kMaxRL; ++j)
      if (j < cnt) {
        y = dv[j] - cv[j] * y;
        dv[j] = y;
      }
  }

  // ---- back substitution x_k = y_k ib_k - g_k x_{k+1} -----------------------------------
  double ibv[kMaxRL];
#pragma unroll
  for (int j = 0; j < kMaxRL; ++j) {
    const bool in = act && j < cnt;
    ibv[j] = in ? fib[j] : 0.0;
    cv[j] = in ? fg[j] : 0.0;
  }
  if (solver) {
    double A = 0.0, B = 1.0;
#pragma unroll
    for (int j = kMaxRL - 1; j >= 0; --j)
      if (j < cnt) {
        A = dv[j] * ibv[j] - cv[j] * A;
        B = -cv[j] * B;
      }
    for (int off = 1; off < gw; off <<= 1) {
      const double Ao = __shfl_down_sync(0xffffffffu, A, off, gw);
      const double Bo = __shfl_down_sync(0xffffffffu, B, off, gw);
      if (l + off < gw) {
        A = A + B * Ao;
        B = B * Bo;
      }
    }
    Aex = __shfl_down_sync(0xffffffffu, A, 1, gw);
    Bex = __shfl_down_sync(0xffffffffu, B, 1, gw);
    if (l == gw - 1) {
      Aex = 0.0;
      Bex = 1.0;
    }
    if (act && l == 0) {
      bwd[rhs][0] = B;
      bwd[rhs][1] = A;
    }
  }
  cluster.sync();
  carry = 0.0;                                        // x at the row after this CTA
  if (solver) carry = compose_maps(cluster, &bwd[0][0], rhs, act, l, gw, rank, CL, false);
  if (solver && act) {
    double x = Aex + Bex * carry;
#pragma unroll
    for (int j = kMaxRL - 1; j >= 0; --j)
      if (j < cnt) {
        x = dv[j] * ibv[j] - cv[j] * x;
        d[j] = x;
      }
  }
  // last access to another CTA's shared memory is done; the matching wait sits at the end
  cluster_arrive();
  __syncthreads();

  // ---- fields of the owned nodes: (node, group) per thread ------------------------------
  // group 0: B-perp from B+ / B-, b = b_spe + b_beam and E-perp; group 1: Bz and Ez
  const auto field_row = [&](int k) {
    const int job = grp, i = r0 + k + 1;
    if (job == 0) {
      double bs[2][2], bb[2][2];
      if (m == 0) {
        bs[0][0] = (i == 1) ? 0.0 : dsm[0 * R + k];
        bs[0][1] = (i == 1) ? 0.0 : dsm[1 * R + k];
      } else {
        const bool zero = (i == 1 && m != 1);
        const double b1re = dsm[0 * R + k], b2re = dsm[1 * R + k];
        const double b1im = dsm[4 * R + k], b2im = dsm[5 * R + k];
        bs[0][0] = zero ? 0.0 : 0.5 * (b1re + b2re);
        bs[1][0] = zero ? 0.0 : 0.5 * (b1im + b2im);
        bs[0][1] = zero ? 0.0 : 0.5 * (b1im - b2im);
        bs[1][1] = zero ? 0.0 : 0.5 * (-b1re + b2re);
      }
      for (int h = 0; h < nh; ++h)
        for (int c = 0; c < 2; ++c) bb[h][c] = bs[h][c] + bbm[(c * 2 + h) * W + (i - wb)];
      const auto Bn = [&](int p, int c, int) { return p == pr ? bb[0][c] : bb[1][c]; };
      double et[4];
      row_et(G, m, i, Bn, PS, et);
      double ee[2][2];
      if (m == 0) {
        ee[0][0] = et[0];
        ee[0][1] = et[1];
      } else {
        ee[0][0] = et[0];
        ee[1][0] = et[1];
        ee[0][1] = et[2];
        ee[1][1] = et[3];
      }
      for (int h = 0; h < nh; ++h) {
        const int p = h == 0 ? pr : pi;
        for (int c = 0; c < 2; ++c) {
          a.b_spe[fidx(ld, 3, p, c, i)] = bs[h][c];
          a.b[fidx(ld, 3, p, c, i)] = bb[h][c];
          a.e[fidx(ld, 3, p, c, i)] = ee[h][c];
        }
        if (a.gtab) {
          float* T = a.gtab + ((size_t)i * P + p) * 6;
          T[0] = (float)ee[h][0];
          T[1] = (float)ee[h][1];
          T[3] = (float)bb[h][0];
          T[4] = (float)bb[h][1];
        }
      }
    } else {
      double bz[2], ez[2];
      if (m == 0) {
        bz[0] = dsm[2 * R + k];
        ez[0] = dsm[3 * R + k];
      } else {
        bz[0] = (i == 1) ? 0.0 : dsm[2 * R + k];
        bz[1] = (i == 1) ? 0.0 : dsm[6 * R + k];
        ez[0] = (i == 1) ? 0.0 : dsm[3 * R + k];
        ez[1] = (i == 1) ? 0.0 : dsm[7 * R + k];
      }
      for (int h = 0; h < nh; ++h) {
        const int p = h == 0 ? pr : pi;
        const double bzt = bz[h] + bbm[(2 * 2 + h) * W + (i - wb)];
        a.b_spe[fidx(ld, 3, p, 2, i)] = bz[h];
        a.b[fidx(ld, 3, p, 2, i)] = bzt;
        a.e[fidx(ld, 3, p, 2, i)] = ez[h];
        if (a.gtab) {
          float* T = a.gtab + ((size_t)i * P + p) * 6;
          T[2] = (float)ez[h];
          T[5] = (float)bzt;
        }
      }
    }
  };
  for (int q = t; q < Rc; q += blockDim.x)
    if (!special(r0 + q + 1) && !gave_up) field_row(q);
  {
    const bool v0 = Rc > 0 && special(r0 + 1), v1 = Rc > 1 && special(r0 + 2), v2 = Rc > 2 && special(r0 + Rc);
    const int ns = (int)v0 + (int)v1 + (int)v2;
    const int sidx = (int)blockDim.x - 1 - t;
    if (sidx < ns && !gave_up) {
      int w = sidx, k = -1;
      if (v0) k = w-- == 0 ? 0 : k;
      if (v1 && k < 0) k = w-- == 0 ? 1 : k;
      if (v2 && k < 0) k = w == 0 ? Rc - 1 : k;
      field_row(k);
    }
  }

  // guard nodes (0, nr + 1): nothing here writes b_spe or E there, so b = b_spe + b_beam and
  // their gather-table records stay as k_iter_e wrote them at the start of the slice

  // ---- stores nothing in this kernel waits for: the finished deposits, dJ/dxi, and the
  // cleared raw deposits (every CTA of the cluster staged its window before the forward
  // barrier); threads first, first + stride, ...
  const auto late_stores = [&](int first, int stride) {
    if (gave_up) return;
    const int i0 = rank == 0 ? 0 : r0 + 1, i1 = rank == CL - 1 ? nr + 1 : r1;
    const int nn = i1 - i0 + 1;
    for (int q = first; q < c8_n * nh * nn; q += stride) {
      const int c8 = c8_lo + q / (nh * nn), h = (q / nn) % nh, i = i0 + q % nn;
      const int p = h == 0 ? pr : pi;
      const double v = win[(c8 * 2 + h) * W + (i - wb)];
      if (c8 < 3) {
        a.cu[fidx(ld, 3, p, c8, i)] = v;
        raw_cu[fidx(ld, 3, p, c8, i)] = 0.0;
      } else if (c8 < 6) {
        a.amu[fidx(ld, 3, p, c8 - 3, i)] = v;
        raw_amu[fidx(ld, 3, p, c8 - 3, i)] = 0.0;
      } else {
        a.acu[fidx(ld, 2, p, c8 - 6, i)] = v;
        raw_acu[fidx(ld, 2, p, c8 - 6, i)] = 0.0;
      }
    }
    for (int q = first; q < (grp == 0 ? 2 * nh * Rc : 0); q += stride) {
      const int c = q / (nh * Rc), h = (q / Rc) % nh, k = q % Rc;
      a.dcu[fidx(ld, 2, h == 0 ? pr : pi, c, r0 + k + 1)] = djs[(2 * h + c) * R + k];
    }
  };
  bool late_done = false;

  // ---- convergence test (group 0, which owns B-perp) ------------------------------------
  if (grp == 0) {
  __syncthreads();                                    // this CTA's B-perp is written
  if (t == 0) s_ticket = atom_add_acq_rel(&a.tickets[rank], 1u);   // releases it, acquires the others'
  __syncthreads();
  if (s_ticket == (unsigned)G.M) {                    // the last mode of this node range: its record
    double* s_re = a.conv;
    double* s_im = a.conv + nr;
    int it_prev = 0, jp = 1;
    if (t == 0 && a.L.iter_ctr) {                     // loop state, read in case this CTA decides
      it_prev = __ldcg(a.L.iter_ctr);
      if (a.L.stats && a.L.jp) jp = __ldcg(a.L.jp);
    }
    // maxima as the bit patterns of non-negative doubles: integer order is numeric order,
    // so the max over nodes is exact, order independent and off the FP64 pipe
    unsigned long long mo = 0ull, mn = 0ull;
    // the warps the record needs take it; the others issue the late stores meanwhile
    const int rth = min((int)blockDim.x, 32 * ((Rc + 31) / 32));
    if (rth < (int)blockDim.x) {
      if (t >= rth) late_stores(t - rth, (int)blockDim.x - rth);
      late_done = true;
    }
    for (int k = t; k < Rc && t < rth; k += rth) {
      const int i = r0 + k + 1;
      double bv[QPAD_MAX_PARTS];                     // every mode's B_phi here, loads in flight together
#pragma unroll
      for (int p = 0; p < QPAD_MAX_PARTS; ++p) bv[p] = p < P ? __ldcg(a.b_spe + fidx(ld, 3, p, kCompConv, i)) : 0.0;
      const double ore = __ldcg(s_re + i - 1), oim = __ldcg(s_im + i - 1);
      const auto Bc = [&](int p, int, int) {
        double v = 0.0;
#pragma unroll
        for (int q = 0; q < QPAD_MAX_PARTS; ++q)
          if (q == p) v = bv[q];
        return v;
      };
      double nre, nim, xo = 0.0, xn = 0.0;
      conv_node_v(G, Bc, kCompConv, i, ore, oim, true, nre, nim, xo, xn);
      if (!gave_up) {
        s_re[i - 1] = nre;
        s_im[i - 1] = nim;
      }
      mo = max(mo, (unsigned long long)__double_as_longlong(xo));
      mn = max(mn, (unsigned long long)__double_as_longlong(xn));
    }
    for (int off = 16; off > 0; off >>= 1) {
      mo = max(mo, __shfl_down_sync(0xffffffffu, mo, off));
      mn = max(mn, __shfl_down_sync(0xffffffffu, mn, off));
    }
    __shared__ unsigned long long rmo[kIterThreads / 32], rmn[kIterThreads / 32];
    if ((t & 31) == 0) {
      rmo[t >> 5] = mo;
      rmn[t >> 5] = mn;
    }
    __syncthreads();                                  // also orders this CTA's record stores
    if (t == 0) {
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
        mo = max(mo, rmo[w]);
        mn = max(mn, rmn[w]);
      }
      unsigned long long* mx = a.maxima;
      if (mo && !gave_up) red_max_u64(mx, mo);
      if (mn && !gave_up) red_max_u64(mx + 1, mn);
      a.tickets[rank] = 0u;
      if (atom_add_acq_rel(&a.tickets[CL], 1u) == (unsigned)(CL - 1)) {   // the last range: the decision
        // (the error word loads with the maxima: no extra latency on the decision)
        const unsigned long long vo = __ldcg(mx), vn = __ldcg(mx + 1);
        const unsigned ev = __ldcg(a.err);
        mx[0] = 0ull;
        mx[1] = 0ull;
        a.tickets[CL] = 0u;
        // after a give-up the iteration ends the slice (its results are invalid)
        const bool failed = gave_up || ev != 0u;
        conv_decide_at(__longlong_as_double((long long)vo), failed ? 0.0 : __longlong_as_double((long long)vn),
                       a.reltol, a.abstol, a.conv + 2 * nr, a.L, it_prev, jp);
      }
    }
  }
  }

  if (!late_done) late_stores(t, (int)blockDim.x);
  cluster_wait();
  if (gave_up && s_bulk && t == 0) {
    // drain: bulk copies into this CTA's shared memory must land before it retires; a copy
    // that has not completed after this second bounded wait cannot be cancelled
    int spins = 0;
    while (!mbar_try_wait(&mbar, 0u) && ++spins <= (1 << 22)) {
    }
  }
}

// ------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------
static int cluster_for(int nr) { return std::max(1, std::min(16, nr / 32)); }

// Lanes per right-hand side for R rows per CTA: a power of two in 4..32 giving at most 4
// rows per lane where possible (and at most kMaxRL); 8 right-hand sides fit 256 threads.
static int solve_lanes(int R) {
  int g = 4;
  while (g < 32 && (R + g - 1) / g > 4) g *= 2;
  return g;
}

// Uses cluster size cl for k_iterate if the kernel can launch with it; nonzero otherwise.
static void (*iterate_kernel(int smooth))(IterArgs) {
  return smooth > 0 && smooth <= kWindowSmooth ? k_iterate<true> : k_iterate<false>;
}

// Smoothing orders above kWindowSmooth (amjdp_species2d's cu / dcu / amu%smooth(),
// species2d_class.f03:270-272, ufield::smooth_f1 applied smooth_order times,
// ufield_class.f03:274-339): one CTA per deposit row (8 components) and mode part finishes
// the raw line, applies every pass and stores the finished, smoothed line in place; the
// iteration kernel then takes it as it is (IterArgs::prefinished).  (It cannot go back to
// raw form: the smoothing's axis rule may leave a value on an axis node that the finishing
// zeroes.)
__global__ void __launch_bounds__(256) k_smooth_raw(GridDev G, double* __restrict__ raw, const int* __restrict__ guard) {
  if (guard && *guard) return;                   // a part of an unrolled loop body after the loop ended
  extern __shared__ double sl[];                 // two lines of ld doubles
  const int row = blockIdx.x % 8, p = blockIdx.x / 8;
  const int m = (p + 1) / 2, ld = G.ld, nr = G.nr;
  const size_t P1 = (size_t)G.P * ld;
  const int which = row < 3 ? 0 : (row < 6 ? 1 : 2), comp = row < 3 ? row : (row < 6 ? row - 3 : row - 6);
  double* line = raw + (size_t)(row < 6 ? (row < 3 ? 0 : 3) : 6) * P1 +
                 ((size_t)p * (which == 2 ? 2 : 3) + comp) * ld;
  double* a = sl;
  double* b = sl + ld;
  for (int i = threadIdx.x; i < ld; i += blockDim.x) a[i] = finish_amj(G, m, which, comp, i, line[i]);
  __syncthreads();
  const bool ax = smooth_ax(which == 2 ? 2 : 1, m, comp);
  for (int pass = 0; pass < G.smooth; ++pass) {
    for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) b[i] = smooth_node(G, i, ax, a[i - 1], a[i], a[i + 1]);
    __syncthreads();
    for (int i = 1 + threadIdx.x; i <= nr; i += blockDim.x) a[i] = b[i];
    __syncthreads();
  }
  for (int i = threadIdx.x; i < ld; i += blockDim.x) line[i] = a[i];
}

int launch_smooth_raw(qpad_ctx* ctx) {
  if (ctx->g.smooth <= kWindowSmooth) return 0;
  const size_t smem = 2 * (size_t)ctx->g.ld * sizeof(double);
  if (int r = raise_dyn_smem(ctx, (const void*)k_smooth_raw, smem)) return r;
  k_smooth_raw<<<8 * ctx->g.P, 256, smem, ctx->stream>>>(ctx->g, ctx->raw, iter_guard(ctx));
  return check_launch(ctx, "k_smooth_raw");
}

int iterate_try_cluster(qpad_ctx* ctx, int cl) {
  if (cl < 1 || cl > 16 || cl > ctx->g.nr) return QPAD_E_ARG;
  if ((ctx->g.nr + cl - 1) / cl > 32 * kMaxRL) return QPAD_E_CAPACITY;      // rows per CTA beyond the solver
  const auto kern = iterate_kernel(ctx->g.smooth);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return cuda_check(ctx, e, "cluster attribute");
  const int R = (ctx->g.nr + cl - 1) / cl;
  const size_t smem = iterate_smem_doubles(R, ctx->g.ld, ctx->g.smooth) * sizeof(double);
  if (smem > 200 * 1024) return QPAD_E_CAPACITY;
  if (int r = raise_dyn_smem(ctx, (const void*)kern, smem)) return r;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2 * cl * (ctx->g.M + 1));
  cfg.blockDim = dim3(kIterThreads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int ncl = 0;
  e = cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg);
  if (e != cudaSuccess || ncl < 1) {
    cudaGetLastError();
    return QPAD_E_CAPACITY;
  }
  ctx->iter_cl = cl;
  ctx->iter_rows = R;
  return 0;
}

int iterate_setup(qpad_ctx* ctx) {
  if (ctx->iter_cl > 0) return 0;
  for (int cl = cluster_for(ctx->g.nr); cl >= 1; cl /= 2)
    if (iterate_try_cluster(ctx, cl) == 0) return 0;
  cudaGetLastError();
  return set_err(ctx, QPAD_E_CUDA, "no cluster shape of the iteration kernel fits this grid and GPU");
}

int launch_iterate(qpad_ctx* ctx, int loop_state, cudaGraphConditionalHandle h, int use_h, int after_deposit) {
  if (int r = iterate_setup(ctx)) return r;
  IterArgs a;
  a.G = ctx->g;
  a.fac = ctx->fac;
  a.raw = ctx->raw;
  a.cu = ctx->f[QPAD_F_CU];
  a.amu = ctx->f[QPAD_F_AMU];
  a.acu = ctx->f[QPAD_F_ACU];
  a.dcu = ctx->f[QPAD_F_DCU];
  a.b_spe = ctx->f[QPAD_F_B_SPE];
  a.b_beam = ctx->f[QPAD_F_B_BEAM];
  a.b = ctx->f[QPAD_F_B];
  a.e = ctx->f[QPAD_F_E];
  a.psi = ctx->f[QPAD_F_PSI];
  a.gtab = ctx->precision == QPAD_PREC_MIXED ? ctx->gtab : nullptr;
  a.conv = ctx->conv;
  a.tickets = ctx->iter_tickets;
  a.maxima = reinterpret_cast<unsigned long long*>(ctx->iter_tickets + kIterMaxWords);
  a.L = ConvLoop{};
  if (loop_state) {
    a.L.iter_ctr = ctx->d_iter;
    a.L.stats = ctx->d_stats;
    a.L.jp = ctx->d_j;
    a.L.iter_max = ctx->iter_max;
    a.L.h = h;
    a.L.use_h = use_h;
    a.L.stop = iter_stop_out(ctx);
  }
  a.reltol = ctx->reltol;
  a.abstol = ctx->abstol;
  a.R = ctx->iter_rows;
  a.gw = solve_lanes(a.R);
  a.tma = (ctx->g.nr % 2 == 0 && a.R % 2 == 0) ? 1 : 0;
  a.err = ctx->iter_tickets + kIterErrWord;
  a.prefinished = ctx->g.smooth > kWindowSmooth ? 1 : 0;
  a.guard = iter_guard(ctx);
  a.skip_out = loop_state ? iter_stop_out(ctx) : nullptr;
  const int cl = ctx->iter_cl;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2 * cl * (ctx->g.M + 1));
  cfg.blockDim = dim3(kIterThreads);
  cfg.dynamicSmemBytes = iterate_smem_doubles(a.R, ctx->g.ld, ctx->g.smooth) * sizeof(double);
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  // directly after the plasma deposit: start as its programmatic dependent, so that the
  // launch and the staging of everything the deposit does not write overlap it
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = (after_deposit && ctx->pdl) ? 2 : 1;
  prof_begin(ctx, "iterate");
  cudaError_t e = cudaLaunchKernelEx(&cfg, iterate_kernel(ctx->g.smooth), a);
  prof_end(ctx, "iterate");
  if (e != cudaSuccess) return cuda_check(ctx, e, "k_iterate launch");
  return check_launch(ctx, "k_iterate");
}

}  // namespace qpad
