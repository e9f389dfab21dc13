// qpad_internal.cuh -- shared device/host declarations of the GB300 quasi-static slice loop.
//
// Device data layout (all FP64 in the reference-arithmetic path):
//   slice field f1    f[(p*nc + c)*ld + i]          p = mode part (0: m=0, 2m-1: Re m, 2m: Im m)
//                                                   c = component, i = node 0..nr+1 (ld = nr+2)
//   3D store f2       f[(((s-1)*P + p)*nc + c)*ld + i]   s = xi slice 1..nz+1
//   particles         structure of arrays, one float64 array per coordinate
// The layouts are the reference's f1(dim, 0:nr+1) per mode part with the component
// index moved outward, so that each radial line is contiguous for the tridiagonal
// solves and coalesced for the source builders.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/qpad_gpu.h"

#define QPAD_MAX_MODE 8
#define QPAD_MAX_PARTS (2 * QPAD_MAX_MODE + 1)

namespace qpad {

// Kinds of tridiagonal operator with distinct matrices (field_solver_class.f03:256-561).
// psi, Ez and Bz share one matrix per mode (their interior rows and boundary rows are
// identical), the beam B-perp potential differs only in its m = 0 outer row.
enum OpKind { OK_GEN = 0, OK_BT = 1, OK_BPLUS = 2, OK_BMINUS = 3, OK_NKINDS = 4 };

struct GridDev {
  int nr, nz, M, P, ld, bnd;
  double dr, dxi, idr, relax_fac;
  // per-node factors of the reference's finite differences and deposit scaling, computed
  // once with the same FP64 expressions: ir[i] = idr / (i-1), inv[i] = 1 / (i-1) (i >= 2);
  // entry i sits at ir[i - toff] (toff = 0 for the full tables, the window start for a
  // window of them staged in shared memory)
  const double* ir;
  const double* inv;
  int toff;
  int smooth;     // binomial smoothing passes of the species deposits (0..2)
};

__host__ __device__ inline int part_re(int m) { return m == 0 ? 0 : 2 * m - 1; }
__host__ __device__ inline int part_im(int m) { return 2 * m; }

__host__ __device__ inline size_t fidx(int ld, int nc, int p, int c, int i) {
  return ((size_t)p * nc + c) * (size_t)ld + (size_t)i;
}

// Factor tables for one (kind, mode): forward multipliers w, reciprocal pivots ib and
// back-substitution multipliers g of the Thomas factorisation, each of length nr.
__host__ __device__ inline size_t fac_off(int nr, int M, int kind, int m) {
  return ((size_t)kind * (M + 1) + m) * 3 * (size_t)nr;
}

int field_ncomp(int field);

// Loop state of the predictor-corrector iteration, updated by the convergence test:
// iterations taken, per-slice statistics and, inside a CUDA graph, the WHILE-node
// condition (continue while not converged and below iter_max, simulation_class.f03:370-398).
struct ConvLoop {
  int* iter_ctr;                 // iterations taken in the current slice
  qpad_slice_stats* stats;       // per-slice statistics [nz]
  const int* jp;                 // current slice (1-based)
  int iter_max;
  cudaGraphConditionalHandle h;  // WHILE-node handle
  int use_h;
  int* stop;                     // unrolled graph bodies: set to 1 when the loop has ended, else 0
};

struct Species;
struct Beam;

}  // namespace qpad

static constexpr int kMaxSmoothOrder = 64;    // smoothing passes of the species deposits, at most
static constexpr int kIterMaxWords = 64;      // k_iterate's two 64-bit maxima in the ticket buffer
static constexpr int kIterErrWord = 127;       // k_iterate's error word in the ticket buffer
static constexpr int kMaxUnroll = 4;          // iterations per body of the graph's iteration loop, at most

struct qpad_ctx {
  qpad::GridDev g;
  int iter_max;
  double reltol, abstol, dt;
  int precision;
  int device;
  cudaStream_t stream = nullptr;
  double* fac = nullptr;                       // device factor tables
  double* rtab = nullptr;                      // ir / inv node tables (2 x ld)
  double* f[QPAD_NFIELDS] = {};                // slice fields
  double* f2[QPAD_NFIELDS] = {};               // 3D stores (only some fields have one)
  double* qn = nullptr;                        // neutralising background (sum over species)
  double* qraw = nullptr;                      // raw charge deposit scratch
  double* raw = nullptr;                       // raw current deposits of the loop [cu 3|amu 3|acu 2] x P x ld
  unsigned int* iter_tickets = nullptr;        // [0,17) tickets, [64,68) maxima, [127] error word of k_iterate
  int iter_cl = 0, iter_rows = 0;              // cluster size and rows per CTA of k_iterate
  int item_ppl = 4;                            // particles per lane of a mixed deposit work item
  bool pdl = true;                             // k_iterate as programmatic dependent of the deposit
  // (the smoothing order lives in g.smooth)
  struct qpad_guess_state* guess = nullptr;    // learned predictor-corrector guess (learn.cu)
  int extrap = 0;                              // polynomial order of the initial B-perp guess (0: carried)
  double* qbg = nullptr;                       // qn + the ions of every neutral gas (when there is one)
  unsigned int* d_neut_err = nullptr;          // set when a neutral's particle buffer overflowed
  std::vector<struct qpad_laser*> lasers;      // laser envelopes (laser.cu)
  double* la = nullptr;                        // the lasers' sum of a slice: a_r, a_i, their gradients
  double* chi = nullptr;                       // susceptibility of a slice, and its store
  double* chi2 = nullptr;
  double* ltbuf = nullptr;                     // the envelope solve's coupling terms
  double extrap_w = 1.0;                       // weight of the extrapolation's correction to the carried value
  double* conv = nullptr;                      // s_re[nr], s_im[nr], res[8]
  float* gtab = nullptr;                       // FP32 gather table [node][part][E0..2,B0..2] (mixed)
  double* scratch = nullptr;                   // per-call deposit scratch (cu, amu, acu)
  double* beam_scratch = nullptr;              // per-beam charge store scratch
  double* h_res = nullptr;                     // pinned mirror of res
  std::vector<qpad_species*> species;
  std::vector<qpad_beam*> beams;
  std::string err;
  int slice_counter = 0;
  bool field_attr_done = false;
  // device-side loop state of the slice driver
  int* d_j = nullptr;                          // current slice (1-based)
  int* d_iter = nullptr;                       // [0] predictor-corrector iterations in this slice,
                                               // [1 + u] loop ended after part u of an unrolled body
  int unroll = 2;                              // iterations per body of the graph's iteration loop
  int iter_part = -1;                          // part of the unrolled body being captured (-1: none)
  qpad_slice_stats* d_stats = nullptr;         // per-slice statistics [nz]
  int* h_j = nullptr;                          // pinned staging of the slice index
  // CUDA graph of the whole slice loop (WHILE over slices, WHILE over iterations)
  cudaGraphExec_t step_exec = nullptr;
  std::string step_key;                        // configuration the graph was built for
  std::string graph_status;                    // why the graph path is off, if it is
  bool use_graph = true;
  int64_t g_pro = 0, g_it = 0, g_epi = 0;      // kernels per slice prologue / iteration / epilogue
  int64_t g_once = 0;                          // kernels once per graph step
  std::vector<qpad_slice_stats> h_stats;       // per-slice statistics read back after a graph step
  int64_t launches = 0;                        // kernels launched on this context
  // per-kernel-family CUDA-event timing (qpad_profile_enable / qpad_profile_read)
  bool prof_on = false;
  struct Prof { std::vector<cudaEvent_t> pending; double ms = 0.0; int64_t n = 0; };
  std::map<std::string, Prof> prof;
  std::vector<cudaEvent_t> ev_pool;
};

struct qpad_species {
  qpad_ctx* ctx;
  double qbm;
  int push_type, neutralized, sort_freq;
  int64_t np, npmax;
  // SoA particle state; [0] active, [1] scratch for compaction / sorting
  double *x[2], *y[2], *px[2], *py[2], *pz[2], *gamma[2], *psi[2], *q[2];
  int32_t* key = nullptr;       // cell keys / flags
  int32_t* aux = nullptr;       // per-particle rank / index scratch
  int32_t* blk = nullptr;       // per-block counts / histograms
  int64_t blk_cap = 0;
  int64_t* d_count = nullptr;   // device particle count
  int64_t* d_total = nullptr;   // scan total scratch
  int64_t* h_count = nullptr;   // pinned mirror
  double* pristine = nullptr;   // device copy of the last uploaded particles (8 x npmax)
  int64_t np_pristine = 0;
  // mixed-precision state (QPAD_PREC_MIXED): position = (cell + offset) * dr per axis,
  // cell packed as two int16 in cxy, offsets in [0,1); FP32 momenta, charge, gamma, psi.
  int32_t* cxy[2] = {};
  float *fx[2] = {}, *fy[2] = {}, *mpx[2] = {}, *mpy[2] = {}, *mpz[2] = {}, *mq[2] = {}, *mgam[2] = {},
        *mpsi[2] = {};
  int32_t* mkey[2] = {};        // radial cell key 1..nr (nr+1: left the box), sorted ascending
  int32_t* hist = nullptr;      // nr+2 counters
  int32_t* cursor = nullptr;    // nr+2 scatter cursors
  int4* items = nullptr;        // deposit work items {cell, first, count} of the sorted state
  int* d_nitems = nullptr;      // number of work items
  int64_t items_cap = 0;
  void* mixed_block = nullptr;
  void* mixed_pristine = nullptr;
  double* qf = nullptr;         // this species' charge density (finished deposit)
  double* qn = nullptr;         // this species' neutralising background
  struct qpad_neutral_state* neut = nullptr;   // ionisation state when this species is a neutral gas
  int ppc_r = 2;                               // radial particles per cell (chi's axis factor)
};

struct qpad_beam {
  qpad_ctx* ctx;
  double qbm;
  int push_type, evolution;
  int64_t nb, npmax;
  double *x[2], *y[2], *z[2], *px[2], *py[2], *pz[2], *q[2];
  int32_t* key = nullptr;
  int32_t* blk = nullptr;
  int64_t blk_cap = 0;
  int64_t* d_count = nullptr;
  int64_t* d_total = nullptr;
  int32_t* aux = nullptr;
  int64_t* h_count = nullptr;
};

namespace qpad {

// ---- unrolled iteration loop of the step graph ------------------------------------------
// A body of the graph's iteration loop holds `unroll` iterations.  Part u > 0 runs only if
// the loop had not ended after part u - 1: its kernels read that part's flag d_iter[u] (1 =
// ended) and return at once if it is set.  A part's convergence decision writes its own flag
// d_iter[1 + u]; a part that returned at once sets it to 1 for the part after it.
inline const int* iter_guard(const qpad_ctx* ctx) {
  return ctx->iter_part > 0 ? ctx->d_iter + ctx->iter_part : nullptr;
}
inline int* iter_stop_out(const qpad_ctx* ctx) {
  return ctx->iter_part >= 0 && ctx->unroll > 1 ? ctx->d_iter + 1 + ctx->iter_part : nullptr;
}

// ---- status helpers (capi.cu) -----------------------------------------------------------
int set_err(qpad_ctx* ctx, int code, const std::string& msg);
int cuda_check(qpad_ctx* ctx, cudaError_t e, const char* what);
int check_launch(qpad_ctx* ctx, const char* what, int nlaunch = 1);
// CUDA-event bracket of one launch family on ctx->stream (no-ops unless profiling is on)
void prof_begin(qpad_ctx* ctx, const char* name);
void prof_end(qpad_ctx* ctx, const char* name);
void prof_collect(qpad_ctx* ctx);   // folds completed pairs into the totals (stream idle)

// ---- field kernels (fields.cu) ----------------------------------------------------------
int build_factors(qpad_ctx* ctx);
// raises (never lowers) a kernel's dynamic shared-memory limit on the context's device
int raise_dyn_smem(qpad_ctx* ctx, const void* func, size_t bytes);
enum FieldOp {
  FOP_PSI = 0, FOP_BZ, FOP_BT_BEAM, FOP_BT_ITER, FOP_EZ, FOP_ET, FOP_DJDXI
};
struct FieldArgs {
  double* out;        // destination field
  const double* in0;  // first source
  const double* in1;  // second source (psi for ET, cu for BT_ITER, amu for DJDXI)
};
int launch_field_op(qpad_ctx* ctx, int op, FieldArgs a);
// loop_state: count iterations, store per-slice stats, and (use_h) drive the WHILE node h
int launch_conv(qpad_ctx* ctx, const double* b, int comp, int op, int loop_state = 0,
                cudaGraphConditionalHandle h = 0, int use_h = 0);
// ++slice, set the slice WHILE condition, re-arm the iteration WHILE condition
int launch_advance(qpad_ctx* ctx, cudaGraphConditionalHandle hs, cudaGraphConditionalHandle hi);
int launch_set_slice(qpad_ctx* ctx, int j);                         // slice index = j on the device
// fused phases of one slice
int launch_slice_begin(qpad_ctx* ctx, int neutralized_any);   // slice index read from ctx->d_j
int launch_iter_e(qpad_ctx* ctx);
int launch_iter_b(qpad_ctx* ctx);
int launch_slice_end(qpad_ctx* ctx);
int launch_finish_q(qpad_ctx* ctx, const double* raw, double* out, int add_qn, int smooth);
int launch_finish_amj(qpad_ctx* ctx, double* cu, double* amu, double* acu);
// learned guess of the slice's initial B-perp and J-perp predictor (learn.cu)
int guess_enqueue(qpad_ctx* ctx);
void guess_free(qpad_ctx* ctx);
// one predictor-corrector iteration after the deposit, as a cluster kernel (iterate.cu)
int iterate_setup(qpad_ctx* ctx);
int iterate_try_cluster(qpad_ctx* ctx, int cl);
int launch_smooth_raw(qpad_ctx* ctx);
int launch_iterate(qpad_ctx* ctx, int loop_state, cudaGraphConditionalHandle h, int use_h,
                   int after_deposit = 0);

// ---- particle kernels (plasma.cu, beam.cu) ---------------------------------------------
int species_qdeposit_raw(qpad_species* sp, double* qraw);
int qdeposit_arrays(qpad_ctx* ctx, const int64_t* d_count, int64_t n_bound, const double* x, const double* y,
                    const double* q, double* qraw);
// neutral gas species (neutral.cu)
int neutral_step_begin(qpad_ctx* ctx);
int neutral_slice_prologue(qpad_ctx* ctx);
int neutral_slice_update(qpad_ctx* ctx);
bool has_neutrals(const qpad_ctx* ctx);
void neutral_free(qpad_species* sp);
// laser envelopes and the species that see them (laser.cu)
int laser_state_ensure(qpad_ctx* ctx);
int laser_slice_prologue(qpad_ctx* ctx);
int laser_amjdp_raw(qpad_species* sp, const double* ef, const double* bf, double* cu, double* amu, double* acu,
                    double dt);
int laser_push_u(qpad_species* sp, const double* ef, const double* bf, double dt, int fuse_x);
int laser_deposit_chi(qpad_ctx* ctx);
int lasers_advance(qpad_ctx* ctx);
void lasers_free(qpad_ctx* ctx);
inline bool is_pgc(int push_type) { return push_type == QPAD_PUSH2_STD_PGC || push_type == QPAD_PUSH2_ROBUST_PGC; }
int species_amjdp_raw(qpad_species* sp, const double* ef, const double* bf, double* cu, double* amu,
                      double* acu, double dt);
int species_push_u(qpad_species* sp, const double* ef, const double* bf, double dt, int fuse_x);
int species_push_x(qpad_species* sp, double dt);
int species_compact(qpad_species* sp);
int species_sort(qpad_species* sp);
int species_interp_psi(qpad_species* sp, const double* psif);
int species_sync_count(qpad_species* sp);
// ---- mixed-precision particle path (mixed.cu) ------------------------------------------
int mixed_alloc(qpad_species* sp);
void mixed_free(qpad_species* sp);
int mixed_from_fp64(qpad_species* sp);      // FP64 buffers [0] -> mixed state, sorted
int mixed_to_fp64(qpad_species* sp);        // mixed state -> FP64 buffers [0]
int mixed_save_pristine(qpad_species* sp);
int mixed_restore_pristine(qpad_species* sp);
int mixed_qdeposit_raw(qpad_species* sp, double* qraw);
int mixed_amjdp_raw(qpad_species* sp, const float* gtab, double* cu, double* amu, double* acu, double dt);
// push_u (do_u) and/or push_x + update_bound + sort (do_x)
int mixed_push(qpad_species* sp, const float* gtab, double dt, int do_u, int do_x);
int mixed_sort_public(qpad_species* sp);
int mixed_index(qpad_species* sp);          // deposit work items of an already sorted state
int mixed_interp_psi(qpad_species* sp, const double* psif);
int launch_gtab(qpad_ctx* ctx, const double* e, const double* b);   // FP32 gather table of (e, b)

int beam_qdeposit(qpad_beam* bm, double* q2);
int beam_finish_q(qpad_ctx* ctx, double* q2);
int beam_push(qpad_beam* bm, const double* e2, const double* b2);

}  // namespace qpad
