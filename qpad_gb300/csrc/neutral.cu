// neutral.cu -- an ionising neutral gas (the reference's neutral species, neutral_class.f03).
//
// A neutral gas is a plasma species (FP64 path) that starts every 3D step with no electrons.
// Per angle k = 0..n_theta-1 and radial cell j it carries the fractions of the gas in each
// ionisation level 1..L and the neutral fraction, and the mean ionisation quantised to the
// particles per cell.  At the end of every slice the ADK rate of each level, from |E| at the
// cell centre and angle, advances the level cascade over one slice step (ionize_neutral,
// :600-753); every rise of the quantised mean brings new electrons at rest, evenly spaced in
// r across the cell at that angle (add_particles, :755-837), which are then pushed with the
// species.  Their ions stay where they were born: at the next slice start their charge is
// deposited into the gas's ion density rho_ion, which is kept for the rest of the 3D step
// and added to the charge source with the neutralising background (qdeposit_neutral,
// ion_deposit_neutral, :880-930).
//
// Layouts: ionisation state mi[(k * nr + j) * (L + 2) + l], l < L the levels, l = L the
// neutral fraction, l = L + 1 the quantised mean; ion_old[k * nr + j]; ppc_add likewise.
#include <cmath>
#include <new>

#include "qpad_internal.cuh"

struct qpad_neutral_state {
  int levels = 0, num_theta = 0, ppc_tot = 0;
  double wp = 0.0, density = 0.0, coef = 0.0;
  double* adk = nullptr;         // [levels][p1, p2, p3] on the device
  double* mi = nullptr;          // ionisation state
  double* ion_old = nullptr;
  int32_t* add = nullptr;        // new electrons per (angle, cell) of the last update
  double *ax = nullptr, *ay = nullptr, *aq = nullptr;   // their ions (capacity npmax)
  int64_t* d_nadd = nullptr;
  double* raw_add = nullptr;     // ion charge deposit scratch (P x ld)
  double* rho_add = nullptr;
  double* rho_ion = nullptr;     // the gas's ions so far in this 3D step (P x ld)
};

namespace qpad {

struct NeutDev {
  int L, nth, ppc_tot;
  double wp, density, coef;
  const double* adk;
  double* mi;
  double* ion_old;
  int32_t* add;
};

static NeutDev neut_dev(const qpad_neutral_state* n) {
  return NeutDev{n->levels, n->num_theta, n->ppc_tot, n->wp, n->density, n->coef, n->adk, n->mi, n->ion_old, n->add};
}

__global__ void k_neut_reset(NeutDev N, int nr, int64_t* d_count, int64_t* d_nadd) {
  const int ncell = N.nth * nr;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
    for (int l = 0; l < N.L + 2; ++l) N.mi[(size_t)c * (N.L + 2) + l] = l == N.L ? 1.0 : 0.0;
    N.ion_old[c] = 0.0;
    N.add[c] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *d_count = 0;
    *d_nadd = 0;
  }
}

// ionize_neutral (neutral_class.f03:600-753) for one (angle, cell) per thread.  The mode sum
// takes the Re part of mode m for both its Re and its Im term, as the reference does
// (its e_im points at rf_re(m)); kept for identical results.
__global__ void __launch_bounds__(256) k_neut_ionize(GridDev G, NeutDev N, const double* __restrict__ e) {
  const int nr = G.nr, L = N.L;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N.nth * nr) return;
  const int k = c / nr, j = c % nr;               // cell j + 1 of the reference: nodes j + 1, j + 2
  double* mi = N.mi + (size_t)c * (L + 2);
  N.ion_old[c] = mi[L + 1];
  N.add[c] = 0;
  const double pi = 3.14159265358979323846;
  const double theta = 2.0 * pi / (double)N.nth * (double)k;
  const double inc_r = cos(theta), inc_i = sin(theta);
  double ev[3];
#pragma unroll
  for (int cc = 0; cc < 3; ++cc) ev[cc] = 0.5 * (e[fidx(G.ld, 3, 0, cc, j + 1)] + e[fidx(G.ld, 3, 0, cc, j + 2)]);
  double ph_r = 1.0, ph_i = 0.0;
  for (int m = 1; m <= G.M; ++m) {
    const double t = ph_r * inc_r - ph_i * inc_i;
    ph_i = ph_r * inc_i + ph_i * inc_r;
    ph_r = t;
    const int pr = part_re(m);
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      const double er = e[fidx(G.ld, 3, pr, cc, j + 1)] + e[fidx(G.ld, 3, pr, cc, j + 2)];
      ev[cc] = ev[cc] + er * ph_r - er * ph_i;
    }
  }
  const double eij = sqrt(ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2]) * N.wp * 1.708e-12;
  if (!(eij > 1.0e-6) || !(mi[L + 1] < (double)L)) return;
  const double dt = G.dxi;
  const auto rate = [&](int i) {
    return N.adk[3 * i] * pow(eij, -N.adk[3 * i + 2]) * exp(-N.adk[3 * i + 1] / eij) / N.wp;
  };
  bool shoot = false;
  double w = rate(0);
  double cons = mi[L] * w * dt * (1.0 + 0.5 * w * dt);
  if (cons > mi[L]) { shoot = true; cons = mi[L]; }
  mi[L] = mi[L] - cons;
  for (int i = 1; i <= L - 1; ++i) {
    const double inj = cons;
    double dens = 0.0;
    if (shoot) { dens = inj * 0.5; shoot = false; }
    w = rate(i);
    cons = (mi[i - 1] + dens) * w * dt * (1.0 + 0.5 * w * dt);
    if (cons > mi[i - 1] + dens) { shoot = true; cons = mi[i - 1] + dens; }
    mi[i - 1] = fmin(mi[i - 1] - cons + inj, 1.0);
  }
  mi[L - 1] = fmin(mi[L - 1] + cons, 1.0);
  double avg = 0.0;
  for (int i = 1; i <= L; ++i) avg = avg + (double)i * mi[i - 1];
  mi[L + 1] = (double)L / (double)N.ppc_tot * (double)(int)(avg * (double)N.ppc_tot / (double)L + 0.5);
  N.add[c] = (int)((mi[L + 1] - N.ion_old[c]) / (double)L * (double)N.ppc_tot + 0.5);
}

// add_particles (neutral_class.f03:755-837): one CTA; the cells in the reference's order
// (angle, then cell), each cell's new electrons after all earlier cells' (an exclusive scan).
__global__ void __launch_bounds__(1024) k_neut_inject(GridDev G, NeutDev N, int64_t* __restrict__ d_count,
                                                      int64_t npmax, double* x, double* y, double* px, double* py,
                                                      double* pz, double* gam, double* psi, double* q,
                                                      double* ax, double* ay, double* aq, int64_t* d_nadd,
                                                      unsigned int* err) {
  __shared__ int wsum[32];
  __shared__ long long carry_s;
  const int nr = G.nr, ncell = N.nth * nr, t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
  const long long n0 = *d_count;
  if (t == 0) carry_s = 0;
  __syncthreads();
  const double pi = 3.14159265358979323846, dth = 2.0 * pi / (double)N.nth;
  for (int base = 0; base < ncell; base += blockDim.x) {
    const int c = base + t;
    const int a = c < ncell ? N.add[c] : 0;
    int v = a;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int o = __shfl_up_sync(0xffffffffu, v, off);
      if (lane >= off) v += o;
    }
    if (lane == 31) wsum[wid] = v;
    __syncthreads();
    if (wid == 0) {
      int s = lane < nw ? wsum[lane] : 0;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int o = __shfl_up_sync(0xffffffffu, s, off);
        if (lane >= off) s += o;
      }
      wsum[lane] = s;                              // inclusive over warps
    }
    __syncthreads();
    const long long before = carry_s + (wid > 0 ? wsum[wid - 1] : 0) + (v - a);
    const int chunk_total = wsum[nw - 1];
    if (a > 0) {
      const int k = c / nr, j = c % nr;
      const double th = (double)k * dth, cs = cos(th), sn = sin(th);
      for (int i = 1; i <= a; ++i) {
        const long long slot = before + i - 1;
        const long long p = n0 + slot;
        if (p >= npmax) {                          // no room: the step's results are not valid
          atomicOr(err, 1u);
          break;
        }
        const double rn = (double)j + ((double)i - 0.5) / (double)a;
        x[p] = rn * G.dr * cs;
        y[p] = rn * G.dr * sn;
        q[p] = rn * 1.0 * 1.0 * N.density * N.coef;
        px[p] = 0.0; py[p] = 0.0; pz[p] = 0.0;
        gam[p] = 1.0; psi[p] = 0.0;
        ax[slot] = x[p]; ay[slot] = y[p]; aq[slot] = -q[p];
      }
    }
    __syncthreads();
    if (t == 0) carry_s += chunk_total;
    __syncthreads();
  }
  if (t == 0) {
    const long long total = carry_s;
    const long long n1 = n0 + total < npmax ? n0 + total : npmax;
    *d_nadd = n1 - n0;
    *d_count = n1;
  }
}

__global__ void k_neut_sum(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ c,
                           size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    c[i] = a[i] + b[i];
}

static int grid_of(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 4096); }

bool has_neutrals(const qpad_ctx* ctx) {
  for (auto* s : ctx->species)
    if (s->neut) return true;
  return false;
}

int neutral_step_begin(qpad_ctx* ctx) {
  for (auto* s : ctx->species) {
    qpad_neutral_state* n = s->neut;
    if (!n) continue;
    const size_t n1 = (size_t)ctx->g.P * ctx->g.ld;
    k_neut_reset<<<grid_of((size_t)n->num_theta * ctx->g.nr), 256, 0, ctx->stream>>>(neut_dev(n), ctx->g.nr,
                                                                                     s->d_count, n->d_nadd);
    if (cudaMemsetAsync(n->rho_ion, 0, n1 * sizeof(double), ctx->stream) != cudaSuccess)
      return check_launch(ctx, "neutral reset", 0);
    if (int r = check_launch(ctx, "k_neut_reset")) return r;
  }
  if (ctx->d_neut_err && cudaMemsetAsync(ctx->d_neut_err, 0, sizeof(unsigned int), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "neutral error word", 0);
  return 0;
}

// Slice start: the ions born at the end of the previous slice into every gas's rho_ion, and
// the charge background qbg = qn + sum of rho_ion.
int neutral_slice_prologue(qpad_ctx* ctx) {
  if (!ctx->qbg) return 0;
  const size_t n1 = (size_t)ctx->g.P * ctx->g.ld;
  if (cudaMemcpyAsync(ctx->qbg, ctx->qn, n1 * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
    return check_launch(ctx, "qbg", 0);
  for (auto* s : ctx->species) {
    qpad_neutral_state* n = s->neut;
    if (!n) continue;
    if (cudaMemsetAsync(n->raw_add, 0, n1 * sizeof(double), ctx->stream) != cudaSuccess)
      return check_launch(ctx, "ion raw", 0);
    if (int r = qdeposit_arrays(ctx, n->d_nadd, s->npmax, n->ax, n->ay, n->aq, n->raw_add)) return r;
    if (int r = launch_finish_q(ctx, n->raw_add, n->rho_add, 0, 0)) return r;
    k_neut_sum<<<grid_of(n1), 256, 0, ctx->stream>>>(n->rho_ion, n->rho_add, n->rho_ion, n1);
    k_neut_sum<<<grid_of(n1), 256, 0, ctx->stream>>>(ctx->qbg, n->rho_ion, ctx->qbg, n1);
    if (cudaMemsetAsync(n->d_nadd, 0, sizeof(int64_t), ctx->stream) != cudaSuccess)
      return check_launch(ctx, "ion count", 0);
    if (int r = check_launch(ctx, "neutral ions", 2)) return r;
  }
  return 0;
}

// Slice end (before the species push): ionisation and the new electrons of every gas.
int neutral_slice_update(qpad_ctx* ctx) {
  for (auto* s : ctx->species) {
    qpad_neutral_state* n = s->neut;
    if (!n) continue;
    const int ncell = n->num_theta * ctx->g.nr;
    k_neut_ionize<<<(ncell + 255) / 256, 256, 0, ctx->stream>>>(ctx->g, neut_dev(n), ctx->f[QPAD_F_E]);
    k_neut_inject<<<1, 1024, 0, ctx->stream>>>(ctx->g, neut_dev(n), s->d_count, s->npmax, s->x[0], s->y[0],
                                               s->px[0], s->py[0], s->pz[0], s->gamma[0], s->psi[0], s->q[0], n->ax,
                                               n->ay, n->aq, n->d_nadd, ctx->d_neut_err);
    if (int r = check_launch(ctx, "neutral update", 2)) return r;
  }
  return 0;
}

void neutral_free(qpad_species* sp) {
  qpad_neutral_state* n = sp->neut;
  if (!n) return;
  void* ptrs[] = {n->adk, n->mi, n->ion_old, n->add, n->ax, n->ay, n->aq, n->d_nadd, n->raw_add, n->rho_add,
                  n->rho_ion};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete n;
  sp->neut = nullptr;
}

}  // namespace qpad

using namespace qpad;

namespace {
int nmalloc(qpad_ctx* ctx, void** p, size_t bytes, const char* what) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return set_err(ctx, QPAD_E_NOMEM, std::string("cudaMalloc(") + what + ")");
  }
  return 0;
}
}  // namespace

extern "C" int qpad_neutral_create(qpad_ctx* ctx, const qpad_neutral_desc* d, qpad_species** out) {
  if (!ctx || !d || !out) return QPAD_E_ARG;
  *out = nullptr;
  if (ctx->precision != QPAD_PREC_FP64) return set_err(ctx, QPAD_E_ARG, "neutral gas: built on the FP64 path only");
  if (ctx->g.smooth != 0) return set_err(ctx, QPAD_E_ARG, "neutral gas: needs smooth_order 0");
  if (is_pgc(d->push_type)) return set_err(ctx, QPAD_E_ARG, "neutral gas: the reference pushes its electrons without lasers");
  if (d->levels < 1 || d->levels > 16 || !d->adk || !(d->wp > 0.0) || !(d->density > 0.0) || d->ppc1 < 1 ||
      d->ppc2 < 1 || d->num_theta < 1 || d->npmax < 1 || d->qm == 0.0 || d->qbm == 0.0)
    return set_err(ctx, QPAD_E_ARG, "invalid neutral gas descriptor");
  qpad_species_desc sd;
  sd.qbm = d->qbm;
  sd.push_type = d->push_type;
  sd.neutralized = 0;
  sd.npmax = d->npmax;
  sd.sort_freq = 0;
  qpad_species* sp = nullptr;
  if (int r = qpad_species_create(ctx, &sd, nullptr, nullptr, nullptr, nullptr, nullptr, 0, &sp)) return r;
  qpad_neutral_state* n = new (std::nothrow) qpad_neutral_state();
  if (!n) {
    qpad_species_destroy(sp);
    return set_err(ctx, QPAD_E_NOMEM, "neutral state");
  }
  sp->neut = n;
  n->levels = d->levels;
  n->num_theta = d->num_theta;
  n->ppc_tot = d->ppc1 * d->ppc2;
  n->wp = d->wp;
  n->density = d->density;
  n->coef = (double)d->levels * (d->qm < 0.0 ? -1.0 : 1.0) / ((double)n->ppc_tot * (double)d->num_theta);
  const size_t ncell = (size_t)d->num_theta * ctx->g.nr, n1 = (size_t)ctx->g.P * ctx->g.ld;
  int r = nmalloc(ctx, (void**)&n->adk, sizeof(double) * 3 * d->levels, "neutral rates");
  if (!r) r = nmalloc(ctx, (void**)&n->mi, sizeof(double) * ncell * (d->levels + 2), "ionisation state");
  if (!r) r = nmalloc(ctx, (void**)&n->ion_old, sizeof(double) * ncell, "ionisation state");
  if (!r) r = nmalloc(ctx, (void**)&n->add, sizeof(int32_t) * ncell, "new electrons");
  if (!r) r = nmalloc(ctx, (void**)&n->ax, sizeof(double) * d->npmax, "ions");
  if (!r) r = nmalloc(ctx, (void**)&n->ay, sizeof(double) * d->npmax, "ions");
  if (!r) r = nmalloc(ctx, (void**)&n->aq, sizeof(double) * d->npmax, "ions");
  if (!r) r = nmalloc(ctx, (void**)&n->d_nadd, sizeof(int64_t), "ion count");
  if (!r) r = nmalloc(ctx, (void**)&n->raw_add, sizeof(double) * n1, "ion deposit");
  if (!r) r = nmalloc(ctx, (void**)&n->rho_add, sizeof(double) * n1, "ion deposit");
  if (!r) r = nmalloc(ctx, (void**)&n->rho_ion, sizeof(double) * n1, "ion density");
  if (!r && !ctx->qbg) r = nmalloc(ctx, (void**)&ctx->qbg, sizeof(double) * n1, "charge background");
  if (!r && !ctx->d_neut_err) r = nmalloc(ctx, (void**)&ctx->d_neut_err, sizeof(unsigned int), "neutral error");
  if (!r) r = cuda_check(ctx, cudaMemcpyAsync(n->adk, d->adk, sizeof(double) * 3 * d->levels, cudaMemcpyHostToDevice,
                                              ctx->stream), "neutral rates");
  // every launch of the species covers its capacity: the electrons are born on the device
  sp->np = sp->npmax;
  if (!r) r = neutral_step_begin(ctx);
  if (!r) r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "neutral create");
  if (r) {
    qpad_species_destroy(sp);
    return r;
  }
  ctx->step_key.clear();
  *out = sp;
  return 0;
}

extern "C" int qpad_neutral_state_download(qpad_species* sp, double* state) {
  if (!sp || !sp->neut || !state) return sp ? set_err(sp->ctx, QPAD_E_ARG, "not a neutral gas") : QPAD_E_ARG;
  qpad_ctx* ctx = sp->ctx;
  const size_t n = (size_t)sp->neut->num_theta * ctx->g.nr * (sp->neut->levels + 2);
  if (int r = cuda_check(ctx, cudaMemcpyAsync(state, sp->neut->mi, n * sizeof(double), cudaMemcpyDeviceToHost,
                                              ctx->stream), "ionisation state"))
    return r;
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "ionisation state");
}
