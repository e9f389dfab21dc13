// capi.cu -- the C ABI (include/qpad_gpu.h): contexts, fields, species, beams and the
// fused slice / 3D-step drivers of run_simulation (simulation_class.f03:294-512).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "particles.cuh"

using namespace qpad;

namespace qpad {

int set_err(qpad_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_check(qpad_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return QPAD_OK;
  return set_err(ctx, QPAD_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int check_launch(qpad_ctx* ctx, const char* what, int nlaunch) {
  if (ctx) ctx->launches += nlaunch;
  return cuda_check(ctx, cudaGetLastError(), what);
}

static cudaEvent_t ev_get(qpad_ctx* ctx) {
  if (!ctx->ev_pool.empty()) {
    cudaEvent_t e = ctx->ev_pool.back();
    ctx->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void prof_begin(qpad_ctx* ctx, const char* name) {
  if (!ctx->prof_on) return;
  cudaEvent_t e = ev_get(ctx);
  cudaEventRecord(e, ctx->stream);
  ctx->prof[name].pending.push_back(e);
}

void prof_end(qpad_ctx* ctx, const char* name) {
  if (!ctx->prof_on) return;
  cudaEvent_t e = ev_get(ctx);
  cudaEventRecord(e, ctx->stream);
  ctx->prof[name].pending.push_back(e);
}

void prof_collect(qpad_ctx* ctx) {
  for (auto& kv : ctx->prof) {
    auto& pr = kv.second;
    const size_t npair = pr.pending.size() / 2;
    for (size_t k = 0; k < npair; ++k) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, pr.pending[2 * k], pr.pending[2 * k + 1]) == cudaSuccess) {
        pr.ms += ms;
        pr.n += 1;
      }
      ctx->ev_pool.push_back(pr.pending[2 * k]);
      ctx->ev_pool.push_back(pr.pending[2 * k + 1]);
    }
    pr.pending.erase(pr.pending.begin(), pr.pending.begin() + 2 * npair);
  }
  cudaGetLastError();
}

}  // namespace qpad

namespace {

static thread_local std::string g_create_err;

bool has_store(int f) {
  switch (f) {
    case QPAD_F_Q_BEAM: case QPAD_F_E: case QPAD_F_B: case QPAD_F_PSI: case QPAD_F_B_SPE:
    case QPAD_F_E_SPE: case QPAD_F_CU: case QPAD_F_Q_SPE: return true;
    default: return false;
  }
}

size_t f1_elems(const qpad_ctx* c, int f) { return (size_t)c->g.P * field_ncomp(f) * c->g.ld; }
size_t f2_elems(const qpad_ctx* c, int f) { return f1_elems(c, f) * (size_t)(c->g.nz + 1); }

int dmalloc(qpad_ctx* ctx, void** p, size_t bytes, const char* what) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 8);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, e == cudaErrorMemoryAllocation ? QPAD_E_NOMEM : QPAD_E_CUDA,
                   std::string("cudaMalloc(") + what + "): " + cudaGetErrorString(e));
  }
  return cudaMemsetAsync(*p, 0, bytes ? bytes : 8, ctx->stream) == cudaSuccess ? 0 : QPAD_E_CUDA;
}

bool valid_field(int f) { return f >= 0 && f < QPAD_NFIELDS; }

// ---- small elementwise kernels over whole slice fields ------------------------------
__global__ void k_fill(double* a, size_t n, double v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) a[i] = v;
}
__global__ void k_add(const double* a, const double* b, double* c, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    c[i] = a[i] + b[i];
}
__global__ void k_add2(double* q, const double* a, const double* b, size_t n) {   // q = (q + a) + b
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double v = q[i] + a[i];
    if (b) v = v + b[i];
    q[i] = v;
  }
}
__global__ void k_scale(double* a, size_t n, double s) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    a[i] = a[i] * s;
}
// b(bdim,:) += a(adim,:) for every mode part
__global__ void k_add_dim(const double* a, int nca, int ca, double* b, int ncb, int cb, int P, int ld) {
  const int p = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ld; i += gridDim.x * blockDim.x) {
    double* d = b + ((size_t)p * ncb + cb) * ld + i;
    *d = *d + a[((size_t)p * nca + ca) * ld + i];
  }
}
__global__ void k_neg(const double* a, double* b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = a[i] * -1.0;
}
__global__ void k_deinterleave(const double* __restrict__ src, int64_t n, int nc, double* d0, double* d1,
                               double* d2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  d0[i] = src[nc * i];
  d1[i] = src[nc * i + 1];
  if (nc == 3) d2[i] = src[nc * i + 2];
}
__global__ void k_interleave(double* __restrict__ dst, int64_t n, int nc, const double* d0, const double* d1,
                             const double* d2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  dst[nc * i] = d0[i];
  dst[nc * i + 1] = d1[i];
  if (nc == 3) dst[nc * i + 2] = d2[i];
}

int elem_grid(size_t n) {
  size_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

// ---- particle upload / download (Fortran layouts x(nc,np), p(3,np)) ------------------
int upload_vec(qpad_ctx* ctx, double* staging, const double* host, int64_t n, int nc, double* d0, double* d1,
               double* d2) {
  if (n == 0) return 0;
  cudaError_t e = cudaMemcpyAsync(staging, host, sizeof(double) * nc * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "upload");
  k_deinterleave<<<(int)((n + 255) / 256), 256, 0, ctx->stream>>>(staging, n, nc, d0, d1, d2);
  return check_launch(ctx, "deinterleave");
}

int download_vec(qpad_ctx* ctx, double* staging, double* host, int64_t n, int nc, const double* d0, const double* d1,
                 const double* d2) {
  if (n == 0) return 0;
  k_interleave<<<(int)((n + 255) / 256), 256, 0, ctx->stream>>>(staging, n, nc, d0, d1, d2);
  if (int r = check_launch(ctx, "interleave")) return r;
  cudaError_t e = cudaMemcpyAsync(host, staging, sizeof(double) * nc * n, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "download");
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "download sync");
}

int h2d(qpad_ctx* ctx, double* d, const double* h, int64_t n) {
  if (n == 0) return 0;
  return cuda_check(ctx, cudaMemcpyAsync(d, h, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream), "h2d");
}
int d2h(qpad_ctx* ctx, double* h, const double* d, int64_t n) {
  if (n == 0) return 0;
  return cuda_check(ctx, cudaMemcpyAsync(h, d, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream), "d2h");
}

// neutralising background of one species: qn = -(finished charge deposit) (species2d_class.f03:114-129)
int species_set_background(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  const size_t n1 = f1_elems(ctx, QPAD_F_Q_SPE);
  if (cudaMemsetAsync(ctx->qraw, 0, n1 * sizeof(double), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "memset qraw");
  if (int r = species_qdeposit_raw(sp, ctx->qraw)) return r;
  if (int r = launch_finish_q(ctx, ctx->qraw, sp->qf, 0, 0)) return r;   // qn is not smoothed
  k_neg<<<elem_grid(n1), 256, 0, ctx->stream>>>(sp->qf, sp->qn, n1);
  return check_launch(ctx, "qn");
}

// ctx->qn = sum of the neutralised species' backgrounds
int rebuild_total_background(qpad_ctx* ctx) {
  const size_t n1 = f1_elems(ctx, QPAD_F_Q_SPE);
  if (cudaMemsetAsync(ctx->qn, 0, n1 * sizeof(double), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "memset qn");
  for (qpad_species* s : ctx->species)
    if (s->neutralized) {
      k_add<<<elem_grid(n1), 256, 0, ctx->stream>>>(ctx->qn, s->qn, ctx->qn, n1);
      if (int r = check_launch(ctx, "qn sum")) return r;
    }
  return 0;
}

int save_pristine(qpad_species* sp) {
  qpad_ctx* ctx = sp->ctx;
  const double* src[8] = {sp->x[0], sp->y[0], sp->px[0], sp->py[0], sp->pz[0], sp->gamma[0], sp->psi[0], sp->q[0]};
  for (int a = 0; a < 8; ++a)
    if (sp->np > 0 && cudaMemcpyAsync(sp->pristine + (size_t)a * sp->npmax, src[a], sizeof(double) * sp->np,
                                      cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
      return check_launch(ctx, "pristine copy");
  sp->np_pristine = sp->np;
  return 0;
}

int species_load(qpad_species* sp, const double* x, const double* p, const double* gamma, const double* psi,
                 const double* q, int64_t np) {
  qpad_ctx* ctx = sp->ctx;
  if (np < 0 || np > sp->npmax) return set_err(ctx, QPAD_E_CAPACITY, "particle count exceeds npmax");
  if (np > 0 && (!x || !p || !gamma || !psi || !q)) return set_err(ctx, QPAD_E_ARG, "null particle array");
  sp->np = np;
  double* staging = sp->x[1];   // scratch buffers are 8 * npmax doubles in total (contiguous)
  if (int r = upload_vec(ctx, staging, x, np, 2, sp->x[0], sp->y[0], nullptr)) return r;
  if (int r = upload_vec(ctx, staging + 2 * np, p, np, 3, sp->px[0], sp->py[0], sp->pz[0])) return r;
  if (int r = h2d(ctx, sp->gamma[0], gamma, np)) return r;
  if (int r = h2d(ctx, sp->psi[0], psi, np)) return r;
  if (int r = h2d(ctx, sp->q[0], q, np)) return r;
  *sp->h_count = np;
  if (cudaMemcpyAsync(sp->d_count, sp->h_count, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
    return check_launch(ctx, "count upload");
  if (int r = save_pristine(sp)) return r;
  // the neutralising background is deposited in FP64 from the FP64 particles in both paths
  if (int r = species_set_background(sp)) return r;
  if (int r = rebuild_total_background(ctx)) return r;
  if (ctx->precision == QPAD_PREC_MIXED) {
    if (int r = mixed_from_fp64(sp)) return r;           // convert + sort by cell
    if (int r = species_sync_count(sp)) return r;
    sp->np_pristine = sp->np;
    if (int r = mixed_save_pristine(sp)) return r;
  }
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "species load");
}

bool is_mixed(const qpad_species* sp) { return sp->ctx->precision == QPAD_PREC_MIXED; }

// FP64 buffers [0] mirror the mixed state before any read of particle data
int sync_fp64_view(qpad_species* sp) { return is_mixed(sp) ? mixed_to_fp64(sp) : 0; }

int beam_load(qpad_beam* bm, const double* x, const double* p, const double* q, int64_t nb) {
  qpad_ctx* ctx = bm->ctx;
  if (nb < 0 || nb > bm->npmax) return set_err(ctx, QPAD_E_CAPACITY, "beam particle count exceeds npmax");
  if (nb > 0 && (!x || !p || !q)) return set_err(ctx, QPAD_E_ARG, "null beam array");
  bm->nb = nb;
  double* staging = bm->x[1];
  if (int r = upload_vec(ctx, staging, x, nb, 3, bm->x[0], bm->y[0], bm->z[0])) return r;
  if (int r = upload_vec(ctx, staging + 3 * nb, p, nb, 3, bm->px[0], bm->py[0], bm->pz[0])) return r;
  if (int r = h2d(ctx, bm->q[0], q, nb)) return r;
  *bm->h_count = nb;
  if (cudaMemcpyAsync(bm->d_count, bm->h_count, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
    return check_launch(ctx, "count upload");
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "beam load");
}

int beam_sync_count(qpad_beam* bm) {
  qpad_ctx* ctx = bm->ctx;
  cudaError_t e = cudaMemcpyAsync(bm->h_count, bm->d_count, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "beam count");
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_check(ctx, e, "beam count sync");
  bm->nb = *bm->h_count;
  return 0;
}

}  // namespace

// =====================================================================================
// context
// =====================================================================================
extern "C" int qpad_ctx_create(const qpad_grid_desc* d, qpad_ctx** out) {
  if (!d || !out) return QPAD_E_ARG;
  *out = nullptr;
  if (d->nr < 8 || d->nr > 4096 || d->nz < 1 || d->max_mode < 0 || d->max_mode > QPAD_MAX_MODE || !(d->dr > 0) ||
      !(d->dxi > 0) || d->iter_max < 1 || (d->bnd != QPAD_BND_OPEN && d->bnd != QPAD_BND_ZERO)) {
    g_create_err = "invalid grid descriptor (8 <= nr <= 4096, 0 <= max_mode <= 8, dr, dxi > 0, iter_max >= 1)";
    return QPAD_E_ARG;
  }
  qpad_ctx* ctx = new (std::nothrow) qpad_ctx();
  if (!ctx) return QPAD_E_NOMEM;
  GridDev& g = ctx->g;
  g.nr = d->nr; g.nz = d->nz; g.M = d->max_mode; g.P = 2 * d->max_mode + 1; g.ld = d->nr + 2; g.bnd = d->bnd;
  g.dr = d->dr; g.dxi = d->dxi; g.idr = 1.0 / d->dr; g.toff = 0; g.smooth = 0;
  g.relax_fac = d->relax_fac >= 0.0 ? d->relax_fac : 1.0e-3 * ((d->dr / 0.02) * (d->dr / 0.02));
  ctx->iter_max = d->iter_max; ctx->reltol = d->iter_reltol; ctx->abstol = d->iter_abstol; ctx->dt = d->dt;
  ctx->precision = d->precision; ctx->device = d->device;
  int r = cuda_check(ctx, cudaSetDevice(d->device), "cudaSetDevice");
  if (!r) r = cuda_check(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream");
  for (int f = 0; f < QPAD_NFIELDS && !r; ++f) {
    r = dmalloc(ctx, (void**)&ctx->f[f], f1_elems(ctx, f) * sizeof(double), "field");
    if (!r && has_store(f)) r = dmalloc(ctx, (void**)&ctx->f2[f], f2_elems(ctx, f) * sizeof(double), "store");
  }
  if (!r) r = dmalloc(ctx, (void**)&ctx->qn, f1_elems(ctx, QPAD_F_Q_SPE) * sizeof(double), "qn");
  if (!r) r = dmalloc(ctx, (void**)&ctx->qraw, f1_elems(ctx, QPAD_F_Q_SPE) * sizeof(double), "qraw");
  if (!r) r = dmalloc(ctx, (void**)&ctx->conv, (2 * (size_t)g.nr + 8) * sizeof(double), "conv");
  if (!r && ctx->precision == QPAD_PREC_MIXED)
    r = dmalloc(ctx, (void**)&ctx->gtab, (size_t)g.ld * g.P * 6 * sizeof(float), "gather table");
  if (!r) r = dmalloc(ctx, (void**)&ctx->d_j, 2 * sizeof(int), "slice index");
  if (!r) r = dmalloc(ctx, (void**)&ctx->d_iter, (1 + kMaxUnroll) * sizeof(int), "iteration counter");
  if (!r) r = dmalloc(ctx, (void**)&ctx->d_stats, (size_t)g.nz * sizeof(qpad_slice_stats), "slice stats");
  if (!r) r = cuda_check(ctx, cudaMallocHost((void**)&ctx->h_j, 2 * sizeof(int)), "pinned slice index");
  if (!r) r = cuda_check(ctx, cudaMallocHost((void**)&ctx->h_res, 8 * sizeof(double)), "pinned");
  if (!r) r = dmalloc(ctx, (void**)&ctx->raw, 8 * (size_t)g.P * g.ld * sizeof(double), "raw deposits");
  if (!r) r = dmalloc(ctx, (void**)&ctx->iter_tickets, 128 * sizeof(unsigned int), "iteration tickets");
  if (!r) r = cuda_check(ctx, cudaMemsetAsync(ctx->raw, 0, 8 * (size_t)g.P * g.ld * sizeof(double), ctx->stream),
                         "raw deposits");
  if (!r) r = cuda_check(ctx, cudaMemsetAsync(ctx->iter_tickets, 0, 128 * sizeof(unsigned int), ctx->stream),
                         "iteration tickets");
  if (!r) r = build_factors(ctx);
  if (!r) r = iterate_setup(ctx);
  if (!r) r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "create sync");
  if (r) {
    g_create_err = ctx->err;
    qpad_ctx_destroy(ctx);
    return r;
  }
  *out = ctx;
  return QPAD_OK;
}

extern "C" int qpad_ctx_destroy(qpad_ctx* ctx) {
  if (!ctx) return QPAD_OK;
  std::vector<qpad_species*> sps = ctx->species;
  for (auto* s : sps) qpad_species_destroy(s);
  std::vector<qpad_beam*> bms = ctx->beams;
  for (auto* b : bms) qpad_beam_destroy(b);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (int f = 0; f < QPAD_NFIELDS; ++f) {
    if (ctx->f[f]) cudaFree(ctx->f[f]);
    if (ctx->f2[f]) cudaFree(ctx->f2[f]);
  }
  if (ctx->fac) cudaFree(ctx->fac);
  if (ctx->rtab) cudaFree(ctx->rtab);
  if (ctx->qn) cudaFree(ctx->qn);
  if (ctx->qbg) cudaFree(ctx->qbg);
  if (ctx->d_neut_err) cudaFree(ctx->d_neut_err);
  lasers_free(ctx);
  guess_free(ctx);
  if (ctx->qraw) cudaFree(ctx->qraw);
  if (ctx->raw) cudaFree(ctx->raw);
  if (ctx->iter_tickets) cudaFree(ctx->iter_tickets);
  if (ctx->conv) cudaFree(ctx->conv);
  if (ctx->scratch) cudaFree(ctx->scratch);
  if (ctx->gtab) cudaFree(ctx->gtab);
  if (ctx->beam_scratch) cudaFree(ctx->beam_scratch);
  if (ctx->d_j) cudaFree(ctx->d_j);
  if (ctx->d_iter) cudaFree(ctx->d_iter);
  if (ctx->d_stats) cudaFree(ctx->d_stats);
  if (ctx->h_j) cudaFreeHost(ctx->h_j);
  if (ctx->step_exec) cudaGraphExecDestroy(ctx->step_exec);
  if (ctx->h_res) cudaFreeHost(ctx->h_res);
  prof_collect(ctx);
  for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return QPAD_OK;
}

extern "C" const char* qpad_last_error(const qpad_ctx* ctx) {
  if (!ctx) return g_create_err.c_str();
  return ctx->err.c_str();
}

extern "C" int qpad_synchronize(qpad_ctx* ctx) {
  if (!ctx) return QPAD_E_ARG;
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "synchronize");
}

extern "C" int qpad_field_layout(const qpad_ctx* ctx, int field, int* ncomp, int64_t* ld) {
  if (!ctx || !valid_field(field)) return QPAD_E_ARG;
  if (ncomp) *ncomp = field_ncomp(field);
  if (ld) *ld = ctx->g.ld;
  return QPAD_OK;
}

extern "C" int qpad_device_count(int* count) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  if (count) *count = n;
  return QPAD_OK;
}

extern "C" int qpad_set_graph(qpad_ctx* ctx, int on) {
  if (!ctx) return QPAD_E_ARG;
  ctx->use_graph = on != 0;
  if (on) ctx->graph_status.clear();
  return QPAD_OK;
}

extern "C" int qpad_graph_active(const qpad_ctx* ctx, int* active) {
  if (!ctx || !active) return QPAD_E_ARG;
  *active = (ctx->use_graph && ctx->step_exec != nullptr) ? 1 : 0;
  return QPAD_OK;
}

extern "C" int qpad_set_smooth(qpad_ctx* ctx, int order) {
  if (!ctx) return QPAD_E_ARG;
  if (order < 0 || order > kMaxSmoothOrder)
    return set_err(ctx, QPAD_E_ARG, "smooth order: 0 .. " + std::to_string(kMaxSmoothOrder));
  if (order > 0 && has_neutrals(ctx)) return set_err(ctx, QPAD_E_ARG, "smoothing with a neutral gas is not built");
  const int old = ctx->g.smooth;
  ctx->g.smooth = order;
  // the iteration kernel's shared memory grows with smoothing: check its shape still fits
  if (ctx->iter_cl > 0 && iterate_try_cluster(ctx, ctx->iter_cl) != 0) {
    cudaGetLastError();
    ctx->g.smooth = old;
    iterate_try_cluster(ctx, ctx->iter_cl);
    return set_err(ctx, QPAD_E_CAPACITY, "smoothing scratch does not fit the iteration kernel's shape");
  }
  return QPAD_OK;
}

extern "C" const char* qpad_graph_status(const qpad_ctx* ctx) { return ctx ? ctx->graph_status.c_str() : ""; }

extern "C" int qpad_launch_count(const qpad_ctx* ctx, int64_t* count) {
  if (!ctx || !count) return QPAD_E_ARG;
  *count = ctx->launches;
  return QPAD_OK;
}

extern "C" int qpad_profile_enable(qpad_ctx* ctx, int on) {
  if (!ctx) return QPAD_E_ARG;
  if (int r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "profile sync")) return r;
  prof_collect(ctx);
  ctx->prof_on = on != 0;
  if (on) ctx->prof.clear();
  return QPAD_OK;
}

extern "C" int qpad_profile_read(qpad_ctx* ctx, const char* name, double* total_ms, int64_t* launches) {
  if (!ctx || !name) return QPAD_E_ARG;
  if (int r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "profile sync")) return r;
  prof_collect(ctx);
  auto it = ctx->prof.find(name);
  if (total_ms) *total_ms = it == ctx->prof.end() ? 0.0 : it->second.ms;
  if (launches) *launches = it == ctx->prof.end() ? 0 : it->second.n;
  return QPAD_OK;
}

// =====================================================================================
// fields
// =====================================================================================
namespace {
int part_ok(const qpad_ctx* ctx, int part) { return part >= 0 && part < ctx->g.P; }

// host f1(dim, 0:nr+1) <-> device [c][i] line block of one part
int f1_transfer(qpad_ctx* ctx, double* dev_part, int nc, double* host, bool upload) {
  const int ld = ctx->g.ld;
  std::vector<double> tmp((size_t)nc * ld);
  if (upload) {
    for (int i = 0; i < ld; ++i)
      for (int c = 0; c < nc; ++c) tmp[(size_t)c * ld + i] = host[(size_t)i * nc + c];
    if (int r = h2d(ctx, dev_part, tmp.data(), (int64_t)nc * ld)) return r;
    return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "upload sync");
  }
  if (int r = d2h(ctx, tmp.data(), dev_part, (int64_t)nc * ld)) return r;
  if (int r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "download sync")) return r;
  for (int i = 0; i < ld; ++i)
    for (int c = 0; c < nc; ++c) host[(size_t)i * nc + c] = tmp[(size_t)c * ld + i];
  return 0;
}
}  // namespace

extern "C" int qpad_field_upload(qpad_ctx* ctx, int field, int part, const double* f1) {
  if (!ctx || !valid_field(field) || !part_ok(ctx, part) || !f1) return ctx ? set_err(ctx, QPAD_E_ARG, "bad args") : QPAD_E_ARG;
  const int nc = field_ncomp(field);
  return f1_transfer(ctx, ctx->f[field] + (size_t)part * nc * ctx->g.ld, nc, const_cast<double*>(f1), true);
}

extern "C" int qpad_field_download(qpad_ctx* ctx, int field, int part, double* f1) {
  if (!ctx || !valid_field(field) || !part_ok(ctx, part) || !f1) return ctx ? set_err(ctx, QPAD_E_ARG, "bad args") : QPAD_E_ARG;
  const int nc = field_ncomp(field);
  return f1_transfer(ctx, ctx->f[field] + (size_t)part * nc * ctx->g.ld, nc, f1, false);
}

extern "C" int qpad_store_download(qpad_ctx* ctx, int field, int slice, int part, double* f1) {
  if (!ctx || !valid_field(field) || !has_store(field) || !part_ok(ctx, part) || !f1 || slice < 1 ||
      slice > ctx->g.nz + 1)
    return ctx ? set_err(ctx, QPAD_E_ARG, "bad store args") : QPAD_E_ARG;
  const int nc = field_ncomp(field);
  double* dev = ctx->f2[field] + ((size_t)(slice - 1) * ctx->g.P + part) * nc * ctx->g.ld;
  return f1_transfer(ctx, dev, nc, f1, false);
}

extern "C" int qpad_store_upload(qpad_ctx* ctx, int field, int slice, int part, const double* f1) {
  if (!ctx || !valid_field(field) || !has_store(field) || !part_ok(ctx, part) || !f1 || slice < 1 ||
      slice > ctx->g.nz + 1)
    return ctx ? set_err(ctx, QPAD_E_ARG, "bad store args") : QPAD_E_ARG;
  const int nc = field_ncomp(field);
  double* dev = ctx->f2[field] + ((size_t)(slice - 1) * ctx->g.P + part) * nc * ctx->g.ld;
  return f1_transfer(ctx, dev, nc, const_cast<double*>(f1), true);
}

extern "C" int qpad_store_read(qpad_ctx* ctx, int field, int slice_lo, int nslices, double* host) {
  if (!ctx || !valid_field(field) || !has_store(field) || !host || nslices < 0 || slice_lo < 1 ||
      (int64_t)slice_lo + nslices - 1 > ctx->g.nz + 1)
    return ctx ? set_err(ctx, QPAD_E_ARG, "bad store range") : QPAD_E_ARG;
  const size_t per = f1_elems(ctx, field);
  if (nslices == 0) return 0;
  if (int r = cuda_check(ctx, cudaMemcpyAsync(host, ctx->f2[field] + (size_t)(slice_lo - 1) * per,
                                              per * (size_t)nslices * sizeof(double), cudaMemcpyDeviceToHost,
                                              ctx->stream), "store read"))
    return r;
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "store read sync");
}

extern "C" int qpad_field_fill(qpad_ctx* ctx, int field, double v) {
  if (!ctx || !valid_field(field)) return QPAD_E_ARG;
  const size_t n = f1_elems(ctx, field);
  k_fill<<<elem_grid(n), 256, 0, ctx->stream>>>(ctx->f[field], n, v);
  return check_launch(ctx, "fill");
}

extern "C" int qpad_store_fill(qpad_ctx* ctx, int field, double v) {
  if (!ctx || !valid_field(field) || !has_store(field)) return ctx ? set_err(ctx, QPAD_E_ARG, "no store") : QPAD_E_ARG;
  const size_t n = f2_elems(ctx, field);
  k_fill<<<elem_grid(n), 256, 0, ctx->stream>>>(ctx->f2[field], n, v);
  return check_launch(ctx, "store fill");
}

extern "C" int qpad_field_add(qpad_ctx* ctx, int a, int b, int c) {
  if (!ctx || !valid_field(a) || !valid_field(b) || !valid_field(c) || field_ncomp(a) != field_ncomp(c) ||
      field_ncomp(b) != field_ncomp(c))
    return ctx ? set_err(ctx, QPAD_E_ARG, "field_add: mismatched fields") : QPAD_E_ARG;
  const size_t n = f1_elems(ctx, c);
  k_add<<<elem_grid(n), 256, 0, ctx->stream>>>(ctx->f[a], ctx->f[b], ctx->f[c], n);
  return check_launch(ctx, "add");
}

extern "C" int qpad_field_add_dim(qpad_ctx* ctx, int a, int b, const int32_t* adim, const int32_t* bdim, int n) {
  if (!ctx || !valid_field(a) || !valid_field(b) || !adim || !bdim || n < 0) return QPAD_E_ARG;
  for (int k = 0; k < n; ++k) {
    if (adim[k] < 1 || adim[k] > field_ncomp(a) || bdim[k] < 1 || bdim[k] > field_ncomp(b))
      return set_err(ctx, QPAD_E_ARG, "add_dim: component out of range");
    dim3 grid((ctx->g.ld + 255) / 256, ctx->g.P);
    k_add_dim<<<grid, 256, 0, ctx->stream>>>(ctx->f[a], field_ncomp(a), adim[k] - 1, ctx->f[b], field_ncomp(b),
                                             bdim[k] - 1, ctx->g.P, ctx->g.ld);
    if (int r = check_launch(ctx, "add_dim")) return r;
  }
  return QPAD_OK;
}

extern "C" int qpad_field_scale(qpad_ctx* ctx, int field, double s) {
  if (!ctx || !valid_field(field)) return QPAD_E_ARG;
  const size_t n = f1_elems(ctx, field);
  k_scale<<<elem_grid(n), 256, 0, ctx->stream>>>(ctx->f[field], n, s);
  return check_launch(ctx, "scale");
}

extern "C" int qpad_field_copy_slice(qpad_ctx* ctx, int field, int slice, int dir) {
  if (!ctx || !valid_field(field) || !has_store(field) || slice < 1 || slice > ctx->g.nz + 1 ||
      (dir != QPAD_COPY_1TO2 && dir != QPAD_COPY_2TO1))
    return ctx ? set_err(ctx, QPAD_E_ARG, "copy_slice: bad args") : QPAD_E_ARG;
  const size_t n = f1_elems(ctx, field);
  double* s2 = ctx->f2[field] + (size_t)(slice - 1) * n;
  double* dst = dir == QPAD_COPY_1TO2 ? s2 : ctx->f[field];
  const double* src = dir == QPAD_COPY_1TO2 ? ctx->f[field] : s2;
  return cuda_check(ctx, cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream),
                    "copy_slice");
}

namespace {
int solve_checked(qpad_ctx* ctx, int op, int out, int in0, int in1, int nc_out, int nc0, int nc1) {
  if (!ctx) return QPAD_E_ARG;
  if (!valid_field(out) || !valid_field(in0) || (in1 >= 0 && !valid_field(in1)) || field_ncomp(out) != nc_out ||
      field_ncomp(in0) != nc0 || (in1 >= 0 && field_ncomp(in1) != nc1))
    return set_err(ctx, QPAD_E_ARG, "solve: field ids do not match the operation");
  FieldArgs a{ctx->f[out], ctx->f[in0], in1 >= 0 ? ctx->f[in1] : nullptr};
  return launch_field_op(ctx, op, a);
}
}  // namespace

extern "C" int qpad_solve_psi(qpad_ctx* ctx, int psi, int q) { return solve_checked(ctx, FOP_PSI, psi, q, -1, 1, 1, 0); }
extern "C" int qpad_solve_bz(qpad_ctx* ctx, int b, int cu) { return solve_checked(ctx, FOP_BZ, b, cu, -1, 3, 3, 0); }
extern "C" int qpad_solve_bt_beam(qpad_ctx* ctx, int b, int q) {
  return solve_checked(ctx, FOP_BT_BEAM, b, q, -1, 3, 1, 0);
}
extern "C" int qpad_solve_bt_iter(qpad_ctx* ctx, int b, int dcu, int cu) {
  return solve_checked(ctx, FOP_BT_ITER, b, dcu, cu, 3, 2, 3);
}
extern "C" int qpad_solve_ez(qpad_ctx* ctx, int e, int cu) { return solve_checked(ctx, FOP_EZ, e, cu, -1, 3, 3, 0); }
extern "C" int qpad_solve_et(qpad_ctx* ctx, int e, int b, int psi) {
  return solve_checked(ctx, FOP_ET, e, b, psi, 3, 3, 1);
}
extern "C" int qpad_solve_djdxi(qpad_ctx* ctx, int dcu, int acu, int amu) {
  return solve_checked(ctx, FOP_DJDXI, dcu, acu, amu, 2, 2, 3);
}

extern "C" int qpad_conv_test(qpad_ctx* ctx, int b, int dim, int op, double* rel_res, double* abs_res) {
  if (!ctx || !valid_field(b) || field_ncomp(b) != 3 || dim < 1 || dim > 3 || (op != 0 && op != 1))
    return ctx ? set_err(ctx, QPAD_E_ARG, "conv_test: bad args") : QPAD_E_ARG;
  if (int r = launch_conv(ctx, ctx->f[b], dim - 1, op)) return r;
  if (op == 1) {
    if (int r = d2h(ctx, ctx->h_res, ctx->conv + 2 * ctx->g.nr, 3)) return r;
    if (int r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "conv sync")) return r;
    if (rel_res) *rel_res = ctx->h_res[0];
    if (abs_res) *abs_res = ctx->h_res[1];
  }
  return QPAD_OK;
}

// =====================================================================================
// species
// =====================================================================================
extern "C" int qpad_species_create(qpad_ctx* ctx, const qpad_species_desc* d, const double* x, const double* p,
                                   const double* gamma, const double* psi, const double* q, int64_t np,
                                   qpad_species** out) {
  if (!ctx || !d || !out) return QPAD_E_ARG;
  *out = nullptr;
  if (d->npmax < 1 || d->npmax > (int64_t)1 << 30 || np > d->npmax || np < 0 ||
      (d->push_type != QPAD_PUSH2_STD && d->push_type != QPAD_PUSH2_ROBUST && !is_pgc(d->push_type)) ||
      d->qbm == 0.0)
    return set_err(ctx, QPAD_E_ARG, "invalid species descriptor");
  if (is_pgc(d->push_type)) {
    if (ctx->precision != QPAD_PREC_FP64) return set_err(ctx, QPAD_E_ARG, "PGC species: built on the FP64 path only");
    if (int r = laser_state_ensure(ctx)) return r;   // (zero envelope until a laser is added)
  }
  qpad_species* sp = new (std::nothrow) qpad_species();
  if (!sp) return set_err(ctx, QPAD_E_NOMEM, "species");
  sp->ctx = ctx;
  sp->qbm = d->qbm; sp->push_type = d->push_type; sp->neutralized = d->neutralized; sp->sort_freq = d->sort_freq;
  sp->npmax = d->npmax;
  const int64_t cap = d->npmax;
  double* block = nullptr;
  int r = dmalloc(ctx, (void**)&block, sizeof(double) * 16 * (size_t)cap, "particles");
  if (!r) {
    double** arrs[8] = {sp->x, sp->y, sp->px, sp->py, sp->pz, sp->gamma, sp->psi, sp->q};
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 8; ++a) arrs[a][b] = block + ((size_t)b * 8 + a) * cap;
  }
  if (!r) r = dmalloc(ctx, (void**)&sp->pristine, sizeof(double) * 8 * (size_t)cap, "pristine");
  if (!r) r = dmalloc(ctx, (void**)&sp->key, sizeof(int32_t) * cap, "keys");
  if (!r) r = dmalloc(ctx, (void**)&sp->aux, sizeof(int32_t) * cap, "aux");
  const int64_t ntiles = (cap + 1023) / 1024;
  const int64_t nh = ntiles * ctx->g.nr;
  int64_t need = 2 * nh + scan_tmp_elems(nh);
  if (scan_tmp_elems(cap) > need) need = scan_tmp_elems(cap);
  sp->blk_cap = need + 64;
  if (!r) r = dmalloc(ctx, (void**)&sp->blk, sizeof(int32_t) * sp->blk_cap, "blocks");
  if (!r) r = dmalloc(ctx, (void**)&sp->d_count, sizeof(int64_t), "count");
  if (!r) r = dmalloc(ctx, (void**)&sp->d_total, sizeof(int64_t), "total");
  if (!r) r = cuda_check(ctx, cudaMallocHost((void**)&sp->h_count, sizeof(int64_t)), "pinned count");
  if (!r) r = dmalloc(ctx, (void**)&sp->qf, f1_elems(ctx, QPAD_F_Q_SPE) * sizeof(double), "species q");
  if (!r) r = dmalloc(ctx, (void**)&sp->qn, f1_elems(ctx, QPAD_F_Q_SPE) * sizeof(double), "species qn");
  if (!r && ctx->precision == QPAD_PREC_MIXED) r = mixed_alloc(sp);
  if (!r) {
    ctx->species.push_back(sp);
    r = species_load(sp, x, p, gamma, psi, q, np);
  }
  if (r) {
    qpad_species_destroy(sp);
    return r;
  }
  *out = sp;
  return QPAD_OK;
}

extern "C" int qpad_species_destroy(qpad_species* sp) {
  if (!sp) return QPAD_OK;
  qpad_ctx* ctx = sp->ctx;
  cudaStreamSynchronize(ctx->stream);
  if (sp->x[0]) cudaFree(sp->x[0] < sp->x[1] ? sp->x[0] : sp->x[1]);
  if (sp->key) cudaFree(sp->key);
  if (sp->aux) cudaFree(sp->aux);
  if (sp->blk) cudaFree(sp->blk);
  if (sp->d_count) cudaFree(sp->d_count);
  if (sp->d_total) cudaFree(sp->d_total);
  if (sp->h_count) cudaFreeHost(sp->h_count);
  if (sp->qf) cudaFree(sp->qf);
  if (sp->qn) cudaFree(sp->qn);
  if (sp->pristine) cudaFree(sp->pristine);
  mixed_free(sp);
  neutral_free(sp);
  for (size_t i = 0; i < ctx->species.size(); ++i)
    if (ctx->species[i] == sp) { ctx->species.erase(ctx->species.begin() + i); break; }
  delete sp;
  rebuild_total_background(ctx);
  return QPAD_OK;
}

extern "C" int qpad_species_renew(qpad_species* sp, const double* x, const double* p, const double* gamma,
                                  const double* psi, const double* q, int64_t np) {
  if (!sp) return QPAD_E_ARG;
  if (sp->neut) return set_err(sp->ctx, QPAD_E_ARG, "a neutral gas's electrons are born, not loaded");
  return species_load(sp, x, p, gamma, psi, q, np);
}

extern "C" int qpad_species_reset(qpad_species* sp) {
  if (!sp) return QPAD_E_ARG;
  qpad_ctx* ctx = sp->ctx;
  if (sp->neut) return neutral_step_begin(ctx);   // (every neutral gas of the context)
  sp->np = sp->np_pristine;
  if (is_mixed(sp)) {
    if (int r = mixed_restore_pristine(sp)) return r;
  } else {
    double* dst[8] = {sp->x[0], sp->y[0], sp->px[0], sp->py[0], sp->pz[0], sp->gamma[0], sp->psi[0], sp->q[0]};
    for (int a = 0; a < 8; ++a)
      if (sp->np > 0 && cudaMemcpyAsync(dst[a], sp->pristine + (size_t)a * sp->npmax, sizeof(double) * sp->np,
                                        cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
        return check_launch(ctx, "reset copy");
  }
  *sp->h_count = sp->np;
  if (int r = cuda_check(ctx, cudaMemcpyAsync(sp->d_count, sp->h_count, sizeof(int64_t), cudaMemcpyHostToDevice,
                                              ctx->stream), "reset count"))
    return r;
  return is_mixed(sp) ? mixed_index(sp) : 0;
}

extern "C" int qpad_species_count(qpad_species* sp, int64_t* np) {
  if (!sp) return QPAD_E_ARG;
  if (int r = species_sync_count(sp)) return r;
  if (np) *np = *sp->h_count;
  return QPAD_OK;
}

extern "C" int qpad_species_download(qpad_species* sp, double* x, double* p, double* gamma, double* psi, double* q,
                                     int64_t* np) {
  if (!sp) return QPAD_E_ARG;
  qpad_ctx* ctx = sp->ctx;
  if (int r = species_sync_count(sp)) return r;
  if (int r = sync_fp64_view(sp)) return r;
  const int64_t n = *sp->h_count;
  if (np) *np = n;
  double* staging = sp->x[1];
  if (x) if (int r = download_vec(ctx, staging, x, n, 2, sp->x[0], sp->y[0], nullptr)) return r;
  if (p) if (int r = download_vec(ctx, staging, p, n, 3, sp->px[0], sp->py[0], sp->pz[0])) return r;
  if (gamma) if (int r = d2h(ctx, gamma, sp->gamma[0], n)) return r;
  if (psi) if (int r = d2h(ctx, psi, sp->psi[0], n)) return r;
  if (q) if (int r = d2h(ctx, q, sp->q[0], n)) return r;
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "species download");
}

extern "C" int qpad_species_qdp(qpad_species* sp, int q) {
  if (!sp || !valid_field(q) || field_ncomp(q) != 1) return sp ? set_err(sp->ctx, QPAD_E_ARG, "qdp: bad field") : QPAD_E_ARG;
  qpad_ctx* ctx = sp->ctx;
  const size_t n1 = f1_elems(ctx, QPAD_F_Q_SPE);
  if (cudaMemsetAsync(ctx->qraw, 0, n1 * sizeof(double), ctx->stream) != cudaSuccess) return check_launch(ctx, "memset");
  if (int r = is_mixed(sp) ? mixed_qdeposit_raw(sp, ctx->qraw) : species_qdeposit_raw(sp, ctx->qraw)) return r;
  if (int r = launch_finish_q(ctx, ctx->qraw, sp->qf, 0, ctx->g.smooth)) return r;
  k_add2<<<elem_grid(n1), 256, 0, ctx->stream>>>(ctx->f[q], sp->qf, sp->neutralized ? sp->qn : nullptr, n1);
  return check_launch(ctx, "qdp add");
}

namespace {
int ensure_scratch(qpad_ctx* ctx) {
  if (ctx->scratch) return 0;
  const size_t n = (size_t)ctx->g.P * 8 * ctx->g.ld;
  return dmalloc(ctx, (void**)&ctx->scratch, n * sizeof(double), "scratch");
}
}  // namespace

extern "C" int qpad_species_cbq(qpad_species* sp, int q, int cu, int slice) {
  if (!sp) return QPAD_E_ARG;
  qpad_ctx* ctx = sp->ctx;
  if (!valid_field(q) || field_ncomp(q) != 1 || !has_store(q) || !valid_field(cu) || field_ncomp(cu) != 3)
    return set_err(ctx, QPAD_E_ARG, "cbq: q must be a one-component field with a 3D store, cu a three-component one");
  if (slice < 1 || slice > ctx->g.nz + 1) return set_err(ctx, QPAD_E_ARG, "cbq: slice out of range");
  const int32_t a = 3, b = 1;
  if (int r = qpad_field_add_dim(ctx, cu, q, &a, &b, 1)) return r;
  return qpad_field_copy_slice(ctx, q, slice, QPAD_COPY_1TO2);
}

extern "C" int qpad_species_amjdp(qpad_species* sp, int ef, int bf, int cu, int amu, int dcu, double dt) {
  if (!sp || !valid_field(ef) || !valid_field(bf) || !valid_field(cu) || !valid_field(amu) || !valid_field(dcu) ||
      field_ncomp(ef) != 3 || field_ncomp(bf) != 3 || field_ncomp(cu) != 3 || field_ncomp(amu) != 3 ||
      field_ncomp(dcu) != 2 || !(dt > 0))
    return sp ? set_err(sp->ctx, QPAD_E_ARG, "amjdp: bad args") : QPAD_E_ARG;
  qpad_ctx* ctx = sp->ctx;
  if (int r = ensure_scratch(ctx)) return r;
  const size_t n3 = f1_elems(ctx, QPAD_F_CU), n2 = f1_elems(ctx, QPAD_F_ACU);
  double* scu = ctx->scratch;
  double* samu = scu + n3;
  double* sacu = samu + n3;
  if (cudaMemsetAsync(scu, 0, (2 * n3 + n2) * sizeof(double), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "memset");
  if (is_mixed(sp)) {
    if (int r = launch_gtab(ctx, ctx->f[ef], ctx->f[bf])) return r;
    if (int r = mixed_amjdp_raw(sp, ctx->gtab, scu, samu, sacu, dt)) return r;
  } else {
    if (int r = species_amjdp_raw(sp, ctx->f[ef], ctx->f[bf], scu, samu, sacu, dt)) return r;
  }
  if (int r = launch_finish_amj(ctx, scu, samu, sacu)) return r;
  k_add<<<elem_grid(n3), 256, 0, ctx->stream>>>(ctx->f[cu], scu, ctx->f[cu], n3);
  k_add<<<elem_grid(n3), 256, 0, ctx->stream>>>(ctx->f[amu], samu, ctx->f[amu], n3);
  k_add<<<elem_grid(n2), 256, 0, ctx->stream>>>(ctx->f[dcu], sacu, ctx->f[dcu], n2);
  return check_launch(ctx, "amjdp add", 3);
}

// ---- current deposit without any device allocation ---------------------------------
// qpad_species_amjdp allocates its deposit scratch with cudaMalloc on its first call.
// Some callers cannot allow that: a host code whose device memory is handed out by its
// own pool and capped at start-up, a caller that runs under a tool or a stream-ordered
// allocator where a stray cudaMalloc fails or stalls the device, or a caller that wants
// every allocation of the run to happen before its first slice.  For them the deposit
// scratch below is a fixed device array in this library's module image: the CUDA driver
// reserves it when the module loads, on every GPU that loads the library, and it stays
// reserved until the process exits.  Its size is fixed at kNoAllocScratchDoubles doubles
// (1 MiB); a grid needing more is rejected with QPAD_E_CAPACITY.
namespace {
constexpr size_t kNoAllocScratchDoubles = (size_t)1 << 17;
constexpr int kNoAllocMaxDevices = 64;
__device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// In host code g_noalloc_scratch names a host-side shadow, not device memory: the device
// address comes from cudaGetSymbolAddress, taken once per device with that device current.
int noalloc_scratch(qpad_ctx* ctx, double** out) {
  const int dev = ctx->device;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return set_err(ctx, QPAD_E_ARG, "no-alloc amjdp: device ordinal");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    int cur = -1;
    if (int r = cuda_check(ctx, cudaGetDevice(&cur), "cudaGetDevice")) return r;
    if (cur != dev)
      if (int r = cuda_check(ctx, cudaSetDevice(dev), "cudaSetDevice")) return r;
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (cur != dev) cudaSetDevice(cur);
    if (int r = cuda_check(ctx, e, "cudaGetSymbolAddress")) return r;
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return QPAD_OK;
}
}  // namespace

extern "C" int qpad_species_amjdp_noalloc(qpad_species* sp, int ef, int bf, int cu, int amu, int dcu, double dt) {
  if (!sp || !valid_field(ef) || !valid_field(bf) || !valid_field(cu) || !valid_field(amu) || !valid_field(dcu) ||
      field_ncomp(ef) != 3 || field_ncomp(bf) != 3 || field_ncomp(cu) != 3 || field_ncomp(amu) != 3 ||
      field_ncomp(dcu) != 2 || !(dt > 0))
    return sp ? set_err(sp->ctx, QPAD_E_ARG, "amjdp_noalloc: bad args") : QPAD_E_ARG;
  qpad_ctx* ctx = sp->ctx;
  const size_t n3 = f1_elems(ctx, QPAD_F_CU), n2 = f1_elems(ctx, QPAD_F_ACU);
  if (2 * n3 + n2 > kNoAllocScratchDoubles)
    return set_err(ctx, QPAD_E_CAPACITY,
                   "amjdp_noalloc: grid needs " + std::to_string(2 * n3 + n2) + " scratch doubles, limit is " +
                       std::to_string(kNoAllocScratchDoubles) + " (8 * (2*max_mode+1) * (nr+2) must fit)");
  double* scu = nullptr;
  if (int r = noalloc_scratch(ctx, &scu)) return r;
  double* samu = scu + n3;
  double* sacu = samu + n3;
  // the array keeps whatever the previous call left in it
  if (cudaMemsetAsync(scu, 0, (2 * n3 + n2) * sizeof(double), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "memset");
  if (is_mixed(sp)) {
    if (int r = launch_gtab(ctx, ctx->f[ef], ctx->f[bf])) return r;
    if (int r = mixed_amjdp_raw(sp, ctx->gtab, scu, samu, sacu, dt)) return r;
  } else {
    if (int r = species_amjdp_raw(sp, ctx->f[ef], ctx->f[bf], scu, samu, sacu, dt)) return r;
  }
  if (int r = launch_finish_amj(ctx, scu, samu, sacu)) return r;
  k_add<<<elem_grid(n3), 256, 0, ctx->stream>>>(ctx->f[cu], scu, ctx->f[cu], n3);
  k_add<<<elem_grid(n3), 256, 0, ctx->stream>>>(ctx->f[amu], samu, ctx->f[amu], n3);
  k_add<<<elem_grid(n2), 256, 0, ctx->stream>>>(ctx->f[dcu], sacu, ctx->f[dcu], n2);
  return check_launch(ctx, "amjdp_noalloc add", 3);
}

extern "C" int qpad_species_push_u(qpad_species* sp, int ef, int bf, double dt) {
  if (!sp || !valid_field(ef) || !valid_field(bf) || field_ncomp(ef) != 3 || field_ncomp(bf) != 3)
    return sp ? set_err(sp->ctx, QPAD_E_ARG, "push_u: bad args") : QPAD_E_ARG;
  if (is_mixed(sp)) {
    if (int r = launch_gtab(sp->ctx, sp->ctx->f[ef], sp->ctx->f[bf])) return r;
    return mixed_push(sp, sp->ctx->gtab, dt, 1, 0);
  }
  return species_push_u(sp, sp->ctx->f[ef], sp->ctx->f[bf], dt, 0);
}

extern "C" int qpad_species_push_x(qpad_species* sp, double dt) {
  if (!sp) return QPAD_E_ARG;
  if (is_mixed(sp)) return mixed_push(sp, sp->ctx->gtab, dt, 0, 1);
  return species_push_x(sp, dt);
}

extern "C" int qpad_species_interp_psi(qpad_species* sp, int psi) {
  if (!sp || !valid_field(psi) || field_ncomp(psi) != 1) return sp ? set_err(sp->ctx, QPAD_E_ARG, "interp_psi") : QPAD_E_ARG;
  if (is_mixed(sp)) return mixed_interp_psi(sp, sp->ctx->f[psi]);
  return species_interp_psi(sp, sp->ctx->f[psi]);
}

extern "C" int qpad_species_sort(qpad_species* sp) {
  if (!sp) return QPAD_E_ARG;
  // the mixed path keeps its particles sorted by cell (order inside a cell not kept)
  if (is_mixed(sp)) return mixed_sort_public(sp);
  return species_sort(sp);
}

// =====================================================================================
// beams
// =====================================================================================
extern "C" int qpad_beam_create(qpad_ctx* ctx, const qpad_beam_desc* d, const double* x, const double* p,
                                const double* q, int64_t nb, qpad_beam** out) {
  if (!ctx || !d || !out) return QPAD_E_ARG;
  *out = nullptr;
  if (d->npmax < 1 || d->npmax > (int64_t)1 << 31 || nb < 0 || nb > d->npmax ||
      (d->push_type != QPAD_PUSH3_REDUCED && d->push_type != QPAD_PUSH3_BORIS))
    return set_err(ctx, QPAD_E_ARG, "invalid beam descriptor");
  qpad_beam* bm = new (std::nothrow) qpad_beam();
  if (!bm) return set_err(ctx, QPAD_E_NOMEM, "beam");
  bm->ctx = ctx;
  bm->qbm = d->qbm; bm->push_type = d->push_type; bm->evolution = d->evolution; bm->npmax = d->npmax;
  const int64_t cap = d->npmax;
  double* block = nullptr;
  int r = dmalloc(ctx, (void**)&block, sizeof(double) * 14 * (size_t)cap, "beam particles");
  if (!r) {
    double** arrs[7] = {bm->x, bm->y, bm->z, bm->px, bm->py, bm->pz, bm->q};
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 7; ++a) arrs[a][b] = block + ((size_t)b * 7 + a) * cap;
  }
  if (!r) r = dmalloc(ctx, (void**)&bm->key, sizeof(int32_t) * cap, "beam keys");
  if (!r) r = dmalloc(ctx, (void**)&bm->aux, sizeof(int32_t) * cap, "beam aux");
  bm->blk_cap = scan_tmp_elems(cap) + 64;
  if (!r) r = dmalloc(ctx, (void**)&bm->blk, sizeof(int32_t) * bm->blk_cap, "beam blocks");
  if (!r) r = dmalloc(ctx, (void**)&bm->d_count, sizeof(int64_t), "beam count");
  if (!r) r = dmalloc(ctx, (void**)&bm->d_total, sizeof(int64_t), "beam total");
  if (!r) r = cuda_check(ctx, cudaMallocHost((void**)&bm->h_count, sizeof(int64_t)), "pinned");
  if (!r) {
    ctx->beams.push_back(bm);
    r = beam_load(bm, x, p, q, nb);
  }
  if (r) {
    qpad_beam_destroy(bm);
    return r;
  }
  *out = bm;
  return QPAD_OK;
}

extern "C" int qpad_beam_destroy(qpad_beam* bm) {
  if (!bm) return QPAD_OK;
  qpad_ctx* ctx = bm->ctx;
  cudaStreamSynchronize(ctx->stream);
  if (bm->x[0]) cudaFree(bm->x[0] < bm->x[1] ? bm->x[0] : bm->x[1]);
  if (bm->key) cudaFree(bm->key);
  if (bm->aux) cudaFree(bm->aux);
  if (bm->blk) cudaFree(bm->blk);
  if (bm->d_count) cudaFree(bm->d_count);
  if (bm->d_total) cudaFree(bm->d_total);
  if (bm->h_count) cudaFreeHost(bm->h_count);
  for (size_t i = 0; i < ctx->beams.size(); ++i)
    if (ctx->beams[i] == bm) { ctx->beams.erase(ctx->beams.begin() + i); break; }
  delete bm;
  return QPAD_OK;
}

extern "C" int qpad_beam_count(qpad_beam* bm, int64_t* nb) {
  if (!bm) return QPAD_E_ARG;
  if (int r = beam_sync_count(bm)) return r;
  if (nb) *nb = bm->nb;
  return QPAD_OK;
}

extern "C" int qpad_beam_download(qpad_beam* bm, double* x, double* p, double* q, int64_t* nb) {
  if (!bm) return QPAD_E_ARG;
  qpad_ctx* ctx = bm->ctx;
  if (int r = beam_sync_count(bm)) return r;
  const int64_t n = bm->nb;
  if (nb) *nb = n;
  double* staging = bm->x[1];
  if (x) if (int r = download_vec(ctx, staging, x, n, 3, bm->x[0], bm->y[0], bm->z[0])) return r;
  if (p) if (int r = download_vec(ctx, staging, p, n, 3, bm->px[0], bm->py[0], bm->pz[0])) return r;
  if (q) if (int r = d2h(ctx, q, bm->q[0], n)) return r;
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "beam download");
}

extern "C" int qpad_beam_qdp(qpad_beam* bm, int q) {
  if (!bm || !valid_field(q) || field_ncomp(q) != 1 || !has_store(q))
    return bm ? set_err(bm->ctx, QPAD_E_ARG, "beam qdp: field needs a 3D store") : QPAD_E_ARG;
  qpad_ctx* ctx = bm->ctx;
  // this%q = 0; deposit; corrections; q += this%q   (beam3d_class.f03:193-221)
  if (!ctx->beam_scratch) {
    if (int r = dmalloc(ctx, (void**)&ctx->beam_scratch, f2_elems(ctx, QPAD_F_Q_BEAM) * sizeof(double), "beam q"))
      return r;
  }
  const size_t n2 = f2_elems(ctx, QPAD_F_Q_BEAM);
  if (cudaMemsetAsync(ctx->beam_scratch, 0, n2 * sizeof(double), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "memset beam q");
  if (int r = beam_qdeposit(bm, ctx->beam_scratch)) return r;
  if (int r = beam_finish_q(ctx, ctx->beam_scratch)) return r;
  k_add<<<elem_grid(n2), 256, 0, ctx->stream>>>(ctx->f2[q], ctx->beam_scratch, ctx->f2[q], n2);
  return check_launch(ctx, "beam qdp add");
}

extern "C" int qpad_beam_push(qpad_beam* bm, int ef, int bf) {
  if (!bm || !valid_field(ef) || !valid_field(bf) || !has_store(ef) || !has_store(bf) || field_ncomp(ef) != 3 ||
      field_ncomp(bf) != 3)
    return bm ? set_err(bm->ctx, QPAD_E_ARG, "beam push: fields need 3D stores") : QPAD_E_ARG;
  return beam_push(bm, bm->ctx->f2[ef], bm->ctx->f2[bf]);
}

// =====================================================================================
// fused drivers
// =====================================================================================
namespace {

// ---- the three phases of one slice, shared by the host-driven and the graph drivers ----
// Prologue (simulation_class.f03:344-364): charge deposit, beam B-perp, psi, Bz, record.
int enqueue_slice_prologue(qpad_ctx* ctx, cudaGraphConditionalHandle hi, int use_h) {
  const size_t n1 = f1_elems(ctx, QPAD_F_Q_SPE);
  int any_ntd = 0;
  for (auto* s : ctx->species) any_ntd |= s->neutralized;
  const bool mixed = ctx->precision == QPAD_PREC_MIXED;
  if (int r = guess_enqueue(ctx)) return r;          // before anything reads b_spe or cu
  if (cudaMemsetAsync(ctx->d_iter, 0, (1 + kMaxUnroll) * sizeof(int), ctx->stream) != cudaSuccess ||
      cudaMemsetAsync(ctx->qraw, 0, n1 * sizeof(double), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "slice prologue memsets", 0);
  for (auto* s : ctx->species)
    if (int r = mixed ? mixed_qdeposit_raw(s, ctx->qraw) : species_qdeposit_raw(s, ctx->qraw)) return r;
  // the ions of any neutral gas join the background (neutral_class.f03:904-930)
  if (int r = neutral_slice_prologue(ctx)) return r;
  if (int r = launch_slice_begin(ctx, any_ntd || ctx->qbg != nullptr)) return r;
  // E of the first iteration (later iterations get theirs from k_iterate)
  if (int r = launch_iter_e(ctx)) return r;
  // the lasers' envelope and gradients of this slice (simulation_class.f03:362-367)
  if (int r = laser_slice_prologue(ctx)) return r;
  for (auto* s : ctx->species)
    if ((s->push_type == QPAD_PUSH2_STD || s->push_type == QPAD_PUSH2_STD_PGC) &&
        !s->neut)   // (the reference interpolates psi for species only)
      if (int r = mixed ? mixed_interp_psi(s, ctx->f[QPAD_F_PSI]) : species_interp_psi(s, ctx->f[QPAD_F_PSI]))
        return r;
  // the convergence record of B_phi: in the graph the last iteration of the previous slice
  // left it (nothing changes B_phi in between; the step start zeroes both), unless the
  // learned or extrapolated guess has just replaced b_spe
  if (use_h && !ctx->guess && !ctx->extrap) return 0;
  return launch_conv(ctx, ctx->f[QPAD_F_B_SPE], 1, 0, use_h, hi, use_h);
}

// One predictor-corrector iteration (simulation_class.f03:372-396).
// The deposit goes to the raw buffers; k_iterate finishes it, solves B-perp, Bz and the
// next iteration's E, and runs the convergence test.
int enqueue_iteration(qpad_ctx* ctx, cudaGraphConditionalHandle h, int use_h) {
  const bool mixed = ctx->precision == QPAD_PREC_MIXED;
  const size_t P1 = (size_t)ctx->g.P * ctx->g.ld;
  double* rcu = ctx->raw;
  double* ramu = ctx->raw + 3 * P1;
  double* racu = ctx->raw + 6 * P1;
  for (auto* s : ctx->species) {
    const int r = mixed ? mixed_amjdp_raw(s, ctx->gtab, rcu, ramu, racu, ctx->g.dxi)
                        : species_amjdp_raw(s, ctx->f[QPAD_F_E], ctx->f[QPAD_F_B], rcu, ramu, racu, ctx->g.dxi);
    if (r) return r;
  }
  if (int r = launch_smooth_raw(ctx)) return r;       // smoothing orders above the window's
  return launch_iterate(ctx, 1, h, use_h, 1);
}

// Epilogue (simulation_class.f03:403-456): stores, final fields, J-perp predictor, push.
int enqueue_slice_epilogue(qpad_ctx* ctx, int sort_now) {
  const bool mixed = ctx->precision == QPAD_PREC_MIXED;
  if (int r = laser_deposit_chi(ctx)) return r;       // (simulation_class.f03:400-401)
  if (int r = launch_slice_end(ctx)) return r;
  if (int r = neutral_slice_update(ctx)) return r;   // ionisation and new electrons before the push
  for (auto* s : ctx->species) {
    if (mixed) {
      if (int r = mixed_push(s, ctx->gtab, ctx->g.dxi, 1, 1)) return r;   // sorts by cell every slice
      continue;
    }
    if (int r = species_push_u(s, ctx->f[QPAD_F_E], ctx->f[QPAD_F_B], ctx->g.dxi, 1)) return r;
    if (sort_now && s->sort_freq > 0)
      if (int r = species_sort(s)) return r;
  }
  return 0;
}

// Graph of the whole slice loop: WHILE(j <= nz) { prologue; WHILE(not converged) { iteration }; epilogue; ++j }.
// The iteration condition is set by the convergence kernel, the slice condition by k_advance.
// Adds to `top` one simulation's slice loop: a kernel that sets its slice index to 1, then
// WHILE(j <= nz) { prologue; WHILE(not converged) { iteration }; epilogue; ++j }.  The
// iteration condition is set by the convergence test, the slice condition by k_advance.
// Branches added for different contexts are independent and run concurrently.
int add_slice_loop(qpad_ctx* ctx, cudaGraph_t top) {
  cudaGraphConditionalHandle hs = 0, hi = 0;
  cudaGraphNode_t nslice = nullptr, niter = nullptr;
  cudaGraph_t sbody = nullptr, ibody = nullptr;
  const bool prof = ctx->prof_on;
  ctx->prof_on = false;                          // event nodes are not allowed in conditional bodies
  const int64_t l0 = ctx->launches;
  int64_t l1 = l0, l2 = l0, l3 = l0;
  int r = cuda_check(ctx, cudaGraphConditionalHandleCreate(&hs, top, 1, cudaGraphCondAssignDefault), "slice handle");
  if (!r) r = cuda_check(ctx, cudaStreamBeginCaptureToGraph(ctx->stream, top, nullptr, nullptr, 0,
                                                            cudaStreamCaptureModeThreadLocal), "capture step");
  if (!r) {
    r = launch_set_slice(ctx, 1);
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (!r) r = cuda_check(ctx, cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, &cg, &deps, nullptr, &nd), "capture info");
    if (!r) {
      cudaGraphNodeParams p = {};
      p.type = cudaGraphNodeTypeConditional;
      p.conditional.handle = hs;
      p.conditional.type = cudaGraphCondTypeWhile;
      p.conditional.size = 1;
      r = cuda_check(ctx, cudaGraphAddNode(&nslice, cg, deps, nullptr, nd, &p), "slice while node");
      if (!r) sbody = p.conditional.phGraph_out[0];
      if (!r)
        r = cuda_check(ctx, cudaStreamUpdateCaptureDependencies(ctx->stream, &nslice, nullptr, 1,
                                                                cudaStreamSetCaptureDependencies), "capture deps");
    }
    cudaGraph_t out = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &out);
    if (!r) r = cuda_check(ctx, e, "end capture step");
  }
  const int64_t lset = ctx->launches;
  if (!r) r = cuda_check(ctx, cudaGraphConditionalHandleCreate(&hi, sbody, 1, cudaGraphCondAssignDefault), "iter handle");
  if (!r) r = cuda_check(ctx, cudaStreamBeginCaptureToGraph(ctx->stream, sbody, nullptr, nullptr, 0,
                                                            cudaStreamCaptureModeThreadLocal), "capture slice");
  l1 = l2 = l3 = lset;
  if (!r) {
    r = enqueue_slice_prologue(ctx, hi, 1);
    l1 = ctx->launches;
    if (!r) {
      cudaStreamCaptureStatus cs;
      cudaGraph_t cg = nullptr;
      const cudaGraphNode_t* deps = nullptr;
      size_t nd = 0;
      r = cuda_check(ctx, cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, &cg, &deps, nullptr, &nd), "capture info");
      if (!r) {
        cudaGraphNodeParams p = {};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = hi;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        r = cuda_check(ctx, cudaGraphAddNode(&niter, cg, deps, nullptr, nd, &p), "iteration while node");
        if (!r) ibody = p.conditional.phGraph_out[0];
        if (!r)
          r = cuda_check(ctx, cudaStreamUpdateCaptureDependencies(ctx->stream, &niter, nullptr, 1,
                                                                  cudaStreamSetCaptureDependencies), "capture deps");
      }
    }
    if (!r) r = enqueue_slice_epilogue(ctx, 1);
    if (!r) r = launch_advance(ctx, hs, hi);
    l2 = ctx->launches;
    cudaGraph_t out = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &out);
    if (!r) r = cuda_check(ctx, e, "end capture slice");
  }
  if (!r) r = cuda_check(ctx, cudaStreamBeginCaptureToGraph(ctx->stream, ibody, nullptr, nullptr, 0,
                                                            cudaStreamCaptureModeThreadLocal), "capture iteration");
  if (!r) {
    // the loop body holds `unroll` iterations: a WHILE-node round trip costs several times a
    // kernel-to-kernel dependency, and the parts after the first return at once when the
    // loop ended before them (iter_guard)
    const int64_t l2b = ctx->launches;
    const int U = std::max(1, std::min(kMaxUnroll, ctx->unroll));
    for (int u = 0; u < U && !r; ++u) {
      ctx->iter_part = U > 1 ? u : -1;
      r = enqueue_iteration(ctx, hi, 1);
    }
    ctx->iter_part = -1;
    l3 = l2 + (ctx->launches - l2b);
    cudaGraph_t out = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &out);
    if (!r) r = cuda_check(ctx, e, "end capture iteration");
  }
  // captured launches are not executions: keep the per-phase counts, undo the increments
  ctx->g_once = lset - l0;                        // the slice-index kernel, once per step
  ctx->g_pro = l1 - lset;
  ctx->g_epi = l2 - l1;
  ctx->g_it = l3 - l2;
  ctx->launches = l0;
  ctx->prof_on = prof;
  cudaGetLastError();
  return r;
}

int build_step_graph(qpad_ctx* ctx) {
  cudaGraph_t top = nullptr;
  int r = cuda_check(ctx, cudaGraphCreate(&top, 0), "graph create");
  if (!r) r = add_slice_loop(ctx, top);
  cudaGraphExec_t exec = nullptr;
  if (!r) r = cuda_check(ctx, cudaGraphInstantiate(&exec, top, 0), "graph instantiate");
  // a graph whose conditional body saw an invalidated capture is left alone (its
  // destruction is not safe); only the error path leaks it
  if (top && !r) cudaGraphDestroy(top);
  cudaGetLastError();
  if (r) return r;
  if (ctx->step_exec) cudaGraphExecDestroy(ctx->step_exec);
  ctx->step_exec = exec;
  return 0;
}

std::string step_key(const qpad_ctx* ctx) {
  std::string k = std::to_string(ctx->precision) + "/" + std::to_string(ctx->iter_cl) + "/" +
                  std::to_string(ctx->item_ppl) + "/" + std::to_string(ctx->guess != nullptr) + "/" +
                  std::to_string(ctx->extrap) + "/" + std::to_string(ctx->extrap_w) + "/" +
                  std::to_string(ctx->pdl) + "/" + std::to_string(ctx->g.smooth) + "/" +
                  std::to_string(ctx->lasers.size()) + "/" + std::to_string(ctx->unroll);
  for (auto* s : ctx->species)
    k += "|" + std::to_string((long long)s->np) + ":" + std::to_string(s->push_type) + ":" +
         std::to_string(s->neutralized) + ":" + std::to_string(s->sort_freq);
  return k;
}

int slice_step(qpad_ctx* ctx, int j, qpad_slice_stats* st) {
  const GridDev& g = ctx->g;
  // slice index lives on the device (the graph driver advances it there)
  *ctx->h_j = j;
  if (cudaMemcpyAsync(ctx->d_j, ctx->h_j, sizeof(int), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
    return check_launch(ctx, "slice index", 0);
  if (int r = enqueue_slice_prologue(ctx, 0, 0)) return r;
  int l;
  double rel = 0.0, ab = 0.0;
  for (l = 1; l <= ctx->iter_max; ++l) {
    if (int r = enqueue_iteration(ctx, 0, 0)) return r;
    if (int r = d2h(ctx, ctx->h_res, ctx->conv + 2 * g.nr, 3)) return r;
    if (int r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "iteration sync")) return r;
    if (ctx->prof_on) prof_collect(ctx);
    rel = ctx->h_res[0];
    ab = ctx->h_res[1];
    if (ctx->h_res[2] != 0.0) break;
  }
  if (st) {
    st->iters = l > ctx->iter_max ? ctx->iter_max : l;
    st->rel_res = rel;
    st->abs_res = ab;
  }
  int sort_now = 0;
  for (auto* s : ctx->species) sort_now |= (s->sort_freq > 0 && (j % s->sort_freq) == 0);
  return enqueue_slice_epilogue(ctx, sort_now);
}

}  // namespace

extern "C" int qpad_slice_step(qpad_ctx* ctx, int j, qpad_slice_stats* stats) {
  if (!ctx || j < 1 || j > ctx->g.nz) return ctx ? set_err(ctx, QPAD_E_ARG, "slice index out of range") : QPAD_E_ARG;
  return slice_step(ctx, j, stats);
}

namespace {
// 3D-step work before the slice loop (simulation_class.f03:309-341): beam charge deposit
// into the store, zeroed slice fields.
int step_begin(qpad_ctx* ctx) {
  if (int r = qpad_store_fill(ctx, QPAD_F_Q_BEAM, 0.0)) return r;
  if (int r = qpad_store_fill(ctx, QPAD_F_Q_SPE, 0.0)) return r;
  for (auto* b : ctx->beams)
    if (int r = beam_qdeposit(b, ctx->f2[QPAD_F_Q_BEAM])) return r;
  if (!ctx->beams.empty())
    if (int r = beam_finish_q(ctx, ctx->f2[QPAD_F_Q_BEAM])) return r;
  const int zero_fields[] = {QPAD_F_B, QPAD_F_E, QPAD_F_B_SPE, QPAD_F_E_SPE, QPAD_F_PSI,
                             QPAD_F_CU, QPAD_F_ACU, QPAD_F_AMU};
  for (int f : zero_fields)
    if (cudaMemsetAsync(ctx->f[f], 0, f1_elems(ctx, f) * sizeof(double), ctx->stream) != cudaSuccess)
      return check_launch(ctx, "zero fields");
  // the convergence record of the zeroed B_phi
  if (cudaMemsetAsync(ctx->conv, 0, 2 * (size_t)ctx->g.nr * sizeof(double), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "zero record");
  return neutral_step_begin(ctx);           // every neutral gas starts the step un-ionised
}

bool graph_ok(const qpad_ctx* ctx) {
  bool ok = ctx->use_graph;
  for (auto* s : ctx->species) ok &= (s->sort_freq == 0);
  return ok;
}

// After a graph-run slice loop has been enqueued: its statistics, counted launches.
int step_graph_stats(qpad_ctx* ctx, qpad_slice_stats* stats) {
  ctx->h_stats.resize(ctx->g.nz);
  if (int r = cuda_check(ctx, cudaMemcpyAsync(ctx->h_stats.data(), ctx->d_stats, sizeof(qpad_slice_stats) * ctx->g.nz,
                                              cudaMemcpyDeviceToHost, ctx->stream), "stats"))
    return r;
  if (int r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "graph step")) return r;
  // kernels the graph ran: per slice the prologue and epilogue, per execution of the
  // iteration loop's body (ceil(iterations / unroll) of them) the body's launches
  const int64_t U = std::max(1, std::min(kMaxUnroll, ctx->unroll));
  int64_t bodies = 0;
  for (const auto& s : ctx->h_stats) bodies += (s.iters + U - 1) / U;
  ctx->launches += ctx->g_once + (int64_t)ctx->g.nz * (ctx->g_pro + ctx->g_epi) + bodies * ctx->g_it;
  if (stats) std::copy(ctx->h_stats.begin(), ctx->h_stats.end(), stats);
  return 0;
}

// 3D-step work after the slice loop (simulation_class.f03:487-492): beam push, counts.
int step_end(qpad_ctx* ctx, int push_beams) {
  if (int r = lasers_advance(ctx)) return r;          // (simulation_class.f03:485-486)
  if (push_beams)
    for (auto* b : ctx->beams)
      if (int r = beam_push(b, ctx->f2[QPAD_F_E], ctx->f2[QPAD_F_B])) return r;
  prof_end(ctx, "step");
  for (auto* s : ctx->species)
    if (int r = species_sync_count(s)) return r;
  if (int r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "3d step")) return r;
  unsigned int werr = 0;
  if (int r = cuda_check(ctx, cudaMemcpy(&werr, ctx->iter_tickets + kIterErrWord, sizeof(werr), cudaMemcpyDeviceToHost),
                         "iteration error word"))
    return r;
  if (werr) {
    cudaMemsetAsync(ctx->iter_tickets + kIterErrWord, 0, sizeof(werr), ctx->stream);
    return set_err(ctx, QPAD_E_CUDA, "field iteration: a bulk-copy wait gave up (staging incomplete)");
  }
  if (ctx->d_neut_err) {
    unsigned int nerr = 0;
    if (int r = cuda_check(ctx, cudaMemcpy(&nerr, ctx->d_neut_err, sizeof(nerr), cudaMemcpyDeviceToHost),
                           "neutral error word"))
      return r;
    if (nerr) return set_err(ctx, QPAD_E_CAPACITY, "a neutral gas ionised more electrons than its npmax holds");
  }
  return QPAD_OK;
}
}  // namespace

extern "C" int qpad_3d_step(qpad_ctx* ctx, int push_beams, qpad_slice_stats* stats) {
  if (!ctx) return QPAD_E_ARG;
  prof_begin(ctx, "step");
  if (int r = step_begin(ctx)) return r;
  // the slice loop runs as one CUDA graph when the configuration allows it (sorting every
  // few slices is host-driven); otherwise the host drives it slice by slice
  bool use_graph = graph_ok(ctx);
  if (use_graph) {
    const std::string key = step_key(ctx);
    if (!ctx->step_exec || ctx->step_key != key) {
      int rb = build_step_graph(ctx);
      std::string why;
      if (rb && ctx->pdl) {                          // a graph with programmatic edges was refused:
        why = ctx->err;                              // build it with plain edges
        cudaGetLastError();
        ctx->pdl = false;
        rb = build_step_graph(ctx);
      }
      if (int r = rb) {
        ctx->graph_status = "graph build failed: " + ctx->err;
        ctx->use_graph = false;
        use_graph = false;
        cudaGetLastError();
      } else {
        ctx->step_key = step_key(ctx);
        ctx->graph_status = why.empty() ? "" : "programmatic edges refused, plain edges: " + why;
      }
    }
  }
  if (use_graph) {
    if (int r = cuda_check(ctx, cudaGraphLaunch(ctx->step_exec, ctx->stream), "graph launch")) return r;
    if (int r = step_graph_stats(ctx, stats)) return r;
  } else {
    for (int j = 1; j <= ctx->g.nz; ++j)
      if (int r = slice_step(ctx, j, stats ? stats + (j - 1) : nullptr)) return r;
  }
  return step_end(ctx, push_beams);
}

// =====================================================================================
// batches of independent simulations
// =====================================================================================
struct qpad_batch {
  std::vector<qpad_ctx*> ctxs;
  std::vector<std::string> keys;
  std::vector<cudaEvent_t> ev;      // per simulation: its pre-loop work is done
  cudaEvent_t done = nullptr;       // the batch graph is done
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool shaped = false;              // the iteration kernels' cluster shapes are set for the batch
  std::string err;
};

extern "C" int qpad_batch_create(qpad_ctx* const* ctxs, int n, qpad_batch** out) {
  if (!ctxs || n < 1 || !out) return QPAD_E_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (!ctxs[i] || ctxs[i]->device != ctxs[0]->device || has_neutrals(ctxs[i]) || !ctxs[i]->lasers.empty() ||
        ctxs[i]->la)
      return QPAD_E_ARG;   // (neutral gases and lasers run in single 3D steps only)
  qpad_batch* b = new (std::nothrow) qpad_batch();
  if (!b) return QPAD_E_NOMEM;
  b->ctxs.assign(ctxs, ctxs + n);
  b->keys.resize(n);
  b->ev.resize(n, nullptr);
  cudaError_t e = cudaSetDevice(ctxs[0]->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&b->ev[i], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    qpad_batch_destroy(b);
    return QPAD_E_CUDA;
  }
  *out = b;
  return QPAD_OK;
}

extern "C" int qpad_batch_destroy(qpad_batch* b) {
  if (!b) return QPAD_OK;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (cudaEvent_t e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->done) cudaEventDestroy(b->done);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return QPAD_OK;
}

extern "C" const char* qpad_batch_last_error(const qpad_batch* b) { return b ? b->err.c_str() : "null batch"; }

// One 3D step of every simulation of the batch; their slice loops (every slice, every
// predictor-corrector iteration of all of them) run as one CUDA graph launch, the
// simulations in independent branches.  stats[i] (nz entries) may be null.
extern "C" int qpad_batch_step(qpad_batch* b, int push_beams, qpad_slice_stats* const* stats) {
  if (!b) return QPAD_E_ARG;
  const int n = (int)b->ctxs.size();
  for (int i = 0; i < n; ++i)
    if (!graph_ok(b->ctxs[i])) {
      b->err = "simulation " + std::to_string(i) + " cannot run as a graph (sorting every few slices or graph off)";
      return QPAD_E_STATE;
    }
  // a batch is throughput-bound: every simulation's iteration kernel takes the smallest
  // cluster that fits its grid (the most rows per CTA, the fewest CTAs), which the
  // single-simulation autotuner, tuning for latency, does not choose
  // (qpad_batch_autotune times the other policies and keeps the fastest)
  if (!b->shaped) {
    for (auto* c : b->ctxs) {
      int r = QPAD_E_CUDA;
      for (int cl = 1; cl <= 16 && r; cl *= 2) r = iterate_try_cluster(c, cl);
      cudaGetLastError();
      if (r) {
        b->err = "no cluster shape of the iteration kernel fits: " + c->err;
        return r;
      }
    }
    b->shaped = true;
  }
  bool rebuild = !b->exec;
  for (int i = 0; i < n; ++i) rebuild |= (b->keys[i] != step_key(b->ctxs[i]));
  if (rebuild) {
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    const auto attempt = [&]() {
      cudaGraph_t top = nullptr;
      int r = cudaGraphCreate(&top, 0) == cudaSuccess ? 0 : QPAD_E_CUDA;
      for (int i = 0; i < n && !r; ++i) {
        r = add_slice_loop(b->ctxs[i], top);
        if (r) b->err = "simulation " + std::to_string(i) + ": " + b->ctxs[i]->err;
      }
      if (!r && cudaGraphInstantiate(&b->exec, top, 0) != cudaSuccess) {
        b->err = "batch graph instantiate failed";
        r = QPAD_E_CUDA;
      }
      if (top && !r) cudaGraphDestroy(top);      // left alone after a failed capture, as above
      cudaGetLastError();
      return r;
    };
    int r = attempt();
    bool any_pdl = false;
    for (auto* c : b->ctxs) any_pdl |= c->pdl;
    if (r && any_pdl) {                          // programmatic edges refused: plain edges
      for (auto* c : b->ctxs) c->pdl = false;
      b->exec = nullptr;
      r = attempt();
    }
    if (r) return r;
    for (int i = 0; i < n; ++i) b->keys[i] = step_key(b->ctxs[i]);
  }
  for (int i = 0; i < n; ++i) {
    qpad_ctx* c = b->ctxs[i];
    prof_begin(c, "step");
    if (int r = step_begin(c)) {
      b->err = "simulation " + std::to_string(i) + ": " + c->err;
      return r;
    }
    if (cudaEventRecord(b->ev[i], c->stream) != cudaSuccess || cudaStreamWaitEvent(b->stream, b->ev[i], 0) != cudaSuccess)
      return QPAD_E_CUDA;
  }
  if (cudaGraphLaunch(b->exec, b->stream) != cudaSuccess || cudaEventRecord(b->done, b->stream) != cudaSuccess) {
    b->err = "batch graph launch failed";
    return QPAD_E_CUDA;
  }
  for (int i = 0; i < n; ++i) {
    qpad_ctx* c = b->ctxs[i];
    if (cudaStreamWaitEvent(c->stream, b->done, 0) != cudaSuccess) return QPAD_E_CUDA;
    int r = step_graph_stats(c, stats ? stats[i] : nullptr);
    if (!r) r = step_end(c, push_beams);
    if (r) {
      b->err = "simulation " + std::to_string(i) + ": " + c->err;
      return r;
    }
  }
  return QPAD_OK;
}

// Launch shapes of a batch: policy 0 gives every simulation's iteration kernel the smallest
// cluster that fits its grid; policy c > 0 the single-simulation shape (up to 16 CTAs, 32
// rows each) capped at c CTAs.  `unroll` iterations per body of every iteration loop.
static int batch_shape(qpad_batch* b, int policy, int unroll) {
  for (auto* c : b->ctxs) {
    int r = QPAD_E_CUDA;
    if (policy == 0) {
      for (int cl = 1; cl <= 16 && r; cl *= 2) r = iterate_try_cluster(c, cl);
    } else {
      const int top = std::min(policy, std::max(1, std::min(16, c->g.nr / 32)));
      for (int cl = top; cl >= 1 && r; cl /= 2) r = iterate_try_cluster(c, cl);
    }
    cudaGetLastError();
    if (r) {
      b->err = "no cluster shape of the iteration kernel fits: " + c->err;
      return r;
    }
    c->unroll = unroll;
  }
  b->shaped = true;
  return 0;
}

// Times whole batch steps (beams not pushed, every species renewed from its uploaded state
// before each step, so the simulations end where they began) under the cluster policies
// {smallest fitting, capped at 4, 8, 16} with two iterations per loop body, then 1 and 4
// iterations per body with the fastest policy, and keeps the fastest.
extern "C" int qpad_batch_autotune(qpad_batch* b, int reps, qpad_batch_tune_result* out) {
  if (!b || reps < 1) return QPAD_E_ARG;
  const auto renew = [&]() -> int {
    for (auto* c : b->ctxs)
      for (auto* s : c->species)
        if (s->np_pristine > 0 || s->neut)
          if (int r = qpad_species_reset(s)) return r;
    return 0;
  };
  const auto timed = [&](int policy, int unroll, double* ms) -> int {
    *ms = 1e300;
    if (batch_shape(b, policy, unroll)) return 0;                  // a policy no shape of which fits: skipped
    if (int r = renew()) return r;
    if (int r = qpad_batch_step(b, 0, nullptr)) return r;            // graph build and warm-up
    double best = 1e300;
    for (int k = 0; k < reps; ++k) {
      if (int r = renew()) return r;
      for (auto* c : b->ctxs)
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) return QPAD_E_CUDA;
      const auto t0 = std::chrono::steady_clock::now();
      if (int r = qpad_batch_step(b, 0, nullptr)) return r;            // (synchronises every simulation)
      best = std::min(best, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    }
    *ms = best;
    return 0;
  };
  int best_p = 0, best_u = 2;
  double best_ms = 1e300;
  for (int policy : {0, 4, 8, 16}) {
    double ms = 0.0;
    if (int r = timed(policy, 2, &ms)) return r;
    if (ms < best_ms) { best_ms = ms; best_p = policy; }
  }
  for (int unroll : {1, 4}) {
    double ms = 0.0;
    if (int r = timed(best_p, unroll, &ms)) return r;
    if (ms < best_ms) { best_ms = ms; best_u = unroll; }
  }
  if (int r = batch_shape(b, best_p, best_u)) return r;
  if (out) {
    out->policy = best_p;
    out->unroll = best_u;
    out->step_ms = best_ms;
  }
  return renew();
}

// =====================================================================================
// autotuner
// =====================================================================================
extern "C" int qpad_set_launch_shapes(qpad_ctx* ctx, int iter_cluster, int item_ppl) {
  if (!ctx) return QPAD_E_ARG;
  if (iter_cluster != 0 && (iter_cluster < 1 || iter_cluster > 16 || (iter_cluster & (iter_cluster - 1)) != 0))
    return set_err(ctx, QPAD_E_ARG, "iteration cluster size must be 1, 2, 4, 8 or 16");
  if (item_ppl != 0 && item_ppl != 1 && item_ppl != 2 && item_ppl != 4)
    return set_err(ctx, QPAD_E_ARG, "particles per lane must be 1, 2 or 4");
  if (iter_cluster)
    if (int r = iterate_try_cluster(ctx, iter_cluster)) return r;
  if (item_ppl && item_ppl != ctx->item_ppl) {
    ctx->item_ppl = item_ppl;
    if (ctx->precision == QPAD_PREC_MIXED)
      for (auto* s : ctx->species)
        if (int r = mixed_index(s)) return r;
  }
  return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "launch shapes");
}

extern "C" int qpad_set_graph_unroll(qpad_ctx* ctx, int iterations) {
  if (!ctx) return QPAD_E_ARG;
  if (iterations < 1 || iterations > kMaxUnroll)
    return set_err(ctx, QPAD_E_ARG, "iterations per loop body must be 1 .. " + std::to_string(kMaxUnroll));
  ctx->unroll = iterations;
  return QPAD_OK;
}

extern "C" int qpad_autotune(qpad_ctx* ctx, int reps, qpad_tune_result* out) {
  if (!ctx || reps < 1) return QPAD_E_ARG;
  // the slice fields are scratch for the timing runs (a 3D step zeroes them anyway)
  const int zero_fields[] = {QPAD_F_B, QPAD_F_E, QPAD_F_B_SPE, QPAD_F_E_SPE, QPAD_F_PSI, QPAD_F_CU,
                             QPAD_F_ACU, QPAD_F_AMU, QPAD_F_DCU, QPAD_F_B_BEAM};
  for (int f : zero_fields)
    if (cudaMemsetAsync(ctx->f[f], 0, f1_elems(ctx, f) * sizeof(double), ctx->stream) != cudaSuccess)
      return check_launch(ctx, "autotune zero", 0);
  if (ctx->gtab && cudaMemsetAsync(ctx->gtab, 0, (size_t)ctx->g.ld * ctx->g.P * 6 * sizeof(float), ctx->stream) != cudaSuccess)
    return check_launch(ctx, "autotune zero", 0);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return QPAD_E_CUDA;
  auto timed = [&](auto&& body, double* us) -> int {
    for (int w = 0; w < 3; ++w)
      if (int r = body()) return r;
    cudaEventRecord(e0, ctx->stream);
    for (int k = 0; k < reps; ++k)
      if (int r = body()) return r;
    cudaEventRecord(e1, ctx->stream);
    if (int r = cuda_check(ctx, cudaEventSynchronize(e1), "autotune sync")) return r;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    *us = 1e3 * ms / reps;
    return 0;
  };
  qpad_tune_result res{};
  int r = 0;
  // cluster size of the iteration kernel
  const int64_t l0 = ctx->launches;
  double best = 1e30;
  int best_cl = ctx->iter_cl;
  for (int cl = 16; cl >= 1 && !r; cl /= 2) {
    if (iterate_try_cluster(ctx, cl)) continue;
    double us = 0.0;
    r = timed([&]() { return launch_iterate(ctx, 0, 0, 0); }, &us);
    if (!r && us < best) {
      best = us;
      best_cl = cl;
    }
  }
  if (!r) r = iterate_try_cluster(ctx, best_cl);
  res.iter_cluster = best_cl;
  res.iter_us = best;
  // work-item size of the mixed deposit
  res.item_ppl = ctx->item_ppl;
  res.deposit_us = 0.0;
  bool mixed = ctx->precision == QPAD_PREC_MIXED && !ctx->species.empty();
  if (!r && mixed) {
    const size_t P1 = (size_t)ctx->g.P * ctx->g.ld;
    double bestd = 1e30;
    int best_ppl = ctx->item_ppl;
    for (int ppl : {1, 2, 4}) {
      ctx->item_ppl = ppl;
      for (auto* s : ctx->species)
        if (!r) r = mixed_index(s);
      double us = 0.0;
      if (!r)
        r = timed([&]() {
          for (auto* s : ctx->species)
            if (int q = mixed_amjdp_raw(s, ctx->gtab, ctx->raw, ctx->raw + 3 * P1, ctx->raw + 6 * P1, ctx->g.dxi))
              return q;
          return 0;
        }, &us);
      if (!r && us < bestd) {
        bestd = us;
        best_ppl = ppl;
      }
    }
    ctx->item_ppl = best_ppl;
    for (auto* s : ctx->species)
      if (!r) r = mixed_index(s);
    res.item_ppl = best_ppl;
    res.deposit_us = bestd;
  }
  if (!r && cudaMemsetAsync(ctx->raw, 0, 8 * (size_t)ctx->g.P * ctx->g.ld * sizeof(double), ctx->stream) != cudaSuccess)
    r = check_launch(ctx, "autotune raw", 0);
  if (!r) r = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "autotune");
  ctx->launches = l0;                            // tuning launches are not part of the simulation
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (out) *out = res;
  return r;
}
