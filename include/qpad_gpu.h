/*
 * qpad_gpu.h -- C ABI of the GB300 (sm_103a) implementation of QPAD's per-xi-slice
 * quasi-static loop.
 *
 * The reference plugs alternative algorithms in by Fortran type extension: a
 * `simulation_gpu extends simulation` project overrides the type-bound procedures
 * that run_simulation calls (source/simulation_class.f03:283-510).  Each entry point
 * below is what such an extension would bind through ISO_C_BINDING in place of one
 * reference procedure; the procedure it replaces is cited beside it.
 *
 * Conventions
 *  - Every function returns 0 on success or a positive QPAD_E_* code; nothing aborts
 *    or traps.  qpad_last_error() gives the message for the last failure on a context.
 *  - The library owns all device memory.  Host buffers stay owned by the caller and
 *    are only read or written during the call.
 *  - Host array layouts are the reference's Fortran layouts:
 *      particles   x(2,np) / x(3,nb) and p(3,np), component fastest; gamma, psi, q (np)
 *      slice field f1(dim, 0:nr+1) of one mode part, component fastest
 *    Mode parts are numbered p = 0 (m=0), 2m-1 (Re m), 2m (Im m): the reference's
 *    rf_re(0:M) / rf_im(1:M) (source/fields/field_class.f03:136-142).
 *  - One context = one simulation on one GPU and one CUDA stream; a context is used
 *    from one host thread at a time, like one reference MPI rank.
 */
#ifndef QPAD_GPU_H
#define QPAD_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------------- */
enum {
  QPAD_OK = 0,
  QPAD_E_ARG = 1,        /* invalid argument / size */
  QPAD_E_CUDA = 2,       /* CUDA runtime error (message has the CUDA error string) */
  QPAD_E_NOMEM = 3,      /* device or host allocation failed */
  QPAD_E_CAPACITY = 4,   /* particle buffer too small */
  QPAD_E_STATE = 5       /* call order / missing object */
};

/* ---- enums mirroring source/param.f03 ------------------------------------------- */
enum { QPAD_BND_ZERO = 2, QPAD_BND_OPEN = 3 };                     /* param.f03:72-74 */
enum { QPAD_PUSH2_STD = 0, QPAD_PUSH2_ROBUST = 1,                   /* param.f03:63-64 */
       QPAD_PUSH2_STD_PGC = 4, QPAD_PUSH2_ROBUST_PGC = 5 };          /* species that see the lasers */
enum { QPAD_PUSH3_REDUCED = 1, QPAD_PUSH3_BORIS = 2 };             /* param.f03:62 */
enum { QPAD_COPY_1TO2 = 1, QPAD_COPY_2TO1 = -1 };                  /* param.f03:125 */
enum { QPAD_PREC_FP64 = 0, QPAD_PREC_MIXED = 1 };

/* Field objects of sim_fields (source/sim_fields_class.f03:45-89). */
enum {
  QPAD_F_PSI = 0, QPAD_F_E, QPAD_F_E_SPE, QPAD_F_B, QPAD_F_B_SPE, QPAD_F_B_BEAM,
  QPAD_F_CU, QPAD_F_AMU, QPAD_F_ACU, QPAD_F_DCU, QPAD_F_Q_SPE, QPAD_F_Q_BEAM,
  QPAD_NFIELDS
};

/* ---- context ------------------------------------------------------------------- */
typedef struct qpad_ctx qpad_ctx;
typedef struct qpad_species qpad_species;
typedef struct qpad_laser qpad_laser;
typedef struct qpad_beam qpad_beam;

typedef struct qpad_grid_desc {
  int32_t nr, nz, max_mode;   /* simulation.grid(1:2), simulation.max_mode */
  int32_t bnd;                /* simulation.field_boundary */
  double dr, dxi;             /* options_class.f03:82-94 */
  double relax_fac;           /* < 0: default 1e-3*(dr/0.02)^2, sim_fields_class.f03:137-140 */
  int32_t iter_max;           /* simulation.iter_max */
  double iter_reltol, iter_abstol;
  double dt;                  /* simulation.dt (3D step, beam push) */
  int32_t precision;          /* QPAD_PREC_FP64 (reference arithmetic) or QPAD_PREC_MIXED */
  int32_t device;             /* CUDA device ordinal */
} qpad_grid_desc;

/* simulation::new + sim_fields::new (simulation_class.f03:105-199, sim_fields_class.f03:91-160) */
int qpad_ctx_create(const qpad_grid_desc* desc, qpad_ctx** out);
int qpad_ctx_destroy(qpad_ctx* ctx);
const char* qpad_last_error(const qpad_ctx* ctx);
int qpad_synchronize(qpad_ctx* ctx);
/* Components and radial line length (nr+2) of a slice field's device layout
 * [part][component][node]. */
int qpad_field_layout(const qpad_ctx* ctx, int field, int* ncomp, int64_t* ld);
/* Number of visible CUDA devices (no context needed; 0 when there is no GPU). */
int qpad_device_count(int* count);
/* Kernel launches issued on this context so far (all kernels of this library). */
int qpad_launch_count(const qpad_ctx* ctx, int64_t* count);
/* qpad_3d_step runs its slice loop as one CUDA graph (a WHILE node over slices holding a
 * WHILE node over predictor-corrector iterations, both conditions set on the device) when
 * on != 0 (the default); off, the host drives slices and iterations. */
int qpad_set_graph(qpad_ctx* ctx, int on);
/* Binomial (1,2,1) smoothing of the species' charge and current deposits, `order` passes
 * (0, the default, up to 64): the species' smooth_order (sim_plasma_class.f03:139-142),
 * applied as qdp_species2d / amjdp_species2d do (species2d_class.f03:202, 270-272) with
 * ufield::smooth_f1 (ufield_class.f03:274-339) `order` times (field_src_class.f03:114-121);
 * the neutralising background is not smoothed.  Orders above 64 are refused (QPAD_E_ARG). */
int qpad_set_smooth(qpad_ctx* ctx, int order);
/* 1 if the last 3D step ran as a graph. */
int qpad_graph_active(const qpad_ctx* ctx, int* active);
/* Why the graph path was switched off, or that it runs with plain instead of programmatic
 * edges ("" while it runs as designed). */
const char* qpad_graph_status(const qpad_ctx* ctx);
/* Per-kernel CUDA-event timing on the context's stream: enable/disable, then read the
 * accumulated device time (ms) and launch count of one kernel family by name
 * ("amjdp", "qdeposit", "push", "field", "beam_push", "beam_qdeposit"). */
int qpad_profile_enable(qpad_ctx* ctx, int on);
int qpad_profile_read(qpad_ctx* ctx, const char* name, double* total_ms, int64_t* launches);

/* ---- fields (source/fields/) ------------------------------------------------------ */
/* ufield f1 host mirror <-> device, one mode part; f1 is (dim, 0:nr+1) */
int qpad_field_upload(qpad_ctx* ctx, int field, int part, const double* f1);
int qpad_field_download(qpad_ctx* ctx, int field, int part, double* f1);
/* 3D store f2(dim, 0:nr+1, slice) of one slice and part (slice 1..nz+1) */
int qpad_store_download(qpad_ctx* ctx, int field, int slice, int part, double* f1);
int qpad_store_upload(qpad_ctx* ctx, int field, int slice, int part, const double* f1);
/* Slices slice_lo .. slice_lo+nslices-1 of a 3D store in one copy, in the device layout
 * host[s][part][component][node] (node 0..nr+1): what the reference's diagnostics read from
 * ufield%f2 (field_class.f03 write_hdf5, diagnostics_class.f03:822-944), without the
 * per-part transposition of qpad_store_download. */
int qpad_store_read(qpad_ctx* ctx, int field, int slice_lo, int nslices, double* host);
/* field = value (assign_f1, field_class.f03:917-950) and field%as (f2) */
int qpad_field_fill(qpad_ctx* ctx, int field, double value);
int qpad_store_fill(qpad_ctx* ctx, int field, double value);
/* c = a + b (add_f1_binary, field_class.f03:1031-1050) */
int qpad_field_add(qpad_ctx* ctx, int a, int b, int c);
/* b(bdim(k),:) += a(adim(k),:) (add_f1_unitary_dim, field_class.f03:1009-1029); dims 1-based */
int qpad_field_add_dim(qpad_ctx* ctx, int a, int b, const int32_t* adim, const int32_t* bdim, int n);
/* field *= s (dot_f1_unitary, field_class.f03:1159-1178) */
int qpad_field_scale(qpad_ctx* ctx, int field, double s);
/* ufield%copy_slice (ufield_class.f03:341-383): dir = QPAD_COPY_1TO2 / QPAD_COPY_2TO1 */
int qpad_field_copy_slice(qpad_ctx* ctx, int field, int slice, int dir);

/* field solves; the ids name the sim_fields objects taking part */
int qpad_solve_psi(qpad_ctx* ctx, int psi, int q);                  /* field_psi_class.f03:218-254 */
int qpad_solve_bz(qpad_ctx* ctx, int b, int cu);                    /* field_b_class.f03:760-796 */
int qpad_solve_bt_beam(qpad_ctx* ctx, int b, int q);                /* field_b_class.f03:798-834 */
int qpad_solve_bt_iter(qpad_ctx* ctx, int b, int dcu, int cu);      /* field_b_class.f03:836-879 */
int qpad_solve_ez(qpad_ctx* ctx, int e, int cu);                    /* field_e_class.f03:298-334 */
int qpad_solve_et(qpad_ctx* ctx, int e, int b, int psi);            /* field_e_class.f03:412-514 */
int qpad_solve_djdxi(qpad_ctx* ctx, int dcu, int acu, int amu);     /* field_src_class.f03:273-405 */
/* convergence_tester (simulation_class.f03:522-606) on component dim of field b:
 * op 0 = 'record', op 1 = 'compare' (writes rel_res, abs_res). */
int qpad_conv_test(qpad_ctx* ctx, int b, int dim, int op, double* rel_res, double* abs_res);

/* ---- plasma species (source/species/) -------------------------------------------- */
typedef struct qpad_species_desc {
  double qbm;            /* q/m */
  int32_t push_type;     /* QPAD_PUSH2_* (sim_plasma_class.f03:123-137) */
  int32_t neutralized;   /* species(k).neutralized */
  int64_t npmax;         /* particle capacity */
  int32_t sort_freq;     /* species(k).sort_freq: sort every n slices, 0 = never */
} qpad_species_desc;

/* species2d::new (species2d_class.f03:75-134): uploads the loaded particles and sets
 * the neutralising background qn = -(their charge deposit). */
int qpad_species_create(qpad_ctx* ctx, const qpad_species_desc* desc, const double* x,
                        const double* p, const double* gamma, const double* psi,
                        const double* q, int64_t np, qpad_species** out);
int qpad_species_destroy(qpad_species* sp);
/* species2d::renew (species2d_class.f03:154-184) with freshly loaded particles */
int qpad_species_renew(qpad_species* sp, const double* x, const double* p, const double* gamma,
                       const double* psi, const double* q, int64_t np);
int qpad_species_download(qpad_species* sp, double* x, double* p, double* gamma, double* psi,
                          double* q, int64_t* np);
/* renew from the device-resident copy of the last uploaded particles (no host traffic);
 * equivalent to qpad_species_renew with the same arrays. */
int qpad_species_reset(qpad_species* sp);
int qpad_species_count(qpad_species* sp, int64_t* np);
/* species2d::qdp (species2d_class.f03:186-208): q += deposit (+ qn if neutralized) */
int qpad_species_qdp(qpad_species* sp, int q);
/* species2d::cbq (species2d_class.f03:396-410): the species' charge density after the
 * slice's iteration, rho = (rho - Jz) + Jz, i.e. q(1) += cu(3) over every mode part and node,
 * then q's slice is stored at `slice` of its 3D store (copy_slice 1to2).  q and cu name the
 * fields holding this species' own (rho - Jz) and current. */
int qpad_species_cbq(qpad_species* sp, int q, int cu, int slice);
/* species2d::amjdp (species2d_class.f03:233-280): cu, amu, dcu += deposits */
int qpad_species_amjdp(qpad_species* sp, int ef, int bf, int cu, int amu, int dcu, double dt);
/* No counterpart in the reference.  Same arguments and result as qpad_species_amjdp, but
 * the call allocates no device memory (no cudaMalloc, cudaFree or allocating library
 * routine), for callers whose device memory is fixed by their own pool or that must not
 * allocate once the run has started.  Its deposit scratch is one static device array of
 * 1 MiB (131072 doubles) in the library image, held on every GPU that loads the library
 * until the process exits; grids with 8 * (2*max_mode+1) * (nr+2) > 131072 are rejected
 * with QPAD_E_CAPACITY.  The first call on a device looks up that array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.  All calls in
 * the process share the one array, so calls that overlap on the GPU (other streams, other
 * contexts on the same device) race; calls on one stream are ordered and safe. */
int qpad_species_amjdp_noalloc(qpad_species* sp, int ef, int bf, int cu, int amu, int dcu, double dt);
/* species2d::push_u (species2d_class.f03:282-309) */
int qpad_species_push_u(qpad_species* sp, int ef, int bf, double dt);
/* species2d::push_x (species2d_class.f03:311-327): push_x + update_bound */
int qpad_species_push_x(qpad_species* sp, double dt);
/* species2d::interp_psi (species2d_class.f03:437-452) */
int qpad_species_interp_psi(qpad_species* sp, int psi);
/* part2d::sort (part2d_class.f03:2498-2579): exact reference permutation */
int qpad_species_sort(qpad_species* sp);

/* ---- neutral gas (source/species/neutral_class.f03) ------------------------------ */
/* An ionising neutral gas: a species with no electrons at the start of every 3D step, whose
 * gas ionises level by level at the ADK rates of |E| at the cell centres and angles
 * 2 pi k / num_theta (ionize_neutral, neutral_class.f03:600-753), whose new electrons are
 * born at rest evenly across each cell (add_particles, :755-837) and then pushed like any
 * species, and whose ions stay put and join the charge source (ion_deposit_neutral,
 * :904-930).  The rate of level i is adk[i][0] E^-adk[i][2] exp(-adk[i][1] / E) per second
 * with E in GV/m (the reference's table of elements gives these numbers per element; the
 * caller passes them, e.g. from qpad_gb300.neutrals.adk_coefficients).  Uniform gas; the
 * FP64 path; no deposit smoothing.  The reference's mode sum for |E| reads the Re part of
 * each mode m >= 1 for both its Re and Im terms (neutral_class.f03:652-659); this does the
 * same, for identical results. */
typedef struct qpad_neutral_desc {
  double qm;             /* charge of the ionised particle (-1: electrons) */
  double qbm;            /* its charge-to-mass ratio */
  int32_t push_type;     /* QPAD_PUSH2_* */
  int32_t levels;        /* ionisation levels followed (the reference's max_e), 1..16 */
  const double* adk;     /* [levels][3]: p1, p2, p3 */
  double wp;             /* plasma frequency of n0 (1/s): E is converted with m_e c wp / e */
  double density;        /* gas density / n0 */
  int32_t ppc1, ppc2, num_theta;   /* particles per cell as the reference's ppc, num_theta */
  int64_t npmax;         /* capacity for the step's ionised electrons (exceeding it fails the step) */
} qpad_neutral_desc;
int qpad_neutral_create(qpad_ctx* ctx, const qpad_neutral_desc* desc, qpad_species** out);
/* ionisation state [num_theta][nr][levels + 2]: the fractions in levels 1..levels, the neutral
 * fraction, and the mean ionisation quantised to the particles per cell */
int qpad_neutral_state_download(qpad_species* sp, double* state);

/* ---- laser envelopes (source/laser/, sim_lasers_class.f03) ------------------------
 * A laser is the envelope a = a_r + i a_i of its vector potential, held per xi slice in the
 * azimuthal modes (field_laser_class.f03; the launch profiles of profile_laser_class.f03 are
 * evaluated by the caller, e.g. qpad_gb300.lasers.launch).  With lasers on the context, every
 * 3D step gathers per slice the sum of their envelopes and gradients for the species of push
 * type QPAD_PUSH2_*_PGC (amjdeposit_*_pgc, push_u_*_pgc, part2d_class.f03:1012-1602,
 * 1967-2219), deposits every species' susceptibility chi into a store after the slice's
 * iteration (deposit_chi :361-476; its axis factor needs the species' radial particles per
 * cell, qpad_species_set_radial_ppc), and after the slice loop advances each envelope by the
 * 3D time step (set_rhs + solve, field_laser_class.f03:393-927, with the penta-diagonal
 * cyclic reduction of fpcr_penta_class.f03).  FP64 path; nr a power of two; at most 7 modes.
 * Replaces sim_lasers%new/advance/deposit_chi (sim_lasers_class.f03:83-223). */
typedef struct qpad_laser_desc {
  double k0;             /* central wavenumber (laser(i).k0) */
  int32_t iter;          /* implicit iterations per slice of the advance (laser(i).iteration) */
} qpad_laser_desc;
/* ar, ai: the initial envelope [nz][P][nr] (nodes 1..nr; the on-axis values of m >= 1 are
 * taken as zero, as the advance leaves them) */
int qpad_laser_create(qpad_ctx* ctx, const qpad_laser_desc* desc, const double* ar, const double* ai,
                      qpad_laser** out);
/* the envelope [nz][P][nr + 2] (slices 1..nz) */
int qpad_laser_download(qpad_laser* laser, double* ar, double* ai);
/* the susceptibility store of the last 3D step [nz][P][nr + 2] */
int qpad_laser_chi_download(qpad_ctx* ctx, double* chi);
/* lasers%advance on its own (qpad_3d_step runs it after the slice loop) */
int qpad_lasers_advance(qpad_ctx* ctx);
/* the species' radial particles per cell (pf%ppc(1)): chi's on-axis factor
 * 12 ppc_r^2 / (1 + 2 ppc_r^2) (get_deposit_ax_corr, part2d_class.f03:2581-2586); default 2 */
int qpad_species_set_radial_ppc(qpad_species* sp, int32_t ppc_r);

/* ---- beams (source/beam/) -------------------------------------------------------- */
typedef struct qpad_beam_desc {
  double qbm;
  int32_t push_type;     /* QPAD_PUSH3_* (beam3d_class.f03:139-154) */
  int32_t evolution;     /* beam(k).evolution */
  int64_t npmax;
} qpad_beam_desc;

int qpad_beam_create(qpad_ctx* ctx, const qpad_beam_desc* desc, const double* x, const double* p,
                     const double* q, int64_t nb, qpad_beam** out);       /* beam3d_class.f03:121-177 */
int qpad_beam_destroy(qpad_beam* bm);
int qpad_beam_download(qpad_beam* bm, double* x, double* p, double* q, int64_t* nb);
int qpad_beam_count(qpad_beam* bm, int64_t* nb);
/* beam3d::qdp (beam3d_class.f03:193-221): q (3D store) += beam charge */
int qpad_beam_qdp(qpad_beam* bm, int q);
/* beam3d::push (beam3d_class.f03:223-254): push + update_bound with the e, b 3D stores */
int qpad_beam_push(qpad_beam* bm, int ef, int bf);

/* ---- fused drivers --------------------------------------------------------------- */
typedef struct qpad_slice_stats {
  int32_t iters;         /* predictor-corrector iterations taken */
  double rel_res, abs_res;
} qpad_slice_stats;

/* One xi slice j (1..nz) of run_simulation (simulation_class.f03:342-469) over all
 * species and the stored beam charge. */
int qpad_slice_step(qpad_ctx* ctx, int j, qpad_slice_stats* stats);
/* One whole 3D step (simulation_class.f03:294-512 without diagnostics): beam deposit,
 * slices 1..nz, beam push; per-slice stats into stats[nz] (may be NULL).  Returns
 * QPAD_E_CUDA with a message if the field iteration's bounded wait for its staged inputs
 * gave up during the step (the step's results are then not valid). */
int qpad_3d_step(qpad_ctx* ctx, int push_beams, qpad_slice_stats* stats);

/* ---- batches of independent simulations (no counterpart in the reference) -----------
 * A scan over drivers runs as many contexts on one GPU.  qpad_batch_step advances every
 * context of the batch by one 3D step (qpad_3d_step semantics for each); the slice loops
 * of all of them, every slice and predictor-corrector iteration, run as ONE CUDA graph
 * launch, each simulation an independent branch with its own device-side loop conditions.
 * The contexts must share a device and must not sort every few slices (sort_freq = 0).
 * The first step of a batch gives every context's iteration kernel the smallest cluster
 * that fits its grid (a batch is throughput-bound); qpad_autotune afterwards restores a
 * context's single-simulation shape. */
typedef struct qpad_batch qpad_batch;
int qpad_batch_create(qpad_ctx* const* ctxs, int n, qpad_batch** out);
int qpad_batch_destroy(qpad_batch* batch);
const char* qpad_batch_last_error(const qpad_batch* batch);
/* stats[i] receives context i's nz per-slice statistics (stats or stats[i] may be null) */
int qpad_batch_step(qpad_batch* batch, int push_beams, qpad_slice_stats* const* stats);
/* Autotuner of a batch's launch shapes (no counterpart in the reference): times `reps` whole
 * batch steps (beams not pushed; every species renewed from its uploaded particles before
 * each step and at the end) for each cluster policy of the iteration kernels (0: the smallest
 * cluster that fits each grid, the default of qpad_batch_step; c = 4, 8, 16: each
 * simulation's own shape capped at c CTAs) and iterations per loop body (1, 2, 4), and keeps
 * the fastest.  The 3D stores hold the last timed step's fields afterwards. */
typedef struct qpad_batch_tune_result {
  int32_t policy;             /* 0 or the cluster cap */
  int32_t unroll;             /* iterations per body of the iteration loops */
  double step_ms;             /* the fastest batch step (host clock, milliseconds) */
} qpad_batch_tune_result;
int qpad_batch_autotune(qpad_batch* batch, int reps, qpad_batch_tune_result* out);

/* ---- autotuner (no counterpart in the reference) ---------------------------------------
 * Times the launch shapes this context can use on this GPU and keeps the fastest: the
 * cluster size of the fused predictor-corrector kernel (16, 8, 4, 2, 1 CTAs per mode) and,
 * on the mixed path, the particles per lane of the deposit work items (1, 2 or 4).  Runs
 * `reps` timed launches of each; overwrites the slice fields (call it before a 3D step). */
typedef struct qpad_tune_result {
  int32_t iter_cluster;       /* CTAs per mode of the iteration kernel */
  double iter_us;             /* its time per launch */
  int32_t item_ppl;           /* particles per lane of a mixed deposit work item */
  double deposit_us;          /* the mixed deposit's time per launch (0 on the FP64 path) */
} qpad_tune_result;
int qpad_autotune(qpad_ctx* ctx, int reps, qpad_tune_result* out);
/* Sets the launch shapes by hand (0 keeps one): the iteration kernel's CTAs per mode (1, 2, 4,
 * 8, 16) and the mixed deposit's particles per lane (1, 2, 4). */
int qpad_set_launch_shapes(qpad_ctx* ctx, int iter_cluster, int item_ppl);
/* Predictor-corrector iterations per body of the step graph's iteration loop (1 .. 4,
 * default 2; no counterpart in the reference, whose loop is `do while` on the host,
 * simulation_class.f03:370-398).  Each WHILE-node round trip of the graph costs several
 * microseconds; the iterations after the first in a body return at once when the loop has
 * ended before them, so results and iteration counts do not depend on this setting. */
int qpad_set_graph_unroll(qpad_ctx* ctx, int iterations);

/* ---- loaders (host; project RNG substituting gfortran random_number) ------------- */
typedef struct qpad_rng { uint64_t s; int32_t have; double next; } qpad_rng;
void qpad_rng_seed(qpad_rng* r, uint64_t seed);
/* fdist2d::inject (fdist2d_class.f03:289-357), uniform profile; returns the count or -1 */
int64_t qpad_load_plasma(int nr, double dr, qpad_rng* r, int ppc1, int ppc2, int num_theta,
                         double qm, double density, const double uth[3], double* x, double* p,
                         double* gamma, double* psi, double* q, int64_t cap);
typedef struct qpad_beam_load_desc {
  int64_t tot_num; double tot_charge, qm, gamma;
  double center[3], sigma[3], range_lo[3], range_hi[3];
  double uth[3]; int32_t quiet;
} qpad_beam_load_desc;
/* fdist3d_rnd::inject (fdist3d_rnd_class.f03:360-514), Gaussian profiles */
int64_t qpad_load_beam(int nr, int nz, double dr, double dxi, qpad_rng* r,
                       const qpad_beam_load_desc* d, double* x, double* p, double* q, int64_t cap);

/* ---- diagnostic and restart files in the reference's HDF5 layout ----------------------
 * Written and read by this library's own implementation of the HDF5 file format (the
 * subset libhdf5 produces with default settings; no HDF5 library is needed).  Errors of the
 * file-level calls are in qpad_h5_last_error(). */
typedef struct qpad_h5_grid_info {
  double time;                  /* root attribute TIME (tstep * dt) */
  int32_t iter;                 /* ITER and the file's 8-digit step number */
  double dt;                    /* DT */
  const char* timeunit;         /* TIME UNIT */
  const char* units;            /* dataset UNITS */
  const char* label;            /* dataset LONG_NAME */
  double axis_min[2], axis_max[2];                  /* AXIS/AXIS1 (r), AXIS/AXIS2 (xi) */
  const char* axis_name[2];
  const char* axis_label[2];
  const char* axis_units[2];
  const char* type;             /* root attribute TYPE: null or "grid" (with the AXIS group), else e.g.
                                   "restart" (no AXIS group, as wrattr_file, hdf5io_class.f03:264-300) */
} qpad_h5_grid_info;
const char* qpad_h5_last_error(void);
/* One grid file as pwfield_2d writes it (hdf5io_class.f03:398-452, attributes :264-335): root
 * attributes NAME, TYPE "grid", TIME, ITER, DT, TIME UNIT; group AXIS with AXIS1, AXIS2; the
 * dataset `dataname` of shape [nz][nr] (data row-major, radial node fastest). */
int qpad_h5_write_grid(const char* path, const char* dataname, const double* data, int nz, int nr,
                       const qpad_h5_grid_info* info);
/* One particle file as wpart writes it (hdf5io_class.f03:1584-1710): root attributes as above
 * with TYPE "restart" and tp = n; datasets x [n][3], p [n][3], q [n] (none when n = 0). */
int qpad_h5_write_particles(const char* path, const char* dataname, const double* x, const double* p,
                            const double* q, int64_t n, int iter, double time, double dt);
/* A float or integer dataset (path "name" or "group/name") as doubles; count, rank and dims
 * (up to 8) are returned; out may be null to query them. */
int qpad_h5_read_dataset(const char* path, const char* name, double* out, int64_t cap, int64_t* count,
                         int32_t* rank, int64_t* dims);
/* An attribute of the root ("" object) or of a member: numbers into *value, strings into text. */
int qpad_h5_read_attr(const char* path, const char* object, const char* attr, double* value, char* text,
                      int64_t text_cap);
/* The field diagnostic of one component of a field's 3D store, every mode part
 * (sim_diag::run, diagnostics_class.f03:822-944, files per part from add_diag_cym :947-1045):
 * dir/Re0/, dir/Re1/, dir/Im1/, ... each <dataname>_<iter, 8 digits>.h5, dataset [nz][nr]
 * over nodes 1..nr and slices 1..nz. */
int qpad_diag_write_field(qpad_ctx* ctx, int field, int comp, const char* dir, const char* dataname,
                          const char* units, const char* label, int iter, double time, double dt);
/* beam3d::wrst (part3d_class.f03:827-845): the beam's particles into the restart file `path`
 * (the reference names it ./RST/Beam<ii>/RST-beam<ii>-<rank, 6 digits>_<step, 8 digits>.h5). */
int qpad_beam_write_rst(qpad_beam* bm, const char* path, const char* dataname, int iter, double time, double dt);
/* beam3d::rrst (part3d_class.f03:847-865): a restart file's particles into host arrays
 * x[n][3], p[n][3], q[n]; with all three null only *n is returned. */
int qpad_rst_read(const char* path, double* x, double* p, double* q, int64_t cap, int64_t* n);

/* ---- learned predictor-corrector guess (no counterpart in the reference) ------------
 * A radial 1D conv net (layers x conv1d(ksize), width channels, GELU between layers),
 * trained and evaluated by this library's own BF16 tensor-core kernels with FP32
 * accumulation.  Host arrays are sample-major [sample][channel][nr]. */
typedef struct qpad_learn qpad_learn;
int qpad_learn_create(int cin, int cout, int width, int layers, int ksize, uint64_t seed, int device,
                      qpad_learn** out);
int qpad_learn_destroy(qpad_learn* net);
const char* qpad_learn_last_error(const qpad_learn* net);
int qpad_learn_param_count(const qpad_learn* net, int64_t* n);
int qpad_learn_get_params(qpad_learn* net, float* params);
int qpad_learn_set_params(qpad_learn* net, const float* params);
int qpad_learn_predict(qpad_learn* net, const float* x, int64_t ns, int nr, float* y);
/* mean squared error of y(x) against t and its gradient w.r.t. every parameter */
int qpad_learn_grad(qpad_learn* net, const float* x, const float* t, int64_t ns, int nr, double* loss,
                    float* grad);
/* Adam, `epochs` shuffled passes in mini-batches; losses[epoch] = mean training loss */
int qpad_learn_train(qpad_learn* net, const float* x, const float* t, int64_t ns, int nr, int epochs,
                     int batch, float lr, uint64_t seed, double* losses);
/* Replaces the carried initial b_spe (simulation_class.f03:324-326, 360) and the J-perp
 * predictor (:425-426) of every slice j >= 3 by the nets' guess from slices j-1, j-2:
 * net0 (10 -> 4 channels) for m = 0, net1 (20 -> 8) for the modes m >= 1.  The iteration
 * still runs to iter_reltol.  Null net0 detaches.  The nets must outlive the attachment.
 * Nets of width 64, 4 layers, kernel 5 run as one fused kernel per slice from BF16 copies of
 * their weights taken here: attach again after changing the weights. */
int qpad_guess_attach(qpad_ctx* ctx, qpad_learn* net0, qpad_learn* net1);
/* Initial B-perp guess of every slice from the stored B-perp of the previous slices, without
 * a net (no counterpart in the reference, which carries B-perp(j-1), simulation_class.f03:
 * 324-326, 360): order 0 keeps the carried value (the default), 1 extrapolates linearly from
 * slices j-1, j-2, 2 quadratically from j-1..j-3; weight w in [0, 2] applies that fraction of
 * the extrapolation's change to the carried value (1: the full extrapolation).  The iteration
 * still runs to iter_reltol.  Attached nets take precedence. */
int qpad_set_guess_extrapolation(qpad_ctx* ctx, int order, double weight);
/* Which parts of the guess are applied (bit 0: B-perp, bit 1: the J-perp predictor; both by
 * default) and the weight w in [0, 1] of the net's correction: guess = carried + w (net - carried). */
int qpad_guess_config(qpad_ctx* ctx, int apply, double weight);
/* Runs the configured initial guess of slice j (3 <= j <= nz) from the 3D stores of the
 * step before, as the slice loop does at the start of slice j, and leaves it in the b_spe and
 * cu slice fields (no counterpart in the reference; for tests and diagnostics). */
int qpad_guess_apply(qpad_ctx* ctx, int j);
/* One training sample of mode m at slice j (3 <= j <= nz) from the 3D stores of the last
 * step: inputs x [10 or 20][nr], targets t [4 or 8][nr], both in units of *scale. */
int qpad_guess_sample(qpad_ctx* ctx, int j, int m, float* x, float* t, float* scale);
/* The same for slices j_lo .. j_hi in one call: x [n][10 or 20][nr], t [n][4 or 8][nr], scale [n]. */
int qpad_guess_samples(qpad_ctx* ctx, int j_lo, int j_hi, int m, float* x, float* t, float* scale);

#ifdef __cplusplus
}
#endif
#endif
