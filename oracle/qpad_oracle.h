/*
 * qpad_oracle.h -- CPU FP64 restatement of QPAD's per-xi-slice quasi-static loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle and the timed
 * CPU baseline.  Nothing in the product (qpad_gb300/, include/) links, loads or
 * calls it; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do.
 *
 * Parity status: UNPINNED against the reference itself.  The reference (Fortran
 * 2003 + MPI + HYPRE + json-fortran + HDF5) cannot be compiled here, and its own
 * test programs hold no assertions, stored outputs or golden vectors.  The oracle
 * is pinned instead by project-written known-answer tests (manufactured solutions
 * of every tridiagonal operator, hand-expanded single-particle pushes, charge
 * conservation) kept under tests/.
 *
 * Every routine restates one reference routine; the file:line it follows is given
 * beside it (paths relative to the QPAD source tree).  Arithmetic follows the
 * reference's operation order; build with -ffp-contract=off.  Single-rank semantics
 * throughout: noff = 0, one pipeline stage, guard cells never exchanged.  The HYPRE
 * cyclic-reduction solve (fields/field_solver_class.f03:172-177) is replaced by an
 * exact Thomas solve of the same matrix (both are direct solves).
 *
 * Layouts (host, row-major C):
 *   slice field ("f1")   f[((p*nc)+c)*(nr+2) + i]       p = mode part, c = component,
 *                                                       i = Fortran node index 0..nr+1
 *   3D store ("f2")      f[(((s-1)*P + p)*nc + c)*(nr+2) + i]   s = xi slice 1..nz+1
 *   mode parts           p = 0: m=0;  p = 2m-1: Re m;  p = 2m: Im m   (P = 2M+1)
 *   particles            structure of arrays (x, y, px, py, pz, q, gamma, psi)
 */
#ifndef QPAD_ORACLE_H
#define QPAD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BND_ZERO = 2, ORC_BND_OPEN = 3 };                  /* param.f03:72-74 */
enum { ORC_FK_PSI = 0, ORC_FK_EZ = 1, ORC_FK_BZ = 2, ORC_FK_BT = 3,
       ORC_FK_BPLUS = 4, ORC_FK_BMINUS = 5 };                   /* param.f03:76-84 */
enum { ORC_PUSH_STD = 0, ORC_PUSH_ROBUST = 1, ORC_PUSH_STD_PGC = 4, ORC_PUSH_ROBUST_PGC = 5 };  /* param.f03:63-64 */
enum { ORC_PUSH3_REDUCED = 1, ORC_PUSH3_BORIS = 2 };            /* param.f03:62 */

typedef struct orc_grid {
  int nr;            /* radial cells (nodes 1..nr, guards 0 and nr+1) */
  int nz;            /* xi slices */
  int max_mode;      /* M */
  int bnd;           /* ORC_BND_OPEN or ORC_BND_ZERO */
  double dr, dxi;
  double relax_fac;  /* B-perp predictor-corrector relaxation, sim_fields_class.f03:137-140 */
} orc_grid;

/* ---- tridiagonal operators (field_solver_class.f03:256-561) ------------------- */
/* a,b,c sized nr (row k at index k-1): lower, diagonal, upper, already / dr^2. */
void orc_build_matrix(const orc_grid* g, int kind, int mode, double* a, double* b, double* c);
/* Thomas solve in place (rhs -> solution), length n. */
void orc_thomas(int n, const double* a, const double* b, const double* c, double* rhs);

/* ---- field solves (slice fields, single rank) ---------------------------------- */
void orc_solve_psi(const orc_grid* g, const double* q, double* psi);          /* field_psi_class.f03:218-254 */
void orc_solve_bz(const orc_grid* g, const double* cu, double* b);            /* field_b_class.f03:760-796 */
void orc_solve_bt_beam(const orc_grid* g, const double* q, double* b);       /* field_b_class.f03:798-834 */
void orc_solve_bt_iter(const orc_grid* g, const double* dcu, const double* cu, double* b); /* :836-879 */
void orc_solve_ez(const orc_grid* g, const double* cu, double* e);           /* field_e_class.f03:298-334 */
void orc_solve_et(const orc_grid* g, const double* b, const double* psi, double* e); /* :412-514 */
void orc_solve_djdxi(const orc_grid* g, const double* acu, const double* amu, double* dcu); /* field_src_class.f03:273-405 */
/* convergence_tester, simulation_class.f03:522-606 (dim = 2, i.e. B_phi) */
void orc_conv_record(const orc_grid* g, const double* b, double* s_re, double* s_im);
void orc_conv_compare(const orc_grid* g, const double* b, double* s_re, double* s_im,
                      double* rel_res, double* abs_res);

/* ---- plasma particles (part2d_class.f03) --------------------------------------- */
void orc_qdeposit(const orc_grid* g, int64_t np, const double* x, const double* y,
                  const double* q, double* qf);                                  /* :231-359 */
void orc_amjdeposit(const orc_grid* g, int push_type, double qbm, double dt, int64_t np,
                    const double* x, const double* y, const double* px, const double* py,
                    const double* pz, const double* q, double* gamma, double* psi,
                    const double* ef, const double* bf, double* cu, double* amu,
                    double* dcu, int nthreads);                                  /* :478-1010 */
/* a laser envelope's slice fields as the PGC pushers gather them: a_r, a_i ([P][nr+2]) and
 * their gradients ([P][3][nr+2], r / phi / xi) */
typedef struct orc_laser_f1 { const double *ar, *ai, *gr, *gi; } orc_laser_f1;
void orc_amjdeposit_pgc(const orc_grid* g, int push_type, double qbm, double dt, int64_t np,
                        const double* x, const double* y, const double* px, const double* py,
                        const double* pz, const double* q, double* gamma, double* psi, const double* ef,
                        const double* bf, const orc_laser_f1* lf, double* cu, double* amu, double* dcu);
void orc_push_u_pgc(const orc_grid* g, double qbm, double dt, int64_t np, const double* x, const double* y,
                    double* px, double* py, double* pz, double* gamma, const double* psi, const double* ef,
                    const double* bf, const orc_laser_f1* lf);
void orc_deposit_chi(const orc_grid* g, double qbm, int ppc_r, int64_t np, const double* x, const double* y,
                     const double* q, const double* psi, double* chi);
/* ---- laser envelope (laser/field_laser_class.f03) and its PCR penta-diagonal solver -- */
void orc_pcr_coef(int n, const double* a, const double* b, const double* c, const double* d, const double* e,
                  double* cm1, double* cm2, double* cp1, double* cp2, double* cfin);
void orc_pcr_solve(int n, const double* cm1, const double* cm2, const double* cp1, const double* cp2,
                   const double* cfin, double* rhs);
void orc_laser_matrix(int nr, int m, double k0, double ds, double dr, double dz, double* a, double* b, double* c,
                      double* d, double* e);
void orc_laser_grad(const orc_grid* g, const double* lr, const double* li, int j, double* gr, double* gi);
void orc_push_u(const orc_grid* g, int push_type, double qbm, double dt, int64_t np,
                const double* x, const double* y, double* px, double* py, double* pz,
                double* gamma, const double* psi, const double* ef, const double* bf,
                int nthreads);                                                   /* :1790-1965 */
void orc_push_x(int64_t np, double dt, double* x, double* y, const double* px,
                const double* py, const double* pz, const double* gamma);        /* :2221-2262 */
/* update_bound (:2307-2353): swaps the last particle in; returns the new count */
int64_t orc_update_bound(const orc_grid* g, int64_t np, double* x, double* y, double* px,
                         double* py, double* pz, double* gamma, double* psi, double* q);
void orc_interp_psi(const orc_grid* g, int64_t np, const double* x, const double* y,
                    const double* psif, double* psi);                            /* :2264-2305 */
/* sort (:2498-2579 + sort_module.f03:10-41): keys (1-based cell) and the scatter
 * index written out; particle arrays permuted in place.                          */
void orc_sort(const orc_grid* g, int64_t np, double* x, double* y, double* px, double* py,
              double* pz, double* gamma, double* psi, double* q, int32_t* keys,
              int32_t* sort_idx);

/* ---- beam particles (part3d_class.f03) ----------------------------------------- */
void orc_beam_qdeposit(const orc_grid* g, int64_t nb, const double* x, const double* y,
                       const double* z, const double* q, double* q2);            /* :221-356 */
void orc_beam_push(const orc_grid* g, int push_type, double qbm, double dt, int64_t nb,
                   double* x, double* y, double* z, double* px, double* py, double* pz,
                   const double* e2, const double* b2, int nthreads);            /* :358-576, 691-790 */
int64_t orc_beam_update_bound(const orc_grid* g, int64_t nb, double* x, double* y, double* z,
                              double* px, double* py, double* pz, double* q);    /* :640-689 */

/* ---- loaders with the project's own RNG (see oracle.c) ------------------------- */
typedef struct orc_rng { uint64_t s; int have; double next; } orc_rng;
void orc_rng_seed(orc_rng* r, uint64_t seed);
double orc_rand_uniform(orc_rng* r);  /* (0,1) */
double orc_rand_norm(orc_rng* r);     /* math_module.f03:77-102 pairing */
/* fdist2d_class.f03:289-357, uniform profile; returns particle count */
int64_t orc_load_plasma(const orc_grid* g, orc_rng* r, int ppc1, int ppc2, int num_theta,
                        double qm, double density, const double uth[3], double* x, double* y,
                        double* px, double* py, double* pz, double* gamma, double* psi, double* q);
/* fdist3d_rnd_class.f03:360-514, Gaussian profile in cartesian geometry */
typedef struct orc_beam_desc {
  int64_t tot_num; double tot_charge, qm, gamma;
  double center[3], sigma[3], range_lo[3], range_hi[3];  /* xi coordinates already box-relative */
  double uth[3]; int quiet;
} orc_beam_desc;
int64_t orc_load_beam(const orc_grid* g, orc_rng* r, const orc_beam_desc* d, double* x, double* y,
                      double* z, double* px, double* py, double* pz, double* q);

/* ---- whole-loop driver: one 3D step, simulation_class.f03:294-512 --------------- */
typedef struct orc_sim orc_sim;
typedef struct orc_sim_desc {
  orc_grid g;
  int iter_max; double iter_reltol, iter_abstol;
  double dt3d;                 /* beam push time step */
  /* one plasma species */
  double sp_qbm; int sp_push_type; int sp_neutralized;
  int64_t sp_npmax;
  /* beams */
  int nbeams; double beam_qbm[4]; int beam_push_type[4]; int64_t beam_npmax[4];
  int nthreads;                /* OpenMP threads for particle loops (1 = serial) */
  int smooth_order;            /* binomial smoothing passes of the species deposits (0 = none) */
  int extrap;                  /* initial B-perp guess of a slice: 0 = carried (the reference),
                                  1 / 2 = linear / quadratic extrapolation from the stored slices
                                  (the product's optional guess, restated here to check it) */
  /* an ionising neutral gas (neutral_class.f03), none when neut_levels = 0 */
  int neut_levels;             /* ionisation levels followed (multi_max), at most 16 */
  double neut_adk[48];         /* per level: p1, p2, p3 of the rate p1 E^-p3 exp(-p2 / E), E in GV/m */
  double neut_wp;              /* plasma frequency (1/s) */
  double neut_density;         /* gas density / n0 (uniform) */
  int neut_ppc1, neut_ppc2, neut_num_theta;
  double neut_qm, neut_qbm;    /* charge and charge-to-mass ratio of the ionised electrons */
  int neut_push_type;
  int64_t neut_npmax;
  /* laser envelopes (field_laser_class.f03), none when nlasers = 0; the initial envelopes
     come from orc_sim_set_laser.  nr must be a power of two (the PCR solver's size 2 nr). */
  int nlasers;
  double laser_k0[4];          /* central wavenumber */
  int laser_iter[4];           /* implicit iterations per slice of the envelope advance */
  int sp_ppc_r;                /* the species' radial particles per cell (chi's axis factor) */
} orc_sim_desc;

/* One binomial (1,2,1) smoothing pass of a deposit field (ufield::smooth_f1,
 * ufield_class.f03:274-339, with the axis switches of field_rho / field_jay / field_djdxi
 * ::smooth, field_src_class.f03:102-125, 169-199, 243-271): kind 0 = rho (1 comp),
 * 1 = jay (3 comps: cu, amu), 2 = djdxi (2 comps: the acu deposit). */
void orc_smooth(const orc_grid* g, int kind, double* f);
orc_sim* orc_sim_create(const orc_sim_desc* d);
void orc_sim_destroy(orc_sim* s);
/* Load a fresh plasma slice state (species2d::new / renew, species2d_class.f03:75-184):
 * copies the particles and sets the neutralising background qn = -(their deposit). */
void orc_sim_set_plasma(orc_sim* s, int64_t np, const double* x, const double* y,
                        const double* px, const double* py, const double* pz,
                        const double* gamma, const double* psi, const double* q);
void orc_sim_set_beam(orc_sim* s, int k, int64_t nb, const double* x, const double* y,
                      const double* z, const double* px, const double* py, const double* pz,
                      const double* q);
/* Runs one 3D step; per-slice iteration counts and final rel_res go to iters/rel (nz).
 * The same step in phases: begin (beam deposit, field reset), slices j = 1..nz, end
 * (beam push). */
void orc_sim_run_3dstep(orc_sim* s, int push_beams, int* iters, double* rel);
void orc_sim_begin_3dstep(orc_sim* s);
void orc_sim_slice(orc_sim* s, int j, int* iters, double* rel);
void orc_sim_end_3dstep(orc_sim* s, int push_beams);
/* Accessors (pointers into the oracle's own arrays). */
double* orc_sim_field(orc_sim* s, const char* name, int* ncomp);   /* f1 */
double* orc_sim_store(orc_sim* s, const char* name, int* ncomp);   /* f2 */
int64_t orc_sim_plasma(orc_sim* s, double** x, double** y, double** px, double** py,
                       double** pz, double** gamma, double** psi, double** q);
/* the neutral's electrons, and its ionisation state [n_theta][nr][levels + 2] (levels 1..L,
 * then the neutral fraction, then the mean ionisation quantised to the particles per cell) */
int64_t orc_sim_neutral(orc_sim* s, double** x, double** y, double** px, double** py, double** pz,
                        double** gamma, double** psi, double** q);
double* orc_sim_multi_ion(orc_sim* s);
/* laser k's envelope initial values: ar, ai [nz][P][nr] (nodes 1..nr) */
void orc_sim_set_laser(orc_sim* s, int k, const double* ar, const double* ai);
/* laser k's envelope store, slices -1..nz+1: [(nz + 3)][P][nr + 2] */
void orc_sim_laser(orc_sim* s, int k, double** ar, double** ai);
int64_t orc_sim_beam(orc_sim* s, int k, double** x, double** y, double** z, double** px,
                     double** py, double** pz, double** q);

#ifdef __cplusplus
}
#endif
#endif
