/*
 * CPU oracle for the Phantom per-step SPH hot path (test infrastructure).
 *
 * This is a serial C++ restatement of the reference Fortran routines that the
 * GPU path replaces. It exists only to check the CUDA path and to time a CPU
 * baseline; nothing in the product library links or calls it.
 *
 * Parity pins: the golden known-answer values restated from the reference's
 * own test suite (src/tests/test_derivs.f90:179-262 lattice counts and gradh,
 * test_kernel.f90 kernel identities, test_neigh.f90 brute-force neighbour
 * counts, test_gravity.f90 direct-sum agreement) are checked against this
 * oracle in tests/test_oracle_golden.py. The reference itself cannot be
 * compiled here (no Fortran compiler), so parity is pinned by those tests.
 */
#ifndef PHANTOM_ORACLE_H
#define PHANTOM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Run-time and compile-time switches of the reference (config.F90 `module dim`,
 * options.f90, shock_capturing.f90, timestep.f90, eos.f90 defaults). */
typedef struct ora_params {
  int32_t periodic;        /* PERIODIC */
  int32_t mhd;             /* MHD (ideal, fast_divcurlB) */
  int32_t gravity;         /* GRAVITY (self-gravity, dual-tree walk) */
  int32_t isothermal;      /* ISOTHERMAL (maxvxyzu = 3) */
  int32_t ieos;            /* 1 = isothermal, 2 = adiabatic */
  int32_t ipdv_heating;    /* eos.f90:1897 default 1 */
  int32_t ishock_heating;  /* eos.f90:1896 default 1 */
  int32_t iresistive_heating; /* eos.f90:1898 default 1 */
  int32_t divB_hj_prepass; /* 1: divcurlB uses the h_j held at entry of the
                              density pass (race-free form of the reference's
                              fast_divcurlB read of xyzh(4,j)); 0: serial order */
  int32_t nthreads;        /* OpenMP threads for the cell loops (1 = serial) */
  int32_t f64_store;       /* 1: the force reads gradh (1/Omega, gradsoft) kept in FP64
                              instead of the reference's float32 storage (a smooth
                              function of the positions, for finite-difference checks
                              of gradients); 0: the reference's float32 storage */
  int32_t minpart;         /* leaf size (config.F90:113 minpart); 0 = the reference's 10 */
  double xmin, xmax, ymin, ymax, zmin, zmax; /* boundary.f90 */
  double hfact, tolh, massoftype;
  double alpha, alphau, alphaB, beta;
  double gamma, polyk;
  double C_cour, C_force, tolv, dtmax;
  double psidecayfac, overcleanfac;
  double tree_accuracy;
  int64_t maxp;            /* allocation size: fixes ncellsmax = 2*maxp */
  double alphamax;         /* shock_capturing.f90:35 (Cullen-Dehnen upper bound) */
  int32_t nalpha;          /* config.F90:158-162: 0 = CONST_AV, 3 = Cullen-Dehnen switch */
  int32_t ind_timesteps;   /* IND_TIMESTEPS: individual particle timesteps (power-of-two bins) */
  int32_t curlv;           /* CURLV (config.F90:166,384): divcurlv holds ndivcurlv = 4 rows,
                              div v and curl v; 0: the one row div v */
} ora_params;

typedef struct ora_stats {
  int64_t nneightry;     /* dens.F90:1672 */
  int64_t nneighact;     /* dens.F90:1673 */
  int64_t maxneightry;
  int64_t maxneighact;
  int64_t ncalc;         /* dens.F90:1679 */
  int64_t np;
  int64_t ncalls_neigh;  /* redo walks, dens.F90:362 */
  int64_t ncells;
  int64_t maxlevel;
  int64_t minlevel;
  double rhomax;
} ora_stats;

void *ora_create(const ora_params *p);
void ora_destroy(void *o);
int ora_set_params(void *o, const ora_params *p);
/* particle arrays in the reference layout: xyzh(4,n), vxyzu(4,n), Bevol(4,n) */
int ora_set_particles(void *o, int64_t n, const double *xyzh, const double *vxyzu,
                      const double *Bevol);
int ora_get_particles(void *o, double *xyzh, double *vxyzu, double *Bevol);

int ora_maketree(void *o);
/* alphaind(1,:) (the evolved viscosity parameter, float) of the particles */
int ora_set_alpha(void *o, const float *alpha);
/* alphaind(3,:) (alpha, alphaloc, div a) and dvdx(9,:), float, caller order */
int ora_get_alpha(void *o, float *alphaind, float *dvdx);
/* initial.F90:736-742: alphaind(1) = max(alphaind(1), alphaloc) after the initial derivs */
int ora_alpha_initial(void *o);
/* Individual timesteps (IND_TIMESTEPS). ora_ind_init after the initial
 * derivs (evol_init / init_step, step_leapfrog.f90:45-84); ora_ind_substep
 * one pass of the evolve loop (evol_prestep, step, evol_poststep: one
 * substep of dtmax / 2^nbinmax), returning the new time and the number of
 * active particles; ora_ind_state the bins, twas and counters. */
int ora_ind_init(void *o, double time);
int ora_ind_substep(void *o, double *time, int64_t *nactive);
int ora_ind_state(void *o, int8_t *ibin, double *twas, int32_t *counters);
/* revtree (kdtree.F90:1851-2037) on new positions of the same particles */
int ora_revtree(void *o, const double *xyzh);
int64_t ora_get_ncells(void *o);
/* node records of nodes 1..ncells (index 0 of each output row = node 1) */
int ora_get_tree(void *o, int32_t *inodeparts, int32_t *inoderange /*2*ncells*/,
                 double *xcen /*3*ncells*/, double *size, double *hmax,
                 double *mass, int32_t *left, int32_t *right, int32_t *parent,
                 int32_t *leaf_is_active, double *quads /*6*ncells or NULL*/);

int ora_densityiterate(void *o, int icall);
int ora_get_density(void *o, float *gradh /*2,n*/, float *divcurlv, float *divcurlB /*4,n*/,
                    int32_t *nneigh, uint64_t *neighhash, ora_stats *st);
int ora_cons2prim(void *o);
int ora_force(void *o, int icall, double dt);
int ora_get_force(void *o, double *fxyzu /*4,n*/, double *dBevol /*4,n*/,
                  float *divcurlv, float *divBsymm, float *poten, double *eos /*2,n*/,
                  double *dtcourant, double *dtforce);
/* derivs(icall): tree (icall==1) + density (icall==1) + cons2prim + force */
int ora_derivs(void *o, int icall, double dt, double *dtnew);
/* one global-timestep leapfrog step (step_leapfrog.f90:91-760) */
int ora_step(void *o, double t, double dtsph, double *dtnew, int32_t *its_out);
double ora_get_dterr(void *o);
/* brute-force O(N^2) neighbour count of particle i within radkern*h_i */
int ora_bruteforce_count(void *o, int64_t i, int32_t *count);
/* analytic kernel for golden tests */
/* compute_M2L (kdtree.F90:1702-1781): adds the expansion of a node of mass
 * `mass` and quadrupole quads(6) at separation dx = x_dst - x_src, dr1 =
 * 1/|dx|, to fnode(20); expand_fgrav_in_taylor_series (kdtree.F90:1799-1840)
 * at offset dx from the expansion centre: force f3 and potential */
void ora_m2l(double dx, double dy, double dz, double dr1, double mass, const double *quads, double *fnode);
void ora_taylor(const double *fnode, double dx, double dy, double dz, double *f3, double *phi);
void ora_kernel(double q2, double q, double *w, double *gr, double *dphidh,
                double *potsoft, double *fsoft);

#ifdef __cplusplus
}
#endif
#endif
