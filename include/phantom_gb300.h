/*
 * phantom_gb300 — C ABI of the GB300 (sm_103a) implementation of Phantom's
 * per-step SPH particle hot path: kd-tree build with leaf-cell neighbour
 * lists, the density h-rho Newton-Raphson solve, the hydro/MHD force pair
 * loop and the leapfrog step.
 *
 * Array conventions follow the reference (src/main/part.F90:47-391):
 * Fortran column-major (k,N) arrays, i.e. k consecutive values per particle,
 * particle indices in the caller's order. xyzh(4,N), vxyzu(maxvxyzu,N), Bevol(4,N),
 * fxyzu(maxvxyzu,N), dBevol(4,N) are double; gradh(2,N), divcurlv(ndivcurlv,N)
 * (ndivcurlv = 4 with params.curlv, else 1), divcurlB(4,N), divBsymm(N),
 * poten(N) are float, as in the reference's DOUBLEPRECISION build.
 *
 * Every entry point returns 0 on success or a PH_ERR_* code. Device-side
 * failures are reported through an error word, never through a trap.
 * Calls are synchronous on return. A context is single-threaded and owns one
 * CUDA stream on the device that was current when ph_init was called.
 */
#ifndef PHANTOM_GB300_H
#define PHANTOM_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PH_OK = 0,
  PH_ERR_ARG = 1,          /* invalid argument */
  PH_ERR_CUDA = 2,         /* CUDA runtime error */
  PH_ERR_NAN_POS = 3,      /* NaN particle position (kdtree.F90:391-393) */
  PH_ERR_NOPART = 4,       /* no live particles (kdtree.F90:162-164) */
  PH_ERR_TREE = 5,         /* tree build inconsistency (kdtree.F90:588-591, 851-853) */
  PH_ERR_STACK = 6,        /* walk stack overflow (kdtree.F90:1305) */
  PH_ERR_DENS_NOCONV = 7,  /* h-rho iteration did not converge (dens.F90:1443-1456) */
  PH_ERR_NEG_H = 8,        /* negative smoothing length (dens.F90:1566,1598; force.F90:2271) */
  PH_ERR_DT = 9,           /* invalid Courant timestep (force.F90:3214) */
  PH_ERR_TOLV = 10,        /* leapfrog velocity iterations not converged (step_leapfrog.f90:753-756) */
  PH_ERR_LIST = 11,        /* neighbour list pool exhausted (retried internally) */
  PH_ERR_CAPACITY = 12,    /* npart exceeds the context capacity */
  PH_ERR_STATE = 13,       /* call order: e.g. force before density */
  PH_ERR_NOT_BUILT = 14,   /* feature not compiled into this library */
  PH_ERR_SCRATCH_LIMIT = 15, /* npart above PH_NOALLOC_MAX_PARTICLES (ph_conservation_noalloc) */
  PH_ERR_IND = 16,         /* timestep bins inconsistent: a bin above nbinmax or a step count
                              that does not divide (utils_indtimesteps.f90:135-139, 195-198) */
  PH_ERR_IND_DT = 17       /* a timestep below the smallest bin (step_leapfrog.f90:426-431) */
};

enum { PH_PREC_FP64 = 0, PH_PREC_MIXED = 1 };

/* Compile-time switches (config.F90 `module dim`) and run-time options of the
 * reference, gathered in one record. */
typedef struct ph_params {
  int32_t periodic;           /* PERIODIC */
  int32_t mhd;                /* MHD (ideal; fast_divcurlB) */
  int32_t gravity;            /* GRAVITY */
  int32_t isothermal;         /* ISOTHERMAL: vxyzu holds no u */
  int32_t ieos;               /* 1 isothermal, 2 adiabatic (eos.f90:184-237) */
  int32_t ipdv_heating;       /* eos.f90:1897 */
  int32_t ishock_heating;     /* eos.f90:1896 */
  int32_t iresistive_heating; /* eos.f90:1898 */
  int32_t precision;          /* PH_PREC_FP64 or PH_PREC_MIXED */
  int32_t minpart;            /* leaf size (config.F90:113 minpart, a compile-time
                                 constant there): 0 selects the reference's 10;
                                 2..16 accepted (PH_ERR_ARG otherwise) */
  double xmin, xmax, ymin, ymax, zmin, zmax; /* boundary.f90 */
  double hfact, tolh, massoftype;            /* options.f90:92-93, part.F90 */
  double alpha, alphau, alphaB, beta;        /* shock_capturing.f90:47-65 */
  double gamma, polyk;                       /* eos.f90 */
  double C_cour, C_force, tolv, dtmax;       /* timestep.f90:52-62 */
  double psidecayfac, overcleanfac;          /* timestep.f90:60-61 */
  double tree_accuracy;                      /* kdtree.F90:46 */
  int64_t maxp;                              /* allocation size (config.F90:393) */
  double alphamax;            /* shock_capturing.f90:35 upper bound of the Cullen-Dehnen switch
                                 (0 selects the reference's 1.0) */
  int32_t nalpha;             /* config.F90:158-162: 0 = CONST_AV (alpha constant), 3 = the
                                 Cullen & Dehnen switch (alpha per particle, alphaind(3,:)) */
  int32_t ind_timesteps;      /* IND_TIMESTEPS: individual particle timesteps in power-of-two
                                 bins of dtmax (ph_ind_*); 0 = global timestep (ph_step) */
  int32_t maxvxyzu;           /* config.F90:50-53: rows of the caller's vxyzu and fxyzu
                                 arrays (part.F90:465,516). 0 or 4: four rows; 3: the
                                 ISOTHERMAL layout vxyzu(3,N), fxyzu(3,N), isothermal = 1 only */
  int32_t curlv;              /* CURLV (config.F90:166,384): 1 = divcurlv holds ndivcurlv = 4 rows,
                                 div v and curl v (dens.F90:919-923, from the density's
                                 velocity-derivative sums); 0 = the one row div v */
} ph_params;

/* Neighbour statistics of the last density call (dens.F90:1137-1199). */
typedef struct ph_neigh_stats {
  int64_t nneightry, nneighact, maxneightry, maxneighact;
  int64_t ncalc, np, ncalls_neigh, ncells, maxlevel, minlevel;
  double rhomax;
} ph_neigh_stats;

typedef struct ph_ctx ph_ctx;

/* Create a context for up to maxp particles (allocates device memory).
 * Replaces the allocation done by allocate_neigh/allocate_kdtree
 * (neigh_kdtree.f90:56-72, kdtree.F90:75-87). */
int ph_init(const ph_params *params, int64_t maxp, ph_ctx **ctx);
int ph_set_params(ph_ctx *ctx, const ph_params *params);
void ph_finalize(ph_ctx *ctx);
const char *ph_strerror(int code);

/* Copy particle state to the device (caller order, reference layout).
 * Bevol may be NULL when mhd == 0. */
int ph_upload(ph_ctx *ctx, int64_t npart, const double *xyzh, const double *vxyzu,
              const double *Bevol);
int ph_download(ph_ctx *ctx, double *xyzh, double *vxyzu, double *Bevol);

/* maketree (kdtree.F90:117-314) via build_tree (neigh_kdtree.f90:161-208):
 * builds the tree on the device-resident positions (applying the periodic
 * wrap of construct_root_node), and optionally returns the particle
 * permutation inodeparts (1-based, as in kdtree.F90:32) and ncells as
 * maketree returns it (kdtree.F90:167-179, 299-301, 820-833): 2^(maxlevel+1)-1
 * while the tree stays within the 2^k-indexed levels (maxlevel_indexed from
 * ncellsmax = 2 maxp), else that indexed extent plus one per deeper node; the
 * number of nodes built is ph_get_nodes' count. xyzh (optional) receives the
 * wrapped positions. ph_last_timings then holds the build's device time in
 * ms8[0]. */
int ph_build_tree(ph_ctx *ctx, double *xyzh, int32_t *inodeparts, int64_t *ncells);

/* revtree (kdtree.F90:1851-2037): every node's centre of mass, size, hmax,
 * mass (and quadrupoles with self-gravity) recomputed from new positions
 * xyzh(4,:) of the same particles (caller order), on the structure of the
 * tree built last (no rebuild: particle order, ranges and children kept, no
 * periodic wrap). Density and force state is invalidated. ph_last_timings
 * then holds the refit's device time (after the copy of xyzh) in ms8[0]. */
int ph_revtree(ph_ctx *ctx, const double *xyzh);

/* The nodes of the current tree (the reference's module array `node`,
 * dtype_kdtree.F90:53-68) in this library's node order: inoderange(2,:)
 * 1-based as kdtree.F90:31, xcen(3,:), size, hmax, mass, and 1 for leaves.
 * *nnodes receives the node count; with any array NULL only the count is
 * returned. */
int ph_get_nodes(ph_ctx *ctx, int64_t *nnodes, int32_t *inoderange, double *xcen, double *size,
                 double *hmax, double *mass, int32_t *isleaf);

/* densityiterate(icall,...) (dens.F90:117-568) on the last built tree.
 * Outputs (optional, caller order): xyzh(4,:) with updated h, gradh(2,:),
 * divcurlv(ndivcurlv,:) (rows 2-4 curl v with curlv), divcurlB(4,:),
 * per-particle neighbour count and an
 * order-independent hash of the neighbour set, statistics. */
int ph_density(ph_ctx *ctx, int icall, double *xyzh, float *gradh, float *divcurlv,
               float *divcurlB, int32_t *nneigh, uint64_t *neighhash, ph_neigh_stats *stats);

/* cons2prim_everything (cons2prim.f90:274-456) followed by
 * force(icall,...) (force.F90:193-905). Outputs (optional, caller order):
 * fxyzu(4,:), dBevol(4,:), divcurlv(ndivcurlv,:) (row 1 div v from the
 * force loop; rows 2-4, with curlv, curl v of the last density call),
 * divBsymm(:), poten(:), and the global dtcourant / dtforce minima. */
int ph_force(ph_ctx *ctx, int icall, double dt, double *fxyzu, double *dBevol, float *divcurlv,
             float *divBsymm, float *poten, double *dtcourant, double *dtforce);

/* derivs(icall,...) (deriv.f90:37-232): tree + density (icall == 1),
 * cons2prim, force; returns dtnew = min(dtforce, dtcourant, dtmax). */
int ph_derivs(ph_ctx *ctx, int icall, double dt, double *dtnew);

/* One global-timestep leapfrog step, step(...) (step_leapfrog.f90:91-760),
 * entirely on the device. Returns dtnew, the velocity-iteration count and
 * dterr (check_velocity_error, step_leapfrog.f90:769-843). */
int ph_step(ph_ctx *ctx, double t, double dtsph, double *dtnew, int32_t *its, double *dterr);

/* Total momentum, kinetic + thermal (+ magnetic) energy and their rates, in
 * FP64, of the device-resident state (energies.f90:65-711 formulas). out[8]:
 * px, py, pz, ekin, etherm, emag, epot, sum_i m_i (v_i.a_i + du_i/dt). */
int ph_conservation(ph_ctx *ctx, double *out);

/* Full integrator state transfer (caller order): positions/h, velocities/u,
 * B/rho and psi, the accelerations and dB/dt of the last force evaluation and
 * divcurlv(ndivcurlv,:) (float). ph_upload_state makes the state ready for ph_step without a
 * preceding ph_derivs; used when the caller owns the step loop on the host.
 * Bevol and dBevol may be NULL when mhd == 0. */
int ph_upload_state(ph_ctx *ctx, int64_t npart, const double *xyzh, const double *vxyzu,
                    const double *Bevol, const double *fxyzu, const double *dBevol,
                    const float *divcurlv);
int ph_download_state(ph_ctx *ctx, double *xyzh, double *vxyzu, double *Bevol, double *fxyzu,
                      double *dBevol, float *divcurlv);

/* Timing of the last derivs/step call in milliseconds (CUDA events on the
 * context stream): ms8[0..3] tree, density, force, integrate phases;
 * ms8[4] the dominant force pair-loop kernel; ms8[5] the density pass kernels;
 * ms8[6] the neighbour walks; ms8[7] the whole ph_step call. */
int ph_last_timings(ph_ctx *ctx, double *ms8);

/* Work counters of the last derivs/step call: out[0] sum over leaf cells of
 * the force trial-list length, out[1] the same over all density passes,
 * out[2] force (i, trial j) pairs visited, out[3] density pairs visited. */
int ph_work_counters(ph_ctx *ctx, int64_t *out4);

/* Kernel launch counter of the context since creation (all kernels). */
int64_t ph_kernel_launches(ph_ctx *ctx);

/* Adjoint of one derivs evaluation (differentiation form; the reference has
 * no adjoint, the entry point follows its array conventions). For the
 * context's current state (xyzh, vxyzu as uploaded) and a cotangent
 * w_fxyzu(4,N) on the results fxyzu(4,N) of ph_derivs, returns the gradient
 * of L = sum w_fxyzu . fxyzu with respect to xyzh(1:3) (g_xyzh(4,N); the h
 * slot is 0: h follows from the positions through the density solve) and
 * vxyzu(1:4) (g_vxyzu(4,N)). The tree, the converged density solve
 * (dens.F90:117-1681) and the force trial lists are recomputed when the
 * state changed; pair terms (force.F90:914-1990) are recomputed, not stored.
 * Differentiated model: the converged h-rho solve with 1/Omega in FP64
 * (implicit differentiation of rho(h) = sum m W). Ideal MHD contexts also
 * return the gradient with respect to Bevol(1:4) in g_Bevol(4,N) (required).
 * With the Cullen-Dehnen switch (nalpha = 3) the per-particle
 * alpha of the evaluation (ph_set_alpha / the state) is held fixed, as it is
 * within one derivs; gradients through its evolution across steps are not
 * built. With self-gravity the gradient includes the softened near field
 * with its gradsoft term (force.F90:1303-1340, differentiated through the
 * density solve like 1/Omega), the 1/r^2 trial pairs (force.F90:1991-2053)
 * and the far field: the M2L sums of the node centres of mass and
 * quadrupoles, their propagation and expansion (kdtree.F90:1702-1840), with
 * the walk's near/far decisions those of the tree built from the uploaded
 * h. A context with individual timesteps returns PH_ERR_NOT_BUILT (its
 * evaluations re-compute the active particles' forces only). */
int ph_adjoint(ph_ctx *ctx, const double *w_fxyzu, double *g_xyzh, double *g_vxyzu, double *g_Bevol);

/* ph_adjoint with a cotangent of dBevol as well (MHD; w_dBevol(4,N), may be
 * NULL): the gradient of sum w_fxyzu . fxyzu + sum w_dBevol . dBevol. Adds
 * the reverse of the induction, artificial resistivity and psi cleaning
 * terms of d(B/rho)/dt (force.F90:1630-1671), of dpsi/dt with its div B
 * diffusion, decay and div v terms (force.F90:3107-3123; written, as there,
 * with psidecayfac > 0) and of the resistive heating in du/dt; g_Bevol(4,N)
 * holds the gradients with respect to B/rho and psi. */
int ph_adjoint_full(ph_ctx *ctx, const double *w_fxyzu, const double *w_dBevol, double *g_xyzh,
                    double *g_vxyzu, double *g_Bevol);

/* Adjoint through a rollout (differentiation form; no counterpart in the
 * reference, whose step loop this follows: step_leapfrog.f90:91-760 with one
 * corrector pass, its tolv > 1e2 branch). From the state of the last
 * ph_upload: one derivs, then nsteps global-timestep leapfrog steps with the
 * given timesteps dts[nsteps], entirely on the device; *loss receives
 * L = sum w_fxyzu . fxyzu of the last force evaluation (w_fxyzu(maxvxyzu,N)),
 * g_xyzh(4,N) and g_vxyzu(maxvxyzu,N) the gradient of L with respect to the
 * initial positions (h slot 0) and velocities and thermal energies. The
 * state is checkpointed in device memory every ckpt steps; the reverse pass
 * recomputes each segment forward from its checkpoint and reverses it step
 * by step with one adjoint (ph_adjoint's) per force evaluation, neighbour
 * lists and pair terms recomputed. The device state is left at the initial
 * state with its forces. ph_last_timings: ms8[0] the forward rollout, ms8[1]
 * the reverse pass, ms8[2] its adjoint evaluations, ms8[3] its segment
 * recomputes, ms8[7] the whole call. With self-gravity each adjoint starts
 * from the h its forward evaluation started from (the predicted h of the
 * step, the uploaded h for the first), so its tree, node hmax and walk are
 * the forward's; otherwise from the converged h. The Cullen-Dehnen switch and individual timesteps return
 * PH_ERR_NOT_BUILT. */
int ph_rollout_adjoint(ph_ctx *ctx, int32_t nsteps, const double *dts, int32_t ckpt, const double *w_fxyzu,
                       double *loss, double *g_xyzh, double *g_vxyzu);

/* ph_rollout_adjoint with MHD: L = sum w_fxyzu . fxyzu + sum w_dBevol . dBevol
 * of the last evaluation (w_dBevol(4,N), may be NULL) and, in g_Bevol(4,N)
 * (may be NULL), its gradient with respect to the initial Bevol (B/rho and
 * psi). Bevol is kicked with dBevol like the velocities (step_leapfrog.f90
 * predict_sph and the corrector) and each evaluation uses the predicted
 * Bevol, as the reference's derivs call does. */
int ph_rollout_adjoint_full(ph_ctx *ctx, int32_t nsteps, const double *dts, int32_t ckpt, const double *w_fxyzu,
                            const double *w_dBevol, double *loss, double *g_xyzh, double *g_vxyzu,
                            double *g_Bevol);

/* Cullen & Dehnen viscosity switch (nalpha = 3, the reference's default
 * build): alphaind(1,:) is the evolved alpha of each particle (float, as
 * part.F90:50), zero after ph_upload (part.F90:688). ph_set_alpha sets it
 * (e.g. from the 'alpha' array of a dump); ph_get_alpha returns alphaind(3,:)
 * (alpha, alphaloc of the last cons2prim, d(div v)/dt of the last density)
 * and dvdx(9,:) (either may be NULL); ph_alpha_initial applies
 * alpha = max(alpha, alphaloc) after the initial derivs (initial.F90:736-742).
 * With nalpha = 0 these are no-ops and alpha = ph_params.alpha. */
int ph_set_alpha(ph_ctx *ctx, const float *alpha);
int ph_get_alpha(ph_ctx *ctx, float *alphaind, float *dvdx);
int ph_alpha_initial(ph_ctx *ctx);

/* Individual timesteps (ind_timesteps = 1; utils_indtimesteps.f90,
 * step_leapfrog.f90, evolve.f90). Particle i steps with dtmax / 2^ibin(i);
 * a substep advances time by dtmax / 2^nbinmax and updates the particles
 * whose bin divides the step count (density and force on active leaf cells
 * and active particles only, neighbours of active particles woken, bins
 * limited to one below their neighbours'). After the initial ph_derivs
 * (all particles active; bins from the forces), ph_ind_init(time) starts
 * the scheme (init_step, step_leapfrog.f90:45-84); each ph_ind_substep is
 * one pass of the evolve loop (evol_prestep, step, evol_poststep) and
 * returns the new time and the number of particles it updated;
 * ph_ind_state returns ibin (int8), twas and counters (nbinmax,
 * istepfrac, ibinnow, 0). */
int ph_ind_init(ph_ctx *ctx, double time);
int ph_ind_substep(ph_ctx *ctx, double *time, int64_t *nactive);
int ph_ind_state(ph_ctx *ctx, int8_t *ibin, double *twas, int32_t *counters);

/* Launch configuration and leaf size of a context. No counterpart in the
 * reference: its leaf size is the compile-time minpart (config.F90:113) and
 * its cell loops are OpenMP-scheduled (dens.F90:270, force.F90:420). */
typedef struct ph_tune {
  int32_t minpart;      /* leaf size of the trees the context builds */
  int32_t dens_warps;   /* warps (one leaf cell each) per block, density pair kernel */
  int32_t force_warps;  /* warps per block, force pair kernel */
  int32_t walk_warps;   /* warps per block, neighbour walks */
  double ms_before;     /* last ph_autotune: one ph_derivs(icall=1) (tree + density
                           + force, ms) with the configuration found on entry */
  double ms_after;      /* the same with the configuration it chose */
  int32_t force_sym;    /* FP64 force without self-gravity, global timesteps: 1 (default)
                           evaluates each unordered neighbour pair once and adds its terms
                           to both particles' sums; 0 evaluates it from each side, as the
                           reference's loop does. Results agree to rounding (1e-12 of the
                           largest magnitude), not bit for bit */
} ph_tune;

enum { PH_TUNE_LEAF = 1 }; /* ph_autotune flag: also tune the leaf size */

/* Small autotuner for the particle set last uploaded: times ph_derivs(icall=1)
 * with 1, 2 and 4 warps per block for the density pair, force pair and walk
 * kernels (best of three runs) and keeps, per kernel family, the fastest when it
 * beats the setting found on entry by more than 2 %; with PH_TUNE_LEAF it then tries leaf sizes
 * 6, 8, 10, 12 and 16. Warps per block change no result bit. The leaf size
 * changes the trial lists and the summation order, so results then agree with
 * the reference's minpart = 10 to rounding, not bit for bit: it is tuned only
 * on request. The device state is restored afterwards: the context is as after
 * the last ph_upload (call ph_derivs before ph_step). out may be NULL. */
int ph_autotune(ph_ctx *ctx, int flags, ph_tune *out);
/* The configuration in use; ph_set_tune sets it (warps 1, 2 or 4, minpart
 * 2..16 or 0 for the reference's 10; a changed leaf size invalidates the
 * tree). */
int ph_get_tune(ph_ctx *ctx, ph_tune *out);
int ph_set_tune(ph_ctx *ctx, const ph_tune *in);

/* No counterpart in the reference: an entry point of this library only.
 * The sums of ph_conservation (same out[8]) over arrays the caller keeps in
 * device memory, for callers that cannot let the library allocate: codes
 * whose device arrays come from their own allocator (OpenACC, CUDA Fortran,
 * a pool that reserved the memory up front), which have no context, and
 * which cannot afford the device-wide synchronisation of cudaMalloc/cudaFree
 * in the middle of a step. It allocates nothing. Its scratch is a fixed
 * 1 MiB array in the library's device image (8 doubles per 256 particles),
 * held on every GPU that loads the library until the process exits, so
 * npart is limited to PH_NOALLOC_MAX_PARTICLES (PH_ERR_SCRATCH_LIMIT above).
 * xyzh, vxyzu, fxyzu (and Bevol when params->mhd, poten when
 * params->gravity) are device arrays of the current device in the layouts
 * above (vxyzu and fxyzu with params->maxvxyzu rows); out is a device array
 * of 8 doubles. The work is enqueued on
 * `stream` (a cudaStream_t; NULL = default stream) and the call returns
 * without waiting: out is valid after the stream has been synchronised.
 * Each call looks up the scratch address on the current device (a lookup, no
 * allocation; a cudaDeviceReset may move it). The first call on a device also
 * loads the library's device image there: make that first call before any
 * stream capture. An error already pending in the calling thread is returned
 * as PH_ERR_CUDA, left pending, and nothing is launched. Every call shares the one
 * scratch array, so calls whose work overlaps on the GPU (other streams,
 * other host threads) race and give wrong sums: serialise them. */
#define PH_NOALLOC_MAX_PARTICLES 4194304
int ph_conservation_noalloc(const ph_params *params, int64_t npart, const double *xyzh,
                            const double *vxyzu, const double *fxyzu, const double *Bevol,
                            const float *poten, double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
