// Host-side context of the phantom_gb300 library (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "ph_common.cuh"

namespace ph {

constexpr int SMALL = 2048;  // nodes with <= SMALL particles are built by the generation kernels
constexpr int CHUNK = 2048;  // elements per block in the large-node level kernels
constexpr int PSUM = 24;     // per-particle pair-sum slots (density, force and adjoint pair kernels)
constexpr int LENFG = 20;    // gravity far-field coefficients per node (kdtree.F90 lenfgrav)
constexpr int ADJREC = 48;   // adjoint per-particle record (doubles)
constexpr int ANODE = 32;    // adjoint per-node record of the far field (doubles)

// a node of at most SMALL particles waiting to be built, with its bounding box
struct GenEntry {
  int id, start, count, level, parent, pad;
  double bb[6];
};

struct DeviceBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

// launch bookkeeping shared by all translation units
void count_launch(ph_ctx *c, int k = 1);
cudaError_t check_launch(ph_ctx *c);

// exclusive scan of n ints (out may alias in); total written to *d_total if non-null
void scan_int(ph_ctx *c, const int *in, int *out, int n, int *d_total);
void fill_int(ph_ctx *c, int *a, int n, int v);
int grow_pool(ph_ctx *c);

int build_tree(ph_ctx *c);
int revtree(ph_ctx *c);
int alloc_ind(ph_ctx *c);
int ind_after_tree(ph_ctx *c);
int alloc_dvsum(ph_ctx *c);
int alloc_curlv(ph_ctx *c);
int copy_divcurlv_d2h(ph_ctx *c, float *host, size_t n);
int copy_divcurlv_h2d(ph_ctx *c, const float *host, size_t n);
int get_nodes(ph_ctx *c, int64_t *nnodes, int32_t *range, double *xcen, double *size, double *hmax, double *mass,
              int32_t *isleaf);
int ref_ncells(ph_ctx *c, int64_t *ncells);
int density(ph_ctx *c, int icall);
int force_dev(ph_ctx *c, const double *vel, const double *Bv);
int derivs_dev(ph_ctx *c, int icall, const double *vel, const double *Bv, double *dtnew);
int force_lists(ph_ctx *c);
// symmetric FP64 pair loop: cell_at / cell_tbase (per position / cell), the
// flattened trial offsets toff (pool capacity) and the j-side buffer jbuf
// (nj values x stride doubles), grown to the sizes asked for
int alloc_sym(ph_ctx *c, int64_t jbuf_stride, int nj);
// device buffer of the rollout adjoint (checkpoints, segment states, cotangents), grown to `doubles`
int alloc_rollout(ph_ctx *c, size_t doubles);
int gravity_far(ph_ctx *c);
int alloc_gravity(ph_ctx *c);
int alloc_adjoint(ph_ctx *c);
// the adjoint on the device-resident state (device cotangents and gradients, caller order)
int adjoint_dev(ph_ctx *c, const double *w_dev, const double *wB_dev, double *gx_d, double *gv_d, double *gb_d);
int gravity_adjoint_far(ph_ctx *c, const double *w, int wstride, double *out, int64_t ps);
int dual_walk(ph_ctx *c);
int far_levels(ph_ctx *c);
constexpr int LV_MAXDEPTH = 96;  // deepest node chain of the far field (the walks' MAXBRANCH)
int alloc_levels(ph_ctx *c, int64_t need);
int gravity_down(ph_ctx *c);
// accumulate the elapsed time of an event pair into last_ms[slot] (after a sync)
void add_elapsed(ph_ctx *c, int slot, cudaEvent_t a, cudaEvent_t b);
void reset_timers(ph_ctx *c);
// host copies of the caller's (maxvxyzu, N) vxyzu / fxyzu arrays (ph_capi.cu)
void copy_vrows_h2d(ph_ctx *c, double *dst, const double *src, size_t n);
void copy_vrows_d2h(ph_ctx *c, double *dst, const double *src, size_t n);

}  // namespace ph

struct ph_ctx {
  ph_params hp{};
  ph::Params dp{};
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t cap = 0;  // particle capacity
  int64_t n = 0;    // live particle count (caller order)
  int64_t launches = 0;
  bool have_tree = false, have_density = false, have_force = false, have_force_lists = false;
  // kernel attributes (dynamic shared memory) set on this context's device:
  // bit 0 density pair kernels, bit 1 force pair kernels, bit 2 adjoint
  unsigned attr_done = 0;
  // warps (leaf cells) per block of the pair and walk kernels (ph_autotune)
  int dens_warps = 4, force_warps = 4, walk_warps = 2;
  double tune_ms_before = 0.0, tune_ms_after = 0.0;  // last ph_autotune

  // caller-order particle state (reference layout)
  double *xyzh = nullptr, *vxyzu = nullptr, *Bevol = nullptr;
  double *fxyzu = nullptr, *dBevol = nullptr;
  double *vpred = nullptr, *Bpred = nullptr;  // step_leapfrog.f90 vpred, Bpred
  double *eos = nullptr;                      // eos_vars(igasP, ics)
  float *gradh = nullptr, *divcurlv = nullptr, *divcurlB = nullptr, *divBsymm = nullptr, *poten = nullptr;
  float *gradh_t = nullptr;  // gradh(2,:) in tree order (read by the force prologue)
  // Cullen & Dehnen switch: alphaind(1,:) caller order (state); alphaloc,
  // d(div v)/dt, dvdx(9,:) and the density's div v normalisation in tree order
  float *alpha1 = nullptr, *alphaloc_t = nullptr, *ddivvdt_c = nullptr, *dvdx_c = nullptr;
  double *dvterm_t = nullptr;
  double *dvsum = nullptr;  // the 25 per-particle sums of the dv pass (slot-major, allocated on first use)
  float *curl3 = nullptr;   // curl v, 3 rows per particle, caller order (curlv; allocated on first use)
  float *dcv_stage = nullptr;  // the caller's divcurlv(4,N) staged for one copy (curlv)
  const double *dens_vel = nullptr;  // velocities of the density's dv sums (vxyzu or vpred)
  const double *dens_B = nullptr;    // Bevol of the density's div B, curl B sums (Bevol or Bpred)
  // individual timesteps: bins, twas and activity per particle (caller order),
  // their tree-order copies for the pair kernels, the active leaf cells
  int8_t *ibin = nullptr, *ibin_old = nullptr, *ibin_wake = nullptr, *ibin_old_t = nullptr;
  double *twas = nullptr;
  unsigned char *actf = nullptr, *actf_t = nullptr, *wakemark = nullptr;
  int *cell_act = nullptr, *d_ind = nullptr;
  int ncell_act = 0;
  int nbinmax = 0, istepfrac = 0, ibinnow = 0;
  int ind_icall = 1;          // derivs icall of the force (get_newbin may move a bin down for icall < 2)
  bool ind_too_small = false;  // a force timestep below the smallest bin
  double ind_tlast = 0.0, ind_dtsub = 0.0;
  double ibin_dts[4][ph::MAXBINS + 1] = {};  // itdt, ithdt, itdt1, ittwas
  // the density's caller-order outputs that no later kernel reads (gradh,
  // divcurlv, divcurlB, neighbour counts and hashes) are written only when a
  // ph_density call asks for them
  bool want_diag = false;
  int32_t *nneigh = nullptr;
  uint64_t *nhash = nullptr;

  // tree-order copies (treecache, kdtree.F90 part.F90 treecache(5,:))
  int64_t ntree = 0;
  double *tx = nullptr, *ty = nullptr, *tz = nullptr, *th = nullptr;
  int *perm = nullptr;      // tree position -> caller index (0-based)
  int *iperm = nullptr;     // caller index -> tree position
  int *alive = nullptr;     // scratch flags / scan
  int *pairpos = nullptr;   // partition scratch

  // nodes
  ph::Node *nodes = nullptr;
  ph::NodeF *nodesf = nullptr;  // FP32 mirror of the nodes (walk node tests)
  int *node_list = nullptr;      // ids of the nodes built by generations (all nodes: [0, nbig) + these)
  int nbig_nodes = 0, nsmall_nodes = 0;
  double *fb = nullptr;          // gravity: M2L coefficients per node id (LENFG each)
  double *gleaf = nullptr;       // gravity: far-field coefficients per leaf index
  // gravity, level-by-level far field: nodes grouped by depth, each node's
  // opened list (offset, length into opool), leaf node -> cell index
  int *lv_nodes = nullptr, *lv_depth = nullptr, *lv_hist = nullptr, *lv_flag = nullptr;
  int *o_off = nullptr, *o_len = nullptr, *opool = nullptr, *cell_of_node = nullptr;
  long long opool_cap = 0;
  float4 *mqf = nullptr;         // FP32 node mass and quadrupole (mixed form), two float4 per node id
  int *leaf_of = nullptr;        // gravity: leaf index of each tree position
  double *nmass = nullptr, *nquads = nullptr;
  int node_cap = 0, subbase = 0, root = 0;
  int *leaf_at = nullptr;   // tree position -> leaf node id starting there (or -1)
  int *leaves = nullptr;    // leaf node ids in ascending start order
  int nleaves = 0;
  int *d_maxlevel = nullptr;  // [maxlevel, minlevel]
  int maxlevel = 0, minlevel = 0;

  // level-build scratch
  int *lvl_a = nullptr, *lvl_b = nullptr;
  double *lvl_bb_a = nullptr, *lvl_bb_b = nullptr;
  ph::GenEntry *gen_a = nullptr, *gen_b = nullptr;  // small-node generation lists
  double *gen_com = nullptr;  // per generation entry: centre of mass and hmax
  double *mtab = nullptr;    // mtab[k]: sequential sum of k particle masses, k <= SMALL
  double mtab_pm = -1.0;     // the particle mass mtab was built for
  int gen_cap = 0;
  int *lvl_misc = nullptr;   // per level node: axis, nl, noswap
  double *lvl_pivot = nullptr;
  int *cbase = nullptr;
  double *part_d = nullptr;  // chunk partials (doubles)
  int *part_i = nullptr;     // chunk partials (ints)
  // device counters (64 ints): [0] nbig_next, [1] nsmall, [3], [4], [12] tree
  // build, [8] density cells of the next pass, [16..17] opened-list pool top
  // (64-bit), [20] nodes below the indexed levels (ncells)
  int *counters = nullptr;
  int lvl_cap = 0, chunk_cap = 0;

  // density state (per leaf index / per tree position)
  double *hcur = nullptr, *hold = nullptr;   // tree order
  double *gradh64 = nullptr;                 // 1/Omega (FP64) per tree position from the last density call
  double *gsoft64 = nullptr;                 // gradsoft (FP64) per tree position (self-gravity)
  double *adj_node = nullptr;                // adjoint far-field records per node id (self-gravity)
  double *adj = nullptr;                     // adjoint per-particle records (allocated on first use)
  float *adjf = nullptr;                     // their FP32 copy (precision form)
  double *psum = nullptr;                    // per tree position pair sums, PSUM slots of stride cap
  int *cell_nits = nullptr, *cell_state = nullptr;
  double *cell_hmax = nullptr;
  int *act_a = nullptr, *act_b = nullptr;

  // symmetric FP64 pair loop (each unordered pair once): leaf cell index at
  // its first tree position, per-cell base and per-entry flattened index of
  // the owned trial entries, j-side sums of the owned entries (value-major)
  bool force_sym = true;
  int *cell_at = nullptr, *cell_tbase = nullptr, *toff = nullptr;
  int64_t toff_cap = 0;
  double *jbuf = nullptr;
  int64_t jbuf_stride = 0, jbuf_bytes = 0;
  int64_t sym_total = 0;  // owned trial entries of the current lists (jbuf rows in use)

  double *ro_buf = nullptr;  // rollout adjoint buffer (ph_rollout_adjoint)
  size_t ro_cap = 0;

  // trial-list pool (leaf entries)
  ph::LeafEntry *pool = nullptr;
  int64_t pool_cap = 0;
  unsigned long long *pool_top = nullptr;
  int *cell_off = nullptr, *cell_nleaf = nullptr, *cell_ntrial = nullptr;

  // force state (tree order)
  double *jrec = nullptr;    // per tree position j-side record (force prologue)
  float *jrecf = nullptr;    // FP32 copy of the j records (mixed precision form)
  float4 *txf = nullptr;     // float x,y,z,h for the FP32 prefilter
  float4 *bjf = nullptr;     // FP32 B rho per tree position (mixed MHD density)
  double pf_hmin = 0.0;      // below this h the FP32 prefilter is bypassed
  double *red = nullptr;     // reductions: dtcourant, dtforce, rhomax, ...
  unsigned long long *stats = nullptr;

  int *d_err = nullptr;
  std::vector<ph::DeviceBuf> allocs;
  cudaEvent_t ev[8] = {};
  cudaEvent_t evk[8] = {};   // kernel-level event pairs: force, density pass, walk
  double last_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  double dtcourant = 1.e29, dtforce = 1.e29, dterr = 1.e29;

  // scan scratch
  int *scan_tmp = nullptr;
  int scan_cap = 0;
};

// stream sync + device error flag of a context (ph_capi.cu)
int check_cuda(ph_ctx *c);
