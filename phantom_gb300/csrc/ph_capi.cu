// C ABI of phantom_gb300: context lifetime, host<->device transfer and the
// entry points that replace maketree / densityiterate / force / step.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "ph_internal.h"

using namespace ph;

namespace {

template <typename T>
int dalloc(ph_ctx *c, T **p, size_t count) {
  size_t bytes = sizeof(T) * (count > 0 ? count : 1);
  void *q = nullptr;
  if (cudaMalloc(&q, bytes) != cudaSuccess) return PH_ERR_CUDA;
  cudaMemset(q, 0, bytes);
  c->allocs.push_back(DeviceBuf{q, bytes});
  *p = static_cast<T *>(q);
  return 0;
}

void dfree(ph_ctx *c, void *p) {
  for (size_t k = 0; k < c->allocs.size(); ++k)
    if (c->allocs[k].p == p) {
      cudaFree(p);
      c->allocs.erase(c->allocs.begin() + k);
      return;
    }
}

int alloc_all(ph_ctx *c, int64_t cap) {
  int r = 0;
  const size_t n = (size_t)cap;
  r |= dalloc(c, &c->xyzh, 4 * n); r |= dalloc(c, &c->vxyzu, 4 * n); r |= dalloc(c, &c->Bevol, 4 * n);
  r |= dalloc(c, &c->fxyzu, 4 * n); r |= dalloc(c, &c->dBevol, 4 * n);
  r |= dalloc(c, &c->vpred, 4 * n); r |= dalloc(c, &c->Bpred, 4 * n); r |= dalloc(c, &c->eos, 2 * n);
  r |= dalloc(c, &c->gradh, 2 * n); r |= dalloc(c, &c->divcurlv, n); r |= dalloc(c, &c->divcurlB, 4 * n);
  r |= dalloc(c, &c->gradh_t, 2 * n);
  r |= dalloc(c, &c->alpha1, n); r |= dalloc(c, &c->alphaloc_t, n); r |= dalloc(c, &c->ddivvdt_c, n);
  r |= dalloc(c, &c->dvdx_c, 9 * n); r |= dalloc(c, &c->dvterm_t, n);
  r |= dalloc(c, &c->divBsymm, n); r |= dalloc(c, &c->poten, n);
  r |= dalloc(c, &c->nneigh, n); r |= dalloc(c, &c->nhash, n);
  r |= dalloc(c, &c->tx, n); r |= dalloc(c, &c->ty, n); r |= dalloc(c, &c->tz, n); r |= dalloc(c, &c->th, n);
  r |= dalloc(c, &c->perm, n); r |= dalloc(c, &c->iperm, n); r |= dalloc(c, &c->alive, n + 1);
  r |= dalloc(c, &c->pairpos, n + 1);
  // nodes: large-node levels first, then 2 ids per particle for the warp-built subtrees
  int bigcap = (int)(4 * (n / SMALL + 1) * 64 + 64);
  c->subbase = bigcap;
  c->node_cap = bigcap + (int)(2 * n) + 2;
  r |= dalloc(c, &c->nodes, (size_t)c->node_cap);
  r |= dalloc(c, &c->nodesf, (size_t)c->node_cap);
  r |= dalloc(c, &c->node_list, (size_t)c->node_cap);
  r |= dalloc(c, &c->nmass, (size_t)c->node_cap);
  r |= dalloc(c, &c->nquads, 6 * (size_t)c->node_cap);
  r |= dalloc(c, &c->leaf_at, n); r |= dalloc(c, &c->leaves, n);
  r |= dalloc(c, &c->d_maxlevel, 4);
  c->lvl_cap = (int)(2 * (n / SMALL + 2) + 8);
  r |= dalloc(c, &c->lvl_a, (size_t)c->lvl_cap); r |= dalloc(c, &c->lvl_b, (size_t)c->lvl_cap);
  // a generation holds the children of nodes of more than minpart particles
  // (sized for the smallest accepted leaf size)
  c->gen_cap = (int)(2 * (n / (MINPART_LO + 1)) + 2 * (size_t)c->lvl_cap + 64);
  r |= dalloc(c, &c->gen_a, (size_t)c->gen_cap); r |= dalloc(c, &c->gen_b, (size_t)c->gen_cap);
  r |= dalloc(c, &c->mtab, (size_t)SMALL + 1);
  r |= dalloc(c, &c->gen_com, 4 * (size_t)c->gen_cap);
  r |= dalloc(c, &c->lvl_bb_a, 6 * (size_t)c->lvl_cap); r |= dalloc(c, &c->lvl_bb_b, 6 * (size_t)c->lvl_cap);
  r |= dalloc(c, &c->lvl_misc, 4 * (size_t)c->lvl_cap); r |= dalloc(c, &c->lvl_pivot, (size_t)c->lvl_cap);
  c->chunk_cap = (int)(n / CHUNK + c->lvl_cap + 8);
  r |= dalloc(c, &c->cbase, (size_t)c->lvl_cap + 1);
  r |= dalloc(c, &c->part_d, 16 * (size_t)std::max<int64_t>(c->chunk_cap, 2048));
  r |= dalloc(c, &c->part_i, 3 * (size_t)c->chunk_cap);
  r |= dalloc(c, &c->counters, 64);
  r |= dalloc(c, &c->hcur, n); r |= dalloc(c, &c->hold, n); r |= dalloc(c, &c->psum, PSUM * n);
  r |= dalloc(c, &c->gradh64, n); r |= dalloc(c, &c->gsoft64, n);
  r |= dalloc(c, &c->cell_nits, n); r |= dalloc(c, &c->cell_state, n); r |= dalloc(c, &c->cell_hmax, n);
  r |= dalloc(c, &c->act_a, n); r |= dalloc(c, &c->act_b, n);
  r |= dalloc(c, &c->cell_off, n); r |= dalloc(c, &c->cell_nleaf, n); r |= dalloc(c, &c->cell_ntrial, n);
  c->pool_cap = (int64_t)std::max<int64_t>(65536, (int64_t)n * 48);
  r |= dalloc(c, &c->pool, (size_t)c->pool_cap);
  r |= dalloc(c, &c->pool_top, 1);
  r |= dalloc(c, &c->txf, n);
  r |= dalloc(c, &c->bjf, n);
  r |= dalloc(c, &c->jrec, 32 * n);
  r |= dalloc(c, &c->jrecf, 32 * n);
  r |= dalloc(c, &c->red, 16);
  r |= dalloc(c, &c->stats, 16);
  r |= dalloc(c, &c->d_err, 4);
  c->scan_cap = (int)(2 * (n / 1024 + 8) + 64);
  r |= dalloc(c, &c->scan_tmp, (size_t)c->scan_cap);
  return r ? PH_ERR_CUDA : 0;
}



}  // namespace

int check_cuda(ph_ctx *c) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    fprintf(stderr, "phantom_gb300: CUDA error %s\n", cudaGetErrorString(e));
    return PH_ERR_CUDA;
  }
  int herr = 0;
  cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  return herr;
}

namespace ph {

int grow_pool(ph_ctx *c) {
  int64_t ncap = c->pool_cap * 2;
  LeafEntry *np_ = nullptr;
  if (cudaMalloc(&np_, sizeof(LeafEntry) * (size_t)ncap) != cudaSuccess) return PH_ERR_CUDA;
  cudaMemcpyAsync(np_, c->pool, sizeof(LeafEntry) * (size_t)c->pool_cap, cudaMemcpyDeviceToDevice, c->stream);
  cudaStreamSynchronize(c->stream);
  dfree(c, c->pool);
  c->allocs.push_back(DeviceBuf{np_, sizeof(LeafEntry) * (size_t)ncap});
  c->pool = np_;
  c->pool_cap = ncap;
  return 0;
}

int alloc_sym(ph_ctx *c, int64_t jbuf_stride, int nj) {
  int r = 0;
  if (!c->cell_at) {
    r |= dalloc(c, &c->cell_at, (size_t)c->cap);
    r |= dalloc(c, &c->cell_tbase, (size_t)c->cap + 1);
  }
  if (c->toff_cap < c->pool_cap) {
    if (c->toff) dfree(c, c->toff);
    c->toff = nullptr;
    r |= dalloc(c, &c->toff, (size_t)c->pool_cap);
    c->toff_cap = c->pool_cap;
  }
  const int64_t bytes = (int64_t)sizeof(double) * nj * jbuf_stride;
  if (c->jbuf_bytes < bytes || c->jbuf_stride < jbuf_stride) {
    if (c->jbuf) dfree(c, c->jbuf);
    c->jbuf = nullptr;
    // room for 25 % more trial entries than this build has
    const int64_t stride = jbuf_stride + jbuf_stride / 4 + 1024;
    r |= dalloc(c, &c->jbuf, (size_t)nj * (size_t)stride);
    c->jbuf_stride = stride;
    c->jbuf_bytes = (int64_t)sizeof(double) * nj * stride;
  }
  return r ? PH_ERR_CUDA : 0;
}

int alloc_rollout(ph_ctx *c, size_t doubles) {
  if (c->ro_cap >= doubles) return 0;
  if (c->ro_buf) dfree(c, c->ro_buf);
  c->ro_buf = nullptr;
  c->ro_cap = 0;
  if (dalloc(c, &c->ro_buf, doubles) != 0) return PH_ERR_CUDA;
  c->ro_cap = doubles;
  return 0;
}

// gravity far-field buffers, allocated on the first force evaluation with
// self-gravity (about 160 bytes per node id)
int alloc_gravity(ph_ctx *c) {
  if (c->fb) return 0;
  int r = 0;
  r |= dalloc(c, &c->fb, (size_t)LENFG * (size_t)c->node_cap);
  r |= dalloc(c, &c->gleaf, (size_t)LENFG * (size_t)c->cap);
  r |= dalloc(c, &c->leaf_of, (size_t)c->cap);
  return r ? PH_ERR_CUDA : 0;
}

// level-by-level far field: per-node arrays once, the opened-list pool
// (re)allocated to at least `need` entries
int alloc_levels(ph_ctx *c, int64_t need) {
  if (!c->lv_nodes) {
    const size_t nc = (size_t)c->node_cap;
    int r = 0;
    r |= dalloc(c, &c->lv_nodes, nc); r |= dalloc(c, &c->lv_depth, nc);
    r |= dalloc(c, &c->o_off, nc); r |= dalloc(c, &c->o_len, nc); r |= dalloc(c, &c->cell_of_node, nc);
    r |= dalloc(c, &c->lv_hist, 2 * (size_t)(LV_MAXDEPTH + 1)); r |= dalloc(c, &c->lv_flag, 4);
    r |= dalloc(c, &c->mqf, 2 * nc);
    if (r) return PH_ERR_CUDA;
  }
  if (c->opool_cap < need) {
    if (c->opool) dfree(c, c->opool);
    c->opool = nullptr;
    c->opool_cap = 0;
    if (dalloc(c, &c->opool, (size_t)need)) return PH_ERR_CUDA;
    c->opool_cap = need;
  }
  return 0;
}

// individual-timestep state (allocated for contexts with ind_timesteps)
int alloc_ind(ph_ctx *c) {
  if (c->ibin) return 0;
  const size_t n = (size_t)c->cap;
  int r = 0;
  r |= dalloc(c, &c->ibin, n); r |= dalloc(c, &c->ibin_old, n); r |= dalloc(c, &c->ibin_wake, n);
  r |= dalloc(c, &c->ibin_old_t, n); r |= dalloc(c, &c->twas, n);
  r |= dalloc(c, &c->actf, n); r |= dalloc(c, &c->actf_t, n); r |= dalloc(c, &c->wakemark, n);
  r |= dalloc(c, &c->cell_act, n); r |= dalloc(c, &c->d_ind, 8);
  return r ? PH_ERR_CUDA : 0;
}

// sums of the velocity-derivative pass of the Cullen & Dehnen switch
int alloc_dvsum(ph_ctx *c) {
  if (c->dvsum) return 0;
  return dalloc(c, &c->dvsum, 25 * (size_t)c->cap) ? PH_ERR_CUDA : 0;
}

// curl v (3 rows per particle, caller order) and the staging array of the
// caller's divcurlv(4,N), allocated on first use
int alloc_curlv(ph_ctx *c) {
  if (c->curl3) return 0;
  int r = dalloc(c, &c->curl3, 3 * (size_t)c->cap);
  r |= dalloc(c, &c->dcv_stage, 4 * (size_t)c->cap);
  return r ? PH_ERR_CUDA : 0;
}

// divcurlv(ndivcurlv, N) of the caller from the device's div v row and, with
// curl v, its three rows
__global__ void k_pack_divcurlv(int n, const float *divv, const float *curl3, float *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[4 * (size_t)i] = divv[i];
  for (int k = 0; k < 3; ++k) out[4 * (size_t)i + 1 + k] = curl3[3 * (size_t)i + k];
}
__global__ void k_unpack_divcurlv(int n, const float *in, float *divv, float *curl3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  divv[i] = in[4 * (size_t)i];
  for (int k = 0; k < 3; ++k) curl3[3 * (size_t)i + k] = in[4 * (size_t)i + 1 + k];
}

int copy_divcurlv_d2h(ph_ctx *c, float *host, size_t n) {
  if (!c->dp.curlv) {
    cudaMemcpyAsync(host, c->divcurlv, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream);
    return 0;
  }
  if (alloc_curlv(c) != 0) return PH_ERR_CUDA;
  k_pack_divcurlv<<<(int)((n + 255) / 256), 256, 0, c->stream>>>((int)n, c->divcurlv, c->curl3, c->dcv_stage);
  count_launch(c);
  cudaMemcpyAsync(host, c->dcv_stage, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, c->stream);
  return 0;
}

int copy_divcurlv_h2d(ph_ctx *c, const float *host, size_t n) {
  if (!c->dp.curlv) {
    cudaMemcpyAsync(c->divcurlv, host, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream);
    return 0;
  }
  if (alloc_curlv(c) != 0) return PH_ERR_CUDA;
  cudaMemcpyAsync(c->dcv_stage, host, sizeof(float) * 4 * n, cudaMemcpyHostToDevice, c->stream);
  k_unpack_divcurlv<<<(int)((n + 255) / 256), 256, 0, c->stream>>>((int)n, c->dcv_stage, c->divcurlv, c->curl3);
  count_launch(c);
  return 0;
}

// adjoint per-particle records (ADJREC doubles each)
int alloc_adjoint(ph_ctx *c) {
  int r = 0;
  if (!c->adj) r |= dalloc(c, &c->adj, (size_t)ADJREC * (size_t)c->cap);
  // the precision form's FP32 copy of the records
  if (!c->adjf && c->dp.precision == PH_PREC_MIXED) r |= dalloc(c, &c->adjf, (size_t)ADJREC * (size_t)c->cap);
  // self-gravity: per-node records of the far field's reverse
  if (!c->adj_node && c->dp.gravity) r |= dalloc(c, &c->adj_node, (size_t)ANODE * (size_t)c->node_cap);
  return r ? PH_ERR_CUDA : 0;
}

}  // namespace ph

namespace ph {

// Host copies of the caller's (maxvxyzu, N) arrays vxyzu and fxyzu to and
// from the four-row device layout. With maxvxyzu = 3 (ISOTHERMAL) a pitched
// copy moves the three rows of each particle and the device's fourth row
// (u, unused) is zero.
void copy_vrows_h2d(ph_ctx *c, double *dst, const double *src, size_t n) {
  if (n == 0) return;
  if (c->hp.maxvxyzu != 3) {
    cudaMemcpyAsync(dst, src, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, c->stream);
    return;
  }
  cudaMemsetAsync(dst, 0, sizeof(double) * 4 * n, c->stream);
  cudaMemcpy2DAsync(dst, 4 * sizeof(double), src, 3 * sizeof(double), 3 * sizeof(double), n,
                    cudaMemcpyHostToDevice, c->stream);
}
void copy_vrows_d2h(ph_ctx *c, double *dst, const double *src, size_t n) {
  if (n == 0) return;
  if (c->hp.maxvxyzu != 3) {
    cudaMemcpyAsync(dst, src, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, c->stream);
    return;
  }
  cudaMemcpy2DAsync(dst, 3 * sizeof(double), src, 4 * sizeof(double), 3 * sizeof(double), n,
                    cudaMemcpyDeviceToHost, c->stream);
}

}  // namespace ph

extern "C" {

const char *ph_strerror(int code) {
  switch (code) {
    case PH_OK: return "ok";
    case PH_ERR_ARG: return "invalid argument";
    case PH_ERR_CUDA: return "CUDA runtime error";
    case PH_ERR_NAN_POS: return "NaN in particle position";
    case PH_ERR_NOPART: return "no particles or all particles dead/accreted";
    case PH_ERR_TREE: return "tree build inconsistency";
    case PH_ERR_STACK: return "stack overflow in tree walk";
    case PH_ERR_DENS_NOCONV: return "could not converge in density";
    case PH_ERR_NEG_H: return "negative smoothing length";
    case PH_ERR_DT: return "invalid timestep";
    case PH_ERR_TOLV: return "velocity iterations not converged";
    case PH_ERR_LIST: return "neighbour list pool exhausted";
    case PH_ERR_CAPACITY: return "npart exceeds context capacity";
    case PH_ERR_STATE: return "call order (tree/density required first)";
    case PH_ERR_NOT_BUILT: return "feature not built";
    case PH_ERR_SCRATCH_LIMIT: return "npart exceeds the static scratch limit of ph_conservation_noalloc (4194304)";
    case PH_ERR_IND: return "timestep bins inconsistent";
    case PH_ERR_IND_DT: return "timestep below the smallest bin";
    default: return "unknown error";
  }
}

static bool params_ok(const ph_params *p) {
  return (p->minpart == 0 || (p->minpart >= MINPART_LO && p->minpart <= MAXCELL)) &&
         (p->nalpha == 0 || p->nalpha == 3) && (p->ind_timesteps == 0 || p->ind_timesteps == 1) &&
         (p->maxvxyzu == 0 || p->maxvxyzu == 4 || (p->maxvxyzu == 3 && p->isothermal)) &&
         (p->curlv == 0 || p->curlv == 1);
}

int ph_init(const ph_params *params, int64_t maxp, ph_ctx **out) {
  if (!params || !out || maxp <= 0 || maxp > (int64_t)1 << 28) return PH_ERR_ARG;
  if (!params_ok(params)) return PH_ERR_ARG;
  ph_ctx *c = new ph_ctx();
  c->hp = *params;
  c->dp = make_params(*params);
  cudaGetDevice(&c->device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { delete c; return PH_ERR_CUDA; }
  c->cap = maxp;
  if (alloc_all(c, maxp) != 0) { ph_finalize(c); return PH_ERR_CUDA; }
  for (int k = 0; k < 8; ++k) { cudaEventCreate(&c->ev[k]); cudaEventCreate(&c->evk[k]); }
  *out = c;
  return 0;
}

int ph_set_params(ph_ctx *c, const ph_params *params) {
  if (!c || !params || !params_ok(params)) return PH_ERR_ARG;
  if ((params->minpart > 0 ? params->minpart : MINPART) != c->dp.minpart)
    c->have_tree = c->have_density = c->have_force = c->have_force_lists = false;  // a new leaf size needs a new tree
  c->hp = *params;
  c->dp = make_params(*params);
  return 0;
}

void ph_finalize(ph_ctx *c) {
  if (!c) return;
  cudaStreamSynchronize(c->stream);
  for (auto &b : c->allocs) cudaFree(b.p);
  c->allocs.clear();
  for (int k = 0; k < 8; ++k) {
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
    if (c->evk[k]) cudaEventDestroy(c->evk[k]);
  }
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int ph_upload(ph_ctx *c, int64_t npart, const double *xyzh, const double *vxyzu, const double *Bevol) {
  if (!c || !xyzh || !vxyzu || npart <= 0) return PH_ERR_ARG;
  if (npart > c->cap) return PH_ERR_CAPACITY;
  c->n = npart;
  size_t b4 = sizeof(double) * 4 * (size_t)npart;
  cudaMemcpyAsync(c->xyzh, xyzh, b4, cudaMemcpyHostToDevice, c->stream);
  copy_vrows_h2d(c, c->vxyzu, vxyzu, (size_t)npart);
  if (Bevol) cudaMemcpyAsync(c->Bevol, Bevol, b4, cudaMemcpyHostToDevice, c->stream);
  else cudaMemsetAsync(c->Bevol, 0, b4, c->stream);
  cudaMemsetAsync(c->fxyzu, 0, b4, c->stream);
  cudaMemsetAsync(c->dBevol, 0, b4, c->stream);
  cudaMemsetAsync(c->divcurlv, 0, sizeof(float) * (size_t)npart, c->stream);
  if (c->curl3) cudaMemsetAsync(c->curl3, 0, sizeof(float) * 3 * (size_t)npart, c->stream);
  cudaMemsetAsync(c->gradh, 0, sizeof(float) * 2 * (size_t)npart, c->stream);
  cudaMemsetAsync(c->alpha1, 0, sizeof(float) * (size_t)npart, c->stream);  // part.F90:688
  cudaMemsetAsync(c->alphaloc_t, 0, sizeof(float) * (size_t)npart, c->stream);
  cudaMemsetAsync(c->ddivvdt_c, 0, sizeof(float) * (size_t)npart, c->stream);
  cudaMemsetAsync(c->dvdx_c, 0, sizeof(float) * 9 * (size_t)npart, c->stream);
  if (c->dp.ind) {  // initial.F90:160-165: bins 0, every particle active
    if (alloc_ind(c) != 0) return PH_ERR_CUDA;
    cudaMemsetAsync(c->ibin, 0, (size_t)npart, c->stream);
    cudaMemsetAsync(c->ibin_old, 0, (size_t)npart, c->stream);
    cudaMemsetAsync(c->ibin_wake, 0, (size_t)npart, c->stream);
    cudaMemsetAsync(c->twas, 0, sizeof(double) * (size_t)npart, c->stream);
    cudaMemsetAsync(c->actf, 1, (size_t)npart, c->stream);
    c->nbinmax = 0; c->istepfrac = 0; c->ibinnow = 0;
  }
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  c->have_tree = c->have_density = c->have_force = c->have_force_lists = false;
  // FP32 pre-filter guard: h must exceed 4e-4 of the coordinate scale
  double xs = 0.0;
  const double b[6] = {c->hp.xmin, c->hp.xmax, c->hp.ymin, c->hp.ymax, c->hp.zmin, c->hp.zmax};
  for (int k = 0; k < 6; ++k) xs = std::max(xs, std::fabs(b[k]));
  c->pf_hmin = 4.0e-4 * std::max(xs, 1.0e-300) * 4.0;
  return check_cuda(c);
}

int ph_download(ph_ctx *c, double *xyzh, double *vxyzu, double *Bevol) {
  if (!c) return PH_ERR_ARG;
  size_t b4 = sizeof(double) * 4 * (size_t)c->n;
  if (xyzh) cudaMemcpyAsync(xyzh, c->xyzh, b4, cudaMemcpyDeviceToHost, c->stream);
  if (vxyzu) copy_vrows_d2h(c, vxyzu, c->vxyzu, (size_t)c->n);
  if (Bevol) cudaMemcpyAsync(Bevol, c->Bevol, b4, cudaMemcpyDeviceToHost, c->stream);
  return check_cuda(c);
}

int ph_build_tree(ph_ctx *c, double *xyzh, int32_t *inodeparts, int64_t *ncells) {
  if (!c || c->n <= 0) return PH_ERR_ARG;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  reset_timers(c);
  cudaEventRecord(c->ev[0], c->stream);
  int r = build_tree(c);
  if (r) return r;
  cudaEventRecord(c->ev[1], c->stream);
  cudaEventSynchronize(c->ev[1]);
  add_elapsed(c, 0, c->ev[0], c->ev[1]);
  if (xyzh) cudaMemcpyAsync(xyzh, c->xyzh, sizeof(double) * 4 * (size_t)c->n, cudaMemcpyDeviceToHost, c->stream);
  if (inodeparts) {
    std::vector<int> tmp((size_t)c->ntree);
    cudaMemcpyAsync(tmp.data(), c->perm, sizeof(int) * (size_t)c->ntree, cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    for (int64_t k = 0; k < c->ntree; ++k) inodeparts[k] = tmp[(size_t)k] + 1;
  }
  if (ncells && (r = ref_ncells(c, ncells)) != 0) return r;
  return check_cuda(c);
}

int ph_revtree(ph_ctx *c, const double *xyzh) {
  if (!c || !xyzh) return PH_ERR_ARG;
  if (!c->have_tree) return PH_ERR_STATE;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  cudaMemcpyAsync(c->xyzh, xyzh, sizeof(double) * 4 * (size_t)c->n, cudaMemcpyHostToDevice, c->stream);
  reset_timers(c);
  cudaEventRecord(c->ev[0], c->stream);
  const int r = revtree(c);
  if (r) return r;
  cudaEventRecord(c->ev[1], c->stream);
  cudaEventSynchronize(c->ev[1]);
  add_elapsed(c, 0, c->ev[0], c->ev[1]);  // the refit's device time in the tree slot
  return check_cuda(c);
}

int ph_get_nodes(ph_ctx *c, int64_t *nnodes, int32_t *inoderange, double *xcen, double *size, double *hmax,
                 double *mass, int32_t *isleaf) {
  if (!c || !nnodes) return PH_ERR_ARG;
  const int r = get_nodes(c, nnodes, inoderange, xcen, size, hmax, mass, isleaf);
  if (r) return r;
  return check_cuda(c);
}

int ph_density(ph_ctx *c, int icall, double *xyzh, float *gradh, float *divcurlv, float *divcurlB,
               int32_t *nneigh, uint64_t *neighhash, ph_neigh_stats *stats) {
  if (!c) return PH_ERR_ARG;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  c->want_diag = gradh || divcurlv || divcurlB || nneigh || neighhash;
  int r = density(c, icall);
  c->want_diag = false;
  if (r) return r;
  const size_t n = (size_t)c->n;
  if (xyzh) cudaMemcpyAsync(xyzh, c->xyzh, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, c->stream);
  if (gradh) cudaMemcpyAsync(gradh, c->gradh, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, c->stream);
  if (divcurlv && copy_divcurlv_d2h(c, divcurlv, n) != 0) return PH_ERR_CUDA;
  if (divcurlB) cudaMemcpyAsync(divcurlB, c->divcurlB, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, c->stream);
  if (nneigh) cudaMemcpyAsync(nneigh, c->nneigh, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, c->stream);
  if (neighhash) cudaMemcpyAsync(neighhash, c->nhash, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, c->stream);
  if (stats) {
    unsigned long long s[8];
    double red[8];
    cudaMemcpyAsync(s, c->stats, sizeof(s), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(red, c->red, sizeof(red), cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    stats->nneightry = (int64_t)s[0]; stats->nneighact = (int64_t)s[1];
    stats->maxneightry = (int64_t)s[2]; stats->maxneighact = (int64_t)s[3];
    stats->ncalc = (int64_t)s[4]; stats->np = (int64_t)s[5]; stats->ncalls_neigh = (int64_t)s[6];
    if ((r = ref_ncells(c, &stats->ncells)) != 0) return r;
    stats->maxlevel = c->maxlevel; stats->minlevel = c->minlevel;
    stats->rhomax = red[2];
  }
  return check_cuda(c);
}

int64_t ph_kernel_launches(ph_ctx *c) { return c ? c->launches : 0; }

int ph_last_timings(ph_ctx *c, double *ms8) {
  if (!c || !ms8) return PH_ERR_ARG;
  for (int k = 0; k < 8; ++k) ms8[k] = c->last_ms[k];
  return 0;
}

}  // extern "C"
