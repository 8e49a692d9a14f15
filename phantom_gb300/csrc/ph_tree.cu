// kd-tree build on the GPU (K1/K2): construct_root_node, construct_node and
// sort_particles_in_cell of kdtree.F90:117-1001, restated for sm_103a.
//
// Layout: the tree-order copies tx/ty/tz/th/perm play the role of the
// reference's treecache/inodeparts (kdtree.F90:429-456). Nodes larger than
// SMALL particles are built level by level with multi-block kernels; each node
// of at most SMALL particles is then built, with its whole subtree, by one warp
// (depth-first, like the reference's per-thread subtree build, kdtree.F90:243-293).
//
// Parity notes: the two-pointer partition of
// sort_particles_in_cell is reproduced exactly by pairing the k-th
// misplaced element of the left region (left to right) with the k-th
// misplaced element of the right region (right to left). Centre-of-mass sums of
// nodes of at most SMALL particles are accumulated sequentially in particle
// order, as the serial reference does; for larger nodes they are blocked sums
// in a fixed order (last-ulp differences; the partition only changes if a
// coordinate lies within that rounding gap of the pivot).
#include <cstdio>

#include "ph_internal.h"

namespace ph {

// ------------------------------------------------------------------ root
// construct_root_node kdtree.F90:385-401: periodic wrap (boundary.f90:123-160),
// NaN check and alive flags.
__global__ void k_root_wrap(Params p, double *__restrict__ xyzh, int n, int *__restrict__ alive,
                            int *err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *x = xyzh + 4 * (size_t)i;
  bool a = !(x[3] < TINY_D);
  alive[i] = a ? 1 : 0;
  if (!a) return;
  if (p.periodic) {
    if (x[0] < p.xmin) x[0] = dadd(x[0], p.dxbound); else if (x[0] > p.xmax) x[0] = dsub(x[0], p.dxbound);
    if (x[1] < p.ymin) x[1] = dadd(x[1], p.dybound); else if (x[1] > p.ymax) x[1] = dsub(x[1], p.dybound);
    if (x[2] < p.zmin) x[2] = dadd(x[2], p.dzbound); else if (x[2] > p.zmax) x[2] = dsub(x[2], p.dzbound);
  }
  if (isnan(x[0]) || isnan(x[1]) || isnan(x[2])) set_error(err, PH_ERR_NAN_POS);
}

// scatter live particles to tree order (kdtree.F90:429-456)
__global__ void k_root_fill(const double *__restrict__ xyzh, int n, const int *__restrict__ alive,
                            const int *__restrict__ pos, double *tx, double *ty, double *tz, double *th,
                            int *perm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !alive[i]) return;
  int k = pos[i];
  const double *x = xyzh + 4 * (size_t)i;
  tx[k] = x[0]; ty[k] = x[1]; tz[k] = x[2]; th[k] = x[3];
  perm[k] = i;
}

// bounding box of the tree-order range [0,n) -> part[6*block]
__global__ void k_bbox_partial(const double *tx, const double *ty, const double *tz, int n, double *part) {
  __shared__ double s[6][8];
  double mn[3] = {HUGE_D, HUGE_D, HUGE_D}, mx[3] = {-HUGE_D, -HUGE_D, -HUGE_D};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v[3] = {tx[i], ty[i], tz[i]};
    for (int k = 0; k < 3; ++k) { mn[k] = fmin(mn[k], v[k]); mx[k] = fmax(mx[k], v[k]); }
  }
  for (int k = 0; k < 3; ++k) { mn[k] = warp_min(mn[k]); mx[k] = warp_max(mx[k]); }
  int w = threadIdx.x >> 5;
  if (lane_id() == 0) for (int k = 0; k < 3; ++k) { s[k][w] = mn[k]; s[3 + k][w] = mx[k]; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int nw = blockDim.x >> 5;
    for (int k = 0; k < 3; ++k) {
      double a = s[k][0], b = s[3 + k][0];
      for (int q = 1; q < nw; ++q) { a = fmin(a, s[k][q]); b = fmax(b, s[3 + k][q]); }
      part[6 * blockIdx.x + k] = a; part[6 * blockIdx.x + 3 + k] = b;
    }
  }
}

// root node record + level list seed
__global__ void k_root_node(const double *part, int nparts, int n, Node *nodes, int *lvl, double *lvl_bb,
                            int *small_list, double *small_bb, int *counters) {
  double bb[6];
  for (int k = 0; k < 3; ++k) { bb[k] = part[k]; bb[3 + k] = part[3 + k]; }
  for (int q = 1; q < nparts; ++q)
    for (int k = 0; k < 3; ++k) { bb[k] = fmin(bb[k], part[6 * q + k]); bb[3 + k] = fmax(bb[3 + k], part[6 * q + 3 + k]); }
  Node r{};
  r.left = -1; r.right = -1; r.start = 0; r.count = n; r.parent = -1; r.level = 0;
  nodes[0] = r;
  if (n > SMALL) {
    lvl[0] = 0;
    for (int k = 0; k < 6; ++k) lvl_bb[k] = bb[k];
    counters[0] = 1;
  } else {
    small_list[0] = 0;
    for (int k = 0; k < 6; ++k) small_bb[k] = bb[k];
    counters[1] = 1;
  }
}

// ------------------------------------------------------------------ large-node levels
// chunk table: cbase[k] = sum_{q<k} ceil(count_q / CHUNK)
__global__ void k_chunk_table(const int *lvl, int nb, const Node *nodes, int *cbase) {
  if (threadIdx.x != 0) return;
  int acc = 0;
  for (int k = 0; k < nb; ++k) {
    cbase[k] = acc;
    acc += (nodes[lvl[k]].count + CHUNK - 1) / CHUNK;
  }
  cbase[nb] = acc;
}

__device__ __forceinline__ int find_chunk_node(const int *cbase, int nb, int c) {
  int lo = 0, hi = nb;  // cbase[lo] <= c < cbase[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (cbase[mid] <= c) lo = mid; else hi = mid;
  }
  return lo;
}

template <int NV>
__device__ __forceinline__ void block_sum_fixed(double (&v)[NV], double (*s)[NV]) {
  // deterministic tree reduction over 256 threads
  int t = threadIdx.x;
  for (int k = 0; k < NV; ++k) s[t][k] = v[k];
  __syncthreads();
  for (int stride = 128; stride > 0; stride >>= 1) {
    if (t < stride) for (int k = 0; k < NV; ++k) s[t][k] = s[t][k] + s[t + stride][k];
    __syncthreads();
  }
  for (int k = 0; k < NV; ++k) v[k] = s[0][k];
  __syncthreads();
}

// kdtree.F90:639-651 sums of fac*x, mass and max h over each chunk
__global__ void __launch_bounds__(256) k_big_props1(Params p, const int *lvl, int nb, const int *cbase,
                                                    const Node *nodes, const double *tx, const double *ty,
                                                    const double *tz, const double *th, double *part) {
  __shared__ double s[256][5];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  double pm = p.massoftype, dfac = (pm > 0.0) ? 1.0 / pm : 1.0, fac = pm * dfac;
  double v[5] = {0, 0, 0, 0, 0};
  for (int i = b + threadIdx.x; i < e; i += 256) {
    v[0] = dadd(v[0], dmul(fac, tx[i])); v[1] = dadd(v[1], dmul(fac, ty[i]));
    v[2] = dadd(v[2], dmul(fac, tz[i])); v[3] = dadd(v[3], pm); v[4] = fmax(v[4], th[i]);
  }
  double hm = v[4];
  v[4] = 0.0;
  block_sum_fixed<5>(v, s);
  __shared__ double smax[8];
  hm = warp_max(hm);
  if (lane_id() == 0) smax[threadIdx.x >> 5] = hm;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < 8; ++q) hm = fmax(hm, smax[q]);
    double *o = part + 8 * (size_t)c;
    o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; o[3] = v[3]; o[4] = hm;
  }
}

// kdtree.F90:669-675 centre of mass, node mass, hmax
__global__ void k_big_fin1(Params p, const int *lvl, int nb, const int *cbase, Node *nodes, double *nmass,
                           const double *part) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  double pm = p.massoftype, dfac = (pm > 0.0) ? 1.0 / pm : 1.0;
  double sx = 0, sy = 0, sz = 0, sm = 0, hm = 0;
  for (int c = cbase[k]; c < cbase[k + 1]; ++c) {
    const double *o = part + 8 * (size_t)c;
    sx = sx + o[0]; sy = sy + o[1]; sz = sz + o[2]; sm = sm + o[3]; hm = fmax(hm, o[4]);
  }
  Node &nd = nodes[lvl[k]];
  double d = sm * dfac;
  if (sm > 0.0) { sx = sx / d; sy = sy / d; sz = sz / d; }
  nd.x = sx; nd.y = sy; nd.z = sz; nd.hmax = hm;
  nmass[lvl[k]] = sm;
}

// kdtree.F90:734-752 r2max and quadrupoles
__global__ void __launch_bounds__(256) k_big_props2(Params p, const int *lvl, int nb, const int *cbase,
                                                    const Node *nodes, const double *tx, const double *ty,
                                                    const double *tz, double *part) {
  __shared__ double s[256][6];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  double pm = p.massoftype;
  double q[6] = {0, 0, 0, 0, 0, 0}, r2m = 0.0;
  for (int i = b + threadIdx.x; i < e; i += 256) {
    double dx = tx[i] - nd.x, dy = ty[i] - nd.y, dz = tz[i] - nd.z;
    double dr2 = r2_exact(dx, dy, dz);
    r2m = fmax(r2m, dr2);
    if (p.gravity) {
      q[0] = q[0] + pm * (dx * dx); q[1] = q[1] + pm * (dx * dy); q[2] = q[2] + pm * (dx * dz);
      q[3] = q[3] + pm * (dy * dy); q[4] = q[4] + pm * (dy * dz); q[5] = q[5] + pm * (dz * dz);
    }
  }
  if (p.gravity) block_sum_fixed<6>(q, s);
  __shared__ double smax[8];
  r2m = warp_max(r2m);
  if (lane_id() == 0) smax[threadIdx.x >> 5] = r2m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) r2m = fmax(r2m, smax[w]);
    double *o = part + 8 * (size_t)c;
    o[0] = r2m;
    for (int w = 0; w < 6; ++w) o[1 + w] = q[w];
  }
}

// kdtree.F90:780-816 size, quads, split axis and pivot
__global__ void k_big_fin2(Params p, const int *lvl, int nb, const int *cbase, Node *nodes, double *nquads,
                           const double *part, const double *lvl_bb, int *misc, double *pivot) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  double r2m = 0.0, q[6] = {0, 0, 0, 0, 0, 0};
  for (int c = cbase[k]; c < cbase[k + 1]; ++c) {
    const double *o = part + 8 * (size_t)c;
    r2m = fmax(r2m, o[0]);
    for (int w = 0; w < 6; ++w) q[w] = q[w] + o[1 + w];
  }
  int id = lvl[k];
  Node &nd = nodes[id];
  nd.size = sqrt(r2m) + EPS_D;
  if (p.gravity) for (int w = 0; w < 6; ++w) nquads[6 * (size_t)id + w] = q[w];
  const double *bb = lvl_bb + 6 * (size_t)k;
  double ext[3] = {bb[3] - bb[0], bb[4] - bb[1], bb[5] - bb[2]};
  int ax = 0;
  if (ext[1] > ext[ax]) ax = 1;
  if (ext[2] > ext[ax]) ax = 2;
  misc[4 * k + 0] = ax;
  pivot[k] = ax == 0 ? nd.x : (ax == 1 ? nd.y : nd.z);
}

__device__ __forceinline__ double coord(const double *tx, const double *ty, const double *tz, int ax, int i) {
  return ax == 0 ? tx[i] : (ax == 1 ? ty[i] : tz[i]);
}

// count x(axis) <= pivot per chunk (kdtree.F90:954-955)
__global__ void __launch_bounds__(256) k_big_count(const int *lvl, int nb, const int *cbase, const Node *nodes,
                                                   const double *tx, const double *ty, const double *tz,
                                                   const int *misc, const double *pivot, int *cnt) {
  __shared__ int s[8];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  int ax = misc[4 * k];
  double pv = pivot[k];
  int m = 0;
  for (int i = b + threadIdx.x; i < e; i += 256) m += (coord(tx, ty, tz, ax, i) <= pv) ? 1 : 0;
  m = warp_sum_int(m);
  if (lane_id() == 0) s[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < 8; ++w) t += s[w];
    cnt[c] = t;
  }
}

__global__ void k_big_fin3(const int *lvl, int nb, const int *cbase, const Node *nodes, const int *cnt,
                           int *misc) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  int nl = 0;
  for (int c = cbase[k]; c < cbase[k + 1]; ++c) nl += cnt[c];
  int n = nodes[lvl[k]].count;
  int noswap = 0;
  if (nl == n || nl == 0) { nl = n / 2; noswap = 1; }  // kdtree.F90:856-865
  misc[4 * k + 1] = nl;
  misc[4 * k + 2] = noswap;
}

// block-wide exclusive scan of per-thread counts (256 threads)
__device__ __forceinline__ int block_excl_scan(int v, int *s, int &total) {
  int lane = lane_id(), w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int q = 0; q < 8; ++q) { int t = s[q]; s[q] = acc; acc += t; }
    s[8] = acc;
  }
  __syncthreads();
  int r = s[w] + x - v;
  total = s[8];
  __syncthreads();
  return r;
}

// per-chunk numbers of misplaced elements: bigs left of the boundary, smalls right of it
__global__ void __launch_bounds__(256) k_big_rank(const int *lvl, int nb, const int *cbase, const Node *nodes,
                                                  const double *tx, const double *ty, const double *tz,
                                                  const int *misc, const double *pivot, int *bl, int *sr) {
  __shared__ int s[16];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  if (misc[4 * k + 2]) { if (threadIdx.x == 0) { bl[c] = 0; sr[c] = 0; } return; }
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  int ax = misc[4 * k], bnd = nd.start + misc[4 * k + 1];
  double pv = pivot[k];
  int nb_ = 0, ns_ = 0;
  for (int i = b + threadIdx.x; i < e; i += 256) {
    bool small = coord(tx, ty, tz, ax, i) <= pv;
    if (i < bnd) nb_ += small ? 0 : 1; else ns_ += small ? 1 : 0;
  }
  nb_ = warp_sum_int(nb_); ns_ = warp_sum_int(ns_);
  if (lane_id() == 0) { s[threadIdx.x >> 5] = nb_; s[8 + (threadIdx.x >> 5)] = ns_; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int a = 0, d = 0;
    for (int w = 0; w < 8; ++w) { a += s[w]; d += s[8 + w]; }
    bl[c] = a; sr[c] = d;
  }
}

// chunk bases of the ranks: bigs ranked left->right, smalls right->left
__global__ void k_big_fin4(const int *lvl, int nb, const int *cbase, int *bl, int *sr) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  int acc = 0;
  for (int c = cbase[k]; c < cbase[k + 1]; ++c) { int t = bl[c]; bl[c] = acc; acc += t; }
  acc = 0;
  for (int c = cbase[k + 1] - 1; c >= cbase[k]; --c) { int t = sr[c]; sr[c] = acc; acc += t; }
}

// record the positions of the right-region smalls by rank (from the right)
__global__ void __launch_bounds__(256) k_big_pairs(const int *lvl, int nb, const int *cbase, const Node *nodes,
                                                   const double *tx, const double *ty, const double *tz,
                                                   const int *misc, const double *pivot, const int *sr,
                                                   int *pairpos) {
  __shared__ int s[16];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  if (misc[4 * k + 2]) return;
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  int ax = misc[4 * k], bnd = nd.start + misc[4 * k + 1];
  double pv = pivot[k];
  // each thread owns 8 consecutive elements (thread order == position order)
  int i0 = b + threadIdx.x * 8;
  int flags = 0, cntl = 0;
  for (int q = 0; q < 8; ++q) {
    int i = i0 + q;
    bool f = (i < e) && (i >= bnd) && (coord(tx, ty, tz, ax, i) <= pv);
    if (f) { flags |= 1 << q; ++cntl; }
  }
  int total;
  int pre = block_excl_scan(cntl, s, total);
  // rank from the right within the chunk = number of flagged elements after me
  int after = total - pre - cntl;
  int base = sr[c];
  for (int q = 7; q >= 0; --q) {
    if (flags & (1 << q)) {
      pairpos[nd.start + base + after] = i0 + q;
      ++after;
    }
  }
}

__device__ __forceinline__ void swap_rows(double *tx, double *ty, double *tz, double *th, int *perm, int a, int b) {
  double t;
  t = tx[a]; tx[a] = tx[b]; tx[b] = t;
  t = ty[a]; ty[a] = ty[b]; ty[b] = t;
  t = tz[a]; tz[a] = tz[b]; tz[b] = t;
  t = th[a]; th[a] = th[b]; th[b] = t;
  int u = perm[a]; perm[a] = perm[b]; perm[b] = u;
}

// swap each left-region big with its paired right-region small (kdtree.F90:969-977)
__global__ void __launch_bounds__(256) k_big_swap(const int *lvl, int nb, const int *cbase, const Node *nodes,
                                                  double *tx, double *ty, double *tz, double *th, int *perm,
                                                  const int *misc, const double *pivot, const int *bl,
                                                  const int *pairpos) {
  __shared__ int s[16];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  if (misc[4 * k + 2]) return;
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  int ax = misc[4 * k], bnd = nd.start + misc[4 * k + 1];
  double pv = pivot[k];
  int i0 = b + threadIdx.x * 8;
  int flags = 0, cntl = 0;
  for (int q = 0; q < 8; ++q) {
    int i = i0 + q;
    bool f = (i < e) && (i < bnd) && !(coord(tx, ty, tz, ax, i) <= pv);
    if (f) { flags |= 1 << q; ++cntl; }
  }
  int total;
  int pre = block_excl_scan(cntl, s, total);
  int r = bl[c] + pre;
  for (int q = 0; q < 8; ++q) {
    if (flags & (1 << q)) {
      int partner = pairpos[nd.start + r];
      swap_rows(tx, ty, tz, th, perm, i0 + q, partner);
      ++r;
    }
  }
}

// child bounding boxes (kdtree.F90:868-896): partial min/max per chunk and side
__global__ void __launch_bounds__(256) k_big_cbounds(const int *lvl, int nb, const int *cbase, const Node *nodes,
                                                     const double *tx, const double *ty, const double *tz,
                                                     const int *misc, double *part) {
  __shared__ double s[12][8];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  int bnd = nd.start + misc[4 * k + 1];
  double v[12];
  for (int q = 0; q < 2; ++q)
    for (int a = 0; a < 3; ++a) { v[6 * q + a] = HUGE_D; v[6 * q + 3 + a] = -HUGE_D; }
  for (int i = b + threadIdx.x; i < e; i += 256) {
    int q = (i < bnd) ? 0 : 1;
    double x[3] = {tx[i], ty[i], tz[i]};
    for (int a = 0; a < 3; ++a) { v[6 * q + a] = fmin(v[6 * q + a], x[a]); v[6 * q + 3 + a] = fmax(v[6 * q + 3 + a], x[a]); }
  }
  for (int q = 0; q < 2; ++q)
    for (int a = 0; a < 3; ++a) { v[6 * q + a] = warp_min(v[6 * q + a]); v[6 * q + 3 + a] = warp_max(v[6 * q + 3 + a]); }
  int w = threadIdx.x >> 5;
  if (lane_id() == 0) for (int t = 0; t < 12; ++t) s[t][w] = v[t];
  __syncthreads();
  if (threadIdx.x == 0) {
    double *o = part + 16 * (size_t)c;
    for (int t = 0; t < 12; ++t) {
      double r = s[t][0];
      bool ismin = (t % 6) < 3;
      for (int q = 1; q < 8; ++q) r = ismin ? fmin(r, s[t][q]) : fmax(r, s[t][q]);
      o[t] = r;
    }
  }
}

// children creation, next-level lists
__global__ void k_big_fin5(const int *lvl, int nb, const int *cbase, Node *nodes, const int *misc,
                           const double *part, int child_base, int *lvl_next, double *bb_next,
                           int *small_list, double *small_bb, int *counters, int small_cap, int *err) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  double bb[12];
  for (int q = 0; q < 2; ++q)
    for (int a = 0; a < 3; ++a) { bb[6 * q + a] = HUGE_D; bb[6 * q + 3 + a] = -HUGE_D; }
  for (int c = cbase[k]; c < cbase[k + 1]; ++c) {
    const double *o = part + 16 * (size_t)c;
    for (int t = 0; t < 12; ++t) bb[t] = ((t % 6) < 3) ? fmin(bb[t], o[t]) : fmax(bb[t], o[t]);
  }
  int id = lvl[k];
  Node &nd = nodes[id];
  int nl = misc[4 * k + 1];
  int il = child_base + 2 * k, ir = il + 1;
  nd.left = il; nd.right = ir;
  for (int q = 0; q < 2; ++q) {
    Node ch{};
    ch.left = -1; ch.right = -1; ch.parent = id; ch.level = nd.level + 1;
    ch.start = q == 0 ? nd.start : nd.start + nl;
    ch.count = q == 0 ? nl : nd.count - nl;
    int cid = q == 0 ? il : ir;
    nodes[cid] = ch;
    if (ch.count > SMALL) {
      int slot = atomicAdd(&counters[0], 1);
      lvl_next[slot] = cid;
      for (int t = 0; t < 6; ++t) bb_next[6 * (size_t)slot + t] = bb[6 * q + t];
    } else {
      int slot = atomicAdd(&counters[1], 1);
      if (slot >= small_cap) { set_error(err, PH_ERR_TREE); continue; }
      small_list[slot] = cid;
      for (int t = 0; t < 6; ++t) small_bb[6 * (size_t)slot + t] = bb[6 * q + t];
    }
  }
}

// ------------------------------------------------------------------ small subtrees
constexpr int SUB_WARPS = 1;
constexpr int SUB_STACK = 64;

struct SubEntry {
  int id, start, count, level, parent, pad;
  double bb[6];
};

// One warp builds the complete subtree of a node with <= SMALL particles,
// depth first (push left then right, pop right first; kdtree.F90:264-290).
__global__ void __launch_bounds__(32 * SUB_WARPS) k_subtree(Params p, const int *small_list, int nsmall,
                                                           const double *small_bb, Node *nodes, double *nmass,
                                                           double *nquads, double *tx, double *ty, double *tz,
                                                           double *th, int *perm, int subbase, int *leaf_at,
                                                           int *lvlstat, int *err) {
  __shared__ int sbig[SUB_WARPS][SMALL];
  __shared__ int ssml[SUB_WARPS][SMALL];
  __shared__ SubEntry sstack[SUB_WARPS][SUB_STACK];
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int gw = blockIdx.x * SUB_WARPS + w;
  if (gw >= nsmall) return;
  const unsigned FULL = 0xffffffffu;
  int *bigs = sbig[w], *smls = ssml[w];
  SubEntry *stk = sstack[w];
  const int rootid = small_list[gw];
  const Node rn = nodes[rootid];
  int idbase = subbase + 2 * rn.start, nextk = 0;
  int top = 0;
  if (lane == 0) {
    SubEntry e;
    e.id = rootid; e.start = rn.start; e.count = rn.count; e.level = rn.level; e.parent = rn.parent;
    for (int t = 0; t < 6; ++t) e.bb[t] = small_bb[6 * (size_t)gw + t];
    stk[0] = e;
  }
  top = 1;
  __syncwarp();
  const double pm = p.massoftype, dfac = (pm > 0.0) ? 1.0 / pm : 1.0, fac = pm * dfac;
  while (top > 0) {
    --top;
    SubEntry e = stk[top];
    __syncwarp();
    const int s = e.start, n = e.count;
    // centre of mass: sequential in particle order (kdtree.F90:654-666)
    double sx = 0, sy = 0, sz = 0, sm = 0, hm = 0;
    for (int base = s; base < s + n; base += 32) {
      int i = base + lane;
      bool v = i < s + n;
      double x = v ? tx[i] : 0.0, y = v ? ty[i] : 0.0, z = v ? tz[i] : 0.0, h = v ? th[i] : 0.0;
      hm = fmax(hm, h);
      int cnt = min(32, s + n - base);
      for (int q = 0; q < cnt; ++q) {
        double xq = __shfl_sync(FULL, x, q), yq = __shfl_sync(FULL, y, q), zq = __shfl_sync(FULL, z, q);
        sx = dadd(sx, dmul(fac, xq)); sy = dadd(sy, dmul(fac, yq)); sz = dadd(sz, dmul(fac, zq));
        sm = dadd(sm, pm);
      }
    }
    hm = warp_max(hm);
    double d = sm * dfac;
    if (sm > 0.0) { sx = ddiv(sx, d); sy = ddiv(sy, d); sz = ddiv(sz, d); }
    sx = __shfl_sync(FULL, sx, 0); sy = __shfl_sync(FULL, sy, 0); sz = __shfl_sync(FULL, sz, 0);
    sm = __shfl_sync(FULL, sm, 0);
    // size and quadrupoles (kdtree.F90:734-752); quads summed sequentially
    double r2m = 0.0, q6[6] = {0, 0, 0, 0, 0, 0};
    for (int base = s; base < s + n; base += 32) {
      int i = base + lane;
      bool v = i < s + n;
      double dx = v ? tx[i] - sx : 0.0, dy = v ? ty[i] - sy : 0.0, dz = v ? tz[i] - sz : 0.0;
      if (v) r2m = fmax(r2m, r2_exact(dx, dy, dz));
      if (p.gravity) {
        int cnt = min(32, s + n - base);
        for (int q = 0; q < cnt; ++q) {
          double a = __shfl_sync(FULL, dx, q), b = __shfl_sync(FULL, dy, q), cz = __shfl_sync(FULL, dz, q);
          q6[0] = dadd(q6[0], dmul(pm, dmul(a, a))); q6[1] = dadd(q6[1], dmul(pm, dmul(a, b)));
          q6[2] = dadd(q6[2], dmul(pm, dmul(a, cz))); q6[3] = dadd(q6[3], dmul(pm, dmul(b, b)));
          q6[4] = dadd(q6[4], dmul(pm, dmul(b, cz))); q6[5] = dadd(q6[5], dmul(pm, dmul(cz, cz)));
        }
      }
    }
    r2m = warp_max(r2m);
    Node nd{};
    nd.x = sx; nd.y = sy; nd.z = sz; nd.size = sqrt(r2m) + EPS_D; nd.hmax = hm;
    nd.start = s; nd.count = n; nd.level = e.level;
    nd.parent = e.parent;
    bool split = n > MINPART;
    int il = -1, ir = -1, nl = 0;
    double cbb[12];
    if (split) {
      double ext[3] = {e.bb[3] - e.bb[0], e.bb[4] - e.bb[1], e.bb[5] - e.bb[2]};
      int ax = 0;
      if (ext[1] > ext[ax]) ax = 1;
      if (ext[2] > ext[ax]) ax = 2;
      double pv = ax == 0 ? sx : (ax == 1 ? sy : sz);
      const double *cx = ax == 0 ? tx : (ax == 1 ? ty : tz);
      for (int base = s; base < s + n; base += 32) {
        int i = base + lane;
        bool f = (i < s + n) && (cx[i] <= pv);
        nl += __popc(__ballot_sync(FULL, f));
      }
      bool noswap = (nl == n || nl == 0);
      if (noswap) nl = n / 2;  // kdtree.F90:856-865
      if (!noswap) {
        int bnd = s + nl, m = 0;
        for (int base = s; base < bnd; base += 32) {  // bigs left of bnd, ascending
          int i = base + lane;
          bool f = (i < bnd) && !(cx[i] <= pv);
          unsigned bal = __ballot_sync(FULL, f);
          if (f) bigs[m + __popc(bal & ((1u << lane) - 1))] = i;
          m += __popc(bal);
        }
        int m2 = 0;
        for (int tp = s + n - 1; tp >= bnd; tp -= 32) {  // smalls right of bnd, descending
          int i = tp - lane;
          bool f = (i >= bnd) && (cx[i] <= pv);
          unsigned bal = __ballot_sync(FULL, f);
          if (f) smls[m2 + __popc(bal & ((1u << lane) - 1))] = i;
          m2 += __popc(bal);
        }
        if (m != m2) { if (lane == 0) set_error(err, PH_ERR_TREE); }
        __syncwarp();
        for (int q = lane; q < m; q += 32) swap_rows(tx, ty, tz, th, perm, bigs[q], smls[q]);
        __syncwarp();
      }
      // child bounds
      for (int t = 0; t < 6; ++t) { cbb[t] = (t < 3) ? HUGE_D : -HUGE_D; cbb[6 + t] = (t < 3) ? HUGE_D : -HUGE_D; }
      for (int base = s; base < s + n; base += 32) {
        int i = base + lane;
        if (i < s + n) {
          int q = (i < s + nl) ? 0 : 1;
          double x[3] = {tx[i], ty[i], tz[i]};
          for (int a = 0; a < 3; ++a) { cbb[6 * q + a] = fmin(cbb[6 * q + a], x[a]); cbb[6 * q + 3 + a] = fmax(cbb[6 * q + 3 + a], x[a]); }
        }
      }
      for (int t = 0; t < 12; ++t) cbb[t] = ((t % 6) < 3) ? warp_min(cbb[t]) : warp_max(cbb[t]);
      il = idbase + nextk; ir = il + 1; nextk += 2;
      if (nextk > 2 * rn.count) { if (lane == 0) set_error(err, PH_ERR_TREE); split = false; }
    }
    nd.left = split ? il : -1; nd.right = split ? ir : -1;
    if (lane == 0) {
      nodes[e.id] = nd;
      nmass[e.id] = sm;
      if (p.gravity) for (int t = 0; t < 6; ++t) nquads[6 * (size_t)e.id + t] = q6[t];
      if (!split) {
        leaf_at[s] = e.id;
        atomicMax(&lvlstat[0], e.level);
        atomicMin(&lvlstat[1], e.level);
      } else {
        if (top + 2 > SUB_STACK) { set_error(err, PH_ERR_STACK); }
        else {
          SubEntry a, b;
          a.id = il; a.start = s; a.count = nl; a.level = e.level + 1; a.parent = e.id;
          b.id = ir; b.start = s + nl; b.count = n - nl; b.level = e.level + 1; b.parent = e.id;
          for (int t = 0; t < 6; ++t) { a.bb[t] = cbb[t]; b.bb[t] = cbb[6 + t]; }
          stk[top] = a; stk[top + 1] = b;
        }
      }
    }
    if (split) top += 2;
    if (top > SUB_STACK) top = 0;  // error already flagged
    __syncwarp();
  }
}

__global__ void k_fill_int(int *a, int n, int v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}
__global__ void k_flag_leaves(const int *leaf_at, int n, int *flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = leaf_at[i] >= 0 ? 1 : 0;
}
__global__ void k_compact_leaves(const int *leaf_at, const int *pos, int n, int *leaves) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && leaf_at[i] >= 0) leaves[pos[i]] = leaf_at[i];
}
__global__ void k_iperm(const int *perm, int n, int *iperm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) iperm[perm[i]] = i;
}

static inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }

// maketree (kdtree.F90:117-314) driver
int build_tree(ph_ctx *c) {
  cudaStream_t st = c->stream;
  const int n = (int)c->n;
  const Params p = c->dp;
  k_root_wrap<<<nblk(n, 256), 256, 0, st>>>(p, c->xyzh, n, c->alive, c->d_err);
  scan_int(c, c->alive, c->pairpos, n, c->counters + 4);
  int nalive = 0;
  cudaMemcpyAsync(&nalive, c->counters + 4, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  count_launch(c, 1);
  if (nalive <= 0) return PH_ERR_NOPART;
  c->ntree = nalive;
  k_root_fill<<<nblk(n, 256), 256, 0, st>>>(c->xyzh, n, c->alive, c->pairpos, c->tx, c->ty, c->tz, c->th, c->perm);
  int nbb = std::min(nblk(nalive, 256), 1024);
  k_bbox_partial<<<nbb, 256, 0, st>>>(c->tx, c->ty, c->tz, nalive, c->part_d);
  cudaMemsetAsync(c->counters, 0, 4 * sizeof(int), st);
  k_root_node<<<1, 1, 0, st>>>(c->part_d, nbb, nalive, c->nodes, c->lvl_a, c->lvl_bb_a, c->small_list,
                              c->small_bb, c->counters);
  k_fill_int<<<nblk(nalive, 256), 256, 0, st>>>(c->leaf_at, nalive, -1);
  int lvlinit[2] = {0, 1 << 30};
  cudaMemcpyAsync(c->d_maxlevel, lvlinit, 2 * sizeof(int), cudaMemcpyHostToDevice, st);
  count_launch(c, 4);
  int counters[2] = {0, 0};
  cudaMemcpyAsync(counters, c->counters, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  int nb = counters[0];
  int next_id = 1;
  int *lvl = c->lvl_a, *lvl_next = c->lvl_b;
  double *bb = c->lvl_bb_a, *bb_next = c->lvl_bb_b;
  int guard = 0;
  while (nb > 0) {
    if (++guard > 200 || next_id + 2 * nb > c->subbase) return PH_ERR_TREE;
    int maxchunks = nalive / CHUNK + nb + 1;
    if (maxchunks > c->chunk_cap) return PH_ERR_TREE;
    int *cb = c->cbase;
    int *cnt = c->part_i, *bl = c->part_i + c->chunk_cap, *sr = c->part_i + 2 * c->chunk_cap;
    k_chunk_table<<<1, 32, 0, st>>>(lvl, nb, c->nodes, cb);
    k_big_props1<<<maxchunks, 256, 0, st>>>(p, lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->th, c->part_d);
    k_big_fin1<<<nblk(nb, 64), 64, 0, st>>>(p, lvl, nb, cb, c->nodes, c->nmass, c->part_d);
    k_big_props2<<<maxchunks, 256, 0, st>>>(p, lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->part_d);
    k_big_fin2<<<nblk(nb, 64), 64, 0, st>>>(p, lvl, nb, cb, c->nodes, c->nquads, c->part_d, bb, c->lvl_misc,
                                            c->lvl_pivot);
    k_big_count<<<maxchunks, 256, 0, st>>>(lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->lvl_misc, c->lvl_pivot, cnt);
    k_big_fin3<<<nblk(nb, 64), 64, 0, st>>>(lvl, nb, cb, c->nodes, cnt, c->lvl_misc);
    k_big_rank<<<maxchunks, 256, 0, st>>>(lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->lvl_misc, c->lvl_pivot, bl, sr);
    k_big_fin4<<<nblk(nb, 64), 64, 0, st>>>(lvl, nb, cb, bl, sr);
    k_big_pairs<<<maxchunks, 256, 0, st>>>(lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->lvl_misc, c->lvl_pivot,
                                           sr, c->pairpos);
    k_big_swap<<<maxchunks, 256, 0, st>>>(lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->th, c->perm, c->lvl_misc,
                                          c->lvl_pivot, bl, c->pairpos);
    k_big_cbounds<<<maxchunks, 256, 0, st>>>(lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->lvl_misc, c->part_d);
    cudaMemsetAsync(c->counters, 0, sizeof(int), st);
    k_big_fin5<<<nblk(nb, 64), 64, 0, st>>>(lvl, nb, cb, c->nodes, c->lvl_misc, c->part_d, next_id, lvl_next,
                                            bb_next, c->small_list, c->small_bb, c->counters,
                                            c->lvl_cap * 64, c->d_err);
    count_launch(c, 13);
    next_id += 2 * nb;
    cudaMemcpyAsync(counters, c->counters, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    nb = counters[0];
    std::swap(lvl, lvl_next);
    std::swap(bb, bb_next);
  }
  int nsmall = counters[1];
  if (nsmall > 0) {
    k_subtree<<<nblk(nsmall, SUB_WARPS), 32 * SUB_WARPS, 0, st>>>(
        p, c->small_list, nsmall, c->small_bb, c->nodes, c->nmass, c->nquads, c->tx, c->ty, c->tz, c->th, c->perm,
        c->subbase, c->leaf_at, c->d_maxlevel, c->d_err);
    count_launch(c, 1);
  }
  // leaf list in ascending start order
  k_flag_leaves<<<nblk(nalive, 256), 256, 0, st>>>(c->leaf_at, nalive, c->alive);
  scan_int(c, c->alive, c->pairpos, nalive, c->counters + 4);
  k_compact_leaves<<<nblk(nalive, 256), 256, 0, st>>>(c->leaf_at, c->pairpos, nalive, c->leaves);
  k_iperm<<<nblk(nalive, 256), 256, 0, st>>>(c->perm, nalive, c->iperm);
  count_launch(c, 3);
  int hostv[3];
  cudaMemcpyAsync(hostv, c->counters + 4, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hostv + 1, c->d_maxlevel, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  cudaError_t ce = check_launch(c);
  if (ce != cudaSuccess) return PH_ERR_CUDA;
  int herr = 0;
  cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (herr) return herr;
  c->nleaves = hostv[0];
  c->maxlevel = hostv[1];
  c->minlevel = hostv[2];
  c->root = 0;
  c->have_tree = true;
  c->have_density = c->have_force_lists = false;
  return 0;
}

}  // namespace ph
