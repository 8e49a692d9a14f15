// kd-tree build on the GPU (K1/K2): construct_root_node, construct_node and
// sort_particles_in_cell of kdtree.F90:117-1001, restated for sm_103a.
//
// Layout: the tree-order copies tx/ty/tz/th/perm play the role of the
// reference's treecache/inodeparts (kdtree.F90:429-456), with an FP32 copy of
// the positions (txf) that moves with them. Nodes larger than SMALL particles
// are built level by level with multi-block kernels (chunk partials, then one
// warp per node to combine them); nodes of at most SMALL particles are then
// built generation by generation (k_small_com, k_small_split).
//
// Parity notes: the two-pointer partition of sort_particles_in_cell pairs the
// k-th misplaced element of the left region (left to right) with the k-th
// misplaced element of the right region (right to left); the kernels
// reproduce it by ranking the misplaced elements. Centre-of-mass sums of
// nodes of at most SMALL particles are accumulated sequentially in particle
// order, as the serial reference does; for larger nodes they are blocked sums
// in a fixed order (last-ulp differences; the partition only changes if a
// coordinate lies within that rounding gap of the pivot).
#include <algorithm>
#include <cstdio>

#include <cuda_pipeline.h>

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
// (with the FP32 copy of the position that the build's bounds and the pair
// pre-filters use; it moves with the particle through every swap)
__global__ void k_root_fill(const double *__restrict__ xyzh, int n, const int *__restrict__ alive,
                            const int *__restrict__ pos, double *tx, double *ty, double *tz, double *th,
                            int *perm, float4 *txf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !alive[i]) return;
  int k = pos[i];
  const double *x = xyzh + 4 * (size_t)i;
  tx[k] = x[0]; ty[k] = x[1]; tz[k] = x[2]; th[k] = x[3];
  perm[k] = i;
  txf[k] = make_float4((float)x[0], (float)x[1], (float)x[2], 0.0f);
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

// root node record + level list seed (one block of 256 threads combines the
// bounding-box partials)
__global__ void __launch_bounds__(256) k_root_node(const double *part, int nparts, int n, Node *nodes, int *lvl,
                                                   double *lvl_bb, GenEntry *gen, int *counters) {
  __shared__ double s[6][8];
  double bb[6] = {HUGE_D, HUGE_D, HUGE_D, -HUGE_D, -HUGE_D, -HUGE_D};
  for (int q = threadIdx.x; q < nparts; q += blockDim.x)
    for (int k = 0; k < 3; ++k) { bb[k] = fmin(bb[k], part[6 * q + k]); bb[3 + k] = fmax(bb[3 + k], part[6 * q + 3 + k]); }
  for (int k = 0; k < 3; ++k) { bb[k] = warp_min(bb[k]); bb[3 + k] = warp_max(bb[3 + k]); }
  if (lane_id() == 0) for (int k = 0; k < 6; ++k) s[k][threadIdx.x >> 5] = bb[k];
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
    for (int k = 0; k < 3; ++k) { bb[k] = fmin(bb[k], s[k][w]); bb[3 + k] = fmax(bb[3 + k], s[3 + k][w]); }
  Node r{};
  r.left = -1; r.right = -1; r.start = 0; r.count = n; r.parent = -1; r.level = 0;
  nodes[0] = r;
  if (n > SMALL) {
    lvl[0] = 0;
    for (int k = 0; k < 6; ++k) lvl_bb[k] = bb[k];
    counters[0] = 1;
  } else {
    GenEntry g;
    g.id = 0; g.start = 0; g.count = n; g.level = 0; g.parent = -1; g.pad = 0;
    for (int k = 0; k < 6; ++k) g.bb[k] = bb[k];
    gen[0] = g;
    counters[1] = 1;
  }
}

// ------------------------------------------------------------------ large-node levels
// chunk table: cbase[k] = sum_{q<k} ceil(count_q / CHUNK) (one block of 1024
// threads scans the level's nodes a tile at a time)
__global__ void __launch_bounds__(1024) k_chunk_table(const int *lvl, int nb, const Node *nodes, int *cbase) {
  __shared__ int ws[32];
  __shared__ int carry;
  const int lane = lane_id(), w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < nb; b0 += 1024) {
    const int k = b0 + threadIdx.x;
    const int v = k < nb ? (nodes[lvl[k]].count + CHUNK - 1) / CHUNK : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) { const int y = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += y; }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = ws[lane];
      for (int o = 1; o < 32; o <<= 1) { const int y = __shfl_up_sync(0xffffffffu, t, o); if (lane >= o) t += y; }
      ws[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    const int excl = carry + (w > 0 ? ws[w - 1] : 0) + x - v;
    if (k < nb) cbase[k] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry += ws[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) cbase[nb] = carry;
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

constexpr int PER = CHUNK / 256;  // particles of a chunk per thread
static_assert(CHUNK % 256 == 0, "chunk kernels run 256 threads");

// kdtree.F90:639-651 sums of fac*x, mass and max h over each chunk. Each
// thread sums its particles sequentially; with fac = pm dfac = 1 (one
// particle mass) the products are the coordinates themselves, and the
// thread's mass sum is the sequential sum of its count of equal masses,
// read from the table. hmax is a max over the bit patterns (h > 0 for every
// particle in the tree; a NaN is skipped as fmax would).
__global__ void __launch_bounds__(256) k_big_props1(Params p, const int *lvl, int nb, const int *cbase,
                                                    const Node *nodes, const double *tx, const double *ty,
                                                    const double *tz, const double *th, const double *mtab,
                                                    double *part) {
  __shared__ double s[256][4];
  __shared__ unsigned long long smax[8];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  double pm = p.massoftype, dfac = (pm > 0.0) ? 1.0 / pm : 1.0, fac = pm * dfac;
  double v[4] = {0, 0, 0, 0};
  int cnt = 0;
  unsigned long long hb = 0ull;
  // all of the thread's loads first, then its sums in particle order
  double xs[PER], ys[PER], zs[PER];
  unsigned long long hs[PER];
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int i = b + threadIdx.x + 256 * q;
    if (i < e) {
      xs[q] = tx[i]; ys[q] = ty[i]; zs[q] = tz[i]; hs[q] = (unsigned long long)__double_as_longlong(th[i]);
    }
  }
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    if (b + threadIdx.x + 256 * q < e) {
      if (fac == 1.0) {
        v[0] = dadd(v[0], xs[q]); v[1] = dadd(v[1], ys[q]); v[2] = dadd(v[2], zs[q]);
      } else {
        v[0] = dadd(v[0], dmul(fac, xs[q])); v[1] = dadd(v[1], dmul(fac, ys[q]));
        v[2] = dadd(v[2], dmul(fac, zs[q]));
      }
      if (hs[q] <= 0x7ff0000000000000ull) hb = max(hb, hs[q]);
      ++cnt;
    }
  }
  v[3] = mtab[cnt];
  block_sum_fixed<4>(v, s);
  for (int o = 16; o > 0; o >>= 1) hb = max(hb, __shfl_xor_sync(0xffffffffu, hb, o));
  if (lane_id() == 0) smax[threadIdx.x >> 5] = hb;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < 8; ++q) hb = max(hb, smax[q]);
    double *o = part + 8 * (size_t)c;
    o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; o[3] = v[3]; o[4] = __longlong_as_double((long long)hb);
  }
}

// The level "fin" kernels take one warp per node: lanes stride over the
// node's chunk partials, then a fixed-order butterfly combines the lanes.
constexpr int FIN_WARPS = 4;
__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// kdtree.F90:669-675 centre of mass, node mass, hmax; kdtree.F90:800-816
// split axis (longest bounding-box extent) and pivot (the centre of mass)
__global__ void __launch_bounds__(32 * FIN_WARPS) k_big_fin1(Params p, const int *lvl, int nb, const int *cbase,
                                                             Node *nodes, double *nmass, const double *part,
                                                             const double *lvl_bb, int *misc, double *pivot) {
  const int k = blockIdx.x * FIN_WARPS + (threadIdx.x >> 5), lane = lane_id();
  if (k >= nb) return;
  double pm = p.massoftype, dfac = (pm > 0.0) ? 1.0 / pm : 1.0;
  double sx = 0, sy = 0, sz = 0, sm = 0, hm = 0;
  for (int c = cbase[k] + lane; c < cbase[k + 1]; c += 32) {
    const double *o = part + 8 * (size_t)c;
    sx = sx + o[0]; sy = sy + o[1]; sz = sz + o[2]; sm = sm + o[3]; hm = fmax(hm, o[4]);
  }
  sx = warp_sum_d(sx); sy = warp_sum_d(sy); sz = warp_sum_d(sz); sm = warp_sum_d(sm); hm = warp_max(hm);
  if (lane != 0) return;
  Node &nd = nodes[lvl[k]];
  double d = sm * dfac;
  if (sm > 0.0) { sx = sx / d; sy = sy / d; sz = sz / d; }
  nd.x = sx; nd.y = sy; nd.z = sz; nd.hmax = hm;
  nmass[lvl[k]] = sm;
  if (!misc) return;  // revtree: no split
  const double *bb = lvl_bb + 6 * (size_t)k;
  double ext[3] = {bb[3] - bb[0], bb[4] - bb[1], bb[5] - bb[2]};
  int ax = 0;
  if (ext[1] > ext[ax]) ax = 1;
  if (ext[2] > ext[ax]) ax = 2;
  misc[4 * k + 0] = ax;
  pivot[k] = ax == 0 ? sx : (ax == 1 ? sy : sz);
}

__device__ __forceinline__ float block_max_f(float v, float *s) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane_id() == 0) s[threadIdx.x >> 5] = v;
  __syncthreads();
  float r = s[0];
  for (int q = 1; q < 8; ++q) r = fmaxf(r, s[q]);
  __syncthreads();
  return r;
}

// kdtree.F90:734-752 r2max and quadrupoles, and the count of particles at
// or left of the pivot (kdtree.F90:954-955, compared on order-preserving
// integer keys). Without self-gravity the chunk's r2max is found as in the
// small-node split: FP32 bounds on every r^2, the exact FP64 r^2 only for
// the particles whose upper bound reaches the chunk's largest lower bound.
__global__ void __launch_bounds__(256) k_big_props2(Params p, const int *lvl, int nb, const int *cbase,
                                                    const Node *nodes, const double *tx, const double *ty,
                                                    const double *tz, const float4 *txf, const int *misc,
                                                    const double *pivot, double *part, int *cnt) {
  __shared__ double s[256][6];
  __shared__ float sf[8];
  __shared__ int sc[8];
  __shared__ double smax[8];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  const int ax = misc ? misc[4 * k] : 0;  // revtree (no misc): no left count
  const long long pk = misc ? dkey(pivot[k]) : KEY_HI;
  const double *cx = ax == 0 ? tx : (ax == 1 ? ty : tz);
  double pm = p.massoftype;
  double q[6] = {0, 0, 0, 0, 0, 0}, r2m = 0.0;
  int m = 0;
  if (p.gravity) {
    for (int i = b + threadIdx.x; i < e; i += 256) {
      double dx = tx[i] - nd.x, dy = ty[i] - nd.y, dz = tz[i] - nd.z;
      double dr2 = r2_exact(dx, dy, dz);
      r2m = fmax(r2m, dr2);
      q[0] = q[0] + pm * (dx * dx); q[1] = q[1] + pm * (dx * dy); q[2] = q[2] + pm * (dx * dz);
      q[3] = q[3] + pm * (dy * dy); q[4] = q[4] + pm * (dy * dz); q[5] = q[5] + pm * (dz * dz);
      m += (dkey(cx[i]) <= pk) ? 1 : 0;
    }
    block_sum_fixed<6>(q, s);
  } else {
    const float cxf = (float)nd.x, cyf = (float)nd.y, czf = (float)nd.z;
    const float eps23 = 1.1920929e-7f;
    float4 ts[PER];
    long long ks[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int i = b + threadIdx.x + 256 * q;
      if (i < e) { ts[q] = txf[i]; ks[q] = dkey(cx[i]); }
    }
    float lbmax = 0.0f;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      if (b + threadIdx.x + 256 * q < e) {
        const float4 t = ts[q];
        const float dx = t.x - cxf, dy = t.y - cyf, dz = t.z - czf;
        const float ex = eps23 * (fabsf(t.x) + fabsf(cxf) + fabsf(dx));
        const float ey = eps23 * (fabsf(t.y) + fabsf(cyf) + fabsf(dy));
        const float ez = eps23 * (fabsf(t.z) + fabsf(czf) + fabsf(dz));
        const float bx = fmaxf(fabsf(dx) - ex, 0.0f), by = fmaxf(fabsf(dy) - ey, 0.0f),
                    bz = fmaxf(fabsf(dz) - ez, 0.0f);
        lbmax = fmaxf(lbmax, bx * bx + by * by + bz * bz);
        m += (ks[q] <= pk) ? 1 : 0;
      }
    }
    lbmax = block_max_f(lbmax, sf) * 0.999999f;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int i = b + threadIdx.x + 256 * q;
      if (i < e) {
        const float4 t = ts[q];
        const float dx = t.x - cxf, dy = t.y - cyf, dz = t.z - czf;
        const float ex = eps23 * (fabsf(t.x) + fabsf(cxf) + fabsf(dx));
        const float ey = eps23 * (fabsf(t.y) + fabsf(cyf) + fabsf(dy));
        const float ez = eps23 * (fabsf(t.z) + fabsf(czf) + fabsf(dz));
        const float bx = fabsf(dx) + ex, by = fabsf(dy) + ey, bz = fabsf(dz) + ez;
        if ((bx * bx + by * by + bz * bz) * 1.000001f >= lbmax)
          r2m = fmax(r2m, r2_exact(tx[i] - nd.x, ty[i] - nd.y, tz[i] - nd.z));
      }
    }
  }
  r2m = warp_max(r2m);
  m = warp_sum_int(m);
  if (lane_id() == 0) { smax[threadIdx.x >> 5] = r2m; sc[threadIdx.x >> 5] = m; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = sc[0];
    for (int w = 1; w < 8; ++w) { r2m = fmax(r2m, smax[w]); t += sc[w]; }
    double *o = part + 8 * (size_t)c;
    o[0] = r2m;
    for (int w = 0; w < 6; ++w) o[1 + w] = q[w];
    if (cnt) cnt[c] = t;
  }
}

// kdtree.F90:780-796 size and quadrupoles; the left count and the
// all-on-one-side fallback (kdtree.F90:856-865)
__global__ void __launch_bounds__(32 * FIN_WARPS) k_big_fin2(Params p, const int *lvl, int nb, const int *cbase,
                                                             Node *nodes, double *nquads, const double *part,
                                                             const int *cnt, int *misc) {
  const int k = blockIdx.x * FIN_WARPS + (threadIdx.x >> 5), lane = lane_id();
  if (k >= nb) return;
  double r2m = 0.0, q[6] = {0, 0, 0, 0, 0, 0};
  int nl = 0;
  for (int c = cbase[k] + lane; c < cbase[k + 1]; c += 32) {
    const double *o = part + 8 * (size_t)c;
    r2m = fmax(r2m, o[0]);
    for (int w = 0; w < 6; ++w) q[w] = q[w] + o[1 + w];
    if (cnt) nl += cnt[c];
  }
  r2m = warp_max(r2m);
  for (int w = 0; w < 6; ++w) q[w] = warp_sum_d(q[w]);
  nl = warp_sum_int(nl);
  if (lane != 0) return;
  int id = lvl[k];
  Node &nd = nodes[id];
  nd.size = sqrt(r2m) + EPS_D;
  if (p.gravity) for (int w = 0; w < 6; ++w) nquads[6 * (size_t)id + w] = q[w];
  if (!misc) return;  // revtree: no split
  const int n = nd.count;
  int noswap = 0;
  if (nl == n || nl == 0) { nl = n / 2; noswap = 1; }
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
  const long long pk = dkey(pivot[k]);
  const double *cx = ax == 0 ? tx : (ax == 1 ? ty : tz);
  int nb_ = 0, ns_ = 0;
  for (int i = b + threadIdx.x; i < e; i += 256) {
    bool small = dkey(cx[i]) <= pk;
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
// (exclusive warp scans over the node's chunks, 32 at a time)
__global__ void __launch_bounds__(32 * FIN_WARPS) k_big_fin4(const int *lvl, int nb, const int *cbase, int *bl,
                                                             int *sr) {
  const int k = blockIdx.x * FIN_WARPS + (threadIdx.x >> 5), lane = lane_id();
  if (k >= nb) return;
  const int c0 = cbase[k], c1 = cbase[k + 1];
  int acc = 0;
  for (int b = c0; b < c1; b += 32) {
    const int c = b + lane;
    const int v = c < c1 ? bl[c] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) { const int y = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += y; }
    if (c < c1) bl[c] = acc + x - v;
    acc += __shfl_sync(0xffffffffu, x, 31);
  }
  acc = 0;
  for (int b = c1 - 1; b >= c0; b -= 32) {
    const int c = b - lane;
    const int v = c >= c0 ? sr[c] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) { const int y = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += y; }
    if (c >= c0) sr[c] = acc + x - v;
    acc += __shfl_sync(0xffffffffu, x, 31);
  }
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
  const long long pk = dkey(pivot[k]);
  const double *cx = ax == 0 ? tx : (ax == 1 ? ty : tz);
  // each thread owns 8 consecutive elements (thread order == position order)
  int i0 = b + threadIdx.x * 8;
  int flags = 0, cntl = 0;
  for (int q = 0; q < 8; ++q) {
    int i = i0 + q;
    bool f = (i < e) && (i >= bnd) && (dkey(cx[i]) <= pk);
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

__device__ __forceinline__ void swap_rows(double *tx, double *ty, double *tz, double *th, int *perm, float4 *txf,
                                          int a, int b) {
  double t;
  t = tx[a]; tx[a] = tx[b]; tx[b] = t;
  t = ty[a]; ty[a] = ty[b]; ty[b] = t;
  t = tz[a]; tz[a] = tz[b]; tz[b] = t;
  t = th[a]; th[a] = th[b]; th[b] = t;
  int u = perm[a]; perm[a] = perm[b]; perm[b] = u;
  float4 f = txf[a]; txf[a] = txf[b]; txf[b] = f;
}

// swap each left-region big with its paired right-region small (kdtree.F90:969-977)
__global__ void __launch_bounds__(256) k_big_swap(const int *lvl, int nb, const int *cbase, const Node *nodes,
                                                  double *tx, double *ty, double *tz, double *th, int *perm,
                                                  float4 *txf, const int *misc, const double *pivot,
                                                  const int *bl, const int *pairpos) {
  __shared__ int s[16];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  if (misc[4 * k + 2]) return;
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  int ax = misc[4 * k], bnd = nd.start + misc[4 * k + 1];
  const long long pk = dkey(pivot[k]);
  const double *cx = ax == 0 ? tx : (ax == 1 ? ty : tz);
  int i0 = b + threadIdx.x * 8;
  int flags = 0, cntl = 0;
  for (int q = 0; q < 8; ++q) {
    int i = i0 + q;
    bool f = (i < e) && (i < bnd) && !(dkey(cx[i]) <= pk);
    if (f) { flags |= 1 << q; ++cntl; }
  }
  int total;
  int pre = block_excl_scan(cntl, s, total);
  int r = bl[c] + pre;
  for (int q = 0; q < 8; ++q) {
    if (flags & (1 << q)) {
      int partner = pairpos[nd.start + r];
      swap_rows(tx, ty, tz, th, perm, txf, i0 + q, partner);
      ++r;
    }
  }
}

// child bounding boxes (kdtree.F90:868-896): partial min/max per chunk and
// side, on order-preserving integer keys
__global__ void __launch_bounds__(256) k_big_cbounds(const int *lvl, int nb, const int *cbase, const Node *nodes,
                                                     const double *tx, const double *ty, const double *tz,
                                                     const int *misc, double *part) {
  __shared__ long long s[12][8];
  int c = blockIdx.x;
  if (c >= cbase[nb]) return;
  int k = find_chunk_node(cbase, nb, c);
  const Node nd = nodes[lvl[k]];
  int b = nd.start + (c - cbase[k]) * CHUNK, e = min(b + CHUNK, nd.start + nd.count);
  int bnd = nd.start + misc[4 * k + 1];
  long long v[12];
  for (int q = 0; q < 2; ++q)
    for (int a = 0; a < 3; ++a) { v[6 * q + a] = KEY_HI; v[6 * q + 3 + a] = KEY_LO; }
  for (int i = b + threadIdx.x; i < e; i += 256) {
    const long long kx = dkey(tx[i]), ky = dkey(ty[i]), kz = dkey(tz[i]);
    if (i < bnd) {
      v[0] = min(v[0], kx); v[1] = min(v[1], ky); v[2] = min(v[2], kz);
      v[3] = max(v[3], kx); v[4] = max(v[4], ky); v[5] = max(v[5], kz);
    } else {
      v[6] = min(v[6], kx); v[7] = min(v[7], ky); v[8] = min(v[8], kz);
      v[9] = max(v[9], kx); v[10] = max(v[10], ky); v[11] = max(v[11], kz);
    }
  }
  for (int t = 0; t < 12; ++t) {
    const bool ismin = (t % 6) < 3;
    for (int o = 16; o > 0; o >>= 1) {
      const long long y = __shfl_xor_sync(0xffffffffu, v[t], o);
      v[t] = ismin ? min(v[t], y) : max(v[t], y);
    }
  }
  int w = threadIdx.x >> 5;
  if (lane_id() == 0) for (int t = 0; t < 12; ++t) s[t][w] = v[t];
  __syncthreads();
  if (threadIdx.x == 0) {
    double *o = part + 16 * (size_t)c;
    for (int t = 0; t < 12; ++t) {
      long long r = s[t][0];
      const bool ismin = (t % 6) < 3;
      for (int q = 1; q < 8; ++q) r = ismin ? min(r, s[t][q]) : max(r, s[t][q]);
      o[t] = dunkey(r);
    }
  }
}

// children creation, next-level lists
__global__ void __launch_bounds__(32 * FIN_WARPS) k_big_fin5(const int *lvl, int nb, const int *cbase, Node *nodes,
                                                             const int *misc, const double *part, int child_base,
                                                             int *lvl_next, double *bb_next, GenEntry *gen,
                                                             int *counters, int gen_cap, int *err) {
  const int k = blockIdx.x * FIN_WARPS + (threadIdx.x >> 5), lane = lane_id();
  if (k >= nb) return;
  double bb[12];
  for (int q = 0; q < 2; ++q)
    for (int a = 0; a < 3; ++a) { bb[6 * q + a] = HUGE_D; bb[6 * q + 3 + a] = -HUGE_D; }
  for (int c = cbase[k] + lane; c < cbase[k + 1]; c += 32) {
    const double *o = part + 16 * (size_t)c;
    for (int t = 0; t < 12; ++t) bb[t] = ((t % 6) < 3) ? fmin(bb[t], o[t]) : fmax(bb[t], o[t]);
  }
  for (int t = 0; t < 12; ++t) bb[t] = ((t % 6) < 3) ? warp_min(bb[t]) : warp_max(bb[t]);
  if (lane != 0) return;
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
      if (slot >= gen_cap) { set_error(err, PH_ERR_TREE); continue; }
      GenEntry g;
      g.id = cid; g.start = ch.start; g.count = ch.count; g.level = ch.level; g.parent = id; g.pad = 0;
      for (int t = 0; t < 6; ++t) g.bb[t] = bb[6 * q + t];
      gen[slot] = g;
    }
  }
}

// ------------------------------------------------------------------ small nodes
// Nodes of at most SMALL particles are built generation by generation, the
// children of one generation forming the next, with what construct_node does
// for each (kdtree.F90:639-896). FP64 work on this GPU is expensive (one warp
// instruction per ~17 SM cycles whatever the active lanes, 68-cycle dependent
// latency), so only the reference's sequential centre-of-mass sums (the
// pivot, hence the partition, depends on their rounding) are FP64 chains, one
// lane per node; the quadrupoles, which no tree decision reads, are parallel
// FP64 sums; everything else is integer or FP32, with exact FP64 only where
// an FP32 bound cannot decide:
// * node mass: the sequential sum of n particle masses, from a table;
// * hmax, child bounding boxes and the pivot test: order-preserving integer
//   keys of the FP64 values (exact);
// * size: max of the exact FP64 r^2 over the particles that FP32 bounds
//   cannot exclude from being the maximum.
// Node ids in this part do not depend on the order of the generation list: a
// right child is the only right child starting at its first particle s (id
// subbase + 2 s + 1), a left child the only left child ending at its last
// particle e (id subbase + 2 e).
__global__ void k_mass_table(double pm, double *mtab) {
  double sm = 0.0;
  mtab[0] = 0.0;
  for (int k = 1; k <= SMALL; ++k) { sm = dadd(sm, pm); mtab[k] = sm; }
}

// K1 of a generation: centre of mass of the nodes, one lane per node and
// axis, each lane running the reference's sequential FP64 sum of one
// coordinate over its node. The chains are latency bound (68 cycles per
// dependent FP64 add) and the early generations hold few nodes, so the three
// axes take three lanes, and the particles must be in shared memory before
// the chain reaches them: the warp copies 16-particle tiles of its 32 chains
// with asynchronous copies, two tiles in flight while the chains consume the
// current one. com[4 * g + a] = coordinate a of the centre of mass of entry g.
constexpr int TILE = 16, NBUF = 3;

__global__ void __launch_bounds__(32) k_small_com(Params p, const GenEntry *cur, int ncur, const double *mtab,
                                                  const double *tx, const double *ty, const double *tz,
                                                  double *com) {
  __shared__ double tile[NBUF][TILE][33];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x;
  const int gq = blockIdx.x * 32 + lane;  // chain: node gq / 3, axis gq % 3
  const int g = gq / 3, axis = gq - 3 * g;
  const bool valid = g < ncur;
  int s = 0, n = 0;
  if (valid) { const GenEntry e = cur[g]; s = e.start; n = e.count; }
  const double *src = axis == 0 ? tx : (axis == 1 ? ty : tz);
  const int nmax = (int)__reduce_max_sync(FULL, (unsigned)n);
  const double pm = p.massoftype, dfac = (pm > 0.0) ? 1.0 / pm : 1.0, fac = pm * dfac;
  const bool fac1 = fac == 1.0;
  // lane l copies particle base + (l & 15) of chains k + (l >> 4), k even
  const int half = lane >> 4, el = lane & (TILE - 1);
  auto issue = [&](int buf, int base) {
    for (int k = 0; k < 32; k += 2) {
      const int nk = __shfl_sync(FULL, n, k + half), sk = __shfl_sync(FULL, s, k + half);
      const double *sp = reinterpret_cast<const double *>(
          __shfl_sync(FULL, reinterpret_cast<unsigned long long>(src), k + half));
      const int i = base + el;
      if (i < nk) __pipeline_memcpy_async(&tile[buf][el][k + half], sp + sk + i, sizeof(double));
    }
  };
  double acc = 0.0;
  const int nt = (nmax + TILE - 1) / TILE;
  // NBUF - 1 tiles in flight ahead of the chains (one commit group per tile,
  // empty groups past the end keep the wait count uniform)
  for (int t = 0; t < NBUF - 1; ++t) {
    if (t < nt) issue(t, t * TILE);
    __pipeline_commit();
  }
  for (int t = 0; t < nt; ++t) {
    const int buf = t % NBUF;
    if (t + NBUF - 1 < nt) issue((t + NBUF - 1) % NBUF, (t + NBUF - 1) * TILE);
    __pipeline_commit();
    __pipeline_wait_prior(NBUF - 1);
    __syncwarp();
    const int cnt = min(TILE, n - t * TILE);
    if (fac1) {
      for (int q = 0; q < cnt; ++q) acc = dadd(acc, tile[buf][q][lane]);
    } else {
      for (int q = 0; q < cnt; ++q) acc = dadd(acc, dmul(fac, tile[buf][q][lane]));
    }
    __syncwarp();  // the buffer is refilled NBUF - 1 iterations later
  }
  const double sm = valid ? mtab[n] : 0.0;
  const double d = sm * dfac;
  if (sm > 0.0) acc = ddiv(acc, d);
  if (valid) com[4 * (size_t)g + axis] = acc;
}

__device__ __forceinline__ long long warp_min_ll(long long v) {
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ long long warp_max_ll(long long v) {
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// K2 of a generation: a segment of SEG lanes per node (32 / SEG nodes per
// warp), lanes over its particles (coalesced): size, hmax, the count on the
// pivot's left, both sides' bounding boxes, the partition and the node
// record; the children go to the next generation. Segment reductions are
// xor butterflies inside the segment; the partition's ballots run a
// warp-uniform number of rounds. Slots in the next generation and the node
// list are taken with one atomic per warp. maxcnt receives the largest child
// count (the next generation's segment width).
constexpr int SPLIT_WARPS = 4;

template <int SEG>
__device__ __forceinline__ long long seg_min_ll(long long v) {
  for (int o = SEG / 2; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
template <int SEG>
__device__ __forceinline__ long long seg_max_ll(long long v) {
  for (int o = SEG / 2; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
template <int SEG>
__device__ __forceinline__ int seg_sum_int(int v) {
  for (int o = SEG / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int SEG>
__global__ void __launch_bounds__(32 * SPLIT_WARPS) k_small_split(
    Params p, const GenEntry *cur, int ncur, const double *com, GenEntry *next, int *nnext, int next_cap,
    const double *mtab, Node *nodes, double *nmass, double *nquads, double *tx, double *ty, double *tz, double *th,
    int *perm, float4 *txf, int *pairpos, int subbase, int *leaf_at, int *lvlstat, NodeF *nodesf, int *node_list,
    int *node_count, int *maxcnt, int *err) {
  const unsigned FULL = 0xffffffffu;
  constexpr int NSEG = 32 / SEG;
  const int lane = lane_id(), seg = lane / SEG, sl = lane % SEG;
  const unsigned segmask = (SEG == 32) ? FULL : (((1u << SEG) - 1u) << (seg * SEG));
  const unsigned lt = (1u << lane) - 1u;
  const int wg = blockIdx.x * SPLIT_WARPS + (threadIdx.x >> 5);
  if (wg * NSEG >= ncur) return;  // warp-uniform
  const int g = wg * NSEG + seg;
  const bool valid = g < ncur;
  GenEntry e{};
  if (valid) e = cur[g];
  const int s = e.start, n = valid ? e.count : 0, end = s + n;
  double sx = 0.0, sy = 0.0, sz = 0.0;
  if (valid) { sx = com[4 * (size_t)g]; sy = com[4 * (size_t)g + 1]; sz = com[4 * (size_t)g + 2]; }
  const bool split = valid && n > p.minpart;  // kdtree.F90:792
  int ax = 0;
  if (split) {  // longest bounding-box extent (kdtree.F90:800-816)
    const double ext0 = e.bb[3] - e.bb[0], ext1 = e.bb[4] - e.bb[1], ext2 = e.bb[5] - e.bb[2];
    double em = ext0;
    if (ext1 > em) { ax = 1; em = ext1; }
    if (ext2 > em) ax = 2;
  }
  const double pv = ax == 0 ? sx : (ax == 1 ? sy : sz);
  const long long pk = dkey(pv);
  // size (kdtree.F90:734-741): FP32 separations d' obey |d' - d| <= E with
  // E = 2^-23 (|x'| + |c'| + |d'|) per axis, which brackets each r^2; only
  // particles whose upper bound reaches the largest lower bound can hold the
  // maximum, and their r^2 is evaluated exactly in FP64.
  const float cxf = (float)sx, cyf = (float)sy, czf = (float)sz;
  const float eps23 = 1.1920929e-7f;
  float lbmax = 0.0f;
  long long l0 = KEY_HI, l1 = KEY_HI, l2 = KEY_HI, l3 = KEY_LO, l4 = KEY_LO, l5 = KEY_LO;
  long long r0 = KEY_HI, r1 = KEY_HI, r2 = KEY_HI, r3 = KEY_LO, r4 = KEY_LO, r5 = KEY_LO;
  long long hk = KEY_LO;
  int nl = 0;
  for (int i = s + sl; i < end; i += SEG) {
    const float4 q = txf[i];
    const float dx = q.x - cxf, dy = q.y - cyf, dz = q.z - czf;
    const float ex = eps23 * (fabsf(q.x) + fabsf(cxf) + fabsf(dx));
    const float ey = eps23 * (fabsf(q.y) + fabsf(cyf) + fabsf(dy));
    const float ez = eps23 * (fabsf(q.z) + fabsf(czf) + fabsf(dz));
    const float bx = fmaxf(fabsf(dx) - ex, 0.0f), by = fmaxf(fabsf(dy) - ey, 0.0f), bz = fmaxf(fabsf(dz) - ez, 0.0f);
    lbmax = fmaxf(lbmax, bx * bx + by * by + bz * bz);
    hk = max(hk, dkey(th[i]));  // hmax (kdtree.F90:661): a max, so lanes over particles
    if (split) {
      // count on the pivot's left (kdtree.F90:954-955) and both sides' boxes
      const long long kx = dkey(tx[i]), ky = dkey(ty[i]), kz = dkey(tz[i]);
      const long long kc = ax == 0 ? kx : (ax == 1 ? ky : kz);
      if (kc <= pk) {
        ++nl;
        l0 = min(l0, kx); l1 = min(l1, ky); l2 = min(l2, kz); l3 = max(l3, kx); l4 = max(l4, ky); l5 = max(l5, kz);
      } else {
        r0 = min(r0, kx); r1 = min(r1, ky); r2 = min(r2, kz); r3 = max(r3, kx); r4 = max(r4, ky); r5 = max(r5, kz);
      }
    }
  }
  for (int o = SEG / 2; o > 0; o >>= 1) lbmax = fmaxf(lbmax, __shfl_xor_sync(FULL, lbmax, o));
  lbmax *= 0.999999f;
  long long r2k = 0;
  for (int i = s + sl; i < end; i += SEG) {
    const float4 q = txf[i];
    const float dx = q.x - cxf, dy = q.y - cyf, dz = q.z - czf;
    const float ex = eps23 * (fabsf(q.x) + fabsf(cxf) + fabsf(dx));
    const float ey = eps23 * (fabsf(q.y) + fabsf(cyf) + fabsf(dy));
    const float ez = eps23 * (fabsf(q.z) + fabsf(czf) + fabsf(dz));
    const float bx = fabsf(dx) + ex, by = fabsf(dy) + ey, bz = fabsf(dz) + ez;
    if ((bx * bx + by * by + bz * bz) * 1.000001f >= lbmax) {
      const double ddx = tx[i] - sx, ddy = ty[i] - sy, ddz = tz[i] - sz;
      r2k = max(r2k, dkey(r2_exact(ddx, ddy, ddz)));
    }
  }
  r2k = seg_max_ll<SEG>(r2k);
  const double hm = fmax(0.0, dunkey(seg_max_ll<SEG>(hk)));
  if (p.gravity) {
    // quadrupoles (kdtree.F90:744-752): m sum of dx_a dx_b; lanes over
    // particles, then a fixed-order butterfly (no tree decision reads them)
    double q0 = 0, q1 = 0, q2 = 0, q3 = 0, q4 = 0, q5 = 0;
    for (int i = s + sl; i < end; i += SEG) {
      const double dx = tx[i] - sx, dy = ty[i] - sy, dz = tz[i] - sz;
      q0 = fma(dx, dx, q0); q1 = fma(dx, dy, q1); q2 = fma(dx, dz, q2);
      q3 = fma(dy, dy, q3); q4 = fma(dy, dz, q4); q5 = fma(dz, dz, q5);
    }
    for (int o = SEG / 2; o > 0; o >>= 1) {
      q0 += __shfl_xor_sync(FULL, q0, o); q1 += __shfl_xor_sync(FULL, q1, o); q2 += __shfl_xor_sync(FULL, q2, o);
      q3 += __shfl_xor_sync(FULL, q3, o); q4 += __shfl_xor_sync(FULL, q4, o); q5 += __shfl_xor_sync(FULL, q5, o);
    }
    if (valid && sl == 0) {
      const double pm = p.massoftype;
      double *qo = nquads + 6 * (size_t)e.id;
      qo[0] = pm * q0; qo[1] = pm * q1; qo[2] = pm * q2; qo[3] = pm * q3; qo[4] = pm * q4; qo[5] = pm * q5;
    }
  }
  nl = seg_sum_int<SEG>(nl);
  const bool noswap = split && (nl == n || nl == 0);
  if (noswap) {
    // no split along the axis: halves by position, no swaps (kdtree.F90:856-865)
    nl = n / 2;
    l0 = l1 = l2 = r0 = r1 = r2 = KEY_HI;
    l3 = l4 = l5 = r3 = r4 = r5 = KEY_LO;
    for (int i = s + sl; i < end; i += SEG) {
      const long long kx = dkey(tx[i]), ky = dkey(ty[i]), kz = dkey(tz[i]);
      if (i < s + nl) {
        l0 = min(l0, kx); l1 = min(l1, ky); l2 = min(l2, kz); l3 = max(l3, kx); l4 = max(l4, ky); l5 = max(l5, kz);
      } else {
        r0 = min(r0, kx); r1 = min(r1, ky); r2 = min(r2, kz); r3 = max(r3, kx); r4 = max(r4, ky); r5 = max(r5, kz);
      }
    }
  }
  l0 = seg_min_ll<SEG>(l0); l1 = seg_min_ll<SEG>(l1); l2 = seg_min_ll<SEG>(l2);
  l3 = seg_max_ll<SEG>(l3); l4 = seg_max_ll<SEG>(l4); l5 = seg_max_ll<SEG>(l5);
  r0 = seg_min_ll<SEG>(r0); r1 = seg_min_ll<SEG>(r1); r2 = seg_min_ll<SEG>(r2);
  r3 = seg_max_ll<SEG>(r3); r4 = seg_max_ll<SEG>(r4); r5 = seg_max_ll<SEG>(r5);
  // partition: the k-th element > pivot left of the boundary (counted from
  // the left) swaps with the k-th element <= pivot right of it (counted
  // from the right), as the two-pointer loop of the reference pairs them
  const bool part = split && !noswap;
  const double *cx = ax == 0 ? tx : (ax == 1 ? ty : tz);
  const int bnd = s + nl;
  const int tr = part ? (end - bnd + SEG - 1) / SEG : 0, tl = part ? (nl + SEG - 1) / SEG : 0;
  const int trmax = (int)__reduce_max_sync(FULL, (unsigned)tr), tlmax = (int)__reduce_max_sync(FULL, (unsigned)tl);
  int m2 = 0;
  for (int t = 0; t < trmax; ++t) {
    const int i = end - 1 - t * SEG - sl;
    const bool f = t < tr && i >= bnd && dkey(cx[i]) <= pk;
    const unsigned bal = __ballot_sync(FULL, f) & segmask;
    if (f) pairpos[s + m2 + __popc(bal & lt)] = i;
    m2 += __popc(bal);
  }
  __syncwarp();
  int m = 0;
  for (int t = 0; t < tlmax; ++t) {
    const int i = s + t * SEG + sl;
    const bool f = t < tl && i < bnd && dkey(cx[i]) > pk;
    const unsigned bal = __ballot_sync(FULL, f) & segmask;
    if (f) {
      const int r = m + __popc(bal & lt);
      if (r < m2) swap_rows(tx, ty, tz, th, perm, txf, i, pairpos[s + r]);
    }
    m += __popc(bal);
  }
  if (part && m != m2 && sl == 0) set_error(err, PH_ERR_TREE);
  __syncwarp();
  // node records, next-generation entries and statistics (segment leaders)
  const bool lead = valid && sl == 0;
  const double sm = valid ? mtab[n] : 0.0;
  Node nd{};
  nd.x = sx; nd.y = sy; nd.z = sz; nd.size = sqrt(dunkey(r2k)) + EPS_D; nd.hmax = hm;
  nd.start = s; nd.count = n; nd.level = e.level; nd.parent = e.parent;
  nd.left = -1; nd.right = -1;
  const unsigned bsplit = __ballot_sync(FULL, lead && split);
  const unsigned bleaf = __ballot_sync(FULL, lead && !split);
  int base_list = 0, base_next = 0;
  if (bsplit) {
    const int first = __ffs(bsplit) - 1;
    if (lane == first) {
      base_list = atomicAdd(node_count, 2 * __popc(bsplit));
      base_next = atomicAdd(nnext, 2 * __popc(bsplit));
    }
    base_list = __shfl_sync(FULL, base_list, first);
    base_next = __shfl_sync(FULL, base_next, first);
  }
  // deepest and shallowest leaf levels, one atomic each per warp
  int lmax = (lead && !split) ? e.level : 0, lmin = (lead && !split) ? e.level : (1 << 30);
  for (int o = 16; o > 0; o >>= 1) {
    lmax = max(lmax, __shfl_xor_sync(FULL, lmax, o));
    lmin = min(lmin, __shfl_xor_sync(FULL, lmin, o));
  }
  // largest child count of the warp (the next generation's segment width)
  int cmax = (lead && split) ? max(nl, n - nl) : 0;
  for (int o = 16; o > 0; o >>= 1) cmax = max(cmax, __shfl_xor_sync(FULL, cmax, o));
  if (lane == 0) {
    if (bleaf) { atomicMax(&lvlstat[0], lmax); atomicMin(&lvlstat[1], lmin); }
    if (bsplit) atomicMax(maxcnt, cmax);
  }
  if (!lead) return;
  if (!split) {
    nodes[e.id] = nd;
    nodesf[e.id] = make_nodef(nd);
    nmass[e.id] = sm;
    leaf_at[s] = e.id;
    return;
  }
  const int il = subbase + 2 * (s + nl - 1), ir = subbase + 2 * (s + nl) + 1;
  nd.left = il; nd.right = ir;
  nodes[e.id] = nd;
  nodesf[e.id] = make_nodef(nd);
  nmass[e.id] = sm;
  const int rank = 2 * __popc(bsplit & lt);
  const int ls = base_list + rank;
  node_list[ls] = il;
  node_list[ls + 1] = ir;
  const int slot = base_next + rank;
  if (slot + 2 > next_cap) { set_error(err, PH_ERR_TREE); return; }
  GenEntry a, b;
  a.id = il; a.start = s; a.count = nl; a.level = e.level + 1; a.parent = e.id; a.pad = 0;
  b.id = ir; b.start = s + nl; b.count = n - nl; b.level = e.level + 1; b.parent = e.id; b.pad = 0;
  a.bb[0] = dunkey(l0); a.bb[1] = dunkey(l1); a.bb[2] = dunkey(l2);
  a.bb[3] = dunkey(l3); a.bb[4] = dunkey(l4); a.bb[5] = dunkey(l5);
  b.bb[0] = dunkey(r0); b.bb[1] = dunkey(r1); b.bb[2] = dunkey(r2);
  b.bb[3] = dunkey(r3); b.bb[4] = dunkey(r4); b.bb[5] = dunkey(r5);
  next[slot] = a;
  next[slot + 1] = b;
}

// ------------------------------------------------------------------ revtree
// revtree (kdtree.F90:1851-2037): every node's centre of mass, size, hmax,
// mass and quadrupoles from new positions of the same particles, on the
// tree structure built last (particle order, ranges and children kept).
// Nodes of more than SMALL particles take the level kernels' blocked sums,
// the others the sequential chains of the generations (particle order is
// the tree order, as the reference's revtree reads treecache).
__global__ void k_rev_gather(const double *__restrict__ xyzh, int n, const int *__restrict__ perm, double *tx,
                             double *ty, double *tz, double *th, float4 *txf) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double *x = xyzh + 4 * (size_t)perm[k];
  tx[k] = x[0]; ty[k] = x[1]; tz[k] = x[2]; th[k] = x[3];
  txf[k] = make_float4((float)x[0], (float)x[1], (float)x[2], 0.0f);
}

__global__ void k_rev_entries(const int *ids, int m, const Node *nodes, GenEntry *gen) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m) return;
  const Node nd = nodes[ids[g]];
  GenEntry e{};
  e.id = ids[g]; e.start = nd.start; e.count = nd.count; e.level = nd.level; e.parent = nd.parent;
  gen[g] = e;
}

// size, hmax, mass and quadrupoles of small nodes from their centres of mass
// (k_small_com), one warp per node; the node's structure is kept
__global__ void __launch_bounds__(128) k_rev_small(Params p, const GenEntry *cur, int ncur, const double *com,
                                                   const double *mtab, Node *nodes, double *nmass, double *nquads,
                                                   const double *tx, const double *ty, const double *tz,
                                                   const double *th, const float4 *txf, NodeF *nodesf) {
  const unsigned FULL = 0xffffffffu;
  const int g = blockIdx.x * 4 + (threadIdx.x >> 5), lane = lane_id();
  if (g >= ncur) return;
  const GenEntry e = cur[g];
  const int s = e.start, end = s + e.count;
  const double sx = com[4 * (size_t)g], sy = com[4 * (size_t)g + 1], sz = com[4 * (size_t)g + 2];
  const float cxf = (float)sx, cyf = (float)sy, czf = (float)sz;
  const float eps23 = 1.1920929e-7f;
  float lbmax = 0.0f;
  long long hk = KEY_LO;
  for (int i = s + lane; i < end; i += 32) {
    const float4 q = txf[i];
    const float dx = q.x - cxf, dy = q.y - cyf, dz = q.z - czf;
    const float ex = eps23 * (fabsf(q.x) + fabsf(cxf) + fabsf(dx));
    const float ey = eps23 * (fabsf(q.y) + fabsf(cyf) + fabsf(dy));
    const float ez = eps23 * (fabsf(q.z) + fabsf(czf) + fabsf(dz));
    const float bx = fmaxf(fabsf(dx) - ex, 0.0f), by = fmaxf(fabsf(dy) - ey, 0.0f), bz = fmaxf(fabsf(dz) - ez, 0.0f);
    lbmax = fmaxf(lbmax, bx * bx + by * by + bz * bz);
    hk = max(hk, dkey(fabs(th[i])));
  }
  for (int o = 16; o > 0; o >>= 1) lbmax = fmaxf(lbmax, __shfl_xor_sync(FULL, lbmax, o));
  lbmax *= 0.999999f;
  long long r2k = 0;
  for (int i = s + lane; i < end; i += 32) {
    const float4 q = txf[i];
    const float dx = q.x - cxf, dy = q.y - cyf, dz = q.z - czf;
    const float ex = eps23 * (fabsf(q.x) + fabsf(cxf) + fabsf(dx));
    const float ey = eps23 * (fabsf(q.y) + fabsf(cyf) + fabsf(dy));
    const float ez = eps23 * (fabsf(q.z) + fabsf(czf) + fabsf(dz));
    const float bx = fabsf(dx) + ex, by = fabsf(dy) + ey, bz = fabsf(dz) + ez;
    if ((bx * bx + by * by + bz * bz) * 1.000001f >= lbmax)
      r2k = max(r2k, dkey(r2_exact(tx[i] - sx, ty[i] - sy, tz[i] - sz)));
  }
  r2k = warp_max_ll(r2k);
  hk = warp_max_ll(hk);
  if (p.gravity) {
    double q0 = 0, q1 = 0, q2 = 0, q3 = 0, q4 = 0, q5 = 0;
    for (int i = s + lane; i < end; i += 32) {
      const double dx = tx[i] - sx, dy = ty[i] - sy, dz = tz[i] - sz;
      q0 = fma(dx, dx, q0); q1 = fma(dx, dy, q1); q2 = fma(dx, dz, q2);
      q3 = fma(dy, dy, q3); q4 = fma(dy, dz, q4); q5 = fma(dz, dz, q5);
    }
    for (int o = 16; o > 0; o >>= 1) {
      q0 += __shfl_xor_sync(FULL, q0, o); q1 += __shfl_xor_sync(FULL, q1, o); q2 += __shfl_xor_sync(FULL, q2, o);
      q3 += __shfl_xor_sync(FULL, q3, o); q4 += __shfl_xor_sync(FULL, q4, o); q5 += __shfl_xor_sync(FULL, q5, o);
    }
    if (lane == 0) {
      const double pm = p.massoftype;
      double *qo = nquads + 6 * (size_t)e.id;
      qo[0] = pm * q0; qo[1] = pm * q1; qo[2] = pm * q2; qo[3] = pm * q3; qo[4] = pm * q4; qo[5] = pm * q5;
    }
  }
  if (lane != 0) return;
  Node nd = nodes[e.id];
  nd.x = sx; nd.y = sy; nd.z = sz;
  nd.size = sqrt(dunkey(r2k)) + EPS_D;  // kdtree.F90:2007
  nd.hmax = fmax(0.0, dunkey(hk));
  nodes[e.id] = nd;
  nodesf[e.id] = make_nodef(nd);
  nmass[e.id] = mtab[e.count];
}

// the tree's nodes in library order (ph_get_nodes)
__global__ void k_get_nodes(const int *ids, int m, const Node *nodes, const double *nmass, int *range, double *xcen,
                            double *size, double *hmax, double *mass, int *isleaf) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m) return;
  const Node nd = nodes[ids[g]];
  range[2 * g] = nd.start + 1; range[2 * g + 1] = nd.start + nd.count;  // inoderange, 1-based
  xcen[3 * g] = nd.x; xcen[3 * g + 1] = nd.y; xcen[3 * g + 2] = nd.z;
  size[g] = nd.size; hmax[g] = nd.hmax; mass[g] = nmass[ids[g]];
  isleaf[g] = nd.left < 0 ? 1 : 0;
}

// nodes deeper than a level (big nodes are ids [0, nbig), the others listed)
__global__ void k_count_deep(const Node *nodes, int nbig, const int *node_list, int nsmall, int level, int *out) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const bool deep = g < nbig + nsmall && nodes[g < nbig ? g : node_list[g - nbig]].level > level;
  const unsigned b = __ballot_sync(0xffffffffu, deep);
  if (lane_id() == 0 && b) atomicAdd(out, __popc(b));
}

// FP32 mirror of the nodes built by the level kernels (ids below next_id)
__global__ void k_node_mirror(const Node *nodes, int n, NodeF *nodesf) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) nodesf[k] = make_nodef(nodes[k]);
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
  k_root_fill<<<nblk(n, 256), 256, 0, st>>>(c->xyzh, n, c->alive, c->pairpos, c->tx, c->ty, c->tz, c->th, c->perm,
                                            c->txf);
  int nbb = std::min(nblk(nalive, 256), 1024);
  k_bbox_partial<<<nbb, 256, 0, st>>>(c->tx, c->ty, c->tz, nalive, c->part_d);
  cudaMemsetAsync(c->counters, 0, 4 * sizeof(int), st);
  k_root_node<<<1, 256, 0, st>>>(c->part_d, nbb, nalive, c->nodes, c->lvl_a, c->lvl_bb_a, c->gen_a, c->counters);
  k_fill_int<<<nblk(nalive, 256), 256, 0, st>>>(c->leaf_at, nalive, -1);
  int lvlinit[2] = {0, 1 << 30};
  cudaMemcpyAsync(c->d_maxlevel, lvlinit, 2 * sizeof(int), cudaMemcpyHostToDevice, st);
  count_launch(c, 4);
  int counters[2] = {0, 0};
  cudaMemcpyAsync(counters, c->counters, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  int nb = counters[0];
  int next_id = 1;
  // sequential sums of k equal particle masses (node masses, chunk partials)
  if (c->mtab_pm != p.massoftype) {
    k_mass_table<<<1, 1, 0, st>>>(p.massoftype, c->mtab);
    count_launch(c, 1);
    c->mtab_pm = p.massoftype;
  }

  int *lvl = c->lvl_a, *lvl_next = c->lvl_b;
  double *bb = c->lvl_bb_a, *bb_next = c->lvl_bb_b;
  int guard = 0;
  while (nb > 0) {
    if (++guard > 200 || next_id + 2 * nb > c->subbase) return PH_ERR_TREE;
    int maxchunks = nalive / CHUNK + nb + 1;
    if (maxchunks > c->chunk_cap) return PH_ERR_TREE;
    int *cb = c->cbase;
    int *cnt = c->part_i, *bl = c->part_i + c->chunk_cap, *sr = c->part_i + 2 * c->chunk_cap;
    k_chunk_table<<<1, 1024, 0, st>>>(lvl, nb, c->nodes, cb);
    k_big_props1<<<maxchunks, 256, 0, st>>>(p, lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->th, c->mtab,
                                            c->part_d);
    k_big_fin1<<<nblk(nb, FIN_WARPS), 32 * FIN_WARPS, 0, st>>>(p, lvl, nb, cb, c->nodes, c->nmass, c->part_d, bb,
                                                             c->lvl_misc, c->lvl_pivot);
    k_big_props2<<<maxchunks, 256, 0, st>>>(p, lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->txf, c->lvl_misc,
                                            c->lvl_pivot, c->part_d, cnt);
    k_big_fin2<<<nblk(nb, FIN_WARPS), 32 * FIN_WARPS, 0, st>>>(p, lvl, nb, cb, c->nodes, c->nquads, c->part_d, cnt,
                                                             c->lvl_misc);
    k_big_rank<<<maxchunks, 256, 0, st>>>(lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->lvl_misc, c->lvl_pivot, bl, sr);
    k_big_fin4<<<nblk(nb, FIN_WARPS), 32 * FIN_WARPS, 0, st>>>(lvl, nb, cb, bl, sr);
    k_big_pairs<<<maxchunks, 256, 0, st>>>(lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->lvl_misc, c->lvl_pivot,
                                           sr, c->pairpos);
    k_big_swap<<<maxchunks, 256, 0, st>>>(lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->th, c->perm, c->txf,
                                          c->lvl_misc, c->lvl_pivot, bl, c->pairpos);
    k_big_cbounds<<<maxchunks, 256, 0, st>>>(lvl, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->lvl_misc, c->part_d);
    cudaMemsetAsync(c->counters, 0, sizeof(int), st);
    k_big_fin5<<<nblk(nb, FIN_WARPS), 32 * FIN_WARPS, 0, st>>>(lvl, nb, cb, c->nodes, c->lvl_misc, c->part_d,
                                                             next_id, lvl_next, bb_next, c->gen_a, c->counters,
                                                             c->gen_cap, c->d_err);
    count_launch(c, 11);
    next_id += 2 * nb;
    cudaMemcpyAsync(counters, c->counters, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    nb = counters[0];
    std::swap(lvl, lvl_next);
    std::swap(bb, bb_next);
  }
  k_node_mirror<<<nblk(next_id, 256), 256, 0, st>>>(c->nodes, next_id, c->nodesf);
  count_launch(c, 1);
  c->nbig_nodes = next_id;
  cudaMemsetAsync(c->counters + 12, 0, sizeof(int), st);
  // small nodes, generation by generation
  GenEntry *gcur = c->gen_a, *gnext = c->gen_b;
  int ncur = counters[1];
  int gmax = SMALL;  // largest node of the generation
  for (int gen = 0; ncur > 0; ++gen) {
    if (gen > 4 * SMALL) return PH_ERR_TREE;
    cudaMemsetAsync(c->counters + 2, 0, 2 * sizeof(int), st);
    k_small_com<<<nblk(3 * (int64_t)ncur, 32), 32, 0, st>>>(p, gcur, ncur, c->mtab, c->tx, c->ty, c->tz, c->gen_com);
#define PH_SPLIT(SEG)                                                                                              \
  k_small_split<SEG><<<nblk(nblk(ncur, 32 / SEG), SPLIT_WARPS), 32 * SPLIT_WARPS, 0, st>>>(                       \
      p, gcur, ncur, c->gen_com, gnext, c->counters + 2, c->gen_cap, c->mtab, c->nodes, c->nmass, c->nquads, c->tx, \
      c->ty, c->tz, c->th, c->perm, c->txf, c->pairpos, c->subbase, c->leaf_at, c->d_maxlevel, c->nodesf,          \
      c->node_list, c->counters + 12, c->counters + 3, c->d_err)
    if (gmax > 96) PH_SPLIT(32);
    else if (gmax > 24) PH_SPLIT(16);
    else PH_SPLIT(8);
#undef PH_SPLIT
    count_launch(c, 2);
    int nv[2];
    cudaMemcpyAsync(nv, c->counters + 2, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    ncur = nv[0];
    gmax = nv[1];
    std::swap(gcur, gnext);
  }
  // leaf list in ascending start order
  k_flag_leaves<<<nblk(nalive, 256), 256, 0, st>>>(c->leaf_at, nalive, c->alive);
  scan_int(c, c->alive, c->pairpos, nalive, c->counters + 4);
  k_compact_leaves<<<nblk(nalive, 256), 256, 0, st>>>(c->leaf_at, c->pairpos, nalive, c->leaves);
  k_iperm<<<nblk(nalive, 256), 256, 0, st>>>(c->perm, nalive, c->iperm);
  count_launch(c, 3);
  int hostv[4];
  cudaMemcpyAsync(hostv, c->counters + 4, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hostv + 3, c->counters + 12, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hostv + 1, c->d_maxlevel, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  cudaError_t ce = check_launch(c);
  if (ce != cudaSuccess) return PH_ERR_CUDA;
  int herr = 0;
  cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (herr) return herr;
  c->nleaves = hostv[0];
  c->nsmall_nodes = hostv[3];
  c->maxlevel = hostv[1];
  c->minlevel = hostv[2];
  c->root = 0;
  c->have_tree = true;
  c->have_density = c->have_force_lists = false;
  if (p.ind && c->ibin) return ind_after_tree(c);  // active flags and cells in the new tree order
  return 0;
}

// revtree driver: c->xyzh holds the new positions (caller order)
int revtree(ph_ctx *c) {
  if (!c->have_tree) return PH_ERR_STATE;
  cudaStream_t st = c->stream;
  const Params p = c->dp;
  const int nt = (int)c->ntree, nbig = c->nbig_nodes, nsmall = c->nsmall_nodes;
  k_rev_gather<<<nblk(nt, 256), 256, 0, st>>>(c->xyzh, nt, c->perm, c->tx, c->ty, c->tz, c->th, c->txf);
  count_launch(c, 1);
  if (c->mtab_pm != p.massoftype) {
    k_mass_table<<<1, 1, 0, st>>>(p.massoftype, c->mtab);
    count_launch(c, 1);
    c->mtab_pm = p.massoftype;
  }
  // node ids [0, nbig) come from the level kernels: group those of more than
  // SMALL particles by level; the rest, with the generation-built nodes, are
  // refitted as small nodes
  std::vector<Node> big((size_t)nbig);
  cudaMemcpyAsync(big.data(), c->nodes, sizeof(Node) * (size_t)nbig, cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  std::vector<std::vector<int>> bylevel;
  std::vector<int> small_ids;
  for (int id = 0; id < nbig; ++id) {
    if (big[(size_t)id].count > SMALL) {
      const int L = big[(size_t)id].level;
      if ((int)bylevel.size() <= L) bylevel.resize((size_t)L + 1);
      bylevel[(size_t)L].push_back(id);
    } else {
      small_ids.push_back(id);
    }
  }
  for (const auto &lv : bylevel) {
    const int nb = (int)lv.size();
    if (nb == 0) continue;
    if (nb > c->lvl_cap) return PH_ERR_TREE;
    int64_t chunks = nb;
    for (int id : lv) chunks += big[(size_t)id].count / CHUNK;
    if (chunks > c->chunk_cap) return PH_ERR_TREE;
    cudaMemcpyAsync(c->lvl_a, lv.data(), sizeof(int) * (size_t)nb, cudaMemcpyHostToDevice, st);
    int *cb = c->cbase;
    const int maxchunks = (int)chunks + 1;
    k_chunk_table<<<1, 1024, 0, st>>>(c->lvl_a, nb, c->nodes, cb);
    k_big_props1<<<maxchunks, 256, 0, st>>>(p, c->lvl_a, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->th, c->mtab,
                                            c->part_d);
    k_big_fin1<<<nblk(nb, FIN_WARPS), 32 * FIN_WARPS, 0, st>>>(p, c->lvl_a, nb, cb, c->nodes, c->nmass, c->part_d,
                                                             nullptr, nullptr, nullptr);
    k_big_props2<<<maxchunks, 256, 0, st>>>(p, c->lvl_a, nb, cb, c->nodes, c->tx, c->ty, c->tz, c->txf, nullptr,
                                            nullptr, c->part_d, nullptr);
    k_big_fin2<<<nblk(nb, FIN_WARPS), 32 * FIN_WARPS, 0, st>>>(p, c->lvl_a, nb, cb, c->nodes, c->nquads, c->part_d,
                                                             nullptr, nullptr);
    count_launch(c, 5);
  }
  if (nbig > 0) {
    k_node_mirror<<<nblk(nbig, 256), 256, 0, st>>>(c->nodes, nbig, c->nodesf);
    count_launch(c, 1);
  }
  // small nodes in batches of the generation capacity: the ids of [0, nbig)
  // first, then the generation-built ones (node_list)
  const int64_t nsm = (int64_t)small_ids.size() + nsmall;
  int *ids = c->act_a;  // scratch of n ints
  const int64_t batch = std::min<int64_t>({(int64_t)c->gen_cap, c->cap});
  for (int64_t b0 = 0; b0 < nsm; b0 += batch) {
    const int m = (int)std::min<int64_t>(batch, nsm - b0);
    // ids b0 .. b0 + m of the concatenated list
    const int64_t nh = (int64_t)small_ids.size();
    const int64_t h0 = std::min(b0, nh), h1 = std::min(b0 + m, nh);
    if (h1 > h0) cudaMemcpyAsync(ids, small_ids.data() + h0, sizeof(int) * (size_t)(h1 - h0), cudaMemcpyHostToDevice, st);
    const int64_t l0 = std::max<int64_t>(b0 - nh, 0), l1 = b0 + m - nh;
    if (l1 > l0)
      cudaMemcpyAsync(ids + (h1 - h0), c->node_list + l0, sizeof(int) * (size_t)(l1 - l0), cudaMemcpyDeviceToDevice, st);
    k_rev_entries<<<nblk(m, 256), 256, 0, st>>>(ids, m, c->nodes, c->gen_a);
    k_small_com<<<nblk(3 * (int64_t)m, 32), 32, 0, st>>>(p, c->gen_a, m, c->mtab, c->tx, c->ty, c->tz, c->gen_com);
    k_rev_small<<<nblk(m, 4), 128, 0, st>>>(p, c->gen_a, m, c->gen_com, c->mtab, c->nodes, c->nmass, c->nquads, c->tx,
                                            c->ty, c->tz, c->th, c->txf, c->nodesf);
    count_launch(c, 3);
  }
  cudaStreamSynchronize(st);
  if (check_launch(c) != cudaSuccess) return PH_ERR_CUDA;
  int herr = 0;
  cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (herr) return herr;
  // positions changed: density, force lists and far field follow the refit
  c->have_density = c->have_force = c->have_force_lists = false;
  return 0;
}

// the tree's nodes in library order: ids [0, nbig) then the generation-built
int get_nodes(ph_ctx *c, int64_t *nnodes, int32_t *range, double *xcen, double *size, double *hmax, double *mass,
              int32_t *isleaf) {
  if (!c->have_tree) return PH_ERR_STATE;
  const int nbig = c->nbig_nodes, m = nbig + c->nsmall_nodes;
  *nnodes = m;
  if (!range || !xcen || !size || !hmax || !mass || !isleaf) return 0;
  cudaStream_t st = c->stream;
  std::vector<int> iota((size_t)nbig);
  for (int k = 0; k < nbig; ++k) iota[(size_t)k] = k;
  int *ids = nullptr, *dr = nullptr, *dl = nullptr;
  double *dx = nullptr, *ds = nullptr, *dh = nullptr, *dm = nullptr;
  bool ok = cudaMalloc(&ids, sizeof(int) * (size_t)m) == cudaSuccess &&
            cudaMalloc(&dr, sizeof(int) * 2 * (size_t)m) == cudaSuccess &&
            cudaMalloc(&dl, sizeof(int) * (size_t)m) == cudaSuccess &&
            cudaMalloc(&dx, sizeof(double) * 3 * (size_t)m) == cudaSuccess &&
            cudaMalloc(&ds, sizeof(double) * (size_t)m) == cudaSuccess &&
            cudaMalloc(&dh, sizeof(double) * (size_t)m) == cudaSuccess &&
            cudaMalloc(&dm, sizeof(double) * (size_t)m) == cudaSuccess;
  if (ok) {
    cudaMemcpyAsync(ids, iota.data(), sizeof(int) * (size_t)nbig, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(ids + nbig, c->node_list, sizeof(int) * (size_t)c->nsmall_nodes, cudaMemcpyDeviceToDevice, st);
    k_get_nodes<<<nblk(m, 256), 256, 0, st>>>(ids, m, c->nodes, c->nmass, dr, dx, ds, dh, dm, dl);
    count_launch(c, 1);
    cudaMemcpyAsync(range, dr, sizeof(int) * 2 * (size_t)m, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(isleaf, dl, sizeof(int) * (size_t)m, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(xcen, dx, sizeof(double) * 3 * (size_t)m, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(size, ds, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(hmax, dh, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(mass, dm, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
  }
  for (void *q : {(void *)ids, (void *)dr, (void *)dl, (void *)dx, (void *)ds, (void *)dh, (void *)dm})
    if (q) cudaFree(q);
  return ok ? 0 : PH_ERR_CUDA;
}

// maketree's ncells (kdtree.F90:167-179, 299-301, 820-833): 2^(maxlevel+1) - 1
// while the tree stays within the 2^k-indexed levels (maxlevel_indexed from
// ncellsmax = 2 maxp, config.F90:393), else the indexed part plus two slots
// per split below it, i.e. one per node deeper than maxlevel_indexed
int ref_ncells(ph_ctx *c, int64_t *ncells) {
  if (!c->have_tree) return PH_ERR_STATE;
  const int64_t ncellsmax = 2 * c->cap;
  const int mli = (int)(std::log((double)(ncellsmax + 1)) / std::log(2.0)) - 1;
  if (c->maxlevel < mli) {
    *ncells = ((int64_t)1 << (c->maxlevel + 1)) - 1;
    return 0;
  }
  int *d = c->counters + 20, deep = 0;  // a counter slot no build or pass uses
  cudaMemsetAsync(d, 0, sizeof(int), c->stream);
  const int m = c->nbig_nodes + c->nsmall_nodes;
  k_count_deep<<<nblk(m, 256), 256, 0, c->stream>>>(c->nodes, c->nbig_nodes, c->node_list, c->nsmall_nodes, mli, d);
  count_launch(c, 1);
  cudaMemcpyAsync(&deep, d, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return PH_ERR_CUDA;
  *ncells = ((int64_t)1 << (mli + 1)) - 1 + deep;
  return 0;
}

// ------------------------------------------------------------------ individual timesteps
// tree-order activity and ibin_old of the particles, cleared wake marks, and
// the leaf cells holding an active particle (kdtree.F90:575-579, 800-812)
__global__ void k_ind_gather(int n, const int *perm, const unsigned char *actf, const int8_t *ibin_old,
                             unsigned char *actf_t, int8_t *ibin_old_t, unsigned char *wakemark) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int pid = perm[k];
  actf_t[k] = actf[pid];
  ibin_old_t[k] = ibin_old[pid];
  wakemark[k] = 0;
}
__global__ void k_ind_cells(int ncell, const int *leaves, const Node *nodes, const unsigned char *actf_t, int *flag) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncell) return;
  const Node nd = nodes[leaves[cell]];
  int a = 0;
  for (int q = 0; q < nd.count; ++q) a |= actf_t[nd.start + q];
  flag[cell] = a ? 1 : 0;
}
__global__ void k_ind_compact(int ncell, const int *flag, const int *pos, int *list) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell < ncell && flag[cell]) list[pos[cell]] = cell;
}

int ind_after_tree(ph_ctx *c) {
  cudaStream_t st = c->stream;
  const int nt = (int)c->ntree, ncell = c->nleaves;
  k_ind_gather<<<nblk(nt, 256), 256, 0, st>>>(nt, c->perm, c->actf, c->ibin_old, c->actf_t, c->ibin_old_t,
                                              c->wakemark);
  k_ind_cells<<<nblk(ncell, 256), 256, 0, st>>>(ncell, c->leaves, c->nodes, c->actf_t, c->alive);
  scan_int(c, c->alive, c->pairpos, ncell, c->counters + 4);
  k_ind_compact<<<nblk(ncell, 256), 256, 0, st>>>(ncell, c->alive, c->pairpos, c->cell_act);
  count_launch(c, 3);
  int na = 0;
  cudaMemcpyAsync(&na, c->counters + 4, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  c->ncell_act = na;
  return check_launch(c) == cudaSuccess ? 0 : PH_ERR_CUDA;
}

}  // namespace ph
