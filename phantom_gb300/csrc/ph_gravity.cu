// Self-gravity far field (K7): getneigh_dual (kdtree.F90:1357-1461) with
// node_interaction / open_nodes (:1591-1694), compute_M2L (:1702-1781),
// propagate_fnode_to_node (:1527-1560) and expand_fgrav_in_taylor_series
// (:1799-1840).
//
// The reference walks, for every leaf, pairs (dst, src) in which dst runs
// down the leaf's chain of ancestors while src descends the tree; a well
// separated pair adds the M2L expansion of src to the coefficients of that
// ancestor, and the leaf's final coefficients propagate the ancestors'
// coefficients down the chain. Which src nodes meet an ancestor A depends only
// on A's own chain, so every leaf below A would compute the same sum for A
// (the reference caches it, fnodecache). Here each node's sum is computed once
// (k_grav_m2l, one warp per node), the coefficients are propagated down each
// leaf's chain (k_grav_down, one thread per leaf), and the near-field trial
// list of each leaf comes from the same dual walk (k_dual_walk). Pair
// decisions use FP32 bounds with an exact FP64 fallback, so trial lists are
// the reference's.
#include <type_traits>

#include <algorithm>

#include "ph_internal.h"
#include "ph_walk.cuh"

namespace ph {

constexpr int MAXBRANCH = 96;
constexpr int DUAL_STK = 1024;

// get_sep of two node centres (kdtree.F90:1468-1501), dx = x_dst - x_src
__device__ __forceinline__ void node_sep(const Params &p, double xd, double yd, double zd, double xs, double ys,
                                        double zs, double &dx, double &dy, double &dz, int &code) {
  dx = dsub(xd, xs); dy = dsub(yd, ys); dz = dsub(zd, zs);
  code = 0;
  if (p.periodic) {
    if (fabs(dx) > p.hdlx) { double o = dmul(p.dxbound, sign1(dx)); dx = dsub(dx, o); code |= (o > 0 ? 1 : 2); }
    if (fabs(dy) > p.hdly) { double o = dmul(p.dybound, sign1(dy)); dy = dsub(dy, o); code |= (o > 0 ? 1 : 2) << 2; }
    if (fabs(dz) > p.hdlz) { double o = dmul(p.dzbound, sign1(dz)); dz = dsub(dz, o); code |= (o > 0 ? 1 : 2) << 4; }
  }
}

// node_interaction (kdtree.F90:1653-1694): whether (dst, src) must be opened,
// i.e. is not well separated, in the reference's FP64 rounding
__device__ __forceinline__ bool pair_open_exact(const Params &p, const Node &d, const Node &s, double tree_acc2,
                                                int &code) {
  double dx, dy, dz;
  node_sep(p, d.x, d.y, d.z, s.x, s.y, s.z, dx, dy, dz, code);
  const double r2 = r2_exact(dx, dy, dz);
  const double rcut = fmax(dmul(d.hmax, RADKERN), dmul(s.hmax, RADKERN));
  const double t = dadd(dadd(d.size, s.size), rcut);
  const double s2 = dadd(d.size, s.size);
  const bool wellsep = (dmul(tree_acc2, r2) > dmul(s2, s2)) && (r2 > dmul(t, t));
  return !wellsep;
}

// the same decision on the FP32 mirrors with error bounds (as node_open in
// the leaf walk); undecidable pairs are repeated exactly
__device__ __forceinline__ bool pair_open(const Params &p, const NodeF &d, const NodeF &s, const Node *__restrict__ nodes,
                                          int id, int is, double tree_acc2, float tacc2f, int &code) {
  const float E0 = 2.384185791015625e-07f;  // 2^-22
  float dx = d.x - s.x, dy = d.y - s.y, dz = d.z - s.z;
  float ex = E0 * (fabsf(d.x) + fabsf(s.x)), ey = E0 * (fabsf(d.y) + fabsf(s.y)), ez = E0 * (fabsf(d.z) + fabsf(s.z));
  code = 0;
  bool amb = false;
  if (p.periodic) {
    const float hx = 0.5f * p.dxboundf, hy = 0.5f * p.dyboundf, hz = 0.5f * p.dzboundf;
    const float bx = ex + E0 * hx, by = ey + E0 * hy, bz = ez + E0 * hz;
    if (fabsf(dx) > hx + bx) {
      const float o = copysignf(p.dxboundf, dx); dx -= o; code |= (o > 0.0f ? 1 : 2); ex += E0 * p.dxboundf;
    } else if (fabsf(dx) >= hx - bx) amb = true;
    if (fabsf(dy) > hy + by) {
      const float o = copysignf(p.dyboundf, dy); dy -= o; code |= (o > 0.0f ? 1 : 2) << 2; ey += E0 * p.dyboundf;
    } else if (fabsf(dy) >= hy - by) amb = true;
    if (fabsf(dz) > hz + bz) {
      const float o = copysignf(p.dzboundf, dz); dz -= o; code |= (o > 0.0f ? 1 : 2) << 4; ez += E0 * p.dzboundf;
    } else if (fabsf(dz) >= hz - bz) amb = true;
  }
  if (!amb) {
    const float lx = fmaxf(fabsf(dx) - ex, 0.0f), ly = fmaxf(fabsf(dy) - ey, 0.0f), lz = fmaxf(fabsf(dz) - ez, 0.0f);
    const float ux = fabsf(dx) + ex, uy = fabsf(dy) + ey, uz = fabsf(dz) + ez;
    const float lb = (lx * lx + ly * ly + lz * lz) * (1.0f - 1.0e-5f);
    const float ub = (ux * ux + uy * uy + uz * uz) * (1.0f + 1.0e-5f);
    const float s2 = d.size + s.size;
    const float t = s2 + 2.0f * fmaxf(d.hmax, s.hmax);
    const float slo = s2 * (1.0f - 1.0e-5f), shi = s2 * (1.0f + 1.0e-5f);
    const float tlo = t * (1.0f - 1.0e-5f), thi = t * (1.0f + 1.0e-5f);
    // wellsep = (tacc2 r2 > s2^2) .and. (r2 > t^2)
    const int a = (tacc2f * lb > shi * shi) ? 1 : ((tacc2f * ub < slo * slo) ? 0 : 2);
    const int b = (lb > thi * thi) ? 1 : ((ub < tlo * tlo) ? 0 : 2);
    if (a == 0 || b == 0) return true;
    if (a == 1 && b == 1) return false;
  }
  const Node nd = nodes[id], ns = nodes[is];
  return pair_open_exact(p, nd, ns, tree_acc2, code);
}

// chain of ancestors: branch[0] = node, branch[nbr - 1] = root
__device__ __forceinline__ int build_branch(const Node *__restrict__ nodes, int node, int *branch) {
  int nbr = 0, j = node;
  while (j >= 0 && nbr < MAXBRANCH) { branch[nbr++] = j; j = nodes[j].parent; }
  return j >= 0 ? -1 : nbr;
}

// ------------------------------------------------------------------ M2L sums per node
// compute_M2L (kdtree.F90:1702-1781): adds the p=3 expansion about the dst
// centre of a src node's monopole + quadrupole field, dx = x_dst - x_src
// The 20 terms are handed to sink(k, value) in order: k = 0..2 force, 3..8
// its gradient, 9..18 second derivatives, 19 potential.
template <typename T, class Sink>
__device__ __forceinline__ void m2l_terms(T dx, T dy, T dz, T dr1, T q0, const T *qd, Sink &&sink) {
  const T dr12 = dr1 * dr1;
  const T dx2 = dx * dx, dx3 = dx * dx2, dy2 = dy * dy, dy3 = dy * dy2, dz2 = dz * dz, dz3 = dz * dz2;
  const T g0 = -dr1;
  const T g1 = dr12 * g0;
  const T g2 = T(-3) * dr12 * g1;
  const T g3 = T(-5) * dr12 * g2;
  const T g2dx = g2 * dx, g2dy = g2 * dy, g2dz = g2 * dz;
  T D3[10], D2[6], D1[3];
  D3[0] = T(3) * g2dx + g3 * dx3;
  D3[1] = g2dy + g3 * dx2 * dy;
  D3[2] = g2dz + g3 * dx2 * dz;
  D3[3] = g2dx + g3 * dy2 * dx;
  D3[4] = g3 * dx * dy * dz;
  D3[5] = g2dx + g3 * dz2 * dx;
  D3[6] = T(3) * g2dy + g3 * dy3;
  D3[7] = g2dz + g3 * dy2 * dz;
  D3[8] = g2dy + g3 * dz2 * dy;
  D3[9] = T(3) * g2dz + g3 * dz3;
  D2[0] = g1 + g2 * dx2; D2[1] = g2dx * dy; D2[2] = g2dx * dz;
  D2[3] = g1 + g2 * dy2; D2[4] = g2dy * dz; D2[5] = g1 + g2 * dz2;
  D1[0] = g1 * dx; D1[1] = g1 * dy; D1[2] = g1 * dz;
  const T qxx = qd[0], qxy = qd[1], qxz = qd[2], qyy = qd[3], qyz = qd[4], qzz = qd[5];
  const T h = T(0.5);
  sink(0, D1[0] * q0 + h * (D3[0] * qxx + T(2) * (D3[1] * qxy + D3[2] * qxz + D3[4] * qyz) + D3[3] * qyy + D3[5] * qzz));
  sink(1, D1[1] * q0 + h * (D3[1] * qxx + T(2) * (D3[3] * qxy + D3[4] * qxz + D3[7] * qyz) + D3[6] * qyy + D3[8] * qzz));
  sink(2, D1[2] * q0 + h * (D3[2] * qxx + T(2) * (D3[4] * qxy + D3[5] * qxz + D3[8] * qyz) + D3[7] * qyy + D3[9] * qzz));
  for (int k = 0; k < 6; ++k) sink(3 + k, D2[k] * q0);
  for (int k = 0; k < 10; ++k) sink(9 + k, D3[k] * q0);
  sink(19, g0 * q0 - h * (D2[0] * qxx + D2[3] * qyy + D2[5] * qzz + T(2) * (D2[1] * qxy + D2[2] * qxz + D2[4] * qyz)));
}
template <typename T>
__device__ __forceinline__ void m2l(T dx, T dy, T dz, T dr1, T q0, const T *qd, T *f) {
  m2l_terms(dx, dy, dz, dr1, q0, qd, [&](int k, T v) { f[k] += v; });
}

struct M2LShared {
  int2 stk[DUAL_STK];
  int branch[MAXBRANCH];
  int pend[96];
};

// The dual walk for node A down A's chain (sh.branch[0, nbr), A first) to
// A's level, where the well-separated src nodes are collected in sh.pend and
// handed to flush(cnt) (sh.pend[0, cnt), up to 32 at a time). Returns false
// when the stack overflowed.
template <class Flush>
__device__ __forceinline__ bool m2l_walk(const Params &p, const Node *nodes, const NodeF *nodesf, int root, int nbr,
                                         bool aleaf, M2LShared &sh, Flush &&flush) {
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id();
  const double tree_acc2 = p.tree_accuracy * p.tree_accuracy;
  const float tacc2f = (float)tree_acc2;
  if (lane == 0) sh.stk[0] = make_int2(root, nbr);
  __syncwarp();
  int top = 1, npend = 0;
  while (top > 0) {
    const int k = min(32, top);
    int2 e = make_int2(-1, 0);
    if (lane < k) e = sh.stk[top - k + lane];
    top -= k;
    __syncwarp();
    bool rec = false;
    int npush = 0, c0 = -1, c1 = -1, ibn = 0;
    if (e.x >= 0) {
      const int src = e.x, ib = e.y;
      const int dst = sh.branch[ib - 1];
      bool open = true;
      int code = 0;
      if (dst != src) open = pair_open(p, nodesf[dst], nodesf[src], nodes, dst, src, tree_acc2, tacc2f, code);
      if (ib == 1) {
        // A's level: well separated -> M2L. Opened pairs stop there for an
        // internal A (their children meet A's children); for a leaf A the
        // reference keeps descending src against A itself (open_nodes with
        // isdstleaf), so an opened internal src pushes its children again.
        rec = !open;
        if (open && aleaf) {
          const NodeF sf = nodesf[src];
          if (sf.left >= 0) { npush = 2; c0 = sf.left; c1 = sf.right; ibn = 1; }
        }
      } else if (open) {
        ibn = ib - 1;
        const NodeF sf = nodesf[src];
        if (sf.left < 0) { npush = 1; c0 = src; }
        else { npush = 2; c0 = sf.left; c1 = sf.right; }
      }
    }
    const unsigned br = __ballot_sync(FULL, rec);
    if (rec) sh.pend[npend + __popc(br & ((1u << lane) - 1))] = e.x;
    npend += __popc(br);
    int pos = npush;
    for (int o = 1; o < 32; o <<= 1) { const int y = __shfl_up_sync(FULL, pos, o); if (lane >= o) pos += y; }
    const int tot = __shfl_sync(FULL, pos, 31);
    pos -= npush;
    if (top + tot > DUAL_STK) return false;
    if (npush >= 1) sh.stk[top + pos] = make_int2(c0, ibn);
    if (npush == 2) sh.stk[top + pos + 1] = make_int2(c1, ibn);
    top += tot;
    __syncwarp();
    if (npend >= 32) {
      flush(32);
      __syncwarp();
      for (int q = 32 + lane; q < npend; q += 32) sh.pend[q - 32] = sh.pend[q];
      npend -= 32;
      __syncwarp();
    }
  }
  flush(npend);
  return true;
}

// the node id of enumeration index w: big ids first, then node_list
__device__ __forceinline__ int node_at(int w, int nbig, const int *node_list) {
  return w < nbig ? w : node_list[w - nbig];
}

// One warp per node A (ids [0, nbig) and node_list[0, nsmall)): the dual
// walk down A's chain to A's level, where the well-separated src nodes
// contribute their M2L expansion to fb[A]. Lanes evaluate the M2L terms
// of 32 pending src nodes at a time (FP64, or FP32 in the mixed form) and the
// lane sums are combined in FP64.
template <bool MIXED>
__global__ void __launch_bounds__(32) k_grav_m2l(Params p, const Node *nodes, const NodeF *nodesf, int root,
                                                 int nbig, const int *node_list, int nsmall, const double *nmass,
                                                 const double *nquads, double *fb, int *err) {
  __shared__ M2LShared sh;
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id();
  const int w = blockIdx.x;
  if (w >= nbig + nsmall) return;
  const int A = node_at(w, nbig, node_list);
  if (lane == 0) {
    const int nbr = build_branch(nodes, A, sh.branch);
    sh.pend[0] = nbr;
  }
  __syncwarp();
  const int nbr = sh.pend[0];
  __syncwarp();
  if (nbr <= 0) { if (lane == 0) set_error(err, PH_ERR_STACK); return; }
  const Node na = nodes[A];
  typedef typename std::conditional<MIXED, float, double>::type T;
  T acc[LENFG];
  for (int k = 0; k < LENFG; ++k) acc[k] = T(0);
  auto flush = [&](int cnt) {
    if (lane < cnt) {
      const int s = sh.pend[lane];
      const Node ns = nodes[s];
      double dx, dy, dz;
      int code;
      node_sep(p, na.x, na.y, na.z, ns.x, ns.y, ns.z, dx, dy, dz, code);
      const double r2 = r2_exact(dx, dy, dz);
      const double dr1 = 1.0 / sqrt(r2);
      T qd[6];
      for (int k = 0; k < 6; ++k) qd[k] = (T)nquads[6 * (size_t)s + k];
      m2l<T>((T)dx, (T)dy, (T)dz, (T)dr1, (T)nmass[s], qd, acc);
    }
  };
  if (!m2l_walk(p, nodes, nodesf, root, nbr, na.left < 0, sh, flush)) {
    if (lane == 0) set_error(err, PH_ERR_STACK);
    return;
  }
  for (int k = 0; k < LENFG; ++k) {
    double v = (double)acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    if (lane == 0) fb[LENFG * (size_t)A + k] = v;
  }
}

// ------------------------------------------------------------------ downward pass
// propagate_fnode_to_node (kdtree.F90:1527-1560): the expansion s about a
// parent centre, re-expanded about a point displaced by (dx, dy, dz)
__device__ __forceinline__ void propagate(double *f, const double *s, double dx, double dy, double dz) {
  f[0] = s[0] + dx * (s[3] + 0.5 * (dx * s[9] + dy * s[10] + dz * s[11]))
              + dy * (s[4] + 0.5 * (dx * s[10] + dy * s[12] + dz * s[13]))
              + dz * (s[5] + 0.5 * (dx * s[11] + dy * s[13] + dz * s[14]));
  f[1] = s[1] + dx * (s[4] + 0.5 * (dx * s[10] + dy * s[12] + dz * s[13]))
              + dy * (s[6] + 0.5 * (dx * s[12] + dy * s[15] + dz * s[16]))
              + dz * (s[7] + 0.5 * (dx * s[13] + dy * s[16] + dz * s[17]));
  f[2] = s[2] + dx * (s[5] + 0.5 * (dx * s[11] + dy * s[13] + dz * s[14]))
              + dy * (s[7] + 0.5 * (dx * s[13] + dy * s[16] + dz * s[17]))
              + dz * (s[8] + 0.5 * (dx * s[14] + dy * s[17] + dz * s[18]));
  f[3] = s[3] + dx * s[9] + dy * s[10] + dz * s[11];
  f[4] = s[4] + dx * s[10] + dy * s[12] + dz * s[13];
  f[5] = s[5] + dx * s[11] + dy * s[13] + dz * s[14];
  f[6] = s[6] + dx * s[12] + dy * s[15] + dz * s[16];
  f[7] = s[7] + dx * s[13] + dy * s[16] + dz * s[17];
  f[8] = s[8] + dx * s[14] + dy * s[17] + dz * s[18];
  for (int k = 9; k < 19; ++k) f[k] = s[k];
  f[19] = s[19] + dx * (s[0] + 0.5 * (dx * s[3] + dy * s[4] + dz * s[5]))
                + dy * (s[1] + 0.5 * (dx * s[4] + dy * s[6] + dz * s[7]))
                + dz * (s[2] + 0.5 * (dx * s[5] + dy * s[7] + dz * s[8]));
}

// One thread per leaf: coefficients of the leaf = the chain's sums propagated
// from the root down (getneigh_dual downward pass, kdtree.F90:1427-1459);
// also the leaf index of each of its particles
__global__ void k_grav_down(Params p, const Node *nodes, const int *leaves, int nleaves, const double *fb,
                            double *gleaf, int *leaf_of, int *err) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nleaves) return;
  const int leaf = leaves[l];
  int chain[MAXBRANCH];
  const int nbr = build_branch(nodes, leaf, chain);
  if (nbr <= 0) { set_error(err, PH_ERR_STACK); return; }
  double g[LENFG], f[LENFG];
  for (int k = 0; k < LENFG; ++k) g[k] = fb[LENFG * (size_t)chain[nbr - 1] + k];
  for (int i = nbr - 1; i >= 1; --i) {
    const Node a = nodes[chain[i]], b = nodes[chain[i - 1]];
    double dx, dy, dz;
    int code;
    node_sep(p, b.x, b.y, b.z, a.x, a.y, a.z, dx, dy, dz, code);
    propagate(f, g, dx, dy, dz);
    const double *fc = fb + LENFG * (size_t)chain[i - 1];
    for (int k = 0; k < LENFG; ++k) g[k] = f[k] + fc[k];
  }
  for (int k = 0; k < LENFG; ++k) gleaf[LENFG * (size_t)l + k] = g[k];
  const Node nl = nodes[leaf];
  for (int q = 0; q < nl.count; ++q) leaf_of[nl.start + q] = l;
}

// ------------------------------------------------------------------ leaf trial lists
struct DualShared {
  int2 stk[DUAL_STK];
  int branch[MAXBRANCH];
  LeafEntry em[WALK_EM];
  int nbr;
};

// getneigh_dual's trial list of one leaf cell per warp: src leaves reached at
// the leaf's own level without being well separated, in descending order of
// their first particle (the order of the reference's right-first pops)
__global__ void __launch_bounds__(32) k_dual_walk(Params p, const Node *nodes, const NodeF *nodesf, int root,
                                                  const int *leaves, int ncell, LeafEntry *pool, long long pool_cap,
                                                  unsigned long long *pool_top, int *cell_off, int *cell_nleaf,
                                                  int *cell_ntrial, int *err) {
  __shared__ DualShared sh;
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id();
  const int cell = blockIdx.x;
  if (cell >= ncell) return;
  const int leaf = leaves[cell];
  if (lane == 0) sh.nbr = build_branch(nodes, leaf, sh.branch);
  __syncwarp();
  const int nbr = sh.nbr;
  if (nbr <= 0) { if (lane == 0) set_error(err, PH_ERR_STACK); return; }
  const double tree_acc2 = p.tree_accuracy * p.tree_accuracy;
  const float tacc2f = (float)tree_acc2;
  if (lane == 0) sh.stk[0] = make_int2(root, nbr);
  __syncwarp();
  int top = 1, nem = 0;
  bool overflow = false;
  while (top > 0) {
    const int k = min(32, top);
    int2 e = make_int2(-1, 0);
    if (lane < k) e = sh.stk[top - k + lane];
    top -= k;
    __syncwarp();
    bool emit = false;
    LeafEntry le{0, 0};
    int npush = 0, c0 = -1, c1 = -1, ibn = 0;
    if (e.x >= 0) {
      const int src = e.x, ib = e.y;
      const int dst = sh.branch[ib - 1];
      bool open = true;
      int code = 0;
      if (dst != src) open = pair_open(p, nodesf[dst], nodesf[src], nodes, dst, src, tree_acc2, tacc2f, code);
      if (open) {  // open_nodes (kdtree.F90:1591-1645)
        const bool dstleaf = ib - 1 <= 0;
        ibn = dstleaf ? ib : ib - 1;
        const NodeF sf = nodesf[src];
        if (sf.left < 0) {
          if (dstleaf) { emit = true; le.start = sf.right; le.cc = sf.count | (code << 8); }
          else { npush = 1; c0 = src; }
        } else { npush = 2; c0 = sf.left; c1 = sf.right; }
      }
    }
    const unsigned be = __ballot_sync(FULL, emit);
    if (emit) {
      const int pos = nem + __popc(be & ((1u << lane) - 1));
      if (pos < WALK_EM) sh.em[pos] = le;
    }
    nem += __popc(be);
    int pos = npush;
    for (int o = 1; o < 32; o <<= 1) { const int y = __shfl_up_sync(FULL, pos, o); if (lane >= o) pos += y; }
    const int tot = __shfl_sync(FULL, pos, 31);
    pos -= npush;
    if (top + tot > DUAL_STK || nem > WALK_EM) { overflow = true; break; }
    if (npush >= 1) sh.stk[top + pos] = make_int2(c0, ibn);
    if (npush == 2) sh.stk[top + pos + 1] = make_int2(c1, ibn);
    top += tot;
    __syncwarp();
  }
  if (overflow) { if (lane == 0) set_error(err, PH_ERR_STACK); return; }
  __syncwarp();
  int tot = 0;
  for (int e = lane; e < nem; e += 32) tot += sh.em[e].cc & 255;
  tot = warp_sum_int(tot);
  unsigned long long off = 0;
  if (lane == 0) off = atomicAdd(pool_top, (unsigned long long)nem);
  off = __shfl_sync(FULL, off, 0);
  if ((long long)(off + nem) > pool_cap) { if (lane == 0) set_error(err, PH_ERR_LIST); return; }
  write_ranked(sh.em, nem, pool, off);
  if (lane == 0) { cell_off[cell] = (int)off; cell_nleaf[cell] = nem; cell_ntrial[cell] = tot; }
}

static inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }

// ------------------------------------------------------------------ level by level
// The same dual walk level by level. For a node X the candidates at X's level
// are the expansion of the src nodes opened against X's parent (a leaf src
// stays itself, an internal one gives its two children; the root starts from
// itself): exactly the pairs the walk from the root meets at X's level. A
// well-separated candidate adds its M2L term to fb[X]; an opened one joins
// X's opened list (internal X), or, for a leaf X, descends further against X
// (internal src) or becomes a near-field trial leaf (leaf src), as in
// k_grav_m2l and k_dual_walk. Each node tests only its parent's expanded
// list instead of walking its whole chain from the root. A buffer or pool
// that overflows sets flag[0]; the caller then uses the walks from the root.
constexpr int OBUF = 2 * WALK_EM;  // opened-list buffer per warp (ints), the near entries of a leaf alias it

struct LevelShared {
  int stk[DUAL_STK];
  int pend[96];
  union {
    int obuf[OBUF];
    LeafEntry em[WALK_EM];
  } u;
};

template <bool MIXED>
__global__ void __launch_bounds__(32) k_far_level(Params p, const Node *nodes, const NodeF *nodesf, const int *lv_nodes,
                                                  int nlv, int *o_off, int *o_len, int *opool, long long opool_cap,
                                                  unsigned long long *opool_top, const double *nmass,
                                                  const double *nquads, const float4 *mqf, double *fb,
                                                  const int *cell_of_node,
                                                  LeafEntry *pool, long long pool_cap,
                                                  unsigned long long *pool_top, int *cell_off, int *cell_nleaf,
                                                  int *cell_ntrial, int *flag, int *err) {
  __shared__ LevelShared sh;
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id();
  const int w = blockIdx.x;
  if (w >= nlv) return;
  const int X = lv_nodes[w];
  const Node na = nodes[X];
  const bool xleaf = na.left < 0;
  const double tree_acc2 = p.tree_accuracy * p.tree_accuracy;
  const float tacc2f = (float)tree_acc2;
  typedef typename std::conditional<MIXED, float, double>::type T;
  T acc[LENFG];
  for (int k = 0; k < LENFG; ++k) acc[k] = T(0);
  auto flush = [&](int cnt) {
    if (lane < cnt) {
      const int s = sh.pend[lane];
      const Node ns = nodes[s];
      double dx, dy, dz;
      int code;
      node_sep(p, na.x, na.y, na.z, ns.x, ns.y, ns.z, dx, dy, dz, code);
      if constexpr (MIXED) {
        // the separation formed in FP64, rounded on the integer pipe; 1/r,
        // mass and quadrupole in FP32 (the FP32 mirror of the node moments)
        const float fx = d2f_rn(dx), fy = d2f_rn(dy), fz = d2f_rn(dz);
        const float dr1 = rsqrt_nr(fx * fx + fy * fy + fz * fz);
        const float4 m0 = mqf[2 * (size_t)s], m1 = mqf[2 * (size_t)s + 1];
        const float qd[6] = {m0.y, m0.z, m0.w, m1.x, m1.y, m1.z};
        m2l<float>(fx, fy, fz, dr1, m0.x, qd, acc);
      } else {
        const double r2 = r2_exact(dx, dy, dz);
        const double dr1 = 1.0 / sqrt(r2);
        double qd[6];
        for (int k = 0; k < 6; ++k) qd[k] = nquads[6 * (size_t)s + k];
        m2l<double>(dx, dy, dz, dr1, nmass[s], qd, acc);
      }
    }
  };
  int pbeg = 0, plen = 0, top = 0;
  if (na.parent >= 0) {
    pbeg = o_off[na.parent];
    plen = o_len[na.parent];
  } else {
    if (lane == 0) sh.stk[0] = X;
    top = 1;
  }
  __syncwarp();
  int pnext = 0, npend = 0, nob = 0;
  const int obcap = xleaf ? WALK_EM : OBUF;
  bool overflow = false;
  for (;;) {
    if (top < 64 && pnext < plen) {  // refill from the parent's opened list
      const int kk = min(32, plen - pnext);
      int ne = 0, c0 = -1, c1 = -1;
      if (lane < kk) {
        const int s = opool[pbeg + pnext + lane];
        const NodeF sf = nodesf[s];
        if (sf.left < 0) { ne = 1; c0 = s; }
        else { ne = 2; c0 = sf.left; c1 = sf.right; }
      }
      int pos = ne;
      for (int o = 1; o < 32; o <<= 1) { const int y = __shfl_up_sync(FULL, pos, o); if (lane >= o) pos += y; }
      const int tot = __shfl_sync(FULL, pos, 31);
      pos -= ne;
      if (top + tot > DUAL_STK) { overflow = true; break; }
      if (ne >= 1) sh.stk[top + pos] = c0;
      if (ne == 2) sh.stk[top + pos + 1] = c1;
      top += tot;
      pnext += kk;
      __syncwarp();
    }
    if (top == 0) break;
    const int k = min(32, top);
    int src = -1;
    if (lane < k) src = sh.stk[top - k + lane];
    top -= k;
    __syncwarp();
    bool rec = false, keep = false;
    int npush = 0, d0 = -1, d1 = -1, kv = 0;
    if (src >= 0) {
      int code = 0;
      bool open = true;
      if (src != X) open = pair_open(p, nodesf[X], nodesf[src], nodes, X, src, tree_acc2, tacc2f, code);
      if (!open) {
        rec = true;
      } else if (!xleaf) {
        keep = true; kv = src;
      } else {
        const NodeF sf = nodesf[src];
        if (sf.left < 0) { keep = true; kv = src; d0 = code; }  // near-field trial leaf (d0: offset code)
        else { npush = 2; d0 = sf.left; d1 = sf.right; }
      }
    }
    const unsigned br = __ballot_sync(FULL, rec);
    if (rec) sh.pend[npend + __popc(br & ((1u << lane) - 1))] = src;
    npend += __popc(br);
    const unsigned bk = __ballot_sync(FULL, keep);
    if (keep) {
      const int pos = nob + __popc(bk & ((1u << lane) - 1));
      if (pos < obcap) {
        if (xleaf) {
          const NodeF sf = nodesf[kv];
          LeafEntry le; le.start = sf.right; le.cc = sf.count | (d0 << 8);
          sh.u.em[pos] = le;
        } else {
          sh.u.obuf[pos] = kv;
        }
      }
    }
    nob += __popc(bk);
    int pos = npush;
    for (int o = 1; o < 32; o <<= 1) { const int y = __shfl_up_sync(FULL, pos, o); if (lane >= o) pos += y; }
    const int tot = __shfl_sync(FULL, pos, 31);
    pos -= npush;
    if (top + tot > DUAL_STK || nob > obcap) { overflow = true; break; }
    if (npush == 2) { sh.stk[top + pos] = d0; sh.stk[top + pos + 1] = d1; }
    top += tot;
    __syncwarp();
    if (npend >= 32) {
      flush(32);
      __syncwarp();
      for (int q = 32 + lane; q < npend; q += 32) sh.pend[q - 32] = sh.pend[q];
      npend -= 32;
      __syncwarp();
    }
  }
  if (overflow) { if (lane == 0) atomicOr(flag, 1); return; }
  flush(npend);
  for (int k = 0; k < LENFG; ++k) {
    // lane sums in the evaluation's type (FP32 in the mixed form: a lane-wide
    // FP64 reduction would cost the FP64 pipe more than the M2L terms do)
    T v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    if (lane == 0) fb[LENFG * (size_t)X + k] = (double)v;
  }
  __syncwarp();
  if (!xleaf) {
    unsigned long long off = 0;
    if (lane == 0) off = atomicAdd(opool_top, (unsigned long long)nob);
    off = __shfl_sync(FULL, off, 0);
    if ((long long)(off + nob) > opool_cap) { if (lane == 0) atomicOr(flag, 1); return; }
    for (int e = lane; e < nob; e += 32) opool[off + e] = sh.u.obuf[e];
    if (lane == 0) { o_off[X] = (int)off; o_len[X] = nob; }
    return;
  }
  // a leaf: its near-field trial list, ranked as the walk from the root
  const int cell = cell_of_node[X];
  int tot = 0;
  for (int e = lane; e < nob; e += 32) tot += sh.u.em[e].cc & 255;
  tot = warp_sum_int(tot);
  unsigned long long off = 0;
  if (lane == 0) off = atomicAdd(pool_top, (unsigned long long)nob);
  off = __shfl_sync(FULL, off, 0);
  if ((long long)(off + nob) > pool_cap) { if (lane == 0) set_error(err, PH_ERR_LIST); return; }
  write_ranked(sh.u.em, nob, pool, off);
  if (lane == 0) { cell_off[cell] = (int)off; cell_nleaf[cell] = nob; cell_ntrial[cell] = tot; }
}

// FP32 mirror of the node moments for the mixed form's M2L terms: mass and
// quadrupole (xx, xy, xz, yy, yz, zz), two float4 per node id
__global__ void k_moments_f32(int nbig, const int *node_list, int nsmall, const double *nmass, const double *nquads,
                              float4 *mqf) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nbig + nsmall) return;
  const int a = w < nbig ? w : node_list[w - nbig];
  const double *q = nquads + 6 * (size_t)a;
  mqf[2 * (size_t)a] = make_float4(d2f_rn(nmass[a]), d2f_rn(q[0]), d2f_rn(q[1]), d2f_rn(q[2]));
  mqf[2 * (size_t)a + 1] = make_float4(d2f_rn(q[3]), d2f_rn(q[4]), d2f_rn(q[5]), 0.0f);
}

// depth of every node of the enumeration (big ids, then node_list) and the
// histogram of depths
__global__ void k_node_depth(const Node *nodes, int nbig, const int *node_list, int nsmall, int *depth, int *hist,
                             int *err) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nbig + nsmall) return;
  int j = w < nbig ? w : node_list[w - nbig];
  int d = 0;
  while (nodes[j].parent >= 0 && d < MAXBRANCH) { j = nodes[j].parent; ++d; }
  if (d >= MAXBRANCH) { set_error(err, PH_ERR_STACK); d = MAXBRANCH - 1; }
  depth[w] = d;
  atomicAdd(&hist[d], 1);
}
__global__ void k_level_scatter(int nbig, const int *node_list, int nsmall, const int *depth, int *cursor,
                                int *lv_nodes) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nbig + nsmall) return;
  lv_nodes[atomicAdd(&cursor[depth[w]], 1)] = w < nbig ? w : node_list[w - nbig];
}
__global__ void k_cell_of_node(const int *leaves, int ncell, int *cell_of_node) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell < ncell) cell_of_node[leaves[cell]] = cell;
}

// The far field (fb per node) and the leaf trial lists level by level.
// Returns 0, -1 when a buffer or the opened-list pool overflowed (the caller
// then uses the walks from the root; the pool is doubled for the next build),
// or an error code.
int far_levels(ph_ctx *c) {
  cudaStream_t st = c->stream;
  const Params p = c->dp;
  const int nn = c->nbig_nodes + c->nsmall_nodes;
  const int ncell = c->nleaves;
  static_assert(LV_MAXDEPTH == MAXBRANCH, "level arrays sized by the walks' chain limit");
  if (alloc_levels(c, std::max<int64_t>(128ll * nn, c->opool_cap)) != 0) return PH_ERR_CUDA;
  int *hist = c->lv_hist, *cursor = c->lv_hist + (MAXBRANCH + 1);
  cudaMemsetAsync(hist, 0, sizeof(int) * (MAXBRANCH + 1), st);
  cudaMemsetAsync(c->lv_flag, 0, sizeof(int), st);
  cudaMemsetAsync(c->counters + 16, 0, sizeof(unsigned long long), st);  // opened-list pool top
  k_node_depth<<<nblk(nn, 256), 256, 0, st>>>(c->nodes, c->nbig_nodes, c->node_list, c->nsmall_nodes, c->lv_depth,
                                             hist, c->d_err);
  int h[MAXBRANCH + 1];
  cudaMemcpyAsync(h, hist, sizeof(h), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  int off[MAXBRANCH + 1];
  int acc = 0, nlev = 0;
  for (int d = 0; d <= MAXBRANCH; ++d) { off[d] = acc; acc += h[d]; if (h[d]) nlev = d + 1; }
  cudaMemcpyAsync(cursor, off, sizeof(off), cudaMemcpyHostToDevice, st);
  k_level_scatter<<<nblk(nn, 256), 256, 0, st>>>(c->nbig_nodes, c->node_list, c->nsmall_nodes, c->lv_depth, cursor,
                                                c->lv_nodes);
  k_cell_of_node<<<nblk(ncell, 256), 256, 0, st>>>(c->leaves, ncell, c->cell_of_node);
  count_launch(c, 3);
  if (p.precision == PH_PREC_MIXED) {
    k_moments_f32<<<nblk(nn, 256), 256, 0, st>>>(c->nbig_nodes, c->node_list, c->nsmall_nodes, c->nmass, c->nquads,
                                                 c->mqf);
    count_launch(c, 1);
  }
  unsigned long long *otop = reinterpret_cast<unsigned long long *>(c->counters + 16);
  for (int d = 0; d < nlev; ++d) {
    if (h[d] == 0) continue;
#define PH_FAR_LEVEL(M)                                                                                          \
  k_far_level<M><<<h[d], 32, 0, st>>>(p, c->nodes, c->nodesf, c->lv_nodes + off[d], h[d], c->o_off, c->o_len,      \
                                      c->opool, c->opool_cap, otop, c->nmass, c->nquads, c->mqf, c->fb,            \
                                      c->cell_of_node,                                                             \
                                      c->pool, c->pool_cap, c->pool_top, c->cell_off, c->cell_nleaf,              \
                                      c->cell_ntrial, c->lv_flag, c->d_err)
    if (p.precision == PH_PREC_MIXED) PH_FAR_LEVEL(true);
    else PH_FAR_LEVEL(false);
#undef PH_FAR_LEVEL
    count_launch(c, 1);
  }
  int fl = 0;
  cudaMemcpyAsync(&fl, c->lv_flag, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  if (!fl) return 0;
  if (alloc_levels(c, 2 * c->opool_cap) != 0) return PH_ERR_CUDA;
  return -1;
}

// the downward pass: each leaf's coefficients from its chain's sums
int gravity_down(ph_ctx *c) {
  k_grav_down<<<nblk(c->nleaves, 128), 128, 0, c->stream>>>(c->dp, c->nodes, c->leaves, c->nleaves, c->fb, c->gleaf,
                                                            c->leaf_of, c->d_err);
  count_launch(c, 1);
  return 0;
}


// far-field coefficients of every leaf (per tree build and density; positions
// do not change between force evaluations of one step)
int gravity_far(ph_ctx *c) {
  cudaStream_t st = c->stream;
  const Params p = c->dp;
  const int nnodes = c->nbig_nodes + c->nsmall_nodes;
  if (p.precision == PH_PREC_MIXED)
    k_grav_m2l<true><<<nnodes, 32, 0, st>>>(p, c->nodes, c->nodesf, c->root, c->nbig_nodes, c->node_list,
                                            c->nsmall_nodes, c->nmass, c->nquads, c->fb, c->d_err);
  else
    k_grav_m2l<false><<<nnodes, 32, 0, st>>>(p, c->nodes, c->nodesf, c->root, c->nbig_nodes, c->node_list,
                                             c->nsmall_nodes, c->nmass, c->nquads, c->fb, c->d_err);
  count_launch(c, 1);
  return gravity_down(c);
}

int dual_walk(ph_ctx *c) {
  const Params p = c->dp;
  k_dual_walk<<<c->nleaves, 32, 0, c->stream>>>(p, c->nodes, c->nodesf, c->root, c->leaves, c->nleaves, c->pool,
                                                c->pool_cap, c->pool_top, c->cell_off, c->cell_nleaf,
                                                c->cell_ntrial, c->d_err);
  count_launch(c, 1);
  return 0;
}


// ------------------------------------------------------------------ adjoint of the far field
// The far-field force on particle i is its leaf's expansion g_leaf at
// d = x_i - c_leaf (expand_fgrav_in_taylor_series), g_leaf the M2L sums
// fb[X] of the leaf's chain X propagated down the chain
// (propagate_fnode_to_node). For the force terms (coefficients 0..18) both
// steps are exact translations of a quadratic polynomial, so in exact
// arithmetic
//   a_i = sum_{X in chain(i)} F(fb[X], x_i - c_X),
//   F_a(f, d) = f_a + D_ab d_b + 1/2 T_abc d_b d_c
// with D = f[3..8] and T = f[9..18] the symmetric tensors (x_i - c_X without
// a periodic wrap, which equals the chain's wrapped offsets while every node
// centre lies within half a box of its parent's). With cotangents w_i of a_i
// the reverse is
//   fbar[X] = the moments of w over the particles of X about c_X,
//   cbar[X] = -sum_{i in X} (dF/dd)^T w_i (c_X in F) + the reverse of the M2L
//             terms with X as receiver or source,
//   Qbar[X] = the reverse of the M2L terms with X as source,
//   xbar_i  = J_i^T w_i (J_i the Jacobian of the leaf's expansion at x_i)
//             + sum_{X in chain(i)} [m/M_X cbar[X] + m dQ_X/dx_i : Qbar[X]],
// for the centre of mass c_X = sum m x / M_X and the quadrupole
// Q_X = m sum (x - c_X)(x - c_X)^T (kdtree.F90:669-675, 744-752), whose
// derivative through c_X vanishes (sum m (x - c_X) = 0).
// ANODE doubles per node id: fbar[0..19], cbar[20..22], Qbar[23..28]
static_assert(ANODE >= LENFG + 9, "adjoint node record");

// slot of the symmetric pair (a, b) in xx, xy, xz, yy, yz, zz
__device__ __forceinline__ int sym2(int a, int b) {
  const int lo = min(a, b), hi = max(a, b);
  return lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
}
// slot of the symmetric triple (a, b, c) in xxx, xxy, xxz, xyy, xyz, xzz,
// yyy, yyz, yzz, zzz
__device__ __forceinline__ int sym3(int a, int b, int c) {
  const int nx = (a == 0) + (b == 0) + (c == 0), nz = (a == 2) + (b == 2) + (c == 2);
  const int base = nx == 3 ? 0 : (nx == 2 ? 1 : (nx == 1 ? 3 : 6));
  return base + nz;
}

// forward-mode derivative with respect to the three components of a
// separation (the reverse of compute_M2L in its geometry)
struct Dual3 {
  double v, x, y, z;
  __device__ Dual3() : v(0.0), x(0.0), y(0.0), z(0.0) {}
  __device__ Dual3(double a) : v(a), x(0.0), y(0.0), z(0.0) {}
  __device__ Dual3(double a, double b, double c, double d) : v(a), x(b), y(c), z(d) {}
};
__device__ __forceinline__ Dual3 operator+(const Dual3 &a, const Dual3 &b) {
  return Dual3(a.v + b.v, a.x + b.x, a.y + b.y, a.z + b.z);
}
__device__ __forceinline__ Dual3 operator-(const Dual3 &a, const Dual3 &b) {
  return Dual3(a.v - b.v, a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ Dual3 operator-(const Dual3 &a) { return Dual3(-a.v, -a.x, -a.y, -a.z); }
__device__ __forceinline__ Dual3 operator*(const Dual3 &a, const Dual3 &b) {
  return Dual3(a.v * b.v, a.x * b.v + a.v * b.x, a.y * b.v + a.v * b.y, a.z * b.v + a.v * b.z);
}
__device__ __forceinline__ Dual3 operator*(double s, const Dual3 &a) { return Dual3(s * a.v, s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ Dual3 &operator+=(Dual3 &a, const Dual3 &b) { a = a + b; return a; }

// d/dd of sum_k fbar[k] M2L_k(d, m, Q) (k < 19: the potential has no cotangent)
__device__ __forceinline__ void m2l_grad(double dx, double dy, double dz, double m, const double *q,
                                         const double *fbar, double &gx, double &gy, double &gz) {
  const Dual3 X(dx, 1.0, 0.0, 0.0), Y(dy, 0.0, 1.0, 0.0), Z(dz, 0.0, 0.0, 1.0);
  const double r2 = dx * dx + dy * dy + dz * dz;
  const double r1 = 1.0 / sqrt(r2), c = -r1 * r1 * r1;  // d(1/r)/dd = -d / r^3
  const Dual3 dr1(r1, c * dx, c * dy, c * dz);
  Dual3 qd[6];
  for (int k = 0; k < 6; ++k) qd[k] = Dual3(q[k]);
  Dual3 acc;
  m2l_terms<Dual3>(X, Y, Z, dr1, Dual3(m), qd, [&](int k, const Dual3 &v) {
    if (k < 19) acc += fbar[k] * v;
  });
  gx = acc.x; gy = acc.y; gz = acc.z;
}

// d/dQ of sum_k fbar[k] M2L_k(d, m, Q): Q enters the force terms only, as
// 1/2 D3_abc Q_bc (off-diagonal entries twice)
__device__ __forceinline__ void m2l_qgrad(double dx, double dy, double dz, const double *fbar, double *g) {
  const double r1 = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
  const double zq[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double D3[10];
  m2l_terms<double>(dx, dy, dz, r1, 1.0, zq, [&](int k, double v) {
    if (k >= 9 && k < 19) D3[k - 9] = v;
  });
  const double F0 = fbar[0], F1 = fbar[1], F2 = fbar[2];
  g[0] += 0.5 * (F0 * D3[0] + F1 * D3[1] + F2 * D3[2]);
  g[1] += F0 * D3[1] + F1 * D3[3] + F2 * D3[4];
  g[2] += F0 * D3[2] + F1 * D3[4] + F2 * D3[5];
  g[3] += 0.5 * (F0 * D3[3] + F1 * D3[6] + F2 * D3[7]);
  g[4] += F0 * D3[4] + F1 * D3[7] + F2 * D3[8];
  g[5] += 0.5 * (F0 * D3[5] + F1 * D3[8] + F2 * D3[9]);
}

// one warp per node X: moments of the cotangents w over X's particles about
// c_X -> fbar[X] and the part of cbar[X] from c_X in F (fixed-order sums)
__global__ void __launch_bounds__(128) k_adj_far_moments(int nbig, const int *node_list, int nsmall,
                                                          const Node *nodes, const double *tx, const double *ty,
                                                          const double *tz, const double *w, int wstride,
                                                          const double *fb, double *anode) {
  const int wi = blockIdx.x * 4 + (threadIdx.x >> 5), lane = lane_id();
  if (wi >= nbig + nsmall) return;
  const int X = node_at(wi, nbig, node_list);
  const Node nd = nodes[X];
  // W0[a], W1[a][b] = sum w_a d_b, W2[a][bc] = sum w_a d_b d_c (bc symmetric)
  double W[30];
  for (int k = 0; k < 30; ++k) W[k] = 0.0;
  for (int k = nd.start + lane; k < nd.start + nd.count; k += 32) {
    const double d[3] = {tx[k] - nd.x, ty[k] - nd.y, tz[k] - nd.z};
    const double *wk = w + (size_t)wstride * k;
    for (int a = 0; a < 3; ++a) {
      const double wa = wk[a];
      W[a] += wa;
      for (int b = 0; b < 3; ++b) W[3 + 3 * a + b] += wa * d[b];
      W[12 + 6 * a + 0] += wa * d[0] * d[0]; W[12 + 6 * a + 1] += wa * d[0] * d[1];
      W[12 + 6 * a + 2] += wa * d[0] * d[2]; W[12 + 6 * a + 3] += wa * d[1] * d[1];
      W[12 + 6 * a + 4] += wa * d[1] * d[2]; W[12 + 6 * a + 5] += wa * d[2] * d[2];
    }
  }
  for (int k = 0; k < 30; ++k)
    for (int o = 16; o > 0; o >>= 1) W[k] += __shfl_xor_sync(0xffffffffu, W[k], o);
  if (lane != 0) return;
  const double *f = fb + LENFG * (size_t)X;
  double *o = anode + ANODE * (size_t)X;
  double fbar[LENFG];
  for (int k = 0; k < LENFG; ++k) fbar[k] = 0.0;
  for (int a = 0; a < 3; ++a) {
    fbar[a] = W[a];
    for (int b = 0; b < 3; ++b) {
      fbar[3 + sym2(a, b)] += W[3 + 3 * a + b];
      for (int c = 0; c < 3; ++c) fbar[9 + sym3(a, b, c)] += 0.5 * W[12 + 6 * a + sym2(b, c)];
    }
  }
  for (int k = 0; k < LENFG; ++k) o[k] = fbar[k];
  for (int l = 0; l < 3; ++l) {
    double cb = 0.0;
    for (int a = 0; a < 3; ++a) {
      cb += W[a] * f[3 + sym2(a, l)];
      for (int m = 0; m < 3; ++m) cb += W[3 + 3 * a + m] * f[9 + sym3(a, l, m)];
    }
    o[20 + l] = -cb;
  }
  for (int k = 23; k < ANODE; ++k) o[k] = 0.0;
}

// one warp per node A, the walk of k_grav_m2l: for each well-separated src S
// met at A's level, the reverse of S's term in fb[A] (receiver A) and of A's
// term in fb[S] (the relation is symmetric: S meets A in S's own walk), kept
// for A's centre and quadrupole; no atomics
__global__ void __launch_bounds__(32) k_adj_m2l(Params p, const Node *nodes, const NodeF *nodesf, int root,
                                                int nbig, const int *node_list, int nsmall, const double *nmass,
                                                const double *nquads, double *anode, int *err) {
  __shared__ M2LShared sh;
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id();
  const int w = blockIdx.x;
  if (w >= nbig + nsmall) return;
  const int A = node_at(w, nbig, node_list);
  if (lane == 0) sh.pend[0] = build_branch(nodes, A, sh.branch);
  __syncwarp();
  const int nbr = sh.pend[0];
  __syncwarp();
  if (nbr <= 0) { if (lane == 0) set_error(err, PH_ERR_STACK); return; }
  const Node na = nodes[A];
  double fa[19], qa[6];
  for (int k = 0; k < 19; ++k) fa[k] = anode[ANODE * (size_t)A + k];
  for (int k = 0; k < 6; ++k) qa[k] = nquads[6 * (size_t)A + k];
  const double ma = nmass[A];
  double cb[3] = {0.0, 0.0, 0.0}, qb[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  auto flush = [&](int cnt) {
    if (lane < cnt) {
      const int s = sh.pend[lane];
      const Node ns = nodes[s];
      double dx, dy, dz;
      int code;
      node_sep(p, na.x, na.y, na.z, ns.x, ns.y, ns.z, dx, dy, dz, code);
      double qs[6], fs[19];
      for (int k = 0; k < 6; ++k) qs[k] = nquads[6 * (size_t)s + k];
      for (int k = 0; k < 19; ++k) fs[k] = anode[ANODE * (size_t)s + k];
      double gx, gy, gz;
      // A receives from S, d = c_A - c_S
      m2l_grad(dx, dy, dz, nmass[s], qs, fa, gx, gy, gz);
      cb[0] += gx; cb[1] += gy; cb[2] += gz;
      // S receives from A, d' = c_S - c_A = -d
      m2l_grad(-dx, -dy, -dz, ma, qa, fs, gx, gy, gz);
      cb[0] -= gx; cb[1] -= gy; cb[2] -= gz;
      m2l_qgrad(-dx, -dy, -dz, fs, qb);
    }
  };
  if (!m2l_walk(p, nodes, nodesf, root, nbr, na.left < 0, sh, flush)) {
    if (lane == 0) set_error(err, PH_ERR_STACK);
    return;
  }
  for (int k = 0; k < 3; ++k)
    for (int o = 16; o > 0; o >>= 1) cb[k] += __shfl_xor_sync(FULL, cb[k], o);
  for (int k = 0; k < 6; ++k)
    for (int o = 16; o > 0; o >>= 1) qb[k] += __shfl_xor_sync(FULL, qb[k], o);
  if (lane == 0) {
    double *o = anode + ANODE * (size_t)A;
    o[20] += cb[0]; o[21] += cb[1]; o[22] += cb[2];
    for (int k = 0; k < 6; ++k) o[23 + k] = qb[k];
  }
}

// one thread per tree position: the Jacobian term of the leaf's expansion
// and the chain's centre and quadrupole cotangents -> out[k * ps + ip], k < 3
__global__ void k_adj_far_dist(Params p, int nt, const Node *nodes, const int *leaves, const int *leaf_of,
                               const double *gleaf, const double *tx, const double *ty, const double *tz,
                               const double *w, int wstride, const double *nmass, const double *anode, double *out,
                               int64_t ps) {
  const int ip = blockIdx.x * blockDim.x + threadIdx.x;
  if (ip >= nt) return;
  const int l = leaf_of[ip];
  int X = leaves[l];
  const double x[3] = {tx[ip], ty[ip], tz[ip]};
  const double *wi = w + (size_t)wstride * ip;
  const double *g = gleaf + LENFG * (size_t)l;
  const Node nl = nodes[X];
  const double dl[3] = {x[0] - nl.x, x[1] - nl.y, x[2] - nl.z};
  double gx[3];
  for (int b = 0; b < 3; ++b) {
    double s = 0.0;
    for (int a = 0; a < 3; ++a) {
      double j = g[3 + sym2(a, b)];
      for (int m = 0; m < 3; ++m) j += g[9 + sym3(a, b, m)] * dl[m];
      s += wi[a] * j;
    }
    gx[b] = s;
  }
  const double pm = p.massoftype;
  for (int depth = 0; X >= 0 && depth < MAXBRANCH; ++depth) {
    const Node nd = nodes[X];
    const double *o = anode + ANODE * (size_t)X;
    const double d0 = x[0] - nd.x, d1 = x[1] - nd.y, d2 = x[2] - nd.z;
    const double s = pm / nmass[X];
    gx[0] += s * o[20] + pm * (2.0 * o[23] * d0 + o[24] * d1 + o[25] * d2);
    gx[1] += s * o[21] + pm * (o[24] * d0 + 2.0 * o[26] * d1 + o[27] * d2);
    gx[2] += s * o[22] + pm * (o[25] * d0 + o[27] * d1 + 2.0 * o[28] * d2);
    X = nd.parent;
  }
  for (int b = 0; b < 3; ++b) out[b * ps + ip] = gx[b];
}

// The far field's share of the position gradients: out[k * ps + ip] (k < 3,
// tree order) from the cotangents w (wstride doubles per tree position, the
// three acceleration cotangents first). Needs the far-field state of the
// last force evaluation (fb, gleaf, leaf_of) on the current tree.
int gravity_adjoint_far(ph_ctx *c, const double *w, int wstride, double *out, int64_t ps) {
  cudaStream_t st = c->stream;
  const Params p = c->dp;
  const int nn = c->nbig_nodes + c->nsmall_nodes;
  const int nt = (int)c->ntree;
  k_adj_far_moments<<<nblk(nn, 4), 128, 0, st>>>(c->nbig_nodes, c->node_list, c->nsmall_nodes, c->nodes, c->tx,
                                                 c->ty, c->tz, w, wstride, c->fb, c->adj_node);
  k_adj_m2l<<<nn, 32, 0, st>>>(p, c->nodes, c->nodesf, c->root, c->nbig_nodes, c->node_list, c->nsmall_nodes,
                               c->nmass, c->nquads, c->adj_node, c->d_err);
  k_adj_far_dist<<<nblk(nt, 256), 256, 0, st>>>(p, nt, c->nodes, c->leaves, c->leaf_of, c->gleaf, c->tx, c->ty,
                                                c->tz, w, wstride, c->nmass, c->adj_node, out, ps);
  count_launch(c, 3);
  return 0;
}

}  // namespace ph
