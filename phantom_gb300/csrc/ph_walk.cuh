// Leaf-cell neighbour walk (K3): getneigh (kdtree.F90:1221-1347) with
// cache_neighbours (kdtree.F90:1175-1213), one warp per leaf cell.
//
// The warp expands up to 32 stack entries at a time. The reference walk pops
// the right child first, so its trial list is the opened leaves in decreasing
// order of their first particle; each emitted leaf is written to the slot of
// its rank in that order, which reproduces the reference trial list exactly
// (including which entries fall inside the 1000-entry position cache).
#pragma once
#include "ph_common.cuh"

namespace ph {

constexpr int WALK_STK = 512;
constexpr int WALK_EM = 1024;

struct WalkShared {
  int stk[WALK_STK];
  LeafEntry em[WALK_EM];
};

// Writes the nem emitted leaves of a warp to pool[off ...] in the reference
// walk's order (descending first particle; first particles are distinct).
__device__ __forceinline__ void write_ranked(const LeafEntry *em, int nem, LeafEntry *__restrict__ pool,
                                             unsigned long long off) {
  for (int e = lane_id(); e < nem; e += 32) {
    const LeafEntry me = em[e];
    int rank = 0;
    for (int q = 0; q < nem; ++q) rank += (em[q].start > me.start) ? 1 : 0;
    pool[off + rank] = me;
  }
}

// ------------------------------------------------------------------ staging
// The trial list of a cell is a list of whole leaves. For the pair loops it is
// expanded, window by window, into a flat per-warp array in shared memory:
// the tree index of each trial particle, its periodic offset code and its FP32
// position with the offset applied (w = the caller's 4th component of txf).
// Entry k of window `base` is trial-list position n = base + k, which decides
// whether the reference would use its cached position (n < 1000).
constexpr int STAGE = 256;

template <int W>
struct StageN {
  float4 pos[W];
  int jidx[W];
  unsigned char code[W];
};
using Stage = StageN<STAGE>;

template <int W>
__device__ __forceinline__ int stage_window_n(const Params &p, const LeafEntry *__restrict__ pool, int off,
                                              int nleaf, int ntrial, int base, const float4 *__restrict__ txf,
                                              StageN<W> &st) {
  const int lane = lane_id();
  const int end = min(ntrial, base + W);
  int acc = 0;
  for (int e0 = 0; e0 < nleaf && acc < end; e0 += 32) {
    const int e = e0 + lane;
    LeafEntry le{0, 0};
    if (e < nleaf) le = pool[off + e];
    const int jc = le.cc & 255;
    int x = jc;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    const int n_first = acc + x - jc;
    if (jc > 0 && n_first < end && n_first + jc > base) {
      const int code = le.cc >> 8;
      const float ox = offset_of_f(code, 0, p.dxboundf), oy = offset_of_f(code, 1, p.dyboundf),
                  oz = offset_of_f(code, 2, p.dzboundf);
      for (int t = 0; t < jc; ++t) {
        const int n = n_first + t;
        if (n >= base && n < end) {
          const int k = n - base;
          float4 q = txf[le.start + t];
          q.x += ox; q.y += oy; q.z += oz;
          st.pos[k] = q;
          st.jidx[k] = le.start + t;
          st.code[k] = (unsigned char)code;
        }
      }
    }
    acc += __shfl_sync(0xffffffffu, x, 31);
  }
  __syncwarp();
  return end - base;
}

__device__ __forceinline__ int stage_window(const Params &p, const LeafEntry *__restrict__ pool, int off,
                                            int nleaf, int ntrial, int base, const float4 *__restrict__ txf,
                                            Stage &st) {
  return stage_window_n<STAGE>(p, pool, off, nleaf, ntrial, base, txf, st);
}

// ------------------------------------------------------------------ mixed-form separation
// Pair separation of the mixed form: formed in FP64 from the FP64 positions,
// rounded to FP32. The periodic image is the staged leaf's offset (code) plus
// the wrap decided on the FP32 separation of the staged copy (dxf, dyf, dzf);
// per axis the two add up to a shift of m box lengths, |m| <= 2. Unshifted
// pairs (nearly all) cost three FP64 subtractions. Shifted ones take their
// own branch: an FP64 warp instruction holds the FP64 pipe for the same time
// whether or not its lanes are predicated on, so the shift must not be issued
// for warps that have none.
__device__ __forceinline__ int image_shift(int code, int axis, bool wrap, float d) {
  const int c = (code >> (2 * axis)) & 3;
  return (c == 1 ? 1 : (c == 2 ? -1 : 0)) + (wrap ? (d > 0.0f ? 1 : -1) : 0);
}
__device__ __forceinline__ double shift_len(int m, double L) {
  return m == 0 ? 0.0 : (m == 1 ? L : (m == -1 ? -L : (double)m * L));
}
__device__ __forceinline__ void separation_mixed(const Params &p, double xi, double yi, double zi, double xj,
                                                 double yj, double zj, int code, float dxf, float dyf, float dzf,
                                                 float &dx, float &dy, float &dz) {
  bool wx = false, wy = false, wz = false;
  if (p.periodic) {
    wx = fabsf(dxf) > 0.5f * p.dxboundf; wy = fabsf(dyf) > 0.5f * p.dyboundf; wz = fabsf(dzf) > 0.5f * p.dzboundf;
  }
  const int mx = image_shift(code, 0, wx, dxf), my = image_shift(code, 1, wy, dyf),
            mz = image_shift(code, 2, wz, dzf);
  if ((mx | my | mz) == 0) {
    dx = d2f_rn(xi - xj); dy = d2f_rn(yi - yj); dz = d2f_rn(zi - zj);
  } else {
    dx = d2f_rn((xi - xj) - shift_len(mx, p.dxbound));
    dy = d2f_rn((yi - yj) - shift_len(my, p.dybound));
    dz = d2f_rn((zi - zj) - shift_len(mz, p.dzbound));
  }
}

// ------------------------------------------------------------------ active particles of a cell
// With individual timesteps a cell's pair loops run over its active
// particles only (dens.F90:1293-1378, force.F90 start_cell skip inactive
// ones). The warp takes the ballot of the cell's activity flags (tree
// order; null when every particle is active): np becomes the active count
// and slot k of the cell maps to tree position s0 + cell_pos(m, k).
__device__ __forceinline__ unsigned cell_active_mask(const unsigned char *actf, int s0, int np_all, int &np) {
  const int lane = lane_id();
  const unsigned m = __ballot_sync(0xffffffffu, lane < np_all && (!actf || actf[s0 + lane]));
  np = __popc(m);
  return m;
}
__device__ __forceinline__ int cell_pos(unsigned m, int k) { return (int)__fns(m, 0, k + 1); }

// ------------------------------------------------------------------ pair queues
// Most staged trial entries fail the cheap distance test (about 1 in 8 is a
// neighbour), so a pair body run directly inside the test loop executes with
// a few lanes of the warp active. Instead, lane (il, stripe) tests entries
// stripe, stripe + S, ... of the window for particle il and appends the
// accepted window indices to il's queue, in window order; a queue that may
// overflow in the next round, and every queue at the end of the window, is
// drained by the S lanes of its particle (queue entry m by lane m % S). The
// bodies then run with nearly every lane active.
constexpr int QCAP = 64;

struct PairQ {
  unsigned short k[MAXCELL][QCAP];
};

// per-warp dynamic shared memory of the pair kernels
struct PairSmem {
  Stage st;
  PairQ q;
};

template <class Test, class Body>
__device__ __forceinline__ void queue_window(int cnt, int S, bool act, int il, int stripe, PairQ &q, Test &&test,
                                             Body &&body) {
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id();
  const unsigned gmask = !act ? 0u : (S >= 32 ? FULL : (((1u << S) - 1u) << (il * S)));
  const unsigned lt = (1u << lane) - 1u;
  const int nr = (cnt + S - 1) / S;
  int qn = 0;
  for (int r = 0; r < nr; ++r) {
    const int k = r * S + stripe;
    const bool ok = act && k < cnt && test(k);
    const unsigned b = __ballot_sync(FULL, ok);
    if (ok) q.k[il][qn + __popc(b & gmask & lt)] = (unsigned short)k;
    qn += __popc(b & gmask);
    // qn <= QCAP - S before this round's appends, so no queue overflows
    if (r == nr - 1 || (int)__reduce_max_sync(FULL, (unsigned)qn) > QCAP - S) {
      __syncwarp();
      for (int m = stripe; act && m < qn; m += S) body((int)q.k[il][m]);
      __syncwarp();
      qn = 0;
    }
  }
}

// The walking cell: position, size and search radius (exact and FP32).
struct WalkCell {
  double xp, yp, zp, xsizei, rcuti;
  float xpf, ypf, zpf, xsf, rcf;
};

// Node test of getneigh (kdtree.F90:1251-1290, get_sep :1468-1501) in the
// reference's FP64 rounding. Returns whether the node is opened; code gets
// the periodic offset code (2 bits per axis, 1: +L, 2: -L).
template <bool GET_HJ>
__device__ __forceinline__ bool node_open_exact(const Params &p, const Node &n, const WalkCell &w, double tree_acc2,
                                                int &code) {
  double dx = dsub(w.xp, n.x), dy = dsub(w.yp, n.y), dz = dsub(w.zp, n.z);
  code = 0;
  if (p.periodic) {
    if (fabs(dx) > p.hdlx) { double o = dmul(p.dxbound, sign1(dx)); dx = dsub(dx, o); code |= (o > 0 ? 1 : 2); }
    if (fabs(dy) > p.hdly) { double o = dmul(p.dybound, sign1(dy)); dy = dsub(dy, o); code |= (o > 0 ? 1 : 2) << 2; }
    if (fabs(dz) > p.hdlz) { double o = dmul(p.dzbound, sign1(dz)); dz = dsub(dz, o); code |= (o > 0 ? 1 : 2) << 4; }
  }
  const double r2 = r2_exact(dx, dy, dz);
  double rcut = w.rcuti;
  if (GET_HJ) { double rcutj = dmul(RADKERN, n.hmax); rcut = fmax(w.rcuti, rcutj); }
  const double t = dadd(dadd(w.xsizei, n.size), rcut);
  bool open = r2 < dmul(t, t);
  if (p.gravity) {
    const double s2 = dadd(w.xsizei, n.size);
    open = open || (dmul(tree_acc2, r2) < dmul(s2, s2));
  }
  return open;
}

// The same test decided in FP32 on the node mirror: each FP32 separation d'
// is within E = 2^-22 (|x'_cell| + |x'_node|) of the FP64 one (+ 2^-22 L
// after a periodic shift), which brackets r^2 and the wrap decisions; the
// thresholds carry a 1e-5 relative margin for their FP32 rounding. A test
// the bounds cannot decide is repeated exactly on the FP64 node record, so
// the outcome is always the reference's.
template <bool GET_HJ>
__device__ __forceinline__ bool node_open(const Params &p, const NodeF &nf, const Node *__restrict__ nodes, int nd,
                                          const WalkCell &w, double tree_acc2, float tacc2f, int &code) {
  const float E0 = 2.384185791015625e-07f;  // 2^-22
  float dx = w.xpf - nf.x, dy = w.ypf - nf.y, dz = w.zpf - nf.z;
  float ex = E0 * (fabsf(w.xpf) + fabsf(nf.x)), ey = E0 * (fabsf(w.ypf) + fabsf(nf.y)),
        ez = E0 * (fabsf(w.zpf) + fabsf(nf.z));
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
    const float rc = GET_HJ ? fmaxf(w.rcf, 2.0f * nf.hmax) : w.rcf;
    const float t = w.xsf + nf.size + rc;
    const float tlo = t * (1.0f - 1.0e-5f), thi = t * (1.0f + 1.0e-5f);
    int st = (ub < tlo * tlo) ? 1 : ((lb > thi * thi) ? 0 : 2);
    if (p.gravity && st != 1) {
      const float s2 = w.xsf + nf.size;
      const float slo = s2 * (1.0f - 1.0e-5f), shi = s2 * (1.0f + 1.0e-5f);
      const int g = (tacc2f * ub < slo * slo) ? 1 : ((tacc2f * lb > shi * shi) ? 0 : 2);
      st = (g == 1) ? 1 : ((st == 0 && g == 0) ? 0 : 2);
    }
    if (st != 2) return st == 1;
  }
  const Node n = nodes[nd];
  return node_open_exact<GET_HJ>(p, n, w, tree_acc2, code);
}

// Walk of one cell by a warp. Returns the number of emitted leaves (in walk
// order, in sh.em) or -1 on overflow. All 32 lanes must call it.
template <bool GET_HJ>
__device__ int walk_cell(const Params &p, const Node *__restrict__ nodes, const NodeF *__restrict__ nodesf, int root,
                         const WalkCell &wc, WalkShared &sh) {
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id();
  const double tree_acc2 = p.tree_accuracy * p.tree_accuracy;
  const float tacc2f = (float)tree_acc2;
  if (lane == 0) sh.stk[0] = root;
  __syncwarp();
  int top = 1, nem = 0;
  bool overflow = false;
  while (top > 0) {
    int k = min(32, top);
    int nd = (lane < k) ? sh.stk[top - k + lane] : -1;
    top -= k;
    __syncwarp();
    bool emit = false, push = false;
    LeafEntry le{0, 0};
    int il = -1, ir = -1;
    if (nd >= 0) {
      const NodeF nf = nodesf[nd];
      int code;
      if (node_open<GET_HJ>(p, nf, nodes, nd, wc, tree_acc2, tacc2f, code)) {
        if (nf.left < 0) { emit = true; le.start = nf.right; le.cc = nf.count | (code << 8); }
        else { push = true; il = nf.left; ir = nf.right; }
      }
    }
    unsigned be = __ballot_sync(FULL, emit);
    if (emit) {
      int pos = nem + __popc(be & ((1u << lane) - 1));
      if (pos < WALK_EM) sh.em[pos] = le;
    }
    nem += __popc(be);
    unsigned bp = __ballot_sync(FULL, push);
    if (push) {
      int pos = top + 2 * __popc(bp & ((1u << lane) - 1));
      if (pos + 1 < WALK_STK) { sh.stk[pos] = il; sh.stk[pos + 1] = ir; }
    }
    top += 2 * __popc(bp);
    if (top >= WALK_STK || nem > WALK_EM) { overflow = true; break; }
    __syncwarp();
  }
  __syncwarp();
  if (overflow) return -1;
  return nem;
}

// K3 for the density: walk the cells of `act` whose redo flag is set
// W warps (cells) per block, W in {1, 2, 4} (static shared memory, <= 40 KB)
template <bool GET_HJ, int W>
__global__ void __launch_bounds__(32 * W) k_walk(Params p, const Node *nodes, const NodeF *nodesf, int root,
                                                          const int *leaves,
                                                          const int *act, int nact, const int *need,
                                                          const double *cell_hmax, LeafEntry *pool,
                                                          long long pool_cap, unsigned long long *pool_top,
                                                          int *cell_off, int *cell_nleaf, int *cell_ntrial,
                                                          int *err) {
  __shared__ WalkShared sh[W];
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int a = blockIdx.x * W + w;
  if (a >= nact) return;
  const int cell = act ? act[a] : a;
  if (need && !need[cell]) return;
  const Node nd = nodes[leaves[cell]];
  WalkCell wc;
  wc.xp = nd.x; wc.yp = nd.y; wc.zp = nd.z; wc.xsizei = nd.size;
  wc.rcuti = dmul(RADKERN, cell_hmax ? cell_hmax[cell] : nd.hmax);
  wc.xpf = (float)wc.xp; wc.ypf = (float)wc.yp; wc.zpf = (float)wc.zp; wc.xsf = (float)wc.xsizei;
  wc.rcf = (float)wc.rcuti;
  int nem = walk_cell<GET_HJ>(p, nodes, nodesf, root, wc, sh[w]);
  if (nem < 0) {
    if (lane == 0) set_error(err, PH_ERR_STACK);
    return;
  }
  int tot = 0;
  for (int e = lane; e < nem; e += 32) tot += sh[w].em[e].cc & 255;
  tot = warp_sum_int(tot);
  unsigned long long off = 0;
  if (lane == 0) off = atomicAdd(pool_top, (unsigned long long)nem);
  off = __shfl_sync(0xffffffffu, off, 0);
  if ((long long)(off + nem) > pool_cap) {
    if (lane == 0) set_error(err, PH_ERR_LIST);
    return;
  }
  write_ranked(sh[w].em, nem, pool, off);
  if (lane == 0) { cell_off[cell] = (int)off; cell_nleaf[cell] = nem; cell_ntrial[cell] = tot; }
}

// k_walk with the context's warps per block (1, 2 or 4)
template <bool GET_HJ, class... A>
inline void launch_walk(int warps, int ncells, cudaStream_t st, A... args) {
  if (warps >= 4) k_walk<GET_HJ, 4><<<(ncells + 3) / 4, 128, 0, st>>>(args...);
  else if (warps == 2) k_walk<GET_HJ, 2><<<(ncells + 1) / 2, 64, 0, st>>>(args...);
  else k_walk<GET_HJ, 1><<<ncells, 32, 0, st>>>(args...);
}

}  // namespace ph
