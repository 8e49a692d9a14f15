// Leaf-cell neighbour walk (K3): getneigh (kdtree.F90:1221-1347) with
// cache_neighbours (kdtree.F90:1175-1213), one warp per leaf cell.
//
// The warp expands up to 32 stack entries at a time. The reference walk pops
// the right child first, so its trial list is the opened leaves in decreasing
// order of their first particle; the emitted leaves are sorted into that order
// before they are written, which reproduces the reference trial list exactly
// (including which entries fall inside the 1000-entry position cache).
#pragma once
#include "ph_common.cuh"

namespace ph {

constexpr int WALK_WARPS = 2;
constexpr int WALK_STK = 512;
constexpr int WALK_EM = 1024;

struct WalkShared {
  int stk[WALK_STK];
  LeafEntry em[WALK_EM];
  LeafEntry sorted[WALK_EM];
};

// Returns the number of emitted leaves (sorted, in sh.sorted) or -1 on overflow.
// All 32 lanes must call it.
// ------------------------------------------------------------------ staging
// The trial list of a cell is a list of whole leaves. For the pair loops it is
// expanded, window by window, into a flat per-warp array in shared memory:
// the tree index of each trial particle, its periodic offset code and its FP32
// position with the offset applied (w = the caller's 4th component of txf).
// Entry k of window `base` is trial-list position n = base + k, which decides
// whether the reference would use its cached position (n < 1000).
constexpr int STAGE = 512;

struct Stage {
  float4 pos[STAGE];
  int jidx[STAGE];
  unsigned char code[STAGE];
};

__device__ __forceinline__ int stage_window(const Params &p, const LeafEntry *__restrict__ pool, int off,
                                            int nleaf, int ntrial, int base, const float4 *__restrict__ txf,
                                            Stage &st) {
  const int lane = lane_id();
  const int end = min(ntrial, base + STAGE);
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
      const float ox = (float)offset_of(code, 0, p.dxbound), oy = (float)offset_of(code, 1, p.dybound),
                  oz = (float)offset_of(code, 2, p.dzbound);
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

template <bool GET_HJ>
__device__ int walk_cell(const Params &p, const Node *__restrict__ nodes, int root, double xp, double yp,
                         double zp, double xsizei, double rcuti, WalkShared &sh) {
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id();
  const double tree_acc2 = p.tree_accuracy * p.tree_accuracy;
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
      const Node n = nodes[nd];
      // get_sep kdtree.F90:1468-1501
      double dx = dsub(xp, n.x), dy = dsub(yp, n.y), dz = dsub(zp, n.z);
      int code = 0;
      if (p.periodic) {
        if (fabs(dx) > p.hdlx) { double o = dmul(p.dxbound, sign1(dx)); dx = dsub(dx, o); code |= (o > 0 ? 1 : 2); }
        if (fabs(dy) > p.hdly) { double o = dmul(p.dybound, sign1(dy)); dy = dsub(dy, o); code |= (o > 0 ? 1 : 2) << 2; }
        if (fabs(dz) > p.hdlz) { double o = dmul(p.dzbound, sign1(dz)); dz = dsub(dz, o); code |= (o > 0 ? 1 : 2) << 4; }
      }
      double r2 = r2_exact(dx, dy, dz);
      double rcut = rcuti;
      if (GET_HJ) { double rcutj = dmul(RADKERN, n.hmax); rcut = fmax(rcuti, rcutj); }
      double t = dadd(dadd(xsizei, n.size), rcut);
      double rcut2 = dmul(t, t);
      bool open = r2 < rcut2;
      if (p.gravity) {
        double s2 = dadd(xsizei, n.size);
        open = open || (dmul(tree_acc2, r2) < dmul(s2, s2));
      }
      if (open) {
        if (n.left < 0) { emit = true; le.start = n.start; le.cc = n.count | (code << 8); }
        else { push = true; il = n.left; ir = n.right; }
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
  // order as the reference walk produces it: descending first particle
  for (int e = lane; e < nem; e += 32) {
    LeafEntry me = sh.em[e];
    int rank = 0;
    for (int q = 0; q < nem; ++q) rank += (sh.em[q].start > me.start) ? 1 : 0;
    sh.sorted[rank] = me;
  }
  __syncwarp();
  return nem;
}

// K3 for the density: walk the cells of `act` whose redo flag is set
template <bool GET_HJ>
__global__ void __launch_bounds__(32 * WALK_WARPS) k_walk(Params p, const Node *nodes, int root, const int *leaves,
                                                          const int *act, int nact, const int *need,
                                                          const double *cell_hmax, LeafEntry *pool,
                                                          long long pool_cap, unsigned long long *pool_top,
                                                          int *cell_off, int *cell_nleaf, int *cell_ntrial,
                                                          int *err) {
  __shared__ WalkShared sh[WALK_WARPS];
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int a = blockIdx.x * WALK_WARPS + w;
  if (a >= nact) return;
  const int cell = act ? act[a] : a;
  if (need && !need[cell]) return;
  const Node nd = nodes[leaves[cell]];
  double rcuti = dmul(RADKERN, cell_hmax ? cell_hmax[cell] : nd.hmax);
  int nem = walk_cell<GET_HJ>(p, nodes, root, nd.x, nd.y, nd.z, nd.size, rcuti, sh[w]);
  if (nem < 0) {
    if (lane == 0) set_error(err, PH_ERR_STACK);
    return;
  }
  int tot = 0;
  for (int e = lane; e < nem; e += 32) tot += sh[w].sorted[e].cc & 255;
  tot = warp_sum_int(tot);
  unsigned long long off = 0;
  if (lane == 0) off = atomicAdd(pool_top, (unsigned long long)nem);
  off = __shfl_sync(0xffffffffu, off, 0);
  if ((long long)(off + nem) > pool_cap) {
    if (lane == 0) set_error(err, PH_ERR_LIST);
    return;
  }
  for (int e = lane; e < nem; e += 32) pool[off + e] = sh[w].sorted[e];
  if (lane == 0) { cell_off[cell] = (int)off; cell_nleaf[cell] = nem; cell_ntrial[cell] = tot; }
}

}  // namespace ph
