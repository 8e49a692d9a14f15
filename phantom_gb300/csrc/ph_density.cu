// Density h-rho Newton-Raphson solve (K4): densityiterate (dens.F90:117-568)
// with get_density_sums (dens.F90:578-857), finish_cell (dens.F90:1382-1466),
// compute_hmax (dens.F90:1275-1289) and store_results (dens.F90:1511-1681).
//
// Work decomposition: k_density_pairs takes one warp per active leaf cell. A
// cell holds np <= 10 particles; the warp's lanes are split into np groups of
// S = 32/np lanes. Lane (i, s) tests the trial-list entries s, s+S, ... of each
// staged window for particle i and queues the ones that pass the distance
// pre-filter; the queued pairs are then summed with every lane busy. The sums
// of each particle go to a per-particle array, and k_density_finish (one thread
// per cell) takes the Newton-Raphson update, the cell-wide convergence test,
// the neighbour-list redo decision and store_results. Cells iterate in
// device-wide passes; a cell whose hmax grew is re-walked before its next
// pass, as the reference does per cell.
//
// Neighbour decisions are exact: an FP32 pre-filter with a 1e-3 margin in q^2
// only discards pairs that are provably outside the kernel, and every other
// pair is tested in FP64 with the reference's rounding (no FMA contraction,
// cached positions x_j + offset for the first 1000 trial entries).
#include "ph_internal.h"
#include "ph_walk.cuh"

namespace ph {

constexpr int NACC = 13;  // rho, gradh, gradsoft, divB + 9 dB/dx sums

// cubic spline W and dW/dq (kernel_cubic.f90:34-50), exact rounding
__device__ __forceinline__ void kern_exact(double q2, double q, double &w, double &g) {
  if (q < 1.0) {
    w = dadd(dsub(dmul(dmul(0.75, q2), q), dmul(1.5, q2)), 1.0);
    g = dmul(q, dsub(dmul(2.25, q), 3.0));
  } else if (q < 2.0) {
    double t = dsub(q, 2.0);
    w = dmul(-0.25, dmul(dmul(t, t), t));
    g = dmul(-0.75, dmul(t, t));
  } else {
    w = 0.0; g = 0.0;
  }
}
// get_kernel_grav1 (kernel_cubic.f90:78-99) dphidh term
__device__ __forceinline__ double dphidh_exact(double q2, double q) {
  if (q < 1.0) {
    double q4 = dmul(q2, q2);
    return dadd(dsub(dadd(dmul(dmul(-0.6, q4), q), dmul(1.5, q4)), dmul(2.0, q2)), 1.4);
  } else if (q < 2.0) {
    double q4 = dmul(q2, q2);
    return dadd(dsub(dadd(dsub(dmul(dmul(0.2, q4), q), dmul(1.5, q4)), dmul(dmul(4.0, q2), q)), dmul(4.0, q2)), 1.6);
  }
  return 0.0;
}

// the same term in FP32 (mixed form). For 1 <= q < 2 the reference's
// polynomial vanishes at q = 2 out of terms ~30; in t = 2 - q it is exactly
// t^4 (1/2 - t/5), evaluated that way.
__device__ __forceinline__ float dphidh_f(float q2, float q) {
  if (q < 1.0f) {
    const float q4 = q2 * q2;
    return -0.6f * q4 * q + 1.5f * q4 - 2.0f * q2 + 1.4f;
  } else if (q < 2.0f) {
    const float t = 2.0f - q, t2 = t * t;
    return t2 * t2 * (0.5f - 0.2f * t);
  }
  return 0.0f;
}

// FP32 B_j rho_j per tree position for the mixed MHD sums, rho_j from h_j at
// entry of the density call (the value the divcurlB sums read)
__global__ void k_dens_bprep(Params p, int n, const int *perm, const double *Bevol, const double *hj_entry,
                             float4 *bjf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double rho = rhoh(hj_entry[i], p.massoftype, p.hfact);
  const double *b = Bevol + 4 * (size_t)perm[i];
  bjf[i] = make_float4((float)(b[0] * rho), (float)(b[1] * rho), (float)(b[2] * rho), 0.0f);
}

// gather per-particle tree-order inputs: h, and h into the FP32 copy (its
// x, y, z are set by the tree build)
__global__ void k_dens_gather(int n, const int *perm, const double *xyzh, const double *tx, const double *ty,
                              const double *tz, double *hcur, double *hold, float4 *txf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double h = xyzh[4 * (size_t)perm[i] + 3];
  hcur[i] = h; hold[i] = h;
  txf[i].w = (float)h;
}

__global__ void k_dens_init_cells(int ncell, const int *leaves, const Node *nodes, double *cell_hmax,
                                  int *cell_nits, int *act) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  cell_hmax[c] = nodes[leaves[c]].hmax;
  cell_nits[c] = 0;
  act[c] = c;
}

// per-particle pair sums written by k_density_pairs (tree order, slot-major
// with stride ps): slots 0..NACC-1 the sums, then the neighbour count and the
// neighbour-set hash (bit pattern) of each particle, self excluded
constexpr int DSLOT_NN = NACC, DSLOT_HASH = NACC + 1;

struct DensOut {
  double *xyzh;
  float *gradh, *divcurlv, *divcurlB;
  int32_t *nneigh;
  uint64_t *nhash;
  double *th;            // treecache h update (dens.F90:1596)
  double *gradh64;       // 1/Omega in FP64 per tree position (read by the adjoint)
  double *gsoft64;       // gradsoft in FP64 per tree position (self-gravity; read by the adjoint)
  float *gradh_t;        // gradh(2,:) per tree position (read by the force)
  int diag;              // write the caller-order gradh, divcurlv, divcurlB, nneigh, nhash
  double *dvterm;        // cnormk gradh / (rho h^4) per tree position for the dv pass (or null)
  double *rhomax;
  unsigned long long *stats;  // nneightry, nneighact, maxneightry, maxneighact, ncalc, np, ncalls
};

// get_density_sums (dens.F90:578-857) for the active cells: one warp per cell,
// lanes (particle il, stripe), accepted pairs drained from per-particle queues.
template <bool MIXED, bool MHD, bool GRAV>
__global__ void __launch_bounds__(32 * MAX_WARPS) k_density_pairs(
    Params p, const Node *nodes, const int *leaves, const int *act, int nact, const LeafEntry *pool,
    const int *cell_off, const int *cell_nleaf, const int *cell_ntrial, const int *perm, const double *tx,
    const double *ty, const double *tz, const float4 *txf, const double *hcur, const double *Bevol,
    const double *hj_entry, const float4 *bjf, double *psum, int64_t ps, unsigned long long *stats, double pf_hmin,
    const unsigned char *actf, int want_hash, int *err) {
  extern __shared__ __align__(16) unsigned char dsm[];
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int a = blockIdx.x * (blockDim.x >> 5) + w;
  if (a >= nact) return;
  const int cell = act[a];
  const Node nd = nodes[leaves[cell]];
  const int np_all = nd.count, s0 = nd.start;
  if (np_all < 1 || np_all > MAXCELL) {
    if (lane == 0) set_error(err, PH_ERR_TREE);
    return;
  }
  int np;
  const unsigned am = cell_active_mask(actf, s0, np_all, np);  // active particles (individual timesteps)
  if (np == 0) return;
  const int S = 32 / np;
  const bool active_lane = lane < np * S;
  const int il = active_lane ? lane / S : 0, stripe = active_lane ? lane % S : 0;
  const int i = s0 + cell_pos(am, il);
  const double pm = p.massoftype;
  const double xi = tx[i], yi = ty[i], zi = tz[i];
  const double hi = hcur[i], hi1 = ddiv(1.0, hi), hi21 = dmul(hi1, hi1);
  const float4 xif = txf[i];
  const float hi21f = (float)hi21;
  const bool use_pf = hi > pf_hmin;
  const float q2lim = 4.0f * 1.001f;
  double bxi = 0, byi = 0, bzi = 0, rhoi_b = 0;
  float bxrf = 0.0f, byrf = 0.0f, bzrf = 0.0f;  // B_i rho_i (mixed form)
  if (MHD) {
    const double *b = Bevol + 4 * (size_t)perm[i];
    bxi = b[0]; byi = b[1]; bzi = b[2];
    rhoi_b = rhoh(hi, pm, p.hfact);
    bxrf = (float)(bxi * rhoi_b); byrf = (float)(byi * rhoi_b); bzrf = (float)(bzi * rhoi_b);
  }
  double acc[NACC];
  for (int k = 0; k < NACC; ++k) acc[k] = 0.0;
  Kahan kacc[NACC];
  const float hi1f = (float)hi1, pmf = (float)pm;
  int nn = 0;
  unsigned long long hh = 0;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
  const int ntrial = cell_ntrial[cell];
  if (lane == 0) {
    atomicAdd(&stats[9], (unsigned long long)ntrial);
    atomicAdd(&stats[11], (unsigned long long)np * (unsigned long long)ntrial);
  }
  PairSmem &sm = reinterpret_cast<PairSmem *>(dsm)[w];
  for (int base = 0; base < ntrial; base += STAGE) {
    const int cnt = stage_window(p, pool, off, nleaf, ntrial, base, txf, sm.st);
    auto test = [&](int k) -> bool {
      if (sm.st.jidx[k] == i) return false;  // ignoreself (dens.F90:650)
      if (!(use_pf || MIXED)) return true;
      const float4 xj = sm.st.pos[k];
      float dxf = xif.x - xj.x, dyf = xif.y - xj.y, dzf = xif.z - xj.z;
      if (p.periodic) {
        if (fabsf(dxf) > 0.5f * p.dxboundf) dxf -= copysignf(p.dxboundf, dxf);
        if (fabsf(dyf) > 0.5f * p.dyboundf) dyf -= copysignf(p.dyboundf, dyf);
        if (fabsf(dzf) > 0.5f * p.dzboundf) dzf -= copysignf(p.dzboundf, dzf);
      }
      const float r2f = dxf * dxf + dyf * dyf + dzf * dzf;
      return r2f * hi21f < q2lim;
    };
    // mixed form: the pair's operands, then its body
    struct PF { int j, code; float4 xj; double x, y, z; };
    auto load = [&](int k) -> PF {
      PF f;
      f.j = sm.st.jidx[k]; f.code = sm.st.code[k]; f.xj = sm.st.pos[k];
      f.x = tx[f.j]; f.y = ty[f.j]; f.z = tz[f.j];
      return f;
    };
    auto body_m = [&](const PF &pf) {
      const int j = pf.j;
      {
        // separation formed in FP64 (the periodic image chosen on the FP32
        // copy), rounded to FP32; W, dW/dh and the sums in FP32 (Kahan)
        const float4 xj = pf.xj;
        float dx, dy, dz;
        separation_mixed(p, xi, yi, zi, pf.x, pf.y, pf.z, pf.code, xif.x - xj.x, xif.y - xj.y, xif.z - xj.z, dx,
                         dy, dz);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float q2 = r2 * hi21f;
        if (q2 < 4.0f) {
          const float rij = sqrtf(r2), q = rij * hi1f;
          float wab, grk;
          if (q < 1.0f) { wab = 0.75f * q2 * q - 1.5f * q2 + 1.0f; grk = q * (2.25f * q - 3.0f); }
          else { const float t2 = q - 2.0f; wab = -0.25f * t2 * t2 * t2; grk = -0.75f * t2 * t2; }
          kacc[0].add(wab * pmf);
          kacc[1].add((-q * grk - 3.0f * wab) * pmf);
          if (GRAV) kacc[2].add(dphidh_f(q2, q) * pmf);
          ++nn;
          if (want_hash) hh += mix64((unsigned long long)perm[j] + 1ull);
          if (MHD) {
            const float r1g = grk / (rij + 1.0e-30f);
            const float rux = dx * r1g * pmf, ruy = dy * r1g * pmf, ruz = dz * r1g * pmf;
            const float4 bj = bjf[j];
            const float dBx = bxrf - bj.x, dBy = byrf - bj.y, dBz = bzrf - bj.z;
            kacc[3].add(dBx * rux + dBy * ruy + dBz * ruz);
            kacc[4].add(dBx * rux); kacc[5].add(dBx * ruy); kacc[6].add(dBx * ruz);
            kacc[7].add(dBy * rux); kacc[8].add(dBy * ruy); kacc[9].add(dBy * ruz);
            kacc[10].add(dBz * rux); kacc[11].add(dBz * ruy); kacc[12].add(dBz * ruz);
          }
        }
      }
    };
    auto body = [&](int k) {
      const int n = base + k, j = sm.st.jidx[k];
      const int code = sm.st.code[k];
      const double ox = offset_of(code, 0, p.dxbound), oy = offset_of(code, 1, p.dybound),
                   oz = offset_of(code, 2, p.dzbound);
      double dx, dy, dz;
      if (n < CELLCACHE && code != 0) {
        dx = dsub(xi, dadd(tx[j], ox)); dy = dsub(yi, dadd(ty[j], oy)); dz = dsub(zi, dadd(tz[j], oz));
      } else {
        dx = dsub(xi, tx[j]); dy = dsub(yi, ty[j]); dz = dsub(zi, tz[j]);
      }
      dx = wrap(dx, p.dxbound, p.hdlx, p.periodic); dy = wrap(dy, p.dybound, p.hdly, p.periodic);
      dz = wrap(dz, p.dzbound, p.hdlz, p.periodic);
      const double rij2 = r2_exact(dx, dy, dz);
      const double q2i = dmul(rij2, hi21);
      if (q2i < RADKERN2) {
        const double rij = sqrt(rij2);
        const double qi = dmul(rij, hi1);
        double wab, grk;
        kern_exact(q2i, qi, wab, grk);
        const double dwdh = dsub(-dmul(qi, grk), dmul(3.0, wab));
        acc[0] = dadd(acc[0], dmul(wab, pm));
        acc[1] = dadd(acc[1], dmul(dwdh, pm));
        if (GRAV) acc[2] = dadd(acc[2], dmul(dphidh_exact(q2i, qi), pm));
        ++nn;
        if (want_hash) hh += mix64((unsigned long long)perm[j] + 1ull);
        if (MHD) {  // dens.F90:745-829 (getdB)
          const double rij1 = ddiv(1.0, dadd(rij, EPS_D));
          const double r1g = dmul(rij1, grk);
          const double rux = dmul(dmul(dx, r1g), pm), ruy = dmul(dmul(dy, r1g), pm), ruz = dmul(dmul(dz, r1g), pm);
          const double rhoj = rhoh(hj_entry[j], pm, p.hfact);
          const double *bj = Bevol + 4 * (size_t)perm[j];
          const double dBx = dsub(dmul(bxi, rhoi_b), dmul(bj[0], rhoj));
          const double dBy = dsub(dmul(byi, rhoi_b), dmul(bj[1], rhoj));
          const double dBz = dsub(dmul(bzi, rhoi_b), dmul(bj[2], rhoj));
          acc[3] = dadd(acc[3], dadd(dadd(dmul(dBx, rux), dmul(dBy, ruy)), dmul(dBz, ruz)));
          acc[4] = dadd(acc[4], dmul(dBx, rux)); acc[5] = dadd(acc[5], dmul(dBx, ruy)); acc[6] = dadd(acc[6], dmul(dBx, ruz));
          acc[7] = dadd(acc[7], dmul(dBy, rux)); acc[8] = dadd(acc[8], dmul(dBy, ruy)); acc[9] = dadd(acc[9], dmul(dBy, ruz));
          acc[10] = dadd(acc[10], dmul(dBz, rux)); acc[11] = dadd(acc[11], dmul(dBz, ruy)); acc[12] = dadd(acc[12], dmul(dBz, ruz));
        }
      }
    };
    if constexpr (MIXED) queue_window(cnt, S, active_lane, il, stripe, sm.q, test, [&](int k) { body_m(load(k)); });
    else queue_window(cnt, S, active_lane, il, stripe, sm.q, test, body);
  }
  if constexpr (MIXED) {
    for (int k = 0; k < NACC; ++k) acc[k] = kacc[k].value();
  }
  // combine the stripes of each particle in stripe order (the staged window
  // is no longer needed: its shared memory holds the partial sums)
  constexpr int RW = NACC + 2;
  double *red = reinterpret_cast<double *>(&sm.st);
  __syncwarp();
  for (int k = 0; k < NACC; ++k) red[lane * RW + k] = acc[k];
  red[lane * RW + DSLOT_NN] = (double)nn;
  red[lane * RW + DSLOT_HASH] = __longlong_as_double((long long)hh);
  __syncwarp();
  if (lane < np) {
    double r[NACC];
    for (int k = 0; k < NACC; ++k) r[k] = 0.0;
    double nni = 0.0;
    unsigned long long hhi = 0;
    for (int q = 0; q < S; ++q) {
      const double *src = red + (lane * S + q) * RW;
      for (int k = 0; k < NACC; ++k) r[k] = dadd(r[k], src[k]);
      nni += src[DSLOT_NN];
      hhi += (unsigned long long)__double_as_longlong(src[DSLOT_HASH]);
    }
    const size_t ip = (size_t)(s0 + cell_pos(am, lane));
    for (int k = 0; k < NACC; ++k) psum[k * ps + ip] = r[k];
    psum[DSLOT_NN * ps + ip] = nni;
    psum[DSLOT_HASH * ps + ip] = __longlong_as_double((long long)hhi);
  }
}

// ------------------------------------------------------------------ velocity derivatives
// Sums for the Cullen & Dehnen switch (getdv, dens.F90:745-802): div v, the
// velocity and acceleration gradients and the R matrix, over each cell's
// final trial list with the h of its converged iteration (the reference
// stores the sums of that iteration, dens.F90:1630-1663), in one pass after
// the h-rho solve. Then, per particle, the exact-linear gradients
// (dens.F90:866-1101): div v, dvdx(9) and d(div v)/dt. vf holds the pass's
// velocities and accelerations (vx, vy, vz, ax, ay, az) in tree order, vff
// an FP32 copy (mixed form).
constexpr int NDV = 25;  // div v, dv_a/dx_b (9), da_a/dx_b (9), R (6)

__global__ void k_dv_gather(int n, const int *perm, const double *vel, const double *fxyzu, double *vf, float *vff) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const size_t pid = (size_t)perm[j];
  double *o = vf + 6 * (size_t)j;
  for (int k = 0; k < 3; ++k) { o[k] = vel[4 * pid + k]; o[3 + k] = fxyzu[4 * pid + k]; }
  if (vff) for (int k = 0; k < 6; ++k) vff[6 * (size_t)j + k] = d2f_rn(o[k]);
}

// dens.F90:866-891, 899-989, 997-1055, 1086-1101 (reference rounding)
__device__ __forceinline__ void exactlinear3(double ax, double ay, double az, const double *rm, double ddenom,
                                             double &gx, double &gy, double &gz) {
  gx = dmul(dadd(dadd(dmul(ax, rm[0]), dmul(ay, rm[1])), dmul(az, rm[2])), ddenom);
  gy = dmul(dadd(dadd(dmul(ax, rm[1]), dmul(ay, rm[3])), dmul(az, rm[4])), ddenom);
  gz = dmul(dadd(dadd(dmul(ax, rm[2]), dmul(ay, rm[4])), dmul(az, rm[5])), ddenom);
}
__device__ void dv_from_sums(const double *rs, double term, double &divv, double &ddivvdt, double *dv) {
  // rs[0]: div v; rs[1..9]: dv_a/dx_b; rs[10..18]: da_a/dx_b; rs[19..24]: rxx rxy rxz ryy ryz rzz
  const double rxx = rs[19], rxy = rs[20], rxz = rs[21], ryy = rs[22], ryz = rs[23], rzz = rs[24];
  const double denom = dsub(dsub(dsub(dadd(dmul(dmul(rxx, ryy), rzz), dmul(dmul(dmul(2.0, rxy), rxz), ryz)),
                                      dmul(dmul(rxx, ryz), ryz)),
                                 dmul(dmul(ryy, rxz), rxz)),
                            dmul(dmul(rzz, rxy), rxy));
  double rm[6];
  rm[0] = dsub(dmul(ryy, rzz), dmul(ryz, ryz)); rm[1] = dsub(dmul(rxz, ryz), dmul(rzz, rxy));
  rm[2] = dsub(dmul(rxy, ryz), dmul(rxz, ryy)); rm[3] = dsub(dmul(rzz, rxx), dmul(rxz, rxz));
  rm[4] = dsub(dmul(rxy, rxz), dmul(rxx, ryz)); rm[5] = dsub(dmul(rxx, ryy), dmul(rxy, rxy));
  divv = dmul(-rs[0], term);
  double div_a;
  if (fabs(denom) > TINY_D) {
    const double ddenom = ddiv(1.0, denom);
    double g0, g1, g2, gax, gay, gaz;
    exactlinear3(rs[10], rs[11], rs[12], rm, ddenom, gax, g1, g2);
    exactlinear3(rs[13], rs[14], rs[15], rm, ddenom, g0, gay, g2);
    exactlinear3(rs[16], rs[17], rs[18], rm, ddenom, g0, g1, gaz);
    div_a = -dadd(dadd(gax, gay), gaz);
    for (int a = 0; a < 3; ++a) {
      double gx, gy, gz;
      exactlinear3(rs[1 + 3 * a], rs[2 + 3 * a], rs[3 + 3 * a], rm, ddenom, gx, gy, gz);
      dv[3 * a] = -gx; dv[3 * a + 1] = -gy; dv[3 * a + 2] = -gz;
    }
  } else {
    div_a = dmul(-term, dadd(dadd(rs[10], rs[14]), rs[18]));
    for (int q = 0; q < 9; ++q) dv[q] = dmul(-rs[1 + q], term);
  }
  const double sq = dadd(dadd(dmul(dv[0], dv[0]), dmul(dv[4], dv[4])), dmul(dv[8], dv[8]));
  const double cr = dadd(dadd(dmul(dv[1], dv[3]), dmul(dv[2], dv[6])), dmul(dv[5], dv[7]));
  ddivvdt = dsub(div_a, dadd(sq, dmul(2.0, cr)));
}

template <bool MIXED>
__global__ void __launch_bounds__(32 * MAX_WARPS) k_density_dv(
    Params p, const Node *nodes, const int *leaves, int ncell, const LeafEntry *pool, const int *cell_off,
    const int *cell_nleaf, const int *cell_ntrial, const int *perm, const double *tx, const double *ty,
    const double *tz, const float4 *txf, const double *hcur, const double *vf, const float *vff,
    double *dvsum, int64_t ps, double pf_hmin, const int *cells, const unsigned char *actf) {
  extern __shared__ __align__(16) unsigned char dsm[];
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int a = blockIdx.x * (blockDim.x >> 5) + w;
  if (a >= ncell) return;
  const int cell = cells ? cells[a] : a;
  const Node nd = nodes[leaves[cell]];
  const int np_all = nd.count, s0 = nd.start;
  if (np_all < 1 || np_all > MAXCELL) return;  // reported by k_density_pairs
  int np;
  const unsigned am = cell_active_mask(actf, s0, np_all, np);
  if (np == 0) return;
  const int S = 32 / np;
  const bool active_lane = lane < np * S;
  const int il = active_lane ? lane / S : 0, stripe = active_lane ? lane % S : 0;
  const int i = s0 + cell_pos(am, il);
  const double pm = p.massoftype;
  const double xi = tx[i], yi = ty[i], zi = tz[i];
  const double hi = hcur[i], hi1 = ddiv(1.0, hi), hi21 = dmul(hi1, hi1);
  const float4 xif = txf[i];
  const float hi21f = (float)hi21, hi1f = (float)hi1, pmf = (float)pm;
  const bool use_pf = hi > pf_hmin;
  const float q2lim = 4.0f * 1.001f;
  const double *vfi = vf + 6 * (size_t)i;
  double acc[NDV];
  for (int k = 0; k < NDV; ++k) acc[k] = 0.0;
  Kahan kacc[MIXED ? NDV : 1];
  float vfif[6];
  if (MIXED) for (int k = 0; k < 6; ++k) vfif[k] = vff[6 * (size_t)i + k];
  const int off = cell_off[cell], nleaf = cell_nleaf[cell], ntrial = cell_ntrial[cell];
  PairSmem &sm = reinterpret_cast<PairSmem *>(dsm)[w];
  for (int base = 0; base < ntrial; base += STAGE) {
    const int cnt = stage_window(p, pool, off, nleaf, ntrial, base, txf, sm.st);
    auto test = [&](int k) -> bool {
      if (sm.st.jidx[k] == i) return false;  // ignoreself
      if (!(use_pf || MIXED)) return true;
      const float4 xj = sm.st.pos[k];
      float dxf = xif.x - xj.x, dyf = xif.y - xj.y, dzf = xif.z - xj.z;
      if (p.periodic) {
        if (fabsf(dxf) > 0.5f * p.dxboundf) dxf -= copysignf(p.dxboundf, dxf);
        if (fabsf(dyf) > 0.5f * p.dyboundf) dyf -= copysignf(p.dyboundf, dyf);
        if (fabsf(dzf) > 0.5f * p.dzboundf) dzf -= copysignf(p.dzboundf, dzf);
      }
      return (dxf * dxf + dyf * dyf + dzf * dzf) * hi21f < q2lim;
    };
    auto body = [&](int k) {
      const int n = base + k, j = sm.st.jidx[k];
      const int code = sm.st.code[k];
      if constexpr (MIXED) {
        const float4 xj = sm.st.pos[k];
        float dx, dy, dz;
        separation_mixed(p, xi, yi, zi, tx[j], ty[j], tz[j], code, xif.x - xj.x, xif.y - xj.y, xif.z - xj.z, dx, dy,
                         dz);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float q2 = r2 * hi21f;
        if (q2 < 4.0f) {
          const float rij = sqrtf(r2), q = rij * hi1f;
          const float grk = q < 1.0f ? q * (2.25f * q - 3.0f) : -0.75f * (q - 2.0f) * (q - 2.0f);
          const float r1g = grk / (rij + 1.0e-30f);
          const float rux = dx * r1g * pmf, ruy = dy * r1g * pmf, ruz = dz * r1g * pmf;
          const float *vj = vff + 6 * (size_t)j;
          const float dvx = vfif[0] - vj[0], dvy = vfif[1] - vj[1], dvz = vfif[2] - vj[2];
          const float dax = vfif[3] - vj[3], day = vfif[4] - vj[4], daz = vfif[5] - vj[5];
          kacc[0].add(dvx * rux + dvy * ruy + dvz * ruz);
          kacc[1].add(dvx * rux); kacc[2].add(dvx * ruy); kacc[3].add(dvx * ruz);
          kacc[4].add(dvy * rux); kacc[5].add(dvy * ruy); kacc[6].add(dvy * ruz);
          kacc[7].add(dvz * rux); kacc[8].add(dvz * ruy); kacc[9].add(dvz * ruz);
          kacc[10].add(dax * rux); kacc[11].add(dax * ruy); kacc[12].add(dax * ruz);
          kacc[13].add(day * rux); kacc[14].add(day * ruy); kacc[15].add(day * ruz);
          kacc[16].add(daz * rux); kacc[17].add(daz * ruy); kacc[18].add(daz * ruz);
          kacc[19].add(-dx * rux); kacc[20].add(-dx * ruy); kacc[21].add(-dx * ruz);
          kacc[22].add(-dy * ruy); kacc[23].add(-dy * ruz); kacc[24].add(-dz * ruz);
        }
        return;
      }
      const double ox = offset_of(code, 0, p.dxbound), oy = offset_of(code, 1, p.dybound),
                   oz = offset_of(code, 2, p.dzbound);
      double dx, dy, dz;
      if (n < CELLCACHE && code != 0) {
        dx = dsub(xi, dadd(tx[j], ox)); dy = dsub(yi, dadd(ty[j], oy)); dz = dsub(zi, dadd(tz[j], oz));
      } else {
        dx = dsub(xi, tx[j]); dy = dsub(yi, ty[j]); dz = dsub(zi, tz[j]);
      }
      dx = wrap(dx, p.dxbound, p.hdlx, p.periodic); dy = wrap(dy, p.dybound, p.hdly, p.periodic);
      dz = wrap(dz, p.dzbound, p.hdlz, p.periodic);
      const double rij2 = r2_exact(dx, dy, dz);
      const double q2i = dmul(rij2, hi21);
      if (q2i < RADKERN2) {
        const double rij = sqrt(rij2);
        const double qi = dmul(rij, hi1);
        double wab, grk;
        kern_exact(q2i, qi, wab, grk);
        const double rij1 = ddiv(1.0, dadd(rij, EPS_D));
        const double r1g = dmul(rij1, grk);
        const double rux = dmul(dmul(dx, r1g), pm), ruy = dmul(dmul(dy, r1g), pm), ruz = dmul(dmul(dz, r1g), pm);
        const double *vj = vf + 6 * (size_t)j;
        const double dvx = dsub(vfi[0], vj[0]), dvy = dsub(vfi[1], vj[1]), dvz = dsub(vfi[2], vj[2]);
        acc[0] = dadd(acc[0], dadd(dadd(dmul(dvx, rux), dmul(dvy, ruy)), dmul(dvz, ruz)));
        acc[1] = dadd(acc[1], dmul(dvx, rux)); acc[2] = dadd(acc[2], dmul(dvx, ruy)); acc[3] = dadd(acc[3], dmul(dvx, ruz));
        acc[4] = dadd(acc[4], dmul(dvy, rux)); acc[5] = dadd(acc[5], dmul(dvy, ruy)); acc[6] = dadd(acc[6], dmul(dvy, ruz));
        acc[7] = dadd(acc[7], dmul(dvz, rux)); acc[8] = dadd(acc[8], dmul(dvz, ruy)); acc[9] = dadd(acc[9], dmul(dvz, ruz));
        const double dax = dsub(vfi[3], vj[3]), day = dsub(vfi[4], vj[4]), daz = dsub(vfi[5], vj[5]);
        acc[10] = dadd(acc[10], dmul(dax, rux)); acc[11] = dadd(acc[11], dmul(dax, ruy)); acc[12] = dadd(acc[12], dmul(dax, ruz));
        acc[13] = dadd(acc[13], dmul(day, rux)); acc[14] = dadd(acc[14], dmul(day, ruy)); acc[15] = dadd(acc[15], dmul(day, ruz));
        acc[16] = dadd(acc[16], dmul(daz, rux)); acc[17] = dadd(acc[17], dmul(daz, ruy)); acc[18] = dadd(acc[18], dmul(daz, ruz));
        acc[19] = dsub(acc[19], dmul(dx, rux)); acc[20] = dsub(acc[20], dmul(dx, ruy)); acc[21] = dsub(acc[21], dmul(dx, ruz));
        acc[22] = dsub(acc[22], dmul(dy, ruy)); acc[23] = dsub(acc[23], dmul(dy, ruz)); acc[24] = dsub(acc[24], dmul(dz, ruz));
      }
    };
    queue_window(cnt, S, active_lane, il, stripe, sm.q, test, body);
  }
  // stripes of each particle in stripe order (the whole per-warp scratch):
  // FP64 in the FP64 form; in the mixed form each stripe's compensated sum
  // is read out and the stripes added in FP32
  double *red = reinterpret_cast<double *>(&sm);
  float *redf = reinterpret_cast<float *>(&sm);
  static_assert(32 * NDV * sizeof(double) <= sizeof(PairSmem), "dv reduction scratch");
  __syncwarp();
  if constexpr (MIXED) {
    for (int k = 0; k < NDV; ++k) redf[lane * NDV + k] = __fsub_rn(kacc[k].s, kacc[k].c);
  } else {
    for (int k = 0; k < NDV; ++k) red[lane * NDV + k] = acc[k];
  }
  __syncwarp();
  if (lane < np) {
    const size_t ip = (size_t)(s0 + cell_pos(am, lane));
    for (int k = 0; k < NDV; ++k) {
      if constexpr (MIXED) {
        float r = 0.0f;
        for (int q = 0; q < S; ++q) r += redf[(lane * S + q) * NDV + k];
        dvsum[k * ps + ip] = (double)r;
      } else {
        double r = 0.0;
        for (int q = 0; q < S; ++q) r = dadd(r, red[(lane * S + q) * NDV + k]);
        dvsum[k * ps + ip] = r;
      }
    }
  }
}

// per particle: the exact-linear gradients from the sums (dense lanes: the
// FP64 pipe costs the same per warp instruction whatever its active lanes)
__global__ void k_dv_finish(int n, const double *dvsum, int64_t ps, const double *dvterm, const int *perm,
                            float *ddivvdt_c, float *dvdx_c, float *divcurlv, float *curl3, int diag,
                            const unsigned char *actf) {
  const int ip = blockIdx.x * blockDim.x + threadIdx.x;
  if (ip >= n || (actf && !actf[ip])) return;
  double rs[NDV];
  for (int k = 0; k < NDV; ++k) rs[k] = dvsum[k * ps + ip];
  double divv, ddivvdt, dv[9];
  dv_from_sums(rs, dvterm[ip], divv, ddivvdt, dv);
  // caller order: with individual timesteps inactive particles keep theirs
  // across tree builds
  const size_t pid = (size_t)perm[ip];
  ddivvdt_c[pid] = (float)ddivvdt;
  for (int q = 0; q < 9; ++q) dvdx_c[9 * pid + q] = (float)dv[q];
  if (diag) divcurlv[pid] = (float)divv;
  if (curl3) {  // curl v (dens.F90:919-923): sums 1..9 are dv_a r_b (a, b = x, y, z)
    const double t = dvterm[ip];
    curl3[3 * pid] = (float)(-(rs[8] - rs[6]) * t);
    curl3[3 * pid + 1] = (float)(-(rs[3] - rs[7]) * t);
    curl3[3 * pid + 2] = (float)(-(rs[4] - rs[2]) * t);
  }
}

// Newton-Raphson update of one particle from its sums (finish_rhosum
// dens.F90:1486-1500, finish_cell dens.F90:1425-1462)
struct DensNR {
  double rhoi, gradhi, dhdrhoi, omegai, hmine;
  bool conv;
};
__device__ __forceinline__ DensNR dens_nr(const Params &p, double r0, double r1, double hme, double h_old) {
  const double pm = p.massoftype;
  DensNR o;
  const double h1 = ddiv(1.0, hme), h21 = dmul(h1, h1), h31 = dmul(h1, h21), h41 = dmul(h21, h21);
  o.rhoi = dmul(dmul(CNORMK, dadd(r0, dmul(1.0, pm))), h31);
  o.gradhi = dmul(dmul(CNORMK, dadd(r1, dmul(-3.0, pm))), h41);
  o.dhdrhoi = dhdrho(hme, pm, p.hfact);
  o.omegai = dsub(1.0, dmul(o.dhdrhoi, o.gradhi));
  const double rhohi = rhoh(hme, pm, p.hfact);
  const double func = dsub(rhohi, o.rhoi);
  const double dfdh1 = (o.omegai > TINY_D) ? ddiv(o.dhdrhoi, o.omegai) : ddiv(o.dhdrhoi, fabs(dadd(o.omegai, EPS_D)));
  double hnew = dsub(hme, dmul(func, dfdh1));
  if (hnew > dmul(1.2, hme)) hnew = dmul(1.2, hme);
  else if (hnew < dmul(0.8, hme)) hnew = dmul(0.8, hme);
  o.conv = (ddiv(fabs(dsub(hnew, hme)), h_old) < p.tolh) && o.omegai > 0.0 && hme > 0.0;
  o.hmine = o.conv ? hme : hnew;
  return o;
}

// finish_cell + compute_hmax (dens.F90:1275-1289) + the redo decision and,
// for converged cells, store_results (dens.F90:1561-1677). A cell takes a
// 16-lane segment of a warp, lane q its particle q: the cell-wide convergence
// test and hmax are segment shuffles, the cell's own decisions are taken by
// lane 0 of the segment, and the global maxima and statistics are reduced
// per block before one atomic each (a per-particle atomic on rhomax would
// serialise 2M updates on one address).
constexpr int FIN_SEG = 16;  // lanes per cell, >= MAXCELL
constexpr int FIN_THREADS = 256;
static_assert(MAXCELL <= FIN_SEG, "a finish segment holds a whole cell");

__global__ void __launch_bounds__(FIN_THREADS) k_density_finish(
    Params p, int icall, const Node *nodes, Node *nodes_w, const int *leaves, const int *act, int nact,
    const double *psum, int64_t ps, const int *cell_ntrial, const int *perm, double *hcur, const double *hold,
    double *cell_hmax, int *cell_nits, int *need_walk, int *next_act, int *nnext, DensOut out, NodeF *nodesf,
    const unsigned char *actf, int *err) {
  __shared__ unsigned long long bst[8];  // stats 0..6, rhomax bits
  if (threadIdx.x < 8) bst[threadIdx.x] = 0ull;
  __syncthreads();
  const unsigned FULL = 0xffffffffu;
  const int lane = lane_id(), q = lane & (FIN_SEG - 1);
  const long long a = ((long long)blockIdx.x * FIN_THREADS + threadIdx.x) / FIN_SEG;
  bool cell_ok = a < nact;
  int cell = 0, leaf = 0, np = 0, s0 = 0;
  if (cell_ok) {
    cell = act[a];
    leaf = leaves[cell];
    np = nodes[leaf].count;
    s0 = nodes[leaf].start;
    cell_ok = np >= 1 && np <= MAXCELL;  // else reported by k_density_pairs
  }
  // the cell's active particles (individual timesteps): this segment's bits of the ballot
  const unsigned bal = __ballot_sync(FULL, cell_ok && q < np && (!actf || actf[s0 + q]));
  const unsigned segm = (bal >> (lane & ~(FIN_SEG - 1))) & ((1u << FIN_SEG) - 1u);
  np = __popc(segm);
  const bool mine = cell_ok && q < np;
  const size_t ip = (size_t)(s0 + (mine ? (int)__fns(segm, 0, q + 1) : q));
  const double pm = p.massoftype;
  DensNR o{};
  if (mine) o = dens_nr(p, psum[ip], psum[ps + ip], hcur[ip], hold[ip]);
  int conv = (!mine || o.conv) ? 1 : 0;
  double hm = mine ? o.hmine : 0.0;
  for (int m = 1; m < FIN_SEG; m <<= 1) {
    conv &= __shfl_xor_sync(FULL, conv, m);
    hm = fmax(hm, __shfl_xor_sync(FULL, hm, m));
  }
  if (icall == 0) conv = 1;
  const double hmax_new = dmul(1.01, hm);
  const int nits = cell_ok ? cell_nits[cell] + 1 : 0;
  const bool lead = cell_ok && q == 0;
  bool append = false, redo = false;
  if (cell_ok && !conv) {
    if (nits >= MAXDENSITS) {
      if (lead) set_error(err, PH_ERR_DENS_NOCONV);
    } else {
      if (mine) hcur[ip] = o.hmine;
      if (lead) {
        redo = hmax_new > cell_hmax[cell];
        cell_nits[cell] = nits;
        cell_hmax[cell] = hmax_new;
        if (redo) {
          // set_hmaxcell neigh_kdtree.f90:115-131
          nodes_w[leaf].hmax = hmax_new;
          const float hf = (float)hmax_new;
          nodesf[leaf].hmax = hf;
          int pa = nodes[leaf].parent;
          while (pa >= 0) {
            atomic_max_pos(&nodes_w[pa].hmax, hmax_new);
            atomicMax(reinterpret_cast<int *>(&nodesf[pa].hmax), __float_as_int(hf));
            pa = nodes[pa].parent;
          }
        }
        need_walk[cell] = redo ? 1 : 0;
        append = true;
      }
    }
  }
  // cells for the next pass: one atomic per warp
  const unsigned ba = __ballot_sync(FULL, append);
  if (ba) {
    const int first = __ffs(ba) - 1;
    int base = 0;
    if (lane == first) base = atomicAdd(nnext, __popc(ba));
    base = __shfl_sync(FULL, base, first);
    if (append) next_act[base + __popc(ba & ((1u << lane) - 1))] = cell;
  }
  unsigned long long sv[5] = {0ull, 0ull, 0ull, 0ull, 0ull}, mx[2] = {0ull, 0ull};
  double rhoi_max = 0.0;
  if (cell_ok && conv) {
    if (lead) { cell_hmax[cell] = hmax_new; cell_nits[cell] = nits; need_walk[cell] = 0; }
    const double hme = mine ? hcur[ip] : 0.0;
    if (mine && hme < 0.0) set_error(err, PH_ERR_NEG_H);
    if (mine && hme >= 0.0) {
      const int ntry = cell_ntrial[cell];
      const int pid = perm[ip];
      const double h1 = ddiv(1.0, hme), h21 = dmul(h1, h1), h41 = dmul(h21, h21);
      const double grad = ddiv(1.0, o.omegai);
      const double hfin = hrho(o.rhoi, pm, p.hfact);
      out.xyzh[4 * (size_t)pid + 3] = hfin;
      out.th[ip] = hfin;
      if (hfin < 0.0) set_error(err, PH_ERR_NEG_H);
      const float gradf = (float)grad;
      out.gradh64[ip] = grad;
      float gsf = 0.0f;
      if (p.gravity) {
        double gs = dmul(dadd(psum[2 * ps + ip], dmul(DPHIDH0, pm)), h21);
        gs = dmul(gs, o.dhdrhoi);
        gsf = (float)gs;
        out.gsoft64[ip] = gs;
      }
      out.gradh_t[2 * ip] = gradf;
      out.gradh_t[2 * ip + 1] = gsf;
      if (out.diag || p.ind) {  // individual timesteps: the force reads gradh in caller order
        out.gradh[2 * (size_t)pid] = gradf;
        if (p.gravity || p.ind) out.gradh[2 * (size_t)pid + 1] = gsf;
      }
      rhoi_max = o.rhoi;
      const double term = dmul(dmul(dmul(CNORMK, (double)gradf), ddiv(1.0, o.rhoi)), h41);
      if (out.dvterm) out.dvterm[ip] = term;
      // getdv is .false. under CONST_AV (dens.F90:1638-1640)
      if (out.diag) out.divcurlv[pid] = -(float)(0.0 * term);
      if (p.mhd && out.diag) {
        const double r3 = psum[3 * ps + ip], r5 = psum[5 * ps + ip], r6 = psum[6 * ps + ip],
                     r7 = psum[7 * ps + ip], r9 = psum[9 * ps + ip], r10 = psum[10 * ps + ip],
                     r11 = psum[11 * ps + ip];
        float *db = out.divcurlB + 4 * (size_t)pid;
        db[0] = (float)(dmul(-r3, term));
        db[1] = (float)(dmul(-dsub(r11, r9), term));
        db[2] = (float)(dmul(-dsub(r6, r10), term));
        db[3] = (float)(dmul(-dsub(r7, r5), term));
      }
      const int nni = (int)psum[DSLOT_NN * ps + ip] + 1;  // + self
      if (out.diag) {
        out.nneigh[pid] = nni;
        out.nhash[pid] = (uint64_t)__double_as_longlong(psum[DSLOT_HASH * ps + ip]);
      }
      // nneightry, nneighact, ncalc, np summed; maxneightry, maxneighact
      sv[0] = (unsigned long long)ntry; sv[1] = (unsigned long long)nni; sv[2] = (unsigned long long)nits;
      sv[3] = 1ull;
      mx[0] = (unsigned long long)ntry; mx[1] = (unsigned long long)nni;
    }
  }
  sv[4] = (lead && redo) ? 1ull : 0ull;
  for (int m = 16; m > 0; m >>= 1) {
    for (int k = 0; k < 5; ++k) sv[k] += __shfl_xor_sync(FULL, sv[k], m);
    for (int k = 0; k < 2; ++k) mx[k] = max(mx[k], __shfl_xor_sync(FULL, mx[k], m));
  }
  rhoi_max = warp_max(rhoi_max);
  if (lane == 0) {
    if (sv[3]) {
      atomicAdd(&bst[0], sv[0]); atomicAdd(&bst[1], sv[1]); atomicMax(&bst[2], mx[0]);
      atomicMax(&bst[3], mx[1]); atomicAdd(&bst[4], sv[2]); atomicAdd(&bst[5], sv[3]);
      atomicMax(&bst[7], (unsigned long long)__double_as_longlong(rhoi_max));
    }
    if (sv[4]) atomicAdd(&bst[6], sv[4]);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (bst[5]) {
      atomicAdd(&out.stats[0], bst[0]); atomicAdd(&out.stats[1], bst[1]); atomicMax(&out.stats[2], bst[2]);
      atomicMax(&out.stats[3], bst[3]); atomicAdd(&out.stats[4], bst[4]); atomicAdd(&out.stats[5], bst[5]);
      atomic_max_pos(out.rhomax, __longlong_as_double((long long)bst[7]));
    }
    if (bst[6]) atomicAdd(&out.stats[6], bst[6]);
  }
}

static inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }

// densityiterate driver
int density(ph_ctx *c, int icall) {
  if (!c->have_tree) return PH_ERR_STATE;
  c->have_force_lists = false;  // the density walks reuse the list pool
  cudaStream_t st = c->stream;
  const int nt = (int)c->ntree, ncell = c->nleaves;
  const Params p = c->dp;
  k_dens_gather<<<nblk(nt, 256), 256, 0, st>>>(nt, c->perm, c->xyzh, c->tx, c->ty, c->tz, c->hcur, c->hold, c->txf);
  k_dens_init_cells<<<nblk(ncell, 256), 256, 0, st>>>(ncell, c->leaves, c->nodes, c->cell_hmax, c->cell_nits, c->act_a);
  cudaMemsetAsync(c->stats, 0, 8 * sizeof(unsigned long long), st);
  cudaMemsetAsync(c->red, 0, 8 * sizeof(double), st);
  count_launch(c, 2);
  // h_j used by the divcurlB sums: the value at entry of the pass (race-free
  // form of the reference's fast_divcurlB read of xyzh(4,j), dens.F90:811)
  const double *hj_entry = c->hold;
  // the Bevol of the evaluation (Bpred in a step: derivs passes its Bevol
  // argument on to densityiterate, deriv.f90:135)
  const double *Bd = c->dens_B ? c->dens_B : c->Bevol;
  if (p.mhd && p.precision == PH_PREC_MIXED) {
    k_dens_bprep<<<nblk(nt, 256), 256, 0, st>>>(p, nt, c->perm, Bd, hj_entry, c->bjf);
    count_launch(c, 1);
  }
  int nact = ncell;
  const unsigned char *actf = p.ind ? c->actf_t : nullptr;
  if (p.ind) {  // individual timesteps: leaf cells holding an active particle only
    cudaMemcpyAsync(c->act_a, c->cell_act, sizeof(int) * (size_t)c->ncell_act, cudaMemcpyDeviceToDevice, st);
    nact = c->ncell_act;
  }
  int *act = c->act_a, *nxt = c->act_b;
  int *need = c->cell_state;  // redo flags
  fill_int(c, need, ncell, 1);
  cudaMemsetAsync(c->pool_top, 0, sizeof(unsigned long long), st);
  // dens.F90:202-203: velocity derivatives for the viscosity switch
  // velocity derivatives for the Cullen & Dehnen switch or curl v (dens.F90:202-203)
  const bool getdv = (p.nalpha >= 2 || p.curlv) && (icall <= 1 || icall == 3);
  DensOut out{c->xyzh, c->gradh, c->divcurlv, c->divcurlB, c->nneigh, c->nhash, c->th, c->gradh64, c->gsoft64,
              c->gradh_t,
              c->want_diag ? 1 : 0, getdv ? c->dvterm_t : nullptr, c->red + 2, c->stats};
  double pf_hmin = c->pf_hmin;
  const int dw = c->dens_warps, ww = c->walk_warps;
  const int smem = dw * (int)sizeof(PairSmem);
  if (!(c->attr_done & 1u)) {
    const int smax = MAX_WARPS * (int)sizeof(PairSmem);
    cudaFuncSetAttribute(k_density_pairs<true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    cudaFuncSetAttribute(k_density_pairs<true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    cudaFuncSetAttribute(k_density_pairs<true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    cudaFuncSetAttribute(k_density_pairs<true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    cudaFuncSetAttribute(k_density_pairs<false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    cudaFuncSetAttribute(k_density_pairs<false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    cudaFuncSetAttribute(k_density_pairs<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    cudaFuncSetAttribute(k_density_pairs<false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smax);
    c->attr_done |= 1u;
  }
  for (int pass = 0; nact > 0; ++pass) {
    if (pass > MAXDENSITS + 2) return PH_ERR_DENS_NOCONV;
    for (int attempt = 0;; ++attempt) {
      cudaEventRecord(c->evk[4], st);
      launch_walk<false>(ww, nact, st,
          p, c->nodes, c->nodesf, c->root, c->leaves, act, nact, need, c->cell_hmax, c->pool, c->pool_cap, c->pool_top,
          c->cell_off, c->cell_nleaf, c->cell_ntrial, c->d_err);
      cudaEventRecord(c->evk[5], st);
      count_launch(c, 1);
      int herr = 0;
      cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
      cudaStreamSynchronize(st);
      add_elapsed(c, 6, c->evk[4], c->evk[5]);
      if (herr == PH_ERR_LIST && attempt < 4) {
        cudaMemsetAsync(c->d_err, 0, sizeof(int), st);
        if (grow_pool(c) != 0) return PH_ERR_LIST;
        continue;
      }
      if (herr) return herr;
      break;
    }
    cudaMemsetAsync(c->counters + 8, 0, sizeof(int), st);
    cudaEventRecord(c->evk[2], st);
#define PH_DENS(X, M, G)                                                                                         \
  k_density_pairs<X, M, G><<<nblk(nact, dw), 32 * dw, smem, st>>>(                                    \
      p, c->nodes, c->leaves, act, nact, c->pool, c->cell_off, c->cell_nleaf, c->cell_ntrial, c->perm, c->tx, c->ty,  \
      c->tz, c->txf, c->hcur, Bd, hj_entry, c->bjf, c->psum, c->cap, c->stats, pf_hmin, actf,             \
      c->want_diag ? 1 : 0, c->d_err)
    if (p.precision == PH_PREC_MIXED) {
      if (p.mhd) { if (p.gravity) PH_DENS(true, true, true); else PH_DENS(true, true, false); }
      else { if (p.gravity) PH_DENS(true, false, true); else PH_DENS(true, false, false); }
    } else {
      if (p.mhd) { if (p.gravity) PH_DENS(false, true, true); else PH_DENS(false, true, false); }
      else { if (p.gravity) PH_DENS(false, false, true); else PH_DENS(false, false, false); }
    }
#undef PH_DENS
    k_density_finish<<<nblk((int64_t)nact * FIN_SEG, FIN_THREADS), FIN_THREADS, 0, st>>>(p, icall, c->nodes, c->nodes, c->leaves, act, nact, c->psum,
                                                      c->cap, c->cell_ntrial, c->perm, c->hcur, c->hold,
                                                      c->cell_hmax, c->cell_nits, need, nxt, c->counters + 8, out,
                                                      c->nodesf, actf, c->d_err);
    cudaEventRecord(c->evk[3], st);
    count_launch(c, 2);
    int hv[2];
    cudaMemcpyAsync(&hv[0], c->counters + 8, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&hv[1], c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    add_elapsed(c, 5, c->evk[2], c->evk[3]);
    if (hv[1]) return hv[1];
    nact = hv[0];
    std::swap(act, nxt);
  }
  if (getdv) {  // velocity derivatives on the final lists (Cullen & Dehnen switch)
    const double *vel = c->dens_vel ? c->dens_vel : c->vxyzu;
    const bool mixed = p.precision == PH_PREC_MIXED;
    k_dv_gather<<<nblk(nt, 256), 256, 0, st>>>(nt, c->perm, vel, c->fxyzu, c->jrec, mixed ? c->jrecf : nullptr);
    if (!c->dvsum && alloc_dvsum(c) != 0) return PH_ERR_CUDA;
    const int dw = c->dens_warps;
    const int smem = dw * (int)sizeof(PairSmem);
    const int *dv_cells = p.ind ? c->cell_act : nullptr;
    const int ndv = p.ind ? c->ncell_act : ncell;
    if (mixed)
      k_density_dv<true><<<nblk(ndv, dw), 32 * dw, smem, st>>>(
          p, c->nodes, c->leaves, ndv, c->pool, c->cell_off, c->cell_nleaf, c->cell_ntrial, c->perm, c->tx, c->ty,
          c->tz, c->txf, c->hcur, c->jrec, c->jrecf, c->dvsum, c->cap, pf_hmin, dv_cells, actf);
    else
      k_density_dv<false><<<nblk(ndv, dw), 32 * dw, smem, st>>>(
          p, c->nodes, c->leaves, ndv, c->pool, c->cell_off, c->cell_nleaf, c->cell_ntrial, c->perm, c->tx, c->ty,
          c->tz, c->txf, c->hcur, c->jrec, nullptr, c->dvsum, c->cap, pf_hmin, dv_cells, actf);
    if (p.curlv && alloc_curlv(c) != 0) return PH_ERR_CUDA;
    k_dv_finish<<<nblk(nt, 256), 256, 0, st>>>(nt, c->dvsum, c->cap, c->dvterm_t, c->perm, c->ddivvdt_c, c->dvdx_c,
                                                c->divcurlv, p.curlv ? c->curl3 : nullptr, c->want_diag ? 1 : 0,
                                                actf);
    count_launch(c, 3);
  }
  if (check_launch(c) != cudaSuccess) return PH_ERR_CUDA;
  c->have_density = true;
  return 0;
}

}  // namespace ph
