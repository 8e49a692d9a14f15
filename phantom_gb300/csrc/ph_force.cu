// Force pair loop (K5/K6/K8): cons2prim_everything (cons2prim.f90:326-394,
// eos.f90:184-237), start_cell (force.F90:2172-2514), compute_forces
// (force.F90:914-2060) and finish_cell_and_store_results (force.F90:2649-3330)
// for gas particles: pressure, artificial viscosity and conductivity, ideal MHD
// (anisotropic Lorentz stress, artificial resistivity, div B cleaning) and the
// self-gravity near field; global Courant/force timestep minima.
//
// Decomposition mirrors the density: one warp per leaf cell, lanes split into
// (particle i, stripe s) pairs over the trial list; pairs that pass the
// distance pre-filter are queued per particle and evaluated with every lane
// busy, and the per-particle sums go to k_force_finish (one thread per
// particle) for finish_cell_and_store_results. The j-side quantities that
// compute_forces recomputes for every pair (rho_j, P_j/rho_j^2, v_wave,j, the
// magnetic stress, ...) are computed once per particle by k_force_prologue and
// read per pair. The neighbour test q_i^2 < 4 .or. q_j^2 < 4 is evaluated with
// the reference's rounding; an FP32 pre-filter skips pairs provably outside
// both kernels.
#include "ph_internal.h"
#include "ph_walk.cuh"

namespace ph {

constexpr int JREC = 16;   // doubles per particle, hydro record
constexpr int JMHD = 16;   // doubles per particle, MHD record
constexpr int NF = 12;     // fsum entries
constexpr int JRECF = 16, JMHDF = 16;  // floats per particle, FP32 copies of the records (mixed form)

// M4 dW/dq (kernel_cubic.f90:56-66)
__device__ __forceinline__ double grkern(double q) {
  if (q < 1.0) return q * (2.25 * q - 3.0);
  if (q < 2.0) { double t = q - 2.0; return -0.75 * (t * t); }
  return 0.0;
}
// kernel_softening (kernel_cubic.f90:101-120)
__device__ __forceinline__ void kernel_softening(double q2, double q, double &pot, double &fs) {
  if (q < 1.0) {
    double q4 = q2 * q2;
    pot = q4 * q / 10.0 - 3.0 * q4 / 10.0 + 2.0 * q2 / 3.0 - 7.0 / 5.0;
    fs = q * (15.0 * q2 * q - 36.0 * q2 + 40.0) / 30.0;
  } else if (q < 2.0) {
    double q4 = q2 * q2, q6 = q4 * q2;
    pot = (q * (-q4 * q + 9.0 * q4 - 30.0 * q2 * q + 40.0 * q2 - 48.0) + 2.0) / (30.0 * q);
    fs = (-5.0 * q6 + 36.0 * q4 * q - 90.0 * q4 + 80.0 * q2 * q - 2.0) / (30.0 * q2);
  } else {
    pot = -1.0 / q;
    fs = 1.0 / q2;
  }
}

// get_stress (force.F90:2068-2168) without physical viscosity / radiation
__device__ __forceinline__ void get_stress(const Params &p, double pri, double cs, double rhoi, double rho1i,
                                           double bx, double by, double bz, double &pro2, double &vwave,
                                           double *s) {
  const double pm = p.massoftype;
  if (p.mhd) {
    double brx = bx * rho1i, bry = by * rho1i, brz = bz * rho1i;
    double bro2 = brx * brx + bry * bry + brz * brz;
    double va2 = bro2 * rhoi;
    vwave = sqrt(cs * cs + va2);
    s[0] = -pm * brx * brx; s[1] = -pm * brx * bry; s[2] = -pm * brx * brz;
    s[3] = -pm * bry * bry; s[4] = -pm * bry * brz; s[5] = -pm * brz * brz;
    pro2 = pri * rho1i * rho1i + 0.5 * bro2;
  } else {
    for (int k = 0; k < 6; ++k) s[k] = 0.0;
    pro2 = pri * rho1i * rho1i;
    vwave = cs;
  }
}

// eos + j-side record per tree position
// shock_capturing.f90:151-177 xi_limiter (dvdx float, arithmetic in FP64)
__device__ __forceinline__ double xi_limiter(const float *dvdxf) {
  double d[9];
  for (int q = 0; q < 9; ++q) d[q] = (double)dvdxf[q];
  const double divv = dadd(dadd(d[0], d[4]), d[8]);
  const double cx = dsub(d[7], d[5]), cy = dsub(d[2], d[6]), cz = dsub(d[3], d[1]);
  const double m = fmax(-divv, 0.0);
  const double fac = dmul(m, m);
  const double traceS = dadd(dadd(dmul(cx, cx), dmul(cy, cy)), dmul(cz, cz));
  if (dadd(fac, traceS) > EPS_D) return ddiv(fac, dadd(fac, traceS));
  return 1.0;
}
// shock_capturing.f90:131-143 get_alphaloc
__device__ __forceinline__ double get_alphaloc(double divvdti, double spsoundi, double hi, double xi,
                                               double alpha_min, double alpha_max) {
  const double source = dmul(dmul(dmul(10.0, dmul(hi, hi)), xi), fmax(-divvdti, 0.0));
  const double temp = dmul(spsoundi, spsoundi);
  if (temp > EPS_D) return fmax(fmin(ddiv(source, temp), alpha_max), alpha_min);
  return alpha_min;
}

// The precision form's prologue: the FP32 particle records formed in FP32
// from the FP64 state rounded on the integer pipe (the FP64 form's exact
// divisions and square roots hold the FP64 pipe; the mixed pair kernels read
// FP32 records only), and of the FP64 ones what the force finish reads: the
// equation of state, u and, with MHD, Bevol and psi. cons2prim
// (cons2prim.f90:326-456) and get_stress (force.F90:2068-2168) as in
// k_force_prologue, in FP32.
__global__ void k_force_prologue_mixed(Params p, int n, const int *perm, const double *th, const double *vel,
                                       const double *Bv, const float *gradh, double *eos_t, double *jrec,
                                       double *jmhd, float *jrecf, float *jmhdf, float4 *txf, const float *alpha1,
                                       const float *ddivvdt_c, const float *dvdx_c, float *alphaloc_t, int *err) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int pid = perm[j];
  const double h = th[j];
  if (h < 0.0) set_error(err, PH_ERR_NEG_H);
  const float pmf = d2f_rn(p.massoftype);
  const float hf = d2f_rn(h);
  const float h1 = 1.0f / hf;
  const float t3 = d2f_rn(p.hfact) * h1;
  const float rho = pmf * (t3 * t3 * t3), rho1 = 1.0f / rho;
  const double *v = vel + 4 * (size_t)pid;
  const float u = p.isothermal ? 0.0f : d2f_rn(v[3]);
  float ponrho, cs;
  if (p.ieos == 1) { ponrho = d2f_rn(p.polyk); cs = sqrtf(ponrho); }
  else {
    ponrho = (p.gamma > 1.0001) ? d2f_rn(p.gamma - 1.0) * u : (2.0f / 3.0f) * u;
    cs = sqrtf(d2f_rn(p.gamma) * ponrho);
  }
  const float P = ponrho * rho;
  eos_t[2 * (size_t)j] = (double)P;
  eos_t[2 * (size_t)j + 1] = (double)cs;
  if (p.nalpha >= 2) {  // cons2prim.f90:413-418 Cullen & Dehnen alphaloc (FP64, as the FP64 form)
    const double xi = xi_limiter(dvdx_c + 9 * (size_t)pid);
    alphaloc_t[j] = (float)get_alphaloc((double)ddivvdt_c[pid], (double)cs, h, xi, p.alpha, p.alphamax);
  }
  float pro2 = P * rho1 * rho1, vwave = cs;
  float *q = jmhdf + JMHDF * (size_t)j;
  if (p.mhd) {
    // B/rho is Bevol; B = Bevol rho; stress -m (B/rho)(B/rho), P/rho^2 + |B/rho|^2/2,
    // v_wave = sqrt(c_s^2 + |B/rho|^2 rho)
    const double *b = Bv + 4 * (size_t)pid;
    const float brx = d2f_rn(b[0]), bry = d2f_rn(b[1]), brz = d2f_rn(b[2]);
    const float bro2 = brx * brx + bry * bry + brz * brz;
    vwave = sqrtf(cs * cs + bro2 * rho);
    pro2 += 0.5f * bro2;
    q[0] = brx * rho; q[1] = bry * rho; q[2] = brz * rho; q[3] = d2f_rn(b[3]);
    q[4] = -pmf * brx * brx; q[5] = -pmf * brx * bry; q[6] = -pmf * brx * brz;
    q[7] = -pmf * bry * bry; q[8] = -pmf * bry * brz; q[9] = -pmf * brz * brz;
    q[10] = brx; q[11] = bry; q[12] = brz;
    double *m = jmhd + JMHD * (size_t)j;  // the finish's B/rho and psi
    m[3] = b[3]; m[10] = b[0]; m[11] = b[1]; m[12] = b[2];
  }
  const size_t g = p.ind ? (size_t)pid : (size_t)j;
  const float mrho5 = 0.5f * pmf * rho1;
  float *o = jrecf + JRECF * (size_t)j;
  o[0] = h1; o[1] = rho; o[2] = rho1; o[3] = pro2; o[4] = vwave; o[5] = P;
  o[6] = mrho5 * d2f_rn(p.alphau); o[7] = gradh[2 * g];
  o[8] = d2f_rn(v[0]); o[9] = d2f_rn(v[1]); o[10] = d2f_rn(v[2]); o[11] = u;
  o[12] = gradh[2 * g + 1];
  o[13] = mrho5 * d2f_rn(p.alphaB) * rho1;
  o[14] = p.nalpha > 0 ? alpha1[pid] : d2f_rn(p.alpha);
  o[15] = rho1 * rho1;
  jrec[JREC * (size_t)j + 11] = p.isothermal ? 0.0 : v[3];  // the finish's u
  txf[j].w = h1;
}

__global__ void k_force_prologue(Params p, int n, const int *perm, const double *tx, const double *ty,
                                 const double *tz, const double *th, const double *vel, const double *Bv,
                                 const float *gradh, double *eos_t, double *jrec, double *jmhd, float *jrecf,
                                 float *jmhdf, float4 *txf, const float *alpha1, const float *ddivvdt_c,
                                 const float *dvdx_c, float *alphaloc_t, int *err) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double pm = p.massoftype;
  const int pid = perm[j];
  const double h = th[j];
  if (h < 0.0) set_error(err, PH_ERR_NEG_H);
  // cons2prim: rho = rhoh(h) (cons2prim.f90:343), P = (gamma-1) u rho or cs^2 rho
  const double rho_c = rhoh(h, pm, p.hfact);
  const double *v = vel + 4 * (size_t)pid;
  double ponrho, cs;
  if (p.ieos == 1) { ponrho = p.polyk; cs = sqrt(ponrho); }
  else {
    double u = v[3];
    ponrho = (p.gamma > 1.0001) ? (p.gamma - 1.0) * u : 2.0 / 3.0 * u;
    cs = sqrt(p.gamma * ponrho);
  }
  const double P = ponrho * rho_c;
  eos_t[2 * (size_t)j] = P;
  eos_t[2 * (size_t)j + 1] = cs;
  if (p.nalpha >= 2) {  // cons2prim.f90:413-418 Cullen & Dehnen alphaloc
    const double xi = xi_limiter(dvdx_c + 9 * (size_t)pid);
    alphaloc_t[j] = (float)get_alphaloc((double)ddivvdt_c[pid], cs, h, xi, p.alpha, p.alphamax);
  }
  // j-side of compute_forces (force.F90:1428-1511)
  const double hj1 = 1.0 / h;
  const double hj = 1.0 / hj1;
  const double rhoj = rhoh(hj, pm, p.hfact);
  const double rho1j = 1.0 / rhoj;
  double bx = 0, by = 0, bz = 0;
  if (p.mhd) {
    const double *b = Bv + 4 * (size_t)pid;
    bx = b[0] * rho_c; by = b[1] * rho_c; bz = b[2] * rho_c;
  }
  double pro2, vwave, s[6];
  get_stress(p, P, cs, rhoj, rho1j, bx, by, bz, pro2, vwave, s);
  const double mrhoj5 = 0.5 * pm * rho1j;
  double *r = jrec + JREC * (size_t)j;
  r[0] = hj1; r[1] = rhoj; r[2] = rho1j; r[3] = pro2; r[4] = vwave; r[5] = P;
  r[6] = mrhoj5 * p.alphau;
  // gradh in tree order; with individual timesteps in caller order, where
  // inactive particles keep the values of their last density solve
  const size_t g = p.ind ? (size_t)pid : (size_t)j;
  r[7] = (double)gradh[2 * g];
  r[8] = v[0]; r[9] = v[1]; r[10] = v[2]; r[11] = p.isothermal ? 0.0 : v[3];
  r[12] = (double)gradh[2 * g + 1];
  r[13] = mrhoj5 * p.alphaB * rho1j;
  r[14] = p.nalpha > 0 ? (double)alpha1[pid] : p.alpha;  // alphaind(1,j) (force.F90:1478, 2430-2433)
  r[15] = rho1j * rho1j;
  if (p.mhd) {
    double *m = jmhd + JMHD * (size_t)j;
    m[0] = bx; m[1] = by; m[2] = bz; m[3] = Bv[4 * (size_t)pid + 3];
    for (int k = 0; k < 6; ++k) m[4 + k] = s[k];
    m[10] = Bv[4 * (size_t)pid]; m[11] = Bv[4 * (size_t)pid + 1]; m[12] = Bv[4 * (size_t)pid + 2];
  }
  if (jrecf) {  // FP32 copies for the mixed form (rounded on the integer pipe)
    float *o = jrecf + JRECF * (size_t)j;
    for (int k = 0; k < JREC; ++k) o[k] = d2f_rn(r[k]);
    if (p.mhd) {
      const double *m = jmhd + JMHD * (size_t)j;
      float *q = jmhdf + JMHDF * (size_t)j;
      for (int k = 0; k < 13; ++k) q[k] = d2f_rn(m[k]);
    }
  }
  txf[j].w = (float)(1.0 / h);  // x, y, z: set by the tree build
}

struct ForceOut {
  double *fxyzu, *dBevol;
  float *divcurlv, *divBsymm, *poten;
  double *dtmin;  // [0] dtcourant, [1] dtforce (atomic min of positive doubles)
  unsigned long long *stats;
  const int *cell_ntrial;
};

// expand_fgrav_in_taylor_series (kdtree.F90:1799-1840): far-field force and
// potential at an offset (dx, dy, dz) from the leaf centre. The potential
// line keeps the reference's dz*dfxy term as written there.
__device__ __forceinline__ void expand_taylor(const double *f, double dx, double dy, double dz, double &fxi,
                                              double &fyi, double &fzi, double &poti) {
  fxi = f[0]; fyi = f[1]; fzi = f[2];
  const double dfxx = f[3], dfxy = f[4], dfxz = f[5], dfyy = f[6], dfyz = f[7], dfzz = f[8];
  const double d2fxxx = f[9], d2fxxy = f[10], d2fxxz = f[11], d2fxyy = f[12], d2fxyz = f[13], d2fxzz = f[14],
               d2fyyy = f[15], d2fyyz = f[16], d2fyzz = f[17], d2fzzz = f[18];
  poti = f[19];
  fxi = fxi + dx * (dfxx + 0.5 * (dx * d2fxxx + dy * d2fxxy + dz * d2fxxz))
            + dy * (dfxy + 0.5 * (dx * d2fxxy + dy * d2fxyy + dz * d2fxyz))
            + dz * (dfxz + 0.5 * (dx * d2fxxz + dy * d2fxyz + dz * d2fxzz));
  fyi = fyi + dx * (dfxy + 0.5 * (dx * d2fxxy + dy * d2fxyy + dz * d2fxyz))
            + dy * (dfyy + 0.5 * (dx * d2fxyy + dy * d2fyyy + dz * d2fyyz))
            + dz * (dfyz + 0.5 * (dx * d2fxyz + dy * d2fyyz + dz * d2fyzz));
  fzi = fzi + dx * (dfxz + 0.5 * (dx * d2fxxz + dy * d2fxyz + dz * d2fxzz))
            + dy * (dfyz + 0.5 * (dx * d2fxyz + dy * d2fyyz + dz * d2fyzz))
            + dz * (dfzz + 0.5 * (dx * d2fxzz + dy * d2fyzz + dz * d2fzzz));
  poti = poti - (dx * (fxi - 0.5 * (dx * dfxx + dy * dfxy + dz * dfxy)) +
                 dy * (fyi - 0.5 * (dx * dfxy + dy * dfyy + dz * dfyz)) +
                 dz * (fzi - 0.5 * (dx * dfxz + dy * dfyz + dz * dfzz)));
}

// gravity far field seen by the finish kernel
struct FarField {
  const double *gleaf;  // LENFG coefficients per leaf index
  const int *leaf_of;   // leaf index per tree position
  const int *leaves;
  const Node *nodes;
  const double *tx, *ty, *tz;
};

// per-particle pair sums written by the force pair kernels (tree order, slot
// major with stride ps): slots 0..NF-1 the fsum entries, slot NF vsigmax
constexpr int FSLOT_VSIG = NF;
// individual timesteps: slot NF+1 the largest ibin_old of the SPH neighbours
// (force.F90:1346-1353, the Saitoh-Makino limiter's input)
constexpr int FSLOT_NBIN = NF + 1;

// finish_cell_and_store_results (force.F90:2773-3328): one thread per particle
// (tree position ip) from its pair sums; timestep minima per warp, then one
// atomic per warp.
// individual timesteps in the finish: the particles' bins (caller order) and
// the step's counters; ibin null with global timesteps
struct IndFin {
  const unsigned char *actf_t;  // active flag per tree position
  int8_t *ibin;
  int *counters;                // [0] max new bin, [1] particles binned, [2] dt too small
  int nbinmax, istepfrac, allow_decrease;
};

// get_newbin (utils_indtimesteps.f90:230-287): the bin of a particle's new
// timestep; a shorter step moves it up at once, a longer one down by one bin
// and only where the lower bin's step ends on this substep
__device__ __forceinline__ int get_newbin(double dti, double dtmax, int ibini, const IndFin &ind, int &too_small) {
  const double dlog2 = 1.4426950408889634;
  int ibin_new;
  if (dti > dtmax) ibin_new = 0;
  else if (dti < TINY_D) ibin_new = MAXBINS;
  else ibin_new = max((int)(log(2.0 * dtmax / dti) * dlog2 - EPS_D), 0);
  if (ibin_new > MAXBINS) too_small = 1;
  if (ibin_new > ibini) return ibin_new;
  if (ibin_new < ibini && ibini <= ind.nbinmax && ind.allow_decrease &&
      (long long)ind.istepfrac % (1ll << (ind.nbinmax - (ibini - 1))) == 0)
    return ibini - 1;
  return ibini;
}

// The precision form's finish (MIXED): the per-particle chain (density, the
// pdV factor, div v, the MHD stress and cleaning, the timestep estimates) in
// FP32 from the FP64 values rounded on the integer pipe, where the FP64 form's
// divisions and square roots would hold the FP64 pipe; the accelerations and
// the dissipation sums stay the FP64 values of the pair sums, and the gravity
// far field stays FP64.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_force_finish(Params p, int nt, const double *psum, int64_t ps,
                                                      const int *perm, const double *th, const double *jrec,
                                                      const double *jmhd, const double *eos_t, FarField ff,
                                                      ForceOut out, IndFin ind, int *err) {
  const int ipr = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = ipr < nt && (!ind.actf_t || ind.actf_t[ipr]);  // inactive particles keep their forces
  const int ip = valid ? ipr : 0;
  const double pm = p.massoftype;
  const bool adiab = !p.isothermal;
  double fs[NF];
  for (int k = 0; k < NF; ++k) fs[k] = psum[k * ps + ip];
  const double vsm = psum[FSLOT_VSIG * ps + ip];
  const int pid = perm[ip];
  const double h = th[ip];
  const double pr = eos_t[2 * (size_t)ip], cs = eos_t[2 * (size_t)ip + 1];
  const double *rr = jrec + JREC * (size_t)ip;
  if (p.gravity) {
    // self-potential and far field (force.F90 finish_cell_and_store_results,
    // kdtree.F90:1799-1840); kernel_softening(0) potential = -7/5
    double epoti = 0.5 * pm * (fs[3] + pm * (-1.4) * (1.0 / h));
    const int l = ff.leaf_of[ip];
    const Node nl = ff.nodes[ff.leaves[l]];
    double fxi, fyi, fzi, poti;
    expand_taylor(ff.gleaf + LENFG * (size_t)l, ff.tx[ip] - nl.x, ff.ty[ip] - nl.y, ff.tz[ip] - nl.z, fxi, fyi, fzi,
                  poti);
    fs[0] += fxi; fs[1] += fyi; fs[2] += fzi;
    epoti += 0.5 * pm * poti;
    if (valid) out.poten[pid] = (float)epoti;
  }
  double *fo = out.fxyzu + 4 * (size_t)pid;
  double dtc = p.dtmax, dtf = BIGNUMBER, dtclean = BIGNUMBER;
  if constexpr (MIXED) {
    const float pmf = d2f_rn(pm), hf = d2f_rn(h), h1f = 1.0f / hf;
    const float t3 = d2f_rn(p.hfact) * (1.0f / fabsf(hf));
    const float rhof = pmf * (t3 * t3 * t3), rho1f = 1.0f / rhof;
    const float prf = d2f_rn(pr), csf = d2f_rn(cs);  // FP32 values held in FP64: exact
    float vwavef = csf, psif = 0.0f;
    if (p.mhd) {
      // B = rho B/rho, v_wave = sqrt(c_s^2 + |B/rho|^2 rho) (get_stress,
      // force.F90:2068-2168); the div B subtraction from the FP64 sums
      const double *m = jmhd + JMHD * (size_t)ip;
      const float brx = d2f_rn(m[10]), bry = d2f_rn(m[11]), brz = d2f_rn(m[12]);
      psif = d2f_rn(m[3]);
      const float bxf = brx * rhof, byf = bry * rhof, bzf = brz * rhof;
      vwavef = sqrtf(csf * csf + (brx * brx + bry * bry + brz * brz) * rhof);
      const float b2f = bxf * bxf + byf * byf + bzf * bzf;
      float frac = 0.0f;
      if (b2f > 0.0f) {
        const float betai = 2.0f * prf / b2f;
        frac = (betai < 2.0f) ? 1.0f : ((betai < 10.0f) ? (10.0f - betai) * 0.125f : 0.0f);
      }
      const double divBsymmi = fs[7];
      fs[0] -= (double)(bxf * frac) * divBsymmi;
      fs[1] -= (double)(byf * frac) * divBsymmi;
      fs[2] -= (double)(bzf * frac) * divBsymmi;
      if (valid) out.divBsymm[pid] = rhof * d2f_rn(divBsymmi);
    }
    if (valid) { fo[0] = fs[0]; fo[1] = fs[1]; fo[2] = fs[2]; }
    const float fxf = d2f_rn(fs[0]), fyf = d2f_rn(fs[1]), fzf = d2f_rn(fs[2]);
    const float f2f = fxf * fxf + fyf * fyf + fzf * fzf;
    const float drhodtf = pmf * d2f_rn(fs[4]);
    const float divvf = -drhodtf * rho1f;
    if (valid) out.divcurlv[pid] = divvf;
    double fxyz4 = 0.0;
    if (adiab) {
      if (p.ipdv_heating > 0) fxyz4 += (double)(prf * rho1f * rho1f * drhodtf);
      if (p.ishock_heating > 0) fxyz4 += fs[5];
      fxyz4 += fs[6];
    }
    if (p.mhd) {
      double *db = out.dBevol + 4 * (size_t)pid;
      if (valid) { db[0] = fs[8]; db[1] = fs[9]; db[2] = fs[10]; }
      if (p.psidecayfac > 0.0) {
        const float vclean = d2f_rn(p.overcleanfac) * vwavef;
        const float dtau = d2f_rn(p.psidecayfac) * vclean * h1f;
        if (valid) db[3] = (double)(-vclean * d2f_rn(fs[11]) * rho1f - psif * dtau - 0.5f * psif * divvf);
        dtclean = (double)(d2f_rn(p.C_cour) * hf / (vclean + TINY_F));
      }
    }
    const float vsigdtc = fmaxf(d2f_rn(vsm), vwavef);
    if (vsigdtc > TINY_F) dtc = (double)(d2f_rn(p.C_cour) * hf / (vsigdtc * fmaxf(d2f_rn(p.alpha), 1.0f)));
    if (adiab) {
      const double eni_ = rr[11];
      if (eni_ + dtc * fxyz4 < EPS_D && eni_ > EPS_D) fxyz4 = fxyz4 / (1.0 - dtc * fxyz4 / eni_);
      if (valid) fo[3] = fxyz4;
    }
    if (fabsf(f2f) > (float)EPS_D) dtf = (double)(d2f_rn(p.C_force) * sqrtf(hf / sqrtf(f2f)));
  } else {
    const double h1 = 1.0 / h;
    const double t3b = p.hfact * (1.0 / fabs(h));
    const double rho = pm * (t3b * t3b * t3b), rho1 = 1.0 / rho;
    double vwave = cs, bx = 0, by = 0, bz = 0, b2 = 0, psi = 0;
    if (p.mhd) {
      const double *m = jmhd + JMHD * (size_t)ip;
      bx = m[10] * rho; by = m[11] * rho; bz = m[12] * rho;
      psi = m[3];
      double pro2, s[6];
      get_stress(p, pr, cs, rho, rho1, bx, by, bz, pro2, vwave, s);
      b2 = bx * bx + by * by + bz * bz;
      const double divBsymmi = fs[7];
      double frac = 0.0;
      if (b2 > 0.0) {
        const double betai = 2.0 * pr / b2;
        frac = (betai < 2.0) ? 1.0 : ((betai < 10.0) ? (10.0 - betai) * 0.125 : 0.0);
      }
      fs[0] -= bx * divBsymmi * frac; fs[1] -= by * divBsymmi * frac; fs[2] -= bz * divBsymmi * frac;
      if (valid) out.divBsymm[pid] = (float)(rho * divBsymmi);
    }
    const double f2i = fs[0] * fs[0] + fs[1] * fs[1] + fs[2] * fs[2];
    if (valid) { fo[0] = fs[0]; fo[1] = fs[1]; fo[2] = fs[2]; }
    const double drhodti = pm * fs[4];
    const double divvi = -drhodti * rho1;
    if (valid) out.divcurlv[pid] = (float)divvi;
    double fxyz4 = 0.0;
    if (adiab) {
      if (p.ipdv_heating > 0) fxyz4 += pr * rho1 * rho1 * drhodti;
      if (p.ishock_heating > 0) fxyz4 += fs[5];
      fxyz4 += fs[6];
    }
    if (p.mhd) {
      double *db = out.dBevol + 4 * (size_t)pid;
      if (valid) { db[0] = fs[8]; db[1] = fs[9]; db[2] = fs[10]; }
      if (p.psidecayfac > 0.0) {
        const double vclean = p.overcleanfac * vwave;
        const double dtau = p.psidecayfac * vclean * h1;
        if (valid) db[3] = -vclean * fs[11] * rho1 - psi * dtau - 0.5 * psi * divvi;
        dtclean = p.C_cour * h / (vclean + TINY_D);
      }
    }
    const double vsigdtc = fmax(vsm, vwave);
    if (vsigdtc > TINY_D) dtc = p.C_cour * h / (vsigdtc * fmax(p.alpha, 1.0));
    if (adiab) {
      const double eni_ = rr[11];
      if (eni_ + dtc * fxyz4 < EPS_D && eni_ > EPS_D) fxyz4 = fxyz4 / (1.0 - dtc * fxyz4 / eni_);
      if (valid) fo[3] = fxyz4;
    }
    if (fabs(f2i) > EPS_D) dtf = p.C_force * sqrt(h / sqrt(f2i));
  }
  if (valid && (dtc < TINY_D || dtc > HUGE_D)) set_error(err, PH_ERR_DT);
  // warp minima on the bit patterns: for the positive timesteps the unsigned
  // order is the numeric order (as the atomic), and no FP64 instruction runs
  unsigned long long a = (unsigned long long)__double_as_longlong(valid ? dtc : HUGE_D);
  unsigned long long b = (unsigned long long)__double_as_longlong(valid ? fmin(dtf, dtclean) : HUGE_D);
  for (int o = 16; o > 0; o >>= 1) {
    a = min(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if (lane_id() == 0) {
    atomicMin(reinterpret_cast<unsigned long long *>(&out.dtmin[0]), a);
    atomicMin(reinterpret_cast<unsigned long long *>(&out.dtmin[1]), b);
  }
  if (ind.ibin) {
    // force.F90:3273-3310: the particle's bin from min(dtc, dtf, dtclean), then
    // the Saitoh-Makino limiter (no more than one bin below any neighbour)
    int nb = 0, cnt = 0, small = 0;
    if (valid) {
      double dti = dtc;
      const double dtitmp = fmin(dtf, dtclean);
      if (dtitmp < dti + TINY_D && dtitmp < p.dtmax) dti = dtitmp;
      int bi = get_newbin(dti, p.dtmax, (int)ind.ibin[pid], ind, small);
      bi = max(bi, (int)psum[FSLOT_NBIN * ps + ip] - 1);
      // a bin above MAXBINS is reported (dt too small, the step stops before
      // its corrector); the stored bin stays within the bin tables
      bi = min(bi, MAXBINS);
      ind.ibin[pid] = (int8_t)bi;
      nb = bi; cnt = 1;
    }
    for (int o = 16; o > 0; o >>= 1) {
      nb = max(nb, __shfl_xor_sync(0xffffffffu, nb, o));
      cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
      small |= __shfl_xor_sync(0xffffffffu, small, o);
    }
    if (lane_id() == 0 && cnt) {
      atomicMax(&ind.counters[0], nb);
      atomicAdd(&ind.counters[1], cnt);
      if (small) atomicOr(&ind.counters[2], 1);
    }
  }
}

// wake the neighbours found by the active particles' force sums
// (force.F90:1346-1353): ibin_wake = max(ibin_wake, ibinnow - 1)
__global__ void k_wake_apply(int nt, const int *perm, const unsigned char *wakemark, int8_t *ibin_wake, int level) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nt || !wakemark[k]) return;
  const int pid = perm[k];
  if ((int)ibin_wake[pid] < level) ibin_wake[pid] = (int8_t)level;
}

// the stripes of each particle summed in stripe order through shared memory
// (the staged window's memory, no longer needed), written to psum by lanes < np
template <bool IND, class Get>
__device__ __forceinline__ void store_pair_sums(PairSmem &sm, int lane, int np, int S, int s0, unsigned am,
                                                double *psum, int64_t ps, Get get) {
  constexpr int RW = IND ? NF + 2 : NF + 1;
  double *red = reinterpret_cast<double *>(&sm.st);
  __syncwarp();
  for (int k = 0; k < RW; ++k) red[lane * RW + k] = get(k);
  __syncwarp();
  if (lane < np) {
    double fs[NF];
    for (int k = 0; k < NF; ++k) fs[k] = 0.0;
    double vsm = 0.0, nb = 0.0;
    for (int q = 0; q < S; ++q) {
      const double *src = red + (lane * S + q) * RW;
      for (int k = 0; k < NF; ++k) fs[k] += src[k];
      vsm = fmax(vsm, src[NF]);
      if (IND) nb = fmax(nb, src[NF + 1]);
    }
    const size_t ip = (size_t)(s0 + (IND ? cell_pos(am, lane) : lane));
    for (int k = 0; k < NF; ++k) psum[k * ps + ip] = fs[k];
    psum[FSLOT_VSIG * ps + ip] = vsm;
    if (IND) psum[FSLOT_NBIN * ps + ip] = nb;
  }
}

// max of two non-negative doubles on the integer pipe (signal speeds: the
// FP64 max would occupy the scarce FP64 pipe)
__device__ __forceinline__ double fmax_pos(double a, double b) {
  return __longlong_as_double(max(__double_as_longlong(a), __double_as_longlong(b)));
}

// ------------------------------------------------------------------ FP64 pair terms
// The i-side quantities of the FP64 pair loop (start_cell force.F90:2270-2340
// and compute_cell :2606-2629) for tree position i.
struct IFp64 {
  double hi, hi1, hi21, rhoi, rho1i, rho21i, pri, csi;
  double bxi, byi, bzi, psii, vxi, vyi, vzi, eni;
  double sxx, sxy, sxz, syy, syz, szz, pro2i, vwavei;
  double gradsofti, hfacgrkern, mrhoi5, auterm, avBterm, alphai;
  double xi, yi, zi;
};

template <bool MHD, bool GRAV>
__device__ __forceinline__ IFp64 ifp64_init(const Params &p, int i, const double *tx, const double *ty,
                                            const double *tz, const double *th, const double *jrec,
                                            const double *jmhd, const double *eos_t) {
  IFp64 I;
  const double pm = p.massoftype;
  I.hi = th[i];
  I.hi1 = 1.0 / fabs(I.hi);
  const double t3 = p.hfact * I.hi1;
  I.rhoi = pm * (t3 * t3 * t3);
  I.rho1i = 1.0 / I.rhoi;
  const double *ri = jrec + JREC * (size_t)i;
  I.pri = eos_t[2 * (size_t)i]; I.csi = eos_t[2 * (size_t)i + 1];
  I.bxi = 0; I.byi = 0; I.bzi = 0; I.psii = 0;
  if (MHD) {
    // B_i = Bevol_i * rho_i with rho_i from rhoanddhdrho (force.F90:2309-2311)
    const double *m = jmhd + JMHD * (size_t)i;
    I.bxi = m[10] * I.rhoi; I.byi = m[11] * I.rhoi; I.bzi = m[12] * I.rhoi;
    I.psii = m[3];
  }
  I.vxi = ri[8]; I.vyi = ri[9]; I.vzi = ri[10]; I.eni = ri[11];
  {
    double s[6];
    get_stress(p, I.pri, I.csi, I.rhoi, I.rho1i, I.bxi, I.byi, I.bzi, I.pro2i, I.vwavei, s);
    I.sxx = s[0]; I.sxy = s[1]; I.sxz = s[2]; I.syy = s[3]; I.syz = s[4]; I.szz = s[5];
  }
  const double gradhraw = ri[7];
  const double gradhi = (gradhraw > 0.0) ? gradhraw : 1.0;
  I.gradsofti = GRAV ? ri[12] : 0.0;
  I.hi21 = I.hi1 * I.hi1;
  const double hi41 = I.hi21 * I.hi21;
  I.hfacgrkern = hi41 * CNORMK * gradhi;
  I.rho21i = I.rho1i * I.rho1i;
  I.mrhoi5 = 0.5 * pm * I.rho1i;
  I.auterm = I.mrhoi5 * p.alphau;
  I.avBterm = I.mrhoi5 * p.alphaB * I.rho1i;
  I.alphai = jrec[JREC * (size_t)i + 14];
  I.xi = tx[i]; I.yi = ty[i]; I.zi = tz[i];
  return I;
}

// j-side pair sums of the symmetric evaluation: the force components, d(rho)/dt
// (f[4]), du/dt dissipation (f[5]) and conductivity (f[6]), then with MHD the
// divBsymm, dB/dt and div B diffusion terms, and the signal speed (last)
template <bool MHD>
struct NJS { static constexpr int n = MHD ? 12 : 7; };
// the psum slot of each j-side value
__device__ __forceinline__ int njs_slot(int v, bool mhd) {
  const int last = mhd ? 11 : 6;
  if (v == last) return NF;  // FSLOT_VSIG
  return v < 3 ? v : v + 1;  // 0,1,2 -> 0,1,2; 3.. -> 4..
}

// One trial pair (i, j) of compute_forces (force.F90:914-2060) in FP64 with the
// reference's neighbour test and cached-position rule; n is j's position in
// i's trial list. The i-side sums go to f / vsigmax / nbi. With SYM the pair's
// contribution to j's own sums (j's force loop over i, the same pair term seen
// from j) is returned in jv; it is only requested for pairs without gravity
// and with global timesteps.
template <bool MHD, bool GRAV, bool IND, bool SYM>
__device__ __forceinline__ void force_pair_fp64(const Params &p, const IFp64 &I, int n, int j, int code,
                                                const double *tx, const double *ty, const double *tz,
                                                const double *jrec, const double *jmhd,
                                                const int8_t *ibin_old_t, unsigned char *wakemark,
                                                double (&f)[NF], double &vsigmax, int &nbi,
                                                double (&jv)[NJS<MHD>::n]) {
  const double pm = p.massoftype;
  const bool adiab = !p.isothermal;
  const double beta = p.beta;
  const double ox = offset_of(code, 0, p.dxbound), oy = offset_of(code, 1, p.dybound),
               oz = offset_of(code, 2, p.dzbound);
  double dx, dy, dz;
  if (n < CELLCACHE && code != 0) {
    dx = dsub(I.xi, dadd(tx[j], ox)); dy = dsub(I.yi, dadd(ty[j], oy)); dz = dsub(I.zi, dadd(tz[j], oz));
  } else {
    dx = dsub(I.xi, tx[j]); dy = dsub(I.yi, ty[j]); dz = dsub(I.zi, tz[j]);
  }
  dx = wrap(dx, p.dxbound, p.hdlx, p.periodic); dy = wrap(dy, p.dybound, p.hdly, p.periodic);
      dz = wrap(dz, p.dzbound, p.hdlz, p.periodic);
  const double rij2 = r2_exact(dx, dy, dz);
  const double *rj = jrec + JREC * (size_t)j;
  const double hj1 = rj[0];
  const double q2i = dmul(rij2, I.hi21);
  const double hj21 = dmul(hj1, hj1);
  const double q2j = dmul(rij2, hj21);
  const bool qi_in = q2i < RADKERN2, qj_in = q2j < RADKERN2;
  if (qi_in || qj_in) {
    if (IND) {  // force.F90:1346-1353: j is woken for the next step; the limiter's neighbour bin
      wakemark[j] = 1;
      nbi = max(nbi, (int)ibin_old_t[j]);
    }
    double rij1, qi;
    if (rij2 > TINY_D) { rij1 = rsqrt(rij2); qi = (rij2 * rij1) * I.hi1; }
    else { rij1 = 0.0; qi = 0.0; }
    double grkerni = 0.0, fgravi = 0.0, phii = 0.0;
    if (qi_in) {
      grkerni = grkern(qi) * I.hfacgrkern;
      if (GRAV) {
        double fmi;
        kernel_softening(q2i, qi, phii, fmi);
        phii = phii * I.hi1;
        fmi = fmi * I.hi21;
        fgravi = fmi + I.gradsofti * grkerni;
      }
    } else if (GRAV) {
      phii = -rij1; fgravi = rij1 * rij1;
    }
    const double runix = dx * rij1, runiy = dy * rij1, runiz = dz * rij1;
    double grkernj = 0.0, fgravj = 0.0;
    bool usej;
    if (qj_in) {
      const double qj = (rij2 * rij1) * hj1;
      grkernj = grkern(qj) * hj21 * hj21 * CNORMK * rj[7];
      if (GRAV) {
        double phij, fmj;
        kernel_softening(q2j, qj, phij, fmj);
        fgravj = fmj * hj21 + rj[12] * grkernj;
      }
      usej = true;
    } else {
      if (GRAV) fgravj = rij1 * rij1;
      usej = false;
    }
    if (MHD) usej = true;
    if (adiab && !GRAV) usej = true;
    // seen from j, i's terms are used when q_i < 2 (or always, as usej)
    const bool usei = qi_in || MHD || (adiab && !GRAV);
    const double fgrav = GRAV ? 0.5 * (pm * fgravi + pm * fgravj) : 0.0;
    const double dvx = I.vxi - rj[8], dvy = I.vyi - rj[9], dvz = I.vzi - rj[10];
    const double projv = dvx * runix + dvy * runiy + dvz * runiz;
    const double denij = adiab ? I.eni - rj[11] : 0.0;
    const double vsigi = fmax(I.vwavei - beta * projv, 0.0);
    const double vsigavi = fmax(I.alphai * I.vwavei - beta * projv, 0.0);
    vsigmax = fmax_pos(vsigmax, vsigi);
    double rho1j = 0, rho21j = 0, pro2j = 0, vwavej = 0, autermj = 0, avBtermj = 0, vsigavj = 0, prj = 0;
    double vsigj = 0.0;
    double rhoj = rj[1];
    if (usej || SYM) {
      rho1j = rj[2]; rho21j = rj[15]; pro2j = rj[3]; vwavej = rj[4]; prj = rj[5];
      autermj = rj[6]; avBtermj = rj[13];
      vsigj = fmax(vwavej - beta * projv, 0.0);
      vsigavj = fmax(rj[14] * vwavej - beta * projv, 0.0);  // alphaj = alphaind(1,j)
      if (usej) vsigmax = fmax_pos(vsigmax, vsigj);
    }
    double qrho2i = 0.0, qrho2j = 0.0;
    if (projv < 0.0) {
      qrho2i = -0.5 * I.rho1i * vsigavi * projv;
      if (usej || SYM) qrho2j = -0.5 * rho1j * vsigavj * projv;
    }
    const double dudtdissi = pm * qrho2i * projv * grkerni;
    const double gradpi = pm * (I.pro2i + qrho2i) * grkerni;
    const double gradpj = usej ? pm * (pro2j + qrho2j) * grkernj : 0.0;
    double dendiss = 0.0;
    if (adiab) {
      double vsigu;
      if (GRAV) vsigu = fabs(projv);
      else vsigu = sqrt(fabs(I.pri - prj) * (2.0 / (I.rhoi + rhoj)));
      dendiss = vsigu * denij * (I.auterm * grkerni + autermj * grkernj);
    }
    double projsx = 0, projsy = 0, projsz = 0, dudtresist = 0.0;
    if (MHD) {
      const double *mj = jmhd + JMHD * (size_t)j;
      const double bxj = mj[0], byj = mj[1], bzj = mj[2], psij = mj[3];
      const double dBx = I.bxi - bxj, dBy = I.byi - byj, dBz = I.bzi - bzj;
      const double projBi = I.bxi * runix + I.byi * runiy + I.bzi * runiz;
      const double projBj = bxj * runix + byj * runiy + bzj * runiz;
      const double projdB = dBx * runix + dBy * runiy + dBz * runiz;
      const double dB2 = dBx * dBx + dBy * dBy + dBz * dBz;
      f[11] += -pm * projdB * grkerni;  // divBdiffterm
      const double tx_ = dvx - projv * runix, ty_ = dvy - projv * runiy, tz_ = dvz - projv * runiz;
      const double vsigB = sqrt(tx_ * tx_ + ty_ * ty_ + tz_ * tz_);
      const double dBdiss = (I.avBterm * grkerni + avBtermj * grkernj) * vsigB;
      if (p.iresistive_heating > 0 && adiab) dudtresist = -0.5 * dB2 * dBdiss;
      const double pmi = pm * I.rho21i * grkerni, pmj = pm * rho21j * grkernj;
      const double termi = pmi * projBi;
      const double f7 = termi + pmj * projBj;
      f[7] += f7;  // divBsymmterm
      const double dpsi = p.overcleanfac * (pmi * I.psii * I.vwavei + pmj * psij * vwavej);
      f[8] += -termi * dvx + dBdiss * dBx - dpsi * runix;
      f[9] += -termi * dvy + dBdiss * dBy - dpsi * runiy;
      f[10] += -termi * dvz + dBdiss * dBz - dpsi * runiz;
      projsx = (I.sxx * runix + I.sxy * runiy + I.sxz * runiz) * grkerni +
               (mj[4] * runix + mj[5] * runiy + mj[6] * runiz) * grkernj;
      projsy = (I.sxy * runix + I.syy * runiy + I.syz * runiz) * grkerni +
               (mj[5] * runix + mj[7] * runiy + mj[8] * runiz) * grkernj;
      projsz = (I.sxz * runix + I.syz * runiy + I.szz * runiz) * grkerni +
               (mj[6] * runix + mj[8] * runiy + mj[9] * runiz) * grkernj;
      if (SYM) {
        // from j: r -> -r, dv -> -dv, dB -> -dB; its own term -pmj (B_j . r) dv
        const double termj = pmj * projBj;
        jv[6] = -f7;
        jv[7] = -termj * dvx - dBdiss * dBx + dpsi * runix;
        jv[8] = -termj * dvy - dBdiss * dBy + dpsi * runiy;
        jv[9] = -termj * dvz - dBdiss * dBz + dpsi * runiz;
        jv[10] = -pm * projdB * grkernj;
      }
    }
    // the zero terms of a build without gravity or MHD are not added (x + 0 = x)
    const double gp = GRAV ? (gradpi + gradpj) + fgrav : gradpi + gradpj;
    double fx = -runix * gp, fy = -runiy * gp, fz = -runiz * gp;
    if (MHD) { fx -= projsx; fy -= projsy; fz -= projsz; }
    f[0] += fx; f[1] += fy; f[2] += fz;
    if (GRAV) f[3] += pm * phii;
    f[4] += projv * grkerni;
    if (adiab) { f[5] += MHD ? dudtdissi + dudtresist : dudtdissi; f[6] += dendiss; }
    if (SYM) {
      jv[0] = -fx; jv[1] = -fy; jv[2] = -fz;
      jv[3] = projv * grkernj;
      if (adiab) {
        const double dj = pm * qrho2j * projv * grkernj;
        jv[4] = MHD ? dj + dudtresist : dj;
        jv[5] = -dendiss;
      } else {
        jv[4] = 0.0; jv[5] = 0.0;
      }
      jv[NJS<MHD>::n - 1] = usei ? fmax_pos(vsigj, vsigi) : vsigj;
    }
  } else if (GRAV) {
    // plain 1/r^2 for trial pairs outside both kernels (force.F90:1991-2053)
    const double rij1 = 1.0 / sqrt(rij2);
    const double fgj = rij1 * rij1 * rij1 * pm;
    f[0] -= dx * fgj; f[1] -= dy * fgj; f[2] -= dz * fgj;
    f[3] += pm * (-rij1);
  } else if (SYM) {
    for (int v = 0; v < NJS<MHD>::n; ++v) jv[v] = 0.0;
  }
}

template <bool MHD, bool GRAV, bool IND>
__global__ void __launch_bounds__(32 * MAX_WARPS) k_force(
    Params p, const Node *nodes, const int *leaves, int ncell, const LeafEntry *pool, const int *cell_off,
    const int *cell_nleaf, const int *perm, const double *tx, const double *ty, const double *tz, const double *th,
    const float4 *txf, const double *jrec, const double *jmhd, const double *eos_t, ForceOut out, double *psum,
    int64_t ps, double pf_hmin,
    const int *cells, const unsigned char *actf, const int8_t *ibin_old_t,
    unsigned char *wakemark, int *err) {
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int a = blockIdx.x * (blockDim.x >> 5) + w;
  if (a >= ncell) return;
  const int cell = cells ? cells[a] : a;  // individual timesteps: the cells holding active particles
  const Node nd = nodes[leaves[cell]];
  const int np_all = nd.count, s0 = nd.start;
  if (np_all < 1 || np_all > MAXCELL) { if (lane == 0) set_error(err, PH_ERR_TREE); return; }
  // individual timesteps (IND): the cell's active particles take the lanes;
  // inactive ones keep their forces
  int np = np_all;
  unsigned am = 0u;
  if (IND) am = cell_active_mask(actf, s0, np_all, np);
  if (np == 0) return;
  const int S = 32 / np;
  const bool act = lane < np * S;
  const int il = act ? lane / S : 0, stripe = act ? lane % S : 0;
  const int i = s0 + (IND ? cell_pos(am, il) : il);
  const IFp64 I = ifp64_init<MHD, GRAV>(p, i, tx, ty, tz, th, jrec, jmhd, eos_t);
  const float4 xif = txf[i];
  const float hi21f = (float)I.hi21;
  const bool pf_i = (I.hi > pf_hmin) && !GRAV;
  const float q2lim = 4.0f * 1.001f;
  const float pf_h1max = (float)(1.0 / pf_hmin);
  double f[NF];
  for (int k = 0; k < NF; ++k) f[k] = 0.0;
  double vsigmax = 0.0;
  int nbi = 0;  // largest ibin_old of the SPH neighbours (individual timesteps)
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
  if (lane == 0) {
    atomicAdd(&out.stats[8], (unsigned long long)out.cell_ntrial[cell]);
    atomicAdd(&out.stats[10], (unsigned long long)np * (unsigned long long)out.cell_ntrial[cell]);
  }
  const int ntrial = out.cell_ntrial[cell];
  extern __shared__ __align__(16) unsigned char dsm[];
  PairSmem &sm = reinterpret_cast<PairSmem *>(dsm)[w];
  Stage &stg = sm.st;
  for (int base = 0; base < ntrial; base += STAGE) {
    const int cnt = stage_window(p, pool, off, nleaf, ntrial, base, txf, stg);
    auto test = [&](int k) -> bool {
      if (stg.jidx[k] == i) return false;
      if (!pf_i) return true;
      const float4 xj = stg.pos[k];  // x, y, z (+ offset), 1/h
      if (xj.w >= pf_h1max) return true;
      float dxf = xif.x - xj.x, dyf = xif.y - xj.y, dzf = xif.z - xj.z;
      if (p.periodic) {
        if (fabsf(dxf) > 0.5f * p.dxboundf) dxf -= copysignf(p.dxboundf, dxf);
        if (fabsf(dyf) > 0.5f * p.dyboundf) dyf -= copysignf(p.dyboundf, dyf);
        if (fabsf(dzf) > 0.5f * p.dzboundf) dzf -= copysignf(p.dzboundf, dzf);
      }
      const float r2f = dxf * dxf + dyf * dyf + dzf * dzf;
      return r2f * fminf(hi21f, xj.w * xj.w) < q2lim;
    };
    auto body = [&](int k) {
      double jv[NJS<MHD>::n];
      force_pair_fp64<MHD, GRAV, IND, false>(p, I, base + k, stg.jidx[k], stg.code[k], tx, ty, tz, jrec, jmhd,
                                             ibin_old_t, wakemark, f, vsigmax, nbi, jv);
    };
    queue_window(cnt, S, act, il, stripe, sm.q, test, body);
  }
  store_pair_sums<IND>(sm, lane, np, S, s0, am, psum, ps, [&](int q) -> double {
    return q < NF ? f[q] : (q == NF ? vsigmax : (double)nbi);
  });
}

// ------------------------------------------------------------------ symmetric FP64 pair loop
// Each unordered neighbour pair evaluated once (FP64, hydro and ideal MHD
// without self-gravity, global timesteps). A pair (i, j) of leaf cells A, B is
// evaluated by the cell whose leaf starts first in tree order: A takes the
// entries of its trial list whose first particle is at or after its own,
// which is a prefix of the list (the list is in decreasing order of first
// particle, the reference's stack order), and within its own leaf the pairs
// j > i. Every neighbour pair (q_i < 2 or q_j < 2) lies in both cells' trial
// lists (the walk opens every node within 2 max(h_i, h_j) of a cell), so it is
// evaluated exactly once; an entry present in one list only holds no
// neighbour pair and contributes nothing.
//
// The i-side sums are kept per lane as in k_force. The pair's contribution to
// j's sums is the same pair term seen from j (the reference evaluates it again
// in j's loop): it is added, in a fixed order, into a per-window array of the
// warp (lanes holding the same j are combined in lane order first), and each
// window's array is written to jbuf at j's flattened trial index of A's list.
// k_force_gather then adds, for every particle, the contributions that the
// cells before it left for it, in its own list's order. Pair terms and
// neighbour tests are those of force_pair_fp64 (the reference's rounding and
// cached-position rule from the evaluating cell's list); seen from j they differ
// from the reference's own evaluation by rounding only.
constexpr int STAGE_S = 128;
template <bool MHD>
struct SymSmem {
  union {
    StageN<STAGE_S> st;
    double red[32 * (NF + 1)];
  } u;
  PairQ q;
  double js[NJS<MHD>::n][STAGE_S];
};

template <bool MHD>
__global__ void __launch_bounds__(32 * MAX_WARPS) k_force_sym(
    Params p, const Node *nodes, const int *leaves, int ncell, const LeafEntry *pool, const int *cell_off,
    const int *cell_nleaf, const double *tx, const double *ty, const double *tz, const double *th,
    const float4 *txf, const double *jrec, const double *jmhd, const double *eos_t, ForceOut out, double *psum,
    int64_t ps, double pf_hmin, const int *toff, double *jbuf, int64_t jstride, int *err) {
  constexpr int NJ = NJS<MHD>::n;
  const unsigned FULL = 0xffffffffu;
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int cell = blockIdx.x * (blockDim.x >> 5) + w;
  if (cell >= ncell) return;
  const Node nd = nodes[leaves[cell]];
  const int np = nd.count, s0 = nd.start;
  if (np < 1 || np > MAXCELL) { if (lane == 0) set_error(err, PH_ERR_TREE); return; }
  const int S = 32 / np;
  const bool act = lane < np * S;
  const int il = act ? lane / S : 0, stripe = act ? lane % S : 0;
  const int i = s0 + il;
  const IFp64 I = ifp64_init<MHD, false>(p, i, tx, ty, tz, th, jrec, jmhd, eos_t);
  const float4 xif = txf[i];
  const float hi21f = (float)I.hi21;
  const bool pf_i = I.hi > pf_hmin;
  const float q2lim = 4.0f * 1.001f;
  const float pf_h1max = (float)(1.0 / pf_hmin);
  double f[NF];
  for (int k = 0; k < NF; ++k) f[k] = 0.0;
  double vsigmax = 0.0;
  int nbi = 0;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
  // the owned prefix of the list: entries starting at or after s0
  int nown = 0, town = 0;
  for (int e0 = 0; e0 < nleaf; e0 += 32) {
    const int e = e0 + lane;
    LeafEntry le{0, 0};
    if (e < nleaf) le = pool[off + e];
    const bool own = e < nleaf && le.start >= s0;
    nown += __popc(__ballot_sync(FULL, own));
    town += warp_sum_int(own ? (le.cc & 255) : 0);
    if (!__all_sync(FULL, e >= nleaf || own)) break;
  }
  if (lane == 0) {
    atomicAdd(&out.stats[8], (unsigned long long)out.cell_ntrial[cell]);
    atomicAdd(&out.stats[10], (unsigned long long)np * (unsigned long long)town);
  }
  const int64_t tb = (int64_t)toff[off];  // flattened trial index of the list's first entry
  extern __shared__ __align__(16) unsigned char dsm[];
  SymSmem<MHD> &sm = reinterpret_cast<SymSmem<MHD> *>(dsm)[w];
  StageN<STAGE_S> &stg = sm.u.st;
  const unsigned gmask = !act ? 0u : (S >= 32 ? FULL : (((1u << S) - 1u) << (il * S)));
  const unsigned lt = (1u << lane) - 1u;
  for (int base = 0; base < town; base += STAGE_S) {
    const int cnt = stage_window_n<STAGE_S>(p, pool, off, nown, town, base, txf, stg);
    for (int q = lane; q < NJ * STAGE_S; q += 32) (&sm.js[0][0])[q] = 0.0;
    __syncwarp();
    auto test = [&](int k) -> bool {
      const int j = stg.jidx[k];
      if (j <= i && j >= s0) return false;  // own leaf: each pair once (j > i); the self pair never
      if (!pf_i) return true;
      const float4 xj = stg.pos[k];
      if (xj.w >= pf_h1max) return true;
      float dxf = xif.x - xj.x, dyf = xif.y - xj.y, dzf = xif.z - xj.z;
      if (p.periodic) {
        if (fabsf(dxf) > 0.5f * p.dxboundf) dxf -= copysignf(p.dxboundf, dxf);
        if (fabsf(dyf) > 0.5f * p.dyboundf) dyf -= copysignf(p.dyboundf, dyf);
        if (fabsf(dzf) > 0.5f * p.dzboundf) dzf -= copysignf(p.dzboundf, dzf);
      }
      const float r2f = dxf * dxf + dyf * dyf + dzf * dzf;
      return r2f * fminf(hi21f, xj.w * xj.w) < q2lim;
    };
    // the test sweep and per-particle queues of queue_window; the drain runs
    // in warp-uniform steps so that lanes holding the same j can be combined
    const int nr = (cnt + S - 1) / S;
    int qn = 0;
    for (int r = 0; r < nr; ++r) {
      const int k = r * S + stripe;
      const bool ok = act && k < cnt && test(k);
      const unsigned b = __ballot_sync(FULL, ok);
      if (ok) sm.q.k[il][qn + __popc(b & gmask & lt)] = (unsigned short)k;
      qn += __popc(b & gmask);
      if (r == nr - 1 || (int)__reduce_max_sync(FULL, (unsigned)qn) > QCAP - S) {
        __syncwarp();
        const int nst = (act && qn > stripe) ? (qn - stripe + S - 1) / S : 0;
        const int nstmax = (int)__reduce_max_sync(FULL, (unsigned)nst);
        // the particles of a cell accept nearly the same j in nearly the same
        // order, so aligned queues would put the same j in many lanes at once;
        // each particle starts at its own rotation of its queue instead
        const int rot = act && qn > 0 ? (il * qn) / np : 0;
        for (int t = 0; t < nstmax; ++t) {
          int m = stripe + t * S + rot;
          if (m >= qn) m -= qn;
          const bool valid = t < nst;
          const int kk = valid ? (int)sm.q.k[il][m] : -1;
          double jv[NJ];
          for (int v = 0; v < NJ; ++v) jv[v] = 0.0;
          if (valid)
            force_pair_fp64<MHD, false, false, true>(p, I, base + kk, stg.jidx[kk], stg.code[kk], tx, ty, tz, jrec,
                                                     jmhd, nullptr, nullptr, f, vsigmax, nbi, jv);
          // lanes holding the same j: the lowest adds the others' values in
          // lane order, then adds the group's sum to j's window slot
          const unsigned g = __match_any_sync(FULL, valid ? kk : -1 - lane);
          const int gs = __popc(g);
          const int gmax = (int)__reduce_max_sync(FULL, (unsigned)gs);
          const bool lead = valid && (g & lt) == 0u;
          for (int u = 1; u < gmax; ++u) {
            const int src = u < gs ? (int)__fns(g, 0, u + 1) : lane;
            for (int v = 0; v < NJ - 1; ++v) {
              const double y = __shfl_sync(FULL, jv[v], src);
              if (lead && u < gs) jv[v] += y;
            }
            const double y = __shfl_sync(FULL, jv[NJ - 1], src);
            if (lead && u < gs) jv[NJ - 1] = fmax_pos(jv[NJ - 1], y);
          }
          if (lead) {
            for (int v = 0; v < NJ - 1; ++v) sm.js[v][kk] += jv[v];
            sm.js[NJ - 1][kk] = fmax_pos(sm.js[NJ - 1][kk], jv[NJ - 1]);
          }
          __syncwarp();
        }
        qn = 0;
      }
    }
    __syncwarp();
    // this window's j-side sums -> jbuf (value-major, flattened trial index)
    for (int v = 0; v < NJ; ++v)
      for (int k = lane; k < cnt; k += 32) jbuf[(int64_t)v * jstride + tb + base + k] = sm.js[v][k];
    __syncwarp();
  }
  // the stripes of each particle in stripe order (store_pair_sums)
  constexpr int RW = NF + 1;
  double *red = sm.u.red;
  __syncwarp();
  for (int k = 0; k < RW; ++k) red[lane * RW + k] = k < NF ? f[k] : vsigmax;
  __syncwarp();
  if (lane < np) {
    double fs[NF];
    for (int k = 0; k < NF; ++k) fs[k] = 0.0;
    double vsm = 0.0;
    for (int q = 0; q < S; ++q) {
      const double *src = red + (lane * S + q) * RW;
      for (int k = 0; k < NF; ++k) fs[k] += src[k];
      vsm = fmax(vsm, src[NF]);
    }
    const size_t ip = (size_t)(s0 + lane);
    for (int k = 0; k < NF; ++k) psum[k * ps + ip] = fs[k];
    psum[FSLOT_VSIG * ps + ip] = vsm;
  }
}

// Per leaf cell B: add to its particles' pair sums the j-side contributions
// that k_force_sym left in jbuf: its own leaf's (the self entry) and those of
// every cell A before it in tree order whose list holds B (found by a binary
// search of A's list, which is in decreasing order of first particle), in the
// order of B's own trial list.
template <bool MHD>
__global__ void k_force_gather(const Node *nodes, const int *leaves, int ncell, const LeafEntry *pool,
                               const int *cell_off, const int *cell_nleaf, const int *cell_at, const int *toff,
                               const double *jbuf, int64_t jstride, double *psum, int64_t ps, int *err) {
  constexpr int NJ = NJS<MHD>::n;
  const unsigned FULL = 0xffffffffu;
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int cell = blockIdx.x * (blockDim.x >> 5) + w;
  if (cell >= ncell) return;
  const Node nd = nodes[leaves[cell]];
  const int np = nd.count, s0 = nd.start;
  if (np < 1 || np > MAXCELL) return;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
  // per lane: the sums of (value v, particle t) pairs c = lane, lane + 32, ...
  constexpr int NC = (NJ * MAXCELL + 31) / 32;
  double acc[NC];
  for (int r = 0; r < NC; ++r) acc[r] = 0.0;
  // incoming entries: the suffix of B's list starting at or before s0
  for (int e0 = nleaf - 1; e0 >= 0; e0 -= 32) {
    // lanes take entries e0, e0-1, ... (descending index = ascending start),
    // then the warp walks them back in list order
    const int e = e0 - lane;
    int slot = -1;
    bool in = false;
    if (e >= 0) {
      const LeafEntry le = pool[off + e];
      in = le.start <= s0;
      if (le.start == s0) {
        slot = toff[off + e];
      } else if (in) {
        const int A = cell_at[le.start];
        const int aoff = cell_off[A];
        int lo = 0, hi = cell_nleaf[A] - 1;
        while (lo <= hi) {  // A's list: starts in decreasing order
          const int mid = (lo + hi) >> 1;
          const int st = pool[aoff + mid].start;
          if (st == s0) { slot = toff[aoff + mid]; break; }
          if (st > s0) lo = mid + 1; else hi = mid - 1;
        }
      }
    }
    const unsigned inb = __ballot_sync(FULL, in);
    const int nin = __popc(inb);  // a prefix of the lanes (suffix of the list)
    for (int q = nin - 1; q >= 0; --q) {  // in list order (lane nin-1 holds the first incoming entry)
      const int sl = __shfl_sync(FULL, slot, q);
      if (sl < 0) continue;
      for (int r = 0; r < NC; ++r) {
        const int c = lane + 32 * r;
        const int v = c / MAXCELL, t = c % MAXCELL;
        if (v < NJ && t < np) {
          const double y = jbuf[(int64_t)v * jstride + sl + t];
          acc[r] = (v == NJ - 1) ? fmax_pos(acc[r], y) : acc[r] + y;
        }
      }
    }
    if (nin < 32) break;  // the rest of the list starts after s0
  }
  for (int r = 0; r < NC; ++r) {
    const int c = lane + 32 * r;
    const int v = c / MAXCELL, t = c % MAXCELL;
    if (v < NJ && t < np) {
      double *dst = psum + (int64_t)njs_slot(v, MHD) * ps + s0 + t;
      *dst = (v == NJ - 1) ? fmax_pos(*dst, acc[r]) : *dst + acc[r];
    }
  }
}

// trial entries each cell evaluates in the symmetric loop: those of its list
// entries starting at or after its own first particle
__global__ void k_owned_trials(const Node *nodes, const int *leaves, int ncell, const LeafEntry *pool,
                               const int *cell_off, const int *cell_nleaf, int *town) {
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int cell = blockIdx.x * (blockDim.x >> 5) + w;
  if (cell >= ncell) return;
  const int s0 = nodes[leaves[cell]].start;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
  int t = 0;
  for (int e = lane; e < nleaf; e += 32) {
    const LeafEntry le = pool[off + e];
    if (le.start >= s0) t += le.cc & 255;
  }
  t = warp_sum_int(t);
  if (lane == 0) town[cell] = t;
}

// flattened trial index of every pool entry: the cell's base (scan of the
// cells' trial counts) plus the counts of the entries before it in its list
__global__ void k_entry_offsets(int ncell, const int *cell_off, const int *cell_nleaf, const int *cell_tbase,
                                const LeafEntry *pool, int *toff) {
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int cell = blockIdx.x * (blockDim.x >> 5) + w;
  if (cell >= ncell) return;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
  int acc = cell_tbase[cell];
  for (int e0 = 0; e0 < nleaf; e0 += 32) {
    const int e = e0 + lane;
    const int cnt = e < nleaf ? (pool[off + e].cc & 255) : 0;
    int x = cnt;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (e < nleaf) toff[off + e] = acc + x - cnt;
    acc += __shfl_sync(0xffffffffu, x, 31);
  }
}

// cell index of every leaf, at the tree position of its first particle
__global__ void k_cell_at(const Node *nodes, const int *leaves, int ncell, int *cell_at) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell < ncell) cell_at[nodes[leaves[cell]].start] = cell;
}

// ------------------------------------------------------------------ mixed precision
// Precision form: the pair separation is formed in FP64 (positions stay FP64)
// and rounded to FP32; W, grad W and every pair term are evaluated in FP32
// and accumulated per particle in FP32 with compensated (Kahan) summation. The
// per-particle finish (accelerations, du/dt, dB/dt, timesteps) is FP64.

__device__ __forceinline__ float grkernf(float q) {
  if (q < 1.0f) return q * (2.25f * q - 3.0f);
  if (q < 2.0f) { float t = q - 2.0f; return -0.75f * (t * t); }
  return 0.0f;
}
// kernel_softening in FP32. For 1 <= q < 2 the reference's polynomials
// cancel to a few digits near q = 2 (numerators ~30 out of terms ~1000), so
// they are evaluated in t = 2 - q, where they read
//   30 q^2 fs = 30 - 30 t^4 + 24 t^5 - 5 t^6,  30 q pot = -30 + 3 t^5 - t^6
// (the same polynomials, expanded about q = 2).
__device__ __forceinline__ void kernel_softeningf(float q2, float q, float &pot, float &fs) {
  if (q < 1.0f) {
    float q4 = q2 * q2;
    pot = q4 * q * 0.1f - 0.3f * q4 + (2.0f / 3.0f) * q2 - 1.4f;
    fs = q * (15.0f * q2 * q - 36.0f * q2 + 40.0f) * (1.0f / 30.0f);
  } else if (q < 2.0f) {
    const float t = 2.0f - q, t4 = (t * t) * (t * t);
    const float q1 = 1.0f / q;
    pot = (-1.0f + t4 * t * (0.1f - t * (1.0f / 30.0f))) * q1;
    fs = (1.0f - t4 * (1.0f - t * (0.8f - t * (1.0f / 6.0f)))) * (q1 * q1);
  } else {
    pot = -1.0f / q;
    fs = 1.0f / q2;
  }
}


template <bool MHD, bool GRAV, bool IND>
__global__ void __launch_bounds__(32 * MAX_WARPS) k_force_mixed(
    Params p, const Node *nodes, const int *leaves, int ncell, const LeafEntry *pool, const int *cell_off,
    const int *cell_nleaf, const int *perm, const double *tx, const double *ty, const double *tz, const double *th,
    const float4 *txf, const double *jrec, const double *jmhd, const float *jrecf, const float *jmhdf,
    const double *eos_t, ForceOut out, double *psum, int64_t ps, const int *cells, const unsigned char *actf, const int8_t *ibin_old_t,
    unsigned char *wakemark, int *err) {
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int a = blockIdx.x * (blockDim.x >> 5) + w;
  if (a >= ncell) return;
  const int cell = cells ? cells[a] : a;  // individual timesteps: the cells holding active particles
  const Node nd = nodes[leaves[cell]];
  const int np_all = nd.count, s0 = nd.start;
  if (np_all < 1 || np_all > MAXCELL) { if (lane == 0) set_error(err, PH_ERR_TREE); return; }
  // individual timesteps (IND): the cell's active particles take the lanes;
  // inactive ones keep their forces
  int np = np_all;
  unsigned am = 0u;
  if (IND) am = cell_active_mask(actf, s0, np_all, np);
  if (np == 0) return;
  const int S = 32 / np;
  const bool act = lane < np * S;
  const int il = act ? lane / S : 0, stripe = act ? lane % S : 0;
  const int i = s0 + (IND ? cell_pos(am, il) : il);
  const float pmf = (float)p.massoftype;
  const bool adiab = !p.isothermal;
  // i-side from the FP32 particle record (its density is rhoh(1/(1/h)) rather
  // than rhoanddhdrho's m (hfact/h)^3: a last-ulp difference in FP64, nil in FP32)
  const float *ri = jrecf + JRECF * (size_t)i;
  const float hi1f = ri[0], hi21f = hi1f * hi1f;
  const float gradhi = (ri[7] > 0.0f) ? ri[7] : 1.0f;
  const float hfacgrkern = hi21f * hi21f * (float)CNORMK * gradhi;
  const float gradsofti = GRAV ? ri[12] : 0.0f;
  const float rhoif = ri[1], rho1if = ri[2], rho21i = ri[15], pro2if = ri[3], vwaveif = ri[4], prif = ri[5];
  const float auterm = ri[6], avBterm = ri[13];
  const float alphai = ri[14], beta = (float)p.beta, ocf = (float)p.overcleanfac;
  const float vxi = ri[8], vyi = ri[9], vzi = ri[10], eni = ri[11];
  float bxif = 0, byif = 0, bzif = 0, psiif = 0, sx[6] = {0, 0, 0, 0, 0, 0};
  if (MHD) {
    const float *mi = jmhdf + JMHDF * (size_t)i;
    bxif = mi[0]; byif = mi[1]; bzif = mi[2]; psiif = mi[3];
    for (int k = 0; k < 6; ++k) sx[k] = mi[4 + k];
  }
  const double xi = tx[i], yi = ty[i], zi = tz[i];
  const float4 xif = txf[i];
  const bool pf_i = !GRAV;
  const float q2lim = 4.0f * 1.001f;
  const float hLx = 0.5f * p.dxboundf, hLy = 0.5f * p.dyboundf, hLz = 0.5f * p.dzboundf;
  Kahan f[NF];
  float vsigmax = 0.0f;
  int nbi = 0;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
  if (lane == 0) {
    atomicAdd(&out.stats[8], (unsigned long long)out.cell_ntrial[cell]);
    atomicAdd(&out.stats[10], (unsigned long long)np * (unsigned long long)out.cell_ntrial[cell]);
  }
  const int ntrial = out.cell_ntrial[cell];
  extern __shared__ __align__(16) unsigned char dsm[];
  PairSmem &sm = reinterpret_cast<PairSmem *>(dsm)[w];
  Stage &stg = sm.st;
  for (int base = 0; base < ntrial; base += STAGE) {
    const int cnt = stage_window(p, pool, off, nleaf, ntrial, base, txf, stg);
    auto test = [&](int k) -> bool {
      if (stg.jidx[k] == i) return false;
      if (!pf_i && !GRAV) return true;
      const float4 xj = stg.pos[k];  // x, y, z (+ offset), 1/h
      const float ux = xif.x - xj.x, uy = xif.y - xj.y, uz = xif.z - xj.z;
      float dxf = ux, dyf = uy, dzf = uz;
      if (p.periodic) {
        if (fabsf(dxf) > hLx) dxf -= copysignf(p.dxboundf, dxf);
        if (fabsf(dyf) > hLy) dyf -= copysignf(p.dyboundf, dyf);
        if (fabsf(dzf) > hLz) dzf -= copysignf(p.dzboundf, dzf);
      }
      const float r2f = dxf * dxf + dyf * dyf + dzf * dzf;
      const bool near = r2f * fminf(hi21f, xj.w * xj.w) < q2lim;
      if (!GRAV || near) return near;
      // self-gravity: a trial pair provably outside both kernels takes only
      // the 1/r^2 term (force.F90:1991-2053, the body's else branch), formed
      // here from the FP64 separation without queueing the pair
      const int j = stg.jidx[k];
      float dx, dy, dz;
      separation_mixed(p, xi, yi, zi, tx[j], ty[j], tz[j], stg.code[k], ux, uy, uz, dx, dy, dz);
      const float rij1 = rsqrt_nr(dx * dx + dy * dy + dz * dz);
      const float fgj = rij1 * rij1 * rij1 * pmf;
      f[0].add(-dx * fgj); f[1].add(-dy * fgj); f[2].add(-dz * fgj);
      f[3].add(-pmf * rij1);
      return false;
    };
    struct PF { int j, code; float4 xj; double x, y, z; float4 r0, r1, r2, r3; };
    auto load = [&](int k) -> PF {
      PF f;
      f.j = stg.jidx[k]; f.code = stg.code[k]; f.xj = stg.pos[k];
      f.x = tx[f.j]; f.y = ty[f.j]; f.z = tz[f.j];
      const float4 *r4 = reinterpret_cast<const float4 *>(jrecf + JRECF * (size_t)f.j);
      f.r0 = r4[0]; f.r1 = r4[1]; f.r2 = r4[2]; f.r3 = r4[3];
      return f;
    };
    auto body = [&](const PF &pf) {
      const int j = pf.j;
      const float4 xj = pf.xj;
      float dx, dy, dz;
      separation_mixed(p, xi, yi, zi, pf.x, pf.y, pf.z, pf.code, xif.x - xj.x, xif.y - xj.y, xif.z - xj.z, dx,
                       dy, dz);
      const float rij2 = dx * dx + dy * dy + dz * dz;
      const float rj[JRECF] = {pf.r0.x, pf.r0.y, pf.r0.z, pf.r0.w, pf.r1.x, pf.r1.y, pf.r1.z, pf.r1.w,
                               pf.r2.x, pf.r2.y, pf.r2.z, pf.r2.w, pf.r3.x, pf.r3.y, pf.r3.z, pf.r3.w};
      const float hj1 = rj[0];
      const float hj21 = hj1 * hj1;
      const float q2i = rij2 * hi21f, q2j = rij2 * hj21;
      const bool qi_in = q2i < 4.0f, qj_in = q2j < 4.0f;
      if (qi_in || qj_in) {
        if (IND) {  // force.F90:1346-1353: j is woken for the next step; the limiter's neighbour bin
          wakemark[j] = 1;
          nbi = max(nbi, (int)ibin_old_t[j]);
        }
        // coincident particles: no direction, rij1 = 0 (force.F90:1293-1298)
        const float rij1 = rij2 > TINY_F ? rsqrt_nr(rij2) : 0.0f;
        const float rij = rij2 * rij1;
        const float qi = rij * hi1f;
        float grkerni = 0.0f, fgravi = 0.0f, phii = 0.0f;
        if (qi_in) {
          grkerni = grkernf(qi) * hfacgrkern;
          if (GRAV) {
            float fmi;
            kernel_softeningf(q2i, qi, phii, fmi);
            phii *= hi1f;
            fgravi = fmi * hi21f + gradsofti * grkerni;
          }
        } else if (GRAV) {
          phii = -rij1; fgravi = rij1 * rij1;
        }
        const float runix = dx * rij1, runiy = dy * rij1, runiz = dz * rij1;
        float grkernj = 0.0f, fgravj = 0.0f;
        bool usej;
        if (qj_in) {
          const float qj = rij * hj1;
          grkernj = grkernf(qj) * (hj21 * hj21 * (float)CNORMK) * rj[7];
          if (GRAV) {
            float phij, fmj;
            kernel_softeningf(q2j, qj, phij, fmj);
            fgravj = fmj * hj21 + rj[12] * grkernj;
          }
          usej = true;
        } else {
          if (GRAV) fgravj = rij1 * rij1;
          usej = false;
        }
        if (MHD) usej = true;
        if (adiab && !GRAV) usej = true;
        const float fgrav = 0.5f * pmf * (fgravi + fgravj);
        const float dvx = vxi - rj[8], dvy = vyi - rj[9], dvz = vzi - rj[10];
        const float projv = dvx * runix + dvy * runiy + dvz * runiz;
        const float denij = adiab ? eni - rj[11] : 0.0f;
        vsigmax = fmaxf(vsigmax, fmaxf(vwaveif - beta * projv, 0.0f));
        const float vsigavi = fmaxf(alphai * vwaveif - beta * projv, 0.0f);
        float rho1j = 0, rho21j = 0, pro2j = 0, vwavej = 0, autermj = 0, avBtermj = 0, vsigavj = 0, prj = 0;
        const float rhoj = rj[1];
        if (usej) {
          rho1j = rj[2]; rho21j = rj[15]; pro2j = rj[3]; vwavej = rj[4]; prj = rj[5];
          autermj = rj[6]; avBtermj = rj[13];
          vsigmax = fmaxf(vsigmax, fmaxf(vwavej - beta * projv, 0.0f));
          vsigavj = fmaxf(rj[14] * vwavej - beta * projv, 0.0f);  // alphaj = alphaind(1,j)
        }
        float qrho2i = 0.0f, qrho2j = 0.0f;
        if (projv < 0.0f) {
          qrho2i = -0.5f * rho1if * vsigavi * projv;
          if (usej) qrho2j = -0.5f * rho1j * vsigavj * projv;
        }
        const float gradpi = pmf * (pro2if + qrho2i) * grkerni;
        const float gradpj = usej ? pmf * (pro2j + qrho2j) * grkernj : 0.0f;
        if (adiab) {
          const float vsigu = GRAV ? fabsf(projv) : sqrtf(fabsf(prif - prj) * __fdividef(2.0f, rhoif + rhoj));
          f[5].add(pmf * qrho2i * projv * grkerni);
          f[6].add(vsigu * denij * (auterm * grkerni + autermj * grkernj));
        }
        float projsx = 0, projsy = 0, projsz = 0;
        if (MHD) {
          const float *mj = jmhdf + JMHDF * (size_t)j;
          const float bxj = mj[0], byj = mj[1], bzj = mj[2], psij = mj[3];
          const float dBx = bxif - bxj, dBy = byif - byj, dBz = bzif - bzj;
          const float projBi = bxif * runix + byif * runiy + bzif * runiz;
          const float projBj = bxj * runix + byj * runiy + bzj * runiz;
          const float projdB = dBx * runix + dBy * runiy + dBz * runiz;
          const float dB2 = dBx * dBx + dBy * dBy + dBz * dBz;
          f[11].add(-pmf * projdB * grkerni);
          const float tx_ = dvx - projv * runix, ty_ = dvy - projv * runiy, tz_ = dvz - projv * runiz;
          const float vsigB = sqrtf(tx_ * tx_ + ty_ * ty_ + tz_ * tz_);
          const float dBdiss = (avBterm * grkerni + avBtermj * grkernj) * vsigB;
          if (p.iresistive_heating > 0 && adiab) f[5].add(-0.5f * dB2 * dBdiss);
          const float pmi = pmf * rho21i * grkerni, pmj = pmf * rho21j * grkernj;
          const float termi = pmi * projBi;
          f[7].add(termi + pmj * projBj);
          const float dpsi = ocf * (pmi * psiif * vwaveif + pmj * psij * vwavej);
          f[8].add(-termi * dvx + dBdiss * dBx - dpsi * runix);
          f[9].add(-termi * dvy + dBdiss * dBy - dpsi * runiy);
          f[10].add(-termi * dvz + dBdiss * dBz - dpsi * runiz);
          projsx = (sx[0] * runix + sx[1] * runiy + sx[2] * runiz) * grkerni +
                   (mj[4] * runix + mj[5] * runiy + mj[6] * runiz) * grkernj;
          projsy = (sx[1] * runix + sx[3] * runiy + sx[4] * runiz) * grkerni +
                   (mj[5] * runix + mj[7] * runiy + mj[8] * runiz) * grkernj;
          projsz = (sx[2] * runix + sx[4] * runiy + sx[5] * runiz) * grkerni +
                   (mj[6] * runix + mj[8] * runiy + mj[9] * runiz) * grkernj;
        }
        const float gradp = gradpi + gradpj + fgrav;
        f[0].add(-runix * gradp - projsx);
        f[1].add(-runiy * gradp - projsy);
        f[2].add(-runiz * gradp - projsz);
        if (GRAV) f[3].add(pmf * phii);
        f[4].add(projv * grkerni);
      } else if (GRAV) {
        const float rij1 = rsqrt_nr(rij2);
        const float fgj = rij1 * rij1 * rij1 * pmf;
        f[0].add(-dx * fgj); f[1].add(-dy * fgj); f[2].add(-dz * fgj);
        f[3].add(-pmf * rij1);
      }
    };
    // operands loaded right before their pair: at 96 registers 20 warps per SM
    // hide the load latency better than a one-pair prefetch at 113 registers
    // and 16 warps (4.94 -> 4.37 ms per Sedov 128^3 launch)
    queue_window(cnt, S, act, il, stripe, sm.q, test, [&](int k) { body(load(k)); });
  }
  store_pair_sums<IND>(sm, lane, np, S, s0, am, psum, ps, [&](int q) -> double {
    return q < NF ? f[q].value() : (q == NF ? (double)vsigmax : (double)nbi);
  });
}

static inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }

// whether this context's force evaluation takes the symmetric FP64 pair loop
static bool use_sym(const ph_ctx *c) {
  const Params &p = c->dp;
  return c->force_sym && p.precision != PH_PREC_MIXED && !p.gravity && !(p.ind && c->ibin);
}

// The flattened trial offsets of the owned entries of the force lists and the
// j-side buffer of the symmetric pair loop (after every list build).
static int prepare_sym(ph_ctx *c) {
  cudaStream_t st = c->stream;
  const int ncell = c->nleaves;
  const int nj = c->dp.mhd ? NJS<true>::n : NJS<false>::n;
  if (alloc_sym(c, 0, nj) != 0) return PH_ERR_CUDA;
  k_cell_at<<<nblk(ncell, 256), 256, 0, st>>>(c->nodes, c->leaves, ncell, c->cell_at);
  k_owned_trials<<<nblk(ncell, 4), 128, 0, st>>>(c->nodes, c->leaves, ncell, c->pool, c->cell_off, c->cell_nleaf,
                                                  c->cell_tbase);
  scan_int(c, c->cell_tbase, c->cell_tbase, ncell, c->cell_tbase + ncell);
  k_entry_offsets<<<nblk(ncell, 4), 128, 0, st>>>(ncell, c->cell_off, c->cell_nleaf, c->cell_tbase, c->pool,
                                                   c->toff);
  count_launch(c, 3);
  int total = 0;
  cudaMemcpyAsync(&total, c->cell_tbase + ncell, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return PH_ERR_CUDA;
  if (total < 0) return PH_ERR_LIST;
  c->sym_total = total;
  return alloc_sym(c, (int64_t)total, nj) != 0 ? PH_ERR_CUDA : 0;
}

// Force trial lists (getneigh with the j-side hmax, or getneigh_dual with
// self-gravity, whose far-field coefficients are computed with them). They
// depend only on the tree and the node hmax values, so a force-only
// re-evaluation (velocity iterations, derivs icall=2) reuses the lists of the
// previous walk: the reference re-walks and gets the same lists.
int force_lists(ph_ctx *c) {
  cudaStream_t st = c->stream;
  const int ncell = c->nleaves;
  const Params p = c->dp;
  if (p.gravity && alloc_gravity(c) != 0) return PH_ERR_CUDA;
  bool levels_ok = false;
  for (int attempt = 0; !c->have_force_lists; ++attempt) {
    cudaMemsetAsync(c->pool_top, 0, sizeof(unsigned long long), st);
    cudaEventRecord(c->evk[4], st);
    if (p.gravity) {
      // getneigh_dual: the far field and the trial lists level by level, or
      // by the walks from the root when a level buffer overflowed
      const int fr = far_levels(c);
      if (fr > 0) return fr;
      levels_ok = fr == 0;
      if (!levels_ok) {
        cudaMemsetAsync(c->pool_top, 0, sizeof(unsigned long long), st);
        dual_walk(c);
      }
    } else {
      // individual timesteps: the cells holding active particles
      const bool ind = p.ind && c->ibin;
      const int nw = ind ? c->ncell_act : ncell;
      if (nw > 0) {
        launch_walk<true>(c->walk_warps, nw, st,
            p, c->nodes, c->nodesf, c->root, c->leaves, ind ? c->cell_act : nullptr, nw, nullptr, nullptr, c->pool,
            c->pool_cap, c->pool_top, c->cell_off, c->cell_nleaf, c->cell_ntrial, c->d_err);
        count_launch(c, 1);
      }
    }
    cudaEventRecord(c->evk[5], st);
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
    if (use_sym(c)) {
      const int r = prepare_sym(c);
      if (r) return r;
    }
    c->have_force_lists = true;
    // the far field depends on the same tree, positions and node hmax
    if (p.gravity) {
      if (levels_ok) gravity_down(c);
      else gravity_far(c);
    }
  }
  return 0;
}

// cons2prim + force driver on the device-resident state; vel/Bv are the
// velocity and magnetic arrays the forces are evaluated with (vxyzu/Bevol or
// the step's predicted vpred/Bpred).
int force_dev(ph_ctx *c, const double *vel, const double *Bv) {
  if (!c->have_density) return PH_ERR_STATE;
  cudaStream_t st = c->stream;
  const int nt = (int)c->ntree, ncell = c->nleaves;
  const Params p = c->dp;
  double *eos_t = c->eos;  // tree order
  double *jmhd = c->jrec + JREC * (size_t)c->cap;
  const bool mixed = p.precision == PH_PREC_MIXED;
  float *jmhdf = c->jrecf + JRECF * (size_t)c->cap;
  if (mixed)
    k_force_prologue_mixed<<<nblk(nt, 256), 256, 0, st>>>(p, nt, c->perm, c->th, vel, Bv,
                                                          p.ind ? c->gradh : c->gradh_t, eos_t, c->jrec, jmhd,
                                                          c->jrecf, jmhdf, c->txf, c->alpha1, c->ddivvdt_c,
                                                          c->dvdx_c, c->alphaloc_t, c->d_err);
  else
    k_force_prologue<<<nblk(nt, 256), 256, 0, st>>>(p, nt, c->perm, c->tx, c->ty, c->tz, c->th, vel, Bv,
                                                    p.ind ? c->gradh : c->gradh_t, eos_t, c->jrec, jmhd, nullptr,
                                                    nullptr, c->txf, c->alpha1, c->ddivvdt_c, c->dvdx_c,
                                                    c->alphaloc_t, c->d_err);
  count_launch(c, 1);
  const int lr = force_lists(c);
  if (lr) return lr;
  const double init[2] = {BIGNUMBER, BIGNUMBER};
  cudaMemcpyAsync(c->red, init, 2 * sizeof(double), cudaMemcpyHostToDevice, st);
  ForceOut out{c->fxyzu, c->dBevol, c->divcurlv, c->divBsymm, c->poten, c->red, c->stats, c->cell_ntrial};
  if (!(c->attr_done & 2u)) {
    const int bytes = MAX_WARPS * (int)sizeof(PairSmem);
#define PH_FORCE_ATTR(K, M, G, I) cudaFuncSetAttribute(K<M, G, I>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)
#define PH_FORCE_ATTR4(K, I) \
    PH_FORCE_ATTR(K, false, false, I); PH_FORCE_ATTR(K, true, false, I); PH_FORCE_ATTR(K, false, true, I); \
    PH_FORCE_ATTR(K, true, true, I)
    PH_FORCE_ATTR4(k_force_mixed, false); PH_FORCE_ATTR4(k_force_mixed, true);
    PH_FORCE_ATTR4(k_force, false); PH_FORCE_ATTR4(k_force, true);
#undef PH_FORCE_ATTR4
#undef PH_FORCE_ATTR
    cudaFuncSetAttribute(k_force_sym<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         MAX_WARPS * (int)sizeof(SymSmem<false>));
    cudaFuncSetAttribute(k_force_sym<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         MAX_WARPS * (int)sizeof(SymSmem<true>));
    c->attr_done |= 2u;
  }
  const int fw = c->force_warps;
  // individual timesteps: only the cells holding active particles
  const bool ind = p.ind && c->ibin;
  const int *cells = ind ? c->cell_act : nullptr;
  const int nfc = ind ? c->ncell_act : ncell;
  const unsigned char *actf = ind ? c->actf_t : nullptr;
  const int8_t *ibo = ind ? c->ibin_old_t : nullptr;
  unsigned char *wake = ind ? c->wakemark : nullptr;
  IndFin indf{nullptr, nullptr, nullptr, 0, 0, 0};
  if (ind) {
    indf = IndFin{c->actf_t, c->ibin, c->d_ind, c->nbinmax, c->istepfrac, c->ind_icall < 2 ? 1 : 0};
    cudaMemsetAsync(c->d_ind, 0, 3 * sizeof(int), st);
  }
  if (nfc == 0) {
    cudaEventRecord(c->evk[0], st);
  } else if (mixed) {
    cudaEventRecord(c->evk[0], st);
#define PH_FORCE_MIXED(M, G)                                                                                     \
  do { if (ind) PH_FORCE_MIXED_I(M, G, true); else PH_FORCE_MIXED_I(M, G, false); } while (0)
#define PH_FORCE_MIXED_I(M, G, I)                                                                                \
  k_force_mixed<M, G, I><<<nblk(nfc, fw), 32 * fw, fw * sizeof(PairSmem), st>>>(              \
      p, c->nodes, c->leaves, nfc, c->pool, c->cell_off, c->cell_nleaf, c->perm, c->tx, c->ty, c->tz, c->th,       \
      c->txf, c->jrec, jmhd, c->jrecf, jmhdf, eos_t, out, c->psum, c->cap, cells, actf, ibo, wake, c->d_err)
    if (p.mhd) { if (p.gravity) PH_FORCE_MIXED(true, true); else PH_FORCE_MIXED(true, false); }
    else { if (p.gravity) PH_FORCE_MIXED(false, true); else PH_FORCE_MIXED(false, false); }
#undef PH_FORCE_MIXED
#undef PH_FORCE_MIXED_I
  } else if (use_sym(c)) {
    cudaEventRecord(c->evk[0], st);
    if (p.mhd) {
      k_force_sym<true><<<nblk(nfc, fw), 32 * fw, fw * sizeof(SymSmem<true>), st>>>(
          p, c->nodes, c->leaves, nfc, c->pool, c->cell_off, c->cell_nleaf, c->tx, c->ty, c->tz, c->th, c->txf,
          c->jrec, jmhd, eos_t, out, c->psum, c->cap, c->pf_hmin, c->toff, c->jbuf, c->jbuf_stride, c->d_err);
      k_force_gather<true><<<nblk(nfc, 4), 128, 0, st>>>(c->nodes, c->leaves, nfc, c->pool, c->cell_off,
                                                         c->cell_nleaf, c->cell_at, c->toff, c->jbuf,
                                                         c->jbuf_stride, c->psum, c->cap, c->d_err);
    } else {
      k_force_sym<false><<<nblk(nfc, fw), 32 * fw, fw * sizeof(SymSmem<false>), st>>>(
          p, c->nodes, c->leaves, nfc, c->pool, c->cell_off, c->cell_nleaf, c->tx, c->ty, c->tz, c->th, c->txf,
          c->jrec, jmhd, eos_t, out, c->psum, c->cap, c->pf_hmin, c->toff, c->jbuf, c->jbuf_stride, c->d_err);
      k_force_gather<false><<<nblk(nfc, 4), 128, 0, st>>>(c->nodes, c->leaves, nfc, c->pool, c->cell_off,
                                                          c->cell_nleaf, c->cell_at, c->toff, c->jbuf,
                                                          c->jbuf_stride, c->psum, c->cap, c->d_err);
    }
    count_launch(c, 1);
  } else {
    cudaEventRecord(c->evk[0], st);
#define PH_FORCE_FP64(M, G)                                                                                      \
  do { if (ind) PH_FORCE_FP64_I(M, G, true); else PH_FORCE_FP64_I(M, G, false); } while (0)
#define PH_FORCE_FP64_I(M, G, I)                                                                                 \
  k_force<M, G, I><<<nblk(nfc, fw), 32 * fw, fw * sizeof(PairSmem), st>>>(                    \
      p, c->nodes, c->leaves, nfc, c->pool, c->cell_off, c->cell_nleaf, c->perm, c->tx, c->ty, c->tz, c->th,       \
      c->txf, c->jrec, jmhd, eos_t, out, c->psum, c->cap, c->pf_hmin, cells, actf, ibo, wake, c->d_err)
    if (p.mhd) { if (p.gravity) PH_FORCE_FP64(true, true); else PH_FORCE_FP64(true, false); }
    else { if (p.gravity) PH_FORCE_FP64(false, true); else PH_FORCE_FP64(false, false); }
#undef PH_FORCE_FP64
#undef PH_FORCE_FP64_I
  }
  const FarField ff{c->gleaf, c->leaf_of, c->leaves, c->nodes, c->tx, c->ty, c->tz};
  if (mixed)
    k_force_finish<true><<<nblk(nt, 256), 256, 0, st>>>(p, nt, c->psum, c->cap, c->perm, c->th, c->jrec, jmhd,
                                                        eos_t, ff, out, indf, c->d_err);
  else
    k_force_finish<false><<<nblk(nt, 256), 256, 0, st>>>(p, nt, c->psum, c->cap, c->perm, c->th, c->jrec, jmhd,
                                                         eos_t, ff, out, indf, c->d_err);
  if (ind) {
    k_wake_apply<<<nblk(nt, 256), 256, 0, st>>>(nt, c->perm, c->wakemark, c->ibin_wake, c->ibinnow - 1);
    count_launch(c, 1);
  }
  cudaEventRecord(c->evk[1], st);
  count_launch(c, 2);
  c->have_force = true;
  return 0;
}

}  // namespace ph
