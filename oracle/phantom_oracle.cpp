// CPU oracle for the Phantom per-step SPH hot path — TEST INFRASTRUCTURE ONLY.
//
// A serial (optionally OpenMP over leaf cells) C++ restatement of the
// reference Fortran routines on the hot path. Only tests/, the smoke check and
// the CPU-baseline leg of bench.py use it; the product library never links it.
//
// Every routine cites the reference file:line it restates (paths relative to
// the phantom source tree). Arithmetic is written operand-for-operand in the
// Fortran evaluation order and compiled with -ffp-contract=off so that it
// rounds like gfortran -O3 on x86-64 (no FMA contraction).
//
// Parity pinning: the reference cannot be compiled here (no Fortran compiler);
// the oracle is pinned by restated known-answer tests of the reference suite
// (tests/test_oracle_golden.py), see oracle.h.

#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- constants
// physcon.f90:23 (pi is a 10-digit literal, not M_PI)
const double PI_PHANTOM = 3.1415926536;
// kernel_cubic.f90:23-30
const double RADKERN = 2.0, RADKERN2 = 4.0;
const double CNORMK = 1.0 / PI_PHANTOM;
const double WAB0 = 1.0, GRADH0 = -3.0 * 1.0, DPHIDH0 = 1.4;
const int MINPART = 10;            // config.F90:113 (default of ora_params.minpart)
const int MAXLEAF = 16;            // largest leaf size accepted
const double AVDECAYCONST = 0.1;   // shock_capturing.f90:32
const int MAXDEPTH = 32;           // kdtree.F90:42
const int ISIZECELLCACHE = 1000;   // dens.F90:99 and force.F90:58 (maxcellcache)
const int MAXDENSITS = 100;        // dens.F90:101
const double BIGNUMBER = 1.e29;    // timestep.f90:40
const double EPS_D = 2.220446049250313e-16;     // epsilon(0.d0)
const double TINY_D = 2.2250738585072014e-308;  // tiny(0.d0)
const double HUGE_D = 1.7976931348623157e308;   // huge(0.d0)
const int LENFGRAV = 20;           // dtype_kdtree.F90:21

inline double sq(double x) { return x * x; }
inline double cube(double x) { double t = x * x; return t * x; }  // x**3
inline double fsign1(double x) { return std::signbit(x) ? -1.0 : 1.0; }  // SIGN(1.0,x)
inline double fmax_f(double a, double b) { return (a > b) ? a : b; }  // MAX(a,b)
inline double fmin_f(double a, double b) { return (a < b) ? a : b; }

// kernel_cubic.f90:34-50 get_kernel / grkern
inline void get_kernel(double q2, double q, double &w, double &g) {
  if (q < 1.0) {
    w = 0.75 * q2 * q - 1.5 * q2 + 1.0;
    g = q * (2.25 * q - 3.0);
  } else if (q < 2.0) {
    w = -0.25 * cube(q - 2.0);
    g = -0.75 * sq(q - 2.0);
  } else {
    w = 0.0;
    g = 0.0;
  }
}
inline double grkern(double q2, double q) {
  (void)q2;
  if (q < 1.0) return q * (2.25 * q - 3.0);
  if (q < 2.0) return -0.75 * sq(q - 2.0);
  return 0.0;
}
// kernel_cubic.f90:78-99 get_kernel_grav1
inline void get_kernel_grav1(double q2, double q, double &w, double &g, double &dphidh) {
  if (q < 1.0) {
    double q4 = q2 * q2;
    w = 0.75 * q2 * q - 1.5 * q2 + 1.0;
    g = q * (2.25 * q - 3.0);
    dphidh = -0.6 * q4 * q + 1.5 * q4 - 2.0 * q2 + 1.4;
  } else if (q < 2.0) {
    double q4 = q2 * q2;
    w = -0.25 * cube(q - 2.0);
    g = -0.75 * sq(q - 2.0);
    dphidh = 0.2 * q4 * q - 1.5 * q4 + 4.0 * q2 * q - 4.0 * q2 + 1.6;
  } else {
    w = 0.0; g = 0.0; dphidh = 0.0;
  }
}
// kernel_cubic.f90:101-120 kernel_softening
inline void kernel_softening(double q2, double q, double &potensoft, double &fsoft) {
  if (q < 1.0) {
    double q4 = q2 * q2;
    potensoft = q4 * q / 10.0 - 3.0 * q4 / 10.0 + 2.0 * q2 / 3.0 - 7.0 / 5.0;
    fsoft = q * (15.0 * q2 * q - 36.0 * q2 + 40.0) / 30.0;
  } else if (q < 2.0) {
    double q4 = q2 * q2;
    double q6 = q4 * q2;
    potensoft = (q * (-q4 * q + 9.0 * q4 - 30.0 * q2 * q + 40.0 * q2 - 48.0) + 2.0) / (30.0 * q);
    fsoft = (-5.0 * q6 + 36.0 * q4 * q - 90.0 * q4 + 80.0 * q2 * q - 2.0) / (30.0 * q2);
  } else {
    potensoft = -1.0 / q;
    fsoft = 1.0 / q2;
  }
}

struct Node {
  double xcen[3];
  double size, hmax, mass;
  int left, right, parent;
  double quads[6];
};

// cell state of densityiterate (mpi_dens.F90 celldens, restricted to the path)
struct CellDens {
  int icell, npcell, nits, nneightry;
  int arr_index[MAXLEAF + 2];
  double x[MAXLEAF + 2][3], v[MAXLEAF + 2][3], B[MAXLEAF + 2][4];
  double h[MAXLEAF + 2], h_old[MAXLEAF + 2];
  double rhosums[MAXLEAF + 2][40];
  int nneigh[MAXLEAF + 2];
  uint64_t nhash[MAXLEAF + 2];
  double xpos[3], xsizei, rcuti, hmax;
};

inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Oracle {
  ora_params p;
  int64_t n = 0;
  std::vector<double> xyzh, vxyzu, Bevol, fxyzu, dBevol, eos;
  std::vector<float> gradh, divcurlv, divcurlB, divBsymm, poten;
  std::vector<float> alphaind, dvdx;  // part.F90:50 alphaind(nalpha,:) and dvdx(9,:), real*4
  // individual timesteps (part.F90 ibin, ibin_old, ibin_wake, twas, iphase activity;
  // utils_indtimesteps.f90 nbinmax, istepfrac, ibinnow; step_leapfrog.f90 ibin_dts)
  static const int MAXBINS = 30;   // utils_indtimesteps.f90 maxbins
  std::vector<int8_t> ibin, ibin_old, ibin_wake;
  std::vector<uint8_t> activef;
  std::vector<double> twas;
  int nbinmax = 0, istepfrac = 0, ibinnow = 0;
  double ibin_dts[4][MAXBINS + 1] = {};  // itdt, ithdt, itdt1, ittwas
  double tlast = 0.0, dtsub = 0.0;
  bool dt_too_small = false;
  int dt_too_small_any = 0;
  const double *dens_vel = nullptr;   // velocities the density's dv sums read (vxyzu or vpred)
  const double *dens_B = nullptr;     // Bevol the density's div B and curl B sums read (Bevol or Bpred:
                                      // derivs passes its Bevol argument on, deriv.f90:135)
  std::vector<double> gradh_d;  // FP64 copy of gradh read by the force when p.f64_store
  std::vector<int32_t> nneigh_out;
  std::vector<uint64_t> nhash_out;
  // tree (kdtree.F90:31-32, neigh_kdtree.f90:28-38)
  int64_t ncellsmax = 0, ncells = 0;
  int maxlevel_indexed = 0, maxlevel = 0, minlevel = 0;
  std::vector<Node> node;
  std::vector<int32_t> leaf_is_active, inodeparts, inoderange;  // inoderange(2,ncellsmax+1)
  std::vector<double> treecache;  // treecache(5,n)
  ora_stats stats{};
  double dxbound = 0, dybound = 0, dzbound = 0, hdlx = 0, hdly = 0, hdlz = 0;
  double dtcourant = BIGNUMBER, dtforce = BIGNUMBER, dterr = BIGNUMBER;
  // step-loop predicted arrays (step_leapfrog.f90 vpred, Bpred)
  std::vector<double> vpred, Bpred;
  bool have_tree = false;

  void set_params(const ora_params *pp) {
    p = *pp;
    dxbound = p.xmax - p.xmin; dybound = p.ymax - p.ymin; dzbound = p.zmax - p.zmin;  // boundary.f90:105
    hdlx = 0.5 * dxbound; hdly = 0.5 * dybound; hdlz = 0.5 * dzbound;                 // boundary.f90:109
  }
  int threads() const { return p.nthreads > 0 ? p.nthreads : 1; }
  double alphamax() const { return p.alphamax > 0.0 ? p.alphamax : 1.0; }  // shock_capturing.f90:55

  double rhoh(double h) const { double t = p.hfact / std::fabs(h); return p.massoftype * cube(t); }  // part.F90:779
  double dhdrho(double h) const { double r = rhoh(h); return -h / (3.0 * r); }                      // part.F90:791
  double hrho(double rho) const { return p.hfact * std::pow(p.massoftype / std::fabs(rho), 1.0 / 3.0); }  // part.F90:845

  // ---------------------------------------------------------- boundary
  // boundary.f90:123-160 cross_boundary
  void cross_boundary(double *xyz) const {
    if (xyz[0] < p.xmin) xyz[0] = xyz[0] + dxbound; else if (xyz[0] > p.xmax) xyz[0] = xyz[0] - dxbound;
    if (xyz[1] < p.ymin) xyz[1] = xyz[1] + dybound; else if (xyz[1] > p.ymax) xyz[1] = xyz[1] - dybound;
    if (xyz[2] < p.zmin) xyz[2] = xyz[2] + dzbound; else if (xyz[2] > p.zmax) xyz[2] = xyz[2] - dzbound;
  }
  // gradh as the force reads it: float32 as stored by the reference, or the
  // FP64 value when f64_store is set
  double gh(size_t k) const { return p.f64_store ? gradh_d[k] : (double)gradh[k]; }
  // rows of divcurlv (config.F90:165,384: ndivcurlv = 4 with curlv)
  int ndivcurlv() const { return p.curlv ? 4 : 1; }

  // kdtree.F90:1468-1501 get_sep
  void get_sep(const double *x1, const double *x2, double &dx, double &dy, double &dz,
               double &xo, double &yo, double &zo, double *r2) const {
    xo = 0.0; yo = 0.0; zo = 0.0;
    dx = x1[0] - x2[0]; dy = x1[1] - x2[1]; dz = x1[2] - x2[2];
    if (p.periodic) {
      if (std::fabs(dx) > hdlx) { xo = dxbound * fsign1(dx); dx = dx - xo; }
      if (std::fabs(dy) > hdly) { yo = dybound * fsign1(dy); dy = dy - yo; }
      if (std::fabs(dz) > hdlz) { zo = dzbound * fsign1(dz); dz = dz - zo; }
    }
    if (r2) *r2 = dx * dx + dy * dy + dz * dz;
  }

  // ---------------------------------------------------------- tree build
  struct StackEntry { int node, parent, level, npnode; double xmin[3], xmax[3]; };

  int maketree() {  // kdtree.F90:117-314 (serial: nqueue = 1, queue phase skipped)
    ncellsmax = 2 * p.maxp;  // config.F90:393
    if ((int64_t)node.size() < ncellsmax + 2) {
      node.assign(ncellsmax + 2, Node{});
      leaf_is_active.assign(ncellsmax + 2, 0);
      inoderange.assign(2 * (ncellsmax + 2), 0);
    }
    std::fill(leaf_is_active.begin(), leaf_is_active.end(), 0);
    inodeparts.assign(n + 1, 0);
    treecache.assign(5 * (n + 1), 0.0);
    // construct_root_node kdtree.F90:347-488
    double xminp = xyzh[0], yminp = xyzh[1], zminp = xyzh[2];
    double xmaxp = xminp, ymaxp = yminp, zmaxp = zminp;
    for (int64_t i = 0; i < n; ++i) {
      double *xi = &xyzh[4 * i];
      if (xi[3] < TINY_D) continue;
      if (p.periodic) cross_boundary(xi);
      if (std::isnan(xi[0]) || std::isnan(xi[1]) || std::isnan(xi[2])) return 2;  // NaN position
      xminp = std::min(xminp, xi[0]);
      yminp = std::min(yminp, xi[1]); zminp = std::min(zminp, xi[2]);
      xmaxp = std::max(xmaxp, xi[0]); ymaxp = std::max(ymaxp, xi[1]); zmaxp = std::max(zmaxp, xi[2]);
    }
    int nproot = 0;
    for (int64_t i = 0; i < n; ++i) {
      if (xyzh[4 * i + 3] < TINY_D) continue;
      ++nproot;
      inodeparts[nproot] = activef.empty() || activef[i] ? (int32_t)(i + 1) : -(int32_t)(i + 1);  // -ve if inactive
      for (int k = 0; k < 4; ++k) treecache[5 * nproot + k] = xyzh[4 * i + k];
      treecache[5 * nproot + 4] = p.massoftype;
    }
    if (nproot == 0) return 3;
    inoderange[2 * 1 + 0] = 1; inoderange[2 * 1 + 1] = nproot;
    maxlevel = 0; minlevel = MAXDEPTH - 1;
    maxlevel_indexed = (int)(std::log((double)(ncellsmax + 1)) / std::log(2.0)) - 1;
    ncells = ((int64_t)1 << (maxlevel_indexed + 1)) - 1;
    std::vector<StackEntry> stack;
    stack.reserve(512);
    StackEntry root{1, 0, 0, nproot, {xminp, yminp, zminp}, {xmaxp, ymaxp, zmaxp}};
    stack.push_back(root);
    while (!stack.empty()) {
      StackEntry e = stack.back(); stack.pop_back();
      StackEntry l, r;
      bool wassplit = false;
      int err = construct_node(e, l, r, wassplit);
      if (err) return err;
      if (wassplit) {
        if (stack.size() + 2 > 512) return 4;  // kdtree.F90:281 stack overflow
        stack.push_back(l); stack.push_back(r);
      }
    }
    if (maxlevel < maxlevel_indexed) ncells = ((int64_t)1 << (maxlevel + 1)) - 1;
    stats.ncells = ncells; stats.maxlevel = maxlevel; stats.minlevel = minlevel;
    have_tree = true;
    return 0;
  }

  // kdtree.F90:1851-2037 revtree: node properties recomputed from the
  // current positions on the existing tree structure (serial, no dead
  // particles, no individual timesteps: every leaf is active)
  int revtree() {
    if (!have_tree) return 1;
    int nptot = 0;  // kdtree.F90:1874-1880
    for (int64_t i = 1; i <= ncells; ++i) {
      if (i > 1 && node[i].parent == 0) continue;
      if (inoderange[2 * i] > 0 && inoderange[2 * i + 1] >= inoderange[2 * i]) nptot = std::max(nptot, inoderange[2 * i + 1]);
    }
    for (int i = 1; i <= nptot; ++i) {  // kdtree.F90:1891-1910
      if (inodeparts[i] == 0) continue;
      const int ip = std::abs(inodeparts[i]) - 1;
      for (int k = 0; k < 4; ++k) treecache[5 * i + k] = xyzh[4 * ip + k];
      treecache[5 * i + 4] = p.massoftype;
    }
    const double pmass = p.massoftype;
    for (int64_t in = 1; in <= ncells; ++in) {  // kdtree.F90:1928-2033
      if (in > 1 && node[in].parent == 0) continue;
      Node &nd = node[in];
      for (int k = 0; k < 3; ++k) nd.xcen[k] = 0.0;
      nd.size = 0.0; nd.hmax = 0.0; nd.mass = 0.0;
      for (int k = 0; k < 6; ++k) nd.quads[k] = 0.0;
      leaf_is_active[in] = 0;
      const int i1 = inoderange[2 * in], i2 = inoderange[2 * in + 1];
      if (i1 <= 0 || i2 < i1) continue;
      double xc = 0.0, yc = 0.0, zc = 0.0, totmass = 0.0, hmax = 0.0;
      const double dfac = (pmass > 0.0) ? 1.0 / pmass : 1.0;
      for (int i = i1; i <= i2; ++i) {
        if (inodeparts[i] == 0) continue;
        const double *t = &treecache[5 * i];
        if (t[3] <= 0.0) continue;
        const double fac = t[4] * dfac;
        xc = xc + fac * t[0]; yc = yc + fac * t[1]; zc = zc + fac * t[2];
        totmass = totmass + t[4];
        hmax = std::max(std::fabs(t[3]), hmax);
      }
      if (totmass <= 0.0) continue;
      const double x0[3] = {xc / (totmass * dfac), yc / (totmass * dfac), zc / (totmass * dfac)};
      double r2max = 0.0, q[6] = {0, 0, 0, 0, 0, 0};
      for (int i = i1; i <= i2; ++i) {
        const double *t = &treecache[5 * i];
        if (t[3] <= 0.0) continue;
        const double dx = t[0] - x0[0], dy = t[1] - x0[1], dz = t[2] - x0[2];
        const double dr2 = dx * dx + dy * dy + dz * dz;
        r2max = std::max(dr2, r2max);
        if (p.gravity) {
          q[0] = q[0] + t[4] * (dx * dx); q[1] = q[1] + t[4] * (dx * dy); q[2] = q[2] + t[4] * (dx * dz);
          q[3] = q[3] + t[4] * (dy * dy); q[4] = q[4] + t[4] * (dy * dz); q[5] = q[5] + t[4] * (dz * dz);
        }
      }
      for (int k = 0; k < 3; ++k) nd.xcen[k] = x0[k];
      nd.size = std::sqrt(r2max) + EPS_D;
      nd.hmax = hmax;
      nd.mass = totmass;  // kept without gravity too, as construct_node here does
      if (p.gravity) for (int k = 0; k < 6; ++k) nd.quads[k] = q[k];
      if (nd.left == 0 && nd.right == 0) leaf_is_active[in] = 1;
    }
    return 0;
  }

  // kdtree.F90:531-929 construct_node
  int construct_node(StackEntry &e, StackEntry &lo, StackEntry &ro, bool &wassplit) {
    int nnode = e.node, npnode = e.npnode, level = e.level;
    int i1 = inoderange[2 * nnode + 0];
    int npcounter = (i1 > 0) ? inoderange[2 * nnode + 1] - i1 + 1 : 0;
    if (npcounter != npnode) return 5;
    wassplit = false;
    if (npnode < 1) return 0;
    double pmassi = p.massoftype, dfac = (pmassi > 0.0) ? 1.0 / pmassi : 1.0;
    double hmax = 0.0, totmass = 0.0, xc = 0.0, yc = 0.0, zc = 0.0;
    for (int i = i1; i <= i1 + npnode - 1; ++i) {  // kdtree.F90:654-666
      const double *t = &treecache[5 * i];
      double pm = t[4];
      double fac = pm * dfac;
      hmax = fmax_f(hmax, t[3]);
      totmass = totmass + pm;
      xc = xc + fac * t[0]; yc = yc + fac * t[1]; zc = zc + fac * t[2];
    }
    double cofm[3] = {xc, yc, zc};
    if (totmass > 0.0) {
      double d = totmass * dfac;
      cofm[0] = cofm[0] / d; cofm[1] = cofm[1] / d; cofm[2] = cofm[2] / d;
    }
    if (totmass <= 0.0) return 6;
    double r2max = 0.0, quads[6] = {0, 0, 0, 0, 0, 0};
    for (int i = i1; i <= i1 + npnode - 1; ++i) {  // kdtree.F90:734-752
      const double *t = &treecache[5 * i];
      double dx = t[0] - cofm[0], dy = t[1] - cofm[1], dz = t[2] - cofm[2];
      double dr2 = dx * dx + dy * dy + dz * dz;
      r2max = fmax_f(r2max, dr2);
      if (p.gravity) {
        double pm = t[4];
        quads[0] = quads[0] + pm * (dx * dx);
        quads[1] = quads[1] + pm * (dx * dy);
        quads[2] = quads[2] + pm * (dx * dz);
        quads[3] = quads[3] + pm * (dy * dy);
        quads[4] = quads[4] + pm * (dy * dz);
        quads[5] = quads[5] + pm * (dz * dz);
      }
    }
    Node &nd = node[nnode];
    for (int k = 0; k < 3; ++k) nd.xcen[k] = cofm[k];
    nd.size = std::sqrt(r2max) + EPS_D;  // kdtree.F90:782
    nd.hmax = hmax;
    nd.parent = e.parent;
    nd.mass = totmass;
    for (int k = 0; k < 6; ++k) nd.quads[k] = quads[k];
    wassplit = (npnode > (p.minpart > 0 ? p.minpart : MINPART));  // kdtree.F90:792
    if (!wassplit) {
      nd.left = 0; nd.right = 0;
      maxlevel = std::max(level, maxlevel);
      minlevel = std::min(level, minlevel);
      bool nodeisactive = true;
      if (p.ind_timesteps) {  // kdtree.F90:800-812: active if it holds an active particle
        nodeisactive = false;
        for (int ip = i1; ip <= i1 + npnode - 1; ++ip) nodeisactive = nodeisactive || inodeparts[ip] > 0;
      }
      leaf_is_active[nnode] = nodeisactive ? 1 : -1;
      return 0;
    }
    // split along the longest axis at the centre of mass (kdtree.F90:815-816)
    double ext[3] = {e.xmax[0] - e.xmin[0], e.xmax[1] - e.xmin[1], e.xmax[2] - e.xmin[2]};
    int iaxis = 0;
    if (ext[1] > ext[iaxis]) iaxis = 1;
    if (ext[2] > ext[iaxis]) iaxis = 2;
    double xpivot = cofm[iaxis];
    int il, ir;
    if (level < maxlevel_indexed) { il = 2 * nnode; ir = il + 1; }
    else {
      ncells += 2; ir = (int)ncells; il = (int)(ncells - 1);
      if (ir > ncellsmax) return 7;
    }
    nd.left = il; nd.right = ir;
    leaf_is_active[nnode] = 0;
    int nl, nr;
    sort_particles_in_cell(iaxis, inoderange[2 * nnode], inoderange[2 * nnode + 1],
                           inoderange[2 * il], inoderange[2 * il + 1],
                           inoderange[2 * ir], inoderange[2 * ir + 1], nl, nr, xpivot);
    if (nl + nr != npnode) return 8;
    if (nl == npnode || nr == npnode) {  // kdtree.F90:856-865
      nl = npnode / 2;
      inoderange[2 * il] = inoderange[2 * nnode];
      inoderange[2 * il + 1] = inoderange[2 * nnode] + nl - 1;
      inoderange[2 * ir] = inoderange[2 * nnode] + nl;
      inoderange[2 * ir + 1] = inoderange[2 * nnode + 1];
      nr = npnode - nl;
    }
    auto bounds = [&](int a, int b, double *mn, double *mx) {  // kdtree.F90:868-896
      for (int k = 0; k < 3; ++k) mn[k] = mx[k] = treecache[5 * a + k];
      for (int ip = a + 1; ip <= b; ++ip)
        for (int k = 0; k < 3; ++k) {
          mn[k] = std::min(mn[k], treecache[5 * ip + k]);
          mx[k] = std::max(mx[k], treecache[5 * ip + k]);
        }
    };
    lo = StackEntry{il, nnode, level + 1, nl, {0, 0, 0}, {0, 0, 0}};
    ro = StackEntry{ir, nnode, level + 1, nr, {0, 0, 0}, {0, 0, 0}};
    bounds(inoderange[2 * il], inoderange[2 * il + 1], lo.xmin, lo.xmax);
    bounds(inoderange[2 * ir], inoderange[2 * ir + 1], ro.xmin, ro.xmax);
    return 0;
  }

  void swap_rows(int a, int b) {
    std::swap(inodeparts[a], inodeparts[b]);
    for (int k = 0; k < 5; ++k) std::swap(treecache[5 * a + k], treecache[5 * b + k]);
  }
  // kdtree.F90:937-1001 sort_particles_in_cell (two-pointer partition)
  void sort_particles_in_cell(int iaxis, int imin, int imax, int &min_l, int &max_l, int &min_r,
                              int &max_r, int &nl, int &nr, double xpivot) {
    int i = imin, j = imax;
    bool ilt = treecache[5 * i + iaxis] <= xpivot;
    bool jlt = treecache[5 * j + iaxis] <= xpivot;
    while (i < j) {
      if (ilt) {
        ++i; ilt = treecache[5 * i + iaxis] <= xpivot;
      } else if (!jlt) {
        --j; jlt = treecache[5 * j + iaxis] <= xpivot;
      } else {
        swap_rows(i, j);
        ++i; --j;
        ilt = treecache[5 * i + iaxis] <= xpivot;
        jlt = treecache[5 * j + iaxis] <= xpivot;
      }
    }
    if (!ilt) i = i - 1;
    if (jlt) j = j + 1;
    min_l = imin; max_l = i; min_r = j; max_r = imax;
    nl = max_l - min_l + 1; nr = max_r - min_r + 1;
  }

  // ---------------------------------------------------------- neighbour walks
  struct TrialList {
    std::vector<int32_t> list;       // listneigh (1-based particle ids)
    std::vector<double> cache;       // xyzcache(maxcache, ISIZECELLCACHE)
    int nneigh = 0;
  };
  // kdtree.F90:1175-1213 cache_neighbours
  void cache_neighbours(TrialList &tl, int isrc, int maxcache, double xo, double yo, double zo) const {
    int a = inoderange[2 * isrc], b = inoderange[2 * isrc + 1];
    int npnode = b - a + 1;
    int num_to_cache;
    if (tl.nneigh + npnode <= ISIZECELLCACHE) num_to_cache = npnode;
    else if (tl.nneigh < ISIZECELLCACHE) num_to_cache = ISIZECELLCACHE - tl.nneigh;
    else num_to_cache = 0;
    if ((int)tl.list.size() < tl.nneigh + npnode) tl.list.resize(tl.nneigh + npnode + 1024);
    for (int ip = 1; ip <= npnode; ++ip) {
      int row = a + ip - 1;
      tl.list[tl.nneigh + ip - 1] = std::abs(inodeparts[row]);
      if (ip <= num_to_cache) {
        double *c = &tl.cache[4 * (tl.nneigh + ip - 1)];
        c[0] = treecache[5 * row + 0] + xo;
        c[1] = treecache[5 * row + 1] + yo;
        c[2] = treecache[5 * row + 2] + zo;
        if (maxcache >= 4) c[3] = 1.0 / treecache[5 * row + 3];
      }
    }
    tl.nneigh += npnode;
  }
  // kdtree.F90:1221-1347 getneigh (no long-range M2L: force uses the dual walk)
  int getneigh(const double *xpos, double xsizei, double rcuti, TrialList &tl, int maxcache, bool get_hj) const {
    double tree_acc2 = p.tree_accuracy * p.tree_accuracy;
    tl.nneigh = 0;
    if (tl.cache.size() < 4 * (size_t)ISIZECELLCACHE) tl.cache.assign(4 * ISIZECELLCACHE, 0.0);
    int nstack[MAXDEPTH + 8];
    int istack = 0;
    nstack[istack++] = 1;
    while (istack != 0) {
      int nn = nstack[--istack];
      double dx, dy, dz, xo, yo, zo, r2;
      get_sep(xpos, node[nn].xcen, dx, dy, dz, xo, yo, zo, &r2);
      double xsizej = node[nn].size;
      int il = node[nn].left, ir = node[nn].right;
      double rcut = rcuti;
      if (get_hj) { double rcutj = RADKERN * node[nn].hmax; rcut = fmax_f(rcuti, rcutj); }
      double rcut2 = sq(xsizei + xsizej + rcut);
      bool open_tree_node = false;
      if (p.gravity) open_tree_node = tree_acc2 * r2 < sq(xsizei + xsizej);
      if ((r2 < rcut2) || open_tree_node) {
        if (leaf_is_active[nn] != 0) {
          cache_neighbours(tl, nn, maxcache, xo, yo, zo);
        } else {
          if (istack + 2 > MAXDEPTH + 6) return 9;  // stack overflow
          if (il != 0) nstack[istack++] = il;
          if (ir != 0) nstack[istack++] = ir;
        }
      }
    }
    return 0;
  }

  // kdtree.F90:1702-1781 compute_M2L
  static void compute_M2L(double dx, double dy, double dz, double dr1, double q0, const double *quads, double *fnode) {
    double dr12 = dr1 * dr1;
    double dx2 = dx * dx, dx3 = dx * dx2, dy2 = dy * dy, dy3 = dy * dy2, dz2 = dz * dz, dz3 = dz * dz2;
    double g0 = -dr1;
    double g1 = 1.0 * dr12 * g0;
    double g2 = -3.0 * dr12 * g1;
    double g3 = -5.0 * dr12 * g2;
    double g2dx = g2 * dx, g2dy = g2 * dy, g2dz = g2 * dz;
    double D3[10], D2[6], D1[3];
    D3[0] = 3.0 * g2dx + g3 * dx3;
    D3[1] = g2dy + g3 * dx2 * dy;
    D3[2] = g2dz + g3 * dx2 * dz;
    D3[3] = g2dx + g3 * dy2 * dx;
    D3[4] = g3 * dx * dy * dz;
    D3[5] = g2dx + g3 * dz2 * dx;
    D3[6] = 3.0 * g2dy + g3 * dy3;
    D3[7] = g2dz + g3 * dy2 * dz;
    D3[8] = g2dy + g3 * dz2 * dy;
    D3[9] = 3.0 * g2dz + g3 * dz3;
    D2[0] = g1 + g2 * dx2; D2[1] = g2dx * dy; D2[2] = g2dx * dz;
    D2[3] = g1 + g2 * dy2; D2[4] = g2dy * dz; D2[5] = g1 + g2 * dz2;
    D1[0] = g1 * dx; D1[1] = g1 * dy; D1[2] = g1 * dz;
    double qxx = quads[0], qxy = quads[1], qxz = quads[2], qyy = quads[3], qyz = quads[4], qzz = quads[5];
    fnode[0] = fnode[0] + (D1[0] * q0 + 0.5 * (D3[0] * qxx + 2.0 * (D3[1] * qxy + D3[2] * qxz + D3[4] * qyz) + D3[3] * qyy + D3[5] * qzz));
    fnode[1] = fnode[1] + (D1[1] * q0 + 0.5 * (D3[1] * qxx + 2.0 * (D3[3] * qxy + D3[4] * qxz + D3[7] * qyz) + D3[6] * qyy + D3[8] * qzz));
    fnode[2] = fnode[2] + (D1[2] * q0 + 0.5 * (D3[2] * qxx + 2.0 * (D3[4] * qxy + D3[5] * qxz + D3[8] * qyz) + D3[7] * qyy + D3[9] * qzz));
    for (int k = 0; k < 6; ++k) fnode[3 + k] = fnode[3 + k] + D2[k] * q0;
    for (int k = 0; k < 10; ++k) fnode[9 + k] = fnode[9 + k] + D3[k] * q0;
    fnode[19] = fnode[19] + g0 * q0 - 0.5 * (D2[0] * qxx + D2[3] * qyy + D2[5] * qzz + 2.0 * (D2[1] * qxy + D2[2] * qxz + D2[4] * qyz));
  }
  // kdtree.F90:1527-1560 propagate_fnode_to_node
  static void propagate(double *f, const double *s, double dx, double dy, double dz) {
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
  // kdtree.F90:1799-1840 expand_fgrav_in_taylor_series (poti uses dz*dfxy as written there)
  static void expand_taylor(const double *f, double dx, double dy, double dz, double &fxi, double &fyi,
                            double &fzi, double &poti) {
    fxi = f[0]; fyi = f[1]; fzi = f[2];
    double dfxx = f[3], dfxy = f[4], dfxz = f[5], dfyy = f[6], dfyz = f[7], dfzz = f[8];
    double d2fxxx = f[9], d2fxxy = f[10], d2fxxz = f[11], d2fxyy = f[12], d2fxyz = f[13], d2fxzz = f[14],
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

  // kdtree.F90:1357-1461 getneigh_dual (+ node_interaction :1653-1694, open_nodes :1591-1645).
  // The per-node first-writer cache (fnodecache, :1427-1457) only avoids recomputing an
  // ancestor's M2L sum, which is identical for every leaf below it; it is not modelled.
  int getneigh_dual(int icell, const double *xpos, double xsizei, double rcuti, TrialList &tl,
                    int maxcache, double *fnode_out) const {
    (void)xpos; (void)xsizei; (void)rcuti;
    double tree_acc2 = p.tree_accuracy * p.tree_accuracy;
    int branch[MAXDEPTH + 8];
    int nparents = 1;
    branch[0] = icell;
    for (int j = icell; node[j].parent != 0;) {
      j = node[j].parent;
      if (nparents >= MAXDEPTH + 6) return 10;
      branch[nparents++] = j;
    }
    std::vector<double> fb((size_t)LENFGRAV * (nparents + 1), 0.0);
    double facc[LENFGRAV] = {0};
    tl.nneigh = 0;
    if (tl.cache.size() < 4 * (size_t)ISIZECELLCACHE) tl.cache.assign(4 * ISIZECELLCACHE, 0.0);
    int stk[3][4 * MAXDEPTH + 16];
    int istack = 0;
    stk[0][0] = 1; stk[1][0] = 1; stk[2][0] = nparents; istack = 1;
    while (istack > 0) {
      --istack;
      int idst = stk[0][istack], isrc = stk[1][istack], ib = stk[2][istack];
      bool stackit;
      double xo = 0, yo = 0, zo = 0;
      if (idst == isrc) {
        stackit = true;
      } else {
        const Node &nd = node[idst], &ns = node[isrc];
        double dx, dy, dz, r2;
        get_sep(nd.xcen, ns.xcen, dx, dy, dz, xo, yo, zo, &r2);
        double rcut_src = ns.hmax * RADKERN, rcut_dst = nd.hmax * RADKERN;
        double rcut = fmax_f(rcut_dst, rcut_src);
        double rcut2 = sq(nd.size + ns.size + rcut);
        bool wellsep = (tree_acc2 * r2 > sq(nd.size + ns.size)) && (r2 > rcut2);
        if (wellsep) {
          double dr1 = 1.0 / std::sqrt(r2);
          compute_M2L(dx, dy, dz, dr1, ns.mass, ns.quads, &fb[(size_t)LENFGRAV * ib]);
          stackit = false;
        } else {
          stackit = true;
        }
      }
      if (stackit) {  // open_nodes
        int il = node[isrc].left, ir = node[isrc].right;
        int ibn; bool isdstleaf;
        if (ib - 1 > 0) { ibn = ib - 1; isdstleaf = false; } else { ibn = ib; isdstleaf = true; }
        int idstnext = branch[ibn - 1];
        if (istack + 2 > 4 * MAXDEPTH + 14) return 11;
        if (leaf_is_active[isrc] != 0) {
          if (isdstleaf) {
            cache_neighbours(tl, isrc, maxcache, xo, yo, zo);
          } else {
            stk[0][istack] = idstnext; stk[1][istack] = isrc; stk[2][istack] = ibn; ++istack;
          }
        } else {
          if (il != 0) { stk[0][istack] = idstnext; stk[1][istack] = il; stk[2][istack] = ibn; ++istack; }
          if (ir != 0) { stk[0][istack] = idstnext; stk[1][istack] = ir; stk[2][istack] = ibn; ++istack; }
        }
      }
    }
    // downward pass kdtree.F90:1427-1459
    double fnode[LENFGRAV];
    for (int i = nparents; i >= 2; --i) {
      int iparent = branch[i - 1];
      double dx, dy, dz, xo, yo, zo;
      get_sep(node[branch[i - 2]].xcen, node[iparent].xcen, dx, dy, dz, xo, yo, zo, nullptr);
      for (int k = 0; k < LENFGRAV; ++k) fnode[k] = facc[k] + fb[(size_t)LENFGRAV * i + k];
      propagate(facc, fnode, dx, dy, dz);
    }
    for (int k = 0; k < LENFGRAV; ++k) fnode_out[k] = facc[k] + fb[(size_t)LENFGRAV * 1 + k];
    return 0;
  }

  // ---------------------------------------------------------- density
  // dens.F90:1293-1378 start_cell
  void dens_start_cell(CellDens &c) const {
    c.npcell = 0;
    for (int ip = inoderange[2 * c.icell]; ip <= inoderange[2 * c.icell + 1]; ++ip) {
      int i = inodeparts[ip];
      if (i < 0) continue;
      int k = c.npcell++;
      c.arr_index[k] = ip;
      const double *x = &xyzh[4 * (i - 1)];
      for (int d = 0; d < 3; ++d) c.x[k][d] = x[d];
      c.h[k] = x[3]; c.h_old[k] = x[3];
      for (int d = 0; d < 3; ++d) c.v[k][d] = vxyzu[4 * (i - 1) + d];
      if (p.mhd) for (int d = 0; d < 4; ++d) c.B[k][d] = dens_B[4 * (i - 1) + d];
    }
  }
  // dens.F90:578-857 get_density_sums (path subset: gas only, getdv = .false. under
  // CONST_AV, getdB = mhd, calculate_divcurlB = .true.)
  void get_density_sums(int i, const CellDens &c, int k, double hi, double hi1, double hi21,
                        const TrialList &tl, double *rhosum, int &nneighi, uint64_t &nh,
                        const double *hj_base, int hj_stride, bool getdv) const {
    for (int q = 0; q < 40; ++q) rhosum[q] = 0.0;
    nneighi = 1;  // self (ignoreself)
    nh = 0;
    double dphidhi = 0.0;
    double pmassj = p.massoftype, pmassi = p.massoftype;
    // dens.F90:640-644 f_i for the div a sums (fext = 0 here)
    const double *fi = &fxyzu[4 * (i - 1)];
    const double *vi = &dens_vel[4 * (i - 1)];
    for (int nn = 1; nn <= tl.nneigh; ++nn) {
      int j = tl.list[nn - 1];
      if (j == i) continue;
      double dx, dy, dz;
      if (nn <= ISIZECELLCACHE) {
        const double *cc = &tl.cache[4 * (nn - 1)];
        dx = c.x[k][0] - cc[0]; dy = c.x[k][1] - cc[1]; dz = c.x[k][2] - cc[2];
      } else {
        const double *xj = &xyzh[4 * (j - 1)];
        dx = c.x[k][0] - xj[0]; dy = c.x[k][1] - xj[1]; dz = c.x[k][2] - xj[2];
      }
      if (p.periodic) {
        if (std::fabs(dx) > 0.5 * dxbound) dx = dx - dxbound * fsign1(dx);
        if (std::fabs(dy) > 0.5 * dybound) dy = dy - dybound * fsign1(dy);
        if (std::fabs(dz) > 0.5 * dzbound) dz = dz - dzbound * fsign1(dz);
      }
      double rij2 = dx * dx + dy * dy + dz * dz;
      double q2i = rij2 * hi21;
      if (q2i < RADKERN2) {
        double rij = std::sqrt(rij2);
        double qi = rij * hi1;
        double wabi, grkerni;
        if (p.gravity) get_kernel_grav1(q2i, qi, wabi, grkerni, dphidhi);
        else get_kernel(q2i, qi, wabi, grkerni);
        double dwdhi = (-qi * grkerni - 3.0 * wabi);
        rhosum[1] = rhosum[1] + wabi * pmassj;
        rhosum[2] = rhosum[2] + dwdhi * pmassj;
        rhosum[3] = rhosum[3] + dphidhi * pmassj;
        nneighi = nneighi + 1;
        nh += mix64((uint64_t)j);
        if (getdv || p.mhd) {  // (getdv .or. getdB) .and. calculate_divcurlB (dens.F90:745-756)
          double rij1 = 1.0 / (rij + EPS_D);
          double rij1grkern = rij1 * grkerni;
          double runix = dx * rij1grkern * pmassj;
          double runiy = dy * rij1grkern * pmassj;
          double runiz = dz * rij1grkern * pmassj;
          if (getdv) {  // dens.F90:758-802
            const double *vj = &dens_vel[4 * (j - 1)];
            double dvx = vi[0] - vj[0], dvy = vi[1] - vj[1], dvz = vi[2] - vj[2];
            double projv = dvx * runix + dvy * runiy + dvz * runiz;
            rhosum[4] = rhosum[4] + projv;
            rhosum[5] = rhosum[5] + dvx * runix; rhosum[6] = rhosum[6] + dvx * runiy; rhosum[7] = rhosum[7] + dvx * runiz;
            rhosum[8] = rhosum[8] + dvy * runix; rhosum[9] = rhosum[9] + dvy * runiy; rhosum[10] = rhosum[10] + dvy * runiz;
            rhosum[11] = rhosum[11] + dvz * runix; rhosum[12] = rhosum[12] + dvz * runiy; rhosum[13] = rhosum[13] + dvz * runiz;
            if (p.nalpha > 1) {  // div a for the Cullen & Dehnen switch
              const double *fj = &fxyzu[4 * (j - 1)];
              double dax = fi[0] - fj[0], day = fi[1] - fj[1], daz = fi[2] - fj[2];
              rhosum[14] = rhosum[14] + dax * runix; rhosum[15] = rhosum[15] + dax * runiy; rhosum[16] = rhosum[16] + dax * runiz;
              rhosum[17] = rhosum[17] + day * runix; rhosum[18] = rhosum[18] + day * runiy; rhosum[19] = rhosum[19] + day * runiz;
              rhosum[20] = rhosum[20] + daz * runix; rhosum[21] = rhosum[21] + daz * runiy; rhosum[22] = rhosum[22] + daz * runiz;
            }
            rhosum[23] = rhosum[23] - dx * runix; rhosum[24] = rhosum[24] - dx * runiy;
            rhosum[25] = rhosum[25] - dx * runiz; rhosum[26] = rhosum[26] - dy * runiy;
            rhosum[27] = rhosum[27] - dy * runiz; rhosum[28] = rhosum[28] - dz * runiz;
          }
          if (p.mhd) {  // getdB (dens.F90:806-829)
            double rhoi = rhoh(hi);
            double rhoj = rhoh(hj_base[(size_t)hj_stride * (j - 1)]);
            double dBx = c.B[k][0] * rhoi - dens_B[4 * (j - 1) + 0] * rhoj;
            double dBy = c.B[k][1] * rhoi - dens_B[4 * (j - 1) + 1] * rhoj;
            double dBz = c.B[k][2] * rhoi - dens_B[4 * (j - 1) + 2] * rhoj;
            double projdB = dBx * runix + dBy * runiy + dBz * runiz;
            rhosum[29] = rhosum[29] + projdB;
            rhosum[30] = rhosum[30] + dBx * runix; rhosum[31] = rhosum[31] + dBx * runiy; rhosum[32] = rhosum[32] + dBx * runiz;
            rhosum[33] = rhosum[33] + dBy * runix; rhosum[34] = rhosum[34] + dBy * runiy; rhosum[35] = rhosum[35] + dBy * runiz;
            rhosum[36] = rhosum[36] + dBz * runix; rhosum[37] = rhosum[37] + dBz * runiy; rhosum[38] = rhosum[38] + dBz * runiz;
          }
        }
      }
    }
    (void)pmassi;
  }
  // dens.F90:866-891 calculate_rmatrix_from_sums
  static void rmatrix_from_sums(const double *rs, double &denom, double *rm) {
    const double rxx = rs[23], rxy = rs[24], rxz = rs[25], ryy = rs[26], ryz = rs[27], rzz = rs[28];
    denom = rxx * ryy * rzz + 2.0 * rxy * rxz * ryz - rxx * ryz * ryz - ryy * rxz * rxz - rzz * rxy * rxy;
    rm[0] = ryy * rzz - ryz * ryz; rm[1] = rxz * ryz - rzz * rxy; rm[2] = rxy * ryz - rxz * ryy;
    rm[3] = rzz * rxx - rxz * rxz; rm[4] = rxy * rxz - rxx * ryz; rm[5] = rxx * ryy - rxy * rxy;
  }
  // dens.F90:1086-1101 exactlinear
  static void exactlinear(double &gx, double &gy, double &gz, double ax, double ay, double az, const double *rm,
                          double ddenom) {
    gx = (ax * rm[0] + ay * rm[1] + az * rm[2]) * ddenom;
    gy = (ax * rm[1] + ay * rm[3] + az * rm[4]) * ddenom;
    gz = (ax * rm[2] + ay * rm[4] + az * rm[5]) * ddenom;
  }
  // dens.F90:899-989 calculate_divcurlv_from_sums (ndivcurlv = 1, nalpha >= 2,
  // use_exact_linear) and dens.F90:997-1055 calculate_strain_from_sums:
  // div v, d(div v)/dt for the switch (divcurlvi(5)) and the strain dvdx(9)
  static void dv_from_sums(const double *rs, double term, double &divv, double &ddivvdt, double *dv) {
    double denom, rm[6];
    rmatrix_from_sums(rs, denom, rm);
    divv = -rs[4] * term;
    double gax = 0, gay = 0, gaz = 0, gv[9];
    if (std::fabs(denom) > TINY_D) {
      const double ddenom = 1.0 / denom;
      double t1, t2, t3;
      exactlinear(gax, t1, t2, rs[14], rs[15], rs[16], rm, ddenom);
      exactlinear(t1, gay, t2, rs[17], rs[18], rs[19], rm, ddenom);
      exactlinear(t1, t2, gaz, rs[20], rs[21], rs[22], rm, ddenom);
      exactlinear(gv[0], gv[1], gv[2], rs[5], rs[6], rs[7], rm, ddenom);
      exactlinear(gv[3], gv[4], gv[5], rs[8], rs[9], rs[10], rm, ddenom);
      exactlinear(gv[6], gv[7], gv[8], rs[11], rs[12], rs[13], rm, ddenom);
      for (int q = 0; q < 9; ++q) dv[q] = -gv[q];
      const double div_a = -(gax + gay + gaz);
      ddivvdt = div_a - (dv[0] * dv[0] + dv[4] * dv[4] + dv[8] * dv[8] +
                         2.0 * (dv[1] * dv[3] + dv[2] * dv[6] + dv[5] * dv[7]));
    } else {
      const double div_a = -term * (rs[14] + rs[18] + rs[22]);
      for (int q = 0; q < 9; ++q) dv[q] = -rs[5 + q] * term;
      ddivvdt = div_a - (dv[0] * dv[0] + dv[4] * dv[4] + dv[8] * dv[8] +
                         2.0 * (dv[1] * dv[3] + dv[2] * dv[6] + dv[5] * dv[7]));
    }
  }
  // shock_capturing.f90:151-177 xi_limiter
  static double xi_limiter(const float *dvdxf) {
    double d[9];
    for (int q = 0; q < 9; ++q) d[q] = (double)dvdxf[q];
    const double divv = d[0] + d[4] + d[8];
    const double cx = d[7] - d[5], cy = d[2] - d[6], cz = d[3] - d[1];
    const double m = std::max(-divv, 0.0);
    const double fac = m * m;
    const double traceS = cx * cx + cy * cy + cz * cz;
    if (fac + traceS > EPS_D) return fac / (fac + traceS);
    return 1.0;
  }
  // shock_capturing.f90:131-143 get_alphaloc
  static double get_alphaloc(double divvdti, double spsoundi, double hi, double xi, double alpha_min,
                             double alpha_max) {
    const double source = 10.0 * (hi * hi) * xi * std::max(-divvdti, 0.0);
    const double temp = spsoundi * spsoundi;
    if (temp > EPS_D) return std::max(std::min(source / temp, alpha_max), alpha_min);
    return alpha_min;
  }
  // dens.F90:1470-1507 finish_rhosum
  void finish_rhosum(const double *rhosum, double hi, bool iterating, double &rhoi, double &gradhi,
                     double &rhohi, double &dhdrhoi, double &omegai, double &gradsofti) const {
    double pmassi = p.massoftype;
    double hi1 = 1.0 / hi, hi21 = hi1 * hi1, hi31 = hi1 * hi21, hi41 = hi21 * hi21;
    rhoi = CNORMK * (rhosum[1] + WAB0 * pmassi) * hi31;
    gradhi = CNORMK * (rhosum[2] + GRADH0 * pmassi) * hi41;
    dhdrhoi = dhdrho(hi);
    omegai = 1.0 - dhdrhoi * gradhi;
    gradhi = 1.0 / omegai;
    if (iterating) {
      rhohi = rhoh(hi);
    } else {
      gradsofti = (rhosum[3] + DPHIDH0 * pmassi) * hi21;
      gradsofti = gradsofti * dhdrhoi;
    }
  }
  // dens.F90:1382-1466 finish_cell
  int finish_cell(CellDens &c, bool &cell_converged) const {
    c.nits = c.nits + 1;
    cell_converged = true;
    for (int k = 0; k < c.npcell; ++k) {
      double hi = c.h[k], hi_old = c.h_old[k];
      double rhoi, gradhi, rhohi, dhdrhoi, omegai, gs;
      finish_rhosum(c.rhosums[k], hi, true, rhoi, gradhi, rhohi, dhdrhoi, omegai, gs);
      double func = rhohi - rhoi;
      double dfdh1 = (omegai > TINY_D) ? dhdrhoi / omegai : dhdrhoi / std::fabs(omegai + EPS_D);
      double hnew = hi - func * dfdh1;
      if (hnew > 1.2 * hi) hnew = 1.2 * hi;
      else if (hnew < 0.8 * hi) hnew = 0.8 * hi;
      bool conv = ((std::fabs(hnew - hi) / hi_old) < p.tolh && omegai > 0.0 && hi > 0.0);
      if (cell_converged) cell_converged = conv;
      if (!conv && c.nits >= MAXDENSITS) return 20;  // dens.F90:1443-1456 fatal
      c.h[k] = conv ? hi : hnew;
    }
    return 0;
  }
  // neigh_kdtree.f90:115-131 set_hmaxcell
  void set_hmaxcell(int inode, double hmaxcell) {
    int nn = inode;
    node[nn].hmax = hmaxcell;
    while (node[nn].parent != 0) {
      nn = node[nn].parent;
#pragma omp critical(ora_hmax)
      node[nn].hmax = fmax_f(node[nn].hmax, hmaxcell);
    }
  }

  int densityiterate(int icall) {  // dens.F90:117-568 (local cells; no MPI)
    if (!have_tree) return 30;
    // dens.F90:202-203: velocity derivatives for the viscosity switch or curl v
    const bool getdv = (p.nalpha >= 2 || p.curlv) && (icall <= 1 || icall == 3);
    const int ndv = ndivcurlv();
    // a direct call reads the state's arrays (pointers reset on every return:
    // the state vectors may be reallocated by the next set_particles)
    const bool own_v = !dens_vel, own_B = !dens_B;
    if (own_v) dens_vel = vxyzu.data();
    if (own_B) dens_B = Bevol.data();
    struct Reset {
      const double **a, **b;
      bool ra, rb;
      ~Reset() { if (ra) *a = nullptr; if (rb) *b = nullptr; }
    } reset{&dens_vel, &dens_B, own_v, own_B};
    ora_stats st{};
    st.ncells = stats.ncells; st.maxlevel = stats.maxlevel; st.minlevel = stats.minlevel;
    std::vector<double> h_entry;
    if (p.mhd) {
      if (p.divB_hj_prepass) {
        h_entry.resize(n);
        for (int64_t i = 0; i < n; ++i) h_entry[i] = xyzh[4 * i + 3];
      }
    }
    nneigh_out.assign(n, 0);
    nhash_out.assign(n, 0);
    int err_all = 0;
    double rhomax = 0.0;
    int64_t nneightry = 0, nneighact = 0, maxneightry = 0, maxneighact = 0, ncalc = 0, np = 0, ncalls = 0;
#pragma omp parallel num_threads(threads()) reduction(+:nneightry,nneighact,ncalc,np,ncalls) \
    reduction(max:maxneightry,maxneighact,rhomax)
    {
      TrialList tl;
      CellDens c;
      // h_j read by the divcurlB sums: the live array (serial order) or the entry copy
      const double *hj_base = (p.mhd && p.divB_hj_prepass) ? h_entry.data() : xyzh.data() + 3;
      const int hj_stride = (p.mhd && p.divB_hj_prepass) ? 1 : 4;
#pragma omp for schedule(dynamic, 16)
      for (int64_t icell = 1; icell <= ncells; ++icell) {
        if (leaf_is_active[icell] <= 0) continue;
        if (err_all) continue;
        int err = 0;
        double xsz = node[icell].size, rc = RADKERN * node[icell].hmax;
        err = getneigh(node[icell].xcen, xsz, rc, tl, 3, false);
        c.icell = (int)icell; c.nits = 0;
        dens_start_cell(c);
        for (int d = 0; d < 3; ++d) c.xpos[d] = node[icell].xcen[d];
        c.xsizei = xsz; c.rcuti = rc; c.hmax = node[icell].hmax;
        auto compute_cell = [&]() {  // dens.F90:1203-1271
          for (int k = 0; k < c.npcell; ++k) {
            int lli = inodeparts[c.arr_index[k]];
            double hi = c.h[k], hi1 = 1.0 / hi, hi21 = hi1 * hi1;
            get_density_sums(lli, c, k, hi, hi1, hi21, tl, c.rhosums[k], c.nneigh[k], c.nhash[k],
                             hj_base, hj_stride, getdv);
          }
          c.nneightry = tl.nneigh;
        };
        compute_cell();
        bool converged = false;
        while (!converged && !err) {
          err = finish_cell(c, converged);
          if (err) break;
          // compute_hmax dens.F90:1275-1289
          bool redo = false;
          if (c.npcell > 0) {
            double hmax_old = c.hmax;
            double hm = c.h[0];
            for (int k = 1; k < c.npcell; ++k) hm = std::max(hm, c.h[k]);
            double hmax = 1.01 * hm;
            if (hmax > hmax_old) redo = true;
            c.hmax = hmax; c.rcuti = RADKERN * hmax;
          }
          if (icall == 0) converged = true;
          if (!converged) {
            if (redo) {
              set_hmaxcell(c.icell, c.hmax);
              err = getneigh(c.xpos, c.xsizei, c.rcuti, tl, 3, false);
              ++ncalls;
            }
            compute_cell();
          }
        }
        if (err) {
#pragma omp atomic write
          err_all = err;
          continue;
        }
        // store_results dens.F90:1511-1681
        for (int k = 0; k < c.npcell; ++k) {
          int lli = inodeparts[c.arr_index[k]];
          double hi = c.h[k];
          if (hi < 0.0) { err = 21; break; }
          double hi1 = 1.0 / hi, hi21 = hi1 * hi1, hi41 = hi21 * hi21;
          (void)hi21;
          double rhoi, gradhi, rhohi, dhdrhoi, omegai, gradsofti;
          finish_rhosum(c.rhosums[k], hi, false, rhoi, gradhi, rhohi, dhdrhoi, omegai, gradsofti);
          double hnew = hrho(rhoi);
          xyzh[4 * (lli - 1) + 3] = hnew;
          treecache[5 * c.arr_index[k] + 3] = hnew;
          if (hnew < 0.0) { err = 22; break; }
          gradh[2 * (lli - 1) + 0] = (float)gradhi;
          if (p.gravity) gradh[2 * (lli - 1) + 1] = (float)gradsofti;
          gradh_d[2 * (lli - 1) + 0] = gradhi;
          if (p.gravity) gradh_d[2 * (lli - 1) + 1] = gradsofti;
          rhomax = fmax_f(rhomax, rhoi);
          double gradhf = (double)gradh[2 * (lli - 1) + 0];
          double rho1i = 1.0 / rhoi;
          double term = CNORMK * gradhf * rho1i * hi41;
          if (getdv) {  // dens.F90:1630-1637, 1655-1663
            const double *rs = c.rhosums[k];
            if (p.nalpha >= 2) {
              double divv, ddivvdt, dv[9];
              dv_from_sums(rs, term, divv, ddivvdt, dv);
              divcurlv[(size_t)ndv * (lli - 1)] = (float)divv;
              alphaind[3 * (lli - 1) + 2] = (float)ddivvdt;
              for (int q = 0; q < 9; ++q) dvdx[9 * (lli - 1) + q] = (float)dv[q];
            } else {
              divcurlv[(size_t)ndv * (lli - 1)] = (float)(-rs[4] * term);
            }
            if (p.curlv) {  // dens.F90:919-923 curl v from the velocity-gradient sums
              float *cv = &divcurlv[(size_t)ndv * (lli - 1)];
              cv[1] = (float)(-(rs[12] - rs[10]) * term);
              cv[2] = (float)(-(rs[7] - rs[11]) * term);
              cv[3] = (float)(-(rs[8] - rs[6]) * term);
            }
          } else {
            divcurlv[(size_t)ndv * (lli - 1)] = -(float)(c.rhosums[k][4] * term);
            if (p.nalpha >= 2) alphaind[3 * (lli - 1) + 1] = 0.0f;  // dens.F90:1640
          }
          if (p.mhd) {
            const double *rs = c.rhosums[k];
            divcurlB[4 * (lli - 1) + 0] = (float)(-rs[29] * term);
            divcurlB[4 * (lli - 1) + 1] = (float)(-(rs[37] - rs[35]) * term);
            divcurlB[4 * (lli - 1) + 2] = (float)(-(rs[32] - rs[36]) * term);
            divcurlB[4 * (lli - 1) + 3] = (float)(-(rs[33] - rs[31]) * term);
          }
          nneightry += c.nneightry;
          nneighact += c.nneigh[k];
          maxneightry = std::max<int64_t>(maxneightry, c.nneightry);
          maxneighact = std::max<int64_t>(maxneighact, c.nneigh[k]);
          nneigh_out[lli - 1] = c.nneigh[k];
          nhash_out[lli - 1] = c.nhash[k];
        }
        np += c.npcell;
        ncalc += (int64_t)c.npcell * c.nits;
        if (err) {
#pragma omp atomic write
          err_all = err;
        }
      }
    }
    if (err_all) return err_all;
    st.nneightry = nneightry; st.nneighact = nneighact; st.maxneightry = maxneightry;
    st.maxneighact = maxneighact; st.ncalc = ncalc; st.np = np; st.ncalls_neigh = ncalls;
    st.rhomax = rhomax;
    stats = st;
    return 0;
  }

  // ---------------------------------------------------------- EOS
  // cons2prim.f90:326-394 + eos.f90:184-237
  void cons2prim(const std::vector<double> &vel) {
    eos.assign(2 * n, 0.0);
    for (int64_t i = 0; i < n; ++i) {
      double hi = xyzh[4 * i + 3];
      if (hi < TINY_D) continue;
      double rhoi = rhoh(hi);
      double ponrhoi, spsound;
      if (p.ieos == 1) {
        ponrhoi = p.polyk; spsound = std::sqrt(ponrhoi);
      } else {
        double eni = vel[4 * i + 3];
        if (p.gamma > 1.0001) ponrhoi = (p.gamma - 1.0) * eni; else ponrhoi = 2.0 / 3.0 * eni;
        spsound = std::sqrt(p.gamma * ponrhoi);
      }
      eos[2 * i + 0] = ponrhoi * rhoi;
      eos[2 * i + 1] = spsound;
      if (p.nalpha >= 2) {  // cons2prim.f90:413-418 Cullen & Dehnen alphaloc
        const double xi = xi_limiter(&dvdx[9 * i]);
        alphaind[3 * i + 1] = (float)get_alphaloc((double)alphaind[3 * i + 2], spsound, hi, xi, p.alpha,
                                                  alphamax());
      }
    }
  }

  // ---------------------------------------------------------- force
  // force.F90:2068-2168 get_stress (no physical viscosity, no radiation)
  void get_stress(double pri, double spsoundi, double rhoi, double rho1i, double Bxi, double Byi,
                  double Bzi, double &pro2i, double &vwavei, double *s) const {
    double pmassi = p.massoftype;
    for (int k = 0; k < 6; ++k) s[k] = 0.0;
    double stressiso = 0.0;
    if (p.mhd) {
      double Brhoxi = Bxi * rho1i, Brhoyi = Byi * rho1i, Brhozi = Bzi * rho1i;
      double Bro2i = Brhoxi * Brhoxi + Brhoyi * Brhoyi + Brhozi * Brhozi;
      double valfven2i = Bro2i * rhoi;
      vwavei = std::sqrt(spsoundi * spsoundi + valfven2i);
      s[0] = s[0] - pmassi * Brhoxi * Brhoxi;
      s[1] = s[1] - pmassi * Brhoxi * Brhoyi;
      s[2] = s[2] - pmassi * Brhoxi * Brhozi;
      s[3] = s[3] - pmassi * Brhoyi * Brhoyi;
      s[4] = s[4] - pmassi * Brhoyi * Brhozi;
      s[5] = s[5] - pmassi * Brhozi * Brhozi;
      pro2i = (pri + 0.0) * rho1i * rho1i + stressiso + 0.5 * Bro2i;
    } else {
      pro2i = (pri + 0.0) * rho1i * rho1i + stressiso;
      vwavei = spsoundi;
    }
  }

  struct ForceI {  // force.F90 xpartvec subset (start_cell :2172-2514)
    int ip;
    double x[3], h, gradh1, gradh2, v[3], en, B[4], alpha, rho, vwave, pr, cs, s[6], pro2;
  };

  int force(int icall, double dt, const std::vector<double> &vel, const std::vector<double> &Bv) {
    (void)dt;
    if (!have_tree) return 30;
    if (!p.ind_timesteps) {  // with individual timesteps inactive particles keep their forces
      fxyzu.assign(4 * n, 0.0);
      dBevol.assign(4 * n, 0.0);
      divBsymm.assign(n, 0.0f);
      poten.assign(n, 0.0f);
    }
    double dtc_glob = BIGNUMBER, dtf_glob = BIGNUMBER;
    int err_all = 0;
    int nbinmaxnew = 0, ncheckbin = 0;
    dt_too_small_any = 0;
    const double pmass = p.massoftype;
    const bool adiab = !p.isothermal;  // maxvxyzu >= 4
#pragma omp parallel num_threads(threads()) reduction(min:dtc_glob,dtf_glob) reduction(max:nbinmaxnew) \
    reduction(+:ncheckbin)
    {
      TrialList tl;
      std::vector<ForceI> cell;
      cell.reserve(MAXLEAF + 2);
#pragma omp for schedule(dynamic, 16)
      for (int64_t icell = 1; icell <= ncells; ++icell) {
        if (leaf_is_active[icell] <= 0) continue;
        if (err_all) continue;
        int err = 0;
        cell.clear();
        for (int ip = inoderange[2 * icell]; ip <= inoderange[2 * icell + 1]; ++ip) {
          int i = inodeparts[ip];
          if (i < 0) continue;
          ForceI f{};
          f.ip = ip;
          double hi = xyzh[4 * (i - 1) + 3];
          if (hi < 0.0) { err = 23; break; }
          // rhoanddhdrho part.F90:802-817
          double hi1 = 1.0 / std::fabs(hi);
          double rhoi = pmass * cube(p.hfact * hi1);
          double rho1i = 1.0 / rhoi;
          double Bxi = 0, Byi = 0, Bzi = 0;
          if (p.mhd) {
            Bxi = Bv[4 * (i - 1) + 0] * rhoi; Byi = Bv[4 * (i - 1) + 1] * rhoi; Bzi = Bv[4 * (i - 1) + 2] * rhoi;
          }
          double pri = eos[2 * (i - 1)], cs = eos[2 * (i - 1) + 1];
          get_stress(pri, cs, rhoi, rho1i, Bxi, Byi, Bzi, f.pro2, f.vwave, f.s);
          for (int d = 0; d < 3; ++d) f.x[d] = xyzh[4 * (i - 1) + d];
          f.h = hi;
          f.gradh1 = gh(2 * (i - 1));
          f.gradh2 = gh(2 * (i - 1) + 1);
          for (int d = 0; d < 3; ++d) f.v[d] = vel[4 * (i - 1) + d];
          f.en = adiab ? vel[4 * (i - 1) + 3] : 0.0;
          if (p.mhd) for (int d = 0; d < 4; ++d) f.B[d] = Bv[4 * (i - 1) + d];
          f.alpha = p.nalpha > 0 ? (double)alphaind[3 * (i - 1)] : p.alpha;  // force.F90:2430-2433
          f.rho = rhoi; f.pr = pri; f.cs = cs;
          cell.push_back(f);
        }
        if (err) {
#pragma omp atomic write
          err_all = err;
          continue;
        }
        if (cell.empty()) continue;
        double fgrav[LENFGRAV] = {0};
        if (p.gravity) {
          err = getneigh_dual((int)icell, node[icell].xcen, node[icell].size, RADKERN * node[icell].hmax, tl, 4, fgrav);
        } else {
          err = getneigh(node[icell].xcen, node[icell].size, RADKERN * node[icell].hmax, tl, 4, true);
        }
        if (err) {
#pragma omp atomic write
          err_all = err;
          continue;
        }
        for (size_t ic = 0; ic < cell.size(); ++ic) {
          const ForceI &fi = cell[ic];
          int i = inodeparts[fi.ip];
          double fsum[20];
          double vsigmax;
          int ibin_neighi = 0;
          compute_forces(i, fi, tl, vel, Bv, fsum, vsigmax, p.ind_timesteps ? ibin_wake.data() : nullptr,
                         ibinnow - 1, ibin_neighi);
          // finish_cell_and_store_results force.F90:2649-3330
          double hi = fi.h, hi1 = 1.0 / hi;
          double rhoi = fi.rho, rho1i = 1.0 / rhoi, pri = fi.pr, vwavei = fi.vwave;
          double dtc = p.dtmax, dtf = BIGNUMBER, dtclean = BIGNUMBER;
          double Bxyz[3] = {0, 0, 0}, B2i = 0.0;
          if (p.mhd) {
            Bxyz[0] = fi.B[0] * rhoi; Bxyz[1] = fi.B[1] * rhoi; Bxyz[2] = fi.B[2] * rhoi;
            B2i = sq(Bxyz[0]) + sq(Bxyz[1]) + sq(Bxyz[2]);
          }
          if (p.gravity) {
            double potensoft0, dum;
            kernel_softening(0.0, 0.0, potensoft0, dum);
            double epoti = 0.5 * pmass * (fsum[3] + pmass * potensoft0 * hi1);
            double dx = fi.x[0] - node[icell].xcen[0], dy = fi.x[1] - node[icell].xcen[1], dz = fi.x[2] - node[icell].xcen[2];
            double fxi, fyi, fzi, poti;
            expand_taylor(fgrav, dx, dy, dz, fxi, fyi, fzi, poti);
            fsum[0] = fsum[0] + fxi; fsum[1] = fsum[1] + fyi; fsum[2] = fsum[2] + fzi;
            epoti = epoti + 0.5 * pmass * poti;
            poten[i - 1] = (float)epoti;
          }
          if (p.mhd) {
            double divBsymmi = fsum[7], frac_divB;
            if (B2i > 0.0) {
              double betai = 2.0 * pri / B2i;
              if (betai < 2.0) frac_divB = 1.0;
              else if (betai < 10.0) frac_divB = (10.0 - betai) * 0.125;
              else frac_divB = 0.0;
            } else frac_divB = 0.0;
            fsum[0] = fsum[0] - Bxyz[0] * divBsymmi * frac_divB;
            fsum[1] = fsum[1] - Bxyz[1] * divBsymmi * frac_divB;
            fsum[2] = fsum[2] - Bxyz[2] * divBsymmi * frac_divB;
            divBsymm[i - 1] = (float)(rhoi * divBsymmi);
          }
          double f2i = sq(fsum[0]) + sq(fsum[1]) + sq(fsum[2]);
          double *fo = &fxyzu[4 * (i - 1)];
          fo[0] = fsum[0]; fo[1] = fsum[1]; fo[2] = fsum[2];
          double drhodti = pmass * fsum[4];
          double divvi = -drhodti * rho1i;
          divcurlv[(size_t)ndivcurlv() * (i - 1)] = (float)divvi;
          if (adiab) {
            double fxyz4 = 0.0, fac = rhoi / rhoi;
            double pdv_work = fac * pri * rho1i * rho1i * drhodti;
            if (p.ipdv_heating > 0) fxyz4 = fxyz4 + pdv_work;
            if (p.ishock_heating > 0) fxyz4 = fxyz4 + fac * fsum[5];
            fxyz4 = fxyz4 + fac * fsum[6];
            fo[3] = fxyz4;
          }
          if (p.mhd) {
            double *db = &dBevol[4 * (i - 1)];
            db[0] = fsum[8]; db[1] = fsum[9]; db[2] = fsum[10];
            if (p.psidecayfac > 0.0) {
              double vcleani = p.overcleanfac * vwavei;
              double dtau = p.psidecayfac * vcleani * hi1;
              double psii = fi.B[3];
              db[3] = -vcleani * fsum[11] * rho1i - psii * dtau - 0.5 * psii * divvi;
              dtclean = p.C_cour * hi / (vcleani + TINY_D);
            }
          }
          double vsigdtc = fmax_f(vsigmax, vwavei);
          if (vsigdtc > TINY_D) dtc = p.C_cour * hi / (vsigdtc * fmax_f(p.alpha, 1.0));
          if (adiab) {
            double eni = fi.en;
            if (eni + dtc * fo[3] < EPS_D && eni > EPS_D) fo[3] = fo[3] / (1.0 - dtc * fo[3] / eni);
          }
          if (dtc < TINY_D || dtc > HUGE_D) { err = 24; break; }
          if (std::fabs(f2i) > EPS_D) dtf = p.C_force * std::sqrt(hi / std::sqrt(f2i));
          if (p.ind_timesteps) {  // force.F90:3273-3310
            double dti = dtc;
            const double dtitmp = fmin_f(dtf, dtclean);
            if (dtitmp < dti + TINY_D && dtitmp < p.dtmax) dti = dtitmp;
            int8_t b = ibin[i - 1];
            get_newbin(dti, p.dtmax, b, icall < 2);
            b = (int8_t)std::max((int)b, ibin_neighi - 1);  // Saitoh-Makino limiter
            ibin[i - 1] = b;
            nbinmaxnew = std::max(nbinmaxnew, (int)b);
            ++ncheckbin;
          }
          dtc_glob = fmin_f(dtc_glob, dtc);
          dtf_glob = fmin_f(fmin_f(dtf_glob, dtf), dtclean);  // force.F90:3316
        }
        if (err) {
#pragma omp atomic write
          err_all = err;
        }
      }
    }
    if (err_all) return err_all;
    if (dt_too_small_any) dt_too_small = true;
    (void)icall;
    if (p.ind_timesteps) nbinmax = ncheckbin == 0 ? nbinmax : nbinmaxnew;  // force.F90:749-756, 792
    dtcourant = dtc_glob;
    dtforce = dtf_glob;
    return 0;
  }
  // utils_indtimesteps.f90:230-287 get_newbin
  void get_newbin(double dti, double dtmax, int8_t &ibini, bool allow_decrease) {
    const double dlog2 = 1.4426950408889634;
    const int ibin_oldi = ibini;
    int ibin_newi;
    if (dti > dtmax) ibin_newi = 0;
    else if (dti < TINY_D) ibin_newi = MAXBINS;
    else ibin_newi = std::max((int)(std::log(2.0 * dtmax / dti) * dlog2 - EPS_D), 0);
    if (ibin_newi > MAXBINS) {
#pragma omp atomic write
      dt_too_small_any = 1;
    }
    if (ibin_newi > ibin_oldi) {
      ibini = (int8_t)ibin_newi;
    } else if (ibin_newi < ibin_oldi && ibin_oldi <= nbinmax && allow_decrease) {
      if ((long long)istepfrac % (1ll << (nbinmax - (ibin_oldi - 1))) == 0) ibini = (int8_t)(ibini - 1);
    }
  }

  // force.F90:914-2060 compute_forces (gas-gas hydro + ideal MHD + self-gravity)
  void compute_forces(int i, const ForceI &fi, const TrialList &tl, const std::vector<double> &vel,
                      const std::vector<double> &Bv, double *fsum, double &vsigmax, int8_t *wake, int ibinnow_m1,
                      int &ibin_neighi) const {
    ibin_neighi = 0;  // force.F90:1143
    const double pmassi = p.massoftype, pmassj = p.massoftype;
    const bool adiab = !p.isothermal;
    double hi = fi.h, hi1 = 1.0 / hi, hi21 = hi1 * hi1, hi41 = hi21 * hi21;
    double gradhi = (fi.gradh1 > 0.0) ? fi.gradh1 : 1.0;
    double gradsofti = p.gravity ? fi.gradh2 : 0.0;
    double xi = fi.x[0], yi = fi.x[1], zi = fi.x[2];
    double vxi = fi.v[0], vyi = fi.v[1], vzi = fi.v[2];
    double eni = fi.en, vwavei = fi.vwave, rhoi = fi.rho, pri = fi.pr, pro2i = fi.pro2, alphai = fi.alpha;
    double sxxi = fi.s[0], sxyi = fi.s[1], sxzi = fi.s[2], syyi = fi.s[3], syzi = fi.s[4], szzi = fi.s[5];
    double rho1i = 1.0 / rhoi;
    for (int k = 0; k < 20; ++k) fsum[k] = 0.0;
    vsigmax = 0.0;
    double hfacgrkern = hi41 * CNORMK * gradhi;
    double Bxi = 0, Byi = 0, Bzi = 0, psii = 0;
    if (p.mhd) { Bxi = fi.B[0] * rhoi; Byi = fi.B[1] * rhoi; Bzi = fi.B[2] * rhoi; psii = fi.B[3]; }
    double rho21i = rho1i * rho1i;
    double mrhoi5 = 0.5 * pmassi * rho1i;
    double auterm = mrhoi5 * p.alphau;
    double avBterm = mrhoi5 * p.alphaB * rho1i;
    bool usej = false;
    double grkernj = 0, alphaj = alphai, rhoj = 0, rho1j = 0, mrhoj5 = 0, gradpj = 0;
    double projsxj = 0, projsyj = 0, projszj = 0, dudtresist = 0, dpsiterm = 0;
    double fgravi = 0, fgravj = 0, phii = 0, phij = 0;
    double Bxj = 0, Byj = 0, Bzj = 0, psij = 0;
    double rho21j = 0, autermj = 0, avBtermj = 0, projBj = 0, prj = 0, pro2j = 0, vwavej = 0, vsigavj = 0,
           spsoundj = 0;
    double sj[6] = {0, 0, 0, 0, 0, 0};
    const double beta = p.beta;
    for (int nn = 1; nn <= tl.nneigh; ++nn) {
      int j = tl.list[nn - 1];
      if (i == j) continue;
      double xj, yj, zj, hj1;
      bool cached = nn <= ISIZECELLCACHE;
      if (cached) {
        const double *cc = &tl.cache[4 * (nn - 1)];
        xj = cc[0]; yj = cc[1]; zj = cc[2];
      } else {
        xj = xyzh[4 * (j - 1)]; yj = xyzh[4 * (j - 1) + 1]; zj = xyzh[4 * (j - 1) + 2];
      }
      double dx = xi - xj, dy = yi - yj, dz = zi - zj;
      if (p.periodic) {
        if (std::fabs(dx) > 0.5 * dxbound) dx = dx - dxbound * fsign1(dx);
        if (std::fabs(dy) > 0.5 * dybound) dy = dy - dybound * fsign1(dy);
        if (std::fabs(dz) > 0.5 * dzbound) dz = dz - dzbound * fsign1(dz);
      }
      double rij2 = dx * dx + dy * dy + dz * dz;
      double q2i = rij2 * hi21;
      hj1 = cached ? tl.cache[4 * (nn - 1) + 3] : 1.0 / xyzh[4 * (j - 1) + 3];
      double hj21 = hj1 * hj1;
      double q2j = rij2 * hj21;
      bool is_neigh = (q2i < RADKERN2 || q2j < RADKERN2);
      if (is_neigh) {
        double rij1, qi;
        if (rij2 > TINY_D) { rij1 = 1.0 / std::sqrt(rij2); qi = (rij2 * rij1) * hi1; }
        else { rij1 = 0.0; qi = 0.0; }
        double grkerni;
        if (q2i < RADKERN2) {
          grkerni = grkern(q2i, qi) * hfacgrkern;
          if (p.gravity) {
            double fmi;
            kernel_softening(q2i, qi, phii, fmi);
            phii = phii * hi1;
            fmi = fmi * hi21;
            double dsofti = gradsofti * grkerni;
            fgravi = fmi + dsofti;
          }
        } else {
          grkerni = 0.0;
          if (p.gravity) { phii = -rij1; double fmi = rij1 * rij1; fgravi = fmi; }
        }
        double runix = dx * rij1, runiy = dy * rij1, runiz = dz * rij1;
        if (q2j < RADKERN2) {
          double qj = (rij2 * rij1) * hj1;
          grkernj = grkern(q2j, qj) * hj21 * hj21 * CNORMK * gh(2 * (j - 1));
          if (p.gravity) {
            double fmj;
            kernel_softening(q2j, qj, phij, fmj);
            fmj = fmj * hj21;
            double dsoftj = gh(2 * (j - 1) + 1) * grkernj;
            fgravj = fmj + dsoftj;
          }
          usej = true;
        } else {
          grkernj = 0.0;
          if (p.gravity) { double fmj = rij1 * rij1; fgravj = fmj; }
          usej = false;
        }
        if (p.mhd) usej = true;
        if (adiab && !p.gravity) usej = true;
        if (p.ind_timesteps) {  // force.F90:1346-1353: j may need waking next step
          int8_t *wj = &wake[j - 1];
          int8_t cur;
#pragma omp atomic read
          cur = *wj;
          while ((int)cur < ibinnow_m1) {
            int8_t want = (int8_t)ibinnow_m1;
            if (__atomic_compare_exchange_n(wj, &cur, want, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) break;
          }
          ibin_neighi = std::max(ibin_neighi, (int)ibin_old[j - 1]);
        }
        double fgrav = 0.5 * (pmassj * fgravi + pmassi * fgravj);
        double vxj = vel[4 * (j - 1)], vyj = vel[4 * (j - 1) + 1], vzj = vel[4 * (j - 1) + 2];
        double dvx = vxi - vxj, dvy = vyi - vyj, dvz = vzi - vzj;
        double projv = dvx * runix + dvy * runiy + dvz * runiz;
        double denij = 0.0;
        if (adiab) { double enj = vel[4 * (j - 1) + 3]; denij = eni - enj; }
        double vsigi = fmax_f(vwavei - beta * projv, 0.0);
        double vsigavi = fmax_f(alphai * vwavei - beta * projv, 0.0);
        if (vsigi > vsigmax) vsigmax = vsigi;
        double dBx = 0, dBy = 0, dBz = 0, projBi = 0, projdB = 0, dB2 = 0, divBdiffterm = 0;
        if (p.mhd) {
          double hjm = xyzh[4 * (j - 1) + 3];
          double rhojm = rhoh(hjm);
          Bxj = Bv[4 * (j - 1)] * rhojm; Byj = Bv[4 * (j - 1) + 1] * rhojm; Bzj = Bv[4 * (j - 1) + 2] * rhojm;
          psij = Bv[4 * (j - 1) + 3];
          dBx = Bxi - Bxj; dBy = Byi - Byj; dBz = Bzi - Bzj;
          projBi = Bxi * runix + Byi * runiy + Bzi * runiz;
          if (usej) projBj = Bxj * runix + Byj * runiy + Bzj * runiz;
          projdB = dBx * runix + dBy * runiy + dBz * runiz;
          dB2 = dBx * dBx + dBy * dBy + dBz * dBz;
          divBdiffterm = -pmassj * projdB * grkerni;
          rhoj = rhojm;
        }
        if (usej) {
          double hj = 1.0 / hj1;
          rhoj = rhoh(hj);
          rho1j = 1.0 / rhoj;
          rho21j = rho1j * rho1j;
          prj = eos[2 * (j - 1)];
          spsoundj = eos[2 * (j - 1) + 1];
          get_stress(prj, spsoundj, rhoj, rho1j, Bxj, Byj, Bzj, pro2j, vwavej, sj);
          mrhoj5 = 0.5 * pmassj * rho1j;
          autermj = mrhoj5 * p.alphau;
          avBtermj = mrhoj5 * p.alphaB * rho1j;
          if (p.nalpha > 0) alphaj = (double)alphaind[3 * (j - 1)];  // force.F90:1478
          double vsigj = fmax_f(vwavej - beta * projv, 0.0);
          vsigavj = fmax_f(alphaj * vwavej - beta * projv, 0.0);
          if (vsigj > vsigmax) vsigmax = vsigj;
        } else {
          rho1j = 0; rho21j = 0; mrhoj5 = 0; autermj = 0; avBtermj = 0; psij = 0; gradpj = 0;
          projsxj = 0; projsyj = 0; projszj = 0; projBj = 0; prj = 0; pro2j = 0; vwavej = 0; vsigavj = 0;
          spsoundj = 0;
          for (int k = 0; k < 6; ++k) sj[k] = 0.0;
        }
        // gas-gas (force.F90:1539-1850)
        double qrho2i = 0.0, qrho2j = 0.0;
        if (projv < 0.0) {
          qrho2i = -0.5 * rho1i * vsigavi * projv;
          if (usej) qrho2j = -0.5 * rho1j * vsigavj * projv;
        }
        double dudtdissi = pmassj * qrho2i * projv * grkerni;
        double gradpi = pmassj * (pro2i + qrho2i) * grkerni;
        if (usej) gradpj = pmassj * (pro2j + qrho2j) * grkernj;
        double dendissterm = 0.0;
        if (adiab) {
          double vsigu;
          if (p.gravity) vsigu = std::fabs(projv);
          else { double rhoav1 = 2.0 / (rhoi + rhoj); vsigu = std::sqrt(std::fabs(pri - prj) * rhoav1); }
          dendissterm = vsigu * denij * (auterm * grkerni + autermj * grkernj);
        }
        double dBevolx = 0, dBevoly = 0, dBevolz = 0, divBsymmterm = 0;
        if (p.mhd) {
          double vsigB = std::sqrt(sq(dvx - projv * runix) + sq(dvy - projv * runiy) + sq(dvz - projv * runiz));
          double dBdissterm = (avBterm * grkerni + avBtermj * grkernj) * vsigB;
          if (p.iresistive_heating > 0) dudtresist = -0.5 * dB2 * dBdissterm;
          double pmjrho21grkerni = pmassj * rho21i * grkerni;
          double pmjrho21grkernj = pmassj * rho21j * grkernj;
          double termi = pmjrho21grkerni * projBi;
          divBsymmterm = termi + pmjrho21grkernj * projBj;
          double dBrhoterm = -termi;
          dpsiterm = p.overcleanfac * (pmjrho21grkerni * psii * vwavei + pmjrho21grkernj * psij * vwavej);
          dBevolx = dBrhoterm * dvx + dBdissterm * dBx - dpsiterm * runix;
          dBevoly = dBrhoterm * dvy + dBdissterm * dBy - dpsiterm * runiy;
          dBevolz = dBrhoterm * dvz + dBdissterm * dBz - dpsiterm * runiz;
        }
        double projsxi = (sxxi * runix + sxyi * runiy + sxzi * runiz) * grkerni;
        double projsyi = (sxyi * runix + syyi * runiy + syzi * runiz) * grkerni;
        double projszi = (sxzi * runix + syzi * runiy + szzi * runiz) * grkerni;
        if (usej) {
          projsxj = (sj[0] * runix + sj[1] * runiy + sj[2] * runiz) * grkernj;
          projsyj = (sj[1] * runix + sj[3] * runiy + sj[4] * runiz) * grkernj;
          projszj = (sj[2] * runix + sj[4] * runiy + sj[5] * runiz) * grkernj;
        }
        double gradp = gradpi + gradpj;
        double projsx = projsxi + projsxj, projsy = projsyi + projsyj, projsz = projszi + projszj;
        fsum[0] = fsum[0] - runix * (gradp + fgrav) - projsx;
        fsum[1] = fsum[1] - runiy * (gradp + fgrav) - projsy;
        fsum[2] = fsum[2] - runiz * (gradp + fgrav) - projsz;
        fsum[3] = fsum[3] + pmassj * phii;
        fsum[4] = fsum[4] + projv * grkerni;
        if (adiab) {
          fsum[5] = fsum[5] + dudtdissi + dudtresist;
          fsum[6] = fsum[6] + dendissterm;
        }
        if (p.mhd) {
          fsum[7] = fsum[7] + divBsymmterm;
          fsum[8] = fsum[8] + dBevolx; fsum[9] = fsum[9] + dBevoly; fsum[10] = fsum[10] + dBevolz;
          fsum[11] = fsum[11] + divBdiffterm;
        }
      } else if (p.gravity) {
        // trial neighbour outside both kernels: plain 1/r^2 (force.F90:1991-2053)
        double rij1 = 1.0 / std::sqrt(rij2);
        double fg = rij1 * rij1 * rij1;
        double ph = -rij1;
        double fgj = fg * pmassj;
        fsum[0] = fsum[0] - dx * fgj;
        fsum[1] = fsum[1] - dy * fgj;
        fsum[2] = fsum[2] - dz * fgj;
        fsum[3] = fsum[3] + pmassj * ph;
      }
    }
    (void)rho21j;
  }

  // ---------------------------------------------------------- derivs + step
  int derivs(int icall, double dt, const std::vector<double> &vel, const std::vector<double> &Bv, double *dtnew) {
    int err = 0;
    if (icall == 1 || icall == 0) { err = maketree(); if (err) return err; }
    if (icall == 1) {
      dens_vel = vel.data();
      dens_B = Bv.data();
      err = densityiterate(1);
      dens_vel = nullptr;
      dens_B = nullptr;
      if (err) return err;
    }
    cons2prim(vel);
    err = force(icall, dt, vel, Bv);
    if (err) return err;
    if (dtnew) *dtnew = fmin_f(fmin_f(dtforce, dtcourant), fmin_f(BIGNUMBER, p.dtmax));  // deriv.f90:226
    return 0;
  }

  // ---------------------------------------------------------- individual timesteps
  static double get_dt(double dtmax, int ibini) { return dtmax / std::ldexp(1.0, ibini); }  // utils_indtimesteps.f90:45
  // evol_init (evolve.f90:77-81) + init_step (step_leapfrog.f90:45-84), after the initial derivs
  void ind_init(double time) {
    dtsub = p.dtmax / std::ldexp(1.0, nbinmax);
    if (time < TINY_D) for (int64_t i = 0; i < n; ++i) ibin[i] = (int8_t)nbinmax;
    for (int64_t i = 0; i < n; ++i) twas[i] = time + 0.5 * get_dt(p.dtmax, ibin[i]);
    for (int b = 0; b <= MAXBINS; ++b) {
      ibin_dts[0][b] = get_dt(p.dtmax, b);
      ibin_dts[1][b] = 0.5 * ibin_dts[0][b];
      ibin_dts[2][b] = 1.0 / ibin_dts[0][b];
      ibin_dts[3][b] = time + 0.5 * get_dt(p.dtmax, b);
    }
    istepfrac = 0;
    tlast = time;
  }
  // one pass of the evolve loop (evolve.f90:132-154): evol_prestep, step, evol_poststep
  int ind_substep(double &time, int64_t &nactive) {
    if (nbinmax > MAXBINS) return 42;  // a bin above maxbins: dt too small (step_leapfrog.f90:427-433)
    const int nbinmaxprev = nbinmax;
    istepfrac = istepfrac + 1;  // evolve.f90:206
    if (istepfrac > (1 << nbinmax)) return 40;
    nactive = 0;  // utils_indtimesteps.f90:114-178 set_active_particles
    for (int64_t i = 0; i < n; ++i) {
      if (xyzh[4 * i + 3] <= 0.0) { activef[i] = 0; continue; }
      if (ibin[i] > nbinmax) return 41;
      activef[i] = (istepfrac % (1 << (nbinmax - ibin[i])) == 0) ? 1 : 0;
      nactive += activef[i];
    }
    ibinnow = nbinmax;
    for (int b = 0; ibinnow == nbinmax && b < nbinmax; ++b)
      if (istepfrac % (1 << (nbinmax - b)) == 0) ibinnow = b;
    int err = ind_step(time, dtsub);
    if (err) return err;
    // evolve_utils.F90:65-91 update_time_and_dt
    time = tlast + (double)istepfrac / (double)(1 << nbinmaxprev) * p.dtmax;
    if (nbinmax != nbinmaxprev) {  // utils_indtimesteps.f90:186-223 change_nbinmax
      if (nbinmax < nbinmaxprev && istepfrac % (1 << (nbinmaxprev - nbinmax)) != 0) return 43;
      if (nbinmax > nbinmaxprev) istepfrac = istepfrac * (1 << (nbinmax - nbinmaxprev));
      else istepfrac = istepfrac / (1 << (nbinmaxprev - nbinmax));
      if (nbinmax > MAXBINS) return 44;
      dtsub = p.dtmax / std::ldexp(1.0, nbinmax);
    }
    if (istepfrac == (1 << nbinmax)) {  // end of a dtmax interval (evolve.f90:437-440)
      istepfrac = 0;
      tlast = time;
    }
    return 0;
  }
  // step_leapfrog.f90:91-760 with individual timesteps (one corrector pass)
  int ind_step(double timei, double dtsph) {
    const bool adiab = !p.isothermal;
    const int nv = adiab ? 4 : 3;
    const double time_now = timei + dtsph;
    for (int b = 0; b <= MAXBINS; ++b)  // step_leapfrog.f90:157-163
      ibin_dts[3][b] = ((double)(int64_t)(time_now * ibin_dts[2][b]) + 0.5) * ibin_dts[0][b];
    for (int64_t i = 0; i < n; ++i) {  // predictor: synchronise to the half steps
      if (xyzh[4 * i + 3] < TINY_D) continue;
      if (activef[i]) ibin_old[i] = ibin[i];
      const double hdti = twas[i] - timei;
      for (int k = 0; k < nv; ++k) vxyzu[4 * i + k] = vxyzu[4 * i + k] + hdti * fxyzu[4 * i + k];
      if (p.mhd) for (int k = 0; k < 4; ++k) Bevol[4 * i + k] = Bevol[4 * i + k] + hdti * dBevol[4 * i + k];
    }
    for (int64_t i = 0; i < n; ++i) {  // substep_sph drift (substepping.F90:241-264)
      if (xyzh[4 * i + 3] < TINY_D) continue;
      for (int k = 0; k < 3; ++k) xyzh[4 * i + k] = xyzh[4 * i + k] + dtsph * vxyzu[4 * i + k];
    }
    timei = timei + dtsph;
    vpred.assign(4 * n, 0.0);
    Bpred.assign(4 * n, 0.0);
    for (int64_t i = 0; i < n; ++i) {  // predict_sph (step_leapfrog.f90:296-398)
      if (xyzh[4 * i + 3] < TINY_D) continue;
      double h = xyzh[4 * i + 3];
      xyzh[4 * i + 3] = h - dtsph * dhdrho(h) * rhoh(h) * (double)divcurlv[(size_t)ndivcurlv() * i];
      const double hdti = timei - twas[i];
      for (int k = 0; k < nv; ++k) vpred[4 * i + k] = vxyzu[4 * i + k] + hdti * fxyzu[4 * i + k];
      if (p.mhd) for (int k = 0; k < 4; ++k) Bpred[4 * i + k] = Bevol[4 * i + k] + hdti * dBevol[4 * i + k];
      if (p.nalpha >= 2) {
        const double hi = xyzh[4 * i + 3];
        const double tdecay1 = AVDECAYCONST * eos[2 * i + 1] / hi;
        const double ddenom = 1.0 / (1.0 + dtsph * tdecay1);
        const double alphaloci = (double)alphaind[3 * i + 1];
        if ((double)alphaind[3 * i] < alphaloci) alphaind[3 * i] = (float)alphaloci;
        else alphaind[3 * i] = (float)(((double)alphaind[3 * i] + dtsph * alphaloci * tdecay1) * ddenom);
      }
    }
    dt_too_small = false;
    int err = derivs(1, dtsph, vpred, p.mhd ? Bpred : Bevol, nullptr);
    if (err) return err;
    if (dt_too_small) return 42;  // step_leapfrog.f90:427-433: fatal before the corrector
    for (int64_t i = 0; i < n; ++i) {  // corrector (step_leapfrog.f90:482-560)
      if (xyzh[4 * i + 3] < TINY_D) continue;
      if (activef[i]) {
        ibin_wake[i] = 0;
        const double hdti = timei - twas[i];
        const double dti = hdti + ibin_dts[1][ibin[i]];
        for (int k = 0; k < nv; ++k) vxyzu[4 * i + k] = vxyzu[4 * i + k] + dti * fxyzu[4 * i + k];
        if (p.mhd) for (int k = 0; k < 4; ++k) Bevol[4 * i + k] = Bevol[4 * i + k] + dti * dBevol[4 * i + k];
        twas[i] = twas[i] + dti;
      }
      const double hdti = timei - twas[i];
      for (int k = 0; k < nv; ++k) vxyzu[4 * i + k] = vxyzu[4 * i + k] + hdti * fxyzu[4 * i + k];
      if (p.mhd) for (int k = 0; k < 4; ++k) Bevol[4 * i + k] = Bevol[4 * i + k] + hdti * dBevol[4 * i + k];
      if (ibin_wake[i] > ibin[i]) {  // wake the particle for the next step
        ibin_wake[i] = (int8_t)std::min(nbinmax, (int)ibin_wake[i]);
        twas[i] = ibin_dts[3][ibin_wake[i]];
        ibin[i] = ibin_wake[i];
        ibin_wake[i] = 0;
      }
    }
    return 0;
  }

  // step_leapfrog.f90:91-760 (global timesteps) and :769-843 check_velocity_error
  int step(double t, double dtsph, double *dtnew, int *its_out) {
    (void)t;
    double hdtsph = 0.5 * dtsph;
    dterr = BIGNUMBER;
    const bool adiab = !p.isothermal;
    // predictor
    for (int64_t i = 0; i < n; ++i) {
      if (xyzh[4 * i + 3] < TINY_D) continue;
      for (int k = 0; k < (adiab ? 4 : 3); ++k) vxyzu[4 * i + k] = vxyzu[4 * i + k] + hdtsph * fxyzu[4 * i + k];
      if (p.mhd) for (int k = 0; k < 4; ++k) Bevol[4 * i + k] = Bevol[4 * i + k] + hdtsph * dBevol[4 * i + k];
    }
    // substep_sph drift substepping.F90:241-264
    for (int64_t i = 0; i < n; ++i) {
      if (xyzh[4 * i + 3] < TINY_D) continue;
      for (int k = 0; k < 3; ++k) xyzh[4 * i + k] = xyzh[4 * i + k] + dtsph * vxyzu[4 * i + k];
    }
    // predict_sph
    vpred.assign(4 * n, 0.0);
    Bpred.assign(4 * n, 0.0);
    for (int64_t i = 0; i < n; ++i) {
      if (xyzh[4 * i + 3] < TINY_D) continue;
      double h = xyzh[4 * i + 3];
      xyzh[4 * i + 3] = h - dtsph * dhdrho(h) * rhoh(h) * (double)divcurlv[(size_t)ndivcurlv() * i];
      double hdti = 0.5 * dtsph;
      for (int k = 0; k < (adiab ? 4 : 3); ++k) vpred[4 * i + k] = vxyzu[4 * i + k] + hdti * fxyzu[4 * i + k];
      if (p.mhd) for (int k = 0; k < 4; ++k) Bpred[4 * i + k] = Bevol[4 * i + k] + hdti * dBevol[4 * i + k];
      if (p.nalpha >= 2) {  // step_leapfrog.f90:378-391 viscosity switch (Cullen & Dehnen)
        const double hi = xyzh[4 * i + 3];
        const double spsoundi = eos[2 * i + 1];
        const double tdecay1 = AVDECAYCONST * spsoundi / hi;
        const double ddenom = 1.0 / (1.0 + dtsph * tdecay1);
        const double alphaloci = (double)alphaind[3 * i + 1];
        if ((double)alphaind[3 * i] < alphaloci) alphaind[3 * i] = (float)alphaloci;
        else alphaind[3 * i] = (float)(((double)alphaind[3 * i] + dtsph * alphaloci * tdecay1) * ddenom);
      }
    }
    int err = derivs(1, dtsph, vpred, p.mhd ? Bpred : Bevol, dtnew);
    if (err) return err;
    const int maxits = 30;
    int its = 0;
    bool converged = false;
    double errmaxmean = 0.0;
    while (its < maxits && !converged) {
      ++its;
      double errmax = 0.0, v2mean = 0.0;
      int64_t np = 0;
      for (int64_t i = 0; i < n; ++i) {
        if (xyzh[4 * i + 3] < TINY_D) continue;
        double *v = &vxyzu[4 * i];
        const double *f = &fxyzu[4 * i];
        double vxi = v[0] + hdtsph * f[0], vyi = v[1] + hdtsph * f[1], vzi = v[2] + hdtsph * f[2];
        double eni = adiab ? v[3] + hdtsph * f[3] : 0.0;
        double erri = sq(vxi - vpred[4 * i]) + sq(vyi - vpred[4 * i + 1]) + sq(vzi - vpred[4 * i + 2]);
        errmax = fmax_f(errmax, erri);
        double v2i = vxi * vxi + vyi * vyi + vzi * vzi;
        v2mean = v2mean + v2i;
        ++np;
        v[0] = vxi; v[1] = vyi; v[2] = vzi;
        if (adiab) v[3] = eni;
        if (p.mhd) for (int k = 0; k < 4; ++k) Bevol[4 * i + k] = Bevol[4 * i + k] + hdtsph * dBevol[4 * i + k];
      }
      // check_velocity_error
      v2mean = (np > 0) ? v2mean / (double)np : 0.0;
      errmax = (v2mean > TINY_D) ? errmax / std::sqrt(v2mean) : 0.0;
      errmaxmean = errmaxmean + errmax;
      double errtol = p.tolv;
      dterr = HUGE_D;
      if (p.tolv < 1.e2) {
        double dtf = fmin_f(dtcourant, dtforce);
        if (dtf > dtsph && dtf < BIGNUMBER) errtol = errtol * sq(dtsph / dtf);
        if (its == 1) {
          if (errtol > TINY_D && errmax > EPS_D) dterr = dtsph * std::sqrt(errtol / errmax);
        }
        converged = (errmax < p.tolv);
      } else {
        converged = true;
      }
      if (!converged) {
        for (int64_t i = 0; i < n; ++i) {
          for (int k = 0; k < 4; ++k) vpred[4 * i + k] = vxyzu[4 * i + k];
          if (p.mhd) for (int k = 0; k < 4; ++k) Bpred[4 * i + k] = Bevol[4 * i + k];
          for (int k = 0; k < (adiab ? 4 : 3); ++k) vxyzu[4 * i + k] = vxyzu[4 * i + k] - hdtsph * fxyzu[4 * i + k];
          if (p.mhd) for (int k = 0; k < 4; ++k) Bevol[4 * i + k] = Bevol[4 * i + k] - hdtsph * dBevol[4 * i + k];
        }
        err = derivs(2, dtsph, vpred, p.mhd ? Bpred : Bevol, dtnew);
        if (err) return err;
      }
    }
    if (its_out) *its_out = its;
    if (its >= maxits) return 40;
    return 0;
  }
};

}  // namespace

extern "C" {

void *ora_create(const ora_params *p) {
  if (p->minpart != 0 && (p->minpart < 2 || p->minpart > MAXLEAF)) return nullptr;
  Oracle *o = new Oracle();
  o->set_params(p);
  return o;
}
void ora_destroy(void *o) { delete static_cast<Oracle *>(o); }
int ora_set_params(void *o, const ora_params *p) {
  if (p->minpart != 0 && (p->minpart < 2 || p->minpart > MAXLEAF)) return 1;
  static_cast<Oracle *>(o)->set_params(p);
  return 0;
}

int ora_set_particles(void *vo, int64_t n, const double *xyzh, const double *vxyzu, const double *Bevol) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (n <= 0 || n > o->p.maxp) return 1;
  o->n = n;
  o->xyzh.assign(xyzh, xyzh + 4 * n);
  o->vxyzu.assign(vxyzu, vxyzu + 4 * n);
  if (Bevol) o->Bevol.assign(Bevol, Bevol + 4 * n); else o->Bevol.assign(4 * n, 0.0);
  o->fxyzu.assign(4 * n, 0.0);
  o->dBevol.assign(4 * n, 0.0);
  o->gradh.assign(2 * n, 0.0f);
  o->gradh_d.assign(2 * n, 0.0);
  o->divcurlv.assign((size_t)o->ndivcurlv() * n, 0.0f);
  o->divcurlB.assign(4 * n, 0.0f);
  o->divBsymm.assign(n, 0.0f);
  o->poten.assign(n, 0.0f);
  o->eos.assign(2 * n, 0.0);
  o->alphaind.assign(3 * n, 0.0f);  // part.F90:688
  o->dvdx.assign(9 * n, 0.0f);
  o->ibin.assign(n, 0); o->ibin_old.assign(n, 0); o->ibin_wake.assign(n, 0);  // initial.F90:160-165
  o->activef.assign(n, 1); o->twas.assign(n, 0.0);
  o->nbinmax = 0; o->istepfrac = 0; o->ibinnow = 0;
  o->have_tree = false;
  return 0;
}
int ora_get_particles(void *vo, double *xyzh, double *vxyzu, double *Bevol) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (xyzh) std::memcpy(xyzh, o->xyzh.data(), sizeof(double) * 4 * o->n);
  if (vxyzu) std::memcpy(vxyzu, o->vxyzu.data(), sizeof(double) * 4 * o->n);
  if (Bevol) std::memcpy(Bevol, o->Bevol.data(), sizeof(double) * 4 * o->n);
  return 0;
}
int ora_maketree(void *vo) { return static_cast<Oracle *>(vo)->maketree(); }
int ora_set_alpha(void *vo, const float *alpha) {
  Oracle *o = static_cast<Oracle *>(vo);
  for (int64_t i = 0; i < o->n; ++i) o->alphaind[3 * i] = alpha[i];
  return 0;
}
int ora_get_alpha(void *vo, float *alphaind, float *dvdx) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (alphaind) std::memcpy(alphaind, o->alphaind.data(), sizeof(float) * 3 * o->n);
  if (dvdx) std::memcpy(dvdx, o->dvdx.data(), sizeof(float) * 9 * o->n);
  return 0;
}
int ora_alpha_initial(void *vo) {  // initial.F90:736-742
  Oracle *o = static_cast<Oracle *>(vo);
  if (o->p.nalpha < 2) return 0;
  for (int64_t i = 0; i < o->n; ++i) o->alphaind[3 * i] = std::max(o->alphaind[3 * i], o->alphaind[3 * i + 1]);
  return 0;
}
int ora_ind_init(void *vo, double time) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (!o->p.ind_timesteps) return 1;
  o->ind_init(time);
  return 0;
}
int ora_ind_substep(void *vo, double *time, int64_t *nactive) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (!o->p.ind_timesteps) return 1;
  return o->ind_substep(*time, *nactive);
}
int ora_ind_state(void *vo, int8_t *ibin, double *twas, int32_t *counters) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (ibin) std::memcpy(ibin, o->ibin.data(), (size_t)o->n);
  if (twas) std::memcpy(twas, o->twas.data(), sizeof(double) * o->n);
  if (counters) { counters[0] = o->nbinmax; counters[1] = o->istepfrac; counters[2] = o->ibinnow; counters[3] = 0; }
  return 0;
}
// revtree on new positions xyzh(4,n) of the same particles (caller order)
int ora_revtree(void *vo, const double *xyzh) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (!o->have_tree) return 1;
  std::memcpy(o->xyzh.data(), xyzh, sizeof(double) * 4 * o->n);
  return o->revtree();
}
int64_t ora_get_ncells(void *vo) { return static_cast<Oracle *>(vo)->ncells; }
int ora_get_tree(void *vo, int32_t *inodeparts, int32_t *inoderange, double *xcen, double *size,
                 double *hmax, double *mass, int32_t *left, int32_t *right, int32_t *parent,
                 int32_t *leaf_is_active, double *quads) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (inodeparts) for (int64_t k = 0; k < o->n; ++k) inodeparts[k] = o->inodeparts[k + 1];
  for (int64_t c = 1; c <= o->ncells; ++c) {
    int64_t r = c - 1;
    const Node &nd = o->node[c];
    if (inoderange) { inoderange[2 * r] = o->inoderange[2 * c]; inoderange[2 * r + 1] = o->inoderange[2 * c + 1]; }
    if (xcen) for (int k = 0; k < 3; ++k) xcen[3 * r + k] = nd.xcen[k];
    if (size) size[r] = nd.size;
    if (hmax) hmax[r] = nd.hmax;
    if (mass) mass[r] = nd.mass;
    if (left) left[r] = nd.left;
    if (right) right[r] = nd.right;
    if (parent) parent[r] = nd.parent;
    if (leaf_is_active) leaf_is_active[r] = o->leaf_is_active[c];
    if (quads) for (int k = 0; k < 6; ++k) quads[6 * r + k] = nd.quads[k];
  }
  return 0;
}
int ora_densityiterate(void *vo, int icall) { return static_cast<Oracle *>(vo)->densityiterate(icall); }
int ora_get_density(void *vo, float *gradh, float *divcurlv, float *divcurlB, int32_t *nneigh,
                    uint64_t *neighhash, ora_stats *st) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (gradh) std::memcpy(gradh, o->gradh.data(), sizeof(float) * 2 * o->n);
  if (divcurlv) std::memcpy(divcurlv, o->divcurlv.data(), sizeof(float) * o->ndivcurlv() * o->n);
  if (divcurlB) std::memcpy(divcurlB, o->divcurlB.data(), sizeof(float) * 4 * o->n);
  if (nneigh && !o->nneigh_out.empty()) std::memcpy(nneigh, o->nneigh_out.data(), sizeof(int32_t) * o->n);
  if (neighhash && !o->nhash_out.empty()) std::memcpy(neighhash, o->nhash_out.data(), sizeof(uint64_t) * o->n);
  if (st) *st = o->stats;
  return 0;
}
int ora_cons2prim(void *vo) {
  Oracle *o = static_cast<Oracle *>(vo);
  o->cons2prim(o->vxyzu);
  return 0;
}
int ora_force(void *vo, int icall, double dt) {
  Oracle *o = static_cast<Oracle *>(vo);
  return o->force(icall, dt, o->vxyzu, o->Bevol);
}
int ora_get_force(void *vo, double *fxyzu, double *dBevol, float *divcurlv, float *divBsymm, float *poten,
                  double *eos, double *dtcourant, double *dtforce) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (fxyzu) std::memcpy(fxyzu, o->fxyzu.data(), sizeof(double) * 4 * o->n);
  if (dBevol) std::memcpy(dBevol, o->dBevol.data(), sizeof(double) * 4 * o->n);
  if (divcurlv) std::memcpy(divcurlv, o->divcurlv.data(), sizeof(float) * o->ndivcurlv() * o->n);
  if (divBsymm) std::memcpy(divBsymm, o->divBsymm.data(), sizeof(float) * o->n);
  if (poten) std::memcpy(poten, o->poten.data(), sizeof(float) * o->n);
  if (eos) std::memcpy(eos, o->eos.data(), sizeof(double) * 2 * o->n);
  if (dtcourant) *dtcourant = o->dtcourant;
  if (dtforce) *dtforce = o->dtforce;
  return 0;
}
int ora_derivs(void *vo, int icall, double dt, double *dtnew) {
  Oracle *o = static_cast<Oracle *>(vo);
  return o->derivs(icall, dt, o->vxyzu, o->Bevol, dtnew);
}
int ora_step(void *vo, double t, double dtsph, double *dtnew, int32_t *its_out) {
  int its = 0;
  int r = static_cast<Oracle *>(vo)->step(t, dtsph, dtnew, &its);
  if (its_out) *its_out = its;
  return r;
}
double ora_get_dterr(void *vo) { return static_cast<Oracle *>(vo)->dterr; }

int ora_bruteforce_count(void *vo, int64_t i, int32_t *count) {
  Oracle *o = static_cast<Oracle *>(vo);
  if (i < 0 || i >= o->n) return 1;
  const double *xi = &o->xyzh[4 * i];
  double hi1 = 1.0 / xi[3], hi21 = hi1 * hi1;
  int c = 1;
  for (int64_t j = 0; j < o->n; ++j) {
    if (j == i) continue;
    double dx = xi[0] - o->xyzh[4 * j], dy = xi[1] - o->xyzh[4 * j + 1], dz = xi[2] - o->xyzh[4 * j + 2];
    if (o->p.periodic) {
      if (std::fabs(dx) > 0.5 * o->dxbound) dx = dx - o->dxbound * fsign1(dx);
      if (std::fabs(dy) > 0.5 * o->dybound) dy = dy - o->dybound * fsign1(dy);
      if (std::fabs(dz) > 0.5 * o->dzbound) dz = dz - o->dzbound * fsign1(dz);
    }
    double q2 = (dx * dx + dy * dy + dz * dz) * hi21;
    if (q2 < RADKERN2) ++c;
  }
  *count = c;
  return 0;
}

void ora_m2l(double dx, double dy, double dz, double dr1, double mass, const double *quads, double *fnode) {
  Oracle::compute_M2L(dx, dy, dz, dr1, mass, quads, fnode);
}
void ora_taylor(const double *fnode, double dx, double dy, double dz, double *f3, double *phi) {
  double fx, fy, fz, p;
  Oracle::expand_taylor(fnode, dx, dy, dz, fx, fy, fz, p);
  f3[0] = fx; f3[1] = fy; f3[2] = fz;
  *phi = p;
}
void ora_kernel(double q2, double q, double *w, double *gr, double *dphidh, double *potsoft, double *fsoft) {
  double ww, gg, dd, ps, fs;
  get_kernel_grav1(q2, q, ww, gg, dd);
  kernel_softening(q2, q, ps, fs);
  if (w) *w = ww;
  if (gr) *gr = gg;
  if (dphidh) *dphidh = dd;
  if (potsoft) *potsoft = ps;
  if (fsoft) *fsoft = fs;
}

}  // extern "C"
