// Shared device definitions of the phantom_gb300 CUDA path (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "phantom_gb300.h"

namespace ph {

// ------------------------------------------------------------ constants
// physcon.f90:23 (pi as the reference defines it) and kernel_cubic.f90:23-30
constexpr double PI_PHANTOM = 3.1415926536;
constexpr double CNORMK = 1.0 / PI_PHANTOM;
constexpr double RADKERN2 = 4.0;
constexpr double RADKERN = 2.0;
constexpr double DPHIDH0 = 1.4;
constexpr int MINPART = 10;          // config.F90:113 (the default leaf size; ph_params.minpart)
constexpr int CELLCACHE = 1000;      // dens.F90:99, force.F90:58: first 1000 trial entries use cached positions
constexpr int MAXDENSITS = 100;      // dens.F90:101
constexpr double AVDECAYCONST = 0.1; // shock_capturing.f90:32
constexpr int MAXBINS = 30;          // utils_indtimesteps.f90 maxbins
constexpr double BIGNUMBER = 1.e29;  // timestep.f90:40
constexpr double EPS_D = 2.220446049250313e-16;
constexpr double TINY_D = 2.2250738585072014e-308;
constexpr float TINY_F = 1.17549435e-38f;  // tiny() of the FP32 kind
constexpr double HUGE_D = 1.7976931348623157e308;
constexpr int MAXCELL = 16;          // leaf cells hold <= minpart <= MAXCELL particles
constexpr int MINPART_LO = 2;        // smallest leaf size accepted
// warps (one leaf cell each) per block of the pair kernels are set per
// context at run time (ph_autotune), at most MAX_WARPS (their launch bound)
constexpr int MAX_WARPS = 4;

// Device view of ph_params (passed by value to kernels).
struct Params {
  int periodic, mhd, gravity, isothermal, ieos;
  int ipdv_heating, ishock_heating, iresistive_heating, precision;
  int minpart;  // leaf size: a node of more than minpart particles is split (kdtree.F90:792)
  int nalpha;   // 0: constant alpha (CONST_AV); 3: Cullen & Dehnen switch
  int curlv;    // divcurlv with curl v (ndivcurlv = 4)
  int ind;      // individual timesteps
  double alphamax;
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double dxbound, dybound, dzbound, hdlx, hdly, hdlz;
  double hfact, tolh, massoftype;
  double alpha, alphau, alphaB, beta;
  double gamma, polyk;
  double C_cour, C_force, tolv, dtmax;
  double psidecayfac, overcleanfac;
  double tree_accuracy;
  float dxboundf, dyboundf, dzboundf;
};

inline Params make_params(const ph_params &p) {
  Params d{};
  d.periodic = p.periodic; d.mhd = p.mhd; d.gravity = p.gravity; d.isothermal = p.isothermal;
  d.ieos = p.ieos; d.ipdv_heating = p.ipdv_heating; d.ishock_heating = p.ishock_heating;
  d.iresistive_heating = p.iresistive_heating; d.precision = p.precision;
  d.minpart = p.minpart > 0 ? p.minpart : MINPART;
  d.nalpha = p.nalpha;
  d.curlv = p.curlv;
  d.ind = p.ind_timesteps;
  d.alphamax = p.alphamax > 0.0 ? p.alphamax : 1.0;  // shock_capturing.f90:55
  d.xmin = p.xmin; d.xmax = p.xmax; d.ymin = p.ymin; d.ymax = p.ymax; d.zmin = p.zmin; d.zmax = p.zmax;
  d.dxbound = p.xmax - p.xmin; d.dybound = p.ymax - p.ymin; d.dzbound = p.zmax - p.zmin;  // boundary.f90:105
  d.hdlx = 0.5 * d.dxbound; d.hdly = 0.5 * d.dybound; d.hdlz = 0.5 * d.dzbound;        // boundary.f90:109
  d.hfact = p.hfact; d.tolh = p.tolh; d.massoftype = p.massoftype;
  d.alpha = p.alpha; d.alphau = p.alphau; d.alphaB = p.alphaB; d.beta = p.beta;
  d.gamma = p.gamma; d.polyk = p.polyk;
  d.C_cour = p.C_cour; d.C_force = p.C_force; d.tolv = p.tolv; d.dtmax = p.dtmax;
  d.psidecayfac = p.psidecayfac; d.overcleanfac = p.overcleanfac; d.tree_accuracy = p.tree_accuracy;
  d.dxboundf = (float)d.dxbound; d.dyboundf = (float)d.dybound; d.dzboundf = (float)d.dzbound;
  return d;
}

// kd-tree node, 64 bytes (the path's subset of kdnode, dtype_kdtree.F90:53-68)
struct __align__(16) Node {
  double x, y, z, size;
  double hmax;
  int left, right;   // node ids, -1 = none
  int start, count;  // particle range in tree order
  int parent, level;
};

// FP32 mirror of a node for the walks' node tests (32 bytes): leaves keep
// left = -1, right = first particle, count = particles; internal nodes their
// children in left/right
struct __align__(16) NodeF {
  float x, y, z, size, hmax;
  int left, right, count;
};
__device__ __forceinline__ NodeF make_nodef(const Node &n) {
  NodeF f;
  f.x = (float)n.x; f.y = (float)n.y; f.z = (float)n.z; f.size = (float)n.size; f.hmax = (float)n.hmax;
  f.left = n.left;
  f.right = n.left < 0 ? n.start : n.right;
  f.count = n.count;
  return f;
}

// ------------------------------------------------------------ error word
__device__ __forceinline__ void set_error(int *err, int code) { atomicCAS(err, 0, code); }

// ------------------------------------------------------------ exact FP64 helpers
// Neighbour decisions are evaluated without FMA contraction so that they round
// exactly like the reference (gfortran on x86-64 has no FMA).
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double r2_exact(double dx, double dy, double dz) {
  return dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
}
__device__ __forceinline__ double sign1(double x) { return signbit(x) ? -1.0 : 1.0; }
// periodic wrap of a separation (dens.F90:667-669, force.F90:1267-1269);
// hL = 0.5 L, exact in FP64 and computed once per context
__device__ __forceinline__ double wrap(double d, double L, double hL, bool periodic) {
  if (periodic && fabs(d) > hL) d = dsub(d, dmul(L, sign1(d)));
  return d;
}

// Exact-rounding FP64 restatements of scalar formulae (no contraction).
// rhoh: part.F90:779-785  rho = m (hfact/|h|)^3
__device__ __forceinline__ double rhoh(double h, double m, double hfact) {
  double t = ddiv(hfact, fabs(h));
  return dmul(m, dmul(dmul(t, t), t));
}
// dhdrho: part.F90:791-799
__device__ __forceinline__ double dhdrho(double h, double m, double hfact) {
  double r = rhoh(h, m, hfact);
  return ddiv(-h, dmul(3.0, r));
}
// hrho: part.F90:845-850
__device__ __forceinline__ double hrho(double rho, double m, double hfact) {
  return dmul(hfact, pow(ddiv(m, fabs(rho)), 1.0 / 3.0));
}

// order-preserving int64 key of a double (non-NaN; -0.0 and +0.0 share the
// key of +0.0): min, max and <= on keys agree with the FP64 comparisons, and
// cost integer instructions instead of FP64-pipe ones
__device__ __forceinline__ long long dkey(double v) {
  long long b = __double_as_longlong(v);
  if (b == (long long)0x8000000000000000ull) b = 0;
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
__device__ __forceinline__ double dunkey(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll));
}
constexpr long long KEY_LO = (long long)0x8000000000000000ull;  // below every key
constexpr long long KEY_HI = 0x7fffffffffffffffll;              // above every key

// double -> float rounded to nearest (ties to even), assembled from the
// IEEE-754 fields with integer instructions: the conversion instruction runs
// on the FP64 pipe, which is the scarce unit here. Results below the float
// normal range flush to signed zero; |x| must stay below 2^127 (pair
// separations and positions do).
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 896;  // biased float exponent
  unsigned fb = sign | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rem = lo & 0x1fffffffu;
  fb += (rem > 0x10000000u || (rem == 0x10000000u && (fb & 1u))) ? 1u : 0u;
  return __uint_as_float(e > 0 ? fb : sign);
}

// ------------------------------------------------------------ warp helpers
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int warp_sum_int(int v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// atomic max of a non-negative double (bit order == numeric order)
__device__ __forceinline__ void atomic_max_pos(double *addr, double v) {
  atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_min_pos(double *addr, double v) {
  atomicMin(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

// neighbour-set hash term (order independent sum of mixed ids)
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// leaf entry of a trial list: contiguous particle range + periodic offset code
struct LeafEntry {
  int start;
  int cc;  // count | (offset code << 8); code: 2 bits per axis (0: 0, 1: +L, 2: -L)
};
__device__ __forceinline__ double offset_of(int code, int axis, double L) {
  int c = (code >> (2 * axis)) & 3;
  return c == 0 ? 0.0 : (c == 1 ? L : -L);
}

__device__ __forceinline__ float offset_of_f(int code, int axis, float L) {
  int c = (code >> (2 * axis)) & 3;
  return c == 0 ? 0.0f : (c == 1 ? L : -L);
}

// 1/sqrt(x) in FP32: the hardware estimate refined by one Newton step on the
// residual e = 1 - x y^2 (y' = y + y e / 2), which removes the estimate's
// few-ulp bias; gravity sums over thousands of pairs cancel to a small net
// force and would otherwise keep that bias
__device__ __forceinline__ float rsqrt_nr(float x) {
  const float y = rsqrtf(x);
  const float e = fmaf(-x * y, y, 1.0f);
  return fmaf(0.5f * y, e, y);
}

// compensated (Kahan) FP32 accumulator; value() returns the corrected sum in FP64
struct Kahan {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

}  // namespace ph
