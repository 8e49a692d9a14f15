// Adjoint of density + force (differentiation form): gradients of
//   L = sum_i sum_k w(k,i) fxyzu(k,i)
// (accelerations and du/dt of one derivs evaluation, force.F90:914-3330 on
// the density solve of dens.F90:117-1681) with respect to the positions,
// velocities and thermal energies, for hydrodynamics (adiabatic or
// isothermal equation of state, artificial viscosity and conductivity, the
// viscosity parameter constant or per particle (Cullen & Dehnen switch:
// alphaind(1) is an input of one derivs, held fixed) and, for the
// accelerations, ideal MHD (magnetic pressure and
// anisotropic stress, the signal speed sqrt(c_s^2 + v_A^2) in the viscosity,
// the div B subtraction force.F90:2873-2890), also with respect to B/rho,
// and self-gravity: the softened near field of the trial pairs with its
// gradsoft term (force.F90:1303-1340) and the plain 1/r^2 pairs outside both
// kernels (force.F90:1991-2053), gradsoft = dh/drho h^-2 sum_j m dphi/dh
// (dens.F90, get_kernel_grav1) differentiated through the h-rho solve like
// 1/Omega, and the far field (kdtree.F90:1702-1840; its reverse is in the
// gravity source).
//
// Model differentiated: the converged h-rho solve, i.e. h_i the root of
// rho(h_i) = sum_j m W(r_ij, h_i), with Omega_i = 1 - (dh/drho)_i dRho_i/dh
// (gradh = 1/Omega) kept in FP64 (the reference stores it in float32; its
// rounding has no derivative). Implicit differentiation gives
//   dh_i/dx = (dh/drho)_i / Omega_i * d rho_i/dx  at fixed h_i.
//
// Work decomposition (nothing is stored between the forward and the adjoint
// beyond per-particle values; pair terms are recomputed):
//  1. k_adj_pairs: one warp per leaf cell over the force trial lists. Every
//     unordered pair {i,j} contributes c_ij + c_ji to L (c_ab: what a receives
//     from b, weighted by a's cotangents). Particle i evaluates the reverse
//     of both terms and keeps the derivatives with respect to its own
//     variables (explicit x_i, v_i and the per-particle primitives h, 1/Omega,
//     1/rho, P/rho^2, c_s, P, rho, u), so every pair is gathered on both sides
//     without atomics. It also sums d^2 rho_i/dh^2.
//  2. k_adj_coef: per particle, the chain rule to h and u and the coefficients
//     A_i (on d rho_i/dx) and B_i (on d(d rho_i/dh)/dx) of the implicit solve.
//  3. k_adj_dens: one warp per leaf cell, the gather of
//     m [A_k dW(r,h_k)/dr + B_k d2W(r,h_k)/dhdr + A_j dW(r,h_j)/dr + B_j d2W(r,h_j)/dhdr] r_kj/r
//     (with self-gravity also C_k dphi_h(r,h_k)/dr + C_j dphi_h(r,h_j)/dr,
//     C the coefficient on the gradsoft sum).
//  4. With self-gravity, the far field's reverse (gravity_adjoint_far).
#include "ph_internal.h"
#include "ph_walk.cuh"

namespace ph {

constexpr int ADJ_WARPS = 4;
constexpr int NADJ = 24;  // pass-1 accumulators per particle

// adjoint record slots (tree order, ADJREC doubles per particle)
// (AR_CS holds the signal speed v_wave the viscosity uses: c_s, or
// sqrt(c_s^2 + v_A^2) with MHD; AR_CS0 the sound speed)
enum {
  AR_H = 0, AR_H1, AR_G, AR_RHO, AR_RHO1, AR_PRO2, AR_CS, AR_P, AR_U, AR_VX, AR_VY, AR_VZ,
  AR_WX, AR_WY, AR_WZ, AR_S, AR_A, AR_B, AR_GX, AR_GY, AR_GZ, AR_GVX, AR_GVY, AR_GVZ, AR_GU,
  AR_BX, AR_BY, AR_BZ, AR_KAP, AR_CS0, AR_GBX, AR_GBY, AR_GBZ, AR_ALPHA, AR_GS, AR_C,
  // MHD: psi, the cotangents of d(B/rho)/dt (OX..OZ) and dpsi/dt (ZETA), the
  // weights of the div B diffusion and drho/dt sums in dpsi/dt, and psi's
  // gradient
  AR_PSI, AR_OX, AR_OY, AR_OZ, AR_ZETA, AR_K11, AR_K4, AR_GPSI, AR_NSLOTS
};
static_assert(AR_NSLOTS <= ADJREC, "adjoint record slots");
// pass-1 accumulator slots (psum)
// (PA_GS: cotangent of gradsoft; PA_SG: sum m q dphi_h/dq over the kernel;
// PA_PSI: cotangent of psi; PA_FS4, PA_FS11: the forward drho/dt and div B
// diffusion sums of the receiver)
enum { PA_X = 0, PA_Y, PA_Z, PA_VX, PA_VY, PA_VZ, PA_H, PA_G, PA_RHO1, PA_PRO2, PA_CS, PA_P, PA_RHO, PA_U, PA_D2,
       PA_BX, PA_BY, PA_BZ, PA_DIVB, PA_GS, PA_SG, PA_PSI, PA_FS4, PA_FS11, PA_NSLOTS };
static_assert(PA_NSLOTS == NADJ && NADJ <= PSUM, "pass-1 slots");
static_assert(32 * NADJ * sizeof(double) <= sizeof(PairSmem), "pass-1 lane sums staged in the pair smem");

// per-lane accumulator of the adjoint pair sums: FP64 sums for the plain
// form, FP32 compensated (Kahan) sums for the precision form
template <typename T>
struct Acc;
template <>
struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void operator+=(double x) { s += x; }
  __device__ __forceinline__ void operator-=(double x) { s -= x; }
  __device__ __forceinline__ double value() const { return s; }
};
template <>
struct Acc<float> {
  Kahan k;
  __device__ __forceinline__ void operator+=(float x) { k.add(x); }
  __device__ __forceinline__ void operator-=(float x) { k.add(-x); }
  __device__ __forceinline__ double value() const { return k.value(); }
};

// M4 kernel shape w(q) (cnormk h^-3 separate) and its first two derivatives
template <typename T>
__device__ __forceinline__ void wshape(T q, T &w, T &w1, T &w2) {
  if (q < T(1.0)) {
    w = T(1.0) - T(1.5) * q * q + T(0.75) * q * q * q;
    w1 = q * (T(2.25) * q - T(3.0));
    w2 = T(4.5) * q - T(3.0);
  } else if (q < T(2.0)) {
    const T t = T(2.0) - q;
    w = T(0.25) * t * t * t;
    w1 = -T(0.75) * t * t;
    w2 = T(1.5) * t;
  } else {
    w = w1 = w2 = T(0.0);
  }
}

// kernel_softening's force term fsoft(q) (kernel_cubic.f90:101-120) and
// its derivative: q (15 q^3 - 36 q^2 + 40) / 30 inside q < 1,
// (-5 q^6 + 36 q^5 - 90 q^4 + 80 q^3 - 2) / (30 q^2) for 1 <= q < 2, 1/q^2
// outside
template <typename T>
__device__ __forceinline__ void softening(T q, T &fs, T &dfs) {
  if (q < T(1.0)) {
    const T q2 = q * q;
    fs = q * (T(0.5) * q2 * q - T(1.2) * q2 + T(4.0 / 3.0));
    dfs = T(2.0) * q2 * q - T(3.6) * q2 + T(4.0 / 3.0);
  } else if (q < T(2.0)) {
    const T q2 = q * q, q1 = T(1.0) / q;
    fs = q * (-T(1.0 / 6.0) * q2 * q + T(1.2) * q2 - T(3.0) * q + T(8.0 / 3.0)) - T(1.0 / 15.0) * q1 * q1;
    dfs = -T(2.0 / 3.0) * q2 * q + T(3.6) * q2 - T(6.0) * q + T(8.0 / 3.0) + T(2.0 / 15.0) * q1 * q1 * q1;
  } else {
    const T q1 = T(1.0) / q;
    fs = q1 * q1;
    dfs = -T(2.0) * q1 * q1 * q1;
  }
}

// d/dq of get_kernel_grav1's dphidh (kernel_cubic.f90:78-99):
// -3 q^4 + 6 q^3 - 4 q inside q < 1, q (q - 2)^3 for 1 <= q < 2
template <typename T>
__device__ __forceinline__ T dphidh_dq(T q) {
  if (q < T(1.0)) return q * (q * q * (T(6.0) - T(3.0) * q) - T(4.0));
  if (q < T(2.0)) { const T t = q - T(2.0); return q * t * t * t; }
  return T(0.0);
}

template <typename T>
struct AdjConst {
  T m, alpha, beta, alphau, cn;
  T alphaB, oc;  // artificial resistivity, overcleaning factor (MHD)
  bool adiab, pdv, shock, mhd, grav;
  bool induct;   // MHD: the dB/dt and dpsi/dt terms carry cotangents (or resistive heating is on)
  bool resist;   // resistive heating in du/dt (eos.f90:1898, adiabatic)
};

template <typename T>
struct Side {
  T h1, G, rho1, pro2, cs, P, rho, u, alpha;  // alpha: alphaind(1) (force.F90:1478, 2430-2433)
  T bx, by, bz;  // B/rho (MHD)
  T psi;         // Bevol(4) (MHD)
  T gs;          // gradsoft (self-gravity)
};

// 1/r of a pair, 0 for coincident particles as the forward (force.F90:1293-
// 1298): their terms have no direction and contribute no cotangents
template <typename T>
__device__ __forceinline__ T inv_sep(T r2, T r) {
  return r2 > (sizeof(T) == 8 ? T(TINY_D) : T(TINY_F)) ? T(1.0) / r : T(0.0);
}

// a receiver's cotangents: w of its acceleration, s of du/dt, kap of its div
// B sum (the div B subtraction), o of d(B/rho)/dt, k11 and k4 of its div B
// diffusion and drho/dt sums (through dpsi/dt)
template <typename T>
struct Wt {
  T wx, wy, wz, s, kap, ox, oy, oz, k11, k4;
};

// cotangents of one side's variables (divB, fs4, fs11: the forward div B,
// drho/dt and div B diffusion sums of a receiver, accumulated alongside)
template <typename T>
struct Bar {
  Acc<T> h, G, rho1, pro2, cs, P, rho, u, vx, vy, vz, bx, by, bz, divB, gs, psi, fs4, fs11;
};

// Reverse of the ordered pair term c = w . da_a + s . du_a + kap . divB_a
// (what receiver a gets from sender b, force.F90:1428-1990), d = x_a - x_b,
// dv = v_a - v_b. With MHD, da_a also holds the anisotropic stress
// -(S_a n gk_a + S_b n gk_b), S = -m (B/rho)(B/rho)^T, and divB_a gets
// m (gk_a (B_a/rho_a).n / rho_a ... ) as divBsymm (force.F90:1800-1830);
// kap is the receiver's cotangent of its divB sum (from the div B
// subtraction in the finish); c also holds o . d(B_a/rho_a)/dt, the div B
// diffusion and drho/dt sums weighted by k11 and k4, and the resistive
// heating. Accumulates the cotangents of side a (KEEP_A) or side b into g,
// or with BOTH those of a into g and those of b into *gb, and returns dc/dd
// in (gdx, gdy, gdz).
template <typename T, bool KEEP_A, bool IND, bool BOTH = false>
__device__ __forceinline__ void pair_rev(const AdjConst<T> &k, T dx, T dy, T dz, T dvx, T dvy,
                                         T dvz, const Side<T> &a, const Side<T> &b, const Wt<T> &wt,
                                         Bar<T> &g, T &gdx, T &gdy, T &gdz, Bar<T> *gb = nullptr) {
  const T wx = wt.wx, wy = wt.wy, wz = wt.wz, s = wt.s, kap = wt.kap;
  const T r2 = dx * dx + dy * dy + dz * dz;
  const T r = sqrt(r2), rinv = inv_sep(r2, r);
  const T nx = dx * rinv, ny = dy * rinv, nz = dz * rinv;
  const T qa = r * a.h1, qb = r * b.h1;
  T wa, wpa, wppa, wb, wpb, wppb;
  wshape(qa, wa, wpa, wppa);
  wshape(qb, wb, wpb, wppb);
  const T hfa = k.cn * (a.h1 * a.h1) * (a.h1 * a.h1), hfb = k.cn * (b.h1 * b.h1) * (b.h1 * b.h1);
  const T gka = wpa * hfa * a.G, gkb = wpb * hfb * b.G;
  const T pv = dvx * nx + dvy * ny + dvz * nz;
  const T vsa_raw = a.alpha * a.cs - k.beta * pv, vsb_raw = b.alpha * b.cs - k.beta * pv;
  const T vsa = fmax(vsa_raw, T(0.0)), vsb = fmax(vsb_raw, T(0.0));
  const bool neg = pv < T(0.0);
  const T q2a = neg ? -T(0.5) * a.rho1 * vsa * pv : T(0.0), q2b = neg ? -T(0.5) * b.rho1 * vsb * pv : T(0.0);
  const T gpa = k.m * (a.pro2 + q2a) * gka, gpb = k.m * (b.pro2 + q2b) * gkb;
  // self-gravity: fg = m/2 (fg_a + fg_b), fg_a = fsoft(q_a)/h_a^2 + gradsoft_a gk_a
  // inside a's kernel, 1/r^2 outside (force.F90:1303-1340, 1991-2053)
  T fsa = T(0.0), dfsa = T(0.0), fsb = T(0.0), dfsb = T(0.0), fg = T(0.0);
  if (k.grav) {
    softening(qa, fsa, dfsa);
    softening(qb, fsb, dfsb);
    const T fga = qa < T(2.0) ? fsa * a.h1 * a.h1 + a.gs * gka : rinv * rinv;
    const T fgb = qb < T(2.0) ? fsb * b.h1 * b.h1 + b.gs * gkb : rinv * rinv;
    fg = T(0.5) * k.m * (fga + fgb);
  }
  // da_a = -n (gpa + gpb + fg)
  const T wn = wx * nx + wy * ny + wz * nz;
  const T gpt = k.grav ? (gpa + gpb) + fg : gpa + gpb;
  T nbx = -gpt * wx, nby = -gpt * wy, nbz = -gpt * wz;
  const T gp_bar = -wn;
  T gka_b = T(0.0), gkb_b = T(0.0), pv_b = T(0.0), q2a_b = T(0.0), q2b_b = T(0.0);
  T pro2a_b = T(0.0), pro2b_b = T(0.0), rho1a_b = T(0.0), rho1b_b = T(0.0), csa_b = T(0.0), csb_b = T(0.0);
  T Pa_b = T(0.0), Pb_b = T(0.0), rhoa_b = T(0.0), rhob_b = T(0.0), ua_b = T(0.0), ub_b = T(0.0);
  if (k.adiab && s != T(0.0)) {
    // du_a = [pdv] m P_a/rho_a^2 (pv gka) + [shock] m q2a pv gka + vsigu (u_a - u_b)(au_a gka + au_b gkb);
    // the pdV work uses the gas pressure (P_a rho_a^-2: without the magnetic
    // part that P/rho^2 of the stress carries with MHD)
    if (k.pdv) {
      if (k.mhd) {
        const T r2 = a.rho1 * a.rho1, c = s * k.m * pv * gka, pg = a.P * r2;
        Pa_b += c * r2;
        rho1a_b += c * T(2.0) * a.P * a.rho1;
        pv_b += s * k.m * pg * gka;
        gka_b += s * k.m * pg * pv;
      } else {  // P/rho^2 of the record is the gas value
        pro2a_b += s * k.m * pv * gka;
        const T t4b = s * k.m * a.pro2;
        pv_b += t4b * gka;
        gka_b += t4b * pv;
      }
    }
    if (k.shock) { q2a_b += s * k.m * pv * gka; pv_b += s * k.m * q2a * gka; gka_b += s * k.m * q2a * pv; }
    // conductivity signal speed: sqrt(2 |P_a - P_b| / (rho_a + rho_b)), or
    // |v_ab . n| with self-gravity (force.F90:1605-1621)
    const T dP = a.P - b.P, rs = a.rho + b.rho;
    const T X = fabs(dP) * T(2.0) / rs;
    const T vsigu = k.grav ? fabs(pv) : sqrt(X);
    const T den = a.u - b.u;
    const T aua = T(0.5) * k.m * k.alphau * a.rho1, aub = T(0.5) * k.m * k.alphau * b.rho1;
    const T E = aua * gka + aub * gkb;
    const T vsigu_b = s * den * E, den_b = s * vsigu * E;
    const T aua_b = s * vsigu * den * gka, aub_b = s * vsigu * den * gkb;
    gka_b += s * vsigu * den * aua;
    gkb_b += s * vsigu * den * aub;
    ua_b += den_b; ub_b -= den_b;
    rho1a_b += aua_b * T(0.5) * k.m * k.alphau;
    rho1b_b += aub_b * T(0.5) * k.m * k.alphau;
    if (k.grav) {
      if (pv != T(0.0)) pv_b += pv > T(0.0) ? vsigu_b : -vsigu_b;
    } else if (X > T(0.0)) {
      const T X_b = vsigu_b / (T(2.0) * vsigu);
      const T sg = dP > T(0.0) ? T(1.0) : -T(1.0);
      Pa_b += X_b * sg * T(2.0) / rs; Pb_b -= X_b * sg * T(2.0) / rs;
      rhoa_b -= X_b * X / rs; rhob_b -= X_b * X / rs;
    }
  }
  T bxa_b = T(0.0), bya_b = T(0.0), bza_b = T(0.0), bxb_b = T(0.0), byb_b = T(0.0), bzb_b = T(0.0), divb = T(0.0);
  if (k.mhd) {
    // stress: -w . (S_a n gka + S_b n gkb) = m [(w.B_a)(B_a.n) gka + (w.B_b)(B_b.n) gkb]
    const T wBa = wx * a.bx + wy * a.by + wz * a.bz, wBb = wx * b.bx + wy * b.by + wz * b.bz;
    const T Ban = a.bx * nx + a.by * ny + a.bz * nz, Bbn = b.bx * nx + b.by * ny + b.bz * nz;
    gka_b += k.m * wBa * Ban; gkb_b += k.m * wBb * Bbn;
    nbx += k.m * (wBa * gka * a.bx + wBb * gkb * b.bx);
    nby += k.m * (wBa * gka * a.by + wBb * gkb * b.by);
    nbz += k.m * (wBa * gka * a.bz + wBb * gkb * b.bz);
    bxa_b += k.m * gka * (wx * Ban + wBa * nx); bya_b += k.m * gka * (wy * Ban + wBa * ny);
    bza_b += k.m * gka * (wz * Ban + wBa * nz);
    bxb_b += k.m * gkb * (wx * Bbn + wBb * nx); byb_b += k.m * gkb * (wy * Bbn + wBb * ny);
    bzb_b += k.m * gkb * (wz * Bbn + wBb * nz);
    // divB_a += m (gka rho1a (B_a.n) + gkb rho1b (B_b.n)), weighted by kap
    divb = k.m * (gka * a.rho1 * Ban + gkb * b.rho1 * Bbn);
    if (kap != T(0.0)) {
      gka_b += kap * k.m * a.rho1 * Ban; gkb_b += kap * k.m * b.rho1 * Bbn;
      rho1a_b += kap * k.m * gka * Ban; rho1b_b += kap * k.m * gkb * Bbn;
      const T ca = kap * k.m * gka * a.rho1, cb = kap * k.m * gkb * b.rho1;
      bxa_b += ca * nx; bya_b += ca * ny; bza_b += ca * nz;
      bxb_b += cb * nx; byb_b += cb * ny; bzb_b += cb * nz;
      nbx += ca * a.bx + cb * b.bx; nby += ca * a.by + cb * b.by; nbz += ca * a.bz + cb * b.bz;
    }
  }
  T psia_b = T(0.0), psib_b = T(0.0), dvbx = T(0.0), dvby = T(0.0), dvbz = T(0.0), fs4 = T(0.0), fs11 = T(0.0);
  if (IND && k.mhd && k.induct) {
    // d(B_a/rho_a)/dt += -m rho_a^-2 gk_a (B_a.n) dv + dBdiss dB - dpsi n, with
    // dBdiss = (A_a gk_a + A_b gk_b) |dv - (dv.n) n|, A = m alphaB rho^-2 / 2,
    // dpsi = oc m (rho_a^-2 gk_a psi_a vw_a + rho_b^-2 gk_b psi_b vw_b);
    // fs11_a += -m (dB.n) gk_a; fs4_a += (dv.n) gk_a; du_a/dt += -|dB|^2 dBdiss / 2
    // (force.F90:1630-1671), B = (B/rho) rho
    const T Bax = a.bx * a.rho, Bay = a.by * a.rho, Baz = a.bz * a.rho;
    const T dBx = Bax - b.bx * b.rho, dBy = Bay - b.by * b.rho, dBz = Baz - b.bz * b.rho;
    const T r2a = a.rho1 * a.rho1, r2b = b.rho1 * b.rho1;
    const T pma = k.m * r2a * gka, pmb = k.m * r2b * gkb;
    const T projBa = Bax * nx + Bay * ny + Baz * nz;
    const T projdB = dBx * nx + dBy * ny + dBz * nz;
    const T tX = dvx - pv * nx, tY = dvy - pv * ny, tZ = dvz - pv * nz;
    const T vsigB = sqrt(tX * tX + tY * tY + tZ * tZ);
    const T hab = T(0.5) * k.m * k.alphaB;
    const T Aa = hab * r2a, Ab = hab * r2b;
    const T E = Aa * gka + Ab * gkb;
    const T dpsi = k.oc * (pma * a.psi * a.cs + pmb * b.psi * b.cs);
    fs4 = pv * gka;
    fs11 = -k.m * projdB * gka;
    const T odv = wt.ox * dvx + wt.oy * dvy + wt.oz * dvz;
    const T odB = wt.ox * dBx + wt.oy * dBy + wt.oz * dBz;
    const T on = wt.ox * nx + wt.oy * ny + wt.oz * nz;
    T Bbx = T(0.0), Bby = T(0.0), Bbz = T(0.0);  // cotangent of B_a
    T dBbx = E * vsigB * wt.ox, dBby = E * vsigB * wt.oy, dBbz = E * vsigB * wt.oz;  // of dB
    T E_b = vsigB * odB, vsB_b = E * odB;
    T pma_b = -projBa * odv, pmb_b = T(0.0);
    const T projBa_b = -pma * odv;
    Bbx += projBa_b * nx; Bby += projBa_b * ny; Bbz += projBa_b * nz;
    nbx += projBa_b * Bax - dpsi * wt.ox; nby += projBa_b * Bay - dpsi * wt.oy; nbz += projBa_b * Baz - dpsi * wt.oz;
    dvbx -= pma * projBa * wt.ox; dvby -= pma * projBa * wt.oy; dvbz -= pma * projBa * wt.oz;
    const T cl_b = -k.oc * on;
    pma_b += cl_b * a.psi * a.cs; psia_b += cl_b * pma * a.cs; csa_b += cl_b * pma * a.psi;
    pmb_b += cl_b * b.psi * b.cs; psib_b += cl_b * pmb * b.cs; csb_b += cl_b * pmb * b.psi;
    if (wt.k11 != T(0.0)) {
      const T c11 = -wt.k11 * k.m;
      dBbx += c11 * gka * nx; dBby += c11 * gka * ny; dBbz += c11 * gka * nz;
      nbx += c11 * gka * dBx; nby += c11 * gka * dBy; nbz += c11 * gka * dBz;
      gka_b += c11 * projdB;
    }
    if (wt.k4 != T(0.0)) { pv_b += wt.k4 * gka; gka_b += wt.k4 * pv; }
    if (k.resist && s != T(0.0)) {
      const T dB2 = dBx * dBx + dBy * dBy + dBz * dBz;
      dBbx -= s * E * vsigB * dBx; dBby -= s * E * vsigB * dBy; dBbz -= s * E * vsigB * dBz;
      E_b -= T(0.5) * s * dB2 * vsigB;
      vsB_b -= T(0.5) * s * dB2 * E;
    }
    gka_b += E_b * Aa + pma_b * k.m * r2a;
    gkb_b += E_b * Ab + pmb_b * k.m * r2b;
    const T r2a_b = E_b * gka * hab + pma_b * k.m * gka, r2b_b = E_b * gkb * hab + pmb_b * k.m * gkb;
    rho1a_b += T(2.0) * a.rho1 * r2a_b;
    rho1b_b += T(2.0) * b.rho1 * r2b_b;
    if (vsigB > T(0.0)) {
      const T c = vsB_b / vsigB;
      const T tbx = c * tX, tby = c * tY, tbz = c * tZ;
      const T ntb = nx * tbx + ny * tby + nz * tbz;
      dvbx += tbx - ntb * nx; dvby += tby - ntb * ny; dvbz += tbz - ntb * nz;
      nbx -= pv * tbx + ntb * dvx; nby -= pv * tby + ntb * dvy; nbz -= pv * tbz + ntb * dvz;
    }
    Bbx += dBbx; Bby += dBby; Bbz += dBbz;
    bxa_b += Bbx * a.rho; bya_b += Bby * a.rho; bza_b += Bbz * a.rho;
    rhoa_b += Bbx * a.bx + Bby * a.by + Bbz * a.bz;
    bxb_b -= dBbx * b.rho; byb_b -= dBby * b.rho; bzb_b -= dBbz * b.rho;
    rhob_b -= dBbx * b.bx + dBby * b.by + dBbz * b.bz;
  }
  pro2a_b += gp_bar * k.m * gka; q2a_b += gp_bar * k.m * gka; gka_b += gp_bar * k.m * (a.pro2 + q2a);
  pro2b_b += gp_bar * k.m * gkb; q2b_b += gp_bar * k.m * gkb; gkb_b += gp_bar * k.m * (b.pro2 + q2b);
  // self-gravity: fsoft(r/h)/h^2 has d/dr = fsoft' h^-3, d/dh = -h^-3 (q fsoft' + 2 fsoft)
  T rg_b = T(0.0), hag_b = T(0.0), hbg_b = T(0.0), gsa_b = T(0.0), gsb_b = T(0.0);
  if (k.grav) {
    const T fg_b = T(0.5) * k.m * gp_bar;
    if (qa < T(2.0)) {
      const T h3 = a.h1 * a.h1 * a.h1;
      rg_b += fg_b * dfsa * h3;
      hag_b -= fg_b * h3 * (qa * dfsa + T(2.0) * fsa);
      gsa_b += fg_b * gka;
      gka_b += fg_b * a.gs;
    } else {
      rg_b -= fg_b * T(2.0) * rinv * rinv * rinv;
    }
    if (qb < T(2.0)) {
      const T h3 = b.h1 * b.h1 * b.h1;
      rg_b += fg_b * dfsb * h3;
      hbg_b -= fg_b * h3 * (qb * dfsb + T(2.0) * fsb);
      gsb_b += fg_b * gkb;
      gkb_b += fg_b * b.gs;
    } else {
      rg_b -= fg_b * T(2.0) * rinv * rinv * rinv;
    }
  }
  T vsa_b = T(0.0), vsb_b = T(0.0);
  if (neg) {
    rho1a_b += q2a_b * (-T(0.5) * vsa * pv); vsa_b = q2a_b * (-T(0.5) * a.rho1 * pv); pv_b += q2a_b * (-T(0.5) * a.rho1 * vsa);
    rho1b_b += q2b_b * (-T(0.5) * vsb * pv); vsb_b = q2b_b * (-T(0.5) * b.rho1 * pv); pv_b += q2b_b * (-T(0.5) * b.rho1 * vsb);
  }
  if (vsa_raw > T(0.0)) { csa_b += vsa_b * a.alpha; pv_b -= vsa_b * k.beta; }
  if (vsb_raw > T(0.0)) { csb_b += vsb_b * b.alpha; pv_b -= vsb_b * k.beta; }
  // pv = dv . n
  nbx += pv_b * dvx; nby += pv_b * dvy; nbz += pv_b * dvz;
  // gk = w'(q) cn h^-4 G, q = r / h
  T r_b = rg_b, ha_b = hag_b, hb_b = hbg_b, Ga_b = T(0.0), Gb_b = T(0.0);
  if (qa < T(2.0)) {
    Ga_b = gka_b * wpa * hfa;
    const T qa_b = gka_b * wppa * hfa * a.G;
    ha_b += gka_b * (-T(4.0) * gka * a.h1) - qa_b * qa * a.h1;
    r_b += qa_b * a.h1;
  }
  if (qb < T(2.0)) {
    Gb_b = gkb_b * wpb * hfb;
    const T qb_b = gkb_b * wppb * hfb * b.G;
    hb_b += gkb_b * (-T(4.0) * gkb * b.h1) - qb_b * qb * b.h1;
    r_b += qb_b * b.h1;
  }
  // n = d / r, r = |d|
  const T nn = nbx * nx + nby * ny + nbz * nz;
  gdx = (nbx - nn * nx) * rinv + r_b * nx;
  gdy = (nby - nn * ny) * rinv + r_b * ny;
  gdz = (nbz - nn * nz) * rinv + r_b * nz;
  // (accumulators of physics that is off stay untouched: x + 0 costs an FP64
  // add, which IEEE arithmetic does not let the compiler drop)
  auto add_a = [&](Bar<T> &ga) {
    ga.h += ha_b; ga.G += Ga_b; ga.rho1 += rho1a_b; ga.pro2 += pro2a_b; ga.cs += csa_b; ga.P += Pa_b;
    ga.rho += rhoa_b; ga.u += ua_b;
    if (IND) { ga.vx += pv_b * nx + dvbx; ga.vy += pv_b * ny + dvby; ga.vz += pv_b * nz + dvbz; }
    else { ga.vx += pv_b * nx; ga.vy += pv_b * ny; ga.vz += pv_b * nz; }
    if (k.mhd) { ga.bx += bxa_b; ga.by += bya_b; ga.bz += bza_b; ga.divB += divb; }
    if (k.grav) ga.gs += gsa_b;
    if (IND) { ga.psi += psia_b; ga.fs4 += fs4; ga.fs11 += fs11; }
  };
  auto add_b = [&](Bar<T> &gbb) {
    gbb.h += hb_b; gbb.G += Gb_b; gbb.rho1 += rho1b_b; gbb.pro2 += pro2b_b; gbb.cs += csb_b; gbb.P += Pb_b;
    gbb.rho += rhob_b; gbb.u += ub_b;
    if (IND) { gbb.vx -= pv_b * nx + dvbx; gbb.vy -= pv_b * ny + dvby; gbb.vz -= pv_b * nz + dvbz; }
    else { gbb.vx -= pv_b * nx; gbb.vy -= pv_b * ny; gbb.vz -= pv_b * nz; }
    if (k.mhd) { gbb.bx += bxb_b; gbb.by += byb_b; gbb.bz += bzb_b; }
    if (k.grav) gbb.gs += gsb_b;
    if (IND) gbb.psi += psib_b;
  };
  if (BOTH) { add_a(g); add_b(*gb); }
  else if (KEEP_A) add_a(g);
  else add_b(g);
}

template <typename T>
__device__ __forceinline__ Side<T> load_side(const T *rec) {
  Side<T> sd;
  sd.h1 = rec[AR_H1]; sd.G = rec[AR_G]; sd.rho1 = rec[AR_RHO1]; sd.pro2 = rec[AR_PRO2]; sd.cs = rec[AR_CS];
  sd.P = rec[AR_P]; sd.rho = rec[AR_RHO]; sd.u = rec[AR_U]; sd.alpha = rec[AR_ALPHA];
  sd.bx = rec[AR_BX]; sd.by = rec[AR_BY]; sd.bz = rec[AR_BZ];
  sd.psi = rec[AR_PSI];
  sd.gs = rec[AR_GS];
  return sd;
}

template <typename T>
__device__ __forceinline__ Wt<T> load_wt(const T *rec) {
  Wt<T> w;
  w.wx = rec[AR_WX]; w.wy = rec[AR_WY]; w.wz = rec[AR_WZ]; w.s = rec[AR_S]; w.kap = rec[AR_KAP];
  w.ox = rec[AR_OX]; w.oy = rec[AR_OY]; w.oz = rec[AR_OZ]; w.k11 = rec[AR_K11]; w.k4 = rec[AR_K4];
  return w;
}

// fraction of the div B term subtracted from the force (force.F90:2873-2890)
// as a function of beta = 2 P / B^2, and its derivative
__device__ __forceinline__ void divb_frac(double beta, double &f, double &df) {
  if (beta < 2.0) { f = 1.0; df = 0.0; }
  else if (beta < 10.0) { f = (10.0 - beta) * 0.125; df = -0.125; }
  else { f = 0.0; df = 0.0; }
}

// the pair separation in the pass's arithmetic type: FP64 as formed, or
// rounded to FP32 (on the integer pipe) for the precision form
template <typename T>
__device__ __forceinline__ T sep_t(double d);
template <>
__device__ __forceinline__ double sep_t<double>(double d) { return d; }
template <>
__device__ __forceinline__ float sep_t<float>(double d) { return d2f_rn(d); }

// per-particle record: primitives of the force (cons2prim, eos.f90:184-237,
// rho = rhoh(h)), the velocities the force was evaluated with, and the
// cotangents w (accelerations) and s (du/dt) gathered to tree order
__global__ void k_adj_prologue(Params p, int n, const int *perm, const double *th, const double *gradh64,
                               const double *gsoft64, const double *vel, const double *Bevol, const double *w4,
                               const double *wB4, const float *alpha1, double *adj, float *adjf, float4 *txf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pid = perm[i];
  const double pm = p.massoftype;
  const double h = th[i];
  double *r = adj + ADJREC * (size_t)i;
  const double rho = rhoh(h, pm, p.hfact);
  const double *v = vel + 4 * (size_t)pid;
  double P, cs, u = 0.0;
  if (p.ieos == 1) { P = p.polyk * rho; cs = sqrt(p.polyk); }
  else {
    u = v[3];
    const double ponrho = (p.gamma > 1.0001) ? (p.gamma - 1.0) * u : 2.0 / 3.0 * u;
    P = ponrho * rho;
    cs = sqrt(p.gamma * ponrho);
  }
  r[AR_H] = h; r[AR_H1] = 1.0 / h; r[AR_G] = gradh64[i]; r[AR_RHO] = rho; r[AR_RHO1] = 1.0 / rho;
  r[AR_PRO2] = P / (rho * rho); r[AR_CS] = cs; r[AR_CS0] = cs; r[AR_P] = P; r[AR_U] = u;
  r[AR_VX] = v[0]; r[AR_VY] = v[1]; r[AR_VZ] = v[2];
  const double *w = w4 + 4 * (size_t)pid;
  r[AR_WX] = w[0]; r[AR_WY] = w[1]; r[AR_WZ] = w[2]; r[AR_S] = p.isothermal ? 0.0 : w[3];
  r[AR_BX] = r[AR_BY] = r[AR_BZ] = 0.0; r[AR_KAP] = 0.0;
  // the viscosity parameter of the evaluation: a fixed input of one derivs
  // (alphaind(1) evolves in the step, not in derivs)
  r[AR_ALPHA] = p.nalpha > 0 ? (double)alpha1[pid] : p.alpha;
  r[AR_GS] = p.gravity ? gsoft64[i] : 0.0;
  r[AR_C] = 0.0;
  r[AR_PSI] = r[AR_OX] = r[AR_OY] = r[AR_OZ] = r[AR_ZETA] = r[AR_K11] = r[AR_K4] = r[AR_GPSI] = 0.0;
  if (p.mhd) {
    // get_stress (force.F90:2068-2168): P/rho^2 + |B/rho|^2 / 2, v_wave^2 = c_s^2 + |B/rho|^2 rho;
    // div B subtraction weight kap = -(w . B) frac(beta), B = (B/rho) rho
    const double *b = Bevol + 4 * (size_t)pid;
    const double b2r = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
    r[AR_BX] = b[0]; r[AR_BY] = b[1]; r[AR_BZ] = b[2];
    r[AR_PRO2] += 0.5 * b2r;
    r[AR_CS] = sqrt(cs * cs + b2r * rho);
    const double B2 = b2r * rho * rho;
    double f = 0.0, df;
    if (B2 > 0.0) divb_frac(2.0 * P / B2, f, df);
    r[AR_KAP] = -(w[0] * b[0] + w[1] * b[1] + w[2] * b[2]) * rho * f;
    r[AR_PSI] = b[3];
    if (wB4) {
      // cotangents o of d(B/rho)/dt and zeta of dpsi/dt; dpsi/dt =
      // -vclean fs11 / rho - psi vclean psidecayfac / h + psi m fs4 / (2 rho)
      // (force.F90:3107-3123, vclean = overcleanfac v_wave; written only with
      // psidecayfac > 0) weights the div B diffusion sum fs11 by
      // k11 = -zeta vclean / rho and the drho/dt sum fs4 by k4 = zeta psi m / (2 rho)
      const double *wb = wB4 + 4 * (size_t)pid;
      r[AR_OX] = wb[0]; r[AR_OY] = wb[1]; r[AR_OZ] = wb[2];
      if (p.psidecayfac > 0.0) {
        const double vclean = p.overcleanfac * r[AR_CS];
        r[AR_ZETA] = wb[3];
        r[AR_K11] = -wb[3] * vclean / rho;
        r[AR_K4] = 0.5 * wb[3] * b[3] * pm / rho;
      }
    }
  }
  txf[i].w = (float)(1.0 / h);
  if (adjf) {  // FP32 copy of the record for the precision form's pair passes
    float *q = adjf + ADJREC * (size_t)i;
    for (int k = 0; k < AR_NSLOTS; ++k) q[k] = (float)r[k];
  }
}

// pass 1: pair reverse terms gathered per particle
// T = double: the plain form (FP64 pair terms); T = float: the precision
// form (pair separation formed in FP64 and rounded to FP32, pair terms in
// FP32 from the FP32 record copy, per-lane sums Kahan-compensated).
// IND: with the MHD induction, resistivity and cleaning terms (cotangents of
// dBevol, or resistive heating)
template <typename T, bool IND>
__global__ void __launch_bounds__(32 * ADJ_WARPS) k_adj_pairs(Params p, AdjConst<T> kc, const Node *nodes,
                                                              const int *leaves, int ncell, const LeafEntry *pool,
                                                              const int *cell_off, const int *cell_nleaf,
                                                              const int *cell_ntrial, const double *tx,
                                                              const double *ty, const double *tz, const float4 *txf,
                                                              const T *adj, double *psum, int64_t ps,
                                                              double pf_hmin, int *err) {
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int cell = blockIdx.x * ADJ_WARPS + w;
  if (cell >= ncell) return;
  const Node nd = nodes[leaves[cell]];
  const int np = nd.count, s0 = nd.start;
  if (np < 1 || np > MAXCELL) { if (lane == 0) set_error(err, PH_ERR_TREE); return; }
  const int S = 32 / np;
  const bool act = lane < np * S;
  const int il = act ? lane / S : 0, stripe = act ? lane % S : 0;
  const int i = s0 + il;
  const T *ri = adj + ADJREC * (size_t)i;
  const Side<T> si = load_side(ri);
  const double xi = tx[i], yi = ty[i], zi = tz[i];
  const T vxi = ri[AR_VX], vyi = ri[AR_VY], vzi = ri[AR_VZ];
  const Wt<T> wti = load_wt(ri);
  const double hi = ri[AR_H];
  const float4 xif = txf[i];
  const float hi21f = xif.w * xif.w;
  // with self-gravity every trial pair has a term (no distance pre-filter)
  const bool pf_i = hi > pf_hmin && !p.gravity;
  const float pf_h1max = (float)(1.0 / pf_hmin);
  const float q2lim = 4.0f * 1.001f;
  Acc<T> gx, gy, gz, d2, sg;
  Bar<T> gi;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell], ntrial = cell_ntrial[cell];
  const T h51 = si.h1 * si.h1 * si.h1 * si.h1 * si.h1;
  extern __shared__ __align__(16) unsigned char dsm[];
  PairSmem &sm = reinterpret_cast<PairSmem *>(dsm)[w];
  Stage &stg = sm.st;
  for (int base = 0; base < ntrial; base += STAGE) {
    const int cnt = stage_window(p, pool, off, nleaf, ntrial, base, txf, stg);
    auto test = [&](int k) -> bool {
      if (stg.jidx[k] == i) return false;
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
    auto body = [&](int k) {
      const int j = stg.jidx[k];
      const int code = stg.code[k];
      double dx = xi - (tx[j] + offset_of(code, 0, p.dxbound));
      double dy = yi - (ty[j] + offset_of(code, 1, p.dybound));
      double dz = zi - (tz[j] + offset_of(code, 2, p.dzbound));
      dx = wrap(dx, p.dxbound, p.hdlx, p.periodic); dy = wrap(dy, p.dybound, p.hdly, p.periodic);
      dz = wrap(dz, p.dzbound, p.hdlz, p.periodic);
      const T dxt = sep_t<T>(dx), dyt = sep_t<T>(dy), dzt = sep_t<T>(dz);
      const T *rj = adj + ADJREC * (size_t)j;
      const Side<T> sj = load_side(rj);
      const T dvx = vxi - rj[AR_VX], dvy = vyi - rj[AR_VY], dvz = vzi - rj[AR_VZ];
      T ax, ay, az;
      // i receives from j (weights of i) ...
      pair_rev<T, true, IND>(kc, dxt, dyt, dzt, dvx, dvy, dvz, si, sj, wti, gi, ax, ay, az);
      gx += ax; gy += ay; gz += az;
      // ... and j receives from i (weights of j); d -> -d
      pair_rev<T, false, IND>(kc, -dxt, -dyt, -dzt, -dvx, -dvy, -dvz, sj, si, load_wt(rj), gi, ax, ay, az);
      gx -= ax; gy -= ay; gz -= az;
      // d^2 rho_i / dh_i^2 = sum m cn h^-5 (12 w + 8 q w' + q^2 w'')
      const T q = sqrt(dxt * dxt + dyt * dyt + dzt * dzt) * si.h1;
      if (q < T(2.0)) {
        T w0, w1, w2;
        wshape(q, w0, w1, w2);
        d2 += kc.m * kc.cn * h51 * (T(12.0) * w0 + T(8.0) * q * w1 + q * q * w2);
        if (kc.grav) sg += kc.m * q * dphidh_dq(q);
      }
    };
    queue_window(cnt, S, act, il, stripe, sm.q, test, body);
  }
  // stripes of each particle summed in order through shared memory
  const double acc[NADJ] = {gx.value(),    gy.value(),   gz.value(),    gi.vx.value(),  gi.vy.value(),
                            gi.vz.value(), gi.h.value(), gi.G.value(),  gi.rho1.value(), gi.pro2.value(),
                            gi.cs.value(), gi.P.value(), gi.rho.value(), gi.u.value(),   d2.value(),
                            gi.bx.value(), gi.by.value(), gi.bz.value(), gi.divB.value(), gi.gs.value(),
                            sg.value(),    gi.psi.value(), gi.fs4.value(), gi.fs11.value()};
  double *red = reinterpret_cast<double *>(&sm.st);
  __syncwarp();
  for (int k = 0; k < NADJ; ++k) red[lane * NADJ + k] = acc[k];
  __syncwarp();
  if (lane < np) {
    double t[NADJ];
    for (int k = 0; k < NADJ; ++k) t[k] = 0.0;
    for (int q = 0; q < S; ++q)
      for (int k = 0; k < NADJ; ++k) t[k] += red[(lane * S + q) * NADJ + k];
    const size_t ip = (size_t)(s0 + lane);
    for (int k = 0; k < NADJ; ++k) psum[k * ps + ip] = t[k];
  }
}

// ------------------------------------------------------------------ symmetric pass 1 (FP64 hydro)
// Pass 1 with every unordered pair evaluated once, by the rule of the
// symmetric FP64 force loop: cell A takes the owned prefix of its trial list
// (entries starting at or after its first particle) and, in its own leaf, the
// pairs j > i; every pair within either kernel lies in both cells' lists.
// Both ordered terms of a pair (c_ij with i's cotangents, c_ji with j's) are
// reversed once with both sides kept: two reverse terms per pair instead of
// the four of k_adj_pairs. i's cotangents stay in the lane; j's NJA values
// are combined in a per-window array of the warp (lanes holding the same j
// add in lane order) written to jbuf at j's flattened trial index, and
// k_adj_gather adds them to j's sums in the order of j's own list.
constexpr int NJA = 15;  // j side: d-gradient (3), v (3), h, G, rho1, pro2, cs, P, rho, u, d2 rho/dh2
constexpr int STAGE_A = 128;
__device__ __forceinline__ int nja_slot(int v) {
  return v < 3 ? PA_X + v : (v < 6 ? PA_VX + (v - 3) : (v == 14 ? PA_D2 : PA_H + (v - 6)));
}
static_assert(PA_H + 7 == PA_U && PA_D2 == PA_U + 1, "j-side slots h..u follow each other");
struct SymAdjSmem {
  union {
    StageN<STAGE_A> st;
    double red[32 * NADJ];
  } u;
  PairQ q;
  double js[NJA][STAGE_A];
};

__global__ void __launch_bounds__(32 * ADJ_WARPS) k_adj_pairs_sym(
    Params p, AdjConst<double> kc, const Node *nodes, const int *leaves, int ncell, const LeafEntry *pool,
    const int *cell_off, const int *cell_nleaf, const double *tx, const double *ty, const double *tz,
    const float4 *txf, const double *adj, double *psum, int64_t ps, double pf_hmin, const int *toff, double *jbuf,
    int64_t jstride, int *err) {
  const unsigned FULL = 0xffffffffu;
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int cell = blockIdx.x * ADJ_WARPS + w;
  if (cell >= ncell) return;
  const Node nd = nodes[leaves[cell]];
  const int np = nd.count, s0 = nd.start;
  if (np < 1 || np > MAXCELL) { if (lane == 0) set_error(err, PH_ERR_TREE); return; }
  const int S = 32 / np;
  const bool act = lane < np * S;
  const int il = act ? lane / S : 0, stripe = act ? lane % S : 0;
  const int i = s0 + il;
  const double *ri = adj + ADJREC * (size_t)i;
  const Side<double> si = load_side(ri);
  const Wt<double> wti = load_wt(ri);
  const double xi = tx[i], yi = ty[i], zi = tz[i];
  const double vxi = ri[AR_VX], vyi = ri[AR_VY], vzi = ri[AR_VZ];
  const float4 xif = txf[i];
  const float hi21f = xif.w * xif.w;
  const bool pf_i = ri[AR_H] > pf_hmin;
  const float pf_h1max = (float)(1.0 / pf_hmin);
  const float q2lim = 4.0f * 1.001f;
  const double mcn = kc.m * kc.cn;
  const double h51i = si.h1 * si.h1 * si.h1 * si.h1 * si.h1;
  double gx = 0.0, gy = 0.0, gz = 0.0, d2 = 0.0;
  Bar<double> gi;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
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
  const int64_t tb = (int64_t)toff[off];
  extern __shared__ __align__(16) unsigned char dsm[];
  SymAdjSmem &sm = reinterpret_cast<SymAdjSmem *>(dsm)[w];
  StageN<STAGE_A> &stg = sm.u.st;
  const unsigned gmask = !act ? 0u : (S >= 32 ? FULL : (((1u << S) - 1u) << (il * S)));
  const unsigned lt = (1u << lane) - 1u;
  for (int base = 0; base < town; base += STAGE_A) {
    const int cnt = stage_window_n<STAGE_A>(p, pool, off, nown, town, base, txf, stg);
    for (int q = lane; q < NJA * STAGE_A; q += 32) (&sm.js[0][0])[q] = 0.0;
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
        // each particle starts at its own rotation of its queue (the cell's
        // particles accept nearly the same j in nearly the same order)
        const int rot = act && qn > 0 ? (il * qn) / np : 0;
        for (int t = 0; t < nstmax; ++t) {
          int m = stripe + t * S + rot;
          if (m >= qn) m -= qn;
          const bool valid = t < nst;
          const int kk = valid ? (int)sm.q.k[il][m] : -1;
          double jv[NJA];
          for (int v = 0; v < NJA; ++v) jv[v] = 0.0;
          if (valid) {
            const int j = stg.jidx[kk], code = stg.code[kk];
            double dx = xi - (tx[j] + offset_of(code, 0, p.dxbound));
            double dy = yi - (ty[j] + offset_of(code, 1, p.dybound));
            double dz = zi - (tz[j] + offset_of(code, 2, p.dzbound));
            dx = wrap(dx, p.dxbound, p.hdlx, p.periodic); dy = wrap(dy, p.dybound, p.hdly, p.periodic);
            dz = wrap(dz, p.dzbound, p.hdlz, p.periodic);
            const double *rj = adj + ADJREC * (size_t)j;
            const Side<double> sj = load_side(rj);
            const double dvx = vxi - rj[AR_VX], dvy = vyi - rj[AR_VY], dvz = vzi - rj[AR_VZ];
            Bar<double> gj;
            double ax, ay, az;
            // i receives from j (i's cotangents) ...
            pair_rev<double, true, false, true>(kc, dx, dy, dz, dvx, dvy, dvz, si, sj, wti, gi, ax, ay, az, &gj);
            gx += ax; gy += ay; gz += az;
            double jgx = -ax, jgy = -ay, jgz = -az;
            // ... and j receives from i (j's cotangents); d -> -d
            pair_rev<double, true, false, true>(kc, -dx, -dy, -dz, -dvx, -dvy, -dvz, sj, si, load_wt(rj), gj, ax, ay,
                                                az, &gi);
            jgx += ax; jgy += ay; jgz += az;
            gx -= ax; gy -= ay; gz -= az;
            // d^2 rho / dh^2 of both (m cn h^-5 (12 w + 8 q w' + q^2 w''))
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            double w0, w1, w2;
            const double qi = r * si.h1, qj = r * sj.h1;
            if (qi < 2.0) { wshape(qi, w0, w1, w2); d2 += mcn * h51i * (12.0 * w0 + 8.0 * qi * w1 + qi * qi * w2); }
            double jd2 = 0.0;
            if (qj < 2.0) {
              const double h5 = sj.h1 * sj.h1 * sj.h1 * sj.h1 * sj.h1;
              wshape(qj, w0, w1, w2);
              jd2 = mcn * h5 * (12.0 * w0 + 8.0 * qj * w1 + qj * qj * w2);
            }
            jv[0] = jgx; jv[1] = jgy; jv[2] = jgz;
            jv[3] = gj.vx.value(); jv[4] = gj.vy.value(); jv[5] = gj.vz.value();
            jv[6] = gj.h.value(); jv[7] = gj.G.value(); jv[8] = gj.rho1.value(); jv[9] = gj.pro2.value();
            jv[10] = gj.cs.value(); jv[11] = gj.P.value(); jv[12] = gj.rho.value(); jv[13] = gj.u.value();
            jv[14] = jd2;
          }
          // lanes holding the same j: the lowest adds the others' values in
          // lane order, then adds the group's sum to j's window slot
          const unsigned g = __match_any_sync(FULL, valid ? kk : -1 - lane);
          const int gsz = __popc(g);
          const int gmax = (int)__reduce_max_sync(FULL, (unsigned)gsz);
          const bool lead = valid && (g & lt) == 0u;
          for (int u = 1; u < gmax; ++u) {
            const int src = u < gsz ? (int)__fns(g, 0, u + 1) : lane;
            for (int v = 0; v < NJA; ++v) {
              const double y = __shfl_sync(FULL, jv[v], src);
              if (lead && u < gsz) jv[v] += y;
            }
          }
          if (lead)
            for (int v = 0; v < NJA; ++v) sm.js[v][kk] += jv[v];
          __syncwarp();
        }
        qn = 0;
      }
    }
    __syncwarp();
    for (int v = 0; v < NJA; ++v)
      for (int k = lane; k < cnt; k += 32) jbuf[(int64_t)v * jstride + tb + base + k] = sm.js[v][k];
    __syncwarp();
  }
  // the stripes of each particle summed in order (the pass-1 slots; the
  // physics this pass covers leaves the MHD and gravity slots zero)
  double *red = sm.u.red;
  __syncwarp();
  for (int k = 0; k < NADJ; ++k) {
    double v = 0.0;
    if (k < 3) v = k == 0 ? gx : (k == 1 ? gy : gz);
    else if (k == PA_VX) v = gi.vx.value();
    else if (k == PA_VY) v = gi.vy.value();
    else if (k == PA_VZ) v = gi.vz.value();
    else if (k == PA_H) v = gi.h.value();
    else if (k == PA_G) v = gi.G.value();
    else if (k == PA_RHO1) v = gi.rho1.value();
    else if (k == PA_PRO2) v = gi.pro2.value();
    else if (k == PA_CS) v = gi.cs.value();
    else if (k == PA_P) v = gi.P.value();
    else if (k == PA_RHO) v = gi.rho.value();
    else if (k == PA_U) v = gi.u.value();
    else if (k == PA_D2) v = d2;
    red[lane * NADJ + k] = v;
  }
  __syncwarp();
  if (lane < np) {
    const size_t ip = (size_t)(s0 + lane);
    for (int k = 0; k < NADJ; ++k) {
      double t = 0.0;
      for (int q = 0; q < S; ++q) t += red[(lane * S + q) * NADJ + k];
      psum[k * ps + ip] = t;
    }
  }
}

// Pass 2 on the symmetric lists (FP64 hydro): the pair coefficient
// m/r [A_i dW(r,h_i)/dr + B_i d2W(r,h_i)/dhdr + A_j dW(r,h_j)/dr + B_j d2W(r,h_j)/dhdr]
// is symmetric in i and j, so an owned pair adds coef d to i and -coef d to
// j (d = x_i - x_j); j's three values go through jbuf and k_adj_gather as in
// pass 1 (NJ = 3 slots: the position gradient)
struct SymDensSmem {
  union {
    StageN<STAGE_A> st;
    double red[32 * 3];
  } u;
  PairQ q;
  double js[3][STAGE_A];
};

__global__ void __launch_bounds__(32 * ADJ_WARPS) k_adj_dens_sym(
    Params p, const Node *nodes, const int *leaves, int ncell, const LeafEntry *pool, const int *cell_off,
    const int *cell_nleaf, const double *tx, const double *ty, const double *tz, const float4 *txf,
    const double *adj, double *psum, int64_t ps, double pf_hmin, const int *toff, double *jbuf, int64_t jstride,
    int *err) {
  const unsigned FULL = 0xffffffffu;
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int cell = blockIdx.x * ADJ_WARPS + w;
  if (cell >= ncell) return;
  const Node nd = nodes[leaves[cell]];
  const int np = nd.count, s0 = nd.start;
  if (np < 1 || np > MAXCELL) { if (lane == 0) set_error(err, PH_ERR_TREE); return; }
  const int S = 32 / np;
  const bool act = lane < np * S;
  const int il = act ? lane / S : 0, stripe = act ? lane % S : 0;
  const int i = s0 + il;
  const double *ri = adj + ADJREC * (size_t)i;
  const double pm = p.massoftype;
  const double xi = tx[i], yi = ty[i], zi = tz[i];
  const double h1i = ri[AR_H1], Ai = ri[AR_A], Bi = ri[AR_B];
  const double h4i = CNORMK * h1i * h1i * h1i * h1i, h5i = h4i * h1i;
  const float4 xif = txf[i];
  const float hi21f = xif.w * xif.w;
  const bool pf_i = ri[AR_H] > pf_hmin;
  const float pf_h1max = (float)(1.0 / pf_hmin);
  const float q2lim = 4.0f * 1.001f;
  double gx = 0.0, gy = 0.0, gz = 0.0;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
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
  const int64_t tb = (int64_t)toff[off];
  extern __shared__ __align__(16) unsigned char dsm[];
  SymDensSmem &sm = reinterpret_cast<SymDensSmem *>(dsm)[w];
  StageN<STAGE_A> &stg = sm.u.st;
  const unsigned gmask = !act ? 0u : (S >= 32 ? FULL : (((1u << S) - 1u) << (il * S)));
  const unsigned lt = (1u << lane) - 1u;
  for (int base = 0; base < town; base += STAGE_A) {
    const int cnt = stage_window_n<STAGE_A>(p, pool, off, nown, town, base, txf, stg);
    for (int q = lane; q < 3 * STAGE_A; q += 32) (&sm.js[0][0])[q] = 0.0;
    __syncwarp();
    auto test = [&](int k) -> bool {
      const int j = stg.jidx[k];
      if (j <= i && j >= s0) return false;
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
        const int rot = act && qn > 0 ? (il * qn) / np : 0;
        for (int t = 0; t < nstmax; ++t) {
          int m = stripe + t * S + rot;
          if (m >= qn) m -= qn;
          const bool valid = t < nst;
          const int kk = valid ? (int)sm.q.k[il][m] : -1;
          double jv0 = 0.0, jv1 = 0.0, jv2 = 0.0;
          if (valid) {
            const int j = stg.jidx[kk], code = stg.code[kk];
            double dx = xi - (tx[j] + offset_of(code, 0, p.dxbound));
            double dy = yi - (ty[j] + offset_of(code, 1, p.dybound));
            double dz = zi - (tz[j] + offset_of(code, 2, p.dzbound));
            dx = wrap(dx, p.dxbound, p.hdlx, p.periodic); dy = wrap(dy, p.dybound, p.hdly, p.periodic);
            dz = wrap(dz, p.dzbound, p.hdlz, p.periodic);
            const double r2 = dx * dx + dy * dy + dz * dz, r = sqrt(r2), rinv = inv_sep(r2, r);
            const double *rj = adj + ADJREC * (size_t)j;
            double coef = 0.0, w0, w1, w2;
            const double qi = r * h1i;
            if (qi < 2.0) {
              wshape(qi, w0, w1, w2);
              coef += Ai * h4i * w1 + Bi * h5i * (-4.0 * w1 - qi * w2);
            }
            const double h1j = rj[AR_H1];
            const double qj = r * h1j;
            if (qj < 2.0) {
              wshape(qj, w0, w1, w2);
              const double h4j = CNORMK * h1j * h1j * h1j * h1j;
              coef += rj[AR_A] * h4j * w1 + rj[AR_B] * h4j * h1j * (-4.0 * w1 - qj * w2);
            }
            coef *= pm * rinv;
            gx += coef * dx; gy += coef * dy; gz += coef * dz;
            jv0 = -coef * dx; jv1 = -coef * dy; jv2 = -coef * dz;
          }
          const unsigned g = __match_any_sync(FULL, valid ? kk : -1 - lane);
          const int gsz = __popc(g);
          const int gmax = (int)__reduce_max_sync(FULL, (unsigned)gsz);
          const bool lead = valid && (g & lt) == 0u;
          for (int u = 1; u < gmax; ++u) {
            const int src = u < gsz ? (int)__fns(g, 0, u + 1) : lane;
            const double y0 = __shfl_sync(FULL, jv0, src), y1 = __shfl_sync(FULL, jv1, src),
                         y2 = __shfl_sync(FULL, jv2, src);
            if (lead && u < gsz) { jv0 += y0; jv1 += y1; jv2 += y2; }
          }
          if (lead) { sm.js[0][kk] += jv0; sm.js[1][kk] += jv1; sm.js[2][kk] += jv2; }
          __syncwarp();
        }
        qn = 0;
      }
    }
    __syncwarp();
    for (int v = 0; v < 3; ++v)
      for (int k = lane; k < cnt; k += 32) jbuf[(int64_t)v * jstride + tb + base + k] = sm.js[v][k];
    __syncwarp();
  }
  double *red = sm.u.red;
  __syncwarp();
  red[lane * 3] = gx; red[lane * 3 + 1] = gy; red[lane * 3 + 2] = gz;
  __syncwarp();
  if (lane < np) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int q = 0; q < S; ++q) {
      const double *src = red + (lane * S + q) * 3;
      t0 += src[0]; t1 += src[1]; t2 += src[2];
    }
    const size_t ip = (size_t)(s0 + lane);
    psum[ip] = t0; psum[ps + ip] = t1; psum[2 * ps + ip] = t2;
  }
}

// Per leaf cell B: add to its particles' pass-1 (NJ = NJA) or pass-2 (NJ = 3)
// sums the j-side values that k_adj_pairs_sym or k_adj_dens_sym left in jbuf (its own leaf's entry and those of the cells
// before it whose lists hold B, found by a binary search), in the order of
// B's own list (as k_force_gather)
template <int NJ>
__global__ void k_adj_gather(const Node *nodes, const int *leaves, int ncell, const LeafEntry *pool,
                             const int *cell_off, const int *cell_nleaf, const int *cell_at, const int *toff,
                             const double *jbuf, int64_t jstride, double *psum, int64_t ps) {
  const unsigned FULL = 0xffffffffu;
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int cell = blockIdx.x * (blockDim.x >> 5) + w;
  if (cell >= ncell) return;
  const Node nd = nodes[leaves[cell]];
  const int np = nd.count, s0 = nd.start;
  if (np < 1 || np > MAXCELL) return;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell];
  constexpr int NC = (NJ * MAXCELL + 31) / 32;
  double acc[NC];
  for (int r = 0; r < NC; ++r) acc[r] = 0.0;
  for (int e0 = nleaf - 1; e0 >= 0; e0 -= 32) {
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
    const int nin = __popc(inb);
    for (int q = nin - 1; q >= 0; --q) {
      const int sl = __shfl_sync(FULL, slot, q);
      if (sl < 0) continue;
      for (int r = 0; r < NC; ++r) {
        const int c = lane + 32 * r;
        const int v = c / MAXCELL, t = c % MAXCELL;
        if (v < NJ && t < np) acc[r] += jbuf[(int64_t)v * jstride + sl + t];
      }
    }
    if (nin < 32) break;
  }
  for (int r = 0; r < NC; ++r) {
    const int c = lane + 32 * r;
    const int v = c / MAXCELL, t = c % MAXCELL;
    if (v < NJ && t < np) psum[(int64_t)nja_slot(v) * ps + s0 + t] += acc[r];
  }
}

// chain rule per particle and the implicit-solve coefficients
__global__ void k_adj_coef(Params p, int n, const double *psum, int64_t ps, double *adj, float *adjf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *r = adj + ADJREC * (size_t)i;
  const double pm = p.massoftype;
  const double h = r[AR_H], rho = r[AR_RHO], rho1 = r[AR_RHO1], G = r[AR_G], u = r[AR_U], cs = r[AR_CS0];
  auto ps_ = [&](int k) { return psum[k * ps + i]; };
  double P_b = ps_(PA_P), rho_b = ps_(PA_RHO) - ps_(PA_RHO1) * rho1 * rho1, cs_b = ps_(PA_CS);
  double bx_b = 0.0, by_b = 0.0, bz_b = 0.0, psi_b = 0.0, h_fin = 0.0;
  if (p.mhd) {
    psi_b = ps_(PA_PSI);
    const double zeta = r[AR_ZETA];
    if (zeta != 0.0) {
      // dpsi/dt = -vclean fs11 rho1 - psi dtau + psi m fs4 rho1 / 2, vclean =
      // overcleanfac v_wave, dtau = psidecayfac vclean / h (force.F90:3107-3123)
      const double psi = r[AR_PSI], fs4 = ps_(PA_FS4), fs11 = ps_(PA_FS11);
      const double vclean = p.overcleanfac * r[AR_CS], dtau = p.psidecayfac * vclean / h;
      psi_b += zeta * (-dtau + 0.5 * pm * fs4 * rho1);
      cs_b += zeta * p.overcleanfac * (-fs11 * rho1 - psi * p.psidecayfac / h);  // v_wave
      rho_b -= zeta * (-vclean * fs11 + 0.5 * psi * pm * fs4) * rho1 * rho1;
      h_fin = zeta * psi * dtau / h;
    }
    const double bx = r[AR_BX], by = r[AR_BY], bz = r[AR_BZ], b2r = bx * bx + by * by + bz * bz;
    bx_b = ps_(PA_BX); by_b = ps_(PA_BY); bz_b = ps_(PA_BZ);
    // P/rho^2 + |B/rho|^2/2: the magnetic part
    const double pro2_b = ps_(PA_PRO2);
    bx_b += pro2_b * bx; by_b += pro2_b * by; bz_b += pro2_b * bz;
    // v_wave = sqrt(c_s^2 + |B/rho|^2 rho)
    const double vw = r[AR_CS], vw_b = cs_b;
    cs_b = vw > 0.0 ? vw_b * cs / vw : 0.0;
    if (vw > 0.0) {
      bx_b += vw_b * rho * bx / vw; by_b += vw_b * rho * by / vw; bz_b += vw_b * rho * bz / vw;
      rho_b += vw_b * b2r / (2.0 * vw);
    }
    // div B subtraction: kap = -(w . B/rho) rho frac(beta), beta = 2 P / (|B/rho|^2 rho^2), times the sum
    const double D = ps_(PA_DIVB), P = r[AR_P];
    const double B2 = b2r * rho * rho;
    if (B2 > 0.0 && D != 0.0) {
      const double beta = 2.0 * P / B2;
      double f, df;
      divb_frac(beta, f, df);
      const double wb = r[AR_WX] * bx + r[AR_WY] * by + r[AR_WZ] * bz;
      bx_b += D * (-r[AR_WX] * rho * f + wb * rho * df * 2.0 * beta * bx / b2r);
      by_b += D * (-r[AR_WY] * rho * f + wb * rho * df * 2.0 * beta * by / b2r);
      bz_b += D * (-r[AR_WZ] * rho * f + wb * rho * df * 2.0 * beta * bz / b2r);
      rho_b += D * (-wb * f + wb * rho * df * 2.0 * beta / rho);
      P_b += D * (-wb * rho * df * beta / P);
    }
  }
  // rho-dependence of 1/rho, P/rho^2, P (eos); then h through rho = m (hfact/h)^3
  double u_b = ps_(PA_U);
  if (p.ieos == 1) {
    rho_b += P_b * p.polyk - ps_(PA_PRO2) * p.polyk * rho1 * rho1;
  } else {
    const double gm1 = (p.gamma > 1.0001) ? (p.gamma - 1.0) : 2.0 / 3.0;
    rho_b += P_b * gm1 * u - ps_(PA_PRO2) * gm1 * u * rho1 * rho1;
    u_b += P_b * gm1 * rho + ps_(PA_PRO2) * gm1 * rho1;
    if (cs > 0.0) u_b += cs_b * p.gamma * gm1 / (2.0 * cs);  // c_s = sqrt(gamma gm1 u)
  }
  double h_b = ps_(PA_H) + rho_b * (-3.0 * rho / h) + h_fin;
  // self-gravity: gradsoft = -K (S_phi + 1.4 m), K = h^2 / (3 m hfact^3),
  // S_phi = sum_j m dphi_h(r_ij/h): d/dh at fixed x = 2 gradsoft/h + K SG/h
  // (SG = sum m q dphi_h/dq), and the coefficient C = -K gradsoft_bar on
  // dS_phi/dx for pass 2
  double C = 0.0;
  if (p.gravity) {
    const double K = h * h / (3.0 * pm * p.hfact * p.hfact * p.hfact);
    const double GS_b = ps_(PA_GS);
    h_b += GS_b * (2.0 * r[AR_GS] + K * ps_(PA_SG)) / h;
    C = -GS_b * K;
  }
  r[AR_C] = C;
  const double G_b = ps_(PA_G);
  // implicit solve: Omega = 1 - dhdrho S, S = d rho / dh (at fixed x)
  const double dhdrho = -h / (3.0 * rho);
  const double Om = 1.0 / G;
  const double S = (1.0 - Om) / dhdrho;
  // d2 rho/dh2 including the self term m cn h^-5 * 12
  const double h1 = 1.0 / h;
  const double d2 = ps_(PA_D2) + pm * CNORMK * 12.0 * h1 * h1 * h1 * h1 * h1;
  const double dOm_dh = -(4.0 * dhdrho * h1) * S - dhdrho * d2;
  const double dG_dh = -G * G * dOm_dh;
  const double H = h_b + G_b * dG_dh;
  r[AR_A] = H * dhdrho * G;
  r[AR_B] = G_b * G * G * dhdrho;
  if (adjf) {
    float *q = adjf + ADJREC * (size_t)i;
    q[AR_A] = (float)r[AR_A]; q[AR_B] = (float)r[AR_B]; q[AR_C] = (float)C;
  }
  r[AR_GX] = ps_(PA_X); r[AR_GY] = ps_(PA_Y); r[AR_GZ] = ps_(PA_Z);
  r[AR_GVX] = ps_(PA_VX); r[AR_GVY] = ps_(PA_VY); r[AR_GVZ] = ps_(PA_VZ);
  r[AR_GU] = u_b;
  r[AR_GBX] = bx_b; r[AR_GBY] = by_b; r[AR_GBZ] = bz_b; r[AR_GPSI] = psi_b;
}

// pass 2: positions through the density sums
template <typename T>
__global__ void __launch_bounds__(32 * ADJ_WARPS) k_adj_dens(Params p, const Node *nodes, const int *leaves,
                                                             int ncell, const LeafEntry *pool, const int *cell_off,
                                                             const int *cell_nleaf, const int *cell_ntrial,
                                                             const double *tx, const double *ty, const double *tz,
                                                             const float4 *txf, const T *adj, double *psum,
                                                             int64_t ps, double pf_hmin, int *err) {
  const int w = threadIdx.x >> 5, lane = lane_id();
  const int cell = blockIdx.x * ADJ_WARPS + w;
  if (cell >= ncell) return;
  const Node nd = nodes[leaves[cell]];
  const int np = nd.count, s0 = nd.start;
  if (np < 1 || np > MAXCELL) { if (lane == 0) set_error(err, PH_ERR_TREE); return; }
  const int S = 32 / np;
  const bool act = lane < np * S;
  const int il = act ? lane / S : 0, stripe = act ? lane % S : 0;
  const int i = s0 + il;
  const T *ri = adj + ADJREC * (size_t)i;
  const T pm = (T)p.massoftype;
  const double xi = tx[i], yi = ty[i], zi = tz[i];
  const T h1i = ri[AR_H1], Ai = ri[AR_A], Bi = ri[AR_B], Ci = ri[AR_C];
  const bool grav = p.gravity != 0;
  const double hi = ri[AR_H];
  const T h4i = T(CNORMK) * h1i * h1i * h1i * h1i, h5i = h4i * h1i;
  const float4 xif = txf[i];
  const float hi21f = xif.w * xif.w;
  const bool pf_i = hi > pf_hmin;
  const float pf_h1max = (float)(1.0 / pf_hmin);
  const float q2lim = 4.0f * 1.001f;
  Acc<T> gx, gy, gz;
  const int off = cell_off[cell], nleaf = cell_nleaf[cell], ntrial = cell_ntrial[cell];
  extern __shared__ __align__(16) unsigned char dsm[];
  PairSmem &sm = reinterpret_cast<PairSmem *>(dsm)[w];
  Stage &stg = sm.st;
  for (int base = 0; base < ntrial; base += STAGE) {
    const int cnt = stage_window(p, pool, off, nleaf, ntrial, base, txf, stg);
    auto test = [&](int k) -> bool {
      if (stg.jidx[k] == i) return false;
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
    auto body = [&](int k) {
      const int j = stg.jidx[k];
      const int code = stg.code[k];
      double dx = xi - (tx[j] + offset_of(code, 0, p.dxbound));
      double dy = yi - (ty[j] + offset_of(code, 1, p.dybound));
      double dz = zi - (tz[j] + offset_of(code, 2, p.dzbound));
      dx = wrap(dx, p.dxbound, p.hdlx, p.periodic); dy = wrap(dy, p.dybound, p.hdly, p.periodic);
      dz = wrap(dz, p.dzbound, p.hdlz, p.periodic);
      const T dxt = sep_t<T>(dx), dyt = sep_t<T>(dy), dzt = sep_t<T>(dz);
      const T r2 = dxt * dxt + dyt * dyt + dzt * dzt, r = sqrt(r2), rinv = inv_sep(r2, r);
      const T *rj = adj + ADJREC * (size_t)j;
      T coef = T(0.0), w0, w1, w2;
      const T qi = r * h1i;
      if (qi < T(2.0)) {  // dW/dr = cn h^-4 w', d2W/dhdr = cn h^-5 (-4 w' - q w'')
        wshape(qi, w0, w1, w2);
        coef += Ai * h4i * w1 + Bi * h5i * (T(-4.0) * w1 - qi * w2);
        if (grav) coef += Ci * h1i * dphidh_dq(qi);
      }
      const T h1j = rj[AR_H1];
      const T qj = r * h1j;
      if (qj < T(2.0)) {
        wshape(qj, w0, w1, w2);
        const T h4j = T(CNORMK) * h1j * h1j * h1j * h1j;
        coef += rj[AR_A] * h4j * w1 + rj[AR_B] * h4j * h1j * (T(-4.0) * w1 - qj * w2);
        if (grav) coef += rj[AR_C] * h1j * dphidh_dq(qj);
      }
      coef *= pm * rinv;
      gx += coef * dxt; gy += coef * dyt; gz += coef * dzt;
    };
    queue_window(cnt, S, act, il, stripe, sm.q, test, body);
  }
  double *red = reinterpret_cast<double *>(&sm.st);
  __syncwarp();
  red[lane * 3] = gx.value(); red[lane * 3 + 1] = gy.value(); red[lane * 3 + 2] = gz.value();
  __syncwarp();
  if (lane < np) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int q = 0; q < S; ++q) {
      const double *src = red + (lane * S + q) * 3;
      t0 += src[0]; t1 += src[1]; t2 += src[2];
    }
    const size_t ip = (size_t)(s0 + lane);
    psum[ip] = t0; psum[ps + ip] = t1; psum[2 * ps + ip] = t2;
  }
}

// results in the caller's order: gradients with respect to xyzh (h slot 0:
// h is not an independent input), vxyzu and, with MHD, Bevol (B/rho and psi)
__global__ void k_adj_out(int n, const int *perm, const double *adj, const double *psum, int64_t ps, int grav,
                          double *gxyzh, double *gvxyzu, double *gBevol) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int pid = perm[i];
  const double *r = adj + ADJREC * (size_t)i;
  double *gx = gxyzh + 4 * (size_t)pid, *gv = gvxyzu + 4 * (size_t)pid;
  gx[0] = r[AR_GX] + psum[i]; gx[1] = r[AR_GY] + psum[ps + i]; gx[2] = r[AR_GZ] + psum[2 * ps + i]; gx[3] = 0.0;
  if (grav) {  // the far field's share (slots 3..5)
    gx[0] += psum[3 * ps + i]; gx[1] += psum[4 * ps + i]; gx[2] += psum[5 * ps + i];
  }
  gv[0] = r[AR_GVX]; gv[1] = r[AR_GVY]; gv[2] = r[AR_GVZ]; gv[3] = r[AR_GU];
  if (gBevol) {
    double *gb = gBevol + 4 * (size_t)pid;
    gb[0] = r[AR_GBX]; gb[1] = r[AR_GBY]; gb[2] = r[AR_GBZ]; gb[3] = r[AR_GPSI];
  }
}

static inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }

}  // namespace ph

using namespace ph;

namespace ph {

// The adjoint on the device-resident state: cotangents w of fxyzu and, with
// MHD, wB of dBevol (caller order, 4 rows per particle, device; wB may be
// null) -> gradients gx, gv (and gb with MHD), caller order, device. The tree, density and force lists are recomputed unless the
// state flags say they are current. Records ev[0..2] around the recompute and
// the adjoint passes and evk[0..1] around the pair passes.
int adjoint_dev(ph_ctx *c, const double *w_dev, const double *wB_dev, double *gx_d, double *gv_d, double *gb_d) {
  const Params p = c->dp;
  if (alloc_adjoint(c) != 0) return PH_ERR_CUDA;
  cudaStream_t st = c->stream;
  cudaEventRecord(c->ev[0], st);
  // forward state at the uploaded positions: tree, density, force lists
  int r = 0;
  if (!c->have_tree) { r = build_tree(c); if (r) return r; }
  if (!c->have_density) { r = density(c, 1); if (r) return r; }
  r = force_lists(c);
  if (r) return r;
  cudaEventRecord(c->ev[1], st);
  const int nt = (int)c->ntree, ncell = c->nleaves;
  // cotangents staged in the pair-sum buffer (caller order, 4 per particle)
  const size_t n4 = 4 * (size_t)c->n;
  const bool wB = p.mhd && wB_dev;
  cudaMemcpyAsync(c->psum, w_dev, sizeof(double) * n4, cudaMemcpyDeviceToDevice, st);
  if (wB) cudaMemcpyAsync(c->psum + n4, wB_dev, sizeof(double) * n4, cudaMemcpyDeviceToDevice, st);
  const bool mixed = p.precision == PH_PREC_MIXED;
  k_adj_prologue<<<nblk(nt, 256), 256, 0, st>>>(p, nt, c->perm, c->th, c->gradh64, c->gsoft64, c->vxyzu, c->Bevol,
                                                c->psum, wB ? c->psum + n4 : nullptr,
                                                c->alpha1, c->adj, mixed ? c->adjf : nullptr, c->txf);
  const int smem = ADJ_WARPS * (int)sizeof(PairSmem);
  if (!(c->attr_done & 4u)) {
    cudaFuncSetAttribute(k_adj_pairs<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_adj_pairs<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_adj_dens<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_adj_pairs<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_adj_pairs<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_adj_pairs_sym, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         ADJ_WARPS * (int)sizeof(SymAdjSmem));
    cudaFuncSetAttribute(k_adj_dens<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    c->attr_done |= 4u;
  }
  cudaEventRecord(c->evk[0], st);
  if (mixed) {
    AdjConst<float> kc;
    kc.m = (float)p.massoftype; kc.alpha = (float)p.alpha; kc.beta = (float)p.beta; kc.alphau = (float)p.alphau;
    kc.cn = (float)CNORMK;
    kc.adiab = !p.isothermal; kc.pdv = p.ipdv_heating > 0; kc.shock = p.ishock_heating > 0; kc.mhd = p.mhd != 0;
    kc.grav = p.gravity != 0;
    kc.alphaB = (float)p.alphaB; kc.oc = (float)p.overcleanfac;
    kc.resist = p.mhd && p.iresistive_heating > 0 && !p.isothermal;
    kc.induct = p.mhd && (wB || kc.resist);
    (kc.induct ? k_adj_pairs<float, true> : k_adj_pairs<float, false>)<<<nblk(ncell, ADJ_WARPS), 32 * ADJ_WARPS,
                                                                        smem, st>>>(
        p, kc, c->nodes, c->leaves, ncell, c->pool, c->cell_off, c->cell_nleaf, c->cell_ntrial, c->tx, c->ty,
        c->tz, c->txf, c->adjf, c->psum, c->cap, c->pf_hmin, c->d_err);
    k_adj_coef<<<nblk(nt, 256), 256, 0, st>>>(p, nt, c->psum, c->cap, c->adj, c->adjf);
    k_adj_dens<float><<<nblk(ncell, ADJ_WARPS), 32 * ADJ_WARPS, smem, st>>>(
        p, c->nodes, c->leaves, ncell, c->pool, c->cell_off, c->cell_nleaf, c->cell_ntrial, c->tx, c->ty, c->tz,
        c->txf, c->adjf, c->psum, c->cap, c->pf_hmin, c->d_err);
  } else {
    AdjConst<double> kc;
    kc.m = p.massoftype; kc.alpha = p.alpha; kc.beta = p.beta; kc.alphau = p.alphau; kc.cn = CNORMK;
    kc.adiab = !p.isothermal; kc.pdv = p.ipdv_heating > 0; kc.shock = p.ishock_heating > 0; kc.mhd = p.mhd != 0;
    kc.grav = p.gravity != 0;
    kc.alphaB = p.alphaB; kc.oc = p.overcleanfac;
    kc.resist = p.mhd && p.iresistive_heating > 0 && !p.isothermal;
    kc.induct = p.mhd && (wB || kc.resist);
    // FP64 hydro on the symmetric force lists: each pair once (k_adj_pairs_sym)
    const bool sym = !p.mhd && !p.gravity && c->force_sym && c->toff && c->sym_total > 0;
    if (sym) {
      if (alloc_sym(c, c->sym_total, NJA) != 0) return PH_ERR_CUDA;
      k_adj_pairs_sym<<<nblk(ncell, ADJ_WARPS), 32 * ADJ_WARPS, ADJ_WARPS * (int)sizeof(SymAdjSmem), st>>>(
          p, kc, c->nodes, c->leaves, ncell, c->pool, c->cell_off, c->cell_nleaf, c->tx, c->ty, c->tz, c->txf,
          c->adj, c->psum, c->cap, c->pf_hmin, c->toff, c->jbuf, c->jbuf_stride, c->d_err);
      k_adj_gather<NJA><<<nblk(ncell, 4), 128, 0, st>>>(c->nodes, c->leaves, ncell, c->pool, c->cell_off,
                                                        c->cell_nleaf, c->cell_at, c->toff, c->jbuf,
                                                        c->jbuf_stride, c->psum, c->cap);
      count_launch(c, 1);
    } else {
      (kc.induct ? k_adj_pairs<double, true> : k_adj_pairs<double, false>)<<<nblk(ncell, ADJ_WARPS),
                                                                            32 * ADJ_WARPS, smem, st>>>(
          p, kc, c->nodes, c->leaves, ncell, c->pool, c->cell_off, c->cell_nleaf, c->cell_ntrial, c->tx, c->ty,
          c->tz, c->txf, c->adj, c->psum, c->cap, c->pf_hmin, c->d_err);
    }
    k_adj_coef<<<nblk(nt, 256), 256, 0, st>>>(p, nt, c->psum, c->cap, c->adj, nullptr);
    if (sym) {
      k_adj_dens_sym<<<nblk(ncell, ADJ_WARPS), 32 * ADJ_WARPS, ADJ_WARPS * (int)sizeof(SymDensSmem), st>>>(
          p, c->nodes, c->leaves, ncell, c->pool, c->cell_off, c->cell_nleaf, c->tx, c->ty, c->tz, c->txf, c->adj,
          c->psum, c->cap, c->pf_hmin, c->toff, c->jbuf, c->jbuf_stride, c->d_err);
      k_adj_gather<3><<<nblk(ncell, 4), 128, 0, st>>>(c->nodes, c->leaves, ncell, c->pool, c->cell_off,
                                                      c->cell_nleaf, c->cell_at, c->toff, c->jbuf, c->jbuf_stride,
                                                      c->psum, c->cap);
      count_launch(c, 1);
    } else {
      k_adj_dens<double><<<nblk(ncell, ADJ_WARPS), 32 * ADJ_WARPS, smem, st>>>(
          p, c->nodes, c->leaves, ncell, c->pool, c->cell_off, c->cell_nleaf, c->cell_ntrial, c->tx, c->ty, c->tz,
          c->txf, c->adj, c->psum, c->cap, c->pf_hmin, c->d_err);
    }
  }
  // self-gravity: the far field's share of the position gradients (slots 3..5)
  if (p.gravity) gravity_adjoint_far(c, c->adj + AR_WX, ADJREC, c->psum + 3 * c->cap, c->cap);
  cudaEventRecord(c->evk[1], st);
  k_adj_out<<<nblk(nt, 256), 256, 0, st>>>(nt, c->perm, c->adj, c->psum, c->cap, p.gravity ? 1 : 0, gx_d, gv_d,
                                           gb_d);
  count_launch(c, 5);
  cudaEventRecord(c->ev[2], st);
  return 0;
}

}  // namespace ph

extern "C" {

int ph_adjoint_full(ph_ctx *c, const double *w_fxyzu, const double *w_dBevol, double *g_xyzh, double *g_vxyzu,
                    double *g_Bevol) {
  if (!c || !w_fxyzu || !g_xyzh || !g_vxyzu) return PH_ERR_ARG;
  if (c->n <= 0) return PH_ERR_NOPART;
  const Params p = c->dp;
  // individual timesteps: an evaluation re-computes the active particles'
  // forces only (the inactive ones keep theirs), and its lists cover the
  // active cells only; its adjoint is not built
  if (p.ind) return PH_ERR_NOT_BUILT;
  if (p.mhd && !g_Bevol) return PH_ERR_ARG;
  if (alloc_adjoint(c) != 0) return PH_ERR_CUDA;
  cudaStream_t st = c->stream;
  reset_timers(c);
  const size_t n = (size_t)c->n;
  const bool wB = p.mhd && w_dBevol;
  // cotangents in caller order, staged where the recompute of the tree and
  // density (whose pair sums use psum, whose velocity-derivative pass uses
  // jrec) cannot overwrite them
  if (alloc_rollout(c, 8 * n) != 0) return PH_ERR_CUDA;
  copy_vrows_h2d(c, c->ro_buf, w_fxyzu, (size_t)n);
  if (wB) cudaMemcpyAsync(c->ro_buf + 4 * n, w_dBevol, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, st);
  double *gx_d = c->jrec, *gv_d = c->jrec + 4 * n, *gb_d = p.mhd ? c->jrec + 8 * n : nullptr;
  int r = adjoint_dev(c, c->ro_buf, wB ? c->ro_buf + 4 * n : nullptr, gx_d, gv_d, gb_d);
  if (r) return r;
  cudaMemcpyAsync(g_xyzh, gx_d, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, st);
  copy_vrows_d2h(c, g_vxyzu, gv_d, (size_t)n);
  if (p.mhd) cudaMemcpyAsync(g_Bevol, gb_d, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return PH_ERR_CUDA;
  int herr = 0;
  cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (herr) return herr;
  float ms;
  // device time: [0] forward recompute (tree, density, lists), [2] adjoint
  // passes, [4] the pair passes, [7] total (cotangent upload included,
  // gradient download excluded)
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]); c->last_ms[0] = ms;
  cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]); c->last_ms[2] = ms;
  add_elapsed(c, 4, c->evk[0], c->evk[1]);
  cudaEventElapsedTime(&ms, c->ev[0], c->ev[2]); c->last_ms[7] = ms;
  return check_launch(c) == cudaSuccess ? 0 : PH_ERR_CUDA;
}

int ph_adjoint(ph_ctx *c, const double *w_fxyzu, double *g_xyzh, double *g_vxyzu, double *g_Bevol) {
  return ph_adjoint_full(c, w_fxyzu, nullptr, g_xyzh, g_vxyzu, g_Bevol);
}

}  // extern "C"
