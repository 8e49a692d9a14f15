// Leapfrog KDK integrator (K9) and the derivs driver: step (step_leapfrog.f90:
// 91-760) with substep_sph (substepping.F90:241-264), check_velocity_error
// (step_leapfrog.f90:769-843) and derivs (deriv.f90:37-232), all on the device.
// Global reductions (velocity error, conservation sums) are FP64 with a fixed
// summation order.
#include <cmath>

#include "ph_internal.h"

namespace ph {

static inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }
constexpr int RED_BLOCKS = 1024;

// predictor: v,u += dt/2 f; B += dt/2 dB (step_leapfrog.f90:183-234), then the
// drift x += dt v (substepping.F90:249-262) and predict_sph (:307-374): h from
// div v, vpred = v + dt/2 f, Bpred = B + dt/2 dB.
__global__ void k_predict(Params p, int n, double hdt, double dt, double *xyzh, double *vxyzu, const double *fxyzu,
                          double *Bevol, const double *dBevol, const float *divcurlv, double *vpred, double *Bpred,
                          float *alpha1, const float *alphaloc_t, const double *eos_t, const int *iperm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *x = xyzh + 4 * (size_t)i;
  if (x[3] < TINY_D) return;
  double *v = vxyzu + 4 * (size_t)i;
  const double *f = fxyzu + 4 * (size_t)i;
  const int nv = p.isothermal ? 3 : 4;
  for (int k = 0; k < nv; ++k) v[k] = v[k] + hdt * f[k];
  if (p.mhd) {
    double *b = Bevol + 4 * (size_t)i;
    const double *db = dBevol + 4 * (size_t)i;
    for (int k = 0; k < 4; ++k) b[k] = b[k] + hdt * db[k];
  }
  for (int k = 0; k < 3; ++k) x[k] = x[k] + dt * v[k];
  const double h = x[3];
  const double pm = p.massoftype;
  x[3] = h - dt * dhdrho(h, pm, p.hfact) * rhoh(h, pm, p.hfact) * (double)divcurlv[i];
  double *vp = vpred + 4 * (size_t)i;
  for (int k = 0; k < nv; ++k) vp[k] = v[k] + (0.5 * dt) * f[k];
  if (p.mhd) {
    const double *b = Bevol + 4 * (size_t)i;
    const double *db = dBevol + 4 * (size_t)i;
    double *bp = Bpred + 4 * (size_t)i;
    for (int k = 0; k < 4; ++k) bp[k] = b[k] + (0.5 * dt) * db[k];
  }
  if (p.nalpha >= 2) {  // step_leapfrog.f90:378-391 (Cullen & Dehnen), with the predicted h
    const int t = iperm[i];  // tree position of the last build (alphaloc and c_s of the last derivs)
    const double hi = x[3];
    const double tdecay1 = ddiv(dmul(AVDECAYCONST, eos_t[2 * (size_t)t + 1]), hi);
    const double ddenom = ddiv(1.0, dadd(1.0, dmul(dt, tdecay1)));
    const double alphaloci = (double)alphaloc_t[t];
    const double a = (double)alpha1[i];
    alpha1[i] = (a < alphaloci) ? (float)alphaloci : (float)dmul(dadd(a, dmul(dmul(dt, alphaloci), tdecay1)), ddenom);
  }
}

// initial.F90:736-742: alpha = max(alpha, alphaloc) after the initial derivs
__global__ void k_alpha_initial(int n, float *alpha1, const float *alphaloc_t, const int *iperm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  alpha1[i] = fmaxf(alpha1[i], alphaloc_t[iperm[i]]);
}

// alphaind(3,:) and dvdx(9,:) in caller order (alphaloc, a tree-order field, through iperm)
__global__ void k_alpha_gather(int n, const float *alpha1, const float *alphaloc_t, const float *ddivvdt_c,
                               const float *dvdx_c, const int *iperm, float *alphaind, float *dvdx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int t = iperm ? iperm[i] : -1;
  alphaind[3 * (size_t)i] = alpha1[i];
  alphaind[3 * (size_t)i + 1] = t >= 0 ? alphaloc_t[t] : 0.0f;
  alphaind[3 * (size_t)i + 2] = t >= 0 ? ddivvdt_c[i] : 0.0f;
  for (int q = 0; q < 9; ++q) dvdx[9 * (size_t)i + q] = t >= 0 ? dvdx_c[9 * (size_t)i + q] : 0.0f;
}

// corrector (step_leapfrog.f90:582-620) + per-block partials of errmax and sum v^2
__global__ void __launch_bounds__(256) k_correct(Params p, int n, double hdt, double *vxyzu, const double *fxyzu,
                                                 const double *vpred, double *Bevol, const double *dBevol,
                                                 const double *xyzh, double *part) {
  __shared__ double se[8], sv[8];
  double emax = 0.0, v2 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (xyzh[4 * (size_t)i + 3] < TINY_D) continue;
    double *v = vxyzu + 4 * (size_t)i;
    const double *f = fxyzu + 4 * (size_t)i;
    const double *vp = vpred + 4 * (size_t)i;
    const double vx = v[0] + hdt * f[0], vy = v[1] + hdt * f[1], vz = v[2] + hdt * f[2];
    const double ex = vx - vp[0], ey = vy - vp[1], ez = vz - vp[2];
    emax = fmax(emax, ex * ex + ey * ey + ez * ez);
    v2 += vx * vx + vy * vy + vz * vz;
    v[0] = vx; v[1] = vy; v[2] = vz;
    if (!p.isothermal) v[3] = v[3] + hdt * f[3];
    if (p.mhd) {
      double *b = Bevol + 4 * (size_t)i;
      const double *db = dBevol + 4 * (size_t)i;
      for (int k = 0; k < 4; ++k) b[k] = b[k] + hdt * db[k];
    }
  }
  emax = warp_max(emax);
  for (int o = 16; o > 0; o >>= 1) v2 += __shfl_xor_sync(0xffffffffu, v2, o);
  if (lane_id() == 0) { se[threadIdx.x >> 5] = emax; sv[threadIdx.x >> 5] = v2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) { emax = fmax(emax, se[w]); v2 += sv[w]; }
    part[2 * blockIdx.x] = emax;
    part[2 * blockIdx.x + 1] = v2;
  }
}

// undo the corrector before a velocity iteration (step_leapfrog.f90:650-700)
__global__ void k_uncorrect(Params p, int n, double hdt, double *vxyzu, const double *fxyzu, double *vpred,
                            double *Bevol, const double *dBevol, double *Bpred) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *v = vxyzu + 4 * (size_t)i;
  const double *f = fxyzu + 4 * (size_t)i;
  double *vp = vpred + 4 * (size_t)i;
  for (int k = 0; k < 4; ++k) vp[k] = v[k];
  const int nv = p.isothermal ? 3 : 4;
  for (int k = 0; k < nv; ++k) v[k] = v[k] - hdt * f[k];
  if (p.mhd) {
    double *b = Bevol + 4 * (size_t)i;
    const double *db = dBevol + 4 * (size_t)i;
    double *bp = Bpred + 4 * (size_t)i;
    for (int k = 0; k < 4; ++k) { bp[k] = b[k]; b[k] = b[k] - hdt * db[k]; }
  }
}

// conservation sums: momentum, kinetic/thermal/magnetic/potential energy and
// the energy rate sum m (v.a + du/dt) (energies.f90:65-711 formulas)
__global__ void __launch_bounds__(256) k_conserve(Params p, int n, const double *xyzh, const double *vxyzu,
                                                  const double *fxyzu, const double *Bevol, const float *poten,
                                                  double *part, int vs) {
  __shared__ double s[8][8];
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const double pm = p.massoftype;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double *x = xyzh + 4 * (size_t)i;
    if (x[3] < TINY_D) continue;
    const double *v = vxyzu + vs * (size_t)i;  // vs: rows of vxyzu and fxyzu (maxvxyzu)
    const double *f = fxyzu + vs * (size_t)i;
    acc[0] += pm * v[0]; acc[1] += pm * v[1]; acc[2] += pm * v[2];
    acc[3] += 0.5 * pm * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (!p.isothermal) acc[4] += pm * v[3];
    if (p.mhd) {
      const double rho = rhoh(x[3], pm, p.hfact);
      const double *b = Bevol + 4 * (size_t)i;
      acc[5] += 0.5 * pm * rho * (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    }
    if (p.gravity) acc[6] += (double)poten[i];
    acc[7] += pm * (v[0] * f[0] + v[1] * f[1] + v[2] * f[2] + (p.isothermal ? 0.0 : f[3]));
  }
  for (int k = 0; k < 8; ++k)
    for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
  if (lane_id() == 0) for (int k = 0; k < 8; ++k) s[threadIdx.x >> 5][k] = acc[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 8; ++k) {
      double t = s[0][k];
      for (int w = 1; w < 8; ++w) t += s[w][k];
      part[8 * blockIdx.x + k] = t;
    }
  }
}

__global__ void k_sum_partials(const double *part, int nb, int stride, int nk, int nmax, double *out) {
  // fixed-order final reduction by one warp: lane l combines blocks l, l+32,
  // ... in order, then a butterfly over the lanes; the first nmax entries
  // are maxima, the rest sums
  const int lane = threadIdx.x & 31;
  if (threadIdx.x >= 32) return;
  for (int k = 0; k < nk; ++k) {
    const bool mx = k < nmax;
    double t = mx ? -HUGE_D : 0.0;
    for (int b = lane; b < nb; b += 32) t = mx ? fmax(t, part[stride * b + k]) : t + part[stride * b + k];
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_xor_sync(0xffffffffu, t, o);
      t = mx ? fmax(t, y) : t + y;
    }
    if (lane == 0) out[k] = t;
  }
}

struct StepTimer {
  ph_ctx *c;
  explicit StepTimer(ph_ctx *cc) : c(cc) {}
  void mark(int k) { cudaEventRecord(c->ev[k], c->stream); }
};

int derivs_dev(ph_ctx *c, int icall, const double *vel, const double *Bv, double *dtnew) {
  int r = 0;
  cudaEventRecord(c->ev[0], c->stream);
  if (icall == 1 || icall == 0) { r = build_tree(c); if (r) return r; }
  cudaEventRecord(c->ev[1], c->stream);
  if (icall == 1) {
    c->dens_vel = vel;  // the velocity derivatives of the switch use the evaluation's velocities
    c->dens_B = Bv;     // and the div B, curl B sums its Bevol (Bpred in a step)
    r = density(c, icall);
    c->dens_vel = nullptr;
    c->dens_B = nullptr;
    if (r) return r;
  }
  cudaEventRecord(c->ev[2], c->stream);
  c->ind_icall = icall;
  r = force_dev(c, vel, Bv);
  if (r) return r;
  cudaEventRecord(c->ev[3], c->stream);
  double dts[2];
  int ic[3] = {0, 0, 0};
  const bool ind = c->dp.ind && c->ibin;
  cudaMemcpyAsync(dts, c->red, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (ind) cudaMemcpyAsync(ic, c->d_ind, 3 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return PH_ERR_CUDA;
  int herr = 0;
  cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (herr) return herr;
  float ms;
  if (icall == 1 || icall == 0) { cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]); c->last_ms[0] += ms; }
  if (icall == 1) { cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]); c->last_ms[1] += ms; }
  cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]); c->last_ms[2] += ms;
  add_elapsed(c, 4, c->evk[0], c->evk[1]);
  c->dtcourant = dts[0];
  c->dtforce = dts[1];
  if (ind) {  // force.F90:749-756, 792: nbinmax from the particles binned by this force call
    if (ic[1] > 0) c->nbinmax = ic[0];
    if (ic[2]) c->ind_too_small = true;
  }
  // deriv.f90:226 dtnew = min(dtforce, dtcourant, dtrad, dtmax)
  if (dtnew) *dtnew = std::fmin(std::fmin(c->dtforce, c->dtcourant), std::fmin(BIGNUMBER, c->dp.dtmax));
  return 0;
}

}  // namespace ph

using namespace ph;

extern "C" {

int ph_force(ph_ctx *c, int icall, double dt, double *fxyzu, double *dBevol, float *divcurlv, float *divBsymm,
             float *poten, double *dtcourant, double *dtforce) {
  (void)icall; (void)dt;
  if (!c) return PH_ERR_ARG;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  reset_timers(c);
  int r = derivs_dev(c, 2, c->vxyzu, c->Bevol, nullptr);
  if (r) return r;
  const size_t n = (size_t)c->n;
  if (fxyzu) copy_vrows_d2h(c, fxyzu, c->fxyzu, n);
  if (dBevol) cudaMemcpyAsync(dBevol, c->dBevol, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, c->stream);
  if (divcurlv && copy_divcurlv_d2h(c, divcurlv, n) != 0) return PH_ERR_CUDA;
  if (divBsymm) cudaMemcpyAsync(divBsymm, c->divBsymm, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream);
  if (poten) cudaMemcpyAsync(poten, c->poten, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return PH_ERR_CUDA;
  if (dtcourant) *dtcourant = c->dtcourant;
  if (dtforce) *dtforce = c->dtforce;
  return 0;
}

int ph_derivs(ph_ctx *c, int icall, double dt, double *dtnew) {
  (void)dt;
  if (!c || icall < 0 || icall > 2) return PH_ERR_ARG;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  reset_timers(c);
  return derivs_dev(c, icall, c->vxyzu, c->Bevol, dtnew);
}

int ph_set_alpha(ph_ctx *c, const float *alpha) {
  if (!c || !alpha) return PH_ERR_ARG;
  cudaMemcpyAsync(c->alpha1, alpha, sizeof(float) * (size_t)c->n, cudaMemcpyHostToDevice, c->stream);
  return check_cuda(c);
}

int ph_get_alpha(ph_ctx *c, float *alphaind, float *dvdx) {
  if (!c) return PH_ERR_ARG;
  const int n = (int)c->n;
  if (n <= 0 || (!alphaind && !dvdx)) return 0;
  float *da = nullptr, *dd = nullptr;
  if (cudaMalloc(&da, sizeof(float) * 3 * (size_t)n) != cudaSuccess ||
      cudaMalloc(&dd, sizeof(float) * 9 * (size_t)n) != cudaSuccess) {
    if (da) cudaFree(da);
    return PH_ERR_CUDA;
  }
  k_alpha_gather<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->alpha1, c->alphaloc_t, c->ddivvdt_c, c->dvdx_c,
                                                      c->have_tree ? c->iperm : nullptr, da, dd);
  count_launch(c);
  if (alphaind) cudaMemcpyAsync(alphaind, da, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  if (dvdx) cudaMemcpyAsync(dvdx, dd, sizeof(float) * 9 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  cudaFree(da);
  cudaFree(dd);
  return check_cuda(c);
}

int ph_alpha_initial(ph_ctx *c) {
  if (!c) return PH_ERR_ARG;
  if (c->dp.nalpha < 2) return 0;
  if (!c->have_force) return PH_ERR_STATE;
  const int n = (int)c->n;
  k_alpha_initial<<<nblk(n, 256), 256, 0, c->stream>>>(n, c->alpha1, c->alphaloc_t, c->iperm);
  count_launch(c);
  return check_cuda(c);
}

int ph_step(ph_ctx *c, double t, double dtsph, double *dtnew, int32_t *its_out, double *dterr_out) {
  (void)t;
  if (!c || !(dtsph > 0.0)) return PH_ERR_ARG;
  if (!c->have_force) return PH_ERR_STATE;
  cudaStream_t st = c->stream;
  const int n = (int)c->n;
  const Params p = c->dp;
  const double hdt = 0.5 * dtsph;
  reset_timers(c);
  cudaEventRecord(c->evk[6], st);
  cudaMemsetAsync(c->d_err, 0, sizeof(int), st);
  cudaEventRecord(c->ev[4], st);
  k_predict<<<nblk(n, 256), 256, 0, st>>>(p, n, hdt, dtsph, c->xyzh, c->vxyzu, c->fxyzu, c->Bevol, c->dBevol,
                                          c->divcurlv, c->vpred, c->Bpred, c->alpha1, c->alphaloc_t, c->eos,
                                          c->iperm);
  count_launch(c);
  cudaEventRecord(c->ev[5], st);
  double dtn = 0.0;
  const double *Bv = p.mhd ? c->Bpred : c->Bevol;
  int r = derivs_dev(c, 1, c->vpred, Bv, &dtn);
  if (r) return r;
  const int maxits = 30;
  int its = 0;
  bool converged = false;
  double dterr = BIGNUMBER;
  double *part = c->jrec;  // scratch: the j records are rebuilt by the next force call
  double *res = c->red + 8;
  float ms_int = 0.0f, ms;
  cudaEventElapsedTime(&ms, c->ev[4], c->ev[5]);
  ms_int += ms;
  while (its < maxits && !converged) {
    ++its;
    cudaEventRecord(c->ev[6], st);
    int nb = std::min(RED_BLOCKS, nblk(n, 256));
    k_correct<<<nb, 256, 0, st>>>(p, n, hdt, c->vxyzu, c->fxyzu, c->vpred, c->Bevol, c->dBevol, c->xyzh, part);
    k_sum_partials<<<1, 32, 0, st>>>(part, nb, 2, 2, 1, res);
    count_launch(c, 2);
    double hv[2];
    cudaMemcpyAsync(hv, res, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaEventRecord(c->ev[7], st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return PH_ERR_CUDA;
    cudaEventElapsedTime(&ms, c->ev[6], c->ev[7]);
    ms_int += ms;
    // check_velocity_error (step_leapfrog.f90:790-838)
    double errmax = hv[0], v2mean = hv[1] / (double)n;
    errmax = (v2mean > TINY_D) ? errmax / std::sqrt(v2mean) : 0.0;
    double errtol = p.tolv;
    dterr = HUGE_D;
    if (p.tolv < 1.e2) {
      const double dtf = std::fmin(c->dtcourant, c->dtforce);
      if (dtf > dtsph && dtf < BIGNUMBER) errtol = errtol * (dtsph / dtf) * (dtsph / dtf);
      if (its == 1 && errtol > TINY_D && errmax > EPS_D) dterr = dtsph * std::sqrt(errtol / errmax);
      converged = errmax < p.tolv;
    } else {
      converged = true;
    }
    c->dterr = dterr;  // dterr is reset on every call of check_velocity_error (step_leapfrog.f90:807)
    if (!converged) {
      k_uncorrect<<<nblk(n, 256), 256, 0, st>>>(p, n, hdt, c->vxyzu, c->fxyzu, c->vpred, c->Bevol, c->dBevol,
                                                c->Bpred);
      count_launch(c);
      r = derivs_dev(c, 2, c->vpred, Bv, &dtn);
      if (r) return r;
    }
  }
  c->last_ms[3] = ms_int;
  cudaEventRecord(c->evk[7], st);
  cudaEventSynchronize(c->evk[7]);
  add_elapsed(c, 7, c->evk[6], c->evk[7]);
  if (its_out) *its_out = its;
  if (dterr_out) *dterr_out = c->dterr;
  if (dtnew) *dtnew = dtn;
  // step_leapfrog.f90:753-756: fatal once its reaches maxits, also when the
  // last iteration converged
  if (its >= maxits) return PH_ERR_TOLV;
  return 0;
}

int ph_upload_state(ph_ctx *c, int64_t npart, const double *xyzh, const double *vxyzu, const double *Bevol,
                    const double *fxyzu, const double *dBevol, const float *divcurlv) {
  if (!c || !fxyzu || !divcurlv) return PH_ERR_ARG;
  int r = ph_upload(c, npart, xyzh, vxyzu, Bevol);
  if (r) return r;
  const size_t n = (size_t)npart;
  copy_vrows_h2d(c, c->fxyzu, fxyzu, n);
  if (dBevol) cudaMemcpyAsync(c->dBevol, dBevol, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, c->stream);
  if (copy_divcurlv_h2d(c, divcurlv, n) != 0) return PH_ERR_CUDA;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return PH_ERR_CUDA;
  c->have_force = true;
  return 0;
}

int ph_download_state(ph_ctx *c, double *xyzh, double *vxyzu, double *Bevol, double *fxyzu, double *dBevol,
                      float *divcurlv) {
  if (!c) return PH_ERR_ARG;
  const size_t n = (size_t)c->n;
  if (xyzh) cudaMemcpyAsync(xyzh, c->xyzh, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, c->stream);
  if (vxyzu) copy_vrows_d2h(c, vxyzu, c->vxyzu, n);
  if (Bevol) cudaMemcpyAsync(Bevol, c->Bevol, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, c->stream);
  if (fxyzu) copy_vrows_d2h(c, fxyzu, c->fxyzu, n);
  if (dBevol) cudaMemcpyAsync(dBevol, c->dBevol, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, c->stream);
  if (divcurlv && copy_divcurlv_d2h(c, divcurlv, n) != 0) return PH_ERR_CUDA;
  return cudaStreamSynchronize(c->stream) == cudaSuccess ? 0 : PH_ERR_CUDA;
}

int ph_work_counters(ph_ctx *c, int64_t *out4) {
  if (!c || !out4) return PH_ERR_ARG;
  unsigned long long s[4];
  cudaMemcpy(s, c->stats + 8, sizeof(s), cudaMemcpyDeviceToHost);
  for (int k = 0; k < 4; ++k) out4[k] = (int64_t)s[k];
  return 0;
}

int ph_conservation(ph_ctx *c, double *out) {
  if (!c || !out) return PH_ERR_ARG;
  const int n = (int)c->n;
  int nb = std::min(RED_BLOCKS, nblk(n, 256));
  double *part = c->jrec;
  k_conserve<<<nb, 256, 0, c->stream>>>(c->dp, n, c->xyzh, c->vxyzu, c->fxyzu, c->Bevol, c->poten, part, 4);
  k_sum_partials<<<1, 32, 0, c->stream>>>(part, nb, 8, 8, 0, c->red + 8);
  count_launch(c, 2);
  cudaMemcpyAsync(out, c->red + 8, 8 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  return cudaStreamSynchronize(c->stream) == cudaSuccess ? 0 : PH_ERR_CUDA;
}

}  // extern "C"
