// Individual particle timesteps (IND_TIMESTEPS): power-of-two bins of dtmax.
// set_active_particles (utils_indtimesteps.f90:114-178), the substep of
// step_leapfrog.f90:91-760 with individual timesteps (predictor to the
// particles' half steps, drift, predict_sph, derivs on the active particles,
// corrector of the active particles, synchronisation and waking of the
// rest; one corrector pass), init_step (step_leapfrog.f90:45-84) and the
// evolve loop's time and bin bookkeeping (evolve.f90:132-154, 206, 437-440;
// evolve_utils.F90:65-91 update_time_and_dt; utils_indtimesteps.f90:186-223
// change_nbinmax).
//
// Bins, twas and the wake bins are per particle in caller order; the force
// sets each active particle's new bin (get_newbin and the Saitoh-Makino
// limiter, in k_force_finish) and marks the neighbours it found for waking.
#include <cmath>

#include "ph_internal.h"

namespace ph {

static inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }

// ibin_dts(itdt / ithdt / itdt1 / ittwas, 0:maxbins) of step_leapfrog.f90:157-163
struct BinDts {
  double t[4][MAXBINS + 1];
};

// set_active_particles: active if the particle's bin ends its step on this
// substep; counters[0] active count, counters[1] a bin above nbinmax
__global__ void k_set_active(int n, const double *xyzh, const int8_t *ibin, unsigned char *actf, int nbinmax,
                             int istepfrac, int *counters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int a = 0, bad = 0;
  if (i < n) {
    if (xyzh[4 * (size_t)i + 3] <= 0.0) {
      actf[i] = 0;
    } else {
      const int b = ibin[i];
      if (b > nbinmax) bad = 1;
      else a = (istepfrac % (1 << (nbinmax - b)) == 0) ? 1 : 0;
      actf[i] = (unsigned char)a;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if (lane_id() == 0) {
    if (a) atomicAdd(&counters[0], a);
    if (bad) atomicOr(&counters[1], 1);
  }
}

// predictor (step_leapfrog.f90:183-234 with twas: each particle to the time
// of the step, from its own half step), drift (substepping.F90:241-264),
// predict_sph (step_leapfrog.f90:296-398) and the viscosity switch
__global__ void k_ind_predict(Params p, int n, double timei, double dtsph, const double *twas, const int8_t *ibin,
                              int8_t *ibin_old, const unsigned char *actf, double *xyzh, double *vxyzu,
                              const double *fxyzu, double *Bevol, const double *dBevol, const float *divcurlv,
                              double *vpred, double *Bpred, float *alpha1, const float *alphaloc_t,
                              const double *eos_t, const int *iperm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *x = xyzh + 4 * (size_t)i;
  if (x[3] < TINY_D) return;
  if (actf[i]) ibin_old[i] = ibin[i];
  double *v = vxyzu + 4 * (size_t)i;
  const double *f = fxyzu + 4 * (size_t)i;
  const int nv = p.isothermal ? 3 : 4;
  const double hdti = twas[i] - timei;
  for (int k = 0; k < nv; ++k) v[k] = v[k] + hdti * f[k];
  if (p.mhd) {
    double *b = Bevol + 4 * (size_t)i;
    const double *db = dBevol + 4 * (size_t)i;
    for (int k = 0; k < 4; ++k) b[k] = b[k] + hdti * db[k];
  }
  for (int k = 0; k < 3; ++k) x[k] = x[k] + dtsph * v[k];
  const double tnew = timei + dtsph;
  const double h = x[3];
  const double pm = p.massoftype;
  x[3] = h - dtsph * dhdrho(h, pm, p.hfact) * rhoh(h, pm, p.hfact) * (double)divcurlv[i];
  const double hdtp = tnew - twas[i];
  double *vp = vpred + 4 * (size_t)i;
  for (int k = 0; k < nv; ++k) vp[k] = v[k] + hdtp * f[k];
  if (p.mhd) {
    const double *b = Bevol + 4 * (size_t)i;
    const double *db = dBevol + 4 * (size_t)i;
    double *bp = Bpred + 4 * (size_t)i;
    for (int k = 0; k < 4; ++k) bp[k] = b[k] + hdtp * db[k];
  }
  if (p.nalpha >= 2) {  // step_leapfrog.f90:378-391 with the substep
    const int t = iperm[i];
    const double hi = x[3];
    const double tdecay1 = ddiv(dmul(AVDECAYCONST, eos_t[2 * (size_t)t + 1]), hi);
    const double ddenom = ddiv(1.0, dadd(1.0, dmul(dtsph, tdecay1)));
    const double alphaloci = (double)alphaloc_t[t];
    const double a = (double)alpha1[i];
    alpha1[i] = (a < alphaloci) ? (float)alphaloci
                                : (float)dmul(dadd(a, dmul(dmul(dtsph, alphaloci), tdecay1)), ddenom);
  }
}

// corrector (step_leapfrog.f90:482-560): active particles take the full
// kick to the end of their new step's first half; every particle is
// synchronised to the time of the step; a particle marked by an active
// neighbour moves to the wake bin and restarts its step there
__global__ void k_ind_correct(Params p, int n, double timei, BinDts dts, int nbinmax, const unsigned char *actf,
                              int8_t *ibin, int8_t *ibin_wake, double *twas, double *vxyzu, const double *fxyzu,
                              double *Bevol, const double *dBevol, const double *xyzh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (xyzh[4 * (size_t)i + 3] < TINY_D) return;
  double *v = vxyzu + 4 * (size_t)i;
  const double *f = fxyzu + 4 * (size_t)i;
  const int nv = p.isothermal ? 3 : 4;
  double *b = Bevol + 4 * (size_t)i;
  const double *db = dBevol + 4 * (size_t)i;
  int bi = ibin[i], bw = ibin_wake[i];
  double tw = twas[i];
  if (actf[i]) {
    bw = 0;
    const double dti = (timei - tw) + dts.t[1][bi];
    for (int k = 0; k < nv; ++k) v[k] = v[k] + dti * f[k];
    if (p.mhd) for (int k = 0; k < 4; ++k) b[k] = b[k] + dti * db[k];
    tw = tw + dti;
  }
  const double hdti = timei - tw;
  for (int k = 0; k < nv; ++k) v[k] = v[k] + hdti * f[k];
  if (p.mhd) for (int k = 0; k < 4; ++k) b[k] = b[k] + hdti * db[k];
  if (bw > bi) {
    bw = min(nbinmax, bw);
    tw = dts.t[3][bw];
    bi = bw;
    bw = 0;
  }
  ibin[i] = (int8_t)bi;
  ibin_wake[i] = (int8_t)bw;
  twas[i] = tw;
}

// init_step: twas = time + dt(ibin)/2 and, at t = 0, every particle in bin nbinmax
__global__ void k_ind_init(int n, double time, double dtmax, int nbinmax, int8_t *ibin, double *twas) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (time < TINY_D) ibin[i] = (int8_t)nbinmax;
  twas[i] = time + 0.5 * (dtmax / (double)(1ll << ibin[i]));
}

static double bin_dt(double dtmax, int b) { return dtmax / std::ldexp(1.0, b); }  // utils_indtimesteps.f90:45

}  // namespace ph

using namespace ph;

extern "C" {

int ph_ind_init(ph_ctx *c, double time) {
  if (!c) return PH_ERR_ARG;
  if (!c->dp.ind || !c->ibin) return PH_ERR_ARG;
  if (!c->have_force) return PH_ERR_STATE;
  const int n = (int)c->n;
  c->ind_dtsub = bin_dt(c->dp.dtmax, c->nbinmax);
  k_ind_init<<<nblk(n, 256), 256, 0, c->stream>>>(n, time, c->dp.dtmax, c->nbinmax, c->ibin, c->twas);
  count_launch(c);
  for (int b = 0; b <= MAXBINS; ++b) {
    c->ibin_dts[0][b] = bin_dt(c->dp.dtmax, b);
    c->ibin_dts[1][b] = 0.5 * c->ibin_dts[0][b];
    c->ibin_dts[2][b] = 1.0 / c->ibin_dts[0][b];
    c->ibin_dts[3][b] = time + 0.5 * bin_dt(c->dp.dtmax, b);
  }
  c->istepfrac = 0;
  c->ind_tlast = time;
  return check_cuda(c);
}

int ph_ind_substep(ph_ctx *c, double *time, int64_t *nactive) {
  if (!c || !time) return PH_ERR_ARG;
  if (!c->dp.ind || !c->ibin) return PH_ERR_ARG;
  if (!c->have_force) return PH_ERR_STATE;
  if (c->nbinmax > MAXBINS) return PH_ERR_IND_DT;
  cudaStream_t st = c->stream;
  const int n = (int)c->n;
  const Params p = c->dp;
  reset_timers(c);
  cudaEventRecord(c->evk[6], st);
  cudaMemsetAsync(c->d_err, 0, sizeof(int), st);
  const int nbinmaxprev = c->nbinmax;
  if (c->istepfrac + 1 > (1 << c->nbinmax)) return PH_ERR_IND;  // checked before any state changes
  c->istepfrac += 1;  // evolve.f90:206
  cudaMemsetAsync(c->d_ind + 4, 0, 2 * sizeof(int), st);
  k_set_active<<<nblk(n, 256), 256, 0, st>>>(n, c->xyzh, c->ibin, c->actf, c->nbinmax, c->istepfrac, c->d_ind + 4);
  count_launch(c);
  int hc[2] = {0, 0};
  cudaMemcpyAsync(hc, c->d_ind + 4, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return PH_ERR_CUDA;
  if (hc[1]) return PH_ERR_IND;
  if (nactive) *nactive = hc[0];
  // ibinnow: the lowest bin whose step ends on this substep
  c->ibinnow = c->nbinmax;
  for (int b = 0; c->ibinnow == c->nbinmax && b < c->nbinmax; ++b)
    if (c->istepfrac % (1 << (c->nbinmax - b)) == 0) c->ibinnow = b;
  // step_leapfrog.f90:157-163: the start of each bin's current step
  const double timei = *time, dtsph = c->ind_dtsub;
  const double time_now = timei + dtsph;
  for (int b = 0; b <= MAXBINS; ++b)
    c->ibin_dts[3][b] = ((double)(int64_t)(time_now * c->ibin_dts[2][b]) + 0.5) * c->ibin_dts[0][b];
  cudaEventRecord(c->ev[4], st);
  k_ind_predict<<<nblk(n, 256), 256, 0, st>>>(p, n, timei, dtsph, c->twas, c->ibin, c->ibin_old, c->actf, c->xyzh,
                                              c->vxyzu, c->fxyzu, c->Bevol, c->dBevol, c->divcurlv, c->vpred,
                                              c->Bpred, c->alpha1, c->alphaloc_t, c->eos, c->iperm);
  count_launch(c);
  cudaEventRecord(c->ev[5], st);
  c->ind_too_small = false;
  const double *Bv = p.mhd ? c->Bpred : c->Bevol;
  double dtn = 0.0;
  int r = derivs_dev(c, 1, c->vpred, Bv, &dtn);
  if (r) return r;
  if (c->ind_too_small) return PH_ERR_IND_DT;  // step_leapfrog.f90:427-433: fatal before the corrector
  BinDts dts;
  for (int k = 0; k < 4; ++k)
    for (int b = 0; b <= MAXBINS; ++b) dts.t[k][b] = c->ibin_dts[k][b];
  cudaEventRecord(c->ev[6], st);
  k_ind_correct<<<nblk(n, 256), 256, 0, st>>>(p, n, time_now, dts, c->nbinmax, c->actf, c->ibin, c->ibin_wake,
                                              c->twas, c->vxyzu, c->fxyzu, c->Bevol, c->dBevol, c->xyzh);
  count_launch(c);
  cudaEventRecord(c->ev[7], st);
  cudaEventRecord(c->evk[7], st);
  if (cudaEventSynchronize(c->evk[7]) != cudaSuccess) return PH_ERR_CUDA;
  float ms = 0.0f, ms2 = 0.0f;
  cudaEventElapsedTime(&ms, c->ev[4], c->ev[5]);
  cudaEventElapsedTime(&ms2, c->ev[6], c->ev[7]);
  c->last_ms[3] = ms + ms2;
  add_elapsed(c, 7, c->evk[6], c->evk[7]);
  const int e = check_cuda(c);
  if (e) return e;
  // update_time_and_dt and change_nbinmax
  *time = c->ind_tlast + (double)c->istepfrac / (double)(1 << nbinmaxprev) * p.dtmax;
  if (c->nbinmax != nbinmaxprev) {
    if (c->nbinmax < nbinmaxprev && c->istepfrac % (1 << (nbinmaxprev - c->nbinmax)) != 0) return PH_ERR_IND;
    if (c->nbinmax > nbinmaxprev) c->istepfrac = c->istepfrac * (1 << (c->nbinmax - nbinmaxprev));
    else c->istepfrac = c->istepfrac / (1 << (nbinmaxprev - c->nbinmax));
    if (c->nbinmax > MAXBINS) return PH_ERR_IND_DT;
    c->ind_dtsub = bin_dt(p.dtmax, c->nbinmax);
  }
  if (c->istepfrac == (1 << c->nbinmax)) {  // end of a dtmax interval
    c->istepfrac = 0;
    c->ind_tlast = *time;
  }
  return 0;
}

int ph_ind_state(ph_ctx *c, int8_t *ibin, double *twas, int32_t *counters) {
  if (!c) return PH_ERR_ARG;
  if (!c->dp.ind || !c->ibin) return PH_ERR_ARG;
  const size_t n = (size_t)c->n;
  if (ibin) cudaMemcpyAsync(ibin, c->ibin, n, cudaMemcpyDeviceToHost, c->stream);
  if (twas) cudaMemcpyAsync(twas, c->twas, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return PH_ERR_CUDA;
  if (counters) { counters[0] = c->nbinmax; counters[1] = c->istepfrac; counters[2] = c->ibinnow; counters[3] = 0; }
  return 0;
}

}  // extern "C"
