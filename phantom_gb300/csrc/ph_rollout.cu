// Differentiation form through a multi-step rollout, resident on the device:
// K global-timestep leapfrog steps (step_leapfrog.f90:91-760 with one
// corrector pass, the reference's tolv > 1e2 branch) from the uploaded
// state, L = sum w . fxyzu of the last force evaluation, and the gradient of
// L with respect to the initial positions, velocities and thermal energies.
//
// Forward: the initial derivs, then the K steps (k_predict, derivs at the
// drifted positions with the predicted velocities, k_correct); every ckpt
// steps the state (xyzh, vxyzu, fxyzu, div v) is copied to a checkpoint in
// HBM. Reverse, segment by segment from the last checkpoint: the segment is
// recomputed from its checkpoint (the kernels are deterministic, so the
// recomputed states are the forward's bit for bit), keeping each step's
// evaluation point (drifted positions with the predicted h that the step's
// tree build and h-rho solve started from, predicted velocities); then each
// step is reversed:
//   step:    vs = v + dt/2 f,  x1 = x + dt vs,  vp = vs + dt/2 f,
//            f1 = F(x1, vp),   v1 = vs + dt/2 f1
//   reverse: f1b = fb + dt/2 vb;  (gx, gv) = F's adjoint at (x1, vp) on f1b;
//            x1b = xb + gx;  vsb = vb + gv + dt x1b;  fb <- dt/2 (gv + vsb);
//            xb <- x1b;  vb <- vsb
// and finally the initial evaluation f0 = F(x0, v0) is reversed. Neighbour
// lists and pair terms are recomputed inside each adjoint, nothing else is
// stored. The h prediction of k_predict only seeds the h-rho iteration, whose
// converged root is what is differentiated. With self-gravity the adjoint
// still starts from it (and the initial evaluation from the uploaded h): the
// node hmax of the tree built from it decides which node pairs of the walk
// are well separated, and from the converged h a few pairs would move
// between the near field and the M2L sums, another function of the
// positions. Without self-gravity the adjoint's recompute starts from the
// converged h (one density pass instead of the step's iterations; the same
// solution within tolh). Every adjoint recomputes its state from the stored
// evaluation point, so the checkpoint spacing changes no result bit.
#include "ph_internal.h"

namespace ph {

__global__ void k_predict(Params p, int n, double hdt, double dt, double *xyzh, double *vxyzu, const double *fxyzu,
                          double *Bevol, const double *dBevol, const float *divcurlv, double *vpred, double *Bpred,
                          float *alpha1, const float *alphaloc_t, const double *eos_t, const int *iperm);
__global__ void k_correct(Params p, int n, double hdt, double *vxyzu, const double *fxyzu, const double *vpred,
                          double *Bevol, const double *dBevol, const double *xyzh, double *part);
__global__ void k_sum_partials(const double *part, int nb, int stride, int nk, int nmax, double *out);

static inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }
constexpr int RO_RED_BLOCKS = 1024;

// f1b = fb + dt/2 vb (rows 0..nv-1; the u row zero without u)
__global__ void k_ro_cot(int n, int nv, double hdt, const double *fb, const double *vb, double *f1b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 4; ++k) {
    const size_t q = 4 * (size_t)i + k;
    f1b[q] = k < nv ? fb[q] + hdt * vb[q] : 0.0;
  }
}

// one step reversed after the adjoint of its evaluation (gx, gv)
__global__ void k_ro_back(int n, int nv, double dt, const double *gx, const double *gv, double *xb, double *vb,
                          double *fb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *x = xb + 4 * (size_t)i, *v = vb + 4 * (size_t)i, *f = fb + 4 * (size_t)i;
  const double *g = gx + 4 * (size_t)i, *h = gv + 4 * (size_t)i;
  const double hdt = 0.5 * dt;
  for (int k = 0; k < 3; ++k) x[k] += g[k];
  x[3] = 0.0;
  for (int k = 0; k < 4; ++k) {
    if (k >= nv) { v[k] = 0.0; f[k] = 0.0; continue; }
    double vs = v[k] + h[k];
    if (k < 3) vs += dt * x[k];
    f[k] = hdt * h[k] + hdt * vs;
    v[k] = vs;
  }
}

// MHD: the step of Bevol (B/rho, psi), the same kick as v without a drift:
// Bs = B + dt/2 dB, Bp = Bs + dt/2 dB, (f1, dB1) = F(x1, vp, Bp),
// B1 = Bs + dt/2 dB1; reversed with gB the adjoint's Bp gradient:
// Bsb = Bb + gB, dBb <- dt/2 (gB + Bsb), Bb <- Bsb. final: the initial
// evaluation, Bb += gB.
__global__ void k_ro_bfield(int n, double dt, int final, const double *gB, double *Bb, double *dBb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 4; ++k) {
    const size_t q = 4 * (size_t)i + k;
    const double bs = Bb[q] + gB[q];
    if (!final) dBb[q] = 0.5 * dt * (gB[q] + bs);
    Bb[q] = bs;
  }
}

// the initial evaluation reversed: xb += gx, vb += gv
__global__ void k_ro_final(int n, int nv, const double *gx, const double *gv, double *xb, double *vb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 3; ++k) xb[4 * (size_t)i + k] += gx[4 * (size_t)i + k];
  xb[4 * (size_t)i + 3] = 0.0;
  for (int k = 0; k < 4; ++k) vb[4 * (size_t)i + k] = k < nv ? vb[4 * (size_t)i + k] + gv[4 * (size_t)i + k] : 0.0;
}

// per-block partial sums of w . f (+ w2 . f2 when w2 is given; fixed order),
// completed by k_sum_partials
__global__ void __launch_bounds__(256) k_ro_dot(int n, const double *w, const double *f, const double *w2,
                                                const double *f2, double *part) {
  __shared__ double s[8];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int k = 0; k < 4; ++k) acc += w[4 * (size_t)i + k] * f[4 * (size_t)i + k];
    if (w2)
      for (int k = 0; k < 4; ++k) acc += w2[4 * (size_t)i + k] * f2[4 * (size_t)i + k];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane_id() == 0) s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = s[0];
    for (int k = 1; k < 8; ++k) t += s[k];
    part[blockIdx.x] = t;
  }
}

namespace {

// the device state that a checkpoint holds (b, db: Bevol and dBevol, MHD)
struct Snap {
  double *x, *v, *f, *b, *db;
  float *dv;
};

void save(ph_ctx *c, const Snap &s) {
  const size_t n = (size_t)c->n;
  cudaMemcpyAsync(s.x, c->xyzh, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(s.v, c->vxyzu, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(s.f, c->fxyzu, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(s.dv, c->divcurlv, sizeof(float) * n, cudaMemcpyDeviceToDevice, c->stream);
  if (s.b) {
    cudaMemcpyAsync(s.b, c->Bevol, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(s.db, c->dBevol, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
  }
}

void restore(ph_ctx *c, const Snap &s) {
  const size_t n = (size_t)c->n;
  cudaMemcpyAsync(c->xyzh, s.x, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(c->vxyzu, s.v, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(c->fxyzu, s.f, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
  cudaMemcpyAsync(c->divcurlv, s.dv, sizeof(float) * n, cudaMemcpyDeviceToDevice, c->stream);
  if (s.b) {
    cudaMemcpyAsync(c->Bevol, s.b, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(c->dBevol, s.db, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, c->stream);
  }
  c->have_tree = c->have_density = c->have_force_lists = false;
  c->have_force = true;
}

// one leapfrog step with one corrector pass; the evaluation point (drifted
// positions with the predicted h under self-gravity, else the converged h;
// predicted velocities and, with MHD, predicted Bevol) is copied to (x1, vp,
// bp)
int step_once(ph_ctx *c, double dt, double *part, double *x1, double *vp, double *bp) {
  const Params p = c->dp;
  const int n = (int)c->n;
  cudaStream_t st = c->stream;
  const double hdt = 0.5 * dt;
  k_predict<<<nblk(n, 256), 256, 0, st>>>(p, n, hdt, dt, c->xyzh, c->vxyzu, c->fxyzu, c->Bevol, c->dBevol,
                                          c->divcurlv, c->vpred, c->Bpred, c->alpha1, c->alphaloc_t, c->eos,
                                          c->iperm);
  count_launch(c);
  if (x1 && p.gravity) cudaMemcpyAsync(x1, c->xyzh, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
  if (vp) cudaMemcpyAsync(vp, c->vpred, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
  if (bp) cudaMemcpyAsync(bp, c->Bpred, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
  double dtn = 0.0;
  const int r = derivs_dev(c, 1, c->vpred, p.mhd ? c->Bpred : c->Bevol, &dtn);
  if (r) return r;
  if (x1 && !p.gravity) cudaMemcpyAsync(x1, c->xyzh, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
  const int nb = nblk(n, 256) < RO_RED_BLOCKS ? nblk(n, 256) : RO_RED_BLOCKS;
  k_correct<<<nb, 256, 0, st>>>(p, n, hdt, c->vxyzu, c->fxyzu, c->vpred, c->Bevol, c->dBevol, c->xyzh, part);
  count_launch(c);
  return 0;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

}  // namespace
}  // namespace ph

using namespace ph;

extern "C" {

int ph_rollout_adjoint_full(ph_ctx *c, int32_t nsteps, const double *dts, int32_t ckpt, const double *w_fxyzu,
                            const double *w_dBevol, double *loss, double *g_xyzh, double *g_vxyzu,
                            double *g_Bevol) {
  if (!c || !dts || !w_fxyzu || !g_xyzh || !g_vxyzu || nsteps < 1 || ckpt < 1) return PH_ERR_ARG;
  for (int k = 0; k < nsteps; ++k)
    if (!(dts[k] > 0.0)) return PH_ERR_ARG;
  if (c->n <= 0) return PH_ERR_NOPART;
  const Params p = c->dp;
  // the Cullen-Dehnen switch (alpha evolves with the state) and individual
  // timesteps are not built for rollouts
  if (p.nalpha > 0 || p.ind) return PH_ERR_NOT_BUILT;
  const bool mhd = p.mhd != 0;
  const size_t n = (size_t)c->n;
  const int ni = (int)n;
  const int nv = p.isothermal ? 3 : 4;
  const int ncp = (nsteps + ckpt - 1) / ckpt;
  const int seg = ckpt < nsteps ? ckpt : nsteps;
  // HBM: checkpoints (3 x 4n doubles + n floats each, 2 x 4n more with MHD),
  // the segment's evaluation points (2 x 4n each, 3 x 4n with MHD), xb, vb,
  // fb, f1b, gx, gv, w and the uploaded xyzh (8 x 4n; with MHD also Bb, dBb,
  // dB1b, gB and wB, 5 x 4n), and the reduction partials
  const size_t per_cp = (mhd ? 20 : 12) * n + (n + 1) / 2;
  const size_t per_ev = (mhd ? 12 : 8) * n;
  const size_t need = (size_t)ncp * per_cp + (size_t)seg * per_ev + (mhd ? 52 : 32) * n + 2 * RO_RED_BLOCKS + 8;
  if (alloc_rollout(c, need) != 0) return PH_ERR_CUDA;
  double *base = c->ro_buf;
  std::vector<Snap> cps(ncp);
  for (int k = 0; k < ncp; ++k) {
    double *b = base + (size_t)k * per_cp;
    cps[k] = Snap{b, b + 4 * n, b + 8 * n, mhd ? b + 12 * n : nullptr, mhd ? b + 16 * n : nullptr,
                  reinterpret_cast<float *>(b + (mhd ? 20 : 12) * n)};
  }
  double *segb = base + (size_t)ncp * per_cp;
  double *xb = segb + (size_t)seg * per_ev, *vb = xb + 4 * n, *fb = vb + 4 * n, *f1b = fb + 4 * n;
  double *gx = f1b + 4 * n, *gv = gx + 4 * n, *wd = gv + 4 * n, *x0in = wd + 4 * n, *part = x0in + 4 * n;
  double *Bb = nullptr, *dBb = nullptr, *dB1b = nullptr, *gB = nullptr, *wBd = nullptr;
  if (mhd) {
    Bb = part; dBb = Bb + 4 * n; dB1b = dBb + 4 * n; gB = dB1b + 4 * n; wBd = gB + 4 * n;
    part = wBd + 4 * n;
  }
  double *res = part + 2 * RO_RED_BLOCKS;
  cudaStream_t st = c->stream;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), st);
  reset_timers(c);
  cudaEvent_t e[6];
  for (auto &ev : e) cudaEventCreate(&ev);
  float ms_adj = 0.0f, ms_rec = 0.0f;
  int r = 0;
  copy_vrows_h2d(c, wd, w_fxyzu, n);
  if (mhd) {
    if (w_dBevol) cudaMemcpyAsync(wBd, w_dBevol, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, st);
    else cudaMemsetAsync(wBd, 0, sizeof(double) * 4 * n, st);
  }
  cudaMemcpyAsync(x0in, c->xyzh, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, st);
  // ---- forward rollout
  cudaEventRecord(e[0], st);
  double dt0 = 0.0;
  r = derivs_dev(c, 1, c->vxyzu, c->Bevol, &dt0);
  for (int m = 0; m < nsteps && !r; ++m) {
    if (m % ckpt == 0) save(c, cps[m / ckpt]);
    r = step_once(c, dts[m], part, nullptr, nullptr, nullptr);
  }
  if (!r) {
    const int nb = nblk(ni, 256) < RO_RED_BLOCKS ? nblk(ni, 256) : RO_RED_BLOCKS;
    k_ro_dot<<<nb, 256, 0, st>>>(ni, wd, c->fxyzu, mhd ? wBd : nullptr, c->dBevol, part);
    k_sum_partials<<<1, 32, 0, st>>>(part, nb, 1, 1, 0, res);
    count_launch(c, 2);
  }
  cudaEventRecord(e[1], st);
  // ---- reverse: xb = vb = 0, fb = w (Bb = 0, dBb = wB)
  if (!r) {
    cudaMemsetAsync(xb, 0, sizeof(double) * 8 * n, st);  // xb, vb
    cudaMemcpyAsync(fb, wd, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, st);
    if (mhd) {
      cudaMemsetAsync(Bb, 0, sizeof(double) * 4 * n, st);
      cudaMemcpyAsync(dBb, wBd, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, st);
    }
  }
  for (int k = ncp - 1; k >= 0 && !r; --k) {
    const int m0 = k * ckpt, m1 = m0 + ckpt < nsteps ? m0 + ckpt : nsteps;
    cudaEventRecord(e[2], st);
    restore(c, cps[k]);
    for (int m = m0; m < m1 && !r; ++m) {
      double *x1 = segb + (size_t)(m - m0) * per_ev;
      r = step_once(c, dts[m], part, x1, x1 + 4 * n, mhd ? x1 + 8 * n : nullptr);
    }
    cudaEventRecord(e[3], st);
    for (int m = m1 - 1; m >= m0 && !r; --m) {
      const double *x1 = segb + (size_t)(m - m0) * per_ev;
      k_ro_cot<<<nblk(ni, 256), 256, 0, st>>>(ni, nv, 0.5 * dts[m], fb, vb, f1b);
      count_launch(c);
      if (mhd) {
        k_ro_cot<<<nblk(ni, 256), 256, 0, st>>>(ni, 4, 0.5 * dts[m], dBb, Bb, dB1b);
        count_launch(c);
        cudaMemcpyAsync(c->Bevol, x1 + 8 * n, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, st);
      }
      cudaMemcpyAsync(c->xyzh, x1, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(c->vxyzu, x1 + 4 * n, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, st);
      c->have_tree = c->have_density = c->have_force = c->have_force_lists = false;
      r = adjoint_dev(c, f1b, mhd ? dB1b : nullptr, gx, gv, gB);
      if (r) break;
      k_ro_back<<<nblk(ni, 256), 256, 0, st>>>(ni, nv, dts[m], gx, gv, xb, vb, fb);
      count_launch(c);
      if (mhd) {
        k_ro_bfield<<<nblk(ni, 256), 256, 0, st>>>(ni, dts[m], 0, gB, Bb, dBb);
        count_launch(c);
      }
    }
    cudaEventRecord(e[4], st);
    if (cudaEventSynchronize(e[4]) != cudaSuccess) r = PH_ERR_CUDA;
    ms_rec += elapsed(e[2], e[3]);
    ms_adj += elapsed(e[3], e[4]);
  }
  // the initial evaluation, then leave the context at the initial state
  // with its forces (as after ph_derivs)
  if (!r) {
    cudaEventRecord(e[2], st);
    restore(c, cps[0]);
    if (p.gravity) cudaMemcpyAsync(c->xyzh, x0in, sizeof(double) * 4 * n, cudaMemcpyDeviceToDevice, st);
    c->have_force = false;
    r = adjoint_dev(c, fb, mhd ? dBb : nullptr, gx, gv, gB);
    if (!r) {
      k_ro_final<<<nblk(ni, 256), 256, 0, st>>>(ni, nv, gx, gv, xb, vb);
      count_launch(c);
      if (mhd) {
        k_ro_bfield<<<nblk(ni, 256), 256, 0, st>>>(ni, 0.0, 1, gB, Bb, dBb);
        count_launch(c);
      }
      restore(c, cps[0]);
      cudaEventRecord(e[4], st);
    }
  }
  if (!r) {
    cudaMemcpyAsync(g_xyzh, xb, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, st);
    copy_vrows_d2h(c, g_vxyzu, vb, n);
    if (mhd && g_Bevol) cudaMemcpyAsync(g_Bevol, Bb, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, st);
    double L = 0.0;
    cudaMemcpyAsync(&L, res, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) r = PH_ERR_CUDA;
    if (!r && loss) *loss = L;
    if (!r) {
      ms_adj += elapsed(e[2], e[4]);
      // [0] forward rollout, [1] reverse (recomputes + adjoints), [2] the
      // adjoint evaluations and reverse updates, [3] the segment recomputes,
      // [7] total
      c->last_ms[0] = elapsed(e[0], e[1]);
      c->last_ms[1] = ms_rec + ms_adj;
      c->last_ms[2] = ms_adj;
      c->last_ms[3] = ms_rec;
      c->last_ms[7] = elapsed(e[0], e[4]);
      int herr = 0;
      cudaMemcpy(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost);
      r = herr;
    }
  }
  for (auto &ev : e) cudaEventDestroy(ev);
  if (r) c->have_tree = c->have_density = c->have_force = c->have_force_lists = false;
  return r;
}

int ph_rollout_adjoint(ph_ctx *c, int32_t nsteps, const double *dts, int32_t ckpt, const double *w_fxyzu,
                       double *loss, double *g_xyzh, double *g_vxyzu) {
  return ph_rollout_adjoint_full(c, nsteps, dts, ckpt, w_fxyzu, nullptr, loss, g_xyzh, g_vxyzu, nullptr);
}

}  // extern "C"
