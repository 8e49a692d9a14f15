// ph_conservation_noalloc: the conservation sums of ph_conservation for a
// caller that owns every device array and cannot let the library allocate.
//
// Who needs it: a host code that keeps its particle arrays on the device in
// its own allocator (an OpenACC or CUDA Fortran build of the particle arrays,
// or a code that reserves almost all HBM for itself at start-up) and wants the
// momentum and energy diagnostics of that state without creating a context.
// ph_init allocates every buffer of a context with cudaMalloc, and cudaMalloc
// and cudaFree also synchronise the whole device, which such a caller cannot
// accept in the middle of a step that overlaps work on several streams.
//
// The reduction needs scratch for one row of eight partial sums per block of
// 256 particles. Here that scratch is a fixed array in the library's own
// device image, so the call itself allocates nothing: no cudaMalloc, no
// cudaFree, no allocating library routine.
#include <cuda_runtime.h>

#include "phantom_gb300.h"
#include "ph_common.cuh"

namespace ph {

// the conservation reduction kernels (defined with ph_conservation)
__global__ void __launch_bounds__(256) k_conserve(Params p, int n, const double *xyzh, const double *vxyzu,
                                                  const double *fxyzu, const double *Bevol, const float *poten,
                                                  double *part, int vs);
__global__ void k_sum_partials(const double *part, int nb, int stride, int nk, int nmax, double *out);

}  // namespace ph

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_MAX_BLOCKS = PH_NOALLOC_MAX_PARTICLES / NA_THREADS;  // 16384 blocks

// The scratch: 8 partial sums per block, 1 MiB. Every GPU that loads this
// library holds it until the process exits. In host code this name is only a
// stand-in for the symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double na_partials[NA_MAX_BLOCKS * 8];

// Device address of na_partials on the current device. The first call on a
// device also loads the library's device image there (lazy module loading),
// which is why that first call must come before any stream capture. The
// address is looked up again on every call (a lookup, no allocation): after a
// cudaDeviceReset the image is loaded anew, possibly at another address, and
// a cached pointer would then point at freed memory.
int na_scratch(double **out) {
  double *ptr = nullptr;
  if (cudaGetSymbolAddress((void **)&ptr, na_partials) != cudaSuccess || !ptr) return PH_ERR_CUDA;
  *out = ptr;
  return 0;
}

}  // namespace

extern "C" {

int ph_conservation_noalloc(const ph_params *params, int64_t npart, const double *xyzh, const double *vxyzu,
                            const double *fxyzu, const double *Bevol, const float *poten, double *out,
                            void *stream) {
  if (!params || !xyzh || !vxyzu || !fxyzu || !out) return PH_ERR_ARG;
  if (params->mhd && !Bevol) return PH_ERR_ARG;
  if (params->gravity && !poten) return PH_ERR_ARG;
  if (!(params->maxvxyzu == 0 || params->maxvxyzu == 4 || (params->maxvxyzu == 3 && params->isothermal)))
    return PH_ERR_ARG;
  if (npart < 1) return PH_ERR_NOPART;
  if (npart > PH_NOALLOC_MAX_PARTICLES) return PH_ERR_SCRATCH_LIMIT;
  // an error the caller's own earlier work left pending is theirs: report
  // it without clearing it, and launch nothing
  if (cudaPeekAtLastError() != cudaSuccess) return PH_ERR_CUDA;
  double *part = nullptr;
  if (int e = na_scratch(&part)) return e;
  const ph::Params p = ph::make_params(*params);
  const int n = (int)npart;
  // one thread per particle; every block writes all 8 of its partial sums, so
  // the rows left by an earlier call are never read and need no clearing
  const int nb = (n + NA_THREADS - 1) / NA_THREADS;
  cudaStream_t st = (cudaStream_t)stream;
  ph::k_conserve<<<nb, NA_THREADS, 0, st>>>(p, n, xyzh, vxyzu, fxyzu, Bevol, poten, part,
                                            params->maxvxyzu == 3 ? 3 : 4);
  if (cudaGetLastError() != cudaSuccess) return PH_ERR_CUDA;
  ph::k_sum_partials<<<1, 32, 0, st>>>(part, nb, 8, 8, 0, out);
  if (cudaGetLastError() != cudaSuccess) return PH_ERR_CUDA;
  return 0;
}

}  // extern "C"
