// Device-wide utilities: exclusive scan of int arrays, launch bookkeeping.
#include "ph_internal.h"

namespace ph {

void count_launch(ph_ctx *c, int k) { c->launches += k; }

void add_elapsed(ph_ctx *c, int slot, cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) c->last_ms[slot] += ms;
}

void reset_timers(ph_ctx *c) {
  for (int k = 0; k < 8; ++k) c->last_ms[k] = 0.0;
  cudaMemsetAsync(c->stats + 8, 0, 8 * sizeof(unsigned long long), c->stream);
}

cudaError_t check_launch(ph_ctx *c) {
  (void)c;
  return cudaGetLastError();
}

constexpr int SCAN_B = 1024;

// per-block inclusive scan of 1024 elements (one per thread); block totals out
__global__ void __launch_bounds__(SCAN_B) k_scan_block(const int *in, int *out, int n, int *bsum) {
  __shared__ int s[32];
  int i = blockIdx.x * SCAN_B + threadIdx.x;
  int v = (i < n) ? in[i] : 0;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = s[lane];
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    s[lane] = t;
  }
  __syncthreads();
  int incl = x + (w > 0 ? s[w - 1] : 0);
  if (i < n) out[i] = incl - v;  // exclusive
  if (threadIdx.x == SCAN_B - 1) bsum[blockIdx.x] = incl;
}

__global__ void k_scan_add(int *out, int n, const int *boff) {
  int i = blockIdx.x * SCAN_B + threadIdx.x;
  if (i < n && blockIdx.x > 0) out[i] += boff[blockIdx.x];
}

__global__ void k_scan_total(const int *in, const int *out, int n, int *total) {
  if (n > 0) *total = out[n - 1] + in[n - 1];
  else *total = 0;
}

// recursive exclusive scan using ctx scratch (scan_tmp holds block sums)
static void scan_rec(ph_ctx *c, const int *in, int *out, int n, int *tmp) {
  int nb = (n + SCAN_B - 1) / SCAN_B;
  int *bsum = tmp;
  k_scan_block<<<nb, SCAN_B, 0, c->stream>>>(in, out, n, bsum);
  count_launch(c);
  if (nb > 1) {
    int *boff = tmp + nb;
    scan_rec(c, bsum, boff, nb, tmp + 2 * nb);
    k_scan_add<<<nb, SCAN_B, 0, c->stream>>>(out, n, boff);
    count_launch(c);
  }
}

void scan_int(ph_ctx *c, const int *in, int *out, int n, int *d_total) {
  if (n <= 0) {
    if (d_total) cudaMemsetAsync(d_total, 0, sizeof(int), c->stream);
    return;
  }
  // keep the last input value for the total (out may alias in)
  int *last = c->scan_tmp;
  cudaMemcpyAsync(last, in + (n - 1), sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
  scan_rec(c, in, out, n, c->scan_tmp + 1);
  if (d_total) {
    k_scan_total<<<1, 1, 0, c->stream>>>(last, out + (n - 1), 1, d_total);
    count_launch(c);
  }
}

__global__ void k_fill_int_u(int *a, int n, int v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

void fill_int(ph_ctx *c, int *a, int n, int v) {
  if (n <= 0) return;
  k_fill_int_u<<<(n + 255) / 256, 256, 0, c->stream>>>(a, n, v);
  count_launch(c);
}

}  // namespace ph
