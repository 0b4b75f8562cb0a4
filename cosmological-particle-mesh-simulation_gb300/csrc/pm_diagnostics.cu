// Diagnostics of a density grid: the slab projection of plot_helper.py:65-72 and the matter
// power spectrum.
//
// Power spectrum, from the grid's half spectrum: shell-averaged
// P(k) = <|delta_k|^2> box^3 / n^6 in integer shells of |m| (m: mode index), delta = rho /
// mean(rho) - 1.  The reference has no estimator; this one has the binning of the oracle's
// power_spectrum: bin b = floor(|m| + 0.5) for 0 < b < nbins, modes with 0 < kx < n/2
// weighted 2 (they stand for the mirrored half of the full spectrum).
//
// Deterministic: the grid of CTAs is fixed; a warp walks rows of kx, where the bin is
// non-decreasing along the row, so equal bins are contiguous lanes and a segmented
// shuffle scan sums them in lane order; each warp owns its bins in shared memory, the CTA
// adds its warps in order, and the last kernel adds the CTAs in order.
#include "pm_common.cuh"

namespace pm {

namespace {

constexpr int PK_NT = 256;
constexpr int PK_WARPS = PK_NT / 32;

__device__ __forceinline__ int pk_freq(int m, int n) { return m < n / 2 ? m : m - n; }

// per-CTA partial sums: partial[(cta * 3 + q) * nbins + b], q = 0: sum w |X|^2, 1: sum w |m|, 2: sum w
__global__ void __launch_bounds__(PK_NT) k_pk_bins(const float2* __restrict__ spec, int n, int pitch, int nbins,
                                                     double* __restrict__ partial) {
  extern __shared__ double pk_sm[];  // [PK_WARPS][3][nbins]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < PK_WARPS * 3 * nbins; i += PK_NT) pk_sm[i] = 0.0;
  __syncthreads();
  double* mine = pk_sm + (size_t)warp * 3 * nbins;
  const int w = n / 2 + 1;
  const long long rows = (long long)n * n;
  const long long gw = (long long)blockIdx.x * PK_WARPS + warp, nw = (long long)gridDim.x * PK_WARPS;
  for (long long r = gw; r < rows; r += nw) {
    const int ky = (int)(r % n), kz = (int)(r / n);
    const int fy = pk_freq(ky, n), fz = pk_freq(kz, n);
    const int base = fy * fy + fz * fz;
    if (base >= nbins * nbins) continue;  // the whole row lies outside the last shell
    const float2* row = spec + r * pitch;
    for (int x0 = 0; x0 < w; x0 += 32) {
      const int kx = x0 + lane;
      int b = nbins;  // sentinel: not binned
      double p = 0.0, m = 0.0, c = 0.0;
      if (kx < w) {
        const int m2 = base + kx * kx;
        const double mm = sqrt((double)m2);
        const int bb = (int)floor(mm + 0.5);
        if (bb > 0 && bb < nbins) {
          const float2 v = __ldg(&row[kx]);
          const double wt = (kx == 0 || 2 * kx == n) ? 1.0 : 2.0;
          b = bb;
          p = wt * ((double)v.x * v.x + (double)v.y * v.y);
          m = wt * mm;
          c = wt;
        }
      }
      // segmented inclusive scan over equal, contiguous bins (lane order)
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int bu = __shfl_up_sync(0xffffffffu, b, o);
        const double pu = __shfl_up_sync(0xffffffffu, p, o);
        const double mu = __shfl_up_sync(0xffffffffu, m, o);
        const double cu = __shfl_up_sync(0xffffffffu, c, o);
        if (lane >= o && bu == b) {
          p += pu;
          m += mu;
          c += cu;
        }
      }
      const int bn = __shfl_down_sync(0xffffffffu, b, 1);
      if (b < nbins && (lane == 31 || bn != b)) {  // last lane of its segment
        mine[b] += p;
        mine[nbins + b] += m;
        mine[2 * nbins + b] += c;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 3 * nbins; i += PK_NT) {
    double t = 0.0;
    for (int k = 0; k < PK_WARPS; ++k) t += pk_sm[(size_t)k * 3 * nbins + i];
    partial[(size_t)blockIdx.x * 3 * nbins + i] = t;
  }
}

// out[b] = (k_b, P_b, modes_b) for b = 1 .. nbins - 1 (row-major, 3 per bin)
__global__ void k_pk_final(const double* __restrict__ partial, int ctas, int nbins, const float2* __restrict__ spec,
                           int n, double box, double* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (b >= nbins) return;
  double p = 0.0, m = 0.0, c = 0.0;
  for (int k = 0; k < ctas; ++k) {
    const double* q = partial + (size_t)k * 3 * nbins;
    p += q[b];
    m += q[nbins + b];
    c += q[2 * nbins + b];
  }
  const double n3 = (double)n * n * n;
  const double mean = (double)spec[0].x / n3;  // the k = 0 mode is the sum of the grid
  const double scale = box * box * box / (n3 * n3) / (mean * mean);
  double* o = out + 3 * (b - 1);
  o[0] = c > 0.0 ? m / c * 2.0 * M_PI / box : NAN;
  o[1] = c > 0.0 ? p / c * scale : NAN;
  o[2] = c;
}

// plot_helper.py:65-72: out[y][x] = sum over i < n_slices of rho[i][y][x], in float64 and
// in plane order (as the reference's loop).  One thread per (y, x): reads are coalesced.
__global__ void k_project(const float* __restrict__ rho, int n, int n_slices, double* __restrict__ out) {
  const long long plane = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < plane;
       e += (long long)gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int i = 0; i < n_slices; ++i) t += (double)__ldg(&rho[i * plane + e]);
    out[e] = t;
  }
}

}  // namespace

cudaError_t launch_project(const float* rho, int n, int n_slices, double* out, int ctas, cudaStream_t st) {
  k_project<<<ctas, 256, 0, st>>>(rho, n, n_slices, out);
  return cudaGetLastError();
}

int pk_ctas() { return 256; }

size_t pk_partial_doubles(int nbins) { return (size_t)pk_ctas() * 3 * nbins; }

cudaError_t launch_power_spectrum(const float2* spec, int n, int pitch, int nbins, double box, double* partial,
                                  double* out, cudaStream_t st) {
  const size_t sm = (size_t)PK_WARPS * 3 * nbins * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(k_pk_bins, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e) return e;
  k_pk_bins<<<pk_ctas(), PK_NT, sm, st>>>(spec, n, pitch, nbins, partial);
  e = cudaGetLastError();
  if (e) return e;
  k_pk_final<<<(nbins + 127) / 128, 128, 0, st>>>(partial, pk_ctas(), nbins, spec, n, box, out);
  return cudaGetLastError();
}

}  // namespace pm
