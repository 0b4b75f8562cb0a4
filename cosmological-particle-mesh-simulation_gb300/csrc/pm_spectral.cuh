// Spectral kernels of the Poisson solve (potential.py:7-29 of the reference):
//
//   x_r2c    real rows -> half-spectrum rows   (R2C along x, via a length-n/2 complex FFT)
//   y_pass   complex FFT along y, forward or inverse
//   z_green  forward FFT along z, multiply by the Green function, inverse FFT along z
//   x_c2r    half-spectrum rows -> real rows   (C2R along x)
//
// Every kernel is specialised for one grid size N and is persistent over a work list
// that may span many simulations of that size: a CTA finds its simulation from the
// work prefix.  Each N is instantiated in its own translation unit (pm_spectral_n.cu
// compiled with -DPM_N=<N>), so that register allocation is per size and the build
// runs in parallel.
#pragma once
#include "pm_common.cuh"
#include "pm_fft.cuh"

namespace pm {

constexpr int SP_NT = 256;          // threads per CTA of every spectral kernel
constexpr int SP_ELEMS = 8192;      // complex elements held per CTA (64 KB)

// ---------------------------------------------------------------------------------
// Per-n configuration
// ---------------------------------------------------------------------------------
__host__ __device__ constexpr int cx_rows(int n) {
  // rows of the x passes per CTA: ~SP_ELEMS complex, a multiple of 8, at most n*n
  return (SP_ELEMS / (n / 2)) / 8 * 8 > n * n ? n * n : (SP_ELEMS / (n / 2)) / 8 * 8;
}
__host__ __device__ constexpr int cline_width(int n) { return n >= 768 ? 8 : 16; }
__host__ __device__ constexpr int cline_bpc(int n) {
  return SP_ELEMS / (n * cline_width(n)) < 1 ? 1 : SP_ELEMS / (n * cline_width(n));
}
__host__ __device__ constexpr int chalf(int n) { return n / 2 + 1; }
__host__ __device__ constexpr int cbundles_per_plane(int n) {
  return (chalf(n) + cline_width(n) - 1) / cline_width(n);
}

__host__ __device__ constexpr size_t x_smem_bytes(int n) {
  return (size_t)(n / 2 + 1) * (cx_rows(n) + 1) * sizeof(float2);
}
__host__ __device__ constexpr size_t line_smem_bytes(int n) {
  return (size_t)n * cline_width(n) * cline_bpc(n) * sizeof(float2);
}

// ---------------------------------------------------------------------------------
// x_r2c
// ---------------------------------------------------------------------------------
template <int N>
__device__ __forceinline__ void x_r2c_body(const Sim& S, int unit, float2* s) {
  constexpr int M = N / 2, NR = cx_rows(N), LS = NR + 1;
  constexpr int NT = SP_NT;
  const long long nrows = (long long)N * N;
  const long long row0 = (long long)unit * NR;
  const float2* __restrict__ src = reinterpret_cast<const float2*>(S.rho);
  // load NR rows of M complex (pairs of reals), transposed into s[j][r]
  constexpr int NU = NR * M;
  constexpr int KU = (NU + NT - 1) / NT;
  float2 buf[KU];
#pragma unroll
  for (int k = 0; k < KU; ++k) {
    const int u = threadIdx.x + k * NT;
    const int r = u / M, j = u % M;
    buf[k] = make_float2(0.f, 0.f);
    if ((NU % NT == 0 || u < NU) && row0 + r < nrows) buf[k] = __ldg(&src[(row0 + r) * M + j]);
  }
#pragma unroll
  for (int k = 0; k < KU; ++k) {
    const int u = threadIdx.x + k * NT;
    if (NU % NT == 0 || u < NU) s[(u % M) * LS + u / M] = buf[k];
  }
  __syncthreads();
  fft_lines<M, NR, LS, NT, false>(s, S.tw, 2);
  // untangle: X[k] = E[k] + W^k O[k], k = 0..M
  float2* __restrict__ dst = S.spec;
  const int P = S.pitch;
  for (int u = threadIdx.x; u < NR * (M + 1); u += NT) {
    const int r = u / (M + 1), k = u % (M + 1);
    if (row0 + r >= nrows) continue;
    const float2 zk = s[(k == M ? 0 : k) * LS + r];
    const float2 zc = conjf2(s[(k == 0 ? 0 : M - k) * LS + r]);
    const float2 e = cscale(cadd(zk, zc), 0.5f);
    const float2 o = cscale(mul_mi<false>(csub(zk, zc)), 0.5f);
    const float2 w = __ldg(&S.tw[k]);
    dst[(row0 + r) * P + k] = cadd(e, cmul(w, o));
  }
}

template <int N>
__global__ void __launch_bounds__(SP_NT) k_x_r2c(const Sim* __restrict__ sims, Work w) {
  extern __shared__ float4 smem_f4[];
  float2* s = reinterpret_cast<float2*>(smem_f4);
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    x_r2c_body<N>(sims[si], unit - __ldg(&w.prefix[si]), s);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// x_c2r
// ---------------------------------------------------------------------------------
template <int N>
__device__ __forceinline__ void x_c2r_body(const Sim& S, int unit, float2* s) {
  constexpr int M = N / 2, NR = cx_rows(N), LS = NR + 1;
  constexpr int NT = SP_NT;
  const long long nrows = (long long)N * N;
  const long long row0 = (long long)unit * NR;
  const float2* __restrict__ src = S.spec;
  const int P = S.pitch;
  constexpr int NU = NR * (M + 1);
  constexpr int KU = (NU + NT - 1) / NT;
  float2 buf[KU];
#pragma unroll
  for (int k = 0; k < KU; ++k) {
    const int u = threadIdx.x + k * NT;
    const int r = u / (M + 1), j = u % (M + 1);
    buf[k] = make_float2(0.f, 0.f);
    if ((NU % NT == 0 || u < NU) && row0 + r < nrows) buf[k] = __ldg(&src[(row0 + r) * P + j]);
  }
#pragma unroll
  for (int k = 0; k < KU; ++k) {
    const int u = threadIdx.x + k * NT;
    if (NU % NT == 0 || u < NU) s[(u % (M + 1)) * LS + u / (M + 1)] = buf[k];
  }
  __syncthreads();
  // tangle: Z[k] = (X[k] + X*[M-k]) + i W^-k (X[k] - X*[M-k]), handled in pairs (k, M-k)
  for (int u = threadIdx.x; u < NR * (M / 2 + 1); u += NT) {
    const int r = u / (M / 2 + 1), k = u % (M / 2 + 1);
    const float2 xk = s[k * LS + r];
    const float2 xm = s[(M - k) * LS + r];
    const float2 a = cadd(xk, conjf2(xm));
    const float2 b = csub(xk, conjf2(xm));
    const float2 w = __ldg(&S.tw[k]);
    const float2 t = cmul(conjf2(w), b);
    const float2 zk = make_float2(a.x - t.y, a.y + t.x);  // a + i t
    s[k * LS + r] = zk;
    if (k != 0 && 2 * k != M) {
      const float2 t2 = cmul(w, conjf2(b));
      s[(M - k) * LS + r] = make_float2(a.x - t2.y, -a.y + t2.x);  // conj(a) + i t2
    }
  }
  __syncthreads();
  fft_lines<M, NR, LS, NT, true>(s, S.tw, 2);
  float2* __restrict__ dst = reinterpret_cast<float2*>(S.phi);
  for (int u = threadIdx.x; u < NR * M; u += NT) {
    const int r = u / M, j = u % M;
    if (row0 + r < nrows) dst[(row0 + r) * M + j] = s[j * LS + r];
  }
}

template <int N>
__global__ void __launch_bounds__(SP_NT) k_x_c2r(const Sim* __restrict__ sims, Work w) {
  extern __shared__ float4 smem_f4[];
  float2* s = reinterpret_cast<float2*>(smem_f4);
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    x_c2r_body<N>(sims[si], unit - __ldg(&w.prefix[si]), s);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// line passes (y, and z with the Green multiply)
// ---------------------------------------------------------------------------------
// Bundles are BW consecutive kx of one plane; plane = z for the y pass, y for the z pass.
template <int N, bool ZAXIS>
__device__ __forceinline__ void load_bundles(const Sim& S, int unit, float2* s) {
  constexpr int BW = cline_width(N), BPC = cline_bpc(N), NL = BW * BPC, LS = NL;
  constexpr int W = chalf(N), NBP = cbundles_per_plane(N);
  constexpr int U = BW / 2;              // float4 units per bundle row
  constexpr int NU = BPC * N * U;
  constexpr int NT = SP_NT;
  constexpr int KU = (NU + NT - 1) / NT;
  const long long P = S.pitch;
  const long long es = ZAXIS ? (long long)N * P : P;
  const long long ps = ZAXIS ? P : (long long)N * P;
  const int nb = N * NBP;
  const float2* __restrict__ src = S.spec;
  float4 buf[KU];
#pragma unroll
  for (int k = 0; k < KU; ++k) {
    const int u = threadIdx.x + k * NT;
    const int i = u / (N * U), rem = u % (N * U);
    const int j = rem / U, c = (rem % U) * 2;
    const int b = unit * BPC + i;
    buf[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    if ((NU % NT == 0 || u < NU) && b < nb) {
      const int plane = b / NBP, kx0 = (b % NBP) * BW;
      if (kx0 + c < W) {
        buf[k] = __ldg(reinterpret_cast<const float4*>(src + plane * ps + j * es + kx0 + c));
        if (kx0 + c + 1 >= W) { buf[k].z = 0.f; buf[k].w = 0.f; }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < KU; ++k) {
    const int u = threadIdx.x + k * NT;
    if (NU % NT == 0 || u < NU) {
      const int i = u / (N * U), rem = u % (N * U);
      const int j = rem / U, c = (rem % U) * 2;
      *reinterpret_cast<float4*>(&s[j * LS + i * BW + c]) = buf[k];
    }
  }
}

template <int N, bool ZAXIS>
__device__ __forceinline__ void store_bundles(const Sim& S, int unit, const float2* s) {
  constexpr int BW = cline_width(N), BPC = cline_bpc(N), NL = BW * BPC, LS = NL;
  constexpr int W = chalf(N), NBP = cbundles_per_plane(N);
  constexpr int U = BW / 2;
  constexpr int NU = BPC * N * U;
  constexpr int NT = SP_NT;
  const long long P = S.pitch;
  const long long es = ZAXIS ? (long long)N * P : P;
  const long long ps = ZAXIS ? P : (long long)N * P;
  const int nb = N * NBP;
  float2* __restrict__ dst = S.spec;
  for (int u = threadIdx.x; u < NU; u += NT) {
    const int i = u / (N * U), rem = u % (N * U);
    const int j = rem / U, c = (rem % U) * 2;
    const int b = unit * BPC + i;
    if (b >= nb) continue;
    const int plane = b / NBP, kx0 = (b % NBP) * BW;
    if (kx0 + c < W)
      *reinterpret_cast<float4*>(dst + plane * ps + j * es + kx0 + c) =
          *reinterpret_cast<const float4*>(&s[j * LS + i * BW + c]);
  }
}

template <int N, bool INV>
__device__ __forceinline__ void y_body(const Sim& S, int unit, float2* s) {
  constexpr int NL = cline_width(N) * cline_bpc(N);
  load_bundles<N, false>(S, unit, s);
  __syncthreads();
  fft_lines<N, NL, NL, SP_NT, INV>(s, S.tw, 1);
  store_bundles<N, false>(S, unit, s);
}

template <int N, bool INV>
__global__ void __launch_bounds__(SP_NT) k_y_pass(const Sim* __restrict__ sims, Work w) {
  extern __shared__ float4 smem_f4[];
  float2* s = reinterpret_cast<float2*>(smem_f4);
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    y_body<N, INV>(sims[si], unit - __ldg(&w.prefix[si]), s);
    __syncthreads();
  }
}

// Green function of potential.py:15 / fourier_utils.py:15-16 (k = 0 -> 0), including
// the 1/n^3 of the unnormalised inverse transforms (folded into S.green).
template <int N, bool TABLE>
__device__ __forceinline__ void z_body(const Sim& S, int unit, float2* s) {
  constexpr int BW = cline_width(N), BPC = cline_bpc(N), NL = BW * BPC;
  constexpr int NBP = cbundles_per_plane(N), W = chalf(N);
  load_bundles<N, true>(S, unit, s);
  __syncthreads();
  fft_lines<N, NL, NL, SP_NT, false>(s, S.tw, 1);
  const float g0 = S.green;
  const float* __restrict__ s2 = S.s2;
  for (int e = threadIdx.x; e < N * NL; e += SP_NT) {
    const int kz = e / NL, line = e % NL;
    const int i = line / BW, c = line % BW;
    const int b = unit * BPC + i;
    const int ky = b / NBP, kx = (b % NBP) * BW + c;
    float g = 0.f;
    if (kx < W && ky < N) {
      if (TABLE) {
        g = g0 * __ldg(&S.fgrid[((long long)kz * N + ky) * N + kx]);
      } else if ((kx | ky | kz) != 0) {
        const float den = __ldg(&s2[kx]) + __ldg(&s2[ky]) + __ldg(&s2[kz]);
        g = __fdividef(g0, den);
      }
    }
    const float2 v = s[e];
    s[e] = make_float2(v.x * g, v.y * g);
  }
  __syncthreads();
  fft_lines<N, NL, NL, SP_NT, true>(s, S.tw, 1);
  store_bundles<N, true>(S, unit, s);
}

template <int N, bool TABLE>
__global__ void __launch_bounds__(SP_NT) k_z_green(const Sim* __restrict__ sims, Work w) {
  extern __shared__ float4 smem_f4[];
  float2* s = reinterpret_cast<float2*>(smem_f4);
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    z_body<N, TABLE>(sims[si], unit - __ldg(&w.prefix[si]), s);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// per-N launcher (explicitly instantiated once per N in pm_spectral_n.cu)
// ---------------------------------------------------------------------------------
template <int N>
cudaError_t spectral_launch(SpecKind kind, const Sim* sims, Work w, int ctas, cudaStream_t st) {
  static bool init = false;
  const size_t xs = x_smem_bytes(N), ls = line_smem_bytes(N);
  if (!init) {
    cudaError_t e = cudaFuncSetAttribute(k_x_r2c<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xs);
    if (!e) e = cudaFuncSetAttribute(k_x_c2r<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xs);
    if (!e) e = cudaFuncSetAttribute(k_y_pass<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ls);
    if (!e) e = cudaFuncSetAttribute(k_y_pass<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ls);
    if (!e) e = cudaFuncSetAttribute(k_z_green<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ls);
    if (!e) e = cudaFuncSetAttribute(k_z_green<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ls);
    if (e) return e;
    init = true;
  }
  switch (kind) {
    case SPEC_PREPARE: return cudaSuccess;
    case SPEC_X_R2C: k_x_r2c<N><<<ctas, SP_NT, xs, st>>>(sims, w); break;
    case SPEC_X_C2R: k_x_c2r<N><<<ctas, SP_NT, xs, st>>>(sims, w); break;
    case SPEC_Y_FWD: k_y_pass<N, false><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    case SPEC_Y_INV: k_y_pass<N, true><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    case SPEC_Z_GREEN: k_z_green<N, false><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    case SPEC_Z_TABLE: k_z_green<N, true><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace pm
