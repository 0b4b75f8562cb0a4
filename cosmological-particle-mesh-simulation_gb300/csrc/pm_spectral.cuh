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
#include <cudaTypedefs.h>

#include "pm_common.cuh"
#include "pm_deposit.cuh"
#include "pm_fft.cuh"
#include "pm_tma.cuh"

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
// Line passes of the 512 and 384 grids run two CTAs per SM, each with 32 / 24 KB TMA
// stages of bundles 8 columns wide; the others one CTA with 64 KB stages (measured: 8-wide
// bundles slow the 256 grid's z pass 0.34 -> 0.41 ms and the 192 grid's 0.50 -> 0.52 ms).
__host__ __device__ constexpr bool line_small(int n) { return n == 512 || n == 384; }
// columns of a line-pass bundle
__host__ __device__ constexpr int cline_width(int n) { return n >= 512 || line_small(n) ? 8 : 16; }
// bundles per unit (per TMA stage)
__host__ __device__ constexpr int cline_bpc(int n) {
  return line_small(n) ? SP_ELEMS / 2 / (n * 8)
                       : (SP_ELEMS / (n * cline_width(n)) < 1 ? 1 : SP_ELEMS / (n * cline_width(n)));
}
__host__ __device__ constexpr int chalf(int n) { return n / 2 + 1; }
__host__ __device__ constexpr int cbundles_per_plane(int n) {
  return (chalf(n) + cline_width(n) - 1) / cline_width(n);
}

__host__ __device__ constexpr int cpitch(int n) { return (chalf(n) + 15) / 16 * 16; }
// Line passes that stream through a TMA ring: boxes of at most 256 rows tiling n.
__host__ __device__ constexpr int line_box_rows(int n) { return n <= 256 ? n : (n % 256 == 0 ? 256 : n / 2); }
__host__ __device__ constexpr bool tma_lines(int n) { return n >= 32 && line_box_rows(n) <= 256; }
// Threads of a line-pass CTA: 512 (up to 128 registers), 256 for the two-CTA sizes; 768,
// transformed line by line, runs 1024.
__host__ __device__ constexpr int line_nt(int n) { return line_small(n) ? 256 : (n == 768 ? 1024 : 512); }
__host__ __device__ constexpr int line_ctas_per_sm(int n) { return line_small(n) ? 2 : 1; }
constexpr int XTMA_NT = 1024;  // x passes
constexpr int TMA_STAGES = 3;
__host__ __device__ constexpr size_t tma_stage_bytes(int n) {
  return (size_t)n * cline_width(n) * cline_bpc(n) * sizeof(float2);
}
__host__ __device__ constexpr size_t tma_smem_bytes(int n) { return TMA_STAGES * tma_stage_bytes(n) + 64; }

// x passes with the row transform in registers (power-of-two n, 64 <= n <= 512): a row of
// M = n/2 complex points is factored M = P x Q and held by T lanes of a warp
// (n: P x Q, T) -- 64: 8x4, 4; 128: 8x8, 8; 256: 16x8, 8; 512: 16x16, 16;
// 96: 4x12, 4; 192: 8x12, 4; 384: 8x24, 8
__host__ __device__ constexpr bool xrow_ok(int n) {
  return n == 64 || n == 128 || n == 256 || n == 512 || n == 96 || n == 192 || n == 384;
}
// (the radix-3 rows with the smaller factor first: x C2R per 134M cells 96: 0.119 -> 0.115,
// 192: 0.315 -> 0.257, 384: 0.269 -> 0.256 ms)
__host__ __device__ constexpr int xrow_P(int n) {
  return n % 3 == 0 ? (n == 96 ? 4 : 8) : (n >= 256 ? 16 : 8);
}
__host__ __device__ constexpr int xrow_Q(int n) { return n / 2 / xrow_P(n); }
__host__ __device__ constexpr int xrow_T(int n) {
  return n == 192 ? 4 : (xrow_Q(n) < xrow_P(n) ? xrow_Q(n) : xrow_P(n));
}
__host__ __device__ constexpr int xrow_rows_per_warp(int n) { return 32 / xrow_T(n); }
// threads of a row-transform CTA: up to 8 warps, their exchange buffers within 40 KB of
// static shared memory
__host__ __device__ constexpr int xrow_warp_bytes(int n) {
  return xrow_rows_per_warp(n) * xrow_Q(n) * (xrow_P(n) + 1) * 8;
}
__host__ __device__ constexpr int xrow_nt(int n) {
  return 32 * (40960 / xrow_warp_bytes(n) < 8 ? (40960 / xrow_warp_bytes(n) < 1 ? 1 : 40960 / xrow_warp_bytes(n)) : 8);
}

// x passes fed by bulk copies into a double-buffered staging area (one simulation per launch)
__host__ __device__ constexpr bool tma_rows(int n);
__host__ __device__ constexpr int xrow_stage_floats(int n) { return n + 4; }  // (n/2 + 2) complex: bulk size % 16 == 0
__host__ __device__ constexpr size_t xtma_fft_bytes(int n);
__host__ __device__ constexpr size_t xtma_smem_bytes(int n);

__host__ __device__ constexpr size_t x_smem_bytes(int n) {
  return (size_t)(n / 2 + 1) * (cx_rows(n) + 1) * sizeof(float2);
}
__host__ __device__ constexpr size_t line_smem_bytes(int n) {
  return (size_t)n * cline_width(n) * cline_bpc(n) * sizeof(float2);
}
__host__ __device__ constexpr size_t xtma_fft_bytes(int n) { return x_smem_bytes(n); }
// two staging buffers of cx_rows(n) rows x (n + 4) floats, the FFT buffer, two mbarriers
__host__ __device__ constexpr size_t xtma_smem_bytes(int n) {
  return 2 * (size_t)cx_rows(n) * xrow_stage_floats(n) * sizeof(float) + xtma_fft_bytes(n) + 64;
}
__host__ __device__ constexpr bool tma_rows(int n) { return n >= 32 && xtma_smem_bytes(n) <= 227 * 1024; }

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

// Plain transform of the bundles of one unit along y (ZAXIS false) or z.
template <int N, bool ZAXIS, bool INV>
__device__ __forceinline__ void line_body(const Sim& S, int unit, float2* s) {
  constexpr int NL = cline_width(N) * cline_bpc(N);
  load_bundles<N, ZAXIS>(S, unit, s);
  __syncthreads();
  fft_lines<N, NL, NL, SP_NT, INV>(s, S.tw, 1);
  store_bundles<N, ZAXIS>(S, unit, s);
}

template <int N, bool ZAXIS, bool INV>
__global__ void __launch_bounds__(SP_NT) k_line_pass(const Sim* __restrict__ sims, Work w) {
  extern __shared__ float4 smem_f4[];
  float2* s = reinterpret_cast<float2*>(smem_f4);
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    line_body<N, ZAXIS, INV>(sims[si], unit - __ldg(&w.prefix[si]), s);
    __syncthreads();
  }
}

// Green function of potential.py:15 / fourier_utils.py:15-16 (k = 0 -> 0), including
// the 1/n^3 of the unnormalised inverse transforms (folded into S.green).
// GRAD: the spectral gradient of axis S.grad_axis - 1 as well (times -i sin(k_d)).
template <int N, bool TABLE, bool GRAD>
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
    if (GRAD) {  // times -i sin(k_d): the spectral central difference along axis d
      const float sg =
          kx < W && ky < N ? g * __ldg(&S.sn[S.grad_axis == 1 ? kx : (S.grad_axis == 2 ? ky : kz)]) : 0.f;
      s[e] = make_float2(sg * v.y, -sg * v.x);
    } else {
      s[e] = make_float2(v.x * g, v.y * g);
    }
  }
  __syncthreads();
  fft_lines<N, NL, NL, SP_NT, true>(s, S.tw, 1);
  store_bundles<N, true>(S, unit, s);
}

template <int N, bool TABLE, bool GRAD = false>
__global__ void __launch_bounds__(SP_NT) k_z_green(const Sim* __restrict__ sims, Work w) {
  extern __shared__ float4 smem_f4[];
  float2* s = reinterpret_cast<float2*>(smem_f4);
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    z_body<N, TABLE, GRAD>(sims[si], unit - __ldg(&w.prefix[si]), s);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// TMA-streamed line pass (y forward / y inverse / z Green) over one or many simulations.
//
// Persistent CTA with a 3-stage shared-memory ring.  A unit is BPC bundles of one
// simulation; a bundle is BW consecutive kx of one plane, loaded as N / BOX TMA boxes of
// {2 BW floats, BOX rows} with the simulation's tensor map (maps[2 s] for y, maps[2 s + 1]
// for z, in device memory).  One elected thread issues the loads of unit i+1 while all
// threads transform unit i; finished bundles leave by TMA bulk store, and a stage is
// refilled only once the store issued from it two iterations earlier has finished
// reading it.  Stages hold the bundles blocked (Blocked layout of pm_fft.cuh).
// ---------------------------------------------------------------------------------
// Green function of potential.py:15 / fourier_utils.py:15-16 (k = 0 -> 0; the 1/n^3 of the
// unnormalised inverse transforms is folded into g0) for element kz of line `line` of a unit
// of the z pass whose first bundle is b0.
template <int N, bool TABLE, bool GRAD = false>
struct GreenEpi {
  float g0;
  const float* s2;
  const float* fgrid;
  int b0, cnt;
  const float* sn;  // GRAD, the spectral gradient of axis grad_axis - 1: times -i sin(k_d) as well
  int grad_axis;
  __device__ __forceinline__ float2 operator()(float2 v, int kz, int line) const {
    constexpr int BW = cline_width(N), NBP = cbundles_per_plane(N), W = chalf(N);
    const int i = line / BW, b = b0 + i;
    const int ky = b / NBP, kx = (b % NBP) * BW + line % BW;
    float g = 0.f;
    if (i < cnt && kx < W) {
      if (TABLE) g = g0 * __ldg(&fgrid[((long long)kz * N + ky) * N + kx]);
      else if ((kx | ky | kz) != 0) g = __fdividef(g0, __ldg(&s2[kx]) + __ldg(&s2[ky]) + __ldg(&s2[kz]));
    }
    if (GRAD) {
      const float sg = i < cnt && kx < W ? g * __ldg(&sn[grad_axis == 1 ? kx : (grad_axis == 2 ? ky : kz)]) : 0.f;
      return make_float2(sg * v.y, -sg * v.x);
    }
    return make_float2(v.x * g, v.y * g);
  }
};

// MODE 0: y forward, 1: y inverse, 2: z Green, 3: z Green (caller table), 4: z forward, 5: z inverse,
// 6: z Green times -i sin(k_d) (spectral gradient of axis S.grad_axis - 1)
template <int N, int MODE>
__global__ void __launch_bounds__(line_nt(N), line_ctas_per_sm(N)) k_line_tma(const CUtensorMap* __restrict__ maps,
                                                        const Sim* __restrict__ sims, Work w, int* err) {
  constexpr int BW = cline_width(N), BPC = cline_bpc(N), NL = BW * BPC;
  constexpr int BOX = line_box_rows(N), NBOX = N / BOX;
  constexpr int NBP = cbundles_per_plane(N), W = chalf(N), NB = N * NBP;
  constexpr unsigned STAGE = (unsigned)tma_stage_bytes(N);
  constexpr unsigned BUNDLE = (unsigned)N * BW * sizeof(float2);
  constexpr bool ZAX = MODE >= 2;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float2* stg0 = reinterpret_cast<float2*>(smem_raw);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + TMA_STAGES * STAGE);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < TMA_STAGES; ++i) mbar_init(&bar[i], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto stage_ptr = [&](int st) { return stg0 + (size_t)st * (STAGE / sizeof(float2)); };
  // unit -> (simulation, first bundle, bundles in the unit)
  auto unit_info = [&](int unit, int& si, int& b0, int& cnt) {
    si = locate_sim(w, unit);
    b0 = (unit - __ldg(&w.prefix[si])) * BPC;
    cnt = NB - b0 < BPC ? NB - b0 : BPC;
  };
  auto coords = [&](int b, int box, int& c0, int& c1, int& c2) {
    const int plane = b / NBP, kx0 = (b % NBP) * BW;
    c0 = 2 * kx0;
    c1 = ZAX ? plane : box * BOX;
    c2 = ZAX ? box * BOX : plane;
  };
  auto issue_load = [&](int unit, int st) {
    int si, b0, cnt;
    unit_info(unit, si, b0, cnt);
    const CUtensorMap* tm = &maps[2 * si + (ZAX ? 1 : 0)];
    mbar_expect_tx(&bar[st], (unsigned)cnt * BUNDLE);
    for (int i = 0; i < cnt; ++i)
#pragma unroll
      for (int box = 0; box < NBOX; ++box) {
        int c0, c1, c2;
        coords(b0 + i, box, c0, c1, c2);
        tma_load_3d(stage_ptr(st) + (i * N + box * BOX) * BW, tm, c0, c1, c2, &bar[st]);
      }
  };
  int unit = blockIdx.x;
  if (threadIdx.x == 0 && unit < w.total) issue_load(unit, 0);
  unsigned parity = 0;  // bit st: parity of the next phase of stage st
  for (int it = 0; unit < w.total; unit += gridDim.x, ++it) {
    const int st = it % TMA_STAGES;
    const int next = unit + gridDim.x;
    if (threadIdx.x == 0 && next < w.total) {
      bulk_wait_read<TMA_STAGES - 2>();  // the store that last read stage (it+1)%3 is done
      issue_load(next, (it + 1) % TMA_STAGES);
    }
    const bool ok = mbar_wait(&bar[st], (parity >> st) & 1u);
    parity ^= 1u << st;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) set_error(err, ERR_TIMEOUT);
      break;
    }
    int si, b0, cnt;
    unit_info(unit, si, b0, cnt);
    const Sim& S = sims[si];
    float2* s = stage_ptr(st);
    if (MODE == 0 || MODE == 4) {
      fft_lines_blocked<N, NL, BW, line_nt(N), false>(s, S.tw, 1);
    } else if (MODE == 1 || MODE == 5) {
      fft_lines_blocked<N, NL, BW, line_nt(N), true>(s, S.tw, 1);
    } else {
      // forward z transform, the Green function, inverse z transform (meeting in registers)
      const GreenEpi<N, MODE == 3, MODE == 6> epi{S.green, S.s2, S.fgrid, b0, cnt, S.sn, S.grad_axis};
      fft_lines_blocked_turn<N, NL, BW, line_nt(N)>(s, S.tw, 1, epi);
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      const CUtensorMap* tm = &maps[2 * si + (ZAX ? 1 : 0)];
      for (int i = 0; i < cnt; ++i)
#pragma unroll
        for (int box = 0; box < NBOX; ++box) {
          int c0, c1, c2;
          coords(b0 + i, box, c0, c1, c2);
          tma_store_3d(tm, c0, c1, c2, s + (i * N + box * BOX) * BW);
        }
      bulk_commit();
    }
  }
  if (threadIdx.x == 0) bulk_wait<0>();
}

// ---------------------------------------------------------------------------------
// x passes, row transform in registers (xrow_ok sizes).  T lanes of a warp own one row of
// M = P Q complex points, j = Q a + b, k = c + P d:
//   pass 1  lane t, b = t + T i: P-point DFT over a of z[Q a + b], times w_M^(b c)
//   (shared-memory exchange inside the row, synchronised by the warp alone)
//   pass 2  lane t, c = t + T i: Q-point DFT over b -> Z[c + P d]
// R2C: z[j] = x[2j] + i x[2j+1] read straight from the density rows, Z untangled into the
// half spectrum.  C2R: the spectrum row is staged, tangled into pass 1, and z written as
// pairs of reals.  Loads and stores of T lanes are consecutive (coalesced).  A work unit
// is the 32 / T rows of one warp.
// ---------------------------------------------------------------------------------
// Pass 1, the in-row exchange and pass 2 of a row transform; v holds z[Q a + t + T i] on
// entry, o holds Z[t + T i + P d] on exit.  rb: the row's exchange buffer (Q (P + 1)).
template <int N, bool INV>
__device__ __forceinline__ void xrow_transform(float2 (&v)[xrow_Q(N) / xrow_T(N)][xrow_P(N)],
                                               float2 (&o)[xrow_P(N) / xrow_T(N)][xrow_Q(N)], float2* rb, int t,
                                               const float2* __restrict__ tw) {
  constexpr int M = N / 2, P = xrow_P(N), Q = xrow_Q(N), T = xrow_T(N);
  constexpr int NB1 = Q / T, NB2 = P / T;
#pragma unroll
  for (int i = 0; i < NB1; ++i) {
    const int b = t + T * i;
    DFT<P, INV>::run(v[i]);
#pragma unroll
    for (int c = 1; c < P; ++c) {
      float2 wv = __ldg(&tw[((b * c) % M) * 2]);
      if (INV) wv.y = -wv.y;
      v[i][c] = cmul(v[i][c], wv);
    }
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < NB1; ++i)
#pragma unroll
    for (int c = 0; c < P; ++c) rb[(t + T * i) * (P + 1) + c] = v[i][c];
  __syncwarp();
#pragma unroll
  for (int i = 0; i < NB2; ++i) {
#pragma unroll
    for (int b = 0; b < Q; ++b) o[i][b] = rb[b * (P + 1) + t + T * i];
    DFT<Q, INV>::run(o[i]);
  }
}

// R2C end of a row: Z (in o) is untangled into the half-spectrum row dst[0..M].
template <int N>
__device__ __forceinline__ void xrow_untangle_store(const float2 (&o)[xrow_P(N) / xrow_T(N)][xrow_Q(N)], float2* rb,
                                                    int t, const float2* __restrict__ tw, float2* __restrict__ dst) {
  constexpr int M = N / 2, P = xrow_P(N), Q = xrow_Q(N), T = xrow_T(N), NB2 = P / T;
  __syncwarp();
#pragma unroll
  for (int i = 0; i < NB2; ++i)
#pragma unroll
    for (int d = 0; d < Q; ++d) rb[t + T * i + P * d] = o[i][d];
  __syncwarp();
  // X[k] = E[k] + W^k O[k], k = 0..M
  for (int k = t; k <= M; k += T) {
    const float2 zk = rb[k == M ? 0 : k];
    const float2 zc = conjf2(rb[k == 0 ? 0 : M - k]);
    const float2 e = cscale(cadd(zk, zc), 0.5f);
    const float2 od = cscale(mul_mi<false>(csub(zk, zc)), 0.5f);
    dst[k] = cadd(e, cmul(__ldg(&tw[k]), od));
  }
}

template <int N, bool C2R>
__global__ void __launch_bounds__(xrow_nt(N)) k_x_row(const Sim* __restrict__ sims, Work w) {
  constexpr int XR_NT = xrow_nt(N);
  constexpr int M = N / 2, P = xrow_P(N), Q = xrow_Q(N), T = xrow_T(N), RPW = 32 / T;
  constexpr int RB = Q * (P + 1);  // exchange buffer of a row (>= M + 1)
  constexpr int NB1 = Q / T, NB2 = P / T;
  static_assert(P * Q == M && Q % T == 0 && P % T == 0 && RB >= M + 1, "row plan");
  __shared__ float2 sbuf[XR_NT / 32][RPW][RB];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int sub = lane / T, t = lane % T;
  float2* rb = sbuf[wid][sub];
  const long long nw = (long long)gridDim.x * (XR_NT / 32);
  for (long long unit = (long long)blockIdx.x * (XR_NT / 32) + wid; unit < w.total; unit += nw) {
    const int si = locate_sim(w, (int)unit);
    const Sim& S = sims[si];
    const long long row = ((long long)unit - __ldg(&w.prefix[si])) * RPW + sub;
    const float2* __restrict__ tw = S.tw;
    float2 v[NB1][P];
    float2 o[NB2][Q];
    if (!C2R) {
      const float2* __restrict__ src = reinterpret_cast<const float2*>(S.rho) + row * M;
#pragma unroll
      for (int i = 0; i < NB1; ++i)
#pragma unroll
        for (int a = 0; a < P; ++a) v[i][a] = __ldg(&src[Q * a + t + T * i]);
      xrow_transform<N, false>(v, o, rb, t, tw);
      xrow_untangle_store<N>(o, rb, t, tw, S.spec + row * S.pitch);
    } else {
      const float2* __restrict__ src = S.spec + row * S.pitch;
      // all loads of the row issued before any store (the row is M + 1 values)
      constexpr int NLD = (M + 1 + T - 1) / T;
      float2 ld[NLD];
#pragma unroll
      for (int i = 0; i < NLD; ++i) {
        const int k = t + T * i;
        ld[i] = k <= M ? __ldg(&src[k]) : make_float2(0.f, 0.f);
      }
      __syncwarp();
#pragma unroll
      for (int i = 0; i < NLD; ++i)
        if (t + T * i <= M) rb[t + T * i] = ld[i];
      __syncwarp();
      // tangle: Z[j] = (X[j] + X*[M-j]) + i W^-j (X[j] - X*[M-j])
#pragma unroll
      for (int i = 0; i < NB1; ++i)
#pragma unroll
        for (int a = 0; a < P; ++a) {
          const int j = Q * a + t + T * i;
          const float2 xk = rb[j], xm = rb[M - j];
          const float2 ap = cadd(xk, conjf2(xm)), bm = csub(xk, conjf2(xm));
          const float2 tt = cmul(conjf2(__ldg(&tw[j])), bm);
          v[i][a] = make_float2(ap.x - tt.y, ap.y + tt.x);
        }
      xrow_transform<N, true>(v, o, rb, t, tw);
      float2* __restrict__ dst = reinterpret_cast<float2*>(S.phi) + row * M;
#pragma unroll
      for (int i = 0; i < NB2; ++i)
#pragma unroll
        for (int d = 0; d < Q; ++d) dst[t + T * i + P * d] = o[i][d];
    }
  }
}

// Tensor map of a half spectrum seen as float32 [z][y][2*pitch], box {2 BW, BOX, 1} for the
// y pass and {2 BW, 1, BOX} for the z pass.
inline bool encode_spectrum_map(CUtensorMap* tm, const void* spec, int n, bool zaxis) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
      return false;
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  const cuuint64_t row = (cuuint64_t)2 * cpitch(n);
  const cuuint32_t box_rows = (cuuint32_t)line_box_rows(n);
  cuuint64_t dims[3] = {row, (cuuint64_t)n, (cuuint64_t)n};
  cuuint64_t strides[2] = {row * 4, row * 4 * (cuuint64_t)n};
  cuuint32_t box[3] = {(cuuint32_t)(2 * cline_width(n)), zaxis ? 1u : box_rows, zaxis ? box_rows : 1u};
  cuuint32_t estr[3] = {1, 1, 1};
  return fn(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(spec), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------------
// x passes fed by bulk copies, one simulation per launch.
//
// Persistent CTA with two staging buffers.  The NR rows of a unit stream into a staging
// buffer (one 1-D bulk copy per row, completing on an mbarrier); unit i is transposed out
// of its buffer into the padded line-interleaved FFT buffer, the buffer is refilled at
// once with unit i+2, and the transform and its coalesced global stores follow.
// ---------------------------------------------------------------------------------
template <int N, bool C2R>
__global__ void __launch_bounds__(XTMA_NT, 1) k_x_tma(const Sim* __restrict__ sims, Work w, int* err) {
  constexpr int M = N / 2, NR = cx_rows(N), LS = NR + 1, RS = xrow_stage_floats(N);
  constexpr int NT = XTMA_NT;
  // bytes copied per row: R2C reads n floats; C2R reads M + 2 complex (= RS floats)
  constexpr unsigned ROWB = C2R ? RS * 4u : N * 4u;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* stage[2] = {reinterpret_cast<float*>(smem_raw),
                     reinterpret_cast<float*>(smem_raw + (size_t)NR * RS * sizeof(float))};
  float2* F = reinterpret_cast<float2*>(smem_raw + 2 * (size_t)NR * RS * sizeof(float));
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + 2 * (size_t)NR * RS * sizeof(float) + xtma_fft_bytes(N));
  const long long nrows = (long long)N * N;
  const int nunits = w.total;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  // warp 0 issues the copies of one unit: lane r copies rows r, r + 32, ...
  auto issue = [&](int unit, int st) {
    const int si = locate_sim(w, unit);
    const Sim& S = sims[si];
    const long long row0 = (long long)(unit - __ldg(&w.prefix[si])) * NR;
    const int rows = (int)(nrows - row0 < NR ? nrows - row0 : NR);
    if (lane == 0) mbar_expect_tx(&bar[st], (unsigned)rows * ROWB);
    __syncwarp();
    for (int r = lane; r < rows; r += 32) {
      const void* src = C2R ? (const void*)(S.spec + (row0 + r) * S.pitch) : (const void*)(S.rho + (row0 + r) * N);
      bulk_load(stage[st] + r * RS, src, ROWB, &bar[st]);
    }
  };
  int unit = blockIdx.x;
  if (warp == 0) {
    if (unit < nunits) issue(unit, 0);
    if (unit + (int)gridDim.x < nunits) issue(unit + gridDim.x, 1);
  }
  unsigned parity = 0;
  for (int it = 0; unit < nunits; unit += gridDim.x, ++it) {
    const int st = it & 1;
    const int si = locate_sim(w, unit);
    const Sim& S = sims[si];
    const long long row0 = (long long)(unit - __ldg(&w.prefix[si])) * NR;
    const bool ok = mbar_wait(&bar[st], (parity >> st) & 1u);
    parity ^= 1u << st;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) set_error(err, ERR_TIMEOUT);
      break;
    }
    const float2* sg = reinterpret_cast<const float2*>(stage[st]);
    if (!C2R) {
      // z[j] = x[2j] + i x[2j+1]: staged row r, complex j -> F[j][r]
      for (int u = threadIdx.x; u < NR * M; u += NT) {
        const int r = u / M, j = u % M;
        F[j * LS + r] = sg[r * (RS / 2) + j];
      }
    } else {
      // tangle: Z[k] = (X[k] + X*[M-k]) + i W^-k (X[k] - X*[M-k]), pairs (k, M-k)
      for (int u = threadIdx.x; u < NR * (M / 2 + 1); u += NT) {
        const int r = u / (M / 2 + 1), k = u % (M / 2 + 1);
        const float2 xk = sg[r * (RS / 2) + k];
        const float2 xm = sg[r * (RS / 2) + (M - k)];
        const float2 a = cadd(xk, conjf2(xm));
        const float2 b = csub(xk, conjf2(xm));
        const float2 w = __ldg(&S.tw[k]);
        const float2 t = cmul(conjf2(w), b);
        F[k * LS + r] = make_float2(a.x - t.y, a.y + t.x);
        if (k != 0 && 2 * k != M) {
          const float2 t2 = cmul(w, conjf2(b));
          F[(M - k) * LS + r] = make_float2(a.x - t2.y, -a.y + t2.x);
        }
      }
    }
    __syncthreads();  // staging buffer st is free again: refill it with the unit after next
    const int after = unit + 2 * (int)gridDim.x;
    if (warp == 0 && after < nunits) issue(after, st);
    fft_lines<M, NR, LS, NT, C2R>(F, S.tw, 2);
    if (!C2R) {
      float2* __restrict__ dst = S.spec;
      const int P = S.pitch;
      for (int u = threadIdx.x; u < NR * (M + 1); u += NT) {
        const int r = u / (M + 1), k = u % (M + 1);
        if (row0 + r >= nrows) continue;
        const float2 zk = F[(k == M ? 0 : k) * LS + r];
        const float2 zc = conjf2(F[(k == 0 ? 0 : M - k) * LS + r]);
        const float2 e = cscale(cadd(zk, zc), 0.5f);
        const float2 o = cscale(mul_mi<false>(csub(zk, zc)), 0.5f);
        dst[(row0 + r) * P + k] = cadd(e, cmul(__ldg(&S.tw[k]), o));
      }
    } else {
      float2* __restrict__ dst = reinterpret_cast<float2*>(S.phi);
      for (int u = threadIdx.x; u < NR * M; u += NT) {
        const int r = u / M, j = u % M;
        if (row0 + r < nrows) dst[(row0 + r) * M + j] = F[j * LS + r];
      }
    }
    __syncthreads();  // F is rewritten by the next unit
  }
}

// ---------------------------------------------------------------------------------
// fused deposit + x R2C: one CTA per deposit tile.  The tile's TZ x TY rows are deposited
// into shared memory (pm_deposit.cuh), converted to float and transformed along x -- by
// the register row transform (T lanes per row) where the size has one, else transposed
// into a padded line-interleaved buffer (reusing the accumulator space) -- and the
// half-spectrum rows are written directly, so the density grid never goes to HBM.
// ---------------------------------------------------------------------------------
// accumulators: 2 words per cell, >= (n/2) * (TZ*TY + 1) * sizeof(float2) for the
// shared-memory transform; with the register row transform each row's low and high words
// are adjacent (row r at word 2 r n) and the row's exchange buffer overlays them
__host__ __device__ constexpr size_t deposit_r2c_smem_bytes(int n) { return (size_t)2 * TZ * TY * n * sizeof(unsigned); }
__host__ __device__ constexpr int deposit_r2c_nt(int n) { return xrow_ok(n) ? DEP_ROW_NT : DEP_NT; }
// sizes whose tile (TZ * TY rows of n cells) divides evenly over the block
__host__ __device__ constexpr bool deposit_r2c_ok(int n) { return (TZ * TY * n) % deposit_r2c_nt(n) == 0; }

// Tiles per CTA of the fused deposit: the register row transform of a tile's 16 rows keeps
// 16 / T warps busy (T lanes per row), so on the sizes with T < 16 a CTA takes several tiles
// at once -- its warps split into one group per tile for the particle loop and share all the
// rows in the transform -- as long as their accumulators stay within 72 KB (three CTAs per
// SM).  The 192 grid (T = 4, 48 complex values per lane) takes its four tiles at two CTAs per
// SM with 128 registers instead (measured 0.90 -> 0.87 ms per 134M-cell deposit).
__host__ __device__ constexpr int dep_ctas_bound(int n) { return n == 192 ? 2 : (xrow_ok(n) ? 3 : 2); }
__host__ __device__ constexpr int dep_tiles(int n) {
  int t = xrow_ok(n) ? 16 / xrow_T(n) : 1;
  while (t > 1 && (size_t)t * deposit_r2c_smem_bytes(n) > (n == 192 ? 100 : 72) * 1024) t /= 2;
  return t;
}

template <int N, int MODE>
__global__ void __launch_bounds__(deposit_r2c_nt(N), dep_ctas_bound(N))
    k_deposit_r2c(const Sim* __restrict__ sims, Work w, Parts p, const unsigned* __restrict__ perm,
                  const unsigned* __restrict__ row_start, int* err, unsigned* __restrict__ next_tile,
                  const unsigned* __restrict__ order) {
  constexpr int NT = deposit_r2c_nt(N);
  constexpr int M = N / 2, NL = TZ * TY, LS = NL + 1;
  constexpr int PER = NL * N / NT;
  constexpr int TPB = dep_tiles(N);  // tiles per CTA
  static_assert(NL * N % NT == 0, "tile cells must divide by the block size");
  static_assert((size_t)M * LS * sizeof(float2) <= deposit_r2c_smem_bytes(N), "FFT buffer must fit");
  static_assert(TPB * 8 <= 32 && NT % (TPB * 32) == 0, "one warp loads the run tables of a CTA's tiles");
  extern __shared__ uint4 acc_raw[];
  // run tables of the CTA's tiles (7 runs each: first sorted index, and inclusive offsets)
  __shared__ unsigned s_begin[TPB][8];
  __shared__ unsigned s_off[TPB][8];
  __shared__ TileSum s_ts[TPB];
  unsigned* lo = reinterpret_cast<unsigned*>(acc_raw);
  // row r: lo at r * RS, hi at r * RS + HO (tiles one after another, NL rows each)
  constexpr int RS = xrow_ok(N) ? 2 * N : N, HO = xrow_ok(N) ? N : NL * N;
  unsigned* hi = lo + HO;
  float2* F = reinterpret_cast<float2*>(acc_raw);
  float* Ff = reinterpret_cast<float*>(acc_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // Tiles are taken from a counter (zero at launch) after the first, TPB per CTA: a tile's
  // work is its particle count, which clustering makes very uneven, so a fixed stride
  // leaves the CTAs that drew the dense tiles running alone at the end.
  // `order` (optional) lists the tiles dense-first; idx is the place in it.
  __shared__ int s_next;
  auto take_next = [&](int idx) -> int {
    return next_tile ? (int)gridDim.x * TPB + (int)atomicAdd(next_tile, (unsigned)TPB) : idx + (int)gridDim.x * TPB;
  };
  auto tile_at = [&](int idx) -> int { return order ? (int)__ldg(&order[idx]) : idx; };
  // the tile at place i of the order: its simulation and first row / plane (false: none)
  auto tile_of = [&](int i, int& si, int& y0, int& z0) -> bool {
    si = 0; y0 = z0 = 0;
    if (i >= w.total) return false;
    const int unit = tile_at(i);
    si = locate_sim(w, unit);
    const int local = unit - __ldg(&w.prefix[si]);
    y0 = (local % (N / TY)) * TY;
    z0 = (local / (N / TY)) * TZ;
    return true;
  };
  if constexpr (xrow_ok(N)) {
    constexpr int NTT = NT / TPB;  // threads per tile group
    constexpr int P = xrow_P(N), Q = xrow_Q(N), T = xrow_T(N), RPW = 32 / T;
    constexpr int NB1 = Q / T, NB2 = P / T;
    static_assert(Q * (P + 1) * sizeof(float2) <= 2 * N * sizeof(unsigned), "exchange buffer in the row");
    const int g = threadIdx.x / NTT, gtid = threadIdx.x % NTT;
    // warp 0: the run tables of the tiles at places idx .. idx + TPB - 1 (8 lanes per tile)
    auto load_tables = [&](int idx) -> RunLoad {
      RunLoad v{0u, 0u};
      int si, y0, z0;
      if (tile_of(idx + (lane >> 3), si, y0, z0)) v = run_load(sims[si], row_start, y0, z0, lane & 7);
      return v;
    };
    int idx = blockIdx.x * TPB;
    if (warp == 0 && idx < w.total) {
      const RunLoad v = load_tables(idx);
      const int tj = lane < TPB * 8 ? lane >> 3 : 0;
      run_table(v, lane, s_begin[tj], s_off[tj], lane < TPB * 8);
    }
    // The accumulators start zero, and each row is zeroed again by its transform lanes once
    // they are done with it, so a tile needs no zeroing phase and barrier of its own
    // (0.468 -> 0.460 ms early, 0.604 -> 0.587 ms at step 980, 256^3 on 512^3).
    for (int i = threadIdx.x; i < TPB * NL * RS / 4; i += NT) acc_raw[i] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    while (idx < w.total) {
      {  // the particles of this group's tile (a group without a tile has an empty table)
        int si, y0, z0;
        tile_of(idx + g, si, y0, z0);
        deposit_tile<MODE, NTT, N>(sims[si], p, perm, row_start, err, y0, z0, lo + g * NL * RS, hi + g * NL * RS, RS,
                                s_begin[g], s_off[g], true, gtid, &s_ts[g], true);
      }
      // the CTA's TPB * NL rows: T lanes per row, rows R = warp * RPW + sub; a row's exchange
      // buffer overlays its own accumulator words once they are read
      const int sub = lane / T, t = lane % T;
      const int R = warp * RPW + sub, tg = R / NL, r = R % NL;
      float2* rb = reinterpret_cast<float2*>(lo + R * RS);
      if (warp * RPW < TPB * NL) {  // warp-uniform
        int tsi, ty0, tz0;
        const bool thas = tile_of(idx + tg, tsi, ty0, tz0);
        const Sim& S = sims[tsi];
        const TileSum ts = s_ts[tg];
        float2 v2[NB1][P];
        float2 o2[NB2][Q];
        const uint2* l2 = reinterpret_cast<const uint2*>(lo + R * RS);
        const uint2* h2 = reinterpret_cast<const uint2*>(lo + R * RS + HO);
#pragma unroll
        for (int i = 0; i < NB1; ++i)
#pragma unroll
          for (int a = 0; a < P; ++a) {
            const int j = Q * a + t + T * i;  // z[j] = x[2j] + i x[2j+1]
            const uint2 ll = l2[j], hh = ts.s ? make_uint2(0u, 0u) : h2[j];
            v2[i][a] = make_float2(sum_to_float(ts, ll.x, hh.x), sum_to_float(ts, ll.y, hh.y));
          }
        // warp 0 takes the next tiles and loads their run tables now, and stores them after the
        // transform, so that the loads' latency hides behind it (the tables are free: the
        // particle loops are over, and the transform reads s_ts)
        int next = 0;
        if (warp == 0) next = __shfl_sync(FULL, lane == 0 ? take_next(idx) : 0, 0);
        RunLoad nl{0u, 0u};
        if (warp == 0 && next < w.total) nl = load_tables(next);
        xrow_transform<N, false>(v2, o2, rb, t, S.tw);
        if (thas) {
          const long long row = (long long)(tz0 + r / TY) * N + (ty0 + r % TY);
          xrow_untangle_store<N>(o2, rb, t, S.tw, S.spec + row * S.pitch);
        }
        __syncwarp();  // the row's lanes are done with its words
        {  // zero what this tile dirtied: the low words and the exchange buffer (which reaches
           // into the high words), and the high words after a two-word tile
          constexpr int XW = 2 * Q * (P + 1);  // words of the exchange buffer
          static_assert(XW % 4 == 0 && RS % 4 == 0, "rows zeroed 4 words at a time");
          const int zw = ts.s ? (XW > N ? XW : N) : RS;
          uint4* z4 = reinterpret_cast<uint4*>(lo + R * RS);
          for (int i = t; i < zw / 4; i += T) z4[i] = make_uint4(0u, 0u, 0u, 0u);
        }
        if (warp == 0 && next < w.total) {
          const int tj = lane < TPB * 8 ? lane >> 3 : 0;
          run_table(nl, lane, s_begin[tj], s_off[tj], lane < TPB * 8);
        }
        if (threadIdx.x == 0) s_next = next;
      }
      __syncthreads();
      idx = s_next;
    }
    return;
  } else {
    bool runs_ready = false;
    for (int idx = blockIdx.x; idx < w.total;) {
      int si, y0, z0;
      tile_of(idx, si, y0, z0);
      const Sim& S = sims[si];
      const TileSum ts = deposit_tile<MODE, NT, N>(S, p, perm, row_start, err, y0, z0, lo, hi, RS, s_begin[0], s_off[0],
                                                runs_ready);
      runs_ready = false;
      float v[PER];
#pragma unroll
      for (int k = 0; k < PER; ++k) {
        const int i = threadIdx.x + k * NT;
        v[k] = sum_to_float(ts, lo[i], ts.s ? 0u : hi[i]);
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < PER; ++k) {
        const int i = threadIdx.x + k * NT;
        const int r = i / N, x = i % N;
        Ff[((x >> 1) * LS + r) * 2 + (x & 1)] = v[k];  // z[j] = x[2j] + i x[2j+1] of row r
      }
      __syncthreads();
      fft_lines<M, NL, LS, NT, false>(F, S.tw, 2);
      float2* __restrict__ dst = S.spec;
      const int P = S.pitch;
      for (int u = threadIdx.x; u < NL * (M + 1); u += NT) {
        const int r = u / (M + 1), k = u % (M + 1);
        const long long row = (long long)(z0 + r / TY) * N + (y0 + r % TY);
        const float2 zk = F[(k == M ? 0 : k) * LS + r];
        const float2 zc = conjf2(F[(k == 0 ? 0 : M - k) * LS + r]);
        const float2 e = cscale(cadd(zk, zc), 0.5f);
        const float2 o = cscale(mul_mi<false>(csub(zk, zc)), 0.5f);
        dst[row * P + k] = cadd(e, cmul(__ldg(&S.tw[k]), o));
      }
      if (threadIdx.x == 0) s_next = take_next(idx);
      __syncthreads();
      idx = s_next;
    }
  }
}

template <int N>
cudaError_t deposit_r2c_launch(const Sim* sims, Work w, Parts p, const unsigned* perm, const unsigned* row_start,
                               int mode, int* err, unsigned* next_tile, const unsigned* order, int ctas,
                               cudaStream_t st) {
  if constexpr (!deposit_r2c_ok(N)) {
    return cudaErrorNotSupported;
  } else {
  static DeviceOnce once;
  const size_t sm = dep_tiles(N) * deposit_r2c_smem_bytes(N);
  const cudaError_t ie = once.run([&]() {
    cudaError_t e = cudaFuncSetAttribute(k_deposit_r2c<N, POS_ABS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (!e) e = cudaFuncSetAttribute(k_deposit_r2c<N, POS_DISP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (!e) e = cudaFuncSetAttribute(k_deposit_r2c<N, POS_ABS>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (!e) e = cudaFuncSetAttribute(k_deposit_r2c<N, POS_DISP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    return e;
  });
  if (ie) return ie;
  if (ctas <= 0) return cudaSuccess;  // attribute setup only
  constexpr int NT = deposit_r2c_nt(N), TPB = dep_tiles(N);
  if (ctas > (w.total + TPB - 1) / TPB) ctas = (w.total + TPB - 1) / TPB;  // TPB tiles per CTA
  if (ctas <= 0) return cudaSuccess;
  if (next_tile) {
    const cudaError_t e = cudaMemsetAsync(next_tile, 0, sizeof(unsigned), st);
    if (e) return e;
  }
  if (mode == POS_ABS)
    k_deposit_r2c<N, POS_ABS><<<ctas, NT, sm, st>>>(sims, w, p, perm, row_start, err, next_tile, order);
  else
    k_deposit_r2c<N, POS_DISP><<<ctas, NT, sm, st>>>(sims, w, p, perm, row_start, err, next_tile, order);
  return cudaGetLastError();
  }
}

template <typename K>
static cudaError_t max_shared(K kern, size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (!e) e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  return e;
}

template <int N>
cudaError_t spectral_launch(SpecKind kind, const Sim* sims, Work w, int ctas, cudaStream_t st,
                            const CUtensorMap* maps, int* err) {
  static DeviceOnce once;
  const size_t xs = x_smem_bytes(N), ls = line_smem_bytes(N);
  const cudaError_t ie = once.run([&]() -> cudaError_t {
    if constexpr (tma_rows(N)) {
      cudaError_t e = max_shared(k_x_tma<N, false>, xtma_smem_bytes(N));
      if (!e) e = max_shared(k_x_tma<N, true>, xtma_smem_bytes(N));
      if (e) return e;
    }
    if constexpr (tma_lines(N)) {
      cudaError_t e = max_shared(k_line_tma<N, 0>, tma_smem_bytes(N));
      if (!e) e = max_shared(k_line_tma<N, 1>, tma_smem_bytes(N));
      if (!e) e = max_shared(k_line_tma<N, 2>, tma_smem_bytes(N));
      if (!e) e = max_shared(k_line_tma<N, 3>, tma_smem_bytes(N));
      if (!e) e = max_shared(k_line_tma<N, 4>, tma_smem_bytes(N));
      if (!e) e = max_shared(k_line_tma<N, 5>, tma_smem_bytes(N));
      if (!e) e = max_shared(k_line_tma<N, 6>, tma_smem_bytes(N));
      if (e) return e;
    }
    cudaError_t e = max_shared(k_x_r2c<N>, xs);
    if (!e) e = max_shared(k_x_c2r<N>, xs);
    if (!e) e = max_shared(k_line_pass<N, false, false>, ls);
    if (!e) e = max_shared(k_line_pass<N, false, true>, ls);
    if (!e) e = max_shared(k_line_pass<N, true, false>, ls);
    if (!e) e = max_shared(k_line_pass<N, true, true>, ls);
    if (!e) e = max_shared(k_z_green<N, false>, ls);
    if (!e) e = max_shared(k_z_green<N, true>, ls);
    if (!e) e = max_shared(k_z_green<N, false, true>, ls);
    return e;
  });
  if (ie) return ie;
  if (kind == SPEC_PREPARE) return cudaSuccess;
  const int grid = w.total < device_sms() ? w.total : device_sms();
  if constexpr (xrow_ok(N)) {
    if (kind == SPEC_X_R2C || kind == SPEC_X_C2R) {
      // ctas: the cap on the CTAs of the persistent row transform (the batch engine tunes it)
      const int per = xrow_nt(N) / 32, want = (w.total + per - 1) / per, cap = ctas > 0 ? ctas : device_sms() * 8;
      const int g = want < cap ? want : cap;
      if (kind == SPEC_X_R2C) k_x_row<N, false><<<g, xrow_nt(N), 0, st>>>(sims, w);
      else k_x_row<N, true><<<g, xrow_nt(N), 0, st>>>(sims, w);
      return cudaGetLastError();
    }
  }
  if constexpr (tma_rows(N)) {
    if (kind == SPEC_X_R2C || kind == SPEC_X_C2R) {
      if (kind == SPEC_X_R2C) k_x_tma<N, false><<<grid, XTMA_NT, xtma_smem_bytes(N), st>>>(sims, w, err);
      else k_x_tma<N, true><<<grid, XTMA_NT, xtma_smem_bytes(N), st>>>(sims, w, err);
      return cudaGetLastError();
    }
  }
  if constexpr (tma_lines(N)) {
    if (maps) {
      const size_t sm = tma_smem_bytes(N);
      const int lcap = line_ctas_per_sm(N) * device_sms();
      const int grid = w.total < lcap ? w.total : lcap;
      switch (kind) {
        case SPEC_Y_FWD: k_line_tma<N, 0><<<grid, line_nt(N), sm, st>>>(maps, sims, w, err); return cudaGetLastError();
        case SPEC_Y_INV: k_line_tma<N, 1><<<grid, line_nt(N), sm, st>>>(maps, sims, w, err); return cudaGetLastError();
        case SPEC_Z_GREEN: k_line_tma<N, 2><<<grid, line_nt(N), sm, st>>>(maps, sims, w, err); return cudaGetLastError();
        case SPEC_Z_TABLE: k_line_tma<N, 3><<<grid, line_nt(N), sm, st>>>(maps, sims, w, err); return cudaGetLastError();
        case SPEC_Z_FWD: k_line_tma<N, 4><<<grid, line_nt(N), sm, st>>>(maps, sims, w, err); return cudaGetLastError();
        case SPEC_Z_INV: k_line_tma<N, 5><<<grid, line_nt(N), sm, st>>>(maps, sims, w, err); return cudaGetLastError();
        case SPEC_Z_GRAD: k_line_tma<N, 6><<<grid, line_nt(N), sm, st>>>(maps, sims, w, err); return cudaGetLastError();
        default: break;
      }
    }
  }
  switch (kind) {
    case SPEC_X_R2C: k_x_r2c<N><<<ctas, SP_NT, xs, st>>>(sims, w); break;
    case SPEC_X_C2R: k_x_c2r<N><<<ctas, SP_NT, xs, st>>>(sims, w); break;
    case SPEC_Y_FWD: k_line_pass<N, false, false><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    case SPEC_Y_INV: k_line_pass<N, false, true><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    case SPEC_Z_FWD: k_line_pass<N, true, false><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    case SPEC_Z_INV: k_line_pass<N, true, true><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    case SPEC_Z_GREEN: k_z_green<N, false><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    case SPEC_Z_TABLE: k_z_green<N, true><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    case SPEC_Z_GRAD: k_z_green<N, false, true><<<ctas, SP_NT, ls, st>>>(sims, w); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace pm
