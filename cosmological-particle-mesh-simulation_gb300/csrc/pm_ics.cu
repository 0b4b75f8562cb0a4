// Initial conditions on the device: the Gaussian random field of
// src/gaussian_random_field.py:9-123 and the Zel'dovich positions and velocities of
// src/zeldovich.py:10-100, computed with the engine's float32 spectral passes.
//
// Input: the two float32 streams of accepted uniform numbers in (-1, 1) of the reference's
// rejection loop (gaussian_random_field.py:35-50; numpy RandomState, drawn by the caller).
// Everything else runs here:
//   * the polar Box-Muller transform (gaussian_random_field.py:53-61), float32 as in the
//     reference, with the float64 recomputation of pairs whose float32 u^2 + v^2 rounds
//     to >= 1 (the reference would produce NaN there);
//   * the power spectrum and its normalisation sum (gaussian_random_field.py:65-123) in
//     float64: the k-dependence is tabulated once per integer |m|^2 (k = 2 pi |m| / box),
//     the sum over the full grid is reduced in a fixed order (deterministic);
//   * Re(ifftn(rho_k)) (gaussian_random_field.py:24-29): the real part of the inverse
//     transform of a non-Hermitian rho_k is the inverse real transform of its Hermitian
//     part (rho_k[k] + conj(rho_k[-k])) / 2, which is built directly in the half spectrum;
//   * fftn of that field, the potential -rho_k / |l|^2 (k = 0 -> 0), -i l_d pot_k * res,
//     and Re(ifftn(.)) * force_resolution per direction (zeldovich.py:17-69); the planes
//     where l_d sits at the Nyquist frequency have no Hermitian part and are zero;
//   * lattice + Dt * disp + jitter, modulo N_CELLS, and A f H Dt * disp
//     (zeldovich.py:71-100), in float64 per particle as numpy does, stored as float32.
//     The jitter is the numpy PCG64 stream of uniform(-2, 2) (x, then y, then z draws),
//     generated here by jumping the 128-bit LCG to each thread's first draw.
#include "pm_host.cuh"

using namespace pm;

namespace {

constexpr int NORM_BLOCKS = 512;  // fixed grid: the reduction order is the same on every device
constexpr int NORM_NT = 256;
constexpr int IC_NT = 256;
constexpr int JIT_CHUNK = 8;      // consecutive jitter draws per thread

// ---- the power spectrum shape (gaussian_random_field.py:65-123) -----------------------
struct Shape {
  double kscale;  // 2 pi / box: k = kscale * sqrt(m2)
  double gamma;   // OMEGA_M0 * H0 * exp(-OMEGA_B0 - OMEGA_B0 / OMEGA_M0)
  double power;
  int lcdm;
};

__device__ double lcdm_transfer(double k, double gamma) {
  const double q = k / gamma;
  const double a = 16.1 * q, b = 5.46 * q, c = 6.71 * q;
  const double f1 = sqrt(1.0 + 3.89 * q + a * a + pow(b, 3.0) + pow(c, 4.0));
  double f2 = 0.0;
  if (q != 0.0) {
    const double l = log(1.0 + 2.34 * q), d = 2.34 * q;
    f2 = (l * l) / (d * d);
  }
  return f2 / f1;
}

// S(m2): the summand of the normalisation, which is also P(k) / A for k != 0.
__global__ void k_shape(double* __restrict__ shape, int m2max, Shape sp) {
  const int m2 = blockIdx.x * blockDim.x + threadIdx.x;
  if (m2 > m2max) return;
  const double k = sp.kscale * sqrt((double)m2);
  double s;
  if (sp.power >= 0.0) {
    const double kp = m2 != 0 ? pow(k, sp.power) : 0.0;
    s = sp.lcdm ? kp * lcdm_transfer(k, sp.gamma) : kp;
  } else {
    const double kinv = m2 != 0 ? pow(k, -sp.power) : 0.0;
    s = kinv != 0.0 ? 1.0 / kinv : 0.0;
  }
  shape[m2] = s;
}

__device__ __forceinline__ int signed_freq(int m, int n) { return m < n / 2 ? m : m - n; }
__device__ __forceinline__ int sq(int m) { return m * m; }

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += red[i];
  return t;
}

// Partial sums of S over the full grid, evaluated on the half spectrum (kx in [0, n/2])
// with weight 2 for the columns that stand for two full-grid columns.
__global__ void __launch_bounds__(NORM_NT) k_norm_partial(const double* __restrict__ shape, int n,
                                                           double* __restrict__ partial) {
  __shared__ double red[NORM_NT / 32];
  const int w = n / 2 + 1;
  const long long total = (long long)n * n * w;
  double acc = 0.0;
  for (long long e = (long long)blockIdx.x * NORM_NT + threadIdx.x; e < total; e += (long long)NORM_BLOCKS * NORM_NT) {
    const int kx = (int)(e % w);
    const long long r = e / w;
    const int ky = (int)(r % n), kz = (int)(r / n);
    const int m2 = sq(signed_freq(kx, n)) + sq(signed_freq(ky, n)) + sq(signed_freq(kz, n));
    const double wt = (kx == 0 || 2 * kx == n) ? 1.0 : 2.0;
    acc += wt * __ldg(&shape[m2]);
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// A = 64 H0^2 Npix^2 / sum (gaussian_random_field.py:104-121), one block, fixed order.
__global__ void __launch_bounds__(NORM_NT) k_norm_final(const double* __restrict__ partial, double sigma_npix2,
                                                         double* __restrict__ norm) {
  __shared__ double red[NORM_NT / 32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < NORM_BLOCKS; i += NORM_NT) acc += partial[i];
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) norm[0] = sigma_npix2 / t;
}

// ---- Gaussian random numbers (gaussian_random_field.py:53-61) -------------------------
__device__ __forceinline__ float2 box_muller(float u, float v) {
  const float s = __fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v));
  float t = __fdiv_rn(-2.0f * logf(s), s);
  if (!(t > 0.0f)) {  // float32 rounding took s to >= 1: float64, clamped at 0
    const double s64 = (double)u * (double)u + (double)v * (double)v;
    const double t64 = -2.0 * log(s64) / s64;
    t = (isfinite(t64) && t64 > 0.0) ? (float)t64 : 0.0f;
  }
  const float r = __fsqrt_rn(t);
  return make_float2(__fmul_rn(u, r), __fmul_rn(v, r));
}

struct GrfArgs {
  int n, pitch;
  const float* u;
  const float* v;
  const double* shape;
  const double* norm;
  double p0;      // P(0) / A
  double d2;      // Dt(A_INIT)^2
  double inv_n3;  // the 1/n^3 of ifftn
  float2* spec;
};

// Hermitian part of rho_k = sqrt(P Dt^2) (f1 + i f2) over the half spectrum, scaled by 1/n^3.
__global__ void __launch_bounds__(IC_NT) k_grf_fill(GrfArgs g) {
  const int n = g.n, P = g.pitch, h = n / 2;
  const long long total = (long long)n * n * P;
  const double A = __ldg(&g.norm[0]);
  for (long long e = (long long)blockIdx.x * IC_NT + threadIdx.x; e < total; e += (long long)gridDim.x * IC_NT) {
    const int kx = (int)(e % P);
    const long long r = e / P;
    const int ky = (int)(r % n), kz = (int)(r / n);
    float2 out = make_float2(0.f, 0.f);
    if (kx <= h) {
      const int m2 = sq(signed_freq(kx, n)) + sq(signed_freq(ky, n)) + sq(signed_freq(kz, n));
      const double p = A * (m2 != 0 ? __ldg(&g.shape[m2]) : g.p0);
      const double amp = sqrt(p * g.d2) * g.inv_n3;
      const long long i = ((long long)kz * n + ky) * n + kx;
      const long long j = ((long long)((n - kz) % n) * n + (n - ky) % n) * n + (n - kx) % n;
      const float2 a = box_muller(__ldg(&g.u[i]), __ldg(&g.v[i]));
      const float2 b = box_muller(__ldg(&g.u[j]), __ldg(&g.v[j]));
      out = make_float2((float)(amp * 0.5 * ((double)a.x + (double)b.x)),
                        (float)(amp * 0.5 * ((double)a.y - (double)b.y)));
    }
    g.spec[e] = out;
  }
}

// ---- Zel'dovich displacement spectrum (zeldovich.py:17-69) ------------------------------
struct ZelArgs {
  int n, pitch, dir;   // dir: axis of the (n, n, n) array (0 = slowest, the z of [z][y][x])
  const double* kax;   // l(m) = (2 pi N_PARTS / BOX) * fftfreq(N_PARTS)[m]
  double coef;         // resolution * force_resolution / n^3
  const float2* in;    // fftn of the density (half spectrum)
  float2* out;
};

__global__ void __launch_bounds__(IC_NT) k_zeld_spectrum(ZelArgs z) {
  const int n = z.n, P = z.pitch, h = n / 2;
  const long long total = (long long)n * n * P;
  for (long long e = (long long)blockIdx.x * IC_NT + threadIdx.x; e < total; e += (long long)gridDim.x * IC_NT) {
    const int kx = (int)(e % P);
    const long long r = e / P;
    const int ky = (int)(r % n), kz = (int)(r / n);
    float2 o = make_float2(0.f, 0.f);
    const int kd = z.dir == 0 ? kz : (z.dir == 1 ? ky : kx);
    if (kx <= h && kd != h && (kx | ky | kz) != 0) {
      const double lx = __ldg(&z.kax[kx]), ly = __ldg(&z.kax[ky]), lz = __ldg(&z.kax[kz]);
      const double l2 = __dadd_rn(__dadd_rn(__dmul_rn(lx, lx), __dmul_rn(ly, ly)), __dmul_rn(lz, lz));
      const double ld = z.dir == 0 ? lz : (z.dir == 1 ? ly : lx);
      const double gd = ld * z.coef / l2;
      const float2 v = z.in[e];
      // i * g * v
      o = make_float2((float)(-gd * (double)v.y), (float)(gd * (double)v.x));
    }
    z.out[e] = o;
  }
}

// ---- numpy PCG64 (128-bit LCG, XSL-RR output) -------------------------------------------
typedef unsigned __int128 u128;

__host__ __device__ __forceinline__ u128 pcg_mult() {
  return ((u128)0x2360ED051FC65DA4ull << 64) | (u128)0x4385DF649FCCF645ull;
}

// State after `delta` more steps of state' = state * M + inc (Brown's jump-ahead).
__host__ __device__ inline u128 pcg_advance(u128 state, u128 inc, unsigned long long delta) {
  u128 cur_mult = pcg_mult(), cur_plus = inc, acc_mult = 1, acc_plus = 0;
  while (delta > 0) {
    if (delta & 1ull) {
      acc_mult *= cur_mult;
      acc_plus = acc_plus * cur_mult + cur_plus;
    }
    cur_plus = (cur_mult + 1) * cur_plus;
    cur_mult *= cur_mult;
    delta >>= 1;
  }
  return acc_mult * state + acc_plus;
}

__host__ __device__ __forceinline__ unsigned long long pcg_output(u128 s) {
  const unsigned long long x = (unsigned long long)(s >> 64) ^ (unsigned long long)s;
  const unsigned rot = (unsigned)(s >> 122);
  return (x >> rot) | (x << ((64u - rot) & 63u));
}

// uniform(-2, 2) of numpy's Generator: -2 + 4 * ((next >> 11) * 2^-53)
__device__ __forceinline__ double jitter_value(unsigned long long x) {
  return __dadd_rn(-2.0, __dmul_rn(4.0, (double)(x >> 11) * (1.0 / 9007199254740992.0)));
}

// numpy float remainder: fmod, moved into the divisor's sign
__device__ __forceinline__ double py_mod(double a, double b) {
  double m = fmod(a, b);
  if (m != 0.0) {
    if ((b < 0.0) != (m < 0.0)) m += b;
  } else {
    m = copysign(0.0, b);
  }
  return m;
}

struct PartArgs {
  int n, dir;
  long long np;          // n^3
  const float* disp;     // displacement field along dir (n^3, already * force_resolution)
  const double* space;   // lattice coordinate per axis index (zeldovich.py:79)
  double lin;            // Dt(A_INIT)
  double vcoef;          // A_INIT * f_0 * h_0 * Dt
  double ncells;
  unsigned long long st_hi, st_lo, inc_hi, inc_lo;  // PCG64 state before the first draw
  float* pos;            // row dir of (3, np)
  float* vel;
};

__global__ void __launch_bounds__(IC_NT) k_zeld_particles(PartArgs a) {
  const long long chunks = (a.np + JIT_CHUNK - 1) / JIT_CHUNK;
  const u128 st0 = ((u128)a.st_hi << 64) | a.st_lo, inc = ((u128)a.inc_hi << 64) | a.inc_lo;
  const long long nn = (long long)a.n * a.n;
  for (long long c = (long long)blockIdx.x * IC_NT + threadIdx.x; c < chunks; c += (long long)gridDim.x * IC_NT) {
    const long long p0 = c * JIT_CHUNK;
    // draw number dir * np + p0 is the (dir * np + p0 + 1)-th step of the generator
    u128 s = pcg_advance(st0, inc, (unsigned long long)(a.dir * a.np + p0));
    for (int k = 0; k < JIT_CHUNK && p0 + k < a.np; ++k) {
      const long long p = p0 + k;
      s = s * pcg_mult() + inc;
      const double jit = jitter_value(pcg_output(s));
      const int id = a.dir == 0 ? (int)(p / nn) : (a.dir == 1 ? (int)((p / a.n) % a.n) : (int)(p % a.n));
      const double d = (double)__ldg(&a.disp[p]);
      double x = __dadd_rn(__ldg(&a.space[id]), __dmul_rn(a.lin, d));
      x = __dadd_rn(x, jit);
      a.pos[p] = (float)py_mod(x, a.ncells);
      a.vel[p] = (float)__dmul_rn(a.vcoef, d);
    }
  }
}

}  // namespace

struct pm_ics {
  int n = 0, device = 0, sms = 1, m2max = 0;
  Tables tab;
  DBuf d_sim, d_prefix, d_maps, d_err;
  DBuf spec_a, spec_b, grid, shape, partial, norm, kax, space;
  bool maps_ok = false;
  std::vector<double> h_kax, h_space;
  Sim h_sims[2];
  int h_err = 0;
  std::string err;
};

namespace {

int ic_fail(pm_ics* g, int code, const std::string& msg) {
  if (g) g->err = msg;
  return code;
}

int ic_cuda(pm_ics* g, cudaError_t e, const char* where) {
  return ic_fail(g, e == cudaErrorMemoryAllocation ? PM_ERR_OOM : PM_ERR_CUDA,
                 std::string(where) + ": " + cudaGetErrorString(e));
}

#define IC_CK(call, where)                                 \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return ic_cuda(g, e_, where);   \
  } while (0)

// cosmology.py:11-36 with the cosmology list [OMEGA_M0, OMEGA_LAMBDA0, OMEGA_K0]
double cosmo_H(double a, double h0, double om, double ol, double ok) {
  return std::sqrt(std::pow(h0, 2.0) * (om / std::pow(a, 3.0) + ok / std::pow(a, 2.0) + ol));
}
double cosmo_Dt(double a, double om, double ol, double ok) {
  (void)ok;
  return 5.0 / 2.0 / om / (std::pow(om, 4.0 / 7.0) - ol + (1.0 + om / 2.0) * (1.0 + ol / 70.0)) * a;
}

}  // namespace

extern "C" {

int pm_ics_create(int n_parts, int device, pm_ics** out) {
  if (!out) return PM_ERR_ARG;
  *out = nullptr;
  if (!spectral_supported(n_parts)) return PM_ERR_ARG;
  pm_ics* g = new pm_ics();
  g->n = n_parts;
  g->device = device;
  const int n = n_parts, h = n / 2;
  g->m2max = 3 * h * h;
  const size_t sb = (size_t)n * n * spec_pitch(n) * sizeof(float2);
  cudaError_t e = cudaSetDevice(device);
  if (!e) g->sms = sm_count(device);
  if (!e) e = g->tab.build(n);
  if (!e) e = g->d_sim.ensure(2 * sizeof(Sim));
  if (!e) e = g->d_prefix.ensure(4 * sizeof(int));
  if (!e) e = g->d_err.ensure(sizeof(int));
  if (!e) e = g->spec_a.ensure(sb);
  if (!e) e = g->spec_b.ensure(sb);
  if (!e) e = g->grid.ensure((size_t)n * n * n * sizeof(float));
  if (!e) e = g->shape.ensure((size_t)(g->m2max + 1) * sizeof(double));
  if (!e) e = g->partial.ensure(NORM_BLOCKS * sizeof(double));
  if (!e) e = g->norm.ensure(sizeof(double));
  if (!e) e = g->kax.ensure(n * sizeof(double));
  if (!e) e = g->space.ensure(n * sizeof(double));
  if (!e) e = cudaMemset(g->d_err.p, 0, sizeof(int));
  if (!e) {
    const int units_x = (int)spectral_units(SPEC_X_R2C, n), units_l = (int)spectral_units(SPEC_Y_FWD, n);
    const int pre[4] = {0, units_x, 0, units_l};
    e = cudaMemcpy(g->d_prefix.p, pre, sizeof(pre), cudaMemcpyHostToDevice);
  }
  if (!e) {
    CUtensorMap m[4];
    if (spectral_encode_maps(n, g->spec_a.p, m) && spectral_encode_maps(n, g->spec_b.p, m + 2)) {
      e = g->d_maps.ensure(sizeof(m));
      if (!e) e = cudaMemcpy(g->d_maps.p, m, sizeof(m), cudaMemcpyHostToDevice);
      if (!e) g->maps_ok = true;
    }
  }
  if (!e) e = spectral_dispatch(SPEC_PREPARE, n, nullptr, Work(), 0, nullptr);
  if (!e) e = cudaDeviceSynchronize();
  if (e) {
    pm_ics_destroy(g);
    return e == cudaErrorMemoryAllocation ? PM_ERR_OOM : PM_ERR_CUDA;
  }
  *out = g;
  return PM_OK;
}

void pm_ics_destroy(pm_ics* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  DBuf* bufs[] = {&g->d_sim, &g->d_prefix, &g->d_maps, &g->d_err, &g->spec_a, &g->spec_b, &g->grid,
                  &g->shape, &g->partial, &g->norm, &g->kax, &g->space};
  for (DBuf* b : bufs) b->release();
  g->tab.release();
  delete g;
}

const char* pm_ics_last_error(const pm_ics* g) { return g ? g->err.c_str() : "null initial-conditions object"; }

int pm_ics_generate(pm_ics* g, const pm_config* cfg, const pm_ic_params* ic, const float* u, const float* v,
                    float* positions, float* velocities, float* grf, void* stream) {
  if (!g) return PM_ERR_ARG;
  if (!cfg || !ic || !u || !v || !positions || !velocities) return ic_fail(g, PM_ERR_ARG, "null argument");
  if (cfg->n_parts != g->n) return ic_fail(g, PM_ERR_ARG, "n_parts differs from the object's size");
  if (cfg->n_cells <= 0 || !(cfg->box_size > 0.0) || !(cfg->omega_m0 != 0.0) || !(cfg->a_init > 0.0))
    return ic_fail(g, PM_ERR_ARG, "invalid configuration");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  IC_CK(cudaSetDevice(g->device), "set device");
  const int n = g->n, pitch = spec_pitch(n);
  const long long np = (long long)n * n * n;
  const double om = cfg->omega_m0, ob = cfg->omega_b0, ok = cfg->omega_k0, ol = cfg->omega_lambda0,
               h0 = cfg->h0, a0 = cfg->a_init, box = cfg->box_size, ncells = cfg->n_cells;

  // host tables: Fourier axis l(m) and lattice coordinates, in numpy's operation order
  g->h_kax.resize(n);
  g->h_space.resize(n);
  const double scale = 2.0 * M_PI * n / box, inv_n = 1.0 / n;
  for (int m = 0; m < n; ++m) g->h_kax[m] = scale * ((double)(m < (n + 1) / 2 ? m : m - n) * inv_n);
  const double res = ncells / n, stop = ncells - res, step = n > 1 ? stop / (n - 1) : 0.0;
  for (int i = 0; i < n; ++i) g->h_space[i] = (i == n - 1 && n > 1 ? stop : i * step) + 0.5;
  IC_CK(cudaMemcpyAsync(g->kax.p, g->h_kax.data(), n * sizeof(double), cudaMemcpyHostToDevice, st), "kax");
  IC_CK(cudaMemcpyAsync(g->space.p, g->h_space.data(), n * sizeof(double), cudaMemcpyHostToDevice, st), "space");

  Sim s[2]{};
  for (int k = 0; k < 2; ++k) {
    s[k].n = n;
    s[k].pitch = pitch;
    s[k].s2 = g->tab.s2.as<float>();
    s[k].tw = g->tab.tw.as<float2>();
  }
  s[0].rho = g->grid.as<float>();   // forward transform of the field
  s[0].spec = g->spec_a.as<float2>();
  s[1].spec = g->spec_b.as<float2>();  // inverse transforms into the field buffer
  s[1].phi = g->grid.as<float>();
  g->h_sims[0] = s[0];
  g->h_sims[1] = s[1];
  IC_CK(cudaMemcpyAsync(g->d_sim.p, g->h_sims, sizeof(g->h_sims), cudaMemcpyHostToDevice, st), "sims");

  // power spectrum normalisation
  Shape sp;
  sp.kscale = 2.0 * M_PI / box;
  sp.gamma = om * h0 * std::exp(-ob - ob / om);
  sp.power = ic->power;
  sp.lcdm = ic->lcdm_transfer ? 1 : 0;
  k_shape<<<(g->m2max + 256) / 256, 256, 0, st>>>(g->shape.as<double>(), g->m2max, sp);
  IC_CK(cudaGetLastError(), "shape");
  k_norm_partial<<<NORM_BLOCKS, NORM_NT, 0, st>>>(g->shape.as<double>(), n, g->partial.as<double>());
  IC_CK(cudaGetLastError(), "norm");
  const double npix = (double)np;
  k_norm_final<<<1, NORM_NT, 0, st>>>(g->partial.as<double>(), 64.0 * std::pow(h0, 2.0) * (npix * npix),
                                      g->norm.as<double>());
  IC_CK(cudaGetLastError(), "norm final");

  const double lin = cosmo_Dt(a0, om, ol, ok);
  GrfArgs ga;
  ga.n = n;
  ga.pitch = pitch;
  ga.u = u;
  ga.v = v;
  ga.shape = g->shape.as<double>();
  ga.norm = g->norm.as<double>();
  // P(k = 0) / A: the reference's k**POWER * lcdm (or div) at k = 0
  ga.p0 = (ic->power >= 0.0 && !ic->lcdm_transfer && ic->power == 0.0) ? 1.0 : 0.0;
  ga.d2 = lin * lin;
  ga.inv_n3 = 1.0 / npix;
  ga.spec = g->spec_b.as<float2>();
  const int ew = grid_for(((long long)n * n * pitch + IC_NT - 1) / IC_NT, g->sms, 8);
  k_grf_fill<<<ew, IC_NT, 0, st>>>(ga);
  IC_CK(cudaGetLastError(), "grf fill");

  const Sim* ds = g->d_sim.as<Sim>();
  const CUtensorMap* maps = g->maps_ok ? g->d_maps.as<CUtensorMap>() : nullptr;
  int* err = g->d_err.as<int>();
  const int* pre = g->d_prefix.as<int>();
  Work wx{pre, 1, (int)spectral_units(SPEC_X_R2C, n)}, wl{pre + 2, 1, (int)spectral_units(SPEC_Y_FWD, n)};
  const int gx = grid_for(wx.total, g->sms, 8), gl = grid_for(wl.total, g->sms, 8);
  auto inverse = [&](const char* what) -> int {  // spec_b -> grid
    const CUtensorMap* mb = maps ? maps + 2 : nullptr;
    IC_CK(spectral_dispatch(SPEC_Z_INV, n, ds + 1, wl, gl, st, mb, err), what);
    IC_CK(spectral_dispatch(SPEC_Y_INV, n, ds + 1, wl, gl, st, mb, err), what);
    IC_CK(spectral_dispatch(SPEC_X_C2R, n, ds + 1, wx, gx, st, mb, err), what);
    return PM_OK;
  };
  int rc = inverse("grf inverse");
  if (rc) return rc;
  if (grf)
    IC_CK(cudaMemcpyAsync(grf, g->grid.p, (size_t)np * sizeof(float), cudaMemcpyDeviceToDevice, st), "grf out");

  // fftn of the field (zeldovich.py:17)
  IC_CK(spectral_dispatch(SPEC_X_R2C, n, ds, wx, gx, st, maps, err), "r2c");
  IC_CK(spectral_dispatch(SPEC_Y_FWD, n, ds, wl, gl, st, maps, err), "y fwd");
  IC_CK(spectral_dispatch(SPEC_Z_FWD, n, ds, wl, gl, st, maps, err), "z fwd");

  const double fres = ncells / box;
  const double f0 = 1.0 / std::sqrt((om + ok * a0 + ol * std::pow(a0, 3.0)) / a0);
  const double hh = cosmo_H(a0, h0, om, ol, ok);
  for (int d = 0; d < 3; ++d) {
    ZelArgs za;
    za.n = n;
    za.pitch = pitch;
    za.dir = d;
    za.kax = g->kax.as<double>();
    za.coef = res * fres / npix;
    za.in = g->spec_a.as<float2>();
    za.out = g->spec_b.as<float2>();
    k_zeld_spectrum<<<ew, IC_NT, 0, st>>>(za);
    IC_CK(cudaGetLastError(), "displacement spectrum");
    rc = inverse("displacement inverse");
    if (rc) return rc;
    PartArgs pa;
    pa.n = n;
    pa.dir = d;
    pa.np = np;
    pa.disp = g->grid.as<float>();
    pa.space = g->space.as<double>();
    pa.lin = lin;
    pa.vcoef = a0 * f0 * hh * lin;
    pa.ncells = ncells;
    pa.st_hi = ic->jitter_state[0];
    pa.st_lo = ic->jitter_state[1];
    pa.inc_hi = ic->jitter_inc[0];
    pa.inc_lo = ic->jitter_inc[1];
    pa.pos = positions + d * np;
    pa.vel = velocities + d * np;
    const int pw = grid_for(((np + JIT_CHUNK - 1) / JIT_CHUNK + IC_NT - 1) / IC_NT, g->sms, 8);
    k_zeld_particles<<<pw, IC_NT, 0, st>>>(pa);
    IC_CK(cudaGetLastError(), "particles");
  }
  // device-side checks of the TMA passes (bounded waits): read back once
  IC_CK(cudaMemcpyAsync(&g->h_err, g->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st), "err");
  IC_CK(cudaStreamSynchronize(st), "sync");
  const int bits = g->h_err;
  if (bits) {
    cudaMemsetAsync(g->d_err.p, 0, sizeof(int), st);
    return ic_fail(g, PM_ERR_DEVICE, "device check failed in the spectral passes (bits " + std::to_string(bits) + ")");
  }
  return PM_OK;
}

}  // extern "C"
