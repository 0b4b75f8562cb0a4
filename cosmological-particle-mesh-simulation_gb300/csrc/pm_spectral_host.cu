// Host-side dispatch of the spectral kernels over the supported grid sizes, and the
// fourier_grid table kernel (fourier_utils.py:5-16 of the reference).
#include "pm_spectral.cuh"

namespace pm {

#define PM_FOR_EACH_N(X) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768) X(1024)

#define PM_EXTERN(NN) extern template cudaError_t spectral_launch<NN>(SpecKind, const Sim*, Work, int, cudaStream_t, const CUtensorMap*, int*);
PM_FOR_EACH_N(PM_EXTERN)
#undef PM_EXTERN
#define PM_EXTERN(NN)                                                                                         \
  extern template cudaError_t deposit_r2c_launch<NN>(const Sim*, Work, Parts, const unsigned*, const unsigned*, \
                                                     int, int*, unsigned*, const unsigned*, int, cudaStream_t);
PM_FOR_EACH_N(PM_EXTERN)
#undef PM_EXTERN

cudaError_t deposit_r2c_dispatch(int n, const Sim* sims, Work w, Parts p, const unsigned* perm,
                                 const unsigned* row_start, int mode, int* err, unsigned* next_tile,
                                 const unsigned* order, int ctas, cudaStream_t st) {
  switch (n) {
#define PM_CASE(NN) \
  case NN: return deposit_r2c_launch<NN>(sims, w, p, perm, row_start, mode, err, next_tile, order, ctas, st);
    PM_FOR_EACH_N(PM_CASE)
#undef PM_CASE
    default: return cudaErrorInvalidValue;
  }
}

bool spectral_encode_maps(int n, const void* spec, CUtensorMap out[2]) {
  if (!tma_lines(n) || !spectral_supported(n)) return false;
  return encode_spectrum_map(&out[0], spec, n, false) && encode_spectrum_map(&out[1], spec, n, true);
}

bool deposit_r2c_supported(int n) { return spectral_supported(n) && deposit_r2c_ok(n); }
bool xrow_supported(int n) { return spectral_supported(n) && xrow_ok(n); }

int deposit_r2c_ctas_per_sm(int n) { return xrow_ok(n) ? 3 : 2; }

bool spectral_supported(int n) {
  switch (n) {
#define PM_CASE(NN) case NN: return true;
    PM_FOR_EACH_N(PM_CASE)
#undef PM_CASE
    default: return false;
  }
}

long long spectral_units(SpecKind kind, int n) {
  if ((kind == SPEC_X_R2C || kind == SPEC_X_C2R) && xrow_ok(n)) return (long long)n * n / xrow_rows_per_warp(n);
  if (kind == SPEC_X_R2C || kind == SPEC_X_C2R) {
    const long long rows = (long long)n * n, nr = cx_rows(n);
    return (rows + nr - 1) / nr;
  }
  const long long nb = (long long)n * cbundles_per_plane(n), bpc = cline_bpc(n);
  return (nb + bpc - 1) / bpc;
}

int spectral_ctas_per_sm(SpecKind kind, int n) {
  const size_t sm = (kind == SPEC_X_R2C || kind == SPEC_X_C2R) ? x_smem_bytes(n) : line_smem_bytes(n);
  int by_smem = (int)((228u * 1024u) / (sm + 1024));
  if (by_smem < 1) by_smem = 1;
  return by_smem > 4 ? 4 : by_smem;
}

cudaError_t spectral_dispatch(SpecKind kind, int n, const Sim* sims, Work w, int ctas, cudaStream_t st,
                              const CUtensorMap* maps, int* err) {
  switch (n) {
#define PM_CASE(NN) case NN: return spectral_launch<NN>(kind, sims, w, ctas, st, maps, err);
    PM_FOR_EACH_N(PM_CASE)
#undef PM_CASE
    default: return cudaErrorInvalidValue;
  }
}

__global__ void k_fourier_grid(const Sim* __restrict__ sims) {
  const Sim& S = sims[0];
  const long long n = S.n, total = n * n * n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % n), y = (int)((i / n) % n), z = (int)(i / (n * n));
    const float den = __ldg(&S.s2[x]) + __ldg(&S.s2[y]) + __ldg(&S.s2[z]);
    S.rho[i] = (den != 0.f) ? 1.0f / den : 0.f;
  }
}

cudaError_t launch_fourier_grid(const Sim* sims, int ctas, cudaStream_t st) {
  k_fourier_grid<<<ctas, 256, 0, st>>>(sims);
  return cudaGetLastError();
}

}  // namespace pm
