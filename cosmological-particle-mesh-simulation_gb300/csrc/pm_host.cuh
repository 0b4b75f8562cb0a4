// Host-side helpers shared by the context (drop-in API) and the batch engine.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pm_common.cuh"
#include "pm_gb300.h"

namespace pm {

constexpr int TILE_Y = 4, TILE_Z = 4;

inline int ceil_log2(long long v) {
  int b = 0;
  while ((1ll << b) < v) ++b;
  return b;
}

inline int spec_pitch(int n) { return ((n / 2 + 1) + 15) / 16 * 16; }

inline bool grid_supported(int n) { return spectral_supported(n) && n % TILE_Y == 0 && n % TILE_Z == 0; }

// Growable device buffer.
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t b) {
    if (b <= bytes && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, b > 0 ? b : 16);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  // as ensure, but growing to at least 3/2 of the current size: fewer reallocations (and so
  // fewer cudaFree calls, each of which synchronises the device) for sizes that creep up
  cudaError_t ensure_geo(size_t b) {
    if (b <= bytes && p) return cudaSuccess;
    return ensure(b > bytes + bytes / 2 ? b : bytes + bytes / 2);
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

// Per-grid-size tables: s2[m] = sin^2(pi m / n) (fourier_utils.py:9-15 per axis),
// sn[m] = sin(2 pi m / n) (the spectral central difference) and tw[m] = exp(-2 pi i m / n),
// built in double precision on the host.
struct Tables {
  int n = 0;
  DBuf s2, tw, sn;
  cudaError_t build(int nn) {
    if (n == nn && s2.p) return cudaSuccess;
    std::vector<float> hs(nn), hn(nn);
    std::vector<float2> ht(nn);
    for (int m = 0; m < nn; ++m) {
      const double s = std::sin(M_PI * (double)m / nn);
      hs[m] = (float)(s * s);
      hn[m] = (float)std::sin(2.0 * M_PI * (double)m / nn);
      const double ang = -2.0 * M_PI * (double)m / nn;
      ht[m] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
    cudaError_t e = s2.ensure(nn * sizeof(float));
    if (!e) e = tw.ensure(nn * sizeof(float2));
    if (!e) e = sn.ensure(nn * sizeof(float));
    if (!e) e = cudaMemcpy(sn.p, hn.data(), nn * sizeof(float), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(s2.p, hs.data(), nn * sizeof(float), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(tw.p, ht.data(), nn * sizeof(float2), cudaMemcpyHostToDevice);
    if (!e) n = nn;
    return e;
  }
  void release() { s2.release(); tw.release(); sn.release(); n = 0; }
};

// Lagrangian lattice of one axis: q = i * (n_cells / n_parts) + 0.5 (zeldovich.py:79-83),
// split into integer and float32 fractional parts.
struct Lattice {
  int np1 = 0, n = 0;
  DBuf qi, qf;
  cudaError_t build(int nparts, int ncells) {
    if (np1 == nparts && n == ncells && qi.p) return cudaSuccess;
    std::vector<int> hi(nparts);
    std::vector<float> hf(nparts);
    const double r = (double)ncells / nparts;
    for (int i = 0; i < nparts; ++i) {
      const double q = i * r + 0.5;
      const double f = std::floor(q);
      hi[i] = (int)f;
      hf[i] = (float)(q - f);
    }
    cudaError_t e = qi.ensure(nparts * sizeof(int));
    if (!e) e = qf.ensure(nparts * sizeof(float));
    if (!e) e = cudaMemcpy(qi.p, hi.data(), nparts * sizeof(int), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(qf.p, hf.data(), nparts * sizeof(float), cudaMemcpyHostToDevice);
    if (!e) { np1 = nparts; n = ncells; }
    return e;
  }
  void release() { qi.release(); qf.release(); np1 = n = 0; }
};

// Sort scratch sized for n elements.
struct SortBufs {
  DBuf keys, vals, keys_alt, vals_alt, hist, digit_tot;
  long long cap = 0;
  cudaError_t ensure(long long n) {
    if (n <= cap && keys.p) return cudaSuccess;
    const size_t b = (size_t)(n > 0 ? n : 1) * sizeof(unsigned);
    cudaError_t e = keys.ensure(b);
    if (!e) e = vals.ensure(b);
    if (!e) e = keys_alt.ensure(b);
    if (!e) e = vals_alt.ensure(b);
    if (!e) e = hist.ensure(sort_scratch_hist_entries(n) * sizeof(unsigned));
    if (!e) e = digit_tot.ensure(SORT_DIGIT_TOTALS * sizeof(unsigned));
    if (!e) cap = n;
    return e;
  }
  SortScratch scratch() const {
    SortScratch s;
    s.keys_alt = keys_alt.as<unsigned>();
    s.vals_alt = vals_alt.as<unsigned>();
    s.hist = hist.as<unsigned>();
    s.digit_tot = digit_tot.as<unsigned>();
    s.capacity = cap;
    s.max_blocks = (int)(hist.bytes / sizeof(unsigned) / SORT_DIGIT_TOTALS);
    return s;
  }
  void release() {
    keys.release(); vals.release(); keys_alt.release(); vals_alt.release(); hist.release();
    digit_tot.release();
    cap = 0;
  }
};

// f(a) of cosmology.py:20-27
inline double cosmo_f(double a, double om, double ol, double ok) {
  return 1.0 / std::sqrt((om + ok * a + ol * a * a * a) / a);
}

inline int sm_count(int device) {
  int v = 0;
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
  return v > 0 ? v : 1;
}

inline int grid_for(long long units, int sms, int per_sm) {
  long long c = (long long)sms * per_sm;
  if (units < c) c = units;
  return (int)(c > 0 ? c : 1);
}

}  // namespace pm
