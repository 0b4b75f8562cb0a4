/*
 * Multi-threaded CPU restatement of the reference's particle loops, for the CPU baseline.
 *
 * TEST INFRASTRUCTURE ONLY (part of the oracle): called by bench.py's cpu_baseline /
 * --impl reference leg and by the tests that check it against oracle/pm_oracle.py; the
 * product never links it.  It restates, in float64 with OpenMP threads over particles (the
 * reference parallelises the same loops with numba prange over N_CPU threads):
 *
 *   cpu_density    src/density.py:7-48      CIC deposit onto grid[z][y][x]; the reference's
 *                                           racy += becomes an atomic add (order-dependent
 *                                           rounding in the last bits, like the reference)
 *   cpu_integrate  src/integrate.py:15-97   cell centres and weights from the positions,
 *                                           then per axis the CIC-weighted central difference
 *                                           of phi at the 8 corners (integrate.py:54-92),
 *                                           kick, drift, wrap (integrate.py:94-95)
 *
 * Positions and velocities are float32 (3, np) arrays as in the reference; the potential
 * is float64 (the reference's complex128 FFT output, real part).  The FFT step between
 * them (potential.py) runs in scipy.fft with the same threads.  Positions are first mapped
 * into [0, n) (the engine's decision for the x == n case, quirk Q4 of oracle/pm_oracle.py).
 */
#include <math.h>
#include <stddef.h>

static inline float canon(float x, float fn) {
  if (x >= fn) x -= fn;
  if (x < 0.f) x += fn;
  if (x >= fn) x = 0.f;
  return x;
}

static inline void cell_of(const float* pos, long long np, long long i, int n, long long c[3], double d[3]) {
  const float fn = (float)n;
  for (int k = 0; k < 3; ++k) {
    const float p = canon(pos[k * np + i], fn);
    const double fl = floor((double)p);
    long long ci = (long long)fl % n;
    if (ci < 0) ci += n;
    c[k] = ci;
    d[k] = (double)p - (double)ci;
  }
}

/* the 8 weights in the order of integrate.py:44-51 and their corner offsets */
static const int CX[8] = {0, 1, 0, 0, 1, 1, 0, 1};
static const int CY[8] = {0, 0, 1, 0, 1, 0, 1, 1};
static const int CZ[8] = {0, 0, 0, 1, 0, 1, 1, 1};

static inline void weights(const double d[3], double w[8]) {
  const double tx = 1.0 - d[0], ty = 1.0 - d[1], tz = 1.0 - d[2];
  w[0] = tx * ty * tz;
  w[1] = d[0] * ty * tz;
  w[2] = tx * d[1] * tz;
  w[3] = tx * ty * d[2];
  w[4] = d[0] * d[1] * tz;
  w[5] = d[0] * ty * d[2];
  w[6] = tx * d[1] * d[2];
  w[7] = d[0] * d[1] * d[2];
}

void cpu_density(const float* pos, long long np, int n, double mass, double* grid) {
  const long long n3 = (long long)n * n * n;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n3; ++i) grid[i] = 0.0;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < np; ++i) {
    long long c[3];
    double d[3], w[8];
    cell_of(pos, np, i, n, c, d);
    weights(d, w);
    for (int k = 0; k < 8; ++k) {
      const long long x = (c[0] + CX[k]) % n, y = (c[1] + CY[k]) % n, z = (c[2] + CZ[k]) % n;
      const double v = mass * w[k];
#pragma omp atomic
      grid[(z * n + y) * n + x] += v;
    }
  }
}

void cpu_integrate(float* pos, float* vel, long long np, int n, const double* phi, double a, double fa1, double da) {
  const double drift = da / ((a + da) * (a + da)) * fa1;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < np; ++i) {
    long long c[3];
    double d[3], w[8];
    cell_of(pos, np, i, n, c, d);
    weights(d, w);
    for (int ax = 0; ax < 3; ++ax) {
      double acc = 0.0;
      for (int k = 0; k < 8; ++k) {
        long long m[3] = {c[0] + CX[k], c[1] + CY[k], c[2] + CZ[k]};
        long long p[3] = {m[0], m[1], m[2]};
        m[ax] -= 1;
        p[ax] += 1;
        for (int q = 0; q < 3; ++q) {
          m[q] = ((m[q] % n) + n) % n;
          p[q] = ((p[q] % n) + n) % n;
        }
        acc += w[k] * (phi[(m[2] * n + m[1]) * n + m[0]] - phi[(p[2] * n + p[1]) * n + p[0]]);
      }
      const double g = acc / 2.0;
      const double v = (double)vel[ax * np + i] + da * fa1 * g;
      double x = fmod((double)pos[ax * np + i] + v * drift, (double)n);
      if (x < 0) x += n;
      vel[ax * np + i] = (float)v;
      pos[ax * np + i] = (float)x;
    }
  }
}
