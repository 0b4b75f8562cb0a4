// Shared device/host declarations of the GB300 particle-mesh engine.
//
// Data layout in HBM (one simulation):
//   real grids (density, potential)  float  [z][y][x], n^3
//   half spectrum                    float2 [z][y][kx], kx in [0, n/2], row pitch `pitch`
//                                    (a multiple of 16 complex = 128 B)
//   particles                        structure of arrays, one float per axis and
//                                    per quantity (the reference's (3, Np) layout)
// Many simulations share one launch per phase: every kernel receives the device
// array of `Sim` descriptors and a per-phase work prefix (CTA -> simulation).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#define PM_FIX_BITS 26          // CIC weights are accumulated as integers w * 2^26
#define PM_MAX_N 1024

namespace pm {

constexpr int PM_MAX_DEVICES = 64;

// Kernel attributes (dynamic shared-memory limits, carve-outs) are state of each device,
// not of the process: DeviceOnce runs a set-up function once for every device it is called
// on (the current device), under a lock, and remembers the devices whose set-up succeeded.
struct DeviceOnce {
  std::atomic<unsigned long long> done{0};
  std::mutex m;
  template <class F>
  cudaError_t run(F fn) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if (dev < 0 || dev >= PM_MAX_DEVICES) return cudaErrorInvalidDevice;
    const unsigned long long bit = 1ull << dev;
    if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
    std::lock_guard<std::mutex> g(m);
    if (done.load(std::memory_order_relaxed) & bit) return cudaSuccess;
    e = fn();
    if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
    return e;
  }
};

// Streaming multiprocessors of the current device (cached per device).
inline int device_sms() {
  static std::atomic<int> cache[PM_MAX_DEVICES];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= PM_MAX_DEVICES) return 1;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

enum : int {
  ERR_OK = 0,
  ERR_CELL_RANGE = 1,   // a particle cell fell outside the grid (NaN/Inf position)
  ERR_SOURCE_ROW = 2,   // deposit: particle outside the tile's source rows (sort broken)
  ERR_NONFINITE = 4,    // kick/drift produced a non-finite coordinate
  ERR_TIMEOUT = 8,      // a bounded wait on an asynchronous copy gave up
};

enum PosMode : int { POS_ABS = 0, POS_DISP = 1 };

// Device-side description of one simulation.  All pointers are device pointers.
struct Sim {
  int n;            // grid cells per side
  int pitch;        // spectrum row pitch in complex elements
  int np1;          // particles per side of the Lagrangian lattice (0: unknown)
  int xbits;        // bits of x in the cell key
  int ty, tz;       // deposit tile: tz planes x ty rows of full x-rows
  int flags;
  int q_step;       // n / np1 when np1 divides n (lattice q = q_step i + 1/2); 0: use the tables
  long long np;        // particle count
  long long part_off;  // first position of this simulation in the sorted order (and in the
                       // state the kick writes: the batch particle arrays after a step)
  long long slot_off;  // first particle slot of this simulation in the state being read by the
                       // keys kernel (differs from part_off right after a retirement)
  unsigned row_base;   // first global row number of this simulation
  unsigned pad1;
  float* rho;          // density n^3 (output of the deposit)
  float2* spec;        // half spectrum
  float* phi;          // potential n^3
  const float* fgrid;  // optional caller Green table n^3 (nullptr: computed in-kernel)
  const float* s2;     // sin^2(pi m / n), m < n
  const float2* tw;    // exp(-2 pi i m / n), m < n
  const int* q_int;    // lattice coordinate, integer part, np1 entries
  const float* q_frac; // lattice coordinate, fractional part, np1 entries
  const float* sn;     // sin(2 pi m / n), m < n (spectral gradient)
  // spectral gradient: grad_axis = d + 1 makes the z pass multiply by -i sin(k_d) as well as
  // by the Green function, so that the inverse passes give the force grid of axis d; grad, for
  // the kick, holds the three force grids (nullptr: central differences of phi)
  int grad_axis, pad2;
  const float* grad[3];
  // per-step coefficients
  float mass_scale;    // particle mass * 2^-PM_FIX_BITS
  float green;         // -3 Om / (8 a) / n^3
  float kick;          // da * f(a + da)
  float drift;         // da * f(a + da) / (a + da)^2
  // time state (fp64, advanced on the device in resident mode)
  double a, da, om, ol, ok, h0;
  int step, nsteps, active, fix_f;
};

// CTA -> simulation map of one phase: prefix[s] = first work unit of simulation s.
struct Work {
  const int* prefix;  // nsims + 1 entries (device)
  int nsims;
  int total;          // prefix[nsims]
};

// Particle arrays of a batch (structure of arrays, indexed by slot).
struct Parts {
  float* x; float* y; float* z;       // positions (POS_ABS) or displacements (POS_DISP)
  float* vx; float* vy; float* vz;
  unsigned* id;                        // Lagrangian particle index (POS_DISP)
  // cell record (POS_DISP, optional), one 16-byte word per particle: the base cell packed
  // x | y << 10 | z << 20 (CELL_BAD if not finite) and the bits of the three in-cell offsets,
  // exactly as computed from the displacement.  The kick writes it with the state so that the
  // deposit reads the cell instead of recomputing it, with one 16-byte load (four separate
  // arrays measured 0.520 -> 0.485 ms per deposit, 256^3 on 512^3).
  uint4* rec;
};

__device__ __forceinline__ int locate_sim(const Work& w, int unit) {
  int lo = 0, hi = w.nsims - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&w.prefix[mid]) <= unit) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void set_error(int* err, int code) {
  if (err) atomicOr(err, code);
}

// ---------------------------------------------------------------------------------
// Launchers (defined in the .cu files, called by the engine)
// ---------------------------------------------------------------------------------
// spectral passes: one kernel per grid size n (supported n: spectral_supported)
enum SpecKind : int { SPEC_X_R2C = 0, SPEC_Y_FWD, SPEC_Z_GREEN, SPEC_Z_TABLE, SPEC_Y_INV, SPEC_X_C2R,
                      SPEC_Z_FWD, SPEC_Z_INV, /* plain z transforms (initial conditions) */
                      SPEC_Z_GRAD, /* z Green times -i sin(k_d): spectral gradient of axis grad_axis - 1 */
                      SPEC_PREPARE /* only set kernel attributes */ };
// maps: device array of tensor maps, two per simulation of `sims` (y pass, z pass; see
// spectral_encode_maps) -- enables the TMA-streamed line passes; nullptr falls back to
// plain loads.  Every kernel finds its simulation through the work prefix.
template <int N>
cudaError_t spectral_launch(SpecKind kind, const Sim* sims, Work w, int ctas, cudaStream_t st,
                            const CUtensorMap* maps, int* err);
// Encodes the y- and z-pass tensor maps of a half spectrum of size n (false if n has no
// TMA line pass).
bool spectral_encode_maps(int n, const void* spec, CUtensorMap out[2]);
bool spectral_supported(int n);
// work units (CTAs' worth of work) of one spectral pass for a grid of size n
long long spectral_units(SpecKind kind, int n);
// resident CTAs per SM of a spectral pass for size n (for persistent grid sizing)
int spectral_ctas_per_sm(SpecKind kind, int n);
cudaError_t spectral_dispatch(SpecKind kind, int n, const Sim* sims, Work w, int ctas, cudaStream_t st,
                              const CUtensorMap* maps = nullptr, int* err = nullptr);
cudaError_t launch_fourier_grid(const Sim* sims, int ctas, cudaStream_t st);
// fused deposit + x R2C (the density grid is not written); ctas <= 0 only prepares.
// next_tile: one device word, the tile counter (zeroed on `st` before the launch); nullptr:
// CTAs take every ctas-th tile.  order (optional, w.total entries): the tiles in the order to
// take them (launch_tile_order).
template <int N>
cudaError_t deposit_r2c_launch(const Sim* sims, Work w, Parts p, const unsigned* perm, const unsigned* row_start,
                               int mode, int* err, unsigned* next_tile, const unsigned* order, int ctas,
                               cudaStream_t st);
bool deposit_r2c_supported(int n);
bool xrow_supported(int n);  // the x passes of size n transform rows in registers (their grid is tunable)
int deposit_r2c_ctas_per_sm(int n);  // resident CTAs per SM of the fused deposit
cudaError_t deposit_r2c_dispatch(int n, const Sim* sims, Work w, Parts p, const unsigned* perm,
                                 const unsigned* row_start, int mode, int* err, unsigned* next_tile,
                                 const unsigned* order, int ctas, cudaStream_t st);

// sum of the first n_slices planes of an n^3 grid, float64 n^2 output (pm_diagnostics.cu)
cudaError_t launch_project(const float* rho, int n, int n_slices, double* out, int ctas, cudaStream_t st);
// shell-averaged power spectrum of a half spectrum (pm_diagnostics.cu): out = (k, P, modes) for bins
// 1 .. nbins - 1; nbins <= n / 2 + 1; partial holds pk_partial_doubles(nbins) doubles
int pk_ctas();
size_t pk_partial_doubles(int nbins);
cudaError_t launch_power_spectrum(const float2* spec, int n, int pitch, int nbins, double box, double* partial,
                                  double* out, cudaStream_t st);

// particle kernels
cudaError_t launch_keys_abs(const Sim* sims, const Work& w, Parts p, unsigned* keys, unsigned* vals,
                            int* err, int ctas, cudaStream_t st, Parts copy = Parts{});
cudaError_t launch_keys_disp(const Sim* sims, const Work& w, Parts p, unsigned* keys, unsigned* vals,
                             int* err, int ctas, cudaStream_t st);
cudaError_t launch_row_start(const unsigned* keys, long long n, int xbits, unsigned nrows,
                             unsigned* row_start, cudaStream_t st);
cudaError_t launch_deposit(const Sim* sims, const Work& w, Parts p, const unsigned* perm,
                           const unsigned* row_start, int mode, int* err, int ctas, size_t smem,
                           cudaStream_t st);
constexpr int KICK_UNIT = 512;  // particles per work unit of the kick
// row_count (displacement mode, with keys_next): the kick also counts the next keys per row
cudaError_t launch_kick(const Sim* sims, const Work& w, Parts in, Parts out, const unsigned* perm,
                        unsigned* keys_next, int mode, int* err, int ctas, cudaStream_t st,
                        unsigned* row_count = nullptr);
cudaError_t launch_coef(Sim* sims, int nsims, int advance, cudaStream_t st);
// dst[k][j] = src[k][idx[j]] for the three rows of (3, np) positions (and velocities unless
// vel is null)
cudaError_t launch_gather_state(const float* pos, const float* vel, long long np, const unsigned* idx, float* spos,
                                float* svel, int sms, cudaStream_t st);
cudaError_t deposit_prepare();  // sets kernel attributes of the current device (call before graph capture)
// order of the fused deposit's tiles (dense tiles first); counts: 2 device words of scratch
cudaError_t launch_tile_order(const Sim* sims, const Work& w, const unsigned* row_start, unsigned* order,
                              unsigned* counts, int sms, cudaStream_t st);
cudaError_t launch_abs_to_disp(const float* pos, const float* vel, long long np, int np1, int n,
                               const int* q_int, const float* q_frac, Parts out, long long off,
                               cudaStream_t st, const unsigned* order = nullptr);
// keys[i] = x-row (tile order) of the cell of absolute position i (n^2 rows)
cudaError_t launch_row_keys_abs(const float* pos, long long np, int n, unsigned* keys, cudaStream_t st);
cudaError_t launch_disp_to_abs(Parts in, long long off, long long np, int np1, int n, const int* q_int,
                               const float* q_frac, float* pos, float* vel, cudaStream_t st);
size_t deposit_smem_bytes(int n, int ty, int tz);

// radix sort of (key, value) pairs, stable, LSD, digits of up to 9 bits
struct SortScratch {
  unsigned* keys_alt; unsigned* vals_alt;
  unsigned* hist;     // 256 * max_blocks
  unsigned* digit_tot;
  long long capacity; int max_blocks;
};
constexpr int SORT_TILE = 4096;
size_t sort_scratch_hist_entries(long long n);
constexpr int SORT_DIGIT_TOTALS = 512;  // entries of SortScratch::digit_tot
int radix_sort_passes(int bits);
// sets the sort's kernel attributes on the current device (once per device; radix_sort calls it)
cudaError_t sort_prepare();
// Sorts keys[0,n) / vals[0,n) on key bits [begin_bit, begin_bit + bits).  Returns via
// *in_alt whether the result sits in the scratch (alt) buffers.  When gen_vals is set,
// vals are not read on the first pass and the identity 0..n-1 is used instead.
cudaError_t radix_sort(unsigned* keys, unsigned* vals, long long n, int begin_bit, int bits, bool gen_vals,
                       const SortScratch& s, bool* in_alt, cudaStream_t st);
// Groups n row keys (< nrows) by row: row_start[0..nrows] (exclusive prefix of the row
// counts) and perm[j] = index of the j-th key in row order (order inside a row not
// specified).  Scratch: count and cursor (nrows each), block_sums (row_sort_block_sums).
size_t row_sort_block_sums(unsigned nrows);
// inv (optional): inv[i] = sorted position of key i.  counted: count already holds the
// row histogram of keys (else it is zeroed and computed here).
cudaError_t row_counting_sort(const unsigned* keys, long long n, unsigned nrows, unsigned* count,
                              unsigned* row_start, unsigned* cursor, unsigned* block_sums, unsigned* perm, int* err,
                              int sms, cudaStream_t st, unsigned* inv = nullptr, bool counted = false);
// count[r] = number of keys equal to r (count zeroed first)
cudaError_t row_histogram(const unsigned* keys, long long n, unsigned nrows, unsigned* count, int* err, int sms,
                          cudaStream_t st);

}  // namespace pm
