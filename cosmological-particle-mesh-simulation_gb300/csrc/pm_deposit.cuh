// Deterministic CIC deposit of one tile (density.py:7-48 of the reference).
//
// A tile is TZ x TY full x-rows.  The particles whose base cell lies in the tile's source
// rows (the tile plus one row and one plane below, periodic: 7 runs of the row-sorted
// order) are found through the row starts; their CIC weights that land inside the tile are
// added to integer accumulators in shared memory (TileSum: one 32-bit word per cell where the
// tile's particle count allows, else a low word and a coarse word).  Integer sums do not
// depend on the order of the atomics, so the deposit is bit-identical run to run.
#pragma once
#include <type_traits>

#include "pm_cells.cuh"

namespace pm {

constexpr int DEP_NT = 512;
constexpr int DEP_ROW_NT = 256;  // fused deposit with the register row transform

constexpr int COARSE_SHIFT = 12;

__device__ __forceinline__ void acc_add(unsigned* lo, unsigned* co, int i, unsigned q) {
  atomicAdd(&lo[i], q);  // results unused: non-returning shared-memory reductions
  atomicAdd(&co[i], q >> COARSE_SHIFT);
}

// The exact sum V from its low word l and its coarse sum c, rounded to float32, times scale.
// V - (c << 12) lies in [0, 2^32), so V = (c << 12) + (l - (c << 12) mod 2^32): its low word
// is l and its high word is c >> 20 plus the carry of that addition.  V < 2^44, so
// V = a 2^23 + b with a, b < 2^23; each is exact as a float (2^23 + a has a as its
// mantissa), and fmaf(a, 2^23, b) rounds once: the value of a round-to-nearest 64-bit
// conversion, computed on the FP32 pipe (GB300 issues 64-bit integer conversions to its
// narrow FP64 pipe).
__device__ __forceinline__ float fixed_to_float(unsigned l, unsigned c, float scale) {
  const unsigned est_lo = c << COARSE_SHIFT;
  const unsigned hi = (c >> (32 - COARSE_SHIFT)) + (l < est_lo ? 1u : 0u);
  const unsigned a = (hi << 9) | (l >> 23), b = l & 0x7fffffu;
  const float fa = __uint_as_float(0x4B000000u | a) - 8388608.f;
  const float fb = __uint_as_float(0x4B000000u | b) - 8388608.f;
  return fmaf(fa, 8388608.f, fb) * scale;
}

// How a tile's sums are held.  Every corner weight is quantised to an integer q <= 2^s and
// added with integer atomics, so a cell's sum -- and the float made from it -- does not depend
// on the order of the additions.  A cell receives at most one corner from each source entry
// of its tile, so its sum is at most total * 2^s: a tile with total < 2^(32 - s) sums in one
// 32-bit word per cell (one atomic per corner).  Tiles whose count allows s >= ONE_WORD_MIN
// use one word at the largest such s (at most 26); denser tiles sum at 2^-26 in a low word
// plus a coarse word (two atomics per corner).
constexpr int ONE_WORD_MIN = 20;

struct TileSum {
  int s;     // one-word quantisation 2^s; 0: two-word sums at 2^-26
  float ms;  // particle mass * 2^-(quantisation bits): the float of a sum times ms is its mass
};

__device__ __forceinline__ TileSum tile_sum(unsigned total, float mass_scale) {
  const int bits = 32 - __clz(total);  // total < 2^bits
  const int s = min(PM_FIX_BITS, 32 - bits);
  TileSum t;
  t.s = s >= ONE_WORD_MIN ? s : 0;
  // mass_scale = mass * 2^-26; one-word sums at 2^-s: times 2^(26 - s), exactly
  t.ms = t.s ? mass_scale * __uint_as_float((unsigned)(127 + PM_FIX_BITS - t.s) << 23) : mass_scale;
  return t;
}

// A one-word sum as a float, times scale (exact split l = a 2^23 + b, one rounding).
__device__ __forceinline__ float word_to_float(unsigned l, float scale) {
  const float fa = __uint_as_float(0x4B000000u | (l >> 23)) - 8388608.f;
  const float fb = __uint_as_float(0x4B000000u | (l & 0x7fffffu)) - 8388608.f;
  return fmaf(fa, 8388608.f, fb) * scale;
}

// The float of a cell's sum: low word l (and, for two-word tiles, coarse word c).
__device__ __forceinline__ float sum_to_float(const TileSum& t, unsigned l, unsigned c) {
  return t.s ? word_to_float(l, t.ms) : fixed_to_float(l, c, t.ms);
}

// Adds the 8 quantised weights q of a particle with base cell (cx, ly, lz) (ly, lz relative
// to the tile, in [-1, TY-1] x [-1, TZ-1]) to the tile accumulators; tile row r of lo / hi
// starts at word r * rs.  The corners go row by row (weights 0 1 | 2 4 | 3 5 | 6 7 of the
// order of cic_weights lie in rows (y, z), (y + 1, z), (y, z + 1), (y + 1, z + 1)); a row
// outside the tile is skipped (a neighbouring tile adds it).  Four row predicates instead of a
// test per corner measured 0.490 -> 0.468 ms per deposit (256^3 on 512^3).  ONE: one-word
// sums (lo only).
template <bool ONE>
__device__ __forceinline__ void deposit_particle(unsigned* lo, unsigned* hi, int n, int rs, int cx, int ly, int lz,
                                                 const unsigned (&q)[8]) {
  const int x1 = cx + 1 == n ? 0 : cx + 1;
  const bool y0 = ly >= 0, y1 = ly + 1 < TY, z0 = lz >= 0, z1 = lz + 1 < TZ;
  const int base = (lz * TY + ly) * rs;
  auto add = [&](int i, unsigned v) {
    if (ONE) atomicAdd(&lo[i], v);  // result unused: a non-returning shared-memory reduction
    else acc_add(lo, hi, i, v);
  };
  if (y0 && z0) { add(base + cx, q[0]); add(base + x1, q[1]); }
  if (y1 && z0) { add(base + rs + cx, q[2]); add(base + rs + x1, q[4]); }
  if (y0 && z1) { add(base + TY * rs + cx, q[3]); add(base + TY * rs + x1, q[5]); }
  if (y1 && z1) { add(base + (TY + 1) * rs + cx, q[6]); add(base + (TY + 1) * rs + x1, q[7]); }
}

// CIC weights of a particle quantised to qscale = 2^s.
// qscale is a power of two, so scaling the x factor by it is exact and each product equals
// cic_weights' weight times qscale bit for bit (same association: (a_x a_y) a_z).
__device__ __forceinline__ void quantised_weights(const Cell& c, float qscale, unsigned (&q)[8]) {
  const float tx = (1.f - c.fx) * qscale, fx = c.fx * qscale;
  const float ty = 1.f - c.fy, tz = 1.f - c.fz, fy = c.fy, fz = c.fz;
  q[0] = __float2uint_rn(tx * ty * tz);
  q[1] = __float2uint_rn(fx * ty * tz);
  q[2] = __float2uint_rn(tx * fy * tz);
  q[3] = __float2uint_rn(tx * ty * fz);
  q[4] = __float2uint_rn(fx * fy * tz);
  q[5] = __float2uint_rn(fx * ty * fz);
  q[6] = __float2uint_rn(tx * fy * fz);
  q[7] = __float2uint_rn(fx * fy * fz);
}

// (Pre-adding the weights of lanes that share a cell, with __match_any_sync and a warp
// reduction, would cut the same-address atomics of clustered tiles, but the match alone made
// the deposit 6x slower on GB300.)
template <bool ONE>
__device__ __forceinline__ void deposit_entry(unsigned* lo, unsigned* hi, int n, int rs, float qscale, bool ok,
                                              const Cell& c, int ly, int lz) {
  if (ok) {
    unsigned q[8];
    quantised_weights(c, qscale, q);
    deposit_particle<ONE>(lo, hi, n, rs, c.x, ly, lz, q);
  }
}

// Source ranges of a tile: the particles whose base cell lies in the tile's rows or one row
// / plane below (periodic) are, in the row-sorted order, 7 runs of consecutive rows (rows
// are numbered tile by tile, TZ x TY inside a tile):
//   0: the tile itself (16 rows)            1: the tile below in z, its last plane (TY rows)
//   2-5: the tile below in y, its last row of each plane    6: the diagonal tile, last row
constexpr int NRUN = 7;

// The run table of a tile: source entry f belongs to the last run r with off[r] <= f, and
// sits at place f + delta[r] (= begin[r] + f - off[r]) of the row-sorted order.
//
// RunTable searches the table in shared memory (a chain of dependent loads before the
// permutation load can issue, but no registers); RunRegs holds it in 14 registers and finds
// the run with compares and selects.  The fused deposit takes RunRegs (0.535 -> 0.521 ms early,
// 0.716 -> 0.636 ms at step 980, 256^3 on 512^3); the standalone deposit, at 40 registers a
// thread, keeps RunTable.
struct RunTable {
  const unsigned *begin, *off;
  __device__ __forceinline__ RunTable(const unsigned* s_begin, const unsigned* s_off) : begin(s_begin), off(s_off) {}
  // Slot of source entry f (0xffffffff past the end): its place in the row-sorted order,
  // through the permutation when there is one (else the state is in row order).
  __device__ __forceinline__ unsigned slot(const unsigned* __restrict__ perm, unsigned f, unsigned total) const {
    if (f >= total) return 0xffffffffu;
    int r = 0;  // last run with off[r] <= f
    if (off[4] <= f) r = 4;
    if (off[r + 2] <= f) r += 2;
    if (r + 1 < NRUN && off[r + 1] <= f) r += 1;
    const unsigned pos = begin[r] + (f - off[r]);
    return perm ? __ldg(&perm[pos]) : pos;
  }
};

struct RunRegs {
  unsigned off[NRUN], delta[NRUN];
  __device__ __forceinline__ RunRegs(const unsigned* s_begin, const unsigned* s_off) {
#pragma unroll
    for (int r = 0; r < NRUN; ++r) {
      off[r] = s_off[r];
      delta[r] = s_begin[r] - s_off[r];
    }
  }
  // Slot of source entry f (0xffffffff past the end): its place in the row-sorted order,
  // through the permutation when there is one (else the state is in row order).
  __device__ __forceinline__ unsigned slot(const unsigned* __restrict__ perm, unsigned f, unsigned total) const {
    if (f >= total) return 0xffffffffu;
    unsigned d = delta[0];
#pragma unroll
    for (int r = 1; r < NRUN; ++r) d = f >= off[r] ? delta[r] : d;
    const unsigned pos = f + d;
    return perm ? __ldg(&perm[pos]) : pos;
  }
};

// Base cell of a source particle relative to the tile, from its loaded words; false if
// absent or bad.  NN: the grid size when known at compile time (0: S.n).
template <int MODE, int NN>
__device__ __forceinline__ bool source_cell(const Sim& S, const Parts& p, const RawCell& raw, int y0, int z0,
                                            int* err, Cell& c, int& ly, int& lz) {
  if (!raw.present) return false;
  c = raw_cell<MODE>(S, p, raw);
  const int n = NN ? NN : S.n;
  int dy = c.y - y0, dz = c.z - z0;
  if (dy >= n - 1) dy -= n;
  if (dz >= n - 1) dz -= n;
  const bool ok = c.ok && dy >= -1 && dy < TY && dz >= -1 && dz < TZ;
  if (!ok) set_error(err, c.ok ? ERR_SOURCE_ROW : ERR_CELL_RANGE);
  ly = dy;
  lz = dz;
  return ok;
}

// The 7 runs of the tile at (y0, z0): lane r < NRUN loads the first sorted index and the
// particle count of run r.
struct RunLoad {
  unsigned beg, cnt;
};

__device__ __forceinline__ RunLoad run_load(const Sim& S, const unsigned* __restrict__ row_start, int y0, int z0,
                                            int lane) {
  RunLoad v{0u, 0u};
  if (lane < NRUN) {
    const int n = S.n;
    const int ym = y0 == 0 ? n - TY : y0 - TY, zm = z0 == 0 ? n - TZ : z0 - TZ;  // tiles below
    const int ntile_y = n / TY;
    const unsigned t_own = (unsigned)(z0 / TZ) * ntile_y + y0 / TY;
    const unsigned t_zb = (unsigned)(zm / TZ) * ntile_y + y0 / TY;
    const unsigned t_yb = (unsigned)(z0 / TZ) * ntile_y + ym / TY;
    const unsigned t_c = (unsigned)(zm / TZ) * ntile_y + ym / TY;
    unsigned r0, nr;
    if (lane == 0) { r0 = t_own * (TZ * TY); nr = TZ * TY; }
    else if (lane == 1) { r0 = t_zb * (TZ * TY) + (TZ - 1) * TY; nr = TY; }
    else if (lane < 6) { r0 = t_yb * (TZ * TY) + (lane - 2) * TY + TY - 1; nr = 1; }
    else { r0 = t_c * (TZ * TY) + (TZ - 1) * TY + TY - 1; nr = 1; }
    r0 += S.row_base;
    v.beg = __ldg(&row_start[r0]);
    v.cnt = __ldg(&row_start[r0 + nr]) - v.beg;
  }
  return v;
}

// Warp-wide (all 32 lanes call it): the run table (first sorted index, and the inclusive scan
// of the counts) of the tile whose runs the 8 lanes of this lane's group of eight loaded
// (lane & 7 = the run).  The lanes with `write` store their group's table at s_begin / s_off.
__device__ __forceinline__ void run_table(const RunLoad& v, int lane, unsigned* s_begin, unsigned* s_off,
                                          bool write) {
  const int r = lane & 7;
  unsigned incl = v.cnt;
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    const unsigned t = __shfl_up_sync(FULL, incl, o, 8);
    if (r >= o) incl += t;
  }
  if (!write) return;
  if (r < NRUN) {
    s_begin[r] = v.beg;
    s_off[r + 1] = incl;
  }
  if (r == 0) s_off[0] = 0;
}

// The particle loop of a tile: two source entries per lane and iteration, so that their
// loads overlap; the slots (the permutation entries) of the next iteration are in flight
// while this one adds its particles.
template <int MODE, int NT, bool ONE, int NN>
__device__ __forceinline__ void deposit_sources(const Sim& S, const Parts& p, const unsigned* __restrict__ perm,
                                                int* err, int y0, int z0, unsigned* lo, unsigned* hi, int rs,
                                                const unsigned* s_begin, const unsigned* s_off, unsigned total,
                                                float qscale, int tid) {
  const int lane = tid & 31, warp = tid >> 5;
  const int n = NN ? NN : S.n;
  using Runs = typename std::conditional<NN != 0, RunRegs, RunTable>::type;
  const Runs runs(s_begin, s_off);
  unsigned base = (unsigned)warp * 32u;
  unsigned sl0 = runs.slot(perm, base + lane, total);
  unsigned sl1 = runs.slot(perm, base + NT + lane, total);
  for (; base < total; base += 2 * NT) {
    const RawCell q0 = load_raw_cell<MODE>(p, sl0), q1 = load_raw_cell<MODE>(p, sl1);
    sl0 = runs.slot(perm, base + 2 * NT + lane, total);
    sl1 = runs.slot(perm, base + 3 * NT + lane, total);
    Cell c0, c1;
    int ly0 = 0, lz0 = 0, ly1 = 0, lz1 = 0;
    const bool ok0 = source_cell<MODE, NN>(S, p, q0, y0, z0, err, c0, ly0, lz0);
    const bool ok1 = source_cell<MODE, NN>(S, p, q1, y0, z0, err, c1, ly1, lz1);
    deposit_entry<ONE>(lo, hi, n, rs, qscale, ok0, c0, ly0, lz0);
    deposit_entry<ONE>(lo, hi, n, rs, qscale, ok1, c1, ly1, lz1);
  }
}

// Accumulate the tile at (y0, z0) of simulation S into lo/hi: TZ * TY rows of n cells, row r
// of lo at word r * rs and of hi at the same offset from hi (hi is only written by two-word
// tiles).  s_begin / s_off: NRUN + 1 words each, already holding the tile's run table when
// runs_ready.  Done by NT threads, tid = 0 .. NT - 1 (a whole CTA, or a group of its warps
// with one tile each: every group calls it together, it synchronises the whole CTA).  Returns
// how the sums are held (tile_sum), also written to *ts_out when given.  NN: the grid size
// when known at compile time (0: S.n).  zeroed: lo (and hi) are already zero, so the zeroing
// phase and its barrier are skipped.
template <int MODE, int NT, int NN = 0>
__device__ __forceinline__ TileSum deposit_tile(const Sim& S, const Parts& p, const unsigned* __restrict__ perm,
                                                const unsigned* __restrict__ row_start, int* err, int y0, int z0,
                                                unsigned* lo, unsigned* hi, int rs, unsigned* s_begin,
                                                unsigned* s_off, bool runs_ready = false, int tid = -1,
                                                TileSum* ts_out = nullptr, bool zeroed = false) {
  if (tid < 0) tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int n = NN ? NN : S.n;
  if (!runs_ready) {
    if (warp == 0) run_table(run_load(S, row_start, y0, z0, lane), lane, s_begin, s_off, lane < 8);
    __syncthreads();
  }
  const unsigned total = s_off[NRUN];
  const TileSum ts = tile_sum(total, S.mass_scale);
  if (ts_out && tid == 0) *ts_out = ts;  // visible to the whole CTA after the barrier below
  // zero the rows of lo (and of hi for two-word sums), 4 words per store
  if (!zeroed) {
    const int q4 = n / 4;
    for (int i = tid; i < TZ * TY * q4; i += NT) {
      const int off = (i / q4) * rs + (i % q4) * 4;
      *reinterpret_cast<uint4*>(lo + off) = make_uint4(0u, 0u, 0u, 0u);
      if (!ts.s) *reinterpret_cast<uint4*>(hi + off) = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();
  }
  if (ts.s)
    deposit_sources<MODE, NT, true, NN>(S, p, perm, err, y0, z0, lo, hi, rs, s_begin, s_off, total,
                                    __uint_as_float((unsigned)(127 + ts.s) << 23), tid);
  else
    deposit_sources<MODE, NT, false, NN>(S, p, perm, err, y0, z0, lo, hi, rs, s_begin, s_off, total,
                                     (float)(1u << PM_FIX_BITS), tid);
  __syncthreads();
  return ts;
}

}  // namespace pm
