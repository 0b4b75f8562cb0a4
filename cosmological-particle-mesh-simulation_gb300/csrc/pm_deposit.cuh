// Deterministic CIC deposit of one tile (density.py:7-48 of the reference).
//
// A tile is TZ x TY full x-rows.  The particles whose base cell lies in the tile's source
// rows (the tile plus one row and one plane below, periodic) are found through the row
// starts of the cell-key sort; their CIC weights that land inside the tile are added to
// integer accumulators in shared memory: weights quantised to 2^-26, a 32-bit low word
// with carry into a 32-bit high word.  Integer sums do not depend on the order of the
// atomics, so the deposit is bit-identical run to run.
#pragma once
#include "pm_cells.cuh"

namespace pm {

constexpr int DEP_NT = 512;
constexpr int DEP_ROW_NT = 256;  // fused deposit with the register row transform

__device__ __forceinline__ void acc_add(unsigned* lo, unsigned* hi, int i, unsigned q) {
  const unsigned old = atomicAdd(&lo[i], q);
  if (old + q < old) atomicAdd(&hi[i], 1u);
}

__device__ __forceinline__ float fixed_to_float(unsigned l, unsigned h, float scale) {
  return (h == 0u ? __uint2float_rn(l) : __ull2float_rn(((unsigned long long)h << 32) | l)) * scale;
}

// Adds the 8 weights of a particle with base cell (cx, ly, lz) (ly, lz relative to the
// tile, in [-1, TY-1] x [-1, TZ-1]) to the tile accumulators; tile row r of lo / hi starts
// at word r * rs.
__device__ __forceinline__ void deposit_particle(unsigned* lo, unsigned* hi, int n, int rs, int cx, int ly, int lz,
                                                 const float (&wt)[8]) {
  const int x1 = cx + 1 == n ? 0 : cx + 1;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int ty2 = ly + corner_y(k), tz2 = lz + corner_z(k);
    if (ty2 >= 0 && ty2 < TY && tz2 >= 0 && tz2 < TZ)
      acc_add(lo, hi, (tz2 * TY + ty2) * rs + (corner_x(k) ? x1 : cx),
              __float2uint_rn(wt[k] * (float)(1u << PM_FIX_BITS)));
  }
}

// Base cell of source entry f relative to the tile; false if the entry is absent or bad.
template <int MODE>
__device__ __forceinline__ bool source_cell(const Sim& S, const Parts& p, const unsigned* __restrict__ perm,
                                            const unsigned* s_begin, const unsigned* s_off, unsigned f,
                                            unsigned total, int y0, int z0, int* err, Cell& c, int& ly,
                                            int& lz) {
  if (f >= total) return false;
  int r = 0;  // last source row with s_off[r] <= f
#pragma unroll
  for (int step = 16; step > 0; step >>= 1)
    if (r + step < NSRC && s_off[r + step] <= f) r += step;
  const unsigned pos = s_begin[r] + (f - s_off[r]);
  const unsigned slot = perm ? __ldg(&perm[pos]) : pos;  // no permutation: the state is in row order
  c = particle_cell<MODE>(S, p, slot);
  const int n = S.n;
  int dy = c.y - y0, dz = c.z - z0;
  if (dy >= n - 1) dy -= n;
  if (dz >= n - 1) dz -= n;
  const bool ok = c.ok && dy >= -1 && dy < TY && dz >= -1 && dz < TZ;
  if (!ok) set_error(err, c.ok ? ERR_SOURCE_ROW : ERR_CELL_RANGE);
  ly = dy;
  lz = dz;
  return ok;
}

// Accumulate the tile at (y0, z0) of simulation S into lo/hi (TZ * TY rows of n cells,
// row r at word r * rs of each; lo and hi together are 2 * TZ * TY * n contiguous words).
// Entered and left by all NT threads, synchronised.
template <int MODE, int NT>
__device__ __forceinline__ void deposit_tile(const Sim& S, const Parts& p, const unsigned* __restrict__ perm,
                                             const unsigned* __restrict__ row_start, int* err, int y0, int z0,
                                             unsigned* lo, unsigned* hi, int rs, unsigned* s_begin, unsigned* s_off) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = S.n;
  const int ncell = TZ * TY * n;  // zero 2 * ncell words
  uint4* z4 = reinterpret_cast<uint4*>(lo);
  for (int i = threadIdx.x; i < ncell / 2; i += NT) z4[i] = make_uint4(0u, 0u, 0u, 0u);
  if (warp == 0) {
    // source rows (lz, ly) in [-1, TZ-1] x [-1, TY-1]: begin and an inclusive scan of counts
    unsigned beg = 0, cnt = 0;
    if (lane < NSRC) {
      const int lz = lane / (TY + 1) - 1, ly = lane % (TY + 1) - 1;
      const int z = z0 + lz < 0 ? z0 + lz + n : z0 + lz;
      const int y = y0 + ly < 0 ? y0 + ly + n : y0 + ly;
      const unsigned r = S.row_base + row_number(y, z, n);
      beg = __ldg(&row_start[r]);
      cnt = __ldg(&row_start[r + 1]) - beg;
    }
    unsigned incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane < NSRC) {
      s_begin[lane] = beg;
      s_off[lane + 1] = incl;
    }
    if (lane == 0) s_off[0] = 0;
  }
  __syncthreads();
  const unsigned total = s_off[NSRC];
  // two source entries per lane and iteration, so that their loads overlap
  for (unsigned base = (unsigned)warp * 32u; base < total; base += 2 * NT) {
    Cell c0, c1;
    int ly0 = 0, lz0 = 0, ly1 = 0, lz1 = 0;
    const bool ok0 = source_cell<MODE>(S, p, perm, s_begin, s_off, base + lane, total, y0, z0, err, c0, ly0, lz0);
    const bool ok1 =
        source_cell<MODE>(S, p, perm, s_begin, s_off, base + NT + lane, total, y0, z0, err, c1, ly1, lz1);
    if (ok0) {
      float wt[8];
      cic_weights(c0, wt);
      deposit_particle(lo, hi, n, rs, c0.x, ly0, lz0, wt);
    }
    if (ok1) {
      float wt[8];
      cic_weights(c1, wt);
      deposit_particle(lo, hi, n, rs, c1.x, ly1, lz1, wt);
    }
  }
  __syncthreads();
}

}  // namespace pm
