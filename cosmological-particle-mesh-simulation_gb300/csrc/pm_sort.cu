// Stable LSD radix sort of (key, value) pairs, digits of up to 9 bits, reduce-then-scan.
//
// Per digit pass:
//   upsweep    per-tile digit histogram            hist[d * nblocks + tile]
//   scan       per digit, exclusive scan over tiles (one CTA per digit), digit totals
//   downsweep  per tile: stable rank of every item inside its digit (warp match-based
//              multisplit, warps in tile order, batches in order), staging in shared
//              memory by digit, coalesced write to digit_base[d] + tile_offset + rank
//
// A sort over `bits` key bits takes ceil(bits / 9) passes of equal width.  Only integer
// arithmetic: the output is bit-exact and independent of scheduling.
#include "pm_common.cuh"

namespace pm {

constexpr int SORT_NT = 256;
constexpr int SORT_IPT = SORT_TILE / SORT_NT;  // 16 items per thread
constexpr int SORT_WARPS = SORT_NT / 32;
constexpr int SORT_SCAN_NT = 1024;
constexpr int MAX_DIGIT_BITS = 9;
constexpr int MAX_RADIX = 1 << MAX_DIGIT_BITS;
constexpr int DPT = MAX_RADIX / SORT_NT;  // digits per thread in per-digit loops

__global__ void __launch_bounds__(SORT_NT) k_sort_upsweep(const unsigned* __restrict__ keys, long long n,
                                                          int shift, int dbits, unsigned* __restrict__ hist,
                                                          int nblocks) {
  __shared__ unsigned h[SORT_WARPS][MAX_RADIX];
  const int warp = threadIdx.x >> 5;
  const unsigned mask = (1u << dbits) - 1u, radix = 1u << dbits;
  for (int i = threadIdx.x; i < SORT_WARPS * MAX_RADIX; i += SORT_NT) (&h[0][0])[i] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * SORT_TILE;
  unsigned k[SORT_IPT];
#pragma unroll
  for (int i = 0; i < SORT_IPT; ++i) {
    const long long idx = base + i * SORT_NT + threadIdx.x;
    k[i] = idx < n ? __ldg(&keys[idx]) : 0u;
  }
#pragma unroll
  for (int i = 0; i < SORT_IPT; ++i) {
    const long long idx = base + i * SORT_NT + threadIdx.x;
    if (idx < n) atomicAdd(&h[warp][(k[i] >> shift) & mask], 1u);
  }
  __syncthreads();
  for (unsigned d = threadIdx.x; d < radix; d += SORT_NT) {
    unsigned s = 0;
#pragma unroll
    for (int w = 0; w < SORT_WARPS; ++w) s += h[w][d];
    hist[(long long)d * nblocks + blockIdx.x] = s;
  }
}

// Block-wide exclusive scan of one value per thread; returns the block total in `total`.
template <int NT>
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* ws, unsigned& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned t = lane < NT / 32 ? ws[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < NT / 32) ws[lane] = t;
  }
  __syncthreads();
  total = ws[NT / 32 - 1];
  const unsigned res = x - v + (warp > 0 ? ws[warp - 1] : 0u);
  __syncthreads();
  return res;
}

__global__ void __launch_bounds__(SORT_SCAN_NT) k_sort_scan(unsigned* __restrict__ hist, int nblocks,
                                                            unsigned* __restrict__ digit_tot) {
  __shared__ unsigned ws[32];
  unsigned* row = hist + (long long)blockIdx.x * nblocks;
  unsigned carry = 0;
  for (int base = 0; base < nblocks; base += SORT_SCAN_NT) {
    const int i = base + threadIdx.x;
    const unsigned v = i < nblocks ? row[i] : 0u;
    unsigned tot;
    const unsigned ex = block_exclusive_scan<SORT_SCAN_NT>(v, ws, tot);
    if (i < nblocks) row[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) digit_tot[blockIdx.x] = carry;
}

struct DownSmem {
  unsigned skey[SORT_TILE];
  unsigned sval[SORT_TILE];
  unsigned wcnt[SORT_WARPS][MAX_RADIX];
  unsigned dstart[MAX_RADIX];
  unsigned gofs[MAX_RADIX];
  unsigned ws[32];
};

__global__ void __launch_bounds__(SORT_NT) k_sort_downsweep(const unsigned* __restrict__ keys_in,
                                                            const unsigned* __restrict__ vals_in,
                                                            unsigned* __restrict__ keys_out,
                                                            unsigned* __restrict__ vals_out, long long n,
                                                            int shift, int dbits,
                                                            const unsigned* __restrict__ hist,
                                                            const unsigned* __restrict__ digit_tot,
                                                            int nblocks, int gen_vals) {
  extern __shared__ uint4 down_raw[];
  DownSmem& sm = *reinterpret_cast<DownSmem*>(down_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned mask = (1u << dbits) - 1u, radix = 1u << dbits;
  const long long base = (long long)blockIdx.x * SORT_TILE;
  for (int i = threadIdx.x; i < SORT_WARPS * MAX_RADIX; i += SORT_NT) (&sm.wcnt[0][0])[i] = 0;
  // global start of each digit for this tile: exclusive scan of the digit totals
  {
    unsigned t[DPT], s = 0;
#pragma unroll
    for (int j = 0; j < DPT; ++j) {
      const unsigned d = threadIdx.x * DPT + j;
      t[j] = d < radix ? digit_tot[d] : 0u;
      s += t[j];
    }
    unsigned tot;
    unsigned ex = block_exclusive_scan<SORT_NT>(s, sm.ws, tot);
#pragma unroll
    for (int j = 0; j < DPT; ++j) {
      const unsigned d = threadIdx.x * DPT + j;
      if (d < radix) sm.gofs[d] = ex + hist[(long long)d * nblocks + blockIdx.x];
      ex += t[j];
    }
  }
  __syncthreads();
  unsigned key[SORT_IPT], val[SORT_IPT], rank[SORT_IPT];
  const unsigned lt_mask = (1u << lane) - 1u;
  const long long wbase = base + (long long)warp * 32 * SORT_IPT;
#pragma unroll
  for (int i = 0; i < SORT_IPT; ++i) {
    const long long idx = wbase + i * 32 + lane;
    const bool valid = idx < n;
    key[i] = valid ? keys_in[idx] : 0u;
    val[i] = valid ? (gen_vals ? (unsigned)idx : vals_in[idx]) : 0u;
  }
#pragma unroll
  for (int i = 0; i < SORT_IPT; ++i) {
    const long long idx = wbase + i * 32 + lane;
    const bool valid = idx < n;
    const unsigned d = valid ? ((key[i] >> shift) & mask) : (unsigned)MAX_RADIX + lane;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned prior = valid ? sm.wcnt[warp][d] : 0u;
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) sm.wcnt[warp][d] = prior + __popc(peers);
    __syncwarp();
    rank[i] = prior + __popc(peers & lt_mask);
  }
  __syncthreads();
  // per digit: warp prefix counts and the tile-local digit start
  {
    unsigned run[DPT], s = 0;
#pragma unroll
    for (int j = 0; j < DPT; ++j) {
      const unsigned d = threadIdx.x * DPT + j;
      unsigned r = 0;
      if (d < radix) {
#pragma unroll
        for (int w = 0; w < SORT_WARPS; ++w) {
          const unsigned c = sm.wcnt[w][d];
          sm.wcnt[w][d] = r;
          r += c;
        }
      }
      run[j] = r;
      s += r;
    }
    unsigned tot;
    unsigned ex = block_exclusive_scan<SORT_NT>(s, sm.ws, tot);
#pragma unroll
    for (int j = 0; j < DPT; ++j) {
      const unsigned d = threadIdx.x * DPT + j;
      if (d < radix) sm.dstart[d] = ex;
      ex += run[j];
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < SORT_IPT; ++i) {
    const long long idx = wbase + i * 32 + lane;
    if (idx < n) {
      const unsigned d = (key[i] >> shift) & mask;
      const unsigned p = sm.dstart[d] + sm.wcnt[warp][d] + rank[i];
      sm.skey[p] = key[i];
      sm.sval[p] = val[i];
    }
  }
  __syncthreads();
  const long long rem = n - base;
  const int cnt = rem < SORT_TILE ? (int)rem : SORT_TILE;
  for (int p = threadIdx.x; p < cnt; p += SORT_NT) {
    const unsigned k = sm.skey[p];
    const unsigned d = (k >> shift) & mask;
    const unsigned g = sm.gofs[d] + (unsigned)p - sm.dstart[d];
    keys_out[g] = k;
    vals_out[g] = sm.sval[p];
  }
}

size_t sort_scratch_hist_entries(long long n) {
  const long long nb = (n + SORT_TILE - 1) / SORT_TILE;
  return (size_t)MAX_RADIX * (nb > 0 ? nb : 1);
}

cudaError_t sort_prepare() {
  static DeviceOnce once;
  return once.run([]() {
    return cudaFuncSetAttribute(k_sort_downsweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(DownSmem));
  });
}

int radix_sort_passes(int bits) { return bits <= 0 ? 1 : (bits + MAX_DIGIT_BITS - 1) / MAX_DIGIT_BITS; }

cudaError_t radix_sort(unsigned* keys, unsigned* vals, long long n, int begin_bit, int bits, bool gen_vals,
                       const SortScratch& s, bool* in_alt, cudaStream_t st) {
  *in_alt = false;
  if (n <= 0) return cudaSuccess;
  if (n > s.capacity || n >= (1ll << 32)) return cudaErrorInvalidValue;
  const int nblocks = (int)((n + SORT_TILE - 1) / SORT_TILE);
  if (nblocks > s.max_blocks) return cudaErrorInvalidValue;
  if (cudaError_t e = sort_prepare()) return e;
  const int passes = radix_sort_passes(bits);
  const int dbits = bits <= 0 ? 1 : (bits + passes - 1) / passes;
  unsigned *ki = keys, *vi = vals, *ko = s.keys_alt, *vo = s.vals_alt;
  for (int p = 0; p < passes; ++p) {
    const int shift = begin_bit + dbits * p;
    k_sort_upsweep<<<nblocks, SORT_NT, 0, st>>>(ki, n, shift, dbits, s.hist, nblocks);
    k_sort_scan<<<1 << dbits, SORT_SCAN_NT, 0, st>>>(s.hist, nblocks, s.digit_tot);
    k_sort_downsweep<<<nblocks, SORT_NT, sizeof(DownSmem), st>>>(ki, vi, ko, vo, n, shift, dbits, s.hist,
                                                                 s.digit_tot, nblocks,
                                                                 (p == 0 && gen_vals) ? 1 : 0);
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    unsigned* t = ki; ki = ko; ko = t;
    t = vi; vi = vo; vo = t;
  }
  *in_alt = (passes % 2) == 1;
  return cudaSuccess;
}



// ---------------------------------------------------------------------------------
// Counting sort of row keys (resident batches).  The deposit and the kick need the
// particles grouped by x-row, not ordered inside a row: a histogram of the rows, its
// exclusive scan (the row starts) and one scatter through per-row cursors replace the
// radix passes.  The order inside a row depends on the scheduling of the cursor atomics;
// nothing downstream depends on it (the deposit sums integers, the kick is per particle).
// Equal keys of a warp are combined by a match first (the state is nearly sorted, so a
// warp touches few rows).  A key 0xffffffff marks an empty slot (a simulation that left a
// batch): it is neither counted nor placed.
// ---------------------------------------------------------------------------------
namespace {

constexpr int CS_NT = 256;
constexpr int SCAN_TILE = 4096;  // rows per block of the row-start scan
constexpr int SCAN_IPT = SCAN_TILE / CS_NT;

// UNR batches of 32 keys per warp and iteration: their loads, matches and atomics overlap.
constexpr int CS_UNR = 4;

__global__ void __launch_bounds__(CS_NT) k_row_hist(const unsigned* __restrict__ keys, long long n, unsigned nrows,
                                                    unsigned* __restrict__ count, int* err) {
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * CS_NT * CS_UNR;
  for (long long b = ((long long)blockIdx.x * CS_NT + (threadIdx.x & ~31)) * CS_UNR; b < n; b += stride) {
    unsigned k[CS_UNR];
#pragma unroll
    for (int u = 0; u < CS_UNR; ++u) {
      const long long i = b + u * 32 + lane;
      k[u] = i < n ? __ldg(&keys[i]) : 0xffffffffu;
      if (k[u] != 0xffffffffu && k[u] >= nrows) {
        set_error(err, ERR_CELL_RANGE);
        k[u] = nrows - 1;
      }
    }
#pragma unroll
    for (int u = 0; u < CS_UNR; ++u) {
      const unsigned grp = __match_any_sync(0xffffffffu, k[u]);
      if (k[u] != 0xffffffffu && lane == __ffs(grp) - 1) atomicAdd(&count[k[u]], (unsigned)__popc(grp));
    }
  }
}

// per-block sums of SCAN_TILE entries
__global__ void __launch_bounds__(CS_NT) k_scan_reduce(const unsigned* __restrict__ in, long long n,
                                                       unsigned* __restrict__ block_sums) {
  __shared__ unsigned ws[CS_NT / 32];
  const long long base = (long long)blockIdx.x * SCAN_TILE;
  unsigned s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) {
    const long long i = base + j * CS_NT + threadIdx.x;
    if (i < n) s += __ldg(&in[i]);
  }
  unsigned total;
  block_exclusive_scan<CS_NT>(s, ws, total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// exclusive scan of the block sums in place (one block, chunks of CS_NT with a carry)
__global__ void __launch_bounds__(CS_NT) k_scan_top(unsigned* __restrict__ block_sums, int nblocks) {
  __shared__ unsigned ws[CS_NT / 32];
  unsigned carry = 0;
  for (int c = 0; c < nblocks; c += CS_NT) {
    const int i = c + threadIdx.x;
    const unsigned v = i < nblocks ? block_sums[i] : 0u;
    unsigned total;
    const unsigned ex = block_exclusive_scan<CS_NT>(v, ws, total);
    if (i < nblocks) block_sums[i] = carry + ex;
    carry += total;
    __syncthreads();
  }
}

// out[i] = exclusive prefix of in, i < n; out[n] = total; cursor = copy of out[0, n)
__global__ void __launch_bounds__(CS_NT) k_scan_apply(const unsigned* __restrict__ in, long long n,
                                                      const unsigned* __restrict__ block_sums,
                                                      unsigned* __restrict__ out, unsigned* __restrict__ cursor) {
  __shared__ unsigned ws[CS_NT / 32];
  const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_IPT;
  unsigned v[SCAN_IPT];
  unsigned s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) {
    const long long i = base + j;
    v[j] = i < n ? __ldg(&in[i]) : 0u;
    s += v[j];
  }
  unsigned total;
  unsigned run = block_sums[blockIdx.x] + block_exclusive_scan<CS_NT>(s, ws, total);
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) {
    const long long i = base + j;
    if (i < n) {
      out[i] = run;
      cursor[i] = run;
    }
    run += v[j];
    if (i == n - 1) out[n] = run;
  }
}

// Each warp scatters one chunk of SCATTER_CHUNK consecutive keys, in order: the keys of a
// row that lie in one chunk keep their order and stay together, so a row's range is made
// of a few ordered runs (one per chunk it spans) and a nearly sorted input stays nearly
// in place -- the next reads through the permutation remain coalesced.
constexpr int SCATTER_CHUNK = 1024;

__global__ void __launch_bounds__(CS_NT) k_row_scatter(const unsigned* __restrict__ keys, long long n, unsigned nrows,
                                                       unsigned* __restrict__ cursor, unsigned* __restrict__ perm,
                                                       unsigned* __restrict__ inv) {
  const int lane = threadIdx.x & 31;
  const long long nchunks = (n + SCATTER_CHUNK - 1) / SCATTER_CHUNK;
  const long long nwarps = (long long)gridDim.x * (CS_NT / 32);
  for (long long c = (long long)blockIdx.x * (CS_NT / 32) + (threadIdx.x >> 5); c < nchunks; c += nwarps) {
    const long long end = (c + 1) * SCATTER_CHUNK < n ? (c + 1) * SCATTER_CHUNK : n;
    for (long long b = c * SCATTER_CHUNK; b < end; b += 32 * CS_UNR) {
      // CS_UNR batches in order: a row's cursor is advanced batch by batch (program order of
      // the same address), and the batches' atomics are in flight together
      unsigned k[CS_UNR], grp[CS_UNR], pos[CS_UNR];
#pragma unroll
      for (int u = 0; u < CS_UNR; ++u) {
        const long long i = b + u * 32 + lane;
        k[u] = i < end ? __ldg(&keys[i]) : 0xffffffffu;
        if (k[u] != 0xffffffffu && k[u] >= nrows) k[u] = nrows - 1;
      }
#pragma unroll
      for (int u = 0; u < CS_UNR; ++u) {
        grp[u] = __match_any_sync(0xffffffffu, k[u]);
        pos[u] = 0;
        if (k[u] != 0xffffffffu && lane == __ffs(grp[u]) - 1) pos[u] = atomicAdd(&cursor[k[u]], (unsigned)__popc(grp[u]));
      }
#pragma unroll
      for (int u = 0; u < CS_UNR; ++u) {
        const unsigned p0 = __shfl_sync(0xffffffffu, pos[u], __ffs(grp[u]) - 1);
        if (k[u] != 0xffffffffu) {
          const long long i = b + u * 32 + lane;
          const unsigned p = p0 + __popc(grp[u] & ((1u << lane) - 1u));
          perm[p] = (unsigned)i;
          if (inv) inv[i] = p;
        }
      }
    }
  }
}

}  // namespace

size_t row_sort_block_sums(unsigned nrows) { return ((size_t)nrows + SCAN_TILE - 1) / SCAN_TILE; }

cudaError_t row_histogram(const unsigned* keys, long long n, unsigned nrows, unsigned* count, int* err, int sms,
                          cudaStream_t st) {
  if (nrows == 0) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(count, 0, (size_t)nrows * sizeof(unsigned), st);
  if (e) return e;
  long long want = (n + CS_NT * CS_UNR - 1) / (CS_NT * CS_UNR);
  const int ctas = (int)(want < (long long)sms * 8 ? (want > 0 ? want : 1) : (long long)sms * 8);
  k_row_hist<<<ctas, CS_NT, 0, st>>>(keys, n, nrows, count, err);
  return cudaGetLastError();
}

cudaError_t row_counting_sort(const unsigned* keys, long long n, unsigned nrows, unsigned* count,
                              unsigned* row_start, unsigned* cursor, unsigned* block_sums, unsigned* perm, int* err,
                              int sms, cudaStream_t st, unsigned* inv, bool counted) {
  if (nrows == 0) return cudaErrorInvalidValue;
  if (!counted) {
    cudaError_t e = row_histogram(keys, n, nrows, count, err, sms, st);
    if (e) return e;
  }
  const int nb = (int)row_sort_block_sums(nrows);
  k_scan_reduce<<<nb, CS_NT, 0, st>>>(count, nrows, block_sums);
  k_scan_top<<<1, CS_NT, 0, st>>>(block_sums, nb);
  k_scan_apply<<<nb, CS_NT, 0, st>>>(count, nrows, block_sums, row_start, cursor);
  const long long chunks = (n + SCATTER_CHUNK - 1) / SCATTER_CHUNK;
  const long long sblocks = (chunks + CS_NT / 32 - 1) / (CS_NT / 32);
  k_row_scatter<<<(int)(sblocks < (long long)sms * 8 ? (sblocks > 0 ? sblocks : 1) : (long long)sms * 8), CS_NT, 0,
                  st>>>(keys, n, nrows, cursor, perm, inv);
  return cudaGetLastError();
}

}  // namespace pm
