// Stable LSD radix sort of (key, value) pairs, 8-bit digits, reduce-then-scan.
//
// Per digit pass:
//   upsweep    per-tile digit histogram            hist[d * nblocks + tile]
//   scan       per digit, exclusive scan over tiles (one CTA per digit), digit totals
//   downsweep  per tile: stable rank of every item inside its digit (warp match-based
//              multisplit, warps in tile order, batches in order), staging in shared
//              memory by digit, coalesced write to digit_base[d] + tile_offset + rank
//
// Only integer arithmetic: the output is bit-exact and independent of scheduling.
#include "pm_common.cuh"

namespace pm {

constexpr int SORT_NT = 256;
constexpr int SORT_IPT = SORT_TILE / SORT_NT;  // 16 items per thread
constexpr int SORT_WARPS = SORT_NT / 32;
constexpr int SORT_SCAN_NT = 1024;

__global__ void __launch_bounds__(SORT_NT) k_sort_upsweep(const unsigned* __restrict__ keys, long long n,
                                                          int shift, unsigned* __restrict__ hist, int nblocks) {
  __shared__ unsigned h[SORT_WARPS][256];
  const int warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < SORT_WARPS * 256; i += SORT_NT) (&h[0][0])[i] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * SORT_TILE;
#pragma unroll 4
  for (int i = 0; i < SORT_IPT; ++i) {
    const long long idx = base + i * SORT_NT + threadIdx.x;
    if (idx < n) atomicAdd(&h[warp][(__ldg(&keys[idx]) >> shift) & 255u], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += SORT_NT) {
    unsigned s = 0;
#pragma unroll
    for (int w = 0; w < SORT_WARPS; ++w) s += h[w][d];
    hist[(long long)d * nblocks + blockIdx.x] = s;
  }
}

// Block-wide exclusive scan of one value per thread; returns the block total.
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

__global__ void __launch_bounds__(SORT_NT) k_sort_downsweep(const unsigned* __restrict__ keys_in,
                                                            const unsigned* __restrict__ vals_in,
                                                            unsigned* __restrict__ keys_out,
                                                            unsigned* __restrict__ vals_out, long long n,
                                                            int shift, const unsigned* __restrict__ hist,
                                                            const unsigned* __restrict__ digit_tot,
                                                            int nblocks, int gen_vals) {
  __shared__ unsigned skey[SORT_TILE];
  __shared__ unsigned sval[SORT_TILE];
  __shared__ unsigned wcnt[SORT_WARPS][256];
  __shared__ unsigned dstart[256];
  __shared__ unsigned gofs[256];
  __shared__ unsigned ws[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long base = (long long)blockIdx.x * SORT_TILE;
  for (int i = threadIdx.x; i < SORT_WARPS * 256; i += SORT_NT) (&wcnt[0][0])[i] = 0;
  // global start of each digit for this tile
  {
    const unsigned t = threadIdx.x < 256 ? digit_tot[threadIdx.x] : 0u;
    unsigned tot;
    const unsigned ex = block_exclusive_scan<SORT_NT>(t, ws, tot);
    if (threadIdx.x < 256) gofs[threadIdx.x] = ex + hist[(long long)threadIdx.x * nblocks + blockIdx.x];
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
    const unsigned d = valid ? ((key[i] >> shift) & 255u) : 256u + lane;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const unsigned prior = valid ? wcnt[warp][d] : 0u;
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = prior + __popc(peers);
    __syncwarp();
    rank[i] = prior + __popc(peers & lt_mask);
  }
  __syncthreads();
  // per digit: warp prefix counts and the tile-local digit start
  {
    unsigned run = 0;
    if (threadIdx.x < 256) {
#pragma unroll
      for (int w = 0; w < SORT_WARPS; ++w) {
        const unsigned c = wcnt[w][threadIdx.x];
        wcnt[w][threadIdx.x] = run;
        run += c;
      }
    }
    unsigned tot;
    const unsigned ex = block_exclusive_scan<SORT_NT>(threadIdx.x < 256 ? run : 0u, ws, tot);
    if (threadIdx.x < 256) dstart[threadIdx.x] = ex;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < SORT_IPT; ++i) {
    const long long idx = wbase + i * 32 + lane;
    if (idx < n) {
      const unsigned d = (key[i] >> shift) & 255u;
      const unsigned p = dstart[d] + wcnt[warp][d] + rank[i];
      skey[p] = key[i];
      sval[p] = val[i];
    }
  }
  __syncthreads();
  const long long rem = n - base;
  const int cnt = rem < SORT_TILE ? (int)rem : SORT_TILE;
  for (int p = threadIdx.x; p < cnt; p += SORT_NT) {
    const unsigned k = skey[p];
    const unsigned d = (k >> shift) & 255u;
    const unsigned g = gofs[d] + (unsigned)p - dstart[d];
    keys_out[g] = k;
    vals_out[g] = sval[p];
  }
}

size_t sort_scratch_hist_entries(long long n) {
  const long long nb = (n + SORT_TILE - 1) / SORT_TILE;
  return (size_t)256 * (nb > 0 ? nb : 1);
}

cudaError_t radix_sort(unsigned* keys, unsigned* vals, long long n, int bits, bool gen_vals,
                       const SortScratch& s, bool* in_alt, cudaStream_t st) {
  *in_alt = false;
  if (n <= 0) return cudaSuccess;
  if (n > s.capacity || n >= (1ll << 32)) return cudaErrorInvalidValue;
  const int nblocks = (int)((n + SORT_TILE - 1) / SORT_TILE);
  if (nblocks > s.max_blocks) return cudaErrorInvalidValue;
  const int passes = bits <= 0 ? 1 : (bits + 7) / 8;
  unsigned *ki = keys, *vi = vals, *ko = s.keys_alt, *vo = s.vals_alt;
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    k_sort_upsweep<<<nblocks, SORT_NT, 0, st>>>(ki, n, shift, s.hist, nblocks);
    k_sort_scan<<<256, SORT_SCAN_NT, 0, st>>>(s.hist, nblocks, s.digit_tot);
    k_sort_downsweep<<<nblocks, SORT_NT, 0, st>>>(ki, vi, ko, vo, n, shift, s.hist, s.digit_tot, nblocks,
                                                  (p == 0 && gen_vals) ? 1 : 0);
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    unsigned* t = ki; ki = ko; ko = t;
    t = vi; vi = vo; vo = t;
  }
  *in_alt = (passes % 2) == 1;
  return cudaSuccess;
}

}  // namespace pm
