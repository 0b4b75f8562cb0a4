// Particle-side kernels of one PM step:
//
//   keys     cell key of every particle            (density.py:19-21 / integrate.py:20)
//   rows     start of every x-row in the sorted particle order
//   deposit  deterministic CIC deposit             (density.py:7-48)
//   kick     CIC gather of the central-difference force, kick and drift
//                                                  (integrate.py:15-97)
//   coef     per-step coefficients from the scale factor, in fp64 (integrate.py:11-13,
//            potential.py:15, cosmology.py:20-27)
//
// Cells, weights and keys are defined in pm_cells.cuh, the deposit's accumulation in
// pm_deposit.cuh (shared with the fused deposit + x-transform kernel).
#include "pm_cells.cuh"
#include "pm_deposit.cuh"
#include "pm_tma.cuh"

namespace pm {

constexpr int KICK_NT = 256;
constexpr int KICK_PPT = KICK_UNIT / KICK_NT;  // particles per thread of the kick
constexpr int KEY_NT = 256;

// ---------------------------------------------------------------------------------
// keys
// ---------------------------------------------------------------------------------
// copy (POS_ABS, optional): the positions are also written there (the keys kernel reads
// them once, e.g. from host memory, and leaves a device copy)
template <int MODE>
__global__ void __launch_bounds__(KEY_NT) k_keys(const Sim* __restrict__ sims, Work w, Parts p,
                                                 unsigned* __restrict__ keys,
                                                 unsigned* __restrict__ vals, int* err, Parts copy) {
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    const Sim& S = sims[si];
    const long long i = (long long)(unit - __ldg(&w.prefix[si])) * KEY_NT + threadIdx.x;
    if (i >= S.np) continue;
    const long long slot = S.slot_off + i;
    // from the state itself (the cell records, if any, are written here)
    Cell c;
    if (MODE == POS_ABS) {
      const float x = p.x[slot], y = p.y[slot], z = p.z[slot];
      if (copy.x) {
        copy.x[slot] = x;
        copy.y[slot] = y;
        copy.z[slot] = z;
      }
      c = cell_abs(x, y, z, S.n);
    } else {
      c = cell_disp(S, p.id[slot], p.x[slot], p.y[slot], p.z[slot]);
      if (p.rec) store_cell_record(p, slot, c);
    }
    if (!c.ok) { set_error(err, ERR_CELL_RANGE); c.x = c.y = c.z = 0; }
    keys[slot] = cell_key(S, c);
    if (vals) vals[slot] = (unsigned)slot;
  }
}

// ---------------------------------------------------------------------------------
// rows: row_start[r] = first sorted index whose row >= r, for r in [0, nrows]
// (keys with row >= nrows, e.g. the sentinel of an empty slot, count as row nrows)
// ---------------------------------------------------------------------------------
__global__ void k_row_start(const unsigned* __restrict__ keys, long long n, int xbits, unsigned nrows,
                            unsigned* __restrict__ row_start) {
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s <= n;
       s += (long long)gridDim.x * blockDim.x) {
    long long rp = -1, rc = nrows;
    if (s > 0) { rp = keys[s - 1] >> xbits; if (rp > nrows) rp = nrows; }
    if (s < n) { rc = keys[s] >> xbits; if (rc > nrows) rc = nrows; }
    for (long long r = rp + 1; r <= rc; ++r) row_start[r] = (unsigned)s;
  }
}

// ---------------------------------------------------------------------------------
// deposit: one CTA per tile (pm_deposit.cuh), then the tile's rows are written once
// ---------------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(DEP_NT, 3) k_deposit(const Sim* __restrict__ sims, Work w, Parts p,
                                                       const unsigned* __restrict__ perm,
                                                       const unsigned* __restrict__ row_start, int* err) {
  extern __shared__ uint4 acc_raw[];
  __shared__ unsigned s_begin[NSRC];
  __shared__ unsigned s_off[NSRC + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    const Sim& S = sims[si];
    const int local = unit - __ldg(&w.prefix[si]);
    const int n = S.n;
    const int ntile_y = n / TY;
    const int y0 = (local % ntile_y) * TY, z0 = (local / ntile_y) * TZ;
    unsigned* lo = reinterpret_cast<unsigned*>(acc_raw);
    unsigned* hi = lo + TZ * TY * n;
    const TileSum ts = deposit_tile<MODE, DEP_NT>(S, p, perm, row_start, err, y0, z0, lo, hi, S.n, s_begin, s_off);
    for (int row = warp; row < TZ * TY; row += DEP_NT / 32) {
      const uint4* l4 = reinterpret_cast<const uint4*>(lo + row * n);
      const uint4* h4 = reinterpret_cast<const uint4*>(hi + row * n);
      float4* dst = reinterpret_cast<float4*>(S.rho + ((long long)(z0 + row / TY) * n + (y0 + row % TY)) * n);
      for (int x4 = lane; x4 < n / 4; x4 += 32) {
        const uint4 l = l4[x4], h = ts.s ? make_uint4(0u, 0u, 0u, 0u) : h4[x4];
        dst[x4] = make_float4(sum_to_float(ts, l.x, h.x), sum_to_float(ts, l.y, h.y), sum_to_float(ts, l.z, h.z),
                              sum_to_float(ts, l.w, h.w));
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------
// kick / drift
//
// For each particle: CIC weights of its base cell, the central difference
// phi[c - e_a] - phi[c + e_a] at the 8 corners for each axis a, interpolated with the
// weights and halved (integrate.py:84-92), then v_a += kick * g_a and
// x_a += drift * v_a (integrate.py:94-95).  All three axes use the cell and weights
// of the position before the step, as the reference's three sweeps do.
//
// POS_ABS: absolute positions, updated in place at their slot (drop-in layout),
//          wrapped into [0, n).
// POS_DISP: displacements; the particle that is i-th in sorted order is written to
//          output slot sort_off + i, together with its cell key for the next step.
// ---------------------------------------------------------------------------------
// Potential rows around a particle, read from global memory: row(oy, oz) is the x-row at
// (y + oy, z + oz) (periodic), oy, oz in {-1, 0, 1, 2}.  The taps are scalar loads: at one
// particle per several cells each lane of a warp reads its own sector, and 16-byte chunk
// loads of the x-1 .. x+2 windows measured 1.5x slower on GB300.
struct GlobalRows {
  const float* phi;
  int n, ys[4], zs[4];  // y - 1, y, y + 1, y + 2 and the same for z, wrapped
  __device__ __forceinline__ GlobalRows(const float* p, int nn, int y, int z) : phi(p), n(nn) {
    ys[1] = y; ys[0] = y == 0 ? n - 1 : y - 1; ys[2] = y + 1 == n ? 0 : y + 1; ys[3] = ys[2] + 1 == n ? 0 : ys[2] + 1;
    zs[1] = z; zs[0] = z == 0 ? n - 1 : z - 1; zs[2] = z + 1 == n ? 0 : z + 1; zs[3] = zs[2] + 1 == n ? 0 : zs[2] + 1;
  }
  __device__ __forceinline__ const float* row(int oy, int oz) const {
    return phi + (size_t)(unsigned)(zs[oz + 1] * n + ys[oy + 1]) * (unsigned)n;
  }
  __device__ __forceinline__ float ld(const float* p) const { return __ldg(p); }
};

// integrate.py:54-97: the 32 potential taps of the three finite-difference gradients at the
// 8 CIC corners, combined with the CIC weights in the reference's order.
template <class ROWS>
__device__ __forceinline__ void gather_taps(const ROWS& R, int n, const Cell& c, float g[3]) {
  float w[8];
  cic_weights(c, w);
  const int xm = c.x == 0 ? n - 1 : c.x - 1, x1 = c.x + 1 == n ? 0 : c.x + 1, x2 = x1 + 1 == n ? 0 : x1 + 1;
  const int x0 = c.x;
  // the 12 x-rows the 32 taps lie in
  const float* r00 = R.row(0, 0); const float* r10 = R.row(1, 0);
  const float* r01 = R.row(0, 1); const float* r11 = R.row(1, 1);
  const float* rm0 = R.row(-1, 0); const float* rm1 = R.row(-1, 1);
  const float* r20 = R.row(2, 0); const float* r21 = R.row(2, 1);
  const float* r0m = R.row(0, -1); const float* r1m = R.row(1, -1);
  const float* r02 = R.row(0, 2); const float* r12 = R.row(1, 2);
  // x gradient taps: rows (y0|y1, z0|z1) at xm, x0, x1, x2   (naming a<y><z><x>)
  const float a00m = R.ld(r00 + xm), a000 = R.ld(r00 + x0), a001 = R.ld(r00 + x1), a002 = R.ld(r00 + x2);
  const float a10m = R.ld(r10 + xm), a100 = R.ld(r10 + x0), a101 = R.ld(r10 + x1), a102 = R.ld(r10 + x2);
  const float a01m = R.ld(r01 + xm), a010 = R.ld(r01 + x0), a011 = R.ld(r01 + x1), a012 = R.ld(r01 + x2);
  const float a11m = R.ld(r11 + xm), a110 = R.ld(r11 + x0), a111 = R.ld(r11 + x1), a112 = R.ld(r11 + x2);
  // y extension rows ym, y2 at x0, x1 (z0, z1)
  const float bm00 = R.ld(rm0 + x0), bm01 = R.ld(rm0 + x1), b200 = R.ld(r20 + x0), b201 = R.ld(r20 + x1);
  const float bm10 = R.ld(rm1 + x0), bm11 = R.ld(rm1 + x1), b210 = R.ld(r21 + x0), b211 = R.ld(r21 + x1);
  // z extension planes zm, z2 at (x0|x1, y0|y1)
  const float cm00 = R.ld(r0m + x0), cm01 = R.ld(r0m + x1), cm10 = R.ld(r1m + x0), cm11 = R.ld(r1m + x1);
  const float c200 = R.ld(r02 + x0), c201 = R.ld(r02 + x1), c210 = R.ld(r12 + x0), c211 = R.ld(r12 + x1);
  // x axis: g(o) = phi[x+ox-1] - phi[x+ox+1]   (corner naming g<ox><oy><oz>)
  const float gx000 = a00m - a001, gx100 = a000 - a002;
  const float gx010 = a10m - a101, gx110 = a100 - a102;
  const float gx001 = a01m - a011, gx101 = a010 - a012;
  const float gx011 = a11m - a111, gx111 = a110 - a112;
  // y axis: g(o) = phi[y+oy-1] - phi[y+oy+1]
  const float gy000 = bm00 - a100, gy100 = bm01 - a101;
  const float gy010 = a000 - b200, gy110 = a001 - b201;
  const float gy001 = bm10 - a110, gy101 = bm11 - a111;
  const float gy011 = a010 - b210, gy111 = a011 - b211;
  // z axis: g(o) = phi[z+oz-1] - phi[z+oz+1]
  const float gz000 = cm00 - a010, gz100 = cm01 - a011;
  const float gz010 = cm10 - a110, gz110 = cm11 - a111;
  const float gz001 = a000 - c200, gz101 = a001 - c201;
  const float gz011 = a100 - c210, gz111 = a101 - c211;
  // integrate.py:92 order: g*t0 + g_x*t1 + g_y*t2 + g_z*t3 + g_xy*t4 + g_xz*t5 + g_yz*t6 + g_xyz*t7
  g[0] = (gx000 * w[0] + gx100 * w[1] + gx010 * w[2] + gx001 * w[3] + gx110 * w[4] + gx101 * w[5] +
          gx011 * w[6] + gx111 * w[7]) * 0.5f;
  g[1] = (gy000 * w[0] + gy100 * w[1] + gy010 * w[2] + gy001 * w[3] + gy110 * w[4] + gy101 * w[5] +
          gy011 * w[6] + gy111 * w[7]) * 0.5f;
  g[2] = (gz000 * w[0] + gz100 * w[1] + gz010 * w[2] + gz001 * w[3] + gz110 * w[4] + gz101 * w[5] +
          gz011 * w[6] + gz111 * w[7]) * 0.5f;
}

__device__ __forceinline__ void gather_force(const float* __restrict__ phi, int n, const Cell& c, float g[3]) {
  gather_taps(GlobalRows(phi, n, c.y, c.z), n, c, g);
}

// The same force from the three force grids of the spectral gradient (each already the halved
// central difference, -i sin(k_d) phi_k transformed back): 8 taps per axis at the CIC corners,
// combined with the weights in the order of integrate.py:92.
__device__ __forceinline__ void gather_grad(const Sim& S, const Cell& c, float g[3]) {
  float w[8];
  cic_weights(c, w);
  const int n = S.n;
  const int x0 = c.x, x1 = c.x + 1 == n ? 0 : c.x + 1;
  const int y1 = c.y + 1 == n ? 0 : c.y + 1, z1 = c.z + 1 == n ? 0 : c.z + 1;
  const size_t r00 = ((size_t)c.z * n + c.y) * n, r10 = ((size_t)c.z * n + y1) * n;
  const size_t r01 = ((size_t)z1 * n + c.y) * n, r11 = ((size_t)z1 * n + y1) * n;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float* __restrict__ G = S.grad[d];
    g[d] = __ldg(&G[r00 + x0]) * w[0] + __ldg(&G[r00 + x1]) * w[1] + __ldg(&G[r10 + x0]) * w[2] +
           __ldg(&G[r01 + x0]) * w[3] + __ldg(&G[r10 + x1]) * w[4] + __ldg(&G[r01 + x1]) * w[5] +
           __ldg(&G[r11 + x0]) * w[6] + __ldg(&G[r11 + x1]) * w[7];
  }
}

// Kick/drift of one particle whose state and force are in registers; writes it out and
// returns its next key (resident mode with keys_next; else 0xffffffff).
template <int MODE>
__device__ __forceinline__ unsigned kick_store(const Sim& S, const Parts& out, long long sp, long long slot, float px,
                                           float py, float pz, float vx, float vy, float vz, unsigned id,
                                           const float (&g)[3], unsigned* __restrict__ keys_next, int* err) {
  const float kk = S.kick, dr = S.drift;
  vx = fmaf(kk, g[0], vx);
  vy = fmaf(kk, g[1], vy);
  vz = fmaf(kk, g[2], vz);
  if (MODE == POS_ABS) {
    // positions may arrive as exactly n: drift the canonical value and wrap
    const float fn = (float)S.n;
    const float nx = canon(fmaf(dr, vx, canon(px, fn)), fn);
    const float ny = canon(fmaf(dr, vy, canon(py, fn)), fn);
    const float nz = canon(fmaf(dr, vz, canon(pz, fn)), fn);
    if (!(isfinite(nx) && isfinite(ny) && isfinite(nz) && isfinite(vx) && isfinite(vy) && isfinite(vz)))
      set_error(err, ERR_NONFINITE);
    out.x[slot] = nx; out.y[slot] = ny; out.z[slot] = nz;
    out.vx[slot] = vx; out.vy[slot] = vy; out.vz[slot] = vz;
  } else {
    const float nx = fmaf(dr, vx, px), ny = fmaf(dr, vy, py), nz = fmaf(dr, vz, pz);
    if (!(isfinite(nx) && isfinite(ny) && isfinite(nz) && isfinite(vx) && isfinite(vy) && isfinite(vz)))
      set_error(err, ERR_NONFINITE);
    out.x[sp] = nx; out.y[sp] = ny; out.z[sp] = nz;
    out.vx[sp] = vx; out.vy[sp] = vy; out.vz[sp] = vz;
    out.id[sp] = id;
    if (keys_next) {
      Cell cn = cell_disp(S, id, nx, ny, nz);
      if (out.rec) store_cell_record(out, sp, cn);
      if (!cn.ok) { set_error(err, ERR_CELL_RANGE); cn.x = cn.y = cn.z = 0; }
      const unsigned key = cell_key(S, cn);
      keys_next[sp] = key;
      return key;
    }
  }
  return 0xffffffffu;
}

// Each thread advances KICK_PPT particles, KICK_NT apart: all their loads (state, then the
// 32 potential taps each) are issued before any store, so that they overlap.
template <int MODE>
// row_count (optional, with keys_next): histogram of the next keys, for the next step's
// counting sort
__global__ void __launch_bounds__(KICK_NT, 4) k_kick(const Sim* __restrict__ sims, Work w, Parts in, Parts out,
                                                  const unsigned* __restrict__ perm,
                                                  unsigned* __restrict__ keys_next, int* err,
                                                  unsigned* __restrict__ row_count) {
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    const Sim& S = sims[si];
    const long long i0 = (long long)(unit - __ldg(&w.prefix[si])) * (KICK_NT * KICK_PPT) + threadIdx.x;
    long long sp[KICK_PPT], slot[KICK_PPT];
    float px[KICK_PPT], py[KICK_PPT], pz[KICK_PPT], vx[KICK_PPT], vy[KICK_PPT], vz[KICK_PPT];
    unsigned id[KICK_PPT];
    Cell c[KICK_PPT];
#pragma unroll
    for (int q = 0; q < KICK_PPT; ++q) {
      const long long i = i0 + q * KICK_NT;
      sp[q] = S.part_off + i;  // position in sorted order (or slot without perm)
      slot[q] = i < S.np ? (perm ? (long long)__ldg(&perm[sp[q]]) : sp[q]) : -1;
    }
#pragma unroll
    for (int q = 0; q < KICK_PPT; ++q) {
      const long long sl = slot[q] >= 0 ? slot[q] : 0;
      px[q] = in.x[sl]; py[q] = in.y[sl]; pz[q] = in.z[sl];
      vx[q] = in.vx[sl]; vy[q] = in.vy[sl]; vz[q] = in.vz[sl];
      id[q] = MODE == POS_DISP ? in.id[sl] : 0u;
    }
#pragma unroll
    for (int q = 0; q < KICK_PPT; ++q)
      c[q] = MODE == POS_ABS ? cell_abs(px[q], py[q], pz[q], S.n) : cell_disp(S, id[q], px[q], py[q], pz[q]);
    float g[KICK_PPT][3];
#pragma unroll
    for (int q = 0; q < KICK_PPT; ++q) {
      g[q][0] = g[q][1] = g[q][2] = 0.f;
      if (slot[q] >= 0 && c[q].ok) {
        if (S.grad[0]) gather_grad(S, c[q], g[q]);  // spectral gradient: three force grids
        else gather_force(S.phi, S.n, c[q], g[q]);
      }
    }
    unsigned key[KICK_PPT];
#pragma unroll
    for (int q = 0; q < KICK_PPT; ++q) {
      key[q] = 0xffffffffu;
      if (slot[q] < 0) continue;
      if (!c[q].ok) set_error(err, ERR_CELL_RANGE);
      key[q] = kick_store<MODE>(S, out, sp[q], slot[q], px[q], py[q], pz[q], vx[q], vy[q], vz[q], id[q], g[q],
                                keys_next, err);
    }
    if (row_count) {  // the whole warp takes part: equal keys are counted once per warp
      const int lane = threadIdx.x & 31;
#pragma unroll
      for (int q = 0; q < KICK_PPT; ++q) {
        const unsigned grp = __match_any_sync(0xffffffffu, key[q]);
        if (key[q] != 0xffffffffu && lane == __ffs(grp) - 1) atomicAdd(&row_count[key[q]], (unsigned)__popc(grp));
      }
    }
  }
}

// ---------------------------------------------------------------------------------
// coefficients (one thread per simulation, fp64)
// ---------------------------------------------------------------------------------
__global__ void k_coef(Sim* sims, int nsims, int advance) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsims) return;
  Sim& S = sims[s];
  if (advance) {
    S.a += S.da;
    S.step += 1;
  }
  const double a = S.a, da = S.da, a1 = a + da;
  const double n3 = (double)S.n * S.n * S.n;
  S.green = (float)(-3.0 * S.om / 8.0 / a / n3);
  // integrate.py:12 passes [H0, OL, OK]: H0 in the Omega_m slot unless fix_f is set
  const double om_slot = S.fix_f ? S.om : S.h0;
  const double fa1 = 1.0 / sqrt((om_slot + S.ok * a1 + S.ol * a1 * a1 * a1) / a1);
  S.kick = (float)(da * fa1);
  S.drift = (float)(da / (a1 * a1) * fa1);
}

// ---------------------------------------------------------------------------------
// resident-state conversion: absolute (3, np) arrays in particle order <-> displacement
// state at slots [off, off + np)
// ---------------------------------------------------------------------------------
// x-row of the cell of every absolute position (the row part of the cell key, tile order)
__global__ void k_row_keys_abs(const float* __restrict__ pos, long long np, int n, unsigned* __restrict__ keys) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < np;
       i += (long long)gridDim.x * blockDim.x) {
    const Cell c = cell_abs(pos[i], pos[np + i], pos[2 * np + i], n);
    keys[i] = c.ok ? row_number(c.y, c.z, n) : 0u;
  }
}

// order (optional): slot off + i takes particle order[i] (the state is written in row order)
__global__ void k_abs_to_disp(const float* __restrict__ pos, const float* __restrict__ vel, long long np,
                              int np1, int n, const int* __restrict__ q_int, const float* __restrict__ q_frac,
                              Parts out, long long off, const unsigned* __restrict__ order) {
  const float fn = (float)n, half = 0.5f * fn;
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < np;
       s += (long long)gridDim.x * blockDim.x) {
    const long long i = order ? (long long)__ldg(&order[s]) : s;  // the particle
    const unsigned id = (unsigned)i, u1 = (unsigned)np1;
    const unsigned ax[3] = {id / (u1 * u1), (id / u1) % u1, id % u1};
    float* dst[3] = {out.x, out.y, out.z};
    float* vdst[3] = {out.vx, out.vy, out.vz};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float q = (float)__ldg(&q_int[ax[k]]) + __ldg(&q_frac[ax[k]]);
      float d = pos[k * np + i] - q;
      if (d >= half) d -= fn;
      if (d < -half) d += fn;
      dst[k][off + s] = d;
      vdst[k][off + s] = vel[k * np + i];
    }
    out.id[off + s] = pack_lattice(ax[0], ax[1], ax[2]);
  }
}

__global__ void k_disp_to_abs(Parts in, long long off, long long np, int np1, int n,
                              const int* __restrict__ q_int, const float* __restrict__ q_frac,
                              float* __restrict__ pos, float* __restrict__ vel) {
  const float fn = (float)n;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < np;
       j += (long long)gridDim.x * blockDim.x) {
    const long long slot = off + j;
    const unsigned pid = in.id[slot];
    const unsigned ax[3] = {pid >> 20, (pid >> 10) & 1023u, pid & 1023u};
    const long long id = ((long long)ax[0] * np1 + ax[1]) * np1 + ax[2];
    const float dv[3] = {in.x[slot], in.y[slot], in.z[slot]};
    const float vv[3] = {in.vx[slot], in.vy[slot], in.vz[slot]};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float s = __ldg(&q_frac[ax[k]]) + dv[k];
      const float fl = floorf(s);
      float x = (float)wrap_int(__ldg(&q_int[ax[k]]) + (int)fl, n) + (s - fl);
      if (x >= fn) x -= fn;
      pos[k * np + id] = x;
      vel[k * np + id] = vv[k];
    }
  }
}

// ---------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------
cudaError_t launch_abs_to_disp(const float* pos, const float* vel, long long np, int np1, int n,
                               const int* q_int, const float* q_frac, Parts out, long long off,
                               cudaStream_t st, const unsigned* order) {
  long long b = (np + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  k_abs_to_disp<<<(int)b, 256, 0, st>>>(pos, vel, np, np1, n, q_int, q_frac, out, off, order);
  return cudaGetLastError();
}

cudaError_t launch_row_keys_abs(const float* pos, long long np, int n, unsigned* keys, cudaStream_t st) {
  long long b = (np + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  k_row_keys_abs<<<(int)(b > 0 ? b : 1), 256, 0, st>>>(pos, np, n, keys);
  return cudaGetLastError();
}

cudaError_t launch_disp_to_abs(Parts in, long long off, long long np, int np1, int n, const int* q_int,
                               const float* q_frac, float* pos, float* vel, cudaStream_t st) {
  long long b = (np + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  k_disp_to_abs<<<(int)b, 256, 0, st>>>(in, off, np, np1, n, q_int, q_frac, pos, vel);
  return cudaGetLastError();
}

cudaError_t deposit_prepare() {
  static DeviceOnce once;
  return once.run([]() {
  cudaError_t e = cudaFuncSetAttribute(k_deposit<POS_ABS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)deposit_smem_bytes(PM_MAX_N, 4, 4));
  if (!e) e = cudaFuncSetAttribute(k_deposit<POS_DISP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)deposit_smem_bytes(PM_MAX_N, 4, 4));
  if (!e) e = cudaFuncSetAttribute(k_deposit<POS_ABS>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (!e) e = cudaFuncSetAttribute(k_deposit<POS_DISP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  return e;
  });
}

size_t deposit_smem_bytes(int n, int ty, int tz) { return (size_t)n * ty * tz * sizeof(unsigned long long); }

cudaError_t launch_keys_abs(const Sim* sims, const Work& w, Parts p, unsigned* keys, unsigned* vals,
                            int* err, int ctas, cudaStream_t st, Parts copy) {
  k_keys<POS_ABS><<<ctas, KEY_NT, 0, st>>>(sims, w, p, keys, vals, err, copy);
  return cudaGetLastError();
}
cudaError_t launch_keys_disp(const Sim* sims, const Work& w, Parts p, unsigned* keys, unsigned* vals,
                             int* err, int ctas, cudaStream_t st) {
  k_keys<POS_DISP><<<ctas, KEY_NT, 0, st>>>(sims, w, p, keys, vals, err, Parts{});
  return cudaGetLastError();
}

cudaError_t launch_row_start(const unsigned* keys, long long n, int xbits, unsigned nrows,
                             unsigned* row_start, cudaStream_t st) {
  long long work = n + 1;
  int ctas = (int)((work + 255) / 256);
  if (ctas > 152 * 16) ctas = 152 * 16;
  k_row_start<<<ctas, 256, 0, st>>>(keys, n, xbits, nrows, row_start);
  return cudaGetLastError();
}

// Order in which the fused deposit takes its tiles: the dense tiles first.  A tile's work is
// its source-entry count, which clustering makes very uneven; a dense tile taken late runs on
// alone after the others have finished.  Tiles with more than twice the mean count go to the
// front of `order`, the others to the back (their order within each part is immaterial: a
// tile's sums do not depend on when it runs).  counts[0], counts[1]: zero at launch.
__global__ void k_tile_order(const Sim* __restrict__ sims, Work w, const unsigned* __restrict__ row_start,
                             unsigned* __restrict__ order, unsigned* __restrict__ counts) {
  for (int unit = blockIdx.x * blockDim.x + threadIdx.x; unit < w.total; unit += gridDim.x * blockDim.x) {
    const int si = locate_sim(w, unit);
    const Sim& S = sims[si];
    const int n = S.n, local = unit - __ldg(&w.prefix[si]);
    const int y0 = (local % (n / TY)) * TY, z0 = (local / (n / TY)) * TZ;
    unsigned cnt = 0;
#pragma unroll
    for (int r = 0; r < NRUN; ++r) cnt += run_load(S, row_start, y0, z0, r).cnt;
    // mean source entries per tile: each particle once, plus its tile's last plane / row / corner
    const double ntiles = (double)(n / TY) * (n / TZ);
    const double mean = (double)S.np * (1.0 + 1.0 / TZ + 1.0 / TY + 1.0 / (TY * TZ)) / ntiles;
    if (cnt > 2.0 * mean) order[atomicAdd(&counts[0], 1u)] = (unsigned)unit;
    else order[w.total - 1 - (int)atomicAdd(&counts[1], 1u)] = (unsigned)unit;
  }
}

cudaError_t launch_tile_order(const Sim* sims, const Work& w, const unsigned* row_start, unsigned* order,
                              unsigned* counts, int sms, cudaStream_t st) {
  if (w.total <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned), st);
  if (e) return e;
  const int ctas = std::min((w.total + 255) / 256, 4 * sms);
  k_tile_order<<<ctas, 256, 0, st>>>(sims, w, row_start, order, counts);
  return cudaGetLastError();
}

cudaError_t launch_deposit(const Sim* sims, const Work& w, Parts p, const unsigned* perm,
                           const unsigned* row_start, int mode, int* err, int ctas, size_t smem,
                           cudaStream_t st) {
  if (cudaError_t e = deposit_prepare()) return e;
  if (mode == POS_ABS) k_deposit<POS_ABS><<<ctas, DEP_NT, smem, st>>>(sims, w, p, perm, row_start, err);
  else k_deposit<POS_DISP><<<ctas, DEP_NT, smem, st>>>(sims, w, p, perm, row_start, err);
  return cudaGetLastError();
}

cudaError_t launch_kick(const Sim* sims, const Work& w, Parts in, Parts out, const unsigned* perm,
                        unsigned* keys_next, int mode, int* err, int ctas, cudaStream_t st, unsigned* row_count) {
  if (mode == POS_ABS) k_kick<POS_ABS><<<ctas, KICK_NT, 0, st>>>(sims, w, in, out, perm, keys_next, err, nullptr);
  else k_kick<POS_DISP><<<ctas, KICK_NT, 0, st>>>(sims, w, in, out, perm, keys_next, err, row_count);
  return cudaGetLastError();
}

// Absolute state in caller order <-> row order (drop-in step): sorted[j] = state[perm[j]],
// and back, state[i] = sorted[inv[i]] -- gathers, so that the writes stay coalesced.  One
// array per launch: the randomly read source (np floats) then stays in L2.
__global__ void k_gather1(const float* __restrict__ src, long long np, const unsigned* __restrict__ idx,
                          float* __restrict__ dst) {
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < np; j += (long long)gridDim.x * blockDim.x)
    dst[j] = __ldg(&src[__ldg(&idx[j])]);
}

cudaError_t launch_gather_state(const float* pos, const float* vel, long long np, const unsigned* idx, float* spos,
                                float* svel, int sms, cudaStream_t st) {
  long long b = (np + 255) / 256;
  if (b > (long long)sms * 16) b = (long long)sms * 16;
  for (int k = 0; k < 3; ++k) {
    k_gather1<<<(int)b, 256, 0, st>>>(pos + k * np, np, idx, spos + k * np);
    if (vel) k_gather1<<<(int)b, 256, 0, st>>>(vel + k * np, np, idx, svel + k * np);
  }
  return cudaGetLastError();
}

cudaError_t launch_coef(Sim* sims, int nsims, int advance, cudaStream_t st) {
  k_coef<<<(nsims + 127) / 128, 128, 0, st>>>(sims, nsims, advance);
  return cudaGetLastError();
}

}  // namespace pm
