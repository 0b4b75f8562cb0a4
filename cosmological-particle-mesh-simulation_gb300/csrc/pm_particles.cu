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
// Cell key = (global x-row number << xbits) | x, where x-rows are numbered in
// deposit-tile order (a tile is TZ planes x TY rows of full x-rows, TY = TZ = 4).
// Sorting by key groups particles by tile and, inside a tile, by cell.
//
// Resident (displacement) particles carry their Lagrangian lattice index packed as
// ix << 20 | iy << 10 | iz (N_PARTS <= 1024), so no division is needed to find q.
#include "pm_common.cuh"

namespace pm {

constexpr int DEP_NT = 256;
constexpr int KICK_NT = 256;
constexpr int KEY_NT = 256;
constexpr unsigned FULL = 0xffffffffu;
constexpr int TY = 4, TZ = 4, NSRC = (TY + 1) * (TZ + 1);

__host__ __device__ __forceinline__ unsigned pack_lattice(unsigned ix, unsigned iy, unsigned iz) {
  return (ix << 20) | (iy << 10) | iz;
}

// ---------------------------------------------------------------------------------
// cells
// ---------------------------------------------------------------------------------
__device__ __forceinline__ unsigned row_number(int y, int z, int n) {
  const unsigned tile = (unsigned)(z / TZ) * (unsigned)(n / TY) + (unsigned)(y / TY);
  return tile * (unsigned)(TZ * TY) + (unsigned)((z % TZ) * TY + (y % TY));
}

// Q4: a float32 coordinate equal to n (or slightly negative) is mapped into [0, n).
__device__ __forceinline__ float canon(float x, float fn) {
  if (x >= fn) x -= fn;
  if (x < 0.f) x += fn;
  if (x >= fn) x = 0.f;  // -tiny + n rounds to n
  return x;
}

struct Cell {
  int x, y, z;       // base cell
  float fx, fy, fz;  // offsets in [0, 1)
  bool ok;
};

// absolute position -> cell (density.py:19-26 with positions canonicalised)
__device__ __forceinline__ Cell cell_abs(float x, float y, float z, int n) {
  const float fn = (float)n;
  Cell c;
  x = canon(x, fn); y = canon(y, fn); z = canon(z, fn);
  const float lx = floorf(x), ly = floorf(y), lz = floorf(z);
  c.x = (int)lx; c.y = (int)ly; c.z = (int)lz;
  c.fx = x - lx; c.fy = y - ly; c.fz = z - lz;
  c.ok = isfinite(x) && isfinite(y) && isfinite(z) && c.x >= 0 && c.x < n && c.y >= 0 && c.y < n &&
         c.z >= 0 && c.z < n;
  return c;
}

__device__ __forceinline__ int wrap_int(int c, int n) {
  if ((unsigned)c < (unsigned)n) return c;
  if (c >= n && c < 2 * n) return c - n;
  if (c < 0 && c >= -n) return c + n;
  c %= n;
  return c < 0 ? c + n : c;
}

// displacement from the Lagrangian lattice point -> cell:
//   cell = (q_int + floor(q_frac + d)) mod n,  offset = (q_frac + d) - floor(q_frac + d)
__device__ __forceinline__ Cell cell_disp(const Sim& S, unsigned id, float dx, float dy, float dz) {
  const unsigned ix = id >> 20, iy = (id >> 10) & 1023u, iz = id & 1023u;
  const float sx = __ldg(&S.q_frac[ix]) + dx;
  const float sy = __ldg(&S.q_frac[iy]) + dy;
  const float sz = __ldg(&S.q_frac[iz]) + dz;
  const float lx = floorf(sx), ly = floorf(sy), lz = floorf(sz);
  Cell c;
  c.ok = isfinite(sx) && isfinite(sy) && isfinite(sz) && fabsf(lx) < 1e8f && fabsf(ly) < 1e8f &&
         fabsf(lz) < 1e8f;
  const int n = S.n;
  c.x = c.ok ? wrap_int(__ldg(&S.q_int[ix]) + (int)lx, n) : 0;
  c.y = c.ok ? wrap_int(__ldg(&S.q_int[iy]) + (int)ly, n) : 0;
  c.z = c.ok ? wrap_int(__ldg(&S.q_int[iz]) + (int)lz, n) : 0;
  c.fx = sx - lx; c.fy = sy - ly; c.fz = sz - lz;
  return c;
}

template <int MODE>
__device__ __forceinline__ Cell particle_cell(const Sim& S, const Parts& p, long long slot) {
  if (MODE == POS_ABS) return cell_abs(p.x[slot], p.y[slot], p.z[slot], S.n);
  return cell_disp(S, p.id[slot], p.x[slot], p.y[slot], p.z[slot]);
}

__device__ __forceinline__ unsigned cell_key(const Sim& S, const Cell& c) {
  return ((S.row_base + row_number(c.y, c.z, S.n)) << S.xbits) | (unsigned)c.x;
}

// The 8 CIC weights in the order of integrate.py:44-51: [ttt, dtt, tdt, ttd, ddt, dtd, tdd, ddd]
__device__ __forceinline__ void cic_weights(const Cell& c, float w[8]) {
  const float tx = 1.f - c.fx, ty = 1.f - c.fy, tz = 1.f - c.fz;
  w[0] = tx * ty * tz;
  w[1] = c.fx * ty * tz;
  w[2] = tx * c.fy * tz;
  w[3] = tx * ty * c.fz;
  w[4] = c.fx * c.fy * tz;
  w[5] = c.fx * ty * c.fz;
  w[6] = tx * c.fy * c.fz;
  w[7] = c.fx * c.fy * c.fz;
}
// corner offsets of the weights above
__device__ __constant__ int c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                              {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

// ---------------------------------------------------------------------------------
// keys
// ---------------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(KEY_NT) k_keys(const Sim* __restrict__ sims, Work w, Parts p,
                                                 unsigned* __restrict__ keys,
                                                 unsigned* __restrict__ vals, int* err) {
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    const Sim& S = sims[si];
    const long long i = (long long)(unit - __ldg(&w.prefix[si])) * KEY_NT + threadIdx.x;
    if (i >= S.np) continue;
    const long long slot = S.part_off + i;
    Cell c = particle_cell<MODE>(S, p, slot);
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
// deposit
//
// One CTA per deposit tile (tz x ty full x-rows).  It gathers every particle whose base
// cell lies in the tile's source rows (the tile plus one row/plane below, periodic),
// adds the CIC weights that land inside the tile to integer accumulators in shared
// memory (weights quantised to 2^-26; a 32-bit low word with carry into a 32-bit high
// word, so the sum is exact and independent of the order of the atomics), then writes
// the tile's rows once.  Lanes that hit the same cell in one atomic instruction are
// serialised by the hardware; their integer sum is the same in any order.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void acc_add(unsigned* lo, unsigned* hi, int i, unsigned q) {
  const unsigned old = atomicAdd(&lo[i], q);
  if (old + q < old) atomicAdd(&hi[i], 1u);
}

__device__ __forceinline__ float fixed_to_float(unsigned l, unsigned h, float scale) {
  return (h == 0u ? __uint2float_rn(l) : __ull2float_rn(((unsigned long long)h << 32) | l)) * scale;
}

template <int MODE>
__global__ void __launch_bounds__(DEP_NT) k_deposit(const Sim* __restrict__ sims, Work w, Parts p,
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
    const int ncell = TZ * TY * n;  // a multiple of 64
    unsigned* lo = reinterpret_cast<unsigned*>(acc_raw);
    unsigned* hi = lo + ncell;
    for (int i = threadIdx.x; i < ncell / 2; i += DEP_NT) acc_raw[i] = make_uint4(0u, 0u, 0u, 0u);
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
    for (unsigned base = (unsigned)warp * 32u; base < total; base += DEP_NT) {
      const unsigned f = base + lane;
      const bool valid = f < total;
      float wt[8];
      int cx = 0, ly = 0, lz = 0;
      bool ok = false;
      if (valid) {
        int r = 0;  // last source row with s_off[r] <= f
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (r + step < NSRC && s_off[r + step] <= f) r += step;
        const unsigned slot = __ldg(&perm[s_begin[r] + (f - s_off[r])]);
        const Cell c = particle_cell<MODE>(S, p, slot);
        int dy = c.y - y0, dz = c.z - z0;
        if (dy >= n - 1) dy -= n;
        if (dz >= n - 1) dz -= n;
        ok = c.ok && dy >= -1 && dy < TY && dz >= -1 && dz < TZ;
        if (!ok) {
          set_error(err, c.ok ? ERR_SOURCE_ROW : ERR_CELL_RANGE);
        } else {
          cic_weights(c, wt);
          cx = c.x; ly = dy; lz = dz;
        }
      }
      if (ok) {
        const int x1 = cx + 1 == n ? 0 : cx + 1;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int ty2 = ly + c_corner[k][1], tz2 = lz + c_corner[k][2];
          if (ty2 >= 0 && ty2 < TY && tz2 >= 0 && tz2 < TZ)
            acc_add(lo, hi, (tz2 * TY + ty2) * n + (c_corner[k][0] ? x1 : cx),
                    __float2uint_rn(wt[k] * (float)(1u << PM_FIX_BITS)));
        }
      }
    }
    __syncthreads();
    const float ms = S.mass_scale;
    for (int row = warp; row < TZ * TY; row += DEP_NT / 32) {
      const uint4* l4 = reinterpret_cast<const uint4*>(lo + row * n);
      const uint4* h4 = reinterpret_cast<const uint4*>(hi + row * n);
      float4* dst = reinterpret_cast<float4*>(S.rho + ((long long)(z0 + row / TY) * n + (y0 + row % TY)) * n);
      for (int x4 = lane; x4 < n / 4; x4 += 32) {
        const uint4 l = l4[x4], h = h4[x4];
        dst[x4] = make_float4(fixed_to_float(l.x, h.x, ms), fixed_to_float(l.y, h.y, ms),
                              fixed_to_float(l.z, h.z, ms), fixed_to_float(l.w, h.w, ms));
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
__device__ __forceinline__ void gather_force(const float* __restrict__ phi, int n, const Cell& c,
                                             float g[3]) {
  float w[8];
  cic_weights(c, w);
  const int xm = c.x == 0 ? n - 1 : c.x - 1, x1 = c.x + 1 == n ? 0 : c.x + 1, x2 = x1 + 1 == n ? 0 : x1 + 1;
  const int ym = c.y == 0 ? n - 1 : c.y - 1, y1 = c.y + 1 == n ? 0 : c.y + 1, y2 = y1 + 1 == n ? 0 : y1 + 1;
  const int zm = c.z == 0 ? n - 1 : c.z - 1, z1 = c.z + 1 == n ? 0 : c.z + 1, z2 = z1 + 1 == n ? 0 : z1 + 1;
  const int x0 = c.x, y0 = c.y, z0 = c.z;
  const long long nn = n;
  auto P = [&](int x, int y, int z) { return __ldg(&phi[((long long)z * nn + y) * nn + x]); };
  // x gradient: rows (y0|y1, z0|z1) at xm, x0, x1, x2
  const float a00m = P(xm, y0, z0), a000 = P(x0, y0, z0), a001 = P(x1, y0, z0), a002 = P(x2, y0, z0);
  const float a10m = P(xm, y1, z0), a100 = P(x0, y1, z0), a101 = P(x1, y1, z0), a102 = P(x2, y1, z0);
  const float a01m = P(xm, y0, z1), a010 = P(x0, y0, z1), a011 = P(x1, y0, z1), a012 = P(x2, y0, z1);
  const float a11m = P(xm, y1, z1), a110 = P(x0, y1, z1), a111 = P(x1, y1, z1), a112 = P(x2, y1, z1);
  // y extension rows ym, y2 at x0, x1 (z0, z1)
  const float bm00 = P(x0, ym, z0), bm01 = P(x1, ym, z0), b200 = P(x0, y2, z0), b201 = P(x1, y2, z0);
  const float bm10 = P(x0, ym, z1), bm11 = P(x1, ym, z1), b210 = P(x0, y2, z1), b211 = P(x1, y2, z1);
  // z extension planes zm, z2 at (x0|x1, y0|y1)
  const float cm00 = P(x0, y0, zm), cm01 = P(x1, y0, zm), cm10 = P(x0, y1, zm), cm11 = P(x1, y1, zm);
  const float c200 = P(x0, y0, z2), c201 = P(x1, y0, z2), c210 = P(x0, y1, z2), c211 = P(x1, y1, z2);
  // phi at corner (ox, oy, oz): a[oy][oz][ox] with a?? naming: a<y><z><x>
  // x axis: g(o) = phi[x+ox-1] - phi[x+ox+1]
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
  // corner naming g<ox><oy><oz>
  g[0] = (gx000 * w[0] + gx100 * w[1] + gx010 * w[2] + gx001 * w[3] + gx110 * w[4] + gx101 * w[5] +
          gx011 * w[6] + gx111 * w[7]) * 0.5f;
  g[1] = (gy000 * w[0] + gy100 * w[1] + gy010 * w[2] + gy001 * w[3] + gy110 * w[4] + gy101 * w[5] +
          gy011 * w[6] + gy111 * w[7]) * 0.5f;
  g[2] = (gz000 * w[0] + gz100 * w[1] + gz010 * w[2] + gz001 * w[3] + gz110 * w[4] + gz101 * w[5] +
          gz011 * w[6] + gz111 * w[7]) * 0.5f;
}

template <int MODE>
__global__ void __launch_bounds__(KICK_NT) k_kick(const Sim* __restrict__ sims, Work w, Parts in, Parts out,
                                                  const unsigned* __restrict__ perm,
                                                  unsigned* __restrict__ keys_next, int* err) {
  for (int unit = blockIdx.x; unit < w.total; unit += gridDim.x) {
    const int si = locate_sim(w, unit);
    const Sim& S = sims[si];
    const long long i = (long long)(unit - __ldg(&w.prefix[si])) * KICK_NT + threadIdx.x;
    if (i >= S.np) continue;
    const long long sp = S.part_off + i;  // position in sorted order (or slot without perm)
    const long long slot = perm ? (long long)__ldg(&perm[sp]) : sp;
    const float px = in.x[slot], py = in.y[slot], pz = in.z[slot];
    float vx = in.vx[slot], vy = in.vy[slot], vz = in.vz[slot];
    Cell c;
    unsigned id = 0;
    if (MODE == POS_ABS) {
      c = cell_abs(px, py, pz, S.n);
    } else {
      id = in.id[slot];
      c = cell_disp(S, id, px, py, pz);
    }
    float g[3] = {0.f, 0.f, 0.f};
    if (c.ok) gather_force(S.phi, S.n, c, g);
    else set_error(err, ERR_CELL_RANGE);
    const float kk = S.kick, dr = S.drift;
    vx = fmaf(kk, g[0], vx);
    vy = fmaf(kk, g[1], vy);
    vz = fmaf(kk, g[2], vz);
    float nx = fmaf(dr, vx, px), ny = fmaf(dr, vy, py), nz = fmaf(dr, vz, pz);
    if (!(isfinite(nx) && isfinite(ny) && isfinite(nz) && isfinite(vx) && isfinite(vy) && isfinite(vz)))
      set_error(err, ERR_NONFINITE);
    if (MODE == POS_ABS) {
      const float fn = (float)S.n;
      // positions may arrive as exactly n (Q4): wrap the canonical value
      nx = canon(fmaf(dr, vx, canon(px, fn)), fn);
      ny = canon(fmaf(dr, vy, canon(py, fn)), fn);
      nz = canon(fmaf(dr, vz, canon(pz, fn)), fn);
      out.x[slot] = nx; out.y[slot] = ny; out.z[slot] = nz;
      out.vx[slot] = vx; out.vy[slot] = vy; out.vz[slot] = vz;
    } else {
      out.x[sp] = nx; out.y[sp] = ny; out.z[sp] = nz;
      out.vx[sp] = vx; out.vy[sp] = vy; out.vz[sp] = vz;
      out.id[sp] = id;
      if (keys_next) {
        Cell cn = cell_disp(S, id, nx, ny, nz);
        if (!cn.ok) { set_error(err, ERR_CELL_RANGE); cn.x = cn.y = cn.z = 0; }
        keys_next[sp] = cell_key(S, cn);
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
__global__ void k_abs_to_disp(const float* __restrict__ pos, const float* __restrict__ vel, long long np,
                              int np1, int n, const int* __restrict__ q_int, const float* __restrict__ q_frac,
                              Parts out, long long off) {
  const float fn = (float)n, half = 0.5f * fn;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < np;
       i += (long long)gridDim.x * blockDim.x) {
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
      dst[k][off + i] = d;
      vdst[k][off + i] = vel[k * np + i];
    }
    out.id[off + i] = pack_lattice(ax[0], ax[1], ax[2]);
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
                               cudaStream_t st) {
  long long b = (np + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  k_abs_to_disp<<<(int)b, 256, 0, st>>>(pos, vel, np, np1, n, q_int, q_frac, out, off);
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
  cudaError_t e = cudaFuncSetAttribute(k_deposit<POS_ABS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)deposit_smem_bytes(PM_MAX_N, 4, 4));
  if (!e) e = cudaFuncSetAttribute(k_deposit<POS_DISP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)deposit_smem_bytes(PM_MAX_N, 4, 4));
  if (!e) e = cudaFuncSetAttribute(k_deposit<POS_ABS>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (!e) e = cudaFuncSetAttribute(k_deposit<POS_DISP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  return e;
}

size_t deposit_smem_bytes(int n, int ty, int tz) { return (size_t)n * ty * tz * sizeof(unsigned long long); }

cudaError_t launch_keys_abs(const Sim* sims, const Work& w, Parts p, unsigned* keys, unsigned* vals,
                            int* err, int ctas, cudaStream_t st) {
  k_keys<POS_ABS><<<ctas, KEY_NT, 0, st>>>(sims, w, p, keys, vals, err);
  return cudaGetLastError();
}
cudaError_t launch_keys_disp(const Sim* sims, const Work& w, Parts p, unsigned* keys, unsigned* vals,
                             int* err, int ctas, cudaStream_t st) {
  k_keys<POS_DISP><<<ctas, KEY_NT, 0, st>>>(sims, w, p, keys, vals, err);
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

cudaError_t launch_deposit(const Sim* sims, const Work& w, Parts p, const unsigned* perm,
                           const unsigned* row_start, int mode, int* err, int ctas, size_t smem,
                           cudaStream_t st) {
  static bool init = false;
  if (!init) {
    cudaError_t e = deposit_prepare();
    if (e) return e;
    init = true;
  }
  if (mode == POS_ABS) k_deposit<POS_ABS><<<ctas, DEP_NT, smem, st>>>(sims, w, p, perm, row_start, err);
  else k_deposit<POS_DISP><<<ctas, DEP_NT, smem, st>>>(sims, w, p, perm, row_start, err);
  return cudaGetLastError();
}

cudaError_t launch_kick(const Sim* sims, const Work& w, Parts in, Parts out, const unsigned* perm,
                        unsigned* keys_next, int mode, int* err, int ctas, cudaStream_t st) {
  if (mode == POS_ABS) k_kick<POS_ABS><<<ctas, KICK_NT, 0, st>>>(sims, w, in, out, perm, keys_next, err);
  else k_kick<POS_DISP><<<ctas, KICK_NT, 0, st>>>(sims, w, in, out, perm, keys_next, err);
  return cudaGetLastError();
}

cudaError_t launch_coef(Sim* sims, int nsims, int advance, cudaStream_t st) {
  k_coef<<<(nsims + 127) / 128, 128, 0, st>>>(sims, nsims, advance);
  return cudaGetLastError();
}

}  // namespace pm
