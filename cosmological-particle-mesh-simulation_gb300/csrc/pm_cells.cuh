// Particle cells, CIC weights and cell keys, shared by the particle kernels and the fused
// deposit + x-transform kernel.
//
// Cell key = (global x-row number << xbits) | x, where x-rows are numbered in
// deposit-tile order (a tile is TZ planes x TY rows of full x-rows, TY = TZ = 4).
// Sorting by key groups particles by tile and, inside a tile, by cell.
//
// Resident (displacement) particles carry their Lagrangian lattice index packed as
// ix << 20 | iy << 10 | iz (N_PARTS <= 1024), so no division is needed to find q.
#pragma once
#include "pm_common.cuh"

namespace pm {

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

// A float32 coordinate equal to n (or slightly negative) is mapped into [0, n).
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
  // integer lattice step (np1 divides n): q_int = q_step i and q_frac = 1/2 exactly, the
  // same values the tables hold, without the tables' scattered loads
  const int qs = S.q_step;
  const float sx = (qs ? 0.5f : __ldg(&S.q_frac[ix])) + dx;
  const float sy = (qs ? 0.5f : __ldg(&S.q_frac[iy])) + dy;
  const float sz = (qs ? 0.5f : __ldg(&S.q_frac[iz])) + dz;
  const float lx = floorf(sx), ly = floorf(sy), lz = floorf(sz);
  Cell c;
  c.ok = isfinite(sx) && isfinite(sy) && isfinite(sz) && fabsf(lx) < 1e8f && fabsf(ly) < 1e8f &&
         fabsf(lz) < 1e8f;
  const int n = S.n;
  const int qx = qs ? qs * (int)ix : __ldg(&S.q_int[ix]);
  const int qy = qs ? qs * (int)iy : __ldg(&S.q_int[iy]);
  const int qz = qs ? qs * (int)iz : __ldg(&S.q_int[iz]);
  c.x = c.ok ? wrap_int(qx + (int)lx, n) : 0;
  c.y = c.ok ? wrap_int(qy + (int)ly, n) : 0;
  c.z = c.ok ? wrap_int(qz + (int)lz, n) : 0;
  c.fx = sx - lx; c.fy = sy - ly; c.fz = sz - lz;
  return c;
}

constexpr unsigned CELL_BAD = 0xffffffffu;

__device__ __forceinline__ void store_cell_record(const Parts& p, long long i, const Cell& c) {
  p.rec[i] = make_uint4(c.ok ? ((unsigned)c.x | ((unsigned)c.y << 10) | ((unsigned)c.z << 20)) : CELL_BAD,
                        __float_as_uint(c.fx), __float_as_uint(c.fy), __float_as_uint(c.fz));
}

__device__ __forceinline__ Cell record_cell(const uint4& v) {
  Cell c;
  c.ok = v.x != CELL_BAD;
  c.x = (int)(v.x & 1023u);
  c.y = (int)((v.x >> 10) & 1023u);
  c.z = (int)((v.x >> 20) & 1023u);
  c.fx = __uint_as_float(v.y);
  c.fy = __uint_as_float(v.z);
  c.fz = __uint_as_float(v.w);
  return c;
}

__device__ __forceinline__ Cell load_cell_record(const Parts& p, long long i) { return record_cell(p.rec[i]); }

// The base cell of a particle: from its absolute position, its cell record, or its
// displacement (POS_DISP without records).
template <int MODE>
__device__ __forceinline__ Cell particle_cell(const Sim& S, const Parts& p, long long slot) {
  if (MODE == POS_ABS) return cell_abs(p.x[slot], p.y[slot], p.z[slot], S.n);
  if (p.rec) return load_cell_record(p, slot);
  return cell_disp(S, p.id[slot], p.x[slot], p.y[slot], p.z[slot]);
}

// The same in two steps, so that the loads can be issued early: the four words the cell is
// made from (record: cell word and offsets; displacement: id and d; absolute: x, y, z),
// then the cell.  present false: no particle (the words are not loaded).
struct RawCell {
  unsigned w;
  float a, b, c;
  bool present;
};

template <int MODE>
__device__ __forceinline__ RawCell load_raw_cell(const Parts& p, unsigned slot) {
  RawCell r{0u, 0.f, 0.f, 0.f, slot != 0xffffffffu};
  if (!r.present) return r;
  if (MODE == POS_DISP && p.rec) {
    const uint4 v = __ldg(&p.rec[slot]);
    r.w = v.x; r.a = __uint_as_float(v.y); r.b = __uint_as_float(v.z); r.c = __uint_as_float(v.w);
  } else {
    if (MODE == POS_DISP) r.w = p.id[slot];
    r.a = p.x[slot]; r.b = p.y[slot]; r.c = p.z[slot];
  }
  return r;
}

template <int MODE>
__device__ __forceinline__ Cell raw_cell(const Sim& S, const Parts& p, const RawCell& r) {
  if (MODE == POS_ABS) return cell_abs(r.a, r.b, r.c, S.n);
  if (p.rec) return record_cell(make_uint4(r.w, __float_as_uint(r.a), __float_as_uint(r.b), __float_as_uint(r.c)));
  return cell_disp(S, r.w, r.a, r.b, r.c);
}

// xbits == 0 (resident batches): the key is the x-row number alone
__device__ __forceinline__ unsigned cell_key(const Sim& S, const Cell& c) {
  const unsigned row = S.row_base + row_number(c.y, c.z, S.n);
  return S.xbits ? ((row << S.xbits) | (unsigned)c.x) : row;
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
// (corner offsets (ox, oy, oz) of the weights above: 0 (0,0,0), 1 (1,0,0), 2 (0,1,0), 3 (0,0,1),
// 4 (1,1,0), 5 (1,0,1), 6 (0,1,1), 7 (1,1,1))

}  // namespace pm
