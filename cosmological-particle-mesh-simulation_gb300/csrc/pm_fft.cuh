// Shared-memory Stockham FFT for batches of lines (radix 2, 3, 4, 8).
//
// A CTA holds NL lines of L complex elements in shared memory.  Two layouts:
//   Interleaved<LS>: element j of line l at s[j * LS + l];
//   Blocked<L, BW>:  lines in blocks of BW (a TMA box of BW columns), element j of line l at
//                    s[(l / BW) * L * BW + j * BW + l % BW].
// Either way consecutive threads (consecutive lines) touch consecutive words.
// Each pass loads all of its butterflies into registers, synchronises, and writes the
// self-sorted (Stockham) output back in place; the last pass leaves natural order.
// Twiddles come from a table tw[m] = exp(-2 pi i m / (L * tws)) read with stride tws.
#pragma once
#include <cuda_runtime.h>

namespace pm {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i (forward transform) or +i (inverse transform)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---------------------------------------------------------------------------------
// Small DFTs in registers.  Forward uses exp(-2 pi i jk / R), inverse exp(+...).
// ---------------------------------------------------------------------------------
template <int R, bool INV> struct DFT;

template <bool INV> struct DFT<2, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float2 a = v[0];
    v[0] = cadd(a, v[1]);
    v[1] = csub(a, v[1]);
  }
};

template <bool INV> struct DFT<4, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    const float2 t2 = cadd(v[1], v[3]), t3 = mul_mi<INV>(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  }
};

template <bool INV> struct DFT<3, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float s3 = 0.866025403784438646763723f;  // sin(2 pi / 3)
    const float2 s = cadd(v[1], v[2]);
    const float2 d = csub(v[1], v[2]);
    const float2 m = make_float2(v[0].x - 0.5f * s.x, v[0].y - 0.5f * s.y);
    const float2 t = cscale(mul_mi<INV>(d), s3);
    v[0] = cadd(v[0], s);
    v[1] = cadd(m, t);
    v[2] = csub(m, t);
  }
};

template <bool INV> struct DFT<8, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float c = 0.707106781186547524400844f;  // sqrt(1/2)
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    DFT<4, INV>::run(e);
    DFT<4, INV>::run(o);
    // o[k] *= exp(-/+ 2 pi i k / 8)
    const float2 o1 = o[1], o3 = o[3];
    if (!INV) {
      o[1] = make_float2(c * (o1.x + o1.y), c * (o1.y - o1.x));
      o[3] = make_float2(c * (o3.y - o3.x), -c * (o3.x + o3.y));
    } else {
      o[1] = make_float2(c * (o1.x - o1.y), c * (o1.x + o1.y));
      o[3] = make_float2(-c * (o3.x + o3.y), c * (o3.x - o3.y));
    }
    o[2] = mul_mi<INV>(o[2]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = cadd(e[k], o[k]);
      v[k + 4] = csub(e[k], o[k]);
    }
  }
};

// 16 = 4 x 4: j = 4 a + b, k = c + 4 d; twiddles w16^(b c) between the two radix-4 stages.
template <bool INV> struct DFT<16, INV> {
  static __device__ __forceinline__ void run(float2* v) {
    const float c1 = 0.923879532511286756128f, s1 = 0.382683432365089771728f;  // cos, sin(pi/8)
    const float h = 0.707106781186547524400844f;                              // sqrt(1/2)
    // w16^m (forward: exp(-2 pi i m / 16)) for the products b c in {1, 2, 3, 4, 6, 9}
    const float sg = INV ? 1.f : -1.f;
    const float2 w1 = make_float2(c1, sg * s1), w2 = make_float2(h, sg * h), w3 = make_float2(s1, sg * c1);
    const float2 w6 = make_float2(-h, sg * h), w9 = make_float2(-c1, -sg * s1);
    float2 t[4][4];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      float2 x[4] = {v[b], v[4 + b], v[8 + b], v[12 + b]};
      DFT<4, INV>::run(x);
#pragma unroll
      for (int c = 0; c < 4; ++c) t[b][c] = x[c];
    }
    t[1][1] = cmul(t[1][1], w1); t[1][2] = cmul(t[1][2], w2); t[1][3] = cmul(t[1][3], w3);
    t[2][1] = cmul(t[2][1], w2); t[2][2] = mul_mi<INV>(t[2][2]); t[2][3] = cmul(t[2][3], w6);
    t[3][1] = cmul(t[3][1], w3); t[3][2] = cmul(t[3][2], w6); t[3][3] = cmul(t[3][3], w9);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float2 y[4] = {t[0][c], t[1][c], t[2][c], t[3][c]};
      DFT<4, INV>::run(y);
#pragma unroll
      for (int d = 0; d < 4; ++d) v[c + 4 * d] = y[d];
    }
  }
};

// Composite DFT of R = R1 R2 points in registers: j = R2 a + b, k = c + R1 d; an R1-point DFT
// over a for each b, twiddles w_R^(b c) (forward exp(-2 pi i m / R)), an R2-point DFT over b.
// WR::w(m) gives w_R^m for the forward direction.
template <int R1, int R2, class WR, bool INV>
__device__ __forceinline__ void dft_composite(float2* v) {
  float2 t[R2][R1];
#pragma unroll
  for (int b = 0; b < R2; ++b) {
    float2 x[R1];
#pragma unroll
    for (int a = 0; a < R1; ++a) x[a] = v[R2 * a + b];
    DFT<R1, INV>::run(x);
#pragma unroll
    for (int c = 0; c < R1; ++c) {
      if (b * c == 0) {
        t[b][c] = x[c];
      } else {
        float2 w = WR::w((b * c) % (R1 * R2));
        if (INV) w.y = -w.y;
        t[b][c] = cmul(x[c], w);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < R1; ++c) {
    float2 y[R2];
#pragma unroll
    for (int b = 0; b < R2; ++b) y[b] = t[b][c];
    DFT<R2, INV>::run(y);
#pragma unroll
    for (int d = 0; d < R2; ++d) v[c + R1 * d] = y[d];
  }
}

// exp(-2 pi i m / 12) and exp(-2 pi i m / 24): multiples of 30 and 15 degrees
struct W12 {
  static __device__ __forceinline__ float2 w(int m) {
    const float h = 0.5f, r = 0.866025403784438646763723f;  // cos 60, cos 30
    const float c[12] = {1.f, r, h, 0.f, -h, -r, -1.f, -r, -h, 0.f, h, r};
    const float s[12] = {0.f, h, r, 1.f, r, h, 0.f, -h, -r, -1.f, -r, -h};
    return make_float2(c[m], -s[m]);
  }
};
struct W24 {
  static __device__ __forceinline__ float2 w(int m) {
    const float a = 0.965925826289068286749743f, b = 0.258819045102520762348898f;  // cos, sin 15
    const float h = 0.5f, r = 0.866025403784438646763723f, q = 0.707106781186547524400844f;
    const float c[24] = {1.f, a, r, q, h, b, 0.f, -b, -h, -q, -r, -a, -1.f, -a, -r, -q, -h, -b, 0.f, b, h, q, r, a};
    const float s[24] = {0.f, b, h, q, r, a, 1.f, a, r, q, h, b, 0.f, -b, -h, -q, -r, -a, -1.f, -a, -r, -q, -h, -b};
    return make_float2(c[m], -s[m]);
  }
};

template <bool INV> struct DFT<12, INV> {
  static __device__ __forceinline__ void run(float2* v) { dft_composite<3, 4, W12, INV>(v); }
};
template <bool INV> struct DFT<24, INV> {
  static __device__ __forceinline__ void run(float2* v) { dft_composite<3, 8, W24, INV>(v); }
};

// ---------------------------------------------------------------------------------
// Radix plans (product of radices == L).  Fewer passes mean fewer shared-memory round trips:
// the two-pass plans of 128, 192, 256 and 384 and the three-pass plan of 1024 measured, per
// 134M cells (y, z in ms), 128: 0.191, 0.311 -> 0.174, 0.265; 192: 0.243, 0.497 -> 0.228,
// 0.335; 256: 0.208, 0.340 -> 0.190, 0.281; 384: 0.304, 0.843 -> 0.243, 0.631; 1024 (y, per
// 1.07G cells): 1.88 -> 1.51.  512 keeps three radix-8 passes on pairs of lines (16 x 32 line
// by line: z 0.291 -> 0.303 ms, half the threads idle in the radix-32 pass).
// ---------------------------------------------------------------------------------
template <int L> struct Plan;
#define PM_PLAN(L_, ...)                                   \
  template <> struct Plan<L_> {                            \
    static constexpr int r[] = {__VA_ARGS__};              \
    static constexpr int np = sizeof(r) / sizeof(int);     \
  };
PM_PLAN(8, 8)
PM_PLAN(12, 3, 4)
PM_PLAN(16, 4, 4)
PM_PLAN(24, 3, 8)
PM_PLAN(32, 4, 8)
PM_PLAN(48, 3, 4, 4)
PM_PLAN(64, 8, 8)
PM_PLAN(96, 3, 4, 8)
PM_PLAN(128, 8, 16)
PM_PLAN(192, 12, 16)
PM_PLAN(256, 16, 16)
PM_PLAN(384, 24, 16)
PM_PLAN(512, 8, 8, 8)
PM_PLAN(768, 3, 4, 8, 8)
PM_PLAN(1024, 16, 8, 8)
#undef PM_PLAN

template <int LS>
struct Interleaved {
  static __device__ __forceinline__ int at(int j, int line) { return j * LS + line; }
};

template <int L, int BW>
struct Blocked {
  static __device__ __forceinline__ int at(int j, int line) {
    return (line / BW) * (L * BW) + j * BW + (line % BW);
  }
};

// No-op epilogue of a pass.
struct NoEpi {
  __device__ __forceinline__ float2 operator()(float2 v, int /*j*/, int /*line*/) const { return v; }
};

// One Stockham pass of radix R on NL lines (in place through registers).  `epi` maps each
// output value (element j of `line`) before it is stored.
template <int L, int R, int NS, int NL, class LAY, int NT, bool INV, class EPI = NoEpi>
__device__ __forceinline__ void stockham_pass(float2* s, const float2* __restrict__ tw, int tws,
                                              const EPI& epi = EPI()) {
  constexpr int NB = L / R;
  constexpr int NTASK = NL * NB;
  constexpr int TPT = (NTASK + NT - 1) / NT;
  float2 v[TPT][R];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int task = threadIdx.x + t * NT;
    if ((NTASK % NT) == 0 || task < NTASK) {
      const int line = task % NL, j = task / NL;
#pragma unroll
      for (int r = 0; r < R; ++r) v[t][r] = s[LAY::at(j + r * NB, line)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int task = threadIdx.x + t * NT;
    if ((NTASK % NT) == 0 || task < NTASK) {
      const int line = task % NL, j = task / NL;
      const int k = j % NS;
      if (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          float2 w = __ldg(&tw[(r * k * (L / (NS * R))) * tws]);
          if (INV) w.y = -w.y;
          v[t][r] = cmul(v[t][r], w);
        }
      }
      DFT<R, INV>::run(v[t]);
      const int base = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) s[LAY::at(base + r * NS, line)] = epi(v[t][r], base + r * NS, line);
    }
  }
  __syncthreads();
}

template <int L, int P, int NS, int NL, class LAY, int NT, bool INV, class EPI = NoEpi>
__device__ __forceinline__ void fft_passes(float2* s, const float2* __restrict__ tw, int tws,
                                           const EPI& epi = EPI()) {
  if constexpr (P < Plan<L>::np) {
    constexpr int R = Plan<L>::r[P];
    if constexpr (P + 1 == Plan<L>::np) {
      stockham_pass<L, R, NS, NL, LAY, NT, INV, EPI>(s, tw, tws, epi);  // last pass: natural order
    } else {
      stockham_pass<L, R, NS, NL, LAY, NT, INV>(s, tw, tws);
      fft_passes<L, P + 1, NS * R, NL, LAY, NT, INV, EPI>(s, tw, tws, epi);
    }
  }
}

// Lengths whose blocked transforms run on pairs of lines: the plans of radix 8 or less, and
// 128 (8 x 16).  The radix-12/16/24 plans hold too many values per pair of lines and run
// line by line (on pairs they spill).
__host__ __device__ constexpr bool blocked_pairs(int L) { return L % 3 != 0 && L != 256 && L != 1024; }

// Whether task j of a stride-1 pass over NP pairs of lines stores its R outputs in the order
// r ^ 1: with 4 pairs, the 8 lanes of a quarter-warp (one phase of a 128-bit shared-memory
// access) hold j and j + 1, whose outputs R j + r lie R 16-byte words apart -- a multiple
// of the 8 words of a bank row, so in the same banks.  Odd j then write the neighbouring
// word first, which sits 4 banks over: conflict-free phases.  The swap costs selects, so
// only the shared-memory-bound z pass takes it (BANKS); the HBM-bound y passes do not.  The
// swap pairs outputs r and r ^ 1, so the radix R must be even.
template <int NS, int NP, int R>
__device__ __forceinline__ bool store_swap(int j) {
  return NS == 1 && NP == 4 && R % 2 == 0 && (j & 1);
}

// The same pass over pairs of adjacent lines of the Blocked layout (BW even): the two lines
// share their element addresses' 16-byte words, so every shared-memory access is a
// float4 (half the instructions) and every twiddle serves both lines.
template <int L, int R, int NS, int NL, int BW, int NT, bool INV, class EPI = NoEpi, bool BANKS = false>
__device__ __forceinline__ void stockham_pass_pairs(float2* s, const float2* __restrict__ tw, int tws,
                                                    const EPI& epi = EPI()) {
  static_assert(BW % 2 == 0 && NL % 2 == 0, "pairs of lines");
  using LAY = Blocked<L, BW>;
  constexpr int NB = L / R, NP = NL / 2;
  constexpr int NTASK = NP * NB;
  constexpr int TPT = (NTASK + NT - 1) / NT;
  float4* s4 = reinterpret_cast<float4*>(s);
  float2 a[TPT][R], b[TPT][R];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int task = threadIdx.x + t * NT;
    if ((NTASK % NT) == 0 || task < NTASK) {
      const int line = 2 * (task % NP), j = task / NP;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float4 q = s4[LAY::at(j + r * NB, line) >> 1];
        a[t][r] = make_float2(q.x, q.y);
        b[t][r] = make_float2(q.z, q.w);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int task = threadIdx.x + t * NT;
    if ((NTASK % NT) == 0 || task < NTASK) {
      const int line = 2 * (task % NP), j = task / NP;
      const int k = j % NS;
      if (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          float2 w = __ldg(&tw[(r * k * (L / (NS * R))) * tws]);
          if (INV) w.y = -w.y;
          a[t][r] = cmul(a[t][r], w);
          b[t][r] = cmul(b[t][r], w);
        }
      }
      DFT<R, INV>::run(a[t]);
      DFT<R, INV>::run(b[t]);
      const int base = (j - k) * R + k;
      // stride-1 stores of 4 pairs per j: the 8 lanes of a quarter-warp hold two j whose
      // outputs fall in the same banks; odd j store in the order r ^ 1 (other banks)
      const bool sw = BANKS && store_swap<NS, NP, R>(j);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int e = base + (sw ? r ^ 1 : r) * NS;
        const float2 av = sw ? a[t][r ^ 1] : a[t][r], bv = sw ? b[t][r ^ 1] : b[t][r];
        const float2 x = epi(av, e, line), y = epi(bv, e, line + 1);
        s4[LAY::at(e, line) >> 1] = make_float4(x.x, x.y, y.x, y.y);
      }
    }
  }
  __syncthreads();
}

template <int L, int P, int NS, int NL, int BW, int NT, bool INV, class EPI = NoEpi>
__device__ __forceinline__ void fft_passes_pairs(float2* s, const float2* __restrict__ tw, int tws,
                                                 const EPI& epi = EPI()) {
  if constexpr (P < Plan<L>::np) {
    constexpr int R = Plan<L>::r[P];
    if constexpr (P + 1 == Plan<L>::np) {
      stockham_pass_pairs<L, R, NS, NL, BW, NT, INV, EPI>(s, tw, tws, epi);
    } else {
      stockham_pass_pairs<L, R, NS, NL, BW, NT, INV>(s, tw, tws);
      fft_passes_pairs<L, P + 1, NS * R, NL, BW, NT, INV, EPI>(s, tw, tws, epi);
    }
  }
}

// ---------------------------------------------------------------------------------
// Forward transform, a pointwise map, inverse transform (the z pass of the Poisson solve).
//
// The last forward pass (radix R, stride NS = L / R) leaves in each thread the R outputs
// j + r L / R of one line (or pair of lines): exactly the inputs of the first pass of an
// inverse transform whose first radix is also R.  The inverse therefore runs the plan in
// reverse order (its first radix is the forward's last), and the two passes meet in
// registers -- the map is applied between them -- instead of through shared memory: one
// shared-memory round trip and two barriers fewer per transform pair.
// ---------------------------------------------------------------------------------
template <int L, int P, bool REV>
__host__ __device__ constexpr int plan_radix() {
  return REV ? Plan<L>::r[Plan<L>::np - 1 - P] : Plan<L>::r[P];
}

// Passes P .. PEND-1 of the plan (reversed with REV), entered with stride NS.
template <int L, int P, int PEND, int NS, int NL, int BW, int NT, bool INV, bool REV>
__device__ __forceinline__ void passes_span(float2* s, const float2* __restrict__ tw, int tws) {
  if constexpr (P < PEND) {
    constexpr int R = plan_radix<L, P, REV>();
    if constexpr (blocked_pairs(L))
      stockham_pass_pairs<L, R, NS, NL, BW, NT, INV, NoEpi, true>(s, tw, tws);
    else
      stockham_pass<L, R, NS, NL, Blocked<L, BW>, NT, INV>(s, tw, tws);
    passes_span<L, P + 1, PEND, NS * R, NL, BW, NT, INV, REV>(s, tw, tws);
  }
}

// The turn: last forward pass, `epi` on each output (element e of line), first inverse pass.
template <int L, int R, int NL, int BW, int NT, class EPI>
__device__ __forceinline__ void stockham_turn(float2* s, const float2* __restrict__ tw, int tws, const EPI& epi) {
  using LAY = Blocked<L, BW>;
  constexpr int NS = L / R;  // forward stride of the last pass == the inverse's block count
  constexpr bool PAIRS = blocked_pairs(L);
  constexpr int NG = PAIRS ? NL / 2 : NL;  // line groups: pairs of lines, or lines
  constexpr int NTASK = NG * NS;
  constexpr int TPT = (NTASK + NT - 1) / NT;
  float4* s4 = reinterpret_cast<float4*>(s);
  float2 a[TPT][R], b[TPT][R];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int task = threadIdx.x + t * NT;
    if ((NTASK % NT) == 0 || task < NTASK) {
      const int line = PAIRS ? 2 * (task % NG) : task % NG, j = task / NG;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if constexpr (PAIRS) {
          const float4 q = s4[LAY::at(j + r * NS, line) >> 1];
          a[t][r] = make_float2(q.x, q.y);
          b[t][r] = make_float2(q.z, q.w);
        } else {
          a[t][r] = s[LAY::at(j + r * NS, line)];
        }
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int task = threadIdx.x + t * NT;
    if ((NTASK % NT) == 0 || task < NTASK) {
      const int line = PAIRS ? 2 * (task % NG) : task % NG, j = task / NG;
      // forward: k = j (j < NS); the twiddle index r k L / (NS R) = r k
      if (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const float2 w = __ldg(&tw[(r * j) * tws]);
          a[t][r] = cmul(a[t][r], w);
          if constexpr (PAIRS) b[t][r] = cmul(b[t][r], w);
        }
      }
      DFT<R, false>::run(a[t]);
      if constexpr (PAIRS) DFT<R, false>::run(b[t]);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        a[t][r] = epi(a[t][r], j + r * NS, line);
        if constexpr (PAIRS) b[t][r] = epi(b[t][r], j + r * NS, line + 1);
      }
      // inverse, first pass (stride 1: no twiddles), outputs j R + r
      DFT<R, true>::run(a[t]);
      if constexpr (PAIRS) DFT<R, true>::run(b[t]);
      const bool sw = PAIRS && store_swap<1, NG, R>(j);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int rr = sw ? r ^ 1 : r;
        if constexpr (PAIRS) {
          const float2 av = sw ? a[t][r ^ 1] : a[t][r], bv = sw ? b[t][r ^ 1] : b[t][r];
          s4[LAY::at(j * R + rr, line) >> 1] = make_float4(av.x, av.y, bv.x, bv.y);
        } else {
          s[LAY::at(j * R + r, line)] = a[t][r];
        }
      }
    }
  }
  __syncthreads();
}

// Unnormalised forward DFT of NL lines (Blocked layout), `epi` on every spectral value
// (element j of line), unnormalised inverse DFT.  Entered by all NT threads after a
// __syncthreads(); returns synchronised.
template <int L, int NL, int BW, int NT, class EPI>
__device__ __forceinline__ void fft_lines_blocked_turn(float2* s, const float2* __restrict__ tw, int tws,
                                                       const EPI& epi) {
  constexpr int NPL = Plan<L>::np, RL = Plan<L>::r[NPL - 1];
  passes_span<L, 0, NPL - 1, 1, NL, BW, NT, false, false>(s, tw, tws);
  stockham_turn<L, RL, NL, BW, NT>(s, tw, tws, epi);
  passes_span<L, 1, NPL, RL, NL, BW, NT, true, true>(s, tw, tws);
}

// Unnormalised DFT of NL interleaved lines of length L held in shared memory.
// Must be entered by all NT threads after a __syncthreads(); returns synchronised.
template <int L, int NL, int LS, int NT, bool INV>
__device__ __forceinline__ void fft_lines(float2* s, const float2* __restrict__ tw, int tws) {
  fft_passes<L, 0, 1, NL, Interleaved<LS>, NT, INV>(s, tw, tws);
}

// Same on NL lines stored in blocks of BW lines (Blocked layout); `epi` maps every output
// value (element j of line) as the last pass stores it.
template <int L, int NL, int BW, int NT, bool INV, class EPI = NoEpi>
__device__ __forceinline__ void fft_lines_blocked(float2* s, const float2* __restrict__ tw, int tws,
                                                  const EPI& epi = EPI()) {
  if constexpr (blocked_pairs(L))
    fft_passes_pairs<L, 0, 1, NL, BW, NT, INV, EPI>(s, tw, tws, epi);
  else
    fft_passes<L, 0, 1, NL, Blocked<L, BW>, NT, INV, EPI>(s, tw, tws, epi);
}

}  // namespace pm
