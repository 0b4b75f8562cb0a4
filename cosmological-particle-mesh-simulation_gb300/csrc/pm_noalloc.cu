// pm_density_noalloc: the CIC deposit for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc at all:
// * code that runs while a CUDA stream is being captured into a graph (allocation is not
//   a capturable operation);
// * hosts whose device memory is carved up by a pool or arena up front, where a library
//   that allocates on its own breaks the budget;
// * latency-critical loops where an allocation (and the device synchronisation that
//   cudaMalloc/cudaFree can imply) is not acceptable.
// For them this entry point keeps every piece of scratch memory it needs -- the
// simulation descriptor, the work table, the sort's key/value buffers and histograms,
// the x-row starts -- in one file-scope static device array of fixed size.  Every GPU
// that loads the library holds that array until the process exits.
//
// Limits: at most NOALLOC_MAX_PARTICLES particles and grids of at most NOALLOC_MAX_N
// cells per side.  Larger requests are rejected with PM_ERR_ARG; pm_density, which
// allocates, has no such limit.
//
// The array is shared by every call: two calls whose work overlaps on the GPU (different
// streams, or different host threads, without ordering between them) race on it.  Each
// call writes all the scratch it reads before reading it, and clears the device check
// word it uses, so one call never sees stale data from the one before.
#include "pm_host.cuh"

using namespace pm;

namespace {

constexpr long long NOALLOC_MAX_PARTICLES = 1ll << 18;  // 262,144 particles (64^3)
constexpr int NOALLOC_MAX_N = 128;                      // grid cells per side
constexpr long long NOALLOC_MAX_ROWS = (long long)NOALLOC_MAX_N * NOALLOC_MAX_N;
constexpr int NOALLOC_MAX_BLOCKS = (int)((NOALLOC_MAX_PARTICLES + SORT_TILE - 1) / SORT_TILE);
constexpr int MAX_DEVICES = 64;

struct NoAllocScratch {
  Sim sim;
  int prefix[6];  // [keys, deposit] x {start, end}, then padding
  int err;
  int pad;
  unsigned keys[NOALLOC_MAX_PARTICLES];
  unsigned vals[NOALLOC_MAX_PARTICLES];
  unsigned keys_alt[NOALLOC_MAX_PARTICLES];
  unsigned vals_alt[NOALLOC_MAX_PARTICLES];
  unsigned hist[SORT_DIGIT_TOTALS * NOALLOC_MAX_BLOCKS];
  unsigned digit_tot[SORT_DIGIT_TOTALS];
  unsigned row_start[NOALLOC_MAX_ROWS + 1];
};

// The scratch: about 4.3 MB.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// Device address of g_noalloc_scratch per device, found once per device by the first call.
// In host code the array's name only stands for the symbol: its device address must come
// from cudaGetSymbolAddress with that device current.
NoAllocScratch* g_scratch_ptr[MAX_DEVICES] = {};

int setup(int device, NoAllocScratch** out) {
  if (device < 0 || device >= MAX_DEVICES) return PM_ERR_ARG;
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return PM_ERR_CUDA;
    if (deposit_prepare() != cudaSuccess) return PM_ERR_CUDA;
    g_scratch_ptr[device] = static_cast<NoAllocScratch*>(p);
  }
  *out = g_scratch_ptr[device];
  return PM_OK;
}

}  // namespace

extern "C" int pm_density_noalloc(const float* positions, long long np, int n_cells, double mass, float* rho,
                                  void* stream) {
  if (!positions || !rho) return PM_ERR_ARG;
  if (np <= 0 || np > NOALLOC_MAX_PARTICLES) return PM_ERR_ARG;
  if (n_cells > NOALLOC_MAX_N || !grid_supported(n_cells)) return PM_ERR_ARG;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return PM_ERR_CUDA;
  NoAllocScratch* s = nullptr;
  if (int r = setup(device, &s)) return r;
  cudaStream_t st = (cudaStream_t)stream;

  struct {
    Sim sim;
    int prefix[6];
  } host{};
  Sim& d = host.sim;
  d.n = n_cells;
  d.pitch = spec_pitch(n_cells);
  d.xbits = ceil_log2(n_cells);
  d.ty = TILE_Y;
  d.tz = TILE_Z;
  d.np = np;
  d.rho = rho;
  d.mass_scale = (float)(mass / (double)(1u << PM_FIX_BITS));
  const int key_units = (int)((np + 255) / 256);
  const int dep_units = (n_cells / TILE_Y) * (n_cells / TILE_Z);
  host.prefix[0] = 0;
  host.prefix[1] = key_units;
  host.prefix[2] = 0;
  host.prefix[3] = dep_units;
  if (cudaMemcpyAsync(s, &host, sizeof(host), cudaMemcpyHostToDevice, st) != cudaSuccess) return PM_ERR_CUDA;
  if (cudaMemsetAsync(&s->err, 0, sizeof(int), st) != cudaSuccess) return PM_ERR_CUDA;

  Parts p{};
  p.x = const_cast<float*>(positions);
  p.y = p.x + np;
  p.z = p.x + 2 * np;
  Work wk{s->prefix + 0, 1, key_units};
  Work wd{s->prefix + 2, 1, dep_units};
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return PM_ERR_CUDA;
  if (launch_keys_abs(&s->sim, wk, p, s->keys, nullptr, &s->err, grid_for(key_units, sms, 16), st))
    return PM_ERR_CUDA;
  SortScratch ss;
  ss.keys_alt = s->keys_alt;
  ss.vals_alt = s->vals_alt;
  ss.hist = s->hist;
  ss.digit_tot = s->digit_tot;
  ss.capacity = NOALLOC_MAX_PARTICLES;
  ss.max_blocks = NOALLOC_MAX_BLOCKS;
  const long long nrows = (long long)n_cells * n_cells;
  bool alt = false;
  if (radix_sort(s->keys, s->vals, np, 0, ceil_log2(nrows) + d.xbits, true, ss, &alt, st)) return PM_ERR_CUDA;
  unsigned* perm = alt ? s->vals_alt : s->vals;
  unsigned* skeys = alt ? s->keys_alt : s->keys;
  if (launch_row_start(skeys, np, d.xbits, (unsigned)nrows, s->row_start, st)) return PM_ERR_CUDA;
  if (launch_deposit(&s->sim, wd, p, perm, s->row_start, POS_ABS, &s->err, grid_for(dep_units, sms, 3),
                     deposit_smem_bytes(n_cells, TILE_Y, TILE_Z), st))
    return PM_ERR_CUDA;
  return PM_OK;
}
