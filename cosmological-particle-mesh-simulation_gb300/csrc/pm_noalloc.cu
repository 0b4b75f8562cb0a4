// pm_density_noalloc: the CIC deposit for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc at all:
// * hosts whose device memory is carved up up front by a pool or an arena (a framework's
//   caching allocator, a fixed budget per tenant): a library that allocates on its own
//   either fails there or breaks the host's accounting;
// * latency-critical loops, where an allocation and the device-wide synchronisation that
//   cudaMalloc / cudaFree can imply are not acceptable;
// * plugin hosts that hand every buffer to their plugins and forbid them to allocate.
// For them this entry point keeps every piece of scratch memory it needs -- the
// simulation descriptor, the work table, the sort's key/value buffers and histograms,
// the x-row starts -- in one file-scope static device array of fixed size.  Every GPU
// that loads the library holds that array until the process exits.
//
// Limits: at most NOALLOC_MAX_PARTICLES particles and grids of at most NOALLOC_MAX_N
// cells per side.  Larger requests are rejected with PM_ERR_ARG; pm_density, which
// allocates, has no such limit.
//
// The first call on a device does a one-time set-up with that device current: it looks up
// the array's device address (cudaGetSymbolAddress) and sets the kernels' attributes.
// The set-up is thread-safe (one lock per process).  Make that first call before any
// stream capture.
//
// The array is shared by every call: two calls whose work overlaps on the GPU (different
// streams, or different host threads, without ordering between them) race on it.  Each
// call writes all the scratch it reads before reading it -- the descriptor and the work
// table come from a kernel that receives them as arguments, which also clears the device
// check word -- so one call never sees stale data from the one before.
#include "pm_host.cuh"

using namespace pm;

namespace {

constexpr long long NOALLOC_MAX_PARTICLES = 1ll << 18;  // 262,144 particles (64^3)
constexpr int NOALLOC_MAX_N = 128;                      // grid cells per side
constexpr long long NOALLOC_MAX_ROWS = (long long)NOALLOC_MAX_N * NOALLOC_MAX_N;
constexpr int NOALLOC_MAX_BLOCKS = (int)((NOALLOC_MAX_PARTICLES + SORT_TILE - 1) / SORT_TILE);

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
std::atomic<NoAllocScratch*> g_scratch_ptr[PM_MAX_DEVICES];
std::mutex g_setup_lock;

int setup(int device, NoAllocScratch** out) {
  if (device < 0 || device >= PM_MAX_DEVICES) return PM_ERR_ARG;
  NoAllocScratch* p = g_scratch_ptr[device].load(std::memory_order_acquire);
  if (!p) {
    std::lock_guard<std::mutex> g(g_setup_lock);
    p = g_scratch_ptr[device].load(std::memory_order_relaxed);
    if (!p) {
      void* a = nullptr;
      if (cudaGetSymbolAddress(&a, g_noalloc_scratch) != cudaSuccess || !a) return PM_ERR_CUDA;
      if (deposit_prepare() != cudaSuccess || sort_prepare() != cudaSuccess) return PM_ERR_CUDA;
      p = static_cast<NoAllocScratch*>(a);
      g_scratch_ptr[device].store(p, std::memory_order_release);
    }
  }
  *out = p;
  return PM_OK;
}

// Writes the call's descriptor and work table into the scratch and clears its check word.
// They arrive as kernel arguments, which the launch copies: nothing is read from host
// memory after this call has returned.
__global__ void k_noalloc_begin(NoAllocScratch* s, Sim sim, int key_units, int dep_units) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    s->sim = sim;
    s->prefix[0] = 0;
    s->prefix[1] = key_units;
    s->prefix[2] = 0;
    s->prefix[3] = dep_units;
    s->err = 0;
  }
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

  Sim d{};
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
  k_noalloc_begin<<<1, 32, 0, st>>>(s, d, key_units, dep_units);
  if (cudaGetLastError() != cudaSuccess) return PM_ERR_CUDA;

  Parts p{};
  p.x = const_cast<float*>(positions);
  p.y = p.x + np;
  p.z = p.x + 2 * np;
  Work wk{s->prefix + 0, 1, key_units};
  Work wd{s->prefix + 2, 1, dep_units};
  const int sms = device_sms();
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
