// C ABI: resident batch engine (pm_batch_*).
//
// Simulations are resident in HBM.  Particles of all simulations live in one set of
// structure-of-arrays buffers (double buffered), stored as float32 displacements from
// their Lagrangian lattice point plus the particle index; every step the kick writes
// the state back in the order of the step's cell-key sort, so that the next step reads
// it almost in order.  Simulation s owns the x-rows [row_base_s, row_base_s + N_s^2) of the
// common key space and, in the sorted order (and so in the state a step writes), the range
// [part_off_s, part_off_s + np_s), in the same order, so one counting sort over the rows
// serves the whole batch.  Every phase is one launch over all simulations (the spectral
// phases: one per distinct grid size).  A step is captured once into a CUDA graph per plan
// and replayed; the scale factor and the step coefficients advance on the device.
//
// Admission and retirement do not drain the device.  A new simulation is converted into the
// free slots after the last one.  A finished one has its final state extracted on the step
// stream (an event marks its completion) and simply leaves the plan: its slots hold no keys
// (0xffffffff, skipped by the sort), so the next step's sort and kick write the survivors
// back compactly -- no copy of the resident state.  Grids of retired simulations are kept
// for reuse (per grid size) instead of being freed, since cudaFree synchronises the device.
#include <algorithm>
#include <chrono>
#include <cstddef>
#include <map>
#include <memory>

#include "pm_host.cuh"

using namespace pm;

namespace {

struct SimRec {
  int id = 0;
  pm_config cfg{};
  int n = 0, np1 = 0;
  long long np = 0;
  int nsteps = 0, done = 0;
  double a = 0.0, da = 0.0;
  bool resident = false;  // particles in the batch arrays
  DBuf grid, spec, rho;   // potential (and density unless keep_density), spectrum, density
  DBuf fin_pos, fin_vel;  // final state once retired (absolute, particle order)
  cudaEvent_t fin_ev = nullptr;  // recorded after the final state's extraction
  CUtensorMap maps[2];           // y- and z-pass tensor maps of its spectrum (encoded at admission)
  long long part_off = 0;  // offset in the sorted order (compact)
  long long in_off = 0;    // slot offset in the state the next step reads
  unsigned row_base = 0;
};

enum Phase { PH_KEYS = 0, PH_DEP, PH_KICK, PH_FIXED };

// Schedule of the phases of one grid size, chosen by the autotuner (autotune below).  Every
// choice leaves every result bit-identical: the deposit's integer sums do not depend on which
// tiles run when or where, the fused and the separate deposit convert the same sums, and the
// persistent kernels compute each work unit the same way whatever their grid.
enum DepMode : int { DEP_FUSED_DENSE_FIRST = 0, DEP_FUSED_INDEX = 1, DEP_SEPARATE = 2 };
struct Shape {
  int dep = DEP_FUSED_DENSE_FIRST;  // deposit of the sizes that can fuse it with the x R2C
  int dep_cps = 0;                  // fused deposit CTAs per SM (0: as many as fit)
  int x_cps = 8;                    // CTAs per SM of the x passes' row transforms
};

struct Plan {
  int nsims = 0;
  long long ptot = 0;
  unsigned rows = 0;
  int xbits = 0, bits = 0;
  std::vector<int> sizes;  // distinct grid sizes
  int fixed_total[PH_FIXED]{};
  std::vector<int> x_total, line_total;  // per distinct size
  std::vector<int> single;               // per distinct size: the only simulation of that size, or -1
  std::vector<int> fused, fdep_total;    // per distinct size: deposit fused with the x R2C, its tiles
  std::vector<Shape> shape;              // per distinct size: the tuned schedule
  int kick_cps = 16;                     // kick CTAs per SM
  int max_dep_smem = 0;
  int max_n = 0;
  long long sort_n = 0;  // slots the next step's sort reads (> ptot right after a retirement)
};

// x y z vx vy vz id (4 bytes a particle each) and the cell record (16 bytes)
const int kStateArrays = 8;
constexpr size_t state_elem_bytes(int k) { return k == 7 ? 16 : 4; }
constexpr size_t kStateBytes = 7 * 4 + 16;  // per particle

// Schedules found by the autotuner, for the whole process: per (grid size, volume class of the
// size's deposit tiles in the batch), and the kick's per volume class of its work units; a
// class spans a factor 8 of work, so that a serving mix whose simulations come and go meets
// few new classes.
std::mutex g_tune_lock;
std::map<std::pair<int, int>, Shape> g_shapes;
std::map<int, int> g_kick_cps;

int ilog2(long long v) {
  int b = 0;
  while (v > 1) { v >>= 1; ++b; }
  return b;
}

int volume_class(long long units) { return ilog2(units > 1 ? units : 1) / 3; }

}  // namespace

struct pm_batch {
  int device = 0, sms = 1;
  size_t cap = 0;
  std::vector<std::unique_ptr<SimRec>> sims;  // resident, in slot order
  std::vector<std::unique_ptr<SimRec>> retired;
  std::map<int, std::unique_ptr<Tables>> tables;
  std::map<long long, std::unique_ptr<Lattice>> lattices;
  int next_id = 1;
  // particle state, two copies; arrays x y z vx vy vz id and the cell record cell fx fy fz
  DBuf st[2][kStateArrays];
  long long pcap = 0;
  int cur = 0;
  SortBufs sort;
  DBuf row_start, d_sims, d_prefix, d_err, d_maps;
  DBuf tile_next;   // per distinct size: tile counter of the fused deposit, 2 words of ordering scratch
  DBuf tile_order;  // per distinct size (at its tile prefix): the fused deposit's tiles, dense first
  DBuf d_one;       // descriptor + work table of a one-simulation deposit (pm_batch_density)
  DBuf row_count, row_cursor, scan_sums;  // counting sort of the row keys
  Plan plan;
  bool dirty = true, keys_valid = false;
  bool graphs = true;
  bool autotune = true;     // tune the schedule of new plans (see autotune)
  bool tuned = false;       // the current plan's schedule is settled
  int plan_steps = 0;       // steps run since the plan was built
  bool sparse = false;      // the state the next step reads has empty slots (after a retirement)
  long long in_total = 0;   // slots of that state
  // Executable graphs of a step from state 0 and from state 1.  A new plan marks them stale:
  // the next capture updates them in place (cudaGraphExecUpdate, no instantiation) and only
  // a change of the graph's shape instantiates a new one -- destroying an executable graph
  // synchronises with the device, which stalled the serving loop at every re-plan.
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  bool gstale[2] = {false, false};
  cudaStream_t own = nullptr;     // used when the caller passes the legacy stream (captures need one)
  cudaStream_t admit = nullptr;   // admission conversions
  cudaEvent_t last_step = nullptr;  // recorded after the last enqueued step
  // The spectral chains of the distinct grid sizes (fused deposit, y, z, y^-1, x C2R) touch
  // disjoint grids: a step runs them on one stream per size, forked after the sort and joined
  // before the kick, so that the kernels of one size fill the tails of another's.
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> side_ev;
  cudaEvent_t fork_ev = nullptr;
  // grids (potential, spectrum) of retired simulations by grid size, and final-state
  // buffers by particle count, kept for reuse
  std::map<int, std::vector<std::pair<DBuf, DBuf>>> grid_pool;
  std::map<long long, std::vector<std::pair<DBuf, DBuf>>> fin_pool;
  DBuf stage_pos, stage_vel;  // admission staging of host initial conditions
  DBuf adm_count, adm_start, adm_cursor, adm_sums;  // row counting sort of an admission
  // pinned host staging of the plan's uploads (two, used in turn; an event marks when the
  // device has read one), so that re-planning never waits for enqueued work
  void* plan_host[2] = {nullptr, nullptr};
  size_t plan_host_bytes[2] = {0, 0};
  cudaEvent_t plan_ev[2] = {nullptr, nullptr};
  int plan_turn = 0;
  // host seconds: admission, planning, graph capture, retirement, tuning, and the part of
  // planning spent waiting for the device to release a staging buffer (not in planning's)
  double host_s[6] = {0, 0, 0, 0, 0, 0};
  std::string err;
};

namespace {

int bfail(pm_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}

int bcuda(pm_batch* b, cudaError_t e, const char* where) {
  return bfail(b, e == cudaErrorMemoryAllocation ? PM_ERR_OOM : PM_ERR_CUDA,
               std::string(where) + ": " + cudaGetErrorString(e));
}

#define PB_CK(call, where)                                  \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return bcuda(b, e_, where);      \
  } while (0)

Parts state(pm_batch* b, int which) {
  Parts p;
  p.x = b->st[which][0].as<float>();
  p.y = b->st[which][1].as<float>();
  p.z = b->st[which][2].as<float>();
  p.vx = b->st[which][3].as<float>();
  p.vy = b->st[which][4].as<float>();
  p.vz = b->st[which][5].as<float>();
  p.id = b->st[which][6].as<unsigned>();
  p.rec = b->st[which][7].as<uint4>();
  return p;
}

long long resident_particles(pm_batch* b) {
  long long t = 0;
  for (auto& s : b->sims) t += s->np;
  return t;
}

size_t footprint(const pm_config& c) {
  const size_t n = c.n_cells;
  const size_t np = (size_t)c.n_parts * c.n_parts * c.n_parts;
  size_t f = n * n * n * sizeof(float);                          // potential / density
  if (c.flags & PM_FLAG_KEEP_DENSITY) f += n * n * n * sizeof(float);
  f += n * n * (size_t)spec_pitch((int)n) * sizeof(float2);      // spectrum
  f += np * (2 * kStateBytes + 4 * 4);                           // state x2, keys/vals x2
  f += np * 6 * sizeof(float);                                   // final state
  f += 3 * n * n * sizeof(unsigned) + 4096;                      // row starts, counts, cursors, tables
  return f;
}

size_t used_bytes(pm_batch* b) {
  size_t u = 0;
  for (auto& s : b->sims) u += footprint(s->cfg);
  for (auto& s : b->retired) u += (size_t)s->np * 6 * sizeof(float);
  return u;
}

// Device bytes held for reuse (grids and final-state buffers of simulations that left).
size_t pooled_bytes(pm_batch* b) {
  size_t u = 0;
  for (auto& e : b->grid_pool)
    for (auto& g : e.second) u += g.first.bytes + g.second.bytes;
  for (auto& e : b->fin_pool)
    for (auto& g : e.second) u += g.first.bytes + g.second.bytes;
  return u;
}

// Frees pooled buffers until `need` more bytes fit under the cap next to what is in use
// (cudaFree synchronises the device: only when memory is short).
void trim_pools(pm_batch* b, size_t need) {
  if (!b->cap) return;
  auto over = [&]() { return used_bytes(b) + pooled_bytes(b) + need > b->cap; };
  for (auto& e : b->grid_pool)
    while (over() && !e.second.empty()) {
      e.second.back().first.release();
      e.second.back().second.release();
      e.second.pop_back();
    }
  for (auto& e : b->fin_pool)
    while (over() && !e.second.empty()) {
      e.second.back().first.release();
      e.second.back().second.release();
      e.second.pop_back();
    }
}

// Accumulates the host time of a scope into one of pm_batch::host_s.
struct HostTimer {
  double& acc;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  explicit HostTimer(double& a) : acc(a) {}
  ~HostTimer() { acc += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

// Room for `need` slots; the current state's first in_total slots are kept (rare: capacity
// grows by half each time, after the device has finished all enqueued work).
cudaError_t grow_state(pm_batch* b, long long need) {
  if (need <= b->pcap) return cudaSuccess;
  long long cap = std::max(need, b->pcap + b->pcap / 2);
  const long long keep = b->in_total;
  cudaError_t e = cudaDeviceSynchronize();
  if (e) return e;
  for (int w = 0; w < 2; ++w) {
    for (int k = 0; k < kStateArrays; ++k) {
      DBuf nb;
      e = nb.ensure((size_t)cap * state_elem_bytes(k));
      if (e) return e;
      if (w == b->cur && keep > 0 && b->st[w][k].p) {
        e = cudaMemcpy(nb.p, b->st[w][k].p, (size_t)keep * state_elem_bytes(k), cudaMemcpyDeviceToDevice);
        if (e) return e;
      }
      b->st[w][k].release();
      b->st[w][k] = nb;
    }
  }
  b->pcap = cap;
  b->keys_valid = false;  // the sort buffers are reallocated
  return b->sort.ensure(cap);
}

// The step graphs no longer match the plan: marked stale (updated at their next capture), or
// destroyed with `destroy`.  Returns the host seconds it took (counted as graph work:
// capture, instantiation, update and destruction).
double drop_graphs(pm_batch* b, bool destroy = false) {
  double s = 0;
  {
    HostTimer timer(s);
    for (int c = 0; c < 2; ++c) {
      b->gstale[c] = b->gexec[c] != nullptr;
      if (destroy && b->gexec[c]) {
        cudaGraphExecDestroy(b->gexec[c]);
        b->gexec[c] = nullptr;
        b->gstale[c] = false;
      }
    }
  }
  b->host_s[2] += s;
  return s;
}

Tables* tables_for(pm_batch* b, int n) {
  auto& t = b->tables[n];
  if (!t) t.reset(new Tables());
  return t.get();
}

Lattice* lattice_for(pm_batch* b, int np1, int n) {
  auto& l = b->lattices[((long long)np1 << 32) | (unsigned)n];
  if (!l) l.reset(new Lattice());
  return l.get();
}

// Build the plan (Sim descriptors, work prefixes) for the resident simulations.
int build_plan(pm_batch* b, cudaStream_t st) {
  HostTimer timer(b->host_s[1]);
  Plan& P = b->plan;
  P = Plan();
  P.nsims = (int)b->sims.size();
  if (P.nsims == 0) return PM_OK;
  // Resident keys are the global x-row number alone: the deposit needs particles grouped by
  // row, not ordered inside a row (its integer sums do not depend on the order), so a
  // counting sort over the batch's rows (< 2^32) groups them.
  P.xbits = 0;
  std::vector<Sim> hs(P.nsims);
  const int S = P.nsims;
  std::vector<int> pre;  // [phase][S+1]
  long long off = 0;
  unsigned rows = 0;
  for (int i = 0; i < S; ++i) {
    SimRec& r = *b->sims[i];
    r.part_off = off;
    r.row_base = rows;
    off += r.np;
    if ((long long)rows + (long long)r.n * r.n >= (1ll << 32)) return bfail(b, PM_ERR_ADMIT, "too many x-rows");
    rows += (unsigned)((long long)r.n * r.n);
    if (std::find(P.sizes.begin(), P.sizes.end(), r.n) == P.sizes.end()) P.sizes.push_back(r.n);
  }
  P.ptot = off;
  P.rows = rows;
  P.sort_n = b->sparse ? b->in_total : P.ptot;
  P.bits = ceil_log2((long long)rows) + P.xbits;  // keys are < rows
  if (P.bits > 32) return bfail(b, PM_ERR_ADMIT, "batch key space exceeds 32 bits");
  std::sort(P.sizes.begin(), P.sizes.end());
  const int nph = PH_FIXED + 3 * (int)P.sizes.size();
  for (int n : P.sizes) {
    bool f = deposit_r2c_supported(n);
    for (auto& sp : b->sims)
      if (sp->n == n && (sp->cfg.flags & PM_FLAG_KEEP_DENSITY)) f = false;
    P.fused.push_back(f ? 1 : 0);
  }
  pre.assign((size_t)nph * (S + 1), 0);
  auto at = [&](int ph, int s) -> int& { return pre[(size_t)ph * (S + 1) + s]; };
  for (int i = 0; i < S; ++i) {
    SimRec& r = *b->sims[i];
    Sim& d = hs[i];
    d = Sim();
    d.n = r.n;
    d.pitch = spec_pitch(r.n);
    d.np1 = r.np1;
    d.xbits = P.xbits;
    d.ty = TILE_Y;
    d.tz = TILE_Z;
    d.np = r.np;
    d.part_off = r.part_off;
    d.slot_off = r.in_off;
    d.row_base = r.row_base;
    d.phi = r.grid.as<float>();
    d.rho = (r.cfg.flags & PM_FLAG_KEEP_DENSITY) ? r.rho.as<float>() : r.grid.as<float>();
    d.spec = r.spec.as<float2>();
    Tables* t = tables_for(b, r.n);
    d.s2 = t->s2.as<float>();
    d.tw = t->tw.as<float2>();
    Lattice* l = lattice_for(b, r.np1, r.n);
    d.q_int = l->qi.as<int>();
    d.q_frac = l->qf.as<float>();
    d.q_step = r.np1 > 0 && r.n % r.np1 == 0 ? r.n / r.np1 : 0;
    d.mass_scale = (float)(std::pow((double)r.n / r.np1, 3) / (double)(1u << PM_FIX_BITS));
    d.a = r.a;
    d.da = r.da;
    d.om = r.cfg.omega_m0;
    d.ol = r.cfg.omega_lambda0;
    d.ok = r.cfg.omega_k0;
    d.h0 = r.cfg.h0;
    d.step = r.done;
    d.nsteps = r.nsteps;
    d.active = 1;
    d.fix_f = (r.cfg.flags & PM_FLAG_FIX_COSMO_F) ? 1 : 0;
    const int tiles = (r.n / TILE_Y) * (r.n / TILE_Z);
    bool fused_here = false;
    for (size_t g = 0; g < P.sizes.size(); ++g)
      if (P.sizes[g] == r.n) fused_here = P.fused[g] != 0;
    at(PH_KEYS, i + 1) = at(PH_KEYS, i) + (int)((r.np + 255) / 256);
    at(PH_DEP, i + 1) = at(PH_DEP, i) + (fused_here ? 0 : tiles);
    at(PH_KICK, i + 1) = at(PH_KICK, i) + (int)((r.np + KICK_UNIT - 1) / KICK_UNIT);
    P.max_n = std::max(P.max_n, r.n);
    for (size_t g = 0; g < P.sizes.size(); ++g) {
      const bool mine = P.sizes[g] == r.n;
      const int phx = PH_FIXED + 3 * (int)g, phl = phx + 1, phd = phx + 2;
      at(phx, i + 1) = at(phx, i) + (mine ? (int)spectral_units(SPEC_X_R2C, r.n) : 0);
      at(phl, i + 1) = at(phl, i) + (mine ? (int)spectral_units(SPEC_Y_FWD, r.n) : 0);
      at(phd, i + 1) = at(phd, i) + (mine && P.fused[g] ? tiles : 0);
    }
    P.max_dep_smem = std::max(P.max_dep_smem, (int)deposit_smem_bytes(r.n, TILE_Y, TILE_Z));
  }
  for (int ph = 0; ph < PH_FIXED; ++ph) P.fixed_total[ph] = at(ph, S);
  for (size_t g = 0; g < P.sizes.size(); ++g) {
    P.x_total.push_back(at(PH_FIXED + 3 * (int)g, S));
    P.line_total.push_back(at(PH_FIXED + 3 * (int)g + 1, S));
    P.fdep_total.push_back(at(PH_FIXED + 3 * (int)g + 2, S));
    int only = -1, count = 0;
    for (int i = 0; i < S; ++i)
      if (b->sims[i]->n == P.sizes[g]) { only = i; ++count; }
    P.single.push_back(count == 1 ? only : -1);
  }
  PB_CK(b->d_maps.ensure_geo(sizeof(CUtensorMap) * 2 * (size_t)S), "alloc maps");
  PB_CK(b->d_sims.ensure_geo(sizeof(Sim) * S), "alloc sims");
  PB_CK(b->d_prefix.ensure_geo(sizeof(int) * pre.size()), "alloc prefix");
  PB_CK(b->row_start.ensure_geo(sizeof(unsigned) * ((size_t)rows + 1)), "alloc rows");
  PB_CK(b->row_count.ensure_geo(sizeof(unsigned) * (size_t)rows), "alloc rows");
  {
    size_t tiles = 1;
    for (int t : P.fdep_total) tiles += (size_t)t;
    PB_CK(b->tile_order.ensure_geo(sizeof(unsigned) * tiles), "alloc tile order");
    PB_CK(b->tile_next.ensure_geo(4 * sizeof(unsigned) * P.sizes.size()), "alloc tile counters");
    while (b->side.size() < P.sizes.size()) {
      cudaStream_t s = nullptr;
      cudaEvent_t e = nullptr;
      PB_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
      if (cudaError_t ee = cudaEventCreateWithFlags(&e, cudaEventDisableTiming)) {
        cudaStreamDestroy(s);
        return bcuda(b, ee, "event");
      }
      b->side.push_back(s);
      b->side_ev.push_back(e);
    }
  }
  PB_CK(b->row_cursor.ensure_geo(sizeof(unsigned) * (size_t)rows), "alloc rows");
  PB_CK(b->scan_sums.ensure_geo(sizeof(unsigned) * row_sort_block_sums(rows)), "alloc rows");
  {  // tensor maps (for the TMA line passes), descriptors and work prefixes, through pinned staging
    const size_t mb = sizeof(CUtensorMap) * 2 * (size_t)S, sbytes = sizeof(Sim) * S, pbytes = sizeof(int) * pre.size();
    const size_t o_sims = (mb + 255) / 256 * 256, o_pre = o_sims + (sbytes + 255) / 256 * 256, total = o_pre + pbytes;
    const int t = b->plan_turn;
    if (!b->plan_ev[t]) PB_CK(cudaEventCreateWithFlags(&b->plan_ev[t], cudaEventDisableTiming), "event");
    else {  // its last uploads have been read
      double waited = 0;
      {
        HostTimer wt(waited);
        PB_CK(cudaEventSynchronize(b->plan_ev[t]), "staging");
      }
      b->host_s[1] -= waited;  // (the planning timer adds the whole scope)
      b->host_s[5] += waited;
    }
    if (b->plan_host_bytes[t] < total) {
      if (b->plan_host[t]) cudaFreeHost(b->plan_host[t]);
      b->plan_host[t] = nullptr;
      b->plan_host_bytes[t] = 0;
      // doubled, so that a batch whose simulation count creeps up reallocates rarely: each
      // cudaFreeHost synchronises the device, and the serving loop re-plans at every admission
      const size_t want = std::max(2 * total, (size_t)256 << 10);
      PB_CK(cudaMallocHost(&b->plan_host[t], want), "alloc staging");
      b->plan_host_bytes[t] = want;
    }
    char* h = static_cast<char*>(b->plan_host[t]);
    for (int i = 0; i < S; ++i) std::memcpy(h + sizeof(CUtensorMap) * 2 * i, b->sims[i]->maps, sizeof(CUtensorMap) * 2);
    std::memcpy(h + o_sims, hs.data(), sbytes);
    std::memcpy(h + o_pre, pre.data(), pbytes);
    PB_CK(cudaMemcpyAsync(b->d_maps.p, h, mb, cudaMemcpyHostToDevice, st), "upload maps");
    PB_CK(cudaMemcpyAsync(b->d_sims.p, h + o_sims, sbytes, cudaMemcpyHostToDevice, st), "upload sims");
    PB_CK(cudaMemcpyAsync(b->d_prefix.p, h + o_pre, pbytes, cudaMemcpyHostToDevice, st), "upload prefix");
    PB_CK(cudaEventRecord(b->plan_ev[t], st), "event");
    b->plan_turn = 1 - t;
  }
  PB_CK(launch_coef(b->d_sims.as<Sim>(), S, 0, st), "coef");
  // (the uploads are ordered on `st` after the steps already enqueued: pageable host memory is
  // staged before cudaMemcpyAsync returns, so no synchronisation is needed here)
  for (size_t g = 0; g < P.sizes.size(); ++g) {
    PB_CK(spectral_dispatch(SPEC_PREPARE, P.sizes[g], nullptr, Work(), 0, st), "prepare");
    if (P.fused[g])
      PB_CK(deposit_r2c_dispatch(P.sizes[g], nullptr, Work(), Parts(), nullptr, nullptr, POS_DISP, nullptr, nullptr,
                                 nullptr, 0, st),
            "prepare fused deposit");
  }
  PB_CK(deposit_prepare(), "prepare deposit");
  {  // the schedule: tuned values from the process-wide cache, defaults for the rest
    std::lock_guard<std::mutex> g(g_tune_lock);
    b->tuned = true;
    P.shape.assign(P.sizes.size(), Shape());
    for (size_t i = 0; i < P.sizes.size(); ++i) {
      const auto key = std::make_pair(P.sizes[i], volume_class(P.fdep_total[i] ? P.fdep_total[i] : P.x_total[i]));
      auto it = g_shapes.find(key);
      if (it != g_shapes.end()) P.shape[i] = it->second;
      else b->tuned = false;
      if (!P.fused[i]) P.shape[i].dep = DEP_SEPARATE;
    }
    auto kt = g_kick_cps.find(volume_class(P.fixed_total[PH_KICK]));
    if (kt != g_kick_cps.end()) P.kick_cps = kt->second;
    else b->tuned = false;
  }
  b->host_s[1] -= drop_graphs(b);  // (counted as graph work, not planning)
  b->dirty = false;
  b->plan_steps = 0;
  return PM_OK;
}

Work work_of(pm_batch* b, int ph, int total) {
  Work w;
  w.prefix = b->d_prefix.as<int>() + (size_t)ph * (b->plan.nsims + 1);
  w.nsims = b->plan.nsims;
  w.total = total;
  return w;
}

// Phases timed by pm_batch_profile, in launch order.
enum ProfPhase { PP_SORT = 0, PP_ROWS, PP_DEPOSIT, PP_X_R2C, PP_Y_FWD, PP_Z_GREEN, PP_Y_INV, PP_X_C2R, PP_KICK,
                 PP_COEF, PP_COUNT };

// The deposit of the simulations of distinct size g that can fuse it with the x R2C, on the
// schedule `sh` (a separate deposit leaves the x R2C to the spectral phase).
int enqueue_deposit(pm_batch* b, int g, const Shape& sh, Parts in, const unsigned* perm, cudaStream_t st) {
  const Plan& P = b->plan;
  const Sim* ds = b->d_sims.as<Sim>();
  int* err = b->d_err.as<int>();
  const int n = P.sizes[g], tot = P.fdep_total[g];
  const Work wg = work_of(b, PH_FIXED + 3 * g + 2, tot);
  // this size's tile counter and ordering scratch, and its part of the tile order
  unsigned* next = b->tile_next.as<unsigned>() + 4 * g;
  unsigned* order = b->tile_order.as<unsigned>();
  for (int i = 0; i < g; ++i) order += P.fdep_total[i];
  if (sh.dep == DEP_SEPARATE) {
    PB_CK(launch_deposit(ds, wg, in, perm, b->row_start.as<unsigned>(), POS_DISP, err, grid_for(tot, b->sms, 3),
                         deposit_smem_bytes(n, TILE_Y, TILE_Z), st),
          "deposit");
    return PM_OK;
  }
  if (sh.dep == DEP_FUSED_DENSE_FIRST)
    PB_CK(launch_tile_order(ds, wg, b->row_start.as<unsigned>(), order, next + 2, b->sms, st), "tile order");
  PB_CK(deposit_r2c_dispatch(n, ds, wg, in, perm, b->row_start.as<unsigned>(), POS_DISP, err, next,
                             sh.dep == DEP_FUSED_DENSE_FIRST ? order : nullptr,
                             grid_for(tot, b->sms, sh.dep_cps ? sh.dep_cps : deposit_r2c_ctas_per_sm(n)), st),
        "fused deposit");
  return PM_OK;
}

// Enqueue one step (state in b->st[cur] -> b->st[1 - cur]).  With `ev` (PP_COUNT + 1
// events) an event is recorded before the first phase and after every phase.
int enqueue_step(pm_batch* b, int cur, cudaStream_t st, cudaEvent_t* ev = nullptr) {
  Plan& P = b->plan;
  auto mark = [&](int i) -> cudaError_t { return ev ? cudaEventRecord(ev[i], st) : cudaSuccess; };
  PB_CK(mark(0), "event");
  const Sim* ds = b->d_sims.as<Sim>();
  int* err = b->d_err.as<int>();
  Parts in = state(b, cur), out = state(b, 1 - cur);
  // group the particles by x-row: row starts and the permutation to row order
  unsigned* perm = b->sort.vals.as<unsigned>();
  // (the row histogram of the keys was made by the previous kick, or by ensure_keys)
  PB_CK(row_counting_sort(b->sort.keys.as<unsigned>(), P.sort_n, P.rows, b->row_count.as<unsigned>(),
                          b->row_start.as<unsigned>(), b->row_cursor.as<unsigned>(), b->scan_sums.as<unsigned>(),
                          perm, err, b->sms, st, nullptr, true),
        "sort");
  PB_CK(mark(1 + PP_SORT), "event");
  PB_CK(mark(1 + PP_ROWS), "event");  // the row starts come out of the counting sort
  if (P.fixed_total[PH_DEP] > 0)
    PB_CK(launch_deposit(ds, work_of(b, PH_DEP, P.fixed_total[PH_DEP]), in, perm, b->row_start.as<unsigned>(),
                         POS_DISP, err, grid_for(P.fixed_total[PH_DEP], b->sms, 3), P.max_dep_smem, st),
          "deposit");
  const SpecKind order[5] = {SPEC_X_R2C, SPEC_Y_FWD, SPEC_Z_GREEN, SPEC_Y_INV, SPEC_X_C2R};
  auto spectral = [&](int o, int g, cudaStream_t s) -> int {
    const SpecKind k = order[o];
    if (k == SPEC_X_R2C && P.shape[g].dep != DEP_SEPARATE) return PM_OK;  // done by the fused deposit
    const bool xk = (k == SPEC_X_R2C || k == SPEC_X_C2R);
    const int ph = PH_FIXED + 3 * g + (xk ? 0 : 1);
    const int tot = xk ? P.x_total[g] : P.line_total[g];
    PB_CK(spectral_dispatch(k, P.sizes[g], ds, work_of(b, ph, tot),
                            xk ? grid_for(tot, b->sms, P.shape[g].x_cps) : grid_for(tot, b->sms, 8), s,
                            b->d_maps.as<CUtensorMap>(), err),
          "spectral");
    return PM_OK;
  };
  if (!ev && P.sizes.size() > 1 && b->side.size() >= P.sizes.size()) {
    // one stream per distinct size: deposit and transforms of that size in order, the sizes
    // side by side
    PB_CK(cudaEventRecord(b->fork_ev, st), "event");
    for (size_t g = 0; g < P.sizes.size(); ++g) {
      cudaStream_t s = b->side[g];
      PB_CK(cudaStreamWaitEvent(s, b->fork_ev, 0), "fork");
      if (P.fused[g])
        if (int r = enqueue_deposit(b, (int)g, P.shape[g], in, perm, s)) return r;
      for (int o = 0; o < 5; ++o)
        if (int r = spectral(o, (int)g, s)) return r;
      PB_CK(cudaEventRecord(b->side_ev[g], s), "event");
      PB_CK(cudaStreamWaitEvent(st, b->side_ev[g], 0), "join");
    }
  } else {
    // phase by phase (the profiled order: an event after every phase)
    for (size_t g = 0; g < P.sizes.size(); ++g)
      if (P.fused[g])
        if (int r = enqueue_deposit(b, (int)g, P.shape[g], in, perm, st)) return r;
    PB_CK(mark(1 + PP_DEPOSIT), "event");
    for (int o = 0; o < 5; ++o) {
      for (size_t g = 0; g < P.sizes.size(); ++g)
        if (int r = spectral(o, (int)g, st)) return r;
      PB_CK(mark(1 + PP_X_R2C + o), "event");
    }
  }
  // the kick writes the next keys and counts them per row for the next step's sort
  PB_CK(cudaMemsetAsync(b->row_count.p, 0, sizeof(unsigned) * (size_t)P.rows, st), "count reset");
  PB_CK(launch_kick(ds, work_of(b, PH_KICK, P.fixed_total[PH_KICK]), in, out, perm, b->sort.keys.as<unsigned>(),
                    POS_DISP, err, grid_for(P.fixed_total[PH_KICK], b->sms, P.kick_cps), st,
                    b->row_count.as<unsigned>()),
        "kick");
  PB_CK(mark(1 + PP_KICK), "event");
  PB_CK(launch_coef(b->d_sims.as<Sim>(), P.nsims, 1, st), "coef");
  PB_CK(mark(1 + PP_COEF), "event");
  return PM_OK;
}

// Kernel launches of one step for the current plan.
int launches_per_step(pm_batch* b) {
  const Plan& P = b->plan;
  // counting sort: 3 scan kernels and the scatter (the kick makes the histogram; the count
  // reset is a memset)
  int n = 4 + (P.fixed_total[PH_DEP] > 0 ? 1 : 0) + 5 * (int)P.sizes.size() + 1 + 1;
  // a fused size replaces its x R2C launch by the fused deposit (with a dense-first tile
  // order, one launch more); a separate one adds its deposit launch
  for (size_t g = 0; g < P.sizes.size(); ++g)
    if (P.fused[g]) n += P.shape[g].dep == DEP_FUSED_INDEX ? 0 : 1;
  return n;
}

int ensure_keys(pm_batch* b, cudaStream_t st) {
  if (b->keys_valid) return PM_OK;
  Plan& P = b->plan;
  // slots without a resident particle (left by retired simulations) hold no key
  PB_CK(cudaMemsetAsync(b->sort.keys.p, 0xff, sizeof(unsigned) * (size_t)P.sort_n, st), "clear keys");
  PB_CK(launch_keys_disp(b->d_sims.as<Sim>(), work_of(b, PH_KEYS, P.fixed_total[PH_KEYS]), state(b, b->cur),
                         b->sort.keys.as<unsigned>(), nullptr, b->d_err.as<int>(),
                         grid_for(P.fixed_total[PH_KEYS], b->sms, 16), st),
        "keys");
  PB_CK(row_histogram(b->sort.keys.as<unsigned>(), P.sort_n, P.rows, b->row_count.as<unsigned>(), b->d_err.as<int>(),
                      b->sms, st),
        "row histogram");
  b->keys_valid = true;
  return PM_OK;
}

// Steps a new plan runs (on the defaults or cached schedules) before it is tuned: the state of a
// newly admitted simulation is in particle order until its first step has sorted it, and its
// permutation reads are then scattered -- not the steady state that the timings must represent.
constexpr int TUNE_AFTER_STEPS = 2;

// Autotuner: for each grid size of the plan whose schedule is not in the process-wide cache,
// and for the kick, time the candidate schedules on the batch's own data (one warm-up launch,
// then the mean of three) and keep the fastest.  The candidates are the deposit modes (fused
// with dense-first tiles, or separate from the x R2C), the fused deposit's CTAs per SM, the x
// passes' CTAs per SM and the kick's.  (Fused tiles in index order is not a candidate: it can
// win on the even particle distribution of early steps, where it is timed, and then loses
// badly once particles cluster -- 1.01 against 0.72 ms at step 980 of the 256^3 / 512^3 run.)  Runs between steps: the trials write
// only buffers that the next step rewrites from scratch (spectra, grids, the next state, tile
// counters) or scratch (the kick's keys and histogram go to unused sort buffers), never the
// state the step reads or the histogram its sort consumes.
int autotune(pm_batch* b, cudaStream_t st) {
  Plan& P = b->plan;
  if (b->tuned || !b->autotune) return PM_OK;
  HostTimer timer(b->host_s[4]);
  const Sim* ds = b->d_sims.as<Sim>();
  int* err = b->d_err.as<int>();
  Parts in = state(b, b->cur), out = state(b, 1 - b->cur);
  unsigned* perm = b->sort.vals.as<unsigned>();
  // the row starts and permutation of the current keys (the step recomputes the same)
  PB_CK(row_counting_sort(b->sort.keys.as<unsigned>(), P.sort_n, P.rows, b->row_count.as<unsigned>(),
                          b->row_start.as<unsigned>(), b->row_cursor.as<unsigned>(), b->scan_sums.as<unsigned>(),
                          perm, err, b->sms, st, nullptr, true),
        "sort");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  PB_CK(cudaEventCreate(&e0), "event");
  PB_CK(cudaEventCreate(&e1), "event");
  int rc = PM_OK;
  // mean milliseconds of `launch` (a callable returning a PM status)
  auto time3 = [&](auto&& launch, float& ms) -> int {
    if (int r = launch()) return r;
    PB_CK(cudaEventRecord(e0, st), "event");
    for (int i = 0; i < 3; ++i)
      if (int r = launch()) return r;
    PB_CK(cudaEventRecord(e1, st), "event");
    PB_CK(cudaEventSynchronize(e1), "tune sync");
    PB_CK(cudaEventElapsedTime(&ms, e0, e1), "event");
    ms /= 3.f;
    return PM_OK;
  };
  std::vector<std::pair<std::pair<int, int>, Shape>> found;
  for (size_t g = 0; g < P.sizes.size() && !rc; ++g) {
    const int n = P.sizes[g];
    const auto key = std::make_pair(n, volume_class(P.fdep_total[g] ? P.fdep_total[g] : P.x_total[g]));
    {
      std::lock_guard<std::mutex> lk(g_tune_lock);
      if (g_shapes.count(key)) continue;
    }
    Shape best = P.shape[g];
    const Work wx = work_of(b, PH_FIXED + 3 * (int)g, P.x_total[g]);
    if (P.fused[g]) {  // deposit mode and grid (a separate deposit is timed with its x R2C)
      const int occ = deposit_r2c_ctas_per_sm(n);
      std::vector<Shape> cands;
      for (int cps = occ; cps >= 1; --cps) cands.push_back(Shape{DEP_FUSED_DENSE_FIRST, cps, best.x_cps});
      cands.push_back(Shape{DEP_SEPARATE, occ, best.x_cps});
      float best_ms = 1e30f;
      for (const Shape& c : cands) {
        float ms = 0.f;
        rc = time3([&]() -> int {
          if (int r = enqueue_deposit(b, (int)g, c, in, perm, st)) return r;
          if (c.dep == DEP_SEPARATE)
            PB_CK(spectral_dispatch(SPEC_X_R2C, n, ds, wx, grid_for(wx.total, b->sms, c.x_cps), st,
                                    b->d_maps.as<CUtensorMap>(), err),
                  "x r2c");
          return PM_OK;
        }, ms);
        if (rc) break;
        if (ms < best_ms) { best_ms = ms; best.dep = c.dep; best.dep_cps = c.dep_cps; }
      }
    }
    if (!rc && xrow_supported(n)) {  // x passes' grid (register row transforms)
      float best_ms = 1e30f;
      for (int cps : {4, 8, 16}) {
        float ms = 0.f;
        rc = time3([&]() -> int {
          PB_CK(spectral_dispatch(SPEC_X_C2R, n, ds, wx, grid_for(wx.total, b->sms, cps), st,
                                  b->d_maps.as<CUtensorMap>(), err),
                "x c2r");
          return PM_OK;
        }, ms);
        if (rc) break;
        if (ms < best_ms) { best_ms = ms; best.x_cps = cps; }
      }
    }
    if (!rc) {
      P.shape[g] = best;
      found.emplace_back(key, best);
    }
  }
  const int kkey = volume_class(P.fixed_total[PH_KICK]);
  bool kick_known;
  {
    std::lock_guard<std::mutex> lk(g_tune_lock);
    kick_known = g_kick_cps.count(kkey) != 0;
  }
  if (!rc && !kick_known) {  // the kick's grid; its keys and histogram go to scratch buffers
    const Work wk = work_of(b, PH_KICK, P.fixed_total[PH_KICK]);
    float best_ms = 1e30f;
    for (int cps : {4, 8, 16, 32}) {
      float ms = 0.f;
      rc = time3([&]() -> int {
        PB_CK(launch_kick(ds, wk, in, out, perm, b->sort.vals_alt.as<unsigned>(), POS_DISP, err,
                          grid_for(wk.total, b->sms, cps), st, b->row_cursor.as<unsigned>()),
              "kick");
        return PM_OK;
      }, ms);
      if (rc) break;
      if (ms < best_ms) { best_ms = ms; P.kick_cps = cps; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  {
    std::lock_guard<std::mutex> lk(g_tune_lock);
    for (auto& f : found) g_shapes[f.first] = f.second;
    if (!kick_known) g_kick_cps[kkey] = P.kick_cps;
  }
  b->tuned = true;
  b->host_s[4] -= drop_graphs(b);  // (counted as graph work, not tuning)
  return PM_OK;
}

// After a step the state is compact: every simulation's slots are its sorted range.
void compacted(pm_batch* b) {
  if (!b->sparse) return;
  b->sparse = false;
  for (auto& s : b->sims) s->in_off = s->part_off;
  b->in_total = b->plan.ptot;
  b->plan.sort_n = b->plan.ptot;
}

int run_steps(pm_batch* b, int k, cudaStream_t st) {
  for (int i = 0; i < k; ++i) {
    const int cur = b->cur;
    if (b->graphs && !b->sparse) {
      if (!b->gexec[cur] || b->gstale[cur]) {
        HostTimer timer(b->host_s[2]);
        cudaGraph_t g = nullptr;
        PB_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
        const int r = enqueue_step(b, cur, st);
        const cudaError_t e = cudaStreamEndCapture(st, &g);
        if (r) {
          if (g) cudaGraphDestroy(g);
          return r;
        }
        PB_CK(e, "end capture");
        cudaError_t ie = cudaSuccess;
        if (b->gexec[cur]) {  // stale: update in place when the graph's shape allows it
          cudaGraphExecUpdateResultInfo info;
          if (cudaGraphExecUpdate(b->gexec[cur], g, &info) != cudaSuccess) {
            cudaGetLastError();  // (not sticky: the shape changed)
            cudaGraphExecDestroy(b->gexec[cur]);
            b->gexec[cur] = nullptr;
          }
        }
        if (!b->gexec[cur]) ie = cudaGraphInstantiate(&b->gexec[cur], g, 0);
        b->gstale[cur] = false;
        cudaGraphDestroy(g);
        PB_CK(ie, "instantiate");
      }
      PB_CK(cudaGraphLaunch(b->gexec[cur], st), "graph launch");
    } else {
      // (the first step after a retirement reads a state with empty slots: launched directly,
      // the graphs are captured for the compact state that follows)
      if (int r = enqueue_step(b, cur, st)) return r;
    }
    b->cur = 1 - cur;
    compacted(b);
  }
  return PM_OK;
}

// Finished simulations leave the batch: their final state is extracted on `st` (fin_ev marks
// its completion) and their grids go to the pool.  The others stay where they are; the next
// step's sort skips the empty slots and its kick writes the survivors back compactly.
int retire_finished(pm_batch* b, cudaStream_t st) {
  bool any = false;
  for (auto& s : b->sims) any |= s->done >= s->nsteps;
  if (!any) return PM_OK;
  HostTimer timer(b->host_s[3]);
  Parts curp = state(b, b->cur);
  std::vector<std::unique_ptr<SimRec>> keep;
  for (auto& s : b->sims) {
    if (s->done >= s->nsteps) {
      const size_t pb = (size_t)3 * s->np * sizeof(float);
      auto& fp = b->fin_pool[s->np];
      if (!fp.empty()) {
        s->fin_pos = fp.back().first;
        s->fin_vel = fp.back().second;
        fp.pop_back();
      }
      PB_CK(s->fin_pos.ensure(pb), "alloc final");
      PB_CK(s->fin_vel.ensure(pb), "alloc final");
      Lattice* l = lattice_for(b, s->np1, s->n);
      PB_CK(launch_disp_to_abs(curp, s->in_off, s->np, s->np1, s->n, l->qi.as<int>(), l->qf.as<float>(),
                               s->fin_pos.as<float>(), s->fin_vel.as<float>(), st),
            "extract");
      if (!s->fin_ev) PB_CK(cudaEventCreateWithFlags(&s->fin_ev, cudaEventDisableTiming), "event");
      PB_CK(cudaEventRecord(s->fin_ev, st), "event");
      s->resident = false;
      b->grid_pool[s->n].emplace_back(s->grid, s->spec);  // reused in stream order on `st`
      s->grid = DBuf();
      s->spec = DBuf();
      s->rho.release();
      b->retired.push_back(std::move(s));
      b->sparse = true;
    } else {
      keep.push_back(std::move(s));
    }
  }
  b->sims = std::move(keep);
  b->dirty = true;
  b->keys_valid = false;
  if (b->sims.empty()) {  // nothing left to read: the next admission starts a fresh state
    b->sparse = false;
    b->in_total = 0;
  }
  return PM_OK;
}

SimRec* find_sim(pm_batch* b, int id) {
  for (auto& s : b->sims)
    if (s->id == id) return s.get();
  for (auto& s : b->retired)
    if (s->id == id) return s.get();
  return nullptr;
}

int read_back_a(pm_batch* b, cudaStream_t st) {
  // host mirrors of a / step are advanced in run_steps; nothing to read
  (void)b;
  (void)st;
  return PM_OK;
}

}  // namespace

extern "C" {

size_t pm_sim_footprint(const pm_config* cfg) { return cfg ? footprint(*cfg) : 0; }

int pm_batch_create(int device, size_t mem_cap_bytes, pm_batch** out) {
  if (!out) return PM_ERR_ARG;
  *out = nullptr;
  pm_batch* b = new pm_batch();
  b->device = device;
  b->cap = mem_cap_bytes;
  cudaError_t e = cudaSetDevice(device);
  if (!e) b->sms = sm_count(device);
  if (!e) e = b->d_err.ensure(sizeof(int));
  if (!e) e = b->tile_next.ensure(4 * sizeof(unsigned));
  if (!e) e = cudaMemset(b->d_err.p, 0, sizeof(int));
  if (!e) e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
  if (!e) e = cudaStreamCreateWithFlags(&b->admit, cudaStreamNonBlocking);
  if (!e) e = cudaEventCreateWithFlags(&b->last_step, cudaEventDisableTiming);
  if (!e) e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
  if (!e) e = cudaDeviceSynchronize();
  if (e) {
    pm_batch_destroy(b);
    return e == cudaErrorMemoryAllocation ? PM_ERR_OOM : PM_ERR_CUDA;
  }
  *out = b;
  return PM_OK;
}

void pm_batch_destroy(pm_batch* b) {
  if (!b) return;
  drop_graphs(b, true);
  for (int w = 0; w < 2; ++w)
    for (int k = 0; k < kStateArrays; ++k) b->st[w][k].release();
  for (auto& s : b->sims) {
    s->grid.release(); s->spec.release(); s->rho.release(); s->fin_pos.release(); s->fin_vel.release();
  }
  for (auto& s : b->retired) {
    s->fin_pos.release(); s->fin_vel.release();
    if (s->fin_ev) cudaEventDestroy(s->fin_ev);
  }
  for (auto& e : b->grid_pool)
    for (auto& g : e.second) { g.first.release(); g.second.release(); }
  for (auto& e : b->fin_pool)
    for (auto& g : e.second) { g.first.release(); g.second.release(); }
  b->stage_pos.release();
  b->stage_vel.release();
  b->adm_count.release();
  b->adm_start.release();
  b->adm_cursor.release();
  b->adm_sums.release();
  for (auto& t : b->tables) t.second->release();
  for (auto& l : b->lattices) l.second->release();
  b->sort.release();
  b->row_start.release();
  b->row_count.release();
  b->row_cursor.release();
  b->scan_sums.release();
  b->d_sims.release();
  b->d_prefix.release();
  b->d_err.release();
  b->tile_next.release();
  b->tile_order.release();
  b->d_maps.release();
  b->d_one.release();
  if (b->own) cudaStreamDestroy(b->own);
  if (b->admit) cudaStreamDestroy(b->admit);
  for (int t = 0; t < 2; ++t) {
    if (b->plan_ev[t]) cudaEventDestroy(b->plan_ev[t]);
    if (b->plan_host[t]) cudaFreeHost(b->plan_host[t]);
  }
  if (b->last_step) cudaEventDestroy(b->last_step);
  if (b->fork_ev) cudaEventDestroy(b->fork_ev);
  for (auto s : b->side) cudaStreamDestroy(s);
  for (auto e : b->side_ev) cudaEventDestroy(e);
  delete b;
}

const char* pm_batch_last_error(const pm_batch* b) { return b ? b->err.c_str() : "null batch"; }

int pm_batch_set_graphs(pm_batch* b, int enable) {
  if (!b) return PM_ERR_ARG;
  b->graphs = enable != 0;
  drop_graphs(b, true);
  return PM_OK;
}

int pm_batch_admits(pm_batch* b, const pm_config* cfg) {
  if (!b || !cfg) return 0;
  return (!b->cap || used_bytes(b) + footprint(*cfg) <= b->cap) ? 1 : 0;
}

int pm_batch_add(pm_batch* b, const pm_config* cfg, const float* positions, const float* velocities,
                 int on_device, int* sim_id) {
  if (!b) return PM_ERR_ARG;
  if (!cfg || !positions || !velocities || !sim_id) return bfail(b, PM_ERR_ARG, "null argument");
  if (!grid_supported(cfg->n_cells)) return bfail(b, PM_ERR_ARG, "unsupported N_CELLS");
  if (cfg->n_parts <= 0 || cfg->n_parts > 1024) return bfail(b, PM_ERR_ARG, "unsupported N_PARTS");
  if (cfg->steps <= 0 || !(cfg->a_init > 0.0) || !(cfg->a_end > cfg->a_init))
    return bfail(b, PM_ERR_ARG, "bad time range");
  const size_t need = footprint(*cfg);
  if (b->cap && used_bytes(b) + need > b->cap) return bfail(b, PM_ERR_ADMIT, "memory cap reached");
  std::unique_ptr<SimRec> r(new SimRec());
  r->id = b->next_id++;
  r->cfg = *cfg;
  r->n = cfg->n_cells;
  r->np1 = cfg->n_parts;
  r->np = (long long)cfg->n_parts * cfg->n_parts * cfg->n_parts;
  r->da = (cfg->a_end - cfg->a_init) / cfg->steps;
  r->a = cfg->a_init;
  {  // pmesh.py:56,63 loop count
    double a = cfg->a_init;
    int k = 0;
    while (a < cfg->a_end - r->da) { a += r->da; ++k; }
    r->nsteps = k;
  }
  HostTimer timer(b->host_s[0]);
  const size_t gb = (size_t)r->n * r->n * r->n * sizeof(float);
  const size_t sb = (size_t)r->n * r->n * spec_pitch(r->n) * sizeof(float2);
  auto& gp = b->grid_pool[r->n];
  if (!gp.empty()) {  // a retired simulation's grids (stream-ordered reuse by the next step)
    r->grid = gp.back().first;
    r->spec = gp.back().second;
    gp.pop_back();
  } else {
    trim_pools(b, gb + sb);
    PB_CK(r->grid.ensure(gb), "alloc grid");
    PB_CK(r->spec.ensure(sb), "alloc spectrum");
  }
  if (cfg->flags & PM_FLAG_KEEP_DENSITY) PB_CK(r->rho.ensure(gb), "alloc density");
  std::memset(r->maps, 0, sizeof(r->maps));
  spectral_encode_maps(r->n, r->spec.p, r->maps);
  PB_CK(tables_for(b, r->n)->build(r->n), "tables");
  Lattice* l = lattice_for(b, r->np1, r->n);
  PB_CK(l->build(r->np1, r->n), "lattice");
  // the new simulation takes the slots after the last ones of the state the next step reads
  const long long off = b->in_total;
  PB_CK(grow_state(b, off + r->np), "alloc state");
  // Convert on the admission stream once the steps already enqueued are done (an earlier
  // step may still write these slots), and wait for it here: the caller's arrays are free
  // when this returns.
  cudaStream_t st = b->admit;
  PB_CK(cudaStreamWaitEvent(st, b->last_step, 0), "wait steps");
  const float* dp = positions;
  const float* dv = velocities;
  const size_t pb = (size_t)3 * r->np * sizeof(float);
  if (!on_device) {
    PB_CK(b->stage_pos.ensure_geo(pb), "alloc staging");
    PB_CK(b->stage_vel.ensure_geo(pb), "alloc staging");
    PB_CK(cudaMemcpyAsync(b->stage_pos.p, positions, pb, cudaMemcpyHostToDevice, st), "h2d");
    PB_CK(cudaMemcpyAsync(b->stage_vel.p, velocities, pb, cudaMemcpyHostToDevice, st), "h2d");
    dp = b->stage_pos.as<float>();
    dv = b->stage_vel.as<float>();
  }
  {  // the state is written in row order (the counting sort of the new particles' rows), so that
     // its first step reads it almost in order like every later one (a step sorts the state
     // it writes)
    const unsigned nrows = (unsigned)((long long)r->n * r->n);
    PB_CK(b->adm_count.ensure_geo(sizeof(unsigned) * nrows), "alloc rows");
    PB_CK(b->adm_start.ensure_geo(sizeof(unsigned) * ((size_t)nrows + 1)), "alloc rows");
    PB_CK(b->adm_cursor.ensure_geo(sizeof(unsigned) * nrows), "alloc rows");
    PB_CK(b->adm_sums.ensure_geo(sizeof(unsigned) * row_sort_block_sums(nrows)), "alloc rows");
    unsigned* keys = b->sort.keys.as<unsigned>();  // free: the enqueued steps are done
    unsigned* order = b->sort.vals.as<unsigned>();
    PB_CK(launch_row_keys_abs(dp, r->np, r->n, keys, st), "admission keys");
    PB_CK(row_counting_sort(keys, r->np, nrows, b->adm_count.as<unsigned>(), b->adm_start.as<unsigned>(),
                            b->adm_cursor.as<unsigned>(), b->adm_sums.as<unsigned>(), order, nullptr, b->sms, st),
          "admission sort");
    PB_CK(launch_abs_to_disp(dp, dv, r->np, r->np1, r->n, l->qi.as<int>(), l->qf.as<float>(), state(b, b->cur),
                             off, st, order),
          "convert");
  }
  PB_CK(cudaStreamSynchronize(st), "sync");
  r->in_off = off;
  b->in_total = off + r->np;
  r->resident = true;
  *sim_id = r->id;
  b->sims.push_back(std::move(r));
  b->dirty = true;
  b->keys_valid = false;
  return PM_OK;
}

int pm_batch_step(pm_batch* b, int nsteps, void* stream) {
  if (!b) return PM_ERR_ARG;
  if (nsteps < 0) return bfail(b, PM_ERR_ARG, "negative step count");
  cudaStream_t st = stream ? (cudaStream_t)stream : b->own;
  if (!stream) PB_CK(cudaDeviceSynchronize(), "sync");  // order after legacy-stream work
  int left = nsteps;
  while (left > 0 && !b->sims.empty()) {
    if (int r = retire_finished(b, st)) return r;
    if (b->sims.empty()) break;
    if (b->dirty) {
      if (int r = build_plan(b, st)) return r;
    }
    int k = left;
    for (auto& s : b->sims) k = std::min(k, s->nsteps - s->done);
    if (k <= 0) break;
    if (int r = ensure_keys(b, st)) return r;
    if (!b->tuned && b->autotune) {
      if (b->plan_steps >= TUNE_AFTER_STEPS) {
        if (int r = autotune(b, st)) return r;
      } else {
        k = std::min(k, TUNE_AFTER_STEPS - b->plan_steps);  // a sorted state first
      }
    }
    if (int r = run_steps(b, k, st)) return r;
    b->plan_steps += k;
    for (auto& s : b->sims) {
      for (int i = 0; i < k; ++i) s->a += s->da;
      s->done += k;
    }
    left -= k;
  }
  const int r = retire_finished(b, st);
  if (r == PM_OK) PB_CK(cudaEventRecord(b->last_step, st), "event");
  if (!stream && r == PM_OK) PB_CK(cudaStreamSynchronize(st), "sync");
  return r;
}

int pm_batch_active(pm_batch* b, int sim_id) {
  if (!b) return -1;
  for (auto& s : b->sims)
    if (s->id == sim_id) return 1;
  for (auto& s : b->retired)
    if (s->id == sim_id) {
      if (!s->fin_ev) return 0;
      const cudaError_t q = cudaEventQuery(s->fin_ev);
      if (q == cudaErrorNotReady) return 1;  // its last steps are still running on the device
      if (q != cudaSuccess) cudaGetLastError();  // reported by the next call that synchronises
      return 0;
    }
  return -1;
}

int pm_batch_get(pm_batch* b, int sim_id, float* positions, float* velocities, int to_device, double* a,
                 int* steps_done, void* stream) {
  if (!b) return PM_ERR_ARG;
  SimRec* s = find_sim(b, sim_id);
  if (!s) return bfail(b, PM_ERR_ARG, "unknown simulation id");
  cudaStream_t st = (cudaStream_t)stream;
  if (a) *a = s->a;
  if (steps_done) *steps_done = s->done;
  if (!positions && !velocities) return PM_OK;
  const size_t pb = (size_t)3 * s->np * sizeof(float);
  const float* sp;
  const float* sv;
  DBuf tp, tv;
  // after the steps enqueued on the batch's stream (and the final-state extraction)
  PB_CK(cudaStreamWaitEvent(st, s->resident || !s->fin_ev ? b->last_step : s->fin_ev, 0), "wait");
  if (s->resident) {
    PB_CK(tp.ensure(pb), "alloc staging");
    PB_CK(tv.ensure(pb), "alloc staging");
    Lattice* l = lattice_for(b, s->np1, s->n);
    PB_CK(launch_disp_to_abs(state(b, b->cur), s->in_off, s->np, s->np1, s->n, l->qi.as<int>(),
                             l->qf.as<float>(), tp.as<float>(), tv.as<float>(), st),
          "extract");
    sp = tp.as<float>();
    sv = tv.as<float>();
  } else {
    sp = s->fin_pos.as<float>();
    sv = s->fin_vel.as<float>();
  }
  const cudaMemcpyKind kind = to_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (positions) PB_CK(cudaMemcpyAsync(positions, sp, pb, kind, st), "copy out");
  if (velocities) PB_CK(cudaMemcpyAsync(velocities, sv, pb, kind, st), "copy out");
  PB_CK(cudaStreamSynchronize(st), "sync");
  tp.release();
  tv.release();
  return read_back_a(b, st);
}

int pm_batch_density(pm_batch* b, int sim_id, float* rho, void* stream) {
  if (!b) return PM_ERR_ARG;
  if (!rho) return bfail(b, PM_ERR_ARG, "null array");
  cudaStream_t st = stream ? (cudaStream_t)stream : b->own;
  if (!stream) PB_CK(cudaDeviceSynchronize(), "sync");
  int idx = -1;
  for (size_t i = 0; i < b->sims.size(); ++i)
    if (b->sims[i]->id == sim_id) idx = (int)i;
  if (idx < 0) return bfail(b, PM_ERR_ARG, find_sim(b, sim_id) ? "simulation is no longer resident" : "unknown simulation id");
  if (b->dirty) {
    if (int r = build_plan(b, st)) return r;
  }
  if (int r = ensure_keys(b, st)) return r;
  const Plan& P = b->plan;
  // group the batch's particles by row from the current keys (the row histogram the last kick
  // or ensure_keys made is only read: the next step's sort finds it unchanged)
  unsigned* perm = b->sort.vals.as<unsigned>();
  int* err = b->d_err.as<int>();
  PB_CK(cudaStreamWaitEvent(st, b->last_step, 0), "wait");
  PB_CK(row_counting_sort(b->sort.keys.as<unsigned>(), P.sort_n, P.rows, b->row_count.as<unsigned>(),
                          b->row_start.as<unsigned>(), b->row_cursor.as<unsigned>(), b->scan_sums.as<unsigned>(),
                          perm, err, b->sms, st, nullptr, true),
        "sort");
  // this simulation's descriptor with the caller's grid as the deposit's output
  Sim s{};
  PB_CK(cudaMemcpyAsync(&s, b->d_sims.as<Sim>() + idx, sizeof(Sim), cudaMemcpyDeviceToHost, st), "read sim");
  PB_CK(cudaStreamSynchronize(st), "sync");
  s.rho = rho;
  struct {
    Sim sim;
    int prefix[2];
  } one{s, {0, (s.n / TILE_Y) * (s.n / TILE_Z)}};
  PB_CK(b->d_one.ensure(sizeof(one)), "alloc descriptor");
  PB_CK(cudaMemcpy(b->d_one.p, &one, sizeof(one), cudaMemcpyHostToDevice), "upload descriptor");
  auto* d = b->d_one.as<char>();
  const Work w{reinterpret_cast<const int*>(d + offsetof(decltype(one), prefix)), 1, one.prefix[1]};
  PB_CK(launch_deposit(reinterpret_cast<const Sim*>(d), w, state(b, b->cur), perm, b->row_start.as<unsigned>(),
                       POS_DISP, err, grid_for(one.prefix[1], b->sms, 3), deposit_smem_bytes(s.n, TILE_Y, TILE_Z),
                       st),
        "deposit");
  PB_CK(cudaEventRecord(b->last_step, st), "event");
  if (!stream) PB_CK(cudaStreamSynchronize(st), "sync");
  return PM_OK;
}

int pm_batch_remove(pm_batch* b, int sim_id) {
  if (!b) return PM_ERR_ARG;
  for (size_t i = 0; i < b->retired.size(); ++i) {
    SimRec& r = *b->retired[i];
    if (r.id == sim_id) {
      // its buffers are reused in the order of the batch's stream, after the extraction
      if (r.fin_ev) {
        PB_CK(cudaEventSynchronize(r.fin_ev), "sync");
        cudaEventDestroy(r.fin_ev);
        r.fin_ev = nullptr;
      }
      if (r.fin_pos.p) b->fin_pool[r.np].emplace_back(r.fin_pos, r.fin_vel);
      r.fin_pos = DBuf();
      r.fin_vel = DBuf();
      b->retired.erase(b->retired.begin() + i);
      return PM_OK;
    }
  }
  for (auto& s : b->sims) {
    if (s->id == sim_id) {
      s->done = s->nsteps;  // retire now, then drop
      if (int r = retire_finished(b, b->own)) return r;
      PB_CK(cudaEventRecord(b->last_step, b->own), "event");
      return pm_batch_remove(b, sim_id);
    }
  }
  return bfail(b, PM_ERR_ARG, "unknown simulation id");
}

int pm_batch_set_autotune(pm_batch* b, int enable) {
  if (!b) return PM_ERR_ARG;
  b->autotune = enable != 0;
  if (!b->autotune) b->dirty = true;  // back to the defaults and cached schedules at the next plan
  return PM_OK;
}

int pm_batch_schedule(pm_batch* b, int* out, int cap) {
  if (!b || !out || cap < 0) return -1;
  const Plan& P = b->plan;
  int k = 0;
  for (size_t g = 0; g < P.sizes.size() && k + 4 <= cap; ++g) {
    const Shape& sh = P.shape.size() > g ? P.shape[g] : Shape();
    out[k++] = P.sizes[g];
    out[k++] = sh.dep;
    out[k++] = sh.dep_cps ? sh.dep_cps : deposit_r2c_ctas_per_sm(P.sizes[g]);
    out[k++] = sh.x_cps;
  }
  if (k + 4 <= cap && !P.sizes.empty()) {
    out[k++] = 0;
    out[k++] = P.kick_cps;
    out[k++] = b->tuned ? 1 : 0;
    out[k++] = 0;
  }
  return k;
}

int pm_batch_host_seconds(pm_batch* b, double* out, int n) {
  if (!b || !out || n < 0) return PM_ERR_ARG;
  for (int i = 0; i < n && i < 6; ++i) out[i] = b->host_s[i];
  return PM_OK;
}

int pm_batch_profile(pm_batch* b, int nsteps, float* phase_ms, int nphase, void* stream) {
  if (!b || !phase_ms || nphase < PP_COUNT) return PM_ERR_ARG;
  cudaStream_t st = stream ? (cudaStream_t)stream : b->own;
  if (!stream) PB_CK(cudaDeviceSynchronize(), "sync");
  for (int i = 0; i < nphase; ++i) phase_ms[i] = 0.f;
  if (int r = retire_finished(b, st)) return r;
  if (b->sims.empty()) return bfail(b, PM_ERR_ARG, "no active simulation");
  if (b->dirty) {
    if (int r = build_plan(b, st)) return r;
  }
  int k = nsteps;
  for (auto& s : b->sims) k = std::min(k, s->nsteps - s->done);
  if (int r = ensure_keys(b, st)) return r;
  if (b->plan_steps >= TUNE_AFTER_STEPS)
    if (int r = autotune(b, st)) return r;
  cudaEvent_t ev[PP_COUNT + 1];
  for (auto& e : ev) PB_CK(cudaEventCreate(&e), "event");
  int rc = PM_OK;
  for (int i = 0; i < k && rc == PM_OK; ++i) {
    rc = enqueue_step(b, b->cur, st, ev);
    if (rc) break;
    b->cur = 1 - b->cur;
    compacted(b);
    b->plan_steps += 1;
    for (auto& s : b->sims) { s->a += s->da; s->done += 1; }
    cudaError_t e = cudaEventSynchronize(ev[PP_COUNT]);
    if (e) { rc = bcuda(b, e, "profile sync"); break; }
    for (int p = 0; p < PP_COUNT; ++p) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[p], ev[p + 1]);
      phase_ms[p] += ms / (float)k;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  const int r = retire_finished(b, st);
  if (r == PM_OK) PB_CK(cudaEventRecord(b->last_step, st), "event");
  return r;
}

int pm_batch_launches_per_step(pm_batch* b) {
  if (!b) return -1;
  if (b->dirty && !b->sims.empty()) {
    if (build_plan(b, b->own)) return -1;
  }
  return b->sims.empty() ? 0 : launches_per_step(b);
}

int pm_batch_check(pm_batch* b, void* stream, int* bits) {
  if (!b || !bits) return PM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int h = 0;
  PB_CK(cudaMemcpyAsync(&h, b->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st), "read flags");
  PB_CK(cudaMemsetAsync(b->d_err.p, 0, sizeof(int), st), "clear flags");
  PB_CK(cudaStreamSynchronize(st), "sync");
  *bits = h;
  return h ? bfail(b, PM_ERR_DEVICE, "device check bits " + std::to_string(h)) : PM_OK;
}

}  // extern "C"
