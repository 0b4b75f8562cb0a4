// C ABI: context and drop-in hot-path entry points (see include/pm_gb300.h).
#include "pm_host.cuh"

using namespace pm;

struct pm_ctx {
  pm_config cfg{};
  int device = 0;
  int sms = 1;
  int n = 0;
  Tables tab;
  SortBufs sort;
  DBuf d_sim, d_prefix, d_err, d_maps;
  DBuf tile_next;  // tile counter of the fused deposit
  const void* maps_for = nullptr;     // spectrum the device tensor maps describe
  DBuf row_start, spec, phi, rho;     // scratch grids
  DBuf hpos, hvel;                    // device copies for pm_step_host
  DBuf pk_partial, pk_out;            // power spectrum scratch
  DBuf row_count, row_cursor, scan_sums;  // counting sort of row keys
  DBuf spos, svel;                        // the state in row order (drop-in step)
  // spectral gradient: spectra and force grids of the y and z axes (x uses spec and phi), the
  // three descriptors of the inverse passes and their work tables and tensor maps
  DBuf gspec[2], ggrid[2], d_sim3, d_prefix3, d_maps3;
  const void* maps3_for = nullptr;
  cudaStream_t side = nullptr;            // velocity copy of pm_step_host
  cudaEvent_t ev_start = nullptr, ev_vel = nullptr;
  std::vector<double> pk_host;
  std::string err;
};

namespace {

enum Phase { PH_KEYS = 0, PH_DEP, PH_KICK, PH_X, PH_LINE, PH_COUNT };

int fail(pm_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(pm_ctx* c, cudaError_t e, const char* where) {
  return fail(c, e == cudaErrorMemoryAllocation ? PM_ERR_OOM : PM_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

#define PM_CK(call, where)                                   \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, where);   \
  } while (0)

// Host image of the single-simulation descriptor + its work prefixes.
struct Call {
  Sim sim{};
  int prefix[PH_COUNT][2]{};
  Parts parts{};
};

Sim base_sim(pm_ctx* c, long long np) {
  Sim s{};
  s.n = c->n;
  s.pitch = spec_pitch(c->n);
  s.np1 = c->cfg.n_parts;
  s.xbits = ceil_log2(c->n);
  s.ty = TILE_Y;
  s.tz = TILE_Z;
  s.np = np;
  s.part_off = 0;
  s.row_base = 0;
  s.s2 = c->tab.s2.as<float>();
  s.sn = c->tab.sn.as<float>();
  s.tw = c->tab.tw.as<float2>();
  s.om = c->cfg.omega_m0;
  s.ol = c->cfg.omega_lambda0;
  s.ok = c->cfg.omega_k0;
  s.h0 = c->cfg.h0;
  s.fix_f = (c->cfg.flags & PM_FLAG_FIX_COSMO_F) ? 1 : 0;
  return s;
}

void set_prefix(Call& k, long long np, int n) {
  k.prefix[PH_KEYS][1] = (int)((np + 255) / 256);
  k.prefix[PH_DEP][1] = (n / TILE_Y) * (n / TILE_Z);
  k.prefix[PH_KICK][1] = (int)((np + KICK_UNIT - 1) / KICK_UNIT);
  k.prefix[PH_X][1] = (int)spectral_units(SPEC_X_R2C, n);
  k.prefix[PH_LINE][1] = (int)spectral_units(SPEC_Y_FWD, n);
}

Work work(pm_ctx* c, const Call& k, Phase ph) {
  Work w;
  w.prefix = c->d_prefix.as<int>() + 2 * ph;
  w.nsims = 1;
  w.total = k.prefix[ph][1];
  return w;
}

Parts abs_parts(float* pos, float* vel, long long np) {
  Parts p{};
  p.x = pos;
  p.y = pos ? pos + np : nullptr;
  p.z = pos ? pos + 2 * np : nullptr;
  p.vx = vel;
  p.vy = vel ? vel + np : nullptr;
  p.vz = vel ? vel + 2 * np : nullptr;
  p.id = nullptr;
  return p;
}

int check_np(pm_ctx* c, long long np) {
  if (np <= 0) return fail(c, PM_ERR_ARG, "particle count must be positive");
  if (np >= (1ll << 31)) return fail(c, PM_ERR_ARG, "particle count must be below 2^31");
  return PM_OK;
}

int upload(pm_ctx* c, Call& k, cudaStream_t st) {
  PM_CK(cudaMemcpyAsync(c->d_sim.p, &k.sim, sizeof(Sim), cudaMemcpyHostToDevice, st), "upload sim");
  PM_CK(cudaMemcpyAsync(c->d_prefix.p, k.prefix, sizeof(k.prefix), cudaMemcpyHostToDevice, st),
        "upload work");
  return PM_OK;
}

// keys -> sort -> row starts for absolute positions; leaves perm / sorted keys pointers.
int sort_particles(pm_ctx* c, Call& k, cudaStream_t st, unsigned** perm, unsigned** skeys) {
  const long long np = k.sim.np;
  PM_CK(c->sort.ensure(np), "alloc sort");
  const Sim* ds = c->d_sim.as<Sim>();
  PM_CK(launch_keys_abs(ds, work(c, k, PH_KEYS), k.parts, c->sort.keys.as<unsigned>(), nullptr,
                        c->d_err.as<int>(), grid_for(k.prefix[PH_KEYS][1], c->sms, 16), st),
        "keys");
  const long long nrows = (long long)c->n * c->n;
  const int bits = ceil_log2(nrows) + k.sim.xbits;
  bool alt = false;
  PM_CK(radix_sort(c->sort.keys.as<unsigned>(), c->sort.vals.as<unsigned>(), np, 0, bits, true,
                   c->sort.scratch(), &alt, st),
        "sort");
  *perm = alt ? c->sort.vals_alt.as<unsigned>() : c->sort.vals.as<unsigned>();
  *skeys = alt ? c->sort.keys_alt.as<unsigned>() : c->sort.keys.as<unsigned>();
  return PM_OK;
}

// keys (x-row numbers: k.sim.xbits must be 0) -> counting sort: row starts in c->row_start
// and the permutation to row order.  The deposit and the kick need the particles grouped
// by row only; their results do not depend on the order inside a row.
int group_particles(pm_ctx* c, Call& k, cudaStream_t st, unsigned** perm, unsigned* inv = nullptr,
                    float* pos_copy = nullptr) {
  const long long np = k.sim.np;
  const unsigned nrows = (unsigned)((long long)c->n * c->n);
  PM_CK(c->sort.ensure(np), "alloc sort");
  PM_CK(c->row_start.ensure(((size_t)nrows + 1) * sizeof(unsigned)), "alloc rows");
  PM_CK(c->row_count.ensure((size_t)nrows * sizeof(unsigned)), "alloc rows");
  PM_CK(c->row_cursor.ensure((size_t)nrows * sizeof(unsigned)), "alloc rows");
  PM_CK(c->scan_sums.ensure(row_sort_block_sums(nrows) * sizeof(unsigned)), "alloc rows");
  PM_CK(launch_keys_abs(c->d_sim.as<Sim>(), work(c, k, PH_KEYS), k.parts, c->sort.keys.as<unsigned>(), nullptr,
                        c->d_err.as<int>(), grid_for(k.prefix[PH_KEYS][1], c->sms, 16), st,
                        pos_copy ? abs_parts(pos_copy, nullptr, np) : Parts{}),
        "keys");
  *perm = c->sort.vals.as<unsigned>();
  PM_CK(row_counting_sort(c->sort.keys.as<unsigned>(), np, nrows, c->row_count.as<unsigned>(),
                          c->row_start.as<unsigned>(), c->row_cursor.as<unsigned>(), c->scan_sums.as<unsigned>(),
                          *perm, c->d_err.as<int>(), c->sms, st, inv),
        "sort");
  return PM_OK;
}

int deposit(pm_ctx* c, Call& k, unsigned* perm, cudaStream_t st) {
  PM_CK(launch_deposit(c->d_sim.as<Sim>(), work(c, k, PH_DEP), k.parts, perm, c->row_start.as<unsigned>(),
                       POS_ABS, c->d_err.as<int>(), grid_for(k.prefix[PH_DEP][1], c->sms, 8),
                       deposit_smem_bytes(c->n, TILE_Y, TILE_Z), st),
        "deposit");
  return PM_OK;
}

int gradient_solve(pm_ctx* c, Call& k, cudaStream_t st);

int spectral(pm_ctx* c, Call& k, bool table, cudaStream_t st, bool skip_r2c = false, bool gradient = false) {
  const Sim* ds = c->d_sim.as<Sim>();
  const int n = c->n;
  const int gx = grid_for(k.prefix[PH_X][1], c->sms, 8), gl = grid_for(k.prefix[PH_LINE][1], c->sms, 8);
  const CUtensorMap* maps = c->maps_for ? c->d_maps.as<CUtensorMap>() : nullptr;
  int* err = c->d_err.as<int>();
  if (!skip_r2c) PM_CK(spectral_dispatch(SPEC_X_R2C, n, ds, work(c, k, PH_X), gx, st, maps, err), "x r2c");
  PM_CK(spectral_dispatch(SPEC_Y_FWD, n, ds, work(c, k, PH_LINE), gl, st, maps, err), "y fwd");
  if (gradient) return gradient_solve(c, k, st);
  PM_CK(spectral_dispatch(table ? SPEC_Z_TABLE : SPEC_Z_GREEN, n, ds, work(c, k, PH_LINE), gl, st, maps, err),
        "z green");
  PM_CK(spectral_dispatch(SPEC_Y_INV, n, ds, work(c, k, PH_LINE), gl, st, maps, err), "y inv");
  PM_CK(spectral_dispatch(SPEC_X_C2R, n, ds, work(c, k, PH_X), gx, st, maps, err), "x c2r");
  return PM_OK;
}

// The spectral gradient (PM_FLAG_SPECTRAL_GRADIENT): from the spectrum after the forward y
// pass, three copies go through the z pass with the Green function times -i sin(k_d) and the
// inverse y and x passes -- one launch each over three descriptors -- into phi (x) and two more
// grids (y, z); k.sim.grad then points the kick at them.
int gradient_solve(pm_ctx* c, Call& k, cudaStream_t st) {
  const int n = c->n;
  const size_t sb = (size_t)n * n * spec_pitch(n) * sizeof(float2), gb = (size_t)n * n * n * sizeof(float);
  for (int i = 0; i < 2; ++i) {
    PM_CK(c->gspec[i].ensure(sb), "alloc gradient spectrum");
    PM_CK(c->ggrid[i].ensure(gb), "alloc gradient grid");
  }
  PM_CK(c->d_sim3.ensure(3 * sizeof(Sim)), "alloc descriptors");
  PM_CK(c->d_prefix3.ensure(8 * sizeof(int)), "alloc work");
  const CUtensorMap* maps = nullptr;
  if (c->maps_for && c->maps3_for != c->gspec[1].p) {  // tensor maps of the three spectra
    CUtensorMap m[6];
    const void* specs[3] = {c->spec.p, c->gspec[0].p, c->gspec[1].p};
    bool ok = true;
    for (int i = 0; i < 3; ++i) ok = ok && spectral_encode_maps(n, specs[i], &m[2 * i]);
    c->maps3_for = nullptr;
    if (ok) {
      PM_CK(c->d_maps3.ensure(sizeof(m)), "alloc maps");
      PM_CK(cudaMemcpy(c->d_maps3.p, m, sizeof(m), cudaMemcpyHostToDevice), "tensor maps");
      c->maps3_for = c->gspec[1].p;
    }
  }
  if (c->maps_for && c->maps3_for == c->gspec[1].p) maps = c->d_maps3.as<CUtensorMap>();
  Sim s3[3];
  for (int i = 0; i < 3; ++i) {
    s3[i] = k.sim;
    s3[i].grad_axis = i + 1;
    s3[i].spec = i == 0 ? c->spec.as<float2>() : c->gspec[i - 1].as<float2>();
    s3[i].phi = i == 0 ? c->phi.as<float>() : c->ggrid[i - 1].as<float>();
  }
  const int lu = (int)spectral_units(SPEC_Y_FWD, n), xu = (int)spectral_units(SPEC_X_C2R, n);
  const int pre[8] = {0, lu, 2 * lu, 3 * lu, 0, xu, 2 * xu, 3 * xu};
  PM_CK(cudaMemcpyAsync(c->d_sim3.p, s3, sizeof(s3), cudaMemcpyHostToDevice, st), "upload descriptors");
  PM_CK(cudaMemcpyAsync(c->d_prefix3.p, pre, sizeof(pre), cudaMemcpyHostToDevice, st), "upload work");
  PM_CK(cudaMemcpyAsync(c->gspec[0].p, c->spec.p, sb, cudaMemcpyDeviceToDevice, st), "copy spectrum");
  PM_CK(cudaMemcpyAsync(c->gspec[1].p, c->spec.p, sb, cudaMemcpyDeviceToDevice, st), "copy spectrum");
  const Sim* ds = c->d_sim3.as<Sim>();
  const Work wl{c->d_prefix3.as<int>(), 3, 3 * lu}, wx{c->d_prefix3.as<int>() + 4, 3, 3 * xu};
  const int gl = grid_for(wl.total, c->sms, 8), gx = grid_for(wx.total, c->sms, 8);
  int* err = c->d_err.as<int>();
  PM_CK(spectral_dispatch(SPEC_Z_GRAD, n, ds, wl, gl, st, maps, err), "z green gradient");
  PM_CK(spectral_dispatch(SPEC_Y_INV, n, ds, wl, gl, st, maps, err), "y inv");
  PM_CK(spectral_dispatch(SPEC_X_C2R, n, ds, wx, gx, st, maps, err), "x c2r");
  k.sim.grad[0] = c->phi.as<float>();
  k.sim.grad[1] = c->ggrid[0].as<float>();
  k.sim.grad[2] = c->ggrid[1].as<float>();
  return PM_OK;
}

int prepare_spectral(pm_ctx* c, Call& k) {
  const size_t sb = (size_t)c->n * c->n * spec_pitch(c->n) * sizeof(float2);
  cudaError_t e = c->spec.ensure(sb);
  if (e) return cuda_fail(c, e, "alloc spectrum");
  k.sim.spec = c->spec.as<float2>();
  if (c->maps_for != c->spec.p) {  // tensor maps of the spectrum for the TMA line passes
    CUtensorMap m[2];
    c->maps_for = nullptr;
    if (spectral_encode_maps(c->n, c->spec.p, m)) {
      e = c->d_maps.ensure(sizeof(m));
      if (!e) e = cudaMemcpy(c->d_maps.p, m, sizeof(m), cudaMemcpyHostToDevice);
      if (e) return cuda_fail(c, e, "tensor maps");
      c->maps_for = c->spec.p;
    }
  }
  return PM_OK;
}

void set_green(pm_ctx* c, Sim& s, double a) {
  const double n3 = (double)c->n * c->n * c->n;
  s.green = (float)(-3.0 * c->cfg.omega_m0 / 8.0 / a / n3);
}

void set_kick(Sim& s, double a, double f_a1, double da) {
  s.kick = (float)(da * f_a1);
  s.drift = (float)(da / ((a + da) * (a + da)) * f_a1);
}

double f_step(pm_ctx* c, double a, double da) {
  const double slot = (c->cfg.flags & PM_FLAG_FIX_COSMO_F) ? c->cfg.omega_m0 : c->cfg.h0;
  return cosmo_f(a + da, slot, c->cfg.omega_lambda0, c->cfg.omega_k0);
}

int kick(pm_ctx* c, Call& k, unsigned* perm, cudaStream_t st) {
  PM_CK(launch_kick(c->d_sim.as<Sim>(), work(c, k, PH_KICK), k.parts, k.parts, perm, nullptr, POS_ABS,
                    c->d_err.as<int>(), grid_for(k.prefix[PH_KICK][1], c->sms, 16), st),
        "kick");
  return PM_OK;
}

}  // namespace

extern "C" {

int pm_supported_n(int n) { return grid_supported(n) ? 1 : 0; }

double pm_cosmo_f(double a, double om, double ol, double ok) { return cosmo_f(a, om, ol, ok); }

int pm_ctx_create(const pm_config* cfg, int device, pm_ctx** out) {
  if (!cfg || !out) return PM_ERR_ARG;
  *out = nullptr;
  if (!grid_supported(cfg->n_cells)) return PM_ERR_ARG;
  if (cfg->n_parts <= 0) return PM_ERR_ARG;
  pm_ctx* c = new pm_ctx();
  c->cfg = *cfg;
  c->device = device;
  c->n = cfg->n_cells;
  cudaError_t e = cudaSetDevice(device);
  if (!e) c->sms = sm_count(device);
  if (!e) e = c->tab.build(c->n);
  if (!e) e = c->d_sim.ensure(sizeof(Sim));
  if (!e) e = c->d_prefix.ensure(sizeof(int) * 2 * PH_COUNT);
  if (!e) e = c->d_err.ensure(sizeof(int));
  if (!e) e = c->tile_next.ensure(sizeof(unsigned));
  if (!e) e = cudaMemset(c->d_err.p, 0, sizeof(int));
  if (!e) e = cudaDeviceSynchronize();
  if (e) {
    pm_ctx_destroy(c);
    return e == cudaErrorMemoryAllocation ? PM_ERR_OOM : PM_ERR_CUDA;
  }
  *out = c;
  return PM_OK;
}

void pm_ctx_destroy(pm_ctx* c) {
  if (!c) return;
  c->tab.release();
  c->sort.release();
  c->d_sim.release();
  c->d_prefix.release();
  c->d_err.release();
  c->tile_next.release();
  c->d_maps.release();
  c->row_start.release();
  c->spec.release();
  c->phi.release();
  c->rho.release();
  c->hpos.release();
  c->hvel.release();
  c->pk_partial.release();
  c->pk_out.release();
  c->row_count.release();
  c->spos.release();
  c->svel.release();
  if (c->side) cudaStreamDestroy(c->side);
  if (c->ev_start) cudaEventDestroy(c->ev_start);
  if (c->ev_vel) cudaEventDestroy(c->ev_vel);
  c->row_cursor.release();
  c->scan_sums.release();
  for (int i = 0; i < 2; ++i) { c->gspec[i].release(); c->ggrid[i].release(); }
  c->d_sim3.release();
  c->d_prefix3.release();
  c->d_maps3.release();
  delete c;
}

const char* pm_last_error(const pm_ctx* c) { return c ? c->err.c_str() : "null context"; }

int pm_check_device(pm_ctx* c, void* stream, int* bits) {
  if (!c || !bits) return PM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int h = 0;
  PM_CK(cudaMemcpyAsync(&h, c->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st), "read flags");
  PM_CK(cudaMemsetAsync(c->d_err.p, 0, sizeof(int), st), "clear flags");
  PM_CK(cudaStreamSynchronize(st), "sync");
  *bits = h;
  return h ? fail(c, PM_ERR_DEVICE, "device check bits " + std::to_string(h)) : PM_OK;
}

int pm_density(pm_ctx* c, const float* positions, long long np, double mass, float* rho, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!positions || !rho) return fail(c, PM_ERR_ARG, "null array");
  if (int r = check_np(c, np)) return r;
  cudaStream_t st = (cudaStream_t)stream;
  Call k;
  k.sim = base_sim(c, np);
  k.sim.xbits = 0;  // row keys
  k.sim.rho = rho;
  k.sim.mass_scale = (float)(mass / (double)(1u << PM_FIX_BITS));
  set_prefix(k, np, c->n);
  k.parts = abs_parts(const_cast<float*>(positions), nullptr, np);
  if (int r = upload(c, k, st)) return r;
  unsigned* perm = nullptr;
  if (int r = group_particles(c, k, st, &perm)) return r;
  // deposit from a row-ordered copy of the positions (sequential reads of each row)
  PM_CK(c->spos.ensure((size_t)3 * np * sizeof(float)), "alloc state");
  PM_CK(launch_gather_state(positions, nullptr, np, perm, c->spos.as<float>(), nullptr, c->sms, st), "gather");
  k.parts = abs_parts(c->spos.as<float>(), nullptr, np);
  return deposit(c, k, nullptr, st);
}

int pm_fourier_grid(pm_ctx* c, float* fgrid, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!fgrid) return fail(c, PM_ERR_ARG, "null array");
  cudaStream_t st = (cudaStream_t)stream;
  Call k;
  k.sim = base_sim(c, 1);
  k.sim.rho = fgrid;
  if (int r = upload(c, k, st)) return r;
  PM_CK(launch_fourier_grid(c->d_sim.as<Sim>(), c->sms * 8, st), "fourier grid");
  return PM_OK;
}

int pm_potential(pm_ctx* c, const float* rho, const float* fgrid, double a, float* phi, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!rho || !phi) return fail(c, PM_ERR_ARG, "null array");
  if (!(a > 0.0)) return fail(c, PM_ERR_ARG, "scale factor must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  Call k;
  k.sim = base_sim(c, 1);
  k.sim.rho = const_cast<float*>(rho);
  k.sim.phi = phi;
  k.sim.fgrid = fgrid;
  set_green(c, k.sim, a);
  set_prefix(k, 1, c->n);
  if (int r = prepare_spectral(c, k)) return r;
  if (int r = upload(c, k, st)) return r;
  return spectral(c, k, fgrid != nullptr, st);
}

int pm_integrate(pm_ctx* c, float* positions, float* velocities, long long np, double a, double f_a1,
                 double da, const float* phi, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!positions || !velocities || !phi) return fail(c, PM_ERR_ARG, "null array");
  if (int r = check_np(c, np)) return r;
  cudaStream_t st = (cudaStream_t)stream;
  Call k;
  k.sim = base_sim(c, np);
  k.sim.xbits = 0;  // row keys: the kick reads the particles grouped by row (locality)
  k.sim.phi = const_cast<float*>(phi);
  set_kick(k.sim, a, f_a1, da);
  set_prefix(k, np, c->n);
  k.parts = abs_parts(positions, velocities, np);
  if (int r = upload(c, k, st)) return r;
  unsigned* perm = nullptr;
  if (int r = group_particles(c, k, st, &perm)) return r;
  return kick(c, k, perm, st);
}

int pm_advance_time(pm_ctx* c, const float* rho, float* positions, float* velocities, long long np,
                    const float* fgrid, double a, double da, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!rho || !positions || !velocities) return fail(c, PM_ERR_ARG, "null array");
  if (int r = check_np(c, np)) return r;
  if (!(a > 0.0)) return fail(c, PM_ERR_ARG, "scale factor must be positive");
  const size_t gb = (size_t)c->n * c->n * c->n * sizeof(float);
  PM_CK(c->phi.ensure(gb), "alloc phi");
  if (int r = pm_potential(c, rho, fgrid, a, c->phi.as<float>(), stream)) return r;
  return pm_integrate(c, positions, velocities, np, a, f_step(c, a, da), da, c->phi.as<float>(), stream);
}

}  // extern "C"

namespace {

// Where a step reads and writes the caller's state.
struct StepIO {
  const float* pos_in;    // read once by the keys kernel (device-accessible: device or pinned host)
  float* pos_copy;        // device copy the keys kernel leaves (null: pos_in is device memory)
  const float* vel_in;    // device
  cudaEvent_t vel_ready;  // vel_in complete (null: already)
  float* pos_out;         // result in particle order (device or pinned host)
  float* vel_out;
  // pinned host velocities: copied to vel_in on `side` once the keys kernel has read the
  // positions (the two transfers would share the link)
  const float* vel_host = nullptr;
  cudaStream_t side = nullptr;
  cudaEvent_t keys_done = nullptr;
};

// src/pmesh.py:60-61 on absolute positions: keys -> counting sort by row -> row-ordered copy
// of the state (the caller's arrays are in particle order, which scatters every row across
// memory) -> deposit (fused with the x R2C when the density is not requested) -> Poisson
// solve -> kick/drift in row order -> gathered back into particle order.
int step_core(pm_ctx* c, const StepIO& io, long long np, double mass, double a, double da, float* rho_out,
              cudaStream_t st) {
  const bool gradient = (c->cfg.flags & PM_FLAG_SPECTRAL_GRADIENT) != 0;
  const size_t gb = (size_t)c->n * c->n * c->n * sizeof(float);
  float* rho = rho_out;
  if (!rho) {
    PM_CK(c->rho.ensure(gb), "alloc rho");
    rho = c->rho.as<float>();
  }
  PM_CK(c->phi.ensure(gb), "alloc phi");
  Call k;
  k.sim = base_sim(c, np);
  k.sim.xbits = 0;  // row keys
  k.sim.rho = rho;
  k.sim.phi = c->phi.as<float>();
  k.sim.mass_scale = (float)(mass / (double)(1u << PM_FIX_BITS));
  set_green(c, k.sim, a);
  set_kick(k.sim, a, f_step(c, a, da), da);
  set_prefix(k, np, c->n);
  k.parts = abs_parts(const_cast<float*>(io.pos_in), nullptr, np);
  if (int r = prepare_spectral(c, k)) return r;
  if (int r = upload(c, k, st)) return r;
  const size_t pb = (size_t)3 * np * sizeof(float);
  PM_CK(c->spos.ensure(pb), "alloc state");
  PM_CK(c->svel.ensure(pb), "alloc state");
  PM_CK(c->sort.ensure(np), "alloc sort");
  unsigned* perm = nullptr;
  unsigned* inv = c->sort.vals_alt.as<unsigned>();
  if (int r = group_particles(c, k, st, &perm, inv, io.pos_copy)) return r;
  if (io.vel_host) {
    PM_CK(cudaEventRecord(io.keys_done, st), "event");
    PM_CK(cudaStreamWaitEvent(io.side, io.keys_done, 0), "event");
    PM_CK(cudaMemcpyAsync(const_cast<float*>(io.vel_in), io.vel_host, pb, cudaMemcpyHostToDevice, io.side),
          "h2d velocities");
    PM_CK(cudaEventRecord(io.vel_ready, io.side), "event");
  }
  PM_CK(launch_gather_state(io.pos_copy ? io.pos_copy : io.pos_in, nullptr, np, perm, c->spos.as<float>(), nullptr,
                            c->sms, st),
        "gather");
  Parts sp = abs_parts(c->spos.as<float>(), c->svel.as<float>(), np);
  k.parts = sp;
  if (!rho_out && deposit_r2c_supported(c->n)) {
    // the density is not requested: deposit straight into the x-transformed spectrum
    PM_CK(deposit_r2c_dispatch(c->n, c->d_sim.as<Sim>(), work(c, k, PH_DEP), sp, nullptr,
                               c->row_start.as<unsigned>(), POS_ABS, c->d_err.as<int>(), c->tile_next.as<unsigned>(),
                               nullptr, grid_for(k.prefix[PH_DEP][1], c->sms, deposit_r2c_ctas_per_sm(c->n)), st),
          "fused deposit");
    if (int r = spectral(c, k, false, st, true, gradient)) return r;
  } else {
    if (int r = deposit(c, k, nullptr, st)) return r;
    if (int r = spectral(c, k, false, st, false, gradient)) return r;
  }
  if (gradient)  // the kick's descriptor now names the three force grids
    PM_CK(cudaMemcpyAsync(c->d_sim.p, &k.sim, sizeof(Sim), cudaMemcpyHostToDevice, st), "upload sim");
  if (io.vel_ready) PM_CK(cudaStreamWaitEvent(st, io.vel_ready, 0), "wait velocities");
  PM_CK(launch_gather_state(io.vel_in, nullptr, np, perm, c->svel.as<float>(), nullptr, c->sms, st), "gather");
  if (int r = kick(c, k, nullptr, st)) return r;
  PM_CK(launch_gather_state(c->spos.as<float>(), c->svel.as<float>(), np, inv, io.pos_out, io.vel_out, c->sms, st),
        "gather back");
  return PM_OK;
}

bool pinned_host(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

}  // namespace

extern "C" {

int pm_step(pm_ctx* c, float* positions, float* velocities, long long np, double mass, double a, double da,
            float* rho_out, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!positions || !velocities) return fail(c, PM_ERR_ARG, "null array");
  if (int r = check_np(c, np)) return r;
  if (!(a > 0.0)) return fail(c, PM_ERR_ARG, "scale factor must be positive");
  StepIO io{positions, nullptr, velocities, nullptr, positions, velocities};
  return step_core(c, io, np, mass, a, da, rho_out, (cudaStream_t)stream);
}

int pm_step_host(pm_ctx* c, float* h_positions, float* h_velocities, long long np, double mass, double a,
                 double da, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!h_positions || !h_velocities) return fail(c, PM_ERR_ARG, "null array");
  if (int r = check_np(c, np)) return r;
  if (!(a > 0.0)) return fail(c, PM_ERR_ARG, "scale factor must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t pb = (size_t)3 * np * sizeof(float);
  PM_CK(c->hpos.ensure(pb), "alloc positions");
  PM_CK(c->hvel.ensure(pb), "alloc velocities");
  if (pinned_host(h_positions) && pinned_host(h_velocities)) {
    // Pinned arrays: the keys kernel reads the positions over the host link and leaves a
    // device copy; the velocities then cross on a copy engine while the deposit and the
    // solve run (the kick needs them first); the result is gathered back straight into the
    // host arrays.
    if (!c->side) {
      PM_CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking), "side stream");
      PM_CK(cudaEventCreateWithFlags(&c->ev_start, cudaEventDisableTiming), "event");
      PM_CK(cudaEventCreateWithFlags(&c->ev_vel, cudaEventDisableTiming), "event");
    }
    StepIO io{h_positions, c->hpos.as<float>(), c->hvel.as<float>(), c->ev_vel, h_positions, h_velocities};
    io.vel_host = h_velocities;
    io.side = c->side;
    io.keys_done = c->ev_start;
    if (int r = step_core(c, io, np, mass, a, da, nullptr, st)) return r;
  } else {  // pageable: copy engines both ways
    PM_CK(cudaMemcpyAsync(c->hpos.p, h_positions, pb, cudaMemcpyHostToDevice, st), "h2d positions");
    PM_CK(cudaMemcpyAsync(c->hvel.p, h_velocities, pb, cudaMemcpyHostToDevice, st), "h2d velocities");
    StepIO io{c->hpos.as<float>(), nullptr, c->hvel.as<float>(), nullptr, c->hpos.as<float>(), c->hvel.as<float>()};
    if (int r = step_core(c, io, np, mass, a, da, nullptr, st)) return r;
    PM_CK(cudaMemcpyAsync(h_positions, c->hpos.p, pb, cudaMemcpyDeviceToHost, st), "d2h positions");
    PM_CK(cudaMemcpyAsync(h_velocities, c->hvel.p, pb, cudaMemcpyDeviceToHost, st), "d2h velocities");
  }
  PM_CK(cudaStreamSynchronize(st), "sync");
  return PM_OK;
}

int pm_sort_keys(pm_ctx* c, const float* positions, long long np, unsigned* keys_out, unsigned* sorted_keys,
                 unsigned* perm_out, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!positions) return fail(c, PM_ERR_ARG, "null array");
  if (int r = check_np(c, np)) return r;
  cudaStream_t st = (cudaStream_t)stream;
  Call k;
  k.sim = base_sim(c, np);
  set_prefix(k, np, c->n);
  k.parts = abs_parts(const_cast<float*>(positions), nullptr, np);
  if (int r = upload(c, k, st)) return r;
  PM_CK(c->sort.ensure(np), "alloc sort");
  if (keys_out) {
    PM_CK(launch_keys_abs(c->d_sim.as<Sim>(), work(c, k, PH_KEYS), k.parts, keys_out, nullptr,
                          c->d_err.as<int>(), grid_for(k.prefix[PH_KEYS][1], c->sms, 16), st),
          "keys");
  }
  unsigned *perm = nullptr, *skeys = nullptr;
  if (int r = sort_particles(c, k, st, &perm, &skeys)) return r;
  const size_t b = (size_t)np * sizeof(unsigned);
  if (sorted_keys) PM_CK(cudaMemcpyAsync(sorted_keys, skeys, b, cudaMemcpyDeviceToDevice, st), "copy keys");
  if (perm_out) PM_CK(cudaMemcpyAsync(perm_out, perm, b, cudaMemcpyDeviceToDevice, st), "copy perm");
  return PM_OK;
}

int pm_project(pm_ctx* c, const float* rho, int n_slices, double* out, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!rho || !out) return fail(c, PM_ERR_ARG, "null array");
  if (n_slices < 0 || n_slices > c->n) return fail(c, PM_ERR_ARG, "n_slices must lie in [0, N]");
  const long long plane = (long long)c->n * c->n;
  PM_CK(launch_project(rho, c->n, n_slices, out, grid_for((plane + 255) / 256, c->sms, 8), (cudaStream_t)stream),
        "project");
  return PM_OK;
}

int pm_power_spectrum(pm_ctx* c, const float* rho, double box_size, int nbins, double* k_out, double* pk_out,
                      double* modes_out, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!rho || !k_out || !pk_out || !modes_out) return fail(c, PM_ERR_ARG, "null array");
  const int n = c->n;
  if (nbins <= 0) nbins = n / 2 + 1;
  if (nbins < 2 || nbins > n / 2 + 1) return fail(c, PM_ERR_ARG, "nbins must lie in [2, n/2 + 1]");
  if (!(box_size > 0.0)) return fail(c, PM_ERR_ARG, "box size must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  Call k;
  k.sim = base_sim(c, 1);
  k.sim.rho = const_cast<float*>(rho);
  set_prefix(k, 1, n);
  if (int r = prepare_spectral(c, k)) return r;
  if (int r = upload(c, k, st)) return r;
  const Sim* ds = c->d_sim.as<Sim>();
  const int gx = grid_for(k.prefix[PH_X][1], c->sms, 8), gl = grid_for(k.prefix[PH_LINE][1], c->sms, 8);
  const CUtensorMap* maps = c->maps_for ? c->d_maps.as<CUtensorMap>() : nullptr;
  int* err = c->d_err.as<int>();
  PM_CK(spectral_dispatch(SPEC_X_R2C, n, ds, work(c, k, PH_X), gx, st, maps, err), "x r2c");
  PM_CK(spectral_dispatch(SPEC_Y_FWD, n, ds, work(c, k, PH_LINE), gl, st, maps, err), "y fwd");
  PM_CK(spectral_dispatch(SPEC_Z_FWD, n, ds, work(c, k, PH_LINE), gl, st, maps, err), "z fwd");
  const int nb = nbins - 1;
  PM_CK(c->pk_partial.ensure(pk_partial_doubles(nbins) * sizeof(double)), "alloc pk");
  PM_CK(c->pk_out.ensure((size_t)3 * nb * sizeof(double)), "alloc pk");
  PM_CK(launch_power_spectrum(c->spec.as<float2>(), n, spec_pitch(n), nbins, box_size, c->pk_partial.as<double>(),
                              c->pk_out.as<double>(), st),
        "power spectrum");
  c->pk_host.resize((size_t)3 * nb);
  PM_CK(cudaMemcpyAsync(c->pk_host.data(), c->pk_out.p, (size_t)3 * nb * sizeof(double), cudaMemcpyDeviceToHost, st),
        "d2h pk");
  PM_CK(cudaStreamSynchronize(st), "sync");
  for (int b = 0; b < nb; ++b) {
    k_out[b] = c->pk_host[3 * b];
    pk_out[b] = c->pk_host[3 * b + 1];
    modes_out[b] = c->pk_host[3 * b + 2];
  }
  return PM_OK;
}

}  // extern "C"
