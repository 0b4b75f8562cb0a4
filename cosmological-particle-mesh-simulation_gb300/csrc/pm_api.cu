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
  const void* maps_for = nullptr;     // spectrum the device tensor maps describe
  DBuf row_start, spec, phi, rho;     // scratch grids
  DBuf hpos, hvel;                    // device copies for pm_step_host
  DBuf pk_partial, pk_out;            // power spectrum scratch
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

int deposit(pm_ctx* c, Call& k, unsigned* perm, unsigned* skeys, cudaStream_t st) {
  const long long nrows = (long long)c->n * c->n;
  PM_CK(c->row_start.ensure((nrows + 1) * sizeof(unsigned)), "alloc rows");
  PM_CK(launch_row_start(skeys, k.sim.np, k.sim.xbits, (unsigned)nrows, c->row_start.as<unsigned>(), st),
        "rows");
  PM_CK(launch_deposit(c->d_sim.as<Sim>(), work(c, k, PH_DEP), k.parts, perm, c->row_start.as<unsigned>(),
                       POS_ABS, c->d_err.as<int>(), grid_for(k.prefix[PH_DEP][1], c->sms, 8),
                       deposit_smem_bytes(c->n, TILE_Y, TILE_Z), st),
        "deposit");
  return PM_OK;
}

int spectral(pm_ctx* c, Call& k, bool table, cudaStream_t st, bool skip_r2c = false) {
  const Sim* ds = c->d_sim.as<Sim>();
  const int n = c->n;
  const int gx = grid_for(k.prefix[PH_X][1], c->sms, 8), gl = grid_for(k.prefix[PH_LINE][1], c->sms, 8);
  const CUtensorMap* maps = c->maps_for ? c->d_maps.as<CUtensorMap>() : nullptr;
  int* err = c->d_err.as<int>();
  if (!skip_r2c) PM_CK(spectral_dispatch(SPEC_X_R2C, n, ds, work(c, k, PH_X), gx, st, maps, err), "x r2c");
  PM_CK(spectral_dispatch(SPEC_Y_FWD, n, ds, work(c, k, PH_LINE), gl, st, maps, err), "y fwd");
  PM_CK(spectral_dispatch(table ? SPEC_Z_TABLE : SPEC_Z_GREEN, n, ds, work(c, k, PH_LINE), gl, st, maps, err),
        "z green");
  PM_CK(spectral_dispatch(SPEC_Y_INV, n, ds, work(c, k, PH_LINE), gl, st, maps, err), "y inv");
  PM_CK(spectral_dispatch(SPEC_X_C2R, n, ds, work(c, k, PH_X), gx, st, maps, err), "x c2r");
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
  c->d_maps.release();
  c->row_start.release();
  c->spec.release();
  c->phi.release();
  c->rho.release();
  c->hpos.release();
  c->hvel.release();
  c->pk_partial.release();
  c->pk_out.release();
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
  k.sim.rho = rho;
  k.sim.mass_scale = (float)(mass / (double)(1u << PM_FIX_BITS));
  set_prefix(k, np, c->n);
  k.parts = abs_parts(const_cast<float*>(positions), nullptr, np);
  if (int r = upload(c, k, st)) return r;
  unsigned *perm = nullptr, *skeys = nullptr;
  if (int r = sort_particles(c, k, st, &perm, &skeys)) return r;
  return deposit(c, k, perm, skeys, st);
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
  k.sim.phi = const_cast<float*>(phi);
  set_kick(k.sim, a, f_a1, da);
  set_prefix(k, np, c->n);
  k.parts = abs_parts(positions, velocities, np);
  if (int r = upload(c, k, st)) return r;
  unsigned *perm = nullptr, *skeys = nullptr;
  if (int r = sort_particles(c, k, st, &perm, &skeys)) return r;
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

int pm_step(pm_ctx* c, float* positions, float* velocities, long long np, double mass, double a, double da,
            float* rho_out, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!positions || !velocities) return fail(c, PM_ERR_ARG, "null array");
  if (int r = check_np(c, np)) return r;
  if (!(a > 0.0)) return fail(c, PM_ERR_ARG, "scale factor must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t gb = (size_t)c->n * c->n * c->n * sizeof(float);
  float* rho = rho_out;
  if (!rho) {
    PM_CK(c->rho.ensure(gb), "alloc rho");
    rho = c->rho.as<float>();
  }
  PM_CK(c->phi.ensure(gb), "alloc phi");
  Call k;
  k.sim = base_sim(c, np);
  k.sim.rho = rho;
  k.sim.phi = c->phi.as<float>();
  k.sim.mass_scale = (float)(mass / (double)(1u << PM_FIX_BITS));
  set_green(c, k.sim, a);
  set_kick(k.sim, a, f_step(c, a, da), da);
  set_prefix(k, np, c->n);
  k.parts = abs_parts(positions, velocities, np);
  if (int r = prepare_spectral(c, k)) return r;
  if (int r = upload(c, k, st)) return r;
  unsigned *perm = nullptr, *skeys = nullptr;
  if (int r = sort_particles(c, k, st, &perm, &skeys)) return r;
  if (!rho_out && deposit_r2c_supported(c->n)) {
    // the density is not requested: deposit straight into the x-transformed spectrum
    const long long nrows = (long long)c->n * c->n;
    PM_CK(c->row_start.ensure((nrows + 1) * sizeof(unsigned)), "alloc rows");
    PM_CK(launch_row_start(skeys, np, k.sim.xbits, (unsigned)nrows, c->row_start.as<unsigned>(), st), "rows");
    PM_CK(deposit_r2c_dispatch(c->n, c->d_sim.as<Sim>(), work(c, k, PH_DEP), k.parts, perm,
                               c->row_start.as<unsigned>(), POS_ABS, c->d_err.as<int>(),
                               grid_for(k.prefix[PH_DEP][1], c->sms, deposit_r2c_ctas_per_sm(c->n)), st),
          "fused deposit");
    if (int r = spectral(c, k, false, st, true)) return r;
    return kick(c, k, perm, st);
  }
  if (int r = deposit(c, k, perm, skeys, st)) return r;
  if (int r = spectral(c, k, false, st)) return r;
  return kick(c, k, perm, st);
}

int pm_step_host(pm_ctx* c, float* h_positions, float* h_velocities, long long np, double mass, double a,
                 double da, void* stream) {
  if (!c) return PM_ERR_ARG;
  if (!h_positions || !h_velocities) return fail(c, PM_ERR_ARG, "null array");
  if (int r = check_np(c, np)) return r;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t pb = (size_t)3 * np * sizeof(float);
  PM_CK(c->hpos.ensure(pb), "alloc positions");
  PM_CK(c->hvel.ensure(pb), "alloc velocities");
  PM_CK(cudaMemcpyAsync(c->hpos.p, h_positions, pb, cudaMemcpyHostToDevice, st), "h2d positions");
  PM_CK(cudaMemcpyAsync(c->hvel.p, h_velocities, pb, cudaMemcpyHostToDevice, st), "h2d velocities");
  if (int r = pm_step(c, c->hpos.as<float>(), c->hvel.as<float>(), np, mass, a, da, nullptr, stream)) return r;
  PM_CK(cudaMemcpyAsync(h_positions, c->hpos.p, pb, cudaMemcpyDeviceToHost, st), "d2h positions");
  PM_CK(cudaMemcpyAsync(h_velocities, c->hvel.p, pb, cudaMemcpyDeviceToHost, st), "d2h velocities");
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
