/*
 * pm_gb300.h -- C ABI of the GB300 particle-mesh engine (libpm_gb300.so).
 *
 * The drop-in entry points replace, one for one, the functions of the per-step hot
 * path of grkooij/Cosmological-Particle-Mesh-Simulation (citations are path:line in
 * that project).  Sizes and cosmology come from a pm_config that mirrors
 * src/configure_me.py.  Arrays follow the reference's layouts:
 *
 *   positions, velocities   float32, (3, np) row-major: x[np], then y[np], then z[np]
 *   density, potential,     float32, (N, N, N) indexed [z][y][x]
 *   fourier grid
 *
 * All array arguments are DEVICE pointers unless the name says host; `stream` is a
 * cudaStream_t (NULL = legacy default stream).  Every call returns PM_OK or a
 * nonzero status; pm_last_error() returns the message of the last failure.  The
 * caller owns all arrays it passes; a context owns its scratch memory and tables.
 * Contexts are not thread-safe: use one per host thread.
 */
#ifndef PM_GB300_H
#define PM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PM_OK 0
#define PM_ERR_ARG 1      /* invalid argument or unsupported size */
#define PM_ERR_CUDA 2     /* CUDA runtime error */
#define PM_ERR_OOM 3      /* device allocation failed */
#define PM_ERR_DEVICE 4   /* device-side check failed (see pm_check_device) */
#define PM_ERR_ADMIT 5    /* batch admission refused: memory cap */

/* device check bits reported by pm_check_device */
#define PM_DEV_CELL_RANGE 1  /* a particle coordinate was not finite / off grid */
#define PM_DEV_SOURCE_ROW 2  /* deposit found a particle outside its tile (unsorted input) */
#define PM_DEV_NONFINITE 4   /* kick/drift produced a non-finite value */

/* flags of pm_config */
#define PM_FLAG_FIX_COSMO_F 1  /* f(a) with Omega_m in its slot; the reference passes H0
                                  there (src/integrate.py:12) and is followed by default */
#define PM_FLAG_KEEP_DENSITY 2 /* batch: keep the density grid apart from the potential */
#define PM_FLAG_SPECTRAL_GRADIENT 4 /* pm_step / pm_step_host: the force from three force grids,
                                       -i sin(k_d) phi_k transformed back (the spectral form of
                                       the central difference of src/integrate.py:84-92, equal
                                       up to rounding), instead of 32 potential taps */

/* Mirrors src/configure_me.py:7-40 (plotting / saving switches omitted). */
typedef struct pm_config {
  int n_cells;          /* N_CELLS, grid cells per side (configure_me.py:8) */
  int n_parts;          /* N_PARTS, particles per side (configure_me.py:7) */
  double box_size;      /* BOX_SIZE in Mpc/h (configure_me.py:9) */
  double omega_m0;      /* OMEGA_M0 (configure_me.py:34) */
  double omega_b0;      /* OMEGA_B0 (configure_me.py:35) */
  double omega_k0;      /* OMEGA_K0 (configure_me.py:36) */
  double omega_lambda0; /* OMEGA_LAMBDA0 (configure_me.py:37) */
  double h0;            /* H0 (configure_me.py:38) */
  double a_init;        /* A_INIT (configure_me.py:39) */
  double a_end;         /* A_END (configure_me.py:40) */
  int steps;            /* STEPS (configure_me.py:14) */
  int flags;            /* PM_FLAG_* */
} pm_config;

typedef struct pm_ctx pm_ctx;

/* ---- context ------------------------------------------------------------------- */
int pm_ctx_create(const pm_config* cfg, int device, pm_ctx** out);
void pm_ctx_destroy(pm_ctx* ctx);
const char* pm_last_error(const pm_ctx* ctx);
/* Synchronises `stream`, returns (and clears) the device check bits in *bits. */
int pm_check_device(pm_ctx* ctx, void* stream, int* bits);
/* Grid sizes the kernels support (N = 2^a 3^b, 16 <= N <= 1024, N % 8 == 0 or N = 24). */
int pm_supported_n(int n);

/* ---- drop-in hot path ----------------------------------------------------------- */
/* src/density.py:7-48  density(positions, mass) -> grid.
   Deterministic: cell-key radix sort + tiled integer-accumulated CIC deposit. */
int pm_density(pm_ctx* ctx, const float* positions, long long np, double mass, float* rho,
               void* stream);

/* src/fourier_utils.py:5-16  fourier_grid() -> 1/sum(sin^2(k/2)), k=0 entry 0. */
int pm_fourier_grid(pm_ctx* ctx, float* fgrid, void* stream);

/* src/potential.py:7-29  potential(density, fgrid, a) -> phi.
   fgrid == NULL evaluates the reference Green function in-kernel (no table read). */
int pm_potential(pm_ctx* ctx, const float* rho, const float* fgrid, double a, float* phi,
                 void* stream);

/* src/integrate.py:15-97  integrate(positions, velocities, a_val, f_a1, da, potentials);
   positions and velocities are updated in place. */
int pm_integrate(pm_ctx* ctx, float* positions, float* velocities, long long np, double a,
                 double f_a1, double da, const float* phi, void* stream);

/* src/integrate.py:9-13  advance_time(density, positions, velocities, fgrid, a, da);
   positions and velocities are updated in place. */
int pm_advance_time(pm_ctx* ctx, const float* rho, float* positions, float* velocities,
                    long long np, const float* fgrid, double a, double da, void* stream);

/* src/pmesh.py:60-61  loop body: rho = density(positions, mass);
   advance_time(rho, positions, velocities, fgrid, a, da).  rho_out may be NULL. */
int pm_step(pm_ctx* ctx, float* positions, float* velocities, long long np, double mass,
            double a, double da, float* rho_out, void* stream);

/* Same as pm_step on HOST arrays (pinned for full speed): copies in, steps, copies out. */
int pm_step_host(pm_ctx* ctx, float* h_positions, float* h_velocities, long long np,
                 double mass, double a, double da, void* stream);

/* src/cosmology.py:20-27  f(a, [om, ol, ok]). */
double pm_cosmo_f(double a, double om, double ol, double ok);

/* Cell keys of the deposit ordering and their stable sort (bit-exact integer work):
   keys_out[i] = key of particle i; sorted_keys / perm = the sorted keys and the
   particle index of each sorted entry.  Any output may be NULL. */
int pm_sort_keys(pm_ctx* ctx, const float* positions, long long np, unsigned* keys_out,
                 unsigned* sorted_keys, unsigned* perm, void* stream);

/* src/plot_helper.py:65-72  project(rho, n_slices): out[y][x] = sum of rho[i][y][x] over the
   first n_slices planes (float64, N x N, device). */
int pm_project(pm_ctx* ctx, const float* rho, int n_slices, double* out, void* stream);

/* Matter power spectrum of a density grid (no counterpart in the reference; the
   accuracy statistic of a run): delta = rho / mean(rho) - 1, P(k) = <|delta_k|^2> box^3 / N^6
   averaged over integer shells b = floor(|m| + 0.5) of the mode index m, 0 < b < nbins
   (nbins <= N/2 + 1; 0 selects N/2 + 1); rfft modes with 0 < kx < N/2 count twice.
   Writes nbins - 1 entries to each HOST array: shell k (h/Mpc, the mean |k| of its modes),
   P(k) ((Mpc/h)^3) and the weighted mode count.  Deterministic; returns after completion. */
int pm_power_spectrum(pm_ctx* ctx, const float* rho, double box_size, int nbins, double* k_out,
                      double* pk_out, double* modes_out, void* stream);

/* The CIC deposit of pm_density for callers that cannot allocate device memory: hosts whose
   device memory is carved up up front by a pool or an arena (a library that allocates on
   its own fails there or breaks the host's accounting), latency-critical loops that cannot
   take the synchronisation cudaMalloc / cudaFree can imply, plugin hosts that hand every
   buffer to their plugins.  No counterpart in the reference.  The caller passes the
   positions and the density grid; all scratch lives in one static device array of the
   library (about 4.3 MB per GPU that loads the library, held until the process exits).
   Limits: at most 262,144 particles and n_cells <= 128; larger requests return PM_ERR_ARG
   and do nothing.  Calls no cudaMalloc, cudaFree or other allocating routine.  The first
   call on a device sets up (with that device current, thread-safe): it looks up the array's
   device address with cudaGetSymbolAddress and sets kernel attributes; make that first call
   before any stream capture.  Every call shares the array and rewrites all of it that it
   reads, so calls that overlap on the GPU race; particles with non-finite or off-grid
   coordinates are skipped without a report. */
int pm_density_noalloc(const float* positions, long long np, int n_cells, double mass, float* rho,
                       void* stream);

/* ---- initial conditions on the device -------------------------------------------- */
/* Parameters of src/gaussian_random_field.py and of the Zel'dovich jitter. */
typedef struct pm_ic_params {
  double power;                       /* POWER (configure_me.py:31) */
  int lcdm_transfer;                  /* LCDM_TRANSFER_FUNCTION (configure_me.py:32) */
  unsigned long long jitter_state[2]; /* numpy PCG64(RANDOM_SEED) 128-bit state: high, low word */
  unsigned long long jitter_inc[2];   /* its increment: high, low word */
} pm_ic_params;

typedef struct pm_ics pm_ics;

/* Scratch and tables for N_PARTS^3 initial conditions (N_PARTS: a pm_supported_n size). */
int pm_ics_create(int n_parts, int device, pm_ics** out);
void pm_ics_destroy(pm_ics* g);
const char* pm_ics_last_error(const pm_ics* g);
/* src/gaussian_random_field.py:9-123 then src/zeldovich.py:10-100 on the device.
   u, v: the N_PARTS^3 accepted uniform pairs of the reference's rejection loop
   (gaussian_random_field.py:35-50), float32.  Writes positions and velocities (3, N_PARTS^3)
   and, when grf != NULL, the random field (N_PARTS^3).  The jitter (uniform in [-2, 2),
   zeldovich.py:89-91) is numpy's PCG64 stream from jitter_state / jitter_inc: x draws, then
   y, then z.  Device pointers; returns after the work on `stream` has completed. */
int pm_ics_generate(pm_ics* g, const pm_config* cfg, const pm_ic_params* ic, const float* u,
                    const float* v, float* positions, float* velocities, float* grf, void* stream);

/* ---- resident engine: batches of simulations ------------------------------------ */
typedef struct pm_batch pm_batch;

/* mem_cap_bytes = 0: no cap.  Simulations advance together, one launch per phase. */
int pm_batch_create(int device, size_t mem_cap_bytes, pm_batch** out);
void pm_batch_destroy(pm_batch* b);
const char* pm_batch_last_error(const pm_batch* b);
/* Device bytes a simulation of this configuration holds while resident. */
size_t pm_sim_footprint(const pm_config* cfg);
/* Admits a simulation from absolute positions/velocities (3, N_PARTS^3) at cfg->a_init;
   on_device selects device or host input arrays (device arrays must be complete: work that
   writes them on another stream has finished).  The state is stored in the row order of the
   particles' cells (a counting sort of their rows), as every later step leaves it.  The arrays
   are no longer used when this returns.  It waits for the steps already enqueued, not for the
   device as a whole.  PM_ERR_ADMIT if over the cap. */
int pm_batch_add(pm_batch* b, const pm_config* cfg, const float* positions,
                 const float* velocities, int on_device, int* sim_id);
/* 1 if pm_batch_add of this configuration would pass the memory cap now, else 0. */
int pm_batch_admits(pm_batch* b, const pm_config* cfg);
/* Advances every active simulation by up to nsteps steps (a simulation stops after the
   src/pmesh.py:56 loop count).  Work is enqueued on `stream` (CUDA graphs); with a NULL
   stream the call returns after the work has finished.  A simulation that has run its last
   step leaves the batch (its final state is extracted on `stream`). */
int pm_batch_step(pm_batch* b, int nsteps, void* stream);
/* Copies a simulation's state out (absolute positions in particle order). */
int pm_batch_get(pm_batch* b, int sim_id, float* positions, float* velocities, int to_device,
                 double* a, int* steps_done, void* stream);
/* src/density.py:7-48 on a resident simulation: the CIC density of its current state into
   rho (device, N_CELLS^3, [z][y][x]), the grid src/save_data.py:17-18 writes when
   SAVE_DENSITY is set.  Deterministic (the deposit of pm_batch_step's step, written out). */
int pm_batch_density(pm_batch* b, int sim_id, float* rho, void* stream);
/* 1 while the simulation still has steps to run or its last steps are still running on the
   device, 0 once its final state is complete, <0 if unknown id. */
int pm_batch_active(pm_batch* b, int sim_id);
int pm_batch_remove(pm_batch* b, int sim_id);
int pm_batch_set_graphs(pm_batch* b, int enable);
/* Device check bits of the batch (synchronises). */
int pm_batch_check(pm_batch* b, void* stream, int* bits);
/* Runs up to nsteps steps with direct launches and CUDA events between phases, and
   writes the mean milliseconds of each phase to phase_ms[0..9]: sort, row starts,
   deposit, x R2C, y forward, z Green, y inverse, x C2R, kick/drift, coefficients. */
int pm_batch_profile(pm_batch* b, int nsteps, float* phase_ms, int nphase, void* stream);
/* Kernel launches per step for the resident simulations (-1 on error). */
int pm_batch_launches_per_step(pm_batch* b);
/* The launch schedule of each grid size is tuned on the batch's own data when a plan meets a
   size (and class of work volume) it has not timed before in this process: deposit fused with
   the x R2C or separate, CTAs per SM of the fused deposit, of the x passes and of the kick.  Every candidate gives bit-identical results.  enable = 0 keeps
   the defaults (and schedules already tuned).  No counterpart in the reference: its FFTs are
   planned by FFTW (src/potential.py:20,27). */
int pm_batch_set_autotune(pm_batch* b, int enable);
/* The current plan's schedule: 4 ints per grid size (n, deposit mode 0 fused dense-first /
   1 fused index order / 2 separate, fused-deposit CTAs per SM, x-pass CTAs per SM), then
   (0, kick CTAs per SM, 1 if tuned, 0).  Returns the ints written (-1 on error). */
int pm_batch_schedule(pm_batch* b, int* out, int cap);
/* Host seconds the batch has spent so far (out[0..n-1], n <= 6): admissions, planning, CUDA
   graph capture and instantiation, retirements, tuning (pm_batch_set_autotune), and the time
   planning waited for the device to finish reading an earlier plan's uploads (back-pressure
   from enqueued steps; not counted in planning). */
int pm_batch_host_seconds(pm_batch* b, double* out, int n);

#ifdef __cplusplus
}
#endif
#endif /* PM_GB300_H */
