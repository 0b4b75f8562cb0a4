# Simulation configuration, read by every module by name (as src/configure_me.py of the
# reference).  The values below are the README workload: 256^3 particles on a 512^3 grid.

###################################################
# General simulation settings
###################################################
N_PARTS          = 256   # particles per side
N_CELLS          = 512   # grid cells per side
BOX_SIZE         = 250   # box side in Mpc/h

N_CPU            = 16    # host threads for the initial-condition FFTs
RANDOM_SEED      = 0     # seed of the Gaussian random field (and of the Zel'dovich jitter)

STEPS            = 1000  # number of time steps between A_INIT and A_END
N_SAVE_FILES     = 100   # number of snapshots
N_PLOTS          = 100   # kept for compatibility (plots are not produced)

PLOT_STEPS       = False
PLOT_PROJECTIONS = False
PLOT_GRF         = False
SAVE_DATA        = False
SAVE_DENSITY     = False
PRINT_STATUS     = True

RESTART          = False # restart from snapshot RESTART_FROM_N
RESTART_FROM_N   = 0

# GPU engine: run the whole time loop resident on the GPU (True) or call the per-step
# drop-in functions from the driver loop like the reference does (False)
RESIDENT         = True

###################################################
# Cosmology settings
###################################################
POWER                  = 0.96
LCDM_TRANSFER_FUNCTION = True

OMEGA_M0               = 0.30
OMEGA_B0               = 0.04
OMEGA_K0               = 0.00
OMEGA_LAMBDA0          = 0.70
H0                     = 0.70
A_INIT                 = 0.02
A_END                  = 1.00
