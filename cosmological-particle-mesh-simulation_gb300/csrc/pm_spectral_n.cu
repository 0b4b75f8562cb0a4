// One grid size of the spectral kernels: compiled once per N with -DPM_N=<N>.
#include "pm_spectral.cuh"

#ifndef PM_N
#error "compile with -DPM_N=<grid size>"
#endif

namespace pm {
template cudaError_t spectral_launch<PM_N>(SpecKind, const Sim*, Work, int, cudaStream_t, const CUtensorMap*, int*);
template cudaError_t deposit_r2c_launch<PM_N>(const Sim*, Work, Parts, const unsigned*, const unsigned*, int, int*,
                                              unsigned*, const unsigned*, int, cudaStream_t);
}
