// Host-side launchers of the CE Monte Carlo kernels.
#pragma once
#include <cuda_runtime.h>

#include "cemc_launch.h"

namespace cemc {

// Capacity (doubles) of the fixed scratch array behind cemc_recompute_noalloc.
constexpr size_t kNoAllocScratchDoubles = (size_t)1 << 20;
// Device address of that array on the current device (resolved once per device).
double *noalloc_scratch(cudaError_t *err);

size_t recompute_blocks(const DevGeo &g);
size_t warp_kernel_smem(const DevGeo &g);
cudaError_t launch_recompute(const DevGeo &g, int n_chains, const int8_t *occ, const double *eci, double *cf,
                             double *energy, double *scratch, cudaStream_t st);
cudaError_t launch_apply(const DevGeo &g, int8_t *occ, double *cf, double *energy, const double *eci, int n,
                         const int32_t *sites, const int8_t *old_sym, const int8_t *new_sym, int32_t *status,
                         cudaStream_t st);
cudaError_t launch_delta(const DevGeo &g, const int8_t *occ, const double *eci, int move, int sa, int sb, int na,
                         double *de, double *dcf, cudaStream_t st);
cudaError_t launch_energy(const DevGeo &g, int n_chains, const double *eci, const double *cf, double *energy,
                          cudaStream_t st);
cudaError_t launch_pt(int n, int direction, uint64_t seed, uint64_t round, const double *energy, double *kT,
                      int32_t *replica_of, int32_t *position_of, int32_t *n_accept, cudaStream_t st);

}  // namespace cemc
