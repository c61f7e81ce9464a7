// Device tables of the binary spin-basis evaluation path of the Monte Carlo
// kernel (mc_kernel<..., SPIN=true> in cemc_mc.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "cemc_launch.h"

#define CEMC_SPIN_MAX_CL 32  // cluster ECIs of a spin-basis geometry
#define CEMC_SPIN_MAX_COLS 64

namespace cemc {

// One cluster ECI in the spin basis: its pair terms folded into one shell
// mask, its other terms spread over the lanes of the warp.
struct SpinEci {
  int32_t eci;        // index in the sorted ECI list
  int32_t n_pairs;    // pair terms folded into pair_lo / pair_hi
  uint32_t pair_lo, pair_hi;
  int32_t n_multi;    // terms with two or more other members
  int32_t pad0, pad1, pad2;
};

// Device tables of the spin path.  The n_masks multi-site terms are sorted by
// cluster ECI and cut into 32 contiguous lane ranges [lane_term[l],
// lane_term[l+1]); term t of lane l adds its parity at bit shift[t] = 6 * (its
// cluster-ECI index - lane_first[l]) of a per-lane packed counter (at most 5
// ECIs and 63 terms per lane, checked on the host).
struct SpinDev {
  int n_cl, n_masks, minus_id, singlet_eci;
  const SpinEci *eci;        // [n_cl]
  const uint2 *masks;        // [n_masks] (lo, hi) column masks
  const uint8_t *shift;      // [n_masks]
  const int32_t *lane_term;  // [33]
  const int32_t *lane_first; // [32]
  // Half-warp form (one flip per 16 lanes): the same terms cut into 16 lane
  // ranges; usable when half_ok (at most 16 cluster ECIs, counters fit).
  int half_ok;
  const uint8_t *half_shift;       // [n_masks]
  const int32_t *half_lane_term;   // [17]
  const int32_t *half_lane_first;  // [16]
  // Quarter-warp form (one flip per 8 lanes): the terms cut into 8 lane ranges; usable when
  // qtr_ok (at most 8 cluster ECIs, at most 255 terms per ECI, counters fit).
  int qtr_ok;
  const uint8_t *qtr_shift;       // [n_masks]
  const int32_t *qtr_lane_term;   // [9]
  const int32_t *qtr_lane_first;  // [8]
};

}  // namespace cemc
