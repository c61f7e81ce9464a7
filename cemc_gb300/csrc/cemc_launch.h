// Launch arguments and the shared-memory layout of the Monte Carlo kernel,
// computed identically on the host (to size the launch) and on the device.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "cemc_device.cuh"

namespace cemc {

struct RunArgs {
  int n_chains, warps;
  int cl;                  // CTAs per chain (1, or 2 for a thread-block cluster pair)
  int tpw;                 // trials per evaluating warp and round (2: one per half-warp, spin flips)
  int ring_bits;           // log2 of the draw / neighbour-row ring size
  int occ_smem, trk_smem;  // 1: the chain's occupation / swap tracker lives in shared memory
  int stamp_bits;          // log2 of the size of each of the two conflict-stamp tables
  uint32_t *gstamp;        // exact stamp tables in global memory (2 << stamp_bits words per chain), or NULL
  uint64_t seed, n_trials;
  int8_t *occ;
  double *cf, *energy;
  const double *eci, *kT;
  uint64_t *trial;
  cemc_accum *accum;
  int32_t *trk, *loc;
  const int32_t *trk_start, *trk_count;
  int32_t *trace_site;
  int8_t *trace_acc;
  double *trace_de;
  int32_t *status;
  const uint32_t *chain_key;
  const int32_t *accum_slot;
  const uint64_t *chain_trials;
  uint64_t chunk_offset;  // trials of this chain already run by earlier chunks of the same call
  const uint8_t *site_allow;  // move constraints (see cemc_run_desc), NULL = none
  const uint32_t *frozen;
  int max_attempts;
  int accept_first;  // the first trial of the call (chunk offset 0) is accepted whatever its energy change
  int cons;          // 1: the build with the constraint redraw loop and first-move acceptance (one CTA per chain)
};

constexpr int kMaxEval = 16;   // trial-evaluating warps per CTA; two or three more warps are helpers
constexpr int kRoundSlots = 64;  // trial records per round (trials per round <= 60)
constexpr int kPrefetchRounds = 3;  // the fetcher draws this many rounds of trials ahead

// Trials per round of a launch shape.
__host__ __device__ inline int round_trials(int cl, int warps, int tpw) { return cl * warps * tpw; }
// Booker warps per CTA: two when one CTA holds a round of more than 32 trials.
__host__ __device__ inline int n_bookers(int cl, int warps, int tpw) {
  return (cl == 1 && round_trials(cl, warps, tpw) > 32) ? 2 : 1;
}
// Launch bound of every kernel build: at most 16 evaluating warps and three helpers
// (608 threads), which leaves the compiler 102 registers a thread instead of the 64 of a
// 1024-thread bound (wider CTAs were never the faster shape; the bound is worth 2-6 %).
constexpr int kMcMaxThreads = 640;
// Evaluating warps per CTA (larger requests are clamped).
__host__ __device__ inline int max_eval_warps(int cl, int tpw) {
  (void)cl;
  (void)tpw;
  return kMaxEval;
}
// Ring size (log2): more than kPrefetchRounds rounds of trials.
__host__ __device__ inline int ring_bits_for(int cw) { return kPrefetchRounds * cw < 128 ? 7 : 8; }

// Per-trial draw, written by the helper warp: site (flips), Philox words.
struct Draw {
  int32_t site;
  uint32_t w1, w2, w3, w0, x0, x1, pad;
};

struct McLayout {
  size_t cf, eci, w, acc, cfw, coef, bf, terms, lane_term, kind, misc, grp;
  size_t sp_eci, sp_masks, sp_shift, sp_lane;  // spin-basis tables (empty unless n_cl > 0)
  // per-round trial records (two buffers, by round parity), kRoundSlots entries each
  size_t rec, rec_stride, rec_sa, rec_sb, rec_de, rec_ds, rec_acc, rec_la, rec_lb, rec_A, rec_B;
  size_t drow;  // [2][warps * tpw][n_eci] correlation-function changes of this CTA's trials
  size_t cfp;   // spin form: per-lane sums of booked change rows [2][n_eci][32] (int32)
  size_t ftab, geos;  // table form
  size_t draws, rows;
  size_t warp0, warp_stride, warp_part;
  size_t occ, trk, stamp;
  int stamp_bits;
  size_t total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Shared-memory carve-up of mc_kernel for `warps` evaluating warps per CTA.
// Trial-evaluation forms of the kernel.
constexpr int kFormGeneric = 0;  // basis-function products term by term; tracks correlation functions
constexpr int kFormSpin = 1;     // binary +1/-1 basis: bit-packed neighbourhoods
constexpr int kFormTable = 2;    // one lookup per cluster geometry; correlation functions by a final recompute
constexpr int kFormRecycle = 3;  // the generic evaluation with waste-recycled acceptance and running sums

__host__ __device__ inline McLayout mc_layout(const DevGeo &g, int warps, int move, int rsize, int occ_smem,
                                              int trk_smem, int stamp_bits, int n_cl, int n_masks, int ring_bits,
                                              int form, int tpw, bool gstamp = false) {
  const bool spin = form == kFormSpin, table = form == kFormTable;
  McLayout L;
  size_t o = 0;
  const size_t K = (size_t)g.n_eci;
  const size_t S = kRoundSlots;
  L.cf = o;
  o = align16(o + 8 * K);
  L.eci = o;
  o = align16(o + 8 * K);
  L.w = o;
  o = align16(o + 8 * K);
  L.acc = o;  // per-lane running sums of up to two bookers [2][14][32], then singlets at launch start (4), 1/N
  o = align16(o + 8 * (size_t)(2 * (2 + 3 * CEMC_MAX_BF) * 32 + CEMC_MAX_BF + 1));
  L.cfw = o;  // per-booker sums of committed correlation-function changes [2][n_eci]
  o = align16(o + 8 * 2 * K);
  L.coef = o;
  o = align16(o + (size_t)rsize * K);
  L.bf = o;
  o = align16(o + (size_t)rsize * g.n_bf * g.n_sym);
  L.terms = o;
  o = align16(o + 8 * (size_t)g.n_terms);
  L.lane_term = o;  // one block of lane-chunk tables per translation group
  o = align16(o + 4 * (size_t)(g.n_groups > 1 ? g.n_groups : 1) * group_lane_ints(g.n_eci));
  L.kind = o;
  o = align16(o + 2 * K);
  L.misc = o;
  o = align16(o + 4 * 64);
  L.grp = o;  // per translation group: scale (as R), then the table-form geometry ranges
  o = align16(o + 8 * CEMC_MAX_GROUPS + 4 * (CEMC_MAX_GROUPS + 1));
  L.sp_eci = o;
  o = align16(o + 32 * (size_t)n_cl);
  L.sp_masks = o;  // per multi-site term: {mask lo, mask hi, 32-lane shift, 16-lane shift}
  o = align16(o + 16 * (size_t)n_masks);
  L.sp_shift = o;  // (unused)
  L.sp_lane = o;
  if (n_cl > 0) o = align16(o + 4 * (33 + 32 + 17 + 16 + 9 + 8));
  size_t r = 0;
  L.rec_sa = r;
  r += 4 * S;
  L.rec_sb = r;
  r += 4 * S;
  L.rec_la = r;
  r += 4 * S;
  L.rec_lb = r;
  r += 4 * S;
  L.rec_de = r;
  r += (size_t)rsize * S;
  L.rec_ds = r;
  r += (size_t)rsize * S * CEMC_MAX_BF;
  L.rec_acc = r;
  r += S;
  L.rec_A = r;
  r += S;
  L.rec_B = r;
  r += S;
  L.rec_stride = align16(r);
  L.rec = o;
  o = align16(o + 2 * L.rec_stride);
  L.drow = o;  // two buffers (round parity) of [warps * tpw][n_eci] (none in the table form)
  if (!table) o = align16(o + 2 * (size_t)rsize * warps * tpw * K);
  L.cfp = o;
  if (spin) o = align16(o + 4 * 2 * 32 * K);
  L.ftab = o;  // table form: per-chain pattern tables F, then the geometry list
  if (table) o = align16(o + (size_t)rsize * g.tab_len);
  L.geos = o;
  if (table) o = align16(o + 16 * (size_t)g.n_geo);
  const size_t ring = (size_t)1 << ring_bits;
  L.draws = o;
  o = align16(o + sizeof(Draw) * ring);
  L.rows = o;
  if (move == CEMC_MOVE_FLIP) o = align16(o + 4 * ring * g.cpad);
  const size_t vals = (size_t)rsize * g.vals_len * (move == CEMC_MOVE_SWAP ? 2 : 1);
  L.warp_part = align16(vals);
  L.warp_stride = spin ? 0 : align16(L.warp_part + (size_t)rsize * g.n_slots * 32);
  if (table) L.warp_stride = 2 * align16((size_t)g.n_cols + 1);  // species of the two rows of a trial
  L.warp0 = o;
  o = align16(o + L.warp_stride * (size_t)warps);
  L.stamp_bits = stamp_bits;
  L.stamp = o;
  if (!gstamp) o = align16(o + 2 * 4 * ((size_t)1 << stamp_bits));
  L.occ = o;
  if (occ_smem) o = align16(o + (size_t)g.n_sites);
  L.trk = o;
  if (trk_smem) o = align16(o + 8 * (size_t)g.n_sites);
  L.total = o;
  return L;
}

struct SpinDev;
cudaError_t launch_mc(const DevGeo &g, const RunArgs &a, int move, int precision, size_t smem, cudaStream_t st,
                      int form, const SpinDev *spin);
// Clusters of `cl` CTAs (each with `smem` bytes) that can be resident at once; 0 if none.
int max_active_clusters(const DevGeo &g, const RunArgs &a, int move, int precision, size_t smem, int form);

}  // namespace cemc
