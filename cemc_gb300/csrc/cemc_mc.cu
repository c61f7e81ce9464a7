// Fused Metropolis Monte Carlo kernel: trial-move energy change, accept test
// and in-place commit of occupation, correlation functions and energy.
//
// Replaces the reference's per-trial Python -> C++ round trip
// (Montecarlo._mc_step, cemc/mcmc/montecarlo.py:970-1038, calling
// CEUpdater::calculate / undo_changes / clear_history,
// cpp/src/ce_updater.cpp:313-555) by one launch that runs many trials of many
// chains.
//
// One CTA owns one chain for the whole launch; the chain's occupation (int8
// species ids) sits in shared memory when it fits.  A chain is a sequential
// Markov chain, so parallelism inside it comes from speculation.  Each round,
// evaluating warp w computes trial t0 + w against the state at the start of
// the round.  A trial's energy change depends only on the species of its own
// sites and of their neighbour columns, so it stays valid unless an earlier
// ACCEPTED trial of the same round changed one of those sites.  Accepted
// trials stamp their site and its neighbourhood in a shared-memory table with
// (round, trial) marks; warp 0 then reads one stamp per trial, commits the
// longest prefix with no earlier conflicting accept (exactly what sequential
// Metropolis over the same stream does) and the first conflicting trial is
// re-evaluated next round.  When the stamp table is smaller than the
// supercell it is indexed by site & mask: an alias can only report a false
// conflict, which shortens the committed prefix and never changes a result.
// The neighbour relation is symmetric (checked when the geometry is built),
// so "accepted site in my neighbourhood" equals "my site in its neighbourhood".
//
// One extra helper warp runs off the critical path: it precomputes the
// counter-based draws (philox.h) of upcoming trials, prefetches their
// neighbour-table rows from L2/HBM into a shared-memory ring with cp.async two
// rounds ahead (single-site flips, whose site does not depend on the state),
// and folds the previous round's records (double-buffered) into per-lane
// running sums of energy and singlets.  Each evaluating warp adds the
// correlation-function changes of its own committed accepted trials to
// per-warp sums; the correlation functions and the energy are brought up to
// date in FP64 once, at the end of the launch.
#include <cuda_runtime.h>

#include <type_traits>

#include "cemc_device.cuh"
#include "cemc_launch.h"
#include "cemc_spin.h"

namespace cemc {

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// vals of a flip whose neighbour row sits in shared memory.
template <typename R>
__device__ __forceinline__ void gather_smem_row(const DevGeo &g, const int8_t *occ, const R *bf_s, const int32_t *row,
                                                int old_s, int new_s, R *vals, int (&nbr)[4], int lane) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = lane + 32 * j;
    nbr[j] = -1;
    if (c < g.n_cols) {
      const int s = row[c];
      nbr[j] = s;
      const int o = occ[s];
      for (int d = 0; d < g.n_bf; ++d) vals[c * g.n_bf + d] = bf_s[d * g.n_sym + o];
    }
  }
  if (lane == 0) {
    vals[g.one_idx] = (R)1;
    for (int d = 0; d < g.n_bf; ++d) vals[g.one_idx + 1 + d] = bf_s[d * g.n_sym + new_s] - bf_s[d * g.n_sym + old_s];
  }
}

// Spin word of a neighbour row (binary +1/-1 basis): bit c = 1 when column c
// holds the -1 species; one ballot per 32 columns.  `ovr_site` reads as spin
// bit `ovr_bit` (the first half of a swap already applied).
__device__ __forceinline__ void spin_ballot(const DevGeo &g, const int8_t *occ, const int32_t *row, uint32_t xorv,
                                            int ovr_site, uint32_t ovr_bit, uint32_t &lo, uint32_t &hi,
                                            int (&nbr)[4], int lane) {
  uint32_t b0 = 0, b1 = 0;
  nbr[0] = nbr[1] = nbr[2] = nbr[3] = -1;
  if (lane < g.n_cols) {
    const int s = row[lane];
    nbr[0] = s;
    b0 = (s == ovr_site) ? ovr_bit : ((uint32_t)occ[s] ^ xorv);
  }
  if (lane + 32 < g.n_cols) {
    const int s = row[lane + 32];
    nbr[1] = s;
    b1 = (s == ovr_site) ? ovr_bit : ((uint32_t)occ[s] ^ xorv);
  }
  lo = __ballot_sync(kFull, b0);
  hi = __ballot_sync(kFull, b1);
}

// Parities of this lane's multi-site terms, packed 6 bits per cluster-ECI slot.
__device__ __forceinline__ uint32_t spin_lane_parities(const uint2 *masks, const uint8_t *shift, int lo_t, int hi_t,
                                                       uint32_t lo, uint32_t hi) {
  uint32_t packed = 0;
  for (int t = lo_t; t < hi_t; ++t) {
    const uint2 m = masks[t];
    packed += (uint32_t)(__popc((lo & m.x) ^ (hi & m.y)) & 1) << shift[t];
  }
  return packed;
}

// Number of odd-parity multi-site terms of cluster ECI k over the warp.
__device__ __forceinline__ int spin_odd(uint32_t packed, int k, int first) {
  const int sl = k - first;
  const int v = (sl >= 0 && sl < 5) ? (int)((packed >> (6 * sl)) & 63u) : 0;
  return __reduce_add_sync(kFull, v);
}

template <typename R, int MOVE, bool SPIN>
__global__ void __launch_bounds__(1024, 1) mc_kernel(DevGeo g, RunArgs a, SpinDev sd) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr bool SWAP = (MOVE == CEMC_MOVE_SWAP);
  const int W = a.warps;  // evaluating warps; warp W is the helper
  const McLayout L = mc_layout(g, W, MOVE, (int)sizeof(R), a.occ_smem, a.trk_smem, a.stamp_bits, SPIN ? sd.n_cl : 0,
                               SPIN ? sd.n_masks : 0);
  const int chain = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool helper = (warp == W);
  const int N = g.n_sites, n_eci = g.n_eci, cpad = g.cpad;
  const uint32_t hmask = (1u << L.stamp_bits) - 1u;

  double *cf_s = reinterpret_cast<double *>(smem + L.cf);
  double *eci_s = reinterpret_cast<double *>(smem + L.eci);
  double *w_s = reinterpret_cast<double *>(smem + L.w);
  // Running sums of this launch, FP64 in FP64 mode and double-float in FP32
  // mode.  The thermodynamic sums are kept per lane of the helper warp (lane =
  // position of a trial in its round) and the committed correlation-function
  // changes per evaluating warp, so no round needs a cross-lane or cross-warp
  // reduction of them; both are reduced once, in fixed order, in the epilogue.
  constexpr bool DF = (sizeof(R) == 4);
  using A = typename std::conditional<DF, df64, double>::type;
  constexpr int NACC = 2 + 3 * CEMC_MAX_BF;
  constexpr int NBF = SPIN ? 1 : CEMC_MAX_BF;
  A *lacc = reinterpret_cast<A *>(smem + L.acc);  // [NACC][32]
  A *s_start = lacc + NACC * 32;                  // [CEMC_MAX_BF] singlets at launch start, then 1/N
  A *cfw = reinterpret_cast<A *>(smem + L.cfw);   // [W][n_eci]
  R *coef_s = reinterpret_cast<R *>(smem + L.coef);
  R *bf_s = reinterpret_cast<R *>(smem + L.bf);
  uint16_t *terms_s = reinterpret_cast<uint16_t *>(smem + L.terms);
  int32_t *lane_term_s = reinterpret_cast<int32_t *>(smem + L.lane_term);
  int32_t *first_s = lane_term_s + 33;
  int32_t *eci_lane_s = first_s + 32;
  int8_t *kind_s = reinterpret_cast<int8_t *>(smem + L.kind);
  int8_t *dec_s = kind_s + n_eci;
  // misc: [0] committed count, [1] status, [2] species present, [4..12) present ids,
  //       [12..20) site-list starts, [20..28) site-list counts
  int32_t *misc = reinterpret_cast<int32_t *>(smem + L.misc);
  Draw *draws = reinterpret_cast<Draw *>(smem + L.draws);
  int32_t *rows = reinterpret_cast<int32_t *>(smem + L.rows);
  uint32_t *stamp = reinterpret_cast<uint32_t *>(smem + L.stamp);
  unsigned char *rec0 = smem + L.rec;
  unsigned char *wbase = smem + L.warp0 + (size_t)(helper ? 0 : warp) * L.warp_stride;
  R *va = reinterpret_cast<R *>(wbase);
  R *vb = va + g.vals_len;
  R *part = reinterpret_cast<R *>(wbase + L.warp_part);

  SpinEci *sp_eci = reinterpret_cast<SpinEci *>(smem + L.sp_eci);
  uint2 *sp_masks = reinterpret_cast<uint2 *>(smem + L.sp_masks);
  uint8_t *sp_shift = reinterpret_cast<uint8_t *>(smem + L.sp_shift);
  int32_t *sp_lane_term = reinterpret_cast<int32_t *>(smem + L.sp_lane);
  int32_t *sp_lane_first = sp_lane_term + 33;
  const uint32_t xorv = SPIN ? (uint32_t)(sd.minus_id ^ 1) : 0u;  // spin bit = occ ^ xorv (1 = the -1 species)

  int8_t *occ = a.occ_smem ? reinterpret_cast<int8_t *>(smem + L.occ) : a.occ + (size_t)chain * N;
  int32_t *trk = nullptr, *loc = nullptr;
  if (SWAP) {
    trk = a.trk_smem ? reinterpret_cast<int32_t *>(smem + L.trk) : a.trk + (size_t)chain * N;
    loc = a.trk_smem ? trk + N : a.loc + (size_t)chain * N;
  }

  // ---- prologue: stage tables and the chain's state -------------------------
  for (int k = tid; k < n_eci; k += blockDim.x) {
    const int kind = g.eci_kind[k];
    const double e = a.eci[(size_t)chain * n_eci + k];
    cf_s[k] =a.cf[(size_t)chain * n_eci + k];
    eci_s[k] = e;
    w_s[k] = (kind == 2) ? g.eci_w[k] : 0.0;
    coef_s[k] = (R)(kind == 2 ? e * (double)N * g.eci_w[k] : (kind == 1 ? e : 0.0));
    kind_s[k] = (int8_t)kind;
    dec_s[k] = (int8_t)g.eci_dec[k];
    eci_lane_s[2 * k] = g.eci_lane[2 * k];
    eci_lane_s[2 * k + 1] = g.eci_lane[2 * k + 1];
  }
  for (int i = tid; i < g.n_bf * g.n_sym; i += blockDim.x) bf_s[i] = (R)g.bf[i];
  for (int i = tid; i < 33; i += blockDim.x) lane_term_s[i] = g.lane_term[i];
  for (int i = tid; i < 32; i += blockDim.x) first_s[i] = g.lane_first_eci[i];
  {
    const uint2 *src = reinterpret_cast<const uint2 *>(g.terms);
    uint2 *dst = reinterpret_cast<uint2 *>(terms_s);
    for (int i = tid; i < g.n_terms; i += blockDim.x) dst[i] = src[i];
  }
  for (uint32_t i = tid; i <= hmask; i += blockDim.x) stamp[i] = 0u;
  for (int i = tid; i < W * n_eci; i += blockDim.x) cfw[i] = acc_from<A>(0.0);
  for (int i = tid; i < NACC * 32; i += blockDim.x) lacc[i] = acc_from<A>(0.0);
  {
    // zero the change rows of both record buffers (the spin path writes only
    // the entries of cluster and singlet ECIs)
    for (int i = tid; i < 2 * 32 * n_eci; i += blockDim.x) {
      const int buf = i / (32 * n_eci), j = i - buf * 32 * n_eci;
      reinterpret_cast<R *>(rec0 + (size_t)buf * L.rec_stride + L.rec_d)[j] = (R)0;
    }
  }
  if (SPIN) {
    for (int k = tid; k < sd.n_cl; k += blockDim.x) sp_eci[k] = sd.eci[k];
    for (int t = tid; t < sd.n_masks; t += blockDim.x) {
      sp_masks[t] = sd.masks[t];
      sp_shift[t] = sd.shift[t];
    }
    for (int i = tid; i < 33; i += blockDim.x) sp_lane_term[i] = sd.lane_term[i];
    for (int i = tid; i < 32; i += blockDim.x) sp_lane_first[i] = sd.lane_first[i];
  }
  if (a.occ_smem) {
    const int8_t *src = a.occ + (size_t)chain * N;
    for (int i = tid; i < N; i += blockDim.x) occ[i] = src[i];
  }
  if (SWAP && a.trk_smem) {
    const int32_t *st = a.trk + (size_t)chain * N, *sl = a.loc + (size_t)chain * N;
    for (int i = tid; i < N; i += blockDim.x) {
      trk[i] = st[i];
      loc[i] = sl[i];
    }
  }
  if (tid == 0) {
    misc[1] = 0;
    if (SWAP) {
      int np = 0;
      for (int s = 0; s < g.n_sym; ++s) {
        const int cnt = a.trk_count[(size_t)chain * g.n_sym + s];
        misc[12 + s] = a.trk_start[(size_t)chain * g.n_sym + s];
        misc[20 + s] = cnt;
        if (cnt > 0) misc[4 + np++] = s;
      }
      misc[2] = np;
      if (np < 2) misc[1] = CEMC_ERR_STATE;
    }
    for (int b = 0; b < CEMC_MAX_BF; ++b)
      s_start[b] = acc_from<A>(b < g.n_bf ? a.cf[(size_t)chain * n_eci + g.singlet_eci[b]] : 0.0);
    s_start[CEMC_MAX_BF] = acc_from<A>(1.0 / (double)N);
  }

  const double kT = a.kT[chain];
  const float inv_kT = (float)(1.0 / kT);
  const uint32_t key = a.chain_key ? a.chain_key[chain] : (uint32_t)chain;
  uint64_t my_trials = a.n_trials;
  if (a.chain_trials) {
    // this chunk covers trials [chunk_offset, chunk_offset + n_trials) of the call
    const uint64_t total = a.chain_trials[chain];
    my_trials = total <= a.chunk_offset ? 0 : (total - a.chunk_offset < a.n_trials ? total - a.chunk_offset : a.n_trials);
  }
  const uint64_t t_first = a.trial[chain];
  const uint64_t t_end = t_first + my_trials;
  const int acc_row = a.accum_slot ? a.accum_slot[chain] : chain;
  const double e_ref = a.accum ? a.accum[acc_row].e_ref : 0.0;

  // Helper-warp state: energy relative to e_ref and, per singlet, the launch's
  // summed singlet changes (the singlet after a trial is start + sum / N).
  A eoff = acc_from<A>(a.energy[chain] - e_ref);
  A dsum[NBF];
#pragma unroll
  for (int b = 0; b < NBF; ++b) dsum[b] = acc_from<A>(0.0);
  uint64_t n_acc_launch = 0;
  uint64_t fill_end = t_first;

  // Draws (and, for flips, neighbour rows) of trials [fill_end, min(t0 + 3W, t_end)).
  auto prefetch = [&](uint64_t t0) {
    uint64_t want = t0 + 3 * (uint64_t)W;
    if (want > t_end) want = t_end;
    for (uint64_t t = fill_end + lane; t < want; t += 32) {
      const int slot = (int)(t & (kRing - 1));
      const cemc_u32x4 w0 = cemc_trial_draw(a.seed, key, t, 0);
      Draw d;
      d.w0 = w0.v[0];
      d.w1 = w0.v[1];
      d.w2 = w0.v[2];
      d.w3 = w0.v[3];
      d.pad = 0;
      if (SWAP) {
        const cemc_u32x4 w1 = cemc_trial_draw(a.seed, key, t, 1);
        d.x0 = w1.v[0];
        d.x1 = w1.v[1];
        d.site = -1;
      } else {
        d.x0 = d.x1 = 0;
        d.site = (int)cemc_below(w0.v[0], (uint32_t)N);
        const int32_t *src = g.table + (size_t)d.site * cpad;
        int32_t *dst = rows + (size_t)slot * cpad;
        for (int q = 0; q < cpad; q += 4) cp_async16(dst + q, src + q);
      }
      draws[slot] = d;
    }
    if (want > fill_end) fill_end = want;
    cp_async_commit();
  };

  // Fold round records (buffer `rec`, `ks` committed trials) into the running
  // sums.  Lane j handles trial j of the round: one inclusive scan gives the
  // energy and singlet offsets after each trial, and each lane adds its own
  // values to its own sums; a round without accepted trials needs no scan.
  auto book = [&](const unsigned char *rec, int ks) {
    const int8_t *tacc = reinterpret_cast<const int8_t *>(rec + L.rec_acc);
    const R *tder = reinterpret_cast<const R *>(rec + L.rec_der);
    const R *tD = reinterpret_cast<const R *>(rec + L.rec_d);
    const bool mine = lane < ks;
    const bool acc = mine && tacc[lane];
    const unsigned am = __ballot_sync(kFull, acc);
    n_acc_launch += (uint64_t)__popc(am);
    if (!a.accum) return;
    R x = acc ? tder[lane] : (R)0;
    R ds[NBF];
#pragma unroll
    for (int b = 0; b < NBF; ++b) ds[b] = (acc && b < g.n_bf) ? tD[(size_t)lane * n_eci + g.singlet_eci[b]] : (R)0;
    if (am) {
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const R nx = __shfl_up_sync(kFull, x, o);
        R nd[NBF];
#pragma unroll
        for (int b = 0; b < NBF; ++b) nd[b] = __shfl_up_sync(kFull, ds[b], o);
        if (lane >= o) {
          x += nx;
#pragma unroll
          for (int b = 0; b < NBF; ++b) ds[b] += nd[b];
        }
      }
    }
    if (mine) {
      const A ve = acc_add_x(eoff, x);
      lacc[lane] = acc_add(lacc[lane], ve);
      lacc[32 + lane] = acc_add(lacc[32 + lane], acc_mul(ve, ve));
#pragma unroll
      for (int b = 0; b < NBF; ++b) {
        if (b < g.n_bf) {
          const A vs = acc_add(s_start[b], acc_mul(acc_add_x(dsum[b], ds[b]), s_start[CEMC_MAX_BF]));
          A *l = lacc + (2 + b) * 32 + lane;
          l[0] = acc_add(l[0], vs);
          l[CEMC_MAX_BF * 32] = acc_add(l[CEMC_MAX_BF * 32], acc_mul(vs, vs));
          l[2 * CEMC_MAX_BF * 32] = acc_add(l[2 * CEMC_MAX_BF * 32], acc_mul(vs, ve));
        }
      }
    }
    if (am) {
      eoff = acc_add_x(eoff, __shfl_sync(kFull, x, ks - 1));
#pragma unroll
      for (int b = 0; b < NBF; ++b) dsum[b] = acc_add_x(dsum[b], __shfl_sync(kFull, ds[b], ks - 1));
    }
  };

  __syncthreads();
  if (misc[1] != 0) {
    if (tid == 0 && a.status) a.status[chain] = misc[1];
    return;
  }
  if (helper) {
    prefetch(t_first);
    cp_async_wait_all();
  }
  __syncthreads();

  const int n_present = SWAP ? misc[2] : 0;
  // spin path: lane k of every evaluating warp holds cluster ECI k and its coefficient
  SpinEci sp_e{};
  R sp_coef = (R)0;
  unsigned sp_multi = 0;  // cluster ECIs with multi-site terms
  if (SPIN) {
    if (lane < sd.n_cl) {
      sp_e = sp_eci[lane];
      sp_coef = coef_s[sp_e.eci];
    }
    sp_multi = __ballot_sync(kFull, lane < sd.n_cl && sp_e.n_multi > 0);
  }
  uint64_t t0 = t_first;
  uint32_t round = 1;
  int ks_prev = 0;
  while (t0 < t_end) {
    unsigned char *rec = rec0 + (size_t)(round & 1) * L.rec_stride;
    int32_t *tsa = reinterpret_cast<int32_t *>(rec + L.rec_tsa);
    int32_t *tsb = reinterpret_cast<int32_t *>(rec + L.rec_tsb);
    int8_t *tacc = reinterpret_cast<int8_t *>(rec + L.rec_acc);
    R *tder = reinterpret_cast<R *>(rec + L.rec_der);
    R *tD = reinterpret_cast<R *>(rec + L.rec_d);
    if (!helper) {
      // ---- phase A: every evaluating warp computes one trial speculatively ----
      const uint64_t t = t0 + (uint64_t)warp;
      if (t < t_end) {
        const int slot = (int)(t & (kRing - 1));
        const Draw dr = draws[slot];
        int sa, sb = -1, na;
        int nbra[4], nbrb[4] = {-1, -1, -1, -1};
        uint32_t ua, ub;
        uint32_t occ_a_bit = 0, wa_lo = 0, wa_hi = 0, wb_lo = 0, wb_hi = 0;  // spin path
        if (!SWAP) {
          sa = dr.site;
          const int oa = occ[sa];
          const int k = (int)cemc_below(dr.w1, (uint32_t)(g.n_sym - 1));
          na = k + (k >= oa);
          ua = dr.w2;
          ub = dr.w3;
          if (!SPIN) {
            gather_smem_row<R>(g, occ, bf_s, rows + (size_t)slot * cpad, oa, na, va, nbra, lane);
          } else {
            occ_a_bit = (uint32_t)oa ^ xorv;
            spin_ballot(g, occ, rows + (size_t)slot * cpad, xorv, -1, 0u, wa_lo, wa_hi, nbra, lane);
          }
        } else {
          const int ia = (int)cemc_below(dr.w0, (uint32_t)n_present);
          int ib = (int)cemc_below(dr.w1, (uint32_t)(n_present - 1));
          ib += (ib >= ia);
          const int A = misc[4 + ia], B = misc[4 + ib];
          sa = trk[misc[12 + A] + (int)cemc_below(dr.w2, (uint32_t)misc[20 + A])];
          sb = trk[misc[12 + B] + (int)cemc_below(dr.w3, (uint32_t)misc[20 + B])];
          na = B;
          ua = dr.x0;
          ub = dr.x1;
          // first half: site a takes B; second half: site b takes A with a already changed
          if (!SPIN) {
            gather_vals<R>(g, occ, bf_s, sa, A, B, -1, 0, va, nbra, lane);
            gather_vals<R>(g, occ, bf_s, sb, B, A, sa, B, vb, nbrb, lane);
          } else {
            occ_a_bit = (uint32_t)A ^ xorv;
            spin_ballot(g, occ, g.table + (size_t)sa * cpad, xorv, -1, 0u, wa_lo, wa_hi, nbra, lane);
            spin_ballot(g, occ, g.table + (size_t)sb * cpad, xorv, sa, occ_a_bit ^ 1u, wb_lo, wb_hi, nbrb, lane);
          }
        }
        R de;
        if (!SPIN) {
          __syncwarp();
          lane_terms<R, SWAP>(g, terms_s, lane_term_s, va, vb, part, lane);
          __syncwarp();
          de = eci_changes<R, SWAP>(g, eci_lane_s, first_s, kind_s, dec_s, coef_s, part, va, vb,
                                    tD + (size_t)warp * n_eci, lane);
        } else {
          // P_k = sum over the terms of cluster ECI k of the product of the other
          // members' spins; D_k = delta * P_k with delta = -2 s_a the spin change.
          // Lane k evaluates cluster ECI k: its pair terms by popcounts of its shell
          // masks, its multi-site terms from one warp reduction per ECI that has any.
          R *Dw = tD + (size_t)warp * n_eci;
          const int delta = ((occ_a_bit) ? 2 : -2);
          const int t_lo = sp_lane_term[lane], t_hi = sp_lane_term[lane + 1], first = sp_lane_first[lane];
          const uint32_t pa = spin_lane_parities(sp_masks, sp_shift, t_lo, t_hi, wa_lo, wa_hi);
          const uint32_t pb = SWAP ? spin_lane_parities(sp_masks, sp_shift, t_lo, t_hi, wb_lo, wb_hi) : 0u;
          int my_odd = 0;
          for (unsigned mm = sp_multi; mm; mm &= mm - 1) {
            const int k = __ffs(mm) - 1;
            const int sl = k - first;
            int v = (sl >= 0 && sl < 5) ? (int)((pa >> (6 * sl)) & 63u) : 0;
            if (SWAP) v -= (sl >= 0 && sl < 5) ? (int)((pb >> (6 * sl)) & 63u) : 0;
            const int odd = __reduce_add_sync(kFull, v);
            if (lane == k) my_odd = odd;
          }
          int P = 0;
          if (lane < sd.n_cl) {
            if (!SWAP) {
              P = sp_e.n_pairs - 2 * (__popc(wa_lo & sp_e.pair_lo) + __popc(wa_hi & sp_e.pair_hi)) + sp_e.n_multi -
                  2 * my_odd;
            } else {
              // P(a) - P(b after a): the term counts cancel
              P = -2 * (__popc(wa_lo & sp_e.pair_lo) + __popc(wa_hi & sp_e.pair_hi) - __popc(wb_lo & sp_e.pair_lo) -
                        __popc(wb_hi & sp_e.pair_hi)) - 2 * my_odd;
            }
            Dw[sp_e.eci] = (R)(delta * P);
          }
          R sum = warp_sum(sp_coef * (R)P);
          if (sd.singlet_eci >= 0) {
            if (lane == 0) Dw[sd.singlet_eci] = (R)(SWAP ? 0 : delta);
            if (!SWAP) sum += coef_s[sd.singlet_eci];
          }
          de = (R)delta * sum;
        }
        int acc = 0;
        if (lane == 0) {
          acc = metropolis<R>(de, ua, ub, kT, inv_kT);
          tsa[warp] = sa;
          tsb[warp] = SWAP ? sb : na;
          tacc[warp] = (int8_t)acc;
          tder[warp] = de;
        }
        acc = __shfl_sync(kFull, acc, 0);
        if (acc) {
          const uint32_t mark = (round << 5) | (uint32_t)(31 - warp);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (nbra[q] >= 0) atomicMax(&stamp[(uint32_t)nbra[q] & hmask], mark);
            if (SWAP && nbrb[q] >= 0) atomicMax(&stamp[(uint32_t)nbrb[q] & hmask], mark);
          }
          if (lane == 0) {
            atomicMax(&stamp[(uint32_t)sa & hmask], mark);
            if (SWAP) atomicMax(&stamp[(uint32_t)sb & hmask], mark);
          }
        }
      }
    } else {
      // ---- helper: book the previous round, then draw / prefetch ahead ----------
      if (round > 1) book(rec0 + (size_t)((round - 1) & 1) * L.rec_stride, ks_prev);
      prefetch(t0);
      cp_async_wait_prev();
    }
    __syncthreads();

    if (!helper) {
      // ---- phase B: every warp finds the first trial invalidated by an earlier
      // accept (the committed prefix) and commits its own trial if inside it.
      const int nv = (t_end - t0) < (uint64_t)W ? (int)(t_end - t0) : W;
      bool conflict = false;
      if (lane < nv) {
        const uint32_t v = stamp[(uint32_t)tsa[lane] & hmask];
        conflict = ((v >> 5) == round) && ((31u - (v & 31u)) < (uint32_t)lane);
        if (SWAP) {
          const uint32_t v2 = stamp[(uint32_t)tsb[lane] & hmask];
          conflict |= ((v2 >> 5) == round) && ((31u - (v2 & 31u)) < (uint32_t)lane);
        }
      }
      const unsigned cm = __ballot_sync(kFull, conflict);
      const int ks = cm ? (__ffs(cm) - 1) : nv;
      if (lane == 0 && warp < ks) {
        const int sa = tsa[warp];
        if (tacc[warp]) {
          if (!SWAP) {
            occ[sa] = (int8_t)tsb[warp];
          } else {
            const int sb = tsb[warp];
            const int A = occ[sa], B = occ[sb];
            const int la = loc[sa], lb = loc[sb];
            occ[sa] = (int8_t)B;
            occ[sb] = (int8_t)A;
            trk[misc[12 + A] + la] = sb;
            loc[sb] = la;
            trk[misc[12 + B] + lb] = sa;
            loc[sa] = lb;
          }
        }
        if (a.trace_acc) {
          const size_t idx = (size_t)chain * a.n_trials + (size_t)(t0 + warp - t_first);
          a.trace_site[2 * idx] = sa;
          a.trace_site[2 * idx + 1] = tsb[warp];
          a.trace_acc[idx] = tacc[warp];
          a.trace_de[idx] = (double)tder[warp];
        }
      }
      if (warp < ks && tacc[warp]) {
        // this warp's committed accepted trial: add its change row to the warp's sums
        const R *Dw = tD + (size_t)warp * n_eci;
        A *cw = cfw + (size_t)warp * n_eci;
        for (int k = lane; k < n_eci; k += 32) cw[k] = acc_add_x(cw[k], Dw[k]);
      }
      if (warp == 0 && lane == 0) misc[0] = ks;
    }
    __syncthreads();
    const int ks = misc[0];
    t0 += (uint64_t)ks;
    ks_prev = ks;
    ++round;
  }

  if (helper) {
    if (round > 1) book(rec0 + (size_t)((round - 1) & 1) * L.rec_stride, ks_prev);
    cp_async_wait_all();
  }
  __syncthreads();

  // ---- epilogue: write the chain's state back ----------------------------------
  if (a.occ_smem) {
    int8_t *dst = a.occ + (size_t)chain * N;
    for (int i = tid; i < N; i += blockDim.x) dst[i] = occ[i];
  }
  if (SWAP && a.trk_smem) {
    int32_t *st = a.trk + (size_t)chain * N, *sl = a.loc + (size_t)chain * N;
    for (int i = tid; i < N; i += blockDim.x) {
      st[i] = trk[i];
      sl[i] = loc[i];
    }
  }
  // apply the launch's correlation-function changes: the per-warp sums in warp
  // order (exact for integer-valued changes), then one scaling per ECI
  for (int k = tid; k < n_eci; k += blockDim.x) {
    const int kind = kind_s[k];
    double d = 0.0;
    for (int w = 0; w < W; ++w) d += acc_to(cfw[(size_t)w * n_eci + k]);
    if (kind == 2) cf_s[k] = cf_s[k] + d * w_s[k];
    else if (kind == 1) cf_s[k] = cf_s[k] + d / (double)N;
  }
  __syncthreads();
  for (int k = tid; k < n_eci; k += blockDim.x) a.cf[(size_t)chain * n_eci + k] = cf_s[k];
  if (a.accum && tid < NACC) {
    // running sum `tid` over the helper's lanes, in lane order
    const int b = tid < 2 ? 0 : (tid - 2) % CEMC_MAX_BF;
    if (tid < 2 || b < g.n_bf) {
      double v = 0.0;
      for (int l = 0; l < 32; ++l) v += acc_to(lacc[tid * 32 + l]);
      double *sums = &a.accum[acc_row].sum_e;  // sum_e, sum_e2, sum_s[], sum_s2[], sum_se[] in NACC order
      sums[tid] += v;
    }
  }
  if (helper && lane == 0) {
    // energy = N * eci . cf in sorted-name order (ce_updater.cpp:236-242)
    double e = 0.0;
    for (int k = 0; k < n_eci; ++k) e += eci_s[k] * cf_s[k];
    a.energy[chain] = e * (double)(unsigned)N;
    a.trial[chain] = t_end;
    if (a.accum) {
      cemc_accum *ac = a.accum + acc_row;
      ac->n_samples += my_trials;
      ac->n_accept += n_acc_launch;
    }
    if (a.status) a.status[chain] = 0;
  }
}

template <typename R, int MOVE, bool SPIN>
static cudaError_t launch_t(const DevGeo &g, const RunArgs &a, size_t smem, cudaStream_t st, const SpinDev &sd) {
  auto k = mc_kernel<R, MOVE, SPIN>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<a.n_chains, (a.warps + 1) * 32, smem, st>>>(g, a, sd);
  return cudaGetLastError();
}

template <bool SPIN>
static cudaError_t launch_p(const DevGeo &g, const RunArgs &a, int move, int precision, size_t smem, cudaStream_t st,
                            const SpinDev &sd) {
  if (precision == CEMC_PREC_F32)
    return move == CEMC_MOVE_SWAP ? launch_t<float, CEMC_MOVE_SWAP, SPIN>(g, a, smem, st, sd)
                                  : launch_t<float, CEMC_MOVE_FLIP, SPIN>(g, a, smem, st, sd);
  return move == CEMC_MOVE_SWAP ? launch_t<double, CEMC_MOVE_SWAP, SPIN>(g, a, smem, st, sd)
                                : launch_t<double, CEMC_MOVE_FLIP, SPIN>(g, a, smem, st, sd);
}

cudaError_t launch_mc(const DevGeo &g, const RunArgs &a, int move, int precision, size_t smem, cudaStream_t st,
                      const SpinDev *spin) {
  if (spin) return launch_p<true>(g, a, move, precision, smem, st, *spin);
  return launch_p<false>(g, a, move, precision, smem, st, SpinDev{});
}

}  // namespace cemc
