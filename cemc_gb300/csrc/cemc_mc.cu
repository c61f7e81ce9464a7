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
// and folds the previous round's accepted changes into the FP64 correlation
// functions, energy and running sums (double-buffered trial records).
#include <cuda_runtime.h>

#include "cemc_device.cuh"
#include "cemc_launch.h"

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

template <typename R, int MOVE>
__global__ void __launch_bounds__(1024, 1) mc_kernel(DevGeo g, RunArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr bool SWAP = (MOVE == CEMC_MOVE_SWAP);
  const int W = a.warps;  // evaluating warps; warp W is the helper
  const McLayout L = mc_layout(g, W, MOVE, (int)sizeof(R), a.occ_smem, a.trk_smem, a.stamp_bits);
  const int chain = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool helper = (warp == W);
  const int N = g.n_sites, n_eci = g.n_eci, cpad = g.cpad;
  const uint32_t hmask = (1u << L.stamp_bits) - 1u;

  double *cf_s = reinterpret_cast<double *>(smem + L.cf);
  double *eci_s = reinterpret_cast<double *>(smem + L.eci);
  double *w_s = reinterpret_cast<double *>(smem + L.w);
  double *acc_s = reinterpret_cast<double *>(smem + L.acc);  // 2 + 3 * CEMC_MAX_BF running sums of this launch
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
    cf_s[k] = a.cf[(size_t)chain * n_eci + k];
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
    for (int i = 0; i < 2 + 3 * CEMC_MAX_BF; ++i) acc_s[i] = 0.0;
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

  // Helper-warp state.
  double energy = a.energy[chain];
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

  // Fold round records (buffer `rec`, `ks` committed trials) into the FP64 state.
  auto book = [&](const unsigned char *rec, int ks) {
    const int8_t *tacc = reinterpret_cast<const int8_t *>(rec + L.rec_acc);
    const R *tder = reinterpret_cast<const R *>(rec + L.rec_der);
    const R *tD = reinterpret_cast<const R *>(rec + L.rec_d);
    const bool mine = lane < ks;
    const bool acc = mine && tacc[lane];
    n_acc_launch += (uint64_t)__popc(__ballot_sync(kFull, acc));
    const R X = warp_scan_incl<R>(acc ? tder[lane] : (R)0, lane);  // energy offset after trial `lane`
    const R x_tot = __shfl_sync(kFull, X, ks - 1);
    if (a.accum) {
      const R sX = warp_sum(mine ? X : (R)0);
      const R sX2 = warp_sum(mine ? X * X : (R)0);
      const double ea = energy - e_ref;
      if (lane == 0) {
        acc_s[0] += (double)ks * ea + (double)sX;
        acc_s[1] += (double)ks * ea * ea + 2.0 * ea * (double)sX + (double)sX2;
      }
      for (int b = 0; b < g.n_bf; ++b) {
        const int kb = g.singlet_eci[b];
        const R DS = warp_scan_incl<R>(acc ? tD[lane * n_eci + kb] : (R)0, lane);  // N * singlet offset
        const R sD = warp_sum(mine ? DS : (R)0);
        const R sD2 = warp_sum(mine ? DS * DS : (R)0);
        const R sDX = warp_sum(mine ? DS * X : (R)0);
        if (lane == 0) {
          const double s0 = cf_s[kb], inv_n = 1.0 / (double)N;
          acc_s[2 + b] += (double)ks * s0 + (double)sD * inv_n;
          acc_s[2 + CEMC_MAX_BF + b] += (double)ks * s0 * s0 + 2.0 * s0 * (double)sD * inv_n +
                                        (double)sD2 * inv_n * inv_n;
          acc_s[2 + 2 * CEMC_MAX_BF + b] += (double)ks * s0 * ea + s0 * (double)sX + ea * (double)sD * inv_n +
                                            (double)sDX * inv_n;
        }
      }
    }
    __syncwarp();
    for (int k = lane; k < n_eci; k += 32) {
      const int kind = kind_s[k];
      if (kind == 0) continue;
      R dsum = (R)0;
      for (int j = 0; j < ks; ++j)
        if (tacc[j]) dsum += tD[j * n_eci + k];
      cf_s[k] = (kind == 2) ? cf_s[k] + (double)dsum * w_s[k] : cf_s[k] + (double)dsum / (double)N;
    }
    energy += (double)x_tot;
    __syncwarp();
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
        if (!SWAP) {
          sa = dr.site;
          const int oa = occ[sa];
          const int k = (int)cemc_below(dr.w1, (uint32_t)(g.n_sym - 1));
          na = k + (k >= oa);
          ua = dr.w2;
          ub = dr.w3;
          gather_smem_row<R>(g, occ, bf_s, rows + (size_t)slot * cpad, oa, na, va, nbra, lane);
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
          gather_vals<R>(g, occ, bf_s, sa, A, B, -1, 0, va, nbra, lane);
          gather_vals<R>(g, occ, bf_s, sb, B, A, sa, B, vb, nbrb, lane);
        }
        __syncwarp();
        lane_terms<R, SWAP>(g, terms_s, lane_term_s, va, vb, part, lane);
        __syncwarp();
        const R de = eci_changes<R, SWAP>(g, eci_lane_s, first_s, kind_s, dec_s, coef_s, part, va, vb,
                                          tD + (size_t)warp * n_eci, lane);
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

    if (warp == 0) {
      // ---- phase B: first trial invalidated by an earlier accept; commit the prefix --
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
      if (lane < ks && tacc[lane]) {
        const int sa = tsa[lane];
        if (!SWAP) {
          occ[sa] = (int8_t)tsb[lane];
        } else {
          const int sb = tsb[lane];
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
      if (a.trace_acc && lane < ks) {
        const size_t idx = (size_t)chain * a.n_trials + (size_t)(t0 + lane - t_first);
        a.trace_site[2 * idx] = tsa[lane];
        a.trace_site[2 * idx + 1] = tsb[lane];
        a.trace_acc[idx] = tacc[lane];
        a.trace_de[idx] = (double)tder[lane];
      }
      if (lane == 0) misc[0] = ks;
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
  for (int k = tid; k < n_eci; k += blockDim.x) a.cf[(size_t)chain * n_eci + k] = cf_s[k];
  if (helper && lane == 0) {
    // energy = N * eci . cf in sorted-name order (ce_updater.cpp:236-242)
    double e = 0.0;
    for (int k = 0; k < n_eci; ++k) e += eci_s[k] * cf_s[k];
    a.energy[chain] = e * (double)(unsigned)N;
    a.trial[chain] = t_end;
    if (a.accum) {
      cemc_accum *ac = a.accum + acc_row;
      ac->sum_e += acc_s[0];
      ac->sum_e2 += acc_s[1];
      for (int b = 0; b < g.n_bf; ++b) {
        ac->sum_s[b] += acc_s[2 + b];
        ac->sum_s2[b] += acc_s[2 + CEMC_MAX_BF + b];
        ac->sum_se[b] += acc_s[2 + 2 * CEMC_MAX_BF + b];
      }
      ac->n_samples += my_trials;
      ac->n_accept += n_acc_launch;
    }
    if (a.status) a.status[chain] = 0;
  }
}

template <typename R, int MOVE>
static cudaError_t launch_t(const DevGeo &g, const RunArgs &a, size_t smem, cudaStream_t st) {
  auto k = mc_kernel<R, MOVE>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<a.n_chains, (a.warps + 1) * 32, smem, st>>>(g, a);
  return cudaGetLastError();
}

cudaError_t launch_mc(const DevGeo &g, const RunArgs &a, int move, int precision, size_t smem, cudaStream_t st) {
  if (precision == CEMC_PREC_F32)
    return move == CEMC_MOVE_SWAP ? launch_t<float, CEMC_MOVE_SWAP>(g, a, smem, st)
                                  : launch_t<float, CEMC_MOVE_FLIP>(g, a, smem, st);
  return move == CEMC_MOVE_SWAP ? launch_t<double, CEMC_MOVE_SWAP>(g, a, smem, st)
                                : launch_t<double, CEMC_MOVE_FLIP>(g, a, smem, st);
}

}  // namespace cemc
