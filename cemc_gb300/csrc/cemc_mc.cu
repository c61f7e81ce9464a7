// Fused Metropolis Monte Carlo kernel: trial-move energy change, accept test
// and in-place commit of occupation, correlation functions and energy.
//
// Replaces the reference's per-trial Python -> C++ round trip
// (Montecarlo._mc_step, cemc/mcmc/montecarlo.py:970-1038, calling
// CEUpdater::calculate / undo_changes / clear_history,
// cpp/src/ce_updater.cpp:313-555) by one launch that runs many trials of many
// chains.
//
// A chain is owned by one CTA, or by a pair of CTAs on two SMs (a
// thread-block cluster of two).  Each CTA keeps a full copy of the chain's
// occupation (int8 species ids) in shared memory when it fits.  A chain is a
// sequential Markov chain, so parallelism inside it comes from speculation:
// each round evaluates trials t0 .. t0 + CW - 1 (CW = CTAs x evaluating warps)
// against the state at the start of the round, one trial per warp.  A trial's
// energy change depends only on the species of its own sites and of their
// neighbour columns, so it stays valid unless an earlier ACCEPTED trial of the
// same round changed one of those sites.  Accepted trials stamp their site
// and its neighbourhood with (round, trial) marks into a shared-memory table
// (both CTAs' tables in a pair); after the round barrier every warp reads one
// stamp per trial, finds the longest prefix with no earlier conflicting
// accept (exactly what sequential Metropolis over the same stream does) and
// applies all of its accepted moves itself.  These stores are idempotent
// (committed moves touch disjoint sites, and a swap's list positions are
// recorded with the trial), so no second barrier is needed before the next
// round reads the occupation; stamp tables and trial records alternate by
// round parity, so the next round's writes never meet this round's reads.
// The first conflicting trial is re-evaluated next round.  When a stamp table
// is smaller than the supercell it is indexed by site & mask: an alias can
// only report a false conflict, which shortens the committed prefix and never
// changes a result.  The neighbour relation is symmetric (checked when the
// geometry is built), so "accepted site in my neighbourhood" equals "my site
// in its neighbourhood".
//
// In a pair, each CTA writes its trial records and stamps into both CTAs'
// shared memory (distributed shared memory stores and reductions), so every
// warp of both CTAs reads the same data after the cluster barrier and
// computes the same committed prefix.  Both CTAs also exchange their round
// start before each barrier; a mismatch stops both with CEMC_ERR_INTERNAL
// instead of letting them wait at different barriers.
//
// Two or three helper warps per CTA run off the critical path.  The fetcher
// precomputes the counter-based draws (philox.h) of upcoming trials and
// prefetches their neighbour-table rows from L2/HBM into a shared-memory ring
// with cp.async (single-site flips, whose site does not depend on the state).
// One or two bookers fold each finished round, one round late: booker q keeps
// per-lane running sums of energy and singlets for trials 32q .. 32q + 31 of
// each round (carrying the other half's totals), writes their trace entries,
// and adds the correlation-function changes of its CTA's committed accepted
// trials (change rows double-buffered by round parity) to a row of sums.
// Correlation functions and energy are brought up to date in FP64 once, at
// the end of the launch.
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
// Hint that the 128-byte line holding p will be read soon (global memory, into L1).
__device__ __forceinline__ void prefetch_l1(const void *p) {
  asm volatile("prefetch.global.L1 [%0];\n" ::"l"(p));
}
// Every line of one neighbour row of the table.
__device__ __forceinline__ void prefetch_row(const int32_t *row, int cpad) {
  const uintptr_t b = reinterpret_cast<uintptr_t>(row) & ~(uintptr_t)127;
  const uintptr_t e = reinterpret_cast<uintptr_t>(row + cpad);
  for (uintptr_t q = b; q < e; q += 128) prefetch_l1(reinterpret_cast<const void *>(q));
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
__device__ __forceinline__ void spin_ballot(const DevGeo &g, const int8_t *occ, const RowRef &row, uint32_t xorv,
                                            int ovr_site, uint32_t ovr_bit, uint32_t &lo, uint32_t &hi,
                                            int (&nbr)[4], int lane) {
  uint32_t b0 = 0, b1 = 0;
  nbr[0] = nbr[1] = nbr[2] = nbr[3] = -1;
  if (lane < g.n_cols) {
    const int s = row_at(g, row, lane);
    nbr[0] = s;
    b0 = (s == ovr_site) ? ovr_bit : ((uint32_t)occ[s] ^ xorv);
  }
  if (lane + 32 < g.n_cols) {
    const int s = row_at(g, row, lane + 32);
    nbr[1] = s;
    b1 = (s == ovr_site) ? ovr_bit : ((uint32_t)occ[s] ^ xorv);
  }
  lo = __ballot_sync(kFull, b0);
  hi = __ballot_sync(kFull, b1);
}

// Parities of this lane's multi-site terms, packed 6 bits per cluster-ECI slot.
// terms[t] = {mask lo, mask hi, shift in the 32-lane cut, shift in the 16-lane cut}.
template <bool HALF>
__device__ __forceinline__ uint32_t spin_lane_parities(const uint4 *terms, int lo_t, int hi_t, uint32_t lo,
                                                       uint32_t hi) {
  uint32_t packed = 0;
#pragma unroll 4
  for (int t = lo_t; t < hi_t; ++t) {
    const uint4 m = terms[t];
    packed += (uint32_t)(__popc((lo & m.x) ^ (hi & m.y)) & 1) << (HALF ? m.w : m.z);
  }
  return packed;
}



// ---- move constraints -------------------------------------------------------------
// A change (site, old -> new) passes the move constraints: species `old` is not
// frozen (FixedElement) and species `new` may be placed on the site
// (ConstrainElementByTag, FixEdgeLayers); allow NULL = every species.
__device__ __forceinline__ bool change_legal(const uint8_t *allow, uint32_t frozen, int site, int old_s, int new_s) {
  return !((frozen >> old_s) & 1u) && (allow == nullptr || ((allow[site] >> new_s) & 1u));
}

// ---- table form ---------------------------------------------------------------
// Species of the neighbour columns of `row` into sp[0..n_cols) (site `ovr` read
// as species `ovr_s`); each lane keeps the site ids of its columns in nbr[] for
// the conflict stamps.
__device__ __forceinline__ void table_gather(const DevGeo &g, const int8_t *occ, const RowRef &row, int ovr,
                                             int ovr_s, int8_t *sp, int (&nbr)[4], int lane) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = lane + 32 * j;
    nbr[j] = -1;
    if (c < g.n_cols) {
      const int s = row_at(g, row, c);
      nbr[j] = s;
      sp[c] = (int8_t)(s == ovr ? ovr_s : occ[s]);
    }
  }
}

// Energy change of one flip (or, TWO, of a swap's two flips) from the pattern
// tables: one lookup per cluster geometry, F[off + on * S^m + s1 + S s2 + S^2 s3]
// with on = old * S + new and the member species s_j of the geometry's columns.
// Geometries [lo, hi) are those of the changed site's translation group.
template <typename R, bool TWO>
__device__ __forceinline__ R table_de(const DevGeo &g, const uint4 *geos, const R *F, const int8_t *spa,
                                      const int8_t *spb, int on_a, int on_b, int lo, int hi, int lane) {
  const int S = g.n_sym, S2 = S * S;
  R sum = (R)0;
  for (int i = lo + lane; i < hi; i += 32) {
    const uint4 e = geos[i];
    const int c1 = e.x & 0xff, c2 = (e.x >> 8) & 0xff, c3 = (e.x >> 16) & 0xff;
    sum += F[e.y + on_a * e.z + spa[c1] + S * spa[c2] + S2 * spa[c3]];
    if (TWO) sum += F[e.y + on_b * e.z + spb[c1] + S * spb[c2] + S2 * spb[c3]];
  }
  return warp_sum(sum);
}

// ---- thread-block cluster pairs ---------------------------------------------
__device__ __forceinline__ unsigned cluster_cta_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}
// Every thread of both CTAs; release / acquire orders the shared-memory
// stores (local and remote) made before it against the reads after it.
__device__ __forceinline__ void cluster_barrier() {
  __syncwarp();  // the .aligned forms want every lane of the warp at the same instruction
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t peer_addr(const void *p, unsigned rank) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_peer(uint32_t a, int32_t v) {
  asm volatile("st.shared::cluster.s32 [%0], %1;\n" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void st_peer(uint32_t a, int8_t v) {
  asm volatile("st.shared::cluster.s8 [%0], %1;\n" ::"r"(a), "r"((int)v) : "memory");
}
__device__ __forceinline__ void st_peer(uint32_t a, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;\n" ::"r"(a), "f"(v) : "memory");
}
__device__ __forceinline__ void st_peer(uint32_t a, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;\n" ::"r"(a), "d"(v) : "memory");
}
__device__ __forceinline__ void st_peer(uint32_t a, uint64_t v) {
  asm volatile("st.shared::cluster.u64 [%0], %1;\n" ::"r"(a), "l"(v) : "memory");
}
// Conflict stamp into this CTA's shared table when `on`: a predicated reduction
// with no returned value and no branch, so a lane's stamps issue back to back.
__device__ __forceinline__ void red_max_shared_if(const uint32_t *p, bool on, uint32_t v) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("{\n.reg .pred q;\nsetp.ne.u32 q, %2, 0;\n@q red.shared.max.u32 [%0], %1;\n}\n" ::"r"(a), "r"(v),
               "r"((uint32_t)on)
               : "memory");
}
__device__ __forceinline__ void red_max_peer(uint32_t a, uint32_t v) {
  asm volatile("red.shared::cluster.max.u32 [%0], %1;\n" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ double ld_peer_acc(const double *p, unsigned rank) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];\n" : "=d"(v) : "r"(peer_addr(p, rank)) : "memory");
  return v;
}
__device__ __forceinline__ double ld_peer_acc(const df64 *p, unsigned rank) {
  float hi, lo;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];\n" : "=f"(hi), "=f"(lo) : "r"(peer_addr(p, rank)) : "memory");
  return (double)hi + (double)lo;
}

// CONS: this build runs the move-constraint redraw loop and the first-move acceptance (one
// trial per warp, one CTA per chain); unconstrained launches take builds without them.
template <typename R, int MOVE, int FORM, int CL, int TPW, bool CONS>
__global__ void __launch_bounds__(kMcMaxThreads, 1) mc_kernel(DevGeo g, RunArgs a, SpinDev sd) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr bool SWAP = (MOVE == CEMC_MOVE_SWAP);
  constexpr bool SPIN = (FORM == kFormSpin), TAB = (FORM == kFormTable);
  constexpr bool RECYCLE = (FORM == kFormRecycle);  // generic evaluation, waste-recycled acceptance and sums
  const int W = a.warps;   // evaluating warps per CTA, then NB booker warps and one fetcher warp
  const int CW = round_trials(CL, W, TPW);  // trials per round
  const int NB = n_bookers(CL, W, TPW);
  const McLayout L = mc_layout(g, W, MOVE, (int)sizeof(R), a.occ_smem, a.trk_smem, a.stamp_bits, SPIN ? sd.n_cl : 0,
                               SPIN ? sd.n_masks : 0, a.ring_bits, FORM, TPW, a.gstamp != nullptr);
  const uint32_t rmask = (1u << a.ring_bits) - 1u;
  const int rank = (CL == 2) ? (int)cluster_cta_rank() : 0;
  const unsigned peer = (unsigned)(rank ^ 1);
  const int chain = blockIdx.x / CL;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool helper = (warp >= W);
  const bool booker = helper && warp < W + NB, fetcher = (warp == W + NB);
  // booker q books trials 32q .. 32q + 31 of each round: q = CTA rank in a pair, else the booker's index
  const int bq = (CL == 2) ? rank : (booker ? warp - W : 0);
  const int gidx = rank * W + warp;  // this warp's trial slot in a round
  const int N = g.n_sites, n_eci = g.n_eci, cpad = g.cpad;
  const uint32_t hmask = (1u << L.stamp_bits) - 1u;

  double *cf_s = reinterpret_cast<double *>(smem + L.cf);
  double *eci_s = reinterpret_cast<double *>(smem + L.eci);
  double *w_s = reinterpret_cast<double *>(smem + L.w);
  // Running sums of this launch, FP64 in FP64 mode and double-float in FP32
  // mode.  The thermodynamic sums are kept per lane of the booker warps
  // (lane j of booker q takes trial 32q + j of each round) and the committed
  // correlation-function changes per booker and ECI, so no round needs a
  // cross-lane or cross-warp reduction of them; both are reduced once, in
  // fixed order, in the epilogue.
  constexpr bool DF = (sizeof(R) == 4);
  using A = typename std::conditional<DF, df64, double>::type;
  constexpr int NACC = 2 + 3 * CEMC_MAX_BF;
  constexpr int NBF = SPIN ? 1 : CEMC_MAX_BF;
  A *lacc0 = reinterpret_cast<A *>(smem + L.acc);   // [2][NACC][32], one block per booker of this CTA
  A *lacc = lacc0 + (CL == 1 ? bq : 0) * NACC * 32;  // this booker's block
  A *s_start = lacc0 + 2 * NACC * 32;                // [CEMC_MAX_BF] singlets at launch start, then 1/N
  A *cfw = reinterpret_cast<A *>(smem + L.cfw);   // [2][n_eci], one row per booker of this CTA
  R *coef_s = reinterpret_cast<R *>(smem + L.coef);
  R *bf_s = reinterpret_cast<R *>(smem + L.bf);
  uint16_t *terms_s = reinterpret_cast<uint16_t *>(smem + L.terms);
  int32_t *lane_term_s = reinterpret_cast<int32_t *>(smem + L.lane_term);  // [groups][group_lane_ints]
  R *gscale_s = reinterpret_cast<R *>(smem + L.grp);                          // [groups]
  int32_t *gstart_s = reinterpret_cast<int32_t *>(smem + L.grp + 8 * CEMC_MAX_GROUPS);  // [groups + 1]
  int8_t *kind_s = reinterpret_cast<int8_t *>(smem + L.kind);
  int8_t *dec_s = kind_s + n_eci;
  // misc: [1] status, [2] species present, [3] a trial ran out of constraint redraws, [4..12) present ids, [12..20) site-list
  //       starts, [20..28) site-list counts, [32..36) round starts written by the peer CTA,
  //       [36..40) accept counts of this CTA's bookers
  int32_t *misc = reinterpret_cast<int32_t *>(smem + L.misc);
  uint64_t *t0_slot = reinterpret_cast<uint64_t *>(misc + 32);
  uint64_t *nacc_slot = reinterpret_cast<uint64_t *>(misc + 36);  // [2] accept counts of this CTA's bookers
  Draw *draws = reinterpret_cast<Draw *>(smem + L.draws);
  int32_t *rows = reinterpret_cast<int32_t *>(smem + L.rows);
  // two conflict-stamp tables of hmask + 1 entries: shared memory, or (large supercells,
  // exact) this chain's region of a global buffer shared by both CTAs of a pair
  const bool gst = a.gstamp != nullptr;
  uint32_t *stamp = gst ? a.gstamp + (size_t)chain * 2 * (hmask + 1) : reinterpret_cast<uint32_t *>(smem + L.stamp);
  unsigned char *rec0 = smem + L.rec;
  // change rows of this CTA's trials: exact integers in the spin basis
  using DT = typename std::conditional<SPIN, int32_t, R>::type;
  DT *drow = reinterpret_cast<DT *>(smem + L.drow);
  unsigned char *wbase = smem + L.warp0 + (size_t)(helper ? 0 : warp) * L.warp_stride;
  R *va = reinterpret_cast<R *>(wbase);
  int8_t *sp_a = reinterpret_cast<int8_t *>(wbase);  // table form: species of the trial's rows
  int8_t *sp_b = sp_a + align16((size_t)g.n_cols + 1);
  R *ftab = reinterpret_cast<R *>(smem + L.ftab);
  uint4 *geos_s = reinterpret_cast<uint4 *>(smem + L.geos);
  R *vb = va + g.vals_len;
  R *part = reinterpret_cast<R *>(wbase + L.warp_part);

  SpinEci *sp_eci = reinterpret_cast<SpinEci *>(smem + L.sp_eci);
  uint4 *sp_terms = reinterpret_cast<uint4 *>(smem + L.sp_masks);
  int32_t *sp_lane_term = reinterpret_cast<int32_t *>(smem + L.sp_lane);
  int32_t *sp_lane_first = sp_lane_term + 33;
  int32_t *sp_half_term = sp_lane_first + 32;  // [17]
  int32_t *sp_half_first = sp_half_term + 17;  // [16]
  int32_t *sp_qtr_term = sp_half_first + 16;   // [9]
  int32_t *sp_qtr_first = sp_qtr_term + 9;     // [8]
  const uint32_t xorv = SPIN ? (uint32_t)(sd.minus_id ^ 1) : 0u;  // spin bit = occ ^ xorv (1 = the -1 species)

  int8_t *occ = a.occ_smem ? reinterpret_cast<int8_t *>(smem + L.occ) : a.occ + (size_t)chain * N;
  int32_t *trk = nullptr, *loc = nullptr;
  if (SWAP) {
    trk = a.trk_smem ? reinterpret_cast<int32_t *>(smem + L.trk) : a.trk + (size_t)chain * N;
    loc = a.trk_smem ? trk + N : a.loc + (size_t)chain * N;
  }

  // A chain with no trials in this launch (an empty serving slot) leaves its
  // state untouched; both CTAs of a pair see the same count and leave together.
  if (a.chain_trials && a.chain_trials[chain] <= a.chunk_offset) return;

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
  }
  for (int i = tid; i < g.n_bf * g.n_sym; i += blockDim.x) bf_s[i] = (R)g.bf[i];
  {
    const int LG = group_lane_ints(n_eci);
    for (int i = tid; i < g.n_groups * LG; i += blockDim.x) {
      const int q = i / LG, r = i - q * LG;
      lane_term_s[i] = r < 33 ? g.lane_term[33 * q + r]
                              : (r < 65 ? g.lane_first_eci[32 * q + r - 33] : g.eci_lane[(size_t)2 * n_eci * q + r - 65]);
    }
    for (int q = tid; q < g.n_groups; q += blockDim.x) gscale_s[q] = (R)g.group_scale[q];
    for (int q = tid; q <= g.n_groups; q += blockDim.x) gstart_s[q] = g.geo_start[q];
  }
  {
    const uint2 *src = reinterpret_cast<const uint2 *>(g.terms);
    uint2 *dst = reinterpret_cast<uint2 *>(terms_s);
    for (int i = tid; i < g.n_terms; i += blockDim.x) dst[i] = src[i];
  }
  if (!gst || rank == 0)
    for (uint32_t i = tid; i < 2 * (hmask + 1); i += blockDim.x) stamp[i] = 0u;
  for (int i = tid; i < 2 * n_eci; i += blockDim.x) cfw[i] = acc_from<A>(0.0);
  if (!TAB)
    for (int i = tid; i < 2 * TPW * W * n_eci; i += blockDim.x)
      drow[i] = (DT)0;  // the spin path writes only the entries of cluster and singlet ECIs
  if (SPIN)
    for (int i = tid; i < 2 * 32 * n_eci; i += blockDim.x) reinterpret_cast<int32_t *>(smem + L.cfp)[i] = 0;
  if (TAB) {
    // this chain's pattern tables F(old, new, member species), in FP64 then rounded to R
    const int S = g.n_sym;
    for (int i = tid; i < g.n_geo; i += blockDim.x) geos_s[i] = g.geo_list[i];
    for (int idx = tid; idx < g.tab_len; idx += blockDim.x) {
      int p = 0;
      while (p + 1 < g.n_pat && g.pat_info[p + 1].y <= idx) ++p;
      const int4 pi = g.pat_info[p];
      int stride = 1;
      for (int j = 0; j < pi.x; ++j) stride *= S;
      const int li = idx - pi.y, on = li / stride, tup = li - on * stride;
      const int old_s = on / S, new_s = on - old_s * S;
      double v = 0.0;
      for (int t = pi.z; t < pi.w; ++t) {
        const int pk = g.pat_terms[t];
        const int k = pk & 0xff, dr = (pk >> 8) & 15;
        double prod = g.bf[dr * S + new_s] - g.bf[dr * S + old_s];
        int tt = tup;
        for (int j = 0; j < pi.x; ++j) {
          const int sj = tt % S;
          tt /= S;
          prod *= g.bf[((pk >> (12 + 4 * j)) & 15) * S + sj];
        }
        v += a.eci[(size_t)chain * n_eci + k] * (double)N * g.eci_w[k] * prod;
      }
      ftab[idx] = (R)v;
    }
    if (!helper && lane == 0) {
      sp_a[g.n_cols] = 0;  // the absent member of a smaller cluster reads species 0
      sp_b[g.n_cols] = 0;
    }
  }
  for (int i = tid; i < 2 * NACC * 32; i += blockDim.x) lacc0[i] = acc_from<A>(0.0);
  if (SPIN) {
    for (int k = tid; k < sd.n_cl; k += blockDim.x) sp_eci[k] = sd.eci[k];
    for (int t = tid; t < sd.n_masks; t += blockDim.x)
      sp_terms[t] = make_uint4(sd.masks[t].x, sd.masks[t].y, sd.shift[t],
                               TPW == 2 ? sd.half_shift[t] : (TPW == 4 ? sd.qtr_shift[t] : 0u));
    for (int i = tid; i < 33; i += blockDim.x) sp_lane_term[i] = sd.lane_term[i];
    for (int i = tid; i < 32; i += blockDim.x) sp_lane_first[i] = sd.lane_first[i];
    if (TPW == 2) {
      for (int i = tid; i < 17; i += blockDim.x) sp_half_term[i] = sd.half_lane_term[i];
      for (int i = tid; i < 16; i += blockDim.x) sp_half_first[i] = sd.half_lane_first[i];
    }
    if (TPW == 4) {
      for (int i = tid; i < 9; i += blockDim.x) sp_qtr_term[i] = sd.qtr_lane_term[i];
      for (int i = tid; i < 8; i += blockDim.x) sp_qtr_first[i] = sd.qtr_lane_first[i];
    }
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
    misc[3] = 0;
    t0_slot[0] = t0_slot[1] = 0;
    nacc_slot[0] = nacc_slot[1] = 0;
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
      s_start[b] = acc_from<A>((b < g.n_bf && g.singlet_eci[b] >= 0) ? a.cf[(size_t)chain * n_eci + g.singlet_eci[b]]
                                                                     : 0.0);
    s_start[CEMC_MAX_BF] = acc_from<A>(1.0 / (double)N);
  }

  const double kT = a.kT[chain];
  // move constraints of this chain (the redraw loop runs only when there are any; the half-warp
  // form takes no constraints, and keeping these out of it at compile time keeps its code as fast)
  const uint8_t *allow = (CONS && a.site_allow) ? a.site_allow + (size_t)chain * N : nullptr;
  const uint32_t frz = (CONS && a.frozen) ? a.frozen[chain] : 0u;
  const bool cons = CONS && (allow != nullptr || frz != 0u);
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

  // Helper-warp state (CTA 0): energy relative to e_ref and, per singlet, the
  // launch's summed singlet changes (the singlet after a trial is start + sum / N).
  A eoff = acc_from<A>(a.energy[chain] - e_ref);
  A dsum[NBF];
#pragma unroll
  for (int b = 0; b < NBF; ++b) dsum[b] = acc_from<A>(0.0);
  uint64_t n_acc_launch = 0;
  uint64_t fill_end = t_first;

  // Draws (and, for flips, neighbour rows) of trials [fill_end, min(t0 + 3 CW, t_end)).
  auto prefetch = [&](uint64_t t0) {
    uint64_t want = t0 + (uint64_t)kPrefetchRounds * (uint64_t)CW;
    if (want > t_end) want = t_end;
    for (uint64_t t = fill_end + lane; t < want; t += 32) {
      const uint32_t slot = (uint32_t)t & rmask;
      const cemc_u32x4 w0 = cemc_trial_draw(a.seed, key, t, 0);
      Draw d;
      d.w0 = w0.v[0];
      d.w1 = w0.v[1];
      d.w2 = w0.v[2];
      d.w3 = w0.v[3];
      d.pad = 0;  // flips: the site's translation group
      if (SWAP) {
        const cemc_u32x4 w1 = cemc_trial_draw(a.seed, key, t, 1);
        d.x0 = w1.v[0];
        d.x1 = w1.v[1];
        d.site = -1;
        // The sites are read from the site lists when the trial is evaluated, rounds from
        // now; the lists' extents do not change (swaps keep every species count), so the
        // sites at the trial's two list slots now are almost always the ones it will
        // read: warm L1 with their neighbour rows.  Only a hint; a stale guess costs the
        // L2 latency the evaluation pays without it.
        const int np = misc[2];
        if (np >= 2) {
          const int ia = (int)cemc_below(w0.v[0], (uint32_t)np);
          int ib = (int)cemc_below(w0.v[1], (uint32_t)(np - 1));
          ib += (ib >= ia);
          const int A = misc[4 + ia], B = misc[4 + ib];
          const int pa = trk[misc[12 + A] + (int)cemc_below(w0.v[2], (uint32_t)misc[20 + A])];
          const int pb = trk[misc[12 + B] + (int)cemc_below(w0.v[3], (uint32_t)misc[20 + B])];
          if (g.box_L == 0 && (unsigned)pa < (unsigned)N) prefetch_row(g.table + (size_t)pa * cpad, cpad);
          if (g.box_L == 0 && (unsigned)pb < (unsigned)N) prefetch_row(g.table + (size_t)pb * cpad, cpad);
        }
      } else {
        d.x0 = d.x1 = 0;
        if constexpr (TPW >= 2) {
          // unconstrained flips: the acceptance test's parts of the uniform in w2, w3 (read with
          // the site), the uniform's words in x0, x1 (read only by the exact fallback)
          float lnu, mu;
          metropolis_parts(d.w2, lnu, mu);
          d.x0 = d.w2;
          d.x1 = d.w3;
          d.w2 = __float_as_uint(lnu);
          d.w3 = __float_as_uint(mu);
        }
        // the flipped site: uniform over the movable sites (all sites without a background)
        d.site = g.n_movable == N ? (int)cemc_below(w0.v[0], (uint32_t)N)
                                  : g.movable[cemc_below(w0.v[0], (uint32_t)g.n_movable)];
        if (g.n_groups > 1) d.pad = (uint32_t)g.site_group[d.site];
        const int32_t *src = g.table + (size_t)d.site * cpad;
        int32_t *dst = rows + (size_t)slot * cpad;
        for (int q = 0; q < cpad; q += 4) cp_async16(dst + q, src + q);
      }
      draws[slot] = d;
    }
    if (want > fill_end) fill_end = want;
    cp_async_commit();
  };

  // Fold trials [off, off + kh) of round records `rec` into the running sums.
  // Lane j takes trial off + j: one inclusive scan gives the energy and singlet
  // offsets after each trial, and each lane adds its own values to its own
  // sums; a half without accepted trials needs no scan.
  auto book_half = [&](const unsigned char *rec, int off, int kh, uint64_t tb) {
    const int8_t *r_acc = reinterpret_cast<const int8_t *>(rec + L.rec_acc);
    const R *r_de = reinterpret_cast<const R *>(rec + L.rec_de);
    const R *r_ds = reinterpret_cast<const R *>(rec + L.rec_ds);
    const int gg = off + lane;
    const bool mine = lane < kh;
    const bool acc = mine && r_acc[gg];
    if (a.trace_acc && mine) {  // the round started at trial tb
      const int32_t *r_sa = reinterpret_cast<const int32_t *>(rec + L.rec_sa);
      const int32_t *r_sb = reinterpret_cast<const int32_t *>(rec + L.rec_sb);
      const size_t idx = (size_t)chain * a.n_trials + (size_t)(tb + (uint64_t)gg - t_first);
      a.trace_site[2 * idx] = r_sa[gg];
      a.trace_site[2 * idx + 1] = r_sb[gg];
      a.trace_acc[idx] = r_acc[gg];
      a.trace_de[idx] = (double)r_de[gg];
    }
    const unsigned am = __ballot_sync(kFull, acc);
    n_acc_launch += (uint64_t)__popc(am);
    if (!a.accum) return;
    R x = acc ? r_de[gg] : (R)0;
    R ds[NBF];
#pragma unroll
    for (int b = 0; b < NBF; ++b) ds[b] = (acc && b < g.n_bf) ? r_ds[b * kRoundSlots + gg] : (R)0;
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
    if (mine && !RECYCLE) {
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
    if constexpr (RECYCLE) {
      // Waste recycling (mc_observers.py:231-258, montecarlo.py:805-809): every trial adds
      // p0 x (value before it) + p1 x (value of its proposal), p1 = 1 / (1 + exp(dE / kT)).
      // The energies are those of the state before and of the proposed state; the singlets
      // are the calculator's before and after the step (after a rejection both are the
      // state before, as the reference's observer reads them).
      if (mine) {
        const R dE = r_de[gg];
        const double p1d = 1.0 / (1.0 + exp((double)dE / kT));
        const A P1 = acc_from<A>(p1d), P0 = acc_from<A>(1.0 - p1d);
        const A e_after = acc_add_x(eoff, x);
        const A e_before = acc ? acc_add_x(e_after, -dE) : e_after;
        const A e_prop = acc_add_x(e_before, dE);
        lacc[lane] = acc_add(lacc[lane], acc_add(acc_mul(P0, e_before), acc_mul(P1, e_prop)));
        lacc[32 + lane] = acc_add(lacc[32 + lane], acc_add(acc_mul(P0, acc_mul(e_before, e_before)),
                                                           acc_mul(P1, acc_mul(e_prop, e_prop))));
#pragma unroll
        for (int b = 0; b < NBF; ++b) {
          if (b < g.n_bf) {
            const R own = acc ? r_ds[b * kRoundSlots + gg] : (R)0;
            const A s_after = acc_add(s_start[b], acc_mul(acc_add_x(dsum[b], ds[b]), s_start[CEMC_MAX_BF]));
            const A s_before = acc_add(s_start[b], acc_mul(acc_add_x(dsum[b], ds[b] - own), s_start[CEMC_MAX_BF]));
            A *l = lacc + (2 + b) * 32 + lane;
            l[0] = acc_add(l[0], acc_add(acc_mul(P0, s_before), acc_mul(P1, s_after)));
            l[CEMC_MAX_BF * 32] = acc_add(l[CEMC_MAX_BF * 32], acc_add(acc_mul(P0, acc_mul(s_before, s_before)),
                                                                     acc_mul(P1, acc_mul(s_after, s_after))));
            l[2 * CEMC_MAX_BF * 32] = acc_add(l[2 * CEMC_MAX_BF * 32], acc_add(acc_mul(P0, acc_mul(s_before, e_before)),
                                                                             acc_mul(P1, acc_mul(s_after, e_prop))));
          }
        }
      }
    }
    if (am) {
      eoff = acc_add_x(eoff, __shfl_sync(kFull, x, kh - 1));
#pragma unroll
      for (int b = 0; b < NBF; ++b) dsum[b] = acc_add_x(dsum[b], __shfl_sync(kFull, ds[b], kh - 1));
    }
  };
  // Totals of trials [off, off + kh) added to the running offsets only (the
  // other CTA of a pair books those trials).
  auto carry_half = [&](const unsigned char *rec, int off, int kh) {
    if (!a.accum) return;
    const int8_t *r_acc = reinterpret_cast<const int8_t *>(rec + L.rec_acc);
    const R *r_de = reinterpret_cast<const R *>(rec + L.rec_de);
    const R *r_ds = reinterpret_cast<const R *>(rec + L.rec_ds);
    const int gg = off + lane;
    const bool acc = lane < kh && r_acc[gg];
    if (!__ballot_sync(kFull, acc)) return;
    eoff = acc_add_x(eoff, warp_sum(acc ? r_de[gg] : (R)0));
#pragma unroll
    for (int b = 0; b < NBF; ++b)
      if (b < g.n_bf) dsum[b] = acc_add_x(dsum[b], warp_sum(acc ? r_ds[b * kRoundSlots + gg] : (R)0));
  };
  // Correlation-function changes of this CTA's committed accepted trials in
  // slots [own_lo, own_hi) (change rows dbuf[slot - own_lo] in a pair, dbuf[slot]
  // otherwise), summed by the booker: lane takes ECIs lane, lane + 32, ... in
  // registers; exact 64-bit integers for the spin basis (integer changes).
  const int own_lo = (CL == 2) ? rank * W * TPW : 32 * bq;
  const int own_hi = (CL == 2) ? own_lo + W * TPW : own_lo + 32;
  A *cfb = cfw + (size_t)(CL == 1 ? bq : 0) * n_eci;
  using CFA = typename std::conditional<SPIN, long long, A>::type;
  CFA cfr[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) cfr[i] = CFA{};
  auto cf_add = [](CFA &c, DT d) {
    if constexpr (SPIN) c += (long long)d;
    else c = acc_add_x(c, d);
  };
  auto cf_sum_out = [](const CFA &c) -> A {
    if constexpr (SPIN) return acc_from<A>((double)c);
    else return c;
  };
  // Spin form: the change rows are integers, so lane j adds the row of its own
  // slot own_lo + j to lane-private int32 sums cfp[k][j] (no exchange between
  // lanes per round), folded into the 64-bit sums every kCfFoldRounds rounds and
  // at the end.  A row entry is 2 P with |P| <= 64 pair terms + 32 x 63 multi-site
  // terms, so 32 lanes x 4096 rounds of it stay below 2^31.
  constexpr uint32_t kCfFoldRounds = 4096;
  int32_t *cfp = reinterpret_cast<int32_t *>(smem + L.cfp) + (size_t)(CL == 1 ? bq : 0) * n_eci * 32;
  auto cf_fold = [&]() {
    if constexpr (SPIN) {
      for (int k = 0; k < n_eci; ++k) {
        const int tot = __reduce_add_sync(kFull, cfp[32 * k + lane]);
        cfp[32 * k + lane] = 0;
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if ((k >> 5) == i && (k & 31) == lane) cfr[i] += (long long)tot;
      }
    }
  };
  auto book_cf = [&](const unsigned char *rec, const DT *dbuf, int ks) {
    const int8_t *r_acc = reinterpret_cast<const int8_t *>(rec + L.rec_acc);
    const int hi = ks < own_hi ? ks : own_hi;
    const int j = own_lo + lane;
    if constexpr (SPIN) {
      if (j < hi && r_acc[j]) {
        const DT *D = dbuf + (size_t)(j - (CL == 2 ? own_lo : 0)) * n_eci;
        for (int k0 = 0; k0 < n_eci; k0 += 16) {
          int32_t d[16];  // the row first: loads that no store of cfp has to precede
#pragma unroll
          for (int i = 0; i < 16; ++i) d[i] = k0 + i < n_eci ? (int32_t)D[k0 + i] : 0;
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (k0 + i < n_eci) cfp[32 * (k0 + i) + lane] += d[i];
        }
      }
      __syncwarp();
      return;
    }
    unsigned am = __ballot_sync(kFull, j < hi && r_acc[j]);
    while (am) {
      const int jj = own_lo + __ffs(am) - 1;
      am &= am - 1;
      const DT *D = dbuf + (size_t)(jj - (CL == 2 ? own_lo : 0)) * n_eci;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int k = lane + 32 * i;
        if (k < n_eci) cf_add(cfr[i], D[k]);
      }
    }
  };
  auto book = [&](const unsigned char *rec, const DT *dbuf, int ks, uint64_t tb) {
    const int k0 = ks < 32 ? ks : 32, k1 = ks - k0;
    if (bq == 0) {
      book_half(rec, 0, k0, tb);
      if (k1 > 0) carry_half(rec, 32, k1);
    } else {
      carry_half(rec, 0, k0);
      if (k1 > 0) book_half(rec, 32, k1, tb);
    }
    if constexpr (!TAB) book_cf(rec, dbuf, ks);  // the table form leaves the CFs to a recompute
  };

  // Store into this CTA's shared memory and, in a pair, the peer's copy.
  auto put = [&](auto *p, auto v) {
    *p = v;
    if (CL == 2) st_peer(peer_addr(p, peer), v);
  };

  if (CL == 2)
    cluster_barrier();  // the peer's tables are initialised before any remote store
  else
    __syncthreads();
  if (misc[1] != 0) {  // same verdict in both CTAs of a pair: it depends on the chain's inputs only
    if (tid == 0 && rank == 0 && a.status) a.status[chain] = misc[1];
    return;
  }
  if (fetcher) {
    prefetch(t_first);
    cp_async_wait_all();
  }
  __syncthreads();

  const int n_present = SWAP ? misc[2] : 0;
  // spin path: lane k of every evaluating warp holds cluster ECI k and its coefficient
  SpinEci sp_e{};
  R sp_coef = (R)0;
  unsigned sp_multi = 0;  // cluster ECIs with multi-site terms
  // Flips at one or two trials per warp: the odd-term counts of all multi-site ECIs by one
  // packed butterfly (odd_counts_packed) when each has at most 255 terms and their 8-bit
  // fields fit one 64-bit word; else one reduction per ECI.
  bool sp_pk = false;
  int sp_tlo = 0, sp_thi = 0, sp_first = 0;  // this lane's range of multi-site terms
  if (SPIN) {
    // two trials per warp: lane l works for trial l / 16 on cluster ECI (and term range) l % 16
    // TPW trials per warp: lane l works for trial l / (32 / TPW) on cluster ECI (and term range) l % (32 / TPW)
    const int el = lane % (32 / TPW);
    sp_tlo = TPW == 4 ? sp_qtr_term[el] : (TPW == 2 ? sp_half_term[el] : sp_lane_term[el]);
    sp_thi = TPW == 4 ? sp_qtr_term[el + 1] : (TPW == 2 ? sp_half_term[el + 1] : sp_lane_term[el + 1]);
    sp_first = TPW == 4 ? sp_qtr_first[el] : (TPW == 2 ? sp_half_first[el] : sp_lane_first[el]);
    if (el < sd.n_cl) {
      sp_e = sp_eci[el];
      sp_coef = coef_s[sp_e.eci];
    }
    sp_multi = __ballot_sync(kFull, el < sd.n_cl && sp_e.n_multi > 0);
    if constexpr (TPW >= 2) sp_multi &= (1u << (32 / TPW)) - 1u;
    // (not for swaps: their second site's fields cost the FP64 swap build registers it spills)
    if constexpr (TPW <= 2 && !SWAP)
      sp_pk = __popc(sp_multi) <= 8 && __all_sync(kFull, el >= sd.n_cl || sp_e.n_multi <= 255);
  }
  // Lane group of LW lanes: counters pa (and pb, the second site of a swap) of this lane's
  // terms, 6 bits per cluster ECI from sp_first on; the group's total for ECI el of each
  // multi-site ECI, in field (its rank among the multi-site ECIs) of one 64-bit word summed
  // by a butterfly.  Every partial sum is part of a total <= 255, so no field carries.
  auto odd_counts_packed = [&](uint32_t pa, uint32_t pb, int el, auto lw_tag) -> int {
    constexpr int LWP = decltype(lw_tag)::value;
    uint64_t wsum = 0;
#pragma unroll
    for (int sl = 0; sl < 5; ++sl) {
      const int k = sp_first + sl;
      if (k < 32 && ((sp_multi >> k) & 1u)) {
        const int m = __popc(sp_multi & ((1u << k) - 1u));
        wsum += (uint64_t)((pa >> (6 * sl)) & 63u) << (8 * m);
        if (SWAP) wsum += (uint64_t)((pb >> (6 * sl)) & 63u) << (8 * (m + 4));
      }
    }
#pragma unroll
    for (int o = 1; o < LWP; o <<= 1) wsum += __shfl_xor_sync(kFull, wsum, o);
    int odd = 0;
    if ((sp_multi >> el) & 1u) {
      const int m = __popc(sp_multi & ((1u << el) - 1u));
      odd = (int)((wsum >> (8 * m)) & 255u);
      if (SWAP) odd -= (int)((wsum >> (8 * (m + 4))) & 255u);
    }
    return odd;
  };

  // One round: every warp, whatever its role, meets the round barrier once and
  // computes the same committed prefix `ks`, so the role loops below run in
  // lockstep.  Returns false when the launch is over, or when a pair's round
  // starts disagree (CEMC_ERR_INTERNAL, both CTAs stop at the same barrier).
  auto end_round = [&](uint32_t round, uint64_t t0, bool active, int &ks) -> bool {
    if (CL == 2) {
      if (tid == 0) st_peer(peer_addr(&t0_slot[round & 1], peer), t0);
      cluster_barrier();
      if (t0_slot[round & 1] != t0) {
        if (tid == 0) misc[1] = CEMC_ERR_INTERNAL;
        return false;
      }
    } else {
      __syncthreads();
    }
    if (!active) return false;
    const unsigned char *rec = rec0 + (size_t)(round & 1) * L.rec_stride;
    const int32_t *r_sa = reinterpret_cast<const int32_t *>(rec + L.rec_sa);
    const int32_t *r_sb = reinterpret_cast<const int32_t *>(rec + L.rec_sb);
    const uint32_t *tab = stamp + ((size_t)(round & 1) << L.stamp_bits);
    const int nv = (t_end - t0) < (uint64_t)CW ? (int)(t_end - t0) : CW;
    auto conflicted = [&](int gg) {
      const uint32_t v = tab[(uint32_t)r_sa[gg] & hmask];
      bool c = ((v >> 6) == round) && ((uint32_t)(63 - (v & 63u)) < (uint32_t)gg);
      if (SWAP) {
        const uint32_t v2 = tab[(uint32_t)r_sb[gg] & hmask];
        c |= ((v2 >> 6) == round) && ((uint32_t)(63 - (v2 & 63u)) < (uint32_t)gg);
      }
      return c;
    };
    const bool c0 = lane < nv && conflicted(lane);
    const bool c1 = lane + 32 < nv && conflicted(lane + 32);
    const unsigned m0 = __ballot_sync(kFull, c0);
    const unsigned m1 = __ballot_sync(kFull, c1);
    ks = m0 ? (__ffs(m0) - 1) : (m1 ? (31 + __ffs(m1)) : nv);
    return true;
  };

  uint64_t t0 = t_first;
  uint32_t round = 1;
  if (!helper) {
    // ---- evaluating warps: speculate, then apply the committed prefix ----------
    while (true) {
      const bool active = t0 < t_end;
      unsigned char *rec = rec0 + (size_t)(round & 1) * L.rec_stride;
      int32_t *r_sa = reinterpret_cast<int32_t *>(rec + L.rec_sa);
      int32_t *r_sb = reinterpret_cast<int32_t *>(rec + L.rec_sb);
      int32_t *r_la = reinterpret_cast<int32_t *>(rec + L.rec_la);
      int32_t *r_lb = reinterpret_cast<int32_t *>(rec + L.rec_lb);
      int8_t *r_acc = reinterpret_cast<int8_t *>(rec + L.rec_acc);
      int8_t *r_A = reinterpret_cast<int8_t *>(rec + L.rec_A);
      int8_t *r_B = reinterpret_cast<int8_t *>(rec + L.rec_B);
      R *r_de = reinterpret_cast<R *>(rec + L.rec_de);
      R *r_ds = reinterpret_cast<R *>(rec + L.rec_ds);
      uint32_t *tab = stamp + ((size_t)(round & 1) << L.stamp_bits);
      DT *dbuf = drow + (size_t)(round & 1) * TPW * W * n_eci;  // this round's change rows
      DT *Dw = dbuf + (size_t)warp * n_eci;
      if constexpr (TPW >= 2) {
        // ---- phase A, TPW flips per warp: lane group h = lane / LW evaluates trial slot TPW warp + h ----
        constexpr int LW = 32 / TPW;      // lanes per trial (16 or 8)
        constexpr int NJ = 64 / LW;       // column chunks of a neighbour row
        constexpr int FB = 32 / TPW;      // bits of a trial's field in the shared reductions
        constexpr uint32_t LMASK = (1u << LW) - 1u;
        if (active && t0 + (uint64_t)(rank * TPW * W + TPW * warp) < t_end) {
          const int h = lane / LW, hl = lane % LW;
          const int gh = rank * TPW * W + TPW * warp + h;  // trial slot in the round (pairs: CTA 1 after CTA 0)
          const uint64_t t = t0 + (uint64_t)gh;
          const bool has = t < t_end;  // the last groups of the last warp may have no trial
          const uint32_t slot = (uint32_t)t & rmask;
          int sa = 0, na = 0, oa = 0;
          float lnu = 0.f, mu = 0.f;
          if (has) {
            const uint4 dr = *reinterpret_cast<const uint4 *>(&draws[slot]);  // site, w1, w2, w3
            sa = (int)dr.x;
            oa = occ[sa];
            const int k = (int)cemc_below(dr.y, (uint32_t)(g.n_sym - 1));
            na = k + (k >= oa);
            lnu = __uint_as_float(dr.z);
            mu = __uint_as_float(dr.w);
          }
          const uint32_t occ_a_bit = (uint32_t)oa ^ xorv;
          // spin word of the neighbour row: bit c = column c, from NJ ballots of LW
          // columns (c = hl + LW j) of which each lane group keeps its own LW bits
          const int32_t *row = rows + (size_t)slot * cpad;
          int nbr[NJ];
          uint32_t wl = 0, wh = 0;
#pragma unroll
          for (int j = 0; j < NJ; ++j) {
            const int c = hl + LW * j;
            uint32_t bit = 0;
            nbr[j] = -1;
            if (has && c < g.n_cols) {
              const int sn = row[c];
              nbr[j] = sn;
              bit = (uint32_t)occ[sn] ^ xorv;
            }
            const uint32_t chunk = (__ballot_sync(kFull, bit) >> (LW * h)) & LMASK;
            if (LW * j < 32) wl |= chunk << (LW * j);
            else wh |= chunk << (LW * j - 32);
          }
          const uint32_t pa = spin_lane_parities<true>(sp_terms, sp_tlo, sp_thi, wl, wh);
          // odd-parity counts of each multi-site cluster ECI: one reduction serves every
          // lane group (group h's count in bits FB h .. FB h + FB - 1; at most 255 when FB = 8)
          int my_odd = 0;
          if constexpr (TPW == 4) {
            // at most 8 cluster ECIs of at most 255 terms: every ECI's count in an 8-bit field
            // of one 64-bit word, summed over the trial's 8 lanes by a butterfly (each partial
            // sum is part of a total <= 255, so no field carries into the next)
            uint64_t wsum = 0;
#pragma unroll
            for (int sl = 0; sl < 5; ++sl)
              if (sp_first + sl < 8) wsum |= (uint64_t)((pa >> (6 * sl)) & 63u) << (8 * (sp_first + sl));
            if (sp_multi) {
#pragma unroll
              for (int o = 1; o < LW; o <<= 1) wsum += __shfl_xor_sync(kFull, wsum, o);
            }
            my_odd = (int)((wsum >> (8 * (hl & 7))) & 255u);
          } else if (sp_pk) {
            my_odd = odd_counts_packed(pa, 0u, hl, std::integral_constant<int, LW>{});
          } else {
            for (unsigned mm = sp_multi; mm; mm &= mm - 1) {
              const int k = __ffs(mm) - 1;
              const int sl = k - sp_first;
              const uint32_t v = (sl >= 0 && sl < 5) ? ((pa >> (6 * sl)) & 63u) : 0u;
              const uint32_t tot = __reduce_add_sync(kFull, v << (FB * h));
              if (hl == k) my_odd = (int)((tot >> (FB * h)) & ((1u << FB) - 1u));
            }
          }
          const int delta = occ_a_bit ? 2 : -2;
          DT *Dh = dbuf + (size_t)(TPW * warp + h) * n_eci;  // this CTA's change row of the trial
          int P = 0;
          if (hl < sd.n_cl) {
            P = sp_e.n_pairs - 2 * (__popc(wl & sp_e.pair_lo) + __popc(wh & sp_e.pair_hi)) + sp_e.n_multi - 2 * my_odd;
            if (has) Dh[sp_e.eci] = delta * P;
          }
          R sum = sp_coef * (R)P;
#pragma unroll
          for (int o = LW / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
          if (sd.singlet_eci >= 0) {
            if (hl == 0 && has) Dh[sd.singlet_eci] = delta;
            sum += coef_s[sd.singlet_eci];
          }
          const R de = (R)delta * sum;
          int acc = 0;
          if (hl == 0 && has) {
            acc = metropolis_pre<R>(de, lnu, mu, &draws[slot].x0, kT, inv_kT);
            put(&r_sa[gh], (int32_t)sa);
            put(&r_sb[gh], (int32_t)na);
            put(&r_acc[gh], (int8_t)acc);
            put(&r_de[gh], de);
            put(&r_ds[gh], (R)delta);  // the singlet change (one decoration)
          }
          acc = __shfl_sync(kFull, acc, LW * h);
          const uint32_t mark = (round << 6) | (uint32_t)(63 - gh);
          if (CL == 1 && !gst) {
#pragma unroll
            for (int j = 0; j < NJ; ++j) red_max_shared_if(&tab[(uint32_t)nbr[j] & hmask], acc && nbr[j] >= 0, mark);
            red_max_shared_if(&tab[(uint32_t)sa & hmask], acc && hl == 0, mark);
          } else if (acc) {
#pragma unroll
            for (int j = 0; j < NJ; ++j)
              if (nbr[j] >= 0) {
                uint32_t *p = &tab[(uint32_t)nbr[j] & hmask];
                atomicMax(p, mark);
                if (CL == 2 && !gst) red_max_peer(peer_addr(p, peer), mark);
              }
            if (hl == 0) {
              uint32_t *p = &tab[(uint32_t)sa & hmask];
              atomicMax(p, mark);
              if (CL == 2 && !gst) red_max_peer(peer_addr(p, peer), mark);
            }
          }
        }
      } else {
        // ---- phase A: every evaluating warp computes one trial speculatively ----
        const uint64_t t = t0 + (uint64_t)gidx;
        if (active && t < t_end) {
          const uint32_t slot = (uint32_t)t & rmask;
          const Draw dr = draws[slot];
          int sa = 0, sb = -1, na = 0, A_ = 0, B_ = 0, old_a = 0;
          int nbra[4] = {-1, -1, -1, -1}, nbrb[4] = {-1, -1, -1, -1};
          uint32_t ua, ub;
          uint32_t occ_a_bit = 0, wa_lo = 0, wa_hi = 0, wb_lo = 0, wb_hi = 0;  // spin path
          // Move constraints: an illegal proposal is redrawn, proposal k of trial t from
          // counter streams 2k, 2k + 1, until one is legal or max_attempts redraws are spent
          // (montecarlo.py:976-988: spending the last redraw fails even if it is legal);
          // a failed search rejects the trial and marks the chain CEMC_ERR_NO_MOVE.
          bool no_move = false;
          if (!SWAP) {
            sa = dr.site;
            int oa = occ[sa];
            int k = (int)cemc_below(dr.w1, (uint32_t)(g.n_sym - 1));
            na = k + (k >= oa);
            ua = dr.w2;
            ub = dr.w3;
            const int32_t *frow = rows + (size_t)slot * cpad;  // prefetched by the fetcher
            if (cons) {
              int att = 0;
              while (!change_legal(allow, frz, sa, oa, na) && att < a.max_attempts) {
                ++att;
                const cemc_u32x4 w = cemc_trial_draw(a.seed, key, t, (uint32_t)(2 * att));
                sa = g.n_movable == N ? (int)cemc_below(w.v[0], (uint32_t)N)
                                      : g.movable[cemc_below(w.v[0], (uint32_t)g.n_movable)];
                oa = occ[sa];
                k = (int)cemc_below(w.v[1], (uint32_t)(g.n_sym - 1));
                na = k + (k >= oa);
                ua = w.v[2];
                ub = w.v[3];
              }
              no_move = att == a.max_attempts;
              if (att > 0) frow = g.table + (size_t)sa * cpad;  // a redrawn site's row comes from L2
            }
            old_a = oa;
            if constexpr (TAB) {
              table_gather(g, occ, row_mem(frow), -1, 0, sp_a, nbra, lane);
            } else if constexpr (!SPIN) {
              gather_smem_row<R>(g, occ, bf_s, frow, oa, na, va, nbra, lane);
            } else {
              occ_a_bit = (uint32_t)oa ^ xorv;
              spin_ballot(g, occ, row_mem(frow), xorv, -1, 0u, wa_lo, wa_hi, nbra, lane);
            }
          } else {
            int ia = (int)cemc_below(dr.w0, (uint32_t)n_present);
            int ib = (int)cemc_below(dr.w1, (uint32_t)(n_present - 1));
            ib += (ib >= ia);
            A_ = misc[4 + ia];
            B_ = misc[4 + ib];
            sa = trk[misc[12 + A_] + (int)cemc_below(dr.w2, (uint32_t)misc[20 + A_])];
            sb = trk[misc[12 + B_] + (int)cemc_below(dr.w3, (uint32_t)misc[20 + B_])];
            ua = dr.x0;
            ub = dr.x1;
            if (cons) {
              int att = 0;
              while (!(change_legal(allow, frz, sa, A_, B_) && change_legal(allow, frz, sb, B_, A_)) &&
                     att < a.max_attempts) {
                ++att;
                const cemc_u32x4 w = cemc_trial_draw(a.seed, key, t, (uint32_t)(2 * att));
                const cemc_u32x4 x = cemc_trial_draw(a.seed, key, t, (uint32_t)(2 * att + 1));
                ia = (int)cemc_below(w.v[0], (uint32_t)n_present);
                ib = (int)cemc_below(w.v[1], (uint32_t)(n_present - 1));
                ib += (ib >= ia);
                A_ = misc[4 + ia];
                B_ = misc[4 + ib];
                sa = trk[misc[12 + A_] + (int)cemc_below(w.v[2], (uint32_t)misc[20 + A_])];
                sb = trk[misc[12 + B_] + (int)cemc_below(w.v[3], (uint32_t)misc[20 + B_])];
                ua = x.v[0];
                ub = x.v[1];
              }
              no_move = att == a.max_attempts;
            }
            na = B_;
            // first half: site a takes B; second half: site b takes A with a already changed
            if constexpr (TAB) {
              table_gather(g, occ, row_of_site(g, sa), -1, 0, sp_a, nbra, lane);
              table_gather(g, occ, row_of_site(g, sb), sa, B_, sp_b, nbrb, lane);
            } else if constexpr (!SPIN) {
              gather_vals<R>(g, occ, bf_s, sa, A_, B_, -1, 0, va, nbra, lane);
              gather_vals<R>(g, occ, bf_s, sb, B_, A_, sa, B_, vb, nbrb, lane);
            } else {
              occ_a_bit = (uint32_t)A_ ^ xorv;
              spin_ballot(g, occ, row_of_site(g, sa), xorv, -1, 0u, wa_lo, wa_hi, nbra, lane);
              spin_ballot(g, occ, row_of_site(g, sb), xorv, sa, occ_a_bit ^ 1u, wb_lo, wb_hi, nbrb, lane);
            }
          }
          R de;
          int delta = 0;
          // translation groups of the changed sites (the spin form has one group)
          int ga = 0, gb = 0;
          if (!SPIN && g.n_groups > 1) {
            if (!SWAP) {
              ga = (int)dr.pad;
            } else {
              ga = g.site_group[sa];
              gb = g.site_group[sb];
            }
          }
          if constexpr (TAB) {
            __syncwarp();
            const int S = g.n_sym;
            if (!SWAP) {
              de = table_de<R, false>(g, geos_s, ftab, sp_a, sp_b, old_a * S + na, 0, gstart_s[ga], gstart_s[ga + 1],
                                      lane);
              for (int b = 0; b < g.n_bf; ++b)
                if (g.singlet_eci[b] >= 0)
                  de += coef_s[g.singlet_eci[b]] * (bf_s[b * S + na] - bf_s[b * S + old_a]);
            } else if (ga == gb) {
              de = table_de<R, true>(g, geos_s, ftab, sp_a, sp_b, A_ * S + B_, B_ * S + A_, gstart_s[ga],
                                     gstart_s[ga + 1], lane);
            } else {
              de = table_de<R, false>(g, geos_s, ftab, sp_a, sp_a, A_ * S + B_, 0, gstart_s[ga], gstart_s[ga + 1], lane) +
                   table_de<R, false>(g, geos_s, ftab, sp_b, sp_b, B_ * S + A_, 0, gstart_s[gb], gstart_s[gb + 1], lane);
            }
            __syncwarp();
          } else if constexpr (!SPIN) {
            __syncwarp();
            de = site_changes<R, SWAP>(g, terms_s, lane_term_s, kind_s, dec_s, coef_s, gscale_s, part, va, vb, Dw, ga,
                                       gb, lane);
            __syncwarp();
          } else {
            // P_k = sum over the terms of cluster ECI k of the product of the other
            // members' spins; D_k = delta * P_k with delta = -2 s_a the spin change.
            // Lane k evaluates cluster ECI k: its pair terms by popcounts of its shell
            // masks, its multi-site terms from one warp reduction per ECI that has any.
            delta = ((occ_a_bit) ? 2 : -2);
            const int first = sp_first;
            const uint32_t pa = spin_lane_parities<false>(sp_terms, sp_tlo, sp_thi, wa_lo, wa_hi);
            const uint32_t pb = SWAP ? spin_lane_parities<false>(sp_terms, sp_tlo, sp_thi, wb_lo, wb_hi) : 0u;
            int my_odd = 0;
            if (sp_pk) {
              my_odd = odd_counts_packed(pa, pb, lane, std::integral_constant<int, 32>{});
            } else {
              for (unsigned mm = sp_multi; mm; mm &= mm - 1) {
                const int k = __ffs(mm) - 1;
                const int sl = k - first;
                int v = (sl >= 0 && sl < 5) ? (int)((pa >> (6 * sl)) & 63u) : 0;
                if (SWAP) v -= (sl >= 0 && sl < 5) ? (int)((pb >> (6 * sl)) & 63u) : 0;
                const int odd = __reduce_add_sync(kFull, v);
                if (lane == k) my_odd = odd;
              }
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
              Dw[sp_e.eci] = delta * P;
            }
            R sum = warp_sum(sp_coef * (R)P);
            if (sd.singlet_eci >= 0) {
              if (lane == 0) Dw[sd.singlet_eci] = SWAP ? 0 : delta;
              if (!SWAP) sum += coef_s[sd.singlet_eci];
            }
            de = (R)delta * sum;
          }
          int acc = 0;
          if (lane == 0) {
            // accept_first_trial_move_after_reset: the call's first trial is accepted outright
            const bool first = CONS && a.accept_first && a.chunk_offset == 0 && t == t_first;
            if constexpr (RECYCLE)
              acc = no_move ? 0 : (first ? 1 : barker<R>(de, ua, ub, kT));
            else
              acc = no_move ? 0 : (first ? 1 : metropolis<R>(de, ua, ub, kT, inv_kT));
            if (CONS && no_move) put(&misc[3], 1);  // reported in the status at the end of the launch
            put(&r_sa[gidx], (int32_t)sa);
            put(&r_sb[gidx], (int32_t)(SWAP ? sb : na));
            put(&r_acc[gidx], (int8_t)acc);
            put(&r_de[gidx], de);
            for (int b = 0; b < g.n_bf; ++b) {
              R v = (R)0;
              if constexpr (SPIN)
                v = (R)(SWAP ? 0 : delta);
              else if constexpr (TAB)
                v = SWAP ? (R)0 : bf_s[b * g.n_sym + na] - bf_s[b * g.n_sym + old_a];
              else if (g.singlet_eci[b] >= 0)
                v = Dw[g.singlet_eci[b]];
              put(&r_ds[b * kRoundSlots + gidx], v);
            }
            if (SWAP) {
              put(&r_la[gidx], (int32_t)loc[sa]);
              put(&r_lb[gidx], (int32_t)loc[sb]);
              put(&r_A[gidx], (int8_t)A_);
              put(&r_B[gidx], (int8_t)B_);
            }
          }
          acc = __shfl_sync(kFull, acc, 0);
          if (CL == 1 && !gst) {
            const uint32_t mark = (round << 6) | (uint32_t)(63 - gidx);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              red_max_shared_if(&tab[(uint32_t)nbra[q] & hmask], acc && nbra[q] >= 0, mark);
              if (SWAP) red_max_shared_if(&tab[(uint32_t)nbrb[q] & hmask], acc && nbrb[q] >= 0, mark);
            }
            red_max_shared_if(&tab[(uint32_t)sa & hmask], acc && lane == 0, mark);
            if (SWAP) red_max_shared_if(&tab[(uint32_t)sb & hmask], acc && lane == 0, mark);
          } else if (acc) {
            const uint32_t mark = (round << 6) | (uint32_t)(63 - gidx);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              if (nbra[q] >= 0) {
                uint32_t *p = &tab[(uint32_t)nbra[q] & hmask];
                atomicMax(p, mark);
                if (CL == 2 && !gst) red_max_peer(peer_addr(p, peer), mark);
              }
              if (SWAP && nbrb[q] >= 0) {
                uint32_t *p = &tab[(uint32_t)nbrb[q] & hmask];
                atomicMax(p, mark);
                if (CL == 2 && !gst) red_max_peer(peer_addr(p, peer), mark);
              }
            }
            if (lane == 0) {
              uint32_t *p = &tab[(uint32_t)sa & hmask];
              atomicMax(p, mark);
              if (CL == 2 && !gst) red_max_peer(peer_addr(p, peer), mark);
              if (SWAP) {
                p = &tab[(uint32_t)sb & hmask];
                atomicMax(p, mark);
                if (CL == 2 && !gst) red_max_peer(peer_addr(p, peer), mark);
              }
            }
          }
        }
      }
      int ks;
      if (!end_round(round, t0, active, ks)) break;
      // ---- phase B: apply every accepted move of the committed prefix ----------
      {
        for (int gg = lane; gg < ks; gg += 32) {
          if (r_acc[gg]) {
            const int sa = r_sa[gg];
            if (!SWAP) {
              occ[sa] = (int8_t)r_sb[gg];
            } else {
              const int sb = r_sb[gg], A_ = r_A[gg], B_ = r_B[gg], la = r_la[gg], lb = r_lb[gg];
              occ[sa] = (int8_t)B_;
              occ[sb] = (int8_t)A_;
              trk[misc[12 + A_] + la] = sb;
              loc[sb] = la;
              trk[misc[12 + B_] + lb] = sa;
              loc[sa] = lb;
            }
          }
        }
        __syncwarp();
      }
      t0 += (uint64_t)ks;
      ++round;
    }
  } else if (booker) {
    // ---- bookers: fold round r - 1 while round r is evaluated ------------------
    int ks_prev = 0;
    while (true) {
      const bool active = t0 < t_end;
      if (round > 1)
        book(rec0 + (size_t)((round - 1) & 1) * L.rec_stride, drow + (size_t)((round - 1) & 1) * TPW * W * n_eci,
             ks_prev, t0 - (uint64_t)ks_prev);
      if constexpr (SPIN)
        if ((round & (kCfFoldRounds - 1)) == 0) cf_fold();
      int ks;
      if (!end_round(round, t0, active, ks)) break;
      ks_prev = ks;
      t0 += (uint64_t)ks;
      ++round;
    }
    if constexpr (SPIN) cf_fold();
    for (int i = 0; i < 4; ++i) {
      const int k = lane + 32 * i;
      if (k < n_eci) cfb[k] = cf_sum_out(cfr[i]);
    }
  } else {
    // ---- fetcher: draws and neighbour rows kPrefetchRounds rounds ahead --------
    while (true) {
      const bool active = t0 < t_end;
      if (active) prefetch(t0);
      cp_async_wait_prev();
      int ks;
      if (!end_round(round, t0, active, ks)) break;
      t0 += (uint64_t)ks;
      ++round;
    }
  }

  if (fetcher) cp_async_wait_all();
  if (CL == 1 && booker && lane == 0) nacc_slot[bq] = n_acc_launch;
  if (CL == 2) {
    if (booker && lane == 0) nacc_slot[CL == 1 ? bq : 0] = n_acc_launch;
    cluster_barrier();  // the peer's sums are final and readable
  } else {
    __syncthreads();
  }

  // ---- epilogue --------------------------------------------------------------
  const bool ok = misc[1] == 0;
  double sum_v = 0.0;         // thread tid < NACC: running sum `tid` over the bookers' lanes
  uint64_t n_acc_total = 0;   // thread 0 of CTA 0: accepted trials of the launch
  if (rank == 0 && ok) {
    // the launch's correlation-function changes: the bookers' sums of both CTAs
    // in fixed order (exact for integer-valued changes), then one scaling per ECI
    for (int k = tid; k < n_eci; k += blockDim.x) {
      const int kind = kind_s[k];
      double d = 0.0;
      for (int q = 0; q < NB; ++q) d += acc_to(cfw[(size_t)q * n_eci + k]);
      if (CL == 2) d += ld_peer_acc(&cfw[k], peer);
      if (kind == 2) cf_s[k] = cf_s[k] + d * w_s[k];
      else if (kind == 1) cf_s[k] = cf_s[k] + d / (double)N;
    }
    if (a.accum && tid < NACC) {
      for (int q = 0; q < NB; ++q)
        for (int l = 0; l < 32; ++l) sum_v += acc_to(lacc0[(q * NACC + tid) * 32 + l]);
      if (CL == 2)
        for (int l = 0; l < 32; ++l) sum_v += ld_peer_acc(&lacc0[tid * 32 + l], peer);
    }
    if (tid == 0) {
      n_acc_total = nacc_slot[0] + nacc_slot[1];
      if (CL == 2) {
        uint64_t v;
        asm volatile("ld.shared::cluster.u64 %0, [%1];\n" : "=l"(v) : "r"(peer_addr(nacc_slot, peer)) : "memory");
        n_acc_total += v;
      }
    }
  }
  if (CL == 2) cluster_barrier();  // CTA 1's shared memory stays alive until CTA 0 has read it
  if (rank != 0) return;
  if (!ok) {
    if (tid == 0 && a.status) a.status[chain] = misc[1];
    return;
  }
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
  __syncthreads();
  for (int k = tid; k < n_eci; k += blockDim.x) a.cf[(size_t)chain * n_eci + k] = cf_s[k];
  if (a.accum && tid < NACC) {
    const int b = tid < 2 ? 0 : (tid - 2) % CEMC_MAX_BF;
    if (tid < 2 || b < g.n_bf) {
      double *sums = &a.accum[acc_row].sum_e;  // sum_e, sum_e2, sum_s[], sum_s2[], sum_se[] in NACC order
      sums[tid] += sum_v;
    }
  }
  if (tid == 0) {
    // energy = N * eci . cf in sorted-name order (ce_updater.cpp:236-242)
    double e = 0.0;
    for (int k = 0; k < n_eci; ++k) e += eci_s[k] * cf_s[k];
    a.energy[chain] = e * (double)(unsigned)N;
    a.trial[chain] = t_end;
    if (a.accum) {
      cemc_accum *ac = a.accum + acc_row;
      ac->n_samples += my_trials;
      ac->n_accept += n_acc_total;
    }
    if (a.status) a.status[chain] = (CONS && misc[3]) ? CEMC_ERR_NO_MOVE : 0;
  }
}

// Threads of one CTA: evaluating warps, bookers, fetcher.
static unsigned block_threads(const RunArgs &a) {
  return (unsigned)((a.warps + n_bookers(a.cl, a.warps, a.tpw) + 1) * 32);
}

template <typename R, int MOVE, int FORM, int CL, int TPW, bool CONS = false>
static cudaError_t launch_t(const DevGeo &g, const RunArgs &a, size_t smem, cudaStream_t st, const SpinDev &sd) {
  auto k = mc_kernel<R, MOVE, FORM, CL, TPW, CONS>;
  if (block_threads(a) > kMcMaxThreads) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(a.n_chains * CL));
  cfg.blockDim = dim3(block_threads(a));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = (CL == 2) ? 1 : 0;
  e = cudaLaunchKernelEx(&cfg, k, g, a, sd);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <typename R, int MOVE, int FORM>
static int clusters_t(const RunArgs &a, size_t smem) {
  auto k = mc_kernel<R, MOVE, FORM, 2, 1, false>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(a.n_chains * 2));
  cfg.blockDim = dim3(block_threads(a));
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

template <typename R, int MOVE, int FORM>
static cudaError_t launch_f(const DevGeo &g, const RunArgs &a, size_t smem, cudaStream_t st, const SpinDev &sd) {
  if (a.cons) return launch_t<R, MOVE, FORM, 1, 1, true>(g, a, smem, st, sd);  // one CTA per chain (host checks)
  return a.cl == 2 ? launch_t<R, MOVE, FORM, 2, 1>(g, a, smem, st, sd) : launch_t<R, MOVE, FORM, 1, 1>(g, a, smem, st, sd);
}

template <typename R>
static cudaError_t launch_r(const DevGeo &g, const RunArgs &a, int move, size_t smem, cudaStream_t st, int form,
                            const SpinDev *spin) {
  const SpinDev none{};
  if (move == CEMC_MOVE_SWAP) {
    if (form == kFormSpin) return launch_f<R, CEMC_MOVE_SWAP, kFormSpin>(g, a, smem, st, *spin);
    if (form == kFormTable) return launch_f<R, CEMC_MOVE_SWAP, kFormTable>(g, a, smem, st, none);
    return launch_f<R, CEMC_MOVE_SWAP, kFormGeneric>(g, a, smem, st, none);
  }
  if (form == kFormSpin) {
    if (a.tpw == 4) return launch_t<R, CEMC_MOVE_FLIP, kFormSpin, 1, 4>(g, a, smem, st, *spin);
    if (a.tpw == 2)
      return a.cl == 2 ? launch_t<R, CEMC_MOVE_FLIP, kFormSpin, 2, 2>(g, a, smem, st, *spin)
                       : launch_t<R, CEMC_MOVE_FLIP, kFormSpin, 1, 2>(g, a, smem, st, *spin);
    return launch_f<R, CEMC_MOVE_FLIP, kFormSpin>(g, a, smem, st, *spin);
  }
  if (form == kFormTable) return launch_f<R, CEMC_MOVE_FLIP, kFormTable>(g, a, smem, st, none);
  return launch_f<R, CEMC_MOVE_FLIP, kFormGeneric>(g, a, smem, st, none);
}

template <typename R>
static cudaError_t launch_recycle(const DevGeo &g, const RunArgs &a, int move, size_t smem, cudaStream_t st) {
  const SpinDev none{};
  return move == CEMC_MOVE_SWAP ? launch_t<R, CEMC_MOVE_SWAP, kFormRecycle, 1, 1, true>(g, a, smem, st, none)
                                : launch_t<R, CEMC_MOVE_FLIP, kFormRecycle, 1, 1, true>(g, a, smem, st, none);
}

cudaError_t launch_mc(const DevGeo &g, const RunArgs &a, int move, int precision, size_t smem, cudaStream_t st,
                      int form, const SpinDev *spin) {
  // two trials per warp: spin flips on one CTA per chain only (checked by the caller)
  if (a.tpw >= 2 && (form != kFormSpin || move != CEMC_MOVE_FLIP || a.cons)) return cudaErrorInvalidValue;
  if (a.tpw == 4 && a.cl != 1) return cudaErrorInvalidValue;
  if (a.cons && a.cl != 1) return cudaErrorInvalidValue;
  if (form == kFormSpin && !spin) return cudaErrorInvalidValue;
  if (form == kFormRecycle) {
    if (a.cl != 1 || a.tpw != 1) return cudaErrorInvalidValue;
    return precision == CEMC_PREC_F32 ? launch_recycle<float>(g, a, move, smem, st)
                                      : launch_recycle<double>(g, a, move, smem, st);
  }
  return precision == CEMC_PREC_F32 ? launch_r<float>(g, a, move, smem, st, form, spin)
                                    : launch_r<double>(g, a, move, smem, st, form, spin);
}

template <typename R, int FORM>
static int clusters_m(const RunArgs &a, int move, size_t smem) {
  return move == CEMC_MOVE_SWAP ? clusters_t<R, CEMC_MOVE_SWAP, FORM>(a, smem) : clusters_t<R, CEMC_MOVE_FLIP, FORM>(a, smem);
}

int max_active_clusters(const DevGeo &, const RunArgs &a, int move, int precision, size_t smem, int form) {
  const bool f32 = precision == CEMC_PREC_F32;
  if (form == kFormSpin) return f32 ? clusters_m<float, kFormSpin>(a, move, smem) : clusters_m<double, kFormSpin>(a, move, smem);
  if (form == kFormTable) return f32 ? clusters_m<float, kFormTable>(a, move, smem) : clusters_m<double, kFormTable>(a, move, smem);
  return f32 ? clusters_m<float, kFormGeneric>(a, move, smem) : clusters_m<double, kFormGeneric>(a, move, smem);
}

}  // namespace cemc
