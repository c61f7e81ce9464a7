// Local-field Monte Carlo kernel: semi-grand-canonical single-site flips in a
// binary +1/-1 basis with the per-site cluster counts kept in shared memory
// (tables and layout: cemc_field.h).
//
// Same chain as mc_kernel (cemc_mc.cu) and the reference's _mc_step loop
// (cemc/mcmc/montecarlo.py:970-1038 over CEUpdater::calculate,
// cpp/src/ce_updater.cpp:313-406): trial t of a chain draws its site and
// uniform from the counter-based stream, and the committed chain is exactly the
// sequential Metropolis chain over that stream.  What changes is the cost of a
// trial.  Every site i of the chain carries c_k(i), the number of terms of
// cluster ECI k at reference site i whose member product is -1, packed into one
// or two words; a trial's energy change is a dot product of those counts with
// the chain's coefficients, computed by ONE lane.  An accepted flip of site j
// changes the counts of the sites that share a cluster with j: for each such
// target the pair terms toggle with s_j and each multi-site term through j
// toggles with the parity of its other members, read from a 64-bit spin word of
// j's neighbour row.  Those increments are packed like the counts, so one
// shared-memory atomicAdd per target word applies them.
//
// A round of up to 64 trials:
//   phase A  the worker warps evaluate the round's trials (one lane each) against
//            the state at the start of the round and record them; for each of
//            its accepted trials a warp stamps the trial's neighbourhood with
//            (round, trial) into the conflict table (atomicMax keeps the earliest
//            trial), records the spin word of the trial's neighbour row and
//            appends the trial to the round's list of accepted trials;
//   barrier  every warp finds the committed prefix: trials before the first
//            one whose site an earlier accepted trial stamped (an exact test:
//            the neighbour row of a site lists every site sharing a cluster
//            with it, and the relation is symmetric);
//   phase B  the committed accepted flips update the counts of their neighbours
//            and their own occupation, as units of (flip, 32 columns) spread
//            over the worker warps, one target column per lane.  Two
//            committed flips never share a cluster (that would have been a
//            conflict), so their updates commute and read stable spins;
//   barrier  the next round sees the committed state.
// Two fetcher warps draw the trials and copy their neighbour rows into a
// shared-memory ring with cp.async three or more rounds ahead; one or two
// booker warps fold each finished round into the running sums and the
// correlation-function changes one round late, as in mc_kernel.
#include <cuda_runtime.h>

#include <type_traits>

#include "cemc_device.cuh"
#include "cemc_field.h"
#include "cemc_launch.h"

namespace cemc {

namespace {

__device__ __forceinline__ void fcp_async16(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void fcp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void fcp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void fcp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

struct FieldDraw {
  int32_t site;
  uint32_t ua, ub, pad;
};

}  // namespace

template <typename R>
__global__ void __launch_bounds__(1024, 1) field_kernel(DevGeo g, RunArgs a, FieldDev fd) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int W = a.warps;            // worker warps
  const int CW = field_round(W);    // trials per round
  const int TW = (CW + W - 1) / W;  // trials a worker warp evaluates per round
  const int NB = CW > 32 ? 2 : 1;   // booker warps
  constexpr int NF = kFieldFetchers;
  const bool gst = a.gstamp != nullptr;
  const FieldLayout L = field_layout(g, fd.n_cl, fd.pw, fd.n_cnt, fd.n_upd, (int)sizeof(R), a.ring_bits, gst);
  const uint32_t rmask = (1u << a.ring_bits) - 1u;
  const int pf = (int)((1u << a.ring_bits) / (uint32_t)CW);  // rounds the fetcher runs ahead (>= 3)
  const int chain = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool worker = warp < W;
  const bool booker = !worker && warp < W + NB;
  const bool fetcher = warp >= W + NB && warp < W + NB + NF;
  const int bq = booker ? warp - W : 0;
  const int fq = fetcher ? warp - W - NB : 0;
  const int N = g.n_sites, n_eci = g.n_eci, cpad = g.cpad, n_cols = g.n_cols;
  const int PW = fd.pw, NCL = fd.n_cl;
  const uint32_t xorv = (uint32_t)(fd.minus_id ^ 1);  // spin bit = occ ^ xorv (1 = the -1 species)

  constexpr bool DF = (sizeof(R) == 4);
  using A = typename std::conditional<DF, df64, double>::type;
  constexpr int NACC = 2 + 3 * CEMC_MAX_BF;
  double *cf_s = reinterpret_cast<double *>(smem + L.cf);
  double *eci_s = reinterpret_cast<double *>(smem + L.eci);
  double *w_s = reinterpret_cast<double *>(smem + L.w);
  A *lacc0 = reinterpret_cast<A *>(smem + L.acc);  // [2][NACC][32]
  A *lacc = lacc0 + bq * NACC * 32;
  A *s_start = lacc0 + 2 * NACC * 32;  // singlet at launch start, then 1/N
  A *cfw = reinterpret_cast<A *>(smem + L.cfw);  // [2][n_eci]
  R *coef_s = reinterpret_cast<R *>(smem + L.coef);
  int8_t *kind_s = reinterpret_cast<int8_t *>(smem + L.kind);
  int32_t *misc = reinterpret_cast<int32_t *>(smem + L.misc);  // [1] status
  uint64_t *nacc_slot = reinterpret_cast<uint64_t *>(misc + 36);
  uint32_t *meta_s = reinterpret_cast<uint32_t *>(smem + L.meta);
  R *scoef_s = reinterpret_cast<R *>(smem + L.scoef);
  uint4 *cnt_s = reinterpret_cast<uint4 *>(smem + L.cnt);
  uint2 *pairinc_s = reinterpret_cast<uint2 *>(smem + L.pairinc);
  int32_t *ustart_s = reinterpret_cast<int32_t *>(smem + L.ustart);
  uint4 *upd_s = reinterpret_cast<uint4 *>(smem + L.upd);
  unsigned char *rec0 = smem + L.rec;
  int32_t *alist0 = reinterpret_cast<int32_t *>(smem + L.alist);  // [2][kFieldRound + 1], count last
  FieldDraw *draws = reinterpret_cast<FieldDraw *>(smem + L.draws);
  int32_t *rows = reinterpret_cast<int32_t *>(smem + L.rows);
  uint32_t *stamp = gst ? a.gstamp + (size_t)chain * ((size_t)2 << a.stamp_bits)
                        : reinterpret_cast<uint32_t *>(smem + L.stamp);
  uint32_t *pc = reinterpret_cast<uint32_t *>(smem + L.pc);  // packed counts [N][PW]
  int8_t *occ = reinterpret_cast<int8_t *>(smem + L.occ);

  // A chain with no trials in this launch (an empty serving slot) leaves its state untouched.
  if (a.chain_trials && a.chain_trials[chain] <= a.chunk_offset) return;

  // ---- prologue: tables and the chain's state --------------------------------
  for (int k = tid; k < n_eci; k += blockDim.x) {
    const int kind = g.eci_kind[k];
    const double e = a.eci[(size_t)chain * n_eci + k];
    cf_s[k] = a.cf[(size_t)chain * n_eci + k];
    eci_s[k] = e;
    w_s[k] = (kind == 2) ? g.eci_w[k] : 0.0;
    coef_s[k] = (R)(kind == 2 ? e * (double)N * g.eci_w[k] : (kind == 1 ? e : 0.0));
    kind_s[k] = (int8_t)kind;
  }
  for (int q = tid; q < NCL; q += blockDim.x) {
    const int k = fd.slot_eci[q];
    meta_s[q] = fd.slot_meta[q];
    scoef_s[q] = (R)(a.eci[(size_t)chain * n_eci + k] * (double)N * g.eci_w[k]);
  }
  for (int e = tid; e < fd.n_cnt; e += blockDim.x) cnt_s[e] = fd.cnt[e];
  for (int c = tid; c < n_cols; c += blockDim.x) pairinc_s[c] = fd.pairinc[c];
  for (int c = tid; c <= n_cols; c += blockDim.x) ustart_s[c] = fd.ustart[c];
  for (int e = tid; e < fd.n_upd; e += blockDim.x) upd_s[e] = fd.upd[e];
  for (int i = tid; i < 2 * n_eci; i += blockDim.x) cfw[i] = acc_from<A>(0.0);
  for (int i = tid; i < 2 * NACC * 32; i += blockDim.x) lacc0[i] = acc_from<A>(0.0);
  for (int i = tid; i < N; i += blockDim.x) stamp[i] = 0u;
  {
    const int8_t *src = a.occ + (size_t)chain * N;
    for (int i = tid; i < N; i += blockDim.x) occ[i] = src[i];
  }
  if (tid == 0) {
    misc[1] = 0;
    nacc_slot[0] = nacc_slot[1] = 0;
    alist0[kFieldRound] = alist0[2 * kFieldRound + 1] = 0;
    for (int b = 0; b < CEMC_MAX_BF; ++b)
      s_start[b] = acc_from<A>((b < g.n_bf && g.singlet_eci[b] >= 0) ? a.cf[(size_t)chain * n_eci + g.singlet_eci[b]]
                                                                     : 0.0);
    s_start[CEMC_MAX_BF] = acc_from<A>(1.0 / (double)N);
  }
  __syncthreads();
  // Packed counts of every site from its neighbour row: pair entries count the
  // -1 spins under their shell mask, multi-site entries add their parity.
  for (int i = tid; i < N; i += blockDim.x) {
    const int32_t *row = g.table + (size_t)i * cpad;
    uint32_t lo = 0, hi = 0;
    for (int c = 0; c < n_cols; c += 4) {
      const int4 v = __ldg(reinterpret_cast<const int4 *>(row + c));
      const int s4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int cc = c + q;
        if (cc < n_cols) {
          const uint32_t b = ((uint32_t)occ[s4[q]] ^ xorv) & 1u;
          if (cc < 32) lo |= b << cc;
          else hi |= b << (cc - 32);
        }
      }
    }
    uint32_t w0 = 0, w1 = 0;
    for (int e = 0; e < fd.n_cnt; ++e) {
      const uint4 m = cnt_s[e];
      uint32_t v = (uint32_t)(__popc(lo & m.x) + __popc(hi & m.y));
      if (e >= NCL) v &= 1u;
      w0 += v * m.z;
      w1 += v * m.w;
    }
    pc[(size_t)i * PW] = w0;
    if (PW == 2) pc[(size_t)i * PW + 1] = w1;
  }

  const double kT = a.kT[chain];
  const float inv_kT = (float)(1.0 / kT);
  const uint32_t key = a.chain_key ? a.chain_key[chain] : (uint32_t)chain;
  uint64_t my_trials = a.n_trials;
  if (a.chain_trials) {
    const uint64_t total = a.chain_trials[chain];
    my_trials = total <= a.chunk_offset ? 0 : (total - a.chunk_offset < a.n_trials ? total - a.chunk_offset : a.n_trials);
  }
  const uint64_t t_first = a.trial[chain];
  const uint64_t t_end = t_first + my_trials;
  const int acc_row = a.accum_slot ? a.accum_slot[chain] : chain;
  const double e_ref = a.accum ? a.accum[acc_row].e_ref : 0.0;

  A eoff = acc_from<A>(a.energy[chain] - e_ref);  // booker state: energy relative to e_ref
  A dsum = acc_from<A>(0.0);                     // summed singlet changes of the launch
  uint64_t n_acc_launch = 0;
  uint64_t fill_end = t_first;

  // Draws and neighbour rows of trials [fill_end, min(t0 + pf * CW, t_end)).
  auto prefetch = [&](uint64_t t0) {
    uint64_t want = t0 + (uint64_t)pf * (uint64_t)CW;
    if (want > t_end) want = t_end;
    for (uint64_t t = fill_end + (uint64_t)(32 * fq + lane); t < want; t += 32 * NF) {
      const uint32_t slot = (uint32_t)t & rmask;
      const cemc_u32x4 w0 = cemc_trial_draw(a.seed, key, t, 0);
      FieldDraw d;
      d.site = (int)cemc_below(w0.v[0], (uint32_t)N);
      d.ua = w0.v[2];
      d.ub = w0.v[3];
      d.pad = 0;
      const int32_t *src = g.table + (size_t)d.site * cpad;
      int32_t *dst = rows + (size_t)slot * cpad;
      for (int q = 0; q < cpad; q += 4) fcp_async16(dst + q, src + q);
      draws[slot] = d;
    }
    if (want > fill_end) fill_end = want;
    fcp_async_commit();
  };

  // Committed prefix of round `round` (trials t0 ..): the first trial whose site an
  // earlier accepted trial of the round stamped.  Same value on every warp.
  auto prefix = [&](uint32_t round, uint64_t t0) -> int {
    const unsigned char *rec = rec0 + (size_t)(round & 1) * L.rec_stride;
    const int32_t *r_sa = reinterpret_cast<const int32_t *>(rec + L.rec_sa);
    const int nv = (t_end - t0) < (uint64_t)CW ? (int)(t_end - t0) : CW;
    auto conflicted = [&](int gg) {
      const uint32_t v = stamp[r_sa[gg]];
      return ((v >> 6) == round) && ((uint32_t)(63 - (v & 63u)) < (uint32_t)gg);
    };
    const bool c0 = lane < nv && conflicted(lane);
    const bool c1 = lane + 32 < nv && conflicted(lane + 32);
    const unsigned m0 = __ballot_sync(kFull, c0);
    const unsigned m1 = __ballot_sync(kFull, c1);
    return m0 ? (__ffs(m0) - 1) : (m1 ? (31 + __ffs(m1)) : nv);
  };

  // ---- booker helpers (round records of round r - 1) --------------------------
  auto book_half = [&](const unsigned char *rec, int off, int kh, uint64_t tb) {
    const int8_t *r_acc = reinterpret_cast<const int8_t *>(rec + L.rec_acc);
    const R *r_de = reinterpret_cast<const R *>(rec + L.rec_de);
    const R *r_ds = reinterpret_cast<const R *>(rec + L.rec_ds);
    const int gg = off + lane;
    const bool mine = lane < kh;
    const bool acc = mine && r_acc[gg];
    if (a.trace_acc && mine) {
      const int32_t *r_sa = reinterpret_cast<const int32_t *>(rec + L.rec_sa);
      const int8_t *r_ns = reinterpret_cast<const int8_t *>(rec + L.rec_ns);
      const size_t idx = (size_t)chain * a.n_trials + (size_t)(tb + (uint64_t)gg - t_first);
      a.trace_site[2 * idx] = r_sa[gg];
      a.trace_site[2 * idx + 1] = (int32_t)r_ns[gg];
      a.trace_acc[idx] = r_acc[gg];
      a.trace_de[idx] = (double)r_de[gg];
    }
    const unsigned am = __ballot_sync(kFull, acc);
    n_acc_launch += (uint64_t)__popc(am);
    if (!a.accum) return;
    R x = acc ? r_de[gg] : (R)0;
    R ds = acc ? r_ds[gg] : (R)0;
    if (am) {
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const R nx = __shfl_up_sync(kFull, x, o);
        const R nd = __shfl_up_sync(kFull, ds, o);
        if (lane >= o) {
          x += nx;
          ds += nd;
        }
      }
    }
    if (mine) {
      const A ve = acc_add_x(eoff, x);
      lacc[lane] = acc_add(lacc[lane], ve);
      lacc[32 + lane] = acc_add(lacc[32 + lane], acc_mul(ve, ve));
      if (g.n_bf > 0) {
        const A vs = acc_add(s_start[0], acc_mul(acc_add_x(dsum, ds), s_start[CEMC_MAX_BF]));
        A *l = lacc + 2 * 32 + lane;
        l[0] = acc_add(l[0], vs);
        l[CEMC_MAX_BF * 32] = acc_add(l[CEMC_MAX_BF * 32], acc_mul(vs, vs));
        l[2 * CEMC_MAX_BF * 32] = acc_add(l[2 * CEMC_MAX_BF * 32], acc_mul(vs, ve));
      }
    }
    if (am) {
      eoff = acc_add_x(eoff, __shfl_sync(kFull, x, kh - 1));
      dsum = acc_add_x(dsum, __shfl_sync(kFull, ds, kh - 1));
    }
  };
  auto carry_half = [&](const unsigned char *rec, int off, int kh) {
    if (!a.accum) return;
    const int8_t *r_acc = reinterpret_cast<const int8_t *>(rec + L.rec_acc);
    const R *r_de = reinterpret_cast<const R *>(rec + L.rec_de);
    const R *r_ds = reinterpret_cast<const R *>(rec + L.rec_ds);
    const int gg = off + lane;
    const bool acc = lane < kh && r_acc[gg];
    if (!__ballot_sync(kFull, acc)) return;
    eoff = acc_add_x(eoff, warp_sum(acc ? r_de[gg] : (R)0));
    dsum = acc_add_x(dsum, warp_sum(acc ? r_ds[gg] : (R)0));
  };
  // Correlation-function changes of the committed accepted trials in this
  // booker's half (lane j takes trial 32 bq + j): delta * (K_q - 2 c_q) per
  // cluster slot q, summed over the lanes with one reduction per slot and kept
  // by lane q as an exact 64-bit integer; the singlet change is the sum of delta.
  long long cfr = 0, sing = 0;
  auto book_cf = [&](const unsigned char *rec, int ks) {
    const int8_t *r_acc = reinterpret_cast<const int8_t *>(rec + L.rec_acc);
    const int8_t *r_dl = reinterpret_cast<const int8_t *>(rec + L.rec_dl);
    const uint32_t *r_p = reinterpret_cast<const uint32_t *>(rec + L.rec_p);
    const int gg = 32 * bq + lane;
    const bool v = gg < ks && r_acc[gg];
    if (!__ballot_sync(kFull, v)) return;
    const int dl = v ? (int)r_dl[gg] : 0;
    const uint32_t p0 = v ? r_p[2 * gg] : 0u, p1 = v ? r_p[2 * gg + 1] : 0u;
    sing += (long long)__reduce_add_sync(kFull, dl);
    for (int q = 0; q < NCL; ++q) {
      const uint32_t m = meta_s[q];
      const uint32_t bits = (m >> 16) & 31u;
      const int c = (int)(((((m >> 13) & 1u) ? p1 : p0) >> ((m >> 8) & 31u)) & ((1u << bits) - 1u));
      const int tot = __reduce_add_sync(kFull, dl * ((int)(m & 255u) - 2 * c));
      if (lane == q) cfr += (long long)tot;
    }
  };
  auto book = [&](const unsigned char *rec, int ks, uint64_t tb) {
    const int k0 = ks < 32 ? ks : 32, k1 = ks - k0;
    if (bq == 0) {
      book_half(rec, 0, k0, tb);
      if (k1 > 0) carry_half(rec, 32, k1);
    } else {
      carry_half(rec, 0, k0);
      if (k1 > 0) book_half(rec, 32, k1, tb);
    }
    book_cf(rec, ks);
  };

  __syncthreads();  // counts complete
  if (fetcher) {
    prefetch(t_first);
    fcp_async_wait_all();
  }
  __syncthreads();

  uint64_t t0 = t_first;
  uint32_t round = 1;
  if (worker) {
    const int g0 = warp * TW;
    while (true) {
      const bool active = t0 < t_end;
      unsigned char *rec = rec0 + (size_t)(round & 1) * L.rec_stride;
      int32_t *r_sa = reinterpret_cast<int32_t *>(rec + L.rec_sa);
      int8_t *r_ns = reinterpret_cast<int8_t *>(rec + L.rec_ns);
      int8_t *r_acc = reinterpret_cast<int8_t *>(rec + L.rec_acc);
      int8_t *r_dl = reinterpret_cast<int8_t *>(rec + L.rec_dl);
      R *r_de = reinterpret_cast<R *>(rec + L.rec_de);
      R *r_ds = reinterpret_cast<R *>(rec + L.rec_ds);
      uint32_t *r_p = reinterpret_cast<uint32_t *>(rec + L.rec_p);
      uint2 *r_sw = reinterpret_cast<uint2 *>(rec + L.rec_sw);
      int32_t *alist = alist0 + (round & 1) * (kFieldRound + 1);
      // ---- phase A: one lane per trial ---------------------------------------
      int site = 0;
      bool acc = false;
      if (active && lane < TW) {
        const int gg = g0 + lane;
        const uint64_t t = t0 + (uint64_t)gg;
        if (gg < CW && t < t_end) {
          const FieldDraw d = draws[(uint32_t)t & rmask];
          site = d.site;
          const int o = occ[site];
          const uint32_t b = ((uint32_t)o ^ xorv) & 1u;
          const uint32_t p0 = pc[(size_t)site * PW];
          const uint32_t p1 = PW == 2 ? pc[(size_t)site * PW + 1] : 0u;
          R sum = (R)0;
          for (int q = 0; q < NCL; ++q) {
            const uint32_t m = meta_s[q];
            const uint32_t wv = ((m >> 13) & 1u) ? p1 : p0;
            const uint32_t bits = (m >> 16) & 31u;
            const int c = (int)((wv >> ((m >> 8) & 31u)) & ((1u << bits) - 1u));
            sum += scoef_s[q] * (R)((int)(m & 255u) - 2 * c);
          }
          if (fd.singlet_eci >= 0) sum += coef_s[fd.singlet_eci];
          const int dl = b ? 2 : -2;  // s_new - s_old
          const R de = (R)dl * sum;
          acc = metropolis<R>(de, d.ua, d.ub, kT, inv_kT) != 0;
          r_sa[gg] = site;
          r_ns[gg] = (int8_t)(o ^ 1);
          r_acc[gg] = (int8_t)acc;
          r_dl[gg] = (int8_t)dl;
          r_de[gg] = de;
          r_ds[gg] = (R)dl;
          r_p[2 * gg] = p0;
          r_p[2 * gg + 1] = p1;
        }
      }
      // this warp's accepted trials: conflict stamps on the site and its row, the spin word
      // of the row (the state phase B reads if the trial commits), an entry in the round's list
      unsigned am = __ballot_sync(kFull, acc);
      while (am) {
        const int l = __ffs(am) - 1;
        am &= am - 1;
        const int gg = g0 + l;
        const int s = __shfl_sync(kFull, site, l);
        const uint32_t mark = (round << 6) | (uint32_t)(63 - gg);
        const int32_t *row = rows + (size_t)((uint32_t)(t0 + (uint64_t)gg) & rmask) * cpad;
        const int s0 = lane < n_cols ? row[lane] : -1;
        const int s1 = lane + 32 < n_cols ? row[lane + 32] : -1;
        if (s0 >= 0) atomicMax(&stamp[s0], mark);
        if (s1 >= 0) atomicMax(&stamp[s1], mark);
        const uint32_t lo = __ballot_sync(kFull, s0 >= 0 && (((uint32_t)occ[s0] ^ xorv) & 1u));
        const uint32_t hi = __ballot_sync(kFull, s1 >= 0 && (((uint32_t)occ[s1] ^ xorv) & 1u));
        if (lane == 0) {
          atomicMax(&stamp[s], mark);
          r_sw[gg] = make_uint2(lo, hi);
          alist[atomicAdd(&alist[kFieldRound], 1)] = gg;
        }
      }
      __syncthreads();  // records and stamps of the round are complete
      if (!active) break;
      const int ks = prefix(round, t0);
      // ---- phase B: committed accepted flips as (flip, column half) units --------
      {
        const int na = alist[kFieldRound];  // accepted trials of the round, committed or not
        if (warp == 0 && lane == 0) alist0[((round + 1) & 1) * (kFieldRound + 1) + kFieldRound] = 0;
        for (int u = warp; u < 2 * na; u += W) {
          const int gg = alist[u >> 1], h = u & 1;
          if (gg >= ks) continue;  // not committed: re-evaluated next round
          const int ns = r_ns[gg];
          const uint32_t bj = ((uint32_t)(ns ^ 1) ^ xorv) & 1u;  // spin bit of the site before the flip
          const uint32_t bjm = 0u - bj;
          const uint2 sw = r_sw[gg];
          const int c = lane + 32 * h;
          if (c < n_cols) {
            const int32_t *row = rows + (size_t)((uint32_t)(t0 + (uint64_t)gg) & rmask) * cpad;
            const int target = row[c];
            const uint2 pi = pairinc_s[c];
            uint32_t d0 = bj ? 0u - pi.x : pi.x;
            uint32_t d1 = bj ? 0u - pi.y : pi.y;
            const uint32_t xl = sw.x ^ bjm, xh = sw.y ^ bjm;
            const int e1 = ustart_s[c + 1];
#pragma unroll 4
            for (int e = ustart_s[c]; e < e1; ++e) {
              const uint4 ue = upd_s[e];
              // kind 1: members - 2 x (members whose spin differs from s_j's); kind 0: +-1 by parity
              const int odd = __popc(xl & ue.x) + __popc(xh & ue.y);
              const uint32_t par = bj ^ ((uint32_t)__popc((sw.x & ue.x) ^ (sw.y & ue.y)) & 1u);
              const uint32_t v = (ue.w & 2u) ? ue.z * (uint32_t)((int)(ue.w >> 8) - 2 * odd) : (par ? 0u - ue.z : ue.z);
              if (ue.w & 1u) d1 += v;
              else d0 += v;
            }
            if (d0) atomicAdd(&pc[(size_t)target * PW], d0);
            if (PW == 2 && d1) atomicAdd(&pc[(size_t)target * PW + 1], d1);
          }
          if (h == 0 && lane == 0) occ[r_sa[gg]] = (int8_t)ns;
        }
      }
      __syncthreads();  // the next round reads the committed counts and occupation
      t0 += (uint64_t)ks;
      ++round;
    }
  } else if (booker) {
    int ks_prev = 0;
    while (true) {
      const bool active = t0 < t_end;
      if (round > 1) book(rec0 + (size_t)((round - 1) & 1) * L.rec_stride, ks_prev, t0 - (uint64_t)ks_prev);
      __syncthreads();
      if (!active) break;
      const int ks = prefix(round, t0);
      __syncthreads();
      ks_prev = ks;
      t0 += (uint64_t)ks;
      ++round;
    }
    A *cfb = cfw + (size_t)bq * n_eci;
    if (lane < NCL) cfb[fd.slot_eci[lane]] = acc_from<A>((double)cfr);
    if (lane == 0 && fd.singlet_eci >= 0) cfb[fd.singlet_eci] = acc_from<A>((double)sing);
    if (lane == 0) nacc_slot[bq] = n_acc_launch;
  } else if (fetcher) {
    while (true) {
      const bool active = t0 < t_end;
      if (active) prefetch(t0);
      fcp_async_wait_prev();
      __syncthreads();
      if (!active) break;
      const int ks = prefix(round, t0);
      __syncthreads();
      t0 += (uint64_t)ks;
      ++round;
    }
    fcp_async_wait_all();
  } else {
    // threads beyond the roles (none with the host's launch shape) only meet the barriers
    while (true) {
      const bool active = t0 < t_end;
      __syncthreads();
      if (!active) break;
      const int ks = prefix(round, t0);
      __syncthreads();
      t0 += (uint64_t)ks;
      ++round;
    }
  }
  __syncthreads();

  // ---- epilogue ---------------------------------------------------------------
  if (misc[1] != 0) {
    if (tid == 0 && a.status) a.status[chain] = misc[1];
    return;
  }
  double sum_v = 0.0;
  for (int k = tid; k < n_eci; k += blockDim.x) {
    const int kind = kind_s[k];
    double d = 0.0;
    for (int q = 0; q < NB; ++q) d += acc_to(cfw[(size_t)q * n_eci + k]);
    if (kind == 2) cf_s[k] = cf_s[k] + d * w_s[k];
    else if (kind == 1) cf_s[k] = cf_s[k] + d / (double)N;
  }
  if (a.accum && tid < NACC)
    for (int q = 0; q < NB; ++q)
      for (int l = 0; l < 32; ++l) sum_v += acc_to(lacc0[(q * NACC + tid) * 32 + l]);
  {
    int8_t *dst = a.occ + (size_t)chain * N;
    for (int i = tid; i < N; i += blockDim.x) dst[i] = occ[i];
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
    double e = 0.0;
    for (int k = 0; k < n_eci; ++k) e += eci_s[k] * cf_s[k];  // energy = N * eci . cf (ce_updater.cpp:236-242)
    a.energy[chain] = e * (double)(unsigned)N;
    a.trial[chain] = t_end;
    if (a.accum) {
      cemc_accum *ac = a.accum + acc_row;
      ac->n_samples += my_trials;
      ac->n_accept += nacc_slot[0] + nacc_slot[1];
    }
    if (a.status) a.status[chain] = 0;
  }
}

template <typename R>
static cudaError_t launch_field_t(const DevGeo &g, const RunArgs &a, const FieldDev &fd, size_t smem, cudaStream_t st) {
  auto k = field_kernel<R>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<dim3((unsigned)a.n_chains), dim3((unsigned)field_threads(a.warps)), smem, st>>>(g, a, fd);
  return cudaGetLastError();
}

cudaError_t launch_field(const DevGeo &g, const RunArgs &a, const FieldDev &fd, int precision, size_t smem,
                         cudaStream_t st) {
  if (a.warps < 1 || a.warps > kFieldMaxWarps) return cudaErrorInvalidValue;
  return precision == CEMC_PREC_F32 ? launch_field_t<float>(g, a, fd, smem, st)
                                    : launch_field_t<double>(g, a, fd, smem, st);
}

}  // namespace cemc
