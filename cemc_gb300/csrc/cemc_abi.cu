// C ABI of libcemc_gb300.so (declared in include/cemc_gb300.h).
//
// Host-side work here: validating descriptors, packing a geometry's cluster
// terms into the per-lane chunks the kernels walk, sizing shared memory and
// launching.  No entry point throws; failures return a status code and leave a
// message for cemc_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <array>
#include <map>
#include <mutex>
#include <tuple>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cemc_field.h"
#include "cemc_kernels.h"
#include "cemc_spin.h"

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(CEMC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

struct cemc_geometry {
  cemc::DevGeo g;
  cemc::SpinDev spin{};  // tables of the binary spin-basis kernel (spin_ok)
  bool spin_ok = false;
  cemc::FieldDev field{};  // tables of the local-field kernel (field_ok)
  bool field_ok = false;
  void *dev = nullptr;  // one device allocation holding every table
  size_t dev_bytes = 0;  // its size
  int max_smem = 0;     // opt-in shared memory per block of the current device
  int n_sms = 0;        // multiprocessors of the current device
  // resident cluster pairs per launch configuration (warps, move, precision, spin, smem)
  mutable std::mutex mu;
  mutable std::map<std::tuple<int, int, int, int, size_t>, int> pairs;
};

extern "C" int cemc_last_error(char *buf, size_t len) {
  if (!buf || len == 0) return CEMC_ERR_ARG;
  snprintf(buf, len, "%s", g_err.c_str());
  return CEMC_OK;
}

extern "C" int cemc_version(int32_t *major, int32_t *minor, int32_t *sm) {
  if (major) *major = 1;
  if (minor) *minor = 0;
  if (sm) *sm = 103;
  return CEMC_OK;
}

extern "C" int cemc_geometry_create(const cemc_geometry_desc *d, cemc_geometry **out) {
  if (!d || !out) return fail(CEMC_ERR_ARG, "null descriptor or output");
  *out = nullptr;
  const int N = d->n_sites, C = d->n_cols, S = d->n_sym, B = d->n_bf, K = d->n_eci, T = d->n_terms;
  if (N <= 0 || C <= 0 || K <= 0 || T < 0) return fail(CEMC_ERR_ARG, "empty geometry");
  if (C > CEMC_MAX_COLS) return fail(CEMC_ERR_LIMIT, "%d neighbour columns exceed the limit %d", C, CEMC_MAX_COLS);
  if (B < 1 || B > CEMC_MAX_BF || S != B + 1 || S > 8)
    return fail(CEMC_ERR_LIMIT, "unsupported species count %d", S);
  if (K > CEMC_MAX_ECI) return fail(CEMC_ERR_LIMIT, "%d ECIs exceed the limit %d", K, CEMC_MAX_ECI);
  if (!d->table || !d->bf || !d->eci_kind || !d->eci_dec || !d->eci_weight || !d->eci_full_weight ||
      (T > 0 && (!d->term_eci || !d->term_ref || !d->term_size || !d->term_nb)))
    return fail(CEMC_ERR_ARG, "null table pointer");
  const int one_idx = C * B;
  if (one_idx + 1 + B >= (1 << cemc::kRefBits)) return fail(CEMC_ERR_LIMIT, "neighbour table too wide");
  for (size_t i = 0; i < (size_t)N * C; ++i)
    if (d->table[i] < 0 || d->table[i] >= N) return fail(CEMC_ERR_ARG, "table entry %zu out of range", i);
  // Movable (non-background) sites: ascending, in range; every other site is background.
  std::vector<int32_t> movable;
  std::vector<int8_t> site_active(N, 1);
  if (d->movable && d->n_movable < N) {
    if (d->n_movable < 2) return fail(CEMC_ERR_ARG, "fewer than two movable sites");
    movable.assign(d->movable, d->movable + d->n_movable);
    std::fill(site_active.begin(), site_active.end(), 0);
    for (int i = 0; i < d->n_movable; ++i) {
      if (movable[i] < 0 || movable[i] >= N || (i > 0 && movable[i] <= movable[i - 1]))
        return fail(CEMC_ERR_ARG, "movable sites must be ascending site indices");
      site_active[movable[i]] = 1;
    }
  }
  const int n_movable = movable.empty() ? N : (int)movable.size();
  if (movable.empty()) movable.assign(1, 0);
  int singlet[CEMC_MAX_BF];
  for (int b = 0; b < CEMC_MAX_BF; ++b) singlet[b] = 0;
  for (int k = 0; k < K; ++k) {
    if (d->eci_kind[k] < 0 || d->eci_kind[k] > 2) return fail(CEMC_ERR_ARG, "bad ECI kind");
    if (d->eci_kind[k] == 1) {
      if (d->eci_dec[k] < 0 || d->eci_dec[k] >= B) return fail(CEMC_ERR_ARG, "bad singlet decoration");
      singlet[d->eci_dec[k]] = k;
    }
  }
  // Translation-symmetry groups: each owns a contiguous, ECI-sorted range of
  // terms; a one-group geometry is group 0 with every term.
  const int G = d->n_groups > 1 ? d->n_groups : 1;
  if (G > CEMC_MAX_GROUPS) return fail(CEMC_ERR_LIMIT, "%d translation groups exceed the limit %d", G, CEMC_MAX_GROUPS);
  std::vector<int32_t> gterm(G + 1, 0);
  std::vector<double> gscale(G, 1.0);
  std::vector<int8_t> sgroup(N, 0);
  gterm[G] = T;
  if (G > 1) {
    if (!d->site_group || !d->group_terms || !d->group_scale) return fail(CEMC_ERR_ARG, "null group table");
    for (int q = 0; q <= G; ++q) gterm[q] = d->group_terms[q];
    if (gterm[0] != 0 || gterm[G] != T) return fail(CEMC_ERR_ARG, "group term ranges must cover the terms");
    for (int q = 0; q < G; ++q) {
      if (gterm[q + 1] < gterm[q]) return fail(CEMC_ERR_ARG, "group term ranges must ascend");
      gscale[q] = d->group_scale[q];
      if (!(gscale[q] > 0.0) || !std::isfinite(gscale[q])) return fail(CEMC_ERR_ARG, "bad group scale");
    }
    for (int i = 0; i < N; ++i) {
      if (!site_active[i]) continue;
      const int q = d->site_group[i];
      if (q < 0 || q >= G) return fail(CEMC_ERR_ARG, "site %d has no translation group", i);
      sgroup[i] = (int8_t)q;
    }
  }
  bool equal_groups = true;
  for (int q = 0; q < G; ++q) equal_groups = equal_groups && gscale[q] == 1.0;
  for (int t = 0; t < T; ++t) {
    const int k = d->term_eci[t];
    const bool group_start = std::find(gterm.begin(), gterm.end(), t) != gterm.end();
    if (k < 0 || k >= K || d->eci_kind[k] != 2) return fail(CEMC_ERR_ARG, "term %d has a bad ECI", t);
    if (t > 0 && !group_start && k < d->term_eci[t - 1]) return fail(CEMC_ERR_ARG, "terms are not sorted by ECI");
    if (d->term_size[t] < 2 || d->term_size[t] > 4) return fail(CEMC_ERR_ARG, "term %d has a bad size", t);
    if (d->term_ref[t] < 0 || d->term_ref[t] >= B) return fail(CEMC_ERR_ARG, "term %d has a bad decoration", t);
    for (int j = 0; j < d->term_size[t] - 1; ++j)
      if (d->term_nb[3 * t + j] < 0 || d->term_nb[3 * t + j] >= one_idx)
        return fail(CEMC_ERR_ARG, "term %d has a bad member", t);
  }

  // Lane chunks, per group: [G][33] bounds, [G][32] first ECI, [G][2K] lane range per ECI.
  std::vector<int32_t> lane_term(33 * (size_t)G), first(32 * (size_t)G, 0), eci_lane(2 * (size_t)K * G);
  int n_slots = 1;
  std::vector<uint16_t> terms(4 * (size_t)std::max(T, 1), 0);
  for (int q = 0; q < G; ++q) {
    const int t0 = gterm[q], Tg = gterm[q + 1] - gterm[q];
    int32_t *lt = lane_term.data() + 33 * q, *fi = first.data() + 32 * q, *el = eci_lane.data() + 2 * (size_t)K * q;
    for (int l = 0; l <= 32; ++l) lt[l] = t0 + (int32_t)(((long long)l * Tg) / 32);
    for (int k = 0; k < K; ++k) {
      el[2 * k] = 0;
      el[2 * k + 1] = -1;
    }
    std::vector<int> lo_seen(K, 33), hi_seen(K, -1);
    for (int l = 0; l < 32; ++l) {
      const int lo = lt[l], hi = lt[l + 1];
      if (lo >= hi) continue;
      fi[l] = d->term_eci[lo];
      n_slots = std::max(n_slots, d->term_eci[hi - 1] - fi[l] + 1);
      for (int i = lo; i < hi; ++i) {
        const int k = d->term_eci[i];
        lo_seen[k] = std::min(lo_seen[k], l);
        hi_seen[k] = std::max(hi_seen[k], l);
      }
    }
    for (int k = 0; k < K; ++k)
      if (hi_seen[k] >= 0) {
        el[2 * k] = lo_seen[k];
        el[2 * k + 1] = hi_seen[k];
      }
    for (int l = 0; l < 32; ++l)
      for (int i = lt[l]; i < lt[l + 1]; ++i) {
        const int slot = d->term_eci[i] - fi[l];
        terms[4 * i] = (uint16_t)((one_idx + 1 + d->term_ref[i]) | (slot << cemc::kRefBits));
        for (int j = 0; j < 3; ++j)
          terms[4 * i + 1 + j] = (uint16_t)(j < d->term_size[i] - 1 ? d->term_nb[3 * i + j] : one_idx);
      }
  }
  if (n_slots > cemc::kMaxSlots) return fail(CEMC_ERR_LIMIT, "a lane chunk spans %d ECIs", n_slots);
  std::vector<uint8_t> fterms(8 * (size_t)std::max(T, 1), 0);
  for (int i = 0; i < T; ++i) {
    for (int j = 0; j < 3; ++j) {
      const bool has = j < d->term_size[i] - 1;
      fterms[8 * i + j] = (uint8_t)(has ? d->term_nb[3 * i + j] / B : 0);
      fterms[8 * i + 3 + j] = (uint8_t)(has ? d->term_nb[3 * i + j] % B : 0);
    }
    fterms[8 * i + 6] = (uint8_t)d->term_ref[i];
    fterms[8 * i + 7] = (uint8_t)d->term_size[i];
  }
  // Term range of each (group, ECI): fterm_off[q * (K + 1) + k].
  std::vector<int32_t> fterm_off((size_t)G * (K + 1), 0);
  for (int q = 0; q < G; ++q) {
    int t = gterm[q];
    for (int k = 0; k < K; ++k) {
      fterm_off[(size_t)q * (K + 1) + k] = t;
      while (t < gterm[q + 1] && d->term_eci[t] == k) ++t;
    }
    fterm_off[(size_t)q * (K + 1) + K] = gterm[q + 1];
  }
  // Table form of the trial energy change: the terms grouped by cluster geometry
  // (the ordered member columns of a sub-cluster with the changed site as
  // reference); geometries whose terms carry the same (ECI, decorations) list
  // share a pattern, and each chain's kernel tabulates per pattern
  // F(old, new, member species) = sum over its terms of coef * (bf[d_ref][new] -
  // bf[d_ref][old]) * prod bf[d_j][s_j], so a flip costs one lookup per geometry.
  // With several translation groups each group has its own geometry range
  // (geo_start) and the groups share patterns; the table stores group 0's
  // weights, so it needs equal group sizes.
  std::vector<uint32_t> geo_list;  // per geometry: {packed columns, F offset, stride S^m, 0}
  std::vector<int32_t> pat_info;   // per pattern: {m, F offset, first term, end term}
  std::vector<int32_t> pat_terms;  // k | d_ref << 8 | d1 << 12 | d2 << 16 | d3 << 20
  std::vector<int32_t> geo_start(G + 1, 0);
  int n_geo = 0, n_pat = 0, tab_len = 0;
  bool table_ok = C < 255 && S <= 8 && equal_groups;
  std::map<std::vector<std::array<int, 5>>, int> pats;
  for (int q = 0; q < G && table_ok; ++q) {
    geo_start[q] = (int)(geo_list.size() / 4);
    std::map<std::vector<int>, std::vector<std::array<int, 5>>> geos;  // member columns -> terms
    std::vector<std::vector<int>> geo_order;
    for (int t = gterm[q]; t < gterm[q + 1]; ++t) {
      const int m = d->term_size[t] - 1;
      std::vector<int> cols(m);
      std::array<int, 5> term{d->term_eci[t], d->term_ref[t], 0, 0, 0};
      for (int j = 0; j < m; ++j) {
        cols[j] = d->term_nb[3 * t + j] / B;
        term[2 + j] = d->term_nb[3 * t + j] % B;
      }
      auto it = geos.find(cols);
      if (it == geos.end()) {
        geo_order.push_back(cols);
        it = geos.emplace(cols, std::vector<std::array<int, 5>>{}).first;
      }
      it->second.push_back(term);
    }
    for (const auto &cols : geo_order) {
      std::vector<std::array<int, 5>> sig = geos[cols];
      std::sort(sig.begin(), sig.end());
      const int m = (int)cols.size();
      auto it = pats.find(sig);
      if (it == pats.end()) {
        int stride = 1;
        for (int j = 0; j < m; ++j) stride *= S;
        const int id = (int)pats.size();
        it = pats.emplace(sig, id).first;
        pat_info.insert(pat_info.end(), {m, tab_len, (int)pat_terms.size(), 0});
        for (const auto &tm : sig)
          pat_terms.push_back(tm[0] | (tm[1] << 8) | (tm[2] << 12) | (tm[3] << 16) | (tm[4] << 20));
        pat_info[4 * id + 3] = (int)pat_terms.size();
        tab_len += S * S * stride;
      }
      const int id = it->second;
      uint32_t packed = 0;
      for (int j = 0; j < 3; ++j) packed |= (uint32_t)(j < m ? cols[j] : C) << (8 * j);  // column C: species 0
      int stride = 1;
      for (int j = 0; j < m; ++j) stride *= S;
      geo_list.insert(geo_list.end(), {packed, (uint32_t)pat_info[4 * id + 1], (uint32_t)stride, 0u});
    }
  }
  n_geo = (int)(geo_list.size() / 4);
  n_pat = (int)pats.size();
  geo_start[G] = n_geo;
  if (tab_len > cemc::kMaxTable || n_geo > cemc::kMaxGeo) table_ok = false;
  if (geo_list.empty()) geo_list.assign(4, 0u);
  if (pat_info.empty()) pat_info.assign(4, 0);
  if (pat_terms.empty()) pat_terms.assign(1, 0);

  // The trial kernel's conflict test needs a symmetric neighbour relation:
  // j in row(i) <=> i in row(j).
  {
    std::vector<int32_t> sorted_rows(d->table, d->table + (size_t)N * C);
    for (int i = 0; i < N; ++i) std::sort(sorted_rows.begin() + (size_t)i * C, sorted_rows.begin() + (size_t)(i + 1) * C);
    for (int i = 0; i < N; ++i)
      for (int c = 0; c < C; ++c) {
        const int j = d->table[(size_t)i * C + c];
        auto b = sorted_rows.begin() + (size_t)j * C, e = b + C;
        if (!std::binary_search(b, e, i))
          return fail(CEMC_ERR_ARG, "neighbour relation is not symmetric (site %d in row %d but not back)", j, i);
      }
  }
  const int cpad = (C + 3) & ~3;
  std::vector<int32_t> table_pad((size_t)N * cpad);
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < cpad; ++c) table_pad[(size_t)i * cpad + c] = d->table[(size_t)i * C + (c < C ? c : 0)];
  std::vector<int32_t> table_cm((size_t)N * C);
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < C; ++c) table_cm[(size_t)c * N + i] = d->table[(size_t)i * C + c];
  std::vector<double> w(d->eci_weight, d->eci_weight + K), fw(d->eci_full_weight, d->eci_full_weight + K);

  // Binary spin basis (values +1 / -1): pair terms of a cluster ECI folded into
  // one shell mask; the other terms sorted by ECI and cut into 32 lane ranges.
  std::vector<cemc::SpinEci> spin_eci;
  std::vector<uint32_t> spin_masks;  // (lo, hi) pairs
  std::vector<int> spin_mask_cl;     // cluster-ECI slot of each mask
  std::vector<uint8_t> spin_shift;
  std::vector<int32_t> spin_lane_term(33, 0), spin_lane_first(32, 0);
  std::vector<int32_t> half_lane_term(17, 0), half_lane_first(16, 0);  // the same terms over 16 lanes
  std::vector<uint8_t> half_shift;
  int minus_id = -1, singlet_eci = -1;
  bool spin_ok = (B == 1 && S == 2 && C <= CEMC_SPIN_MAX_COLS && G == 1);
  if (spin_ok) {
    if (d->bf[0] == 1.0 && d->bf[1] == -1.0)
      minus_id = 1;
    else if (d->bf[0] == -1.0 && d->bf[1] == 1.0)
      minus_id = 0;
    else
      spin_ok = false;
  }
  for (int k = 0; spin_ok && k < K; ++k) {
    if (d->eci_kind[k] == 1) singlet_eci = k;
    if (d->eci_kind[k] != 2) continue;
    cemc::SpinEci e{};
    e.eci = k;
    uint64_t pairs = 0;
    for (int t = fterm_off[k]; t < fterm_off[k + 1]; ++t) {
      uint64_t m = 0;
      for (int j = 0; j < d->term_size[t] - 1; ++j) m |= (uint64_t)1 << (d->term_nb[3 * t + j]);
      if (d->term_size[t] == 2 && !(pairs & m)) {
        pairs |= m;
        e.n_pairs++;
      } else {
        spin_masks.push_back((uint32_t)m);
        spin_masks.push_back((uint32_t)(m >> 32));
        spin_mask_cl.push_back((int)spin_eci.size());
        e.n_multi++;
      }
    }
    e.pair_lo = (uint32_t)pairs;
    e.pair_hi = (uint32_t)(pairs >> 32);
    spin_eci.push_back(e);
  }
  if (spin_ok && (spin_eci.empty() || spin_eci.size() > CEMC_SPIN_MAX_CL)) spin_ok = false;
  const int n_masks = (int)spin_mask_cl.size();
  if (spin_ok) {
    const int q = (n_masks + 31) / 32;
    for (int l = 0; l <= 32; ++l) spin_lane_term[l] = std::min(l * q, n_masks);
    spin_shift.assign(std::max(n_masks, 1), 0);
    for (int l = 0; l < 32 && spin_ok; ++l) {
      const int lo = spin_lane_term[l], hi = spin_lane_term[l + 1];
      if (lo >= hi) continue;
      spin_lane_first[l] = spin_mask_cl[lo];
      for (int t = lo; t < hi; ++t) {
        const int sl = spin_mask_cl[t] - spin_lane_first[l];
        if (sl > 4 || hi - lo > 63) spin_ok = false;  // 5 six-bit counters per lane
        spin_shift[t] = (uint8_t)(6 * sl);
      }
    }
  }
  // Half-warp form (two flips per warp): cluster ECIs on lanes 0..15, the
  // multi-site terms cut into 16 lane ranges with the same 6-bit counters.
  bool half_ok = spin_ok && spin_eci.size() <= 16;
  if (half_ok) {
    const int q = (n_masks + 15) / 16;
    for (int l = 0; l <= 16; ++l) half_lane_term[l] = std::min(l * q, n_masks);
    half_shift.assign(std::max(n_masks, 1), 0);
    for (int l = 0; l < 16 && half_ok; ++l) {
      const int lo = half_lane_term[l], hi = half_lane_term[l + 1];
      if (lo >= hi) continue;
      half_lane_first[l] = spin_mask_cl[lo];
      for (int t = lo; t < hi; ++t) {
        const int sl = spin_mask_cl[t] - half_lane_first[l];
        if (sl > 4 || hi - lo > 63) half_ok = false;
        half_shift[t] = (uint8_t)(6 * sl);
      }
    }
  }
  // Local-field form (single-site flips in the spin basis, cemc_field.h): one
  // count field per cluster ECI, packed into at most two words per site, and
  // the update list of a changed site j, derived from site 0's neighbourhood
  // and verified to hold at every site (a periodic supercell of one
  // translation group); rows must list distinct sites other than the site.
  bool field_ok = spin_ok && n_movable == N && N <= cemc::kFieldMaxSites &&
                  (int)spin_eci.size() <= cemc::kFieldMaxCl;
  int field_pw = 1;
  std::vector<int32_t> f_slot_eci, f_ustart(C + 1, 0);
  std::vector<uint32_t> f_meta, f_cnt, f_pairinc, f_upd;
  if (field_ok) {
    const int ncl = (int)spin_eci.size();
    std::vector<int> fword(ncl, 0), fshift(ncl, 0);
    int word = 0, used = 0;
    for (int q = 0; q < ncl && field_ok; ++q) {
      const int Kq = spin_eci[q].n_pairs + spin_eci[q].n_multi;
      int bits = 1;
      while ((1 << bits) <= Kq) ++bits;
      if (Kq > 255) field_ok = false;
      if (used + bits > 32) {
        ++word;
        used = 0;
      }
      if (word > 1) field_ok = false;
      fword[q] = word;
      fshift[q] = used;
      used += bits;
      f_slot_eci.push_back(spin_eci[q].eci);
      f_meta.push_back((uint32_t)Kq | ((uint32_t)fshift[q] << 8) | ((uint32_t)word << 13) | ((uint32_t)bits << 16));
    }
    field_pw = word + 1;
    auto add_inc = [&](int q, uint32_t *w) { w[fword[q]] += 1u << fshift[q]; };
    // (site, column) keys of every row, sorted by site: the column of a site in a row
    std::vector<uint64_t> keys(field_ok ? (size_t)N * C : 0);
    for (int i = 0; i < N && field_ok; ++i) {
      uint64_t *k = keys.data() + (size_t)i * C;
      for (int c = 0; c < C; ++c) {
        const int s = d->table[(size_t)i * C + c];
        if (s == i) field_ok = false;
        k[c] = ((uint64_t)(uint32_t)s << 8) | (uint64_t)c;
      }
      std::sort(k, k + C);
      for (int c = 1; c < C; ++c)
        if ((k[c] >> 8) == (k[c - 1] >> 8)) field_ok = false;
    }
    auto col_of = [&](int i, int x) -> int {
      const uint64_t *b = keys.data() + (size_t)i * C, *e = b + C;
      const uint64_t *p = std::lower_bound(b, e, (uint64_t)(uint32_t)x << 8);
      return (p != e && (*p >> 8) == (uint64_t)(uint32_t)x) ? (int)(*p & 255u) : -1;
    };
    std::vector<int> inv(C, -1);  // row_{row_j[c]}[inv[c]] = j
    for (int c = 0; c < C && field_ok; ++c) {
      inv[c] = col_of(d->table[c], 0);
      if (inv[c] < 0) field_ok = false;
    }
    std::vector<std::array<int, 3>> cmap;  // (c, c2, c3): row_j[c3] = row_{row_j[c]}[c2]
    if (field_ok) {
      for (int q = 0; q < ncl; ++q) {  // count entries: pair shells, then multi-site terms
        uint32_t w[2] = {0, 0};
        add_inc(q, w);
        f_cnt.insert(f_cnt.end(), {spin_eci[q].pair_lo, spin_eci[q].pair_hi, w[0], w[1]});
      }
      for (int t = 0; t < n_masks; ++t) {
        uint32_t w[2] = {0, 0};
        add_inc(spin_mask_cl[t], w);
        f_cnt.insert(f_cnt.end(), {spin_masks[2 * t], spin_masks[2 * t + 1], w[0], w[1]});
      }
      for (int c = 0; c < C && field_ok; ++c) {
        f_ustart[c] = (int32_t)(f_upd.size() / 4);
        const int i = d->table[c];  // the target row_0[c]
        const int cp = inv[c];      // site 0 seen from the target
        const uint64_t bit = (uint64_t)1 << cp;
        uint32_t pinc[2] = {0, 0};
        for (int q = 0; q < ncl; ++q)
          if ((((uint64_t)spin_eci[q].pair_hi << 32) | spin_eci[q].pair_lo) & bit) add_inc(q, pinc);
        f_pairinc.insert(f_pairinc.end(), {pinc[0], pinc[1]});
        // Terms at the target through site 0, by cluster slot: those with one other member
        // are counted together (one mask; the count of -1 products is a popcount), the
        // others (and repeated single members) toggle one by one with their parity.
        std::vector<uint64_t> single(ncl, 0);
        std::vector<uint64_t> multi;
        std::vector<int> multi_q;
        for (int t = 0; t < n_masks && field_ok; ++t) {
          const uint64_t m = ((uint64_t)spin_masks[2 * t + 1] << 32) | spin_masks[2 * t];
          if (!(m & bit)) continue;
          uint64_t others = m & ~bit, mj = 0;
          while (others) {
            const int c2 = __builtin_ctzll(others);
            others &= others - 1;
            const int c3 = col_of(0, d->table[(size_t)i * C + c2]);
            if (c3 < 0) {
              field_ok = false;
              break;
            }
            mj |= (uint64_t)1 << c3;
            cmap.push_back({c, c2, c3});
          }
          const int q = spin_mask_cl[t];
          if (__builtin_popcountll(mj) == 1 && !(single[q] & mj)) {
            single[q] |= mj;
          } else {
            multi.push_back(mj);
            multi_q.push_back(q);
          }
        }
        // entry {mask lo, mask hi, field increment, word | kind << 1 | members << 8}
        for (int q = 0; q < ncl && field_ok; ++q)
          if (single[q])
            f_upd.insert(f_upd.end(), {(uint32_t)single[q], (uint32_t)(single[q] >> 32), 1u << fshift[q],
                                       (uint32_t)fword[q] | 2u | ((uint32_t)__builtin_popcountll(single[q]) << 8)});
        for (size_t e = 0; e < multi.size() && field_ok; ++e) {
          const int q = multi_q[e];
          f_upd.insert(f_upd.end(), {(uint32_t)multi[e], (uint32_t)(multi[e] >> 32), 1u << fshift[q],
                                     (uint32_t)fword[q]});
        }
      }
      f_ustart[C] = (int32_t)(f_upd.size() / 4);
      std::sort(cmap.begin(), cmap.end());
      cmap.erase(std::unique(cmap.begin(), cmap.end()), cmap.end());
    }
    for (int j = 1; j < N && field_ok; ++j) {
      const int32_t *rj = d->table + (size_t)j * C;
      for (int c = 0; c < C; ++c)
        if (col_of(rj[c], j) != inv[c]) field_ok = false;
      for (const auto &m : cmap)
        if (col_of(j, d->table[(size_t)rj[m[0]] * C + m[1]]) != m[2]) field_ok = false;
    }
  }
  if (!field_ok) {
    f_slot_eci.assign(1, 0);
    f_meta.assign(1, 0u);
    f_cnt.assign(4, 0u);
    f_pairinc.assign(2 * (size_t)C, 0u);
    f_ustart.assign(C + 1, 0);
    f_upd.assign(4, 0u);
  }
  if (f_upd.empty()) f_upd.assign(4, 0u);
  // Quarter-warp form (four flips per warp): cluster ECIs on lanes 0..7, the multi-site terms cut
  // into 8 lane ranges with the same 6-bit counters; a trial's odd-term count of one cluster ECI
  // is summed in an 8-bit field of one warp reduction, so no ECI may have more than 255 terms.
  std::vector<int32_t> qtr_lane_term(9, 0), qtr_lane_first(8, 0);
  std::vector<uint8_t> qtr_shift;
  bool qtr_ok = spin_ok && spin_eci.size() <= 8;
  for (const auto &e : spin_eci) qtr_ok = qtr_ok && e.n_multi <= 255;
  if (qtr_ok) {
    const int q = (n_masks + 7) / 8;
    for (int l = 0; l <= 8; ++l) qtr_lane_term[l] = std::min(l * q, n_masks);
    qtr_shift.assign(std::max(n_masks, 1), 0);
    for (int l = 0; l < 8 && qtr_ok; ++l) {
      const int lo = qtr_lane_term[l], hi = qtr_lane_term[l + 1];
      if (lo >= hi) continue;
      qtr_lane_first[l] = spin_mask_cl[lo];
      for (int t = lo; t < hi; ++t) {
        const int sl = spin_mask_cl[t] - qtr_lane_first[l];
        if (sl > 4 || hi - lo > 63) qtr_ok = false;
        qtr_shift[t] = (uint8_t)(6 * sl);
      }
    }
  }
  if (qtr_shift.empty()) qtr_shift.assign(1, 0);
  if (half_shift.empty()) half_shift.assign(1, 0);
  if (spin_eci.empty()) spin_eci.push_back(cemc::SpinEci{});
  if (spin_masks.empty()) spin_masks.assign(2, 0u);
  if (spin_shift.empty()) spin_shift.assign(1, 0);

  // Periodic box of cells (DevGeo::box_L): sites ((x * L + y) * L + z) * nb + b, and at every
  // site the table holds the same (cell offset, basis site) per (b, column) as at cell 0.  Tried
  // for one translation group without background sites, for each basis count nb <= 8 with N / nb
  // a cube; every entry of the table and the multiply-high divisions are checked.
  int box_L = 0, box_nb = 0;
  uint32_t box_mnb = 0, box_mL = 0;
  std::vector<uint32_t> box_off;
  auto umulhi = [](uint32_t a, uint32_t m) { return (uint32_t)(((uint64_t)a * m) >> 32); };
  auto magic = [](uint32_t dv) { return (uint32_t)((((uint64_t)1 << 32) + dv - 1) / dv); };  // ceil(2^32 / dv)
  for (int nb = 1; nb <= 8 && box_L == 0 && G == 1 && n_movable == N; ++nb) {
    if (N % nb) continue;
    const int cells = N / nb;
    const int L = (int)std::lround(std::cbrt((double)cells));
    if ((long long)L * L * L != cells || L > 255) continue;
    auto decode = [&](int site, int &x, int &y, int &z) {
      int c = site / nb;
      z = c % L;
      c /= L;
      y = c % L;
      x = c / L;
      return site % nb;
    };
    auto near = [&](int v) { return 2 * v > L ? v - L : v; };  // minimal image in (-L/2, L/2]
    std::vector<uint32_t> off((size_t)nb * C);
    for (int b = 0; b < nb; ++b)
      for (int c = 0; c < C; ++c) {
        int x, y, z;
        const int bb = decode(d->table[(size_t)b * C + c], x, y, z);
        off[(size_t)b * C + c] = (uint32_t)(near(x) + 128) | ((uint32_t)(near(y) + 128) << 8) |
                                 ((uint32_t)(near(z) + 128) << 16) | ((uint32_t)bb << 24);
      }
    bool ok = true;
    for (int site = 0; site < N && ok; ++site) {
      int x, y, z;
      const int b = decode(site, x, y, z);
      for (int c = 0; c < C; ++c) {
        const uint32_t o = off[(size_t)b * C + c];
        int nx = x + (int)(o & 255u) - 128, ny = y + (int)((o >> 8) & 255u) - 128, nz = z + (int)((o >> 16) & 255u) - 128;
        nx += nx < 0 ? L : 0;
        nx -= nx >= L ? L : 0;
        ny += ny < 0 ? L : 0;
        ny -= ny >= L ? L : 0;
        nz += nz < 0 ? L : 0;
        nz -= nz >= L ? L : 0;
        if (((nx * L + ny) * L + nz) * nb + (int)(o >> 24) != d->table[(size_t)site * C + c]) {
          ok = false;
          break;
        }
      }
    }
    const uint32_t mnb = nb > 1 ? magic((uint32_t)nb) : 0u, mL = L > 1 ? magic((uint32_t)L) : 0u;
    for (uint32_t v = 0; ok && nb > 1 && v < (uint32_t)N; ++v) ok = umulhi(v, mnb) == v / (uint32_t)nb;
    for (uint32_t v = 0; ok && L > 1 && v < (uint32_t)cells; ++v) ok = umulhi(v, mL) == v / (uint32_t)L;
    if (ok) {
      box_L = L;
      box_nb = nb;
      box_mnb = mnb;
      box_mL = mL;
      box_off.swap(off);
    }
  }
  if (box_off.empty()) box_off.assign(1, 0u);

  // One device allocation for all tables.
  struct Part {
    const void *src;
    size_t bytes;
    size_t off;
  };
  std::vector<Part> parts = {
      {table_pad.data(), sizeof(int32_t) * N * cpad, 0}, {table_cm.data(), sizeof(int32_t) * N * C, 0},
      {terms.data(), terms.size() * 2, 0},         {lane_term.data(), lane_term.size() * 4, 0},
      {first.data(), first.size() * 4, 0},         {eci_lane.data(), eci_lane.size() * 4, 0},
      {d->eci_kind, sizeof(int32_t) * K, 0},       {d->eci_dec, sizeof(int32_t) * K, 0},
      {w.data(), sizeof(double) * K, 0},           {fw.data(), sizeof(double) * K, 0},
      {d->bf, sizeof(double) * B * S, 0},          {fterms.data(), fterms.size(), 0},
      {fterm_off.data(), fterm_off.size() * 4, 0},
      {spin_eci.data(), spin_eci.size() * sizeof(cemc::SpinEci), 0},
      {spin_masks.data(), spin_masks.size() * 4, 0},
      {spin_shift.data(), spin_shift.size(), 0},
      {spin_lane_term.data(), 33 * 4, 0},
      {spin_lane_first.data(), 32 * 4, 0},
      {half_shift.data(), half_shift.size(), 0},
      {half_lane_term.data(), 17 * 4, 0},
      {half_lane_first.data(), 16 * 4, 0},
      {geo_list.data(), geo_list.size() * 4, 0},
      {pat_info.data(), pat_info.size() * 4, 0},
      {pat_terms.data(), pat_terms.size() * 4, 0},
      {movable.data(), movable.size() * 4, 0},
      {site_active.data(), site_active.size(), 0},
      {sgroup.data(), sgroup.size(), 0},
      {geo_start.data(), geo_start.size() * 4, 0},
      {gscale.data(), gscale.size() * 8, 0},
      {f_slot_eci.data(), f_slot_eci.size() * 4, 0},
      {f_meta.data(), f_meta.size() * 4, 0},
      {f_cnt.data(), f_cnt.size() * 4, 0},
      {f_pairinc.data(), f_pairinc.size() * 4, 0},
      {f_ustart.data(), f_ustart.size() * 4, 0},
      {f_upd.data(), f_upd.size() * 4, 0},
      {box_off.data(), box_off.size() * 4, 0},
      {qtr_shift.data(), qtr_shift.size(), 0},
      {qtr_lane_term.data(), 9 * 4, 0},
      {qtr_lane_first.data(), 8 * 4, 0},
  };
  size_t total = 0;
  for (auto &p : parts) {
    p.off = total;
    total = align_up(total + p.bytes, 256);
  }
  cemc_geometry *geo = new cemc_geometry();
  geo->dev_bytes = total;
  cudaError_t e = cudaMalloc(&geo->dev, total);
  if (e != cudaSuccess) {
    delete geo;
    return cuda_fail(e, "cudaMalloc(geometry tables)");
  }
  std::vector<unsigned char> host(total, 0);
  for (auto &p : parts) memcpy(host.data() + p.off, p.src, p.bytes);
  e = cudaMemcpy(geo->dev, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(geo->dev);
    delete geo;
    return cuda_fail(e, "cudaMemcpy(geometry tables)");
  }
  unsigned char *base = static_cast<unsigned char *>(geo->dev);
  cemc::DevGeo &g = geo->g;
  g.n_sites = N;
  g.n_cols = C;
  g.n_sym = S;
  g.n_bf = B;
  g.n_eci = K;
  g.n_terms = T;
  g.vals_len = one_idx + 1 + B;
  g.one_idx = one_idx;
  g.n_slots = n_slots;
  g.cpad = cpad;
  g.table = reinterpret_cast<const int32_t *>(base + parts[0].off);
  g.table_cm = reinterpret_cast<const int32_t *>(base + parts[1].off);
  g.terms = reinterpret_cast<const uint16_t *>(base + parts[2].off);
  g.lane_term = reinterpret_cast<const int32_t *>(base + parts[3].off);
  g.lane_first_eci = reinterpret_cast<const int32_t *>(base + parts[4].off);
  g.eci_lane = reinterpret_cast<const int32_t *>(base + parts[5].off);
  g.eci_kind = reinterpret_cast<const int32_t *>(base + parts[6].off);
  g.eci_dec = reinterpret_cast<const int32_t *>(base + parts[7].off);
  g.eci_w = reinterpret_cast<const double *>(base + parts[8].off);
  g.eci_fw = reinterpret_cast<const double *>(base + parts[9].off);
  g.bf = reinterpret_cast<const double *>(base + parts[10].off);
  g.fterms = reinterpret_cast<const uint8_t *>(base + parts[11].off);
  g.fterm_off = reinterpret_cast<const int32_t *>(base + parts[12].off);
  for (int b = 0; b < CEMC_MAX_BF; ++b) g.singlet_eci[b] = singlet[b];
  g.table_ok = table_ok ? 1 : 0;
  g.n_geo = n_geo;
  g.n_pat = n_pat;
  g.tab_len = tab_len;
  g.geo_list = reinterpret_cast<const uint4 *>(base + parts[21].off);
  g.pat_info = reinterpret_cast<const int4 *>(base + parts[22].off);
  g.pat_terms = reinterpret_cast<const int32_t *>(base + parts[23].off);
  g.n_movable = n_movable;
  g.movable = reinterpret_cast<const int32_t *>(base + parts[24].off);
  g.site_active = n_movable == N ? nullptr : reinterpret_cast<const int8_t *>(base + parts[25].off);
  g.n_groups = G;
  g.site_group = reinterpret_cast<const int8_t *>(base + parts[26].off);
  g.geo_start = reinterpret_cast<const int32_t *>(base + parts[27].off);
  g.group_scale = reinterpret_cast<const double *>(base + parts[28].off);
  g.box_L = box_L;
  g.box_nb = box_nb;
  g.box_mnb = box_mnb;
  g.box_mL = box_mL;
  g.box_off = reinterpret_cast<const uint32_t *>(base + parts[35].off);
  g.pm1_minus = -1;
  if (B == 1 && S == 2) {
    if (d->bf[0] == 1.0 && d->bf[1] == -1.0) g.pm1_minus = 1;
    else if (d->bf[0] == -1.0 && d->bf[1] == 1.0) g.pm1_minus = 0;
  }
  geo->spin_ok = spin_ok;
  geo->spin.n_cl = spin_ok ? (int)spin_eci.size() : 0;
  geo->spin.n_masks = spin_ok ? n_masks : 0;
  geo->spin.minus_id = minus_id;
  geo->spin.singlet_eci = singlet_eci;
  geo->spin.eci = reinterpret_cast<const cemc::SpinEci *>(base + parts[13].off);
  geo->spin.masks = reinterpret_cast<const uint2 *>(base + parts[14].off);
  geo->spin.shift = reinterpret_cast<const uint8_t *>(base + parts[15].off);
  geo->spin.lane_term = reinterpret_cast<const int32_t *>(base + parts[16].off);
  geo->spin.lane_first = reinterpret_cast<const int32_t *>(base + parts[17].off);
  geo->spin.qtr_ok = qtr_ok ? 1 : 0;
  geo->spin.qtr_shift = reinterpret_cast<const uint8_t *>(base + parts[36].off);
  geo->spin.qtr_lane_term = reinterpret_cast<const int32_t *>(base + parts[37].off);
  geo->spin.qtr_lane_first = reinterpret_cast<const int32_t *>(base + parts[38].off);
  geo->spin.half_ok = half_ok ? 1 : 0;
  geo->spin.half_shift = reinterpret_cast<const uint8_t *>(base + parts[18].off);
  geo->spin.half_lane_term = reinterpret_cast<const int32_t *>(base + parts[19].off);
  geo->spin.half_lane_first = reinterpret_cast<const int32_t *>(base + parts[20].off);
  geo->field_ok = field_ok;
  geo->field.n_cl = field_ok ? (int)f_slot_eci.size() : 0;
  geo->field.pw = field_pw;
  geo->field.n_cnt = field_ok ? (int)(f_cnt.size() / 4) : 0;
  geo->field.n_upd = field_ok ? (int)f_ustart[C] : 0;
  geo->field.minus_id = minus_id;
  geo->field.singlet_eci = singlet_eci;
  geo->field.slot_eci = reinterpret_cast<const int32_t *>(base + parts[29].off);
  geo->field.slot_meta = reinterpret_cast<const uint32_t *>(base + parts[30].off);
  geo->field.cnt = reinterpret_cast<const uint4 *>(base + parts[31].off);
  geo->field.pairinc = reinterpret_cast<const uint2 *>(base + parts[32].off);
  geo->field.ustart = reinterpret_cast<const int32_t *>(base + parts[33].off);
  geo->field.upd = reinterpret_cast<const uint4 *>(base + parts[34].off);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&geo->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&geo->n_sms, cudaDevAttrMultiProcessorCount, dev);
  *out = geo;
  return CEMC_OK;
}

extern "C" int cemc_geometry_destroy(cemc_geometry *geo) {
  if (!geo) return CEMC_OK;
  cudaError_t e = cudaFree(geo->dev);
  delete geo;
  if (e != cudaSuccess) return cuda_fail(e, "cudaFree(geometry tables)");
  return CEMC_OK;
}

extern "C" size_t cemc_geometry_device_bytes(const cemc_geometry *geo) { return geo ? geo->dev_bytes : 0; }

extern "C" size_t cemc_stamp_words(const cemc_geometry *geo, int32_t n_chains) {
  if (!geo || n_chains <= 0) return 0;
  int bits = 5;
  while ((1 << bits) < geo->g.n_sites) ++bits;
  return 2 * ((size_t)1 << bits) * (size_t)n_chains;
}

extern "C" int cemc_run(const cemc_geometry *geo, cemc_run_desc *r, void *stream) {
  if (!geo || !r) return fail(CEMC_ERR_ARG, "null geometry or run descriptor");
  const cemc::DevGeo &g = geo->g;
  if (r->n_chains <= 0) return fail(CEMC_ERR_ARG, "no chains");
  if (r->move != CEMC_MOVE_FLIP && r->move != CEMC_MOVE_SWAP) return fail(CEMC_ERR_ARG, "unknown move type");
  if (r->precision != CEMC_PREC_F32 && r->precision != CEMC_PREC_F64) return fail(CEMC_ERR_ARG, "unknown precision");
  if (!r->occ || !r->cf || !r->energy || !r->eci || !r->kT || !r->trial)
    return fail(CEMC_ERR_ARG, "null chain state pointer");
  if (r->move == CEMC_MOVE_SWAP && (!r->trk || !r->loc || !r->trk_start || !r->trk_count))
    return fail(CEMC_ERR_ARG, "swap moves need the per-species site lists");
  if ((r->trace_site || r->trace_acc || r->trace_de) && !(r->trace_site && r->trace_acc && r->trace_de))
    return fail(CEMC_ERR_ARG, "trace buffers must be given together");
  if (r->n_chains > 65535 * 32) return fail(CEMC_ERR_LIMIT, "too many chains in one launch");
  r->kernel_used = CEMC_KERNEL_AUTO;  // nothing launched yet
  if (r->n_trials == 0) return CEMC_OK;
  if (r->kernel < CEMC_KERNEL_AUTO || r->kernel > CEMC_KERNEL_SPIN_QUARTER)
    return fail(CEMC_ERR_ARG, "unknown kernel %d", (int)r->kernel);
  if (r->cluster < 0 || r->cluster > 2) return fail(CEMC_ERR_ARG, "cluster must be 0 (auto), 1 or 2");
  // waste recycling runs its own build of the generic form, one CTA per chain
  const bool recycle = r->recycle_waste != 0;
  if (recycle && r->kernel != CEMC_KERNEL_AUTO && r->kernel != CEMC_KERNEL_GENERIC)
    return fail(CEMC_ERR_ARG, "waste recycling runs the generic kernel form");
  if (recycle && r->cluster == 2) return fail(CEMC_ERR_ARG, "waste recycling runs one CTA per chain");
  if ((r->site_allow || r->frozen || r->accept_first) && r->cluster == 2)
    return fail(CEMC_ERR_ARG, "move constraints and first-move acceptance run one CTA per chain");
  const bool want_spin = r->kernel == CEMC_KERNEL_SPIN || r->kernel == CEMC_KERNEL_SPIN_HALFWARP ||
                         r->kernel == CEMC_KERNEL_SPIN_QUARTER;
  if (want_spin && !geo->spin_ok)
    return fail(CEMC_ERR_ARG, "the spin-basis kernel needs two species with basis values +1/-1, <= 64 columns and "
                              "one translation-symmetry group");
  const bool use_spin = want_spin || (r->kernel == CEMC_KERNEL_AUTO && geo->spin_ok && !recycle);
  if (r->kernel == CEMC_KERNEL_TABLE && !g.table_ok)
    return fail(CEMC_ERR_LIMIT, "the table kernel needs translation groups of equal size and pattern tables of at "
                                "most %d entries", cemc::kMaxTable);
  // move constraints are checked (and redrawn) by the one-trial-per-warp forms
  const bool constrained = r->site_allow != nullptr || r->frozen != nullptr || r->accept_first != 0 || recycle;
  if (r->max_attempts < 0) return fail(CEMC_ERR_ARG, "max_attempts must be >= 0");
  const bool half_ok = use_spin && geo->spin.half_ok && r->move == CEMC_MOVE_FLIP && !constrained;
  if (r->kernel == CEMC_KERNEL_SPIN_QUARTER &&
      !(use_spin && geo->spin.qtr_ok && r->move == CEMC_MOVE_FLIP && !constrained && r->cluster != 2))
    return fail(CEMC_ERR_ARG, "the quarter-warp spin kernel runs unconstrained single-site flips with at most 8 "
                              "cluster ECIs, one CTA per chain");
  if (r->kernel == CEMC_KERNEL_SPIN_HALFWARP && !half_ok)
    return fail(CEMC_ERR_ARG, "the half-warp spin kernel runs unconstrained single-site flips with at most 16 "
                              "cluster ECIs");
  // Local-field form: unconstrained single-site flips of a geometry with field tables, one CTA
  // per chain, when asked for (its state fits in shared memory, with the conflict table in the
  // caller's stamp buffer when it does not fit beside the counts).
  const bool field_possible = geo->field_ok && r->move == CEMC_MOVE_FLIP && !constrained && r->cluster != 2;
  if (r->kernel == CEMC_KERNEL_FIELD && !field_possible)
    return fail(CEMC_ERR_ARG, "the local-field kernel runs unconstrained single-site flips of a periodic binary "
                              "+1/-1 geometry of one translation group without background sites, one CTA per chain");
  if (field_possible && r->kernel == CEMC_KERNEL_FIELD) {
    const cemc::FieldDev &fd = geo->field;
    cemc::RunArgs fa{};
    fa.n_chains = r->n_chains;
    fa.warps = r->warps > 0 ? std::min(r->warps, cemc::kFieldMaxWarps) : 16;
    fa.cl = 1;
    fa.tpw = 1;
    fa.ring_bits = cemc::field_ring_bits(cemc::field_round(fa.warps));
    fa.occ_smem = 1;
    int bits = 5;
    while ((1 << bits) < g.n_sites) ++bits;
    fa.stamp_bits = bits;
    const int rs = r->precision == CEMC_PREC_F32 ? 4 : 8;
    size_t smem = cemc::field_layout(g, fd.n_cl, fd.pw, fd.n_cnt, fd.n_upd, rs, fa.ring_bits, false).total;
    if (smem > (size_t)geo->max_smem && r->stamps && r->stamp_words >= cemc_stamp_words(geo, r->n_chains)) {
      fa.gstamp = r->stamps;
      smem = cemc::field_layout(g, fd.n_cl, fd.pw, fd.n_cnt, fd.n_upd, rs, fa.ring_bits, true).total;
    }
    if (smem <= (size_t)geo->max_smem) {
      fa.seed = r->seed;
      fa.occ = r->occ;
      fa.cf = r->cf;
      fa.energy = r->energy;
      fa.eci = r->eci;
      fa.kT = r->kT;
      fa.trial = r->trial;
      fa.accum = r->accum;
      fa.trace_site = r->trace_site;
      fa.trace_acc = r->trace_acc;
      fa.trace_de = r->trace_de;
      fa.status = r->status;
      fa.chain_key = r->chain_key;
      fa.accum_slot = r->accum_slot;
      fa.chain_trials = r->chain_trials;
      const uint64_t max_chunk = (uint64_t)1 << 25;  // round numbers fit the 26 upper bits of a stamp
      if (r->n_trials > max_chunk && r->trace_acc)
        return fail(CEMC_ERR_LIMIT, "traced runs are limited to %llu trials per call", (unsigned long long)max_chunk);
      for (uint64_t done = 0; done < r->n_trials;) {
        const uint64_t n = std::min(max_chunk, r->n_trials - done);
        fa.n_trials = n;
        fa.chunk_offset = done;
        cudaError_t e = cemc::launch_field(g, fa, fd, r->precision, smem, static_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return cuda_fail(e, "local-field Monte Carlo kernel launch");
        done += n;
      }
      r->kernel_used = CEMC_KERNEL_FIELD;
      return CEMC_OK;
    }
    if (r->kernel == CEMC_KERNEL_FIELD)
      return fail(CEMC_ERR_LIMIT, "the local-field kernel needs %zu bytes of shared memory (limit %d); pass a stamp "
                                  "buffer or use another kernel", smem, geo->max_smem);
  }
  // two trials per warp: asked for, or chosen when eligible and no CTA pair was asked for
  // (a CTA pair takes the half-warp form only when that form is asked for explicitly)
  const int tpw = r->kernel == CEMC_KERNEL_SPIN_QUARTER ? 4 :
                  (r->kernel == CEMC_KERNEL_SPIN_HALFWARP || (r->kernel == CEMC_KERNEL_AUTO && half_ok &&
                                                                r->cluster != 2)) ? 2 : 1;
  // Default round width: 16 evaluating warps, fewer where most trials of a
  // round would conflict.  A changed site reaches about n_cols sites, so with
  // n_movable / (2 n_cols sites-per-move) trials a round about half the round
  // commits (a 2048-site swap chain: 9 trials, about 4 commits a round); a
  // wider round only adds latency.  The same cap decides whether a chain may
  // take a CTA pair (twice the trials per round) when none is asked for.
  int warps = r->warps;
  int round_cap = 0;  // 0: the caller chose the width
  if (warps <= 0) {
    const int per_move = r->move == CEMC_MOVE_SWAP ? 2 : 1;
    round_cap = std::max(4, g.n_movable / (2 * g.n_cols * per_move));
    warps = std::max(2, std::min(16, round_cap / tpw));
  }
  const int rsize = r->precision == CEMC_PREC_F32 ? 4 : 8;
  cemc::RunArgs a{};
  a.n_chains = r->n_chains;
  a.warps = warps;
  a.seed = r->seed;
  a.occ = r->occ;
  a.cf = r->cf;
  a.energy = r->energy;
  a.eci = r->eci;
  a.kT = r->kT;
  a.trial = r->trial;
  a.accum = r->accum;
  a.trk = r->trk;
  a.loc = r->loc;
  a.trk_start = r->trk_start;
  a.trk_count = r->trk_count;
  a.trace_site = r->trace_site;
  a.trace_acc = r->trace_acc;
  a.trace_de = r->trace_de;
  a.status = r->status;
  a.chain_key = r->chain_key;
  a.accum_slot = r->accum_slot;
  a.chain_trials = r->chain_trials;
  a.site_allow = r->site_allow;
  a.frozen = r->frozen;
  a.max_attempts = r->max_attempts > 0 ? r->max_attempts : 10000;
  a.accept_first = r->accept_first != 0;
  a.cons = constrained ? 1 : 0;
  a.tpw = tpw;
  const int n_cl = use_spin ? geo->spin.n_cl : 0, n_masks = use_spin ? geo->spin.n_masks : 0;
  // Evaluation forms to try, in order: spin, or table then generic (AUTO), or the one asked for.
  std::vector<int> forms;
  if (recycle)
    forms = {cemc::kFormRecycle};
  else if (use_spin)
    forms = {cemc::kFormSpin};
  else if (r->kernel == CEMC_KERNEL_TABLE && r->n_chains > 65535)
    return fail(CEMC_ERR_LIMIT, "the table kernel ends with a recompute of at most 65535 chains per call");
  else if (r->kernel == CEMC_KERNEL_TABLE)
    forms = {cemc::kFormTable};
  else if (r->kernel == CEMC_KERNEL_GENERIC)
    forms = {cemc::kFormGeneric};
  else if (g.table_ok && r->n_chains <= 65535)
    forms = {cemc::kFormTable, cemc::kFormGeneric};
  else
    forms = {cemc::kFormGeneric};
  // Shared memory: the occupation, then (swaps) the site lists, then exact
  // stamp tables (one entry per site) are preferred; fall back in that order.
  const size_t budget = (size_t)geo->max_smem;
  int exact_bits = 0;
  while ((1 << exact_bits) < g.n_sites) ++exact_bits;
  if (exact_bits < 5) exact_bits = 5;
  const int is_swap = r->move == CEMC_MOVE_SWAP;
  struct Choice {
    int occ, trk, min_bits, global;
  };
  // exact tables in a caller buffer come before hashed shared-memory ones (hashing only costs speed)
  const bool gbuf = r->stamps && r->stamp_words >= cemc_stamp_words(geo, r->n_chains);
  std::vector<Choice> choices = {{1, is_swap, exact_bits, 0}, {1, 0, exact_bits, 0}};
  if (gbuf) choices.insert(choices.end(), {{1, is_swap, exact_bits, 1}, {1, 0, exact_bits, 1}});
  choices.insert(choices.end(), {{1, 0, 12, 0}, {0, 0, 12, 0}});
  if (gbuf) choices.push_back({0, 0, exact_bits, 1});
  choices.push_back({0, 0, 5, 0});
  int form = forms[0];
  auto fit = [&](int cl, cemc::McLayout &L, cemc::RunArgs &x) {
    const int w = std::min(warps, cemc::max_eval_warps(cl, tpw));
    const int rb = cemc::ring_bits_for(cemc::round_trials(cl, w, tpw));
    for (const Choice &ch : choices) {
      for (int bits = exact_bits; bits >= std::min(ch.min_bits, exact_bits); --bits) {
        L = cemc::mc_layout(g, w, r->move, rsize, ch.occ, ch.trk, bits, n_cl, n_masks, rb, form, tpw, ch.global);
        if (L.total <= budget) {
          x.occ_smem = ch.occ;
          x.trk_smem = ch.trk;
          x.stamp_bits = bits;
          x.gstamp = ch.global ? r->stamps : nullptr;
          x.ring_bits = rb;
          x.cl = cl;
          x.warps = w;
          return true;
        }
      }
    }
    return false;
  };
  // Resident cluster pairs of this configuration (cached per geometry).
  auto resident_pairs = [&](const cemc::McLayout &L, const cemc::RunArgs &x) {
    const auto key = std::make_tuple(x.warps, (int)r->move, (int)r->precision, form, L.total);
    std::lock_guard<std::mutex> lock(geo->mu);
    auto it = geo->pairs.find(key);
    if (it != geo->pairs.end()) return it->second;
    const int n = cemc::max_active_clusters(g, x, r->move, r->precision, L.total, form);
    geo->pairs[key] = n;
    return n;
  };
  cemc::McLayout L{};
  bool found = false;
  for (size_t fi = 0; fi < forms.size() && !found; ++fi) {
    form = forms[fi];
    if (r->cluster == 2 || (tpw == 1 && r->cluster == 0 && !constrained && 2 * r->n_chains <= geo->n_sms &&
                            (round_cap == 0 || round_cap >= 2 * warps))) {
      cemc::RunArgs x = a;
      cemc::McLayout L2{};
      if (fit(2, L2, x)) {
        const int n = resident_pairs(L2, x);
        if (r->cluster == 2 && n < 1) return fail(CEMC_ERR_LIMIT, "no CTA pair of this size fits on the device");
        if (r->cluster == 2 || n >= r->n_chains) {
          a = x;
          L = L2;
          found = true;
        }
      } else if (r->cluster == 2 && fi + 1 == forms.size()) {
        return fail(CEMC_ERR_LIMIT, "shared memory of a CTA pair exceeds %zu bytes; use fewer warps", budget);
      }
    }
    if (!found && r->cluster != 2) found = fit(1, L, a);
  }
  if (!found) return fail(CEMC_ERR_LIMIT, "shared memory exceeds %zu bytes; use fewer warps", budget);
  // The table form leaves correlation functions to a full recompute at the end of the call.
  double *rscratch = nullptr;
  if (form == cemc::kFormTable) {
    const size_t need = cemc::recompute_blocks(g) * (size_t)r->n_chains * (size_t)g.n_eci;
    if (r->scratch && r->scratch_doubles < need)
      return fail(CEMC_ERR_ARG, "the table kernel's final recompute needs a scratch buffer of %zu doubles, the run "
                                "descriptor gives %llu", need, (unsigned long long)r->scratch_doubles);
    if (r->scratch) {
      rscratch = r->scratch;
    } else if (need <= cemc::kNoAllocScratchDoubles) {
      cudaError_t err = cudaSuccess;
      rscratch = cemc::noalloc_scratch(&err);
      if (!rscratch) return cuda_fail(err, "cudaGetSymbolAddress(recompute scratch)");
    } else {
      return fail(CEMC_ERR_LIMIT, "the table kernel needs a recompute scratch of %zu doubles (run desc scratch)", need);
    }
  }
  // Rounds are numbered in the upper 26 bits of the stamp marks: split very long runs.
  const uint64_t max_chunk = (uint64_t)1 << 25;
  if (r->n_trials > max_chunk && r->trace_acc)
    return fail(CEMC_ERR_LIMIT, "traced runs are limited to %llu trials per call", (unsigned long long)max_chunk);
  for (uint64_t done = 0; done < r->n_trials;) {
    const uint64_t n = std::min(max_chunk, r->n_trials - done);
    a.n_trials = n;
    a.chunk_offset = done;
    cudaError_t e = cemc::launch_mc(g, a, r->move, r->precision, L.total, static_cast<cudaStream_t>(stream), form,
                                    use_spin ? &geo->spin : nullptr);
    if (e != cudaSuccess) return cuda_fail(e, "Monte Carlo kernel launch");
    done += n;
  }
  r->kernel_used = form == cemc::kFormTable ? CEMC_KERNEL_TABLE
                  : (form == cemc::kFormGeneric || form == cemc::kFormRecycle) ? CEMC_KERNEL_GENERIC
                  : (a.tpw == 4 ? CEMC_KERNEL_SPIN_QUARTER : a.tpw == 2 ? CEMC_KERNEL_SPIN_HALFWARP : CEMC_KERNEL_SPIN);
  if (form == cemc::kFormTable) {
    cudaError_t e = cemc::launch_recompute(g, r->n_chains, r->occ, r->eci, r->cf, r->energy, rscratch,
                                           static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "recompute after the table kernel");
  }
  return CEMC_OK;
}

extern "C" size_t cemc_recompute_scratch_doubles(const cemc_geometry *geo, int32_t n_chains) {
  if (!geo || n_chains <= 0) return 0;
  return cemc::recompute_blocks(geo->g) * (size_t)n_chains * (size_t)geo->g.n_eci;
}

extern "C" int cemc_recompute(const cemc_geometry *geo, int32_t n_chains, const int8_t *occ, const double *eci,
                              double *cf, double *energy, double *scratch, void *stream) {
  if (!geo || n_chains <= 0 || !occ || !eci || !cf || !energy || !scratch)
    return fail(CEMC_ERR_ARG, "bad recompute arguments");
  if (n_chains > 65535) return fail(CEMC_ERR_LIMIT, "too many chains in one recompute");
  cudaError_t e = cemc::launch_recompute(geo->g, n_chains, occ, eci, cf, energy, scratch,
                                         static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "recompute kernel launch");
  return CEMC_OK;
}

extern "C" int cemc_recompute_noalloc(const cemc_geometry *geo, int32_t n_chains, const int8_t *occ,
                                      const double *eci, double *cf, double *energy, void *stream) {
  if (!geo || n_chains <= 0 || !occ || !eci || !cf || !energy)
    return fail(CEMC_ERR_ARG, "bad recompute_noalloc arguments");
  if (n_chains > 65535) return fail(CEMC_ERR_LIMIT, "too many chains in one recompute");
  const size_t need = cemc::recompute_blocks(geo->g) * (size_t)n_chains * (size_t)geo->g.n_eci;
  if (need > cemc::kNoAllocScratchDoubles)
    return fail(CEMC_ERR_LIMIT,
                "recompute_noalloc needs %zu scratch doubles but its fixed array holds %zu "
                "(reduce n_chains or call cemc_recompute with a caller buffer)",
                need, cemc::kNoAllocScratchDoubles);
  cudaError_t err = cudaSuccess;
  double *scratch = cemc::noalloc_scratch(&err);
  if (!scratch) return cuda_fail(err, "cudaGetSymbolAddress(recompute_noalloc scratch)");
  // Each scratch entry the second kernel reads is written by the first kernel
  // of the same call, so nothing has to be cleared between calls.
  cudaError_t e = cemc::launch_recompute(geo->g, n_chains, occ, eci, cf, energy, scratch,
                                         static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "recompute_noalloc kernel launch");
  return CEMC_OK;
}

extern "C" int cemc_energy(const cemc_geometry *geo, int32_t n_chains, const double *eci, const double *cf,
                           double *energy, void *stream) {
  if (!geo || n_chains <= 0 || !eci || !cf || !energy) return fail(CEMC_ERR_ARG, "bad energy arguments");
  cudaError_t e = cemc::launch_energy(geo->g, n_chains, eci, cf, energy, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "energy kernel launch");
  return CEMC_OK;
}

extern "C" int cemc_apply_changes(const cemc_geometry *geo, int8_t *occ, double *cf, double *energy,
                                  const double *eci, int32_t n_changes, const int32_t *sites, const int8_t *old_sym,
                                  const int8_t *new_sym, int32_t *status, void *stream) {
  if (!geo || !occ || !cf || !energy || !eci || n_changes < 0 || (n_changes > 0 && (!sites || !old_sym || !new_sym)))
    return fail(CEMC_ERR_ARG, "bad apply_changes arguments");
  if (cemc::warp_kernel_smem(geo->g) > (size_t)geo->max_smem) return fail(CEMC_ERR_LIMIT, "tables too large");
  cudaError_t e = cemc::launch_apply(geo->g, occ, cf, energy, eci, n_changes, sites, old_sym, new_sym, status,
                                     static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "apply_changes kernel launch");
  return CEMC_OK;
}

extern "C" int cemc_delta_e(const cemc_geometry *geo, const int8_t *occ, const double *eci, int32_t move,
                            int32_t site_a, int32_t site_b, int32_t new_a, double *de_out, double *dcf_out,
                            void *stream) {
  if (!geo || !occ || !eci || !de_out || !dcf_out) return fail(CEMC_ERR_ARG, "bad delta_e arguments");
  const cemc::DevGeo &g = geo->g;
  if (site_a < 0 || site_a >= g.n_sites) return fail(CEMC_ERR_ARG, "site out of range");
  if (move == CEMC_MOVE_SWAP && (site_b < 0 || site_b >= g.n_sites || site_b == site_a))
    return fail(CEMC_ERR_ARG, "bad swap partner");
  if (move == CEMC_MOVE_FLIP && (new_a < 0 || new_a >= g.n_sym)) return fail(CEMC_ERR_ARG, "bad species");
  cudaError_t e = cemc::launch_delta(g, occ, eci, move, site_a, site_b, new_a, de_out, dcf_out,
                                     static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "delta_e kernel launch");
  return CEMC_OK;
}

extern "C" int cemc_pt_exchange(int32_t n_replicas, int32_t direction, uint64_t seed, uint64_t round,
                                const double *energy, double *kT, int32_t *replica_of, int32_t *position_of,
                                int32_t *n_accept, void *stream) {
  if (n_replicas < 1 || !energy || !kT || !replica_of || (direction != 0 && direction != 1))
    return fail(CEMC_ERR_ARG, "bad replica-exchange arguments");
  cudaError_t e = cemc::launch_pt(n_replicas, direction, seed, round, energy, kT, replica_of, position_of, n_accept,
                                  static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "replica-exchange kernel launch");
  return CEMC_OK;
}
