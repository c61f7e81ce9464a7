// Device-side data layout and building blocks shared by the CE Monte Carlo kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cemc_gb300.h"
#include "philox.h"

namespace cemc {

constexpr int kWarp = 32;
constexpr int kMaxWarps = 32;
constexpr int kMaxSlots = 31;      // ECIs one lane's chunk of terms may touch (5-bit field)
constexpr int kRefBits = 11;       // low bits of a term's first field: vals index of the delta
constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxTable = 16384;   // table-form entries per chain (shared memory)
constexpr int kMaxGeo = 2048;      // cluster geometries per site in the table form

// Device copy of one geometry (supercell + cluster expansion).
//
// Trial-move terms: the flattened (cluster ECI, equivalent decoration,
// sub-cluster) products of a site, sorted by ECI and cut into 32 contiguous
// chunks, one per lane.  Each term is 4 x uint16:
//   f[0] = (vals index of delta[d_ref]) | (slot << 11)
//   f[1..3] = vals index of (column, decoration) of members 1..3, or the
//             index of the constant 1.0 for absent members.
// "vals" is a per-warp array: bf[d][species of neighbour c] at c * n_bf + d,
// 1.0 at n_cols * n_bf, delta[d] = bf[d][new] - bf[d][old] right after.
// The slot is the ECI index relative to the first ECI of the lane's chunk.
struct DevGeo {
  int n_sites, n_cols, n_sym, n_bf, n_eci, n_terms;
  int vals_len;    // n_cols * n_bf + 1 + n_bf
  int one_idx;     // n_cols * n_bf
  int n_slots;     // max ECIs per lane chunk
  int cpad;        // row stride of `table`: n_cols rounded up to a multiple of 4 (16-byte rows)
  const int32_t *table;     // [n_sites * cpad] row-major (trial moves), padding columns repeat column 0
  const int32_t *table_cm;  // [n_cols * n_sites] column-major (full recompute)
  const uint16_t *terms;    // [n_terms * 4]
  const int32_t *lane_term; // [33] chunk boundaries
  const int32_t *lane_first_eci;  // [32]
  const int32_t *eci_lane;  // [n_eci * 2] first and last lane holding terms of the ECI (last < first: none)
  const int32_t *eci_kind;  // [n_eci]
  const int32_t *eci_dec;   // [n_eci]
  const double *eci_w;      // [n_eci] increment weight (cluster), 0 otherwise
  const double *eci_fw;     // [n_eci] full-recompute weight (cluster)
  const double *bf;         // [n_bf * n_sym]
  const uint8_t *fterms;    // [n_terms * 8] {col0, col1, col2, d0, d1, d2, d_ref, size}
  const int32_t *fterm_off; // [n_eci + 1] ranges of fterms per ECI
  int singlet_eci[CEMC_MAX_BF];
  int pm1_minus;  // binary basis with values exactly +1 / -1: species id of -1; otherwise -1
  // table form of the trial energy change (see cemc_geometry_create)
  int table_ok, n_geo, n_pat, tab_len;
  const uint4 *geo_list;     // [n_geo] {columns c1 | c2 << 8 | c3 << 16 (absent: n_cols), F offset, S^m, 0}
  const int4 *pat_info;      // [n_pat] {m, F offset, first term, end term}
  const int32_t *pat_terms;  // k | d_ref << 8 | d1 << 12 | d2 << 16 | d3 << 20
  int n_movable;             // sites that may change (n_sites when there is no background)
  const int32_t *movable;    // [n_movable] ascending (used when n_movable < n_sites)
  const int8_t *site_active; // [n_sites] 1 = movable; NULL when every site is
  // Translation-symmetry groups (1 = one group).  The lane-chunk tables
  // (lane_term [G][33], lane_first_eci [G][32], eci_lane [G][2 n_eci]) and
  // fterm_off ([G][n_eci + 1]) hold one block per group; a site's table row
  // lists its group's columns.
  int n_groups;
  const int8_t *site_group;    // [n_sites]
  const int32_t *geo_start;    // [n_groups + 1] table-form geometry range of each group
  const double *group_scale;   // [n_groups] factor on a site's cluster-ECI changes
  // Periodic box (0 = none): sites numbered ((x * box_L + y) * box_L + z) * box_nb + b over an
  // L^3 box of cells with box_nb basis sites, and the table equal to a fixed cell offset and basis
  // site per (b, column) at every site (checked when the geometry is built).  Then a swap trial
  // computes its neighbour sites instead of loading the two rows.
  int box_L, box_nb;
  uint32_t box_mnb, box_mL;    // ceil(2^32 / d) for d = box_nb, box_L (division by multiply-high, checked)
  const uint32_t *box_off;     // [box_nb * n_cols] (dx + 128) | (dy + 128) << 8 | (dz + 128) << 16 | b' << 24
};

// A neighbour row: in memory (the table, or a row copied to shared memory), or
// computed from the site's cell in a periodic box.
struct RowRef {
  const int32_t *row;  // nullptr: computed
  int cx, cy, cz, b;
};
__device__ __forceinline__ RowRef row_mem(const int32_t *row) {
  RowRef r;
  r.row = row;
  r.cx = r.cy = r.cz = r.b = 0;
  return r;
}
__device__ __forceinline__ RowRef row_of_site(const DevGeo &g, int site) {
  RowRef r;
  if (g.box_L == 0) {
    r.row = g.table + (size_t)site * g.cpad;
    r.cx = r.cy = r.cz = r.b = 0;
    return r;
  }
  r.row = nullptr;
  const uint32_t L = (uint32_t)g.box_L;
  const uint32_t cell = g.box_nb == 1 ? (uint32_t)site : __umulhi((uint32_t)site, g.box_mnb);
  r.b = site - (int)(cell * (uint32_t)g.box_nb);
  const uint32_t q = L == 1 ? cell : __umulhi(cell, g.box_mL);
  r.cz = (int)(cell - q * L);
  const uint32_t q2 = L == 1 ? q : __umulhi(q, g.box_mL);
  r.cy = (int)(q - q2 * L);
  r.cx = (int)q2;
  return r;
}
__device__ __forceinline__ int row_at(const DevGeo &g, const RowRef &r, int c) {
  if (r.row) return r.row[c];
  const uint32_t o = __ldg(g.box_off + r.b * g.n_cols + c);
  const int L = g.box_L;
  int x = r.cx + (int)(o & 255u) - 128, y = r.cy + (int)((o >> 8) & 255u) - 128, z = r.cz + (int)((o >> 16) & 255u) - 128;
  x += x < 0 ? L : 0;
  x -= x >= L ? L : 0;
  y += y < 0 ? L : 0;
  y -= y >= L ? L : 0;
  z += z < 0 ? L : 0;
  z -= z >= L ? L : 0;
  return ((x * L + y) * L + z) * g.box_nb + (int)(o >> 24);
}

// Ints of one group's block of lane-chunk tables in shared memory:
// [33] chunk bounds, [32] first ECI per lane, [2 n_eci] lane range per ECI.
__host__ __device__ inline int group_lane_ints(int n_eci) { return 65 + 2 * n_eci; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
template <typename R>
__device__ __forceinline__ R warp_scan_incl(R v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const R n = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

// Double-float: a value carried as an unevaluated sum hi + lo of two floats
// (about 48 significant bits), added and multiplied on the FP32 pipe with the
// error-free transformations TwoSum (Knuth) and TwoProd (by fused multiply-add).
// The Monte Carlo kernel keeps its per-round running sums in this form in FP32
// mode: FP64 instructions are slow to issue on this part and would otherwise
// sit on the critical path of every round.  Values move to FP64 once per launch.
struct df64 {
  float hi, lo;
};
__device__ __forceinline__ df64 df_from(double d) {
  df64 r;
  r.hi = (float)d;
  r.lo = (float)(d - (double)r.hi);
  return r;
}
__device__ __forceinline__ double df_to(df64 a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ df64 df_norm(float s, float e) {
  const float hi = __fadd_rn(s, e);
  df64 r;
  r.hi = hi;
  r.lo = __fsub_rn(e, __fsub_rn(hi, s));
  return r;
}
__device__ __forceinline__ df64 df_add(df64 a, float b) {
  const float s = __fadd_rn(a.hi, b);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df_norm(s, __fadd_rn(a.lo, e));
}
__device__ __forceinline__ df64 df_add(df64 a, df64 b) { return df_add(df_add(a, b.hi), b.lo); }
__device__ __forceinline__ df64 df_mul(df64 a, float b) {
  const float p = __fmul_rn(a.hi, b);
  const float e = __fmaf_rn(a.hi, b, -p);
  return df_norm(p, __fmaf_rn(a.lo, b, e));
}
__device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.hi, -p);
  return df_norm(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e)));
}

// Running-sum arithmetic shared by both precisions: A = double in FP64 mode,
// df64 in FP32 mode; x is a per-trial value of the mode's type.
__device__ __forceinline__ double acc_add(double a, double b) { return a + b; }
__device__ __forceinline__ df64 acc_add(df64 a, df64 b) { return df_add(a, b); }
__device__ __forceinline__ double acc_mul(double a, double b) { return a * b; }
__device__ __forceinline__ df64 acc_mul(df64 a, df64 b) { return df_mul(a, b); }
__device__ __forceinline__ double acc_add_x(double a, double x) { return a + x; }
__device__ __forceinline__ df64 acc_add_x(df64 a, float x) { return df_add(a, x); }
__device__ __forceinline__ double acc_to(double a) { return a; }
__device__ __forceinline__ double acc_to(df64 a) { return df_to(a); }
template <typename A>
__device__ __forceinline__ A acc_from(double d);
template <>
__device__ __forceinline__ double acc_from<double>(double d) { return d; }
template <>
__device__ __forceinline__ df64 acc_from<df64>(double d) { return df_from(d); }

// Metropolis test of the reference, accept = (dE < 0) or (u <= exp(-dE / kT))
// (cemc/mcmc/montecarlo.py:950-956), with u the 53-bit uniform of words (a, b).
// The test is first made in single precision as ln(u) + dE/kT against a
// margin that bounds every single-precision error involved: u is taken as
// a * 2^-32 (within 2^-27 of the 53-bit u), ln on the special-function unit,
// x = dE/kT rounded to float.  Only trials inside the margin evaluate the
// exact double-precision form, so the decision equals the double-precision
// one while the common case issues no FP64 instruction (the FP64 pipe of this
// part is narrow).
template <typename R>
__device__ __forceinline__ int metropolis(R de, uint32_t ua, uint32_t ub, double kT, float inv_kT) {
  if (de < (R)0) return 1;
  const float x = (float)de * inv_kT;
  const float uf = (float)ua * 2.3283064e-10f;  // a * 2^-32
  const float y = __logf(uf) + x;
  const float margin = 1e-4f + 1e-6f * x + 1e-8f / uf;  // uf == 0 gives an infinite margin
  if (y < -margin) return 1;
  if (y > margin) return 0;
  return cemc_u01_53(ua, ub) <= exp(-(double)de / kT);
}

// The same test with the uniform's parts precomputed (by the fetcher, off the
// evaluating warps' path): lnu = __logf(u) and mu = 1e-4 + 1e-8 / u for
// u = ua * 2^-32.  The margin can differ from metropolis()'s in its last bit,
// which only moves a trial between the single-precision test and the exact one.
// `uw` points at the uniform's two words, read only inside the margin.
template <typename R>
__device__ __forceinline__ int metropolis_pre(R de, float lnu, float mu, const uint32_t *uw, double kT,
                                              float inv_kT) {
  if (de < (R)0) return 1;
  const float x = (float)de * inv_kT;
  const float y = lnu + x;
  const float margin = mu + 1e-6f * x;  // u == 0 gives an infinite margin
  if (y < -margin) return 1;
  if (y > margin) return 0;
  return cemc_u01_53(uw[0], uw[1]) <= exp(-(double)de / kT);
}
__device__ __forceinline__ void metropolis_parts(uint32_t ua, float &lnu, float &mu) {
  const float uf = (float)ua * 2.3283064e-10f;  // a * 2^-32
  lnu = __logf(uf);
  mu = 1e-4f + 1e-8f / uf;
}

// Two-state acceptance of waste recycling (Frenkel, PNAS 101, 17571 (2004);
// montecarlo.py:937-948): the reference draws the next state from the weights
// exp(-E / kT) of the current and the proposed state, i.e. it accepts when
// u > p0 = 1 / (1 + exp(-dE / kT)), evaluated here in FP64.
template <typename R>
__device__ __forceinline__ int barker(R de, uint32_t ua, uint32_t ub, double kT) {
  const double p0 = 1.0 / (1.0 + exp(-(double)de / kT));
  return cemc_u01_53(ua, ub) > p0;
}

// Fill one warp's vals array for a change of `site` from species `old_s` to
// `new_s`.  Neighbour species come from `occ`, except that `ovr_site` (if >=
// 0) is read as species `ovr_s` (the first half of a swap already applied).
// Each lane keeps the neighbour site ids of its columns in nbr[] for the
// conflict test.
template <typename R>
__device__ __forceinline__ void gather_vals(const DevGeo &g, const int8_t *occ, const R *bf_s, int site, int old_s,
                                            int new_s, int ovr_site, int ovr_s, R *vals, int (&nbr)[4], int lane) {
  const RowRef row = row_of_site(g, site);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = lane + 32 * j;
    nbr[j] = -1;
    if (c < g.n_cols) {
      const int s = row_at(g, row, c);
      nbr[j] = s;
      const int o = (s == ovr_site) ? ovr_s : (int)occ[s];
      for (int d = 0; d < g.n_bf; ++d) vals[c * g.n_bf + d] = bf_s[d * g.n_sym + o];
    }
  }
  if (lane == 0) {
    vals[g.one_idx] = (R)1;
    for (int d = 0; d < g.n_bf; ++d) vals[g.one_idx + 1 + d] = bf_s[d * g.n_sym + new_s] - bf_s[d * g.n_sym + old_s];
  }
}

// Sum this lane's chunk of terms into per-slot partials part[slot * 32 + lane].
// With TWO, the product over a second vals array (the second site of a swap)
// is added term by term.
template <typename R, bool TWO>
__device__ __forceinline__ void lane_terms(const DevGeo &g, const uint16_t *terms_s, const int32_t *lane_term_s,
                                           const R *va, const R *vb, R *part, int lane) {
  for (int s = 0; s < g.n_slots; ++s) part[s * 32 + lane] = (R)0;
  const int lo = lane_term_s[lane], hi = lane_term_s[lane + 1];
  if (lo >= hi) return;
  int cur = terms_s[4 * lo] >> kRefBits;
  R acc = (R)0;
  for (int i = lo; i < hi; ++i) {
    const uint2 packed = *reinterpret_cast<const uint2 *>(terms_s + 4 * i);
    const int f0 = packed.x & 0xffff, f1 = packed.x >> 16, f2 = packed.y & 0xffff, f3 = packed.y >> 16;
    const int sl = f0 >> kRefBits, ri = f0 & ((1 << kRefBits) - 1);
    if (sl != cur) {
      part[cur * 32 + lane] = acc;
      acc = (R)0;
      cur = sl;
    }
    R p = va[ri] * va[f1] * va[f2] * va[f3];
    if (TWO) p += vb[ri] * vb[f1] * vb[f2] * vb[f3];
    acc += p;
  }
  part[cur * 32 + lane] = acc;
}

// Combine per-lane partials into the per-ECI change D[k] (term sum times the
// site group's scale for cluster ECIs, delta[d] for singlets) and return the
// energy change sum_k coef[k] * D[k] (coef = N * eci * weight), identical on
// all lanes.  ADD adds to D instead of overwriting it.
template <typename R, bool TWO, bool ADD = false>
__device__ __forceinline__ R eci_changes(const DevGeo &g, const int32_t *eci_lane_s, const int32_t *first_s,
                                         const int8_t *kind_s, const int8_t *dec_s, const R *coef_s, const R *part,
                                         const R *va, const R *vb, R *D, int lane, R gscale = (R)1) {
  R de = (R)0;
  for (int k = lane; k < g.n_eci; k += 32) {
    R v = (R)0;
    const int kind = kind_s[k];
    if (kind == 2) {
      const int lo = eci_lane_s[2 * k], hi = eci_lane_s[2 * k + 1];
      for (int l = lo; l <= hi; ++l) v += part[(k - first_s[l]) * 32 + l];
      v *= gscale;
    } else if (kind == 1) {
      const int d = dec_s[k];
      v = va[g.one_idx + 1 + d];
      if (TWO) v += vb[g.one_idx + 1 + d];
    }
    D[k] = ADD ? D[k] + v : v;
    de += coef_s[k] * v;
  }
  return warp_sum(de);
}

// Energy change and per-ECI changes D of one flip (va) or swap (va, then vb
// with the first site already changed) whose sites belong to translation
// groups ga and gb.  lane_s holds the groups' lane-chunk blocks
// (group_lane_ints each), gscale_s their scales.  Two sites of one group walk
// the group's terms once for both vals arrays; two groups take one pass each.
template <typename R, bool SWAP>
__device__ __forceinline__ R site_changes(const DevGeo &g, const uint16_t *terms_s, const int32_t *lane_s,
                                          const int8_t *kind_s, const int8_t *dec_s, const R *coef_s,
                                          const R *gscale_s, R *part, const R *va, const R *vb, R *D, int ga, int gb,
                                          int lane) {
  const int LG = group_lane_ints(g.n_eci);
  const int32_t *la = lane_s + ga * LG;
  if (!SWAP || ga == gb) {
    lane_terms<R, SWAP>(g, terms_s, la, va, vb, part, lane);
    __syncwarp();
    return eci_changes<R, SWAP>(g, la + 65, la + 33, kind_s, dec_s, coef_s, part, va, vb, D, lane, gscale_s[ga]);
  }
  const int32_t *lb = lane_s + gb * LG;
  lane_terms<R, false>(g, terms_s, la, va, va, part, lane);
  __syncwarp();
  R de = eci_changes<R, false>(g, la + 65, la + 33, kind_s, dec_s, coef_s, part, va, va, D, lane, gscale_s[ga]);
  __syncwarp();
  lane_terms<R, false>(g, terms_s, lb, vb, vb, part, lane);
  __syncwarp();
  de += eci_changes<R, false, true>(g, lb + 65, lb + 33, kind_s, dec_s, coef_s, part, vb, vb, D, lane, gscale_s[gb]);
  return de;
}

}  // namespace cemc
