// Local-field form of the Monte Carlo kernel (single-site flips in a binary
// +1/-1 basis): tables and the shared-memory layout, shared by the host
// (cemc_abi.cu, to size the launch) and the device (cemc_field.cu).
//
// The energy change of flipping site i is
//   dE = delta_i * (sum_k coef_k * P_k(i) + coef_singlet),   delta_i = s_new - s_old,
// with P_k(i) the sum over the terms of cluster ECI k at reference site i of
// the product of the other members' spins (ce_updater.cpp:244-285 for the
// products, 391-402 for the normalisation folded into coef_k).  Writing
// P_k(i) = K_k - 2 c_k(i), where K_k is the number of such terms and c_k(i)
// the number of them whose product is -1, the kernel keeps c_k(i) of every
// site of a chain packed into one or two 32-bit words in shared memory
// (bit fields wide enough for 0..K_k).  A trial then reads one or two words;
// an accepted flip of site j adds +-1 to the fields of every neighbour whose
// terms contain j, which is the only work that grows with the cluster set.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "cemc_launch.h"

namespace cemc {

constexpr int kFieldMaxCl = 32;     // cluster ECIs of a local-field geometry
constexpr int kFieldMaxSites = 32768;  // larger supercells do not fit one CTA's shared memory
constexpr int kFieldRound = 64;     // trials per round (at most; one stamp-slot byte each)

// Device tables of the local-field form (built in cemc_geometry_create).
//   slot_meta[q] = K_q | shift << 8 | word << 13 | bits << 16: cluster ECI q's count
//     field, bits (shift, bits) of word `word` of a site's packed counts;
//   cnt: n_cl pair entries (count = popcount of the spin word under the mask),
//     then one entry per multi-site term (count = parity under the mask), each
//     {mask lo, mask hi, field increment in word 0, in word 1} in the column
//     space of the counted site's own row;
//   pairinc[c]: packed increments of the pair terms that join a changed site j
//     to the target site row_j[c] (one per pair ECI whose shell holds c);
//   upd[ustart[c] .. ustart[c+1]): the multi-site terms at target row_j[c] that
//     contain j, in j's column space, each {mask lo, mask hi, field increment,
//     word | kind << 1 | members << 8}: kind 1 counts together the terms of one
//     cluster ECI with a single other member (mask = those members; after the
//     flip the count of -1 products changes by members - 2 x the members whose
//     spin differs from s_j's old spin), kind 0 is one term whose product
//     toggles with the parity of its other members.  Verified on the host to be
//     the same at every site.
struct FieldDev {
  int n_cl, pw, n_cnt, n_upd, minus_id, singlet_eci;
  const int32_t *slot_eci;    // [n_cl]
  const uint32_t *slot_meta;  // [n_cl]
  const uint4 *cnt;           // [n_cnt]
  const uint2 *pairinc;       // [n_cols]
  const int32_t *ustart;      // [n_cols + 1]
  const uint4 *upd;           // [n_upd]
};

struct FieldLayout {
  size_t cf, eci, w, acc, cfw, coef, kind, misc;
  size_t meta, scoef, cnt, pairinc, ustart, upd;
  size_t rec, rec_stride, rec_sa, rec_ns, rec_acc, rec_dl, rec_de, rec_ds, rec_p, rec_sw;
  size_t alist;  // [2][kFieldRound + 1]: per round parity, the accepted slots and their count
  size_t draws, rows, stamp, pc, occ, total;
};

__host__ __device__ inline size_t falign16(size_t x) { return (x + 15) & ~(size_t)15; }

// Shared-memory carve-up of field_kernel.  gstamp: the conflict table lives in
// a caller buffer in device memory instead.
__host__ __device__ inline FieldLayout field_layout(const DevGeo &g, int n_cl, int pw, int n_cnt, int n_upd,
                                                    int rsize, int ring_bits, bool gstamp) {
  FieldLayout L;
  size_t o = 0;
  const size_t K = (size_t)g.n_eci;
  L.cf = o;
  o = falign16(o + 8 * K);
  L.eci = o;
  o = falign16(o + 8 * K);
  L.w = o;
  o = falign16(o + 8 * K);
  L.acc = o;  // per-lane running sums of two bookers [2][2 + 3 * MAX_BF][32], singlets at launch start, 1/N
  o = falign16(o + 8 * (size_t)(2 * (2 + 3 * CEMC_MAX_BF) * 32 + CEMC_MAX_BF + 1));
  L.cfw = o;  // per-booker sums of committed correlation-function changes [2][n_eci]
  o = falign16(o + 8 * 2 * K);
  L.coef = o;
  o = falign16(o + (size_t)rsize * K);
  L.kind = o;
  o = falign16(o + 2 * K);
  L.misc = o;
  o = falign16(o + 4 * 64);
  L.meta = o;
  o = falign16(o + 4 * (size_t)n_cl);
  L.scoef = o;  // coefficient of each cluster slot
  o = falign16(o + (size_t)rsize * n_cl);
  L.cnt = o;
  o = falign16(o + 16 * (size_t)n_cnt);
  L.pairinc = o;
  o = falign16(o + 8 * (size_t)g.n_cols);
  L.ustart = o;
  o = falign16(o + 4 * (size_t)(g.n_cols + 1));
  L.upd = o;
  o = falign16(o + 16 * (size_t)n_upd);
  const size_t S = kFieldRound;
  size_t r = 0;
  L.rec_sa = r;
  r += 4 * S;
  L.rec_p = r;
  r += 4 * S * 2;
  L.rec_sw = r;  // spin word of an accepted trial's neighbour row at the start of its round
  r += 4 * S * 2;
  L.rec_de = r;
  r += (size_t)rsize * S;
  L.rec_ds = r;
  r += (size_t)rsize * S;
  L.rec_ns = r;
  r += S;
  L.rec_acc = r;
  r += S;
  L.rec_dl = r;
  r += S;
  L.rec_stride = falign16(r);
  L.rec = o;
  o = falign16(o + 2 * L.rec_stride);
  L.alist = o;
  o = falign16(o + 4 * 2 * (S + 1));
  const size_t ring = (size_t)1 << ring_bits;
  L.draws = o;  // FieldDraw (16 bytes) per ring slot
  o = falign16(o + 16 * ring);
  L.rows = o;
  o = falign16(o + 4 * ring * (size_t)g.cpad);
  L.stamp = o;
  if (!gstamp) o = falign16(o + 4 * (size_t)g.n_sites);
  L.pc = o;
  o = falign16(o + 4 * (size_t)pw * g.n_sites);
  L.occ = o;
  o = falign16(o + (size_t)g.n_sites);
  L.total = o;
  return L;
}

// Ring slots (log2) for rounds of `cw` trials: the fetcher stays at least
// three rounds ahead, so every row a round reads was copied two rounds earlier.
__host__ __device__ inline int field_ring_bits(int cw) {
  int b = 5;
  while ((1 << b) < 3 * cw) ++b;
  return b;
}

// Trials per round of `warps` worker warps: 64, or 32 for a single worker warp.
__host__ __device__ inline int field_round(int warps) { return warps >= 2 ? kFieldRound : 32; }
constexpr int kFieldFetchers = 2;   // fetcher warps
constexpr int kFieldMaxWarps = 28;  // worker warps; two bookers and two fetchers make 32 warps at most
// Threads of a field_kernel CTA with `warps` worker warps.
__host__ __device__ inline int field_threads(int warps) {
  return (warps + (field_round(warps) > 32 ? 2 : 1) + kFieldFetchers) * 32;
}

cudaError_t launch_field(const DevGeo &g, const RunArgs &a, const FieldDev &fd, int precision, size_t smem,
                         cudaStream_t st);

}  // namespace cemc
