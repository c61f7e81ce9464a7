// Correlation-function kernels besides the fused MC loop:
//   * full recompute over all sites (validation and FP64 drift reset),
//   * sequential application of explicit site changes (calculator path),
//   * the energy change of one move without committing it (replay / debug),
//   * replica exchange over a temperature ladder.
#include <cuda_runtime.h>

#include <mutex>
#include <unordered_map>

#include "cemc_device.cuh"
#include "cemc_kernels.h"

namespace cemc {

// Scratch of cemc_recompute_noalloc: the per-block partial sums of the full
// recompute live in this fixed device array instead of a caller buffer, so
// that entry point allocates nothing.  Every GPU that loads the library holds
// it (8 MiB) until the process exits.  Host code must not use the symbol as a
// pointer: noalloc_scratch() resolves its device address per device.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

double *noalloc_scratch(cudaError_t *err) {
  static std::mutex mu;
  static std::unordered_map<int, double *> addr;  // device ordinal -> address of g_noalloc_scratch there
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *err = e;
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  auto it = addr.find(dev);
  if (it != addr.end()) return it->second;
  double *p = nullptr;
  e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_noalloc_scratch);
  if (e != cudaSuccess) {
    *err = e;
    return nullptr;
  }
  addr[dev] = p;
  return p;
}

// ---------------------------------------------------------------------------
// Full recompute.  Block (bx, chain) handles sites [bx*256, bx*256+256) of one
// chain: it stages the species of every neighbour column of its sites in
// shared memory (coalesced reads of the column-major table), then walks the
// cluster terms ECI by ECI, one site per thread.  A binary geometry whose
// basis values are exactly +1 and -1 (g.pm1_minus >= 0) stages one "is the -1
// species" bit per column instead and takes the sign of each product as the
// parity of its members' bits: integer sums, exact, with no FP64 arithmetic.
// Other bases multiply their FP64 basis values.  Each warp's sum of an ECI
// goes to shared memory; after the last ECI thread k adds the eight warps in
// order into scratch[(chain * n_blocks + bx) * n_eci + k], and recompute_finish
// adds the blocks in order, so the result is deterministic.
constexpr int kCfThreads = 256;

template <bool PM1>
__global__ void __launch_bounds__(kCfThreads) recompute_partial(DevGeo g, const int8_t *occ_all, double *scratch,
                                                                int n_blocks) {
  extern __shared__ __align__(16) unsigned char smem[];
  int8_t *nb = reinterpret_cast<int8_t *>(smem);  // [n_cols][256] species, or -1-species bits
  double *red = reinterpret_cast<double *>(smem + align16((size_t)g.n_cols * kCfThreads));  // [8][n_eci]
  double *bf_s = red + (kCfThreads / 32) * g.n_eci;                                        // [n_bf * n_sym]
  const int chain = blockIdx.y, bx = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int N = g.n_sites;
  const int i = bx * kCfThreads + tid;
  const bool valid = i < N && (!g.site_active || g.site_active[i]);  // background sites hold no clusters
  const int8_t *occ = occ_all + (size_t)chain * N;
  const int minus = g.pm1_minus;
  if (!PM1)
    for (int q = tid; q < g.n_bf * g.n_sym; q += kCfThreads) bf_s[q] = g.bf[q];
  for (int c = 0; c < g.n_cols; ++c) {
    int8_t v = 0;
    if (valid) {
      const int o = occ[g.table_cm[(size_t)c * N + i]];
      v = PM1 ? (int8_t)(o == minus) : (int8_t)o;
    }
    nb[c * kCfThreads + tid] = v;
  }
  const int me = valid ? occ[i] : 0;
  const int me_bit = (me == minus) ? 1 : 0;
  // the term ranges of the site's translation group
  const int32_t *foff = g.fterm_off + (size_t)(valid && g.n_groups > 1 ? g.site_group[i] : 0) * (g.n_eci + 1);
  __syncthreads();
  for (int k = 0; k < g.n_eci; ++k) {
    const int kind = g.eci_kind[k];
    if (kind == 0) continue;
    const int f0 = foff[k], f1 = foff[k + 1];
    double s;
    if (PM1) {
      int cnt = 0;
      if (valid) {
        if (kind == 1) {
          cnt = 1 - 2 * me_bit;
        } else {
          for (int f = f0; f < f1; ++f) {
            const uint2 t = __ldg(reinterpret_cast<const uint2 *>(g.fterms) + f);
            const int c0 = t.x & 0xff, c1 = (t.x >> 8) & 0xff, c2 = (t.x >> 16) & 0xff;
            const int size = (t.y >> 24) & 0xff;
            int bit = me_bit ^ nb[c0 * kCfThreads + tid];
            if (size >= 3) bit ^= nb[c1 * kCfThreads + tid];
            if (size >= 4) bit ^= nb[c2 * kCfThreads + tid];
            cnt += 1 - 2 * bit;
          }
        }
      }
      s = (double)__reduce_add_sync(kFull, cnt);
    } else {
      s = 0.0;
      if (valid && kind == 1) {
        s = bf_s[g.eci_dec[k] * g.n_sym + me];
      } else if (valid && kind == 2) {
        for (int f = f0; f < f1; ++f) {
          const uint2 t = __ldg(reinterpret_cast<const uint2 *>(g.fterms) + f);
          const int c0 = t.x & 0xff, c1 = (t.x >> 8) & 0xff, c2 = (t.x >> 16) & 0xff;
          const int d0 = (t.x >> 24) & 0xff, d1 = t.y & 0xff, d2 = (t.y >> 8) & 0xff, dr = (t.y >> 16) & 0xff;
          const int size = (t.y >> 24) & 0xff;
          double p = bf_s[dr * g.n_sym + me] * bf_s[d0 * g.n_sym + nb[c0 * kCfThreads + tid]];
          if (size >= 3) p *= bf_s[d1 * g.n_sym + nb[c1 * kCfThreads + tid]];
          if (size >= 4) p *= bf_s[d2 * g.n_sym + nb[c2 * kCfThreads + tid]];
          s += p;
        }
      }
      s = warp_sum(s);
    }
    if (lane == 0) red[warp * g.n_eci + k] = s;
  }
  __syncthreads();
  for (int k = tid; k < g.n_eci; k += kCfThreads) {
    if (g.eci_kind[k] == 0) continue;
    double b = 0.0;
    for (int w = 0; w < kCfThreads / 32; ++w) b += red[w * g.n_eci + k];
    scratch[((size_t)chain * n_blocks + bx) * g.n_eci + k] = b;
  }
}

__global__ void recompute_finish(DevGeo g, int n_blocks, const double *scratch, const double *eci, double *cf,
                                 double *energy) {
  extern __shared__ __align__(16) unsigned char smem[];
  double *cf_s = reinterpret_cast<double *>(smem);
  const int chain = blockIdx.x;
  for (int k = threadIdx.x; k < g.n_eci; k += blockDim.x) {
    const int kind = g.eci_kind[k];
    double v;
    if (kind == 0) {
      v = 1.0;
    } else {
      double s = 0.0;
      for (int b = 0; b < n_blocks; ++b) s += scratch[((size_t)chain * n_blocks + b) * g.n_eci + k];
      v = (kind == 1) ? s / (double)g.n_sites : s * g.eci_fw[k];
    }
    cf_s[k] = v;
    cf[(size_t)chain * g.n_eci + k] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // N * sum(eci * cf) in sorted-name order (ce_updater.cpp:236-242).
    double e = 0.0;
    for (int k = 0; k < g.n_eci; ++k) e += eci[(size_t)chain * g.n_eci + k] * cf_s[k];
    energy[chain] = e * (double)(unsigned)g.n_sites;
  }
}

__global__ void energy_kernel(int n_chains, int n_eci, int n_sites, const double *eci, const double *cf,
                              double *energy) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_chains) return;
  double e = 0.0;
  for (int k = 0; k < n_eci; ++k) e += eci[(size_t)c * n_eci + k] * cf[(size_t)c * n_eci + k];
  energy[c] = e * (double)(unsigned)n_sites;
}

// ---------------------------------------------------------------------------
// Single-warp FP64 kernels over explicit moves.
struct WarpLayout {
  size_t terms, lane, gscale, kind, coef, bf, va, vb, part, d, total;
};

__host__ __device__ inline WarpLayout warp_layout(const DevGeo &g) {
  WarpLayout L;
  size_t o = 0;
  L.terms = o;
  o = align16(o + 8 * (size_t)g.n_terms);
  L.lane = o;  // one block of lane-chunk tables per translation group
  o = align16(o + 4 * (size_t)g.n_groups * group_lane_ints(g.n_eci));
  L.gscale = o;
  o = align16(o + 8 * (size_t)g.n_groups);
  L.kind = o;
  o = align16(o + 2 * (size_t)g.n_eci);
  L.coef = o;
  o = align16(o + 8 * (size_t)g.n_eci);
  L.bf = o;
  o = align16(o + 8 * (size_t)g.n_bf * g.n_sym);
  L.va = o;
  o = align16(o + 8 * (size_t)g.vals_len);
  L.vb = o;
  o = align16(o + 8 * (size_t)g.vals_len);
  L.part = o;
  o = align16(o + 8 * (size_t)g.n_slots * 32);
  L.d = o;
  o = align16(o + 8 * (size_t)g.n_eci);
  L.total = o;
  return L;
}

size_t warp_kernel_smem(const DevGeo &g) { return warp_layout(g).total; }

struct WarpSmem {
  uint16_t *terms;
  int32_t *lane_term;  // [groups][group_lane_ints]
  int8_t *kind, *dec;
  double *gscale, *coef, *bf, *va, *vb, *part, *d;
};

__device__ WarpSmem warp_stage(const DevGeo &g, const double *eci, unsigned char *smem) {
  const WarpLayout L = warp_layout(g);
  WarpSmem s;
  s.terms = reinterpret_cast<uint16_t *>(smem + L.terms);
  s.lane_term = reinterpret_cast<int32_t *>(smem + L.lane);
  s.gscale = reinterpret_cast<double *>(smem + L.gscale);
  s.kind = reinterpret_cast<int8_t *>(smem + L.kind);
  s.dec = s.kind + g.n_eci;
  s.coef = reinterpret_cast<double *>(smem + L.coef);
  s.bf = reinterpret_cast<double *>(smem + L.bf);
  s.va = reinterpret_cast<double *>(smem + L.va);
  s.vb = reinterpret_cast<double *>(smem + L.vb);
  s.part = reinterpret_cast<double *>(smem + L.part);
  s.d = reinterpret_cast<double *>(smem + L.d);
  const int tid = threadIdx.x;
  for (int i = tid; i < g.n_terms; i += blockDim.x)
    reinterpret_cast<uint2 *>(s.terms)[i] = reinterpret_cast<const uint2 *>(g.terms)[i];
  const int LG = group_lane_ints(g.n_eci);
  for (int i = tid; i < g.n_groups * LG; i += blockDim.x) {
    const int q = i / LG, r = i - q * LG;
    s.lane_term[i] = r < 33 ? g.lane_term[33 * q + r]
                            : (r < 65 ? g.lane_first_eci[32 * q + r - 33] : g.eci_lane[(size_t)2 * g.n_eci * q + r - 65]);
  }
  for (int q = tid; q < g.n_groups; q += blockDim.x) s.gscale[q] = g.group_scale[q];
  for (int k = tid; k < g.n_eci; k += blockDim.x) {
    const int kind = g.eci_kind[k];
    s.kind[k] = (int8_t)kind;
    s.dec[k] = (int8_t)g.eci_dec[k];
    s.coef[k] = kind == 2 ? eci[k] * (double)g.n_sites * g.eci_w[k] : (kind == 1 ? eci[k] : 0.0);
  }
  for (int i = tid; i < g.n_bf * g.n_sym; i += blockDim.x) s.bf[i] = g.bf[i];
  __syncthreads();
  return s;
}

// Sequential single-site changes (CEUpdater::update_cf applied in order,
// ce_updater.cpp:845-853), committed in place.  One warp.
__global__ void apply_changes_kernel(DevGeo g, int8_t *occ, double *cf, double *energy, const double *eci,
                                     int n_changes, const int32_t *sites, const int8_t *old_sym,
                                     const int8_t *new_sym, int32_t *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  WarpSmem s = warp_stage(g, eci, smem);
  const int lane = threadIdx.x;
  int nbr[4];
  int rc = 0;
  for (int i = 0; i < n_changes; ++i) {
    const int site = sites[i];
    const int o = occ[site], n = new_sym[i];
    if (o != old_sym[i]) {
      rc = CEMC_ERR_STATE;
      break;
    }
    if (o == n) continue;
    const int grp = g.n_groups > 1 ? g.site_group[site] : 0;
    gather_vals<double>(g, occ, s.bf, site, o, n, -1, 0, s.va, nbr, lane);
    __syncwarp();
    site_changes<double, false>(g, s.terms, s.lane_term, s.kind, s.dec, s.coef, s.gscale, s.part, s.va, s.vb, s.d, grp,
                                grp, lane);
    for (int k = lane; k < g.n_eci; k += 32) {
      const int kind = s.kind[k];
      if (kind == 2) cf[k] = cf[k] + s.d[k] * g.eci_w[k];
      else if (kind == 1) cf[k] = cf[k] + s.d[k] / (double)g.n_sites;
    }
    __syncwarp();
    if (lane == 0) occ[site] = (int8_t)n;
    __syncwarp();
  }
  if (lane == 0) {
    double e = 0.0;
    for (int k = 0; k < g.n_eci; ++k) e += eci[k] * cf[k];
    *energy = e * (double)(unsigned)g.n_sites;
    if (status) *status = rc;
  }
}

__global__ void delta_e_kernel(DevGeo g, const int8_t *occ, const double *eci, int move, int site_a, int site_b,
                               int new_a, double *de_out, double *dcf_out) {
  extern __shared__ __align__(16) unsigned char smem[];
  WarpSmem s = warp_stage(g, eci, smem);
  const int lane = threadIdx.x;
  int nbra[4], nbrb[4];
  double de;
  const int ga = g.n_groups > 1 ? g.site_group[site_a] : 0;
  if (move == CEMC_MOVE_SWAP) {
    const int A = occ[site_a], B = occ[site_b];
    const int gb = g.n_groups > 1 ? g.site_group[site_b] : 0;
    gather_vals<double>(g, occ, s.bf, site_a, A, B, -1, 0, s.va, nbra, lane);
    gather_vals<double>(g, occ, s.bf, site_b, B, A, site_a, B, s.vb, nbrb, lane);
    __syncwarp();
    de = site_changes<double, true>(g, s.terms, s.lane_term, s.kind, s.dec, s.coef, s.gscale, s.part, s.va, s.vb, s.d,
                                    ga, gb, lane);
  } else {
    const int A = occ[site_a];
    gather_vals<double>(g, occ, s.bf, site_a, A, new_a, -1, 0, s.va, nbra, lane);
    __syncwarp();
    de = site_changes<double, false>(g, s.terms, s.lane_term, s.kind, s.dec, s.coef, s.gscale, s.part, s.va, s.vb,
                                     s.d, ga, ga, lane);
  }
  __syncwarp();
  for (int k = lane; k < g.n_eci; k += 32) {
    const int kind = s.kind[k];
    dcf_out[k] = kind == 2 ? s.d[k] * g.eci_w[k] : (kind == 1 ? s.d[k] / (double)g.n_sites : 0.0);
  }
  if (lane == 0) *de_out = de;
}

// ---------------------------------------------------------------------------
// Replica exchange (ParallelTempering._perform_exchange_move,
// cemc/mcmc/parallel_tempering.py:153-175): ladder pairs "up" (i, i+1) for
// even i, or "down" (i, i-1) for i = n-1, n-3, ...; acceptance
// u < exp((1/kT_1 - 1/kT_2) (E_1 - E_2)) (parallel_tempering.py:138-144,167).
// The two chains exchange temperatures and ladder positions.
__global__ void pt_exchange_kernel(int n, int direction, uint64_t seed, uint64_t round, const double *energy,
                                   double *kT, int32_t *replica_of, int32_t *position_of, int32_t *n_accept) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int acc_count = 0;
  if (direction == 0) {
    for (int i = 0; i + 1 < n; i += 2) {
      const int p = i, q = i + 1;
      const int ci = replica_of[p], cj = replica_of[q];
      const double b1 = 1.0 / kT[ci], b2 = 1.0 / kT[cj];
      const double prob = exp((b1 - b2) * (energy[ci] - energy[cj]));
      const cemc_u32x4 w = cemc_philox4x32_10((uint32_t)round, (uint32_t)(round >> 32), (uint32_t)p, 0xA5A5u,
                                              (uint32_t)seed, (uint32_t)(seed >> 32));
      const double u = cemc_u01_53(w.v[0], w.v[1]);
      if (u < prob) {
        const double t = kT[ci];
        kT[ci] = kT[cj];
        kT[cj] = t;
        replica_of[p] = cj;
        replica_of[q] = ci;
        ++acc_count;
      }
    }
  } else {
    for (int i = n - 1; i > 0; i -= 2) {
      const int p = i, q = i - 1;
      const int ci = replica_of[p], cj = replica_of[q];
      const double b1 = 1.0 / kT[ci], b2 = 1.0 / kT[cj];
      const double prob = exp((b1 - b2) * (energy[ci] - energy[cj]));
      const cemc_u32x4 w = cemc_philox4x32_10((uint32_t)round, (uint32_t)(round >> 32), (uint32_t)p, 0xA5A5u,
                                              (uint32_t)seed, (uint32_t)(seed >> 32));
      const double u = cemc_u01_53(w.v[0], w.v[1]);
      if (u < prob) {
        const double t = kT[ci];
        kT[ci] = kT[cj];
        kT[cj] = t;
        replica_of[p] = cj;
        replica_of[q] = ci;
        ++acc_count;
      }
    }
  }
  if (n_accept) *n_accept = acc_count;
  if (position_of)
    for (int p = 0; p < n; ++p) position_of[replica_of[p]] = p;
}

// ---------------------------------------------------------------------------
size_t recompute_blocks(const DevGeo &g) { return (size_t)((g.n_sites + kCfThreads - 1) / kCfThreads); }

cudaError_t launch_recompute(const DevGeo &g, int n_chains, const int8_t *occ, const double *eci, double *cf,
                             double *energy, double *scratch, cudaStream_t st) {
  const int nb = (int)recompute_blocks(g);
  const size_t smem1 =
      align16((size_t)g.n_cols * kCfThreads) + 8 * ((kCfThreads / 32) * (size_t)g.n_eci + (size_t)g.n_bf * g.n_sym);
  auto kern = g.pm1_minus >= 0 ? recompute_partial<true> : recompute_partial<false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
  if (e != cudaSuccess) return e;
  kern<<<dim3(nb, n_chains), kCfThreads, smem1, st>>>(g, occ, scratch, nb);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  recompute_finish<<<n_chains, 128, 8 * (size_t)g.n_eci, st>>>(g, nb, scratch, eci, cf, energy);
  return cudaGetLastError();
}

cudaError_t launch_apply(const DevGeo &g, int8_t *occ, double *cf, double *energy, const double *eci, int n,
                         const int32_t *sites, const int8_t *old_sym, const int8_t *new_sym, int32_t *status,
                         cudaStream_t st) {
  const size_t smem = warp_kernel_smem(g);
  cudaError_t e = cudaFuncSetAttribute(apply_changes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  apply_changes_kernel<<<1, 32, smem, st>>>(g, occ, cf, energy, eci, n, sites, old_sym, new_sym, status);
  return cudaGetLastError();
}

cudaError_t launch_delta(const DevGeo &g, const int8_t *occ, const double *eci, int move, int sa, int sb, int na,
                         double *de, double *dcf, cudaStream_t st) {
  const size_t smem = warp_kernel_smem(g);
  cudaError_t e = cudaFuncSetAttribute(delta_e_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  delta_e_kernel<<<1, 32, smem, st>>>(g, occ, eci, move, sa, sb, na, de, dcf);
  return cudaGetLastError();
}

cudaError_t launch_energy(const DevGeo &g, int n_chains, const double *eci, const double *cf, double *energy,
                          cudaStream_t st) {
  energy_kernel<<<(n_chains + 127) / 128, 128, 0, st>>>(n_chains, g.n_eci, g.n_sites, eci, cf, energy);
  return cudaGetLastError();
}

cudaError_t launch_pt(int n, int direction, uint64_t seed, uint64_t round, const double *energy, double *kT,
                      int32_t *replica_of, int32_t *position_of, int32_t *n_accept, cudaStream_t st) {
  pt_exchange_kernel<<<1, 32, 0, st>>>(n, direction, seed, round, energy, kT, replica_of, position_of, n_accept);
  return cudaGetLastError();
}

}  // namespace cemc
