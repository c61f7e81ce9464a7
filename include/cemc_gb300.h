/* C ABI of the GB300 cluster-expansion Monte Carlo library (libcemc_gb300.so).
 *
 * Every entry point returns int status (0 = OK, never throws, never traps);
 * the message of the last failure on the calling thread is available from
 * cemc_last_error().  Device buffers are owned by the caller (PyTorch tensors
 * on the Python side) and passed as raw pointers plus a cudaStream_t (void*).
 * The only allocation the library makes is the device copy of a geometry's
 * tables in cemc_geometry_create().
 *
 * The entry points replace the reference's native CE updater,
 * cpp/include/ce_updater.hpp:47-213 (class CEUpdater), as bound by
 * cemc/cpp_ext/pyce_updater.pyx:5-60 (PyCEUpdater).  Each declaration names
 * the reference member it stands in for.
 */
#ifndef CEMC_GB300_H
#define CEMC_GB300_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CEMC_OK 0
#define CEMC_ERR_ARG 1        /* invalid argument (sizes, null pointers) */
#define CEMC_ERR_CUDA 2       /* a CUDA runtime call failed */
#define CEMC_ERR_BACKGROUND 3 /* attempted to move a background site (ce_updater.cpp:330-332) */
#define CEMC_ERR_STATE 4      /* move inconsistent with the current occupation (ce_updater.cpp:530-537) */
#define CEMC_ERR_LIMIT 5      /* a compiled-in limit was exceeded */
#define CEMC_ERR_TIMEOUT 6    /* a bounded device wait ran out */
#define CEMC_ERR_INTERNAL 7   /* a device-side consistency check failed (the chain's state was not written) */
#define CEMC_ERR_NO_MOVE 8    /* no trial move satisfying the move constraints within max_attempts draws
                                 (CanNotFindLegalMoveError, montecarlo.py:984-987) */

#define CEMC_MAX_BF 4         /* decorations per site (species - 1) */
#define CEMC_MAX_ECI 128      /* ECIs per cluster expansion */
#define CEMC_MAX_COLS 128     /* distinct neighbour columns per site */
#define CEMC_MAX_GROUPS 8     /* translation-symmetry groups */

/* Running sums a chain accumulates after every trial (accepted or not).
 * Energies are taken relative to e_ref to keep the squares well conditioned;
 * the reference keeps the same sums in Averager objects and SGCObserver
 * (cemc/mcmc/montecarlo.py:802-814, cemc/mcmc/mc_observers.py:222-271). */
typedef struct {
  double e_ref;                  /* energy offset of the sums below */
  double sum_e;                  /* sum of (E - e_ref) */
  double sum_e2;                 /* sum of (E - e_ref)^2 */
  double sum_s[CEMC_MAX_BF];     /* sum of singlet correlation functions */
  double sum_s2[CEMC_MAX_BF];    /* sum of squared singlets */
  double sum_se[CEMC_MAX_BF];    /* sum of singlet * (E - e_ref) */
  uint64_t n_samples;            /* trials accumulated */
  uint64_t n_accept;             /* accepted trials */
} cemc_accum;

/* Host description of one supercell geometry and cluster expansion.  All
 * arrays are host memory; cemc_geometry_create() copies them to the device.
 * Layout of the flattened cluster "terms" (one per sub-cluster and
 * equivalent decoration of a cluster ECI):
 *   term_eci[t]   ECI index the term contributes to
 *   term_ref[t]   decoration index applied to the changed site
 *   term_size[t]  cluster size (2..4)
 *   term_nb[t*3+j] packed (column * n_bf + decoration) of member j
 * Terms are sorted by ECI; eci_weight[k] = size / (|eq deco| * M_k * N_s)
 * is the reference's increment normalisation (ce_updater.cpp:400-402).
 *
 * Several translation-symmetry groups (the reference's trans_symm_group,
 * ce_updater.cpp:733-776): each group has its own terms, which sit in one
 * contiguous range sorted by ECI (group g owns terms [group_terms[g],
 * group_terms[g+1])), and its own columns: the table row of a site lists the
 * neighbours its group's terms name, in the group's column order (unused
 * trailing columns point at the site itself).  eci_weight holds the
 * normalisation of group 0; the cluster-ECI change of a site of group g is
 * multiplied by group_scale[g] = N_0 / N_g (1 when the groups have equal
 * sizes, as translation classes of a periodic supercell do). */
typedef struct {
  int32_t n_sites;        /* N, including background sites */
  int32_t n_cols;         /* neighbour columns per site */
  int32_t n_sym;          /* species */
  int32_t n_bf;           /* decorations = n_sym - 1 */
  int32_t n_eci;          /* ECIs, sorted-name order */
  int32_t n_terms;        /* flattened cluster terms */
  const int32_t *table;   /* [n_sites * n_cols] neighbour site of (site, column) */
  const double *bf;       /* [n_bf * n_sym] basis function values */
  const int32_t *eci_kind;   /* [n_eci] 0 = c0, 1 = singlet, 2 = cluster */
  const int32_t *eci_dec;    /* [n_eci] decoration of a singlet, else -1 */
  const double *eci_weight;  /* [n_eci] increment weight of cluster ECIs */
  const double *eci_full_weight; /* [n_eci] full-recompute weight (weight / size) */
  const int32_t *term_eci;   /* [n_terms] */
  const int32_t *term_ref;   /* [n_terms] */
  const int32_t *term_size;  /* [n_terms] */
  const int32_t *term_nb;    /* [n_terms * 3] */
  /* Sites that may change (not background, ce_updater.cpp:1015-1026), ascending; single-site
   * flips draw their site from this list and swap trackers hold only these sites; background
   * sites keep species id 0 in the occupations, belong to no cluster and are skipped by the
   * full recompute.  NULL (or n_movable == n_sites) = every site. */
  const int32_t *movable;
  int32_t n_movable;
  int32_t n_groups;            /* translation-symmetry groups; 0 or 1 = one group (the fields below unused) */
  const int32_t *site_group;   /* [n_sites] group of each site (background sites: ignored) */
  const int32_t *group_terms;  /* [n_groups + 1] term range of each group */
  const double *group_scale;   /* [n_groups] factor on a site's cluster-ECI change, N_0 / N_g */
} cemc_geometry_desc;

typedef struct cemc_geometry cemc_geometry;

/* Build the device-resident tables of one geometry (replaces the table
 * parsing in CEUpdater::init, ce_updater.cpp:32-234). */
int cemc_geometry_create(const cemc_geometry_desc *desc, cemc_geometry **out);
int cemc_geometry_destroy(cemc_geometry *geo);

/* Bytes of device memory the geometry's tables hold (the one allocation
 * cemc_geometry_create makes), for callers that budget device memory.  No
 * reference counterpart (the reference keeps its tables in host memory). */
size_t cemc_geometry_device_bytes(const cemc_geometry *geo);

/* Ensembles of a trial move. */
#define CEMC_MOVE_FLIP 0  /* semi-grand-canonical single-site flip (sgc_montecarlo.py:62-76) */
#define CEMC_MOVE_SWAP 1  /* canonical two-site swap (montecarlo.py:890-908) */

/* Precision of the trial-move energy change. */
#define CEMC_PREC_F64 0
#define CEMC_PREC_F32 1

/* Per-launch description of a batch of chains sharing one geometry.  All
 * pointers are device memory laid out chain-major.
 *   occ      [n_chains * n_sites] int8 species ids (sorted-symbol order)
 *   cf       [n_chains * n_eci]   FP64 correlation functions
 *   energy   [n_chains]           FP64 total energy N * sum(eci * cf)
 *   eci      [n_chains * n_eci]   FP64 ECIs (chemical potentials folded in)
 *   kT       [n_chains]           FP64 k_B * T in eV
 *   trial    [n_chains]           uint64 first trial index (RNG counter), advanced by n_trials
 *   accum    [n_chains]           running sums, may be NULL
 *   trk/loc  [n_chains * n_sites] per-species site lists of swap moves (NULL for flips)
 *   trk_start[n_chains * n_sym], trk_count [n_chains * n_sym] list extents (NULL for flips)
 * Optional per-trial trace (device, n_chains * n_trials entries, NULL = off):
 *   trace_site [.. * 2] int32 sites, trace_acc int8 decision, trace_de FP64 energy change. */
typedef struct {
  int32_t n_chains;
  int32_t move;        /* CEMC_MOVE_* */
  int32_t precision;   /* CEMC_PREC_* */
  int32_t warps;       /* evaluating warps per CTA, at most 16, larger values are clamped (trials per round =
                          warps x trials per warp x CTAs per chain); 0 = default */
  uint64_t seed;
  uint64_t n_trials;   /* trials per chain in this launch */
  int8_t *occ;
  double *cf;
  double *energy;
  const double *eci;
  const double *kT;
  uint64_t *trial;
  cemc_accum *accum;
  int32_t *trk;
  int32_t *loc;
  const int32_t *trk_start;
  const int32_t *trk_count;
  int32_t *trace_site;
  int8_t *trace_acc;
  double *trace_de;
  int32_t *status;     /* [n_chains] device status words, may be NULL */
  const uint32_t *chain_key; /* [n_chains] RNG key of each chain (device), NULL = chain index */
  const int32_t *accum_slot; /* [n_chains] row of `accum` each chain adds to (device), NULL = chain index;
                                lets a temperature ladder keep its sums per temperature */
  const uint64_t *chain_trials; /* [n_chains] trials of each chain in this launch (device, each <= n_trials),
                                   NULL = n_trials for every chain; lets a batch mix jobs with different budgets */
  int32_t kernel;      /* CEMC_KERNEL_*: which implementation runs the trials */
  int32_t cluster;     /* CTAs per chain: 1, 2 (a thread-block cluster pair on two SMs, twice the trials
                          per round), or 0 = 2 when every chain's pair fits on the GPU at once, else 1 */
  double *scratch;     /* table kernel: buffer for the final recompute, at least cemc_recompute_scratch_doubles()
                          doubles (a smaller buffer is refused with CEMC_ERR_ARG).  NULL = the fixed array
                          behind cemc_recompute_noalloc(), under the same rules: at most 1048576 doubles
                          (CEMC_ERR_LIMIT beyond), the first such call on a device looks up the array's
                          address and should come before any stream capture, and every call that uses
                          the array shares it, so such calls (and cemc_recompute_noalloc calls) that
                          overlap on the GPU race: order them on one stream. */
  uint64_t scratch_doubles;
  uint32_t *stamps;    /* optional device buffer for exact conflict tables of large supercells, used when
                          the shared-memory table would have to be hashed (hashing only costs speed):
                          cemc_stamp_words() words; NULL = shared memory only */
  uint64_t stamp_words;
  int32_t kernel_used; /* output: the CEMC_KERNEL_* form cemc_run launched (CEMC_KERNEL_TABLE: the call
                          already ended with a full recompute) */
  /* Move constraints (mc_constraints.py; redraw loop of montecarlo.py:976-988).  A change (site,
   * old, new) is legal when species `old` is not frozen and species `new` is allowed at `site`;
   * a move is legal when all its changes are.  An illegal proposal is redrawn (draw k of trial t
   * uses counter streams 2k, 2k+1) up to max_attempts times; when the redraws run out the trial
   * is rejected and the chain's status becomes CEMC_ERR_NO_MOVE.  All NULL = unconstrained. */
  const uint8_t *site_allow;    /* [n_chains * n_sites] bit s: species s may be placed on the site, or NULL */
  const uint32_t *frozen;       /* [n_chains] bit s: a site holding species s may not change, or NULL */
  int32_t max_attempts;         /* redraws per trial; 0 = 10000 (the reference's default) */
  int32_t accept_first;         /* 1: the first trial of this call is accepted whatever its energy change
                                   (accept_first_trial_move_after_reset, montecarlo.py:932-935) */
  int32_t recycle_waste;        /* 1: waste recycling (Frenkel 2004; montecarlo.py:937-948): accept when
                                   u > 1 / (1 + exp(-dE / kT)), and every trial adds p0 x (value before) +
                                   p1 x (value of the proposal) to the running sums; generic form, one CTA */
} cemc_run_desc;

/* Kernel selection of cemc_run.  AUTO takes the binary spin-basis form when
 * the geometry allows it (two species with basis values +1 and -1, at most 64
 * neighbour columns, at most 32 cluster ECIs) — the half-warp spin form for
 * single-site flips with at most 16 cluster ECIs when no CTA pair is asked
 * for — else the table form when its tables fit, else the generic form.  All
 * give the same decisions for the same stream.  The spin forms evaluate a
 * trial from a bit-packed neighbourhood (popcounts of shell masks, parities of
 * multi-site terms), one trial per warp or one per 16 lanes; the generic form
 * multiplies basis values term by term and keeps the correlation functions up
 * to date trial by trial; the table form looks up one precomputed energy change
 * per cluster geometry (tables built per chain from its ECIs at launch) and
 * brings correlation functions and energies up to date with a full recompute
 * at the end of the call (run desc `scratch`). */
#define CEMC_KERNEL_AUTO 0
#define CEMC_KERNEL_GENERIC 1
#define CEMC_KERNEL_SPIN 2
#define CEMC_KERNEL_SPIN_HALFWARP 3  /* spin basis, flips only, two trials per warp (one per 16 lanes) */
#define CEMC_KERNEL_TABLE 4  /* one table lookup per cluster geometry; CFs and energies by a final recompute */
#define CEMC_KERNEL_FIELD 5  /* local field: spin basis, unconstrained flips of a periodic one-group supercell;
                                every site keeps its per-ECI odd-term counts in shared memory, a trial reads
                                them (one lane per trial) and an accepted flip updates its neighbours' counts */
#define CEMC_KERNEL_SPIN_QUARTER 6  /* spin basis, flips only, four trials per warp (one per 8 lanes), at most 8
                                       cluster ECIs, one CTA per chain */

/* Run n_trials Metropolis trials on every chain in one launch: trial-move
 * energy change, accept test and in-place commit of occupation, correlation
 * functions and energy (replaces the Montecarlo._mc_step loop,
 * montecarlo.py:970-1038, over CEUpdater::calculate / undo_changes /
 * clear_history, ce_updater.cpp:313-555). */
int cemc_run(const cemc_geometry *geo, cemc_run_desc *run, void *stream);

/* Words of a cemc_run_desc.stamps buffer for n_chains chains of this geometry:
 * two exact tables of 2^ceil(log2 N) entries per chain.  No reference counterpart
 * (the reference evaluates one trial at a time and needs no conflict test). */
size_t cemc_stamp_words(const cemc_geometry *geo, int32_t n_chains);

/* Full correlation-function recompute over all sites of every chain, used for
 * validation and to reset FP64 drift; also rewrites energy = N * eci . cf.
 * The reference obtains these from ase.clease CorrFunction.get_cf
 * (cemc/ce_calculator.py:169-177).  scratch: device FP64 buffer of
 * cemc_recompute_scratch_doubles() entries. */
size_t cemc_recompute_scratch_doubles(const cemc_geometry *geo, int32_t n_chains);
int cemc_recompute(const cemc_geometry *geo, int32_t n_chains, const int8_t *occ, const double *eci,
                   double *cf, double *energy, double *scratch, void *stream);

/* Full recompute that allocates nothing (no reference counterpart: the
 * reference computes correlation functions on the host).  Same results as
 * cemc_recompute(), but its scratch is a fixed array inside the library
 * instead of a caller buffer, for callers that cannot allocate device memory
 * when they call it -- for example a process that has already handed its
 * whole device-memory budget to a pre-reserved pool, or a latency-critical
 * path where cudaMalloc's implicit device synchronisation is not acceptable.
 * Limit: recompute_blocks * n_chains * n_eci <= 1048576 scratch doubles
 * (8 MiB, held on every GPU that loads the library until exit); larger
 * requests return CEMC_ERR_LIMIT without launching anything, where
 * recompute_blocks = ceil(n_sites / 256).  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture.  All calls share the one array, so
 * calls that overlap on the GPU (other streams, other threads) race: order
 * them on one stream or synchronise between them.  The array's address is
 * cached per device ordinal for the life of the process, so the library must
 * not be used on a device again after cudaDeviceReset() there.  It never calls
 * cudaMalloc, cudaFree or an allocating library routine. */
int cemc_recompute_noalloc(const cemc_geometry *geo, int32_t n_chains, const int8_t *occ, const double *eci,
                           double *cf, double *energy, void *stream);

/* Energy N * sum_k eci[k] * cf[k] of every chain, summed in sorted-name order
 * (CEUpdater::get_energy + NamedArray::dot, ce_updater.cpp:236-242,
 * named_array.cpp:25-33).  Device pointers. */
int cemc_energy(const cemc_geometry *geo, int32_t n_chains, const double *eci, const double *cf, double *energy,
                void *stream);

/* Apply an explicit list of single-site changes in sequence to one chain
 * (CEUpdater::calculate / update_cf, ce_updater.cpp:313-406, 471-519, 845-853):
 * sites[i] takes species new_sym[i]; cf and energy are updated in place.
 * old_sym[i] must match the current species or CEMC_ERR_STATE is returned
 * through *status.  Device pointers; status is a device int32. */
int cemc_apply_changes(const cemc_geometry *geo, int8_t *occ, double *cf, double *energy, const double *eci,
                       int32_t n_changes, const int32_t *sites, const int8_t *old_sym, const int8_t *new_sym,
                       int32_t *status, void *stream);

/* Energy change of a single flip or a swap without committing it (the
 * replay / debug path).  move: CEMC_MOVE_FLIP uses (site_a, new_a);
 * CEMC_MOVE_SWAP exchanges the species of site_a and site_b.  Writes the
 * FP64 energy change and the correlation-function change (n_eci) to device
 * memory. */
int cemc_delta_e(const cemc_geometry *geo, const int8_t *occ, const double *eci, int32_t move, int32_t site_a,
                 int32_t site_b, int32_t new_a, double *de_out, double *dcf_out, void *stream);

/* Replica exchange over a ladder of chains (ParallelTempering
 * _perform_exchange_move, cemc/mcmc/parallel_tempering.py:138-175): pairs
 * (i, i+1) of ladder positions starting at parity `direction`, accepted when
 * u < exp((1/kT_i - 1/kT_j)(E_i - E_j)).  Temperatures are exchanged, not
 * configurations: replica_of[pos] names the chain at ladder position pos and
 * is permuted in place; kT[chain] is rewritten accordingly, and position_of
 * (may be NULL) receives the inverse permutation, position_of[chain] = pos. */
int cemc_pt_exchange(int32_t n_replicas, int32_t direction, uint64_t seed, uint64_t round,
                     const double *energy, double *kT, int32_t *replica_of, int32_t *position_of, int32_t *n_accept,
                     void *stream);

/* Message of the last failure on this thread. */
int cemc_last_error(char *buf, size_t len);

/* Library version and the compute capability it was compiled for. */
int cemc_version(int32_t *major, int32_t *minor, int32_t *sm);

#ifdef __cplusplus
}
#endif
#endif
