/* CPU oracle of the cluster-expansion MC hot path -- TEST INFRASTRUCTURE ONLY.
 * See ce_oracle.c for what each function restates. */
#ifndef CE_ORACLE_H
#define CE_ORACLE_H
#include <stdint.h>

#include "../include/cemc_gb300.h"

#define ORC_MAX_SYM 8
#define ORC_MOVE_FLIP 0
#define ORC_MOVE_SWAP 1
#define ORC_ERR_ARG 1
#define ORC_ERR_BACKGROUND 3
#define ORC_ERR_STATE 4
#define ORC_ERR_NO_MOVE 8 /* no legal trial move within max_attempts redraws */

/* Reference-shaped model: per-cluster members/order lists and equivalent
 * decorations, as CEUpdater holds them (cpp/include/cluster.hpp:14-54). */
typedef struct {
  int32_t n_sites, n_cols, n_sym, n_bf, n_eci, n_types, n_groups, n_movable;
  const int32_t *table;       /* [n_sites * n_cols] */
  const int32_t *site_group;  /* [n_sites] translation-symmetry group, -1 = background */
  const int32_t *group_count; /* [n_groups] sites per group */
  const int32_t *movable;     /* [n_movable] non-background sites */
  const double *bf;           /* [n_bf * n_sym] */
  const int32_t *type_size;   /* [n_types] */
  const int32_t *type_m;      /* [n_types * n_groups] sub-clusters in each group */
  const int32_t *type_M;      /* [n_types] sub-clusters summed over groups */
  const int32_t *type_off;    /* [n_types * n_groups] first sub-cluster row */
  const int32_t *members;     /* [rows * 3] neighbour columns */
  const int32_t *order;       /* [rows * 4] canonical order */
  const int32_t *eci_kind;    /* [n_eci] 0 c0, 1 singlet, 2 cluster */
  const int32_t *eci_type;    /* [n_eci] decoration (singlet) or type (cluster) */
  const int32_t *eq_off;      /* [n_eci + 1] */
  const int32_t *eq_decos;    /* [total * 4] */
  const int32_t *singlet_eci; /* [n_bf] ECI index of c1_b */
} orc_model;

typedef struct {
  int8_t *occ;
  double *cf;
  const double *eci;
  double kT;
  double *energy;
  cemc_accum *acc;
  int32_t *trk, *loc;
  const int32_t *trk_start, *trk_count;
  /* Move constraints (mc_constraints.py, redraw loop montecarlo.py:976-988): a change (site,
   * old, new) is legal when old is not in `frozen` and new is allowed at the site
   * (allow[site] bit new; allow NULL = every species).  max_attempts 0 = 10000. */
  const uint8_t *allow;
  uint32_t frozen;
  int32_t max_attempts;
  int32_t accept_first; /* 1: the run's first trial is accepted outright (montecarlo.py:932-935) */
  int32_t recycle;      /* 1: waste recycling (montecarlo.py:937-948, mc_observers.py:231-258) */
} orc_chain;

typedef struct {
  int32_t *site; /* [2 * n] site a, then site b (swap) or the new species (flip) */
  int8_t *acc;   /* [n] */
  double *de;    /* [n] */
  double *u;     /* [n] */
} orc_trace;

double orc_energy(const orc_model *m, const double *eci, const double *cf);
int orc_update_cf(const orc_model *m, const int8_t *occ, int site, int new_id, const double *cf_in, double *cf_out);
void orc_full_cf(const orc_model *m, const int8_t *occ, double *cf_out);
void orc_tracker_init(const orc_model *m, const int8_t *occ, int32_t *trk, int32_t *loc, int32_t *start,
                      int32_t *count);
int orc_run_chain(const orc_model *m, orc_chain *c, int move, uint64_t seed, uint32_t chain_id, uint64_t t_begin,
                  uint64_t n_trials, orc_trace *trace);
int orc_run_many(const orc_model *m, orc_chain *chains, int n_chains, const uint32_t *chain_ids, int move,
                 uint64_t seed, uint64_t t_begin, uint64_t n_trials, int n_threads);
#endif
