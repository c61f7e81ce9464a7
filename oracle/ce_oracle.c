/* CPU oracle of the cluster-expansion Monte Carlo hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C and FP64, the
 * reference's CE updater and Metropolis loop so that the GPU path can be
 * checked against it.  Only the tests, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py may load it; the product path never does.
 *
 * What it follows (reference paths relative to the CEMC project root):
 *   orc_update_cf      CEUpdater::update_cf            cpp/src/ce_updater.cpp:313-406
 *   spin_product       CEUpdater::spin_product_one_atom cpp/src/ce_updater.cpp:244-285
 *                      CEUpdater::sort_indices          cpp/src/ce_updater.cpp:981-994
 *   orc_energy         CEUpdater::get_energy + NamedArray::dot
 *                                                       cpp/src/ce_updater.cpp:236-242,
 *                                                       cpp/src/named_array.cpp:25-33
 *   orc_full_cf        the brute-force correlation functions the reference's
 *                      tests compare against (ase.clease CorrFunction.get_cf,
 *                      tests/test_CE_updater.py:40-59), restated from the
 *                      normalisation the increment implies
 *   orc_run_chain      Montecarlo._mc_step / _accept    cemc/mcmc/montecarlo.py:910-1038
 *                      SGCMonteCarlo._get_trial_move    cemc/mcmc/sgc_montecarlo.py:62-76
 *                      SwapMoveIndexTracker             cemc/mcmc/swap_move_index_tracker.py:22-74
 * Floating-point operations are issued in the reference's order and with its
 * integer/double conversions, so results are bit-identical to the compiled
 * reference on the same inputs (build with -ffp-contract=off).
 * Trial proposals and uniforms come from the counter-based stream of
 * cemc_gb300/csrc/philox.h instead of numpy's global Mersenne Twister, so
 * that the GPU path can replay exactly the same moves.
 */
#include "ce_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../cemc_gb300/csrc/philox.h"

double orc_energy(const orc_model *m, const double *eci, const double *cf) {
  double e = 0.0;
  for (int k = 0; k < m->n_eci; ++k) e += eci[k] * cf[k];
  return e * (double)(unsigned)m->n_sites;
}

static double spin_product(const orc_model *m, const int8_t *occ, int site, int t, int g, const int32_t *deco,
                           int ref_id) {
  const int size = m->type_size[t];
  const int msub = m->type_m[t * m->n_groups + g];
  const int off = m->type_off[t * m->n_groups + g];
  double sp = 0.0;
  for (int i = 0; i < msub; ++i) {
    const int sub = off + i;
    double sp_temp = 1.0;
    int indices[4], sorted[4];
    indices[0] = site;
    for (int j = 0; j < size - 1; ++j) indices[j + 1] = m->table[(size_t)site * m->n_cols + m->members[sub * 3 + j]];
    for (int j = 0; j < size; ++j) sorted[j] = indices[m->order[sub * 4 + j]];
    for (int j = 0; j < size; ++j) {
      const int id = (sorted[j] == site) ? ref_id : occ[sorted[j]];
      sp_temp *= m->bf[deco[j] * m->n_sym + id];
    }
    sp += sp_temp;
  }
  return sp;
}

int orc_update_cf(const orc_model *m, const int8_t *occ, int site, int new_id, const double *cf_in, double *cf_out) {
  const int old_id = occ[site];
  const int g = m->site_group[site];
  if (g < 0) return ORC_ERR_BACKGROUND;
  if (old_id == new_id) {
    if (cf_out != cf_in) memcpy(cf_out, cf_in, sizeof(double) * m->n_eci);
    return 0;
  }
  const double n_total = (double)(unsigned)m->n_sites;
  for (int k = 0; k < m->n_eci; ++k) {
    const int kind = m->eci_kind[k];
    if (kind == 0) {
      cf_out[k] = cf_in[k];
      continue;
    }
    if (kind == 1) {
      const int dec = m->eci_type[k];
      cf_out[k] = cf_in[k] + (m->bf[dec * m->n_sym + new_id] - m->bf[dec * m->n_sym + old_id]) / n_total;
      continue;
    }
    const int t = m->eci_type[k];
    if (m->type_m[t * m->n_groups + g] == 0) {
      cf_out[k] = cf_in[k];
      continue;
    }
    const unsigned size = (unsigned)m->type_size[t];
    double delta_sp = 0.0;
    const int e0 = m->eq_off[k], e1 = m->eq_off[k + 1];
    for (int e = e0; e < e1; ++e) {
      const int32_t *deco = m->eq_decos + (size_t)e * 4;
      const double sp_ref = spin_product(m, occ, site, t, g, deco, old_id);
      const double sp_new = spin_product(m, occ, site, t, g, deco, new_id);
      delta_sp += sp_new - sp_ref;
    }
    delta_sp *= ((double)size / (double)(size_t)(e1 - e0));
    delta_sp /= (double)(m->type_M[t] * m->group_count[g]);
    cf_out[k] = cf_in[k] + delta_sp;
  }
  return 0;
}

void orc_full_cf(const orc_model *m, const int8_t *occ, double *cf_out) {
  const int n = m->n_sites;
  for (int k = 0; k < m->n_eci; ++k) {
    const int kind = m->eci_kind[k];
    if (kind == 0) {
      cf_out[k] = 1.0;
      continue;
    }
    if (kind == 1) {
      const int dec = m->eci_type[k];
      double s = 0.0;
      for (int i = 0; i < n; ++i)
        if (m->site_group[i] >= 0) s += m->bf[dec * m->n_sym + occ[i]];
      cf_out[k] = s / (double)n;
      continue;
    }
    const int t = m->eci_type[k];
    const int size = m->type_size[t];
    const int e0 = m->eq_off[k], e1 = m->eq_off[k + 1];
    double s = 0.0;
    long long norm = 0;
    for (int g = 0; g < m->n_groups; ++g) norm += (long long)m->type_m[t * m->n_groups + g] * m->group_count[g];
    for (int i = 0; i < n; ++i) {
      const int g = m->site_group[i];
      if (g < 0) continue;
      const int msub = m->type_m[t * m->n_groups + g];
      const int off = m->type_off[t * m->n_groups + g];
      for (int e = e0; e < e1; ++e) {
        const int32_t *deco = m->eq_decos + (size_t)e * 4;
        for (int q = 0; q < msub; ++q) {
          const int sub = off + q;
          int idx[4];
          idx[0] = i;
          for (int j = 0; j < size - 1; ++j) idx[j + 1] = m->table[(size_t)i * m->n_cols + m->members[sub * 3 + j]];
          double p = 1.0;
          for (int j = 0; j < size; ++j) p *= m->bf[deco[j] * m->n_sym + occ[idx[m->order[sub * 4 + j]]]];
          s += p;
        }
      }
    }
    cf_out[k] = s / ((double)(e1 - e0) * (double)norm);
  }
}

void orc_tracker_init(const orc_model *m, const int8_t *occ, int32_t *trk, int32_t *loc, int32_t *start,
                      int32_t *count) {
  for (int s = 0; s < m->n_sym; ++s) count[s] = 0;
  for (int i = 0; i < m->n_sites; ++i)
    if (m->site_group[i] >= 0) count[occ[i]]++;
  int acc = 0;
  for (int s = 0; s < m->n_sym; ++s) {
    start[s] = acc;
    acc += count[s];
  }
  int fill[ORC_MAX_SYM] = {0};
  for (int i = 0; i < m->n_sites; ++i) {
    if (m->site_group[i] < 0) {
      loc[i] = -1;
      continue;
    }
    const int s = occ[i];
    trk[start[s] + fill[s]] = i;
    loc[i] = fill[s];
    fill[s]++;
  }
}

/* A change (site, old -> new) passes the constraints: FixedElement blocks a change whose
 * old symbol is the fixed element (mc_constraints.py:95-107 compares the change's old symbol;
 * its index field never equals a symbol), ConstrainElementByTag requires the new symbol to be
 * allowed at the site (187-190), FixEdgeLayers allows no change on a fixed site (156-164). */
static int change_legal(const orc_chain *c, int site, int old_s, int new_s) {
  if ((c->frozen >> old_s) & 1u) return 0;
  if (c->allow && !((c->allow[site] >> new_s) & 1u)) return 0;
  return 1;
}

/* Waste recycling (Frenkel 2004): every trial adds p0 x (value before) + p1 x (value of the
 * proposal), p1 = 1 / (1 + exp(dE / kT)); energies of the state before and of the proposed
 * state (montecarlo.py:805-809), singlets as the calculator reports them before and after the
 * step, i.e. unchanged after a rejection (mc_observers.py:231-258). */
static void accumulate_recycled(const orc_model *m, const double *cf_before, const double *cf_after, double e_before,
                                double e_prop, double p1, cemc_accum *acc) {
  if (!acc) return;
  const double p0 = 1.0 - p1;
  const double db = e_before - acc->e_ref, dp = e_prop - acc->e_ref;
  acc->sum_e += p0 * db + p1 * dp;
  acc->sum_e2 += p0 * db * db + p1 * dp * dp;
  for (int b = 0; b < m->n_bf; ++b) {
    const double sb = cf_before[m->singlet_eci[b]], sa = cf_after[m->singlet_eci[b]];
    acc->sum_s[b] += p0 * sb + p1 * sa;
    acc->sum_s2[b] += p0 * sb * sb + p1 * sa * sa;
    acc->sum_se[b] += p0 * sb * db + p1 * sa * dp;
  }
  acc->n_samples++;
}

static void accumulate(const orc_model *m, const double *cf, double e, cemc_accum *acc) {
  if (!acc) return;
  const double de = e - acc->e_ref;
  acc->sum_e += de;
  acc->sum_e2 += de * de;
  for (int b = 0; b < m->n_bf; ++b) {
    const double s = cf[m->singlet_eci[b]];
    acc->sum_s[b] += s;
    acc->sum_s2[b] += s * s;
    acc->sum_se[b] += s * de;
  }
  acc->n_samples++;
}

int orc_run_chain(const orc_model *m, orc_chain *c, int move, uint64_t seed, uint32_t chain_id, uint64_t t_begin,
                  uint64_t n_trials, orc_trace *trace) {
  const int n_eci = m->n_eci;
  double *next = (double *)malloc(sizeof(double) * n_eci);
  double *next2 = (double *)malloc(sizeof(double) * n_eci);
  double *cf_before = (double *)malloc(sizeof(double) * n_eci); /* waste recycling: singlets before a trial */
  if (!next || !next2 || !cf_before) {
    free(next);
    free(next2);
    free(cf_before);
    return ORC_ERR_ARG;
  }
  int present[ORC_MAX_SYM];
  int n_present = 0;
  if (move == ORC_MOVE_SWAP) {
    for (int s = 0; s < m->n_sym; ++s)
      if (c->trk_count[s] > 0) present[n_present++] = s;
    if (n_present < 2) {
      free(next);
      free(next2);
      free(cf_before);
      return ORC_ERR_STATE;
    }
  }
  double e_cur = *c->energy;
  int rc = 0;
  const int constrained = c->allow != NULL || c->frozen != 0;
  const int max_att = c->max_attempts > 0 ? c->max_attempts : 10000;
  for (uint64_t it = 0; it < n_trials; ++it) {
    const uint64_t t = t_begin + it;
    int a, b = -1, na, nb = -1;
    double u;
    double *cf_new;
    /* Proposal k of trial t uses counter streams 2k (and 2k + 1): an illegal proposal is
     * redrawn until one is legal or max_att redraws are spent; like the reference
     * (montecarlo.py:984-987), spending the last redraw ends the search in failure even if
     * that redraw is legal, and the trial is then rejected with status ORC_ERR_NO_MOVE. */
    int att = 0, no_move = 0;
    if (move == ORC_MOVE_FLIP) {
      int old;
      for (;;) {
        const cemc_u32x4 w = cemc_trial_draw(seed, chain_id, t, (uint32_t)(2 * att));
        a = m->movable[cemc_below(w.v[0], (uint32_t)m->n_movable)];
        old = c->occ[a];
        const int k = (int)cemc_below(w.v[1], (uint32_t)(m->n_sym - 1));
        na = k + (k >= old);
        u = cemc_u01_53(w.v[2], w.v[3]);
        if (!constrained || change_legal(c, a, old, na) || att == max_att) break;
        ++att;
      }
      no_move = constrained && att == max_att;
      orc_update_cf(m, c->occ, a, na, c->cf, next);
      cf_new = next;
    } else {
      int A, B;
      for (;;) {
        const cemc_u32x4 w = cemc_trial_draw(seed, chain_id, t, (uint32_t)(2 * att));
        const cemc_u32x4 x = cemc_trial_draw(seed, chain_id, t, (uint32_t)(2 * att + 1));
        const int ia = (int)cemc_below(w.v[0], (uint32_t)n_present);
        int ib = (int)cemc_below(w.v[1], (uint32_t)(n_present - 1));
        ib += (ib >= ia);
        A = present[ia];
        B = present[ib];
        const int ra = (int)cemc_below(w.v[2], (uint32_t)c->trk_count[A]);
        const int rb = (int)cemc_below(w.v[3], (uint32_t)c->trk_count[B]);
        a = c->trk[c->trk_start[A] + ra];
        b = c->trk[c->trk_start[B] + rb];
        u = cemc_u01_53(x.v[0], x.v[1]);
        if (!constrained || (change_legal(c, a, A, B) && change_legal(c, b, B, A)) || att == max_att) break;
        ++att;
      }
      no_move = constrained && att == max_att;
      na = B;
      nb = A;
      /* Two sequential single-site updates, the second seeing the first
       * already applied (ce_updater.cpp:845-853). */
      orc_update_cf(m, c->occ, a, B, c->cf, next);
      c->occ[a] = (int8_t)B;
      orc_update_cf(m, c->occ, b, A, next, next2);
      c->occ[a] = (int8_t)A;
      cf_new = next2;
    }
    const double e_new = orc_energy(m, c->eci, cf_new);
    int accept;
    if (no_move) {
      accept = 0;
      rc = ORC_ERR_NO_MOVE;
    } else if (c->accept_first && it == 0) {
      accept = 1;
    } else if (c->recycle) {
      /* the next state drawn from the weights of the current and the proposed state */
      accept = u > 1.0 / (1.0 + exp(-(e_new - e_cur) / c->kT));
    } else if (e_new < e_cur) {
      accept = 1;
    } else {
      const double prob = exp(-(e_new - e_cur) / c->kT);
      accept = (u <= prob);
    }
    const double e_before = e_cur;
    if (c->recycle) memcpy(cf_before, c->cf, sizeof(double) * n_eci);
    if (trace) {
      trace->site[2 * it] = a;
      trace->site[2 * it + 1] = (move == ORC_MOVE_FLIP) ? na : b;
      trace->acc[it] = (int8_t)accept;
      trace->de[it] = e_new - e_cur;
      trace->u[it] = u;
    }
    if (accept) {
      memcpy(c->cf, cf_new, sizeof(double) * n_eci);
      e_cur = e_new;
      if (move == ORC_MOVE_FLIP) {
        c->occ[a] = (int8_t)na;
      } else {
        const int A = nb, B = na;
        const int la = c->loc[a], lb = c->loc[b];
        c->occ[a] = (int8_t)B;
        c->occ[b] = (int8_t)A;
        c->trk[c->trk_start[A] + la] = b;
        c->loc[b] = la;
        c->trk[c->trk_start[B] + lb] = a;
        c->loc[a] = lb;
      }
      if (c->acc) c->acc->n_accept++;
    }
    if (c->recycle)
      accumulate_recycled(m, cf_before, c->cf, e_before, e_new, 1.0 / (1.0 + exp((e_new - e_before) / c->kT)),
                          c->acc);
    else
      accumulate(m, c->cf, e_cur, c->acc);
  }
  *c->energy = e_cur;
  free(next);
  free(next2);
  free(cf_before);
  return rc;
}

typedef struct {
  const orc_model *m;
  orc_chain *chains;
  int n_chains, move, stride, first;
  uint64_t seed, t_begin, n_trials;
  const uint32_t *chain_ids;
  int rc;
} worker_arg;

static void *worker(void *p) {
  worker_arg *w = (worker_arg *)p;
  for (int i = w->first; i < w->n_chains; i += w->stride) {
    const int r = orc_run_chain(w->m, &w->chains[i], w->move, w->seed, w->chain_ids ? w->chain_ids[i] : (uint32_t)i,
                                w->t_begin, w->n_trials, NULL);
    if (r) w->rc = r;
  }
  return NULL;
}

int orc_run_many(const orc_model *m, orc_chain *chains, int n_chains, const uint32_t *chain_ids, int move,
                 uint64_t seed, uint64_t t_begin, uint64_t n_trials, int n_threads) {
  if (n_threads < 1) n_threads = 1;
  if (n_threads > n_chains) n_threads = n_chains;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * n_threads);
  worker_arg *args = (worker_arg *)malloc(sizeof(worker_arg) * n_threads);
  int rc = 0;
  for (int i = 0; i < n_threads; ++i) {
    args[i] = (worker_arg){m, chains, n_chains, move, n_threads, i, seed, t_begin, n_trials, chain_ids, 0};
    pthread_create(&th[i], NULL, worker, &args[i]);
  }
  for (int i = 0; i < n_threads; ++i) {
    pthread_join(th[i], NULL);
    if (args[i].rc) rc = args[i].rc;
  }
  free(th);
  free(args);
  return rc;
}
