/*
 * CPU oracle for the pansim_gb300 hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of khbence/pansim's per-timestep agent loop, used by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker.  The product never links or calls it.  Each function cites the
 * reference file:line it follows.  Parity is pinned against the reference's
 * own C++ compiled from its sources (oracle/ref_harness), see tests.
 *
 * It operates in place on host arrays laid out exactly like the C ABI's
 * snapshot structs (include/pansim_gb300.h).
 */
#ifndef PSIM_ORACLE_H
#define PSIM_ORACLE_H
#include "../include/pansim_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct psim_oracle psim_oracle;

typedef psim_replicas psim_oracle_replicas;

psim_oracle* psim_oracle_create(const psim_model* m, psim_agents* a, psim_locations* l,
                                const psim_params* p, const psim_oracle_replicas* reps);
void psim_oracle_destroy(psim_oracle* o);
void psim_oracle_set_params(psim_oracle* o, const psim_params* p);

/* one phase each */
void psim_oracle_movement(psim_oracle* o, uint32_t t);
void psim_oracle_regroup(psim_oracle* o);
/* infection; hazard_f [L] (float r_l), sum_fix [L] (2^-40 fixed point),
 * sum64 [L] (FP64 sequential sum), r64 [L] (FP64 hazard, expm1), p64 [N]
 * (FP64 probability) — any may be NULL.  Returns the expected infections
 * (sum of min(1,p)) per replica into exp_out [R] (may be NULL). */
void psim_oracle_infect(psim_oracle* o, uint32_t t, uint32_t variant, float* hazard_f, int64_t* sum_fix,
                        double* sum64, double* r64, double* p64, double* exp_out);
void psim_oracle_step(psim_oracle* o, uint32_t t, const uint32_t* variant_active);
void psim_oracle_test(psim_oracle* o, uint32_t t, uint32_t* tpp /* [R*3] */);
void psim_oracle_progress(psim_oracle* o, uint32_t t);
void psim_oracle_stats(psim_oracle* o, uint32_t t, psim_day_stats* out /* [R] */);
void psim_oracle_plan(psim_oracle* o, uint32_t t);
void psim_oracle_midnight(psim_oracle* o, uint32_t t, psim_day_stats* out /* [R] */);
void psim_oracle_run_day(psim_oracle* o, uint32_t day, psim_day_stats* out /* [R] */);
/* closure rule ExposeToMutation: infect with variant v at timestamp t */
void psim_oracle_expose(psim_oracle* o, uint32_t t, uint32_t v, double fraction);
/* host threads of the parallel loops (OpenMP) */
int psim_oracle_threads(void);
/* immunization: categories (init), Immunization::update (immunize; returns immunizedToday) */
void psim_oracle_immunization_init(psim_oracle* o, const psim_immunization* imm);
uint32_t psim_oracle_immunize(psim_oracle* o, uint32_t t);
/* Simulation::otherDisease: options (NULL or enabled 0 = off) and the pass at midnight t */
void psim_oracle_other_disease_init(psim_oracle* o, const psim_other_disease* od);
void psim_oracle_other_disease(psim_oracle* o, uint32_t t);

/* CSR access */
const uint32_t* psim_oracle_csr_offsets(psim_oracle* o);
const uint32_t* psim_oracle_csr_agents(psim_oracle* o);

/* Philox self-check helper: raw block */
void psim_oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double psim_oracle_one_minus_exp(double x);
float psim_oracle_one_minus_expf(float x);
/* seasonality multiplier of infectionPolicies.h:443-478 */
double psim_oracle_seasonality(const psim_params* p, uint32_t t, uint32_t steps_per_day);

#ifdef __cplusplus
}
#endif
#endif
