/*
 * pansim_gb300 — C ABI of the GB300-native PanSim per-timestep agent loop.
 *
 * The library replaces the reference's per-step and per-day device work
 * (khbence/pansim):
 *   movement        RealMovement::movement        include/policies/movementPolicies.h:1625-1751
 *                   RealMovementOps::doMovement   include/policies/movementPolicies.h:263-1041
 *   regrouping      Util::updatePerLocationAgentLists  src/tools/util.cpp:55-108
 *   infection       BasicInfection::infectionsAtLocations include/policies/infectionPolicies.h:481-588
 *                   LocationsList::infectAgents   include/locationList.h:233-310
 *   progression     Simulation::updateAgents      include/simulation.h:425-471
 *                   DynamicPPState::update        src/agentData/dynamicPPState.cpp:246-303
 *   daily plan      RealMovement::planLocations   include/policies/movementPolicies.h:1428-1622
 *   testing         DetailedTesting::performTests include/policies/testingPolicies.h:370-475
 *   statistics      Simulation::refreshAndPrintStatistics include/simulation.h:473-665
 *   step loop       Simulation::runSimulation     include/simulation.h:899-926
 *
 * Every entry point returns 0 on success and a negative psim_status on
 * failure; psim_last_error() gives a message.  Only plain pointers, sizes and
 * POD structs cross the boundary.  Host pointers in psim_snapshot are read by
 * psim_upload and written by psim_download; device memory is owned by the
 * context.  All work of a context is issued on its own CUDA stream.
 */
#ifndef PANSIM_GB300_H
#define PANSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PSIM_MAX_STRAINS 7   /* MAX_STRAINS, include/datatypes.h:17 */
#define PSIM_MAX_BANDS 16
#define PSIM_NO_LOCATION 0xFFFFFFFFu

typedef enum psim_status {
    PSIM_OK = 0,
    PSIM_ERR_ARG = -1,        /* invalid argument or inconsistent snapshot */
    PSIM_ERR_CUDA = -2,       /* a CUDA call failed */
    PSIM_ERR_ALLOC = -3,      /* device allocation failed */
    PSIM_ERR_RANGE = -4,      /* out-of-range index found in the snapshot */
    PSIM_ERR_DEVICE = -5,     /* a kernel reported an error (bounded wait expired) */
    PSIM_ERR_STATE = -6       /* call out of order (e.g. step before upload) */
} psim_status;

/* Model tables (immutable during a run).  Progression tables follow
 * MultiBadMatrix (src/tools/progressionMatrices/multiBadMatrix.cpp:43-83) and
 * LengthOfState (src/tools/progressionMatrices/basicLengthAbstract.cpp:31-53). */
typedef struct psim_model {
    uint32_t n_states;
    uint32_t n_variants;            /* active strains, <= PSIM_MAX_STRAINS */
    uint32_t n_prog;                /* progression tables (age band x pre-condition) */
    uint32_t n_agent_types;
    uint32_t n_trans;               /* total transition entries */
    uint32_t n_events;              /* total schedule events */
    uint32_t first_infected_state;  /* DynamicPPState::gotInfected */
    uint32_t noncovid_dead_state;
    uint32_t dead_state;            /* first state with WB == D */
    uint32_t pad0;
    /* per state [n_states] */
    const uint8_t* state_wb;        /* states::WBStates: W=0 N=1 M=2 S=3 D=4 */
    const float* state_infectious;
    const uint8_t* state_susceptible;
    const uint8_t* state_infected;
    const float* state_acc_pcr;
    const float* state_acc_antigen;
    /* per variant [n_variants] */
    const float* variant_multiplier;  /* --infectiousnessMultiplier */
    const float* prog_scaling;        /* --diseaseProgressionScaling */
    const float* death_scaling;       /* --diseaseProgressionDeathScaling */
    /* progression tables, index (prog * n_states + state) */
    const uint32_t* tr_bad_begin;
    const uint32_t* tr_bad_count;
    const uint32_t* tr_neu_begin;
    const uint32_t* tr_neu_count;
    const uint32_t* tr_next;          /* [n_trans] */
    const float* tr_chance;           /* [n_trans] */
    /* dwell lengths, index ((prog * n_states + state) * PSIM_MAX_STRAINS + variant) */
    const float* len_avg;
    const float* len_max;
    const double* len_p;              /* geometric p after calculateModifiedP */
    /* schedules: AgentTypeList (include/agentData/agentType.h:10-45) */
    const uint32_t* event_offset;     /* [n_agent_types * 28 + 1] */
    const uint32_t* ev_loc_type;      /* [n_events] */
    const float* ev_chance;
    const uint16_t* ev_start;         /* minutes of day, TimeDay semantics */
    const uint16_t* ev_end;
    const uint16_t* ev_duration;      /* minutes; >= 25*60 means "until midnight" */
} psim_model;

/* Agent state, structure of arrays [n_agents] unless noted. */
typedef struct psim_agents {
    uint32_t n;
    uint32_t n_poss;                  /* entries of the per-agent location CSR */
    /* immutable */
    const uint8_t* type;              /* agent type index */
    const uint8_t* age;
    const uint8_t* band;              /* age band for the band susceptibility */
    const uint16_t* prog_id;          /* progression table index */
    const float* symptom_scaling;     /* BasicAgentMeta::getScalingSymptoms */
    const uint32_t* loc_offset;       /* [n+1] per-agent location CSR */
    const uint32_t* poss_loc;         /* [n_poss] */
    const uint8_t* poss_type;         /* [n_poss] location type of each entry */
    /* mutable */
    uint32_t* location;
    uint32_t* steps_until_move;
    int8_t* state;
    int16_t* days;                    /* daysBeforeNextState */
    uint8_t* variant;
    float* infectious;
    float* susceptible;               /* [n_variants * n], variant-major */
    uint8_t* diagnosed;
    uint8_t* quarantined;
    uint8_t* stayed_home;
    uint8_t* no_work;
    uint32_t* last_test;              /* DetailedTesting::lastTest */
    /* AgentStats (include/agentData/agentStats.h:5-22) */
    uint32_t* st_infected_ts;
    uint32_t* st_infected_loc;
    uint32_t* st_worst_ts;
    uint32_t* st_worst_end_ts;
    uint32_t* st_diagnosed_ts;
    uint32_t* st_quarantined_ts;
    uint32_t* st_quarantined_until;
    uint32_t* st_days_in_quarantine;
    uint32_t* st_hospitalized_ts;
    uint32_t* st_hospitalized_until;
    uint32_t* st_immunization_ts;
    uint32_t* st_recovered_ts;
    uint32_t* st_variant_mask;
    uint8_t* st_immunization_count;
    uint8_t* st_infected_count;
    int8_t* st_worst_state;
    /* immunization (include/immunization.h); each may be NULL */
    const uint8_t* precond;           /* BasicAgentMeta::preCondIdx; NULL = 0 */
    uint8_t* imm_round;               /* Immunization::immunizationRound; NULL = 0 */
    float* symptom_scaling_v;         /* [n_variants * n], variant-major: BasicAgentMeta::scalingSymptoms
                                         of the states up to 6 (agentMeta.cpp:83-84), which the
                                         immunization rescales; NULL = symptom_scaling */
    const uint8_t* sex;               /* BasicAgentMeta::sex: 0 = F, 1 = M (agentMeta.cpp:53-60); NULL = 0 */
} psim_agents;

/* Locations (include/locationList.h:46-67) [n_locations], cemetery last. */
typedef struct psim_locations {
    uint32_t n;                       /* at most 2^30 - 2 */
    uint32_t n_schools;
    uint32_t n_classrooms;
    uint32_t pad0;
    const uint8_t* type;
    float* infectiousness;            /* w_l, multiplied by closure masks */
    uint8_t* open;                    /* LocationsList::states */
    const uint8_t* essential;
    uint32_t* closed_until;
    uint32_t* quarantine_until;
    const uint32_t* schools;          /* [n_schools] */
    const uint32_t* classrooms;       /* [n_classrooms] */
    const uint32_t* classroom_offsets;/* [n_schools + 1] */
} psim_locations;

/* Run parameters.  Policies may change the mutable ones between days. */
typedef struct psim_params {
    uint32_t time_step;               /* minutes (--deltat) */
    uint32_t start_day;               /* weekday of day 0, Monday = 0 (--startDay) */
    uint32_t start_date;              /* day of year of day 0 (--startDate) */
    uint32_t home_type, work_type, school_type, classroom_type;
    uint32_t hospital_type, doctor_type, public_type, nursery_type;
    uint32_t cemetery_loc;
    uint32_t quarantine_policy;       /* --quarantinePolicy */
    uint32_t quarantine_length;       /* days, --quarantineLength */
    uint32_t enable_curfew;
    uint32_t curfew_begin;            /* in steps of the day */
    uint32_t curfew_end;              /* in steps of the day */
    uint32_t school_age_restriction;
    uint32_t holiday_mode;
    uint32_t quarantine_immune;
    uint32_t lockdown_nonvacc;
    uint32_t testing_enabled;         /* DetailedTesting (1) or NoTesting (0) */
    uint32_t testing_delay;           /* --testingRepeatDelay */
    uint32_t use_pcr;
    uint32_t n_bands;
    uint32_t tracked;                 /* unused on the device */
    uint32_t pad0;
    double k;                         /* --infectionCoefficient */
    double c0, trunc;                 /* seasonality, infectionPolicies.h:443-478 */
    int32_t d_offset0, d_offset1, d_peak_offset, n_d_offset;
    double t_random, t_home, t_work, t_school, t_hospital, t_nursery;
    uint64_t seed;                    /* Philox key */
    float sigma_band[PSIM_MAX_BANDS]; /* age-band susceptibility, 1 = reference */
} psim_params;

/* Replicas batched in one context (ensembles of uneven populations).  Agents and
 * locations of replica r occupy [agent_offset[r], agent_offset[r+1]) and
 * [loc_offset[r], loc_offset[r+1]); location indices in the snapshot are
 * global.  Each replica has its own Philox key and infection coefficient;
 * draws are addressed by the agent's index inside its replica, so a replica
 * gives the same trajectory alone or in a batch.  NULL = one replica made of
 * the whole snapshot with params->seed, params->k and params->cemetery_loc. */
typedef struct psim_replicas {
    uint32_t n;
    uint32_t pad0;
    const uint32_t* agent_offset;   /* [n+1] */
    const uint32_t* loc_offset;     /* [n+1] */
    const uint64_t* seed;           /* [n] */
    const double* k;                /* [n] */
    const uint32_t* cemetery;       /* [n] */
} psim_replicas;

/* Per-day statistics row, the reference's TSV row (simulation.h:473-665). */
#define PSIM_STATS_MAX 64
typedef struct psim_day_stats {
    uint32_t n;                        /* entries used in v */
    uint32_t new_infections;           /* NI */
    uint32_t v[PSIM_STATS_MAX];
    uint32_t variant_counts[PSIM_MAX_STRAINS]; /* infected per variant (countVariantCases) */
    double expected_new_infections;    /* sum of infection probabilities since the last midnight */
} psim_day_stats;

/* Launch and algorithm choices of the per-step kernels, picked per device
 * and workload by the autotuner (pansim_gb300/autotune.py).  A new context
 * starts with agg_slot 0, blocks_per_sm 4, scan_items 4, scan_mode 3. */
typedef struct psim_tuning {
    uint32_t agg_count;      /* no effect (the histogram is updated by movers only) */
    uint32_t agg_slot;       /* warp-aggregated agent-list slot atomics */
    uint32_t blocks_per_sm;  /* 256-thread blocks per SM of the step kernel; 0 = occupancy */
    uint32_t variant;        /* the day graph's step kernel (agent list rebuilt at the steps
                                where agents took new locations, draws over the agents at
                                locations with an infectious agent, decisions of the agents
                                whose decision step it is): 3 = one launch per timestep,
                                4 = one launch for the whole day with a grid barrier between
                                timesteps (slower on GB300 at 2M and 20M agents) */
    uint32_t scan_items;     /* locations per thread of the scan: 2, 4 or 8 (0 = 8) */
    uint32_t scan_mode;      /* 0 = single pass with decoupled look-back, 1 = tile sums + scan,
                                2 = tile sums + scan with each thread owning consecutive
                                locations (scan_items 4 or 8; with 2 it falls back to 1),
                                3 = single pass with look-back, consecutive locations per
                                thread (scan_items 4 or 8; with 2 it falls back to 0) */
} psim_tuning;

typedef struct psim_ctx psim_ctx;

/* Library */
const char* psim_version(void);
/* sizeof of the ABI structs in the order model, agents, locations, params,
 * replicas, day_stats: lets bindings verify their mirrors. */
int psim_abi_sizes(uint64_t* out, int n);
int psim_device_count(int* out);

/* Context: allocates device storage for the snapshot's sizes on device `device`. */
int psim_create(int device, const psim_model* model, const psim_agents* agents,
                const psim_locations* locs, const psim_params* params,
                const psim_replicas* replicas, psim_ctx** out);
int psim_destroy(psim_ctx* ctx);
const char* psim_last_error(const psim_ctx* ctx);

/* State transfer: host SoA <-> device SoA (all mutable arrays). */
int psim_upload(psim_ctx* ctx, const psim_agents* agents, const psim_locations* locs);
/* The byte offsets (offsets[n_fields] = the total) of the mutable state that
 * psim_upload and psim_download move, for n agents, locations and variants,
 * in this order: the agents' location, steps_until_move, state, days,
 * variant, infectious, susceptible, diagnosed, quarantined, stayed_home,
 * no_work, last_test, st_infected_ts, st_infected_loc, st_worst_ts,
 * st_worst_end_ts, st_diagnosed_ts, st_quarantined_ts, st_quarantined_until,
 * st_days_in_quarantine, st_hospitalized_ts, st_hospitalized_until,
 * st_immunization_ts, st_recovered_ts, st_variant_mask,
 * st_immunization_count, st_infected_count, st_worst_state, imm_round,
 * symptom_scaling_v, then the locations' infectiousness, open, closed_until,
 * quarantine_until (34 fields, each at a 256-byte aligned offset).  Host
 * arrays laid out this way from agents->location on (pinned memory: one
 * block) move in one copy each way. */
int psim_state_layout(uint32_t n_agents, uint32_t n_locations, uint32_t n_variants, uint64_t* offsets,
                      uint32_t* n_fields);
int psim_download(psim_ctx* ctx, psim_agents* agents, psim_locations* locs);
int psim_set_params(psim_ctx* ctx, const psim_params* params);

/* Per-step phases (runSimulation, simulation.h:918-922). t = timestamp. */
int psim_movement(psim_ctx* ctx, uint32_t t);          /* doMovement for all agents */
int psim_regroup(psim_ctx* ctx);                        /* CSR of agents by location */
int psim_infect(psim_ctx* ctx, uint32_t t, uint32_t variant); /* fused reduce + draw */
int psim_step(psim_ctx* ctx, uint32_t t);              /* movement + regroup + infection of active variants */

/* Midnight phases (simulation.h:906-917). */
int psim_test_day(psim_ctx* ctx, uint32_t t, uint32_t* out_tpp /* [replicas*3] or NULL */);
int psim_progress_day(psim_ctx* ctx, uint32_t t);
int psim_stats_day(psim_ctx* ctx, uint32_t t, psim_day_stats* out /* [replicas] */);
int psim_plan_day(psim_ctx* ctx, uint32_t t);
/* test (t > 0) -> progress (t > 0) -> statistics -> closure rules (when set)
 * -> plan, the midnight block of runSimulation. */
int psim_midnight(psim_ctx* ctx, uint32_t t, psim_day_stats* out /* [replicas] */);

/* Closure rules: RuleClosure (closurePolicies.h:48-479) with the rule list of
 * closureRules.json (closuresFormat.h:7-22).  Rule names Masks, Curfew,
 * HolidayMode, QuarantineImmune, LockdownNonvacc, QuarantinePolicy,
 * SchoolAgeRestriction, ExposeToMutation, ReduceMovement and TestingProb act
 * on the named policy switch; any other name closes its location types.
 * Condition types: afterDays, hospitalizedFraction, newDeadFraction
 * (closurePolicies.h:109-232) and newCasesFraction, which has no reference
 * counterpart: the fraction of the population newly infected in the last
 * 24 h (the NI column), with hospitalizedFraction's close/open hysteresis.
 * `header` is the statistics header (state names, then H, T, P1, ...; the
 * statesHeader of simulation.h:749); hospital states are the columns whose
 * name contains "_h", the dead column is "D1".  With enable_closures == 0
 * only the named switches are kept (closurePolicies.h:103-108).  Rules are
 * evaluated by psim_midnight after the statistics, on the row of replica 0;
 * contexts with more than one replica reject rules.  n_rules == 0 removes
 * the rules. */
#define PSIM_CLOSURE_MAX_TYPES 10
typedef struct psim_closure_rule {
    char name[64];
    char condition_type[32];
    double threshold;
    double threshold2;
    char parameter[64];               /* the rule's parameter as text ("0.8", "2000-0500", ...) */
    int32_t close_after;
    int32_t open_after;
    uint32_t n_types;                 /* entries of types, < PSIM_CLOSURE_MAX_TYPES */
    int32_t types[PSIM_CLOSURE_MAX_TYPES]; /* locationTypesToClose */
} psim_closure_rule;
int psim_closures_init(psim_ctx* ctx, const psim_closure_rule* rules, uint32_t n_rules, const char* header,
                       int enable_closures);
/* Evaluates the rules on a statistics row (what psim_midnight does after its
 * statistics); `t` is the midnight timestamp. */
int psim_closures_midnight(psim_ctx* ctx, uint32_t t, const psim_day_stats* row);
/* State of the engine: per condition its active flag, per rule whether its
 * locations/switch are open (previousOpenState); either pointer may be NULL. */
int psim_closures_status(psim_ctx* ctx, uint8_t* cond_active /* [n_rules] */, uint8_t* rule_open /* [n_rules] */,
                         uint32_t* n_rules);
/* The policy switches of Simulation::processFlags (simulation.h:779-897) that
 * act on the locations, for the runForDay binding (matlab/mexPanSim.cpp:92-126):
 * the non-essential locations of the listed types (at most 10) become open
 * or closed ("PLNONE" / "PL0"), and the weight of every non-home location is
 * divided (divide != 0) or multiplied by coef in double precision ("MA1.0" /
 * "MA0.8"). */
int psim_set_types_open(psim_ctx* ctx, const uint32_t* types, uint32_t n_types, int open);
int psim_scale_location_weights(psim_ctx* ctx, double coef, int divide);
/* Immunization (include/immunization.h:24-900): categories, first doses in
 * category order, booster rounds by age group, and the daily waning of
 * susceptibility and symptom scaling of susceptible agents.  The location
 * and per-agent-location types of the categories are the reference's fixed
 * ids (work entry 4, hospital 12/14, nursery 22, school 3).  A context with
 * immunization set runs Immunization::update in psim_midnight after the
 * progression (simulation.h:912) and reports the day's doses in the VAC
 * column; contexts with more than one replica reject it. */
#define PSIM_IMM_CATEGORIES 10
#define PSIM_IMM_MAX_ROUNDS 8
#define PSIM_IMM_MAX_WEEKS 160
typedef struct psim_immunization {
    uint32_t start_after_day;         /* --immunizationStart */
    uint32_t daily_doses;             /* --immunizationsPerWeek given as a number: that / 7 */
    uint32_t n_vacc_weeks;            /* > 0: --immunizationsPerWeek given as a file of weekly doses */
    uint32_t n_booster_rounds;        /* entries of --boosterStart */
    uint32_t daily_boosters;          /* --boostersPerWeek given as a number: that / 7 */
    uint32_t pad0;
    float vacc_per_week[PSIM_IMM_MAX_WEEKS];
    int32_t booster_start_after_day[PSIM_IMM_MAX_ROUNDS];
    uint32_t n_booster_weeks[PSIM_IMM_MAX_ROUNDS];   /* 0: daily_boosters */
    float booster_per_week[PSIM_IMM_MAX_ROUNDS][PSIM_IMM_MAX_WEEKS];
    float booster_age_percent[PSIM_IMM_MAX_ROUNDS][10];
    int32_t order[PSIM_IMM_CATEGORIES];              /* --immunizationOrder */
    float group_level[PSIM_IMM_CATEGORIES];          /* --vaccinationGroupLevel */
    float protection_infection[10], protection_infection_waning[10];
    float protection_symptomatic[10], protection_symptomatic_waning[10];
    float protection_hospitalization[10], protection_hospitalization_waning[10];
    int32_t variant_similarity[PSIM_MAX_STRAINS];
    float variant_similar_multiplier[PSIM_MAX_STRAINS];
} psim_immunization;
/* Sets the parameters and assigns the categories (Immunization::initCategories,
 * immunization.h:263-437: one draw per agent and category pass, stream
 * (agent, 0, IMM_CATEGORY + pass)).  imm == NULL switches immunization off. */
int psim_immunization_init(psim_ctx* ctx, const psim_immunization* imm);
/* Immunization::update for the midnight at t (what psim_midnight runs). */
int psim_immunize_day(psim_ctx* ctx, uint32_t t, uint32_t* immunized_today);

/* Non-COVID hospitalization and death (Simulation::otherDisease,
 * include/simulation.h:169-423; --otherDisease, on by default in the
 * reference, off in a new context).  Per living agent at each midnight, from
 * the stream (agent, t, OTHER_DISEASE): the end of a non-COVID hospital stay
 * kills with the table's probability; agents not dead, not severe and not in
 * hospital draw the (disabled) sudden death and then a hospitalization, whose
 * length in days is geometric with mean (unsigned)avgLength.  The
 * hospitalization probability is the table's times the yearly occupancy
 * multiplier, or, on the days that total_hospitalizations covers, times
 * max(0, target - in_hospital_with_covid * 9730000/179500) / 48000, with
 * in_hospital_with_covid counted per replica as in the reference
 * (due_with_covid 0: states 6..8; 1: infected agents at a hospital location
 * not discharged today).  psim_midnight runs it after the immunization
 * (simulation.h:911-912). */
typedef struct psim_other_disease {
    uint32_t enabled;                       /* --otherDisease */
    uint32_t due_with_covid;                /* --dueWithCOVID */
    uint32_t n_targets;                     /* days of --totalHospitalizations (0: none) */
    uint32_t pad0;
    const int32_t* total_hospitalizations;  /* [n_targets], per simulated day */
} psim_other_disease;
/* od == NULL or od->enabled == 0 switches it off. */
int psim_other_disease_init(psim_ctx* ctx, const psim_other_disease* od);
/* Simulation::otherDisease for the midnight at t (what psim_midnight runs). */
int psim_other_disease_day(psim_ctx* ctx, uint32_t t);

/* The current run parameters (closure rules change curfew, policy, testing
 * probabilities, ...). */
int psim_get_params(psim_ctx* ctx, psim_params* out);
/* The current schedule table (ReduceMovement edits it): event_offset
 * [n_agent_types*28+1] and, when non-NULL, up to `capacity` events. */
int psim_get_events(psim_ctx* ctx, uint32_t* event_offset, uint32_t* loc_type, float* chance, uint16_t* start,
                    uint16_t* end, uint16_t* duration, uint32_t capacity, uint32_t* n_events);

/* All steps of one day as one CUDA graph launch (captured on first use and
 * after any psim_set_params / psim_set_tracking). */
int psim_run_steps(psim_ctx* ctx, uint32_t day);
/* One day: psim_midnight at t = day*steps_per_day, then psim_run_steps. */
int psim_run_day(psim_ctx* ctx, uint32_t day, psim_day_stats* out /* [replicas] */);

/* Sets the tuning of the per-step kernels (recaptures the day graph). */
int psim_set_tuning(psim_ctx* ctx, const psim_tuning* tuning);
int psim_get_tuning(psim_ctx* ctx, psim_tuning* tuning);

/* Differentiable calibration (no counterpart in the reference: the gradient of
 * expected daily new infections over replicas and days).
 * theta = (k, location-type weights, age-band susceptibilities).
 * w_l = w_by_type[type_l]; slot_of_type[type] = weight slot 0..7 of that type
 * in the gradient (-1: not a parameter; NULL keeps the current table). */
int psim_set_type_weights(psim_ctx* ctx, const float* w_by_type /*[256]*/, const int8_t* slot_of_type /*[256]*/);
/* infection coefficient per replica */
int psim_set_replica_k(psim_ctx* ctx, const double* k /*[replicas]*/);
/* on != 0: while the steps run, accumulate sum_r weights[r] * d E_r / d theta,
 * E_r = sum over the steps of min(1, p_i) of susceptible agents (the expected
 * new infections given the sampled state), in FP64; weights NULL keeps them. */
int psim_set_adjoint(psim_ctx* ctx, int on, const double* weights /*[replicas]*/);
/* out[0] = d/dk, out[1..8] = d/dw of weight slots 0..7, out[9..24] = d/dsigma
 * of age bands 0..15 */
int psim_get_gradient(psim_ctx* ctx, double* out /*[25]*/, int reset);
/* device copies of the whole mutable state (per-day checkpoints: the backward
 * pass restores a day and recomputes its movement and draws) */
int psim_checkpoint_save(psim_ctx* ctx, uint32_t slot);
int psim_checkpoint_restore(psim_ctx* ctx, uint32_t slot);
int psim_checkpoint_drop(psim_ctx* ctx, uint32_t slot);
int psim_checkpoint_free(psim_ctx* ctx);
int psim_checkpoint_bytes(psim_ctx* ctx, uint64_t* out);

/* Accumulate the expected new infections (sum of infection probabilities of
 * susceptible agents, reported in psim_day_stats) during the steps. */
int psim_set_tracking(psim_ctx* ctx, int expected);

/* Location CSR (LocationsList::locationListOffsets / locationAgentList) of
 * the current positions.  With canonical != 0 each location's agents are
 * sorted by id, which equals thrust::stable_sort_by_key's output
 * (util.cpp:69).  After day graphs (whose step kernel keeps agent lists only
 * for the locations its draws visit) the full list is built first. */
int psim_get_csr(psim_ctx* ctx, int canonical, uint32_t* offsets /*[L+1]*/, uint32_t* agents /*[N]*/);
/* Per-location hazard r_l of the last psim_infect call (infectionRatios). */
int psim_get_hazard(psim_ctx* ctx, float* out /*[L]*/, int64_t* fixed_sum /*[L] or NULL*/);

/* Step t as the day graph runs it, after movement(t) with the sums afresh and
 * a rebuild of the agent list pending, with CUDA events around the step
 * kernel's three phases launched apart: the rebuild, the draws of t and the
 * queue + decisions of t + 1; ms[3] receives those three durations.  t and
 * t + 1 must lie in the same day. */
int psim_time_step_kernels(psim_ctx* ctx, uint32_t t, float* ms /* [3] */);
/* Timing of the last psim_run_steps graph launch, milliseconds. */
int psim_last_day_ms(psim_ctx* ctx, float* ms);
/* With on != 0 the day graph is captured with timeline stamps in its kernels
 * (the global nanosecond timer at every block's entry, at the end of each
 * phase of the step kernel and at its exit; one atomic per block and stamp)
 * and counters.  For the last psim_run_steps: psim_day_kernel_ms gives ms[5]
 * = {the day's first movement kernel, the step kernel's rebuilds (listing +
 * agent-list slots), its draws, its queues + decisions, and the time between
 * the kernels}, summed over the day; psim_day_timeline gives per step
 * s, at us[7*s .. 7*s+6], {the kernel's span from its first block's entry to
 * its last block's exit, the rebuild's listing, its slots, the draws, the
 * queue, the decisions (0 when the phase did not run), the time since the
 * previous kernel's last exit}, microseconds;
 * psim_day_counts gives out[7] = {agent-list entries the draws expanded,
 * those at a location with a nonzero ratio, agents queued for a decision,
 * steps at which agents were queued, steps that rebuilt the agent list,
 * locations and agents those rebuilds listed}, summed over the day's
 * steps. */
int psim_set_profiling(psim_ctx* ctx, int on);
int psim_day_kernel_ms(psim_ctx* ctx, float* ms /* [5] */);
int psim_day_timeline(psim_ctx* ctx, float* us /* [7 * steps_per_day] */);
int psim_day_counts(psim_ctx* ctx, uint64_t* out /* [7] */);
/* Counts of kernel launches issued by the library since creation. */
int psim_launch_count(psim_ctx* ctx, uint64_t* out);
/* The context's cudaStream_t (as void*), for callers that order their own work after it. */
int psim_stream_handle(psim_ctx* ctx, void** out);
/* Runs a device wait on a flag that nothing sets, bounded by `iters`
 * iterations; returns PSIM_ERR_DEVICE when the bound expires (it always
 * does) and leaves the context usable.  Exercises the error path of every
 * bounded wait in the library without faulting the GPU. */
int psim_bounded_wait_selftest(psim_ctx* ctx, uint32_t iters);
/* Test hook of the allocation-failure paths (no counterpart in the
 * reference, which checks allocations only at initialization,
 * simulation.h:762-765): the next `allowed` device allocations of the
 * library succeed and the one after fails as if the device were out of
 * memory (PSIM_ERR_ALLOC); allowed < 0 switches the hook off.  Process-wide.
 * A context whose creation failed is returned for psim_last_error and frees
 * everything it took in psim_destroy. */
int psim_set_alloc_fault(long long allowed);

/* psim_csr_build_noalloc — no counterpart in the reference.
 * For callers that cannot call cudaMalloc (their device memory belongs to
 * another allocator such as a framework's caching allocator or a pool set up
 * once, plug-ins that must not grow the device footprint, latency-sensitive
 * loops where cudaMalloc/cudaFree would synchronize the device): builds the
 * location CSR of a device array d_location[n_agents] (values < n_locations)
 * into caller-owned device buffers d_offsets[n_locations+1] and
 * d_agents[n_agents], on `stream` (a cudaStream_t, may be NULL), allocating
 * nothing.  Its scratch is one file-scope __device__ array sized for
 * PSIM_NOALLOC_MAX_LOCATIONS locations (about 16.8 MB, held by every GPU that
 * loads the library until the process exits); larger sizes are rejected with
 * PSIM_ERR_ARG and a message in psim_noalloc_last_error() (cleared at the
 * start of every call, so it describes the last call only).  The first call
 * on a device, and the first after that device's context changed (a device
 * reset, another context made current), looks up the array's device address
 * (cudaGetSymbolAddress, keyed by the context's unique id): make that first
 * call before any stream capture.  All calls share the array and it keeps
 * the last call's contents (the histogram is cleared at the start of each
 * call); calls that overlap on the GPU race.  The order of the agents within
 * a location is unspecified; locations >= n_locations are left out (then
 * d_offsets[n_locations] < n_agents and only that prefix of d_agents is
 * written). */
#define PSIM_NOALLOC_MAX_LOCATIONS (1u << 21)
#define PSIM_NOALLOC_MAX_AGENTS 0xFFFFFFF0u
int psim_csr_build_noalloc(const uint32_t* d_location, uint32_t n_agents, uint32_t n_locations,
                           uint32_t* d_offsets, uint32_t* d_agents, void* stream);
const char* psim_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
