/*
 * CPU oracle for the pansim_gb300 hot path — TEST INFRASTRUCTURE ONLY.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
 * as the checker.  Plain C restatement of khbence/pansim, one function per
 * reference routine (citations are paths inside the reference project).
 *
 * Deterministic conventions shared with the GPU path (and stated where the
 * reference itself has no defined result):
 *  - random draws: Philox streams of pansim_gb300/csrc/psim_rng.h, one stream
 *    per (replica seed, agent index within replica, timestamp, phase);
 *  - location quarantine written during movement is read back only from the
 *    next step on, and concurrent writes combine with max() (the reference
 *    races, movementPolicies.h:203,240);
 *  - setNoWorkToday picks the lowest agent id of a home (what the reference's
 *    single-threaded CPU loop does; its GPU atomicAdd picks an arbitrary one);
 *  - per-location sums are the exact 2^-40 fixed-point sums, the hazard is
 *    psim_hazard(): FP32 operations with a cancellation-free 1 - exp(-x)
 *    (reference: 1 - expf(x) in FP32, infectionPolicies.h:545); the FP64
 *    evaluation is returned beside it for the tolerance checks.
 * Build: gcc -O2 -ffp-contract=off (no FMA contraction: results must match
 * the device bit for bit).
 */
#include "psim_oracle.h"
#include "../pansim_gb300/csrc/psim_rng.h"
#include "../pansim_gb300/csrc/psim_immunity.h"
#include "../pansim_gb300/csrc/psim_other_disease.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NONE 0xFFFFFFFFu
#define WB_W 0
#define WB_N 1
#define WB_M 2
#define WB_S 3
#define WB_D 4

struct psim_oracle {
    const psim_model* m;
    psim_agents* a;
    psim_locations* l;
    psim_params p;
    psim_oracle_replicas r;
    uint32_t* agent_rep;   /* [N] */
    uint32_t* loc_rep;     /* [L] */
    uint32_t* csr_off;     /* [L+1] */
    uint32_t* csr_agents;  /* [N] */
    uint32_t* cursor;      /* [L+1] scatter cursors of the regroup */
    uint32_t* qu_pending;  /* [L] */
    uint32_t* no_work_loc; /* [L] */
    uint8_t* loc_flags;    /* [L] testing flags */
    uint8_t* hcw;          /* [N] healthcare workers */
    uint32_t* hcw_count;   /* [R] */
    uint32_t* tpp;         /* [R*3] last testing stats */
    uint32_t* variant_active; /* [R*V] */
    double* expected;      /* [R] expected infections since the last midnight */
    uint32_t spd;          /* steps per day */
    /* immunization (include/immunization.h) */
    int imm_on;
    psim_immunization imm;
    psim_imm_tables imm_tab;
    int imm_groups_ready;
    float imm_frac[PSIM_IMM_MAX_ROUNDS][10];
    uint32_t imm_category;   /* Immunization::currentCategory */
    uint32_t imm_today;      /* immunizedToday */
    /* non-COVID hospitalization and death (simulation.h:169-423) */
    int od_on;
    uint32_t od_due_with_covid;
    uint32_t od_n_targets;
    int32_t* od_targets;
};

static inline uint32_t wb_of(const psim_oracle* o, uint32_t i) { return o->m->state_wb[(uint8_t)o->a->state[i]]; }
static inline int infected_of(const psim_oracle* o, uint32_t i) { return o->m->state_infected[(uint8_t)o->a->state[i]] != 0; }

/* DynamicPPState::updateMeta, src/agentData/dynamicPPState.cpp:54-64 */
static void update_meta(psim_oracle* o, uint32_t i) {
    const psim_model* m = o->m;
    uint8_t s = (uint8_t)o->a->state[i];
    o->a->infectious[i] = m->state_infectious[s] * m->variant_multiplier[o->a->variant[i]];
    float su = m->state_susceptible[s] ? 1.0f : 0.0f;
    for (uint32_t v = 0; v < m->n_variants; ++v) o->a->susceptible[(size_t)v * o->a->n + i] = su;
}

/* RealMovementOps::findActualLocationForType, movementPolicies.h:69-122.
 * f0, f1, f2: the types resolved by first match (the callers pass home,
 * school, work, except the plan helpers, :1073-1080, :1144, :1209-1214). */
static uint32_t find_location3(psim_oracle* o, uint32_t i, uint32_t loc_type, int retry, psim_stream* rng,
                               uint32_t f0, uint32_t f1, uint32_t f2) {
    const uint32_t* off = o->a->loc_offset;
    const uint32_t* pl = o->a->poss_loc;
    const uint8_t* pt = o->a->poss_type;
    if (loc_type == f0 || loc_type == f1 || loc_type == f2) {
        for (uint32_t k = off[i]; k < off[i + 1]; ++k)
            if (loc_type == pt[k]) return pl[k];
        return NONE;
    }
    uint32_t counter = 0, pos = 0;
    for (uint32_t k = off[i]; k < off[i + 1]; ++k) {
        if (loc_type == pt[k]) {
            if (counter == 0) pos = k;
            counter++;
        }
    }
    if (counter == 1) return pl[pos];
    if (counter > 1) {
        uint32_t counter2 = counter, rand_idx = counter2;
        for (;;) {
            while (rand_idx == counter2) rand_idx = psim_below(rng, counter);
            counter2 = 0;
            for (uint32_t k = pos; k < off[i + 1]; ++k) {
                if (loc_type == pt[k]) {
                    if (counter2 == rand_idx) {
                        if (retry && o->l->open[pl[k]] == 0) {
                            retry = 0;
                            break;
                        }
                        return pl[k];
                    }
                    counter2++;
                }
            }
        }
    }
    return NONE;
}

static uint32_t find_location(psim_oracle* o, uint32_t i, uint32_t loc_type, int retry, psim_stream* rng) {
    return find_location3(o, i, loc_type, retry, rng, o->p.home_type, o->p.school_type, o->p.work_type);
}


/* quarantine written during a step: combined with max (atomically, as agents
 * move in parallel) and made visible from the next step */
static void qu_write(psim_oracle* o, uint32_t loc, uint32_t until) {
    if (loc == NONE || loc >= o->l->n) return;
    uint32_t cur = __atomic_load_n(&o->qu_pending[loc], __ATOMIC_RELAXED);
    while (cur < until &&
           !__atomic_compare_exchange_n(&o->qu_pending[loc], &cur, until, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
}

/* RealMovementOps::quarantineAgent, movementPolicies.h:176-245 */
static void quarantine_agent(psim_oracle* o, uint32_t i, uint32_t t, uint32_t until, psim_stream* rng) {
    const psim_params* p = &o->p;
    psim_agents* a = o->a;
    if (p->quarantine_policy == 0) return;
    if (a->st_diagnosed_ts[i] > 0 && !infected_of(o, i) && !p->quarantine_immune) return;
    if (!a->diagnosed[i] && a->st_immunization_ts[i] > 0 && !p->quarantine_immune) return;
    a->quarantined[i] = 1;
    a->st_quarantined_ts[i] = t;
    uint32_t prev_until = a->st_quarantined_until[i];
    a->st_quarantined_until[i] = until;
    a->st_days_in_quarantine[i] += (until - t) / (24u * 60u / p->time_step);
    if (a->diagnosed[i]) {
        uint32_t my_home = find_location(o, i, p->home_type, 0, rng);
        if (p->quarantine_policy > 1) qu_write(o, my_home, until);
        if (p->quarantine_policy > 2 && prev_until < t) {
            uint32_t classroom = find_location(o, i, p->classroom_type, 0, rng);
            uint32_t work = find_location(o, i, p->work_type, 0, rng);
            uint32_t to_close[2] = {classroom, work};
            for (int c = 0; c < 2; ++c) {
                uint32_t loc = to_close[c];
                if (loc != NONE && (o->l->type[loc] == p->work_type || o->l->type[loc] == p->classroom_type) &&
                    o->l->quarantine_until[loc] < t && o->l->open[loc] && o->l->closed_until[loc] < t)
                    qu_write(o, loc, until);
            }
        }
    }
}

static inline uint32_t steps_until_midnight(uint32_t minutes, uint32_t dt) { return (1440u - minutes) / dt; }

/* minutes of TimeDayDuration(unsigned mins) (timeDay.cpp:64): the hours are an
 * unsigned char, so a difference that went negative folds modulo 256 hours */
static inline uint32_t td_minutes(uint32_t mins) { return (uint32_t)(uint8_t)(mins / 60u) * 60u + mins % 60u; }

static int is_quarantine_type(const psim_oracle* o, uint32_t loc) {
    uint32_t ty = o->l->type[loc];
    const psim_params* p = &o->p;
    return ty == p->home_type || ty == p->school_type || ty == p->classroom_type || ty == p->work_type;
}

static void diagnose_and_quarantine(psim_oracle* o, uint32_t i, uint32_t t, uint32_t minutes, psim_stream* rng) {
    psim_agents* a = o->a;
    const psim_params* p = &o->p;
    a->diagnosed[i] = 1;
    a->st_diagnosed_ts[i] = t;
    if (steps_until_midnight(minutes, p->time_step) == 24u * 60u / p->time_step) a->st_diagnosed_ts[i]++;
    quarantine_agent(o, i, t, t + p->quarantine_length * 24u * 60u / p->time_step, rng);
}

/* RealMovementOps::doMovement, movementPolicies.h:263-1041 */
static void do_movement(psim_oracle* o, uint32_t i, uint32_t t, uint32_t minutes, uint32_t day) {
    psim_agents* a = o->a;
    const psim_params* p = &o->p;
    const psim_model* m = o->m;
    const uint32_t dt = p->time_step;
    const uint32_t rep = o->agent_rep[i];
    const uint32_t li = i - o->r.agent_offset[rep];
    const uint32_t cemetery = o->r.cemetery[rep];
    const uint32_t agent_type = a->type[i];
    psim_stream rng;
    psim_stream_init(&rng, o->r.seed[rep], li, t, PSIM_PHASE_MOVE);
    const uint32_t sum = steps_until_midnight(minutes, dt);

    /* curfew, :267-326 */
    if (p->enable_curfew && p->curfew_begin == minutes / dt) {
        uint32_t wb = wb_of(o, i);
        int dead_or_hosp = (wb == WB_D || wb == WB_S);
        int hosp_noncovid = (a->st_hospitalized_ts[i] <= t && a->st_hospitalized_until[i] > t);
        if (!dead_or_hosp && !hosp_noncovid) {
            if (agent_type + 1 == 7) {
                uint32_t workplace = find_location(o, i, p->work_type, 0, &rng);
                if (a->location[i] != workplace || workplace == NONE || o->l->open[workplace] == 0) {
                    a->location[i] = find_location(o, i, p->home_type, 0, &rng);
                    if (workplace == NONE || o->l->open[workplace] == 0) {
                        a->steps_until_move[i] = sum;
                        return;
                    }
                }
            } else {
                a->steps_until_move[i] = sum;
                a->location[i] = find_location(o, i, p->home_type, 0, &rng);
                return;
            }
        }
    }

    /* countdown, :328-331 */
    if (a->steps_until_move[i] > 0) {
        a->steps_until_move[i]--;
        return;
    }

    if (a->st_quarantined_until[i] <= t) a->quarantined[i] = 0;

    uint32_t wb = wb_of(o, i);
    if (wb == WB_D) {
        a->steps_until_move[i] = NONE;
        a->location[i] = cemetery;
        return;
    }

    uint32_t agent_home = find_location(o, i, p->home_type, 0, &rng);

    /* non-COVID hospitalization, :355-403 */
    if (a->st_hospitalized_ts[i] <= t && a->st_hospitalized_until[i] > t && wb != WB_S && wb != WB_D) {
        uint32_t x = a->st_hospitalized_until[i] - t - 1;
        a->steps_until_move[i] = x < sum ? x : sum;
        a->location[i] = find_location(o, i, p->hospital_type, 0, &rng);
        if (!a->diagnosed[i] && a->infectious[i] != 0.0f) diagnose_and_quarantine(o, i, t, minutes, &rng);
        return;
    }

    /* severe: hospital, :405-442 */
    if (wb == WB_S) {
        a->steps_until_move[i] = sum;
        a->location[i] = find_location(o, i, p->hospital_type, 0, &rng);
        if (!a->diagnosed[i] && a->infectious[i] != 0.0f) diagnose_and_quarantine(o, i, t, minutes, &rng);
        return;
    }

    /* location under quarantine, :445-513 */
    {
        uint32_t loc = a->location[i];
        if (p->quarantine_policy > 1 && t < o->l->quarantine_until[loc] && is_quarantine_type(o, loc)) {
            if (a->quarantined[i] == 0) quarantine_agent(o, i, t, o->l->quarantine_until[loc], &rng);
            if (a->quarantined[i]) {
                uint32_t x = o->l->quarantine_until[a->location[i]] - t - 1;
                a->steps_until_move[i] = x < sum ? x : sum;
                uint32_t home_location = find_location(o, i, p->home_type, 0, &rng);
                if (home_location != a->location[i]) a->location[i] = home_location;
                if (agent_home != NONE && a->location[i] != agent_home && a->steps_until_move[i] > 60u / dt)
                    a->stayed_home[i] = 0;
                return;
            }
        }
    }

    /* recent diagnosis, :515-583 */
    if ((p->quarantine_policy > 0 &&
         (a->diagnosed[i] || (a->st_diagnosed_ts[i] > 0 &&
                              (t - a->st_diagnosed_ts[i]) < p->quarantine_length * 24u * 60u / dt))) ||
        (p->quarantine_policy > 0 && a->quarantined[i])) {
        if (p->quarantine_policy > 0 && !a->quarantined[i])
            quarantine_agent(o, i, t, t + p->quarantine_length * 24u * 60u / dt, &rng);
        if (a->quarantined[i]) {
            a->location[i] = find_location(o, i, p->home_type, 0, &rng);
            a->steps_until_move[i] = sum;
            if (agent_home != NONE && a->location[i] != agent_home && a->steps_until_move[i] > 60u / dt)
                a->stayed_home[i] = 0;
            return;
        }
    }

    /* schedule window, :585-604 (AgentTypeList::getOffsetIndex, agentType.cpp:13-15) */
    uint32_t off_idx = 7u * wb + day + agent_type * 28u;
    uint32_t ev_b = m->event_offset[off_idx], ev_e = m->event_offset[off_idx + 1];
    int act_b = -1, act_e = -1;
    for (uint32_t j = ev_b; j < ev_e; ++j) {
        if (minutes >= m->ev_start[j] && minutes < m->ev_end[j] && act_b == -1) act_b = (int)j;
        if (minutes < m->ev_start[j]) {
            act_e = (int)j;
            break;
        }
        if (j == ev_e - 1) {
            if (minutes >= m->ev_start[j] && minutes < m->ev_end[j]) act_e = (int)ev_e;
        }
    }

    uint32_t new_type = NONE;
    /* Case 1, :634-656 */
    if (act_b == -1 && act_e == -1) {
        new_type = wb == WB_S ? p->hospital_type : p->home_type;
        a->location[i] = find_location(o, i, new_type, 0, &rng);
        a->steps_until_move[i] = sum;
    }
    /* Case 2 and 4, :658-855 */
    if (act_b != -1) {
        uint32_t num_pot = (uint32_t)((act_e == -1 ? act_b + 1 : act_e) - act_b);
        uint32_t picked = 0;
        uint32_t dur = 0;
        if (num_pot == 1) {
            new_type = m->ev_loc_type[act_b];
            dur = m->ev_duration[act_b];
        } else {
            double rnd = psim_u01(&rng) * 1.0;
            double thr = m->ev_chance[act_b];
            uint32_t idx = 0;
            while (rnd > thr && idx < num_pot) {
                idx++;
                thr += m->ev_chance[act_b + idx];
            }
            if (idx == num_pot) idx--;
            picked = idx;
            new_type = m->ev_loc_type[act_b + idx];
            dur = m->ev_duration[act_b + idx];
        }
        if (a->no_work[i] != 0 && new_type == p->work_type) {
            new_type = p->home_type;
            num_pot = 1;
            if (a->quarantined[i] == 0) a->st_days_in_quarantine[i]++;
        }
        uint32_t new_loc = find_location(o, i, new_type, num_pot == 1, &rng);
        int school_too_old = (new_type == p->school_type || new_type == p->classroom_type) &&
                             a->age[i] >= p->school_age_restriction;
        if (school_too_old ||
            ((o->l->open[new_loc] == 0 || o->l->closed_until[new_loc] > t) && new_type != p->work_type) ||
            (p->lockdown_nonvacc && a->st_immunization_ts[i] == 0)) {
            if (num_pot > 1) {
                double rnd = psim_u01(&rng) * 1.0;
                double thr = (picked == 0) ? 0.0
                                           : m->ev_chance[act_b] / (1.0 - m->ev_chance[act_b + picked]);
                uint32_t idx = 0;
                while (rnd > thr && idx < num_pot) {
                    idx++;
                    thr += (picked == idx) ? 0.0
                                           : m->ev_chance[act_b + idx] / (1.0 - m->ev_chance[act_b + picked]);
                }
                if (idx == num_pot) idx--;
                new_type = m->ev_loc_type[act_b + idx];
                dur = m->ev_duration[act_b + idx];
                new_loc = find_location(o, i, new_type, 0, &rng);
                if (school_too_old ||
                    ((o->l->open[new_loc] == 0 || o->l->closed_until[new_loc] > t) && new_type != p->work_type) ||
                    (p->lockdown_nonvacc && a->st_immunization_ts[i] == 0)) {
                    new_loc = find_location(o, i, p->home_type, 0, &rng);
                }
            } else {
                new_loc = find_location(o, i, p->home_type, 0, &rng);
            }
        } else if (new_type == p->school_type) {
            uint32_t my_class = find_location(o, i, p->classroom_type, 0, &rng);
            if (my_class != NONE && o->l->closed_until[my_class] > t)
                new_loc = find_location(o, i, p->home_type, 0, &rng);
        }
        a->location[i] = new_loc;
        if (dur / 60u > 24u) {
            a->steps_until_move[i] = sum;
        } else if (act_e == -1) {
            if (minutes + dur >= 1440u)
                a->steps_until_move[i] = sum;
            else
                a->steps_until_move[i] = dur / dt;
        } else {
            /* a read past the last event yields a 24:00 window */
            uint32_t nstart = (uint32_t)act_e < m->n_events ? m->ev_start[act_e] : 1440u;
            uint32_t nend = (uint32_t)act_e < m->n_events ? m->ev_end[act_e] : 1440u;
            if (minutes + dur < nstart) {
                a->steps_until_move[i] = dur / dt;
            } else if (minutes + dur > nend) {
                a->steps_until_move[i] = td_minutes(nend - minutes) / dt - 1u;
            } else {
                uint32_t st = td_minutes(nend - (minutes + dur)) / dt;
                uint32_t extra = psim_below(&rng, st);
                a->steps_until_move[i] = dur / dt + extra;
            }
        }
        if (agent_type + 1 == 7 && p->enable_curfew &&
            (p->curfew_begin <= minutes / dt || p->curfew_end > minutes / dt)) {
            int work_closed = (new_type == p->work_type &&
                               (o->l->open[new_loc] == 0 || o->l->closed_until[new_loc] > t));
            if (work_closed || (new_type != p->work_type && new_type != p->home_type)) a->location[i] = agent_home;
        }
    }
    /* Case 3, :858-911 */
    if (act_b == -1 && act_e != -1) {
        uint32_t length_steps = td_minutes((uint32_t)m->ev_end[act_e] - (uint32_t)m->ev_start[act_e]) / dt;
        uint32_t delay = psim_below(&rng, length_steps);
        a->steps_until_move[i] = td_minutes((uint32_t)m->ev_start[act_e] - minutes) / dt + delay;
        uint32_t left = a->steps_until_move[i];
        if (left < 30u / dt) {
            /* 3a: stay */
        } else if (left < 60u / dt) {
            new_type = p->public_type;
            a->location[i] = find_location(o, i, p->public_type, 0, &rng);
        } else {
            new_type = p->home_type;
            a->location[i] = find_location(o, i, p->home_type, 0, &rng);
        }
    }

    /* arrived at a quarantined place, :914-977 */
    {
        uint32_t loc = a->location[i];
        if (p->quarantine_policy > 1 && t < o->l->quarantine_until[loc] && is_quarantine_type(o, loc)) {
            if (!a->quarantined[i]) quarantine_agent(o, i, t, o->l->quarantine_until[loc], &rng);
            if (a->quarantined[i]) {
                uint32_t x = o->l->quarantine_until[a->location[i]] - t - 1;
                a->steps_until_move[i] = x < sum ? x : sum;
                uint32_t home_location = find_location(o, i, p->home_type, 0, &rng);
                if (home_location != a->location[i]) a->location[i] = home_location;
                if (agent_home != NONE && a->location[i] != agent_home && a->steps_until_move[i] > 60u / dt)
                    a->stayed_home[i] = 0;
                return;
            }
        }
    }

    /* diagnosis at hospital / doctor, :1012-1033 */
    if (new_type == p->hospital_type || (new_type == p->doctor_type && psim_u01(&rng) * 1.0 < 0.7)) {
        if (!a->diagnosed[i] && a->infectious[i] != 0.0f) diagnose_and_quarantine(o, i, t, minutes, &rng);
    }
    if (agent_home != NONE && a->location[i] != agent_home && a->steps_until_move[i] > 60u / dt)
        a->stayed_home[i] = 0;
    a->steps_until_move[i]--;
}

static uint32_t day_of_week(const psim_oracle* o, uint32_t t) {
    if (o->p.holiday_mode) return 6u; /* Days::SUNDAY, movementPolicies.h:1713 */
    return (o->p.start_day + t / o->spd) % 7u;
}

/* RealMovement::movement, movementPolicies.h:1625-1724 */
void psim_oracle_movement(psim_oracle* o, uint32_t t) {
    uint32_t minutes = (t % o->spd) * o->p.time_step;
    uint32_t day = day_of_week(o, t);
    const int64_t N = o->a->n, L = o->l->n;
    /* every agent touches only its own state (plus the max-combined
     * quarantine writes), so the agents run in parallel */
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t i = 0; i < N; ++i) do_movement(o, (uint32_t)i, t, minutes, day);
    /* location quarantine written this step becomes visible from the next one */
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < L; ++l) {
        if (o->qu_pending[l] > o->l->quarantine_until[l]) o->l->quarantine_until[l] = o->qu_pending[l];
        o->qu_pending[l] = 0;
    }
}

/* Util::updatePerLocationAgentLists, util.cpp:55-108 with the stable sort of
 * :69: agents grouped by location, ascending agent id within a location. */
static int cmp_u32(const void* x, const void* y) {
    uint32_t a = *(const uint32_t*)x, b = *(const uint32_t*)y;
    return a < b ? -1 : a > b;
}

void psim_oracle_regroup(psim_oracle* o) {
    const int64_t L = o->l->n, N = o->a->n;
    memset(o->csr_off, 0, sizeof(uint32_t) * (L + 1));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i) __atomic_fetch_add(&o->csr_off[o->a->location[i] + 1], 1u, __ATOMIC_RELAXED);
    /* inclusive prefix of csr_off[1..L]: per-chunk sums, then the chunks in parallel */
    {
        enum { CHUNKS = 64 };
        uint32_t part[CHUNKS + 1];
        const int64_t per = (L + CHUNKS - 1) / CHUNKS;
        part[0] = 0;
#pragma omp parallel for schedule(static)
        for (int c = 0; c < CHUNKS; ++c) {
            uint32_t acc = 0;
            const int64_t b = 1 + (int64_t)c * per, e = b + per < L + 1 ? b + per : L + 1;
            for (int64_t l = b; l < e; ++l) acc += o->csr_off[l];
            part[c + 1] = acc;
        }
        for (int c = 0; c < CHUNKS; ++c) part[c + 1] += part[c];
#pragma omp parallel for schedule(static)
        for (int c = 0; c < CHUNKS; ++c) {
            uint32_t acc = part[c];
            const int64_t b = 1 + (int64_t)c * per, e = b + per < L + 1 ? b + per : L + 1;
            for (int64_t l = b; l < e; ++l) {
                acc += o->csr_off[l];
                o->csr_off[l] = acc;
            }
        }
    }
    uint32_t* cur = o->cursor;
    memcpy(cur, o->csr_off, sizeof(uint32_t) * (L + 1));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; ++i)
        o->csr_agents[__atomic_fetch_add(&cur[o->a->location[i]], 1u, __ATOMIC_RELAXED)] = (uint32_t)i;
    /* ascending agent id inside each location (the stable sort's order) */
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t l = 0; l < L; ++l) {
        uint32_t b = o->csr_off[l], e = o->csr_off[l + 1];
        uint32_t* x = o->csr_agents + b;
        uint32_t n = e - b;
        if (n > 32) {
            qsort(x, n, sizeof(uint32_t), cmp_u32);
            continue;
        }
        for (uint32_t j = 1; j < n; ++j) {
            uint32_t v = x[j], q = j;
            while (q > 0 && x[q - 1] > v) {
                x[q] = x[q - 1];
                --q;
            }
            x[q] = v;
        }
    }
}

/* BasicInfection::infectionsAtLocations (infectionPolicies.h:481-546) and
 * LocationsList::infectAgents (locationList.h:233-310). */
void psim_oracle_infect(psim_oracle* o, uint32_t t, uint32_t v, float* hazard_f, int64_t* sum_fix,
                        double* sum64, double* r64, double* p64, double* exp_out) {
    psim_agents* a = o->a;
    const psim_params* p = &o->p;
    const psim_model* m = o->m;
    uint32_t L = o->l->n, N = a->n;
    float season_f = (float)psim_oracle_seasonality(p, t, o->spd);
    double season_d = psim_oracle_seasonality(p, t, o->spd);
    float* r = (float*)malloc(sizeof(float) * L);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t ll = 0; ll < (int64_t)L; ++ll) {
        uint32_t l = (uint32_t)ll;
        uint32_t b = o->csr_off[l], e = o->csr_off[l + 1];
        int64_t fix = 0;
        double s64 = 0.0;
        for (uint32_t j = b; j < e; ++j) {
            uint32_t ag = o->csr_agents[j];
            float inf = (a->variant[ag] == v) ? a->infectious[ag] : 0.0f;
            fix += (int64_t)llrintf(inf * PSIM_FIX_SCALE_F);
            s64 += (double)inf;
        }
        uint32_t rep = o->loc_rep[l];
        float k_f = (float)o->r.k[rep];
        float rf = 0.0f;
        double rd = 0.0;
        if (fix != 0 && e > b) rf = psim_hazard(fix, e - b, k_f, o->l->infectiousness[l], season_f, p->time_step);
        if (s64 != 0.0 && e > b) {
            double x = o->r.k[rep] * (s64 / (double)(e - b)) * (double)o->l->infectiousness[l] * season_d *
                       (double)p->time_step;
            rd = -expm1(-x);
        }
        r[l] = rf;
        if (hazard_f) hazard_f[l] = rf;
        if (sum_fix) sum_fix[l] = fix;
        if (sum64) sum64[l] = s64;
        if (r64) r64[l] = rd;
    }
    if (exp_out)
        for (uint32_t q = 0; q < o->r.n; ++q) exp_out[q] = 0.0;
    /* per-thread partial sums of the expected infections, added in thread order */
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    const uint32_t R = o->r.n;
    double* part = (double*)calloc((size_t)nt * R, sizeof(double));
#pragma omp parallel
    {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double* mine = part + (size_t)tid * R;
#pragma omp for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
        uint32_t i = (uint32_t)ii;
        uint32_t loc = a->location[i];
        float su = a->susceptible[(size_t)v * N + i];
        float s_eff = su * p->sigma_band[a->band[i]];
        if (p64) {
            p64[i] = (r64 ? r64[loc] : (double)r[loc]) * (double)su * (double)p->sigma_band[a->band[i]];
        }
        /* a zero ratio cannot infect (U >= 0): no draw */
        if (s_eff > 0.0f && r[loc] > 0.0f) {
            float pf = r[loc] * s_eff;
            uint32_t rep = o->agent_rep[i];
            uint32_t li = i - o->r.agent_offset[rep];
            double term = pf < 1.0f ? (double)pf : 1.0;
            mine[rep] += term;
            double U = psim_u01_once(o->r.seed[rep], li, t, PSIM_PHASE_INFECT + v);
            if (U < (double)pf) {
                /* DynamicPPState::gotInfected, dynamicPPState.cpp:235-244 */
                a->state[i] = (int8_t)m->first_infected_state;
                a->variant[i] = (uint8_t)v;
                a->days[i] = -2;
                update_meta(o, i);
                a->st_infected_ts[i] = t;
                a->st_infected_count[i]++;
                a->st_infected_loc[i] = loc;
                a->st_worst_state[i] = a->state[i];
                a->st_worst_ts[i] = t;
                a->st_variant_mask[i] |= 1u << v;
            }
        }
    }
    }
    for (int q = 0; q < nt; ++q)
        for (uint32_t rr = 0; rr < R; ++rr) {
            o->expected[rr] += part[(size_t)q * R + rr];
            if (exp_out) exp_out[rr] += part[(size_t)q * R + rr];
        }
    free(part);
    free(r);
}

/* one step of Simulation::runSimulation, simulation.h:918-922 */
void psim_oracle_step(psim_oracle* o, uint32_t t, const uint32_t* variant_active) {
    psim_oracle_movement(o, t);
    psim_oracle_regroup(o);
    for (uint32_t v = 0; v < o->m->n_variants; ++v) {
        int any = 0;
        for (uint32_t q = 0; q < o->r.n; ++q) any |= (variant_active ? variant_active[q * o->m->n_variants + v]
                                                                    : o->variant_active[q * o->m->n_variants + v]) != 0;
        if (any) psim_oracle_infect(o, t, v, NULL, NULL, NULL, NULL, NULL, NULL);
    }
}

/* LengthOfState::calculateDays, basicLengthAbstract.cpp:48-53 */
static int calc_days(psim_oracle* o, uint32_t pid, uint32_t state, uint32_t v, psim_stream* rng) {
    const psim_model* m = o->m;
    size_t idx = ((size_t)pid * m->n_states + state) * PSIM_MAX_STRAINS + v;
    if (m->len_avg[idx] == -1.0f) return -1;
    uint32_t thr = psim_geometric_threshold(m->len_p[idx]);
    int days = psim_geometric(rng, thr);
    while (m->len_max[idx] < (float)days) days = psim_geometric(rng, thr);
    return days;
}

/* MultiBadMatrix::NextStates::selectNext, multiBadMatrix.cpp:9-31 */
static uint32_t select_next(psim_oracle* o, uint32_t pid, uint32_t state, float scaling, psim_stream* rng, int* bad) {
    const psim_model* m = o->m;
    size_t ti = (size_t)pid * m->n_states + state;
    uint32_t bb = m->tr_bad_begin[ti], bc = m->tr_bad_count[ti];
    uint32_t nb = m->tr_neu_begin[ti], nc = m->tr_neu_count[ti];
    if (nc == 0) scaling = 1.0f;
    double random = psim_u01(rng);
    double pre = 0.0, bad_sum = 0.0;
    for (uint32_t k = 0; k < bc; ++k) {
        float c = m->tr_chance[bb + k] * scaling;
        pre += (double)c;
        if (random < pre) {
            *bad = 1;
            return m->tr_next[bb + k];
        }
        bad_sum += (double)m->tr_chance[bb + k];
    }
    double bad_scaling = 1.0 + ((bad_sum - pre) / (1.0 - bad_sum));
    if (bc == 0) bad_scaling = 1.0;
    uint32_t idx = 0;
    do {
        double c = (double)m->tr_chance[nb + idx] * bad_scaling;
        pre += c;
        ++idx;
    } while (pre < random && idx < nc);
    idx--;
    *bad = 0;
    return m->tr_next[nb + idx];
}

/* Simulation::updateAgents (simulation.h:425-471) -> DynamicPPState::update
 * (dynamicPPState.cpp:246-303) -> MultiBadMatrix::calculateNextState
 * (multiBadMatrix.cpp:120-125). */
void psim_oracle_progress(psim_oracle* o, uint32_t t) {
    psim_agents* a = o->a;
    const psim_model* m = o->m;
    const psim_params* p = &o->p;
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t ii = 0; ii < (int64_t)a->n; ++ii) {
        uint32_t i = (uint32_t)ii;
        uint32_t rep = o->agent_rep[i];
        uint32_t li = i - o->r.agent_offset[rep];
        psim_stream rng;
        psim_stream_init(&rng, o->r.seed[rep], li, t, PSIM_PHASE_PROGRESS);
        uint32_t v = a->variant[i];
        uint32_t st = (uint8_t)a->state[i];
        uint32_t pid = a->prog_id[i];
        /* BasicAgentMeta::getScalingSymptoms(v, st), agentMeta.cpp:84: slot
         * v*7 + max(6, st) -- the per-variant slot 6 up to state 6, the
         * unscaled value (slot never written) beyond */
        float meta = (st <= 6u && a->symptom_scaling_v) ? a->symptom_scaling_v[(size_t)v * a->n + i]
                                                       : a->symptom_scaling[i];
        float prog = (st == 7) ? m->death_scaling[v] / meta : m->prog_scaling[v];
        float scaling = meta * prog;
        int recovered = 0;
        int16_t days = a->days[i];
        int go = 1;
        if (days == -2) {
            days = (int16_t)calc_days(o, pid, st, v, &rng);
            if (v >= 3) days = (days * 0.7 == 0) ? 1 : (int16_t)(days * 0.7);
        } else if (days > 0) {
            --days;
            go = 0;
        }
        if (go && days == 0) {
            uint32_t old_state = st;
            int was_infected = m->state_infected[st] != 0;
            int bad = 0;
            uint32_t next = select_next(o, pid, st, scaling, &rng, &bad);
            int nd = calc_days(o, pid, next, v, &rng);
            a->state[i] = (int8_t)next;
            update_meta(o, i);
            days = (int16_t)nd;
            if (v >= 3 && next < 8) {
                float mul = next < 6 ? 0.7f : 0.5f;
                days = (days * mul == 0) ? 1 : (int16_t)(days * mul);
            }
            if (bad) {
                a->st_worst_state[i] = (int8_t)next;
                a->st_worst_ts[i] = t;
                a->st_worst_end_ts[i] = t + ((uint32_t)((int)days * 60 * 24)) / p->time_step;
            } else if (old_state != next) {
                if (was_infected && !m->state_infected[next]) {
                    a->st_recovered_ts[i] = t;
                    recovered = 1;
                }
            }
        }
        a->days[i] = days;
        if (recovered) a->diagnosed[i] = 0;
    }
}

static int quarantine_window_ok(uint32_t qu, uint32_t t, uint32_t ql_steps, uint32_t day_steps) {
    /* testingPolicies.h:89-95 */
    return qu == 0 || (qu != 0 && (qu - ql_steps >= t - day_steps || qu < t));
}

/* DetailedTesting::performTests, testingPolicies.h:370-475 (flagLocations
 * :64-148, doTesting :162-281). */
void psim_oracle_test(psim_oracle* o, uint32_t t, uint32_t* tpp) {
    psim_agents* a = o->a;
    const psim_params* p = &o->p;
    const psim_model* m = o->m;
    const uint32_t day_steps = 24u * 60u / p->time_step;
    const uint32_t ql_steps = p->quarantine_length * 24u * 60u / p->time_step;
    memset(o->loc_flags, 0, o->l->n);
    for (uint32_t i = 0; i < a->n; ++i) {
        if (a->st_diagnosed_ts[i] > t - day_steps) {
            uint32_t rep_ = o->agent_rep[i];
            psim_stream frng;
            psim_stream_init(&frng, o->r.seed[rep_], i - o->r.agent_offset[rep_], t, PSIM_PHASE_TEST_FLAG);
            
            uint32_t home = find_location(o, i, p->home_type, 0, &frng);
            if (home != NONE) o->loc_flags[home] = 1;
            uint32_t work = find_location(o, i, p->work_type, 0, &frng);
            if (work != NONE && quarantine_window_ok(o->l->quarantine_until[work], t, ql_steps, day_steps))
                o->loc_flags[work] = 1;
            uint32_t school = find_location(o, i, p->school_type, 0, &frng);
            if (school != NONE && quarantine_window_ok(o->l->quarantine_until[school], t, ql_steps, day_steps)) {
                o->loc_flags[school] = 1;
                uint32_t classroom = find_location(o, i, p->classroom_type, 0, &frng);
                if (classroom != NONE &&
                    quarantine_window_ok(o->l->quarantine_until[classroom], t, ql_steps, day_steps))
                    o->loc_flags[classroom] = 1;
            }
        }
    }
    const uint32_t delay_steps = p->testing_delay * 24u * 60u / p->time_step;
    for (uint32_t i = 0; i < a->n; ++i) {
        if (t > delay_steps && a->last_test[i] != NONE && a->last_test[i] > t - delay_steps) continue;
        if (wb_of(o, i) == WB_D || a->diagnosed[i]) continue;
        uint32_t rep = o->agent_rep[i];
        uint32_t li = i - o->r.agent_offset[rep];
        psim_stream rng;
        psim_stream_init(&rng, o->r.seed[rep], li, t, PSIM_PHASE_TEST);
        uint32_t home = find_location(o, i, p->home_type, 0, &rng);
        int home_flag = home != NONE ? o->loc_flags[home] : 0;
        uint32_t work = find_location(o, i, p->work_type, 0, &rng);
        int work_flag = work != NONE ? o->loc_flags[work] : 0;
        uint32_t school = find_location(o, i, p->school_type, 0, &rng);
        int school_flag = 0, class_flag = 0;
        if (school != NONE) {
            school_flag = o->loc_flags[school];
            uint32_t classroom = find_location(o, i, p->classroom_type, 0, &rng);
            if (classroom != NONE) class_flag = 1;
        }
        double prob = p->t_random;
        prob = prob + (double)home_flag * p->t_home;
        prob = prob + (double)work_flag * p->t_work;
        prob = prob + (double)school_flag * p->t_school;
        prob = prob + ((double)class_flag * 3.0) * p->t_school;
        if (work != NONE && (o->l->type[work] == p->doctor_type || o->l->type[work] == p->hospital_type))
            prob = prob + p->t_hospital;
        if (work != NONE && o->l->type[work] == p->nursery_type) prob = prob + p->t_nursery;
        if (a->st_hospitalized_ts[i] <= t && a->st_hospitalized_until[i] > t) prob = prob + p->t_hospital;
        if (prob > 1.0 || psim_u01(&rng) * 1.0 < prob) {
            a->last_test[i] = t;
            if (infected_of(o, i)) {
                uint8_t st = (uint8_t)a->state[i];
                float acc = p->use_pcr ? m->state_acc_pcr[st] : m->state_acc_antigen[st];
                if ((double)acc > psim_u01(&rng) * 1.0) {
                    a->diagnosed[i] = 1;
                    a->st_diagnosed_ts[i] = t;
                }
            } else {
                if (a->st_quarantined_until[i] > t && (home != NONE && o->l->quarantine_until[home] < t)) {
                    if (a->st_days_in_quarantine[i] > 0)
                        a->st_days_in_quarantine[i] -= (a->st_quarantined_until[i] - t) / day_steps;
                    a->st_quarantined_until[i] = t;
                }
            }
        }
    }
    for (uint32_t q = 0; q < o->r.n; ++q) {
        uint32_t tests = 0, p1 = 0, p2 = 0;
        for (uint32_t i = o->r.agent_offset[q]; i < o->r.agent_offset[q + 1]; ++i) {
            tests += a->last_test[i] == t;
            p1 += a->st_diagnosed_ts[i] == t;
            p2 += (a->st_diagnosed_ts[i] < t && a->st_diagnosed_ts[i] > t - day_steps);
        }
        o->tpp[q * 3 + 0] = tests;
        o->tpp[q * 3 + 1] = p1;
        o->tpp[q * 3 + 2] = p2;
        if (tpp) {
            tpp[q * 3 + 0] = tests;
            tpp[q * 3 + 1] = p1;
            tpp[q * 3 + 2] = p2;
        }
    }
}

/* Simulation::refreshAndPrintStatistics, simulation.h:473-665, the TSV row
 * per replica; also countVariantCases (:768-777). */
void psim_oracle_stats(psim_oracle* o, uint32_t t, psim_day_stats* out) {
    psim_agents* a = o->a;
    const psim_model* m = o->m;
    const psim_params* p = &o->p;
    const uint32_t S = m->n_states, V = m->n_variants;
    const uint32_t day_steps = 24u * 60u / p->time_step;
    for (uint32_t q = 0; q < o->r.n; ++q) {
        psim_day_stats* d = &out[q];
        memset(d, 0, sizeof(*d));
        uint32_t b = o->r.agent_offset[q], e = o->r.agent_offset[q + 1];
        uint32_t hist[256] = {0};
        uint32_t hosp = 0, qn = 0, qt = 0, nq = 0, stayed = 0, ni = 0, inf_once = 0, reinf = 0, bstr = 0;
        uint32_t all_inf = 0, var_inf[PSIM_MAX_STRAINS] = {0}, infv[PSIM_MAX_STRAINS] = {0};
        double imm[PSIM_MAX_STRAINS] = {0};
        uint32_t hci = 0, hce = 0, infh = 0, vni = 0;
        for (uint32_t i = b; i < e; ++i) {
            uint8_t st = (uint8_t)a->state[i];
            hist[st]++;
            uint32_t wb = m->state_wb[st];
            int inf = m->state_infected[st] != 0;
            if (wb != WB_D && wb != WB_S && t < a->st_hospitalized_until[i]) hosp++;
            int isq = a->st_quarantined_ts[i] <= t && a->st_quarantined_until[i] > t;
            qn += isq;
            qt += isq && inf;
            nq += !isq && inf;
            stayed += a->stayed_home[i] != 0;
            int new_inf = a->st_infected_ts[i] > t - day_steps && a->st_infected_ts[i] <= t;
            ni += new_inf;
            inf_once += a->st_infected_count[i] > 0;
            reinf += a->st_infected_count[i] > 1 ? a->st_infected_count[i] - 1u : 0u;
            bstr += a->st_immunization_count[i] > 1 ? a->st_immunization_count[i] - 1u : 0u;
            if (inf) {
                all_inf++;
                var_inf[a->variant[i]]++;
            }
            for (uint32_t v = 0; v < V; ++v) {
                imm[v] += 1.0 - (double)a->susceptible[(size_t)v * a->n + i];
                if (a->st_variant_mask[i] & (1u << v)) infv[v]++;
            }
            if (o->hcw[i]) {
                hci += (inf || a->quarantined[i]) ? 1u : 0u;
                hce += new_inf;
            }
            if (inf && o->l->type[a->location[i]] == p->hospital_type) infh++;
            vni += a->st_infected_count[i] == 0 && a->st_immunization_count[i] > 0;
        }
        uint32_t n = 0;
        for (uint32_t s = 0; s < S; ++s) d->v[n++] = hist[s];
        d->v[n++] = hosp;
        d->v[n++] = o->tpp[q * 3 + 0];
        d->v[n++] = o->tpp[q * 3 + 1];
        d->v[n++] = o->tpp[q * 3 + 2];
        d->v[n++] = qn;
        d->v[n++] = qt;
        d->v[n++] = nq;
        if (V > 1) {
            for (uint32_t v = 1; v < V; ++v)
                d->v[n++] = all_inf ? (uint32_t)((double)var_inf[v] / (double)all_inf * 100.0) : 0u;
        } else {
            d->v[n++] = 0;
        }
        d->v[n] = stayed - d->v[10] - d->v[11];
        n++;
        d->v[n++] = o->imm_on ? o->imm_today : 0; /* VAC: immunized today */
        d->v[n++] = ni;
        d->v[n++] = inf_once;
        d->v[n++] = reinf;
        d->v[n++] = bstr;
        for (uint32_t v = 0; v < V; ++v) d->v[n++] = (uint32_t)imm[v];
        d->v[n++] = (hci * 100u) / (o->hcw_count[q] > 1 ? o->hcw_count[q] : 1u);
        d->v[n++] = hce;
        for (uint32_t v = 0; v < V; ++v) d->v[n++] = infv[v];
        d->v[n++] = infh;
        d->v[n++] = vni;
        d->n = n;
        d->new_infections = ni;
        for (uint32_t v = 0; v < V; ++v) {
            d->variant_counts[v] = var_inf[v];
            o->variant_active[q * V + v] = var_inf[v] > 0;
        }
        d->expected_new_infections = o->expected[q];
        o->expected[q] = 0.0;
    }
}

/* RealMovement::planLocations, movementPolicies.h:1428-1622 */
void psim_oracle_plan(psim_oracle* o, uint32_t t) {
    psim_agents* a = o->a;
    psim_locations* L = o->l;
    const psim_params* p = &o->p;
    for (uint32_t i = 0; i < a->n; ++i) {
        a->steps_until_move[i] = p->curfew_end;
        a->stayed_home[i] = 1;
        a->no_work[i] = 0;
    }
    memset(o->no_work_loc, 0, sizeof(uint32_t) * L->n);
    /* checkSchoolQuarantine, :1285-1310 */
    if (p->quarantine_policy > 3) {
        for (uint32_t s = 0; s < L->n_schools; ++s) {
            uint32_t school = L->schools[s];
            if (L->quarantine_until[school] > t) continue;
            uint32_t counter = 0, mx = 0;
            for (uint32_t c = L->classroom_offsets[s]; c < L->classroom_offsets[s + 1]; ++c) {
                uint32_t cl = L->classrooms[c];
                if (L->quarantine_until[cl] > t) {
                    counter++;
                    mx = mx > L->quarantine_until[cl] ? mx : L->quarantine_until[cl];
                }
            }
            if (counter > 1) {
                L->quarantine_until[school] = mx;
                for (uint32_t c = L->classroom_offsets[s]; c < L->classroom_offsets[s + 1]; ++c)
                    L->quarantine_until[L->classrooms[c]] = mx;
            }
        }
    }
    if (p->quarantine_policy > 2) {
        /* checkSchoolWorkQuarantine, :1188-1240 */
        for (uint32_t i = 0; i < a->n; ++i) {
            if (a->quarantined[i]) continue;
            if (a->st_diagnosed_ts[i] > 0 && !infected_of(o, i)) continue;
            uint32_t rep_ = o->agent_rep[i];
            psim_stream frng;
            psim_stream_init(&frng, o->r.seed[rep_], i - o->r.agent_offset[rep_], t, PSIM_PHASE_PLAN_SWQ);
            uint32_t work = find_location3(o, i, p->work_type, 0, &frng, p->home_type, p->school_type, p->classroom_type);
            uint32_t school = find_location3(o, i, p->school_type, 0, &frng, p->home_type, p->school_type, p->classroom_type);
            uint32_t classroom = find_location3(o, i, p->classroom_type, 0, &frng, p->home_type, p->school_type, p->classroom_type);
            uint32_t until = 0;
            if (school != NONE && L->quarantine_until[school] > t)
                until = L->quarantine_until[school];
            else if (classroom != NONE && L->quarantine_until[classroom] > t)
                until = L->quarantine_until[classroom];
            else if (work != NONE && L->quarantine_until[work] > t)
                until = L->quarantine_until[work];
            if (until > 0) {
                a->quarantined[i] = 1;
                a->st_quarantined_ts[i] = t;
                a->st_quarantined_until[i] = until;
                a->st_days_in_quarantine[i] += (until - t) / (24u * 60u / p->time_step);
            }
        }
        /* :1571-1583 */
        for (uint32_t l = 0; l < L->n; ++l) {
            uint32_t ty = L->type[l];
            if (L->quarantine_until[l] > t && (ty == p->school_type || ty == p->classroom_type)) {
                L->closed_until[l] = L->quarantine_until[l];
                L->quarantine_until[l] = 0;
            } else if (L->quarantine_until[l] > t && ty == p->work_type) {
                L->quarantine_until[l] = 0;
            }
        }
    }
    /* checkUnderageAtHome, :1056-1094 */
    for (uint32_t i = 0; i < a->n; ++i) {
        if (a->age[i] > 14) continue;
        uint32_t rep_ = o->agent_rep[i];
        psim_stream frng;
        psim_stream_init(&frng, o->r.seed[rep_], i - o->r.agent_offset[rep_], t, PSIM_PHASE_PLAN_UNDERAGE);
        uint32_t home = find_location3(o, i, p->home_type, 0, &frng, p->home_type, p->school_type, p->classroom_type);
        if (a->quarantined[i]) {
            if (home != NONE) o->no_work_loc[home] = 1;
        } else {
            uint32_t school = find_location3(o, i, p->school_type, 0, &frng, p->home_type, p->school_type, p->classroom_type);
            uint32_t classroom = find_location3(o, i, p->classroom_type, 0, &frng, p->home_type, p->school_type, p->classroom_type);
            int too_old = a->age[i] >= p->school_age_restriction;
            if (too_old || (school != NONE && (L->open[school] == 0 || L->closed_until[school] > t)) ||
                (classroom != NONE && (L->open[classroom] == 0 || L->closed_until[classroom] > t))) {
                if (home != NONE) o->no_work_loc[home] = 1;
            }
        }
    }
    /* setNoWorkToday, :1137-1158 (sequential: first eligible adult of a home) */
    for (uint32_t i = 0; i < a->n; ++i) {
        if (a->age[i] > 26 && a->age[i] < 65) {
            uint32_t rep_ = o->agent_rep[i];
            psim_stream frng;
            psim_stream_init(&frng, o->r.seed[rep_], i - o->r.agent_offset[rep_], t, PSIM_PHASE_PLAN_NOWORK);
            uint32_t home = find_location3(o, i, p->home_type, 0, &frng, p->home_type, p->home_type, p->home_type);
            if (home != NONE && o->no_work_loc[home] == 1) {
                o->no_work_loc[home] = 2;
                a->no_work[i] = 1;
            }
        }
    }
}

/* the midnight block of runSimulation, simulation.h:906-917 */
void psim_oracle_midnight(psim_oracle* o, uint32_t t, psim_day_stats* out) {
    if (t > 0 && o->p.testing_enabled) psim_oracle_test(o, t, NULL);
    if (t > 0) psim_oracle_progress(o, t);
    if (o->imm_on) psim_oracle_immunize(o, t);
    if (o->od_on) psim_oracle_other_disease(o, t);
    psim_oracle_stats(o, t, out);
    psim_oracle_plan(o, t);
}

void psim_oracle_run_day(psim_oracle* o, uint32_t day, psim_day_stats* out) {
    uint32_t t0 = day * o->spd;
    psim_oracle_midnight(o, t0, out);
    for (uint32_t s = 0; s < o->spd; ++s) psim_oracle_step(o, t0 + s, NULL);
}

/* host threads the parallel loops use */
int psim_oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Closure rule ExposeToMutation, closurePolicies.h:349-392: each agent with
 * susceptibility s > 0 for the variant is infected when a uniform draw is
 * below fraction * s; the draw comes from the agent's EXPOSE stream. */
void psim_oracle_expose(psim_oracle* o, uint32_t t, uint32_t v, double fraction) {
    psim_agents* a = o->a;
    const psim_model* m = o->m;
    const uint32_t N = a->n;
    for (uint32_t i = 0; i < N; ++i) {
        float su = a->susceptible[(size_t)v * N + i];
        if (!(su > 0.0f)) continue;
        uint32_t rep = o->agent_rep[i];
        uint32_t li = i - o->r.agent_offset[rep];
        double U = psim_u01_once(o->r.seed[rep], li, t, PSIM_PHASE_EXPOSE);
        if (U < fraction * (double)su) {
            a->state[i] = (int8_t)m->first_infected_state;
            a->variant[i] = (uint8_t)v;
            a->days[i] = -2;
            update_meta(o, i);
            a->st_infected_ts[i] = t;
            a->st_infected_loc[i] = a->location[i];
            a->st_infected_count[i]++;
            a->st_worst_state[i] = a->state[i];
            a->st_worst_ts[i] = t;
            a->st_variant_mask[i] |= 1u << v;
        }
    }
}

/* ---- Immunization (include/immunization.h:24-900) ---------------------- */

static int imm_has_entry(const psim_oracle* o, uint32_t i, uint32_t pa, uint32_t pb, uint32_t la, uint32_t lb,
                         int essential) {
    const psim_agents* a = o->a;
    for (uint32_t q = a->loc_offset[i]; q < a->loc_offset[i + 1]; ++q) {
        uint32_t pt = a->poss_type[q];
        if (pt != pa && pt != pb) continue;
        uint32_t loc = a->poss_loc[q];
        if (essential) {
            if (o->l->essential[loc] == 1) return 1;
        } else {
            uint32_t lt = o->l->type[loc];
            if (lt == la || lt == lb) return 1;
        }
    }
    return 0;
}

/* the category lambdas of initCategories, immunization.h:277-375 */
static int imm_in_category(const psim_oracle* o, uint32_t i, uint32_t g) {
    uint32_t age = o->a->age[i], pre = o->a->precond ? o->a->precond[i] : 0;
    switch (g) {
        case 0: return imm_has_entry(o, i, 4, 4, 12, 14, 0);
        case 1: return imm_has_entry(o, i, 4, 2, 22, 22, 0);
        case 2: return pre > 0 && age >= 60;
        case 3: return age >= 60;
        case 4: return pre > 0 && age >= 18 && age < 60;
        case 5: return imm_has_entry(o, i, 4, 4, 0, 0, 1);
        case 6: return imm_has_entry(o, i, 4, 4, 3, 3, 0);
        case 7: return age > 17 && age < 60;
        case 8: return age >= 12 && age < 18;
        default: return age >= 5 && age < 12;
    }
}

/* age group of initAgeGroups / the booster passes: [10g, 10g+10), the last [90, 200) */
static uint32_t imm_age_group(uint32_t age) { return age >= 200u ? 10u : (age >= 90u ? 9u : age / 10u); }

static uint32_t imm_local(const psim_oracle* o, uint32_t i, uint64_t* seed) {
    uint32_t rep = o->agent_rep[i];
    *seed = o->r.seed[rep];
    return i - o->r.agent_offset[rep];
}

/* Immunization::initializeArgs + initCategories, immunization.h:170-437 */
void psim_oracle_immunization_init(psim_oracle* o, const psim_immunization* imm) {
    psim_agents* a = o->a;
    o->imm_on = imm != NULL;
    if (!imm) return;
    o->imm = *imm;
    psim_imm_make_tables(&o->imm_tab, imm->protection_infection, imm->protection_infection_waning,
                         imm->protection_symptomatic, imm->protection_symptomatic_waning,
                         imm->protection_hospitalization, imm->protection_hospitalization_waning,
                         imm->variant_similarity, imm->variant_similar_multiplier);
    o->imm_groups_ready = 0;
    o->imm_category = 0;
    o->imm_today = 0;
    for (int v = 1; v <= PSIM_IMM_CATEGORIES; ++v)
        for (uint32_t g = 0; g < PSIM_IMM_CATEGORIES; ++g) {
            if (imm->order[g] != v) continue;
            for (uint32_t i = 0; i < a->n; ++i) {
                if (a->imm_round[i] != 0 || !imm_in_category(o, i, g)) continue;
                uint64_t seed;
                uint32_t li = imm_local(o, i, &seed);
                double U = psim_u01_once(seed, li, 0, PSIM_PHASE_IMM_CATEGORY + g);
                a->imm_round[i] = U < (double)imm->group_level[g] ? (uint8_t)imm->order[g] : (uint8_t)255;
            }
        }
}

static uint32_t imm_vaccines_today(const psim_immunization* p, uint32_t t, uint32_t spd) {
    uint32_t day = t / spd;
    if (day < p->start_after_day) return 0;
    if (p->n_vacc_weeks == 0) return p->daily_doses;
    uint32_t week = (day - p->start_after_day) / 7;
    return (uint32_t)(p->vacc_per_week[week >= p->n_vacc_weeks ? p->n_vacc_weeks - 1 : week] / 7.0);
}

static uint32_t imm_boosters_today(const psim_immunization* p, uint32_t t, uint32_t spd, uint32_t r) {
    uint32_t day = t / spd;
    if (day < (uint32_t)p->booster_start_after_day[r]) return 0;
    if (p->n_booster_weeks[r] == 0) return p->daily_boosters;
    uint32_t week = (day - (uint32_t)p->booster_start_after_day[r]) / 7;
    return (uint32_t)(p->booster_per_week[r][week >= p->n_booster_weeks[r] ? p->n_booster_weeks[r] - 1 : week] / 7.0);
}

static int imm_booster_ok(const psim_oracle* o, uint32_t i, uint32_t ts, uint32_t spd) {
    const psim_agents* a = o->a;
    return a->st_immunization_ts[i] > 0 && a->st_immunization_count[i] >= 1 &&
           (ts - a->st_immunization_ts[i]) / spd > 120u && wb_of(o, i) == 0 && ts >= spd * 90u &&
           a->st_diagnosed_ts[i] < ts - spd * 120u;
}

static int imm_primary_ok(const psim_oracle* o, uint32_t i, uint32_t ts, uint32_t spd) {
    const psim_agents* a = o->a;
    uint32_t d = a->st_diagnosed_ts[i];
    return a->st_immunization_count[i] == 0 && wb_of(o, i) == 0 &&
           ((ts < spd * 90u && d == 0) || (ts >= spd * 90u && d < ts - spd * 90u));
}

/* Immunization::update, immunization.h:481-900 */
uint32_t psim_oracle_immunize(psim_oracle* o, uint32_t t) {
    psim_agents* a = o->a;
    const psim_immunization* p = &o->imm;
    const uint32_t N = a->n, V = o->m->n_variants, spd = o->spd;
    if (!o->imm_on) return 0;
    if (!o->imm_groups_ready) {
        uint32_t hist[11] = {0};
        for (uint32_t i = 0; i < N; ++i) hist[imm_age_group(a->age[i])]++;
        for (uint32_t r = 0; r < p->n_booster_rounds; ++r) {
            uint32_t size[10], sum = 0;
            for (int g = 0; g < 10; ++g) {
                size[g] = (uint32_t)((float)hist[g] * p->booster_age_percent[r][g]);
                sum += size[g];
            }
            for (int g = 0; g < 10; ++g) o->imm_frac[r][g] = (float)size[g] / (float)sum;
        }
        o->imm_groups_ready = 1;
    }
    uint32_t ts = t == 0 ? 1u : t;
    /* waning of every susceptible agent */
    for (uint32_t i = 0; i < N; ++i) {
        if (a->state[i] != 0) continue;
        float susc[PSIM_MAX_STRAINS], scale[PSIM_MAX_STRAINS];
        uint8_t set[PSIM_MAX_STRAINS];
        uint32_t wi = (ts - a->st_infected_ts[i]) / (7u * spd);
        uint32_t wv = (ts - a->st_immunization_ts[i]) / (7u * spd);
        psim_imm_wane(&o->imm_tab, V, a->st_infected_count[i], a->st_immunization_count[i], wi, wv,
                      a->st_variant_mask[i], susc, scale, set);
        for (uint32_t v = 0; v < V; ++v) {
            if (set[v]) a->symptom_scaling_v[(size_t)v * N + i] = a->symptom_scaling[i] * scale[v];
            a->susceptible[(size_t)v * N + i] = susc[v];
        }
    }
    /* booster rounds */
    for (uint32_t r = 0; r < p->n_booster_rounds; ++r) {
        uint32_t available = imm_boosters_today(p, t, spd, r);
        if (!available) continue;
        uint32_t counts[11] = {0};
        for (uint32_t i = 0; i < N; ++i)
            if (imm_booster_ok(o, i, ts, spd)) counts[imm_age_group(a->age[i])]++;
        for (uint32_t g = 0; g < 10; ++g) {
            uint32_t avail_g = (uint32_t)((float)available * o->imm_frac[r][g]);
            float prob = counts[g] < avail_g ? 1.0f : (float)avail_g / (float)counts[g];
            for (uint32_t i = 0; i < N; ++i) {
                if (imm_age_group(a->age[i]) != g || !imm_booster_ok(o, i, ts, spd)) continue;
                int give = prob == 1.0f;
                if (!give) {
                    uint64_t seed;
                    uint32_t li = imm_local(o, i, &seed);
                    give = psim_u01_once(seed, li, ts, PSIM_PHASE_IMM_BOOSTER + r) < (double)prob;
                }
                if (give) {
                    a->st_immunization_ts[i] = ts;
                    a->st_immunization_count[i]++;
                }
            }
        }
    }
    /* first doses in category order */
    uint32_t available = imm_vaccines_today(p, t, spd);
    while (available > 0 && o->imm_category < PSIM_IMM_CATEGORIES) {
        uint32_t count = 0;
        while (count == 0 && o->imm_category <= PSIM_IMM_CATEGORIES) {
            uint32_t cc = o->imm_category + 1;
            for (uint32_t i = 0; i < N; ++i)
                if ((a->imm_round[i] == cc || cc == PSIM_IMM_CATEGORIES + 1) && imm_primary_ok(o, i, ts, spd)) count++;
            if (count == 0) o->imm_category++;
        }
        float prob = count < available ? 1.0f : (float)available / (float)count;
        uint32_t cc = o->imm_category + 1;
        for (uint32_t i = 0; i < N; ++i) {
            if (a->imm_round[i] != cc || !imm_primary_ok(o, i, ts, spd)) continue;
            int give = prob == 1.0f;
            if (!give) {
                uint64_t seed;
                uint32_t li = imm_local(o, i, &seed);
                give = psim_u01_once(seed, li, ts, PSIM_PHASE_IMM_PRIMARY + o->imm_category) < (double)prob;
            }
            if (give) {
                a->st_immunization_ts[i] = ts;
                a->st_immunization_count[i] = 1;
            }
        }
        available -= count < available ? count : available;
    }
    o->imm_today = 0;
    for (uint32_t i = 0; i < N; ++i) o->imm_today += a->st_immunization_ts[i] == ts;
    return o->imm_today;
}

/* Simulation::flagHealthcareWorkers, simulation.h:670-693 */
static void flag_hcw(psim_oracle* o) {
    psim_agents* a = o->a;
    memset(o->hcw_count, 0, sizeof(uint32_t) * o->r.n);
    for (uint32_t i = 0; i < a->n; ++i) {
        uint8_t f = 0;
        for (uint32_t k = a->loc_offset[i]; k < a->loc_offset[i + 1]; ++k) {
            uint32_t lt = o->l->type[a->poss_loc[k]];
            if (a->poss_type[k] == 4 && (lt == 12 || lt == 14)) {
                f = 1;
                break;
            }
        }
        o->hcw[i] = f;
        o->hcw_count[o->agent_rep[i]] += f;
    }
}

psim_oracle* psim_oracle_create(const psim_model* m, psim_agents* a, psim_locations* l, const psim_params* p,
                                const psim_oracle_replicas* reps) {
    psim_oracle* o = (psim_oracle*)calloc(1, sizeof(psim_oracle));
    o->m = m;
    o->a = a;
    o->l = l;
    o->p = *p;
    o->r = *reps;
    o->spd = 1440u / p->time_step;
    o->agent_rep = (uint32_t*)malloc(sizeof(uint32_t) * (a->n ? a->n : 1));
    o->loc_rep = (uint32_t*)malloc(sizeof(uint32_t) * (l->n ? l->n : 1));
    for (uint32_t q = 0; q < reps->n; ++q) {
        for (uint32_t i = reps->agent_offset[q]; i < reps->agent_offset[q + 1]; ++i) o->agent_rep[i] = q;
        for (uint32_t j = reps->loc_offset[q]; j < reps->loc_offset[q + 1]; ++j) o->loc_rep[j] = q;
    }
    o->csr_off = (uint32_t*)calloc(l->n + 1, sizeof(uint32_t));
    o->csr_agents = (uint32_t*)calloc(a->n ? a->n : 1, sizeof(uint32_t));
    o->cursor = (uint32_t*)calloc(l->n + 1, sizeof(uint32_t));
    o->qu_pending = (uint32_t*)calloc(l->n ? l->n : 1, sizeof(uint32_t));
    o->no_work_loc = (uint32_t*)calloc(l->n ? l->n : 1, sizeof(uint32_t));
    o->loc_flags = (uint8_t*)calloc(l->n ? l->n : 1, 1);
    o->hcw = (uint8_t*)calloc(a->n ? a->n : 1, 1);
    o->hcw_count = (uint32_t*)calloc(reps->n, sizeof(uint32_t));
    o->tpp = (uint32_t*)calloc(reps->n * 3, sizeof(uint32_t));
    o->variant_active = (uint32_t*)calloc((size_t)reps->n * m->n_variants, sizeof(uint32_t));
    o->expected = (double*)calloc(reps->n, sizeof(double));
    flag_hcw(o);
    psim_oracle_regroup(o); /* LocationsList::initialize, locationList.h:224-230 */
    /* countVariantCases before the first day */
    for (uint32_t i = 0; i < a->n; ++i)
        if (m->state_infected[(uint8_t)a->state[i]])
            o->variant_active[o->agent_rep[i] * m->n_variants + a->variant[i]] = 1;
    return o;
}

void psim_oracle_set_params(psim_oracle* o, const psim_params* p) { o->p = *p; }

void psim_oracle_destroy(psim_oracle* o) {
    if (!o) return;
    free(o->agent_rep);
    free(o->loc_rep);
    free(o->csr_off);
    free(o->csr_agents);
    free(o->cursor);
    free(o->qu_pending);
    free(o->no_work_loc);
    free(o->loc_flags);
    free(o->hcw);
    free(o->hcw_count);
    free(o->od_targets);
    free(o->tpp);
    free(o->variant_active);
    free(o->expected);
    free(o);
}

const uint32_t* psim_oracle_csr_offsets(psim_oracle* o) { return o->csr_off; }
const uint32_t* psim_oracle_csr_agents(psim_oracle* o) { return o->csr_agents; }

void psim_oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    psim_ctr4 c;
    for (int i = 0; i < 4; ++i) c.v[i] = ctr[i];
    psim_ctr4 r = psim_philox4x32_10(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

double psim_oracle_one_minus_exp(double x) { return psim_one_minus_exp(x); }
float psim_oracle_one_minus_expf(float x) { return psim_one_minus_expf(x); }

/* BasicInfection::seasonalityMultiplier, infectionPolicies.h:443-478 */
double psim_oracle_seasonality(const psim_params* p, uint32_t t, uint32_t spd) {
    unsigned sim_day = t / spd;
    int d = (int)p->start_date + (int)sim_day;
    int d_peak = 59 + 22;
    d += 6;
    double c0 = 3.08;
    double trunc_val = 0.5;
    if (sim_day > 250 && sim_day < 450) {
        d += p->d_offset0;
        d_peak += p->d_peak_offset;
        c0 = p->c0;
    } else if (sim_day > 600) {
        trunc_val = p->trunc;
        if (p->n_d_offset > 1) d += p->d_offset1;
    }
    int d_mod = d % 366;
    if (d_mod > 366 / 2) d_mod = 366 - d_mod;
    double a1 = 0.5 * c0 * cos(2.0 * M_PI * (double)(d_mod - d_peak) / 366.0);
    double b1 = 1.0 - 0.5 * c0;
    double a2 = 0.5 * c0 * cos(2.0 * M_PI * (double)(d_peak - d_peak) / 366.0);
    double normed = (a1 + b1) / (a2 + b1);
    double calc = normed > trunc_val ? normed : trunc_val;
    calc = calc < 1.0 ? calc : 1.0;
    if (d_mod < d_peak) return 1.0;
    return calc;
}

/* Simulation::otherDisease, include/simulation.h:169-423, per replica.
 * In hospital with COVID (:177-195): dueWithCOVID 0 counts the states 6..8
 * of the reference's model; 1 counts infected agents whose location is a
 * hospital, less those of WB below S discharged today. */
static uint32_t od_with_covid(psim_oracle* o, uint32_t q, uint32_t t) {
    const psim_agents* a = o->a;
    uint32_t n = 0;
    for (uint32_t i = o->r.agent_offset[q]; i < o->r.agent_offset[q + 1]; ++i) {
        uint32_t s = (uint8_t)a->state[i];
        if (o->od_due_with_covid == 0) {
            n += (s >= 6 && s <= 8);
        } else {
            uint32_t loc = a->location[i];
            uint32_t lt = loc < o->l->n ? o->l->type[loc] : NONE;
            int discharged = wb_of(o, i) < WB_S && t > 0 && a->st_hospitalized_until[i] == t;
            n += o->m->state_infected[s] && lt == o->p.hospital_type && !discharged;
        }
    }
    return n;
}

void psim_oracle_other_disease_init(psim_oracle* o, const psim_other_disease* od) {
    free(o->od_targets);
    o->od_targets = NULL;
    o->od_on = od && od->enabled;
    o->od_n_targets = 0;
    if (!o->od_on) return;
    o->od_due_with_covid = od->due_with_covid;
    o->od_n_targets = od->n_targets;
    if (od->n_targets) {
        o->od_targets = (int32_t*)malloc(sizeof(int32_t) * od->n_targets);
        memcpy(o->od_targets, od->total_hospitalizations, sizeof(int32_t) * od->n_targets);
    }
}

/* the agents' pass (:214-421) for the midnight at t */
void psim_oracle_other_disease(psim_oracle* o, uint32_t t) {
    psim_agents* a = o->a;
    const psim_model* m = o->m;
    const uint32_t R = o->r.n, dt = o->p.time_step;
    const uint32_t day = t / o->spd;
    float* mul = (float*)calloc(R ? R : 1, sizeof(float));
    if (day < o->od_n_targets)
        for (uint32_t q = 0; q < R; ++q) {
            /* targetHospitalized (unsigned) and probabilityMul (float), :199-203 */
            double x = (double)o->od_targets[day] - (double)od_with_covid(o, q, t) * (9730000.0 / 179500.0);
            unsigned target = (unsigned)(x > 0.0 ? x : 0.0);
            mul[q] = (float)((double)(float)target / 48000.0);
        }
    /* the yearly occupancy multiplier (:389-393); past day 1194 the last one */
    uint32_t yi = 0;
    while (yi < 3 && (int32_t)day > psim_od_year_day[yi]) yi++;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)a->n; ++ii) {
        uint32_t i = (uint32_t)ii;
        uint32_t wb = wb_of(o, i);
        if (wb == WB_D) continue;
        uint32_t rep = o->agent_rep[i];
        psim_stream rng;
        psim_stream_init(&rng, o->r.seed[rep], i - o->r.agent_offset[rep], t, PSIM_PHASE_OTHER_DISEASE);
        uint32_t age = a->age[i];
        uint32_t ag = age < 5 ? 0 : age < 15 ? 1 : age < 30 ? 2 : age < 60 ? 3 : age < 70 ? 4 : age < 80 ? 5 : 6;
        uint32_t sex = (a->sex && a->sex[i]) ? 1 : 0;
        uint32_t pre = a->precond ? a->precond[i] : 0;
        uint32_t kind = pre == 2 ? 1 : (pre == 4 ? 2 : 0);
        /* the end of a non-COVID stay (:350-365) */
        if (t > 0 && a->st_hospitalized_until[i] == t) {
            if (psim_u01(&rng) * 1.0 < psim_od_prob[kind][1][sex][ag]) {
                /* DynamicPPState::die(false), dynamicPPState.cpp:313-325 */
                a->state[i] = (int8_t)m->noncovid_dead_state;
                a->days[i] = -1;
                update_meta(o, i);
                a->st_worst_state[i] = (int8_t)m->noncovid_dead_state;
                a->st_worst_ts[i] = t;
                continue;
            }
        }
        /* dead, severe or in hospital (:371-373) */
        if (wb == WB_S || t < a->st_hospitalized_until[i]) continue;
        /* sudden death (:376): the draw happens, the comparison is ANDed with false */
        (void)psim_u01(&rng);
        /* hospitalization (:395-416) */
        double prob = psim_od_prob[kind][0][sex][ag] * (mul[rep] > 0.0f ? (double)mul[rep] : psim_od_year_mult[yi]);
        if (psim_u01(&rng) * 1.0 < prob) {
            unsigned avg = (unsigned)psim_od_avg_length[kind];
            unsigned len = (unsigned)psim_geometric(&rng, psim_geometric_threshold(1.0 / (double)avg));
            if (len == 0) len = 1;
            a->st_hospitalized_ts[i] = t;
            a->st_hospitalized_until[i] = t + len * 24u * 60u / dt;
        }
    }
    free(mul);
}
