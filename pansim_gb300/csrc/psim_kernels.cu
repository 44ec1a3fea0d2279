// Hand-written sm_103a kernels of the PanSim per-timestep agent loop.
//
// The day graph (psim_api.cu): k_movement (RealMovementOps::doMovement,
// movementPolicies.h:263-1041, for every agent at the day's first step, with
// the per-location histogram and the per-location infectiousness sums of
// Util::reduce_by_location, util.h:48-101, as exact 2^-40 fixed-point int64
// sums), then one k_step per timestep: the agent list rebuilt where agents
// took new locations (replaces thrust::stable_sort_by_key, util.cpp:69), the
// infection ratio and draws over the locations with an infectious agent
// (infectionPolicies.h:520-546, LocationsList::infectAgents,
// locationList.h:233-310), and the decisions of the agents whose decision
// step comes next.
// The per-phase entry points (psim_movement, psim_regroup, psim_infect) use
// k_movement, the scans (k_scan / k_scan_v: prefix of the histogram, ratio
// of every dirty location) and k_scatter_draw (slots and agent-ordered draws).
// Per day: k_progress (DynamicPPState::update), k_test_flag/k_test (DetailedTesting),
// k_stats (refreshAndPrintStatistics), k_plan_* (RealMovement::planLocations).
//
// Built with --fmad=false: no multiply-add contraction, so every floating-point
// expression rounds exactly like the host oracle compiled with -ffp-contract=off.
#include <algorithm>

#include "psim_device.cuh"

namespace psim {

__device__ __forceinline__ uint32_t wb_of(const KArgs& k, uint32_t i) {
    return k.m.state_wb[(uint8_t)k.a.state[i]];
}
__device__ __forceinline__ bool infected_of(const KArgs& k, uint32_t i) {
    return k.m.state_infected[(uint8_t)k.a.state[i]] != 0;
}
__device__ __forceinline__ uint8_t loc_open(const KArgs& k, uint32_t l) { return l < k.l.n ? k.l.open[l] : 0; }
__device__ __forceinline__ uint32_t loc_closed_until(const KArgs& k, uint32_t l) {
    return l < k.l.n ? k.l.closed_until[l] : 0u;
}
__device__ __forceinline__ uint32_t loc_qu(const KArgs& k, uint32_t l) { return l < k.l.n ? k.l.quarantine_until[l] : 0u; }
__device__ __forceinline__ uint32_t loc_type(const KArgs& k, uint32_t l) { return l < k.l.n ? k.l.type[l] : NONE; }

// Entry j of the per-agent location lists: x = location, y = its type.
__device__ __forceinline__ uint2 poss_entry(const KArgs& k, uint32_t j) {
    if (k.a.poss4) {
        const uint32_t v = k.a.poss4[j];
        return make_uint2(v & 0x3FFFFFFu, v >> 26);
    }
    return k.a.poss[j];
}

// RealMovementOps::findActualLocationForType, movementPolicies.h:69-122.
// f0, f1, f2: the types resolved by first match (home, school, work except in
// the plan helpers, movementPolicies.h:1073-1080, :1144, :1209-1214).
// [b, e): the agent's entries in the per-agent location list.
__device__ uint32_t find_location_range(const KArgs& k, uint32_t b, uint32_t e, uint32_t lt, int retry,
                                        psim_stream* rng, uint32_t f0, uint32_t f1, uint32_t f2) {
    if (lt == f0 || lt == f1 || lt == f2) {
        for (uint32_t j = b; j < e; ++j) {
            const uint2 en = poss_entry(k, j);
            if (lt == en.y) return en.x;
        }
        return NONE;
    }
    uint32_t counter = 0, pos = 0, first = NONE;
    for (uint32_t j = b; j < e; ++j) {
        const uint2 en = poss_entry(k, j);
        if (lt == en.y) {
            if (counter == 0) {
                pos = j;
                first = en.x;
            }
            counter++;
        }
    }
    if (counter == 1) return first;
    if (counter > 1) {
        uint32_t counter2 = counter, rand_idx = counter2;
        // the reference loops until the pick is open or its one retry is
        // spent: a second pass always ends (retry is 0 by then)
        for (int pass = 0; pass < 2; ++pass) {
            while (rand_idx == counter2) rand_idx = psim_below(rng, counter);
            counter2 = 0;
            for (uint32_t j = pos; j < e; ++j) {
                const uint2 en = poss_entry(k, j);
                if (lt == en.y) {
                    if (counter2 == rand_idx) {
                        if (retry && loc_open(k, en.x) == 0) {
                            retry = 0;
                            break;
                        }
                        return en.x;
                    }
                    counter2++;
                }
            }
        }
    }
    return NONE;
}

__device__ __forceinline__ uint32_t find_location3(const KArgs& k, uint32_t i, uint32_t lt, int retry, psim_stream* rng,
                                                   uint32_t f0, uint32_t f1, uint32_t f2) {
    return find_location_range(k, k.a.loc_offset[i], k.a.loc_offset[i + 1], lt, retry, rng, f0, f1, f2);
}

__device__ __forceinline__ uint32_t find_location(const KArgs& k, uint32_t i, uint32_t lt, int retry, psim_stream* rng) {
    return find_location3(k, i, lt, retry, rng, k.p.home_type, k.p.school_type, k.p.work_type);
}

// A location quarantine written by a decision at step t: merged into
// quarantine_until by the scan of step t (build[3] = the step whose decisions
// wrote; every writer of a step stores the same value).
__device__ __forceinline__ void qu_write(const KArgs& k, uint32_t loc, uint32_t until, uint32_t t) {
    if (loc < k.l.n) {
        atomicMax(&k.l.qu_pending[loc], until);
        k.l.build[3] = t;
    }
}

// RealMovementOps::quarantineAgent, movementPolicies.h:176-245
// Returns whether the agent was quarantined (its flag set).
__device__ bool quarantine_agent(const KArgs& k, uint32_t i, uint32_t t, uint32_t until, psim_stream* rng) {
    const psim_params& p = k.p;
    if (p.quarantine_policy == 0) return false;
    if (k.a.st_diagnosed_ts[i] > 0 && !infected_of(k, i) && !p.quarantine_immune) return false;
    if (!k.a.diagnosed[i] && k.a.st_immunization_ts[i] > 0 && !p.quarantine_immune) return false;
    k.a.quarantined[i] = 1;
    k.a.st_quarantined_ts[i] = t;
    uint32_t prev_until = k.a.st_quarantined_until[i];
    k.a.st_quarantined_until[i] = until;
    k.a.st_days_in_quarantine[i] += (until - t) / (24u * 60u / p.time_step);
    if (k.a.diagnosed[i]) {
        uint32_t my_home = find_location(k, i, p.home_type, 0, rng);
        if (p.quarantine_policy > 1) qu_write(k, my_home, until, t);
        if (p.quarantine_policy > 2 && prev_until < t) {
            uint32_t classroom = find_location(k, i, p.classroom_type, 0, rng);
            uint32_t work = find_location(k, i, p.work_type, 0, rng);
            uint32_t to_close[2] = {classroom, work};
            for (int c = 0; c < 2; ++c) {
                uint32_t loc = to_close[c];
                if (loc != NONE && (loc_type(k, loc) == p.work_type || loc_type(k, loc) == p.classroom_type) &&
                    loc_qu(k, loc) < t && loc_open(k, loc) && loc_closed_until(k, loc) < t)
                    qu_write(k, loc, until, t);
            }
        }
    }
    return true;
}

// minutes of TimeDayDuration(unsigned mins) (timeDay.cpp:64): the hours are
// an unsigned char, so a difference that went negative folds modulo 256 hours
__device__ __forceinline__ uint32_t td_minutes(uint32_t mins) { return (uint32_t)(uint8_t)(mins / 60u) * 60u + mins % 60u; }

__device__ void diagnose_and_quarantine(const KArgs& k, uint32_t i, uint32_t t, uint32_t sum, psim_stream* rng) {
    const uint32_t dt = k.p.time_step;
    k.a.diagnosed[i] = 1;
    k.a.st_diagnosed_ts[i] = t;
    if (sum == 24u * 60u / dt) k.a.st_diagnosed_ts[i]++;
    (void)quarantine_agent(k, i, t, t + k.p.quarantine_length * 24u * 60u / dt, rng);
}

// S: the agent's countdown (stepsUntilMove) as the decision just set it;
// cur: the agent's location as the decision left it
__device__ __forceinline__ void stayed_home_check(const KArgs& k, uint32_t i, uint32_t agent_home, uint32_t cur,
                                                  uint32_t S) {
    if (agent_home != NONE && cur != agent_home && S > 60u / k.p.time_step) k.a.stayed_home[i] = 0;
}

// The agent's fields that a decision reads, loaded together before it
// starts: read where they are needed, behind branches and stores, each would
// cost a round trip of its own.  The decision keeps its own copies of the two
// it writes (location, quarantined flag).
struct DecisionIn {
    uint32_t loc, q_until, h_ts, h_until, lb, le, diag_ts, rep;
    float inf;
    uint8_t state, type, diag, no_work, age, quarantined;
};
__device__ __forceinline__ void decision_in(const KArgs& k, uint32_t i, DecisionIn& d) {
    d.loc = k.a.location[i];
    d.q_until = k.a.st_quarantined_until[i];
    d.h_ts = k.a.st_hospitalized_ts[i];
    d.h_until = k.a.st_hospitalized_until[i];
    d.lb = k.a.loc_offset[i];
    d.le = k.a.loc_offset[i + 1];
    d.diag_ts = k.a.st_diagnosed_ts[i];
    d.rep = k.a.rep[i];
    d.inf = k.a.infectious[i];
    d.state = (uint8_t)k.a.state[i];
    d.type = k.a.type[i];
    d.diag = k.a.diagnosed[i];
    d.no_work = k.a.no_work[i];
    d.age = k.a.age[i];
    d.quarantined = k.a.quarantined[i];
}

// Quarantine end and type of a location (the quarantine rule's inputs);
// neither changes during a step's decisions.
struct LocQ {
    uint32_t qu, ty;
};
__device__ __forceinline__ LocQ loc_q(const KArgs& k, uint32_t loc) {
    LocQ q;
    q.qu = loc_qu(k, loc);
    q.ty = loc_type(k, loc);
    return q;
}
__device__ __forceinline__ bool quarantine_type(const KArgs& k, uint32_t ty) {
    return ty == k.p.home_type || ty == k.p.school_type || ty == k.p.classroom_type || ty == k.p.work_type;
}

// The full per-agent decision of doMovement once the countdown reached zero
// (movementPolicies.h:333-1040).  The curfew and countdown prologue is in
// move_agent.  S receives the agent's new countdown (stepsUntilMove after
// the step); the caller turns it into the absolute timestamp of the next
// decision, cur the agent's location after it (d.loc before).  The
// location-dependent inputs (the quarantine rule's at the current and at the
// chosen location, the chosen location's flags) load together as soon as the
// location is known.
__device__ void move_decide(const KArgs& k, uint32_t i, uint32_t t, uint32_t minutes, uint32_t day, uint32_t sum,
                            psim_stream* rng, uint32_t& S, const DecisionIn& d, uint32_t& cur) {
    const psim_params& p = k.p;
    const uint32_t dt = p.time_step;
    const bool qrule = p.quarantine_policy > 1;
    const LocQ q_now = qrule ? loc_q(k, d.loc) : LocQ{0u, NONE};
    auto fl = [&](uint32_t lt, int retry) {
        return find_location_range(k, d.lb, d.le, lt, retry, rng, p.home_type, p.school_type, p.work_type);
    };
    cur = d.loc;
    auto set_loc = [&](uint32_t l) {
        cur = l;
        k.a.location[i] = l;
    };
    bool quar = d.quarantined != 0;
    if (d.q_until <= t) {
        quar = false;
        k.a.quarantined[i] = 0;
    }

    const uint32_t wb = k.m.state_wb[d.state];
    if (wb == WB_D) {
        S = NONE;
        set_loc(k.r.cemetery[d.rep]);
        return;
    }
    const uint32_t agent_home = fl(p.home_type, 0);

    if (d.h_ts <= t && d.h_until > t && wb != WB_S && wb != WB_D) {
        uint32_t x = d.h_until - t - 1;
        S = x < sum ? x : sum;
        set_loc(fl(p.hospital_type, 0));
        if (!d.diag && d.inf != 0.0f) diagnose_and_quarantine(k, i, t, sum, rng);
        return;
    }
    if (wb == WB_S) {
        S = sum;
        set_loc(fl(p.hospital_type, 0));
        if (!d.diag && d.inf != 0.0f) diagnose_and_quarantine(k, i, t, sum, rng);
        return;
    }
    if (qrule && t < q_now.qu && quarantine_type(k, q_now.ty)) {
        if (!quar) quar = quarantine_agent(k, i, t, q_now.qu, rng);
        if (quar) {
            // the location is still the current one
            uint32_t x = q_now.qu - t - 1;
            S = x < sum ? x : sum;
            uint32_t home_location = fl(p.home_type, 0);
            if (home_location != cur) set_loc(home_location);
            stayed_home_check(k, i, agent_home, cur, S);
            return;
        }
    }
    if ((p.quarantine_policy > 0 &&
         (d.diag || (d.diag_ts > 0 && (t - d.diag_ts) < p.quarantine_length * 24u * 60u / dt))) ||
        (p.quarantine_policy > 0 && quar)) {
        if (p.quarantine_policy > 0 && !quar) quar = quarantine_agent(k, i, t, t + p.quarantine_length * 24u * 60u / dt, rng);
        if (quar) {
            set_loc(fl(p.home_type, 0));
            S = sum;
            stayed_home_check(k, i, agent_home, cur, S);
            return;
        }
    }

    // schedule window (AgentTypeList::getOffsetIndex, agentType.cpp:13-15;
    // the window of the slot at this step, movementPolicies.h:585-603, from
    // the table the host computed)
    const uint32_t agent_type = d.type;
    const uint32_t off_idx = 7u * wb + day + agent_type * 28u;
    const int2 win = k.m.window[(size_t)off_idx * k.spd + minutes / dt];
    const int act_b = win.x, act_e = win.y;

    uint32_t new_type = NONE;
    // the quarantine rule's inputs at a location loaded with its flags
    uint32_t spec_loc = NONE;
    LocQ spec_q{0u, NONE};
    if (act_b == -1 && act_e == -1) {  // Case 1
        new_type = wb == WB_S ? p.hospital_type : p.home_type;
        set_loc(fl(new_type, 0));
        S = sum;
    }
    if (act_b != -1) {  // Case 2 and 4
        uint32_t num_pot = (uint32_t)((act_e == -1 ? act_b + 1 : act_e) - act_b);
        uint32_t picked = 0, dur = 0;
        if (num_pot == 1) {
            new_type = k.m.ev_loc_type[act_b];
            dur = k.m.ev_duration[act_b];
        } else {
            double rnd = psim_u01(rng) * 1.0;
            double thr = k.m.ev_chance[act_b];
            uint32_t idx = 0;
            while (rnd > thr && idx < num_pot) {
                idx++;
                thr += k.m.ev_chance[act_b + idx];
            }
            if (idx == num_pot) idx--;
            picked = idx;
            new_type = k.m.ev_loc_type[act_b + idx];
            dur = k.m.ev_duration[act_b + idx];
        }
        if (d.no_work != 0 && new_type == p.work_type) {
            new_type = p.home_type;
            num_pot = 1;
            if (!quar) k.a.st_days_in_quarantine[i]++;
        }
        uint32_t new_loc = fl(new_type, num_pot == 1);
        bool too_old = (new_type == p.school_type || new_type == p.classroom_type) && d.age >= p.school_age_restriction;
        // the new location's flags and quarantine inputs load together
        const uint8_t nl_open = loc_open(k, new_loc);
        const uint32_t nl_closed = loc_closed_until(k, new_loc);
        if (qrule) {
            spec_loc = new_loc;
            spec_q = loc_q(k, new_loc);
        }
        if (too_old || ((nl_open == 0 || nl_closed > t) && new_type != p.work_type) ||
            (p.lockdown_nonvacc && k.a.st_immunization_ts[i] == 0)) {
            if (num_pot > 1) {
                double rnd = psim_u01(rng) * 1.0;
                double pc = k.m.ev_chance[act_b + picked];
                double thr = (picked == 0) ? 0.0 : k.m.ev_chance[act_b] / (1.0 - pc);
                uint32_t idx = 0;
                while (rnd > thr && idx < num_pot) {
                    idx++;
                    thr += (picked == idx) ? 0.0 : k.m.ev_chance[act_b + idx] / (1.0 - pc);
                }
                if (idx == num_pot) idx--;
                new_type = k.m.ev_loc_type[act_b + idx];
                dur = k.m.ev_duration[act_b + idx];
                new_loc = fl(new_type, 0);
                if (too_old ||
                    ((loc_open(k, new_loc) == 0 || loc_closed_until(k, new_loc) > t) && new_type != p.work_type) ||
                    (p.lockdown_nonvacc && k.a.st_immunization_ts[i] == 0))
                    new_loc = fl(p.home_type, 0);
            } else {
                new_loc = fl(p.home_type, 0);
            }
        } else if (new_type == p.school_type) {
            uint32_t my_class = fl(p.classroom_type, 0);
            if (my_class != NONE && loc_closed_until(k, my_class) > t) new_loc = fl(p.home_type, 0);
        }
        set_loc(new_loc);
        if (dur / 60u > 24u) {
            S = sum;
        } else if (act_e == -1) {
            S = (minutes + dur >= 1440u) ? sum : dur / dt;
        } else {
            // a read past the last event yields a 24:00 window
            const bool in = (uint32_t)act_e < k.m.n_events;
            uint32_t nstart = in ? k.m.ev_start[act_e] : 1440u, nend = in ? k.m.ev_end[act_e] : 1440u;
            if (minutes + dur < nstart) {
                S = dur / dt;
            } else if (minutes + dur > nend) {
                S = td_minutes(nend - minutes) / dt - 1u;
            } else {
                uint32_t st = td_minutes(nend - (minutes + dur)) / dt;
                uint32_t extra = psim_below(rng, st);
                S = dur / dt + extra;
            }
        }
        if (agent_type + 1 == 7 && p.enable_curfew && (p.curfew_begin <= minutes / dt || p.curfew_end > minutes / dt)) {
            bool work_closed = new_type == p.work_type && (loc_open(k, new_loc) == 0 || loc_closed_until(k, new_loc) > t);
            if (work_closed || (new_type != p.work_type && new_type != p.home_type)) set_loc(agent_home);
        }
    }
    if (act_b == -1 && act_e != -1) {  // Case 3
        uint32_t length_steps = td_minutes((uint32_t)k.m.ev_end[act_e] - (uint32_t)k.m.ev_start[act_e]) / dt;
        uint32_t delay = psim_below(rng, length_steps);
        S = td_minutes((uint32_t)k.m.ev_start[act_e] - minutes) / dt + delay;
        uint32_t left = S;
        if (left < 30u / dt) {
        } else if (left < 60u / dt) {
            new_type = p.public_type;
            set_loc(fl(p.public_type, 0));
        } else {
            new_type = p.home_type;
            set_loc(fl(p.home_type, 0));
        }
    }
    if (qrule) {
        const LocQ q = cur == spec_loc ? spec_q : cur == d.loc ? q_now : loc_q(k, cur);
        if (t < q.qu && quarantine_type(k, q.ty)) {
            if (!quar) quar = quarantine_agent(k, i, t, q.qu, rng);
            if (quar) {
                uint32_t x = q.qu - t - 1;
                S = x < sum ? x : sum;
                uint32_t home_location = fl(p.home_type, 0);
                if (home_location != cur) set_loc(home_location);
                stayed_home_check(k, i, agent_home, cur, S);
                return;
            }
        }
    }
    if (new_type == p.hospital_type || (new_type == p.doctor_type && psim_u01(rng) * 1.0 < 0.7)) {
        if (!d.diag && d.inf != 0.0f) diagnose_and_quarantine(k, i, t, sum, rng);
    }
    stayed_home_check(k, i, agent_home, cur, S);
    S = S - 1u;
}

// curfew prologue of doMovement (movementPolicies.h:267-326); returns true if
// the agent's step is finished (S, the countdown, then holds `sum`).
__device__ bool curfew_prologue(const KArgs& k, uint32_t i, uint32_t t, uint32_t sum, psim_stream* rng, uint32_t& S) {
    const psim_params& p = k.p;
    uint32_t wb = wb_of(k, i);
    bool dead_or_hosp = (wb == WB_D || wb == WB_S);
    bool hosp_noncovid = (k.a.st_hospitalized_ts[i] <= t && k.a.st_hospitalized_until[i] > t);
    if (dead_or_hosp || hosp_noncovid) return false;
    if (k.a.type[i] + 1u == 7u) {
        uint32_t workplace = find_location(k, i, p.work_type, 0, rng);
        if (k.a.location[i] != workplace || workplace == NONE || loc_open(k, workplace) == 0) {
            k.a.location[i] = find_location(k, i, p.home_type, 0, rng);
            if (workplace == NONE || loc_open(k, workplace) == 0) {
                S = sum;
                return true;
            }
        }
        return false;
    }
    S = sum;
    k.a.location[i] = find_location(k, i, p.home_type, 0, rng);
    return true;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Hazard of variant 0 at `loc` and whether an infectious agent is there, for
// the agent-ordered draws of the per-phase entry points (the scan computed
// the location's hazards this step; elsewhere every hazard is 0): the hazard
// itself is gathered only at infectious locations.
__device__ __forceinline__ float hazard_at(const KArgs& k, uint32_t loc, bool* any) {
    const uint32_t w = k.l.hmask[loc >> 5];
    *any = ((w >> (loc & 31u)) & 1u) != 0;
    return *any ? k.l.hazard[loc] : 0.0f;
}

// ---------------------------------------------------------------------------
// Per-agent pieces of a step.

struct StepClock {
    uint32_t t, minutes, day, sum;
    bool curfew_now;
};

__device__ __forceinline__ StepClock step_clock(const KArgs& k, uint32_t step) {
    StepClock c;
    const uint32_t dt = k.p.time_step;
    c.t = k.clock->t0 + step;
    c.minutes = step * dt;
    c.day = k.clock->day_of_week;
    c.sum = (1440u - c.minutes) / dt;
    c.curfew_now = k.p.enable_curfew && k.p.curfew_begin == c.minutes / dt;
    return c;
}

// The countdown of the reference (stepsUntilMove: decremented every step,
// a decision when it reaches zero) is kept as the absolute timestamp of the
// agent's next decision, move_at = t + 1 + stepsUntilMove after step t (u32
// arithmetic: the dead agents' NONE countdown wraps like the reference's).
// Before step t the countdown is move_at - t; only a decision or the curfew
// prologue writes move_at, so the steps in between touch nothing.  The
// library converts to and from countdowns at upload and download (time base
// t_next, psim_api.cu).
//
// Steps of the running day at which some agent decides: one bit per step in
// move_mask, set by whoever writes such a move_at (through a block-shared
// copy, one global atomic per word and block).  The day graph's kernels read
// it to skip the steps nobody decides at.
__device__ __forceinline__ void mask_clear_shared(uint32_t* s_mm) {
    for (uint32_t w = threadIdx.x; w < MOVE_MASK_WORDS; w += blockDim.x) s_mm[w] = 0u;
    __syncthreads();
}
__device__ __forceinline__ void mask_note(const KArgs& k, uint32_t* s_mm, uint32_t m) {
    const uint32_t s = m - k.clock->t0;
    if (s < k.spd) {
        // most deciders of a step land on a few steps: read before the
        // atomic, whose lanes on one word would queue
        const uint32_t bit = 1u << (s & 31u);
        if (!(s_mm[s >> 5] & bit)) atomicOr(&s_mm[s >> 5], bit);
    }
}
__device__ __forceinline__ void mask_flush(const KArgs& k, uint32_t* s_mm) {
    __syncthreads();
    for (uint32_t w = threadIdx.x; w < MOVE_MASK_WORDS; w += blockDim.x)
        if (s_mm[w]) atomicOr(&k.a.move_mask[w], s_mm[w]);
}

// doMovement for agent i at step c.t; s = its countdown before the step
// (move_at - c.t).  Writes move_at when the agent decides or the curfew
// prologue resets its countdown.  pre: the decision's inputs when the caller
// loaded them (its agents all decide), else null (loaded here if needed).
// Returns the agent's location after the step (loc0: before it).
__device__ __forceinline__ uint32_t move_agent(const KArgs& k, uint32_t i, const StepClock& c, uint32_t s,
                                               uint32_t* s_mm, const DecisionIn* pre, uint32_t loc0) {
    if (!(c.curfew_now || s == 0)) return loc0;  // counts down: move_at stays
    DecisionIn d;
    if (pre)
        d = *pre;
    else
        decision_in(k, i, d);
    psim_stream rng;
    psim_stream_init(&rng, k.r.seed[d.rep], i - k.r.agent_off[d.rep], c.t, PSIM_PHASE_MOVE);
    bool done = false;
    uint32_t S = s;
    if (c.curfew_now) {
        done = curfew_prologue(k, i, c.t, c.sum, &rng, S);
        d.loc = k.a.location[i];  // the prologue may have sent the agent home
    }
    uint32_t cur = d.loc;
    if (!done) {
        if (S > 0)
            S = S - 1u;
        else
            move_decide(k, i, c.t, c.minutes, c.day, c.sum, &rng, S, d, cur);
    }
    const uint32_t m = c.t + 1u + S;
    k.a.move_at[i] = m;
    mask_note(k, s_mm, m);
    return cur;
}

// Scan tiles: 256 threads x ITEMS locations (ITEMS = 2, 4 or 8, a tuning
// choice); the masks hold one 32-bit word per warp and item.
constexpr int SCAN_THREADS = 256;

// A location that receives an infectious term sets its hazard-mask bit at
// once, so the mask is always a superset of the locations with a nonzero sum
// (the step kernel's rebuild lists from it and clears the bits of zero sums;
// the per-phase scans recompute the bits of their dirty locations).
__device__ __forceinline__ void mark_hazardous(const KArgs& k, uint32_t loc) {
    atomicOr(&k.l.hmask[loc >> 5], 1u << (loc & 31u));
}

// The full pass of a day's first step (k_movement, after a reset of the
// sums): an agent whose location changed from loc0 to loc moves one count
// (two fire-and-forget reductions), and every infectious agent adds its term
// at its (new) location.  Returns whether the agent took a new location (its
// kernel then publishes the timestamp of the new locations, publish_moved).
__device__ __forceinline__ bool count_agent(const KArgs& k, bool act, uint32_t loc0, uint32_t loc, float inf,
                                            uint32_t variant) {
    const uint32_t L = k.l.n;
    if (act && loc >= L) {
        atomicOr(k.err, ERR_LOCATION);
        loc = NONE;
    }
    const bool mv = act && loc != loc0;
    if (mv) {
        if (loc0 < L) atomicSub(&k.l.counts[loc0], 1u);
        if (loc != NONE) atomicAdd(&k.l.counts[loc], 1u);
    }
    if (act && loc != NONE && inf > 0.0f) {
        const long long q = __float2ll_rn(inf * PSIM_FIX_SCALE_F);
        atomicAdd(&k.l.sfix[(size_t)variant * L + loc], (unsigned long long)q);
        atomicAdd(&k.l.sfix_b[(size_t)variant * L + loc], (unsigned long long)q);
        atomicOr(&k.l.smask[loc >> 5], 1u << (loc & 31u));
        mark_hazardous(k, loc);
    }
    return mv;
}

// Within a day the per-location sums persist: an agent changes them only
// when it moves or its infectiousness changes (a draw that infects).  The
// first step of a day (k_movement after a reset of the sums) adds every
// agent's term afresh.
// The agent went from (loc0, inf0, var0) to (loc, inf, var) in a step
// kernel's decision: its count moves, its fixed-point term leaves (loc0,
// var0) and joins (loc, var).  The step kernel computes every ratio from the
// sums, so it keeps no dirty marks (the day graph marks every location dirty
// at its start: a scan after it recomputes every ratio).  Returns whether the
// agent took a new location.
__device__ __forceinline__ bool count_agent_delta(const KArgs& k, bool act, uint32_t loc0, uint32_t loc, float inf0,
                                                  uint32_t var0, float inf, uint32_t var) {
    const uint32_t L = k.l.n;
    if (act && loc >= L) {
        atomicOr(k.err, ERR_LOCATION);
        loc = NONE;
    }
    const bool mv = act && loc != loc0;
    if (mv) {
        if (loc0 < L) atomicSub(&k.l.counts[loc0], 1u);
        if (loc != NONE) atomicAdd(&k.l.counts[loc], 1u);
    }
    if (act) {
        const long long q0 = (loc0 < L && inf0 > 0.0f) ? __float2ll_rn(inf0 * PSIM_FIX_SCALE_F) : 0ll;
        const long long q1 = (loc != NONE && inf > 0.0f) ? __float2ll_rn(inf * PSIM_FIX_SCALE_F) : 0ll;
        if (mv || q0 != q1 || var0 != var) {
            // both copies of the step kernel's sums (the next step reads
            // the other one)
            if (q0) {
                atomicAdd(&k.l.sfix[(size_t)var0 * L + loc0], (unsigned long long)(-q0));
                atomicAdd(&k.l.sfix_b[(size_t)var0 * L + loc0], (unsigned long long)(-q0));
            }
            if (q1) {
                atomicAdd(&k.l.sfix[(size_t)var * L + loc], (unsigned long long)q1);
                atomicAdd(&k.l.sfix_b[(size_t)var * L + loc], (unsigned long long)q1);
                mark_hazardous(k, loc);
            }
        }
    }
    return mv;
}

// The full histogram of the current positions (after a reset of counts and sums).
__device__ __forceinline__ void count_full(const KArgs& k, bool act, uint32_t loc, float inf, uint32_t variant) {
    const uint32_t L = k.l.n;
    if (!act) return;
    if (loc >= L) {
        atomicOr(k.err, ERR_LOCATION);
        return;
    }
    atomicAdd(&k.l.counts[loc], 1u);
    if (inf > 0.0f) {
        const long long q = __float2ll_rn(inf * PSIM_FIX_SCALE_F);
        atomicAdd(&k.l.sfix[(size_t)variant * L + loc], (unsigned long long)q);
        atomicAdd(&k.l.sfix_b[(size_t)variant * L + loc], (unsigned long long)q);
        atomicOr(&k.l.smask[loc >> 5], 1u << (loc & 31u));
        mark_hazardous(k, loc);
    }
}

// CSR slot of an agent: a warp-aggregated returning atomic on the location's
// cursor, which the scan set to the location's first slot.  Warp-collective.
// the slot of an agent whose step keeps the agent list of the step before
constexpr uint32_t SLOT_KEEP = 0xFFFFFFFEu;

__device__ __forceinline__ uint32_t take_slot(const KArgs& k, bool ok, uint32_t loc, bool rebuild) {
    if (!rebuild) return SLOT_KEEP;
    if (!k.tune.agg_slot) return ok ? atomicAdd(&k.l.cursor[loc], 1u) : NONE;
    const unsigned valid = __ballot_sync(0xffffffffu, ok);
    uint32_t pos = NONE;
    if (ok) {
        const unsigned peers = __match_any_sync(valid, loc);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(&k.l.cursor[loc], (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        pos = base + (uint32_t)__popc(peers & lanemask_lt());
    }
    return pos;
}

__device__ __forceinline__ void store_slot(const KArgs& k, uint32_t pos, uint32_t i) {
    if (pos == SLOT_KEEP) return;
    if (pos < k.a.n)
        k.l.csr_agents[pos] = i;
    else
        atomicOr(k.err, ERR_LOCATION);
}

// Infection draws of agent i at location loc with hazard h0 of variant 0
// (LocationsList::infectAgents, locationList.h:233-310; DynamicPPState::gotInfected,
// dynamicPPState.cpp:235-244).  Returns the sum of min(1, p) over the draws.
// d p / d theta of one draw (p = r * s * sigma_band, r = 1 - exp(-x),
// x = k * S/n * w * season * dt), weighted by the replica's dL/dE, added to the
// block's FP64 accumulators
// x: the location's hazard argument k*S/n*w*season*dt for variant v
__device__ __noinline__ void adjoint_terms(const KArgs& k, uint32_t i, uint32_t loc, uint32_t v, uint32_t rep, float r,
                                           float su, float s_eff, double* s_grad, float x_f) {
    const double g = k.adj.weight[rep];
    if (g == 0.0) return;
    const double x = (double)x_f;
    const double dpdx = (double)s_eff * (1.0 - (double)r);
    const double kf = (double)k.r.k_f[rep];
    if (kf != 0.0) atomicAdd(&s_grad[GRAD_K], g * dpdx * x / kf);
    const int slot = k.adj.type_slot[k.l.type[loc]];
    const double w = (double)k.l.infectiousness[loc];
    if (slot >= 0 && w != 0.0) atomicAdd(&s_grad[GRAD_W + slot], g * dpdx * x / w);
    atomicAdd(&s_grad[GRAD_SIGMA + k.a.band[i]], g * (double)r * (double)su);
}

__device__ __forceinline__ double draw_agent(const KArgs& k, uint32_t i, uint32_t loc, uint32_t t, float h0,
                                             double* s_grad) {
    const uint32_t N = k.a.n, L = k.l.n, V = k.m.n_variants;
    // the agent's fields load together (variant 0's susceptibility: a draw
    // that infects rewrites the later variants' before they are read)
    const uint32_t rep = k.a.rep[i];
    const float sigma = k.p.sigma_band[k.a.band[i]];
    const float su0 = k.a.susceptible[i];
    const unsigned long long seed = k.r.seed[rep];
    const uint32_t li = i - k.r.agent_off[rep];
    double term_sum = 0.0;
    for (uint32_t v = 0; v < V; ++v) {
        const float h = v == 0 ? h0 : k.l.hazard[(size_t)v * L + loc];
        if (!(h > 0.0f)) continue;
        if (!k.r.variant_active[rep * V + v]) continue;
        const float su = v == 0 ? su0 : k.a.susceptible[(size_t)v * N + i];
        const float s_eff = su * sigma;
        if (!(s_eff > 0.0f)) continue;
        const float pf = h * s_eff;
        term_sum += pf < 1.0f ? (double)pf : 1.0;
        if (k.adj.on && pf < 1.0f)
            adjoint_terms(k, i, loc, v, rep, h, su, s_eff, s_grad, k.l.hazard_x[(size_t)v * L + loc]);
        const double U = psim_u01_once(seed, li, t, PSIM_PHASE_INFECT + v);
        if (U < (double)pf) {
            k.a.state[i] = (int8_t)k.m.first_infected;
            k.a.variant[i] = (uint8_t)v;
            k.a.days[i] = -2;
            update_meta(k, i);
            k.a.st_infected_ts[i] = t;
            k.a.st_infected_count[i] = k.a.st_infected_count[i] + 1;
            k.a.st_infected_loc[i] = loc;
            k.a.st_worst_state[i] = (int8_t)k.m.first_infected;
            k.a.st_worst_ts[i] = t;
            k.a.st_variant_mask[i] |= 1u << v;
        }
    }
    return term_sum;
}

__device__ __forceinline__ void grad_begin(const KArgs& k, double* s_grad) {
    if (!k.adj.on) return;
    if (threadIdx.x < GRAD_N) s_grad[threadIdx.x] = 0.0;
    __syncthreads();
}

// one global atomic per block and parameter
__device__ __forceinline__ void grad_end(const KArgs& k, double* s_grad) {
    if (!k.adj.on) return;
    __syncthreads();
    if (threadIdx.x < GRAD_N && s_grad[threadIdx.x] != 0.0) atomicAdd(&k.adj.grad[threadIdx.x], s_grad[threadIdx.x]);
}

// expected-infection accumulation: one atomic per replica present in the warp
__device__ __forceinline__ void add_expected(const KArgs& k, bool act, uint32_t i, double term) {
    const unsigned am = __ballot_sync(0xffffffffu, act && term != 0.0);
    if (!(act && term != 0.0)) return;
    const uint32_t rep = k.a.rep[i];
    const unsigned peers = __match_any_sync(am, rep);
    const int leader = __ffs(peers) - 1;
    unsigned rest = peers;
    double tot = 0.0;
    while (rest) {
        const int src = __ffs(rest) - 1;
        tot += __shfl_sync(peers, term, src);
        rest &= rest - 1;
    }
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(&k.r.expected[rep], tot);
}

// Timeline stamps of the profiled day graph (KArgs::prof): one atomic per
// block, from thread 0, on the global nanosecond timer.
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// the block's entry (no wait for the other threads)
__device__ __forceinline__ void prof_enter(const KArgs& k, uint32_t slot) {
    if (k.prof && threadIdx.x == 0) atomicMax(&k.prof[slot], ~global_ns());
}
// the block's threads are past this point (every thread calls it)
__device__ __forceinline__ void prof_mark(const KArgs& k, uint32_t slot) {
    if (!k.prof) return;
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(&k.prof[slot], global_ns());
}

// Movement of every agent + histogram + fixed-point infectiousness sums (the
// day's first step, after a reset of the sums, and the per-phase entry
// points).  Records the steps of the day at which agents decide next.
__global__ void __launch_bounds__(256) k_movement(KArgs k, uint32_t step) {
    __shared__ uint32_t s_mm[MOVE_MASK_WORDS];
    if (step == 0) prof_enter(k, PROF_N);
    mask_clear_shared(s_mm);
    const uint32_t N = k.a.n;
    const StepClock c = step_clock(k, step);
    const uint32_t stride = gridDim.x * blockDim.x;
    bool moved = false;
    for (uint32_t base = blockIdx.x * blockDim.x; base < N; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool act = i < N;
        uint32_t loc = NONE, loc0 = NONE, var = 0;
        float inf = 0.0f;
        if (act) {
            const uint32_t m0 = k.a.move_at[i];
            const uint32_t s = m0 - c.t;
            loc0 = k.a.location[i];
            inf = k.a.infectious[i];
            loc = move_agent(k, i, c, s, s_mm, nullptr, loc0);
            if (!(c.curfew_now || s == 0)) mask_note(k, s_mm, m0);  // an agent counting down decides later today
            if (inf > 0.0f) var = k.a.variant[i];
        }
        moved |= count_agent(k, act, loc0, loc, inf, var);
    }
    publish_moved(k, moved, c.t);
    mask_flush(k, s_mm);
    if (step == 0) prof_mark(k, PROF_N + 1);
}

// Histogram + fixed-point sums without movement (regroup after an upload).
__global__ void __launch_bounds__(256) k_count(KArgs k) {
    const uint32_t N = k.a.n;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < N; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool act = i < N;
        uint32_t loc = NONE, var = 0;
        float inf = 0.0f;
        if (act) {
            loc = k.a.location[i];
            inf = k.a.infectious[i];
            if (inf > 0.0f) var = k.a.variant[i];
        }
        count_full(k, act, loc, inf, var);
    }
}

// ---------------------------------------------------------------------------
// Scan of the histogram in two passes (reduce, then scan): k_tile_sums adds up
// each tile of 256 x ITEMS locations; k_scan adds the sums of the tiles before its
// own (every block reads at most a few thousand 4-byte sums, so the prefix
// needs no inter-block waiting), scans its tile warp-striped (coalesced),
// writes the cursor (exclusive prefix = first CSR slot of the location)
// and evaluates the infection ratio of every location
// with a non-zero infectiousness sum.

__device__ __forceinline__ uint32_t block_sum_256(uint32_t v, uint32_t* s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    uint32_t tot = 0;
#pragma unroll
    for (int q = 0; q < SCAN_THREADS / 32; ++q) tot += s_red[q];
    __syncthreads();
    return tot;
}

template <int ITEMS>
__global__ void __launch_bounds__(SCAN_THREADS) k_tile_sums(KArgs k, uint32_t step) {
    constexpr int TILE = SCAN_THREADS * ITEMS;
    __shared__ uint32_t s_red[SCAN_THREADS / 32];
    if (!csr_decide(k, k.clock->t0 + step)) return;  // the tile sums serve the rebuild only
    const uint32_t L = k.l.n;
    const uint32_t base = blockIdx.x * TILE;
    uint32_t v = 0;
#pragma unroll
    for (int q = 0; q < ITEMS; ++q) {
        const uint32_t l = base + q * SCAN_THREADS + threadIdx.x;
        v += l < L ? k.l.counts[l] : 0u;
    }
    v = block_sum_256(v, s_red);
    if (threadIdx.x == 0) k.l.tile_sums[blockIdx.x] = v;
}

// Single-pass form (LOOKBACK): decoupled look-back (Merrill & Garland, "Single-
// pass parallel prefix scan with decoupled look-back", 2016).  A tile takes a
// ticket (so every tile it waits on has already started), publishes its
// aggregate, and warp 0 walks back over the predecessors' status words 32 at
// a time until it meets an inclusive prefix.  Status words carry a launch
// epoch, so they need no reset between launches; every wait is bounded
// (ERR_SCAN_WAIT, then the tile proceeds).
constexpr uint32_t SCAN_SPIN_LIMIT = 1u << 22;

__device__ __forceinline__ uint64_t ld_volatile_u64(const uint64_t* p) {
    return *((const volatile uint64_t*)p);
}

// the block's tile (its ticket) and the launch epoch, in shared memory
__device__ __forceinline__ void scan_take_ticket(const KArgs& k, uint32_t* s_tile, uint32_t* s_epoch) {
    if (threadIdx.x == 0) {
        // the epoch is read before the ticket: the last ticket advances it
        *s_epoch = *((volatile uint32_t*)&k.l.scan_state[0]);
        __threadfence();
        *s_tile = atomicAdd(&k.l.scan_state[1], 1u);
    }
    __syncthreads();
}

// Publishes the tile's aggregate, lets warp 0 walk back over the
// predecessors' status words to an inclusive prefix, publishes that, and
// returns the exclusive prefix (every thread calls it).  The block holding
// the last ticket resets the ticket counter and advances the epoch.
__device__ __forceinline__ uint32_t scan_lookback(const KArgs& k, uint32_t tile, uint32_t epoch_raw, uint32_t agg,
                                                  uint32_t* s_prefix) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t epoch = epoch_raw & 0x3FFFFFFFu;
    uint64_t* st = k.l.scan_status;
    const uint64_t ep = (uint64_t)epoch << 34;
    if (threadIdx.x == 0) *((volatile uint64_t*)&st[tile]) = ep | ((uint64_t)(tile == 0 ? 2u : 1u) << 32) | agg;
    if (warp == 0) {
        uint32_t acc = 0;
        if (tile > 0) {
            int32_t look = (int32_t)tile - 1;
            for (;;) {
                const int32_t idx = look - lane;
                uint64_t w = 0;
                uint32_t fl = 2u;  // before tile 0: an empty prefix
                for (uint32_t spin = 0;; ++spin) {
                    if (idx >= 0) {
                        w = ld_volatile_u64(&st[idx]);
                        fl = (uint32_t)(w >> 34) == epoch ? (uint32_t)(w >> 32) & 3u : 0u;
                    }
                    if (__all_sync(0xffffffffu, fl != 0u)) break;
                    if (spin >= SCAN_SPIN_LIMIT) {
                        if (lane == 0) atomicOr(k.err, ERR_SCAN_WAIT);
                        if (fl == 0u) {
                            fl = 2u;
                            w = 0;
                        }
                        break;
                    }
                }
                const unsigned pm = __ballot_sync(0xffffffffu, fl == 2u);
                const int first_p = pm ? __ffs(pm) - 1 : 31;
                uint32_t v = lane <= first_p ? (uint32_t)w : 0u;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                acc += v;
                if (pm) break;
                look -= 32;
            }
            if (lane == 0) *((volatile uint64_t*)&st[tile]) = ep | (2ull << 32) | (uint64_t)(acc + agg);
        }
        if (lane == 0) *s_prefix = acc;
    }
    __syncthreads();
    const uint32_t prefix = *s_prefix;
    if (threadIdx.x == 0 && tile == gridDim.x - 1) {
        k.l.scan_state[1] = 0u;
        __threadfence();
        k.l.scan_state[0] = epoch_raw + 1u;
    }
    return prefix;
}

template <int ITEMS, bool LOOKBACK>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan(KArgs k, uint32_t step, int with_hazard, int merge_q) {
    constexpr int TILE = SCAN_THREADS * ITEMS;
    __shared__ uint32_t s_red[SCAN_THREADS / 32];
    __shared__ uint32_t s_warp[SCAN_THREADS / 32];
    __shared__ uint32_t s_tile, s_epoch, s_prefix;
    const uint32_t L = k.l.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the single-pass form is the step's first kernel and decides; the
    // two-pass form reads the decision of its tile-sum kernel.  Without a
    // rebuild no ticket is taken and the cursors keep the ends of the step
    // before (no prefix, no cursor writes).
    const uint32_t t_step = k.clock->t0 + step;
    const bool rebuild = LOOKBACK ? csr_decide(k, t_step) : csr_rebuild(k, t_step);
    // merge_q 1: the location quarantines are merged at the steps whose
    // decisions wrote some (the day graph); 2: at every call
    merge_q = merge_q == 2 || (merge_q == 1 && k.l.build[3] == t_step);
    if (!rebuild && !with_hazard && !merge_q) return;
    uint32_t tile = blockIdx.x;
    if (LOOKBACK && rebuild) {
        scan_take_ticket(k, &s_tile, &s_epoch);
        tile = s_tile;
    }
    const uint32_t wbase = tile * TILE + (uint32_t)warp * (32 * ITEMS);
    uint32_t c[ITEMS], ex[ITEMS];
#pragma unroll
    for (int q = 0; q < ITEMS; ++q) {
        const uint32_t l = wbase + q * 32 + lane;
        c[q] = l < L ? k.l.counts[l] : 0u;
    }
    uint32_t prefix = 0;
    if (!rebuild) {
    } else if (LOOKBACK) {
        uint32_t mine = 0;
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) mine += c[q];
        prefix = scan_lookback(k, tile, s_epoch, block_sum_256(mine, s_red), &s_prefix);
    } else {
    // sum of the tiles before this one
    uint32_t pre = 0;
    {
        uint32_t p0 = 0, p1 = 0, p2 = 0, p3 = 0;
        uint32_t j = threadIdx.x;
        for (; j + 3 * SCAN_THREADS < tile; j += 4 * SCAN_THREADS) {
            p0 += k.l.tile_sums[j];
            p1 += k.l.tile_sums[j + SCAN_THREADS];
            p2 += k.l.tile_sums[j + 2 * SCAN_THREADS];
            p3 += k.l.tile_sums[j + 3 * SCAN_THREADS];
        }
        for (; j < tile; j += SCAN_THREADS) p0 += k.l.tile_sums[j];
        pre = p0 + p1 + p2 + p3;
    }
    prefix = block_sum_256(pre, s_red);
    }
    if (rebuild) {
        uint32_t carry = 0;
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
            uint32_t x = c[q];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            ex[q] = carry + x - c[q];
            carry += __shfl_sync(0xffffffffu, x, 31);
        }
        if (lane == 0) s_warp[warp] = carry;
        __syncthreads();
        uint32_t woff = 0;
        for (int q = 0; q < warp; ++q) woff += s_warp[q];
        const uint32_t base = prefix + woff;
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
            const uint32_t l = wbase + q * 32 + lane;
            if (l < L) k.l.cursor[l] = base + ex[q];
        }
    }
    const uint32_t dt = k.p.time_step;
    const float season = k.clock->season;
    const uint32_t V = k.m.n_variants;
    if (with_hazard) {
        // only the locations marked dirty (their sum or, with a nonzero sum,
        // their count changed) are read; their hazards are recomputed from
        // the persistent sums and their hazard-mask bits (sum nonzero)
        // rewritten.  Elsewhere hazards and mask bits stay as they are.
        uint32_t sws[ITEMS];
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) sws[q] = k.l.smask[(wbase + q * 32) >> 5];
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
            const uint32_t l = wbase + q * 32 + lane;
            const uint32_t wi = (wbase + q * 32) >> 5;
            const uint32_t sw = sws[q];
            if (!sw) continue;  // warp-uniform
            bool nz = false;
            if (l < L && ((sw >> lane) & 1u)) {
                // the location's fields load together with its sums
                const uint32_t rep = k.l.rep[l];
                const float w_l = k.l.infectiousness[l];
                const float k_f = k.r.k_f[rep];
                for (uint32_t v = 0; v < V; ++v) {
                    const size_t idx = (size_t)v * L + l;
                    const long long fix = (long long)k.l.sfix[idx];
                    float h = 0.0f, x = 0.0f;
                    if (fix != 0) {
                        h = psim_hazard_x(fix, c[q], k_f, w_l, season, dt, &x);
                        nz = true;
                    }
                    k.l.hazard[idx] = h;
                    if (k.adj.on) k.l.hazard_x[idx] = x;
                }
            }
            // one word per 32 locations (wbase is a multiple of 32)
            const unsigned nzw = __ballot_sync(0xffffffffu, nz);
            if (lane == 0) {
                k.l.hmask[wi] = (k.l.hmask[wi] & ~sw) | nzw;
                k.l.smask[wi] = 0u;
            }
        }
    }
    if (merge_q) {
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
            const uint32_t l = wbase + q * 32 + lane;
            if (l < L) {
                const uint32_t qq = k.l.qu_pending[l];
                if (qq) {
                    if (qq > k.l.quarantine_until[l]) k.l.quarantine_until[l] = qq;
                    k.l.qu_pending[l] = 0u;
                }
            }
        }
    }
}

// Thread-contiguous form of the two-pass scan (scan_mode 2): every thread
// owns 4 x Q consecutive locations, loaded and stored as 16-byte vectors; the
// in-thread prefix is serial, so a thread total needs one 5-step warp scan
// instead of one per item.  Same outputs as k_tile_sums + k_scan.
template <int Q>
__device__ __forceinline__ void load_counts4(const KArgs& k, uint32_t l0, uint32_t* c) {
    const uint32_t L = k.l.n;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const uint32_t l = l0 + 4u * q;
        if (l + 3u < L) {
            const uint4 v = *reinterpret_cast<const uint4*>(k.l.counts + l);
            c[4 * q] = v.x;
            c[4 * q + 1] = v.y;
            c[4 * q + 2] = v.z;
            c[4 * q + 3] = v.w;
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) c[4 * q + e] = l + e < L ? k.l.counts[l + e] : 0u;
        }
    }
}

template <int Q>
__global__ void __launch_bounds__(SCAN_THREADS) k_tile_sums_v(KArgs k, uint32_t step) {
    constexpr int PER = 4 * Q;
    __shared__ uint32_t s_red[SCAN_THREADS / 32];
    if (!csr_decide(k, k.clock->t0 + step)) return;  // the tile sums serve the rebuild only
    uint32_t c[PER];
    load_counts4<Q>(k, blockIdx.x * (SCAN_THREADS * PER) + threadIdx.x * PER, c);
    uint32_t v = 0;
#pragma unroll
    for (int e = 0; e < PER; ++e) v += c[e];
    v = block_sum_256(v, s_red);
    if (threadIdx.x == 0) k.l.tile_sums[blockIdx.x] = v;
}

// LOOKBACK: the single-pass form (decoupled look-back, as k_scan<ITEMS, true>):
// the step's only scan kernel, so it decides the rebuild and needs no tile
// sums; a step without a rebuild launches nothing else for its scan.
template <int Q, bool LOOKBACK>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_v(KArgs k, uint32_t step, int with_hazard, int merge_q) {
    constexpr int PER = 4 * Q;
    __shared__ uint32_t s_red[SCAN_THREADS / 32];
    __shared__ uint32_t s_warp[SCAN_THREADS / 32];
    __shared__ uint32_t s_tile, s_epoch, s_prefix;
    const uint32_t L = k.l.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // without a rebuild the cursors keep the ends of the step before, and
    // the counts are read at the flagged locations only
    const uint32_t t_step = k.clock->t0 + step;
    const bool rebuild = LOOKBACK ? csr_decide(k, t_step) : csr_rebuild(k, t_step);
    merge_q = merge_q == 2 || (merge_q == 1 && k.l.build[3] == t_step);
    if (!rebuild && !with_hazard && !merge_q) return;
    uint32_t tile = blockIdx.x;
    if (LOOKBACK && rebuild) {
        scan_take_ticket(k, &s_tile, &s_epoch);
        tile = s_tile;
    }
    const uint32_t l0 = tile * (SCAN_THREADS * PER) + threadIdx.x * PER;
    uint32_t c[PER] = {};
    if (rebuild) {
        load_counts4<Q>(k, l0, c);
        // in-thread exclusive prefix
        uint32_t ex[PER];
        uint32_t tot = 0;
#pragma unroll
        for (int e = 0; e < PER; ++e) {
            ex[e] = tot;
            tot += c[e];
        }
        // the sum of the tiles before this one
        uint32_t prefix;
        if (LOOKBACK) {
            prefix = scan_lookback(k, tile, s_epoch, block_sum_256(tot, s_red), &s_prefix);
        } else {
            uint32_t p0 = 0, p1 = 0, p2 = 0, p3 = 0;
            uint32_t j = threadIdx.x;
            for (; j + 3 * SCAN_THREADS < tile; j += 4 * SCAN_THREADS) {
                p0 += k.l.tile_sums[j];
                p1 += k.l.tile_sums[j + SCAN_THREADS];
                p2 += k.l.tile_sums[j + 2 * SCAN_THREADS];
                p3 += k.l.tile_sums[j + 3 * SCAN_THREADS];
            }
            for (; j < tile; j += SCAN_THREADS) p0 += k.l.tile_sums[j];
            prefix = block_sum_256(p0 + p1 + p2 + p3, s_red);
        }
        // the warp and block offsets
        uint32_t x = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        uint32_t woff = 0;
        for (int q = 0; q < warp; ++q) woff += s_warp[q];
        const uint32_t base = prefix + woff + x - tot;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const uint32_t l = l0 + 4u * q;
            if (l + 3u < L) {
                *reinterpret_cast<uint4*>(k.l.cursor + l) =
                    make_uint4(base + ex[4 * q], base + ex[4 * q + 1], base + ex[4 * q + 2], base + ex[4 * q + 3]);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (l + e < L) k.l.cursor[l + e] = base + ex[4 * q + e];
            }
        }
    }
    if (with_hazard) {
        const uint32_t dt = k.p.time_step;
        const float season = k.clock->season;
        const uint32_t V = k.m.n_variants;
        // PER consecutive locations lie in one mask word (PER divides 32);
        // only the dirty ones are read (see k_scan)
        const uint32_t wi = l0 >> 5;
        const uint32_t sw = k.l.smask[wi];
        const uint32_t mine = (sw >> (l0 & 31u)) & ((PER == 32) ? 0xFFFFFFFFu : ((1u << PER) - 1u));
        uint32_t nzb = 0;  // my dirty locations whose sum is nonzero, as bits of the word
        if (mine) {
#pragma unroll
            for (int e = 0; e < PER; ++e) {
                if (!((mine >> e) & 1u)) continue;
                const uint32_t l = l0 + e;
                if (l >= L) continue;
                // the location's fields load together with its sums
                const uint32_t rep = k.l.rep[l];
                const float w_l = k.l.infectiousness[l];
                const uint32_t n_l = rebuild ? c[e] : k.l.counts[l];
                const float k_f = k.r.k_f[rep];
                for (uint32_t v = 0; v < V; ++v) {
                    const size_t idx = (size_t)v * L + l;
                    const long long fix = (long long)k.l.sfix[idx];
                    float h = 0.0f, xx = 0.0f;
                    if (fix != 0) {
                        h = psim_hazard_x(fix, n_l, k_f, w_l, season, dt, &xx);
                        nzb |= 1u << ((l0 & 31u) + e);
                    }
                    k.l.hazard[idx] = h;
                    if (k.adj.on) k.l.hazard_x[idx] = xx;
                }
            }
        }
        // the word's bits from the 32 / PER consecutive threads that share it
#pragma unroll
        for (int o = 1; o < 32 / PER; o <<= 1) nzb |= __shfl_xor_sync(0xffffffffu, nzb, o);
        if ((l0 & 31u) == 0u && sw) {
            k.l.hmask[wi] = (k.l.hmask[wi] & ~sw) | nzb;
            k.l.smask[wi] = 0u;
        }
    }
    if (merge_q) {
#pragma unroll
        for (int e = 0; e < PER; ++e) {
            const uint32_t l = l0 + e;
            if (l < L) {
                const uint32_t qq = k.l.qu_pending[l];
                if (qq) {
                    if (qq > k.l.quarantine_until[l]) k.l.quarantine_until[l] = qq;
                    k.l.qu_pending[l] = 0u;
                }
            }
        }
    }
}

// CSR scatter and/or infection draw of one step.
__global__ void __launch_bounds__(256) k_scatter_draw(KArgs k, uint32_t step, int scatter, int draw) {
    __shared__ double s_grad[GRAD_N];
    grad_begin(k, s_grad);
    const uint32_t N = k.a.n, L = k.l.n;
    const uint32_t t = k.clock->t0 + step;
    const bool rebuild = csr_rebuild(k, t);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < N; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool act = i < N;
        double term = 0.0;
        const uint32_t loc = act ? k.a.location[i] : NONE;
        const bool ok = act && loc < L;
        bool hz = false;
        const float h0 = (draw && ok) ? hazard_at(k, loc, &hz) : 0.0f;
        if (scatter) {
            const uint32_t pos = take_slot(k, ok, loc, rebuild);
            if (ok) store_slot(k, pos, i);
        }
        if (ok && draw && hz) term = draw_agent(k, i, loc, t, h0, s_grad);
        if (k.track_expected) add_expected(k, act, i, term);
    }
    grad_end(k, s_grad);
}

// ---------------------------------------------------------------------------
// The day graph's step kernel.  One launch per timestep t (step s of the day),
// a persistent grid (every block resident; see launch_step) whose phases are
// separated by grid barriers only where one phase needs another's results:
//   rebuild   only when agents took new locations for t (or a rebuild is
//             pending): the locations with a nonzero sum listed and their
//             segments reserved | every agent at a listed location takes a
//             slot, which keeps its id, its susceptibility x age-band factor
//             of every variant and its location.  The step's location
//             quarantine writes are merged here too (or alone when there were
//             some but no rebuild).
//   draw      every listed entry, one per thread: the location's infection
//             ratio from its sum and the agent's draws (LocationsList::
//             infectAgents, locationList.h:233-310); the infections' sum
//             changes are applied once every draw of t is done
//   decide    only when some agent decides at s + 1 (or everyone at the
//             curfew step): the block queues its own agents that decide |
//             doMovement of the queued agents for s + 1 (work segments taken
//             in turn) and the histogram and sum deltas of their moves
// A step at which nobody takes a new location and nobody decides next runs
// the draw alone, without a barrier: its cost is the listed entries, not the
// whole population.

// Grid barrier of the persistent step kernel: the last block to arrive
// resets the count and advances the generation the others wait on (a
// two-level arrival, 8 groups then the grid, measured slower: the second
// atomic round trip costs more than the serialized arrivals it saves).
// Every wait is bounded: on expiry the block records ERR_BARRIER and returns
// false, and every later barrier and step kernel returns at once, so a
// failure ends in an error report, never a hang.  The block's writes reach
// the other blocks through the arrival (release: the block's threads' writes
// are ordered before it by the __syncthreads before) and the generation read
// (acquire).
constexpr uint32_t BARRIER_SPIN_LIMIT = 1u << 24;
__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t atom_add_acq_rel_gpu(uint32_t* p, uint32_t x) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(x) : "memory");
    return old;
}
__device__ __forceinline__ void st_relaxed_gpu(uint32_t* p, uint32_t x) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(x) : "memory");
}
__device__ __forceinline__ bool grid_barrier(const KArgs& k, bool* s_ok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        bool ok = (ld_acquire_gpu(k.err) & ERR_BARRIER) == 0;
        if (ok) {
            const uint32_t gen = ld_acquire_gpu(&k.l.bar[1]);
            const uint32_t arrived = atom_add_acq_rel_gpu(&k.l.bar[0], 1u) + 1u;
            if (arrived == gridDim.x) {
                st_relaxed_gpu(&k.l.bar[0], 0u);
                atom_add_acq_rel_gpu(&k.l.bar[1], 1u);
            } else {
                uint32_t spins = 0;
                while (ld_acquire_gpu(&k.l.bar[1]) == gen) {
                    if (++spins > BARRIER_SPIN_LIMIT) {
                        atomicOr(k.err, ERR_BARRIER);
                        ok = false;
                        break;
                    }
                    __nanosleep(32);
                }
            }
        }
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok;
}

// Slot data of the agent list: csr_agents[pos] = agent, slot_su[v][pos] =
// its susceptibility to variant v times its age band's factor (the product
// the draw compares with), written when the list is rebuilt and by the draw
// that infects the agent.
__device__ __forceinline__ void slot_fill(const KArgs& k, uint32_t pos, uint32_t i) {
    const uint32_t N = k.a.n;
    if (pos >= N) {
        atomicOr(k.err, ERR_LOCATION);
        return;
    }
    k.l.csr_agents[pos] = i;
    const float sigma = k.p.sigma_band[k.a.band[i]];
    for (uint32_t v = 0; v < k.m.n_variants; ++v)
        k.l.slot_su[(size_t)v * N + pos] = k.a.susceptible[(size_t)v * N + i] * sigma;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    uint32_t tot = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) tot += s_red[q];
    __syncthreads();
    return tot;
}

// the step's location quarantine writes into quarantine_until (grid-stride)
__device__ __forceinline__ void merge_quarantine(const KArgs& k) {
    const uint32_t L = k.l.n;
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < L; l += gridDim.x * blockDim.x) {
        const uint32_t qq = k.l.qu_pending[l];
        if (qq) {
            if (qq > k.l.quarantine_until[l]) k.l.quarantine_until[l] = qq;
            k.l.qu_pending[l] = 0u;
        }
    }
}

// Exclusive prefix of v over the block's threads in thread order; *total
// receives the block's sum.  Every thread calls it.
__device__ __forceinline__ uint32_t block_scan_excl(uint32_t v, uint32_t* s_red, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_red[warp] = x;
    __syncthreads();
    uint32_t woff = 0, tot = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
        const uint32_t wq = s_red[q];
        if (q < warp) woff += wq;
        tot += wq;
    }
    __syncthreads();
    *total = tot;
    return woff + x - v;
}

// the set bits of mask word w whose location has a nonzero sum of some
// variant (returned) and the agents at those locations (*agents); the loads of
// four set bits at a time are issued together
__device__ __forceinline__ uint32_t nonzero_sum_bits(const KArgs& k, const unsigned long long* sums, uint32_t hm,
                                                     uint32_t w, uint32_t* agents) {
    const uint32_t L = k.l.n, V = k.m.n_variants;
    uint32_t keep = 0, rest = hm, cnt = 0;
    while (rest) {
        uint32_t b[4], l[4];
        unsigned long long f[4];
        uint32_t c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            b[u] = rest ? (uint32_t)(__ffs(rest) - 1) : 32u;
            if (rest) rest &= rest - 1u;
            l[u] = b[u] < 32u ? w * 32u + b[u] : NONE;
            const bool in = l[u] < L;
            f[u] = in ? sums[l[u]] : 0ull;
            c[u] = in ? k.l.counts[l[u]] : 0u;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (l[u] >= L) continue;
            bool nz = f[u] != 0ull;
            for (uint32_t v = 1; v < V && !nz; ++v) nz = sums[(size_t)v * L + l[u]] != 0ull;
            if (nz) {
                keep |= 1u << b[u];
                cnt += c[u];
            }
        }
    }
    *agents = cnt;
    return keep;
}

// Rebuild of the agent list.  Only the locations with a nonzero sum are
// listed, because the draws of every step until the next rebuild need no
// other location: until then no other location gains a nonzero sum (nobody
// moves, since a move makes the next step rebuild, and a draw infects only
// agents at a location with a nonzero sum).  The hazard mask is a superset of
// those locations (every kernel that adds an infectious term sets the bit at
// once); the listing clears the bits of the locations whose sums are zero
// again.  The listed locations' agents fill the first *n_listed slots, each
// slot with its agent, susceptibility products and location; the order of
// the locations' segments is the order in which their chunks reserved them
// (the draws do not depend on it).  In two parts between grid barriers:
// 1 (listing): per chunk of 256 mask words of the block's range, the listed
// locations, one atomic on the listing counter reserving the chunk's slots,
// each location's first slot (cursor); 2 (slots): every agent at a listed
// location takes a slot (one returning atomic on the location's cursor, or
// one per location and warp with agg_slot).  Returns false when a barrier
// expired.
__device__ bool phase_rebuild(const KArgs& k, const unsigned long long* sums, uint32_t* s_red, bool* s_ok,
                              uint32_t tl, uint32_t* s_base, uint32_t* n_listed) {
    const uint32_t L = k.l.n, N = k.a.n;
    const uint32_t n_words = (L + 31u) >> 5;
    const uint32_t per = (n_words + gridDim.x - 1) / gridDim.x;
    const uint32_t wb = min(n_words, blockIdx.x * per), we = min(n_words, wb + per);
    // 1
    uint32_t locs = 0, agents = 0;
    for (uint32_t c0 = wb; c0 < we; c0 += blockDim.x) {  // block-uniform trips
        const uint32_t w = c0 + threadIdx.x;
        uint32_t hm = w < we ? k.l.hmask[w] : 0u;
        uint32_t wc = 0;
        if (hm) {
            const uint32_t keep = nonzero_sum_bits(k, sums, hm, w, &wc);
            if (keep != hm) k.l.hmask[w] = keep;
            hm = keep;
        }
        uint32_t chunk = 0;
        const uint32_t ex = block_scan_excl(wc, s_red, &chunk);
        if (chunk == 0) continue;  // block-uniform
        if (threadIdx.x == 0) *s_base = atomicAdd(&k.l.bar[BAR_LISTED], chunk);
        __syncthreads();
        uint32_t run = *s_base + ex;
        __syncthreads();
        locs += __popc(hm);
        agents += chunk;
        while (hm) {
            const uint32_t l = w * 32u + (uint32_t)(__ffs(hm) - 1);
            hm &= hm - 1u;
            if (l < L) {
                k.l.cursor[l] = run;
                run += k.l.counts[l];
            }
        }
    }
    if (k.prof) {
        const uint32_t nl = block_sum(locs, s_red);
        if (threadIdx.x == 0 && (nl | agents)) {
            atomicAdd(&k.prof[PROF_LISTED_LOCATIONS], (unsigned long long)nl);
            atomicAdd(&k.prof[PROF_LISTED_AGENTS], (unsigned long long)agents);
        }
    }
    if (!grid_barrier(k, s_ok)) return false;
    prof_mark(k, tl + 1);
    *n_listed = k.l.bar[BAR_LISTED];  // every block's reservation is in
    // 3: four consecutive agents per thread (one 16-byte load of their
    // locations), two quads in flight
    const bool one = k.m.n_variants == 1;
    const uint32_t quads = (N + 3u) >> 2;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t q0 = blockIdx.x * blockDim.x; q0 < quads; q0 += 2u * stride) {  // warp-uniform trips
        uint32_t loc[8];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t q = q0 + (uint32_t)h * stride + threadIdx.x;
            const uint32_t i0 = q * 4u;
            if (i0 + 3u < N) {
                const uint4 v = *reinterpret_cast<const uint4*>(k.a.location + i0);
                loc[4 * h + 0] = v.x;
                loc[4 * h + 1] = v.y;
                loc[4 * h + 2] = v.z;
                loc[4 * h + 3] = v.w;
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) loc[4 * h + u] = i0 + u < N ? k.a.location[i0 + u] : NONE;
            }
        }
        uint32_t lw[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) lw[u] = loc[u] < L ? k.l.hmask[loc[u] >> 5] : 0u;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const uint32_t i = (q0 + (uint32_t)(u >> 2) * stride + threadIdx.x) * 4u + (uint32_t)(u & 3);
            const bool ok = loc[u] < L && ((lw[u] >> (loc[u] & 31u)) & 1u);
            float su = 0.0f;
            if (ok && one) su = k.a.susceptible[i] * k.p.sigma_band[k.a.band[i]];
            const uint32_t pos = take_slot(k, ok, loc[u], true);
            if (!ok) continue;
            if (!one) {
                slot_fill(k, pos, i);
            } else if (pos < N) {
                k.l.csr_agents[pos] = i;
                k.l.slot_su[pos] = su;
            } else {
                atomicOr(k.err, ERR_LOCATION);
            }
            if (pos < N) k.l.slot_loc[pos] = loc[u];
        }
    }
    if (!grid_barrier(k, s_ok)) return false;
    // every block has read the listing counter: block 0 keeps the count for
    // the steps until the next rebuild and starts the counter at 0 for it
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        k.l.build[5] = *n_listed;
        k.l.bar[BAR_LISTED] = 0u;
    }
    return true;
}

// expected-infection accumulation of the draws: one atomic per replica
// present in the warp (warp-collective; rep given, not looked up)
__device__ __forceinline__ void add_expected_rep(const KArgs& k, bool act, uint32_t rep, double term) {
    const unsigned am = __ballot_sync(0xffffffffu, act && term != 0.0);
    if (!(act && term != 0.0)) return;
    const unsigned peers = __match_any_sync(am, rep);
    const int leader = __ffs(peers) - 1;
    unsigned rest = peers;
    double tot = 0.0;
    while (rest) {
        const int src = __ffs(rest) - 1;
        tot += __shfl_sync(peers, term, src);
        rest &= rest - 1;
    }
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(&k.r.expected[rep], tot);
}

// DynamicPPState::gotInfected (dynamicPPState.cpp:235-244) and the agent's
// statistics (locationList.h:283-304)
__device__ __forceinline__ void infect_agent(const KArgs& k, uint32_t i, uint32_t v, uint32_t loc, uint32_t t) {
    k.a.state[i] = (int8_t)k.m.first_infected;
    k.a.variant[i] = (uint8_t)v;
    k.a.days[i] = -2;
    update_meta(k, i);
    k.a.st_infected_ts[i] = t;
    k.a.st_infected_count[i] = k.a.st_infected_count[i] + 1;
    k.a.st_infected_loc[i] = loc;
    k.a.st_worst_state[i] = (int8_t)k.m.first_infected;
    k.a.st_worst_ts[i] = t;
    k.a.st_variant_mask[i] |= 1u << v;
}

// U < p for the 53-bit uniform U = K * 2^-53 of the words (a, b)
// (psim_u01_from) and a float probability p > 0, in integers: p * 2^53 is
// exact in float (a power-of-two scaling of a normal or subnormal p), and
// K < p * 2^53 holds exactly when K < ceil(p * 2^53).
__device__ __forceinline__ bool u01_below(uint32_t a, uint32_t b, float p) {
    if (p >= 1.0f) return true;
    const unsigned long long K = ((unsigned long long)(a >> 5) << 26) | (unsigned long long)(b >> 6);
    return K < __float2ull_ru(p * 9007199254740992.0f);
}

// Infection ratio of variant v at location loc (count cnt, weight wl,
// replica coefficient kf) from the location's fixed-point sum as the step
// started: the formula the scans evaluate (psim_hazard_x), so every entry of
// a location computes the same value.  x receives its argument.
__device__ __forceinline__ float entry_hazard(const KArgs& k, const unsigned long long* sums, uint32_t loc, uint32_t v,
                                              uint32_t cnt, float wl, float kf, float season, uint32_t dt, float* x) {
    const long long fix = (long long)sums[(size_t)v * k.l.n + loc];
    *x = 0.0f;
    return fix != 0 ? psim_hazard_x(fix, cnt, kf, wl, season, dt, x) : 0.0f;
}

// The sums of the step kernel are kept twice: step s of the day reads copy
// s & 1 (sfix, sfix_b) as the step started, and every change of step s goes
// to the other copy, which step s + 1 reads.  The decisions change both
// copies (they come after the step's draws); an infection changes the other
// copy at once and is listed (list s % 3), and step s + 1 applies the list to
// the copy it does not read, so that copy is complete when step s + 2 reads it
// (apply_previous_infections).
__device__ __forceinline__ unsigned long long* sums_read(const KArgs& k, uint32_t step) {
    return (step & 1u) ? k.l.sfix_b : k.l.sfix;
}
__device__ __forceinline__ unsigned long long* sums_next(const KArgs& k, uint32_t step) {
    return (step & 1u) ? k.l.sfix : k.l.sfix_b;
}
__device__ __forceinline__ void add_infection_change(const KArgs& k, unsigned long long* sums, uint32_t loc,
                                                     float inf0, uint32_t var0, float inf, uint32_t var) {
    const uint32_t L = k.l.n;
    const long long q0 = inf0 > 0.0f ? __float2ll_rn(inf0 * PSIM_FIX_SCALE_F) : 0ll;
    const long long q1 = inf > 0.0f ? __float2ll_rn(inf * PSIM_FIX_SCALE_F) : 0ll;
    if (q0) atomicAdd(&sums[(size_t)var0 * L + loc], (unsigned long long)(-q0));
    if (q1) {
        atomicAdd(&sums[(size_t)var * L + loc], (unsigned long long)q1);
        mark_hazardous(k, loc);
    }
}
__device__ __forceinline__ void record_infection(const KArgs& k, uint32_t step, uint32_t loc, float inf0,
                                                 uint32_t var0, float inf, uint32_t var) {
    add_infection_change(k, sums_next(k, step), loc, inf0, var0, inf, var);
    const uint32_t list = step % 3u;
    const uint32_t j = atomicAdd(&k.l.bar[BAR_INFECTIONS + list], 1u);
    if (j < k.a.n)
        k.l.inf_pending[(size_t)list * k.a.n + j] =
            make_uint4(loc, __float_as_uint(inf0), __float_as_uint(inf), var0 | (var << 8));
    else
        atomicOr(k.err, ERR_AGENT_LIST);
}

// A replica's infection coefficient, seed and first agent.
struct RepConst {
    float kf;
    uint32_t off;
    unsigned long long seed;
};
__device__ __forceinline__ RepConst rep_const(const KArgs& k, uint32_t rep) {
    RepConst c;
    c.kf = k.r.k_f[rep];
    c.off = k.r.agent_off[rep];
    c.seed = k.r.seed[rep];
    return c;
}

// The draws of one agent-list entry: the agent in slot pos at location loc
// of replica rep (count cnt, weight wl).  Returns the sum of min(1, p) over
// its draws when expected infections are tracked (else 0).  An agent that is
// infected updates its slot's susceptibility products (read by no other
// entry) and records its location's sum change for the next steps.
__device__ __forceinline__ double draw_entry(const KArgs& k, const unsigned long long* sums, uint32_t step,
                                             uint32_t pos, uint32_t i, uint32_t loc, uint32_t rep, uint32_t cnt,
                                             float wl, float su0, const RepConst& rc, float season, uint32_t t,
                                             double* s_grad, bool* any_h) {
    const uint32_t N = k.a.n, V = k.m.n_variants, dt = k.p.time_step;
    const float kf = rc.kf;
    const unsigned long long seed = rc.seed;
    const uint32_t li = i - rc.off;
    double term = 0.0;
    bool infected = false;
    float inf0 = 0.0f, sigma = 0.0f;
    uint32_t var0 = 0;
    for (uint32_t v = 0; v < V; ++v) {
        float x;
        const float h = entry_hazard(k, sums, loc, v, cnt, wl, kf, season, dt, &x);
        if (!(h > 0.0f)) continue;
        *any_h = true;
        if (!k.r.variant_active[rep * V + v]) continue;
        // after an infection the later variants read the agent's new
        // susceptibility (what the slot then gets)
        float s_eff;
        if (!infected)
            s_eff = v == 0 ? su0 : k.l.slot_su[(size_t)v * N + pos];
        else
            s_eff = k.a.susceptible[(size_t)v * N + i] * sigma;
        if (!(s_eff > 0.0f)) continue;
        const float pf = h * s_eff;
        if (k.track_expected) term += pf < 1.0f ? (double)pf : 1.0;
        if (k.adj.on && pf < 1.0f)
            adjoint_terms(k, i, loc, v, rep, h, k.a.susceptible[(size_t)v * N + i], s_eff, s_grad, x);
        // the uniform of the stream (seed, agent, t, infection + v), as
        // psim_u01_once draws it
        psim_ctr4 c;
        c.v[0] = li;
        c.v[1] = t;
        c.v[2] = PSIM_PHASE_INFECT + v;
        c.v[3] = 0u;
        const psim_ctr4 o = psim_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        if (u01_below(o.v[0], o.v[1], pf)) {
            if (!infected) {
                inf0 = k.a.infectious[i];
                var0 = inf0 > 0.0f ? k.a.variant[i] : 0u;
                sigma = k.p.sigma_band[k.a.band[i]];
                infected = true;
            }
            infect_agent(k, i, v, loc, t);
        }
    }
    if (infected) {
        for (uint32_t v = 0; v < V; ++v) k.l.slot_su[(size_t)v * N + pos] = k.a.susceptible[(size_t)v * N + i] * sigma;
        const float inf = k.a.infectious[i];
        const uint32_t var = inf > 0.0f ? k.a.variant[i] : 0u;
        const long long q0 = inf0 > 0.0f ? __float2ll_rn(inf0 * PSIM_FIX_SCALE_F) : 0ll;
        const long long q1 = inf > 0.0f ? __float2ll_rn(inf * PSIM_FIX_SCALE_F) : 0ll;
        if (q0 != q1 || var0 != var) record_infection(k, step, loc, inf0, var0, inf, var);
    }
    return term;
}

// The draw phase: every entry of the agent list (the agents at the locations
// the last rebuild listed, build[5] of them), one per thread, slots in order
// (coalesced loads of the slot's location, agent and susceptibility
// products).  Each entry evaluates its location's ratio from the location's
// sum, count and weight (the same inputs give the same value at every entry)
// and draws from the agent's Philox stream (seed, agent, t).  The work is the
// listed entries, spread evenly over the grid, whatever the number of
// locations.
// First-trip slot of a thread (its slot, agent and variant-0 product),
// loaded by the step's prologue with the step's words when the step does not
// rebuild (its slots are then the last rebuild's).
struct SlotPre {
    uint32_t loc, i;
    float su0;
    bool ok;
};
__device__ __forceinline__ SlotPre slot_pre(const KArgs& k, bool draws) {
    SlotPre p{NONE, NONE, 0.0f, false};
    const uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (draws && pos < k.a.n) {  // issued before the step's words arrive
        p.loc = k.l.slot_loc[pos];
        p.i = k.l.csr_agents[pos];
        p.su0 = k.l.slot_su[pos];
        p.ok = true;
    }
    return p;
}

__device__ void phase_draw(const KArgs& k, uint32_t step, uint32_t t, uint32_t n_listed, float season,
                           const SlotPre& pre, double* s_grad, uint32_t* n_entries, uint32_t* n_hazard) {
    const unsigned long long* sums = sums_read(k, step);
    const uint32_t L = k.l.n, N = k.a.n;
    const uint32_t stride = gridDim.x * blockDim.x;
    const bool one_rep = k.r.n == 1;
    const RepConst rc0 = rep_const(k, 0);
    uint32_t entries = 0, hazard = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n_listed; base += stride) {  // block-uniform trips
        const uint32_t pos = base + threadIdx.x;
        bool act = pos < n_listed && pos < N;
        uint32_t loc = NONE, i = NONE, rep = 0, cnt = 0;
        float wl = 0.0f, su0 = 0.0f;
        if (act) {
            const bool first = base == blockIdx.x * blockDim.x && pre.ok;
            loc = first ? pre.loc : k.l.slot_loc[pos];
            i = first ? pre.i : k.l.csr_agents[pos];
            su0 = first ? pre.su0 : k.l.slot_su[pos];
            if (loc >= L || i >= N) {
                atomicOr(k.err, ERR_AGENT_LIST);
                act = false;
            } else {
                cnt = k.l.counts[loc];
                wl = k.l.infectiousness[loc];
                rep = one_rep ? 0u : k.l.rep[loc];
            }
        }
        bool any_h = false;
        const double term =
            act ? draw_entry(k, sums, step, pos, i, loc, rep, cnt, wl, su0, one_rep ? rc0 : rep_const(k, rep), season, t,
                             s_grad, &any_h)
                : 0.0;
        entries += act ? 1u : 0u;
        hazard += any_h ? 1u : 0u;
        if (k.track_expected) add_expected_rep(k, act, rep, term);
    }
    *n_entries += entries;
    *n_hazard += hazard;
}

// The infections of step s - 1 into the copy of the sums that step s does not
// read (every thread of the grid takes a share; list (s - 1) % 3, complete
// since the kernel of step s - 1 ended).  Block 0 also empties list
// (s + 1) % 3, applied by step s - 1 and next written by step s + 1.
__device__ __forceinline__ void apply_previous_infections(const KArgs& k, uint32_t step) {
    if (blockIdx.x == 0 && threadIdx.x == 0) k.l.bar[BAR_INFECTIONS + (step + 1u) % 3u] = 0u;
    if (step == 0) return;  // the day's first step: the sums are afresh
    const uint32_t list = (step + 2u) % 3u;
    const uint32_t n = min(k.l.bar[BAR_INFECTIONS + list], k.a.n);
    unsigned long long* sums = sums_next(k, step);
    // from the grid's last block down: the draws fill the first blocks
    const uint32_t g = (gridDim.x - 1u - blockIdx.x) * blockDim.x + threadIdx.x;
    for (uint32_t j = g; j < n; j += gridDim.x * blockDim.x) {
        const uint4 e = k.l.inf_pending[(size_t)list * k.a.n + j];
        add_infection_change(k, sums, e.x, __uint_as_float(e.y), e.w & 0xFFu, __uint_as_float(e.z), (e.w >> 8) & 0xFFu);
    }
}

// The block's agents that decide at s1, in its own segment of the work list
// (shared-memory counter: no global contention).  Reads one word per agent:
// four consecutive agents per thread (one 16-byte load), two quads in flight.
__device__ __forceinline__ uint32_t phase_queue(const KArgs& k, uint32_t s1, uint32_t cap, uint32_t* s_cnt) {
    if (threadIdx.x == 0) *s_cnt = 0u;
    __syncthreads();
    const uint32_t N = k.a.n;
    const bool curfew_now = k.p.enable_curfew && k.p.curfew_begin == s1;
    const uint32_t t1 = k.clock->t0 + s1;
    const uint32_t quads = (N + 3u) >> 2;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t* seg = k.a.worklist + (size_t)blockIdx.x * cap;
    const int lane = threadIdx.x & 31;
    for (uint32_t q0 = blockIdx.x * blockDim.x; q0 < quads; q0 += 2u * stride) {  // warp-uniform trips
        uint32_t m[8];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t i0 = (q0 + (uint32_t)h * stride + threadIdx.x) * 4u;
            if (i0 + 3u < N) {
                const uint4 v = *reinterpret_cast<const uint4*>(k.a.move_at + i0);
                m[4 * h + 0] = v.x;
                m[4 * h + 1] = v.y;
                m[4 * h + 2] = v.z;
                m[4 * h + 3] = v.w;
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) m[4 * h + u] = i0 + u < N ? k.a.move_at[i0 + u] : t1 + 1u;
            }
        }
        // each quad's deciders in agent order: the warp's 128 agents of the
        // first quad, then those of the second
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t i0 = (q0 + (uint32_t)h * stride + threadIdx.x) * 4u;
            uint32_t flags = 0;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i0 + u < N && (curfew_now || m[4 * h + u] == t1)) flags |= 1u << u;
            const uint32_t mine = __popc(flags);
            uint32_t inc = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += y;
            }
            const uint32_t wtot = __shfl_sync(0xffffffffu, inc, 31);
            if (wtot) {
                uint32_t basew = 0;
                if (lane == 31) basew = atomicAdd(s_cnt, wtot);
                uint32_t pos = __shfl_sync(0xffffffffu, basew, 31) + inc - mine;
                while (flags) {
                    const int u = __ffs(flags) - 1;
                    flags &= flags - 1u;
                    seg[pos++] = i0 + (uint32_t)u;
                }
            }
        }
    }
    __syncthreads();
    return *s_cnt;
}

// doMovement of the agents the block queued for s1 (its own segment, whose
// count the queue left in shared memory: every block starts its decisions at
// the same barrier, so handing segments out by ticket balanced nothing), then
// the histogram and sum deltas of the agents that took a new location.
__device__ void phase_decide(const KArgs& k, uint32_t step, uint32_t cap, uint32_t* s_mm, const uint32_t* s_cnt) {
    const uint32_t s1 = step + 1;
    const StepClock c = step_clock(k, s1);
    bool moved = false;
    {
        uint32_t n = *s_cnt;
        if (n > cap) {
            if (threadIdx.x == 0) atomicOr(k.err, ERR_AGENT_LIST);
            n = 0;
        }
        const uint32_t* seg = k.a.worklist + (size_t)blockIdx.x * cap;
        const uint32_t trips = (n + blockDim.x - 1) / blockDim.x;  // uniform per block
        for (uint32_t it = 0; it < trips; ++it) {
            const uint32_t j = it * blockDim.x + threadIdx.x;
            bool act = j < n;
            uint32_t loc0 = NONE, loc = NONE, var = 0;
            float inf = 0.0f;
            const uint32_t i = act ? seg[j] : NONE;
            if (act && i >= k.a.n) {
                atomicOr(k.err, ERR_AGENT_LIST);
                act = false;
            }
            if (act) {
                // every queued agent decides: its inputs load at once
                DecisionIn d;
                decision_in(k, i, d);
                const uint32_t m0 = k.a.move_at[i];
                const uint32_t vr = k.a.variant[i];
                loc0 = d.loc;
                inf = d.inf;
                if (inf > 0.0f) var = vr;
                loc = move_agent(k, i, c, m0 - c.t, s_mm, &d, loc0);
            }
            moved |= count_agent_delta(k, act, loc0, loc, inf, var, inf, var);
        }
    }
    publish_moved(k, moved, c.t);
}

// Block-shared scratch of the step kernel.
struct StepShared {
    double grad[GRAD_N];
    uint32_t mm[MOVE_MASK_WORDS];
    uint32_t red[32];
    uint32_t cnt, base;
    bool ok;
};

// One timestep of the step kernel (see the section comment); false when a
// grid barrier expired (the kernel then ends).  cap = the work-list segment
// size of a block.
__device__ __forceinline__ bool step_body(const KArgs& k, uint32_t step, uint32_t phases, uint32_t cap,
                                          StepShared& sh) {
    const uint32_t tl = PROF_T + PROF_TW * step;  // the step's timeline slots (profiled graph)
    prof_enter(k, tl);
    // the words the step's phases start from, loaded together: the error
    // flags, the clock, the rebuild words (a block that starts after block 0
    // turned BUILD_PENDING into t decides the same), the step of the last
    // quarantine writes, the decision-mask word of the next step (the
    // decisions of this step mark later steps only)
    const uint32_t err0 = *((volatile uint32_t*)k.err);
    const uint32_t t0 = k.clock->t0;
    const float season = k.clock->season;
    const uint32_t moved = k.l.build[0], force = k.l.build[1], q_step = k.l.build[3];
    uint32_t n_listed = k.l.build[5];  // the last rebuild's entries (this step's if it rebuilds)
    const uint32_t s1 = step + 1;
    const uint32_t mm_word = s1 < k.spd ? k.a.move_mask[s1 >> 5] : 0u;
    // the first-trip slots of the draws, loaded with the words above; used
    // only when this launch does not rebuild them (moved / force as read)
    SlotPre pre = slot_pre(k, (phases & PH_DRAW) != 0);
    const uint32_t t = t0 + step;
    if ((phases & PH_REBUILD) && (moved == t || force == t || force == BUILD_PENDING)) pre.ok = false;
    if (err0 & ERR_BARRIER) return false;  // an earlier barrier expired
    if (phases & PH_REBUILD) {
        const bool rebuild = csr_decide_from(k, t, moved, force);
        if (rebuild) {
            if (k.prof && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&k.prof[PROF_REBUILDS], 1ull);
            if (!phase_rebuild(k, sums_read(k, step), sh.red, &sh.ok, tl, &sh.base, &n_listed)) return false;
            prof_mark(k, tl + 2);
        }
        // the step's location quarantine writes (decisions of step t)
        if (k.p.quarantine_policy > 1 && q_step == t) merge_quarantine(k);
    }
    if (phases & PH_DRAW) {
        apply_previous_infections(k, step);
        grad_begin(k, sh.grad);
        uint32_t entries = 0, hazard = 0;
        phase_draw(k, step, t, n_listed, season, pre, sh.grad, &entries, &hazard);
        if (k.prof) {
            entries = __reduce_add_sync(0xffffffffu, entries);
            hazard = __reduce_add_sync(0xffffffffu, hazard);
            if ((threadIdx.x & 31) == 0 && (entries | hazard)) {
                atomicAdd(&k.prof[PROF_DRAW_ENTRIES], (unsigned long long)entries);
                atomicAdd(&k.prof[PROF_DRAW_HAZARD], (unsigned long long)hazard);
            }
        }
        grad_end(k, sh.grad);
        prof_mark(k, tl + 3);
    }
    const bool decides = (k.p.enable_curfew && k.p.curfew_begin == s1) || ((mm_word >> (s1 & 31u)) & 1u) != 0;
    if ((phases & PH_DECIDE) && s1 < k.spd && decides) {
        mask_clear_shared(sh.mm);
        const uint32_t n = phase_queue(k, step + 1, cap, &sh.cnt);
        if (k.prof && threadIdx.x == 0) {
            if (n) atomicAdd(&k.prof[PROF_MOVERS], (unsigned long long)n);
            if (blockIdx.x == 0) atomicAdd(&k.prof[PROF_QUEUE_STEPS], 1ull);
        }
        prof_mark(k, tl + 4);
        // every draw and every block's queue before any decision
        if (!grid_barrier(k, &sh.ok)) return false;
        phase_decide(k, step, cap, sh.mm, &sh.cnt);
        mask_flush(k, sh.mm);
    }
    prof_mark(k, tl + 5);
    return true;
}

// The step kernel: timesteps step0 .. step0 + nsteps - 1, a grid barrier
// between two (the day graph launches it per timestep, or for the whole day
// with tuning variant 4).
__global__ void __launch_bounds__(256, 4) k_step(KArgs k, uint32_t step0, uint32_t nsteps, uint32_t phases,
                                                 uint32_t cap) {
    __shared__ StepShared sh;
    for (uint32_t j = 0; j < nsteps; ++j) {
        if (!step_body(k, step0 + j, phases, cap, sh)) return;
        if (j + 1 < nsteps && !grid_barrier(k, &sh.ok)) return;
    }
}

// Canonical CSR order (ascending agent id inside a location, the output of
// thrust::stable_sort_by_key): the final position of agent x in its segment is
// the number of agents of the segment with a smaller id.  O(sum n_l^2); used
// on demand only.  off = CSR offsets [L+1].
__global__ void k_canonical_rank(KArgs k, const uint32_t* off, uint32_t* tmp) {
    const uint32_t N = k.a.n;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
        const uint32_t x = k.l.csr_agents[j];
        const uint32_t l = k.a.location[x];
        const uint32_t b = off[l], e = off[l + 1];
        uint32_t cnt = 0;
        for (uint32_t q = b; q < e; ++q) cnt += k.l.csr_agents[q] < x;
        tmp[b + cnt] = x;
    }
}

// CSR offsets from the cursors after a complete scatter: cursor[l] = end of l.
__global__ void k_offsets_from_cursor(KArgs k, uint32_t* off) {
    const uint32_t L = k.l.n;
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l <= L; l += gridDim.x * blockDim.x)
        off[l] = l == 0 ? 0u : k.l.cursor[l - 1];
}

// ---------------------------------------------------------------------------
// Daily progression: Simulation::updateAgents (simulation.h:425-471),
// DynamicPPState::update (dynamicPPState.cpp:246-303),
// MultiBadMatrix::calculateNextState / selectNext (multiBadMatrix.cpp:9-31,120-125),
// LengthOfState::calculateDays (basicLengthAbstract.cpp:48-53).
// The transition tables are staged in shared memory.
struct ProgTables {
    const uint32_t* bad_begin;
    const uint32_t* bad_count;
    const uint32_t* neu_begin;
    const uint32_t* neu_count;
    const uint32_t* next;
    const float* chance;
};

__device__ int calc_days(const KArgs& k, uint32_t pid, uint32_t state, uint32_t v, psim_stream* rng) {
    const size_t idx = ((size_t)pid * k.m.n_states + state) * PSIM_MAX_STRAINS + v;
    if (k.m.len_avg[idx] == -1.0f) return -1;
    const uint32_t thr = k.m.len_thr[idx];
    const float mx = k.m.len_max[idx];
    int days = psim_geometric(rng, thr);
    while (mx < (float)days) days = psim_geometric(rng, thr);
    return days;
}

__device__ uint32_t select_next(const ProgTables& T, size_t ti, float scaling, psim_stream* rng, int* bad) {
    const uint32_t bb = T.bad_begin[ti], bc = T.bad_count[ti], nb = T.neu_begin[ti], nc = T.neu_count[ti];
    if (nc == 0) scaling = 1.0f;
    const double random = psim_u01(rng);
    double pre = 0.0, bad_sum = 0.0;
    for (uint32_t q = 0; q < bc; ++q) {
        float c = T.chance[bb + q] * scaling;
        pre += (double)c;
        if (random < pre) {
            *bad = 1;
            return T.next[bb + q];
        }
        bad_sum += (double)T.chance[bb + q];
    }
    double bad_scaling = 1.0 + ((bad_sum - pre) / (1.0 - bad_sum));
    if (bc == 0) bad_scaling = 1.0;
    uint32_t idx = 0;
    do {
        double c = (double)T.chance[nb + idx] * bad_scaling;
        pre += c;
        ++idx;
    } while (pre < random && idx < nc);
    idx--;
    *bad = 0;
    return T.next[nb + idx];
}

__global__ void __launch_bounds__(256) k_progress(KArgs k, uint32_t t, int staged) {
    extern __shared__ uint32_t smem[];
    const uint32_t nt = k.m.n_prog * k.m.n_states;
    ProgTables T;
    if (staged) {
        uint32_t* s = smem;
        uint32_t* bb = s;
        uint32_t* bc = bb + nt;
        uint32_t* nb = bc + nt;
        uint32_t* nc = nb + nt;
        uint32_t* nx = nc + nt;
        float* ch = (float*)(nx + k.m.n_trans);
        for (uint32_t j = threadIdx.x; j < nt; j += blockDim.x) {
            bb[j] = k.m.tr_bad_begin[j];
            bc[j] = k.m.tr_bad_count[j];
            nb[j] = k.m.tr_neu_begin[j];
            nc[j] = k.m.tr_neu_count[j];
        }
        for (uint32_t j = threadIdx.x; j < k.m.n_trans; j += blockDim.x) {
            nx[j] = k.m.tr_next[j];
            ch[j] = k.m.tr_chance[j];
        }
        __syncthreads();
        T = ProgTables{bb, bc, nb, nc, nx, ch};
    } else {
        T = ProgTables{k.m.tr_bad_begin, k.m.tr_bad_count, k.m.tr_neu_begin, k.m.tr_neu_count, k.m.tr_next,
                       k.m.tr_chance};
    }
    const uint32_t N = k.a.n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        int16_t days = k.a.days[i];
        if (days > 0) {  // the common case: count down
            k.a.days[i] = days - 1;
            continue;
        }
        if (days != -2 && days != 0) continue;
        const uint32_t rep = k.a.rep[i];
        psim_stream rng;
        psim_stream_init(&rng, k.r.seed[rep], i - k.r.agent_off[rep], t, PSIM_PHASE_PROGRESS);
        const uint32_t v = k.a.variant[i];
        const uint32_t st = (uint8_t)k.a.state[i];
        const uint32_t pid = k.a.prog_id[i];
        // BasicAgentMeta::getScalingSymptoms(v, st) reads slot v*7 + max(6, st):
        // the per-variant slot 6 for states up to 6, the unscaled value beyond
        const float meta = st <= 6u ? k.a.scaling_v[(size_t)v * k.a.n + i] : k.a.symptom_scaling[i];
        const float prog = (st == 7) ? k.m.death_scaling[v] / meta : k.m.prog_scaling[v];
        const float scaling = meta * prog;
        if (days == -2) {
            days = (int16_t)calc_days(k, pid, st, v, &rng);
            if (v >= 3) days = (days * 0.7 == 0) ? 1 : (int16_t)(days * 0.7);
        }
        bool recovered = false;
        if (days == 0) {
            const bool was_infected = k.m.state_infected[st] != 0;
            int bad = 0;
            const uint32_t next = select_next(T, (size_t)pid * k.m.n_states + st, scaling, &rng, &bad);
            const int nd = calc_days(k, pid, next, v, &rng);
            k.a.state[i] = (int8_t)next;
            update_meta(k, i);
            days = (int16_t)nd;
            if (v >= 3 && next < 8) {
                const float mul = next < 6 ? 0.7f : 0.5f;
                days = (days * mul == 0) ? 1 : (int16_t)(days * mul);
            }
            if (bad) {
                k.a.st_worst_state[i] = (int8_t)next;
                k.a.st_worst_ts[i] = t;
                k.a.st_worst_end_ts[i] = t + ((uint32_t)((int)days * 60 * 24)) / k.p.time_step;
            } else if (st != next) {
                if (was_infected && !k.m.state_infected[next]) {
                    k.a.st_recovered_ts[i] = t;
                    recovered = true;
                }
            }
        }
        k.a.days[i] = days;
        if (recovered) k.a.diagnosed[i] = 0;
    }
}

// ---------------------------------------------------------------------------
// Testing: DetailedTesting::performTests (testingPolicies.h:370-475)
__device__ __forceinline__ bool quarantine_window_ok(uint32_t qu, uint32_t t, uint32_t ql_steps, uint32_t day_steps) {
    return qu == 0 || (qu != 0 && (qu - ql_steps >= t - day_steps || qu < t));
}

// flagLocations, testingPolicies.h:64-148
__global__ void __launch_bounds__(256) k_test_flag(KArgs k, uint32_t t) {
    const psim_params& p = k.p;
    const uint32_t day_steps = 24u * 60u / p.time_step;
    const uint32_t ql_steps = p.quarantine_length * 24u * 60u / p.time_step;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        if (!(k.a.st_diagnosed_ts[i] > t - day_steps)) continue;
        const uint32_t rep = k.a.rep[i];
        psim_stream rng;
        psim_stream_init(&rng, k.r.seed[rep], i - k.r.agent_off[rep], t, PSIM_PHASE_TEST_FLAG);
        uint32_t home = k.a.home[i];
        if (home != NONE && home < k.l.n) k.l.flags[home] = 1;
        uint32_t work = find_location(k, i, p.work_type, 0, &rng);
        if (work != NONE && work < k.l.n && quarantine_window_ok(k.l.quarantine_until[work], t, ql_steps, day_steps))
            k.l.flags[work] = 1;
        uint32_t school = find_location(k, i, p.school_type, 0, &rng);
        if (school != NONE && school < k.l.n &&
            quarantine_window_ok(k.l.quarantine_until[school], t, ql_steps, day_steps)) {
            k.l.flags[school] = 1;
            uint32_t classroom = find_location(k, i, p.classroom_type, 0, &rng);
            if (classroom != NONE && classroom < k.l.n &&
                quarantine_window_ok(k.l.quarantine_until[classroom], t, ql_steps, day_steps))
                k.l.flags[classroom] = 1;
        }
    }
}

// doTesting, testingPolicies.h:162-281
__global__ void __launch_bounds__(256) k_test(KArgs k, uint32_t t) {
    const psim_params& p = k.p;
    const uint32_t day_steps = 24u * 60u / p.time_step;
    const uint32_t delay_steps = p.testing_delay * 24u * 60u / p.time_step;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        if (t > delay_steps && k.a.last_test[i] != NONE && k.a.last_test[i] > t - delay_steps) continue;
        if (wb_of(k, i) == WB_D || k.a.diagnosed[i]) continue;
        const uint32_t rep = k.a.rep[i];
        psim_stream rng;
        psim_stream_init(&rng, k.r.seed[rep], i - k.r.agent_off[rep], t, PSIM_PHASE_TEST);
        uint32_t home = k.a.home[i];
        int home_flag = (home != NONE && home < k.l.n) ? k.l.flags[home] : 0;
        uint32_t work = find_location(k, i, p.work_type, 0, &rng);
        int work_flag = (work != NONE && work < k.l.n) ? k.l.flags[work] : 0;
        uint32_t school = find_location(k, i, p.school_type, 0, &rng);
        int school_flag = 0, class_flag = 0;
        if (school != NONE && school < k.l.n) {
            school_flag = k.l.flags[school];
            uint32_t classroom = find_location(k, i, p.classroom_type, 0, &rng);
            if (classroom != NONE) class_flag = 1;
        }
        double prob = p.t_random;
        prob = prob + (double)home_flag * p.t_home;
        prob = prob + (double)work_flag * p.t_work;
        prob = prob + (double)school_flag * p.t_school;
        prob = prob + ((double)class_flag * 3.0) * p.t_school;
        if (work != NONE && (loc_type(k, work) == p.doctor_type || loc_type(k, work) == p.hospital_type))
            prob = prob + p.t_hospital;
        if (work != NONE && loc_type(k, work) == p.nursery_type) prob = prob + p.t_nursery;
        if (k.a.st_hospitalized_ts[i] <= t && k.a.st_hospitalized_until[i] > t) prob = prob + p.t_hospital;
        if (prob > 1.0 || psim_u01(&rng) * 1.0 < prob) {
            k.a.last_test[i] = t;
            if (infected_of(k, i)) {
                const uint8_t st = (uint8_t)k.a.state[i];
                const float acc = p.use_pcr ? k.m.state_acc_pcr[st] : k.m.state_acc_antigen[st];
                if ((double)acc > psim_u01(&rng) * 1.0) {
                    k.a.diagnosed[i] = 1;
                    k.a.st_diagnosed_ts[i] = t;
                }
            } else {
                if (k.a.st_quarantined_until[i] > t && (home != NONE && loc_qu(k, home) < t)) {
                    if (k.a.st_days_in_quarantine[i] > 0)
                        k.a.st_days_in_quarantine[i] -= (k.a.st_quarantined_until[i] - t) / day_steps;
                    k.a.st_quarantined_until[i] = t;
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Daily statistics (Simulation::refreshAndPrintStatistics, simulation.h:473-665;
// Statistic::refreshandGetAfterMidnight, statistics.h:28-56; countVariantCases
// :768-777; the testing counts of performTests, testingPolicies.h:458-473).
// One pass over the agents; raw counters per replica, the row is assembled on
// the host.
constexpr int STAT_FIELDS = 48;

// A warp's counters live in its lanes: field f in word f / 32 of lane f % 32.
// Each agent sets one bit per counted flag in two words (bit f of word w is
// field 32 w + f); a 32 x 32 bit transpose across the warp hands lane f the
// column of bit f, whose population count is the warp's count of field f.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, int lane) {
#pragma unroll
    for (int j = 16; j > 0; j >>= 1) {
        const uint32_t m = j == 16 ? 0x0000FFFFu : j == 8 ? 0x00FF00FFu : j == 4 ? 0x0F0F0F0Fu : j == 2 ? 0x33333333u : 0x55555555u;
        const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
        x = (lane & j) ? ((x & ~m) | ((y & ~m) >> j)) : ((x & m) | ((y & m) << j));
    }
    return x;
}

// adds a warp's counters (lane-distributed), its lanes' sums of the two
// counted values (reinfections, boosters) and its lanes' immunity sums to
// replica `rep`: into the block's shared row when `rep` is the block's
// replica, else into the global row; then clears them
template <int VM>
__device__ __forceinline__ void stats_flush_warp(const KArgs& k, uint32_t rep, uint32_t block_rep, unsigned* acc,
                                                 unsigned* val, double* imm, uint32_t V, unsigned* s_c, double* s_imm) {
    const int lane = threadIdx.x & 31;
    const bool shared_row = rep == block_rep;
    const unsigned reinf = __reduce_add_sync(0xffffffffu, val[0]);
    const unsigned bstr = __reduce_add_sync(0xffffffffu, val[1]);
    if (lane == SC_REINF) acc[0] += reinf;
    if (lane == SC_BSTR) acc[0] += bstr;
    val[0] = val[1] = 0u;
#pragma unroll
    for (int w = 0; w < 2; ++w) {
        const int f = w * 32 + lane;
        if (f < STAT_FIELDS && rep != NONE && acc[w]) {
            if (shared_row)
                atomicAdd(&s_c[f], acc[w]);
            else
                atomicAdd(&k.stats[rep].c[f], acc[w]);
        }
        acc[w] = 0;
    }
#pragma unroll
    for (int v = 0; v < VM; ++v) {
        if ((uint32_t)v < V) {
            double x = imm[v];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0 && rep != NONE && x != 0.0) {
                if (shared_row)
                    atomicAdd(&s_imm[v], x);
                else
                    atomicAdd(&k.stats[rep].imm[v], x);
            }
        }
        imm[v] = 0.0;
    }
}

// The statistics row (Simulation::refreshAndPrintStatistics, simulation.h:473-665)
// in one pass: each block walks a contiguous range of agents; a warp counts
// its 32 agents' flags per field by a bit transpose, keeps the counts in its
// lanes, and adds them to the block's shared row (or, for another replica
// than the block's last one, to the global row) when its replica changes and
// at the end.  A warp whose agents span two replicas counts them one replica
// at a time.
// VM: the largest number of variants the kernel accumulates immunity for
// (at least the context's); the per-lane sums take registers.
template <int VM>
__global__ void __launch_bounds__(256, VM > 2 ? 4 : 5) k_stats(KArgs k, uint32_t t, int with_tests) {
    static_assert(SC_P2 < 17 && SC_HIST == 17 && SC_VAR == 33 && SC_INFV == 40 && PSIM_MAX_STRAINS <= 7,
                  "the flag words hold fields 0-31 and 32-46");
    __shared__ unsigned s_c[STAT_FIELDS];
    __shared__ double s_imm[PSIM_MAX_STRAINS];
    const uint32_t N = k.a.n, V = k.m.n_variants;
    const uint32_t day_steps = 24u * 60u / k.p.time_step;
    const uint32_t vmask = (1u << V) - 1u;
    const int lane = threadIdx.x & 31;
    const uint32_t per = ((N + gridDim.x - 1) / gridDim.x + 255u) & ~255u;
    const uint32_t begin = blockIdx.x * per, end = min(N, begin + per);
    if (threadIdx.x < STAT_FIELDS) s_c[threadIdx.x] = 0u;
    if (threadIdx.x < PSIM_MAX_STRAINS) s_imm[threadIdx.x] = 0.0;
    // the replica of the block's last agent takes the shared row
    const uint32_t block_rep = begin < end ? (uint32_t)k.a.rep[end - 1] : NONE;
    __syncthreads();
    unsigned acc[2] = {0u, 0u}, val[2] = {0u, 0u};
    double imm[VM];
#pragma unroll
    for (int v = 0; v < VM; ++v) imm[v] = 0.0;
    uint32_t cur = NONE;
    for (uint32_t base = begin; base < end; base += 256u) {
        const uint32_t i = base + threadIdx.x;
        const bool act = i < end;
        // every field is loaded at once, for idle lanes from a valid agent:
        // no load waits for the value of another
        const uint32_t j = act ? i : begin;
        const uint32_t rep = act ? (uint32_t)k.a.rep[j] : NONE;
        const uint8_t st = (uint8_t)k.a.state[j];
        const uint32_t h_until = k.a.st_hospitalized_until[j];
        const uint32_t q_ts = k.a.st_quarantined_ts[j], q_until = k.a.st_quarantined_until[j];
        const uint32_t its = k.a.st_infected_ts[j];
        const uint32_t ic = k.a.st_infected_count[j], mc = k.a.st_immunization_count[j];
        const bool stayed = k.a.stayed_home[j] != 0, hcw = k.a.hcw[j] != 0, quar = k.a.quarantined[j] != 0;
        const uint32_t var = k.a.variant[j], vmask_i = k.a.st_variant_mask[j];
        const uint32_t ltype = loc_type(k, k.a.location[j]);
        const uint32_t tested = with_tests ? k.a.last_test[j] : NONE;
        const uint32_t d = with_tests ? k.a.st_diagnosed_ts[j] : NONE;
        float sus[VM];
#pragma unroll
        for (int v = 0; v < VM; ++v) sus[v] = (uint32_t)v < V ? k.a.susceptible[(size_t)v * N + j] : 1.0f;
        uint32_t wa = 0u, wb = 0u, reinf = 0u, bstr = 0u;
        if (act) {
            const uint32_t wbs = k.m.state_wb[st];
            const bool inf = k.m.state_infected[st] != 0;
            const bool hosp = wbs != WB_D && wbs != WB_S && t < h_until;
            const bool isq = q_ts <= t && q_until > t;
            const bool new_inf = its > t - day_steps && its <= t;
            wa = (uint32_t)hosp << SC_HOSP | (uint32_t)isq << SC_Q | (uint32_t)(isq && inf) << SC_QT |
                 (uint32_t)(!isq && inf) << SC_NQ | (uint32_t)stayed << SC_STAYED | (uint32_t)new_inf << SC_NI |
                 (uint32_t)(ic > 0) << SC_INF_ONCE | (uint32_t)inf << SC_ALL_INF |
                 (uint32_t)(hcw && (inf || quar)) << SC_HCI | (uint32_t)(hcw && new_inf) << SC_HCE |
                 (uint32_t)(inf && ltype == k.p.hospital_type) << SC_INFH | (uint32_t)(ic == 0 && mc > 0) << SC_VNI;
            if (with_tests)
                wa |= (uint32_t)(tested == t) << SC_TESTS | (uint32_t)(d == t) << SC_P1 |
                      (uint32_t)(d < t && d > t - day_steps) << SC_P2;
            // the state histogram: states 0-14 in the first word, 15 in the second
            if (st < 15)
                wa |= 1u << (SC_HIST + st);
            else if (st == 15)
                wb |= 1u;
            if (inf && var < (uint32_t)PSIM_MAX_STRAINS) wb |= 1u << (SC_VAR - 32 + var);
            wb |= (vmask_i & vmask) << (SC_INFV - 32);
            reinf = ic > 1 ? ic - 1 : 0u;
            bstr = mc > 1 ? mc - 1 : 0u;
        }
        // one replica of the warp at a time (almost always one)
        unsigned todo = __ballot_sync(0xffffffffu, act);
        while (todo) {
            const uint32_t r = __shfl_sync(0xffffffffu, rep, __ffs(todo) - 1);
            const bool sel = act && rep == r;
            todo &= ~__ballot_sync(0xffffffffu, sel);
            if (r != cur) {
                stats_flush_warp<VM>(k, cur, block_rep, acc, val, imm, V, s_c, s_imm);
                cur = r;
            }
            acc[0] += (unsigned)__popc(warp_transpose32(sel ? wa : 0u, lane));
            acc[1] += (unsigned)__popc(warp_transpose32(sel ? wb : 0u, lane));
            if (sel) {
                val[0] += reinf;
                val[1] += bstr;
#pragma unroll
                for (int v = 0; v < VM; ++v)
                    if ((uint32_t)v < V) imm[v] += 1.0 - (double)sus[v];
            }
        }
    }
    stats_flush_warp<VM>(k, cur, block_rep, acc, val, imm, V, s_c, s_imm);
    __syncthreads();
    if (block_rep != NONE) {
        if (threadIdx.x < STAT_FIELDS && s_c[threadIdx.x]) atomicAdd(&k.stats[block_rep].c[threadIdx.x], s_c[threadIdx.x]);
        if (threadIdx.x < V && s_imm[threadIdx.x] != 0.0) atomicAdd(&k.stats[block_rep].imm[threadIdx.x], s_imm[threadIdx.x]);
    }
}

// The variant gating alone, without the statistics (after an upload): a
// variant is active in a replica when one of its agents is infected with it.
__global__ void __launch_bounds__(256) k_variant_flags(KArgs k) {
    const uint32_t N = k.a.n, V = k.m.n_variants;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        if (!k.m.state_infected[(uint8_t)k.a.state[i]]) continue;
        uint8_t* f = &k.r.variant_active[(size_t)k.a.rep[i] * V + k.a.variant[i]];
        if (*f == 0) *f = 1;
    }
}

// variant gating of the next day (countVariantCases, simulation.h:768-777)
__global__ void k_variant_active(KArgs k) {
    const uint32_t R = k.r.n, V = k.m.n_variants;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < R * V; j += gridDim.x * blockDim.x) {
        const uint32_t q = j / V, v = j % V;
        k.r.variant_active[j] = k.stats[q].c[SC_VAR + v] > 0;
    }
}

// ---------------------------------------------------------------------------
// planLocations, movementPolicies.h:1428-1622
// checkSchoolQuarantine, :1285-1310 (quarantinePolicy > 3)
__global__ void k_plan_schools(KArgs k, uint32_t t) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < k.l.n_schools; s += gridDim.x * blockDim.x) {
        const uint32_t school = k.l.schools[s];
        if (k.l.quarantine_until[school] > t) continue;
        uint32_t counter = 0, mx = 0;
        for (uint32_t c = k.l.classroom_offsets[s]; c < k.l.classroom_offsets[s + 1]; ++c) {
            const uint32_t cl = k.l.classrooms[c];
            const uint32_t q = k.l.quarantine_until[cl];
            if (q > t) {
                counter++;
                mx = mx > q ? mx : q;
            }
        }
        if (counter > 1) {
            k.l.quarantine_until[school] = mx;
            for (uint32_t c = k.l.classroom_offsets[s]; c < k.l.classroom_offsets[s + 1]; ++c)
                k.l.quarantine_until[k.l.classrooms[c]] = mx;
        }
    }
}

// resets + checkSchoolWorkQuarantine (:1188-1240)
__global__ void __launch_bounds__(256) k_plan_agents(KArgs k, uint32_t t) {
    const psim_params& p = k.p;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        k.a.move_at[i] = t + p.curfew_end;  // stepsUntilMove = curfewEnd before step t
        k.a.stayed_home[i] = 1;
        k.a.no_work[i] = 0;
        if (p.quarantine_policy > 2) {
            if (k.a.quarantined[i]) continue;
            if (k.a.st_diagnosed_ts[i] > 0 && !infected_of(k, i)) continue;
            const uint32_t rep = k.a.rep[i];
            psim_stream rng;
            psim_stream_init(&rng, k.r.seed[rep], i - k.r.agent_off[rep], t, PSIM_PHASE_PLAN_SWQ);
            const uint32_t work = find_location3(k, i, p.work_type, 0, &rng, p.home_type, p.school_type, p.classroom_type);
            const uint32_t school = find_location3(k, i, p.school_type, 0, &rng, p.home_type, p.school_type, p.classroom_type);
            const uint32_t classroom = find_location3(k, i, p.classroom_type, 0, &rng, p.home_type, p.school_type, p.classroom_type);
            uint32_t until = 0;
            if (school != NONE && loc_qu(k, school) > t)
                until = loc_qu(k, school);
            else if (classroom != NONE && loc_qu(k, classroom) > t)
                until = loc_qu(k, classroom);
            else if (work != NONE && loc_qu(k, work) > t)
                until = loc_qu(k, work);
            if (until > 0) {
                k.a.quarantined[i] = 1;
                k.a.st_quarantined_ts[i] = t;
                k.a.st_quarantined_until[i] = until;
                k.a.st_days_in_quarantine[i] += (until - t) / (24u * 60u / p.time_step);
            }
        }
    }
}

// clear quarantine flags, close quarantined schools/classrooms (:1571-1583)
__global__ void __launch_bounds__(256) k_plan_locations(KArgs k, uint32_t t) {
    const psim_params& p = k.p;
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < k.l.n; l += gridDim.x * blockDim.x) {
        k.l.no_work_loc[l] = 0u;
        if (p.quarantine_policy > 2) {
            const uint32_t ty = k.l.type[l];
            const uint32_t q = k.l.quarantine_until[l];
            if (q > t && (ty == p.school_type || ty == p.classroom_type)) {
                k.l.closed_until[l] = q;
                k.l.quarantine_until[l] = 0u;
            } else if (q > t && ty == p.work_type) {
                k.l.quarantine_until[l] = 0u;
            }
        }
    }
}

// checkUnderageAtHome, :1056-1094 (flag = 0xFFFFFFFF)
__global__ void __launch_bounds__(256) k_plan_underage(KArgs k, uint32_t t) {
    const psim_params& p = k.p;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        if (k.a.age[i] > 14) continue;
        const uint32_t rep = k.a.rep[i];
        psim_stream rng;
        psim_stream_init(&rng, k.r.seed[rep], i - k.r.agent_off[rep], t, PSIM_PHASE_PLAN_UNDERAGE);
        const uint32_t home = k.a.home[i];
        bool flag = false;
        if (k.a.quarantined[i]) {
            flag = true;
        } else {
            const uint32_t school = find_location3(k, i, p.school_type, 0, &rng, p.home_type, p.school_type, p.classroom_type);
            const uint32_t classroom = find_location3(k, i, p.classroom_type, 0, &rng, p.home_type, p.school_type, p.classroom_type);
            const bool too_old = k.a.age[i] >= p.school_age_restriction;
            flag = too_old || (school != NONE && (loc_open(k, school) == 0 || loc_closed_until(k, school) > t)) ||
                   (classroom != NONE && (loc_open(k, classroom) == 0 || loc_closed_until(k, classroom) > t));
        }
        if (flag && home < k.l.n) k.l.no_work_loc[home] = NONE;
    }
}

// setNoWorkToday, :1137-1158: the lowest-id eligible adult of a flagged home
// (the home is a first match: the agent's stream is not drawn from)
__global__ void __launch_bounds__(256) k_plan_nowork_min(KArgs k, uint32_t t) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        const uint8_t age = k.a.age[i];
        if (!(age > 26 && age < 65)) continue;
        const uint32_t home = k.a.home[i];
        // 0 = home not flagged, NONE = flagged, else 1 + the lowest claiming id
        if (home < k.l.n && k.l.no_work_loc[home] != 0u) atomicMin(&k.l.no_work_loc[home], i + 1u);
    }
}

__global__ void __launch_bounds__(256) k_plan_nowork_set(KArgs k, uint32_t t) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        const uint8_t age = k.a.age[i];
        if (!(age > 26 && age < 65)) continue;
        const uint32_t home = k.a.home[i];
        if (home < k.l.n && k.l.no_work_loc[home] == i + 1u) k.a.no_work[i] = 1;
    }
}

// The agents' homes (findActualLocationForType for the home type,
// movementPolicies.h:69-122: the first entry of that type, no draw).
__global__ void k_homes(KArgs k) {
    const uint32_t ht = k.p.home_type;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        uint32_t h = NONE;
        for (uint32_t j = k.a.loc_offset[i]; j < k.a.loc_offset[i + 1]; ++j)
            if (k.a.poss_type[j] == ht) {
                h = k.a.poss_loc[j];
                break;
            }
        k.a.home[i] = h;
    }
}

// Simulation::flagHealthcareWorkers, simulation.h:670-693 (type ids 4 / 12 / 14 as
// hard-coded in the reference)
__global__ void k_flag_hcw(KArgs k) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        uint8_t f = 0;
        for (uint32_t j = k.a.loc_offset[i]; j < k.a.loc_offset[i + 1]; ++j) {
            const uint32_t lt = loc_type(k, k.a.poss_loc[j]);
            if (k.a.poss_type[j] == 4 && (lt == 12 || lt == 14)) {
                f = 1;
                break;
            }
        }
        k.a.hcw[i] = f;
    }
}

// w_l = w of the location's type (psim_set_type_weights)
__global__ void k_type_weights(KArgs k, const float* w_by_type) {
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < k.l.n; l += gridDim.x * blockDim.x)
        k.l.infectiousness[l] = w_by_type[k.l.type[l]];
}

// Closure rule Masks (closurePolicies.h:236-268): the w of every non-home
// location multiplied (masks on) or divided (masks off) by the coefficient,
// float * double rounded to float as in the reference's lambda.
__global__ void k_masks(KArgs k, uint32_t home_type, double coef, int open) {
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < k.l.n; l += gridDim.x * blockDim.x) {
        if (k.l.type[l] == home_type) continue;
        const double w = (double)k.l.infectiousness[l];
        k.l.infectiousness[l] = (float)(open ? w / coef : w * coef);
    }
}

// A closure rule over location types (closurePolicies.h:424-468): every
// non-essential location whose type is listed becomes open/closed.
__global__ void k_close_types(KArgs k, ClosureTypes ty, int open) {
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < k.l.n; l += gridDim.x * blockDim.x) {
        if (k.l.essential[l] == 1) continue;
        const uint32_t t = k.l.type[l];
        for (uint32_t q = 0; q < ty.n; ++q)
            if (t == ty.v[q]) {
                k.l.open[l] = open ? 1 : 0;
                break;
            }
    }
}

// Closure rule ExposeToMutation (closurePolicies.h:349-392): every agent with
// susceptibility s > 0 for the variant is infected with it when a uniform
// draw is below fraction * s.
__global__ void k_expose(KArgs k, uint32_t t, uint32_t v, double fraction) {
    const uint32_t N = k.a.n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const float su = k.a.susceptible[(size_t)v * N + i];
        if (!(su > 0.0f)) continue;
        const uint32_t rep = k.a.rep[i];
        const double U = psim_u01_once(k.r.seed[rep], i - k.r.agent_off[rep], t, PSIM_PHASE_EXPOSE);
        if (U < fraction * (double)su) {
            k.a.state[i] = (int8_t)k.m.first_infected;
            k.a.variant[i] = (uint8_t)v;
            k.a.days[i] = -2;
            update_meta(k, i);
            k.a.st_infected_ts[i] = t;
            k.a.st_infected_loc[i] = k.a.location[i];
            k.a.st_infected_count[i] = k.a.st_infected_count[i] + 1;
            k.a.st_worst_state[i] = (int8_t)k.m.first_infected;
            k.a.st_worst_ts[i] = t;
            k.a.st_variant_mask[i] |= 1u << v;
        }
    }
}

// A wait on a flag that nothing sets, bounded by `iters`: reports
// ERR_TEST_WAIT and returns.  Exercises the bounded-wait error path.
__global__ void k_bounded_wait_probe(KArgs k, uint32_t iters) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    volatile uint32_t* flag = &k.clock->pad[0];
    uint32_t n = 0;
    while (*flag == 0u) {
        if (++n >= iters) {
            atomicOr(k.err, ERR_TEST_WAIT);
            return;
        }
    }
}

// ---------------------------------------------------------------------------
// launchers
static int g_sm_count = 0;
static int sm_count() {
    if (g_sm_count == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (g_sm_count <= 0) g_sm_count = 152;
    }
    return g_sm_count;
}

static unsigned grid_for(uint32_t n, int per_sm) {
    unsigned want = (n + 255) / 256;
    unsigned cap = (unsigned)(sm_count() * per_sm);
    if (want > cap) want = cap;
    return want ? want : 1u;
}

// one full wave of resident 256-thread blocks (grid-stride kernels)
template <typename K>
static unsigned wave_grid(K kernel, uint32_t n) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess || per_sm < 1) per_sm = 4;
    return grid_for(n, per_sm);
}

static unsigned agent_grid(const KArgs& k, unsigned wave) {
    unsigned g = k.tune.blocks_per_sm ? (unsigned)(sm_count() * k.tune.blocks_per_sm) : wave;
    return std::min(g, grid_for(k.a.n, 1 << 20));
}

void launch_movement(const KArgs& k, uint32_t step, cudaStream_t s) {
    static unsigned g = 0;
    if (!g) g = wave_grid(k_movement, 1u << 30);
    k_movement<<<agent_grid(k, g), 256, 0, s>>>(k, step);
}
// The step kernel's grid: every block resident at once (its grid barriers
// need that), tune.blocks_per_sm capped at the kernel's occupancy, and no
// more blocks than the population and locations give work to.  Each block's
// work-list segment holds the agents its queue pass visits.
static unsigned step_blocks_per_sm() {
    static int occ = 0;
    if (!occ) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_step, 256, 0) != cudaSuccess || occ < 1) occ = 1;
    }
    return (unsigned)occ;
}
static void step_geometry(const KArgs& k, unsigned* grid, uint32_t* cap) {
    const unsigned occ = step_blocks_per_sm();
    const unsigned bps = k.tune.blocks_per_sm ? std::min<unsigned>(k.tune.blocks_per_sm, occ) : occ;
    const size_t want = std::max<size_t>(((size_t)k.a.n + 255) / 256, (((size_t)k.l.n + 31) / 32 + 7) / 8);
    unsigned g = (unsigned)std::min<size_t>((size_t)sm_count() * bps, std::max<size_t>(want, 1));
    g = std::min(g, (unsigned)WORK_MAX_BLOCKS);
    *grid = g;
    // the queue's quads: ceil(quads / (g * 256)) per thread, 4 agents each
    const size_t quads = ((size_t)k.a.n + 3) / 4;
    *cap = (uint32_t)(((quads + (size_t)g * 256 - 1) / ((size_t)g * 256)) * 1024);
}
void launch_steps(const KArgs& k, uint32_t step0, uint32_t nsteps, uint32_t phases, cudaStream_t s) {
    unsigned g;
    uint32_t cap;
    step_geometry(k, &g, &cap);
    k_step<<<g, 256, 0, s>>>(k, step0, nsteps, phases, cap);
}
void launch_step(const KArgs& k, uint32_t step, uint32_t phases, cudaStream_t s) { launch_steps(k, step, 1, phases, s); }
void launch_count(const KArgs& k, cudaStream_t s) { k_count<<<grid_for(k.a.n, 8), 256, 0, s>>>(k); }
// the scan of the histogram with 256 x tune.scan_items locations per tile:
// single pass with decoupled look-back (tune.scan_mode 0) or tile sums, then
// the scan (scan_mode 1)
template <int ITEMS>
static void launch_scan_items(const KArgs& k, uint32_t step, int with_hazard, int merge_q, cudaStream_t s) {
    unsigned tiles = (k.l.n + SCAN_THREADS * ITEMS - 1) / (SCAN_THREADS * ITEMS);
    if (!tiles) tiles = 1;
    if ((k.tune.scan_mode == 2 || k.tune.scan_mode == 3) && (ITEMS == 4 || ITEMS == 8)) {
        // thread-contiguous: ITEMS / 4 vectors of 4 locations per thread;
        // two passes (2) or one with look-back (3)
        constexpr int Q = ITEMS >= 8 ? 2 : 1;
        if (k.tune.scan_mode == 3) {
            k_scan_v<Q, true><<<tiles, SCAN_THREADS, 0, s>>>(k, step, with_hazard, merge_q);
        } else {
            k_tile_sums_v<Q><<<tiles, SCAN_THREADS, 0, s>>>(k, step);
            k_scan_v<Q, false><<<tiles, SCAN_THREADS, 0, s>>>(k, step, with_hazard, merge_q);
        }
        return;
    }
    if (k.tune.scan_mode == 0 || k.tune.scan_mode == 3) {
        k_scan<ITEMS, true><<<tiles, SCAN_THREADS, 0, s>>>(k, step, with_hazard, merge_q);
    } else {
        k_tile_sums<ITEMS><<<tiles, SCAN_THREADS, 0, s>>>(k, step);
        k_scan<ITEMS, false><<<tiles, SCAN_THREADS, 0, s>>>(k, step, with_hazard, merge_q);
    }
}
// step: the step in the day whose CSR the scan prepares (rebuilt only when
// agents took new locations for it, see csr_decide)
void launch_scan(const KArgs& k, uint32_t step, int with_hazard, int merge_q, cudaStream_t s) {
    if (k.tune.scan_items == 2)
        launch_scan_items<2>(k, step, with_hazard, merge_q, s);
    else if (k.tune.scan_items == 4)
        launch_scan_items<4>(k, step, with_hazard, merge_q, s);
    else
        launch_scan_items<8>(k, step, with_hazard, merge_q, s);
}
int scan_kernels(const KArgs& k) { return k.tune.scan_mode == 0 || k.tune.scan_mode == 3 ? 1 : 2; }
void launch_scatter_draw(const KArgs& k, uint32_t step, int scatter, int draw, cudaStream_t s) {
    static unsigned g = 0;
    if (!g) g = wave_grid(k_scatter_draw, 1u << 30);
    k_scatter_draw<<<agent_grid(k, g), 256, 0, s>>>(k, step, scatter, draw);
}
void launch_offsets(const KArgs& k, cudaStream_t s) {
    k_offsets_from_cursor<<<grid_for(k.l.n + 1, 8), 256, 0, s>>>(k, k.l.csr_off);
}
void launch_canonical_csr(const KArgs& k, cudaStream_t s) {
    // csr_off must be current (launch_offsets); the rank buffer is scratch
    k_canonical_rank<<<grid_for(k.a.n, 16), 256, 0, s>>>(k, k.l.csr_off, k.a.rank);
    cudaMemcpyAsync(k.l.csr_agents, k.a.rank, sizeof(uint32_t) * k.a.n, cudaMemcpyDeviceToDevice, s);
}
void launch_progress(const KArgs& k, uint32_t t, cudaStream_t s) {
    const size_t nt = (size_t)k.m.n_prog * k.m.n_states;
    const size_t bytes = nt * 4 * sizeof(uint32_t) + (size_t)k.m.n_trans * (sizeof(uint32_t) + sizeof(float));
    const int staged = bytes <= 48 * 1024;
    k_progress<<<grid_for(k.a.n, 8), 256, staged ? bytes : 0, s>>>(k, t, staged);
}
void launch_test(const KArgs& k, uint32_t t, cudaStream_t s) {
    cudaMemsetAsync(k.l.flags, 0, k.l.n, s);
    k_test_flag<<<grid_for(k.a.n, 8), 256, 0, s>>>(k, t);
    k_test<<<grid_for(k.a.n, 8), 256, 0, s>>>(k, t);
}
void launch_stats(const KArgs& k, uint32_t t, cudaStream_t s) {
    cudaMemsetAsync(k.stats, 0, sizeof(DevStatsAcc) * k.r.n, s);
    static unsigned g[3] = {0, 0, 0};
    if (!g[0]) {
        g[0] = wave_grid(k_stats<1>, 1u << 30);
        g[1] = wave_grid(k_stats<2>, 1u << 30);
        g[2] = wave_grid(k_stats<PSIM_MAX_STRAINS>, 1u << 30);
    }
    const int vi = k.m.n_variants <= 1 ? 0 : k.m.n_variants <= 2 ? 1 : 2;
    unsigned blocks = std::min(g[vi], (unsigned)((k.a.n + 255) / 256));
    if (!blocks) blocks = 1;
    if (vi == 0)
        k_stats<1><<<blocks, 256, 0, s>>>(k, t, 1);
    else if (vi == 1)
        k_stats<2><<<blocks, 256, 0, s>>>(k, t, 1);
    else
        k_stats<PSIM_MAX_STRAINS><<<blocks, 256, 0, s>>>(k, t, 1);
    k_variant_active<<<1, 256, 0, s>>>(k);
}
void launch_variant_flags(const KArgs& k, cudaStream_t s) {
    cudaMemsetAsync(k.r.variant_active, 0, (size_t)k.r.n * k.m.n_variants, s);
    k_variant_flags<<<grid_for(k.a.n, 8), 256, 0, s>>>(k);
}
void launch_plan(const KArgs& k, uint32_t t, cudaStream_t s) {
    if (k.p.quarantine_policy > 3 && k.l.n_schools) k_plan_schools<<<grid_for(k.l.n_schools, 4), 256, 0, s>>>(k, t);
    k_plan_agents<<<grid_for(k.a.n, 8), 256, 0, s>>>(k, t);
    k_plan_locations<<<grid_for(k.l.n, 8), 256, 0, s>>>(k, t);
    k_plan_underage<<<grid_for(k.a.n, 8), 256, 0, s>>>(k, t);
    k_plan_nowork_min<<<grid_for(k.a.n, 8), 256, 0, s>>>(k, t);
    k_plan_nowork_set<<<grid_for(k.a.n, 8), 256, 0, s>>>(k, t);
}
void launch_flag_hcw(const KArgs& k, cudaStream_t s) { k_flag_hcw<<<grid_for(k.a.n, 8), 256, 0, s>>>(k); }
void launch_homes(const KArgs& k, cudaStream_t s) { k_homes<<<grid_for(k.a.n, 8), 256, 0, s>>>(k); }
void launch_type_weights(const KArgs& k, const float* w_by_type, cudaStream_t s) {
    k_type_weights<<<grid_for(k.l.n, 8), 256, 0, s>>>(k, w_by_type);
}
void launch_masks(const KArgs& k, uint32_t home_type, double coef, int open, cudaStream_t s) {
    k_masks<<<grid_for(k.l.n, 8), 256, 0, s>>>(k, home_type, coef, open);
}
void launch_close_types(const KArgs& k, const ClosureTypes& ty, int open, cudaStream_t s) {
    k_close_types<<<grid_for(k.l.n, 8), 256, 0, s>>>(k, ty, open);
}
void launch_expose(const KArgs& k, uint32_t t, uint32_t variant, double fraction, cudaStream_t s) {
    k_expose<<<grid_for(k.a.n, 8), 256, 0, s>>>(k, t, variant, fraction);
}
void launch_bounded_wait_probe(const KArgs& k, uint32_t iters, cudaStream_t s) {
    k_bounded_wait_probe<<<1, 32, 0, s>>>(k, iters);
}
// countdowns <-> absolute decision timestamps (upload, download)
__global__ void k_time_shift(uint32_t* a, uint32_t n, uint32_t delta) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] += delta;
}
void launch_time_shift(uint32_t* a, uint32_t n, uint32_t delta, cudaStream_t s) {
    if (n && delta) k_time_shift<<<grid_for(n, 8), 256, 0, s>>>(a, n, delta);
}

}  // namespace psim
