// Test driver — TEST INFRASTRUCTURE ONLY: the GB300 policies of
// include/gb300_policies.h in a stand-in of the reference's Simulation
// (simulation.h:53-97) whose containers have the reference's member names
// and element layouts, run in runSimulation's order (simulation.h:899-926).
// The host midnight consumer Simulation::updateAgents (simulation.h:425-471)
// runs on the host containers between the adapters' device phases (here the
// oracle's restatement of it, on a copy of the containers), so the run
// exercises the adapters' hand-over of the state in both directions.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gb300_policies.h"
#include "psim_oracle.h"

namespace {

// the reference's element types: same members, same order
struct PPStateStandIn {
    float infectious;
    unsigned progressionID;
    char state;
    short daysBeforeNextState;
    float susceptible[PSIM_MAX_STRAINS];
    uint8_t variant;
};
struct MetaStandIn {
    float scalingSymptoms[7 * PSIM_MAX_STRAINS];
    float scalingAgeSex;
    uint8_t age;
    uint8_t preCondIdx;
    bool sex;
};
struct StatsStandIn {
    unsigned infectedTimestamp = 0, infectedLocation = 0, worstStateTimestamp = 0, worstStateEndTimestamp = 0;
    unsigned diagnosedTimestamp = 0, quarantinedTimestamp = 0, quarantinedUntilTimestamp = 0, daysInQuarantine = 0;
    unsigned hospitalizedTimestamp = 0, hospitalizedUntilTimestamp = 0, immunizationTimestamp = 0;
    unsigned recoveredTimestamp = 0;
    uint8_t immunizationCount = 0;
    unsigned variant = 0;
    uint8_t infectedCount = 0;
    char worstState = 0;
};
struct AgentsStandIn {
    std::vector<PPStateStandIn> PPValues;
    std::vector<MetaStandIn> agentMetaData;
    std::vector<StatsStandIn> agentStats;
    std::vector<unsigned> location, types;
    std::vector<bool> diagnosed, quarantined, stayedHome;
    std::vector<unsigned long> locationOffset;
    std::vector<unsigned> possibleLocations, possibleTypes;
};
struct LocsStandIn {
    std::vector<unsigned> locType;
    std::vector<float> infectiousness;
    std::vector<bool> states;
    std::vector<unsigned> closedUntil, quarantineUntil, schools, classrooms, classroomOffsets;
    std::vector<uint8_t> essential;
};
struct LocationTypesStandIn {
    unsigned publicSpace, home, hospital, doctor, school, classroom, work, nurseryhome;
};
struct TimeStandIn {
    uint32_t ts;
    uint32_t getTimestamp() const { return ts; }
};

template <template <class> class Mv, template <class> class In, template <class> class Te, template <class> class Cl>
class StandInSim : private Mv<StandInSim<Mv, In, Te, Cl>>,
                   private In<StandInSim<Mv, In, Te, Cl>>,
                   private Te<StandInSim<Mv, In, Te, Cl>>,
                   private Cl<StandInSim<Mv, In, Te, Cl>> {
    using Self = StandInSim<Mv, In, Te, Cl>;
    friend class Mv<Self>;
    friend class In<Self>;
    friend class Te<Self>;
    friend class Cl<Self>;

public:
    AgentsStandIn* agents;
    LocsStandIn* locs;
    unsigned timeStep;
    pansim_gb300::Bridge scratch;   // the oracle's copy for updateAgents
    psim_oracle* oracle = nullptr;
    // the one replica of the oracle's copy
    uint32_t rep_agents[2] = {0, 0}, rep_locs[2] = {0, 0}, rep_cemetery = 0;
    uint64_t rep_seed = 0;
    double rep_k = 0.0;
    psim_replicas reps{};

    StandInSim(AgentsStandIn* a, LocsStandIn* l, unsigned dt) : agents(a), locs(l), timeStep(dt) {}
    ~StandInSim() {
        if (oracle) psim_oracle_destroy(oracle);
    }
    Mv<Self>& movementPolicy() { return *this; }
    Te<Self>& testingPolicy() { return *this; }

    // Simulation::updateAgents on the host containers
    void updateAgents(uint32_t t, const psim_params* p) {
        if (!oracle) {
            scratch.gather(this, true);
            scratch.bind();
            rep_agents[1] = scratch.N;
            rep_locs[1] = scratch.L;
            rep_cemetery = p->cemetery_loc;
            rep_seed = p->seed;
            rep_k = p->k;
            reps.n = 1;
            reps.agent_offset = rep_agents;
            reps.loc_offset = rep_locs;
            reps.seed = &rep_seed;
            reps.k = &rep_k;
            reps.cemetery = &rep_cemetery;
            oracle = psim_oracle_create(pansim_gb300::model_slot(), &scratch.a, &scratch.l, p, &reps);
            if (!oracle) throw pansim_gb300::Error("psim_oracle_create failed");
        }
        scratch.gather(this, false);
        psim_oracle_progress(oracle, t);
        scratch.scatter(this);
    }

    // runSimulation's loop (simulation.h:899-926) for `days` days
    void run(uint32_t days, const psim_params* p) {
        const uint32_t spd = 1440u / timeStep;
        std::vector<unsigned> stats;
        for (uint32_t d = 0; d < days; ++d) {
            TimeStandIn tm{d * spd};
            if (tm.ts > 0) Te<Self>::performTests(tm, timeStep);
            if (tm.ts > 0) updateAgents(tm.ts, p);
            Cl<Self>::midnight(tm, timeStep, stats);
            Mv<Self>::planLocations(tm, timeStep);
            for (uint32_t s = 0; s < spd; ++s) {
                TimeStandIn ts{d * spd + s};
                Mv<Self>::movement(ts, timeStep);
                Cl<Self>::step(ts, timeStep);
                In<Self>::infectionsAtLocations(ts, timeStep, 0);
            }
        }
        // the device state back into the host containers
        Mv<Self>::gb300.pull(this);
    }
};

using Sim = StandInSim<Gb300Movement, Gb300Infection, Gb300Testing, Gb300Closure>;

template <class T>
void copy_field(T* dst, const T* src, size_t n) {
    if (dst && src) std::memcpy(dst, src, n * sizeof(T));
}

}  // namespace

extern "C" int adapter_run(const psim_model* m, psim_agents* a, psim_locations* l, const psim_params* p, uint32_t days,
                           char* err, int err_len) {
    try {
        const uint32_t N = a->n, L = l->n, V = m->n_variants;
        AgentsStandIn ag;
        LocsStandIn lc;
        ag.PPValues.resize(N);
        ag.agentMetaData.resize(N);
        ag.agentStats.resize(N);
        ag.location.assign(a->location, a->location + N);
        ag.types.assign(a->type, a->type + N);
        ag.diagnosed.resize(N);
        ag.quarantined.resize(N);
        ag.stayedHome.resize(N);
        ag.locationOffset.assign(a->loc_offset, a->loc_offset + N + 1);
        ag.possibleLocations.assign(a->poss_loc, a->poss_loc + a->n_poss);
        ag.possibleTypes.assign(a->poss_type, a->poss_type + a->n_poss);
        const uint32_t* st[13] = {a->st_infected_ts,      a->st_infected_loc,      a->st_worst_ts,
                                  a->st_worst_end_ts,     a->st_diagnosed_ts,      a->st_quarantined_ts,
                                  a->st_quarantined_until, a->st_days_in_quarantine, a->st_hospitalized_ts,
                                  a->st_hospitalized_until, a->st_immunization_ts, a->st_recovered_ts,
                                  a->st_variant_mask};
        for (uint32_t i = 0; i < N; ++i) {
            PPStateStandIn& q = ag.PPValues[i];
            std::memset(&q, 0, sizeof(q));
            q.infectious = a->infectious[i];
            q.progressionID = a->prog_id[i];
            q.state = (char)a->state[i];
            q.daysBeforeNextState = a->days[i];
            for (uint32_t v = 0; v < V; ++v) q.susceptible[v] = a->susceptible[(size_t)v * N + i];
            q.variant = a->variant[i];
            MetaStandIn& mm = ag.agentMetaData[i];
            std::memset(&mm, 0, sizeof(mm));
            for (int j = 0; j < 7 * PSIM_MAX_STRAINS; ++j) mm.scalingSymptoms[j] = a->symptom_scaling[i];
            for (uint32_t v = 0; v < V; ++v)
                mm.scalingSymptoms[v * 7 + 6] = a->symptom_scaling_v ? a->symptom_scaling_v[(size_t)v * N + i] : a->symptom_scaling[i];
            mm.scalingAgeSex = a->symptom_scaling[i];
            mm.age = a->age[i];
            mm.preCondIdx = a->precond ? a->precond[i] : 0;
            mm.sex = a->sex ? a->sex[i] != 0 : false;
            StatsStandIn& s = ag.agentStats[i];
            unsigned* sv[13] = {&s.infectedTimestamp,      &s.infectedLocation,          &s.worstStateTimestamp,
                                &s.worstStateEndTimestamp, &s.diagnosedTimestamp,        &s.quarantinedTimestamp,
                                &s.quarantinedUntilTimestamp, &s.daysInQuarantine,       &s.hospitalizedTimestamp,
                                &s.hospitalizedUntilTimestamp, &s.immunizationTimestamp, &s.recoveredTimestamp,
                                &s.variant};
            for (int j = 0; j < 13; ++j) *sv[j] = st[j][i];
            s.immunizationCount = a->st_immunization_count[i];
            s.infectedCount = a->st_infected_count[i];
            s.worstState = (char)a->st_worst_state[i];
            ag.diagnosed[i] = a->diagnosed[i] != 0;
            ag.quarantined[i] = a->quarantined[i] != 0;
            ag.stayedHome[i] = a->stayed_home[i] != 0;
        }
        lc.locType.assign(l->type, l->type + L);
        lc.infectiousness.assign(l->infectiousness, l->infectiousness + L);
        lc.states.resize(L);
        for (uint32_t j = 0; j < L; ++j) lc.states[j] = l->open[j] != 0;
        lc.closedUntil.assign(l->closed_until, l->closed_until + L);
        lc.quarantineUntil.assign(l->quarantine_until, l->quarantine_until + L);
        lc.essential.assign(l->essential, l->essential + L);
        lc.schools.assign(l->schools, l->schools + l->n_schools);
        lc.classrooms.assign(l->classrooms, l->classrooms + l->n_classrooms);
        if (l->n_schools) lc.classroomOffsets.assign(l->classroom_offsets, l->classroom_offsets + l->n_schools + 1);

        pansim_gb300::set_model(m);
        Sim sim(&ag, &lc, p->time_step);
        // the options the reference's command line would give (initializeArgs)
        auto& mv = sim.movementPolicy();
        auto& o = mv.gb300.opt;
        o.start_day = p->start_day;
        o.start_date = p->start_date;
        o.quarantine_length = p->quarantine_length;
        o.k = p->k;
        o.c0 = p->c0;
        o.trunc = p->trunc;
        o.d_offset.clear();
        if (p->n_d_offset > 0) o.d_offset.push_back(p->d_offset0);
        if (p->n_d_offset > 1) o.d_offset.push_back(p->d_offset1);
        o.d_peak_offset = p->d_peak_offset;
        const double tp[6] = {p->t_random, p->t_home, p->t_work, p->t_school, p->t_hospital, p->t_nursery};
        for (int j = 0; j < 6; ++j) o.testing[j] = tp[j];
        o.testing_delay = p->testing_delay;
        o.use_pcr = p->use_pcr != 0;
        o.seed = p->seed;
        o.tracked = p->tracked;
        mv.quarantinePolicy = p->quarantine_policy;
        mv.enableCurfew = p->enable_curfew != 0;
        mv.curfewBegin = p->curfew_begin;
        mv.curfewEnd = p->curfew_end;
        mv.curfewTimeConverted = true;
        mv.schoolAgeRestriction = p->school_age_restriction;
        mv.holidayModeActive = p->holiday_mode != 0;
        mv.quarantineImmuneActive = p->quarantine_immune != 0;
        mv.lockdownNonvaccActive = p->lockdown_nonvacc != 0;
        const LocationTypesStandIn lt{p->public_type, p->home_type,      p->hospital_type, p->doctor_type,
                                      p->school_type, p->classroom_type, p->work_type,     p->nursery_type};
        mv.init(lt, p->cemetery_loc);
        sim.testingPolicy().init(lt);
        sim.run(days, p);

        // the final host containers into the caller's arrays
        pansim_gb300::Bridge out;
        out.gather(&sim, true);
        out.bind();
        copy_field(a->location, out.a.location, N);
        copy_field(a->state, out.a.state, N);
        copy_field(a->days, out.a.days, N);
        copy_field(a->variant, out.a.variant, N);
        copy_field(a->infectious, out.a.infectious, N);
        copy_field(a->susceptible, out.a.susceptible, (size_t)N * V);
        copy_field(a->diagnosed, out.a.diagnosed, N);
        copy_field(a->quarantined, out.a.quarantined, N);
        copy_field(a->stayed_home, out.a.stayed_home, N);
        uint32_t* dst[13] = {a->st_infected_ts,      a->st_infected_loc,      a->st_worst_ts,
                             a->st_worst_end_ts,     a->st_diagnosed_ts,      a->st_quarantined_ts,
                             a->st_quarantined_until, a->st_days_in_quarantine, a->st_hospitalized_ts,
                             a->st_hospitalized_until, a->st_immunization_ts, a->st_recovered_ts,
                             a->st_variant_mask};
        for (int j = 0; j < 13; ++j) copy_field(dst[j], out.st[j].data(), N);
        copy_field(a->st_immunization_count, out.a.st_immunization_count, N);
        copy_field(a->st_infected_count, out.a.st_infected_count, N);
        copy_field(a->st_worst_state, out.a.st_worst_state, N);
        copy_field(l->infectiousness, out.l.infectiousness, L);
        copy_field(l->open, out.l.open, L);
        copy_field(l->closed_until, out.l.closed_until, L);
        copy_field(l->quarantine_until, out.l.quarantine_until, L);
        return 0;
    } catch (const std::exception& e) {
        std::snprintf(err, (size_t)err_len, "%s", e.what());
        return -1;
    }
}
