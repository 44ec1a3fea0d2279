/*
 * gb300_policies.h — the reference's policy concept over the pansim_gb300 C ABI.
 *
 * khbence/pansim selects its per-step work at compile time: Simulation<...,
 * Movement, Infection, Testing, Closure> (include/simulation.h:53-97)
 * inherits one class template per policy and befriends them (:130-133), and
 * configTypes.h names them (cmake/config/in/configTypes.h.in:9-16).  This
 * header gives four templates with the same surface that run the work on a
 * GB300 through include/pansim_gb300.h:
 *
 *   Gb300Movement<Sim>   replaces RealMovement   (policies/movementPolicies.h:1340-1751):
 *                        addProgramParameters, initializeArgs, init(LocationTypes,
 *                        cemetery), planLocations, movement, and the public
 *                        switches enableCurfew ... quarantinePolicy (:1359-1367)
 *   Gb300Infection<Sim>  replaces BasicInfection (policies/infectionPolicies.h:88-588):
 *                        addProgramParameters, initializeArgs, infectionsAtLocations,
 *                        finalize
 *   Gb300Testing<Sim>    replaces DetailedTesting (policies/testingPolicies.h:318-475):
 *                        addProgramParameters, initializeArgs, init, performTests,
 *                        getStats, updateTestingProbs
 *   Gb300Closure<Sim>    replaces RuleClosure    (policies/closurePolicies.h:48-479):
 *                        addProgramParameters, initializeArgs, init(LocationTypes,
 *                        ClosureRules, header), midnight, step
 *
 * The four are used together (a configTypes.h selecting them is
 * include/gb300_config_types.h).  They are written against the members the
 * reference's policies use, not against its headers, so they compile with the
 * reference's Simulation and with any class that offers the same members:
 *   sim->agents: PPValues (elements laid out as DynamicPPState), agentMetaData
 *     (laid out as BasicAgentMeta), agentStats (AgentStats), location, types,
 *     diagnosed, quarantined, stayedHome, locationOffset, possibleLocations,
 *     possibleTypes;
 *   sim->locs: locType, infectiousness, states, closedUntil, quarantineUntil,
 *     essential, schools, classrooms, classroomOffsets;
 *   sim->timeStep.
 * DynamicPPState and BasicAgentMeta keep their fields private; the adapters
 * read and write them through field mirrors (PPStateFields, AgentMetaFields)
 * whose sizes are checked against the element types at compile time.
 *
 * State ownership.  The simulation state lives in one pansim_gb300 context,
 * created at the first planLocations (every container is loaded by then).
 * During a simulated day the device copy is the current one: planLocations
 * first copies the reference's containers to the device (they hold what the
 * midnight code on the host changed: updateAgents, immunization,
 * otherDisease, the closure rules), and performTests, the first call of the
 * next midnight, ends with the device state copied back into the
 * reference's containers, so that the host midnight code reads the day's
 * results.  The per-location agent list stays on the device (the reference
 * keeps it in locs->locationAgentList / locationListOffsets,
 * movementPolicies.h:1724); Gb300Movement::agentList() copies it out on
 * demand.
 *
 * The model tables the device needs (states, progression tables, dwell
 * lengths, schedules) are the run's input files; the caller hands them over
 * as a psim_model with pansim_gb300::set_model() before the first
 * planLocations (the project's reader of the reference's input files builds
 * it from the same files the reference's DataProvider reads).
 *
 * Errors of the library are thrown as pansim_gb300::Error (the reference
 * throws its CustomErrors at initialization and has no runtime checks).
 */
#ifndef GB300_POLICIES_H
#define GB300_POLICIES_H

#include <cmath>
#include <cstdint>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "pansim_gb300.h"

// The option declarations need cxxopts (the reference's command-line
// library); without it the policies still compile, without
// addProgramParameters.
#if defined(__has_include)
#if __has_include("cxxopts.hpp")
#include "cxxopts.hpp"
#define GB300_POLICIES_HAVE_CXXOPTS 1
#endif
#endif

namespace pansim_gb300 {

struct Error : std::runtime_error {
    explicit Error(const std::string& m) : std::runtime_error(m) {}
};

inline void check(int rc, const psim_ctx* ctx, const char* what) {
    if (rc) throw Error(std::string("pansim_gb300 ") + what + ": " + (ctx ? psim_last_error(ctx) : "error"));
}

// Field mirrors of the reference's agent state classes (same member order and
// types): DynamicPPState (include/agentData/dynamicPPState.h:15-21) and
// BasicAgentMeta (include/agentData/agentMeta.h:24-28).
struct PPStateFields {
    float infectious;
    unsigned progressionID;
    char state;
    short daysBeforeNextState;
    float susceptible[PSIM_MAX_STRAINS];
    uint8_t variant;
};
struct AgentMetaFields {
    float scalingSymptoms[7 * PSIM_MAX_STRAINS];
    float scalingAgeSex;
    uint8_t age;
    uint8_t preCondIdx;
    bool sex;
};

// The run's model tables (set before the first planLocations).
inline const psim_model*& model_slot() {
    static const psim_model* m = nullptr;
    return m;
}
inline void set_model(const psim_model* m) { model_slot() = m; }

// Options the adapters read at initializeArgs (the reference's option
// names and defaults).
struct RunOptions {
    uint32_t start_day = 0, start_date = 0;
    uint32_t quarantine_policy = 3, quarantine_length = 10, tracked = 0xFFFFFFFFu;
    double k = 0.000347;
    double c0 = 3.08, trunc = 0.5;
    std::vector<int> d_offset{-5};
    int d_peak_offset = 0;
    double testing[6] = {0.00005, 0.01, 0.0005, 0.0005, 0.005, 0.05};
    uint32_t testing_delay = 5;
    bool use_pcr = true;
    uint64_t seed = 1;
    bool enable_closures = true;
};

inline std::vector<double> split_doubles(const std::string& s) {
    std::vector<double> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, ',')) out.push_back(std::stod(item));
    return out;
}
inline std::vector<int> split_ints(const std::string& s) {
    std::vector<int> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, ',')) out.push_back(std::stoi(item));
    return out;
}

// element-wise copies between the reference's containers (host or Thrust
// vectors) and host arrays
template <class Vec, class T>
void copy_out(const Vec& v, T* out, size_t n) {
    for (size_t i = 0; i < n; ++i) out[i] = (T)v[i];
}
template <class Vec, class T>
void copy_in(Vec& v, const T* in, size_t n) {
    for (size_t i = 0; i < n; ++i) v[i] = in[i];
}

// One simulation's context and the host arrays of its snapshot (structure of
// arrays, the C ABI's layout).
struct Bridge {
    psim_ctx* ctx = nullptr;
    psim_params params{};
    psim_agents a{};
    psim_locations l{};
    uint32_t N = 0, L = 0, V = 0;
    RunOptions opt;
    // location types of LocationTypes (locationTypesFormat.h:7-26) and the cemetery
    uint32_t home = 0, work = 0, school = 0, classroom = 0, hospital = 0, doctor = 0, public_space = 0, nursery = 0;
    uint32_t cemetery = 0;
    std::vector<psim_closure_rule> rules;
    std::string header;
    // immutable agent data
    std::vector<uint8_t> type, age, band, precond, sex, poss_type;
    std::vector<uint16_t> prog_id;
    std::vector<float> scaling;
    std::vector<uint32_t> loc_offset, poss_loc;
    // mutable agent state
    std::vector<uint32_t> location, steps, last_test, st[13];
    std::vector<int8_t> state, worst_state;
    std::vector<int16_t> days;
    std::vector<uint8_t> variant, diagnosed, quarantined, stayed_home, no_work, imm_count, inf_count, imm_round;
    std::vector<float> infectious, susceptible, scaling_v;
    // locations
    std::vector<uint8_t> ltype, open, essential;
    std::vector<float> w;
    std::vector<uint32_t> closed_until, quarantine_until, schools, classrooms, classroom_offsets;

    Bridge() = default;
    Bridge(const Bridge&) = delete;
    Bridge& operator=(const Bridge&) = delete;
    ~Bridge() {
        if (ctx) psim_destroy(ctx);
    }

    void bind() {
        a.n = N;
        a.n_poss = (uint32_t)poss_loc.size();
        a.type = type.data();
        a.age = age.data();
        a.band = band.data();
        a.prog_id = prog_id.data();
        a.symptom_scaling = scaling.data();
        a.loc_offset = loc_offset.data();
        a.poss_loc = poss_loc.data();
        a.poss_type = poss_type.data();
        a.location = location.data();
        a.steps_until_move = steps.data();
        a.state = state.data();
        a.days = days.data();
        a.variant = variant.data();
        a.infectious = infectious.data();
        a.susceptible = susceptible.data();
        a.diagnosed = diagnosed.data();
        a.quarantined = quarantined.data();
        a.stayed_home = stayed_home.data();
        a.no_work = no_work.data();
        a.last_test = last_test.data();
        uint32_t** stf[13] = {&a.st_infected_ts,     &a.st_infected_loc,    &a.st_worst_ts,          &a.st_worst_end_ts,
                              &a.st_diagnosed_ts,    &a.st_quarantined_ts,  &a.st_quarantined_until, &a.st_days_in_quarantine,
                              &a.st_hospitalized_ts, &a.st_hospitalized_until, &a.st_immunization_ts, &a.st_recovered_ts,
                              &a.st_variant_mask};
        for (int j = 0; j < 13; ++j) *stf[j] = st[j].data();
        a.st_immunization_count = imm_count.data();
        a.st_infected_count = inf_count.data();
        a.st_worst_state = worst_state.data();
        a.precond = precond.data();
        a.imm_round = imm_round.data();
        a.symptom_scaling_v = scaling_v.data();
        a.sex = sex.data();
        l.n = L;
        l.n_schools = (uint32_t)schools.size();
        l.n_classrooms = (uint32_t)classrooms.size();
        l.type = ltype.data();
        l.infectiousness = w.data();
        l.open = open.data();
        l.essential = essential.data();
        l.closed_until = closed_until.data();
        l.quarantine_until = quarantine_until.data();
        l.schools = schools.data();
        l.classrooms = classrooms.data();
        l.classroom_offsets = classroom_offsets.data();
    }

    // the reference's agent and location containers -> the host arrays
    // (mutable state; `all` also the immutable data)
    template <class Sim>
    void gather(Sim* sim, bool all) {
        auto* ag = sim->agents;
        auto* lc = sim->locs;
        using PPS = typename std::decay<decltype(ag->PPValues)>::type::value_type;
        using Meta = typename std::decay<decltype(ag->agentMetaData)>::type::value_type;
        using Stats = typename std::decay<decltype(ag->agentStats)>::type::value_type;
        static_assert(sizeof(PPS) == sizeof(PPStateFields), "PPValues elements are not laid out as DynamicPPState");
        static_assert(sizeof(Meta) == sizeof(AgentMetaFields),
                      "agentMetaData elements are not laid out as BasicAgentMeta");
        if (all) {
            N = (uint32_t)ag->PPValues.size();
            L = (uint32_t)lc->locType.size();
            const psim_model* m = model_slot();
            V = m ? m->n_variants : 1;
            type.resize(N);
            age.resize(N);
            band.resize(N);
            precond.resize(N);
            sex.resize(N);
            prog_id.resize(N);
            scaling.resize(N);
            loc_offset.resize(N + 1);
            location.resize(N);
            steps.resize(N);
            last_test.resize(N);
            for (auto& x : st) x.resize(N);
            state.resize(N);
            worst_state.resize(N);
            days.resize(N);
            for (auto* x : {&variant, &diagnosed, &quarantined, &stayed_home, &no_work, &imm_count, &inf_count, &imm_round})
                x->assign(N, 0);
            infectious.resize(N);
            susceptible.resize((size_t)N * V);
            scaling_v.resize((size_t)N * V);
            // policy-owned state starts as the reference's policies start it
            // (DetailedTesting's lastTest, testingPolicies.h:381-384)
            last_test.assign(N, 0xFFFFFFFFu);
            copy_out(ag->types, type.data(), N);
            std::vector<unsigned long> off(N + 1);
            copy_out(ag->locationOffset, off.data(), N + 1);
            for (uint32_t i = 0; i <= N; ++i) loc_offset[i] = (uint32_t)off[i];
            poss_loc.resize(loc_offset[N]);
            poss_type.resize(loc_offset[N]);
            copy_out(ag->possibleLocations, poss_loc.data(), poss_loc.size());
            copy_out(ag->possibleTypes, poss_type.data(), poss_type.size());
            for (uint32_t i = 0; i < N; ++i) {
                Meta mm = ag->agentMetaData[i];
                AgentMetaFields f;
                std::memcpy(&f, (const void*)&mm, sizeof(f));
                age[i] = f.age;
                band[i] = (uint8_t)std::min<unsigned>(f.age / 10u, PSIM_MAX_BANDS - 1);
                precond[i] = f.preCondIdx;
                sex[i] = f.sex ? 1 : 0;
                scaling[i] = f.scalingAgeSex;
                PPS pp = ag->PPValues[i];
                PPStateFields q;
                std::memcpy(&q, (const void*)&pp, sizeof(q));
                prog_id[i] = (uint16_t)q.progressionID;
            }
            ltype.resize(L);
            w.resize(L);
            open.resize(L);
            essential.resize(L);
            closed_until.resize(L);
            quarantine_until.resize(L);
            copy_out(lc->locType, ltype.data(), L);
            copy_out(lc->essential, essential.data(), L);
            schools.resize(lc->schools.size());
            classrooms.resize(lc->classrooms.size());
            classroom_offsets.resize(lc->classroomOffsets.size());
            copy_out(lc->schools, schools.data(), schools.size());
            copy_out(lc->classrooms, classrooms.data(), classrooms.size());
            copy_out(lc->classroomOffsets, classroom_offsets.data(), classroom_offsets.size());
        }
        copy_out(ag->location, location.data(), N);
        copy_out(ag->diagnosed, diagnosed.data(), N);
        copy_out(ag->quarantined, quarantined.data(), N);
        copy_out(ag->stayedHome, stayed_home.data(), N);
        for (uint32_t i = 0; i < N; ++i) {
            PPS pp = ag->PPValues[i];
            PPStateFields q;
            std::memcpy(&q, (const void*)&pp, sizeof(q));
            infectious[i] = q.infectious;
            state[i] = (int8_t)q.state;
            days[i] = q.daysBeforeNextState;
            variant[i] = q.variant;
            for (uint32_t v = 0; v < V; ++v) susceptible[(size_t)v * N + i] = q.susceptible[v];
            Meta mm = ag->agentMetaData[i];
            AgentMetaFields f;
            std::memcpy(&f, (const void*)&mm, sizeof(f));
            for (uint32_t v = 0; v < V; ++v) scaling_v[(size_t)v * N + i] = f.scalingSymptoms[v * 7 + 6];
            const Stats s = ag->agentStats[i];
            const uint32_t vals[13] = {s.infectedTimestamp,      s.infectedLocation,          s.worstStateTimestamp,
                                       s.worstStateEndTimestamp, s.diagnosedTimestamp,        s.quarantinedTimestamp,
                                       s.quarantinedUntilTimestamp, s.daysInQuarantine,       s.hospitalizedTimestamp,
                                       s.hospitalizedUntilTimestamp, s.immunizationTimestamp, s.recoveredTimestamp,
                                       s.variant};
            for (int j = 0; j < 13; ++j) st[j][i] = vals[j];
            imm_count[i] = s.immunizationCount;
            inf_count[i] = s.infectedCount;
            worst_state[i] = (int8_t)s.worstState;
        }
        copy_out(lc->infectiousness, w.data(), L);
        copy_out(lc->states, open.data(), L);
        copy_out(lc->closedUntil, closed_until.data(), L);
        copy_out(lc->quarantineUntil, quarantine_until.data(), L);
    }

    // the host arrays -> the reference's containers (mutable state)
    template <class Sim>
    void scatter(Sim* sim) {
        auto* ag = sim->agents;
        auto* lc = sim->locs;
        using PPS = typename std::decay<decltype(ag->PPValues)>::type::value_type;
        using Meta = typename std::decay<decltype(ag->agentMetaData)>::type::value_type;
        using Stats = typename std::decay<decltype(ag->agentStats)>::type::value_type;
        copy_in(ag->location, location.data(), N);
        for (uint32_t i = 0; i < N; ++i) {
            ag->diagnosed[i] = diagnosed[i] != 0;
            ag->quarantined[i] = quarantined[i] != 0;
            ag->stayedHome[i] = stayed_home[i] != 0;
            PPS pp = ag->PPValues[i];
            PPStateFields q;
            std::memcpy(&q, (const void*)&pp, sizeof(q));
            q.infectious = infectious[i];
            q.state = (char)state[i];
            q.daysBeforeNextState = days[i];
            q.variant = variant[i];
            for (uint32_t v = 0; v < V; ++v) q.susceptible[v] = susceptible[(size_t)v * N + i];
            std::memcpy((void*)&pp, &q, sizeof(q));
            ag->PPValues[i] = pp;
            Meta mm = ag->agentMetaData[i];
            AgentMetaFields f;
            std::memcpy(&f, (const void*)&mm, sizeof(f));
            for (uint32_t v = 0; v < V; ++v) f.scalingSymptoms[v * 7 + 6] = scaling_v[(size_t)v * N + i];
            std::memcpy((void*)&mm, &f, sizeof(f));
            ag->agentMetaData[i] = mm;
            Stats s = ag->agentStats[i];
            s.infectedTimestamp = st[0][i];
            s.infectedLocation = st[1][i];
            s.worstStateTimestamp = st[2][i];
            s.worstStateEndTimestamp = st[3][i];
            s.diagnosedTimestamp = st[4][i];
            s.quarantinedTimestamp = st[5][i];
            s.quarantinedUntilTimestamp = st[6][i];
            s.daysInQuarantine = st[7][i];
            s.hospitalizedTimestamp = st[8][i];
            s.hospitalizedUntilTimestamp = st[9][i];
            s.immunizationTimestamp = st[10][i];
            s.recoveredTimestamp = st[11][i];
            s.variant = st[12][i];
            s.immunizationCount = imm_count[i];
            s.infectedCount = inf_count[i];
            s.worstState = (char)worst_state[i];
            ag->agentStats[i] = s;
        }
        copy_in(lc->infectiousness, w.data(), L);
        for (uint32_t j = 0; j < L; ++j) lc->states[j] = open[j] != 0;
        copy_in(lc->closedUntil, closed_until.data(), L);
        copy_in(lc->quarantineUntil, quarantine_until.data(), L);
    }

    // the run parameters from the options, the location types and the
    // movement policy's switches (curfew times in minutes, as the reference's
    // closure rules set them before its planLocations converts them)
    template <class Mv>
    void set_params(const Mv& mv, uint32_t time_step) {
        psim_params& p = params;
        p.time_step = time_step;
        p.start_day = opt.start_day;
        p.start_date = opt.start_date;
        p.home_type = home;
        p.work_type = work;
        p.school_type = school;
        p.classroom_type = classroom;
        p.hospital_type = hospital;
        p.doctor_type = doctor;
        p.public_type = public_space;
        p.nursery_type = nursery;
        p.cemetery_loc = cemetery;
        p.quarantine_policy = mv.quarantinePolicy;
        p.quarantine_length = opt.quarantine_length;
        p.enable_curfew = mv.enableCurfew ? 1u : 0u;
        p.curfew_begin = mv.curfewTimeConverted ? mv.curfewBegin : mv.curfewBegin / time_step;
        p.curfew_end = mv.curfewTimeConverted ? mv.curfewEnd : mv.curfewEnd / time_step;
        p.school_age_restriction = mv.schoolAgeRestriction;
        p.holiday_mode = mv.holidayModeActive ? 1u : 0u;
        p.quarantine_immune = mv.quarantineImmuneActive ? 1u : 0u;
        p.lockdown_nonvacc = mv.lockdownNonvaccActive ? 1u : 0u;
        p.testing_enabled = 1;
        p.testing_delay = opt.testing_delay;
        p.use_pcr = opt.use_pcr ? 1u : 0u;
        p.n_bands = PSIM_MAX_BANDS;
        p.tracked = opt.tracked;
        p.k = opt.k;
        p.c0 = opt.c0;
        p.trunc = opt.trunc;
        p.d_offset0 = opt.d_offset.size() > 0 ? opt.d_offset[0] : 0;
        p.d_offset1 = opt.d_offset.size() > 1 ? opt.d_offset[1] : 0;
        p.d_peak_offset = opt.d_peak_offset;
        p.n_d_offset = (int32_t)opt.d_offset.size();
        p.t_random = opt.testing[0];
        p.t_home = opt.testing[1];
        p.t_work = opt.testing[2];
        p.t_school = opt.testing[3];
        p.t_hospital = opt.testing[4];
        p.t_nursery = opt.testing[5];
        p.seed = opt.seed;
        for (int b = 0; b < PSIM_MAX_BANDS; ++b) p.sigma_band[b] = 1.0f;
    }

    // the reference's switches back from the context (closure rules change them)
    template <class Mv>
    void get_switches(Mv& mv) {
        check(psim_get_params(ctx, &params), ctx, "get_params");
        mv.enableCurfew = params.enable_curfew != 0;
        mv.curfewBegin = params.curfew_begin;
        mv.curfewEnd = params.curfew_end;
        mv.curfewTimeConverted = true;
        mv.schoolAgeRestriction = params.school_age_restriction;
        mv.holidayModeActive = params.holiday_mode != 0;
        mv.quarantineImmuneActive = params.quarantine_immune != 0;
        mv.lockdownNonvaccActive = params.lockdown_nonvacc != 0;
        mv.quarantinePolicy = params.quarantine_policy;
        opt.testing[0] = params.t_random;
        opt.testing[1] = params.t_home;
        opt.testing[2] = params.t_work;
        opt.testing[3] = params.t_school;
        opt.testing[4] = params.t_hospital;
        opt.testing[5] = params.t_nursery;
    }

    template <class Sim, class Mv>
    void create(Sim* sim, const Mv& mv) {
        const psim_model* m = model_slot();
        if (!m) throw Error("pansim_gb300: no model tables (call pansim_gb300::set_model before the first day)");
        gather(sim, true);
        bind();
        set_params(mv, sim->timeStep);
        const int rc = psim_create(0, m, &a, &l, &params, nullptr, &ctx);
        if (rc) {
            const std::string msg = ctx ? psim_last_error(ctx) : "psim_create";
            if (ctx) psim_destroy(ctx);
            ctx = nullptr;
            throw Error("pansim_gb300 create: " + msg);
        }
        if (!rules.empty() || !opt.enable_closures)
            check(psim_closures_init(ctx, rules.data(), (uint32_t)rules.size(), header.c_str(), opt.enable_closures ? 1 : 0),
                  ctx, "closures_init");
    }

    // host containers -> device (the switches of `mv` included)
    template <class Sim, class Mv>
    void push(Sim* sim, const Mv& mv) {
        gather(sim, false);
        set_params(mv, sim->timeStep);
        check(psim_set_params(ctx, &params), ctx, "set_params");
        check(psim_upload(ctx, &a, &l), ctx, "upload");
    }

    // device -> host containers
    template <class Sim>
    void pull(Sim* sim) {
        check(psim_download(ctx, &a, &l), ctx, "download");
        scatter(sim);
    }
};

}  // namespace pansim_gb300

// ---------------------------------------------------------------------------
// RealMovement's surface (movementPolicies.h:1340-1751).  Owns the context.
template <typename SimulationType>
class Gb300Movement {
public:
    bool enableCurfew = false;
    unsigned curfewBegin = 0;
    unsigned curfewEnd = 0;
    bool curfewTimeConverted = false;
    unsigned schoolAgeRestriction = 99;
    bool holidayModeActive = false;
    bool quarantineImmuneActive = false;
    bool lockdownNonvaccActive = false;
    unsigned quarantinePolicy = 3;
    pansim_gb300::Bridge gb300;

#ifdef GB300_POLICIES_HAVE_CXXOPTS
    template <class Options>
    static void addProgramParameters(Options& options) {
        options.add_options()("trace", "Trace movements of agent",
                              cxxopts::value<unsigned>()->default_value(std::to_string(0xFFFFFFFFu)))(
            "quarantinePolicy",
            "Quarantine policy: 0 - None, 1 - Agent only, 2 - Agent and household, 3 - + classroom/work, 4 - + school",
            cxxopts::value<unsigned>()->default_value("3"))(
            "quarantineLength", "Length of quarantine in days", cxxopts::value<unsigned>()->default_value("10"))(
            "gb300Seed", "Philox key of the GB300 run's random streams", cxxopts::value<unsigned>()->default_value("1"));
    }
#endif
    template <class Result>
    void initializeArgs(const Result& result) {
        gb300.opt.tracked = result["trace"].template as<unsigned>();
        quarantinePolicy = result["quarantinePolicy"].template as<unsigned>();
        gb300.opt.quarantine_policy = quarantinePolicy;
        gb300.opt.quarantine_length = result["quarantineLength"].template as<unsigned>();
        gb300.opt.seed = result["gb300Seed"].template as<unsigned>();
        try {
            gb300.opt.start_day = result["startDay"].template as<unsigned>();
            gb300.opt.start_date = result["startDate"].template as<unsigned>();
        } catch (...) {
        }
    }
    template <class LocationTypes>
    void init(const LocationTypes& data, unsigned cemeteryID) {
        gb300.home = data.home;
        gb300.work = data.work;
        gb300.school = data.school;
        gb300.classroom = data.classroom;
        gb300.hospital = data.hospital;
        gb300.doctor = data.doctor;
        gb300.public_space = data.publicSpace;
        gb300.nursery = data.nurseryhome;
        gb300.cemetery = cemeteryID;
    }

    // the context exists from the first midnight on
    void gb300Ensure() {
        auto* sim = static_cast<SimulationType*>(this);
        if (!gb300.ctx) gb300.create(sim, *this);
    }

    // RealMovement::planLocations (movementPolicies.h:1428-1622): the host
    // containers (changed by the midnight code) go to the device first
    template <class TimeHandler>
    void planLocations(TimeHandler simTime, unsigned timeStep) {
        (void)timeStep;
        auto* sim = static_cast<SimulationType*>(this);
        if (!gb300.ctx)
            gb300.create(sim, *this);
        else
            gb300.push(sim, *this);
        if (!curfewTimeConverted) {
            curfewBegin /= sim->timeStep;
            curfewEnd /= sim->timeStep;
            curfewTimeConverted = true;
        }
        const uint32_t t = simTime.getTimestamp();
        pansim_gb300::check(psim_plan_day(gb300.ctx, t), gb300.ctx, "plan_day");
    }

    // RealMovement::movement (movementPolicies.h:1625-1724): doMovement for
    // every agent and the per-location agent list of the new positions (on
    // the device; agentList() copies it out)
    template <class TimeHandler>
    void movement(TimeHandler simTime, unsigned timeStep) {
        (void)timeStep;
        gb300Ensure();
        const uint32_t t = simTime.getTimestamp();
        pansim_gb300::check(psim_movement(gb300.ctx, t), gb300.ctx, "movement");
        pansim_gb300::check(psim_regroup(gb300.ctx), gb300.ctx, "regroup");
    }

    // locationListOffsets / locationAgentList of the current positions, each
    // location's agents in ascending id order (stable_sort_by_key's output)
    void agentList(std::vector<uint32_t>& offsets, std::vector<uint32_t>& agentsByLocation) {
        gb300Ensure();
        offsets.resize(gb300.L + 1);
        agentsByLocation.resize(gb300.N);
        pansim_gb300::check(psim_get_csr(gb300.ctx, 1, offsets.data(), agentsByLocation.data()), gb300.ctx, "get_csr");
    }
};

// BasicInfection's surface (infectionPolicies.h:88-588).
template <typename SimulationType>
class Gb300Infection {
    uint32_t lastStep = 0xFFFFFFFFu;

public:
#ifdef GB300_POLICIES_HAVE_CXXOPTS
    template <class Options>
    static void addProgramParameters(Options& options) {
        options.add_options()("k,infectionCoefficient", "Infection: >0 :infectiousness coefficient ",
                              cxxopts::value<double>()->default_value("0.000347"))(
            "d_offset", "seasonality day offset ", cxxopts::value<std::string>()->default_value("-5"))(
            "d_peak_offset", "seasonality peak day offset ", cxxopts::value<int>()->default_value("0"))(
            "trunc", "seasonality truncation value for Omicron ", cxxopts::value<double>()->default_value("0.5"))(
            "c0", "seasonality c0 value ", cxxopts::value<double>()->default_value("3.08"));
    }
#endif
    void finalize() {}

    template <class Result>
    void initializeArgs(const Result& result) {
        auto& b = mv().gb300;
        b.opt.k = result["infectionCoefficient"].template as<double>();
        b.opt.d_offset = pansim_gb300::split_ints(result["d_offset"].template as<std::string>());
        b.opt.d_peak_offset = result["d_peak_offset"].template as<int>();
        b.opt.c0 = result["c0"].template as<double>();
        b.opt.trunc = result["trunc"].template as<double>();
    }

    // BasicInfection::infectionsAtLocations (infectionPolicies.h:481-546):
    // the per-location ratio and the draws.  The device draws every active
    // variant of an agent in one pass (sequential per agent, as the
    // reference's calls per variant are), at the step's first call.
    template <class TimeHandler>
    void infectionsAtLocations(TimeHandler& simTime, unsigned timeStep, uint8_t variant) {
        (void)timeStep;
        (void)variant;
        auto& m = mv();
        m.gb300Ensure();
        const uint32_t t = simTime.getTimestamp();
        if (t == lastStep) return;
        lastStep = t;
        pansim_gb300::check(psim_infect(m.gb300.ctx, t, 0), m.gb300.ctx, "infect");
    }

private:
    Gb300Movement<SimulationType>& mv() {
        return static_cast<Gb300Movement<SimulationType>&>(*static_cast<SimulationType*>(this));
    }
};

// DetailedTesting's surface (testingPolicies.h:318-475).
template <typename SimulationType>
class Gb300Testing {
    uint32_t tests = 0, positive1 = 0, positive2 = 0;

public:
#ifdef GB300_POLICIES_HAVE_CXXOPTS
    template <class Options>
    static void addProgramParameters(Options& options) {
        options.add_options()("testingProbabilities",
                              "Testing probabilities for random, if someone else was diagnosed at home/work/school, and "
                              "random for hospital workers: comma-delimited string "
                              "random,home,work,school,hospital,nurseryHome",
                              cxxopts::value<std::string>()->default_value("0.00005,0.01,0.0005,0.0005,0.005,0.05"))(
            "testingRepeatDelay", "Minimum number of days between taking tests",
            cxxopts::value<unsigned>()->default_value("5"))(
            "testingMethod", "default method for testing. Can be PCR (default) on antigen.",
            cxxopts::value<std::string>()->default_value("PCR"));
    }
#endif
    void updateTestingProbs(const std::string& probsString) {
        auto& b = mv().gb300;
        const std::vector<double> v = pansim_gb300::split_doubles(probsString);
        for (size_t j = 0; j < v.size() && j < 6; ++j) b.opt.testing[j] = v[j];
        if (b.ctx) {
            b.set_params(mv(), static_cast<SimulationType*>(this)->timeStep);
            pansim_gb300::check(psim_set_params(b.ctx, &b.params), b.ctx, "set_params");
        }
    }
    template <class Result>
    void initializeArgs(const Result& result) {
        auto& b = mv().gb300;
        b.opt.testing_delay = result["testingRepeatDelay"].template as<unsigned>();
        updateTestingProbs(result["testingProbabilities"].template as<std::string>());
        const std::string method = result["testingMethod"].template as<std::string>();
        if (method == "PCR")
            b.opt.use_pcr = true;
        else if (method == "antigen")
            b.opt.use_pcr = false;
        else
            throw pansim_gb300::Error("unrecognized testingMethod " + method + " must be either PCR or antigen");
    }
    template <class LocationTypes>
    void init(const LocationTypes& data) {
        (void)data;
    }
    // (tests, positive PCR, positive antigen) of the last performTests
    auto getStats() {
#if defined(THRUST_VERSION)
        return thrust::make_tuple(tests, positive1, positive2);
#else
        return std::make_tuple(tests, positive1, positive2);
#endif
    }

    // DetailedTesting::performTests (testingPolicies.h:370-475), the first
    // call of a midnight: afterwards the device state is copied back into the
    // host containers for the midnight code that runs on them
    template <class TimeHandler>
    void performTests(TimeHandler simTime, unsigned timeStep) {
        (void)timeStep;
        auto& m = mv();
        m.gb300Ensure();
        uint32_t tpp[3] = {0, 0, 0};
        pansim_gb300::check(psim_test_day(m.gb300.ctx, simTime.getTimestamp(), tpp), m.gb300.ctx, "test_day");
        tests = tpp[0];
        positive1 = tpp[1];
        positive2 = tpp[2];
        m.gb300.pull(static_cast<SimulationType*>(this));
    }

private:
    Gb300Movement<SimulationType>& mv() {
        return static_cast<Gb300Movement<SimulationType>&>(*static_cast<SimulationType*>(this));
    }
};

// RuleClosure's surface (closurePolicies.h:48-479) over the library's rule
// engine (psim_closures_init / psim_closures_midnight).
template <typename SimulationType>
class Gb300Closure {
public:
#ifdef GB300_POLICIES_HAVE_CXXOPTS
    template <class Options>
    static void addProgramParameters(Options& options) {
        options.add_options()("enableClosures", "enable(1)/disable(0) closure rules defined in closureRules.json",
                              cxxopts::value<unsigned>()->default_value("1"));
    }
#endif
    template <class Result>
    void initializeArgs(const Result& result) {
        mv().gb300.opt.enable_closures = result["enableClosures"].template as<unsigned>() != 0;
    }
    // the rules of closureRules.json (closuresFormat.h:7-22) and the
    // statistics header (simulation.h:749)
    template <class LocationTypes, class ClosureRules>
    void init(const LocationTypes& data, const ClosureRules& rules, std::string header) {
        (void)data;
        auto& b = mv().gb300;
        b.rules.clear();
        for (const auto& r : rules.rules) {
            psim_closure_rule q;
            std::memset(&q, 0, sizeof(q));
            std::strncpy(q.name, r.name.c_str(), sizeof(q.name) - 1);
            std::strncpy(q.condition_type, r.conditionType.c_str(), sizeof(q.condition_type) - 1);
            q.threshold = r.threshold;
            q.threshold2 = r.threshold2;
            std::strncpy(q.parameter, r.parameter.c_str(), sizeof(q.parameter) - 1);
            q.close_after = r.closeAfter;
            q.open_after = r.openAfter;
            if (r.locationTypesToClose.size() >= PSIM_CLOSURE_MAX_TYPES)
                throw pansim_gb300::Error("closure rule " + r.name + ": too many location types");
            q.n_types = (uint32_t)r.locationTypesToClose.size();
            for (uint32_t j = 0; j < q.n_types; ++j) q.types[j] = r.locationTypesToClose[j];
            b.rules.push_back(q);
        }
        b.header = header;
    }

    // RuleClosure::midnight on the statistics row of the day; the rules'
    // location and switch changes come back into the host containers and the
    // movement policy's switches (which planLocations then sends back)
    template <class TimeHandler>
    void midnight(TimeHandler simTime, unsigned timeStep, std::vector<unsigned>& stats) {
        (void)timeStep;
        auto& m = mv();
        auto& b = m.gb300;
        m.gb300Ensure();
        if (b.rules.empty()) return;
        psim_day_stats row;
        std::memset(&row, 0, sizeof(row));
        row.n = (uint32_t)std::min<size_t>(stats.size(), PSIM_STATS_MAX);
        for (uint32_t j = 0; j < row.n; ++j) row.v[j] = stats[j];
        auto* sim = static_cast<SimulationType*>(this);
        // the host containers are current at midnight: the rules act on them
        b.push(sim, m);
        pansim_gb300::check(psim_closures_midnight(b.ctx, simTime.getTimestamp(), &row), b.ctx, "closures_midnight");
        b.get_switches(m);
        b.pull(sim);
    }
    template <class TimeHandler>
    void step(TimeHandler simTime, unsigned timeStep) {
        (void)simTime;
        (void)timeStep;
    }

private:
    Gb300Movement<SimulationType>& mv() {
        return static_cast<Gb300Movement<SimulationType>&>(*static_cast<SimulationType*>(this));
    }
};

#endif
