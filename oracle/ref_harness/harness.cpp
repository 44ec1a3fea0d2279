// Reference-compiled harness — TEST INFRASTRUCTURE ONLY.
//
// Drives khbence/pansim's own hot-path code, compiled from the reference's
// sources (see oracle/ref_build.py), on a snapshot laid out like the C ABI's
// structs.  Reference code exercised:
//   RealMovementOps::doMovement / findActualLocationForType / quarantineAgent,
//   checkSchoolQuarantine / checkSchoolWorkQuarantine / checkUnderageAtHome /
//   setNoWorkToday               (include/policies/movementPolicies.h)
//   DetailedTestingOps::flagLocations / doTesting (include/policies/testingPolicies.h)
//   Util::updatePerLocationAgentLists, Util::reduce_by_location (src/tools/util.cpp, util.h)
//   DynamicPPState::initTransitionMatrix / update / gotInfected (src/agentData/dynamicPPState.cpp)
//   MultiBadMatrix, LengthOfState (src/tools/progressionMatrices/*.cpp)
//   AgentTypeList::addSchedule / setStayHome / unsetStayHome, TimeDay, Timehandler
//                                (src/agentData/agentType.cpp, src/tools/*.cpp)
//   RuleClosure::init / midnight (include/policies/closurePolicies.h), driven
//                                through a minimal stand-in of Simulation
// The per-step and per-day orchestration (simulation.h:899-926, 425-471;
// movementPolicies.h:1428-1622, 1625-1724; testingPolicies.h:370-475;
// locationList.h:233-310) is restated here around those calls.
//
// Modes:
//  stream mode (pin): the interposed RandomGenerator draws from per-agent Philox
//    streams, agents run sequentially, location quarantine written by an agent
//    becomes visible from the next step with concurrent writes combined by max,
//    and the infection ratio is evaluated from the exact fixed-point sum with
//    psim_hazard; results must equal the oracle bit for bit.
//  native mode: std::mt19937_64 per OpenMP thread with the reference's own
//    distributions, the reference's FP32 reduction (Util::reduce_by_location)
//    and ratio (1 - expf, infectionPolicies.h:545), OpenMP loops as in the
//    reference's CPU build; used for the statistical comparison and as the
//    reference CPU implementation in the benchmark.
#include <fstream>
#include <iterator>

#include "datatypes.h"
#include "timeHandler.h"
#include "timeDay.h"
#include "operators.h"
#include "globalStates.h"
#include "agentStats.h"
#include "agentType.h"
#include "randomGenerator.h"
#include "util.h"
#include "dynamicPPState.h"
#include "agentMeta.h"
#include "progressionType.h"
#include "movementPolicies.h"
#include "testingPolicies.h"
// closurePolicies.h relies on its includer for these
#include <functional>
#include "closuresFormat.h"
#include "locationTypesFormat.h"
#include "closurePolicies.h"
#include "immunization.h"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/pansim_gb300.h"

namespace harness_rng {
int native_mode = 0;
thread_local psim_stream* current = nullptr;
std::vector<std::mt19937_64> generators;
void seed_native(unsigned long long seed) {
    generators.clear();
    int n = omp_get_max_threads();
    for (int i = 0; i < n; ++i) generators.emplace_back(seed * 1000003ull + (unsigned long long)i);
}
}  // namespace harness_rng

namespace {

// Layout mirrors of the reference's classes with private members, used to set
// and read their state (same member order and types).
struct PPMirror {
    float infectious;
    unsigned progressionID;
    char state;
    short daysBeforeNextState;
    float susceptible[MAX_STRAINS];
    uint8_t variant;
};
static_assert(sizeof(PPMirror) == sizeof(DynamicPPState), "DynamicPPState layout");
struct MetaMirror {
    float scalingSymptoms[7 * MAX_STRAINS];
    float scalingAgeSex;
    uint8_t age;
    uint8_t preCondIdx;
    bool sex;
};
static_assert(sizeof(MetaMirror) == sizeof(BasicAgentMeta), "BasicAgentMeta layout");

const char* WB_NAMES[5] = {"W", "N", "M", "S", "D"};

double minutes_to_hmm(unsigned m) {
    if (m >= 255u * 60u) return -1.0;  // undefined duration
    return (double)(m / 60u) + (double)(m % 60u) / 100.0;
}

struct Harness {
    const psim_model* m;
    psim_agents* sa;
    psim_locations* sl;
    psim_params p;
    uint64_t seed;
    double k;
    uint32_t cemetery;
    uint32_t N, L, V, spd;
    bool native;
    AgentTypeList types;
    thrust::device_vector<DynamicPPState> pp;
    std::vector<BasicAgentMeta> meta;
    std::vector<AgentStats> stats;
    std::unique_ptr<bool[]> diagnosed, quarantined, stayedHome, locStates, locFlags;
    thrust::device_vector<unsigned> location, locationIdsOfAgents, locationAgentList, locationListOffsets;
    std::vector<unsigned> types_, steps, lastTest, locType, closedUntil, quarantineUntil, capacity, noWorkLoc;
    std::vector<unsigned long> locOffset;
    std::vector<unsigned> possLoc, possType;
    std::vector<uint8_t> noWorkAgent, essential;
    std::vector<unsigned> schools, classrooms, classroomOffsets;
    std::vector<uint32_t> variantActive;
    thrust::device_vector<float> fullInfectedCounts;
};

void set_stream(psim_stream* s, const Harness& h, uint32_t agent, uint32_t tick, uint32_t phase) {
    psim_stream_init(s, h.seed, agent, tick, phase);
    harness_rng::current = s;
}

void pp_from_snapshot(Harness& h, uint32_t i) {
    PPMirror mm;
    mm.infectious = h.sa->infectious[i];
    mm.progressionID = h.sa->prog_id[i];
    mm.state = (char)h.sa->state[i];
    mm.daysBeforeNextState = h.sa->days[i];
    for (int v = 0; v < MAX_STRAINS; ++v) mm.susceptible[v] = (uint32_t)v < h.V ? h.sa->susceptible[(size_t)v * h.N + i] : 0.0f;
    mm.variant = h.sa->variant[i];
    DynamicPPState tmp = h.pp[i];
    std::memcpy((void*)&tmp, &mm, sizeof(mm));
    h.pp[i] = tmp;
}

void pp_to_snapshot(Harness& h, uint32_t i) {
    DynamicPPState tmp = h.pp[i];
    PPMirror mm;
    std::memcpy(&mm, (const void*)&tmp, sizeof(mm));
    h.sa->infectious[i] = mm.infectious;
    h.sa->state[i] = (int8_t)mm.state;
    h.sa->days[i] = mm.daysBeforeNextState;
    for (uint32_t v = 0; v < h.V; ++v) h.sa->susceptible[(size_t)v * h.N + i] = mm.susceptible[v];
    h.sa->variant[i] = mm.variant;
}

AgentStats stats_from_snapshot(const psim_agents* a, uint32_t i) {
    AgentStats s;
    s.infectedTimestamp = a->st_infected_ts[i];
    s.infectedLocation = a->st_infected_loc[i];
    s.worstStateTimestamp = a->st_worst_ts[i];
    s.worstStateEndTimestamp = a->st_worst_end_ts[i];
    s.diagnosedTimestamp = a->st_diagnosed_ts[i];
    s.quarantinedTimestamp = a->st_quarantined_ts[i];
    s.quarantinedUntilTimestamp = a->st_quarantined_until[i];
    s.daysInQuarantine = a->st_days_in_quarantine[i];
    s.hospitalizedTimestamp = a->st_hospitalized_ts[i];
    s.hospitalizedUntilTimestamp = a->st_hospitalized_until[i];
    s.immunizationTimestamp = a->st_immunization_ts[i];
    s.recoveredTimestamp = a->st_recovered_ts[i];
    s.immunizationCount = a->st_immunization_count[i];
    s.variant = a->st_variant_mask[i];
    s.infectedCount = a->st_infected_count[i];
    s.worstState = (char)a->st_worst_state[i];
    return s;
}

void stats_to_snapshot(const AgentStats& s, psim_agents* a, uint32_t i) {
    a->st_infected_ts[i] = s.infectedTimestamp;
    a->st_infected_loc[i] = s.infectedLocation;
    a->st_worst_ts[i] = s.worstStateTimestamp;
    a->st_worst_end_ts[i] = s.worstStateEndTimestamp;
    a->st_diagnosed_ts[i] = s.diagnosedTimestamp;
    a->st_quarantined_ts[i] = s.quarantinedTimestamp;
    a->st_quarantined_until[i] = s.quarantinedUntilTimestamp;
    a->st_days_in_quarantine[i] = s.daysInQuarantine;
    a->st_hospitalized_ts[i] = s.hospitalizedTimestamp;
    a->st_hospitalized_until[i] = s.hospitalizedUntilTimestamp;
    a->st_immunization_ts[i] = s.immunizationTimestamp;
    a->st_recovered_ts[i] = s.recoveredTimestamp;
    a->st_immunization_count[i] = s.immunizationCount;
    a->st_variant_mask[i] = s.variant;
    a->st_infected_count[i] = s.infectedCount;
    a->st_worst_state[i] = (int8_t)s.worstState;
}

// DynamicPPState::initTransitionMatrix from the snapshot's tables
void init_progression(Harness& h) {
    const psim_model* m = h.m;
    const uint32_t S = m->n_states;
    parser::ProgressionDirectory cfg;
    for (uint32_t s = 0; s < S; ++s) cfg.stateInformation.stateNames.push_back("s" + std::to_string(s));
    cfg.stateInformation.firstInfectedState = "s" + std::to_string(m->first_infected_state);
    cfg.stateInformation.nonCOVIDDeadState = "s" + std::to_string(m->noncovid_dead_state);
    for (uint32_t s = 0; s < S; ++s) {
        if (m->state_susceptible[s]) cfg.stateInformation.susceptibleStates.push_back("s" + std::to_string(s));
        if (m->state_infected[s]) cfg.stateInformation.infectedStates.push_back("s" + std::to_string(s));
        parser::ProgressionDirectory::SingleState st;
        st.stateName = "s" + std::to_string(s);
        st.WB = WB_NAMES[m->state_wb[s]];
        st.infectious = m->state_infectious[s];
        st.accuracyPCR = m->state_acc_pcr[s];
        st.accuracyAntigen = m->state_acc_antigen[s];
        cfg.states.push_back(st);
    }
    std::map<ProgressionType, std::pair<parser::TransitionFormat, unsigned>, std::less<>> input;
    for (uint32_t pid = 0; pid < m->n_prog; ++pid) {
        parser::TransitionFormat tf;
        for (uint32_t s = 0; s < S; ++s) {
            parser::TransitionFormat::SingleState ss;
            ss.stateName = "s" + std::to_string(s);
            const size_t ti = (size_t)pid * S + s;
            for (uint32_t v = 0; v < h.V; ++v) {
                const size_t li = ti * PSIM_MAX_STRAINS + v;
                ss.avgLength.push_back(m->len_avg[li]);
                ss.maxlength.push_back(m->len_max[li] == FLT_MAX ? -1.0f : m->len_max[li]);
            }
            // MultiBadMatrix::NextStatesInit::cleanUp adds the self loop of an empty row
            const bool empty = m->tr_bad_count[ti] == 0 && m->tr_neu_count[ti] == 1 && m->tr_next[m->tr_neu_begin[ti]] == s &&
                               m->tr_chance[m->tr_neu_begin[ti]] == 1.0f && m->len_avg[ti * PSIM_MAX_STRAINS] == -1.0f;
            if (!empty) {
                for (uint32_t q = 0; q < m->tr_bad_count[ti]; ++q) {
                    parser::TransitionFormat::SingleState::Progression pr;
                    pr.name = "s" + std::to_string(m->tr_next[m->tr_bad_begin[ti] + q]);
                    pr.chance = m->tr_chance[m->tr_bad_begin[ti] + q];
                    pr.isBadProgression = true;
                    ss.progressions.push_back(pr);
                }
                for (uint32_t q = 0; q < m->tr_neu_count[ti]; ++q) {
                    parser::TransitionFormat::SingleState::Progression pr;
                    pr.name = "s" + std::to_string(m->tr_next[m->tr_neu_begin[ti] + q]);
                    pr.chance = m->tr_chance[m->tr_neu_begin[ti] + q];
                    pr.isBadProgression = false;
                    ss.progressions.push_back(pr);
                }
            }
            tf.states.push_back(ss);
        }
        parser::ProgressionDirectory::ProgressionFile f;
        f.fileName = "p" + std::to_string(pid);
        f.age = {(int)(pid * 1000), (int)(pid * 1000 + 999)};
        f.preCond = "0";
        input.emplace(ProgressionType(f), std::make_pair(tf, pid));
    }
    std::vector<float> mult(m->variant_multiplier, m->variant_multiplier + h.V);
    DynamicPPState::initTransitionMatrix(input, cfg, mult);
}

void init_meta(Harness& h) {
    parser::Parameters par;
    parser::Parameters::Sex f, mm;
    f.name = "F";
    f.symptoms = 1.0;
    mm.name = "M";
    mm.symptoms = 1.0;
    par.sex = {f, mm};
    parser::Parameters::Age a;
    a.from = 0;
    a.to = -1;
    a.symptoms = 1.0;
    a.transmission = 1.0;
    par.age = {a};
    parser::Parameters::PreCondition pc;
    pc.ID = "0";
    pc.condition = "none";
    pc.symptoms = 1.0;
    par.preCondition = {pc};
    static bool done = false;
    if (!done) {
        BasicAgentMeta::initData(par);
        done = true;
    }
    h.meta.clear();
    h.meta.reserve(h.N);
    for (uint32_t i = 0; i < h.N; ++i) {
        BasicAgentMeta bm('F', h.sa->age[i], "0");
        MetaMirror mir;
        std::memcpy(&mir, (const void*)&bm, sizeof(mir));
        for (int j = 0; j < 7 * MAX_STRAINS; ++j) mir.scalingSymptoms[j] = h.sa->symptom_scaling[i];
        mir.scalingAgeSex = h.sa->symptom_scaling[i];
        // slot v*7+6: the per-variant scaling the immunization rewrites
        if (h.sa->symptom_scaling_v)
            for (uint32_t v = 0; v < h.m->n_variants; ++v)
                mir.scalingSymptoms[v * 7 + 6] = h.sa->symptom_scaling_v[(size_t)v * h.N + i];
        mir.preCondIdx = h.sa->precond ? h.sa->precond[i] : 0;
        std::memcpy((void*)&bm, &mir, sizeof(mir));
        h.meta.push_back(bm);
    }
}

void init_schedules(Harness& h) {
    const psim_model* m = h.m;
    h.types = AgentTypeList(m->n_agent_types);
    for (uint32_t ty = 0; ty < m->n_agent_types; ++ty)
        for (uint32_t wb = 0; wb < 4; ++wb)
            for (uint32_t day = 0; day < 7; ++day) {
                const uint32_t idx = ty * 28 + 7 * wb + day;
                std::vector<AgentTypeList::Event> evs;
                for (uint32_t j = m->event_offset[idx]; j < m->event_offset[idx + 1]; ++j) {
                    parser::AgentTypes::Type::ScheduleUnique::Event e;
                    e.type = (int)m->ev_loc_type[j];
                    e.chance = m->ev_chance[j];
                    e.start = minutes_to_hmm(m->ev_start[j]);
                    e.end = minutes_to_hmm(m->ev_end[j]);
                    e.duration = minutes_to_hmm(m->ev_duration[j]);
                    evs.emplace_back(e);
                }
                if (!evs.empty()) h.types.addSchedule(ty, std::make_pair((states::WBStates)wb, (Days)day), evs);
            }
}

void count_variants(Harness& h) {
    h.variantActive.assign(h.V, 0u);
    for (uint32_t i = 0; i < h.N; ++i) {
        DynamicPPState s = h.pp[i];
        if (s.isInfected()) h.variantActive[s.getVariant()] = 1;
    }
}

RealMovementOps::MovementArguments<DynamicPPState, BasicAgentMeta, unsigned> movement_args(Harness& h, uint32_t t) {
    RealMovementOps::MovementArguments<DynamicPPState, BasicAgentMeta, unsigned> a;
    a.quarantinePolicy = h.p.quarantine_policy;
    a.quarantineLength = h.p.quarantine_length;
    a.tracked = 0xFFFFFFFFu;
    a.hospitalType = h.p.hospital_type;
    a.homeType = h.p.home_type;
    a.publicPlaceType = h.p.public_type;
    a.doctorType = h.p.doctor_type;
    a.timeStep = h.p.time_step;
    a.simTime = TimeDay((unsigned)((t % h.spd) * h.p.time_step));
    a.cemeteryLoc = h.cemetery;
    a.schoolType = h.p.school_type;
    a.classroomType = h.p.classroom_type;
    a.workType = h.p.work_type;
    a.enableCurfew = h.p.enable_curfew != 0;
    a.curfewBegin = h.p.curfew_begin;
    a.curfewEnd = h.p.curfew_end;
    a.schoolAgeRestriction = h.p.school_age_restriction;
    a.quarantineImmuneActive = h.p.quarantine_immune != 0;
    a.lockdownNonvaccActive = h.p.lockdown_nonvacc != 0;
    a.locationStatesPtr = h.locStates.get();
    a.closedUntilPtr = h.closedUntil.data();
    a.locationCapacitiesPtr = h.capacity.data();
    a.locationQuarantineUntilPtr = h.quarantineUntil.data();
    a.locationTypePtr = h.locType.data();
    a.essentialLocPtr = h.essential.data();
    a.agentLocationsPtr = thrust::raw_pointer_cast(h.location.data());
    a.agentTypesPtr = h.types_.data();
    a.agentStatesPtr = thrust::raw_pointer_cast(h.pp.data());
    a.agentMetaDataPtr = h.meta.data();
    a.diagnosedPtr = h.diagnosed.get();
    a.stayedHomePtr = h.stayedHome.get();
    a.quarantinedPtr = h.quarantined.get();
    a.agentStatsPtr = h.stats.data();
    a.stepsUntilMovePtr = h.steps.data();
    a.noWorkAgentPtr = h.noWorkAgent.data();
    a.locationOffsetPtr = h.locOffset.data();
    a.possibleLocationsPtr = h.possLoc.data();
    a.possibleTypesPtr = h.possType.data();
    a.eventOffsetPtr = thrust::raw_pointer_cast(h.types.eventOffset.data());
    a.eventsPtr = thrust::raw_pointer_cast(h.types.events.data());
    a.day = h.p.holiday_mode ? Days::SUNDAY : (Days)((h.p.start_day + t / h.spd) % 7u);
    a.timestamp = t;
    return a;
}

// RealMovement::movement (movementPolicies.h:1625-1724)
void movement(Harness& h, uint32_t t) {
    auto a = movement_args(h, t);
    if (h.native) {
#pragma omp parallel for
        for (unsigned i = 0; i < h.N; i++) RealMovementOps::doMovement(i, a);
    } else if (h.p.quarantine_policy > 1) {
        // location quarantine written during the step becomes visible from the
        // next step; concurrent writes combine with max
        std::vector<unsigned> start(h.quarantineUntil), pending(h.L, 0u);
        psim_stream s;
        for (unsigned i = 0; i < h.N; i++) {
            set_stream(&s, h, i, t, PSIM_PHASE_MOVE);
            RealMovementOps::doMovement(i, a);
            for (unsigned long q = h.locOffset[i]; q < h.locOffset[i + 1]; ++q) {
                const unsigned l = h.possLoc[q];
                if (h.quarantineUntil[l] != start[l]) {
                    pending[l] = std::max(pending[l], h.quarantineUntil[l]);
                    h.quarantineUntil[l] = start[l];
                }
            }
        }
        for (unsigned l = 0; l < h.L; ++l) h.quarantineUntil[l] = std::max(start[l], pending[l]);
    } else {
        psim_stream s;
        for (unsigned i = 0; i < h.N; i++) {
            set_stream(&s, h, i, t, PSIM_PHASE_MOVE);
            RealMovementOps::doMovement(i, a);
        }
    }
    Util::updatePerLocationAgentLists(h.location, h.locationIdsOfAgents, h.locationAgentList, h.locationListOffsets);
}

// BasicInfection::seasonalityMultiplier (infectionPolicies.h:443-478), the
// reference's formula with its default options
double seasonality(const psim_params& p, uint32_t t, uint32_t spd) {
    unsigned simDay = t / spd;
    int d = (int)p.start_date + (int)simDay;
    int d_peak = 59 + 22;
    d += 6;
    double c0 = 3.08;
    double trunc_val = 0.5;
    if (simDay > 250 && simDay < 450) {
        d += p.d_offset0;
        d_peak += p.d_peak_offset;
        c0 = p.c0;
    } else if (simDay > 600) {
        trunc_val = p.trunc;
        if (p.n_d_offset > 1) d += p.d_offset1;
    }
    int d_mod = d % 366;
    if (d_mod > 366 / 2) d_mod = 366 - d_mod;
    double normed = (0.5 * c0 * cos(2.0 * M_PI * (double)(d_mod - d_peak) / 366.0) + (1.0 - 0.5 * c0)) /
                    (0.5 * c0 * cos(2.0 * M_PI * (double)(d_peak - d_peak) / 366.0) + (1.0 - 0.5 * c0));
    double calc_val = std::min(std::max(normed, trunc_val), 1.0);
    if (d_mod < d_peak) return 1.0;
    return calc_val;
}

// BasicInfection::infectionsAtLocations (infectionPolicies.h:481-546) and
// LocationsList::infectAgents (locationList.h:233-310)
void infection(Harness& h, uint32_t t, uint8_t variant) {
    std::vector<float> ratio(h.L, 0.0f);
    const unsigned* off = thrust::raw_pointer_cast(h.locationListOffsets.data());
    const unsigned* lst = thrust::raw_pointer_cast(h.locationAgentList.data());
    const float season = (float)seasonality(h.p, t, h.spd);
    const float tmpK = (float)h.k;
    if (h.native) {
        h.fullInfectedCounts.resize(h.L);
        thrust::fill(h.fullInfectedCounts.begin(), h.fullInfectedCounts.end(), 0.0f);
        Util::reduce_by_location(h.locationListOffsets, h.locationAgentList, h.fullInfectedCounts, h.pp, h.location,
                                 h.locationIdsOfAgents,
                                 [variant](const DynamicPPState& s) -> float { return s.isInfectious(variant); });
        const float* S = thrust::raw_pointer_cast(h.fullInfectedCounts.data());
        const float dtf = (float)h.p.time_step;
#pragma omp parallel for
        for (unsigned l = 0; l < h.L; ++l) {
            const float num = S[l];
            if (num == 0.0f) continue;
            const float dens = num / (off[l + 1] - off[l]);
            ratio[l] = 1.0f - expf(-tmpK * dens * h.sl->infectiousness[l] * season * dtf);
        }
    } else {
        for (unsigned l = 0; l < h.L; ++l) {
            long long fix = 0;
            for (unsigned j = off[l]; j < off[l + 1]; ++j) {
                DynamicPPState s = h.pp[lst[j]];
                fix += (long long)llrintf(s.isInfectious(variant) * PSIM_FIX_SCALE_F);
            }
            ratio[l] = psim_hazard(fix, off[l + 1] - off[l], tmpK, h.sl->infectiousness[l], season, h.p.time_step);
        }
    }
    DynamicPPState* pp = thrust::raw_pointer_cast(h.pp.data());
    const unsigned* loc = thrust::raw_pointer_cast(h.location.data());
    auto body = [&](unsigned i) {
        DynamicPPState& ppstate = pp[i];
        const float r = ratio[loc[i]];
        if (ppstate.getSusceptible(variant) > 0.0f && RandomGenerator::randomUnit() < r * ppstate.getSusceptible(variant)) {
            ppstate.gotInfected(variant);
            AgentStats& st = h.stats[i];
            st.infectedTimestamp = t;
            st.infectedCount++;
            st.infectedLocation = loc[i];
            st.worstState = ppstate.getStateIdx();
            st.worstStateTimestamp = t;
            st.variant |= 1 << variant;
        }
    };
    if (h.native) {
#pragma omp parallel for
        for (unsigned i = 0; i < h.N; ++i) body(i);
    } else {
        psim_stream s;
        for (unsigned i = 0; i < h.N; ++i) {
            set_stream(&s, h, i, t, PSIM_PHASE_INFECT + variant);
            body(i);
        }
    }
}

// Simulation::updateAgents (simulation.h:425-471)
void progress(Harness& h, uint32_t t) {
    DynamicPPState* pp = thrust::raw_pointer_cast(h.pp.data());
    auto body = [&](unsigned i) {
        DynamicPPState& ppstate = pp[i];
        BasicAgentMeta& meta = h.meta[i];
        float progScaling;
        if (ppstate.getStateIdx() == 7)
            progScaling = h.m->death_scaling[ppstate.getVariant()] / meta.getScalingSymptoms(ppstate.getVariant(), ppstate.getStateIdx());
        else
            progScaling = h.m->prog_scaling[ppstate.getVariant()];
        bool recovered = ppstate.update(meta.getScalingSymptoms(ppstate.getVariant(), ppstate.getStateIdx()) * progScaling,
                                        h.stats[i], meta, t, i, 0xFFFFFFFFu, h.p.time_step);
        if (recovered) h.diagnosed[i] = false;
    };
    if (h.native) {
#pragma omp parallel for
        for (unsigned i = 0; i < h.N; ++i) body(i);
    } else {
        psim_stream s;
        for (unsigned i = 0; i < h.N; ++i) {
            set_stream(&s, h, i, t, PSIM_PHASE_PROGRESS);
            body(i);
        }
    }
}

// DetailedTesting::performTests (testingPolicies.h:370-475)
void testing(Harness& h, uint32_t t) {
    DetailedTestingOps::TestingArguments<DynamicPPState, unsigned> a;
    a.timestamp = t;
    std::fill(h.locFlags.get(), h.locFlags.get() + h.L, false);
    a.tracked = 0xFFFFFFFFu;
    a.locationFlagsPtr = h.locFlags.get();
    a.lastTestPtr = h.lastTest.data();
    a.hospitalType = h.p.hospital_type;
    a.homeType = h.p.home_type;
    a.publicPlaceType = h.p.public_type;
    a.doctorType = h.p.doctor_type;
    a.timeStep = h.p.time_step;
    a.schoolType = h.p.school_type;
    a.classroomType = h.p.classroom_type;
    a.nurseryhomeType = h.p.nursery_type;
    a.workType = h.p.work_type;
    a.testingHome = h.p.t_home;
    a.testingWork = h.p.t_work;
    a.testingSchool = h.p.t_school;
    a.testingRandomHospital = h.p.t_hospital;
    a.testingRandom = h.p.t_random;
    a.testingDelay = h.p.testing_delay;
    a.quarantineLength = h.p.quarantine_length;
    a.testingNurseryHome = h.p.t_nursery;
    a.usePCR = h.p.use_pcr != 0;
    a.agentStatsPtr = h.stats.data();
    a.agentStatesPtr = thrust::raw_pointer_cast(h.pp.data());
    a.diagnosedPtr = h.diagnosed.get();
    a.locationTypePtr = h.locType.data();
    a.locationOffsetPtr = h.locOffset.data();
    a.possibleLocationsPtr = h.possLoc.data();
    a.possibleTypesPtr = h.possType.data();
    a.locationQuarantineUntilPtr = h.quarantineUntil.data();
    if (h.native) {
#pragma omp parallel for
        for (unsigned i = 0; i < h.N; i++) DetailedTestingOps::flagLocations(i, a);
#pragma omp parallel for
        for (unsigned i = 0; i < h.N; i++) DetailedTestingOps::doTesting(i, a);
    } else {
        psim_stream s;
        for (unsigned i = 0; i < h.N; i++) {
            set_stream(&s, h, i, t, PSIM_PHASE_TEST_FLAG);
            DetailedTestingOps::flagLocations(i, a);
        }
        for (unsigned i = 0; i < h.N; i++) {
            set_stream(&s, h, i, t, PSIM_PHASE_TEST);
            DetailedTestingOps::doTesting(i, a);
        }
    }
}

// RealMovement::planLocations (movementPolicies.h:1428-1622)
void plan(Harness& h, uint32_t t) {
    std::fill(h.steps.begin(), h.steps.end(), h.p.curfew_end);
    std::fill(h.stayedHome.get(), h.stayedHome.get() + h.N, true);
    std::fill(h.noWorkLoc.begin(), h.noWorkLoc.end(), 0u);
    std::fill(h.noWorkAgent.begin(), h.noWorkAgent.end(), (uint8_t)0);
    const unsigned home = h.p.home_type, work = h.p.work_type, school = h.p.school_type, classroom = h.p.classroom_type;
    psim_stream s;
    if (h.p.quarantine_policy > 3) {
        for (unsigned i = 0; i < h.schools.size(); i++)
            RealMovementOps::checkSchoolQuarantine(i, h.schools.data(), h.classrooms.data(), h.classroomOffsets.data(),
                                                   h.quarantineUntil.data(), t);
    }
    if (h.p.quarantine_policy > 2) {
        for (unsigned i = 0; i < h.N; i++) {
            if (!h.native) set_stream(&s, h, i, t, PSIM_PHASE_PLAN_SWQ);
            RealMovementOps::checkSchoolWorkQuarantine(i, h.stats.data(), thrust::raw_pointer_cast(h.pp.data()),
                                                       h.quarantined.get(), h.quarantineUntil.data(), h.locOffset.data(),
                                                       h.possLoc.data(), h.possType.data(), home, work, school, classroom, t,
                                                       h.p.time_step, 0xFFFFFFFFu);
        }
        for (unsigned l = 0; l < h.L; ++l) {
            if (h.quarantineUntil[l] > t && (h.locType[l] == school || h.locType[l] == classroom)) {
                h.closedUntil[l] = h.quarantineUntil[l];
                h.quarantineUntil[l] = 0;
            } else if (h.quarantineUntil[l] > t && h.locType[l] == work) {
                h.quarantineUntil[l] = 0;
            }
        }
    }
    for (unsigned i = 0; i < h.N; i++) {
        if (!h.native) set_stream(&s, h, i, t, PSIM_PHASE_PLAN_UNDERAGE);
        RealMovementOps::checkUnderageAtHome(i, h.noWorkLoc.data(), h.meta.data(), h.quarantined.get(), h.locStates.get(),
                                             h.closedUntil.data(), h.locOffset.data(), h.possLoc.data(), h.possType.data(),
                                             home, school, classroom, t, h.p.school_age_restriction);
    }
    for (unsigned i = 0; i < h.N; i++) {
        if (!h.native) set_stream(&s, h, i, t, PSIM_PHASE_PLAN_NOWORK);
        RealMovementOps::setNoWorkToday(i, h.noWorkLoc.data(), h.noWorkAgent.data(), h.meta.data(), h.locOffset.data(),
                                        h.possLoc.data(), h.possType.data(), home);
    }
}


// ---------------------------------------------------------------------------
// RuleClosure driven through a stand-in of Simulation: the members and
// switches RuleClosure reaches through its CRTP cast (closurePolicies.h:84-471,
// simulation.h:963-973), backed by the harness state.  Location and agent
// arrays are copied into the stand-in's containers around each midnight call.
struct ClosureLocs {
    thrust::device_vector<float> infectiousness;
    thrust::device_vector<unsigned> locType;
    thrust::device_vector<bool> states;
    thrust::device_vector<uint8_t> essential;
};
struct ClosureAgents {
    thrust::device_vector<unsigned>& location;
    thrust::device_vector<DynamicPPState>& PPValues;
    thrust::device_vector<AgentStats> agentStats;
    AgentTypeList& agentTypes;
};
struct ClosureSim : public RuleClosure<ClosureSim> {
    using TypeOfLocation_t = unsigned;
    using PPState_t = DynamicPPState;
    Harness* h = nullptr;
    ClosureLocs locsStore;
    ClosureLocs* locs = &locsStore;
    std::unique_ptr<ClosureAgents> agentsStore;
    ClosureAgents* agents = nullptr;
    double currentMaskValue = 1.0;
    std::vector<float> infectiousnessMultiplier;
    uint32_t now = 0;
    // Simulation::toggle* (simulation.h:963-973); the harness keeps curfew
    // times in steps, which RealMovement::planLocations converts to on its
    // next call (movementPolicies.h:1440-1444)
    void toggleCurfew(bool enable, unsigned b, unsigned e) {
        h->p.enable_curfew = enable;
        h->p.curfew_begin = b / h->p.time_step;
        h->p.curfew_end = e / h->p.time_step;
    }
    void setSchoolAgeRestriction(unsigned limit) { h->p.school_age_restriction = limit; }
    void toggleHolidayMode(bool enable) { h->p.holiday_mode = enable; }
    void toggleQuarantineImmune(bool enable) { h->p.quarantine_immune = enable; }
    void toggleLockdownNonvacc(bool enable) { h->p.lockdown_nonvacc = enable; }
    void quarantinePolicy(unsigned qp) { h->p.quarantine_policy = qp; }
    // DetailedTesting::updateTestingProbs (testingPolicies.h:328-338)
    void updateTestingProbs(const std::string& probs) {
        std::vector<double> v = splitStringDouble(probs, ',');
        double* dst[6] = {&h->p.t_random, &h->p.t_home, &h->p.t_work, &h->p.t_school, &h->p.t_hospital, &h->p.t_nursery};
        for (size_t q = 0; q < v.size() && q < 6; ++q) *dst[q] = v[q];
    }
    Timehandler getSimTime() {
        Timehandler th(h->p.time_step, 0, Days::MONDAY, 0);
        for (uint32_t q = 0; q < now; ++q) ++th;
        return th;
    }
    void pull() {
        const uint32_t L = h->L;
        locs->infectiousness.assign(h->sl->infectiousness, h->sl->infectiousness + L);
        locs->locType.assign(h->locType.begin(), h->locType.end());
        locs->states.resize(L);
        for (uint32_t j = 0; j < L; ++j) locs->states[j] = h->locStates[j];
        locs->essential.assign(h->essential.begin(), h->essential.end());
        agents->agentStats.assign(h->stats.begin(), h->stats.end());
    }
    void push() {
        for (uint32_t j = 0; j < h->L; ++j) {
            h->sl->infectiousness[j] = locs->infectiousness[j];
            h->locStates[j] = locs->states[j];
        }
        for (uint32_t i = 0; i < h->N; ++i) h->stats[i] = agents->agentStats[i];
    }
};
std::unique_ptr<ClosureSim> g_closure;

// ---------------------------------------------------------------------------
// Immunization driven through a stand-in of Simulation (the members
// Immunization reaches through its `sim` pointer, immunization.h:25-900),
// with the harness state copied in and out around each call.
struct ImmAgents {
    thrust::device_vector<DynamicPPState>& PPValues;
    thrust::device_vector<AgentStats> agentStats;
    thrust::device_vector<BasicAgentMeta> agentMetaData;
    thrust::device_vector<unsigned long> locationOffset;
    thrust::device_vector<unsigned> possibleTypes, possibleLocations;
};
struct ImmLocs {
    thrust::device_vector<unsigned> locType;
    thrust::device_vector<uint8_t> essential;
};
struct ImmSim {
    using PPState_t = DynamicPPState;
    using AgentMeta_t = BasicAgentMeta;
    ImmAgents* agents = nullptr;
    ImmLocs* locs = nullptr;
    std::vector<float> infectiousnessMultiplier;
};
struct ImmHarness {
    Harness* h = nullptr;
    std::unique_ptr<ImmAgents> agents;
    ImmLocs locs;
    ImmSim sim;
    std::unique_ptr<Immunization<ImmSim>> imm;
    void pull() {
        agents->agentStats.assign(h->stats.begin(), h->stats.end());
        agents->agentMetaData.assign(h->meta.begin(), h->meta.end());
    }
    void push() {
        for (uint32_t i = 0; i < h->N; ++i) {
            h->stats[i] = agents->agentStats[i];
            h->meta[i] = agents->agentMetaData[i];
        }
    }
};
std::unique_ptr<ImmHarness> g_imm;
std::string join_floats(const float* v, int n) {
    std::string s;
    char buf[64];
    for (int q = 0; q < n; ++q) {
        std::snprintf(buf, sizeof(buf), "%.9g", (double)v[q]);
        s += (q ? "," : "") + std::string(buf);
    }
    return s;
}
std::string join_ints(const int32_t* v, int n) {
    std::string s;
    for (int q = 0; q < n; ++q) s += (q ? "," : "") + std::to_string(v[q]);
    return s;
}

}  // namespace

extern "C" {

void* ref_create(const psim_model* m, psim_agents* a, psim_locations* l, const psim_params* p, int native,
                 unsigned long long native_seed) {
    Harness* h = new Harness();
    h->m = m;
    h->sa = a;
    h->sl = l;
    h->p = *p;
    h->seed = p->seed;
    h->k = p->k;
    h->cemetery = p->cemetery_loc;
    h->N = a->n;
    h->L = l->n;
    h->V = m->n_variants;
    h->spd = 1440u / p->time_step;
    h->native = native != 0;
    harness_rng::native_mode = native;
    if (native) harness_rng::seed_native(native_seed);
    psim_stream dummy;
    psim_stream_init(&dummy, 0, 0, 0, 0);
    harness_rng::current = &dummy;
    init_progression(*h);
    init_meta(*h);
    init_schedules(*h);
    const uint32_t N = h->N, L = h->L;
    h->pp = thrust::device_vector<DynamicPPState>(N);
    for (uint32_t i = 0; i < N; ++i) pp_from_snapshot(*h, i);
    h->stats.resize(N);
    for (uint32_t i = 0; i < N; ++i) h->stats[i] = stats_from_snapshot(a, i);
    h->diagnosed.reset(new bool[N]);
    h->quarantined.reset(new bool[N]);
    h->stayedHome.reset(new bool[N]);
    for (uint32_t i = 0; i < N; ++i) {
        h->diagnosed[i] = a->diagnosed[i] != 0;
        h->quarantined[i] = a->quarantined[i] != 0;
        h->stayedHome[i] = a->stayed_home[i] != 0;
    }
    h->location = thrust::device_vector<unsigned>(a->location, a->location + N);
    h->locationIdsOfAgents.resize(N);
    h->locationAgentList.resize(N);
    h->locationListOffsets.resize(L + 1);
    h->types_.assign(a->type, a->type + N);
    h->steps.assign(a->steps_until_move, a->steps_until_move + N);
    h->lastTest.assign(a->last_test, a->last_test + N);
    h->noWorkAgent.assign(a->no_work, a->no_work + N);
    h->locOffset.assign(a->loc_offset, a->loc_offset + N + 1);
    h->possLoc.assign(a->poss_loc, a->poss_loc + a->n_poss);
    h->possType.assign(a->poss_type, a->poss_type + a->n_poss);
    h->locType.assign(l->type, l->type + L);
    h->locStates.reset(new bool[L]);
    h->locFlags.reset(new bool[L]);
    for (uint32_t j = 0; j < L; ++j) h->locStates[j] = l->open[j] != 0;
    h->closedUntil.assign(l->closed_until, l->closed_until + L);
    h->quarantineUntil.assign(l->quarantine_until, l->quarantine_until + L);
    h->capacity.assign(L, 0xFFFFFFFFu);
    h->essential.assign(l->essential, l->essential + L);
    h->noWorkLoc.assign(L, 0u);
    if (l->n_schools) {
        h->schools.assign(l->schools, l->schools + l->n_schools);
        h->classrooms.assign(l->classrooms, l->classrooms + l->n_classrooms);
        h->classroomOffsets.assign(l->classroom_offsets, l->classroom_offsets + l->n_schools + 1);
    }
    // LocationsList::initialize (locationList.h:224-230)
    Util::updatePerLocationAgentLists(h->location, h->locationIdsOfAgents, h->locationAgentList, h->locationListOffsets);
    count_variants(*h);
    return h;
}

void ref_destroy(void* hp) { delete (Harness*)hp; }

void ref_set_params(void* hp, const psim_params* p) { ((Harness*)hp)->p = *p; }

// the midnight block of runSimulation (simulation.h:906-917) without statistics
void ref_midnight(void* hp, uint32_t t) {
    Harness& h = *(Harness*)hp;
    if (t > 0 && h.p.testing_enabled) testing(h, t);
    if (t > 0) progress(h, t);
    plan(h, t);
    count_variants(h);
}

void ref_movement(void* hp, uint32_t t) { movement(*(Harness*)hp, t); }

void ref_step(void* hp, uint32_t t) {
    Harness& h = *(Harness*)hp;
    movement(h, t);
    for (uint32_t v = 0; v < h.V; ++v)
        if (h.variantActive[v]) infection(h, t, (uint8_t)v);
}

void ref_run_day(void* hp, uint32_t day) {
    Harness& h = *(Harness*)hp;
    const uint32_t t0 = day * h.spd;
    ref_midnight(hp, t0);
    for (uint32_t s = 0; s < h.spd; ++s) ref_step(hp, t0 + s);
}

// AoS state -> the snapshot's SoA arrays
void ref_sync_out(void* hp) {
    Harness& h = *(Harness*)hp;
    psim_agents* a = h.sa;
    for (uint32_t i = 0; i < h.N; ++i) {
        pp_to_snapshot(h, i);
        stats_to_snapshot(h.stats[i], a, i);
        a->location[i] = h.location[i];
        a->steps_until_move[i] = h.steps[i];
        a->diagnosed[i] = h.diagnosed[i] ? 1 : 0;
        a->quarantined[i] = h.quarantined[i] ? 1 : 0;
        a->stayed_home[i] = h.stayedHome[i] ? 1 : 0;
        a->no_work[i] = h.noWorkAgent[i];
        a->last_test[i] = h.lastTest[i];
        if (a->symptom_scaling_v) {
            MetaMirror mir;
            std::memcpy(&mir, (const void*)&h.meta[i], sizeof(mir));
            for (uint32_t v = 0; v < h.m->n_variants; ++v) a->symptom_scaling_v[(size_t)v * h.N + i] = mir.scalingSymptoms[v * 7 + 6];
        }
    }
    for (uint32_t j = 0; j < h.L; ++j) {
        h.sl->closed_until[j] = h.closedUntil[j];
        h.sl->quarantine_until[j] = h.quarantineUntil[j];
        h.sl->open[j] = h.locStates[j] ? 1 : 0;
    }
}

void ref_csr(void* hp, uint32_t* off, uint32_t* agents) {
    Harness& h = *(Harness*)hp;
    for (uint32_t j = 0; j <= h.L; ++j) off[j] = h.locationListOffsets[j];
    for (uint32_t i = 0; i < h.N; ++i) agents[i] = h.locationAgentList[i];
}

// schedule times as the reference's TimeDay parses the H.MM encoding
void ref_event_minutes(void* hp, uint16_t* start, uint16_t* end, uint16_t* dur) {
    Harness& h = *(Harness*)hp;
    for (size_t j = 0; j < h.types.events.size(); ++j) {
        AgentTypeList::Event e = h.types.events[j];
        start[j] = (uint16_t)e.start.getMinutes();
        end[j] = (uint16_t)e.end.getMinutes();
        dur[j] = (uint16_t)e.duration.getMinutes();
    }
}

int ref_threads(void) { return omp_get_max_threads(); }

// test + progression (the midnight block before the statistics)
void ref_midnight_pre(void* hp, uint32_t t) {
    Harness& h = *(Harness*)hp;
    if (t > 0 && h.p.testing_enabled) testing(h, t);
    if (t > 0) progress(h, t);
}

// daily plan, then the variant gate (the midnight block after the rules)
void ref_plan(void* hp, uint32_t t) {
    Harness& h = *(Harness*)hp;
    plan(h, t);
    count_variants(h);
}

void ref_get_params(void* hp, psim_params* out) { *out = ((Harness*)hp)->p; }

// RuleClosure::init with the rules given as C-ABI structs
int ref_closures_init(void* hp, const psim_closure_rule* rules, uint32_t n, const char* header, int enable) {
    Harness& h = *(Harness*)hp;
    g_closure.reset(new ClosureSim());
    ClosureSim& cs = *g_closure;
    cs.h = &h;
    cs.agentsStore.reset(new ClosureAgents{h.location, h.pp, {}, h.types});
    cs.agents = cs.agentsStore.get();
    cs.infectiousnessMultiplier.assign(h.V, 1.0f);
    cs.enableClosures = enable ? 1u : 0u;
    cs.diagnosticLevel = 0;
    cs.pull();
    parser::LocationTypes lt{};
    lt.home = h.p.home_type;
    parser::ClosureRules cr;
    for (uint32_t q = 0; q < n; ++q) {
        parser::ClosureRules::Rule r;
        r.name = rules[q].name;
        r.conditionType = rules[q].condition_type;
        r.threshold = rules[q].threshold;
        r.threshold2 = rules[q].threshold2;
        r.parameter = rules[q].parameter;
        r.closeAfter = rules[q].close_after;
        r.openAfter = rules[q].open_after;
        for (uint32_t j = 0; j < rules[q].n_types; ++j) r.locationTypesToClose.push_back(rules[q].types[j]);
        cr.rules.push_back(r);
    }
    try {
        cs.init(lt, cr, std::string(header));
    } catch (const std::exception&) {
        return 1;
    }
    return 0;
}

// RuleClosure::midnight on a statistics row
void ref_closures_midnight(void* hp, uint32_t t, const uint32_t* row, uint32_t n) {
    ClosureSim& cs = *g_closure;
    cs.now = t;
    std::vector<unsigned> stats(row, row + n);
    cs.pull();
    Timehandler th = cs.getSimTime();
    // ExposeToMutation draws inside a for_each that does not expose the agent
    // index: one shared stream (tests make those draws outcome-free)
    psim_stream s;
    set_stream(&s, *cs.h, 0, t, PSIM_PHASE_EXPOSE);
    cs.midnight(th, cs.h->p.time_step, stats);
    harness_rng::current = nullptr;
    cs.push();
}

void ref_closures_status(void* hp, uint8_t* active, uint8_t* open, uint32_t* n) {
    ClosureSim& cs = *g_closure;
    *n = (uint32_t)cs.rules.size();
    for (size_t q = 0; q < cs.rules.size(); ++q) {
        active[q] = cs.rules[q].conditions[0]->active ? 1 : 0;
        open[q] = cs.rules[q].previousOpenState ? 1 : 0;
    }
}

// Immunization::initializeArgs (options given as the reference's strings; the
// weekly schedules as files under `dir`) + initCategories
int ref_immunization_init(void* hp, const psim_immunization* p, const char* dir) {
    Harness& h = *(Harness*)hp;
    g_imm.reset(new ImmHarness());
    ImmHarness& ih = *g_imm;
    ih.h = &h;
    ih.agents.reset(new ImmAgents{h.pp, {}, {}, {}, {}, {}});
    ih.agents->locationOffset.assign(h.locOffset.begin(), h.locOffset.end());
    ih.agents->possibleTypes.assign(h.possType.begin(), h.possType.end());
    ih.agents->possibleLocations.assign(h.possLoc.begin(), h.possLoc.end());
    ih.locs.locType.assign(h.locType.begin(), h.locType.end());
    ih.locs.essential.assign(h.essential.begin(), h.essential.end());
    ih.sim.agents = ih.agents.get();
    ih.sim.locs = &ih.locs;
    ih.sim.infectiousnessMultiplier.assign(h.V, 1.0f);
    cxxopts::ParseResult r;
    const std::string d(dir);
    r.values["immunizationStart"] = std::to_string(p->start_after_day);
    std::string bs;
    for (uint32_t q = 0; q < p->n_booster_rounds; ++q) bs += (q ? "," : "") + std::to_string(p->booster_start_after_day[q]);
    r.values["boosterStart"] = bs;
    if (p->n_vacc_weeks) {
        std::ofstream f(d + "/vacc.txt");
        f << join_floats(p->vacc_per_week, (int)p->n_vacc_weeks);
        r.values["immunizationsPerWeek"] = d + "/vacc.txt";
    } else {
        r.values["immunizationsPerWeek"] = std::to_string(p->daily_doses * 7u);
    }
    {
        std::ofstream f(d + "/booster.txt");
        for (uint32_t q = 0; q < p->n_booster_rounds; ++q) {
            f << join_floats(p->booster_per_week[q], (int)p->n_booster_weeks[q]) << '\n';
            f << join_floats(p->booster_age_percent[q], 10) << '\n';
        }
        r.values["boostersPerWeek"] = d + "/booster.txt";
    }
    r.values["immunizationOrder"] = join_ints(p->order, 10);
    r.values["vaccinationGroupLevel"] = join_floats(p->group_level, 10);
    r.values["protectionInfection"] = join_floats(p->protection_infection, 10);
    r.values["protectionInfectionWaning"] = join_floats(p->protection_infection_waning, 10);
    r.values["protectionSymptomatic"] = join_floats(p->protection_symptomatic, 10);
    r.values["protectionSymptomaticWaning"] = join_floats(p->protection_symptomatic_waning, 10);
    r.values["protectionHospitalization"] = join_floats(p->protection_hospitalization, 10);
    r.values["protectionHospitalizationWaning"] = join_floats(p->protection_hospitalization_waning, 10);
    r.values["variantSimilarity"] = join_ints(p->variant_similarity, PSIM_MAX_STRAINS);
    r.values["variantSimilarMultiplier"] = join_floats(p->variant_similar_multiplier, PSIM_MAX_STRAINS);
    r.values["diags"] = "0";
    ih.imm.reset(new Immunization<ImmSim>(&ih.sim));
    try {
        ih.imm->initializeArgs(r);
        ih.pull();
        ih.imm->initCategories();
        ih.push();
    } catch (const std::exception&) {
        return 1;
    }
    return 0;
}

// Immunization::update at the midnight t; returns immunizedToday
uint32_t ref_immunize(void* hp, uint32_t t) {
    ImmHarness& ih = *g_imm;
    ih.pull();
    Timehandler th(ih.h->p.time_step, 0, Days::MONDAY, 0);
    for (uint32_t q = 0; q < t; ++q) ++th;
    psim_stream s;
    set_stream(&s, *ih.h, 0, t, PSIM_PHASE_IMMUNIZE);
    ih.imm->update(th, ih.h->p.time_step);
    harness_rng::current = nullptr;
    ih.push();
    return ih.imm->immunizedToday;
}

// the schedule table: offsets, then per event type and chance
uint32_t ref_events(void* hp, uint32_t* offsets, uint32_t* types, float* chance, uint32_t cap) {
    Harness& h = *(Harness*)hp;
    for (size_t j = 0; j < h.types.eventOffset.size(); ++j) offsets[j] = h.types.eventOffset[j];
    const size_t ne = h.types.events.size();
    for (size_t j = 0; j < ne && j < cap; ++j) {
        AgentTypeList::Event e = h.types.events[j];
        types[j] = e.locationType;
        chance[j] = e.chance;
    }
    return (uint32_t)ne;
}

}  // extern "C"
