// Closure rules: a host-side restatement of RuleClosure
// (include/policies/closurePolicies.h:48-479) driving the device state of a
// context.  Conditions are evaluated on the day's statistics row after
// midnight; rules then flip policy switches (psim_params), location
// open/closed flags and infectiousness multipliers, the schedule table
// (ReduceMovement, AgentTypeList::setStayHome/unsetStayHome,
// src/agentData/agentType.cpp:28-119) or infect agents with a variant
// (ExposeToMutation).
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "psim_ctx.h"

namespace psim {

enum CondKind { COND_AFTER_DAYS, COND_HOSPITALIZED, COND_NEW_DEAD, COND_NEW_CASES };
enum RuleKind {
    R_MASKS,
    R_CURFEW,
    R_HOLIDAY,
    R_QUARANTINE_IMMUNE,
    R_LOCKDOWN_NONVACC,
    R_QUARANTINE_POLICY,
    R_SCHOOL_AGE,
    R_EXPOSE,
    R_REDUCE_MOVEMENT,
    R_TESTING_PROB,
    R_CLOSE_TYPES
};

struct ClosureCond {
    CondKind kind = COND_AFTER_DAYS;
    std::vector<uint32_t> cols;  // hospital columns, or the dead column
    uint32_t prev_dead = 0;      // dead count of the previous midnight
    std::vector<double> history; // afterDays: [0] = day counter
    int pos = 0;
    bool active = false;
    double threshold = 0.0, threshold2 = 0.0;
    int close_after = 0, open_after = 0;
};

struct ClosureRule {
    std::string name;
    RuleKind kind = R_CLOSE_TYPES;
    size_t cond = 0;
    bool prev_open = true;         // previousOpenState
    double num = 0.0;              // mask coefficient / exposed fraction / stay-home probability
    int inum = 0;                  // quarantine policy / age limit / variant
    uint32_t curfew_begin = 0, curfew_end = 0;  // minutes of day
    std::vector<double> probs;     // TestingProb
    ClosureTypes types{};
};

struct ClosureEngine {
    std::vector<ClosureCond> conds;
    std::vector<ClosureRule> rules;
    double current_mask = 1.0;     // Simulation::currentMaskValue
};

}  // namespace psim

using namespace psim;

namespace {

// ClosureHelpers::splitHeader: characters are read with operator>> (white
// space skipped) and a token ends where the next character is a tab.
std::vector<std::string> split_header(const std::string& h) {
    std::vector<std::string> out;
    std::string arg;
    size_t i = 0;
    while (i < h.size()) {
        const char ch = h[i++];
        if (std::isspace((unsigned char)ch)) continue;
        arg.push_back(ch);
        if (i < h.size() && h[i] == '\t') {
            if (!arg.empty()) {
                out.push_back(arg);
                arg.clear();
            }
            ++i;
        }
    }
    if (!arg.empty()) out.push_back(arg);
    return out;
}

int pos_mod(int a, int b) {
    const int r = a % b;
    return r < 0 ? r + b : r;
}

// the close/open hysteresis of hospitalizedFraction and newDeadFraction
// (closurePolicies.h:130-166, 186-213)
bool hysteresis(ClosureCond& c, double value) {
    const int H = (int)c.history.size();
    c.history[c.pos] = value;
    c.pos = (c.pos + 1) % H;
    if (!c.active && value > c.threshold) {
        bool was_below = false;
        for (int i = pos_mod(c.pos - c.close_after, H); i != c.pos; i = (i + 1) % H)
            was_below |= c.history[i] < c.threshold;
        return was_below ? c.active : true;
    } else if (c.active && value <= c.threshold2) {
        bool was_above = false;
        for (int i = pos_mod(c.pos - c.open_after, H); i != c.pos; i = (i + 1) % H)
            was_above |= c.history[i] >= c.threshold2;
        return was_above ? c.active : false;
    }
    return c.active;
}

uint32_t stat_at(const psim_day_stats* row, uint32_t col) { return col < row->n ? row->v[col] : 0u; }

bool parse_double(const char* s, double* out) {
    char* end = nullptr;
    errno = 0;
    const double v = std::strtod(s, &end);
    if (end == s) return false;
    *out = v;
    return true;
}

bool parse_int(const char* s, int* out) {
    char* end = nullptr;
    const long v = std::strtol(s, &end, 10);
    if (end == s) return false;
    *out = (int)v;
    return true;
}

bool is_switch_rule(const std::string& n) {
    return n == "Masks" || n == "Curfew" || n == "HolidayMode" || n == "SchoolAgeRestriction" ||
           n == "ExposeToMutation" || n == "ReduceMovement" || n == "QuarantinePolicy" || n == "QuarantineImmune" ||
           n == "LockdownNonvacc" || n == "TestingProb";
}

// re-upload the host schedule table after an edit
int upload_events(psim_ctx* c) {
    DevModel& dm = c->k.m;
    const size_t no = c->h_event_offset.size(), ne = c->h_ev_loc_type.size();
    auto put = [&](const void* host, size_t bytes, void** dst) -> int {
        void* d = nullptr;
        const size_t b = bytes ? bytes : 16;
        cudaError_t e = psim_device_malloc((void**)&d, b);
        if (e != cudaSuccess) return fail(c, PSIM_ERR_ALLOC, std::string("schedule table: ") + cudaGetErrorString(e));
        c->allocs.push_back(d);
        if (bytes) {
            e = cudaMemcpyAsync(d, host, bytes, cudaMemcpyHostToDevice, c->stream);
            if (e != cudaSuccess) return fail(c, PSIM_ERR_CUDA, std::string("schedule table: ") + cudaGetErrorString(e));
        }
        *dst = d;
        return 0;
    };
    int rc;
    void* p = nullptr;
    if ((rc = put(c->h_event_offset.data(), no * 4, &p))) return rc;
    dm.event_offset = (const uint32_t*)p;
    if ((rc = put(c->h_ev_loc_type.data(), ne * 4, &p))) return rc;
    dm.ev_loc_type = (const uint32_t*)p;
    if ((rc = put(c->h_ev_chance.data(), ne * 4, &p))) return rc;
    dm.ev_chance = (const float*)p;
    if ((rc = put(c->h_ev_start.data(), ne * 2, &p))) return rc;
    dm.ev_start = (const uint16_t*)p;
    if ((rc = put(c->h_ev_end.data(), ne * 2, &p))) return rc;
    dm.ev_end = (const uint16_t*)p;
    if ((rc = put(c->h_ev_duration.data(), ne * 2, &p))) return rc;
    dm.ev_duration = (const uint16_t*)p;
    dm.n_events = (uint32_t)ne;
    CK(cudaStreamSynchronize(c->stream));
    if ((rc = upload_window_table(c))) return rc;
    c->graph_dirty = true;
    return 0;
}

}  // namespace

namespace {

// AgentTypeList::setStayHome (agentType.cpp:63-119): in every window of
// events with the same start the home event's chance becomes
// c + (1 - c) * p (inserted with chance p where a window has none) and every
// other event's chance is scaled by 1 - p.  Windows are found by equal start
// times and, as in the reference, may run on into the next schedule slot.
void set_stay_home(psim_ctx* c, double p, uint32_t home) {
    std::vector<uint32_t>& off = c->h_event_offset;
    std::vector<uint32_t>& ty = c->h_ev_loc_type;
    std::vector<float>& ch = c->h_ev_chance;
    std::vector<uint16_t>&st = c->h_ev_start, &en = c->h_ev_end, &du = c->h_ev_duration;
    for (size_t s = 0; s + 1 < off.size(); ++s) {
        uint32_t ws = off[s], we = ws;
        while (ws < off[s + 1]) {
            while (we < ty.size() && st[we] == st[ws]) ++we;
            bool home_present = false;
            for (uint32_t i = ws; i < we; ++i)
                if (ty[i] == home) {
                    home_present = true;
                    ch[i] = (float)((double)ch[i] + (1.0 - (double)ch[i]) * p);
                    break;
                }
            if (home_present && we - ws == 1) {
                ws = we;
                continue;
            }
            if (!home_present) {
                const uint16_t s0 = st[ws], e0 = en[ws], d0 = du[ws];
                ty.insert(ty.begin() + ws, home);
                ch.insert(ch.begin() + ws, (float)p);
                st.insert(st.begin() + ws, s0);
                en.insert(en.begin() + ws, e0);
                du.insert(du.begin() + ws, d0);
                ++we;
                for (size_t q = s + 1; q < off.size(); ++q) off[q]++;
            }
            for (uint32_t i = ws; i < we; ++i)
                if (ty[i] != home) ch[i] = (float)((double)ch[i] * (1.0 - p));
            ws = we;
        }
    }
}

// AgentTypeList::unsetStayHome (agentType.cpp:28-61): the inverse scaling;
// a home event whose chance falls below 1e-10 is erased.  After an erase the
// reference continues from the old window end, one event further on; that is
// kept.
void unset_stay_home(psim_ctx* c, double p, uint32_t home) {
    std::vector<uint32_t>& off = c->h_event_offset;
    std::vector<uint32_t>& ty = c->h_ev_loc_type;
    std::vector<float>& ch = c->h_ev_chance;
    std::vector<uint16_t>&st = c->h_ev_start, &en = c->h_ev_end, &du = c->h_ev_duration;
    for (size_t s = 0; s + 1 < off.size(); ++s) {
        uint32_t ws = off[s], we = ws;
        while (ws < off[s + 1]) {
            while (we < ty.size() && st[we] == st[ws]) ++we;
            for (uint32_t i = ws; i < we; ++i)
                if (ty[i] != home) ch[i] = (float)((double)ch[i] / (1.0 - p));
            for (uint32_t i = ws; i < we; ++i) {
                if (ty[i] == home) {
                    ch[i] = (float)(((double)ch[i] - p) / (1.0 - p));
                    if (std::fabs((double)ch[i]) < 1e-10) {
                        ty.erase(ty.begin() + i);
                        ch.erase(ch.begin() + i);
                        st.erase(st.begin() + i);
                        en.erase(en.begin() + i);
                        du.erase(du.begin() + i);
                        for (size_t q = s + 1; q < off.size(); ++q) off[q]--;
                    }
                    break;
                }
            }
            ws = we;
        }
    }
}

int push_params(psim_ctx* c) {
    c->k.p = c->params;
    c->graph_dirty = true;
    c->clock_valid = false;
    return 0;
}

}  // namespace

void closures_free(psim_ctx* c) {
    delete c->closures;
    c->closures = nullptr;
}

// ClosurePolicy::midnight (closurePolicies.h:474-477): every condition, then
// every rule.
int closures_apply(psim_ctx* c, uint32_t t, const psim_day_stats* row) {
    ClosureEngine* E = c->closures;
    if (!E) return 0;
    const double n_agents = (double)c->N;
    for (ClosureCond& q : E->conds) {
        switch (q.kind) {
            case COND_AFTER_DAYS: {
                const int day = (int)q.history[0];
                q.history[0] += 1.0;
                q.active = day >= q.threshold && day < q.threshold + q.open_after;
                break;
            }
            case COND_HOSPITALIZED: {
                double acc = 0.0;
                for (uint32_t col : q.cols) acc += stat_at(row, col);
                q.active = hysteresis(q, acc / n_agents);
                break;
            }
            case COND_NEW_DEAD: {
                const uint32_t dead = stat_at(row, q.cols[0]);
                const double value = (double)(uint32_t)(dead - q.prev_dead) / n_agents;
                q.prev_dead = dead;
                q.active = hysteresis(q, value);
                break;
            }
            case COND_NEW_CASES:
                q.active = hysteresis(q, (double)row->new_infections / n_agents);
                break;
        }
    }
    bool params_changed = false;
    for (ClosureRule& r : E->rules) {
        const bool close = E->conds[r.cond].active;
        const bool open = !close;
        const bool toggled = r.prev_open != open;
        switch (r.kind) {
            case R_MASKS:
                if (toggled) {
                    E->current_mask = open ? 1.0 : r.num;
                    launch_masks(c->k, c->params.home_type, r.num, open ? 1 : 0, c->stream);
                    c->launches += 1;
                    r.prev_open = open;
                }
                break;
            case R_CURFEW:
                if (toggled) {
                    c->params.enable_curfew = close ? 1u : 0u;
                    c->params.curfew_begin = r.curfew_begin / c->params.time_step;
                    c->params.curfew_end = r.curfew_end / c->params.time_step;
                    params_changed = true;
                    r.prev_open = open;
                }
                break;
            case R_HOLIDAY:
            case R_QUARANTINE_IMMUNE:
            case R_LOCKDOWN_NONVACC:
                if (toggled) {
                    uint32_t& f = r.kind == R_HOLIDAY            ? c->params.holiday_mode
                                  : r.kind == R_QUARANTINE_IMMUNE ? c->params.quarantine_immune
                                                                  : c->params.lockdown_nonvacc;
                    f = close ? 1u : 0u;
                    params_changed = true;
                    r.prev_open = open;
                }
                break;
            case R_QUARANTINE_POLICY:
                if (close) {
                    c->params.quarantine_policy = (uint32_t)r.inum;
                    params_changed = true;
                    r.prev_open = close;
                }
                break;
            case R_SCHOOL_AGE:
                if (toggled) {
                    c->params.school_age_restriction = close ? (uint32_t)r.inum : 99u;
                    params_changed = true;
                    r.prev_open = open;
                }
                break;
            case R_TESTING_PROB:
                if (close) {
                    double* dst[6] = {&c->params.t_random, &c->params.t_home,     &c->params.t_work,
                                      &c->params.t_school, &c->params.t_hospital, &c->params.t_nursery};
                    for (size_t q = 0; q < r.probs.size() && q < 6; ++q) *dst[q] = r.probs[q];
                    params_changed = true;
                }
                break;
            case R_EXPOSE:
                if (close) {
                    launch_expose(c->k, t, (uint32_t)r.inum, r.num, c->stream);
                    c->launches += 1;
                }
                break;
            case R_REDUCE_MOVEMENT:
                if (toggled) {
                    if (open)
                        unset_stay_home(c, r.num, c->params.home_type);
                    else
                        set_stay_home(c, r.num, c->params.home_type);
                    int rc = upload_events(c);
                    if (rc) return rc;
                    r.prev_open = open;
                }
                break;
            case R_CLOSE_TYPES:
                if (toggled) {
                    launch_close_types(c->k, r.types, open ? 1 : 0, c->stream);
                    c->launches += 1;
                    r.prev_open = open;
                }
                break;
        }
    }
    if (params_changed) push_params(c);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, PSIM_ERR_CUDA, std::string("closure kernels: ") + cudaGetErrorString(e));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

extern "C" {

// RuleClosure::init (closurePolicies.h:84-471)
int psim_closures_init(psim_ctx* c, const psim_closure_rule* rules, uint32_t n_rules, const char* header,
                       int enable_closures) {
    if (!c) return PSIM_ERR_ARG;
    closures_free(c);
    if (n_rules == 0) return 0;
    if (!rules) return fail(c, PSIM_ERR_ARG, "closures: null rule array");
    if (c->R != 1) return fail(c, PSIM_ERR_ARG, "closures: rules need a context with one replica");
    const std::vector<std::string> cols = split_header(header ? header : "");
    std::vector<uint32_t> hosp_cols, dead_cols;
    for (uint32_t i = 0; i < cols.size(); ++i) {
        if (cols[i].find("_h") != std::string::npos) hosp_cols.push_back(i);
        if (cols[i] == "D1") dead_cols.push_back(i);
    }
    ClosureEngine* E = new ClosureEngine();
    E->conds.reserve(n_rules);
    E->rules.reserve(n_rules);
    auto bad = [&](const std::string& m) {
        delete E;
        return fail(c, PSIM_ERR_ARG, "closures: " + m);
    };
    for (uint32_t q = 0; q < n_rules; ++q) {
        const psim_closure_rule& in = rules[q];
        const std::string name(in.name, strnlen(in.name, sizeof(in.name)));
        const std::string ctype(in.condition_type, strnlen(in.condition_type, sizeof(in.condition_type)));
        const std::string param(in.parameter, strnlen(in.parameter, sizeof(in.parameter)));
        if (!enable_closures && !is_switch_rule(name)) continue;
        ClosureCond cd;
        cd.threshold = in.threshold;
        cd.threshold2 = in.threshold2;
        cd.close_after = in.close_after;
        cd.open_after = in.open_after;
        if (ctype == "afterDays") {
            if (in.close_after >= 0 || in.open_after <= 0)
                return bad("for 'afterDays', closeAfter must be -1 and openAfter > 0 (rule " + name + ")");
            cd.kind = COND_AFTER_DAYS;
            cd.history.assign(1, 0.0);
        } else if (ctype == "hospitalizedFraction" || ctype == "newDeadFraction" || ctype == "newCasesFraction") {
            if (in.close_after <= 0 || in.open_after <= 0)
                return bad("for '" + ctype + "', closeAfter and openAfter must be > 0 (rule " + name + ")");
            cd.kind = ctype == "hospitalizedFraction" ? COND_HOSPITALIZED
                      : ctype == "newDeadFraction"    ? COND_NEW_DEAD
                                                      : COND_NEW_CASES;
            if (cd.kind == COND_HOSPITALIZED) cd.cols = hosp_cols;
            if (cd.kind == COND_NEW_DEAD) {
                if (dead_cols.empty()) return bad("newDeadFraction needs a D1 column in the header");
                // the reference keeps the previous count in the slot after the
                // D1 positions, which starts at 0 when there is one D1 column
                cd.cols.assign(1, dead_cols[0]);
                cd.prev_dead = dead_cols.size() > 1 ? dead_cols[1] : 0u;
            }
            cd.history.assign((size_t)std::max(in.close_after, in.open_after) + 2, 0.0);
        } else {
            return bad("unknown closure type " + ctype);
        }
        E->conds.push_back(cd);
        ClosureRule r;
        r.name = name;
        r.cond = E->conds.size() - 1;
        if (name == "Masks") {
            r.kind = R_MASKS;
            if (!parse_double(param.c_str(), &r.num)) return bad("Masks parameter is not a number");
        } else if (name == "Curfew") {
            r.kind = R_CURFEW;
            if (param.size() == 9) {
                r.curfew_begin = (uint32_t)(std::atoi(param.substr(0, 2).c_str()) * 60 + std::atoi(param.substr(2, 2).c_str()));
                r.curfew_end = (uint32_t)(std::atoi(param.substr(5, 2).c_str()) * 60 + std::atoi(param.substr(7, 2).c_str()));
            } else if (!param.empty()) {
                return bad("curfew parameter string needs to be exactly 9 characters long");
            }
        } else if (name == "HolidayMode") {
            r.kind = R_HOLIDAY;
        } else if (name == "QuarantineImmune") {
            r.kind = R_QUARANTINE_IMMUNE;
        } else if (name == "LockdownNonvacc") {
            r.kind = R_LOCKDOWN_NONVACC;
        } else if (name == "QuarantinePolicy") {
            r.kind = R_QUARANTINE_POLICY;
            if (!parse_int(param.c_str(), &r.inum)) return bad("QuarantinePolicy parameter is not an integer");
        } else if (name == "SchoolAgeRestriction") {
            r.kind = R_SCHOOL_AGE;
            if (!parse_int(param.c_str(), &r.inum)) return bad("SchoolAgeRestriction parameter is not an integer");
        } else if (name == "ExposeToMutation") {
            r.kind = R_EXPOSE;
            if (!parse_double(param.c_str(), &r.num)) return bad("ExposeToMutation parameter is not a number");
            r.inum = (int)in.threshold2;
            if (r.inum < 0 || (uint32_t)r.inum >= c->V)
                return bad("More ExposeToMutation events defined than infectiousnessMultiplier specified");
        } else if (name == "ReduceMovement") {
            r.kind = R_REDUCE_MOVEMENT;
            if (!parse_double(param.c_str(), &r.num)) return bad("ReduceMovement parameter is not a number");
        } else if (name == "TestingProb") {
            r.kind = R_TESTING_PROB;
            size_t s0 = 0;
            while (s0 <= param.size()) {
                size_t e0 = param.find(',', s0);
                if (e0 == std::string::npos) e0 = param.size();
                double v = 0.0;
                if (e0 > s0 && parse_double(param.substr(s0, e0 - s0).c_str(), &v)) r.probs.push_back(v);
                s0 = e0 + 1;
            }
        } else {
            r.kind = R_CLOSE_TYPES;
            if (in.n_types >= PSIM_CLOSURE_MAX_TYPES)
                return bad("Closure Rule " + name + " has over 10 location types to close");
            r.types.n = in.n_types;
            for (uint32_t j = 0; j < in.n_types; ++j) r.types.v[j] = (uint32_t)in.types[j];
        }
        E->rules.push_back(r);
    }
    c->closures = E;
    return 0;
}

int psim_closures_midnight(psim_ctx* c, uint32_t t, const psim_day_stats* row) {
    if (!c || !row) return PSIM_ERR_ARG;
    if (!c->uploaded) return PSIM_ERR_STATE;
    return closures_apply(c, t, row);
}

// processFlags' location closures (simulation.h:794-828): the non-essential
// locations of the listed types open or closed
int psim_set_types_open(psim_ctx* c, const uint32_t* types, uint32_t n_types, int open) {
    if (!c || (n_types && !types)) return PSIM_ERR_ARG;
    if (!c->uploaded) return PSIM_ERR_STATE;
    ClosureTypes ty{};
    if (n_types > sizeof(ty.v) / sizeof(ty.v[0])) return fail(c, PSIM_ERR_ARG, "too many location types");
    ty.n = n_types;
    for (uint32_t q = 0; q < n_types; ++q) ty.v[q] = types[q];
    launch_close_types(c->k, ty, open ? 1 : 0, c->stream);
    c->launches += 1;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, PSIM_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return check_device_err(c);
}

// processFlags' masks (simulation.h:846-891): the weight of every non-home
// location divided (divide != 0) or multiplied by coef, in double precision
int psim_scale_location_weights(psim_ctx* c, double coef, int divide) {
    if (!c) return PSIM_ERR_ARG;
    if (!c->uploaded) return PSIM_ERR_STATE;
    if (!(coef > 0.0)) return fail(c, PSIM_ERR_ARG, "coef must be positive");
    launch_masks(c->k, c->params.home_type, coef, divide ? 1 : 0, c->stream);
    c->launches += 1;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, PSIM_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return check_device_err(c);
}

int psim_closures_status(psim_ctx* c, uint8_t* cond_active, uint8_t* rule_open, uint32_t* n_rules) {
    if (!c) return PSIM_ERR_ARG;
    const ClosureEngine* E = c->closures;
    const uint32_t n = E ? (uint32_t)E->rules.size() : 0u;
    if (n_rules) *n_rules = n;
    for (uint32_t q = 0; q < n; ++q) {
        if (cond_active) cond_active[q] = E->conds[E->rules[q].cond].active ? 1 : 0;
        if (rule_open) rule_open[q] = E->rules[q].prev_open ? 1 : 0;
    }
    return 0;
}

}  // extern "C"
