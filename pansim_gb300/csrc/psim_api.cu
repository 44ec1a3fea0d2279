// C ABI of pansim_gb300 (include/pansim_gb300.h): context lifetime, host<->device
// transfer of the SoA snapshot, the per-step and per-day phases, and the
// per-day CUDA graph that replaces the reference's host loop with a
// cudaDeviceSynchronize after every launch (simulation.h:899-926).
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "psim_ctx.h"

using namespace psim;

// the kernels' error flags: reads and clears them
int check_device_err(psim_ctx* c) {
    uint32_t e = 0;
    CK(cudaMemcpyAsync(&e, c->k.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (e) {
        CK(cudaMemsetAsync(c->k.err, 0, sizeof(uint32_t), c->stream));
        std::string m = "device error flags 0x" + std::to_string(e) + ":";
        if (e & ERR_LOCATION) m += " agent on an invalid location;";
        if (e & ERR_TEST_WAIT) m += " bounded wait expired;";
        if (e & ERR_SCAN_WAIT) m += " scan tile wait expired;";
        if (e & ERR_AGENT_LIST) m += " agent list inconsistent;";
        if (e & ERR_BARRIER) m += " step kernel grid barrier expired;";
        return fail(c, PSIM_ERR_DEVICE, m);
    }
    return 0;
}

// Allocation-failure hook: the device allocations still allowed before one
// fails (negative: off).  Process-wide, for tests of the error paths.
static std::atomic<long long> g_alloc_budget{-1};

cudaError_t psim_device_malloc(void** p, size_t bytes) {
    long long b = g_alloc_budget.load();
    while (b >= 0) {
        if (b == 0) {
            *p = nullptr;
            return cudaErrorMemoryAllocation;
        }
        if (g_alloc_budget.compare_exchange_weak(b, b - 1)) break;
    }
    return cudaMalloc(p, bytes);
}

namespace {

const char* kVersion = "pansim_gb300 0.1.0 (sm_103a)";

template <typename T>
int dalloc(psim_ctx* c, T** p, size_t count) {
    size_t bytes = count * sizeof(T);
    if (bytes == 0) bytes = 16;
    void* q = nullptr;
    cudaError_t e = psim_device_malloc(&q, bytes);
    if (e != cudaSuccess) return fail(c, PSIM_ERR_ALLOC, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    cudaMemsetAsync(q, 0, bytes, c->stream);
    c->allocs.push_back(q);
    *p = (T*)q;
    return 0;
}

// The mutable state (what psim_upload / psim_download move) lives in one
// device allocation: these fields in this order, each at a 256-byte aligned
// offset (psim_state_layout).  A caller whose host arrays follow the same
// layout from agents->location on moves the whole state in one copy.
#define PSIM_AGENT_STATE(X)                                                                                         \
    X(location, location, N) X(move_at, steps_until_move, N) X(state, state, N) X(days, days, N)          \
    X(variant, variant, N) X(infectious, infectious, N) X(susceptible, susceptible, N* V)                          \
    X(diagnosed, diagnosed, N) X(quarantined, quarantined, N) X(stayed_home, stayed_home, N)                       \
    X(no_work, no_work, N) X(last_test, last_test, N) X(st_infected_ts, st_infected_ts, N)                         \
    X(st_infected_loc, st_infected_loc, N) X(st_worst_ts, st_worst_ts, N) X(st_worst_end_ts, st_worst_end_ts, N)   \
    X(st_diagnosed_ts, st_diagnosed_ts, N) X(st_quarantined_ts, st_quarantined_ts, N)                              \
    X(st_quarantined_until, st_quarantined_until, N) X(st_days_in_quarantine, st_days_in_quarantine, N)            \
    X(st_hospitalized_ts, st_hospitalized_ts, N) X(st_hospitalized_until, st_hospitalized_until, N)                \
    X(st_immunization_ts, st_immunization_ts, N) X(st_recovered_ts, st_recovered_ts, N)                            \
    X(st_variant_mask, st_variant_mask, N) X(st_immunization_count, st_immunization_count, N)                      \
    X(st_infected_count, st_infected_count, N) X(st_worst_state, st_worst_state, N) X(imm_round, imm_round, N)     \
    X(scaling_v, symptom_scaling_v, N* V)
#define PSIM_LOC_STATE(X) \
    X(infectiousness, infectiousness, L) X(open, open, L) X(closed_until, closed_until, L) X(quarantine_until, quarantine_until, L)

constexpr uint32_t STATE_FIELDS = 34;

// offsets of the state fields for N agents, L locations and V variants
// (off[STATE_FIELDS] = the total); returns the total
size_t state_layout(size_t N, size_t L, size_t V, uint64_t* off) {
    size_t o = 0;
    uint32_t f = 0;
    auto put = [&](size_t bytes) {
        if (off) off[f] = o;
        ++f;
        o += (bytes + 255) & ~(size_t)255;
    };
#define XA(dev, host, cnt) put(sizeof(*DevAgents{}.dev) * (size_t)(cnt));
#define XL(dev, host, cnt) put(sizeof(*DevLocs{}.dev) * (size_t)(cnt));
    PSIM_AGENT_STATE(XA) PSIM_LOC_STATE(XL)
#undef XA
#undef XL
    if (off) off[f] = o;
    return o;
}

template <typename T>
int dcopy_in(psim_ctx* c, const T* dptr, const T* host, size_t count) {
    if (count == 0) return 0;
    if (!host) return fail(c, PSIM_ERR_ARG, "missing host array");
    CK(cudaMemcpyAsync((void*)dptr, host, count * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    return 0;
}

template <typename T>
int dupload(psim_ctx* c, const T** dst, const T* host, size_t count) {
    T* d = nullptr;
    int rc = dalloc(c, &d, count);
    if (rc) return rc;
    rc = dcopy_in(c, d, host, count);
    if (rc) return rc;
    *dst = d;
    return 0;
}

int launch_check(psim_ctx* c) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, PSIM_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return 0;
}

// BasicInfection::seasonalityMultiplier, infectionPolicies.h:443-478
double seasonality(const psim_params& p, uint32_t t, uint32_t spd) {
    unsigned sim_day = t / spd;
    int d = (int)p.start_date + (int)sim_day;
    int d_peak = 59 + 22;
    d += 6;
    double c0 = 3.08;
    double trunc_val = 0.5;
    if (sim_day > 250 && sim_day < 450) {
        d += p.d_offset0;
        d_peak += p.d_peak_offset;
        c0 = p.c0;
    } else if (sim_day > 600) {
        trunc_val = p.trunc;
        if (p.n_d_offset > 1) d += p.d_offset1;
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

// set the device clock for the day containing t
// sync = false: the copy is left in the stream; the caller synchronises
// before the next set_clock (the copy reads the pinned clock when it runs)
int set_clock(psim_ctx* c, uint32_t t, bool sync = true) {
    uint32_t t0 = t - t % c->spd;
    DevClock nc = c->h_clock;
    nc.t0 = t0;
    nc.day_of_week = c->params.holiday_mode ? 6u : (c->params.start_day + t0 / c->spd) % 7u;
    nc.season = (float)seasonality(c->params, t0, c->spd);
    if (c->clock_valid && nc.t0 == c->h_clock.t0 && nc.day_of_week == c->h_clock.day_of_week &&
        nc.season == c->h_clock.season)
        return 0;
    c->h_clock = nc;
    *c->h_clock_pin = nc;
    // only the first three fields; the scan bookkeeping stays on the device
    CK(cudaMemcpyAsync(c->k.clock, c->h_clock_pin, 3 * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
    if (sync) CK(cudaStreamSynchronize(c->stream));
    c->clock_valid = true;
    return 0;
}

int validate(psim_ctx* c, const psim_model* m, const psim_agents* a, const psim_locations* l) {
    if (!m || !a || !l) return fail(c, PSIM_ERR_ARG, "null snapshot part");
    if (m->n_variants == 0 || m->n_variants > PSIM_MAX_STRAINS) return fail(c, PSIM_ERR_ARG, "n_variants out of range");
    if (m->n_states == 0 || m->n_states > 16) return fail(c, PSIM_ERR_ARG, "n_states must be 1..16");
    if (l->n == 0) return fail(c, PSIM_ERR_ARG, "no locations");
    if (a->n == 0) return fail(c, PSIM_ERR_ARG, "no agents");
    const uint32_t N = a->n, L = l->n;
    if (!a->loc_offset || a->loc_offset[0] != 0 || a->loc_offset[N] != a->n_poss)
        return fail(c, PSIM_ERR_RANGE, "per-agent location offsets inconsistent");
    for (uint32_t i = 0; i < N; ++i) {
        if (a->loc_offset[i + 1] < a->loc_offset[i]) return fail(c, PSIM_ERR_RANGE, "per-agent offsets not monotonic");
        if (a->location[i] >= L) return fail(c, PSIM_ERR_RANGE, "agent " + std::to_string(i) + " location out of range");
        if ((uint8_t)a->state[i] >= m->n_states) return fail(c, PSIM_ERR_RANGE, "agent state out of range");
        if (a->prog_id[i] >= m->n_prog) return fail(c, PSIM_ERR_RANGE, "progression id out of range");
        if (a->type[i] >= m->n_agent_types) return fail(c, PSIM_ERR_RANGE, "agent type out of range");
        if (a->variant[i] >= m->n_variants) return fail(c, PSIM_ERR_RANGE, "variant out of range");
        if (a->band[i] >= PSIM_MAX_BANDS) return fail(c, PSIM_ERR_RANGE, "age band out of range");
    }
    for (uint32_t j = 0; j < a->n_poss; ++j)
        if (a->poss_loc[j] >= L) return fail(c, PSIM_ERR_RANGE, "per-agent location entry out of range");
    const uint32_t ne = m->event_offset[m->n_agent_types * 28];
    if (ne != m->n_events) return fail(c, PSIM_ERR_ARG, "event offsets do not match n_events");
    for (uint32_t s = 0; s < m->n_prog * m->n_states; ++s) {
        if (m->tr_bad_begin[s] + m->tr_bad_count[s] > m->n_trans || m->tr_neu_begin[s] + m->tr_neu_count[s] > m->n_trans)
            return fail(c, PSIM_ERR_RANGE, "transition table out of range");
    }
    for (uint32_t j = 0; j < m->n_trans; ++j)
        if (m->tr_next[j] >= m->n_states) return fail(c, PSIM_ERR_RANGE, "transition target out of range");
    for (uint32_t s = 0; s < l->n_schools; ++s)
        if (l->schools[s] >= L) return fail(c, PSIM_ERR_RANGE, "school out of range");
    for (uint32_t s = 0; s < l->n_classrooms; ++s)
        if (l->classrooms[s] >= L) return fail(c, PSIM_ERR_RANGE, "classroom out of range");
    return 0;
}

// whether the host arrays follow the state layout from a->location on
bool state_packed(const psim_ctx* c, const psim_agents* a, const psim_locations* l) {
    uint64_t off[STATE_FIELDS + 1];
    state_layout(c->N, c->L, c->V, off);
    const char* base = (const char*)a->location;
    bool ok = base != nullptr;
    uint32_t f = 0;
#define XA(dev, host, cnt) ok = ok && (const char*)a->host == base + off[f++];
#define XL(dev, host, cnt) ok = ok && (const char*)l->host == base + off[f++];
    PSIM_AGENT_STATE(XA) PSIM_LOC_STATE(XL)
#undef XA
#undef XL
    return ok;
}

int upload_mutable(psim_ctx* c, const psim_agents* a, const psim_locations* l) {
    const size_t N = c->N, L = c->L;
    DevAgents& d = c->k.a;
    int rc = 0;
    if (state_packed(c, a, l)) {
        CK(cudaMemcpyAsync(c->state_slab, a->location, c->state_bytes, cudaMemcpyHostToDevice, c->stream));
        // countdowns -> absolute decision timestamps
        launch_time_shift(d.move_at, c->N, c->t_next, c->stream);
        return launch_check(c);
    }
#define UP(field, cnt) \
    if ((rc = dcopy_in(c, d.field, a->field, cnt))) return rc;
    if ((rc = dcopy_in(c, d.move_at, a->steps_until_move, N))) return rc;
    launch_time_shift(d.move_at, c->N, c->t_next, c->stream);
    UP(location, N) UP(state, N) UP(days, N) UP(variant, N) UP(infectious, N)
    UP(susceptible, N * c->V) UP(diagnosed, N) UP(quarantined, N) UP(stayed_home, N) UP(no_work, N) UP(last_test, N)
    UP(st_infected_ts, N) UP(st_infected_loc, N) UP(st_worst_ts, N) UP(st_worst_end_ts, N) UP(st_diagnosed_ts, N)
    UP(st_quarantined_ts, N) UP(st_quarantined_until, N) UP(st_days_in_quarantine, N) UP(st_hospitalized_ts, N)
    UP(st_hospitalized_until, N) UP(st_immunization_ts, N) UP(st_recovered_ts, N) UP(st_variant_mask, N)
    UP(st_immunization_count, N) UP(st_infected_count, N) UP(st_worst_state, N)
#undef UP
    // optional immunization fields: neutral values when absent
    if (a->imm_round) {
        if ((rc = dcopy_in(c, d.imm_round, a->imm_round, N))) return rc;
    } else {
        CK(cudaMemsetAsync(d.imm_round, 0, N, c->stream));
    }
    if (a->symptom_scaling_v) {
        if ((rc = dcopy_in(c, d.scaling_v, a->symptom_scaling_v, N * c->V))) return rc;
    } else {
        for (uint32_t v = 0; v < c->V; ++v)
            CK(cudaMemcpyAsync(d.scaling_v + (size_t)v * N, d.symptom_scaling, 4 * N, cudaMemcpyDeviceToDevice, c->stream));
    }
    DevLocs& dl = c->k.l;
    if ((rc = dcopy_in(c, dl.infectiousness, l->infectiousness, L))) return rc;
    if ((rc = dcopy_in(c, dl.open, l->open, L))) return rc;
    if ((rc = dcopy_in(c, dl.closed_until, l->closed_until, L))) return rc;
    if ((rc = dcopy_in(c, dl.quarantine_until, l->quarantine_until, L))) return rc;
    return 0;
}

// LocationsList::initialize (locationList.h:224-230) and the variant gates
// The per-location sums start afresh: zero, and every location marked for
// the next scan.  Called before a pass that adds every agent's term
// (k_movement, k_count): the first step of each day and the regroups.
int reset_sums(psim_ctx* c) {
    CK(cudaMemsetAsync(c->k.l.sfix, 0, sizeof(unsigned long long) * c->L * c->V, c->stream));
    CK(cudaMemsetAsync(c->k.l.sfix_b, 0, sizeof(unsigned long long) * c->L * c->V, c->stream));
    CK(cudaMemsetAsync(c->k.l.smask, 0xFF, sizeof(uint32_t) * (((size_t)c->L + 2047) / 2048 * 64 + 64), c->stream));
    return 0;
}

// the next scan rebuilds the CSR whatever moved
int force_rebuild(psim_ctx* c) {
    CK(cudaMemsetAsync(c->k.l.build + 1, 0xFF, sizeof(uint32_t), c->stream));
    return 0;
}

int initial_regroup(psim_ctx* c) {
    int rc0 = force_rebuild(c);
    if (rc0) return rc0;
    CK(cudaMemsetAsync(c->k.l.counts, 0, sizeof(uint32_t) * c->L, c->stream));
    if ((rc0 = reset_sums(c))) return rc0;
    launch_count(c->k, c->stream);
    launch_scan(c->k, 0, 1, 0, c->stream);
    launch_scatter_draw(c->k, 0, 1, 0, c->stream);
    c->list_sparse = false;
    // the variant gating of the first steps (the statistics come at midnight)
    launch_variant_flags(c->k, c->stream);
    c->launches += 3 + (uint64_t)scan_kernels(c->k);
    int rc = launch_check(c);
    if (rc) return rc;
    c->csr_fresh = true;
    return check_device_err(c);
}

int do_step(psim_ctx* c, uint32_t step, bool draw, bool movement) {
    const int merge_q = c->params.quarantine_policy > 1 ? 2 : 0;
    if (movement) {
        int rc = reset_sums(c);
        if (rc) return rc;
        launch_movement(c->k, step, c->stream);
    }
    launch_scan(c->k, step, 1, merge_q, c->stream);
    launch_scatter_draw(c->k, step, 1, draw ? 1 : 0, c->stream);
    c->launches += (movement ? 2 : 1) + (uint64_t)scan_kernels(c->k);
    c->list_sparse = false;
    return launch_check(c);
}

int capture_day_graph(psim_ctx* c) {
    if (c->day_graph) {
        cudaGraphExecDestroy(c->day_graph);
        c->day_graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    // profiled: the step kernel's counters and timeline stamps (KArgs::prof)
    c->k.prof = c->profile ? c->d_prof : nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    // (the capture stays open until EndCapture: errors are checked after it)
    // The day's first step: the sums afresh (every location dirty), the
    // agent list rebuilt (its slots take the susceptibilities the midnight
    // phases left), the mask of decision steps recomputed from every agent.
    cudaError_t me = cudaMemsetAsync(c->k.l.sfix, 0, sizeof(unsigned long long) * c->L * c->V, c->stream);
    if (me == cudaSuccess) me = cudaMemsetAsync(c->k.l.sfix_b, 0, sizeof(unsigned long long) * c->L * c->V, c->stream);
    if (me == cudaSuccess)
        me = cudaMemsetAsync(c->k.l.smask, 0xFF, sizeof(uint32_t) * (((size_t)c->L + 2047) / 2048 * 64 + 64), c->stream);
    if (me == cudaSuccess) me = cudaMemsetAsync(c->k.a.move_mask, 0, sizeof(uint32_t) * MOVE_MASK_WORDS, c->stream);
    if (me == cudaSuccess) me = cudaMemsetAsync(c->k.l.build + 1, 0xFF, sizeof(uint32_t), c->stream);
    if (me == cudaSuccess) me = cudaMemsetAsync(c->k.l.bar, 0, sizeof(uint32_t) * BAR_WORDS, c->stream);
    if (me == cudaSuccess && c->profile) me = cudaMemsetAsync(c->d_prof, 0, sizeof(unsigned long long) * PROF_WORDS, c->stream);
    launch_movement(c->k, 0, c->stream);
    // Per timestep one launch of the step kernel (rebuild, draws, decisions
    // for the next timestep, grid barriers between its phases), or with
    // tuning variant 4 one launch for the whole day with a grid barrier
    // between timesteps (measured slower on GB300: a barrier takes longer than
    // the gap between two kernel nodes of the graph); the profiled graph is
    // the same launches with the kernel's timeline stamps.
    if (c->k.tune.variant == 4)
        launch_steps(c->k, 0, c->spd, PH_ALL, c->stream);
    else
        for (uint32_t s = 0; s < c->spd; ++s) launch_step(c->k, s, PH_ALL, c->stream);
    // the day's final sums are in the copy its next step would read: with an
    // odd number of steps that is the second one
    if (me == cudaSuccess && (c->spd & 1u))
        me = cudaMemcpyAsync(c->k.l.sfix, c->k.l.sfix_b, sizeof(unsigned long long) * c->L * c->V,
                             cudaMemcpyDeviceToDevice, c->stream);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e == cudaSuccess && me != cudaSuccess) {
        cudaGraphDestroy(g);
        e = me;
    }
    if (e != cudaSuccess) return fail(c, PSIM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&c->day_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(c, PSIM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    // movement(0) and the step kernel launches
    c->graph_kernels = 1 + (c->k.tune.variant == 4 ? 1ull : (uint64_t)c->spd);
    c->graph_dirty = false;
    c->prof_valid = false;
    return 0;
}

void assemble_stats(psim_ctx* c, uint32_t t, psim_day_stats* out) {
    const uint32_t S = c->S, V = c->V;
    const bool tests = c->params.testing_enabled && t > 0;
    for (uint32_t q = 0; q < c->R; ++q) {
        const DevStatsAcc& a = c->h_stats[q];
        psim_day_stats& d = out[q];
        memset(&d, 0, sizeof(d));
        uint32_t n = 0;
        for (uint32_t s = 0; s < S; ++s) d.v[n++] = a.c[SC_HIST + s];
        d.v[n++] = a.c[SC_HOSP];
        d.v[n++] = tests ? a.c[SC_TESTS] : 0u;
        d.v[n++] = tests ? a.c[SC_P1] : 0u;
        d.v[n++] = tests ? a.c[SC_P2] : 0u;
        d.v[n++] = a.c[SC_Q];
        d.v[n++] = a.c[SC_QT];
        d.v[n++] = a.c[SC_NQ];
        if (V > 1) {
            for (uint32_t v = 1; v < V; ++v)
                d.v[n++] = a.c[SC_ALL_INF] ? (uint32_t)((double)a.c[SC_VAR + v] / (double)a.c[SC_ALL_INF] * 100.0) : 0u;
        } else {
            d.v[n++] = 0u;
        }
        d.v[n] = a.c[SC_STAYED] - d.v[10] - d.v[11];
        n++;
        d.v[n++] = immunized_today(c);  // VAC: immunized today
        d.v[n++] = a.c[SC_NI];
        d.v[n++] = a.c[SC_INF_ONCE];
        d.v[n++] = a.c[SC_REINF];
        d.v[n++] = a.c[SC_BSTR];
        for (uint32_t v = 0; v < V; ++v) d.v[n++] = (uint32_t)a.imm[v];
        d.v[n++] = (a.c[SC_HCI] * 100u) / (c->hcw_count[q] > 1 ? c->hcw_count[q] : 1u);
        d.v[n++] = a.c[SC_HCE];
        for (uint32_t v = 0; v < V; ++v) d.v[n++] = a.c[SC_INFV + v];
        d.v[n++] = a.c[SC_INFH];
        d.v[n++] = a.c[SC_VNI];
        d.n = n;
        d.new_infections = a.c[SC_NI];
        for (uint32_t v = 0; v < V; ++v) d.variant_counts[v] = a.c[SC_VAR + v];
        d.expected_new_infections = c->h_expected[q];
    }
}

}  // namespace

// The schedule window of doMovement (movementPolicies.h:585-603) for every
// schedule slot and step of the day: act_b = the first event of the slot
// active at the step's minute, act_e = the first event starting after it (or
// the slot's end when its last event is the active one), -1 where none.
int upload_window_table(psim_ctx* c) {
    const std::vector<uint32_t>& off = c->h_event_offset;
    const std::vector<uint16_t>&st = c->h_ev_start, &en = c->h_ev_end;
    const size_t n_slots = off.empty() ? 0 : off.size() - 1;
    const uint32_t spd = c->spd, dt = 1440u / spd;
    std::vector<int2> win(n_slots * spd);
    for (size_t q = 0; q < n_slots; ++q) {
        const uint32_t ev_b = off[q], ev_e = off[q + 1];
        for (uint32_t s = 0; s < spd; ++s) {
            const uint32_t minutes = s * dt;
            int act_b = -1, act_e = -1;
            for (uint32_t j = ev_b; j < ev_e; ++j) {
                const uint32_t a = st[j], b = en[j];
                if (minutes >= a && minutes < b && act_b == -1) act_b = (int)j;
                if (minutes < a) {
                    act_e = (int)j;
                    break;
                }
                if (j == ev_e - 1 && minutes >= a && minutes < b) act_e = (int)ev_e;
            }
            win[q * spd + s] = make_int2(act_b, act_e);
        }
    }
    int2* d = nullptr;
    const size_t bytes = std::max<size_t>(win.size() * sizeof(int2), 16);
    cudaError_t e = psim_device_malloc((void**)&d, bytes);
    if (e != cudaSuccess) return fail(c, PSIM_ERR_ALLOC, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    c->allocs.push_back(d);
    if (!win.empty()) CK(cudaMemcpyAsync(d, win.data(), win.size() * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->k.m.window = d;
    return 0;
}


extern "C" {

const char* psim_version(void) { return kVersion; }

int psim_abi_sizes(uint64_t* out, int n) {
    const uint64_t s[6] = {sizeof(psim_model), sizeof(psim_agents), sizeof(psim_locations),
                           sizeof(psim_params), sizeof(psim_replicas), sizeof(psim_day_stats)};
    for (int i = 0; i < n && i < 6; ++i) out[i] = s[i];
    return 0;
}

int psim_device_count(int* out) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) n = 0;
    if (out) *out = n;
    return e == cudaSuccess ? 0 : PSIM_ERR_CUDA;
}

const char* psim_last_error(const psim_ctx* c) { return c ? c->err.c_str() : "null context"; }

int psim_create(int device, const psim_model* m, const psim_agents* a, const psim_locations* l,
                const psim_params* p, const psim_replicas* reps, psim_ctx** out) {
    if (!out) return PSIM_ERR_ARG;
    *out = nullptr;
    psim_ctx* c = new psim_ctx();
    auto bail = [&](int rc) {
        *out = c;  // keep the context so that psim_last_error works; caller destroys it
        return rc;
    };
    if (!p) return bail(fail(c, PSIM_ERR_ARG, "null params"));
    int rc = validate(c, m, a, l);
    if (rc) return bail(rc);
    if (p->time_step == 0 || 1440 % p->time_step) return bail(fail(c, PSIM_ERR_ARG, "time_step must divide 1440"));
    if (l->n >= 0x3FFFFFFFu) return bail(fail(c, PSIM_ERR_ARG, "more than 2^30 - 2 locations"));
    c->N = a->n;
    c->L = l->n;
    c->V = m->n_variants;
    c->S = m->n_states;
    c->n_poss = a->n_poss;
    c->params = *p;
    c->spd = 1440 / p->time_step;
    // replicas
    if (reps && reps->n > 0) {
        c->R = reps->n;
        c->rep_agent_off.assign(reps->agent_offset, reps->agent_offset + c->R + 1);
        c->rep_loc_off.assign(reps->loc_offset, reps->loc_offset + c->R + 1);
        c->rep_seed.assign(reps->seed, reps->seed + c->R);
        c->rep_k.assign(reps->k, reps->k + c->R);
        c->rep_cemetery.assign(reps->cemetery, reps->cemetery + c->R);
    } else {
        c->R = 1;
        c->rep_agent_off = {0u, c->N};
        c->rep_loc_off = {0u, c->L};
        c->rep_seed = {p->seed};
        c->rep_k = {p->k};
        c->rep_cemetery = {p->cemetery_loc};
    }
    if (c->R > 65535) return bail(fail(c, PSIM_ERR_ARG, "too many replicas"));
    if (c->rep_agent_off[c->R] != c->N || c->rep_loc_off[c->R] != c->L || c->rep_agent_off[0] || c->rep_loc_off[0])
        return bail(fail(c, PSIM_ERR_ARG, "replica offsets do not cover the snapshot"));
    for (uint32_t q = 0; q < c->R; ++q) {
        if (c->rep_agent_off[q + 1] < c->rep_agent_off[q] || c->rep_loc_off[q + 1] < c->rep_loc_off[q])
            return bail(fail(c, PSIM_ERR_ARG, "replica offsets not monotonic"));
        // the cemetery is the location appended last (locationList.h:168-175)
        if (c->rep_loc_off[q + 1] == c->rep_loc_off[q] || c->rep_cemetery[q] != c->rep_loc_off[q + 1] - 1)
            return bail(fail(c, PSIM_ERR_RANGE, "cemetery is not the last location of its replica"));
        // replicas do not share locations
        for (uint32_t i = c->rep_agent_off[q]; i < c->rep_agent_off[q + 1]; ++i) {
            if (a->location[i] < c->rep_loc_off[q] || a->location[i] >= c->rep_loc_off[q + 1])
                return bail(fail(c, PSIM_ERR_RANGE, "agent " + std::to_string(i) + " outside its replica's locations"));
            for (uint32_t j = a->loc_offset[i]; j < a->loc_offset[i + 1]; ++j)
                if (a->poss_loc[j] < c->rep_loc_off[q] || a->poss_loc[j] >= c->rep_loc_off[q + 1])
                    return bail(fail(c, PSIM_ERR_RANGE,
                                     "agent " + std::to_string(i) + " has a location outside its replica"));
        }
    }
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return bail(fail(c, PSIM_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e)));
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(fail(c, PSIM_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e)));
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    const size_t N = c->N, L = c->L, V = c->V, R = c->R;
    KArgs& k = c->k;
    // model tables
    DevModel& dm = k.m;
    dm.n_states = m->n_states;
    dm.n_variants = m->n_variants;
    dm.n_prog = m->n_prog;
    dm.n_agent_types = m->n_agent_types;
    dm.first_infected = m->first_infected_state;
    dm.noncovid_dead = m->noncovid_dead_state;
    dm.dead_state = m->dead_state;
    dm.n_trans = m->n_trans;
    dm.n_events = m->n_events;
    const size_t S = m->n_states, PS = (size_t)m->n_prog * S;
    std::vector<uint32_t> thr(PS * PSIM_MAX_STRAINS);
    for (size_t j = 0; j < thr.size(); ++j) thr[j] = psim_geometric_threshold(m->len_p[j]);
#define UPM(field, cnt) \
    if ((rc = dupload(c, &dm.field, m->field, cnt))) return bail(rc);
    UPM(state_wb, S) UPM(state_susceptible, S) UPM(state_infected, S) UPM(state_infectious, S) UPM(state_acc_pcr, S)
    UPM(state_acc_antigen, S) UPM(variant_multiplier, V) UPM(prog_scaling, V) UPM(death_scaling, V)
    UPM(tr_bad_begin, PS) UPM(tr_bad_count, PS) UPM(tr_neu_begin, PS) UPM(tr_neu_count, PS)
    UPM(tr_next, m->n_trans) UPM(tr_chance, m->n_trans) UPM(len_avg, PS * PSIM_MAX_STRAINS)
    UPM(len_max, PS * PSIM_MAX_STRAINS) UPM(event_offset, (size_t)m->n_agent_types * 28 + 1)
    UPM(ev_loc_type, m->n_events) UPM(ev_chance, m->n_events) UPM(ev_start, m->n_events) UPM(ev_end, m->n_events)
    UPM(ev_duration, m->n_events)
#undef UPM
    {
        const size_t no = (size_t)m->n_agent_types * 28 + 1, ne = m->n_events;
        c->h_event_offset.assign(m->event_offset, m->event_offset + no);
        c->h_ev_loc_type.assign(m->ev_loc_type, m->ev_loc_type + ne);
        c->h_ev_chance.assign(m->ev_chance, m->ev_chance + ne);
        c->h_ev_start.assign(m->ev_start, m->ev_start + ne);
        c->h_ev_end.assign(m->ev_end, m->ev_end + ne);
        c->h_ev_duration.assign(m->ev_duration, m->ev_duration + ne);
    }
    if ((rc = upload_window_table(c))) return bail(rc);
    if ((rc = dupload(c, &dm.len_thr, thr.data(), thr.size()))) return bail(rc);
    // agents: immutable
    DevAgents& da = k.a;
    da.n = c->N;
    std::vector<uint16_t> arep(N), lrep(L);
    for (uint32_t q = 0; q < c->R; ++q) {
        for (uint32_t i = c->rep_agent_off[q]; i < c->rep_agent_off[q + 1]; ++i) arep[i] = (uint16_t)q;
        for (uint32_t j = c->rep_loc_off[q]; j < c->rep_loc_off[q + 1]; ++j) lrep[j] = (uint16_t)q;
    }
#define UPA(field, cnt) \
    if ((rc = dupload(c, &da.field, a->field, cnt))) return bail(rc);
    UPA(type, N) UPA(age, N) UPA(band, N) UPA(prog_id, N) UPA(symptom_scaling, N) UPA(loc_offset, N + 1)
    UPA(poss_loc, c->n_poss) UPA(poss_type, c->n_poss)
#undef UPA
    {
        // the location lists packed for the decisions: 4 bytes per entry when
        // every location and type fits, else 8
        bool fits = L < (1u << 26);
        for (size_t j = 0; fits && j < c->n_poss; ++j) fits = a->poss_loc[j] < (1u << 26) && a->poss_type[j] < 64u;
        if (fits) {
            std::vector<uint32_t> packed(c->n_poss);
            for (size_t j = 0; j < c->n_poss; ++j) packed[j] = a->poss_loc[j] | (uint32_t)a->poss_type[j] << 26;
            if ((rc = dupload(c, &da.poss4, packed.data(), c->n_poss))) return bail(rc);
            da.poss = nullptr;
        } else {
            std::vector<uint2> packed(c->n_poss);
            for (size_t j = 0; j < c->n_poss; ++j) packed[j] = make_uint2(a->poss_loc[j], a->poss_type[j]);
            if ((rc = dupload(c, &da.poss, packed.data(), c->n_poss))) return bail(rc);
            da.poss4 = nullptr;
        }
    }
    if (a->precond) {
        if ((rc = dupload(c, &da.precond, a->precond, N))) return bail(rc);
    } else {
        uint8_t* z = nullptr;
        if ((rc = dalloc(c, &z, N))) return bail(rc);
        da.precond = z;
    }
    if (a->sex) {
        if ((rc = dupload(c, &da.sex, a->sex, N))) return bail(rc);
    } else {
        uint8_t* z = nullptr;
        if ((rc = dalloc(c, &z, N))) return bail(rc);
        da.sex = z;
    }
    if ((rc = dupload(c, &da.rep, arep.data(), N))) return bail(rc);
    // the mutable state: one allocation (state_layout)
    {
        uint64_t off[STATE_FIELDS + 1];
        uint8_t* slab = nullptr;
        if ((rc = dalloc(c, &slab, state_layout(N, L, V, off)))) return bail(rc);
        c->state_slab = slab;
        c->state_bytes = off[STATE_FIELDS];
        uint32_t f = 0;
#define XA(dev, host, cnt) da.dev = (decltype(da.dev))(slab + off[f++]);
#define XL(dev, host, cnt) k.l.dev = (decltype(k.l.dev))(slab + off[f++]);
        PSIM_AGENT_STATE(XA) PSIM_LOC_STATE(XL)
#undef XA
#undef XL
    }
#define AL(field, cnt) \
    if ((rc = dalloc(c, &da.field, cnt))) return bail(rc);
    AL(hcw, N) AL(rank, N) AL(home, N)
    AL(worklist, (size_t)N + (size_t)WORK_MAX_BLOCKS * 1024 + 4)
    AL(move_mask, MOVE_MASK_WORDS)
#undef AL
    // locations
    DevLocs& dl = k.l;
    dl.n = c->L;
    dl.n_schools = l->n_schools;
    if ((rc = dupload(c, &dl.type, l->type, L))) return bail(rc);
    if ((rc = dupload(c, &dl.essential, l->essential, L))) return bail(rc);
    if ((rc = dupload(c, &dl.schools, l->schools, l->n_schools))) return bail(rc);
    if ((rc = dupload(c, &dl.classrooms, l->classrooms, l->n_classrooms))) return bail(rc);
    if ((rc = dupload(c, &dl.classroom_offsets, l->classroom_offsets, l->n_schools ? l->n_schools + 1 : 0)))
        return bail(rc);
    if ((rc = dupload(c, &dl.rep, lrep.data(), L))) return bail(rc);
    if ((rc = dalloc(c, &dl.counts, L))) return bail(rc);
    if ((rc = dalloc(c, &dl.csr_off, L + 1))) return bail(rc);
    if ((rc = dalloc(c, &dl.cursor, L))) return bail(rc);
    if ((rc = dalloc(c, &dl.csr_agents, N))) return bail(rc);
    if ((rc = dalloc(c, &dl.slot_loc, N))) return bail(rc);
    if ((rc = dalloc(c, &dl.inf_pending, 3 * N))) return bail(rc);
    if ((rc = dalloc(c, &dl.slot_su, N * V))) return bail(rc);
    if ((rc = dalloc(c, &dl.qu_pending, L))) return bail(rc);
    if ((rc = dalloc(c, &dl.sfix, L * V))) return bail(rc);
    if ((rc = dalloc(c, &dl.sfix_b, L * V))) return bail(rc);
    if ((rc = dalloc(c, &dl.hazard, L * V))) return bail(rc);
    if ((rc = dalloc(c, &dl.hazard_x, L * V))) return bail(rc);
    if ((rc = dalloc(c, &dl.hmask, ((size_t)L + 2047) / 2048 * 64 + 64))) return bail(rc);
    if ((rc = dalloc(c, &dl.smask, ((size_t)L + 2047) / 2048 * 64 + 64))) return bail(rc);
    if ((rc = dalloc(c, &dl.no_work_loc, L))) return bail(rc);
    if ((rc = dalloc(c, &dl.flags, L))) return bail(rc);
    const size_t tiles = (L + 511) / 512 + 1;
    if ((rc = dalloc(c, &dl.tile_sums, tiles))) return bail(rc);
    if ((rc = dalloc(c, &dl.bar, BAR_WORDS))) return bail(rc);
    if ((rc = dalloc(c, &dl.scan_status, tiles))) return bail(rc);
    if ((rc = dalloc(c, &dl.scan_state, 2))) return bail(rc);
    if ((rc = dalloc(c, &dl.build, 8))) return bail(rc);
    if ((rc = dalloc(c, &c->d_prof, PROF_WORDS))) return bail(rc);
    // replicas
    DevReps& dr = k.r;
    dr.n = c->R;
    std::vector<float> kf(R);
    for (size_t q = 0; q < R; ++q) kf[q] = (float)c->rep_k[q];
    if ((rc = dupload(c, &dr.agent_off, c->rep_agent_off.data(), R + 1))) return bail(rc);
    if ((rc = dupload(c, &dr.loc_off, c->rep_loc_off.data(), R + 1))) return bail(rc);
    if ((rc = dupload(c, &dr.seed, (const unsigned long long*)c->rep_seed.data(), R))) return bail(rc);
    if ((rc = dupload(c, &dr.k_f, kf.data(), R))) return bail(rc);
    if ((rc = dupload(c, &dr.cemetery, c->rep_cemetery.data(), R))) return bail(rc);
    if ((rc = dalloc(c, &dr.variant_active, R * V))) return bail(rc);
    if ((rc = dalloc(c, &dr.expected, R))) return bail(rc);
    if ((rc = dalloc(c, &k.clock, 1))) return bail(rc);
    if ((rc = dalloc(c, &k.err, 1))) return bail(rc);
    if ((rc = dalloc(c, &k.stats, R))) return bail(rc);
    if ((rc = dalloc(c, &c->d_adj_weight, R))) return bail(rc);
    if ((rc = dalloc(c, &c->d_grad, 32))) return bail(rc);
    if ((rc = dalloc(c, &c->d_type_slot, 256))) return bail(rc);
    if ((rc = dalloc(c, &c->d_w_by_type, 256))) return bail(rc);
    {
        std::vector<int8_t> none(256, (int8_t)-1);
        if ((rc = dcopy_in(c, c->d_type_slot, none.data(), 256))) return bail(rc);
    }
    k.adj.on = 0;
    k.adj.weight = c->d_adj_weight;
    k.adj.grad = c->d_grad;
    k.adj.type_slot = c->d_type_slot;
    // the mutable state saved by a checkpoint
    {
        auto add = [&](void* ptr, size_t bytes) { c->regions.push_back({ptr, bytes}); c->checkpoint_bytes += bytes; };
        DevAgents& a2 = k.a;
        add(a2.location, 4 * N); add(a2.move_at, 4 * N); add(a2.state, N); add(a2.days, 2 * N);
        add(a2.variant, N); add(a2.infectious, 4 * N); add(a2.susceptible, 4 * N * V); add(a2.diagnosed, N);
        add(a2.quarantined, N); add(a2.stayed_home, N); add(a2.no_work, N); add(a2.last_test, 4 * N);
        add(a2.st_infected_ts, 4 * N); add(a2.st_infected_loc, 4 * N); add(a2.st_worst_ts, 4 * N);
        add(a2.st_worst_end_ts, 4 * N); add(a2.st_diagnosed_ts, 4 * N); add(a2.st_quarantined_ts, 4 * N);
        add(a2.st_quarantined_until, 4 * N); add(a2.st_days_in_quarantine, 4 * N); add(a2.st_hospitalized_ts, 4 * N);
        add(a2.st_hospitalized_until, 4 * N); add(a2.st_immunization_ts, 4 * N); add(a2.st_recovered_ts, 4 * N);
        add(a2.st_variant_mask, 4 * N); add(a2.st_immunization_count, N); add(a2.st_infected_count, N);
        add(a2.st_worst_state, N); add(a2.imm_round, N); add(a2.scaling_v, 4 * N * V);
        add(dl.infectiousness, 4 * L); add(dl.open, L); add(dl.closed_until, 4 * L); add(dl.quarantine_until, 4 * L);
        // the histogram is kept incrementally across steps and days
        add(dl.counts, 4 * L); add(dl.sfix, 8 * L * V); add(dl.smask, 4 * ((L + 2047) / 2048 * 64 + 64));
        add(dr.variant_active, R * V); add(dr.expected, 8 * R);
    }
    k.p = c->params;
    k.spd = c->spd;
    k.track_expected = 0;
    // the fastest choice measured on GB300 at 2M agents; the autotuner
    // (pansim_gb300/autotune.py) picks per device and workload
    k.tune.agg_count = 0;
    k.tune.scan_items = 4;
    k.tune.scan_mode = 3;
    k.tune.agg_slot = 0;
    k.tune.blocks_per_sm = 4;
    k.tune.variant = 3;
    {
        const size_t b_stats = sizeof(DevStatsAcc) * R, b_exp = sizeof(double) * R;
        const size_t bytes = b_stats + b_exp + sizeof(DevClock) + 64;
        if (cudaMallocHost(&c->pinned, bytes) != cudaSuccess) {
            c->pinned = nullptr;
            return bail(fail(c, PSIM_ERR_ALLOC, "pinned host buffers"));
        }
        std::memset(c->pinned, 0, bytes);
        char* p = (char*)c->pinned;
        c->h_stats = (DevStatsAcc*)p;
        c->h_expected = (double*)(p + b_stats);
        c->h_clock_pin = (DevClock*)(p + b_stats + b_exp);
        c->h_err_pin = (uint32_t*)(p + b_stats + b_exp + sizeof(DevClock) + 32);
    }
    // healthcare workers per replica (Simulation::flagHealthcareWorkers, simulation.h:670-693)
    c->hcw_count.assign(R, 0u);
    for (uint32_t q = 0; q < c->R; ++q)
        for (uint32_t i = c->rep_agent_off[q]; i < c->rep_agent_off[q + 1]; ++i)
            for (uint32_t j = a->loc_offset[i]; j < a->loc_offset[i + 1]; ++j) {
                const uint32_t lt = l->type[a->poss_loc[j]];
                if (a->poss_type[j] == 4 && (lt == 12 || lt == 14)) {
                    c->hcw_count[q]++;
                    break;
                }
            }
    if ((rc = upload_mutable(c, a, l))) return bail(rc);
    if ((rc = set_clock(c, 0))) return bail(rc);
    launch_flag_hcw(k, c->stream);
    launch_homes(k, c->stream);
    c->home_type_done = c->params.home_type;
    c->launches += 2;
    if ((rc = initial_regroup(c))) return bail(rc);
    c->uploaded = true;
    *out = c;
    return 0;
}

int psim_destroy(psim_ctx* c) {
    if (!c) return 0;
    if (c->stream) cudaStreamSynchronize(c->stream);
    closures_free(c);
    immunization_free(c);
    other_disease_free(c);
    for (auto& kv : c->checkpoints)
        if (kv.second) cudaFree(kv.second);
    if (c->day_graph) cudaGraphExecDestroy(c->day_graph);
    for (void* p : c->allocs) cudaFree(p);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->pinned) cudaFreeHost(c->pinned);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return 0;
}

int psim_upload(psim_ctx* c, const psim_agents* a, const psim_locations* l) {
    if (!c) return PSIM_ERR_ARG;
    if (!a || !l || a->n != c->N || l->n != c->L) return fail(c, PSIM_ERR_ARG, "snapshot size mismatch");
    int rc = upload_mutable(c, a, l);
    if (rc) return rc;
    // locations are checked on the device by the histogram pass
    rc = initial_regroup(c);
    if (rc == PSIM_ERR_DEVICE && c->err.find("invalid location") != std::string::npos)
        return fail(c, PSIM_ERR_RANGE, "agent location out of range");
    return rc;
}

int psim_download(psim_ctx* c, psim_agents* a, psim_locations* l) {
    if (!c) return PSIM_ERR_ARG;
    if (!a || !l || a->n != c->N || l->n != c->L) return fail(c, PSIM_ERR_ARG, "snapshot size mismatch");
    const size_t N = c->N, L = c->L;
    const DevAgents& d = c->k.a;
    // absolute decision timestamps -> countdowns for the copy, and back
    launch_time_shift(d.move_at, c->N, 0u - c->t_next, c->stream);
    if (state_packed(c, a, l)) {
        CK(cudaMemcpyAsync(a->location, c->state_slab, c->state_bytes, cudaMemcpyDeviceToHost, c->stream));
        launch_time_shift(d.move_at, c->N, c->t_next, c->stream);
        CK(cudaStreamSynchronize(c->stream));
        int rc = launch_check(c);
        if (rc) return rc;
        return check_device_err(c);
    }
#define DN(field, cnt) \
    if (a->field) CK(cudaMemcpyAsync(a->field, d.field, (cnt) * sizeof(*a->field), cudaMemcpyDeviceToHost, c->stream));
    if (a->steps_until_move)
        CK(cudaMemcpyAsync(a->steps_until_move, d.move_at, N * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    launch_time_shift(d.move_at, c->N, c->t_next, c->stream);
    DN(location, N) DN(state, N) DN(days, N) DN(variant, N) DN(infectious, N)
    DN(susceptible, N * c->V) DN(diagnosed, N) DN(quarantined, N) DN(stayed_home, N) DN(no_work, N) DN(last_test, N)
    DN(st_infected_ts, N) DN(st_infected_loc, N) DN(st_worst_ts, N) DN(st_worst_end_ts, N) DN(st_diagnosed_ts, N)
    DN(st_quarantined_ts, N) DN(st_quarantined_until, N) DN(st_days_in_quarantine, N) DN(st_hospitalized_ts, N)
    DN(st_hospitalized_until, N) DN(st_immunization_ts, N) DN(st_recovered_ts, N) DN(st_variant_mask, N)
    DN(st_immunization_count, N) DN(st_infected_count, N) DN(st_worst_state, N) DN(imm_round, N)
#undef DN
    if (a->symptom_scaling_v)
        CK(cudaMemcpyAsync(a->symptom_scaling_v, d.scaling_v, 4 * N * c->V, cudaMemcpyDeviceToHost, c->stream));
    const DevLocs& dl = c->k.l;
    if (l->infectiousness) CK(cudaMemcpyAsync(l->infectiousness, dl.infectiousness, L * 4, cudaMemcpyDeviceToHost, c->stream));
    if (l->open) CK(cudaMemcpyAsync(l->open, dl.open, L, cudaMemcpyDeviceToHost, c->stream));
    if (l->closed_until) CK(cudaMemcpyAsync(l->closed_until, dl.closed_until, L * 4, cudaMemcpyDeviceToHost, c->stream));
    if (l->quarantine_until)
        CK(cudaMemcpyAsync(l->quarantine_until, dl.quarantine_until, L * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int rc = launch_check(c);
    if (rc) return rc;
    return check_device_err(c);
}

int psim_state_layout(uint32_t n_agents, uint32_t n_locations, uint32_t n_variants, uint64_t* offsets,
                      uint32_t* n_fields) {
    if (n_fields) *n_fields = STATE_FIELDS;
    if (offsets) state_layout(n_agents, n_locations, n_variants, offsets);
    return 0;
}

int psim_get_params(psim_ctx* c, psim_params* out) {
    if (!c || !out) return PSIM_ERR_ARG;
    *out = c->params;
    return 0;
}

int psim_get_events(psim_ctx* c, uint32_t* event_offset, uint32_t* loc_type, float* chance, uint16_t* start,
                    uint16_t* end, uint16_t* duration, uint32_t capacity, uint32_t* n_events) {
    if (!c) return PSIM_ERR_ARG;
    const size_t ne = c->h_ev_loc_type.size();
    if (n_events) *n_events = (uint32_t)ne;
    if (event_offset) std::memcpy(event_offset, c->h_event_offset.data(), sizeof(uint32_t) * c->h_event_offset.size());
    const size_t m = ne < capacity ? ne : capacity;
    if (loc_type) std::memcpy(loc_type, c->h_ev_loc_type.data(), sizeof(uint32_t) * m);
    if (chance) std::memcpy(chance, c->h_ev_chance.data(), sizeof(float) * m);
    if (start) std::memcpy(start, c->h_ev_start.data(), sizeof(uint16_t) * m);
    if (end) std::memcpy(end, c->h_ev_end.data(), sizeof(uint16_t) * m);
    if (duration) std::memcpy(duration, c->h_ev_duration.data(), sizeof(uint16_t) * m);
    return 0;
}

int psim_set_params(psim_ctx* c, const psim_params* p) {
    if (!c || !p) return PSIM_ERR_ARG;
    if (p->time_step != c->params.time_step) return fail(c, PSIM_ERR_ARG, "time_step cannot change");
    c->params = *p;
    c->k.p = *p;
    c->graph_dirty = true;
    c->clock_valid = false;
    if (c->uploaded && p->home_type != c->home_type_done) {
        launch_homes(c->k, c->stream);
        c->launches += 1;
        c->home_type_done = p->home_type;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return fail(c, PSIM_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    }
    return 0;
}

int psim_set_tuning(psim_ctx* c, const psim_tuning* t) {
    if (!c || !t) return PSIM_ERR_ARG;
    if (t->blocks_per_sm > 64) return fail(c, PSIM_ERR_ARG, "blocks_per_sm out of range");
    c->k.tune.agg_count = t->agg_count ? 1u : 0u;
    c->k.tune.agg_slot = t->agg_slot ? 1u : 0u;
    c->k.tune.blocks_per_sm = t->blocks_per_sm;
    if (t->variant != 3 && t->variant != 4)
        return fail(c, PSIM_ERR_ARG, "variant must be 3 (a launch per timestep) or 4 (a launch per day)");
    c->k.tune.variant = t->variant;
    if (t->scan_items != 0 && t->scan_items != 2 && t->scan_items != 4 && t->scan_items != 8)
        return fail(c, PSIM_ERR_ARG, "scan_items must be 2, 4 or 8");
    c->k.tune.scan_items = t->scan_items ? t->scan_items : 8u;
    if (t->scan_mode > 3) return fail(c, PSIM_ERR_ARG, "scan_mode must be 0, 1, 2 or 3");
    c->k.tune.scan_mode = t->scan_mode;
    c->graph_dirty = true;
    return 0;
}

int psim_get_tuning(psim_ctx* c, psim_tuning* t) {
    if (!c || !t) return PSIM_ERR_ARG;
    t->agg_count = c->k.tune.agg_count;
    t->agg_slot = c->k.tune.agg_slot;
    t->blocks_per_sm = c->k.tune.blocks_per_sm;
    t->variant = c->k.tune.variant;
    t->scan_items = c->k.tune.scan_items;
    t->scan_mode = c->k.tune.scan_mode;
    return 0;
}

int psim_set_type_weights(psim_ctx* c, const float* w_by_type, const int8_t* slot_of_type) {
    if (!c || !c->uploaded || !w_by_type) return PSIM_ERR_ARG;
    if (slot_of_type) {
        for (int j = 0; j < 256; ++j)
            if (slot_of_type[j] >= 8) return fail(c, PSIM_ERR_ARG, "weight slot must be < 8 (or -1)");
        CK(cudaMemcpyAsync(c->d_type_slot, slot_of_type, 256, cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaMemcpyAsync(c->d_w_by_type, w_by_type, 256 * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    launch_type_weights(c->k, c->d_w_by_type, c->stream);
    c->launches += 1;
    int rc = launch_check(c);
    if (rc) return rc;
    return check_device_err(c);
}

int psim_set_replica_k(psim_ctx* c, const double* k) {
    if (!c || !k) return PSIM_ERR_ARG;
    std::vector<float> kf(c->R);
    for (uint32_t q = 0; q < c->R; ++q) {
        c->rep_k[q] = k[q];
        kf[q] = (float)k[q];
    }
    CK(cudaMemcpyAsync((void*)c->k.r.k_f, kf.data(), sizeof(float) * c->R, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int psim_set_adjoint(psim_ctx* c, int on, const double* weights) {
    if (!c) return PSIM_ERR_ARG;
    if (weights) {
        CK(cudaMemcpyAsync(c->d_adj_weight, weights, sizeof(double) * c->R, cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    const uint32_t o = on ? 1u : 0u;
    if (o != c->k.adj.on) {
        c->k.adj.on = o;
        c->graph_dirty = true;
    }
    return 0;
}

int psim_get_gradient(psim_ctx* c, double* out, int reset) {
    if (!c || !out) return PSIM_ERR_ARG;
    CK(cudaMemcpyAsync(out, c->d_grad, sizeof(double) * GRAD_N, cudaMemcpyDeviceToHost, c->stream));
    if (reset) CK(cudaMemsetAsync(c->d_grad, 0, sizeof(double) * 32, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int psim_checkpoint_save(psim_ctx* c, uint32_t slot) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    if (!c->checkpoints.count(slot) || !c->checkpoints[slot]) {
        void* p = nullptr;
        cudaError_t e = psim_device_malloc(&p, c->checkpoint_bytes);
        if (e != cudaSuccess) return fail(c, PSIM_ERR_ALLOC, std::string("checkpoint: ") + cudaGetErrorString(e));
        c->checkpoints[slot] = p;
    }
    c->checkpoint_t_next[slot] = c->t_next;
    char* dst = (char*)c->checkpoints[slot];
    for (auto& r : c->regions) {
        CK(cudaMemcpyAsync(dst, r.first, r.second, cudaMemcpyDeviceToDevice, c->stream));
        dst += r.second;
    }
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int psim_checkpoint_restore(psim_ctx* c, uint32_t slot) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    auto it = c->checkpoints.find(slot);
    if (it == c->checkpoints.end() || !it->second) return fail(c, PSIM_ERR_ARG, "no such checkpoint");
    const char* src = (const char*)it->second;
    for (auto& r : c->regions) {
        CK(cudaMemcpyAsync(r.first, src, r.second, cudaMemcpyDeviceToDevice, c->stream));
        src += r.second;
    }
    c->t_next = c->checkpoint_t_next[slot];
    // the restored locations need not match the agent list of the last step
    int rc = force_rebuild(c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    c->csr_fresh = false;
    return 0;
}

int psim_checkpoint_free(psim_ctx* c) {
    if (!c) return PSIM_ERR_ARG;
    cudaStreamSynchronize(c->stream);
    for (auto& kv : c->checkpoints)
        if (kv.second) cudaFree(kv.second);
    c->checkpoints.clear();
    return 0;
}

int psim_checkpoint_drop(psim_ctx* c, uint32_t slot) {
    if (!c) return PSIM_ERR_ARG;
    auto it = c->checkpoints.find(slot);
    if (it == c->checkpoints.end()) return 0;
    cudaStreamSynchronize(c->stream);
    if (it->second) cudaFree(it->second);
    c->checkpoints.erase(it);
    return 0;
}

int psim_checkpoint_bytes(psim_ctx* c, uint64_t* out) {
    if (!c || !out) return PSIM_ERR_ARG;
    *out = c->checkpoint_bytes;
    return 0;
}

int psim_set_tracking(psim_ctx* c, int expected) {
    if (!c) return PSIM_ERR_ARG;
    c->k.track_expected = expected ? 1u : 0u;
    c->graph_dirty = true;
    return 0;
}

int psim_movement(psim_ctx* c, uint32_t t) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    int rc = set_clock(c, t);
    if (rc) return rc;
    if ((rc = reset_sums(c))) return rc;
    launch_movement(c->k, t % c->spd, c->stream);
    c->launches += 1;
    c->csr_fresh = true;
    c->t_next = t + 1;
    rc = launch_check(c);
    if (rc) return rc;
    return check_device_err(c);
}

int psim_regroup(psim_ctx* c) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    int rc0 = force_rebuild(c);
    if (rc0) return rc0;
    if (!c->csr_fresh) {
        CK(cudaMemsetAsync(c->k.l.counts, 0, sizeof(uint32_t) * c->L, c->stream));
        if ((rc0 = reset_sums(c))) return rc0;
        launch_count(c->k, c->stream);
        c->launches += 1;
    }
    launch_scan(c->k, 0, 1, c->params.quarantine_policy > 1 ? 2 : 0, c->stream);
    launch_scatter_draw(c->k, 0, 1, 0, c->stream);
    c->launches += 1 + (uint64_t)scan_kernels(c->k);
    c->csr_fresh = false;
    c->list_sparse = false;
    int rc = launch_check(c);
    if (rc) return rc;
    return check_device_err(c);
}

int psim_infect(psim_ctx* c, uint32_t t, uint32_t variant) {
    // the hazard of the last regroup was computed for all variants; the draw
    // runs for the active ones (variant selects nothing more: draws of
    // several variants are sequential per agent as in the reference)
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    (void)variant;
    int rc = set_clock(c, t);
    if (rc) return rc;
    // the draw only (the CSR was scattered by psim_regroup)
    launch_scatter_draw(c->k, t % c->spd, 0, 1, c->stream);
    c->launches += 1;
    rc = launch_check(c);
    if (rc) return rc;
    return check_device_err(c);
}

int psim_step(psim_ctx* c, uint32_t t) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    int rc = set_clock(c, t);
    if (rc) return rc;
    rc = do_step(c, t % c->spd, true, true);
    if (rc) return rc;
    c->csr_fresh = false;
    c->t_next = t + 1;
    return check_device_err(c);
}

int psim_test_day(psim_ctx* c, uint32_t t, uint32_t* tpp) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    launch_test(c->k, t, c->stream);
    c->launches += 2;
    int rc = launch_check(c);
    if (rc) return rc;
    if (tpp) {
        launch_stats(c->k, t, c->stream);
        c->launches += 2;
        CK(cudaMemcpyAsync(c->h_stats, c->k.stats, sizeof(DevStatsAcc) * c->R, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        for (uint32_t q = 0; q < c->R; ++q) {
            tpp[3 * q + 0] = c->h_stats[q].c[SC_TESTS];
            tpp[3 * q + 1] = c->h_stats[q].c[SC_P1];
            tpp[3 * q + 2] = c->h_stats[q].c[SC_P2];
        }
    }
    return check_device_err(c);
}

int psim_progress_day(psim_ctx* c, uint32_t t) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    launch_progress(c->k, t, c->stream);
    c->launches += 1;
    int rc = launch_check(c);
    if (rc) return rc;
    return check_device_err(c);
}

int psim_stats_day(psim_ctx* c, uint32_t t, psim_day_stats* out) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    launch_stats(c->k, t, c->stream);
    c->launches += 2;
    int rc = launch_check(c);
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->h_stats, c->k.stats, sizeof(DevStatsAcc) * c->R, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(c->h_expected, c->k.r.expected, sizeof(double) * c->R, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemsetAsync(c->k.r.expected, 0, sizeof(double) * c->R, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (out) assemble_stats(c, t, out);
    return check_device_err(c);
}

int psim_plan_day(psim_ctx* c, uint32_t t) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    launch_plan(c->k, t, c->stream);
    c->launches += 5 + (c->params.quarantine_policy > 3 && c->k.l.n_schools ? 1 : 0);
    c->t_next = t;  // the plan sets every countdown relative to midnight t
    int rc = launch_check(c);
    if (rc) return rc;
    return check_device_err(c);
}

int psim_midnight(psim_ctx* c, uint32_t t, psim_day_stats* out) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    int rc = 0;
    if (t > 0 && c->params.testing_enabled) {
        launch_test(c->k, t, c->stream);
        c->launches += 2;
    }
    if (t > 0) {
        launch_progress(c->k, t, c->stream);
        c->launches += 1;
    }
    if (c->immunization && (rc = immunization_apply(c, t))) return rc;
    if (c->other_disease && (rc = other_disease_apply(c, t))) return rc;
    if (c->closures) {
        // the rules read replica 0's row even when the caller passes no buffer
        std::vector<psim_day_stats> rows(c->R);
        if ((rc = psim_stats_day(c, t, rows.data()))) return rc;
        if (out) std::memcpy(out, rows.data(), sizeof(psim_day_stats) * c->R);
        if ((rc = closures_apply(c, t, &rows[0]))) return rc;
    } else if ((rc = psim_stats_day(c, t, out))) {
        return rc;
    }
    return psim_plan_day(c, t);
}

int psim_run_steps(psim_ctx* c, uint32_t day) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    int rc = set_clock(c, day * c->spd);
    if (rc) return rc;
    if (c->graph_dirty || !c->day_graph) {
        if ((rc = capture_day_graph(c))) return rc;
    }
    CK(cudaEventRecord(c->ev0, c->stream));
    CK(cudaGraphLaunch(c->day_graph, c->stream));
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    CK(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
    c->launches += c->graph_kernels;
    c->prof_valid = c->profile;
    c->csr_fresh = false;
    c->list_sparse = true;
    c->t_next = (day + 1) * c->spd;
    return check_device_err(c);
}

int psim_run_day(psim_ctx* c, uint32_t day, psim_day_stats* out) {
    if (!c) return PSIM_ERR_ARG;
    if (!c->uploaded) return PSIM_ERR_STATE;
    const uint32_t t = day * c->spd;
    if (c->closures || c->immunization || c->other_disease) {
        // host logic between the midnight phases (rules on the statistics
        // row, dose budgets): phase by phase
        int rc = psim_midnight(c, t, out);
        if (rc) return rc;
        return psim_run_steps(c, day);
    }
    // The midnight phases, the clock and the day graph in stream order with
    // one synchronisation at the end: the statistics and the error flags come
    // back through pinned buffers.
    int rc = 0;
    if (c->graph_dirty || !c->day_graph) {
        if ((rc = capture_day_graph(c))) return rc;
    }
    if (t > 0 && c->params.testing_enabled) {
        launch_test(c->k, t, c->stream);
        c->launches += 2;
    }
    if (t > 0) {
        launch_progress(c->k, t, c->stream);
        c->launches += 1;
    }
    launch_stats(c->k, t, c->stream);
    c->launches += 2;
    CK(cudaMemcpyAsync(c->h_stats, c->k.stats, sizeof(DevStatsAcc) * c->R, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(c->h_expected, c->k.r.expected, sizeof(double) * c->R, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemsetAsync(c->k.r.expected, 0, sizeof(double) * c->R, c->stream));
    launch_plan(c->k, t, c->stream);
    c->launches += 5 + (c->params.quarantine_policy > 3 && c->k.l.n_schools ? 1 : 0);
    c->t_next = t;
    if ((rc = launch_check(c))) return rc;
    if ((rc = set_clock(c, t, false))) return rc;
    CK(cudaEventRecord(c->ev0, c->stream));
    CK(cudaGraphLaunch(c->day_graph, c->stream));
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaMemcpyAsync(c->h_err_pin, c->k.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1));
    c->launches += c->graph_kernels;
    c->prof_valid = c->profile;
    c->csr_fresh = false;
    c->list_sparse = true;
    c->t_next = (day + 1) * c->spd;
    if (*c->h_err_pin) return check_device_err(c);
    if (out) assemble_stats(c, t, out);
    return 0;
}

int psim_get_csr(psim_ctx* c, int canonical, uint32_t* offsets, uint32_t* agents) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    if (c->list_sparse) {
        // the step kernel lists only the locations its draws visit: the full
        // agent list of the current positions (prefix of the histogram,
        // slots), which no later step reads (the day graph's and the step
        // kernel's first step rebuild)
        int rc = force_rebuild(c);
        if (rc) return rc;
        launch_scan(c->k, 0, 0, 0, c->stream);
        launch_scatter_draw(c->k, 0, 1, 0, c->stream);
        c->launches += 1 + (uint64_t)scan_kernels(c->k);
        c->list_sparse = false;
    }
    launch_offsets(c->k, c->stream);
    c->launches += 1;
    if (canonical) {
        launch_canonical_csr(c->k, c->stream);
        c->launches += 1;
        int rc = launch_check(c);
        if (rc) return rc;
    }
    if (offsets) CK(cudaMemcpyAsync(offsets, c->k.l.csr_off, sizeof(uint32_t) * (c->L + 1), cudaMemcpyDeviceToHost, c->stream));
    if (agents) CK(cudaMemcpyAsync(agents, c->k.l.csr_agents, sizeof(uint32_t) * c->N, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return check_device_err(c);
}

int psim_get_hazard(psim_ctx* c, float* out, int64_t* fixed_sum) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    (void)fixed_sum;
    if (!out) return 0;
    // hazards are kept only where the mask says some variant's is > 0
    std::vector<uint32_t> mask((c->L + 31) / 32);
    CK(cudaMemcpyAsync(out, c->k.l.hazard, sizeof(float) * c->L * c->V, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(mask.data(), c->k.l.hmask, sizeof(uint32_t) * mask.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (uint32_t l = 0; l < c->L; ++l)
        if (!((mask[l >> 5] >> (l & 31)) & 1u))
            for (uint32_t v = 0; v < c->V; ++v) out[(size_t)v * c->L + l] = 0.0f;
    return 0;
}

int psim_last_day_ms(psim_ctx* c, float* ms) {
    if (!c || !ms) return PSIM_ERR_ARG;
    *ms = c->last_ms;
    return 0;
}

int psim_set_profiling(psim_ctx* c, int on) {
    if (!c) return PSIM_ERR_ARG;
    if ((on != 0) != c->profile) {
        c->profile = on != 0;
        c->graph_dirty = true;
    }
    c->prof_valid = false;
    return 0;
}

// the profiled day's timeline, copied back (stamps in ns; first entries
// stored as complements, see PROF_T)
static int read_timeline(psim_ctx* c, std::vector<unsigned long long>& h) {
    if (!c->prof_valid) return fail(c, PSIM_ERR_STATE, "no profiled day: psim_set_profiling(1), then psim_run_steps");
    h.assign(PROF_WORDS, 0ull);
    CK(cudaMemcpyAsync(h.data(), c->d_prof, sizeof(unsigned long long) * PROF_WORDS, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

// Per step of the profiled day, in microseconds (TL_COLS values): the
// kernel's span (first block entry to last block exit), the rebuild's
// listing, its slots, the draws, the queue, the decisions (0 where the phase
// did not run), and the time from the previous kernel's last exit to this
// kernel's first entry.
constexpr int TL_COLS = 7;
static void step_times(psim_ctx* c, const std::vector<unsigned long long>& h, uint32_t s, float* o) {
    const unsigned long long* T = &h[PROF_T + PROF_TW * (size_t)s];
    const unsigned long long t0 = ~T[0], r1 = T[1], r2 = T[2], drw = T[3], que = T[4], end = T[5];
    const unsigned long long prev = s == 0 ? h[PROF_N + 1] : h[PROF_T + PROF_TW * (size_t)(s - 1) + 5];
    auto us = [](unsigned long long a, unsigned long long b) { return b > a ? (float)((double)(b - a) * 1e-3) : 0.0f; };
    o[0] = us(t0, end);
    o[1] = r1 ? us(t0, r1) : 0.0f;
    o[2] = r2 ? us(r1, r2) : 0.0f;
    o[3] = us(r2 ? r2 : t0, drw);
    o[4] = que ? us(drw, que) : 0.0f;
    o[5] = que ? us(que, end) : 0.0f;
    o[6] = us(prev, t0);
}

int psim_day_kernel_ms(psim_ctx* c, float* ms) {
    if (!c || !ms) return PSIM_ERR_ARG;
    std::vector<unsigned long long> h;
    int rc = read_timeline(c, h);
    if (rc) return rc;
    ms[0] = h[PROF_N + 1] > ~h[PROF_N] ? (float)((double)(h[PROF_N + 1] - ~h[PROF_N]) * 1e-6) : 0.0f;
    ms[1] = ms[2] = ms[3] = ms[4] = 0.f;
    for (uint32_t s = 0; s < c->spd; ++s) {
        float o[TL_COLS];
        step_times(c, h, s, o);
        ms[1] += (o[1] + o[2]) * 1e-3f;
        ms[2] += o[3] * 1e-3f;
        ms[3] += (o[4] + o[5]) * 1e-3f;
        ms[4] += o[6] * 1e-3f;
    }
    return 0;
}

int psim_day_timeline(psim_ctx* c, float* us) {
    if (!c || !us) return PSIM_ERR_ARG;
    std::vector<unsigned long long> h;
    int rc = read_timeline(c, h);
    if (rc) return rc;
    for (uint32_t s = 0; s < c->spd; ++s) step_times(c, h, s, us + TL_COLS * (size_t)s);
    return 0;
}

int psim_day_counts(psim_ctx* c, uint64_t* out) {
    if (!c || !out) return PSIM_ERR_ARG;
    if (!c->prof_valid) return fail(c, PSIM_ERR_STATE, "no profiled day: psim_set_profiling(1), then psim_run_steps");
    unsigned long long h[PROF_N];
    CK(cudaMemcpyAsync(h, c->d_prof, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    out[0] = h[PROF_DRAW_ENTRIES];
    out[1] = h[PROF_DRAW_HAZARD];
    out[2] = h[PROF_MOVERS];
    out[3] = h[PROF_QUEUE_STEPS];
    out[4] = h[PROF_REBUILDS];
    out[5] = h[PROF_LISTED_LOCATIONS];
    out[6] = h[PROF_LISTED_AGENTS];
    return 0;
}

int psim_launch_count(psim_ctx* c, uint64_t* out) {
    if (!c || !out) return PSIM_ERR_ARG;
    *out = c->launches;
    return 0;
}

int psim_stream_handle(psim_ctx* c, void** out) {
    if (!c || !out) return PSIM_ERR_ARG;
    *out = (void*)c->stream;
    return 0;
}

int psim_time_step_kernels(psim_ctx* c, uint32_t t, float* ms) {
    if (!c || !c->uploaded || !ms) return PSIM_ERR_ARG;
    if (t % c->spd + 1 >= c->spd) return fail(c, PSIM_ERR_ARG, "t and t+1 must lie in the same day");
    int rc = set_clock(c, t);
    if (rc) return rc;
    cudaEvent_t ev[4];
    for (int j = 0; j < 4; ++j) CK(cudaEventCreate(&ev[j]));
    const uint32_t step = t % c->spd;
    // step t as the day graph runs it, from movement(t) with the sums afresh
    // and the agent list rebuilt: the rebuild, the draws, the queue +
    // decisions of t + 1 (the step kernel's phases as separate launches);
    // then step t + 1 untimed
    if ((rc = reset_sums(c))) return rc;
    CK(cudaMemsetAsync(c->k.a.move_mask, 0, sizeof(uint32_t) * MOVE_MASK_WORDS, c->stream));
    CK(cudaMemsetAsync(c->k.l.bar, 0, sizeof(uint32_t) * BAR_WORDS, c->stream));
    if ((rc = force_rebuild(c))) return rc;
    launch_movement(c->k, step, c->stream);
    CK(cudaEventRecord(ev[0], c->stream));
    launch_step(c->k, step, PH_REBUILD, c->stream);
    CK(cudaEventRecord(ev[1], c->stream));
    launch_step(c->k, step, PH_DRAW, c->stream);
    CK(cudaEventRecord(ev[2], c->stream));
    launch_step(c->k, step, PH_DECIDE, c->stream);
    CK(cudaEventRecord(ev[3], c->stream));
    launch_step(c->k, step + 1, PH_REBUILD | PH_DRAW, c->stream);
    c->launches += 5;
    // the sums as the step after them reads them, in the first copy
    if ((step + 2) & 1u)
        CK(cudaMemcpyAsync(c->k.l.sfix, c->k.l.sfix_b, sizeof(unsigned long long) * c->L * c->V,
                           cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int j = 0; j < 3; ++j) CK(cudaEventElapsedTime(&ms[j], ev[j], ev[j + 1]));
    for (int j = 0; j < 4; ++j) cudaEventDestroy(ev[j]);
    c->csr_fresh = false;
    c->list_sparse = true;
    c->t_next = t + 2;
    rc = launch_check(c);
    if (rc) return rc;
    return check_device_err(c);
}

int psim_set_alloc_fault(long long allowed) {
    g_alloc_budget.store(allowed < 0 ? -1 : allowed);
    return 0;
}

int psim_bounded_wait_selftest(psim_ctx* c, uint32_t iters) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    launch_bounded_wait_probe(c->k, iters, c->stream);
    c->launches += 1;
    int rc = launch_check(c);
    if (rc) return rc;
    return check_device_err(c);
}

}  // extern "C"
