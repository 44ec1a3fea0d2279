// Device-side data layout of a pansim_gb300 context and the launch helpers
// shared by psim_kernels.cu (kernels) and psim_api.cu (C ABI, graphs).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pansim_gb300.h"
#include "psim_rng.h"

namespace psim {

constexpr uint32_t NONE = 0xFFFFFFFFu;
constexpr int WB_W = 0, WB_N = 1, WB_M = 2, WB_S = 3, WB_D = 4;

// error bits written by kernels into DevCtx::err
constexpr uint32_t ERR_LOCATION = 2u;      // an agent ended on an invalid location
constexpr uint32_t ERR_TEST_WAIT = 4u;     // bounded-wait self test expired (expected in tests)
constexpr uint32_t ERR_SCAN_WAIT = 1u;     // a scan tile gave up waiting for its predecessors
constexpr uint32_t ERR_AGENT_LIST = 8u;    // the agent list disagrees with the histogram or work list
constexpr uint32_t ERR_BARRIER = 16u;      // a grid barrier of the step kernel gave up waiting

struct DevModel {
    uint32_t n_states, n_variants, n_prog, n_agent_types;
    uint32_t first_infected, noncovid_dead, dead_state, n_trans;
    uint32_t n_events, pad0;
    const uint8_t* state_wb;
    const uint8_t* state_susceptible;
    const uint8_t* state_infected;
    const float* state_infectious;
    const float* state_acc_pcr;
    const float* state_acc_antigen;
    const float* variant_multiplier;
    const float* prog_scaling;
    const float* death_scaling;
    const uint32_t* tr_bad_begin;
    const uint32_t* tr_bad_count;
    const uint32_t* tr_neu_begin;
    const uint32_t* tr_neu_count;
    const uint32_t* tr_next;
    const float* tr_chance;
    const float* len_avg;
    const float* len_max;
    const uint32_t* len_thr;   // Bernoulli threshold of the geometric dwell draw
    const uint32_t* event_offset;
    const uint32_t* ev_loc_type;
    const float* ev_chance;
    const uint16_t* ev_start;
    const uint16_t* ev_end;
    const uint16_t* ev_duration;
    // per schedule slot and step of the day, the decision's active event
    // window (first event active at the step, first event starting after it;
    // -1 for none), computed on the host from the schedule table
    const int2* window;        // [n_agent_types * 28 * steps_per_day]
};

struct DevAgents {
    uint32_t n;
    const uint8_t* type;
    const uint8_t* age;
    const uint8_t* band;
    const uint16_t* prog_id;
    const float* symptom_scaling;
    const uint32_t* loc_offset;
    const uint32_t* poss_loc;
    const uint8_t* poss_type;
    const uint2* poss;            // the same entries packed: x = location, y = its type (one
                                  // 8-byte load per entry for the decisions); null when poss4
                                  // holds them
    const uint32_t* poss4;        // the same entries in 4 bytes when they fit (locations below
                                  // 2^26, types below 64): location | type << 26; else null
    const uint16_t* rep;          // replica of each agent
    uint32_t* location;
    uint32_t* move_at;            // absolute timestamp of the agent's next decision: the
                                  // reference's countdown stepsUntilMove after step t is
                                  // move_at - t - 1 (u32 arithmetic)
    int8_t* state;
    int16_t* days;
    uint8_t* variant;
    float* infectious;
    float* susceptible;           // [V][N]
    uint8_t* diagnosed;
    uint8_t* quarantined;
    uint8_t* stayed_home;
    uint8_t* no_work;
    uint32_t* last_test;
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
    const uint8_t* precond;       // pre-condition index (immunization categories, other disease)
    const uint8_t* sex;           // 0 = F, 1 = M (other disease)
    uint8_t* imm_round;           // immunization category round (0 = unassigned, 255 = declined)
    float* scaling_v;             // [V*N] symptom scaling of the states up to 6, per variant
    uint8_t* hcw;                 // healthcare worker flag
    uint32_t* rank;               // scratch of the canonical CSR ordering
    uint32_t* worklist;           // agents that decide at the next step (k_queue), one segment
                                  // per queue block
    uint32_t* home;               // [N] the agent's home: the first home-type entry of its location
                                  // list (findActualLocationForType's first match, no draw),
                                  // computed when the context is made or the home type changes
    uint32_t* move_mask;          // [MOVE_MASK_WORDS] bit s: some agent decides at step s of the
                                  // running day (a superset; rebuilt by the day's first step)
};

struct DevLocs {
    uint32_t n;
    uint32_t n_schools;
    const uint8_t* type;
    float* infectiousness;
    uint8_t* open;
    const uint8_t* essential;
    uint32_t* closed_until;
    uint32_t* quarantine_until;
    const uint32_t* schools;
    const uint32_t* classrooms;
    const uint32_t* classroom_offsets;
    const uint16_t* rep;
    uint32_t* counts;             // agents per location, built by movement
    uint32_t* cursor;             // [n] next free CSR slot of each location (scan: first slot)
    uint32_t* csr_off;            // [n+1] CSR offsets, derived from the cursors on demand
    uint32_t* csr_agents;         // [N]
    float* slot_su;               // [V][N] beside each agent-list slot: the agent's susceptibility
                                  // to the variant times its age band's factor
    uint32_t* qu_pending;         // quarantine writes of the running step
    unsigned long long* sfix;     // [V][n] fixed-point infectiousness sums
    unsigned long long* sfix_b;   // [V][n] the step kernel's second copy: even steps of the day
                                  // read sfix, odd steps sfix_b (see k_step)
    float* hazard;                // [V][n] infection ratio of the last step
    uint32_t* hmask;              // bit l: some variant's hazard at location l is > 0
    uint32_t* smask;              // bit l: some variant's fixed-point sum at l received a term this step
    float* hazard_x;              // [V][n] its argument x = k*S/n*w*season*dt (adjoint mode)
    uint32_t* no_work_loc;
    uint8_t* flags;               // testing flags
    uint32_t* tile_sums;          // per-tile sums of the histogram (two-pass scan)
    uint32_t* bar;                // the step kernel's grid barrier ([0] arrivals, [1] generation),
                                  // the counts of the three infection lists, the listing counter
    uint32_t* slot_loc;           // [N] the location of each agent-list slot the step kernel listed
    uint4* inf_pending;           // [3][N] the infections of a step (location, infectiousness
                                  // before and after, variants), in list step % 3
    uint64_t* scan_status;        // per-tile status words of the single-pass scan (epoch | flag | value)
    uint32_t* scan_state;         // [0] epoch of the next single-pass scan, [1] its tile ticket
    uint32_t* build;              // [0] timestamp at which agents last took new locations,
                                  // [1] BUILD_PENDING (rebuild at the next scan) or the timestamp
                                  //     of the scan that took the pending rebuild,
                                  // [2] the timestamp of the last step that rebuilt (decided by
                                  //     the step's first scan kernel, read by its later kernels),
                                  // [3] the timestamp of the last step whose decisions wrote a
                                  //     location quarantine (merged by that step's scan),
                                  // [5] the agent-list entries the step kernel's last rebuild
                                  //     listed
};

// Incremental CSR: at most steps of a day no agent moves, and then the
// histogram, the offsets and the agent list of the step before are this
// step's too.  A step rebuilds them (tile sums, prefix, cursors, slot
// atomics, CSR writes) only when agents took new locations for it, or after
// the state was replaced (upload, restore, explicit regroup).
constexpr uint32_t BUILD_PENDING = 0xFFFFFFFFu;

struct DevReps {
    uint32_t n;
    const uint32_t* agent_off;
    const uint32_t* loc_off;
    const unsigned long long* seed;
    const float* k_f;             // (float)k, as the reference casts it
    const uint32_t* cemetery;
    uint8_t* variant_active;      // [R][V]
    double* expected;             // [R] expected infections accumulated since the last midnight
};

// Clock of the running day, in device memory so that one captured day graph
// can be replayed for every day.
struct DevClock {
    uint32_t t0;          // timestamp of the day's midnight
    uint32_t day_of_week; // Days, holiday mode already applied
    float season;         // seasonality multiplier of the day
    uint32_t pad[5];
};

struct DevStatsAcc {      // raw per-replica daily counters
    unsigned int c[48];
    double imm[PSIM_MAX_STRAINS];
};

// launch/algorithm choices picked by the autotuner (psim_tuning)
struct DevTune {
    uint32_t agg_count;      // no effect: the histogram is updated by movers only
    uint32_t agg_slot;       // warp-aggregate the CSR slot atomics
    uint32_t blocks_per_sm;  // grid of the per-agent kernels (0 = one occupancy wave)
    uint32_t variant;        // 3: the location-ordered step (the only form)
    uint32_t scan_items;     // locations per scan thread: 2, 4 or 8 (tile = 256 x items)
    uint32_t scan_mode;      // 0 = single pass with decoupled look-back, 1 = tile sums + scan,
                             // 2 = tile sums + scan with thread-contiguous locations (items 4, 8)
};

// Adjoint accumulation (gradient of the expected new infections with respect
// to k, the location-type weights and the age-band susceptibilities)
constexpr int GRAD_K = 0;
constexpr int GRAD_W = 1;       // 8 location-type slots
constexpr int GRAD_SIGMA = 9;   // 16 age bands
constexpr int GRAD_N = 25;
struct DevAdjoint {
    uint32_t on;
    uint32_t pad;
    const double* weight;         // [R] dL/dE of the replica for the running day
    double* grad;                 // [GRAD_N] accumulated sum over replicas
    const int8_t* type_slot;      // [256] location type -> weight slot (-1: none)
};

// counters of the profiled day graph (KArgs::prof, null otherwise), summed
// over the day's steps
enum {
    PROF_DRAW_ENTRIES = 0,   // agent-list entries the draw kernel expanded
    PROF_DRAW_HAZARD = 1,    // entries at a location with a nonzero ratio
    PROF_MOVERS = 2,         // agents queued for a decision
    PROF_QUEUE_STEPS = 3,    // steps whose queue kernel passed over the agents
    PROF_REBUILDS = 4,       // steps that rebuilt the agent list
    PROF_LISTED_LOCATIONS = 5,  // locations the rebuilds listed
    PROF_LISTED_AGENTS = 6,     // agents the rebuilds listed
    PROF_N = 8,
    // Then the day's timeline (globaltimer, ns; a first entry is kept as the
    // maximum of complements, so one zero fill starts every slot):
    // [PROF_N] ~first block entry of the day's first movement, [PROF_N + 1]
    // its last block exit; per step s at PROF_T + PROF_TW * s: ~first block
    // entry, the last block past the rebuild's listing, past its slots, past
    // the draws, past the queue, last block exit (the rebuild and queue
    // slots stay 0 at steps without that phase).
    PROF_T = PROF_N + 2,
    PROF_TW = 6,
    PROF_WORDS = PROF_T + PROF_TW * 1440
};

struct KArgs {
    DevModel m;
    DevAgents a;
    DevLocs l;
    DevReps r;
    psim_params p;
    DevClock* clock;
    uint32_t* err;
    DevStatsAcc* stats;   // [R]
    uint32_t spd;         // steps per day
    uint32_t track_expected;
    DevTune tune;
    DevAdjoint adj;
    unsigned long long* prof;  // [PROF_WORDS] or null
};

// raw counter slots of DevStatsAcc::c
enum {
    SC_HOSP = 0, SC_Q, SC_QT, SC_NQ, SC_STAYED, SC_NI, SC_INF_ONCE, SC_REINF, SC_BSTR,
    SC_ALL_INF, SC_HCI, SC_HCE, SC_INFH, SC_VNI, SC_TESTS, SC_P1, SC_P2,
    SC_HIST = 17,          // 16 state slots follow... histogram lives in c[SC_HIST + s] for s < 16
    SC_VAR = 33,           // infected per variant, 7 slots
    SC_INFV = 40           // ever infected per variant, 7 slots (ends at 47)
};

#if defined(__CUDACC__)
// The first scan kernel of the step at timestamp t decides whether the CSR is
// rebuilt (agents took new locations for t, or a rebuild is pending) and
// records the decision in build[2]; its block 0 turns BUILD_PENDING into t,
// which leaves the decision of its other blocks unchanged.  Movers of the
// same launch only write build[0] for t + 1, which this launch does not
// read after its start.
// The words are written by earlier kernels (or by block 0 here, which leaves
// the decision unchanged): plain loads, so that the warps of an SM share one
// L1 line instead of queueing on one L2 address.
__device__ __forceinline__ bool csr_decide_from(const KArgs& k, uint32_t t, uint32_t moved, uint32_t force) {
    const bool r = moved == t || force == t || force == BUILD_PENDING;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (force == BUILD_PENDING) k.l.build[1] = t;
        k.l.build[2] = r ? t : NONE;
    }
    return r;
}
__device__ __forceinline__ bool csr_decide(const KArgs& k, uint32_t t) {
    return csr_decide_from(k, t, k.l.build[0], k.l.build[1]);
}
// the decision, in the later kernels of the step at t
__device__ __forceinline__ bool csr_rebuild(const KArgs& k, uint32_t t) { return k.l.build[2] == t; }
// the same decision from the words csr_decide reads, for a kernel that runs
// beside the first scan kernel (block 0's turning BUILD_PENDING into t leaves
// it unchanged)
__device__ __forceinline__ bool csr_peek(const KArgs& k, uint32_t t) {
    const uint32_t moved = k.l.build[0], force = k.l.build[1];
    return moved == t || force == t || force == BUILD_PENDING;
}
// movers of a block publish the timestamp of their new locations (one store
// per block; every thread of the block calls this)
__device__ __forceinline__ void publish_moved(const KArgs& k, bool any, uint32_t t_new) {
    if (__syncthreads_or(any) && threadIdx.x == 0) k.l.build[0] = t_new;
}

// DynamicPPState::updateMeta, dynamicPPState.cpp:54-64
__device__ __forceinline__ void update_meta(const KArgs& k, uint32_t i) {
    uint8_t s = (uint8_t)k.a.state[i];
    k.a.infectious[i] = k.m.state_infectious[s] * k.m.variant_multiplier[k.a.variant[i]];
    float su = k.m.state_susceptible[s] ? 1.0f : 0.0f;
    for (uint32_t v = 0; v < k.m.n_variants; ++v) k.a.susceptible[(size_t)v * k.a.n + i] = su;
}
#endif

// launchers (psim_kernels.cu)
void launch_movement(const KArgs& k, uint32_t step_in_day, cudaStream_t s);
void launch_count(const KArgs& k, cudaStream_t s);
// merge_quarantine: 0 no, 1 at the steps whose decisions wrote location
// quarantines, 2 always
void launch_scan(const KArgs& k, uint32_t step_in_day, int with_hazard, int merge_quarantine, cudaStream_t s);
void launch_scatter_draw(const KArgs& k, uint32_t step_in_day, int scatter, int draw, cudaStream_t s);
void launch_offsets(const KArgs& k, cudaStream_t s);
int scan_kernels(const KArgs& k);
// the step kernel (psim_kernels.cu, k_step): the phases a launch runs, and
// launches of one timestep or of a range of timesteps (grid barriers between)
constexpr uint32_t PH_REBUILD = 1u, PH_DRAW = 2u, PH_DECIDE = 4u, PH_ALL = 7u;
void launch_step(const KArgs& k, uint32_t step_in_day, uint32_t phases, cudaStream_t s);
void launch_steps(const KArgs& k, uint32_t step0, uint32_t nsteps, uint32_t phases, cudaStream_t s);
void launch_time_shift(uint32_t* a, uint32_t n, uint32_t delta, cudaStream_t s);
// words of the barrier array: two for the barrier, then the counts of the
// infections of the steps in lists 0-2 (step % 3), then the rebuild's listing
// counter (slots reserved so far)
constexpr uint32_t BAR_INFECTIONS = 2;
constexpr uint32_t BAR_LISTED = BAR_INFECTIONS + 3;
constexpr uint32_t BAR_WORDS = BAR_LISTED + 1;
// work-list segments of the decisions (blocks of the queue kernel at most)
constexpr uint32_t WORK_MAX_BLOCKS = 152u * 64u;
// words of the per-day mask of decision steps (1440 steps of one minute at most)
constexpr uint32_t MOVE_MASK_WORDS = 48;

// closure rules
struct ClosureTypes {
    uint32_t n;
    uint32_t v[10];
};
void launch_masks(const KArgs& k, uint32_t home_type, double coef, int open, cudaStream_t s);
void launch_close_types(const KArgs& k, const ClosureTypes& ty, int open, cudaStream_t s);
void launch_expose(const KArgs& k, uint32_t t, uint32_t variant, double fraction, cudaStream_t s);
void launch_canonical_csr(const KArgs& k, cudaStream_t s);
void launch_progress(const KArgs& k, uint32_t t, cudaStream_t s);
void launch_test(const KArgs& k, uint32_t t, cudaStream_t s);
void launch_stats(const KArgs& k, uint32_t t, cudaStream_t s);
void launch_variant_flags(const KArgs& k, cudaStream_t s);
void launch_homes(const KArgs& k, cudaStream_t s);
void launch_plan(const KArgs& k, uint32_t t, cudaStream_t s);
void launch_flag_hcw(const KArgs& k, cudaStream_t s);
void launch_bounded_wait_probe(const KArgs& k, uint32_t iters, cudaStream_t s);
void launch_type_weights(const KArgs& k, const float* w_by_type, cudaStream_t s);

}  // namespace psim
