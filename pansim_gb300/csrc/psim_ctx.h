// Host-side context of the C ABI, shared by the translation units that
// implement it (psim_api.cu, psim_closures.cu, psim_immunization.cu,
// psim_other_disease.cu).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "psim_device.cuh"

namespace psim {
struct ClosureEngine;
struct ImmunizationEngine;
struct OtherDiseaseEngine;
}  // namespace psim

using psim::KArgs;
using psim::DevClock;
using psim::DevStatsAcc;

struct psim_ctx {
    // host copy of the schedule table (closure rule ReduceMovement edits it)
    std::vector<uint32_t> h_event_offset, h_ev_loc_type;
    std::vector<float> h_ev_chance;
    std::vector<uint16_t> h_ev_start, h_ev_end, h_ev_duration;
    psim::ClosureEngine* closures = nullptr;
    psim::ImmunizationEngine* immunization = nullptr;
    psim::OtherDiseaseEngine* other_disease = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    // Time base of the agents' decision timestamps: the next step that
    // movement will process.  The device keeps move_at (absolute); a host
    // countdown S (stepsUntilMove) is move_at - t_next.
    uint32_t t_next = 0;
    // counters of the profiled day graph (KArgs::prof when profiling)
    unsigned long long* d_prof = nullptr;
    std::string err;
    KArgs k{};
    std::vector<void*> allocs;
    // the mutable state's one device allocation and its size
    void* state_slab = nullptr;
    size_t state_bytes = 0;
    // the home type the agents' home column was computed for
    uint32_t home_type_done = 0xFFFFFFFFu;
    uint32_t N = 0, L = 0, V = 0, R = 0, S = 0, spd = 144;
    uint64_t n_poss = 0;
    psim_params params{};
    std::vector<uint32_t> rep_agent_off, rep_loc_off, rep_cemetery, hcw_count;
    std::vector<uint64_t> rep_seed;
    std::vector<double> rep_k;
    // host copies of the per-day clock
    DevClock h_clock{};
    bool clock_valid = false;
    // graph of the steps of one day
    cudaGraphExec_t day_graph = nullptr;
    bool graph_dirty = true;
    uint64_t graph_kernels = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = 0.f;
    uint64_t launches = 0;
    bool uploaded = false;
    bool csr_fresh = false;      // counts of the current positions are built
    bool list_sparse = false;    // the agent list holds only the locations the step kernel's
                                 // last rebuild listed (psim_get_csr builds the full one)
    // pinned host memory (one block): the statistics accumulators and the
    // expected-infection sums copied back, the clock copied in, the error
    // flags copied back, so that a day needs no synchronisation in between
    void* pinned = nullptr;
    DevStatsAcc* h_stats = nullptr;   // [R]
    double* h_expected = nullptr;     // [R]
    DevClock* h_clock_pin = nullptr;
    uint32_t* h_err_pin = nullptr;
    // adjoint
    double* d_adj_weight = nullptr;
    double* d_grad = nullptr;
    int8_t* d_type_slot = nullptr;
    float* d_w_by_type = nullptr;
    // per-day checkpoints of the mutable state (device copies)
    std::vector<std::pair<void*, size_t>> regions;
    size_t checkpoint_bytes = 0;
    std::map<uint32_t, void*> checkpoints;
    std::map<uint32_t, uint32_t> checkpoint_t_next;
    // per-kernel timing inside the day graph: event-record nodes around the
    // movement of step 0 and every kernel group of every step
    bool profile = false;
    bool prof_valid = false;
};


inline int fail(psim_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return fail(c, PSIM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));        \
    } while (0)

// device error flags of the kernels since the last check (psim_api.cu)
int check_device_err(psim_ctx* c);

// cudaMalloc through the allocation-failure test hook (psim_set_alloc_fault):
// when the hook's count runs out the allocation fails without calling CUDA
cudaError_t psim_device_malloc(void** p, size_t bytes);
// the decisions' event windows of the current host schedule table, uploaded
// into a new device table (DevModel::window)
int upload_window_table(psim_ctx* c);

// non-COVID hospitalization and death (psim_other_disease.cu)
void other_disease_free(psim_ctx* c);
int other_disease_apply(psim_ctx* c, uint32_t t);

// immunization (psim_immunization.cu)
void immunization_free(psim_ctx* c);
int immunization_apply(psim_ctx* c, uint32_t t);
uint32_t immunized_today(const psim_ctx* c);

// closure rules (psim_closures.cu)
void closures_free(psim_ctx* c);
int closures_apply(psim_ctx* c, uint32_t t, const psim_day_stats* row);
