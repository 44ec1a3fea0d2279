// Non-COVID hospitalization and death at each midnight (Simulation::otherDisease,
// include/simulation.h:169-423): one kernel over the agents; when daily
// hospitalization targets cover the day, a count per replica of the agents
// in hospital with COVID comes first and sets that replica's multiplier.
#include <algorithm>
#include <vector>

#include "psim_ctx.h"
#include "psim_other_disease.h"

namespace psim {

struct OtherDiseaseEngine {
    uint32_t due_with_covid = 0;
    std::vector<int32_t> targets;   // per simulated day
    uint32_t* d_counts = nullptr;   // [R]
    float* d_mul = nullptr;         // [R]
};

}  // namespace psim

using namespace psim;

namespace {

__device__ __forceinline__ uint32_t od_wb(const KArgs& k, uint32_t i) { return k.m.state_wb[(uint8_t)k.a.state[i]]; }

// agents in hospital with COVID, per replica (simulation.h:177-195): with
// due_with_covid 0 the states 6..8 of the reference's model (I5_h, I6_h,
// R_h); with 1 the infected agents at a hospital location that were not
// discharged today (WB below S and hospitalizedUntil == t, t > 0)
__global__ void __launch_bounds__(256) k_od_count(KArgs k, uint32_t t, uint32_t due_with_covid, uint32_t* counts) {
    const uint32_t N = k.a.n, L = k.l.n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const uint32_t s = (uint8_t)k.a.state[i];
        bool hit;
        if (due_with_covid == 0) {
            hit = s >= 6u && s <= 8u;
        } else {
            const uint32_t loc = k.a.location[i];
            const uint32_t lt = loc < L ? k.l.type[loc] : NONE;
            const bool discharged = od_wb(k, i) < (uint32_t)WB_S && t > 0 && k.a.st_hospitalized_until[i] == t;
            hit = k.m.state_infected[s] != 0 && lt == k.p.hospital_type && !discharged;
        }
        if (hit) atomicAdd(&counts[k.a.rep[i]], 1u);
    }
}

// the per-agent pass (simulation.h:214-421), draws from the stream
// (agent, t, OTHER_DISEASE) in the reference's order: death at the end of a
// stay, sudden death (ignored), hospitalization, its length
__global__ void __launch_bounds__(256) k_other_disease(KArgs k, uint32_t t, uint32_t year_idx, const float* mul) {
    const uint32_t N = k.a.n;
    const uint32_t dt = k.p.time_step;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const uint32_t wb = od_wb(k, i);
        if (wb == (uint32_t)WB_D) continue;
        const uint32_t rep = k.a.rep[i];
        psim_stream rng;
        psim_stream_init(&rng, k.r.seed[rep], i - k.r.agent_off[rep], t, PSIM_PHASE_OTHER_DISEASE);
        const uint32_t ag = psim_od_age_group(k.a.age[i]);
        const uint32_t sex = k.a.sex[i] != 0 ? 1u : 0u;
        const uint32_t kind = psim_od_kind(k.a.precond[i]);
        const uint32_t until = k.a.st_hospitalized_until[i];
        if (t > 0 && until == t) {
            if (psim_u01(&rng) * 1.0 < psim_od_prob[kind][1][sex][ag]) {
                // DynamicPPState::die(false), dynamicPPState.cpp:313-325
                k.a.state[i] = (int8_t)k.m.noncovid_dead;
                k.a.days[i] = -1;
                update_meta(k, i);
                k.a.st_worst_state[i] = (int8_t)k.m.noncovid_dead;
                k.a.st_worst_ts[i] = t;
                continue;
            }
        }
        if (wb == (uint32_t)WB_S || t < until) continue;
        (void)psim_u01(&rng);  // sudden death: drawn, never applied
        const float pm = mul[rep];
        const double prob = psim_od_prob[kind][0][sex][ag] * (pm > 0.0f ? (double)pm : psim_od_year_mult[year_idx]);
        if (psim_u01(&rng) * 1.0 < prob) {
            const uint32_t avg = (uint32_t)psim_od_avg_length[kind];
            uint32_t len = (uint32_t)psim_geometric(&rng, psim_geometric_threshold(1.0 / (double)avg));
            if (len == 0) len = 1;
            k.a.st_hospitalized_ts[i] = t;
            k.a.st_hospitalized_until[i] = t + len * 24u * 60u / dt;
        }
    }
}

unsigned od_grid(uint32_t n) {
    unsigned g = (n + 255) / 256;
    if (g > 152u * 8u) g = 152u * 8u;
    return g ? g : 1u;
}

}  // namespace

void other_disease_free(psim_ctx* c) {
    if (!c->other_disease) return;
    if (c->other_disease->d_counts) cudaFree(c->other_disease->d_counts);
    if (c->other_disease->d_mul) cudaFree(c->other_disease->d_mul);
    delete c->other_disease;
    c->other_disease = nullptr;
}

int other_disease_apply(psim_ctx* c, uint32_t t) {
    OtherDiseaseEngine* E = c->other_disease;
    if (!E) return 0;
    const uint32_t day = t / c->spd;
    const unsigned grid = od_grid(c->N);
    std::vector<float> mul(c->R, 0.0f);
    if (day < E->targets.size()) {
        CK(cudaMemsetAsync(E->d_counts, 0, sizeof(uint32_t) * c->R, c->stream));
        k_od_count<<<grid, 256, 0, c->stream>>>(c->k, t, E->due_with_covid, E->d_counts);
        c->launches += 1;
        CK(cudaGetLastError());
        std::vector<uint32_t> with_covid(c->R);
        CK(cudaMemcpyAsync(with_covid.data(), E->d_counts, sizeof(uint32_t) * c->R, cudaMemcpyDeviceToHost,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
        for (uint32_t q = 0; q < c->R; ++q) mul[q] = psim_od_target_mul(E->targets[day], with_covid[q]);
    }
    CK(cudaMemcpyAsync(E->d_mul, mul.data(), sizeof(float) * c->R, cudaMemcpyHostToDevice, c->stream));
    k_other_disease<<<grid, 256, 0, c->stream>>>(c->k, t, psim_od_year_index((int32_t)day), E->d_mul);
    c->launches += 1;
    CK(cudaGetLastError());
    // the host copy of `mul` must outlive the copy
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

extern "C" {

int psim_other_disease_init(psim_ctx* c, const psim_other_disease* od) {
    if (!c) return PSIM_ERR_ARG;
    other_disease_free(c);
    if (!od || !od->enabled) return 0;
    if (!c->uploaded) return PSIM_ERR_STATE;
    if (od->n_targets && !od->total_hospitalizations)
        return fail(c, PSIM_ERR_ARG, "other disease: n_targets without total_hospitalizations");
    if (od->due_with_covid > 1) return fail(c, PSIM_ERR_ARG, "dueWithCOVID must be 0 or 1");
    OtherDiseaseEngine* E = new OtherDiseaseEngine();
    E->due_with_covid = od->due_with_covid;
    E->targets.assign(od->total_hospitalizations, od->total_hospitalizations + od->n_targets);
    if (psim_device_malloc((void**)&E->d_counts, sizeof(uint32_t) * c->R) != cudaSuccess ||
        psim_device_malloc((void**)&E->d_mul, sizeof(float) * c->R) != cudaSuccess) {
        if (E->d_counts) cudaFree(E->d_counts);
        delete E;
        return fail(c, PSIM_ERR_ALLOC, "other disease: cudaMalloc failed");
    }
    c->other_disease = E;
    return 0;
}

int psim_other_disease_day(psim_ctx* c, uint32_t t) {
    if (!c || !c->uploaded) return PSIM_ERR_STATE;
    if (!c->other_disease) return fail(c, PSIM_ERR_STATE, "other disease is off: psim_other_disease_init first");
    int rc = other_disease_apply(c, t);
    if (rc) return rc;
    return check_device_err(c);
}

}  // extern "C"
