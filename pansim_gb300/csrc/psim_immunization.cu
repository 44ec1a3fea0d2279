// Immunization (include/immunization.h:24-900): category assignment, daily
// waning, booster rounds by age group and first doses in category order.
// The per-agent passes run as kernels; the counting and the dose budgets
// (numberOfVaccinesToday / numberOfBoostersToday, the category cursor) stay
// on the host as in the reference.
#include <cstring>
#include <string>
#include <vector>

#include "psim_ctx.h"
#include "psim_immunity.h"

namespace psim {

struct ImmunizationEngine {
    psim_immunization prm;
    psim_imm_tables tables;
    bool age_groups_ready = false;
    std::vector<float> group_frac;   // [rounds * 10]
    uint32_t current_category = 0;   // Immunization::currentCategory
    uint32_t immunized_today = 0;
    uint32_t* d_counts = nullptr;    // [16] device counters
};

}  // namespace psim

using namespace psim;

namespace {

constexpr uint32_t WB_W = 0;

__device__ __forceinline__ bool has_entry(const KArgs& k, uint32_t i, uint32_t poss_type_a, uint32_t poss_type_b,
                                          uint32_t loc_type_a, uint32_t loc_type_b, bool essential) {
    for (uint32_t q = k.a.loc_offset[i]; q < k.a.loc_offset[i + 1]; ++q) {
        const uint32_t pt = k.a.poss_type[q];
        if (pt != poss_type_a && pt != poss_type_b) continue;
        const uint32_t loc = k.a.poss_loc[q];
        if (essential) {
            if (k.l.essential[loc] == 1) return true;
        } else {
            const uint32_t lt = k.l.type[loc];
            if (lt == loc_type_a || lt == loc_type_b) return true;
        }
    }
    return false;
}

// the ten categories of initCategories (immunization.h:277-375)
__device__ bool in_category(const KArgs& k, uint32_t i, uint32_t g) {
    const uint32_t age = k.a.age[i], pre = k.a.precond[i];
    switch (g) {
        case 0: return has_entry(k, i, 4, 4, 12, 14, false);   // health workers
        case 1: return has_entry(k, i, 4, 2, 22, 22, false);   // nursery home workers and residents
        case 2: return pre > 0 && age >= 60;                   // 60+ with an underlying condition
        case 3: return age >= 60;                              // 60+
        case 4: return pre > 0 && age >= 18 && age < 60;       // 18-59 with an underlying condition
        case 5: return has_entry(k, i, 4, 4, 0, 0, true);      // essential workers
        case 6: return has_entry(k, i, 4, 4, 3, 3, false);     // school workers
        case 7: return age > 17 && age < 60;                   // 18-59
        case 8: return age >= 12 && age < 18;                  // 12-17
        default: return age >= 5 && age < 12;                  // 5-11
    }
}

__device__ __forceinline__ uint32_t age_group(uint32_t age) {
    if (age >= 200u) return 10u;
    return age >= 90u ? 9u : age / 10u;
}

__device__ __forceinline__ uint32_t local_id(const KArgs& k, uint32_t i, uint32_t* rep) {
    *rep = k.a.rep[i];
    return i - k.r.agent_off[*rep];
}

__global__ void k_imm_categories(KArgs k, uint32_t g, uint32_t order_value, float level) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        if (k.a.imm_round[i] != 0 || !in_category(k, i, g)) continue;
        uint32_t rep;
        const uint32_t li = local_id(k, i, &rep);
        const double U = psim_u01_once(k.r.seed[rep], li, 0, PSIM_PHASE_IMM_CATEGORY + g);
        k.a.imm_round[i] = U < (double)level ? (uint8_t)order_value : (uint8_t)255;
    }
}

__global__ void k_imm_age_hist(KArgs k, uint32_t* out) {
    __shared__ uint32_t s[11];
    if (threadIdx.x < 11) s[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x)
        atomicAdd(&s[age_group(k.a.age[i])], 1u);
    __syncthreads();
    if (threadIdx.x < 10 && s[threadIdx.x]) atomicAdd(&out[threadIdx.x], s[threadIdx.x]);
}

// waning of every susceptible (state 0) agent (immunization.h:563-693)
__global__ void k_imm_wane(KArgs k, psim_imm_tables tab, uint32_t ts, uint32_t week_steps) {
    const uint32_t N = k.a.n, V = k.m.n_variants;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        if (k.a.state[i] != 0) continue;
        float susc[PSIM_MAX_STRAINS], scale[PSIM_MAX_STRAINS];
        uint8_t set[PSIM_MAX_STRAINS];
        const uint32_t wi = (ts - k.a.st_infected_ts[i]) / week_steps;
        const uint32_t wv = (ts - k.a.st_immunization_ts[i]) / week_steps;
        psim_imm_wane(&tab, V, k.a.st_infected_count[i], k.a.st_immunization_count[i], wi, wv,
                      k.a.st_variant_mask[i], susc, scale, set);
        const float base = k.a.symptom_scaling[i];
        for (uint32_t v = 0; v < V; ++v) {
            if (set[v]) k.a.scaling_v[(size_t)v * N + i] = base * scale[v];
            k.a.susceptible[(size_t)v * N + i] = susc[v];
        }
    }
}

// booster eligibility (immunization.h:713-723, 768-774)
__device__ __forceinline__ bool booster_eligible(const KArgs& k, uint32_t i, uint32_t ts, uint32_t spd) {
    return k.a.st_immunization_ts[i] > 0 && k.a.st_immunization_count[i] >= 1 &&
           (ts - k.a.st_immunization_ts[i]) / spd > 120u && k.m.state_wb[(uint8_t)k.a.state[i]] == WB_W &&
           ts >= spd * 90u && k.a.st_diagnosed_ts[i] < ts - spd * 120u;
}

__global__ void k_imm_booster_count(KArgs k, uint32_t ts, uint32_t spd, uint32_t* out) {
    __shared__ uint32_t s[11];
    if (threadIdx.x < 11) s[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x)
        if (booster_eligible(k, i, ts, spd)) atomicAdd(&s[age_group(k.a.age[i])], 1u);
    __syncthreads();
    if (threadIdx.x < 10 && s[threadIdx.x]) atomicAdd(&out[threadIdx.x], s[threadIdx.x]);
}

struct GroupProbs {
    float p[10];
};

__global__ void k_imm_booster_apply(KArgs k, uint32_t ts, uint32_t spd, uint32_t round, GroupProbs pr) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        const uint32_t g = age_group(k.a.age[i]);
        if (g >= 10 || !booster_eligible(k, i, ts, spd)) continue;
        const float prob = pr.p[g];
        bool give = prob == 1.0f;
        if (!give) {
            uint32_t rep;
            const uint32_t li = local_id(k, i, &rep);
            give = psim_u01_once(k.r.seed[rep], li, ts, PSIM_PHASE_IMM_BOOSTER + round) < (double)prob;
        }
        if (give) {
            k.a.st_immunization_ts[i] = ts;
            k.a.st_immunization_count[i] = k.a.st_immunization_count[i] + 1;
        }
    }
}

// first-dose eligibility (immunization.h:814-826, 840-846)
__device__ __forceinline__ bool primary_eligible(const KArgs& k, uint32_t i, uint32_t ts, uint32_t spd) {
    const uint32_t d = k.a.st_diagnosed_ts[i];
    return k.a.st_immunization_count[i] == 0 && k.m.state_wb[(uint8_t)k.a.state[i]] == WB_W &&
           ((ts < spd * 90u && d == 0) || (ts >= spd * 90u && d < ts - spd * 90u));
}

__global__ void k_imm_primary_count(KArgs k, uint32_t cc, uint32_t all, uint32_t ts, uint32_t spd, uint32_t* out) {
    uint32_t n = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x)
        if ((k.a.imm_round[i] == cc || all) && primary_eligible(k, i, ts, spd)) ++n;
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(out, n);
}

__global__ void k_imm_primary_apply(KArgs k, uint32_t cc, uint32_t ts, uint32_t spd, float prob, uint32_t cat) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x) {
        if (k.a.imm_round[i] != cc || !primary_eligible(k, i, ts, spd)) continue;
        bool give = prob == 1.0f;
        if (!give) {
            uint32_t rep;
            const uint32_t li = local_id(k, i, &rep);
            give = psim_u01_once(k.r.seed[rep], li, ts, PSIM_PHASE_IMM_PRIMARY + cat) < (double)prob;
        }
        if (give) {
            k.a.st_immunization_ts[i] = ts;
            k.a.st_immunization_count[i] = 1;
        }
    }
}

__global__ void k_imm_count_today(KArgs k, uint32_t ts, uint32_t* out) {
    uint32_t n = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.a.n; i += gridDim.x * blockDim.x)
        n += k.a.st_immunization_ts[i] == ts ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(out, n);
}

unsigned grid_n(uint32_t n) {
    unsigned g = (n + 255) / 256;
    if (g > 152u * 8u) g = 152u * 8u;
    return g ? g : 1u;
}

// counters: zero, run `launch`, read `n` values back
template <typename F>
int count_on_device(psim_ctx* c, uint32_t n, F launch, uint32_t* out) {
    ImmunizationEngine* E = c->immunization;
    CK(cudaMemsetAsync(E->d_counts, 0, sizeof(uint32_t) * 16, c->stream));
    launch();
    c->launches += 1;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, E->d_counts, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

// numberOfVaccinesToday (immunization.h:55-70)
uint32_t vaccines_today(const psim_immunization& p, uint32_t t, uint32_t spd) {
    const uint32_t day = t / spd;
    if (day < p.start_after_day) return 0;
    if (p.n_vacc_weeks == 0) return p.daily_doses;
    const uint32_t week = (day - p.start_after_day) / 7;
    const uint32_t w = week >= p.n_vacc_weeks ? p.n_vacc_weeks - 1 : week;
    return (uint32_t)(p.vacc_per_week[w] / 7.0);
}

// numberOfBoostersToday (immunization.h:72-81)
uint32_t boosters_today(const psim_immunization& p, uint32_t t, uint32_t spd, uint32_t r) {
    const uint32_t day = t / spd;
    if (day < (uint32_t)p.booster_start_after_day[r]) return 0;
    if (p.n_booster_weeks[r] == 0) return p.daily_boosters;
    const uint32_t week = (day - (uint32_t)p.booster_start_after_day[r]) / 7;
    const uint32_t w = week >= p.n_booster_weeks[r] ? p.n_booster_weeks[r] - 1 : week;
    return (uint32_t)(p.booster_per_week[r][w] / 7.0);
}

}  // namespace

void immunization_free(psim_ctx* c) {
    if (!c->immunization) return;
    if (c->immunization->d_counts) cudaFree(c->immunization->d_counts);
    delete c->immunization;
    c->immunization = nullptr;
}

// Immunization::update (immunization.h:481-900) for the midnight at t
int immunization_apply(psim_ctx* c, uint32_t t) {
    ImmunizationEngine* E = c->immunization;
    if (!E) return 0;
    const psim_immunization& p = E->prm;
    const uint32_t spd = c->spd;
    const unsigned grid = grid_n(c->N);
    int rc;
    // initAgeGroups (immunization.h:460-479), on the first call
    if (!E->age_groups_ready) {
        uint32_t hist[10];
        if ((rc = count_on_device(c, 10, [&] { k_imm_age_hist<<<grid, 256, 0, c->stream>>>(c->k, E->d_counts); }, hist)))
            return rc;
        E->group_frac.assign((size_t)p.n_booster_rounds * 10, 0.0f);
        for (uint32_t r = 0; r < p.n_booster_rounds; ++r) {
            uint32_t size[10], sum = 0;
            for (int g = 0; g < 10; ++g) {
                size[g] = (uint32_t)((float)hist[g] * p.booster_age_percent[r][g]);
                sum += size[g];
            }
            for (int g = 0; g < 10; ++g) E->group_frac[r * 10 + g] = (float)size[g] / (float)sum;
        }
        E->age_groups_ready = true;
    }
    const uint32_t ts = t == 0 ? 1u : t;
    k_imm_wane<<<grid, 256, 0, c->stream>>>(c->k, E->tables, ts, 7u * spd);
    c->launches += 1;
    // boosters, round by round (immunization.h:699-790)
    for (uint32_t r = 0; r < p.n_booster_rounds; ++r) {
        const uint32_t available = boosters_today(p, t, spd, r);
        if (!available) continue;
        uint32_t counts[10];
        if ((rc = count_on_device(
                 c, 10, [&] { k_imm_booster_count<<<grid, 256, 0, c->stream>>>(c->k, ts, spd, E->d_counts); }, counts)))
            return rc;
        GroupProbs pr;
        for (int g = 0; g < 10; ++g) {
            const uint32_t avail_g = (uint32_t)((float)available * E->group_frac[r * 10 + g]);
            pr.p[g] = counts[g] < avail_g ? 1.0f : (float)avail_g / (float)counts[g];
        }
        k_imm_booster_apply<<<grid, 256, 0, c->stream>>>(c->k, ts, spd, r, pr);
        c->launches += 1;
    }
    // first doses in category order (immunization.h:803-861)
    E->immunized_today = 0;
    uint32_t available = vaccines_today(p, t, spd);
    while (available > 0 && E->current_category < PSIM_IMM_CATEGORIES) {
        uint32_t count = 0;
        while (count == 0 && E->current_category <= PSIM_IMM_CATEGORIES) {
            const uint32_t cc = E->current_category + 1;
            const uint32_t all = cc == PSIM_IMM_CATEGORIES + 1 ? 1u : 0u;
            if ((rc = count_on_device(
                     c, 1,
                     [&] { k_imm_primary_count<<<grid, 256, 0, c->stream>>>(c->k, cc, all, ts, spd, E->d_counts); },
                     &count)))
                return rc;
            if (count == 0) E->current_category++;
        }
        const float prob = count < available ? 1.0f : (float)available / (float)count;
        k_imm_primary_apply<<<grid, 256, 0, c->stream>>>(c->k, E->current_category + 1, ts, spd, prob,
                                                         E->current_category);
        c->launches += 1;
        const uint32_t used = count < available ? count : available;
        E->immunized_today += used;
        available -= used;
    }
    uint32_t today = 0;
    if ((rc = count_on_device(c, 1, [&] { k_imm_count_today<<<grid, 256, 0, c->stream>>>(c->k, ts, E->d_counts); },
                              &today)))
        return rc;
    E->immunized_today = today;
    return 0;
}

uint32_t immunized_today(const psim_ctx* c) { return c->immunization ? c->immunization->immunized_today : 0u; }

extern "C" {

// Immunization::initializeArgs + initCategories (immunization.h:170-437)
int psim_immunization_init(psim_ctx* c, const psim_immunization* imm) {
    if (!c) return PSIM_ERR_ARG;
    immunization_free(c);
    if (!imm) return 0;
    if (!c->uploaded) return PSIM_ERR_STATE;
    if (c->R != 1) return fail(c, PSIM_ERR_ARG, "immunization needs a context with one replica");
    if (imm->n_vacc_weeks > PSIM_IMM_MAX_WEEKS || imm->n_booster_rounds > PSIM_IMM_MAX_ROUNDS)
        return fail(c, PSIM_ERR_ARG, "immunization: schedule longer than the ABI limits");
    for (uint32_t r = 0; r < imm->n_booster_rounds; ++r)
        if (imm->n_booster_weeks[r] > PSIM_IMM_MAX_WEEKS)
            return fail(c, PSIM_ERR_ARG, "immunization: booster schedule longer than the ABI limits");
    for (int g = 0; g < PSIM_IMM_CATEGORIES; ++g)
        if (imm->order[g] > PSIM_IMM_CATEGORIES)
            return fail(c, PSIM_ERR_ARG, "immunizationOrder values have to be less or equal to 10");
    ImmunizationEngine* E = new ImmunizationEngine();
    E->prm = *imm;
    psim_imm_make_tables(&E->tables, imm->protection_infection, imm->protection_infection_waning,
                         imm->protection_symptomatic, imm->protection_symptomatic_waning,
                         imm->protection_hospitalization, imm->protection_hospitalization_waning,
                         imm->variant_similarity, imm->variant_similar_multiplier);
    cudaError_t e = psim_device_malloc((void**)&E->d_counts, sizeof(uint32_t) * 16);
    if (e != cudaSuccess) {
        delete E;
        return fail(c, PSIM_ERR_ALLOC, std::string("immunization: ") + cudaGetErrorString(e));
    }
    c->immunization = E;
    // categories: for each order value 1..10, every category carrying it in
    // index order; an agent still without a round draws once
    const unsigned grid = grid_n(c->N);
    for (int v = 1; v <= PSIM_IMM_CATEGORIES; ++v)
        for (uint32_t g = 0; g < PSIM_IMM_CATEGORIES; ++g)
            if (imm->order[g] == v) {
                k_imm_categories<<<grid, 256, 0, c->stream>>>(c->k, g, (uint32_t)(uint8_t)imm->order[g],
                                                              imm->group_level[g]);
                c->launches += 1;
            }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int psim_immunize_day(psim_ctx* c, uint32_t t, uint32_t* out) {
    if (!c) return PSIM_ERR_ARG;
    if (!c->uploaded) return PSIM_ERR_STATE;
    int rc = immunization_apply(c, t);
    if (rc) return rc;
    if (out) *out = immunized_today(c);
    return 0;
}

}  // extern "C"
