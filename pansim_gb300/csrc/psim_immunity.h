// Waning protection of a susceptible agent (the first pass of
// Immunization::update, include/immunization.h:563-693), shared by the CUDA
// kernels and the CPU oracle so that both evaluate the same float/double
// expressions in the same order.
//
// Protection tables: for table T (0 = prior infection, 1 = two doses,
// 2 = three doses, 3 = infection + two doses, 4 = infection + three doses)
// and entry j = (1 - similar) * 3 + k with k = 0 infection, 1 symptomatic,
// 2 hospitalization, wan[T][j] is the weekly waning and eff[T][j] the
// efficiency, i.e. column 2T + (1 - similar) of the --protection* options
// (immunization.h:500-529).
//
// For each variant the result is the agent's new susceptibility and, where
// the reference sets it, the symptom-scaling multiplier of the states up to
// 6.  The reference calls setScalingSymptoms three times (states 2, 4, 5),
// and all three write slot variant*7 + max(6, state) = variant*7 + 6, so
// the state-5 value (hospitalization over symptomatic) is the one kept.
#pragma once
#include <stdint.h>

#include "psim_rng.h"

typedef struct psim_imm_tables {
    float wan[5][6];
    float eff[5][6];
    int32_t similarity[7];
    float similar_multiplier[7];
} psim_imm_tables;

// MIN of include/datatypes.h:18 (a NaN second operand is returned)
PSIM_HD float psim_imm_minf(float a, float b) { return a < b ? a : b; }

// -w*weeks + e, or its blend towards the other similarity column
PSIM_HD float psim_imm_level(const psim_imm_tables* t, int tab, int a, int b, int k, uint32_t weeks, int blend,
                             float vsm) {
    const float wa = t->wan[tab][a + k], ea = t->eff[tab][a + k];
    if (blend) {
        const float wb = t->wan[tab][b + k], eb = t->eff[tab][b + k];
        return -1.0f * (wa + (wb - wa) * vsm) * (float)weeks + ea + (eb - ea) * vsm;
    }
    return -1.0f * wa * (float)weeks + ea;
}

// the infection level with the 0.95 literal (a double) for a variant the
// agent already had
PSIM_HD float psim_imm_inf_level(const psim_imm_tables* t, int tab, int a, int b, uint32_t weeks, int had, int blend,
                                 float vsm) {
    if (blend) return psim_imm_level(t, tab, a, b, 0, weeks, 1, vsm);
    const float wa = t->wan[tab][a];
    const float x = -1.0f * wa * (float)weeks;
    return (float)((double)x + (had ? 0.95 : (double)t->eff[tab][a]));
}

// Returns, per variant v < n_variants, susc[v] (already clamped with
// MIN(1, .)) and, where set_scale[v] != 0, the multiplier scale[v].
PSIM_HD void psim_imm_wane(const psim_imm_tables* t, uint32_t n_variants, uint32_t inf_count, uint32_t imm_count,
                           uint32_t weeks_inf, uint32_t weeks_imm, uint32_t prior, float* susc, float* scale,
                           uint8_t* set_scale) {
    for (uint32_t v = 0; v < n_variants; ++v) {
        susc[v] = 1.0f;
        set_scale[v] = 0;
        scale[v] = 1.0f;
    }
    const int case1 = inf_count > 0 && (imm_count == 0 || (imm_count == 1 && weeks_imm < 4));
    const int case2 = !case1 && inf_count == 0 && imm_count > 0;
    const int case3 = !case1 && !case2 && inf_count > 0 && imm_count > 0;
    for (uint32_t v = 0; v < n_variants; ++v) {
        const float vsm = t->similar_multiplier[v];
        if (case1 || case3) {
            int similar = 0;
            for (uint32_t j = 0; j < n_variants; ++j)
                similar = similar || ((prior & (1u << j)) && t->similarity[v] == t->similarity[j]);
            const int had = (prior & (1u << v)) != 0;
            const int blend = similar && !had && vsm > 0.0f;
            int tab;
            uint32_t weeks;
            if (case1) {
                tab = 0;
                weeks = weeks_inf;
            } else {
                if (imm_count == 1)
                    tab = 3;
                else if (imm_count > 1)
                    tab = 4;
                else
                    continue;
                weeks = weeks_inf < weeks_imm ? weeks_inf : weeks_imm;
            }
            const int a = (1 - similar) * 3, b = similar * 3;
            const float vs_inf = psim_imm_inf_level(t, tab, a, b, weeks, had, blend, vsm);
            susc[v] = 1.0f - vs_inf;
            const float vs_sympt = psim_imm_level(t, tab, a, b, 1, weeks, blend, vsm);
            const float vs_hosp = psim_imm_level(t, tab, a, b, 2, weeks, blend, vsm);
            scale[v] = psim_imm_minf(1.0f, (1.0f - vs_hosp) / (1.0f - vs_sympt));
            set_scale[v] = 1;
        } else if (case2) {
            const int similar = t->similarity[v] == 0;  // vaccines are for variant type 0
            const int a = (1 - similar) * 3, b = similar * 3;
            if (imm_count == 1 && weeks_imm == 0) continue;  // no protection in the first week
            float vs_inf, vs_sympt, vs_hosp;
            if (imm_count == 1 && weeks_imm < 4) {
                vs_inf = (-1.0f * t->wan[1][a] * (float)weeks_imm + t->eff[1][a]) / 2.0f;
                vs_sympt = (-1.0f * t->wan[1][a + 1] * (float)weeks_imm + t->eff[1][a + 1]) / 2.0f;
                vs_hosp = (-1.0f * t->wan[1][a + 2] * (float)weeks_imm + t->eff[1][a + 2]) / 2.0f;
            } else {
                const int tab = imm_count == 1 ? 1 : 2;
                const int blend = similar && vsm > 0.0f;
                vs_inf = psim_imm_level(t, tab, a, b, 0, weeks_imm, blend, vsm);
                vs_sympt = psim_imm_level(t, tab, a, b, 1, weeks_imm, blend, vsm);
                vs_hosp = psim_imm_level(t, tab, a, b, 2, weeks_imm, blend, vsm);
            }
            susc[v] = 1.0f - vs_inf;
            scale[v] = (1.0f - vs_hosp) / (1.0f - vs_sympt);
            set_scale[v] = 1;
        }
    }
    for (uint32_t v = 0; v < n_variants; ++v) susc[v] = psim_imm_minf(1.0f, susc[v]);
}

// the --protection* options (10 values each) as tables
PSIM_HD void psim_imm_make_tables(psim_imm_tables* t, const float* p_inf, const float* w_inf, const float* p_sym,
                                  const float* w_sym, const float* p_hosp, const float* w_hosp, const int32_t* sim,
                                  const float* vsm) {
    for (int tab = 0; tab < 5; ++tab)
        for (int d = 0; d < 2; ++d) {
            const int col = 2 * tab + d;
            t->wan[tab][d * 3 + 0] = w_inf[col];
            t->eff[tab][d * 3 + 0] = p_inf[col];
            t->wan[tab][d * 3 + 1] = w_sym[col];
            t->eff[tab][d * 3 + 1] = p_sym[col];
            t->wan[tab][d * 3 + 2] = w_hosp[col];
            t->eff[tab][d * 3 + 2] = p_hosp[col];
        }
    for (int v = 0; v < 7; ++v) {
        t->similarity[v] = sim[v];
        t->similar_multiplier[v] = vsm[v];
    }
}
