// Non-COVID hospitalization and death (Simulation::otherDisease,
// include/simulation.h:169-423): the reference's probability tables and the
// helpers that index them, shared by the CUDA kernel and the CPU oracle.
// The per-agent logic is written out in each of them.
//
// Tables by [kind][outcome][sex][age group]: kind 0 general, 1 cardiovascular
// (pre-condition 2), 2 pulmonary (pre-condition 4); outcome 0 daily
// hospitalization, 1 death at the end of a non-COVID stay; sex 0 = F, 1 = M;
// age groups 0-4, 5-14, 15-29, 30-59, 60-69, 70-79, 80+ (simulation.h:229-308,
// 326-340).  The values are model data and have to be those of the reference.
#pragma once
#include <stdint.h>

#include "psim_rng.h"

#if defined(__CUDACC__)
#define PSIM_OD_TABLE __device__ __constant__ static const
#else
#define PSIM_OD_TABLE static const
#endif

PSIM_OD_TABLE double psim_od_prob[3][2][2][7] = {
    {  // general
        {{9.52062E-05, 6.34708E-05, 0.000328928, 0.000986754, 0.00044981, 0.000623826, 0.000855563},  // hospitalization: F
         {0.00017785, 0.000118567, 0.000614453, 0.003174864, 0.001016573, 0.0011019, 0.000926381}},  // M
        {{0.003390532, 0.002260355, 0.00452071, 0.009394699, 0.016018856, 0.022216016, 0.030468759},  // death at the end of a stay: F
         {0.006333678, 0.004222452, 0.008444904, 0.030227275, 0.036202732, 0.03924143, 0.032990764}},  // M
    },
    {  // cardiovascular
        {{9.97603E-05, 6.65068E-05, 0.000335, 0.000999373, 0.000471326, 0.000653666, 0.000896488},  // hospitalization: F
         {0.000364207, 0.000242805, 0.001240249, 0.006390329, 0.002081773, 0.002256508, 0.001897075}},  // M
        {{0.001472731, 0.000981821, 0.001963642, 0.004080736, 0.006958043, 0.009649877, 0.013234587},  // death at the end of a stay: F
         {0.002751133, 0.001834089, 0.003668178, 0.013129695, 0.015725228, 0.017045135, 0.014330059}},  // M
    },
    {  // pulmonary
        {{9.84773E-05, 6.56515E-05, 0.000333289, 0.000995818, 0.000465264, 0.000645259, 0.000884959},  // hospitalization: F
         {0.00036181, 0.000241207, 0.001237053, 0.006378891, 0.002068074, 0.002241659, 0.001884591}},  // M
        {{0.006537022, 0.004358015, 0.008716029, 0.018113189, 0.030884712, 0.042832973, 0.058744446},  // death at the end of a stay: F
         {0.012211473, 0.008140982, 0.016281963, 0.058278861, 0.069799674, 0.075658351, 0.063606928}},  // M
    },
};
// The sudden-death draw (simulation.h:311-324, 373) never kills: the
// reference ANDs its comparison with false.  The draw is still made, so
// that the hospitalization draw comes after it in the agent's stream.
// average stay in days by kind, truncated to unsigned before use (simulation.h:309, 395)
PSIM_OD_TABLE double psim_od_avg_length[3] = {5.55, 2.78, 5.24};
// yearly hospital occupancy multipliers from day 99 of each year (simulation.h:389-390)
PSIM_OD_TABLE int32_t psim_od_year_day[4] = {99, 99 + 365, 99 + 2 * 365, 99 + 3 * 365};
PSIM_OD_TABLE double psim_od_year_mult[4] = {0.82, 0.67, 0.9, 0.9};

PSIM_HD uint32_t psim_od_age_group(uint32_t age) {
    return age < 5 ? 0u : age < 15 ? 1u : age < 30 ? 2u : age < 60 ? 3u : age < 70 ? 4u : age < 80 ? 5u : 6u;
}
PSIM_HD uint32_t psim_od_kind(uint32_t precond) { return precond == 2u ? 1u : (precond == 4u ? 2u : 0u); }
// index of the yearly multiplier of simulated day `day` (simulation.h:391-393).
// The reference's loop reads one element past both tables after day 1194;
// here the last multiplier holds from then on.
PSIM_HD uint32_t psim_od_year_index(int32_t day) {
    uint32_t d = 0;
    while (d < 3u && day > psim_od_year_day[d]) d++;
    return d;
}
// the daily hospitalization target's multiplier (simulation.h:196-205):
// max(0, target - with_covid * 9730000/179500) as unsigned, over 48000
static inline float psim_od_target_mul(int32_t target, uint32_t with_covid) {
    const double x = (double)target - (double)with_covid * (9730000.0 / 179500.0);
    const unsigned th = (unsigned)(x > 0.0 ? x : 0.0);
    return (float)((double)(float)th / 48000.0);
}
