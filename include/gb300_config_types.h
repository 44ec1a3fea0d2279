/*
 * gb300_config_types.h — the reference's configTypes.h
 * (cmake/config/in/configTypes.h.in:1-17) with the GB300 policies of
 * gb300_policies.h in place of the movement, infection, testing and closure
 * policies.  A build of the reference's main (src/main.cpp) against this
 * file instead of the generated configTypes.h runs the per-step work on a
 * GB300; the rest of the reference (input reader, progression tables,
 * statistics, immunization, output) is unchanged.
 */
#pragma once
#include <array>
#include "progressionMatrices.h"
#include "dynamicPPState.h"
#include "simulation.h"
#include "gb300_policies.h"

namespace config {
using PositionType = std::array<double, 2>;
using TypeOfLocation = unsigned;
using ProgressionMatrix = MultiBadMatrix;
using PPStates = DynamicPPState;
using Simulation_t = Simulation<PositionType, TypeOfLocation, PPStates, BasicAgentMeta, Gb300Movement, Gb300Infection,
                                Gb300Testing, Gb300Closure>;
}  // namespace config
