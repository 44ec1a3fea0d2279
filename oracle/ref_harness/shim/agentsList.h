// Shim of the reference's include/agentsList.h: dynamicPPState.h includes it
// only for AgentStats; the real header pulls the JSON data provider.
#pragma once
#include "agentStats.h"
