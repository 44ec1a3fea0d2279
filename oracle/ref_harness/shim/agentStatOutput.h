// Shim of the reference's include/IO/outputs/agentStatOutput.h: the JSON agent
// statistics writer needs rapidjson (an empty submodule).  The headers the
// harness compiles include it without using it.
#pragma once
// The writer's interface (constructed on the agent statistics, writeFile),
// for code that instantiates AgentList::printAgentStatJSON
// (agentsList.h:279-283); it writes nothing.
#include <string>
class AgentStatOutput {
public:
    template <class Stats>
    explicit AgentStatOutput(const Stats&) {}
    void writeFile(const std::string&) {}
};
