// Shim of the reference's include/IO/outputs/agentStatOutput.h: the JSON agent
// statistics writer needs rapidjson (an empty submodule).  The headers the
// harness compiles include it without using it.
#pragma once
