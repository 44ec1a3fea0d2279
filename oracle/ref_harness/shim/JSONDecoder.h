// Shim of the reference's include/IO/JSONDecoder.h (rapidjson-based; the
// rapidjson submodule is empty).  The input-format headers only need the
// member-declaration macros; with these definitions they declare plain
// structs.  No JSON is parsed by the harness: it builds the format structs
// from the snapshot.
#pragma once
#include <stdexcept>
#include <string>
#include <vector>
#include "customExceptions.h"

namespace jsond {
template <typename T>
struct JSONDecodable {};
}  // namespace jsond

#define BEGIN_MEMBER_DECLARATIONS() static_assert(true, "")
#define DECODABLE_MEMBER(type, name) type name
#define END_MEMBER_DECLARATIONS() static_assert(true, "")
#define DECODE_JSON_FILE(file, type) (throw std::runtime_error("JSON input is not available in the harness"), type{})
