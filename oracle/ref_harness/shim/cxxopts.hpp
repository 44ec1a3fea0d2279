// Minimal shim of the cxxopts API used by the reference's headers (the
// cxxopts submodule is empty): option declaration chains compile, and
// ParseResult returns values from a string map set by the harness.
#pragma once
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>

namespace cxxopts {
struct Value : std::enable_shared_from_this<Value> {
    std::string def;
    std::shared_ptr<Value> default_value(const std::string& d) {
        def = d;
        return shared_from_this();
    }
};
template <typename T>
std::shared_ptr<Value> value() {
    return std::make_shared<Value>();
}
struct OptionAdder {
    template <typename... A>
    OptionAdder& operator()(A&&...) {
        return *this;
    }
};
struct Options {
    Options(const std::string& = "", const std::string& = "") {}
    OptionAdder add_options(const std::string& = "") { return OptionAdder(); }
};
struct OptionValue {
    std::string s;
    template <typename T>
    T as() const {
        std::istringstream in(s);
        T v{};
        in >> v;
        return v;
    }
};
template <>
inline std::string OptionValue::as<std::string>() const {
    return s;
}
struct ParseResult {
    std::map<std::string, std::string> values;
    OptionValue operator[](const std::string& k) const {
        auto it = values.find(k);
        if (it == values.end()) throw std::out_of_range("option " + k);
        return OptionValue{it->second};
    }
    size_t count(const std::string& k) const { return values.count(k); }
};
}  // namespace cxxopts
