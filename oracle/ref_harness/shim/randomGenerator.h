// Interposed RandomGenerator (include/tools/randomGenerator.h) for the
// reference-compiled harness.  Two modes:
//  - stream mode: every call draws from the calling thread's current Philox
//    stream of pansim_gb300/csrc/psim_rng.h (the harness selects the stream
//    (seed, agent, tick, phase) before each per-agent reference call), with
//    the same mappings as the GPU kernels; used to pin the oracle bit for bit;
//  - native mode: per-thread std::mt19937_64 with the reference's own CPU
//    distributions (randomGenerator.h:31-94), seeded from a given seed instead
//    of std::random_device; used for the statistical comparison and timing.
#pragma once
#include <limits.h>
#include <omp.h>

#include <random>
#include <vector>

#include "datatypes.h"
#include "timing.h"
#include "../../../pansim_gb300/csrc/psim_rng.h"

namespace harness_rng {
extern int native_mode;
extern thread_local psim_stream* current;
extern std::vector<std::mt19937_64> generators;
void seed_native(unsigned long long seed);
// the calling thread's stream; threads the harness did not give one (workers
// of a reference for_each whose draws do not decide anything) use a fixed one
inline psim_stream* stream() {
    if (current) return current;
    thread_local psim_stream fallback;
    thread_local bool ready = false;
    if (!ready) {
        psim_stream_init(&fallback, 0, 0, 0, 0);
        ready = true;
    }
    return &fallback;
}
}  // namespace harness_rng

class RandomGenerator {
public:
    static void init(unsigned) {}
    static void resize(unsigned) {}
    [[nodiscard]] static double randomUnit() {
        if (harness_rng::native_mode) {
            std::uniform_real_distribution<double> dis(0, 1);
            return dis(harness_rng::generators[omp_get_thread_num()]);
        }
        return psim_u01(harness_rng::stream());
    }
    [[nodiscard]] static double randomReal(double max) {
        if (harness_rng::native_mode) {
            std::uniform_real_distribution<double> dis(0, max);
            return dis(harness_rng::generators[omp_get_thread_num()]);
        }
        return max * psim_u01(harness_rng::stream());
    }
    [[nodiscard]] static unsigned randomUnsigned(unsigned max) {
        if (max == 0) return 0u;
        if (harness_rng::native_mode) {
            std::uniform_int_distribution<unsigned> dis(0, max - 1);
            return dis(harness_rng::generators[omp_get_thread_num()]);
        }
        return psim_below(harness_rng::stream(), max);
    }
    [[nodiscard]] static int geometric(double p) {
        if (harness_rng::native_mode) {
            std::geometric_distribution<> dis(p);
            return dis(harness_rng::generators[omp_get_thread_num()]);
        }
        return psim_geometric(harness_rng::stream(), psim_geometric_threshold(p));
    }
};
