// Checks of the merged-set grid autotuner's host logic (GridTuner): built
// with the library's tuner.cpp and run by tests/test_tuner.py.
#include <cstdio>
#include <cstdlib>

#include "../../ns3d_gb300/csrc/tuner.h"

static int failures = 0;
#define CHECK(cond)                                                  \
    do {                                                             \
        if (!(cond)) {                                               \
            std::printf("FAILED line %d: %s\n", __LINE__, #cond);   \
            ++failures;                                              \
        }                                                            \
    } while (0)

int main() {
    using ns3d::GridTuner;
    GridTuner t;
    const uint64_t k = ns3d::tuner_key(0, 500, 1);
    // exploration visits the candidates round robin, kSamples times each
    int seen[GridTuner::kCandidates] = {0, 0, 0, 0};
    for (int i = 0; i < GridTuner::kCandidates * GridTuner::kSamples; ++i) {
        const int c = t.choose(k);
        CHECK(c == i % GridTuner::kCandidates);
        seen[c]++;
        t.report(k, c, c == 2 ? 1.0 : 2.0 + c, 1.0);  // candidate 2 is the fastest
    }
    for (int c = 0; c < GridTuner::kCandidates; ++c) CHECK(seen[c] == GridTuner::kSamples);
    CHECK(t.choose(k) == 2);
    t.report(k, 0, 1e-9, 1.0);  // after the pick, reports change nothing
    CHECK(t.choose(k) == 2);
    // classes are independent; invalid reports are ignored
    const uint64_t k2 = ns3d::tuner_key(3, 5000, 2);
    CHECK(k2 != k);
    t.report(k2, 0, -1.0, 1.0);
    t.report(k2, 0, 1.0, 0.0);
    t.report(k2, 7, 1.0, 1.0);
    CHECK(t.choose(k2) == 0);
    // the pick is by mean cost per row-iteration
    for (int i = 0; i < GridTuner::kCandidates * GridTuner::kSamples; ++i) {
        const int c = t.choose(k2);
        t.report(k2, c, c == 3 ? 2.0 : 4.0, c == 3 ? 4.0 : 1.0);  // candidate 3: 0.5 per row-iteration
    }
    CHECK(t.choose(k2) == 3);
    // disabled: the base grid; enabled again: the pick
    t.set_enabled(false);
    CHECK(t.choose(k) == 0 && t.choose(k2) == 0);
    t.set_enabled(true);
    CHECK(t.choose(k) == 2);
    // the table lists both classes with their picks
    const std::string tab = t.table();
    CHECK(tab.find("kind=0") != std::string::npos && tab.find("pick=2") != std::string::npos);
    CHECK(tab.find("kind=3") != std::string::npos && tab.find("pick=3") != std::string::npos);
    // reset forgets every class
    t.reset();
    CHECK(t.table().empty());
    CHECK(t.choose(k) == 0);
    // size buckets: powers of two
    CHECK(ns3d::tuner_key(0, 1, 1) == ns3d::tuner_key(0, 1, 1));
    CHECK(ns3d::tuner_key(0, 2, 1) == ns3d::tuner_key(0, 3, 1));
    CHECK(ns3d::tuner_key(0, 3, 1) != ns3d::tuner_key(0, 4, 1));
    CHECK(ns3d::tuner_key(0, 1024, 1) == ns3d::tuner_key(0, 2047, 1));
    CHECK(ns3d::tuner_key(0, 1024, 1) != ns3d::tuner_key(0, 1024, 2));
    if (failures == 0) std::printf("OK\n");
    return failures == 0 ? 0 : 1;
}
