// tuner.cpp -- the online grid autotuner of merged solve sets (tuner.h) and
// its C-ABI.
#include "tuner.h"

#include <algorithm>
#include <cstdio>
#include <cstring>

#include "../../include/ns3d_capi.h"

namespace ns3d {

int GridTuner::choose(uint64_t key) {
    std::lock_guard<std::mutex> lk(mu_);
    if (!enabled_) return 0;
    Entry &e = t_[key];
    if (e.pick >= 0) return e.pick;
    int c = 0;  // the least-sampled candidate (round robin)
    for (int k = 1; k < kCandidates; ++k)
        if (e.n[k] < e.n[c]) c = k;
    return c;
}

void GridTuner::report(uint64_t key, int c, double ms, double row_iters) {
    if (c < 0 || c >= kCandidates || !(ms > 0) || !(row_iters > 0)) return;
    std::lock_guard<std::mutex> lk(mu_);
    if (!enabled_) return;
    Entry &e = t_[key];
    if (e.pick >= 0) return;
    e.n[c] += 1;
    e.cost[c] += ms / row_iters;
    for (int k = 0; k < kCandidates; ++k)
        if (e.n[k] < kSamples) return;
    int best = 0;
    for (int k = 1; k < kCandidates; ++k)
        if (e.cost[k] / e.n[k] < e.cost[best] / e.n[best]) best = k;
    e.pick = best;
}

std::string GridTuner::table() {
    std::lock_guard<std::mutex> lk(mu_);
    std::string out;
    char line[256];
    for (const auto &kv : t_) {
        const Entry &e = kv.second;
        std::snprintf(line, sizeof line, "kind=%d units<2^%d lanes=%u pick=%d ns/row-it:", (int)(kv.first >> 48),
                      (int)((kv.first >> 32) & 0xffff) + 1, (unsigned)(kv.first & 0xffffffffu), e.pick);
        out += line;
        for (int k = 0; k < kCandidates; ++k) {
            std::snprintf(line, sizeof line, " /%d:%.4g(%d)", 1 << k, e.n[k] ? 1e6 * e.cost[k] / e.n[k] : 0.0,
                          e.n[k]);
            out += line;
        }
        out += "\n";
    }
    return out;
}

void GridTuner::set_enabled(bool on) {
    std::lock_guard<std::mutex> lk(mu_);
    enabled_ = on;
}

void GridTuner::reset() {
    std::lock_guard<std::mutex> lk(mu_);
    t_.clear();
}

GridTuner &grid_tuner() {
    static GridTuner t;
    return t;
}

}  // namespace ns3d

extern "C" {

NS3D_API int ns3d_autotune_enable(int32_t mode) {
    if (mode < 0 || mode > 2) return NS3D_ERR_ARG;
    if (mode == 2) ns3d::grid_tuner().reset();
    ns3d::grid_tuner().set_enabled(mode != 0);
    return NS3D_OK;
}

NS3D_API int ns3d_autotune_table(char *buf, int32_t cap) {
    if (!buf || cap <= 0) return NS3D_ERR_ARG;
    const std::string t = ns3d::grid_tuner().table();
    const size_t n = std::min((size_t)cap - 1, t.size());
    std::memcpy(buf, t.data(), n);
    buf[n] = 0;
    return (int)t.size();
}

}  // extern "C"
