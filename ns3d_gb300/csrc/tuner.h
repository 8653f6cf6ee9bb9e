// tuner.h -- online autotuner of the loop-kernel grid of merged solve sets.
//
// A merged set's persistent loop kernel can run on any number of blocks:
// every system reduces in its fixed order whatever block processes a chunk,
// so the grid changes the speed and never the bits.  The best grid depends
// on the set: large sets stream from HBM and want every SM; sets of small,
// latency-bound systems (short multilevel passes, few chunks per system)
// spend most of an iteration in grid barriers, whose cost grows with the
// number of blocks.  The tuner times each candidate grid -- the set's base
// grid divided by 1, 2, 4, 8 -- on kSamples live launches per class of set
// (solver kind, size bucket, lanes), in round-robin order, and from then on
// launches that class with the candidate of the lowest mean time per
// row-iteration.
#pragma once

#include <cstdint>
#include <map>
#include <mutex>
#include <string>

namespace ns3d {

class GridTuner {
  public:
    static constexpr int kCandidates = 4;  // grid = base >> c, c < kCandidates
    static constexpr int kSamples = 3;     // timed launches per candidate
    // the candidate to launch this class with (the base grid when disabled)
    int choose(uint64_t key);
    // a launch of class `key` with candidate c took `ms` for `row_iters`
    // row-iterations
    void report(uint64_t key, int c, double ms, double row_iters);
    // one line per class: key fields, samples and mean cost per candidate,
    // the pick (-1 while exploring)
    std::string table();
    void set_enabled(bool on);
    void reset();

  private:
    struct Entry {
        int n[kCandidates] = {0, 0, 0, 0};
        double cost[kCandidates] = {0, 0, 0, 0};
        int pick = -1;
    };
    std::mutex mu_;
    std::map<uint64_t, Entry> t_;
    bool enabled_ = true;
};

GridTuner &grid_tuner();

// class of a merged set: kind (0 FP64; 1 mixed five-phase; 2 mixed fused;
// 3 mixed with multilevel systems), work units (power-of-two bucket) and the
// lanes sharing the SMs
inline uint64_t tuner_key(int kind, long units, int share) {
    int bucket = 0;
    while (bucket < 62 && (2L << bucket) <= units) ++bucket;
    return ((uint64_t)kind << 48) | ((uint64_t)bucket << 32) | (uint32_t)share;
}

}  // namespace ns3d
