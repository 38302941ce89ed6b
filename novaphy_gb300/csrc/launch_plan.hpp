// Further steps of a serving launch (csrc/pbf_serve.cu): a launch takes one
// step of each scene with pending work, then, when it is heavily loaded, more
// steps of the scenes with the deepest queues, run as consecutive steps of the
// batch.  Host-only, so the policy is tested without a GPU.
#pragma once

#include <algorithm>
#include <functional>
#include <utility>
#include <vector>

namespace pbf_plan {

struct PlanItem {
    long long n = 0;      // particles of the scene
    int avail = 0;        // further steps it may take in this launch (issuable, same dt)
    long long depth = 0;  // unissued steps after its first one (deepest queue first)
};

// Steps per item (each >= 1).  Level by level: step index s >= 1 takes the
// items that took every step before it and have a further step available,
// deepest queue first (ties: lower index), while the launch's particle-steps
// stay under min(cap, 2 x its particles).  A step index is only added when it
// holds at least max(min_step, particles / 4) particles: a batch step has a
// fixed cost, and a launch under light load must stay short for the requests
// that arrive meanwhile.  At most max_steps steps per item.
inline std::vector<int> plan_steps(const std::vector<PlanItem>& items, long long cap,
                                   long long min_step, int max_steps) {
    std::vector<int> steps(items.size(), 1);
    long long particles = 0;
    for (const PlanItem& it : items) particles += it.n;
    long long work = particles;
    const long long extra_cap = std::min(cap, 2 * particles);
    const long long level_min = std::max(std::max(min_step, 0LL), particles / 4);
    for (int level = 1; level < max_steps; ++level) {
        std::vector<std::pair<long long, int>> c;  // (depth, -item)
        for (size_t k = 0; k < items.size(); ++k)
            if (steps[k] == level && items[k].avail >= level) c.push_back({items[k].depth, -(int)k});
        std::sort(c.begin(), c.end(), std::greater<std::pair<long long, int>>());
        std::vector<size_t> take;
        long long level_particles = 0;
        for (const auto& e : c) {
            const size_t k = (size_t)(-e.second);
            if (work + level_particles + items[k].n > extra_cap) continue;
            take.push_back(k);
            level_particles += items[k].n;
        }
        if (take.empty() || level_particles < level_min) break;
        for (size_t k : take) ++steps[k];
        work += level_particles;
    }
    return steps;
}

}  // namespace pbf_plan
