// Host-side planning of the engine's request scheduling (pure functions, no CUDA; unit-tested on the CPU
// by tests/test_serve_plan.py through tests/serve_plan_check.cpp).
//
// A lane serves the requests of one lemma. Each request owns a frontier queue on the device. A step of
// the lane takes elements from the tops of its requests' queues into one batch (continuous batching:
// requests that arrived while others were running join the next step), runs the static recursion,
// hull join and dynamic re-split over the batch, and appends each element's children back to the queue
// of the request it came from. A request is finished when its queue is empty after a step.
#pragma once

#include <algorithm>
#include <cstdint>
#include <utility>
#include <vector>

namespace sid {
namespace plan {

/// Device bytes of a request: its frontier queue (nargs double2 columns plus a depth byte per element)
/// and its critical-box store (2*nargs doubles per box).
inline std::uint64_t request_bytes(int nargs, std::uint64_t queue_cap, std::uint64_t crit_cap) {
    return queue_cap * (std::uint64_t(nargs) * 16 + 1) + crit_cap * std::uint64_t(nargs) * 16;
}

/// How many of the pending requests (in arrival order, with their initial byte needs) to admit: in order
/// while the budget allows and slots are free. A request larger than the whole budget is admitted only
/// when nothing else is running, so it neither starves nor overcommits a busy device.
inline std::size_t admit_count(const std::vector<std::uint64_t>& pending_bytes, std::uint64_t used,
                               std::uint64_t budget, std::size_t running, std::size_t free_slots) {
    std::size_t k = 0;
    while(k < pending_bytes.size() && k < free_slots) {
        const std::uint64_t b = pending_bytes[k];
        const bool fits = used + b <= budget;
        if(!fits && !(running == 0 && k == 0)) break;
        used += b;
        ++running;
        ++k;
    }
    return k;
}

struct Take {
    int slot;              // request slot
    std::uint64_t begin;   // first taken queue position (the queue keeps [0, begin))
    std::uint64_t count;   // elements taken from the top
    std::uint64_t dst;     // position in the step batch
};

/// Fill one step of at most `cap` elements from the active requests, given as (slot, queue size) in
/// arrival order. Every request with work gets an equal share (cap / requests with work, rounded down)
/// so that small requests are not held behind large ones; the rest goes to the oldest requests first.
inline std::vector<Take> fill_step(const std::vector<std::pair<int, std::uint64_t>>& active, std::uint64_t cap) {
    std::vector<std::uint64_t> give(active.size(), 0);
    std::size_t with_work = 0;
    for(const auto& a : active) with_work += a.second > 0 ? 1 : 0;
    std::uint64_t left = cap;
    if(with_work > 0 && cap > 0) {
        const std::uint64_t share = cap / with_work;
        for(std::size_t i = 0; i < active.size() && left > 0; ++i) {
            const std::uint64_t g = std::min({active[i].second, share, left});
            give[i] = g;
            left -= g;
        }
        for(std::size_t i = 0; i < active.size() && left > 0; ++i) {
            const std::uint64_t g = std::min(active[i].second - give[i], left);
            give[i] += g;
            left -= g;
        }
    }
    std::vector<Take> out;
    std::uint64_t dst = 0;
    for(std::size_t i = 0; i < active.size(); ++i) {
        if(give[i] == 0) continue;
        out.push_back(Take{active[i].first, active[i].second - give[i], give[i], dst});
        dst += give[i];
    }
    return out;
}

/// Queue capacity a request needs before a step takes `taken` of its `qsize` elements: the untouched
/// part plus the worst-case children of the taken ones (each yields at most `fanout` queue entries).
inline std::uint64_t queue_need(std::uint64_t qsize, std::uint64_t taken, std::uint64_t fanout) {
    return (qsize - taken) + taken * fanout;
}

/// New capacity for a queue of capacity `cap` that must hold `need` elements (at least doubling).
inline std::uint64_t grow_capacity(std::uint64_t cap, std::uint64_t need) {
    return need <= cap ? cap : std::max(need, 2 * cap);
}

} // namespace plan
} // namespace sid
