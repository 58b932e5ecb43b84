// Collects critical cuboids into a vector (the reference's ivarp/critical_collector.hpp:34-57).
#pragma once

#include <array>
#include <mutex>
#include <vector>

#include "run_prover.hpp"

namespace ivarp {

template<typename ProverInputType> using CriticalCollection =
    std::vector<std::vector<typename ProverInputType::NumberType>>;

template<typename ProverInputType> class CriticalCollector {
public:
    CriticalCollector(CriticalCollection<ProverInputType>* out, std::mutex* lock) : out(out), lock(lock) {}
    template<typename Context, typename Values> void operator()(const Context&, const Values& v) const {
        std::lock_guard<std::mutex> g(*lock);
        out->emplace_back(v, v + n);
    }
    std::size_t n = 0;

private:
    CriticalCollection<ProverInputType>* out;
    std::mutex* lock;
};

} // namespace ivarp
