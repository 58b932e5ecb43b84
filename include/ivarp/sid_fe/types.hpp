// Basic value types of the prover API: outward-rounded intervals, prover settings and the proof
// statistics. Field names and defaults follow the reference
// (ivarp/include/ivarp/number/interval.hpp, prover_input.hpp:124-159,
// prover/proof_information.hpp:32-44, default_progress_observer.hpp).
#pragma once

#include <chrono>
#include <cmath>
#include <limits>
#include <cstddef>
#include <cstdint>
#include <exception>
#include <ostream>
#include <vector>

namespace ivarp {

/// A closed interval [lb, ub] of a floating-point type with a "possibly undefined" flag.
template<typename T> class Interval {
public:
    using NumberType = T;
    Interval() = default;
    Interval(T l, T u, bool undef = false) : m_lb(l), m_ub(u), m_undefined(undef) {}
    explicit Interval(T v) : m_lb(v), m_ub(v), m_undefined(false) {}

    T lb() const noexcept { return m_lb; }
    T ub() const noexcept { return m_ub; }
    bool possibly_undefined() const noexcept { return m_undefined; }
    void set_lb(T v) noexcept { m_lb = v; }
    void set_ub(T v) noexcept { m_ub = v; }
    void set_undefined(bool u = true) noexcept { m_undefined = u; }
    bool finite_lb() const noexcept { return std::isfinite(m_lb); }
    bool finite_ub() const noexcept { return std::isfinite(m_ub); }
    bool same(const Interval& o) const noexcept {
        return m_lb == o.m_lb && m_ub == o.m_ub && m_undefined == o.m_undefined;
    }

private:
    T m_lb{}, m_ub{};
    bool m_undefined{false};
};

using IFloat = Interval<float>;
using IDouble = Interval<double>;

/// "[lb, ub]" with the digits needed to read the endpoints back exactly, "~" in front when possibly
/// undefined (the reference's float_interval_print.hpp:30-40).
template<typename T> inline std::ostream& operator<<(std::ostream& o, const Interval<T>& i) {
    const std::streamsize saved = o.precision(std::numeric_limits<T>::max_digits10);
    if(i.possibly_undefined()) o << '~';
    o << '[' << i.lb() << ", " << i.ub() << ']';
    o.precision(saved);
    return o;
}

/// Lexicographic order of intervals and boxes (used to sort reported criticals).
template<typename IT> struct IntervalLexicographicalCompare {
    bool operator()(const IT& a, const IT& b) const noexcept {
        if(a.lb() != b.lb()) return a.lb() < b.lb();
        return a.ub() < b.ub();
    }
};

template<typename NT> struct DefaultContextWithNumberType {
    using NumberType = NT;
    static constexpr bool analyze_monotonicity = false;
    static constexpr unsigned monotonicity_derivative_levels = 0;
    static constexpr unsigned irrational_precision = 256;
};

template<std::uint64_t... V> struct U64Pack {
    static constexpr std::size_t size = sizeof...(V);
    static std::vector<std::uint64_t> values() { return {V...}; }
};

constexpr std::uint64_t dynamic_subdivision(std::uint32_t initial, std::uint32_t subdivision) {
    return (std::uint64_t(initial) << 32u) | subdivision;
}

struct ProverSettings {
    /// Device ids to use; {-1} means device 0 (the engine drives one GPU).
    std::vector<int> cuda_device_ids = {-1};
    /// Number of generations of dynamic subdivision.
    unsigned generation_count = 8;
    /// Host threads (only used by CPU tooling; the proof itself runs on the GPU).
    int thread_count = -1;
    /// Queue elements expanded per engine step; <= 0 selects the engine default.
    int dequeue_buffer_size = -1;
    int cuda_threads_per_block = 256;
    std::chrono::milliseconds start_progress_after{8000};
    std::chrono::milliseconds progress_every{2000};
    /// Passes over the static splits per queue element (<= 1: one pass, as the published proofs use); -1 (unset):
    /// the reference CPU core's default of 4.
    int max_iterations_per_node = -1;
    float iteration_volume_criterion = -1.f;
    float iteration_single_dimension_criterion = -1.f;
};

struct ProofInformation {
    std::size_t num_cuboids{0};
    std::size_t num_leaf_cuboids{0};
    std::size_t num_critical_cuboids{0};
    std::size_t num_repeated_nodes{0};
};

struct ProgressInfo {
    std::size_t queue_size{0};
    std::size_t cuboid_count{0};
    std::size_t leaf_count{0};
    std::size_t critical_count{0};
};

struct DefaultProgressObserver {
    template<typename Context, typename EntryType>
    void observe_progress(const Context&, const EntryType&, const ProgressInfo&) const noexcept {}
    void observe_done() const noexcept {}
    void observe_error(std::exception_ptr, std::size_t) const noexcept {}
};

} // namespace ivarp
