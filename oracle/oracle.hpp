// CPU ORACLE -- test infrastructure only.
//
// A restatement, on the CPU, of the reference prover's algorithm for the
// lemma IR: this is the checker that the GPU engine is compared with, and the
// timed CPU baseline ("port"). It is never linked into the product.
//
// What it follows (reference file:line):
//  * interval arithmetic in a global round-down FPU mode with the "opposite
//    trick" -((-a) op b) for upper bounds (ivarp/src/init_rounding.cpp:57;
//    number/float_interval_addsub.hpp:53-102, float_interval_mul.hpp:55-144,
//    float_interval_div.hpp:45-107, interval_div.hpp:113-261);
//  * sign-specialised multiplication/division/square root selected by the
//    children's compile-time bounds (tag_traits.hpp:53-76, float_interval_mul.hpp:146-164,
//    interval_div.hpp:263-288, math_fn/interval_sqrt.hpp:98-116);
//  * square = general product clamped at 0 (math_fn/fixed_pow.hpp:177-187) and
//    the CPU variant of higher integer powers (fixed_pow.hpp:93-126);
//  * min/max, if_then_else join, IBool comparisons and sequencing junctors
//    (number/minmax.hpp:58-87, eval/if_then_else.hpp:64-81,
//    number/interval_comparisons.hpp:32-119, predicate_eval/n_ary.hpp:77-120,
//    predicate_eval/basic.hpp:40-58);
//  * bound application (constraints_to_bounds/compile_time_bound.hpp:42-85,
//    number/fixed_point_bounds.hpp:111-122);
//  * worklist propagation with iteration/recursion limits
//    (bound_propagation/iterated_recursive.hpp:59-131,
//    dynamic_bound_application.hpp:59-128, index_queue_set.hpp:38-101);
//  * the proof driver: root partition, static-split recursion with hull
//    join, dynamic re-split, final generation (prover/proof_driver.hpp:302-438,491-509,
//    pd_impl_split_into.hpp:37-75, cpu_prover/cpu_prover_core.hpp:52-256);
//  * the splitter (splitter.hpp:44-59) and initial runtime bounds
//    (refactor_constraints_impl.hpp:71-101).
// Parity is pinned by the reference's published per-lemma cuboid/leaf counts
// (README.md:48-69, prover_output_23_11_2020.txt) and its known-answer tests
// (ivarp/test/expected_criticals.cpp, expected_criticals2.cpp), re-expressed in tests/.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace sido {

struct Counts {
    std::uint64_t cuboids = 0, leaves = 0, criticals = 0, repeated = 0;
    std::uint64_t fp32_refuted = 0, escalated = 0;   // precision form: children decided in float / passed on
    Counts& operator+=(const Counts& o) {
        cuboids += o.cuboids; leaves += o.leaves; criticals += o.criticals; repeated += o.repeated;
        fp32_refuted += o.fp32_refuted; escalated += o.escalated;
        return *this;
    }
};

struct ProveOptions {
    unsigned generations = 8;
    int max_iterations = 1;
    float iteration_volume = 0.25f;
    float iteration_single = 0.66f;
    int threads = 0;                 // 0: hardware concurrency
    std::uint64_t max_criticals = 0; // criticals stored
    bool fp32_first = false;         // precision form (double lemmas): children are first evaluated in
                                     // float, rounded outward; only those float cannot refute are
                                     // evaluated in double, whose results are used
    std::uint32_t fp32_level_mask = ~0u;  // precision form: levels that use the float pass (bit d: dynamic
                                          // level d, bit D + j: static level j)
    std::uint32_t fp32_noprop_mask = ~0u; // precision form: float-pass levels that test the rows on the child's
                                          // float box without bound propagation (the engine's default: all)
    std::uint32_t part_index = 0;         // sharding: with part_count > 1 only the children i of the root's
    std::uint32_t part_count = 0;         // first split with i % part_count == part_index
};

struct ProveResult {
    Counts counts;
    std::vector<double> criticals;   // (lo,hi) per variable per stored critical
    double seconds = 0;
};

/// Run a whole proof of the lemma given as IR text.
ProveResult prove(const std::string& ir, const ProveOptions& opt);

/// Leaf evaluation of n boxes (structure of arrays lo[v*n+i]): propagate after a change of the last
/// variable (it = nargs, rec = 4) and test all constraints. verdict: 0 survives, 1 empty, 2 violated.
/// float_rows_first: test the constraints in float on the box rounded outward first, and in double only
/// where float does not refute them (the device's order; same results, used to count its operations).
void eval_batch(const std::string& ir, const double* lo, const double* hi, std::uint64_t n,
                double* out_lo, double* out_hi, std::int8_t* verdict, int threads, bool float_rows_first = false);

/// Node ids of the expressions compared by the constraints' runtime comparisons (left, right per
/// comparison; constraints in table order, predicate trees in pre-order).
std::vector<int> operand_nodes(const std::string& ir);

/// Those expressions evaluated on n raw boxes (SoA lo/hi, rounded outward to float when use_float): out
/// receives (lo, hi) per box and operand, und the possibly-undefined flag.
void eval_operands(const std::string& ir, const double* lo, const double* hi, std::uint64_t n, bool use_float,
                   double* out, std::int8_t* und, int threads);

/// The op-counting build (-DSIDO_COUNT_OPS): IEEE directed-rounding operations executed since the last
/// call (additions/subtractions, multiplications, divisions, square roots, arc cosines), then reset.
void count_ops(unsigned long long out[10]);   // per kind (see make_ops_table.py), double then float

/// Test each constraint row in the engine's order (cheapest not yet evaluated constraint first) instead of the
/// reference's table order: same results, the engine's operation counts.
void set_device_row_order(bool on);
std::vector<std::vector<int>> device_row_order(const std::string& ir);   // constraint ids per row, in that order

/// Initial runtime box (2*nargs doubles).
std::vector<double> root_box(const std::string& ir);

} // namespace sido
