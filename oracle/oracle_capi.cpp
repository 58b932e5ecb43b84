// CPU ORACLE -- test infrastructure only: a C ABI over oracle.hpp for the Python tests and the CPU
// baseline leg of bench.py (loaded with ctypes).
#include "oracle.hpp"
#include "acos_cr.hpp"

#include <cfenv>
#include <cstring>
#include <exception>
#include <string>

namespace {
thread_local std::string last_error;
}

extern "C" {

const char* sido_last_error(void) { return last_error.c_str(); }

/* counts_out: cuboids, leaves, criticals, repeated, fp32_refuted, escalated. crit_out may be NULL; it
 * receives up to crit_cap criticals (2*nargs doubles each); *crit_n receives the number of stored (lo,hi)
 * pairs. fp32_first selects the precision form, fp32_level_mask its levels that use the float pass,
 * fp32_noprop_mask those of them that skip bound propagation; part_index/part_count shard the root
 * partition's first split (part_count <= 1: whole proof). */
int sido_prove(const char* ir, unsigned generations, int max_iterations, float vol, float single, int threads,
               int fp32_first, unsigned fp32_level_mask, unsigned fp32_noprop_mask, unsigned part_index,
               unsigned part_count, unsigned long long* counts_out, double* seconds,
               double* crit_out, unsigned long long crit_cap, unsigned long long* crit_n) {
    try {
        sido::ProveOptions o;
        o.fp32_first = fp32_first != 0;
        o.fp32_level_mask = fp32_level_mask;
        o.fp32_noprop_mask = fp32_noprop_mask;
        o.part_index = part_index;
        o.part_count = part_count;
        o.generations = generations;
        o.max_iterations = max_iterations;
        o.iteration_volume = vol;
        o.iteration_single = single;
        o.threads = threads;
        o.max_criticals = crit_out ? crit_cap : 0;
        sido::ProveResult r = sido::prove(ir, o);
        counts_out[0] = r.counts.cuboids;
        counts_out[1] = r.counts.leaves;
        counts_out[2] = r.counts.criticals;
        counts_out[3] = r.counts.repeated;
        counts_out[4] = r.counts.fp32_refuted;
        counts_out[5] = r.counts.escalated;
        if(seconds) *seconds = r.seconds;
        if(crit_out && !r.criticals.empty()) {
            std::memcpy(crit_out, r.criticals.data(), r.criticals.size() * sizeof(double));
        }
        if(crit_n) *crit_n = r.criticals.empty() ? 0 : (unsigned long long)(r.criticals.size()) / 2ull;
        return 0;
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

int sido_root_box(const char* ir, double* out) {
    try {
        auto b = sido::root_box(ir);
        std::memcpy(out, b.data(), b.size() * sizeof(double));
        return 0;
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

int sido_eval_batch(const char* ir, const double* lo, const double* hi, unsigned long long n, double* out_lo,
                    double* out_hi, signed char* verdict, int threads, int float_rows_first) {
    try {
        sido::eval_batch(ir, lo, hi, n, out_lo, out_hi, reinterpret_cast<std::int8_t*>(verdict), threads,
                         float_rows_first != 0);
        return 0;
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

/* Operand expressions of the runtime comparisons: their node ids (cap entries at most; returns the count or
 * -1), and their intervals on n boxes in float (use_float != 0) or double. */
int sido_operand_nodes(const char* ir, int* ids, int cap) {
    try {
        std::vector<int> v = sido::operand_nodes(ir);
        for(std::size_t i = 0; i < v.size() && int(i) < cap; ++i) ids[i] = v[i];
        return int(v.size());
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

int sido_eval_operands(const char* ir, const double* lo, const double* hi, unsigned long long n, int use_float,
                       double* out, signed char* und, int threads) {
    try {
        sido::eval_operands(ir, lo, hi, n, use_float != 0, out, reinterpret_cast<std::int8_t*>(und), threads);
        return 0;
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

/* Constraint order of rows in the oracle's provers created from now on: 1 the engine's, 0 the reference's. */
int sido_set_device_row_order(int on) {
    sido::set_device_row_order(on != 0);
    return 0;
}

/* The engine's constraint order of row `row`: up to cap constraint ids into out; returns their number or -1. */
int sido_device_row_order(const char* ir, int row, int* out, int cap) {
    try {
        const auto rows = sido::device_row_order(std::string(ir));
        if(row < 0 || row >= int(rows.size())) return 0;
        const auto& r = rows[std::size_t(row)];
        for(std::size_t k = 0; k < r.size() && int(k) < cap; ++k) out[k] = r[k];
        return int(r.size());
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

/* Op-counting build only: operations since the last call (add/sub, mul, div, sqrt, acos), ten counts: in
 * double, then in float; 0 or -1. */
int sido_count_ops(unsigned long long* out) {
    try {
        sido::count_ops(out);
        return 0;
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

/* acos(x) rounded down (up == 0) or up, for double (n doubles) and float (n floats); 0 or -1. */
int sido_acos_rounded(const double* x, unsigned long long n, int up, double* out) {
    try {
        for(unsigned long long i = 0; i < n; ++i) out[i] = sido::acos_rounded<double>(x[i], up != 0);
        return 0;
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

/// The float pass's arc cosine bound of lemmas in double (lower for up = 0), in the oracle's round-down mode.
int sido_acos_bound_f32(const float* x, unsigned long long n, int up, float* out) {
    try {
        const int saved = std::fegetround();
        std::fesetround(FE_DOWNWARD);
        for(unsigned long long i = 0; i < n; ++i) out[i] = sido::acos_bound_f32(x[i], up != 0);
        std::fesetround(saved);
        return 0;
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

int sido_acos_rounded_f32(const float* x, unsigned long long n, int up, float* out) {
    try {
        for(unsigned long long i = 0; i < n; ++i) out[i] = sido::acos_rounded<float>(x[i], up != 0);
        return 0;
    } catch(const std::exception& e) {
        last_error = e.what();
        return -1;
    }
}

}
