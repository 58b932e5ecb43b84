// The C++ entry point on the GPU: proves the known-answer systems (golden/kat_systems.hpp) through
// ivarp::run_prover, the reference's interface (ivarp/include/ivarp/run_prover.hpp:57-88), linked against
// libsid.so, with the settings of the reference's own tests, and prints what run_prover returned, the
// ProofInformation it filled, the critical boxes handed to on_critical and the progress observer's calls.
// Driven and checked by tests/test_gpu_run_prover.py. Output, one record per line:
//   run <name> <generations> <max_iterations> <result 0|1> <cuboids> <leaves> <criticals> <repeated>
//       <on_critical calls> <observe_progress calls> <observe_done calls> <observe_error calls>
//   box <name> <lo hi per variable, as hex floats>           (one per critical, for runs that keep boxes)
//   printer <first line a ProgressPrinter wrote to a non-terminal stream>
//   error <status> <message>                                  (an ivarp::EngineError thrown by run_prover)
#include <chrono>
#include <cstdio>
#include <cstring>
#include <exception>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <ivarp/progress_printer.hpp>

#include "golden/kat_systems.hpp"

namespace {

struct Setting {
    const char* name;
    unsigned generations;
    int max_iterations;   // -1: left unset (run_prover's default)
    bool boxes;           // print the critical boxes
};

// the settings of the reference's tests: expected_criticals.cpp:73-75, expected_criticals2.cpp:105-106,154-155,
// 175-176,201-202, positive_and_negative_proof1.cpp:76-77,97-98, positive_and_negative_proof2.cpp:38-39,59-60,
// run_prover.cpp:63-64,86-87; plus expected_critical with the settings left at their defaults
const Setting kSettings[] = {
    {"expected_critical_f64", 2, 1, true},   {"expected_critical_f32", 2, 1, true},
    {"expected_critical_f64", 2, -1, true},  {"expected_critical2_f64", 0, 0, true},
    {"expected_critical2_f64", 1, 0, false}, {"expected_critical2_f64", 2, 0, false},
    {"expected_critical2_f32", 2, 0, false}, {"pos_neg1_sat", 7, 1, true},
    {"pos_neg1_unsat", 7, 1, false},         {"pos_neg2_sat", 16, 0, false},
    {"pos_neg2_unsat", 16, 0, false},        {"run_prover_sat_f64", 11, 1, true},
    {"run_prover_unsat_f64", 11, 1, false},  {"run_prover_sat_f32", 11, 1, true},
    {"run_prover_unsat_f32", 11, 1, false},
};

struct Counts {
    int progress = 0, done = 0, errors = 0;
};

/// A progress observer that counts the engine's calls.
struct CountingObserver {
    Counts* c;
    template<typename Context, typename Entry>
    void observe_progress(const Context&, const Entry& head, const ivarp::ProgressInfo& info) {
        if(!head.elements.empty() && info.cuboid_count > 0) ++c->progress;
    }
    void observe_done() { ++c->done; }
    void observe_error(std::exception_ptr, std::size_t) { ++c->errors; }
};

template<typename Input> void prove(const char* name, const Input& input, const Setting& s) {
    using NT = typename Input::NumberType;
    std::mutex mtx;
    std::vector<std::vector<double>> boxes;
    std::size_t calls = 0;
    const std::size_t nargs = input.num_args();
    auto on_critical = [&](const auto&, const NT* box) {
        std::lock_guard<std::mutex> lock(mtx);
        ++calls;
        if(!s.boxes) return;
        std::vector<double> b;
        for(std::size_t v = 0; v < nargs; ++v) {
            b.push_back(double(box[v].lb()));
            b.push_back(double(box[v].ub()));
        }
        boxes.push_back(std::move(b));
    };
    ivarp::ProverSettings settings;
    settings.generation_count = s.generations;
    if(s.max_iterations >= 0) settings.max_iterations_per_node = s.max_iterations;
    settings.start_progress_after = std::chrono::milliseconds(0);
    settings.progress_every = std::chrono::milliseconds(0);
    settings.dequeue_buffer_size = 64;   // several engine steps, so the observer is called between them
    ivarp::ProofInformation info;
    Counts c;
    const bool result = ivarp::run_prover(input, on_critical, &info, settings, CountingObserver{&c});
    std::printf("run %s %u %d %d %zu %zu %zu %zu %zu %d %d %d\n", name, s.generations, s.max_iterations, result ? 1 : 0,
                info.num_cuboids, info.num_leaf_cuboids, info.num_critical_cuboids, info.num_repeated_nodes, calls,
                c.progress, c.done, c.errors);
    for(const auto& b : boxes) {
        std::printf("box %s", name);
        for(double x : b) std::printf(" %a", x);
        std::printf("\n");
    }
}

} // namespace

int main() {
    using namespace ivarp;
    using namespace ivarp::args;
    for(const Setting& s : kSettings) {
        kat::for_each_system([&](const char* name, const auto&, const auto& input) {
            if(std::strcmp(name, s.name) == 0) prove(name, input, s);
        });
    }
    // the progress printer of the lemma programs (src/proof_auxiliaries.hpp:46) on a non-terminal stream:
    // one line per update
    kat::for_each_system([&](const char* name, const auto& system, const auto& input) {
        if(std::strcmp(name, "pos_neg1_unsat") != 0) return;
        std::ostringstream out;
        ProgressPrinter printer(out, 3, &system);
        ProverSettings settings;
        settings.generation_count = 7;
        settings.max_iterations_per_node = 1;
        settings.start_progress_after = std::chrono::milliseconds(0);
        settings.progress_every = std::chrono::milliseconds(0);
        settings.dequeue_buffer_size = 64;
        ProofInformation info;
        run_prover(input, [](const auto&, const auto*) {}, &info, settings, printer);
        const std::string text = out.str();
        std::printf("printer %s\n", text.substr(0, text.find('\n')).c_str());
    });
    // a system whose kernels were not generated (another split of expected_critical): the engine's error
    // surfaces as ivarp::EngineError
    {
        const auto x = x0;
        const auto y = x1;
        const auto cs = constraint_system(variable(x, "x", 0_Z, 2_Z), variable(y, "y", 0_Z, 2_Z),
                                          x >= y, x <= 3_Z - y, y <= 3_Z - x);
        using Split = U64Pack<dynamic_subdivision(8, 2), 5>;
        try {
            run_prover(prover_input<DefaultContextWithNumberType<IDouble>, Split>(cs), [](const auto&, const auto*) {});
            std::printf("error 0 no error\n");
        } catch(const EngineError& e) {
            std::printf("error %d %s\n", e.status, e.what());
        }
    }
    return 0;
}
