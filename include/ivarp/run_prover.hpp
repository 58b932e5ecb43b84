// ivarp::run_prover for the GB300 engine.
//
// Same signatures and results as the reference (ivarp/include/ivarp/run_prover.hpp:57-88):
// returns true iff no critical cuboid remains, fills *info with the counts, calls
// on_critical(Context{}, const NumberType* box) for every critical cuboid and
// feeds the progress observer. The proof itself runs on the GPU through the C ABI
// in sid.h; there is no CPU fallback. With the environment variable
// SID_EXPORT_DIR set, run_prover only writes the compiled lemma IR to that
// directory (lemma_<n>.sidir in call order) and returns true: this is how the
// lemma IR files are produced from unchanged lemma sources on machines without a GPU.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "prover.hpp"
#include "../sid.h"

namespace ivarp {

/// Thrown when the engine reports an error (the reference throws CUDAError, with_cuda/ivarp_cuda/error.hpp:37-59).
struct EngineError : std::runtime_error {
    EngineError(const std::string& what, int status) : std::runtime_error(what), status(status) {}
    int status;
};

/// Queue element passed to progress observers (the reference's ProofDriverQueueEntry).
template<typename NT> struct QueueHeadEntry {
    std::vector<NT> elements;
    std::size_t depth = 0;
};

namespace sid_fe {

inline void check_status(int status, const char* what) {
    if(status != SID_OK) {
        throw EngineError(std::string(what) + ": " + sid_last_error(), status);
    }
}

/// One engine per process and device, created on first use.
inline sid_engine* process_engine(int device) {
    static std::mutex mtx;
    static std::vector<std::pair<int, sid_engine*>> engines;
    std::lock_guard<std::mutex> lock(mtx);
    for(auto& e : engines) if(e.first == device) return e.second;
    sid_engine* eng = nullptr;
    check_status(sid_engine_create(device, &eng), "sid_engine_create");
    engines.emplace_back(device, eng);
    return eng;
}

inline bool export_ir(const std::string& ir) {
    const char* dir = std::getenv("SID_EXPORT_DIR");
    if(!dir || !*dir) return false;
    static int counter = 0;
    char name[64];
    std::snprintf(name, sizeof(name), "/lemma_%02d.sidir", counter++);
    std::ofstream out(std::string(dir) + name, std::ios::binary);
    out << ir;
    if(!out) throw std::runtime_error("cannot write lemma IR to SID_EXPORT_DIR");
    return true;
}

template<typename Observer, typename Context> struct ProgressBridge {
    Observer* observer;
    int nargs;
    static void call(void* user, const sid_progress* p) {
        auto* self = static_cast<ProgressBridge*>(user);
        using NT = typename Context::NumberType;
        using T = typename NT::NumberType;
        ProgressInfo info;
        info.queue_size = p->queue_size;
        info.cuboid_count = p->cuboid_count;
        info.leaf_count = p->leaf_count;
        info.critical_count = p->critical_count;
        if(p->queue_head) {
            QueueHeadEntry<NT> e;
            for(int i = 0; i < self->nargs; ++i) e.elements.emplace_back(T(p->queue_head[2 * i]), T(p->queue_head[2 * i + 1]));
            self->observer->observe_progress(Context{}, e, info);
        }
    }
};

} // namespace sid_fe

template<typename Context, typename ProgressObserver, typename OnCritical>
inline bool run_prover(const ProverInput<Context>& input, const OnCritical& c, ProofInformation* info,
                       const ProverSettings& s, ProgressObserver progress)
{
    using NT = typename Context::NumberType;
    using T = typename NT::NumberType;
    ProofInformation local;
    if(!info) info = &local;
    if(sid_fe::export_ir(input.ir)) {
        *info = ProofInformation{};
        return true;
    }

    int device = (s.cuda_device_ids.empty() || s.cuda_device_ids.front() < 0) ? 0 : s.cuda_device_ids.front();
    sid_engine* eng = sid_fe::process_engine(device);
    int lemma = -1;
    sid_fe::check_status(sid_lemma_register(eng, input.ir.data(), input.ir.size(), &lemma), "sid_lemma_register");

    sid_prove_opts opts;
    sid_prove_opts_default(&opts);
    opts.generation_count = s.generation_count;
    // the CPU prover core's default for unset values is 4 iterations (cpu_prover_core.hpp:79-92)
    opts.max_iterations_per_node = s.max_iterations_per_node < 0 ? 4 : s.max_iterations_per_node;
    opts.iteration_volume_criterion = s.iteration_volume_criterion < 0 ? 0.25f : s.iteration_volume_criterion;
    opts.iteration_single_dimension_criterion =
        s.iteration_single_dimension_criterion < 0 ? 0.66f : s.iteration_single_dimension_criterion;
    if(s.dequeue_buffer_size > 0) opts.batch_elements = s.dequeue_buffer_size;
    sid_fe::ProgressBridge<ProgressObserver, Context> bridge{&progress, int(input.num_args())};
    opts.progress = &sid_fe::ProgressBridge<ProgressObserver, Context>::call;
    opts.progress_user = &bridge;
    opts.progress_first_ms = std::uint32_t(s.start_progress_after.count());
    opts.progress_every_ms = std::uint32_t(s.progress_every.count());

    sid_result res{};
    try {
        sid_fe::check_status(sid_prove(eng, lemma, &opts, &res), "sid_prove");
    } catch(...) {
        progress.observe_error(std::current_exception(), 0);
        throw;
    }
    progress.observe_done();

    info->num_cuboids = res.num_cuboids;
    info->num_leaf_cuboids = res.num_leaf_cuboids;
    info->num_critical_cuboids = res.num_critical_cuboids;
    info->num_repeated_nodes = res.num_repeated_nodes;

    if(res.criticals_stored > 0) {
        const std::size_t nargs = input.num_args();
        std::vector<double> buf(std::size_t(res.criticals_stored) * 2 * nargs);
        std::uint64_t got = 0;
        sid_fe::check_status(sid_fetch_criticals(eng, lemma, buf.data(), res.criticals_stored, &got),
                             "sid_fetch_criticals");
        std::vector<NT> box(nargs);
        for(std::uint64_t k = 0; k < got; ++k) {
            for(std::size_t v = 0; v < nargs; ++v) {
                box[v] = NT(T(buf[(k * nargs + v) * 2]), T(buf[(k * nargs + v) * 2 + 1]));
            }
            c(Context{}, static_cast<const NT*>(box.data()));
        }
    }
    return info->num_critical_cuboids == 0;
}

template<typename Context, typename OnCritical>
inline bool run_prover(const ProverInput<Context>& input, const OnCritical& c, ProofInformation* info = nullptr,
                       const ProverSettings& s = {})
{
    return run_prover(input, c, info, s, DefaultProgressObserver{});
}

template<typename Context, typename OnCritical>
inline bool run_prover(const ProverInput<Context>& input, const OnCritical& c, const ProverSettings& s) {
    return run_prover(input, c, nullptr, s, DefaultProgressObserver{});
}

} // namespace ivarp
