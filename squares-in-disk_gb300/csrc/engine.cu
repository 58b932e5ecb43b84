// Host side of the GB300 prover engine: the C ABI of include/sid.h.
//
// A proof replaces the reference's ProofDriver + prover core
// (prover/proof_driver.hpp:218-627, cpu_prover/cpu_prover_core.hpp:31-260):
//   init   root partition over the dynamic variables (proof_driver.hpp:320-391)
//   loop   take a batch of queue elements (the queue is a device-resident LIFO stack);
//          run the static-split levels with hull join (cpu_prover_core.hpp:221-256);
//          route each hull: final generation -> static levels again, storing criticals
//          (proof_driver.hpp:413-423); otherwise dynamic re-split into the queue with
//          depth+1 (pd_impl_split_into.hpp:37-75).
// Each level is one kernel launch over all (item, child) pairs; level lists are processed
// in chunks so memory stays bounded. Cuboid counts are known on the host from the launch
// sizes; leaf and critical counts are accumulated on the device.
#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sid.h"
#include "engine.cuh"
#include "engine_internal.hpp"
#include "lemma_ir.hpp"

namespace sid {
extern const LemmaKernels* const kAllLemmas[];
extern const int kNumLemmas;
}

namespace {

// fixed-size storage: reporting an error never allocates
thread_local char g_last_error[512];

void set_last_error(const char* msg) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s", msg ? msg : "");
}

struct SidError {
    int status;
    std::string msg;
};

[[noreturn]] void fail(int status, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw SidError{status, buf};
}

void cuda_check(cudaError_t e, const char* what) {
    if(e != cudaSuccess) {
        if(e == cudaErrorMemoryAllocation) fail(SID_ERR_NOMEM, "%s: %s", what, cudaGetErrorString(e));
        fail(SID_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }
}

template<class F> int guarded(F&& f) {
    try {
        f();
        return SID_OK;
    } catch(const SidError& e) {
        set_last_error(e.msg.c_str());
        return e.status;
    } catch(const std::exception& e) {
        set_last_error(e.what());
        return SID_ERR_INVALID;
    }
}

/// Owning device allocation.
template<class T> struct DevBuf {
    T* p = nullptr;
    std::size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if(p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void reserve(std::size_t count) {
        if(count <= n) return;
        release();
        cuda_check(cudaMalloc(&p, std::max<std::size_t>(count, 1) * sizeof(T)), "cudaMalloc");
        n = count;
    }
};

/// A list of boxes (structure of arrays: nargs columns of `cap` double2) with per-item metadata.
struct BoxList {
    int nargs = 0;
    std::uint64_t cap = 0;
    DevBuf<double2> box;
    DevBuf<std::uint32_t> elem;
    DevBuf<std::uint64_t> path;
    DevBuf<std::uint8_t> depth;

    void reserve(int na, std::uint64_t c, bool with_elem, bool with_path, bool with_depth) {
        if(c <= cap && na == nargs) return;
        nargs = na;
        cap = c;
        box.release();
        box.reserve(std::size_t(na) * c);
        if(with_elem) { elem.release(); elem.reserve(c); }
        if(with_path) { path.release(); path.reserve(c); }
        if(with_depth) { depth.release(); depth.reserve(c); }
    }
};

struct Lemma {
    sid::LemmaIR ir;
    const sid::LemmaKernels* k = nullptr;
    DevBuf<double2> root;                // initial runtime box, computed once at registration
    std::vector<double> criticals;       // from the last proof
};

} // namespace

struct sid_engine {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<std::unique_ptr<Lemma>> lemmas;
    // scratch reused across proofs
    int sm_count = 0;
    DevBuf<unsigned long long> counters;   // [0] leaves [1] criticals [2] out_count [3] fin [4] nf
                                           // [5] escalation list length [6] escalated in total
    DevBuf<unsigned int> overflow;
    DevBuf<std::uint32_t> esc;             // precision form: escalation list of one chunk of children
    DevBuf<unsigned long long> hull;       // 4 * batch * nargs
    DevBuf<double> crit;
    BoxList queue, fin, nonfin;
    std::vector<std::unique_ptr<BoxList>> stat_levels, dyn_levels;
    DevBuf<double> batch_in_lo, batch_in_hi, batch_out_lo, batch_out_hi;
    DevBuf<std::int8_t> batch_verdict;
};

namespace sid {

struct HullArgs {
    const unsigned long long* hull_lo;
    const unsigned long long* hull_hi;
    const unsigned long long* hull_zlo;
    const unsigned long long* hull_zhi;
    const std::uint8_t* depth;          // depth of each batch element
    std::uint64_t depth_stride_base;    // element e has depth depth[e + base]
    std::uint32_t n_elem;
    int nargs;
    unsigned generations;
    // outputs: final (depth >= generations) and non-final hulls
    double2* fin_box; std::uint8_t* fin_depth; unsigned long long* fin_count;
    double2* nf_box; std::uint8_t* nf_depth; unsigned long long* nf_count;
    std::uint64_t out_stride;
};

/// Decode the per-element hull keys (AddToRange, cpu_prover_core.hpp:97-111: min of lower bounds, max
/// of upper bounds, ties kept from the first leaf in static-split order) and route each non-empty hull.
__global__ void k_hull_finalize(const HullArgs h) {
    const std::uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if(e >= h.n_elem) return;
    const std::uint64_t b0 = std::uint64_t(e) * h.nargs;
    if(h.hull_lo[b0] == ~0ull) return;           // no leaf survived
    const std::uint8_t d = h.depth[h.depth_stride_base + e];
    const bool fin = d >= h.generations;
    unsigned long long slot = atomicAdd(fin ? h.fin_count : h.nf_count, 1ull);
    double2* out = fin ? h.fin_box : h.nf_box;
    (fin ? h.fin_depth : h.nf_depth)[slot] = d;
    for(int v = 0; v < h.nargs; ++v) {
        double lo = key_value(h.hull_lo[b0 + v]);
        double hi = key_value(h.hull_hi[b0 + v]);
        if(lo == 0.0) lo = (h.hull_zlo[b0 + v] & 1ull) ? -0.0 : 0.0;
        if(hi == 0.0) hi = (h.hull_zhi[b0 + v] & 1ull) ? -0.0 : 0.0;
        out[std::uint64_t(v) * h.out_stride + slot] = make_double2(lo, hi);
    }
}

/// Lemmas without static splits: every element is itself the only leaf of its static recursion
/// (cpu_prover_core.hpp:250-256). Route elements [base, base+n) by depth like k_hull_finalize.
__global__ void k_route_elements(const double2* box, std::uint64_t stride, const std::uint8_t* depth, std::uint64_t base,
                                 std::uint64_t n, int nargs, unsigned generations,
                                 double2* fin_box, std::uint8_t* fin_depth, unsigned long long* fin_count,
                                 double2* nf_box, std::uint8_t* nf_depth, unsigned long long* nf_count,
                                 std::uint64_t out_stride) {
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const std::uint8_t d = depth[base + i];
    const bool fin = d >= generations;
    const unsigned long long slot = atomicAdd(fin ? fin_count : nf_count, 1ull);
    double2* out = fin ? fin_box : nf_box;
    (fin ? fin_depth : nf_depth)[slot] = d;
    for(int v = 0; v < nargs; ++v) out[std::uint64_t(v) * out_stride + slot] = box[std::uint64_t(v) * stride + base + i];
}

/// Lemmas without static splits, final generation: every element is a critical.
__global__ void k_store_criticals(const double2* box, std::uint64_t stride, std::uint64_t n, int nargs, double* crit,
                                  std::uint64_t crit_cap, unsigned long long* crit_count) {
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const unsigned long long slot = atomicAdd(crit_count, 1ull);
    if(slot >= crit_cap) return;
    for(int v = 0; v < nargs; ++v) {
        double2 b = box[std::uint64_t(v) * stride + i];
        crit[(slot * nargs + v) * 2] = b.x;
        crit[(slot * nargs + v) * 2 + 1] = b.y;
    }
}

} // namespace sid

namespace {

using namespace sid;

constexpr std::uint64_t kLevelCapItems = std::uint64_t(8) << 20;   // items per intermediate level list
constexpr std::uint64_t kDefaultBatch = std::uint64_t(1) << 16;    // queue elements per step
constexpr std::uint64_t kEscChunk = std::uint64_t(1) << 24;        // children per precision-form pass pair
constexpr unsigned kEscBlocksPerSM = 8;                            // grid of the escalated (double) pass

struct Prover {
    sid_engine* eng;
    Lemma* lem;
    const sid_prove_opts& opts;
    int n = 0;
    std::vector<IrSplit> dyn, stat;
    std::uint64_t batch = kDefaultBatch;
    std::uint64_t qsize = 0;
    std::uint64_t cuboids = 0;
    unsigned long long* d_leaf = nullptr;
    unsigned long long* d_crit = nullptr;
    unsigned long long* d_out = nullptr;
    unsigned long long* d_fin = nullptr;
    unsigned long long* d_nf = nullptr;
    std::uint64_t crit_cap = 0;
    std::uint64_t host_leaves = 0;     // leaves counted on the host (lemmas without static splits)
    bool fp32_first = false;           // precision form
    unsigned long long* d_esc = nullptr;
    unsigned long long* d_esc_total = nullptr;

    Prover(sid_engine* e, Lemma* l, const sid_prove_opts& o) : eng(e), lem(l), opts(o) {
        n = l->ir.nargs;
        dyn = l->ir.dynamic_splits();
        stat = l->ir.static_splits();
        if(o.batch_elements > 0) batch = std::uint64_t(o.batch_elements);
        fp32_first = o.precision == SID_PRECISION_FP32_ESCALATE && l->k->filter_f32 != nullptr;
    }

    cudaStream_t s() const { return eng->stream; }

    unsigned long long read_counter(unsigned long long* d) {
        unsigned long long v = 0;
        cuda_check(cudaMemcpyAsync(&v, d, sizeof(v), cudaMemcpyDeviceToHost, s()), "read counter");
        cuda_check(cudaStreamSynchronize(s()), "stream sync");
        return v;
    }
    void set_counter(unsigned long long* d, unsigned long long v) {
        cuda_check(cudaMemcpyAsync(d, &v, sizeof(v), cudaMemcpyHostToDevice, s()), "set counter");
    }

    LevelArgs base_args() {
        LevelArgs a{};
        a.leaf_count = d_leaf;
        a.crit_count = d_crit;
        a.crit = eng->crit.p;
        a.crit_cap = crit_cap;
        a.overflow = eng->overflow.p;
        a.out_count = d_out;
        return a;
    }

    void launch(int mode, const LevelArgs& a0) {
        const std::uint64_t total = a0.n_in * std::uint64_t(a0.nsub);
        cuboids += total;
        if(!fp32_first) {
            cuda_check(lem->k->level(mode, a0, s()), "level kernel launch");
            return;
        }
        // precision form: float pass over a chunk of children, then double pass over its escalation list
        for(std::uint64_t cb = 0; cb < total; cb += kEscChunk) {
            LevelArgs a = a0;
            a.child_begin = cb;
            a.n_child = std::min(kEscChunk, total - cb);
            a.esc = eng->esc.p;
            a.esc_count = d_esc;
            a.esc_total = d_esc_total;
            cuda_check(cudaMemsetAsync(d_esc, 0, sizeof(unsigned long long), s()), "reset escalation count");
            cuda_check(lem->k->filter_f32(a, s()), "float pass launch");
            const std::uint64_t want = (a.n_child + 127) / 128;
            const unsigned blocks = unsigned(std::min<std::uint64_t>(want, std::uint64_t(eng->sm_count) * kEscBlocksPerSM));
            cuda_check(lem->k->level_esc(mode, a, blocks, s()), "escalated pass launch");
        }
    }

    BoxList& stat_level(std::size_t j) {
        while(eng->stat_levels.size() <= j) eng->stat_levels.emplace_back(new BoxList);
        return *eng->stat_levels[j];
    }
    BoxList& dyn_level(std::size_t j) {
        while(eng->dyn_levels.size() <= j) eng->dyn_levels.emplace_back(new BoxList);
        return *eng->dyn_levels[j];
    }

    /// Ensure the queue can hold `need` elements, preserving its first qsize entries.
    void queue_reserve(std::uint64_t need) {
        BoxList& q = eng->queue;
        if(need <= q.cap && q.nargs == n) return;
        std::uint64_t ncap = std::max<std::uint64_t>(need, q.nargs == n ? q.cap * 2 : 0);
        ncap = std::max<std::uint64_t>(ncap, 1 << 16);
        DevBuf<double2> nb;
        DevBuf<std::uint8_t> nd;
        nb.reserve(std::size_t(n) * ncap);
        nd.reserve(ncap);
        if(qsize > 0 && q.nargs == n) {
            for(int v = 0; v < n; ++v) {
                cuda_check(cudaMemcpyAsync(nb.p + std::uint64_t(v) * ncap, q.box.p + std::uint64_t(v) * q.cap,
                                           qsize * sizeof(double2), cudaMemcpyDeviceToDevice, s()), "queue grow");
            }
            cuda_check(cudaMemcpyAsync(nd.p, q.depth.p, qsize, cudaMemcpyDeviceToDevice, s()), "queue grow");
        }
        cuda_check(cudaStreamSynchronize(s()), "queue grow sync");
        std::swap(q.box.p, nb.p); std::swap(q.box.n, nb.n);
        std::swap(q.depth.p, nd.p); std::swap(q.depth.n, nd.n);
        q.cap = ncap;
        q.nargs = n;
    }

    /// Dynamic levels d.. (root partition or re-split). Input items carry a depth.
    void run_dynamic(std::size_t d, const double2* in_box, std::uint64_t in_stride, const std::uint8_t* in_depth,
                     std::uint8_t depth_value, std::uint64_t n_in, bool initial, std::uint8_t depth_add) {
        const IrSplit& sp = dyn[d];
        const int nsub = int(initial ? sp.initial : sp.subdivisions);
        const int it_limit = 2 * n;
        const int rec_limit = initial ? std::min(n, 255) : std::min(n, 32);
        const bool last = d + 1 == dyn.size();
        std::uint64_t chunk;
        BoxList* out = nullptr;
        if(last) {
            chunk = std::max<std::uint64_t>(1, kLevelCapItems / std::uint64_t(nsub));
        } else {
            out = &dyn_level(d + 1);
            std::uint64_t cap = std::min<std::uint64_t>(kLevelCapItems, std::max<std::uint64_t>(n_in, 1) * nsub);
            out->reserve(n, std::max(out->cap, cap), false, false, true);
            chunk = std::max<std::uint64_t>(1, out->cap / std::uint64_t(nsub));
        }
        for(std::uint64_t off = 0; off < n_in; off += chunk) {
            const std::uint64_t len = std::min(chunk, n_in - off);
            LevelArgs a = base_args();
            a.in_box = in_box;
            a.in_stride = in_stride;
            a.in_depth = in_depth;
            a.depth_value = depth_value;
            a.in_begin = off;
            a.n_in = len;
            a.var = sp.arg;
            a.nsub = nsub;
            a.it_limit = it_limit;
            a.rec_limit = rec_limit;
            if(last) {
                queue_reserve(qsize + len * std::uint64_t(nsub));
                a.row_begin = n - 1;
                a.row_end = n;
                a.out_box = eng->queue.box.p;
                a.out_stride = eng->queue.cap;
                a.out_cap = eng->queue.cap;
                a.out_depth = eng->queue.depth.p;
                a.depth_add = depth_add;
                set_counter(d_out, qsize);
                launch(MODE_QUEUE, a);
                qsize = read_counter(d_out);
            } else {
                a.row_begin = a.row_end = 0;
                a.out_box = out->box.p;
                a.out_stride = out->cap;
                a.out_cap = out->cap;
                a.out_depth = out->depth.p;
                set_counter(d_out, 0);
                launch(MODE_EMIT, a);
                std::uint64_t cnt = read_counter(d_out);
                run_dynamic(d + 1, out->box.p, out->cap, out->depth.p, 0, cnt, initial, depth_add);
            }
        }
    }

    /// Static levels j.. over items; innermost level joins hulls (MODE_HULL) or stores criticals (MODE_CRIT).
    void run_static(std::size_t j, const double2* in_box, std::uint64_t in_stride, const std::uint32_t* in_elem,
                    const std::uint64_t* in_path, std::uint64_t in_begin, std::uint64_t n_in, int final_mode) {
        const IrSplit& sp = stat[j];
        const int nsub = int(sp.subdivisions);
        const bool last = j + 1 == stat.size();
        const int row_end = last ? n : stat[j + 1].arg;
        if(last) {
            std::uint64_t chunk = std::max<std::uint64_t>(1, (std::uint64_t(1) << 30) / std::uint64_t(nsub));
            for(std::uint64_t off = 0; off < n_in; off += chunk) {
                LevelArgs a = base_args();
                a.in_box = in_box; a.in_stride = in_stride; a.in_elem = in_elem; a.in_path = in_path;
                a.in_begin = in_begin + off; a.n_in = std::min(chunk, n_in - off);
                a.elem_base = std::uint32_t(off);
                a.var = sp.arg; a.nsub = nsub; a.it_limit = n; a.rec_limit = 4;
                a.row_begin = sp.arg; a.row_end = row_end;
                a.hull_lo = eng->hull.p;
                a.hull_hi = eng->hull.p + batch * n;
                a.hull_zlo = eng->hull.p + 2 * batch * n;
                a.hull_zhi = eng->hull.p + 3 * batch * n;
                launch(final_mode, a);
            }
            return;
        }
        BoxList& out = stat_level(j + 1);
        std::uint64_t cap = std::min<std::uint64_t>(kLevelCapItems, std::max<std::uint64_t>(n_in, 1) * nsub);
        out.reserve(n, std::max(out.cap, cap), true, true, false);
        const std::uint64_t chunk = std::max<std::uint64_t>(1, out.cap / std::uint64_t(nsub));
        for(std::uint64_t off = 0; off < n_in; off += chunk) {
            LevelArgs a = base_args();
            a.in_box = in_box; a.in_stride = in_stride; a.in_elem = in_elem; a.in_path = in_path;
            a.in_begin = in_begin + off; a.n_in = std::min(chunk, n_in - off);
            a.elem_base = std::uint32_t(off);
            a.var = sp.arg; a.nsub = nsub; a.it_limit = n; a.rec_limit = 4;
            a.row_begin = sp.arg; a.row_end = row_end;
            a.out_box = out.box.p; a.out_stride = out.cap; a.out_cap = out.cap;
            a.out_elem = out.elem.p; a.out_path = out.path.p;
            set_counter(d_out, 0);
            launch(MODE_EMIT, a);
            std::uint64_t cnt = read_counter(d_out);
            run_static(j + 1, out.box.p, out.cap, out.elem.p, out.path.p, 0, cnt, final_mode);
        }
    }

    void progress(std::chrono::steady_clock::time_point t0, std::chrono::steady_clock::time_point& last_cb, bool& first_done) {
        if(!opts.progress) return;
        auto now = std::chrono::steady_clock::now();
        auto since_start = std::chrono::duration_cast<std::chrono::milliseconds>(now - t0).count();
        auto since_last = std::chrono::duration_cast<std::chrono::milliseconds>(now - last_cb).count();
        if(!first_done ? since_start < long(opts.progress_first_ms) : since_last < long(opts.progress_every_ms)) return;
        first_done = true;
        last_cb = now;
        sid_progress p{};
        p.queue_size = qsize;
        p.cuboid_count = cuboids;
        p.leaf_count = read_counter(d_leaf);
        p.critical_count = read_counter(d_crit);
        std::vector<double> head(std::size_t(2 * n));
        if(qsize > 0) {
            for(int v = 0; v < n; ++v) {
                double2 b;
                cuda_check(cudaMemcpy(&b, eng->queue.box.p + std::uint64_t(v) * eng->queue.cap + qsize - 1, sizeof(b),
                                      cudaMemcpyDeviceToHost), "queue head");
                head[std::size_t(2 * v)] = b.x;
                head[std::size_t(2 * v + 1)] = b.y;
            }
            p.queue_head = head.data();
        }
        opts.progress(opts.progress_user, &p);
    }

    void run(sid_result* res) {
        if(opts.max_iterations_per_node > 1) {
            fail(SID_ERR_UNSUPPORTED, "max_iterations_per_node > 1 (re-iteration of a node) is not supported; use 1");
        }
        crit_cap = opts.max_criticals_kept;
        eng->counters.reserve(8);
        eng->overflow.reserve(1);
        eng->hull.reserve(4 * batch * std::uint64_t(n));
        eng->crit.reserve(std::max<std::uint64_t>(1, crit_cap) * 2 * std::uint64_t(n));
        d_leaf = eng->counters.p;
        d_crit = eng->counters.p + 1;
        d_out = eng->counters.p + 2;
        d_fin = eng->counters.p + 3;
        d_nf = eng->counters.p + 4;
        d_esc = eng->counters.p + 5;
        d_esc_total = eng->counters.p + 6;
        if(fp32_first) eng->esc.reserve(kEscChunk);
        cuda_check(cudaMemsetAsync(eng->counters.p, 0, 8 * sizeof(unsigned long long), s()), "memset counters");
        cuda_check(cudaMemsetAsync(eng->overflow.p, 0, sizeof(unsigned int), s()), "memset overflow");
        eng->fin.reserve(n, batch, false, false, true);
        eng->nonfin.reserve(n, batch, false, false, true);
        qsize = 0;
        cuboids = 0;

        cudaEvent_t ev0, ev1;
        cuda_check(cudaEventCreate(&ev0), "event");
        cuda_check(cudaEventCreate(&ev1), "event");
        cuda_check(cudaEventRecord(ev0, s()), "event record");
        auto t0 = std::chrono::steady_clock::now();
        auto last_cb = t0;
        bool first_done = false;

        // root partition of the lemma's initial runtime box
        queue_reserve(1 << 16);
        run_dynamic(0, lem->root.p, 1, nullptr, 0, 1, true, 0);

        while(qsize > 0) {
            const std::uint64_t B = std::min(qsize, batch);
            const std::uint64_t base = qsize - B;
            set_counter(d_fin, 0);
            set_counter(d_nf, 0);
            if(stat.empty()) {
                host_leaves += B;
                k_route_elements<<<unsigned((B + 127) / 128), 128, 0, s()>>>(
                    eng->queue.box.p, eng->queue.cap, eng->queue.depth.p, base, B, n, opts.generation_count,
                    eng->fin.box.p, eng->fin.depth.p, d_fin, eng->nonfin.box.p, eng->nonfin.depth.p, d_nf, batch);
                cuda_check(cudaGetLastError(), "route elements");
            } else {
                // reset hulls: lo keys to max, hi keys to 0, first-zero paths to max
                cuda_check(cudaMemsetAsync(eng->hull.p, 0xff, B * n * sizeof(unsigned long long), s()), "hull reset");
                cuda_check(cudaMemsetAsync(eng->hull.p + batch * n, 0, B * n * sizeof(unsigned long long), s()), "hull reset");
                cuda_check(cudaMemsetAsync(eng->hull.p + 2 * batch * n, 0xff, 2 * batch * n * sizeof(unsigned long long), s()), "hull reset");
                run_static(0, eng->queue.box.p, eng->queue.cap, nullptr, nullptr, base, B, MODE_HULL);
                finalize_hulls(B, base);
            }
            const std::uint64_t nfin = read_counter(d_fin);
            const std::uint64_t nnf = read_counter(d_nf);
            qsize = base;
            if(nfin > 0) {
                if(stat.empty()) {
                    host_leaves += nfin;
                    k_store_criticals<<<unsigned((nfin + 127) / 128), 128, 0, s()>>>(
                        eng->fin.box.p, batch, nfin, n, eng->crit.p, crit_cap, d_crit);
                    cuda_check(cudaGetLastError(), "store criticals");
                } else {
                    run_static(0, eng->fin.box.p, batch, nullptr, nullptr, 0, nfin, MODE_CRIT);
                }
            }
            if(nnf > 0) run_dynamic(0, eng->nonfin.box.p, batch, eng->nonfin.depth.p, 0, nnf, false, 1);
            progress(t0, last_cb, first_done);
        }
        finish(ev0, ev1, res);
    }

    void finalize_hulls(std::uint64_t B, std::uint64_t base) {
            HullArgs h{};
            h.hull_lo = eng->hull.p;
            h.hull_hi = eng->hull.p + batch * n;
            h.hull_zlo = eng->hull.p + 2 * batch * n;
            h.hull_zhi = eng->hull.p + 3 * batch * n;
            h.depth = eng->queue.depth.p;
            h.depth_stride_base = base;
            h.n_elem = std::uint32_t(B);
            h.nargs = n;
            h.generations = opts.generation_count;
            h.fin_box = eng->fin.box.p; h.fin_depth = eng->fin.depth.p; h.fin_count = d_fin;
            h.nf_box = eng->nonfin.box.p; h.nf_depth = eng->nonfin.depth.p; h.nf_count = d_nf;
            h.out_stride = batch;
            k_hull_finalize<<<unsigned((B + 127) / 128), 128, 0, s()>>>(h);
            cuda_check(cudaGetLastError(), "hull finalize");
    }

    void finish(cudaEvent_t ev0, cudaEvent_t ev1, sid_result* res) {
        cuda_check(cudaEventRecord(ev1, s()), "event record");
        cuda_check(cudaEventSynchronize(ev1), "event sync");
        float ms = 0;
        cuda_check(cudaEventElapsedTime(&ms, ev0, ev1), "elapsed");
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);

        unsigned int ovf = 0;
        cuda_check(cudaMemcpy(&ovf, eng->overflow.p, sizeof(ovf), cudaMemcpyDeviceToHost), "overflow flag");
        if(ovf) fail(SID_ERR_CUDA, "internal error: a level list overflowed");
        res->num_cuboids = cuboids;
        res->num_leaf_cuboids = read_counter(d_leaf) + host_leaves;
        res->num_critical_cuboids = read_counter(d_crit);
        res->num_repeated_nodes = 0;
        res->criticals_stored = std::min<std::uint64_t>(res->num_critical_cuboids, crit_cap);
        res->escalated = fp32_first ? read_counter(d_esc_total) : 0;
        res->seconds = double(ms) / 1000.0;
        lem->criticals.assign(std::size_t(res->criticals_stored) * 2 * std::size_t(n), 0.0);
        if(res->criticals_stored) {
            cuda_check(cudaMemcpy(lem->criticals.data(), eng->crit.p, lem->criticals.size() * sizeof(double),
                                  cudaMemcpyDeviceToHost), "copy criticals");
        }
    }
};

Lemma* get_lemma(sid_engine* e, int id) {
    if(!e) fail(SID_ERR_INVALID, "null engine");
    if(id < 0 || id >= int(e->lemmas.size())) fail(SID_ERR_INVALID, "bad lemma id %d", id);
    return e->lemmas[std::size_t(id)].get();
}

void set_device(sid_engine* e) { cuda_check(cudaSetDevice(e->device), "cudaSetDevice"); }

} // namespace

namespace sid {

void internal_set_error(const char* msg) { set_last_error(msg); }

int internal_lemma_view(sid_engine* engine, int lemma_id, LemmaView* out) {
    if(!engine || !out || lemma_id < 0 || lemma_id >= int(engine->lemmas.size())) return SID_ERR_INVALID;
    const Lemma* l = engine->lemmas[std::size_t(lemma_id)].get();
    out->kernels = l->k;
    out->device = engine->device;
    out->nargs = l->ir.nargs;
    out->last_static_arg = -1;
    out->last_static_subdivisions = 0;
    for(const auto& s : l->ir.splits) {
        if(!s.dynamic) {
            out->last_static_arg = s.arg;
            out->last_static_subdivisions = int(s.subdivisions);
        }
    }
    return SID_OK;
}

} // namespace sid

extern "C" {

void sid_prove_opts_default(sid_prove_opts* o) {
    if(!o) return;
    std::memset(o, 0, sizeof(*o));
    o->generation_count = 8;
    o->max_iterations_per_node = 1;
    o->iteration_volume_criterion = 0.25f;
    o->iteration_single_dimension_criterion = 0.66f;
    o->batch_elements = 0;
    o->precision = SID_PRECISION_PLAIN;
    o->max_criticals_kept = 1u << 20;
    o->progress_first_ms = 8000;
    o->progress_every_ms = 2000;
}

const char* sid_last_error(void) { return g_last_error; }

int sid_engine_create(int device, sid_engine** out) {
    return guarded([&] {
        if(!out) fail(SID_ERR_INVALID, "null output pointer");
        int count = 0;
        cuda_check(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
        if(device < 0 || device >= count) fail(SID_ERR_INVALID, "device %d not present (%d devices)", device, count);
        auto e = std::make_unique<sid_engine>();
        e->device = device;
        set_device(e.get());
        cuda_check(cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, device), "SM count");
        cuda_check(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        *out = e.release();
    });
}

void sid_engine_destroy(sid_engine* engine) {
    if(!engine) return;
    cudaSetDevice(engine->device);
    if(engine->stream) cudaStreamSynchronize(engine->stream);
    {
        std::unique_ptr<sid_engine> owner(engine);
        cudaStream_t s = engine->stream;
        engine->lemmas.clear();
        owner.reset();
        if(s) cudaStreamDestroy(s);
    }
}

int sid_lemma_register(sid_engine* engine, const char* ir, size_t ir_len, int* lemma_id) {
    return guarded([&] {
        if(!engine || !ir || !lemma_id) fail(SID_ERR_INVALID, "null argument");
        auto lem = std::make_unique<Lemma>();
        lem->ir = parse_lemma_ir(std::string(ir, ir_len));
        for(int i = 0; i < kNumLemmas; ++i) {
            if(kAllLemmas[i]->fingerprint == lem->ir.fingerprint) { lem->k = kAllLemmas[i]; break; }
        }
        if(!lem->k) {
            fail(SID_ERR_NOT_COMPILED,
                 "no GPU kernels were generated for lemma '%s' (fingerprint %016llx); add its IR to the build",
                 lem->ir.name.c_str(), (unsigned long long)lem->ir.fingerprint);
        }
        for(std::size_t i = 0; i < engine->lemmas.size(); ++i) {
            if(engine->lemmas[i]->ir.fingerprint == lem->ir.fingerprint) { *lemma_id = int(i); return; }
        }
        // initial runtime bounds, once per lemma (the reference computes them when building its
        // prover input, refactor_constraints_impl.hpp:90-101)
        set_device(engine);
        lem->root.reserve(std::size_t(lem->ir.nargs));
        cuda_check(lem->k->root_box(lem->root.p, engine->stream), "root box");
        cuda_check(cudaStreamSynchronize(engine->stream), "root box sync");
        engine->lemmas.push_back(std::move(lem));
        *lemma_id = int(engine->lemmas.size() - 1);
    });
}

int sid_lemma_info(sid_engine* engine, int lemma_id, int* nargs, uint64_t* fingerprint) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(nargs) *nargs = l->ir.nargs;
        if(fingerprint) *fingerprint = l->ir.fingerprint;
    });
}

int sid_lemma_root_box(sid_engine* engine, int lemma_id, double* out_lohi) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(!out_lohi) fail(SID_ERR_INVALID, "null output");
        set_device(engine);
        cuda_check(cudaMemcpyAsync(out_lohi, l->root.p, sizeof(double2) * std::size_t(l->ir.nargs),
                                   cudaMemcpyDeviceToHost, engine->stream), "root box copy");
        cuda_check(cudaStreamSynchronize(engine->stream), "root box sync");
    });
}

int sid_prove(sid_engine* engine, int lemma_id, const sid_prove_opts* opts, sid_result* result) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(!result) fail(SID_ERR_INVALID, "null result");
        sid_prove_opts o;
        if(opts) o = *opts; else sid_prove_opts_default(&o);
        if(o.precision != SID_PRECISION_PLAIN && o.precision != SID_PRECISION_FP32_ESCALATE) {
            fail(SID_ERR_INVALID, "unknown precision mode %d", o.precision);
        }
        if(o.generation_count > 250) fail(SID_ERR_INVALID, "generation_count too large");
        set_device(engine);
        std::memset(result, 0, sizeof(*result));
        Prover p(engine, l, o);
        p.run(result);
    });
}

int sid_fetch_criticals(sid_engine* engine, int lemma_id, double* out, uint64_t capacity, uint64_t* n_out) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        const std::uint64_t per = 2 * std::uint64_t(l->ir.nargs);
        const std::uint64_t have = l->criticals.size() / per;
        const std::uint64_t n = std::min(have, capacity);
        if(n && !out) fail(SID_ERR_INVALID, "null output");
        if(n) std::memcpy(out, l->criticals.data(), n * per * sizeof(double));
        if(n_out) *n_out = n;
        if(have > capacity) fail(SID_ERR_CAPACITY, "%llu criticals stored, capacity %llu",
                                 (unsigned long long)have, (unsigned long long)capacity);
    });
}

int sid_eval_batch_device(sid_engine* engine, int lemma_id, const double* lo, const double* hi, uint64_t n,
                          double* out_lo, double* out_hi, int8_t* verdict, void* stream) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(l->k->is_f32) fail(SID_ERR_UNSUPPORTED, "batch evaluation supports double lemmas");
        set_device(engine);
        BatchArgs a{lo, hi, out_lo, out_hi, verdict, n};
        cuda_check(l->k->eval_batch(a, static_cast<cudaStream_t>(stream)), "eval batch");
    });
}

int sid_eval_batch(sid_engine* engine, int lemma_id, const double* lo, const double* hi, uint64_t n,
                   double* out_lo, double* out_hi, int8_t* verdict) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(l->k->is_f32) fail(SID_ERR_UNSUPPORTED, "batch evaluation supports double lemmas");
        set_device(engine);
        const std::size_t cnt = std::size_t(n) * std::size_t(l->ir.nargs);
        engine->batch_in_lo.reserve(cnt);
        engine->batch_in_hi.reserve(cnt);
        engine->batch_out_lo.reserve(cnt);
        engine->batch_out_hi.reserve(cnt);
        engine->batch_verdict.reserve(std::size_t(n));
        cudaStream_t s = engine->stream;
        cuda_check(cudaMemcpyAsync(engine->batch_in_lo.p, lo, cnt * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
        cuda_check(cudaMemcpyAsync(engine->batch_in_hi.p, hi, cnt * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
        BatchArgs a{engine->batch_in_lo.p, engine->batch_in_hi.p, engine->batch_out_lo.p, engine->batch_out_hi.p,
                    engine->batch_verdict.p, n};
        cuda_check(l->k->eval_batch(a, s), "eval batch");
        cuda_check(cudaMemcpyAsync(out_lo, engine->batch_out_lo.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
        cuda_check(cudaMemcpyAsync(out_hi, engine->batch_out_hi.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
        cuda_check(cudaMemcpyAsync(verdict, engine->batch_verdict.p, std::size_t(n), cudaMemcpyDeviceToHost, s), "D2H");
        cuda_check(cudaStreamSynchronize(s), "eval batch sync");
    });
}

} // extern "C"
