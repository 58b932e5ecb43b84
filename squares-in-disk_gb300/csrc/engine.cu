// Host side of the GB300 prover engine: the C ABI of include/sid.h.
//
// A proof replaces the reference's ProofDriver + prover core
// (prover/proof_driver.hpp:218-627, cpu_prover/cpu_prover_core.hpp:31-260):
//   init   root partition over the dynamic variables (proof_driver.hpp:320-391)
//   loop   take elements from the top of the queue (a device-resident LIFO stack);
//          run the static-split levels with hull join (cpu_prover_core.hpp:221-256);
//          route each hull: final generation -> static levels again, storing criticals
//          (proof_driver.hpp:413-423); otherwise dynamic re-split into the queue with
//          depth+1 (pd_impl_split_into.hpp:37-75).
// Each level is one kernel launch over all (item, child) pairs; level lists are processed
// in chunks so memory stays bounded. Counts are accumulated on the device per request.
//
// Work is organised in lanes: a lane owns the scratch of one lemma and serves any number of requests
// of that lemma; every element carries the tag (slot) of its request, whose counters, frontier queue
// and critical store live in a device table. sid_prove runs one request on a lane cached in the
// engine; the server (sid_server_*) runs one lane per lemma on its own thread and stream and batches
// the elements of all admitted requests of that lemma into each step.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sid.h"
#include "engine.cuh"
#include "engine_internal.hpp"
#include "lemma_ir.hpp"
#include "proof_loop.cuh"
#include "serve_plan.hpp"

namespace sid {
extern const LemmaKernels* const kAllLemmas[];
extern const int kNumLemmas;
extern const BundleKernels* const kAllBundles[];
extern const int kNumBundles;
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

// Host-side fault injection (sid_debug_inject_failure): per kind, the number of failure points still to pass
// before one fails (0: disarmed). Nothing is ever injected on the device.
std::atomic<long long> g_inject_countdown[3];

bool inject_now(int kind) {
    std::atomic<long long>& c = g_inject_countdown[kind];
    long long v = c.load();
    while(v > 0) {
        if(c.compare_exchange_weak(v, v - 1)) return v == 1;
    }
    return false;
}

/// Called before each launch of the proof and batch paths: an armed launch injection fails here, before
/// anything is launched.
void launch_gate(const char* what) {
    if(inject_now(SID_INJECT_LAUNCH)) {
        fail(SID_ERR_CUDA, "%s: %s (injected; nothing was launched)", what, cudaGetErrorString(cudaErrorLaunchFailure));
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

/// Owning device allocation; reserve_on allocates stream-ordered (freed in order on the same stream,
/// without the device-wide synchronisation of cudaFree).
template<class T> struct DevBuf {
    T* p = nullptr;
    std::size_t n = 0;
    cudaStream_t ordered = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if(p) {
            if(ordered) cudaFreeAsync(p, ordered);
            else cudaFree(p);
        }
        p = nullptr;
        n = 0;
        ordered = nullptr;
    }
    void reserve(std::size_t count) {
        if(count <= n) return;
        release();
        cuda_check(inject_now(SID_INJECT_ALLOC) ? cudaErrorMemoryAllocation
                                                : cudaMalloc(&p, std::max<std::size_t>(count, 1) * sizeof(T)),
                   "cudaMalloc");
        n = count;
    }
    void reserve_on(std::size_t count, cudaStream_t s) {
        if(count <= n) return;
        release();
        cuda_check(inject_now(SID_INJECT_ALLOC)
                       ? cudaErrorMemoryAllocation
                       : cudaMallocAsync(reinterpret_cast<void**>(&p), std::max<std::size_t>(count, 1) * sizeof(T), s),
                   "cudaMallocAsync");
        n = count;
        ordered = s;
    }
    void swap(DevBuf& o) {
        std::swap(p, o.p);
        std::swap(n, o.n);
        std::swap(ordered, o.ordered);
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
    DevBuf<std::uint32_t> tag;

    void reserve(int na, std::uint64_t c, bool with_elem, bool with_path, bool with_depth, bool with_tag) {
        if(c <= cap && na == nargs) return;
        nargs = 0;   // the list has no capacity until every column is allocated (an allocation may fail)
        cap = 0;
        box.release();
        box.reserve(std::size_t(na) * c);
        if(with_elem) { elem.release(); elem.reserve(c); }
        if(with_path) { path.release(); path.reserve(c); }
        if(with_depth) { depth.release(); depth.reserve(c); }
        if(with_tag) { tag.release(); tag.reserve(c); }
        nargs = na;
        cap = c;
    }
};

struct Lemma {
    sid::LemmaIR ir;
    const sid::LemmaKernels* k = nullptr;
    DevBuf<double2> root;                // initial runtime box, computed once at registration
    std::vector<double> root_host;       // the same, (lo, hi) per variable
    bool tuned = false;                  // sid_lemma_autotune has chosen the precision-form configuration
    sid_tuning tuning{};
    std::vector<double> criticals;       // from the last sid_prove
    // batch ordering of sid_eval_batch*: the mode, and the share of a sampled call's cuboids whose
    // constraints the float test left to double (-1: no sample yet), read without blocking once the
    // sampled call's copy of its counter has completed
    int batch_order = SID_BATCH_ORDER_AUTO;
    double batch_double_share = -1.0;
    DevBuf<unsigned long long> batch_sample;
    unsigned long long* batch_sample_host = nullptr;   // pinned
    cudaEvent_t batch_sample_ev = nullptr;
    bool batch_sample_pending = false;
    std::uint64_t batch_sample_n = 0;
    Lemma() = default;
    Lemma(const Lemma&) = delete;
    Lemma& operator=(const Lemma&) = delete;
    ~Lemma() {
        if(batch_sample_ev) cudaEventDestroy(batch_sample_ev);
        if(batch_sample_host) cudaFreeHost(batch_sample_host);
    }
};

using Clock = std::chrono::steady_clock;

/// The state of a proof between two steps, as a checkpoint file holds it.
struct ProofState {
    std::uint64_t fingerprint = 0;
    std::uint32_t nargs = 0, generations = 0, steps = 0;
    std::uint64_t cnt[sid::RC_N] = {};
    std::vector<double2> boxes;          // variable-major: boxes[v * qsize + i]
    std::vector<std::uint8_t> depth;
    std::vector<double> criticals;       // stored criticals, 2*nargs doubles each
};

/// One request: a whole-lemma proof or a set of sub-boxes, with its device frontier and results.
/// The lane thread owns the device parts; `view`, `state` and the times are shared under the server lock.
struct Request {
    std::uint64_t id = 0;
    int lemma_id = -1;
    Lemma* lem = nullptr;
    int slot = -1;
    bool full = true;                    // whole lemma (root partition) or sub-boxes
    std::uint32_t part_index = 0, part_count = 0;   // whole lemma: only this part of the root partition
    const ProofState* resume = nullptr;  // continue from a checkpoint instead
    std::vector<double> boxes;           // sub-boxes, box-major (lo, hi) pairs
    std::uint64_t nboxes = 0;
    unsigned generations = 8;
    std::uint64_t crit_cap = 0;
    DevBuf<double2> qbox;
    DevBuf<std::uint8_t> qdepth;
    std::uint64_t qcap = 0;
    DevBuf<double> crit;
    std::uint64_t bytes = 0;             // device bytes held (frontier + critical store)
    sid::ReqDev view{};                  // device counters after the last step
    int state = SID_REQ_PENDING;
    bool admitted = false;
    std::string error;
    int error_status = SID_OK;           // the status a failed request reports (SID_ERR_NOMEM, SID_ERR_CUDA, ...)
    Clock::time_point t_submit, t_admit, t_done;
    std::vector<double> criticals;
};

} // namespace

struct sid_engine;

namespace sid {

constexpr std::uint64_t kLevelCapItems = std::uint64_t(8) << 20;   // items per intermediate level list
constexpr std::uint64_t kDefaultStep = std::uint64_t(1) << 16;     // queue elements per step
constexpr std::uint64_t kEscChunk = std::uint64_t(1) << 24;        // children per precision-form pass pair
constexpr std::uint64_t kHoistBytes = std::uint64_t(256) << 20;     // split-invariant values of one chunk's parents
constexpr unsigned kEscBlocksPerSM = 8;                            // grid of the escalated (double) pass
constexpr int kDefaultSlots = 1024;

struct HullArgs {
    const unsigned long long* hull_lo;
    const unsigned long long* hull_hi;
    const unsigned long long* hull_zlo;
    const unsigned long long* hull_zhi;
    const std::uint8_t* depth;          // depth of each batch element
    const std::uint32_t* tag;           // request of each batch element
    ReqDev* req;
    std::uint32_t n_elem;
    int nargs;
    // outputs: final (depth >= the request's generations) and non-final hulls
    double2* fin_box; std::uint8_t* fin_depth; std::uint32_t* fin_tag; unsigned long long* fin_count;
    double2* nf_box; std::uint8_t* nf_depth; std::uint32_t* nf_tag; unsigned long long* nf_count;
    std::uint64_t out_stride;
    // node re-iteration (cpu_prover_core.hpp:113-134): with `iterate`, a hull that should_iterate accepts
    // against its element's box (elem_box[v*elem_stride + e]) goes to the iteration list instead of being routed
    bool iterate;
    bool f32;                           // the lemma computes in float (the criteria then compare in float)
    double single, volume;              // iteration_single_dimension / iteration_volume criteria
    const double2* elem_box;
    std::uint64_t elem_stride;
    double2* it_box; std::uint8_t* it_depth; std::uint32_t* it_tag; unsigned long long* it_count;
    std::uint64_t it_stride;            // variable stride of it_box (the iteration list's capacity)
};

/// CPUProverCore::p_should_iterate (cpu_prover_core.hpp:151-177) in the lemma's number type, with the
/// reference's round-down arithmetic: re-run the static splits on the hull if some variable's hull width
/// exceeds `single` times its old width (negated widths lb - ub, rounded down), or the hull's volume exceeds
/// `volume` times the old volume (product of the negated first width and the other widths, rounded down).
template<class T> __device__ bool should_iterate(const double2* nw, const double2* old, int nargs, T single, T volume) {
    for(int i = 0; i < nargs; ++i) {
        const T mnw = Dir<T>::sub_rd(T(nw[i].x), T(nw[i].y));
        const T mow = Dir<T>::sub_rd(T(old[i].x), T(old[i].y));
        if(Dir<T>::mul_rd(mow, single) > mnw) return true;
    }
    T mnv = Dir<T>::sub_rd(T(nw[0].x), T(nw[0].y));
    T mov = Dir<T>::sub_rd(T(old[0].x), T(old[0].y));
    for(int i = 1; i < nargs; ++i) {
        mnv = Dir<T>::mul_rd(mnv, Dir<T>::sub_rd(T(nw[i].y), T(nw[i].x)));
        mov = Dir<T>::mul_rd(mov, Dir<T>::sub_rd(T(old[i].y), T(old[i].x)));
    }
    return Dir<T>::mul_rd(mov, volume) > mnv;
}

constexpr int kMaxArgs = 32;   // variables of a lemma (the IR parser rejects more)

/// Decode the per-element hull keys (AddToRange, cpu_prover_core.hpp:97-111: min of lower bounds, max
/// of upper bounds, ties kept from the first leaf in static-split order) and route each non-empty hull, or,
/// with re-iteration, list it for another pass over the static splits (counted as a repeated node and a
/// cuboid, cpu_prover_core.hpp:129-131).
__global__ void k_hull_finalize(const HullArgs h) {
    const std::uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if(e >= h.n_elem) return;
    const std::uint64_t b0 = std::uint64_t(e) * h.nargs;
    if(h.hull_lo[b0] == ~0ull) return;           // no leaf survived
    const std::uint8_t d = h.depth[e];
    const std::uint32_t t = h.tag[e];
    double2 box[kMaxArgs];
    for(int v = 0; v < h.nargs; ++v) {
        double lo = key_value(h.hull_lo[b0 + v]);
        double hi = key_value(h.hull_hi[b0 + v]);
        if(lo == 0.0) lo = (h.hull_zlo[b0 + v] & 1ull) ? -0.0 : 0.0;
        if(hi == 0.0) hi = (h.hull_zhi[b0 + v] & 1ull) ? -0.0 : 0.0;
        box[v] = make_double2(lo, hi);
    }
    if(h.iterate) {
        double2 old[kMaxArgs];
        for(int v = 0; v < h.nargs; ++v) old[v] = h.elem_box[std::uint64_t(v) * h.elem_stride + e];
        const bool again = h.f32 ? should_iterate<float>(box, old, h.nargs, float(h.single), float(h.volume))
                                 : should_iterate<double>(box, old, h.nargs, h.single, h.volume);
        if(again) {
            const unsigned long long slot = atomicAdd(h.it_count, 1ull);
            h.it_depth[slot] = d;
            h.it_tag[slot] = t;
            for(int v = 0; v < h.nargs; ++v) h.it_box[std::uint64_t(v) * h.it_stride + slot] = box[v];
            atomicAdd(&h.req[t].cnt[RC_REPEATED], 1ull);
            atomicAdd(&h.req[t].cnt[RC_CUBOIDS], 1ull);
            return;
        }
    }
    const bool fin = d >= h.req[t].generations;
    unsigned long long slot = atomicAdd(fin ? h.fin_count : h.nf_count, 1ull);
    double2* out = fin ? h.fin_box : h.nf_box;
    (fin ? h.fin_depth : h.nf_depth)[slot] = d;
    (fin ? h.fin_tag : h.nf_tag)[slot] = t;
    for(int v = 0; v < h.nargs; ++v) out[std::uint64_t(v) * h.out_stride + slot] = box[v];
}

/// Re-iteration of an element that is its own hull (a lemma without static splits): should_iterate compares
/// the element with itself on every pass, so the element runs max_iter passes if it accepts, else one.
struct RouteIteration {
    int max_iter;
    bool f32;
    double single, volume;
};

/// Lemmas without static splits: every element is itself the only leaf of its static recursion
/// (cpu_prover_core.hpp:250-256). Count it (once per pass when re-iterated) and route it by depth like
/// k_hull_finalize.
__global__ void k_route_elements(const double2* box, std::uint64_t stride, const std::uint8_t* depth,
                                 const std::uint32_t* tag, std::uint64_t n, int nargs, ReqDev* req,
                                 double2* fin_box, std::uint8_t* fin_depth, std::uint32_t* fin_tag,
                                 unsigned long long* fin_count, double2* nf_box, std::uint8_t* nf_depth,
                                 std::uint32_t* nf_tag, unsigned long long* nf_count, std::uint64_t out_stride,
                                 const RouteIteration itr) {
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const std::uint8_t d = depth[i];
    const std::uint32_t t = tag[i];
    unsigned long long passes = 1;
    if(itr.max_iter > 1) {
        double2 e[kMaxArgs];
        for(int v = 0; v < nargs; ++v) e[v] = box[std::uint64_t(v) * stride + i];
        const bool again = itr.f32 ? should_iterate<float>(e, e, nargs, float(itr.single), float(itr.volume))
                                   : should_iterate<double>(e, e, nargs, itr.single, itr.volume);
        if(again) passes = (unsigned long long)itr.max_iter;
    }
    atomicAdd(&req[t].cnt[RC_LEAVES], passes);
    if(passes > 1) {
        atomicAdd(&req[t].cnt[RC_REPEATED], passes - 1);
        atomicAdd(&req[t].cnt[RC_CUBOIDS], passes - 1);
    }
    const bool fin = d >= req[t].generations;
    const unsigned long long slot = atomicAdd(fin ? fin_count : nf_count, 1ull);
    double2* out = fin ? fin_box : nf_box;
    (fin ? fin_depth : nf_depth)[slot] = d;
    (fin ? fin_tag : nf_tag)[slot] = t;
    for(int v = 0; v < nargs; ++v) out[std::uint64_t(v) * out_stride + slot] = box[std::uint64_t(v) * stride + i];
}

/// Lemmas without static splits, final generation: every element is a leaf and a critical.
__global__ void k_store_criticals(const double2* box, std::uint64_t stride, const std::uint32_t* tag, std::uint64_t n,
                                  int nargs, ReqDev* req) {
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i >= n) return;
    ReqDev* r = req + tag[i];
    atomicAdd(&r->cnt[RC_LEAVES], 1ull);
    const unsigned long long slot = atomicAdd(&r->cnt[RC_CRITICALS], 1ull);
    if(slot >= r->crit_cap) return;
    for(int v = 0; v < nargs; ++v) {
        double2 b = box[std::uint64_t(v) * stride + i];
        r->crit[(slot * nargs + v) * 2] = b.x;
        r->crit[(slot * nargs + v) * 2 + 1] = b.y;
    }
}

/// Precision form, per-parent pass: each parent's box rounded outward to float, and for the split
/// variable RD(lb), RU(lb), RD(w), RU(w), RU(ub) with w = (ub - lb) / nsub computed in double exactly as
/// split_child does. One thread per parent, so the double work is paid once per parent, not per child.
__global__ void k_parent_f32(const double2* in_box, std::uint64_t in_stride, std::uint64_t item0, std::uint64_t n_items,
                             int nargs, int var, int nsub, float2* pbox, float4* psplit, std::uint64_t pstride,
                             unsigned long long* reset) {
    const std::uint64_t j = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(j == 0 && reset) *reset = 0;   // the chunk's escalation count, which the float pass after this kernel fills
    if(j >= n_items) return;
    for(int v = 0; v < nargs; ++v) {
        const double2 b = in_box[std::uint64_t(v) * in_stride + item0 + j];
        pbox[std::uint64_t(v) * pstride + j] = make_float2(__double2float_rd(b.x), __double2float_ru(b.y));
        if(v == var) {
            const double w = __ddiv_rd(__dsub_rd(b.y, b.x), double(nsub));
            psplit[j] = make_float4(__double2float_rd(w), __double2float_ru(b.x), __double2float_ru(w), 0.0f);
        }
    }
}

/// Quantization of the batch ordering: cell of a corner coordinate x = (float(x) - off) * scale.
struct MortonQuant {
    float off[16];
    float scale[16];     // 2^bits / (root range), so cells are 0 .. 2^bits - 1
};

constexpr int kTileLog = 18;         // ordering tile: 2^18 consecutive cuboids (~12 MB of boxes, L2-resident)
constexpr int kTileKeyBits = 16;     // Morton key bits within a tile (bits per variable = 16 / nargs, >= 1)

/// Batch ordering (sid_eval_batch*), step 1: bucket of each cuboid = (its tile, Morton code of its lower
/// corner quantized over the lemma's root box; in float: only the cell matters), and the histogram.
__global__ void k_order_keys(const double* lo, std::uint64_t n, std::uint64_t stride, int nargs, const MortonQuant qp,
                             int bits, std::uint32_t* key, std::uint32_t* count) {
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i >= n) return;
    std::uint32_t k = 0;
    std::uint32_t q[16];
    const float top = float((1u << bits) - 1u);
    for(int v = 0; v < nargs; ++v) {
        float u = (__double2float_rn(lo[std::uint64_t(v) * stride + i]) - qp.off[v]) * qp.scale[v];
        u = u > 0.0f ? (u < top ? u : top) : 0.0f;   // NaN and out-of-box corners are clamped
        q[v] = std::uint32_t(u);
    }
    for(int b = bits - 1; b >= 0; --b) {
        for(int v = nargs - 1; v >= 0; --v) k = (k << 1) | ((q[v] >> b) & 1u);
    }
    k |= std::uint32_t(i >> kTileLog) << kTileKeyBits;
    key[i] = k;
    atomicAdd(&count[k], 1u);
}

/// Exclusive scan of `x` (n <= 2^24 entries) in place, in three launches: per-block scans of 4096
/// entries with block totals, a one-block scan of the totals, and the addition of block offsets.
__global__ void __launch_bounds__(1024) k_scan_blocks(std::uint32_t* x, std::uint64_t n, std::uint32_t* totals) {
    __shared__ std::uint32_t warp_sums[32];
    const std::uint64_t base = std::uint64_t(blockIdx.x) * 4096 + std::uint64_t(threadIdx.x) * 4;
    std::uint32_t v[4];
    std::uint32_t sum = 0;
    for(int k = 0; k < 4; ++k) {
        v[k] = base + k < n ? x[base + k] : 0u;
        sum += v[k];
    }
    std::uint32_t incl = sum;
    for(int d = 1; d < 32; d <<= 1) {
        const std::uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
        if(int(threadIdx.x & 31u) >= d) incl += y;
    }
    if((threadIdx.x & 31u) == 31u) warp_sums[threadIdx.x >> 5] = incl;
    __syncthreads();
    if(threadIdx.x < 32) {
        std::uint32_t w = warp_sums[threadIdx.x];
        for(int d = 1; d < 32; d <<= 1) {
            const std::uint32_t y = __shfl_up_sync(0xffffffffu, w, d);
            if(int(threadIdx.x) >= d) w += y;
        }
        warp_sums[threadIdx.x] = w;
    }
    __syncthreads();
    const std::uint32_t warp_off = (threadIdx.x >> 5) ? warp_sums[(threadIdx.x >> 5) - 1] : 0u;
    std::uint32_t run = warp_off + incl - sum;
    for(int k = 0; k < 4; ++k) {
        if(base + k < n) x[base + k] = run;
        run += v[k];
    }
    if(threadIdx.x == blockDim.x - 1) totals[blockIdx.x] = warp_off + incl;
}

__global__ void k_scan_add(std::uint32_t* x, std::uint64_t n, const std::uint32_t* offsets) {
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i < n) x[i] += offsets[i / 4096];
}

/// Step 3: place each cuboid at the next free position of its bucket. The order within a bucket is
/// immaterial (every cuboid's result is independent of its neighbours), and a cuboid never leaves its tile.
__global__ void k_order_scatter(const std::uint32_t* key, std::uint64_t n, std::uint32_t* offset, std::uint32_t* order) {
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i >= n) return;
    order[atomicAdd(&offset[key[i]], 1u)] = std::uint32_t(i);
}


struct GatherEntry {
    std::uint32_t slot;
    std::uint32_t pad;
    unsigned long long begin, count, dst;
};

/// Copy the elements [begin, begin + count) of each entry's request queue to the step batch at dst, and
/// pop them (the request's queue size becomes begin; its children are appended from there).
__global__ void k_gather(const GatherEntry* ent, int n_ent, unsigned long long total, ReqDev* req, int nargs,
                         double2* dst_box, std::uint64_t dst_stride, std::uint8_t* dst_depth, std::uint32_t* dst_tag) {
    const unsigned long long i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i >= total) return;
    int lo = 0, hi = n_ent - 1;                  // last entry with dst <= i
    while(lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if(ent[mid].dst <= i) lo = mid; else hi = mid - 1;
    }
    const GatherEntry g = ent[lo];
    const ReqDev* r = req + g.slot;
    const unsigned long long src = g.begin + (i - g.dst);
    for(int v = 0; v < nargs; ++v) dst_box[std::uint64_t(v) * dst_stride + i] = r->qbox[std::uint64_t(v) * r->qcap + src];
    dst_depth[i] = r->qdepth[src];
    dst_tag[i] = g.slot;
    if(i == g.dst) req[g.slot].cnt[RC_QSIZE] = g.begin;
}

/// Lane: the scratch of one lemma and the device table of the requests it serves. Not thread-safe:
/// one host thread drives a lane.
struct Lane {
    sid_engine* eng = nullptr;
    Lemma* lem = nullptr;
    int n = 0;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::vector<IrSplit> dyn, stat;
    std::uint64_t step_cap = kDefaultStep;
    bool fp32_first = false;
    std::uint32_t fp32_mask = ~0u;         // levels (dynamic d, static D + j) that use the float pass
    std::uint32_t noprop_mask = 0;         // float-pass levels without bound propagation (split-invariant form)
    std::uint32_t root_part_index = 0, root_part_count = 0;   // the root partition being admitted (sharding)
    int max_iter = 1;                      // node re-iteration (max_iterations_per_node; <= 1: none)
    double iter_single = 0.66, iter_volume = 0.25;
    BoxList iter_in, iter_out;             // elements re-run on their hulls (re-iteration)
    std::uint64_t fanout = 1, root_fanout = 1;
    int sm_count = 1;
    int max_slots = kDefaultSlots;
    DevBuf<ReqDev> req_dev;
    std::vector<ReqDev> req_host;          // host copy of the table (counters as of the last read)
    std::vector<Request*> slot_req;
    DevBuf<unsigned long long> counters;   // [0] out_count [1] fin [2] nf [3] escalation list length [4] re-iterated
    DevBuf<unsigned int> overflow;
    DevBuf<unsigned long long> hull;       // 4 * step_cap * nargs
    BoxList step, fin, nonfin;
    std::vector<std::unique_ptr<BoxList>> stat_levels, dyn_levels;
    DevBuf<std::uint32_t> esc;
    DevBuf<float2> pbox;                  // precision form: per-parent float boxes of one chunk
    DevBuf<float4> psplit;
    DevBuf<float2> hval;                  // split-invariant float pass: stored values per parent of one chunk
    DevBuf<std::uint64_t> hbits;
    DevBuf<GatherEntry> gather;
    std::vector<GatherEntry> gather_host;
    long long grown_bytes = 0;             // device bytes request queues grew by since the last take_grown_bytes
    DevBuf<unsigned long long> level_esc;  // escalated children per level (float pass), for tuning
    std::vector<unsigned long long> level_children;

    Lane(sid_engine* e, Lemma* l, cudaStream_t s, bool own, int sms, int slots)
        : eng(e), lem(l), st(s), own_stream(own), sm_count(sms), max_slots(slots) {
        n = l->ir.nargs;
        dyn = l->ir.dynamic_splits();
        stat = l->ir.static_splits();
        for(const auto& sp : dyn) {
            fanout *= std::uint64_t(sp.subdivisions);
            root_fanout *= std::uint64_t(sp.initial);
        }
        req_host.assign(std::size_t(max_slots), ReqDev{});
        slot_req.assign(std::size_t(max_slots), nullptr);
        req_dev.reserve(std::size_t(max_slots));
        cuda_check(cudaMemsetAsync(req_dev.p, 0, sizeof(ReqDev) * std::size_t(max_slots), st), "request table");
        counters.reserve(8);
        overflow.reserve(1);
        cuda_check(cudaMemsetAsync(overflow.p, 0, sizeof(unsigned int), st), "overflow flag");
    }
    Lane(const Lane&) = delete;
    Lane& operator=(const Lane&) = delete;
    ~Lane() {
        if(st) cudaStreamSynchronize(st);
        if(stage) cudaFreeHost(stage);
        if(slots_pinned) cudaFreeHost(slots_pinned);
        if(own_stream && st) cudaStreamDestroy(st);
    }

    /// Pinned host copies of the device loop's small transfers (its request slot going in, its control words and
    /// counters coming back), so that they are asynchronous and share one wait.
    struct LoopStage {
        ReqDev in, out;
        LoopCtl ctl;
        unsigned long long words[8];     // counters read back between levels (read_counters)
    };
    LoopStage* stage = nullptr;
    LoopStage& loop_stage() {
        if(!stage) {
            void* p = nullptr;
            cuda_check(cudaMallocHost(&p, sizeof(LoopStage)), "pinned loop staging");
            stage = static_cast<LoopStage*>(p);
        }
        return *stage;
    }

    /// Node re-iteration settings (ProverSettings::max_iterations_per_node and the two criteria).
    void set_iteration(int max_iterations, float volume, float single) {
        max_iter = max_iterations;
        iter_volume = double(volume);
        iter_single = double(single);
        if(max_iter > 1) {
            iter_in.reserve(n, std::max(iter_in.cap, step_cap), false, false, true, true);
            iter_out.reserve(n, std::max(iter_out.cap, step_cap), false, false, true, true);
        }
    }

    void configure(std::uint64_t step_elements, bool fp32, std::uint32_t mask = ~0u, std::uint32_t noprop = 0) {
        step_cap = step_elements > 0 ? step_elements : kDefaultStep;
        fp32_first = fp32 && lem->k->filter_f32 != nullptr;
        fp32_mask = mask;
        noprop_mask = noprop;
        level_esc.reserve(SID_MAX_LEVELS);
        cuda_check(cudaMemsetAsync(level_esc.p, 0, SID_MAX_LEVELS * sizeof(unsigned long long), st), "level stats");
        level_children.assign(SID_MAX_LEVELS, 0);
        hull.reserve(4 * step_cap * std::uint64_t(n));
        step.reserve(n, std::max(step.cap, step_cap), false, false, true, true);
        fin.reserve(n, std::max(fin.cap, step_cap), false, false, true, true);
        nonfin.reserve(n, std::max(nonfin.cap, step_cap), false, false, true, true);
        if(fp32_first) esc.reserve(kEscChunk);
    }

    long long take_grown_bytes() {
        long long d = grown_bytes;
        grown_bytes = 0;
        return d;
    }

    const ReqDev& counters_of(const Request* r) const { return req_host[std::size_t(r->slot)]; }
    std::uint64_t queue_size(const Request* r) const { return counters_of(r).cnt[RC_QSIZE]; }

    /// Read k adjacent device counters (one copy into pinned memory, one wait).
    const unsigned long long* read_counters(const unsigned long long* d, int k) {
        LoopStage& sg = loop_stage();
        cuda_check(cudaMemcpyAsync(sg.words, d, sizeof(unsigned long long) * std::size_t(k), cudaMemcpyDeviceToHost, st),
                   "read counter");
        cuda_check(cudaStreamSynchronize(st), "stream sync");
        return sg.words;
    }
    unsigned long long read_counter(const unsigned long long* d) { return read_counters(d, 1)[0]; }
    void zero_counter(unsigned long long* d) {
        cuda_check(cudaMemsetAsync(d, 0, sizeof(unsigned long long), st), "reset counter");
    }

    int free_slots() const {
        int k = 0;
        for(auto* r : slot_req) k += r ? 0 : 1;
        return k;
    }

    std::uint64_t initial_queue_cap(const Request& r) const {
        if(r.resume) return std::max<std::uint64_t>(r.resume->cnt[RC_QSIZE], 64);
        return std::max<std::uint64_t>(r.full ? root_fanout : r.nboxes, 64);
    }
    /// Device bytes a request holds right after admission.
    std::uint64_t initial_bytes(const Request& r) const {
        return plan::request_bytes(n, initial_queue_cap(r), std::max<std::uint64_t>(r.crit_cap, 1));
    }

    /// Write the queue pointers and capacity of a slot without touching its device counters.
    void patch_queue(int slot) {
        const ReqDev& h = req_host[std::size_t(slot)];
        char* dst = reinterpret_cast<char*>(req_dev.p + slot) + offsetof(ReqDev, qbox);
        const char* src = reinterpret_cast<const char*>(&h) + offsetof(ReqDev, qbox);
        cuda_check(cudaMemcpyAsync(dst, src, offsetof(ReqDev, crit) - offsetof(ReqDev, qbox), cudaMemcpyHostToDevice, st),
                   "request queue patch");
        cuda_check(cudaStreamSynchronize(st), "request queue patch");
    }

    /// Admit a request: device slot, frontier queue, critical store; then its root partition (whole
    /// lemma; left to the device proof loop with root_on_device) or its sub-boxes as depth-0 elements.
    void admit(Request* r, bool root_on_device = false) {
        int slot = -1;
        for(int i = 0; i < max_slots; ++i) {
            if(!slot_req[std::size_t(i)]) { slot = i; break; }
        }
        if(slot < 0) fail(SID_ERR_CAPACITY, "no free request slot");
        r->slot = slot;
        slot_req[std::size_t(slot)] = r;
        double2* qbox = nullptr;
        std::uint8_t* qdepth = nullptr;
        if(root_on_device) {
            // the device loop's queue belongs to the lane and is reused by its proofs
            r->qcap = loop_queue_cap();
            if(loop_qcap < r->qcap) {
                loop_qbox.release();
                loop_qdepth.release();
                loop_qcap = 0;
                loop_qbox.reserve(std::size_t(n) * r->qcap);
                loop_qdepth.reserve(r->qcap);
                loop_qcap = r->qcap;
            }
            r->qcap = loop_qcap;
            qbox = loop_qbox.p;
            qdepth = loop_qdepth.p;
        } else {
            r->qcap = initial_queue_cap(*r);
            r->qbox.reserve_on(std::size_t(n) * r->qcap, st);
            r->qdepth.reserve_on(r->qcap, st);
            qbox = r->qbox.p;
            qdepth = r->qdepth.p;
        }
        r->crit.reserve_on(std::max<std::uint64_t>(r->crit_cap, 1) * 2 * std::uint64_t(n), st);
        r->bytes = initial_bytes(*r);
        ReqDev& h = req_host[std::size_t(slot)];
        h = ReqDev{};
        h.qbox = qbox;
        h.qdepth = qdepth;
        h.qcap = r->qcap;
        h.crit = r->crit.p;
        h.crit_cap = r->crit_cap;
        h.generations = r->generations;
        if(r->resume) {
            const ProofState& ps = *r->resume;
            const std::uint64_t q = ps.cnt[RC_QSIZE];
            std::memcpy(h.cnt, ps.cnt, sizeof(h.cnt));
            for(int v = 0; v < n; ++v) {
                cuda_check(cudaMemcpyAsync(r->qbox.p + std::uint64_t(v) * r->qcap, ps.boxes.data() + std::uint64_t(v) * q,
                                           q * sizeof(double2), cudaMemcpyHostToDevice, st), "resume upload");
            }
            cuda_check(cudaMemcpyAsync(r->qdepth.p, ps.depth.data(), std::size_t(q), cudaMemcpyHostToDevice, st), "resume upload");
            const std::size_t keep = std::min(ps.criticals.size(), std::size_t(r->crit_cap) * 2 * std::size_t(n));
            if(keep) {
                cuda_check(cudaMemcpyAsync(r->crit.p, ps.criticals.data(), keep * sizeof(double), cudaMemcpyHostToDevice, st),
                           "resume upload");
            }
            cuda_check(cudaStreamSynchronize(st), "resume upload");
        } else if(!r->full) {
            h.cnt[RC_QSIZE] = r->nboxes;
            h.cnt[RC_CUBOIDS] = r->nboxes;
            std::vector<double2> col(std::size_t(r->nboxes));
            for(int v = 0; v < n; ++v) {
                for(std::uint64_t b = 0; b < r->nboxes; ++b) {
                    const std::size_t k = std::size_t(2 * (b * std::uint64_t(n) + std::uint64_t(v)));
                    col[std::size_t(b)] = make_double2(r->boxes[k], r->boxes[k + 1]);
                }
                cuda_check(cudaMemcpyAsync(r->qbox.p + std::uint64_t(v) * r->qcap, col.data(),
                                           col.size() * sizeof(double2), cudaMemcpyHostToDevice, st), "sub-box upload");
                cuda_check(cudaStreamSynchronize(st), "sub-box upload");
            }
            cuda_check(cudaMemsetAsync(r->qdepth.p, 0, std::size_t(r->nboxes), st), "sub-box depth");
        }
        if(root_on_device) {
            // the loop's own read-back gives the counts; no wait here (the staging copy is pinned, and the loop's
            // read-back waits for the stream before the stage is written again)
            LoopStage& sg = loop_stage();
            sg.in = h;
            cuda_check(cudaMemcpyAsync(req_dev.p + slot, &sg.in, sizeof(ReqDev), cudaMemcpyHostToDevice, st), "request slot");
            return;
        }
        LoopStage& sg = loop_stage();   // pinned; the wait below ends the copy before the stage is written again
        sg.in = h;
        cuda_check(cudaMemcpyAsync(req_dev.p + slot, &sg.in, sizeof(ReqDev), cudaMemcpyHostToDevice, st), "request slot");
        cuda_check(cudaStreamSynchronize(st), "request slot");
        if(r->full && !r->resume && !root_on_device) {
            root_part_index = r->part_index;
            root_part_count = r->part_count;
            run_dynamic(0, lem->root.p, 1, nullptr, nullptr, std::uint32_t(slot), 0, 1, true, 0);
            root_part_index = root_part_count = 0;
        }
        read_slots();
    }

    // device proof loop: control words, a queue reused by its proofs, per-block scratch (cached, grown as needed)
    DevBuf<LoopCtl> loop_ctl;
    DevBuf<double2> loop_qbox;
    DevBuf<std::uint8_t> loop_qdepth;
    std::uint64_t loop_qcap = 0;
    DevBuf<double2> lb_sbox[kLoopMaxLevels], lb_dbox[kLoopMaxLevels], lb_hull;
    DevBuf<std::uint32_t> lb_selem[kLoopMaxLevels], lb_esc;
    DevBuf<std::uint64_t> lb_spath[kLoopMaxLevels];
    DevBuf<std::uint8_t> lb_ddepth[kLoopMaxLevels];
    DevBuf<float2> lb_pbox;
    DevBuf<float4> lb_psplit;
    DevBuf<unsigned long long> lb_ctl;
    DevBuf<std::uint8_t> lb_hull_depth;
    static constexpr int kLoopGroupMax = 128;                   // elements a block takes at once, at most

    static constexpr std::uint64_t kBlockListItems = 2048;       // items of one per-block list
    static constexpr std::uint64_t kBlockEscChildren = 1 << 14;  // children per float-pass chunk of a block
    static constexpr std::uint64_t kLoopQueueBytes = std::uint64_t(1) << 30;   // most the loop's queue may hold

    /// Queue capacity for a device-loop proof: the root partition and one full step's children, twice over,
    /// within kLoopQueueBytes.
    std::uint64_t loop_queue_cap() const {
        const std::uint64_t per = 16 * std::uint64_t(n) + 1;
        const std::uint64_t want = 2 * std::max<std::uint64_t>(root_fanout, step_cap * fanout);
        return std::max<std::uint64_t>(64, std::min(want, kLoopQueueBytes / per));
    }

    /// Loop arguments for a whole-lemma request admitted with root_on_device (its queue is the lane's loop queue), on a
    /// grid of G blocks: the root partition's lists and the per-block scratch sized for G, control words zeroed on the
    /// lane's stream. la.sync is this lane's own control word (a bundle points it to its shared one).
    void prepare_loop(Request* r, unsigned G, LoopArgs& la) {
        const int D = int(dyn.size()), S = int(stat.size());
        if(D < 1 || D > kLoopMaxLevels || S > kLoopMaxLevels) fail(SID_ERR_UNSUPPORTED, "device loop: too many levels");
        la = LoopArgs{};
        la.req = req_dev.p;
        la.tag = std::uint32_t(r->slot);
        la.nargs = n;
        la.n_dyn = D;
        la.n_stat = S;
        for(int d = 0; d < D; ++d) {
            la.dyn[d] = LoopSplit{dyn[std::size_t(d)].arg, int(dyn[std::size_t(d)].initial), int(dyn[std::size_t(d)].subdivisions)};
        }
        for(int j = 0; j < S; ++j) la.stat[j] = LoopSplit{stat[std::size_t(j)].arg, 0, int(stat[std::size_t(j)].subdivisions)};
        la.root = lem->root.p;
        la.part_index = r->part_index;
        la.part_count = r->part_count;
        la.fp32 = fp32_first;
        la.fp32_mask = fp32_mask;
        la.step = step_cap;
        la.max_steps = std::uint64_t(1) << 40;
        la.step_box = step.box.p;
        la.step_depth = step.depth.p;
        la.step_tag = step.tag.p;
        la.step_cap = step_cap;
        la.hull = hull.p;
        // root partition lists (grid-wide): the initial subdivisions' products
        std::uint64_t root_items = 1, p_cap = 1;
        for(int d = 1; d < D; ++d) {
            root_items *= std::uint64_t(dyn[std::size_t(d - 1)].initial);
            BoxList& l = dyn_level(std::size_t(d));
            l.reserve(n, std::max(l.cap, root_items), false, false, true, true);
            la.dl_box[d] = l.box.p; la.dl_depth[d] = l.depth.p; la.dl_tag[d] = l.tag.p; la.dl_cap[d] = l.cap;
            p_cap = std::max(p_cap, l.cap);
        }
        // elements a block takes at once: enough for about one child per thread on the first static level (or the
        // re-split's first level); the per-block lists of their levels
        const int nsub0 = S > 0 ? int(stat[0].subdivisions) : int(dyn[0].subdivisions);
        la.group_max = std::uint32_t(std::max(1, std::min(kLoopGroupMax, 128 / std::max(nsub0, 1))));
        std::uint64_t bp_cap = 1, items = la.group_max;
        for(int j = 1; j < S; ++j) {
            items = std::min(items * std::uint64_t(stat[std::size_t(j - 1)].subdivisions), kBlockListItems);
            lb_sbox[j].reserve(std::size_t(G) * items * std::uint64_t(n));
            lb_selem[j].reserve(std::size_t(G) * items);
            lb_spath[j].reserve(std::size_t(G) * items);
            la.bs_box[j] = lb_sbox[j].p; la.bs_elem[j] = lb_selem[j].p; la.bs_path[j] = lb_spath[j].p; la.bs_cap[j] = items;
            bp_cap = std::max(bp_cap, items);
        }
        items = la.group_max;
        for(int d = 1; d < D; ++d) {
            items = std::min(items * std::uint64_t(dyn[std::size_t(d - 1)].subdivisions), kBlockListItems);
            lb_dbox[d].reserve(std::size_t(G) * items * std::uint64_t(n));
            lb_ddepth[d].reserve(std::size_t(G) * items);
            la.bd_box[d] = lb_dbox[d].p; la.bd_depth[d] = lb_ddepth[d].p; la.bd_cap[d] = items;
            bp_cap = std::max(bp_cap, items);
        }
        lb_hull.reserve(std::size_t(G) * 2 * la.group_max * std::uint64_t(n));
        lb_hull_depth.reserve(std::size_t(G) * 2 * la.group_max);
        lb_ctl.reserve(std::size_t(G) * kBlockCtlWords);
        la.b_hull_box = lb_hull.p;
        la.b_hull_depth = lb_hull_depth.p;
        la.b_ctl = lb_ctl.p;
        if(fp32_first) {
            esc.reserve(kEscChunk);
            pbox.reserve(std::size_t(n) * p_cap);
            psplit.reserve(std::size_t(p_cap));
            la.esc = esc.p; la.esc_cap = kEscChunk; la.pbox = pbox.p; la.psplit = psplit.p; la.p_cap = p_cap;
            lb_pbox.reserve(std::size_t(G) * bp_cap * std::uint64_t(n));
            lb_psplit.reserve(std::size_t(G) * bp_cap);
            lb_esc.reserve(std::size_t(G) * kBlockEscChildren);
            la.b_pbox = lb_pbox.p; la.b_psplit = lb_psplit.p; la.b_p_cap = bp_cap;
            la.b_esc = lb_esc.p; la.b_esc_cap = kBlockEscChildren;
        }
        loop_ctl.reserve(1);
        cuda_check(cudaMemsetAsync(loop_ctl.p, 0, sizeof(LoopCtl), st), "loop control");
        la.ctl = loop_ctl.p;
        la.sync = loop_ctl.p;
    }

    /// After a loop kernel: this proof's control words and counters, read back on the lane's stream (which the
    /// kernel ran on, or which waits for it). Returns false if the proof's queue or a list would have overflowed
    /// (its counts are then incomplete; the caller redoes the proof on the host-driven loop).
    bool finish_loop(Request* r) {
        LoopStage& sg = loop_stage();
        cuda_check(cudaMemcpyAsync(&sg.ctl, loop_ctl.p, sizeof(LoopCtl), cudaMemcpyDeviceToHost, st), "loop control");
        cuda_check(cudaMemcpyAsync(&sg.out, req_dev.p + r->slot, sizeof(ReqDev), cudaMemcpyDeviceToHost, st), "request");
        cuda_check(cudaStreamSynchronize(st), "device proof loop");
        const LoopCtl c = sg.ctl;
        const ReqDev h = sg.out;
        if(c.error == kLoopTimeout) fail(SID_ERR_TIMEOUT, "device proof loop: a grid barrier gave up");
        // an append that did not fit is counted, not written
        if(c.error != kLoopOk || c.overflow != 0 || h.cnt[RC_OVERFLOW] != 0 || h.cnt[RC_QSIZE] != 0) return false;
        std::memcpy(req_host[std::size_t(r->slot)].cnt, h.cnt, sizeof(h.cnt));
        loop_steps = std::uint32_t(c.steps);
        return true;
    }

    /// A whole-lemma request admitted with root_on_device, proved entirely in the device proof loop
    /// (proof_loop.cuh) on `blocks` co-resident blocks (clamped to the device's limit for the kernel). Returns false
    /// if the queue or a list would have overflowed; throws SID_ERR_TIMEOUT if a barrier gave up.
    bool run_device_loop(Request* r, unsigned blocks) {
        const int occ = lem->k->proof_loop_occupancy ? lem->k->proof_loop_occupancy() : 0;
        if(occ <= 0) fail(SID_ERR_UNSUPPORTED, "device loop: the kernel cannot be resident");
        const unsigned G = std::max(1u, std::min(blocks, unsigned(occ) * unsigned(std::max(sm_count, 1))));
        LoopArgs la;
        prepare_loop(r, G, la);
        launch_gate("device proof loop");
        cuda_check(lem->k->proof_loop(la, G, st), "device proof loop launch");
        return finish_loop(r);
    }
    std::uint32_t loop_steps = 0;

    /// Drop a request's device state (after completion or failure).
    void release(Request* r) {
        if(r->slot < 0) return;
        cuda_check(cudaStreamSynchronize(st), "release sync");
        slot_req[std::size_t(r->slot)] = nullptr;
        req_host[std::size_t(r->slot)] = ReqDev{};
        r->slot = -1;
        r->qbox.release();
        r->qdepth.release();
        r->crit.release();
    }

    /// Copy the counters of the used slots from the device table; checks the overflow flags.
    /// Pinned host copy of the request table and the list-overflow flag, read back after every step.
    ReqDev* slots_pinned = nullptr;
    unsigned int* ovf_pinned = nullptr;

    void read_slots() {
        int hi = 0;
        for(int i = 0; i < max_slots; ++i) if(slot_req[std::size_t(i)]) hi = i + 1;
        if(!slots_pinned) {
            void* p = nullptr;
            cuda_check(cudaMallocHost(&p, sizeof(ReqDev) * std::size_t(max_slots) + sizeof(ReqDev)), "pinned request table");
            slots_pinned = static_cast<ReqDev*>(p);
            ovf_pinned = reinterpret_cast<unsigned int*>(slots_pinned + max_slots);
        }
        const ReqDev* tmp = slots_pinned;
        if(hi > 0) {
            cuda_check(cudaMemcpyAsync(slots_pinned, req_dev.p, sizeof(ReqDev) * std::size_t(hi), cudaMemcpyDeviceToHost, st),
                       "request table");
        }
        cuda_check(cudaMemcpyAsync(ovf_pinned, overflow.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, st), "overflow flag");
        cuda_check(cudaStreamSynchronize(st), "request table sync");
        if(*ovf_pinned) fail(SID_ERR_CUDA, "internal error: a level list overflowed");
        for(int i = 0; i < hi; ++i) {
            if(!slot_req[std::size_t(i)]) continue;
            std::memcpy(req_host[std::size_t(i)].cnt, tmp[std::size_t(i)].cnt, sizeof(tmp[0].cnt));
            if(tmp[std::size_t(i)].cnt[RC_OVERFLOW]) fail(SID_ERR_CUDA, "internal error: a request queue overflowed");
        }
    }

    /// The request's state between steps: counters, frontier queue, stored criticals.
    void snapshot(Request* r, ProofState& ps) {
        const ReqDev& c = counters_of(r);
        std::memcpy(ps.cnt, c.cnt, sizeof(ps.cnt));
        const std::uint64_t q = c.cnt[RC_QSIZE];
        ps.nargs = std::uint32_t(n);
        ps.boxes.resize(std::size_t(q * std::uint64_t(n)));
        ps.depth.resize(std::size_t(q));
        for(int v = 0; v < n; ++v) {
            cuda_check(cudaMemcpyAsync(ps.boxes.data() + std::uint64_t(v) * q, r->qbox.p + std::uint64_t(v) * r->qcap,
                                       q * sizeof(double2), cudaMemcpyDeviceToHost, st), "checkpoint copy");
        }
        cuda_check(cudaMemcpyAsync(ps.depth.data(), r->qdepth.p, std::size_t(q), cudaMemcpyDeviceToHost, st), "checkpoint copy");
        const std::uint64_t k = std::min<std::uint64_t>(c.cnt[RC_CRITICALS], r->crit_cap);
        ps.criticals.resize(std::size_t(k * 2 * std::uint64_t(n)));
        if(k) {
            cuda_check(cudaMemcpyAsync(ps.criticals.data(), r->crit.p, ps.criticals.size() * sizeof(double),
                                       cudaMemcpyDeviceToHost, st), "checkpoint copy");
        }
        cuda_check(cudaStreamSynchronize(st), "checkpoint copy");
    }

    /// Critical boxes stored for a request (after it finished).
    void fetch_criticals(Request* r) {
        const std::uint64_t k = std::min<std::uint64_t>(counters_of(r).cnt[RC_CRITICALS], r->crit_cap);
        r->criticals.assign(std::size_t(k * 2 * std::uint64_t(n)), 0.0);
        if(k) {
            cuda_check(cudaMemcpyAsync(r->criticals.data(), r->crit.p, r->criticals.size() * sizeof(double),
                                       cudaMemcpyDeviceToHost, st), "copy criticals");
            cuda_check(cudaStreamSynchronize(st), "copy criticals");
        }
    }

    LevelArgs base_args() {
        LevelArgs a{};
        a.req = req_dev.p;
        a.overflow = overflow.p;
        a.out_count = counters.p;
        return a;
    }

    /// Per-level escalation counts since configure(): (children, escalated) per level.
    std::vector<std::pair<unsigned long long, unsigned long long>> level_stats() {
        std::vector<unsigned long long> esc_h(SID_MAX_LEVELS, 0);
        cuda_check(cudaMemcpyAsync(esc_h.data(), level_esc.p, SID_MAX_LEVELS * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, st), "level stats");
        cuda_check(cudaStreamSynchronize(st), "level stats");
        std::vector<std::pair<unsigned long long, unsigned long long>> out;
        for(int l = 0; l < SID_MAX_LEVELS; ++l) out.emplace_back(level_children[std::size_t(l)], esc_h[std::size_t(l)]);
        return out;
    }

    void launch(int mode, const LevelArgs& a0, int level) {
        const std::uint64_t total = a0.n_in * std::uint64_t(a0.nsub);
        if(total == 0) return;
        launch_gate("level kernel launch");
        // the root's first split of a sharded proof runs the dense kernel, which applies the part filter
        const bool level_fp32 = fp32_first && level < SID_MAX_LEVELS && ((fp32_mask >> level) & 1u) && a0.part_count <= 1;
        if(level_fp32) level_children[std::size_t(level)] += total;
        if(!level_fp32) {
            LevelArgs a = a0;
            a.count_cuboids = true;
            a.float_rows = fp32_first;   // precision form, level without the float pass: float-first rows
            a.lane_shift = lane_shift_for(total, std::uint64_t(std::max(sm_count, 1)) * 128u);
            cuda_check(lem->k->level(mode, a, st), "level kernel launch");
            return;
        }
        // precision form: per-parent float data, float pass over a chunk of children, then double pass over
        // the chunk's escalation list. Without propagation, where the lemma has a split-invariant form of the
        // level, the float pass runs in two kernels: once per parent (k_prelude_f32), then per child.
        const bool noprop = ((noprop_mask >> level) & 1u) != 0;
        const int nval = noprop && lem->k->hoist_values ? lem->k->hoist_values(level) : -1;
        std::uint64_t chunk = kEscChunk;
        if(nval > 0) {   // keep the stored values of a chunk's parents within kHoistBytes
            const std::uint64_t parents = std::max<std::uint64_t>(1, kHoistBytes / (sizeof(float2) * std::uint64_t(nval)));
            chunk = std::min(kEscChunk, std::max<std::uint64_t>(1, parents - 1) * std::uint64_t(a0.nsub));
        }
        for(std::uint64_t cb = 0; cb < total; cb += chunk) {
            LevelArgs a = a0;
            a.count_cuboids = false;
            a.fp32_noprop = noprop;
            a.child_begin = cb;
            a.n_child = std::min(chunk, total - cb);
            a.esc = esc.p;
            a.esc_count = counters.p + 3;
            const std::uint64_t nsub = std::uint64_t(a.nsub);
            const std::uint64_t first = cb / nsub, n_items = (cb + a.n_child - 1) / nsub - first + 1;
            pbox.reserve(std::size_t(n) * n_items);
            psplit.reserve(n_items);
            k_parent_f32<<<unsigned((n_items + 127) / 128), 128, 0, st>>>(a.in_box, a.in_stride, a.in_begin + first,
                                                                          n_items, n, a.var, a.nsub, pbox.p, psplit.p,
                                                                          n_items, a.esc_count);
            cuda_check(cudaGetLastError(), "parent pass launch");
            a.pbox = pbox.p;
            a.psplit = psplit.p;
            a.pstride = n_items;
            a.pitem_begin = first;
            if(nval >= 0) {
                hval.reserve(std::size_t(std::max(nval, 1)) * n_items);
                hbits.reserve(n_items);
                cuda_check(lem->k->prelude_f32(level, a, n_items, hval.p, hbits.p, st), "parent float pass launch");
                a.hval = hval.p;
                a.hbits = hbits.p;
                cuda_check(lem->k->filter_hoisted(level, a, st), "float pass launch");
            } else {
                cuda_check(lem->k->filter_f32(a, st), "float pass launch");
            }
            a.esc_stat = level_esc.p + level;   // the double pass adds the chunk's escalations to the level's count
            const std::uint64_t want = (a.n_child + 127) / 128;
            const unsigned blocks = unsigned(std::min<std::uint64_t>(want, std::uint64_t(sm_count) * kEscBlocksPerSM));
            cuda_check(lem->k->level_esc(mode, a, blocks, st), "escalated pass launch");
        }
    }

    BoxList& stat_level(std::size_t j) {
        while(stat_levels.size() <= j) stat_levels.emplace_back(new BoxList);
        return *stat_levels[j];
    }
    BoxList& dyn_level(std::size_t j) {
        while(dyn_levels.size() <= j) dyn_levels.emplace_back(new BoxList);
        return *dyn_levels[j];
    }

    /// Dynamic levels d.. (root partition or re-split); the last one appends to the requests' queues.
    void run_dynamic(std::size_t d, const double2* in_box, std::uint64_t in_stride, const std::uint8_t* in_depth,
                     const std::uint32_t* in_tag, std::uint32_t tag_value, std::uint8_t depth_value, std::uint64_t n_in,
                     bool initial, std::uint8_t depth_add) {
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
            out->reserve(n, std::max(out->cap, cap), false, false, true, true);
            chunk = std::max<std::uint64_t>(1, out->cap / std::uint64_t(nsub));
        }
        for(std::uint64_t off = 0; off < n_in; off += chunk) {
            const std::uint64_t len = std::min(chunk, n_in - off);
            LevelArgs a = base_args();
            a.in_box = in_box;
            a.in_stride = in_stride;
            a.in_depth = in_depth;
            a.in_tag = in_tag;
            a.tag_value = tag_value;
            a.depth_value = depth_value;
            a.in_begin = off;
            a.n_in = len;
            a.var = sp.arg;
            a.nsub = nsub;
            a.it_limit = it_limit;
            a.rec_limit = rec_limit;
            if(d == 0 && initial) {
                a.part_index = root_part_index;
                a.part_count = root_part_count;
            }
            if(last) {
                a.row_begin = n - 1;
                a.row_end = n;
                a.depth_add = depth_add;
                launch(MODE_QUEUE, a, int(d));
            } else {
                a.row_begin = a.row_end = 0;
                a.out_box = out->box.p;
                a.out_stride = out->cap;
                a.out_cap = out->cap;
                a.out_depth = out->depth.p;
                a.out_tag = out->tag.p;
                zero_counter(counters.p);
                launch(MODE_EMIT, a, int(d));
                std::uint64_t cnt = read_counter(counters.p);
                run_dynamic(d + 1, out->box.p, out->cap, out->depth.p, out->tag.p, 0, 0, cnt, initial, depth_add);
            }
        }
    }

    /// Static levels j.. over items; innermost level joins hulls (MODE_HULL) or stores criticals (MODE_CRIT).
    void run_static(std::size_t j, const double2* in_box, std::uint64_t in_stride, const std::uint32_t* in_elem,
                    const std::uint64_t* in_path, const std::uint32_t* elem_tag, std::uint64_t in_begin, std::uint64_t n_in,
                    int final_mode) {
        const IrSplit& sp = stat[j];
        const int nsub = int(sp.subdivisions);
        const bool last = j + 1 == stat.size();
        const int row_end = last ? n : stat[j + 1].arg;
        if(last) {
            std::uint64_t chunk = std::max<std::uint64_t>(1, (std::uint64_t(1) << 30) / std::uint64_t(nsub));
            for(std::uint64_t off = 0; off < n_in; off += chunk) {
                LevelArgs a = base_args();
                a.in_box = in_box; a.in_stride = in_stride; a.in_elem = in_elem; a.in_path = in_path;
                a.elem_tag = elem_tag;
                a.in_begin = in_begin + off; a.n_in = std::min(chunk, n_in - off);
                a.elem_base = std::uint32_t(off);
                a.var = sp.arg; a.nsub = nsub; a.it_limit = n; a.rec_limit = 4;
                a.row_begin = sp.arg; a.row_end = row_end;
                a.hull_lo = hull.p;
                a.hull_hi = hull.p + step_cap * n;
                a.hull_zlo = hull.p + 2 * step_cap * n;
                a.hull_zhi = hull.p + 3 * step_cap * n;
                launch(final_mode, a, int(dyn.size() + j));
            }
            return;
        }
        BoxList& out = stat_level(j + 1);
        std::uint64_t cap = std::min<std::uint64_t>(kLevelCapItems, std::max<std::uint64_t>(n_in, 1) * nsub);
        out.reserve(n, std::max(out.cap, cap), true, true, false, false);
        const std::uint64_t chunk = std::max<std::uint64_t>(1, out.cap / std::uint64_t(nsub));
        for(std::uint64_t off = 0; off < n_in; off += chunk) {
            LevelArgs a = base_args();
            a.in_box = in_box; a.in_stride = in_stride; a.in_elem = in_elem; a.in_path = in_path;
            a.elem_tag = elem_tag;
            a.in_begin = in_begin + off; a.n_in = std::min(chunk, n_in - off);
            a.elem_base = std::uint32_t(off);
            a.var = sp.arg; a.nsub = nsub; a.it_limit = n; a.rec_limit = 4;
            a.row_begin = sp.arg; a.row_end = row_end;
            a.out_box = out.box.p; a.out_stride = out.cap; a.out_cap = out.cap;
            a.out_elem = out.elem.p; a.out_path = out.path.p;
            zero_counter(counters.p);
            launch(MODE_EMIT, a, int(dyn.size() + j));
            std::uint64_t cnt = read_counter(counters.p);
            run_static(j + 1, out.box.p, out.cap, out.elem.p, out.path.p, elem_tag, 0, cnt, final_mode);
        }
    }

    /// Make room in a request's queue before a step takes `taken` of its elements.
    void ensure_queue(Request* r, std::uint64_t taken, std::uint64_t at_least = 0) {
        const std::uint64_t qsize = queue_size(r);
        const std::uint64_t need = std::max(plan::queue_need(qsize, taken, fanout), at_least);
        if(need <= r->qcap) return;
        const std::uint64_t ncap = plan::grow_capacity(r->qcap, need);
        DevBuf<double2> nb;
        DevBuf<std::uint8_t> nd;
        nb.reserve_on(std::size_t(n) * ncap, st);
        nd.reserve_on(ncap, st);
        for(int v = 0; v < n; ++v) {
            cuda_check(cudaMemcpyAsync(nb.p + std::uint64_t(v) * ncap, r->qbox.p + std::uint64_t(v) * r->qcap,
                                       qsize * sizeof(double2), cudaMemcpyDeviceToDevice, st), "queue grow");
        }
        cuda_check(cudaMemcpyAsync(nd.p, r->qdepth.p, qsize, cudaMemcpyDeviceToDevice, st), "queue grow");
        cuda_check(cudaStreamSynchronize(st), "queue grow sync");
        r->qbox.swap(nb);
        r->qdepth.swap(nd);
        const std::uint64_t old_bytes = r->bytes;
        r->qcap = ncap;
        r->bytes = plan::request_bytes(n, r->qcap, std::max<std::uint64_t>(r->crit_cap, 1));
        grown_bytes += (long long)(r->bytes - old_bytes);
        ReqDev& h = req_host[std::size_t(r->slot)];
        h.qbox = r->qbox.p;
        h.qdepth = r->qdepth.p;
        h.qcap = r->qcap;
        patch_queue(r->slot);
    }

    /// One step over the given active requests (arrival order). Returns the number of elements expanded.
    std::uint64_t run_step(const std::vector<Request*>& active) {
        std::vector<std::pair<int, std::uint64_t>> q;
        for(Request* r : active) q.emplace_back(r->slot, queue_size(r));
        const std::vector<plan::Take> takes = plan::fill_step(q, step_cap);
        if(takes.empty()) return 0;
        gather_host.clear();
        std::uint64_t B = 0;
        for(const auto& t : takes) {
            Request* r = slot_req[std::size_t(t.slot)];
            ensure_queue(r, t.count);
            gather_host.push_back(GatherEntry{std::uint32_t(t.slot), 0u, t.begin, t.count, t.dst});
            B = t.dst + t.count;
        }
        gather.reserve(gather_host.size());
        cuda_check(cudaMemcpyAsync(gather.p, gather_host.data(), gather_host.size() * sizeof(GatherEntry),
                                   cudaMemcpyHostToDevice, st), "gather table");
        launch_gate("gather");
        k_gather<<<unsigned((B + 127) / 128), 128, 0, st>>>(gather.p, int(gather_host.size()), B, req_dev.p, n, step.box.p,
                                                            step.cap, step.depth.p, step.tag.p);
        cuda_check(cudaGetLastError(), "gather");

        zero_counter(counters.p + 1);
        zero_counter(counters.p + 2);
        if(stat.empty()) {
            const RouteIteration itr{max_iter, lem->k->is_f32, iter_single, iter_volume};
            k_route_elements<<<unsigned((B + 127) / 128), 128, 0, st>>>(
                step.box.p, step.cap, step.depth.p, step.tag.p, B, n, req_dev.p, fin.box.p, fin.depth.p, fin.tag.p,
                counters.p + 1, nonfin.box.p, nonfin.depth.p, nonfin.tag.p, counters.p + 2, step_cap, itr);
            cuda_check(cudaGetLastError(), "route elements");
        } else {
            // pass p over the static splits (p = 1, 2, ...): hulls of the elements, then routing; with re-iteration
            // (p < max_iter) a hull that should_iterate accepts is re-run as the element of the next pass
            // (p_handle_cuboid_nf, cpu_prover_core.hpp:113-134)
            const BoxList* in = &step;
            std::uint64_t n_elem = B;
            for(int pass = 1; n_elem > 0; ++pass) {
                // reset hulls: lo keys to max, hi keys to 0, first-zero paths to max
                cuda_check(cudaMemsetAsync(hull.p, 0xff, n_elem * n * sizeof(unsigned long long), st), "hull reset");
                cuda_check(cudaMemsetAsync(hull.p + step_cap * n, 0, n_elem * n * sizeof(unsigned long long), st),
                           "hull reset");
                cuda_check(cudaMemsetAsync(hull.p + 2 * step_cap * n, 0xff, 2 * step_cap * n * sizeof(unsigned long long),
                                           st), "hull reset");
                run_static(0, in->box.p, in->cap, nullptr, nullptr, in->tag.p, 0, n_elem, MODE_HULL);
                HullArgs h{};
                h.hull_lo = hull.p;
                h.hull_hi = hull.p + step_cap * n;
                h.hull_zlo = hull.p + 2 * step_cap * n;
                h.hull_zhi = hull.p + 3 * step_cap * n;
                h.depth = in->depth.p;
                h.tag = in->tag.p;
                h.req = req_dev.p;
                h.n_elem = std::uint32_t(n_elem);
                h.nargs = n;
                h.fin_box = fin.box.p; h.fin_depth = fin.depth.p; h.fin_tag = fin.tag.p; h.fin_count = counters.p + 1;
                h.nf_box = nonfin.box.p; h.nf_depth = nonfin.depth.p; h.nf_tag = nonfin.tag.p; h.nf_count = counters.p + 2;
                h.out_stride = step_cap;
                h.iterate = pass < max_iter;
                if(h.iterate) {
                    h.f32 = lem->k->is_f32;
                    h.single = iter_single;
                    h.volume = iter_volume;
                    h.elem_box = in->box.p;
                    h.elem_stride = in->cap;
                    BoxList& out = (in == &iter_in) ? iter_out : iter_in;
                    h.it_box = out.box.p; h.it_depth = out.depth.p; h.it_tag = out.tag.p; h.it_count = counters.p + 4;
                    h.it_stride = out.cap;
                    zero_counter(counters.p + 4);
                }
                launch_gate("hull finalize");
                k_hull_finalize<<<unsigned((n_elem + 127) / 128), 128, 0, st>>>(h);
                cuda_check(cudaGetLastError(), "hull finalize");
                if(!h.iterate) break;
                n_elem = read_counter(counters.p + 4);
                in = (in == &iter_in) ? &iter_out : &iter_in;
            }
        }
        const unsigned long long* fin_nf = read_counters(counters.p + 1, 2);
        const std::uint64_t nfin = fin_nf[0];
        const std::uint64_t nnf = fin_nf[1];
        if(nfin > 0) {
            if(stat.empty()) {
                k_store_criticals<<<unsigned((nfin + 127) / 128), 128, 0, st>>>(fin.box.p, step_cap, fin.tag.p, nfin, n,
                                                                                 req_dev.p);
                cuda_check(cudaGetLastError(), "store criticals");
            } else {
                run_static(0, fin.box.p, step_cap, nullptr, nullptr, fin.tag.p, 0, nfin, MODE_CRIT);
            }
        }
        if(nnf > 0) run_dynamic(0, nonfin.box.p, step_cap, nonfin.depth.p, nonfin.tag.p, 0, 0, nnf, false, 1);
        read_slots();
        return B;
    }
};

} // namespace sid

struct sid_engine {
    int device = 0;
    int sm_count = 1;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_in = nullptr, copy_out = nullptr;   // sid_eval_batch's transfer streams
    std::vector<std::unique_ptr<Lemma>> lemmas;
    std::map<int, std::unique_ptr<sid::Lane>> prove_lanes;   // lanes of sid_prove, one per lemma
    DevBuf<double> batch_in_lo, batch_in_hi, batch_out_lo, batch_out_hi;
    DevBuf<std::int8_t> batch_verdict;
    DevBuf<std::uint32_t> batch_key, batch_order, batch_count, batch_totals;
    DevBuf<std::uint64_t> batch_slow;             // deferred cuboids of a batch call (BatchArgs::slow)
    DevBuf<unsigned long long> batch_slow_count;
    bool batch_profile = false;
    std::vector<cudaEvent_t> batch_events;   // four per profiled call: start, ordered, evaluated, scattered
    std::uint64_t batch_launches = 0;        // kernels launched by profiled calls
};

namespace {

using namespace sid;

Lemma* get_lemma(sid_engine* e, int id) {
    if(!e) fail(SID_ERR_INVALID, "null engine");
    if(id < 0 || id >= int(e->lemmas.size())) fail(SID_ERR_INVALID, "bad lemma id %d", id);
    return e->lemmas[std::size_t(id)].get();
}

void set_device(sid_engine* e) { cuda_check(cudaSetDevice(e->device), "cudaSetDevice"); }

void profile_mark(sid_engine* eng, cudaStream_t s) {
    if(!eng->batch_profile) return;
    cudaEvent_t ev;
    cuda_check(cudaEventCreate(&ev), "profile event");
    eng->batch_events.push_back(ev);
    cuda_check(cudaEventRecord(ev, s), "profile event record");
}

void profile_clear(sid_engine* eng) {
    for(cudaEvent_t ev : eng->batch_events) cudaEventDestroy(ev);
    eng->batch_events.clear();
    eng->batch_launches = 0;
}


constexpr double kOrderShare = 0.01;   // AUTO orders batches when more cuboids than this need double constraints

/// Hands a batch call's count of double-constraint cuboids to the host: a store into pinned host memory from
/// the evaluation stream (no copy engine, so the sample never waits behind the large output copies), then
/// the device counter is cleared for the next sampled call.
__global__ void k_publish_sample(unsigned long long* dev, unsigned long long* host) {
    if(blockIdx.x != 0 || threadIdx.x != 0) return;
    *reinterpret_cast<volatile unsigned long long*>(host) = *dev;
    *dev = 0;
    __threadfence_system();
}

/// The share of cuboids that needed the double constraints in the lemma's last sampled batch call, if that
/// call's counter has arrived (never blocks).
void poll_batch_sample(Lemma* lem) {
    if(!lem->batch_sample_pending) return;
    const cudaError_t q = cudaEventQuery(lem->batch_sample_ev);
    if(q == cudaErrorNotReady) {
        if(cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();
        return;
    }
    cuda_check(q, "batch sample");
    lem->batch_double_share = double(*lem->batch_sample_host) / double(std::max<std::uint64_t>(lem->batch_sample_n, 1));
    lem->batch_sample_pending = false;
}

/// Evaluate a batch of n cuboids (SoA, device, variables `stride` apart; 0: n); results go to the cuboids' own
/// positions. Asynchronous on `s`. With ordering (the lemma's batch mode, see sid_lemma_batch_order) the
/// cuboids are evaluated in the order (tile of 2^18 cuboids, Morton code of the lower corner), which keeps a
/// warp's cuboids on the same branches of the double constraints; without it, in their own order, which
/// saves the sort when the float test decides nearly every cuboid. Every call whose predecessor's sample has
/// arrived counts the cuboids that needed the double constraints.
void eval_batch_ordered(sid_engine* eng, Lemma* lem, const double* lo, const double* hi, std::uint64_t n, double* out_lo,
                        double* out_hi, std::int8_t* verdict, cudaStream_t s, std::uint64_t stride = 0, bool plain = false) {
    if(stride == 0) stride = n;
    const int nargs = lem->ir.nargs;
    profile_mark(eng, s);
    poll_batch_sample(lem);
    // the all-double kernel (plain) always orders: nearly every cuboid there reaches the double constraints
    const bool want_order = plain || lem->batch_order == SID_BATCH_ORDER_ON ||
                            (lem->batch_order == SID_BATCH_ORDER_AUTO &&
                             (lem->batch_double_share < 0.0 || lem->batch_double_share > kOrderShare));
    const std::uint32_t* order = nullptr;
    const std::uint64_t tiles = (n + (std::uint64_t(1) << kTileLog) - 1) >> kTileLog;
    const std::uint64_t buckets = tiles << kTileKeyBits;
    const std::uint64_t blocks = (buckets + 4095) / 4096;
    if(want_order && n >= 4096 && n <= 0xffffffffull && nargs <= 16 && blocks <= 4096) {
        const int bits = std::max(1, kTileKeyBits / std::max(nargs, 1));
        MortonQuant qp{};
        for(int v = 0; v < nargs; ++v) {
            const double rl = lem->root_host[std::size_t(2 * v)], rh = lem->root_host[std::size_t(2 * v + 1)];
            const double range = rh - rl;
            qp.off[v] = float(rl);
            qp.scale[v] = range > 0.0 && range < 1e300 ? float(double(1u << bits) / range) : 0.0f;
        }
        eng->batch_key.reserve(std::size_t(n));
        eng->batch_order.reserve(std::size_t(n));
        eng->batch_count.reserve(std::size_t(buckets));
        eng->batch_totals.reserve(std::size_t(blocks) + 1);
        cuda_check(cudaMemsetAsync(eng->batch_count.p, 0, buckets * sizeof(std::uint32_t), s), "order histogram reset");
        const unsigned g = unsigned((n + 255) / 256);
        k_order_keys<<<g, 256, 0, s>>>(lo, n, stride, nargs, qp, bits, eng->batch_key.p, eng->batch_count.p);
        k_scan_blocks<<<unsigned(blocks), 1024, 0, s>>>(eng->batch_count.p, buckets, eng->batch_totals.p);
        k_scan_blocks<<<1, 1024, 0, s>>>(eng->batch_totals.p, blocks, eng->batch_totals.p + blocks);
        k_scan_add<<<unsigned((buckets + 255) / 256), 256, 0, s>>>(eng->batch_count.p, buckets, eng->batch_totals.p);
        k_order_scatter<<<g, 256, 0, s>>>(eng->batch_key.p, n, eng->batch_count.p, eng->batch_order.p);
        cuda_check(cudaGetLastError(), "batch ordering");
        order = eng->batch_order.p;
        if(eng->batch_profile) eng->batch_launches += 5;
    }
    profile_mark(eng, s);
    BatchArgs a{lo, hi, out_lo, out_hi, verdict, n, order, stride, nullptr, nullptr, nullptr, 0u};
    a.slow_blocks = unsigned(std::max(eng->sm_count, 1)) * 8u;
    launch_gate("eval batch");
    if(plain) {
        cuda_check(lem->k->eval_batch_plain(a, s), "eval batch (plain)");
        if(eng->batch_profile) eng->batch_launches += n > 0 ? 1u : 0u;
        profile_mark(eng, s);
        profile_mark(eng, s);
        return;
    }
    const bool defers = batch_defers(nargs);
    if(defers) {
        eng->batch_slow.reserve(std::size_t(n));
        eng->batch_slow_count.reserve(2);   // one counter per kind of deferred cuboid
        a.slow = eng->batch_slow.p;
        a.slow_count = eng->batch_slow_count.p;
    }
    const bool sample = !lem->batch_sample_pending && !lem->k->is_f32 && n > 0;
    if(sample) {
        if(!lem->batch_sample.p) {   // once per lemma: cleared device counter, pinned (device-visible) host word
            lem->batch_sample.reserve(1);
            cuda_check(cudaMemsetAsync(lem->batch_sample.p, 0, sizeof(unsigned long long), s), "batch sample");
        }
        if(!lem->batch_sample_ev) {
            cuda_check(cudaEventCreateWithFlags(&lem->batch_sample_ev, cudaEventDisableTiming), "batch sample");
        }
        if(!lem->batch_sample_host) {
            cuda_check(cudaMallocHost(reinterpret_cast<void**>(&lem->batch_sample_host), sizeof(unsigned long long)),
                       "batch sample");
        }
        a.double_rows = lem->batch_sample.p;
    }
    cuda_check(lem->k->eval_batch(a, s), "eval batch");
    if(eng->batch_profile) eng->batch_launches += n > 0 ? 1u + (defers ? 1u : 0u) + (sample ? 1u : 0u) : 0u;
    if(sample) {
        k_publish_sample<<<1, 1, 0, s>>>(lem->batch_sample.p, lem->batch_sample_host);
        cuda_check(cudaGetLastError(), "batch sample");
        cuda_check(cudaEventRecord(lem->batch_sample_ev, s), "batch sample");
        lem->batch_sample_pending = true;
        lem->batch_sample_n = n;
    }
    profile_mark(eng, s);
    profile_mark(eng, s);
}

constexpr std::uint64_t kBatchChunk = std::uint64_t(1) << 20;   // cuboids per transfer chunk of sid_eval_batch

void check_precision(int precision) {
    if(precision != SID_PRECISION_PLAIN && precision != SID_PRECISION_FP32_ESCALATE &&
       precision != SID_PRECISION_FP32_TUNED) {
        fail(SID_ERR_INVALID, "unknown precision mode %d", precision);
    }
}

constexpr char kCheckpointMagic[8] = {'S', 'I', 'D', 'C', 'K', 'P', 'T', '2'};   // 2: repeated-node counter

void write_checkpoint(const char* path, const ProofState& ps) {
    std::string tmp = std::string(path) + ".part";
    std::FILE* f = std::fopen(tmp.c_str(), "wb");
    if(!f) fail(SID_ERR_INVALID, "cannot write checkpoint %s", tmp.c_str());
    const std::uint64_t q = ps.cnt[RC_QSIZE], crit = ps.criticals.size();
    bool ok = std::fwrite(kCheckpointMagic, 1, 8, f) == 8 &&
              std::fwrite(&ps.fingerprint, sizeof ps.fingerprint, 1, f) == 1 &&
              std::fwrite(&ps.nargs, sizeof ps.nargs, 1, f) == 1 &&
              std::fwrite(&ps.generations, sizeof ps.generations, 1, f) == 1 &&
              std::fwrite(&ps.steps, sizeof ps.steps, 1, f) == 1 &&
              std::fwrite(ps.cnt, sizeof ps.cnt, 1, f) == 1 &&
              std::fwrite(&crit, sizeof crit, 1, f) == 1 &&
              (q == 0 || std::fwrite(ps.boxes.data(), sizeof(double2), ps.boxes.size(), f) == ps.boxes.size()) &&
              (q == 0 || std::fwrite(ps.depth.data(), 1, ps.depth.size(), f) == ps.depth.size()) &&
              (crit == 0 || std::fwrite(ps.criticals.data(), sizeof(double), crit, f) == crit);
    ok = (std::fclose(f) == 0) && ok;
    if(!ok || std::rename(tmp.c_str(), path) != 0) fail(SID_ERR_INVALID, "writing checkpoint %s failed", path);
}

void read_checkpoint(const char* path, ProofState& ps) {
    std::FILE* f = std::fopen(path, "rb");
    if(!f) fail(SID_ERR_INVALID, "cannot open checkpoint %s", path);
    char magic[8];
    std::uint64_t crit = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kCheckpointMagic, 8) == 0 &&
              std::fread(&ps.fingerprint, sizeof ps.fingerprint, 1, f) == 1 &&
              std::fread(&ps.nargs, sizeof ps.nargs, 1, f) == 1 &&
              std::fread(&ps.generations, sizeof ps.generations, 1, f) == 1 &&
              std::fread(&ps.steps, sizeof ps.steps, 1, f) == 1 &&
              std::fread(ps.cnt, sizeof ps.cnt, 1, f) == 1 && std::fread(&crit, sizeof crit, 1, f) == 1 &&
              ps.nargs > 0 && ps.nargs <= 64 && ps.cnt[RC_QSIZE] <= (std::uint64_t(1) << 36) && crit <= (std::uint64_t(1) << 36);
    if(ok) {
        const std::uint64_t q = ps.cnt[RC_QSIZE];
        ps.boxes.resize(std::size_t(q * ps.nargs));
        ps.depth.resize(std::size_t(q));
        ps.criticals.resize(std::size_t(crit));
        ok = (q == 0 || std::fread(ps.boxes.data(), sizeof(double2), ps.boxes.size(), f) == ps.boxes.size()) &&
             (q == 0 || std::fread(ps.depth.data(), 1, ps.depth.size(), f) == ps.depth.size()) &&
             (crit == 0 || std::fread(ps.criticals.data(), sizeof(double), crit, f) == crit);
    }
    std::fclose(f);
    if(!ok) fail(SID_ERR_INVALID, "%s is not a complete checkpoint", path);
}

/// A whole proof of one lemma (sid_prove): one request on the engine's lane of that lemma. A non-zero
/// step/mask override the step size and the float-pass levels (autotuning); `resume` continues from a
/// checkpoint.
void prove_one(sid_engine* eng, int lemma_id, const sid_prove_opts& o, sid_result* res, std::uint64_t step_override = 0,
               const std::uint32_t* mask_override = nullptr, const ProofState* resume = nullptr,
               const std::uint32_t* noprop_override = nullptr) {
    Lemma* lem = get_lemma(eng, lemma_id);
    auto& slot = eng->prove_lanes[lemma_id];
    if(!slot) slot.reset(new Lane(eng, lem, eng->stream, false, eng->sm_count, 1));
    Lane& lane = *slot;
    const bool tuned = o.precision == SID_PRECISION_FP32_TUNED && lem->tuned;
    const std::uint64_t step = o.batch_elements > 0 ? std::uint64_t(o.batch_elements)
                                                    : (tuned ? std::uint64_t(lem->tuning.step_elements) : kDefaultStep);
    lane.configure(step_override ? step_override : step, o.precision != SID_PRECISION_PLAIN,
                   mask_override ? *mask_override : (tuned ? lem->tuning.fp32_level_mask : o.fp32_level_mask),
                   noprop_override ? *noprop_override : (tuned ? lem->tuning.fp32_noprop_mask : o.fp32_noprop_mask));
    lane.set_iteration(o.max_iterations_per_node, o.iteration_volume_criterion, o.iteration_single_dimension_criterion);

    if(o.part_count > 1 && o.part_index >= o.part_count) {
        fail(SID_ERR_INVALID, "part_index %u outside part_count %u", o.part_index, o.part_count);
    }
    Request r;
    r.lem = lem;
    r.lemma_id = lemma_id;
    r.full = true;
    r.part_index = o.part_index;
    r.part_count = o.part_count;
    r.generations = o.generation_count;
    r.crit_cap = o.max_criticals_kept;
    r.resume = resume;
    std::uint32_t steps = resume ? resume->steps : 0;
    bool complete = true;

    cudaEvent_t ev0, ev1;
    cuda_check(cudaEventCreate(&ev0), "event");
    cuda_check(cudaEventCreate(&ev1), "event");
    ReqDev last{};
    try {
        cuda_check(cudaEventRecord(ev0, lane.st), "event record");
        const auto t0 = Clock::now();
        auto last_cb = t0;
        bool first_done = false;
        // the device proof loop takes the whole proof (root partition included) when asked for and when the proof
        // needs nothing between steps from the host
        const unsigned loop_blocks = o.device_loop_blocks > 0 ? o.device_loop_blocks : (tuned ? lem->tuning.loop_blocks : 0u);
        const bool loop = loop_blocks > 0 && !resume && o.max_iterations_per_node <= 1 && !o.checkpoint_path &&
                          !o.stop_after_steps && !o.progress;
        lane.admit(&r, loop);
        if(loop) {
            if(lane.run_device_loop(&r, loop_blocks)) {
                steps = lane.loop_steps;
            } else {
                // the queue or a list outgrew the loop's room: prove on the host-driven loop from the start
                lane.release(&r);
                lane.admit(&r, false);
            }
        }
        const std::vector<Request*> active{&r};
        auto checkpoint = [&]() {
            ProofState ps;
            lane.snapshot(&r, ps);
            ps.fingerprint = lem->ir.fingerprint;
            ps.generations = o.generation_count;
            ps.steps = steps;
            write_checkpoint(o.checkpoint_path, ps);
        };
        while(lane.queue_size(&r) > 0) {
            if(o.stop_after_steps && steps >= (resume ? resume->steps : 0) + o.stop_after_steps) {
                complete = false;
                if(o.checkpoint_path) checkpoint();
                break;
            }
            lane.run_step(active);
            ++steps;
            if(o.checkpoint_path && o.checkpoint_every_steps && steps % o.checkpoint_every_steps == 0 &&
               lane.queue_size(&r) > 0) {
                checkpoint();
            }
            if(o.progress) {
                const auto now = Clock::now();
                const long long since_start = std::chrono::duration_cast<std::chrono::milliseconds>(now - t0).count();
                const long long since_last = std::chrono::duration_cast<std::chrono::milliseconds>(now - last_cb).count();
                if(first_done ? since_last >= (long long)o.progress_every_ms : since_start >= (long long)o.progress_first_ms) {
                    first_done = true;
                    last_cb = now;
                    const ReqDev& c = lane.counters_of(&r);
                    sid_progress p{};
                    p.queue_size = c.cnt[RC_QSIZE];
                    p.cuboid_count = c.cnt[RC_CUBOIDS];
                    p.leaf_count = c.cnt[RC_LEAVES];
                    p.critical_count = c.cnt[RC_CRITICALS];
                    std::vector<double> head(std::size_t(2 * lane.n));
                    if(p.queue_size > 0) {
                        for(int v = 0; v < lane.n; ++v) {
                            double2 b;
                            cuda_check(cudaMemcpyAsync(&b, r.qbox.p + std::uint64_t(v) * r.qcap + p.queue_size - 1, sizeof(b),
                                                       cudaMemcpyDeviceToHost, lane.st), "queue head");
                            cuda_check(cudaStreamSynchronize(lane.st), "queue head");
                            head[std::size_t(2 * v)] = b.x;
                            head[std::size_t(2 * v + 1)] = b.y;
                        }
                        p.queue_head = head.data();
                    }
                    o.progress(o.progress_user, &p);
                }
            }
        }
        cuda_check(cudaEventRecord(ev1, lane.st), "event record");
        cuda_check(cudaEventSynchronize(ev1), "event sync");
        lane.fetch_criticals(&r);
        last = lane.counters_of(&r);
    } catch(...) {
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        lane.release(&r);
        throw;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    lane.release(&r);
    res->num_cuboids = last.cnt[RC_CUBOIDS];
    res->num_leaf_cuboids = last.cnt[RC_LEAVES];
    res->num_critical_cuboids = last.cnt[RC_CRITICALS];
    res->num_repeated_nodes = last.cnt[RC_REPEATED];
    res->criticals_stored = std::min<std::uint64_t>(res->num_critical_cuboids, r.crit_cap);
    res->escalated = last.cnt[RC_ESCALATED];
    res->seconds = double(ms) / 1000.0;
    res->complete = complete ? 1 : 0;
    res->steps = steps;
    lem->criticals = std::move(r.criticals);
}

/// Configure the cached sid_prove lane of a lemma for a whole proof with options `o` (as prove_one does).
Lane& prove_lane(sid_engine* eng, int lemma_id, const sid_prove_opts& o) {
    Lemma* lem = get_lemma(eng, lemma_id);
    auto& slot = eng->prove_lanes[lemma_id];
    if(!slot) slot.reset(new Lane(eng, lem, eng->stream, false, eng->sm_count, 1));
    Lane& lane = *slot;
    const bool tuned = o.precision == SID_PRECISION_FP32_TUNED && lem->tuned;
    const std::uint64_t step = o.batch_elements > 0 ? std::uint64_t(o.batch_elements)
                                                    : (tuned ? std::uint64_t(lem->tuning.step_elements) : kDefaultStep);
    lane.configure(step, o.precision != SID_PRECISION_PLAIN, tuned ? lem->tuning.fp32_level_mask : o.fp32_level_mask,
                   tuned ? lem->tuning.fp32_noprop_mask : o.fp32_noprop_mask);
    lane.set_iteration(o.max_iterations_per_node, o.iteration_volume_criterion, o.iteration_single_dimension_criterion);
    return lane;
}

/// Whole proofs of several lemmas in one bundle kernel (sid_prove_bundle): the caller's j-th lemma is proof pos[j]
/// of the compiled bundle `bk`. Each proof is one request on its lemma's cached lane, admitted with its root on the
/// device; all these lanes run on the engine's stream, which the bundle kernel runs on too. A proof whose queue or
/// lists outgrew the loop's room is proved again on its host-driven lane, as sid_prove does.
void prove_bundle(sid_engine* eng, const BundleKernels* bk, const std::vector<int>& ids, const std::vector<int>& pos,
                  const sid_prove_opts& o, sid_result* res) {
    const std::size_t n = ids.size();
    std::vector<Lane*> lanes(n);
    std::vector<Request> reqs(n);
    for(std::size_t j = 0; j < n; ++j) {
        lanes[j] = &prove_lane(eng, ids[j], o);
        Request& r = reqs[j];
        r.lem = get_lemma(eng, ids[j]);
        r.lemma_id = ids[j];
        r.full = true;
        r.generations = o.generation_count;
        r.crit_cap = o.max_criticals_kept;
    }
    const int occ = bk->occupancy();
    if(occ <= 0) fail(SID_ERR_UNSUPPORTED, "bundle %s: the kernel cannot be resident", bk->name);
    const unsigned most = unsigned(occ) * unsigned(std::max(eng->sm_count, 1));
    const unsigned G = o.device_loop_blocks > 0 ? std::max(1u, std::min(o.device_loop_blocks, most)) : most;
    cudaEvent_t ev0, ev1;
    cuda_check(cudaEventCreate(&ev0), "event");
    cuda_check(cudaEventCreate(&ev1), "event");
    std::vector<std::uint32_t> steps(n, 0);
    auto release_all = [&] {
        for(std::size_t j = 0; j < n; ++j) {
            try { lanes[j]->release(&reqs[j]); } catch(...) {}
        }
    };
    try {
        cuda_check(cudaEventRecord(ev0, eng->stream), "event record");
        BundleArgs b{};
        b.n = int(n);
        for(std::size_t j = 0; j < n; ++j) {
            lanes[j]->admit(&reqs[j], true);
            lanes[j]->prepare_loop(&reqs[j], G, b.p[pos[j]]);
        }
        LoopCtl* sync = b.p[0].ctl;
        for(std::size_t i = 0; i < n; ++i) b.p[i].sync = sync;
        launch_gate("bundle proof loop");
        cuda_check(bk->launch(b, G, eng->stream), "bundle proof loop launch");
        LoopCtl c{};
        cuda_check(cudaMemcpyAsync(&c, sync, sizeof(LoopCtl), cudaMemcpyDeviceToHost, eng->stream), "bundle control");
        cuda_check(cudaStreamSynchronize(eng->stream), "bundle proof loop");
        if(c.error == kLoopTimeout) fail(SID_ERR_TIMEOUT, "bundle proof loop: a grid barrier gave up");
        for(std::size_t j = 0; j < n; ++j) {
            Lane& lane = *lanes[j];
            Request& r = reqs[j];
            if(lane.finish_loop(&r) && c.error == kLoopOk) {
                steps[j] = lane.loop_steps;
                continue;
            }
            // the loop stopped early: this proof again on the host-driven loop, from its root
            lane.release(&r);
            lane.admit(&r, false);
            const std::vector<Request*> active{&r};
            while(lane.queue_size(&r) > 0) {
                lane.run_step(active);
                ++steps[j];
            }
        }
        cuda_check(cudaEventRecord(ev1, eng->stream), "event record");
        cuda_check(cudaEventSynchronize(ev1), "event sync");
        for(std::size_t j = 0; j < n; ++j) lanes[j]->fetch_criticals(&reqs[j]);
    } catch(...) {
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        release_all();
        throw;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    for(std::size_t j = 0; j < n; ++j) {
        const ReqDev last = lanes[j]->counters_of(&reqs[j]);
        lanes[j]->release(&reqs[j]);
        sid_result* out = res + j;
        out->num_cuboids = last.cnt[RC_CUBOIDS];
        out->num_leaf_cuboids = last.cnt[RC_LEAVES];
        out->num_critical_cuboids = last.cnt[RC_CRITICALS];
        out->num_repeated_nodes = last.cnt[RC_REPEATED];
        out->criticals_stored = std::min<std::uint64_t>(out->num_critical_cuboids, reqs[j].crit_cap);
        out->escalated = last.cnt[RC_ESCALATED];
        out->seconds = double(ms) / 1000.0;
        out->complete = 1;
        out->steps = steps[j];
        reqs[j].lem->criticals = std::move(reqs[j].criticals);
    }
}

} // namespace

/// The served form: one worker thread, stream and lane per lemma.
struct sid_server {
    struct Worker {
        int lemma_id = -1;
        std::unique_ptr<sid::Lane> lane;
        std::thread th;
        std::deque<Request*> pending;
        std::vector<Request*> active;
        std::condition_variable cv;
    };

    sid_engine* eng = nullptr;
    sid_server_opts opts{};
    std::mutex mu;
    std::condition_variable cv_done;
    std::unordered_map<std::uint64_t, std::unique_ptr<Request>> reqs;
    std::map<int, std::unique_ptr<Worker>> workers;
    std::uint64_t next_id = 1;
    std::uint64_t mem_used = 0;          // device bytes held by admitted requests
    bool stopping = false;

    std::uint64_t budget() const { return opts.memory_budget_bytes ? opts.memory_budget_bytes : (std::uint64_t(16) << 30); }

    /// The lane of a worker: its own stream, the lemma's kernels and scratch, configured for the server.
    void make_lane(Worker* w) {
        cuda_check(cudaSetDevice(eng->device), "cudaSetDevice");
        Lemma* lem = eng->lemmas[std::size_t(w->lemma_id)].get();
        cudaStream_t s = nullptr;
        cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
        const int slots = int(opts.max_requests_per_lane > 0 ? opts.max_requests_per_lane : kDefaultSlots);
        std::unique_ptr<sid::Lane> lane;
        try {
            lane.reset(new Lane(eng, lem, s, true, eng->sm_count, slots));
        } catch(...) {
            cudaStreamDestroy(s);
            throw;
        }
        const bool tuned = opts.precision == SID_PRECISION_FP32_TUNED && lem->tuned;
        lane->configure(opts.step_elements > 0 ? std::uint64_t(opts.step_elements)
                                               : (tuned ? std::uint64_t(lem->tuning.step_elements) : kDefaultStep),
                        opts.precision != SID_PRECISION_PLAIN, tuned ? lem->tuning.fp32_level_mask : ~0u,
                        tuned ? lem->tuning.fp32_noprop_mask : ~0u);
        lane->set_iteration(opts.max_iterations_per_node, opts.iteration_volume_criterion,
                            opts.iteration_single_dimension_criterion);
        w->lane = std::move(lane);
    }

    /// One round of a worker: admit what fits, run one step over the admitted requests, retire the finished ones.
    void serve_round(Worker* w, std::vector<Request*>& held) {
        Lane& lane = *w->lane;
        std::vector<Request*> admit;
        {
            std::lock_guard<std::mutex> lk(mu);
            std::vector<std::uint64_t> need;
            for(Request* r : w->pending) need.push_back(lane.initial_bytes(*r));
            const std::size_t k = plan::admit_count(need, mem_used, budget(), w->active.size(),
                                                    std::size_t(lane.free_slots()));
            for(std::size_t i = 0; i < k; ++i) {
                Request* r = w->pending.front();
                w->pending.pop_front();
                r->bytes = need[i];          // charged to the budget from here on, whatever happens next
                mem_used += need[i];
                admit.push_back(r);
                held.push_back(r);
            }
        }
        for(Request* r : admit) {
            lane.admit(r);
            std::lock_guard<std::mutex> lk(mu);
            r->state = SID_REQ_RUNNING;
            r->admitted = true;
            r->t_admit = Clock::now();
            r->view = lane.counters_of(r);
            w->active.push_back(r);
        }
        if(!w->active.empty()) lane.run_step(w->active);
        std::vector<Request*> done;
        for(Request* r : w->active) if(lane.queue_size(r) == 0) done.push_back(r);
        std::vector<sid::ReqDev> final_counts;
        for(Request* r : done) {
            lane.fetch_criticals(r);
            final_counts.push_back(lane.counters_of(r));
            lane.release(r);
            held.erase(std::find(held.begin(), held.end(), r));
        }
        std::lock_guard<std::mutex> lk(mu);
        mem_used += std::uint64_t(std::max<long long>(0, lane.take_grown_bytes()));
        for(Request* r : w->active) if(r->slot >= 0) r->view = lane.counters_of(r);
        for(std::size_t i = 0; i < done.size(); ++i) {
            Request* r = done[i];
            r->view = final_counts[i];
            mem_used -= std::min(mem_used, r->bytes);
            r->state = SID_REQ_DONE;
            r->t_done = Clock::now();
            w->active.erase(std::find(w->active.begin(), w->active.end(), r));
        }
        if(!done.empty()) cv_done.notify_all();
    }

    /// After a round threw: the requests admitted to the lane fail (their device state is dropped and their
    /// memory returned to the budget); the lane and the waiting requests carry on. Without a lane (its set-up
    /// failed) no request can run, so the waiting ones fail too.
    void recover(Worker* w, std::vector<Request*>& held, int status, const std::string& msg) {
        if(w->lane) {
            for(Request* r : held) {
                try { w->lane->release(r); } catch(...) {}
            }
        }
        std::lock_guard<std::mutex> lk(mu);
        const auto now = Clock::now();
        for(Request* r : held) {
            r->state = SID_REQ_FAILED;
            r->error = msg;
            r->error_status = status;
            r->t_done = now;
            mem_used -= std::min(mem_used, r->bytes);
        }
        held.clear();
        w->active.clear();
        if(!w->lane) {
            for(Request* r : w->pending) {
                r->state = SID_REQ_FAILED;
                r->error = msg;
                r->error_status = status;
                r->t_done = now;
            }
            w->pending.clear();
        }
        cv_done.notify_all();
    }

    void worker_loop(Worker* w) {
        std::vector<Request*> held;   // admitted requests whose device state must be released on exit
        for(;;) {
            {
                std::unique_lock<std::mutex> lk(mu);
                w->cv.wait(lk, [&] { return stopping || !w->pending.empty() || !w->active.empty(); });
                if(stopping) break;
            }
            try {
                if(!w->lane) make_lane(w);
                serve_round(w, held);
            } catch(const SidError& e) {
                recover(w, held, e.status, e.msg);
            } catch(const std::exception& e) {
                recover(w, held, SID_ERR_INVALID, e.what());
            }
        }
        if(w->lane) {
            for(Request* r : held) {
                try { w->lane->release(r); } catch(...) {}
            }
            w->lane.reset();
        }
    }

    static void fill_status(const Request& r, sid_request_status* st) {
        std::memset(st, 0, sizeof(*st));
        st->state = r.state;
        st->num_cuboids = r.view.cnt[RC_CUBOIDS];
        st->num_leaf_cuboids = r.view.cnt[RC_LEAVES];
        st->num_critical_cuboids = r.view.cnt[RC_CRITICALS];
        st->escalated = r.view.cnt[RC_ESCALATED];
        st->num_repeated_nodes = r.view.cnt[RC_REPEATED];
        st->criticals_stored = std::min<std::uint64_t>(r.view.cnt[RC_CRITICALS], r.crit_cap);
        st->proved = r.state == SID_REQ_DONE && r.view.cnt[RC_CRITICALS] == 0;
        if(r.admitted) st->seconds_queued = std::chrono::duration<double>(r.t_admit - r.t_submit).count();
        if(r.state == SID_REQ_DONE || r.state == SID_REQ_FAILED) {
            st->seconds_to_verdict = std::chrono::duration<double>(r.t_done - r.t_submit).count();
        }
    }
};

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
    o->fp32_level_mask = ~0u;
    o->fp32_noprop_mask = ~0u;
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
        cuda_check(cudaStreamCreateWithFlags(&e->copy_in, cudaStreamNonBlocking), "cudaStreamCreate");
        cuda_check(cudaStreamCreateWithFlags(&e->copy_out, cudaStreamNonBlocking), "cudaStreamCreate");
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
        cudaStream_t ci = engine->copy_in, co = engine->copy_out;
        engine->prove_lanes.clear();
        engine->lemmas.clear();
        profile_clear(engine);
        owner.reset();
        if(s) cudaStreamDestroy(s);
        if(ci) cudaStreamDestroy(ci);
        if(co) cudaStreamDestroy(co);
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
        lem->root_host.assign(std::size_t(2 * lem->ir.nargs), 0.0);
        cuda_check(cudaMemcpyAsync(lem->root_host.data(), lem->root.p, sizeof(double2) * std::size_t(lem->ir.nargs),
                                   cudaMemcpyDeviceToHost, engine->stream), "root box copy");
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
        get_lemma(engine, lemma_id);
        if(!result) fail(SID_ERR_INVALID, "null result");
        sid_prove_opts o;
        if(opts) o = *opts; else sid_prove_opts_default(&o);
        check_precision(o.precision);
        if(o.generation_count > 250) fail(SID_ERR_INVALID, "generation_count too large");
        set_device(engine);
        std::memset(result, 0, sizeof(*result));
        prove_one(engine, lemma_id, o, result);
    });
}

int sid_prove_resume(sid_engine* engine, int lemma_id, const sid_prove_opts* opts, const char* checkpoint_path,
                     sid_result* result) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(!result || !checkpoint_path) fail(SID_ERR_INVALID, "null argument");
        sid_prove_opts o;
        if(opts) o = *opts; else sid_prove_opts_default(&o);
        check_precision(o.precision);
        ProofState ps;
        read_checkpoint(checkpoint_path, ps);
        if(ps.fingerprint != l->ir.fingerprint) fail(SID_ERR_INVALID, "checkpoint %s belongs to another lemma", checkpoint_path);
        if(int(ps.nargs) != l->ir.nargs) fail(SID_ERR_INVALID, "checkpoint %s has %u variables", checkpoint_path, ps.nargs);
        if(ps.generations != o.generation_count) {
            fail(SID_ERR_INVALID, "checkpoint %s was written with generation_count %u", checkpoint_path, ps.generations);
        }
        set_device(engine);
        std::memset(result, 0, sizeof(*result));
        prove_one(engine, lemma_id, o, result, 0, nullptr, &ps);
    });
}

int sid_prove_bundle(sid_engine* engine, int n, const int* lemma_ids, const sid_prove_opts* opts, sid_result* results) {
    return guarded([&] {
        if(!engine || !lemma_ids || !results) fail(SID_ERR_INVALID, "null argument");
        if(n < 1 || n > kBundleMax) fail(SID_ERR_INVALID, "a bundle proves 1 to %d lemmas, not %d", kBundleMax, n);
        sid_prove_opts o;
        if(opts) o = *opts; else sid_prove_opts_default(&o);
        check_precision(o.precision);
        if(o.generation_count > 250) fail(SID_ERR_INVALID, "generation_count too large");
        if(o.max_iterations_per_node > 1 || o.checkpoint_path || o.stop_after_steps || o.progress || o.part_count > 1) {
            fail(SID_ERR_UNSUPPORTED, "bundled proofs take no node re-iteration, checkpoints, progress or parts");
        }
        std::vector<int> ids(lemma_ids, lemma_ids + n);
        std::vector<std::uint64_t> fps;
        for(int j = 0; j < n; ++j) {
            Lemma* l = get_lemma(engine, ids[std::size_t(j)]);
            if(l->k->is_f32) fail(SID_ERR_UNSUPPORTED, "bundles hold double lemmas; '%s' is a float lemma", l->ir.name.c_str());
            for(int k = 0; k < j; ++k) {
                if(ids[std::size_t(k)] == ids[std::size_t(j)]) fail(SID_ERR_INVALID, "lemma %d appears twice", ids[std::size_t(j)]);
            }
            fps.push_back(l->ir.fingerprint);
        }
        // the compiled bundle of exactly these lemmas, in any order
        const BundleKernels* bk = nullptr;
        std::vector<int> pos(std::size_t(n), -1);
        for(int b = 0; b < kNumBundles && !bk; ++b) {
            const BundleKernels* c = kAllBundles[b];
            if(!c || c->n != n) continue;
            std::vector<int> p(std::size_t(n), -1);
            std::vector<bool> used(std::size_t(n), false);
            bool all = true;
            for(int j = 0; j < n && all; ++j) {
                all = false;
                for(int i = 0; i < n; ++i) {
                    if(!used[std::size_t(i)] && c->fingerprints[i] == fps[std::size_t(j)]) {
                        used[std::size_t(i)] = true;
                        p[std::size_t(j)] = i;
                        all = true;
                        break;
                    }
                }
            }
            if(all) { bk = c; pos = p; }
        }
        if(!bk) fail(SID_ERR_NOT_COMPILED, "no bundle kernel was generated for these %d lemmas; list them in a bundles.txt", n);
        set_device(engine);
        std::memset(results, 0, sizeof(sid_result) * std::size_t(n));
        prove_bundle(engine, bk, ids, pos, o, results);
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
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        eval_batch_ordered(engine, l, lo, hi, n, out_lo, out_hi, verdict, s);
    });
}

int sid_eval_batch_plain_device(sid_engine* engine, int lemma_id, const double* lo, const double* hi, uint64_t n,
                                double* out_lo, double* out_hi, int8_t* verdict, void* stream) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(l->k->is_f32) fail(SID_ERR_UNSUPPORTED, "batch evaluation supports double lemmas");
        if(n > 0 && (!lo || !hi || !out_lo || !out_hi || !verdict)) fail(SID_ERR_INVALID, "null buffer");
        set_device(engine);
        eval_batch_ordered(engine, l, lo, hi, n, out_lo, out_hi, verdict, static_cast<cudaStream_t>(stream), 0, true);
    });
}

int sid_lemma_operands(sid_engine* engine, int lemma_id, uint32_t* count) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(!count) fail(SID_ERR_INVALID, "null output");
        *count = std::uint32_t(l->k->n_operands);
    });
}

int sid_eval_operands_device(sid_engine* engine, int lemma_id, const double* lo, const double* hi, uint64_t n,
                             int use_float, double* out_lohi, int8_t* out_undefined, void* stream) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(n == 0 || l->k->n_operands == 0) return;
        if(!lo || !hi || !out_lohi || !out_undefined) fail(SID_ERR_INVALID, "null buffer");
        set_device(engine);
        cuda_check(l->k->eval_operands(use_float ? 1 : 0, lo, hi, n, 0, reinterpret_cast<double2*>(out_lohi), out_undefined,
                                       static_cast<cudaStream_t>(stream)),
                   "operand kernel");
    });
}

int sid_eval_batch(sid_engine* engine, int lemma_id, const double* lo, const double* hi, uint64_t n,
                   double* out_lo, double* out_hi, int8_t* verdict) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(l->k->is_f32) fail(SID_ERR_UNSUPPORTED, "batch evaluation supports double lemmas");
        set_device(engine);
        const int nargs = l->ir.nargs;
        const std::size_t cnt = std::size_t(n) * std::size_t(nargs);
        engine->batch_in_lo.reserve(cnt);
        engine->batch_in_hi.reserve(cnt);
        engine->batch_out_lo.reserve(cnt);
        engine->batch_out_hi.reserve(cnt);
        engine->batch_verdict.reserve(std::size_t(n));
        // Pipeline in chunks: copies in on copy_in, ordering + evaluation on the engine stream, copies out on
        // copy_out, so transfers of one chunk overlap the evaluation of its neighbours. Nothing overlaps the
        // copy-in of the first chunk or the copy-out of the last, so large batches start and end with
        // chunks of 1/8, 1/8, 1/4, 1/2 of the steady-state size.
        const std::uint64_t chunk = kBatchChunk;
        std::vector<std::uint64_t> lens;
        if(n >= 4 * chunk) {
            const std::uint64_t ramp[4] = {chunk / 8, chunk / 8, chunk / 4, chunk / 2};
            for(std::uint64_t r : ramp) lens.push_back(r);
            for(std::uint64_t rest = n - 2 * chunk; rest > 0;) {
                const std::uint64_t l = std::min(chunk, rest);
                lens.push_back(l);
                rest -= l;
            }
            for(int k = 3; k >= 0; --k) lens.push_back(ramp[k]);
        } else {
            for(std::uint64_t c0 = 0; c0 < n; c0 += chunk) lens.push_back(std::min(chunk, n - c0));
        }
        const std::size_t pitch = std::size_t(n) * sizeof(double);   // one row per variable
        std::vector<cudaEvent_t> evs;
        auto event = [&]() {
            cudaEvent_t e;
            cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
            evs.push_back(e);
            return e;
        };
        try {
            std::uint64_t c0 = 0;
            for(const std::uint64_t len : lens) {
                const std::size_t row = std::size_t(len) * sizeof(double);
                cuda_check(cudaMemcpy2DAsync(engine->batch_in_lo.p + c0, pitch, lo + c0, pitch, row, std::size_t(nargs),
                                             cudaMemcpyHostToDevice, engine->copy_in), "H2D");
                cuda_check(cudaMemcpy2DAsync(engine->batch_in_hi.p + c0, pitch, hi + c0, pitch, row, std::size_t(nargs),
                                             cudaMemcpyHostToDevice, engine->copy_in), "H2D");
                cudaEvent_t in_done = event();
                cuda_check(cudaEventRecord(in_done, engine->copy_in), "event record");
                cuda_check(cudaStreamWaitEvent(engine->stream, in_done, 0), "stream wait");
                eval_batch_ordered(engine, l, engine->batch_in_lo.p + c0, engine->batch_in_hi.p + c0, len,
                                   engine->batch_out_lo.p + c0, engine->batch_out_hi.p + c0, engine->batch_verdict.p + c0,
                                   engine->stream, n);
                cudaEvent_t eval_done = event();
                cuda_check(cudaEventRecord(eval_done, engine->stream), "event record");
                cuda_check(cudaStreamWaitEvent(engine->copy_out, eval_done, 0), "stream wait");
                cuda_check(cudaMemcpy2DAsync(out_lo + c0, pitch, engine->batch_out_lo.p + c0, pitch, row, std::size_t(nargs),
                                             cudaMemcpyDeviceToHost, engine->copy_out), "D2H");
                cuda_check(cudaMemcpy2DAsync(out_hi + c0, pitch, engine->batch_out_hi.p + c0, pitch, row, std::size_t(nargs),
                                             cudaMemcpyDeviceToHost, engine->copy_out), "D2H");
                cuda_check(cudaMemcpyAsync(verdict + c0, engine->batch_verdict.p + c0, std::size_t(len),
                                           cudaMemcpyDeviceToHost, engine->copy_out), "D2H");
                c0 += len;
            }
            cuda_check(cudaStreamSynchronize(engine->copy_out), "eval batch sync");
        } catch(...) {
            cudaStreamSynchronize(engine->copy_in);
            cudaStreamSynchronize(engine->stream);
            cudaStreamSynchronize(engine->copy_out);
            for(cudaEvent_t e : evs) cudaEventDestroy(e);
            throw;
        }
        for(cudaEvent_t e : evs) cudaEventDestroy(e);
    });
}

int sid_debug_inject_failure(int kind, int64_t countdown) {
    return guarded([&] {
        if(kind != SID_INJECT_ALLOC && kind != SID_INJECT_LAUNCH) fail(SID_ERR_INVALID, "unknown injection kind %d", kind);
        if(countdown < 0) fail(SID_ERR_INVALID, "negative countdown");
        g_inject_countdown[kind].store((long long)countdown);
    });
}

constexpr double kLoopTuneBelowSeconds = 0.005;   // proofs shorter than this also try the device proof loop

int sid_lemma_autotune(sid_engine* engine, int lemma_id, double max_seconds, sid_tuning* out) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(!out) fail(SID_ERR_INVALID, "null output");
        set_device(engine);
        sid_tuning t{};
        t.step_elements = std::int64_t(kDefaultStep);
        t.fp32_level_mask = ~0u;
        t.escalation_threshold = 1.01f;
        const int levels = int(l->ir.dynamic_splits().size() + l->ir.static_splits().size());
        t.levels = levels;
        for(int k = 0; k < SID_MAX_LEVELS; ++k) t.level_escalation[k] = -1.0;
        sid_prove_opts o;
        sid_prove_opts_default(&o);
        o.precision = SID_PRECISION_FP32_ESCALATE;
        o.max_criticals_kept = 0;
        double spent = 0;
        std::uint32_t noprop = ~0u;   // the default precision form: no float propagation
        t.fp32_noprop_mask = ~0u;
        auto timed = [&](std::uint64_t step, std::uint32_t mask, sid_result& best) {
            for(int rep = 0; rep < 2; ++rep) {
                sid_result r{};
                prove_one(engine, lemma_id, o, &r, step, &mask, nullptr, &noprop);
                spent += r.seconds;
                if(rep == 0 || r.seconds < best.seconds) best = r;
            }
        };
        // baseline: every level on the float pass, the default step; per-level escalation rates
        sid_result base{};
        const std::uint32_t all = ~0u;
        timed(kDefaultStep, all, base);
        t.default_seconds = base.seconds;
        t.seconds = base.seconds;
        t.candidates = 1;
        if(l->k->filter_f32 != nullptr) {
            const auto stats = engine->prove_lanes[lemma_id]->level_stats();
            for(int k = 0; k < std::min(levels, SID_MAX_LEVELS); ++k) {
                if(stats[std::size_t(k)].first) {
                    t.level_escalation[k] = double(stats[std::size_t(k)].second) / double(stats[std::size_t(k)].first);
                }
            }
            auto same = [&](const sid_result& r) {
                return r.num_cuboids == base.num_cuboids && r.num_leaf_cuboids == base.num_leaf_cuboids &&
                       r.num_critical_cuboids == base.num_critical_cuboids;
            };
            // candidate masks from thresholds on the measured rates
            std::vector<std::pair<float, std::uint32_t>> masks;
            for(float thr : {0.95f, 0.8f, 0.6f}) {
                std::uint32_t m = ~0u;
                for(int k = 0; k < std::min(levels, SID_MAX_LEVELS); ++k) {
                    if(t.level_escalation[k] > double(thr)) m &= ~(1u << k);
                }
                bool seen = m == all;
                for(const auto& e : masks) seen = seen || e.second == m;
                if(!seen) masks.emplace_back(thr, m);
            }
            for(const auto& cand : masks) {
                if(spent > max_seconds) break;
                sid_result r{};
                timed(kDefaultStep, cand.second, r);
                ++t.candidates;
                if(same(r) && r.seconds < t.seconds) {
                    t.seconds = r.seconds;
                    t.fp32_level_mask = cand.second;
                    t.escalation_threshold = cand.first;
                }
            }
            // float passes with propagation: on every level, or on all but the innermost static level (whose
            // split-invariant form is usually the fastest float pass)
            const std::uint32_t innermost = levels > 0 ? 1u << std::min(levels - 1, SID_MAX_LEVELS - 1) : 0u;
            for(std::uint32_t cand : {0u, innermost}) {
                if(spent > max_seconds || cand == t.fp32_noprop_mask) continue;
                sid_result r{};
                noprop = cand;
                timed(kDefaultStep, t.fp32_level_mask, r);
                ++t.candidates;
                if(same(r) && r.seconds < t.seconds) {
                    t.seconds = r.seconds;
                    t.fp32_noprop_mask = cand;
                }
            }
            noprop = t.fp32_noprop_mask;
            for(std::uint64_t step : {std::uint64_t(1) << 15, std::uint64_t(1) << 17, std::uint64_t(1) << 14}) {
                if(spent > max_seconds) break;
                sid_result r{};
                timed(step, t.fp32_level_mask, r);
                ++t.candidates;
                if(same(r) && r.seconds < t.seconds) {
                    t.seconds = r.seconds;
                    t.step_elements = std::int64_t(step);
                }
            }
            // the device proof loop, for proofs short enough that launches and host reads dominate; there a level
            // of a few hundred children may also be done sooner by the dense double kernel (float-first rows) than
            // by the float pass and its two extra grid barriers, so the loop is also tried with no float pass
            if(t.seconds < kLoopTuneBelowSeconds) {
                const std::uint32_t chosen = t.fp32_level_mask;
                for(std::uint32_t mask : {chosen, 0u}) {
                    for(unsigned blocks : {38u, 152u, 608u}) {
                        if(spent > max_seconds) break;
                        sid_result r{};
                        o.device_loop_blocks = blocks;
                        timed(std::uint64_t(t.step_elements), mask, r);
                        o.device_loop_blocks = 0;
                        ++t.candidates;
                        if(same(r) && r.seconds < t.seconds) {
                            t.seconds = r.seconds;
                            t.loop_blocks = blocks;
                            t.fp32_level_mask = mask;
                        }
                    }
                }
            }
        }
        l->tuning = t;
        l->tuned = true;
        *out = t;
    });
}

int sid_lemma_batch_order(sid_engine* engine, int lemma_id, int mode, double* double_share) {
    return guarded([&] {
        Lemma* l = get_lemma(engine, lemma_id);
        if(mode > SID_BATCH_ORDER_OFF) fail(SID_ERR_INVALID, "unknown batch order mode %d", mode);
        set_device(engine);
        if(mode >= 0) l->batch_order = mode;
        poll_batch_sample(l);
        if(double_share) *double_share = l->batch_double_share;
    });
}

int sid_eval_batch_profile(sid_engine* engine, int enable) {
    return guarded([&] {
        if(!engine) fail(SID_ERR_INVALID, "null engine");
        set_device(engine);
        engine->batch_profile = enable != 0;
        if(!enable) profile_clear(engine);
    });
}

int sid_eval_batch_profile_read(sid_engine* engine, uint64_t* calls, double* order_ms, double* eval_ms,
                                uint64_t* launches) {
    return guarded([&] {
        if(!engine || !calls || !order_ms || !eval_ms) fail(SID_ERR_INVALID, "null argument");
        if(launches) *launches = engine->batch_launches;
        engine->batch_launches = 0;
        set_device(engine);
        *calls = 0;
        *order_ms = 0;
        *eval_ms = 0;
        const std::size_t k = engine->batch_events.size() / 4 * 4;
        for(std::size_t i = 0; i < k; i += 4) {
            cuda_check(cudaEventSynchronize(engine->batch_events[i + 3]), "profile event wait");
            float a = 0, b = 0, c = 0;
            cuda_check(cudaEventElapsedTime(&a, engine->batch_events[i], engine->batch_events[i + 1]), "profile time");
            cuda_check(cudaEventElapsedTime(&b, engine->batch_events[i + 1], engine->batch_events[i + 2]), "profile time");
            cuda_check(cudaEventElapsedTime(&c, engine->batch_events[i + 2], engine->batch_events[i + 3]), "profile time");
            *order_ms += a + c;
            *eval_ms += b;
            *calls += 1;
        }
        profile_clear(engine);
    });
}

void sid_server_opts_default(sid_server_opts* o) {
    if(!o) return;
    std::memset(o, 0, sizeof(*o));
    o->memory_budget_bytes = std::uint64_t(16) << 30;
    o->step_elements = std::int64_t(kDefaultStep);
    o->precision = SID_PRECISION_FP32_ESCALATE;
    o->generation_count = 8;
    o->max_criticals_per_request = 1024;
    o->max_requests_per_lane = kDefaultSlots;
    o->max_iterations_per_node = 1;
    o->iteration_volume_criterion = 0.25f;
    o->iteration_single_dimension_criterion = 0.66f;
}

int sid_server_create(sid_engine* engine, const sid_server_opts* opts, sid_server** out) {
    return guarded([&] {
        if(!engine || !out) fail(SID_ERR_INVALID, "null argument");
        auto s = std::make_unique<sid_server>();
        s->eng = engine;
        if(opts) s->opts = *opts; else sid_server_opts_default(&s->opts);
        check_precision(s->opts.precision);
        if(s->opts.generation_count == 0) s->opts.generation_count = 8;
        if(s->opts.generation_count > 250) fail(SID_ERR_INVALID, "generation_count too large");
        *out = s.release();
    });
}

void sid_server_destroy(sid_server* server) {
    if(!server) return;
    {
        std::lock_guard<std::mutex> lk(server->mu);
        server->stopping = true;
        for(auto& w : server->workers) w.second->cv.notify_all();
    }
    for(auto& w : server->workers) {
        if(w.second->th.joinable()) w.second->th.join();
    }
    delete server;
}

int sid_submit(sid_server* server, int lemma_id, const double* boxes, uint64_t nboxes, uint64_t* request_id) {
    return guarded([&] {
        if(!server || !request_id) fail(SID_ERR_INVALID, "null argument");
        Lemma* lem = get_lemma(server->eng, lemma_id);
        if(boxes && nboxes == 0) fail(SID_ERR_INVALID, "empty sub-box request");
        if(boxes && nboxes > (std::uint64_t(1) << 31)) fail(SID_ERR_INVALID, "too many sub-boxes");
        auto r = std::make_unique<Request>();
        r->lem = lem;
        r->lemma_id = lemma_id;
        r->full = boxes == nullptr;
        if(boxes) {
            r->nboxes = nboxes;
            r->boxes.assign(boxes, boxes + 2 * nboxes * std::uint64_t(lem->ir.nargs));
            for(std::uint64_t i = 0; i < nboxes * std::uint64_t(lem->ir.nargs); ++i) {
                const double lo = r->boxes[std::size_t(2 * i)], hi = r->boxes[std::size_t(2 * i + 1)];
                if(!(lo <= hi)) fail(SID_ERR_INVALID, "sub-box %llu has an empty or NaN range",
                                     (unsigned long long)(i / std::uint64_t(lem->ir.nargs)));
            }
        }
        r->generations = server->opts.generation_count;
        r->crit_cap = server->opts.max_criticals_per_request;
        r->t_submit = Clock::now();
        std::lock_guard<std::mutex> lk(server->mu);
        if(server->stopping) fail(SID_ERR_INVALID, "server is stopping");
        r->id = server->next_id++;
        Request* raw = r.get();
        server->reqs[r->id] = std::move(r);
        auto& w = server->workers[lemma_id];
        if(!w) {
            w.reset(new sid_server::Worker);
            w->lemma_id = lemma_id;
            sid_server::Worker* wp = w.get();
            w->th = std::thread([server, wp] { server->worker_loop(wp); });
        }
        w->pending.push_back(raw);
        w->cv.notify_all();
        *request_id = raw->id;
    });
}

int sid_request_poll(sid_server* server, uint64_t request_id, sid_request_status* status) {
    return guarded([&] {
        if(!server || !status) fail(SID_ERR_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(server->mu);
        auto it = server->reqs.find(request_id);
        if(it == server->reqs.end()) fail(SID_ERR_INVALID, "unknown request %llu", (unsigned long long)request_id);
        sid_server::fill_status(*it->second, status);
        if(it->second->state == SID_REQ_FAILED) {
            fail(it->second->error_status, "request failed: %s", it->second->error.c_str());
        }
    });
}

int sid_request_wait(sid_server* server, uint64_t request_id, int timeout_ms, sid_request_status* status) {
    return guarded([&] {
        if(!server || !status) fail(SID_ERR_INVALID, "null argument");
        std::unique_lock<std::mutex> lk(server->mu);
        auto it = server->reqs.find(request_id);
        if(it == server->reqs.end()) fail(SID_ERR_INVALID, "unknown request %llu", (unsigned long long)request_id);
        Request* r = it->second.get();
        auto finished = [&] { return r->state == SID_REQ_DONE || r->state == SID_REQ_FAILED; };
        if(timeout_ms < 0) server->cv_done.wait(lk, finished);
        else server->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), finished);
        sid_server::fill_status(*r, status);
        if(r->state == SID_REQ_FAILED) fail(r->error_status, "request failed: %s", r->error.c_str());
        if(!finished()) fail(SID_ERR_TIMEOUT, "request %llu not finished after %d ms", (unsigned long long)request_id,
                             timeout_ms);
    });
}

int sid_request_criticals(sid_server* server, uint64_t request_id, double* out, uint64_t capacity, uint64_t* n_out) {
    return guarded([&] {
        if(!server) fail(SID_ERR_INVALID, "null server");
        std::lock_guard<std::mutex> lk(server->mu);
        auto it = server->reqs.find(request_id);
        if(it == server->reqs.end()) fail(SID_ERR_INVALID, "unknown request %llu", (unsigned long long)request_id);
        Request* r = it->second.get();
        if(r->state != SID_REQ_DONE) fail(SID_ERR_INVALID, "request %llu has not finished", (unsigned long long)request_id);
        const std::uint64_t per = 2 * std::uint64_t(r->lem->ir.nargs);
        const std::uint64_t have = r->criticals.size() / per;
        const std::uint64_t n = std::min(have, capacity);
        if(n && !out) fail(SID_ERR_INVALID, "null output");
        if(n) std::memcpy(out, r->criticals.data(), n * per * sizeof(double));
        if(n_out) *n_out = n;
        if(have > capacity) fail(SID_ERR_CAPACITY, "%llu criticals stored, capacity %llu",
                                 (unsigned long long)have, (unsigned long long)capacity);
    });
}

int sid_request_release(sid_server* server, uint64_t request_id) {
    return guarded([&] {
        if(!server) fail(SID_ERR_INVALID, "null server");
        std::lock_guard<std::mutex> lk(server->mu);
        auto it = server->reqs.find(request_id);
        if(it == server->reqs.end()) fail(SID_ERR_INVALID, "unknown request %llu", (unsigned long long)request_id);
        const int st = it->second->state;
        if(st != SID_REQ_DONE && st != SID_REQ_FAILED) fail(SID_ERR_INVALID, "request %llu has not finished",
                                                            (unsigned long long)request_id);
        server->reqs.erase(it);
    });
}

} // extern "C"
