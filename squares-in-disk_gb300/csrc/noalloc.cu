// Allocation-free leaf-hull entry point (sid_leaf_hull_noalloc, see include/sid.h).
//
// Runs the innermost static level of the prover core over caller-provided parent cuboids and joins the
// surviving leaves of each parent into its hull -- the same level kernel the proof uses
// (k_level in MODE_HULL), but with its scratch (the per-parent hull accumulators and the leaf counter)
// taken from a fixed, file-scope device array instead of engine allocations. Nothing here calls
// cudaMalloc, cudaFree or any other allocating routine, on the host or on the device.
#include <cstdint>
#include <cstdio>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/sid.h"
#include "engine.cuh"
#include "engine_internal.hpp"

namespace {

using namespace sid;

// 8 MiB per device, held from library load until process exit.
constexpr std::size_t kScratchBytes = std::size_t(8) << 20;
constexpr std::size_t kScratchWords = kScratchBytes / sizeof(unsigned long long);
// header: words 0..12 the request record the level kernel counts into (ReqDev: word 1 = leaves),
// word 16 the list-overflow flag; keys start at word 32
constexpr std::size_t kHeaderWords = 32;
static_assert(sizeof(ReqDev) <= 16 * sizeof(unsigned long long), "request record must fit the header");
// four accumulator arrays (lo key, hi key, first-zero lo, first-zero hi) of n * nargs words each
constexpr std::uint64_t kMaxItemVars = (kScratchWords - kHeaderWords) / 4;

static __device__ __align__(256) unsigned long long g_leaf_hull_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned long long* g_scratch_addr[kMaxDevices] = {};

/// Decode each parent's accumulators (order keys, first-zero sign) into its hull.
__global__ void k_leaf_hull_decode(const unsigned long long* scratch, std::uint64_t n, int nargs, double2* hulls,
                                   std::uint8_t* nonempty, unsigned long long* leaves_out) {
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i == 0 && leaves_out) *leaves_out = reinterpret_cast<const ReqDev*>(scratch)->cnt[RC_LEAVES];
    if(i >= n) return;
    const std::uint64_t m = n * std::uint64_t(nargs);
    const unsigned long long* lo = scratch + kHeaderWords;
    const unsigned long long* hi = lo + m;
    const unsigned long long* zlo = hi + m;
    const unsigned long long* zhi = zlo + m;
    const std::uint64_t b = i * std::uint64_t(nargs);
    if(lo[b] == ~0ull) {
        nonempty[i] = 0;
        return;
    }
    nonempty[i] = 1;
    for(int v = 0; v < nargs; ++v) {
        double l = key_value(lo[b + v]);
        double h = key_value(hi[b + v]);
        if(l == 0.0) l = (zlo[b + v] & 1ull) ? -0.0 : 0.0;
        if(h == 0.0) h = (zhi[b + v] & 1ull) ? -0.0 : 0.0;
        hulls[std::uint64_t(v) * n + i] = make_double2(l, h);
    }
}

int fail_status(int status, const char* msg) {
    internal_set_error(msg);
    return status;
}

int cuda_status(cudaError_t e, const char* what) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return fail_status(e == cudaErrorMemoryAllocation ? SID_ERR_NOMEM : SID_ERR_CUDA, buf);
}

} // namespace

extern "C" int sid_leaf_hull_noalloc(sid_engine* engine, int lemma_id, const double* boxes, uint64_t n,
                                     double* hulls, uint8_t* nonempty, unsigned long long* leaves, void* stream) {
    LemmaView view;
    if(internal_lemma_view(engine, lemma_id, &view) != SID_OK) {
        return fail_status(SID_ERR_INVALID, "sid_leaf_hull_noalloc: unknown engine or lemma id");
    }
    if(view.last_static_arg < 0) {
        return fail_status(SID_ERR_UNSUPPORTED, "sid_leaf_hull_noalloc: the lemma has no static split");
    }
    if(view.kernels->is_f32) {
        return fail_status(SID_ERR_UNSUPPORTED, "sid_leaf_hull_noalloc: supports double lemmas (as sid_eval_batch)");
    }
    if(view.device < 0 || view.device >= kMaxDevices) return fail_status(SID_ERR_INVALID, "device id out of range");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if(n == 0) {
        // no parents: no leaves
        if(!leaves) return SID_OK;
        cudaError_t e = cudaSetDevice(view.device);
        if(e == cudaSuccess) e = cudaMemsetAsync(leaves, 0, sizeof(unsigned long long), s);
        return e == cudaSuccess ? SID_OK : cuda_status(e, "cudaMemsetAsync(leaves)");
    }
    if(!boxes || !hulls || !nonempty) return fail_status(SID_ERR_INVALID, "sid_leaf_hull_noalloc: null buffer");
    if(n > kMaxItemVars / std::uint64_t(view.nargs)) {
        char buf[256];
        std::snprintf(buf, sizeof(buf),
                      "sid_leaf_hull_noalloc: %llu cuboids x %d variables exceeds the allocation-free limit of "
                      "%llu cuboid-variables (8 MiB device scratch); split the call",
                      (unsigned long long)n, view.nargs, (unsigned long long)kMaxItemVars);
        return fail_status(SID_ERR_CAPACITY, buf);
    }

    cudaError_t e = cudaSetDevice(view.device);
    if(e != cudaSuccess) return cuda_status(e, "cudaSetDevice");
    unsigned long long* scratch = nullptr;
    {
        // one-time set-up per device: the device address of the file-scope scratch array (kept for the life of
        // the process; a device reset after this point is not supported, sid.h says so)
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if(!g_scratch_addr[view.device]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_leaf_hull_scratch);
            if(e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(leaf hull scratch)");
            g_scratch_addr[view.device] = static_cast<unsigned long long*>(p);
        }
        scratch = g_scratch_addr[view.device];
    }

    const std::uint64_t m = n * std::uint64_t(view.nargs);
    unsigned long long* lo = scratch + kHeaderWords;
    // the array keeps the previous call's contents: reset counters and accumulators
    if((e = cudaMemsetAsync(scratch, 0, kHeaderWords * sizeof(unsigned long long), s)) != cudaSuccess ||
       (e = cudaMemsetAsync(lo, 0xff, m * sizeof(unsigned long long), s)) != cudaSuccess ||
       (e = cudaMemsetAsync(lo + m, 0, m * sizeof(unsigned long long), s)) != cudaSuccess ||
       (e = cudaMemsetAsync(lo + 2 * m, 0xff, 2 * m * sizeof(unsigned long long), s)) != cudaSuccess) {
        return cuda_status(e, "cudaMemsetAsync(leaf hull scratch)");
    }

    LevelArgs a{};
    a.in_box = reinterpret_cast<const double2*>(boxes);
    a.in_stride = n;
    a.in_begin = 0;
    a.n_in = n;
    a.var = view.last_static_arg;
    a.nsub = view.last_static_subdivisions;
    a.it_limit = view.nargs;
    a.rec_limit = 4;
    a.row_begin = view.last_static_arg;
    a.row_end = view.nargs;
    a.req = reinterpret_cast<ReqDev*>(scratch);   // one request, tag 0, zeroed above
    a.tag_value = 0;
    a.count_cuboids = false;
    a.overflow = reinterpret_cast<unsigned int*>(scratch + 16);
    a.hull_lo = lo;
    a.hull_hi = lo + m;
    a.hull_zlo = lo + 2 * m;
    a.hull_zhi = lo + 3 * m;
    if((e = view.kernels->level(MODE_HULL, a, s)) != cudaSuccess) return cuda_status(e, "leaf hull level kernel");
    k_leaf_hull_decode<<<unsigned((n + 127) / 128), 128, 0, s>>>(scratch, n, view.nargs,
                                                                 reinterpret_cast<double2*>(hulls), nonempty, leaves);
    if((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e, "leaf hull decode kernel");
    return SID_OK;
}
