// Frontier kernels of the GB300 prover engine, templated on a generated lemma type L.
//
// The reference processes one queue element at a time on a CPU thread, recursing over the static
// splits (cpu_prover/cpu_prover_core.hpp:221-256) and the dynamic re-splits
// (prover/pd_impl_split_into.hpp:37-66). Here each recursion level is one data-parallel launch over
// all (item, child) pairs of a whole batch of elements:
//   * one thread per child: split the parent's variable (splitter.hpp:44-59), propagate bounds with
//     the reference's worklist semantics, test the constraint rows;
//   * survivors of inner levels are compacted into the next level's list with one atomic per warp
//     (ballot + popc); survivors of the innermost static level are joined into their element's hull
//     with lock-free 64-bit atomics (ordered keys), or stored as criticals in the final generation.
// Counts are order independent (the reference sums per-thread counters), so the level-synchronous
// traversal reproduces them exactly.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "interval.cuh"

namespace sid {

enum BoundResult : int { B_NONE = 0, B_LB = 1, B_UB = 2, B_BOTH = 3, B_EMPTY = 4 };

/// Per-request counters on the device (indices into ReqDev::cnt).
enum ReqCounter : int {
    RC_CUBOIDS = 0,      // cuboids considered
    RC_LEAVES = 1,       // leaf cuboids
    RC_CRITICALS = 2,    // critical cuboids (final generation)
    RC_ESCALATED = 3,    // precision form: children evaluated in double
    RC_QSIZE = 4,        // elements in the request's queue (appended with atomics)
    RC_OVERFLOW = 5,     // a queue append did not fit (the host sizes queues so that this stays 0)
    RC_REPEATED = 6,     // nodes re-iterated on their hull (max_iterations_per_node > 1)
    RC_N = 7
};

/// Device state of one request (a proof, or a set of sub-boxes of a lemma): counters, its frontier queue
/// (a LIFO stack: nargs columns of qcap double2 plus a depth byte) and its critical-box store.
struct ReqDev {
    unsigned long long cnt[RC_N];
    double2* qbox;
    std::uint8_t* qdepth;
    unsigned long long qcap;
    double* crit;                      // 2*nargs doubles per stored critical
    unsigned long long crit_cap;
    unsigned int generations;          // elements of depth >= generations are final
    unsigned int pad;
};

/// Applies a bound function value v to the target interval (CompileTimeBound::apply_to,
/// constraints_to_bounds/compile_time_bound.hpp:42-85).
template<int DIR, bool DEFINED, class T> __device__ __forceinline__ int apply_to(Iv<T>& t, const Iv<T>& v) {
    if(!DEFINED && v.und) return B_NONE;
    if(DIR == 1) {
        if(v.hi < t.hi) { t.hi = v.hi; return v.hi < t.lo ? B_EMPTY : B_UB; }
        return B_NONE;
    } else if(DIR == 2) {
        if(v.lo > t.lo) { t.lo = v.lo; return v.lo > t.hi ? B_EMPTY : B_LB; }
        return B_NONE;
    } else {
        int ch = B_NONE;
        if(v.hi < t.hi) { t.hi = v.hi; ch |= B_UB; }
        if(v.lo > t.lo) { t.lo = v.lo; ch |= B_LB; }
        return (t.hi < t.lo) ? B_EMPTY : ch;
    }
}

template<class T> __device__ __forceinline__ Iv<T> cst(double dlo, double dhi, float flo, float fhi, bool und);
template<> __device__ __forceinline__ Iv<double> cst<double>(double dlo, double dhi, float, float, bool und) {
    return {dlo, dhi, und};
}
template<> __device__ __forceinline__ Iv<float> cst<float>(double, double, float flo, float fhi, bool und) {
    return {flo, fhi, und};
}

template<class L, class T, bool DEFER> __device__ int propagate_packed(int arg, Iv<T>* box, int it_limit, int rec_limit);

/// Worklist bound propagation after a change of variable `arg` (both bounds), with the reference's
/// FIFO order, de-duplication, per-bound recursion limit and "unstable" re-seeding between
/// iterations (bound_propagation/iterated_recursive.hpp:59-131, dynamic_bound_application.hpp:104-123,
/// index_queue_set.hpp:38-101). Returns true if the box became empty.
template<class L, class T> __device__ bool propagate(int arg, Iv<T>* box, int it_limit, int rec_limit) {
    constexpr int NB = L::NBOUNDS;
    if(NB == 0) return false;
    if constexpr(NB <= 16) return propagate_packed<L, T, false>(arg, box, it_limit, rec_limit) == 1;
    const std::uint64_t seed = L::upd_both(arg);
    if(!seed) return false;
    std::uint8_t ring[NB > 0 ? NB : 1];
    std::uint8_t rec[NB > 0 ? NB : 1];
    std::uint8_t ulist[NB > 0 ? NB : 1];
    #pragma unroll
    for(int i = 0; i < NB; ++i) rec[i] = 0;
    std::uint64_t present = 0, unstable = 0;
    int qb = 0, qe = 0, qn = 0, nun = 0;
    for(std::uint64_t m = seed; m; m &= m - 1) {
        int a = __ffsll((long long)m) - 1;
        present |= (1ull << a);
        ring[qe] = std::uint8_t(a);
        qe = (qe + 1 == NB) ? 0 : qe + 1;
        ++qn;
    }
    for(int it = 0; it < it_limit; ++it) {
        while(qn > 0) {
            int k = ring[qb];
            present &= ~(1ull << k);
            qb = (qb + 1 == NB) ? 0 : qb + 1;
            --qn;
            int r = L::template apply_bound<T>(k, box);
            if(r == B_EMPTY) return true;
            if(r == B_NONE) continue;
            const int tgt = L::target(k);
            std::uint64_t upd = r == B_LB ? L::upd_lb(tgt) : (r == B_UB ? L::upd_ub(tgt) : L::upd_both(tgt));
            for(; upd; upd &= upd - 1) {
                int a = __ffsll((long long)upd) - 1;
                std::uint64_t bit = 1ull << a;
                if(rec[a] >= rec_limit) {
                    if(!(present & bit) && !(unstable & bit)) {
                        ulist[nun++] = std::uint8_t(a);
                        unstable |= bit;
                    }
                } else if(!(present & bit)) {
                    present |= bit;
                    ring[qe] = std::uint8_t(a);
                    qe = (qe + 1 == NB) ? 0 : qe + 1;
                    ++qn;
                    rec[a] += 1;
                }
            }
        }
        if(nun == 0) break;
        for(int j = 0; j < nun; ++j) {
            int a = ulist[j];
            std::uint64_t bit = 1ull << a;
            if(!(present & bit)) {
                present |= bit;
                ring[qe] = std::uint8_t(a);
                qe = (qe + 1 == NB) ? 0 : qe + 1;
                ++qn;
            }
        }
        #pragma unroll
        for(int i = 0; i < NB; ++i) rec[i] = 0;
        unstable = 0;
        nun = 0;
    }
    return false;
}

/// propagate for lemmas with at most 16 bounds, with the same order of bound applications, kept in
/// registers: the FIFO and the unstable list are 4-bit bound ids packed into one 64-bit word each (head in
/// the low nibble; a bound is queued at most once, so at most 16 entries), and the per-bound recursion
/// counters are bytes of two 64-bit words (a counter grows only while below rec_limit <= 255, so it never
/// carries into its neighbour). The byte arrays of the general form are indexed at run time and live in
/// local memory. Returns 1 if the box became empty, else 0; with DEFER, 2 as soon as the next bound to
/// apply is one of L::SLOW_BOUNDS (the box is then partly propagated, and the caller starts over elsewhere).
template<class L, class T, bool DEFER> __device__ int propagate_packed(int arg, Iv<T>* box, int it_limit, int rec_limit) {
    static_assert(L::NBOUNDS <= 16, "packed worklist holds 16 bound ids");
    const std::uint64_t seed = L::upd_both(arg);
    if(!seed) return 0;
    std::uint64_t q = 0, ul = 0, rec0 = 0, rec1 = 0;
    std::uint32_t present = 0, unstable = 0;
    int qn = 0, nun = 0;
    for(std::uint64_t m = seed; m; m &= m - 1) {
        const int a = __ffsll((long long)m) - 1;
        present |= 1u << a;
        q |= std::uint64_t(a) << (4 * qn);
        ++qn;
    }
    for(int it = 0; it < it_limit; ++it) {
        while(qn > 0) {
            const int k = int(q & 15u);
            if constexpr(DEFER) {
                if((L::SLOW_BOUNDS >> k) & 1u) return 2;
            }
            q >>= 4;
            --qn;
            present &= ~(1u << k);
            const int r = L::template apply_bound<T>(k, box);
            if(r == B_EMPTY) return 1;
            if(r == B_NONE) continue;
            const int tgt = L::target(k);
            std::uint64_t upd = r == B_LB ? L::upd_lb(tgt) : (r == B_UB ? L::upd_ub(tgt) : L::upd_both(tgt));
            for(; upd; upd &= upd - 1) {
                const int a = __ffsll((long long)upd) - 1;
                const std::uint32_t bit = 1u << a;
                const int sh = 8 * (a & 7);
                const int ra = int(((a < 8 ? rec0 : rec1) >> sh) & 0xffu);
                if(ra >= rec_limit) {
                    if(!(present & bit) && !(unstable & bit)) {
                        ul |= std::uint64_t(a) << (4 * nun);
                        ++nun;
                        unstable |= bit;
                    }
                } else if(!(present & bit)) {
                    present |= bit;
                    q |= std::uint64_t(a) << (4 * qn);
                    ++qn;
                    if(a < 8) rec0 += 1ull << sh;
                    else rec1 += 1ull << sh;
                }
            }
        }
        if(nun == 0) break;
        for(int j = 0; j < nun; ++j) {
            const int a = int((ul >> (4 * j)) & 15u);
            const std::uint32_t bit = 1u << a;
            if(!(present & bit)) {
                present |= bit;
                q |= std::uint64_t(a) << (4 * qn);
                ++qn;
            }
        }
        rec0 = rec1 = 0;
        unstable = 0;
        ul = 0;
        nun = 0;
    }
    return 0;
}

/// Lowest set bit of a non-zero mask, at compile time.
__host__ __device__ constexpr int ctz64(std::uint64_t m) { return (m & 1ull) ? 0 : 1 + ctz64(m >> 1); }

/// The start of a propagation whose seed (the bounds queued first, in increasing id order) is the compile-time
/// mask SEED: the seed bounds are applied in queue order, dispatched at compile time, while each leaves the box
/// unchanged. Until a bound changes the box nothing else is queued, so if a seed bound empties the box, or all
/// of them leave it unchanged, that is the result of the whole propagation (1: empty, 0: not empty). Returns -1
/// as soon as a seed bound changed the box without emptying it, or (with DEFER) before a seed bound of
/// L::SLOW_BOUNDS: the caller then runs the full propagation from the original box, which repeats these
/// applications first and continues exactly as it would have.
template<class L, class T, bool DEFER, std::uint64_t SEED> __device__ __forceinline__ int propagate_seed(Iv<T>* box) {
    if constexpr(SEED == 0) {
        return 0;
    } else {
        constexpr int k = ctz64(SEED);
        if constexpr(DEFER && ((L::SLOW_BOUNDS >> k) & 1ull)) {
            return -1;
        } else {
            const int r = L::template apply_bound_c<k, T>(box);
            if(r == B_EMPTY) return 1;
            if(r != B_NONE) return -1;
            return propagate_seed<L, T, DEFER, SEED & (SEED - 1)>(box);
        }
    }
}

/// Splitter::subrange (splitter.hpp:44-59): width (ub-lb)/n and points lb + i*w, all rounded down
/// like the reference's global rounding mode; the last point is exactly ub.
template<class T> __device__ __forceinline__ void split_child(T lb, T ub, int n, int i, T& lo, T& hi) {
    T w = Dir<T>::div_rd(Dir<T>::sub_rd(ub, lb), T(n));
    lo = (i >= n) ? ub : Dir<T>::add_rd(lb, Dir<T>::mul_rd(T(i), w));
    hi = (i + 1 >= n) ? ub : Dir<T>::add_rd(lb, Dir<T>::mul_rd(T(i + 1), w));
}

enum LevelMode : int {
    MODE_EMIT = 0,       // survivors go to the next level's list (path = path*n + child)
    MODE_HULL = 1,       // innermost static level: survivors are leaves joined into the element hull
    MODE_CRIT = 2,       // innermost static level of the final generation: survivors are criticals
    MODE_QUEUE = 3       // last dynamic level (root partition / re-split): survivors become queue elements
};

/// Order-preserving 64-bit keys for atomicMin/atomicMax on doubles; -0 and +0 share a key.
__device__ __forceinline__ unsigned long long order_key(double v) {
    long long b = __double_as_longlong(v == 0.0 ? 0.0 : v);
    return (unsigned long long)(b < 0 ? ~b : (b | (long long)0x8000000000000000ull));
}
__device__ __forceinline__ double key_value(unsigned long long k) {
    long long b = (long long)((k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k);
    return __longlong_as_double(b);
}

struct LevelArgs {
    // input items: boxes in structure-of-arrays layout box[v*stride + i] (lo, hi)
    const double2* in_box;
    std::uint64_t in_stride;
    const std::uint32_t* in_elem;     // element index of each item (nullptr: item index + elem_base)
    const std::uint64_t* in_path;     // leaf-order path (nullptr: 0)
    const std::uint8_t* in_depth;     // depth of each item (MODE_QUEUE; nullptr: depth_value)
    std::uint64_t in_begin, n_in;     // items [in_begin, in_begin + n_in)
    std::uint32_t elem_base;
    // request of each item: in_tag[item], else elem_tag[element], else tag_value
    const std::uint32_t* in_tag;
    const std::uint32_t* elem_tag;
    std::uint32_t tag_value;
    ReqDev* req;                      // per-request counters, queues (MODE_QUEUE), critical stores
    bool count_cuboids;               // every child counts as one cuboid of its request
    int var, nsub, it_limit, rec_limit;
    int row_begin, row_end;           // constraint rows to test (row_end <= row_begin: none)
    std::uint8_t depth_value;         // depth for MODE_QUEUE when in_depth is null
    std::uint8_t depth_add;           // added to the input depth for MODE_QUEUE
    // outputs (MODE_EMIT; MODE_QUEUE appends to the request's queue instead)
    double2* out_box;
    std::uint64_t out_stride, out_cap;
    std::uint32_t* out_elem;
    std::uint64_t* out_path;
    std::uint8_t* out_depth;
    std::uint32_t* out_tag;
    unsigned long long* out_count;    // slots already used on entry
    // hull (MODE_HULL): per element and variable
    unsigned long long* hull_lo;      // order keys, min
    unsigned long long* hull_hi;      // order keys, max
    unsigned long long* hull_zlo;     // (path<<1 | sign) of the first leaf whose lo is zero
    unsigned long long* hull_zhi;
    unsigned int* overflow;           // set when an output list would overflow
    // precision form (k_filter_f32 / k_level_esc): children [child_begin, child_begin + n_child) of
    // the items, the escalation list (child ids relative to child_begin) and its length
    std::uint64_t child_begin, n_child;
    std::uint32_t* esc;
    unsigned long long* esc_count;
    unsigned long long* esc_stat;     // if set, k_level_esc adds the list's length here (per-level statistics)
    // per-parent float data of the chunk (k_parent_f32): parents from item offset pitem_begin on
    const float2* pbox;               // pbox[v*pstride + j]; for the split variable (RD(lb), RU(ub))
    const float4* psplit;             // (RD(w), RU(lb), RU(w), 0) with w the double split width
    std::uint64_t pstride, pitem_begin;
    bool fp32_noprop;                 // float pass without bound propagation (rows only)
    bool float_rows;                  // k_level in double: test the rows in float first (precision form)
    std::uint32_t part_index, part_count;   // part_count > 1: only children c with c % part_count == part_index
    // split-invariant float pass (k_prelude_f32 / k_filter_hoisted): per parent j, stored subexpression
    // values hval[k*pstride + j] and their flags hbits[j] (kParentRefuted: no child can satisfy the rows)
    const float2* hval;
    const std::uint64_t* hbits;
    // dense levels: each child takes 1 << lane_shift lanes (one of them works), so that a small level's children
    // are spread over more warps (lane_shift_for)
    std::uint32_t lane_shift;
};

/// Lane shift of a dense level with `total` children on `threads` threads (one pass over the GPU's SM
/// sub-partitions: SMs x 128): the largest shift up to 5 (one child per warp) with which the children still fit.
/// GB300 runs a warp's FP64 instruction in its sub-partition's narrow FP64 unit for the same time however many
/// of its lanes take part, so a level of fewer children than the GPU has lanes finishes sooner with fewer
/// children per warp: each warp then executes only its own children's paths through the propagation
/// instead of the union of 32 divergent ones, on otherwise idle sub-partitions.
__host__ __device__ __forceinline__ std::uint32_t lane_shift_for(std::uint64_t total, std::uint64_t threads) {
    std::uint32_t s = 0;
    while(s < 5 && (total << (s + 1)) <= threads) ++s;
    return s;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

/// Parent offset q and child index c of child `id` of a level split nsub ways: a shift and a mask when nsub
/// is a power of two (every fan-out of the shipped lemmas), else a 32-bit division (ids within one launch
/// fit 32 bits), and a 64-bit division only beyond that.
__device__ __forceinline__ void split_index(std::uint64_t id, int nsub, std::uint64_t& q, int& c) {
    const unsigned n = unsigned(nsub);
    if((n & (n - 1u)) == 0u) {
        q = id >> (__ffs(int(n)) - 1);
        c = int(id & std::uint64_t(n - 1u));
    } else if(id <= 0xffffffffull) {
        const unsigned i = unsigned(id), qq = i / n;
        q = qq;
        c = int(i - qq * n);
    } else {
        q = id / n;
        c = int(id % n);
    }
}
__device__ __forceinline__ unsigned lanes_below() { return (1u << lane_id()) - 1u; }

__device__ __forceinline__ std::uint32_t item_elem(const LevelArgs& a, std::uint64_t item) {
    return a.in_elem ? a.in_elem[item] : std::uint32_t(item - a.in_begin) + a.elem_base;
}
__device__ __forceinline__ std::uint32_t item_tag(const LevelArgs& a, std::uint64_t item) {
    return a.in_tag ? a.in_tag[item] : (a.elem_tag ? a.elem_tag[item_elem(a, item)] : a.tag_value);
}

/// Adds per-lane values to the counters F0, F1, F2 (-1: unused) of each lane's request: one atomic per
/// distinct request among the lanes of `active` (all of which call this together, with uniform masks).
template<int F0, int F1, int F2>
__device__ __forceinline__ void add_to_requests(unsigned active, ReqDev* req, std::uint32_t tag, unsigned v0, unsigned v1,
                                                unsigned v2) {
    unsigned pending = active;
    while(pending) {
        const int leader = __ffs(pending) - 1;
        const std::uint32_t t = __shfl_sync(active, tag, leader);
        const bool mine = tag == t;
        const unsigned grp = __ballot_sync(active, mine);
        const unsigned s0 = F0 >= 0 ? __reduce_add_sync(active, mine ? v0 : 0u) : 0u;
        const unsigned s1 = F1 >= 0 ? __reduce_add_sync(active, mine ? v1 : 0u) : 0u;
        const unsigned s2 = F2 >= 0 ? __reduce_add_sync(active, mine ? v2 : 0u) : 0u;
        if(int(lane_id()) == leader) {
            if(F0 >= 0 && s0) atomicAdd(&req[t].cnt[F0 >= 0 ? F0 : 0], (unsigned long long)s0);
            if(F1 >= 0 && s1) atomicAdd(&req[t].cnt[F1 >= 0 ? F1 : 0], (unsigned long long)s1);
            if(F2 >= 0 && s2) atomicAdd(&req[t].cnt[F2 >= 0 ? F2 : 0], (unsigned long long)s2);
        }
        pending &= ~grp;
    }
}

/// Reserves queue slots in each lane's request for the lanes with `want` set (one atomic per request).
__device__ __forceinline__ unsigned long long reserve_queue_slots(unsigned active, ReqDev* req, std::uint32_t tag, bool want) {
    unsigned pending = active;
    unsigned long long slot = 0;
    while(pending) {
        const int leader = __ffs(pending) - 1;
        const std::uint32_t t = __shfl_sync(active, tag, leader);
        const bool mine = tag == t;
        const unsigned grp = __ballot_sync(active, mine);
        const unsigned m = __ballot_sync(active, mine && want);
        unsigned long long base = 0;
        if(int(lane_id()) == leader && m) base = atomicAdd(&req[t].cnt[RC_QSIZE], (unsigned long long)__popc(m));
        base = __shfl_sync(active, base, leader);
        if(mine && want) slot = base + __popc(m & lanes_below());
        pending &= ~grp;
    }
    return slot;
}

/// Replace box[var] by child c of its split into nsub pieces. The variable is known only at run time; a switch per
/// variable keeps every index into the box a constant. (Selecting it inside an unrolled loop over the variables,
/// `if(v == var) box[v] = ...`, let the compiler merge the stores into one store at a computed index, which put
/// the whole box of the level kernels in local memory.)
template<int V, int N, class T> __device__ __forceinline__ void split_box(Iv<T>* box, int var, int nsub, int c) {
    if constexpr(V < N) {
        switch(var) {
            case V: {
                T lo, hi;
                split_child(box[V].lo, box[V].hi, nsub, c, lo, hi);
                box[V] = {lo, hi, false};
                return;
            }
            default: split_box<V + 1, N, T>(box, var, nsub, c);
        }
    }
}

/// Child c of item `item` in T: split the item's variable (splitter.hpp:44-59), propagate, test the
/// level's rows. Returns whether the child survives; `box` is its propagated box. float_rows (double
/// only): the rows are first tested in float on the propagated box rounded outward. Every float interval
/// contains the double interval of the same node, so a float refutation is a double refutation and a
/// float "every constraint holds definitely" makes every double constraint hold; only the remaining
/// children test the rows in double. The result is the double result bit for bit.
template<class L, class T>
__device__ __forceinline__ bool eval_child(const LevelArgs& a, const std::uint64_t item, const int c, Iv<T>* box,
                                           const bool float_rows) {
    constexpr int N = L::NARGS;
    // the split variable is known only at run time: select it in an unrolled loop, so that every index into the
    // box is a constant (an index computed at run time puts the box in local memory)
    #pragma unroll
    for(int v = 0; v < N; ++v) {
        double2 b = a.in_box[std::uint64_t(v) * a.in_stride + item];
        box[v] = {T(b.x), T(b.y), false};
    }
    split_box<0, N, T>(box, a.var, a.nsub, c);
    bool ok = !propagate<L, T>(a.var, box, a.it_limit, a.rec_limit);
    if(ok && a.row_end > a.row_begin) {
        if constexpr(sizeof(T) == sizeof(double)) {
            if(float_rows) {
                Iv<float> fb[N];
                #pragma unroll
                for(int v = 0; v < N; ++v) fb[v] = {__double2float_rd(box[v].lo), __double2float_ru(box[v].hi), false};
                const int st = L::template rows_status<float>(a.row_begin, a.row_end, fb);
                ok = st == 2 || (st == 1 && L::template rows_ok<T>(a.row_begin, a.row_end, box));
            } else {
                ok = L::template rows_ok<T>(a.row_begin, a.row_end, box);
            }
        } else {
            ok = L::template rows_ok<T>(a.row_begin, a.row_end, box);
        }
    }
    return ok;
}

/// Output slots for the threads of a 128-thread block with `want` set, in thread order: one atomic per
/// block on the shared counter (per-warp atomics on one address serialize in L2). All threads call it.
__device__ __forceinline__ unsigned long long block_reserve(unsigned long long* counter, bool want) {
    __shared__ unsigned warp_n[4];
    __shared__ unsigned long long base_sh;
    const unsigned m = __ballot_sync(0xffffffffu, want);
    const int w = int(threadIdx.x >> 5);
    if(lane_id() == 0) warp_n[w] = unsigned(__popc(m));
    __syncthreads();
    if(threadIdx.x == 0) {
        const unsigned total = warp_n[0] + warp_n[1] + warp_n[2] + warp_n[3];
        base_sh = total ? atomicAdd(counter, (unsigned long long)total) : 0ull;
    }
    __syncthreads();
    unsigned off = 0;
    for(int k = 0; k < w; ++k) off += warp_n[k];
    const unsigned long long slot = base_sh + off + __popc(m & lanes_below());
    __syncthreads();   // warp_n and base_sh are free again for the next call
    return slot;
}

/// Cuboid and leaf counts of a 128-thread block's children (all threads call it): one update per counter per
/// block when they all belong to one request, else per warp. Every valid thread writes its tag to tag0; when
/// they differ, whichever value stays fails the uniformity test for some thread and the block falls back.
__device__ __forceinline__ void block_counts(const LevelArgs& a, bool valid, std::uint32_t tag, unsigned cub,
                                             unsigned leaves) {
    __shared__ std::uint32_t tag0;
    if(valid) tag0 = tag;
    __syncthreads();
    if(__syncthreads_and(!valid || tag == tag0)) {
        const int nc = __syncthreads_count(valid && cub != 0);
        const int nl = __syncthreads_count(valid && leaves != 0);
        if(threadIdx.x == 0) {
            ReqDev* r = a.req + tag0;
            if(nc) atomicAdd(&r->cnt[RC_CUBOIDS], (unsigned long long)nc);
            if(nl) atomicAdd(&r->cnt[RC_LEAVES], (unsigned long long)nl);
        }
    } else {
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        if(valid) add_to_requests<RC_CUBOIDS, RC_LEAVES, -1>(active, a.req, tag, cub, leaves, 0u);
    }
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
    #pragma unroll
    for(int o = 16; o > 0; o >>= 1) {
        const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u < v ? u : v;
    }
    return v;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
    #pragma unroll
    for(int o = 16; o > 0; o >>= 1) {
        const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u > v ? u : v;
    }
    return v;
}

/// One child per thread (`in_range` false past the input, then a prefix of the threads has children; with
/// sharding only every part_count-th child is valid): split, propagate, test rows, then emit / queue / join
/// the element hull / store criticals, and count. BLOCK: all threads of
/// the 128-thread block call this together, and output slots and counts are aggregated per block (the
/// dense level kernel, where per-warp atomics on the shared counters serialize); otherwise all lanes of
/// each warp call it and they are aggregated per warp, without block barriers (the escalated children).
template<class L, class T, int MODE, bool BLOCK>
__device__ __forceinline__ void level_child_block(const LevelArgs& a, const bool in_range, const std::uint64_t item, const int c,
                                                  const bool float_rows) {
    constexpr int N = L::NARGS;
    Iv<T> box[N];
    bool ok = false;
    std::uint32_t tag = 0;
    // a child outside the requested part (sharding of the root partition) does not exist for this proof
    const bool valid = in_range && (a.part_count <= 1 || std::uint32_t(c) % a.part_count == a.part_index);
    if(valid) {
        ok = eval_child<L, T>(a, item, c, box, float_rows);
        tag = item_tag(a, item);
    }
    const unsigned leaves = !valid ? 0u : ((MODE == MODE_HULL || MODE == MODE_CRIT) ? 1u : (ok ? 0u : 1u));

    if(MODE == MODE_EMIT) {
        const bool keep = valid && ok;
        unsigned long long slot = 0;
        if(BLOCK) {
            slot = block_reserve(a.out_count, keep);
        } else {
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            unsigned long long base = 0;
            if(lane_id() == 0 && m) base = atomicAdd(a.out_count, (unsigned long long)__popc(m));
            slot = __shfl_sync(0xffffffffu, base, 0) + __popc(m & lanes_below());
        }
        if(keep) {
            if(slot < a.out_cap) {
                #pragma unroll
                for(int v = 0; v < N; ++v) {
                    a.out_box[std::uint64_t(v) * a.out_stride + slot] = make_double2(double(box[v].lo), double(box[v].hi));
                }
                if(a.out_elem) a.out_elem[slot] = item_elem(a, item);
                if(a.out_path) {
                    std::uint64_t p = a.in_path ? a.in_path[item] : 0ull;
                    a.out_path[slot] = p * std::uint64_t(a.nsub) + std::uint64_t(c);
                }
                if(a.out_depth) a.out_depth[slot] = a.in_depth ? a.in_depth[item] : a.depth_value;
                if(a.out_tag) a.out_tag[slot] = tag;
            } else {
                atomicOr(a.overflow, 1u);
            }
        }
    } else {
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        if(valid && MODE == MODE_QUEUE) {
            const unsigned long long slot = reserve_queue_slots(active, a.req, tag, ok);
            if(ok) {
                ReqDev* r = a.req + tag;
                const unsigned long long cap = r->qcap;
                if(slot < cap) {
                    #pragma unroll
                    for(int v = 0; v < N; ++v) r->qbox[std::uint64_t(v) * cap + slot] = make_double2(double(box[v].lo), double(box[v].hi));
                    const std::uint8_t d = a.in_depth ? a.in_depth[item] : a.depth_value;
                    r->qdepth[slot] = std::uint8_t(d + a.depth_add);
                } else {
                    atomicAdd(&r->cnt[RC_OVERFLOW], 1ull);
                }
            }
        } else if(valid && MODE == MODE_HULL) {
            const std::uint32_t e = item_elem(a, item);
            const std::uint64_t path = (a.in_path ? a.in_path[item] : 0ull) * std::uint64_t(a.nsub) + std::uint64_t(c);
            // a full warp of children of one element joins its hull with one atomic per bound: the minimum
            // (maximum) over the warp equals the sequence of per-child atomicMin (atomicMax)
            const bool one_elem = active == 0xffffffffu && __all_sync(0xffffffffu, e == __shfl_sync(0xffffffffu, e, 0));
            const bool any_ok = __any_sync(active, ok);
            if(any_ok) {
                #pragma unroll
                for(int v = 0; v < N; ++v) {
                    const double lo = double(box[v].lo), hi = double(box[v].hi);
                    const std::uint64_t idx = std::uint64_t(e) * N + v;
                    unsigned long long klo = ok ? order_key(lo) : ~0ull, khi = ok ? order_key(hi) : 0ull;
                    unsigned long long zlo = (ok && lo == 0.0) ? ((path << 1) | (__double_as_longlong(lo) < 0 ? 1ull : 0ull)) : ~0ull;
                    unsigned long long zhi = (ok && hi == 0.0) ? ((path << 1) | (__double_as_longlong(hi) < 0 ? 1ull : 0ull)) : ~0ull;
                    if(one_elem) {
                        klo = warp_min_u64(klo);
                        khi = warp_max_u64(khi);
                        zlo = warp_min_u64(zlo);
                        zhi = warp_min_u64(zhi);
                        if(lane_id() == 0) {
                            atomicMin(&a.hull_lo[idx], klo);
                            atomicMax(&a.hull_hi[idx], khi);
                            if(zlo != ~0ull) atomicMin(&a.hull_zlo[idx], zlo);
                            if(zhi != ~0ull) atomicMin(&a.hull_zhi[idx], zhi);
                        }
                    } else if(ok) {
                        atomicMin(&a.hull_lo[idx], klo);
                        atomicMax(&a.hull_hi[idx], khi);
                        if(zlo != ~0ull) atomicMin(&a.hull_zlo[idx], zlo);
                        if(zhi != ~0ull) atomicMin(&a.hull_zhi[idx], zhi);
                    }
                }
            }
        } else if(valid && MODE == MODE_CRIT) {
            if(ok) {
                ReqDev* r = a.req + tag;
                const unsigned long long slot = atomicAdd(&r->cnt[RC_CRITICALS], 1ull);
                if(slot < r->crit_cap) {
                    #pragma unroll
                    for(int v = 0; v < N; ++v) {
                        r->crit[(slot * N + v) * 2] = double(box[v].lo);
                        r->crit[(slot * N + v) * 2 + 1] = double(box[v].hi);
                    }
                }
            }
        }
    }
    if(BLOCK) {
        block_counts(a, valid, tag, (valid && a.count_cuboids) ? 1u : 0u, leaves);
    } else {
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        if(valid) add_to_requests<RC_CUBOIDS, RC_LEAVES, -1>(active, a.req, tag, a.count_cuboids ? 1u : 0u, leaves, 0u);
    }
}

#ifndef SID_LEVEL_MIN_BLOCKS
#define SID_LEVEL_MIN_BLOCKS 4      // resident 128-thread blocks per SM the plain-form level kernel is compiled for
#endif

/// The children of one block of 128 (block `vb` of the level): split, propagate, test rows, output, count. All
/// 128 threads of the executing block call it. k_level runs block blockIdx.x; the device proof loop runs every
/// block of the level on its persistent grid.
template<class L, class T, int MODE> __device__ __forceinline__ void level_vblock(const LevelArgs& a, std::uint64_t vb) {
    const std::uint64_t total = a.n_in * std::uint64_t(a.nsub);
    const std::uint64_t t0 = vb * 128u + threadIdx.x;
    const std::uint64_t t = t0 >> a.lane_shift;
    const bool valid = (t0 & ((std::uint64_t(1) << a.lane_shift) - 1u)) == 0 && t < total;
    std::uint64_t q = 0;
    int c = 0;
    if(valid) split_index(t, a.nsub, q, c);
    level_child_block<L, T, MODE, true>(a, valid, a.in_begin + q, c, a.float_rows);
}

template<class L, class T, int MODE> __global__ void __launch_bounds__(128, SID_LEVEL_MIN_BLOCKS) k_level(const LevelArgs a) {
    level_vblock<L, T, MODE>(a, blockIdx.x);
}

/// Float box of child c of a parent from its k_parent_f32 data: it contains the double child box of
/// split_child. lo = RD(RD(lb) + RD(c*RD(w))) <= RD(lb + RD(c*w)); hi = RU(RU(lb) + RU((c+1)*RU(w))) >=
/// lb + (c+1)*w >= the double split point; the last child ends at RU(ub). (The oracle's precision form
/// builds the same float box.)
__device__ __forceinline__ void split_child_f32(float lb_lo, float ub_hi, float4 sp, int n, int c, float& lo, float& hi) {
    lo = __fadd_rd(lb_lo, __fmul_rd(float(c), sp.x));
    hi = (c + 1 >= n) ? ub_hi : __fadd_ru(sp.y, __fmul_ru(float(c + 1), sp.z));
}

/// Precision form, first pass: children [child_begin, child_begin + n_child) of the launch's items
/// (child id = item offset * nsub + child) are propagated and tested in float on a float box that
/// contains the double child box. A child refuted in float is a leaf (interval arithmetic in float is as
/// sound as in double); every other child id goes to the escalation list, whose children are then
/// evaluated in double by k_level_esc, with double results used throughout.
#ifndef SID_FILTER_MIN_BLOCKS
#define SID_FILTER_MIN_BLOCKS 12    // resident 128-thread blocks per SM the float passes are compiled for (40 registers)
#endif
/// End of a float-pass block (all 128 threads call it; `valid` is false past the chunk): undecided children
/// (ok) are appended to the escalation list, refuted ones count as leaves, every child counts as a cuboid of
/// its request. One escalation-list reservation per block, and, when the block's children all belong to one
/// request (always for a whole-lemma proof), one update per counter per block: per-warp atomics on these
/// few addresses would serialize in L2.
__device__ __forceinline__ void filter_result_block(const LevelArgs& a, bool valid, std::uint32_t tag, std::uint64_t t,
                                                    bool ok) {
    __shared__ unsigned warp_esc[4];
    __shared__ unsigned long long esc_base;
    __shared__ std::uint32_t tag0;
    const bool esc = valid && ok;
    const unsigned m = __ballot_sync(0xffffffffu, esc);
    const int w = int(threadIdx.x >> 5);
    if(lane_id() == 0) warp_esc[w] = unsigned(__popc(m));
    if(valid) tag0 = tag;   // any valid thread's tag; if they differ, the uniformity test below fails
    __syncthreads();
    if(threadIdx.x == 0) {
        const unsigned total = warp_esc[0] + warp_esc[1] + warp_esc[2] + warp_esc[3];
        esc_base = total ? atomicAdd(a.esc_count, (unsigned long long)total) : 0ull;
    }
    const bool one_request = __syncthreads_and(!valid || tag == tag0) != 0;   // also orders esc_base
    unsigned off = 0;
    for(int k = 0; k < w; ++k) off += warp_esc[k];
    if(esc) a.esc[esc_base + off + __popc(m & lanes_below())] = std::uint32_t(t);
    if(one_request) {
        const int nvalid = __syncthreads_count(valid);
        const int nesc = __syncthreads_count(esc);
        if(threadIdx.x == 0 && nvalid > 0) {
            ReqDev* r = a.req + tag0;
            atomicAdd(&r->cnt[RC_CUBOIDS], (unsigned long long)nvalid);
            if(nvalid > nesc) atomicAdd(&r->cnt[RC_LEAVES], (unsigned long long)(nvalid - nesc));
            if(nesc > 0) atomicAdd(&r->cnt[RC_ESCALATED], (unsigned long long)nesc);
        }
    } else {
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        if(valid) add_to_requests<RC_CUBOIDS, RC_LEAVES, RC_ESCALATED>(active, a.req, tag, 1u, ok ? 0u : 1u, ok ? 1u : 0u);
    }
}

/// The float box of child c in place of box[var] (the parent's float range), dispatched per variable as split_box.
template<int V, int N> __device__ __forceinline__ void split_box_f32(Iv<float>* box, int var, float4 sp, int nsub, int c) {
    if constexpr(V < N) {
        switch(var) {
            case V: split_child_f32(box[V].lo, box[V].hi, sp, nsub, c, box[V].lo, box[V].hi); return;
            default: split_box_f32<V + 1, N>(box, var, sp, nsub, c);
        }
    }
}

/// Float pass over block `vb` of a chunk's children (all 128 threads of the executing block call it).
template<class L> __device__ __forceinline__ void filter_f32_vblock(const LevelArgs& a, std::uint64_t vb) {
    constexpr int N = L::NARGS;
    const std::uint64_t t = vb * 128u + threadIdx.x;
    const bool valid = t < a.n_child;
    bool ok = false;
    std::uint32_t tag = 0;
    if(valid) {
        const std::uint64_t id = a.child_begin + t;
        std::uint64_t q;
        int c;
        split_index(id, a.nsub, q, c);
        const std::uint64_t item = a.in_begin + q;
        const std::uint64_t j = q - a.pitem_begin;
        Iv<float> box[N];
        #pragma unroll
        for(int v = 0; v < N; ++v) {
            const float2 f = a.pbox[std::uint64_t(v) * a.pstride + j];
            box[v] = {f.x, f.y, false};
        }
        split_box_f32<0, N>(box, a.var, a.psplit[j], a.nsub, c);
        ok = a.fp32_noprop || !propagate<L, float>(a.var, box, a.it_limit, a.rec_limit);
        if(ok && a.row_end > a.row_begin) ok = L::template rows_ok<float>(a.row_begin, a.row_end, box);
        tag = item_tag(a, item);
    }
    filter_result_block(a, valid, tag, t, ok);
}

template<class L> __global__ void __launch_bounds__(128, SID_FILTER_MIN_BLOCKS) k_filter_f32(const LevelArgs a) {
    filter_f32_vblock<L>(a, blockIdx.x);
}

constexpr std::uint64_t kParentRefuted = 1ull << 63;

/// Split-invariant float pass, per parent: without propagation a child's float box differs from its
/// parent's only in the split variable, so every row subexpression that does not depend on it has one
/// value per parent. H::prelude tests the constraints that do not depend on the split variable (if one
/// fails, no child can pass: kParentRefuted) and stores the values the other constraints consume.
template<class L, class H> __global__ void __launch_bounds__(128) k_prelude_f32(const LevelArgs a, std::uint64_t n_items,
                                                                                 float2* hval, std::uint64_t* hbits) {
    constexpr int N = L::NARGS;
    const std::uint64_t j = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(j >= n_items) return;
    Iv<float> box[N];
    #pragma unroll
    for(int v = 0; v < N; ++v) {
        const float2 f = a.pbox[std::uint64_t(v) * a.pstride + j];
        box[v] = {f.x, f.y, false};
    }
    std::uint64_t bits = 0;
    hbits[j] = H::prelude(box, hval, a.pstride, j, bits) ? bits : kParentRefuted;
}

/// Split-invariant float pass, per child: the constraints that depend on the split variable, from the
/// parent's stored values. Decides exactly as rows_ok on the child's float box without propagation.
template<class L, class H> __global__ void __launch_bounds__(128, SID_FILTER_MIN_BLOCKS) k_filter_hoisted(const LevelArgs a) {
    constexpr int N = L::NARGS;
    const std::uint64_t t = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool valid = t < a.n_child;
    bool ok = false;
    std::uint32_t tag = 0;
    if(valid) {
        const std::uint64_t id = a.child_begin + t;
        std::uint64_t q;
        int c;
        split_index(id, a.nsub, q, c);
        const std::uint64_t item = a.in_begin + q;
        const std::uint64_t j = q - a.pitem_begin;
        const std::uint64_t bits = a.hbits[j];
        ok = (bits & kParentRefuted) == 0;
        if(ok) {
            Iv<float> box[N];
            #pragma unroll
            for(int v = 0; v < N; ++v) {
                const float2 f = a.pbox[std::uint64_t(v) * a.pstride + j];
                box[v] = {f.x, f.y, false};
                if(v == H::VAR) split_child_f32(f.x, f.y, a.psplit[j], a.nsub, c, box[v].lo, box[v].hi);
            }
            ok = H::child(box, a.hval, a.pstride, j, bits);
        }
        tag = item_tag(a, item);
    }
    filter_result_block(a, valid, tag, t, ok);
}

/// Precision form, second pass: the escalated children, in double, with the plain form's outputs.
/// Grid-stride over the list (its length is read on the device, so no host round trip is needed).
#ifndef SID_ESC_MIN_BLOCKS
#define SID_ESC_MIN_BLOCKS 4        // resident 128-thread blocks per SM the double pass is compiled for (128 registers)
#endif

template<class L, int MODE> __device__ __forceinline__ void level_esc_grid(const LevelArgs& a) {
    const std::uint64_t n = *reinterpret_cast<volatile unsigned long long*>(a.esc_count);
    if(a.esc_stat && blockIdx.x == 0 && threadIdx.x == 0 && n) atomicAdd(a.esc_stat, (unsigned long long)n);
    const std::uint64_t stride = std::uint64_t(gridDim.x) * blockDim.x;
    // few escalated children (the float pass refuted nearly all): 2 to 32 lanes each, so that they spread over
    // more warps and each warp runs only its own children's paths (lane_shift_for)
    const std::uint32_t sh = lane_shift_for(n, stride);
    const std::uint64_t nv = n << sh;
    // warp-uniform rounds: every lane of a warp takes part in each of its warp's rounds
    for(std::uint64_t base = std::uint64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u); base < nv; base += stride) {
        const std::uint64_t v = base + lane_id();
        const std::uint64_t j = v >> sh;
        const bool valid = (v & ((std::uint64_t(1) << sh) - 1u)) == 0 && j < n;
        std::uint64_t item = 0;
        int c = 0;
        if(valid) {
            const std::uint64_t id = a.child_begin + a.esc[j];
            std::uint64_t q;
            split_index(id, a.nsub, q, c);
            item = a.in_begin + q;
        }
        level_child_block<L, double, MODE, false>(a, valid, item, c, true);
    }
}

template<class L, int MODE> __global__ void __launch_bounds__(128, SID_ESC_MIN_BLOCKS) k_level_esc(const LevelArgs a) {
    level_esc_grid<L, MODE>(a);
}

/// Initial runtime box: compile-time bounds (fixed point / 1e6, rounded outward) tightened by 50*nargs
/// rounds of all bounds in table order (refactor_constraints_impl.hpp:71-101), stopping early at a round that
/// changes nothing (the later rounds would repeat it).
template<class L, class T> __global__ void k_root_box(double2* out) {
    if(blockIdx.x != 0 || threadIdx.x != 0) return;
    constexpr int N = L::NARGS;
    Iv<T> box[N];
    for(int v = 0; v < N; ++v) {
        long long lb = L::ct_lb(v), ub = L::ct_ub(v);
        double dl = lb <= -0x7fffffffffffffffll ? -Dir<double>::inf() : __ddiv_rd(double(lb), 1000000.0);
        double du = ub >= 0x7fffffffffffffffll ? Dir<double>::inf() : __ddiv_ru(double(ub), 1000000.0);
        box[v] = {T(0), T(0), false};
        if(sizeof(T) == sizeof(double)) {
            box[v].lo = T(dl);
            box[v].hi = T(du);
        } else {
            box[v].lo = T(__double2float_rd(dl));
            box[v].hi = T(__double2float_ru(du));
        }
    }
    for(int round = 0; round < 50 * N; ++round) {
        bool changed = false;
        for(int k = 0; k < L::NBOUNDS; ++k) {
            const int r = L::template apply_bound<T>(k, box);
            if(r == B_EMPTY) {
                changed = true;
                break;
            }
            if(r != B_NONE) changed = true;
        }
        // a whole round that changed nothing: every later round would start from the same box and repeat it, so
        // the rounds left cannot change the result (a single thread spends ~1 us per bound on GB300's FP64 pipe)
        if(!changed) break;
    }
    for(int v = 0; v < N; ++v) out[v] = make_double2(double(box[v].lo), double(box[v].hi));
}

struct BatchArgs {
    const double* lo; const double* hi;
    double* out_lo; double* out_hi;
    std::int8_t* verdict;
    std::uint64_t n;
    const std::uint32_t* order;   // thread t evaluates cuboid order[t] (nullptr: cuboid t)
    std::uint64_t stride;         // distance between variables in lo/hi/out_lo/out_hi (0: n)
    unsigned long long* double_rows;   // if set: += cuboids whose constraints float could not refute
    // deferred cuboids (both set, or neither): the evaluation kernel lists the cuboids whose propagation
    // reaches one of L::SLOW_BOUNDS or whose constraints float cannot refute, and k_eval_batch_slow
    // evaluates them on full warps; slow holds up to n cuboid indices (the two kinds from either end),
    // slow_count[0..1] are cleared per launch
    std::uint64_t* slow;
    unsigned long long* slow_count;
    unsigned slow_blocks;         // grid of k_eval_batch_slow: the device's SMs x 8 resident blocks (0: 1216)
};

/// Whether the batch kernel of a lemma with `nargs` variables defers its rare expensive work (the bounds in
/// L::SLOW_BOUNDS, the double constraints) to k_eval_batch_slow. Measured on 2^22-cuboid batches of every
/// lemma: One Subcontainer 0.208 -> 0.167 ms, Top Packing 1 and 2 0.83 -> 0.77 and 1.07 -> 0.93 ms, Two
/// and Four unchanged; for 5 or more variables the kernel that defers spills far more (>= 5 subcontainers,
/// y_3 <= 0: 548 instead of 60 bytes of spill loads) and is slower (0.153 -> 0.199 ms), so they do not.
/// The host passes the deferred list only to lemmas that use it.
constexpr bool batch_defers(int nargs) { return nargs <= 4; }

/// Deferred work stays in its warp when at least this many of the warp's lanes need it (they run it together
/// with enough active lanes); fewer go to the deferred list. Only for lemmas of at most 2 variables: the
/// code that re-runs the work in place raises the kernel's register pressure, which costs the others more
/// (One Subcontainer, 2^24 cuboids: 0.540 ms without it, 0.563 with it) than it saves them, while the Top
/// Packing lemmas, whose slow bound many lanes reach, gain (2^22 cuboids: 1.22 -> 0.93 ms).
constexpr int kInlineLanes = 8;
__host__ __device__ constexpr bool batch_inline(int nargs) { return nargs <= 2; }

/// Appends the indices of the lanes with `want` to the batch's deferred list (one atomic per warp). Every
/// lane of the warp calls it. The list holds two kinds apart, so that k_eval_batch_slow runs each kind on warps of
/// its own: kind 0 (the propagation reached a slow bound) fills it from the front, counted in slow_count[0];
/// kind 1 (float could not refute the constraints, so they are tested in double) from the back, in slow_count[1].
__device__ __forceinline__ void defer_cuboids(const BatchArgs& a, bool want, std::uint64_t i, int kind) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if(!m) return;
    const int leader = __ffs(m) - 1;
    unsigned long long base = 0;
    if(int(lane_id()) == leader) base = atomicAdd(a.slow_count + kind, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    const unsigned long long slot = base + __popc(m & lanes_below());
    if(want) a.slow[kind == 0 ? slot : a.n - 1 - slot] = i;
}

/// Resident 128-thread blocks per SM the batch kernel is compiled for, and its 128-cuboid tiles per block: 12 blocks
/// (40 registers) of 3 tiles for lemmas with at most 3 variables, where the added warps hide more latency than the
/// spills cost (One Subcontainer, 2^24 cuboids, with the deferred cuboids in two lists by kind: 10 blocks of 4 tiles
/// 0.415 ms, 12 of 4 0.410, 11 of 3 0.403, 12 of 3 0.402-0.403, 13 of 3 0.410, 12 of 2 0.417, 12 of 1 0.419, 14 and
/// 16 of 4 0.431, 10 of 6 0.489, 8 of 4 0.453), 8 blocks (64 registers) of 4 tiles above (Two Subcontainer, 2^22
/// cuboids: 0.170 ms at 8, 0.180 at 10; >= 5 subcontainers 3-4 % slower at 10). SID_BATCH_MIN_BLOCKS and
/// SID_BATCH_TILES override them for tuning builds.
template<class L> constexpr int batch_min_blocks() {
#ifdef SID_BATCH_MIN_BLOCKS
    return SID_BATCH_MIN_BLOCKS;
#else
    return L::NARGS <= 3 ? 12 : 8;
#endif
}
template<class L> __host__ __device__ constexpr int batch_tiles() {
#ifdef SID_BATCH_TILES
    return SID_BATCH_TILES;
#else
    return L::NARGS <= 3 ? 3 : 4;
#endif
}

/// The double row test of the batch kernel, kept out of line: few cuboids reach it, and the kernel's hot
/// code (double propagation, float rows) then fits the instruction cache better.
template<class L, class T> __device__ __noinline__ bool rows_ok_outlined(int r0, int r1, const Iv<T>* box) {
    return L::template rows_ok<T>(r0, r1, box);
}

/// The second stage of the batch kernel for queue entry j (all lanes call it; `valid` marks the lanes with
/// an entry): the cuboid's propagated box, which the first stage wrote, rounded outward to float; the
/// constraints that compute, in float; then, for double lemmas and the cuboids float does not refute, all
/// constraints in double, or with DEFER the cuboid goes to the deferred list.
template<class L, class T, bool DEFER> __device__ __forceinline__ void batch_rest(const BatchArgs& a, std::uint64_t first,
                                                                                  const std::uint32_t* qpos, int j,
                                                                                  bool valid,
                                                                                  unsigned long long& n_double) {
    constexpr int N = L::NARGS;
    bool defer = false;
    std::uint64_t i = 0;
    if(valid) {
        const std::uint64_t st = a.stride ? a.stride : a.n;
        const std::uint64_t t = first + qpos[j];
        i = a.order ? std::uint64_t(a.order[t]) : t;
        Iv<T> box[N];
        Iv<float> fb[N];
        #pragma unroll
        for(int v = 0; v < N; ++v) {
            box[v] = {T(a.out_lo[std::uint64_t(v) * st + i]), T(a.out_hi[std::uint64_t(v) * st + i]), false};
            if constexpr(sizeof(T) == sizeof(double)) fb[v] = {__double2float_rd(box[v].lo), __double2float_ru(box[v].hi), false};
            else fb[v] = {float(box[v].lo), float(box[v].hi), false};
        }
        std::int8_t vd = 0;
        if(!L::template rows_rest<float>(N - 1, N, fb)) {
            vd = 2;
        } else if constexpr(sizeof(T) == sizeof(double)) {
            if constexpr(DEFER) {
                defer = true;
            } else {
                ++n_double;
                if(!rows_ok_outlined<L, T>(N - 1, N, box)) vd = 2;
            }
        }
        if(!defer) a.verdict[i] = vd;
    }
    if constexpr(DEFER) {
        // a few lanes whose constraints float cannot refute go to k_eval_batch_slow; when many of the warp's
        // lanes need the double constraints, they test them here together instead
        const unsigned dm = batch_inline(L::NARGS) ? __ballot_sync(0xffffffffu, defer) : 0u;
        if(__popc(dm) >= kInlineLanes) {
            if(defer) {
                constexpr int N2 = L::NARGS;
                const std::uint64_t st = a.stride ? a.stride : a.n;
                Iv<T> box[N2];
                #pragma unroll
                for(int v = 0; v < N2; ++v) box[v] = {T(a.out_lo[std::uint64_t(v) * st + i]), T(a.out_hi[std::uint64_t(v) * st + i]), false};
                ++n_double;
                a.verdict[i] = rows_ok_outlined<L, T>(N2 - 1, N2, box) ? std::int8_t(0) : std::int8_t(2);
            }
            defer = false;
        }
        defer_cuboids(a, defer, i, 1);
    }
}

/// Stage 1 of the batch kernel for one cuboid per lane (all lanes of each warp call it; `valid` marks the lanes
/// with cuboid i, whose input box is in `box`): the seed bounds decide most cuboids at once (emptied, or left
/// unchanged); the others start over from their input box with the full propagation. Then the comparison-only
/// constraints in the lemma's own type; outputs: the propagated box and, unless the cuboid goes on to stage 2
/// (`push`) or to the deferred list (`defer`), its verdict. With DEFER a cuboid whose propagation reaches a slow
/// bound is deferred, unless kInlineLanes lanes of its warp reached one (then they start over here together).
template<class L, class T, bool DEFER> __device__ __forceinline__ void batch_stage1(const BatchArgs& a, const bool valid,
                                                                                    const std::uint64_t i, Iv<T>* box,
                                                                                    bool& push, bool& defer) {
    constexpr int N = L::NARGS;
    constexpr bool rest = ((L::REST_ROWS >> (N - 1)) & 1ull) != 0;
    constexpr bool DEF = DEFER && L::NBOUNDS <= 16 && L::SLOW_BOUNDS != 0;
    const std::uint64_t st = a.stride ? a.stride : a.n;
    int pr = 0;
    if(valid) {
        pr = propagate_seed<L, T, DEF, L::SEED_LAST>(box);
        if(pr < 0) {
            #pragma unroll
            for(int v = 0; v < N; ++v) box[v] = {T(a.lo[std::uint64_t(v) * st + i]), T(a.hi[std::uint64_t(v) * st + i]), false};
            if constexpr(DEF) {
                pr = propagate_packed<L, T, true>(N - 1, box, N, 4);
            } else {
                pr = propagate<L, T>(N - 1, box, N, 4) ? 1 : 0;
            }
        }
    }
    if constexpr(DEF && !batch_inline(L::NARGS)) {
        defer = pr == 2;
    } else if constexpr(DEF) {
        // a few lanes that reached a slow bound go to k_eval_batch_slow; when many of the warp's lanes did, they
        // start over here together instead
        const unsigned dm = __ballot_sync(0xffffffffu, pr == 2);
        if(__popc(dm) >= kInlineLanes) {
            if(pr == 2) {
                #pragma unroll
                for(int v = 0; v < N; ++v) box[v] = {T(a.lo[std::uint64_t(v) * st + i]), T(a.hi[std::uint64_t(v) * st + i]), false};
                pr = propagate<L, T>(N - 1, box, N, 4) ? 1 : 0;
            }
        } else {
            defer = pr == 2;
        }
    }
    if(valid && !defer) {
        std::int8_t vd = 0;
        if(pr == 1) {
            vd = 1;
        } else if(!L::template row_cheap_c<N - 1, T>(box)) {
            vd = 2;
        } else if(rest) {
            push = true;
        }   // else every constraint of the row only compares, and the test above was the full one
        if(!push) a.verdict[i] = vd;
        #pragma unroll
        for(int v = 0; v < N; ++v) {
            a.out_lo[std::uint64_t(v) * st + i] = double(box[v].lo);
            a.out_hi[std::uint64_t(v) * st + i] = double(box[v].hi);
        }
    }
}

/// Leaf evaluation of independent cuboids: propagate after a change of the last variable
/// (it_limit = nargs, rec_limit = 4) and test all constraints; the verdict is the double one bit for bit.
/// Two stages per block of batch_tiles<L>() tiles of 128 cuboids: (1) one thread per cuboid loads,
/// propagates, writes the propagated box and tests the constraints that only compare variables and
/// constants, in the lemma's own type (exact, and for double lemmas cheaper than rounding the box to
/// float: GB300 issues double comparisons and conversions alike on its narrow FP64 pipe); the cuboids that
/// pass and have constraints that compute go to a queue in shared memory; (2) whenever 128 entries are
/// queued (and for the rest at the end) every thread takes one entry, rounds its box outward to float and
/// tests the constraints that compute in float (every float interval contains the double interval of the
/// same node, so a float refutation is the double one), and in double where float does not refute. Few
/// cuboids reach stage 2 (~10 % of One Subcontainer's synthetic batch), so the conversions and the float
/// constraints run on full warps instead of on the few lanes of every warp that need them. With DEFER
/// (lemmas for which batch_defers holds, given the deferred list), rarer and costlier work leaves the warp
/// too: a cuboid whose propagation reaches one of L::SLOW_BOUNDS, or whose constraints float cannot refute,
/// goes to the deferred list unless kInlineLanes lanes of its warp need the same, and k_eval_batch_slow
/// evaluates the list afterwards. Threads follow `order` when given (the host orders tiles of 2^18 cuboids
/// by the Morton code of the cuboids' positions); results go to each cuboid's own position.
template<class L, class T, bool DEFER> __global__ void __launch_bounds__(128, batch_min_blocks<L>()) k_eval_batch(const BatchArgs a) {
    constexpr int N = L::NARGS;
    constexpr int CAP = 256;
    __shared__ std::uint32_t qpos[CAP];
    __shared__ int qn;
    const std::uint64_t st = a.stride ? a.stride : a.n;
    constexpr int TILES = batch_tiles<L>();
    const std::uint64_t first = std::uint64_t(blockIdx.x) * (128u * TILES);
    unsigned long long n_double = 0;
    if(threadIdx.x == 0) qn = 0;
    __syncthreads();
    for(int tile = 0; tile < TILES; ++tile) {
        const std::uint64_t base = first + std::uint64_t(tile) * 128u;
        if(base >= a.n) break;                                  // uniform over the block
        const std::uint64_t t = base + threadIdx.x;
        const bool valid = t < a.n;
        bool push = false, defer = false;
        std::uint64_t i = 0;
        Iv<T> box[N];
        if(valid) {
            i = a.order ? std::uint64_t(a.order[t]) : t;
            #pragma unroll
            for(int v = 0; v < N; ++v) box[v] = {T(a.lo[std::uint64_t(v) * st + i]), T(a.hi[std::uint64_t(v) * st + i]), false};
        }
        batch_stage1<L, T, DEFER>(a, valid, i, box, push, defer);
        if constexpr(DEFER) defer_cuboids(a, defer, i, 0);
        const unsigned m = __ballot_sync(0xffffffffu, push);
        if(m) {
            int at = 0;
            if(lane_id() == 0) at = atomicAdd(&qn, __popc(m));
            at = __shfl_sync(0xffffffffu, at, 0) + __popc(m & lanes_below());
            if(push) qpos[at] = std::uint32_t(t - first);
        }
        __syncthreads();                                        // the queue and the stage-1 outputs
        const int q = qn;
        __syncthreads();                                        // every warp has read qn before the next tile appends
        if(q >= 128) {
            batch_rest<L, T, DEFER>(a, first, qpos, int(threadIdx.x), true, n_double);
            __syncthreads();
            const int j = int(threadIdx.x) + 128;
            if(j < q) qpos[threadIdx.x] = qpos[j];
            if(threadIdx.x == 0) qn = q - 128;
            __syncthreads();
        }
    }
    const int q = qn;
    if(q > 0) batch_rest<L, T, DEFER>(a, first, qpos, int(threadIdx.x), int(threadIdx.x) < q, n_double);
    if(a.double_rows) {
        const unsigned long long w = __reduce_add_sync(0xffffffffu, unsigned(n_double));
        if(lane_id() == 0 && w) atomicAdd(a.double_rows, w);
    }
    // the deferred-work kernel, launched as this grid's programmatic dependent, may be scheduled once every block
    // got here (it waits for this grid's completion before it reads the list)
    if constexpr(DEFER) asm volatile("griddepcontrol.launch_dependents;");
}

#ifndef SID_SLOW_MIN_BLOCKS
#define SID_SLOW_MIN_BLOCKS 8       // resident 128-thread blocks per SM the deferred-work kernel is compiled for
#endif

/// The deferred cuboids of a batch (BatchArgs::slow: slow_count[0] of kind 0 from the front, slow_count[1] of kind 1
/// from the back), one per thread on full warps, each kind on warps of its own (but the one warp where they meet):
/// each is evaluated from its input box exactly as the first and second stage of k_eval_batch would have
/// (propagation with every bound, the comparison-only constraints in double, the others in float and in
/// double where float does not refute), so its outputs are those of the undeferred evaluation bit for bit.
template<class L, class T> __global__ void __launch_bounds__(128, SID_SLOW_MIN_BLOCKS) k_eval_batch_slow(const BatchArgs a) {
    constexpr int N = L::NARGS;
    // launched as the evaluation kernel's programmatic dependent: wait until that grid has completed and its
    // writes (the list and its counters) are visible; a no-op for an ordinary launch
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const std::uint64_t n0 = a.slow_count[0];
    const std::uint64_t n = n0 + a.slow_count[1];
    const std::uint64_t st = a.stride ? a.stride : a.n;
    const bool rest = L::has_rest(N - 1, N);
    unsigned long long n_double = 0;
    for(std::uint64_t j = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n;
        j += std::uint64_t(gridDim.x) * blockDim.x) {
        const std::uint64_t i = j < n0 ? a.slow[j] : a.slow[a.n - 1 - (j - n0)];
        Iv<T> box[N];
        #pragma unroll
        for(int v = 0; v < N; ++v) box[v] = {T(a.lo[std::uint64_t(v) * st + i]), T(a.hi[std::uint64_t(v) * st + i]), false};
        std::int8_t vd = 0;
        if(propagate<L, T>(N - 1, box, N, 4)) {
            vd = 1;
        } else if(!L::template rows_cheap<T>(N - 1, N, box)) {
            vd = 2;
        } else if(rest) {
            Iv<float> fb[N];
            #pragma unroll
            for(int v = 0; v < N; ++v) {
                if constexpr(sizeof(T) == sizeof(double)) fb[v] = {__double2float_rd(box[v].lo), __double2float_ru(box[v].hi), false};
                else fb[v] = {float(box[v].lo), float(box[v].hi), false};
            }
            if(!L::template rows_rest<float>(N - 1, N, fb)) {
                vd = 2;
            } else if constexpr(sizeof(T) == sizeof(double)) {
                ++n_double;
                if(!rows_ok_outlined<L, T>(N - 1, N, box)) vd = 2;
            }
        }
        a.verdict[i] = vd;
        #pragma unroll
        for(int v = 0; v < N; ++v) {
            a.out_lo[std::uint64_t(v) * st + i] = double(box[v].lo);
            a.out_hi[std::uint64_t(v) * st + i] = double(box[v].hi);
        }
    }
    if(a.double_rows) {
        const unsigned long long w = __reduce_add_sync(0xffffffffu, unsigned(n_double));
        if(lane_id() == 0 && w) atomicAdd(a.double_rows, w);
    }
}

/// The all-double form of the batch evaluation, in the reference's order (the innermost leaf step of
/// cpu_prover_core.hpp:221-256): propagate after a change of the last variable (it_limit = nargs,
/// rec_limit = 4), then the constraints of the last row in the lemma's own type, stopping at the first
/// violated one. No float test, no stages and no deferred list: the FP64 baseline of k_eval_batch, whose
/// outputs it equals bit for bit (a float refutation is a double refutation). One cuboid per thread,
/// through `order` when given.
template<class L, class T> __global__ void __launch_bounds__(128, 8) k_eval_batch_plain(const BatchArgs a) {
    constexpr int N = L::NARGS;
    const std::uint64_t t = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(t >= a.n) return;
    const std::uint64_t st = a.stride ? a.stride : a.n;
    const std::uint64_t i = a.order ? std::uint64_t(a.order[t]) : t;
    Iv<T> box[N];
    #pragma unroll
    for(int v = 0; v < N; ++v) box[v] = {T(a.lo[std::uint64_t(v) * st + i]), T(a.hi[std::uint64_t(v) * st + i]), false};
    std::int8_t vd = 0;
    if(propagate<L, T>(N - 1, box, N, 4)) vd = 1;
    else if(!L::template rows_ok<T>(N - 1, N, box)) vd = 2;
    a.verdict[i] = vd;
    #pragma unroll
    for(int v = 0; v < N; ++v) {
        a.out_lo[std::uint64_t(v) * st + i] = double(box[v].lo);
        a.out_hi[std::uint64_t(v) * st + i] = double(box[v].hi);
    }
}

/// Endpoint dump: every expression the lemma's constraints compare (L::operands, in the oracle's order) on
/// each of n boxes, in T: the box as given (double), or rounded outward to float (the precision form's float
/// pass). Boxes lo[v*stride + i], hi[v*stride + i]; operand j of box i goes to out[j*stride + i] (lo, hi) and
/// und[j*stride + i] (1 if possibly undefined).
template<class L, class T> __global__ void __launch_bounds__(128) k_eval_operands(const double* lo, const double* hi,
                                                                                   std::uint64_t n, std::uint64_t stride,
                                                                                   double2* out, std::int8_t* und) {
    constexpr int N = L::NARGS;
    const std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if(i >= n) return;
    Iv<T> box[N];
    #pragma unroll
    for(int v = 0; v < N; ++v) {
        const double l = lo[std::uint64_t(v) * stride + i], h = hi[std::uint64_t(v) * stride + i];
        if constexpr(sizeof(T) == sizeof(double)) box[v] = {T(l), T(h), false};
        else box[v] = {__double2float_rd(l), __double2float_ru(h), false};
    }
    L::template operands<T>(box, out, und, stride, i);
}

/// Host-side launch table of one compiled lemma.
struct LemmaKernels {
    const char* slug;
    std::uint64_t fingerprint;
    int nargs;
    int nbounds;
    bool is_f32;
    cudaError_t (*level)(int mode, const LevelArgs& a, cudaStream_t s);
    cudaError_t (*root_box)(double2* out, cudaStream_t s);
    cudaError_t (*eval_batch)(const BatchArgs& a, cudaStream_t s);
    // precision form (double lemmas only; null for float lemmas)
    cudaError_t (*filter_f32)(const LevelArgs& a, cudaStream_t s);
    cudaError_t (*level_esc)(int mode, const LevelArgs& a, unsigned blocks, cudaStream_t s);
    // split-invariant float pass per level id (dynamic d, static D + j): stored values per parent, -1 where
    // the level has no such form (no rows, or too many stored values)
    int (*hoist_values)(int level);
    cudaError_t (*prelude_f32)(int level, const LevelArgs& a, std::uint64_t n_items, float2* hval, std::uint64_t* hbits,
                               cudaStream_t s);
    cudaError_t (*filter_hoisted)(int level, const LevelArgs& a, cudaStream_t s);
    cudaError_t (*eval_batch_plain)(const BatchArgs& a, cudaStream_t s);
    int n_operands;                   // expressions compared by the constraints (L::NOPERANDS)
    cudaError_t (*eval_operands)(int use_float, const double* lo, const double* hi, std::uint64_t n, std::uint64_t stride,
                                 double2* out, std::int8_t* und, cudaStream_t s);
    // the device proof loop (proof_loop.cuh): cooperative launch, and its resident blocks per SM
    cudaError_t (*proof_loop)(const struct LoopArgs& a, unsigned blocks, cudaStream_t s);
    int (*proof_loop_occupancy)();
};

template<class L, class T> cudaError_t launch_level(int mode, const LevelArgs& a, cudaStream_t s) {
    const std::uint64_t total = a.n_in * std::uint64_t(a.nsub);
    if(total == 0) return cudaSuccess;
    const unsigned threads = 128;
    if(a.lane_shift > 5) return cudaErrorInvalidValue;
    const std::uint64_t blocks = ((total << a.lane_shift) + threads - 1) / threads;
    if(blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    switch(mode) {
        case MODE_EMIT: k_level<L, T, MODE_EMIT><<<unsigned(blocks), threads, 0, s>>>(a); break;
        case MODE_HULL: k_level<L, T, MODE_HULL><<<unsigned(blocks), threads, 0, s>>>(a); break;
        case MODE_CRIT: k_level<L, T, MODE_CRIT><<<unsigned(blocks), threads, 0, s>>>(a); break;
        case MODE_QUEUE: k_level<L, T, MODE_QUEUE><<<unsigned(blocks), threads, 0, s>>>(a); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template<class L> cudaError_t launch_filter_f32(const LevelArgs& a, cudaStream_t s) {
    if(a.n_child == 0) return cudaSuccess;
    const std::uint64_t blocks = (a.n_child + 127) / 128;
    if(blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    k_filter_f32<L><<<unsigned(blocks), 128, 0, s>>>(a);
    return cudaGetLastError();
}

template<class L, class H> cudaError_t launch_prelude_f32(const LevelArgs& a, std::uint64_t n_items, float2* hval,
                                                          std::uint64_t* hbits, cudaStream_t s) {
    if(n_items == 0) return cudaSuccess;
    const std::uint64_t blocks = (n_items + 127) / 128;
    if(blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    k_prelude_f32<L, H><<<unsigned(blocks), 128, 0, s>>>(a, n_items, hval, hbits);
    return cudaGetLastError();
}

template<class L, class H> cudaError_t launch_filter_hoisted(const LevelArgs& a, cudaStream_t s) {
    if(a.n_child == 0) return cudaSuccess;
    if(a.var != H::VAR) return cudaErrorInvalidValue;
    const std::uint64_t blocks = (a.n_child + 127) / 128;
    if(blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    k_filter_hoisted<L, H><<<unsigned(blocks), 128, 0, s>>>(a);
    return cudaGetLastError();
}

template<class L> cudaError_t launch_level_esc(int mode, const LevelArgs& a, unsigned blocks, cudaStream_t s) {
    if(blocks == 0) return cudaSuccess;
    switch(mode) {
        case MODE_EMIT: k_level_esc<L, MODE_EMIT><<<blocks, 128, 0, s>>>(a); break;
        case MODE_HULL: k_level_esc<L, MODE_HULL><<<blocks, 128, 0, s>>>(a); break;
        case MODE_CRIT: k_level_esc<L, MODE_CRIT><<<blocks, 128, 0, s>>>(a); break;
        case MODE_QUEUE: k_level_esc<L, MODE_QUEUE><<<blocks, 128, 0, s>>>(a); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template<class L, class T> cudaError_t launch_root_box(double2* out, cudaStream_t s) {
    k_root_box<L, T><<<1, 1, 0, s>>>(out);
    return cudaGetLastError();
}

template<class L, class T> cudaError_t launch_eval_batch(const BatchArgs& a, cudaStream_t s) {
    if(a.n == 0) return cudaSuccess;
    const unsigned threads = 128;
    const std::uint64_t per_block = std::uint64_t(threads) * batch_tiles<L>();
    const std::uint64_t blocks = (a.n + per_block - 1) / per_block;
    if constexpr(batch_defers(L::NARGS)) {
        if(a.slow) {
            const cudaError_t e = cudaMemsetAsync(a.slow_count, 0, 2 * sizeof(unsigned long long), s);
            if(e != cudaSuccess) return e;
            k_eval_batch<L, T, true><<<unsigned(blocks), threads, 0, s>>>(a);
            // grid-stride over the deferred list, whose length only the device knows: enough blocks to fill
            // the GPU
            const std::uint64_t want_blocks = (a.n + threads - 1) / threads;
            const std::uint64_t fill = a.slow_blocks ? a.slow_blocks : 1216u;
            const std::uint64_t slow_blocks = want_blocks < fill ? want_blocks : fill;
            // a programmatic dependent launch: its blocks are scheduled as the evaluation's last blocks finish
            // instead of after the whole grid has drained
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(unsigned(slow_blocks));
            cfg.blockDim = dim3(threads);
            cfg.dynamicSmemBytes = 0;
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            return cudaLaunchKernelEx(&cfg, k_eval_batch_slow<L, T>, a);
        }
    }
    k_eval_batch<L, T, false><<<unsigned(blocks), threads, 0, s>>>(a);
    return cudaGetLastError();
}

template<class L, class T> cudaError_t launch_eval_batch_plain(const BatchArgs& a, cudaStream_t s) {
    if(a.n == 0) return cudaSuccess;
    const std::uint64_t blocks = (a.n + 127) / 128;
    if(blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    k_eval_batch_plain<L, T><<<unsigned(blocks), 128, 0, s>>>(a);
    return cudaGetLastError();
}

template<class L, class T> cudaError_t launch_eval_operands(int use_float, const double* lo, const double* hi, std::uint64_t n,
                                                            std::uint64_t stride, double2* out, std::int8_t* und,
                                                            cudaStream_t s) {
    if(n == 0 || L::NOPERANDS == 0) return cudaSuccess;
    if(stride == 0) stride = n;
    const std::uint64_t blocks = (n + 127) / 128;
    if(blocks > 0x7fffffffull || stride < n) return cudaErrorInvalidValue;
    if(use_float) k_eval_operands<L, float><<<unsigned(blocks), 128, 0, s>>>(lo, hi, n, stride, out, und);
    else k_eval_operands<L, T><<<unsigned(blocks), 128, 0, s>>>(lo, hi, n, stride, out, und);
    return cudaGetLastError();
}

} // namespace sid
