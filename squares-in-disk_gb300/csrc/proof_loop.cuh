// Device proof loop: a whole proof in one persistent, cooperatively launched kernel.
//
// The host-driven lane (engine.cu) launches every level of every step and reads each level's size back before
// sizing the next launch; for proofs of a few thousand cuboids those launches and reads are the whole cost.
// Here the same work runs in one kernel on a grid of co-resident blocks:
//   * the root partition (prover/proof_driver.hpp:320-391) level by level over the whole grid, each level a
//     grid-stride loop over the per-block bodies the level kernels use, levels separated by a grid barrier;
//   * then steps: the grid takes up to `step` elements from the top of the request's queue, and each block takes
//     whole elements and runs, block-locally, what the reference's core does for one queue element -- the static
//     recursion with hull join (cpu_prover_core.hpp:221-256), and on the hull either the final generation's
//     static recursion storing criticals or the dynamic re-split into the queue (pd_impl_split_into.hpp:37-75).
//     The levels of an element use per-block lists (processed in chunks that fit them) and block barriers only,
//     so a step costs three grid barriers however many levels it has, and blocks work on elements of different
//     depths at once.
// The precision form runs each level as the float pass over the children (rows on the child's float box without
// propagation, so exact by construction) and the double pass over the children float cannot refute. Counts go
// to the request's device counters exactly as in the lane.
//
// Every grid-barrier wait is bounded: a block that gives up records the error word and every block leaves at
// its next barrier; the host reports SID_ERR_TIMEOUT. A queue or list that would overflow records its own error
// word instead of writing past its end, and the host then proves the lemma with the host-driven lane.
#pragma once

#include <cstdint>

#include "engine.cuh"

namespace sid {

constexpr int kLoopMaxLevels = 8;

struct LoopSplit {
    int arg, initial, subdivisions;
};

/// Control words of one device proof loop (zeroed by the host before the launch).
struct LoopCtl {
    unsigned bar_count, bar_gen;           // grid barrier
    unsigned error;                        // 0 ok, 1 barrier timeout, 2 queue overflow, 3 list overflow
    unsigned overflow;                     // level-list overflow flag (LevelArgs::overflow)
    unsigned long long steps;              // steps run
    unsigned long long dyn[kLoopMaxLevels];   // survivors per dynamic level of the root partition
    unsigned long long esc[2];             // escalation-list lengths of the root partition (alternating chunks)
};

enum : unsigned { kLoopOk = 0, kLoopTimeout = 1, kLoopQueueOverflow = 2, kLoopListOverflow = 3 };

/// Words of a block's own control area (kBlockCtlWords per block).
enum : int { BC_STAT = 0, BC_DYN = kLoopMaxLevels, BC_ESC = 2 * kLoopMaxLevels, kBlockCtlWords = 2 * kLoopMaxLevels + 8 };

struct LoopArgs {
    ReqDev* req;                           // request table; the proof is request `tag`
    std::uint32_t tag;
    int nargs;
    int n_dyn, n_stat;
    LoopSplit dyn[kLoopMaxLevels], stat[kLoopMaxLevels];
    const double2* root;                   // the lemma's root box
    std::uint32_t part_index, part_count;  // sharding of the root partition's first split
    bool fp32;                             // precision form
    std::uint32_t fp32_mask;               // levels (dynamic d, static D + j) that use the float pass
    std::uint64_t step;                    // queue elements per step
    std::uint64_t max_steps;
    // root partition (grid-wide): lists of dynamic level d >= 1, the float data and escalation list of a level
    double2* dl_box[kLoopMaxLevels]; std::uint8_t* dl_depth[kLoopMaxLevels]; std::uint32_t* dl_tag[kLoopMaxLevels];
    std::uint64_t dl_cap[kLoopMaxLevels];
    std::uint32_t* esc; std::uint64_t esc_cap;
    float2* pbox; float4* psplit; std::uint64_t p_cap;
    // steps: the taken elements, their hulls (4 x step_cap x nargs order keys)
    double2* step_box; std::uint8_t* step_depth; std::uint32_t* step_tag; std::uint64_t step_cap;
    unsigned long long* hull;
    // per-block scratch (block b's part starts at b times the per-block size): static list j and dynamic list d
    // of one element, its hull box, the float data and escalation list of one level chunk, the control words
    double2* bs_box[kLoopMaxLevels]; std::uint32_t* bs_elem[kLoopMaxLevels]; std::uint64_t* bs_path[kLoopMaxLevels];
    std::uint64_t bs_cap[kLoopMaxLevels];
    double2* bd_box[kLoopMaxLevels]; std::uint8_t* bd_depth[kLoopMaxLevels];
    std::uint64_t bd_cap[kLoopMaxLevels];
    std::uint32_t group_max;               // elements a block takes at once (at most)
    double2* b_hull_box;                   // per block: two lists (final generation, re-split) of group_max hulls,
    std::uint8_t* b_hull_depth;            // variable-major (box [v * group_max + j]), with their depths
    float2* b_pbox; float4* b_psplit; std::uint64_t b_p_cap;   // b_p_cap parents per block
    std::uint32_t* b_esc; std::uint64_t b_esc_cap;
    unsigned long long* b_ctl;             // kBlockCtlWords per block
    LoopCtl* ctl;                          // this proof's counters (root partition lists, steps, list overflow)
    LoopCtl* sync;                         // the grid barrier and error word: ctl itself, or a bundle's shared one
};

constexpr unsigned kLoopBarrierLimit = 1u << 22;   // polls (with a short sleep each) before a barrier gives up

/// Grid barrier with a bounded wait (the pattern of a cooperative grid synchronisation: block-level barrier,
/// release fence, one arrival per block, the last arrival opens the next generation, acquire fence). Returns
/// false, for every thread of the block alike, once any block recorded an error.
__device__ __forceinline__ bool loop_barrier(LoopCtl* ctl, unsigned& gen) {
    __syncthreads();
    if(threadIdx.x == 0) {
        volatile unsigned* vgen = &ctl->bar_gen;
        volatile unsigned* verr = &ctl->error;
        if(gridDim.x > 1) {
            __threadfence();
            const unsigned arrived = atomicAdd(&ctl->bar_count, 1u) + 1u;
            if(arrived == gridDim.x) {
                ctl->bar_count = 0;
                __threadfence();
                atomicExch(&ctl->bar_gen, gen + 1u);
            } else {
                unsigned k = 0;
                while(*vgen == gen && *verr == 0u) {
                    if(++k > kLoopBarrierLimit) {
                        atomicCAS(&ctl->error, 0u, kLoopTimeout);
                        break;
                    }
                    __nanosleep(64);
                }
            }
            __threadfence();
        }
        gen += 1u;
    }
    return __syncthreads_and(*reinterpret_cast<volatile unsigned*>(&ctl->error) == 0u) != 0;
}

__device__ __forceinline__ unsigned long long loop_read(const unsigned long long* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}

__device__ __forceinline__ void loop_set_error(LoopCtl* ctl, unsigned code) { atomicCAS(&ctl->error, 0u, code); }

/// Per-parent float data of a level (k_parent_f32's body) for parents [first, first + n_items) (thread start t0,
/// stride dt): each parent rounded outward to float, and for the split variable the double split width rounded
/// both ways.
__device__ __forceinline__ void loop_parent_f32(const double2* in_box, std::uint64_t in_stride, std::uint64_t first,
                                                std::uint64_t n_items, int nargs, int var, int nsub, float2* pbox,
                                                float4* psplit, std::uint64_t t0, std::uint64_t dt) {
    for(std::uint64_t j = t0; j < n_items; j += dt) {
        for(int v = 0; v < nargs; ++v) {
            const double2 b = in_box[std::uint64_t(v) * in_stride + first + j];
            pbox[std::uint64_t(v) * n_items + j] = make_float2(__double2float_rd(b.x), __double2float_ru(b.y));
            if(v == var) {
                const double w = __ddiv_rd(__dsub_rd(b.y, b.x), double(nsub));
                psplit[j] = make_float4(__double2float_rd(w), __double2float_ru(b.x), __double2float_ru(w), 0.0f);
            }
        }
    }
}

/// The double pass over a block's escalation list (k_level_esc's body on one block): warp-uniform rounds.
template<class L, int MODE> __device__ __forceinline__ void level_esc_block(const LevelArgs& a) {
    const std::uint64_t n = loop_read(a.esc_count);
    for(std::uint64_t base = threadIdx.x & ~31u; base < n; base += blockDim.x) {
        const std::uint64_t j = base + lane_id();
        const bool valid = j < n;
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

/// One level run by one block over a.n_in items from a.in_begin: the dense body over every child, or on a
/// float-pass level the per-parent float data, then per chunk of children the float pass and the double pass
/// over the escalated ones. Block barriers only.
template<class L, class T, int MODE> __device__ void block_level(const LoopArgs& la, LevelArgs a, int level) {
    const std::uint64_t total = a.n_in * std::uint64_t(a.nsub);
    if(total == 0) return;
    bool fp32 = false;
    if constexpr(sizeof(T) == sizeof(double)) fp32 = la.fp32 && ((la.fp32_mask >> level) & 1u) && a.part_count <= 1;
    if(!fp32) {
        a.count_cuboids = true;
        a.float_rows = la.fp32;
        const std::uint64_t nb = (total + 127) / 128;
        for(std::uint64_t vb = 0; vb < nb; ++vb) level_vblock<L, T, MODE>(a, vb);
        return;
    }
    float2* pbox = la.b_pbox + std::uint64_t(blockIdx.x) * la.b_p_cap * std::uint64_t(L::NARGS);
    float4* psplit = la.b_psplit + std::uint64_t(blockIdx.x) * la.b_p_cap;
    loop_parent_f32(a.in_box, a.in_stride, a.in_begin, a.n_in, L::NARGS, a.var, a.nsub, pbox, psplit, threadIdx.x,
                    blockDim.x);
    unsigned long long* esc_count = la.b_ctl + std::uint64_t(blockIdx.x) * kBlockCtlWords + BC_ESC;
    a.count_cuboids = false;
    a.fp32_noprop = true;                 // rows on the child's float box: exact by construction
    a.pbox = pbox;
    a.psplit = psplit;
    a.pstride = a.n_in;
    a.pitem_begin = 0;
    a.esc = la.b_esc + std::uint64_t(blockIdx.x) * la.b_esc_cap;
    a.esc_count = esc_count;
    for(std::uint64_t cb = 0; cb < total; cb += la.b_esc_cap) {
        if(threadIdx.x == 0) *esc_count = 0;
        __syncthreads();                  // the float data, and the cleared count
        a.child_begin = cb;
        a.n_child = total - cb < la.b_esc_cap ? total - cb : la.b_esc_cap;
        const std::uint64_t cnb = (a.n_child + 127) / 128;
        for(std::uint64_t vb = 0; vb < cnb; ++vb) filter_f32_vblock<L>(a, vb);
        __syncthreads();
        if constexpr(sizeof(T) == sizeof(double)) level_esc_block<L, MODE>(a);
        __syncthreads();
    }
}

template<class L, class T> __device__ __forceinline__ LevelArgs loop_args(const LoopArgs& la) {
    LevelArgs a{};
    a.req = la.req;
    a.tag_value = la.tag;
    a.overflow = &la.ctl->overflow;
    return a;
}

/// Static levels of a group of elements, run by one block (Lane::run_static on the block's lists): depth first, a
/// level's input taken in chunks whose children fit the next list; the innermost level joins each element's hull
/// (MODE_HULL) or stores criticals (MODE_CRIT). Level 0's n0 input items are in_box (stride in_stride), item i
/// being element elem + i. Iterative (an explicit offset per level), so the kernel needs no call stack for it.
template<class L, class T> __device__ void block_static(const LoopArgs& la, const double2* in_box, std::uint64_t in_stride,
                                                     std::uint64_t n0, std::uint32_t elem, int final_mode) {
    const int n = la.nargs;
    const int S = la.n_stat;
    std::uint64_t off[kLoopMaxLevels], cnt_in[kLoopMaxLevels];
    off[0] = 0;
    cnt_in[0] = n0;
    int j = 0;
    while(j >= 0) {
        const LoopSplit& sp = la.stat[j];
        const bool last = j + 1 == S;
        LevelArgs a = loop_args<L, T>(la);
        if(j == 0) {
            a.in_box = in_box;
            a.in_stride = in_stride;
        } else {
            const std::uint64_t cap_in = la.bs_cap[j];
            const std::uint64_t boff = std::uint64_t(blockIdx.x) * cap_in;
            a.in_box = la.bs_box[j] + boff * std::uint64_t(n);
            a.in_stride = cap_in;
            a.in_elem = la.bs_elem[j] + boff;
            a.in_path = la.bs_path[j] + boff;
        }
        a.elem_tag = la.step_tag;
        a.var = sp.arg;
        a.nsub = sp.subdivisions;
        a.it_limit = n;
        a.rec_limit = 4;
        a.row_begin = sp.arg;
        a.row_end = last ? n : la.stat[j + 1].arg;
        const int level = la.n_dyn + j;
        if(last) {
            a.in_begin = 0;
            a.n_in = cnt_in[j];
            a.elem_base = elem;            // level 0 only: item i is element elem + i
            a.hull_lo = la.hull;
            a.hull_hi = la.hull + la.step_cap * n;
            a.hull_zlo = la.hull + 2 * la.step_cap * n;
            a.hull_zhi = la.hull + 3 * la.step_cap * n;
            if(final_mode == MODE_HULL) block_level<L, T, MODE_HULL>(la, a, level);
            else block_level<L, T, MODE_CRIT>(la, a, level);
            __syncthreads();
            --j;
            continue;
        }
        if(off[j] >= cnt_in[j]) {
            --j;
            continue;
        }
        const std::uint64_t cap = la.bs_cap[j + 1];
        const std::uint64_t chunk = cap / std::uint64_t(sp.subdivisions) > 0 ? cap / std::uint64_t(sp.subdivisions) : 1;
        const std::uint64_t boff = std::uint64_t(blockIdx.x) * cap;
        unsigned long long* cnt = la.b_ctl + std::uint64_t(blockIdx.x) * kBlockCtlWords + BC_STAT + j + 1;
        if(threadIdx.x == 0) *cnt = 0;
        __syncthreads();
        a.in_begin = off[j];
        a.n_in = cnt_in[j] - off[j] < chunk ? cnt_in[j] - off[j] : chunk;
        a.elem_base = elem + std::uint32_t(off[j]);   // level 0: item in_begin + i is element elem + in_begin + i
        a.out_box = la.bs_box[j + 1] + boff * std::uint64_t(n);
        a.out_stride = cap;
        a.out_cap = cap;
        a.out_elem = la.bs_elem[j + 1] + boff;
        a.out_path = la.bs_path[j + 1] + boff;
        a.out_count = cnt;
        block_level<L, T, MODE_EMIT>(la, a, level);
        __syncthreads();
        off[j] += a.n_in;
        const std::uint64_t m = loop_read(cnt);
        if(m > 0) {
            ++j;
            off[j] = 0;
            cnt_in[j] = m;
        }
    }
}

/// Dynamic re-split of n0 boxes (elements' hulls, in_box with stride in_stride, their depths in_depth[i]) with
/// depth + 1, run by one block depth first like block_static; the last level appends to the request's queue.
template<class L, class T> __device__ void block_dynamic(const LoopArgs& la, const double2* in_box, std::uint64_t in_stride,
                                                      const std::uint8_t* in_depth, std::uint64_t n0) {
    const int n = la.nargs;
    const int D = la.n_dyn;
    std::uint64_t off[kLoopMaxLevels], cnt_in[kLoopMaxLevels];
    off[0] = 0;
    cnt_in[0] = n0;
    int d = 0;
    while(d >= 0) {
        const LoopSplit& sp = la.dyn[d];
        const bool last = d + 1 == D;
        LevelArgs a = loop_args<L, T>(la);
        if(d == 0) {
            a.in_box = in_box;
            a.in_stride = in_stride;
            a.in_depth = in_depth;
        } else {
            const std::uint64_t cap_in = la.bd_cap[d];
            const std::uint64_t boff = std::uint64_t(blockIdx.x) * cap_in;
            a.in_box = la.bd_box[d] + boff * std::uint64_t(n);
            a.in_stride = cap_in;
            a.in_depth = la.bd_depth[d] + boff;
        }
        a.var = sp.arg;
        a.nsub = sp.subdivisions;
        a.it_limit = 2 * n;
        a.rec_limit = n < 32 ? n : 32;
        if(last) {
            a.in_begin = 0;
            a.n_in = cnt_in[d];
            a.row_begin = n - 1;
            a.row_end = n;
            a.depth_add = 1;
            block_level<L, T, MODE_QUEUE>(la, a, d);
            __syncthreads();
            --d;
            continue;
        }
        if(off[d] >= cnt_in[d]) {
            --d;
            continue;
        }
        a.row_begin = a.row_end = 0;
        const std::uint64_t cap = la.bd_cap[d + 1];
        const std::uint64_t chunk = cap / std::uint64_t(sp.subdivisions) > 0 ? cap / std::uint64_t(sp.subdivisions) : 1;
        const std::uint64_t boff = std::uint64_t(blockIdx.x) * cap;
        unsigned long long* cnt = la.b_ctl + std::uint64_t(blockIdx.x) * kBlockCtlWords + BC_DYN + d + 1;
        if(threadIdx.x == 0) *cnt = 0;
        __syncthreads();
        a.in_begin = off[d];
        a.n_in = cnt_in[d] - off[d] < chunk ? cnt_in[d] - off[d] : chunk;
        a.out_box = la.bd_box[d + 1] + boff * std::uint64_t(n);
        a.out_stride = cap;
        a.out_cap = cap;
        a.out_depth = la.bd_depth[d + 1] + boff;
        a.out_count = cnt;
        block_level<L, T, MODE_EMIT>(la, a, d);
        __syncthreads();
        off[d] += a.n_in;
        const std::uint64_t m = loop_read(cnt);
        if(m > 0) {
            ++d;
            off[d] = 0;
            cnt_in[d] = m;
        }
    }
}

/// Elements a block takes at once in a step that takes `take` elements of a proof on `blocks` blocks: one each while
/// that leaves blocks idle, more while the elements outnumber the blocks, up to la.group_max (enough to give the
/// first static level about one child per thread). Uniform over the grid.
__device__ __forceinline__ std::uint64_t loop_group(const LoopArgs& la, std::uint64_t take, std::uint64_t blocks) {
    const std::uint64_t k = take / blocks;
    return k < 1 ? 1 : (k > la.group_max ? la.group_max : k);
}

/// Queue elements e0 .. e0 + k - 1 of the step list (k <= group_max), by one block: static recursion with hull
/// join, then each non-empty hull's final generation or re-split, the hulls of the group together. Lemmas without
/// static splits: every element is its own only leaf and hull.
template<class L, class T> __device__ void block_elements(const LoopArgs& la, std::uint64_t e0, std::uint64_t k) {
    constexpr int N = L::NARGS;
    ReqDev* r = la.req + la.tag;
    const std::uint64_t G = la.group_max;
    double2* fbox = la.b_hull_box + std::uint64_t(blockIdx.x) * 2 * G * N;    // final generation
    double2* rbox = fbox + G * N;                                             // re-split
    std::uint8_t* fdep = la.b_hull_depth + std::uint64_t(blockIdx.x) * 2 * G;
    std::uint8_t* rdep = fdep + G;
    __shared__ unsigned nfin, nres;
    if(threadIdx.x == 0) {
        nfin = 0;
        nres = 0;
    }
    if(la.n_stat > 0) {
        for(std::uint64_t t = threadIdx.x; t < k * N; t += blockDim.x) {
            const std::uint64_t w = e0 * N + t;
            la.hull[w] = ~0ull;
            la.hull[la.step_cap * N + w] = 0ull;
            la.hull[2 * la.step_cap * N + w] = ~0ull;
            la.hull[3 * la.step_cap * N + w] = ~0ull;
        }
        __syncthreads();
        // level 0's items are the elements: their columns of the step list
        block_static<L, T>(la, la.step_box + e0, la.step_cap, k, std::uint32_t(e0), MODE_HULL);
    } else {
        __syncthreads();
    }
    // each element's hull (k_hull_finalize): min of lower bounds, max of upper bounds, zeros signed as the first
    // leaf's; non-empty hulls go to the final-generation or the re-split list of the block
    for(std::uint64_t j = threadIdx.x; j < k; j += blockDim.x) {
        const std::uint64_t e = e0 + j;
        bool nonempty = true;
        if(la.n_stat > 0) nonempty = loop_read(&la.hull[e * N]) != ~0ull;
        else atomicAdd(&r->cnt[RC_LEAVES], 1ull);
        if(!nonempty) continue;
        const std::uint8_t depth = la.step_depth[e];
        const bool fin = depth >= r->generations;
        const unsigned slot = atomicAdd(fin ? &nfin : &nres, 1u);
        double2* out = fin ? fbox : rbox;
        if(fin) fdep[slot] = depth;
        else rdep[slot] = depth;
        for(int v = 0; v < N; ++v) {
            double2 h;
            if(la.n_stat > 0) {
                double lo = key_value(loop_read(&la.hull[e * N + v]));
                double hi = key_value(loop_read(&la.hull[la.step_cap * N + e * N + v]));
                if(lo == 0.0) lo = (loop_read(&la.hull[2 * la.step_cap * N + e * N + v]) & 1ull) ? -0.0 : 0.0;
                if(hi == 0.0) hi = (loop_read(&la.hull[3 * la.step_cap * N + e * N + v]) & 1ull) ? -0.0 : 0.0;
                h = make_double2(lo, hi);
            } else {
                h = la.step_box[std::uint64_t(v) * la.step_cap + e];
            }
            out[std::uint64_t(v) * G + slot] = h;
        }
    }
    __syncthreads();
    const unsigned nf = nfin, nr = nres;
    __syncthreads();                      // every thread has read the counts before the next group resets them
    if(nf > 0) {
        if(la.n_stat == 0) {
            // the hulls are the leaves: each a leaf and a critical
            for(std::uint64_t j = threadIdx.x; j < nf; j += blockDim.x) {
                atomicAdd(&r->cnt[RC_LEAVES], 1ull);
                const unsigned long long slot = atomicAdd(&r->cnt[RC_CRITICALS], 1ull);
                if(slot < r->crit_cap) {
                    for(int v = 0; v < N; ++v) {
                        const double2 h = fbox[std::uint64_t(v) * G + j];
                        r->crit[(slot * N + v) * 2] = h.x;
                        r->crit[(slot * N + v) * 2 + 1] = h.y;
                    }
                }
            }
            __syncthreads();
        } else {
            block_static<L, T>(la, fbox, G, nf, 0u, MODE_CRIT);
        }
    }
    if(nr > 0) block_dynamic<L, T>(la, rbox, G, rdep, nr);
    __syncthreads();
}

/// One level of the root partition over the whole grid (the lane's `launch`).
template<class L, class T, int MODE> __device__ bool grid_level(const LoopArgs& la, LevelArgs a, int level, unsigned& gen) {
    const std::uint64_t total = a.n_in * std::uint64_t(a.nsub);
    if(total == 0) return true;
    bool fp32 = false;
    if constexpr(sizeof(T) == sizeof(double)) fp32 = la.fp32 && ((la.fp32_mask >> level) & 1u) && a.part_count <= 1;
    if(!fp32) {
        a.count_cuboids = true;
        a.float_rows = la.fp32;
        a.lane_shift = lane_shift_for(total, std::uint64_t(gridDim.x) * blockDim.x);
        const std::uint64_t nb = ((total << a.lane_shift) + 127) / 128;
        for(std::uint64_t vb = blockIdx.x; vb < nb; vb += gridDim.x) level_vblock<L, T, MODE>(a, vb);
        return true;
    }
    loop_parent_f32(a.in_box, a.in_stride, 0, a.n_in, L::NARGS, a.var, a.nsub, la.pbox, la.psplit,
                    std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x, std::uint64_t(gridDim.x) * blockDim.x);
    if(!loop_barrier(la.sync, gen)) return false;
    a.count_cuboids = false;
    a.fp32_noprop = true;
    a.pbox = la.pbox;
    a.psplit = la.psplit;
    a.pstride = a.n_in;
    a.pitem_begin = 0;
    a.esc = la.esc;
    int k = 0;
    for(std::uint64_t cb = 0; cb < total; cb += la.esc_cap, k ^= 1) {
        a.child_begin = cb;
        a.n_child = total - cb < la.esc_cap ? total - cb : la.esc_cap;
        a.esc_count = &la.ctl->esc[k];
        if(blockIdx.x == 0 && threadIdx.x == 0) la.ctl->esc[k ^ 1] = 0;   // the other chunk's counter is free
        const std::uint64_t nb = (a.n_child + 127) / 128;
        for(std::uint64_t vb = blockIdx.x; vb < nb; vb += gridDim.x) filter_f32_vblock<L>(a, vb);
        if(!loop_barrier(la.sync, gen)) return false;
        if constexpr(sizeof(T) == sizeof(double)) level_esc_grid<L, MODE>(a);
        if(!loop_barrier(la.sync, gen)) return false;
    }
    // every chunk's double pass has finished: both counters start the next float-pass level at zero (the
    // caller's barrier orders this before that level's float pass)
    if(blockIdx.x == 0 && threadIdx.x == 0) {
        la.ctl->esc[0] = 0;
        la.ctl->esc[1] = 0;
    }
    return true;
}

/// The root partition (Lane::run_dynamic with the initial subdivisions) over the whole grid; its last level
/// appends to the request's queue.
template<class L, class T> __device__ bool grid_root_partition(const LoopArgs& la, unsigned& gen) {
    const int n = la.nargs;
    const double2* in_box = la.root;
    std::uint64_t in_stride = 1, n_in = 1;
    const std::uint8_t* in_depth = nullptr;
    const std::uint32_t* in_tag = nullptr;
    for(int d = 0; d < la.n_dyn; ++d) {
        const LoopSplit& sp = la.dyn[d];
        const bool last = d + 1 == la.n_dyn;
        LevelArgs a = loop_args<L, T>(la);
        a.in_box = in_box;
        a.in_stride = in_stride;
        a.in_depth = in_depth;
        a.in_tag = in_tag;
        a.in_begin = 0;
        a.n_in = n_in;
        a.var = sp.arg;
        a.nsub = sp.initial;
        a.it_limit = 2 * n;
        a.rec_limit = n < 255 ? n : 255;
        if(d == 0) {
            a.part_index = la.part_index;
            a.part_count = la.part_count;
        }
        if(last) {
            a.row_begin = n - 1;
            a.row_end = n;
            return grid_level<L, T, MODE_QUEUE>(la, a, d, gen) && loop_barrier(la.sync, gen);
        }
        a.row_begin = a.row_end = 0;
        a.out_box = la.dl_box[d + 1];
        a.out_stride = la.dl_cap[d + 1];
        a.out_cap = la.dl_cap[d + 1];
        a.out_depth = la.dl_depth[d + 1];
        a.out_tag = la.dl_tag[d + 1];
        a.out_count = &la.ctl->dyn[d + 1];
        if(!grid_level<L, T, MODE_EMIT>(la, a, d, gen)) return false;
        if(!loop_barrier(la.sync, gen)) return false;
        n_in = loop_read(&la.ctl->dyn[d + 1]);
        if(n_in > la.dl_cap[d + 1]) {
            if(blockIdx.x == 0 && threadIdx.x == 0) loop_set_error(la.sync, kLoopListOverflow);
            return false;
        }
        if(n_in == 0) return true;
        in_box = la.dl_box[d + 1];
        in_stride = la.dl_cap[d + 1];
        in_depth = la.dl_depth[d + 1];
        in_tag = la.dl_tag[d + 1];
    }
    return true;
}

#ifndef SID_LOOP_MIN_BLOCKS
#define SID_LOOP_MIN_BLOCKS 4       // resident 128-thread blocks per SM the proof loop is compiled for
#endif

/// The proof loop (launched cooperatively: every block is resident). Root partition, then steps while the
/// request's queue holds elements: take up to `step` elements from its top; each block processes whole elements.
template<class L, class T> __global__ void __launch_bounds__(128, SID_LOOP_MIN_BLOCKS) k_proof_loop(const LoopArgs la) {
    constexpr int N = L::NARGS;
    unsigned gen = 0;
    ReqDev* r = la.req + la.tag;
    if(!grid_root_partition<L, T>(la, gen)) return;
    for(std::uint64_t step = 0; step < la.max_steps; ++step) {
        const std::uint64_t q = loop_read(&r->cnt[RC_QSIZE]);
        const bool q_over = loop_read(&r->cnt[RC_OVERFLOW]) != 0;
        if(q_over || *reinterpret_cast<volatile unsigned*>(&la.ctl->overflow) != 0u) {
            if(blockIdx.x == 0 && threadIdx.x == 0) loop_set_error(la.sync, q_over ? kLoopQueueOverflow : kLoopListOverflow);
            return;
        }
        if(q == 0) break;
        const std::uint64_t take = q < la.step ? q : la.step;
        const std::uint64_t begin = q - take;
        const std::uint64_t stride = std::uint64_t(gridDim.x) * blockDim.x;
        for(std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < take; i += stride) {
            for(int v = 0; v < N; ++v) la.step_box[std::uint64_t(v) * la.step_cap + i] = r->qbox[std::uint64_t(v) * r->qcap + begin + i];
            la.step_depth[i] = r->qdepth[begin + i];
            la.step_tag[i] = la.tag;
        }
        if(blockIdx.x == 0 && threadIdx.x == 0) la.ctl->steps = step + 1;
        if(!loop_barrier(la.sync, gen)) return;
        // popped: children append from here (a queue append reserves its slot atomically from this size)
        if(blockIdx.x == 0 && threadIdx.x == 0) r->cnt[RC_QSIZE] = begin;
        if(!loop_barrier(la.sync, gen)) return;
        const std::uint64_t k = loop_group(la, take, gridDim.x);
        const std::uint64_t units = (take + k - 1) / k;
        for(std::uint64_t u = blockIdx.x; u < units; u += gridDim.x) {
            const std::uint64_t e0 = u * k;
            block_elements<L, T>(la, e0, take - e0 < k ? take - e0 : k);
        }
        if(!loop_barrier(la.sync, gen)) return;
    }
}

template<class L, class T> cudaError_t launch_proof_loop(const LoopArgs& la, unsigned blocks, cudaStream_t s) {
    void* params[] = {const_cast<LoopArgs*>(&la)};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(&k_proof_loop<L, T>), dim3(blocks), dim3(128), params,
                                       0, s);
}

/// Resident 128-thread blocks per SM of the proof loop (the cooperative grid's limit per SM), asked of the runtime
/// once per process: the query costs host time inside every short proof otherwise.
template<class L, class T> int proof_loop_occupancy() {
    static int cached = -1;
    if(cached >= 0) return cached;
    int n = 0;
    if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_proof_loop<L, T>, 128, 0) != cudaSuccess) return 0;
    cached = n;
    return n;
}

// ---- Bundles: proofs of several lemmas in one persistent kernel over one grid.
//
// A bundle kernel is compiled for a fixed list of lemmas (csrc/codegen.py generates one per configured bundle);
// proof i runs the generated code of the list's i-th lemma. The root partitions run one after the other over the
// whole grid; then every step takes up to `step` elements from the top of each proof's frontier into that proof's
// step list, and the whole grid drains the union of the step lists: block b takes items b, b + grid, ... of the
// concatenation, whatever proof they belong to, so elements of different lemmas and depths are processed side by
// side, and every child goes back to its own proof's frontier. Each proof keeps its own counters, frontier,
// critical store and per-block scratch exactly as in the one-proof loop, so its counts are those of the proof
// run alone. Every proof's `sync` is the bundle's one barrier and error word.

constexpr int kBundleMax = 4;

struct BundleArgs {
    int n;                                 // proofs (at most kBundleMax; the kernel's lemma list has n entries)
    LoopArgs p[kBundleMax];
};
static_assert(sizeof(BundleArgs) <= 32000, "bundle arguments must fit the kernel parameter space");

// Each member type M of a bundle kernel gives its lemma's root partition and element processing as
// M::root(la, gen) and M::elements(la, e0, k): grid_root_partition<L, double> and block_elements<L, double> of the
// lemma, compiled in the lemma's own translation unit with separate compilation (csrc/codegen.py), so the bundle
// kernel's own unit stays small.
template<int I, class L0, class... Ls> __device__ bool bundle_roots(const BundleArgs& b, unsigned& gen) {
    if(I < b.n && !L0::root(b.p[I], gen)) return false;
    if constexpr(sizeof...(Ls) > 0) {
        return bundle_roots<I + 1, Ls...>(b, gen);
    } else {
        return true;
    }
}

template<int I, class L0, class... Ls>
__device__ void bundle_elements(const BundleArgs& b, int i, std::uint64_t e0, std::uint64_t k) {
    if(i == I) {
        L0::elements(b.p[I], e0, k);
    } else {
        if constexpr(sizeof...(Ls) > 0) bundle_elements<I + 1, Ls...>(b, i, e0, k);
    }
}

/// Copy `take` elements from position `begin` of a proof's frontier into its step list (grid-stride).
__device__ __forceinline__ void loop_take(const LoopArgs& la, std::uint64_t begin, std::uint64_t take) {
    const ReqDev* r = la.req + la.tag;
    const std::uint64_t stride = std::uint64_t(gridDim.x) * blockDim.x;
    for(std::uint64_t i = std::uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < take; i += stride) {
        for(int v = 0; v < la.nargs; ++v) {
            la.step_box[std::uint64_t(v) * la.step_cap + i] = r->qbox[std::uint64_t(v) * r->qcap + begin + i];
        }
        la.step_depth[i] = r->qdepth[begin + i];
        la.step_tag[i] = la.tag;
    }
}

/// The bundle loop (launched cooperatively). Double lemmas only; the precision form per proof (LoopArgs::fp32).
template<class... Ls> __global__ void __launch_bounds__(128, SID_LOOP_MIN_BLOCKS) k_proof_loop_bundle(const BundleArgs b) {
    static_assert(sizeof...(Ls) >= 1 && sizeof...(Ls) <= kBundleMax, "a bundle holds 1 to kBundleMax lemmas");
    unsigned gen = 0;
    LoopCtl* sync = b.p[0].sync;
    if(!bundle_roots<0, Ls...>(b, gen)) return;
    for(std::uint64_t step = 0;; ++step) {
        std::uint64_t first[kBundleMax + 1], begin[kBundleMax];
        first[0] = 0;
        bool q_over = false, l_over = false;
        for(int i = 0; i < kBundleMax; ++i) {
            std::uint64_t take = 0;
            begin[i] = 0;
            if(i < b.n) {
                const LoopArgs& la = b.p[i];
                const ReqDev* r = la.req + la.tag;
                const std::uint64_t q = loop_read(&r->cnt[RC_QSIZE]);
                q_over = q_over || loop_read(&r->cnt[RC_OVERFLOW]) != 0;
                l_over = l_over || *reinterpret_cast<volatile unsigned*>(&la.ctl->overflow) != 0u;
                if(step < la.max_steps) take = q < la.step ? q : la.step;
                begin[i] = q - take;
            }
            first[i + 1] = first[i] + take;
        }
        if(q_over || l_over) {
            if(blockIdx.x == 0 && threadIdx.x == 0) loop_set_error(sync, q_over ? kLoopQueueOverflow : kLoopListOverflow);
            return;
        }
        const std::uint64_t total = first[kBundleMax];
        if(total == 0) break;
        // work units: groups of elements of one proof (loop_group, sized by the whole step's elements)
        std::uint64_t ufirst[kBundleMax + 1], group[kBundleMax];
        ufirst[0] = 0;
        for(int i = 0; i < kBundleMax; ++i) {
            const std::uint64_t take = first[i + 1] - first[i];
            group[i] = i < b.n ? loop_group(b.p[i], total, gridDim.x) : 1;
            ufirst[i + 1] = ufirst[i] + (take + group[i] - 1) / group[i];
        }
        for(int i = 0; i < b.n; ++i) {
            const std::uint64_t take = first[i + 1] - first[i];
            if(take == 0) continue;
            loop_take(b.p[i], begin[i], take);
            if(blockIdx.x == 0 && threadIdx.x == 0) b.p[i].ctl->steps = step + 1;
        }
        if(!loop_barrier(sync, gen)) return;
        // popped: children append from here
        if(blockIdx.x == 0 && threadIdx.x == 0) {
            for(int i = 0; i < b.n; ++i) {
                if(first[i + 1] > first[i]) b.p[i].req[b.p[i].tag].cnt[RC_QSIZE] = begin[i];
            }
        }
        if(!loop_barrier(sync, gen)) return;
        for(std::uint64_t u = blockIdx.x; u < ufirst[kBundleMax]; u += gridDim.x) {
            int i = 0;
            while(u >= ufirst[i + 1]) ++i;
            const std::uint64_t e0 = (u - ufirst[i]) * group[i];
            const std::uint64_t take = first[i + 1] - first[i];
            bundle_elements<0, Ls...>(b, i, e0, take - e0 < group[i] ? take - e0 : group[i]);
        }
        if(!loop_barrier(sync, gen)) return;
    }
}

template<class... Ls> cudaError_t launch_proof_loop_bundle(const BundleArgs& b, unsigned blocks, cudaStream_t s) {
    if(b.n != int(sizeof...(Ls))) return cudaErrorInvalidValue;
    void* params[] = {const_cast<BundleArgs*>(&b)};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(&k_proof_loop_bundle<Ls...>), dim3(blocks), dim3(128),
                                       params, 0, s);
}

template<class... Ls> int proof_loop_bundle_occupancy() {
    static int cached = -1;
    if(cached >= 0) return cached;
    int n = 0;
    if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_proof_loop_bundle<Ls...>, 128, 0) != cudaSuccess) return 0;
    cached = n;
    return n;
}

/// Host-side table of one compiled bundle.
struct BundleKernels {
    const char* name;
    int n;
    std::uint64_t fingerprints[kBundleMax];   // of the lemma whose code proof i runs
    cudaError_t (*launch)(const BundleArgs& b, unsigned blocks, cudaStream_t s);
    int (*occupancy)();
};

} // namespace sid
