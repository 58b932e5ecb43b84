/*
 * C ABI of the GB300 interval branch-and-bound engine (libsid.so).
 *
 * The reference has no foreign-function boundary: its lemma programs call the
 * C++ template ivarp::run_prover (ivarp/include/ivarp/run_prover.hpp:57-88),
 * which runs the proof driver (prover/proof_driver.hpp:218-627) with a prover
 * core (cpu_prover/cpu_prover_core.hpp:31-260 or
 * with_cuda/ivarp_cuda/gpu_prover_core.cuh:199-470). Here that driver and core
 * are replaced by this C ABI; the C++ run_prover in include/ivarp/run_prover.hpp
 * is its only caller on the proof path. Each entry point below names the
 * reference interface whose job it takes over.
 *
 * Conventions: every function returns SID_OK (0) or a negative status; no
 * exception crosses the boundary; buffers are caller-owned host memory unless
 * the name ends in _device; an engine handle must not be used from two host
 * threads at once. All device-side waits are bounded and report
 * SID_ERR_TIMEOUT instead of hanging.
 */
#ifndef SID_H
#define SID_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SID_OK 0
#define SID_ERR_INVALID (-1)      /* bad argument or malformed lemma IR */
#define SID_ERR_CUDA (-2)         /* a CUDA call failed; see sid_last_error() */
#define SID_ERR_NOT_COMPILED (-3) /* no GPU kernels were built for this lemma IR */
#define SID_ERR_NOMEM (-4)        /* device allocation failed */
#define SID_ERR_TIMEOUT (-5)      /* a bounded device wait gave up */
#define SID_ERR_UNSUPPORTED (-6)  /* setting or feature not supported */
#define SID_ERR_CAPACITY (-7)     /* result larger than the caller's buffer */

typedef struct sid_engine sid_engine;

/* Proof statistics; field meaning as ivarp::ProofInformation (prover/proof_information.hpp:32-44). */
typedef struct sid_result {
    uint64_t num_cuboids;
    uint64_t num_leaf_cuboids;
    uint64_t num_critical_cuboids;
    uint64_t num_repeated_nodes;
    uint64_t criticals_stored;   /* criticals retained for sid_fetch_criticals */
    uint64_t escalated;          /* cuboids re-evaluated in FP64 (precision form only) */
    double seconds;              /* device wall time of the proof */
    int32_t complete;            /* 0 if the proof stopped early at a checkpoint (opts.stop_after_steps) */
    uint32_t steps;              /* steps run (queue batches expanded) */
} sid_result;

/* Snapshot handed to a progress callback (ivarp::ProgressInfo, default_progress_observer.hpp:30-35). */
typedef struct sid_progress {
    uint64_t queue_size;
    uint64_t cuboid_count;
    uint64_t leaf_count;
    uint64_t critical_count;
    const double* queue_head;    /* 2*nargs doubles (lo,hi per variable) of one queued element, or NULL */
} sid_progress;

typedef void (*sid_progress_fn)(void* user, const sid_progress* progress);

#define SID_PRECISION_PLAIN 0           /* the lemma's own number type, bit-exact with the reference */
#define SID_PRECISION_FP32_ESCALATE 1   /* precision form for double lemmas: every child cuboid is first
                                           tested in FP32 (outward rounded, sound); only the children FP32
                                           cannot refute are evaluated in FP64, whose results are used. By
                                           default the FP32 test skips propagation (fp32_noprop_mask), and
                                           the counts are the plain form's by construction; float lemmas
                                           run plain. */

#define SID_PRECISION_FP32_TUNED 2      /* the precision form with the lemma's autotuned configuration
                                           (sid_lemma_autotune: step size, levels that use the float
                                           pass); before tuning, as SID_PRECISION_FP32_ESCALATE */

/* Settings of one proof; meaning as ivarp::ProverSettings (prover_input.hpp:124-159). */
typedef struct sid_prove_opts {
    uint32_t generation_count;          /* default 8 */
    int32_t max_iterations_per_node;    /* passes over the static splits per queue element (p_handle_cuboid_nf,
                                           cpu_prover_core.hpp:113-134): after a pass, the hull of the surviving
                                           leaves is run again as the element while fewer than this many passes
                                           ran and a criterion below accepts it, each repeat counting one cuboid
                                           and one repeated node; <= 1: one pass (the published proofs use 1) */
    float iteration_volume_criterion;   /* repeat if the hull's volume exceeds this share of the element's */
    float iteration_single_dimension_criterion;   /* repeat if some variable's hull width exceeds this share of
                                                     the element's width (both in the lemma's number type,
                                                     rounded down as the reference computes them) */
    int64_t batch_elements;             /* queue elements expanded per step; <= 0: engine default */
    int32_t precision;                  /* SID_PRECISION_* */
    uint64_t max_criticals_kept;        /* criticals stored for sid_fetch_criticals */
    sid_progress_fn progress;           /* optional, called from the calling thread between steps */
    void* progress_user;
    uint32_t progress_first_ms;         /* delay before the first callback */
    uint32_t progress_every_ms;
    uint32_t fp32_level_mask;           /* precision forms: levels that use the float pass (default all;
                                           SID_PRECISION_FP32_TUNED uses the lemma's tuned mask) */
    const char* checkpoint_path;        /* if set: write the proof's state to this file every
                                           checkpoint_every_steps steps and when stopping early */
    uint32_t checkpoint_every_steps;    /* 0: only when stopping early */
    uint32_t stop_after_steps;          /* > 0: stop after this many steps (with a checkpoint) */
    uint32_t fp32_noprop_mask;          /* precision forms: float-pass levels that skip bound propagation and
                                           test the rows on the child's float box (default: all). Such a level
                                           cannot refute a child that double keeps: the float box then contains
                                           the double box before and after its propagation, so the counts are
                                           the plain form's by construction. Levels with a split-invariant
                                           form evaluate the subexpressions that do not depend on the split
                                           variable once per parent. A level whose bit is clear propagates in
                                           float first (fewer escalations; exact unless the float and double
                                           propagations take different orders). */
    uint32_t part_index;                /* sharding (no counterpart in the reference): with part_count > 1, */
    uint32_t part_count;                /* prove only the children i of the root partition's first split with
                                           i % part_count == part_index. The parts' counts sum to the whole
                                           proof's and their criticals together are the whole proof's, so
                                           parts can run on separate GPUs or processes. 0 or 1: whole proof. */
    uint32_t device_loop_blocks;        /* no counterpart in the reference: > 0 runs the whole proof in one
                                           persistent kernel on this many co-resident 128-thread blocks (at
                                           most the device's limit for that kernel), with no host round trip
                                           between levels or steps; 0 (default) drives each level from the
                                           host. Same counts and criticals either way. Proofs that need
                                           re-iteration, checkpoints or progress callbacks use the host loop; a
                                           proof whose queue outgrows the loop's preallocated room is redone by
                                           the host loop. */
} sid_prove_opts;

/* Fill `opts` with the defaults above. */
void sid_prove_opts_default(sid_prove_opts* opts);

/* Human-readable description of the last error on this thread. */
const char* sid_last_error(void);

/* Create an engine on CUDA device `device` (replaces the device discovery and per-device driver
 * threads of with_cuda/ivarp_cuda/gpu_prover_core.cuh:237-251). */
int sid_engine_create(int device, sid_engine** out);
void sid_engine_destroy(sid_engine* engine);

/* Register a compiled lemma (the text IR written by the front end for an ivarp::ProverInput,
 * prover_input.hpp:118-122). The engine selects the kernels generated for this IR at build time. */
int sid_lemma_register(sid_engine* engine, const char* ir, size_t ir_len, int* lemma_id);
int sid_lemma_info(sid_engine* engine, int lemma_id, int* nargs, uint64_t* fingerprint);

/* Initial runtime box: compile-time bounds tightened by 50*nargs rounds of all bounds
 * (refactor_constraints_impl.hpp:90-101). out_lohi: 2*nargs doubles. */
int sid_lemma_root_box(sid_engine* engine, int lemma_id, double* out_lohi);

/* Run a whole proof (ProofDriver::run, proof_driver.hpp:472-489). Returns SID_OK whether or not
 * criticals remain; the verdict is result->num_critical_cuboids == 0. */
int sid_prove(sid_engine* engine, int lemma_id, const sid_prove_opts* opts, sid_result* result);

/* Continue a proof from a checkpoint written by sid_prove (no counterpart in the reference). The file holds
 * the lemma's fingerprint, the generation limit, the counters and stored criticals, and the frontier queue
 * (boxes and depths) between two steps; the result counts the whole proof, so a resumed proof reports what
 * the uninterrupted one would. opts may checkpoint and stop again. */
int sid_prove_resume(sid_engine* engine, int lemma_id, const sid_prove_opts* opts, const char* checkpoint_path,
                     sid_result* result);

/* Whole proofs of several lemmas at once in one persistent kernel (no counterpart in the reference, whose
 * driver proves one lemma per run_prover call; each proof is ProofDriver::run, proof_driver.hpp:472-489).
 * lemma_ids: n (1 to 4) distinct registered double lemmas for which the build generated a bundle kernel
 * (a line of a bundles.txt beside their IR; SID_ERR_NOT_COMPILED otherwise). The root partitions run one
 * after the other over the whole grid; then every step takes up to opts->batch_elements elements (each
 * lemma's default or tuned step otherwise) from the top of each proof's frontier, and the grid drains
 * them all together, elements of different lemmas and depths side by side, each child returning to its
 * own proof's frontier. results[j] is lemma_ids[j]'s proof with exactly the counts and criticals of
 * sid_prove alone (sid_fetch_criticals per lemma afterwards); seconds is the whole bundle's time.
 * opts: generation_count, precision (per lemma, as sid_prove), batch_elements, max_criticals_kept,
 * fp32 masks, device_loop_blocks (grid size; 0: every block that can be resident). Re-iteration,
 * checkpoints, progress and parts: SID_ERR_UNSUPPORTED. A proof whose frontier outgrows the loop's room
 * is proved again by the host-driven loop. */
int sid_prove_bundle(sid_engine* engine, int n, const int* lemma_ids, const sid_prove_opts* opts, sid_result* results);

/* Copy the criticals retained by the last sid_prove of this lemma: n*2*nargs doubles, per critical
 * the (lo,hi) pairs of all variables (the on_critical calls of cpu_prover_core.hpp:137-149). */
int sid_fetch_criticals(sid_engine* engine, int lemma_id, double* out, uint64_t capacity, uint64_t* n_out);

/* Autotuning of the precision form for one lemma (no counterpart in the reference). Levels are numbered
 * dynamic splits first (root partition and re-splits of dynamic variable d share level d), then static
 * splits (level D + j). A first precision-form proof measures each level's escalation rate (children the
 * float pass cannot refute / children); candidate configurations combine a threshold (levels whose rate
 * exceeds it skip the float pass and go straight to double) with a step size, and are timed by proving
 * the lemma, as long as max_seconds of proving allows. Every candidate must reproduce the first proof's
 * cuboid, leaf and critical counts or it is discarded. Proofs shorter than 5 ms also try the device proof loop
 * (sid_prove_opts.device_loop_blocks) on 38, 152 and 608 blocks, with the chosen float-pass levels and with none
 * (every level in the double kernel with float-first rows). The fastest is stored with the lemma and used by
 * SID_PRECISION_FP32_TUNED proofs and servers (servers drive their lanes from the host). */
#define SID_MAX_LEVELS 16
typedef struct sid_tuning {
    int64_t step_elements;                    /* queue elements per step */
    uint32_t fp32_level_mask;                 /* bit l set: level l uses the float pass */
    float escalation_threshold;               /* the threshold the mask came from */
    int32_t levels;                           /* dynamic + static levels of the lemma */
    uint32_t candidates;                      /* configurations timed */
    double level_escalation[SID_MAX_LEVELS];  /* measured escalation rate per level (-1: no children) */
    double seconds;                           /* proof time with the chosen configuration */
    double default_seconds;                   /* proof time with every level on the float pass, 65536 per step */
    uint32_t fp32_noprop_mask;                /* float-pass levels without propagation (sid_prove_opts; the
                                                 default all, or propagation on some levels if faster) */
    uint32_t loop_blocks;                     /* > 0: tuned proofs run in the device proof loop on this many
                                                 blocks (tried for proofs under 5 ms; sid_prove_opts) */
} sid_tuning;

int sid_lemma_autotune(sid_engine* engine, int lemma_id, double max_seconds, sid_tuning* out);

/* Leaf evaluation of a batch of cuboids: for each cuboid, propagate the bounds after a change of the
 * last variable (it_limit = nargs, rec_limit = 4) and test all constraints -- the innermost step of
 * CPUProverCore::p_handle_cuboid (cpu_prover_core.hpp:221-256). Boxes are structure-of-arrays:
 * lo[v*n + i], hi[v*n + i]. Outputs the propagated box and a verdict per cuboid:
 * 0 = survives (critical at this level), 1 = empty after propagation, 2 = a constraint is violated.
 * Host buffers; the copies to and from the device are part of the call. */
int sid_eval_batch(sid_engine* engine, int lemma_id, const double* lo, const double* hi, uint64_t n,
                   double* out_lo, double* out_hi, int8_t* verdict);

/* Same on device buffers, asynchronous on `stream` (a cudaStream_t; NULL for the legacy stream).
 * When the lemma's order is on (sid_lemma_batch_order; by default while more than 1 % of its cuboids need
 * the double constraints) the evaluation follows, within each tile of 2^18 consecutive cuboids, the Morton
 * order of their lower corners (computed on the device from the lemma's root box), which keeps a warp's
 * cuboids on the same code paths; every result is written to its cuboid's own position, so the output does
 * not depend on the order. The ordering scratch belongs to the engine: calls on one engine must not overlap
 * on different streams. */
int sid_eval_batch_device(sid_engine* engine, int lemma_id, const double* lo, const double* hi, uint64_t n,
                          double* out_lo, double* out_hi, int8_t* verdict, void* stream);

/* The all-double form of sid_eval_batch_device: the same outputs bit for bit, computed in the reference's
 * order only (cpu_prover_core.hpp:221-256 at the innermost level: propagation, then the last row's constraints
 * in double, stopping at the first violated one), without the float test of the constraints. Always evaluated
 * in the Morton order of the cuboids' lower corners within tiles of 2^18 cuboids (ordering scratch of the
 * engine, as sid_eval_batch_device). It is the FP64 baseline the float-first kernel is measured against. */
int sid_eval_batch_plain_device(sid_engine* engine, int lemma_id, const double* lo, const double* hi, uint64_t n,
                                double* out_lo, double* out_hi, int8_t* verdict, void* stream);

/* Interval endpoints of the lemma's criteria (no counterpart in the reference, whose constraint evaluation
 * keeps them internal: runtime_constraint_table.hpp:31-115 evaluates each constraint's comparisons and keeps
 * only the verdict). The lemma's constraints compare pairs of expressions; sid_lemma_operands gives the number
 * of compared expressions K: constraints in table order, each constraint's predicate tree in pre-order, the
 * left and the right operand of every comparison not decided at compile time, each comparison once.
 * sid_eval_operands_device evaluates all K expressions on each of n boxes (device buffers, structure of
 * arrays lo[v*n + i], hi[v*n + i]; pass a propagated box from sid_eval_batch_device to get the values the
 * constraints saw): use_float 0 in the lemma's own number type (double: the plain form's endpoints), 1 in
 * float on the box rounded outward (the precision form's first pass). Outputs (device): out_lohi[2*(j*n + i)]
 * and [2*(j*n + i) + 1] the lower and upper endpoint of expression j on box i, out_undefined[j*n + i] 1 if the
 * value is possibly undefined (e.g. a square root of a possibly negative argument), else 0. Every expression
 * is evaluated whether or not an earlier constraint already failed. Asynchronous on `stream`. */
int sid_lemma_operands(sid_engine* engine, int lemma_id, uint32_t* count);
int sid_eval_operands_device(sid_engine* engine, int lemma_id, const double* lo, const double* hi, uint64_t n,
                             int use_float, double* out_lohi, int8_t* out_undefined, void* stream);

/* Kernel timing of the batch calls, for roofline measurements (no counterpart in the reference).
 * sid_eval_batch_profile(engine, 1) makes every following sid_eval_batch* call record CUDA events on its
 * stream around its evaluation kernel and around its ordering kernel; sid_eval_batch_profile_read waits
 * for the recorded events, returns the
 * number of calls, the summed device milliseconds of the ordering work and of the evaluation kernel, and the
 * number of kernels those calls launched (ordering, evaluation, deferred evaluation, sample hand-over), and clears the record (recording continues until sid_eval_batch_profile(engine, 0)). */
int sid_eval_batch_profile(sid_engine* engine, int enable);

int sid_eval_batch_profile_read(sid_engine* engine, uint64_t* calls, double* order_ms, double* eval_ms,
                                uint64_t* launches);

/* Evaluation order of sid_eval_batch / sid_eval_batch_device for one lemma (no counterpart in the reference).
 * Evaluating a batch in the Morton order of the cuboids' lower corners keeps the threads of a warp on the
 * same branches of the double-precision constraints, which pays off when many cuboids need them, and costs
 * a sort (about 0.6 ms per 2^24 cuboids on a GB300) otherwise; the order never changes a result.
 * SID_BATCH_ORDER_AUTO (the default): each call whose predecessor's sample has arrived counts the cuboids
 * whose constraints the float test could not decide, and later calls are ordered while that share exceeds
 * 1 % (calls before the first sample arrives are ordered). mode < 0 keeps the mode; double_share (may be
 * NULL) receives the last sampled share, -1 before any. */
#define SID_BATCH_ORDER_AUTO 0
#define SID_BATCH_ORDER_ON 1
#define SID_BATCH_ORDER_OFF 2
int sid_lemma_batch_order(sid_engine* engine, int lemma_id, int mode, double* double_share);

/* Allocation-free leaf hulls. No counterpart in the reference: it is an addition of this library.
 *
 * For callers that may not allocate GPU memory: a serving loop that runs under a fixed device-memory
 * budget and must not call the allocator (which can block, fragment memory or synchronize the device)
 * on every request, or a host application that owns all device memory through its own pool and does
 * not let third-party code call cudaMalloc. This call allocates nothing: no cudaMalloc or cudaFree and
 * no other allocating routine, on the host or on the device. Double lemmas only (SID_ERR_UNSUPPORTED for float lemmas).
 *
 * For each of the n parent cuboids in `boxes`, split the lemma's last static variable into its
 * configured number of pieces, propagate bounds and test the constraints (the innermost step of the
 * prover core), and join the surviving pieces into that parent's hull. Layout of `boxes` and `hulls`
 * (device memory): (lo, hi) pairs, variable-major: pair [v*n + i]. nonempty[i] (device) is 1 if any
 * piece of parent i survived, else 0 and hulls for i are left untouched; *leaves (device, may be NULL)
 * receives the number of leaves (every piece is a leaf; 0 when n is 0). Asynchronous on `stream` (a
 * cudaStream_t).
 *
 * Its working memory is one 8 MiB array per device inside libsid.so, held from library load until the
 * process exits; n * nargs must be at most 262,136 (larger calls fail with SID_ERR_CAPACITY). The first
 * call on a device looks up that array's device address and keeps it for the life of the process: make this
 * first call before any stream capture, and do not reset the device (cudaDeviceReset) after it. All calls on a device share the array: calls whose work overlaps on the GPU (different
 * streams or host threads) race and corrupt each other's results, so serialize them. */
int sid_leaf_hull_noalloc(sid_engine* engine, int lemma_id, const double* boxes, uint64_t n, double* hulls,
                          uint8_t* nonempty, unsigned long long* leaves, void* stream);

/* Host-side fault injection, for tests of the error paths (no counterpart in the reference, whose worker
 * errors are rethrown on the caller's thread, proof_driver.hpp:99-118). Arms a countdown in this process: the
 * countdown-th following device allocation of an engine (SID_INJECT_ALLOC) or kernel launch of the proof,
 * served and batch paths (SID_INJECT_LAUNCH) fails as if CUDA had returned cudaErrorMemoryAllocation or
 * cudaErrorLaunchFailure, without allocating or launching anything, and the call that meets it returns
 * SID_ERR_NOMEM or SID_ERR_CUDA (a served request: SID_REQ_FAILED). The engine and its servers stay usable
 * afterwards. countdown 0 disarms; an injection fires once. Nothing is injected on the GPU. */
#define SID_INJECT_ALLOC 1
#define SID_INJECT_LAUNCH 2
int sid_debug_inject_failure(int kind, int64_t countdown);

/* ---- Served form: a request loop with continuous batching. No counterpart in the reference (its
 * driver proves one lemma per run_prover call); an addition of this library for proving many lemmas
 * and sub-boxes at once on one GPU.
 *
 * A server owns one worker thread and CUDA stream per lemma ("lane"). sid_submit queues a request: a
 * whole lemma proof (boxes == NULL: the lemma's root box with its root partition, exactly as sid_prove)
 * or a set of sub-boxes of the lemma (each enters the request's frontier as a depth-0 element and counts
 * as one cuboid). Requests are admitted in arrival order while their frontier queues fit the memory
 * budget; each admitted request keeps its frontier and counters on the device. Every step of a lane
 * takes elements from all of its admitted requests at once (an equal share each, leftovers oldest
 * first), so requests that arrive while others are running join the work already on the GPU; lanes of
 * different lemmas run concurrently. The counts of a request do not depend on what else is running.
 * The server must be destroyed before its engine; register lemmas before submitting requests for them. */
typedef struct sid_server sid_server;

typedef struct sid_server_opts {
    uint64_t memory_budget_bytes;       /* device memory for request frontiers; 0: 16 GiB */
    int64_t step_elements;              /* queue elements per lane step; <= 0: 65536 */
    int32_t precision;                  /* SID_PRECISION_* for every request */
    uint32_t generation_count;          /* generations per request; 0: 8 */
    uint64_t max_criticals_per_request; /* critical boxes stored per request */
    uint32_t max_requests_per_lane;     /* admitted at once per lemma; 0: 1024 */
    int32_t max_iterations_per_node;    /* node re-iteration as in sid_prove_opts; default 1 (none) */
    float iteration_volume_criterion;   /* default 0.25 */
    float iteration_single_dimension_criterion;   /* default 0.66 */
} sid_server_opts;

#define SID_REQ_PENDING 0                /* waiting for admission */
#define SID_REQ_RUNNING 1
#define SID_REQ_DONE 2
#define SID_REQ_FAILED 3                 /* sid_request_poll/wait then fill the status and return the failure's
                                            own status (e.g. SID_ERR_NOMEM, SID_ERR_CUDA); sid_last_error() says
                                            what failed. The server keeps serving other requests. */

typedef struct sid_request_status {
    int32_t state;                      /* SID_REQ_* */
    int32_t proved;                     /* DONE and no critical cuboid */
    uint64_t num_cuboids;
    uint64_t num_leaf_cuboids;
    uint64_t num_critical_cuboids;
    uint64_t escalated;                 /* children evaluated in FP64 (precision form) */
    uint64_t criticals_stored;
    double seconds_queued;              /* submission to admission */
    double seconds_to_verdict;          /* submission to completion (host clock) */
    uint64_t num_repeated_nodes;        /* nodes re-iterated on their hull */
} sid_request_status;

void sid_server_opts_default(sid_server_opts* opts);
int sid_server_create(sid_engine* engine, const sid_server_opts* opts, sid_server** out);
/* Stops the workers after the steps in flight; unfinished requests are dropped. */
void sid_server_destroy(sid_server* server);
/* boxes: NULL for the whole lemma, else nboxes * nargs (lo, hi) pairs, box-major: box b, variable v at
 * boxes[2*(b*nargs + v)]. */
int sid_submit(sid_server* server, int lemma_id, const double* boxes, uint64_t nboxes, uint64_t* request_id);
int sid_request_poll(sid_server* server, uint64_t request_id, sid_request_status* status);
/* Wait up to timeout_ms (< 0: no limit) for the request to finish; SID_ERR_TIMEOUT if it has not. */
int sid_request_wait(sid_server* server, uint64_t request_id, int timeout_ms, sid_request_status* status);
/* Critical boxes stored for a finished request, as sid_fetch_criticals. */
int sid_request_criticals(sid_server* server, uint64_t request_id, double* out, uint64_t capacity, uint64_t* n_out);
/* Forget a finished request. */
int sid_request_release(sid_server* server, uint64_t request_id);

#ifdef __cplusplus
}
#endif

#endif /* SID_H */
