"""Python binding of the GB300 prover engine (libsid.so, C ABI in include/sid.h).

Used by the tests and bench.py. The library is built in-tree by squares-in-disk_gb300/build.py; this
module never falls back to anything else: if the library or a GPU is missing, calls fail loudly.
"""
import ctypes
import glob
import os
import sys

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG)
LIB_PATH = os.path.join(os.environ.get("SID_BUILD_DIR") or os.path.join(PKG, "_build"), "libsid.so")
LEMMA_DIR = os.path.join(PKG, "lemmas")
KAT_DIR = os.path.join(REPO, "tests", "golden", "kat")

SID_OK = 0
STATUS = {0: "ok", -1: "invalid", -2: "cuda", -3: "not_compiled", -4: "nomem", -5: "timeout", -6: "unsupported",
          -7: "capacity"}

EXPORTED = ["sid_prove_opts_default", "sid_last_error", "sid_engine_create", "sid_engine_destroy",
            "sid_lemma_register", "sid_lemma_info", "sid_lemma_root_box", "sid_prove", "sid_fetch_criticals",
            "sid_eval_batch", "sid_eval_batch_device", "sid_leaf_hull_noalloc", "sid_server_opts_default",
            "sid_server_create", "sid_server_destroy", "sid_submit", "sid_request_poll", "sid_request_wait",
            "sid_request_criticals", "sid_request_release", "sid_eval_batch_profile", "sid_eval_batch_profile_read",
            "sid_lemma_autotune", "sid_prove_resume", "sid_prove_bundle", "sid_lemma_batch_order", "sid_eval_batch_plain_device",
            "sid_lemma_operands", "sid_eval_operands_device", "sid_debug_inject_failure"]

PRECISION_PLAIN, PRECISION_FP32, PRECISION_TUNED = 0, 1, 2
INJECT_ALLOC, INJECT_LAUNCH = 1, 2
BATCH_ORDER_AUTO, BATCH_ORDER_ON, BATCH_ORDER_OFF = 0, 1, 2
MAX_LEVELS = 16
REQ_PENDING, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class SidResult(ctypes.Structure):
    _fields_ = [("num_cuboids", ctypes.c_uint64), ("num_leaf_cuboids", ctypes.c_uint64),
                ("num_critical_cuboids", ctypes.c_uint64), ("num_repeated_nodes", ctypes.c_uint64),
                ("criticals_stored", ctypes.c_uint64), ("escalated", ctypes.c_uint64), ("seconds", ctypes.c_double),
                ("complete", ctypes.c_int32), ("steps", ctypes.c_uint32)]


PROGRESS_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p)


class SidProgress(ctypes.Structure):
    _fields_ = [("queue_size", ctypes.c_uint64), ("cuboid_count", ctypes.c_uint64), ("leaf_count", ctypes.c_uint64),
                ("critical_count", ctypes.c_uint64), ("queue_head", ctypes.POINTER(ctypes.c_double))]


PROGRESS_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(SidProgress))


class SidProveOpts(ctypes.Structure):
    _fields_ = [("generation_count", ctypes.c_uint32), ("max_iterations_per_node", ctypes.c_int32),
                ("iteration_volume_criterion", ctypes.c_float),
                ("iteration_single_dimension_criterion", ctypes.c_float),
                ("batch_elements", ctypes.c_int64), ("precision", ctypes.c_int32),
                ("max_criticals_kept", ctypes.c_uint64), ("progress", ctypes.c_void_p),
                ("progress_user", ctypes.c_void_p), ("progress_first_ms", ctypes.c_uint32),
                ("progress_every_ms", ctypes.c_uint32), ("fp32_level_mask", ctypes.c_uint32),
                ("checkpoint_path", ctypes.c_char_p), ("checkpoint_every_steps", ctypes.c_uint32),
                ("stop_after_steps", ctypes.c_uint32), ("fp32_noprop_mask", ctypes.c_uint32),
                ("part_index", ctypes.c_uint32), ("part_count", ctypes.c_uint32),
                ("device_loop_blocks", ctypes.c_uint32)]


class SidServerOpts(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", ctypes.c_uint64), ("step_elements", ctypes.c_int64),
                ("precision", ctypes.c_int32), ("generation_count", ctypes.c_uint32),
                ("max_criticals_per_request", ctypes.c_uint64), ("max_requests_per_lane", ctypes.c_uint32),
                ("max_iterations_per_node", ctypes.c_int32), ("iteration_volume_criterion", ctypes.c_float),
                ("iteration_single_dimension_criterion", ctypes.c_float)]


class SidRequestStatus(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("proved", ctypes.c_int32), ("num_cuboids", ctypes.c_uint64),
                ("num_leaf_cuboids", ctypes.c_uint64), ("num_critical_cuboids", ctypes.c_uint64),
                ("escalated", ctypes.c_uint64), ("criticals_stored", ctypes.c_uint64),
                ("seconds_queued", ctypes.c_double), ("seconds_to_verdict", ctypes.c_double),
                ("num_repeated_nodes", ctypes.c_uint64)]

    def as_dict(self):
        return dict(state=self.state, proved=bool(self.proved), cuboids=self.num_cuboids,
                    leaves=self.num_leaf_cuboids, criticals=self.num_critical_cuboids, escalated=self.escalated,
                    stored=self.criticals_stored, seconds_queued=self.seconds_queued,
                    seconds_to_verdict=self.seconds_to_verdict, repeated=self.num_repeated_nodes)


class SidTuning(ctypes.Structure):
    _fields_ = [("step_elements", ctypes.c_int64), ("fp32_level_mask", ctypes.c_uint32),
                ("escalation_threshold", ctypes.c_float), ("levels", ctypes.c_int32), ("candidates", ctypes.c_uint32),
                ("level_escalation", ctypes.c_double * MAX_LEVELS), ("seconds", ctypes.c_double),
                ("default_seconds", ctypes.c_double), ("fp32_noprop_mask", ctypes.c_uint32),
                ("loop_blocks", ctypes.c_uint32)]


class SidError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%s)" % (msg, STATUS.get(status, status)))
        self.status = status


_lib = None


def load(path=LIB_PATH):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError("engine library not built: %s (run __graft_entry__.build())" % path)
    L = ctypes.CDLL(path)
    L.sid_last_error.restype = ctypes.c_char_p
    L.sid_prove_opts_default.argtypes = [ctypes.POINTER(SidProveOpts)]
    L.sid_engine_create.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    L.sid_engine_destroy.argtypes = [ctypes.c_void_p]
    L.sid_lemma_register.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_int)]
    L.sid_lemma_info.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_uint64)]
    L.sid_lemma_root_box.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.sid_prove.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(SidProveOpts), ctypes.POINTER(SidResult)]
    L.sid_prove_resume.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(SidProveOpts), ctypes.c_char_p,
                                   ctypes.POINTER(SidResult)]
    L.sid_prove_bundle.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(SidProveOpts), ctypes.POINTER(SidResult)]
    L.sid_fetch_criticals.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                                      ctypes.POINTER(ctypes.c_uint64)]
    L.sid_eval_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.sid_eval_batch_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]
    L.sid_eval_batch_plain_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p]
    L.sid_lemma_operands.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)]
    L.sid_eval_operands_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]
    L.sid_debug_inject_failure.argtypes = [ctypes.c_int, ctypes.c_int64]
    L.sid_leaf_hull_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.sid_server_opts_default.argtypes = [ctypes.POINTER(SidServerOpts)]
    L.sid_server_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(SidServerOpts), ctypes.POINTER(ctypes.c_void_p)]
    L.sid_server_destroy.argtypes = [ctypes.c_void_p]
    L.sid_submit.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64,
                             ctypes.POINTER(ctypes.c_uint64)]
    L.sid_request_poll.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(SidRequestStatus)]
    L.sid_request_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(SidRequestStatus)]
    L.sid_request_criticals.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                                        ctypes.POINTER(ctypes.c_uint64)]
    L.sid_request_release.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
    L.sid_eval_batch_profile.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.sid_lemma_batch_order.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    L.sid_lemma_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.POINTER(SidTuning)]
    L.sid_eval_batch_profile_read.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_uint64)]
    _lib = L
    return L


def _check(status):
    if status != SID_OK:
        raise SidError(status, load().sid_last_error().decode())


def inject_failure(kind, countdown):
    """Arm (countdown > 0) or disarm (0) a host-side failure of the countdown-th following device allocation
    (INJECT_ALLOC) or kernel launch (INJECT_LAUNCH), see sid_debug_inject_failure."""
    _check(load().sid_debug_inject_failure(kind, countdown))


def lemma_ir(name):
    """IR text of a lemma by slug (squares-in-disk_gb300/lemmas) or known-answer system (tests/golden/kat)."""
    for d in (LEMMA_DIR, KAT_DIR):
        p = os.path.join(d, name + ".sidir")
        if os.path.exists(p):
            with open(p) as f:
                return f.read()
    raise FileNotFoundError(name)


def lemma_names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(LEMMA_DIR, "*.sidir")))


def ir_nargs(ir_text):
    for line in ir_text.splitlines():
        if line.startswith("nargs "):
            return int(line.split()[1])
    raise ValueError("no nargs line")


def ir_uses(ir_text, op):
    return any(l.startswith("node ") and l.split()[2] == op for l in ir_text.splitlines())


class Engine:
    def __init__(self, device=0):
        self.L = load()
        h = ctypes.c_void_p()
        _check(self.L.sid_engine_create(device, ctypes.byref(h)))
        self.h = h
        self._ids = {}

    def close(self):
        if self.h:
            self.L.sid_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def register(self, ir_text):
        if ir_text in self._ids:
            return self._ids[ir_text]
        lid = ctypes.c_int(-1)
        data = ir_text.encode()
        _check(self.L.sid_lemma_register(self.h, data, len(data), ctypes.byref(lid)))
        self._ids[ir_text] = lid.value
        return lid.value

    def root_box(self, lemma_id, nargs):
        out = np.zeros(2 * nargs, dtype=np.float64)
        _check(self.L.sid_lemma_root_box(self.h, lemma_id, out.ctypes.data))
        return out.reshape(nargs, 2)

    def prove(self, lemma_id, generations=8, max_iterations=1, max_criticals=1 << 20, batch=0, precision=0,
              nargs=None, fetch=False, fp32_level_mask=0xFFFFFFFF, checkpoint=None, checkpoint_every=0, stop_after=0,
              resume_from=None, fp32_noprop_mask=None, part=None, progress=None, progress_first_ms=None,
              progress_every_ms=None, device_loop=0):
        """A whole proof (sid_prove), or its continuation from a checkpoint file (resume_from, sid_prove_resume).
        checkpoint/checkpoint_every/stop_after write checkpoints and stop early (result 'complete' False);
        fp32_noprop_mask: float-pass levels without propagation (None: the engine default, all levels);
        part = (index, count): prove one shard of the root partition (counts of all shards sum to the proof's);
        progress(dict): called between steps with queue_size, cuboids, leaves, criticals and queue_head (the
        (lo, hi) pairs of one queued element, or None) after progress_first_ms, then every progress_every_ms;
        device_loop > 0: the whole proof in one persistent kernel on that many blocks (sid_prove_opts)."""
        opts = SidProveOpts()
        self.L.sid_prove_opts_default(ctypes.byref(opts))
        opts.generation_count = generations
        opts.max_iterations_per_node = max_iterations
        opts.max_criticals_kept = max_criticals
        opts.batch_elements = batch
        opts.precision = precision
        opts.fp32_level_mask = fp32_level_mask
        opts.device_loop_blocks = device_loop
        if fp32_noprop_mask is not None:
            opts.fp32_noprop_mask = fp32_noprop_mask
        if part is not None:
            opts.part_index, opts.part_count = part
        keep = None
        if progress is not None:
            n_vars = nargs

            def _cb(_user, p):
                q = p.contents
                head = None
                if q.queue_head and n_vars:
                    head = np.ctypeslib.as_array(q.queue_head, shape=(2 * n_vars,)).reshape(n_vars, 2).copy()
                progress(dict(queue_size=q.queue_size, cuboids=q.cuboid_count, leaves=q.leaf_count,
                              criticals=q.critical_count, queue_head=head))

            keep = PROGRESS_FN(_cb)
            opts.progress = ctypes.cast(keep, ctypes.c_void_p)
            if progress_first_ms is not None:
                opts.progress_first_ms = progress_first_ms
            if progress_every_ms is not None:
                opts.progress_every_ms = progress_every_ms
        opts.checkpoint_path = checkpoint.encode() if checkpoint else None
        opts.checkpoint_every_steps = checkpoint_every
        opts.stop_after_steps = stop_after
        res = SidResult()
        if resume_from:
            _check(self.L.sid_prove_resume(self.h, lemma_id, ctypes.byref(opts), resume_from.encode(), ctypes.byref(res)))
        else:
            _check(self.L.sid_prove(self.h, lemma_id, ctypes.byref(opts), ctypes.byref(res)))
        out = dict(cuboids=res.num_cuboids, leaves=res.num_leaf_cuboids, criticals=res.num_critical_cuboids,
                   repeated=res.num_repeated_nodes, stored=res.criticals_stored, escalated=res.escalated,
                   seconds=res.seconds, complete=bool(res.complete), steps=res.steps)
        if fetch and res.criticals_stored:
            buf = np.zeros(res.criticals_stored * 2 * nargs, dtype=np.float64)
            got = ctypes.c_uint64()
            _check(self.L.sid_fetch_criticals(self.h, lemma_id, buf.ctypes.data, res.criticals_stored,
                                              ctypes.byref(got)))
            out["boxes"] = buf[: got.value * 2 * nargs].reshape(-1, nargs, 2)
        return out

    def prove_bundle(self, lemma_ids, generations=8, precision=0, batch=0, max_criticals=1 << 20, blocks=0,
                     fp32_level_mask=0xFFFFFFFF, fp32_noprop_mask=None, nargs=None, fetch=False):
        """Whole proofs of several lemmas in one persistent kernel (sid_prove_bundle); a list of result dicts in
        the order of lemma_ids (with fetch and nargs, a list of n_vars per lemma: their critical boxes too)."""
        n = len(lemma_ids)
        opts = SidProveOpts()
        self.L.sid_prove_opts_default(ctypes.byref(opts))
        opts.generation_count = generations
        opts.max_criticals_kept = max_criticals
        opts.batch_elements = batch
        opts.precision = precision
        opts.fp32_level_mask = fp32_level_mask
        opts.device_loop_blocks = blocks
        if fp32_noprop_mask is not None:
            opts.fp32_noprop_mask = fp32_noprop_mask
        ids = (ctypes.c_int * n)(*lemma_ids)
        res = (SidResult * n)()
        _check(self.L.sid_prove_bundle(self.h, n, ids, ctypes.byref(opts), res))
        outs = []
        for j, r in enumerate(res):
            out = dict(cuboids=r.num_cuboids, leaves=r.num_leaf_cuboids, criticals=r.num_critical_cuboids,
                       repeated=r.num_repeated_nodes, stored=r.criticals_stored, escalated=r.escalated,
                       seconds=r.seconds, complete=bool(r.complete), steps=r.steps)
            if fetch and r.criticals_stored:
                nv = nargs[j]
                buf = np.zeros(r.criticals_stored * 2 * nv, dtype=np.float64)
                got = ctypes.c_uint64()
                _check(self.L.sid_fetch_criticals(self.h, lemma_ids[j], buf.ctypes.data, r.criticals_stored,
                                                  ctypes.byref(got)))
                out["boxes"] = buf[: got.value * 2 * nv].reshape(-1, nv, 2)
            outs.append(out)
        return outs

    def eval_batch(self, lemma_id, lo, hi):
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        n = lo.shape[1]
        out_lo = np.empty_like(lo)
        out_hi = np.empty_like(hi)
        verdict = np.empty(n, dtype=np.int8)
        _check(self.L.sid_eval_batch(self.h, lemma_id, lo.ctypes.data, hi.ctypes.data, n, out_lo.ctypes.data,
                                     out_hi.ctypes.data, verdict.ctypes.data))
        return out_lo, out_hi, verdict

    def eval_batch_device(self, lemma_id, lo_ptr, hi_ptr, n, out_lo_ptr, out_hi_ptr, verdict_ptr, stream=0):
        _check(self.L.sid_eval_batch_device(self.h, lemma_id, lo_ptr, hi_ptr, n, out_lo_ptr, out_hi_ptr,
                                            verdict_ptr, stream))

    def eval_batch_plain_device(self, lemma_id, lo_ptr, hi_ptr, n, out_lo_ptr, out_hi_ptr, verdict_ptr, stream=0):
        """The all-double batch evaluation (sid_eval_batch_plain_device) on device buffers."""
        _check(self.L.sid_eval_batch_plain_device(self.h, lemma_id, lo_ptr, hi_ptr, n, out_lo_ptr, out_hi_ptr,
                                                  verdict_ptr, stream))

    def operand_count(self, lemma_id):
        """Number of expressions the lemma's constraints compare (sid_lemma_operands)."""
        k = ctypes.c_uint32()
        _check(self.L.sid_lemma_operands(self.h, lemma_id, ctypes.byref(k)))
        return k.value

    def eval_operands_device(self, lemma_id, lo_ptr, hi_ptr, n, use_float, out_ptr, und_ptr, stream=0):
        """Interval endpoints of the compared expressions on device boxes (sid_eval_operands_device): operand j
        of box i at out[2*(j*n + i)] (lo) and out[2*(j*n + i) + 1] (hi), und[j*n + i]."""
        _check(self.L.sid_eval_operands_device(self.h, lemma_id, lo_ptr, hi_ptr, n, 1 if use_float else 0, out_ptr,
                                               und_ptr, stream))

    def eval_operands(self, lemma_id, lo, hi, use_float):
        """Host convenience over eval_operands_device: lo, hi (nargs, n) float64 -> (lohi (n, k, 2), und (n, k)),
        the layout of the oracle's eval_operands. Needs torch for the device buffers."""
        import torch
        k = self.operand_count(lemma_id)
        n = lo.shape[1]
        d_lo = torch.from_numpy(np.ascontiguousarray(lo, dtype=np.float64)).cuda()
        d_hi = torch.from_numpy(np.ascontiguousarray(hi, dtype=np.float64)).cuda()
        out = torch.empty((max(k, 1), n, 2), dtype=torch.float64, device="cuda")
        und = torch.empty((max(k, 1), n), dtype=torch.int8, device="cuda")
        stream = torch.cuda.current_stream()
        self.eval_operands_device(lemma_id, d_lo.data_ptr(), d_hi.data_ptr(), n, use_float, out.data_ptr(),
                                  und.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        o = out.cpu().numpy()[:k].transpose(1, 0, 2).copy()
        u = und.cpu().numpy()[:k].T.copy()
        return o, u

    def autotune(self, lemma_id, max_seconds=5.0):
        """Choose the precision form's step size and float-pass levels for a lemma (sid_lemma_autotune)."""
        t = SidTuning()
        _check(self.L.sid_lemma_autotune(self.h, lemma_id, max_seconds, ctypes.byref(t)))
        return dict(step_elements=t.step_elements, fp32_level_mask=t.fp32_level_mask,
                    escalation_threshold=t.escalation_threshold, levels=t.levels, candidates=t.candidates,
                    level_escalation=[t.level_escalation[k] for k in range(min(t.levels, MAX_LEVELS))],
                    seconds=t.seconds, default_seconds=t.default_seconds, fp32_noprop_mask=t.fp32_noprop_mask,
                    loop_blocks=t.loop_blocks)

    def batch_profile(self, enable):
        """Record CUDA events around the ordering and evaluation kernels of the following batch calls."""
        _check(self.L.sid_eval_batch_profile(self.h, 1 if enable else 0))

    def batch_order(self, lemma_id, mode=-1):
        """Set the lemma's batch evaluation order (BATCH_ORDER_*; -1 keeps it); returns the last sampled share
        of cuboids whose constraints needed double (-1 before any sample)."""
        share = ctypes.c_double()
        _check(self.L.sid_lemma_batch_order(self.h, lemma_id, mode, ctypes.byref(share)))
        return share.value

    def batch_profile_read(self, with_launches=False):
        """(calls, ordering ms, evaluation ms[, kernels launched]) summed over the recorded batch calls; clears
        the record."""
        calls, a, b, k = ctypes.c_uint64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_uint64()
        _check(self.L.sid_eval_batch_profile_read(self.h, ctypes.byref(calls), ctypes.byref(a), ctypes.byref(b),
                                                  ctypes.byref(k)))
        return (calls.value, a.value, b.value, k.value) if with_launches else (calls.value, a.value, b.value)

    def leaf_hull_noalloc(self, lemma_id, boxes_ptr, n, hulls_ptr, nonempty_ptr, leaves_ptr, stream=0):
        """Allocation-free leaf hulls on caller device buffers (see sid_leaf_hull_noalloc in sid.h)."""
        _check(self.L.sid_leaf_hull_noalloc(self.h, lemma_id, boxes_ptr, n, hulls_ptr, nonempty_ptr, leaves_ptr,
                                            stream))


class Server:
    """The served form (sid_server_*): requests of whole lemmas or sub-boxes, continuously batched per lemma."""

    def __init__(self, engine, precision=PRECISION_FP32, memory_budget=0, step_elements=0, generations=8,
                 max_criticals=1024, max_requests_per_lane=0, max_iterations=1):
        self.engine = engine
        self.L = engine.L
        o = SidServerOpts()
        self.L.sid_server_opts_default(ctypes.byref(o))
        o.precision = precision
        if memory_budget:
            o.memory_budget_bytes = memory_budget
        if step_elements:
            o.step_elements = step_elements
        o.generation_count = generations
        o.max_criticals_per_request = max_criticals
        if max_requests_per_lane:
            o.max_requests_per_lane = max_requests_per_lane
        o.max_iterations_per_node = max_iterations
        h = ctypes.c_void_p()
        _check(self.L.sid_server_create(engine.h, ctypes.byref(o), ctypes.byref(h)))
        self.h = h
        self.nargs = {}

    def close(self):
        if self.h:
            self.L.sid_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, lemma_id, boxes=None):
        """boxes: None for the whole lemma, else an array (nboxes, nargs, 2) of (lo, hi)."""
        rid = ctypes.c_uint64()
        if boxes is None:
            _check(self.L.sid_submit(self.h, lemma_id, None, 0, ctypes.byref(rid)))
        else:
            b = np.ascontiguousarray(boxes, dtype=np.float64)
            self.nargs[rid.value] = b.shape[1]
            _check(self.L.sid_submit(self.h, lemma_id, b.ctypes.data, b.shape[0], ctypes.byref(rid)))
        return rid.value

    def poll(self, rid):
        st = SidRequestStatus()
        _check(self.L.sid_request_poll(self.h, rid, ctypes.byref(st)))
        return st.as_dict()

    def wait(self, rid, timeout_ms=-1):
        st = SidRequestStatus()
        _check(self.L.sid_request_wait(self.h, rid, timeout_ms, ctypes.byref(st)))
        return st.as_dict()

    def criticals(self, rid, nargs, capacity):
        buf = np.zeros(max(capacity, 1) * 2 * nargs, dtype=np.float64)
        got = ctypes.c_uint64()
        _check(self.L.sid_request_criticals(self.h, rid, buf.ctypes.data, capacity, ctypes.byref(got)))
        return buf[: got.value * 2 * nargs].reshape(-1, nargs, 2)

    def release(self, rid):
        _check(self.L.sid_request_release(self.h, rid))


def synthetic_request(root, rng, k=None):
    """A seeded synthetic sub-box request: a region that covers, per coordinate, a uniform fraction in
    [2^-8, 1] of the root range at a uniform offset, delivered as k sub-boxes (a grid partition of the region;
    k = 2^j with j uniform in 0..12 unless given). Returns an array (k, nargs, 2)."""
    nargs = root.shape[0]
    lo = np.empty(nargs)
    hi = np.empty(nargs)
    for v in range(nargs):
        a, b = float(root[v, 0]), float(root[v, 1])
        f = rng.uniform(2.0 ** -8, 1.0)
        w = (b - a) * f
        off = a + rng.uniform(0.0, 1.0) * (b - a - w)
        lo[v], hi[v] = off, min(off + w, b)
    if k is None:
        k = 1 << int(rng.integers(0, 13))
    cells = np.ones(nargs, dtype=np.int64)
    while cells.prod() < k:
        cells[int(np.argmax((hi - lo) / cells))] *= 2
    grids = [np.linspace(lo[v], hi[v], cells[v] + 1) for v in range(nargs)]
    grids = [np.concatenate([g[:-1], [hi[v]]]) for v, g in enumerate(grids)]
    idx = np.stack(np.meshgrid(*[np.arange(c) for c in cells], indexing="ij"), axis=-1).reshape(-1, nargs)
    out = np.empty((idx.shape[0], nargs, 2))
    for v in range(nargs):
        out[:, v, 0] = grids[v][idx[:, v]]
        out[:, v, 1] = grids[v][idx[:, v] + 1]
    return out


def synthetic_batch(root, n, seed=0x5EED0001):
    """Seeded synthetic cuboids inside a root box: per coordinate, lo uniform over the root range and the width
    log-uniform in [2^-24, 2^-4] of the range, clipped to the box. Returns (lo, hi) of shape (nargs, n)."""
    rng = np.random.default_rng(seed)
    nargs = root.shape[0]
    lo = np.empty((nargs, n), dtype=np.float64)
    hi = np.empty((nargs, n), dtype=np.float64)
    for v in range(nargs):
        a, b = float(root[v, 0]), float(root[v, 1])
        r = b - a
        l = rng.uniform(a, b, n)
        w = np.exp2(rng.uniform(-24.0, -4.0, n)) * r
        lo[v] = l
        hi[v] = np.minimum(l + w, b)
    return lo, hi


def describe_ir(ir_text, root=None):
    """A readable account of a compiled lemma, with the sections of the reference's print_prover_input
    (prover_input/print_prover_input_impl.hpp:27-170): [Arguments] (split settings, compile-time bounds and,
    if `root` (nargs x 2) is given, the initial runtime range), [Bounds] (the runtime bound table: target,
    direction, bound function) and [Constraints] (the runtime constraint table, by row). Expressions are
    printed in infix from the IR's nodes; constants as their double enclosure."""
    import urllib.parse
    sys.path.insert(0, os.path.join(PKG, "csrc"))
    import codegen
    import tempfile
    with tempfile.NamedTemporaryFile("w", suffix=".sidir", delete=False) as f:
        f.write(ir_text)
        path = f.name
    try:
        L = codegen.Lemma(path)
    finally:
        os.unlink(path)
    names = {}
    for line in ir_text.splitlines():
        t = line.split()
        if t and t[0] == "arg":
            names[int(t[1])] = urllib.parse.unquote(t[2])
    infix = {"add": "+", "sub": "-", "mul": "*", "div": "/", "lt": "<", "le": "<=", "gt": ">", "ge": ">=",
             "eq": "==", "ne": "!=", "orseq": "||", "andseq": "&&", "or": "|", "and": "&"}

    def fx(v):
        return "%.6f" % (v / 1e6) if abs(v) < 9223372036854775807 else ("inf" if v > 0 else "-inf")

    def text(nid):
        n = L.nodes[nid]
        op = n.op
        if op == "arg":
            return names.get(n.aux, "x%d" % n.aux)
        if op == "const":
            lo, hi = float.fromhex(L.consts[n.aux][0]), float.fromhex(L.consts[n.aux][1])
            return repr(lo) if lo == hi else "[%r, %r]" % (lo, hi)
        if op == "bconst":
            return "true" if n.aux else "false"
        ch = [text(c) for c in n.ch]
        if op in infix:
            return "(" + (" %s " % infix[op]).join(ch) + ")"
        if op == "neg":
            return "-" + ch[0]
        if op == "not":
            return "!" + ch[0]
        if op == "pow":
            return "fixed_pow(%s, %d)" % (ch[0], n.aux)
        if op == "ite":
            return "if_then_else(%s, %s, %s)" % tuple(ch)
        if op in ("min", "max"):
            return ("minimum(" if op == "min" else "maximum(") + ", ".join(ch) + ")"
        return "%s(%s)" % (op, ", ".join(ch))

    out = ["[Arguments]"]
    splits = {s[0]: s for s in L.splits}
    for v in range(L.nargs):
        sp = splits.get(v)
        kind = ("Dynamic variable '%s', initial subs: %d, subs per subdivision: %d" % (names.get(v), sp[1], sp[2])
                if sp and sp[3] else "Static variable '%s', subs per subdivision: %d" % (names.get(v), sp[2])
                if sp else "Value '%s'" % names.get(v))
        lo, hi = L.ct[v]
        line = "    %d: %s, compile time bounds: [%s, %s]" % (v, kind, fx(lo), fx(hi))
        if root is not None:
            line += ", initial range: [%r, %r]" % (float(root[v][0]), float(root[v][1]))
        out.append(line)
    out.append("[Bounds]")
    for k, (tgt, d, fn, defined) in enumerate(L.bounds):
        rel = {1: "<=", 2: ">=", 3: "=="}[d]
        out.append("    %d: '%s' %s %s%s" % (k, names.get(tgt), rel, text(fn), "" if defined else "  (maybe)"))
    out.append("[Constraints]")
    for r in range(L.nargs):
        cs = L.rows.get(r, [])
        if cs:
            out.append("     %d arguments:" % (r + 1))
            for ci in cs:
                out.append("        " + text(L.constraints[ci]))
    return "\n".join(out) + "\n"


def main(argv=None):
    """Command line: prove a lemma once or more on GPU 0 and print the counts.

      python sid_gb300.py prove <lemma> [--precision 0|1|2] [--noprop MASK] [--repeat N] [--generations G]
                                [--device-loop BLOCKS]
      python sid_gb300.py bundle <lemma> <lemma> ... [--precision 0|1|2] [--repeat N] [--blocks BLOCKS]
      python sid_gb300.py describe <lemma> [--root]
    """
    import argparse
    ap = argparse.ArgumentParser(prog="sid_gb300.py")
    sub = ap.add_subparsers(dest="cmd", required=True)
    p = sub.add_parser("prove")
    p.add_argument("lemma")
    p.add_argument("--precision", type=int, default=PRECISION_PLAIN)
    p.add_argument("--repeat", type=int, default=1)
    p.add_argument("--generations", type=int, default=8)
    p.add_argument("--noprop", type=lambda v: int(v, 0), default=None,
                   help="float-pass levels without propagation (default: all)")
    p.add_argument("--device-loop", type=int, default=0,
                   help="prove in one persistent kernel on this many blocks (default: host-driven levels)")
    b = sub.add_parser("bundle", help="prove several lemmas together in one persistent kernel")
    b.add_argument("lemmas", nargs="+")
    b.add_argument("--precision", type=int, default=PRECISION_PLAIN)
    b.add_argument("--repeat", type=int, default=1)
    b.add_argument("--blocks", type=int, default=0, help="grid size (default: every block that can be resident)")
    q = sub.add_parser("describe", help="print a compiled lemma's arguments, bounds and constraints")
    q.add_argument("lemma")
    q.add_argument("--root", action="store_true", help="add the initial runtime range (needs the GPU engine)")
    args = ap.parse_args(argv)
    if args.cmd == "describe":
        ir = lemma_ir(args.lemma)
        root = None
        if args.root:
            eng = Engine(0)
            root = eng.root_box(eng.register(ir), ir_nargs(ir))
            eng.close()
        print(describe_ir(ir, root), end="")
        return 0
    eng = Engine(0)
    if args.cmd == "bundle":
        ids = [eng.register(lemma_ir(n)) for n in args.lemmas]
        for _ in range(args.repeat):
            for n, r in zip(args.lemmas, eng.prove_bundle(ids, precision=args.precision, blocks=args.blocks)):
                print(n, "precision", args.precision, r, flush=True)
        eng.close()
        return 0
    lid = eng.register(lemma_ir(args.lemma))
    for _ in range(args.repeat):
        r = eng.prove(lid, generations=args.generations, precision=args.precision, fp32_noprop_mask=args.noprop,
                      device_loop=args.device_loop)
        print(args.lemma, "precision", args.precision, r, flush=True)
    eng.close()
    return 0


if __name__ == "__main__":
    import sys
    sys.exit(main())
