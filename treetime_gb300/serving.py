"""Request loop: continuous batching of reconstruction and branch-length jobs on one GPU.

A job is one tree with its alignment and model and a number of iterations of
TreeTime's ancestral / branch-length cycle:

  * ``"marginal"``: marginal ancestral reconstruction, repeated (FP32 kernel;
    the site-specific kernel for ``GTR_site_specific`` models);
  * ``"optimize"``: TreeTime's ``optimize_tree_marginal`` (treetime/treeanc.py:
    1297-1360) with its loop run for a fixed number of iterations (no
    log-likelihood stop): marginal reconstruction, then profile-mode Brent on
    every branch below the root from the outgroup and subtree profiles
    (``optimal_marginal_branch_length``, treetime/treeanc.py:1272-1295) with the
    damped update (0.75^(i+1), tolerance 1e-8 + 0.01^(i+1)); a bifurcating
    root's two children are one branch, optimised from the first child's subtree
    profile and the second's times the root's outgroup, and its update is applied
    at the visit of each child, as TreeTime's loop does;
  * ``"joint"``: TreeTime's ``optimize_tree`` in its default joint mode without
    pruning (treetime/treeanc.py:1384-1473): joint reconstruction, then Brent on
    every branch's (parent, child) state-pair counts
    (``optimize_branch_lengths_joint``, :1176-1242), ``iterations`` rounds.
    TreeTime stops early when a reconstruction changes no state; the rounds
    after that reproduce the same states and lengths, so running them all gives
    its result.

The scheduler runs on the calling thread.  Jobs are admitted in arrival order
while a slot is free and the job's device footprint fits the memory budget
(admission by free HBM); an admitted job keeps its schedule, inputs and
profile buffers resident on the device for all its iterations and runs on its
own CUDA stream, so the kernels of every admitted job overlap on the GPU.  At
admission all of a job's iterations and the copy of its results to pinned host
memory are queued on its stream at once (the iterations need no host decision
in between), so the host does no per-iteration round trip.  Submitting a job
stages its tip codes into page-locked memory on the submitting thread (for up
to 2 x max_slots waiting jobs), so the scheduler's upload is one asynchronous
copy; a collector thread turns the
finished jobs' pinned results into arrays.  A job's numbers do not depend on
which other jobs share the GPU with it (each kernel reads only its own job's
buffers)."""

import collections
import copy
import queue
import threading
import time

import numpy as np

from . import engine

KINDS = ("marginal", "optimize", "joint")


class Job:
    """One request: ``inputs`` (an ``engine.TreeInput``), ``gtr`` (GTR or
    GTR_site_specific), ``kind`` and ``iterations``.  After completion
    ``result`` holds ``tree_lh`` (per iteration), ``states`` (the internal
    nodes' reconstructed state indices, [n_int, P]) and ``branch_lengths``
    (the final ones, per node), and ``t_submit`` / ``t_admit`` / ``t_done``
    the host clock at those events (seconds)."""

    _next_id = 0

    def __init__(self, inputs, gtr, kind="marginal", iterations=3, job_id=None):
        if kind not in KINDS:
            raise ValueError("kind must be one of %s" % (KINDS,))
        if kind != "marginal" and getattr(gtr, "is_site_specific", False):
            raise NotImplementedError("branch-length jobs need a standard GTR model")
        if kind == "optimize" and inputs.masks:
            raise NotImplementedError("branch-length jobs with masks are not supported in the serving loop")
        engine.check_alphabet(gtr.n_states, getattr(gtr, "is_site_specific", False))
        self.inputs = inputs
        self.gtr = gtr
        self.kind = kind
        self.iterations = int(iterations)
        if self.iterations < 1:
            raise ValueError("a job runs at least one iteration")
        self.site_specific = bool(getattr(gtr, "is_site_specific", False))
        if job_id is None:
            job_id = Job._next_id
            Job._next_id += 1
        self.id = job_id
        self.t_submit = self.t_admit = self.t_done = None
        self.result = None
        self.error = None
        self.footprint = footprint(inputs, gtr.n_states, kind)
        self._codes_buf = None

    def stage(self, pool):
        """Copy the tip codes into a page-locked buffer of `pool` (done by the
        submitting thread; the admission's upload then copies from it)."""
        codes = self.inputs.tip_codes.reshape(-1)
        buf = pool.take(codes.nbytes)
        np.copyto(buf[:codes.nbytes].numpy(), codes)
        self._codes_buf = buf

    @property
    def node_patterns(self):
        """Node-pattern updates of one iteration."""
        return self.inputs.layout.n_nodes * self.inputs.n_patterns

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit


def footprint(inputs, q, kind):
    """Upper estimate of the device bytes a job holds while admitted: FP32
    partial / posterior / outgroup rows, states, tip codes, branch matrices
    (FP64, FP32 and the paired FP32 copy), schedule arrays."""
    lay, P = inputs.layout, inputs.n_patterns
    w = engine.WIDTHS[q]
    rows = lay.n_int * P * w * 4
    prof = rows * (3 if kind == "optimize" else 2) + (lay.n_tip * P * w * 4 if kind == "optimize" else 0)
    mats = lay.n_nodes * q * w * (8 + 4 + 8)
    other = lay.n_nodes * P + inputs.tip_codes.size + lay.n_nodes * 64 + P * 24
    return int((prof + mats + other) * 1.1) + (1 << 20)


def plan_admissions(queue, free_slots, free_bytes):
    """Jobs to admit now, in arrival order: each while a slot is free and its
    footprint fits the free bytes.  A job that does not fit waits at the head
    of the queue (later, smaller jobs do not overtake it, so none starves)."""
    out = []
    for job in queue:
        if free_slots <= 0 or job.footprint > free_bytes:
            break
        out.append(job)
        free_slots -= 1
        free_bytes -= job.footprint
    return out


class _PinnedPool:
    """Reusable page-locked host buffers by power-of-two size class (a fresh
    page-locked allocation of a large job's results costs milliseconds); shared
    by the submitting, scheduling and collecting threads."""

    def __init__(self):
        self.free = collections.defaultdict(list)
        self.lock = threading.Lock()

    def take(self, nbytes):
        t = engine.torch()
        cls = max(1 << 12, 1 << int(np.ceil(np.log2(max(1, nbytes)))))
        with self.lock:
            if self.free[cls]:
                return self.free[cls].pop()
        return t.empty(cls, dtype=t.uint8, pin_memory=True)

    def give(self, buf):
        with self.lock:
            self.free[buf.numel()].append(buf)


_POOL = None


def pinned_pool():
    """The process's pinned-buffer pool (one per process, so that warm-up runs
    prime it for later servers)."""
    global _POOL
    if _POOL is None:
        _POOL = _PinnedPool()
    return _POOL


def _view(buf, shape, dtype):
    t = engine.torch()
    n = int(np.prod(shape)) * t.empty((), dtype=dtype).element_size()
    return buf[:n].view(dtype).view(shape)


class _Active:
    """Device state of an admitted job."""

    def __init__(self, job, server):
        t = engine.torch()
        self.job = job
        self.pool = server._pinned
        self.stream = server._stream_pool.pop() if server._stream_pool else t.cuda.Stream(device=server.device)
        dev = server.device
        ti = copy.copy(job.inputs)
        ti.model = 0  # the job's own one-model DeviceModel
        if job._codes_buf is not None:
            ti.tip_codes_pinned = job._codes_buf[:ti.tip_codes.size]
        hs = server.host_s
        with t.cuda.stream(self.stream):
            self.forest = engine.Forest([ti], job.gtr.n_states, device=dev)
            hs["admit.forest_host"] += self.forest.build_s[0]
            hs["admit.forest_upload"] += self.forest.build_s[1]
            t0 = time.perf_counter()
            self.bufs = engine.Buffers(self.forest)
            self.model = None if job.site_specific else engine.model_for(job.gtr, dev)
            self.lh = t.zeros(job.iterations, dtype=t.float64, device=dev)
            self.status = t.zeros(1, dtype=t.int32, device=dev)
            t1 = time.perf_counter()
            hs["admit.model"] += t1 - t0
            if job.kind == "optimize":
                self._prepare_optimize(dev)
                hs["admit.optimize_setup"] += time.perf_counter() - t1
            elif job.kind == "joint":
                self._prepare_joint(dev)
                hs["admit.optimize_setup"] += time.perf_counter() - t1
        self.it = 0
        self.done_event = None
        self.host = None
        self.phase_events = [] if server.phase_events else None

    def _prepare_joint(self, dev):
        lay = self.job.inputs.layout
        up = engine.Uploader()
        up.add("char_state", engine.char_state_table(self.job.gtr))
        up.add("bl", np.asarray(self.job.inputs.bl, np.float64))
        d = up.finish(dev)
        self.opt = dict(d, floor=engine.ttconf.MIN_BRANCH_LENGTH / float(self.job.inputs.mult.sum()),
                        root=lay.n_int - 1)

    def _prepare_optimize(self, dev):
        t = engine.torch()
        lay, P = self.job.inputs.layout, self.job.inputs.n_patterns
        k = np.arange(lay.n_nodes)
        has_parent = np.asarray(lay.parent) >= 0
        root = lay.n_int - 1
        rc = lay.child_idx[lay.child_off[root]:lay.child_off[root + 1]]
        pair = None
        if len(rc) == 2:  # a bifurcating root: its two children are one branch
            pair = (int(rc[0]), int(rc[1]))
            has_parent = has_parent & (k != pair[0]) & (k != pair[1])
        internal = k[has_parent & (k < lay.n_int)]
        tips = k[has_parent & (k >= lay.n_int)]
        up = engine.Uploader()
        up.add("n_int32", internal.astype(np.int32)).add("n_tip32", tips.astype(np.int32))
        up.add("int_rows", internal.astype(np.int64) * P).add("tip_rows", (tips - lay.n_int).astype(np.int64) * P)
        up.add("no_rows", np.full(len(tips), -1, np.int64))
        up.add("d_int", internal.astype(np.int64)).add("d_tip", tips.astype(np.int64))
        up.add("bl", np.asarray(self.job.inputs.bl, np.float64))
        d = up.finish(dev)
        rp = None
        if pair is not None:
            rp = engine.RootPair(self.forest, lay, pair[0], pair[1], self.job.inputs.tip_codes, self.job.inputs.tip_row)
        self.opt = dict(d, internal=len(internal) > 0, tips=len(tips) > 0, pair=pair, root_pair=rp,
                        floor=engine.ttconf.MIN_BRANCH_LENGTH / float(self.job.inputs.mult.sum()))

    def enqueue_iteration(self):
        """Queue one iteration on the job's stream (no host synchronisation)."""
        t = engine.torch()
        job = self.job
        ev = self.phase_events
        with t.cuda.stream(self.stream):
            if ev is not None:
                ev.append(("start", self._event()))
            if job.kind == "joint":
                out = engine.joint(self.forest, self.model, self.bufs, sync=False)
            elif job.site_specific:
                out = engine.marginal_site_specific(self.forest, job.gtr, self.bufs, precision="f32", sync=False)
            else:
                keep = job.kind == "optimize"
                out = engine.marginal(self.forest, self.model, self.bufs, precision="f32", keep_outgroup=keep,
                                      tip_outgroup=keep, sync=False)
            self.lh[self.it].copy_(out["tree_lh"][0])
            self.status.copy_(t.maximum(self.status, self.bufs.get("status", (1,), t.int32)))
            if ev is not None:
                ev.append(("marginal", self._event()))
            if job.kind == "optimize":
                self._branch_lengths(out)
                if ev is not None:
                    ev.append(("branch_lengths", self._event()))
            elif job.kind == "joint":
                self._joint_lengths()
                if ev is not None:
                    ev.append(("branch_lengths", self._event()))
            self.out = out
        self.it += 1

    def _event(self):
        e = engine.torch().cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e

    def phase_ms(self):
        """Device milliseconds per phase (marginal, branch_lengths) summed over
        the iterations, from the events recorded when the server was created
        with ``phase_events=True`` (meaningful for a job that ran alone)."""
        out = collections.Counter()
        prev = None
        for name, e in self.phase_events or ():
            if prev is not None and name != "start":
                out[name] += prev.elapsed_time(e)
            prev = e
        return out

    def _joint_lengths(self):
        """optimize_branch_lengths_joint on the device: pair counts of every branch
        from the last joint reconstruction (tips: their characters; gaps
        ignored), truncated to integers, Brent on each, lengths max(0, t); the
        model's lengths are floored at 1e-3 / L for the next reconstruction."""
        import ctypes as C
        t = engine.torch()
        o = self.opt
        q = self.job.gtr.n_states
        gap = self.job.gtr.gap_index
        hist = self.bufs.get("hist", (self.forest.n_nodes, q, q), t.float64)
        hist.zero_()
        states = self.bufs.get("states", (self.forest.state_rows,), t.uint8)
        engine.check(engine._lib.load().tt_state_pairs(
            C.byref(self.forest.struct), engine._p(states), engine._p(o["char_state"]), 0,
            -1 if gap is None else int(gap), 1, None, engine._p(hist), engine._stream()), "tt_state_pairs")
        tt, info = engine.optimal_t_pairs(q, t.trunc(hist), self.model, tol=1e-10)
        new = t.clamp(tt, min=0.0)
        new[o["root"]] = o["bl"][o["root"]]
        o["bl"] = new
        info = info.clone()
        info[o["root"]] = 0  # the root has no branch (TreeTime does not optimise it)
        bad = (info == -1).any().to(t.int32) * engine._lib.TT_ERR_BRACKET
        self.status.copy_(t.maximum(self.status, bad.reshape(1)))
        self.forest.d_bl.copy_(t.clamp(new, min=o["floor"]))

    def _root_pair(self, out, tol, damp):
        """The bifurcating root's children as one branch (treetime/treeanc.py:
        1317-1339): Brent from the first child's subtree profile and the second
        child's subtree profile times the root's outgroup (pi), normalised; the
        damped update of the pair's total length, split in the current ratio,
        applied twice (TreeTime's loop meets the pair at both children)."""
        o = self.opt
        n1, n2 = o["pair"]
        tn = o["root_pair"].optimal_t(self.model, out["partial"], self.job.gtr.gap_index, tol)
        bl = o["bl"]
        for _visit in range(2):
            total = bl[n1] + bl[n2]
            ratio = bl[n1] / total
            upd = tn[0] * (1 - damp) + total * damp
            bl[n1] = upd * ratio
            bl[n2] = upd * (1 - ratio)

    def _branch_lengths(self, out):
        t = engine.torch()
        o = self.opt
        damp = 0.75 ** (self.it + 1)      # iteration i damps with 0.75^(i+1) ...
        old = o["bl"]
        new = old.clone()
        tol = 1e-8 + 0.01 ** (self.it + 1)  # ... and optimises to 1e-8 + 0.01^(i+1)
        gap = self.job.gtr.gap_index
        if o["internal"]:
            ti, _ = engine.optimal_t_profiles_dev(self.forest, self.model, o["n_int32"], out["outgroup"],
                                                  o["int_rows"], out["partial"], o["int_rows"], "f32", gap, True, tol)
            new[o["d_int"]] = ti * (1 - damp) + old[o["d_int"]] * damp
        if o["tips"]:
            tt, _ = engine.optimal_t_profiles_dev(self.forest, self.model, o["n_tip32"], out["tip_outgroup"],
                                                  o["tip_rows"], out["partial"], o["no_rows"], "f32", gap, True, tol)
            new[o["d_tip"]] = tt * (1 - damp) + old[o["d_tip"]] * damp
        o["bl"] = new
        if o["pair"] is not None:
            self._root_pair(out, tol, damp)
            new = o["bl"]
        self.forest.d_bl.copy_(t.clamp(new, min=o["floor"]))

    def enqueue_results(self):
        """Copy the results to pinned host memory on the job's stream."""
        t = engine.torch()
        lay, P = self.job.inputs.layout, self.job.inputs.n_patterns
        pool = self.pool
        with t.cuda.stream(self.stream):
            states = self.out["states"][: lay.n_int * P]
            self._bufs = [pool.take(self.lh.numel() * 8), pool.take(states.numel()),
                          pool.take(self.forest.d_bl.numel() * 8), pool.take(4)]
            self.host = dict(tree_lh=_view(self._bufs[0], self.lh.shape, t.float64),
                             states=_view(self._bufs[1], states.shape, t.uint8),
                             bl=_view(self._bufs[2], self.forest.d_bl.shape, t.float64),
                             status=_view(self._bufs[3], (1,), t.int32))
            self.host["tree_lh"].copy_(self.lh, non_blocking=True)
            self.host["states"].copy_(states, non_blocking=True)
            self.host["bl"].copy_(self.forest.d_bl, non_blocking=True)
            self.host["status"].copy_(self.status, non_blocking=True)
            self.done_event = t.cuda.Event()
            self.done_event.record(self.stream)

    def collect(self):
        """Arrays from the pinned results (the job's stream has finished); a
        device error status becomes the job's ``error``, raised as
        ``engine.check`` raises it.  Returns the pinned buffers to the pool."""
        lay, P = self.job.inputs.layout, self.job.inputs.n_patterns
        try:
            st = int(self.host["status"][0])
            if st:
                engine.check(st, "serving job %s" % self.job.id)
            self.job.result = dict(tree_lh=self.host["tree_lh"].numpy().copy(),
                                   states=self.host["states"].numpy().reshape(lay.n_int, P).copy(),
                                   branch_lengths=self.host["bl"].numpy().copy())
        except Exception as e:  # noqa: BLE001 -- handed to the caller of run()
            self.job.error = e
        finally:
            for b in self._bufs:
                self.pool.give(b)
            if self.job._codes_buf is not None:
                self.pool.give(self.job._codes_buf)
                self.job._codes_buf = None


class Server:
    """Continuous-batching scheduler for one GPU.

    ``max_slots``: jobs admitted at the same time (each gets a CUDA stream);
    ``hbm_bytes``: device-memory budget for admitted jobs (default: 80% of the
    free memory when the server starts)."""

    def __init__(self, device=None, max_slots=16, hbm_bytes=None, poll_s=2e-5, phase_events=False):
        t = engine.torch()
        self.device = engine.require_device(device)
        if hbm_bytes is None:
            free, _ = t.cuda.mem_get_info(self.device)
            hbm_bytes = int(free * 0.8)
        self.max_slots = int(max_slots)
        self.hbm_bytes = int(hbm_bytes)
        self.poll_s = poll_s
        # per-phase device times of each job (job.phase_ms), for jobs run alone
        self.phase_events = bool(phase_events)
        self._queue = collections.deque()
        self._lock = threading.Lock()
        self._active = []
        self._stream_pool = []
        self._pinned = pinned_pool()
        self._finished = queue.Queue()
        self._collecting = 0
        self._staged_waiting = 0
        self._errors = []
        self.done = []
        self.peak_active = 0
        self.peak_bytes = 0
        # host seconds spent per phase (admission, enqueueing, result copies; collection on the
        # collector thread)
        self.host_s = collections.Counter()

    def submit(self, job):
        """Queue a job (thread-safe); the scheduler loop admits it.  While
        fewer than ``2 * max_slots`` queued jobs hold staged codes, the job's
        tip codes are staged into pinned memory on the calling thread (a long
        queue does not pin the host memory of every waiting job; the others
        are packed at admission)."""
        if job.footprint > self.hbm_bytes:
            # it could never be admitted and would hold the head of the queue for good
            raise MemoryError("job %s needs about %d bytes of device memory, the server's budget is %d"
                              % (job.id, job.footprint, self.hbm_bytes))
        job.t_submit = time.perf_counter()
        with self._lock:
            stage = self._staged_waiting < 2 * self.max_slots
            if stage:
                self._staged_waiting += 1
        if stage:
            job.stage(self._pinned)
        with self._lock:
            self._queue.append(job)

    def _used_bytes(self):
        return sum(a.job.footprint for a in self._active)

    def step(self):
        """One scheduler pass; returns True when something happened."""
        busy = False
        # finished jobs leave first: their slots and memory go to the queue, their results to the
        # collector thread
        still = []
        for a in self._active:
            if a.done_event.query():
                self._stream_pool.append(a.stream)
                with self._lock:
                    self._collecting += 1
                self._finished.put(a)
                busy = True
            else:
                still.append(a)
        self._active = still
        with self._lock:
            plan = plan_admissions(self._queue, self.max_slots - len(self._active),
                                   self.hbm_bytes - self._used_bytes())
            for job in plan:
                self._queue.popleft()
                if job._codes_buf is not None:
                    self._staged_waiting -= 1
        for job in plan:
            job.t_admit = time.perf_counter()
            try:
                a = _Active(job, self)
                t1 = time.perf_counter()
                while a.it < job.iterations:
                    a.enqueue_iteration()
                t2 = time.perf_counter()
                a.enqueue_results()
            except Exception as e:  # noqa: BLE001 -- e.g. a device allocation that failed
                # the job fails alone: its slot and budget go back to the queue, run() raises the
                # error once the other jobs have finished
                self._fail_admission(job, e)
                busy = True
                continue
            self.host_s["admit"] += t1 - job.t_admit
            self.host_s["enqueue"] += t2 - t1
            self.host_s["results"] += time.perf_counter() - t2
            self._active.append(a)
            busy = True
        self.peak_active = max(self.peak_active, len(self._active))
        self.peak_bytes = max(self.peak_bytes, self._used_bytes())
        return busy

    def _fail_admission(self, job, err):
        job.error = err
        job.t_done = time.perf_counter()
        if job._codes_buf is not None:
            self._pinned.give(job._codes_buf)
            job._codes_buf = None
        with self._lock:
            self.done.append(job)
            self._errors.append(err)

    def _collect_loop(self):
        while True:
            a = self._finished.get()
            if a is None:
                return
            t0 = time.perf_counter()
            a.collect()
            if a.phase_events is not None:
                a.job.phase_ms = dict(a.phase_ms())
            a.job.t_done = time.perf_counter()
            with self._lock:
                self.host_s["collect"] += a.job.t_done - t0
                self.done.append(a.job)
                if a.job.error is not None:
                    self._errors.append(a.job.error)
                self._collecting -= 1

    def pending(self):
        with self._lock:
            return len(self._queue) + len(self._active) + self._collecting

    def run(self, until=None):
        """Scheduler loop until the queue and the GPU are empty (and, when
        given, until() is true).  Raises the first device error of a job
        finished in this run, after the others have finished."""
        collector = threading.Thread(target=self._collect_loop, daemon=True)
        collector.start()
        try:
            while True:
                busy = self.step()
                if not busy:
                    if self.pending() == 0 and (until is None or until()):
                        break
                    time.sleep(self.poll_s)
        finally:
            self._finished.put(None)
            collector.join()
        with self._lock:
            errors, self._errors = self._errors, []
        if errors:
            raise errors[0]

    def serve(self, jobs, arrival_times):
        """Submit ``jobs`` at ``arrival_times`` (seconds from now, from a feeder
        thread) and run the loop until all are done.  Returns the finished jobs
        and the wall time."""
        order = np.argsort(arrival_times)
        t0 = time.perf_counter()
        fed = threading.Event()

        def feeder():
            for i in order:
                delay = t0 + arrival_times[i] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                self.submit(jobs[i])
            fed.set()

        th = threading.Thread(target=feeder, daemon=True)
        th.start()
        self.run(until=fed.is_set)
        th.join()
        return list(jobs), time.perf_counter() - t0


def latency_stats(jobs):
    """p50 / p99 / max latency (s) and node-pattern updates of finished jobs."""
    lat = np.array([j.latency for j in jobs if j.latency is not None])
    units = sum(j.node_patterns * j.iterations for j in jobs if j.t_done is not None)
    if lat.size == 0:
        return dict(p50=None, p99=None, max=None, node_pattern_updates=units)
    return dict(p50=float(np.percentile(lat, 50)), p99=float(np.percentile(lat, 99)), max=float(lat.max()),
                node_pattern_updates=int(units))
