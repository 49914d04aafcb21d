"""Continuous-batching request loop for the eigensubstitution path.

Jobs (alignment, tree, model, options) arrive over time.  The loop

* admits a waiting job as soon as a device slot is free and its device
  footprint (plan tables + tokens + outputs + workspace estimate) fits the
  memory budget — requests that arrive while others are on the GPU are
  admitted while those run; among waiting jobs the one with the smallest
  estimated device time goes first, less a credit that grows with its wait
  (``aging``), so long jobs are delayed but not starved;
* keeps prepared plans (tree tables, eigendecomposition-derived tables, J(t))
  resident in HBM in an LRU cache keyed by (tree, model), so a repeated
  tree/model pays no preparation;
* stages each job's tokens from pinned host memory on the slot's own CUDA
  stream, enqueues the kernel on that stream and reads the results back on
  it, so the work of concurrent jobs overlaps on the device (a small job's
  grid covers only the SMs its columns need, leaving the rest to others);
* never runs two jobs of the same plan at once (a plan's workspace is
  per-plan), so such a job waits for its twin to finish;
* completes jobs in whatever order their streams finish and records, per job,
  the latency from arrival to results-in-host-memory;
* estimates each job's device time from its shape (``job_cost_ms``): short
  jobs go to high-priority streams, so the block scheduler starts their
  kernels ahead of queued work of long jobs, and long jobs are cut into
  column slices of about ``slice_ms`` each (whole waves of the persistent
  kernels' grids), so a short job waits for at most one slice rather than a
  whole long job.

Results of a job do not depend on what else is in flight: every job runs the
same kernel on the same inputs as it would alone (``tests/test_gpu_serving``
checks this).
"""
from __future__ import annotations

import collections
import ctypes as ct
import hashlib
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .api import Plan
from .models import ensure_diag
from . import batch


@dataclass
class HostRows:
    """A job's alignment held as rows of a larger pinned host buffer: row r
    of the job is row ``rowmap[r]`` of ``base`` (``rowmap`` a CUDA int32
    tensor of R entries, or None for row r), columns [col0, col0 + C).  The
    server uploads it with one gather kernel (subby_gather_rows) on the
    job's stream, the SMs reading the host rows over the host link."""
    base: object          # pinned CPU torch int32 tensor (rows, pitch)
    col0: int
    rowmap: object        # int32 row indices (R,): a CUDA tensor for Server,
    #                       a host array for NativeServer; or None
    R: int
    C: int

    @property
    def shape(self):
        return (self.R, self.C)

    @property
    def nbytes(self):
        return 4 * self.R * self.C


@dataclass
class Job:
    id: int
    alignment: object              # (R, C) int32: host array, CUDA tensor,
    #                                HostRows (rows of a pinned host buffer), or
    #                                a callable(stream, device, out) that fills
    #                                the (R, C) int32 CUDA tensor ``out``
    tree: object
    model: object
    f81: bool = False
    branch_mask: object = "auto"
    want: tuple = ("counts",)      # subset of ("logLike", "counts", "rootProb")
    arrival: float = 0.0           # seconds since the loop started
    shape: tuple = None            # (R, C), required when alignment is a callable
    # filled by the server
    start: float = -1.0
    finish: float = -1.0
    result: dict = field(default_factory=dict)
    error: str = ""                # set when the device reported a failed wait

    @property
    def latency(self):
        return self.finish - self.arrival

    def release(self):
        """Drop the results; their pinned host buffers go back to the server."""
        self.result = {}
        blocks, self._pinned = getattr(self, "_pinned", None), None
        cb = getattr(self, "_give_back", None)
        if blocks and cb is not None:
            cb(blocks)

    @property
    def RC(self):
        return tuple(self.shape) if self.shape is not None else tuple(self.alignment.shape)


def _plan_key(tree, model):
    m = ensure_diag(model)
    h = hashlib.sha1()
    for a in (tree.parentIndex, tree.distanceToParent):
        h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    h.update(batch._key(m).encode())   # every model field, complex ones included
    return h.hexdigest()


STAGE_CAP = 4 << 30   # per-plan staging cap of the large-alphabet path (bytes)

# Device time per (column x tree node), ns, by path (GB300, Counts): used only
# to order and slice work, never to skip any.
_NS_PER_COL_NODE = {("4", False): 0.012, ("4", True): 0.011, ("16", False): 0.30, ("16", True): 0.10,
                    ("64", False): 1.2, ("64", True): 0.70}


def job_cost_ms(R: int, C: int, A: int, f81: bool = False) -> float:
    """Estimated device time of one job's Counts call (ms): kernels, plus
    the host-link time of its tokens (~200 GB/s) and counts (~170 GB/s)."""
    key = ("4" if A <= 8 else "16" if A <= 20 else "64", bool(f81))
    return _NS_PER_COL_NODE[key] * R * C * 1e-6 + 4.0 * C * A * A / 1.7e8 + 4.0 * R * C / 2.0e8


def job_device_bytes(R: int, C: int, A: int) -> int:
    """Device footprint estimate of one in-flight job (bytes): plan tables,
    tokens, outputs and the plan's scratch (per-branch staging of the
    large-alphabet Counts path, capped per plan; slot scratch otherwise)."""
    tables = 4 * R * (A + 1) * A * 6 + 4 * R * (A + 1) * (A * A + 4) * (A <= 8)
    tokens = 4 * R * C
    outputs = 4 * C * (A * A + A + 1)
    if A >= 16:
        scratch = min(STAGE_CAP, 8 * (R - 1) * A * C) + 4 * R * (A + 1) * min(C, 152 * 128)
    else:
        scratch = 4 * R * (A + 2) * min(C, 152 * 256)
    return tables + tokens + outputs + scratch


class Server:
    """Continuous batching over CUDA streams with memory-budget admission."""

    def __init__(self, max_inflight: int = 8, device_budget: int = 16 << 30, plan_cache: int = 64,
                 device=None, short_ms: float = 5.0, slice_ms: float = 8.0, aging: float = 0.2,
                 short_slots: int = 2, wave_cols: int = 0):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.max_inflight = max_inflight
        self.budget = device_budget
        self.short_ms = short_ms
        self.slice_ms = slice_ms
        self.aging = aging          # ms of estimated cost forgiven per ms waited
        self.short_slots = min(short_slots, max_inflight - 1)
        self.wave_cols = wave_cols  # slice granularity (0: one wave of the kernels' grids)
        # one normal- and one high-priority stream per slot
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(max_inflight)]
        self.hi_streams = [torch.cuda.Stream(device=self.device, priority=-8) for _ in range(max_inflight)]
        self.arenas = [None] * max_inflight
        self.nsm = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.free_slots = list(range(max_inflight))
        self.plans = collections.OrderedDict()
        self.plan_cache = plan_cache
        self.inflight = []           # (job, slot, event, bytes, bufs)
        self.used_bytes = 0
        self.completed = []
        self.on_done = None
        self.pinned_free = {}    # size class -> free pinned blocks
        # host seconds spent preparing plans, enqueueing jobs and polling
        self.host_s = {"plan": 0.0, "launch": 0.0, "poll": 0.0, "tokens": 0.0, "run": 0.0, "result": 0.0}
        self.lock = threading.Lock()

    # ------------------------------------------------------- pinned buffers
    # Result buffers come from a server-owned pool of pinned host blocks in
    # power-of-two size classes: page pinning costs milliseconds per large
    # block, so blocks are reused instead of allocated per job.
    def _pinned(self, nbytes: int):
        cls = max(1 << 16, 1 << (max(int(nbytes), 1) - 1).bit_length())
        free = self.pinned_free.setdefault(cls, [])
        return free.pop() if free else self.torch.empty(cls, dtype=self.torch.uint8, pin_memory=True)

    def _give_back(self, blocks):
        for b in blocks:
            self.pinned_free.setdefault(b.numel(), []).append(b)

    def prewarm(self, host_bytes: int = 0, device_bytes: int = 0, per_class: int = 2):
        """Fill the caches before serving: one device block of
        ``device_bytes`` for torch's caching allocator to split, and
        ``per_class`` pinned host blocks of every power-of-two size up to
        ``host_bytes`` in the server's pool."""
        torch = self.torch
        if device_bytes > 0:
            x = torch.empty(int(device_bytes), dtype=torch.uint8, device=self.device)
            del x
        size = 1 << 16
        while size <= host_bytes:
            self._give_back([torch.empty(size, dtype=torch.uint8, pin_memory=True) for _ in range(per_class)])
            size <<= 1

    # ------------------------------------------------------------------ plans
    @staticmethod
    def _key(job):
        k = getattr(job, "_plan_key", None)
        if k is None:
            k = _plan_key(job.tree, job.model)
            job._plan_key = k
        return k

    def plan_for(self, tree, model, key=None) -> Plan:
        k = key or _plan_key(tree, model)
        p = self.plans.get(k)
        if p is not None:
            self.plans.move_to_end(k)
            return p
        t0 = time.perf_counter()
        p = Plan(tree, model, device=self.device)
        self.host_s["plan"] += time.perf_counter() - t0
        self.plans[k] = p
        while len(self.plans) > self.plan_cache:
            self.plans.popitem(last=False)[1].close()
        return p

    # ---------------------------------------------------------------- submit
    # ----------------------------------------------------------- slot arenas
    # Each slot owns one device arena that grows to the largest job it has
    # served; a job's tokens, outputs and slice temporaries are carved from
    # it, so enqueueing a job allocates nothing (allocation calls can stall
    # the host while the device is busy).
    def _arena(self, slot: int, nbytes: int):
        torch = self.torch
        a = self.arenas[slot]
        if a is None or a.numel() < nbytes:
            self.arenas[slot] = None
            a = torch.empty(1 << (max(int(nbytes), 1 << 20) - 1).bit_length(), dtype=torch.uint8,
                            device=self.device)
            self.arenas[slot] = a
        return a

    @staticmethod
    def _carve(buf, plan_list):
        """Views of ``buf`` for [(name, shape, dtype), ...] at 256-byte offsets."""
        out, off = {}, 0
        for name, shape, dtype in plan_list:
            n = int(np.prod(shape)) * dtype.itemsize
            out[name] = buf[off:off + n].view(dtype).view(shape)
            off = (off + n + 255) & ~255
        return out

    def _launch(self, job: Job, now: float):
        torch = self.torch
        R, C = job.RC
        A = len(ensure_diag(job.model).pi)
        nbytes = job_device_bytes(R, C, A)
        slot = self.free_slots.pop()
        cost = job_cost_ms(R, C, A, job.f81)
        stream = (self.hi_streams if cost <= self.short_ms else self.streams)[slot]
        plan = self.plan_for(job.tree, job.model, self._key(job))
        kw = dict(loglike="logLike" in job.want, counts="counts" in job.want,
                  rootprob="rootProb" in job.want, f81=job.f81, branch_mask=job.branch_mask)
        # slices are whole waves of the kernels' persistent grids (a thinner
        # slice runs as long as a full wave on fewer SMs)
        wave = self.wave_cols or self.nsm * (128 if A == 64 else 256)
        nsl = max(1, min(int(np.ceil(cost / self.slice_ms)), (C + wave - 1) // wave))
        if not isinstance(job.branch_mask, str):
            nsl = 1
        cmax = C if nsl == 1 else ((C + nsl - 1) // nsl + wave - 1) // wave * wave
        nsl = (C + cmax - 1) // cmax
        f32, i32 = torch.float32, torch.int32
        shapes = {"logLike": (C,), "counts": (A, A, C), "rootProb": (A, C)}
        want = [k for k in ("logLike", "counts", "rootProb") if k in job.want]
        layout = [("aln", (R, C), i32)] + [(k, shapes[k], f32) for k in want]
        if nsl > 1:
            layout += [("s_aln", (R * cmax,), i32)] + [("s_" + k, (int(np.prod(shapes[k][:-1])) * cmax,), f32)
                                                       for k in want]
        need = sum((int(np.prod(sh)) * dt.itemsize + 255) & ~255 for _, sh, dt in layout)
        v = self._carve(self._arena(slot, need), layout)
        res = {k: v[k] for k in want}
        t_tok = time.perf_counter()
        pinned_in = None
        with torch.cuda.stream(stream):
            if isinstance(job.alignment, HostRows):
                hr = job.alignment
                pitch = int(hr.base.stride(0))
                src = hr.base.data_ptr() + 4 * int(hr.col0)
                rm = hr.rowmap.data_ptr() if hr.rowmap is not None else None
                _lib.check(_lib.load().subby_gather_rows(
                    ct.c_void_p(src), pitch, None if rm is None else ct.c_void_p(rm), R, C,
                    ct.c_void_p(v["aln"].data_ptr()), ct.c_void_p(stream.cuda_stream)), "subby_gather_rows")
                d_aln = v["aln"]
            elif callable(job.alignment):
                job.alignment(stream, self.device, v["aln"])
                d_aln = v["aln"]
            elif isinstance(job.alignment, torch.Tensor) and job.alignment.is_cuda:
                d_aln = job.alignment
            else:
                src = np.ascontiguousarray(job.alignment, dtype=np.int32)
                pinned_in = self._pinned(src.nbytes)
                h = pinned_in[:src.nbytes].view(i32).view(R, C)
                h.numpy()[:] = src
                v["aln"].copy_(h, non_blocking=True)
                d_aln = v["aln"]
            t_run = time.perf_counter()
            self.host_s["tokens"] += t_run - t_tok
            if nsl == 1:
                plan.run(d_aln, stream=stream, out=res, **kw)
            else:
                # long job: column slices of whole 128-column tiles, each its
                # own launch sequence, results gathered on the device
                edges = [min(C, i * cmax) for i in range(nsl)] + [C]
                for c0, c1 in zip(edges[:-1], edges[1:]):
                    cc = c1 - c0
                    if cc <= 0:
                        continue
                    s_aln = v["s_aln"][:R * cc].view(R, cc)
                    s_aln.copy_(d_aln[:, c0:c1])
                    part = {k: v["s_" + k][:int(np.prod(shapes[k][:-1])) * cc].view(shapes[k][:-1] + (cc,))
                            for k in want}
                    plan.run(s_aln, stream=stream, out=part, **kw)
                    for k in want:
                        res[k][..., c0:c1].copy_(part[k])
            t_pin = time.perf_counter()
            self.host_s["run"] += t_pin - t_run
            host, blocks = {}, ([pinned_in] if pinned_in is not None else [])
            for k, r in res.items():
                blk = self._pinned(r.numel() * r.element_size())
                blocks.append(blk)
                hv = blk[:r.numel() * r.element_size()].view(r.dtype).view(r.shape)
                hv.copy_(r, non_blocking=True)
                host[k] = hv
            self.host_s["result"] += time.perf_counter() - t_pin
            ev = torch.cuda.Event()
            ev.record(stream)
        job.start = now
        self.used_bytes += nbytes
        self.inflight.append((job, slot, ev, nbytes, (None, d_aln, res, host, blocks)))

    def _cost(self, job: Job) -> float:
        c = getattr(job, "_cost_ms", None)
        if c is None:
            R, C = job.RC
            c = job._cost_ms = job_cost_ms(R, C, len(ensure_diag(job.model).pi), job.f81)
        return c

    def fits(self, job: Job) -> bool:
        R, C = job.RC
        A = len(ensure_diag(job.model).pi)
        need = job_device_bytes(R, C, A)
        if not self.free_slots:
            return False
        # long jobs may hold all but `short_slots` slots, so that short jobs
        # always find one free
        if self._cost(job) > self.short_ms and \
                sum(self._cost(j) > self.short_ms for j, *_ in self.inflight) >= self.max_inflight - self.short_slots:
            return False
        key = self._key(job)
        if any(self._key(j) == key for j, *_ in self.inflight):
            return False
        return self.used_bytes + need <= self.budget or not self.inflight

    def poll(self, now_fn):
        """Retire finished jobs; returns how many finished."""
        done = 0
        keep = []
        for job, slot, ev, nbytes, bufs in self.inflight:
            if ev.query():
                job.finish = now_fn()
                # numpy views of the pinned result buffers; Job.release()
                # hands the buffers back to the host allocator's cache
                job.result = {k: v.numpy() for k, v in bufs[3].items()}
                job._pinned = bufs[4]
                job._give_back = self._give_back
                # the plan stays cached; its workspace goes back to the pool.
                # A bounded device wait that gave up marks the job failed.
                plan = self.plans.get(self._key(job))
                if plan is not None:
                    try:
                        plan.status()
                    except Exception as exc:  # noqa: BLE001
                        job.error = str(exc)
                    plan.trim()
                self.free_slots.append(slot)
                self.used_bytes -= nbytes
                self.completed.append(job)
                done += 1
                if self.on_done is not None:
                    self.on_done(job)
            else:
                keep.append((job, slot, ev, nbytes, bufs))
        self.inflight = keep
        return done

    # ------------------------------------------------------------------- run
    def run(self, jobs, realtime: bool = True, on_admit=None, on_done=None):
        """Serve ``jobs`` (sorted by ``arrival``).  With ``realtime`` the loop
        admits a job only once the wall clock reaches its arrival time;
        otherwise all jobs are available at t=0.  ``on_done(job)`` runs as
        each job's results land in host memory.  Returns the completed jobs."""
        self.on_done = on_done
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        pending = collections.deque(sorted(jobs, key=lambda j: j.arrival))
        waiting = []
        while pending or waiting or self.inflight:
            t = now()
            while pending and (not realtime or pending[0].arrival <= t):
                j = pending.popleft()
                if not realtime:
                    j.arrival = t
                waiting.append(j)
            while waiting and self.free_slots:
                # shortest estimated job first, aged by its wait so that long
                # jobs are not starved; the first one that fits is admitted
                tn = now()
                order = sorted(waiting, key=lambda w: self._cost(w) - self.aging * 1e3 * (tn - w.arrival))
                j = next((w for w in order if self.fits(w)), None)
                if j is None:
                    break
                waiting.remove(j)
                t1 = time.perf_counter()
                self._launch(j, now())
                self.host_s["launch"] += time.perf_counter() - t1
                if on_admit:
                    on_admit(j)
            t1 = time.perf_counter()
            ndone = self.poll(now)
            self.host_s["poll"] += time.perf_counter() - t1
            if ndone == 0:
                if self.inflight:
                    time.sleep(0.0002)
                elif pending and realtime:
                    time.sleep(max(0.0, min(0.002, pending[0].arrival - now())))
        return self.completed

    def close(self):
        for p in self.plans.values():
            p.close()
        self.plans.clear()


def latency_stats(jobs):
    lat = np.array([j.latency for j in jobs]) * 1000.0
    wait = np.array([j.start - j.arrival for j in jobs]) * 1000.0
    serv = np.array([j.finish - j.start for j in jobs]) * 1000.0
    cols = sum(j.RC[1] for j in jobs)
    span = max(j.finish for j in jobs) - min(j.arrival for j in jobs)
    return {"jobs": len(jobs), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "queue_p50_ms": float(np.percentile(wait, 50)), "queue_p99_ms": float(np.percentile(wait, 99)),
            "service_p50_ms": float(np.percentile(serv, 50)), "service_p99_ms": float(np.percentile(serv, 99)),
            "max_ms": float(lat.max()), "columns": int(cols), "columns_per_s": cols / span, "span_s": span}


class NativeServer:
    """The library's serving engine (subby_server_*): continuous batching run
    by a C++ engine thread, so the Python side only submits descriptors and
    collects results.  Short A = 4 jobs that wait together run as one launch
    of the persistent packed kernel over their (job, column-tile) queue.

    ``submit(job)`` takes a ``Job`` with a reversible model whose alignment
    is ``HostRows`` (rows of a pinned host buffer) or a pinned / device int32
    torch tensor (R, C); ``collect(timeout_ms)`` returns the jobs completed
    since the last call, with ``start`` / ``finish`` on the arrival clock and
    ``result`` numpy views of pinned blocks that ``Job.release()`` hands back
    to the engine.
    """

    def __init__(self, max_inflight: int = 8, device_budget: int = 64 << 30, pinned_prewarm: int = 0,
                 autotune_cache: str = None, **settings):
        """``settings``: scheduling parameters of subby_server_set (short_ms,
        slice_ms, wave_cols, aging, short_slots, plan_cache, pack,
        pack_max_jobs, pack_tiles_*).  ``autotune_cache``: a file written by
        ``autotune_packed`` whose work-item shapes apply unless ``settings``
        gives them."""
        if autotune_cache is not None:
            settings = {**load_autotune(autotune_cache), **settings}
        self._lib = _lib.load()
        h = ct.c_void_p()
        _lib.check(self._lib.subby_server_create(max_inflight, device_budget, pinned_prewarm, ct.byref(h)),
                   "subby_server_create")
        self._h = h
        for k, v in settings.items():
            _lib.check(self._lib.subby_server_set(h, k.encode(), float(v)), f"subby_server_set({k})")
        self._jobs = {}
        self._next = 0
        self._res = (_lib.JobResult * 256)()
        self.t0 = 0.0   # server-clock time of arrival 0

    def clock(self) -> float:
        return float(self._lib.subby_server_clock(self._h))

    def start_clock(self):
        """Arrival times of submitted jobs count from now."""
        self.t0 = self.clock()

    def submit(self, job: Job, arrival: float = None):
        m = ensure_diag(job.model)
        if np.iscomplexobj(np.asarray(m.eigenvalues)) or hasattr(m, "eigenvectors_inv"):
            raise ValueError("NativeServer takes reversible models; irreversible jobs run on Server")
        par = np.ascontiguousarray(job.tree.parentIndex, dtype=np.int32)
        dist = np.ascontiguousarray(job.tree.distanceToParent, dtype=np.float64)
        ev, V, pi = (np.ascontiguousarray(np.asarray(x), dtype=np.float64) for x in (m.eigenvalues, m.eigenvectors, m.pi))
        a = job.alignment
        rowmap = None
        if isinstance(a, HostRows):
            R, C = a.R, a.C
            ptr = a.base.data_ptr() + 4 * int(a.col0)
            pitch = int(a.base.stride(0))
            if a.rowmap is not None:
                rm = a.rowmap
                rowmap = np.ascontiguousarray(rm.cpu().numpy() if hasattr(rm, "cpu") else rm, dtype=np.int32)
        else:
            import torch
            if not isinstance(a, torch.Tensor) or not (a.is_cuda or a.is_pinned()) or a.dtype != torch.int32 \
                    or a.dim() != 2 or a.stride(1) != 1:
                raise ValueError("NativeServer jobs take HostRows or a pinned / CUDA int32 (R, C) tensor")
            R, C = int(a.shape[0]), int(a.shape[1])
            ptr, pitch = a.data_ptr(), int(a.stride(0))
        want = sum(bit for k, bit in (("logLike", _lib.WANT_LOGLIKE), ("counts", _lib.WANT_COUNTS),
                                      ("rootProb", _lib.WANT_ROOTPROB)) if k in job.want)
        if isinstance(job.branch_mask, str):
            mask_mode = _lib.MASK_AUTO
        elif job.branch_mask is None:
            mask_mode = _lib.MASK_NONE
        else:
            raise ValueError("NativeServer: branch_mask must be 'auto' or None")
        tag = self._next
        self._next += 1
        d = _lib.Job(par.ctypes.data, dist.ctypes.data, len(par), ev.ctypes.data, V.ctypes.data, pi.ctypes.data,
                     len(pi), ptr, pitch, None if rowmap is None else rowmap.ctypes.data, C, want,
                     _lib.COUNTS_F81 if job.f81 else _lib.COUNTS_EIGEN, mask_mode,
                     -1.0 if arrival is None else self.t0 + float(arrival), tag)
        _lib.check(self._lib.subby_server_submit(self._h, ct.byref(d)), "subby_server_submit")
        job._A, job._C = len(pi), C
        self._jobs[tag] = job

    def collect(self, timeout_ms: int = 0):
        n = ct.c_int(0)
        _lib.check(self._lib.subby_server_wait(self._h, self._res, len(self._res), int(timeout_ms), ct.byref(n)),
                   "subby_server_wait")
        out = []
        for i in range(n.value):
            r = self._res[i]
            job = self._jobs.pop(r.tag)
            A, C = job._A, job._C
            job.start = r.t_start - self.t0
            job.finish = r.t_finish - self.t0
            if r.status != _lib.OK:
                job.error = f"{self._lib.subby_strerror(r.status).decode()} ({r.status})"
            res = {}
            for key, p, shape in (("logLike", r.logLike, (C,)), ("counts", r.counts, (A, A, C)),
                                  ("rootProb", r.rootProb, (A, C))):
                if p:
                    n_el = int(np.prod(shape))
                    res[key] = np.ctypeslib.as_array((ct.c_float * n_el).from_address(p)).reshape(shape)
            job.result = res
            handle = int(r.handle)
            job._give_back = lambda blocks, h=handle: self._lib.subby_server_release(self._h, h)
            job._pinned = [handle]
            out.append(job)
        return out

    def stats(self):
        b, p, i, w = ct.c_double(), ct.c_int(), ct.c_int(), ct.c_int()
        pj, pl = ct.c_longlong(), ct.c_longlong()
        self._lib.subby_server_stats(self._h, ct.byref(b), ct.byref(p), ct.byref(i), ct.byref(w), ct.byref(pj),
                                     ct.byref(pl))
        return {"engine_busy_s": b.value, "plans_cached": p.value, "inflight": i.value, "waiting": w.value,
                "packed_jobs": pj.value, "packed_launches": pl.value}

    def run(self, jobs, realtime: bool = True, on_done=None):
        """Submit ``jobs`` at their arrival times (all at once when not
        realtime), collect them as they complete; returns the completed jobs."""
        pending = collections.deque(sorted(jobs, key=lambda j: j.arrival))
        self.start_clock()
        t0 = time.perf_counter()
        done, outstanding = [], 0
        while pending or outstanding:
            now = time.perf_counter() - t0
            while pending and (not realtime or pending[0].arrival <= now):
                j = pending.popleft()
                self.submit(j, arrival=j.arrival if realtime else None)
                if not realtime:
                    j.arrival = self.clock() - self.t0
                outstanding += 1
            wait_ms = 0 if pending and realtime and pending[0].arrival - now < 0.002 else 1
            for j in self.collect(timeout_ms=wait_ms):
                outstanding -= 1
                done.append(j)
                if on_done is not None:
                    on_done(j)
        return done

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.subby_server_destroy(self._h)
            self._h = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


# ---------------------------------------------------------------------------
# autotuner of the packed kernel's work-item shape
# ---------------------------------------------------------------------------

PACK_TILE_KEYS = (("pack_tiles_r64", 24), ("pack_tiles_r256", 96), ("pack_tiles_big", 300))


def default_autotune_cache() -> str:
    import os
    return os.environ.get("SUBBY_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "subby_gb300", "autotune.json"))


def autotune_packed(cache: str = None, candidates=(1, 2, 4, 8), n_jobs: int = 48, trials: int = 3,
                    seed: int = 0) -> dict:
    """Choose the packed A = 4 kernel's work-item shape — how many 256-column
    tiles one claimed item spans — for small, medium and large trees, by
    timing each candidate on the device, and write the choice to ``cache``
    (JSON; default ``$SUBBY_AUTOTUNE_CACHE`` or ~/.cache/subby_gb300/
    autotune.json).  Larger items amortise the per-item claim and table
    reload; smaller ones balance the CTAs better.  Per bucket: ``n_jobs``
    HKY85 jobs on random trees of about the bucket's size, C log-uniform in
    100..20000, uniform tokens with 5% gaps, submitted together so they run
    as packed batches; the median wall time over ``trials`` runs of one
    engine per candidate decides.  Returns the settings dict."""
    import json
    import os
    import torch
    from . import synth, models
    rng = np.random.default_rng(seed)
    out, measured = {}, {}
    for key, leaves in PACK_TILE_KEYS:
        jobs = []
        for i in range(n_jobs):
            tree = synth.random_tree(int(leaves * rng.uniform(0.7, 1.3)), 0.1, rng)
            model = models.hky85_diag(2.0, rng.dirichlet(np.ones(4)))
            C = int(np.exp(rng.uniform(np.log(100), np.log(20000))))
            tok = rng.integers(0, 80, size=(len(tree.parentIndex), C))
            aln = torch.from_numpy(np.where(tok < 76, tok % 4, 5).astype(np.int32)).pin_memory()
            jobs.append((tree, model, aln))
        times = {}
        for k in candidates:
            srv = NativeServer(max_inflight=2, device_budget=16 << 30, **{key: k})
            ts = []
            for t in range(trials + 1):
                batch = [Job(id=i, alignment=a, tree=tr, model=m, want=("counts",)) for i, (tr, m, a) in
                         enumerate(jobs)]
                t0 = time.perf_counter()
                done = srv.run(batch, realtime=False, on_done=lambda j: j.release())
                dt = time.perf_counter() - t0
                if any(j.error for j in done):
                    raise RuntimeError("autotune run failed: " + next(j.error for j in done if j.error))
                if t > 0:          # the first run builds the plans
                    ts.append(dt)
            srv.close()
            times[k] = float(np.median(ts))
        out[key] = int(min(times, key=times.get))
        measured[key] = {str(k): round(v * 1e3, 3) for k, v in times.items()}
    cache = cache or default_autotune_cache()
    os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
    with open(cache, "w") as f:
        json.dump({"settings": out, "wall_ms": measured, "device": torch.cuda.get_device_name()}, f, indent=1)
    return out


def load_autotune(cache: str = None) -> dict:
    """Settings of a previous autotune_packed run ({} when there is none)."""
    import json
    import os
    cache = cache or default_autotune_cache()
    if not os.path.exists(cache):
        return {}
    with open(cache) as f:
        return dict(json.load(f).get("settings", {}))
