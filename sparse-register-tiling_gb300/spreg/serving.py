"""Continuous-batching serving loop over resident packed sparse-MLP weights.

A request is a token batch x (d_model x n, one column per token) pushed through a stack of pruned
MLP blocks

    h = relu(W_up x)          W_up   d_ff x d_model   (executor epilogue ReLU)
    x = x + W_down h          W_down d_model x d_ff    (executor load_c: the residual add)

The packed weights stay resident on the device.  `Server`:

* admits queued requests first come, first served, while a slot is free and the request's
  activation buffers (x and h, one block) fit in a fixed device arena -- the activation-memory
  budget.  Nothing is allocated on the device while serving;
* advances every admitted request by one layer per iteration, and puts all of an iteration's SpMMs
  -- whatever their layer or token count -- into one ``spreg_execute_batched`` work list (the
  executor groups them by kernel configuration, so requests at the same layer share one launch
  and read the same packed weight out of L2);
* keeps up to ``max_inflight`` iterations queued on its compute stream and moves inputs in and
  outputs out on a copy stream, so requests that arrive while others run join the next iteration
  and their copies overlap the kernels.

`serve_per_request` is the plain path the server is measured against: each request alone, in
arrival order, one ``spreg_execute`` launch per layer, FP32 storage.

`Scheduler` and `ActivationArena` hold the host-side policy and need no GPU.
"""
from __future__ import annotations

import collections
import ctypes as C
import dataclasses
import time
from typing import Callable, Deque, List, Optional, Sequence

import numpy as np

from . import _lib
from .mapping import Mapping

ARENA_ALIGN = 256
LD_ALIGN = 8  # leading dimension of activations, in elements (16-byte rows for BF16 vector loads)

# numpy view of spreg_work_item (include/spreg.h): packed matrix handle + spreg_exec_args
WORK_ITEM_DTYPE = np.dtype([
    ("a", np.uint64), ("b", np.uint64), ("ldb", np.int64), ("c", np.uint64), ("ldc", np.int64), ("n", np.int64),
    ("b_dtype", np.int32), ("c_dtype", np.int32), ("load_c", np.int32), ("epilogue", np.int32), ("nr", np.int32),
    ("warps_per_cta", np.int32), ("b_staging", np.int32), ("meta_staging", np.int32), ("job_order", np.int32),
    ("panel_rounds", np.int32), ("load_balance", np.int32), ("reserved", np.int32)])
assert WORK_ITEM_DTYPE.itemsize == C.sizeof(_lib.WorkItem)

# numpy view of spreg_dense_rows_item (include/spreg.h): one tensor-core product
TC_ITEM_DTYPE = np.dtype([
    ("a_rows", np.uint64), ("rows", np.int64), ("k", np.int64), ("lda", np.int64), ("row_index", np.uint64),
    ("b", np.uint64), ("ldb", np.int64), ("c", np.uint64), ("ldc", np.int64), ("n", np.int64),
    ("c_dtype", np.int32), ("load_c", np.int32), ("epilogue", np.int32), ("tile_n", np.int32)])
assert TC_ITEM_DTYPE.itemsize == 96


def _handle_int(h) -> int:
    return int(h.value if hasattr(h, "value") else h)


def round_up(x: int, a: int) -> int:
    return (x + a - 1) // a * a


def nr_for_tokens(n: int) -> int:
    """Strip width for a token count: 32 columns per lane-vector element, at most 4 per lane."""
    return 128 if n >= 128 else (64 if n >= 64 else 32)


# ---------------------------------------------------------------------------- host-side policy
class ActivationArena:
    """First-fit allocator of aligned byte ranges in [0, capacity); frees coalesce with neighbours."""

    def __init__(self, capacity: int, align: int = ARENA_ALIGN):
        self.capacity = int(capacity) // align * align
        self.align = align
        self.free_list: List[List[int]] = [[0, self.capacity]] if self.capacity else []  # sorted [off, size]
        self.live = {}
        self.used = 0
        self.peak = 0

    def alloc(self, nbytes: int) -> Optional[int]:
        size = round_up(max(int(nbytes), 1), self.align)
        for i, (off, sz) in enumerate(self.free_list):
            if sz >= size:
                if sz == size:
                    self.free_list.pop(i)
                else:
                    self.free_list[i] = [off + size, sz - size]
                self.live[off] = size
                self.used += size
                self.peak = max(self.peak, self.used)
                return off
        return None

    def free(self, off: int) -> None:
        size = self.live.pop(off)
        self.used -= size
        fl = self.free_list
        i = 0
        while i < len(fl) and fl[i][0] < off:
            i += 1
        fl.insert(i, [off, size])
        if i + 1 < len(fl) and fl[i][0] + fl[i][1] == fl[i + 1][0]:  # merge with the next range
            fl[i][1] += fl.pop(i + 1)[1]
        if i > 0 and fl[i - 1][0] + fl[i - 1][1] == fl[i][0]:  # merge with the previous range
            fl[i - 1][1] += fl.pop(i)[1]

    def largest_free(self) -> int:
        return max((sz for _, sz in self.free_list), default=0)


@dataclasses.dataclass(eq=False)
class Request:
    """One request: ``n`` tokens of input ``x`` (d_model x n, host) arriving at ``arrival``.

    ``arrival`` is seconds after the start of a real-time run, or the iteration before which the
    request is submitted in a lock-step run.  The server fills in the other fields.
    """
    rid: int
    n: int
    x: object = None            # host input (numpy float32 d_model x n, or a prepared pinned tensor)
    arrival: float = 0.0
    out: object = None          # host output (d_model x n view)
    layer: int = 0              # next layer to run
    offset: int = -1            # arena offset of its activation block
    t_admit: float = float("nan")
    t_done: float = float("nan")
    first_iteration: int = -1
    # device-side state kept by the server
    _host_in: object = None
    _host_out: object = None
    _slot: int = -1
    _ready: object = None

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


class Scheduler:
    """Admission and per-iteration planning of a continuous batch (host logic only).

    ``bytes_of(request)`` is the activation memory a request holds from admission until its
    output has left the device; ``num_layers`` layers run one per iteration.
    """

    def __init__(self, num_layers: int, bytes_of: Callable[[Request], int], arena: ActivationArena,
                 max_slots: int):
        if max_slots < 1:
            raise ValueError("max_slots must be >= 1")
        self.num_layers = num_layers
        self.bytes_of = bytes_of
        self.arena = arena
        self.max_slots = max_slots
        self.queue: Deque[Request] = collections.deque()
        self.active: List[Request] = []      # admitted, layers left
        self.draining: List[Request] = []    # all layers queued, output not yet on the host

    def submit(self, req: Request) -> None:
        if self.bytes_of(req) > self.arena.capacity:
            raise ValueError(f"request {req.rid} needs {self.bytes_of(req)} bytes of activations; "
                             f"the budget is {self.arena.capacity}")
        self.queue.append(req)

    def slots_in_use(self) -> int:
        return len(self.active) + len(self.draining)

    def admit(self) -> List[Request]:
        """Admit from the head of the queue while a slot is free and the activations fit."""
        out = []
        while self.queue and self.slots_in_use() < self.max_slots:
            req = self.queue[0]
            off = self.arena.alloc(self.bytes_of(req))
            if off is None:
                break  # first come, first served: a later, smaller request does not overtake
            self.queue.popleft()
            req.offset = off
            req.layer = 0
            self.active.append(req)
            out.append(req)
        return out

    def next_iteration(self) -> List[Request]:
        """Requests advancing one layer now (each runs layer ``req.layer`` before the call returns
        it advanced); requests whose last layer is in this iteration move to ``draining``."""
        batch = list(self.active)
        for r in batch:
            r.layer += 1
        self.active = [r for r in batch if r.layer < self.num_layers]
        self.draining.extend(r for r in batch if r.layer >= self.num_layers)
        return batch

    def release(self, req: Request) -> None:
        self.draining.remove(req)
        self.arena.free(req.offset)
        req.offset = -1

    def idle(self) -> bool:
        return not (self.queue or self.active or self.draining)


# ---------------------------------------------------------------------------- model
def mlp_weights(d_model: int, d_ff: int, blocks: int, sparsity: float, seed: int = 0, std: float = 0.02,
                sigma: float = 0.5, bf16_values: bool = True):
    """[(W_up d_ff x d_model, W_down d_model x d_ff), ...] with magnitude-pruning-like row skew;
    values N(0, std), rounded to BF16-representable FP32 when ``bf16_values``."""
    from . import synth
    out = []
    for b in range(blocks):
        wu = synth.row_skew(d_ff, d_model, sparsity, seed=seed + 2 * b, sigma=sigma, std=std)
        wd = synth.row_skew(d_model, d_ff, sparsity, seed=seed + 2 * b + 1, sigma=sigma, std=std)
        if bf16_values:
            wu, wd = synth.round_bf16(wu), synth.round_bf16(wd)
        out.append((wu, wd))
    return out


def mlp_reference_fp64(weights, x: np.ndarray) -> np.ndarray:
    """The stack in FP64 on the host (dense products of the pruned weights)."""
    x = np.asarray(x, dtype=np.float64)
    for wu, wd in weights:
        h = np.maximum(wu.astype(np.float64) @ x, 0.0)
        x = x + wd.astype(np.float64) @ h
    return x


class SparseMLP:
    """Packed, device-resident weights of a sparse MLP stack, stored as ``dtype`` ("bf16"/"f32");
    activations use the same type and accumulate in FP32.

    ``configs`` (one dict per layer, keys ``mr``, ``mapping``, ``k_tile``; see `tune_mlp`) packs each
    layer with its own panel height, nanokernel set and K tile; by default every layer uses
    ``mapping`` (M_r = 4 identity) untiled.

    ``tc=True`` (BF16 only) keeps every layer as dense BF16 rows for the tensor cores -- the hybrid
    split with a panel-fill threshold of 0, which `spreg.hybrid.tune_tc_fill` picks for these layer
    shapes from N = 128 up -- and runs them with ``spreg_dense_rows_bf16(_batched)``."""

    def __init__(self, weights, dtype: str = "bf16", mapping: Optional[Mapping] = None, device=None,
                 configs: Optional[Sequence[dict]] = None, tc: bool = False):
        import torch
        from .packed import PackedMatrix
        if dtype not in ("bf16", "f32"):
            raise ValueError("dtype must be 'bf16' or 'f32'")
        self.dtype = dtype
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.mapping = mapping if mapping is not None else Mapping.identity(4)
        self.act_code = _lib.BF16 if dtype == "bf16" else _lib.F32
        self.act_torch = torch.bfloat16 if dtype == "bf16" else torch.float32
        self.elem = 2 if dtype == "bf16" else 4
        self.d_ff, self.d_model = weights[0][0].shape
        if configs is not None and len(configs) != 2 * len(weights):
            raise ValueError(f"configs needs one entry per layer ({2 * len(weights)}), got {len(configs)}")
        self.configs = list(configs) if configs is not None else None
        self.tc = bool(tc)
        if self.tc and dtype != "bf16":
            raise ValueError("tensor-core layers take BF16 operands")
        self.layers = []
        self.tc_rows = []   # per layer: (dense BF16 rows M x K8, row index 0 .. M - 1)
        for b, (wu, wd) in enumerate(weights):
            if wu.shape != (self.d_ff, self.d_model) or wd.shape != (self.d_model, self.d_ff):
                raise ValueError("every block needs W_up d_ff x d_model and W_down d_model x d_ff")
            for j, w in enumerate((wu, wd)):
                t = torch.from_numpy(np.ascontiguousarray(w, dtype=np.float32)).to(self.device)
                if self.tc:
                    M, K = w.shape
                    a = torch.zeros((M, round_up(K, 8)), dtype=torch.bfloat16, device=self.device)
                    a[:, :K] = t.to(torch.bfloat16)
                    self.tc_rows.append((a, torch.arange(M, dtype=torch.int32, device=self.device)))
                    del t
                    continue
                mp, kt = self.mapping, 0
                if self.configs is not None:
                    from .autotune import mapping_of
                    cfg = self.configs[2 * b + j]
                    mp, kt = mapping_of(int(cfg["mr"]), cfg["mapping"]), int(cfg.get("k_tile", 0))
                self.layers.append(PackedMatrix.from_dense(t, mp, k_tile=kt, value_dtype=self.act_code))
                del t
        self.blocks = len(weights)

    @property
    def num_layers(self) -> int:
        return 2 * self.blocks

    def ld(self, n: int) -> int:
        return round_up(max(int(n), 1), LD_ALIGN)

    def x_bytes(self, n: int) -> int:
        return round_up(self.d_model * self.ld(n) * self.elem, ARENA_ALIGN)

    def act_bytes(self, n: int) -> int:
        """Activation block of one request: x (d_model x ld) then h (d_ff x ld)."""
        return self.x_bytes(n) + round_up(self.d_ff * self.ld(n) * self.elem, ARENA_ALIGN)

    def _item_template(self) -> np.ndarray:
        """The per-layer fields that do not depend on the request (built once)."""
        if getattr(self, "_template", None) is not None:
            return self._template
        up = np.arange(self.num_layers) % 2 == 0
        if self.tc:
            it = np.zeros(self.num_layers, dtype=TC_ITEM_DTYPE)
            it["a_rows"] = [a.data_ptr() for a, _ in self.tc_rows]
            it["rows"] = [a.shape[0] for a, _ in self.tc_rows]
            it["k"] = np.where(up, self.d_model, self.d_ff)
            it["lda"] = [a.stride(0) for a, _ in self.tc_rows]
            it["row_index"] = [idx.data_ptr() for _, idx in self.tc_rows]
            it["c_dtype"] = _lib.BF16
        else:
            it = np.zeros(self.num_layers, dtype=WORK_ITEM_DTYPE)
            it["a"] = [_handle_int(pm.handle) for pm in self.layers]
            it["b_dtype"] = it["c_dtype"] = self.act_code
            if self.configs is not None:
                it["warps_per_cta"] = [int(c.get("warps", 0)) for c in self.configs]
        it["load_c"] = np.where(up, 0, 1)
        it["epilogue"] = np.where(up, _lib.EPILOGUE_RELU, _lib.EPILOGUE_NONE)
        self._template = it
        return it

    def work_items(self, x_ptr: int, h_ptr: int, n: int) -> np.ndarray:
        """The request's SpMMs, one per layer, as spreg_work_item records (spreg_dense_rows_item
        records for tensor-core layers): layer 2b reads x and writes h, layer 2b + 1 the reverse."""
        it = self._item_template().copy()
        ld = self.ld(n)
        it["b"][0::2], it["c"][0::2] = x_ptr, h_ptr
        it["b"][1::2], it["c"][1::2] = h_ptr, x_ptr
        it["ldb"] = ld
        it["ldc"] = ld
        it["n"] = n
        if not self.tc:
            it["nr"] = nr_for_tokens(n)
        return it

    def forward(self, x_dev, h_dev, n: Optional[int] = None, stream=None):
        """One request through the stack in place on x_dev (d_model x n), h_dev (d_ff x n) as
        scratch: two spreg_execute launches per block."""
        if self.tc:
            from .hybrid import dense_rows_bf16
            for b in range(self.blocks):
                (au, iu), (ad, idd) = self.tc_rows[2 * b], self.tc_rows[2 * b + 1]
                dense_rows_bf16(au, iu, x_dev, h_dev, n=n, epilogue=_lib.EPILOGUE_RELU, stream=stream,
                                check_rows=False)
                dense_rows_bf16(ad, idd, h_dev, x_dev, n=n, load_c=True, stream=stream, check_rows=False)
            return x_dev
        for b in range(self.blocks):
            up, down = self.layers[2 * b], self.layers[2 * b + 1]
            up.execute(x_dev, h_dev, n=n, epilogue=_lib.EPILOGUE_RELU, stream=stream)
            down.execute(h_dev, x_dev, n=n, load_c=True, stream=stream)
        return x_dev


def tune_mlp(weights, dtype: str = "bf16", n: int = 96, batch: int = 32, top: int = 6, device=None):
    """Per-layer packings for `SparseMLP` from the autotuner: block 0's up and down projections are
    tuned for ``batch`` concurrent requests of ``n`` tokens and every block reuses them (all blocks
    share shapes and sparsity).  Returns (configs, tune results)."""
    from .autotune import tune
    # register-tiled packings (tensor-core layers are SparseMLP(tc=True)); the CTA tiling is kept; no
    # panel rounds (the strip width follows each request's token count)
    res = [tune(w, n, dtype, top=top, batch=batch, device=device, tc=False, rounds=False) for w in weights[0]]
    cfg = [{"mr": r.best.mr, "mapping": r.best.mapping, "k_tile": r.best.k_tile, "nr": r.best.nr,
            "warps": r.best.warps} for r in res]
    return [dict(cfg[l % 2]) for l in range(2 * len(weights))], res


# ---------------------------------------------------------------------------- serving
@dataclasses.dataclass
class ServeStats:
    requests: int
    seconds: float
    req_per_s: float
    tokens_per_s: float
    p50_ms: float
    p99_ms: float
    mean_ms: float
    iterations: int = 0
    max_batch: int = 0
    peak_activation_bytes: int = 0

    def as_dict(self) -> dict:
        return dataclasses.asdict(self)


def summarize(reqs: Sequence[Request], seconds: float, **extra) -> ServeStats:
    lat = np.array([r.latency for r in reqs]) * 1e3
    toks = sum(r.n for r in reqs)
    return ServeStats(requests=len(reqs), seconds=seconds, req_per_s=len(reqs) / seconds if seconds > 0 else 0.0,
                      tokens_per_s=toks / seconds if seconds > 0 else 0.0,
                      p50_ms=float(np.percentile(lat, 50)) if len(lat) else float("nan"),
                      p99_ms=float(np.percentile(lat, 99)) if len(lat) else float("nan"),
                      mean_ms=float(lat.mean()) if len(lat) else float("nan"), **extra)


def prepare_requests(model: SparseMLP, reqs: Sequence[Request]) -> None:
    """Pinned host input/output buffers in the model's activation type (the client's buffers)."""
    import torch
    for r in reqs:
        ld = model.ld(r.n)
        hin = torch.zeros((model.d_model, ld), dtype=model.act_torch).pin_memory()
        hin[:, : r.n] = torch.from_numpy(np.ascontiguousarray(r.x, dtype=np.float32)).to(model.act_torch)
        r._host_in = hin
        r._host_out = torch.empty((model.d_model, ld), dtype=model.act_torch).pin_memory()
        r.out = r._host_out[:, : r.n]


class Server:
    """Continuous-batching executor of a `SparseMLP` (see the module docstring)."""

    def __init__(self, model: SparseMLP, budget_bytes: int = 512 << 20, max_slots: int = 128,
                 max_inflight: int = 2):
        import torch
        self.model = model
        self.max_slots = int(max_slots)
        self.max_inflight = max(1, int(max_inflight))
        self.arena_t = torch.empty(int(budget_bytes), dtype=torch.uint8, device=model.device)
        self.base = self.arena_t.data_ptr()
        self.compute = torch.cuda.Stream(model.device)
        self.copy = torch.cuda.Stream(model.device)
        self._dtype = TC_ITEM_DTYPE if model.tc else WORK_ITEM_DTYPE
        # every admitted request's records at a fixed slot: rows slot * L .. slot * L + L - 1
        self._table = np.zeros(max(self.max_slots, 1) * model.num_layers, dtype=self._dtype)
        self._lib = _lib.lib()

    def _x_view(self, r: Request):
        m = self.model
        nb = m.d_model * m.ld(r.n) * m.elem
        return self.arena_t[r.offset: r.offset + nb].view(m.act_torch).view(m.d_model, m.ld(r.n))

    def run(self, reqs: Sequence[Request], realtime: bool = True,
            clock: Callable[[], float] = time.perf_counter) -> ServeStats:
        """Serve ``reqs`` (prepared with `prepare_requests`); returns latency/throughput stats.

        realtime: arrivals are seconds after the start; otherwise arrivals are iteration indices
        (a request is submitted before that iteration), which makes the mix reproducible."""
        import torch
        m = self.model
        arena = ActivationArena(self.arena_t.numel())
        sched = Scheduler(m.num_layers, lambda r: m.act_bytes(r.n), arena, self.max_slots)
        order = sorted(reqs, key=lambda r: (r.arrival, r.rid))
        inflight: Deque = collections.deque()
        free_slots = list(range(self.max_slots - 1, -1, -1))
        L = m.num_layers
        draining: List = []
        nxt, done, it, launches, max_batch = 0, 0, 0, 0, 0
        first_arrival = order[0].arrival if order else 0.0
        t0 = clock()
        while done < len(order):
            now = clock() - t0 if realtime else float(it)
            while nxt < len(order) and order[nxt].arrival <= now:
                sched.submit(order[nxt])
                nxt += 1
            # outputs that reached the host free their slot and memory
            still = []
            for ev, r in draining:
                if ev.query():
                    r.t_done = clock() - t0 if realtime else float(it)
                    sched.release(r)
                    free_slots.append(r._slot)
                    done += 1
                else:
                    still.append((ev, r))
            draining = still
            for r in sched.admit():
                r.t_admit = clock() - t0 if realtime else float(it)
                r.first_iteration = it
                x_ptr = self.base + r.offset
                r._slot = free_slots.pop()
                self._table[r._slot * L:(r._slot + 1) * L] = m.work_items(x_ptr, x_ptr + m.x_bytes(r.n), r.n)
                with torch.cuda.stream(self.copy):
                    self._x_view(r).copy_(r._host_in, non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(self.copy)
                r._ready = ev
            if sched.active:
                batch = sched.next_iteration()
                rows = np.empty(len(batch), dtype=np.int64)
                for i, r in enumerate(batch):
                    if r._ready is not None:
                        self.compute.wait_event(r._ready)
                        r._ready = None
                    rows[i] = r._slot * L + r.layer - 1
                buf = self._table[rows]  # one gather of this iteration's records
                run = self._lib.spreg_dense_rows_bf16_batched if m.tc else self._lib.spreg_execute_batched
                _lib.check(run(buf.ctypes.data, len(batch), self.compute.cuda_stream))
                ev = torch.cuda.Event()
                ev.record(self.compute)
                inflight.append(ev)
                launches += 1
                max_batch = max(max_batch, len(batch))
                it += 1
                for r in batch:
                    if r.layer >= m.num_layers:
                        with torch.cuda.stream(self.copy):
                            self.copy.wait_event(ev)
                            r._host_out.copy_(self._x_view(r), non_blocking=True)
                            eo = torch.cuda.Event()
                            eo.record(self.copy)
                        draining.append((eo, r))
                while len(inflight) > self.max_inflight:
                    inflight.popleft().synchronize()
            elif draining:
                draining[0][0].synchronize()
            elif nxt < len(order):
                if realtime:
                    wait = order[nxt].arrival - (clock() - t0)
                    if wait > 2e-4:
                        time.sleep(wait - 1e-4)
                else:
                    it = max(it, int(np.ceil(order[nxt].arrival)))
        self.compute.synchronize()
        self.copy.synchronize()
        seconds = (max(r.t_done for r in order) - min(first_arrival, 0.0)) if order else 0.0
        st = summarize(order, seconds, iterations=it, max_batch=max_batch,
                       peak_activation_bytes=arena.peak)
        return st


def serve_per_request(model: SparseMLP, reqs: Sequence[Request], realtime: bool = True,
                      clock: Callable[[], float] = time.perf_counter) -> ServeStats:
    """The plain path: each request alone, in arrival order -- input to the device, one
    ``spreg_execute`` per layer, output back -- before the next starts."""
    import torch
    m = model
    order = sorted(reqs, key=lambda r: (r.arrival, r.rid))
    stream = torch.cuda.current_stream(m.device)
    t0 = clock()
    for r in order:
        if realtime:
            wait = r.arrival - (clock() - t0)
            if wait > 2e-4:
                time.sleep(wait - 1e-4)
            while clock() - t0 < r.arrival:
                pass
        r.t_admit = clock() - t0
        ld = m.ld(r.n)
        x = torch.empty((m.d_model, ld), dtype=m.act_torch, device=m.device)
        h = torch.empty((m.d_ff, ld), dtype=m.act_torch, device=m.device)
        x.copy_(r._host_in, non_blocking=True)
        m.forward(x, h, n=r.n, stream=stream)
        r._host_out.copy_(x, non_blocking=True)
        stream.synchronize()
        r.t_done = clock() - t0
    seconds = max(r.t_done for r in order) - min(0.0, order[0].arrival) if order else 0.0
    return summarize(order, seconds, iterations=len(order) * m.num_layers, max_batch=1)


def output_fp32(r: Request) -> np.ndarray:
    """The request's output as an FP32 array (d_model x n)."""
    import torch
    return r.out.to(torch.float32).numpy()
