"""Autotuner for the executor: panel height M_r, nanokernel mapping and strip width N_r per weight.

It reads the same matrix statistics as the reference's selection machinery:
* sparsity and the dense operand's column count (the empirical heuristic's buckets,
  tools/paper/heuristic.py:26-50, tools/experiment_runner.py:86-113);
* the panel pattern histogram (sbench/SOP/distribution.py:18-31);
* per-panel nanokernel groups, entries and values, as the cost model counts them
  (sbench/ilp_pad/nano_solver.py:77-115, sbench/SOP/sop_cost_model.py:107-128).

Cost model (the reference's form, re-fitted for this executor on the GPU):
    t = L0 + strips(n) * (uBase * P + nCheck * G + nBase * U + nCnz * NV * V) / SMs + cCrit * U_max
with P row panels, G (panel, nanokernel id) groups with a nonzero count, U packed entries (column
indices) and V packed values, for one strip of 32 * NV columns; U_max, the entries of the heaviest
panel, stands for the critical path of one warp when there are too few items to spread over the
GPU.  One coefficient set per (M_r, NV, value/B type); `fit_costs` solves non-negative least
squares over measured samples.

For M_r = 8, and for K-tiled M_r = 4 packs, the candidates also include a nanokernel set built for
the matrix from its pattern histogram (`kernel_sets.greedy_kernel_set`, the reference's set-cover
model in greedy form; for K-tiled M_r = 4 with the B-tile executor's penalty for patterns without a
loop of their own).

Beyond the reference's M_r / N_r / mapping, a candidate carries the CTA tiling (`warps`: warps per
CTA of the batched kernel, row panels per job of the B-tile kernel), panel rounds (`rounds`: the
B-tile kernel keeps a job's strip of B resident for that many rounds of panels) and a tensor-core
threshold (`tc_fill`: panels whose fill reaches it run as dense tcgen05 products, `spreg.hybrid`).

`tune` ranks every candidate with the model, times the best few on the device with the reference's
timing protocol (`execute_timed`: median of repeated runs) or as a batch, then times the CTA tiling,
the gather kernel's wide strips, the panel rounds of the best and the tensor-core thresholds
(all panels; the densest tenth), and returns the fastest, so a poor model costs tuning time, not
speed.
"""
from __future__ import annotations

import dataclasses
import json
import math
import os
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np

from .mapping import Mapping

TUNING_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning")
DEFAULT_COSTS = os.path.join(TUNING_DIR, "gb300_costs.json")
SMS = 152

# nanokernel sets tried per panel height (NAMED_MAPPINGS ids, or "identity")
MAPPINGS_FOR_MR = {2: ("identity",), 4: ("identity",), 8: ("identity", "400fa", "747f9")}


@dataclasses.dataclass(frozen=True)
class Candidate:
    mr: int
    mapping: str     # "identity" or a mapping id
    nr: int          # strip width: 32, 64, 128, or wide: 256 (16-bit B at M_r <= 4, FP32 untiled packs)
                     # and 512 (untiled packs, M_r <= 4) columns
    k_tile: int = 0  # K_c of the packing (0: one K tile)
    warps: int = 0   # CTA tiling (spreg_exec_args.warps_per_cta; 0: the executor's choice)
    tc_fill: float = 2.0  # panels with fill >= tc_fill on the tensor cores (> 1: none)
    rounds: int = 0  # panel rounds of the B-tile kernel (spreg_exec_args.panel_rounds; 0: none)

    @property
    def nv(self) -> int:
        return self.nr // 32

    def name(self) -> str:
        """The reference's method grammar, M{Mr}N{nr}_{mapping} (tools/paper/configs.py:54-68), with
        the K tile appended as _K{K_c} when the packing is K-tiled."""
        return (f"M{self.mr}N{self.nr}_{self.mapping}" + (f"_K{self.k_tile}" if self.k_tile else "") +
                (f"_W{self.warps}" if self.warps else "") + (f"_R{self.rounds}" if self.rounds > 1 else "") +
                (f"_TC{self.tc_fill:g}" if self.tc_fill <= 1.0 else ""))


# Mappings built in this process (greedy sets from a matrix's histogram), by mapping id.
GENERATED: Dict[str, Mapping] = {}


def mapping_of(mr: int, name: str) -> Mapping:
    if name == "identity":
        return Mapping.identity(mr)
    if name in GENERATED:
        return GENERATED[name]
    return Mapping.load(name)


def greedy_mapping(mask: np.ndarray, mr: int, budget: int = 19, k_c: int = 128, tile: bool = False) -> Mapping:
    """Nanokernel set for this matrix from its pattern histogram (`kernel_sets`), registered under
    its mapping id so that `mapping_of` finds it.  `tile`: for the B-tile executor (K-tiled packs)."""
    from .kernel_sets import executor_penalty, greedy_kernel_set
    hist = np.bincount(panel_codes(mask, mr).ravel(), minlength=2 ** mr)
    units = ((mask.shape[0] + mr - 1) // mr) * max(1, math.ceil(mask.shape[1] / k_c))
    m = greedy_kernel_set(hist, mr, budget, units, penalty=executor_penalty(mr, tile=tile))
    GENERATED[m.mapping_id] = m
    return m


def candidate_from_name(name: str, A: Optional[np.ndarray] = None) -> Candidate:
    """The candidate a `Candidate.name()` string describes (M{mr}N{nr}_{mapping}[_K..][_W..][_R..]
    [_TC..]).  A mapping id built from a matrix's histogram is rebuilt from `A` (the greedy sets `rank`
    adds for M_r = 8 and for K-tiled M_r = 4), so that `mapping_of` finds it."""
    import re
    m = re.fullmatch(r"M(\d+)N(\d+)_([0-9a-z]+)((?:_[KWR]\d+|_TC[0-9.eE+-]+)*)", name)
    if not m:
        raise ValueError(f"not a candidate name: {name}")
    mr, nr, mapping, rest = int(m.group(1)), int(m.group(2)), m.group(3), m.group(4)
    kw = {}
    for tag, val in re.findall(r"_(K|W|R|TC)([0-9.eE+-]+)", rest):
        if tag == "K":
            kw["k_tile"] = int(val)
        elif tag == "W":
            kw["warps"] = int(val)
        elif tag == "R":
            kw["rounds"] = int(val)
        else:
            kw["tc_fill"] = float(val)
    if mapping != "identity" and mapping not in GENERATED and A is not None:
        mask = A != 0
        for gm in (greedy_mapping(mask, 8), greedy_mapping(mask, 4, budget=15, tile=True)):
            GENERATED.setdefault(gm.mapping_id, gm)
    return Candidate(mr, mapping, nr, **kw)


# ---------------------------------------------------------------------------- statistics
def panel_codes(mask: np.ndarray, mr: int) -> np.ndarray:
    """Pattern code of every (row panel, column): bit r set if row r of the panel is nonzero.
    The last panel is zero-padded to M_r rows."""
    m, k = mask.shape
    P = (m + mr - 1) // mr
    pad = np.zeros((P * mr, k), dtype=bool)
    pad[:m] = mask
    pad = pad.reshape(P, mr, k)
    codes = np.zeros((P, k), dtype=np.int32)
    for r in range(mr):
        codes |= pad[:, r, :].astype(np.int32) << r
    return codes


@dataclasses.dataclass
class PanelStats:
    """Counts the cost model reads, for one M_r and mapping."""
    mr: int
    mapping: str
    P: int          # row panels
    U: int          # packed entries (column indices)
    V: int          # packed values (nnz + padding)
    G: int          # (panel, nanokernel id) groups with a nonzero count
    nnz: int
    padding: int
    max_panel_U: int
    histogram: np.ndarray  # pattern code -> number of (panel, column) occurrences

    def features(self, nv: int) -> np.ndarray:
        return np.array([self.P, self.G, self.U, nv * self.V], dtype=np.float64)


def panel_stats(mask: np.ndarray, mr: int, mapping: Mapping) -> PanelStats:
    codes = panel_codes(mask, mr)
    P = codes.shape[0]
    hist = np.bincount(codes.ravel(), minlength=2 ** mr)
    ids = {p: i for i, p in enumerate(mapping.nanokernels)}
    ent = np.zeros(2 ** mr, dtype=np.int64)
    val = np.zeros(2 ** mr, dtype=np.int64)
    for c in range(1, 2 ** mr):
        ks = mapping(c)
        ent[c] = len(ks)
        val[c] = sum(bin(x).count("1") for x in ks)
    U = int((ent * hist).sum())
    V = int((val * hist).sum())
    nnz = int(mask.sum())
    per_panel_U = ent[codes].sum(axis=1)
    # distinct nanokernel ids per panel
    nk = max(len(ids), 1)
    seen = np.zeros((P, nk), dtype=bool)
    maxlen = max((len(mapping(c)) for c in range(1, 2 ** mr)), default=0)
    for j in range(maxlen):
        lut = np.full(2 ** mr, -1, dtype=np.int64)
        for c in range(1, 2 ** mr):
            ks = mapping(c)
            if j < len(ks) and ks[j] in ids:
                lut[c] = ids[ks[j]]
        idx = lut[codes]
        rows, cols = np.nonzero(idx >= 0)
        seen[rows, idx[rows, cols]] = True
    G = int(seen.sum())
    return PanelStats(mr=mr, mapping=_mapping_name(mapping), P=P, U=U, V=V, G=G,
                      nnz=nnz, padding=V - nnz, max_panel_U=int(per_panel_U.max()) if P else 0, histogram=hist)


def _mapping_name(m: Mapping) -> str:
    return "identity" if all(m.table.get(p, []) == [p] for p in range(1, 2 ** m.mr)) else m.mapping_id


def heuristic_bucket(sparsity: float, n: int) -> Tuple[str, int]:
    """The empirical heuristic's keys: sparsity bucket (0,.7], (.7,.8], (.8,.9], (.9,1] and the
    nearest bCols of {32, 128, 256, 512} (tools/paper/heuristic.py:26-50)."""
    edges = [(0.7, "(0,0.7]"), (0.8, "(0.7,0.8]"), (0.9, "(0.8,0.9]"), (1.01, "(0.9,1]")]
    bucket = next(name for e, name in edges if sparsity <= e)
    bcols = min((32, 128, 256, 512), key=lambda b: abs(math.log2(max(n, 1)) - math.log2(b)))
    return bucket, bcols


# ---------------------------------------------------------------------------- cost model
@dataclasses.dataclass
class Costs:
    """Per-(M_r, NV, dtype) coefficients (ns): L0, uBase, nCheck, nBase, nCnz, cCrit."""
    table: Dict[str, List[float]]

    @staticmethod
    def key(mr: int, nv: int, dtype: str) -> str:
        return f"mr{mr}_nv{nv}_{dtype}"

    @classmethod
    def default(cls) -> "Costs":
        """Prior before any calibration: one warp-step of 4 entries ~ 40 ns on one of 16 warps
        of an SM, an FMA block ~ 2 ns per value-vector; launch ~ 4 us."""
        t = {}
        for mr in (2, 4, 6, 8):
            for nv in (1, 2, 4):
                for dt in ("f32", "bf16"):
                    t[cls.key(mr, nv, dt)] = [4000.0, 20.0, 6.0, 2.5, 0.6, 40.0]
        return cls(t)

    @classmethod
    def load(cls, path: str = DEFAULT_COSTS) -> "Costs":
        c = cls.default()
        if os.path.exists(path):
            with open(path) as f:
                c.table.update(json.load(f)["coefficients"])
        return c

    def save(self, path: str, meta: Optional[dict] = None) -> None:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump({"coefficients": self.table, "meta": meta or {}}, f, indent=1, sort_keys=True)

    def predict_ns(self, st: PanelStats, n: int, nv: int, dtype: str = "f32", sms: int = SMS) -> float:
        coef = self.table.get(self.key(st.mr, nv, dtype), self.default().table["mr4_nv1_f32"])
        return float(np.dot(coef, model_row(st, n, nv, sms)))


def model_row(st: PanelStats, n: int, nv: int, sms: int = SMS) -> np.ndarray:
    strips = math.ceil(max(n, 1) / (32 * nv))
    row = np.zeros(6)
    row[0] = 1.0
    row[1:5] = strips * st.features(nv) / sms
    row[5] = st.max_panel_U
    return row


def fit_costs(samples: Sequence[Tuple[str, PanelStats, int, int, float]], sms: int = SMS,
              prior: Optional[Costs] = None) -> Costs:
    """Non-negative least squares of the model's coefficients per (M_r, NV, dtype).

    samples: (dtype, stats, n, nv, measured_ns)."""
    from scipy.optimize import nnls
    out = prior if prior is not None else Costs.default()
    groups: Dict[str, list] = {}
    for dt, st, n, nv, t in samples:
        groups.setdefault(Costs.key(st.mr, nv, dt), []).append((st, n, nv, t))
    for key, rows in groups.items():
        if len(rows) < 6:
            continue
        A = np.zeros((len(rows), 6))
        b = np.zeros(len(rows))
        for i, (st, n, nv, t) in enumerate(rows):
            A[i] = model_row(st, n, nv, sms)
            b[i] = t
        # relative error: weight each sample by 1 / t
        w = 1.0 / np.maximum(b, 1.0)
        coef, _ = nnls(A * w[:, None], b * w)
        out.table[key] = [float(x) for x in coef]
    return out


# ---------------------------------------------------------------------------- tuning
K_TILES = (0, 128, 256, 512, 1024)


def candidates(n: int, mrs: Iterable[int] = (2, 4, 8), k: int = 0,
               k_tiles: Iterable[int] = K_TILES, wide: bool = False) -> List[Candidate]:
    """Every (M_r, mapping, N_r, K_c) worth trying for n columns of B and K = k (K_c < K only).
    `wide` (16-bit B) adds 256-column strips for M_r <= 4 packs with K_c <= 128: the B-tile
    executor runs them, its stage holding K_c x 256 16-bit values."""
    out = []
    for mr in mrs:
        for mp in MAPPINGS_FOR_MR.get(mr, ("identity",)):
            for nr in (32, 64, 128, 256):
                if nr > 32 and n < nr // 2:
                    continue  # a strip wider than twice the columns only adds masked lanes
                for kt in k_tiles:
                    if kt and not (0 < kt < k):
                        continue
                    if nr == 256 and not (wide and mr <= 4 and 0 < kt <= 128):
                        continue
                    out.append(Candidate(mr, mp, nr, kt))
    return out


@dataclasses.dataclass
class TuneResult:
    best: Candidate
    predicted_ns: Dict[str, float]
    measured_ns: Dict[str, float]
    stats: Dict[str, dict]


def rank(mask: np.ndarray, n: int, dtype: str = "f32", costs: Optional[Costs] = None,
         mrs: Iterable[int] = (2, 4, 8), k_tiles: Iterable[int] = K_TILES, greedy: bool = True
         ) -> Tuple[List[Tuple[float, Candidate]], Dict[Tuple[int, str], PanelStats]]:
    """Candidates sorted by predicted time, and the statistics they were predicted from."""
    costs = costs if costs is not None else Costs.load()
    stats: Dict[Tuple[int, str], PanelStats] = {}
    ranked = []
    cands = candidates(n, mrs, mask.shape[1], k_tiles, wide=dtype != "f32")
    if greedy and 8 in tuple(mrs):
        gid = greedy_mapping(mask, 8).mapping_id
        cands += [Candidate(c.mr, gid, c.nr, c.k_tile) for c in cands if c.mr == 8 and c.mapping == "identity"]
    if greedy and 4 in tuple(mrs):
        gid4 = greedy_mapping(mask, 4, budget=15, tile=True).mapping_id
        if gid4 != mapping_of(4, "identity").mapping_id:
            cands += [Candidate(c.mr, gid4, c.nr, c.k_tile) for c in cands
                      if c.mr == 4 and c.mapping == "identity" and c.k_tile]
    for c in cands:
        key = (c.mr, c.mapping)
        if key not in stats:
            stats[key] = panel_stats(mask, c.mr, mapping_of(c.mr, c.mapping))
        # the model has no K_c term: K tiles only shrink per-warp metadata buffers (occupancy),
        # which the device timing decides; a tiny tie-break keeps untiled first among equals
        # 256-column strips have no fitted coefficients: the 128-column prediction, just ahead of
        # it, so the device timing of the top candidates compares the two
        nv = min(c.nv, 4)
        ranked.append((costs.predict_ns(stats[key], n, nv, dtype) * (1.0 + 1e-6 * (c.k_tile > 0)) *
                       (0.999 if c.nv > 4 else 1.0), c))
    ranked.sort(key=lambda x: x[0])
    return ranked, stats


def _time_batched(pm, Bs, Cs, nr: int, reps: int = 5, warps: int = 0, rounds: int = 0) -> float:
    """ns per SpMM of len(Bs) SpMMs of one packed matrix in one batched call, replayed from a CUDA graph
    (CUDA events): device time, as a serving loop or a batched layer step replays it.  Timing the calls
    themselves would add the host's planning per SpMM (tensor maps, problem tables), which at a few
    microseconds per SpMM is as large as the device time and favours the kernels that plan less."""
    import torch
    from .packed import execute_batched
    work = [(pm, b, c, dict(nr=nr, warps=warps, rounds=rounds)) for b, c in zip(Bs, Cs)]
    cur = torch.cuda.current_stream()
    side = torch.cuda.Stream()
    side.wait_stream(cur)
    with torch.cuda.stream(side):
        execute_batched(work)  # checks the arguments, configures the kernels before the capture
    cur.wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        execute_batched(work)
    g.replay()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(cur)
    for _ in range(reps):
        g.replay()
    e1.record(cur)
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e6 / (reps * len(Bs))


def _time_tc(At, mapping: Mapping, n: int, dtype: str, fill: float, k_tile: int, nb: int, reps: int = 5) -> float:
    """ns per SpMM of the hybrid at threshold `fill`: nb SpMMs of A with distinct B as one HybridBatch
    (one batched register-tiled launch, one tensor-core plan), replayed from a CUDA graph, CUDA events."""
    import torch
    from . import _lib
    from .hybrid import HybridBatch, HybridMatrix
    vd = _lib.BF16 if dtype == "bf16" else _lib.F32
    h = HybridMatrix.from_dense(At, mapping, fill, k_tile=k_tile, value_dtype=vd)
    tdt = torch.bfloat16 if dtype == "bf16" else torch.float32
    Bs = [torch.randn((At.shape[1], n), device=At.device).to(tdt) for _ in range(nb)]
    Cs = [torch.empty((At.shape[0], n), device=At.device) for _ in range(nb)]
    hb = HybridBatch([(h, b, c) for b, c in zip(Bs, Cs)])
    cur = torch.cuda.current_stream()
    side = torch.cuda.Stream()
    side.wait_stream(cur)
    with torch.cuda.stream(side):
        hb.run()
    cur.wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()  # device time, as `_time_batched`
    with torch.cuda.graph(g):
        hb.run()
    g.replay()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(cur)
    for _ in range(reps):
        g.replay()
    e1.record(cur)
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e6 / (reps * nb)


def tc_predict_ns(mask: np.ndarray, n: int, dtype: str, fill: float, mr: int) -> Tuple[float, float]:
    """(predicted ns of the tensor-core part, share of the nonzeros it takes) at threshold `fill`:
    dense products of the panels at or above it at a sustained tensor-core rate (three FP16 passes
    for the FP32-accurate split) plus set-up."""
    m, k = mask.shape
    P = (m + mr - 1) // mr
    nz = np.zeros(P * mr)
    nz[:m] = mask.sum(axis=1)
    pf = nz.reshape(P, mr).sum(axis=1) / float(mr * max(k, 1))
    sel = pf >= fill
    rows = int(sel.sum()) * mr
    passes = 3 if dtype == "f32" else 1
    rate = 0.9e15  # FLOP/s, dense products of these sizes through the plan
    share = float(nz.reshape(P, mr).sum(axis=1)[sel].sum() / max(nz.sum(), 1))
    return 3000.0 + 2.0 * rows * k * n * passes / rate * 1e9, share


def tune(A: np.ndarray, n: int, dtype: str = "f32", top: int = 4, costs: Optional[Costs] = None,
         mrs: Iterable[int] = (2, 4, 8), k_tiles: Iterable[int] = K_TILES, runs: int = 1, batch: int = 1,
         device=None, tc: bool = True, warps: bool = True, rounds: bool = True) -> TuneResult:
    """Pick the fastest candidate for weight A (M x K, float32, zeros pruned) and n columns of B:
    rank by the cost model, then time the ``top`` best on the device -- one SpMM at a time with
    the reference's protocol (execute_timed) when ``batch`` is 1, else ``batch`` SpMMs of A with
    distinct B in one batched launch, as a serving loop runs them.  Then (``warps``) the CTA tiling
    of the best register-tiled candidate, (n >= 256) the gather kernel's wide strips of untiled
    packs (256 and 512 columns), (``rounds``) panel rounds, and (``tc``) the tensor-core
    thresholds: every panel, and the densest tenth of the panels, each timed as a batch of SpMMs
    through `spreg.hybrid`."""
    import torch
    from . import _lib
    from .packed import PackedMatrix
    ranked, stats = rank(A != 0, n, dtype, costs, mrs, k_tiles)
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    vd = _lib.BF16 if dtype == "bf16" else _lib.F32
    tdt = torch.bfloat16 if dtype == "bf16" else torch.float32
    At = torch.from_numpy(np.ascontiguousarray(A, dtype=np.float32)).to(dev)
    nb = max(1, int(batch))
    Bs = [torch.randn((A.shape[1], n), device=dev).to(tdt) for _ in range(nb)]
    Cs = [torch.empty((A.shape[0], n), device=dev, dtype=tdt if nb > 1 else torch.float32) for _ in range(nb)]
    packs = {}
    measured = {}
    by_name = {c.name(): c for _, c in ranked}

    def time_reg(c):
        key = (c.mr, c.mapping, c.k_tile)
        if key not in packs:
            packs[key] = PackedMatrix.from_dense(At, mapping_of(c.mr, c.mapping), k_tile=c.k_tile, value_dtype=vd)
        if nb == 1:
            return packs[key].execute_timed(Bs[0], Cs[0], num_runs=runs, nr=c.nr, warps=c.warps, rounds=c.rounds)
        return _time_batched(packs[key], Bs, Cs, c.nr, warps=c.warps, rounds=c.rounds)

    # the model's top candidates, and the best-ranked candidate of every (M_r, nanokernel set) family,
    # so that a family the model underrates is still timed
    timed = [c for _, c in ranked[:max(1, top)]]
    seen = {(c.mr, c.mapping) for c in timed}
    for _, c in ranked:
        if (c.mr, c.mapping) not in seen:
            seen.add((c.mr, c.mapping))
            timed.append(c)
    for c in timed:
        measured[c.name()] = time_reg(c)
    best_reg = by_name[min(measured, key=measured.get)]
    if warps:
        # CTA tiling: fewer warps per CTA for the batched kernel (8 by default), fewer row panels per
        # job for the B-tile kernel (15 by default)
        for w in ((4,) if best_reg.k_tile == 0 else (8,)):
            c = dataclasses.replace(best_reg, warps=w)
            by_name[c.name()] = c
            measured[c.name()] = time_reg(c)
    best_reg = by_name[min(measured, key=measured.get)]
    if n >= 256:
        # wide strips of the gather kernel (untiled packs), each with the best-ranked nanokernel set
        # of its M_r: 256 columns (16-bit B: M_r <= 4), and 512 at M_r <= 4
        first = {}
        for _, c in ranked:
            if c.k_tile == 0 and c.mr not in first and (dtype == "f32" or c.mr <= 4):
                first[c.mr] = c
        for mr, c0 in sorted(first.items()):
            for nr in ((256, 512) if mr <= 4 and n >= 512 else (256,)):
                c = dataclasses.replace(c0, nr=nr, warps=4)
                by_name[c.name()] = c
                measured[c.name()] = time_reg(c)
        best_reg = by_name[min(measured, key=measured.get)]
    if rounds:
        # panel rounds: the B-tile kernel with the strip of B for every K tile resident, for the best
        # packing at its strip width and the narrower ones (a strip that does not fit shared memory
        # is refused by the executor and skipped)
        base = best_reg
        for nr in sorted({min(base.nr, 128), 64, 32}, reverse=True):
            for r in (4, 16):
                c = dataclasses.replace(base, nr=nr, warps=0, rounds=r)
                try:
                    t = time_reg(c)
                except _lib.SpregError:
                    break
                by_name[c.name()] = c
                measured[c.name()] = t
        best_reg = by_name[min(measured, key=measured.get)]
    predicted = {c.name(): t for t, c in ranked}
    if tc and n >= 16:
        mask = A != 0
        mr = best_reg.mr
        P = (A.shape[0] + mr - 1) // mr
        nz = np.zeros(P * mr)
        nz[:A.shape[0]] = mask.sum(axis=1)
        pf = nz.reshape(P, mr).sum(axis=1) / float(mr * max(A.shape[1], 1))
        fills = sorted({0.0, float(np.quantile(pf, 0.9))}) if P > 1 else [0.0]
        reg_mapping = mapping_of(best_reg.mr, best_reg.mapping)
        reg_ns = measured[best_reg.name()]
        for f in fills:
            c = dataclasses.replace(best_reg, tc_fill=f)
            t_tc, share = tc_predict_ns(mask, n, dtype, f, mr)
            predicted[c.name()] = t_tc + (1.0 - share) * reg_ns  # the register-tiled rest at its measured rate
            if predicted[c.name()] > 3.0 * reg_ns:
                continue  # the model rules it out
            by_name[c.name()] = c
            measured[c.name()] = _time_tc(At, reg_mapping, n, dtype, f, best_reg.k_tile, max(nb, 4))
    best_name = min(measured, key=measured.get)
    best = by_name[best_name]
    return TuneResult(best=best, predicted_ns=predicted, measured_ns=measured,
                      stats={f"M{k[0]}_{k[1]}": {"P": s.P, "U": s.U, "V": s.V, "G": s.G, "padding": s.padding}
                             for k, s in stats.items()})


def calibrate(shapes: Sequence[Tuple[int, int]] = ((512, 512), (2048, 512), (512, 2048), (1024, 4096)),
              sparsities: Sequence[float] = (0.7, 0.8, 0.9, 0.95, 0.98),
              ns: Sequence[int] = (16, 64, 128, 512, 1024), dtypes: Sequence[str] = ("f32", "bf16"),
              mrs: Iterable[int] = (2, 4, 8), seed: int = 0, device=None):
    """Time every (shape, sparsity, n, M_r, mapping, NV, dtype) on the device; returns the samples
    for `fit_costs`."""
    import torch
    from . import _lib, synth
    from .packed import PackedMatrix
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    samples = []
    for si, (m, k) in enumerate(shapes):
        for sp in sparsities:
            A = synth.row_skew(m, k, sp, seed=seed + 97 * si + int(sp * 1000), sigma=0.5, std=0.02)
            At = torch.from_numpy(A).to(dev)
            mask = A != 0
            for dt in dtypes:
                vd = _lib.BF16 if dt == "bf16" else _lib.F32
                tdt = torch.bfloat16 if dt == "bf16" else torch.float32
                for mr in mrs:
                    for mp in MAPPINGS_FOR_MR.get(mr, ("identity",)):
                        st = panel_stats(mask, mr, mapping_of(mr, mp))
                        pm = PackedMatrix.from_dense(At, mapping_of(mr, mp), value_dtype=vd)
                        for n in ns:
                            B = torch.randn((k, n), device=dev).to(tdt)
                            Cm = torch.empty((m, n), device=dev, dtype=torch.float32)
                            for nv in (1, 2, 4):
                                if nv > 1 and n < 16 * nv:
                                    continue
                                t = pm.execute_timed(B, Cm, num_runs=1, nr=32 * nv)
                                samples.append((dt, st, n, nv, t))
                        del pm
    return samples


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="Calibrate the executor cost model on this GPU")
    ap.add_argument("--out", default=DEFAULT_COSTS)
    ap.add_argument("--quick", action="store_true", help="fewer shapes and sparsities")
    args = ap.parse_args(argv)
    kw = {}
    if args.quick:
        kw = dict(shapes=((512, 512), (2048, 512)), sparsities=(0.8, 0.9, 0.95), ns=(32, 128, 512))
    samples = calibrate(**kw)
    costs = fit_costs(samples)
    # goodness of fit per key
    err = {}
    for dt, st, n, nv, t in samples:
        p = costs.predict_ns(st, n, nv, dt)
        err.setdefault(Costs.key(st.mr, nv, dt), []).append(abs(p - t) / t)
    meta = {"samples": len(samples), "median_rel_err": {k: float(np.median(v)) for k, v in err.items()}}
    costs.save(args.out, meta)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
