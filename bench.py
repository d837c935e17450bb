"""Benchmark of the sparse-register-tiling SpMM on GB300.

Workload (default): the FFN-shaped plain-FP32 SpMM -- A 2048 x 512 at 90 % sparsity with
log-normal row skew (sigma 0.5), values N(0, 0.02); B 512 x 512 FP32 N(0, 1).  Packed with
M_r = 4, K tiles of 128 and the nanokernel set chosen from replica 0's pattern histogram
(greedy set cover: the single rows plus the all-rows kernel), executed by the shared-memory
B-tile kernel.  One step runs the SpMM on R independent replicas (distinct seeds) whose working
set (R x ~6 MB) is several times the L2, so every step streams A, B and C from HBM.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl spreg|reference]

Prints one JSON line.  value = algorithmic GB/s of the whole job (packed values + column
indices + nkern_counts + panel descriptors + B + C per SpMM, divided by the device time of
the timed steps); e2e = the same metric through the host-buffer C ABI call
(spreg_matmul_run: B copied in, C copied out, inside the timed region).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "sparse-register-tiling_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = ("SpMM %HBM peak (plain FP32 sparse-register-tiling SpMM, A 2048x512 @90% row-skew, "
          "N=512): algorithmic GB/s")
UNIT = "GB/s"
L2_BYTES = 129 * 2 ** 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["spreg", "reference"], default="spreg")
    ap.add_argument("--replicas", type=int, default=96)
    ap.add_argument("--m", type=int, default=2048)
    ap.add_argument("--k", type=int, default=512)
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--sparsity", type=float, default=0.9)
    ap.add_argument("--nr", type=int, default=0)
    ap.add_argument("--staging", type=int, default=1, help="0 auto, 1 shared-memory B tiles, 2 L1/L2")
    ap.add_argument("--k-tile", type=int, default=128, help="K tile (K_c) of the packing; 0 = one tile")
    ap.add_argument("--mr", type=int, default=4, help="panel height M_r")
    ap.add_argument("--mapping", default="greedy",
                    help="identity, a mapping id, or greedy (set cover on replica 0's pattern histogram)")
    ap.add_argument("--meta", type=int, default=0, help="0 auto, 1 execution-layout kernel, 2 register streams")
    ap.add_argument("--dtype", choices=["f32", "bf16"], default="f32",
                    help="storage of A values and B (FP32 accumulation and FP32 C either way)")
    ap.add_argument("--path", choices=["hybrid", "register"], default="hybrid",
                    help="headline path: hybrid = FP32-accurate tensor-core panels (split FP16 products) beside "
                         "register-tiled panels by the tuned fill threshold; register = the bit-exact register-tiled "
                         "executor alone (it is timed either way)")
    ap.add_argument("--tc-fill", type=float, default=-1.0,
                    help="panel fill threshold of the hybrid; < 0: tuned on replica 0")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--batched", type=int, default=1, help="1: one batched launch per step; 0: one launch per SpMM")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline budget; 0 skips it")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end leg")
    ap.add_argument("--serving", type=int, default=1, help="1: add the serving-loop measurement to the line")
    ap.add_argument("--precision", type=int, default=1, help="1: add the storage-precision sweep to the line")
    ap.add_argument("--precision-only", default="",
                    help="run only this layer of the precision sweep, SHAPE:STORAGE (e.g. 2048x512:bf16); each "
                         "path's first launch is an NVTX range precision_<shape>_<storage>[_tc] for ncu --nvtx")
    ap.add_argument("--precision-configs", default="",
                    help="fixed packings of the precision sweep instead of tuning, f32=NAME,bf16=NAME (autotuner "
                         "candidate names, e.g. f32=M4N128_75a1b_K128): a profiled run makes the plain run's plan")
    ap.add_argument("--tensor-cores", type=int, default=1, help="1: add the tensor-core (tcgen05) leg to the line")
    ap.add_argument("--layers", type=int, default=1,
                    help="1: add the batched uneven transformer-layer measurement to the line")
    ap.add_argument("--ffn-sweep", type=int, default=1,
                    help="1: add the FFN-shaped FP32 sweep (2048x512 / 512x2048 at sparsity 0.7-0.98) to the line")
    ap.add_argument("--extras", type=int, default=1,
                    help="1: add the GPU CSR baseline and the config-1 (512x512) legs to the line")
    ap.add_argument("--serve-requests", type=int, default=768)
    ap.add_argument("--serve-slots", type=int, default=128)
    ap.add_argument("--serve-budget-mb", type=int, default=1024)
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def bench_mapping(args, A0):
    from spreg import Mapping
    if args.mapping == "identity":
        return Mapping.identity(args.mr)
    if args.mapping == "greedy":
        from spreg.kernel_sets import executor_penalty, greedy_kernel_set, pattern_histogram
        units = ((A0.shape[0] + args.mr - 1) // args.mr) * max(1, -(-A0.shape[1] // (args.k_tile or 128)))
        return greedy_kernel_set(pattern_histogram(A0, args.mr), args.mr, 2 ** args.mr - 1, units,
                                 penalty=executor_penalty(args.mr, tile=bool(args.k_tile)))
    return Mapping.load(args.mapping)


def make_inputs(args, rank: int):
    from spreg import synth
    from spreg.replicas import shard_seed
    As, Bs = [], []
    for r in range(args.replicas):
        seed = shard_seed(rank, r)
        As.append(synth.row_skew(args.m, args.k, args.sparsity, seed=seed, sigma=0.5, std=0.02))
        Bs.append(synth.dense(args.k, args.n, seed=seed + 500000))
    return As, Bs


def algorithmic_bytes_oracle(pk, n: int) -> int:
    """Same count as PackedMatrix.algorithmic_bytes for an oracle packing (FP32)."""
    s = pk.sizes
    return int(s["num_values"] * 4 + s["num_col_indices"] * 4 + s["num_units"] * pk.t.num_nkern * 4
               + s["num_units"] * 32 + pk.K * n * 4 + pk.M * n * 4)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 10 ms; `summary` keeps the samples that
    arrived between `mark_start` and `mark_end` (the timed region)."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[tuple] = []
        self.t = None
        self.t0 = None
        self.t1 = None

    def mark_start(self):
        self.t0 = time.perf_counter()

    def mark_end(self):
        self.t1 = time.perf_counter()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "10"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self) -> dict:
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0 = self.t0 if self.t0 is not None else float("-inf")
        t1 = self.t1 if self.t1 is not None else float("inf")
        inside = [ln for t, ln in self.lines if t0 <= t <= t1]
        if not inside and self.lines:  # a region shorter than one sampling interval: the nearest sample
            mid = (t0 + t1) / 2 if self.t0 is not None and self.t1 is not None else self.lines[-1][0]
            inside = [min(self.lines, key=lambda x: abs(x[0] - mid))[1]]
        for ln in inside:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                mhz.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not mhz:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(mhz)}


def load_traffic(key: str, spmms_per_launch: int):
    """DRAM bytes per launch from the ncu summaries in profiles/traffic.json (per-SpMM figure of the
    captured launch x SpMMs per launch), or None when that kernel and workload were not captured."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            e = json.load(f).get(key)
    except (OSError, ValueError):
        return None
    return None if not e else e["dram_bytes_per_spmm"] * spmms_per_launch


def smem_roofline(packs, n: int, bsz: int, k_tile: int, spmm_s: float, sm_mhz, sms: int = 152, warps: int = 15):
    """Shared-memory roofline of the B-tile executor (the bound it actually meets at FP32).

    Per SpMM the consumers read, for every packed entry (panel, column) and every strip of
    32 * NV columns, one B row segment of 32 * NV * bsz bytes out of shared memory, and the tensor
    copies write each K tile's strip of B once per job (W panels).  The peak is 128 bytes per clock
    per SM at the sampled SM clock.
    """
    if not sm_mhz or not k_tile:
        return None
    nv = 4 if n >= 128 else (2 if n >= 64 else 1)
    strip = 32 * nv
    strips = -(-n // strip)
    gathers = fills = 0
    for p in packs:
        i = p.info
        tiles = -(-(i["cols"]) // k_tile)
        gathers += i["num_col_indices"] * strips * strip * bsz
        fills += -(-(i["num_panels"]) // warps) * strips * tiles * k_tile * strip * bsz
    per_spmm = (gathers + fills) / len(packs)
    peak = sms * 128 * sm_mhz * 1e6 / 1e9
    achieved = per_spmm / spmm_s / 1e9
    return {"bound": "shared memory", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "bytes_per_spmm": per_spmm, "gather_bytes_per_spmm": gathers / len(packs),
            "fill_bytes_per_spmm": fills / len(packs), "peak_basis": f"{sms} SMs x 128 B/clk at {sm_mhz:.0f} MHz"}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def serving_bench(args, dev) -> dict:
    """12-block sparse MLP (d_model 1024, d_ff 4096, 90 % row-skew, BF16-representable weights
    N(0, 0.02)) served to requests of log-normal token counts (median 64, sigma 1, 1..2048):
    the continuous-batching BF16 server against the plain per-request FP32 path."""
    import torch
    from spreg import synth
    from spreg.serving import (Request, Server, SparseMLP, mlp_reference_fp64, mlp_weights, output_fp32,
                               prepare_requests, serve_per_request, tune_mlp)
    d_model, d_ff, blocks = 1024, 4096, 12
    w = mlp_weights(d_model, d_ff, blocks, 0.9, seed=77, std=0.02, sigma=0.5)
    t_tune = time.perf_counter()
    configs, tuned = tune_mlp(w, "bf16", n=96, batch=32, device=dev)
    t_tune = time.perf_counter() - t_tune
    bf = SparseMLP(w, "bf16", device=dev, configs=configs)
    # the plain FP32 path at its best single-request packing: the autotuner's choice for one request
    # of the median token count (candidates include the headline's K_c = 128 B-tile packing with the
    # histogram nanokernel set)
    t_fp = time.perf_counter()
    fp_configs, fp_tuned = tune_mlp(w, "f32", n=64, batch=1, device=dev)
    t_fp = time.perf_counter() - t_fp
    fp = SparseMLP(w, "f32", device=dev, configs=fp_configs)
    R = args.serve_requests
    ns = synth.token_counts(R, median=64, sigma=1.0, lo=1, hi=2048, seed=5)
    g = synth.rng(6)
    xs = [synth.round_bf16(g.standard_normal((d_model, int(n))).astype(np.float32)) for n in ns]

    def reqs_for(model, count, rate, seed):
        arr = synth.poisson_arrivals(count, rate, seed=seed)
        rs = [Request(i, int(ns[i]), x=xs[i], arrival=float(arr[i])) for i in range(count)]
        prepare_requests(model, rs)
        return rs

    server = Server(bf, budget_bytes=args.serve_budget_mb << 20, max_slots=args.serve_slots)
    server.run(reqs_for(bf, 16, float("inf"), 1))        # warm-up (first-call set-up, caches)
    serve_per_request(fp, reqs_for(fp, 8, float("inf"), 1))
    torch.cuda.synchronize()

    # capacity: every request queued at t = 0
    rb = reqs_for(bf, R, float("inf"), 2)
    cap_b = server.run(rb)
    n_plain = R  # the same requests as the server
    rp = reqs_for(fp, n_plain, float("inf"), 2)
    cap_p = serve_per_request(fp, rp)

    # the same requests on tensor-core layers (every panel a dense BF16 tcgen05 product)
    tcm = SparseMLP(w, "bf16", device=dev, tc=True)
    server_tc = Server(tcm, budget_bytes=args.serve_budget_mb << 20, max_slots=args.serve_slots)
    server_tc.run(reqs_for(tcm, 16, float("inf"), 1))
    rt = reqs_for(tcm, R, float("inf"), 2)
    cap_t = server_tc.run(rt)
    rt_lat = server_tc.run(reqs_for(tcm, min(R, max(64, int(2.0 * cap_p.req_per_s * 0.5))), 2.0 * cap_p.req_per_s, 30))

    # accuracy of served outputs against the FP64 stack (three small requests)
    pick = [i for i in np.argsort(ns[:n_plain])[:3]]
    err_b = max(float(np.linalg.norm(output_fp32(rb[i]) - (ref := mlp_reference_fp64(w, xs[i])))
                      / np.linalg.norm(ref)) for i in pick)
    err_p = max(float(np.linalg.norm(output_fp32(rp[i]) - (ref := mlp_reference_fp64(w, xs[i])))
                      / np.linalg.norm(ref)) for i in pick)
    err_t = max(float(np.linalg.norm(output_fp32(rt[i]) - (ref := mlp_reference_fp64(w, xs[i])))
                      / np.linalg.norm(ref)) for i in pick)

    # latency under Poisson arrivals at rates relative to the per-request path's capacity
    sweep = []
    for mult in (0.5, 0.9, 2.0, 4.0):
        rate = mult * cap_p.req_per_s
        cnt_b = min(R, max(64, int(rate * 0.5)))
        sb = server.run(reqs_for(bf, cnt_b, rate, 10 + int(mult * 10)))
        row = {"rate_req_s": rate, "batched_bf16": _stat(sb)}
        if mult <= 2.0:
            cnt_p = min(n_plain, max(32, int(rate * 0.3)))
            row["per_request_fp32"] = _stat(serve_per_request(fp, reqs_for(fp, cnt_p, rate, 10 + int(mult * 10))))
        sweep.append(row)
    return {"workload": "12-block sparse MLP d_model 1024 / d_ff 4096 @90% row-skew, BF16-representable weights "
                        "N(0,0.02), tokens log-normal(median 64, sigma 1) in 1..2048, residual stream",
            "batched_bf16": _stat(cap_b) | {"max_batch": cap_b.max_batch, "iterations": cap_b.iterations,
                                           "peak_activation_mib": cap_b.peak_activation_bytes / 2 ** 20,
                                           "slots": args.serve_slots, "budget_mib": args.serve_budget_mb},
            "per_request_fp32": _stat(cap_p) | {"packing": {"up": fp_tuned[0].best.name(), "down": fp_tuned[1].best.name(),
                                                            "tuned_for": "one request of 64 tokens",
                                                            "tune_seconds": t_fp}},
            "autotuned_packing": {"up": tuned[0].best.name(), "down": tuned[1].best.name(),
                                  "tune_seconds": t_tune,
                                  "measured_ns_per_spmm": {"up": tuned[0].measured_ns, "down": tuned[1].measured_ns}},
            "req_s_ratio": cap_b.req_per_s / cap_p.req_per_s,
            "batched_bf16_tensor_cores": _stat(cap_t) | {
                "req_s_ratio_vs_per_request_fp32": cap_t.req_per_s / cap_p.req_per_s,
                "rel_err_vs_fp64": err_t, "poisson_at_2x_per_request_capacity": _stat(rt_lat),
                "note": "every layer as a dense BF16 tcgen05 product: the hybrid split with panel-fill threshold 0"},
            "rel_err_vs_fp64": {"batched_bf16": err_b, "per_request_fp32": err_p, "bf16_tolerance": 1e-2},
            "sweep": sweep,
            "capacity_note": "capacity = all requests queued at t=0; latency = arrival to output in host memory"}


def precision_suite(dev, only: str = "", configs: str = "") -> list:
    """1x1-conv-shaped SpMMs (B = K x 3136: batch 1, 56 x 56 spatial) at sparsity 0.8-0.95 with
    log-normal row skew: rel err against FP64 of FP32, BF16 and FP16 (per-panel scaled) storage,
    FP32 accumulation, and the kernel time of each layer in each storage through the product's best
    path:
    * register-tiled: the autotuner's packing (M_r, nanokernel set, K tile, N_r, CTA tiling, panel
      rounds) for that storage, one SpMM per launch timed with the reference's protocol (median of
      150 x num_runs runs);
    * tensor cores (every panel, `spreg.hybrid`): BF16 storage as BF16 products, FP32 storage as the
      FP32-accurate split products; one SpMM per plan run (no host work), CUDA events over 50 runs.
    `best_*` takes the faster path of each storage; `bf16_speedup_vs_fp32` compares the best paths,
    `bf16_speedup_vs_fp32_register_tiled` the register-tiled ones."""
    import torch
    from oracle import oracle as O
    from spreg import BF16, F16, F32, PackedMatrix, synth
    from spreg.autotune import candidate_from_name, mapping_of, tune
    from spreg.hybrid import HybridBatch, HybridMatrix
    fixed = dict(kv.split("=", 1) for kv in configs.split(",") if kv)

    def tc_time(At, m, vd, Bt, M, tag):
        h = HybridMatrix.from_dense(At, m, 0.0, value_dtype=vd)
        Ch = torch.empty((M, Bt.shape[1]), device=dev)
        hb = HybridBatch([(h, Bt, Ch)])
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push(tag + "_tc")
        hb.run()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        for _ in range(3):
            hb.run()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(50):
            hb.run()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e3 / 50, Ch.cpu().numpy()

    rows = []
    only_shape, _, only_store = only.partition(":")
    for i, (M, K) in enumerate(((64, 256), (128, 512), (256, 1024), (512, 2048), (2048, 512))):
        sp = (0.8, 0.85, 0.9, 0.95, 0.9)[i]
        if only_shape and only_shape != f"{M}x{K}":
            continue
        A = synth.row_skew(M, K, sp, seed=300 + i, sigma=0.5, std=0.02)
        B = synth.dense(K, 3136, seed=400 + i)
        ref = O.dense_fp64(A, B)
        At = torch.from_numpy(A).to(dev)
        row = {"shape": [M, K], "sparsity": sp, "n": 3136}
        tuned = {}
        for name, vd, tdt in (("fp32", F32, torch.float32), ("bf16", BF16, torch.bfloat16), ("fp16", F16, torch.float16)):
            if only_store and only_store != name:
                continue
            tag = f"precision_{M}x{K}_{name}"
            tkey = "f32" if vd == F32 else "bf16"  # FP16 runs the 16-bit executor paths that BF16 tunes
            if tkey not in tuned:
                tuned[tkey] = (candidate_from_name(fixed[tkey], A) if tkey in fixed else
                               tune(A, 3136, tkey, top=4, device=dev, tc=False).best)
            c = tuned[tkey]
            pm = PackedMatrix.from_dense(At, mapping_of(c.mr, c.mapping), k_tile=c.k_tile, value_dtype=vd)
            Bt = torch.from_numpy(B).to(dev).to(tdt)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_push(tag)
            C = pm.execute(Bt, nr=c.nr, warps=c.warps, rounds=c.rounds)
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
            row[f"rel_err_{name}"] = float(O.rel_err(C.cpu().numpy(), ref))
            Cf = torch.empty((M, 3136), device=dev)
            t = pm.execute_timed(Bt, Cf, num_runs=2, nr=c.nr, warps=c.warps, rounds=c.rounds)
            row[f"{name}_us"] = t / 1e3
            row[f"{name}_gflops"] = 2 * int(pm.info["nnz"]) * 3136 / t
            row[f"{name}_gbs"] = pm.algorithmic_bytes(3136, b_bytes=4 if vd == F32 else 2) / t
            row[f"{name}_config"] = c.name()
            row[f"{name}_plan"] = pm.explain(Bt, Cf, nr=c.nr, warps=c.warps, rounds=c.rounds)
            if name != "fp16":
                # every panel on the tensor cores: BF16 products, or the FP32-accurate split
                t_tc, Ct = tc_time(At, mapping_of(c.mr, c.mapping), vd, Bt, M, tag)
                row[f"{name}_tc_us"] = t_tc
                row[f"{name}_tc_gbs"] = pm.algorithmic_bytes(3136, b_bytes=4 if vd == F32 else 2) / (t_tc * 1e3)
                row[f"rel_err_{name}_tc"] = float(O.rel_err(Ct, ref))
                row[f"best_{name}_us"] = min(row[f"{name}_us"], t_tc)
                row[f"best_{name}_path"] = "tensor cores" if t_tc < row[f"{name}_us"] else "register-tiled"
            if name != "fp32":
                # the same storage with its own inputs rounded: the error the kernel adds
                Bq = Bt.float().cpu().numpy()
                row[f"rel_err_{name}_vs_rounded_inputs"] = float(O.rel_err(
                    C.cpu().numpy(), O.dense_fp64(_rounded(A, vd, pm), Bq)))
        if "fp32_us" in row and "bf16_us" in row:
            row["bf16_speedup_vs_fp32_register_tiled"] = row["fp32_us"] / row["bf16_us"]
            row["bf16_speedup_vs_fp32"] = row["best_fp32_us"] / row["best_bf16_us"]
        rows.append(row)
    return rows


def csr_baseline_leg(A, B_dev, pack, args, batched_spmm_us: float) -> dict:
    """The reference's CSR baseline (csr.executor, row x N-tile) on the GPU beside the register-tiled
    executor, as sop_bench.py:197 times them: replica 0, one SpMM per launch, the reference's
    protocol (median of 150 x num_runs runs); bit-exact check against the restated baseline."""
    import ctypes as C

    import torch
    from oracle import oracle as O
    from spreg import _lib, synth
    rp, ci, v = synth.to_csr(A)
    dev = B_dev.device
    trp, tci, tv = (torch.from_numpy(x).to(dev) for x in (rp, ci, v))
    Cc = torch.empty((args.m, args.n), device=dev)
    t = C.c_double()
    _lib.check(_lib.lib().spreg_csr_spmm_timed(args.m, args.k, args.n, int(v.size), trp.data_ptr(), tci.data_ptr(),
                                               tv.data_ptr(), B_dev.data_ptr(), args.n, Cc.data_ptr(), args.n, 64, 10,
                                               C.byref(t), _lib.stream_handle(None)))
    torch.cuda.synchronize()
    exact = bool(np.array_equal(Cc.cpu().numpy(), O.csr_spmm(rp, ci, v, B_dev.cpu().numpy())))
    Cs = torch.empty((args.m, args.n), device=dev)
    sop_ns = pack.execute_timed(B_dev, Cs, num_runs=10)
    nbytes = v.size * 8 + rp.size * 4 + args.k * args.n * 4 + args.m * args.n * 4
    return {"csr_us": t.value / 1e3, "csr_gbs": nbytes / t.value, "csr_bit_exact_vs_oracle": exact,
            "sop_single_us": sop_ns / 1e3, "sop_batched_us": batched_spmm_us,
            "note": "replica 0; one SpMM per launch (median of 150 x 10 runs), except sop_batched_us (96 per launch)"}


def load_balance_leg(dev) -> list:
    """Single-SpMM latency with and without the load-balanced split (spreg_exec_args.load_balance): one
    SpMM per call, the reference's protocol (median of 150 x 10 runs), FP32, K tiles of 128, N = 512,
    the tile executor (b_staging 1) in both arms.  A 2048 x 512 @ 90 % with the headline's row skew
    (sigma 0.5) and with a heavier tail (sigma 1.2).  Alone, a launch has fewer jobs than SMs and the
    heaviest job groups set its time; the split halves their K chains on the idle SMs.  Checked bit
    for bit against the oracle's restatement of the split order and within 1e-6 of the unsplit
    result."""
    import torch
    from oracle import oracle as O
    from spreg import Mapping, PackedMatrix, synth
    rows = []
    m = Mapping.identity(4)
    for sigma in (0.5, 1.2):
        A = synth.row_skew(2048, 512, 0.9, seed=77, sigma=sigma, std=0.02)
        B = synth.dense(512, 512, seed=78)
        pm = PackedMatrix.from_dense(torch.from_numpy(A).to(dev), m, k_tile=128)
        Bd = torch.from_numpy(B).to(dev)
        C = torch.empty((2048, 512), device=dev)
        H, split, heavy = pm.load_balance_plan(Bd, C, staging=1)
        t_plain = pm.execute_timed(Bd, C, num_runs=10, staging=1)
        t_lb = pm.execute_timed(Bd, C, num_runs=10, staging=1, balance=1)
        got = pm.execute(Bd, C, staging=1, balance=1).cpu().numpy()
        want = O.load_balanced_execute(O.Tables.of(m), A, B, heavy, split, 128)
        plain = O.Packed(O.Tables.of(m), A, k_tile=128).execute(B)
        rows.append({"workload": f"A 2048x512 @90% row skew sigma {sigma}, N=512, FP32, K_c=128, M_r=4",
                     "heavy_panels": H, "panels": int(pm.info["num_panels"]), "split_tile": split,
                     "plain_us": t_plain / 1e3, "load_balanced_us": t_lb / 1e3, "speedup": t_plain / t_lb,
                     "bit_exact_vs_stated_order": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32))),
                     "rel_err_vs_unsplit": float(O.rel_err(got, plain))})
    return rows


def sparse_end_leg(dev, nb: int = 32, reps: int = 10) -> dict:
    """The memory-bound end of the FFN workload: 2048 x 512 @ 98 % row skew (sigma 0.5, values N(0, 0.02)),
    N = 512, FP32, nb SpMMs of one A with distinct B per batched launch, replayed from a CUDA graph,
    through these paths: the gather kernel (untiled M_r = 8 pack, 747f9 set, 128-column strips, 4 warps
    per CTA), its wide strips (256 and 512 columns at M_r 2, 4 and 8), panel rounds (64-column strips,
    16 rounds of 15 panels on a resident whole-K strip), and the FP32-accurate tensor-core hybrid
    (every panel).  Each path's first launch is an NVTX range
    sparse_end_<path> (for ncu --nvtx).  Register-tiled paths are checked bit for bit against the
    oracle, the hybrid against its tolerance.  Every path's GB/s divides the same algorithmic bytes,
    those of the M_r = 8 (747f9) pack, so the rates compare directly."""
    import torch
    from oracle import oracle as O
    from spreg import F32, Mapping, PackedMatrix, execute_batched, synth
    from spreg.hybrid import HybridBatch, HybridMatrix
    A = synth.row_skew(2048, 512, 0.98, seed=7098, sigma=0.5, std=0.02)
    Bs = [torch.from_numpy(synth.dense(512, 512, seed=7600 + i)).to(dev) for i in range(nb)]
    Cs = [torch.empty((2048, 512), device=dev) for _ in range(nb)]
    m8 = Mapping.load("747f9")
    peak, _ = measured_peaks()

    def graph_time(run, tag):
        cur = torch.cuda.current_stream()
        side = torch.cuda.Stream()
        side.wait_stream(cur)
        with torch.cuda.stream(side):
            run()
        cur.wait_stream(side)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push(tag)
        run()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            run()
        for _ in range(3):
            g.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            g.replay()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e3 / reps / nb

    out = {"workload": f"A 2048x512 @98% row skew, N=512, FP32, {nb} SpMMs of one A per launch, CUDA graph"}
    At = torch.from_numpy(A).to(dev)
    packs = {}
    B0 = Bs[0].cpu().numpy()
    nbytes = None
    # (path, mapping, executor options): the gather kernel at 128 columns (M_r 8, the tuner's pick
    # among 32-128-column strips), the wide FP32 gather strips, and panel rounds
    paths = (("gather", "747f9", dict(nr=128, warps=4)),
             ("wide_m8_256", "747f9", dict(nr=256, warps=4)),
             ("wide_m4_256", "identity4", dict(nr=256, warps=4)),
             ("wide_m4_512", "identity4", dict(nr=512, warps=4)),
             ("wide_m2_512", "identity2", dict(nr=512, warps=4)),
             ("wide_m2_512_w8", "identity2", dict(nr=512, warps=8)),
             ("rounds", "747f9", dict(nr=64, rounds=16)))
    for name, mname, kw in paths:
        if mname not in packs:
            m = m8 if mname == "747f9" else Mapping.identity(int(mname[-1]))
            pm_ = PackedMatrix.from_dense(At, m)
            packs[mname] = (pm_, O.Packed(O.Tables.of(m), A).execute(B0))
        pm, want = packs[mname]
        nbytes = nbytes or pm.algorithmic_bytes(512)
        work = [(pm, b, c, kw) for b, c in zip(Bs, Cs)]
        us = graph_time(lambda: execute_batched(work), f"sparse_end_{name}")
        got = Cs[0].cpu().numpy()
        out[name] = {"us_per_spmm": us, "gbs": nbytes / us / 1e3, "frac_of_measured_hbm": nbytes / us / 1e3 / peak,
                     "plan": pm.explain(Bs[0], Cs[0], **kw),
                     "bit_exact_vs_oracle": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))}
    # 16-bit storage: BF16 values and B, FP32 C, 512-column gather strips (M_r 2); its GB/s divides
    # the BF16 pack's own algorithmic bytes (2-byte values and B)
    from spreg import BF16
    m2 = Mapping.identity(2)
    pb = PackedMatrix.from_dense(At, m2, value_dtype=BF16)
    Bh = [b.to(torch.bfloat16) for b in Bs]
    wb = O.Packed(O.Tables.of(m2), A, value_dtype=BF16).execute(Bh[0].cpu().view(torch.int16).numpy().view(np.uint16))
    kwb = dict(nr=512, warps=4)
    workb = [(pb, b, c, kwb) for b, c in zip(Bh, Cs)]
    us = graph_time(lambda: execute_batched(workb), "sparse_end_wide_bf16_m2_512")
    nb16 = pb.algorithmic_bytes(512, b_bytes=2)
    out["wide_bf16_m2_512"] = {"us_per_spmm": us, "gbs": nb16 / us / 1e3, "frac_of_measured_hbm": nb16 / us / 1e3 / peak,
                               "plan": pb.explain(Bh[0], Cs[0], **kwb),
                               "bit_exact_vs_oracle": bool(np.array_equal(Cs[0].cpu().numpy().view(np.uint32),
                                                                          wb.view(np.uint32)))}
    pm, want = packs["747f9"]
    h = HybridMatrix.from_dense(torch.from_numpy(A).to(dev), m8, 0.0, value_dtype=F32)
    hb = HybridBatch([(h, b, c) for b, c in zip(Bs, Cs)])
    us = graph_time(hb.run, "sparse_end_tensor_cores")
    out["tensor_cores"] = {"us_per_spmm": us, "gbs": nbytes / us / 1e3, "frac_of_measured_hbm": nbytes / us / 1e3 / peak,
                           "rel_err_vs_oracle": float(O.rel_err(Cs[0].cpu().numpy(), want))}
    return out


def config1_leg(dev) -> dict:
    """The minimum slice as the workload states it: A 512 x 512 at 80 % Bernoulli sparsity, N(0, 1)
    values, B 512 x 256 N(0, 1), M_r = 4, identity mapping 61fee, N_r = 64.  GPU: one SpMM per call
    (median of 150 x 10 runs, the reference's execute_tile protocol, host work of each call included),
    and the same SpMM replayed from a CUDA graph (device time); CPU: the SIMD restatement of the
    reference executor on 1, 2, 4, 8 and all host threads (median of 7 each, the fastest reported
    beside); all checked bit for bit against the oracle, the GPU result also against FP64."""
    import torch
    from oracle import oracle as O
    from spreg import Mapping, PackedMatrix, synth
    A = synth.bernoulli(512, 512, 0.8, seed=0, std=1.0)
    B = synth.dense(512, 256, seed=1, std=1.0)
    m = Mapping.identity(4)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).to(dev), m)
    Bd = torch.from_numpy(B).to(dev)
    C = pm.execute(Bd, nr=64).cpu().numpy()
    ref = O.Packed(O.Tables.of(m), A)
    want = ref.execute(B)
    arena, descs, _ = pm.to_host()
    Cd = torch.empty((512, 256), device=dev)
    gpu_ns = pm.execute_timed(Bd, Cd, num_runs=10, nr=64)
    nbytes = pm.algorithmic_bytes(256)
    flops = pm.flops(256)
    out = {"workload": "A 512x512 @80% Bernoulli, N(0,1) values; B 512x256 N(0,1); M_r=4, N_r=64, mapping 61fee",
           "pack_bit_exact_vs_oracle": bool(np.array_equal(arena, ref.arena) and np.array_equal(descs, ref.descs)),
           "execute_bit_exact_vs_oracle": bool(np.array_equal(C.view(np.uint32), want.view(np.uint32))),
           "rel_err_vs_fp64": float(O.rel_err(C, O.dense_fp64(A, B))),
           "gpu_us": gpu_ns / 1e3, "gpu_gbs": nbytes / gpu_ns, "gpu_gflops": flops / gpu_ns,
           "algorithmic_bytes": nbytes, "flops": flops,
           "note": "one SpMM of 1.4 MB per launch: latency, not bandwidth, bounds the GPU time"}
    # the same SpMM replayed from a CUDA graph: device time without the per-call host work
    g = torch.cuda.CUDAGraph()
    s_ = torch.cuda.Stream()
    s_.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s_):
        pm.execute(Bd, Cd, nr=64)
    torch.cuda.current_stream().wait_stream(s_)
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        pm.execute(Bd, Cd, nr=64)
    for _ in range(5):
        g.replay()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(200):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    out["gpu_graph_us"] = e0.elapsed_time(e1) * 1e3 / 200
    out["gpu_graph_bit_exact"] = bool(np.array_equal(Cd.cpu().numpy().view(np.uint32), want.view(np.uint32)))
    threads = sorted({1, 2, 4, 8, O.max_threads()})
    for th in threads:
        ref.execute_fast(B, threads=th)
        ts = []
        for _ in range(7):
            t0 = time.perf_counter()
            got = ref.execute_fast(B, threads=th)
            ts.append(time.perf_counter() - t0)
        med = statistics.median(ts)
        out[f"cpu_simd_{th}t_us"] = med * 1e6
        out[f"cpu_simd_{th}t_gbs"] = nbytes / med / 1e9
        out[f"cpu_simd_{th}t_bit_exact"] = bool(np.array_equal(got.view(np.uint32), want.view(np.uint32)))
    best = min(threads, key=lambda th: out[f"cpu_simd_{th}t_us"])
    out["cpu_simd_best"] = {"threads": best, "us": out[f"cpu_simd_{best}t_us"]}
    out["gpu_vs_cpu_best"] = out[f"cpu_simd_{best}t_us"] / out["gpu_us"]
    return out


def ffn_sweep(dev, min_replicas: int = 96, steps: int = 20) -> list:
    """The FFN-shaped workload across its sparsities and storage types: A 2048 x 512 and 512 x 2048
    at 0.7, 0.8, 0.9, 0.95 and 0.98 (log-normal row skew, sigma 0.5, values N(0, 0.02)), B K x 512
    N(0, 1); FP32, BF16 and FP16 (per-panel scaled) storage of A values and B, FP32 accumulation
    and FP32 C.

    Each point runs enough distinct replicas that their algorithmic bytes reach 4 x L2 (at least
    `min_replicas`) in one batched launch of the autotuner's register-tiled packing for that point
    and storage (M_r, nanokernel set, N_r, K tile, CTA tiling, panel rounds; tuned on replica 0 as a
    batch of 32, the six best-ranked candidates and the best of every family timed),
    replayed from a CUDA graph.  It reports algorithmic GB/s (2-byte values and B for the 16-bit
    forms) and GFLOP/s (2 nnz N), and checks replica 0 bit for bit against the oracle and against
    FP64.  Beside it, the FP32-accurate tensor-core hybrid with every panel on the tensor cores
    (split FP16 products), timed the same way.
    """
    import torch
    from oracle import oracle as O
    from spreg import BF16, F16, F32, PackedMatrix, execute_batched, synth
    from spreg.autotune import mapping_of, tune
    from spreg.hybrid import HybridBatch, HybridMatrix
    peak, _ = measured_peaks()
    forms = (("fp32", F32, torch.float32), ("bf16", BF16, torch.bfloat16), ("fp16", F16, torch.float16))

    def timed(run):
        run()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            run()
        for _ in range(3):
            g.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(steps):
            g.replay()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / steps

    rows = []
    for M, K in ((2048, 512), (512, 2048)):
        for sp in (0.7, 0.8, 0.9, 0.95, 0.98):
            A0 = synth.row_skew(M, K, sp, seed=7000 + int(sp * 100), sigma=0.5, std=0.02)
            B0 = torch.from_numpy(synth.dense(K, 512, seed=7500 + K)).to(dev)
            exact = O.dense_fp64(A0, B0.cpu().numpy())
            row = {"shape": [M, K], "sparsity": sp, "n": 512}
            tuned = {}
            As = None
            for name, vd, tdt in forms:
                tkey = "f32" if vd == F32 else "bf16"
                if tkey not in tuned:
                    tuned[tkey] = tune(A0, 512, tkey, top=6, batch=32, device=dev, tc=False).best
                c = tuned[tkey]
                m = mapping_of(c.mr, c.mapping)
                p0 = PackedMatrix.from_dense(torch.from_numpy(A0).to(dev), m, k_tile=c.k_tile, value_dtype=vd)
                per = p0.algorithmic_bytes(512, b_bytes=4 if vd == F32 else 2)
                replicas = max(min_replicas, -(-4 * L2_BYTES // per))
                if As is None or len(As) < replicas:
                    As = [A0] + [synth.row_skew(M, K, sp, seed=7000 + 10 * r + int(sp * 100) + 1, sigma=0.5, std=0.02)
                                 for r in range(1, replicas)]
                packs = [p0] + [PackedMatrix.from_dense(torch.from_numpy(A).to(dev), m, k_tile=c.k_tile, value_dtype=vd)
                                for A in As[1:replicas]]
                Bd = [B0.roll(r, 0).to(tdt) for r in range(replicas)]  # a distinct B per replica
                Cd = [torch.empty((M, 512), device=dev) for _ in range(replicas)]
                work = [(p, b, cc, dict(nr=c.nr, warps=c.warps, rounds=c.rounds)) for p, b, cc in zip(packs, Bd, Cd)]
                sec = timed(lambda: execute_batched(work))
                bsz = 4 if vd == F32 else 2
                nbytes = sum(p.algorithmic_bytes(512, b_bytes=bsz) for p in packs)
                flops = sum(p.flops(512) for p in packs)
                got = Cd[0].cpu().numpy()
                Bq = Bd[0].cpu()
                Bref = Bq.numpy() if vd == F32 else Bq.view(torch.int16).numpy().view(np.uint16)
                want = O.Packed(O.Tables.of(m), A0, k_tile=c.k_tile, value_dtype=vd).execute(Bref)
                row[name] = {"spmm_us": sec / replicas * 1e6, "gbs": nbytes / sec / 1e9,
                             "frac_of_measured_hbm": nbytes / sec / 1e9 / peak, "gflops": flops / sec / 1e9,
                             "config": c.name(), "replicas": replicas,
                             "working_set_mib": (nbytes + (0 if vd == F32 else 0)) / 2 ** 20,
                             "bit_exact_vs_oracle": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32))),
                             "rel_err_vs_fp64": float(O.rel_err(got, exact))}
                if name == "fp32":
                    # the FP32-accurate hybrid with every panel on the tensor cores, same replicas
                    hs = [HybridMatrix.from_dense(torch.from_numpy(A).to(dev), m, 0.0, k_tile=c.k_tile, value_dtype=F32)
                          for A in As[:replicas]]
                    Ch = [torch.empty((M, 512), device=dev) for _ in range(replicas)]
                    hb = HybridBatch(list(zip(hs, Bd, Ch)))
                    sec_h = timed(hb.run)
                    gh = Ch[0].cpu().numpy()
                    row["fp32_tensor_cores"] = {
                        "spmm_us": sec_h / replicas * 1e6, "gbs": nbytes / sec_h / 1e9,
                        "frac_of_measured_hbm": nbytes / sec_h / 1e9 / peak, "gflops": flops / sec_h / 1e9,
                        "rel_err_vs_oracle": float(O.rel_err(gh, want)), "rel_err_vs_fp64": float(O.rel_err(gh, exact)),
                        "path": "every panel as a split-FP16 tcgen05 product (hi.hi + hi.lo + lo.hi)"}
                    del hs, Ch, hb
                del packs, Bd, Cd, work
            rows.append(row)
    return rows


def _rounded(A, vd, pm):
    """A's values as the packed storage holds them (BF16 / FP16 with the per-panel scale)."""
    import torch
    from spreg import BF16
    if vd == BF16:
        return torch.from_numpy(A).to(torch.bfloat16).float().numpy()
    arena, descs, scales = pm.to_host()
    mr = pm.info["mr"]
    out = np.zeros_like(A)
    for p in range(pm.info["num_panels"]):
        s = float(scales[p])
        blk = A[p * mr:(p + 1) * mr]
        out[p * mr:(p + 1) * mr] = torch.from_numpy(blk / s).to(torch.float16).float().numpy() * s
    return out


def layers_suite(dev, steps: int = 50) -> dict:
    """The 36 sparse linear layers of a 6-layer transformer (Q/K/V/O 512x512, FFN 2048x512 and
    512x2048) at 90 % row-skew sparsity, BF16 values and B, FP32 output, N per instance uniform in
    16..1024: the fixed-tile plain path (one launch per SpMM: M_r = 4, N_r = 64, untiled) against
    one step of autotuned layers -- M_r, nanokernel set, N_r, K tile, CTA tiling and tensor-core
    threshold per layer -- with every register-tiled part in one batched launch and every
    tensor-core part in one tcgen05 plan, replayed from a CUDA graph."""
    import torch
    from spreg import BF16, Mapping, PackedMatrix, execute_batched, synth
    from spreg.autotune import mapping_of, tune
    from spreg.hybrid import DenseRowsPlan, HybridMatrix, bf16_items
    g = synth.rng(900)
    shapes = []
    for _ in range(6):
        shapes += [(512, 512)] * 4 + [(2048, 512), (512, 2048)]
    ns = [int(x) for x in g.integers(16, 1025, size=len(shapes))]
    As = [synth.row_skew(M, K, 0.9, seed=1000 + i, sigma=0.5, std=0.02) for i, (M, K) in enumerate(shapes)]
    Bs = [torch.from_numpy(synth.dense(K, n, seed=2000 + i)).to(dev).to(torch.bfloat16)
          for i, ((M, K), n) in enumerate(zip(shapes, ns))]
    Cp = [torch.empty((M, n), device=dev) for (M, K), n in zip(shapes, ns)]
    Cb = [torch.empty((M, n), device=dev) for (M, K), n in zip(shapes, ns)]
    m4 = Mapping.identity(4)
    plain = [PackedMatrix.from_dense(torch.from_numpy(A).to(dev), m4, value_dtype=BF16) for A in As]
    flops = sum(2 * int(p.info["nnz"]) * n for p, n in zip(plain, ns))
    t0 = time.perf_counter()
    tuned, cfg = [], []
    cache = {}
    for A, n, (M, K) in zip(As, ns, shapes):
        key = (M, K, min(1024, 1 << max(4, int(n - 1).bit_length())))  # tune once per shape and N octave
        if key not in cache:
            cache[key] = tune(A, n, "bf16", top=6, batch=4, device=dev).best
        c = cache[key]
        cfg.append(c)
        At = torch.from_numpy(A).to(dev)
        if c.tc_fill <= 1.0:
            tuned.append(HybridMatrix.from_dense(At, mapping_of(c.mr, c.mapping), c.tc_fill, k_tile=c.k_tile,
                                                 value_dtype=BF16))
        else:
            tuned.append(PackedMatrix.from_dense(At, mapping_of(c.mr, c.mapping), k_tile=c.k_tile, value_dtype=BF16))
    t_tune = time.perf_counter() - t0

    def plain_step():
        for p, B, C in zip(plain, Bs, Cp):
            p.execute(B, C, nr=64)

    work, tc_rows = [], []
    for t, B, C, c in zip(tuned, Bs, Cb, cfg):
        if isinstance(t, HybridMatrix):
            if t.tc_rows:
                tc_rows.append((t.a_rows, t.row_index, B, C, B.shape[1], t.cols, False, 0))
            if not t.all_tc:
                work.append((t.packed, B, C, dict(nr=c.nr, warps=c.warps, rounds=c.rounds)))
        else:
            work.append((t, B, C, dict(nr=c.nr, warps=c.warps, rounds=c.rounds)))
    plan = DenseRowsPlan(bf16_items(tc_rows)) if tc_rows else None

    def batched_step():
        if work:
            execute_batched(work)  # register-tiled parts first: no load_c, the tensor-core rows follow
        if plan is not None:
            plan.run()

    def time_it(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps * 1e3

    t_plain = time_it(plain_step)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        batched_step()
    torch.cuda.current_stream().wait_stream(s)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        batched_step()
    t_batched = time_it(graph.replay)
    err = max(float((a - b).norm() / max(b.norm(), 1e-30)) for a, b in zip(Cb, Cp))
    # accuracy of every tuned layer against FP64 of its BF16 operands
    err64 = 0.0
    for A, B, C in zip(As, Bs, Cb):
        Aq = torch.from_numpy(A).to(torch.bfloat16).double().to(dev)
        ref = Aq @ B.double()
        err64 = max(err64, float((C.double() - ref).norm() / ref.norm()))
    return {"workload": "36 layers (6 x Q/K/V/O 512x512, FFN 2048x512, 512x2048) @90% row-skew, BF16 values and B, "
                        "FP32 out, N uniform 16..1024 per layer",
            "plain_fixed_tile_us": t_plain, "batched_autotuned_graph_us": t_batched, "speedup": t_plain / t_batched,
            "plain_tflops": flops / t_plain / 1e6, "batched_tflops": flops / t_batched / 1e6,
            "plain_launches_per_step": len(plain), "tune_seconds": t_tune,
            "layers_on_tensor_cores": sum(1 for c in cfg if c.tc_fill <= 1.0),
            "per_layer_config": [{"shape": list(sh), "n": n, "config": c.name()} for sh, n, c in zip(shapes, ns, cfg)],
            "max_rel_diff_batched_vs_plain": err, "max_rel_err_vs_fp64_of_bf16_operands": err64}


def tensor_core_suite(dev, reps: int = 20) -> dict:
    """The tcgen05 dense-rows kernel: a dense BF16 product (4096 x 4096 x 4096, FP32 accumulation)
    against the measured bf16 peak, and the hybrid threshold of the serving layers (90 % row-skew,
    BF16) timed on the device."""
    import torch
    from spreg import Mapping, synth
    from spreg.hybrid import dense_rows_bf16, tune_tc_fill
    M = K = N = 4096
    g = torch.Generator(device=dev).manual_seed(0)
    a = torch.randn((M, K), device=dev, generator=g).to(torch.bfloat16)
    b = torch.randn((K, N), device=dev, generator=g).to(torch.bfloat16)
    c = torch.empty((M, N), device=dev)
    idx = torch.arange(M, device=dev, dtype=torch.int32)
    dense_rows_bf16(a, idx, b, c)  # checks the row indices once
    for _ in range(3):
        dense_rows_bf16(a, idx, b, c, check_rows=False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        dense_rows_bf16(a, idx, b, c, check_rows=False)
    e1.record()
    torch.cuda.synchronize()
    us = e0.elapsed_time(e1) / reps * 1e3
    ref = a[:256].float() @ b.float()
    err = float((c[:256] - ref).norm() / ref.norm())
    tflops = 2.0 * M * N * K / us / 1e6
    # the same product as a reusable plan (tensor maps and tables made once): the kernel alone
    from spreg.hybrid import DenseRowsPlan, bf16_items
    plan = DenseRowsPlan(bf16_items([(a, idx, b, c, N, K, False, 0)]))
    for _ in range(3):
        plan.run()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        plan.run()
    e1.record()
    torch.cuda.synchronize()
    us_plan = e0.elapsed_time(e1) / reps * 1e3
    plan.close()
    tflops_plan = 2.0 * M * N * K / us_plan / 1e6
    peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except (OSError, ValueError, KeyError):
        pass
    hyb = {}
    for (m, k, kt, n) in ((4096, 1024, 512, 128), (1024, 4096, 1024, 128)):
        A = torch.from_numpy(synth.round_bf16(synth.row_skew(m, k, 0.9, seed=3, sigma=0.5, std=0.02))).to(dev)
        hyb[f"{m}x{k}_n{n}"] = tune_tc_fill(A, Mapping.identity(2), n, k_tile=kt)
    return {"dense_bf16_4096^3_us": us, "tflops": tflops, "peak_tflops": peak,
            "frac_of_measured_peak": (tflops / peak) if peak else None,
            "plan_run_us": us_plan, "plan_run_tflops": tflops_plan,
            "plan_run_frac_of_measured_peak": (tflops_plan / peak) if peak else None,
            "rel_err_vs_fp32_of_bf16_inputs": err, "includes": "API call: tcgen05 kernel reading B in place (N-major operand), one CTA per SM, set-up and launch",
            "hybrid_threshold_serving_layers": hyb}


def _stat(st) -> dict:
    return {"req_s": st.req_per_s, "tokens_s": st.tokens_per_s, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms,
            "mean_ms": st.mean_ms, "requests": st.requests}


def cpu_baseline(As, Bs, args, seconds: float, threads: int = 0, mapping=None):
    """Restated reference executor (oracle, OpenMP) on a bounded sample of the same workload."""
    from oracle import oracle as O
    from spreg.mapping import Mapping
    t = O.Tables.of(mapping if mapping is not None else Mapping.identity(args.mr))
    done_bytes, done_flops, runs, i = 0, 0, 0, 0
    packs = {}
    t0 = time.perf_counter()
    elapsed = 0.0
    while elapsed < seconds and runs < 10000:
        r = i % len(As)
        if r not in packs:
            packs[r] = O.Packed(t, As[r], k_tile=args.k_tile)
        pk = packs[r]
        s = time.perf_counter()
        pk.execute_fast(Bs[r], threads=threads)
        elapsed_run = time.perf_counter() - s
        done_bytes += algorithmic_bytes_oracle(pk, args.n)
        done_flops += 2 * pk.sizes["nnz"] * args.n
        runs += 1
        i += 1
        elapsed += elapsed_run
        if time.perf_counter() - t0 > 3 * seconds:
            break
    return {"value": done_bytes / elapsed / 1e9, "unit": UNIT, "gflops": done_flops / elapsed / 1e9,
            "cores": threads if threads > 0 else O.max_threads(), "kind": "port",
            "sample": f"{runs} SpMMs of the workload ({len(packs)} distinct replicas), {elapsed:.1f} s of "
                      "executor time, the reference's register-tiled executor restated as SIMD code "
                      "(oracle/spreg_cpu_fast.c: M_r x 16 accumulators in vector registers, one FMA block per "
                      "nanokernel pattern, bit-identical to the checker) with OpenMP over panels"}


def host_cpu() -> dict:
    """Model and logical CPUs of this host (lscpu where present, else /proc/cpuinfo)."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":")[0].strip() in ("Model name", "Model"):
                model = model or ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    if not model and os.path.exists("/proc/cpuinfo"):
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith(("model name", "cpu part")):
                model = ln.split(":", 1)[1].strip()
                break
    return {"model": model or "unknown", "nproc": os.cpu_count()}


def cpu_baselines(As, Bs, args, mapping, seconds: float = 2.0) -> dict:
    """The CPU protocol around the headline workload, each on a bounded sample (about `seconds` of
    compute per entry): the restated reference executor and the restated CSR baseline
    (pytorch_csr_wrapper.cpp / spmm_csr_c.cpp row x N-tile loop), on 1 thread and on all threads,
    median of 7 repetitions of one SpMM (SPMM_demo.cpp's protocol) after one warm-up."""
    from oracle import oracle as O
    from spreg import synth
    t = O.Tables.of(mapping)
    pk = O.Packed(t, As[0], k_tile=args.k_tile)
    rp, ci, v = synth.to_csr(As[0])
    nbytes = algorithmic_bytes_oracle(pk, args.n)
    flops = 2 * pk.sizes["nnz"] * args.n
    csr_bytes = v.size * 8 + rp.size * 4 + args.k * args.n * 4 + args.m * args.n * 4
    out = {"host": host_cpu(), "sample": "replica 0 of the headline workload, median of 7 runs after 1 warm-up",
           "legs": "simd: vector-register accumulators, FMAs contracted (-ffp-contract=fast), bit-identical to the "
                   "scalar checker (explicit fmaf chain, -ffp-contract=off) that the parity tests use"}
    legs = [("sop_executor_simd", lambda th: pk.execute_fast(Bs[0], threads=th), nbytes, (1, O.max_threads())),
            ("csr_baseline_simd", lambda th: O.csr_spmm_fast(rp, ci, v, Bs[0], threads=th), csr_bytes,
             (1, O.max_threads())),
            ("sop_executor_scalar_checker", lambda th: pk.execute(Bs[0], threads=th), nbytes, (1, O.max_threads())),
            ("csr_baseline_scalar", lambda th: O.csr_spmm(rp, ci, v, Bs[0], threads=th), csr_bytes,
             (1, O.max_threads()))]
    if O.has_ref():  # the reference's own scalar CSR SpMM, compiled from its source where that exists
        legs.append(("spmm_naive", lambda th: O.ref_naive(rp, ci, v, Bs[0]), csr_bytes, (1,)))
    else:
        out["spmm_naive"] = "not built on this host: the reference's source is absent here"
    for name, run, b, thread_counts in legs:
        for th in thread_counts:
            run(th)
            ts = []
            t_end = time.perf_counter() + seconds
            while len(ts) < 7 and (not ts or time.perf_counter() < t_end):
                s = time.perf_counter()
                run(th)
                ts.append(time.perf_counter() - s)
            med = statistics.median(ts)
            out[f"{name}_{th}t"] = {"ms": med * 1e3, "gbs": b / med / 1e9, "gflops": flops / med / 1e9,
                                    "threads": th, "runs": len(ts)}
    return out


def workload_config(args, m, working_set: int) -> dict:
    """`config` of the JSON line: the workload and its packing, the same in both arms."""
    return {"workload": f"spmm_f32_{args.m}x{args.k}_s{args.sparsity}_n{args.n}_x{args.replicas}",
            "replicas": args.replicas, "m": args.m, "k": args.k, "n": args.n, "sparsity": args.sparsity,
            "mr": args.mr, "mapping": m.mapping_id,
            "nanokernels": m.nanokernels if args.mapping != "identity" else "all", "k_tile": args.k_tile,
            "l2": (f"inputs {'larger' if working_set > L2_BYTES else 'SMALLER'} than L2: working set "
                   f"{working_set / 2**20:.0f} MiB per step vs {L2_BYTES / 2**20:.0f} MiB L2")}


def run_reference(args):
    """--impl reference: the reference's CPU algorithm (restated; its own executor source is absent)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build(with_reference=False) if not os.path.exists(O.LIB_PATH) else None
    As, Bs = make_inputs(args, 0)
    m = bench_mapping(args, As[0])
    t = O.Tables.of(m)
    packs = [O.Packed(t, A, k_tile=args.k_tile) for A in As]
    per_step = sum(algorithmic_bytes_oracle(p, args.n) for p in packs)
    for _ in range(args.warmup):
        for p, B in zip(packs, Bs):
            p.execute_fast(B)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for p, B in zip(packs, Bs):
            p.execute_fast(B)
    dt = time.perf_counter() - t0
    v = per_step * args.steps / dt / 1e9
    cores = O.max_threads()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded row-skew sparse A, N(0,1) B)",
            "config": workload_config(args, m, per_step),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"the full workload ({args.replicas} replicas) per step, the reference's "
                                       "register-tiled executor restated as SIMD code (oracle/spreg_cpu_fast.c, "
                                       "bit-identical to the checker), OpenMP over all host threads",
                             "host": host_cpu()},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def hybrid_leg(args, As, Bs, m, dev, step_bytes: int, step_flops: int, clk, peak: float, peak_kind: str) -> dict:
    """The FP32-accurate hybrid on the headline workload: panels whose fill reaches the tuned threshold
    run as split-FP16 tensor-core products (spreg_dense_rows_f32: hi.hi + hi.lo + lo.hi, FP32
    accumulation), the others register-tiled; all replicas per step as one HybridBatch (register-tiled
    parts in one batched launch, tensor-core parts as one reusable plan: B split + one tcgen05
    launch), replayed from a CUDA graph.  Parity: rel err against the oracle's FP32 executor and
    FP64 for replicas 0..3 (tolerance 1e-5)."""
    import torch
    from oracle import oracle as O
    from spreg import F32
    from spreg.hybrid import HybridBatch, HybridMatrix, tune_tc_fill
    t0 = time.perf_counter()
    if args.tc_fill < 0:
        tuned = tune_tc_fill(torch.from_numpy(As[0]).to(dev), m, args.n, fills=(1.01, 0.3, 0.2, 0.15, 0.1, 0.05, 0.0),
                             k_tile=args.k_tile, value_dtype=F32, batch=16)
    else:
        tuned = {"us": {}, "best_fill": args.tc_fill, "batch": 0}
    t_tune = time.perf_counter() - t0
    fill = tuned["best_fill"]
    hs = [HybridMatrix.from_dense(torch.from_numpy(A).to(dev), m, fill, k_tile=args.k_tile, value_dtype=F32)
          for A in As]
    Bd = [torch.from_numpy(B).to(dev) for B in Bs]
    Cd = [torch.empty((args.m, args.n), device=dev) for _ in As]
    batch = HybridBatch(list(zip(hs, Bd, Cd)))
    batch.run()
    torch.cuda.synchronize()
    errs_ref, errs_64 = [], []
    for r in range(min(4, len(As))):
        got = Cd[r].cpu().numpy()
        want = O.Packed(O.Tables.of(m), As[r], k_tile=args.k_tile).execute(Bs[r])
        errs_ref.append(O.rel_err(got, want))
        errs_64.append(O.rel_err(got, O.dense_fp64(As[r], Bs[r])))
    stream = torch.cuda.current_stream()
    graph = None
    if not args.no_graph:
        s2 = torch.cuda.Stream()
        s2.wait_stream(stream)
        with torch.cuda.stream(s2):
            batch.run()
        stream.wait_stream(s2)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            batch.run()
        torch.cuda.synchronize()
    run = graph.replay if graph is not None else batch.run
    for _ in range(max(args.warmup, 3)):
        run()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    lead = args.path == "hybrid"
    if lead:
        clk.mark_start()
    ev0.record(stream)
    for _ in range(args.steps):
        run()
    ev1.record(stream)
    torch.cuda.synchronize()
    if lead:
        clk.mark_end()
    ms = ev0.elapsed_time(ev1)
    step_s = ms / 1e3 / args.steps
    tc_rows = sum(h.tc_rows for h in hs)
    sparse_launch = any(not h.all_tc for h in hs)
    kernels = ["split_cols_kernel", "tc_rows_kernel<256,true>"] + (["exec_tile_kernel"] if sparse_launch else [])
    achieved = step_bytes / step_s / 1e9
    # bytes the split path moves per SpMM (dense split A of the tensor-core rows, B read and its split
    # pair written and read, C written), for comparison with the algorithmic bytes
    moved = (tc_rows / len(hs)) * args.k * 4 + args.k * args.n * (4 + 4 + 4) + args.m * args.n * 4
    return {"value": achieved, "ms": ms, "step_s": step_s, "spmm_us": step_s / len(hs) * 1e6,
            "gflops": step_flops / step_s / 1e9, "tc_fill": fill, "tc_rows_per_spmm": tc_rows / len(hs),
            "tuning": {"us_per_spmm_by_fill": tuned["us"], "best_fill": tuned["best_fill"], "seconds": t_tune,
                       "timed_as": f"{tuned['batch']} SpMMs of replica 0 per HybridBatch run"},
            "rel_err_vs_oracle_fp32_executor": max(errs_ref), "rel_err_vs_fp64": max(errs_64),
            "tolerance": 1e-5, "within_tolerance": max(errs_ref) <= 1e-5 and max(errs_64) <= 1e-5,
            "cuda_graph": graph is not None, "launches_per_step": len(kernels),
            "kernels": kernels, "split_path_bytes_per_spmm": moved,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": f"{peak_kind} hbm_gbs", "kernel": "spreg::tc_rows_kernel<256,true>",
                         "timing": "per step (B split launch + tensor-core launch); the tensor-core kernel's share "
                                   "of the step is in the ncu launch list summary",
                         "algorithmic_bytes_per_step": step_bytes, "launch_us": step_s * 1e6}}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)

    from oracle import oracle as O
    from spreg import Mapping, MatMulSpecialized, PackedMatrix, TileConfig, synth
    from spreg.replicas import max_over_ranks, whole_job_rate

    As, Bs = make_inputs(args, rank)
    m = bench_mapping(args, As[0])
    vd = spreg_dtype = (0 if args.dtype == "f32" else 1)
    tdt = torch.float32 if args.dtype == "f32" else torch.bfloat16
    packs, Bd, Cd = [], [], []
    for A, B in zip(As, Bs):
        packs.append(PackedMatrix.from_dense(torch.from_numpy(A).to(dev), m, k_tile=args.k_tile, value_dtype=vd))
        Bd.append(torch.from_numpy(B).to(dev).to(tdt))
        Cd.append(torch.empty((args.m, args.n), device=dev))
    torch.cuda.synchronize()
    bsz = 4 if args.dtype == "f32" else 2
    bytes_per = [p.algorithmic_bytes(args.n, b_bytes=bsz) for p in packs]
    flops_per = [p.flops(args.n) for p in packs]
    step_bytes, step_flops = sum(bytes_per), sum(flops_per)
    working_set = step_bytes

    # parity spot check of replica 0 against the oracle before timing anything
    ref0 = O.Packed(O.Tables.of(m), As[0], k_tile=args.k_tile, value_dtype=spreg_dtype)
    got0 = packs[0].execute(Bd[0], Cd[0], nr=args.nr, staging=args.staging, meta=args.meta).cpu().numpy()
    B0ref = Bs[0] if args.dtype == "f32" else Bd[0].cpu().view(torch.int16).numpy().view(np.uint16)
    parity_ok = bool(np.array_equal(got0.view(np.uint32), ref0.execute(B0ref).view(np.uint32)))

    stream = torch.cuda.current_stream()
    from spreg.packed import execute_batched
    work = [(p, B, C, dict(nr=args.nr, meta=args.meta, staging=args.staging)) for p, B, C in zip(packs, Bd, Cd)]

    def step():
        if args.batched:
            execute_batched(work)  # all replicas in one launch of the persistent kernel
        else:
            for p, B, C in zip(packs, Bd, Cd):
                p.execute(B, C, nr=args.nr, staging=args.staging, meta=args.meta)

    launches_per_step = 1 if args.batched else len(packs)
    graph = None
    if not args.no_graph:
        try:
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                step()
            torch.cuda.current_stream().wait_stream(s)
            torch.cuda.synchronize()
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                step()
            torch.cuda.synchronize()
        except Exception as e:  # capture unsupported: launch directly
            print(f"graph capture failed ({e}); timing direct launches", file=sys.stderr)
            graph = None

    run = graph.replay if graph is not None else step
    with ClockSampler(dev.index) as clk:  # sampling starts before the warm-up steps
        for _ in range(max(args.warmup, 3)):
            run()
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        if args.path == "register":
            clk.mark_start()
        ev0.record(stream)
        for _ in range(args.steps):
            run()
        ev1.record(stream)
        torch.cuda.synchronize()
        if args.path == "register":
            clk.mark_end()
        peak, peak_kind = measured_peaks()
        hyb = None
        if args.path == "hybrid":
            if ws > 1:
                torch.distributed.barrier()
            hyb = hybrid_leg(args, As, Bs, m, dev, step_bytes, step_flops, clk, peak, peak_kind)
    ms_reg = max_over_ranks(ev0.elapsed_time(ev1), dev)  # replicas: the job takes as long as its slowest rank
    ms = max_over_ranks(hyb["ms"], dev) if hyb is not None else ms_reg
    if ws > 1:
        torch.distributed.barrier()
    sec = ms_reg / 1e3
    value = whole_job_rate(step_bytes, args.steps, ws, ms) / 1e9
    gflops = whole_job_rate(step_flops, args.steps, ws, ms) / 1e9
    ms_per_step = ms / args.steps
    value_reg = whole_job_rate(step_bytes, args.steps, ws, ms_reg) / 1e9
    gflops_reg = whole_job_rate(step_flops, args.steps, ws, ms_reg) / 1e9

    # roofline of the executor kernel (one launch per replica per step)
    launch_s = sec / (args.steps * launches_per_step)
    achieved = (step_bytes / launches_per_step) / launch_s / 1e9
    spmm_us = sec / (args.steps * len(packs)) * 1e6
    kname = ("exec_kernel" if args.meta == 2 else
             "exec_tile_kernel" if args.staging == 1 else "exec_batch_kernel")  # meta 2: register streams
    traffic_key = (f"{kname}/{args.dtype}/{args.m}x{args.k}/s{args.sparsity}/n{args.n}/kt{args.k_tile}/"
                   f"{'identity' if args.mapping == 'identity' else args.mapping}")
    traffic = load_traffic(traffic_key, len(packs) // launches_per_step)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{peak_kind} hbm_gbs", "traffic": traffic, "traffic_key": traffic_key,
                "kernel": "spreg::%s<%d,NV,%s>" % (kname, args.mr, "float,float,float" if args.dtype == "f32" else
                                                    "bf16,bf16,float"),
                "spmm_us": spmm_us, "launches_per_step": launches_per_step,
                "algorithmic_bytes_per_launch": step_bytes / launches_per_step,
                "flops_per_launch": step_flops / launches_per_step, "gflops": gflops_reg,
                "launch_us": launch_s * 1e6}

    # e2e through the host-buffer C ABI (MatMulSpecialized operator()(C, B))
    e2e_n = 0 if (args.no_e2e or args.dtype != "f32") else len(As)
    mms, Bh, Ch = [], [], []
    for A, B in zip(As[:e2e_n], Bs[:e2e_n]):
        rp, ci, v = synth.to_csr(A)
        mms.append(MatMulSpecialized(args.m, args.k, args.n, v, rp, ci, TileConfig(K_c=args.k_tile, nr=args.nr), 1, "",
                                     m))
        Bh.append(torch.from_numpy(B).pin_memory())
        Ch.append(torch.empty((args.m, args.n), dtype=torch.float32).pin_memory())
    for mm, B, C in zip(mms, Bh, Ch):
        mm(C, B)
    e2e_ok = bool(np.array_equal(Ch[0].numpy(), ref0.execute(Bs[0]))) if (parity_ok and e2e_n) else False
    e2e_steps = max(2, args.steps // 4)

    def e2e_step_async():
        for mm, B, C in zip(mms, Bh, Ch):  # every matmul's copy in, product and copy out on its own stream
            mm.run_async(C, B)
        for mm in mms:
            mm.sync()

    def e2e_step_sync():
        for mm, B, C in zip(mms, Bh, Ch):
            mm(C, B)

    def timed_e2e(step_fn):
        step_fn()
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            step_fn()
        return max_over_ranks((time.perf_counter() - t0) * 1e3, dev)

    e2e_ms = timed_e2e(e2e_step_async)
    e2e_ok = e2e_ok and bool(np.array_equal(Ch[0].numpy(), ref0.execute(Bs[0]))) if e2e_n else False
    # every replica's host result equals its device-resident result of the timed steps, bit for bit
    e2e_all = bool(e2e_n) and all(torch.equal(Ch[i], Cd[i].cpu()) for i in range(e2e_n))
    e2e_sync_ms = timed_e2e(e2e_step_sync)
    rate = (lambda ms_: whole_job_rate(sum(bytes_per[:e2e_n]), e2e_steps, ws, ms_) / 1e9) if e2e_n else (lambda ms_: None)
    e2e = {"value": rate(e2e_ms), "unit": UNIT, "synchronous_calls_value": rate(e2e_sync_ms),
           "h2d_bytes_per_step": e2e_n * args.k * args.n * 4, "d2h_bytes_per_step": e2e_n * args.m * args.n * 4,
           "path": "spreg_matmul_run_async per replica (host B copied in, C = A.B stored by the kernel straight "
                   "into the pinned host C, on the matmul's own stream), then spreg_matmul_sync of every replica; "
                   "synchronous_calls_value: spreg_matmul_run per replica",
           "replicas_per_step": e2e_n,
           "bit_exact_vs_oracle": e2e_ok, "all_replicas_equal_device_results": e2e_all}
    del mms

    # the secondary legs describe one GPU: rank 0 alone runs them, the other ranks are done
    lead = rank == 0
    csr_leg = (csr_baseline_leg(As[0], Bd[0], packs[0], args, spmm_us)
               if (lead and args.dtype == "f32" and args.extras) else None)
    cfg1 = config1_leg(dev) if (lead and args.extras) else None
    lbal = load_balance_leg(dev) if (lead and args.extras) else None
    sparse_end = sparse_end_leg(dev) if (lead and args.extras) else None
    serving = serving_bench(args, dev) if (lead and args.serving) else None
    precision = (precision_suite(dev, args.precision_only, args.precision_configs)
                 if (lead and args.precision) else None)
    tensor_cores = tensor_core_suite(dev) if (lead and args.tensor_cores) else None
    layers = layers_suite(dev) if (lead and args.layers) else None
    sweep = ffn_sweep(dev) if (lead and args.ffn_sweep) else None

    cpu = None
    if rank == 0 and args.cpu_seconds > 0:
        cpu = cpu_baseline(As, Bs, args, args.cpu_seconds, mapping=m)
        cpu["protocol"] = cpu_baselines(As, Bs, args, m)

    clocks = clk.summary()
    if args.staging == 1:
        roofline["smem"] = smem_roofline(packs, args.n, bsz, args.k_tile, spmm_us / 1e6, clocks.get("sm_mhz"))
    if rank == 0:
        reg = {"value": value_reg, "unit": UNIT, "gflops": gflops_reg, "ms_per_step": ms_reg / args.steps,
               "roofline": roofline, "parity_bit_exact_vs_oracle": parity_ok,
               "nr": args.nr or "auto", "b_staging": {0: "auto", 1: "shared-memory B tiles", 2: "L1/L2"}[args.staging],
               "cuda_graph": graph is not None, "batched_launch": bool(args.batched),
               "launches_per_step": launches_per_step}
        cfg = workload_config(args, m, working_set) | {"parallelism": f"replicas x{ws}"}
        if hyb is not None:
            path = ("FP32-accurate hybrid: panels with fill >= %g as split-FP16 tcgen05 products (hi.hi + hi.lo + "
                    "lo.hi, FP32 accumulation; rel err <= 1e-5 vs the reference executor and FP64), the rest "
                    "register-tiled" % hyb["tc_fill"])
            launches = hyb["launches_per_step"] * args.steps
            head_roof = hyb.pop("roofline")
            head_roof["traffic"] = load_traffic(f"tc_rows_kernel_split/f32/{args.m}x{args.k}/n{args.n}", len(packs))
            parity = hyb["within_tolerance"]
        else:
            path = "register-tiled executor (bit-exact with the reference executor's FMA order)"
            launches = launches_per_step * args.steps
            head_roof = roofline
            parity = parity_ok
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded row-skew sparse A, N(0,1) B)",
                "config": cfg, "path": path,
                "gflops": gflops, "roofline": head_roof, "hybrid": hyb, "bit_exact_register_tiled": reg,
                "cpu_baseline": cpu, "e2e": e2e, "serving": serving,
                "precision": precision, "batched_layers": layers, "tensor_cores": tensor_cores,
                "ffn_sparsity_sweep": sweep, "gpu_csr_baseline": csr_leg, "config1_minimum_slice": cfg1,
                "load_balanced_single_spmm": lbal, "sparse_end_kernels": sparse_end,
                "clocks": clocks, "gpu_launches": launches,
                "parity": parity}
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
