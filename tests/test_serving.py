"""Serving loop: host-side policy on the CPU, the device loop on the GPU.

The GPU tests check that a request's output is the same alone and in a continuous batch (bit for
bit: every output element is one FP32 fma chain in packed order, whatever else shares the launch),
that BF16 storage stays within rel err 1e-2 of the FP64 stack and FP32 storage within 1e-5, and
that admission respects the activation-memory budget.
"""
import numpy as np
import pytest

from spreg import synth
from spreg.serving import (ActivationArena, Request, Scheduler, mlp_reference_fp64, mlp_weights, nr_for_tokens,
                           round_up)

BF16_TOL = 1e-2
FP32_TOL = 1e-5


def rel_err(got, ref):
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.linalg.norm(np.asarray(got, dtype=np.float64) - ref) / max(np.linalg.norm(ref), 1e-300))


# ---------------------------------------------------------------------------- arena
def test_arena_alloc_free_coalesce():
    a = ActivationArena(4096, align=256)
    x = a.alloc(100)
    y = a.alloc(256)
    z = a.alloc(1000)
    assert (x, y, z) == (0, 256, 512)
    assert a.used == 256 + 256 + 1024
    a.free(y)
    assert a.alloc(300) == 1536  # first fit: the 256-byte hole is too small
    a.free(x)
    assert a.free_list[0] == [0, 512]  # x and y's ranges merged
    a.free(z)
    a.free(1536)
    assert a.free_list == [[0, 4096]] and a.used == 0
    assert a.peak == 256 + 1024 + 512  # x, z and the 512-byte block, after y was freed


def test_arena_full_and_exact_fit():
    a = ActivationArena(1024, align=256)
    offs = [a.alloc(256) for _ in range(4)]
    assert offs == [0, 256, 512, 768]
    assert a.alloc(1) is None
    a.free(512)
    assert a.alloc(256) == 512
    assert a.largest_free() == 0


def test_arena_random_ops_never_overlap():
    g = np.random.default_rng(3)
    a = ActivationArena(1 << 20, align=256)
    live = {}
    for _ in range(3000):
        if live and g.random() < 0.45:
            off = list(live)[g.integers(len(live))]
            a.free(off)
            del live[off]
        else:
            n = int(g.integers(1, 40000))
            off = a.alloc(n)
            if off is None:
                assert a.largest_free() < round_up(n, 256)
                continue
            assert off % 256 == 0 and off + n <= a.capacity
            for o, m in live.items():
                assert off + n <= o or o + m <= off
            live[off] = n
        assert a.used == sum(round_up(v, 256) for v in live.values())
    for off in list(live):
        a.free(off)
    assert a.free_list == [[0, 1 << 20]]


# ---------------------------------------------------------------------------- scheduler
def _sched(layers=4, capacity=10_000, slots=3):
    return Scheduler(layers, lambda r: r.n * 100, ActivationArena(capacity, align=100), slots)


def test_scheduler_slots_and_fcfs_budget():
    s = _sched(capacity=1000, slots=3)
    reqs = [Request(i, n) for i, n in enumerate([3, 3, 5, 1, 1])]
    for r in reqs:
        s.submit(r)
    got = s.admit()
    assert [r.rid for r in got] == [0, 1]  # request 2 (500 B) does not fit in the 400 B left
    assert [r.rid for r in s.queue] == [2, 3, 4]  # 3 and 4 would fit but do not overtake 2
    with pytest.raises(ValueError):
        s.submit(Request(9, 11))  # larger than the whole budget


def test_scheduler_layers_run_once_in_order():
    L = 5
    s = _sched(layers=L, capacity=100_000, slots=4)
    reqs = [Request(i, 1 + i % 3) for i in range(9)]
    runs = {r.rid: [] for r in reqs}
    pending = list(reqs)
    done = []
    it = 0
    while len(done) < len(reqs):
        if pending and it % 2 == 0:
            s.submit(pending.pop(0))
        s.admit()
        for r in s.next_iteration():
            runs[r.rid].append(r.layer - 1)
        assert s.slots_in_use() <= 4
        for r in list(s.draining):
            s.release(r)
            done.append(r.rid)
        it += 1
    assert sorted(done) == list(range(9))
    for rid, layers in runs.items():
        assert layers == list(range(L)), rid
    assert s.idle() and s.arena.used == 0


def test_continuous_batch_simulation_matches_fp64_stack():
    """The host loop's layer order applied in FP64 gives the stack's result for every request."""
    w = mlp_weights(16, 48, 3, 0.7, seed=5, bf16_values=False)
    layers = [m for blk in w for m in blk]
    g = np.random.default_rng(0)
    reqs = [Request(i, int(n), x=g.standard_normal((16, int(n)))) for i, n in enumerate([1, 5, 2, 9, 3, 4])]
    state = {}
    s = Scheduler(len(layers), lambda r: r.n * 64, ActivationArena(1600, align=64), 3)
    for r in reqs:
        s.submit(r)
    finished = {}
    while len(finished) < len(reqs):
        for r in s.admit():
            state[r.rid] = [r.x.astype(np.float64), None]
        for r in s.next_iteration():
            l = r.layer - 1
            x, h = state[r.rid]
            if l % 2 == 0:
                state[r.rid][1] = np.maximum(layers[l].astype(np.float64) @ x, 0.0)
            else:
                state[r.rid][0] = x + layers[l].astype(np.float64) @ h
        for r in list(s.draining):
            finished[r.rid] = state[r.rid][0]
            s.release(r)
    for r in reqs:
        np.testing.assert_allclose(finished[r.rid], mlp_reference_fp64(w, r.x), rtol=1e-12, atol=1e-12)


def test_request_generators():
    n = synth.token_counts(5000, median=64, sigma=1.0, seed=1)
    assert n.min() >= 1 and n.max() <= 2048
    assert 50 <= np.median(n) <= 80
    t = synth.poisson_arrivals(20000, 1000.0, seed=2)
    assert np.all(np.diff(t) >= 0)
    assert abs(len(t) / t[-1] - 1000.0) < 50
    assert np.all(synth.poisson_arrivals(4, float("inf")) == 0)
    assert [nr_for_tokens(k) for k in (1, 63, 64, 127, 128, 2048)] == [32, 32, 64, 64, 128, 128]


def test_round_bf16_matches_torch():
    torch = pytest.importorskip("torch")
    a = (np.random.default_rng(1).standard_normal(50000) * 3).astype(np.float32)
    a[:4] = [0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8]  # ties to even
    np.testing.assert_array_equal(synth.round_bf16(a), torch.from_numpy(a).to(torch.bfloat16).float().numpy())


# ---------------------------------------------------------------------------- GPU
def _model_and_requests(dtype, ns, seed=7, d_model=128, d_ff=512, blocks=3):
    from spreg.serving import SparseMLP, prepare_requests
    w = mlp_weights(d_model, d_ff, blocks, 0.9, seed=seed)
    model = SparseMLP(w, dtype=dtype)
    g = np.random.default_rng(seed)
    reqs = [Request(i, int(n), x=synth.round_bf16(g.standard_normal((d_model, int(n))).astype(np.float32)))
            for i, n in enumerate(ns)]
    prepare_requests(model, reqs)
    return w, model, reqs


@pytest.mark.gpu
def test_serving_alone_equals_mix_bf16(cuda):
    from spreg.serving import Server, output_fp32, prepare_requests
    ns = [1, 7, 64, 130, 300, 33, 5, 257]
    w, model, reqs = _model_and_requests("bf16", ns)
    for i, r in enumerate(reqs):
        r.arrival = float(i % 4)  # joins a batch already in flight
    srv = Server(model, budget_bytes=64 << 20, max_slots=16)
    st = srv.run(reqs, realtime=False)
    assert st.requests == len(ns) and st.max_batch > 1
    mix = [output_fp32(r).copy() for r in reqs]
    for r, out in zip(reqs, mix):
        alone = Request(100 + r.rid, r.n, x=r.x)
        prepare_requests(model, [alone])
        Server(model, budget_bytes=8 << 20, max_slots=1).run([alone], realtime=False)
        np.testing.assert_array_equal(output_fp32(alone), out)
        assert rel_err(out, mlp_reference_fp64(w, r.x)) <= BF16_TOL


@pytest.mark.gpu
def test_serving_fp32_matches_per_request_path(cuda):
    from spreg.serving import Server, output_fp32, serve_per_request
    ns = [3, 64, 200]
    w, model, reqs = _model_and_requests("f32", ns)
    Server(model, budget_bytes=16 << 20, max_slots=8).run(reqs, realtime=False)
    batched = [output_fp32(r).copy() for r in reqs]
    serve_per_request(model, reqs, realtime=False)
    for r, out in zip(reqs, batched):
        np.testing.assert_array_equal(output_fp32(r), out)
        assert rel_err(out, mlp_reference_fp64(w, r.x)) <= FP32_TOL


@pytest.mark.gpu
def test_serving_budget_limits_admission(cuda):
    from spreg.serving import Server, output_fp32
    ns = [512, 512, 512, 64, 8]
    w, model, reqs = _model_and_requests("bf16", ns)
    budget = model.act_bytes(512) * 2  # two of the large requests at a time
    srv = Server(model, budget_bytes=budget, max_slots=16)
    st = srv.run(reqs, realtime=False)
    assert st.peak_activation_bytes <= budget
    assert reqs[2].first_iteration > 0  # the third 512-token request waited for memory
    # first come, first served: the small requests did not overtake it
    assert reqs[3].first_iteration >= reqs[2].first_iteration and reqs[4].first_iteration >= reqs[2].first_iteration
    for r in reqs:
        assert rel_err(output_fp32(r), mlp_reference_fp64(w, r.x)) <= BF16_TOL


@pytest.mark.gpu
def test_serving_realtime_poisson(cuda):
    from spreg.serving import Server, serve_per_request
    ns = synth.token_counts(40, median=32, sigma=1.0, hi=256, seed=3)
    w, model, reqs = _model_and_requests("bf16", ns)
    for r, t in zip(reqs, synth.poisson_arrivals(len(reqs), 2000.0, seed=4)):
        r.arrival = float(t)
    st = Server(model, budget_bytes=64 << 20, max_slots=32).run(reqs)
    assert st.requests == 40 and st.p99_ms >= st.p50_ms > 0 and st.req_per_s > 0
    assert all(r.t_done >= r.t_admit >= r.arrival for r in reqs)
    st2 = serve_per_request(model, reqs)
    assert st2.requests == 40 and all(r.t_done >= r.arrival for r in reqs)


@pytest.mark.gpu
def test_serving_tiled_mixed_configs(cuda):
    """Per-layer packings (M_r 2/8, K tiles, a non-identity mapping) keep alone == mix and the
    FP64 tolerance."""
    from spreg.serving import Server, SparseMLP, output_fp32, prepare_requests
    w = mlp_weights(64, 1024, 2, 0.9, seed=11)
    cfg = [{"mr": 2, "mapping": "identity", "k_tile": 0}, {"mr": 2, "mapping": "identity", "k_tile": 512},
           {"mr": 8, "mapping": "400fa", "k_tile": 0}, {"mr": 4, "mapping": "identity", "k_tile": 256}]
    model = SparseMLP(w, "bf16", configs=cfg)
    g = np.random.default_rng(2)
    ns = [5, 70, 129, 1]
    reqs = [Request(i, n, x=synth.round_bf16(g.standard_normal((64, n)).astype(np.float32)), arrival=float(i))
            for i, n in enumerate(ns)]
    prepare_requests(model, reqs)
    Server(model, budget_bytes=32 << 20, max_slots=8).run(reqs, realtime=False)
    for r in reqs:
        alone = Request(50 + r.rid, r.n, x=r.x)
        prepare_requests(model, [alone])
        Server(model, budget_bytes=8 << 20, max_slots=1).run([alone], realtime=False)
        np.testing.assert_array_equal(output_fp32(alone), output_fp32(r))
        assert rel_err(output_fp32(r), mlp_reference_fp64(w, r.x)) <= BF16_TOL


@pytest.mark.gpu
def test_serving_tensor_core_layers(cuda):
    """Tensor-core layers (every panel dense BF16 on tcgen05): alone == mix bit for bit, the FP64
    tolerance, and the per-request path gives the same outputs."""
    from spreg.serving import Server, SparseMLP, output_fp32, prepare_requests, serve_per_request
    w = mlp_weights(128, 512, 2, 0.9, seed=13)
    model = SparseMLP(w, "bf16", tc=True)
    g = np.random.default_rng(4)
    ns = [3, 64, 130, 1, 257]
    reqs = [Request(i, n, x=synth.round_bf16(g.standard_normal((128, n)).astype(np.float32)), arrival=float(i % 3))
            for i, n in enumerate(ns)]
    prepare_requests(model, reqs)
    Server(model, budget_bytes=32 << 20, max_slots=8).run(reqs, realtime=False)
    mix = [output_fp32(r).copy() for r in reqs]
    for r, out in zip(reqs, mix):
        assert rel_err(out, mlp_reference_fp64(w, r.x)) <= BF16_TOL
        alone = Request(50 + r.rid, r.n, x=r.x)
        prepare_requests(model, [alone])
        Server(model, budget_bytes=8 << 20, max_slots=1).run([alone], realtime=False)
        np.testing.assert_array_equal(output_fp32(alone), out)
    serve_per_request(model, reqs, realtime=False)
    for r, out in zip(reqs, mix):
        np.testing.assert_array_equal(output_fp32(r), out)
