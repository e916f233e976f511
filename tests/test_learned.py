"""Learned conjunct ordering: MLP oracle, GPU gradients, and learned-path parity.

The learner must return exactly what the plain fixed-order two-pass evaluator
returns for every batch (same rows, order, values and validity), whatever the
network predicts; its network's forward/backward kernels must match the float64
oracle; and the trained network must choose better conjunct orders than the
textual order it replaces.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from blazingsql_gb300 import workloads as W
from blazingsql_gb300.types import TypeId as T
from oracle import mlp_ref

from helpers import assert_tables_equal


# ------------------------------------------------------------------ CPU
def test_mlp_oracle_matches_finite_differences():
    rng = np.random.default_rng(7)
    F, H, O, M = 11, 8, 3, 5
    p = rng.normal(0, 0.5, mlp_ref.param_count(F, H, O))
    X = rng.random((M, F))
    Y = np.log(rng.random((M, O)) * 0.9 + 1e-3)
    g, L, _ = mlp_ref.grad(p, X, Y, F, H, O)
    assert L == pytest.approx(mlp_ref.loss(p, X, Y, F, H, O))
    idx = np.arange(0, len(p), 3)
    fd = mlp_ref.finite_difference(p, X, Y, F, H, O, idx)
    np.testing.assert_allclose(g[idx], fd, rtol=1e-5, atol=1e-8)


def test_word_loads_counts_short_circuit():
    keep_a = np.zeros(64, dtype=bool)
    keep_a[3] = True          # word 0 survives conjunct a, word 1 dies
    keep_b = np.ones(64, dtype=bool)
    assert mlp_ref.word_loads([1, 1], [keep_a, keep_b], [0, 1]) == 2 + 1
    assert mlp_ref.word_loads([1, 1], [keep_a, keep_b], [1, 0]) == 2 + 2


def test_c4_generator_selectivity_ranges():
    """Per-batch selectivities of the six conjuncts spread over about 0.1%..90%."""
    sels = []
    for b in range(24):
        x = [c.data for c in W.c4_batch_host(1 << 16, 4, b)]
        sels.append([(x[0] > 100000).mean(), (x[1] == 1000).mean(), (x[2] < 1000).mean(),
                     (x[4] < 1000.0).mean(), (x[5] > 5000.0).mean(), (x[6] < 100.0).mean()])
    s = np.array(sels)
    assert s.min() < 0.01 and s.max() > 0.85
    # the most selective conjunct changes between batches
    assert len(set(np.argmin(s, axis=1))) >= 2


def test_learner_kernels_compile():
    """NVRTC compiles the learner's two kernel variants for sm_103a (no GPU)."""
    import blazingsql_gb300 as g
    plan = g.Plan(W.workload("c4").schema, W.C4_CONDITION, W.C4_PROJECTIONS, nullable=[False] * 8)
    assert plan.num_conjuncts == 6
    src = plan.kernel_source(4, [False] * 8)
    assert "a.order_dev + j_" in src and "a.order[j_]" in src
    assert "s_conj" in plan.kernel_source(5, [False] * 8)
    plan.compile_check(4, [False] * 8)
    plan.compile_check(5, [False] * 8)


# ------------------------------------------------------------------ GPU
def _upload(cols):
    from blazingsql_gb300.api import DeviceColumn
    return [DeviceColumn.from_host(c) for c in cols]


def _host(cols):
    return [c.to_host() for c in cols]


def _c4_plan(g):
    return g.Plan(W.workload("c4").schema, W.C4_CONDITION, W.C4_PROJECTIONS, nullable=[False] * 8)


@pytest.mark.gpu
def test_mlp_gradients_match_oracle():
    import blazingsql_gb300 as g
    rng = np.random.default_rng(11)
    for F, H, O, M in [(88, 64, 6, 64), (11, 16, 3, 7), (33, 64, 16, 1)]:
        p = rng.normal(0, 0.3, mlp_ref.param_count(F, H, O)).astype(np.float32)
        X = rng.random((M, F)).astype(np.float32)
        Y = np.log(rng.random((M, O)) + 1e-6).astype(np.float32)
        grad, loss, z = g.api.mlp_grad(F, H, O, p, X, Y)
        eg, eloss, ez = mlp_ref.grad(p.astype(np.float64), X, Y, F, H, O)
        np.testing.assert_allclose(z, ez, rtol=1e-4, atol=1e-4 * max(1.0, np.abs(ez).max()))
        assert loss == pytest.approx(eloss, rel=1e-4)
        np.testing.assert_allclose(grad, eg, rtol=1e-3, atol=1e-4 * np.abs(eg).max())


@pytest.mark.gpu
def test_sketch_features_match_oracle():
    """The sketch kernels against the oracle's sketch, with the anchors taken
    from the condition's constants; nulls and a column offset included."""
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    plan = _c4_plan(g)
    lr = g.Learner(plan, sketch_stride_words=4)
    for b, n in ((0, 1 << 16), (1, 40_000 + 17)):
        host = W.c4_batch_host(n, 9, b)
        f, anchors = lr.features(_upload(host))
        np.testing.assert_array_equal(anchors, [100000, 1000, 1000, 0, 1000.0, 5000.0, 100.0, 0])
        exp = mlp_ref.sketch_features([c.data for c in host], [None] * 8, anchors, 4)
        np.testing.assert_allclose(f, exp, rtol=1e-5, atol=1e-6)
    # nullable columns with an offset: INT32 / FLOAT64 with 20% nulls
    other = g.Plan([T.INT32, T.FLOAT64], "AND(>($0, 10), <=($1, -2.5))", ["$0", "$1"])
    lr2 = g.Learner(other, sketch_stride_words=2)
    rng = np.random.default_rng(3)
    n, off = 50_000, 37
    x0 = rng.integers(-100, 100, n + off).astype(np.int32)
    x1 = rng.normal(0, 10, n + off)
    v0 = rng.random(n + off) > 0.2
    v1 = rng.random(n + off) > 0.2
    cols = [g.HostColumn(T.INT32, x0, g.pack_validity(v0)), g.HostColumn(T.FLOAT64, x1, g.pack_validity(v1))]
    dev = [DeviceColumn.from_host(c) for c in cols]
    for d in dev:
        d.offset, d.size = off, n
    f, anchors = lr2.features(dev)
    np.testing.assert_array_equal(anchors, [10, -2.5])
    exp = mlp_ref.sketch_features([x0[off:], x1[off:]], [v0[off:], v1[off:]], anchors, 2)
    np.testing.assert_allclose(f, exp, rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("size_outputs", [1, 0])
def test_learned_matches_plain_and_oracle(size_outputs):
    """Warm-up, learned single-pass and relabel batches all return the plain
    path's output; a few batches are also checked against the CPU oracle.  With
    size_outputs=0 the kernel takes the order from device memory."""
    import blazingsql_gb300 as g
    from helpers import OracleEngine
    plan = _c4_plan(g)
    learned = g.Learner(plan, warmup_batches=4, relabel_every=5, train_steps=32, size_outputs=size_outputs,
                        fast_words_per_warp=8)
    plain = g.Learner(plan, policy=g.GX_LEARN_POLICY_PLAIN)
    oracle = OracleEngine(nthreads=4)
    paths = set()
    for b in range(14):
        host = W.c4_batch_host(1 << 16, 4, b)
        dev = _upload(host)
        got, rows, info = learned.execute(dev)
        exp, erows, _ = plain.execute(dev)
        assert rows == erows == info["rows"]
        assert_tables_equal(_host(got), _host(exp), what=f"batch {b} path {info['path']}")
        paths.add(info["path"])
        if b in (0, 6, 13):
            ref = oracle.filter_project(host, W.C4_CONDITION, W.C4_PROJECTIONS)
            assert_tables_equal(_host(got), ref, what=f"oracle batch {b}")
        if info["path"] == 1:
            assert sorted(info["order"]) == list(range(6))
    assert paths == {0, 1}


@pytest.mark.gpu
@pytest.mark.parametrize("offset,variant", [(0, "GX_STAGED"), (1, "GX_STAGED"), (2, "GX_STAGED"), (33, "GX_STAGED"),
                                            (0, "GX_STREAM"), (33, "GX_STREAM")])
def test_staged_single_pass_matches_plain(offset, variant, monkeypatch):
    """The single-pass variants a learner can be asked for return the plain
    path's rows: shared-memory staging of the conjunct columns (GX_STAGED=1,
    used when the columns start on 16-byte boundaries; offset 1 or 33 of an
    8-byte column runs the unstaged kernel) and streaming word slots
    (GX_STREAM=8); ragged sizes, nulls and a column offset included."""
    import blazingsql_gb300 as g
    from blazingsql_gb300.api import DeviceColumn
    rng = np.random.default_rng(21 + offset)
    schema = [T.INT64, T.FLOAT64, T.INT32, T.INT64]
    cond = "AND(>($0, 500), <($1, 0.25), =(MOD($2, 3), 1), IS NOT NULL($3))"
    plan = g.Plan(schema, cond, ["$0", "$1", "$2", "+($3, 1)"], words_per_warp=8)
    monkeypatch.setenv(variant, "1" if variant == "GX_STAGED" else "8")
    textual = g.Learner(plan, policy=g.GX_LEARN_POLICY_TEXTUAL, fast_words_per_warp=8)
    learned = g.Learner(plan, warmup_batches=2, relabel_every=0, size_outputs=0, fast_words_per_warp=8)
    monkeypatch.delenv(variant)
    plain = g.Learner(plan, policy=g.GX_LEARN_POLICY_PLAIN)
    for n in (1, 31, 33, 1000, 1023, 1024 * 9 + 17, 100_000):
        total = n + offset
        x0 = rng.integers(0, 1000, total).astype(np.int64)
        x1 = rng.random(total)
        x2 = rng.integers(-50, 50, total).astype(np.int32)
        x3 = rng.integers(0, 10, total).astype(np.int64)
        v2 = rng.random(total) > 0.1
        v3 = rng.random(total) > 0.2
        cols = [g.HostColumn(T.INT64, x0), g.HostColumn(T.FLOAT64, x1),
                g.HostColumn(T.INT32, x2, g.pack_validity(v2)), g.HostColumn(T.INT64, x3, g.pack_validity(v3))]
        dev = [DeviceColumn.from_host(c) for c in cols]
        for d in dev:
            d.offset, d.size = offset, n
        exp, erows, _ = plain.execute(dev)
        for b in range(3):  # learned: two labelled batches, then single passes
            got, rows, info = learned.execute(dev)
            assert rows == erows
            assert_tables_equal(_host(got), _host(exp), what=f"learned n={n} off={offset} batch {b}")
        got, rows, _ = textual.execute(dev)
        assert rows == erows
        assert_tables_equal(_host(got), _host(exp), what=f"textual n={n} off={offset}")


@pytest.mark.gpu
@pytest.mark.parametrize("size_outputs", [0, 1])
def test_look_ahead_prepare(size_outputs):
    """Batches prepared one step ahead give the same rows as the plain path and
    the same order as computing the prediction in the call; a prepared batch
    that never comes and a batch that was not prepared both still work."""
    import blazingsql_gb300 as g
    plan = _c4_plan(g)
    kw = dict(warmup_batches=3, relabel_every=4, train_steps=8, size_outputs=size_outputs)
    ahead = g.Learner(plan, **kw)
    plain = g.Learner(plan, policy=g.GX_LEARN_POLICY_PLAIN)
    batches = [_upload(W.c4_batch_host(1 << 15, 12, b)) for b in range(10)]
    ahead.prepare(batches[0])
    for b in range(10):
        if b + 1 < 10 and b != 5:  # batch 6 is not prepared
            ahead.prepare(batches[b + 1])
        if b == 7:
            ahead.prepare(batches[2])  # prepared, never executed again
        got, rows, info = ahead.execute(batches[b])
        exp, erows, _ = plain.execute(batches[b])
        assert rows == erows
        assert_tables_equal(_host(got), _host(exp), what=f"batch {b}")
        if info["path"] == 1:
            assert sorted(info["order"]) == list(range(6))


@pytest.mark.gpu
@pytest.mark.parametrize("policy,size_outputs", [("learned", 0), ("learned", 1), ("textual", 0)])
def test_execute_batches_queue(policy, size_outputs):
    """A queue of batches in one call (ragged and empty batches included) gives
    each batch exactly the plain path's output, with the prediction reported
    for the single-pass batches; an invalid batch is named in the error.  With
    full-size outputs (size_outputs=0, or the textual policy) the queue runs
    with one synchronisation at the end."""
    import blazingsql_gb300 as g
    from blazingsql_gb300 import _native as N
    plan = _c4_plan(g)
    sizes = [1 << 15, 1 << 15, 1 << 15, 0, 4097, 1 << 15, 31, 1 << 15, 1 << 14, 1 << 15]
    batches = [_upload(W.c4_batch_host(n, 21, b)) for b, n in enumerate(sizes)]
    pol = g.GX_LEARN_POLICY_LEARNED if policy == "learned" else g.GX_LEARN_POLICY_TEXTUAL
    learned = g.Learner(plan, policy=pol, warmup_batches=3, relabel_every=4, train_steps=8,
                        size_outputs=size_outputs)
    plain = g.Learner(plan, policy=g.GX_LEARN_POLICY_PLAIN)
    out = learned.execute_batches(batches)
    assert len(out) == len(batches)
    for b, (got, rows, info) in enumerate(out):
        exp, erows, _ = plain.execute(batches[b])
        assert rows == erows, f"batch {b}"
        assert_tables_equal(_host(got), _host(exp), what=f"batch {b}")
        assert info["rows"] == rows
        if info["path"] == 1:
            assert sorted(info["order"]) == list(range(6))
            if policy == "learned":
                assert all(0.0 < p < 1.0 for p in info["predicted_sel"])
        elif sizes[b] > 0:
            assert max(info["measured_sel"]) > 0.0
    assert any(info["path"] == 1 for _, _, info in out)
    assert learned.execute_batches([]) == []
    from blazingsql_gb300.api import DeviceColumn
    from blazingsql_gb300.types import HostColumn
    wrong = list(batches[4])
    wrong[0] = DeviceColumn.from_host(HostColumn(T.INT32, np.zeros(4097, dtype=np.int32)))
    with pytest.raises(N.GxError, match="batch 3"):  # column 0 of batch 3 has the wrong type
        learned.execute_batches(list(batches[:3]) + [wrong])


@pytest.mark.gpu
def test_learned_misprediction_reruns():
    """With no capacity margin the predicted output size is often too small; the
    single pass re-runs with the exact count and the result still matches."""
    import blazingsql_gb300 as g
    plan = _c4_plan(g)
    learned = g.Learner(plan, warmup_batches=2, relabel_every=0, train_steps=4, capacity_margin=1.0,
                        capacity_slack=0)
    plain = g.Learner(plan, policy=g.GX_LEARN_POLICY_PLAIN)
    reruns = 0
    for b in range(10):
        dev = _upload(W.c4_batch_host(1 << 15, 5, b))
        got, rows, info = learned.execute(dev)
        exp, erows, _ = plain.execute(dev)
        assert rows == erows
        assert_tables_equal(_host(got), _host(exp), what=f"batch {b}")
        reruns += info["reruns"]
    assert reruns > 0


@pytest.mark.gpu
def test_queued_sized_outputs_rerun_on_misprediction():
    """A queue with outputs sized from the predictions and no capacity margin:
    batches whose rows overflow their prediction run again after the queue,
    and every batch still equals the plain path; the outputs of the others
    hold no more rows than the prediction allowed."""
    import blazingsql_gb300 as g
    plan = _c4_plan(g)
    learned = g.Learner(plan, warmup_batches=2, relabel_every=0, train_steps=4, capacity_margin=1.0,
                        capacity_slack=0, size_outputs=1)
    plain = g.Learner(plan, policy=g.GX_LEARN_POLICY_PLAIN)
    batches = [_upload(W.c4_batch_host(1 << 15, 5, b)) for b in range(10)]
    out = learned.execute_batches(batches)
    reruns = 0
    for b, (got, rows, info) in enumerate(out):
        exp, erows, _ = plain.execute(batches[b])
        assert rows == erows, f"batch {b}"
        assert_tables_equal(_host(got), _host(exp), what=f"batch {b}")
        reruns += info["reruns"]
        if info["path"] == 1 and not info["reruns"]:
            assert got[0].capacity <= max(rows, info["predicted_rows"]) + 1
    assert reruns > 0


@pytest.mark.gpu
def test_labels_are_exact_conjunct_counts():
    """The labelled batches' measured selectivities are each conjunct's exact
    pass fraction over the batch (counted in the fused single pass), for a
    direct call and inside a queue."""
    import blazingsql_gb300 as g
    plan = _c4_plan(g)

    def expected(host):
        x = [c.data for c in host]
        keep = [x[0] > 100000, x[1] == 1000, x[2] < 1000, x[4] < 1000.0, x[5] > 5000.0, x[6] < 100.0]
        return [float(np.count_nonzero(k)) / len(k) for k in keep]

    hosts = [W.c4_batch_host((1 << 15) + 333 * b, 9, b) for b in range(3)]
    direct = g.Learner(plan, warmup_batches=3, relabel_every=0, train_steps=2)
    for h in hosts:
        _, _, info = direct.execute(_upload(h))
        assert info["path"] == 0
        np.testing.assert_array_equal(np.array(info["measured_sel"][:6]), np.array(expected(h)))
    queued = g.Learner(plan, warmup_batches=3, relabel_every=0, train_steps=2)
    for h, (_, _, info) in zip(hosts, queued.execute_batches([_upload(h) for h in hosts])):
        assert info["path"] == 0
        np.testing.assert_array_equal(np.array(info["measured_sel"][:6]), np.array(expected(h)))


@pytest.mark.gpu
def test_learner_policies_agree_and_async_training():
    import blazingsql_gb300 as g
    plan = _c4_plan(g)
    textual = g.Learner(plan, policy=g.GX_LEARN_POLICY_TEXTUAL)
    asyn = g.Learner(plan, warmup_batches=3, relabel_every=2, async_training=1)
    plain = g.Learner(plan, policy=g.GX_LEARN_POLICY_PLAIN)
    for b in range(8):
        dev = _upload(W.c4_batch_host((1 << 14) + 77 * b, 6, b))
        exp, erows, _ = plain.execute(dev)
        for lr in (textual, asyn):
            got, rows, _ = lr.execute(dev)
            assert rows == erows
            assert_tables_equal(_host(got), _host(exp), what=f"batch {b}")


@pytest.mark.gpu
def test_learner_save_load_and_empty_batch(tmp_path):
    import blazingsql_gb300 as g
    plan = _c4_plan(g)
    a = g.Learner(plan, warmup_batches=3, relabel_every=0, train_steps=8)
    for b in range(3):
        a.execute(_upload(W.c4_batch_host(1 << 14, 7, b)))
    path = os.path.join(str(tmp_path), "c4.gxml")
    a.save(path)
    b_ = g.Learner(plan, warmup_batches=3, relabel_every=0)
    b_.load(path)
    dev = _upload(W.c4_batch_host(1 << 14, 7, 9))
    ga, ra, ia = a.execute(dev)
    gb, rb, ib = b_.execute(dev)
    assert ia["path"] == ib["path"] == 1
    assert ia["order"] == ib["order"]
    np.testing.assert_allclose(ia["predicted_sel"], ib["predicted_sel"], rtol=1e-6)
    assert_tables_equal(_host(ga), _host(gb))
    # an empty batch: zero rows through the plain path
    empty = _upload([c for c in W.c4_batch_host(0, 7, 0)])
    cols, rows, info = a.execute(empty)
    assert rows == 0 and all(c.size == 0 for c in cols)
    other = g.Plan([T.INT64, T.INT64], "AND(>($0, 1), <($1, 5))", ["$0"])
    c = g.Learner(other)
    with pytest.raises(g.GxError):
        c.load(path)


@pytest.mark.gpu
def test_trained_network_beats_textual_order():
    """What the network gains over the method without it: over batches after
    warm-up, its conjunct orders read fewer 32-row column words (counted on the
    host from the batch's own pass vectors) than the textual order, come close
    to the per-batch best order, and take less measured kernel time than the
    textual order on the same (larger) batches."""
    import itertools
    import blazingsql_gb300 as g
    plan = _c4_plan(g)
    learned = g.Learner(plan, warmup_batches=12, relabel_every=0, train_steps=48)
    cost = [1] * 6
    totals = {"learned": 0, "textual": 0, "best": 0}
    for b in range(28):
        host = W.c4_batch_host(1 << 16, 8, b)
        _, _, info = learned.execute(_upload(host))
        if info["path"] != 1:
            continue
        x = [c.data for c in host]
        keep = [x[0] > 100000, x[1] == 1000, x[2] < 1000, x[4] < 1000.0, x[5] > 5000.0, x[6] < 100.0]
        totals["learned"] += mlp_ref.word_loads(cost, keep, info["order"])
        totals["textual"] += mlp_ref.word_loads(cost, keep, list(range(6)))
        totals["best"] += min(mlp_ref.word_loads(cost, keep, list(o)) for o in itertools.permutations(range(6)))
    assert totals["learned"] > 0
    assert totals["learned"] <= 0.9 * totals["textual"], totals
    assert totals["learned"] <= 1.15 * totals["best"], totals
    # the single-pass kernel's time (CUDA events around it) under each order,
    # on 4M-row batches: a learner trained on 8 of them (order from device
    # memory, full-size outputs: no re-runs) against the textual order on the
    # next 16
    from blazingsql_gb300 import _native as N
    L = N.lib()
    rows = 1 << 22
    timed = g.Learner(plan, warmup_batches=8, relabel_every=0, train_steps=48, size_outputs=0)
    for b in range(8):
        g.api.free_columns(timed.execute(W.c4_batch_device(rows, 8, b))[0])
    big = [W.c4_batch_device(rows, 8, b) for b in range(8, 24)]

    def kernel_ms(lr):
        for dev in big:  # compiles and warms
            g.api.free_columns(lr.execute(dev)[0])
        L.gx_debug_kernel_ms(1)
        L.gx_debug_set_kernel_timing(1)
        try:
            for _ in range(2):
                for dev in big:
                    cols, _, info = lr.execute(dev)
                    assert info["path"] == 1
                    g.api.free_columns(cols)
        finally:
            L.gx_debug_set_kernel_timing(0)
        return L.gx_debug_kernel_ms(1)

    t_learned = kernel_ms(timed)
    t_textual = kernel_ms(g.Learner(plan, policy=g.GX_LEARN_POLICY_TEXTUAL))
    assert 0 < t_learned <= t_textual, (t_learned, t_textual)
