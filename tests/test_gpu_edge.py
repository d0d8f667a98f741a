"""The learned absorbing edge on the GPU against its CPU oracle.

* forward pass and gradients of the networks (bf16 operands, FP32
  accumulation, the back-propagated errors rounded to bf16 as the oracle
  rounds them) against oracle/edge_ref.py, within tolerances that cover
  FP32 accumulation order and rare one-ulp bf16 rounding flips (measured:
  at most 7.4e-4 relative per weight block, 3.5e-4 per bias block over
  three seeds; a missing term would be of order one);
* an Adam step against the oracle's Adam on the oracle's gradient;
* a fresh edge (zero output layer) leaves a run bit-identical;
* training on a few small media lowers the reflected energy of a held-out
  medium well below that of the transparent strip without the network.
"""
import numpy as np
import pytest

from helpers import compare_state

pytestmark = pytest.mark.gpu


def _case(seed, n=700, scale=0.2):
    from oracle import edge_ref as R
    rng = np.random.default_rng(seed)
    params = (rng.standard_normal(R.SETS * R.SET_PARAMS) * scale).astype(np.float32)
    sets = rng.integers(0, R.SETS, n).astype(np.int32)
    x = rng.standard_normal((n, R.IN)).astype(np.float32)
    t = rng.standard_normal((n, R.OUT)).astype(np.float32)
    return params, sets, x, t


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def test_forward_matches_oracle():
    from fdporo.edge import Edge
    from oracle import edge_ref as R
    params, sets, x, _ = _case(1)
    e = Edge(seed=5)
    e.set_params(params)
    np.testing.assert_array_equal(e.params(), params)
    y = e.forward(sets, x)
    ref = R.forward(params, sets, x)
    assert _rel(y, ref) < 3e-4
    assert np.max(np.abs(y - ref)) < 3e-3 * np.max(np.abs(ref))


def test_gradients_match_oracle():
    from fdporo.edge import Edge
    from oracle import edge_ref as R
    params, sets, x, t = _case(2)
    e = Edge()
    e.set_params(params)
    g, loss = e.gradients(sets, x, t)
    gr, lr_ = R.gradients(params, sets, x, t)
    assert abs(loss - lr_) <= 1e-5 * lr_
    for s in range(R.SETS):
        for name, (o, m) in R.OFF.items():
            a = g[s * R.SET_PARAMS + o:s * R.SET_PARAMS + o + m]
            b = gr[s * R.SET_PARAMS + o:s * R.SET_PARAMS + o + m]
            assert _rel(a, b) < 3e-3, (s, name, _rel(a, b))


def test_adam_step_and_descent():
    from fdporo.edge import Edge
    from oracle import edge_ref as R
    params, sets, x, t = _case(3, n=400)
    e = Edge()
    e.set_params(params)
    gr, _ = R.gradients(params, sets, x, t)
    lr = 1e-3
    e.train_batch(sets, x, t, lr)
    want = R.Adam(params).step(gr, lr)
    d = np.abs(e.params() - want)
    # the first Adam step is about lr * sign(gradient): an element whose
    # gradient is near zero may differ in sign between the two gradients
    assert np.mean(d <= 1e-3 * lr + 1e-7) > 0.99
    # a learnable target: a fixed linear map of the inputs
    rng = np.random.default_rng(4)
    A = rng.standard_normal((R.IN, R.OUT)).astype(np.float32) * 0.05
    target = x @ A
    first = e.train_batch(sets, x, target, 3e-3)
    for _ in range(150):
        last = e.train_batch(sets, x, target, 3e-3)
    assert last < 0.2 * first, (first, last)


def test_fresh_edge_leaves_run_unchanged():
    from fdporo import edge as E
    from fdporo import job
    pair = E.make_pair(11, n=96, margin=40, depth_margin=60, nsteps=80)
    a, b = job.make_engine(pair.trunc), job.make_engine(pair.trunc)
    ed = E.Edge(seed=1)
    ed.attach(b)
    a.time_loop(1, 80)
    b.time_loop(1, 80)
    b.synchronize()
    compare_state(a, b)
    assert np.abs(a.field("UM")).max() > 0


def test_training_lowers_reflection():
    """A transparent 4-cell strip (the method without the network) reflects
    strongly; after training on eight small media, with runs on its own
    between teacher-forced levels, the edge reflects less on a held-out
    medium, with either output kind."""
    from fdporo import edge as E
    L = 600
    kw = dict(n=96, margin=160, depth_margin=200, nsteps=L, f0=100.0, strip="plain")
    pairs = [E.make_pair(s, **kw) for s in range(21, 29)]
    held = E.make_pair(99, **kw)
    plain = E.evaluate(held, L)
    scale = E.field_scales(pairs[0], levels=500, every=25)
    for kind, lr in (("damp", 1e-3), ("correct", 3e-4)):
        ed = E.Edge(scale=scale, seed=3)
        ed.set_output(kind)
        for _ in range(2):
            for p in pairs:
                E.train_pair(ed, p, levels=L, lr=lr, free_every=50, free_run=25)
        learned = E.evaluate(held, L, edge=ed)
        print(kind, "reflected energy: strip alone", plain, "with the network", learned)
        assert learned["reflected_energy"] < 0.3 * plain["reflected_energy"]
        assert learned["seismogram_rel_l2"] < 0.5 * plain["seismogram_rel_l2"]


def test_training_is_bit_reproducible():
    """Each tile's gradient is a partial of its own, added to the gradient in
    tile order: two trainings from the same seed on the same levels end
    with the same parameters, bit for bit."""
    from fdporo import edge as E
    pair = E.make_pair(21, n=96, margin=160, depth_margin=200, nsteps=200, f0=100.0, strip="plain")
    scale = E.field_scales(pair, levels=150, every=25)
    params = []
    for _ in range(2):
        ed = E.Edge(scale=scale, seed=3)
        ed.set_output("correct")
        E.train_pair(ed, pair, levels=200, lr=3e-4, free_every=50, free_run=25)
        params.append(ed.params())
    assert np.any(params[0] != 0)
    np.testing.assert_array_equal(params[0], params[1])


def test_attached_edge_runs_march_contexts_in_place(monkeypatch):
    """A context made with the march variant runs its levels in place while a
    learned edge is attached (the edge's kernels work on the current buffers
    after every level); with a fresh edge, whose corrections are zero, it
    equals the same context without one, which runs march levels."""
    from fdporo import edge as E
    from fdporo import job
    monkeypatch.setenv("FDP_KERNEL_VARIANT", "march")
    pair = E.make_pair(11, n=96, margin=40, depth_margin=60, nsteps=80)
    a, b = job.make_engine(pair.trunc), job.make_engine(pair.trunc)
    assert a.march_info() is not None
    E.Edge(seed=1).attach(b)
    assert b.march_info() is None
    a.time_loop(1, 33)
    b.time_loop(1, 33)
    a.time_loop(34, 80)
    b.time_loop(34, 80)
    b.synchronize()
    compare_state(a, b)
    assert np.abs(a.field("UM")).max() > 0
