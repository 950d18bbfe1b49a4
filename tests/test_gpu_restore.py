"""Repeated solves on one handle, and the bounded grid barrier.

A BCSR handle keeps an undo log of the arcs each solve pushes on; the next
fresh solve restores only those arcs (and their twins) to their capacities,
or every arc after new capacities or a full log.  Every solve here must
equal the oracle and pass the device certificate whatever came before it on
the handle: other terminals, a completed flow (a second, state-mode launch),
an aborted solve, new capacities.

The grid barrier gives up after `barrier_timeout_ns`.  With a timeout of one
nanosecond every wait that is not the last arrival expires while all blocks
still arrive and leave, so the solve returns WBPR_ERR_TIMEOUT without any
block left waiting; the handle must then solve exactly again."""
import numpy as np
import pytest

import oracle
import wbpr_gb300 as W

pytestmark = pytest.mark.gpu


def exact(g, s=None, t=None):
    return oracle.dinic(g.n, g.off, g.dst, g.cap, g.s if s is None else s, g.t if t is None else t)


def certified(d):
    rep = d.verify()
    assert rep["ok"] and rep["label_violations"] == 0, rep


@pytest.mark.parametrize("make", [lambda: W.gen_rmat(14, 16, seed=11), lambda: W.gen_genrmf(8, 16, 1, 10000, 4),
                                  lambda: W.gen_layered(24, 128, 3, 6, 1, 1000, 9), lambda: W.gen_grid(96, 96, 2)])
def test_resolves_with_other_terminals_and_states(make):
    g = make()
    rng = np.random.default_rng(g.n)
    pairs = [(g.s, g.t)]
    deg = np.diff(g.off)
    cand = np.flatnonzero(deg > 0)
    for _ in range(3):
        s, t = rng.choice(cand, 2, replace=False)
        pairs.append((int(s), int(t)))
    with W.DeviceGraph(g, "bcsr") as d:
        for rep in range(2):
            for s, t in pairs:
                for algo in ("vc", "tc"):
                    r = d.solve(algo, s, t)
                    assert r.flow == exact(g, s, t), (rep, s, t, algo)
                    certified(d)
            # a completed flow runs a second launch on the same residuals
            r = d.solve("vc", g.s, g.t)
            d.complete_flow()
            assert d.solve("vc", g.s, g.t).flow == r.flow
            certified(d)


def test_resolve_after_new_capacities_and_many_pushes():
    # a grid makes millions of pushes (the log may fill up: the next restore is
    # then a full rewrite); new capacities also force a full rewrite
    g = W.gen_grid(256, 256, 5)
    with W.DeviceGraph(g, "bcsr") as d:
        for _ in range(2):
            assert d.solve("vc").flow == exact(g)
            certified(d)
        cap = g.cap.copy()
        rng = np.random.default_rng(3)
        idx = rng.choice(g.m, 2000, replace=False)
        cap[idx] = rng.integers(0, 2000, idx.size)
        d.set_capacities(cap)
        h = W.Graph(g.n, g.off, g.dst, cap, g.s, g.t)
        for _ in range(2):
            assert d.solve("vc").flow == exact(h)
            certified(d)


def test_barrier_timeout_is_reported_and_the_handle_recovers():
    g = W.gen_genrmf(8, 16, 1, 10000, 6)  # ~190 rounds: hundreds of grid barriers
    want = exact(g)
    with W.DeviceGraph(g, "bcsr") as d:
        assert d.solve("vc", grid_blocks=8).flow == want
        for algo in ("vc", "tc"):
            with pytest.raises(W.WbprError) as e:
                d.solve(algo, grid_blocks=8, barrier_timeout_ns=1)
            assert e.value.status == 8  # WBPR_ERR_TIMEOUT
            r = d.solve(algo, grid_blocks=8)
            assert r.flow == want
            certified(d)
    with W.DeviceGraph(g, "rcsr") as d:
        with pytest.raises(W.WbprError) as e:
            d.solve("vc", grid_blocks=8, barrier_timeout_ns=1)
        assert e.value.status == 8
        assert d.solve("vc", grid_blocks=8).flow == want
        certified(d)
