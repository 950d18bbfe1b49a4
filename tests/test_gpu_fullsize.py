"""The CUDA path at full size against the oracle's pinned values
(tests/golden/fullsize.json): the scale-22 R-MAT (both layouts), the 2M x 2M
matching, all 4,096 batched instances and a few 512 x 512 grids.  Bit-exact:
every maximum-flow value equals the oracle's, and every single-instance solve
also passes the device certificate."""
import json
import os

import numpy as np
import pytest

import wbpr_gb300 as W
from conftest import ROOT
from wbpr_gb300 import workloads as WL

pytestmark = pytest.mark.gpu
PINS = json.load(open(os.path.join(ROOT, "tests", "golden", "fullsize.json")))


def _solve_pinned(g, pin, layouts=("bcsr", "rcsr"), algos=("vc",)):
    assert WL.csr_hash(g) == pin["csr_hash"]
    for layout in layouts:
        with W.DeviceGraph(g, layout) as d:
            for algo in algos:
                for _ in range(2):  # the second solve restores the first one's residuals
                    assert d.solve(algo).flow == pin["flow"], (layout, algo)
                rep = d.verify()
                assert rep["ok"] and rep["cut_value"] == pin["flow"], (layout, algo, rep)


def test_config1_rmat22_full_size():
    _solve_pinned(WL.config1(), PINS["config1"])


def test_config2_matching_full_size():
    _solve_pinned(WL.config2(), PINS["config2"], layouts=("bcsr",), algos=("vc", "tc"))


def test_config3_all_4096_batched_instances():
    gs = WL.config3(4096)
    want = np.asarray(PINS["config3"]["flows"], np.int64)
    with W.Batch(gs) as b:
        for tile, block in ((8, 512), (16, 256)):
            flows, _ = b.solve(tile=tile, block=block)
            assert np.array_equal(flows, want), (tile, block, int(np.flatnonzero(flows != want)[0]))


def test_config4_grids_full_size():
    for seed in (0, 1, 2):
        g = WL.config4(seed)
        with W.DeviceGraph(g, "bcsr") as d:
            assert d.solve("vc").flow == PINS["config4"]["flows"][seed], seed
            assert d.verify()["ok"]
