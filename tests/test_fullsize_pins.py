"""The full-size pins (tests/golden/fullsize.json, from the CPU oracle) and
the generators they describe.  CPU only: every workload generator must still
produce the very CSR whose maximum flow was pinned (hashes), and the oracle
re-derives a sample of the pinned values.  The GPU tests compare the CUDA
path with these values at full size."""
import json
import os

import pytest

import oracle
from conftest import ROOT
from wbpr_gb300 import workloads as WL

PINS = json.load(open(os.path.join(ROOT, "tests", "golden", "fullsize.json")))


def test_single_instance_generators_match_their_pins():
    for name, make in (("config1", WL.config1), ("config2", WL.config2)):
        g = make()
        p = PINS[name]
        assert (g.n, g.m, g.s, g.t) == (p["n"], p["m"], p["s"], p["t"]), name
        assert WL.csr_hash(g) == p["csr_hash"], name
        assert p["flow"] == p["fifo_pr"]  # two oracle algorithms agree


def test_config1_and_2_values_and_certificate_shape():
    assert PINS["config1"]["flow"] == 1911604
    assert PINS["config2"]["flow"] == 1581980


@pytest.mark.parametrize("seed", range(20))
def test_config0_pins(seed):
    g = WL.config0(seed)
    assert WL.csr_hash(g) == PINS["config0"]["csr_hashes"][seed]
    assert oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t) == PINS["config0"]["flows"][seed]


def test_config3_instances_and_a_sample_of_flows():
    params = WL.config3_params(PINS["config3"]["count"])
    hashes = [int(WL.csr_hash(WL.config3_instance(p)), 16) >> 1 for p in params]
    assert WL.flows_hash(hashes) == PINS["config3"]["csr_hashes_hash"]
    assert WL.flows_hash(PINS["config3"]["flows"]) == PINS["config3"]["flows_hash"]
    for i in range(0, 4096, 256):
        g = WL.config3_instance(params[i])
        assert oracle.dinic(g.n, g.off, g.dst, g.cap, g.s, g.t) == PINS["config3"]["flows"][i], i


@pytest.mark.parametrize("seed", [0, 1, 255])
def test_config4_grid_pins(seed):
    g = WL.config4(seed)
    assert WL.csr_hash(g) == PINS["config4"]["csr_hashes"][seed]
    if seed == 0:
        assert oracle.fifo_pr(g.n, g.off, g.dst, g.cap, g.s, g.t) == PINS["config4"]["flows"][0]
