"""Per-node model parameters (hb_subnet_desc.node_params, an extension of this engine) in the oracle.

The reference takes one parameter row per subnetwork; this engine also takes a row per node, shared by
all sweep points ([nodes, params]) or one table per point ([points, nodes, params]), with swept model
parameters still taking their sweep values at every node. These CPU tests pin the oracle's semantics
against the reference's own paths: identical rows equal no rows, a decoupled network equals one-node
runs with each node's row, and a per-point table of eta equals the reference's per-point
multi-parameter fallback (dfun.rs:99-133) over the same (coupling scale, eta) grid.
"""
import copy

import numpy as np
import pytest

from hyburn_gb300 import SweepParam, SweepPoint, SweepSpec
from hyburn_gb300._abi import HB_SEM_DELAY_RING
from hyburn_gb300.config import InvalidConfig
from oracle.hb_oracle import OracleEngine

from cases import NATIVE_SWEEP, single_model, sweep_values


def with_rows(cfg, rows):
    c = copy.deepcopy(cfg)
    c.network.subnetworks[0].node_params = np.asarray(rows, np.float32)
    return c


@pytest.mark.parametrize("model", ["Generic2dOscillator", "MontbrioPazoRoxin", "Kuramoto", "WilsonCowan"])
def test_identical_rows_change_nothing(model):
    cfg = single_model(model, 10, "heun", "Linear", (0.1,), weights="csr", delays="per_edge", density=0.4)
    p = np.asarray(cfg.network.subnetworks[0].params, np.float32)
    rows = np.tile(p, (10, 1))
    par = SweepParam(0, NATIVE_SWEEP[model])
    vals = sweep_values(model, 3)
    a = OracleEngine.from_config(cfg, 3, semantics=HB_SEM_DELAY_RING).run_sweep(par, vals, 80)
    b = OracleEngine.from_config(with_rows(cfg, rows), 3, semantics=HB_SEM_DELAY_RING).run_sweep(par, vals, 80)
    assert np.array_equal(a.final_states[0], b.final_states[0]) and np.array_equal(a.tavg[0], b.tavg[0])


def test_decoupled_nodes_follow_their_own_rows():
    """Zero coupling weight: node i of the table run equals a one-node run with row i."""
    n, T = 6, 120
    cfg = single_model("Generic2dOscillator", n, "heun", "Linear", (0.0,), weights="csr", density=0.5)
    rng = np.random.default_rng(4)
    p = np.asarray(cfg.network.subnetworks[0].params, np.float32)
    rows = np.tile(p, (n, 1))
    rows[:, 1] = rng.uniform(-0.5, 0.5, n)   # I
    rows[:, 2] = rng.uniform(-3.0, -1.0, n)  # a
    r = OracleEngine.from_config(with_rows(cfg, rows), 1).run_sweep(SweepParam(-1, 0), [0.0], T)
    x0 = np.asarray(cfg.network.subnetworks[0].initial_state, np.float32).reshape(n, 2)
    for i in range(n):
        one = single_model("Generic2dOscillator", 1, "heun", "Linear", (0.0,), weights="scalar")
        one.network.subnetworks[0].initial_state = x0[i].tolist()
        one.network.subnetworks[0].params = rows[i].tolist()
        o = OracleEngine.from_config(one, 1).run_sweep(SweepParam(-1, 0), [0.0], T)
        assert np.array_equal(np.asarray(r.final_states[0]).reshape(n, 2)[i], o.final_states[0])


def test_per_point_table_equals_multi_parameter_fallback():
    """(G, eta) grid: a per-point table of eta with the coupling scale swept per point equals the
    reference's multi-parameter sweep over (coupling a, eta, I_ext) - two model parameters select the
    per-point fallback, which applies eta to every node."""
    n, T = 12, 150
    cfg = single_model("MontbrioPazoRoxin", n, "rk4", "Linear", (1.0,), weights="csr", delays="per_edge", dt=0.05)
    p = np.asarray(cfg.network.subnetworks[0].params, np.float32)
    G = np.linspace(0.0, 1.0, 4).astype(np.float32)
    eta = np.linspace(-6.0, -3.0, 3).astype(np.float32)
    B = G.size * eta.size
    spec = SweepSpec([SweepPoint(-1, 0, G.tolist()), SweepPoint(0, 2, eta.tolist()), SweepPoint(0, 4, [float(p[4])])])
    m = OracleEngine.from_config(cfg, B, semantics=HB_SEM_DELAY_RING).run_sweep_multi(spec, T)
    rows = np.tile(p, (B, n, 1))
    rows[:, :, 2] = np.repeat(np.tile(eta, G.size), n).reshape(B, n)
    g = OracleEngine.from_config(with_rows(cfg, rows), B, semantics=HB_SEM_DELAY_RING).run_sweep(
        SweepParam(-1, 0), np.repeat(G, eta.size), T)
    assert np.array_equal(m.final_states[0], g.final_states[0]) and np.array_equal(m.tavg[0], g.tavg[0])


def test_native_sweep_overrides_node_rows():
    n, T = 8, 60
    cfg = single_model("Kuramoto", n, "heun", "Kuramoto", (1.0,), weights="csr", delays="per_edge")
    omega = np.random.default_rng(2).standard_normal((n, 1)).astype(np.float32)
    vals = [0.3, 0.9]
    a = OracleEngine.from_config(with_rows(cfg, omega), 2, semantics=HB_SEM_DELAY_RING).run_sweep(SweepParam(0, 0), vals, T)
    b = OracleEngine.from_config(cfg, 2, semantics=HB_SEM_DELAY_RING).run_sweep(SweepParam(0, 0), vals, T)
    assert np.array_equal(a.final_states[0], b.final_states[0])


def test_node_rows_of_the_wrong_length_are_rejected():
    cfg = single_model("Kuramoto", 8, "heun", "Kuramoto", (1.0,), weights="csr")
    with pytest.raises(InvalidConfig):
        OracleEngine.from_config(with_rows(cfg, np.zeros(7, np.float32)), 2)
