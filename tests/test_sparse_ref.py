"""The reference's CSR tests (src/engine/sparse.rs:133-395, src/engine/mod.rs:159-236), restated as whole
runs of the batch engine: a CSR projection is the same coupling as the dense matrix it stores.

On the CPU through the oracle, on the GPU through the CUDA engine (each form against the oracle at
rel 1e-5 / abs 1e-6, and CSR against dense within the reference's 1e-5)."""
import numpy as np
import pytest

from hyburn_gb300._abi import HB_SEM_DELAY_RING
from hyburn_gb300.config import DEFAULT_PARAMS, NetworkConfig, ProjectionConfig, SimConfig, SubnetworkConfig
from hyburn_gb300.engine import SweepParam

G2DO = list(DEFAULT_PARAMS["Generic2dOscillator"])
NATIVE = SweepParam(0, 1)
# 5-node directed ring, node i receives from node (i - 1) mod 5 with weight 0.1 (sparse.rs:156-175)
RING_DENSE = [[0, 0, 0, 0, .1], [.1, 0, 0, 0, 0], [0, .1, 0, 0, 0], [0, 0, .1, 0, 0], [0, 0, 0, .1, 0]]
RING_CSR = {"data": [.1] * 5, "indices": [4, 0, 1, 2, 3], "indptr": [0, 1, 2, 3, 4, 5]}
# the 3 x 3 matrix of the matvec test (sparse.rs:134-153): [[0, 2, 0], [0, 0, 3], [1, 0, 0]]
M3_DENSE = [[0, 2, 0], [0, 0, 3], [1, 0, 0]]
M3_CSR = {"data": [2.0, 3.0, 1.0], "indices": [1, 2, 0], "indptr": [0, 1, 2, 3]}


def ring(weights, conn, integrator="heun"):
    """sparse.rs:288-395: G2DO defaults, every state 0.1, delays 1, Linear(a = 1), Heun, dt 0.1."""
    return SimConfig(sim_length=1.0, dt=0.1, integrator=integrator,
                     network=NetworkConfig([SubnetworkConfig("Generic2dOscillator", 5, [0.1] * 10, list(G2DO))],
                                           [ProjectionConfig(0, 0, weights, conn_type=conn, delays=[1] * 5,
                                                             coupling_fn="Linear", coupling_params=[1.0])]))


def matvec_net(weights, conn):
    """Three G2DO nodes with V = [1, 2, 3], W = 0, undelayed Linear(a = 1, b = 0) coupling on V (weights
    None: a scalar projection of weight 0, the uncoupled network)."""
    if weights is None:
        weights, conn = 0.0, "all_to_all"
    projs = [ProjectionConfig(0, 0, weights, conn_type=conn, coupling_fn="Linear", coupling_params=[1.0, 0.0])]
    return SimConfig(sim_length=0.1, dt=0.1, integrator="euler",
                     network=NetworkConfig([SubnetworkConfig("Generic2dOscillator", 3, [1.0, 0.0, 2.0, 0.0, 3.0, 0.0],
                                                             list(G2DO))], projs))


def coupling_from_one_step(engine_cls, weights, conn):
    """One Euler step moves V by dt d tau gamma c (G2DO, dfun.rs:271-316; gamma multiplies I + c), so
    the coupling each node received is the V difference from the uncoupled step over dt d tau gamma."""
    tau, d, gamma = G2DO[0], G2DO[5], G2DO[11]
    v = []
    for w in (weights, None):
        r = engine_cls.from_config(matvec_net(w, conn), 1).run_sweep(NATIVE, [G2DO[1]], 1)
        v.append(np.asarray(r.final_states[0], np.float64).reshape(3, 2)[:, 0])
    return (v[0] - v[1]) / (0.1 * d * tau * gamma)


def oracle():
    from oracle.hb_oracle import OracleEngine
    return OracleEngine


# ---- CPU: the oracle ----

@pytest.mark.parametrize("semantics", [0, HB_SEM_DELAY_RING])
@pytest.mark.parametrize("integrator", ["heun", "rk4"])
def test_engine_csr_from_config_matches_dense(semantics, integrator):  # sparse.rs:288-395, mod.rs:159-236
    out = [oracle().from_config(ring(w, c, integrator), 1, semantics=semantics).run_sweep(NATIVE, [G2DO[1]], 10)
           for w, c in ((RING_DENSE, "all_to_all"), (RING_CSR, "csr"))]
    assert np.abs(out[0].final_states[0] - out[1].final_states[0]).max() < 1e-5
    assert np.abs(out[0].tavg[0] - out[1].tavg[0]).max() < 1e-5


@pytest.mark.parametrize("weights,conn", [(M3_CSR, "csr"), (M3_DENSE, "all_to_all")])
def test_csr_matvec_basic(weights, conn):  # sparse.rs:134-153: W x = [4, 9, 1]
    c = coupling_from_one_step(oracle(), weights, conn)
    assert np.allclose(c, [4.0, 9.0, 1.0], rtol=1e-3), c


# ---- GPU: the CUDA engine ----

@pytest.mark.gpu
@pytest.mark.parametrize("semantics", [0, HB_SEM_DELAY_RING])
@pytest.mark.parametrize("integrator", ["heun", "rk4"])
def test_engine_gpu_csr_matches_dense(semantics, integrator):
    from test_parity_gpu import compare
    g = []
    for w, c in ((RING_DENSE, "all_to_all"), (RING_CSR, "csr")):
        _, _, res, _ = compare(ring(w, c, integrator), 1, NATIVE, [G2DO[1]], 10, semantics=semantics)
        g.append(res)
    assert np.abs(g[0].final_states[0] - g[1].final_states[0]).max() < 1e-5
    assert np.abs(g[0].tavg[0] - g[1].tavg[0]).max() < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("weights,conn", [(M3_CSR, "csr"), (M3_DENSE, "all_to_all")])
def test_engine_gpu_csr_matvec_basic(weights, conn):
    from hyburn_gb300 import BatchHybridEngine
    c = coupling_from_one_step(BatchHybridEngine, weights, conn)
    assert np.allclose(c, [4.0, 9.0, 1.0], rtol=1e-3), c


def _random_pair(seed):
    """A random network twice: dense weights and the same matrix as CSR (seeded)."""
    from cases import sub
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(3, 12))
    w = np.where(rng.random((n, n)) < 0.4, rng.uniform(0.1, 1.0, (n, n)), 0.0).astype(np.float32)
    rows, cols = np.nonzero(w)
    csr = {"data": w[rows, cols].tolist(), "indices": cols.tolist(),
           "indptr": np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))]).tolist()}
    fn, cp = [("Linear", [0.3, 0.01]), ("Sigmoidal", [0.0, 1.0, 0.0, 1.0, 1.0]), ("HyperbolicTangent", [0.1, 1.0, 0.2, 2.0]),
              ("Difference", [0.05])][seed % 4]
    integ = ["heun", "rk4", "euler"][seed % 3]
    delay = [int(rng.integers(0, 6))]
    return [SimConfig(sim_length=1.0, dt=0.1, integrator=integ,
                      network=NetworkConfig([sub("Generic2dOscillator", n, seed)],
                                            [ProjectionConfig(0, 0, weights, conn_type=conn, delays=delay,
                                                              coupling_fn=fn, coupling_params=cp)]))
            for weights, conn in ((w.tolist(), "all_to_all"), (csr, "csr"))]


@pytest.mark.parametrize("seed", range(12))
def test_csr_is_the_dense_matrix_it_stores(seed):
    """The batch engine densifies CSR weights (engine.rs:298-322), so in its default delay semantics a
    CSR projection and the dense matrix it stores give the same run bit for bit: random networks,
    coupling functions, delays and integrators through the oracle."""
    out = [oracle().from_config(cfg, 2).run_sweep(NATIVE, [0.0, 0.3], 40) for cfg in _random_pair(seed)]
    assert np.array_equal(out[0].final_states[0], out[1].final_states[0])
    assert np.array_equal(out[0].tavg[0], out[1].tavg[0])


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(12))
def test_engine_gpu_csr_is_the_dense_matrix_it_stores(seed):
    """The same on the GPU: both forms become the same edge list, so the runs agree bit for bit; the
    dense one against the oracle."""
    from hyburn_gb300 import BatchHybridEngine
    from test_parity_gpu import compare
    dense, csr = _random_pair(seed)
    compare(dense, 2, NATIVE, [0.0, 0.3], 40)
    a, b = (BatchHybridEngine.from_config(c, 2).run_sweep(NATIVE, [0.0, 0.3], 40) for c in (dense, csr))
    assert np.array_equal(a.final_states[0], b.final_states[0]) and np.array_equal(a.tavg[0], b.tavg[0])


def _two_population_dense():
    """engine.rs:1634-1690: two 2-node G2DO populations (initial state [0.1, 0.1, 0.2, 0.2], default
    parameters), an identity dense projection from the first to the second with delay 0, Linear(1.0),
    Euler at dt 0.1."""
    from hyburn_gb300.config import SubnetworkConfig
    subs = [SubnetworkConfig("Generic2dOscillator", 2, [0.1, 0.1, 0.2, 0.2], list(G2DO)) for _ in range(2)]
    proj = ProjectionConfig(0, 1, [[1.0, 0.0], [0.0, 1.0]], delays=[0], coupling_fn="Linear", coupling_params=[1.0])
    return SimConfig(sim_length=10.0, dt=0.1, integrator="euler", network=NetworkConfig(subs, [proj]))


def test_batch_engine_dense_coupling_shape():  # engine.rs:1634-1690
    r = oracle().from_config(_two_population_dense(), 2).run_sweep(NATIVE, [0.0, 0.5], 10)
    assert r.n_sweep == 2 and len(r.tavg) == 2
    assert all(np.isfinite(t).all() and t.size == 2 * 2 * 2 for t in r.tavg)


@pytest.mark.gpu
def test_engine_gpu_dense_coupling_between_populations():
    from test_parity_gpu import compare
    compare(_two_population_dense(), 2, NATIVE, [0.0, 0.5], 10)
