"""The reference's configuration tests (src/config.rs:505-840), restated for the Python mirror of
SimConfig: TOML and JSON loading, integrator kinds, nsig forms, validation, and delays resolved from
tract lengths. Each test cites the reference test it follows."""
import json

import pytest

from hyburn_gb300.config import (InvalidConfig, NetworkConfig, ProjectionConfig, SimConfig, SubnetworkConfig)

G2DO = [1.0, 0.0, -2.0, -10.0, 0.0, 0.02, 3.0, 1.0, 0.0, 1.0, 1.0, 1.0]
HEAD = """
sim_length = 100.0
dt = 0.1
{extra}
[network]
[[network.subnetworks]]
model = "Generic2dOscillator"
nnodes = 2
params = [1.0, 0.0, -2.0, -10.0, 0.0, 0.02, 3.0, 1.0, 0.0, 1.0, 1.0, 1.0]
initial_state = [0.0, 0.5, 0.0, 0.5]
"""


def toml(extra=""):
    return SimConfig.from_toml_str(HEAD.format(extra=extra))


def one_subnet(model="Generic2dOscillator", nvar=2, params=None, dt=0.1, projections=(), speed=3.0):
    return SimConfig(sim_length=100.0, dt=dt, speed=speed,
                     network=NetworkConfig([SubnetworkConfig(model, 2, [0.0] * (nvar * 2), list(params or G2DO))],
                                           list(projections)))


def test_parse_minimal_config():  # config.rs:510-530
    cfg = SimConfig.from_toml_str("""
sim_length = 1000.0
dt = 0.1

[network]
[[network.subnetworks]]
model = "Generic2dOscillator"
 nnodes = 2
params = [1.0, 0.0, -2.0, -10.0, 0.0, 0.02, 3.0, 1.0, 0.0, 1.0, 1.0, 1.0]
initial_state = [0.0, 0.5, 0.0, 0.5]
""")
    assert cfg.sim_length == 1000.0 and cfg.dt == 0.1
    assert len(cfg.network.subnetworks) == 1 and cfg.network.subnetworks[0].model == "Generic2dOscillator"
    assert cfg.integrator == "heun"
    assert cfg.nsig == 0.0
    cfg.validate()


def test_parse_config_with_integrator():  # config.rs:533-551
    cfg = toml('integrator = "euler_stochastic"\nnsig = 0.5')
    assert cfg.integrator == "euler_stochastic" and cfg.nsig == 0.5
    cfg.validate()


def test_validate_invalid_dt():  # config.rs:554-568
    cfg = SimConfig(sim_length=100.0, dt=-0.1, network=NetworkConfig([], []))
    with pytest.raises(InvalidConfig):
        cfg.validate()


@pytest.mark.parametrize("model,nvar,nparams", [  # config.rs:571-604
    ("Generic2dOscillator", 2, 12), ("MontbrioPazoRoxin", 2, 7), ("ReducedWongWang", 1, 8),
    ("Kuramoto", 1, 1), ("JansenRit", 6, 13), ("WilsonCowan", 2, 22)])
def test_validate_all_models(model, nvar, nparams):
    one_subnet(model, nvar, [0.0] * nparams).validate()


def test_validate_unknown_model():  # config.rs:607-633
    with pytest.raises(InvalidConfig) as e:
        one_subnet("NonexistentModel", 2, [0.0] * 12).validate()
    assert "Unknown model" in str(e.value) and "Known models" in str(e.value)


def test_nsig_scalar_and_per_variable_deserialization():  # config.rs:636-667
    assert toml("nsig = 0.05").nsig == 0.05
    assert toml("nsig = [0.01, 0.02]").nsig == [0.01, 0.02]


def test_nsig_to_vec():  # config.rs:670-681
    assert SimConfig(sim_length=1.0, dt=0.1, network=NetworkConfig([]), nsig=0.05).nsig_vec(3) == [0.05] * 3
    cfg = SimConfig(sim_length=1.0, dt=0.1, network=NetworkConfig([]), nsig=[0.01, 0.02])
    assert cfg.nsig_vec(2) == [0.01, 0.02]
    with pytest.raises(InvalidConfig):
        cfg.nsig_vec(3)


@pytest.mark.parametrize("nsig", [0.05, [0.01, 0.02]])
def test_nsig_json(nsig):  # config.rs:684-695
    raw = {"sim_length": 100.0, "dt": 0.1, "nsig": nsig,
           "network": {"subnetworks": [{"model": "Generic2dOscillator", "nnodes": 2, "nmodes": 1, "params": G2DO,
                                        "initial_state": [0.0, 0.5, 0.0, 0.5]}], "projections": []}}
    cfg = SimConfig.from_dict(json.loads(json.dumps(raw)))
    assert cfg.nsig == nsig


@pytest.mark.parametrize("kind", ["rk4", "rk4_stochastic"])
def test_rk4_integrator_deserialization(kind):  # config.rs:698-730
    assert toml(f'integrator = "{kind}"\nnsig = 0.01').integrator == kind


def test_unknown_integrator_is_a_parse_error():  # IntegratorKind has no other variant (config.rs:27-42)
    with pytest.raises(InvalidConfig, match="unknown integrator"):
        toml('integrator = "leapfrog"')


def _tract_projection(delays, lengths):
    return ProjectionConfig(0, 0, 1.0, delays=list(delays), tract_lengths=list(lengths), coupling_fn="Linear",
                            coupling_params=[1.0, 0.0])


def test_resolve_delays_from_tract_lengths():  # config.rs:733-769
    cfg = one_subnet(projections=[_tract_projection([], [30.0, 15.0])])
    cfg.resolve_delays()
    assert cfg.network.projections[0].delays == [100, 50]


def test_resolve_delays_explicit_precedence():  # config.rs:772-807
    cfg = one_subnet(projections=[_tract_projection([5, 10], [30.0, 15.0])])
    cfg.resolve_delays()
    assert cfg.network.projections[0].delays == [5, 10]


def test_resolve_delays_non_positive_speed_error():  # config.rs:810-840
    cfg = one_subnet(projections=[_tract_projection([], [30.0])], speed=0.0)
    with pytest.raises(InvalidConfig):
        cfg.resolve_delays()
