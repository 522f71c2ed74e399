"""The CPU oracle against the reference's own known-answer tests.

Each case restates an assertion of hyburn's unit tests (file:line of the reference test given per
test) and checks the oracle with the reference's tolerance. These pin the oracle before it is
trusted as the checker of the CUDA engine.
"""
import math

import numpy as np

from oracle import hb_oracle as O

G2DO = [1.0, 0.0, -2.0, -10.0, 0.0, 0.02, 3.0, 1.0, 0.0, 1.0, 1.0, 1.0]
MPR = [1.0, 1.0, -5.0, 15.0, 0.0, 1.0, 0.0]
JR = [3.25, 22.0, 0.1, 0.05, 5.52, 0.0025, 0.56, 135.0, 1.0, 0.8, 0.25, 0.25, 0.22]
WC = [12.0, 4.0, 13.0, 11.0, 10.0, 10.0, 1.2, 2.8, 1.0, 0.0, 1.0, 4.0, 1.0, 0.0, 1.0, 1.0, 1.0, 1.0, 0.0, 0.0, 1.0, 1.0]
RWW = [0.270, 0.108, 154.0, 0.641, 100.0, 0.6, 0.2609, 0.33]


# ---- dfun known answers (src/model/*.rs tests) ----

def test_g2do_equilibrium_with_defaults():  # g2do.rs:88-115
    d = O.dfun("Generic2dOscillator", G2DO, [0.0, 0.0], [0.0])[0]
    assert abs(d[0]) < 1e-5
    assert abs(d[1] + 0.04) < 1e-4


def test_g2do_simplified_form():  # g2do.rs:117-144
    p = [1.0, 0.0, 1.0, 1.0, 0.0, 1.0, 0.0, 1.0 / 3.0, 1.0, 1.0, 1.0, 1.0]
    d = O.dfun("Generic2dOscillator", p, [0.5, 0.3], [0.0])[0]
    assert abs(d[0] - 0.7583) < 1e-3
    assert abs(d[1] - 1.2) < 1e-3


def test_mpr_dfun_at_zero():  # mpr.rs:73-97
    d = O.dfun("MontbrioPazoRoxin", MPR, [0.0, 0.0], [0.0, 0.0])[0]
    assert abs(d[0] - 1.0 / math.pi) < 1e-4
    assert abs(d[1] + 5.0) < 1e-4


def test_mpr_dfun_with_state():  # mpr.rs:99-122
    d = O.dfun("MontbrioPazoRoxin", MPR, [0.5, 0.3], [0.0, 0.0])[0]
    assert abs(d[0] - (1.0 / math.pi + 0.3)) < 1e-3
    assert abs(d[1] - (0.09 - math.pi ** 2 * 0.25 - 5.0 + 7.5)) < 1e-3


def test_jr_dfun_at_zero():  # jansen_rit.rs:136-181
    d = O.dfun("JansenRit", JR, [0.0] * 6, [0.0])[0]
    sigm0 = 2.0 * 0.0025 / (1.0 + math.exp(0.56 * 5.52))
    assert abs(d[0]) < 1e-6 and abs(d[1]) < 1e-6 and abs(d[2]) < 1e-6
    assert abs(d[3] - 3.25 * 0.1 * sigm0) < 1e-6
    assert abs(d[4] - 3.25 * 0.1 * (0.22 + 0.8 * 135.0 * sigm0)) < 1e-5
    assert abs(d[5] - 22.0 * 0.05 * 0.25 * 135.0 * sigm0) < 1e-5


def test_jr_dfun_nonzero_state_and_coupling():  # jansen_rit.rs:183-230
    d = O.dfun("JansenRit", JR, [0.1, 0.2, 0.05, 0.0, 0.0, 0.0], [0.1])[0]
    assert abs(d[0]) < 1e-6 and abs(d[1]) < 1e-6 and abs(d[2]) < 1e-6
    assert abs(d[3] + 9.24e-4) < 5e-4
    assert abs(d[4] - 0.2755) < 0.01
    assert abs(d[5] - 0.0428) < 0.005


def test_wc_dfun_at_zero():  # wilson_cowan.rs:102-119
    d = O.dfun("WilsonCowan", WC, [0.0, 0.0], [0.0])[0]
    assert abs(d[0]) < 1e-5 and abs(d[1]) < 1e-5


def test_kuramoto_dfun():  # kuramoto_model.rs:65-80
    d = O.dfun("Kuramoto", [1.0], [0.5], [0.3])[0]
    assert abs(d[0] - 1.3) < 1e-5


def test_rww_dfun_at_zero():  # rww.rs:73-103
    d = O.dfun("ReducedWongWang", RWW, [0.0], [0.0])[0]
    x = np.float32(0.33)
    ax_b = np.float32(0.270) * x - np.float32(0.108)
    h = ax_b / (np.float32(1.0) - np.exp(np.float32(-154.0) * ax_b))
    assert abs(d[0] - h * np.float32(0.641)) < 1e-5


# ---- clamps (mpr.rs:124-136, wilson_cowan.rs:121-133, rww.rs:105-124, dfun.rs:204-207) ----

def test_mpr_clamp():
    x = O.clamp("MontbrioPazoRoxin", [[-0.5, 1.0]])[0]
    assert x[0] == 0.0 and abs(x[1] - 1.0) < 1e-6


def test_wc_clamp():
    x = O.clamp("WilsonCowan", [[-0.5, 1.5]])[0]
    assert x[0] == 0.0 and x[1] == 1.0


def test_rww_clamp():
    assert O.clamp("ReducedWongWang", [[-0.2]])[0, 0] == 0.0
    assert O.clamp("ReducedWongWang", [[1.5]])[0, 0] == 1.0


def test_kuramoto_wrap():
    x = O.clamp("Kuramoto", [[7.0], [-1.0]])[:, 0]
    two_pi = np.float32(2.0) * np.float32(math.pi)
    assert np.all((x >= 0) & (x < two_pi))
    assert abs(x[0] - (7.0 - 2 * math.pi)) < 1e-5


# ---- coupling functions (coupling.rs:497-1225) ----

def test_linear_pre_post():  # coupling.rs:506-521
    x = [[1.0, 2.0], [3.0, 4.0]]
    assert np.allclose(O.coupling_pre("Linear", [2.0, 0.0], x), x)
    assert np.allclose(O.coupling_post("Linear", [2.0, 0.0], x), [[2, 4], [6, 8]])


def test_linear_with_offset():  # coupling.rs:523-533
    assert abs(O.coupling_post("Linear", [2.0, 1.0], [[1.0]])[0, 0] - 3.0) < 1e-6


def test_sigmoidal_5param_post():  # coupling.rs:535-545
    assert abs(O.coupling_post("Sigmoidal", [-1.0, 1.0, 0.0, 1.0, 1.0], [[0.0]])[0, 0]) < 1e-6


def test_sigmoidal_old_3param_compat():  # coupling.rs:547-560: cmin=-1, cmax=1, mid=0, a=1, sigma=2
    gx = 0.7
    got = O.coupling_post("Sigmoidal", [1.0, 0.0, 2.0], [[gx]])[0, 0]
    want = -1.0 + 2.0 / (1.0 + math.exp(-(gx / 2.0)))
    assert abs(got - want) < 1e-6


def test_tanh_pre():  # coupling.rs:577-587
    assert abs(O.coupling_pre("HyperbolicTangent", [1.0, 1.0, 0.0, 1.0], [[0.0]])[0, 0] - 1.0) < 1e-6


def test_kuramoto_pre_two_channel():  # coupling.rs:589-601
    out = O.coupling_pre("Kuramoto", [1.0], [[1.5708]])
    assert out.shape == (1, 2)
    assert abs(out[0, 0] - 1.0) < 1e-4 and abs(out[0, 1]) < 1e-4


def test_kuramoto_post_with_target():  # coupling.rs:603-619
    got = O.coupling_post("Kuramoto", [1.0], [[0.5, 0.3]], x_i=[[0.0]], n_src=2)
    assert got.shape == (1, 1) and abs(got[0, 0] - 0.25) < 1e-5


def test_kuramoto_post_with_target_identity():  # coupling.rs:621-642
    theta, rowsum = 1.23, 0.5
    gx = [[rowsum * math.sin(theta), rowsum * math.cos(theta)]]
    assert abs(O.coupling_post("Kuramoto", [1.0], gx, x_i=[[theta]], n_src=2)[0, 0]) < 1e-5


def test_difference_pre_identity_and_post():  # coupling.rs:644-668
    assert np.allclose(O.coupling_pre("Difference", [0.1], [[1.0, 2.0]]), [[1.0, 2.0]])
    got = O.coupling_post("Difference", [0.1], [[5.0]], x_i=[[2.0]], rowsums=[3.0])[0, 0]
    assert abs(got - (-0.1)) < 1e-6


def _dense(name, params, w, x, x_i=None, n_src=1):
    """dense_coupling (coupling.rs:465-480): post_with_target(W @ pre(x), x_i)."""
    pre = O.coupling_pre(name, params, x)
    gx = np.asarray(w, np.float32) @ pre
    return O.coupling_post(name, params, gx, x_i=x_i, n_src=n_src)


def test_dense_coupling_kuramoto_classic():  # coupling.rs:670-698
    w = [[0.0, 0.5], [0.5, 0.0]]
    x = [[0.0], [math.pi / 2]]
    got = _dense("Kuramoto", [1.0], w, x, x_i=x, n_src=2)[:, 0]
    assert abs(got[0] - 0.25) < 1e-5 and abs(got[1] + 0.25) < 1e-5


def test_dense_coupling_linear_pipeline():  # coupling.rs:700-725
    got = _dense("Linear", [2.0, 1.0], [[1, 0, 0], [0, 1, 1]], [[1, 2], [3, 4], [5, 6]]).ravel()
    assert np.allclose(got, [3.0, 5.0, 17.0, 21.0], atol=1e-5)


def test_dense_coupling_sigmoidal_pipeline():  # coupling.rs:727-748
    got = _dense("Sigmoidal", [0.0, 1.0, 0.0, 1.0, 1.0], [[1.0, 1.0]], [[0.5], [1.5]])[0, 0]
    assert abs(got - 1.0 / (1.0 + math.exp(-2.0))) < 1e-5


def test_dense_coupling_tanh_pipeline():  # coupling.rs:750-771
    got = _dense("HyperbolicTangent", [1.0, 1.0, 0.0, 1.0], [[1.0, 1.0]], [[1.0], [-1.0]])[0, 0]
    assert abs(got - ((1 + math.tanh(1.0)) + (1 + math.tanh(-1.0)))) < 1e-4


def test_presigmoidal_static():  # coupling.rs:773-791
    got = O.coupling_pre("PreSigmoidal", [2.0, 1.0, 3.0, 0.5, 2.0, 0.0, 0.0], [[4.0, 5.0], [6.0, 7.0]]).ravel()
    exp = [2.0 * (1.0 + math.tanh(3.0 * (0.5 * v - 2.0))) for v in (4.0, 5.0, 6.0, 7.0)]
    assert np.allclose(got, exp, atol=1e-5)
    assert abs(got[0] - 2.0) < 0.01


def test_scaled_linear():  # coupling.rs:855-889
    assert abs(O.coupling_post("ScaledLinear", [3.0, 2.0], [[5.0]])[0, 0] - 9.0) < 1e-6
    got = _dense("ScaledLinear", [2.0, 1.0], [[1, 0], [0, 1]], [[3.0], [5.0]])[:, 0]
    assert np.allclose(got, [4.0, 8.0], atol=1e-5)


def test_presigmoidal_dynamic():  # coupling.rs:891-907
    got = O.coupling_pre("PreSigmoidal", [1.0, 0.0, 1.0, 1.0, 0.0, 1.0], [[1.0, 0.5], [2.0, 0.3]])
    assert got.shape == (2, 1)
    assert abs(got[0, 0] - math.tanh(0.5)) < 1e-5 and abs(got[1, 0] - math.tanh(1.7)) < 1e-5


def test_presigmoidal_dynamic_2cvar_collapse():  # coupling.rs:928-945
    got = O.coupling_pre("PreSigmoidal", [2.0, 1.0, 3.0, 0.5, 0.0, 1.0], [[4.0, 1.0], [6.0, 2.0]])[:, 0]
    assert abs(got[0] - 2.0 * (1.0 + math.tanh(3.0 * 1.0))) < 1e-4
    assert abs(got[1] - 2.0 * (1.0 + math.tanh(3.0 * 1.0))) < 1e-4


def test_sjr_pre_legacy_finite_nonnegative():  # coupling.rs:959-983
    got = O.coupling_pre("SigmoidalJansenRit", [1.0, 0.005, 0.56, 6.0], [[6.0, 4.0], [6.0, 4.0]])
    assert np.all(np.isfinite(got)) and np.all(got >= 0)
    got1 = O.coupling_pre("SigmoidalJansenRit", [1.0, 0.005, 0.56, 6.0], [[6.0], [8.0]])
    assert np.all(np.isfinite(got1))


def test_sjr_classic_pre_and_post():  # coupling.rs:985-1033
    got = O.coupling_pre("SigmoidalJansenRit", [2.0, 0.0, 0.01, 0.56, 6.0], [[8.0, 2.0], [4.0, 0.0]])[:, 0]
    for g, diff in zip(got, (6.0, 4.0)):
        assert abs(g - 0.01 / (1.0 + math.exp(0.56 * (6.0 - diff)))) < 1e-5
    post = O.coupling_post("SigmoidalJansenRit", [3.0, 0.0, 0.01, 0.56, 6.0], [[1.0], [2.0]])[:, 0]
    assert np.allclose(post, [3.0, 6.0], atol=1e-5)


def test_sjr_legacy_post_identity():  # coupling.rs:1035-1052
    post = O.coupling_post("SigmoidalJansenRit", [1.0, 0.005, 0.56, 6.0], [[0.01], [0.02]])[:, 0]
    assert np.allclose(post, [0.01, 0.02], atol=1e-7)


def test_kuramoto_pre_3d_channel_expansion():  # coupling.rs:1074-1087
    got = O.coupling_pre("Kuramoto", [1.0], [[0.0], [1.5708]])
    assert got.shape == (2, 2)
    assert abs(got[0, 0]) < 1e-5 and abs(got[0, 1] - 1.0) < 1e-5
    assert abs(got[1, 0] - 1.0) < 1e-5 and abs(got[1, 1]) < 1e-5


# ---- Balloon-Windkessel (bold.rs:173-219, bold_monitor.rs:262-294) ----

def test_bold_step_zero_input():
    sig = O.bold_model_run([0.0, 0.0], 0.001, 100)[-1]
    assert np.all(np.isfinite(sig)) and abs(sig[0]) < 1e-3


def test_bold_step_ramps_up():
    sig = O.bold_model_run([1.0, 1.0], 0.001, 5000)[:, 0]
    assert sig[-1] > 0.1


def test_bold_monitor_output_shape():
    inputs = np.repeat(np.sin(np.arange(20, dtype=np.float32))[:, None], 3, axis=1)
    out, n_samples = O.bold_monitor_run(inputs, 5, 0.01, 2.0, flush=False)
    assert n_samples == 4 and out.shape == (4, 3)
    out, _ = O.bold_monitor_run(inputs, 5, 0.01, 2.0, flush=True)
    assert out.size == 12


def test_bold_monitor_tr_downsample():
    inputs = np.repeat(np.sin(np.arange(100, dtype=np.float32) * 0.1)[:, None], 2, axis=1)
    out, n_samples = O.bold_monitor_run(inputs, 10, 0.025, 1.0, flush=False)
    assert out.shape[1] == 2 and 0 < out.shape[0] <= n_samples


def test_fp64_twin_agrees_on_kats():
    a = O.dfun("JansenRit", JR, [0.1, 0.2, 0.05, 0.0, 0.0, 0.0], [0.1])
    b = O.dfun("JansenRit", JR, [0.1, 0.2, 0.05, 0.0, 0.0, 0.0], [0.1], precision="f64")
    assert np.allclose(a, b, rtol=1e-5, atol=1e-7)
