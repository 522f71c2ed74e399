"""FP32 engine against the FP64 oracle on each benchmark configuration (run on a GPU machine:
``python tests/fp64_drift.py``); prints one line per configuration and output.

The FP64 oracle (hbo64_*) evaluates the reference's operations in the same order in double precision,
so its distance to the FP32 engine is the single-precision integration error of the configuration.
Reported per output: the largest absolute difference, that difference over the output's largest
magnitude, and the median relative difference (phases on the circle for Kuramoto).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

from hyburn_gb300 import BatchHybridEngine, GroupedSweep, SweepParam, inputs  # noqa: E402
from hyburn_gb300._abi import HB_SEM_BOLD_PER_POINT, HB_SEM_DELAY_RING  # noqa: E402
from oracle.hb_oracle import OracleEngine  # noqa: E402

THREADS = os.cpu_count() or 1


def stats(g, o, period=None):
    g, o = np.asarray(g, np.float64).ravel(), np.asarray(o, np.float64).ravel()
    d = g - o
    if period is not None:
        d = (d + period / 2) % period - period / 2
    ad = np.abs(d)
    scale = np.abs(o).max() if o.size else 1.0
    rel = ad / np.maximum(np.abs(o), 1e-12)
    return {"max_abs": float(ad.max()), "max_abs_over_max": float(ad.max() / max(scale, 1e-30)),
            "median_rel": float(np.median(rel))}


def report(name, outputs):
    for what, (g, o, per) in outputs.items():
        print(json.dumps({"config": name, "output": what, **stats(g, o, per)}), flush=True)


def main():
    # cfg 1: single simulation, 10 000 steps
    cfg, _ = inputs.plain_single_sim(10_000)
    par, vals = SweepParam(0, 1), [cfg.network.subnetworks[0].params[1]]
    g = BatchHybridEngine.from_config(cfg, 1).run_sweep(par, vals, 10_000)
    o = OracleEngine.from_config(cfg, 1, precision="f64").run_sweep(par, vals, 10_000)
    report("single-g2do-74n-10000", {"final": (g.final_states[0], o.final_states[0], None),
                                     "tavg": (g.tavg[0], o.tavg[0], None)})
    # cfg 2: the benchmark sweep, 128 x 74 x 20 000, deterministic and with the shared draws
    for stoch in (False, True):
        T = 20_000
        cfg, meta = inputs.batched_sweep(n_steps=T, nsig=1e-3 if stoch else 0.0,
                                         integrator="heun_stochastic" if stoch else "heun")
        noise = inputs.standard_normal((T, 148), 2) if stoch else None
        g = BatchHybridEngine.from_config(cfg, 128, semantics=HB_SEM_DELAY_RING).run_sweep(
            SweepParam(-1, 0), meta["values"], T, noise=noise)
        o = OracleEngine.from_config(cfg, 128, semantics=HB_SEM_DELAY_RING, precision="f64", n_threads=THREADS).run_sweep(
            SweepParam(-1, 0), meta["values"], T, noise=noise)
        report(f"sweep-g2do-74n-128pt-20000-{'stochastic' if stoch else 'deterministic'}",
               {"final": (g.final_states[0], o.final_states[0], None), "tavg": (g.tavg[0], o.tavg[0], None)})
    # cfg 3: every size of the uneven MPR grid, 4 grid points each, 44 000 RK4 steps (BOLD: 2 samples)
    T = 44_000
    members, refs = [], []
    for n in (68, 84, 164, 400):
        cfg, meta = inputs.mpr_grid(n, 4, T, seed=3, bold=True)
        sem = HB_SEM_DELAY_RING | HB_SEM_BOLD_PER_POINT
        members.append((BatchHybridEngine.from_config(cfg, 4, semantics=sem), SweepParam(-1, 0), meta["values"], T, None))
        refs.append(OracleEngine.from_config(cfg, 4, semantics=sem, precision="f64", n_threads=THREADS).run_sweep(
            SweepParam(-1, 0), meta["values"], T))
    grp = GroupedSweep(members)
    grp.execute()
    for n, o, r in zip((68, 84, 164, 400), refs, grp.results()):
        report(f"uneven-mpr-{n}n-4pt-44000", {"final": (r.final_states[0], o.final_states[0], None),
                                              "tavg": (r.tavg[0], o.tavg[0], None), "bold": (r.bold[0], o.bold[0], None)})
    grp.close()
    # cfg 5: Kuramoto 1000 nodes, per-node omega, 4 points x 10 000 steps
    T = 10_000
    cfg, meta = inputs.kuramoto_scale(n=1000, n_points=4, n_steps=T, bold=False)
    vals = [0.2, 0.8, 1.4, 2.0]
    g = BatchHybridEngine.from_config(cfg, 4, semantics=HB_SEM_DELAY_RING).run_sweep(SweepParam(-1, 0), vals, T)
    o = OracleEngine.from_config(cfg, 4, semantics=HB_SEM_DELAY_RING, precision="f64", n_threads=THREADS).run_sweep(
        SweepParam(-1, 0), vals, T)
    report("kuramoto-1000n-4pt-10000", {"final": (g.final_states[0], o.final_states[0], 2 * np.pi)})


if __name__ == "__main__":
    main()
