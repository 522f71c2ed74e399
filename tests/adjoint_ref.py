"""FP64 NumPy restatement of the forward run the FC adjoint differentiates (test infrastructure).

One JansenRit subnetwork, one CSR projection with per-edge delays read with the serial engine's
ring rules (runtime.rs:162-204: current state at step 0, zero for d > s, else the state d steps
back), Sigmoidal or Linear coupling on y0, deterministic Heun (engine.rs:710-720) or RK4
(integrator.rs RK4 stages with the coupling held over the step). The JansenRit
A, B and a may differ per node, which the batched engine does not support; central finite
differences of the FC loss over these per-node parameters are the check of the GPU adjoint.
Pinned against the FP64 oracle at uniform parameters in tests/test_adjoint_ref.py.
"""
import numpy as np


def jr_dfun(p, y, c):
    """dfun.rs Jansen-Rit arm; p: dict of parameters (A, B, a arrays per node), y: [N, 6], c: [N]."""
    A, B, a, b = p["A"], p["B"], p["a"], p["b"]
    v0, nu, r, J = p["v0"], p["nu_max"], p["r"], p["J"]
    a1, a2, a3, a4, mu = p["a1"], p["a2"], p["a3"], p["a4"], p["mu"]

    def sig(v):
        return 2.0 * nu / (1.0 + np.exp(r * (v0 - v)))

    y0, y1, y2, y3, y4, y5 = (y[:, k] for k in range(6))
    d = np.empty_like(y)
    d[:, 0], d[:, 1], d[:, 2] = y3, y4, y5
    d[:, 3] = A * a * sig(y1 - y2) - 2.0 * a * y3 - a * a * y0
    d[:, 4] = A * a * (a2 * J * sig(a1 * J * y0) + mu + c) - 2.0 * a * y4 - a * a * y1
    d[:, 5] = B * b * (a4 * J * sig(a3 * J * y0)) - 2.0 * b * y5 - b * b * y2
    return d


def post(kind, cp, g):
    if kind == "Sigmoidal":
        cmin, cmax, mid, gain, sigma = cp
        return cmin + (cmax - cmin) / (1.0 + np.exp(-gain * (g - mid) / sigma))
    a, bb = cp[0], (cp[1] if len(cp) > 1 else 0.0)
    return a * g + bb


def params_dict(params13, n, A=None, B=None, a=None):
    names = ["A", "B", "a", "b", "v0", "nu_max", "r", "J", "a1", "a2", "a3", "a4", "mu"]
    p = {k: float(v) for k, v in zip(names, params13)}
    p["A"] = np.full(n, p["A"]) if A is None else np.asarray(A, np.float64)
    p["B"] = np.full(n, p["B"]) if B is None else np.asarray(B, np.float64)
    p["a"] = np.full(n, p["a"]) if a is None else np.asarray(a, np.float64)
    return p


def step(p, x, c, dt, integrator):
    """One deterministic Heun or RK4 step of the node states x [N, 6] at coupling c."""
    k1 = jr_dfun(p, x, c)
    if integrator == "rk4":
        k2 = jr_dfun(p, x + 0.5 * dt * k1, c)
        k3 = jr_dfun(p, x + 0.5 * dt * k2, c)
        k4 = jr_dfun(p, x + dt * k3, c)
        return x + (dt / 6.0) * (k1 + 2.0 * k2 + 2.0 * k3 + k4)
    k2 = jr_dfun(p, x + dt * k1, c)
    return x + 0.5 * dt * (k1 + k2)


def forward(p, x0, indptr, indices, weights, delays, kind, cp, dt, n_steps, integrator="heun"):
    """y1 - y2 after every step: [n_steps, N]."""
    n = x0.shape[0]
    x = np.array(x0, np.float64)
    hist = np.zeros((n_steps + 1, n))
    hist[0] = x[:, 0]
    rows = np.repeat(np.arange(n), np.diff(indptr))
    ys = np.empty((n_steps, n))
    for s in range(n_steps):
        if s == 0:
            vals = hist[0][indices]
        else:
            t = s - delays
            vals = np.where(t >= 0, hist[np.maximum(t, 0), indices], 0.0)
        g = np.bincount(rows, weights=weights * vals, minlength=n)
        c = post(kind, cp, g)
        x = step(p, x, c, dt, integrator)
        hist[s + 1] = x[:, 0]
        ys[s] = x[:, 1] - x[:, 2]
    return ys


def fc_loss(ys, target):
    fc = np.corrcoef(ys.T)
    return float(np.mean((fc - target) ** 2)), fc


def jr_vjp(p, y, c, u):
    """u^T df/dy and u . df/dc, df/dA, df/dB, df/da for the Jansen-Rit arm (rows are nodes)."""
    A, B, a, b = p["A"], p["B"], p["a"], p["b"]
    v0, nu, r, J = p["v0"], p["nu_max"], p["r"], p["J"]
    a1, a2, a3, a4, mu = p["a1"], p["a2"], p["a3"], p["a4"], p["mu"]

    def sig(v):
        s = 2.0 * nu / (1.0 + np.exp(r * (v0 - v)))
        return s, s * r * (1.0 - s / (2.0 * nu))

    s0, d0 = sig(y[:, 1] - y[:, 2])
    s1, d1 = sig(a1 * J * y[:, 0])
    s2, d2 = sig(a3 * J * y[:, 0])
    out = np.empty_like(y)
    out[:, 0] = -a * a * u[:, 3] + A * a * a2 * J * d1 * a1 * J * u[:, 4] + B * b * a4 * J * d2 * a3 * J * u[:, 5]
    out[:, 1] = A * a * d0 * u[:, 3] - a * a * u[:, 4]
    out[:, 2] = -A * a * d0 * u[:, 3] - b * b * u[:, 5]
    out[:, 3] = u[:, 0] - 2.0 * a * u[:, 3]
    out[:, 4] = u[:, 1] - 2.0 * a * u[:, 4]
    out[:, 5] = u[:, 2] - 2.0 * b * u[:, 5]
    Mv = a2 * J * s1 + mu + c
    uc = A * a * u[:, 4]
    uA = a * s0 * u[:, 3] + a * Mv * u[:, 4]
    uB = b * a4 * J * s2 * u[:, 5]
    ua = (A * s0 - 2.0 * y[:, 3] - 2.0 * a * y[:, 0]) * u[:, 3] + (A * Mv - 2.0 * y[:, 4] - 2.0 * a * y[:, 1]) * u[:, 4]
    return out, uc, uA, uB, ua


def adjoint(p, x0, indptr, indices, weights, delays, cp, dt, n_steps, target, dtype=np.float64, integrator="heun"):
    """Discrete adjoint of the Heun (or RK4) step for the FC loss (Sigmoidal coupling), the
    algorithm of the GPU kernels restated in NumPy: forward in `dtype`, adjoint in FP64. Returns
    loss and gradients (gain, A, B, a)."""
    n = x0.shape[0]
    rows = np.repeat(np.arange(n), np.diff(indptr))
    cmin, cmax, mid, gain, sigma = cp
    x = np.array(x0, dtype)
    hist = np.zeros((n_steps + 1, n), dtype)
    hist[0] = x[:, 0]
    xs, gs = np.empty((n_steps, n, 6)), np.empty((n_steps, n))
    ys = np.empty((n_steps, n))
    pd = {k: (v.astype(dtype) if isinstance(v, np.ndarray) else dtype(v)) for k, v in p.items()}
    w = weights.astype(dtype)
    for s in range(n_steps):
        vals = hist[0][indices] if s == 0 else np.where(s - delays >= 0, hist[np.maximum(s - delays, 0), indices], 0)
        g = np.bincount(rows, weights=(w * vals).astype(np.float64), minlength=n).astype(dtype)
        c = (cmin + (cmax - cmin) / (1.0 + np.exp(-gain * (g - mid) / sigma))).astype(dtype)
        xs[s], gs[s] = x, g
        if integrator == "rk4":
            x = step(pd, x, c, dtype(dt), "rk4").astype(dtype)
        else:
            k1 = jr_dfun(pd, x, c).astype(dtype)
            k2 = jr_dfun(pd, (x + dtype(dt) * k1).astype(dtype), c).astype(dtype)
            x = (x + dtype(0.5 * dt) * (k1 + k2)).astype(dtype)
        hist[s + 1] = x[:, 0]
        ys[s] = x[:, 1] - x[:, 2]
    T = n_steps
    mu_y, sd = ys.mean(0), ys.std(0)
    z = (ys - mu_y) / sd
    fc = z.T @ z / T
    np.fill_diagonal(fc, 1.0)
    loss = float(np.mean((fc - target) ** 2))
    M = 2.0 * (fc - target) / n ** 2
    np.fill_diagonal(M, 0.0)
    rk = (M * fc).sum(1)
    src = (2.0 / (T * sd)) * (z @ M.T - rk * z)          # [T, N], dL/dy(t) at row t-1
    lam = np.zeros((n, 6))
    lam[:, 1], lam[:, 2] = src[T - 1], -src[T - 1]
    mug = np.zeros((n_steps, n))
    gG = 0.0
    gA, gB, ga = np.zeros(n), np.zeros(n), np.zeros(n)
    # out-edges
    src_of = np.asarray(indices)
    for s in range(n_steps - 1, -1, -1):
        x_s, g = xs[s].astype(np.float64), gs[s].astype(np.float64)
        q = 1.0 / (1.0 + np.exp(-gain * (g - mid) / sigma))
        c = cmin + (cmax - cmin) * q
        k1 = jr_dfun(p, x_s, c)
        if integrator == "rk4":
            # x' = x + h/6 (k1 + 2 k2 + 2 k3 + k4), k_i = f(x_i): x2 = x + h/2 k1, x3 = x + h/2 k2, x4 = x + h k3
            x2 = x_s + 0.5 * dt * k1
            k2 = jr_dfun(p, x2, c)
            x3 = x_s + 0.5 * dt * k2
            k3 = jr_dfun(p, x3, c)
            x4 = x_s + dt * k3
            a4 = (dt / 6.0) * lam
            g4, uc4, uA4, uB4, ua4 = jr_vjp(p, x4, c, a4)
            a3 = (dt / 3.0) * lam + dt * g4
            g3, uc3, uA3, uB3, ua3 = jr_vjp(p, x3, c, a3)
            a2 = (dt / 3.0) * lam + 0.5 * dt * g3
            g2, uc2, uA2, uB2, ua2 = jr_vjp(p, x2, c, a2)
            a1 = (dt / 6.0) * lam + 0.5 * dt * g2
            g1, uc1, uA1, uB1, ua1 = jr_vjp(p, x_s, c, a1)
            lam = lam + g1 + g2 + g3 + g4
            mu_c = uc1 + uc2 + uc3 + uc4
            gA += uA1 + uA2 + uA3 + uA4
            gB += uB1 + uB2 + uB3 + uB4
            ga += ua1 + ua2 + ua3 + ua4
        else:
            pp = x_s + dt * k1
            u2 = 0.5 * dt * lam
            vp, uc2, uA2, uB2, ua2 = jr_vjp(p, pp, c, u2)
            u1 = 0.5 * dt * lam + dt * vp
            vx, uc1, uA1, uB1, ua1 = jr_vjp(p, x_s, c, u1)
            lam = lam + vp + vx
            mu_c = uc1 + uc2
            gA += uA1 + uA2
            gB += uB1 + uB2
            ga += ua1 + ua2
        dq = (cmax - cmin) * q * (1.0 - q)
        gG += float(np.sum(mu_c * dq * (g - mid) / sigma))
        mug[s] = mu_c * dq * gain / sigma
        if s >= 1:
            tt = s + delays
            ok = tt <= n_steps - 1
            contrib = np.where(ok, weights * mug[np.minimum(tt, n_steps - 1), rows], 0.0)
            lam[:, 0] += np.bincount(src_of, weights=contrib, minlength=n)
            lam[:, 1] += src[s - 1]
            lam[:, 2] -= src[s - 1]
    return loss, gG, gA, gB, ga
