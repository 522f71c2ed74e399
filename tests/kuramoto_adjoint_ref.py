"""FP64 NumPy restatement of the Kuramoto forward the order-parameter adjoint differentiates, and of
the discrete adjoint itself (test infrastructure).

Forward (the batched engine's semantics): one Kuramoto subnetwork coupled to itself through one CSR
projection with per-edge delays read with the ring rules of runtime.rs:162-204 (every edge reads
the current state at step 0; a delay longer than the step reads a zero row after pre(), i.e. adds
nothing to either channel; otherwise the state d steps back), Kuramoto coupling
c_i = (a / N) (cos th_i S_i - sin th_i C_i) with S_i, C_i the weighted sums of sin and cos of the
delayed source phases (coupling.rs Kuramoto arm), dth = omega + c (dfun.rs), deterministic Heun with
the coupling held over the step (engine.rs:710-720: both stages see the same c), phases wrapped to
[0, 2 pi) after the step.

Loss: L = (1 / T) sum_{t=1..T} R(t), R = |mean_j exp(i th_j)| (the time-averaged order parameter).
Gradients: dL/da (the coupling scale) and dL/domega: per node when omega is one value per node
(an array), else for the one omega all nodes share.
"""
import numpy as np


def forward(theta0, omega, a, indptr, indices, weights, delays, dt, n_steps):
    """Phases after every step [n_steps + 1, N] (row 0 = theta0) and the sums S, C [n_steps, N]."""
    n = theta0.shape[0]
    rows = np.repeat(np.arange(n), np.diff(indptr))
    th = np.empty((n_steps + 1, n))
    th[0] = theta0
    S, C = np.empty((n_steps, n)), np.empty((n_steps, n))
    for s in range(n_steps):
        if s == 0:
            src = th[0][indices]
            ok = np.ones_like(src, bool)
        else:
            t = s - delays
            ok = t >= 0
            src = th[np.maximum(t, 0), indices]
        S[s] = np.bincount(rows, weights=np.where(ok, weights * np.sin(src), 0.0), minlength=n)
        C[s] = np.bincount(rows, weights=np.where(ok, weights * np.cos(src), 0.0), minlength=n)
        c = (a / n) * (np.cos(th[s]) * S[s] - np.sin(th[s]) * C[s])
        x = th[s] + dt * (omega + c)
        th[s + 1] = np.mod(x, 2.0 * np.pi)
    return th, S, C


def order_loss(th):
    """Time average of R over the post-step phases (rows 1..T)."""
    z = np.exp(1j * th[1:]).mean(axis=1)
    return float(np.mean(np.abs(z)))


def adjoint(theta0, omega, a, indptr, indices, weights, delays, dt, n_steps):
    """Loss and (dL/da, dL/domega) by the discrete adjoint of the forward above; dL/domega is a vector
    over nodes when omega is an array."""
    n = theta0.shape[0]
    th, S, C = forward(theta0, omega, a, indptr, indices, weights, delays, dt, n_steps)
    T = n_steps
    z = np.exp(1j * th[1:]).mean(axis=1)          # [T], for t = 1..T
    R = np.abs(z)
    # dL/dth_j(t) = (1 / (T N R)) (Im z cos th_j - Re z sin th_j)
    src = ((z.imag[:, None] * np.cos(th[1:]) - z.real[:, None] * np.sin(th[1:])) / (T * n * R[:, None]))
    rows = np.repeat(np.arange(n), np.diff(indptr))
    lam = src[T - 1].copy()                      # lambda(T)
    nu_c, nu_s = np.zeros((T, n)), np.zeros((T, n))
    g_a, g_w = 0.0, np.zeros(n)
    k = a / n
    for s in range(T - 1, -1, -1):
        ci, si = np.cos(th[s]), np.sin(th[s])
        q = k * (-si * S[s] - ci * C[s])            # dc_i / dth_i
        g_a += dt * float(np.sum(lam * (ci * S[s] - si * C[s]))) / n
        g_w += dt * lam
        nu_c[s] = lam * dt * k * ci
        nu_s[s] = lam * dt * k * si
        if s == 0:
            break
        new = lam * (1.0 + dt * q) + src[s - 1]
        # delayed terms: th_j(s) is read at step s + d_e by target i_e (s + d_e <= T - 1)
        tt = s + delays
        ok = tt <= T - 1
        ttc = np.minimum(tt, T - 1)
        pc = np.where(ok, weights * nu_c[ttc, rows], 0.0)
        ps = np.where(ok, weights * nu_s[ttc, rows], 0.0)
        new += np.cos(th[s]) * np.bincount(indices, weights=pc, minlength=n)
        new += np.sin(th[s]) * np.bincount(indices, weights=ps, minlength=n)
        lam = new
    return order_loss(th), g_a, (g_w if np.ndim(omega) else float(np.sum(g_w)))
