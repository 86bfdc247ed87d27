"""Reference values of a Kerr null geodesic from its equations of motion at 30 significant
digits (mpmath), independent of the closed forms that the reference and the kernels
evaluate. Test infrastructure for tests/test_conditioning_cpu.py.

In Mino time tau (Gralla & Lupsasca 2020, Phys. Rev. D 101, 044031, eqs. 2), with
R(r) = (r^2 + a^2 - a lam)^2 - Delta (eta + (lam - a)^2), Delta = r^2 - 2r + a^2 and
u = cos(theta), P(u) = (1 - u^2)(eta + a^2 u^2) - lam^2 u^2:
    r'' = R'(r) / 2,   u'' = P'(u) / 2          (the squared first integrals differentiated,
                                                  smooth through the turning points)
    phi' = a (2r - a lam) / Delta + lam / (1 - u^2)
    t'   = (r^2 + a^2)(r^2 + a^2 - a lam) / Delta + a lam - a^2 (1 - u^2)
    sig' = r^2 + a^2 u^2
starting at r = r_o moving inward, u = cos(theta_o) with du/dtau of sign(beta) (beta >= 0:
+). r and u come from mpmath's Taylor-series ODE solver; t, phi, sigma from tanh-sinh
quadrature of the rates along that solution, with split points crowding toward each sample
(the rates grow like 1 / (tau_h - tau) next to the horizon). The reference traces backward
from the observer, so its t, phi and sigma are the negated integrals.
"""
import numpy as np


def geodesic(a, r_o, th_o, alpha, beta, taus, dps=30):
    """(5, len(taus)) array of t, r, theta, phi, sigma at the increasing Mino times taus."""
    import mpmath as mp
    with mp.workdps(dps):
        A = mp.mpf(a)
        th = mp.mpf(th_o)
        lam = -mp.mpf(alpha) * mp.sin(th)
        eta = (mp.mpf(alpha) ** 2 - A ** 2) * mp.cos(th) ** 2 + mp.mpf(beta) ** 2
        k2 = eta + (lam - A) ** 2

        def R(r):
            return (r * r + A * A - A * lam) ** 2 - (r * r - 2 * r + A * A) * k2

        def Rp(r):
            return 4 * r * (r * r + A * A - A * lam) - (2 * r - 2) * k2

        def P(u):
            return (1 - u * u) * (eta + A * A * u * u) - lam * lam * u * u

        def Pp(u):
            return -2 * u * (eta + A * A * u * u) + (1 - u * u) * 2 * A * A * u - 2 * lam * lam * u
        u0 = mp.cos(th)
        y0 = [mp.mpf(r_o), -mp.sqrt(R(mp.mpf(r_o))), u0, (1 if beta >= 0 else -1) * mp.sqrt(max(P(u0), 0))]
        sol = mp.odefun(lambda tau, y: [y[1], Rp(y[0]) / 2, y[3], Pp(y[2]) / 2], 0, y0,
                        tol=mp.mpf(10) ** (-dps + 2), degree=25)

        def rate(i):
            def f(tau):
                r, _, u, _ = sol(tau)
                D = r * r - 2 * r + A * A
                if i == 0:
                    return A * (2 * r - A * lam) / D + lam / (1 - u * u)
                if i == 1:
                    return (r * r + A * A) * (r * r + A * A - A * lam) / D + A * lam - A * A * (1 - u * u)
                return r * r + A * A * u * u
            return f
        out = np.zeros((5, len(taus)))
        prev = mp.mpf(0)
        acc = [mp.mpf(0)] * 3
        for k, tk in enumerate(taus):
            tk = mp.mpf(float(tk))
            if tk > prev:
                pts = [prev] + [tk - (tk - prev) * mp.mpf(10) ** (-j) for j in range(1, 14)] + [tk]
                acc = [acc[i] + mp.quad(rate(i), pts) for i in range(3)]
                prev = tk
            r, _, u, _ = sol(tk)
            out[:, k] = [float(-acc[1]), float(r), float(mp.acos(u)), float(-acc[0]), float(-acc[2])]
        return out
